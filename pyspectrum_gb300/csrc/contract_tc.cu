// Triangle contraction on the 5th-generation tensor cores (tcgen05), split-BF16.
//
// bsum[t] = sum_v F_i(v) F_j(v) F_l(v) for triangles t = (i >= j >= l).
// Each triangle is (pair (i,j), column l).  The kernel evaluates the GEMM
//   D[p, c] = sum_v P_p(v) F_c(v),   P_p = F_i F_j  (pair p = (i, j))
// with pair rows on M (tiles of 128) and shells on N, the voxels on K.  Both
// operands are split into bf16 hi + lo parts (x = hi + lo with lo = x - hi),
// and three MMAs per k-step (hi*hi + hi*lo + lo*hi) accumulate in FP32 in
// tensor memory (TMEM).
//
// CTA layout (1 CTA per SM, persistent over a contiguous voxel range):
//   warps 0-15 (512 threads): producers.  Warp w owns TMEM lane quarter w%4
//     of pair tile w/4: lane l is pair row 128*(w/4) + 32*(w%4) + l.  Per
//     chunk of KC = 32 voxels the fields arrive in shared memory by cp.async
//     (prefetched 3 chunks ahead); each thread forms its pair's products,
//     splits them into hi/lo bf16 and writes them straight into TMEM
//     (tcgen05.st) as the MMA's A operand; the B operand (the shells' hi/lo
//     parts) goes to shared memory in the UMMA K-major core-matrix layout.
//     Then `full[stage]` is signalled.
//   warp 16, lane 0: issues tcgen05.mma (A from TMEM, B from shared memory)
//     and tcgen05.commit to `empty[stage]`.
//   Every SEG chunks the accumulators are drained: the MMA thread commits to
//   `seg`, the producers add the TMEM accumulators into Kahan-compensated
//   float32 sums per triangle in shared memory and arrive on `drained`; the
//   next MMA restarts the accumulators.  At the end each CTA writes one float64
//   partial per triangle; a second kernel adds the partials in a fixed order.
// TMEM columns: [0, C) accumulators; then two A stages of 32 columns per tile.
// Every mbarrier wait is bounded; on timeout the kernel records an error
// code, stops issuing work, waits (bounded) for its MMAs in flight, frees its
// TMEM and returns.
#include <cuda_bf16.h>
#include <string.h>
#include <algorithm>
#include <map>
#include <mutex>
#include <vector>
#include "contract.cuh"

namespace pyspec {

namespace tc {

constexpr int KC = 32;               // voxels per chunk (two k-steps of 16)
constexpr int MAXROWS = 512;         // pair rows per CTA group (4 M-tiles)
constexpr int MAXB = 64;             // shell rows of the B operand
constexpr int NSTAGE = 2;
constexpr int NPROD = 512;           // producer threads (warps 0-15): 4 tiles x 4 TMEM lane quarters
constexpr int PWARPS = NPROD / 32;
constexpr int NTHREADS = NPROD + 32; // + the MMA warp
constexpr int SEG = 64;              // chunks between accumulator drains
constexpr int FSTRIDE = KC + 4;      // padded float row of the field staging buffer
constexpr int MAXGROUPS = 8;
constexpr int MAXTILES = 4;
constexpr int MAXCOLS = 256;         // accumulator columns per group (+ 2 x 4 x 32 A columns <= 512)
constexpr int ACOLS = 32;            // TMEM columns of one tile's A operand per stage (2 k-steps x (8 hi + 8 lo))
constexpr int NFBUF = 8;             // field staging buffers (prefetch distance NFBUF-1 chunks)
constexpr unsigned long long kWaitNs = 2000000000ull;   // 2 s bound on any mbarrier wait

constexpr int B_BYTES = MAXB * KC * 2;         // one of hi / lo
constexpr int STAGE_BYTES = 2 * B_BYTES;
// one staging buffer holds the nshell field rows of a chunk
__host__ __device__ constexpr int f_bytes(int nshell) { return (nshell * FSTRIDE * 4 + 127) / 128 * 128; }

struct Group {
    int rows;              // pair rows used (<= 512)
    int ntiles;            // 128-row tiles
    int tile_n[MAXTILES];  // N of each tile (multiple of 16)
    int tile_col[MAXTILES];// TMEM column offset of each tile
    int ncols;             // TMEM columns allocated (power of 2 >= 32)
    int table_off;         // offset of this group in the row / slot tables
    int nslots;            // triangles (Kahan slots) of this group
};

struct Params {
    const float* fields;
    int64_t V;
    int nshell;
    int nb;                      // B rows (multiple of 16, <= 64)
    int ntri;
    int64_t nchunks;
    int64_t chunks_per_cta;
    const int16_t* pair_ij;      // [group][512][2] shell slots (-1 for padding rows)
    const int32_t* slot_of;      // [group][512][MAXB] accumulator slot of (pair row, shell) or -1
    const int32_t* slot_tri;     // [group][maxslots] triangle index of each slot
    double* partials;            // [gridDim.x][ntri]
    int* err;
    int ngroups;
    int maxslots;
    Group g[MAXGROUPS];
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Waits for the mbarrier phase with the given parity by polling try_wait
// (no suspend hint: a sleeping thread wakes too late for a per-chunk
// handshake); the wait gives up after kWaitNs and returns false.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    if (ok) return true;
    const unsigned long long t0 = globaltimer_ns();
    for (uint32_t it = 1;; ++it) {
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        if (ok) return true;
        if ((it & 255u) == 0 && globaltimer_ns() - t0 > kWaitNs) return false;
    }
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(bar) : "memory");
}

// UMMA shared-memory descriptor, K-major, no swizzle: core matrices of
// 8 rows x 16 bytes; LBO = byte distance between core matrices along K,
// SBO = along M/N.  Bits 46-48 hold the fixed value 0b001.
__device__ __forceinline__ uint64_t make_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor for kind::f16: D f32, A and B bf16, both K-major.
__device__ __forceinline__ uint32_t make_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// byte offset of element (row r, k) in a K-major no-swizzle operand with KC = 32:
// core matrix (r/8, k/8) at (r/8)*512 + (k/8)*128, row r%8 at 16 B, element k%8 at 2 B.
__device__ __forceinline__ int op_off(int r, int kgroup) { return (r >> 3) * 512 + kgroup * 128 + (r & 7) * 16; }

__device__ __forceinline__ uint32_t pack_bf16x2(float lo_half, float hi_half) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo_half, hi_half);   // .x -> low 16 bits
    return *reinterpret_cast<uint32_t*>(&v);
}

// Packed two-lane FP32 arithmetic (sm_100+): one instruction per float2.
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
    float2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(*reinterpret_cast<unsigned long long*>(&r))
        : "l"(*reinterpret_cast<unsigned long long*>(&a)), "l"(*reinterpret_cast<unsigned long long*>(&b)));
    return r;
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    float2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(*reinterpret_cast<unsigned long long*>(&r))
        : "l"(*reinterpret_cast<unsigned long long*>(&a)), "l"(*reinterpret_cast<unsigned long long*>(&b)));
    return r;
}

// Split 8 floats (as 4 float2) into hi/lo bf16 and store 16 B each.
__device__ __forceinline__ void split_store8(const float2* x, char* hi, char* lo) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        h[q] = pack_bf16x2(x[q].x, x[q].y);
        const float2 hv = make_float2(__uint_as_float(h[q] << 16), __uint_as_float(h[q] & 0xFFFF0000u));
        const float2 lv = sub2(x[q], hv);
        l[q] = pack_bf16x2(lv.x, lv.y);
    }
    *reinterpret_cast<uint4*>(hi) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4*>(lo) = make_uint4(l[0], l[1], l[2], l[3]);
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" :: "r"(dst), "l"(src), "r"(bytes) : "memory");
}

// TMEM helpers: 16 consecutive 32-bit columns of the warp's 32 lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t addr, uint32_t* v) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(addr));
}
__device__ __forceinline__ void tmem_st16(uint32_t addr, const uint32_t* v) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
        :: "r"(addr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
           "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
        : "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t addr, uint32_t* v) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                 : "r"(addr));
}
__device__ __forceinline__ void tmem_st8(uint32_t addr, const uint32_t* v) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
                 :: "r"(addr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]),
                    "r"(v[7])
                 : "memory");
}

__global__ void __launch_bounds__(NTHREADS, 1) contract_tc_kernel(const __grid_constant__ Params P) {
    extern __shared__ __align__(1024) unsigned char smem[];
    // this CTA's group descriptor, copied out of parameter space once (a
    // runtime index into the parameter struct would otherwise go to the stack)
    __shared__ Group G;
    if (threadIdx.x == 0) G = P.g[blockIdx.y];
    __syncthreads();
    unsigned char* stage_base = smem;                                          // NSTAGE x (B hi, B lo)
    float* fbuf = reinterpret_cast<float*>(smem + NSTAGE * STAGE_BYTES);       // NFBUF x F_BYTES
    const int F_BYTES = f_bytes(P.nshell);
    float2* acc = reinterpret_cast<float2*>(smem + NSTAGE * STAGE_BYTES + NFBUF * F_BYTES);  // Kahan (sum, comp)
    __shared__ __align__(8) uint64_t bar_full[NSTAGE], bar_empty[NSTAGE], bar_seg, bar_drained;
    __shared__ uint32_t tmem_slot;
    __shared__ int16_t pij[MAXROWS * 2];
    __shared__ int abort_flag_s;
    volatile int& abort_flag = abort_flag_s;

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int64_t c0 = (int64_t)blockIdx.x * P.chunks_per_cta;
    const int64_t c1 = min(P.nchunks, c0 + P.chunks_per_cta);
    const int nch = (int)max((int64_t)0, c1 - c0);
    int C = 0;
    for (int t = 0; t < G.ntiles; ++t) C = max(C, G.tile_col[t] + G.tile_n[t]);

    // ---- set-up ----
    for (int i = tid; i < MAXROWS * 2; i += NTHREADS) pij[i] = P.pair_ij[(size_t)G.table_off * 2 + i];
    for (int i = tid; i < G.nslots; i += NTHREADS) acc[i] = make_float2(0.f, 0.f);
    // zero both B stages once: padding shells stay zero
    for (int i = tid; i < NSTAGE * STAGE_BYTES / 16; i += NTHREADS)
        reinterpret_cast<uint4*>(stage_base)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        abort_flag = 0;
        for (int s = 0; s < NSTAGE; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_full[s])), "r"(PWARPS));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_empty[s])), "r"(1));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_seg)), "r"(1));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_drained)), "r"(PWARPS));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == PWARPS) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&tmem_slot)), "r"(G.ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const int q = warp & 3;                          // TMEM lane quarter of this warp
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    // A operand of tile t, stage s, k-step ks: 8 hi columns then 8 lo columns
    auto acol = [&](int s, int t, int ks) { return (uint32_t)(C + (s * MAXTILES + t) * ACOLS + ks * 16); };

    if (warp < PWARPS) {
        // ================= producers =================
        const int rows = G.rows;
        const int nsh = P.nshell;
        const int mytile = warp >> 2;                 // warp-uniform
        const bool tile_on = mytile < G.ntiles;
        const int row = 128 * mytile + 32 * q + lane;
        const bool row_on = tile_on && row < rows && pij[2 * row] >= 0;
        const int fi = row_on ? pij[2 * row] * FSTRIDE : 0;
        const int fj = row_on ? pij[2 * row + 1] * FSTRIDE : 0;
        int ub_f = -1, ub_off = 0;
        if (tid < nsh * 4) {
            const int g = (tid >= nsh) + (tid >= 2 * nsh) + (tid >= 3 * nsh);
            const int r = tid - g * nsh;
            ub_f = r * FSTRIDE + 8 * g;
            ub_off = op_off(r, g);
        }
        const int ncp = nsh * (KC / 4);                 // 16-byte copies per chunk
        int cp_s = 0, cp_q = 0;
        if (tid < ncp) { cp_s = tid / (KC / 4); cp_q = tid - cp_s * (KC / 4); }
        // Every thread commits one cp.async group per chunk (possibly empty) so
        // that wait_group counts line up across threads.
        const float* cp_src = P.fields + (size_t)cp_s * P.V + (size_t)c0 * KC + cp_q * 4;
        const int64_t cp_v0 = c0 * KC + cp_q * 4;
        const uint32_t cp_dst = smem_u32(fbuf + cp_s * FSTRIDE + cp_q * 4);
#define PYSPEC_ISSUE_FIELDS(cc)                                                                     \
        do {                                                                                        \
            const int c_ = (cc);                                                                    \
            if (c_ < nch && tid < ncp) {                                                            \
                const int64_t v_ = cp_v0 + (int64_t)c_ * KC;                                        \
                int bytes_ = 0;                                                                     \
                if (v_ < P.V) bytes_ = (int)min((int64_t)16, (P.V - v_) * 4);                       \
                cp_async16(cp_dst + (uint32_t)((c_ % NFBUF) * F_BYTES), bytes_ > 0 ? cp_src + (size_t)c_ * KC : P.fields, bytes_); \
            }                                                                                       \
            asm volatile("cp.async.commit_group;" ::: "memory");                                    \
        } while (0)
        for (int c = 0; c < NFBUF - 1; ++c) PYSPEC_ISSUE_FIELDS(c);
        int seg_count = 0;
        // A producer that times out sets abort_flag and skips to the next
        // chunk; every producer reads the flag right after the same named
        // barrier, so they all leave the loop together.
        for (int c = 0; c < nch; ++c) {
            const int s = c & 1;
            asm volatile("cp.async.wait_group %0;" :: "n"(NFBUF - 2) : "memory");   // chunk c has landed
            // named barrier 1 counts exactly the NPROD producer threads
            asm volatile("bar.sync 1, %0;" :: "n"(NPROD) : "memory");   // chunk c landed everywhere; c-1 consumed
            if (abort_flag) break;
            PYSPEC_ISSUE_FIELDS(c + NFBUF - 1);                     // into the buffer chunk c-1 used
            if (c >= NSTAGE) {
                if (!mbar_wait(smem_u32(&bar_empty[s]), ((c - NSTAGE) >> 1) & 1)) {
                    atomicExch(P.err, 1);
                    abort_flag = 1;
                    continue;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            }
            const float* F = fbuf + (size_t)(c % NFBUF) * (F_BYTES / 4);
            char* Bhi = reinterpret_cast<char*>(stage_base) + (size_t)s * STAGE_BYTES;
            char* Blo = Bhi + B_BYTES;
            // B operand: shells 0..nshell-1 (rows >= nshell stay zero)
            if (ub_f >= 0) {
                const float4 a = *reinterpret_cast<const float4*>(F + ub_f);
                const float4 b = *reinterpret_cast<const float4*>(F + ub_f + 4);
                const float2 x[4] = {make_float2(a.x, a.y), make_float2(a.z, a.w), make_float2(b.x, b.y),
                                     make_float2(b.z, b.w)};
                split_store8(x, Bhi + ub_off, Blo + ub_off);
            }
            // A operand: this lane's pair products, straight into TMEM
            if (tile_on) {
#pragma unroll
                for (int ks = 0; ks < KC / 16; ++ks) {
                    uint32_t h[8], l[8];
#pragma unroll
                    for (int g = 0; g < 4; ++g) {
                        float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
                        if (row_on) {
                            a = *reinterpret_cast<const float4*>(F + fi + 16 * ks + 4 * g);
                            b = *reinterpret_cast<const float4*>(F + fj + 16 * ks + 4 * g);
                        }
                        const float2 p0 = mul2(make_float2(a.x, a.y), make_float2(b.x, b.y));
                        const float2 p1 = mul2(make_float2(a.z, a.w), make_float2(b.z, b.w));
                        h[2 * g] = pack_bf16x2(p0.x, p0.y);
                        h[2 * g + 1] = pack_bf16x2(p1.x, p1.y);
                        const float2 l0 = sub2(p0, make_float2(__uint_as_float(h[2 * g] << 16),
                                                               __uint_as_float(h[2 * g] & 0xFFFF0000u)));
                        const float2 l1 = sub2(p1, make_float2(__uint_as_float(h[2 * g + 1] << 16),
                                                               __uint_as_float(h[2 * g + 1] & 0xFFFF0000u)));
                        l[2 * g] = pack_bf16x2(l0.x, l0.y);
                        l[2 * g + 1] = pack_bf16x2(l1.x, l1.y);
                    }
                    tmem_st8(lane_base + acol(s, mytile, ks), h);
                    tmem_st8(lane_base + acol(s, mytile, ks) + 8u, l);
                }
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            // one arrive per warp (the barrier counts warps): the lanes' writes are
            // ordered before lane 0's release by the warp barrier
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&bar_full[s]));
            // drain after the last chunk of every segment: add the segment's
            // accumulators into the Kahan sums in shared memory
            if ((c + 1) % SEG == 0 || c + 1 == nch) {
                if (!mbar_wait(smem_u32(&bar_seg), seg_count & 1)) {
                    atomicExch(P.err, 2);
                    abort_flag = 1;
                    continue;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                // the four warps of this lane quarter take 8-column blocks round-robin
                for (int cb = 8 * (warp >> 2); cb < C; cb += 32) {
                    uint32_t d[8];
                    tmem_ld8(lane_base + (uint32_t)cb, d);
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    int t = 0;
                    while (t + 1 < G.ntiles && cb >= G.tile_col[t + 1]) ++t;
                    if (cb >= G.tile_col[t] + G.tile_n[t]) continue;
                    const int drow = 128 * t + 32 * q + lane;
                    const bool drow_ok = drow < rows;
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const int col = cb - G.tile_col[t] + e;
                        const int slot = drow_ok ? P.slot_of[((size_t)G.table_off + drow) * MAXB + col] : -1;
                        if (slot < 0) continue;
                        const float2 a = acc[slot];
                        const float y = __uint_as_float(d[e]) - a.y;
                        const float sum = a.x + y;
                        acc[slot] = make_float2(sum, (sum - a.x) - y);
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(&bar_drained));
                ++seg_count;
            }
        }
#undef PYSPEC_ISSUE_FIELDS
        asm volatile("cp.async.wait_group 0;" ::: "memory");
    } else if (lane == 0) {
        // ================= MMA issuer =================
        // Small-N MMAs are bound by their issue cost, so every operand address
        // is computed once: B descriptors and A TMEM addresses per (stage, k-step).
        const int ntiles = G.ntiles;
        uint32_t idesc[MAXTILES], dcol[MAXTILES];
#pragma unroll
        for (int t = 0; t < MAXTILES; ++t) {
            idesc[t] = make_idesc(128, G.tile_n[t]);
            dcol[t] = tmem + (uint32_t)G.tile_col[t];
        }
        const uint32_t sbase = smem_u32(stage_base);
        uint64_t dbh[NSTAGE][KC / 16], dbl[NSTAGE][KC / 16];
        uint32_t aad[NSTAGE][KC / 16][MAXTILES];
#pragma unroll
        for (int s = 0; s < NSTAGE; ++s)
#pragma unroll
            for (int ks = 0; ks < KC / 16; ++ks) {
                const uint32_t bhi = sbase + (uint32_t)(s * STAGE_BYTES) + (uint32_t)(ks * 256);
                dbh[s][ks] = make_desc(bhi, 128, 512);
                dbl[s][ks] = make_desc(bhi + B_BYTES, 128, 512);
#pragma unroll
                for (int t = 0; t < MAXTILES; ++t) aad[s][ks][t] = tmem + acol(s, t, ks);
            }
        int seg_count = 0;
        uint32_t first = 0;   // 0: the next MMA of each tile overwrites its accumulator
        for (int c = 0; c < nch; ++c) {
            const int s = c & 1;
            if (!mbar_wait(smem_u32(&bar_full[s]), (c >> 1) & 1)) { atomicExch(P.err, 3); abort_flag = 1; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int ks = 0; ks < KC / 16; ++ks) {
                const uint64_t bh = s ? dbh[1][ks] : dbh[0][ks];
                const uint64_t bl = s ? dbl[1][ks] : dbl[0][ks];
                const uint32_t acc0 = ks == 0 ? first : 1u;
#pragma unroll
                for (int t = 0; t < MAXTILES; ++t) {
                    if (t < ntiles) {
                        const uint32_t ahi = s ? aad[1][ks][t] : aad[0][ks][t];
                        const uint32_t alo = ahi + 8u;
                        asm volatile("{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n"
                                     :: "r"(dcol[t]), "r"(ahi), "l"(bh), "r"(idesc[t]), "r"(acc0));
                        asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, 1;"
                                     :: "r"(dcol[t]), "r"(ahi), "l"(bl), "r"(idesc[t]));
                        asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, 1;"
                                     :: "r"(dcol[t]), "r"(alo), "l"(bh), "r"(idesc[t]));
                    }
                }
            }
            first = 1u;
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         :: "r"(smem_u32(&bar_empty[s])) : "memory");
            if ((c + 1) % SEG == 0 || c + 1 == nch) {
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                             :: "r"(smem_u32(&bar_seg)) : "memory");
                if (!mbar_wait(smem_u32(&bar_drained), seg_count & 1)) { atomicExch(P.err, 4); abort_flag = 1; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                ++seg_count;
                first = 0u;
            }
        }
        // make sure no MMA is still running before the TMEM is released
        if (nch > 0) {
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         :: "r"(smem_u32(&bar_seg)) : "memory");
            mbar_wait(smem_u32(&bar_seg), seg_count & 1);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    // partial sums of this CTA's triangles
    if (!abort_flag) {
        for (int i = tid; i < G.nslots; i += NTHREADS) {
            const int t = P.slot_tri[(size_t)blockIdx.y * P.maxslots + i];
            P.partials[(size_t)blockIdx.x * P.ntri + t] = (double)acc[i].x - (double)acc[i].y;
        }
    }
    if (warp == PWARPS) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(G.ncols));
    }
}

// ---------------------------------------------------------------------------
// host planning: pairs (i, j) = the two largest shell slots of each triangle,
// column = the smallest.  Pairs sorted by (j, i) keep each tile's columns
// short.  Plans are cached per triangle list.
// ---------------------------------------------------------------------------
struct HostPlan {
    Params base;           // pointers filled at launch
    std::vector<int16_t> pair_ij;
    std::vector<int32_t> slot_of;
    std::vector<int32_t> slot_tri;
    size_t smem = 0;
    bool ok = false;
    char why[160] = {0};
};

static std::mutex g_plan_mu;
static std::map<std::vector<int32_t>, HostPlan*> g_plans;

static int pow2_cols(int n) {
    int c = 32;
    while (c < n) c <<= 1;
    return c;
}

static HostPlan* build_plan(int nshell, const int32_t* tri_host, int ntri) {
    HostPlan* hp = new HostPlan();
    Params& P = hp->base;
    memset(&P, 0, sizeof(P));
    if (nshell > MAXB) {
        snprintf(hp->why, sizeof(hp->why), "BF16x3 contraction supports at most %d shells", MAXB);
        return hp;
    }
    std::map<std::pair<int, int>, std::vector<std::pair<int, int>>> pairs;   // (i,j) -> [(l, t)]
    for (int t = 0; t < ntri; ++t) {
        int a = tri_host[t], b = tri_host[ntri + t], c = tri_host[2 * ntri + t];
        if (a < 0 || b < 0 || c < 0 || a >= nshell || b >= nshell || c >= nshell) {
            snprintf(hp->why, sizeof(hp->why), "triangle %d has a slot outside [0, %d)", t, nshell);
            return hp;
        }
        int v[3] = {a, b, c};
        std::sort(v, v + 3);
        pairs[{v[2], v[1]}].push_back({v[0], t});
    }
    std::vector<std::pair<int, int>> order;
    for (auto& kv : pairs) order.push_back(kv.first);
    std::sort(order.begin(), order.end(), [](const std::pair<int, int>& x, const std::pair<int, int>& y) {
        return x.second != y.second ? x.second < y.second : x.first < y.first;
    });
    const int nrows = (int)order.size();
    // N of each 128-row tile: the largest shell column it needs, rounded to 16;
    // and the number of triangles (Kahan slots) it holds
    std::vector<int> tile_n, tile_slots;
    for (int r0 = 0; r0 < nrows; r0 += 128) {
        int maxl = 0, ns = 0;
        for (int r = r0; r < std::min(nrows, r0 + 128); ++r) {
            for (auto& lt : pairs[order[r]]) maxl = std::max(maxl, lt.first);
            ns += (int)pairs[order[r]].size();
        }
        tile_n.push_back(((maxl + 1) + 15) / 16 * 16);
        tile_slots.push_back(ns);
    }
    const int ntiles_all = (int)tile_n.size();
    const size_t fixed = (size_t)NSTAGE * STAGE_BYTES + (size_t)NFBUF * f_bytes(nshell);
    const int budget = (int)((227 * 1024 - 4096 - fixed) / sizeof(float2));
    // Greedy grouping into CTA groups: at most 4 tiles, MAXCOLS accumulator
    // columns (TMEM also holds 2 stages x 4 tiles x 32 A columns) and `budget`
    // Kahan slots in shared memory.
    std::vector<int> group_first;
    {
        int cur_tiles = 0, cur_cols = 0, cur_slots = 0;
        for (int t = 0; t < ntiles_all; ++t) {
            if (tile_slots[t] > budget) {
                snprintf(hp->why, sizeof(hp->why), "a 128-row tile holds %d triangles (limit %d)", tile_slots[t], budget);
                return hp;
            }
            if (cur_tiles == 0 || cur_tiles == MAXTILES || cur_cols + tile_n[t] > MAXCOLS ||
                cur_slots + tile_slots[t] > budget) {
                group_first.push_back(t);
                cur_tiles = cur_cols = cur_slots = 0;
            }
            ++cur_tiles;
            cur_cols += tile_n[t];
            cur_slots += tile_slots[t];
        }
    }
    const int ngroups = (int)group_first.size();
    if (ngroups > MAXGROUPS || ngroups == 0) {
        snprintf(hp->why, sizeof(hp->why), "too many pair rows (%d) for the BF16x3 contraction", nrows);
        return hp;
    }
    P.ngroups = ngroups;
    P.nshell = nshell;
    P.ntri = ntri;
    int nb = 16;
    hp->pair_ij.assign((size_t)ngroups * MAXROWS * 2, (int16_t)-1);
    hp->slot_of.assign((size_t)ngroups * MAXROWS * MAXB, -1);
    std::vector<std::vector<int32_t>> gslots(ngroups);
    int maxslots = 1;
    for (int g = 0; g < ngroups; ++g) {
        Group& G = P.g[g];
        const int t0 = group_first[g];
        const int t1 = g + 1 < ngroups ? group_first[g + 1] : ntiles_all;
        const int r0 = 128 * t0;
        G.rows = std::min(128 * (t1 - t0), nrows - r0);
        G.ntiles = t1 - t0;
        G.table_off = g * MAXROWS;
        int col = 0;
        for (int t = 0; t < MAXTILES; ++t) { G.tile_n[t] = 16; G.tile_col[t] = 0; }
        for (int t = 0; t < G.ntiles; ++t) {
            G.tile_n[t] = tile_n[t0 + t];
            G.tile_col[t] = col;
            col += G.tile_n[t];
            nb = std::max(nb, G.tile_n[t]);
        }
        G.ncols = pow2_cols(col + NSTAGE * MAXTILES * ACOLS);
        if (G.ncols > 512) {
            snprintf(hp->why, sizeof(hp->why), "BF16x3 tile columns exceed TMEM");
            return hp;
        }
        for (int r = 0; r < G.rows; ++r) {
            auto key = order[r0 + r];
            hp->pair_ij[((size_t)G.table_off + r) * 2] = (int16_t)key.first;
            hp->pair_ij[((size_t)G.table_off + r) * 2 + 1] = (int16_t)key.second;
            for (auto& lt : pairs[key]) {
                hp->slot_of[((size_t)G.table_off + r) * MAXB + lt.first] = (int32_t)gslots[g].size();
                gslots[g].push_back(lt.second);
            }
        }
        G.nslots = (int)gslots[g].size();
        maxslots = std::max(maxslots, G.nslots);
    }
    if (nb > MAXB) {
        snprintf(hp->why, sizeof(hp->why), "BF16x3 contraction supports at most %d shells", MAXB);
        return hp;
    }
    P.nb = nb;
    P.maxslots = maxslots;
    hp->slot_tri.assign((size_t)ngroups * maxslots, 0);
    for (int g = 0; g < ngroups; ++g)
        for (size_t i = 0; i < gslots[g].size(); ++i) hp->slot_tri[(size_t)g * maxslots + i] = gslots[g][i];
    hp->smem = fixed + sizeof(float2) * (size_t)maxslots;
    hp->ok = true;
    return hp;
}

static HostPlan* get_plan(int nshell, const int32_t* tri_host, int ntri) {
    std::vector<int32_t> key(tri_host, tri_host + 3 * (size_t)ntri);
    key.push_back(nshell);
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_plans.find(key);
    if (it != g_plans.end()) return it->second;
    HostPlan* hp = build_plan(nshell, tri_host, ntri);
    g_plans[key] = hp;
    return hp;
}

static int grid_x(int64_t nchunks, int ngroups) {
    int sms = 152;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int gx = std::max(1, sms / std::max(1, ngroups));
    if ((int64_t)gx > nchunks) gx = (int)std::max<int64_t>(1, nchunks);
    return gx;
}

static size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace tc

size_t contract_tc_ws(int64_t nvox, int nshell, int ntri) {
    // tables (bounded by the largest plan for nshell <= 64) + partials + error word
    const size_t rows = (size_t)tc::MAXGROUPS * tc::MAXROWS;
    const size_t tables = rows * 2 * 2 + rows * tc::MAXB * 4 + (size_t)tc::MAXGROUPS * (size_t)ntri * 4 + 4096;
    const int64_t nchunks = (nvox + tc::KC - 1) / tc::KC;
    const size_t gx = (size_t)std::min<int64_t>(std::max<int64_t>(nchunks, 1), 1024);
    return tc::al256(tables) + tc::al256(gx * (size_t)std::max(ntri, 1) * sizeof(double)) + 256;
}

int contract_tc_impl(const float* fields, int64_t nvox, int nshell, const int32_t* tri, const int32_t* tri_host,
                     int ntri, double* bsum, void* ws, size_t ws_bytes, cudaStream_t st) {
    using namespace tc;
    PYSPEC_CHECK_ARG(tri_host != nullptr, "the BF16x3 contraction needs the host copy of the triangle list");
    PYSPEC_CHECK_ARG(nvox % 4 == 0, "BF16x3 contraction needs N^3 divisible by 4");
    PYSPEC_CHECK_ARG(((uintptr_t)fields & 15) == 0, "fields must be 16-byte aligned");
    HostPlan* hp = get_plan(nshell, tri_host, ntri);
    if (!hp->ok) {
        set_error("%s", hp->why);
        return PYSPEC_E_UNSUPPORTED;
    }
    const size_t need = contract_tc_ws(nvox, nshell, ntri);
    if (ws_bytes < need) {
        set_error("contract workspace %zu bytes < required %zu", ws_bytes, need);
        return PYSPEC_E_WORKSPACE;
    }
    char* w = reinterpret_cast<char*>(ws);
    size_t off = 0;
    int* d_err = reinterpret_cast<int*>(w + off); off += 256;      // status word first
    int16_t* d_pair = reinterpret_cast<int16_t*>(w + off); off += al256(hp->pair_ij.size() * 2);
    int32_t* d_slot = reinterpret_cast<int32_t*>(w + off); off += al256(hp->slot_of.size() * 4);
    int32_t* d_stri = reinterpret_cast<int32_t*>(w + off); off += al256(hp->slot_tri.size() * 4);
    const int64_t nchunks = (nvox + KC - 1) / KC;
    const int gx = grid_x(nchunks, hp->base.ngroups);
    double* partials = reinterpret_cast<double*>(w + off);
    if (off + al256((size_t)gx * ntri * sizeof(double)) > ws_bytes) {
        set_error("contract workspace too small for %d CTAs", gx);
        return PYSPEC_E_WORKSPACE;
    }
    PYSPEC_CUDA(cudaMemcpyAsync(d_pair, hp->pair_ij.data(), hp->pair_ij.size() * 2, cudaMemcpyHostToDevice, st));
    PYSPEC_CUDA(cudaMemcpyAsync(d_slot, hp->slot_of.data(), hp->slot_of.size() * 4, cudaMemcpyHostToDevice, st));
    PYSPEC_CUDA(cudaMemcpyAsync(d_stri, hp->slot_tri.data(), hp->slot_tri.size() * 4, cudaMemcpyHostToDevice, st));
    PYSPEC_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    PYSPEC_CUDA(cudaMemsetAsync(partials, 0, (size_t)gx * ntri * sizeof(double), st));
    Params P = hp->base;
    P.fields = fields;
    P.V = nvox;
    P.nchunks = nchunks;
    P.chunks_per_cta = (nchunks + gx - 1) / gx;
    P.pair_ij = d_pair;
    P.slot_of = d_slot;
    P.slot_tri = d_stri;
    P.partials = partials;
    P.err = d_err;
    PYSPEC_TRY(allow_smem((const void*)contract_tc_kernel, hp->smem));
    contract_tc_kernel<<<dim3(gx, P.ngroups), NTHREADS, hp->smem, st>>>(P);
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    (void)tri;
    return reduce_partials_launch(partials, gx, ntri, bsum, st);
}

}  // namespace pyspec
