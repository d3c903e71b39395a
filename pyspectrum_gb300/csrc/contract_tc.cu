// Triangle contraction on the 5th-generation tensor cores (tcgen05), split-BF16.
//
// bsum[t] = sum_v F_i(v) F_j(v) F_l(v) for triangles t = (i >= j >= l).
// Each triangle is (pair (i,j), column l).  The kernel evaluates the GEMM
//   D[p, c] = sum_v P_p(v) F_c(v),   P_p = F_i F_j  (pair p = (i, j))
// with pair rows on M (tiles of 128) and shells on N, the voxels on K.  Both
// operands are split into bf16 hi + lo parts (x = hi + lo, lo = x - hi).  The
// B operand holds the hi and lo rows of the shells interleaved in blocks of
// 16 (rows [32b, 32b+16) = hi of shells [16b, 16b+16), the next 16 rows = lo),
// so one MMA with N' = 2N gives A_x * B_hi and A_x * B_lo side by side; two
// MMAs per k-step (A_hi, then A_lo, same B, same accumulator) produce all four
// products (hi+lo)(hi+lo), which are summed over the hi/lo column pairs when
// the accumulators are drained.  Small-N tcgen05.mma instructions are bound
// by a per-instruction cost, so two wide MMAs beat three narrow ones.
//
// CTA layout (1 CTA per SM, persistent over a contiguous voxel range):
//   warps 0-15 (512 threads): producers.  Warp w owns TMEM lane quarter w%4
//     of pair tile w/4: lane l is pair row 128*(w/4) + 32*(w%4) + l.  Per
//     chunk of KC = 32 voxels each thread forms its pair's 32 products,
//     splits them into hi/lo bf16 and writes them straight into TMEM
//     (tcgen05.st) as the MMA's A operand; threads < 4*nshell write the B
//     operand (the shells' hi/lo parts) to shared memory in the UMMA K-major
//     core-matrix layout.  Then `full[stage]` and `fempty[buffer]` are
//     signalled (one arrival per warp).
//   warp 16, lane 0: issues tcgen05.mma (A from TMEM, B from shared memory)
//     and tcgen05.commit to `empty[stage]`.
//   warp 17, lane 0: streams the fields: one TMA tensor copy per chunk
//     (nshell rows x 32 floats, 128-byte swizzle) into a ring of NFBUF
//     buffers, completing on `ffull[buffer]`.
//   Every SEG chunks the accumulators are drained: the MMA thread commits to
//   `seg`, the producers add the TMEM accumulators into Kahan-compensated
//   float32 sums per triangle in shared memory and arrive on `drained`; the
//   next MMA restarts the accumulators.  At the end each CTA writes one float64
//   partial per triangle; a second kernel adds the partials in a fixed order.
// TMEM columns: [0, C) accumulators (2N per tile); then two A stages of 32
// columns per tile.  Every mbarrier wait is bounded; on timeout the kernel
// records an error code, stops issuing work, waits (bounded) for its copies
// and MMAs in flight, frees its TMEM and returns.
#include <cuda.h>
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
constexpr int MAXB = 64;             // shells
constexpr int BROWS = 2 * MAXB;      // B operand rows (hi and lo of each shell)
constexpr int NSTAGE = 2;
constexpr int NPROD = 512;           // producer threads (warps 0-15): 4 tiles x 4 TMEM lane quarters
constexpr int PWARPS = NPROD / 32;
constexpr int MMA_WARP = PWARPS;
constexpr int TMA_WARP = PWARPS + 1;
constexpr int NTHREADS = NPROD + 64; // + the MMA warp + the copy warp
constexpr int SEG = 32;              // chunks between accumulator drains (TMEM float32 accumulation length sets the error: 128 chunks gave a bf16x3 median error of 8e-6 vs FP64, 64 gave 4e-6)
constexpr int MAXGROUPS = 8;
constexpr int MAXTILES = 4;
constexpr int MAXCOLS = 256;         // accumulator columns per group (+ 2 x 4 x 32 A columns <= 512)
constexpr int ACOLS = 32;            // TMEM columns of one tile's A operand per stage (2 k-steps x (8 hi + 8 lo))
constexpr int NFBUF = 6;             // field buffers in the copy ring
constexpr unsigned long long kWaitNs = 2000000000ull;   // 2 s bound on any mbarrier wait

constexpr int STAGE_BYTES = BROWS * KC * 2;    // B operand of one stage (hi and lo rows)
// one field buffer: nshell rows of 128 bytes, in whole 1024-byte swizzle atoms
__host__ __device__ constexpr int f_bytes(int nshell) { return (nshell * 128 + 1023) / 1024 * 1024; }
// dynamic shared memory before the Kahan slots (+1 KB to align the base to 1024)
__host__ __device__ constexpr int fixed_smem(int nshell) { return 1024 + NFBUF * f_bytes(nshell) + NSTAGE * STAGE_BYTES; }

struct Group {
    int rows;              // pair rows used (<= 512)
    int ntiles;            // 128-row tiles
    int tile_n[MAXTILES];  // N of each tile in shells (multiple of 16); the MMA uses 2N columns
    int tile_col[MAXTILES];// TMEM column offset of each tile
    int ncols;             // TMEM columns allocated (power of 2 >= 32)
    int table_off;         // offset of this group in the row / slot tables
    int nslots;            // triangles (Kahan slots) of this group
};

struct Params {
    int64_t V;
    int nshell;
    int ntri;
    int64_t nchunks;
    int64_t chunks_per_cta;
    // [group][512][4] per pair row: i | j << 8 (shell slots; -1 for padding
    // rows), lmin, lmax (the columns l of its triangles) and the first of its
    // Kahan slots; the row's columns l in [lmin, lmax] own consecutive slots
    const int16_t* pair_row;
    const int32_t* slot_tri;     // [group][maxslots] triangle index of each slot (-1: unused)
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

// All lanes of a warp wait; the outcome is made warp-uniform (tcgen05.ld/st
// are warp-collective, so a warp must not split on a wait).
__device__ __forceinline__ bool warp_wait(uint32_t bar, uint32_t parity) {
    return __all_sync(0xffffffffu, mbar_wait(bar, parity));
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

// B operand row of shell s, part p (0 = hi, 1 = lo): hi/lo interleaved in blocks of 16
__host__ __device__ __forceinline__ int brow(int s, int p) { return ((s >> 4) << 5) | (p << 4) | (s & 15); }
// shell of accumulator column c (relative to its tile)
__host__ __device__ __forceinline__ int col_shell(int c) { return ((c >> 5) << 4) | (c & 15); }

// byte offset of the 16-byte chunk q (voxels 4q..4q+3) of field row r in a
// buffer written by the TMA with 128-byte swizzle (chunk index XOR row % 8)
__device__ __forceinline__ int fchunk(int r, int q) { return r * 128 + ((q ^ (r & 7)) << 4); }

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

// TMEM helpers: 8 consecutive 32-bit columns of the warp's 32 lanes.
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

__global__ void __launch_bounds__(NTHREADS, 1)
contract_tc_kernel(const __grid_constant__ Params P, const __grid_constant__ CUtensorMap fmap) {
    extern __shared__ unsigned char smem_raw[];
    // this CTA's group descriptor, copied out of parameter space once (a
    // runtime index into the parameter struct would otherwise go to the stack)
    __shared__ Group G;
    __shared__ __align__(8) uint64_t bar_full[NSTAGE], bar_empty[NSTAGE], bar_ffull[NFBUF], bar_fempty[NFBUF];
    __shared__ __align__(8) uint64_t bar_seg, bar_drained;
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) int16_t pij[MAXROWS * 4];
    __shared__ int abort_flag_s;
    volatile int& abort_flag = abort_flag_s;
    if (threadIdx.x == 0) G = P.g[blockIdx.y];
    // 1024-byte aligned base: the 128-byte swizzle repeats every 1024 bytes
    const uint32_t raw_u32 = smem_u32(smem_raw);
    unsigned char* smem = smem_raw + (((raw_u32 + 1023u) & ~1023u) - raw_u32);
    const int F_BYTES = f_bytes(P.nshell);
    unsigned char* fbuf = smem;                                              // NFBUF x F_BYTES
    unsigned char* stage_base = smem + NFBUF * F_BYTES;                      // NSTAGE x B operand
    float2* acc = reinterpret_cast<float2*>(stage_base + NSTAGE * STAGE_BYTES);   // Kahan (sum, comp)

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int64_t c0 = (int64_t)blockIdx.x * P.chunks_per_cta;
    const int64_t c1 = min(P.nchunks, c0 + P.chunks_per_cta);
    const int nch = (int)max((int64_t)0, c1 - c0);
    __syncthreads();
    int C = 0;
    for (int t = 0; t < G.ntiles; ++t) C = max(C, G.tile_col[t] + 2 * G.tile_n[t]);

    // ---- set-up ----
    for (int i = tid; i < MAXROWS * 4; i += NTHREADS) pij[i] = P.pair_row[(size_t)G.table_off * 4 + i];
    for (int i = tid; i < G.nslots; i += NTHREADS) acc[i] = make_float2(0.f, 0.f);
    // zero both B stages once: padding shells stay zero
    for (int i = tid; i < NSTAGE * STAGE_BYTES / 16; i += NTHREADS)
        reinterpret_cast<uint4*>(stage_base)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        abort_flag = 0;
        for (int s = 0; s < NSTAGE; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_full[s])), "r"(PWARPS / 2));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_empty[s])), "r"(1));
        }
        for (int b = 0; b < NFBUF; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_ffull[b])), "r"(1));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_fempty[b])), "r"(PWARPS / 2));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_seg)), "r"(1));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_drained)), "r"(PWARPS));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == MMA_WARP) {
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
        // Two groups of 8 warps take alternate chunks (group g: chunks c with
        // c % 2 == g, A / B stage g), so one group's shared-memory loads overlap
        // the other's arithmetic.  Warp w of group g owns TMEM lane quarter w % 4
        // of tiles (w % 8) / 4 and (w % 8) / 4 + 2: one pair row per tile.
        const int rows = G.rows;
        const int nsh = P.nshell;
        const int grp = warp >> 3;
        const int gtid = tid & 255;                   // thread index within the group
        int ri[2], rj[2];
        bool ton[2], ron[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int t = ((warp & 7) >> 2) + 2 * u;  // warp-uniform
            const int row = 128 * t + 32 * q + lane;
            ton[u] = t < G.ntiles;
            ron[u] = ton[u] && row < rows && pij[4 * row] >= 0;
            ri[u] = ron[u] ? (pij[4 * row] & 0xff) : 0;
            rj[u] = ron[u] ? (pij[4 * row] >> 8) : 0;
        }
        const int tl[2] = {(warp & 7) >> 2, ((warp & 7) >> 2) + 2};
        // B writer: shell r, k-group g (voxels 8g..8g+7); 4 nshell <= 256 threads per group
        int ub_r = -1, ub_g = 0;
        if (gtid < nsh * 4) {
            ub_g = (gtid >= nsh) + (gtid >= 2 * nsh) + (gtid >= 3 * nsh);
            ub_r = gtid - ub_g * nsh;
        }
        const int nseg = (nch + SEG - 1) / SEG;
        int seg_count = 0;
        bool failed = false;
        // drain the accumulators of segment seg_count (all warps of both groups)
        auto drain = [&]() -> bool {
            if (!warp_wait(smem_u32(&bar_seg), seg_count & 1)) return false;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // the four warps of this lane quarter take 32-column groups
            // (hi and lo columns of 16 shells) round-robin; one thread adds
            // the hi and lo parts of a (row, shell) and updates its slot
            for (int cg = 32 * ((warp >> 2) & 3); cg < C; cg += 128) {
                uint32_t d[32];
                tmem_ld8(lane_base + (uint32_t)cg, d);
                tmem_ld8(lane_base + (uint32_t)cg + 8u, d + 8);
                tmem_ld8(lane_base + (uint32_t)cg + 16u, d + 16);
                tmem_ld8(lane_base + (uint32_t)cg + 24u, d + 24);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                int t = 0;
                while (t + 1 < G.ntiles && cg >= G.tile_col[t + 1]) ++t;
                if (cg >= G.tile_col[t] + 2 * G.tile_n[t]) continue;
                const int drow = 128 * t + 32 * q + lane;
                // this row's columns l in [lmin, lmax] own slots base + (l - lmin)
                const short4 pr = drow < rows ? *reinterpret_cast<const short4*>(&pij[4 * drow])
                                              : make_short4(-1, 0, -1, 0);
                const int sh0 = col_shell(cg - G.tile_col[t]);
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    const int l = sh0 + e;
                    if (pr.x < 0 || l < pr.y || l > pr.z) continue;
                    const int slot = pr.w + (l - pr.y);
                    const float v = __uint_as_float(d[e]) + __uint_as_float(d[16 + e]);
                    const float2 a = acc[slot];
                    const float y = v - a.y;
                    const float sum = a.x + y;
                    acc[slot] = make_float2(sum, (sum - a.x) - y);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&bar_drained));
            ++seg_count;
            return true;
        };
        for (int c = grp; c < nch; c += 2) {
            if (__any_sync(0xffffffffu, abort_flag != 0)) { failed = true; break; }   // warp-uniform exit
            // segments that ended before this chunk are drained first
            while (seg_count < nseg && (seg_count + 1) * SEG - 1 < c) {
                if (!drain()) { atomicExch(P.err, 2); abort_flag = 1; failed = true; break; }
            }
            if (failed) break;
            const int s = grp;                        // == c & 1
            const int b = c % NFBUF;
            if (!warp_wait(smem_u32(&bar_ffull[b]), (uint32_t)(c / NFBUF) & 1u)) {
                atomicExch(P.err, 1);
                abort_flag = 1;
                failed = true;
                break;
            }
            if (c >= NSTAGE) {
                if (!warp_wait(smem_u32(&bar_empty[s]), ((c - NSTAGE) >> 1) & 1)) {
                    atomicExch(P.err, 1);
                    abort_flag = 1;
                    failed = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            }
            const unsigned char* F = fbuf + (size_t)b * F_BYTES;
            char* Bst = reinterpret_cast<char*>(stage_base) + (size_t)s * STAGE_BYTES;
            // B operand: shells 0..nshell-1 (rows of other shells stay zero)
            if (ub_r >= 0) {
                const float4 a = *reinterpret_cast<const float4*>(F + fchunk(ub_r, 2 * ub_g));
                const float4 e = *reinterpret_cast<const float4*>(F + fchunk(ub_r, 2 * ub_g + 1));
                const float2 x[4] = {make_float2(a.x, a.y), make_float2(a.z, a.w), make_float2(e.x, e.y),
                                     make_float2(e.z, e.w)};
                split_store8(x, Bst + op_off(brow(ub_r, 0), ub_g), Bst + op_off(brow(ub_r, 1), ub_g));
            }
            // A operand: this lane's pair products of both tiles, straight into TMEM
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (!ton[u]) continue;                // warp-uniform
#pragma unroll
                for (int ks = 0; ks < KC / 16; ++ks) {
                    uint32_t h[8], l[8];
#pragma unroll
                    for (int g = 0; g < 4; ++g) {
                        float4 a = make_float4(0.f, 0.f, 0.f, 0.f), e = a;
                        if (ron[u]) {
                            a = *reinterpret_cast<const float4*>(F + fchunk(ri[u], 4 * ks + g));
                            e = *reinterpret_cast<const float4*>(F + fchunk(rj[u], 4 * ks + g));
                        }
                        const float2 p0 = mul2(make_float2(a.x, a.y), make_float2(e.x, e.y));
                        const float2 p1 = mul2(make_float2(a.z, a.w), make_float2(e.z, e.w));
                        h[2 * g] = pack_bf16x2(p0.x, p0.y);
                        h[2 * g + 1] = pack_bf16x2(p1.x, p1.y);
                        const float2 l0 = sub2(p0, make_float2(__uint_as_float(h[2 * g] << 16),
                                                               __uint_as_float(h[2 * g] & 0xFFFF0000u)));
                        const float2 l1 = sub2(p1, make_float2(__uint_as_float(h[2 * g + 1] << 16),
                                                               __uint_as_float(h[2 * g + 1] & 0xFFFF0000u)));
                        l[2 * g] = pack_bf16x2(l0.x, l0.y);
                        l[2 * g + 1] = pack_bf16x2(l1.x, l1.y);
                    }
                    tmem_st8(lane_base + acol(s, tl[u], ks), h);
                    tmem_st8(lane_base + acol(s, tl[u], ks) + 8u, l);
                }
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            // one arrive per warp (the barriers count the 8 warps of a group):
            // the lanes' writes and reads are ordered before lane 0's release
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&bar_full[s]));
                mbar_arrive(smem_u32(&bar_fempty[b]));
            }
        }
        // the remaining segments (the last one ends with the last chunk)
        while (!failed && seg_count < nseg) {
            if (!drain()) { atomicExch(P.err, 2); abort_flag = 1; break; }
        }
    } else if (warp == MMA_WARP) {
        if (lane == 0) {
            // ================= MMA issuer =================
            // Every operand address is computed once: B descriptors per
            // (stage, k-step), A TMEM addresses per (stage, k-step, tile).
            const int ntiles = G.ntiles;
            uint32_t idesc[MAXTILES], dcol[MAXTILES];
#pragma unroll
            for (int t = 0; t < MAXTILES; ++t) {
                idesc[t] = make_idesc(128, 2 * G.tile_n[t]);
                dcol[t] = tmem + (uint32_t)G.tile_col[t];
            }
            const uint32_t sbase = smem_u32(stage_base);
            uint64_t bdesc[NSTAGE][KC / 16];
            uint32_t aad[NSTAGE][KC / 16][MAXTILES];
#pragma unroll
            for (int s = 0; s < NSTAGE; ++s)
#pragma unroll
                for (int ks = 0; ks < KC / 16; ++ks) {
                    bdesc[s][ks] = make_desc(sbase + (uint32_t)(s * STAGE_BYTES) + (uint32_t)(ks * 256), 128, 512);
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
                    const uint64_t bd = s ? bdesc[1][ks] : bdesc[0][ks];
                    const uint32_t acc0 = ks == 0 ? first : 1u;
#pragma unroll
                    for (int t = 0; t < MAXTILES; ++t) {
                        if (t < ntiles) {
                            const uint32_t ahi = s ? aad[1][ks][t] : aad[0][ks][t];
                            asm volatile("{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n"
                                         :: "r"(dcol[t]), "r"(ahi), "l"(bd), "r"(idesc[t]), "r"(acc0));
                            asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, 1;"
                                         :: "r"(dcol[t]), "r"(ahi + 8u), "l"(bd), "r"(idesc[t]));
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
    } else if (warp == TMA_WARP && lane == 0) {
        // ================= field copies (TMA) =================
        const uint32_t fb0 = smem_u32(fbuf);
        const uint32_t tx = (uint32_t)(P.nshell * KC * 4);
        int issued = 0;
        for (int c = 0; c < nch; ++c) {
            const int b = c % NFBUF;
            if (c >= NFBUF && !mbar_wait(smem_u32(&bar_fempty[b]), (uint32_t)(c / NFBUF - 1) & 1u)) {
                atomicExch(P.err, 5);
                abort_flag = 1;
                break;
            }
            if (abort_flag) break;
            const uint32_t fb = smem_u32(&bar_ffull[b]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(fb), "r"(tx) : "memory");
            const int x0 = (int)((c0 + c) * KC);
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                :: "r"(fb0 + (uint32_t)(b * F_BYTES)), "l"(reinterpret_cast<uint64_t>(&fmap)), "r"(x0), "r"(0),
                   "r"(fb)
                : "memory");
            issued = c + 1;
        }
        // copies still in flight (only after an abort) land before the CTA exits
        for (int c = max(0, issued - NFBUF); c < issued; ++c)
            mbar_wait(smem_u32(&bar_ffull[c % NFBUF]), (uint32_t)(c / NFBUF) & 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    // partial sums of this CTA's triangles
    if (!abort_flag) {
        for (int i = tid; i < G.nslots; i += NTHREADS) {
            const int t = P.slot_tri[(size_t)blockIdx.y * P.maxslots + i];
            if (t >= 0) P.partials[(size_t)blockIdx.x * P.ntri + t] = (double)acc[i].x - (double)acc[i].y;
        }
    }
    if (warp == MMA_WARP) {
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
    std::vector<int16_t> pair_row;
    std::vector<int32_t> slot_tri;
    std::vector<char> image;      // pair_row | slot_tri, each 256-byte aligned (device layout)
    const void* image_src = nullptr;   // page-locked copy of `image` (or image.data())
    size_t off_stri = 0;
    size_t smem = 0;
    bool ok = false;
    bool invalid = false;         // the triangle list itself is malformed (vs. unsupported)
    char why[160] = {0};
};

static size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

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
    std::map<std::pair<int, int>, std::map<int, int>> pairs;   // (i,j) -> {l: t}
    for (int t = 0; t < ntri; ++t) {
        int a = tri_host[t], b = tri_host[ntri + t], c = tri_host[2 * ntri + t];
        if (a < 0 || b < 0 || c < 0 || a >= nshell || b >= nshell || c >= nshell) {
            snprintf(hp->why, sizeof(hp->why), "triangle %d has a slot outside [0, %d)", t, nshell);
            return hp;
        }
        int v[3] = {a, b, c};
        std::sort(v, v + 3);
        if (!pairs[{v[2], v[1]}].emplace(v[0], t).second) {
            snprintf(hp->why, sizeof(hp->why), "triangle %d repeats an earlier triangle", t);
            hp->invalid = true;
            return hp;
        }
    }
    std::vector<std::pair<int, int>> order;
    for (auto& kv : pairs) order.push_back(kv.first);
    std::sort(order.begin(), order.end(), [](const std::pair<int, int>& x, const std::pair<int, int>& y) {
        return x.second != y.second ? x.second < y.second : x.first < y.first;
    });
    const int nrows = (int)order.size();
    // each row owns the Kahan slots of columns [lmin, lmax] of its triangles
    auto row_slots = [&](const std::pair<int, int>& key) {
        const auto& m = pairs[key];
        return m.rbegin()->first - m.begin()->first + 1;
    };
    // N of each 128-row tile: the largest shell column it needs, rounded to 16;
    // and the number of Kahan slots it holds
    std::vector<int> tile_n, tile_slots;
    for (int r0 = 0; r0 < nrows; r0 += 128) {
        int maxl = 0, ns = 0;
        for (int r = r0; r < std::min(nrows, r0 + 128); ++r) {
            maxl = std::max(maxl, pairs[order[r]].rbegin()->first);
            ns += row_slots(order[r]);
        }
        tile_n.push_back(((maxl + 1) + 15) / 16 * 16);
        tile_slots.push_back(ns);
    }
    const int ntiles_all = (int)tile_n.size();
    const size_t fixed = (size_t)fixed_smem(nshell);
    const int budget = (int)((227 * 1024 - 8192 - fixed) / sizeof(float2));
    // Greedy grouping into CTA groups: at most 4 tiles, MAXCOLS accumulator
    // columns (2N per tile; TMEM also holds 2 stages x 4 tiles x 32 A columns)
    // and `budget` Kahan slots in shared memory.
    std::vector<int> group_first;
    {
        int cur_tiles = 0, cur_cols = 0, cur_slots = 0;
        for (int t = 0; t < ntiles_all; ++t) {
            if (tile_slots[t] > budget) {
                snprintf(hp->why, sizeof(hp->why), "a 128-row tile holds %d triangles (limit %d)", tile_slots[t], budget);
                return hp;
            }
            if (cur_tiles == 0 || cur_tiles == MAXTILES || cur_cols + 2 * tile_n[t] > MAXCOLS ||
                cur_slots + tile_slots[t] > budget) {
                group_first.push_back(t);
                cur_tiles = cur_cols = cur_slots = 0;
            }
            ++cur_tiles;
            cur_cols += 2 * tile_n[t];
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
    hp->pair_row.assign((size_t)ngroups * MAXROWS * 4, (int16_t)0);
    for (size_t r = 0; r < (size_t)ngroups * MAXROWS; ++r) hp->pair_row[4 * r] = -1;
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
            col += 2 * G.tile_n[t];
            if (G.tile_n[t] > MAXB) {
                snprintf(hp->why, sizeof(hp->why), "BF16x3 contraction supports at most %d shells", MAXB);
                return hp;
            }
        }
        G.ncols = pow2_cols(col + NSTAGE * MAXTILES * ACOLS);
        if (G.ncols > 512) {
            snprintf(hp->why, sizeof(hp->why), "BF16x3 tile columns exceed TMEM");
            return hp;
        }
        for (int r = 0; r < G.rows; ++r) {
            auto key = order[r0 + r];
            const auto& m = pairs[key];
            const int lmin = m.begin()->first, lmax = m.rbegin()->first;
            int16_t* pr = &hp->pair_row[((size_t)G.table_off + r) * 4];
            pr[0] = (int16_t)(key.first | (key.second << 8));
            pr[1] = (int16_t)lmin;
            pr[2] = (int16_t)lmax;
            pr[3] = (int16_t)gslots[g].size();
            for (int l = lmin; l <= lmax; ++l) {
                auto it = m.find(l);
                gslots[g].push_back(it == m.end() ? -1 : it->second);
            }
        }
        G.nslots = (int)gslots[g].size();
        if (G.nslots > 32767) {
            snprintf(hp->why, sizeof(hp->why), "too many triangles in one CTA group");
            return hp;
        }
        maxslots = std::max(maxslots, G.nslots);
    }
    P.maxslots = maxslots;
    hp->slot_tri.assign((size_t)ngroups * maxslots, -1);
    for (int g = 0; g < ngroups; ++g)
        for (size_t i = 0; i < gslots[g].size(); ++i) hp->slot_tri[(size_t)g * maxslots + i] = gslots[g][i];
    hp->smem = fixed + sizeof(float2) * (size_t)maxslots;
    hp->off_stri = al256(hp->pair_row.size() * 2);
    hp->image.assign(hp->off_stri + al256(hp->slot_tri.size() * 4), 0);
    memcpy(hp->image.data(), hp->pair_row.data(), hp->pair_row.size() * 2);
    memcpy(hp->image.data() + hp->off_stri, hp->slot_tri.data(), hp->slot_tri.size() * 4);
    hp->image_src = pinned_copy(hp->image.data(), hp->image.size());
    if (hp->image_src == nullptr) hp->image_src = hp->image.data();
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

}  // namespace tc

size_t contract_tc_ws(int64_t nvox, int nshell, int ntri) {
    // tables (bounded by the largest plan: 8 groups of 512 rows, slots <= ntri
    // + one gap slot per row and shell) + partials + error word
    (void)nshell;
    const size_t rows = (size_t)tc::MAXGROUPS * tc::MAXROWS;
    const size_t tables = rows * 4 * 2 + (size_t)tc::MAXGROUPS * ((size_t)ntri + tc::MAXROWS * tc::MAXB) * 4 + 4096;
    const int64_t nchunks = (nvox + tc::KC - 1) / tc::KC;
    const size_t gx = (size_t)std::min<int64_t>(std::max<int64_t>(nchunks, 1), 1024);
    return tc::al256(tables) + tc::al256(gx * (size_t)std::max(ntri, 1) * sizeof(double)) + 256;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

int contract_tc_impl(const float* fields, int64_t nvox, int nshell, const int32_t* tri, const int32_t* tri_host,
                     int ntri, double* bsum, void* ws, size_t ws_bytes, cudaStream_t st) {
    using namespace tc;
    PYSPEC_CHECK_ARG(tri_host != nullptr, "the BF16x3 contraction needs the host copy of the triangle list");
    PYSPEC_CHECK_ARG(nvox % 4 == 0, "BF16x3 contraction needs N^3 divisible by 4");
    PYSPEC_CHECK_ARG(nvox / KC + 1 < (int64_t)INT32_MAX / KC, "BF16x3 contraction supports N^3 < 2^31");
    PYSPEC_CHECK_ARG(((uintptr_t)fields & 15) == 0, "fields must be 16-byte aligned");
    HostPlan* hp = get_plan(nshell, tri_host, ntri);
    if (!hp->ok) {
        set_error("%s", hp->why);
        return hp->invalid ? PYSPEC_E_INVALID : PYSPEC_E_UNSUPPORTED;
    }
    const size_t need = contract_tc_ws(nvox, nshell, ntri);
    if (ws_bytes < need) {
        set_error("contract workspace %zu bytes < required %zu", ws_bytes, need);
        return PYSPEC_E_WORKSPACE;
    }
    EncodeTiledFn enc = encode_tiled();
    if (enc == nullptr) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return PYSPEC_E_CUDA;
    }
    // fields as a 2D tensor: x = voxel (contiguous), y = shell row; one box =
    // all nshell rows x 32 voxels, 128-byte swizzle (conflict-free row reads)
    CUtensorMap fmap;
    const cuuint64_t gdim[2] = {(cuuint64_t)nvox, (cuuint64_t)nshell};
    const cuuint64_t gstride[1] = {(cuuint64_t)nvox * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)KC, (cuuint32_t)nshell};
    const cuuint32_t estride[2] = {1, 1};
    CUresult cr = enc(&fmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(fields), gdim, gstride, box,
                      estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", (int)cr);
        return PYSPEC_E_CUDA;
    }
    char* w = reinterpret_cast<char*>(ws);
    size_t off = 0;
    int* d_err = reinterpret_cast<int*>(w + off); off += 256;      // status word first
    char* d_image = w + off;
    const int16_t* d_rows = reinterpret_cast<const int16_t*>(d_image);
    const int32_t* d_stri = reinterpret_cast<const int32_t*>(d_image + hp->off_stri);
    off += hp->image.size();
    off = al256(off);
    const int64_t nchunks = (nvox + KC - 1) / KC;
    const int gx = grid_x(nchunks, hp->base.ngroups);
    double* partials = reinterpret_cast<double*>(w + off);
    if (off + al256((size_t)gx * ntri * sizeof(double)) > ws_bytes) {
        set_error("contract workspace too small for %d CTAs", gx);
        return PYSPEC_E_WORKSPACE;
    }
    PYSPEC_CUDA(cudaMemcpyAsync(d_image, hp->image_src, hp->image.size(), cudaMemcpyHostToDevice, st));
    PYSPEC_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    PYSPEC_CUDA(cudaMemsetAsync(partials, 0, (size_t)gx * ntri * sizeof(double), st));
    Params P = hp->base;
    P.V = nvox;
    P.nchunks = nchunks;
    P.chunks_per_cta = (nchunks + gx - 1) / gx;
    P.pair_row = d_rows;
    P.slot_tri = d_stri;
    P.partials = partials;
    P.err = d_err;
    PYSPEC_TRY(allow_smem((const void*)contract_tc_kernel, hp->smem));
    contract_tc_kernel<<<dim3(gx, P.ngroups), NTHREADS, hp->smem, st>>>(P, fmap);
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    (void)tri;
    return reduce_partials_launch(partials, gx, ntri, bsum, st);
}

}  // namespace pyspec
