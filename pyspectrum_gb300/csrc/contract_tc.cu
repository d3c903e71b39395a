// Triangle contraction on the 5th-generation tensor cores (tcgen05), split-BF16.
//
// bsum[t] = sum_v F_i(v) F_j(v) F_l(v) for triangles t = (i >= j >= l).
// Each triangle is (pair (i,j), column l).  The kernel evaluates the GEMM
//   D[p, c] = sum_v P_p(v) F_c(v),   P_p = F_i F_j  (pair p = (i, j))
// with pair rows on M (tiles of 128) and shells on N, the voxels on K.  Both
// operands are split into bf16 hi + lo parts (x = hi + lo, lo = x - hi).  The
// B operand holds the hi and lo rows of the shells interleaved in blocks of 8
// (rows [16b, 16b+8) = hi of shells [8b, 8b+8), the next 8 rows = lo).  A
// tcgen05.mma with M = 128, K = 16 issues every 45 cycles whatever its N up
// to N = 80 (N / 2 cycles from N = 128; measured), so the kernel issues as
// few as TMEM allows:
//   wide form: per tile and k-step two MMAs (A_hi, then A_lo) against all
//     2N interleaved B rows, so the accumulator holds A_x B_hi and A_x B_lo
//     side by side (all four products), summed when drained;
//   narrow form (when 2N columns per tile do not fit): three MMAs (A_hi B_hi,
//     A_lo B_hi, A_hi B_lo; A_lo B_lo, 2^-16 of the rest, is dropped) into
//     N columns, B_hi and B_lo read through descriptors that skip the other
//     part's 8-row blocks.
// Per tile the MMAs issue back to back with no branch between them (a
// data-dependent branch in the sequence slowed the issue by ~30 %).
//
// CTA layout (1 CTA per SM, persistent over a contiguous voxel range):
//   warps 0-15 (512 threads): producers, all on every chunk of KC = 32
//     voxels.  Warp w owns TMEM lane quarter w % 4 of the tile pair
//     (w / 4) % 2 in k-step w / 8.  Each thread forms 4 voxels of 8 pair rows
//     (two slots of four rows that share their shells g; 4 rows where the
//     tile pair has one tile), splits the products into hi/lo bf16 and writes
//     them straight into TMEM (tcgen05.st, 16x256b shape) as the MMA's A
//     operand; threads < 4*nshell
//     write the B operand (the shells' hi and lo parts) to shared memory in
//     the UMMA K-major core-matrix layout.  Then `full[stage]` and
//     `fempty[buffer]` are signalled (one arrival per warp).
//   warp 16, lane 0: issues tcgen05.mma (A from TMEM, B from shared memory)
//     and tcgen05.commit to `empty[stage]`.
//   warp 17, lane 0: streams the fields: one TMA tensor copy per chunk
//     (nshell rows x 32 floats, 128-byte swizzle) into a ring of NFBUF
//     buffers, completing on `ffull[buffer]`.
//   Every 2^seg_log2 chunks (32; 8 with PYSPEC_CONTRACT_FINE_DRAIN) the
//   accumulators are drained: the MMA thread commits to
//   `seg`, the producers add the TMEM accumulators into Kahan-compensated
//   float32 sums per triangle in shared memory and arrive on `drained`; the
//   next MMA restarts the accumulators.  At the end each CTA writes one float64
//   partial per triangle; a second kernel adds the partials in a fixed order.
// TMEM columns: [0, C) accumulators (2N or N per tile); then two A stages of 32
// columns per tile.  Every mbarrier wait is bounded; on timeout the kernel
// records an error code, stops issuing work, waits (bounded) for its copies
// and MMAs in flight, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <string.h>
#include <algorithm>
#include <array>
#include <map>
#include <mutex>
#include <vector>
#include "contract.cuh"

namespace pyspec {

namespace tc {

constexpr int KC = 32;               // voxels per chunk (two k-steps of 16)
constexpr int MAXROWS = 512;         // pair rows per CTA group (4 M-tiles)
constexpr int MAXB = 64;             // shells
constexpr int BROWS = 2 * MAXB;      // B operand rows: hi and lo parts of shells 0..63
constexpr int NSTAGE = 2;
constexpr int NPROD = 512;           // producer threads (warps 0-15): 2 k-steps x 2 tile pairs x 4 lane quarters
constexpr int PWARPS = NPROD / 32;
constexpr int MMA_WARP = PWARPS;
constexpr int TMA_WARP = PWARPS + 1;
constexpr int NTHREADS = NPROD + 64; // + the MMA warp + the copy warp
constexpr int SEG_LOG2 = 5;          // default: drain every 32 chunks (the TMEM float32 accumulation length sets the error: 128 chunks gave a bf16x3 median error of 8e-6 vs FP64, 64 gave 4e-6)
constexpr int SEG_LOG2_FINE = 3;     // PYSPEC_CONTRACT_FINE_DRAIN: every 8 chunks
constexpr int MAXGROUPS = 8;
constexpr int MAXTILES = 4;
constexpr int RT_PER_GROUP = 64;     // producer row threads per group: 2 tile pairs x 4 lane quarters x 8
constexpr int RT_WORDS = 3;          // int32 words per row thread in the row-thread table
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
    int wide;              // 1: two MMAs per tile and k-step into 2N columns; 0: three into N
    int tile_n[MAXTILES];  // N of each tile in shells (wide: multiple of 8; narrow: of 16; <= 64)
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
    // [group][64][3] per producer row thread: word 0 = i0 | i1 << 8, words
    // 1 and 2 = the four shells g_{u,y} of slot u (byte y); slot u holds the
    // pair rows (i_u, g_{u,y}), y = 0..3
    const int32_t* rt_tab;
    const int32_t* slot_tri;     // [group][maxslots] triangle index of each slot (-1: unused)
    double* partials;            // [gridDim.x][ntri]
    int* err;
    int seg_log2;                // accumulators drained every 2^seg_log2 chunks
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

// B operand row of shell s, part p (0 = hi, 1 = lo): hi/lo interleaved in blocks of 8
__host__ __device__ __forceinline__ int brow(int s, int p) { return ((s >> 3) << 4) | (p << 3) | (s & 7); }

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

// tcgen05.st 16x256b.x2: 16 TMEM lanes x 16 columns, two repeats of 8
// columns; in repeat k thread t writes (lane t/4, columns 8k + 2(t%4) + {0,1})
// from v[4k], v[4k+1] and (lane t/4 + 8, same columns) from v[4k+2], v[4k+3]
// (layout checked on the GPU for the x1 and x4 forms of the shape)
__device__ __forceinline__ void tmem_st16x256_x2(uint32_t addr, const uint32_t* v) {
    asm volatile("tcgen05.st.sync.aligned.16x256b.x2.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
                 :: "r"(addr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]),
                    "r"(v[7])
                 : "memory");
}

// hi/lo bf16 parts of two floats (packed pairs)
__device__ __forceinline__ void split2(float2 p, uint32_t& h, uint32_t& l) {
    h = pack_bf16x2(p.x, p.y);
    const float2 lv = sub2(p, make_float2(__uint_as_float(h << 16), __uint_as_float(h & 0xFFFF0000u)));
    l = pack_bf16x2(lv.x, lv.y);
}

// hi and third parts of two floats, for the residual pass: x = hi + lo + res
// with hi = bf16(x), lo = bf16(x - hi), res = bf16(x - hi - lo); both
// differences are exact in float32, so hi + lo + res carries ~24 bits.
__device__ __forceinline__ void split2_res(float2 p, uint32_t& h, uint32_t& r) {
    h = pack_bf16x2(p.x, p.y);
    const float2 lv = sub2(p, make_float2(__uint_as_float(h << 16), __uint_as_float(h & 0xFFFF0000u)));
    const uint32_t l = pack_bf16x2(lv.x, lv.y);
    const float2 rv = sub2(lv, make_float2(__uint_as_float(l << 16), __uint_as_float(l & 0xFFFF0000u)));
    r = pack_bf16x2(rv.x, rv.y);
}

// split_store8 for the residual pass: the hi part and the third part.
__device__ __forceinline__ void split_store8_res(const float2* x, char* hi, char* res) {
    uint32_t h[4], r[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) split2_res(x[q], h[q], r[q]);
    *reinterpret_cast<uint4*>(hi) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4*>(res) = make_uint4(r[0], r[1], r[2], r[3]);
}

// One slot of a producer thread into TMEM for its k-step: the products
// fi * fj[y] (4 voxels each) of its four pair rows y = 0..3, which sit at
// lanes x + 8y of the lane quarter (`addr` = quarter base + the tile's A
// columns of this stage and k-step: 8 hi then 8 lo columns).  Rows 0, 1 go
// to the 16-lane block [0, 16), rows 2, 3 to [16, 32); repeat 0 of the x2
// shape carries the hi parts, repeat 1 the lo parts; lane a of the thread
// group owns columns 2a, 2a + 1 of each repeat (voxels 4a .. 4a + 3).
// RES (the residual pass): the lo columns receive the third part instead.
template <bool RES = false>
__device__ __forceinline__ void store_slot(float4 fi, const float4* fj, uint32_t addr) {
#pragma unroll
    for (int blk = 0; blk < 2; ++blk) {
        uint32_t v[8];
#pragma unroll
        for (int yy = 0; yy < 2; ++yy) {
            const float4 f = fj[2 * blk + yy];
            const float2 p0 = mul2(make_float2(fi.x, fi.y), make_float2(f.x, f.y));
            const float2 p1 = mul2(make_float2(fi.z, fi.w), make_float2(f.z, f.w));
            if constexpr (RES) {
                split2_res(p0, v[2 * yy], v[4 + 2 * yy]);
                split2_res(p1, v[2 * yy + 1], v[4 + 2 * yy + 1]);
            } else {
                split2(p0, v[2 * yy], v[4 + 2 * yy]);
                split2(p1, v[2 * yy + 1], v[4 + 2 * yy + 1]);
            }
        }
        tmem_st16x256_x2(addr + ((uint32_t)(16 * blk) << 16), v);
    }
}

// The MMAs of one chunk: per k-step and tile, A_hi then A_lo against the B
// stage (wide form: all 2N interleaved rows), plus A_hi against B_lo (narrow
// form: B_lo blocks 512 bytes after the B_hi blocks).  `abase` = TMEM address
// of the stage's A columns (tile t, k-step ks at + 32 t + 16 ks), `bd0` = the
// stage's B descriptor (k-step ks at + 256 bytes).  `first` == 0 starts each
// accumulator afresh.
// RES (the residual pass, narrow form only): A_res (held in the lo columns)
// against B_hi, then A_hi against B_res (held in the B lo rows).
template <bool WIDE, int NT, bool RES = false>
__device__ __forceinline__ void issue_chunk(const uint32_t (&dcol)[MAXTILES], uint32_t abase, uint64_t bd0,
                                            const uint32_t (&idesc)[MAXTILES], uint32_t first) {
    static_assert(!(RES && WIDE), "the residual pass uses the narrow form");
#pragma unroll
    for (int ks = 0; ks < KC / 16; ++ks) {
        const uint32_t acc0 = ks == 0 ? first : 1u;
        const uint64_t bd = bd0 + (uint64_t)((ks * 256) >> 4);
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            const uint32_t ahi = abase + (uint32_t)(t * ACOLS + ks * 16);
            if constexpr (RES) {
                asm volatile("{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n"
                             :: "r"(dcol[t]), "r"(ahi + 8u), "l"(bd), "r"(idesc[t]), "r"(acc0));
                asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, 1;"
                             :: "r"(dcol[t]), "r"(ahi), "l"(bd + (uint64_t)(512 >> 4)), "r"(idesc[t]));
                continue;
            }
            asm volatile("{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n"
                         :: "r"(dcol[t]), "r"(ahi), "l"(bd), "r"(idesc[t]), "r"(acc0));
            asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, 1;"
                         :: "r"(dcol[t]), "r"(ahi + 8u), "l"(bd), "r"(idesc[t]));
            if constexpr (!WIDE)
                asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, 1;"
                             :: "r"(dcol[t]), "r"(ahi), "l"(bd + (uint64_t)(512 >> 4)), "r"(idesc[t]));
        }
    }
}

__device__ __forceinline__ float4 lds4(const unsigned char* base, uint32_t off) {
    return *reinterpret_cast<const float4*>(base + off);
}

template <bool RES>
__global__ void __launch_bounds__(NTHREADS, 1)
contract_tc_kernel(const __grid_constant__ Params P, const __grid_constant__ CUtensorMap fmap) {
    // RES: the residual pass of the 6-product form, a separate instantiation
    // so the 4-product pass keeps its branch-free producer and MMA sequences
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
    for (int t = 0; t < G.ntiles; ++t) C = max(C, G.tile_col[t] + (G.wide ? 2 : 1) * G.tile_n[t]);

    // ---- set-up ----
    for (int i = tid; i < MAXROWS * 4; i += NTHREADS) pij[i] = P.pair_row[(size_t)G.table_off * 4 + i];
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
        for (int b = 0; b < NFBUF; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_ffull[b])), "r"(1));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_fempty[b])), "r"(PWARPS));
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
        // All 16 warps work on every chunk (A / B stage c % 2).  Warp w owns
        // TMEM lane quarter q = w % 4 of the tile pair p = (w / 4) % 2 (tiles
        // 2p and 2p + 1) in k-step w / 8.  Lane 4x + a: x is one of the warp's
        // 8 row threads, each with two slots; slot u lies in tile 2p + u and
        // holds the pair rows (i_u, J_u + y), y = 0..3, at TMEM lanes
        // 32q + x + 8y.  Lane a forms voxels 4a .. 4a+3 of the warp's 16-voxel
        // k-step of those 8 rows.  The plan gives both slots the same run J
        // wherever it can, so a thread loads 6 field pieces for its 32
        // products.  With two A stages a chunk's A can be written only after
        // the MMAs of the chunk two back complete, so the tensor pipe stays
        // busy only if one chunk is produced within one chunk's MMA time:
        // spreading each chunk over all 16 warps (half a chunk's k-steps per
        // warp) keeps the production of a chunk short.
        const int rows = G.rows;
        const int nsh = P.nshell;
        const int gtid = tid;
        const int tp = (warp >> 2) & 1;
        const int kstep = (warp >> 3) & 1;            // warp-uniform
        const uint32_t kx = kstep ? 64u : 0u;
        const bool tp_on = 2 * tp < G.ntiles;         // warp-uniform
        const bool slot1_on = 2 * tp + 1 < G.ntiles;  // warp-uniform (a 3-tile plan has no tile 3)
        const int ax = lane & 3;
        const int32_t* rtw = P.rt_tab + ((size_t)blockIdx.y * RT_PER_GROUP + tp * 32 + q * 8 + (lane >> 2)) * RT_WORDS;
        const uint32_t code = (uint32_t)rtw[0];
        const uint32_t gs0 = (uint32_t)rtw[1], gs1 = (uint32_t)rtw[2];
        // byte offset of this lane's 16-byte piece of field row r in the
        // warp's k-step (k-step 1: XOR 64, the other half of the 128-byte
        // swizzled row)
        auto foff = [&](int r) {
            r = min(r, nsh - 1);
            return (uint32_t)(r * 128 + ((ax ^ (r & 7)) << 4)) ^ kx;
        };
        const uint32_t oi0 = foff((int)(code & 0xffu)), oi1 = foff((int)((code >> 8) & 0xffu));
        const bool reload = gs1 != gs0;
        uint32_t oj0[4];
#pragma unroll
        for (int y = 0; y < 4; ++y) oj0[y] = foff((int)((gs0 >> (8 * y)) & 0xffu));
        // B writer: shell r, k-group g (voxels 8g..8g+7); 4 nshell <= 512 threads
        int ub_r = -1, ub_g = 0;
        const bool b_warp = (warp * 32) < nsh * 4;    // warp-uniform
        if (gtid < nsh * 4) {
            ub_g = (gtid >= nsh) + (gtid >= 2 * nsh) + (gtid >= 3 * nsh);
            ub_r = gtid - ub_g * nsh;
        }
        const int seg_len = 1 << P.seg_log2;
        const int nseg = (nch + seg_len - 1) >> P.seg_log2;
        int seg_count = 0;
        bool failed = false;
        // drain the accumulators of segment seg_count (all warps of both groups)
        auto drain = [&]() -> bool {
            if (!warp_wait(smem_u32(&bar_seg), seg_count & 1)) return false;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // the four warps of this lane quarter take 16-column groups
            // round-robin (wide form: the hi and lo columns of 8 shells;
            // narrow: 16 shells); one thread adds a (row, shell) into its slot
            const bool wide = G.wide != 0;
            for (int cg = 16 * ((warp >> 2) & 3); cg < C; cg += 64) {
                uint32_t d[16];
                tmem_ld8(lane_base + (uint32_t)cg, d);
                tmem_ld8(lane_base + (uint32_t)cg + 8u, d + 8);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                int t = 0;
                while (t + 1 < G.ntiles && cg >= G.tile_col[t + 1]) ++t;
                const int drow = 128 * t + 32 * q + lane;
                // this row's columns l in [lmin, lmax] own slots base + (l - lmin)
                const short4 pr = drow < rows ? *reinterpret_cast<const short4*>(&pij[4 * drow])
                                              : make_short4(-1, 0, -1, 0);
                const int sh0 = wide ? (cg - G.tile_col[t]) >> 1 : cg - G.tile_col[t];
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    const int l = sh0 + e;
                    if ((wide && e >= 8) || pr.x < 0 || l < pr.y || l > pr.z) continue;
                    const int slot = pr.w + (l - pr.y);
                    const float v = wide ? __uint_as_float(d[e]) + __uint_as_float(d[e + 8]) : __uint_as_float(d[e]);
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
        for (int c = 0; c < nch; ++c) {
            if (__any_sync(0xffffffffu, abort_flag != 0)) { failed = true; break; }   // warp-uniform exit
            const int s = c & 1;
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
                if constexpr (RES) split_store8_res(x, Bst + op_off(brow(ub_r, 0), ub_g), Bst + op_off(brow(ub_r, 1), ub_g));
                else split_store8(x, Bst + op_off(brow(ub_r, 0), ub_g), Bst + op_off(brow(ub_r, 1), ub_g));
            }
            // A operand: this thread's 8 (or 4) pair rows x 4 voxels of its k-step, straight into TMEM
            if (tp_on) {
                const float4 fi0 = lds4(F, oi0);
                // the second slot's pair shell is loaded before the first slot's
                // TMEM stores, which the compiler may not move loads across
                const float4 fi1 = slot1_on ? lds4(F, oi1) : fi0;
                float4 fj[4];
#pragma unroll
                for (int y = 0; y < 4; ++y) fj[y] = lds4(F, oj0[y]);
                store_slot<RES>(fi0, fj, lane_base + acol(s, 2 * tp, kstep));
                if (slot1_on) {
                    if (reload) {
#pragma unroll
                        for (int y = 0; y < 4; ++y) fj[y] = lds4(F, foff((int)((gs1 >> (8 * y)) & 0xffu)));
                    }
                    store_slot<RES>(fi1, fj, lane_base + acol(s, 2 * tp + 1, kstep));
                }
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            // B writes (generic proxy) made visible to the MMA (async proxy):
            // only the warps that hold B writers need the fence
            if (b_warp) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            // one arrive per warp (the barriers count the 16 producer warps):
            // the lanes' writes and reads are ordered before lane 0's release
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&bar_full[s]));
                mbar_arrive(smem_u32(&bar_fempty[b]));
            }
            // a segment that ended before this chunk is drained after the
            // chunk is produced: its MMAs (which wait for the drain) can then
            // start as soon as the drain ends
            while (seg_count < nseg && ((seg_count + 1) << P.seg_log2) - 1 < c) {
                if (!drain()) { atomicExch(P.err, 2); abort_flag = 1; failed = true; break; }
            }
            if (failed) break;
        }
        // the remaining segments (the last one ends with the last chunk)
        while (!failed && seg_count < nseg) {
            if (!drain()) { atomicExch(P.err, 2); abort_flag = 1; break; }
        }
    } else if (warp == MMA_WARP) {
        if (lane == 0) {
            // ================= MMA issuer =================
            // Operand addresses: per chunk a stage base plus constant offsets.
            const int ntiles = G.ntiles;
            const bool wide = G.wide != 0;
            uint32_t idesc[MAXTILES], dcol[MAXTILES];
#pragma unroll
            for (int t = 0; t < MAXTILES; ++t) {
                idesc[t] = make_idesc(128, (wide ? 2 : 1) * G.tile_n[t]);
                dcol[t] = tmem + (uint32_t)G.tile_col[t];
            }
            const uint32_t sbase = smem_u32(stage_base);
            // B descriptor of stage 0, k-step 0: wide form all rows (8-row
            // blocks 512 bytes apart); narrow form the hi blocks only (1024
            // apart; the lo blocks are 512 bytes further)
            const uint64_t bdesc0 = make_desc(sbase, 128, wide ? 512 : 1024);
            // tile count 2, 3 or 4 and the form select one branch-free sequence
            const int mode = (wide ? 3 : 0) + (ntiles == 2 ? 0 : ntiles == 3 ? 1 : 2);
            int seg_count = 0;
            const int seg_mask = (1 << P.seg_log2) - 1;
            uint32_t first = 0;   // 0: the next MMA of each tile overwrites its accumulator
            for (int c = 0; c < nch; ++c) {
                const int s = c & 1;
                if (!mbar_wait(smem_u32(&bar_full[s]), (c >> 1) & 1)) { atomicExch(P.err, 3); abort_flag = 1; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                // one branch-free MMA sequence per (form, tile count): a
                // branch between the MMAs of a chunk slows their issue by ~30 %
                const uint32_t abase = tmem + acol(s, 0, 0);
                const uint64_t bd0 = bdesc0 + (uint64_t)((s * STAGE_BYTES) >> 4);
                if constexpr (RES) {             // narrow form only (the host sets it)
                    switch (ntiles) {
                        case 2: issue_chunk<false, 2, true>(dcol, abase, bd0, idesc, first); break;
                        case 3: issue_chunk<false, 3, true>(dcol, abase, bd0, idesc, first); break;
                        default: issue_chunk<false, 4, true>(dcol, abase, bd0, idesc, first); break;
                    }
                } else {
                    switch (mode) {
                        case 0: issue_chunk<false, 2>(dcol, abase, bd0, idesc, first); break;
                        case 1: issue_chunk<false, 3>(dcol, abase, bd0, idesc, first); break;
                        case 2: issue_chunk<false, 4>(dcol, abase, bd0, idesc, first); break;
                        case 3: issue_chunk<true, 2>(dcol, abase, bd0, idesc, first); break;
                        case 4: issue_chunk<true, 3>(dcol, abase, bd0, idesc, first); break;
                        default: issue_chunk<true, 4>(dcol, abase, bd0, idesc, first); break;
                    }
                }
                first = 1u;
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                             :: "r"(smem_u32(&bar_empty[s])) : "memory");
                if (((c + 1) & seg_mask) == 0 || c + 1 == nch) {
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
// Deep-chunk form: 64 voxels (four k-steps) per hand-over, for plans of 2 or
// 3 tiles that are all wide.  Each producer warp, the MMA thread and the
// copy thread pay their per-chunk synchronisation (waits, fences, arrivals,
// commit) once per 64 voxels instead of once per 32 -- that fixed cost, not
// the work, bounds the 32-voxel kernel.  TMEM keeps the same layout (A_hi of
// a tile and stage: 4 k-steps x 8 columns = 32), the A_lo parts go to shared
// memory (16 KB per tile and stage, K-major core matrices, 64 k per 8-row
// block) and the MMAs read them through descriptors.  Per tile and k-step:
// A_hi (TMEM) and A_lo (shared memory) against all 2N interleaved B rows.
// ---------------------------------------------------------------------------
constexpr int KC64 = 64;
constexpr int STAGE64_BYTES = BROWS * KC64 * 2;     // B operand of one stage: 16 KB
constexpr int ALO_TILE_BYTES = 128 * KC64 * 2;      // A_lo of one tile and stage: 16 KB
constexpr int SEG64_SHIFT = 1;                       // drains every 2^(seg_log2 - 1) deep chunks (same voxels)
constexpr int kDeepSmemLimit = 232448 - 6144;        // dynamic bytes: the 227 KB opt-in less the static arrays
constexpr int NBW64 = 2;                             // B-operand writer warps, after the MMA and copy warps
constexpr int BW0 = PWARPS + 2;
constexpr int NTHREADS64 = NTHREADS + 32 * NBW64;

// A_lo blocks in shared memory: tiles 0 and 1 (tile 2 keeps its A_lo in
// TMEM, in the columns of the absent tile 3)
__host__ __device__ constexpr int alo_smem_tiles(int ntiles) { return ntiles < 2 ? ntiles : 2; }

// dynamic shared memory before the Kahan slots, for nfbuf field buffers of two halves
__host__ __device__ constexpr int fixed_smem64(int nshell, int ntiles, int nfbuf) {
    return 1024 + nfbuf * 2 * f_bytes(nshell) + NSTAGE * STAGE64_BYTES + NSTAGE * alo_smem_tiles(ntiles) * ALO_TILE_BYTES;
}

// K-major no-swizzle operand with 64 k per row block: core matrix (r/8, g) at
// (r/8)*1024 + g*128, row r%8 at 16 B
__device__ __forceinline__ int op_off64(int r, int kgroup) { return (r >> 3) * 1024 + kgroup * 128 + (r & 7) * 16; }

// tcgen05.st 16x256b.x1: repeat 0 of the x2 shape (8 columns)
__device__ __forceinline__ void tmem_st16x256_x1(uint32_t addr, const uint32_t* v) {
    asm volatile("tcgen05.st.sync.aligned.16x256b.x1.b32 [%0], {%1,%2,%3,%4};"
                 :: "r"(addr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]) : "memory");
}

// One slot of a producer thread for one k-step: the hi parts of its four
// rows into TMEM (lanes x + 8y of the quarter, 8 columns at `addr`), the lo
// parts into the tile's A_lo block (`alo` = this thread's address for row
// y = 0; row y lies in the next 8-row block, y * 1024 bytes further).
// RES (the residual pass of the 6-product form): the third parts take the
// place of the lo parts.
template <bool RES = false>
__device__ __forceinline__ void store_slot64(float4 fi, const float4* fj, uint32_t addr, char* alo) {
#pragma unroll
    for (int blk = 0; blk < 2; ++blk) {
        uint32_t h[4], l[4];
#pragma unroll
        for (int yy = 0; yy < 2; ++yy) {
            const float4 f = fj[2 * blk + yy];
            const float2 p0 = mul2(make_float2(fi.x, fi.y), make_float2(f.x, f.y));
            const float2 p1 = mul2(make_float2(fi.z, fi.w), make_float2(f.z, f.w));
            if constexpr (RES) {
                split2_res(p0, h[2 * yy], l[2 * yy]);
                split2_res(p1, h[2 * yy + 1], l[2 * yy + 1]);
            } else {
                split2(p0, h[2 * yy], l[2 * yy]);
                split2(p1, h[2 * yy + 1], l[2 * yy + 1]);
            }
        }
        tmem_st16x256_x1(addr + ((uint32_t)(16 * blk) << 16), h);
        // rows y = 2 blk and 2 blk + 1 sit in 8-row blocks 2 blk and 2 blk + 1 of the quarter
        *reinterpret_cast<uint2*>(alo + (2 * blk) * 1024) = make_uint2(l[0], l[1]);
        *reinterpret_cast<uint2*>(alo + (2 * blk + 1) * 1024) = make_uint2(l[2], l[3]);
    }
}

// store_slot64 for tile 2: the lo parts go to TMEM too (8 columns at `lo_addr`)
template <bool RES = false>
__device__ __forceinline__ void store_slot64_tmem(float4 fi, const float4* fj, uint32_t addr, uint32_t lo_addr) {
#pragma unroll
    for (int blk = 0; blk < 2; ++blk) {
        uint32_t h[4], l[4];
#pragma unroll
        for (int yy = 0; yy < 2; ++yy) {
            const float4 f = fj[2 * blk + yy];
            const float2 p0 = mul2(make_float2(fi.x, fi.y), make_float2(f.x, f.y));
            const float2 p1 = mul2(make_float2(fi.z, fi.w), make_float2(f.z, f.w));
            if constexpr (RES) {
                split2_res(p0, h[2 * yy], l[2 * yy]);
                split2_res(p1, h[2 * yy + 1], l[2 * yy + 1]);
            } else {
                split2(p0, h[2 * yy], l[2 * yy]);
                split2(p1, h[2 * yy + 1], l[2 * yy + 1]);
            }
        }
        tmem_st16x256_x1(addr + ((uint32_t)(16 * blk) << 16), h);
        tmem_st16x256_x1(lo_addr + ((uint32_t)(16 * blk) << 16), l);
    }
}

// The MMAs of one deep chunk (all tiles wide): per k-step and tile, A_hi from
// TMEM (`abase` + 32 t + 8 ks) and A_lo from shared memory (`alo0` + 16 KB t
// + 256 ks; tile 2: from TMEM, `abase` + 32 * 3 + 8 ks) against the stage's
// B rows (`bd0` + 256 ks, 8-row blocks 1024 bytes apart).
// RES (the residual pass, narrow accumulators): per tile and k-step A_res
// (where A_lo would be) against the B_hi blocks (`bd0` then describes the hi
// blocks only, 2048 bytes apart), and A_hi against the B_res blocks (1024
// bytes further).
template <int NT, bool RES = false>
__device__ __forceinline__ void issue_chunk64(const uint32_t (&dcol)[MAXTILES], uint32_t abase, uint64_t alo0,
                                              uint64_t bd0, const uint32_t (&idesc)[MAXTILES], uint32_t first) {
#pragma unroll
    for (int ks = 0; ks < KC64 / 16; ++ks) {
        const uint32_t acc0 = ks == 0 ? first : 1u;
        const uint64_t bd = bd0 + (uint64_t)((ks * 256) >> 4);
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            const uint32_t ahi = abase + (uint32_t)(t * ACOLS + ks * 8);
            const uint64_t alo = alo0 + (uint64_t)((t * ALO_TILE_BYTES + ks * 256) >> 4);
            if constexpr (RES) {
                if (t < 2)
                    asm volatile("{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                                 :: "r"(dcol[t]), "l"(alo), "l"(bd), "r"(idesc[t]), "r"(acc0));
                else
                    asm volatile("{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n"
                                 :: "r"(dcol[t]), "r"(abase + (uint32_t)(3 * ACOLS + ks * 8)), "l"(bd), "r"(idesc[t]),
                                    "r"(acc0));
                asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, 1;"
                             :: "r"(dcol[t]), "r"(ahi), "l"(bd + (uint64_t)(1024 >> 4)), "r"(idesc[t]));
                continue;
            }
            asm volatile("{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n"
                         :: "r"(dcol[t]), "r"(ahi), "l"(bd), "r"(idesc[t]), "r"(acc0));
            if (t < 2)
                asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, 1;"
                             :: "r"(dcol[t]), "l"(alo), "l"(bd), "r"(idesc[t]));
            else
                asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, 1;"
                             :: "r"(dcol[t]), "r"(abase + (uint32_t)(3 * ACOLS + ks * 8)), "l"(bd), "r"(idesc[t]));
        }
    }
}

template <int NFB, bool RES = false, bool BW = false>
__global__ void __launch_bounds__(BW ? NTHREADS64 : NTHREADS, 1)
contract_tc64_kernel(const __grid_constant__ Params P, const __grid_constant__ CUtensorMap fmap) {
    // RES: the residual pass of the 6-product form (narrow accumulators);
    // BW: NBW64 extra warps write the B operand (else the producers do)
    constexpr int NTH = BW ? NTHREADS64 : NTHREADS;
    constexpr int NARR = PWARPS + (BW ? NBW64 : 0);      // arrivals per chunk on bar_full / bar_fempty
    extern __shared__ unsigned char smem_raw[];
    __shared__ Group G;
    __shared__ __align__(8) uint64_t bar_full[NSTAGE], bar_empty[NSTAGE], bar_ffull[NFB], bar_fempty[NFB];
    __shared__ __align__(8) uint64_t bar_seg, bar_drained;
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) int16_t pij[MAXROWS * 4];
    __shared__ int abort_flag_s;
    volatile int& abort_flag = abort_flag_s;
    if (threadIdx.x == 0) G = P.g[blockIdx.y];
    const uint32_t raw_u32 = smem_u32(smem_raw);
    unsigned char* smem = smem_raw + (((raw_u32 + 1023u) & ~1023u) - raw_u32);
    const int F_BYTES = f_bytes(P.nshell);                                   // one 32-voxel half
    unsigned char* fbuf = smem;                                              // NFB x 2 halves
    unsigned char* stage_base = smem + NFB * 2 * F_BYTES;                    // NSTAGE x B operand
    __syncthreads();
    const int ntl = G.ntiles;
    const int nlo = alo_smem_tiles(ntl);
    unsigned char* alo_base = stage_base + NSTAGE * STAGE64_BYTES;            // NSTAGE x nlo x A_lo
    float2* acc = reinterpret_cast<float2*>(alo_base + NSTAGE * nlo * ALO_TILE_BYTES);

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int64_t c0 = (int64_t)blockIdx.x * P.chunks_per_cta;
    const int64_t c1 = min(P.nchunks, c0 + P.chunks_per_cta);
    const int nch = (int)max((int64_t)0, c1 - c0);
    int C = 0;
    for (int t = 0; t < ntl; ++t) C = max(C, G.tile_col[t] + (RES ? 1 : 2) * G.tile_n[t]);

    for (int i = tid; i < MAXROWS * 4; i += NTH) pij[i] = P.pair_row[(size_t)G.table_off * 4 + i];
    for (int i = tid; i < G.nslots; i += NTH) acc[i] = make_float2(0.f, 0.f);
    for (int i = tid; i < NSTAGE * STAGE64_BYTES / 16; i += NTH)
        reinterpret_cast<uint4*>(stage_base)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        abort_flag = 0;
        for (int s = 0; s < NSTAGE; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_full[s])), "r"(NARR));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_empty[s])), "r"(1));
        }
        for (int b = 0; b < NFB; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_ffull[b])), "r"(1));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar_fempty[b])), "r"(NARR));
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
    const int q = warp & 3;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    // A_hi of tile t, stage s, k-step ks (0..3): 8 columns
    auto acol = [&](int s, int t, int ks) { return (uint32_t)(C + (s * MAXTILES + t) * ACOLS + ks * 8); };
    const int seg_log2 = P.seg_log2 - SEG64_SHIFT;

    if (warp < PWARPS) {
        // ================= producers =================
        // Warp w owns TMEM lane quarter w % 4 and forms k-step w / 4 (0..3)
        // of every chunk for all tiles: the row thread of tile pair 0
        // (tiles 0 and 1, A_lo in shared memory) and, with three tiles, that
        // of tile pair 1 (tile 2, A_lo in TMEM) -- the same work for every
        // warp.  k-steps 0, 1 lie in the first 32-voxel half, 2, 3 in the second.
        const int rows = G.rows;
        const int nsh = P.nshell;
        const int ks = warp >> 2;
        const int hh = ks >> 1;
        const uint32_t kx = (ks & 1) ? 64u : 0u;
        const bool b_on = ntl > 2;
        const int ax = lane & 3;
        const int xr = lane >> 2;
        const int32_t* rta = P.rt_tab + ((size_t)blockIdx.y * RT_PER_GROUP + q * 8 + xr) * RT_WORDS;
        const int32_t* rtb = rta + 32 * RT_WORDS;
        const uint32_t code = (uint32_t)rta[0];
        const uint32_t gs0 = (uint32_t)rta[1], gs1 = (uint32_t)rta[2];
        auto foff = [&](int r) {
            r = min(r, nsh - 1);
            return (uint32_t)(r * 128 + ((ax ^ (r & 7)) << 4)) ^ kx;
        };
        const uint32_t oi0 = foff((int)(code & 0xffu)), oi1 = foff((int)((code >> 8) & 0xffu));
        const bool reload = gs1 != gs0;
        uint32_t oj0[4], ojb[4];
#pragma unroll
        for (int y = 0; y < 4; ++y) oj0[y] = foff((int)((gs0 >> (8 * y)) & 0xffu));
        const uint32_t gsb = (uint32_t)rtb[1];
        const uint32_t oib = foff((int)((uint32_t)rtb[0] & 0xffu));
#pragma unroll
        for (int y = 0; y < 4; ++y) ojb[y] = foff((int)((gsb >> (8 * y)) & 0xffu));
        // this thread's A_lo byte offset inside a tile block for k-step ks:
        // row 32q + xr (y = 0), k-group 2 ks + ax / 2, bytes (ax % 2) * 8
        const int alo_thr = (4 * q) * 1024 + (2 * ks + (ax >> 1)) * 128 + xr * 16 + (ax & 1) * 8;
        // without B-writer warps the producers write the B operand: shell r,
        // k-group g (voxels 8g..8g+7 of the 64); 8 nshell <= 512 threads
        int ub_r = -1, ub_g = 0;
        if (!BW && tid < nsh * 8) {
            ub_g = tid / nsh;
            ub_r = tid - ub_g * nsh;
        }
        const int seg_len = 1 << seg_log2;
        const int nseg = (nch + seg_len - 1) >> seg_log2;
        int seg_count = 0;
        bool failed = false;
        auto drain = [&]() -> bool {
            if (!warp_wait(smem_u32(&bar_seg), seg_count & 1)) return false;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int cg = 16 * ((warp >> 2) & 3); cg < C; cg += 64) {
                uint32_t d[16];
                tmem_ld8(lane_base + (uint32_t)cg, d);
                tmem_ld8(lane_base + (uint32_t)cg + 8u, d + 8);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                int t = 0;
                while (t + 1 < ntl && cg >= G.tile_col[t + 1]) ++t;
                const int drow = 128 * t + 32 * q + lane;
                const short4 pr = drow < rows ? *reinterpret_cast<const short4*>(&pij[4 * drow])
                                              : make_short4(-1, 0, -1, 0);
                // wide: the hi and lo columns of 8 shells; narrow (RES): 16 shells
                const int sh0 = RES ? cg - G.tile_col[t] : (cg - G.tile_col[t]) >> 1;
#pragma unroll
                for (int e = 0; e < (RES ? 16 : 8); ++e) {
                    const int l = sh0 + e;
                    if (pr.x < 0 || l < pr.y || l > pr.z) continue;
                    const int slot = pr.w + (l - pr.y);
                    const float v = RES ? __uint_as_float(d[e]) : __uint_as_float(d[e]) + __uint_as_float(d[e + 8]);
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
        for (int c = 0; c < nch; ++c) {
            if (__any_sync(0xffffffffu, abort_flag != 0)) { failed = true; break; }
            const int s = c & 1;
            const int b = c % NFB;
            if (!warp_wait(smem_u32(&bar_ffull[b]), (uint32_t)(c / NFB) & 1u)) {
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
            const unsigned char* F = fbuf + (size_t)b * 2 * F_BYTES;
            char* Alo = reinterpret_cast<char*>(alo_base) + (size_t)s * nlo * ALO_TILE_BYTES;
            if (ub_r >= 0) {
                char* Bst = reinterpret_cast<char*>(stage_base) + (size_t)s * STAGE64_BYTES;
                const unsigned char* Fh = F + (ub_g >> 2) * F_BYTES;
                const int g4 = ub_g & 3;
                const float4 a = *reinterpret_cast<const float4*>(Fh + fchunk(ub_r, 2 * g4));
                const float4 e = *reinterpret_cast<const float4*>(Fh + fchunk(ub_r, 2 * g4 + 1));
                const float2 x[4] = {make_float2(a.x, a.y), make_float2(a.z, a.w), make_float2(e.x, e.y),
                                     make_float2(e.z, e.w)};
                if constexpr (RES) split_store8_res(x, Bst + op_off64(brow(ub_r, 0), ub_g), Bst + op_off64(brow(ub_r, 1), ub_g));
                else split_store8(x, Bst + op_off64(brow(ub_r, 0), ub_g), Bst + op_off64(brow(ub_r, 1), ub_g));
            }
            {
                const unsigned char* Fh = F + hh * F_BYTES;
                const float4 fi0 = lds4(Fh, oi0);
                const float4 fi1 = lds4(Fh, oi1);
                float4 fj[4];
#pragma unroll
                for (int y = 0; y < 4; ++y) fj[y] = lds4(Fh, oj0[y]);
                store_slot64<RES>(fi0, fj, lane_base + acol(s, 0, ks), Alo + alo_thr);
                if (reload) {
#pragma unroll
                    for (int y = 0; y < 4; ++y) fj[y] = lds4(Fh, foff((int)((gs1 >> (8 * y)) & 0xffu)));
                }
                store_slot64<RES>(fi1, fj, lane_base + acol(s, 1, ks), Alo + ALO_TILE_BYTES + alo_thr);
                if (b_on) {
                    const float4 fb = lds4(Fh, oib);
#pragma unroll
                    for (int y = 0; y < 4; ++y) fj[y] = lds4(Fh, ojb[y]);
                    store_slot64_tmem<RES>(fb, fj, lane_base + acol(s, 2, ks), lane_base + acol(s, 3, ks));
                }
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            // A_lo and B writes (generic proxy) made visible to the MMA (async proxy)
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&bar_full[s]));
                mbar_arrive(smem_u32(&bar_fempty[b]));
            }
            while (seg_count < nseg && ((seg_count + 1) << seg_log2) - 1 < c) {
                if (!drain()) { atomicExch(P.err, 2); abort_flag = 1; failed = true; break; }
            }
            if (failed) break;
        }
        while (!failed && seg_count < nseg) {
            if (!drain()) { atomicExch(P.err, 2); abort_flag = 1; break; }
        }
    } else if (warp == MMA_WARP) {
        if (lane == 0) {
            uint32_t idesc[MAXTILES], dcol[MAXTILES];
#pragma unroll
            for (int t = 0; t < MAXTILES; ++t) {
                idesc[t] = make_idesc(128, (RES ? 1 : 2) * G.tile_n[t]);
                dcol[t] = tmem + (uint32_t)G.tile_col[t];
            }
            // all B rows (wide), or the hi blocks only (RES: 2048 bytes apart)
            const uint64_t bdesc0 = make_desc(smem_u32(stage_base), 128, RES ? 2048 : 1024);
            const uint64_t adesc0 = make_desc(smem_u32(alo_base), 128, 1024);
            int seg_count = 0;
            const int seg_mask = (1 << seg_log2) - 1;
            uint32_t first = 0;
            for (int c = 0; c < nch; ++c) {
                const int s = c & 1;
                if (!mbar_wait(smem_u32(&bar_full[s]), (c >> 1) & 1)) { atomicExch(P.err, 3); abort_flag = 1; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t abase = tmem + acol(s, 0, 0);
                const uint64_t bd0 = bdesc0 + (uint64_t)((s * STAGE64_BYTES) >> 4);
                const uint64_t alo0 = adesc0 + (uint64_t)((s * nlo * ALO_TILE_BYTES) >> 4);
                if (ntl == 2) issue_chunk64<2, RES>(dcol, abase, alo0, bd0, idesc, first);
                else issue_chunk64<3, RES>(dcol, abase, alo0, bd0, idesc, first);
                first = 1u;
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                             :: "r"(smem_u32(&bar_empty[s])) : "memory");
                if (((c + 1) & seg_mask) == 0 || c + 1 == nch) {
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                                 :: "r"(smem_u32(&bar_seg)) : "memory");
                    if (!mbar_wait(smem_u32(&bar_drained), seg_count & 1)) { atomicExch(P.err, 4); abort_flag = 1; break; }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    ++seg_count;
                    first = 0u;
                }
            }
            if (nch > 0) {
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                             :: "r"(smem_u32(&bar_seg)) : "memory");
                mbar_wait(smem_u32(&bar_seg), seg_count & 1);
            }
        }
    } else if (BW && warp >= BW0) {
        // ================= B writers =================
        // item (shell r, k-group g: voxels 8g .. 8g + 7 of the 64): its hi and
        // lo rows of the stage's B operand; items bt, bt + 64, ... (8 nshell <= 512)
        const int bt = tid - BW0 * 32;
        const int nsh = P.nshell;
        constexpr int MAXIT = 8 * MAXB / (32 * NBW64);
        uint32_t src0[MAXIT], src1[MAXIT], dhi[MAXIT], dlo[MAXIT];
        int nit = 0;
#pragma unroll
        for (int k = 0; k < MAXIT; ++k) {
            const int it = bt + 32 * NBW64 * k;
            const int g = it / nsh, r = it - g * nsh;
            if (it < 8 * nsh) nit = k + 1;
            src0[k] = (uint32_t)((g >> 2) * F_BYTES + fchunk(r, 2 * (g & 3)));
            src1[k] = (uint32_t)((g >> 2) * F_BYTES + fchunk(r, 2 * (g & 3) + 1));
            dhi[k] = (uint32_t)op_off64(brow(r, 0), g);
            dlo[k] = (uint32_t)op_off64(brow(r, 1), g);
        }
        for (int c = 0; c < nch; ++c) {
            if (__any_sync(0xffffffffu, abort_flag != 0)) break;
            const int s = c & 1;
            const int b = c % NFB;
            if (!warp_wait(smem_u32(&bar_ffull[b]), (uint32_t)(c / NFB) & 1u)) {
                atomicExch(P.err, 1);
                abort_flag = 1;
                break;
            }
            if (c >= NSTAGE) {
                if (!warp_wait(smem_u32(&bar_empty[s]), ((c - NSTAGE) >> 1) & 1)) {
                    atomicExch(P.err, 1);
                    abort_flag = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            }
            const unsigned char* F = fbuf + (size_t)b * 2 * F_BYTES;
            char* Bst = reinterpret_cast<char*>(stage_base) + (size_t)s * STAGE64_BYTES;
#pragma unroll
            for (int k = 0; k < MAXIT; ++k) {
                if (k < nit) {
                    const float4 a = *reinterpret_cast<const float4*>(F + src0[k]);
                    const float4 e = *reinterpret_cast<const float4*>(F + src1[k]);
                    const float2 x[4] = {make_float2(a.x, a.y), make_float2(a.z, a.w), make_float2(e.x, e.y),
                                         make_float2(e.z, e.w)};
                    if constexpr (RES) split_store8_res(x, Bst + dhi[k], Bst + dlo[k]);
                    else split_store8(x, Bst + dhi[k], Bst + dlo[k]);
                }
            }
            // B writes (generic proxy) made visible to the MMA (async proxy)
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&bar_full[s]));
                mbar_arrive(smem_u32(&bar_fempty[b]));
            }
        }
    } else if (warp == TMA_WARP && lane == 0) {
        // two 32-voxel copies per chunk into the buffer's halves, one barrier
        const uint32_t fb0 = smem_u32(fbuf);
        const uint32_t tx = (uint32_t)(P.nshell * KC64 * 4);
        int issued = 0;
        for (int c = 0; c < nch; ++c) {
            const int b = c % NFB;
            if (c >= NFB && !mbar_wait(smem_u32(&bar_fempty[b]), (uint32_t)(c / NFB - 1) & 1u)) {
                atomicExch(P.err, 5);
                abort_flag = 1;
                break;
            }
            if (abort_flag) break;
            const uint32_t fb = smem_u32(&bar_ffull[b]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(fb), "r"(tx) : "memory");
            const int x0 = (int)((c0 + c) * KC64);
#pragma unroll
            for (int h = 0; h < 2; ++h)
                asm volatile(
                    "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                    :: "r"(fb0 + (uint32_t)((2 * b + h) * F_BYTES)), "l"(reinterpret_cast<uint64_t>(&fmap)),
                       "r"(x0 + 32 * h), "r"(0), "r"(fb)
                    : "memory");
            issued = c + 1;
        }
        for (int c = max(0, issued - NFB); c < issued; ++c)
            mbar_wait(smem_u32(&bar_ffull[c % NFB]), (uint32_t)(c / NFB) & 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (!abort_flag) {
        for (int i = tid; i < G.nslots; i += NTH) {
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
// host planning, two kinds of plan (cached per triangle list):
//  - runs: pairs (i, j) = the two largest shell slots of each triangle,
//    column = the smallest.  The pairs of each shell i are cut into runs of
//    four consecutive shells j (a "slot": rows (i, J + y), y = 0..3, some of
//    them padding); two slots with the same run J make one producer row
//    thread (its loads of F_J .. F_J+3 serve both).  Row threads are sorted by
//    J so each tile's columns stay short, and the two threads that share a
//    quarter-warp load phase are matched to keep their shared-memory reads in
//    different banks.
//  - cover (build_cover_plan): any shell pairs that meet every triangle, in
//    blocks shaped like the row threads, where that needs fewer tiles.
// ---------------------------------------------------------------------------
struct HostPlan {
    Params base;           // pointers filled at launch
    std::vector<int16_t> pair_row;
    std::vector<int32_t> rt_tab;
    std::vector<int32_t> slot_tri;
    std::vector<char> image;      // pair_row | rt_tab | slot_tri, each 256-byte aligned (device layout)
    const void* image_src = nullptr;   // page-locked copy of `image` (or image.data())
    size_t off_rt = 0;
    size_t off_stri = 0;
    size_t smem = 0;
    bool ok = false;
    bool invalid = false;         // the triangle list itself is malformed (vs. unsupported)
    bool cover = false;           // rows are a pair cover (3 tiles), not runs
    int nfb64 = 0;                // field buffers of the 64-voxel kernel (0: the plan does not fit it)
    bool bw64 = false;            // ... with B-writer warps (every group has 3 tiles, 3 field buffers)
    size_t smem64 = 0;            // its dynamic shared memory
    char why[160] = {0};
};

static size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

static std::mutex g_plan_mu;
static std::map<std::vector<int32_t>, HostPlan*> g_plans;

// Pads a group's Kahan-slot list so that row `row` (its index in the group)
// starts its columns at a slot with (start - lmin) = row (mod 16): in a
// drain the 16 lanes of a half-warp (16 consecutive rows) then update the
// same column's slots in 16 different 8-byte bank pairs.
static void align_row_slots(std::vector<int32_t>& v, int row, int lmin) {
    while ((((int)v.size() - lmin - row) & 15) != 0) v.push_back(-1);
}

static int pow2_cols(int n) {
    int c = 32;
    while (c < n) c <<= 1;
    return c;
}

struct PlanSlot {
    int i, J, mask;   // rows (i, J + y) for the set bits y of mask
};
struct RowThread {
    PlanSlot s[2];
};

// Extra shared-memory wavefronts when two row threads share a load phase:
// two different field rows conflict when their 16-byte pieces fall in the
// same half of the 128-byte swizzled row (bit 2 of the row index equal).
static int phase_conflicts(const RowThread& A, const RowThread& B) {
    auto clash = [](int r, int t) { return r != t && ((r >> 2) & 1) == ((t >> 2) & 1); };
    int c = clash(A.s[0].i, B.s[0].i) + clash(A.s[1].i, B.s[1].i);
    for (int y = 0; y < 4; ++y) c += clash(A.s[0].J + y, B.s[0].J + y);
    if (A.s[1].J != A.s[0].J || B.s[1].J != B.s[0].J)
        for (int y = 0; y < 4; ++y) c += clash(A.s[1].J + y, B.s[1].J + y);
    return c;
}

// Slot table and the device image of a plan whose rows and row threads are set.
static void finish_plan(HostPlan* hp, int ngroups, int maxslots, const std::vector<std::vector<int32_t>>& gslots,
                        size_t fixed) {
    Params& P = hp->base;
    P.maxslots = maxslots;
    hp->slot_tri.assign((size_t)ngroups * maxslots, -1);
    for (int g = 0; g < ngroups; ++g)
        for (size_t i = 0; i < gslots[g].size(); ++i) hp->slot_tri[(size_t)g * maxslots + i] = gslots[g][i];
    hp->smem = fixed + sizeof(float2) * (size_t)maxslots;
    hp->off_rt = al256(hp->pair_row.size() * 2);
    hp->off_stri = hp->off_rt + al256(hp->rt_tab.size() * 4);
    hp->image.assign(hp->off_stri + al256(hp->slot_tri.size() * 4), 0);
    memcpy(hp->image.data(), hp->pair_row.data(), hp->pair_row.size() * 2);
    memcpy(hp->image.data() + hp->off_rt, hp->rt_tab.data(), hp->rt_tab.size() * 4);
    memcpy(hp->image.data() + hp->off_stri, hp->slot_tri.data(), hp->slot_tri.size() * 4);
    hp->image_src = pinned_copy(hp->image.data(), hp->image.size());
    if (hp->image_src == nullptr) hp->image_src = hp->image.data();
    hp->ok = true;
    // the 64-voxel kernel: every group of 2 or 3 tiles in the wide form, and
    // its buffers (two or three field buffers) in shared memory
    bool deep = true;
    int ntmax = 0;
    for (int g = 0; g < ngroups; ++g) {
        const Group& G = P.g[g];
        deep = deep && (G.ntiles == 2 || G.ntiles == 3) && G.wide;
        ntmax = std::max(ntmax, G.ntiles);
    }
    const int nshell = P.nshell;
    for (int nfb = 3; deep && nfb >= 2; --nfb) {
        const size_t need = (size_t)fixed_smem64(nshell, ntmax, nfb) + sizeof(float2) * (size_t)maxslots;
        if (need <= (size_t)kDeepSmemLimit) {
            hp->nfb64 = nfb;
            hp->smem64 = need;
            break;
        }
    }
    // B-writer warps pay off when the producers form three tiles (measured at
    // 360^3: 40 shells / 3 tiles 6.95 -> 6.79 ms; 30 shells / 2 tiles 5.16 -> 5.36)
    if (hp->nfb64 == 3) {
        hp->bw64 = true;
        for (int g = 0; g < ngroups; ++g) hp->bw64 = hp->bw64 && P.g[g].ntiles == 3;
    }
}

// Cover plan: a D row (a, b) gives B(a, b, c) for every column c, so the rows
// need only be a set of shell pairs that meets every triangle, not the pairs
// of its two largest shells.  Rows come in blocks that match the producer
// threads: up to 32 "two-slot" blocks {f1, f2} x {g0..g3} (tiles 0 and 1,
// one load of each g serves both slots) chosen greedily by triangles newly
// covered, then up to 32 "one-slot" blocks {f} x {g0..g3} (tile 2).  When
// they cover every triangle the contraction runs on 3 tiles (2 when no
// one-slot block is needed) instead of 4: 12 (8) MMAs per chunk instead of
// 16 (Nmax 40: 32 + 29 blocks, 372 rows, against 440 pairs + padding).
// Returns false otherwise (the run plan then rebuilds hp).
static bool build_cover_plan(HostPlan* hp, int nshell, const int32_t* tri_host, int ntri, int budget, size_t fixed) {
    const int S = nshell, T = ntri, W = (T + 63) / 64;
    std::vector<std::array<int, 3>> tri(T);
    for (int t = 0; t < T; ++t) {
        int v[3] = {tri_host[t], tri_host[ntri + t], tri_host[2 * ntri + t]};
        std::sort(v, v + 3);
        tri[t] = {v[2], v[1], v[0]};
    }
    // pm(a, b): triangles that contain both a and b (a == b: twice)
    std::vector<uint64_t> pm((size_t)S * S * W, 0);
    auto PM = [&](int a, int b) { return &pm[((size_t)a * S + b) * W]; };
    auto setbit = [&](int a, int b, int t) {
        PM(a, b)[t >> 6] |= 1ull << (t & 63);
        PM(b, a)[t >> 6] |= 1ull << (t & 63);
    };
    for (int t = 0; t < T; ++t) {
        const int i = tri[t][0], j = tri[t][1], l = tri[t][2];
        setbit(i, j, t);
        setbit(i, l, t);
        setbit(j, l, t);
    }
    std::vector<uint64_t> unc(W, ~0ull);
    if (T % 64) unc[W - 1] = (1ull << (T % 64)) - 1;
    auto remaining = [&]() {
        for (int w = 0; w < W; ++w)
            if (unc[w]) return true;
        return false;
    };
    struct Block { int f[2]; int nf; int g[4]; };
    std::vector<Block> blocks2, blocks1;
    std::vector<uint64_t> cand((size_t)(S + 1) * W), m(W), best_m(W);
    // greedy: for the f set, pick four g one at a time by newly covered triangles
    auto grow = [&](const int* f, int nf, int* g, std::vector<uint64_t>& cov) {
        for (int x = 0; x < S; ++x)
            for (int w = 0; w < W; ++w) {
                uint64_t v = 0;
                for (int k = 0; k < nf; ++k) v |= PM(f[k], x)[w];
                cand[(size_t)x * W + w] = v & unc[w];
            }
        std::fill(cov.begin(), cov.end(), 0ull);
        int total = 0;
        for (int pick = 0; pick < 4; ++pick) {
            int gb = -1, cb = -1;
            for (int x = 0; x < S; ++x) {
                bool used = false;
                for (int k = 0; k < pick; ++k) used |= g[k] == x;
                if (used) continue;
                int c = 0;
                for (int w = 0; w < W; ++w) c += __builtin_popcountll(cand[(size_t)x * W + w] & ~cov[w]);
                if (c > cb) { cb = c; gb = x; }
            }
            g[pick] = gb;
            total += cb;
            for (int w = 0; w < W; ++w) cov[w] |= cand[(size_t)gb * W + w];
        }
        return total;
    };
    std::vector<int> single(S);
    std::vector<std::pair<int, std::pair<int, int>>> order;
    for (int k = 0; k < 32 && remaining(); ++k) {
        Block bb{{0, 0}, 2, {0, 0, 0, 0}};
        int bc = -1;
        // candidates in order of the sum of their shells' one-slot coverage;
        // the scan stops once that sum cannot beat the best pair found
        for (int f = 0; f < S; ++f) {
            int g[4];
            single[f] = grow(&f, 1, g, m);
        }
        order.clear();
        for (int f1 = 0; f1 < S; ++f1)
            for (int f2 = f1 + 1; f2 < S; ++f2) order.push_back({single[f1] + single[f2], {f1, f2}});
        std::sort(order.begin(), order.end(), [](const std::pair<int, std::pair<int, int>>& x,
                                                  const std::pair<int, std::pair<int, int>>& y) {
            return x.first != y.first ? x.first > y.first : x.second < y.second;
        });
        for (const auto& o : order) {
            if (o.first <= bc) break;
            const int f[2] = {o.second.first, o.second.second};
            int g[4];
            const int c = grow(f, 2, g, m);
            if (c > bc) {
                bc = c;
                bb = Block{{f[0], f[1]}, 2, {g[0], g[1], g[2], g[3]}};
                best_m = m;
            }
        }
        if (bc <= 0) break;
        blocks2.push_back(bb);
        for (int w = 0; w < W; ++w) unc[w] &= ~best_m[w];
    }
    for (int k = 0; k < 32 && remaining(); ++k) {
        Block bb{{0, 0}, 1, {0, 0, 0, 0}};
        int bc = -1;
        for (int f1 = 0; f1 < S; ++f1) {
            int g[4];
            const int c = grow(&f1, 1, g, m);
            if (c > bc) {
                bc = c;
                bb = Block{{f1, f1}, 1, {g[0], g[1], g[2], g[3]}};
                best_m = m;
            }
        }
        if (bc <= 0) break;
        blocks1.push_back(bb);
        for (int w = 0; w < W; ++w) unc[w] &= ~best_m[w];
    }
    if (remaining()) return false;
    const int ntiles = blocks1.empty() ? 2 : 3;           // two-slot blocks alone: tiles 0 and 1
    // blocks at positions 2p and 2p + 1 of a lane quarter share quarter-warp
    // load phases: pair them greedily by bank clashes (two field rows clash
    // when they differ and bit 2 of their index agrees: same half of the
    // swizzled row), trying every order of the partner's four g
    auto clash = [](int r, int t) { return r != t && ((r >> 2) & 1) == ((t >> 2) & 1); };
    auto pair_blocks = [&](std::vector<Block>& bl) {
        std::vector<Block> out;
        std::vector<bool> used(bl.size(), false);
        for (size_t a = 0; a < bl.size(); ++a) {
            if (used[a]) continue;
            used[a] = true;
            out.push_back(bl[a]);
            int best = -1, bc = 1 << 30;
            Block bb = bl[a];
            for (size_t b = a + 1; b < bl.size(); ++b) {
                if (used[b]) continue;
                int gp[4] = {0, 1, 2, 3};
                do {
                    int c = 0;
                    for (int k = 0; k < bl[a].nf; ++k) c += clash(bl[a].f[k], bl[b].f[k]);
                    for (int y = 0; y < 4; ++y) c += clash(bl[a].g[y], bl[b].g[gp[y]]);
                    if (c < bc) {
                        bc = c;
                        best = (int)b;
                        bb = bl[b];
                        for (int y = 0; y < 4; ++y) bb.g[y] = bl[b].g[gp[y]];
                    }
                } while (std::next_permutation(gp, gp + 4));
            }
            if (best >= 0) {
                used[best] = true;
                out.push_back(bb);
            }
        }
        bl = out;
    };
    pair_blocks(blocks2);
    pair_blocks(blocks1);
    // rows: two-slot block k at (q, x) = (k / 8, k % 8) in tiles 0 and 1,
    // one-slot block k at the same positions of tile 2; row (f, g_y) at lane 32q + x + 8y
    struct Row { int f, g; std::vector<std::pair<int, int>> cols; };   // (column, triangle)
    std::vector<Row> rows(MAXROWS, Row{-1, -1, {}});
    auto row_of = [](int tile, int k, int y) { return 128 * tile + 32 * (k / 8) + (k % 8) + 8 * y; };
    for (size_t k = 0; k < blocks2.size(); ++k)
        for (int u = 0; u < 2; ++u)
            for (int y = 0; y < 4; ++y) rows[row_of(u, (int)k, y)] = Row{blocks2[k].f[u], blocks2[k].g[y], {}};
    for (size_t k = 0; k < blocks1.size(); ++k)
        for (int y = 0; y < 4; ++y) rows[row_of(2, (int)k, y)] = Row{blocks1[k].f[0], blocks1[k].g[y], {}};
    // each triangle goes to the first row whose pair it contains; column = its third shell
    for (int t = 0; t < T; ++t) {
        bool done = false;
        for (int r = 0; r < MAXROWS && !done; ++r) {
            if (rows[r].f < 0) continue;
            int v[3] = {tri[t][0], tri[t][1], tri[t][2]};
            int a = -1, b = -1;
            for (int z = 0; z < 3; ++z)
                if (a < 0 && v[z] == rows[r].f) a = z;
            for (int z = 0; z < 3; ++z)
                if (b < 0 && z != a && v[z] == rows[r].g) b = z;
            if (a < 0 || b < 0) continue;
            rows[r].cols.push_back({v[3 - a - b], t});
            done = true;
        }
        if (!done) return false;
    }
    Params& P = hp->base;
    Group& G = P.g[0];
    P.ngroups = 1;
    P.nshell = nshell;
    P.ntri = ntri;
    G.ntiles = ntiles;
    G.rows = 128 * G.ntiles;
    G.table_off = 0;
    hp->pair_row.assign((size_t)MAXROWS * 4, (int16_t)0);
    for (int r = 0; r < MAXROWS; ++r) hp->pair_row[4 * r] = -1;
    hp->rt_tab.assign((size_t)RT_PER_GROUP * RT_WORDS, 0);
    auto gword = [](const int* g) {
        return (int32_t)((uint32_t)g[0] | (uint32_t)g[1] << 8 | (uint32_t)g[2] << 16 | (uint32_t)g[3] << 24);
    };
    // two-slot block k: entry k (tiles 0 and 1); one-slot block k: entry
    // 32 + k (tile 2; the warps of tile pair 1 skip slot 1, there is no tile 3)
    for (size_t k = 0; k < blocks2.size(); ++k) {
        int32_t* w = &hp->rt_tab[k * RT_WORDS];
        w[0] = (int32_t)((uint32_t)blocks2[k].f[0] | (uint32_t)blocks2[k].f[1] << 8);
        w[1] = w[2] = gword(blocks2[k].g);
    }
    for (size_t k = 0; k < blocks1.size(); ++k) {
        int32_t* w = &hp->rt_tab[(32 + k) * RT_WORDS];
        w[0] = (int32_t)((uint32_t)blocks1[k].f[0] | (uint32_t)blocks1[k].f[0] << 8);
        w[1] = w[2] = gword(blocks1[k].g);
    }
    std::vector<std::vector<int32_t>> gslots(1);
    int tile_maxl[MAXTILES] = {0, 0, 0, 0};
    for (int r = 0; r < MAXROWS; ++r) {
        Row& R = rows[r];
        if (R.cols.empty()) continue;
        std::sort(R.cols.begin(), R.cols.end());
        const int lmin = R.cols.front().first, lmax = R.cols.back().first;
        int16_t* pr = &hp->pair_row[(size_t)r * 4];
        pr[0] = (int16_t)(R.f | (R.g << 8));
        pr[1] = (int16_t)lmin;
        pr[2] = (int16_t)lmax;
        align_row_slots(gslots[0], r, lmin);
        pr[3] = (int16_t)gslots[0].size();
        size_t c = 0;
        for (int l = lmin; l <= lmax; ++l) {
            if (c < R.cols.size() && R.cols[c].first == l) gslots[0].push_back(R.cols[c++].second);
            else gslots[0].push_back(-1);
        }
        tile_maxl[r / 128] = std::max(tile_maxl[r / 128], lmax);
    }
    if ((int)gslots[0].size() > budget || gslots[0].size() > 32767) return false;
    int wide_cols = 0;
    for (int t = 0; t < G.ntiles; ++t) wide_cols += 2 * ((tile_maxl[t] + 1 + 7) / 8 * 8);
    G.wide = wide_cols <= 512 - NSTAGE * MAXTILES * ACOLS ? 1 : 0;
    int col = 0;
    for (int t = 0; t < MAXTILES; ++t) { G.tile_n[t] = 16; G.tile_col[t] = 0; }
    for (int t = 0; t < G.ntiles; ++t) {
        G.tile_n[t] = G.wide ? (tile_maxl[t] + 1 + 7) / 8 * 8 : (tile_maxl[t] + 1 + 15) / 16 * 16;
        G.tile_col[t] = col;
        col += (G.wide ? 2 : 1) * G.tile_n[t];
    }
    G.ncols = pow2_cols(col + NSTAGE * MAXTILES * ACOLS);
    if (G.ncols > 512) return false;
    G.nslots = (int)gslots[0].size();
    finish_plan(hp, 1, std::max(1, G.nslots), gslots, fixed);
    return true;
}

static HostPlan* build_plan(int nshell, const int32_t* tri_host, int ntri, bool allow_cover) {
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
    // slots: runs of four shells j per pair shell i
    std::map<int, std::vector<int>> byi;
    for (auto& kv : pairs) byi[kv.first.first].push_back(kv.first.second);
    std::map<int, std::vector<PlanSlot>> byJ;
    for (auto& kv : byi) {
        std::vector<int>& js = kv.second;
        std::sort(js.begin(), js.end());
        for (size_t k = 0; k < js.size();) {
            PlanSlot sl{kv.first, js[k], 0};
            while (k < js.size() && js[k] <= sl.J + 3) sl.mask |= 1 << (js[k++] - sl.J);
            byJ[sl.J].push_back(sl);
        }
    }
    // row threads: two slots of the same run; the rest paired in run order
    std::vector<RowThread> rts;
    std::vector<PlanSlot> single;
    for (auto& kv : byJ) {
        const std::vector<PlanSlot>& v = kv.second;
        size_t k = 0;
        for (; k + 1 < v.size(); k += 2) rts.push_back(RowThread{{v[k], v[k + 1]}});
        if (k < v.size()) single.push_back(v[k]);
    }
    for (size_t k = 0; k < single.size(); k += 2) {
        const PlanSlot other = k + 1 < single.size() ? single[k + 1] : PlanSlot{single[k].i, single[k].J, 0};
        rts.push_back(RowThread{{single[k], other}});
    }
    std::stable_sort(rts.begin(), rts.end(), [](const RowThread& x, const RowThread& y) {
        const int jx = std::max(x.s[0].J, x.s[1].J), jy = std::max(y.s[0].J, y.s[1].J);
        return jx != jy ? jx < jy : x.s[0].i < y.s[0].i;
    });
    auto rt_slots = [&](const RowThread& r) {
        int n = 0;
        for (int u = 0; u < 2; ++u)
            for (int y = 0; y < 4; ++y)
                if (r.s[u].mask >> y & 1) {
                    const auto& m = pairs[{r.s[u].i, r.s[u].J + y}];
                    n += m.rbegin()->first - m.begin()->first + 1;
                }
        return n;
    };
    const size_t fixed = (size_t)fixed_smem(nshell);
    const int budget = (int)((227 * 1024 - 8192 - fixed) / sizeof(float2));
    // fewer tiles with a pair cover where the run plan needs 4 (bounded search cost)
    if (allow_cover && rts.size() > (size_t)RT_PER_GROUP / 2 && rts.size() <= (size_t)RT_PER_GROUP && nshell <= 48 &&
        ntri <= 12000 && build_cover_plan(hp, nshell, tri_host, ntri, budget, fixed)) {
        hp->cover = true;
        return hp;
    }
    // CTA groups: up to 64 consecutive row threads and `budget` Kahan slots
    std::vector<size_t> group_first;
    {
        int cur = 0, cur_slots = 0;
        for (size_t k = 0; k < rts.size(); ++k) {
            const int ns = rt_slots(rts[k]);
            if (ns > budget) {
                snprintf(hp->why, sizeof(hp->why), "a row thread holds %d triangles (limit %d)", ns, budget);
                return hp;
            }
            if (k == 0 || cur == RT_PER_GROUP || cur_slots + ns > budget) {
                group_first.push_back(k);
                cur = cur_slots = 0;
            }
            ++cur;
            cur_slots += ns;
        }
    }
    const int ngroups = (int)group_first.size();
    if (ngroups > MAXGROUPS || ngroups == 0) {
        snprintf(hp->why, sizeof(hp->why), "too many pair rows (%zu) for the BF16x3 contraction", pairs.size());
        return hp;
    }
    P.ngroups = ngroups;
    P.nshell = nshell;
    P.ntri = ntri;
    hp->pair_row.assign((size_t)ngroups * MAXROWS * 4, (int16_t)0);
    for (size_t r = 0; r < (size_t)ngroups * MAXROWS; ++r) hp->pair_row[4 * r] = -1;
    hp->rt_tab.assign((size_t)ngroups * RT_PER_GROUP * RT_WORDS, 0);
    std::vector<std::vector<int32_t>> gslots(ngroups);
    int maxslots = 1;
    for (int g = 0; g < ngroups; ++g) {
        Group& G = P.g[g];
        const size_t k0 = group_first[g];
        const size_t k1 = g + 1 < ngroups ? group_first[g + 1] : rts.size();
        const int n = (int)(k1 - k0);
        G.ntiles = n > RT_PER_GROUP / 2 ? 4 : 2;
        G.rows = 128 * G.ntiles;
        G.table_off = g * MAXROWS;
        int tile_maxl[MAXTILES] = {0, 0, 0, 0};
        for (int tp = 0; tp * 32 < n; ++tp) {
            // match the 32 row threads of this tile pair into load-phase partners
            std::vector<RowThread> blk(rts.begin() + k0 + 32 * tp, rts.begin() + k0 + std::min(n, 32 * (tp + 1)));
            std::vector<int> order;
            std::vector<bool> used(blk.size(), false);
            for (size_t x = 0; x < blk.size(); ++x) {
                if (used[x]) continue;
                used[x] = true;
                order.push_back((int)x);
                int best = -1, bc = 0;
                for (size_t y = x + 1; y < blk.size(); ++y) {
                    if (used[y]) continue;
                    const int c = phase_conflicts(blk[x], blk[y]);
                    if (best < 0 || c < bc) { best = (int)y; bc = c; }
                }
                if (best >= 0) { used[best] = true; order.push_back(best); }
            }
            // the rows of a slot may sit in any order: the second thread of a
            // load-phase pair takes the order of its runs that clashes least
            // with its partner's loads
            auto clash = [](int a, int b) { return a != b && ((a >> 2) & 1) == ((b >> 2) & 1); };
            int prev_g[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
            for (size_t pos = 0; pos < order.size(); ++pos) {
                const RowThread& r = blk[order[pos]];
                const int q = (int)pos / 8, x = (int)pos % 8;
                int gy[2][4];
                for (int u = 0; u < 2; ++u)
                    for (int y = 0; y < 4; ++y) gy[u][y] = std::min(r.s[u].J + y, nshell - 1);
                int perm[4] = {0, 1, 2, 3};
                if (pos & 1) {
                    int gp[4] = {0, 1, 2, 3}, bc = 1 << 30;
                    const bool two = r.s[1].J != r.s[0].J;
                    do {
                        int c = 0;
                        for (int y = 0; y < 4; ++y) {
                            c += clash(prev_g[0][y], gy[0][gp[y]]);
                            if (two) c += clash(prev_g[1][y], gy[1][gp[y]]);
                        }
                        if (c < bc) {
                            bc = c;
                            for (int y = 0; y < 4; ++y) perm[y] = gp[y];
                        }
                    } while (std::next_permutation(gp, gp + 4));
                }
                for (int u = 0; u < 2; ++u)
                    for (int y = 0; y < 4; ++y) prev_g[u][y] = gy[u][perm[y]];
                int32_t* w = &hp->rt_tab[((size_t)g * RT_PER_GROUP + 32 * tp + pos) * RT_WORDS];
                w[0] = (int32_t)((uint32_t)r.s[0].i | (uint32_t)r.s[1].i << 8);
                for (int u = 0; u < 2; ++u) {
                    uint32_t gs = 0;
                    for (int y = 0; y < 4; ++y) gs |= (uint32_t)gy[u][perm[y]] << (8 * y);
                    w[1 + u] = (int32_t)gs;
                }
                for (int u = 0; u < 2; ++u) {
                    const int tile = 2 * tp + u;
                    for (int y = 0; y < 4; ++y) {
                        if (!(r.s[u].mask >> perm[y] & 1)) continue;
                        const int i = r.s[u].i, j = r.s[u].J + perm[y];
                        const auto& m = pairs[{i, j}];
                        const int lmin = m.begin()->first, lmax = m.rbegin()->first;
                        const int row = 128 * tile + 32 * q + x + 8 * y;
                        int16_t* pr = &hp->pair_row[((size_t)G.table_off + row) * 4];
                        pr[0] = (int16_t)(i | (j << 8));
                        pr[1] = (int16_t)lmin;
                        pr[2] = (int16_t)lmax;
                        align_row_slots(gslots[g], row, lmin);
                        pr[3] = (int16_t)gslots[g].size();
                        for (int l = lmin; l <= lmax; ++l) {
                            auto it = m.find(l);
                            gslots[g].push_back(it == m.end() ? -1 : it->second);
                        }
                        tile_maxl[tile] = std::max(tile_maxl[tile], lmax);
                    }
                }
            }
        }
        // wide form when the 2N columns of all tiles fit beside the A stages
        int wide_cols = 0;
        for (int t = 0; t < G.ntiles; ++t) wide_cols += 2 * ((tile_maxl[t] + 1 + 7) / 8 * 8);
        G.wide = wide_cols <= 512 - NSTAGE * MAXTILES * ACOLS ? 1 : 0;
        int col = 0;
        for (int t = 0; t < MAXTILES; ++t) { G.tile_n[t] = 16; G.tile_col[t] = 0; }
        for (int t = 0; t < G.ntiles; ++t) {
            G.tile_n[t] = G.wide ? (tile_maxl[t] + 1 + 7) / 8 * 8 : (tile_maxl[t] + 1 + 15) / 16 * 16;
            G.tile_col[t] = col;
            col += (G.wide ? 2 : 1) * G.tile_n[t];
        }
        G.ncols = pow2_cols(col + NSTAGE * MAXTILES * ACOLS);
        if (G.ncols > 512) {
            snprintf(hp->why, sizeof(hp->why), "BF16x3 tile columns exceed TMEM");
            return hp;
        }
        G.nslots = (int)gslots[g].size();
        if (G.nslots > 32767) {
            snprintf(hp->why, sizeof(hp->why), "too many triangles in one CTA group");
            return hp;
        }
        maxslots = std::max(maxslots, G.nslots);
    }
    finish_plan(hp, ngroups, maxslots, gslots, fixed);
    return hp;
}

// run_plan: plan from runs of the triangles' two largest shells even where a
// pair cover would need fewer tiles (PYSPEC_CONTRACT_RUN_PLAN)
static HostPlan* get_plan(int nshell, const int32_t* tri_host, int ntri, bool run_plan = false) {
    std::vector<int32_t> key(tri_host, tri_host + 3 * (size_t)ntri);
    key.push_back(nshell);
    key.push_back(run_plan ? 1 : 0);
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_plans.find(key);
    if (it != g_plans.end()) return it->second;
    HostPlan* hp = build_plan(nshell, tri_host, ntri, !run_plan);
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

size_t contract_tc_ws(int64_t nvox, int nshell, int ntri, bool six) {
    // tables (bounded by the largest plan: 8 groups of 512 rows, slots <= ntri
    // + one gap slot per row and shell) + partials + error word
    (void)nshell;
    const size_t rows = (size_t)tc::MAXGROUPS * tc::MAXROWS;
    const size_t tables = rows * 4 * 2 + (size_t)tc::MAXGROUPS * tc::RT_PER_GROUP * tc::RT_WORDS * 4 +
                          (size_t)tc::MAXGROUPS * ((size_t)ntri + tc::MAXROWS * tc::MAXB) * 4 + 4096;
    const int64_t nchunks = (nvox + tc::KC - 1) / tc::KC;
    const size_t gx = (size_t)std::min<int64_t>(std::max<int64_t>(nchunks, 1), 1024);
    // the 6-product form keeps the partials of both passes
    return tc::al256(tables) + (six ? 2 : 1) * tc::al256(gx * (size_t)std::max(ntri, 1) * sizeof(double)) + 256;
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

// Launches the 64-voxel kernel for plan hp: with B-writer warps, or with
// three or two field buffers.
template <bool RES>
static int launch_tc64(const tc::HostPlan* hp, const tc::Params& X, unsigned gx, cudaStream_t st,
                       const CUtensorMap& fmap) {
    using namespace tc;
    const void* fn = hp->bw64 ? (const void*)contract_tc64_kernel<3, RES, true>
                     : hp->nfb64 == 3 ? (const void*)contract_tc64_kernel<3, RES, false>
                                      : (const void*)contract_tc64_kernel<2, RES, false>;
    PYSPEC_TRY(allow_smem(fn, hp->smem64));
    if (hp->bw64)
        contract_tc64_kernel<3, RES, true><<<dim3(gx, X.ngroups), NTHREADS64, hp->smem64, st>>>(X, fmap);
    else if (hp->nfb64 == 3)
        contract_tc64_kernel<3, RES, false><<<dim3(gx, X.ngroups), NTHREADS, hp->smem64, st>>>(X, fmap);
    else
        contract_tc64_kernel<2, RES, false><<<dim3(gx, X.ngroups), NTHREADS, hp->smem64, st>>>(X, fmap);
    return PYSPEC_OK;
}

int contract_tc_impl(const float* fields, int64_t nvox, int nshell, const int32_t* tri, const int32_t* tri_host,
                     int ntri, double* bsum, void* ws, size_t ws_bytes, cudaStream_t st, bool run_plan,
                     bool fine_drain, bool six, bool kc32) {
    using namespace tc;
    PYSPEC_CHECK_ARG(tri_host != nullptr, "the BF16x3 contraction needs the host copy of the triangle list");
    PYSPEC_CHECK_ARG(nvox % 4 == 0, "BF16x3 contraction needs N^3 divisible by 4");
    PYSPEC_CHECK_ARG(nvox / KC + 1 < (int64_t)INT32_MAX / KC, "BF16x3 contraction supports N^3 < 2^31");
    PYSPEC_CHECK_ARG(((uintptr_t)fields & 15) == 0, "fields must be 16-byte aligned");
    HostPlan* hp = get_plan(nshell, tri_host, ntri, run_plan);
    if (!hp->ok) {
        set_error("%s", hp->why);
        return hp->invalid ? PYSPEC_E_INVALID : PYSPEC_E_UNSUPPORTED;
    }
    const size_t need = contract_tc_ws(nvox, nshell, ntri, six);
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
    const int32_t* d_rt = reinterpret_cast<const int32_t*>(d_image + hp->off_rt);
    const int32_t* d_stri = reinterpret_cast<const int32_t*>(d_image + hp->off_stri);
    off += hp->image.size();
    off = al256(off);
    const int64_t nchunks = (nvox + KC - 1) / KC;
    const int gx = grid_x(nchunks, hp->base.ngroups);
    double* partials = reinterpret_cast<double*>(w + off);
    const int passes = six ? 2 : 1;
    if (off + al256((size_t)passes * gx * ntri * sizeof(double)) > ws_bytes) {
        set_error("contract workspace too small for %d CTAs", gx);
        return PYSPEC_E_WORKSPACE;
    }
    PYSPEC_CUDA(cudaMemcpyAsync(d_image, hp->image_src, hp->image.size(), cudaMemcpyHostToDevice, st));
    PYSPEC_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    PYSPEC_CUDA(cudaMemsetAsync(partials, 0, (size_t)passes * gx * ntri * sizeof(double), st));
    Params P = hp->base;
    P.V = nvox;
    P.nchunks = nchunks;
    P.chunks_per_cta = (nchunks + gx - 1) / gx;
    P.pair_row = d_rows;
    P.rt_tab = d_rt;
    P.slot_tri = d_stri;
    P.partials = partials;
    P.err = d_err;
    P.seg_log2 = (fine_drain || six) ? SEG_LOG2_FINE : SEG_LOG2;
    if (hp->nfb64 > 0 && !kc32) {
        // 64-voxel chunks: the same CTAs, half the chunks
        Params D = P;
        D.nchunks = (nvox + KC64 - 1) / KC64;
        D.chunks_per_cta = (D.nchunks + gx - 1) / gx;
        PYSPEC_TRY(launch_tc64<false>(hp, D, (unsigned)gx, st, fmap));
    } else {
        PYSPEC_TRY(allow_smem((const void*)contract_tc_kernel<false>, hp->smem));
        contract_tc_kernel<false><<<dim3(gx, P.ngroups), NTHREADS, hp->smem, st>>>(P, fmap);
    }
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    if (six) {
        // The 6-product form.  The first pass sums (P_hi + P_lo)(F_hi + F_lo):
        // the products and fields to 16 bits.  With x = hi + lo + res (the
        // third bf16 part, split2_res), the second pass adds
        // sum_v P_res F_hi + P_hi F_res -- the two largest of the terms the
        // first pass leaves out (the rest are ~2^-24 of B).  Same rows and
        // columns; narrow accumulator layout (N columns per tile), two MMAs
        // per tile and k-step; its own CTA partials, added with the first's.
        Params R = P;
        R.seg_log2 = SEG_LOG2;       // its terms are ~2^-16 of B: the default drain is ample
        R.partials = partials + (size_t)gx * ntri;
        for (int g = 0; g < R.ngroups; ++g) {
            Group& G = R.g[g];
            int col = 0;
            for (int t = 0; t < G.ntiles; ++t) {
                G.tile_n[t] = (G.tile_n[t] + 15) / 16 * 16;     // narrow: N a multiple of 16
                G.tile_col[t] = col;
                col += G.tile_n[t];
            }
            G.wide = 0;
            G.ncols = pow2_cols(col + NSTAGE * MAXTILES * ACOLS);
        }
        if (hp->nfb64 > 0 && !kc32) {
            // 64-voxel chunks for this pass too
            R.nchunks = (nvox + KC64 - 1) / KC64;
            R.chunks_per_cta = (R.nchunks + gx - 1) / gx;
            PYSPEC_TRY(launch_tc64<true>(hp, R, (unsigned)gx, st, fmap));
        } else {
            PYSPEC_TRY(allow_smem((const void*)contract_tc_kernel<true>, hp->smem));
            contract_tc_kernel<true><<<dim3(gx, R.ngroups), NTHREADS, hp->smem, st>>>(R, fmap);
        }
        PYSPEC_LAUNCH_CHECK();
        count_launch();
    }
    (void)tri;
    return reduce_partials_launch(partials, passes * gx, ntri, bsum, st);
}

// Verifies a built plan against its triangle list (see pyspec_bk_plan_check).
static bool check_plan(const tc::HostPlan* hp, const int32_t* tri_host, int ntri, char* why, size_t nwhy) {
    using namespace tc;
    const Params& P = hp->base;
    std::vector<int> seen(ntri, 0);
    for (int g = 0; g < P.ngroups; ++g) {
        const Group& G = P.g[g];
        for (int r = 0; r < MAXROWS; ++r) {
            const int16_t* pr = &hp->pair_row[((size_t)G.table_off + r) * 4];
            if (pr[0] < 0) continue;
            const int i = pr[0] & 0xff, j = (pr[0] >> 8) & 0xff, lmin = pr[1], lmax = pr[2];
            const int tile = r / 128, q = (r % 128) / 32, x = r % 8, y = (r % 32) / 8;
            const int tp = tile / 2, u = tile % 2;
            const int32_t* w = &hp->rt_tab[((size_t)g * RT_PER_GROUP + tp * 32 + q * 8 + x) * RT_WORDS];
            const int ri = (w[0] >> (8 * u)) & 0xff, rg = (w[1 + u] >> (8 * y)) & 0xff;
            if (tile >= G.ntiles || ri != i || rg != j || lmin > lmax || lmax >= G.tile_n[tile] ||
                pr[3] + (lmax - lmin) >= G.nslots) {
                snprintf(why, nwhy, "group %d row %d: shells (%d, %d), table (%d, %d), columns [%d, %d]", g, r, i, j,
                         ri, rg, lmin, lmax);
                return false;
            }
            for (int l = lmin; l <= lmax; ++l) {
                const int t = hp->slot_tri[(size_t)g * P.maxslots + pr[3] + (l - lmin)];
                if (t < 0) continue;
                if (t >= ntri) {
                    snprintf(why, nwhy, "group %d row %d: slot holds triangle %d of %d", g, r, t, ntri);
                    return false;
                }
                int a[3] = {i, j, l}, b[3] = {tri_host[t], tri_host[ntri + t], tri_host[2 * ntri + t]};
                std::sort(a, a + 3);
                std::sort(b, b + 3);
                if (a[0] != b[0] || a[1] != b[1] || a[2] != b[2]) {
                    snprintf(why, nwhy, "triangle %d read at shells (%d, %d, %d)", t, i, j, l);
                    return false;
                }
                ++seen[t];
            }
        }
    }
    for (int t = 0; t < ntri; ++t)
        if (seen[t] != 1) {
            snprintf(why, nwhy, "triangle %d is read %d times", t, seen[t]);
            return false;
        }
    return true;
}

}  // namespace pyspec

extern "C" int pyspec_bk_plan_check(int nshell, const int32_t* tri_host, int ntri, int64_t* info, int ninfo) {
    return pyspec_bk_plan_check_flags(nshell, tri_host, ntri, 0, info, ninfo);
}

extern "C" int pyspec_bk_plan_check_flags(int nshell, const int32_t* tri_host, int ntri, int flags, int64_t* info,
                                          int ninfo) {
    using namespace pyspec;
    using namespace pyspec::tc;
    PYSPEC_CHECK_ARG(tri_host != nullptr && ntri > 0, "empty or NULL triangle list");
    PYSPEC_CHECK_ARG(nshell >= 1 && ninfo >= 0 && (info != nullptr || ninfo == 0), "bad arguments");
    PYSPEC_CHECK_ARG((flags & ~(PYSPEC_CONTRACT_RUN_PLAN | PYSPEC_CONTRACT_KC32)) == 0, "unknown plan flags 0x%x", flags);
    HostPlan* hp = get_plan(nshell, tri_host, ntri, (flags & PYSPEC_CONTRACT_RUN_PLAN) != 0);
    if (!hp->ok) {
        set_error("%s", hp->why);
        return hp->invalid ? PYSPEC_E_INVALID : PYSPEC_E_UNSUPPORTED;
    }
    char why[200];
    if (!check_plan(hp, tri_host, ntri, why, sizeof(why))) {
        set_error("contraction plan check failed: %s", why);
        return PYSPEC_E_INVALID;
    }
    const Params& P = hp->base;
    int64_t mma = 0, macs = 0;
    for (int g = 0; g < P.ngroups; ++g) {
        const Group& G = P.g[g];
        mma += (int64_t)G.ntiles * (KC / 16) * (G.wide ? 2 : 3);
        // tensor MACs per voxel: per tile M = 128 rows x (2 MMAs x 2N columns, or 3 x N)
        for (int t = 0; t < G.ntiles; ++t) macs += 128 * (G.wide ? 2 * 2 * G.tile_n[t] : 3 * G.tile_n[t]);
    }
    // shared-memory bank clashes between the row threads that share a
    // quarter-warp load phase (entries 2p, 2p + 1): their F_i0, F_i1 and the
    // four g loads (and the second slot's g where it has its own)
    int64_t clashes = 0;
    auto clash = [](int r, int t) { return r != t && ((r >> 2) & 1) == ((t >> 2) & 1); };
    for (int g = 0; g < P.ngroups; ++g)
        for (int e = 0; e < RT_PER_GROUP; e += 2) {
            const int32_t* a = &hp->rt_tab[((size_t)g * RT_PER_GROUP + e) * RT_WORDS];
            const int32_t* b = a + RT_WORDS;
            for (int k = 0; k < 2; ++k) clashes += clash((a[0] >> (8 * k)) & 0xff, (b[0] >> (8 * k)) & 0xff);
            for (int y = 0; y < 4; ++y) clashes += clash((a[1] >> (8 * y)) & 0xff, (b[1] >> (8 * y)) & 0xff);
            if (a[2] != a[1] || b[2] != b[1])
                for (int y = 0; y < 4; ++y) clashes += clash((a[2] >> (8 * y)) & 0xff, (b[2] >> (8 * y)) & 0xff);
        }
    const bool deep = hp->nfb64 > 0 && !(flags & PYSPEC_CONTRACT_KC32);
    const int64_t vals[10] = {P.ngroups, P.g[0].ntiles, hp->cover ? 1 : 0, mma, P.g[0].nslots, P.g[0].wide, macs,
                              clashes, deep ? KC64 : KC, (deep && hp->bw64) ? 1 : 0};
    for (int k = 0; k < ninfo && k < 10; ++k) info[k] = vals[k];
    return PYSPEC_OK;
}
