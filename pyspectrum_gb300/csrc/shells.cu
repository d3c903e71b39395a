// Shell fields F_j(x) = Re FFT_forward(delta(k) [irk(k) == j]) for every
// shell j (pyspectrum.py:384-404), as three pruned passes on the half grid:
//
//   S1  z-lines : mask by shell, complex FFT along z      (half grid -> work)
//   S2  y-lines : complex FFT along y                      (work, in place)
//   S3  x-rows  : complex-to-real FFT along x, sum of F^2  (work -> fields)
//
// A mode k = (x, y, z) lies in shell j when d2lo <= x^2 + y'^2 + z'^2 <= d2hi
// (y' = min(y, N-y)), the exact integer form of int(|k|/step + 0.5) == j.
// S1 only visits columns (x, y) that can reach the shell; S2 only x blocks
// with x <= |k|max; S3 treats everything S2 skipped as zero.  Small shells
// therefore touch a small part of the work grid, which then stays in L2.
//
// The C2R step uses the classic half-length trick: for a Hermitian spectrum
// X[0..N/2] the N real outputs f are, as N/2 complex values, the length-N/2
// FFT of Z[k] = (X[k] + conj X[N/2-k]) + i e^{-2 pi i k/N} (X[k] - conj X[N/2-k]),
// with X[0] and X[N/2] replaced by their real parts -- this equals
// Re(sum over the full grid) for any half grid, which is what the reference's
// np.real(fftn(...)) computes.
#include <algorithm>
#include "fft_device.cuh"
#include "fft3d.cuh"
#include "shells.cuh"

namespace pyspec {

__host__ __device__ inline int64_t shell_d2lo(int j, int step) {
    if (j <= 0) return 0;
    const int64_t a = (int64_t)(2 * j - 1) * step;
    return (a * a + 3) / 4;            // ceil(a^2/4)
}
__host__ __device__ inline int64_t shell_d2hi(int j, int step) {
    const int64_t a = (int64_t)(2 * j + 1) * step;
    return (a * a + 3) / 4 - 1;        // ceil(a^2/4) - 1
}

__device__ __forceinline__ int fold(int i, int n) { return i <= n - i ? i : n - i; }

// Row stride (in complex elements) of the work grid: n/2+1 rounded up so that
// every row starts on a 16-byte boundary (the x pass copies rows in 16-byte
// pieces).
// Row stride of the work grid (complex elements).  Single precision: an odd
// multiple of 8 elements (64 bytes), so the 64-byte column tiles of the z / y
// passes never straddle a 128-byte line and consecutive rows start on
// different 128-byte phases (measured at 360^3, 40 shells: stride 182 4.06 ms,
// 184 3.82, 192 3.93, 200 3.91).
template <typename C>
__host__ __device__ constexpr int work_stride(int n) {
    return sizeof(C) == 8 ? (((n / 2 + 1) + 7) / 8 % 2 == 1 ? ((n / 2 + 1) + 7) / 8 * 8 : ((n / 2 + 1) + 7) / 8 * 8 + 8)
                          : n / 2 + 1;
}

// rows of the x pass handled by one CTA
__host__ __device__ constexpr int xpass_rows_ct(int n) {
    return (4096 / n) < 1 ? 1 : ((4096 / n) > 16 ? 16 : 4096 / n);
}

// Twiddle tables for the forward (sign -1) transforms of one call, computed
// once into the workspace: exp(-2 pi i m/n) for m < n, then exp(-2 pi i m/(n/2)).
template <typename T>
__global__ void twiddle_table_kernel(typename cplx_t<T>::type* tab, int n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    fill_twiddles<T>(tab, n, -1, t, gridDim.x * blockDim.x);
    fill_twiddles<T>(tab + n, n / 2, -1, t, gridDim.x * blockDim.x);
}

template <typename C>
__device__ __forceinline__ void copy_table(C* dst, const C* __restrict__ src, int m) {
    for (int i = threadIdx.x; i < m; i += blockDim.x) dst[i] = src[i];
}

template <typename T, bool INDICATOR, int NC>
__global__ void __launch_bounds__(256) shell_zpass_kernel(const typename cplx_t<T>::type* __restrict__ half,
                                                          typename cplx_t<T>::type* __restrict__ work, int n_rt,
                                                          int64_t d2lo, int64_t d2hi, RadixPlan plan,
                                                          const typename cplx_t<T>::type* __restrict__ twg) {
    using C = typename cplx_t<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = NC > 0 ? NC : n_rt;
    const int nh = n / 2 + 1;
    constexpr int tx = tile_x<T>();
    const int ntx = (nh + tx - 1) / tx;
    const int y = blockIdx.x / ntx;
    const int x0 = (blockIdx.x % ntx) * tx;
    const int yf = fold(y, n);
    if ((int64_t)x0 * x0 + (int64_t)yf * yf > d2hi) return;   // whole tile outside the shell
    C* tw = reinterpret_cast<C*>(smem_raw);
    C* buf0 = tw + n;
    C* buf1 = buf0 + (size_t)tx * n;
    copy_table(tw, twg, n);
    const int ncol = min(tx, nh - x0);
    const int64_t zstride = (int64_t)n * nh;
    const int64_t base = (int64_t)y * nh + x0;
    const int ws = work_stride<C>(n);
    const int64_t wzstride = (int64_t)n * ws;
    const int64_t wbase = (int64_t)y * ws + x0;
    for (int i = threadIdx.x; i < n * tx; i += blockDim.x) {
        const int z = i / tx, c = i - z * tx;
        C v = mk<T>(0, 0);
        if (c < ncol) {
            const int x = x0 + c, zf = fold(z, n);
            const int64_t d2 = (int64_t)x * x + (int64_t)yf * yf + (int64_t)zf * zf;
            if (d2 >= d2lo && d2 <= d2hi) {
                if constexpr (INDICATOR) v = mk<T>(1, 0);
                else v = half[base + z * zstride + c];
            }
        }
        buf0[i] = v;
    }
    __syncthreads();
    C* res;
    if constexpr (NC > 0) res = ct::fft_tile_ct<T, NC, tx, 0>(buf0, buf1, tw, -1);
    else res = fft_tile<T, tx>(buf0, buf1, tw, plan, tx, -1);
    // pairs of elements per store where a pair is 16 bytes (rows of the work
    // grid are 16-byte aligned and padded, x0 is even)
    constexpr int VEC = sizeof(C) == 8 ? 2 : 1;
    for (int i = threadIdx.x; i < n * (tx / VEC); i += blockDim.x) {
        const int z = i / (tx / VEC), c = (i - z * (tx / VEC)) * VEC;
        if (c >= ncol) continue;
        if constexpr (VEC == 2) {
            const C a = res[z * tx + c], b = res[z * tx + c + 1];
            *reinterpret_cast<float4*>(&work[wbase + z * wzstride + c]) = make_float4(a.x, a.y, b.x, b.y);
        } else {
            work[wbase + z * wzstride + c] = res[z * tx + c];
        }
    }
}

template <typename T, int NC>
__global__ void __launch_bounds__(256) shell_ypass_kernel(typename cplx_t<T>::type* __restrict__ work, int n_rt,
                                                          int64_t d2hi, int ntx_active, RadixPlan plan,
                                                          const typename cplx_t<T>::type* __restrict__ twg) {
    using C = typename cplx_t<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = NC > 0 ? NC : n_rt;
    const int nh = n / 2 + 1;
    constexpr int tx = tile_x<T>();
    const int z = blockIdx.x / ntx_active;
    const int x0 = (blockIdx.x % ntx_active) * tx;
    C* tw = reinterpret_cast<C*>(smem_raw);
    C* buf0 = tw + n;
    C* buf1 = buf0 + (size_t)tx * n;
    copy_table(tw, twg, n);
    const int ncol = min(tx, nh - x0);
    const int ws = work_stride<C>(n);
    const int64_t base = (int64_t)z * n * ws + x0;
    constexpr int VEC = sizeof(C) == 8 ? 2 : 1;   // elements per 16-byte access
    for (int i = threadIdx.x; i < n * (tx / VEC); i += blockDim.x) {
        const int y = i / (tx / VEC), c = (i - y * (tx / VEC)) * VEC;
        const int yf = fold(y, n);
        // rows the z pass did not visit hold zeros
        const bool live = c < ncol && (int64_t)x0 * x0 + (int64_t)yf * yf <= d2hi;
        if constexpr (VEC == 2) {
            float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
            if (live) q = *reinterpret_cast<const float4*>(&work[base + (int64_t)y * ws + c]);
            buf0[y * tx + c] = mk<T>(q.x, q.y);
            buf0[y * tx + c + 1] = mk<T>(q.z, q.w);
        } else {
            buf0[y * tx + c] = live ? work[base + (int64_t)y * ws + c] : mk<T>(0, 0);
        }
    }
    __syncthreads();
    C* res;
    if constexpr (NC > 0) res = ct::fft_tile_ct<T, NC, tx, 0>(buf0, buf1, tw, -1);
    else res = fft_tile<T, tx>(buf0, buf1, tw, plan, tx, -1);
    for (int i = threadIdx.x; i < n * (tx / VEC); i += blockDim.x) {
        const int y = i / (tx / VEC), c = (i - y * (tx / VEC)) * VEC;
        if (c >= ncol) continue;
        if constexpr (VEC == 2) {
            const C a = res[y * tx + c], b = res[y * tx + c + 1];
            *reinterpret_cast<float4*>(&work[base + (int64_t)y * ws + c]) = make_float4(a.x, a.y, b.x, b.y);
        } else {
            work[base + (int64_t)y * ws + c] = res[y * tx + c];
        }
    }
}

// z and y lines for the common grid sizes, in registers: a CTA transforms
// the 8 columns x0..x0+7 of one tile (8 lines of length N = R1*R2) in two
// radix stages.  Stage 1 loads its inputs straight from HBM (8 consecutive
// columns = 64 contiguous bytes per row), applies radix-R1 butterflies and
// writes them to a padded per-column buffer in shared memory; after one
// barrier stage 2 applies the twiddles and radix-R2 butterflies and stores
// the results straight to the work grid.  Thread t handles column t % 8.
//   ZPASS: lines along z, input = delta(k) masked by the shell (or the shell
//          indicator), output = work.  Tiles outside the shell return at once.
//   else:  lines along y, in place in work; rows the z pass did not visit
//          read as zeros.
template <int NC, int R1, int R2>
struct LinePassShape {
    static constexpr int NB1 = NC / (R1 > 0 ? R1 : 1), NB2 = NC / (R2 > 0 ? R2 : 1);   // butterflies per line
    static constexpr int THREADS = 8 * (NB1 > NB2 ? NB1 : NB2);
    // padded column: element p at p + p / R1; stride == 2 (mod 16) complex so
    // the 8 columns of a half-warp fall in different banks
    static constexpr int COLP = ((NC + NB1 + 13) / 16) * 16 + 2;
};

template <int NC, int R1, int R2, bool ZPASS, bool INDICATOR>
__global__ void __launch_bounds__(LinePassShape<NC, R1, R2>::THREADS)
shell_line_pass_kernel(const float2* __restrict__ half, float2* __restrict__ work, int64_t d2lo, int64_t d2hi,
                       int ntx_tiles, const float2* __restrict__ twg) {
    using S = LinePassShape<NC, R1, R2>;
    constexpr int N = NC, NH = N / 2 + 1, WS = work_stride<float2>(N);
    static_assert(R1 * R2 == N, "two radix stages");
    __shared__ float2 buf[8 * S::COLP];
    const int tile = blockIdx.x % ntx_tiles;
    const int other = blockIdx.x / ntx_tiles;   // y (z pass) or z (y pass)
    const int x0 = tile * 8;
    const int c = threadIdx.x & 7, b = threadIdx.x >> 3;
    const int x = x0 + c;
    const bool colok = x < NH;
    const int of = fold(other, N);
    if (ZPASS && (int64_t)x0 * x0 + (int64_t)of * of > d2hi) return;   // whole tile outside the shell
    float2* col = buf + c * S::COLP;
    // ---- stage 1: radix R1, butterfly b over elements b + r*NB1 ----
    if (b < S::NB1) {
        float2 v[R1];
#pragma unroll
        for (int r = 0; r < R1; ++r) {
            const int e = b + r * S::NB1;       // position along the line
            const int ef = fold(e, N);
            float2 val = make_float2(0.f, 0.f);
            if constexpr (ZPASS) {
                const int64_t d2 = (int64_t)x * x + (int64_t)of * of + (int64_t)ef * ef;
                if (colok && d2 >= d2lo && d2 <= d2hi) {
                    if constexpr (INDICATOR) val = make_float2(1.f, 0.f);
                    else val = half[((int64_t)e * N + other) * NH + x];
                }
            } else {
                if (colok && (int64_t)x0 * x0 + (int64_t)ef * ef <= d2hi)
                    val = work[((int64_t)other * N + e) * WS + x];
            }
            v[r] = val;
        }
        small_dft<float, float2, R1>(v, -1);
#pragma unroll
        for (int r = 0; r < R1; ++r) col[b * (R1 + 1) + r] = v[r];   // element b*R1 + r
    }
    __syncthreads();
    // ---- stage 2: radix R2, butterfly j over elements j + r*NB2, twiddle exp(-2 pi i r j / N) ----
    if (b < S::NB2 && colok) {
        float2 v[R2];
#pragma unroll
        for (int r = 0; r < R2; ++r) {
            const int p = b + r * S::NB2;                     // element index (< N)
            const float2 u = col[p + p / R1];
            v[r] = r == 0 || b == 0 ? u : cmul(u, __ldg(&twg[r * b]));
        }
        small_dft<float, float2, R2>(v, -1);
#pragma unroll
        for (int r = 0; r < R2; ++r) {
            const int e = b + r * S::NB2;                       // output position along the line
            if constexpr (ZPASS) work[((int64_t)e * N + other) * WS + x] = v[r];
            else work[((int64_t)other * N + e) * WS + x] = v[r];
        }
    }
}

// x rows: a persistent CTA walks blocks of RL consecutive rows r = z*n + y.
// The rows of the next block are copied into the other staging buffer with
// cp.async while the current block is transformed, so the loads are always in
// flight.  Warp w stages and packs rows w, w+8, ... (no divisions).
template <typename T, int NC>
__global__ void __launch_bounds__(256) shell_xpass_kernel(const typename cplx_t<T>::type* __restrict__ work, int n_rt,
                                                          int xlim, int rl_rt, RadixPlan plan_half,
                                                          T* __restrict__ field, double* __restrict__ part,
                                                          const typename cplx_t<T>::type* __restrict__ twg) {
    using C = typename cplx_t<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = NC > 0 ? NC : n_rt;
    const int rl = NC > 0 ? xpass_rows_ct(NC) : rl_rt;
    const int h = n / 2;
    const int ws = work_stride<C>(n);          // row stride of the work grid and the staging rows
    C* twN = reinterpret_cast<C*>(smem_raw);   // exp(-2 pi i m / n), m < n
    C* twH = twN + n;                          // exp(-2 pi i m / (n/2))
    // 2 x rl * ws staging rows, 16-byte aligned for the asynchronous copies
    C* stage0 = reinterpret_cast<C*>((reinterpret_cast<uintptr_t>(twH + h) + 15) & ~(uintptr_t)15);
    C* buf0 = stage0 + 2 * (size_t)rl * ws;    // rl * h
    C* buf1 = buf0 + (size_t)rl * h;
    __shared__ double red[32];
    copy_table(twN, twg, n + h);               // both tables are contiguous
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    const int64_t nrows = (int64_t)n * n;
    const int64_t nblocks = (nrows + rl - 1) / rl;
    // 16-byte pieces of a row holding its first xlim elements (the rest is
    // treated as zero when the row is packed)
    const int npiece = (int)(((size_t)xlim * sizeof(C) + 15) / 16);
    auto issue = [&](int64_t blk, int sbuf) {
        if (blk < nblocks) {
            const int64_t r0 = blk * rl;
            const int nr = (int)min((int64_t)rl, nrows - r0);
            C* st = stage0 + (size_t)sbuf * rl * ws;
            for (int rr = warp; rr < nr; rr += nwarp) {
                const char* src = reinterpret_cast<const char*>(work + (r0 + rr) * ws);
                const uint32_t dst = (uint32_t)__cvta_generic_to_shared(st + rr * ws);
                for (int q = lane; q < npiece; q += 32)
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" :: "r"(dst + (uint32_t)(q * 16)),
                                 "l"(src + (size_t)q * 16) : "memory");
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    T local = 0;
    int sb = 0;
    issue(blockIdx.x, 0);
    for (int64_t blk = blockIdx.x; blk < nblocks; blk += gridDim.x, sb ^= 1) {
        issue(blk + gridDim.x, sb ^ 1);
        asm volatile("cp.async.wait_group 1;" ::: "memory");
        __syncthreads();
        const int64_t r0 = blk * rl;
        const int nr = (int)min((int64_t)rl, nrows - r0);
        const C* st = stage0 + (size_t)sb * rl * ws;
        for (int rr = warp; rr < nr; rr += nwarp) {
            const C* X = st + rr * ws;
            C* out = buf0 + rr * h;
            for (int k = lane; k < h; k += 32) {
                C a = k < xlim ? X[k] : mk<T>(0, 0);
                C b = h - k < xlim ? X[h - k] : mk<T>(0, 0);
                if (k == 0) { a.y = 0; b.y = 0; }
                const C bc = mk<T>(b.x, -b.y);
                const C e = cadd(a, bc);
                const C o = cmul(csub(a, bc), twN[k]);
                out[k] = mk<T>(e.x - o.y, e.y + o.x);   // e + i*o
            }
        }
        __syncthreads();
        C* res;
        if constexpr (NC > 0) res = ct::fft_tile_ct<T, NC / 2, 0, xpass_rows_ct(NC)>(buf0, buf1, twH, -1);
        else res = fft_tile<T, 0>(buf0, buf1, twH, plan_half, nr, -1);
        C* out = reinterpret_cast<C*>(field + r0 * n);
        for (int i = threadIdx.x; i < nr * h; i += blockDim.x) {
            const C v = res[i];
            out[i] = v;       // f[2m] = Re z[m], f[2m+1] = Im z[m]; rows are contiguous
            local += v.x * v.x + v.y * v.y;
        }
        __syncthreads();      // buffers are rewritten by the next block
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    double acc = (double)local;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < nwarp ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) part[blockIdx.x] = v;
    }
}

// x rows for the common grid sizes, with the half-length FFT of H = R1*R2
// points done in registers: a warp transforms two rows at a time (16 lanes
// per row).  The next pair of rows is copied into a per-warp staging buffer
// by two bulk copies (TMA, cp.async.bulk: one per row, issued by lane 0,
// completing on the warp's barrier of that stage) while the current pair is
// transformed, so the row loads are always in flight.  Stage 1 reads its inputs from the staging buffer, forms
// Z[k] (the C2R packing above) and applies radix-R1 butterflies; the outputs
// cross lanes once through a padded per-row buffer in shared memory (one pad
// element per R1, so neither side has bank conflicts); stage 2 applies the
// twiddles and radix-R2 butterflies and stores the row of F directly.  No
// block-wide barrier: each warp only synchronises with itself.
template <int NC, int R1, int R2>
__host__ __device__ constexpr size_t xpass_reg_smem() {
    return (size_t)8 * 2 * 2 * work_stride<float2>(NC) * sizeof(float2);   // 8 warps x 2 stages x 2 rows
}

template <int NC, int R1, int R2>
__global__ void __launch_bounds__(256, 3) shell_xpass_reg_kernel(const float2* __restrict__ work, int xlim,
                                                              float* __restrict__ field, double* __restrict__ part,
                                                              const float2* __restrict__ twg) {
    constexpr int N = NC, H = N / 2, WS = work_stride<float2>(N);
    static_assert(R1 * R2 == H && R1 <= 16 && R2 <= 16, "two radix stages of at most 16 lanes");
    constexpr int PADH = H + R2;                 // R2 butterflies x (R1 + 1) slots
    __shared__ float2 twN[H];                    // exp(-2 pi i k / N), k < H
    __shared__ float2 twH[H];                    // exp(-2 pi i m / H)
    __shared__ float2 rowbuf[8][2][PADH];
    __shared__ double red[8];
    __shared__ __align__(8) uint64_t stg_bar[8][2];        // per warp and stage: its two rows' bulk copies
    extern __shared__ __align__(16) float2 stage_all[];   // [warp][stage][row][WS]
    for (int i = threadIdx.x; i < H; i += blockDim.x) {
        twN[i] = twg[i];
        twH[i] = twg[N + i];
    }
    if (threadIdx.x < 16) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;"
                     :: "r"((uint32_t)__cvta_generic_to_shared(&stg_bar[threadIdx.x >> 1][threadIdx.x & 1])), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane >> 4, t = lane & 15;
    float2* buf = rowbuf[warp][sub];
    float2* stg = stage_all + (size_t)warp * 2 * 2 * WS;
    const int64_t nrows = (int64_t)N * N;        // even: rows come in pairs
    const int64_t nw = (int64_t)gridDim.x * 8;
    // the first xlim elements of a row in 16-byte pieces (rows start on
    // 16-byte boundaries: the work-grid stride is a multiple of 8 elements)
    const uint32_t row_bytes = (uint32_t)((xlim + 1) / 2) * 16u;
    const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(&stg_bar[warp][0]);
    // one bulk copy (TMA) per row of the pair starting at r0 into stage sb,
    // completing on the warp's barrier of that stage; lane 0 issues them
    // after the warp's reads of the stage (fenced against the async proxy)
    uint32_t pending = 0u, phase = 0u;   // bit sb: stage sb has a copy in flight / its next parity
    auto issue = [&](int64_t r0, int sb) {
        if (r0 >= nrows) return;
        pending |= 1u << sb;
        if (lane == 0) {
            const uint32_t bar = bar0 + 8u * (uint32_t)sb;
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(2u * row_bytes)
                         : "memory");
#pragma unroll
            for (int rr = 0; rr < 2; ++rr) {
                const uint32_t dst = (uint32_t)__cvta_generic_to_shared(stg + ((size_t)sb * 2 + rr) * WS);
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                    :: "r"(dst), "l"(work + (r0 + rr) * WS), "r"(row_bytes), "r"(bar) : "memory");
            }
        }
    };
    // all lanes wait for stage sb (bounded: ~2 s, then false)
    auto wait_stage = [&](int sb) -> bool {
        const uint32_t bar = bar0 + 8u * (uint32_t)sb;
        uint32_t ok = 0;
        unsigned long long t0 = 0;
        for (uint32_t it = 0;; ++it) {
            asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                         : "=r"(ok) : "r"(bar), "r"((phase >> sb) & 1u) : "memory");
            if (ok) break;
            if ((it & 255u) == 0) {
                unsigned long long t;
                asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
                if (t0 == 0) t0 = t;
                else if (t - t0 > 2000000000ull) return false;
            }
        }
        phase ^= 1u << sb;
        pending &= ~(1u << sb);
        return true;
    };
    float local = 0.f;
    int sb = 0;
    int64_t r0 = ((int64_t)blockIdx.x * 8 + warp) * 2;
    issue(r0, 0);
    for (; r0 < nrows; r0 += nw * 2, sb ^= 1) {
        issue(r0 + nw * 2, sb ^ 1);
        if (!__all_sync(0xffffffffu, wait_stage(sb))) {
            local = __int_as_float(0x7fc00000);   // NaN: the shell's sum of squares reports the failure
            break;
        }
        const int64_t row = r0 + sub;
        const float2* X = stg + ((size_t)sb * 2 + sub) * WS;
        if (t < R2) {
            float2 v[R1];
#pragma unroll
            for (int r = 0; r < R1; ++r) {
                const int k = t + r * R2;
                float2 a = k < xlim ? X[k] : make_float2(0.f, 0.f);
                float2 b = H - k < xlim ? X[H - k] : make_float2(0.f, 0.f);
                if (k == 0) { a.y = 0.f; b.y = 0.f; }
                const float2 bc = make_float2(b.x, -b.y);
                const float2 e = cadd(a, bc);
                const float2 o = cmul(csub(a, bc), twN[k]);
                v[r] = make_float2(e.x - o.y, e.y + o.x);      // e + i*o
            }
            small_dft<float, float2, R1>(v, -1);
#pragma unroll
            for (int r = 0; r < R1; ++r) buf[t * (R1 + 1) + r] = v[r];   // element t*R1 + r
        }
        __syncwarp();
        if (t < R1) {
            float2 v[R2];
#pragma unroll
            for (int r = 0; r < R2; ++r) {
                const float2 x = buf[t + r * (R1 + 1)];                   // element t + r*R1
                v[r] = r == 0 ? x : cmul(x, twH[r * t]);                  // r*t < H
            }
            small_dft<float, float2, R2>(v, -1);
            float2* out = reinterpret_cast<float2*>(field + row * N);
#pragma unroll
            for (int r = 0; r < R2; ++r) {
                out[t + r * R1] = v[r];       // f[2m] = Re z[m], f[2m+1] = Im z[m]
                local += v[r].x * v[r].x + v[r].y * v[r].y;
            }
        }
        __syncwarp();                         // buf and this stage are rewritten later
    }
    // no copy may land after the CTA exits: wait (bounded) for any in flight
    for (int k = 0; k < 2; ++k)
        if ((pending >> k) & 1u) (void)__all_sync(0xffffffffu, wait_stage(k));
    double acc = (double)local;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < 8; ++w) v += red[w];
        part[blockIdx.x] = v;
    }
}

__global__ void reduce_rows_kernel(const double* __restrict__ part, int nper, double* __restrict__ out) {
    // one block per output; fixed-order tree reduction (deterministic)
    __shared__ double red[32];
    const double* p = part + (int64_t)blockIdx.x * nper;
    double acc = 0.0;
    for (int i = threadIdx.x; i < nper; i += blockDim.x) acc += p[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) out[blockIdx.x] = v;
    }
}

static int xpass_rows(int n) { return xpass_rows_ct(n); }

// persistent x-pass CTAs: a few per SM, never more than there are row blocks
static int xpass_ctas(int n) {
    int sms = 152, dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t blocks = ((int64_t)n * n + xpass_rows(n) - 1) / xpass_rows(n);
    return (int)std::min<int64_t>(blocks, (int64_t)sms * 3);
}

template <typename T>
size_t shell_workspace_bytes(int n, int nshell) {
    using C = typename cplx_t<T>::type;
    const size_t nblk = (size_t)xpass_ctas(n);
    size_t b = (size_t)work_stride<C>(n) * n * n * sizeof(C);
    b = (b + 255) & ~(size_t)255;
    b += (size_t)nshell * nblk * sizeof(double);
    b = (b + 255) & ~(size_t)255;
    b += (size_t)(n + n / 2) * sizeof(C);          // twiddle tables
    return b;
}

// radix split H = R1 * R2 of the register x pass per grid size
// radix split N = R1 * R2 of the register z / y line pass per grid size (0: none)
constexpr int LR1(int n) { return n == 360 ? 20 : n == 192 ? 16 : n == 256 ? 16 : 0; }
constexpr int LR2(int n) { return n == 360 ? 18 : n == 192 ? 12 : n == 256 ? 16 : 1; }
constexpr int XR1(int n) { return n == 360 ? 12 : n == 192 ? 8 : n == 256 ? 8 : n == 512 ? 16 : 1; }
constexpr int XR2(int n) { return n == 360 ? 15 : n == 192 ? 12 : n == 256 ? 16 : n == 512 ? 16 : 1; }

template <typename T, bool INDICATOR>
int shell_one_impl(const typename cplx_t<T>::type* half, int n, int step, int j, T* field, double* part,
                   typename cplx_t<T>::type* work, const typename cplx_t<T>::type* tw, cudaStream_t st) {
    using C = typename cplx_t<T>::type;
    RadixPlan plan, plan_half;
    PYSPEC_CHECK_ARG(n % 2 == 0 && make_plan(n, &plan) && make_plan(n / 2, &plan_half),
                     "ngrid=%d must be even and factor into 2, 3 and 5", n);
    const int nh = n / 2 + 1, tx = tile_x<T>();
    const int64_t d2lo = shell_d2lo(j, step), d2hi = shell_d2hi(j, step);
    // largest |kx| that can reach the shell (bounded by the half grid)
    int kmax = 0;
    while ((int64_t)(kmax + 1) * (kmax + 1) <= d2hi && kmax + 1 < nh) ++kmax;
    const int ntx = (nh + tx - 1) / tx;
    const int ntx_active = min(ntx, kmax / tx + 1);
    const int xlim = min(nh, ntx_active * tx);
    const size_t sm_zy = sizeof(C) * ((size_t)n + 2 * (size_t)tx * n);
    const int rl = xpass_rows(n);
    const int h = n / 2;
    const size_t sm_x = sizeof(C) * ((size_t)n + h + 2 * (size_t)rl * work_stride<C>(n) + 2 * (size_t)rl * h) + 16;
    const unsigned nblk = (unsigned)xpass_ctas(n);
    // compile-time plans for the common grid sizes (single precision)
#define PYSPEC_SHELL_LAUNCH(NCV)                                                                          \
    do {                                                                                                 \
        PYSPEC_TRY(allow_smem((const void*)shell_zpass_kernel<T, INDICATOR, NCV>, sm_zy));               \
        PYSPEC_TRY(allow_smem((const void*)shell_ypass_kernel<T, NCV>, sm_zy));                          \
        PYSPEC_TRY(allow_smem((const void*)shell_xpass_kernel<T, NCV>, sm_x));                           \
        if constexpr (NCV > 0 && sizeof(T) == 4)                                                         \
            PYSPEC_CUDA(cudaFuncSetAttribute((const void*)shell_xpass_reg_kernel<NCV, XR1(NCV), XR2(NCV)>,  \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,                \
                                             (int)xpass_reg_smem<NCV, XR1(NCV), XR2(NCV)>()));           \
        if constexpr (LR1(NCV) > 0 && sizeof(T) == 4) {                                                   \
            using LS = LinePassShape<NCV, LR1(NCV), LR2(NCV)>;                                            \
            shell_line_pass_kernel<NCV, LR1(NCV), LR2(NCV), true, INDICATOR>                               \
                <<<(unsigned)(ntx * n), LS::THREADS, 0, st>>>(reinterpret_cast<const float2*>(half),      \
                    reinterpret_cast<float2*>(work), d2lo, d2hi, ntx, reinterpret_cast<const float2*>(tw)); \
            PYSPEC_LAUNCH_CHECK();                                                                       \
            shell_line_pass_kernel<NCV, LR1(NCV), LR2(NCV), false, INDICATOR>                              \
                <<<(unsigned)(ntx_active * n), LS::THREADS, 0, st>>>(reinterpret_cast<const float2*>(half), \
                    reinterpret_cast<float2*>(work), d2lo, d2hi, ntx_active,                             \
                    reinterpret_cast<const float2*>(tw));                                                \
            PYSPEC_LAUNCH_CHECK();                                                                       \
        } else {                                                                                         \
            shell_zpass_kernel<T, INDICATOR, NCV><<<(unsigned)(ntx * n), 256, sm_zy, st>>>(half, work, n, d2lo, \
                                                                                             d2hi, plan, tw); \
            PYSPEC_LAUNCH_CHECK();                                                                       \
            shell_ypass_kernel<T, NCV><<<(unsigned)(ntx_active * n), 256, sm_zy, st>>>(work, n, d2hi,     \
                                                                                       ntx_active, plan, tw); \
            PYSPEC_LAUNCH_CHECK();                                                                       \
        }                                                                                                \
        if constexpr (NCV > 0 && sizeof(T) == 4)                                                         \
            shell_xpass_reg_kernel<NCV, XR1(NCV), XR2(NCV)><<<nblk, 256,                                    \
                                                               xpass_reg_smem<NCV, XR1(NCV), XR2(NCV)>(), st>>>( \
                reinterpret_cast<const float2*>(work), xlim, reinterpret_cast<float*>(field), part,          \
                reinterpret_cast<const float2*>(tw));                                                    \
        else                                                                                             \
            shell_xpass_kernel<T, NCV><<<nblk, 256, sm_x, st>>>(work, n, xlim, rl, plan_half, field, part, tw); \
        PYSPEC_LAUNCH_CHECK();                                                                           \
    } while (0)
    bool done = false;
    if constexpr (sizeof(T) == 4) {
        done = true;
        switch (n) {
            case 192: PYSPEC_SHELL_LAUNCH(192); break;
            case 256: PYSPEC_SHELL_LAUNCH(256); break;
            case 360: PYSPEC_SHELL_LAUNCH(360); break;
            case 512: PYSPEC_SHELL_LAUNCH(512); break;
            default: done = false;
        }
    }
    if (!done) PYSPEC_SHELL_LAUNCH(0);
#undef PYSPEC_SHELL_LAUNCH
    count_launch(3);
    return PYSPEC_OK;
}

template <typename T>
int shell_twiddles(typename cplx_t<T>::type* tw, int n, cudaStream_t st) {
    twiddle_table_kernel<T><<<4, 256, 0, st>>>(tw, n);
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    return PYSPEC_OK;
}
template int shell_twiddles<double>(double2*, int, cudaStream_t);

template <typename T, bool INDICATOR>
int shell_fields_impl(const typename cplx_t<T>::type* half, int n, int step, int jmin, int nmax, T* fields,
                      double* p0sum, void* ws, size_t ws_bytes, cudaStream_t st) {
    using C = typename cplx_t<T>::type;
    const int nshell = nmax - jmin + 1;
    PYSPEC_CHECK_ARG(nshell >= 1, "nmax < jmin");
    const size_t need = shell_workspace_bytes<T>(n, nshell);
    if (ws_bytes < need || ws == nullptr) {
        set_error("shell workspace %zu bytes < required %zu", ws_bytes, need);
        return PYSPEC_E_WORKSPACE;
    }
    C* work = reinterpret_cast<C*>(ws);
    size_t off = ((size_t)work_stride<C>(n) * n * n * sizeof(C) + 255) & ~(size_t)255;
    double* part = reinterpret_cast<double*>(reinterpret_cast<char*>(ws) + off);
    const int nblk = xpass_ctas(n);
    const int64_t V = (int64_t)n * n * n;
    off += (size_t)nshell * nblk * sizeof(double);
    off = (off + 255) & ~(size_t)255;
    C* tw = reinterpret_cast<C*>(reinterpret_cast<char*>(ws) + off);
    PYSPEC_TRY(shell_twiddles<T>(tw, n, st));
    for (int s = 0; s < nshell; ++s) {
        PYSPEC_TRY((shell_one_impl<T, INDICATOR>(half, n, step, jmin + s, fields + (int64_t)s * V,
                                                  part + (int64_t)s * nblk, work, tw, st)));
    }
    if (p0sum) {
        reduce_rows_kernel<<<nshell, 256, 0, st>>>(part, nblk, p0sum);
        PYSPEC_LAUNCH_CHECK();
        count_launch();
    }
    return PYSPEC_OK;
}

template size_t shell_workspace_bytes<float>(int, int);
template size_t shell_workspace_bytes<double>(int, int);
template int shell_fields_impl<float, false>(const float2*, int, int, int, int, float*, double*, void*, size_t,
                                             cudaStream_t);
template int shell_fields_impl<double, true>(const double2*, int, int, int, int, double*, double*, void*,
                                             size_t, cudaStream_t);
template int shell_one_impl<double, true>(const double2*, int, int, int, double*, double*, double2*,
                                          const double2*, cudaStream_t);

// Nk[j] for j = 0..nmax over the full grid (pyspectrum.py:380)
__global__ void mode_counts_kernel(int n, int step, int nmax, unsigned long long* __restrict__ nk) {
    extern __shared__ unsigned long long cnt[];
    for (int i = threadIdx.x; i <= nmax; i += blockDim.x) cnt[i] = 0;
    __syncthreads();
    const int64_t nn = n;
    const int64_t tot = nn * nn * nn;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
        const int x = fold((int)(t % nn), n), y = fold((int)((t / nn) % nn), n), z = fold((int)(t / (nn * nn)), n);
        const int64_t d2 = (int64_t)x * x + (int64_t)y * y + (int64_t)z * z;
        const int j = shell_of(d2, step);
        if (j <= nmax) atomicAdd(&cnt[j], 1ull);
    }
    __syncthreads();
    for (int i = threadIdx.x; i <= nmax; i += blockDim.x)
        if (cnt[i]) atomicAdd(&nk[i], cnt[i]);
}

int mode_counts_impl(int n, int step, int nmax, int64_t* nk, cudaStream_t st) {
    PYSPEC_CUDA(cudaMemsetAsync(nk, 0, sizeof(int64_t) * (nmax + 1), st));
    mode_counts_kernel<<<608, 256, sizeof(unsigned long long) * (nmax + 1), st>>>(
        n, step, nmax, reinterpret_cast<unsigned long long*>(nk));
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    return PYSPEC_OK;
}

}  // namespace pyspec

using namespace pyspec;

extern "C" size_t pyspec_shell_fields_workspace(int ngrid, int nshell) {
    if (ngrid < 2 || nshell < 1) return 0;
    return shell_workspace_bytes<float>(ngrid, nshell);
}

extern "C" int pyspec_shell_fields(const float* half, int ngrid, int step, int jmin, int nmax, float* fields,
                                   double* p0sum, void* workspace, size_t ws_bytes, void* stream) {
    PYSPEC_CHECK_ARG(half && fields, "NULL pointer");
    PYSPEC_CHECK_ARG(ngrid >= 4 && ngrid % 2 == 0 && ngrid <= 2048, "ngrid=%d must be even and <= 2048", ngrid);
    PYSPEC_CHECK_ARG(step >= 1 && jmin >= 1 && nmax >= jmin, "need step>=1, 1<=jmin<=nmax");
    PYSPEC_CHECK_ARG(nmax - jmin + 1 <= kMaxShells, "at most %d shells", kMaxShells);
    return shell_fields_impl<float, false>(reinterpret_cast<const float2*>(half), ngrid, step, jmin, nmax, fields,
                                           p0sum, workspace, ws_bytes, as_stream(stream));
}

extern "C" int pyspec_mode_counts(int ngrid, int step, int nmax, int64_t* nk, void* stream) {
    PYSPEC_CHECK_ARG(nk != nullptr, "NULL pointer");
    PYSPEC_CHECK_ARG(ngrid >= 2 && step >= 1 && nmax >= 0 && nmax < 4096, "bad arguments");
    return mode_counts_impl(ngrid, step, nmax, nk, as_stream(stream));
}
