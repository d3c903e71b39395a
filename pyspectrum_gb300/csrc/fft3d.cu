// 3D complex FFT of an N^3 grid ([z][y][x], x fastest), in place, as three
// passes of batched 1D transforms.  Each CTA copies a tile of whole lines into
// shared memory, transforms it there (fft_device.cuh) and writes it back to
// the same addresses, so the transform needs no scratch memory.
//
// Replaces the FFTW call of pyspectrum.py:1073-1075 (FFTW_BACKWARD,
// unnormalised) used by FFT_periodic on the interlaced density grid.
#include "fft_device.cuh"
#include "fft3d.cuh"

namespace pyspec {

// Pass over contiguous lines (the x axis): lines [line0, line0+nl) of length n
// occupy one contiguous run of memory.
template <typename T, int NC>
__global__ void __launch_bounds__(256) fft_contig_kernel(typename cplx_t<T>::type* data, int64_t nlines_total,
                                                         int lx_rt, RadixPlan plan, int sign) {
    using C = typename cplx_t<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = NC > 0 ? NC : plan.n;
    const int lx = NC > 0 ? contig_lines(NC) : lx_rt;
    C* tw = reinterpret_cast<C*>(smem_raw);
    C* buf0 = tw + n;
    C* buf1 = buf0 + (size_t)lx * n;
    const int64_t line0 = (int64_t)blockIdx.x * lx;
    const int nl = (int)min((int64_t)lx, nlines_total - line0);
    fill_twiddles<T>(tw, n, sign, threadIdx.x, blockDim.x);
    C* g = data + line0 * n;
    const int cnt = nl * n;
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) buf0[i] = g[i];
    __syncthreads();
    C* res;
    if constexpr (NC > 0) res = ct::fft_tile_ct<T, NC, 0, contig_lines(NC)>(buf0, buf1, tw, sign);
    else res = fft_tile<T, 0>(buf0, buf1, tw, plan, nl, sign);
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) g[i] = res[i];
}

// Pass over strided lines: a tile is `tx` consecutive x columns x all n
// positions along the transformed axis (row stride `row_stride` elements).
// Tile b covers outer index b / ntx and x block b % ntx.
template <typename T, int NC>
__global__ void __launch_bounds__(256) fft_strided_kernel(typename cplx_t<T>::type* data, int nx, int64_t row_stride,
                                                          int64_t outer_stride, RadixPlan plan, int sign) {
    using C = typename cplx_t<T>::type;
    constexpr int tx = tile_x<T>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = NC > 0 ? NC : plan.n;
    C* tw = reinterpret_cast<C*>(smem_raw);
    C* buf0 = tw + n;
    C* buf1 = buf0 + (size_t)tx * n;
    const int ntx = (nx + tx - 1) / tx;
    const int outer = blockIdx.x / ntx;
    const int x0 = (blockIdx.x % ntx) * tx;
    const int ncol = min(tx, nx - x0);
    fill_twiddles<T>(tw, n, sign, threadIdx.x, blockDim.x);
    C* g = data + (int64_t)outer * outer_stride + x0;
    const int cnt = n * tx;
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        const int r = i / tx, c = i - r * tx;
        if (c < ncol) buf0[i] = g[r * row_stride + c];
    }
    __syncthreads();
    C* res;
    if constexpr (NC > 0) res = ct::fft_tile_ct<T, NC, tx, 0>(buf0, buf1, tw, sign);
    else res = fft_tile<T, tx>(buf0, buf1, tw, plan, tx, sign);
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        const int r = i / tx, c = i - r * tx;
        if (c < ncol) g[r * row_stride + c] = res[i];
    }
}

// Register form of a pass for the common lengths N = R1 * R2: a CTA
// transforms 8 lines in two radix stages with one padded shared-memory
// exchange (as the shell line passes).  CONTIG: 8 consecutive contiguous lines
// (the x axis; lanes run along the line, so loads are coalesced); otherwise 8
// consecutive x columns of lines with element stride `row_stride` (the y and
// z axes; lanes run across the columns).  In place.
template <int NC, int R1, int R2>
struct FftLineShape {
    static constexpr int NB1 = NC / R1, NB2 = NC / R2;
    static constexpr int NBM = NB1 > NB2 ? NB1 : NB2;
    static constexpr int THREADS = 8 * NBM;
    static constexpr int COLP = ((NC + NB1 + 13) / 16) * 16 + 2;   // padded line, == 2 (mod 16)
};

template <int NC, int R1, int R2, bool CONTIG>
__global__ void __launch_bounds__(FftLineShape<NC, R1, R2>::THREADS)
fft_line_kernel(float2* __restrict__ data, int64_t row_stride, int64_t outer_stride, int ntx, int sign) {
    using S = FftLineShape<NC, R1, R2>;
    constexpr int N = NC;
    static_assert(R1 * R2 == N, "two radix stages");
    __shared__ float2 tw[N];
    __shared__ float2 buf[8 * S::COLP];
    fill_twiddles<float>(tw, N, sign, threadIdx.x, blockDim.x);
    int c, b;
    float2* g;
    int64_t es;                                  // element stride along the line
    if constexpr (CONTIG) {
        c = threadIdx.x / S::NBM;
        b = threadIdx.x - c * S::NBM;
        g = data + ((int64_t)blockIdx.x * 8 + c) * N;
        es = 1;
    } else {
        c = threadIdx.x & 7;
        b = threadIdx.x >> 3;
        const int outer = blockIdx.x / ntx;
        const int x0 = (blockIdx.x - outer * ntx) * 8;
        g = data + (int64_t)outer * outer_stride + x0 + c;
        es = row_stride;
    }
    __syncthreads();
    float2* col = buf + c * S::COLP;
    if (b < S::NB1) {
        float2 v[R1];
#pragma unroll
        for (int r = 0; r < R1; ++r) v[r] = g[(int64_t)(b + r * S::NB1) * es];
        small_dft<float, float2, R1>(v, sign);
#pragma unroll
        for (int r = 0; r < R1; ++r) col[b * (R1 + 1) + r] = v[r];    // element b*R1 + r
    }
    __syncthreads();
    if (b < S::NB2) {
        float2 v[R2];
#pragma unroll
        for (int r = 0; r < R2; ++r) {
            const int p = b + r * S::NB2;                               // element index (< N)
            const float2 u = col[p + p / R1];
            v[r] = r == 0 || b == 0 ? u : cmul(u, tw[r * b]);
        }
        small_dft<float, float2, R2>(v, sign);
#pragma unroll
        for (int r = 0; r < R2; ++r) g[(int64_t)(b + r * S::NB2) * es] = v[r];
    }
}

// Radix splits N = R1 * R2 of the register passes, per grid size: variant
// v < nreg(N) uses split v; variant nreg(N) is the shared-memory Stockham
// form (every N with factors 2, 3, 5).  The autotuner of the Python layer
// times them all and picks per N.  Every N listed is a multiple of 8 (the
// strided passes take 8 whole columns per CTA) and every radix has a
// small_dft form.
struct RegSplit { int n, r1, r2; };
constexpr RegSplit kSplits[] = {
    {128, 16, 8}, {128, 8, 16},
    {192, 16, 12}, {192, 12, 16}, {192, 24, 8}, {192, 8, 24},
    {256, 16, 16},
    {360, 20, 18}, {360, 18, 20}, {360, 24, 15}, {360, 15, 24},
};
constexpr int kNSplits = (int)(sizeof(kSplits) / sizeof(kSplits[0]));

// the variant pyspec_fft3d_c2c uses: the first register split of 192, 256
// and 360, the Stockham form for every other size
int fft3d_default_variant(int n) { return (n == 192 || n == 256 || n == 360) ? 0 : fft3d_nreg(n); }

int fft3d_nreg(int n) {
    int c = 0;
    for (int k = 0; k < kNSplits; ++k) c += kSplits[k].n == n;
    return c;
}

// the (r1, r2) of register variant v of size n, or false
static bool reg_split(int n, int v, int* r1, int* r2) {
    for (int k = 0; k < kNSplits; ++k)
        if (kSplits[k].n == n && v-- == 0) {
            *r1 = kSplits[k].r1;
            *r2 = kSplits[k].r2;
            return true;
        }
    return false;
}

template <int NC, int R1, int R2>
static int fft3d_reg(float2* d, int n, int sign, cudaStream_t st) {
    using FS = FftLineShape<NC, R1, R2>;
    const int64_t lines = (int64_t)n * n;
    const int ntx = (n + 7) / 8;
    fft_line_kernel<NC, R1, R2, true><<<(unsigned)(lines / 8), FS::THREADS, 0, st>>>(d, 1, 0, 0, sign);
    PYSPEC_LAUNCH_CHECK();
    fft_line_kernel<NC, R1, R2, false><<<(unsigned)(ntx * n), FS::THREADS, 0, st>>>(d, n, (int64_t)n * n, ntx,
                                                                                    sign);
    PYSPEC_LAUNCH_CHECK();
    fft_line_kernel<NC, R1, R2, false><<<(unsigned)(ntx * n), FS::THREADS, 0, st>>>(d, (int64_t)n * n, n, ntx,
                                                                                    sign);
    PYSPEC_LAUNCH_CHECK();
    return PYSPEC_OK;
}

template <typename T>
int fft3d_c2c_impl(typename cplx_t<T>::type* data, int n, int sign, cudaStream_t st, int variant) {
    using C = typename cplx_t<T>::type;
    RadixPlan plan;
    PYSPEC_CHECK_ARG(make_plan(n, &plan), "ngrid=%d must factor into 2, 3 and 5", n);
    PYSPEC_CHECK_ARG(sign == 1 || sign == -1, "sign must be +1 or -1");
    const int nreg = sizeof(T) == 4 ? fft3d_nreg(n) : 0;
    PYSPEC_CHECK_ARG(variant >= 0 && variant <= nreg, "variant %d out of range [0, %d] for ngrid=%d", variant, nreg,
                     n);
    const int lx = contig_lines(n);
    const size_t sm_c = sizeof(C) * ((size_t)n + 2 * (size_t)lx * n);
    const int64_t lines = (int64_t)n * n;
    const unsigned nbc = (unsigned)((lines + lx - 1) / lx);
    const int tx = tile_x<T>();
    const int ntx = (n + tx - 1) / tx;
    const size_t sm = sizeof(C) * ((size_t)n + 2 * (size_t)tx * n);
#define PYSPEC_FFT3D_LAUNCH(NCV)                                                                          \
    do {                                                                                                 \
        PYSPEC_TRY(allow_smem((const void*)fft_contig_kernel<T, NCV>, sm_c));                            \
        PYSPEC_TRY(allow_smem((const void*)fft_strided_kernel<T, NCV>, sm));                             \
        fft_contig_kernel<T, NCV><<<nbc, 256, sm_c, st>>>(data, lines, lx, plan, sign);                  \
        PYSPEC_LAUNCH_CHECK();                                                                           \
        fft_strided_kernel<T, NCV><<<(unsigned)(ntx * n), 256, sm, st>>>(data, n, n, (int64_t)n * n, plan, sign); \
        PYSPEC_LAUNCH_CHECK();                                                                           \
        fft_strided_kernel<T, NCV><<<(unsigned)(ntx * n), 256, sm, st>>>(data, n, (int64_t)n * n, n, plan, sign); \
        PYSPEC_LAUNCH_CHECK();                                                                           \
    } while (0)
    int r1 = 0, r2 = 0;
    if constexpr (sizeof(T) == 4) {
        if (variant < nreg && reg_split(n, variant, &r1, &r2)) {
            float2* d = reinterpret_cast<float2*>(data);
            int rc = PYSPEC_E_UNSUPPORTED;
#define PYSPEC_FFT3D_REG(NV, A, B) \
    if (n == NV && r1 == A && r2 == B) rc = fft3d_reg<NV, A, B>(d, n, sign, st);
            PYSPEC_FFT3D_REG(128, 16, 8) PYSPEC_FFT3D_REG(128, 8, 16)
            PYSPEC_FFT3D_REG(192, 16, 12) PYSPEC_FFT3D_REG(192, 12, 16) PYSPEC_FFT3D_REG(192, 24, 8)
            PYSPEC_FFT3D_REG(192, 8, 24)
            PYSPEC_FFT3D_REG(256, 16, 16)
            PYSPEC_FFT3D_REG(360, 20, 18) PYSPEC_FFT3D_REG(360, 18, 20) PYSPEC_FFT3D_REG(360, 24, 15)
            PYSPEC_FFT3D_REG(360, 15, 24)
#undef PYSPEC_FFT3D_REG
            PYSPEC_TRY(rc);
            count_launch(3);
            return PYSPEC_OK;
        }
    }
    if (n == 512) PYSPEC_FFT3D_LAUNCH(512);
    else PYSPEC_FFT3D_LAUNCH(0);
#undef PYSPEC_FFT3D_LAUNCH
    count_launch(3);
    return PYSPEC_OK;
}

template int fft3d_c2c_impl<float>(float2*, int, int, cudaStream_t, int);
template int fft3d_c2c_impl<double>(double2*, int, int, cudaStream_t, int);

}  // namespace pyspec

extern "C" int pyspec_fft3d_c2c(float* grid, int ngrid, int sign, void* stream) {
    PYSPEC_CHECK_ARG(grid != nullptr, "grid is NULL");
    PYSPEC_CHECK_ARG(ngrid >= 2 && ngrid <= 2048, "ngrid=%d out of range", ngrid);
    return pyspec::fft3d_c2c_impl<float>(reinterpret_cast<float2*>(grid), ngrid, sign, pyspec::as_stream(stream),
                                         pyspec::fft3d_default_variant(ngrid));
}

extern "C" int pyspec_fft3d_variants(int ngrid, int32_t* r1r2, int cap) {
    const int nreg = pyspec::fft3d_nreg(ngrid);
    for (int v = 0; v <= nreg && v < cap; ++v) {
        int a = 0, b = 0;
        if (v < nreg) pyspec::reg_split(ngrid, v, &a, &b);
        if (r1r2 != nullptr) {
            r1r2[2 * v] = a;
            r1r2[2 * v + 1] = b;
        }
    }
    return nreg + 1;
}

extern "C" int pyspec_fft3d_c2c_variant(float* grid, int ngrid, int sign, int variant, void* stream) {
    PYSPEC_CHECK_ARG(grid != nullptr, "grid is NULL");
    PYSPEC_CHECK_ARG(ngrid >= 2 && ngrid <= 2048, "ngrid=%d out of range", ngrid);
    return pyspec::fft3d_c2c_impl<float>(reinterpret_cast<float2*>(grid), ngrid, sign, pyspec::as_stream(stream),
                                         variant);
}
