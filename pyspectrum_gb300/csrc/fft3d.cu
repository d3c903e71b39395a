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
template <typename T>
__global__ void __launch_bounds__(256) fft_contig_kernel(typename cplx_t<T>::type* data, int64_t nlines_total,
                                                         int lx, RadixPlan plan, int sign) {
    using C = typename cplx_t<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = plan.n;
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
    C* res = fft_tile<T, 0>(buf0, buf1, tw, plan, nl, sign);
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) g[i] = res[i];
}

// Pass over strided lines: a tile is `tx` consecutive x columns x all n
// positions along the transformed axis (row stride `row_stride` elements).
// Tile b covers outer index b / ntx and x block b % ntx.
template <typename T>
__global__ void __launch_bounds__(256) fft_strided_kernel(typename cplx_t<T>::type* data, int nx, int64_t row_stride,
                                                          int64_t outer_stride, RadixPlan plan, int sign) {
    using C = typename cplx_t<T>::type;
    constexpr int tx = tile_x<T>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = plan.n;
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
    C* res = fft_tile<T, tx>(buf0, buf1, tw, plan, tx, sign);
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        const int r = i / tx, c = i - r * tx;
        if (c < ncol) g[r * row_stride + c] = res[i];
    }
}

template <typename T>
int fft3d_c2c_impl(typename cplx_t<T>::type* data, int n, int sign, cudaStream_t st) {
    using C = typename cplx_t<T>::type;
    RadixPlan plan;
    PYSPEC_CHECK_ARG(make_plan(n, &plan), "ngrid=%d must factor into 2, 3 and 5", n);
    PYSPEC_CHECK_ARG(sign == 1 || sign == -1, "sign must be +1 or -1");
    // x lines
    {
        int lx = max(1, min(16, 4096 / n));
        size_t sm = sizeof(C) * ((size_t)n + 2 * (size_t)lx * n);
        PYSPEC_TRY(allow_smem((const void*)fft_contig_kernel<T>, sm));
        int64_t lines = (int64_t)n * n;
        unsigned nb = (unsigned)((lines + lx - 1) / lx);
        fft_contig_kernel<T><<<nb, 256, sm, st>>>(data, lines, lx, plan, sign);
        PYSPEC_LAUNCH_CHECK();
        count_launch();
    }
    // y and z lines
    const int tx = tile_x<T>();
    const int ntx = (n + tx - 1) / tx;
    size_t sm = sizeof(C) * ((size_t)n + 2 * (size_t)tx * n);
    PYSPEC_TRY(allow_smem((const void*)fft_strided_kernel<T>, sm));
    fft_strided_kernel<T><<<(unsigned)(ntx * n), 256, sm, st>>>(data, n, n, (int64_t)n * n, plan, sign);
    PYSPEC_LAUNCH_CHECK();
    fft_strided_kernel<T><<<(unsigned)(ntx * n), 256, sm, st>>>(data, n, (int64_t)n * n, n, plan, sign);
    PYSPEC_LAUNCH_CHECK();
    count_launch(2);
    return PYSPEC_OK;
}

template int fft3d_c2c_impl<float>(float2*, int, int, cudaStream_t);
template int fft3d_c2c_impl<double>(double2*, int, int, cudaStream_t);

}  // namespace pyspec

extern "C" int pyspec_fft3d_c2c(float* grid, int ngrid, int sign, void* stream) {
    PYSPEC_CHECK_ARG(grid != nullptr, "grid is NULL");
    PYSPEC_CHECK_ARG(ngrid >= 2 && ngrid <= 2048, "ngrid=%d out of range", ngrid);
    return pyspec::fft3d_c2c_impl<float>(reinterpret_cast<float2*>(grid), ngrid, sign, pyspec::as_stream(stream));
}
