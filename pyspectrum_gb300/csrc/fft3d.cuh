#pragma once
#include "common.cuh"

namespace pyspec {

// x columns per tile in the strided FFT passes: 8 complex values (a 64-byte
// row for complex64, 128 bytes for complex128), which keeps a tile of 360
// lines at 46 KB (float) so four CTAs fit on an SM.
template <typename T>
__host__ __device__ constexpr int tile_x() { return 8; }

// contiguous lines per CTA in the x pass
__host__ __device__ constexpr int contig_lines(int n) { return (4096 / n) < 1 ? 1 : ((4096 / n) > 16 ? 16 : 4096 / n); }

// variant: 0 .. fft3d_nreg(n) (see fft3d.cu)
template <typename T>
int fft3d_c2c_impl(typename cplx_t<T>::type* data, int n, int sign, cudaStream_t st, int variant = 0);
int fft3d_nreg(int n);
int fft3d_default_variant(int n);

}  // namespace pyspec
