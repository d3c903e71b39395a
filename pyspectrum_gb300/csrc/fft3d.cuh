#pragma once
#include "common.cuh"

namespace pyspec {

// x columns per tile in the strided FFT passes: one 128-byte row of
// complex64 (16 values) or complex128 (8 values).
template <typename T>
constexpr int tile_x() { return sizeof(T) == 4 ? 16 : 8; }

template <typename T>
int fft3d_c2c_impl(typename cplx_t<T>::type* data, int n, int sign, cudaStream_t st);

}  // namespace pyspec
