#pragma once
#include "common.cuh"

namespace pyspec {

// Shell number of a mode with |k|^2 = d2 (units of k_f): the largest n with
// (2n-1)^2 step^2 <= 4 d2, i.e. int(sqrt(d2)/step + 0.5) evaluated exactly.
__host__ __device__ inline int shell_of(int64_t d2, int step) {
    int n = (int)(sqrtf((float)d2) / (float)step + 0.5f);
    const int64_t s2 = (int64_t)step * step;
    while (n > 0 && (int64_t)(2 * n - 1) * (2 * n - 1) * s2 > 4 * d2) --n;
    while ((int64_t)(2 * n + 1) * (2 * n + 1) * s2 <= 4 * d2) ++n;
    return n;
}

template <typename T>
size_t shell_workspace_bytes(int n, int nshell);

template <typename T, bool INDICATOR>
int shell_fields_impl(const typename cplx_t<T>::type* half, int n, int step, int jmin, int nmax, T* fields,
                      double* p0sum, void* ws, size_t ws_bytes, cudaStream_t st);

template <typename T, bool INDICATOR>
int shell_one_impl(const typename cplx_t<T>::type* half, int n, int step, int j, T* field, double* part,
                   typename cplx_t<T>::type* work, const typename cplx_t<T>::type* tw, cudaStream_t st);

// fills the forward twiddle tables used by shell_one_impl: n + n/2 values
template <typename T>
int shell_twiddles(typename cplx_t<T>::type* tw, int n, cudaStream_t st);

int mode_counts_impl(int n, int step, int nmax, int64_t* nk, cudaStream_t st);

}  // namespace pyspec
