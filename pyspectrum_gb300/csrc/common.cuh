// Shared helpers for the pyspectrum_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <stdio.h>
#include "../../include/pyspec_gpu.h"

namespace pyspec {

// Records the message returned by pyspec_last_error() for this host thread.
void set_error(const char* fmt, ...);
// Adds n to the process-wide count of this library's kernel launches.
void count_launch(int n = 1);
// Raises the dynamic shared-memory limit of a kernel once per process.
int allow_smem(const void* func, size_t bytes);
// Page-locked copy of a host byte range that lives as long as the process
// (plans that own one are cached for the process lifetime), so the per-call
// table upload is one asynchronous DMA copy.  Returns NULL if the host
// allocation fails; callers then copy from their pageable buffer.
void* pinned_copy(const void* src, size_t bytes);

#define PYSPEC_CHECK_ARG(cond, ...)                          \
    do {                                                     \
        if (!(cond)) {                                       \
            ::pyspec::set_error(__VA_ARGS__);                \
            return PYSPEC_E_INVALID;                         \
        }                                                    \
    } while (0)

#define PYSPEC_CUDA(call)                                                        \
    do {                                                                         \
        cudaError_t e_ = (call);                                                 \
        if (e_ != cudaSuccess) {                                                 \
            ::pyspec::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call,      \
                                cudaGetErrorString(e_));                         \
            return PYSPEC_E_CUDA;                                                \
        }                                                                        \
    } while (0)

#define PYSPEC_LAUNCH_CHECK() PYSPEC_CUDA(cudaGetLastError())

#define PYSPEC_TRY(call)              \
    do {                              \
        int s_ = (call);              \
        if (s_ != PYSPEC_OK) return s_; \
    } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Exact unsigned division by a runtime constant d (Granlund-Montgomery):
// q = (umulhi(m, x) + x) >> l for all x < 2^31.
struct FastDiv {
    uint32_t m;
    int l;
    uint32_t d;
};
inline FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    f.d = d;
    int l = 0;
    while ((1ull << l) < d) ++l;
    f.l = l;
    f.m = (uint32_t)((((1ull << l) - d) << 32) / d + 1);
    return f;
}
__device__ __forceinline__ uint32_t fdiv(uint32_t x, const FastDiv& f) {
    return (__umulhi(f.m, x) + x) >> f.l;
}

// Radix plan for the mixed-radix FFTs: N = prod(radix[i]); radices in {2,3,4,5,8}.
// ns[s] = product of the radices before stage s; nb[s] = n / radix[s].
struct RadixPlan {
    int n;
    int nstages;
    int radix[16];
    FastDiv ns[16];
    FastDiv nb[16];
};
// Returns false if n has a prime factor > 5.
bool make_plan(int n, RadixPlan* p);

template <typename T> struct cplx_t;
template <> struct cplx_t<float> { using type = float2; };
template <> struct cplx_t<double> { using type = double2; };

template <typename T>
__host__ __device__ __forceinline__ typename cplx_t<T>::type mk(T x, T y) {
    typename cplx_t<T>::type r; r.x = x; r.y = y; return r;
}

// The number of shells is bounded so per-shell tables fit in shared memory.
constexpr int kMaxShells = 128;

}  // namespace pyspec
