#pragma once
#include "common.cuh"

namespace pyspec {

size_t contract_simple_ws(int64_t nvox, int ntri);

template <typename T>
int contract_simple_impl(const T* fields, int64_t fstride, int nshell, const int32_t* tri, int ntri, const T* wts,
                         int64_t nvox, double* bsum, double* partials, cudaStream_t st);

// register-tiled FP32 CUDA-core contraction
size_t contract_fp32_ws(int64_t nvox, int nshell, int ntri);
int contract_fp32_impl(const float* fields, int64_t nvox, int nshell, const int32_t* tri_host, int ntri,
                       double* bsum, void* ws, size_t ws_bytes, cudaStream_t st);
// Exact scratch bytes contract_fp32_impl uses for this list.  may_plan=false
// only consults the plan cache (no host allocation) and fails if the list has
// no cached plan or its tables are not page-locked.
int contract_fp32_need(int64_t nvox, int nshell, const int32_t* tri_host, int ntri, bool may_plan, size_t* need);

// tcgen05 split-BF16 contraction (contract_tc.cu)
size_t contract_tc_ws(int64_t nvox, int nshell, int ntri, bool six = false);
int contract_tc_impl(const float* fields, int64_t nvox, int nshell, const int32_t* tri, const int32_t* tri_host,
                     int ntri, double* bsum, void* ws, size_t ws_bytes, cudaStream_t st, bool run_plan = false,
                     bool fine_drain = false, bool six = false, bool kc32 = false);

// bsum[t] = sum over nblk rows of partials[b][t] (float64, fixed order)
int reduce_partials_launch(const double* partials, int nblk, int ntri, double* bsum, cudaStream_t st);

}  // namespace pyspec
