// Triangle contraction that allocates no device memory.
//
// Some callers cannot allocate device memory at the moment they run the
// contraction: code inside another framework's foreign-function or
// custom-call hook, which receives only its operands and must not call
// cudaMalloc, and code that runs while a stream is being captured, where an
// allocation would break the capture.  This entry point serves them: it runs
// the register-tiled FP32 CUDA-core contraction with its scratch (the tile
// tables and one float64 partial sum per CTA and triangle) in a fixed
// file-scope device array instead of a caller workspace.
//
// The array is PYSPEC_NOALLOC_SCRATCH_BYTES (16 MiB) on every GPU that loads
// this library, for the life of the process.  Each call clears the partial
// sums it uses before the kernel runs.  All calls share the one array, so two
// calls whose work overlaps on the GPU (different streams, or different host
// threads without ordering) race; callers order them.  The first call on a
// device looks the array's device address up with that device current, and
// the first call with a given triangle list builds that list's tile plan in
// page-locked host memory; both are forbidden inside a stream capture, so a
// call made while its stream is capturing fails with PYSPEC_E_INVALID unless
// an earlier call on that device with that list, outside any capture, has
// done them.
#include <mutex>
#include "common.cuh"
#include "contract.cuh"

namespace pyspec {

static __device__ __align__(256) unsigned char g_noalloc_scratch[PYSPEC_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[256] = {nullptr};

// Device address of the array on the current device (looked up once per
// device; while capturing, only an address looked up before is returned).
static int noalloc_scratch(void** out, bool capturing) {
    int dev = 0;
    PYSPEC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) {
        set_error("device ordinal %d out of range", dev);
        return PYSPEC_E_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (g_noalloc_addr[dev] == nullptr) {
        if (capturing) {
            set_error("the first no-alloc call on device %d runs inside a stream capture; make one call on this "
                      "device outside the capture first", dev);
            return PYSPEC_E_INVALID;
        }
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            set_error("cudaGetSymbolAddress of the scratch array failed: %s", cudaGetErrorString(e));
            return PYSPEC_E_CUDA;
        }
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return PYSPEC_OK;
}

}  // namespace pyspec

using namespace pyspec;

extern "C" int pyspec_bk_contract_noalloc(const float* fields, int ngrid, int nshell, const int32_t* tri_host,
                                          int ntri, double* bsum, void* stream) {
    PYSPEC_CHECK_ARG(fields && tri_host && bsum, "NULL pointer");
    PYSPEC_CHECK_ARG(ngrid >= 2 && ngrid % 2 == 0 && nshell >= 1 && nshell <= kMaxShells && ntri >= 0,
                     "bad arguments");
    if (ntri == 0) return PYSPEC_OK;
    const int64_t V = (int64_t)ngrid * ngrid * ngrid;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    PYSPEC_CUDA(cudaStreamIsCapturing(as_stream(stream), &cap));
    const bool capturing = cap != cudaStreamCaptureStatusNone;
    // an upper bound of the scratch from the sizes alone (partial sums of
    // every CTA and the largest tile tables a list of ntri triangles can
    // need): requests beyond the array are refused before any planning
    const size_t bound = contract_fp32_ws(V, nshell, ntri);
    if (bound > (size_t)PYSPEC_NOALLOC_SCRATCH_BYTES) {
        set_error("this contraction may need up to %zu bytes of scratch; the fixed scratch array holds %zu "
                  "(use pyspec_bk_contract with a workspace)", bound, (size_t)PYSPEC_NOALLOC_SCRATCH_BYTES);
        return PYSPEC_E_INVALID;
    }
    // the list's tile plan: built here, or, while the stream is capturing,
    // only taken from the cache (its exact scratch never exceeds the bound)
    size_t need = 0;
    PYSPEC_TRY(contract_fp32_need(V, nshell, tri_host, ntri, !capturing, &need));
    if (need > bound) {
        set_error("internal: planned scratch %zu bytes exceeds its bound %zu", need, bound);
        return PYSPEC_E_INVALID;
    }
    void* scratch = nullptr;
    PYSPEC_TRY(noalloc_scratch(&scratch, capturing));
    return contract_fp32_impl(fields, V, nshell, tri_host, ntri, bsum, scratch, PYSPEC_NOALLOC_SCRATCH_BYTES,
                              as_stream(stream));
}
