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
// device looks the array's device address up with that device current; make
// that first call before any stream capture.
#include <mutex>
#include "common.cuh"
#include "contract.cuh"

namespace pyspec {

static __device__ __align__(256) unsigned char g_noalloc_scratch[PYSPEC_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[256] = {nullptr};

// Device address of the array on the current device (looked up once per device).
static int noalloc_scratch(void** out) {
    int dev = 0;
    PYSPEC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) {
        set_error("device ordinal %d out of range", dev);
        return PYSPEC_E_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (g_noalloc_addr[dev] == nullptr) {
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
    const size_t need = contract_fp32_ws(V, nshell, ntri);
    if (need > (size_t)PYSPEC_NOALLOC_SCRATCH_BYTES) {
        set_error("this contraction needs %zu bytes of scratch; the fixed scratch array holds %zu "
                  "(use pyspec_bk_contract with a workspace)", need, (size_t)PYSPEC_NOALLOC_SCRATCH_BYTES);
        return PYSPEC_E_INVALID;
    }
    void* scratch = nullptr;
    PYSPEC_TRY(noalloc_scratch(&scratch));
    return contract_fp32_impl(fields, V, nshell, tri_host, ntri, bsum, scratch, PYSPEC_NOALLOC_SCRATCH_BYTES,
                              as_stream(stream));
}
