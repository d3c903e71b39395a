// Error reporting, launch accounting and FFT radix planning.
#include <atomic>
#include <map>
#include <mutex>
#include <utility>
#include <stdarg.h>
#include <string.h>
#include "common.cuh"

namespace pyspec {

static thread_local char g_err[512] = {0};
std::atomic<int64_t> g_launches{0};

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

bool make_plan(int n, RadixPlan* p) {
    p->n = n;
    p->nstages = 0;
    int m = n;
    const int order[5] = {8, 4, 5, 3, 2};
    for (int k = 0; k < 5; ++k) {
        while (m % order[k] == 0) {
            if (p->nstages >= 16) return false;
            p->radix[p->nstages++] = order[k];
            m /= order[k];
        }
    }
    if (m != 1 || n < 2) return false;
    int ns = 1;
    for (int s = 0; s < p->nstages; ++s) {
        p->ns[s] = make_fastdiv((uint32_t)ns);
        p->nb[s] = make_fastdiv((uint32_t)(n / p->radix[s]));
        ns *= p->radix[s];
    }
    return true;
}

}  // namespace pyspec

extern "C" int pyspec_abi_version(void) { return PYSPEC_ABI_VERSION; }

extern "C" int pyspec_last_error(char* buf, size_t len) {
    if (!buf || len == 0) return PYSPEC_E_INVALID;
    strncpy(buf, pyspec::g_err, len - 1);
    buf[len - 1] = 0;
    return PYSPEC_OK;
}

extern "C" int64_t pyspec_launch_count(void) { return pyspec::g_launches.load(); }

namespace pyspec {
// The opt-in limit covers static + dynamic shared memory: a launch whose
// dynamic bytes alone stay under the 48 KB default can still exceed it, so
// the attribute is raised for any size above what this function (on this
// device) was last given.
int allow_smem(const void* func, size_t bytes) {
    if (bytes > 227 * 1024) {
        set_error("kernel needs %zu bytes of shared memory (limit 227 KB)", bytes);
        return PYSPEC_E_UNSUPPORTED;
    }
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> raised;
    int dev = 0;
    PYSPEC_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    size_t& cur = raised[{func, dev}];
    if (bytes <= cur) return PYSPEC_OK;
    PYSPEC_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = bytes;
    return PYSPEC_OK;
}

void* pinned_copy(const void* src, size_t bytes) {
    void* p = nullptr;
    if (bytes == 0 || cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();   // clear a failed allocation's sticky-free error state
        return nullptr;
    }
    memcpy(p, src, bytes);
    return p;
}
}  // namespace pyspec
