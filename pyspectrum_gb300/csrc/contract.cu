// Triangle contraction on CUDA cores (the plain-FP32 form), the float64
// triangle counts, and the bispectrum normalisation.
//
// bsum[t] = sum_v F_i(v) F_j(v) F_l(v)      (pyspectrum.py:427-430)
//
// A CTA stages a chunk of voxels of every shell in shared memory (voxel-major,
// padded to avoid bank conflicts); each thread owns up to TPT triangles and
// accumulates their products over the chunk.  Per-chunk float32 partials are
// folded into a Kahan-compensated float32 running sum; each CTA writes one
// float64 partial per triangle and a second kernel adds the CTA partials in a
// fixed order (float64, deterministic).
#include <string.h>
#include <algorithm>
#include <map>
#include <mutex>
#include <vector>
#include "common.cuh"
#include "contract.cuh"
#include "shells.cuh"

namespace pyspec {

constexpr int kTpt = 16;       // triangles per thread
constexpr int kCthreads = 256;
constexpr int kVc = 64;        // voxels per staged chunk

template <typename T>
__global__ void __launch_bounds__(kCthreads) contract_simple_kernel(const T* __restrict__ fields, int64_t fstride,
                                                                    int nshell, const int32_t* __restrict__ tri,
                                                                    int ntri, const T* __restrict__ wts,
                                                                    int64_t nvox, double* __restrict__ partials) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* tile = reinterpret_cast<T*>(smem_raw);
    const int stride = nshell + 1;
    T* wt = tile + kVc * stride;
    const int t0 = blockIdx.y * kTpt * blockDim.x;
    int ii[kTpt], jj[kTpt], ll[kTpt];
    bool ok[kTpt];
#pragma unroll
    for (int k = 0; k < kTpt; ++k) {
        const int t = t0 + threadIdx.x + k * blockDim.x;
        ii[k] = t < ntri ? tri[t] : 0;
        jj[k] = t < ntri ? tri[ntri + t] : 0;
        ll[k] = t < ntri ? tri[2 * ntri + t] : 0;
        // slots outside [0, nshell) are skipped (their partial stays unwritten)
        ok[k] = t < ntri && ii[k] >= 0 && ii[k] < nshell && jj[k] >= 0 && jj[k] < nshell && ll[k] >= 0 &&
                ll[k] < nshell;
        if (!ok[k]) ii[k] = jj[k] = ll[k] = 0;
    }
    T hi[kTpt], lo[kTpt];
#pragma unroll
    for (int k = 0; k < kTpt; ++k) { hi[k] = 0; lo[k] = 0; }
    for (int64_t v0 = (int64_t)blockIdx.x * kVc; v0 < nvox; v0 += (int64_t)gridDim.x * kVc) {
        const int nv = (int)min((int64_t)kVc, nvox - v0);
        __syncthreads();
        for (int i = threadIdx.x; i < nshell * kVc; i += blockDim.x) {
            const int s = i / kVc, c = i - s * kVc;
            tile[c * stride + s] = c < nv ? fields[s * fstride + v0 + c] : T(0);
        }
        if (wts != nullptr)
            for (int c = threadIdx.x; c < kVc; c += blockDim.x) wt[c] = c < nv ? wts[v0 + c] : T(0);
        __syncthreads();
        T loc[kTpt];
#pragma unroll
        for (int k = 0; k < kTpt; ++k) loc[k] = 0;
        for (int c = 0; c < nv; ++c) {
            const T* row = tile + c * stride;
            const T w = wts != nullptr ? wt[c] : T(1);
#pragma unroll
            for (int k = 0; k < kTpt; ++k) loc[k] += (row[ii[k]] * row[jj[k]]) * (row[ll[k]] * w);
        }
#pragma unroll
        for (int k = 0; k < kTpt; ++k) {   // Kahan: hi + lo tracks the running sum
            const T y = loc[k] - lo[k];
            const T s = hi[k] + y;
            lo[k] = (s - hi[k]) - y;
            hi[k] = s;
        }
    }
#pragma unroll
    for (int k = 0; k < kTpt; ++k) {
        const int t = t0 + threadIdx.x + k * blockDim.x;
        if (t < ntri) partials[(int64_t)blockIdx.x * ntri + t] = ok[k] ? (double)hi[k] - (double)lo[k] : 0.0;
    }
}

__global__ void reduce_partials_kernel(const double* __restrict__ partials, int nblk, int ntri,
                                       double* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    double acc = 0.0;
    for (int b = 0; b < nblk; ++b) acc += partials[(int64_t)b * ntri + t];
    out[t] = acc;
}

static void simple_grid(int64_t nvox, int ntri, unsigned* gx, unsigned* gy) {
    const int per_blk = kTpt * kCthreads;
    *gy = (unsigned)((ntri + per_blk - 1) / per_blk);
    int64_t chunks = (nvox + kVc - 1) / kVc;
    int64_t want = (int64_t)(2 * 152 * 2) / (int64_t)(*gy) + 1;
    *gx = (unsigned)(chunks < want ? (chunks < 1 ? 1 : chunks) : want);
}

size_t contract_simple_ws(int64_t nvox, int ntri) {
    unsigned gx, gy;
    simple_grid(nvox, ntri, &gx, &gy);
    return (size_t)gx * ntri * sizeof(double);
}

template <typename T>
int contract_simple_impl(const T* fields, int64_t fstride, int nshell, const int32_t* tri, int ntri, const T* wts,
                         int64_t nvox, double* bsum, double* partials, cudaStream_t st) {
    unsigned gx, gy;
    simple_grid(nvox, ntri, &gx, &gy);
    const size_t sm = sizeof(T) * ((size_t)kVc * (nshell + 1) + kVc);
    PYSPEC_TRY(allow_smem((const void*)contract_simple_kernel<T>, sm));
    contract_simple_kernel<T><<<dim3(gx, gy), kCthreads, sm, st>>>(fields, fstride, nshell, tri, ntri, wts, nvox,
                                                                   partials);
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    return reduce_partials_launch(partials, (int)gx, ntri, bsum, st);
}

int reduce_partials_launch(const double* partials, int nblk, int ntri, double* bsum, cudaStream_t st) {
    reduce_partials_kernel<<<(ntri + 255) / 256, 256, 0, st>>>(partials, nblk, ntri, bsum);
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    return PYSPEC_OK;
}

template int contract_simple_impl<float>(const float*, int64_t, int, const int32_t*, int, const float*, int64_t,
                                         double*, double*, cudaStream_t);
template int contract_simple_impl<double>(const double*, int64_t, int, const int32_t*, int, const double*, int64_t,
                                          double*, double*, cudaStream_t);

// ---------------------------------------------------------------------------
// FP32 CUDA-core contraction, register-tiled.  Triangles are grouped as
// (pair (i, j), shell l) like the tensor-core form: pairs sorted by (j, i),
// four consecutive pairs x eight consecutive l form one thread's micro-tile
// (32 accumulators).  Per voxel pair a thread loads 16 float2 values, forms 4
// pair products and issues 32 packed FP32x2 FMAs.  Voxel chunks are staged in
// shared memory with cp.async (double-buffered); each chunk's FP32 sums are
// folded into Kahan-compensated FP32 totals; CTAs write float64 partials.
// ---------------------------------------------------------------------------
namespace simt {
constexpr int MT = 4, NT = 8, VC = 128, FS = VC + 2;   // padded row of the staging buffer
constexpr int MAXT = 384;                               // micro-tiles per CTA (threads; 168 registers each)

struct Params {
    const float* fields;
    int64_t V;
    int nshell;
    int ntile;                 // micro-tiles
    int tiles_per_cta;         // threads per CTA (multiple of 32)
    const int16_t* tile_rows;  // [ntile][8]: i0..i3, j0..j3 (slot, -1 = empty row)
    const int16_t* tile_l0;    // [ntile]
    const int32_t* tile_tri;   // [ntile][32] triangle index or -1
    int ntri;
    int64_t nchunks, chunks_per_cta;
    double* partials;          // [gridDim.x][ntri]
};

__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    float2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(*reinterpret_cast<unsigned long long*>(&r))
        : "l"(*reinterpret_cast<unsigned long long*>(&a)), "l"(*reinterpret_cast<unsigned long long*>(&b)),
          "l"(*reinterpret_cast<unsigned long long*>(&c)));
    return r;
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
    float2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(*reinterpret_cast<unsigned long long*>(&r))
        : "l"(*reinterpret_cast<unsigned long long*>(&a)), "l"(*reinterpret_cast<unsigned long long*>(&b)));
    return r;
}

__global__ void __launch_bounds__(MAXT, 1) contract_fp32_kernel(const __grid_constant__ Params P) {
    extern __shared__ __align__(16) float sbuf[];       // 2 x (nshell + NT) x FS
    const int tid = threadIdx.x;
    const int rowsz = (P.nshell + NT) * FS;
    const int tile = blockIdx.y * P.tiles_per_cta + tid;
    const bool valid = tid < P.tiles_per_cta && tile < P.ntile;
    const int zero_row = P.nshell * FS;                  // never written by the copies
    // rows nshell .. nshell+NT-1 of both buffers are zero and never copied into
    for (int i = tid; i < NT * FS; i += blockDim.x) { sbuf[zero_row + i] = 0.f; sbuf[rowsz + zero_row + i] = 0.f; }
    int fi[MT], fj[MT];
#pragma unroll
    for (int k = 0; k < MT; ++k) {
        const int i = valid ? P.tile_rows[(size_t)tile * 8 + k] : -1;
        const int j = valid ? P.tile_rows[(size_t)tile * 8 + 4 + k] : -1;
        fi[k] = i >= 0 ? i * FS : zero_row;
        fj[k] = j >= 0 ? j * FS : zero_row;
    }
    // l0 + m <= nshell + NT - 1 always stays inside the buffer
    const int fl0 = (valid ? P.tile_l0[tile] : P.nshell) * FS;
    float hi[MT * NT], lo[MT * NT];
#pragma unroll
    for (int e = 0; e < MT * NT; ++e) { hi[e] = 0.f; lo[e] = 0.f; }

    const int64_t c0 = (int64_t)blockIdx.x * P.chunks_per_cta;
    const int64_t c1 = min(P.nchunks, c0 + P.chunks_per_cta);
    const int nch = (int)max((int64_t)0, c1 - c0);
    const int ncp = P.nshell * (VC / 4);
    auto issue = [&](int c, int buf) {
        const int64_t vbase = (c0 + c) * VC;
        for (int u = tid; u < ncp; u += blockDim.x) {
            const int s = u / (VC / 4), q = u - s * (VC / 4);
            const int64_t v = vbase + 4 * q;
            int bytes = 0;
            if (v < P.V) bytes = (int)min((int64_t)16, (P.V - v) * 4);
            const float* src = P.fields + (size_t)s * P.V + (bytes > 0 ? v : 0);
            const uint32_t dst = (uint32_t)__cvta_generic_to_shared(sbuf + buf * rowsz + s * FS + 4 * q);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" :: "r"(dst), "l"(src),
                         "r"(bytes > 8 ? 8 : bytes) : "memory");
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" :: "r"(dst + 8), "l"(src + 2),
                         "r"(bytes > 8 ? bytes - 8 : 0) : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    if (nch > 0) issue(0, 0);
    for (int c = 0; c < nch; ++c) {
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();
        if (c + 1 < nch) issue(c + 1, (c + 1) & 1);
        const float* F = sbuf + (c & 1) * rowsz;
        float2 cur[MT * NT];
#pragma unroll
        for (int e = 0; e < MT * NT; ++e) cur[e] = make_float2(0.f, 0.f);
        if (valid) {
#pragma unroll 2
            for (int v = 0; v < VC; v += 2) {
                float2 pp[MT], ll[NT];
#pragma unroll
                for (int k = 0; k < MT; ++k)
                    pp[k] = mul2(*reinterpret_cast<const float2*>(F + fi[k] + v),
                                 *reinterpret_cast<const float2*>(F + fj[k] + v));
#pragma unroll
                for (int m = 0; m < NT; ++m) ll[m] = *reinterpret_cast<const float2*>(F + fl0 + m * FS + v);
#pragma unroll
                for (int k = 0; k < MT; ++k)
#pragma unroll
                    for (int m = 0; m < NT; ++m) cur[k * NT + m] = fma2(pp[k], ll[m], cur[k * NT + m]);
            }
        }
#pragma unroll
        for (int e = 0; e < MT * NT; ++e) {   // Kahan fold of the chunk sum
            const float y = (cur[e].x + cur[e].y) - lo[e];
            const float t = hi[e] + y;
            lo[e] = (t - hi[e]) - y;
            hi[e] = t;
        }
        __syncthreads();   // everyone is done with buffer c&1 before it is refilled
    }
    if (valid) {
#pragma unroll
        for (int e = 0; e < MT * NT; ++e) {
            const int t = P.tile_tri[(size_t)tile * 32 + e];
            if (t >= 0) P.partials[(size_t)blockIdx.x * P.ntri + t] = (double)hi[e] - (double)lo[e];
        }
    }
}

static size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

struct HostPlan {
    std::vector<int16_t> rows, l0;
    std::vector<int32_t> tri;
    std::vector<char> image;          // rows | l0 | tri, each 256-byte aligned (device layout)
    const void* image_src = nullptr;  // page-locked copy of `image` (or image.data())
    size_t off_l0 = 0, off_tri = 0;
    int ntile = 0;
    bool ok = false;
};

static std::mutex g_mu;
static std::map<std::vector<int32_t>, HostPlan*> g_plans;

static HostPlan* plan(int nshell, const int32_t* tri_host, int ntri) {
    std::vector<int32_t> key(tri_host, tri_host + 3 * (size_t)ntri);
    key.push_back(nshell);
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_plans.find(key);
    if (it != g_plans.end()) return it->second;
    HostPlan* hp = new HostPlan();
    std::map<std::pair<int, int>, std::vector<std::pair<int, int>>> pairs;
    std::map<std::pair<int, int>, std::vector<bool>> seen;
    bool ok = true;
    for (int t = 0; t < ntri; ++t) {
        int v[3] = {tri_host[t], tri_host[ntri + t], tri_host[2 * ntri + t]};
        if (v[0] < 0 || v[1] < 0 || v[2] < 0 || v[0] >= nshell || v[1] >= nshell || v[2] >= nshell)
            continue;     // documented: such a triangle gets bsum = 0
        std::sort(v, v + 3);
        std::vector<bool>& sv = seen[{v[2], v[1]}];
        if (sv.empty()) sv.assign(nshell, false);
        if (sv[v[0]]) {
            ok = false;   // the same triangle twice
            continue;
        }
        sv[v[0]] = true;
        pairs[{v[2], v[1]}].push_back({v[0], t});
    }
    std::vector<std::pair<int, int>> order;
    for (auto& kv : pairs) order.push_back(kv.first);
    std::sort(order.begin(), order.end(), [](const std::pair<int, int>& a, const std::pair<int, int>& b) {
        return a.second != b.second ? a.second < b.second : a.first < b.first;
    });
    for (size_t g = 0; g < order.size(); g += MT) {
        int lo = 1 << 30, hi = -1;
        for (size_t r = g; r < std::min(order.size(), g + MT); ++r)
            for (auto& lt : pairs[order[r]]) { lo = std::min(lo, lt.first); hi = std::max(hi, lt.first); }
        for (int l0 = lo; l0 <= hi; l0 += NT) {
            int16_t rr[8];
            int32_t tt[32];
            for (int e = 0; e < 32; ++e) tt[e] = -1;
            for (int k = 0; k < MT; ++k) {
                const size_t r = g + k;
                rr[k] = r < order.size() ? (int16_t)order[r].first : (int16_t)-1;
                rr[4 + k] = r < order.size() ? (int16_t)order[r].second : (int16_t)-1;
                if (r >= order.size()) continue;
                for (auto& lt : pairs[order[r]])
                    if (lt.first >= l0 && lt.first < l0 + NT) tt[k * NT + lt.first - l0] = lt.second;
            }
            hp->rows.insert(hp->rows.end(), rr, rr + 8);
            hp->l0.push_back((int16_t)l0);
            hp->tri.insert(hp->tri.end(), tt, tt + 32);
            ++hp->ntile;
        }
    }
    hp->off_l0 = al(hp->rows.size() * 2);
    hp->off_tri = hp->off_l0 + al(hp->l0.size() * 2);
    hp->image.assign(hp->off_tri + al(hp->tri.size() * 4), 0);
    memcpy(hp->image.data(), hp->rows.data(), hp->rows.size() * 2);
    memcpy(hp->image.data() + hp->off_l0, hp->l0.data(), hp->l0.size() * 2);
    memcpy(hp->image.data() + hp->off_tri, hp->tri.data(), hp->tri.size() * 4);
    hp->image_src = pinned_copy(hp->image.data(), hp->image.size());
    if (hp->image_src == nullptr) hp->image_src = hp->image.data();
    hp->ok = ok;
    g_plans[key] = hp;
    return hp;
}

static void grid_dims(int64_t nvox, int ntile, int* gx, int* gy, int* per) {
    *gy = std::max(1, (ntile + MAXT - 1) / MAXT);
    *per = ((ntile + *gy - 1) / *gy + 31) / 32 * 32;
    int sms = 152, dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t nch = (nvox + VC - 1) / VC;
    *gx = (int)std::max<int64_t>(1, std::min<int64_t>(nch, std::max(1, sms / *gy)));
}

// The cached plan of a list, or nullptr (never plans, never allocates).
static HostPlan* find_plan(int nshell, const int32_t* tri_host, int ntri) {
    std::vector<int32_t> key(tri_host, tri_host + 3 * (size_t)ntri);
    key.push_back(nshell);
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_plans.find(key);
    return it == g_plans.end() ? nullptr : it->second;
}

}  // namespace simt

int contract_fp32_need(int64_t nvox, int nshell, const int32_t* tri_host, int ntri, bool may_plan, size_t* need) {
    using namespace simt;
    HostPlan* hp = may_plan ? plan(nshell, tri_host, ntri) : find_plan(nshell, tri_host, ntri);
    if (hp == nullptr) {
        set_error("this triangle list has no plan yet and planning allocates page-locked host memory, which a "
                  "stream capture forbids: make one call with this list outside the capture first");
        return PYSPEC_E_INVALID;
    }
    if (!hp->ok) {
        set_error("the triangle list repeats a triangle");
        return PYSPEC_E_INVALID;
    }
    if (!may_plan && hp->image_src == hp->image.data()) {
        set_error("the tile tables of this list are in pageable host memory (page-locked allocation failed), "
                  "which a captured copy cannot read");
        return PYSPEC_E_INVALID;
    }
    int gx, gy, per;
    grid_dims(nvox, hp->ntile, &gx, &gy, &per);
    *need = hp->image.size() + al((size_t)gx * ntri * sizeof(double));
    return PYSPEC_OK;
}

size_t contract_fp32_ws(int64_t nvox, int nshell, int ntri) {
    // worst-case tile count: plan() emits, for each group of MT pair rows, one
    // tile per NT-wide window of l from the group's lowest to its highest l,
    // empty windows included; a list has at most ntri distinct pairs
    const size_t groups = ((size_t)std::max(1, ntri) + simt::MT - 1) / simt::MT;
    const size_t windows = ((size_t)std::max(1, nshell) + simt::NT - 1) / simt::NT;
    const size_t maxtile = groups * windows;
    const size_t tables = simt::al(maxtile * 16) + simt::al(maxtile * 2) + simt::al(maxtile * 128);
    int sms = 152, dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    (void)nshell;
    (void)nvox;
    return tables + simt::al((size_t)sms * std::max(ntri, 1) * sizeof(double)) + 256;
}

int contract_fp32_impl(const float* fields, int64_t nvox, int nshell, const int32_t* tri_host, int ntri,
                       double* bsum, void* ws, size_t ws_bytes, cudaStream_t st) {
    using namespace simt;
    PYSPEC_CHECK_ARG(tri_host != nullptr, "the FP32 contraction needs the host copy of the triangle list");
    PYSPEC_CHECK_ARG(nvox % 4 == 0 && ((uintptr_t)fields & 15) == 0, "fields must be 16-byte aligned, N^3 % 4 == 0");
    HostPlan* hp = plan(nshell, tri_host, ntri);
    if (!hp->ok) {
        set_error("the triangle list repeats a triangle");
        return PYSPEC_E_INVALID;
    }
    int gx, gy, per;
    grid_dims(nvox, hp->ntile, &gx, &gy, &per);
    char* w = reinterpret_cast<char*>(ws);
    size_t off = 0;
    int16_t* d_rows = reinterpret_cast<int16_t*>(w + off);
    int16_t* d_l0 = reinterpret_cast<int16_t*>(w + off + hp->off_l0);
    int32_t* d_tri = reinterpret_cast<int32_t*>(w + off + hp->off_tri);
    off += hp->image.size();
    double* partials = reinterpret_cast<double*>(w + off);
    off += al((size_t)gx * ntri * sizeof(double));
    if (off > ws_bytes) {
        set_error("contract workspace %zu bytes < required %zu", ws_bytes, off);
        return PYSPEC_E_WORKSPACE;
    }
    PYSPEC_CUDA(cudaMemcpyAsync(d_rows, hp->image_src, hp->image.size(), cudaMemcpyHostToDevice, st));
    PYSPEC_CUDA(cudaMemsetAsync(partials, 0, (size_t)gx * ntri * sizeof(double), st));
    Params P;
    P.fields = fields;
    P.V = nvox;
    P.nshell = nshell;
    P.ntile = hp->ntile;
    P.tiles_per_cta = per;
    P.tile_rows = d_rows;
    P.tile_l0 = d_l0;
    P.tile_tri = d_tri;
    P.ntri = ntri;
    P.nchunks = (nvox + VC - 1) / VC;
    P.chunks_per_cta = (P.nchunks + gx - 1) / gx;
    P.partials = partials;
    const size_t sm = sizeof(float) * 2 * (size_t)(nshell + NT) * FS;
    PYSPEC_TRY(allow_smem((const void*)contract_fp32_kernel, sm));
    contract_fp32_kernel<<<dim3(gx, gy), per, sm, st>>>(P);
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    return reduce_partials_launch(partials, gx, ntri, bsum, st);
}

// ---------------------------------------------------------------------------
// Triangle counts.  The shell indicator fields I_j are invariant under
// permutations of the axes and under x -> N - x on each axis, so the voxel sum
// reduces to the fundamental domain 0 <= a <= b <= c <= N/2 with multiplicity
// (#distinct permutations) x prod(1 if v in {0, N/2} else 2).
// ---------------------------------------------------------------------------
__host__ __device__ inline int64_t domain_size(int n) {
    const int64_t h = n / 2;
    return (h + 1) * (h + 2) * (h + 3) / 6;
}

__global__ void build_domain_kernel(int n, int64_t* __restrict__ vox, double* __restrict__ wts) {
    const int h = n / 2;
    const int64_t m = h + 1;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m * m * m) return;
    const int a = (int)(t % m), b = (int)((t / m) % m), c = (int)(t / (m * m));
    if (!(a <= b && b <= c)) return;
    const int64_t rank = (int64_t)c * (c + 1) * (c + 2) / 6 + (int64_t)b * (b + 1) / 2 + a;
    int perms = (a == b && b == c) ? 1 : ((a == b || b == c) ? 3 : 6);
    auto sg = [h](int v) { return (v == 0 || v == h) ? 1 : 2; };
    vox[rank] = ((int64_t)c * n + b) * n + a;
    wts[rank] = (double)(perms * sg(a) * sg(b) * sg(c));
}

__global__ void gather_kernel(const double* __restrict__ field, const int64_t* __restrict__ vox, int64_t nvox,
                              double* __restrict__ out) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nvox) out[r] = field[vox[r]];
}

__global__ void round_counts_kernel(const double* __restrict__ bsum, int ntri, double vol,
                                    int64_t* __restrict__ counts) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < ntri) counts[t] = llrint(bsum[t] / vol);
}

__global__ void shift_tri_kernel(const int32_t* __restrict__ tri, int n3, int jmin, int32_t* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n3) out[t] = tri[t] - jmin;
}

static int64_t loop_triangles(int jmin, int nmax) {
    int64_t c = 0;
    for (int i = jmin; i <= nmax; ++i)
        for (int j = jmin; j <= i; ++j) c += j - max(i - j, jmin) + 1 > 0 ? j - max(i - j, jmin) + 1 : 0;
    return c;
}

static size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

struct CountsLayout {
    size_t work, tw, field, dom, vox, wts, part, bsum, tri, total;
};


static CountsLayout counts_layout(int n, int step, int jmin, int nmax) {
    CountsLayout L{};
    const int nshell = nmax - jmin + 1;
    const int64_t V = (int64_t)n * n * n;
    const int64_t nd = domain_size(n);
    const int64_t nt = loop_triangles(jmin, nmax);
    size_t o = 0;
    L.work = o; o += al(shell_workspace_bytes<double>(n, 1));
    L.tw = o; o += al((size_t)(n + n / 2) * sizeof(double2));
    L.field = o; o += al((size_t)V * sizeof(double));
    L.dom = o; o += al((size_t)nshell * nd * sizeof(double));
    L.vox = o; o += al((size_t)nd * sizeof(int64_t));
    L.wts = o; o += al((size_t)nd * sizeof(double));
    L.part = o; o += al(contract_simple_ws(nd, (int)nt));
    L.bsum = o; o += al((size_t)nt * sizeof(double));
    L.tri = o; o += al((size_t)3 * nt * sizeof(int32_t));
    L.total = o;
    (void)step;
    return L;
}

// ---------------------------------------------------------------------------
// pyspectrum.py:418-437 and :341-355
// ---------------------------------------------------------------------------
__global__ void bk_normalize_kernel(const double* __restrict__ bsum, const int64_t* __restrict__ counts,
                                    const double* __restrict__ p0sum, const int64_t* __restrict__ nk,
                                    const int32_t* __restrict__ tri, int ntri, double vol, int jmin, int nmax,
                                    int apply_units, double nbar, double kf, double* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    const int i = tri[t], j = tri[ntri + t], l = tri[2 * ntri + t];
    if (i < jmin || i > nmax || j < jmin || j > nmax || l < jmin || l > nmax) {
        for (int r = 0; r < 7; ++r) out[r * ntri + t] = 0.0;
        return;
    }
    auto p0 = [&](int a) { return p0sum[a - jmin] / vol / (double)nk[a]; };   // pyspectrum.py:404
    double pi = p0(i), pj = p0(j), pl = p0(l);
    const double c = (double)counts[t] * vol;
    double fac = 1.0;
    if (i == j && j == l) fac = 6.0;
    else if (i == j || j == l || i == l) fac = 2.0;
    double b = 0, q = 0, cnt = 0, bsn = 0;
    if (counts[t] > 0) {
        b = bsum[t] / c;
        q = b / (pi * pj + pj * pl + pl * pi);
        cnt = (double)counts[t] / fac;
    } else {
        pi = pj = pl = 0;
    }
    if (apply_units && counts[t] > 0) {
        const double tp = 2.0 * 3.14159265358979323846;
        const double u3 = (tp * tp * tp) / (kf * kf * kf);
        pi = pi * u3 - 1.0 / nbar;
        pj = pj * u3 - 1.0 / nbar;
        pl = pl * u3 - 1.0 / nbar;
        bsn = (pi + pj + pl) / nbar + 1.0 / (nbar * nbar);
        b = b * u3 * u3 - bsn;
        q = b / (pi * pj + pi * pl + pj * pl);
    }
    out[t] = pi;
    out[ntri + t] = pj;
    out[2 * ntri + t] = pl;
    out[3 * ntri + t] = b;
    out[4 * ntri + t] = q;
    out[5 * ntri + t] = cnt;
    out[6 * ntri + t] = bsn;
}

}  // namespace pyspec

using namespace pyspec;

extern "C" size_t pyspec_bk_counts_workspace(int ngrid, int step, int jmin, int nmax) {
    if (ngrid < 4 || ngrid % 2 || jmin < 1 || nmax < jmin) return 0;
    return counts_layout(ngrid, step, jmin, nmax).total;
}

extern "C" int pyspec_bk_counts(int ngrid, int step, int jmin, int nmax, const int32_t* tri, int ntri,
                                int64_t* counts, int64_t* nk, void* workspace, size_t ws_bytes, void* stream) {
    PYSPEC_CHECK_ARG(tri && counts, "NULL pointer");
    PYSPEC_CHECK_ARG(ngrid >= 4 && ngrid % 2 == 0 && ngrid <= 2048, "ngrid=%d must be even", ngrid);
    PYSPEC_CHECK_ARG(step >= 1 && jmin >= 1 && nmax >= jmin && nmax - jmin + 1 <= kMaxShells, "bad shells");
    const CountsLayout L = counts_layout(ngrid, step, jmin, nmax);
    PYSPEC_CHECK_ARG(ntri >= 0 && ntri <= loop_triangles(jmin, nmax), "ntri exceeds the triangle loop size");
    if (ws_bytes < L.total || workspace == nullptr) {
        set_error("counts workspace %zu bytes < required %zu", ws_bytes, L.total);
        return PYSPEC_E_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    char* w = reinterpret_cast<char*>(workspace);
    const int n = ngrid, nshell = nmax - jmin + 1;
    const int64_t nd = domain_size(n);
    int64_t* vox = reinterpret_cast<int64_t*>(w + L.vox);
    double* wts = reinterpret_cast<double*>(w + L.wts);
    double* dom = reinterpret_cast<double*>(w + L.dom);
    double* field = reinterpret_cast<double*>(w + L.field);
    const int64_t m = n / 2 + 1;
    build_domain_kernel<<<(unsigned)((m * m * m + 255) / 256), 256, 0, st>>>(n, vox, wts);
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    double* part = reinterpret_cast<double*>(w + L.work + al((size_t)(n / 2 + 1) * n * n * sizeof(double2)));
    double2* tw = reinterpret_cast<double2*>(w + L.tw);
    PYSPEC_TRY(shell_twiddles<double>(tw, n, st));
    for (int s = 0; s < nshell; ++s) {
        // the x pass writes one partial per CTA right after the work grid
        PYSPEC_TRY((shell_one_impl<double, true>(nullptr, n, step, jmin + s, field, part,
                                                  reinterpret_cast<double2*>(w + L.work), tw, st)));
        gather_kernel<<<(unsigned)((nd + 255) / 256), 256, 0, st>>>(field, vox, nd, dom + (int64_t)s * nd);
        PYSPEC_LAUNCH_CHECK();
        count_launch();
    }
    if (ntri > 0) {
        int32_t* slots = reinterpret_cast<int32_t*>(w + L.tri);
        shift_tri_kernel<<<(3 * ntri + 255) / 256, 256, 0, st>>>(tri, 3 * ntri, jmin, slots);
        PYSPEC_LAUNCH_CHECK();
        double* bsum = reinterpret_cast<double*>(w + L.bsum);
        PYSPEC_TRY(contract_simple_impl<double>(dom, nd, nshell, slots, ntri, wts, nd, bsum,
                                                reinterpret_cast<double*>(w + L.part), st));
        round_counts_kernel<<<(ntri + 255) / 256, 256, 0, st>>>(bsum, ntri, (double)n * n * n, counts);
        PYSPEC_LAUNCH_CHECK();
        count_launch(2);
    }
    if (nk) PYSPEC_TRY(mode_counts_impl(n, step, nmax, nk, st));
    return PYSPEC_OK;
}

extern "C" int pyspec_bk_normalize(const double* bsum, const int64_t* counts, const double* p0sum,
                                   const int64_t* nk, const int32_t* tri, int ntri, int ngrid, int jmin, int nmax,
                                   int apply_units, double nbar, double kf, double* out, void* stream) {
    PYSPEC_CHECK_ARG(bsum && counts && p0sum && nk && tri && out, "NULL pointer");
    PYSPEC_CHECK_ARG(ntri >= 0 && ngrid >= 2, "bad arguments");
    if (ntri == 0) return PYSPEC_OK;
    const double vol = (double)ngrid * ngrid * ngrid;
    bk_normalize_kernel<<<(ntri + 127) / 128, 128, 0, as_stream(stream)>>>(bsum, counts, p0sum, nk, tri, ntri, vol,
                                                                          jmin, nmax, apply_units, nbar, kf, out);
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    return PYSPEC_OK;
}

extern "C" size_t pyspec_bk_contract_workspace(int ngrid, int nshell, int ntri, int method) {
    method &= ~(PYSPEC_CONTRACT_RUN_PLAN | PYSPEC_CONTRACT_FINE_DRAIN | PYSPEC_CONTRACT_KC32);
    if (ngrid < 2 || nshell < 1 || ntri < 0) return 0;
    const int64_t V = (int64_t)ngrid * ngrid * ngrid;
    if (method == PYSPEC_CONTRACT_BF16X3) return contract_tc_ws(V, nshell, ntri);
    if (method == PYSPEC_CONTRACT_BF16X6) return contract_tc_ws(V, nshell, ntri, true);
    return std::max(contract_fp32_ws(V, nshell, ntri), contract_simple_ws(V, ntri));
}

extern "C" int pyspec_bk_contract(const float* fields, int ngrid, int nshell, const int32_t* tri,
                                  const int32_t* tri_host, int ntri, int method, double* bsum, void* workspace,
                                  size_t ws_bytes, void* stream) {
    PYSPEC_CHECK_ARG(fields && tri && bsum, "NULL pointer");
    PYSPEC_CHECK_ARG(ngrid >= 2 && nshell >= 1 && nshell <= kMaxShells && ntri >= 0, "bad arguments");
    if (ntri == 0) return PYSPEC_OK;
    const int64_t V = (int64_t)ngrid * ngrid * ngrid;
    const size_t need = pyspec_bk_contract_workspace(ngrid, nshell, ntri, method);
    if (workspace == nullptr || ws_bytes < need) {
        set_error("contract workspace %zu bytes < required %zu", ws_bytes, need);
        return PYSPEC_E_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    const bool run_plan = (method & PYSPEC_CONTRACT_RUN_PLAN) != 0;
    const bool fine_drain = (method & PYSPEC_CONTRACT_FINE_DRAIN) != 0;
    const bool kc32 = (method & PYSPEC_CONTRACT_KC32) != 0;
    method &= ~(PYSPEC_CONTRACT_RUN_PLAN | PYSPEC_CONTRACT_FINE_DRAIN | PYSPEC_CONTRACT_KC32);
    PYSPEC_CHECK_ARG((!run_plan && !fine_drain && !kc32) || method == PYSPEC_CONTRACT_BF16X3 ||
                         method == PYSPEC_CONTRACT_BF16X6,
                     "PYSPEC_CONTRACT_RUN_PLAN, _FINE_DRAIN and _KC32 apply to the tensor-core methods only");
    if (method == PYSPEC_CONTRACT_FP32) {
        if (tri_host == nullptr)   // device-only triangle list: the unplanned kernel
            return contract_simple_impl<float>(fields, V, nshell, tri, ntri, nullptr, V, bsum,
                                               reinterpret_cast<double*>(workspace), st);
        return contract_fp32_impl(fields, V, nshell, tri_host, ntri, bsum, workspace, ws_bytes, st);
    }
    if (method == PYSPEC_CONTRACT_BF16X3)
        return contract_tc_impl(fields, V, nshell, tri, tri_host, ntri, bsum, workspace, ws_bytes, st, run_plan,
                                fine_drain, false, kc32);
    if (method == PYSPEC_CONTRACT_BF16X6)
        return contract_tc_impl(fields, V, nshell, tri, tri_host, ntri, bsum, workspace, ws_bytes, st, run_plan,
                                true, true, kc32);
    set_error("unknown contraction method %d", method);
    return PYSPEC_E_INVALID;
}
