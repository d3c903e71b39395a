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
// four consecutive pairs x one aligned window of eight shells l (l0 a
// multiple of 8) form one thread's micro-tile (32 accumulators).  The
// threads of a warp hold consecutive micro-tiles, so the lanes of one pair
// group read the same F_i, F_j words and a warp's window rows are at most
// five distinct rows per load, which keeps bank conflicts rare.  (Sharing
// does not cut the load cost itself: an LDS.128 takes four wavefronts
// whatever its addresses, so the kernel's bound is the 2 bytes each lane
// loads per FMA, half the FP32 FMA rate at 128 bytes per cycle per SM.)
//
// Voxel chunks of every shell are staged in shared memory by bulk copies
// that one producer warp issues (double-buffered; "full" mbarriers complete
// with the copies, "empty" ones when every compute warp is done with a
// buffer, so no warp waits for another's compute); row r starts at r * RS + 4 * ((r +
// r / 8) % 8) floats, so rows that differ in r % 8 or in r / 8 start in
// different 16-byte bank groups.  Per four voxels a thread loads its eight
// window rows and four (F_i, F_j) pairs and issues 64 packed FP32x2 FMAs;
// each chunk's sums are folded into Kahan-compensated FP32 totals held in
// shared memory; CTAs write float64 partials.
// ---------------------------------------------------------------------------
namespace simt {
constexpr int MT = 4, NT = 8, VC = 128;
constexpr int RS = VC + 32;                             // floats per staged row incl. its bank shift
constexpr int MAXT = 352;                               // micro-tiles (compute threads) per CTA
constexpr int THREADS_MAX = MAXT + 32;                  // + the producer warp
__host__ __device__ constexpr int row_off(int r) { return r * RS + 4 * ((r + (r >> 3)) & 7); }
// floats of one staging buffer: nshell field rows and NT zero rows
__host__ __device__ constexpr size_t buf_floats(int nshell) { return (size_t)(nshell + NT) * RS; }
__host__ __device__ constexpr size_t fp32_smem(int nshell, int threads) {
    return 2 * buf_floats(nshell) * sizeof(float) + (size_t)MT * NT * threads * sizeof(float2);
}

struct Params {
    const float* fields;
    int64_t V;
    int nshell;
    int ntile;                 // micro-tiles
    int tiles_per_cta;         // compute threads per CTA (multiple of 32); the producer warp follows
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
__device__ __forceinline__ float4 lds4f(const float* p) { return *reinterpret_cast<const float4*>(p); }

// bounded wait on an mbarrier phase (~2 s of globaltimer), false on timeout
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
    unsigned long long t0 = 0;
    for (uint32_t it = 0;; ++it) {
        uint32_t ok;
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        if (ok) return true;
        if ((it & 255u) == 0) {
            unsigned long long t;
            asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
            if (t0 == 0) t0 = t;
            else if (t - t0 > 2000000000ull) return false;
        }
    }
}

__global__ void __launch_bounds__(THREADS_MAX, 1) contract_fp32_kernel(const __grid_constant__ Params P) {
    extern __shared__ __align__(16) float sbuf[];        // 2 staging buffers, then the Kahan state
    __shared__ __align__(8) uint64_t full[2], empty[2];
    __shared__ int abort_flag_s;
    volatile int& abort_flag = abort_flag_s;
    const int tid = threadIdx.x, nthr = P.tiles_per_cta;  // compute threads; the producer warp follows
    const int ncw = nthr / 32;
    const size_t BUF = buf_floats(P.nshell);
    float2* kahan = reinterpret_cast<float2*>(sbuf + 2 * BUF);   // [32][nthr]: (sum, compensation)
    const int tile = blockIdx.y * P.tiles_per_cta + tid;
    const bool valid = tid < nthr && tile < P.ntile;
    // rows nshell .. nshell + NT - 1 of both buffers stay zero (never copied into)
    for (size_t i = tid; i < 2 * BUF; i += blockDim.x) sbuf[i] = 0.f;
    for (int i = tid; i < MT * NT * nthr; i += blockDim.x) kahan[i] = make_float2(0.f, 0.f);
    const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(&full[0]);
    const uint32_t ebar0 = (uint32_t)__cvta_generic_to_shared(&empty[0]);
    if (tid == 0) {
        abort_flag = 0;
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar0 + 8u * b), "r"(1));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(ebar0 + 8u * b), "r"(ncw));
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // the zero fill (generic proxy) is ordered before the bulk copies (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    int oi[MT], oj[MT], ol[NT];
#pragma unroll
    for (int k = 0; k < MT; ++k) {
        const int i = valid ? P.tile_rows[(size_t)tile * 8 + k] : -1;
        const int j = valid ? P.tile_rows[(size_t)tile * 8 + 4 + k] : -1;
        oi[k] = row_off(i >= 0 ? i : P.nshell);
        oj[k] = row_off(j >= 0 ? j : P.nshell);
    }
    {
        // l0 is a multiple of NT and l0 + NT - 1 < nshell + NT: inside the buffer
        const int l0 = valid ? P.tile_l0[tile] : P.nshell / NT * NT;
#pragma unroll
        for (int m = 0; m < NT; ++m) ol[m] = row_off(l0 + m);
    }
    const int64_t c0 = (int64_t)blockIdx.x * P.chunks_per_cta;
    const int64_t c1 = min(P.nchunks, c0 + P.chunks_per_cta);
    const int nch = (int)max((int64_t)0, c1 - c0);
    // the producer: chunk c of this CTA into buffer b, one bulk copy per shell row
    auto issue = [&](int c, int b) {
        const int64_t v0 = (c0 + c) * VC;
        const uint32_t bytes = (uint32_t)(min((int64_t)VC, P.V - v0) * 4);
        const uint32_t bar = bar0 + 8u * b;
        const uint32_t dst0 = (uint32_t)__cvta_generic_to_shared(sbuf + (size_t)b * BUF);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(bytes * P.nshell)
                     : "memory");
        for (int r = 0; r < P.nshell; ++r)
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                         :: "r"(dst0 + 4u * (uint32_t)row_off(r)), "l"(P.fields + (size_t)r * P.V + v0), "r"(bytes),
                            "r"(bar)
                         : "memory");
    };
    if (tid >= nthr) {
        // ================= producer warp =================
        if (tid == nthr) {
            int c = 0;
            for (; c < nch; ++c) {
                const int b = c & 1;
                if (c >= 2) {
                    if (!bar_wait(ebar0 + 8u * b, (uint32_t)((c - 2) >> 1) & 1u) || abort_flag) {
                        abort_flag = 1;
                        break;
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                }
                issue(c, b);
            }
            // no copy may land after the CTA exits: wait (bounded) for the last ones
            for (int k = max(0, c - 2); k < c; ++k) (void)bar_wait(bar0 + 8u * (k & 1), (uint32_t)(k >> 1) & 1u);
        }
        return;
    }
    // ================= compute warps =================
    bool ok = true;
    for (int c = 0; c < nch; ++c) {
        const int b = c & 1;
        // warp-uniform: every lane takes the same branch
        const bool landed = __all_sync(0xffffffffu, bar_wait(bar0 + 8u * b, (uint32_t)(c >> 1) & 1u));
        if (!landed || __any_sync(0xffffffffu, abort_flag != 0)) {
            abort_flag = 1;
            ok = false;
            break;
        }
        const float* F = sbuf + (size_t)b * BUF;
        const int nq = (int)(min((int64_t)VC, P.V - (c0 + c) * VC) / 4);
        if (valid) {
            float2 acc[MT * NT];
#pragma unroll
            for (int e = 0; e < MT * NT; ++e) acc[e] = make_float2(0.f, 0.f);
#pragma unroll 1
            for (int q = 0; q < nq; ++q) {
                const int o = 4 * q;
                float4 fl[NT];
#pragma unroll
                for (int m = 0; m < NT; ++m) fl[m] = lds4f(F + ol[m] + o);
#pragma unroll
                for (int k = 0; k < MT; ++k) {
                    const float4 a = lds4f(F + oi[k] + o), bb = lds4f(F + oj[k] + o);
                    const float2 p0 = mul2(make_float2(a.x, a.y), make_float2(bb.x, bb.y));
                    const float2 p1 = mul2(make_float2(a.z, a.w), make_float2(bb.z, bb.w));
#pragma unroll
                    for (int m = 0; m < NT; ++m) {
                        acc[k * NT + m] = fma2(p0, make_float2(fl[m].x, fl[m].y), acc[k * NT + m]);
                        acc[k * NT + m] = fma2(p1, make_float2(fl[m].z, fl[m].w), acc[k * NT + m]);
                    }
                }
            }
#pragma unroll
            for (int e = 0; e < MT * NT; ++e) {   // Kahan fold of the chunk sum
                float2 h = kahan[e * nthr + tid];
                const float y = (acc[e].x + acc[e].y) - h.y;
                const float t = h.x + y;
                h.y = (t - h.x) - y;
                h.x = t;
                kahan[e * nthr + tid] = h;
            }
        }
        __syncwarp();      // this warp is done with buffer b
        if ((tid & 31) == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(ebar0 + 8u * b) : "memory");
    }
    if (!ok) {
        // a copy never completed: report NaN partials for this warp's triangles
        if (valid) {
#pragma unroll 1
            for (int e = 0; e < MT * NT; ++e) {
                const int t = P.tile_tri[(size_t)tile * 32 + e];
                if (t >= 0) P.partials[(size_t)blockIdx.x * P.ntri + t] = __longlong_as_double(0x7ff8000000000000ll);
            }
        }
        return;
    }
    if (valid) {
#pragma unroll
        for (int e = 0; e < MT * NT; ++e) {
            const int t = P.tile_tri[(size_t)tile * 32 + e];
            const float2 h = kahan[e * nthr + tid];
            if (t >= 0) P.partials[(size_t)blockIdx.x * P.ntri + t] = (double)h.x - (double)h.y;
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
        for (int l0 = lo / NT * NT; l0 <= hi; l0 += NT) {
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

// threads (micro-tiles) per CTA that the shared memory leaves room for
static int max_tiles(int nshell) {
    const size_t lim = 227 * 1024, bufs = 2 * buf_floats(nshell) * sizeof(float);
    if (bufs >= lim) return 0;
    return std::min<int>(MAXT, (int)((lim - bufs) / (MT * NT * sizeof(float2))) / 32 * 32);
}

static bool grid_dims(int64_t nvox, int nshell, int ntile, int* gx, int* gy, int* per) {
    const int mt = max_tiles(nshell);
    if (mt < 32) return false;
    *gy = std::max(1, (ntile + mt - 1) / mt);
    *per = ((ntile + *gy - 1) / *gy + 31) / 32 * 32;
    int sms = 152, dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t nch = (nvox + VC - 1) / VC;
    *gx = (int)std::max<int64_t>(1, std::min<int64_t>(nch, std::max(1, sms / *gy)));
    return true;
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
    if (!grid_dims(nvox, nshell, hp->ntile, &gx, &gy, &per)) {
        set_error("%d shells do not fit the FP32 contraction's shared-memory staging", nshell);
        return PYSPEC_E_UNSUPPORTED;
    }
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
    if (!grid_dims(nvox, nshell, hp->ntile, &gx, &gy, &per)) {
        set_error("%d shells do not fit the FP32 contraction's shared-memory staging", nshell);
        return PYSPEC_E_UNSUPPORTED;
    }
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
    const size_t sm = fp32_smem(nshell, per);
    PYSPEC_TRY(allow_smem((const void*)contract_fp32_kernel, sm));
    contract_fp32_kernel<<<dim3(gx, gy), per + 32, sm, st>>>(P);   // + the producer warp
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
