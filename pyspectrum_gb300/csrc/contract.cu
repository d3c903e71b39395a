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
    reduce_partials_kernel<<<(ntri + 255) / 256, 256, 0, st>>>(partials, (int)gx, ntri, bsum);
    PYSPEC_LAUNCH_CHECK();
    count_launch(2);
    return PYSPEC_OK;
}

template int contract_simple_impl<float>(const float*, int64_t, int, const int32_t*, int, const float*, int64_t,
                                         double*, double*, cudaStream_t);
template int contract_simple_impl<double>(const double*, int64_t, int, const int32_t*, int, const double*, int64_t,
                                          double*, double*, cudaStream_t);

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
    size_t work, field, dom, vox, wts, part, bsum, tri, total;
};


static CountsLayout counts_layout(int n, int step, int jmin, int nmax) {
    CountsLayout L{};
    const int nshell = nmax - jmin + 1;
    const int64_t V = (int64_t)n * n * n;
    const int64_t nd = domain_size(n);
    const int64_t nt = loop_triangles(jmin, nmax);
    size_t o = 0;
    L.work = o; o += al(shell_workspace_bytes<double>(n, 1));
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
    for (int s = 0; s < nshell; ++s) {
        // the x pass writes one partial per CTA right after the work grid
        double* part = reinterpret_cast<double*>(w + L.work + al((size_t)(n / 2 + 1) * n * n * sizeof(double2)));
        PYSPEC_TRY((shell_one_impl<double, true>(nullptr, n, step, jmin + s, field, part,
                                                  reinterpret_cast<double2*>(w + L.work), st)));
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
    if (ngrid < 2 || nshell < 1 || ntri < 0) return 0;
    const int64_t V = (int64_t)ngrid * ngrid * ngrid;
    if (method == PYSPEC_CONTRACT_BF16X3) return contract_tc_ws(V, nshell, ntri);
    return contract_simple_ws(V, ntri);
}

extern "C" int pyspec_bk_contract(const float* fields, int ngrid, int nshell, const int32_t* tri, int ntri,
                                  int method, double* bsum, void* workspace, size_t ws_bytes, void* stream) {
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
    if (method == PYSPEC_CONTRACT_FP32)
        return contract_simple_impl<float>(fields, V, nshell, tri, ntri, nullptr, V, bsum,
                                           reinterpret_cast<double*>(workspace), st);
    if (method == PYSPEC_CONTRACT_BF16X3)
        return contract_tc_impl(fields, V, nshell, tri, ntri, bsum, workspace, ws_bytes, st);
    set_error("unknown contraction method %d", method);
    return PYSPEC_E_INVALID;
}
