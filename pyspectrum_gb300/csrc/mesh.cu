// Particles -> delta(k): input preparation, PCS + interlaced mass assignment,
// the interlacing combine / deconvolution, and half <-> full grid helpers.
#include "common.cuh"

namespace pyspec {

// ---------------------------------------------------------------------------
// pyspectrum.py:938-945 and util.py:72-74
// ---------------------------------------------------------------------------
// With clip == false (the survey path, pyspectrum.py:789-793) positions are
// only cast to float32; lbox and the RSD shift are unused.
__global__ void prepare_positions_kernel(const double* __restrict__ xyz, int64_t ds, const double* __restrict__ v,
                                         int64_t vs, int los, double rsd_factor, const double* __restrict__ w,
                                         int64_t np, double lbox, bool clip, float* __restrict__ out,
                                         float* __restrict__ wout) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const double hi = lbox * (1.0 - 1e-6);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double x = xyz[d * ds + i];
        if (clip) {
            if (v != nullptr && d == los) {
                // applyRSD: (x + f*v + L) mod L, numpy's floored modulo
                x = x + (rsd_factor * v[d * vs + i] + lbox);
                x = x - floor(x / lbox) * lbox;
            }
            x = fmin(fmax(x, 0.0), hi);
        }
        out[d * np + i] = (float)x;
    }
    if (wout != nullptr) wout[i] = w ? (float)w[i] : 1.0f;
}

// ---------------------------------------------------------------------------
// estimator.f:284-512 -- PCS weights and cell indices in IEEE single precision
// without contraction (the __f*_rn intrinsics), so the cells chosen match the
// Fortran bit for bit.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pcs_w(float h, float* o) {
    const float h2 = __fmul_rn(h, h);
    const float om = __fsub_rn(1.0f, h);
    const float wm2 = __fmul_rn(__fmul_rn(om, om), om);
    const float wm1 = __fadd_rn(4.0f, __fmul_rn(__fsub_rn(__fmul_rn(3.0f, h), 6.0f), h2));
    const float wp2 = __fmul_rn(h2, h);
    const float wp1 = __fsub_rn(__fsub_rn(__fsub_rn(6.0f, wm2), wm1), wp2);
    o[0] = wm2; o[1] = wm1; o[2] = wp1; o[3] = wp2;
}

__device__ __forceinline__ int wrapi(int c, int n) {
    c %= n;
    return c < 0 ? c + n : c;
}

__global__ void __launch_bounds__(128) assign_pcs_kernel(const float* __restrict__ xyz, const float* __restrict__ w,
                                                         int64_t np, int n, float kf_ks, float offset,
                                                         float* __restrict__ grid) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const float we = w ? w[i] : 1.0f;
    int base[2][3];
    float wt[2][3][4];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float r = xyz[d * np + i];
        const float rx = __fadd_rn(__fadd_rn(__fmul_rn(kf_ks, r), 1.0f), offset);   // estimator.f:302
        const float tx = __fadd_rn(rx, 0.5f);                                      // estimator.f:305
        const int m = __float2int_rz(rx);
        const int q = __float2int_rz(tx);
        pcs_w(__fsub_rn(rx, (float)m), wt[0][d]);
        pcs_w(__fsub_rn(tx, (float)q), wt[1][d]);
        base[0][d] = m;
        base[1][d] = q;
    }
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        int cx[4], cy[4], cz[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            cx[c] = wrapi(base[s][0] - 2 + c, n);
            cy[c] = wrapi(base[s][1] - 2 + c, n);
            cz[c] = wrapi(base[s][2] - 2 + c, n);
        }
#pragma unroll
        for (int c3 = 0; c3 < 4; ++c3) {
#pragma unroll
            for (int c2 = 0; c2 < 4; ++c2) {
                const int64_t row = ((int64_t)cz[c3] * n + cy[c2]) * n;
#pragma unroll
                for (int c1 = 0; c1 < 4; ++c1) {
                    // estimator.f:380: ((hx*hy)*hz)*we
                    const float v = __fmul_rn(__fmul_rn(__fmul_rn(wt[s][0][c1], wt[s][1][c2]), wt[s][2][c3]), we);
                    atomicAdd(grid + 2 * (row + cx[c1]) + s, v);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// estimator.f:605-675 (fcomb_periodic).  One thread per Fortran iteration
// (ix,iy,iz) in [1, N/2+1]^3 (0-based here).  The iteration reads and writes
// the 8-point orbit {ix,icx} x {iy,icy} x {iz,icz}; orbits of different
// iterations are disjoint, so threads never race.  Inside an orbit the
// Fortran's eight assignments alias when ix==icx, iy==icy or iz==icz, and the
// last assignment wins; the slots below replay that order.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) fcomb_kernel(const float2* __restrict__ G, int n, float cf,
                                                    float2* __restrict__ half) {
    const int lnyq = n / 2 + 1;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)lnyq * lnyq * lnyq) return;
    const int ix = (int)(t % lnyq);
    const int iy = (int)((t / lnyq) % lnyq);
    const int iz = (int)(t / ((int64_t)lnyq * lnyq));
    const int icx = (n - ix) % n, icy = (n - iy) % n, icz = (n - iz) % n;

    // exp(-i*pi*k/N) and sinc^4 window per axis (estimator.f:620-623, 632)
    auto rec = [&](int k, float2& r, float& W) {
        float s, c;
        sincospif((float)k / (float)n, &s, &c);
        r = make_float2(c, -s);
        if (k == 0) W = 1.0f;
        else {
            const float a = 3.14159265358979f * (float)k / (float)n;
            const float sn = sinpif((float)k / (float)n) / a;
            const float s2 = sn * sn;
            W = s2 * s2;
        }
    };
    float2 xr, yr, zr;
    float Wx, Wy, Wz;
    rec(ix, xr, Wx);
    rec(iy, yr, Wy);
    rec(iz, zr, Wz);
    const float cfac = cf / (Wx * Wy * Wz);
    auto mul = [](float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
    auto cj = [](float2 a) { return make_float2(a.x, -a.y); };
    auto mi = [](float2 a) { return make_float2(-a.y, a.x); };  // multiply by i
    const float2 xy = mul(xr, yr), xyc = mul(xr, cj(yr));
    const float2 cma = mi(mul(xy, zr));
    const float2 cmb = mi(mul(xy, cj(zr)));
    const float2 cmc = mi(mul(xyc, zr));
    const float2 cmd = mi(mul(xr, cj(mul(yr, zr))));

    const int64_t nn = n;
    int64_t pos[8];
    const int xs[2] = {ix, icx}, ys[2] = {iy, icy}, zs[2] = {iz, icz};
    // slot order: (ix,iy,iz) (ix,iy,icz) (ix,icy,iz) (ix,icy,icz), then the same on icx
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int X = xs[k >> 2], Y = ys[(k >> 1) & 1], Z = zs[k & 1];
        pos[k] = ((int64_t)Z * nn + Y) * nn + X;
    }
    float2 val[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) val[k] = G[pos[k]];
    auto write = [&](int k, float2 v) {
#pragma unroll
        for (int k2 = 0; k2 < 8; ++k2)
            if (pos[k2] == pos[k]) val[k2] = v;
    };
    auto comb = [&](float2 a, float2 b, float2 cm) {
        // a*(1-cm) + conj(b)*(1+cm)
        const float2 one_m = make_float2(1.0f - cm.x, -cm.y), one_p = make_float2(1.0f + cm.x, cm.y);
        const float2 p = mul(a, one_m), q = mul(cj(b), one_p);
        return make_float2((p.x + q.x) * cfac, (p.y + q.y) * cfac);
    };
    const float2 c000 = comb(val[0], val[7], cma);   // estimator.f:652
    const float2 c001 = comb(val[1], val[6], cmb);   // :653
    const float2 c010 = comb(val[2], val[5], cmc);   // :654
    const float2 c011 = comb(val[3], val[4], cmd);   // :655
    write(0, c000);                                  // :658-661
    write(1, c001);
    write(2, c010);
    write(3, c011);
    write(4, cj(val[3]));                            // :662-665
    write(5, cj(val[2]));
    write(6, cj(val[1]));
    write(7, cj(val[0]));
    const int nh = lnyq;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int X = xs[k >> 2], Y = ys[(k >> 1) & 1], Z = zs[k & 1];
        if (X < nh) half[((int64_t)Z * nn + Y) * nh + X] = val[k];
    }
}

// pyspectrum.py:1134-1157
__global__ void reflect_kernel(const float2* __restrict__ half, int n, float2* __restrict__ full) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nn = n;
    if (t >= nn * nn * nn) return;
    const int x = (int)(t % nn), y = (int)((t / nn) % nn), z = (int)(t / (nn * nn));
    const int nh = n / 2 + 1, hg = n / 2;
    float2 v;
    if (x <= hg) v = half[((int64_t)z * nn + y) * nh + x];
    else {
        const float2 u = half[((int64_t)((n - z) % n) * nn + (n - y) % n) * nh + (n - x)];
        v = make_float2(u.x, -u.y);
    }
    const bool cx = (x == 0 || x == hg), cy = (y == 0 || y == hg), cz = (z == 0 || z == hg);
    if (cx && cy && cz && !(x == 0 && y == 0 && z == 0)) v.y = 0.0f;
    full[t] = v;
}

__global__ void half_from_full_kernel(const float2* __restrict__ full, int n, float2* __restrict__ half) {
    const int nh = n / 2 + 1;
    const int64_t nn = n;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nh * nn * nn) return;
    const int x = (int)(t % nh), y = (int)((t / nh) % nn), z = (int)(t / (nh * nn));
    float2 a = full[((int64_t)z * nn + y) * nn + x];
    if (x != 0 && x != n / 2) {
        const float2 b = full[((int64_t)((n - z) % n) * nn + (n - y) % n) * nn + (n - x)];
        a = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
    }
    half[t] = a;
}

}  // namespace pyspec

using namespace pyspec;

extern "C" int pyspec_prepare_positions(const double* xyz, int64_t dim_stride, const double* vxyz,
                                        int64_t vdim_stride, int los, double rsd_factor, const double* w,
                                        int64_t np, double lbox, float* xyz_out, float* w_out, void* stream) {
    PYSPEC_CHECK_ARG(np >= 0, "np < 0");
    if (np == 0) return PYSPEC_OK;
    PYSPEC_CHECK_ARG(xyz && xyz_out, "NULL position pointer");
    PYSPEC_CHECK_ARG(lbox > 0, "lbox must be positive");
    PYSPEC_CHECK_ARG(vxyz == nullptr || (los >= 0 && los < 3), "los must be 0, 1 or 2");
    const int bs = 256;
    prepare_positions_kernel<<<(unsigned)((np + bs - 1) / bs), bs, 0, as_stream(stream)>>>(
        xyz, dim_stride, vxyz, vdim_stride, los, rsd_factor, w, np, lbox, true, xyz_out, w_out);
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    return PYSPEC_OK;
}

extern "C" int pyspec_cast_positions(const double* xyz, int64_t dim_stride, const double* w, int64_t np,
                                     float* xyz_out, float* w_out, void* stream) {
    PYSPEC_CHECK_ARG(np >= 0, "np < 0");
    if (np == 0) return PYSPEC_OK;
    PYSPEC_CHECK_ARG(xyz && xyz_out, "NULL position pointer");
    const int bs = 256;
    prepare_positions_kernel<<<(unsigned)((np + bs - 1) / bs), bs, 0, as_stream(stream)>>>(
        xyz, dim_stride, nullptr, 0, 0, 0.0, w, np, 1.0, false, xyz_out, w_out);
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    return PYSPEC_OK;
}

extern "C" int pyspec_assign_pcs_interlaced(const float* xyz, const float* w, int64_t np, int ngrid,
                                            float kf_ks, float offset, float* grid, void* stream) {
    PYSPEC_CHECK_ARG(np >= 0, "np < 0");
    PYSPEC_CHECK_ARG(ngrid >= 4, "ngrid=%d too small", ngrid);
    if (np == 0) return PYSPEC_OK;
    PYSPEC_CHECK_ARG(xyz && grid, "NULL pointer");
    const int bs = 128;
    assign_pcs_kernel<<<(unsigned)((np + bs - 1) / bs), bs, 0, as_stream(stream)>>>(xyz, w, np, ngrid, kf_ks,
                                                                                  offset, grid);
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    return PYSPEC_OK;
}

static int fcomb_launch(const float* grid, int ngrid, float cf, float* half, void* stream) {
    const int64_t l = ngrid / 2 + 1;
    const int64_t nt = l * l * l;
    const int bs = 128;
    fcomb_kernel<<<(unsigned)((nt + bs - 1) / bs), bs, 0, as_stream(stream)>>>(
        reinterpret_cast<const float2*>(grid), ngrid, cf, reinterpret_cast<float2*>(half));
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    return PYSPEC_OK;
}

extern "C" int pyspec_fcomb_periodic(const float* grid, int ngrid, double wsum, float* half, void* stream) {
    PYSPEC_CHECK_ARG(grid && half, "NULL pointer");
    PYSPEC_CHECK_ARG(ngrid >= 2 && ngrid % 2 == 0, "ngrid=%d must be even", ngrid);
    PYSPEC_CHECK_ARG(wsum != 0.0, "sum of weights is zero");
    // estimator.f:615: cf = 1/(6^3 * 4 * N), single precision
    return fcomb_launch(grid, ngrid, (float)(1.0 / (216.0 * 4.0 * (double)(float)wsum)), half, stream);
}

extern "C" int pyspec_fcomb_survey(const float* grid, int ngrid, float* half, void* stream) {
    PYSPEC_CHECK_ARG(grid && half, "NULL pointer");
    PYSPEC_CHECK_ARG(ngrid >= 2 && ngrid % 2 == 0, "ngrid=%d must be even", ngrid);
    // estimator.f:686: cf = 1/(6^3 * 4), the FKP normalisation is applied later
    return fcomb_launch(grid, ngrid, (float)(1.0 / (216.0 * 4.0)), half, stream);
}

// out = a - alpha * b over n complex64 values (the FKP field F = n_g - alpha n_r
// in Fourier space, pyspectrum.py:126)
__global__ void axpy_kernel(const float2* __restrict__ a, const float2* __restrict__ b, double alpha, int64_t n,
                            float2* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 x = a[i], y = b[i];
    const float al = (float)alpha;        // numpy: complex64 field times a Python float
    out[i] = make_float2(__fsub_rn(x.x, __fmul_rn(al, y.x)), __fsub_rn(x.y, __fmul_rn(al, y.y)));
}

extern "C" int pyspec_combine_fields(const float* a, const float* b, double alpha, int64_t n, float* out,
                                     void* stream) {
    PYSPEC_CHECK_ARG(a && b && out, "NULL pointer");
    PYSPEC_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return PYSPEC_OK;
    const int bs = 256;
    axpy_kernel<<<(unsigned)((n + bs - 1) / bs), bs, 0, as_stream(stream)>>>(
        reinterpret_cast<const float2*>(a), reinterpret_cast<const float2*>(b), alpha, n,
        reinterpret_cast<float2*>(out));
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    return PYSPEC_OK;
}

extern "C" int pyspec_reflect_delta(const float* half, int ngrid, float* full, void* stream) {
    PYSPEC_CHECK_ARG(half && full, "NULL pointer");
    PYSPEC_CHECK_ARG(ngrid >= 2 && ngrid % 2 == 0, "ngrid=%d must be even", ngrid);
    const int64_t nt = (int64_t)ngrid * ngrid * ngrid;
    reflect_kernel<<<(unsigned)((nt + 255) / 256), 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const float2*>(half), ngrid, reinterpret_cast<float2*>(full));
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    return PYSPEC_OK;
}

extern "C" int pyspec_half_from_full(const float* full, int ngrid, float* half, void* stream) {
    PYSPEC_CHECK_ARG(half && full, "NULL pointer");
    PYSPEC_CHECK_ARG(ngrid >= 2 && ngrid % 2 == 0, "ngrid=%d must be even", ngrid);
    const int64_t nt = (int64_t)(ngrid / 2 + 1) * ngrid * ngrid;
    half_from_full_kernel<<<(unsigned)((nt + 255) / 256), 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const float2*>(full), ngrid, reinterpret_cast<float2*>(half));
    PYSPEC_LAUNCH_CHECK();
    count_launch();
    return PYSPEC_OK;
}
