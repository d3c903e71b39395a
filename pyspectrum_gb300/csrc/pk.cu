// Power spectrum: monopole in k_f-wide bins (pyspectrum.py:691-716) and the
// redshift-space multipoles / P(k, mu) of estimator.f:155-264.
//
// Each CTA bins one z-plane into shared-memory histograms (float32 within the
// plane) and adds them to float64 global bins; a finalize kernel forms the
// averages.
#include "common.cuh"
#include "shells.cuh"

namespace pyspec {

__device__ __forceinline__ int foldi(int i, int n) { return i <= n - i ? i : n - i; }

// Each thread takes runs of kPkRun consecutive x of one row: along a row |k|
// (and, mostly, mu) changes slowly, so the thread sums its modes of the same
// bin in float32 registers (at most kPkRun terms) and adds each finished run
// to the float64 shared histogram once, instead of one float64 atomic per mode
// and quantity (float64 arithmetic runs at a small fraction of the float32
// rate on this GPU).
constexpr int kPkRun = 12;

// Monopole on the reflected grid, summed over the half grid: planes x = 0 and
// x = N/2 count once, others twice (k and -k); the seven Nyquist corners use
// the real part only (pyspectrum.py:1149-1156).
__global__ void pk_mono_kernel(const float2* __restrict__ half, int n, double kf, double* __restrict__ acc) {
    extern __shared__ double smd[];
    const int nb = n / 2, nh = n / 2 + 1, hg = n / 2;
    double* ks = smd;
    double* ps = smd + nb;
    unsigned* cnt = reinterpret_cast<unsigned*>(smd + 2 * nb);
    for (int i = threadIdx.x; i < nb; i += blockDim.x) { ks[i] = 0; ps[i] = 0; cnt[i] = 0; }
    __syncthreads();
    const int z = blockIdx.x;
    const int zf = foldi(z, n);
    const int nrun = (nh + kPkRun - 1) / kPkRun;
    for (int item = threadIdx.x; item < n * nrun; item += blockDim.x) {
        const int y = item / nrun, x0 = (item - y * nrun) * kPkRun, x1 = min(nh, x0 + kPkRun);
        const int yf = foldi(y, n);
        const float2* row = half + ((int64_t)z * n + y) * nh;
        int cb = -1;
        float rk_s = 0.0f, p_s = 0.0f;     // run sums (at most kPkRun terms), added to float64 per run
        unsigned c_s = 0;
        for (int x = x0; x < x1; ++x) {
            const int64_t d2 = (int64_t)x * x + (int64_t)yf * yf + (int64_t)zf * zf;
            const int b = shell_of(d2, 1);
            if (b < 1 || b > nb) continue;
            if (b != cb) {
                if (cb >= 1) {
                    atomicAdd(&ks[cb - 1], (double)rk_s * kf);
                    atomicAdd(&ps[cb - 1], (double)p_s);
                    atomicAdd(&cnt[cb - 1], c_s);
                }
                cb = b;
                rk_s = p_s = 0.0f;
                c_s = 0;
            }
            const float2 v = row[x];
            const bool corner = (x == 0 || x == hg) && (y == 0 || y == hg) && (z == 0 || z == hg);
            const float p = corner ? v.x * v.x : v.x * v.x + v.y * v.y;
            const unsigned wgt = (x == 0 || x == hg) ? 1u : 2u;
            rk_s += (float)wgt * sqrtf((float)d2);
            p_s += (float)wgt * p;
            c_s += wgt;
        }
        if (cb >= 1) {
            atomicAdd(&ks[cb - 1], (double)rk_s * kf);
            atomicAdd(&ps[cb - 1], (double)p_s);
            atomicAdd(&cnt[cb - 1], c_s);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        if (cnt[i] == 0) continue;
        atomicAdd(&acc[i], ks[i]);
        atomicAdd(&acc[nb + i], ps[i]);
        atomicAdd(&acc[2 * nb + i], (double)cnt[i]);
    }
}

__global__ void pk_mono_finalize(const double* __restrict__ acc, int nb, double kf, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const double c = acc[2 * nb + i];
    const double tp = 2.0 * 3.14159265358979323846;
    out[i] = c > 0 ? acc[i] / c : 0.0;
    out[nb + i] = c > 0 ? acc[nb + i] / c / (kf * kf * kf) * (tp * tp * tp) : 0.0;
    out[2 * nb + i] = c;
}

// estimator.f:196-244.  Mode selection (imk) is exact integer arithmetic;
// mu follows the Fortran's single-precision expression order without fused
// multiply-add, and the mu bin is exactly int((abs(mu)+dble(mubin))/dble(mubin))
// in float64, so every mode lands in the Fortran's (k, mu) bin.  The summed
// quantities (the Legendre-weighted powers included) are float32 per mode and
// per run of kPkRun modes, float64 from there on: within 1e-6 of the
// Fortran's float64 sums.
struct RsdConst {
    float ct, st, cph, sph;   // cos/sin of thetaobs and phiobs (single precision)
    float kf;                 // tpi/Lbox, single precision
    float mubin;              // 1./real(Nmu)
};

__global__ void pk_rsd_kernel(const float2* __restrict__ half, int n, int nbin, int nmu, RsdConst c,
                              double* __restrict__ acc) {
    extern __shared__ double sm[];
    double* b_nk = sm;
    double* b_k = b_nk + nbin;
    double* b_p0 = b_k + nbin;
    double* b_p2 = b_p0 + nbin;
    double* b_p4 = b_p2 + nbin;
    double* m_n = b_p4 + nbin;
    double* m_k = m_n + nbin * nmu;
    double* m_mu = m_k + nbin * nmu;
    double* m_p = m_mu + nbin * nmu;
    const int tot = 5 * nbin + 4 * nbin * nmu;
    for (int i = threadIdx.x; i < tot; i += blockDim.x) sm[i] = 0;
    __syncthreads();
    const int nh = n / 2 + 1;
    const int iz = blockIdx.x;                         // 0-based z index
    auto sfreq = [n](int i) { return ((i + n / 2 - 1) % n) - n / 2 + 1; };   // estimator.f:198
    const int fz = sfreq(iz);
    const int icz = (n - iz) % n;
    const double mub = (double)c.mubin;
    const float inv_mubf = 1.0f / c.mubin;
    const int nrun = (n + kPkRun - 1) / kPkRun;
    for (int item = threadIdx.x; item < n * nrun; item += blockDim.x) {
        const int iy = item / nrun, x0 = (item - iy * nrun) * kPkRun, x1 = min(n, x0 + kPkRun);
        const int fy = sfreq(iy);
        const float2* row = half + ((int64_t)iz * n + iy) * nh;
        const float2* mrow = half + ((int64_t)icz * n + (n - iy) % n) * nh;    // conjugate row
        // float32 run sums of the current k bin (cb) and (k, mu) cell (cm)
        int cb = -1, cm = -1;
        float s_n = 0, s_k = 0, s_p0 = 0, s_p2 = 0, s_p4 = 0;
        float t_n = 0, t_k = 0, t_mu = 0, t_p = 0;
        auto flush_b = [&]() {
            if (cb < 0) return;
            atomicAdd(&b_nk[cb], (double)s_n);
            atomicAdd(&b_k[cb], (double)s_k);
            atomicAdd(&b_p0[cb], (double)s_p0);
            atomicAdd(&b_p2[cb], (double)s_p2);
            atomicAdd(&b_p4[cb], (double)s_p4);
        };
        auto flush_m = [&]() {
            if (cm < 0) return;
            atomicAdd(&m_n[cm], (double)t_n);
            atomicAdd(&m_k[cm], (double)t_k);
            atomicAdd(&m_mu[cm], (double)t_mu);
            atomicAdd(&m_p[cm], (double)t_p);
        };
        for (int ix = x0; ix < x1; ++ix) {
            const int fx = sfreq(ix);
            const int64_t d2 = (int64_t)fx * fx + (int64_t)fy * fy + (int64_t)fz * fz;
            const int imk = shell_of(d2, 1);
            if (imk > nbin || imk == 0) continue;
            const float rk = __fsqrt_rn((float)d2);
            const float cot1 = __fdiv_rn((float)fz, rk);
            const float sit1 = __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(cot1, cot1)));
            float cc = 0.0f;
            if (sit1 > 0.0f) {
                const float rs = __fmul_rn(rk, sit1);
                const float cp = __fdiv_rn((float)fx, rs);
                const float sp = __fdiv_rn((float)fy, rs);
                cc = __fadd_rn(__fmul_rn(c.sph, sp), __fmul_rn(c.cph, cp));
            }
            // mu: the single-precision expression of estimator.f:218
            const float muf = __fadd_rn(__fmul_rn(c.ct, cot1), __fmul_rn(__fmul_rn(c.st, sit1), cc));
            // imu = int((abs(mu) + dble(mubin)) / dble(mubin)) in float64 (estimator.f:219).  The
            // float32 quotient is within 2e-6 of it, so its integer part is the answer unless it
            // lies within 1e-4 of an integer; there the float64 division decides (float64 runs
            // at a small fraction of the float32 rate on this GPU)
            const float qf = (fabsf(muf) + c.mubin) * inv_mubf;
            int imu = (int)qf;
            const float ff = qf - (float)imu;
            if (ff < 1e-4f || ff > 1.0f - 1e-4f) imu = (int)((fabs((double)muf) + mub) / mub);
            const float mu2 = __fmul_rn(muf, muf);
            const float le2 = -0.5f + 1.5f * mu2;                            // estimator.f:221
            const float le4 = 0.375f - 3.75f * mu2 + 4.375f * mu2 * mu2;     // estimator.f:222
            const float2 ct = ix <= n / 2 ? row[ix] : mrow[(n - ix) % n];
            const float a = hypotf(ct.x, ct.y);               // cabs(ct), single precision
            const float pk = __fmul_rn(a, a);                 // pk = cabs(ct)**2 (estimator.f:230)
            const float kv = __fmul_rn(c.kf, rk);             // kf*rk
            const int b = imk - 1;
            if (b != cb) {
                flush_b();
                cb = b;
                s_n = s_k = s_p0 = s_p2 = s_p4 = 0.0f;
            }
            s_n += 1.0f;
            s_k += kv;
            s_p0 += pk;
            s_p2 += pk * 5.0f * le2;
            s_p4 += pk * 9.0f * le4;
            if (imu <= nmu && imu > 0) {
                const int m = b * nmu + imu - 1;
                if (m != cm) {
                    flush_m();
                    cm = m;
                    t_n = t_k = t_mu = t_p = 0.0f;
                }
                t_n += 1.0f;
                t_k += kv;
                t_mu += fabsf(muf);
                t_p += pk;
            }
        }
        flush_b();
        flush_m();
    }
    __syncthreads();
    for (int i = threadIdx.x; i < tot; i += blockDim.x)
        if (sm[i] != 0.0) atomicAdd(&acc[i], sm[i]);
}

__global__ void pk_rsd_finalize(const double* __restrict__ acc, int nbin, int nmu, float kf, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double kf3 = (double)((kf * kf) * kf);    // dble(kf**3), single-precision power
    // acc layout: nk, k, p0, p2, p4 [nbin]; then n, k, mu, p [nbin*nmu]
    // out layout: k, p0, p2, p4, nk [nbin]; then km, mk, pkm, nkm [nbin*nmu]
    if (i < nbin) {
        const double c = acc[i];
        const bool ok = c > 0;
        out[i] = ok ? acc[nbin + i] / c : 0.0;
        out[nbin + i] = ok ? acc[2 * nbin + i] / c / kf3 : 0.0;
        out[2 * nbin + i] = ok ? acc[3 * nbin + i] / c / kf3 : 0.0;
        out[3 * nbin + i] = ok ? acc[4 * nbin + i] / c / kf3 : 0.0;
        out[4 * nbin + i] = c;
    }
    if (i < nbin * nmu) {
        const double* a = acc + 5 * nbin;
        double* o = out + 5 * nbin;
        const int M = nbin * nmu;
        const double c = a[i];
        const bool ok = c > 0;
        o[i] = ok ? a[M + i] / c : 0.0;
        o[M + i] = ok ? a[2 * M + i] / c : 0.0;
        o[2 * M + i] = ok ? a[3 * M + i] / c / kf3 : 0.0;
        o[3 * M + i] = c;
    }
}

// pyspectrum.py:545-611 (_Pk_periodic_rsd, code='python'): the numpy binning
// over a FULL grid, in float64 with the reference's operation order (no fused
// multiply-add): irk = int(Nbins*rk/k_Nyq + 0.5), mu from the folded (non-
// negative) components, imu = ceil(mu/dmu).  Modes with imu outside
// [1, Nmu] count in Nk but add to neither the (k, mu) table nor P2/P4.
struct RsdPyConst {
    double kf, nyq, dmu;
    double ct, st, cph, sph;   // cos/sin of the observer's theta and phi (float64)
};

__global__ void pk_rsd_python_kernel(const float2* __restrict__ full, int n, int nbin, int nmu, RsdPyConst c,
                                     double* __restrict__ acc) {
    extern __shared__ double sm[];
    double* b_nk = sm;
    double* b_k = b_nk + nbin;
    double* b_p0 = b_k + nbin;
    double* b_p2 = b_p0 + nbin;
    double* b_p4 = b_p2 + nbin;
    double* m_n = b_p4 + nbin;
    double* m_k = m_n + nbin * nmu;
    double* m_mu = m_k + nbin * nmu;
    double* m_p = m_mu + nbin * nmu;
    const int tot = 5 * nbin + 4 * nbin * nmu;
    for (int i = threadIdx.x; i < tot; i += blockDim.x) sm[i] = 0;
    __syncthreads();
    const int z = blockIdx.x;
    const int az = foldi(z, n);
    const double rkz = __dmul_rn(c.kf, (double)az);
    for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
        const int y = i / n, x = i - y * n;
        const int ax = foldi(x, n), ay = foldi(y, n);
        const int64_t d2 = (int64_t)ax * ax + (int64_t)ay * ay + (int64_t)az * az;
        const double rk = __dmul_rn(c.kf, __dsqrt_rn((double)d2));
        const int irk = (int)__dadd_rn(__ddiv_rn(__dmul_rn((double)nbin, rk), c.nyq), 0.5);
        if (irk < 1 || irk > nbin) continue;
        const double cos_t = __ddiv_rn(rkz, rk);
        const double sin_t = __dsqrt_rn(__dsub_rn(1.0, __dmul_rn(cos_t, cos_t)));
        double cc = 0.0;
        if (sin_t > 0.0) {
            const double den = __dmul_rn(rk, sin_t);
            const double cp = __ddiv_rn(__dmul_rn(c.kf, (double)ax), den);
            const double sp = __ddiv_rn(__dmul_rn(c.kf, (double)ay), den);
            cc = __dadd_rn(__dmul_rn(c.sph, sp), __dmul_rn(c.cph, cp));
        }
        const double mu = __dadd_rn(__dmul_rn(c.ct, cos_t), __dmul_rn(__dmul_rn(c.st, sin_t), cc));
        const int imu = (int)ceil(__ddiv_rn(mu, c.dmu));
        const float2 v = full[((int64_t)z * n + y) * n + x];
        const float am = hypotf(v.x, v.y);
        const double p = (double)(am * am);
        const int b = irk - 1;
        atomicAdd(&b_nk[b], 1.0);
        atomicAdd(&b_k[b], rk);
        atomicAdd(&b_p0[b], p);
        if (imu >= 1 && imu <= nmu) {
            const double mu2 = __dmul_rn(mu, mu);
            const double le2 = __dadd_rn(-0.5, __dmul_rn(1.5, mu2));
            const double le4 = __dadd_rn(__dsub_rn(0.375, __dmul_rn(3.75, mu2)), __dmul_rn(4.375, __dmul_rn(mu2, mu2)));
            atomicAdd(&b_p2[b], __dmul_rn(p, le2));
            atomicAdd(&b_p4[b], __dmul_rn(p, le4));
            const int m = b * nmu + imu - 1;
            atomicAdd(&m_n[m], 1.0);
            atomicAdd(&m_k[m], rk);
            atomicAdd(&m_mu[m], mu);
            atomicAdd(&m_p[m], p);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < tot; i += blockDim.x)
        if (sm[i] != 0.0) atomicAdd(&acc[i], sm[i]);
}

// averages and the (2 pi)^3 / kf^3 factors of pyspectrum.py:588-609
__global__ void pk_rsd_python_finalize(const double* __restrict__ acc, int nbin, int nmu, double kf3,
                                       double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double tp = 2.0 * 3.14159265358979323846;
    const double norm = tp * tp * tp;
    if (i < nbin) {
        const double c = acc[i];
        const bool ok = c > 0;
        out[i] = ok ? acc[nbin + i] / c : 0.0;
        out[nbin + i] = ok ? acc[2 * nbin + i] / c / kf3 * norm : 0.0;
        out[2 * nbin + i] = ok ? acc[3 * nbin + i] / c / kf3 * 5.0 * norm : 0.0;
        out[3 * nbin + i] = ok ? acc[4 * nbin + i] / c / kf3 * 9.0 * norm : 0.0;
        out[4 * nbin + i] = c;
    }
    if (i < nbin * nmu) {
        const double* a = acc + 5 * nbin;
        double* o = out + 5 * nbin;
        const int M = nbin * nmu;
        const double c = a[i];
        const bool ok = c > 0;
        o[i] = ok ? a[M + i] / c : 0.0;
        o[M + i] = ok ? a[2 * M + i] / c : 0.0;
        o[2 * M + i] = ok ? a[3 * M + i] / c / kf3 * norm : 0.0;
        o[3 * M + i] = c;
    }
}

}  // namespace pyspec

using namespace pyspec;

// Both entry points accumulate into the second half of the caller's `out`
// buffer (zeroed here) and write the finished arrays into the first half, so
// they need no other memory.

extern "C" int pyspec_pk_monopole(const float* half, int ngrid, double lbox, double* out, void* stream) {
    PYSPEC_CHECK_ARG(half && out, "NULL pointer");
    PYSPEC_CHECK_ARG(ngrid >= 4 && ngrid % 2 == 0, "ngrid=%d must be even", ngrid);
    PYSPEC_CHECK_ARG(lbox > 0, "lbox must be positive");
    cudaStream_t st = as_stream(stream);
    const int nb = ngrid / 2;
    // out holds 3*nb results followed by 3*nb accumulators (6*nb doubles)
    double* acc = out + 3 * nb;
    PYSPEC_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * 3 * nb, st));
    const double kf = 2.0 * 3.14159265358979323846 / lbox;
    const size_t sm = sizeof(double) * 3 * nb;
    PYSPEC_TRY(allow_smem((const void*)pk_mono_kernel, sm));
    pk_mono_kernel<<<ngrid, 256, sm, st>>>(reinterpret_cast<const float2*>(half), ngrid, kf, acc);
    PYSPEC_LAUNCH_CHECK();
    pk_mono_finalize<<<(nb + 127) / 128, 128, 0, st>>>(acc, nb, kf, out);
    PYSPEC_LAUNCH_CHECK();
    count_launch(2);
    return PYSPEC_OK;
}

extern "C" int pyspec_pk_pbox_rsd(const float* half, int ngrid, int irsd, int lbox, int nbin, int nmu,
                                  double* out, void* stream) {
    PYSPEC_CHECK_ARG(half && out, "NULL pointer");
    PYSPEC_CHECK_ARG(ngrid >= 4 && ngrid % 2 == 0, "ngrid=%d must be even", ngrid);
    PYSPEC_CHECK_ARG(irsd >= 0 && irsd <= 2, "irsd must be 0, 1 or 2");
    PYSPEC_CHECK_ARG(nbin == ngrid / 2, "nbin must equal ngrid/2");
    PYSPEC_CHECK_ARG(nmu >= 1 && lbox > 0, "bad nmu or lbox");
    const size_t tot = 5 * (size_t)nbin + 4 * (size_t)nbin * nmu;
    const size_t sm = sizeof(double) * tot;
    PYSPEC_CHECK_ARG(sm <= 200 * 1024, "nbin*nmu too large for one CTA's histogram");
    cudaStream_t st = as_stream(stream);
    // out holds the results followed by the accumulators (2*tot doubles)
    double* acc = out + tot;
    PYSPEC_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * tot, st));
    // estimator.f:164-181 in single precision
    const float pi = 3.141592654f;
    const float half_pi = 0.5f * pi;
    const float theta = irsd == 2 ? 0.0f : half_pi;
    const float phi = irsd == 1 ? half_pi : 0.0f;
    RsdConst c;
    c.ct = (float)cos((double)theta);
    c.st = (float)sin((double)theta);
    c.cph = (float)cos((double)phi);
    c.sph = (float)sin((double)phi);
    c.kf = (2.0f * pi) / (float)lbox;
    c.mubin = 1.0f / (float)nmu;
    PYSPEC_TRY(allow_smem((const void*)pk_rsd_kernel, sm));
    pk_rsd_kernel<<<ngrid, 256, sm, st>>>(reinterpret_cast<const float2*>(half), ngrid, nbin, nmu, c, acc);
    PYSPEC_LAUNCH_CHECK();
    const int m = nbin * nmu > nbin ? nbin * nmu : nbin;
    pk_rsd_finalize<<<(m + 127) / 128, 128, 0, st>>>(acc, nbin, nmu, c.kf, out);
    PYSPEC_LAUNCH_CHECK();
    count_launch(2);
    return PYSPEC_OK;
}

extern "C" int pyspec_pk_rsd_python(const float* full, int ngrid, int irsd, double lbox, int nmu, double* out,
                                    void* stream) {
    PYSPEC_CHECK_ARG(full && out, "NULL pointer");
    PYSPEC_CHECK_ARG(ngrid >= 4 && ngrid % 2 == 0, "ngrid=%d must be even", ngrid);
    PYSPEC_CHECK_ARG(irsd >= 0 && irsd <= 2, "irsd must be 0, 1 or 2");
    PYSPEC_CHECK_ARG(nmu >= 1, "bad nmu");
    const int nbin = ngrid / 2;
    const size_t tot = 5 * (size_t)nbin + 4 * (size_t)nbin * nmu;
    const size_t sm = sizeof(double) * tot;
    PYSPEC_CHECK_ARG(sm <= 200 * 1024, "nbin*nmu too large for one CTA's histogram");
    cudaStream_t st = as_stream(stream);
    double* acc = out + tot;
    PYSPEC_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * tot, st));
    // pyspectrum.py:551-567: kf = 1 without a box size
    const double pi = 3.14159265358979323846;
    RsdPyConst c;
    c.kf = lbox > 0 ? 2.0 * pi / lbox : 1.0;
    c.nyq = c.kf * (double)ngrid / 2.0;
    c.dmu = 1.0 / (double)nmu;
    const double theta = irsd == 2 ? 0.0 : 0.5 * pi;
    const double phi = irsd == 1 ? 0.5 * pi : 0.0;
    c.ct = cos(theta);
    c.st = sin(theta);
    c.cph = cos(phi);
    c.sph = sin(phi);
    PYSPEC_TRY(allow_smem((const void*)pk_rsd_python_kernel, sm));
    pk_rsd_python_kernel<<<ngrid, 256, sm, st>>>(reinterpret_cast<const float2*>(full), ngrid, nbin, nmu, c, acc);
    PYSPEC_LAUNCH_CHECK();
    const int m = nbin * nmu > nbin ? nbin * nmu : nbin;
    pk_rsd_python_finalize<<<(m + 127) / 128, 128, 0, st>>>(acc, nbin, nmu, c.kf * c.kf * c.kf, out);
    PYSPEC_LAUNCH_CHECK();
    count_launch(2);
    return PYSPEC_OK;
}
