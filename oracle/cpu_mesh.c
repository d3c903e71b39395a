/*
 * oracle/cpu_mesh.c -- all-core CPU restatement of the grid stages of the
 * reference's periodic-box path.  TEST INFRASTRUCTURE and the timed CPU
 * baseline only: nothing in the product library links, loads or calls it.
 *
 * Restates, in IEEE single precision like the Fortran (build with
 * -ffp-contract=off so no multiply-add is fused):
 *   cpu_assign_pcs      estimator.f:284-512 (assign_quad, density mode), with
 *                       single-precision accumulation in particle order
 *   cpu_fcomb_periodic  estimator.f:605-675 (fcomb_periodic), in place, with
 *                       the Fortran's write order inside each orbit
 *   cpu_reflect         pyspectrum.py:1134-1157 (reflect_delta)
 *   cpu_shell_extract   pyspectrum.py:387-395 (tempK[irk == j] = delta[irk == j])
 *   cpu_real_part       pyspectrum.py:402-404 (Re(FFT), sum F^2 for p0k)
 *
 * Parallel decomposition (OpenMP), chosen so results do not depend on the
 * thread count:
 *   - assignment: each thread owns a slab of z planes and scans every
 *     particle in order, adding only the contributions that land in its
 *     slab, so every cell sees its particles in the serial order;
 *   - fcomb: Fortran iterations (ix, iy, iz) own disjoint 8-point orbits, so
 *     the iz loop is split across threads;
 *   - float64 sums are taken over fixed voxel ranges, added in range order.
 *
 * Grid layout: complex64 [z][y][x] (x fastest), interleaved (re, im) floats,
 * which is the Fortran array dtl(2N, N, N) / dcl(N, N, N) in column order.
 * Positions: Fortran r(3, np) order, r[3*i + d].
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <omp.h>

static inline int wrapi(int c, int n) {
    c %= n;
    return c < 0 ? c + n : c;
}

/* estimator.f:316-320: PCS weights of the 4 cells, same evaluation order */
static inline void pcs4(float h, float out[4]) {
    const float h2 = h * h;
    const float om = 1.0f - h;
    const float wm2 = (om * om) * om;
    const float wm1 = 4.0f + (3.0f * h - 6.0f) * h2;
    const float wp2 = h2 * h;
    out[0] = wm2;
    out[1] = wm1;
    out[2] = ((6.0f - wm2) - wm1) - wp2;
    out[3] = wp2;
}

void cpu_assign_pcs(const float *r, const float *w, int64_t np, int n, float kf_ks, float offset, float *grid,
                    int nthreads) {
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
    {
        const int nt = omp_get_num_threads(), id = omp_get_thread_num();
        const int z0 = (int)((int64_t)n * id / nt), z1 = (int)((int64_t)n * (id + 1) / nt);
        for (int64_t i = 0; i < np; ++i) {
            /* estimator.f:302-307 in single precision: r*kf + 1 + offset, + 0.5 */
            const float rz = (kf_ks * r[3 * i + 2] + 1.0f) + offset;
            const float tz = rz + 0.5f;
            const int mz = (int)rz, qz = (int)tz;
            int hit = 0;
            for (int c = 0; c < 4 && !hit; ++c) {
                const int a = wrapi(mz - 2 + c, n), b = wrapi(qz - 2 + c, n);
                hit = (a >= z0 && a < z1) || (b >= z0 && b < z1);
            }
            if (!hit) continue;
            const float we = w ? w[i] : 1.0f;
            float rr[3], tt[3], wr[3][4], wt[3][4];
            int m[3], q[3];
            for (int d = 0; d < 3; ++d) {
                rr[d] = (kf_ks * r[3 * i + d] + 1.0f) + offset;
                tt[d] = rr[d] + 0.5f;
                m[d] = (int)rr[d];
                q[d] = (int)tt[d];
                pcs4(rr[d] - (float)m[d], wr[d]);
                pcs4(tt[d] - (float)q[d], wt[d]);
            }
            for (int s = 0; s < 2; ++s) {        /* s = 0: real slots, 1: interlaced (imaginary) */
                const int *base = s ? q : m;
                float (*wk)[4] = s ? wt : wr;
                for (int cz = 0; cz < 4; ++cz) {
                    const int z = wrapi(base[2] - 2 + cz, n);
                    if (z < z0 || z >= z1) continue;
                    for (int cy = 0; cy < 4; ++cy) {
                        const int y = wrapi(base[1] - 2 + cy, n);
                        float *row = grid + ((int64_t)z * n + y) * n * 2;
                        for (int cx = 0; cx < 4; ++cx) {
                            const int x = wrapi(base[0] - 2 + cx, n);
                            /* estimator.f:380: hx*hy*hz*we, left to right */
                            row[2 * x + s] += ((wk[0][cx] * wk[1][cy]) * wk[2][cz]) * we;
                        }
                    }
                }
            }
        }
    }
}

/* complex helpers (single precision, as the Fortran COMPLEX arithmetic) */
typedef struct { float re, im; } c32;
static inline c32 cmul(c32 a, c32 b) {
    c32 r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static inline c32 conj32(c32 a) { c32 r = {a.re, -a.im}; return r; }

void cpu_fcomb_periodic(float *dcl_f, int n, float wsum, int nthreads) {
    if (nthreads > 0) omp_set_num_threads(nthreads);
    c32 *dcl = (c32 *)dcl_f;
    const int lnyq = n / 2 + 1;
    const float cf = 1.0f / (216.0f * 4.0f * wsum);           /* estimator.f:615 */
    const double tpiL = 6.283185307 / (double)n;              /* estimator.f:618 */
    const double piL = -tpiL / 2.0;
    /* the complex*16 recurrences xrec = recx**(ix-1) (estimator.f:620-623, 667),
     * replayed serially so every thread sees the Fortran's values */
    double rec_re[lnyq], rec_im[lnyq];
    float W[lnyq];
    {
        const double cr = cos(piL), ci = sin(piL);
        double xr = 1.0, xi = 0.0;
        for (int k = 0; k < lnyq; ++k) {
            rec_re[k] = xr;
            rec_im[k] = xi;
            const double nr = xr * cr - xi * ci, ni = xr * ci + xi * cr;
            xr = nr;
            xi = ni;
            const float rk = (float)(tpiL * (double)k);       /* estimator.f:631 */
            float wk = 1.0f;
            if (rk != 0.0f) {
                const float s = sinf(rk / 2.0f) / (rk / 2.0f);
                wk = (s * s) * (s * s);                      /* (sin(x)/x)**4 */
            }
            W[k] = wk;
        }
    }
#pragma omp parallel for schedule(static)
    for (int iz = 0; iz < lnyq; ++iz) {
        const int icz = (n - iz) % n;
        for (int iy = 0; iy < lnyq; ++iy) {
            const int icy = (n - iy) % n;
            for (int ix = 0; ix < lnyq; ++ix) {
                const int icx = (n - ix) % n;
                const float cfac = cf / ((W[ix] * W[iy]) * W[iz]);
                /* ci*xrec*yrec*zrec etc. in complex*16, rounded to COMPLEX */
                const double xr = rec_re[ix], xi = rec_im[ix], yr = rec_re[iy], yi = rec_im[iy];
                const double zr = rec_re[iz], zi = rec_im[iz];
                double ar = -xi, ai = xr;                        /* ci * xrec */
                const double pr = ar * yr - ai * yi, pi = ar * yi + ai * yr;   /* * yrec */
                const double qr = ar * yr + ai * yi, qi = -ar * yi + ai * yr;  /* * conj(yrec) */
                const c32 cma = {(float)(pr * zr - pi * zi), (float)(pr * zi + pi * zr)};
                const c32 cmb = {(float)(pr * zr + pi * zi), (float)(-pr * zi + pi * zr)};
                const c32 cmc = {(float)(qr * zr - qi * zi), (float)(qr * zi + qi * zr)};
                /* ci*xrec*conjg(yrec*zrec) */
                const double yzr = yr * zr - yi * zi, yzi = yr * zi + yi * zr;
                const c32 cmd = {(float)(ar * yzr + ai * yzi), (float)(-ar * yzi + ai * yzr)};
                const int xs[2] = {ix, icx}, ys[2] = {iy, icy}, zs[2] = {iz, icz};
                int64_t pos[8];
                c32 v[8];
                for (int k = 0; k < 8; ++k) {   /* (ix,iy,iz) (ix,iy,icz) (ix,icy,iz) (ix,icy,icz), then icx */
                    pos[k] = ((int64_t)zs[k & 1] * n + ys[(k >> 1) & 1]) * n + xs[k >> 2];
                    v[k] = dcl[pos[k]];
                }
                const c32 one = {1.0f, 0.0f};
                c32 c[4];
                const c32 cm[4] = {cma, cmb, cmc, cmd};
                for (int k = 0; k < 4; ++k) {     /* estimator.f:652-655 */
                    const c32 om = {one.re - cm[k].re, -cm[k].im}, op = {one.re + cm[k].re, cm[k].im};
                    const c32 a = cmul(v[k], om), b = cmul(conj32(v[7 - k]), op);
                    c[k].re = a.re + b.re;
                    c[k].im = a.im + b.im;
                }
                /* estimator.f:658-665, in order; aliased slots see the last write */
                for (int k = 0; k < 4; ++k) {
                    c32 val = {c[k].re * cfac, c[k].im * cfac};
                    dcl[pos[k]] = val;
                }
                dcl[pos[4]] = conj32(dcl[pos[3]]);
                dcl[pos[5]] = conj32(dcl[pos[2]]);
                dcl[pos[6]] = conj32(dcl[pos[1]]);
                dcl[pos[7]] = conj32(dcl[pos[0]]);
            }
        }
    }
}

/* pyspectrum.py:1134-1157: full[z][y][x] from the half grid half[z][y][0..n/2]
 * (delta(-k) = conj(delta(k)); the seven Nyquist corners keep their real part) */
void cpu_reflect(const float *half_f, int n, float *full_f, int nthreads) {
    if (nthreads > 0) omp_set_num_threads(nthreads);
    const c32 *half = (const c32 *)half_f;
    c32 *full = (c32 *)full_f;
    const int h = n / 2, nh = n / 2 + 1;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < n; ++z) {
        for (int y = 0; y < n; ++y) {
            c32 *row = full + ((int64_t)z * n + y) * n;
            const c32 *src = half + ((int64_t)z * n + y) * nh;
            const c32 *mir = half + ((int64_t)((n - z) % n) * n + (n - y) % n) * nh;
            for (int x = 0; x <= h; ++x) row[x] = src[x];
            for (int x = h + 1; x < n; ++x) row[x] = conj32(mir[n - x]);
            if ((z == 0 || z == h) && (y == 0 || y == h)) {
                for (int x = 0; x <= h; x += h)
                    if (x + y + z > 0) row[x].im = 0.0f;
            }
        }
    }
}

/* largest m with (2m-1)^2 step^2 <= 4 d2: the shell of a mode with
 * |k|^2 = d2, i.e. int(sqrt(d2)/step + 0.5) (pyspectrum.py:373-378) */
static inline int shell_of(int64_t d2, int step) {
    int m = (int)floor(sqrt((double)d2) / step + 0.5);
    const int64_t s2 = (int64_t)step * step;
    while (m > 0 && (int64_t)(2 * m - 1) * (2 * m - 1) * s2 > 4 * d2) --m;
    while ((int64_t)(2 * m + 1) * (2 * m + 1) * s2 <= 4 * d2) ++m;
    return m;
}

/* tempK = delta where irk == j, else 0 (full complex64 grids) */
void cpu_shell_extract(const float *full_f, int n, int step, int j, float *work_f, int nthreads) {
    if (nthreads > 0) omp_set_num_threads(nthreads);
    const c32 *full = (const c32 *)full_f;
    c32 *work = (c32 *)work_f;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < n; ++z) {
        const int64_t az = z < n - z ? z : n - z;
        for (int y = 0; y < n; ++y) {
            const int64_t ay = y < n - y ? y : n - y;
            const int64_t base = ((int64_t)z * n + y) * n;
            memset(work + base, 0, sizeof(c32) * (size_t)n);
            /* modes of shell j have 4|k|^2 < (2j + 1)^2 step^2 */
            const int64_t r2 = az * az + ay * ay;
            if (4 * r2 >= (int64_t)(2 * j + 1) * (2 * j + 1) * step * step) continue;
            for (int x = 0; x < n; ++x) {
                const int64_t ax = x < n - x ? x : n - x;
                if (shell_of(r2 + ax * ax, step) == j) work[base + x] = full[base + x];
            }
        }
    }
}

/* field[v] = Re(work[v]) as float32; returns sum of field^2 in float64
 * (per-thread partials added in thread order) */
double cpu_real_part(const float *work_f, int64_t nvox, float *field, int nthreads) {
    if (nthreads > 0) omp_set_num_threads(nthreads);
    enum { NPART = 64 };             /* fixed voxel ranges: the sum does not depend on the thread count */
    double part[NPART];
#pragma omp parallel for schedule(static)
    for (int k = 0; k < NPART; ++k) {
        const int64_t v0 = nvox * k / NPART, v1 = nvox * (k + 1) / NPART;
        double s = 0.0;
        for (int64_t v = v0; v < v1; ++v) {
            const float re = work_f[2 * v];
            field[v] = re;
            s += (double)re * (double)re;
        }
        part[k] = s;
    }
    double tot = 0.0;
    for (int k = 0; k < NPART; ++k) tot += part[k];
    return tot;
}
