/*
 * oracle/assign_pcs.c -- CPU restatement of the reference's particle-to-mesh
 * assignment, used ONLY as a test oracle and as the timed CPU baseline.
 * Nothing in the product library links, loads or calls this file.
 *
 * Restates pyspectrum/estimator.f:284-512 (subroutine assign_quad) for the
 * density mode ia=ib=ic=id=0 (estimator.f:292-293), the only mode the
 * periodic-box path uses (called from pyspectrum/pyspectrum.py:951).
 *
 * Arithmetic that decides WHICH cells a particle touches is done exactly as
 * the Fortran does it, in IEEE single precision with no fused multiply-add
 * (build with -ffp-contract=off):
 *   rx  = kf_ks*r + 1 + offset            (estimator.f:302)
 *   tx  = rx + 0.5                         (estimator.f:305)
 *   ixm1 = int(rx), hx = rx - ixm1          (estimator.f:308,314)
 *   weights (1-h)^3, 4+(3h-6)h^2, 6-rest, h^3 (estimator.f:316-320)
 * The 4 cells per axis are the 0-based cells m-2, m-1, m, m+1 (mod N) where
 * m = int(rx) (standard grid, real slots) or m = int(tx) (grid shifted by half
 * a cell, imaginary slots) -- estimator.f:311-313,322-324,347-350,359-362.
 * The Fortran accumulates in single precision; this oracle accumulates in
 * double (an FP64 oracle for the sums, bit-faithful for the cell indices and
 * per-particle weights).
 *
 * Grid layout: complex grid g[z][y][x] (x fastest) stored as interleaved
 * (re, im) doubles, i.e. exactly the Fortran array dtl(2*N, N, N) in column
 * order with re = standard grid, im = interlaced grid.
 */
#include <stdint.h>
#include <math.h>

static inline int wrap(int c, int n) {
    c %= n;
    return c < 0 ? c + n : c;
}

static inline void pcs_weights(float h, float out[4]) {
    /* estimator.f:316-320, same evaluation order */
    float h2 = h * h;
    float om = 1.0f - h;
    float wm2 = (om * om) * om;
    float wm1 = 4.0f + (3.0f * h - 6.0f) * h2;
    float wp2 = h2 * h;
    float wp1 = ((6.0f - wm2) - wm1) - wp2;
    out[0] = wm2; out[1] = wm1; out[2] = wp1; out[3] = wp2;
}

/* r: positions as 3 x np, column-major like the Fortran r(3,Np): r[3*i+d]. */
void oracle_assign_quad(const float *r, const float *w, int64_t np, int ngrid,
                        float kf_ks, float offset, double *grid)
{
    const int n = ngrid;
    for (int64_t i = 0; i < np; ++i) {
        float we = w ? w[i] : 1.0f;
        float rr[3], tt[3];
        int m[3], q[3];
        float wr[3][4], wt[3][4];
        for (int d = 0; d < 3; ++d) {
            float prod = kf_ks * r[3 * i + d];
            float a = prod + 1.0f;
            rr[d] = a + offset;
            tt[d] = rr[d] + 0.5f;
            m[d] = (int)rr[d];
            q[d] = (int)tt[d];
            pcs_weights(rr[d] - (float)m[d], wr[d]);
            pcs_weights(tt[d] - (float)q[d], wt[d]);
        }
        for (int s = 0; s < 2; ++s) {
            const int *base = s == 0 ? m : q;
            float (*wt3)[4] = s == 0 ? wr : wt;
            for (int cz = 0; cz < 4; ++cz) {
                int z = wrap(base[2] - 2 + cz, n);
                for (int cy = 0; cy < 4; ++cy) {
                    int y = wrap(base[1] - 2 + cy, n);
                    for (int cx = 0; cx < 4; ++cx) {
                        int x = wrap(base[0] - 2 + cx, n);
                        /* estimator.f:380: hx*hy*hz*we, left to right */
                        float v = ((wt3[0][cx] * wt3[1][cy]) * wt3[2][cz]) * we;
                        int64_t idx = (((int64_t)z * n + y) * n + x) * 2 + s;
                        grid[idx] += (double)v;
                    }
                }
            }
        }
    }
}
