/*
 * oracle/cpu_tri.c -- all-core CPU triangle sums of the reference's
 * bispectrum loop.  TEST INFRASTRUCTURE and the timed CPU baseline only:
 * nothing in the product library links, loads or calls it.
 *
 * Restates pyspectrum.py:424-430: for every triangle t = (i, j, l),
 *   bsum[t] = sum_v F_i(v) F_j(v) F_l(v)
 * evaluated in float64 (the reference stores the shell fields as float64 and
 * sums with np.einsum).  The reference walks the voxels once per triangle;
 * here the voxels are cut into blocks that stay in the core's L1 cache, each
 * pair product F_i F_j of a block is formed once and reused by every l of
 * the pair, and the blocks are spread over the host cores.
 *
 * cpu_triangle_sums_f32: fields float32 (the values FFTW single precision
 *   produces), products and sums in float64.
 * cpu_triangle_sums_f64: fields float64; also returns sum_v |F_i F_j F_l|
 *   (the condition-number denominator of the accuracy checks).
 *
 * Determinism: the voxel range is split into NPART fixed parts, each summed
 * into its own float64 array, and the parts are added in order, so results
 * do not depend on the thread count or schedule.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <omp.h>

enum { BV = 128, NPART = 64 };

typedef struct {
    int npair;
    int *pi, *pj, *start;     /* pair shells and first entry of each pair */
    int *l, *t;               /* per entry (sorted by pair): column shell, triangle index */
} pairs_t;

static int cmp_key(const void *a, const void *b) {
    const int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return x < y ? -1 : x > y;
}

/* groups the triangles by the pair of their two largest shells */
static int make_pairs(const int32_t *tri, int ntri, int nshell, pairs_t *P) {
    int64_t *key = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ntri > 0 ? ntri : 1));
    P->pi = (int *)malloc(sizeof(int) * (size_t)(ntri + 1));
    P->pj = (int *)malloc(sizeof(int) * (size_t)(ntri + 1));
    P->start = (int *)malloc(sizeof(int) * (size_t)(ntri + 2));
    P->l = (int *)malloc(sizeof(int) * (size_t)(ntri + 1));
    P->t = (int *)malloc(sizeof(int) * (size_t)(ntri + 1));
    int m = 0;
    for (int t = 0; t < ntri; ++t) {
        int v[3] = {tri[t], tri[ntri + t], tri[2 * ntri + t]};
        if (v[0] < 0 || v[1] < 0 || v[2] < 0 || v[0] >= nshell || v[1] >= nshell || v[2] >= nshell) continue;
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2 - a; ++b)
                if (v[b] < v[b + 1]) { int s = v[b]; v[b] = v[b + 1]; v[b + 1] = s; }
        /* key: pair (v0, v1), then column v2, then triangle index */
        key[m++] = ((((int64_t)v[0] * 256 + v[1]) * 256 + v[2]) << 24) | t;
    }
    qsort(key, (size_t)m, sizeof(int64_t), cmp_key);
    P->npair = 0;
    int64_t last = -1;
    for (int e = 0; e < m; ++e) {
        const int64_t k = key[e] >> 24;
        const int t = (int)(key[e] & 0xffffff);
        const int64_t pk = k >> 8;
        if (pk != last) {
            P->pi[P->npair] = (int)(pk >> 8);
            P->pj[P->npair] = (int)(pk & 255);
            P->start[P->npair] = e;
            ++P->npair;
            last = pk;
        }
        P->l[e] = (int)(k & 255);
        P->t[e] = t;
    }
    P->start[P->npair] = m;
    free(key);
    return m;
}

static void free_pairs(pairs_t *P) {
    free(P->pi); free(P->pj); free(P->start); free(P->l); free(P->t);
}

/* acc[t] += sum over the block of prod * fb[l] for every entry of pair p;
 * four columns at a time share the loads of prod */
static void block_pair(const double *prod, const double *fb, const pairs_t *P, int p, double *acc) {
    int e = P->start[p];
    const int e1 = P->start[p + 1];
    for (; e + 4 <= e1; e += 4) {
        const double *a = fb + (size_t)P->l[e] * BV, *b = fb + (size_t)P->l[e + 1] * BV;
        const double *c = fb + (size_t)P->l[e + 2] * BV, *d = fb + (size_t)P->l[e + 3] * BV;
        double sa[4] = {0, 0, 0, 0}, sb[4] = {0, 0, 0, 0}, sc[4] = {0, 0, 0, 0}, sd[4] = {0, 0, 0, 0};
        for (int v = 0; v < BV; v += 4)
            for (int u = 0; u < 4; ++u) {
                const double x = prod[v + u];
                sa[u] += x * a[v + u];
                sb[u] += x * b[v + u];
                sc[u] += x * c[v + u];
                sd[u] += x * d[v + u];
            }
        acc[P->t[e]] += (sa[0] + sa[1]) + (sa[2] + sa[3]);
        acc[P->t[e + 1]] += (sb[0] + sb[1]) + (sb[2] + sb[3]);
        acc[P->t[e + 2]] += (sc[0] + sc[1]) + (sc[2] + sc[3]);
        acc[P->t[e + 3]] += (sd[0] + sd[1]) + (sd[2] + sd[3]);
    }
    for (; e < e1; ++e) {
        const double *a = fb + (size_t)P->l[e] * BV;
        double sa[4] = {0, 0, 0, 0};
        for (int v = 0; v < BV; v += 4)
            for (int u = 0; u < 4; ++u) sa[u] += prod[v + u] * a[v + u];
        acc[P->t[e]] += (sa[0] + sa[1]) + (sa[2] + sa[3]);
    }
}

static void sums(const void *F, int is64, int64_t nvox, int nshell, const int32_t *tri, int ntri, double *bsum,
                 double *absum, int nthreads) {
    if (nthreads > 0) omp_set_num_threads(nthreads);
    pairs_t P;
    make_pairs(tri, ntri, nshell, &P);
    const int64_t nblk = (nvox + BV - 1) / BV;
    double *part = (double *)calloc((size_t)NPART * (size_t)ntri * (absum ? 2 : 1), sizeof(double));
#pragma omp parallel
    {
        double *fb = (double *)malloc(sizeof(double) * (size_t)nshell * BV);
        double *fa = absum ? (double *)malloc(sizeof(double) * (size_t)nshell * BV) : NULL;
        double *prod = (double *)malloc(sizeof(double) * BV);
        double *pabs = (double *)malloc(sizeof(double) * BV);
#pragma omp for schedule(dynamic, 1)
        for (int k = 0; k < NPART; ++k) {
            double *acc = part + (size_t)k * ntri;
            double *aacc = absum ? part + (size_t)(NPART + k) * ntri : NULL;
            for (int64_t b = nblk * k / NPART; b < nblk * (k + 1) / NPART; ++b) {
                const int64_t v0 = b * BV;
                const int nv = (int)(nvox - v0 < BV ? nvox - v0 : BV);
                for (int s = 0; s < nshell; ++s) {
                    double *dst = fb + (size_t)s * BV;
                    if (is64) {
                        const double *src = (const double *)F + (size_t)s * nvox + v0;
                        for (int v = 0; v < nv; ++v) dst[v] = src[v];
                    } else {
                        const float *src = (const float *)F + (size_t)s * nvox + v0;
                        for (int v = 0; v < nv; ++v) dst[v] = (double)src[v];
                    }
                    for (int v = nv; v < BV; ++v) dst[v] = 0.0;
                    if (fa)
                        for (int v = 0; v < BV; ++v) fa[(size_t)s * BV + v] = fabs(dst[v]);
                }
                for (int p = 0; p < P.npair; ++p) {
                    const double *x = fb + (size_t)P.pi[p] * BV, *y = fb + (size_t)P.pj[p] * BV;
                    for (int v = 0; v < BV; ++v) prod[v] = x[v] * y[v];
                    block_pair(prod, fb, &P, p, acc);
                    if (fa) {
                        for (int v = 0; v < BV; ++v) pabs[v] = fabs(prod[v]);
                        block_pair(pabs, fa, &P, p, aacc);
                    }
                }
            }
        }
        free(fb); free(fa); free(prod); free(pabs);
    }
    for (int t = 0; t < ntri; ++t) {
        double s = 0.0, a = 0.0;
        for (int k = 0; k < NPART; ++k) {
            s += part[(size_t)k * ntri + t];
            if (absum) a += part[(size_t)(NPART + k) * ntri + t];
        }
        bsum[t] = s;
        if (absum) absum[t] = a;
    }
    free(part);
    free_pairs(&P);
}

void cpu_triangle_sums_f32(const float *F, int64_t nvox, int nshell, const int32_t *tri, int ntri, double *bsum,
                           int nthreads) {
    sums(F, 0, nvox, nshell, tri, ntri, bsum, NULL, nthreads);
}

void cpu_triangle_sums_f64(const double *F, int64_t nvox, int nshell, const int32_t *tri, int ntri, double *bsum,
                           double *absum, int nthreads) {
    sums(F, 1, nvox, nshell, tri, ntri, bsum, absum, nthreads);
}
