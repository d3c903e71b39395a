/*
 * pyspec_gpu.h -- C ABI of libpyspec_gb300.so, the GB300 (sm_103a) kernels of
 * the periodic-box power-spectrum / bispectrum estimator.
 *
 * This ABI replaces the reference's f2py extension ``estimator``
 * (pyspectrum/estimator.f, imported as ``fEstimate`` at pyspectrum.py:8) and
 * its FFTW calls (pyfftw.builders at pyspectrum.py:397,1073; sfftw_* at
 * estimator.f:69,275).  Each entry point names the reference routine it stands
 * in for.
 *
 * Conventions
 *  - All array arguments are DEVICE pointers owned by the caller, except where
 *    a comment says "host".  Nothing here allocates device memory; routines
 *    that need scratch take (workspace, ws_bytes) and have a *_workspace()
 *    size query.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *    stream).  Every call only enqueues work; no call synchronises the host.
 *  - Grids are stored [z][y][x] with x fastest.  This is the memory order of
 *    the reference's Fortran arrays dtl(x, y, z); a numpy array indexed
 *    [x, y, z] has the same bytes when it is Fortran-ordered.
 *  - Complex values are interleaved (re, im) float32 pairs ("c64").
 *  - A "half grid" holds x in [0, N/2] (N/2+1 values per row), y and z in [0, N).
 *  - Shells are numbered j = jmin..nmax as in the reference (j = 0 holds k = 0).
 *    Shell index of mode k: j = int(|k|/step + 0.5) (pyspectrum.py:373-378),
 *    evaluated exactly in integer arithmetic.
 *  - Return value: 0 on success, a negative PYSPEC_E_* code on failure;
 *    pyspec_last_error() returns the message of the calling thread's last
 *    failure.
 */
#ifndef PYSPEC_GPU_H
#define PYSPEC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PYSPEC_OK 0
#define PYSPEC_E_INVALID (-1)     /* bad argument (shape, size, pointer) */
#define PYSPEC_E_CUDA (-2)        /* a CUDA runtime call failed */
#define PYSPEC_E_UNSUPPORTED (-3) /* valid request this build does not handle */
#define PYSPEC_E_WORKSPACE (-4)   /* workspace smaller than the size query */

#define PYSPEC_ABI_VERSION 1

/* Contraction methods for pyspec_bk_contract. */
#define PYSPEC_CONTRACT_FP32 0    /* FP32 CUDA-core, FP32 per-thread, FP64 across blocks */
#define PYSPEC_CONTRACT_BF16X3 1  /* tcgen05 tensor cores, hi+lo BF16 split, 3 products */
/* tcgen05 tensor cores, 6 products: the BF16X3 sums (drained every 8 chunks)
 * plus a second pass over the voxels with each operand's third bf16 part
 * (x = hi + lo + res): sum P_res F_hi + P_hi F_res.  About twice the BF16X3
 * time, for errors near the FP32 form's. */
#define PYSPEC_CONTRACT_BF16X6 2
/* Flag OR-ed into a tensor-core method: plan the tensor-core tiles from runs of
 * each triangle's two largest shells even where a pair cover would need
 * fewer tiles (same sums; for the autotuner, which times both plans). */
#define PYSPEC_CONTRACT_RUN_PLAN 0x100
/* Flag OR-ed into a tensor-core method: drain the tensor-memory FP32
 * accumulators into the compensated sums every 8 chunks of 32 voxels instead
 * of every 32.  The split-BF16 error is set by the length of that FP32
 * accumulation, so this trades drain time for about 4x smaller errors. */
#define PYSPEC_CONTRACT_FINE_DRAIN 0x200
/* Flag OR-ed into a tensor-core method: keep 32-voxel chunks.  By default a
 * plan of 2 or 3 tiles in the wide MMA form whose buffers fit in shared
 * memory runs with 64-voxel chunks (one hand-over per 64 voxels; the A_lo
 * operand in shared memory); same sums, for the autotuner, which times both. */
#define PYSPEC_CONTRACT_KC32 0x400

int pyspec_abi_version(void);

/* Copies the calling thread's last error message into buf (NUL-terminated). */
int pyspec_last_error(char *buf, size_t len);

/* Number of the library's kernel launches enqueued by this process so far
 * (all threads).  Used to report how many native kernels a step ran. */
int64_t pyspec_launch_count(void);

/* ------------------------------------------------------------------------
 * Input preparation -- pyspectrum.py:931-945 (FFT_periodic) and util.py:54-75
 * (applyRSD).
 * xyz: float64, row d of the (3, np) position array at xyz + d*dim_stride.
 * vxyz: optional (NULL) float64 velocities, same layout; when given, the
 *   coordinate `los` (0,1,2) is shifted by rsd_factor * v_los and wrapped
 *   into [0, lbox) in float64 before clipping (applyRSD).
 * w: optional (NULL) float64 weights; w_out receives them as float32 (or 1).
 * Positions are clipped to [0, lbox*(1-1e-6)] in float64 and stored as a
 * float32 (3, np) array xyz_out (row d at xyz_out + d*np).
 * ---------------------------------------------------------------------- */
int pyspec_prepare_positions(const double *xyz, int64_t dim_stride, const double *vxyz,
                             int64_t vdim_stride, int los, double rsd_factor,
                             const double *w, int64_t np, double lbox,
                             float *xyz_out, float *w_out, void *stream);

/* ------------------------------------------------------------------------
 * Mass assignment -- replaces estimator.f:284-512 (assign_quad, density
 * mode ia=ib=ic=id=0, called at pyspectrum.py:951).
 * Adds each particle onto the complex grid `grid` (N^3 c64, [z][y][x]):
 * real part = PCS (4th-order) grid at r*kf_ks + 1 + offset, imaginary part =
 * the same grid shifted by half a cell (interlacing).  The caller zeroes the
 * grid first (pyspectrum.py:948).  xyz: float32 (3, np) rows; w may be NULL.
 * ---------------------------------------------------------------------- */
int pyspec_assign_pcs_interlaced(const float *xyz, const float *w, int64_t np, int ngrid,
                                 float kf_ks, float offset, float *grid, void *stream);

/* The same assignment (same per-particle arithmetic, same result up to the
 * order of the float additions) with shared-memory tile accumulation: the
 * particles are binned by the tile x tile x tile block of cells their stencil
 * starts in, each block is accumulated in shared memory with its 4-cell halo
 * and added to the grid once.  Pays off when many particles share cells.
 * tile: 4, 8 or 16 (ngrid >= tile + 4); np < 2^31.  Scratch: the caller's
 * workspace of pyspec_assign_tiled_workspace() bytes. */
size_t pyspec_assign_tiled_workspace(int64_t np, int ngrid, int tile);
int pyspec_assign_pcs_interlaced_tiled(const float *xyz, const float *w, int64_t np, int ngrid,
                                       float kf_ks, float offset, int tile, float *grid,
                                       void *workspace, size_t ws_bytes, void *stream);

/* ------------------------------------------------------------------------
 * 3D complex FFT, in place, unnormalised -- replaces the FFTW plan of
 * pyspectrum.py:1073-1075 (sign=+1, FFTW_BACKWARD, normalise_idft=False) and
 * estimator.f:266-282 (ffting).  sign=-1 gives FFTW_FORWARD.
 * ngrid must factor into 2, 3 and 5.
 * ---------------------------------------------------------------------- */
int pyspec_fft3d_c2c(float *grid, int ngrid, int sign, void *stream);

/* Radix-plan variants of the same transform (no counterpart in the
 * reference; for the autotuner).  pyspec_fft3d_variants returns the number
 * of variants of ngrid and writes, for each, its two-stage split (r1, r2)
 * into r1r2[2v], r1r2[2v+1] (up to cap variants; r1r2 may be NULL); (0, 0)
 * marks the shared-memory Stockham form, which exists for every ngrid.
 * pyspec_fft3d_c2c_variant runs variant `variant`; all variants compute the
 * same transform (to float32 rounding). */
int pyspec_fft3d_variants(int ngrid, int32_t *r1r2, int cap);
int pyspec_fft3d_c2c_variant(float *grid, int ngrid, int sign, int variant, void *stream);

/* ------------------------------------------------------------------------
 * Interlacing combine, window deconvolution, normalisation -- replaces
 * estimator.f:605-675 (fcomb_periodic, called at pyspectrum.py:957) together
 * with the half-grid slice at pyspectrum.py:959.  Reads the transformed grid
 * G (N^3 c64) and writes the half grid delta(k) (N/2+1 x N x N c64), with the
 * Fortran routine's write order reproduced at the self-conjugate planes.
 * wsum = sum of the weights.
 * ---------------------------------------------------------------------- */
int pyspec_fcomb_periodic(const float *grid, int ngrid, double wsum, float *half, void *stream);

/* ------------------------------------------------------------------------
 * Survey (FKP) path -- pyspectrum.py:731-826 (FFT_survey_mono) and
 * estimator.f:677-745 (fcomb_survey).
 * pyspec_cast_positions: float64 (3, np) positions (element stride 1, row
 *   stride dim_stride) and optional float64 weights -> float32, no clipping
 *   (survey positions are centred on the origin; the assignment's offset of
 *   N/2 cells moves them into the box).
 * pyspec_fcomb_survey: as pyspec_fcomb_periodic with cf = 1/(6^3 * 4) (no
 *   division by the weight sum; the FKP integrals normalise later).
 * pyspec_combine_fields: out = a - alpha * b over n complex64 values, in
 *   float32 without fused multiply-add (numpy's complex64 arithmetic), the
 *   FKP field delta_g - alpha delta_r of pyspectrum.py:126.
 * ---------------------------------------------------------------------- */
int pyspec_cast_positions(const double *xyz, int64_t dim_stride, const double *w, int64_t np,
                          float *xyz_out, float *w_out, void *stream);
int pyspec_fcomb_survey(const float *grid, int ngrid, float *half, void *stream);
int pyspec_combine_fields(const float *a, const float *b, double alpha, int64_t n, float *out,
                          void *stream);

/* ------------------------------------------------------------------------
 * reflect_delta -- pyspectrum.py:1134-1157: half grid -> full N^3 grid using
 * delta(-k) = conj(delta(k)); the seven Nyquist corners keep their real part.
 * half_from_full is the inverse used by _Bk_periodic when a caller passes a
 * full grid: x in (0, N/2) holds (delta(k) + conj(delta(-k)))/2, the x = 0 and
 * x = N/2 planes are copied (this reproduces Re(FFT) of the full grid).
 * ---------------------------------------------------------------------- */
int pyspec_reflect_delta(const float *half, int ngrid, float *full, void *stream);
int pyspec_half_from_full(const float *full, int ngrid, float *half, void *stream);

/* ------------------------------------------------------------------------
 * Mode counts per shell -- pyspectrum.py:380 (Nk), estimator.f:29-39.
 * nk: int64[nmax+1] (device), exact.
 * ---------------------------------------------------------------------- */
int pyspec_mode_counts(int ngrid, int step, int nmax, int64_t *nk, void *stream);

/* ------------------------------------------------------------------------
 * Shell fields -- pyspectrum.py:384-404 (the masked forward FFT per shell
 * and p0k).  For s = 0..nmax-jmin, shell j = jmin+s:
 *   fields[s*N^3 + v] = Re(FFT_forward(delta * [irk == j]))(v)  (float32)
 *   p0sum[s] = sum_v fields[s][v]^2                              (float64)
 * half: delta(k) half grid.  fields: float32 (nmax-jmin+1) x N^3.
 * ---------------------------------------------------------------------- */
size_t pyspec_shell_fields_workspace(int ngrid, int nshell);
int pyspec_shell_fields(const float *half, int ngrid, int step, int jmin, int nmax,
                        float *fields, double *p0sum, void *workspace, size_t ws_bytes,
                        void *stream);

/* ------------------------------------------------------------------------
 * Triangle contraction -- pyspectrum.py:415-437: for every triangle t,
 *   bsum[t] = sum_v fields[i_t][v] * fields[j_t][v] * fields[l_t][v]  (float64 out)
 * tri: int32 device array [3][ntri] of shell SLOTS (0-based rows of fields).
 * tri_host: the same list in host memory, from which both methods plan
 *   their tiles (plans are cached per list).  Required by
 *   PYSPEC_CONTRACT_BF16X3; with PYSPEC_CONTRACT_FP32 it may be NULL, which
 *   selects an unplanned (slower) CUDA-core kernel that reads tri directly.
 * method: PYSPEC_CONTRACT_FP32 (any nshell <= 128; a triangle with a slot
 *   outside [0, nshell) gets bsum = 0) or PYSPEC_CONTRACT_BF16X3 (nshell <= 64,
 *   fields 16-byte aligned, N^3 divisible by 4; returns PYSPEC_E_UNSUPPORTED
 *   otherwise).  After the stream has run a BF16X3 call, the int32 at
 *   workspace offset 0 is 0, or the code of a bounded wait that timed out.
 *   The planned FP32 kernel stages its voxels with bulk copies under the
 *   same bounded waits; if one times out, the triangles of the CTAs that
 *   met it get bsum = NaN.
 * The triangles of one list must be distinct (as unordered shell triples):
 *   a repeated triangle returns PYSPEC_E_INVALID with either planned method.
 * ---------------------------------------------------------------------- */
size_t pyspec_bk_contract_workspace(int ngrid, int nshell, int ntri, int method);
int pyspec_bk_contract(const float *fields, int ngrid, int nshell, const int32_t *tri,
                       const int32_t *tri_host, int ntri, int method, double *bsum,
                       void *workspace, size_t ws_bytes, void *stream);

/* ------------------------------------------------------------------------
 * Host-side check of the BF16X3 contraction plan of a triangle list (no GPU
 * needed; no counterpart in the reference).  Builds (or reuses) the plan
 * pyspec_bk_contract plans for tri_host and verifies that every triangle is
 * read at exactly one (pair row, column) cell whose three shells are the
 * triangle's, that each row's shells agree with the producer table, that
 * every row lies in its group's tiles and every column below its tile's N.
 * info (may be NULL) receives up to ninfo values: [0] CTA groups, [1] tiles
 * of group 0, [2] 1 if the rows are a pair cover (0: runs of the triangles'
 * two largest shells), [3] MMAs per 32 voxels summed over groups, [4] Kahan
 * slots of group 0, [5] 1 if group 0 uses the wide MMA form, [6] tensor-core
 * multiply-adds per voxel summed over groups (the executed work), [7] shared-
 * memory bank clashes between the producer threads that share load phases,
 * [8] voxels per chunk (64 or 32) the contraction runs with, [9] 1 if that
 * 64-voxel kernel has B-operand writer warps (plans of three tiles).
 * Returns 0; PYSPEC_E_INVALID / PYSPEC_E_UNSUPPORTED where the contraction
 * would; PYSPEC_E_INVALID with a message if the plan fails the check.
 * ---------------------------------------------------------------------- */
int pyspec_bk_plan_check(int nshell, const int32_t *tri_host, int ntri, int64_t *info, int ninfo);
/* The same for the plan that method flags `flags` (PYSPEC_CONTRACT_RUN_PLAN,
 * PYSPEC_CONTRACT_KC32 or both) select. */
int pyspec_bk_plan_check_flags(int nshell, const int32_t *tri_host, int ntri, int flags, int64_t *info,
                               int ninfo);

/* ------------------------------------------------------------------------
 * Triangle contraction without device allocation.  This entry point has no
 * counterpart in the reference.  It is for callers that cannot allocate
 * device memory where they run -- inside another framework's
 * foreign-function / custom-call hook that hands over only the operands, or
 * while a stream is being captured.  It computes what pyspec_bk_contract
 * computes with PYSPEC_CONTRACT_FP32 (same kernel, same sums), with its
 * scratch in a fixed device array of PYSPEC_NOALLOC_SCRATCH_BYTES that the
 * library holds on every GPU that loads it until the process exits.
 *  - Requests whose scratch would exceed that size (roughly ntri x 152 CTAs
 *    x 8 bytes of partial sums plus the tile tables) return PYSPEC_E_INVALID.
 *  - No call allocates device memory (it copies its tile tables from host
 *    memory into the array and clears the partial sums it uses).
 *  - All calls share the one array: calls whose work overlaps on the GPU race
 *    and must be ordered by the caller.
 *  - The first call on a device looks up the array's address with that
 *    device current, and the first call with a given triangle list builds
 *    its tile plan in page-locked host memory.  Neither may happen inside a
 *    stream capture: a call on a capturing stream returns PYSPEC_E_INVALID
 *    (and leaves the capture intact) unless an earlier call, outside any
 *    capture, used the same device and the same triangle list.
 * ---------------------------------------------------------------------- */
#define PYSPEC_NOALLOC_SCRATCH_BYTES (16u << 20)
int pyspec_bk_contract_noalloc(const float *fields, int ngrid, int nshell,
                               const int32_t *tri_host, int ntri, double *bsum, void *stream);

/* ------------------------------------------------------------------------
 * Triangle counts -- pyspectrum.py:962-1030 (_counts_Bk123) and
 * estimator.f:2-102 (bk_counts): counts[t] = round(sum_x I_i I_j I_l / N^3),
 * I_j = FFT of the shell-j indicator, evaluated in float64 and returned as
 * exact int64 (the number of closed k-triangles).  tri as for
 * pyspec_bk_contract but holding shell NUMBERS j (not slots).  nk receives
 * the mode counts (int64[nmax+1]).
 * ---------------------------------------------------------------------- */
size_t pyspec_bk_counts_workspace(int ngrid, int step, int jmin, int nmax);
int pyspec_bk_counts(int ngrid, int step, int jmin, int nmax, const int32_t *tri, int ntri,
                     int64_t *counts, int64_t *nk, void *workspace, size_t ws_bytes,
                     void *stream);

/* ------------------------------------------------------------------------
 * Bispectrum normalisation -- pyspectrum.py:423-437 and 341-355.
 * For triangle t with shells (i,j,l) = tri[.][t] (shell numbers):
 *   p_a   = p0sum[a-jmin] / N^3 / nk[a]                          (p0k, :404)
 *   b     = bsum[t] / (counts[t] * N^3)                            (:435)
 *   q     = b / (p_i p_j + p_j p_l + p_l p_i)                       (:436)
 *   cnt   = counts[t] / fac_t                                      (:437)
 * If apply_units != 0 the shot-noise and unit conversion of Bk_periodic
 * (:346-355) follow with nbar and kf.  out: float64 [7][ntri] =
 * {p0k1, p0k2, p0k3, b123, q123, counts, b123_sn}.  Triangles with a shell
 * outside [jmin, nmax] get zeros (p0sum holds nmax-jmin+1 values, nk nmax+1).
 * ---------------------------------------------------------------------- */
int pyspec_bk_normalize(const double *bsum, const int64_t *counts, const double *p0sum,
                        const int64_t *nk, const int32_t *tri, int ntri, int ngrid, int jmin,
                        int nmax, int apply_units, double nbar, double kf, double *out,
                        void *stream);

/* ------------------------------------------------------------------------
 * Power-spectrum monopole -- pyspectrum.py:691-716 (Pk_periodic) on the
 * reflected grid of `half`.  Bins i = 1..N/2 of width k_f.
 * out: float64 [6][N/2]; rows 0-2 receive {k, p0k (before the -1/nbar),
 * counts}, rows 3-5 are used as accumulators.
 * ---------------------------------------------------------------------- */
int pyspec_pk_monopole(const float *half, int ngrid, double lbox, double *out, void *stream);

/* ------------------------------------------------------------------------
 * Multipoles and P(k, mu) -- replaces estimator.f:155-264 (pk_pbox_rsd,
 * called at pyspectrum.py:634).  irsd: line of sight 0/1/2 = x/y/z; lbox is
 * the Fortran INTEGER box size; nbin must be N/2.
 * out: float64 = {k[nbin], p0[nbin], p2[nbin], p4[nbin], nk[nbin],
 *                 km[nbin][nmu], mk[nbin][nmu], pkm[nbin][nmu], nkm[nbin][nmu]}
 * ((k, mu) tables row-major in k), before the (2 pi)^3 factor of
 * pyspectrum.py:636-640.  `out` holds 2*(5*nbin + 4*nbin*nmu) doubles: the
 * results above, then the same number of doubles used as accumulators.  Mode and mu-bin selection reproduce the Fortran's
 * single-precision arithmetic exactly.
 * ---------------------------------------------------------------------- */
int pyspec_pk_pbox_rsd(const float *half, int ngrid, int irsd, int lbox, int nbin, int nmu,
                       double *out, void *stream);

/* ------------------------------------------------------------------------
 * P(k, mu) with the reference's numpy binning -- pyspectrum.py:545-611
 * (_Pk_periodic_rsd with code='python'), on a FULL grid delta(k) complex64
 * (N, N, N) [z][y][x]: Nbins = N/2 bins irk = int(Nbins*|k|/k_Nyq + 0.5),
 * mu from the folded components in float64, mu bins ceil(mu/dmu).
 * lbox <= 0 means no box size (kf = 1).  out: 2*tot doubles,
 * tot = 5*(N/2) + 4*(N/2)*nmu, results first, in the order
 * k, p0, p2, p4, nk [N/2]; k_kmu, mu_kmu, p_kmu, n_kmu [N/2][nmu],
 * with the (2 pi)^3 factor applied (no shot noise subtracted).
 * ---------------------------------------------------------------------- */
int pyspec_pk_rsd_python(const float *full, int ngrid, int irsd, double lbox, int nmu,
                         double *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PYSPEC_GPU_H */
