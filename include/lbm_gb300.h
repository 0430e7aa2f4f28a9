/*
 * lbm_gb300 -- C ABI of the GB300 (sm_103a) dynamical-core hot path for the
 * PyLBM-Isca linear baroclinic model.
 *
 * Every entry point takes device pointers, plain sizes and a CUDA stream
 * (cudaStream_t passed as void*), launches asynchronously on that stream and
 * returns an int status (LBM_OK = 0).  No C++ exception crosses the ABI and
 * the library allocates no device memory: every buffer is owned by the
 * caller.  Arrays are C-contiguous; "complex" means interleaved (re, im)
 * pairs of the working precision; `prec` selects LBM_F64 (double) or
 * LBM_F32 (float) for every array marked (R).
 *
 * Index conventions follow the reference (pylbm_isca): latitudes north to
 * south, longitudes from 0 east, levels bottom-up (k = 0 is the lowest
 * layer), spectral coefficients indexed [m][n] with n >= m.
 *   M = nmax + 1; NS = M (M + 1) / 2 ("packed": rows (m, n), n = m..nmax,
 *   m-major, row index = m M - m (m - 1) / 2 + n - m).
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------- */
#define LBM_OK 0
#define LBM_ERR_ARG 1          /* bad size, null pointer or unsupported grid   */
#define LBM_ERR_LAUNCH 2       /* CUDA launch or runtime failure               */
#define LBM_ERR_SINGULAR 3     /* zero pivot in a factorisation                */
#define LBM_ERR_NONFINITE 4    /* non-finite prognostic value detected         */
#define LBM_ERR_SCRATCH 5      /* case larger than the static scratch area of
                                  lbm_stepper_run_noalloc                      */

/* ---- precisions ------------------------------------------------------------- */
#define LBM_F64 0
#define LBM_F32 1

/* Library version string. */
const char* lbm_version(void);

/* ============================================================================
 * Setup (always FP64)
 * ==========================================================================*/

/* Gauss-Legendre nodes and weights, north first, weights summing to 1.
 * Replaces numpy leggauss + sort + /2 at spectral.py:58-61.
 * mu[nlat], gw[nlat]. */
int lbm_gauss_legendre(int nlat, double* mu, double* gw, void* stream);

/* Fully normalised associated Legendre functions P[m][n][j] (no
 * Condon-Shortley phase, (1/2) int P^2 = 1) and H = (1 - mu^2) dP/dmu for
 * 0 <= m, n <= nmax (zero for n < m); replaces Spectral._build_legendre,
 * spectral.py:93-154.  pnm, hnm: [M][M][nlat]. */
int lbm_legendre_tables(int nmax, int nlat, const double* mu, double* pnm,
                        double* hnm, void* stream);

/* exp(-2 pi i p / nlon) for p < nlon, complex FP64 [nlon]; twiddles of the
 * longitude FFT (the role numpy's rfft plays at spectral.py:159-172). */
int lbm_fft_twiddles(int nlon, double* tw, void* stream);

/* Per-n gravity-wave matrices of the semi-implicit scheme,
 *   M(n) = diag(fd ft) - dt^2 lap(n) (whmtx + gcmtx ft),
 *   ft = 1 + 2 dt ktt[n], fd = 1 + 2 dt kd[n]
 * (SemiImplicit.prepare, integrator.py:149-158).
 * lap[M], ktt/kd[M][K], whmtx/gcmtx[K][K] -> mats[M][K][K]. */
int lbm_gravity_wave_matrices(int nmax, int kmax, double dt, const double* lap,
                              const double* ktt, const double* kd,
                              const double* whmtx, const double* gcmtx,
                              double* mats, void* stream);

/* Batched inverse by Gauss-Jordan elimination with partial pivoting, FP64
 * (xp.linalg.inv at integrator.py:161 and numpy inv at integrator.py:226).
 * a, ainv: [batch][n][n]; info[batch] = 0, or 1 + the column of a zero pivot
 * (the caller reads info after the stream completes; a nonzero entry means
 * that matrix is singular). n <= 64. */
int lbm_batched_inverse(int batch, int n, const double* a, double* ainv,
                        int* info, void* stream);

/* ============================================================================
 * Spectral transforms on the reference layouts  (spectral.py:159-276)
 *   grid    (R)       [batch][nlat][nlon][ncol]
 *   Fourier (R, cplx) [batch][M][nlat][ncol]
 *   spectral(R, cplx) [batch][M][M][ncol]   rectangle, zero for n < m
 * ==========================================================================*/

/* four = jscale[j] / nlon * rfft(grid) along longitude, m < M
 * (Spectral._fft_fwd, spectral.py:159-164).  jscale (R)[nlat] or NULL.
 * tw: twiddles (R, complex)[nlon] from lbm_fft_twiddles. nlon in {64,128,256}. */
int lbm_fourier_forward(int prec, int batch, int nlat, int nlon, int ncol,
                        int nmax, const void* grid, const void* jscale,
                        const void* tw, void* four, void* stream);

/* grid = jscale[j] * irfft(nlon * four) (Spectral._fft_inv,
 * spectral.py:166-172; imaginary part of m = 0 dropped). */
int lbm_fourier_inverse(int prec, int batch, int nlat, int nlon, int ncol,
                        int nmax, const void* four, const void* jscale,
                        const void* tw, void* grid, void* stream);

/* Legendre analysis (the matmuls of spectral.py:190, 242-243):
 *   spec[b][m][n][c] (+)= nfac[n] * ( ca * sum_j ta[m][n][j] fa[b][m][j][c]
 *                                    + cb * sum_j tb[m][n][j] fb[b][m][j][c] )
 * where ca = i m if ima else 1 (likewise cb with imb) times sign sb for the
 * second term.  fb/tb may be NULL; nfac (R)[M] may be NULL; tables (R)
 * [M][M][nlat]; accumulate = 0 overwrites (and zeroes n < m). */
int lbm_legendre_analysis(int prec, int batch, int nmax, int nlat, int ncol,
                          const void* fa, const void* ta, int ima,
                          const void* fb, const void* tb, int imb, double sb,
                          const void* nfac, int accumulate, void* spec,
                          void* stream);

/* Legendre synthesis (spectral.py:196, 220-221, 271-272):
 *   four[b][m][j][c] = sum_n ta[m][n][j] ca na[n] sa[b][m][n][c]
 *                    + sb * sum_n tb[m][n][j] cb nb[n] sb_[b][m][n][c]
 * ca/cb = i m when ima/imb; na/nb (R)[M] may be NULL (= 1). */
int lbm_legendre_synthesis(int prec, int batch, int nmax, int nlat, int ncol,
                           const void* sa, const void* ta, int ima,
                           const void* na, const void* sb_, const void* tb,
                           int imb, const void* nb, double sb, void* four,
                           void* stream);

/* ============================================================================
 * Linearised tendency, grid-point part  (Dynamics.tendencies,
 * dynamics.py:176-267) on the reference grid layout, one launch for all the
 * pointwise and vertical-column algebra.  Sizes: E members, J x I grid,
 * K levels; 3-D arrays (R)[E][J][I][K], 2-D (R)[E][J][I].  Basic-state
 * arrays carry no member axis.
 * ==========================================================================*/
typedef struct lbm_tend_grid_args {
  int nmem, nlat, nlon, kmax, strictly_linear;
  double kappa, epsvt, rair;
  /* vertical constants (R)[K] (sigm: [K+1]) */
  const void *dsig, *sigm, *alpha, *w3, *wP, *cpg, *sig, *ww, *tmtx, *tref;
  /* basic state: 3-D (R)[J][I][K], sdot (R)[J][I][K+1], 2-D (R)[J][I] */
  const void *ub, *vb, *tb, *qb, *tvb, *absvor, *divb, *x5b, *sdotb;
  const void *pixb, *piyb, *psb;
  /* perturbation inputs */
  const void *u, *v, *t, *q, *vor, *div, *pix, *piy, *ps;
  /* optional grid forcings (NULL = none), member stride in elements */
  const void *frc_t, *frc_ps, *frc_q;
  int64_t frc_t_stride, frc_ps_stride, frc_q_stride;
  /* outputs: 3-D (R)[E][J][I][K], 2-D (R)[E][J][I]; omega may be NULL */
  void *fu, *fv, *ke, *gt, *xu, *xv, *g, *yu, *yv, *gt_pi, *omega, *sdot;
  /* tangent-linear mode: when non-NULL, the kinetic-energy term
   * 0.5 (u^2 + v^2) is replaced by its linearisation u0 u + v0 v about the
   * trajectory (u0, v0) (R)[E][J][I][K]; both NULL = the model's own term */
  const void *lin_u, *lin_v;
} lbm_tend_grid_args;

int lbm_tendency_grid(int prec, const lbm_tend_grid_args* a, void* stream);

/* ============================================================================
 * Semi-implicit leapfrog update  (Integrator.step, integrator.py:264-315) on
 * the rectangle spectral layout (R, complex)[E][M][M][K] ((E)[M][M] for pi).
 * ==========================================================================*/
typedef struct lbm_implicit_args {
  int nmem, nmax, kmax;
  double dt;
  /* operators (R): lap[M]; kv, kd, ktt, kq [M][K]; ww, tmtx [K][K]; gg,
   * dsig [K]; minv [M][K][K]; vdiff minv [K][K] or NULL per variable */
  const void *lap, *kv, *kd, *ktt, *kq, *ww, *tmtx, *gg, *dsig, *minv;
  const void *vd_vor, *vd_div, *vd_t, *vd_q;
  /* previous level and explicit tendencies */
  const void *p_vor, *p_div, *p_t, *p_pi, *p_q;
  const void *w_vor, *w_div, *w_t, *w_pi, *w_q;
  /* new level (outputs) */
  void *n_vor, *n_div, *n_t, *n_pi, *n_q;
} lbm_implicit_args;

int lbm_implicit_step(int prec, const lbm_implicit_args* a, void* stream);

/* ============================================================================
 * Adjoints of the two maps above (the transposes of their linearisations),
 * for the hand-written adjoint of the time step.  Same layouts and sizes.
 * ==========================================================================*/
typedef struct lbm_tend_adj_args {
  int nmem, nlat, nlon, kmax;
  double kappa, epsvt, rair;
  const void *dsig, *sigm, *alpha, *w3, *wP, *cpg, *ww, *tmtx, *tref;
  const void *ub, *vb, *tb, *qb, *tvb, *absvor, *divb, *x5b, *sdotb, *pixb, *piyb;
  /* trajectory (R)[E][J][I][K] of the kinetic-energy linearisation, or both
   * NULL for the strictly linear tendency */
  const void *u0, *v0;
  /* inputs: adjoints of fu fv ke gt xu xv g yu yv (3-D) and gt_pi (2-D) */
  const void *a_fu, *a_fv, *a_ke, *a_gt, *a_xu, *a_xv, *a_g, *a_yu, *a_yv, *a_gt_pi;
  /* outputs: adjoints of u v t q vor div (3-D), pi_x pi_y (2-D) */
  void *a_u, *a_v, *a_t, *a_q, *a_vor, *a_div, *a_pix, *a_piy;
} lbm_tend_adj_args;

/* Replaces: no reference function (the reference has no adjoint); transpose
 * of the grid-point part of Dynamics.tendencies, dynamics.py:176-267. */
int lbm_tendency_grid_adjoint(int prec, const lbm_tend_adj_args* a, void* stream);

typedef struct lbm_implicit_adj_args {
  int nmem, nmax, kmax;
  double dt;
  const void *lap, *kv, *kd, *ktt, *kq, *ww, *tmtx, *gg, *dsig, *minv;
  const void *vd_vor, *vd_div, *vd_t, *vd_q;
  /* inputs: adjoint of the new level */
  const void *an_vor, *an_div, *an_t, *an_pi, *an_q;
  /* outputs: adjoints of the previous level and of the explicit tendencies */
  void *ap_vor, *ap_div, *ap_t, *ap_pi, *ap_q;
  void *aw_vor, *aw_div, *aw_t, *aw_pi, *aw_q;
} lbm_implicit_adj_args;

/* Transpose of Integrator.step, integrator.py:264-315. */
int lbm_implicit_step_adjoint(int prec, const lbm_implicit_adj_args* a, void* stream);

/* ============================================================================
 * Fused ensemble stepper (the hot path).  The prognostic state lives in
 * packed spectral space; each step runs four kernels: grid-point tendency
 * (with the longitude FFTs), Legendre analysis, implicit spectral update with
 * the Robert-Asselin filter, Legendre synthesis.  All arrays (R).
 *
 * Layouts (E members, J lats, I lons, K levels, M = nmax+1, NS packed):
 *   sa3  [E][4][NS][K] cplx  current level (t): vor, div, T, q
 *   sas  [E][4][NS]    cplx  current level surface: pi, and the sigma-weighted
 *                             column sums of psi, chi, div (for sigma-dot)
 *   sb3  [E][4][NS][K] cplx  previous level (t - dt), Robert-Asselin filtered
 *   psa  [E][J][I]           grid ps' of the level before the current one
 *   psb  [E][J][I]           grid ps' of the filtered previous level
 *   sf   [E][M][J][K][6] cplx  synthesis (Fourier) of u cos, v cos, vor, div, T, q
 *   sfs  [E][M][J][5] cplx     pi, H pi, column-sum u cos, v cos, div
 *   af   [E][M][J][K][7] cplx  weighted Fourier inputs of the analysis
 *   afs  [E][M][J][2] cplx     gt_pi, pi(t-dt)
 *   tend [E][4][NS][K] cplx, tends [E][2][NS] cplx   explicit tendencies
 *   grid6 [E][J][6 + 6K][I] float (FP32 mode; NULL in FP64 mode): grid rows
 *        pi, pi_x, pi_y, U-sum, V-sum, D-sum, then per level u, v, vor,
 *        div, T, q (u and v divided by a cos)
 *   grid9 [E][J][2 + 9K][I] float (FP32 mode): gt_pi, pi(t - dt), then per
 *        level gt, xu, g, yu, fu, fv, ke, xv, yv
 *   symp, symh [NS][J/2]       P and H at the northern latitudes, packed rows
 *   tw [I] cplx; jfac [4][J]: gw, gwdel*coslat, 1/(a coslat), coslat
 *   vert [16][K+1]: see LBM_VERT_* below
 *   b3 [14][J][K][I]: ub vb tb qb tvb absvor divb x5b tdev tvdev, then the
 *                   half vertical differences 0.5 (f[k+1] - f[k]) of ub vb tb
 *                   qb (0 at the top level)
 *   bsd [J][K+1][I] basic sigma-dot; b2 [5][J][I]: pixb piyb psbar
 *                   sum_k dsig ub, sum_k dsig vb
 *   ops: lap, invlap, nn1a [M]; kv kd ktt kq [M][K]; ww tmtx [K][K];
 *        minv [nsets][M][K][K] (stored transposed: [n][l][k]);
 *        vdiff [nsets][4][K][K]: implicit vertical-diffusion operator minus
 *        the identity, transposed, with vd_on[4] flags.  ww and tmtx are not
 *        read (may be NULL): the kernels apply both through their level-scan
 *        forms from vert, (WW x)_k = RALPHA_k x_k + sum_{l<k} RDLOG3_l x_l and
 *        (tmtx D)_k = KTREF_k (ALPHA_k D_k + W3_k sum_{l>k} DSIG_l D_l), the
 *        structure vertical.py gives them
 *   dft [M][I/4+1] (cos, sin)(2 pi m i / I): longitude DFT table of the FP32
 *        grid kernel (may be NULL in FP64 mode)
 *   frc3 [Ef][4][NS][K], frcs [Ef][NS]: spectral forcing (NULL = none),
 *        Ef = E or 1 (frc_shared = 1)
 *   err [1] int: set nonzero when a non-finite value is produced
 *   err_member [E] int or NULL: when given, entry e is also set nonzero when
 *        member e produces a non-finite value, so that the host can name the
 *        members that blew up (the reference's FloatingPointError,
 *        model.py:245-247); the kernels only ever set these flags, the caller
 *        clears them
 *   legendre: 0 = the Legendre analysis and synthesis on the FP32 FMA
 *        pipes; 3 or 6 = their level fields on the tensor cores (tcgen05,
 *        FP32 mode only): operands split into three bfloat16 pieces,
 *        products summed in FP32 in tensor memory, 6 = the six products down
 *        to third order (FP32-level accuracy), 3 = the three products of a
 *        two-way split (about 16 bits)
 *   tc_anal: table image of the tensor-core analysis (legendre != 0), 16-byte
 *        aligned: for m = 0..N, for each step s of 16 latitudes, the tables
 *        P, H and nn1a P (in that order), each as three bfloat16 pieces
 *        (b0 = bf16(x), b1 = bf16(x - b0), b2 = bf16(x - b0 - b1), split from
 *        FP64), each piece an NB(m) x 16 tile (NB(m) = N + 1 - m rounded up to
 *        16; rows n - m, zero past N) whose element (r, kk) sits at byte
 *        (r / 8) 256 + (kk / 8) 128 + (r % 8) 16 + (kk % 8) 2; needs nlat a
 *        multiple of 16 and kmax even
 *   tc_synth: table image of the tensor-core synthesis (legendre != 0),
 *        16-byte aligned: JT = nlat if 6 nlat <= 512 latitudes fit, else
 *        nlat / 2 (two parts); for m = 0..N, for each part, for each step s
 *        of 16 rows n = m + 16 s + kk, the tables m P il, -H il, H il and P
 *        (il = -a^2 / (n (n + 1)), the inverse Laplacian factor of row
 *        n (zero for n = 0; rows past N are zero), each as three bfloat16
 *        pieces, each piece a JT x 16 tile (rows = latitudes of the part,
 *        K = kk) in the layout of tc_anal
 *   tc_off: with legendre != 0, bit 0 keeps the Legendre analysis, bit 1
 *        the Legendre synthesis and bit 2 the longitude analysis on the FMA
 *        kernels (0 = all on the tensor cores where supported)
 *   tc_g: at most this many members per 128-lane MMA tile of the tensor-core
 *        kernels (0 = as many as fit, 128 / (2 kmax)); fewer members make
 *        more, smaller units of work (a choice of the tile autotuner)
 *   tc_dft: table image of the longitude analysis of the level rows on the
 *        tensor cores (legendre != 0 with nlon <= 128 a power of two and
 *        9 kmax <= 256; NULL otherwise), 16-byte aligned: for each step s of
 *        16 longitudes, three bfloat16 pieces (split from FP64 as for
 *        tc_anal) of the 128 x 16 tile W[L][i] = cos(2 pi m (16 s + i) /
 *        nlon) / nlon for L = 2m and -sin(...) / nlon for L = 2m + 1 (zero
 *        for m > nmax), in the layout of tc_anal; then nlon FP32 values
 *        cos(2 pi t / nlon), t = 0..nlon-1, the table of the two surface
 *        rows, which stay on the FMA pipes
 * sf, af and grid9 must be 16-byte aligned (LBM_ERR_ARG otherwise).
 * ==========================================================================*/
enum {
  LBM_VERT_DSIG = 0, LBM_VERT_SIGM, LBM_VERT_ALPHA, LBM_VERT_W3, LBM_VERT_WP,
  LBM_VERT_RCPG, LBM_VERT_RDLOG3, LBM_VERT_RALPHA, LBM_VERT_TREF,
  LBM_VERT_KTREF, LBM_VERT_SIG, LBM_VERT_GG, LBM_VERT_COUNT
};

typedef struct lbm_stepper_desc {
  int prec, nmem, nlat, nlon, nmax, kmax, nsets, strictly_linear;
  int vd_on[4];
  int frc_shared;
  double kappa, epsvt, robert;
  const void *symp, *symh, *tw, *jfac, *vert, *b3, *bsd, *b2;
  const void *lap, *invlap, *nn1a, *kv, *kd, *ktt, *kq, *ww, *tmtx, *minv, *vdiff;
  const void *frc3, *frcs, *dft;
  void *sa3, *sas, *sb3, *psa, *psb;
  void *sf, *sfs, *af, *afs, *tend, *tends;
  void *grid6, *grid9;
  int* err;
  int* err_member;
  int legendre;
  const void* tc_anal;
  const void* tc_synth;
  int tc_off;
  int tc_g;
  const void* tc_dft;
} lbm_stepper_desc;

/* Per-step control.  dt: time step of this call; set: which operator set
 * (minv/vdiff) matches dt; ps_mode: how the grid ps of the filtered previous
 * level is brought up to date before this step (0 = already current, 1 =
 * copy of the current level as in a forward start, 2 = Robert-Asselin
 * filter); ra_mode: spectral update of the previous level at the end of the
 * step (0 = copy of the current level, 1 = Robert-Asselin filter). */
typedef struct lbm_step_ctl {
  double dt;
  int set, ps_mode, ra_mode, pad;
} lbm_step_ctl;

/* Synthesis of the current level into sf/sfs (run once after loading a
 * state, before the first step). */
int lbm_stepper_prime(const lbm_stepper_desc* d, void* stream);

/* nsteps steps, one lbm_step_ctl each (host array). */
int lbm_stepper_run(const lbm_stepper_desc* d, const lbm_step_ctl* ctl,
                    int nsteps, void* stream);

/* One kernel of one step, for per-kernel timing and profiling: kernel 0 =
 * grid-point tendency with the longitude transforms, 1 = Legendre analysis,
 * 2 = implicit update, 3 = Legendre synthesis.  Launching 0..3 in order is
 * the same as lbm_stepper_run for that step.  In FP32 mode kernel 0 is three
 * launches, also available one by one: 4 = longitude synthesis (sf, sfs ->
 * grid6), 5 = column algebra (grid6 -> grid9, grid ps), 6 = longitude
 * analysis (grid9 -> af, afs); 4, 5, 6 in order equal 0. */
int lbm_stepper_launch(const lbm_stepper_desc* d, const lbm_step_ctl* ctl,
                       int kernel, void* stream);

/* Apply the pending grid-ps update (ps_mode as in lbm_step_ctl) so that psa
 * holds ps' of the current level and psb that of the filtered previous
 * level, as after the reference's loop body. */
int lbm_stepper_flush(const lbm_stepper_desc* d, int ps_mode, void* stream);

/* Column sums of the current level's psi, chi, div into sas[1..3] (needed
 * after loading a state into sa3). */
int lbm_stepper_colsum(const lbm_stepper_desc* d, void* stream);

/* CUDA graph of nsteps steps captured from lbm_stepper_run on `stream`
 * (capture mode global); launch replays it on any stream.  The handle owns
 * the instantiated graph. */
typedef struct lbm_graph lbm_graph;
int lbm_graph_capture(const lbm_stepper_desc* d, const lbm_step_ctl* ctl,
                      int nsteps, void* stream, lbm_graph** out);
int lbm_graph_launch(lbm_graph* g, void* stream);
int lbm_graph_destroy(lbm_graph* g);

/* Daily history accumulation (model.py:257-277).  The reference writes, per
 * output day, the mean of the trapezoid 0.5 (top(s) + top(s-1)) of its
 * top-of-step diagnostics (psi, chi, u, v, omega, T, z, ps).  All eight are
 * linear in the spectral state and the grid ps', so the stepper accumulates
 * those with the same weights and forms the fields once per day from the
 * mean.  Elementwise over n reals of precision `prec` (a complex value is two):
 *   mode 0: prev = cur                          (start-up step: no sample)
 *   mode 1: acc += w (cur + prev); prev = cur   (w = 1/2 for the trapezoid)
 * acc is FP64 [n]; cur and prev are (R)[n]. */
int lbm_history_accumulate(int prec, int64_t n, const void* cur, void* prev,
                           double* acc, double w, int mode, void* stream);

/* GrADS history records of one output day (replaces the record loop of
 * GradsWriter.add, output.py:46-71).  fields is a host array of 8 device
 * pointers to FP64 grid fields: psi, chi, u, v, w, t, z as [npts][kmax]
 * (latitude, longitude, level; level fastest) and ps as [npts].  For each
 * level of the first seven, then for ps, one Fortran sequential record: a
 * big-endian int32 byte count 4 npts, npts big-endian IEEE float32 values
 * (rounded to nearest), the count again.  With apply_z, z gets
 * (ps * zmul) / zdiv added first (zmul = 100, zdiv = rho0 g; output.py:64-65).
 * out holds (7 kmax + 1) (npts + 2) uint32 words. */
int lbm_grads_records(int64_t npts, int kmax, const double* const* fields, int apply_z,
                      double zmul, double zdiv, uint32_t* out, void* stream);

/* ---- Basic-state preprocessing (basicstate.py), FP64, one thread per column --
 * lbm_z2ps: surface pressure [hPa] from geopotential height z [ncol][nk]
 *   (gpm, level 0 = the highest pressure) and surface height zs [ncol] (m;
 *   NULL = 0) on the pressure levels plev [nk] (hPa): interpolation linear
 *   in ln p between the first level above zs and the one below it
 *   (basicstate.py:115-151).
 * lbm_spline: natural cubic spline through (x [nk], z [ncol][nk]) with a
 *   shared monotonic abscissa, evaluated at xi [ncol][nl] -> out [ncol][nl];
 *   outside the data range the end value, or xmiss where omisb (beyond x_0)
 *   or omist (beyond x_{nk-1}) is set (basicstate.py:176-238); nk <= 64.
 * lbm_zonal_filter: x [nlat][nlon][nk] in place; mode 1 = zonal mean,
 *   mode 2 = deviation from it (basicstate.py:165-173). */
int lbm_z2ps(int64_t ncol, int nk, const double* z, const double* zs, const double* plev,
             double* ps, void* stream);
int lbm_spline(int64_t ncol, int nk, int nl, const double* x, const double* z, const double* xi,
               double* out, int omisb, int omist, double xmiss, void* stream);
int lbm_zonal_filter(int nlat, int nlon, int nk, double* x, int mode, void* stream);

/* ---- Host <-> device transfers over the CPU-GPU link -------------------------
 * No counterpart in the reference (its arrays move by cupy.asarray /
 * cupy.asnumpy, backend.py:80-105).  Copies `bytes` from src to dst with SM
 * loads and stores, so that on a node whose CPU and GPU share a coherent
 * link (NVLink-C2C on Grace-Blackwell) pinned host memory is read or written
 * at the link's rate rather than a copy engine's.  Each pointer is device
 * memory or pinned host memory that the device can address (cudaHostAlloc /
 * cudaHostRegister; pageable memory gives LBM_ERR_ARG); both 16-byte aligned;
 * any byte count.  Asynchronous on `stream`, like cudaMemcpyAsync. */
int lbm_link_copy(void* dst, const void* src, int64_t bytes, void* stream);

/* ---- Stepping without allocating -------------------------------------------
 * No counterpart in the reference, whose step functions allocate their work
 * arrays through the array backend on every call.
 *
 * lbm_stepper_run_noalloc is lbm_stepper_prime followed by lbm_stepper_run
 * (same kernels, same results) for callers that cannot allocate device
 * memory for the intermediate buffers (sf, sfs, af, afs, tend, tends and the
 * FP32 grid rows grid6, grid9): a
 * host that embeds the dynamical core behind an FFI and hands the library
 * only its state, operator and forcing buffers -- for instance because all of
 * its device memory belongs to another runtime's pool, or because cudaMalloc
 * and cudaFree synchronise the device in the middle of its time loop -- and
 * that does not want to keep those buffers (15.8 MiB per member at T42L20 in
 * FP32, 12.4 MiB in FP64) alive between calls.
 *
 * The intermediates come instead from one static device array of
 * LBM_NOALLOC_SCRATCH_BYTES, which every GPU that loads the library holds
 * until the process exits.  The call allocates nothing: no cudaMalloc, no
 * cudaFree, no allocating library routine.
 *   - d: as for lbm_stepper_run; its sf, sfs, af, afs, tend, tends, grid6
 *     and grid9 are ignored (may be NULL).  Every other pointer is the
 *     caller's, and the state (sa3, sas, sb3, psa, psb, err) is updated in
 *     place.
 *   - The call needs E * M * J * (13 K + 7) + E * NS * (4 K + 2) complex
 *     values, plus E * J * I * (15 K + 8) floats in FP32 mode (each buffer
 *     rounded up to 256 bytes); a case larger than LBM_NOALLOC_SCRATCH_BYTES
 *     is rejected with LBM_ERR_SCRATCH before anything is launched (at most
 *     2 members at T42L20 in FP32 or FP64; 8 and 10 at T21L20).
 *   - Each call first clears the part of the area it uses (cudaMemsetAsync
 *     on `stream`) and synthesises the current level into it, so nothing
 *     carries over from an earlier call: the state in d is all there is.
 *   - Set-up: the first call on a device looks up the array's address with
 *     cudaGetSymbolAddress, with that device current, and keeps it.  Make the
 *     first call on each device before any stream capture begins.  The kept
 *     address belongs to the device's primary context, the one the CUDA
 *     runtime uses: only callers that run under that context are supported,
 *     and a device reset (cudaDeviceReset) after the first call leaves the
 *     kept address invalid, so do not call this entry point after one.
 *   - nlon must be 64, 128 or 256 and every size positive (LBM_ERR_ARG);
 *     the whole descriptor is checked before the area is cleared.
 *   - The area is shared by every call on a device: two calls whose work
 *     overlaps on the GPU (different streams, or different host threads with
 *     no ordering between them) race on it and give wrong results.  Order
 *     them on one stream or with events. */
#define LBM_NOALLOC_SCRATCH_BYTES (32u << 20) /* 32 MiB per device */
int lbm_stepper_run_noalloc(const lbm_stepper_desc* d, const lbm_step_ctl* ctl,
                            int nsteps, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* LBM_GB300_H */
