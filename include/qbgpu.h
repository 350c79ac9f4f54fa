/*
 * qbgpu.h — C ABI of libqbgpu, the GB300 (sm_103a) boundary-integral hot path
 * of QuantumBilliards.jl.
 *
 * Conventions
 *   - Every function returns qbg_status (0 = QBG_OK). No exception or longjmp
 *     crosses the ABI. qbg_last_error() returns the calling thread's message.
 *   - Complex numbers are interleaved (re, im) doubles, bit-identical to Julia
 *     ComplexF64 / C double _Complex. Matrices are column-major with leading
 *     dimension equal to their row count (Julia Matrix{ComplexF64}).
 *   - Pointers are host pointers unless a call's flags contain
 *     QBG_PTR_DEVICE, in which case they are device pointers on the current
 *     CUDA device.
 *   - Handles own their device memory and one CUDA stream each. Calls on
 *     different handles may run concurrently from different threads; calls on
 *     the same handle are serialised by the handle.
 *
 * Each entry point names the reference function it replaces
 * (paths inside QuantumBilliards.jl).
 */
#ifndef QBGPU_H
#define QBGPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t qbg_status;

enum {
  QBG_OK = 0,
  QBG_EINVAL = 1,     /* bad argument */
  QBG_ENOMEM = 2,     /* device allocation failed */
  QBG_EBUDGET = 3,    /* request exceeds the handle's HBM budget */
  QBG_ESINGULAR = 4,  /* exactly singular pivot met (factorisation continues, as lu!(; check=false)) */
  QBG_ETIMEOUT = 5,   /* a bounded device wait gave up */
  QBG_ECUDA = 6,      /* CUDA runtime / library error */
  QBG_ENOTSUP = 7     /* combination not implemented */
};

enum { QBG_FORM_DLP = 0, QBG_FORM_CFIE = 1 };
/* Precision forms:
 *   QBG_PREC_FP64  complex128 kernel values, FP64 LU and solves (the drop-in form).
 *   QBG_PREC_MIXED FP64 kernel values stored as a complex64 pair (hi, lo);
 *                  FP32 LU of hi, FP32 solves, and refinement of T X = V with
 *                  residuals of hi + lo in compensated (double-float) FP32
 *                  arithmetic, so the refined solution is that of the FP64 operator.
 *   QBG_PREC_FP32  FP32 kernel values (FP64 geometry, FP64 phase reduction,
 *                  FP64 near-diagonal band |k r| < 12), FP32 LU, refinement
 *                  against the FP32 operator: fastest, accuracy bounded by the
 *                  FP32 rounding of the operator. */
enum { QBG_PREC_FP64 = 0, QBG_PREC_MIXED = 1, QBG_PREC_FP32 = 2 };
/* QBG_SPLIT_LO (qbg_assemble, qbg_assemble_cheb with QBG_PREC_MIXED, deriv 0):
 * outs holds 2 nk pointers, the complex64 high words of A(k_1..k_nk) and then
 * their low words (value - high, rounded to complex64), so high + low carries
 * the kernel value to ~2^-48 relative. */
enum { QBG_PTR_DEVICE = 1, QBG_V_PER_DISK = 2, QBG_SPLIT_LO = 4 };

/* Boundary discretisation (BoundaryPointsCFIE, boundarypoints.jl:487-503),
 * components concatenated; holes already orientation-reversed as
 * evaluate_points returns them (cfie.jl:822-834). */
typedef struct qbg_geom_desc {
  int32_t form;                 /* QBG_FORM_DLP (one component) or QBG_FORM_CFIE */
  int32_t ncomp;                /* number of closed components */
  const int64_t* comp_offsets;  /* ncomp+1 offsets, [0] = 0, [ncomp] = n */
  const double* x;              /* n node coordinates */
  const double* y;
  const double* dx;             /* n first derivatives d gamma / d sigma */
  const double* dy;
  const double* ddx;            /* n second derivatives */
  const double* ddy;
  const double* ts;             /* n computational parameters sigma (Kress log term) */
  const double* ws;             /* n quadrature weights */
  /* optional symmetry reduction (DLP: DLPKressReducedWorkspace, dlp_kress.jl:65-78,
   * the Kress-split entry at (I_a, I_b) plus regular image kernels; CFIE: the
   * reduced workspace of cfie_kress.jl:212-316, sum over the orbit of the
   * Kress-split entries, cfie_kress.jl:512-617): m fundamental nodes, each with
   * norb images (its own index included) */
  int64_t m;                    /* 0 = no reduction */
  int32_t norb;
  const int64_t* fund;          /* m full indices I_a */
  const int64_t* orbit;         /* m*norb full indices of the images of I_b */
  const double* orbit_scale;    /* m*norb complex scale factors (character values) */
  /* CFIE_alpert quadrature (cfie_alpert.jl:947-1013, 1261-1350); quad = 0 is
   * Kress. Every component is a closed curve on a periodic midpoint grid; its
   * self block drops the trapezoid band |i - j| < alpert_a and adds, per
   * target, alpert_j correction nodes on each side whose kernel values are
   * spread over alpert_ninterp grid nodes. */
  int32_t quad;                 /* 0 = Kress log split, 1 = Alpert */
  int32_t alpert_a;
  int32_t alpert_j;
  int32_t alpert_ninterp;
  const double* alpert_w;       /* j rule weights */
  const int64_t* alpert_off;    /* [2][j][ninterp] stencil offsets, + side then - side */
  const double* alpert_wt;      /* [2][j][ninterp] interpolation weights */
  const double* alpert_nodes;   /* [6][j][n]: r+, r-, inner+, inner-, speed+, speed- of the correction
                                   nodes of every target (r = +inf: skipped) */
} qbg_geom_desc;

typedef struct qbg_geom qbg_geom;
typedef struct qbg_beyn qbg_beyn;

/* Library / error helpers */
qbg_status qbg_version(int32_t* major, int32_t* minor);
size_t qbg_last_error(char* buf, size_t len);
qbg_status qbg_device_sync(void);

/* Upload a discretisation; computes the Kress circulant column per component
 * (kress_R!, boundarypoints.jl:310-358) and the speed/curvature terms
 * (cfie_geom_cache, boundarypoints.jl:854-880) on the device.
 * Replaces: build_dlp_kress_workspace (dlp_kress.jl:679-708),
 *           build_cfie_kress_workspace (cfie_kress.jl:230-270). */
qbg_status qbg_geom_create(const qbg_geom_desc* desc, qbg_geom** out);
qbg_status qbg_geom_destroy(qbg_geom* g);
qbg_status qbg_geom_dim(const qbg_geom* g, int64_t* dim);

/* Assemble the boundary matrix (and, with deriv = 1, its first and second
 * k-derivatives) at nk wavenumbers ks (complex, interleaved).
 *   outs: nk*(1+2*deriv) pointers to dim x dim complex matrices, ordered
 *         [A(k_1..k_nk), A'(k_1..k_nk), A''(k_1..k_nk)].
 *   prec = QBG_PREC_FP64: complex128 outputs; QBG_PREC_MIXED (FP64 values
 *   rounded once) and QBG_PREC_FP32: complex64 outputs.
 * Replaces: construct_matrices! (dlp_kress.jl:1627-1679, cfie_kress.jl:893-929),
 *           construct_boundary_matrices! (chebyshev_euclidian_helmholtz_dlp_kress.jl:1110,
 *           ..._cfie_kress.jl:1431) and construct_boundary_matrices_with_derivatives!
 *           (..._dlp_kress.jl:1126). */
qbg_status qbg_assemble(qbg_geom* g, const double* ks, int64_t nk, int32_t deriv, int32_t prec, int32_t flags,
                        void* const* outs);

/* Chebyshev-panel parameters (the reference's n_panels_h, M_h, n_panels_j,
 * M_j keywords; zero fields take the reference defaults 15000, 5, 3000, 5). */
typedef struct qbg_cheb_params {
  int32_t n_panels_h;  /* uniform panels of [0.95 r_min, 1.05 r_max] for H0, H1 */
  int32_t M_h;         /* Chebyshev degree per Hankel panel (2..16) */
  int32_t n_panels_j;  /* uniform panels of [0, 1.05 r_max] for J0, J1 */
  int32_t M_j;
} qbg_cheb_params;

/* Assembly with kernel values interpolated from per-k Chebyshev panels built
 * on the device (the reference's complex-k route:
 * construct_boundary_matrices!(...; use_chebyshev=true),
 * chebyshev_euclidian_helmholtz_cfie_kress.jl:1431-1470,
 * ..._dlp_kress.jl:1110-1124; tables as plan_h / plan_j,
 * chebyshev_bessels.jl:461-528). Same outputs as qbg_assemble; prec FP64 or
 * MIXED; deriv = 1 for DLP in FP64. */
qbg_status qbg_assemble_cheb(qbg_geom* g, const double* ks, int64_t nk, int32_t deriv, int32_t prec, int32_t flags,
                             const qbg_cheb_params* cheb, void* const* outs);

/* Same assembly as qbg_assemble, for callers that cannot allocate device
 * memory during the call (they own every device buffer, e.g. a pre-reserved
 * arena or a loop where cudaMalloc's device synchronisation is not allowed).
 * No counterpart in the reference: it exists only for this library's users.
 * Outputs are device pointers (outs_dev, as in qbg_assemble with
 * QBG_PTR_DEVICE). The wavenumbers and the output-pointer table are staged in
 * a fixed device array of QBG_NOALLOC_MAX_K entries (20 KiB, resident on each
 * device until exit); nk > QBG_NOALLOC_MAX_K is rejected with QBG_EINVAL.
 * Alpert geometries are accepted with prec QBG_PREC_FP64 only (their complex64
 * forms stage FP64 blocks of N^2 entries): other precisions return QBG_ENOTSUP.
 * Calls share that array and are serialised inside the process; each returns
 * after its kernel finished. The first call on a device resolves the array's
 * address on that device: make it before any stream capture. */
#define QBG_NOALLOC_MAX_K 512
qbg_status qbg_assemble_noalloc(qbg_geom* g, const double* ks, int64_t nk, int32_t deriv, int32_t prec,
                                void* const* outs_dev);

/* Beyn contour step (construct_B_matrix, beyn.jl:257-322), device side:
 * create = contour nodes z_j = k0 + R e^{i theta_j}, assembly of all T(z_j),
 * batched LU; moments = T(z_j)^{-1} V for every node and the sums
 * A0 = sum w_j X_j, A1 = sum w_j z_j X_j. The host does the rank-revealing
 * SVD of A0 and the small eigenproblem. moments may be called again with a
 * wider V (the reference's r -> 2r regrowth, beyn.jl:291-309) without
 * refactoring. */
typedef struct qbg_beyn_opts {
  int32_t flags;        /* QBG_PTR_DEVICE: V, A0, A1 are device pointers;
                           QBG_V_PER_DISK: V holds one N x L probe block per disk */
  int32_t max_refine;   /* complex64 forms: maximum compensated refinement sweeps (default 10); refinement
                           also stops when a sweep contracts the residual by less than 2 */
  double refine_tol;    /* complex64 forms: the first correction uses an FP32 residual; later residuals
                           are compensated; once max|R| <= tol * max|V| the correction from that
                           residual is applied and refinement stops (default 1e-6). Each correction
                           contracts the residual by rho ~ cond(T) * 2^-24 (refine_history shows it),
                           so the returned solution's residual is about tol * rho. */
  int32_t nb;           /* LU block size (0 = default) */
  int32_t eval_mode;    /* 0: Chebyshev panels (the reference's default, use_chebyshev=true);
                           1: direct evaluation of H0, H1, J0, J1 */
  qbg_cheb_params cheb; /* panel parameters for eval_mode 0 (zeros = reference defaults) */
  int32_t fp32_sweeps;  /* complex64 forms: corrections from plain FP32 residuals V - hi X before the
                           compensated ones (0 = default 1, at most 4) */
  int32_t solve_block;  /* complex64 forms: rows per block of the triangular solves, nb, 2 nb or 4 nb
                           (0 = default 4 nb for N >= 8 nb) */
  int32_t node_chunk;   /* 0: every contour node's operator stays factored from create on;
                           c > 0: at most c operators are resident and each moments call streams
                           the nodes through them (assemble, factor, solve, accumulate) */
  int32_t resid_engine; /* complex64 forms, the compensated residual R = V - (hi + lo) X:
                           0 = tensor cores (exact 7-bit digit products, 28 B of digits per operator
                           entry held beside the factors), 1 = compensated FP32 on CUDA cores */
} qbg_beyn_opts;

typedef struct qbg_beyn_stats {
  int32_t refine_sweeps;   /* refinement sweeps performed in the last moments call */
  double refine_residual;  /* final max|R| / max|V| (mixed form) */
  int32_t singular;        /* number of contour nodes with an exactly zero pivot */
  double ms_assemble, ms_factor, ms_solve;  /* device time of the phases */
  int32_t nhist;                           /* residuals recorded in refine_history */
  double refine_history[8];                /* max|R|/max|V| before each correction sweep */
  double ms_residual;                      /* device time of the compensated residual launches */
  int32_t n_residual;                      /* number of compensated residual launches */
  int32_t nfp32;                           /* plain FP32 residuals recorded in fp32_history */
  double fp32_history[4];                  /* max|V - hi X| / max|V| of each FP32 residual */
  double ms_solves;                        /* device time of the triangular solves */
  int32_t n_solves;                        /* number of solve passes (each over every contour node) */
} qbg_beyn_stats;

qbg_status qbg_beyn_create(qbg_geom* g, double k0_re, double k0_im, double R, int32_t nq, int32_t prec,
                           const qbg_beyn_opts* opts, qbg_beyn** out);
/* Several disks in one handle: the contour nodes of all disks (disk-major)
 * are assembled in one launch and factored as one batch. This is the loop of
 * compute_spectrum_beyn over its disks (beyn.jl:778-921) with all of them
 * resident at once. k0s: ndisk complex centres (interleaved re, im); Rs:
 * ndisk radii; ndisk * nq <= 65535. */
qbg_status qbg_beyn_create_disks(qbg_geom* g, const double* k0s, const double* Rs, int32_t ndisk, int32_t nq,
                                 int32_t prec, const qbg_beyn_opts* opts, qbg_beyn** out);
/* A0 and A1 hold one N x L block per disk (disk d at offset d * N * L). */
qbg_status qbg_beyn_moments(qbg_beyn* b, const double* V, int64_t L, double* A0, double* A1,
                            qbg_beyn_stats* stats);
/* The moments of V reduced on the device for B = U_k^H A1 W_k Sigma_k^-1
 * (construct_B_matrix, beyn.jl:286-320): the handle keeps every disk's A0 and
 * A1 columns (append = 0 replaces them with this call's L columns, append = 1
 * puts them behind the columns kept so far, the reference's r -> 2r regrowth,
 * beyn.jl:291-309), takes the thin QR A0 = Q R of the m kept columns and
 * returns R (m x m upper triangular) and C = Q^H A1 (m x m), column-major,
 * disk d at offset d * m * m. With R = U_R S W^H the SVD of A0 is
 * (Q U_R) S W^H, so B = U_R,k^H C W_k S_k^-1 on the host from m x m data.
 * m must equal the column count after this call. */
qbg_status qbg_beyn_moments_qr(qbg_beyn* b, const double* V, int64_t L, int32_t append, int64_t m, double* R,
                               double* C, qbg_beyn_stats* stats);
/* construct_B_matrix (beyn.jl:257-322) in one call, for a single-disk handle:
 * the moments of the r probe columns V (N x r, column-major complex128; host,
 * or device with QBG_PTR_DEVICE), the thin SVD of A0 (reduced on the device
 * by a QR, the m x m factor decomposed on the host by one-sided Jacobi), the
 * absolute rank rk = count(S >= svd_tol); when rk == r and 2r < N the block
 * grows once to 2r with V2 (N x r more columns, appended, the first r kept;
 * V2 = NULL skips the regrowth), as the reference's loop leaves after one
 * pass (beyn.jl:307). Outputs: B = U_k^H A1 W_k S_k^-1 (rk x rk, leading
 * dimension rk, host; room for (2r)^2), U_k (N x rk, leading dimension N;
 * host, or device with QBG_PTR_DEVICE; may be NULL), S (the singular values
 * of the final A0, room for 2r; may be NULL), rk and the final column count. */
qbg_status qbg_beyn_B(qbg_beyn* b, const double* V, int64_t r, const double* V2, double svd_tol, double* B,
                      double* Uk, double* S, int64_t* rk, int64_t* r_used, qbg_beyn_stats* stats);
qbg_status qbg_beyn_destroy(qbg_beyn* b);

/* Failure path of the tensor-core kernels (no counterpart in the reference).
 * Every mbarrier wait of the tcgen05 GEMM pipeline gives up after a poll
 * limit (and ~1e9 SM cycles); the kernel then records a sticky error, drains
 * what it started with the full limit, frees its tensor memory and returns
 * without writing its output, and the calling entry reports QBG_ECUDA.
 * qbg_set_tc_wait_limit sets the pipeline waits' poll limit on the current
 * device (polls < 0 restores the built-in limit; 0 makes every pipeline wait
 * give up at once), qbg_clear_tc_error resets the sticky flag there. Both
 * synchronize the device. Meant for tests of that path. */
qbg_status qbg_set_tc_wait_limit(int64_t polls);
/* Validation entry (no counterpart in the reference): the library's batched
 * LU and explicit inverses of `batch` n x n complex128 matrices (host,
 * column-major, contiguous), X = A^{-1}. prec QBG_PREC_FP64: FP64 LU (the
 * path of sigma_min, EBIM and Newton); with sig != NULL also sigma_min of
 * every matrix by the device subspace iteration on its inverse, and with
 * work_out != NULL its final blocks (3 n x 8 complex128 per matrix).
 * prec QBG_PREC_FP32: the matrices rounded to complex64 and factored by the
 * complex64 LU of the Beyn mixed form (panels and tensor-core updates as the
 * current plan and GEMM engine select), X widened back; sig and work_out must
 * be NULL. */
qbg_status qbg_dense_inverse(int32_t n, int32_t batch, int32_t prec, const double* A, double* X, double* sig,
                             double* work_out);
/* Plan of the batched LU, process-wide (no counterpart in the reference):
 * panels per outer block of the two-level factorisation (1..16, default 4;
 * <= 0 keeps the current value), the complex64 panel form (-1 automatic:
 * a cluster of 8 CTAs per panel for batches of at most 4 matrices; 0 one CTA
 * per panel; 1 a cluster) and the number of stream parts a Beyn handle
 * created afterwards factors and solves its operator batch in (1..8,
 * default 4; <= 0 keeps the current value). QBG_LU_OUTER, QBG_LU_CLUSTER and
 * QBG_LU_SPLIT in the environment give the initial values; qbgpu.autotune
 * chooses them by timing. */
qbg_status qbg_set_lu_plan(int32_t outer, int32_t cluster, int32_t parts);
qbg_status qbg_get_lu_plan(int32_t* outer, int32_t* cluster, int32_t* parts);
qbg_status qbg_clear_tc_error(void);

/* Smallest singular value of A(k) for nk real wavenumbers (the :svd branch of
 * @svd_or_det_solve, macros.jl:159-161, called by k_sweep,
 * sweepmethods.jl:132-152): FP64 LU of A(k), then block inverse iteration on
 * (A^H A)^{-1} with 8 vectors and a Rayleigh-Ritz step, until the estimate
 * changes by less than 1e-13 relative (at most 40 sweeps); 0 for an exactly
 * singular A(k). */
qbg_status qbg_sigma_min(qbg_geom* g, const double* ks, int64_t nk, double* sig);

/* EBIM eigen step at a trial wavenumber k (ebim.jl): the eigenpairs of the
 * pencil A v = lambda A' v nearest 0, by FP64 LU of A and block shift-invert
 * iteration on A^{-1} A' (and its adjoint for the left vectors), then the
 * second-order correction eps1 = -lambda, eps2 = -eps1^2/2 (u^H A'' v)/(u^H A' v)
 * (0 when |u^H A' v| <= 1e-15) for every lambda with |Re|, |Im| < dk.
 * Default: solve_krylov! (ebim.jl:464-537): the nev eigenvalues nearest 0, u
 *   the eigenvector of (A^{-1} A')^H, a result kept when |Re(k_c) - k| < dk.
 * QBG_EBIM_FULL: solve_full! (ebim.jl:336-375): every eigenvalue inside the
 *   dk box (nev is the starting block, doubled until the box is covered), u the
 *   left eigenvector of the pencil.
 * Writes up to cap results, nearest first: out_k[2i], out_k[2i+1] = corrected
 * k (complex; the reference returns its real part unless return_imag_part),
 * out_tens[i] = |eps1 + eps2|; *count = the number of results (may exceed
 * cap). iters (optional, 3 values): iterations of the right and left blocks
 * and the final nev. QBG_ESINGULAR when A(k) is exactly singular.
 * qbg_ebim_eig takes the three N x N complex128 column-major matrices (host,
 * or device with QBG_PTR_DEVICE; left unchanged); qbg_ebim_solve assembles
 * A, A', A'' of the geometry at k on the device first (direct FP64 assembly,
 * as qbg_assemble with deriv = 1). */
enum { QBG_EBIM_FULL = 8 };
qbg_status qbg_ebim_eig(int64_t n, const void* A, const void* dA, const void* ddA, double k, double dk, int32_t nev,
                        int32_t flags, int32_t cap, double* out_k, double* out_tens, int32_t* count,
                        int32_t* iters);
qbg_status qbg_ebim_solve(qbg_geom* g, double k, double dk, int32_t nev, int32_t flags, int32_t cap, double* out_k,
                          double* out_tens, int32_t* count, int32_t* iters);
/* Newton refinement of a sweep minimum (newton_refine_svd!,
 * sweepmethods.jl:307-368) on the geometry's discretisation: Newton steps on
 * lambda_min(A(k)^H A(k)) with its first and second k-derivatives (second-order
 * perturbation sum over all eigenpairs of A^H A), k clamped to [a, b], at most
 * maxiter steps, stop when a step is below tol. Writes the refined k and the
 * tension sqrt(lambda_min) there (or at the best k met, when smaller); iters
 * (optional): steps taken. FP64 throughout; A, A', A'' assembled on the device
 * (direct Hankel evaluation). */
qbg_status qbg_newton_refine(qbg_geom* g, double k0, double a, double b, int32_t maxiter, double tol,
                             double* k_out, double* t_out, int32_t* iters);

/* Boundary densities (DLP Kress, dlp_kress.jl:1451-1500, 1914-1949).
 * qbg_adjoint_fredholm: the adjoint Fredholm matrix at real k,
 * A_adj[i, j] = delta_ij - D[j, i] ds_j / ds_i (on a reduced geometry over the
 * fundamental nodes, ds indexed by their full-boundary nodes); ds: the N
 * arc-length weights of the full boundary (pts.ds); out: dim x dim complex128
 * (host, or device with QBG_PTR_DEVICE).
 * qbg_solve_vect: solve_vect's smallest_nullvec_krylov! (dlp.jl:991-1004) on
 * that matrix: the eigenvalue mu of largest modulus of A_adj^-1 (FP64 LU, block
 * iteration), sigma = 1/|mu| and the unit eigenvector u (dim complex). */
qbg_status qbg_adjoint_fredholm(qbg_geom* g, double k, const double* ds, void* out, int32_t flags);
qbg_status qbg_solve_vect(qbg_geom* g, double k, const double* ds, double* sigma, double* u);

/* The host eigen-decomposition behind the EBIM Rayleigh-Ritz step, for
 * validation: eigenvalues w (p complex) and unit eigenvectors V (p x p
 * column-major, complex interleaved) of the p x p complex matrix H (Hessenberg
 * reduction, shifted QR, back substitution; no device work). */
qbg_status qbg_small_eig(int32_t p, const double* H, double* w, double* V);

/* Panel autotuner (chebyshev_params, chebyshev_optimal_panelization.jl:221-307):
 * starting from *io (zeros = 15000, 5, 3000, 5), grows the panel counts by
 * 1.5x per iteration (every 5th iteration the degrees by grow_M instead; the
 * reference uses 2, 0 keeps the degrees fixed) until the
 * max absolute error of the interpolated H0, H1 (on [rmin, rmax]) and J0, J1
 * (on [0, rmax]) at nsample radii is below tol for every wavenumber. Writes
 * the parameters to *io and the worst errors to err4 (may be null). Returns
 * QBG_ETIMEOUT with the best effort when max_iter is reached. */
qbg_status qbg_cheb_autotune(qbg_geom* g, const double* ks, int64_t nk, double tol, int32_t nsample,
                             int32_t max_iter, int32_t grow_M, qbg_cheb_params* io, double* err4);

/* Residuals of Beyn candidates, the device part of residual_and_norm_select
 * and imag_k_check_EXPERIMENTAL (beyn.jl:557-593, 623-721): for each candidate
 * j (lambdas: n complex) assembles T(lambda_j) in FP64 (through the Chebyshev
 * panels when cheb != NULL, zeros = defaults) and writes
 * out[5 j + 0..4] = ||T phi_j||_2, ||T phi_j||_1, opnorm(T, 1), ||phi_j||_1,
 * ||phi_j||_2 with Phi the N x n column-major block (host) of phi_j = U_k Y_j. */
qbg_status qbg_candidate_residuals(qbg_geom* g, const double* lambdas, int64_t n, const double* Phi,
                                   const qbg_cheb_params* cheb, double* out);

/* Device special functions, for validation: out[4*i..] = J0, J1, Y0, Y1 at z[i]
 * (complex interleaved). f32 = 1 selects the FP32 asymptotic evaluator. */
qbg_status qbg_bessel01(const double* z, int64_t n, int32_t f32, double* out);

/* ------------------------------------------------------------------------
 * Request server (no reference counterpart: the reference runs one call at a
 * time). Requests are admitted against an HBM budget (each request's device
 * footprint is estimated before it starts), run on worker threads with their
 * own CUDA streams, and queued Beyn requests on the same geometry with the
 * same contour size, precision and probe count are merged into one multi-disk
 * device batch (continuous batching: a request joins as soon as memory frees,
 * it does not wait for a batch to fill). All buffers in a request are host
 * memory owned by the caller and must stay valid until the request is done.
 * ------------------------------------------------------------------------ */
typedef struct qbg_server qbg_server;

typedef struct qbg_serve_opts {
  int64_t hbm_budget;   /* device bytes the running requests may hold (0 = 80% of free memory) */
  int32_t workers;      /* requests in flight at once (0 = 4) */
  int32_t max_batch;    /* most Beyn requests merged into one device batch (0 = 8; 1 = no merging) */
  int32_t max_sweeps;   /* most sigma_min sweeps running at once (0 = 1); later sweeps wait, other kinds pass them */
} qbg_serve_opts;

enum { QBG_REQ_BEYN = 0, QBG_REQ_EBIM = 1, QBG_REQ_SWEEP = 2 };

typedef struct qbg_request_desc {
  int32_t kind;     /* QBG_REQ_* */
  qbg_geom* geom;
  int32_t prec;     /* Beyn: QBG_PREC_*; EBIM and sweep run in FP64 */
  /* Beyn (construct_B_matrix's device part): contour k0, R, nq; probe block V
   * (N x L, host); outputs A0, A1 (N x L, host) */
  double k0_re, k0_im, R;
  int32_t nq;
  int64_t L;
  const double* V;
  double* A0;
  double* A1;
  /* EBIM (A, A', A'' at one real k, ebim.jl:931-939): outputs N x N each */
  double k;
  double* out_A;
  double* out_dA;
  double* out_ddA;
  /* sweep (sigma_min at nk real wavenumbers, k_sweep): sig[nk] */
  const double* ks;
  int64_t nk;
  double* sig;
} qbg_request_desc;

typedef struct qbg_request_result {
  int32_t status;      /* the request's own status (QBG_OK, ...) */
  int32_t batched;     /* Beyn requests in the device batch this one ran in */
  double queue_ms;     /* submit -> start */
  double run_ms;       /* start -> done */
} qbg_request_result;

qbg_status qbg_serve_create(const qbg_serve_opts* opts, qbg_server** out);
/* QBG_EBUDGET when the request alone does not fit the budget */
qbg_status qbg_serve_submit(qbg_server* s, const qbg_request_desc* req, int64_t* id);
/* done = 1 once the request has finished (successfully or not) */
qbg_status qbg_serve_poll(qbg_server* s, int64_t id, int32_t* done);
/* waits up to timeout_s seconds (< 0: no limit); QBG_ETIMEOUT if still running.
 * On return with QBG_OK the request is finished and forgotten by the server. */
qbg_status qbg_serve_wait(qbg_server* s, int64_t id, double timeout_s, qbg_request_result* res);
/* finishes the queued and running requests, then stops the workers */
qbg_status qbg_serve_destroy(qbg_server* s);

/* Device complex64 GEMM, for validation: C_b = alpha A_b B_b + beta C_b for
 * b < batch, column-major host buffers (complex interleaved floats; A_b at
 * A + 2*b*lda*K, B_b at B + 2*b*ldb*N, C_b at C + 2*b*ldc*N). engine selects
 * the GEMM inside the FP32 LU and solves: 0 = CUDA-core FMA tiles,
 * 1 = tcgen05 tensor cores (3xTF32; for products of at least 4 x 8 output
 * tiles the operands are packed once per call into split tile images that
 * bulk copies stream through a four-stage ring, smaller ones split their
 * operands in registers), 2 = tcgen05 with operands split in registers always. No reference counterpart: the reference's
 * GEMMs run inside LAPACK's getrf/getrs (beyn.jl:270-280). */
qbg_status qbg_cgemm_c64(int32_t engine, int32_t M, int32_t N, int32_t K, const float* alpha, const float* A,
                         int64_t lda, const float* B, int64_t ldb, const float* beta, float* C, int64_t ldc,
                         int32_t batch);

/* Complex128 product on the tensor cores, for validation: C_b -= A_b B_b for
 * b < batch (host buffers, column-major complex128: A lda x K, B ldb x N, C
 * ldc x N per b; the M x K, K x N and M x N leading blocks are used). Both
 * operands are cut into eight 7-bit digits against the row maxima of A and the
 * column maxima of B; the digit products are exact on the tensor cores and
 * summed in double-float (~2^-56 of max|A_i.| max|B_.j| per term). The FP64 LU
 * runs its blocked updates through the same routine. No reference
 * counterpart: the reference's products run inside LAPACK (beyn.jl:270-280). */
qbg_status qbg_zgemm_sub_tc(int32_t M, int32_t N, int32_t K, const double* A, int64_t lda, const double* B,
                            int64_t ldb, double* C, int64_t ldc, int32_t batch);

/* Refinement residual, for validation: R_b = V_b - (Th_b + Tl_b) X_b for b < batch
 * (host buffers, column-major; Th, Tl: n x n complex64 per b, Tl may be NULL;
 * X, V, R: n x L complex128 per b), rmax = max |re R| + |im R|. engine 0 =
 * tensor cores (exact digit products of seven 7-bit digits), 1 = compensated
 * FP32 on CUDA cores, 2 = tensor cores from the leading six digits (the
 * refinement's first residual, ~2^-40 of the row and column scales).
 * No reference counterpart (the reference has no refinement). */
qbg_status qbg_residual_c64(int32_t engine, int32_t n, int32_t L, int32_t batch, const float* Th, const float* Tl,
                            const double* X, const double* V, double* R, double* rmax);

/* Selects the complex64 GEMM engine (0, 1 or 2 as above) for later calls,
 * process-wide; the default is 1. No reference counterpart. */
qbg_status qbg_set_gemm_engine(int32_t engine);

/* Number of CUDA kernels this library has launched in the process so far
 * (diagnostic; no reference counterpart). */
qbg_status qbg_launch_count(uint64_t* count);

/* Device memory cache. Every library buffer comes from a caching allocator:
 * freed blocks are kept for later requests of the same size class (reuse
 * waits for the stream work that last used a block), up to QBG_POOL_BYTES
 * bytes (environment; default a quarter of device memory; 0 disables it).
 * qbg_pool_release returns every cached block to the driver (for callers that
 * share the device with another allocator); qbg_pool_stats reports the cached
 * and live bytes and the reuse hits / driver allocations so far (any pointer
 * may be NULL). No reference counterpart (Julia's GC owns the reference's
 * host arrays). */
qbg_status qbg_pool_release(void);
qbg_status qbg_pool_stats(uint64_t* cached_bytes, uint64_t* live_bytes, uint64_t* hits, uint64_t* misses);

#ifdef __cplusplus
}
#endif
#endif
