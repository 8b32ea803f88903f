/*
 * frico_gpu.h -- C-ABI of the GB300 (sm_103a) Method-of-Moments hot path.
 *
 * The entry points replace FRICO's solver free functions one for one:
 *
 *   compute_matrix / compute_matrix_approx   src/emw_solver.h:85-86,  src/emw_solver.cpp:45-220
 *   update_rhs(delta_gap | plane_wave)       src/emw_solver.h:87-88,  src/emw_solver.cpp:352-416
 *   reorient_deltagap_edges                  src/emw_solver.h:90,     src/emw_solver.cpp:222-350
 *   solve_general / solve_symmetric          src/lapack_wrappers.h:28-35
 *   run_context (fill, rhs, solve, lumping)  src/emw_solver.h:92-167
 *   eval_fields (point and point-set forms)  src/emw_postpro_common.h:33-34
 *   compute_port_values, compute_gain        src/emw_ana_antenna.cpp:33-105
 *   bistatic_RCS_unit_Ei + its 359-pt loop   src/emw_ana_bistatic_rcs.cpp:62-118
 *   make_function_space + connectivity       src/rwg_basis.h:112, src/input_gmsh.cpp:216-322
 *
 * Conventions
 *   - Complex numbers are two doubles {re, im} (layout of std::complex<double>);
 *     matrices are column-major, entry (row j, col i) at j + i*ld, exactly as
 *     FRICO's Eigen zdmatrix stores Z(jbf.matrix_index, ibf.matrix_index).
 *   - Every function returns an int status (FRICO_GPU_OK or a negative code);
 *     nothing aborts, nothing throws across the boundary.
 *   - A context is used from one host thread at a time. Z, the LU factors,
 *     right-hand sides and currents stay resident on the device; host output
 *     pointers are optional (NULL = keep on device only).
 *   - Host pointers may be pageable or pinned.
 */
#ifndef FRICO_GPU_H
#define FRICO_GPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------- */
#define FRICO_GPU_OK          0
#define FRICO_GPU_EINVAL     -1   /* bad argument (FRICO: assert / invalid_argument) */
#define FRICO_GPU_ESINGULAR  -2   /* exactly-zero pivot; *info holds the LAPACK info */
#define FRICO_GPU_ETIMEOUT   -3   /* a bounded device-side wait gave up             */
#define FRICO_GPU_ENOMEM     -4   /* device allocation failed                       */
#define FRICO_GPU_ECUDA      -5   /* other CUDA runtime error                       */
#define FRICO_GPU_ESTATE     -6   /* call out of order (e.g. solve before fill)     */
#define FRICO_GPU_ENOCONV    -7   /* mixed-precision refinement did not converge    */
#define FRICO_GPU_EMESH      -8   /* mesh connectivity error (lonely / multiple)    */

/* ---- enums ---------------------------------------------------------- */
#define FRICO_PREC_FP64       0   /* complex128 fill, LU and solve (the drop-in)     */
#define FRICO_PREC_MIXED      1   /* complex64 LU + FP64 residual refinement        */

#define FRICO_EDGE_LENGTH_XY   0  /* FRICO's measure(edge): hypot(dx, dy)           */
#define FRICO_EDGE_LENGTH_TRUE 1  /* full 3-D length                                */

#define FRICO_HPHASE_COMPAT    0  /* H kernel with exp(+jkR) as eval_fields has it  */
#define FRICO_HPHASE_PHYSICAL  1  /* H kernel with exp(-jkR)                        */

#define FRICO_GAIN_XY 0
#define FRICO_GAIN_YZ 1
#define FRICO_GAIN_XZ 2

typedef struct frico_c128 { double re, im; } frico_c128;

/* Mirrors frico::rwg_basis_function (src/rwg_basis.h:41-52). */
typedef struct frico_rwg {
    double  Aminus;          /* area of T-  (0.5 |e0 x e1|)                  */
    double  Aplus;           /* area of T+                                   */
    int64_t itminus;         /* index of T-                                  */
    int64_t itplus;          /* index of T+                                  */
    double  pminus[3];       /* vertex of T- opposite to the edge            */
    double  pplus[3];        /* vertex of T+ opposite to the edge            */
    double  length;          /* edge length (see FRICO_EDGE_LENGTH_*)        */
    int64_t edge_index;      /* index in the sorted edge list                */
    int64_t matrix_index;    /* row/column of Z                              */
    int32_t has_interface;   /* 1 if the edge lies on a tagged curve         */
    int32_t interface_tag;   /* that curve's tag                             */
} frico_rwg;

/* Mirrors frico::maxwell::config (src/emw_solver.h:41-53), plus GPU knobs. */
typedef struct frico_gpu_options {
    int32_t degree;          /* Dunavant degree, 0..20 (0 behaves as 1)      */
    int32_t approx;          /* 1: compute_matrix_approx (-A)                */
    int32_t force_symmetry;  /* 1: Z <- (Z + Z^T)/2 before the solve (-S)    */
    int32_t precision;       /* FRICO_PREC_*                                 */
    int32_t h_phase_mode;    /* FRICO_HPHASE_*                               */
    int32_t max_refine_iters;/* mixed precision: refinement sweeps (<=0: 30) */
    double  refine_tol;      /* mixed precision: stop at ||r||/||b|| <= tol (<=0: 1e-12) */
    double  Z0;              /* reference impedance for gamma/SWR (-Z)       */
    int32_t profile_kernels; /* 1: CUDA-event timing of every LU update GEMM */
    int32_t gemm_engine;     /* complex64 trailing update: FRICO_GEMM_AUTO or FRICO_GEMM_SIMT */
    int32_t pivoting;        /* FRICO_PIVOT_* (mixed precision only; FP64 always pivots) */
    int32_t refine_mode;     /* FRICO_REFINE_* (mixed precision only)        */
    int32_t residual_mode;   /* FRICO_RESIDUAL_* (mixed precision refinement) */
    int64_t wait_limit_cycles;/* limit, in SM clock cycles, of every device-side wait on another
                                 CTA (chained triangular solves, the pivoted panel's grid
                                 barrier); <= 0: 4e9 (about 2 s). A wait that runs out ends its
                                 kernel, which returns FRICO_GPU_ETIMEOUT; the context stays
                                 usable. The tensor-core GEMM waits only on its own TMA copies
                                 and MMAs and keeps its fixed limit of 4e9 cycles. */
    int32_t fields_engine;   /* FRICO_FIELDS_*: E of many right-hand sides (eval_fields_multi) */
} frico_gpu_options;

#define FRICO_FIELDS_AUTO   0  /* mixed precision: E of >= 8 columns over >= 2^24 (point, triangle) pairs as
                                  tensor-core GEMMs (tcgen05 3xTF32, FP64 phase, double-float sums);
                                  otherwise, FP64 precision and H: the direct kernels */
#define FRICO_FIELDS_DIRECT 1  /* direct (point, triangle) kernels: FP64, or double-float for mixed */
#define FRICO_FIELDS_GEMM   2  /* E as tensor-core GEMMs whatever the precision (error if unavailable) */

#define FRICO_REFINE_AUTO    0  /* classical refinement, GMRES (max(120, 2 x max_refine_iters) iterations) when it contracts slowly */
#define FRICO_REFINE_CLASSIC 1  /* classical refinement only                                           */

#define FRICO_RESIDUAL_AUTO 0  /* b - Z x in double-float on the FP32 pipe (FP64 Z split into FP32 pairs); FP64 if an entry is out of its range */
#define FRICO_RESIDUAL_FP64 1  /* b - Z x on the FP64 pipe                                                          */

#define FRICO_PIVOT_AUTO    0  /* mixed: no interchanges, partial pivoting if that fails */
#define FRICO_PIVOT_PARTIAL 1  /* LAPACK zgetrf partial pivoting                        */
#define FRICO_PIVOT_NONE    2  /* no interchanges (refinement failure is an error)      */

#define FRICO_GEMM_AUTO   0  /* tcgen05 3xTF32 on sm_103, SIMT otherwise */
#define FRICO_GEMM_SIMT   1  /* CUDA-core FP32 complex GEMM               */
#define FRICO_GEMM_TC     2  /* tcgen05 3xTF32 (error if unavailable)     */
#define FRICO_GEMM_TC_F16 3  /* tcgen05; the unpivoted LU's block columns with 3xFP16 operands
                                scaled by powers of two, other updates 3xTF32 (error if unavailable) */

typedef struct frico_c64 { float re, im; } frico_c64;

/* Port values (src/emw_ana_antenna.h:31-38). */
typedef struct frico_port_values {
    frico_c128 voltage, current, power, impedance, gamma;
    double     swr;
} frico_port_values;

/* Per-stage device times of the last calls, CUDA events on the context stream. */
typedef struct frico_gpu_stats {
    double fill_ms, rhs_ms, factor_ms, solve_ms, refine_ms, lump_ms, fields_ms;
    int32_t refine_iters;
    double  refine_residual;     /* final ||b - Z x|| / ||b|| (FP64 sums; products per residual_mode) */
    int64_t n, ntri, nrhs;
    int64_t green_evals;         /* Green-function evaluations of last fill */
    int64_t kernel_launches;     /* kernels launched by this context so far */
    int64_t gemm_launches;       /* LU trailing-update launches timed (profile_kernels) */
    double  gemm_ms;             /* their summed CUDA-event time            */
    double  gemm_flops;          /* their algorithmic real flops (8 m n k)  */
    double  gemm_bytes;          /* their algorithmic bytes: C read+write + L, U reads */
    int32_t pivoting_used;       /* FRICO_PIVOT_PARTIAL / _NONE of the last factorisation */
    int32_t precision_used;      /* FRICO_PREC_FP64 when a mixed solve fell back to FP64 LU */
} frico_gpu_stats;

typedef struct frico_gpu_ctx frico_gpu_ctx;

/* ---- host-side mesh front end (no device work) ------------------------
 * Builds FRICO's connectivity and RWG table from a triangle soup, as
 * load_from_gmsh + compute_connectivity + make_function_space do
 * (src/input_gmsh.cpp:216-406, src/rwg_basis.cpp:27-68):
 *   edges sorted by (min vertex, max vertex) and deduplicated; T- is the lower
 *   triangle index; curves (1-D elements, tagged) that coincide with interior
 *   edges become interfaces; unused vertices are compacted away.
 * Inputs: nv vertices xyz[3*nv]; nt triangles tri[3*nt] (0-based vertex ids);
 * ncurve tagged segments curve[2*ncurve], curve_tag[ncurve] (may be 0/NULL).
 * Outputs: rwg[capacity], *n_rwg; rwg_edge_vertices[2*capacity] (the two
 * compacted vertex ids of each RWG edge, may be NULL); vertices_out[3*nv]
 * (compacted, may be NULL), *nv_out; tri_out[3*nt] (re-indexed, may be NULL).
 * Errors: FRICO_GPU_EMESH for an edge shared by >2 triangles or a curve segment
 * that is not an edge of any triangle; FRICO_GPU_EINVAL if capacity is short
 * (then *n_rwg holds the size needed). */
int frico_gpu_make_function_space(int64_t nv, const double* xyz,
                                  int64_t nt, const int64_t* tri,
                                  int64_t ncurve, const int64_t* curve, const int32_t* curve_tag,
                                  int32_t edge_length_mode,
                                  frico_rwg* rwg, int64_t capacity, int64_t* n_rwg,
                                  int64_t* rwg_edge_vertices,
                                  double* vertices_out, int64_t* nv_out, int64_t* tri_out);

/* Delta-gap orientation signs (src/emw_solver.cpp:222-350). xyz/tri are the
 * compacted mesh, tri_tag[nt] the surface tags, rwg[n] the RWG table and
 * rwg_edge_vertices[2*n] the vertex ids of each RWG edge (as returned above).
 * Writes signs[n] (only the feed entries are meaningful) and *applied = 1 when
 * the reorientation ran (otherwise signs are all +1). */
int frico_gpu_reorient_deltagap(int64_t nv, const double* xyz, const int64_t* tri,
                                const int32_t* tri_tag, int64_t n, const frico_rwg* rwg,
                                const int64_t* rwg_edge_vertices, int32_t n_itf,
                                const int32_t* itf_tags, int32_t force,
                                double* signs, int32_t* applied);

/* ---- context ---------------------------------------------------------- */
int frico_gpu_ctx_create(frico_gpu_ctx** ctx, int device, const frico_gpu_options* opt);
int frico_gpu_ctx_destroy(frico_gpu_ctx* ctx);
int frico_gpu_set_options(frico_gpu_ctx* ctx, const frico_gpu_options* opt);
const char* frico_gpu_last_error(frico_gpu_ctx* ctx);
/* The CUDA stream (cudaStream_t) every kernel of this context runs on. */
int frico_gpu_get_stream(frico_gpu_ctx* ctx, void** stream);

/* Upload mesh + RWG table (the state FRICO keeps in `simulation`). */
int frico_gpu_set_mesh(frico_gpu_ctx* ctx, int64_t nv, const double* xyz,
                       int64_t nt, const int64_t* tri,
                       int64_t n, const frico_rwg* rwg);

/* compute_matrix / compute_matrix_approx at `freq` Hz. Z stays on the device;
 * if Z_out != NULL it is also copied there (column-major, leading dim ldz >= n). */
int frico_gpu_fill(frico_gpu_ctx* ctx, double freq, frico_c128* Z_out, int64_t ldz);

/* Replaces the matrix argument A of solve_general / solve_symmetric
 * (src/lapack_wrappers.h:10-19) for a Z the caller assembled itself: upload the
 * n x n complex matrix (column-major, leading dim ldz >= n, n = the mesh's RWG
 * count) in place of a fill; the next frico_gpu_solve factors it (for
 * FRICO_PREC_MIXED, a complex64 copy refined against this FP64 Z).
 * freq (Hz, > 0) is the frequency Z belongs to, as freq_context::frequency
 * holds it beside Z (src/emw_solver.h:57-75): lumping and field evaluation of
 * the solution use it.
 * With approx or force_symmetry set, FRICO solves with solve_symmetric
 * (zsytrf/zsytrs, uplo = 'U', src/lapack_wrappers.cpp:135-177), which reads
 * only the upper triangle of A: the lower triangle is then taken as the
 * transpose of the upper one, so a non-symmetric Z gives FRICO's answer. */
int frico_gpu_set_matrix(frico_gpu_ctx* ctx, double freq, const frico_c128* Z, int64_t ldz);

/* Set the right-hand-side count (columns of V); resets V to zero. */
int frico_gpu_set_nrhs(frico_gpu_ctx* ctx, int32_t nrhs);
/* update_rhs(delta_gap): V[:,col] += (-j l/(omega mu0)) V0 sign on feed edges.
 * signs may be NULL (all +1). */
int frico_gpu_rhs_delta_gap(frico_gpu_ctx* ctx, double freq, int32_t col,
                            int32_t n_itf, const int32_t* itf_tags,
                            frico_c128 V0, const double* signs);
/* update_rhs(plane_wave): Dunavant-integrated <f, E_inc> / (-j omega mu0). */
int frico_gpu_rhs_plane_wave(frico_gpu_ctx* ctx, double freq, int32_t col,
                             double theta, double phi, frico_c128 Etheta, frico_c128 Ephi);
/* Upload / download V (n x nrhs, column-major, ld >= n). */
int frico_gpu_set_rhs(frico_gpu_ctx* ctx, int32_t nrhs, const frico_c128* V, int64_t ldv);
int frico_gpu_get_rhs(frico_gpu_ctx* ctx, frico_c128* V, int64_t ldv);

/* solve_general: factor the resident Z (LAPACK zgetrf semantics, partial
 * pivoting by max |re|+|im|) and solve Z I = V for all nrhs columns.
 * *info: 0, or k>0 for an exactly-zero pivot in column k (1-based), as zgetrf.
 * I_out (n x nrhs, ld ldi) optional. With FRICO_PREC_MIXED the factorisation
 * is complex64 and the currents are refined against the FP64 Z; with
 * FRICO_PIVOT_AUTO a system the complex64 factors cannot refine (too
 * ill-conditioned, e.g. an electrically small antenna) is re-solved with the
 * FP64 LU (stats.precision_used = FRICO_PREC_FP64). */
int frico_gpu_solve(frico_gpu_ctx* ctx, frico_c128* I_out, int64_t ldi, int32_t* info);
/* Download the LU factors (FP64 path: LAPACK layout) and 1-based ipiv. */
int frico_gpu_get_factors(frico_gpu_ctx* ctx, frico_c128* LU, int64_t ld, int32_t* ipiv);

/* run_context's current lumping for RHS column `col` (src/emw_solver.h:137-164):
 * tri_AJ[nt*3] (row-major rows of 3), tri_AdivJ[nt], tri_J[nt*3]; all optional. */
int frico_gpu_lump_currents(frico_gpu_ctx* ctx, int32_t col,
                            frico_c128* tri_AJ, frico_c128* tri_AdivJ, frico_c128* tri_J);

/* eval_fields at npts points P[3*npts] for RHS column `col` (after lumping).
 * E[3*npts], H[3*npts] (row-major rows of 3). */
int frico_gpu_eval_fields(frico_gpu_ctx* ctx, int32_t col, int64_t npts, const double* P,
                          frico_c128* E, frico_c128* H);

/* Allocation-free form of frico_gpu_eval_fields; no counterpart in FRICO.
 * It serves callers that cannot let the library allocate device memory while
 * they run: an application whose own memory pool holds the device memory, or
 * a post-processing loop that must not pay cudaMalloc's device-wide
 * synchronisation. P_dev[3*npts] (points), E_dev[3*npts], H_dev[3*npts]
 * (row-major rows of 3; either may be NULL) are device memory of the
 * context's device; anything else is EINVAL. The kernels store E and H as
 * 16-byte complex values and read P as doubles: E_dev and H_dev must be
 * 16-byte aligned and P_dev 8-byte aligned, else EINVAL (checked before any
 * launch, so a misaligned view never reaches the GPU). npts <= 43690: the partial sums
 * use one fixed 4 MiB device array per device, and larger npts is EINVAL.
 * The currents of `col` must already be lumped (frico_gpu_lump_currents),
 * else ESTATE. The kernels are queued on the context stream and the call
 * returns without waiting: E_dev/H_dev are valid once that stream reaches
 * them. The scratch array is shared by every context on the device, so calls
 * whose kernels overlap on the GPU race. The first call on each device looks
 * up the scratch address (which may load the library's device code): make
 * it before any stream capture. That address is cached per device for the
 * life of the process: after cudaDeviceReset on a device the cache is stale,
 * so do not call this entry point again in that process. */
int frico_gpu_eval_fields_noalloc(frico_gpu_ctx* ctx, int32_t col, int64_t npts,
                                  const double* P_dev, frico_c128* E_dev, frico_c128* H_dev);

/* ---- batched frequency sweep ------------------------------------------
 * FRICO's per-frequency loop (do_sweep, src/emw_ana_antenna.cpp:236-282 and
 * src/emw_ana_bistatic_rcs.cpp:121-160, over the contexts init_sweep makes,
 * src/emw_solver.cpp:460-468), run as independent concurrent lanes: each lane
 * is a sub-context on the context's device with its own stream and buffers,
 * driven by its own host thread, and takes the next frequency when it is done
 * (fill -> right-hand sides -> factor + solve -> port values -> fields). Every
 * frequency runs exactly the kernels of the single-frequency calls, so its
 * results equal a frico_gpu_fill/solve/... sequence at that frequency.
 *
 * Right-hand sides per frequency (nrhs = (n_itf > 0) + n_pw), in this order:
 * the delta gap on itf_tags (V0, signs as frico_gpu_rhs_delta_gap), then the
 * plane waves pw[6*p .. 6*p+5] = {theta, phi, Re Etheta, Im Etheta, Re Ephi,
 * Im Ephi}.
 * Outputs (each optional): port_out[nfreq] (needs n_itf > 0);
 * I_out[nfreq][nrhs][n] (currents, column-major per frequency);
 * E_out[nfreq][nrhs][npts][3] (E at the npts points P[3*npts]).
 * lanes: number of concurrent frequencies; 0 chooses it (by timing the first
 * frequencies of a long sweep, else from N). The lane contexts are kept with
 * ctx for later sweeps and freed by frico_gpu_ctx_destroy.
 * Mixed precision: frequencies are visited from the highest down; once three
 * have fallen back to the FP64 LU, every frequency at or below the third is
 * solved in FP64 directly (report->fp64_direct): lower frequencies are more
 * ill-conditioned (EFIE low-frequency regime).
 * Returns the first hard error (with the frequency in the message); a
 * refinement that did not reach its tolerance at some frequency is counted in
 * report->not_converged and the call returns FRICO_GPU_ENOCONV after finishing
 * every frequency. */
typedef struct frico_sweep_report {
    double  wall_ms;             /* host wall-clock of the call                     */
    double  fill_ms, rhs_ms, factor_ms, solve_ms, refine_ms, lump_ms, fields_ms;
                                 /* device time per stage, summed over frequencies  */
    int32_t lanes;               /* concurrent lanes of the bulk of the sweep       */
    int32_t autotuned;           /* 1 when the lane count was chosen by timing      */
    int32_t nrhs;
    int32_t max_refine_iters;
    double  max_refine_residual;
    int32_t partial_pivot_fallbacks;  /* mixed path: frequencies factored with pivoting */
    int32_t not_converged;       /* frequencies whose refinement missed its tolerance */
    int32_t fp64_fallbacks;      /* mixed path: frequencies that fell back to the FP64 LU */
    int32_t fp64_direct;         /* mixed path: frequencies at or below a fallback, solved in FP64 */
    int64_t kernel_launches;     /* kernels launched by all lanes during the call   */
} frico_sweep_report;

int frico_gpu_sweep(frico_gpu_ctx* ctx, int32_t nfreq, const double* freqs,
                    int32_t n_itf, const int32_t* itf_tags, frico_c128 V0, const double* signs,
                    int32_t n_pw, const double* pw,
                    int64_t npts, const double* P, int32_t lanes,
                    frico_port_values* port_out, frico_c128* I_out, frico_c128* E_out,
                    frico_sweep_report* report);

/* ---- adjoint sensitivities ---------------------------------------------
 * No counterpart in FRICO (it computes no derivatives): the reverse mode of its
 * antenna pipeline at one frequency, for the fill it runs by default (degree-1
 * quadrature with the sub-triangle split, src/emw_solver.cpp:45-142). Runs
 * fill -> delta-gap RHS -> solve at `freq` (the context's precision), then one
 * transposed solve with the same factors for the two adjoint vectors, and a
 * reverse pass over the fill on the GPU. Outputs the gradients of Re Zin,
 * Im Zin (Zin = V0 / sum_feed l_i s_i I_i, as compute_port_values) and of
 * |E(P_obs)|^2 (eval_fields' E) with respect to every vertex coordinate of
 * the mesh given to frico_gpu_set_mesh (grad_*[3*nv], each may be NULL), and
 * with respect to the frequency (in *out). edge_length_mode must be the one
 * the RWG lengths were made with (FRICO_EDGE_LENGTH_XY as FRICO does). */
typedef struct frico_adjoint_result {
    frico_c128 zin;              /* input impedance                         */
    frico_c128 e[3];             /* E(P_obs)                                */
    double     e2;               /* |E(P_obs)|^2                            */
    double     dzin_re_df, dzin_im_df, de2_df;   /* per Hz                */
} frico_adjoint_result;

int frico_gpu_adjoint(frico_gpu_ctx* ctx, double freq, int32_t n_itf, const int32_t* itf_tags,
                      frico_c128 V0, const double* signs, const double* P_obs,
                      int32_t edge_length_mode,
                      double* grad_zin_re, double* grad_zin_im, double* grad_e2,
                      frico_adjoint_result* out);

/* eval_fields for RHS columns [col0, col0 + ncols) at the same npts points:
 * E[ncols][npts][3], H[ncols][npts][3] (either may be NULL). One pass over
 * (point, triangle) pairs serves every column (the Green function is shared).
 * With fields_engine selecting GEMMs (and H not asked for), E comes from two
 * complex matrix products over the triangles on the tensor cores: the Green
 * function with the point's phase e^{-jk|P|} factored out, times the lumped
 * currents (errors of a few 1e-7 of |E|, against ~1e-12 for the direct kernels). */
int frico_gpu_eval_fields_multi(frico_gpu_ctx* ctx, int32_t col0, int32_t ncols, int64_t npts,
                                const double* P, frico_c128* E, frico_c128* H);
/* bistatic_RCS_unit_Ei at sph2rect(R, theta[i], phi[i]) for every column:
 * out[ncols][npts][2] = {sigma_VV, sigma_HH}. */
int frico_gpu_rcs_points_multi(frico_gpu_ctx* ctx, int32_t col0, int32_t ncols, double R, int64_t npts,
                               const double* theta, const double* phi, double* out);

/* compute_port_values for the delta gap on `itf_tags` (RHS column `col`). */
int frico_gpu_port_values(frico_gpu_ctx* ctx, int32_t col, int32_t n_itf,
                          const int32_t* itf_tags, frico_c128 V0, const double* signs,
                          frico_port_values* out);
/* compute_gain: 360 gains on `plane` at distance R for input power pwr. */
int frico_gpu_gain(frico_gpu_ctx* ctx, int32_t col, double pwr, double R,
                   int32_t plane, double* G360);
/* Bistatic RCS (src/emw_ana_bistatic_rcs.cpp:102-117): out[359*4] rows
 * {VV_theta, HH_theta, VV_phi, HH_phi} for angles 0..358 degrees. */
int frico_gpu_bistatic_rcs(frico_gpu_ctx* ctx, int32_t col, double R, double* out);
/* sigma_VV / sigma_HH at arbitrary (theta, phi) directions, radius R:
 * out[2*npts] = {VV, HH} per direction. */
int frico_gpu_rcs_points(frico_gpu_ctx* ctx, int32_t col, double R, int64_t npts,
                         const double* theta, const double* phi, double* out);

int frico_gpu_last_stats(frico_gpu_ctx* ctx, frico_gpu_stats* stats);

#ifdef __cplusplus
}
#endif
#endif /* FRICO_GPU_H */
