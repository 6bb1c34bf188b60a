/*
 * doug_gpu.h -- C ABI of the GB300 solve path for DOUG
 * (Domain decomposition On Unstructured Grids).
 *
 * One handle = one linear system A x = b and its two-level additive Schwarz
 * preconditioner (overlapping subdomain solves + smoothed-aggregation coarse
 * grid), solved by preconditioned conjugate gradients on one GPU.  All
 * pointers are plain host pointers unless the name says "device"; sizes are
 * ints; no call aborts the process: every call returns a dg_status and
 * dg_last_error() gives the message.  Handles are independent (no global
 * state), one handle per host thread.
 *
 * The entry points replace the following pieces of the reference (paths
 * relative to the DOUG source tree):
 *   dg_load_ctl / dg_set_option  -> CtrlData_initFromFile, util_actionOnCtrlArg
 *                                   (src/utils/DOUG_utils.F90:629-1150)
 *   dg_set_matrix_coo / dg_set_rhs -> ReadInSparseAssembled, Vect_ReadFromFile,
 *                                   parallelDistributeAssembledInput
 *                                   (src/datatypes/SpMtx/SpMtx_class.F90:410-453,
 *                                    src/datatypes/Vect.F90:840-947,
 *                                    src/components/Distribution_assm.F90:49-102)
 *   dg_set_elements, and dg_load_ctl with input_type 1
 *                                -> Mesh_initFromFile, Mesh_readFileFreelists,
 *                                   ElemMtxs_readAndDistribute and the one-process
 *                                   element assembly (src/datatypes/Mesh.F90:293-460,
 *                                   src/datatypes/ElemMtxs/ElemMtxs_distribute.F90:509-631,
 *                                   src/datatypes/ElemMtxs/ElemMtxs_assemble.F90:82-289)
 *   dg_set_partition             -> the partition import of the debug 4321
 *                                   path (src/components/Distribution_assm.F90:202-215)
 *   dg_setup                     -> Partitionings_aggr_InitFine/InitCoarse,
 *                                   CoarsePreconditioner_smooth_Init,
 *                                   FinePreconditioner_Init
 *                                   (src/main/aggr.F90:131-226)
 *   dg_solve / dg_solve_device   -> pcg_weigs (src/solvers/pcg.F90:289-462), including
 *                                   the lazy factorisations (src/solvers/subsolvers.F90:78-163)
 *   dg_write_solution            -> WriteSolutionToFile (src/utils/DOUG_utils.F90:1598-1700)
 *   dg_get_*                     -> parity export of aggregates, subdomains, R, AC
 *   the handle as a whole        -> the stale C extension API src/ext/C/doug_ext.h:4-13
 *                                   (opaque handles, caller-owned buffers), with size
 *                                   queries so callers never hard-code sizes.
 */
#ifndef DOUG_GPU_H
#define DOUG_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dg_handle dg_handle;

typedef enum {
  DG_OK = 0,
  DG_NOT_CONVERGED = 1,   /* maxit reached before the tolerance */
  DG_BREAKDOWN = 2,       /* p.q <= 0 or a NaN in the CG recurrences */
  DG_SINGULAR = 3,        /* a subdomain or coarse matrix is not positive definite */
  DG_BAD_INPUT = 4,       /* malformed control word, file or argument */
  DG_CUDA_ERROR = 5,      /* a CUDA call failed */
  DG_NO_DEVICE = 6,       /* no CUDA device */
  DG_NOT_READY = 7        /* call order: e.g. dg_solve before dg_setup */
} dg_status;

typedef struct {
  int iterations;             /* PCG iterations */
  double init_norm;           /* ||b - A x0||_2 */
  double final_norm;          /* ||r_k||_2 of the recurrence */
  double true_rel_residual;   /* ||b - A x||_2 / ||b - A x0||_2 (FP64 recomputed) */
  double cond_num;            /* Lanczos estimate lambda_max / lambda_min (FP64 path; 0 when the
                                 tridiagonal is degenerate: a zero alpha or a negative beta) */
  double t_setup_s;           /* host setup: aggregation, R, AC, symbolic analysis */
  double t_factor_s;          /* GPU numeric factorisations (subdomains + coarse) */
  double t_iterate_s;         /* GPU PCG iterations */
  double t_total_s;           /* factor + iterate (time to tolerance) */
  int n;                      /* unknowns */
  int nsubdomains;
  int ncoarse;                /* coarse unknowns (fine aggregates) */
  int gpu_launches;           /* kernels launched by the last solve */
  long long factor_nnz;       /* stored factor entries (subdomains) */
  double factor_gflop;        /* partial-Cholesky flops of the subdomain factors */
  /* phase timings, filled when the control word "profile 1" is set (CUDA
   * events around each phase; adds a little overhead, so off by default) */
  double t_subsolve_s;        /* subdomain forward+backward solves, all iterations */
  double subsolve_bytes;      /* algorithmic bytes of one subdomain solve (factor read twice) */
  double t_coarse_s;          /* restriction + coarse solves, all iterations */
  double coarse_bytes;        /* algorithmic bytes of one coarse solve */
  double t_spmv_s;            /* fused direction update + SpMV, all iterations */
  double spmv_bytes;          /* algorithmic bytes of one SpMV */
} dg_stats;

dg_status dg_create(dg_handle **h);
void dg_destroy(dg_handle *h);
const char *dg_last_error(const dg_handle *h);

/* Control words, same names and parsing as a DOUG control file ("name value";
 * the first value given for a name wins, as in the reference).  Extension
 * words of this library: precision (0 = FP64, 1 = mixed FP32 subdomain
 * factors with flexible CG and FP64 residual replacement), replace_every,
 * omega (prolongator smoother weight; the reference hard-codes 1/3),
 * reuse_factors (1: solves after the first keep the numeric factors, for
 * adjoint solves and further right-hand sides of the same matrix). */
dg_status dg_set_option(dg_handle *h, const char *name, const char *value);
/* Parse a control file and read the input files it names: input_type 2,
 * the assembled matrix + optional RHS; input_type 1, the info, freedom-list
 * and element-matrix files (assembled as one DOUG process assembles them).
 * Relative names resolve against the control file's folder. */
dg_status dg_load_ctl(dg_handle *h, const char *path);

/* Assembled matrix as 1-based COO triplets in any order (0-based accepted,
 * as in the reference's reader); duplicates are summed. */
dg_status dg_set_matrix_coo(dg_handle *h, int n, int nnz, const int *rows, const int *cols,
                            const double *vals);
/* Elemental input held in memory: nell elements over ngf global freedoms;
 * element e has the 1-based freedoms efree[eptr[e] .. eptr[e+1]), its
 * nf x nf matrix (nf = eptr[e+1] - eptr[e]) column by column in emat (the
 * elements one after another) and its right-hand side in erhs (laid out
 * like efree).  Assembled exactly like the elemental input files: the
 * unknowns are the used freedoms in increasing order (an element may have
 * no freedoms), entries sum the
 * elements' non-zero values in element order, b sums the elements' RHS. */
dg_status dg_set_elements(dg_handle *h, int nell, int ngf, const int *eptr, const int *efree,
                          const double *emat, const double *erhs);
/* Node coordinates of the elements' mesh (after dg_set_elements; dg_load_ctl
 * reads them from coords_file / freemap_file): coordinate d of node v
 * (1-based) at coords[(v-1)*nsd + d], nsd 2 or 3, and the node of every
 * global freedom f (1-based) at freemap[f-1] (ngf entries).  Replaces the
 * reference's Mesh_readFileCoords / Mesh_readFileFreemap
 * (src/datatypes/Mesh.F90:470-520); the geometric coarse grid of doug_geom
 * (control word "executable geom" with levels 2) is built from them. */
dg_status dg_set_node_geometry(dg_handle *h, int nsd, int nnode, const double *coords, const int *freemap);
/* Right-hand side (n values); without one, b = 1 as in the reference. */
dg_status dg_set_rhs(dg_handle *h, const double *b);
/* Batched independent systems (no reference counterpart: one reference run
 * solves one system).  nsys systems, system k with n_sys[k] unknowns and
 * nnz_sys[k] triplets; rows/cols/vals hold the triplets of all systems one
 * after the other, indices 1-based within each system; b (may be NULL: b = 1)
 * the right-hand sides one after the other.  Every system gets the setup of
 * its own one-process run (aggregation, R, AC, subdomains) and its own PCG
 * (scalars, stopping test, iteration count); the factorisations, the
 * preconditioner applications and the products of all systems share the
 * kernel launches.  dg_solve then takes and returns the concatenated vectors.
 * A partition vector cannot be combined with it. */
dg_status dg_set_systems(dg_handle *h, int nsys, const int *n_sys, const long long *nnz_sys, const int *rows,
                         const int *cols, const double *vals, const double *b);
/* Per-system results of the last batched solve, or per right-hand side of
 * the last dg_solve_multi (each pointer may be NULL; one entry each): iterations, status (DG_OK, DG_NOT_CONVERGED,
 * DG_BREAKDOWN), true relative residual ||b - A x|| / ||b|| and the wall time
 * from the start of the solve to the end of the system's last iteration. */
dg_status dg_get_system_stats(const dg_handle *h, int *iterations, int *status, double *rel_residual,
                              double *seconds);

/* Optional subdomain partition: part[i] in 1..nparts for every unknown.
 * Replaces the coarse-aggregate subdomains of the one-process path. */
dg_status dg_set_partition(dg_handle *h, const int *part, int nparts);

/* Aggregation, restriction, coarse matrix, subdomains, symbolic analysis and
 * device upload.  Must follow the matrix. */
dg_status dg_setup(dg_handle *h);

/* Autotuner (no reference counterpart: the reference's factorisation has no
 * batch parameters).  Times full solves (factorisations + PCG) of the stored
 * RHS over a small grid of the control words nd_leaf, panel_rows, fwd_task_kb
 * and lean_task_kb, keeps the fastest and leaves the handle set up with it.
 * The host aggregation, restriction and coarse matrix are built once.
 * best_seconds (may be NULL) receives the fastest factor + iterate time and
 * chosen (may be NULL) the four words nd_leaf, panel_rows, fwd_task_kb,
 * lean_task_kb in that order. */
dg_status dg_autotune(dg_handle *h, double *best_seconds, int *chosen);

/* Solve with host buffers (b may be NULL: the stored RHS is used).  x must
 * hold n doubles.  stats may be NULL. */
dg_status dg_solve(dg_handle *h, const double *b, double *x, dg_stats *stats);
/* Same with device pointers on the given CUDA stream (NULL: default stream). */
dg_status dg_solve_device(dg_handle *h, const double *d_b, double *d_x, dg_stats *stats,
                          void *cuda_stream);
/* Several right-hand sides of the handle's matrix solved together (no
 * reference counterpart: the reference solves one right-hand side per run).
 * B and X hold nrhs vectors of n doubles one after the other (B may be NULL:
 * the stored right-hand side for every vector).  Each right-hand side runs its
 * own PCG (own scalars, stopping test and iteration count, as dg_solve); the
 * factorisations are shared and every preconditioner, product and vector
 * kernel covers all of them.  dg_get_system_stats reports per right-hand side;
 * stats carries the largest iteration count and residual.  Not with batched
 * systems, fine_method 2 or elemental_matvec 1. */
dg_status dg_solve_multi(dg_handle *h, int nrhs, const double *B, double *X, dg_stats *stats);
dg_status dg_solve_multi_device(dg_handle *h, int nrhs, const double *d_B, double *d_X, dg_stats *stats,
                                void *cuda_stream);
/* Write x with the control file's solution_file / solution_format. */
dg_status dg_write_solution(dg_handle *h, const double *x);

/* FP64 true residual of a caller-held CSR matrix on the device:
 * r = b - A x and *d_norm2 = ||r||_2^2 (all device pointers, 0-based CSR with
 * 64-bit row pointers), on the given CUDA stream.  The same arithmetic as the
 * reference's initial residual (src/solvers/pcg.F90:364-367) and doug_geom's
 * final residual check (src/main/geom.F90:135-142).  Uses stream-ordered
 * scratch (cudaMallocAsync) for the partial sums. */
dg_status dg_residual_csr(int n, const long long *d_rowptr, const int *d_col, const double *d_val,
                          const double *d_x, const double *d_b, double *d_r, double *d_norm2,
                          void *cuda_stream);

/* The same residual without any device allocation, for callers that cannot
 * allocate at this point (a caller-owned memory pool that forbids other
 * allocations, a stream being captured into a CUDA graph, a loop that must
 * not pay for cudaMalloc's synchronisation).  This entry point has no
 * counterpart in the reference.  Its partial sums use a fixed 512 KiB array
 * inside the library that every GPU loading the library keeps until the
 * process exits; n may be at most 67,108,864 (65,536 partial sums of 1,024
 * rows), larger n returns DG_BAD_INPUT.  The first call on each device looks
 * up the array's device address (the calling thread's current device must be
 * the stream's device), so make that first call before any stream capture.
 * The address is kept per device and CUDA context: after a cudaDeviceReset
 * the next call (again outside any capture) looks it up in the new context.
 * All calls share the array: calls that overlap on the GPU (other streams,
 * other threads) race and must be serialised by the caller. */
dg_status dg_residual_csr_noalloc(int n, const long long *d_rowptr, const int *d_col,
                                  const double *d_val, const double *d_x, const double *d_b,
                                  double *d_r, double *d_norm2, void *cuda_stream);

/* Gradients through x = A^-1 b (the reference has no gradients).  Given the
 * adjoint solution d_lambda = A^-1 dL/dx (a second solve with the same
 * handle; with the option reuse_factors 1 it keeps the factors of the first)
 * and the solution d_x, both device vectors of n values:
 *   dg_grad_matrix   -> d_grad[k] = -lambda[row_k] x[col_k] for every input
 *                       triplet k of dg_set_matrix_coo / the control file
 *                       (dL/dA_ij; dL/db is lambda itself);
 *   dg_grad_elements -> d_grad[e] = dL/ds_e for a factor s_e scaling element
 *                       e's matrix (elemental input only): with A_e =
 *                       kappa_e K_e, dL/dkappa_e = d_grad[e] / kappa_e.
 * Both run on the given stream and return without waiting. */
dg_status dg_grad_matrix(dg_handle *h, const double *d_lambda, const double *d_x, double *d_grad,
                         void *cuda_stream);
dg_status dg_grad_elements(dg_handle *h, const double *d_lambda, const double *d_x, double *d_grad,
                           void *cuda_stream);

/* Setup phases of the last dg_setup, in seconds (no reference counterpart;
 * the reference prints its total setup time, src/main/aggr.F90:253-258):
 * the host part up to the fine aggregates (arrangement, scaling, strength,
 * aggregation), the restriction + Galerkin product (device time when they
 * ran on the GPU: *on_device = 1), and the whole dg_setup (host setup,
 * symbolic analysis and upload).  NULL pointers are skipped. */
dg_status dg_get_setup_phases(const dg_handle *h, double *aggregation_s, double *coarse_s, int *on_device,
                              double *total_s);

/* Size queries and parity export (1-based ids as in the reference). */
dg_status dg_get_sizes(const dg_handle *h, int *n, int *nagr_fine, int *nagr_coarse,
                       int *nsubdomains, long long *subdomain_total, int *R_nnz, int *AC_nnz);
dg_status dg_get_aggregates(const dg_handle *h, int *fine_num /* n */,
                            int *coarse_num /* nagr_fine */);
dg_status dg_get_subdomains(const dg_handle *h, long long *starts /* nsubd+1 */,
                            int *nodes /* subdomain_total */);
/* R and AC in the reference's final entry order (COO, 1-based). */
dg_status dg_get_restriction(const dg_handle *h, int *ri, int *rj, double *rv);
dg_status dg_get_coarse_matrix(const dg_handle *h, int *ci, int *cj, double *cv);
/* doug_geom with levels 2: the coordinates of the ncoarse coarse freedoms
 * that R and AC number (nsd per freedom, freedom after freedom; xyz may be
 * NULL to ask for the sizes); DG_NOT_READY otherwise. */
dg_status dg_get_coarse_coords(const dg_handle *h, int *nsd, int *ncoarse, double *xyz);
/* The matrix and right-hand side the handle holds (after dg_set_matrix_coo,
 * dg_set_elements or dg_load_ctl), as given or as assembled from elements:
 * 1-based COO in entry order.  NULL arrays are skipped (ask for n, nnz first). */
dg_status dg_get_input(const dg_handle *h, int *n, int *nnz, int *rows, int *cols, double *vals,
                       double *rhs);

#ifdef __cplusplus
}
#endif
#endif
