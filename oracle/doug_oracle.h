/*
 * doug_oracle.h -- CPU restatement of DOUG's solve path (TEST INFRASTRUCTURE ONLY).
 *
 * This library is the parity oracle for the GB300 solver.  Only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load it;
 * the product library never links or calls it.
 *
 * It restates, in plain C with 1-based arrays, the reference's np=1 path of
 * `doug_aggr` (src/main/aggr.F90:124-251): control-file parsing, assembled
 * input, strength of connection, aggregation, smoothed-aggregation
 * restriction, Galerkin coarse matrix, overlapping subdomains and PCG with the
 * two-level additive Schwarz preconditioner.  Exact subdomain / coarse solves
 * (UMFPACK LU in the reference) are done here by a nested-dissection
 * multifrontal Cholesky (spchol.h).
 *
 * Parity pin: the reference's fixtures tests/assembled/lap4x4 and
 * tests/assembled/lap16x16 (final solutions; see tests/test_oracle.py).
 */
#ifndef DOUG_ORACLE_H
#define DOUG_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Result of one oracle run (all arrays 0-based copies, owned by the result). */
typedef struct orc_result {
  int status;              /* 0 ok, <0 error (message in errmsg) */
  char errmsg[512];
  int n;                   /* unknowns */
  double *x;               /* solution (n) */
  double *b;               /* right-hand side used (n) */
  int iterations;
  double cond_num;
  double init_norm;        /* ||r0||_2 */
  double *res_hist;        /* ||r_k||_2, k=1..iterations */
  /* fine / coarse aggregates (1-based aggregate numbers per node, as DOUG) */
  int nagr_fine;
  int *aggr_fine;          /* n */
  int nagr_fine_full;
  int *aggr_fine_full;     /* n */
  int nagr_coarse;
  int *aggr_coarse;        /* nagr_fine */
  int nagr_coarse_full;
  int *aggr_coarse_full;   /* nagr_fine */
  /* subdomains: 1-based node lists in DOUG order */
  int nsubd;
  int *subd_starts;        /* nsubd+1, 0-based offsets */
  int *subd_nodes;         /* 1-based node numbers */
  /* restriction R (nagr x n) and coarse matrix AC, COO in DOUG's final order, 1-based */
  int R_nrows, R_ncols, R_nnz;
  int *R_i, *R_j; double *R_v;
  int AC_n, AC_nnz;
  int *AC_i, *AC_j; double *AC_v;
  /* effective parameters */
  int overlap, smoothers, levels, method;
  double strong1, strong2;
  int radius1, radius2, minasize1, maxasize1, minasize2, maxasize2;
  double tol;
  int maxit;
  double t_setup, t_factor, t_solve;
  /* doug_geom with levels 2: coordinates of the coarse freedoms that R and
   * AC number (cnsd x AC_n, coordinate after coordinate of each freedom) */
  int cnsd;
  double *cxyz;
} orc_result;

/* Run the full path from a DOUG control file.  `overrides` is a string of
 * "name value" lines applied before the file (DOUG keeps the first value of a
 * repeated word, so overrides win).  `workdir` resolves relative file names
 * (NULL: directory of the control file). */
int orc_run_ctl(const char *ctl_path, const char *overrides, orc_result **out);
/* The same with an imported partition of the unknowns (1-based part ids,
 * length n, nparts parts) in place of the default subdomains. */
int orc_run_ctl_part(const char *ctl_path, const char *overrides, const int *part, int nparts,
                     orc_result **out);
/* Elemental input files (input_type 1) assembled as one DOUG process does;
 * 1-based COO with the reference's flipped indices, malloc'ed (free with
 * orc_free_buffers). */
int orc_read_elemental(const char *info, const char *freel, const char *elemmat, int nblocks,
                       int *n, int *nnz, int **ii, int **jj, double **vv, double **rhs);
void orc_free_buffers(void *a, void *b, void *c, void *d);

/* Run the full path on an in-memory matrix given as COO triplets (1-based,
 * any order, as in the assembled text format), rhs (NULL -> b = 1),
 * control text (same syntax as a control file), and an optional partition
 * vector (1-based part ids, length n; NULL -> DOUG np=1 coarse-aggregate
 * subdomains). */
int orc_run_coo(int n, int nnz, const int *ii, const int *jj, const double *vv,
                const double *rhs, const char *ctl_text, const int *part,
                int nparts, orc_result **out);

/* Setup only (no PCG): aggregates, subdomains, R, AC. */
int orc_setup_coo(int n, int nnz, const int *ii, const int *jj, const double *vv,
                  const char *ctl_text, const int *part, int nparts,
                  orc_result **out);

/* Node geometry for coarse_method 3 (smoothed aggregation over nodal blocks
 * with rigid-body modes), used by the following runs: nsd coordinates per
 * node (nnode nodes) and the 1-based node of each of the n unknowns (a
 * node's unknowns ascending are its components).  nsd 0 clears it. */
void orc_set_geometry(int nsd, int nnode, const double *coords, int n, const int *unode);

void orc_free(orc_result *r);

/* File-format helpers (restated readers/writers). Return 0 on success. */
int orc_read_assembled(const char *path, int format, int *n, int *nnz,
                       int **ii, int **jj, double **vv);
int orc_read_vector(const char *path, int format, int n, double *x);
int orc_write_solution(const char *path, int format, int n, const double *x);

/* A setup kept for repeated solves: orc_session_new runs the setup (its
 * result carries the setup arrays and t_setup); each orc_session_solve runs
 * the numeric factorisations and the PCG on rhs (NULL -> b = 1), filling
 * x, iterations, res_hist, t_factor and t_solve. */
typedef struct orc_session orc_session;
int orc_session_new(int n, int nnz, const int *ii, const int *jj, const double *vv,
                    const char *ctl_text, const int *part, int nparts, orc_session **sess,
                    orc_result **out);
int orc_session_solve(orc_session *sess, const double *rhs, orc_result **out);
void orc_session_free(orc_session *sess);

/* Host threads for the factorisations, subdomain solves and vector loops
 * (default 1).  The results do not depend on the count. */
void orc_set_threads(int threads);

/* Exact solve of a sparse SPD system (nested dissection + multifrontal
 * Cholesky, spchol.h). */
int orc_spd_solve(int n, int nnz, const int *ii, const int *jj, const double *vv,
                  const double *b, double *x);

/* The same solver with the factorisation kept (NULL on failure). */
void *orc_spd_factor(int n, int nnz, const int *ii, const int *jj, const double *vv);
int orc_spd_solve_factored(void *fact, const double *b, double *x);
void orc_spd_free(void *fact);

/* Parse one control-file value the way DOUG does: i10 / f10.5 / l1. */
int orc_parse_i10(const char *s, int *out);
int orc_parse_f10_5(const char *s, double *out);
int orc_parse_l1(const char *s, int *out);

#ifdef __cplusplus
}
#endif
#endif
