/*
 * spchol.h -- exact sparse Cholesky of the oracle (TEST INFRASTRUCTURE ONLY).
 *
 * The reference factors every subdomain matrix and the coarse matrix with
 * UMFPACK (third-party, LGPL, version >= 4.4 per src/solvers/umfpack4wrap.c:6;
 * call sites src/solvers/Fact.F90:102-159, umfpack4wrap.c:196-256), which
 * orders with AMD and factors with dense frontal BLAS kernels.  UMFPACK is not
 * part of the reference tree, so this file restates the published method of
 * a fill-reducing exact sparse factorisation instead: nested dissection by
 * breadth-first level-set separators (George, SIAM J. Numer. Anal. 10 (1973)
 * 345-363; George & Liu, "Computer Solution of Large Sparse Positive Definite
 * Systems", 1981), elimination tree and column counts by row subtrees
 * (Liu, SIAM J. Matrix Anal. Appl. 11 (1990) 134-172), fundamental
 * supernodes and the multifrontal method (Duff & Reid, ACM TOMS 9 (1983)
 * 302-325).  Any exact solve of an SPD system agrees with UMFPACK's to
 * rounding, which is all the parity checks ask of it.
 *
 * Thread-safe: no global state; errors are returned, never longjmp'ed.
 */
#ifndef DOUG_SPCHOL_H
#define DOUG_SPCHOL_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct spchol spchol;

/* Factor the symmetric matrix given as 0-based COO triplets (both triangles
 * or one; entries with row >= column after the ordering are summed, as
 * umf4triplet2col sums duplicates).  Returns NULL and writes a message into
 * err on a non-positive pivot or when memory runs out. */
spchol *spchol_factor(int n, long nnz, const int *ii, const int *jj, const double *vv,
                      char *err, int errsz);
/* x = A^-1 b; work holds spchol_work_size(f) doubles.  b and x may alias. */
void spchol_solve(const spchol *f, const double *b, double *x, double *work);
long spchol_work_size(const spchol *f);
void spchol_free(spchol *f);
/* Stored factor entries (supernodal, including the upper zeros of the
 * diagonal blocks) and the floating-point operations of the factorisation. */
long spchol_nnz(const spchol *f);
double spchol_flops(const spchol *f);

#ifdef __cplusplus
}
#endif
#endif
