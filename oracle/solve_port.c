/*
 * ORACLE — test infrastructure only, never shipped or measured as the product.
 *
 * Restatement of the C++ driver solve_matrix() of GetDP's Sparskit backend
 * (contrib/Sparskit/Sparskit.cpp:108-634) for a matrix that is already in
 * CSR form (what csr_format, Sparskit.cpp:2186-2217, produces):
 *
 *   scaling (scale_matrix / scale_vector, :962-1060, :211-218)
 *   zero-row check (:220-223)
 *   RCMK renumbering via cmkreord + sortcol (:236-285)
 *   ILU0 / DIAGONAL / none (:299-465)
 *   RHS permutation (:469-471), initial guess 0 (:226)
 *   reverse-communication loop over cg/gmres/fgmres (:518-573)
 *   inverse permutation (:598-602) and column scaling (:631-632)
 *
 * It calls the Fortran-style routines restated in sparskit_port.c, exactly
 * as the reference's glue does, so a reference binary linked against that
 * file and this driver produce the same iterates.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#if defined(HAVE_ILU_FLOAT)
typedef float sscalar;
#else
typedef double sscalar;
#endif

void getdia_(int *, int *, int *, double *, int *, int *, int *, double *,
             int *, int *);
void diamua_(int *, int *, double *, int *, int *, double *, double *, int *,
             int *);
void amudia_(int *, int *, double *, int *, int *, double *, double *, int *,
             int *);
void cmkreord_(int *, double *, int *, int *, double *, int *, int *, int *,
               int *, int *, int *, int *, int *, int *);
void sortcol_(int *, double *, int *, int *, int *, double *);
void ilu0_(int *, double *, int *, int *, sscalar *, int *, int *, int *,
           int *);
void lusol_(int *, double *, double *, sscalar *, int *, int *);
void lutsol_(int *, double *, double *, sscalar *, int *, int *);
void amux_(int *, double *, double *, double *, int *, int *);
void atmux_(int *, double *, double *, double *, int *, int *);
void cg_(int *, double *, double *, int *, double *, double *);
void gmres_(int *, double *, double *, int *, double *, double *);
void fgmres_(int *, double *, double *, int *, double *, double *);

/* Sparskit.h:19-46 codes */
enum { SK_CG = 1, SK_GMRES = 8, SK_FGMRES = 9 };
enum { SK_NONE = 0, SK_ILU0 = 6, SK_DIAGONAL = 8 };

typedef struct {
  int algorithm, preconditioner, precond_position, scaling, renumbering;
  int krylov_size, nb_iter_max;
  double stopping_test;
} oracle_params;

/* Returns ipar(1) (0 = converged, <0 = Sparskit failure code, 100+k = zero
   pivot at row k, 200 = zero row, 300 = unsupported option). */
int oracle_solve_csr(int n, const int *indptr0, const int *indices0,
                     const double *data0, const double *b0, double *x,
                     const oracle_params *p, int *its_out, double *res_out)
{
  int *ia, *ja, i, j, k, nnz, ierr = 0, ipar[17], status;
  double *a, *b, fpar[17], *rhs, *sol, *w, *rowscal = NULL;
  int *permr, *rpermr, *permp;
  double *ar = NULL;
  int *iar = NULL, *jar = NULL;
  sscalar *alu = NULL;
  int *jlu = NULL, *ju = NULL;
  int scaled = 0;

  nnz = indptr0[n];
  ia = (int *)malloc(sizeof(int) * (n + 1));
  ja = (int *)malloc(sizeof(int) * (nnz ? nnz : 1));
  a = (double *)malloc(sizeof(double) * (nnz ? nnz : 1));
  b = (double *)malloc(sizeof(double) * (n ? n : 1));
  for(i = 0; i <= n; i++) ia[i] = indptr0[i] + 1;
  for(k = 0; k < nnz; k++) {
    ja[k] = indices0[k] + 1;
    a[k] = data0[k];
  }
  memcpy(b, b0, sizeof(double) * n);

  /* scaling (DIAG_SCALING: symmetric D^-1/2 A D^-1/2, Sparskit.cpp:978-1001) */
  if(p->scaling == 1) {
    int job0 = 0, job1 = 1, ioff = 0, len;
    int *idiag = (int *)malloc(sizeof(int) * n);
    rowscal = (double *)malloc(sizeof(double) * n);
    getdia_(&n, &n, &job0, a, ja, ia, &len, rowscal, idiag, &ioff);
    free(idiag);
    scaled = 1;
    for(i = 0; i < n; i++) {
      if(rowscal[i])
        rowscal[i] = 1. / sqrt(fabs(rowscal[i]));
      else {
        scaled = 0; /* "Diagonal scaling aborted because of zero diagonal" */
        break;
      }
    }
    if(scaled) {
      diamua_(&n, &job1, a, ja, ia, rowscal, a, ja, ia);
      amudia_(&n, &job1, a, ja, ia, rowscal, a, ja, ia);
      for(i = 0; i < n; i++) b[i] *= rowscal[i];
    }
  }
  else if(p->scaling != 0) {
    status = 300;
    goto done_early;
  }

  for(i = 1; i < n; i++)
    if(ia[i] - ia[i - 1] <= 0) {
      status = 200;
      goto done_early;
    }

  rhs = (double *)malloc(sizeof(double) * n);
  sol = (double *)calloc(n, sizeof(double));
  permr = (int *)malloc(sizeof(int) * n);
  rpermr = (int *)malloc(sizeof(int) * n);
  permp = (int *)malloc(sizeof(int) * 2 * n);
  for(i = 0; i < n; i++) permr[i] = rpermr[i] = permp[i + n] = i + 1;

  if(p->renumbering == 1) {
    int *mask = (int *)malloc(sizeof(int) * (nnz > n ? nnz : n));
    int *levels = (int *)malloc(sizeof(int) * (n + 1));
    int one = 1, maskval = 1, nlev = 1;
    double *wk;
    ar = (double *)malloc(sizeof(double) * nnz);
    iar = (int *)malloc(sizeof(int) * (n + 1));
    jar = (int *)malloc(sizeof(int) * nnz);
    cmkreord_(&n, a, ja, ia, ar, jar, iar, &one, permr, mask, &maskval, &nlev,
              rpermr, levels);
    wk = (double *)malloc(sizeof(double) * nnz);
    sortcol_(&n, ar, jar, iar, mask, wk);
    free(wk);
    free(mask);
    free(levels);
    free(a);
    free(ia);
    free(ja);
    a = ar;
    ia = iar;
    ja = jar;
  }

  /* incomplete factorisation */
  if(p->preconditioner == SK_ILU0) {
    int nnz_ilu = nnz + (n + 1);
    int *jw = (int *)malloc(sizeof(int) * (n + 1));
    alu = (sscalar *)malloc(sizeof(sscalar) * nnz_ilu);
    jlu = (int *)malloc(sizeof(int) * nnz_ilu);
    ju = (int *)malloc(sizeof(int) * (n + 1));
    ilu0_(&n, a, ja, ia, alu, jlu, ju, jw, &ierr);
    free(jw);
    if(ierr) {
      status = 100 + ierr;
      goto done;
    }
  }
  else if(p->preconditioner == SK_DIAGONAL) {
    alu = (sscalar *)malloc(sizeof(sscalar) * (n + 1));
    jlu = (int *)malloc(sizeof(int) * (n + 1));
    ju = (int *)malloc(sizeof(int) * (n + 1));
    for(i = 0; i < n; i++) {
      alu[i] = 1.0;
      jlu[i] = n + 2;
      ju[i] = n + 2;
    }
    alu[n] = 0.0;
    jlu[n] = n + 2;
    ju[n] = 0;
  }
  else if(p->preconditioner != SK_NONE) {
    status = 300;
    goto done;
  }

  for(i = 0; i < n; i++) rhs[i] = b[rpermr[i] - 1];

  memset(ipar, 0, sizeof(ipar));
  memset(fpar, 0, sizeof(fpar));
  ipar[1] = 0;
  ipar[2] = (p->preconditioner == SK_NONE) ? 0 : p->precond_position;
  ipar[3] = 1;
  ipar[4] = 0;
  ipar[5] = p->krylov_size;
  ipar[6] = p->nb_iter_max;
  fpar[1] = p->stopping_test;
  fpar[2] = 0.0;
  fpar[11] = 0.0;
  switch(p->algorithm) {
  case SK_CG: ipar[4] = 5 * n; break;
  case SK_GMRES:
    ipar[4] = (n + 3) * (ipar[5] + 2) + (ipar[5] + 1) * ipar[5] / 2;
    break;
  case SK_FGMRES:
    ipar[4] = 2 * n * (ipar[5] + 1) + (ipar[5] + 1) * ipar[5] / 2 +
              3 * ipar[5] + 2;
    break;
  default: status = 300; goto done;
  }
  w = (double *)malloc(sizeof(double) * ipar[4]);

  for(;;) {
    int end = 0;
    switch(p->algorithm) {
    case SK_CG: cg_(&n, rhs, sol, &ipar[1], &fpar[1], w); break;
    case SK_GMRES: gmres_(&n, rhs, sol, &ipar[1], &fpar[1], w); break;
    case SK_FGMRES: fgmres_(&n, rhs, sol, &ipar[1], &fpar[1], w); break;
    }
    switch(ipar[1]) {
    case 1: amux_(&n, &w[ipar[8] - 1], &w[ipar[9] - 1], a, ja, ia); break;
    case 2: atmux_(&n, &w[ipar[8] - 1], &w[ipar[9] - 1], a, ja, ia); break;
    case 3:
    case 5: lusol_(&n, &w[ipar[8] - 1], &w[ipar[9] - 1], alu, jlu, ju); break;
    case 4:
    case 6: lutsol_(&n, &w[ipar[8] - 1], &w[ipar[9] - 1], alu, jlu, ju); break;
    default: end = 1; break;
    }
    if(end) break;
  }
  status = ipar[1];
  if(its_out) *its_out = ipar[7];
  if(res_out) *res_out = fpar[6];
  free(w);

  /* inverse renumbering */
  for(i = 0; i < n; i++) {
    j = permr[i] - 1;
    k = permp[j + n] - 1;
    x[i] = sol[k];
  }
  if(scaled)
    for(i = 0; i < n; i++) x[i] *= rowscal[i];

done:
  free(rhs);
  free(sol);
  free(permr);
  free(rpermr);
  free(permp);
  free(alu);
  free(jlu);
  free(ju);
done_early:
  free(a);
  free(ia);
  free(ja);
  free(b);
  free(rowscal);
  return status;
}
