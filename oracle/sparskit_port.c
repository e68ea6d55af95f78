/*
 * ORACLE — test infrastructure only, never shipped or measured as the product.
 *
 * Plain-C restatement of the Sparskit 2 Fortran routines that GetDP's
 * Sparskit backend calls on the Generate/Solve path (contrib/Sparskit in the
 * GetDP 3.5.0 sources).  No Fortran compiler exists in this image, so the
 * routines are restated here from the published algorithms, keeping the
 * Fortran loop order and 1-based indexing so that results are deterministic
 * and comparable with the original.
 *
 * The exported symbols use the gfortran naming convention (trailing
 * underscore, every argument by pointer) so that the reference's own C++ glue
 * (contrib/Sparskit/Sparskit.cpp, which declares them at :48-97) links
 * against this file unchanged when the reference is compiled from source.
 *
 * Routines outside the hot path (ILUT/ILUTP/ILUD/ILUDP/ILUK/MILU0, CGNR, BCG,
 * DBCG, BCGSTAB, TFQMR, FOM, DQGMRES, PGMRES, FLU, skit/psplot printing) are
 * stubs that report "not restated" through their error codes.
 *
 * The ILU storage type follows contrib/Sparskit/ilut.F:10-14: float when
 * HAVE_ILU_FLOAT is defined (as the official build does), double otherwise.
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

/* 1-based accessors for Fortran-style arrays */
#define IP(k) ipar[(k)-1]
#define FP(k) fpar[(k)-1]

/* ------------------------------------------------------------------------ */
/* BLAS-1: ddot (contrib/Sparskit/blas1.f:52), unit-stride path unrolled by 5 */
/* ------------------------------------------------------------------------ */
static double ddot1(int n, const double *dx, const double *dy)
{
  double dtemp = 0.0;
  int i, m;
  if(n <= 0) return 0.0;
  m = n % 5;
  for(i = 1; i <= m; i++) dtemp = dtemp + dx[i - 1] * dy[i - 1];
  if(n < 5) return dtemp;
  for(i = m + 1; i <= n; i += 5)
    dtemp = dtemp + dx[i - 1] * dy[i - 1] + dx[i] * dy[i] +
            dx[i + 1] * dy[i + 1] + dx[i + 2] * dy[i + 2] +
            dx[i + 3] * dy[i + 3];
  return dtemp;
}

/* distdot (iters.f:3-10) is ddot on one processor */
static double distdot(int n, const double *x, const double *y)
{
  return ddot1(n, x, y);
}

/* dnrm2 (blas1.f:190): only used for the final residual message in
   Sparskit.cpp:586; restated as a plain scaled two-norm. */
double dnrm2_(int *n, double *dx, int *incx)
{
  double scale = 0.0, ssq = 1.0;
  int i, nn = *n, inc = *incx;
  if(nn <= 0 || inc <= 0) return 0.0;
  for(i = 0; i < nn; i++) {
    double v = dx[(size_t)i * inc];
    if(v != 0.0) {
      double a = fabs(v);
      if(scale < a) {
        ssq = 1.0 + ssq * (scale / a) * (scale / a);
        scale = a;
      }
      else
        ssq += (a / scale) * (a / scale);
    }
  }
  return scale * sqrt(ssq);
}

/* ------------------------------------------------------------------------ */
/* amux / atmux (contrib/Sparskit/matvec.f:35, :123)                        */
/* ------------------------------------------------------------------------ */
void amux_(int *n_, double *x, double *y, double *a, int *ja, int *ia)
{
  int n = *n_, i, k;
  for(i = 1; i <= n; i++) {
    double t = 0.0;
    for(k = ia[i - 1]; k <= ia[i] - 1; k++) t = t + a[k - 1] * x[ja[k - 1] - 1];
    y[i - 1] = t;
  }
}

void atmux_(int *n_, double *x, double *y, double *a, int *ja, int *ia)
{
  int n = *n_, i, k;
  for(i = 1; i <= n; i++) y[i - 1] = 0.0;
  for(i = 1; i <= n; i++)
    for(k = ia[i - 1]; k <= ia[i] - 1; k++)
      y[ja[k - 1] - 1] = y[ja[k - 1] - 1] + x[i - 1] * a[k - 1];
}

/* ------------------------------------------------------------------------ */
/* ILU(0) and the triangular solves (contrib/Sparskit/ilut.F:1818, :2297,   */
/* :2349).  Output in MSR form: alu(1:n) = inverted diagonal, then for each */
/* row its L part followed by its U part; ju(i) points at the U part.       */
/* ------------------------------------------------------------------------ */
void ilu0_(int *n_, double *a, int *ja, int *ia, sscalar *alu, int *jlu,
           int *ju, int *iw, int *ierr)
{
  int n = *n_, ju0, i, ii, js, j, jcol, jf, jm, jrow, jj, jw;
  double tl; /* implicit real*8 in ilut.F; the product itself is sscalar */
#define ALU(k) alu[(k)-1]
#define JLU(k) jlu[(k)-1]
#define JU(k) ju[(k)-1]
#define IW(k) iw[(k)-1]
  ju0 = n + 2;
  JLU(1) = ju0;
  for(i = 1; i <= n; i++) IW(i) = 0;
  for(ii = 1; ii <= n; ii++) {
    js = ju0;
    for(j = ia[ii - 1]; j <= ia[ii] - 1; j++) {
      jcol = ja[j - 1];
      if(jcol == ii) {
        ALU(ii) = (sscalar)a[j - 1];
        IW(jcol) = ii;
        JU(ii) = ju0;
      }
      else {
        ALU(ju0) = (sscalar)a[j - 1];
        JLU(ju0) = ja[j - 1];
        IW(jcol) = ju0;
        ju0 = ju0 + 1;
      }
    }
    JLU(ii + 1) = ju0;
    jf = ju0 - 1;
    jm = JU(ii) - 1;
    for(j = js; j <= jm; j++) {
      jrow = JLU(j);
      tl = (sscalar)(ALU(j) * ALU(jrow));
      ALU(j) = (sscalar)tl;
      for(jj = JU(jrow); jj <= JLU(jrow + 1) - 1; jj++) {
        jw = IW(JLU(jj));
        if(jw != 0) ALU(jw) = (sscalar)(ALU(jw) - tl * ALU(jj));
      }
    }
    if(ALU(ii) == 0.0) {
      *ierr = ii;
      return;
    }
    ALU(ii) = (sscalar)(1.0 / ALU(ii));
    IW(ii) = 0;
    for(i = js; i <= jf; i++) IW(JLU(i)) = 0;
  }
  *ierr = 0;
}

void lusol_(int *n_, double *y, double *x, sscalar *alu, int *jlu, int *ju)
{
  int n = *n_, i, k;
  for(i = 1; i <= n; i++) {
    x[i - 1] = y[i - 1];
    for(k = JLU(i); k <= JU(i) - 1; k++)
      x[i - 1] = x[i - 1] - ALU(k) * x[JLU(k) - 1];
  }
  for(i = n; i >= 1; i--) {
    for(k = JU(i); k <= JLU(i + 1) - 1; k++)
      x[i - 1] = x[i - 1] - ALU(k) * x[JLU(k) - 1];
    x[i - 1] = ALU(i) * x[i - 1];
  }
}

void lutsol_(int *n_, double *y, double *x, sscalar *alu, int *jlu, int *ju)
{
  int n = *n_, i, k;
  for(i = 1; i <= n; i++) x[i - 1] = y[i - 1];
  for(i = 1; i <= n; i++) {
    x[i - 1] = x[i - 1] * ALU(i);
    for(k = JU(i); k <= JLU(i + 1) - 1; k++)
      x[JLU(k) - 1] = x[JLU(k) - 1] - ALU(k) * x[i - 1];
  }
  for(i = n; i >= 1; i--)
    for(k = JLU(i); k <= JU(i) - 1; k++)
      x[JLU(k) - 1] = x[JLU(k) - 1] - ALU(k) * x[i - 1];
}
#undef ALU
#undef JLU
#undef JU
#undef IW

/* ------------------------------------------------------------------------ */
/* Scaling helpers (unary.f:765 getdia, blassm.f:785 diamua, :842 amudia,   */
/* unary.f:2521 rnrms, :2572 cnrms)                                         */
/* ------------------------------------------------------------------------ */
void getdia_(int *nrow_, int *ncol_, int *job_, double *a, int *ja, int *ia,
             int *len, double *diag, int *idiag, int *ioff_)
{
  int nrow = *nrow_, ncol = *ncol_, job = *job_, ioff = *ioff_;
  int istart, iend, i, k, ko, kold, kdiag;
  istart = (0 > -ioff) ? 0 : -ioff;
  iend = (nrow < ncol - ioff) ? nrow : ncol - ioff;
  *len = 0;
  for(i = 1; i <= nrow; i++) {
    idiag[i - 1] = 0;
    diag[i - 1] = 0.0;
  }
  for(i = istart + 1; i <= iend; i++) {
    for(k = ia[i - 1]; k <= ia[i] - 1; k++) {
      if(ja[k - 1] - i == ioff) {
        diag[i - 1] = a[k - 1];
        idiag[i - 1] = k;
        *len = *len + 1;
        break;
      }
    }
  }
  if(job == 0 || *len == 0) return;
  ko = 0;
  for(i = 1; i <= nrow; i++) {
    kold = ko;
    kdiag = idiag[i - 1];
    for(k = ia[i - 1]; k <= ia[i] - 1; k++) {
      if(k != kdiag) {
        ko = ko + 1;
        a[ko - 1] = a[k - 1];
        ja[ko - 1] = ja[k - 1];
      }
    }
    ia[i - 1] = kold + 1;
  }
  ia[nrow] = ko + 1;
}

void diamua_(int *nrow_, int *job_, double *a, int *ja, int *ia, double *diag,
             double *b, int *jb, int *ib)
{
  int nrow = *nrow_, ii, k;
  for(ii = 1; ii <= nrow; ii++) {
    double scal = diag[ii - 1];
    for(k = ia[ii - 1]; k <= ia[ii] - 1; k++) b[k - 1] = a[k - 1] * scal;
  }
  if(*job_ == 0) return;
  for(ii = 1; ii <= nrow + 1; ii++) ib[ii - 1] = ia[ii - 1];
  for(k = ia[0]; k <= ia[nrow] - 1; k++) jb[k - 1] = ja[k - 1];
}

void amudia_(int *nrow_, int *job_, double *a, int *ja, int *ia, double *diag,
             double *b, int *jb, int *ib)
{
  int nrow = *nrow_, ii, k;
  for(ii = 1; ii <= nrow; ii++)
    for(k = ia[ii - 1]; k <= ia[ii] - 1; k++)
      b[k - 1] = a[k - 1] * diag[ja[k - 1] - 1];
  if(*job_ == 0) return;
  for(ii = 1; ii <= nrow + 1; ii++) ib[ii - 1] = ia[ii - 1];
  for(k = ia[0]; k <= ia[nrow] - 1; k++) jb[k - 1] = ja[k - 1];
}

void rnrms_(int *nrow_, int *nrm_, double *a, int *ja, int *ia, double *diag)
{
  int nrow = *nrow_, nrm = *nrm_, ii, k;
  (void)ja;
  for(ii = 1; ii <= nrow; ii++) {
    double scal = 0.0;
    for(k = ia[ii - 1]; k <= ia[ii] - 1; k++) {
      if(nrm == 0)
        scal = (scal > fabs(a[k - 1])) ? scal : fabs(a[k - 1]);
      else if(nrm == 1)
        scal = scal + fabs(a[k - 1]);
      else
        scal = scal + a[k - 1] * a[k - 1];
    }
    if(nrm == 2) scal = sqrt(scal);
    diag[ii - 1] = scal;
  }
}

void cnrms_(int *nrow_, int *nrm_, double *a, int *ja, int *ia, double *diag)
{
  int nrow = *nrow_, nrm = *nrm_, ii, k, j;
  for(k = 1; k <= nrow; k++) diag[k - 1] = 0.0;
  for(ii = 1; ii <= nrow; ii++)
    for(k = ia[ii - 1]; k <= ia[ii] - 1; k++) {
      j = ja[k - 1];
      if(nrm == 0)
        diag[j - 1] =
          (diag[j - 1] > fabs(a[k - 1])) ? diag[j - 1] : fabs(a[k - 1]);
      else if(nrm == 1)
        diag[j - 1] = diag[j - 1] + fabs(a[k - 1]);
      else
        diag[j - 1] = diag[j - 1] + a[k - 1] * a[k - 1];
    }
  if(nrm != 2) return;
  for(k = 1; k <= nrow; k++) diag[k - 1] = sqrt(diag[k - 1]);
}

/* ------------------------------------------------------------------------ */
/* Reverse Cuthill-McKee (cmkreord.f:3, reordering.f:15 BFS, :232 perphn,   */
/* :279 add_lvst, :364 rversp, :379 maskdeg, cmkreord.f:114 exchange,       */
/* unary.f:1433 dperm / :1292 rperm / :1365 cperm, cmkreord.f:64/:88        */
/* sort_irv / sortcol)                                                      */
/* ------------------------------------------------------------------------ */
static void add_lvst(int *istart, int *iend, int *riord, const int *ja,
                     const int *ia, int *mask, int maskval)
{
  int nod = *iend, ir, i, k, j;
  for(ir = *istart + 1; ir <= *iend; ir++) {
    i = riord[ir - 1];
    for(k = ia[i - 1]; k <= ia[i] - 1; k++) {
      j = ja[k - 1];
      if(mask[j - 1] == maskval) {
        nod = nod + 1;
        mask[j - 1] = 0;
        riord[nod - 1] = j;
      }
    }
  }
  *istart = *iend;
  *iend = nod;
}

static void bfs(int n, const int *ja, const int *ia, int nfirst,
                const int *iperm, int *mask, int maskval, int *riord,
                int *levels, int *nlev)
{
  int j, ii = 0, nod, istart = 0, iend = nfirst;
  int permut = (iperm[0] != 0);
  *nlev = 0;
  for(j = 1; j <= nfirst; j++) mask[riord[j - 1] - 1] = 0;
  for(;;) {
    *nlev = *nlev + 1;
    levels[*nlev - 1] = istart + 1;
    add_lvst(&istart, &iend, riord, ja, ia, mask, maskval);
    if(istart < iend) continue;
    /* look for an unvisited node to start a new connected component */
    for(;;) {
      ii = ii + 1;
      if(ii > n) break;
      nod = ii;
      if(permut) nod = iperm[nod - 1];
      if(mask[nod - 1] == maskval) break;
    }
    if(ii > n) break;
    istart = iend;
    iend = iend + 1;
    riord[iend - 1] = nod;
    mask[nod - 1] = 0;
  }
  levels[*nlev] = iend + 1;
  for(j = 1; j <= iend; j++) mask[riord[j - 1] - 1] = maskval;
}

static int maskdeg(const int *ja, const int *ia, int nod, const int *mask,
                   int maskval)
{
  int deg = 0, k;
  for(k = ia[nod - 1]; k <= ia[nod] - 1; k++)
    if(mask[ja[k - 1] - 1] == maskval) deg = deg + 1;
  return deg;
}

static void perphn(int n, const int *ja, const int *ia, int *init, int *iperm,
                   int *mask, int maskval, int *nlev, int *riord, int *levels)
{
  int j, nlevp = 0, deg, mindeg, nod;
  for(;;) {
    riord[0] = *init;
    bfs(n, ja, ia, 1, iperm, mask, maskval, riord, levels, nlev);
    if(*nlev > nlevp) {
      mindeg = levels[*nlev] - 1;
      for(j = levels[*nlev - 1]; j <= levels[*nlev] - 1; j++) {
        nod = riord[j - 1];
        deg = maskdeg(ja, ia, nod, mask, maskval);
        if(deg < mindeg) {
          *init = nod;
          mindeg = deg;
        }
      }
      nlevp = *nlev;
      continue;
    }
    break;
  }
}

static void rversp(int n, int *riord)
{
  int j, k;
  for(j = 1; j <= n / 2; j++) {
    k = riord[j - 1];
    riord[j - 1] = riord[n - j];
    riord[n - j] = k;
  }
}

static void rperm(int nrow, const double *a, const int *ja, const int *ia,
                  double *ao, int *jao, int *iao, const int *perm, int job)
{
  int j, i, ii, k, ko;
  for(j = 1; j <= nrow; j++) {
    i = perm[j - 1];
    iao[i] = ia[j] - ia[j - 1];
  }
  iao[0] = 1;
  for(j = 1; j <= nrow; j++) iao[j] = iao[j] + iao[j - 1];
  for(ii = 1; ii <= nrow; ii++) {
    ko = iao[perm[ii - 1] - 1];
    for(k = ia[ii - 1]; k <= ia[ii] - 1; k++) {
      jao[ko - 1] = ja[k - 1];
      if(job == 1) ao[ko - 1] = a[k - 1];
      ko = ko + 1;
    }
  }
}

static void dperm_sym(int nrow, const double *a, const int *ja, const int *ia,
                      double *ao, int *jao, int *iao, const int *perm)
{
  int k, nnz;
  rperm(nrow, a, ja, ia, ao, jao, iao, perm, 1);
  /* cperm in place on (ao, jao, iao) with job 0: permute column indices */
  nnz = iao[nrow] - 1;
  for(k = 1; k <= nnz; k++) jao[k - 1] = perm[jao[k - 1] - 1];
}

void cmkreord_(int *n_, double *a, int *ja, int *ia, double *a0, int *ja0,
               int *ia0, int *init, int *iperm, int *mask, int *maskval,
               int *nlev, int *riord, int *levels)
{
  int n = *n_, i;
  *maskval = 1;
  for(i = 1; i <= n; i++) mask[i - 1] = *maskval;
  iperm[0] = 0;
  perphn(n, ja, ia, init, iperm, mask, *maskval, nlev, riord, levels);
  rversp(n, riord);
  for(i = 1; i <= n; i++) iperm[riord[i - 1] - 1] = i; /* exchange */
  dperm_sym(n, a, ja, ia, a0, ja0, ia0, iperm);
}

static void sort_irv(int *itmp, double *rtmp, int n)
{
  int i, j, jmin, itmpmin, it;
  double rt;
  for(i = 1; i <= n; i++) {
    itmpmin = itmp[i - 1];
    jmin = i;
    for(j = i + 1; j <= n; j++) {
      if(itmp[j - 1] < itmpmin) {
        jmin = j;
        itmpmin = itmp[jmin - 1];
      }
    }
    it = itmp[i - 1];
    itmp[i - 1] = itmp[jmin - 1];
    itmp[jmin - 1] = it;
    rt = rtmp[i - 1];
    rtmp[i - 1] = rtmp[jmin - 1];
    rtmp[jmin - 1] = rt;
  }
}

void sortcol_(int *n_, double *a, int *ja, int *ia, int *iw, double *rw)
{
  int n = *n_, i, j, k, ideb, ifin;
  for(i = 1; i <= n; i++) {
    ideb = ia[i - 1];
    ifin = ia[i] - 1;
    k = 0;
    for(j = ideb; j <= ifin; j++) {
      k = k + 1;
      iw[k - 1] = ja[j - 1];
      rw[k - 1] = a[j - 1];
    }
    sort_irv(iw, rw, ifin - ideb + 1);
    k = 0;
    for(j = ideb; j <= ifin; j++) {
      k = k + 1;
      ja[j - 1] = iw[k - 1];
      a[j - 1] = rw[k - 1];
    }
  }
}

/* csrcoo (formats.f:332), used by the KUL matrix printer */
void csrcoo_(int *nrow_, int *job_, int *nzmax, double *a, int *ja, int *ia,
             int *nnz, double *ao, int *ir, int *jc, int *ierr)
{
  int nrow = *nrow_, job = *job_, k, i, k1, k2;
  *ierr = 0;
  *nnz = ia[nrow] - 1;
  if(*nnz > *nzmax) {
    *ierr = 1;
    return;
  }
  if(job >= 3)
    for(k = 1; k <= *nnz; k++) ao[k - 1] = a[k - 1];
  if(job >= 2)
    for(k = 1; k <= *nnz; k++) jc[k - 1] = ja[k - 1];
  /* copy backward so that ir may share storage with ia */
  for(i = nrow; i >= 1; i--) {
    k1 = ia[i] - 1;
    k2 = ia[i - 1];
    for(k = k1; k >= k2; k--) ir[k - 1] = i;
  }
}

/* ------------------------------------------------------------------------ */
/* Shared Krylov helpers (iters.f:3235 givens, :3275 stopbis, :3333 tidycg, */
/* :3368 brkdn, :3404 bisinit, :3475 mgsro)                                 */
/* ------------------------------------------------------------------------ */
static double fsign(double a, double b) { return (b >= 0.0) ? fabs(a) : -fabs(a); }

static void givens(double *x, double *y, double *c, double *s)
{
  double t;
  if(*x == 0.0 && *y == 0.0) {
    *c = 1.0;
    *s = 0.0;
  }
  else if(fabs(*y) > fabs(*x)) {
    t = *x / *y;
    *x = sqrt(1.0 + t * t);
    *s = fsign(1.0 / *x, *y);
    *c = t * *s;
  }
  else if(fabs(*y) <= fabs(*x)) {
    t = *y / *x;
    *y = sqrt(1.0 + t * t);
    *c = fsign(1.0 / *y, *x);
    *s = t * *c;
  }
  else {
    *x = 0.0;
    *y = 0.0;
    *c = 1.0;
    *s = 0.0;
  }
  *x = fabs(*x * *y);
}

static int stopbis(int n, int *ipar, int mvpi, double *fpar, const double *r,
                   const double *delx, double sx)
{
  int stop = (IP(11) == 1);
  if(IP(6) > 0 && IP(7) >= IP(6)) {
    IP(1) = -1;
    stop = 1;
  }
  if(stop) return 1;
  FP(5) = sqrt(distdot(n, r, r));
  FP(11) = FP(11) + 2 * n;
  if(IP(3) < 0) {
    FP(6) = sx * sqrt(distdot(n, delx, delx));
    FP(11) = FP(11) + 2 * n;
    if(IP(7) < mvpi + mvpi + 1) {
      FP(3) = FP(6);
      if(IP(3) == -1) FP(4) = FP(1) * FP(3) + FP(2);
    }
  }
  else
    FP(6) = FP(5);
  /* written so that a NaN in fpar(6) stops the iteration */
  if(FP(6) > FP(4)) {
    IP(11) = 0;
    return 0;
  }
  IP(11) = 1;
  return 1;
}

static void tidycg(int n, int *ipar, double *fpar, double *sol,
                   const double *delx)
{
  int i;
  if(IP(12) != 0)
    IP(1) = IP(12);
  else if(IP(1) > 0) {
    if((IP(3) == 999 && IP(11) == 1) || FP(6) <= FP(4))
      IP(1) = 0;
    else if(IP(7) >= IP(6) && IP(6) > 0)
      IP(1) = -1;
    else
      IP(1) = -10;
  }
  if(FP(3) > 0.0 && FP(6) > 0.0 && IP(7) > IP(13))
    FP(7) = log10(FP(3) / FP(6)) / (double)(IP(7) - IP(13));
  else
    FP(7) = 0.0;
  for(i = 0; i < n; i++) sol[i] = sol[i] + delx[i];
}

static int brkdn(double alpha, int *ipar)
{
  double beta;
  if(alpha > 0.0) {
    beta = 1.0 / alpha;
    if(!(beta > 0.0)) {
      IP(1) = -9;
      return 1;
    }
  }
  else if(alpha < 0.0) {
    beta = 1.0 / alpha;
    if(!(beta < 0.0)) {
      IP(1) = -9;
      return 1;
    }
  }
  else if(alpha == 0.0) {
    IP(1) = -3;
    return 1;
  }
  else {
    IP(1) = -9;
    return 1;
  }
  return 0;
}

static void bisinit(int *ipar, double *fpar, int wksize, int dsc, int *lp,
                    int *rp, double *wk)
{
  int i;
  if(IP(4) < wksize) {
    IP(1) = -2;
    IP(4) = wksize;
    return;
  }
  if(IP(2) > 2) {
    *lp = 1;
    *rp = 1;
  }
  else if(IP(2) == 2) {
    *lp = 0;
    *rp = 1;
  }
  else if(IP(2) == 1) {
    *lp = 1;
    *rp = 0;
  }
  else {
    *lp = 0;
    *rp = 0;
  }
  if(IP(3) == 0) IP(3) = dsc;
  for(i = 7; i <= 13; i++) IP(i) = 0;
  if(FP(1) < 0.0 || FP(1) >= 1.0 || FP(2) < 0.0 ||
     (FP(1) == 0.0 && FP(2) == 0.0)) {
    if(IP(1) == 0) {
      IP(1) = -4;
      return;
    }
    FP(1) = 1.0e-6;
    FP(2) = 1.0e-16;
  }
  for(i = 3; i <= 10; i++) FP(i) = 0.0;
  if(FP(11) < 0.0) FP(11) = 0.0;
  for(i = 0; i < wksize; i++) wk[i] = 0.0;
}

/* mgsro(.false., lda=n, n, m, ind): orthogonalise column ind of vec (lda x m)
   against columns 1..ind-1 with selective re-orthogonalisation
   (reorth = 0.98 on the squared cosine). */
static void mgsro(int full, int lda, int n, int m, int ind, double *ops,
                  double *vec, double *hh, int *ierr)
{
  int i, k;
  double nrm0, nrm1, fct, thr;
  const double reorth = 0.98;
  double *vi, *vind = vec + (size_t)(ind - 1) * lda;
  nrm0 = distdot(n, vind, vind);
  *ops = *ops + n + n;
  thr = nrm0 * reorth;
  if(nrm0 <= 0.0) {
    *ierr = -1;
    return;
  }
  else if(nrm0 > 0.0 && 1.0 / nrm0 > 0.0)
    *ierr = 0;
  else {
    *ierr = -2;
    return;
  }
  if(full) {
    for(i = ind + 1; i <= m; i++) {
      vi = vec + (size_t)(i - 1) * lda;
      fct = distdot(n, vind, vi);
      hh[i - 1] = fct;
      for(k = 0; k < n; k++) vind[k] = vind[k] - fct * vi[k];
      *ops = *ops + 4 * n + 2;
      if(fct * fct > thr) {
        fct = distdot(n, vind, vi);
        hh[i - 1] = hh[i - 1] + fct;
        for(k = 0; k < n; k++) vind[k] = vind[k] - fct * vi[k];
        *ops = *ops + 4 * n + 1;
      }
      nrm0 = nrm0 - hh[i - 1] * hh[i - 1];
      if(nrm0 < 0.0) nrm0 = 0.0;
      thr = nrm0 * reorth;
    }
  }
  for(i = 1; i <= ind - 1; i++) {
    vi = vec + (size_t)(i - 1) * lda;
    fct = distdot(n, vind, vi);
    hh[i - 1] = fct;
    for(k = 0; k < n; k++) vind[k] = vind[k] - fct * vi[k];
    *ops = *ops + 4 * n + 2;
    if(fct * fct > thr) {
      fct = distdot(n, vind, vi);
      hh[i - 1] = hh[i - 1] + fct;
      for(k = 0; k < n; k++) vind[k] = vind[k] - fct * vi[k];
      *ops = *ops + 4 * n + 1;
    }
    nrm0 = nrm0 - hh[i - 1] * hh[i - 1];
    if(nrm0 < 0.0) nrm0 = 0.0;
    thr = nrm0 * reorth;
  }
  nrm1 = sqrt(distdot(n, vind, vind));
  *ops = *ops + n + n;
  hh[ind - 1] = nrm1;
  if(nrm1 <= 0.0) {
    *ierr = -3;
    return;
  }
  fct = 1.0 / nrm1;
  for(k = 0; k < n; k++) vind[k] = vind[k] * fct;
  *ops = *ops + n + 1;
  *ierr = 0;
}

/* ------------------------------------------------------------------------ */
/* CG with reverse communication (iters.f:379-564).  The preconditioners    */
/* are applied as Ml^-1 A Mr^-1 (it is not PCG).  State lives in statics,   */
/* as the Fortran SAVE does.                                                */
/* ------------------------------------------------------------------------ */
void cg_(int *n_, double *rhs, double *sol, int *ipar, double *fpar, double *w)
{
  static int lp, rp;
  static double alpha;
  int n = *n_, i;
  double *w1 = w, *w2 = w + n, *w3 = w + 2 * (size_t)n, *w4 = w + 3 * (size_t)n,
         *w5 = w + 4 * (size_t)n;

  if(IP(1) <= 0) IP(10) = 0;
  switch(IP(10)) {
  case 1: goto L10;
  case 2: goto L20;
  case 3: goto L40;
  case 4: goto L50;
  case 5: goto L60;
  case 6: goto L70;
  case 7: goto L80;
  default: break;
  }
  bisinit(ipar, fpar, 5 * n, 1, &lp, &rp, w);
  if(IP(1) < 0) return;
  IP(1) = 1;
  IP(8) = n + 1;
  IP(9) = IP(8) + n;
  IP(10) = 1;
  for(i = 0; i < n; i++) w2[i] = sol[i];
  return;
L10:
  IP(7) = IP(7) + 1;
  IP(13) = 1;
  for(i = 0; i < n; i++) w2[i] = rhs[i] - w3[i];
  FP(11) = FP(11) + n;
  if(lp) {
    IP(1) = 3;
    IP(9) = 1;
    IP(10) = 2;
    return;
  }
L20:
  if(lp)
    for(i = 0; i < n; i++) w2[i] = w1[i];
  else
    for(i = 0; i < n; i++) w1[i] = w2[i];
  FP(7) = distdot(n, w, w);
  FP(11) = FP(11) + 2 * n;
  FP(3) = sqrt(FP(7));
  FP(5) = FP(3);
  if(abs(IP(3)) == 2) {
    FP(4) = FP(1) * sqrt(distdot(n, rhs, rhs)) + FP(2);
    FP(11) = FP(11) + 2 * n;
  }
  else if(IP(3) != 999)
    FP(4) = FP(1) * FP(3) + FP(2);
L30:
  if(rp) {
    IP(1) = 5;
    IP(8) = n + 1;
    if(lp)
      IP(9) = IP(8) + n;
    else
      IP(9) = 3 * n + 1;
    IP(10) = 3;
    return;
  }
L40:
  IP(1) = 1;
  if(rp)
    IP(8) = IP(9);
  else
    IP(8) = n + 1;
  if(lp)
    IP(9) = 3 * n + 1;
  else
    IP(9) = n + n + 1;
  IP(10) = 4;
  return;
L50:
  if(lp) {
    IP(1) = 3;
    IP(8) = IP(9);
    IP(9) = n + n + 1;
    IP(10) = 5;
    return;
  }
L60:
  IP(7) = IP(7) + 1;
  alpha = distdot(n, w2, w3);
  FP(11) = FP(11) + 2 * n;
  if(brkdn(alpha, ipar)) goto L900;
  alpha = FP(7) / alpha;
  for(i = 0; i < n; i++) {
    w5[i] = w5[i] + alpha * w2[i];
    w1[i] = w1[i] - alpha * w3[i];
  }
  FP(11) = FP(11) + 4 * n;
  if(IP(3) == 999) {
    IP(1) = 10;
    IP(8) = 4 * n + 1;
    IP(9) = 3 * n + 1;
    IP(10) = 6;
    return;
  }
L70:
  if(IP(3) == 999) {
    if(IP(11) == 1) goto L900;
  }
  else if(stopbis(n, ipar, 1, fpar, w, w2, alpha))
    goto L900;
  alpha = FP(5) * FP(5) / FP(7);
  FP(7) = FP(5) * FP(5);
  for(i = 0; i < n; i++) w2[i] = w1[i] + alpha * w2[i];
  FP(11) = FP(11) + 2 * n;
  goto L30;
L900:
  if(rp) {
    if(IP(1) < 0) IP(12) = IP(1);
    IP(1) = 5;
    IP(8) = 4 * n + 1;
    IP(9) = IP(8) - n;
    IP(10) = 7;
    return;
  }
L80:
  if(rp)
    tidycg(n, ipar, fpar, sol, w4);
  else
    tidycg(n, ipar, fpar, sol, w5);
}

/* ------------------------------------------------------------------------ */
/* GMRES(m) with reverse communication (iters.f:1912-2219)                  */
/* ------------------------------------------------------------------------ */
void gmres_(int *n_, double *rhs, double *sol, int *ipar, double *fpar,
            double *w)
{
  static int lp, rp, m, idx, hess, vc, vs, vrn, k, ptr, p2;
  static double alpha, c, s;
  int n = *n_, i, ii;
#define W(j) w[(size_t)(j)-1]

  if(IP(1) <= 0) IP(10) = 0;
  switch(IP(10)) {
  case 1: goto L10;
  case 2: goto L20;
  case 3: goto L30;
  case 4: goto L40;
  case 5: goto L50;
  case 6: goto L60;
  case 7: goto L70;
  default: break;
  }
  m = (IP(5) <= 1) ? 15 : IP(5);
  idx = n * (m + 1);
  hess = idx + n;
  vc = hess + (m + 1) * m / 2 + 1;
  vs = vc + m;
  vrn = vs + m;
  i = vrn + m + 1;
  bisinit(ipar, fpar, i, 1, &lp, &rp, w);
  if(IP(1) < 0) return;
L100:
  IP(1) = 1;
  IP(8) = n + 1;
  IP(9) = 1;
  IP(10) = 1;
  k = 0;
  for(i = 1; i <= n; i++) W(n + i) = sol[i - 1];
  return;
L10:
  IP(7) = IP(7) + 1;
  IP(13) = IP(13) + 1;
  if(lp) {
    for(i = 1; i <= n; i++) W(n + i) = rhs[i - 1] - W(i);
    IP(1) = 3;
    IP(10) = 2;
    return;
  }
  else
    for(i = 1; i <= n; i++) W(i) = rhs[i - 1] - W(i);
  FP(11) = FP(11) + n;
L20:
  alpha = sqrt(distdot(n, w, w));
  FP(11) = FP(11) + 2 * n;
  if(IP(7) == 1 && IP(3) != 999) {
    if(abs(IP(3)) == 2) {
      FP(4) = FP(1) * sqrt(distdot(n, rhs, rhs)) + FP(2);
      FP(11) = FP(11) + 2 * n;
    }
    else
      FP(4) = FP(1) * alpha + FP(2);
    FP(3) = alpha;
  }
  FP(5) = alpha;
  W(vrn + 1) = alpha;
  if(alpha <= FP(4) && IP(3) >= 0 && IP(3) != 999) {
    IP(1) = 0;
    FP(6) = alpha;
    goto L300;
  }
  alpha = 1.0 / alpha;
  for(ii = 1; ii <= n; ii++) W(ii) = alpha * W(ii);
  FP(11) = FP(11) + n;
L110:
  k = k + 1;
  if(rp) {
    IP(1) = 5;
    IP(8) = k * n - n + 1;
    if(lp)
      IP(9) = k * n + 1;
    else
      IP(9) = idx + 1;
    IP(10) = 3;
    return;
  }
L30:
  IP(1) = 1;
  if(rp)
    IP(8) = IP(9);
  else
    IP(8) = (k - 1) * n + 1;
  if(lp)
    IP(9) = idx + 1;
  else
    IP(9) = 1 + k * n;
  IP(10) = 4;
  return;
L40:
  if(lp) {
    IP(1) = 3;
    IP(8) = IP(9);
    IP(9) = k * n + 1;
    IP(10) = 5;
    return;
  }
L50:
  IP(7) = IP(7) + 1;
  ptr = k * (k - 1) / 2 + hess;
  p2 = IP(9);
  mgsro(0, n, n, k + 1, k + 1, &FP(11), w, &W(ptr + 1), &IP(12));
  if(IP(12) < 0) goto L200;
  p2 = ptr + 1;
  for(i = 1; i <= k - 1; i++) {
    ptr = p2;
    p2 = p2 + 1;
    alpha = W(ptr);
    c = W(vc + i);
    s = W(vs + i);
    W(ptr) = c * alpha + s * W(p2);
    W(p2) = c * W(p2) - s * alpha;
  }
  givens(&W(p2), &W(p2 + 1), &c, &s);
  W(vc + k) = c;
  W(vs + k) = s;
  p2 = vrn + k;
  alpha = -s * W(p2);
  W(p2) = c * W(p2);
  W(p2 + 1) = alpha;
  FP(11) = FP(11) + 6 * k + 2;
  alpha = fabs(alpha);
  FP(5) = alpha;
  if(k < m && !(IP(3) >= 0 && alpha <= FP(4)) &&
     (IP(6) <= 0 || IP(7) < IP(6)))
    goto L110;
L200:
  ptr = hess + k * (k + 1) / 2;
  p2 = vrn + k;
  if(W(ptr) == 0.0) {
    k = k - 1;
    if(k > 0)
      goto L200;
    else {
      IP(1) = -3;
      IP(12) = -4;
      goto L300;
    }
  }
  W(p2) = W(p2) / W(ptr);
  for(i = k - 1; i >= 1; i--) {
    ptr = ptr - i - 1;
    for(ii = 1; ii <= i; ii++) W(vrn + ii) = W(vrn + ii) - W(p2) * W(ptr + ii);
    p2 = p2 - 1;
    W(p2) = W(p2) / W(ptr);
  }
  for(ii = 1; ii <= n; ii++) W(ii) = W(ii) * W(p2);
  for(i = 1; i <= k - 1; i++) {
    ptr = i * n;
    p2 = p2 + 1;
    for(ii = 1; ii <= n; ii++) W(ii) = W(ii) + W(p2) * W(ptr + ii);
  }
  FP(11) = FP(11) + 2 * k * n - n + k * (k + 1);
  if(rp) {
    IP(1) = 5;
    IP(8) = 1;
    IP(9) = idx + 1;
    IP(10) = 6;
    return;
  }
L60:
  if(rp)
    for(i = 1; i <= n; i++) sol[i - 1] = sol[i - 1] + W(idx + i);
  else
    for(i = 1; i <= n; i++) sol[i - 1] = sol[i - 1] + W(i);
  FP(11) = FP(11) + n;
  if(IP(3) == 999) {
    IP(1) = 10;
    IP(8) = -1;
    IP(9) = idx + 1;
    IP(10) = 7;
    return;
  }
  else if(IP(3) < 0) {
    if(IP(7) <= m + 1) {
      FP(3) = fabs(W(vrn + 1));
      if(IP(3) == -1) FP(4) = FP(1) * FP(3) + FP(2);
    }
    FP(6) = fabs(W(vrn + k));
  }
  else
    FP(6) = FP(5);
L70:
  if(IP(12) != 0) {
    IP(1) = -3;
    goto L300;
  }
  if((IP(7) < IP(6) || IP(6) <= 0) &&
     ((IP(3) == 999 && IP(11) == 0) || (IP(3) != 999 && FP(6) > FP(4))))
    goto L100;
  if(IP(1) > 0) {
    if(IP(3) == 999 && IP(11) == 1)
      IP(1) = 0;
    else if(IP(3) != 999 && FP(6) <= FP(4))
      IP(1) = 0;
    else if(IP(7) >= IP(6) && IP(6) > 0)
      IP(1) = -1;
    else
      IP(1) = -10;
  }
L300:
  if(FP(3) != 0.0 && FP(6) != 0.0 && IP(7) > IP(13))
    FP(7) = log10(FP(3) / FP(6)) / (double)(IP(7) - IP(13));
  else
    FP(7) = 0.0;
}

/* ------------------------------------------------------------------------ */
/* FGMRES(m) with reverse communication (iters.f:2522-2806)                 */
/* ------------------------------------------------------------------------ */
void fgmres_(int *n_, double *rhs, double *sol, int *ipar, double *fpar,
             double *w)
{
  static int lp, rp, m, idx, iz, hess, vc, vs, vrn, k, ptr, p2;
  static double alpha, c, s;
  int n = *n_, i, ii;

  if(IP(1) <= 0) IP(10) = 0;
  switch(IP(10)) {
  case 1: goto L10;
  case 2: goto L20;
  case 3: goto L30;
  case 4: goto L40;
  case 5: goto L50;
  case 6: goto L60;
  default: break;
  }
  m = (IP(5) <= 1) ? 15 : IP(5);
  idx = n * (m + 1);
  iz = idx + n;
  hess = iz + n * m;
  vc = hess + (m + 1) * m / 2 + 1;
  vs = vc + m;
  vrn = vs + m;
  i = vrn + m + 1;
  bisinit(ipar, fpar, i, 1, &lp, &rp, w);
  if(IP(1) < 0) return;
L100:
  IP(1) = 1;
  IP(8) = n + 1;
  IP(9) = 1;
  IP(10) = 1;
  k = 0;
  for(ii = 1; ii <= n; ii++) W(ii + n) = sol[ii - 1];
  return;
L10:
  IP(7) = IP(7) + 1;
  IP(13) = IP(13) + 1;
  FP(11) = FP(11) + n;
  if(lp) {
    for(i = 1; i <= n; i++) W(n + i) = rhs[i - 1] - W(i);
    IP(1) = 3;
    IP(10) = 2;
    return;
  }
  else
    for(i = 1; i <= n; i++) W(i) = rhs[i - 1] - W(i);
L20:
  alpha = sqrt(distdot(n, w, w));
  FP(11) = FP(11) + n + n;
  if(IP(7) == 1 && IP(3) != 999) {
    if(abs(IP(3)) == 2) {
      FP(4) = FP(1) * sqrt(distdot(n, rhs, rhs)) + FP(2);
      FP(11) = FP(11) + 2 * n;
    }
    else
      FP(4) = FP(1) * alpha + FP(2);
    FP(3) = alpha;
  }
  FP(5) = alpha;
  W(vrn + 1) = alpha;
  if(alpha <= FP(4) && IP(3) >= 0 && IP(3) != 999) {
    IP(1) = 0;
    FP(6) = alpha;
    goto L300;
  }
  alpha = 1.0 / alpha;
  for(ii = 1; ii <= n; ii++) W(ii) = W(ii) * alpha;
  FP(11) = FP(11) + n;
L110:
  k = k + 1;
  if(rp) {
    IP(1) = 5;
    IP(8) = k * n - n + 1;
    IP(9) = iz + IP(8);
    IP(10) = 3;
    return;
  }
  else
    for(ii = 0; ii <= n - 1; ii++) W(iz + k * n - ii) = W(k * n - ii);
L30:
  IP(1) = 1;
  if(rp)
    IP(8) = IP(9);
  else
    IP(8) = (k - 1) * n + 1;
  if(lp)
    IP(9) = idx + 1;
  else
    IP(9) = 1 + k * n;
  IP(10) = 4;
  return;
L40:
  if(lp) {
    IP(1) = 3;
    IP(8) = IP(9);
    IP(9) = k * n + 1;
    IP(10) = 5;
    return;
  }
L50:
  ptr = k * (k - 1) / 2 + hess;
  p2 = IP(9);
  IP(7) = IP(7) + 1;
  mgsro(0, n, n, k + 1, k + 1, &FP(11), w, &W(ptr + 1), &IP(12));
  if(IP(12) < 0) goto L200;
  p2 = ptr + 1;
  for(i = 1; i <= k - 1; i++) {
    ptr = p2;
    p2 = p2 + 1;
    alpha = W(ptr);
    c = W(vc + i);
    s = W(vs + i);
    W(ptr) = c * alpha + s * W(p2);
    W(p2) = c * W(p2) - s * alpha;
  }
  givens(&W(p2), &W(p2 + 1), &c, &s);
  W(vc + k) = c;
  W(vs + k) = s;
  p2 = vrn + k;
  alpha = -s * W(p2);
  W(p2) = c * W(p2);
  W(p2 + 1) = alpha;
  FP(11) = FP(11) + 6 * k;
  alpha = fabs(alpha);
  FP(5) = alpha;
  if(k < m && !(IP(3) >= 0 && alpha <= FP(4)) &&
     (IP(6) <= 0 || IP(7) < IP(6)))
    goto L110;
L200:
  ptr = hess + k * (k + 1) / 2;
  p2 = vrn + k;
  if(W(ptr) == 0.0) {
    k = k - 1;
    if(k > 0)
      goto L200;
    else {
      IP(1) = -3;
      IP(12) = -4;
      goto L300;
    }
  }
  W(p2) = W(p2) / W(ptr);
  for(i = k - 1; i >= 1; i--) {
    ptr = ptr - i - 1;
    for(ii = 1; ii <= i; ii++) W(vrn + ii) = W(vrn + ii) - W(p2) * W(ptr + ii);
    p2 = p2 - 1;
    W(p2) = W(p2) / W(ptr);
  }
  for(i = 0; i <= k - 1; i++) {
    ptr = iz + i * n;
    for(ii = 1; ii <= n; ii++) sol[ii - 1] = sol[ii - 1] + W(p2) * W(ptr + ii);
    p2 = p2 + 1;
  }
  FP(11) = FP(11) + 2 * k * n + k * (k + 1);
  if(IP(3) == 999) {
    IP(1) = 10;
    IP(8) = -1;
    IP(9) = idx + 1;
    IP(10) = 6;
    return;
  }
  else if(IP(3) < 0) {
    if(IP(7) <= m + 1) {
      FP(3) = fabs(W(vrn + 1));
      if(IP(3) == -1) FP(4) = FP(1) * FP(3) + FP(2);
    }
    FP(6) = fabs(W(vrn + k));
  }
  else if(IP(3) != 999)
    FP(6) = FP(5);
L60:
  if(IP(12) != 0) {
    IP(1) = -3;
    goto L300;
  }
  if((IP(7) < IP(6) || IP(6) <= 0) &&
     ((IP(3) == 999 && IP(11) == 0) || (IP(3) != 999 && FP(6) > FP(4))))
    goto L100;
  if(IP(1) > 0) {
    if(IP(3) == 999 && IP(11) == 1)
      IP(1) = 0;
    else if(IP(3) != 999 && FP(6) <= FP(4))
      IP(1) = 0;
    else if(IP(7) >= IP(6) && IP(6) > 0)
      IP(1) = -1;
    else
      IP(1) = -10;
  }
L300:
  if(FP(3) != 0.0 && FP(6) != 0.0 && IP(7) > IP(13))
    FP(7) = log10(FP(3) / FP(6)) / (double)(IP(7) - IP(13));
  else
    FP(7) = 0.0;
}
#undef W

/* ------------------------------------------------------------------------ */
/* Out-of-scope routines: stubs that report "not restated"                  */
/* ------------------------------------------------------------------------ */
static void not_restated(const char *name)
{
  fprintf(stderr, "Sparskit routine '%s' is not restated in this oracle\n",
          name);
}

void ilut_(int *n, double *a, int *ja, int *ia, int *lfil, double *droptol,
           sscalar *alu, int *jlu, int *ju, int *iwk, double *w, int *jw,
           int *ierr)
{
  not_restated("ilut");
  *ierr = -1;
}
void ilutp_(int *n, double *a, int *ja, int *ia, int *lfil, double *droptol,
            double *permtol, int *mbloc, sscalar *alu, int *jlu, int *ju,
            int *iwk, double *w, int *jw, int *iperm, int *ierr)
{
  not_restated("ilutp");
  *ierr = -1;
}
void ilud_(int *n, double *a, int *ja, int *ia, double *alph, double *tol,
           sscalar *alu, int *jlu, int *ju, int *iwk, double *w, int *jw,
           int *ierr)
{
  not_restated("ilud");
  *ierr = -1;
}
void iludp_(int *n, double *a, int *ja, int *ia, double *alph, double *droptol,
            double *permtol, int *mbloc, sscalar *alu, int *jlu, int *ju,
            int *iwk, double *w, int *jw, int *iperm, int *ierr)
{
  not_restated("iludp");
  *ierr = -1;
}
void iluk_(int *n, double *a, int *ja, int *ia, int *lfil, sscalar *alu,
           int *jlu, int *ju, int *levs, int *iwk, double *w, int *jw,
           int *ierr)
{
  not_restated("iluk");
  *ierr = -1;
}
void milu0_(int *n, double *a, int *ja, int *ia, sscalar *alu, int *jlu,
            int *ju, int *iw, int *ierr)
{
  not_restated("milu0");
  *ierr = -1;
}

#define KRYLOV_STUB(fname, label)                                              \
  void fname(int *n, double *rhs, double *sol, int *ipar, double *fpar,       \
             double *w)                                                        \
  {                                                                            \
    not_restated(label);                                                       \
    IP(1) = -10;                                                               \
  }
KRYLOV_STUB(cgnr_, "cgnr")
KRYLOV_STUB(bcg_, "bcg")
KRYLOV_STUB(dbcg_, "dbcg")
KRYLOV_STUB(bcgstab_, "bcgstab")
KRYLOV_STUB(tfqmr_, "tfqmr")
KRYLOV_STUB(fom_, "fom")
KRYLOV_STUB(dqgmres_, "dqgmres")

void pgmres_(int *n, int *im, double *rhs, double *sol, double *vv,
             double *eps, int *maxits, int *iout, double *aa, int *ja, int *ia,
             sscalar *alu, int *jlu, int *ju, int *ierr)
{
  not_restated("pgmres");
  *ierr = -1;
}
void flu_(int *ipar, double *fpar, double *a, double *lu, int *n, int *nn,
          double *b, double *x, double *dx, double *sol, double *w)
{
  not_restated("flu");
}
void skit_(int *n, double *a, int *ja, int *ia, int *ifmt, int *iounit,
           int *ierr)
{
  not_restated("skit");
  *ierr = 0;
}
void psplot_(int *n, int *ja, int *ia, int *iunt, int *ptitle)
{
  not_restated("psplot");
}
void ma28ad_(void) { not_restated("ma28ad"); }
void ma28cd_(void) { not_restated("ma28cd"); }
