/*
 * ORACLE — test infrastructure only, never shipped or measured as the product.
 *
 * CPU restatement of GetDP's Generate element loop for the canonical
 * Galerkin terms the GPU kernels implement, following the reference's
 * arithmetic order so that element matrices agree to the last bit on the
 * same compiler settings:
 *
 *   Treatment_FemFormulation element loop   src/kernel/Treatment_Formulation.cpp:413-618
 *   Cal_GalerkinTermOfFemEquation           src/kernel/Cal_GalerkinTermOfFemEquation.cpp:531-1014
 *     quadrature loop :757-854, product :838-851, symmetric fill :921-924,
 *     scatter :969-975
 *   Get_BFGeoElement / JacobianVol2D / 3D   src/kernel/Get_Geometry.cpp:42-50, :1099-1124, :1435-1469
 *   Get_InverseMatrix                       src/kernel/Get_Geometry.cpp:1755-1807
 *   ChangeOfCoord_Form1/Form2/Form1P/Form2P src/kernel/Get_Geometry.cpp:1883-1949
 *   BF_Node / BF_GradNode                   src/functions/BF_Node.cpp:28-208, :212-680
 *   BF_PerpendicularEdge / Curl             src/functions/BF_Perpendicular.cpp:36-80
 *   BF_Edge / BF_CurlEdge (+ sign)          src/functions/BF_Edge.cpp:95-130, :364-368, :452-485, :720-726
 *   Gauss_Triangle 3 pts, Gauss_Tetrahedron 4 pts (the truncated literals)
 *                                           src/kernel/Gauss_Triangle.h:13-16, Gauss_Tetrahedron.h:13-22
 *   Cal_ProductValue (scalar/tensor x vector) src/functions/Cal_Value.cpp:626-915
 *   Dof_AssembleInMat (unknown -> A, fixed -> b)  src/kernel/DofData.cpp:1464-1542
 *   LinAlg_AddComplexInMatrix (zero parts skipped) src/kernel/LinAlg_SPARSKIT.cpp:402-413
 *   Cal_AssembleTerm_DtDof (x j*omega)      src/kernel/Cal_AssembleTerm.cpp:105-200
 *
 * Matrix contributions are emitted as COO triplets in the reference's call
 * order; oracle_coo_to_csr sums duplicates in that order (the linked-list
 * accumulation of Sparskit.cpp add_matrix_double) and sorts by (row, col)
 * (csr_format, Sparskit.cpp:2186-2217).  Fixed DOFs are homogeneous
 * (value 0), so their RHS contributions vanish as in the reference.
 *
 * Build with -ffp-contract=off so that no multiply-add is fused, matching
 * the reference's x86-64 build on any host.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* quadrature tables, verbatim literals */
static const double XT3[3] = {0.16666666666666, 0.66666666666666, 0.16666666666666};
static const double YT3[3] = {0.16666666666666, 0.16666666666666, 0.66666666666666};
static const double PT3[3] = {0.16666666666666, 0.16666666666666, 0.16666666666666};
static const double XTET4[4] = {0.138196601125, 0.138196601125, 0.138196601125, 0.585410196625};
static const double YTET4[4] = {0.138196601125, 0.138196601125, 0.585410196625, 0.138196601125};
static const double ZTET4[4] = {0.138196601125, 0.585410196625, 0.138196601125, 0.138196601125};
static const double PTET4[4] = {0.0416666666667, 0.0416666666667, 0.0416666666667, 0.0416666666667};

typedef struct {
  double c11, c12, c13, c21, c22, c23, c31, c32, c33;
} M3;

/* RHS accumulation; with g_babs set, also the sum of |contribution| per row
   (the rounding scale of the same sum taken in another order) */
static double *g_babs = NULL;
void oracle_set_rhs_abs(double *babs) { g_babs = babs; }
static void badd(double *b, int row, double v)
{
  b[row] += v;
  if(g_babs) g_babs[row] += fabs(v);
}

/* the same with the rounding scale of v given (a sum whose terms cancel) */
static void badd_scaled(double *b, int row, double v, double scale)
{
  b[row] += v;
  if(g_babs) g_babs[row] += scale;
}

/* the rounding scale of an addition the reference skips (an element matrix
   entry that is exactly 0 here may be rounding residue in another
   evaluation order) */
static void bscale(int row, double scale)
{
  if(g_babs) g_babs[row] += scale;
}

/* Values of the fixed DOFs (NULL: every fixed DOF is 0).  With a table, a
   negative DOF entry d names fixed DOF -d-1 (2 values, re and im, in the
   complex formulation), and Dof_AssembleInMat's elimination
   (DofData.cpp:1489-1542) adds b_i += (g_j * TF) * -Ek_ij, TF = 1. */
static const double *g_fix = NULL;
void oracle_set_fixed(const double *gfix) { g_fix = gfix; }

/* COO sink in call order */
typedef struct {
  int64_t n, cap;
  int32_t *r, *c;
  double *v;
} Coo;

static void coo_add(Coo *m, int r, int c, double v)
{
  if(m->n < m->cap) {
    m->r[m->n] = r;
    m->c[m->n] = c;
    m->v[m->n] = v;
  }
  m->n++;
}

/* ---------------------------------------------------------------------- */
/* geometry                                                                */
/* ---------------------------------------------------------------------- */
static void grad_tri3(double g[3][3])
{
  g[0][0] = -1.; g[0][1] = -1.; g[0][2] = 0.;
  g[1][0] = 1.;  g[1][1] = 0.;  g[1][2] = 0.;
  g[2][0] = 0.;  g[2][1] = 1.;  g[2][2] = 0.;
}

static void grad_tet4(double g[4][3])
{
  g[0][0] = -1.; g[0][1] = -1.; g[0][2] = -1.;
  g[1][0] = 1.;  g[1][1] = 0.;  g[1][2] = 0.;
  g[2][0] = 0.;  g[2][1] = 1.;  g[2][2] = 0.;
  g[3][0] = 0.;  g[3][1] = 0.;  g[3][2] = 1.;
}

static void node_tet10(double u, double v, double w, double s[10])
{
  double r = 1. - u - v - w;
  s[0] = r * (2. * r - 1.);
  s[1] = u * (2. * u - 1.);
  s[2] = v * (2. * v - 1.);
  s[3] = w * (2. * w - 1.);
  s[4] = 4. * r * u;
  s[5] = 4. * u * v;
  s[6] = 4. * r * v;
  s[7] = 4. * r * w;
  s[8] = 4. * v * w;
  s[9] = 4. * u * w;
}

static void grad_tet10(double u, double v, double w, double s[10][3])
{
  double r = 1. - u - v - w;
  s[0][0] = -(4. * r - 1); s[0][1] = -(4. * r - 1); s[0][2] = -(4. * r - 1);
  s[1][0] = (4. * u - 1);  s[1][1] = 0;             s[1][2] = 0;
  s[2][0] = 0;             s[2][1] = (4. * v - 1);  s[2][2] = 0;
  s[3][0] = 0;             s[3][1] = 0;             s[3][2] = (4. * w - 1);
  s[4][0] = 4. * (r - u);  s[4][1] = -4. * u;       s[4][2] = -4. * u;
  s[5][0] = 4. * v;        s[5][1] = 4. * u;        s[5][2] = 0;
  s[6][0] = -4. * v;       s[6][1] = 4. * (r - v);  s[6][2] = -4. * v;
  s[7][0] = -4. * w;       s[7][1] = -4. * w;       s[7][2] = 4. * (r - w);
  s[8][0] = 0;             s[8][1] = 4. * w;        s[8][2] = 4. * v;
  s[9][0] = 4. * w;        s[9][1] = 0;             s[9][2] = 4. * u;
}

static double jac2d(int nn, const double *x, const double *y,
                    double dndu[][3], M3 *J)
{
  int i;
  J->c11 = 0.; J->c12 = 0.; J->c13 = 0.;
  J->c21 = 0.; J->c22 = 0.; J->c23 = 0.;
  J->c31 = 0.; J->c32 = 0.; J->c33 = 1.;
  for(i = 0; i < nn; i++) {
    J->c11 += x[i] * dndu[i][0];
    J->c21 += x[i] * dndu[i][1];
    J->c12 += y[i] * dndu[i][0];
    J->c22 += y[i] * dndu[i][1];
  }
  return J->c11 * J->c22 - J->c12 * J->c21;
}

static double jac3d(int nn, const double *x, const double *y, const double *z,
                    double dndu[][3], M3 *J)
{
  int i;
  J->c11 = 0.; J->c12 = 0.; J->c13 = 0.;
  J->c21 = 0.; J->c22 = 0.; J->c23 = 0.;
  J->c31 = 0.; J->c32 = 0.; J->c33 = 0.;
  for(i = 0; i < nn; i++) {
    J->c11 += x[i] * dndu[i][0];
    J->c21 += x[i] * dndu[i][1];
    J->c31 += x[i] * dndu[i][2];
    J->c12 += y[i] * dndu[i][0];
    J->c22 += y[i] * dndu[i][1];
    J->c32 += y[i] * dndu[i][2];
    J->c13 += z[i] * dndu[i][0];
    J->c23 += z[i] * dndu[i][1];
    J->c33 += z[i] * dndu[i][2];
  }
  return J->c11 * J->c22 * J->c33 + J->c13 * J->c21 * J->c32 +
         J->c12 * J->c23 * J->c31 - J->c13 * J->c22 * J->c31 -
         J->c11 * J->c23 * J->c32 - J->c12 * J->c21 * J->c33;
}

static void inv3d(double D, const M3 *M, M3 *I)
{
  I->c11 = (M->c22 * M->c33 - M->c23 * M->c32) / D;
  I->c21 = -(M->c21 * M->c33 - M->c23 * M->c31) / D;
  I->c31 = (M->c21 * M->c32 - M->c22 * M->c31) / D;
  I->c12 = -(M->c12 * M->c33 - M->c13 * M->c32) / D;
  I->c22 = (M->c11 * M->c33 - M->c13 * M->c31) / D;
  I->c32 = -(M->c11 * M->c32 - M->c12 * M->c31) / D;
  I->c13 = (M->c12 * M->c23 - M->c13 * M->c22) / D;
  I->c23 = -(M->c11 * M->c23 - M->c13 * M->c21) / D;
  I->c33 = (M->c11 * M->c22 - M->c12 * M->c21) / D;
}

static void form1(const M3 *I, const double u[3], double x[3])
{
  x[0] = u[0] * I->c11 + u[1] * I->c12 + u[2] * I->c13;
  x[1] = u[0] * I->c21 + u[1] * I->c22 + u[2] * I->c23;
  x[2] = u[0] * I->c31 + u[1] * I->c32 + u[2] * I->c33;
}

static void form2(const M3 *J, double D, const double u[3], double x[3])
{
  x[0] = (u[0] * J->c11 + u[1] * J->c21 + u[2] * J->c31) / D;
  x[1] = (u[0] * J->c12 + u[1] * J->c22 + u[2] * J->c32) / D;
  x[2] = (u[0] * J->c13 + u[1] * J->c23 + u[2] * J->c33) / D;
}

static double dot3(const double a[3], const double b[3])
{
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

/* ---------------------------------------------------------------------- */
/* 2D nodal P1 a_z: [nu * Dof{d a}, {d a}] + [-js, {a}]  (real), and the   */
/* complex eddy-current variant adding DtDof[sigma * Dof{a}, {a}].          */
/* ---------------------------------------------------------------------- */
static void tri_geom(const double *nodes, const int *el, int q, double x[3],
                     double y[3], M3 *J, double *D, double n[3])
{
  double g[3][3];
  double u = XT3[q], v = YT3[q];
  int i;
  for(i = 0; i < 3; i++) {
    x[i] = nodes[3 * el[i]];
    y[i] = nodes[3 * el[i] + 1];
  }
  n[0] = 1. - u - v;
  n[1] = u;
  n[2] = v;
  grad_tri3(g);
  *D = jac2d(3, x, y, g, J);
}

/* curl of the perpendicular edge function in real coordinates (Form2P) */
static void tri_curl(const M3 *J, double D, int i, double out[3])
{
  double g[3][3], s[3];
  grad_tri3(g);
  s[0] = g[i][1];
  s[1] = -g[i][0];
  s[2] = 0.;
  out[0] = (s[0] * J->c11 + s[1] * J->c21) / D;
  out[1] = (s[0] * J->c12 + s[1] * J->c22) / D;
  out[2] = 0.;
}

/* Nonlinear a_z (the Newton-Raphson formulation of
   templates/Lib_Magnetostatics_a_phi.pro:186-193) at the current solution x:
     [ nu[{d a}] * {d a}, {d a} ]       NoDof: b -= E
     [ dhdb[{d a}] * Dof{d a}, {d a} ]  matrix (full, row-major call order)
     [ -dhdb[{d a}] * {d a}, {d a} ]    NoDof: b -= E
     [ -js[], {a} ]                     NoDof
   with the .pro functions nu[] = nu0 / (1 + k exp(-|b|^2 / b2)),
   dnudb2[] = nu0 (k / b2) exp(-|b|^2 / b2) / (1 + k exp(...))^2,
   dhdb[] = TensorDiag[1,1,1] nu[b] + 2 dnudb2[b] SquDyadicProduct[b];
   {d a} at a Gauss point = sum_i x_i curl(N_i e_z) (fixed DOFs 0). */
static void nl_law(double nu0, double k, double b2, const double bv[3],
                   double *nu, double T[3][3])
{
  double s = bv[0] * bv[0] + bv[1] * bv[1] + bv[2] * bv[2];
  double ex = exp(-s / b2);
  double den = 1. + k * ex;
  *nu = nu0 / den;
  double d2 = nu0 * (k / b2) * ex / (den * den);
  int a, c;
  for(a = 0; a < 3; a++)
    for(c = 0; c < 3; c++) T[a][c] = (a == c ? *nu : 0.) + 2. * d2 * (bv[a] * bv[c]);
}

int64_t oracle_assemble_tri3_nl(int ne, const double *nodes, const int *elems,
                                const int *edofs, const double *nu0,
                                const double *js, const double *sol, double k,
                                double b2, int64_t cap, int32_t *rr, int32_t *cc,
                                double *vv, double *b)
{
  Coo m = {0, cap, rr, cc, vv};
  int e, q, i, j, c;
  for(e = 0; e < ne; e++) {
    const int *el = elems + 3 * e;
    const int *dof = edofs + 3 * e;
    double Ek[3][3], Eb1[3] = {0., 0., 0.}, Eb3[3] = {0., 0., 0.};
    double Sb1[3] = {0., 0., 0.}, Sb3[3] = {0., 0., 0.};  /* sums of |terms| */
    double x[3], y[3], n[3], D, F;
    M3 J;
    for(i = 0; i < 3; i++)
      for(j = 0; j < 3; j++) Ek[i][j] = 0.;
    for(q = 0; q < 3; q++) {
      double cE[3][3], bv[3] = {0., 0., 0.}, T[3][3], nu, hb[3], tb[3];
      tri_geom(nodes, el, q, x, y, &J, &D, n);
      for(i = 0; i < 3; i++) tri_curl(&J, D, i, cE[i]);
      double bs[3] = {0., 0., 0.};  /* rounding scale of the field */
      for(i = 0; i < 3; i++) {
        double a = dof[i] >= 0 ? sol[dof[i]] : (g_fix ? g_fix[-dof[i] - 1] : 0.);
        for(c = 0; c < 3; c++) {
          bv[c] += a * cE[i][c];
          bs[c] += fabs(a * cE[i][c]);
        }
      }
      nl_law(nu0[e], k, b2, bv, &nu, T);
      F = 1. * (PT3[q] * fabs(D));
      for(c = 0; c < 3; c++) {
        hb[c] = nu * bv[c];
        tb[c] = -(T[c][0] * bv[0] + T[c][1] * bv[1] + T[c][2] * bv[2]);
      }
      for(i = 0; i < 3; i++) {
        Eb1[i] += F * dot3(cE[i], hb);
        Eb3[i] += F * dot3(cE[i], tb);
        /* the field's own rounding (nodal values cancel in the curl) enters
           nu and dhdb with the law's sensitivity 1 + 2 |b|^2 / b2 */
        {
          double sens = 1. + 2. * (bv[0] * bv[0] + bv[1] * bv[1]) / b2;
          for(c = 0; c < 3; c++) {
            double tsc = fabs(T[c][0]) * bs[0] + fabs(T[c][1]) * bs[1] + fabs(T[c][2]) * bs[2];
            Sb1[i] += F * fabs(cE[i][c]) * (fabs(nu) * bs[c]) * sens;
            Sb3[i] += F * fabs(cE[i][c]) * tsc * sens;
          }
        }
        for(j = 0; j < 3; j++) {
          double tc[3];
          for(c = 0; c < 3; c++)
            tc[c] = T[c][0] * cE[j][0] + T[c][1] * cE[j][1] + T[c][2] * cE[j][2];
          Ek[i][j] += F * dot3(cE[i], tc);
        }
      }
    }
    for(i = 0; i < 3; i++)
      if(dof[i] >= 0 && Eb1[i]) badd_scaled(b, dof[i], (1. * 1.) * -Eb1[i], Sb1[i]);
    for(i = 0; i < 3; i++)
      for(j = 0; j < 3; j++) {
        if(dof[i] >= 0 && dof[j] >= 0) coo_add(&m, dof[i], dof[j], Ek[i][j]);
        else if(dof[i] >= 0 && g_fix) {
          double sc = fabs(g_fix[-dof[j] - 1]) * sqrt(fabs(Ek[i][i] * Ek[j][j]));
          if(Ek[i][j])
            badd_scaled(b, dof[i], (g_fix[-dof[j] - 1] * 1.) * -Ek[i][j], sc);
          else
            bscale(dof[i], sc);
        }
      }
    for(i = 0; i < 3; i++)
      if(dof[i] >= 0 && Eb3[i]) badd_scaled(b, dof[i], (1. * 1.) * -Eb3[i], Sb3[i]);
    if(js[e] != 0.) {
      double Es[3] = {0., 0., 0.};
      for(q = 0; q < 3; q++) {
        tri_geom(nodes, el, q, x, y, &J, &D, n);
        F = 1. * (PT3[q] * fabs(D));
        for(i = 0; i < 3; i++) Es[i] += F * ((n[i] / J.c33) * (-js[e]));
      }
      for(i = 0; i < 3; i++) {
        if(dof[i] < 0 || !Es[i]) continue;
        badd(b, dof[i], (1. * 1.) * -Es[i]);
      }
    }
  }
  return m.n;
}

int64_t oracle_assemble_tri_p1(int ne, const double *nodes, const int *elems,
                               const int *edofs, const double *nu,
                               const double *js, const double *sigma,
                               double omega, int complex_mode, int64_t cap,
                               int32_t *rr, int32_t *cc, double *vv, double *b)
{
  Coo m = {0, cap, rr, cc, vv};
  int e, q, i, j, k;
  for(e = 0; e < ne; e++) {
    const int *el = elems + 3 * e;
    const int *dof = edofs + 3 * e;
    double Ek[3][3], x[3], y[3], n[3], D, F;
    M3 J;
    /* term 1: nu * curl . curl, symmetric (lower triangle then mirror) */
    for(i = 0; i < 3; i++)
      for(j = 0; j <= i; j++) Ek[i][j] = 0.;
    for(q = 0; q < 3; q++) {
      double cE[3][3], cD[3][3];
      tri_geom(nodes, el, q, x, y, &J, &D, n);
      for(i = 0; i < 3; i++) tri_curl(&J, D, i, cE[i]);
      for(j = 0; j < 3; j++)
        for(k = 0; k < 3; k++) cD[j][k] = nu[e] * cE[j][k];
      F = 1. * (PT3[q] * fabs(D));
      for(i = 0; i < 3; i++)
        for(j = 0; j <= i; j++) Ek[i][j] += F * dot3(cE[i], cD[j]);
    }
    for(i = 1; i < 3; i++)
      for(j = 0; j < i; j++) Ek[j][i] = Ek[i][j];
    for(i = 0; i < 3; i++)
      for(j = 0; j < 3; j++) {
        if(dof[i] >= 0 && dof[j] < 0 && g_fix) { /* fixed: elimination */
          int f = -dof[j] - 1;
          double sc = sqrt(fabs(Ek[i][i] * Ek[j][j]));  /* rounding scale of Ek_ij */
          if(!complex_mode) {
            if(Ek[i][j])
              badd_scaled(b, dof[i], (g_fix[f] * 1.) * -Ek[i][j], fabs(g_fix[f]) * sc);
            else
              bscale(dof[i], fabs(g_fix[f]) * sc);
          }
          else { /* Val = (Ek, 0): valtmp = (-d1 Val0 + d2 Val1, -d1 Val1 - d2 Val0) */
            double d1 = g_fix[2 * f] * 1., d2 = g_fix[2 * f + 1] * 1.;
            double gs = (fabs(d1) + fabs(d2)) * sc;
            badd_scaled(b, dof[i], -d1 * Ek[i][j] + d2 * 0., gs);
            badd_scaled(b, dof[i] + 1, -d1 * 0. - d2 * Ek[i][j], gs);
          }
        }
        if(dof[i] < 0 || dof[j] < 0) continue;
        if(!complex_mode)
          coo_add(&m, dof[i], dof[j], Ek[i][j]);
        else if(Ek[i][j]) { /* AddComplexInMatrix, imaginary part 0 */
          coo_add(&m, dof[i], dof[j], Ek[i][j]);
          coo_add(&m, dof[i] + 1, dof[j] + 1, Ek[i][j]);
        }
      }
    /* term 2 (complex only, conductors): DtDof [sigma * Dof{a}, {a}] */
    if(complex_mode && sigma && sigma[e] != 0.) {
      for(i = 0; i < 3; i++)
        for(j = 0; j <= i; j++) Ek[i][j] = 0.;
      for(q = 0; q < 3; q++) {
        double vE[3], vD[3];
        tri_geom(nodes, el, q, x, y, &J, &D, n);
        for(i = 0; i < 3; i++) vE[i] = n[i] / J.c33; /* Form1P, z comp */
        for(j = 0; j < 3; j++) vD[j] = sigma[e] * vE[j];
        F = 1. * (PT3[q] * fabs(D));
        for(i = 0; i < 3; i++)
          for(j = 0; j <= i; j++) Ek[i][j] += F * (vE[i] * vD[j]);
      }
      for(i = 1; i < 3; i++)
        for(j = 0; j < i; j++) Ek[j][i] = Ek[i][j];
      for(i = 0; i < 3; i++)
        for(j = 0; j < 3; j++) {
          double d1 = -0. * omega, d2 = Ek[i][j] * omega;
          if(dof[i] >= 0 && dof[j] < 0 && g_fix) { /* Val = (d1, d2) */
            int f = -dof[j] - 1;
            double g1 = g_fix[2 * f] * 1., g2 = g_fix[2 * f + 1] * 1.;
            double gs = (fabs(g1) + fabs(g2)) * omega * sqrt(fabs(Ek[i][i] * Ek[j][j]));
            badd_scaled(b, dof[i], -g1 * d1 + g2 * d2, gs);
            badd_scaled(b, dof[i] + 1, -g1 * d2 - g2 * d1, gs);
          }
          if(dof[i] < 0 || dof[j] < 0) continue;
          if(d1) { /* never: the mass term is real */
            coo_add(&m, dof[i], dof[j], d1);
            coo_add(&m, dof[i] + 1, dof[j] + 1, d1);
          }
          if(d2) {
            coo_add(&m, dof[i], dof[j] + 1, -d2);
            coo_add(&m, dof[i] + 1, dof[j], d2);
          }
        }
    }
    /* term 3: [-js, {a}] (NoDof: b -= Ek) */
    if(js[e] != 0.) {
      double Eb[3] = {0., 0., 0.};
      for(q = 0; q < 3; q++) {
        tri_geom(nodes, el, q, x, y, &J, &D, n);
        F = 1. * (PT3[q] * fabs(D));
        for(i = 0; i < 3; i++) Eb[i] += F * ((n[i] / J.c33) * (-js[e]));
      }
      for(i = 0; i < 3; i++) {
        if(dof[i] < 0 || !Eb[i]) continue;
        badd(b, dof[i], (1. * 1.) * -Eb[i]);
      }
    }
  }
  return m.n;
}

/* ---------------------------------------------------------------------- */
/* 3D P2 elasticity: sum_{ij} [-C_ij * Dof{d u_j}, {d u_i}] + [f_z, {u_z}] */
/* ---------------------------------------------------------------------- */
static void lame_tensor(double E, double nu, int ci, int cj, double T[9])
{
  /* Lib_Elasticity_u.pro:98-119 functions, evaluated left to right */
  double a = E * (1. - nu) / (1. + nu) / (1. - 2. * nu);
  double c = E * nu / (1. + nu) / (1. - 2. * nu);
  double bb = E / 2. / (1. + nu);
  int k;
  for(k = 0; k < 9; k++) T[k] = 0.;
  if(ci == cj) {
    T[0] = bb; T[4] = bb; T[8] = bb;
    T[4 * ci] = a;
  }
  else {
    /* C_ij: c at (i, j), b at (j, i) (row-major 3x3) */
    T[3 * ci + cj] = c;
    T[3 * cj + ci] = bb;
  }
  for(k = 0; k < 9; k++) T[k] = -T[k];
}

static void tensor_vec(const double T[9], const double v[3], double r[3])
{
  double a0 = T[0] * v[0] + T[1] * v[1] + T[2] * v[2];
  double a1 = T[3] * v[0] + T[4] * v[1] + T[5] * v[2];
  double a2 = T[6] * v[0] + T[7] * v[1] + T[8] * v[2];
  r[0] = a0;
  r[1] = a1;
  r[2] = a2;
}

int64_t oracle_assemble_tet10_elasticity(int ne, const double *nodes,
                                         const int *elems, const int *edofs,
                                         const double *E, double poisson,
                                         double fz, int64_t cap, int32_t *rr,
                                         int32_t *cc, double *vv, double *b)
{
  Coo m = {0, cap, rr, cc, vv};
  int e, q, i, j, k, ci, cj;
  for(e = 0; e < ne; e++) {
    const int *el = elems + 10 * e;
    const int *dof = edofs + 30 * e;
    double x[10], y[10], z[10];
    double gx[4][10][3], Fq[4], nq[4][10];
    for(i = 0; i < 10; i++) {
      x[i] = nodes[3 * el[i]];
      y[i] = nodes[3 * el[i] + 1];
      z[i] = nodes[3 * el[i] + 2];
    }
    for(q = 0; q < 4; q++) {
      double dndu[10][3], D;
      M3 J, I;
      node_tet10(XTET4[q], YTET4[q], ZTET4[q], nq[q]);
      grad_tet10(XTET4[q], YTET4[q], ZTET4[q], dndu);
      D = jac3d(10, x, y, z, dndu, &J);
      inv3d(D, &J, &I);
      for(i = 0; i < 10; i++) form1(&I, dndu[i], gx[q][i]);
      Fq[q] = 1. * (PTET4[q] * fabs(D));
    }
    /* with the RHS scale accumulator and fixed values: the diagonal of each
       component's (c, c) term, the rounding scale of the eliminations */
    double Dg[3][10];
    if(g_babs && g_fix)
      for(ci = 0; ci < 3; ci++) {
        double T[9];
        lame_tensor(E[e], poisson, ci, ci, T);
        for(i = 0; i < 10; i++) {
          Dg[ci][i] = 0.;
          for(q = 0; q < 4; q++) {
            double cD[3];
            tensor_vec(T, gx[q][i], cD);
            Dg[ci][i] += Fq[q] * dot3(gx[q][i], cD);
          }
        }
      }
    /* the nine terms in .pro order: (x,x),(x,y),(x,z),(y,x),... */
    for(ci = 0; ci < 3; ci++)
      for(cj = 0; cj < 3; cj++) {
        double T[9], Ek[10][10];
        int sym = (ci == cj);
        lame_tensor(E[e], poisson, ci, cj, T);
        for(i = 0; i < 10; i++)
          for(j = 0; j < (sym ? i + 1 : 10); j++) Ek[i][j] = 0.;
        for(q = 0; q < 4; q++) {
          double cD[10][3];
          for(j = 0; j < 10; j++) tensor_vec(T, gx[q][j], cD[j]);
          for(i = 0; i < 10; i++)
            for(j = 0; j < (sym ? i + 1 : 10); j++)
              Ek[i][j] += Fq[q] * dot3(gx[q][i], cD[j]);
        }
        if(sym)
          for(i = 1; i < 10; i++)
            for(j = 0; j < i; j++) Ek[j][i] = Ek[i][j];
        for(i = 0; i < 10; i++)
          for(j = 0; j < 10; j++) {
            int r = dof[10 * ci + i], c = dof[10 * cj + j];
            if(r >= 0 && c < 0 && g_fix) {
              double sc = g_babs ? fabs(g_fix[-c - 1]) * sqrt(fabs(Dg[ci][i] * Dg[cj][j])) : 0.;
              if(Ek[i][j])
                badd_scaled(b, r, (g_fix[-c - 1] * 1.) * -Ek[i][j], sc);
              else
                bscale(r, sc);
            }
            if(r < 0 || c < 0) continue;
            coo_add(&m, r, c, Ek[i][j]);
          }
      }
    /* [CompZ[f], {uz}] */
    {
      double Eb[10];
      for(i = 0; i < 10; i++) Eb[i] = 0.;
      for(q = 0; q < 4; q++)
        for(i = 0; i < 10; i++) Eb[i] += Fq[q] * (nq[q][i] * fz);
      for(i = 0; i < 10; i++) {
        int r = dof[20 + i];
        if(r < 0 || !Eb[i]) continue;
        badd(b, r, (1. * 1.) * -Eb[i]);
      }
    }
  }
  (void)k;
  return m.n;
}

/* ---------------------------------------------------------------------- */
/* 3D Whitney edges: [nu Dof{d a}, {d a}] + [reg*nu Dof{a}, {a}] + [-js, {a}]
 * with js the ring-coil current evaluated at each Gauss point.            */
/* ---------------------------------------------------------------------- */
static void edge_tet(double u, double v, double w, int k, double s[3])
{
  switch(k) {
  case 0: s[0] = 1. - v - w; s[1] = u; s[2] = u; break;
  case 1: s[0] = v; s[1] = 1. - u - w; s[2] = v; break;
  case 2: s[0] = w; s[1] = w; s[2] = 1. - u - v; break;
  case 3: s[0] = -v; s[1] = u; s[2] = 0.; break;
  case 4: s[0] = -w; s[1] = 0.; s[2] = u; break;
  default: s[0] = 0.; s[1] = -w; s[2] = v; break;
  }
}

static void curl_edge_tet(int k, double s[3])
{
  static const double C[6][3] = {{0., -2., 2.}, {2., 0., -2.}, {-2., 2., 0.},
                                 {0., 0., 2.},  {0., -2., 0.}, {2., 0., 0.}};
  s[0] = C[k][0];
  s[1] = C[k][1];
  s[2] = C[k][2];
}

int64_t oracle_assemble_tet4_curlcurl(int ne, const double *nodes,
                                      const int *elems, const int *edofs,
                                      const signed char *esign,
                                      const double *nu, const double *js,
                                      double reg, int64_t cap,
                                      int32_t *rr, int32_t *cc, double *vv,
                                      double *b)
{
  Coo m = {0, cap, rr, cc, vv};
  int e, q, i, j, k;
  double g[4][3];
  grad_tet4(g);
  for(e = 0; e < ne; e++) {
    const int *el = elems + 4 * e;
    const int *dof = edofs + 6 * e;
    const signed char *sg = esign + 6 * e;
    double x[4], y[4], z[4], Ek[6][6];
    M3 J, I;
    double D;
    for(i = 0; i < 4; i++) {
      x[i] = nodes[3 * el[i]];
      y[i] = nodes[3 * el[i] + 1];
      z[i] = nodes[3 * el[i] + 2];
    }
    /* term 1: curl-curl */
    for(i = 0; i < 6; i++)
      for(j = 0; j <= i; j++) Ek[i][j] = 0.;
    for(q = 0; q < 4; q++) {
      double cE[6][3], cD[6][3], F;
      D = jac3d(4, x, y, z, g, &J);
      for(i = 0; i < 6; i++) {
        double s[3];
        curl_edge_tet(i, s);
        if(sg[i] < 0) { s[0] = -s[0]; s[1] = -s[1]; s[2] = -s[2]; }
        form2(&J, D, s, cE[i]);
      }
      for(j = 0; j < 6; j++)
        for(k = 0; k < 3; k++) cD[j][k] = nu[e] * cE[j][k];
      F = 1. * (PTET4[q] * fabs(D));
      for(i = 0; i < 6; i++)
        for(j = 0; j <= i; j++) Ek[i][j] += F * dot3(cE[i], cD[j]);
    }
    for(i = 1; i < 6; i++)
      for(j = 0; j < i; j++) Ek[j][i] = Ek[i][j];
    for(i = 0; i < 6; i++)
      for(j = 0; j < 6; j++)
        if(dof[i] >= 0 && dof[j] >= 0) coo_add(&m, dof[i], dof[j], Ek[i][j]);
    /* term 2: reg * nu * mass */
    for(i = 0; i < 6; i++)
      for(j = 0; j <= i; j++) Ek[i][j] = 0.;
    for(q = 0; q < 4; q++) {
      double vE[6][3], vD[6][3], F, coef = reg * nu[e];
      D = jac3d(4, x, y, z, g, &J);
      inv3d(D, &J, &I);
      for(i = 0; i < 6; i++) {
        double s[3];
        edge_tet(XTET4[q], YTET4[q], ZTET4[q], i, s);
        if(sg[i] < 0) { s[0] = -s[0]; s[1] = -s[1]; s[2] = -s[2]; }
        form1(&I, s, vE[i]);
      }
      for(j = 0; j < 6; j++)
        for(k = 0; k < 3; k++) vD[j][k] = coef * vE[j][k];
      F = 1. * (PTET4[q] * fabs(D));
      for(i = 0; i < 6; i++)
        for(j = 0; j <= i; j++) Ek[i][j] += F * dot3(vE[i], vD[j]);
    }
    for(i = 1; i < 6; i++)
      for(j = 0; j < i; j++) Ek[j][i] = Ek[i][j];
    for(i = 0; i < 6; i++)
      for(j = 0; j < 6; j++)
        if(dof[i] >= 0 && dof[j] >= 0) coo_add(&m, dof[i], dof[j], Ek[i][j]);
    /* term 3: [ -js[], {a} ] with js[] a constant vector per element
       (the curl of the edge interpolant of an analytic potential) */
    if(js[3 * e] != 0. || js[3 * e + 1] != 0. || js[3 * e + 2] != 0.) {
      double Eb[6] = {0., 0., 0., 0., 0., 0.};
      double jv[3];
      jv[0] = -js[3 * e];
      jv[1] = -js[3 * e + 1];
      jv[2] = -js[3 * e + 2];
      for(q = 0; q < 4; q++) {
        double u = XTET4[q], v = YTET4[q], w = ZTET4[q], F;
        D = jac3d(4, x, y, z, g, &J);
        inv3d(D, &J, &I);
        F = 1. * (PTET4[q] * fabs(D));
        for(i = 0; i < 6; i++) {
          double sv[3], xv[3];
          edge_tet(u, v, w, i, sv);
          if(sg[i] < 0) { sv[0] = -sv[0]; sv[1] = -sv[1]; sv[2] = -sv[2]; }
          form1(&I, sv, xv);
          Eb[i] += F * dot3(xv, jv);
        }
      }
      for(i = 0; i < 6; i++) {
        if(dof[i] < 0 || !Eb[i]) continue;
        badd(b, dof[i], (1. * 1.) * -Eb[i]);
      }
    }
  }
  return m.n;
}

/* ---------------------------------------------------------------------- */
/* COO (call order) -> CSR sorted by (row, col), duplicates summed in call */
/* order.  Two stable counting-sort passes (by col, then by row).          */
/* ---------------------------------------------------------------------- */
int64_t oracle_coo_to_csr(int n, int64_t nz, const int32_t *r, const int32_t *c,
                          const double *v, int32_t *indptr, int32_t *indices,
                          double *data, double *absdata)
{
  /* absdata (may be NULL): per entry, the sum of the absolute values of the
     contributions merged into it -- the scale of the rounding error of a
     sum taken in another order */
  int64_t *cnt = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
  int64_t *p1 = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nz ? nz : 1));
  int64_t *p2 = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nz ? nz : 1));
  int64_t k, out = 0;
  int i;
  /* stable sort by column */
  for(k = 0; k < nz; k++) cnt[c[k] + 1]++;
  for(i = 0; i < n; i++) cnt[i + 1] += cnt[i];
  for(k = 0; k < nz; k++) p1[cnt[c[k]]++] = k;
  /* stable sort by row */
  memset(cnt, 0, sizeof(int64_t) * ((size_t)n + 1));
  for(k = 0; k < nz; k++) cnt[r[p1[k]] + 1]++;
  for(i = 0; i < n; i++) cnt[i + 1] += cnt[i];
  for(k = 0; k < nz; k++) p2[cnt[r[p1[k]]]++] = p1[k];
  /* p2 is sorted by (row, col) and, within equal keys, by call order */
  indptr[0] = 0;
  i = 0;
  for(k = 0; k < nz; k++) {
    int64_t s = p2[k];
    if(out > 0 && r[s] == r[p2[k - 1]] && c[s] == indices[out - 1]) {
      data[out - 1] += v[s];
      if(absdata) absdata[out - 1] += fabs(v[s]);
      continue;
    }
    while(i < r[s]) indptr[++i] = (int32_t)out;
    indices[out] = c[s];
    data[out] = v[s];
    if(absdata) absdata[out] = fabs(v[s]);
    out++;
  }
  while(i < n) indptr[++i] = (int32_t)out;
  free(cnt);
  free(p1);
  free(p2);
  return out;
}
