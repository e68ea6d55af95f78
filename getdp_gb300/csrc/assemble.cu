// The Generate element loop on the GPU.
//
// GetDP evaluates Cal_GalerkinTermOfFemEquation one element at a time
// (src/kernel/Treatment_Formulation.cpp:413-618 ->
// src/kernel/Cal_GalerkinTermOfFemEquation.cpp:531-1014) and scatters each
// local entry with LinAlg_AddDoubleInMatrix.  Here one launch evaluates a
// whole formulation for all elements: geometry (JacobianVol2D/3D,
// Get_Geometry.cpp:1099-1124, :1435-1469), basis functions (BF_Node,
// BF_PerpendicularEdge, BF_Edge with orientation signs), the 3/4-point Gauss
// rules with the reference's truncated literals (Gauss_Triangle.h:13-16,
// Gauss_Tetrahedron.h:13-22), the local products, and the scatter into the
// CSR (position found by binary search in the sorted row, added with an
// FP64 atomic).  Fixed (Dirichlet) DOFs are homogeneous, so their RHS
// elimination (DofData.cpp:1489-1542) adds nothing and is skipped.
#include "sparse.cuh"

namespace gb {

__constant__ double c_xt3[3] = {0.16666666666666, 0.66666666666666, 0.16666666666666};
__constant__ double c_yt3[3] = {0.16666666666666, 0.16666666666666, 0.66666666666666};
__constant__ double c_pt3 = 0.16666666666666;
__constant__ double c_xtet4[4] = {0.138196601125, 0.138196601125, 0.138196601125, 0.585410196625};
__constant__ double c_ytet4[4] = {0.138196601125, 0.138196601125, 0.585410196625, 0.138196601125};
__constant__ double c_ztet4[4] = {0.138196601125, 0.585410196625, 0.138196601125, 0.138196601125};
__constant__ double c_ptet4 = 0.0416666666667;

struct CsrView {
  const int *rowptr;
  const int *col;
  double *val;
  int *err;  // set when an element pair is missing from the pattern
};

__device__ __forceinline__ void scatter(const CsrView &A, int r, int c, double v)
{
  int pos = find_col(A.col, A.rowptr[r], A.rowptr[r + 1], c);
  if(pos < 0) {
    atomicExch(A.err, 1);
    return;
  }
  atomicAdd(&A.val[pos], v);
}

// ---------------------------------------------------------------------------
// 2D a_z on 3-node triangles (real, or complex with a j*omega*sigma mass)
// ---------------------------------------------------------------------------
template <int COMPLEX>
__global__ void __launch_bounds__(256)
k_tri3(int ne, const double *__restrict__ nodes, const int *__restrict__ elems,
       const int *__restrict__ edofs, const double *__restrict__ nu,
       const double *__restrict__ js, const double *__restrict__ sigma,
       double omega, const double *__restrict__ omega_e, CsrView A,
       double *__restrict__ b)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if(e >= ne) return;
  int v0 = elems[3 * e], v1 = elems[3 * e + 1], v2 = elems[3 * e + 2];
  double x0 = nodes[3 * v0], y0 = nodes[3 * v0 + 1];
  double x1 = nodes[3 * v1], y1 = nodes[3 * v1 + 1];
  double x2 = nodes[3 * v2], y2 = nodes[3 * v2 + 1];
  int d[3] = {edofs[3 * e], edofs[3 * e + 1], edofs[3 * e + 2]};
  // JacobianVol2D with the constant P1 gradients (-1,-1), (1,0), (0,1):
  // c11 = sum x dN/du, c21 = sum x dN/dv, c12 = sum y dN/du, c22 = sum y dN/dv
  double c11 = -x0 + x1, c21 = -x0 + x2, c12 = -y0 + y1, c22 = -y0 + y2;
  double D = c11 * c22 - c12 * c21;
  double aD = fabs(D);
  // curl of the perpendicular edge functions, Form2P: rotated gradient
  // (dN/dv, -dN/du) mapped by Jac^T / det
  const double gu[3] = {-1., 1., 0.}, gv[3] = {-1., 0., 1.};
  double cx[3], cy[3];
#pragma unroll
  for(int i = 0; i < 3; i++) {
    double s0 = gv[i], s1 = -gu[i];
    cx[i] = (s0 * c11 + s1 * c21) / D;
    cy[i] = (s0 * c12 + s1 * c22) / D;
  }
  double nue = nu[e];
  double K[3][3];
#pragma unroll
  for(int i = 0; i < 3; i++)
#pragma unroll
    for(int j = 0; j <= i; j++) {
      double p = cx[i] * (nue * cx[j]) + cy[i] * (nue * cy[j]);
      double acc = 0.;
#pragma unroll
      for(int q = 0; q < 3; q++) acc += (c_pt3 * aD) * p;
      K[i][j] = acc;
      K[j][i] = acc;
    }
  double sg = COMPLEX ? sigma[e] : 0.;
  double M[3][3];
  if(COMPLEX && sg != 0.) {
#pragma unroll
    for(int i = 0; i < 3; i++)
#pragma unroll
      for(int j = 0; j <= i; j++) {
        double acc = 0.;
#pragma unroll
        for(int q = 0; q < 3; q++) {
          double u = c_xt3[q], v = c_yt3[q];
          double n[3] = {1. - u - v, u, v};
          acc += (c_pt3 * aD) * (n[i] * (sg * n[j]));
        }
        M[i][j] = acc;
        M[j][i] = acc;
      }
  }
#pragma unroll
  for(int i = 0; i < 3; i++) {
    if(d[i] < 0) continue;
#pragma unroll
    for(int j = 0; j < 3; j++) {
      if(d[j] < 0) continue;
      if(!COMPLEX)
        scatter(A, d[i], d[j], K[i][j]);
      else {
        if(K[i][j] != 0.) {
          scatter(A, d[i], d[j], K[i][j]);
          scatter(A, d[i] + 1, d[j] + 1, K[i][j]);
        }
        if(sg != 0.) {
          double w = M[i][j] * (omega_e ? omega_e[e] : omega);
          if(w != 0.) {
            scatter(A, d[i], d[j] + 1, -w);
            scatter(A, d[i] + 1, d[j], w);
          }
        }
      }
    }
  }
  double J = js ? js[e] : 0.;
  if(J != 0.) {
#pragma unroll
    for(int i = 0; i < 3; i++) {
      if(d[i] < 0) continue;
      double acc = 0.;
#pragma unroll
      for(int q = 0; q < 3; q++) {
        double u = c_xt3[q], v = c_yt3[q];
        double n = (i == 0) ? 1. - u - v : (i == 1 ? u : v);
        acc += (c_pt3 * aD) * (n * (-J));
      }
      atomicAdd(&b[d[i]], -acc);
    }
  }
}

// ---------------------------------------------------------------------------
// 3D P2 elasticity, one warp per 10-node tetrahedron
// ---------------------------------------------------------------------------
constexpr int kElWarps = 4;  // elements per 128-thread block

__device__ __forceinline__ void tet10_dndu(int l, double u, double v, double w,
                                           double s[3], double *N)
{
  double r = 1. - u - v - w;
  switch(l) {
  case 0: s[0] = -(4. * r - 1); s[1] = s[0]; s[2] = s[0]; *N = r * (2. * r - 1.); break;
  case 1: s[0] = 4. * u - 1; s[1] = 0; s[2] = 0; *N = u * (2. * u - 1.); break;
  case 2: s[0] = 0; s[1] = 4. * v - 1; s[2] = 0; *N = v * (2. * v - 1.); break;
  case 3: s[0] = 0; s[1] = 0; s[2] = 4. * w - 1; *N = w * (2. * w - 1.); break;
  case 4: s[0] = 4. * (r - u); s[1] = -4. * u; s[2] = -4. * u; *N = 4. * r * u; break;
  case 5: s[0] = 4. * v; s[1] = 4. * u; s[2] = 0; *N = 4. * u * v; break;
  case 6: s[0] = -4. * v; s[1] = 4. * (r - v); s[2] = -4. * v; *N = 4. * r * v; break;
  case 7: s[0] = -4. * w; s[1] = -4. * w; s[2] = 4. * (r - w); *N = 4. * r * w; break;
  case 8: s[0] = 0; s[1] = 4. * w; s[2] = 4. * v; *N = 4. * v * w; break;
  case 9: s[0] = 4. * w; s[1] = 0; s[2] = 4. * u; *N = 4. * u * w; break;
  default: s[0] = s[1] = s[2] = 0.; *N = 0.; break;
  }
}

__device__ __forceinline__ double wsum_all(double v)
{
  for(int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// node pairs (a, b), a <= b, of the 10-node tetrahedron
__constant__ signed char c_pair_a[55] = {
  0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 2, 2, 3,
  3, 3, 3, 3, 3, 3, 4, 4, 4, 4, 4, 4, 5, 5, 5, 5, 5, 6, 6, 6, 6, 7, 7, 7, 8, 8, 9};
__constant__ signed char c_pair_b[55] = {
  0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 1, 2, 3, 4, 5, 6, 7, 8, 9, 2, 3, 4, 5, 6, 7, 8, 9, 3,
  4, 5, 6, 7, 8, 9, 4, 5, 6, 7, 8, 9, 5, 6, 7, 8, 9, 6, 7, 8, 9, 7, 8, 9, 8, 9, 9};

// The nine terms [-C_ij Dof{d u_j}, {d u_i}] of Lib_Elasticity_u.pro with the
// isotropic tensors (a = E(1-nu)/(1+nu)/(1-2nu), c = E nu/(1+nu)/(1-2nu),
// b = E/2/(1+nu)) give, for the node pair (a, b) and Gauss-weighted
// gradients, the 3 x 3 block
//   K_ij = -(b tr(M) delta_ij + c M_ij + b M_ji),  M_ij = sum_q F_q g_a,i g_b,j
// (the diagonal term a g_a,i g_b,i + b sum_{k != i} g_a,k g_b,k equals
// b (g_a . g_b) + (c + b) g_a,i g_b,i, as a = c + 2b).  K_ba = K_ab^T, so
// only the 55 pairs a <= b are evaluated.  One warp per element: the four
// Gauss points' Jacobians on lanes 0-3, the 40 (point, node) gradients on
// all lanes, then the pairs.
//
// B3: the pattern holds 3 x 3 node blocks (checked from the element table:
// component c of node a is row a + c nn for every node with unknowns), so
// the nine entries of a node pair sit at rowptr[row(a, c)] + c' L_a +
// pos_a(b): one search per node pair instead of nine.
template <int B3>
__global__ void __launch_bounds__(32 * kElWarps)
k_tet10_elasticity(int ne, const double *__restrict__ nodes,
                   const int *__restrict__ elems, const int *__restrict__ edofs,
                   const double *__restrict__ E, double poisson, double fz,
                   CsrView A, double *__restrict__ b)
{
  __shared__ double sx[kElWarps][10][3];
  __shared__ double sinv[kElWarps][4][9];
  __shared__ double sF[kElWarps][4];
  __shared__ double sg[kElWarps][4][10][3];   // gradients
  __shared__ double sgF[kElWarps][4][10][3];  // gradients x F_q
  __shared__ int sd[kElWarps][30];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int e = blockIdx.x * kElWarps + w;
  if(e >= ne) return;  // warp-uniform
  if(lane < 10) {
    int v = elems[10 * e + lane];
    sx[w][lane][0] = nodes[3 * v];
    sx[w][lane][1] = nodes[3 * v + 1];
    sx[w][lane][2] = nodes[3 * v + 2];
  }
  if(lane < 30) sd[w][lane] = edofs[30 * e + lane];
  __syncwarp();
  if(lane < 4) {
    // JacobianVol3D at Gauss point q: c_rc = sum_k x_k,c dN_k/du_r
    const int q = lane;
    double c[3][3] = {{0., 0., 0.}, {0., 0., 0.}, {0., 0., 0.}};
    for(int k = 0; k < 10; k++) {
      double s[3], N;
      tet10_dndu(k, c_xtet4[q], c_ytet4[q], c_ztet4[q], s, &N);
#pragma unroll
      for(int r = 0; r < 3; r++)
#pragma unroll
        for(int cc = 0; cc < 3; cc++) c[r][cc] += sx[w][k][cc] * s[r];
    }
    double D = c[0][0] * c[1][1] * c[2][2] + c[0][2] * c[1][0] * c[2][1] +
               c[0][1] * c[1][2] * c[2][0] - c[0][2] * c[1][1] * c[2][0] -
               c[0][0] * c[1][2] * c[2][1] - c[0][1] * c[1][0] * c[2][2];
    double iD = 1. / D;
    double *I = sinv[w][q];
    // i_ab (a physical, b reference): the inverse of the Jacobian
    I[0] = (c[1][1] * c[2][2] - c[1][2] * c[2][1]) * iD;     // i11
    I[1] = -(c[0][1] * c[2][2] - c[0][2] * c[2][1]) * iD;    // i12
    I[2] = (c[0][1] * c[1][2] - c[0][2] * c[1][1]) * iD;     // i13
    I[3] = -(c[1][0] * c[2][2] - c[1][2] * c[2][0]) * iD;    // i21
    I[4] = (c[0][0] * c[2][2] - c[0][2] * c[2][0]) * iD;     // i22
    I[5] = -(c[0][0] * c[1][2] - c[0][2] * c[1][0]) * iD;    // i23
    I[6] = (c[1][0] * c[2][1] - c[1][1] * c[2][0]) * iD;     // i31
    I[7] = -(c[0][0] * c[2][1] - c[0][1] * c[2][0]) * iD;    // i32
    I[8] = (c[0][0] * c[1][1] - c[0][1] * c[1][0]) * iD;     // i33
    sF[w][q] = c_ptet4 * fabs(D);
  }
  __syncwarp();
  for(int t = lane; t < 40; t += 32) {
    int q = t / 10, a = t % 10;
    double s[3], N;
    tet10_dndu(a, c_xtet4[q], c_ytet4[q], c_ztet4[q], s, &N);
    const double *I = sinv[w][q];
    double F = sF[w][q];
#pragma unroll
    for(int r = 0; r < 3; r++) {
      double g = s[0] * I[3 * r] + s[1] * I[3 * r + 1] + s[2] * I[3 * r + 2];
      sg[w][q][a][r] = g;
      sgF[w][q][a][r] = F * g;
    }
  }
  __syncwarp();
  double Ee = E[e];
  double cc = Ee * poisson / (1. + poisson) / (1. - 2. * poisson);
  double cb = Ee / 2. / (1. + poisson);
  const int *d = sd[w];
  for(int p = lane; p < 55; p += 32) {
    const int a = c_pair_a[p], bn = c_pair_b[p];
    double M[3][3];
#pragma unroll
    for(int i = 0; i < 3; i++)
#pragma unroll
      for(int j = 0; j < 3; j++) {
        double m = 0.;
#pragma unroll
        for(int q = 0; q < 4; q++) m += sgF[w][q][a][i] * sg[w][q][bn][j];
        M[i][j] = m;
      }
    const double tr = M[0][0] + M[1][1] + M[2][2];
    double K[3][3];
#pragma unroll
    for(int i = 0; i < 3; i++)
#pragma unroll
      for(int j = 0; j < 3; j++)
        K[i][j] = -((i == j ? cb * tr : 0.) + cc * M[i][j] + cb * M[j][i]);
    // block (a, bn) = K, block (bn, a) = K^T
    for(int side = 0; side < (a == bn ? 1 : 2); side++) {
      const int ra = side ? bn : a, cb_ = side ? a : bn;
      if(B3) {
        int r0 = d[ra], c0 = d[cb_];
        if(r0 < 0 || c0 < 0) continue;  // a node's components: all unknown or all fixed
        int s0 = A.rowptr[r0];
        int L = (A.rowptr[r0 + 1] - s0) / 3;
        int pos = find_col(A.col, s0, s0 + L, c0);
        if(pos < 0) {
          atomicExch(A.err, 1);
          continue;
        }
        pos -= s0;
#pragma unroll
        for(int i = 0; i < 3; i++) {
          int rs = A.rowptr[d[10 * i + ra]];
#pragma unroll
          for(int j = 0; j < 3; j++)
            atomicAdd(&A.val[rs + j * L + pos], side ? K[j][i] : K[i][j]);
        }
      }
      else {
#pragma unroll
        for(int i = 0; i < 3; i++) {
          int r = d[10 * i + ra];
          if(r < 0) continue;
#pragma unroll
          for(int j = 0; j < 3; j++) {
            int c = d[10 * j + cb_];
            if(c >= 0) scatter(A, r, c, side ? K[j][i] : K[i][j]);
          }
        }
      }
    }
  }
  // body force [f, {u_z}]: b -= -sum_q F_q N_a(q) fz on the z rows
  if(lane < 10) {
    double eb = 0.;
    for(int q = 0; q < 4; q++) {
      double s[3], N;
      tet10_dndu(lane, c_xtet4[q], c_ytet4[q], c_ztet4[q], s, &N);
      eb += sF[w][q] * (N * fz);
    }
    int r = d[20 + lane];
    if(r >= 0 && eb != 0.) atomicAdd(&b[r], -eb);
  }
}

// ---------------------------------------------------------------------------
// 3D Whitney edges on 4-node tets: curl-curl + regularising mass + source
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128)
k_tet4_curlcurl(int ne, const double *__restrict__ nodes,
                const int *__restrict__ elems, const int *__restrict__ edofs,
                const signed char *__restrict__ esign,
                const double *__restrict__ nu, const double *__restrict__ js,
                double reg, CsrView A, double *__restrict__ b)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if(e >= ne) return;
  double x[4], y[4], z[4];
#pragma unroll
  for(int i = 0; i < 4; i++) {
    int v = elems[4 * e + i];
    x[i] = nodes[3 * v];
    y[i] = nodes[3 * v + 1];
    z[i] = nodes[3 * v + 2];
  }
  int d[6];
  double sgn[6];
#pragma unroll
  for(int i = 0; i < 6; i++) {
    d[i] = edofs[6 * e + i];
    sgn[i] = esign[6 * e + i] < 0 ? -1. : 1.;
  }
  // JacobianVol3D with the constant P1 gradients
  double c11 = -x[0] + x[1], c21 = -x[0] + x[2], c31 = -x[0] + x[3];
  double c12 = -y[0] + y[1], c22 = -y[0] + y[2], c32 = -y[0] + y[3];
  double c13 = -z[0] + z[1], c23 = -z[0] + z[2], c33 = -z[0] + z[3];
  double D = c11 * c22 * c33 + c13 * c21 * c32 + c12 * c23 * c31 -
             c13 * c22 * c31 - c11 * c23 * c32 - c12 * c21 * c33;
  double i11 = (c22 * c33 - c23 * c32) / D, i21 = -(c21 * c33 - c23 * c31) / D;
  double i31 = (c21 * c32 - c22 * c31) / D, i12 = -(c12 * c33 - c13 * c32) / D;
  double i22 = (c11 * c33 - c13 * c31) / D, i32 = -(c11 * c32 - c12 * c31) / D;
  double i13 = (c12 * c23 - c13 * c22) / D, i23 = -(c11 * c23 - c13 * c21) / D;
  double i33 = (c11 * c22 - c12 * c21) / D;
  double F = c_ptet4 * fabs(D);
  // constant curls of the edge functions (BF_CurlEdge), Form2: Jac^T s / det
  const double CR[6][3] = {{0., -2., 2.}, {2., 0., -2.}, {-2., 2., 0.},
                           {0., 0., 2.},  {0., -2., 0.}, {2., 0., 0.}};
  double cu[6][3];
#pragma unroll
  for(int i = 0; i < 6; i++) {
    double s0 = sgn[i] * CR[i][0], s1 = sgn[i] * CR[i][1], s2 = sgn[i] * CR[i][2];
    cu[i][0] = (s0 * c11 + s1 * c21 + s2 * c31) / D;
    cu[i][1] = (s0 * c12 + s1 * c22 + s2 * c32) / D;
    cu[i][2] = (s0 * c13 + s1 * c23 + s2 * c33) / D;
  }
  double nue = nu[e], mcoef = reg * nue;
  double K[21];
  {
    int t = 0;
#pragma unroll
    for(int i = 0; i < 6; i++)
#pragma unroll
      for(int j = 0; j <= i; j++, t++) {
        double p = cu[i][0] * (nue * cu[j][0]) + cu[i][1] * (nue * cu[j][1]) +
                   cu[i][2] * (nue * cu[j][2]);
        K[t] = 4. * (F * p);
      }
  }
  // [ -js, {a} ] with js constant on the element: j = -js
  double j0 = 0., j1 = 0., j2 = 0.;
  if(js) {
    j0 = -js[3 * e];
    j1 = -js[3 * e + 1];
    j2 = -js[3 * e + 2];
  }
  const bool cl = (j0 != 0. || j1 != 0. || j2 != 0.);
  double eb[6] = {0., 0., 0., 0., 0., 0.};
#pragma unroll
  for(int q = 0; q < 4; q++) {
    double u = c_xtet4[q], v = c_ytet4[q], w = c_ztet4[q];
    double s[6][3] = {{1. - v - w, u, u}, {v, 1. - u - w, v}, {w, w, 1. - u - v},
                      {-v, u, 0.},        {-w, 0., u},        {0., -w, v}};
    double ve[6][3];
#pragma unroll
    for(int i = 0; i < 6; i++) {
      double s0 = sgn[i] * s[i][0], s1 = sgn[i] * s[i][1], s2 = sgn[i] * s[i][2];
      ve[i][0] = s0 * i11 + s1 * i12 + s2 * i13;
      ve[i][1] = s0 * i21 + s1 * i22 + s2 * i23;
      ve[i][2] = s0 * i31 + s1 * i32 + s2 * i33;
    }
    int t = 0;
#pragma unroll
    for(int i = 0; i < 6; i++)
#pragma unroll
      for(int j = 0; j <= i; j++, t++) {
        double p = ve[i][0] * (mcoef * ve[j][0]) + ve[i][1] * (mcoef * ve[j][1]) +
                   ve[i][2] * (mcoef * ve[j][2]);
        K[t] += F * p;
      }
    if(cl) {
#pragma unroll
      for(int i = 0; i < 6; i++)
        eb[i] += F * (ve[i][0] * j0 + ve[i][1] * j1 + ve[i][2] * j2);
    }
  }
  // note: the curl-curl block is the 4-point sum of a constant, K1 = 4 F p,
  // accumulated in the reference as four additions of F*p (a few ulps)
  {
    int t = 0;
#pragma unroll
    for(int i = 0; i < 6; i++)
#pragma unroll
      for(int j = 0; j <= i; j++, t++) {
        if(d[i] >= 0 && d[j] >= 0) {
          scatter(A, d[i], d[j], K[t]);
          if(i != j) scatter(A, d[j], d[i], K[t]);
        }
      }
  }
  if(cl) {
#pragma unroll
    for(int i = 0; i < 6; i++)
      if(d[i] >= 0 && eb[i] != 0.) atomicAdd(&b[d[i]], -eb[i]);
  }
}

// ---------------------------------------------------------------------------
// 2D nonlinear a_z, the Newton-Raphson formulation of
// templates/Lib_Magnetostatics_a_phi.pro:186-193, at the current solution x:
//   [ nu[{d a}] {d a}, {d a} ] + [ dhdb[{d a}] Dof{d a}, {d a} ]
//   + [ -dhdb[{d a}] {d a}, {d a} ] + [ -js, {a} ]
// nu(b) = nu0 / (1 + k exp(-|b|^2 / b2)), dhdb = nu I + 2 dnu/d|b|^2 b b^T.
// {d a} is constant on a P1 triangle: evaluated once, used at every Gauss
// point (the 3-point sums of the reference, over the same constant).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_tri3_nl(int ne, const double *__restrict__ nodes, const int *__restrict__ elems,
          const int *__restrict__ edofs, const double *__restrict__ nu0,
          const double *__restrict__ js, const double *__restrict__ sol, double k,
          double b2, CsrView A, double *__restrict__ b)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if(e >= ne) return;
  int v0 = elems[3 * e], v1 = elems[3 * e + 1], v2 = elems[3 * e + 2];
  double x0 = nodes[3 * v0], y0 = nodes[3 * v0 + 1];
  double c11 = -x0 + nodes[3 * v1], c21 = -x0 + nodes[3 * v2];
  double c12 = -y0 + nodes[3 * v1 + 1], c22 = -y0 + nodes[3 * v2 + 1];
  double D = c11 * c22 - c12 * c21;
  double aD = fabs(D);
  int d[3] = {edofs[3 * e], edofs[3 * e + 1], edofs[3 * e + 2]};
  const double gu[3] = {-1., 1., 0.}, gv[3] = {-1., 0., 1.};
  double cx[3], cy[3], bx = 0., by = 0.;
#pragma unroll
  for(int i = 0; i < 3; i++) {
    double s0 = gv[i], s1 = -gu[i];
    cx[i] = (s0 * c11 + s1 * c21) / D;
    cy[i] = (s0 * c12 + s1 * c22) / D;
    double a = (sol && d[i] >= 0) ? sol[d[i]] : 0.;
    bx += a * cx[i];
    by += a * cy[i];
  }
  double s = bx * bx + by * by;
  double ex = exp(-s / b2);
  double den = 1. + k * ex;
  double n0 = nu0[e];
  double nu = n0 / den;
  double d2 = n0 * (k / b2) * ex / (den * den);
  double t11 = nu + 2. * d2 * (bx * bx), t12 = 2. * d2 * (bx * by);
  double t22 = nu + 2. * d2 * (by * by);
  double F = 3. * (c_pt3 * aD);  // the three Gauss weights of a constant
  double hb0 = nu * bx, hb1 = nu * by;
  double tb0 = -(t11 * bx + t12 * by), tb1 = -(t12 * bx + t22 * by);
  double rhs[3];
#pragma unroll
  for(int i = 0; i < 3; i++) {
    if(d[i] < 0) continue;
#pragma unroll
    for(int j = 0; j < 3; j++) {
      if(d[j] < 0) continue;
      double tc0 = t11 * cx[j] + t12 * cy[j], tc1 = t12 * cx[j] + t22 * cy[j];
      scatter(A, d[i], d[j], F * (cx[i] * tc0 + cy[i] * tc1));
    }
  }
  const double js_e = js ? js[e] : 0.;
#pragma unroll
  for(int i = 0; i < 3; i++) {
    // -(E1 + E3) from the two explicit terms, + the source (N_i integrates
    // to |D| / 6 on the three Gauss points: weights 1/6 at (1-u-v, u, v))
    double e1 = F * (cx[i] * hb0 + cy[i] * hb1);
    double e3 = F * (cx[i] * tb0 + cy[i] * tb1);
    double es = 0.;
    if(js_e != 0.) {
#pragma unroll
      for(int q = 0; q < 3; q++) {
        double u = c_xt3[q], v = c_yt3[q];
        double n[3] = {1. - u - v, u, v};
        es += (c_pt3 * aD) * (n[i] * (-js_e));
      }
    }
    rhs[i] = -e1 - e3 - es;
  }
#pragma unroll
  for(int i = 0; i < 3; i++)
    if(d[i] >= 0 && rhs[i] != 0.) atomicAdd(&b[d[i]], rhs[i]);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct BatchDev {
  DevBuf<double> nodes, coef, source, coef2, coef3;
  DevBuf<int> elems, edofs;
  DevBuf<signed char> esign;
  DevBuf<unsigned char> cflag;
  const double *p_nodes = nullptr, *p_coef = nullptr, *p_source = nullptr,
               *p_coef2 = nullptr, *p_coef3 = nullptr;
  const int *p_elems = nullptr, *p_edofs = nullptr;
  const signed char *p_esign = nullptr;
};

static int term_shape(const gb300_term_batch *t, int *nv, int *nloc)
{
  switch(t->kind) {
  case GB300_TERM_TRI3_MAGNETOSTATIC:
  case GB300_TERM_TRI3_EDDY_COMPLEX: *nv = 3; *nloc = 3; return GB300_OK;
  case GB300_TERM_TET10_ELASTICITY: *nv = 10; *nloc = 30; return GB300_OK;
  case GB300_TERM_TET4_EDGE_CURLCURL: *nv = 4; *nloc = 6; return GB300_OK;
  case GB300_TERM_TRI3_MAGNETOSTATIC_NL: *nv = 3; *nloc = 3; return GB300_OK;
  default: set_error("unknown term kind %d", t->kind); return GB300_ERR_ARG;
  }
}

template <typename T>
static int stage(cudaStream_t st, const T *src, size_t n, int on_device,
                 DevBuf<T> &buf, const T **out)
{
  if(!src) {
    *out = nullptr;
    return GB300_OK;
  }
  if(on_device) {
    *out = src;
    return GB300_OK;
  }
  GB_TRY(buf.alloc(n));
  GB_CUDA(cudaMemcpyAsync(buf.p, src, n * sizeof(T), cudaMemcpyHostToDevice, st));
  *out = buf.p;
  return GB300_OK;
}

static int stage_batch(gb300_ctx *ctx, const gb300_term_batch *t, BatchDev &B,
                       bool need_geometry)
{
  int nv, nloc;
  GB_TRY(term_shape(t, &nv, &nloc));
  cudaStream_t st = ctx->stream;
  size_t ne = (size_t)t->n_elems;
  GB_TRY(stage(st, t->elem_dofs, ne * nloc, t->on_device, B.edofs, &B.p_edofs));
  if(need_geometry) {
    GB_TRY(stage(st, t->nodes, (size_t)t->n_nodes * 3, t->on_device, B.nodes, &B.p_nodes));
    GB_TRY(stage(st, t->elems, ne * nv, t->on_device, B.elems, &B.p_elems));
    GB_TRY(stage(st, t->elem_sign, ne * nloc, t->on_device, B.esign, &B.p_esign));
    GB_TRY(stage(st, t->coef, ne, t->on_device, B.coef, &B.p_coef));
    const size_t nsrc = (t->kind == GB300_TERM_TET4_EDGE_CURLCURL) ? 3 : 1;
    GB_TRY(stage(st, t->source, ne * nsrc, t->on_device, B.source, &B.p_source));
    GB_TRY(stage(st, t->coef3, ne, t->on_device, B.coef3, &B.p_coef3));
  }
  GB_TRY(stage(st, t->coef2, ne, t->on_device, B.coef2, &B.p_coef2));
  return GB300_OK;
}

__global__ void k_flag_nonzero(int ne, const double *__restrict__ c,
                               unsigned char *__restrict__ f)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if(e < ne) f[e] = (c && c[e] != 0.) ? 1 : 0;
}

// Every element holds the three components of each of its nodes either all
// as unknowns numbered a, a + nn, a + 2 nn (GetDP's component-major order,
// nn = n / 3) or all fixed.  Then the rows of a node's three components
// touch the same elements, and their sorted column lists are the node's
// neighbours once per component, in the same order (3 x 3 node blocks).
__global__ void k_check_elem_components(int ne, const int *__restrict__ edofs,
                                        int nn, int *__restrict__ bad)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if(e >= ne) return;
  for(int a = 0; a < 10; a++) {
    int d0 = edofs[30 * e + a], d1 = edofs[30 * e + 10 + a], d2 = edofs[30 * e + 20 + a];
    bool ok = (d0 < 0 && d1 < 0 && d2 < 0) ||
              (d0 >= 0 && d0 < nn && d1 == d0 + nn && d2 == d0 + 2 * nn);
    if(!ok) atomicExch(bad, 1);
  }
}

static int node_components_ok(const gb300_matrix *A, int ne, const int *edofs, bool *ok)
{
  *ok = false;
  if(A->n % 3 || A->n == 0) return GB300_OK;
  cudaStream_t st = A->ctx->stream;
  DevBuf<int> bad;
  GB_TRY(bad.alloc(1));
  GB_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  if(ne > 0)
    k_check_elem_components<<<grid_for(ne, 256), 256, 0, st>>>(ne, edofs, A->n / 3, bad.p);
  int hb = 0;
  GB_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  *ok = (hb == 0);
  return GB300_OK;
}

int generate_pattern(gb300_matrix *A, const gb300_term_batch *t)
{
  int nv, nloc;
  GB_TRY(term_shape(t, &nv, &nloc));
  if(t->n_elems < 0 || (t->n_elems > 0 && !t->elem_dofs)) {
    set_error("term batch without element DOF table");
    return GB300_ERR_ARG;
  }
  BatchDev B;
  GB_TRY(stage_batch(A->ctx, t, B, false));
  int cplx = (t->kind == GB300_TERM_TRI3_EDDY_COMPLEX);
  const unsigned char *flag = nullptr;
  if(cplx) {
    if(A->n % 2) {
      set_error("complex system needs an even number of unknowns");
      return GB300_ERR_ARG;
    }
    GB_TRY(B.cflag.alloc(t->n_elems > 0 ? t->n_elems : 1));
    k_flag_nonzero<<<grid_for(t->n_elems, 256), 256, 0, A->ctx->stream>>>(
      t->n_elems, B.p_coef2, B.cflag.p);
    flag = B.cflag.p;
  }
  A->hr.clear();
  A->hc.clear();
  A->hv.clear();
  bool blocks = false;
  if(t->kind == GB300_TERM_TET10_ELASTICITY)
    GB_TRY(node_components_ok(A, t->n_elems, B.p_edofs, &blocks));
  GB_TRY(build_pattern_from_elements(A, t->n_elems, nloc, B.p_edofs, flag, cplx,
                                     blocks ? 3 : 1));
  // the elasticity tables number unknowns component by component; the
  // solver checks the block structure itself before relying on it
  A->block3 = (t->kind == GB300_TERM_TET10_ELASTICITY);
  A->block_rows = cplx ? 2 : 1;
  A->node_blocks = blocks;
  return GB300_OK;
}

int generate_values(gb300_matrix *A, gb300_vector *b, const gb300_term_batch *t,
                    const gb300_vector *x)
{
  if(x && x->n != A->n) {
    set_error("solution size %d != matrix size %d", x->n, A->n);
    return GB300_ERR_ARG;
  }
  if(!A->csr_valid) {
    set_error("matrix has no pattern: call gb300_generate_pattern first");
    return GB300_ERR_ARG;
  }
  if(b->n != A->n) {
    set_error("rhs size %d != matrix size %d", b->n, A->n);
    return GB300_ERR_ARG;
  }
  BatchDev B;
  GB_TRY(stage_batch(A->ctx, t, B, true));
  cudaStream_t st = A->ctx->stream;
  DevBuf<int> err;
  GB_TRY(err.alloc(1));
  GB_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  CsrView V{A->rowptr.p, A->col.p, A->val.p, err.p};
  int ne = t->n_elems;
  if(ne > 0) {
    switch(t->kind) {
    case GB300_TERM_TRI3_MAGNETOSTATIC:
      k_tri3<0><<<grid_for(ne, 256), 256, 0, st>>>(ne, B.p_nodes, B.p_elems,
                                                     B.p_edofs, B.p_coef,
                                                     B.p_source, nullptr, 0.,
                                                     nullptr, V, b->d.p);
      break;
    case GB300_TERM_TRI3_EDDY_COMPLEX:
      k_tri3<1><<<grid_for(ne, 256), 256, 0, st>>>(ne, B.p_nodes, B.p_elems,
                                                     B.p_edofs, B.p_coef,
                                                     B.p_source, B.p_coef2,
                                                     t->p0, B.p_coef3, V, b->d.p);
      break;
    case GB300_TERM_TET10_ELASTICITY:
      if(A->node_blocks)
        k_tet10_elasticity<1><<<grid_for(ne, kElWarps), 32 * kElWarps, 0, st>>>(
          ne, B.p_nodes, B.p_elems, B.p_edofs, B.p_coef, t->p0, t->p1, V, b->d.p);
      else
        k_tet10_elasticity<0><<<grid_for(ne, kElWarps), 32 * kElWarps, 0, st>>>(
          ne, B.p_nodes, B.p_elems, B.p_edofs, B.p_coef, t->p0, t->p1, V, b->d.p);
      break;
    case GB300_TERM_TRI3_MAGNETOSTATIC_NL:
      k_tri3_nl<<<grid_for(ne, 256), 256, 0, st>>>(ne, B.p_nodes, B.p_elems, B.p_edofs,
                                                    B.p_coef, B.p_source,
                                                    x ? x->d.p : nullptr, t->p0, t->p1,
                                                    V, b->d.p);
      break;
    case GB300_TERM_TET4_EDGE_CURLCURL:
      if(!B.p_esign) {
        set_error("edge elements need elem_sign");
        return GB300_ERR_ARG;
      }
      k_tet4_curlcurl<<<grid_for(ne, 128), 128, 0, st>>>(
        ne, B.p_nodes, B.p_elems, B.p_edofs, B.p_esign, B.p_coef, B.p_source,
        t->p0, V, b->d.p);
      break;
    }
    GB_CUDA(cudaGetLastError());
  }
  int herr = 0;
  GB_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(herr) {
    set_error("an element couples a DOF pair missing from the matrix pattern");
    return GB300_ERR_ARG;
  }
  A->val32_valid = false;
  return GB300_OK;
}

}  // namespace gb
