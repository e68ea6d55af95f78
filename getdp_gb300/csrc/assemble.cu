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
// FP64 atomic).  Fixed (Dirichlet) DOFs with values are eliminated into the
// RHS as Dof_AssembleInMat does (DofData.cpp:1489-1542): b_i += (g_j * 1) *
// -Ek_ij for every unknown row i and fixed column j of the element.
#include <chrono>

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

// DET: the launch holds elements of one colour (no two share an unknown):
// plain adds, in the same order on every run; else FP64 atomics
template <int DET = 0>
__device__ __forceinline__ void scatter(const CsrView &A, int r, int c, double v)
{
  int pos = find_col(A.col, A.rowptr[r], A.rowptr[r + 1], c);
  if(pos < 0) {
    atomicExch(A.err, 1);
    return;
  }
  if(DET)
    A.val[pos] += v;
  else
    atomicAdd(&A.val[pos], v);
}

template <int DET> __device__ __forceinline__ void radd(double *b, int r, double v)
{
  if(DET)
    b[r] += v;
  else
    atomicAdd(&b[r], v);
}

// ---------------------------------------------------------------------------
// 2D a_z on 3-node triangles (real, or complex with a j*omega*sigma mass)
// ---------------------------------------------------------------------------
template <int COMPLEX, int DET>
__global__ void __launch_bounds__(256)
k_tri3(int ne, const double *__restrict__ nodes, const int *__restrict__ elems,
       const int *__restrict__ edofs, const double *__restrict__ nu,
       const double *__restrict__ js, const double *__restrict__ sigma,
       double omega, const double *__restrict__ omega_e, CsrView A,
       double *__restrict__ b, const double *__restrict__ gfix,
       const int *__restrict__ elist)
{
  int ei = blockIdx.x * blockDim.x + threadIdx.x;
  if(ei >= ne) return;
  const int e = DET ? elist[ei] : ei;
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
        scatter<DET>(A, d[i], d[j], K[i][j]);
      else {
        if(K[i][j] != 0.) {
          scatter<DET>(A, d[i], d[j], K[i][j]);
          scatter<DET>(A, d[i] + 1, d[j] + 1, K[i][j]);
        }
        if(sg != 0.) {
          double w = M[i][j] * (omega_e ? omega_e[e] : omega);
          if(w != 0.) {
            scatter<DET>(A, d[i], d[j] + 1, -w);
            scatter<DET>(A, d[i] + 1, d[j], w);
          }
        }
      }
    }
  }
  if(gfix) {
    // elimination of fixed DOFs with values: [nu Dof{d a}, {d a}] with the
    // complex value (K, 0), then DtDof with (-0, omega M) (Cal_AssembleTerm
    // _DtDof), each as Dof_AssembleInMat's valtmp = (-d1 v0 + d2 v1,
    // -d1 v1 - d2 v0) for the fixed value d1 + i d2
#pragma unroll
    for(int i = 0; i < 3; i++) {
      if(d[i] < 0) continue;
      double br = 0., bi = 0.;
#pragma unroll
      for(int j = 0; j < 3; j++) {
        if(d[j] >= 0) continue;
        const int f = -d[j] - 1;
        if(!COMPLEX) {
          if(K[i][j] != 0.) br += (gfix[f] * 1.) * -K[i][j];
        }
        else {
          const double d1 = gfix[2 * f] * 1., d2 = gfix[2 * f + 1] * 1.;
          br += -d1 * K[i][j] + d2 * 0.;
          bi += -d1 * 0. - d2 * K[i][j];
          if(sg != 0.) {
            double w = M[i][j] * (omega_e ? omega_e[e] : omega);
            br += -d1 * -0. + d2 * w;
            bi += -d1 * w - d2 * -0.;
          }
        }
      }
      if(br != 0.) radd<DET>(b, d[i], br);
      if(COMPLEX && bi != 0.) radd<DET>(b, d[i] + 1, bi);
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
      radd<DET>(b, d[i], -acc);
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

// per element of the 10-node tetrahedron, the sides of the 55 node pairs
// (a <= b: side 0 the block (a, b), side 1 its transpose (b, a), a != b):
// 100 slots, slot of pair p's side 0 = c_pair_slot[p]
constexpr int kPairSides = 100;
__constant__ unsigned char c_pair_slot[55] = {
  0, 1, 3, 5, 7, 9, 11, 13, 15, 17, 19, 20, 22, 24, 26, 28, 30, 32, 34, 36,
  37, 39, 41, 43, 45, 47, 49, 51, 52, 54, 56, 58, 60, 62, 64, 65, 67, 69, 71,
  73, 75, 76, 78, 80, 82, 84, 85, 87, 89, 91, 92, 94, 96, 97, 99};

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
//
// MODE (scatter): 0 finds each node pair's block by a binary search and adds
// with FP64 atomics; 1 reads the block's offset from the cached position
// table (pairpos, k_tet10_pairpos) and adds with atomics; 2 reads the table
// and adds with plain loads and stores, for the elements of one colour
// (elist: no two of them share a node, hence a row), launched colour by
// colour: no atomics, and every entry is summed in the same order on every
// run.  Fixed DOFs with values (gfix) are eliminated row by row in a fixed
// order from the element's blocks kept in shared memory.
template <int B3, int MODE>
__global__ void __launch_bounds__(32 * kElWarps)
k_tet10_elasticity(int ne, const double *__restrict__ nodes,
                   const int *__restrict__ elems, const int *__restrict__ edofs,
                   const double *__restrict__ E, double poisson, double fz,
                   CsrView A, double *__restrict__ b,
                   const double *__restrict__ gfix, const int *__restrict__ pairpos,
                   const int *__restrict__ elist)
{
  __shared__ double sx[kElWarps][10][3];
  __shared__ double sinv[kElWarps][4][9];
  __shared__ double sF[kElWarps][4];
  __shared__ double sg[kElWarps][4][10][3];   // gradients
  __shared__ double sgF[kElWarps][4][10][3];  // gradients x F_q
  __shared__ int sd[kElWarps][30];
  __shared__ double sK[kElWarps][55][9];      // blocks (a, b), a <= b (gfix only)
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int ei = blockIdx.x * kElWarps + w;
  if(ei >= ne) return;  // warp-uniform
  const int e = MODE == 2 ? elist[ei] : ei;
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
    if(gfix) {
#pragma unroll
      for(int i = 0; i < 3; i++)
#pragma unroll
        for(int j = 0; j < 3; j++) sK[w][p][3 * i + j] = K[i][j];
    }
    // block (a, bn) = K, block (bn, a) = K^T
    for(int side = 0; side < (a == bn ? 1 : 2); side++) {
      const int ra = side ? bn : a, cb_ = side ? a : bn;
      if(B3) {
        int r0 = d[ra], c0 = d[cb_];
        if(r0 < 0 || c0 < 0) continue;  // a node's components: all unknown or all fixed
        int s0 = A.rowptr[r0];
        int L = (A.rowptr[r0 + 1] - s0) / 3;
        int pos;
        if(MODE == 0) {
          pos = find_col(A.col, s0, s0 + L, c0);
          if(pos < 0) {
            atomicExch(A.err, 1);
            continue;
          }
          pos -= s0;
        }
        else
          pos = pairpos[(long long)e * kPairSides + c_pair_slot[p] + side];
#pragma unroll
        for(int i = 0; i < 3; i++) {
          int rs = A.rowptr[d[10 * i + ra]];
#pragma unroll
          for(int j = 0; j < 3; j++) {
            double v = side ? K[j][i] : K[i][j];
            if(MODE == 2)
              A.val[rs + j * L + pos] += v;
            else
              atomicAdd(&A.val[rs + j * L + pos], v);
          }
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
  // fixed DOFs with values: row (node a, component i) gets
  // sum over fixed (node bn, component j) of (g * 1) * -K_(a i, bn j), in
  // node and component order, one add per row
  if(gfix) {
    __syncwarp();
    if(lane < 30) {
      const int i = lane / 10, a = lane % 10;
      const int r = d[10 * i + a];
      double acc = 0.;
      if(r >= 0) {
        for(int bn = 0; bn < 10; bn++) {
          const int lo = a < bn ? a : bn, hi = a < bn ? bn : a;
          // pair index of (lo, hi), lo <= hi: pairs before row lo, then hi - lo
          const int pp = lo * 10 - (lo * (lo - 1)) / 2 + (hi - lo);
          for(int j = 0; j < 3; j++) {
            const int c = d[10 * j + bn];
            if(c >= 0) continue;
            const double kij = a <= bn ? sK[w][pp][3 * i + j] : sK[w][pp][3 * j + i];
            if(kij != 0.) acc += (gfix[-c - 1] * 1.) * -kij;
          }
        }
        if(acc != 0.) {
          if(MODE == 2)
            b[r] += acc;
          else
            atomicAdd(&b[r], acc);
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
    if(r >= 0 && eb != 0.) {
      if(MODE == 2)
        b[r] += -eb;
      else
        atomicAdd(&b[r], -eb);
    }
  }
}

// ---------------------------------------------------------------------------
// The same element matrices with LANES lanes per element (4, 8 or 16: eight,
// four or two elements per warp, sixteen per CTA; the tuner picks).  GB300's FP64 pipe (two FMAs per SM per cycle)
// executes a warp instruction at the same cost whatever its active lanes,
// so the warp-per-element layout above, whose Jacobians ran on 4 lanes,
// gradients on 8 of a second pass and node pairs on 23 of a second pass,
// kept the pipe busy with a third of its lanes (measured: 13 active lanes per
// FP64 instruction, pipe 86 % busy).  Here the Jacobian entries (4 points x
// 9), the gradients (4 points x 10 nodes) and the 55 node pairs are spread
// over the eight lanes, and the shape-function derivatives at the Gauss
// points are tabulated once per CTA.  Fixed DOFs with values are not handled
// here (the warp-per-element kernel eliminates them).
// ---------------------------------------------------------------------------
constexpr int kEl8 = 16;  // elements per CTA (16 x LANES threads)

template <int B3, int MODE, int LANES>
__global__ void __launch_bounds__(16 * LANES)
k_tet10_el8(int ne, const double *__restrict__ nodes, const int *__restrict__ elems,
            const int *__restrict__ edofs, const double *__restrict__ E, double poisson,
            double fz, CsrView A, double *__restrict__ b, const int *__restrict__ pairpos,
            const int *__restrict__ elist)
{
  __shared__ double sdN[4][10][3];  // dN_a/du_r at Gauss point q
  __shared__ double sN[4][10];
  __shared__ double sx[kEl8][10][3];
  __shared__ double sJ[kEl8][4][9];
  __shared__ double sinv[kEl8][4][9];
  __shared__ double sF[kEl8][4];
  __shared__ double sg[kEl8][4][10][3];
  __shared__ int sd[kEl8][30];
  const int tid = threadIdx.x;
  for(int t = tid; t < 40; t += 16 * LANES) {
    const int q = t / 10, a = t % 10;
    double s3[3], N;
    tet10_dndu(a, c_xtet4[q], c_ytet4[q], c_ztet4[q], s3, &N);
    sdN[q][a][0] = s3[0];
    sdN[q][a][1] = s3[1];
    sdN[q][a][2] = s3[2];
    sN[q][a] = N;
  }
  __syncthreads();
  const int slot = tid / LANES, sl = tid % LANES;  // element slot, lane in it
  const int ei = blockIdx.x * kEl8 + slot;
  const bool valid = ei < ne;
  const int e = valid ? (MODE == 2 ? elist[ei] : ei) : 0;
  if(valid) {
    for(int k = sl; k < 10; k += LANES) {
      const int v = elems[10LL * e + k];
      sx[slot][k][0] = nodes[3LL * v];
      sx[slot][k][1] = nodes[3LL * v + 1];
      sx[slot][k][2] = nodes[3LL * v + 2];
    }
    for(int k = sl; k < 30; k += LANES) sd[slot][k] = edofs[30LL * e + k];
  }
  __syncwarp();
  // JacobianVol3D entries c_rc(q) = sum_k x_k,c dN_k/du_r, 36 per element
  if(valid)
    for(int t = sl; t < 36; t += LANES) {
      const int q = t / 9, r = (t % 9) / 3, c = t % 3;
      double acc = 0.;
#pragma unroll
      for(int k = 0; k < 10; k++) acc += sx[slot][k][c] * sdN[q][k][r];
      sJ[slot][q][3 * r + c] = acc;
    }
  __syncwarp();
  // determinant and inverse per Gauss point (lanes 0-3)
  if(valid && sl < 4) {
    const int q = sl;
    const double *c = sJ[slot][q];
    // c[3 r + cc] is the reference's c_(r+1)(cc+1)
    const double D = c[0] * c[4] * c[8] + c[2] * c[3] * c[7] + c[1] * c[5] * c[6] -
                     c[2] * c[4] * c[6] - c[0] * c[5] * c[7] - c[1] * c[3] * c[8];
    const double iD = 1. / D;
    double *I = sinv[slot][q];
    I[0] = (c[4] * c[8] - c[5] * c[7]) * iD;
    I[1] = -(c[1] * c[8] - c[2] * c[7]) * iD;
    I[2] = (c[1] * c[5] - c[2] * c[4]) * iD;
    I[3] = -(c[3] * c[8] - c[5] * c[6]) * iD;
    I[4] = (c[0] * c[8] - c[2] * c[6]) * iD;
    I[5] = -(c[0] * c[5] - c[2] * c[3]) * iD;
    I[6] = (c[3] * c[7] - c[4] * c[6]) * iD;
    I[7] = -(c[0] * c[7] - c[1] * c[6]) * iD;
    I[8] = (c[0] * c[4] - c[1] * c[3]) * iD;
    sF[slot][q] = c_ptet4 * fabs(D);
  }
  __syncwarp();
  // gradients, 40 (point, node) per element
  if(valid)
    for(int t = sl; t < 40; t += LANES) {
      const int q = t / 10, a = t % 10;
      const double *I = sinv[slot][q];
      const double s0 = sdN[q][a][0], s1 = sdN[q][a][1], s2 = sdN[q][a][2];
#pragma unroll
      for(int r = 0; r < 3; r++) sg[slot][q][a][r] = s0 * I[3 * r] + s1 * I[3 * r + 1] + s2 * I[3 * r + 2];
    }
  __syncwarp();
  if(!valid) return;  // no warp-wide step follows
  const double Ee = E[e];
  const double cc = Ee * poisson / (1. + poisson) / (1. - 2. * poisson);
  const double cb = Ee / 2. / (1. + poisson);
  const int *d = sd[slot];
  const double F0 = sF[slot][0], F1 = sF[slot][1], F2 = sF[slot][2], F3 = sF[slot][3];
  for(int p = sl; p < 55; p += LANES) {
    const int a = c_pair_a[p], bn = c_pair_b[p];
    double M[3][3];
#pragma unroll
    for(int i = 0; i < 3; i++) {
      const double ga0 = F0 * sg[slot][0][a][i], ga1 = F1 * sg[slot][1][a][i];
      const double ga2 = F2 * sg[slot][2][a][i], ga3 = F3 * sg[slot][3][a][i];
#pragma unroll
      for(int j = 0; j < 3; j++)
        M[i][j] = ga0 * sg[slot][0][bn][j] + ga1 * sg[slot][1][bn][j] +
                  ga2 * sg[slot][2][bn][j] + ga3 * sg[slot][3][bn][j];
    }
    const double tr = M[0][0] + M[1][1] + M[2][2];
    double K[3][3];
#pragma unroll
    for(int i = 0; i < 3; i++)
#pragma unroll
      for(int j = 0; j < 3; j++)
        K[i][j] = -((i == j ? cb * tr : 0.) + cc * M[i][j] + cb * M[j][i]);
    for(int side = 0; side < (a == bn ? 1 : 2); side++) {
      const int ra = side ? bn : a, cb_ = side ? a : bn;
      if(B3) {
        const int r0 = d[ra], c0 = d[cb_];
        if(r0 < 0 || c0 < 0) continue;
        const int s0 = A.rowptr[r0];
        const int L = (A.rowptr[r0 + 1] - s0) / 3;
        int pos;
        if(MODE == 0) {
          pos = find_col(A.col, s0, s0 + L, c0);
          if(pos < 0) {
            atomicExch(A.err, 1);
            continue;
          }
          pos -= s0;
        }
        else
          pos = pairpos[(long long)e * kPairSides + c_pair_slot[p] + side];
#pragma unroll
        for(int i = 0; i < 3; i++) {
          const int rs = A.rowptr[d[10 * i + ra]];
#pragma unroll
          for(int j = 0; j < 3; j++) {
            const double v = side ? K[j][i] : K[i][j];
            if(MODE == 2)
              A.val[rs + j * L + pos] += v;
            else
              atomicAdd(&A.val[rs + j * L + pos], v);
          }
        }
      }
      else {
#pragma unroll
        for(int i = 0; i < 3; i++) {
          const int r = d[10 * i + ra];
          if(r < 0) continue;
#pragma unroll
          for(int j = 0; j < 3; j++) {
            const int c = d[10 * j + cb_];
            if(c >= 0) scatter<MODE == 2>(A, r, c, side ? K[j][i] : K[i][j]);
          }
        }
      }
    }
  }
  // body force [f, {u_z}] on the z rows
  for(int a = sl; a < 10; a += LANES) {
    double eb = 0.;
#pragma unroll
    for(int q = 0; q < 4; q++) eb += sF[slot][q] * (sN[q][a] * fz);
    const int r = d[20 + a];
    if(r >= 0 && eb != 0.) radd<MODE == 2>(b, r, -eb);
  }
}

// ---------------------------------------------------------------------------
// 3D Whitney edges on 4-node tets: curl-curl + regularising mass + source
// ---------------------------------------------------------------------------
template <int DET>
__global__ void __launch_bounds__(128)
k_tet4_curlcurl(int ne, const double *__restrict__ nodes,
                const int *__restrict__ elems, const int *__restrict__ edofs,
                const signed char *__restrict__ esign,
                const double *__restrict__ nu, const double *__restrict__ js,
                double reg, CsrView A, double *__restrict__ b,
                const int *__restrict__ elist)
{
  int ei = blockIdx.x * blockDim.x + threadIdx.x;
  if(ei >= ne) return;
  const int e = DET ? elist[ei] : ei;
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
          scatter<DET>(A, d[i], d[j], K[t]);
          if(i != j) scatter<DET>(A, d[j], d[i], K[t]);
        }
      }
  }
  if(cl) {
#pragma unroll
    for(int i = 0; i < 6; i++)
      if(d[i] >= 0 && eb[i] != 0.) radd<DET>(b, d[i], -eb[i]);
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
template <int DET>
__global__ void __launch_bounds__(256)
k_tri3_nl(int ne, const double *__restrict__ nodes, const int *__restrict__ elems,
          const int *__restrict__ edofs, const double *__restrict__ nu0,
          const double *__restrict__ js, const double *__restrict__ sol, double k,
          double b2, CsrView A, double *__restrict__ b,
          const double *__restrict__ gfix, const int *__restrict__ elist)
{
  int ei = blockIdx.x * blockDim.x + threadIdx.x;
  if(ei >= ne) return;
  const int e = DET ? elist[ei] : ei;
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
    double a = d[i] >= 0 ? (sol ? sol[d[i]] : 0.) : (gfix ? gfix[-d[i] - 1] : 0.);
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
  double rhs[3], elim[3] = {0., 0., 0.};
#pragma unroll
  for(int i = 0; i < 3; i++) {
    if(d[i] < 0) continue;
#pragma unroll
    for(int j = 0; j < 3; j++) {
      double tc0 = t11 * cx[j] + t12 * cy[j], tc1 = t12 * cx[j] + t22 * cy[j];
      double kij = F * (cx[i] * tc0 + cy[i] * tc1);
      if(d[j] >= 0)
        scatter<DET>(A, d[i], d[j], kij);
      else if(gfix && kij != 0.)
        elim[i] += (gfix[-d[j] - 1] * 1.) * -kij;
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
    rhs[i] = -e1 - e3 - es + elim[i];
  }
#pragma unroll
  for(int i = 0; i < 3; i++)
    if(d[i] >= 0 && rhs[i] != 0.) radd<DET>(b, d[i], rhs[i]);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct BatchDev {
  DevBuf<double> nodes, coef, source, coef2, coef3, fixed;
  const double *p_fixed = nullptr;
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
  if(need_geometry && t->fixed_values) {
    if(t->n_fixed < 0 || t->kind == GB300_TERM_TET4_EDGE_CURLCURL) {
      set_error(t->n_fixed < 0 ? "n_fixed < 0"
                               : "fixed DOF values are not supported for edge elements");
      return t->n_fixed < 0 ? GB300_ERR_ARG : GB300_ERR_UNSUPPORTED;
    }
    const size_t nv2 = (t->kind == GB300_TERM_TRI3_EDDY_COMPLEX) ? 2 : 1;
    if(t->n_fixed > 0)
      GB_TRY(stage(st, t->fixed_values, (size_t)t->n_fixed * nv2, t->on_device, B.fixed,
                   &B.p_fixed));
  }
  return GB300_OK;
}

// every fixed entry of the element table names a fixed DOF of the table
// (-n_fixed <= e < 0), so that the kernels' fixed_values reads stay inside it
__global__ void k_check_fixed(long long n, const int *__restrict__ edofs,
                              int n_fixed, int *__restrict__ bad)
{
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n && edofs[i] < -n_fixed) atomicExch(bad, 1);
}

int check_fixed_table(cudaStream_t st, const int *edofs, long long n, int n_fixed)
{
  DevBuf<int> bad;
  GB_TRY(bad.alloc(1));
  GB_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  if(n > 0) k_check_fixed<<<grid_for(n, 256), 256, 0, st>>>(n, edofs, n_fixed, bad.p);
  int hbad = 0;
  GB_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(hbad) {
    set_error("an element names a fixed DOF beyond n_fixed = %d", n_fixed);
    return GB300_ERR_ARG;
  }
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

// ---------------------------------------------------------------------------
// the Generate cache of a context
// ---------------------------------------------------------------------------
struct GenCache {
  unsigned tag = 0;
  int kind = -1, n = 0, ne = 0, nloc = 0, n_nodes = 0;
  DevBuf<int> edofs;            // the element table the pattern was built from
  DevBuf<int> elems;            // and its element -> node table (colouring)
  DevBuf<unsigned char> cflag;  // complex: elements that couple the harmonics
  DevBuf<int> rowptr, col;
  long long nnz = 0;
  bool node_blocks = false, block3 = false;
  int block_rows = 1;
  // node-blocked elasticity: per element and pair side, the block's offset
  // within its row segment (-1 for a pair with a fixed node)
  DevBuf<int> pairpos;
  bool pairpos_ok = false;
  // element colouring (no two elements of a colour share a node): elements
  // listed colour by colour, colour c = [cptr[c], cptr[c + 1])
  DevBuf<int> celems;
  std::vector<int> cptr;
  // launch shape of the element kernel chosen by the tuner (-1: not yet)
  int shape = -1;
};

static unsigned g_gen_tag = 0;

void gen_cache_free(GenCache *c) { delete c; }

__global__ void k_tables_differ(long long n, const int *__restrict__ a,
                                const int *__restrict__ b, int *__restrict__ diff)
{
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n && a[i] != b[i]) atomicExch(diff, 1);
}

__global__ void k_flags_differ(long long n, const unsigned char *__restrict__ a,
                               const unsigned char *__restrict__ b, int *__restrict__ diff)
{
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n && a[i] != b[i]) atomicExch(diff, 1);
}

// the pattern of A (built or copied) is the cache entry's
static bool linked(const gb300_matrix *A, const GenCache *G)
{
  return G && A->csr_valid && A->gen_tag == G->tag && A->gen_pv == A->pattern_version;
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
  cudaStream_t st = A->ctx->stream;
  int cplx = (t->kind == GB300_TERM_TRI3_EDDY_COMPLEX);
  const unsigned char *flag = nullptr;
  if(cplx) {
    if(A->n % 2) {
      set_error("complex system needs an even number of unknowns");
      return GB300_ERR_ARG;
    }
    GB_TRY(B.cflag.alloc(t->n_elems > 0 ? t->n_elems : 1));
    k_flag_nonzero<<<grid_for(t->n_elems, 256), 256, 0, st>>>(
      t->n_elems, B.p_coef2, B.cflag.p);
    flag = B.cflag.p;
  }
  A->hr.clear();
  A->hc.clear();
  A->hv.clear();
  const long long nent = (long long)t->n_elems * nloc;
  GenCache *G = A->ctx->gen;
  // the same element table as the cached pattern's: reuse it
  if(G && G->kind == t->kind && G->n == A->n && G->ne == t->n_elems && G->nloc == nloc) {
    DevBuf<int> diff;
    GB_TRY(diff.alloc(1));
    GB_CUDA(cudaMemsetAsync(diff.p, 0, sizeof(int), st));
    if(nent > 0)
      k_tables_differ<<<grid_for(nent, 256), 256, 0, st>>>(nent, G->edofs.p, B.p_edofs,
                                                           diff.p);
    if(cplx && t->n_elems > 0)
      k_flags_differ<<<grid_for(t->n_elems, 256), 256, 0, st>>>(t->n_elems, G->cflag.p,
                                                                flag, diff.p);
    int hd = 0;
    GB_CUDA(cudaMemcpyAsync(&hd, diff.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if(!hd) {
      if(!linked(A, G)) {
        GB_TRY(A->rowptr.alloc(A->n + 1));
        GB_TRY(A->col.alloc(G->nnz > 0 ? G->nnz : 1));
        GB_TRY(A->val.alloc(G->nnz > 0 ? G->nnz : 1));
        GB_CUDA(cudaMemcpyAsync(A->rowptr.p, G->rowptr.p, sizeof(int) * (A->n + 1),
                                cudaMemcpyDeviceToDevice, st));
        if(G->nnz > 0)
          GB_CUDA(cudaMemcpyAsync(A->col.p, G->col.p, sizeof(int) * G->nnz,
                                  cudaMemcpyDeviceToDevice, st));
        A->nnz = G->nnz;
        A->csr_valid = true;
        A->pattern_version++;
        A->bsr_var32 = A->bsr_var64 = -1;
        choose_tpr(A);
        A->gen_tag = G->tag;
        A->gen_pv = A->pattern_version;
      }
      if(A->nnz > 0) GB_CUDA(cudaMemsetAsync(A->val.p, 0, sizeof(double) * A->nnz, st));
      A->val32_valid = false;
      gb::coarse_values_changed(A);
      A->block3 = G->block3;
      A->node_blocks = G->node_blocks;
      A->block_rows = G->block_rows;
      GB_CUDA(cudaStreamSynchronize(st));
      return GB300_OK;
    }
  }
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
  // remember this pattern on the context (replacing the previous entry)
  delete A->ctx->gen;
  A->ctx->gen = nullptr;
  G = new GenCache();
  G->tag = ++g_gen_tag;
  G->kind = t->kind;
  G->n = A->n;
  G->ne = t->n_elems;
  G->nloc = nloc;
  G->nnz = A->nnz;
  G->block3 = A->block3;
  G->node_blocks = A->node_blocks;
  G->block_rows = A->block_rows;
  int rc = G->edofs.alloc(nent > 0 ? nent : 1);
  if(rc == GB300_OK) rc = G->rowptr.alloc(A->n + 1);
  if(rc == GB300_OK) rc = G->col.alloc(A->nnz > 0 ? A->nnz : 1);
  if(rc == GB300_OK && cplx) rc = G->cflag.alloc(t->n_elems > 0 ? t->n_elems : 1);
  if(rc != GB300_OK) {  // no room for the cache: the next Generate rebuilds
    delete G;
    cudaGetLastError();
    return GB300_OK;
  }
  if(nent > 0)
    GB_CUDA(cudaMemcpyAsync(G->edofs.p, B.p_edofs, sizeof(int) * nent,
                            cudaMemcpyDeviceToDevice, st));
  GB_CUDA(cudaMemcpyAsync(G->rowptr.p, A->rowptr.p, sizeof(int) * (A->n + 1),
                          cudaMemcpyDeviceToDevice, st));
  if(A->nnz > 0)
    GB_CUDA(cudaMemcpyAsync(G->col.p, A->col.p, sizeof(int) * A->nnz,
                            cudaMemcpyDeviceToDevice, st));
  if(cplx && t->n_elems > 0)
    GB_CUDA(cudaMemcpyAsync(G->cflag.p, flag, t->n_elems, cudaMemcpyDeviceToDevice, st));
  GB_CUDA(cudaStreamSynchronize(st));
  A->ctx->gen = G;
  A->gen_tag = G->tag;
  A->gen_pv = A->pattern_version;
  return GB300_OK;
}

// node-pair block offsets within their row segments (one binary search per
// pair side, once per cached pattern); -1 where a node is fixed, and *err
// set where a pair is missing from the pattern
__global__ void k_tet10_pairpos(int ne, const int *__restrict__ edofs,
                                const int *__restrict__ rowptr, const int *__restrict__ col,
                                int *__restrict__ pairpos, int *__restrict__ err)
{
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= (long long)ne * 55) return;
  int e = (int)(t / 55), p = (int)(t % 55);
  const int a = c_pair_a[p], bn = c_pair_b[p];
  const int *d = edofs + 30LL * e;
  for(int side = 0; side < (a == bn ? 1 : 2); side++) {
    const int ra = side ? bn : a, cb_ = side ? a : bn;
    int r0 = d[ra], c0 = d[cb_];
    int out = -1;
    if(r0 >= 0 && c0 >= 0) {
      int s0 = rowptr[r0];
      int L = (rowptr[r0 + 1] - s0) / 3;
      int pos = find_col(col, s0, s0 + L, c0);
      if(pos < 0)
        atomicExch(err, 1);
      else
        out = pos - s0;
    }
    pairpos[(long long)e * kPairSides + c_pair_slot[p] + side] = out;
  }
}

static int ensure_pairpos(gb300_matrix *A, GenCache *G)
{
  if(G->pairpos_ok) return GB300_OK;
  cudaStream_t st = A->ctx->stream;
  GB_TRY(G->pairpos.alloc((size_t)(G->ne > 0 ? G->ne : 1) * kPairSides));
  DevBuf<int> err;
  GB_TRY(err.alloc(1));
  GB_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  long long work = (long long)G->ne * 55;
  if(work > 0)
    k_tet10_pairpos<<<grid_for(work, 256), 256, 0, st>>>(G->ne, G->edofs.p, A->rowptr.p,
                                                          A->col.p, G->pairpos.p, err.p);
  int he = 0;
  GB_CUDA(cudaMemcpyAsync(&he, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(he) {
    set_error("an element couples a DOF pair missing from the matrix pattern");
    return GB300_ERR_ARG;
  }
  G->pairpos_ok = true;
  return GB300_OK;
}

// node -> elements adjacency of an element -> node table
// unknown -> elements adjacency of an element -> unknown table (fixed
// entries skipped)
__global__ void k_node_count(long long total, const int *__restrict__ elems,
                             int n_nodes, int *__restrict__ cnt, int *__restrict__ bad)
{
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= total) return;
  int v = elems[t];
  if(v >= n_nodes)
    atomicExch(bad, 1);
  else if(v >= 0)
    atomicAdd(&cnt[v], 1);
}

__global__ void k_node_fill(long long total, int nv, const int *__restrict__ elems,
                            int n_nodes, const long long *__restrict__ ptr,
                            int *__restrict__ cursor, int *__restrict__ adj)
{
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= total) return;
  int v = elems[t];
  if(v < 0 || v >= n_nodes) return;
  adj[ptr[v] + atomicAdd(&cursor[v], 1)] = (int)(t / nv);
}

__device__ __forceinline__ unsigned elem_prio(unsigned e)
{
  // integer hash (a bijection of 32-bit values), ties impossible
  e ^= e >> 16;
  e *= 0x7feb352du;
  e ^= e >> 15;
  e *= 0x846ca68bu;
  e ^= e >> 16;
  return e;
}

// one Jones-Plassmann round: an uncoloured element whose uncoloured
// neighbours (elements sharing an unknown) all have lower priority takes the
// smallest colour none of its coloured neighbours has; *left counts the
// elements still uncoloured (a neighbour coloured in this round is seen
// either as coloured or as uncoloured with the higher priority, so two
// neighbours never take a colour in the same round)
__global__ void k_elem_jp_round(int ne, int nv, const int *__restrict__ elems,
                                const long long *__restrict__ ptr,
                                const int *__restrict__ adj, int *colour,
                                int *__restrict__ left, int *__restrict__ too_many)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if(e >= ne || colour[e] >= 0) return;
  const unsigned pe = elem_prio((unsigned)e);
  for(int k = 0; k < nv; k++) {
    int v = elems[(long long)e * nv + k];
    if(v < 0) continue;
    for(long long q = ptr[v]; q < ptr[v + 1]; q++) {
      int f = adj[q];
      if(f != e && colour[f] < 0 && elem_prio((unsigned)f) > pe) {
        atomicAdd(left, 1);
        return;
      }
    }
  }
  for(int base = 0; base < 1024; base += 64) {
    unsigned long long used = 0ull;
    for(int k = 0; k < nv; k++) {
      int v = elems[(long long)e * nv + k];
      if(v < 0) continue;
      for(long long q = ptr[v]; q < ptr[v + 1]; q++) {
        int c = colour[adj[q]] - base;
        if(adj[q] != e && c >= 0 && c < 64) used |= 1ull << c;
      }
    }
    if(~used) {
      colour[e] = base + __ffsll((long long)~used) - 1;
      return;
    }
  }
  atomicExch(too_many, 1);
}

// elements grouped by colour (a stable counting sort on the host: once per
// cached pattern); two elements conflict when they share an unknown (the
// complex tables hold one number per unknown pair)
static int ensure_colouring(gb300_matrix *A, GenCache *G)
{
  const int *d_elems = G->edofs.p;
  const int nv = G->nloc;
  const int n_nodes = A->n;
  if(!G->cptr.empty()) return GB300_OK;
  cudaStream_t st = A->ctx->stream;
  const int ne = G->ne;
  const long long total = (long long)ne * nv;
  DevBuf<int> cnt, cursor, adj, colour, left, flag;
  DevBuf<long long> ptr, tmp;
  GB_TRY(cnt.alloc(n_nodes + 1));
  GB_TRY(cursor.alloc(n_nodes + 1));
  GB_TRY(ptr.alloc(n_nodes + 1));
  GB_TRY(colour.alloc(ne > 0 ? ne : 1));
  GB_TRY(left.alloc(1));
  GB_TRY(flag.alloc(1));
  GB_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * (n_nodes + 1), st));
  GB_CUDA(cudaMemsetAsync(cursor.p, 0, sizeof(int) * (n_nodes + 1), st));
  GB_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), st));
  if(total > 0)
    k_node_count<<<grid_for(total, 256), 256, 0, st>>>(total, d_elems, n_nodes, cnt.p,
                                                       flag.p);
  long long nadj = 0;
  GB_TRY(exclusive_scan(cnt.p, n_nodes + 1, ptr.p, &nadj, tmp, st));
  GB_CUDA(cudaStreamSynchronize(st));
  GB_TRY(adj.alloc(nadj > 0 ? nadj : 1));
  if(total > 0)
    k_node_fill<<<grid_for(total, 256), 256, 0, st>>>(total, nv, d_elems, n_nodes, ptr.p,
                                                      cursor.p, adj.p);
  GB_CUDA(cudaMemsetAsync(colour.p, 0xff, sizeof(int) * (ne > 0 ? ne : 1), st));
  int hleft = ne, rounds = 0;
  while(hleft > 0) {
    if(++rounds > ne + 1) {
      set_error("element colouring did not finish");
      return GB300_ERR_CUDA;
    }
    GB_CUDA(cudaMemsetAsync(left.p, 0, sizeof(int), st));
    k_elem_jp_round<<<grid_for(ne, 256), 256, 0, st>>>(ne, nv, d_elems, ptr.p, adj.p,
                                                       colour.p, left.p, flag.p);
    GB_CUDA(cudaMemcpyAsync(&hleft, left.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
  }
  int hflag = 0;
  GB_CUDA(cudaMemcpyAsync(&hflag, flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  std::vector<int> hc(ne > 0 ? ne : 1);
  if(ne > 0)
    GB_CUDA(cudaMemcpyAsync(hc.data(), colour.p, sizeof(int) * ne, cudaMemcpyDeviceToHost,
                            st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(hflag) {
    set_error("element colouring: an unknown number is out of range or an element "
              "has more than 1024 colours around it");
    return GB300_ERR_ARG;
  }
  int nc = 0;
  for(int e = 0; e < ne; e++) nc = hc[e] + 1 > nc ? hc[e] + 1 : nc;
  std::vector<int> cptr(nc + 1, 0), order(ne > 0 ? ne : 1);
  for(int e = 0; e < ne; e++) cptr[hc[e] + 1]++;
  for(int c = 0; c < nc; c++) cptr[c + 1] += cptr[c];
  std::vector<int> fill(cptr.begin(), cptr.end() - 1);
  for(int e = 0; e < ne; e++) order[fill[hc[e]]++] = e;
  GB_TRY(G->celems.alloc(ne > 0 ? ne : 1));
  if(ne > 0)
    GB_CUDA(cudaMemcpyAsync(G->celems.p, order.data(), sizeof(int) * ne,
                            cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaStreamSynchronize(st));
  G->cptr = cptr;
  return GB300_OK;
}

// launch shapes of the element kernels: P2 elasticity 0 = a warp per
// element, 1/2/3 = 4/8/16 lanes per element (8/4/2 elements per warp); the
// thread-per-element kernels 0/1/2 = 64/128/256 threads per CTA (edge
// elements: 64/128)
static int shape_count(int kind)
{
  if(kind == GB300_TERM_TET10_ELASTICITY) return 4;
  return kind == GB300_TERM_TET4_EDGE_CURLCURL ? 2 : 3;
}
constexpr int kTuneMinElements = 16384;  // smaller batches keep the default
constexpr int kTuneElements = 1 << 17;   // elements timed per shape

static int default_shape(int kind)
{
  // 8 lanes per P2 element; 256 (edge elements: 128) threads per CTA
  return kind == GB300_TERM_TET4_EDGE_CURLCURL ? 1 : 2;
}

static int launch_elements(gb300_matrix *A, const gb300_term_batch *t, const BatchDev &B,
                           const CsrView &V, double *bvec, const gb300_vector *x,
                           const double *gfix, const int *pairpos, int mode, const int *el,
                           int n_l, int shape, cudaStream_t st)
{
  const bool coloured = (mode == GB300_SCATTER_COLOURED);
  // thread-per-element kernels: 64, 128 or 256 threads (their launch bounds)
  const int tpb = 64 << (shape < 2 ? shape : 2);
  switch(t->kind) {
  case GB300_TERM_TRI3_MAGNETOSTATIC:
    if(coloured)
      k_tri3<0, 1><<<grid_for(n_l, tpb), tpb, 0, st>>>(
        n_l, B.p_nodes, B.p_elems, B.p_edofs, B.p_coef, B.p_source, nullptr, 0., nullptr, V,
        bvec, gfix, el);
    else
      k_tri3<0, 0><<<grid_for(n_l, tpb), tpb, 0, st>>>(
        n_l, B.p_nodes, B.p_elems, B.p_edofs, B.p_coef, B.p_source, nullptr, 0., nullptr, V,
        bvec, gfix, nullptr);
    break;
  case GB300_TERM_TRI3_EDDY_COMPLEX:
    if(coloured)
      k_tri3<1, 1><<<grid_for(n_l, tpb), tpb, 0, st>>>(
        n_l, B.p_nodes, B.p_elems, B.p_edofs, B.p_coef, B.p_source, B.p_coef2, t->p0,
        B.p_coef3, V, bvec, gfix, el);
    else
      k_tri3<1, 0><<<grid_for(n_l, tpb), tpb, 0, st>>>(
        n_l, B.p_nodes, B.p_elems, B.p_edofs, B.p_coef, B.p_source, B.p_coef2, t->p0,
        B.p_coef3, V, bvec, gfix, nullptr);
    break;
  case GB300_TERM_TET10_ELASTICITY: {
    const bool nb = A->node_blocks;
    if(coloured && !(nb && pairpos)) {
      set_error("the coloured scatter of the P2 elasticity needs 3 x 3 node blocks");
      return GB300_ERR_UNSUPPORTED;
    }
    if(gfix || shape == 0) {  // a warp per element (it also eliminates fixed values)
      const dim3 g(grid_for(n_l, kElWarps)), blk(32 * kElWarps);
#define GB_EL(B3, M, PP, EL)                                                            \
  k_tet10_elasticity<B3, M><<<g, blk, 0, st>>>(n_l, B.p_nodes, B.p_elems, B.p_edofs,  \
                                                 B.p_coef, t->p0, t->p1, V, bvec, gfix, \
                                                 PP, EL)
      if(coloured)
        GB_EL(1, 2, pairpos, el);
      else if(nb && mode == GB300_SCATTER_TABLE)
        GB_EL(1, 1, pairpos, nullptr);
      else if(nb)
        GB_EL(1, 0, nullptr, nullptr);
      else
        GB_EL(0, 0, nullptr, nullptr);
#undef GB_EL
      break;
    }
    const dim3 g8(grid_for(n_l, kEl8));
#define GB_EL8(B3, M, L, PP, EL)                                                        \
  k_tet10_el8<B3, M, L><<<g8, 16 * L, 0, st>>>(n_l, B.p_nodes, B.p_elems, B.p_edofs,   \
                                               B.p_coef, t->p0, t->p1, V, bvec, PP, EL)
#define GB_EL8_ALL(L)                                   \
  if(coloured)                                          \
    GB_EL8(1, 2, L, pairpos, el);                       \
  else if(nb && mode == GB300_SCATTER_TABLE)            \
    GB_EL8(1, 1, L, pairpos, nullptr);                  \
  else if(nb)                                           \
    GB_EL8(1, 0, L, nullptr, nullptr);                  \
  else                                                  \
    GB_EL8(0, 0, L, nullptr, nullptr);
    if(shape == 1) {
      GB_EL8_ALL(4)
    }
    else if(shape == 3) {
      GB_EL8_ALL(16)
    }
    else {
      GB_EL8_ALL(8)
    }
#undef GB_EL8_ALL
#undef GB_EL8
    break;
  }
  case GB300_TERM_TRI3_MAGNETOSTATIC_NL:
    if(coloured)
      k_tri3_nl<1><<<grid_for(n_l, tpb), tpb, 0, st>>>(
        n_l, B.p_nodes, B.p_elems, B.p_edofs, B.p_coef, B.p_source, x ? x->d.p : nullptr,
        t->p0, t->p1, V, bvec, gfix, el);
    else
      k_tri3_nl<0><<<grid_for(n_l, tpb), tpb, 0, st>>>(
        n_l, B.p_nodes, B.p_elems, B.p_edofs, B.p_coef, B.p_source, x ? x->d.p : nullptr,
        t->p0, t->p1, V, bvec, gfix, nullptr);
    break;
  case GB300_TERM_TET4_EDGE_CURLCURL: {
    const int tt = tpb > 128 ? 128 : tpb;  // its launch bounds: 128 threads
    if(coloured)
      k_tet4_curlcurl<1><<<grid_for(n_l, tt), tt, 0, st>>>(
        n_l, B.p_nodes, B.p_elems, B.p_edofs, B.p_esign, B.p_coef, B.p_source, t->p0, V,
        bvec, el);
    else
      k_tet4_curlcurl<0><<<grid_for(n_l, tt), tt, 0, st>>>(
        n_l, B.p_nodes, B.p_elems, B.p_edofs, B.p_esign, B.p_coef, B.p_source, t->p0, V,
        bvec, nullptr);
    break;
  }
  }
  GB_CUDA(cudaGetLastError());
  return GB300_OK;
}

// max |v_i| as the bits of a non-negative double (ordered as integers):
// per thread over a grid stride, per warp by shuffles, one atomic per warp
// (an atomic per entry on the one address had cost ~150 ms at 229 M entries)
__global__ void k_absmax_bits(long long n, const double *__restrict__ v,
                              unsigned long long *__restrict__ out)
{
  unsigned long long m = 0;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(fabs(v[i]));
    m = b > m ? b : m;
  }
  for(int o = 16; o > 0; o >>= 1) {
    const unsigned long long u = __shfl_down_sync(0xffffffffu, m, o);
    m = u > m ? u : m;
  }
  if((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void k_differs(long long n, const double *__restrict__ a,
                          const double *__restrict__ b, double bound, int *__restrict__ bad)
{
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n && !(fabs(a[i] - b[i]) <= bound)) atomicExch(bad, 1);
}

// times every launch shape on the first kTuneElements elements (scratch
// matrix values and RHS, so that A and b are not touched), checks each
// result against the warp-per-element kernel's (shape 0; 1e-12 of the
// largest entry: the shapes differ only in the order of the additions) and
// keeps the fastest shape that agrees in the cache entry
// host time of the first Generate's one-off steps (GB300_TUNE_VERBOSE)
static double now_ms()
{
  return std::chrono::duration<double, std::milli>(
           std::chrono::steady_clock::now().time_since_epoch())
    .count();
}

static int tune_shape(gb300_matrix *A, GenCache *G, const gb300_term_batch *t,
                      const BatchDev &B, const gb300_vector *x, const int *pairpos, int mode,
                      cudaStream_t st)
{
  const bool verbose = getenv("GB300_TUNE_VERBOSE") != nullptr;
  const double t0 = verbose ? now_ms() : 0.;
  const int n_l = t->n_elems < kTuneElements ? t->n_elems : kTuneElements;
  const long long nnz = A->nnz > 0 ? A->nnz : 1;
  DevBuf<double> sval, rval, sb, rb;
  DevBuf<int> serr, bad;
  DevBuf<unsigned long long> amax;
  GB_TRY(sval.alloc(nnz));
  GB_TRY(rval.alloc(nnz));
  GB_TRY(sb.alloc(A->n > 0 ? A->n : 1));
  GB_TRY(rb.alloc(A->n > 0 ? A->n : 1));
  GB_TRY(serr.alloc(1));
  GB_TRY(bad.alloc(1));
  GB_TRY(amax.alloc(1));
  GB_CUDA(cudaMemsetAsync(serr.p, 0, sizeof(int), st));
  if(verbose) {
    GB_CUDA(cudaStreamSynchronize(st));
    fprintf(stderr, "element tuner: scratch allocated in %.2f ms\n", now_ms() - t0);
  }
  CsrView S{A->rowptr.p, A->col.p, sval.p, serr.p};
  // the coloured scatter's element lists are per colour: tune the same
  // kernels with atomics on the prefix (the arithmetic is the same)
  const int tmode = (mode == GB300_SCATTER_COLOURED)
                      ? (pairpos ? GB300_SCATTER_TABLE : GB300_SCATTER_SEARCH)
                      : mode;
  auto run = [&](int sh) -> int {
    GB_CUDA(cudaMemsetAsync(sval.p, 0, sizeof(double) * nnz, st));
    GB_CUDA(cudaMemsetAsync(sb.p, 0, sizeof(double) * (A->n > 0 ? A->n : 1), st));
    return launch_elements(A, t, B, S, sb.p, x, nullptr, pairpos, tmode, nullptr, n_l, sh,
                           st);
  };
  // the reference result: shape 0
  GB_TRY(run(0));
  GB_CUDA(cudaMemcpyAsync(rval.p, sval.p, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, st));
  GB_CUDA(cudaMemcpyAsync(rb.p, sb.p, sizeof(double) * (A->n > 0 ? A->n : 1),
                          cudaMemcpyDeviceToDevice, st));
  double vmax = 0., bmax = 0.;
  for(int k = 0; k < 2; k++) {
    unsigned long long h = 0;
    GB_CUDA(cudaMemsetAsync(amax.p, 0, sizeof(h), st));
    const long long m = k ? (A->n > 0 ? A->n : 1) : nnz;
    k_absmax_bits<<<grid_for(m, 256, kReduceBlocks * 4), 256, 0, st>>>(m, k ? rb.p : rval.p,
                                                                       amax.p);
    GB_CUDA(cudaMemcpyAsync(&h, amax.p, sizeof(h), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    memcpy(k ? &bmax : &vmax, &h, sizeof(double));
  }
  cudaEvent_t e0, e1;
  GB_CUDA(cudaEventCreate(&e0));
  GB_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int bests = 0;
  for(int sh = 0; sh < shape_count(t->kind); sh++) {
    GB_TRY(run(sh));  // warm-up, and the result to check
    GB_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
    k_differs<<<grid_for(nnz, 256), 256, 0, st>>>(nnz, sval.p, rval.p, 1e-12 * vmax, bad.p);
    if(A->n > 0)
      k_differs<<<grid_for(A->n, 256), 256, 0, st>>>(A->n, sb.p, rb.p, 1e-12 * bmax, bad.p);
    int hbad = 0;
    GB_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaMemsetAsync(sval.p, 0, sizeof(double) * nnz, st));
    GB_CUDA(cudaMemsetAsync(sb.p, 0, sizeof(double) * (A->n > 0 ? A->n : 1), st));
    GB_CUDA(cudaEventRecord(e0, st));
    GB_TRY(launch_elements(A, t, B, S, sb.p, x, nullptr, pairpos, tmode, nullptr, n_l, sh,
                           st));
    GB_CUDA(cudaEventRecord(e1, st));
    GB_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    GB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if(getenv("GB300_TUNE_VERBOSE"))
      fprintf(stderr, "element kernel kind %d shape %d: %.4f ms (%d elements)%s\n", t->kind,
              sh, ms, n_l, hbad ? " rejected: result differs" : "");
    if(!hbad && ms < best) {
      best = ms;
      bests = sh;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  int he = 0;
  GB_CUDA(cudaMemcpyAsync(&he, serr.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(he) {
    set_error("an element couples a DOF pair missing from the matrix pattern");
    return GB300_ERR_ARG;
  }
  G->shape = bests;
  if(verbose) fprintf(stderr, "element tuner: %.2f ms in all\n", now_ms() - t0);
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
  const double *gfix = nullptr;
  if(t->fixed_values && t->n_fixed > 0) {  // (no fixed DOF: nothing to read)
    int nv, nloc;
    GB_TRY(term_shape(t, &nv, &nloc));
    GB_TRY(check_fixed_table(st, B.p_edofs, (long long)t->n_elems * nloc, t->n_fixed));
    gfix = B.p_fixed;
  }
  CsrView V{A->rowptr.p, A->col.p, A->val.p, err.p};
  const int ne = t->n_elems;
  if(t->kind == GB300_TERM_TET4_EDGE_CURLCURL && !B.p_esign) {
    set_error("edge elements need elem_sign");
    return GB300_ERR_ARG;
  }
  // scatter: GB300_SCATTER_DEFAULT takes the position table where there is
  // one (node-blocked elasticity on a cached pattern), else the search
  int mode = t->scatter;
  if(mode < GB300_SCATTER_DEFAULT || mode > GB300_SCATTER_COLOURED) {
    set_error("unknown scatter mode %d", mode);
    return GB300_ERR_ARG;
  }
  GenCache *G = A->ctx->gen;
  const bool cached = linked(A, G) && G->kind == t->kind && G->ne == ne;
  const bool table_ok = cached && A->node_blocks && t->kind == GB300_TERM_TET10_ELASTICITY;
  if(mode == GB300_SCATTER_DEFAULT) mode = table_ok ? GB300_SCATTER_TABLE : GB300_SCATTER_SEARCH;
  if(mode == GB300_SCATTER_TABLE && !table_ok) mode = GB300_SCATTER_SEARCH;
  if(mode == GB300_SCATTER_COLOURED && !cached) {
    set_error("the coloured scatter needs the pattern gb300_generate_pattern built "
              "from this element table");
    return GB300_ERR_ARG;
  }
  const int *pairpos = nullptr;
  if(ne > 0 && table_ok && mode != GB300_SCATTER_SEARCH) {
    const bool verbose = getenv("GB300_TUNE_VERBOSE") != nullptr && !G->pairpos_ok;
    const double t0 = verbose ? now_ms() : 0.;
    GB_TRY(ensure_pairpos(A, G));
    if(verbose) fprintf(stderr, "position table: %.2f ms\n", now_ms() - t0);
    pairpos = G->pairpos.p;
  }
  const bool coloured = (mode == GB300_SCATTER_COLOURED);
  if(coloured && ne > 0) GB_TRY(ensure_colouring(A, G));
  // launch shape: tuned once per cached pattern on a prefix of the elements
  // (into scratch values, so that A and b only ever receive one Generate)
  int shape = default_shape(t->kind);
  if(cached && !gfix && ne >= kTuneMinElements) {
    if(G->shape < 0) GB_TRY(tune_shape(A, G, t, B, x, pairpos, mode, st));
    shape = G->shape;
  }
  // one launch per colour (coloured), else one launch over all elements
  const int nlaunch = (coloured && ne > 0) ? (int)G->cptr.size() - 1 : (ne > 0 ? 1 : 0);
  for(int c = 0; c < nlaunch; c++) {
    const int n_l = coloured ? G->cptr[c + 1] - G->cptr[c] : ne;
    const int *el = coloured ? G->celems.p + G->cptr[c] : nullptr;
    if(n_l <= 0) continue;
    GB_TRY(launch_elements(A, t, B, V, b->d.p, x, gfix, pairpos, mode, el, n_l, shape, st));
  }
  int herr = 0;
  GB_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(herr) {
    set_error("an element couples a DOF pair missing from the matrix pattern");
    return GB300_ERR_ARG;
  }
  A->val32_valid = false;
  gb::coarse_values_changed(A);
  return GB300_OK;
}

}  // namespace gb
