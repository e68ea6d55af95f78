// Post-processing on the GPU: the step after Solve, element-parallel like
// Generate.  PostOperation's Print[ q, OnElementsOf ... ] and Print[ q,
// OnPoint {x,y,z} ] evaluate a local quantity of the solution from the
// element's basis functions (Pos_FemInterpolation.cpp, Cal_PostQuantity.cpp,
// located by Pos_Search.cpp for points).  Supported, with the formulations
// of the Generate kernels:
//   2D a_z on triangles (BF_PerpendicularEdge, real or complex): {a} =
//   (0, 0, sum N_i a_i) and {d a} = sum a_i curl(N_i e_z), mapped by Form2P;
//   3D Whitney edges on tetrahedra (BF_Edge): {a} = sum a_e w_e (Form1,
//   inverse Jacobian) and {d a} = sum a_e curl w_e (Form2, J^T / det).
// Fixed unknowns are the homogeneous Dirichlet values (zero).
//
// Points are located through a uniform grid of buckets over the mesh's
// bounding box (each element listed in every bucket its bounding box
// touches).  A point lying in several elements (on a shared face or edge)
// takes the lowest-numbered one, so the result does not depend on thread
// timing.
#include <algorithm>
#include <cmath>

#include "krylov.cuh"

namespace gb {

// ---------------------------------------------------------------------- 2D
struct Tri3Geo {
  double x0, y0, c11, c21, c12, c22, D;
};

__device__ __forceinline__ Tri3Geo tri3_geo(const double *__restrict__ nodes,
                                            const int *__restrict__ elems, int e)
{
  int v0 = elems[3 * e], v1 = elems[3 * e + 1], v2 = elems[3 * e + 2];
  Tri3Geo g;
  g.x0 = nodes[3 * v0];
  g.y0 = nodes[3 * v0 + 1];
  double x1 = nodes[3 * v1], y1 = nodes[3 * v1 + 1];
  double x2 = nodes[3 * v2], y2 = nodes[3 * v2 + 1];
  // JacobianVol2D (Get_Geometry.cpp): c11 = sum x dN/du, c21 = sum x dN/dv,
  // c12 = sum y dN/du, c22 = sum y dN/dv
  g.c11 = -g.x0 + x1;
  g.c21 = -g.x0 + x2;
  g.c12 = -g.y0 + y1;
  g.c22 = -g.y0 + y2;
  g.D = g.c11 * g.c22 - g.c12 * g.c21;
  return g;
}

// curl(N_i e_z) of the three P1 functions (Form2P: rotated reference
// gradient mapped by Jac^T / det)
__device__ __forceinline__ void tri3_curls(const Tri3Geo &g, double cx[3], double cy[3])
{
  const double gu[3] = {-1., 1., 0.}, gv[3] = {-1., 0., 1.};
#pragma unroll
  for(int i = 0; i < 3; i++) {
    double s0 = gv[i], s1 = -gu[i];
    cx[i] = (s0 * g.c11 + s1 * g.c21) / g.D;
    cy[i] = (s0 * g.c12 + s1 * g.c22) / g.D;
  }
}

// value of local DOF k (harmonic h of NH): the unknown's, or for a fixed
// DOF its value (gfix, NH values per fixed DOF; 0 without a table)
__device__ __forceinline__ double dof_value(const int *__restrict__ edofs, int nloc,
                                            int e, int k, int h,
                                            const double *__restrict__ x,
                                            const double *__restrict__ gfix = nullptr,
                                            int nh = 1)
{
  int d = edofs[(size_t)e * nloc + k];
  if(d >= 0) return x[d + h];
  return gfix ? gfix[(size_t)(-d - 1) * nh + h] : 0.;
}

// b = {d a} per element: out[(e * NH + h) * 2 + c]
template <int NH>
__global__ void k_post_tri3(int ne, const double *__restrict__ nodes,
                            const int *__restrict__ elems, const int *__restrict__ edofs,
                            const double *__restrict__ x, double *__restrict__ out,
                            const double *__restrict__ gfix)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if(e >= ne) return;
  Tri3Geo g = tri3_geo(nodes, elems, e);
  double cx[3], cy[3];
  tri3_curls(g, cx, cy);
#pragma unroll
  for(int h = 0; h < NH; h++) {
    double bx = 0., by = 0.;
#pragma unroll
    for(int i = 0; i < 3; i++) {
      double a = dof_value(edofs, 3, e, i, h, x, gfix, NH);
      bx += a * cx[i];
      by += a * cy[i];
    }
    out[((size_t)e * NH + h) * 2] = bx;
    out[((size_t)e * NH + h) * 2 + 1] = by;
  }
}

// ---------------------------------------------------------------------- 3D
struct Tet4Geo {
  double x0, y0, z0;
  double c11, c21, c31, c12, c22, c32, c13, c23, c33, D;
  double i11, i21, i31, i12, i22, i32, i13, i23, i33;
};

__device__ __forceinline__ Tet4Geo tet4_geo(const double *__restrict__ nodes,
                                            const int *__restrict__ elems, int e)
{
  double x[4], y[4], z[4];
#pragma unroll
  for(int i = 0; i < 4; i++) {
    int v = elems[4 * e + i];
    x[i] = nodes[3 * v];
    y[i] = nodes[3 * v + 1];
    z[i] = nodes[3 * v + 2];
  }
  Tet4Geo g;
  g.x0 = x[0];
  g.y0 = y[0];
  g.z0 = z[0];
  g.c11 = -x[0] + x[1];
  g.c21 = -x[0] + x[2];
  g.c31 = -x[0] + x[3];
  g.c12 = -y[0] + y[1];
  g.c22 = -y[0] + y[2];
  g.c32 = -y[0] + y[3];
  g.c13 = -z[0] + z[1];
  g.c23 = -z[0] + z[2];
  g.c33 = -z[0] + z[3];
  g.D = g.c11 * g.c22 * g.c33 + g.c13 * g.c21 * g.c32 + g.c12 * g.c23 * g.c31 -
        g.c13 * g.c22 * g.c31 - g.c11 * g.c23 * g.c32 - g.c12 * g.c21 * g.c33;
  g.i11 = (g.c22 * g.c33 - g.c23 * g.c32) / g.D;
  g.i21 = -(g.c21 * g.c33 - g.c23 * g.c31) / g.D;
  g.i31 = (g.c21 * g.c32 - g.c22 * g.c31) / g.D;
  g.i12 = -(g.c12 * g.c33 - g.c13 * g.c32) / g.D;
  g.i22 = (g.c11 * g.c33 - g.c13 * g.c31) / g.D;
  g.i32 = -(g.c11 * g.c32 - g.c12 * g.c31) / g.D;
  g.i13 = (g.c12 * g.c23 - g.c13 * g.c22) / g.D;
  g.i23 = -(g.c11 * g.c23 - g.c13 * g.c21) / g.D;
  g.i33 = (g.c11 * g.c22 - g.c12 * g.c21) / g.D;
  return g;
}

// reference-element curls of the six Whitney edge functions (BF_CurlEdge,
// local edges (1,2),(1,3),(1,4),(2,3),(2,4),(3,4) of GeoEntity.h)
__constant__ double c_curl_edge[6][3] = {{0., -2., 2.}, {2., 0., -2.}, {-2., 2., 0.},
                                         {0., 0., 2.},  {0., -2., 0.}, {2., 0., 0.}};

// reference-element values of the six edge functions at (u, v, w) (BF_Edge)
__device__ __forceinline__ void edge_ref(double u, double v, double w, double s[6][3])
{
  s[0][0] = 1. - v - w; s[0][1] = u; s[0][2] = u;
  s[1][0] = v; s[1][1] = 1. - u - w; s[1][2] = v;
  s[2][0] = w; s[2][1] = w; s[2][2] = 1. - u - v;
  s[3][0] = -v; s[3][1] = u; s[3][2] = 0.;
  s[4][0] = -w; s[4][1] = 0.; s[4][2] = u;
  s[5][0] = 0.; s[5][1] = -w; s[5][2] = v;
}

// b = {d a} per element: out[e * 3 + c]
__global__ void k_post_tet4_edge(int ne, const double *__restrict__ nodes,
                                 const int *__restrict__ elems,
                                 const int *__restrict__ edofs,
                                 const signed char *__restrict__ esign,
                                 const double *__restrict__ x, double *__restrict__ out)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if(e >= ne) return;
  Tet4Geo g = tet4_geo(nodes, elems, e);
  double b0 = 0., b1 = 0., b2 = 0.;
#pragma unroll
  for(int i = 0; i < 6; i++) {
    double sg = esign[6 * e + i] < 0 ? -1. : 1.;
    double s0 = sg * c_curl_edge[i][0], s1 = sg * c_curl_edge[i][1],
           s2 = sg * c_curl_edge[i][2];
    double a = dof_value(edofs, 6, e, i, 0, x);
    b0 += a * ((s0 * g.c11 + s1 * g.c21 + s2 * g.c31) / g.D);
    b1 += a * ((s0 * g.c12 + s1 * g.c22 + s2 * g.c32) / g.D);
    b2 += a * ((s0 * g.c13 + s1 * g.c23 + s2 * g.c33) / g.D);
  }
  out[(size_t)e * 3] = b0;
  out[(size_t)e * 3 + 1] = b1;
  out[(size_t)e * 3 + 2] = b2;
}

// ------------------------------------------------------------ point search
struct Grid {
  double lo[3], inv[3];  // bounding box corner, cells per unit length
  int n[3];
  int dim;
  __device__ int cell(double x, int d) const
  {
    int c = (int)floor((x - lo[d]) * inv[d]);
    return c < 0 ? 0 : (c >= n[d] ? n[d] - 1 : c);
  }
};

template <int NV>
__device__ __forceinline__ void elem_box(const double *__restrict__ nodes,
                                         const int *__restrict__ elems, int e,
                                         double lo[3], double hi[3])
{
#pragma unroll
  for(int d = 0; d < 3; d++) {
    lo[d] = 1e300;
    hi[d] = -1e300;
  }
#pragma unroll
  for(int i = 0; i < NV; i++) {
    int v = elems[(size_t)NV * e + i];
#pragma unroll
    for(int d = 0; d < 3; d++) {
      double c = nodes[3 * v + d];
      lo[d] = fmin(lo[d], c);
      hi[d] = fmax(hi[d], c);
    }
  }
}

// PASS 0 counts the elements of each bucket, PASS 1 lists them
template <int NV, int PASS>
__global__ void k_bucket(int ne, const double *__restrict__ nodes,
                         const int *__restrict__ elems, Grid G, int *cnt,
                         const long long *__restrict__ ptr, int *__restrict__ list)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if(e >= ne) return;
  double lo[3], hi[3];
  elem_box<NV>(nodes, elems, e, lo, hi);
  int a[3], b[3];
  for(int d = 0; d < 3; d++) {
    if(d < G.dim) {
      a[d] = G.cell(lo[d], d);
      b[d] = G.cell(hi[d], d);
    }
    else
      a[d] = b[d] = 0;
  }
  for(int k = a[2]; k <= b[2]; k++)
    for(int j = a[1]; j <= b[1]; j++)
      for(int i = a[0]; i <= b[0]; i++) {
        int c = (k * G.n[1] + j) * G.n[0] + i;
        int slot = atomicAdd(&cnt[c], 1);
        if(PASS == 1) list[ptr[c] + slot] = e;
      }
}

__device__ __forceinline__ bool inside(double l0, double l1, double l2, double l3)
{
  const double tol = 1e-10;
  return l0 >= -tol && l1 >= -tol && l2 >= -tol && l3 >= -tol;
}

// the local coordinates of (px, py) in triangle g
__device__ __forceinline__ void tri3_uv(const Tri3Geo &g, double px, double py,
                                        double *u, double *v)
{
  double dx = px - g.x0, dy = py - g.y0;
  // x - x0 = c11 u + c21 v, y - y0 = c12 u + c22 v
  *u = (g.c22 * dx - g.c21 * dy) / g.D;
  *v = (-g.c12 * dx + g.c11 * dy) / g.D;
}

__device__ __forceinline__ void tet4_uvw(const Tet4Geo &g, double px, double py,
                                         double pz, double *u, double *v, double *w)
{
  double dx = px - g.x0, dy = py - g.y0, dz = pz - g.z0;
  // [dx dy dz] = [u v w] J with J rows (c11 c12 c13), (c21 c22 c23),
  // (c31 c32 c33); i_ab = (J^-1)_ab, a physical, b reference
  *u = dx * g.i11 + dy * g.i21 + dz * g.i31;
  *v = dx * g.i12 + dy * g.i22 + dz * g.i32;
  *w = dx * g.i13 + dy * g.i23 + dz * g.i33;
}

// 2D points: a (NH values) and b (2 NH values) of the lowest-numbered
// element containing each point
template <int NH>
__global__ void k_post_points_tri3(int np, const double *__restrict__ xyz, Grid G,
                                   const long long *__restrict__ ptr,
                                   const int *__restrict__ list,
                                   const double *__restrict__ nodes,
                                   const int *__restrict__ elems,
                                   const int *__restrict__ edofs,
                                   const double *__restrict__ x, double *__restrict__ fa,
                                   double *__restrict__ fb, int *__restrict__ fe,
                                   const double *__restrict__ gfix)
{
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if(q >= np) return;
  double px = xyz[3 * q], py = xyz[3 * q + 1];
  int c = G.cell(py, 1) * G.n[0] + G.cell(px, 0);
  int best = -1;
  double bu = 0., bv = 0.;
  for(long long k = ptr[c]; k < ptr[c + 1]; k++) {
    int e = list[k];
    if(best >= 0 && e >= best) continue;
    Tri3Geo g = tri3_geo(nodes, elems, e);
    double u, v;
    tri3_uv(g, px, py, &u, &v);
    if(inside(1. - u - v, u, v, 0.)) {
      best = e;
      bu = u;
      bv = v;
    }
  }
  fe[q] = best;
  for(int h = 0; h < NH; h++) {
    double a = 0., bx = 0., by = 0.;
    if(best >= 0) {
      Tri3Geo g = tri3_geo(nodes, elems, best);
      double cx[3], cy[3];
      tri3_curls(g, cx, cy);
      const double N[3] = {1. - bu - bv, bu, bv};
      for(int i = 0; i < 3; i++) {
        double ai = dof_value(edofs, 3, best, i, h, x, gfix, NH);
        a += N[i] * ai;
        bx += ai * cx[i];
        by += ai * cy[i];
      }
    }
    fa[(size_t)q * NH + h] = a;
    fb[((size_t)q * NH + h) * 2] = bx;
    fb[((size_t)q * NH + h) * 2 + 1] = by;
  }
}

// 3D edge points: a (3 values, Form1) and b (3 values, Form2)
__global__ void k_post_points_tet4_edge(int np, const double *__restrict__ xyz, Grid G,
                                        const long long *__restrict__ ptr,
                                        const int *__restrict__ list,
                                        const double *__restrict__ nodes,
                                        const int *__restrict__ elems,
                                        const int *__restrict__ edofs,
                                        const signed char *__restrict__ esign,
                                        const double *__restrict__ x,
                                        double *__restrict__ fa, double *__restrict__ fb,
                                        int *__restrict__ fe)
{
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if(q >= np) return;
  double px = xyz[3 * q], py = xyz[3 * q + 1], pz = xyz[3 * q + 2];
  int c = (G.cell(pz, 2) * G.n[1] + G.cell(py, 1)) * G.n[0] + G.cell(px, 0);
  int best = -1;
  double bu = 0., bv = 0., bw = 0.;
  for(long long k = ptr[c]; k < ptr[c + 1]; k++) {
    int e = list[k];
    if(best >= 0 && e >= best) continue;
    Tet4Geo g = tet4_geo(nodes, elems, e);
    double u, v, w;
    tet4_uvw(g, px, py, pz, &u, &v, &w);
    if(inside(1. - u - v - w, u, v, w)) {
      best = e;
      bu = u;
      bv = v;
      bw = w;
    }
  }
  fe[q] = best;
  double a0 = 0., a1 = 0., a2 = 0., b0 = 0., b1 = 0., b2 = 0.;
  if(best >= 0) {
    Tet4Geo g = tet4_geo(nodes, elems, best);
    double s[6][3];
    edge_ref(bu, bv, bw, s);
    for(int i = 0; i < 6; i++) {
      double sg = esign[6 * best + i] < 0 ? -1. : 1.;
      double ai = dof_value(edofs, 6, best, i, 0, x);
      double s0 = sg * s[i][0], s1 = sg * s[i][1], s2 = sg * s[i][2];
      a0 += ai * (s0 * g.i11 + s1 * g.i12 + s2 * g.i13);
      a1 += ai * (s0 * g.i21 + s1 * g.i22 + s2 * g.i23);
      a2 += ai * (s0 * g.i31 + s1 * g.i32 + s2 * g.i33);
      double r0 = sg * c_curl_edge[i][0], r1 = sg * c_curl_edge[i][1],
             r2 = sg * c_curl_edge[i][2];
      b0 += ai * ((r0 * g.c11 + r1 * g.c21 + r2 * g.c31) / g.D);
      b1 += ai * ((r0 * g.c12 + r1 * g.c22 + r2 * g.c32) / g.D);
      b2 += ai * ((r0 * g.c13 + r1 * g.c23 + r2 * g.c33) / g.D);
    }
  }
  fa[(size_t)q * 3] = a0;
  fa[(size_t)q * 3 + 1] = a1;
  fa[(size_t)q * 3 + 2] = a2;
  fb[(size_t)q * 3] = b0;
  fb[(size_t)q * 3 + 1] = b1;
  fb[(size_t)q * 3 + 2] = b2;
}

// ------------------------------------------------------------------- host
struct PostIn {
  DevBuf<double> nodes, fixed;
  const double *p_fixed = nullptr;
  DevBuf<int> elems, edofs;
  DevBuf<signed char> esign;
  const double *p_nodes = nullptr;
  const int *p_elems = nullptr, *p_edofs = nullptr;
  const signed char *p_esign = nullptr;
};

template <typename T>
static int stage_in(cudaStream_t st, const T *src, size_t n, int on_device,
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
  GB_TRY(buf.alloc(n > 0 ? n : 1));
  if(n) GB_CUDA(cudaMemcpyAsync(buf.p, src, n * sizeof(T), cudaMemcpyHostToDevice, st));
  *out = buf.p;
  return GB300_OK;
}

static int post_shape(const gb300_term_batch *t, int *nv, int *nloc, int *nh,
                      int *dim)
{
  switch(t->kind) {
  case GB300_TERM_TRI3_MAGNETOSTATIC: *nv = 3; *nloc = 3; *nh = 1; *dim = 2; return GB300_OK;
  case GB300_TERM_TRI3_EDDY_COMPLEX: *nv = 3; *nloc = 3; *nh = 2; *dim = 2; return GB300_OK;
  case GB300_TERM_TET4_EDGE_CURLCURL: *nv = 4; *nloc = 6; *nh = 1; *dim = 3; return GB300_OK;
  default:
    set_error("post-processing is not available for term kind %d", t->kind);
    return GB300_ERR_UNSUPPORTED;
  }
}

static int post_stage(cudaStream_t st, const gb300_term_batch *t, PostIn &I)
{
  int nv, nloc, nh, dim;
  GB_TRY(post_shape(t, &nv, &nloc, &nh, &dim));
  size_t ne = (size_t)t->n_elems;
  GB_TRY(stage_in(st, t->nodes, (size_t)t->n_nodes * 3, t->on_device, I.nodes, &I.p_nodes));
  GB_TRY(stage_in(st, t->elems, ne * nv, t->on_device, I.elems, &I.p_elems));
  GB_TRY(stage_in(st, t->elem_dofs, ne * nloc, t->on_device, I.edofs, &I.p_edofs));
  GB_TRY(stage_in(st, t->elem_sign, ne * nloc, t->on_device, I.esign, &I.p_esign));
  if(t->kind == GB300_TERM_TET4_EDGE_CURLCURL && !I.p_esign) {
    set_error("edge elements need elem_sign");
    return GB300_ERR_ARG;
  }
  if(t->fixed_values && t->n_fixed > 0) {
    if(dim != 2) {
      set_error("fixed DOF values are not supported for edge elements");
      return GB300_ERR_UNSUPPORTED;
    }
    GB_TRY(check_fixed_table(st, I.p_edofs, (long long)ne * nloc, t->n_fixed));
    GB_TRY(stage_in(st, t->fixed_values, (size_t)t->n_fixed * nh, t->on_device, I.fixed,
                    &I.p_fixed));
  }
  return GB300_OK;
}

int post_elements(const gb300_term_batch *t, const gb300_vector *x, double *out)
{
  int nv, nloc, nh, dim;
  GB_TRY(post_shape(t, &nv, &nloc, &nh, &dim));
  cudaStream_t st = x->ctx->stream;
  PostIn I;
  GB_TRY(post_stage(st, t, I));
  const int ne = t->n_elems;
  const int ncomp = dim == 2 ? 2 * nh : 3;
  DevBuf<double> d;
  GB_TRY(d.alloc((size_t)(ne > 0 ? ne : 1) * ncomp));
  if(ne > 0) {
    if(t->kind == GB300_TERM_TRI3_MAGNETOSTATIC)
      k_post_tri3<1><<<grid_for(ne, 256), 256, 0, st>>>(ne, I.p_nodes, I.p_elems,
                                                        I.p_edofs, x->d.p, d.p, I.p_fixed);
    else if(t->kind == GB300_TERM_TRI3_EDDY_COMPLEX)
      k_post_tri3<2><<<grid_for(ne, 256), 256, 0, st>>>(ne, I.p_nodes, I.p_elems,
                                                        I.p_edofs, x->d.p, d.p, I.p_fixed);
    else
      k_post_tet4_edge<<<grid_for(ne, 256), 256, 0, st>>>(ne, I.p_nodes, I.p_elems,
                                                          I.p_edofs, I.p_esign, x->d.p,
                                                          d.p);
    GB_CUDA(cudaGetLastError());
    GB_CUDA(cudaMemcpyAsync(out, d.p, sizeof(double) * ne * ncomp, cudaMemcpyDeviceToHost,
                            st));
  }
  GB_CUDA(cudaStreamSynchronize(st));
  return GB300_OK;
}

int post_points(const gb300_term_batch *t, const gb300_vector *x, int np,
                const double *xyz, double *field, double *curl, int *elem)
{
  int nv, nloc, nh, dim;
  GB_TRY(post_shape(t, &nv, &nloc, &nh, &dim));
  if(np <= 0) return GB300_OK;
  cudaStream_t st = x->ctx->stream;
  PostIn I;
  GB_TRY(post_stage(st, t, I));
  const int ne = t->n_elems;
  // bounding box and bucket grid (about one element per bucket)
  std::vector<double> hn((size_t)t->n_nodes * 3);
  if(t->n_nodes > 0)
    GB_CUDA(cudaMemcpyAsync(hn.data(), I.p_nodes, sizeof(double) * hn.size(),
                            cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  Grid G;
  G.dim = dim;
  for(int d = 0; d < 3; d++) {
    double lo = 1e300, hi = -1e300;
    for(int v = 0; v < t->n_nodes; v++) {
      lo = std::min(lo, hn[3 * v + d]);
      hi = std::max(hi, hn[3 * v + d]);
    }
    if(t->n_nodes == 0) lo = hi = 0.;
    int cells = 1;
    if(d < dim) {
      double per = dim == 2 ? std::sqrt((double)std::max(ne, 1))
                            : std::cbrt((double)std::max(ne, 1));
      cells = std::max(1, std::min(4096, (int)per));
    }
    G.lo[d] = lo;
    G.n[d] = cells;
    G.inv[d] = hi > lo ? cells / (hi - lo) : 0.;
  }
  const long long ncell = (long long)G.n[0] * G.n[1] * G.n[2];
  DevBuf<int> cnt, list, dfe;
  DevBuf<long long> ptr, tmp;
  DevBuf<double> dxyz, dfa, dfb;
  GB_TRY(cnt.alloc(ncell + 1));
  GB_TRY(ptr.alloc(ncell + 1));
  GB_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * (ncell + 1), st));
  if(ne > 0) {
    if(dim == 2)
      k_bucket<3, 0><<<grid_for(ne, 256), 256, 0, st>>>(ne, I.p_nodes, I.p_elems, G, cnt.p,
                                                        nullptr, nullptr);
    else
      k_bucket<4, 0><<<grid_for(ne, 256), 256, 0, st>>>(ne, I.p_nodes, I.p_elems, G, cnt.p,
                                                        nullptr, nullptr);
  }
  long long total = 0;
  GB_TRY(exclusive_scan(cnt.p, ncell + 1, ptr.p, &total, tmp, st));
  GB_TRY(list.alloc(total > 0 ? total : 1));
  GB_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * (ncell + 1), st));
  if(ne > 0) {
    if(dim == 2)
      k_bucket<3, 1><<<grid_for(ne, 256), 256, 0, st>>>(ne, I.p_nodes, I.p_elems, G, cnt.p,
                                                        ptr.p, list.p);
    else
      k_bucket<4, 1><<<grid_for(ne, 256), 256, 0, st>>>(ne, I.p_nodes, I.p_elems, G, cnt.p,
                                                        ptr.p, list.p);
  }
  const int na = dim == 2 ? nh : 3, nb = dim == 2 ? 2 * nh : 3;
  GB_TRY(dxyz.alloc((size_t)np * 3));
  GB_TRY(dfa.alloc((size_t)np * na));
  GB_TRY(dfb.alloc((size_t)np * nb));
  GB_TRY(dfe.alloc(np));
  GB_CUDA(cudaMemcpyAsync(dxyz.p, xyz, sizeof(double) * np * 3, cudaMemcpyHostToDevice, st));
  if(t->kind == GB300_TERM_TRI3_MAGNETOSTATIC)
    k_post_points_tri3<1><<<grid_for(np, 128), 128, 0, st>>>(
      np, dxyz.p, G, ptr.p, list.p, I.p_nodes, I.p_elems, I.p_edofs, x->d.p, dfa.p, dfb.p,
      dfe.p, I.p_fixed);
  else if(t->kind == GB300_TERM_TRI3_EDDY_COMPLEX)
    k_post_points_tri3<2><<<grid_for(np, 128), 128, 0, st>>>(
      np, dxyz.p, G, ptr.p, list.p, I.p_nodes, I.p_elems, I.p_edofs, x->d.p, dfa.p, dfb.p,
      dfe.p, I.p_fixed);
  else
    k_post_points_tet4_edge<<<grid_for(np, 128), 128, 0, st>>>(
      np, dxyz.p, G, ptr.p, list.p, I.p_nodes, I.p_elems, I.p_edofs, I.p_esign, x->d.p,
      dfa.p, dfb.p, dfe.p);
  GB_CUDA(cudaGetLastError());
  if(field)
    GB_CUDA(cudaMemcpyAsync(field, dfa.p, sizeof(double) * np * na, cudaMemcpyDeviceToHost,
                            st));
  if(curl)
    GB_CUDA(cudaMemcpyAsync(curl, dfb.p, sizeof(double) * np * nb, cudaMemcpyDeviceToHost,
                            st));
  if(elem)
    GB_CUDA(cudaMemcpyAsync(elem, dfe.p, sizeof(int) * np, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  return GB300_OK;
}

}  // namespace gb
