// Learned correction of the ILU(0) preconditioner: a small message-passing
// network over the matrix graph predicts the values of a sparse matrix G on
// A's pattern, and the preconditioner becomes z = ILU^-1 v, z += G (v - A z)
// (Preconditioner 20 of the solver).
//
// Network (3 message-passing layers, hidden width 32, weights stored in
// BF16 and used as BF16-rounded values, FP32 accumulation):
//   node features f_i = (1, sum_{j != i} |e_ij|, max_{j != i} |e_ij|, deg_i / 8)
//   with e_ij = a_ij / sqrt(a_ii a_jj) (scale-free);
//   h0_i = relu(W_in f_i + b_in);
//   m_i = sum_{j != i} e_ij h_j,  h_i <- relu(W_s h_i + W_n m_i + b)  (x 3);
//   g_ij = sum_c w_o,c h_i,c h_j,c + c_o e_ij (i != j),
//   g_ii = sum_c w_d,c h_i,c + b_d;  G_ij = g_ij / sqrt(a_ii a_jj).
// Training (hand-written backward pass, Adam): for a system with right-hand
// side b and the plain solver's solution x*, z1 = ILU^-1 b, r1 = b - A z1,
// e1 = x* - z1 = A^-1 r1, and the loss is the energy norm of the error left
// after the correction, relative to the ILU(0) step's:
//   loss = (G r1 - e1)^T A (G r1 - e1) / e1^T A e1
//        = 1 + (y^T A y - 2 r1^T y) / S,  y = G r1,  S = e1^T A e1
// (A symmetric positive definite, as the magnetostatic systems and their
// Newton Jacobians are).  The second form needs no solution, so random
// probes v (z1 = ILU^-1 v, r1 = v - A z1) train G too, with S = r1^T D^-1 r1
// in place of the unknown e1^T A e1 (D = diag A).  A Euclidean fit of e1
// let the correction add oscillatory components that A amplifies; the
// energy norm weighs them as the Krylov iteration does.
//
// Kernels: the forward layers on the tensor cores over 16-node tiles
// (k_mp_layer_mma); one warp per node (lane = channel) for the input, the
// output head and the backward pass; weight gradients accumulate per warp in
// registers and are added with FP32 atomics (their order varies, so
// gradients agree with the FP64 CPU check to FP32 rounding, not bit for
// bit).
#include <cuda_bf16.h>

#include <random>

#include "krylov.cuh"

namespace gb {

constexpr int kH = 32;     // hidden width
constexpr int kFin = 4;    // node input features
constexpr int kLayers = 3;
// flat parameter layout
constexpr int kOffWin = 0;
constexpr int kOffBin = kOffWin + kH * kFin;
constexpr int kOffLayer = kOffBin + kH;
constexpr int kLayerSize = 2 * kH * kH + kH;  // W_s, W_n, b
constexpr int kOffWo = kOffLayer + kLayers * kLayerSize;
constexpr int kOffCo = kOffWo + kH;
constexpr int kOffWd = kOffCo + 1;
constexpr int kOffBd = kOffWd + kH;
constexpr int kParams = kOffBd + 1;
constexpr int kNodeWarps = 8;  // nodes per 256-thread CTA

__device__ __forceinline__ float bf16_round(float x)
{
  return __bfloat162float(__float2bfloat16_rn(x));
}

// per system: graph features and activations
struct MpnnGraph {
  int n = 0;
  long long nnz = 0;
  unsigned version = ~0u;
  DevBuf<float> ehat, feat, dscale;  // e_ij (nnz), f_i (n x 4), 1/sqrt(a_ii)
  DevBuf<int> diag, tpos;            // position of a_ii, of (j,i) for entry (i,j)
  DevBuf<float> h, m;                // (L+1) x n x H, L x n x H
  DevBuf<float> dh, dm;              // n x H work for the backward pass
  DevBuf<double> G;                  // nnz correction values
};

}  // namespace gb

struct gb300_mpnn {
  gb300_ctx *ctx = nullptr;
  gb::DevBuf<float> w;       // FP32 master weights
  gb::DevBuf<float> wq;      // BF16-rounded copy used by the kernels
  gb::DevBuf<float> grad, am, av;  // gradient, Adam moments
  int step = 0;
  int loss_mode = 0;  // 0: one-level energy loss; 1: after the coarse correction
  gb::MpnnGraph g;
};

namespace gb {

__global__ void k_round_bf16(int n, const float *__restrict__ w, float *__restrict__ q)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) q[i] = bf16_round(w[i]);
}

// e_ij, node features, 1/sqrt(a_ii), diagonal and transpose positions
__global__ void k_mp_features(int n, const int *__restrict__ rowptr,
                              const int *__restrict__ col, const double *__restrict__ val,
                              float *__restrict__ ehat, float *__restrict__ feat,
                              float *__restrict__ dscale, int *__restrict__ diag,
                              int *__restrict__ tpos, int *__restrict__ bad)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n) return;
  int s = rowptr[i], e = rowptr[i + 1];
  int di = find_col(col, s, e, i);
  if(di < 0 || !(val[di] > 0.)) {
    atomicExch(bad, 1);
    return;
  }
  diag[i] = di;
  dscale[i] = (float)(1. / sqrt(val[di]));
}

__global__ void k_mp_edges(int n, const int *__restrict__ rowptr,
                           const int *__restrict__ col, const double *__restrict__ val,
                           const int *__restrict__ diag, float *__restrict__ ehat,
                           float *__restrict__ feat, int *__restrict__ tpos,
                           int *__restrict__ bad)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n) return;
  int s = rowptr[i], e = rowptr[i + 1];
  double aii = val[diag[i]];
  float sum = 0.f, mx = 0.f;
  for(int k = s; k < e; k++) {
    int j = col[k];
    double ajj = val[diag[j]];
    float v = (float)(val[k] / sqrt(aii * ajj));
    ehat[k] = v;
    int t = find_col(col, rowptr[j], rowptr[j + 1], i);
    if(t < 0) atomicExch(bad, 1);
    tpos[k] = t;
    if(j != i) {
      sum += fabsf(v);
      mx = fmaxf(mx, fabsf(v));
    }
  }
  feat[4 * i] = 1.f;
  feat[4 * i + 1] = sum;
  feat[4 * i + 2] = mx;
  feat[4 * i + 3] = (float)(e - s) / 8.f;
}

// h0 = relu(W_in f + b_in), one warp per node, lane = channel
__global__ void __launch_bounds__(32 * kNodeWarps)
k_mp_input(int n, const float *__restrict__ feat, const float *__restrict__ wq,
           float *__restrict__ h0)
{
  int lane = threadIdx.x & 31;
  for(int i = blockIdx.x * kNodeWarps + (threadIdx.x >> 5); i < n;
      i += gridDim.x * kNodeWarps) {
    float z = wq[kOffBin + lane];
#pragma unroll
    for(int f = 0; f < kFin; f++) z += wq[kOffWin + lane * kFin + f] * feat[4 * i + f];
    h0[(size_t)i * kH + lane] = fmaxf(z, 0.f);
  }
}

// One message-passing layer, m_i = sum_{j != i} e_ij h_j,
// h'_i = relu(W_s h_i + W_n m_i + b), with its dense part on the tensor
// cores (mma.sync m16n8k16, BF16 in, FP32 accumulation).  A warp-per-node
// form on the CUDA cores (lane = channel) was bound by its load/store pipe:
// every lane broadcast its channel by shuffle and read a row of the two
// 32 x 32 weight matrices from shared memory, 64 of each per node and layer
// for 64 FMAs (649 us per layer at 1024^2 against 241 us here).  Here a
// warp takes 16 nodes at a time: it sums
// their messages as above (lane = channel) into a 16 x 64 shared tile
// [h | m], then multiplies the tile by [W_s | W_n]^T held in registers as
// BF16 MMA operands (the weights are BF16-rounded already: exact).  The
// activations are FP32; each is split into three BF16 parts
// (x = hi + mid + lo, each the BF16 rounding of what is left), so the three
// MMAs per k-slice carry 24 bits of every activation and the layer matches
// the FP32 form to FP32 rounding.
__device__ __forceinline__ unsigned bf16x2(float a, float b)
{
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);  // a in the low half
  return *reinterpret_cast<unsigned *>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const unsigned (&a)[4], unsigned b0,
                                         unsigned b1)
{
  asm volatile(
    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
    "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
    : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
    : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int kMmaWarps = 8;  // 16-node tiles per 256-thread CTA at a time

__global__ void __launch_bounds__(32 * kMmaWarps)
k_mp_layer_mma(int n, const int *__restrict__ rowptr, const int *__restrict__ col,
               const float *__restrict__ ehat, const float *__restrict__ wl,
               const float *__restrict__ hin, float *__restrict__ mout,
               float *__restrict__ hout)
{
  __shared__ float X[kMmaWarps][16][2 * kH + 1];  // per warp: [h | m] of 16 nodes
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, tig = lane & 3;
  // B operands: B[k][o] = W[o][k], W = [W_s | W_n] (32 x 64); k-slice kt,
  // output tile nt: rows k = 16 kt + 2 tig + {0,1} (b0) and + 8 (b1), o = 8 nt + g
  unsigned B0[4][4], B1[4][4];
#pragma unroll
  for(int kt = 0; kt < 4; kt++)
#pragma unroll
    for(int nt = 0; nt < 4; nt++) {
      const int o = 8 * nt + g, k0 = 16 * kt + 2 * tig;
      auto w = [&](int k) {
        return k < kH ? wl[o * kH + k] : wl[kH * kH + o * kH + (k - kH)];
      };
      B0[kt][nt] = bf16x2(w(k0), w(k0 + 1));
      B1[kt][nt] = bf16x2(w(k0 + 8), w(k0 + 9));
    }
  float bias[4][2];
#pragma unroll
  for(int nt = 0; nt < 4; nt++) {
    bias[nt][0] = wl[2 * kH * kH + 8 * nt + 2 * tig];
    bias[nt][1] = wl[2 * kH * kH + 8 * nt + 2 * tig + 1];
  }
  const int ntiles = (n + 15) / 16;
  for(int t = blockIdx.x * kMmaWarps + warp; t < ntiles; t += gridDim.x * kMmaWarps) {
    // messages of the tile's 16 nodes: lane = (node r, half hf of the
    // channels), each neighbour's 16 channels gathered as four float4, so a
    // warp walks its 16 rows side by side (each channel summed in the row's
    // order)
    {
      const int r = lane >> 1, hf = lane & 1;
      const int i = 16 * t + r;
      float4 mi[4], hv[4];
#pragma unroll
      for(int q = 0; q < 4; q++) mi[q] = hv[q] = make_float4(0.f, 0.f, 0.f, 0.f);
      if(i < n) {
        for(int k = rowptr[i]; k < rowptr[i + 1]; k++) {
          const int j = col[k];
          if(j == i) continue;
          const float e = ehat[k];
          const float4 *hj = reinterpret_cast<const float4 *>(hin + (size_t)j * kH + 16 * hf);
#pragma unroll
          for(int q = 0; q < 4; q++) {
            const float4 v = __ldg(hj + q);
            mi[q].x += e * v.x;
            mi[q].y += e * v.y;
            mi[q].z += e * v.z;
            mi[q].w += e * v.w;
          }
        }
        const float4 *hs = reinterpret_cast<const float4 *>(hin + (size_t)i * kH + 16 * hf);
        float4 *mo = reinterpret_cast<float4 *>(mout + (size_t)i * kH + 16 * hf);
#pragma unroll
        for(int q = 0; q < 4; q++) {
          hv[q] = __ldg(hs + q);
          mo[q] = mi[q];
        }
      }
#pragma unroll
      for(int q = 0; q < 4; q++) {
        const int c = 16 * hf + 4 * q;
        X[warp][r][c] = hv[q].x;
        X[warp][r][c + 1] = hv[q].y;
        X[warp][r][c + 2] = hv[q].z;
        X[warp][r][c + 3] = hv[q].w;
        X[warp][r][kH + c] = mi[q].x;
        X[warp][r][kH + c + 1] = mi[q].y;
        X[warp][r][kH + c + 2] = mi[q].z;
        X[warp][r][kH + c + 3] = mi[q].w;
      }
    }
    __syncwarp();
    float C[4][4];
#pragma unroll
    for(int nt = 0; nt < 4; nt++) C[nt][0] = C[nt][1] = C[nt][2] = C[nt][3] = 0.f;
#pragma unroll
    for(int kt = 0; kt < 4; kt++) {
      // this thread's 8 activations of the 16 x 16 slice kt
      float x[8];
      const int c0 = 16 * kt + 2 * tig;
      x[0] = X[warp][g][c0];
      x[1] = X[warp][g][c0 + 1];
      x[2] = X[warp][g + 8][c0];
      x[3] = X[warp][g + 8][c0 + 1];
      x[4] = X[warp][g][c0 + 8];
      x[5] = X[warp][g][c0 + 9];
      x[6] = X[warp][g + 8][c0 + 8];
      x[7] = X[warp][g + 8][c0 + 9];
#pragma unroll
      for(int part = 0; part < 3; part++) {
        float y[8];
#pragma unroll
        for(int q = 0; q < 8; q++) {
          y[q] = __bfloat162float(__float2bfloat16_rn(x[q]));
          x[q] -= y[q];  // what the next part carries
        }
        const unsigned a[4] = {bf16x2(y[0], y[1]), bf16x2(y[2], y[3]), bf16x2(y[4], y[5]),
                               bf16x2(y[6], y[7])};
#pragma unroll
        for(int nt = 0; nt < 4; nt++) mma_bf16(C[nt], a, B0[kt][nt], B1[kt][nt]);
      }
    }
    __syncwarp();
    // C[nt]: rows g (c0, c1) and g + 8 (c2, c3), outputs 8 nt + 2 tig + {0,1}
    const int i0 = 16 * t + g, i1 = i0 + 8;
#pragma unroll
    for(int nt = 0; nt < 4; nt++) {
      const int o = 8 * nt + 2 * tig;
      if(i0 < n) {
        hout[(size_t)i0 * kH + o] = fmaxf(C[nt][0] + bias[nt][0], 0.f);
        hout[(size_t)i0 * kH + o + 1] = fmaxf(C[nt][1] + bias[nt][1], 0.f);
      }
      if(i1 < n) {
        hout[(size_t)i1 * kH + o] = fmaxf(C[nt][2] + bias[nt][0], 0.f);
        hout[(size_t)i1 * kH + o + 1] = fmaxf(C[nt][3] + bias[nt][1], 0.f);
      }
    }
  }
}

// output head: G on A's pattern
__global__ void __launch_bounds__(32 * kNodeWarps)
k_mp_output(int n, const int *__restrict__ rowptr, const int *__restrict__ col,
            const float *__restrict__ ehat, const float *__restrict__ dscale,
            const float *__restrict__ wq, const float *__restrict__ h,
            double *__restrict__ G)
{
  int lane = threadIdx.x & 31;
  const float wo = wq[kOffWo + lane], wd = wq[kOffWd + lane];
  const float co = wq[kOffCo], bd = wq[kOffBd];
  for(int i = blockIdx.x * kNodeWarps + (threadIdx.x >> 5); i < n;
      i += gridDim.x * kNodeWarps) {
    float hi = h[(size_t)i * kH + lane];
    for(int k = rowptr[i]; k < rowptr[i + 1]; k++) {
      int j = col[k];
      float t = (j != i) ? wo * hi * h[(size_t)j * kH + lane] : wd * hi;
      t = warp_sum(t);
      if(lane == 0) {
        float gk = (j != i) ? t + co * ehat[k] : t + bd;
        G[k] = (double)(gk * dscale[i] * dscale[j]);
      }
    }
  }
}

// y = G r1, and the partial sums of r1^T y
__global__ void k_mp_gr(int n, const int *__restrict__ rowptr, const int *__restrict__ col,
                        const double *__restrict__ G, const double *__restrict__ r1,
                        double *__restrict__ y, double *__restrict__ part)
{
  double acc = 0.;
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double s = 0.;
    for(int k = rowptr[i]; k < rowptr[i + 1]; k++) s += G[k] * r1[col[k]];
    y[i] = s;
    acc += r1[i] * s;
  }
  double t = block_sum<double, 256>(acc);
  if(threadIdx.x == 0) part[blockIdx.x] = t;
}

// partial sums of r1^T D^-1 r1 (D = diag A; dscale = D^-1/2)
__global__ void k_mp_dnorm(int n, const double *__restrict__ r1,
                           const float *__restrict__ dscale, double *__restrict__ part)
{
  double acc = 0.;
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v = r1[i] * (double)dscale[i];
    acc += v * v;
  }
  double t = block_sum<double, 256>(acc);
  if(threadIdx.x == 0) part[blockIdx.x] = t;
}

// w = A y - r1
__global__ void k_mp_sub(int n, const double *__restrict__ r1, double *__restrict__ w)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) w[i] -= r1[i];
}

// gradient of the loss with respect to g_k (before the 1/sqrt(a_ii a_jj)
// scaling), per entry: 2 w_i r1_j / S, w = A G r1 - r1
__global__ void k_mp_dg(int n, const int *__restrict__ rowptr, const int *__restrict__ col,
                        const float *__restrict__ dscale, const double *__restrict__ y,
                        const double *__restrict__ r1, double inv_e2,
                        float *__restrict__ dg)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n) return;
  for(int k = rowptr[i]; k < rowptr[i + 1]; k++) {
    int j = col[k];
    dg[k] = (float)(2. * y[i] * r1[j] * inv_e2) * dscale[i] * dscale[j];
  }
}

// backward of the output head: weight gradients and dh of the last layer
__global__ void __launch_bounds__(32 * kNodeWarps)
k_mp_output_bwd(int n, const int *__restrict__ rowptr, const int *__restrict__ col,
                const float *__restrict__ ehat, const int *__restrict__ tpos,
                const float *__restrict__ wq, const float *__restrict__ h,
                const float *__restrict__ dg, float *__restrict__ dh,
                float *__restrict__ grad)
{
  int lane = threadIdx.x & 31;
  const float wo = wq[kOffWo + lane], wd = wq[kOffWd + lane];
  float gwo = 0.f, gwd = 0.f, gco = 0.f, gbd = 0.f;
  for(int i = blockIdx.x * kNodeWarps + (threadIdx.x >> 5); i < n;
      i += gridDim.x * kNodeWarps) {
    float hi = h[(size_t)i * kH + lane];
    float dhi = 0.f;
    for(int k = rowptr[i]; k < rowptr[i + 1]; k++) {
      int j = col[k];
      float d = dg[k];
      if(j != i) {
        float hj = h[(size_t)j * kH + lane];
        gwo += d * hi * hj;
        if(lane == 0) gco += d * ehat[k];
        // g_ij and g_ji both depend on h_i
        dhi += (d + dg[tpos[k]]) * wo * hj;
      }
      else {
        gwd += d * hi;
        if(lane == 0) gbd += d;
        dhi += d * wd;
      }
    }
    dh[(size_t)i * kH + lane] = dhi;
  }
  atomicAdd(&grad[kOffWo + lane], gwo);
  atomicAdd(&grad[kOffWd + lane], gwd);
  if(lane == 0) {
    atomicAdd(&grad[kOffCo], gco);
    atomicAdd(&grad[kOffBd], gbd);
  }
}

// backward of a layer, pass 1: dz = dh_out (h_out > 0); weight gradients;
// dm_i = W_n^T dz_i; dh_in_i (own part) = W_s^T dz_i (written to dhin)
__global__ void __launch_bounds__(32 * kNodeWarps)
k_mp_layer_bwd1(int n, const float *__restrict__ wl, const float *__restrict__ hin,
                const float *__restrict__ m, const float *__restrict__ hout,
                const float *__restrict__ dhout, float *__restrict__ dm,
                float *__restrict__ dhin, float *__restrict__ gl)
{
  __shared__ float Ws[kH][kH + 1], Wn[kH][kH + 1];
  __shared__ float acc[kLayerSize];  // the CTA's weight gradients
  for(int t = threadIdx.x; t < kH * kH; t += blockDim.x) {
    Ws[t / kH][t % kH] = wl[t];
    Wn[t / kH][t % kH] = wl[kH * kH + t];
  }
  for(int t = threadIdx.x; t < kLayerSize; t += blockDim.x) acc[t] = 0.f;
  __syncthreads();
  int lane = threadIdx.x & 31;
  float gws[kH], gwn[kH], gb = 0.f;
#pragma unroll
  for(int d = 0; d < kH; d++) gws[d] = gwn[d] = 0.f;
  for(int i = blockIdx.x * kNodeWarps + (threadIdx.x >> 5); i < n;
      i += gridDim.x * kNodeWarps) {
    size_t o = (size_t)i * kH + lane;
    float dz = hout[o] > 0.f ? dhout[o] : 0.f;
    float hi = hin[o], mi = m[o];
    gb += dz;
    float dmi = 0.f, dsi = 0.f;
#pragma unroll
    for(int d = 0; d < kH; d++) {
      // lane = output channel c: dW[c][d] += dz_c x_d
      gws[d] += dz * __shfl_sync(0xffffffffu, hi, d);
      gwn[d] += dz * __shfl_sync(0xffffffffu, mi, d);
      // lane = input channel: sum over c of W[c][lane] dz_c
      float dzc = __shfl_sync(0xffffffffu, dz, d);
      dmi += Wn[d][lane] * dzc;
      dsi += Ws[d][lane] * dzc;
    }
    dm[o] = dmi;
    dhin[o] = dsi;
  }
#pragma unroll
  for(int d = 0; d < kH; d++) {
    atomicAdd(&acc[lane * kH + d], gws[d]);
    atomicAdd(&acc[kH * kH + lane * kH + d], gwn[d]);
  }
  atomicAdd(&acc[2 * kH * kH + lane], gb);
  __syncthreads();
  for(int t = threadIdx.x; t < kLayerSize; t += blockDim.x) atomicAdd(&gl[t], acc[t]);
}

// pass 2: dh_in_i += sum_{j != i} e_ji dm_j  (e symmetric in the pattern:
// the entry of row i towards j carries e_ij = e_ji)
__global__ void __launch_bounds__(32 * kNodeWarps)
k_mp_layer_bwd2(int n, const int *__restrict__ rowptr, const int *__restrict__ col,
                const float *__restrict__ ehat, const int *__restrict__ tpos,
                const float *__restrict__ dm, float *__restrict__ dhin)
{
  int lane = threadIdx.x & 31;
  for(int i = blockIdx.x * kNodeWarps + (threadIdx.x >> 5); i < n;
      i += gridDim.x * kNodeWarps) {
    float acc = 0.f;
    for(int k = rowptr[i]; k < rowptr[i + 1]; k++) {
      int j = col[k];
      if(j != i) acc += ehat[tpos[k]] * dm[(size_t)j * kH + lane];
    }
    dhin[(size_t)i * kH + lane] += acc;
  }
}

__global__ void __launch_bounds__(32 * kNodeWarps)
k_mp_input_bwd(int n, const float *__restrict__ feat, const float *__restrict__ h0,
               const float *__restrict__ dh0, float *__restrict__ grad)
{
  int lane = threadIdx.x & 31;
  float gw[kFin] = {0.f, 0.f, 0.f, 0.f}, gb = 0.f;
  for(int i = blockIdx.x * kNodeWarps + (threadIdx.x >> 5); i < n;
      i += gridDim.x * kNodeWarps) {
    size_t o = (size_t)i * kH + lane;
    float dz = h0[o] > 0.f ? dh0[o] : 0.f;
    gb += dz;
#pragma unroll
    for(int f = 0; f < kFin; f++) gw[f] += dz * feat[4 * i + f];
  }
#pragma unroll
  for(int f = 0; f < kFin; f++) atomicAdd(&grad[kOffWin + lane * kFin + f], gw[f]);
  atomicAdd(&grad[kOffBin + lane], gb);
}

__global__ void k_adam(int np, float *__restrict__ w, const float *__restrict__ g,
                       float *__restrict__ m, float *__restrict__ v, float lr,
                       float b1t, float b2t)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= np) return;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  float gi = g[i];
  m[i] = b1 * m[i] + (1.f - b1) * gi;
  v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
  float mh = m[i] / (1.f - b1t), vh = v[i] / (1.f - b2t);
  w[i] -= lr * mh / (sqrtf(vh) + eps);
}

static int mp_prepare(gb300_mpnn *net, const gb300_matrix *A)
{
  MpnnGraph &g = net->g;
  cudaStream_t st = A->ctx->stream;
  const int n = A->n;
  if(!A->csr_valid || n == 0) {
    set_error("network: matrix not assembled");
    return GB300_ERR_ARG;
  }
  GB_TRY(g.ehat.alloc(A->nnz));
  GB_TRY(g.feat.alloc((size_t)n * 4));
  GB_TRY(g.dscale.alloc(n));
  GB_TRY(g.diag.alloc(n));
  GB_TRY(g.tpos.alloc(A->nnz));
  GB_TRY(g.h.alloc((size_t)(kLayers + 1) * n * kH));
  GB_TRY(g.m.alloc((size_t)kLayers * n * kH));
  GB_TRY(g.dh.alloc((size_t)2 * n * kH));
  GB_TRY(g.dm.alloc((size_t)n * kH));
  GB_TRY(g.G.alloc(A->nnz));
  DevBuf<int> bad;
  GB_TRY(bad.alloc(1));
  GB_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  k_mp_features<<<grid_for(n, 256), 256, 0, st>>>(n, A->rowptr.p, A->col.p, A->val.p,
                                                   g.ehat.p, g.feat.p, g.dscale.p,
                                                   g.diag.p, g.tpos.p, bad.p);
  k_mp_edges<<<grid_for(n, 256), 256, 0, st>>>(n, A->rowptr.p, A->col.p, A->val.p,
                                                g.diag.p, g.ehat.p, g.feat.p, g.tpos.p,
                                                bad.p);
  int hb = 0;
  GB_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(hb) {
    set_error("network: the matrix needs a positive diagonal and a symmetric pattern");
    return GB300_ERR_UNSUPPORTED;
  }
  g.n = n;
  g.nnz = A->nnz;
  return GB300_OK;
}

static int mp_forward(gb300_mpnn *net, const gb300_matrix *A)
{
  MpnnGraph &g = net->g;
  cudaStream_t st = A->ctx->stream;
  const int n = A->n;
  k_round_bf16<<<grid_for(kParams, 256), 256, 0, st>>>(kParams, net->w.p, net->wq.p);
  int grid = grid_for(n, kNodeWarps, kReduceBlocks);
  k_mp_input<<<grid, 32 * kNodeWarps, 0, st>>>(n, g.feat.p, net->wq.p, g.h.p);
  const int gm = grid_for((n + 15) / 16, kMmaWarps, kReduceBlocks);
  for(int l = 0; l < kLayers; l++)
    k_mp_layer_mma<<<gm, 32 * kMmaWarps, 0, st>>>(
      n, A->rowptr.p, A->col.p, g.ehat.p, net->wq.p + kOffLayer + l * kLayerSize,
      g.h.p + (size_t)l * n * kH, g.m.p + (size_t)l * n * kH,
      g.h.p + (size_t)(l + 1) * n * kH);
  k_mp_output<<<grid, 32 * kNodeWarps, 0, st>>>(n, A->rowptr.p, A->col.p, g.ehat.p,
                                                 g.dscale.p, net->wq.p,
                                                 g.h.p + (size_t)kLayers * n * kH, g.G.p);
  GB_CUDA(cudaGetLastError());
  return GB300_OK;
}

static int mp_loss_backward(gb300_mpnn *net, gb300_matrix *A, const double *r1,
                            const double *e1, double *loss)
{
  MpnnGraph &g = net->g;
  cudaStream_t st = A->ctx->stream;
  const int n = A->n;
  const bool two = (net->loss_mode == 1);
  DevBuf<double> y, w, part, ee, t, q;
  DevBuf<float> dg;
  GB_TRY(y.alloc(n));
  GB_TRY(w.alloc(n));
  GB_TRY(part.alloc(kReduceBlocks));
  GB_TRY(dg.alloc(A->nnz));
  GB_TRY(ee.alloc(4));
  if(two) {
    GB_TRY(t.alloc(n));
    GB_TRY(q.alloc(n));
  }
  // S = e1^T A e1 (solution known), else r1^T D^-1 r1
  if(e1) {
    spmv_plain(A, A->val.p, e1, w.p, st);
    dot_part64(n, e1, w.p, part.p, st);
  }
  else
    k_mp_dnorm<<<kReduceBlocks, 256, 0, st>>>(n, r1, g.dscale.p, part.p);
  sum_partials(part.p, ee.p, st);
  // y = G r1, r1^T y; w = A y, y^T A y; w <- w - r1
  k_mp_gr<<<kReduceBlocks, 256, 0, st>>>(n, A->rowptr.p, A->col.p, g.G.p, r1, y.p, part.p);
  sum_partials(part.p, ee.p + 1, st);
  spmv_plain(A, A->val.p, y.p, w.p, st);
  dot_part64(n, y.p, w.p, part.p, st);
  sum_partials(part.p, ee.p + 2, st);
  k_mp_sub<<<grid_for(n, 256), 256, 0, st>>>(n, r1, w.p);
  // two-level loss: the error left after the coarse correction,
  // (e1 - y)^T (A - A C A) (e1 - y), whose gradient in y is 2 (I - A C) w
  // with w = A y - r1; w^T C w is what the coarse correction removes
  GB_CUDA(cudaMemsetAsync(ee.p + 3, 0, sizeof(double), st));
  if(two) GB_TRY(coarse_energy_project(A, w.p, t.p, q.p, ee.p + 3, st));
  double he[4] = {0., 0., 0., 0.};
  GB_CUDA(cudaMemcpyAsync(he, ee.p, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  const double S = he[0];
  if(!(S > 0.)) {
    set_error("network: zero or indefinite normalisation (zero probe, or A not "
              "positive definite)");
    return GB300_ERR_ARG;
  }
  const double hl = S + he[2] - 2. * he[1] - he[3];  // (relative) energy error x S
  const double E = S;
  // dL/dG_ij = 2 (A y - r1)_i r1_j / S
  k_mp_dg<<<grid_for(n, 256), 256, 0, st>>>(n, A->rowptr.p, A->col.p, g.dscale.p, w.p, r1,
                                            1. / S, dg.p);
  int grid = grid_for(n, kNodeWarps, kReduceBlocks);
  float *dhA = g.dh.p, *dhB = g.dh.p + (size_t)n * kH;
  k_mp_output_bwd<<<grid, 32 * kNodeWarps, 0, st>>>(
    n, A->rowptr.p, A->col.p, g.ehat.p, g.tpos.p, net->wq.p,
    g.h.p + (size_t)kLayers * n * kH, dg.p, dhA, net->grad.p);
  // few CTAs for the weight-gradient pass: each CTA adds its sums once
  const int gw = grid_for(n, kNodeWarps, 2 * 152);
  for(int l = kLayers - 1; l >= 0; l--) {
    const float *wl = net->wq.p + kOffLayer + l * kLayerSize;
    k_mp_layer_bwd1<<<gw, 32 * kNodeWarps, 0, st>>>(
      n, wl, g.h.p + (size_t)l * n * kH, g.m.p + (size_t)l * n * kH,
      g.h.p + (size_t)(l + 1) * n * kH, dhA, g.dm.p, dhB,
      net->grad.p + kOffLayer + l * kLayerSize);
    k_mp_layer_bwd2<<<grid, 32 * kNodeWarps, 0, st>>>(n, A->rowptr.p, A->col.p, g.ehat.p,
                                                       g.tpos.p, g.dm.p, dhB);
    std::swap(dhA, dhB);
  }
  k_mp_input_bwd<<<grid, 32 * kNodeWarps, 0, st>>>(n, g.feat.p, g.h.p, dhA, net->grad.p);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(st));
  *loss = hl / E;
  return GB300_OK;
}

}  // namespace gb

using namespace gb;

extern "C" {

int gb300_mpnn_param_count(void) { return kParams; }

int gb300_mpnn_create(gb300_ctx *ctx, unsigned seed, gb300_mpnn **out)
{
  if(!ctx || !out) {
    set_error("network: null argument");
    return GB300_ERR_ARG;
  }
  gb300_mpnn *net = new gb300_mpnn();
  net->ctx = ctx;
  int rc = GB300_OK;
  if((rc = net->w.alloc(kParams)) || (rc = net->wq.alloc(kParams)) ||
     (rc = net->grad.alloc(kParams)) || (rc = net->am.alloc(kParams)) ||
     (rc = net->av.alloc(kParams))) {
    delete net;
    return rc;
  }
  // Glorot-uniform weights, zero biases; the output head starts at zero
  // (G = 0: the plain ILU(0) preconditioner)
  std::vector<float> h(kParams, 0.f);
  std::mt19937 gen(seed);
  auto fill = [&](int off, int fan_in, int fan_out, int count) {
    float a = std::sqrt(6.f / (float)(fan_in + fan_out));
    std::uniform_real_distribution<float> u(-a, a);
    for(int t = 0; t < count; t++) h[off + t] = u(gen);
  };
  fill(kOffWin, kFin, kH, kH * kFin);
  for(int l = 0; l < kLayers; l++) {
    fill(kOffLayer + l * kLayerSize, kH, kH, kH * kH);
    fill(kOffLayer + l * kLayerSize + kH * kH, kH, kH, kH * kH);
  }
  cudaStream_t st = ctx->stream;
  if(cudaMemcpyAsync(net->w.p, h.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice,
                     st) != cudaSuccess ||
     cudaMemsetAsync(net->am.p, 0, sizeof(float) * kParams, st) != cudaSuccess ||
     cudaMemsetAsync(net->av.p, 0, sizeof(float) * kParams, st) != cudaSuccess ||
     cudaMemsetAsync(net->grad.p, 0, sizeof(float) * kParams, st) != cudaSuccess ||
     cudaStreamSynchronize(st) != cudaSuccess) {
    delete net;
    set_error("network: device initialisation failed");
    return GB300_ERR_CUDA;
  }
  *out = net;
  return GB300_OK;
}

int gb300_mpnn_destroy(gb300_mpnn *net)
{
  if(net) {
    cudaStreamSynchronize(net->ctx->stream);
    delete net;
  }
  return GB300_OK;
}

int gb300_mpnn_set_params(gb300_mpnn *net, const float *host)
{
  if(!net || !host) {
    set_error("network: null argument");
    return GB300_ERR_ARG;
  }
  GB_CUDA(cudaMemcpyAsync(net->w.p, host, sizeof(float) * kParams, cudaMemcpyHostToDevice,
                          net->ctx->stream));
  GB_CUDA(cudaStreamSynchronize(net->ctx->stream));
  return GB300_OK;
}

int gb300_mpnn_get_params(const gb300_mpnn *net, float *host)
{
  if(!net || !host) {
    set_error("network: null argument");
    return GB300_ERR_ARG;
  }
  GB_CUDA(cudaMemcpyAsync(host, net->w.p, sizeof(float) * kParams, cudaMemcpyDeviceToHost,
                          net->ctx->stream));
  GB_CUDA(cudaStreamSynchronize(net->ctx->stream));
  return GB300_OK;
}

int gb300_mpnn_infer(gb300_mpnn *net, gb300_matrix *A)
{
  gb::NvtxRange nvtx_range("gb300_mpnn_infer");
  if(!net || !A) {
    set_error("network: null argument");
    return GB300_ERR_ARG;
  }
  GB_TRY(gb300_matrix_assemble(A));
  GB_TRY(mp_prepare(net, A));
  GB_TRY(mp_forward(net, A));
  GB_TRY(A->corr.alloc(A->nnz));
  GB_CUDA(cudaMemcpyAsync(A->corr.p, net->g.G.p, sizeof(double) * A->nnz,
                          cudaMemcpyDeviceToDevice, A->ctx->stream));
  GB_CUDA(cudaStreamSynchronize(A->ctx->stream));
  A->corr_version = A->pattern_version;
  return GB300_OK;
}

int gb300_mpnn_loss_grad(gb300_mpnn *net, gb300_matrix *A, const gb300_vector *r1,
                         const gb300_vector *e1, int accumulate, double *loss,
                         float *grad_host)
{
  gb::NvtxRange nvtx_range("gb300_mpnn_loss_grad");
  if(!net || !A || !r1 || !loss) {
    set_error("network: null argument");
    return GB300_ERR_ARG;
  }
  GB_TRY(gb300_matrix_assemble(A));
  if(r1->n != A->n || (e1 && e1->n != A->n)) {
    set_error("network: vector sizes do not match the matrix");
    return GB300_ERR_ARG;
  }
  cudaStream_t st = A->ctx->stream;
  if(!accumulate) GB_CUDA(cudaMemsetAsync(net->grad.p, 0, sizeof(float) * kParams, st));
  if(net->loss_mode == 1 && !coarse_valid(A)) {
    set_error("network: the two-level loss needs aggregates on the matrix "
              "(gb300_matrix_set_aggregates)");
    return GB300_ERR_ARG;
  }
  GB_TRY(mp_prepare(net, A));
  GB_TRY(mp_forward(net, A));
  GB_TRY(mp_loss_backward(net, A, r1->d.p, e1 ? e1->d.p : nullptr, loss));
  if(grad_host) {
    GB_CUDA(cudaMemcpyAsync(grad_host, net->grad.p, sizeof(float) * kParams,
                            cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
  }
  return GB300_OK;
}

int gb300_mpnn_set_loss(gb300_mpnn *net, int mode)
{
  if(!net || (mode != 0 && mode != 1)) {
    set_error("network: loss mode must be 0 (one-level) or 1 (two-level)");
    return GB300_ERR_ARG;
  }
  net->loss_mode = mode;
  return GB300_OK;
}

int gb300_mpnn_adam_step(gb300_mpnn *net, float lr, float grad_scale)
{
  gb::NvtxRange nvtx_range("gb300_mpnn_adam_step");
  if(!net) {
    set_error("network: null argument");
    return GB300_ERR_ARG;
  }
  cudaStream_t st = net->ctx->stream;
  net->step++;
  float b1t = std::pow(0.9f, (float)net->step), b2t = std::pow(0.999f, (float)net->step);
  if(grad_scale != 1.f) {
    // gradients summed over a mini-batch: average them
    std::vector<float> h(kParams);
    GB_CUDA(cudaMemcpyAsync(h.data(), net->grad.p, sizeof(float) * kParams,
                            cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    for(float &v : h) v *= grad_scale;
    GB_CUDA(cudaMemcpyAsync(net->grad.p, h.data(), sizeof(float) * kParams,
                            cudaMemcpyHostToDevice, st));
  }
  k_adam<<<grid_for(kParams, 256), 256, 0, st>>>(kParams, net->w.p, net->grad.p,
                                                 net->am.p, net->av.p, lr, b1t, b2t);
  GB_CUDA(cudaMemsetAsync(net->grad.p, 0, sizeof(float) * kParams, st));
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(st));
  return GB300_OK;
}

}  // extern "C"
