// Batched GMRES / FGMRES over independent systems (a frequency or material
// sweep, many small meshes of uneven size).
//
// The systems are the diagonal blocks of one matrix: block p owns rows
// [off[p], off[p+1]) and no entry leaves its block.  One launch of each
// Krylov kernel serves every system: the rows are cut into chunks of at
// most kBChunk rows of one system, a CTA takes a chunk at a time, and every
// dot product is formed per chunk and summed per system, in chunk order,
// by a warp or thread of that system in the control kernels.  Each system
// keeps its own Krylov state (Hessenberg matrix, Givens rotations,
// residual, counters, flags), so its iterations are those of the
// single-system solver of gmres.cu (iters.f:1912-2219 for GMRES,
// :2522-2806 for FGMRES, with classical Gram-Schmidt and the selective
// second pass of gmres.cu): it converges, stops
// at its own iteration cap or breaks down on its own; the chunks of a
// system that has stopped are skipped.  All systems run their restart
// cycles in step (a cycle ends early only for a system that has
// converged), so one CUDA graph holds a whole cycle for all of them.  The
// SpMV and the ILU(0) sweeps run on the whole matrix: block-diagonal, they
// are every system's own.
#include "krylov.cuh"

namespace gb {

// rows per chunk: per-chunk work (the system's flags, h into shared memory,
// the block reductions) is amortised over the rows, while enough chunks
// remain to balance the CTAs; measured on 512 systems of 1,922..50,562 rows:
// 512 rows 290, 2048 319, 4096 309, 8192 267 solves/s
constexpr int kBChunk = 2048;
constexpr int kBThreads = 256;
constexpr int kBMaxKrylov = 128;

struct BState {
  double rtol, tol, res, res0, res6, scale;
  double nrm0;  // ||w||^2 before this step's Gram-Schmidt pass
  int its, maxit, status, active, cycle, first, k, did_cycle, breakdown;
  int reorth;   // this step takes the second Gram-Schmidt pass
};

// per-system Krylov arrays, m = restart length
struct BView {
  BState *S;
  double *H;   // nsys x (m+1) x m, column-major per system
  double *cs, *sn, *y, *h1, *h2;  // nsys x m
  double *g;   // nsys x (m+1)
  int m;
  __device__ double *Hcol(int p, int j) const
  {
    return H + ((size_t)p * m + j) * (m + 1);
  }
};

// chunk c: rows [r0[c], r1[c]) of system sys[c]; system p owns chunks
// [cb[p], cb[p+1])
struct Chunks {
  int n;
  const int *sys, *r0, *r1, *cb;
};

// flags[0]: some system is in a cycle; [1]: some system is active;
// [2]: some system has a solution update due
__global__ void k_b_flags(int nsys, BView V, int *flags)
{
  int a = 0, b = 0, c = 0;
  for(int p = threadIdx.x; p < nsys; p += blockDim.x) {
    const BState &s = V.S[p];
    a |= s.cycle;
    b |= s.active;
    c |= (s.active && s.did_cycle);
  }
  a = __syncthreads_or(a);
  b = __syncthreads_or(b);
  c = __syncthreads_or(c);
  if(threadIdx.x == 0) {
    flags[0] = a;
    flags[1] = b;
    flags[2] = c;
  }
}

// r = b - A x over the chunks of active systems, partial ||r||^2 per chunk;
// FINAL: every system, and the partial ||b||^2 in part2
template <int TPR, int FINAL>
__global__ void __launch_bounds__(kBThreads)
k_b_residual(Chunks C, const int *__restrict__ rowptr, const int *__restrict__ col,
             const double *__restrict__ val, const double *__restrict__ x,
             const double *__restrict__ rhs, double *__restrict__ r,
             double *__restrict__ part, double *__restrict__ part2, BView V)
{
  const int lane = threadIdx.x % TPR, sub = threadIdx.x / TPR;
  for(int c = blockIdx.x; c < C.n; c += gridDim.x) {
    if(!FINAL && !V.S[C.sys[c]].active) continue;  // uniform per CTA
    double rr = 0., bb = 0.;
    for(int i = C.r0[c] + sub; i - sub < C.r1[c]; i += kBThreads / TPR) {
      double s = 0.;
      if(i < C.r1[c])
        for(int k = rowptr[i] + lane; k < rowptr[i + 1]; k += TPR) s += val[k] * x[col[k]];
#pragma unroll
      for(int o = TPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, TPR);
      if(lane == 0 && i < C.r1[c]) {
        double ri = rhs[i] - s;
        r[i] = ri;
        rr += ri * ri;
        bb += rhs[i] * rhs[i];
      }
    }
    double t = block_sum<double, kBThreads>(rr);
    if(threadIdx.x == 0) part[c] = t;
    if(FINAL) {
      t = block_sum<double, kBThreads>(bb);
      if(threadIdx.x == 0) part2[c] = t;
    }
  }
}

// w = A z over the chunks of systems in a cycle
template <int TPR>
__global__ void __launch_bounds__(kBThreads)
k_b_spmv(Chunks C, const int *__restrict__ rowptr, const int *__restrict__ col,
         const double *__restrict__ val, const double *__restrict__ z,
         double *__restrict__ w, BView V)
{
  const int lane = threadIdx.x % TPR, sub = threadIdx.x / TPR;
  for(int c = blockIdx.x; c < C.n; c += gridDim.x) {
    if(!V.S[C.sys[c]].cycle) continue;
    for(int i = C.r0[c] + sub; i - sub < C.r1[c]; i += kBThreads / TPR) {
      double s = 0.;
      if(i < C.r1[c])
        for(int k = rowptr[i] + lane; k < rowptr[i + 1]; k += TPR) s += val[k] * z[col[k]];
#pragma unroll
      for(int o = TPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, TPR);
      if(lane == 0 && i < C.r1[c]) w[i] = s;
    }
  }
}

// restart: ||r|| per system, v1 = r / ||r|| follows in k_b_scale
__global__ void k_b_restart(int nsys, BView V, const int *__restrict__ cb,
                            const double *__restrict__ part)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if(p >= nsys) return;
  BState &S = V.S[p];
  if(!S.active) return;
  double rr = 0.;
  for(int c = cb[p]; c < cb[p + 1]; c++) rr += part[c];
  S.its += 1;
  double alpha = sqrt(rr);
  if(S.first) {
    S.tol = S.rtol * alpha + 0.0;
    S.res0 = alpha;
    S.first = 0;
  }
  S.res = alpha;
  V.g[(size_t)p * (V.m + 1)] = alpha;
  S.k = 0;
  S.did_cycle = 0;
  S.breakdown = 0;
  if(alpha <= S.tol) {  // the restart test of gmres.cu (iters.f)
    S.status = 0;
    S.res6 = alpha;
    S.active = 0;
    S.cycle = 0;
    return;
  }
  S.scale = 1. / alpha;
  S.cycle = 1;
}

// y = scale * x (G = 1: systems in a cycle; with K >= 0 only those whose
// last step was step K)
__global__ void k_b_scale(Chunks C, BView V, const double *x, double *y, int K)
{
  for(int c = blockIdx.x; c < C.n; c += gridDim.x) {
    const BState &S = V.S[C.sys[c]];
    if(!S.cycle || (K >= 0 && S.k != K)) continue;
    double s = S.scale;
    for(int i = C.r0[c] + threadIdx.x; i < C.r1[c]; i += blockDim.x) y[i] = s * x[i];
  }
}

// partial dots <V_j, w>, j < k, per chunk: part[j * nchunks + c]; PASS 0
// also <w, w> (column k: V_k is w), PASS 1 only for systems whose step
// takes the second pass
template <int PASS>
__global__ void __launch_bounds__(kBThreads)
k_b_dots(Chunks C, int k, const double *__restrict__ Vb, size_t ldv,
         const double *__restrict__ w, double *__restrict__ part, BView V)
{
  const int kk = PASS == 0 ? k + 1 : k;
  const int j0 = blockIdx.y * 8;  // this CTA's group of (at most) 8 columns
  if(j0 >= kk) return;
  const int cnt = kk - j0 < 8 ? kk - j0 : 8;
  for(int c = blockIdx.x; c < C.n; c += gridDim.x) {
    const BState &s = V.S[C.sys[c]];
    if(!s.cycle || (PASS == 1 && !s.reorth)) continue;
    double acc[8];
#pragma unroll
    for(int u = 0; u < 8; u++) acc[u] = 0.;
    for(int i = C.r0[c] + threadIdx.x; i < C.r1[c]; i += blockDim.x) {
      double wi = w[i];
#pragma unroll
      for(int u = 0; u < 8; u++)
        if(u < cnt) acc[u] += Vb[(size_t)(j0 + u) * ldv + i] * wi;
    }
    double t = block_sum8<kBThreads>(acc);
    if((int)threadIdx.x < cnt) part[(size_t)(j0 + threadIdx.x) * C.n + c] = t;
  }
}

// h_j per system (one warp per system, lanes over j, chunks in order)
__global__ void k_b_reduce(int nsys, int k, Chunks C, const double *__restrict__ part,
                           BView V, int pass)
{
  int p = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if(p >= nsys || !V.S[p].cycle || (pass == 1 && !V.S[p].reorth)) return;
  const int kk = pass == 0 ? k + 1 : k;
  for(int j = lane; j < kk; j += 32) {
    double v = 0.;
    for(int c = C.cb[p]; c < C.cb[p + 1]; c++) v += part[(size_t)j * C.n + c];
    size_t o = (size_t)p * V.m + j;
    if(j == k)
      V.S[p].nrm0 = v;
    else if(pass == 0) {
      V.h1[o] = v;
      V.Hcol(p, k - 1)[j] = v;
    }
    else {
      V.h2[o] = v;
      V.Hcol(p, k - 1)[j] = V.h1[o] + v;
    }
  }
}

// w -= sum_j h_j V_j (h of pass `pass`); with NORM the partial ||w||^2
template <int NORM>
__global__ void __launch_bounds__(kBThreads)
k_b_update(Chunks C, int k, const double *__restrict__ Vb, size_t ldv,
           double *__restrict__ w, double *__restrict__ part, BView V, int pass)
{
  __shared__ double h[kBMaxKrylov];
  for(int c = blockIdx.x; c < C.n; c += gridDim.x) {
    int p = C.sys[c];
    if(!V.S[p].cycle || (pass == 1 && !V.S[p].reorth)) continue;
    const double *hs = (pass == 0 ? V.h1 : V.h2) + (size_t)p * V.m;
    __syncthreads();  // the previous chunk is done with h
    for(int j = threadIdx.x; j < k; j += blockDim.x) h[j] = hs[j];
    __syncthreads();
    double v = 0.;
    for(int i = C.r0[c] + threadIdx.x; i < C.r1[c]; i += blockDim.x) {
      // four independent FMA chains (see gmres.cu, k_gm_update)
      double s0 = 0., s1 = 0., s2 = 0., s3 = 0.;
      int j = 0;
      for(; j + 3 < k; j += 4) {
        s0 += h[j] * Vb[(size_t)j * ldv + i];
        s1 += h[j + 1] * Vb[(size_t)(j + 1) * ldv + i];
        s2 += h[j + 2] * Vb[(size_t)(j + 2) * ldv + i];
        s3 += h[j + 3] * Vb[(size_t)(j + 3) * ldv + i];
      }
      for(; j < k; j++) s0 += h[j] * Vb[(size_t)j * ldv + i];
      double wi = w[i] - ((s0 + s1) + (s2 + s3));
      w[i] = wi;
      v += wi * wi;
    }
    if(NORM) {
      double s = block_sum<double, kBThreads>(v);
      if(threadIdx.x == 0) part[c] = s;
    }
  }
}

// the selective re-orthogonalisation test of gmres.cu per system: a second
// pass when the first removed more than 98 % of ||w||^2
__global__ void k_b_reorth_test(int nsys, Chunks C, const double *__restrict__ pn,
                                BView V)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if(p >= nsys) return;
  BState &S = V.S[p];
  if(!S.cycle) return;
  if(!(S.nrm0 > 0. && 1. / S.nrm0 > 0.)) {
    // mgsro's zero (-1) or abnormal (-2) norm: the cycle ends as a
    // break-down, the step's column unused (gmres.cu, k_gm_dots)
    S.breakdown = (S.nrm0 <= 0.) ? -1 : -2;
    S.its += 1;
    S.cycle = 0;
    S.reorth = 0;
    return;
  }
  double rr = 0.;
  for(int c = C.cb[p]; c < C.cb[p + 1]; c++) rr += pn[c];
  S.reorth = !(rr >= 0.02 * S.nrm0);
}

// end of an Arnoldi step per system: h(k+1,k), rotations, stopping test
__global__ void k_b_step(int nsys, int k, Chunks C, const double *__restrict__ part,
                         BView V)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if(p >= nsys) return;
  BState &S = V.S[p];
  if(!S.cycle) return;
  double rr = 0.;
  for(int c = C.cb[p]; c < C.cb[p + 1]; c++) rr += part[c];
  S.its += 1;
  const int m = V.m;
  double *Hc = V.Hcol(p, k - 1);
  double *cs = V.cs + (size_t)p * m, *sn = V.sn + (size_t)p * m;
  double *g = V.g + (size_t)p * (m + 1);
  double nrm = sqrt(rr);
  Hc[k] = nrm;
  S.k = k;
  S.did_cycle = 1;
  if(!(nrm > 0.)) {
    S.breakdown = -3;
    S.cycle = 0;
    return;
  }
  for(int i = 0; i < k - 1; i++) {
    double a = Hc[i], c = cs[i], s = sn[i];
    Hc[i] = c * a + s * Hc[i + 1];
    Hc[i + 1] = c * Hc[i + 1] - s * a;
  }
  double c, s;
  givens_dev(&Hc[k - 1], &Hc[k], &c, &s);
  cs[k - 1] = c;
  sn[k - 1] = s;
  double alpha = -s * g[k - 1];
  g[k - 1] = c * g[k - 1];
  g[k] = alpha;
  alpha = fabs(alpha);
  S.res = alpha;
  S.scale = 1. / nrm;
  if(!(k < m && !(alpha <= S.tol) && (S.maxit <= 0 || S.its < S.maxit))) S.cycle = 0;
}

// end of a cycle: H y = g per system (upper triangular)
__global__ void k_b_solve_small(int nsys, BView V)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if(p >= nsys) return;
  BState &S = V.S[p];
  if(!S.active || !S.did_cycle) return;
  int k = S.k;
  const int m = V.m;
  while(k > 0 && V.Hcol(p, k - 1)[k - 1] == 0.) k--;
  if(k == 0) {
    S.status = -3;
    S.breakdown = -4;
    S.active = 0;
    S.did_cycle = 0;
    return;
  }
  S.k = k;
  double *y = V.y + (size_t)p * m;
  const double *g = V.g + (size_t)p * (m + 1);
  for(int i = k - 1; i >= 0; i--) {
    double t = g[i];
    for(int j = i + 1; j < k; j++) t -= V.Hcol(p, j)[i] * y[j];
    y[i] = t / V.Hcol(p, i)[i];
  }
}

// u = sum_j y_j V_j (ADD = 0) or x += sum_j y_j Z_j (ADD = 1)
template <int ADD>
__global__ void __launch_bounds__(kBThreads)
k_b_combine(Chunks C, const double *__restrict__ Vb, size_t ldv,
            double *__restrict__ out, BView V)
{
  __shared__ double y[kBMaxKrylov];
  for(int c = blockIdx.x; c < C.n; c += gridDim.x) {
    int p = C.sys[c];
    const BState &S = V.S[p];
    if(!S.active || !S.did_cycle) continue;
    int k = S.k;
    __syncthreads();
    for(int j = threadIdx.x; j < k; j += blockDim.x) y[j] = V.y[(size_t)p * V.m + j];
    __syncthreads();
    for(int i = C.r0[c] + threadIdx.x; i < C.r1[c]; i += blockDim.x) {
      double s = ADD ? out[i] : 0.;
      for(int j = 0; j < k; j++) s += y[j] * Vb[(size_t)j * ldv + i];
      out[i] = s;
    }
  }
}

__global__ void k_b_addto(Chunks C, const double *__restrict__ u,
                          double *__restrict__ x, BView V)
{
  for(int c = blockIdx.x; c < C.n; c += gridDim.x) {
    const BState &S = V.S[C.sys[c]];
    if(!S.active || !S.did_cycle) continue;
    for(int i = C.r0[c] + threadIdx.x; i < C.r1[c]; i += blockDim.x) x[i] += u[i];
  }
}

// after the update: the restart decision per system
__global__ void k_b_after(int nsys, BView V)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if(p >= nsys) return;
  BState &S = V.S[p];
  if(!S.active) return;
  S.res6 = S.res;
  if(S.breakdown != 0) {
    S.status = -3;
    S.active = 0;
    return;
  }
  bool more = (S.its < S.maxit || S.maxit <= 0) && (S.res6 > S.tol);
  if(!more) {
    if(S.res6 <= S.tol)
      S.status = 0;
    else if(S.its >= S.maxit && S.maxit > 0)
      S.status = -1;
    else
      S.status = -10;
    S.active = 0;
  }
}

// rows of the systems whose preconditioner is due: in a cycle (WHICH 0),
// or with a solution update due (WHICH 1)
__global__ void k_b_rowmask(Chunks C, BView V, int which, unsigned char *__restrict__ mask)
{
  for(int c = blockIdx.x; c < C.n; c += gridDim.x) {
    const BState &S = V.S[C.sys[c]];
    unsigned char on = which == 0 ? (S.cycle != 0) : (S.active && S.did_cycle);
    for(int i = C.r0[c] + threadIdx.x; i < C.r1[c]; i += blockDim.x) mask[i] = on;
  }
}

__global__ void k_b_copy(int n, const double *__restrict__ v, double *__restrict__ z,
                         const int *flag)
{
  if(flag && !*flag) return;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (long long)gridDim.x * blockDim.x)
    z[i] = v[i];
}

// every entry of a row lies in the row's block
__global__ void k_b_check_blocks(int n, const int *__restrict__ rowptr,
                                 const int *__restrict__ col,
                                 const int *__restrict__ row_lo,
                                 const int *__restrict__ row_hi, int *__restrict__ bad)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n) return;
  int lo = row_lo[i], hi = row_hi[i];
  for(int k = rowptr[i]; k < rowptr[i + 1]; k++)
    if(col[k] < lo || col[k] >= hi) {
      atomicExch(bad, 1);
      return;
    }
}

__global__ void k_b_row_range(int nsys, const int *__restrict__ off,
                              int *__restrict__ lo, int *__restrict__ hi)
{
  int p = blockIdx.x;
  if(p >= nsys) return;
  for(int i = off[p] + threadIdx.x; i < off[p + 1]; i += blockDim.x) {
    lo[i] = off[p];
    hi[i] = off[p + 1];
  }
}

int gmres_solve_batch(gb300_matrix *A, const double *val, const double *rhs,
                      double *x, const gb300_solver_params *p, int nsys,
                      const int *off, gb300_solve_info *infos, Work &W)
{
  cudaStream_t st = A->ctx->stream;
  const int n = A->n;
  const bool flexible = (p->algorithm == 9);
  if(p->algorithm != 8 && p->algorithm != 9) {
    set_error("batched solve: Algorithm %d is not supported (8 GMRES, 9 FGMRES)",
              p->algorithm);
    return GB300_ERR_UNSUPPORTED;
  }
  if(p->preconditioner != 0 && p->preconditioner != 6) {
    set_error("batched solve: Preconditioner %d is not supported (0, 6)",
              p->preconditioner);
    return GB300_ERR_UNSUPPORTED;
  }
  const int m = p->krylov_size <= 1 ? 15 : p->krylov_size;
  if(m > kBMaxKrylov) {
    set_error("Krylov_Size %d exceeds this backend's maximum %d", m, kBMaxKrylov);
    return GB300_ERR_UNSUPPORTED;
  }
  // chunks
  std::vector<int> hs, h0, h1, hcb(nsys + 1);
  for(int q = 0; q < nsys; q++) {
    hcb[q] = (int)hs.size();
    for(int r = off[q]; r < off[q + 1]; r += kBChunk) {
      hs.push_back(q);
      h0.push_back(r);
      h1.push_back(r + kBChunk < off[q + 1] ? r + kBChunk : off[q + 1]);
    }
  }
  hcb[nsys] = (int)hs.size();
  const int nch = (int)hs.size();
  DevBuf<int> dsys, dr0, dr1, dcb, flags;
  GB_TRY(dsys.alloc(nch > 0 ? nch : 1));
  GB_TRY(dr0.alloc(nch > 0 ? nch : 1));
  GB_TRY(dr1.alloc(nch > 0 ? nch : 1));
  GB_TRY(dcb.alloc(nsys + 1));
  GB_TRY(flags.alloc(4));
  if(nch > 0) {
    GB_CUDA(cudaMemcpyAsync(dsys.p, hs.data(), sizeof(int) * nch, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(dr0.p, h0.data(), sizeof(int) * nch, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(dr1.p, h1.data(), sizeof(int) * nch, cudaMemcpyHostToDevice, st));
  }
  GB_CUDA(cudaMemcpyAsync(dcb.p, hcb.data(), sizeof(int) * (nsys + 1),
                          cudaMemcpyHostToDevice, st));
  Chunks C{nch, dsys.p, dr0.p, dr1.p, dcb.p};

  // per-system state and arrays
  DevBuf<BState> S;
  DevBuf<double> arr;
  GB_TRY(S.alloc(nsys));
  size_t nH = (size_t)nsys * (m + 1) * m, nm = (size_t)nsys * m;
  GB_TRY(arr.alloc(nH + 5 * nm + (size_t)nsys * (m + 1)));
  BView V;
  V.S = S.p;
  V.H = arr.p;
  V.cs = V.H + nH;
  V.sn = V.cs + nm;
  V.y = V.sn + nm;
  V.h1 = V.y + nm;
  V.h2 = V.h1 + nm;
  V.g = V.h2 + nm;
  V.m = m;
  {
    std::vector<BState> h(nsys);
    for(auto &s : h) {
      memset(&s, 0, sizeof(s));
      s.active = 1;
      s.first = 1;
      s.maxit = p->nb_iter_max;
      s.rtol = p->stopping_test;
      s.status = 1;
    }
    GB_CUDA(cudaMemcpyAsync(S.p, h.data(), sizeof(BState) * nsys, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemsetAsync(arr.p, 0, sizeof(double) * arr.n, st));
  }

  bool precond = (p->preconditioner == 6);
  bool fp32 = (p->precision != 0);
  if(precond) {
    int zr = 0;
    GB_TRY(ilu_factor(A, val, fp32, &zr));
    if(zr) {
      set_error("Zero pivot on line %d in ILU", zr);
      return GB300_ERR_ZERO_PIVOT;
    }
  }
  size_t ldv = (size_t)n;
  double *Vb = (double *)W.vec(0, sizeof(double) * ldv * (m + 1));
  double *Z = flexible ? (double *)W.vec(1, sizeof(double) * ldv * m) : nullptr;
  double *r = (double *)W.vec(2, sizeof(double) * n);
  double *u = (double *)W.vec(3, sizeof(double) * n);
  double *zt = (double *)W.vec(4, sizeof(double) * n);
  float *t32 = fp32 ? (float *)W.vec(5, sizeof(float) * n) : nullptr;
  double *part = (double *)W.vec(6, sizeof(double) * (size_t)(nch > 0 ? nch : 1) * (m + 1));
  double *part2 = (double *)W.vec(7, sizeof(double) * (nch > 0 ? nch : 1));
  double *pn = (double *)W.vec(12, sizeof(double) * (nch > 0 ? nch : 1));
  if(!Vb || (flexible && !Z) || !r || !u || !zt || (fp32 && !t32) || !part || !part2 ||
     !pn)
    return GB300_ERR_CUDA;
  GB_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, st));

  const int gchunks = grid_for(nch, 1, kReduceBlocks);
  const int gsys = grid_for(nsys, 128);
  const int gwarp = grid_for(nsys, 8);  // 8 warps per 256-thread block
  DevBuf<unsigned char> rmask;
  GB_TRY(rmask.alloc(n > 0 ? n : 1));
  // the sweeps visit only the rows of systems still iterating
  auto precond_apply = [&](const double *v, double *z, const int *flag, int which) {
    if(precond) {
      k_b_rowmask<<<gchunks, kBThreads, 0, st>>>(C, V, which, rmask.p);
      ilu_apply(A, ilu_mode(p), v, z, t32, flag, st, rmask.p);
    }
    else
      k_b_copy<<<grid_for(n, 256, kReduceBlocks * 4), 256, 0, st>>>(n, v, z, flag);
  };

  cudaGraph_t graph;
  cudaGraphExec_t exec;
  GB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  k_b_residual<2, 0><<<gchunks, kBThreads, 0, st>>>(C, A->rowptr.p, A->col.p, val, x,
                                                    rhs, r, part, nullptr, V);
  k_b_restart<<<gsys, 128, 0, st>>>(nsys, V, dcb.p, part);
  k_b_flags<<<1, 256, 0, st>>>(nsys, V, flags.p);
  k_b_scale<<<gchunks, kBThreads, 0, st>>>(C, V, r, Vb, -1);
  for(int k = 1; k <= m; k++) {
    double *vk = Vb + (size_t)(k - 1) * ldv;
    double *w = Vb + (size_t)k * ldv;
    double *z = flexible ? Z + (size_t)(k - 1) * ldv : zt;
    precond_apply(vk, z, flags.p, 0);
    k_b_spmv<2><<<gchunks, kBThreads, 0, st>>>(C, A->rowptr.p, A->col.p, val, z, w, V);
    k_b_dots<0><<<dim3(gchunks, (k + 1 + 7) / 8), kBThreads, 0, st>>>(C, k, Vb, ldv, w,
                                                                      part, V);
    k_b_reduce<<<gwarp, 256, 0, st>>>(nsys, k, C, part, V, 0);
    k_b_update<1><<<gchunks, kBThreads, 0, st>>>(C, k, Vb, ldv, w, pn, V, 0);
    k_b_reorth_test<<<gsys, 128, 0, st>>>(nsys, C, pn, V);
    k_b_dots<1><<<dim3(gchunks, (k + 7) / 8), kBThreads, 0, st>>>(C, k, Vb, ldv, w, part,
                                                                  V);
    k_b_reduce<<<gwarp, 256, 0, st>>>(nsys, k, C, part, V, 1);
    k_b_update<1><<<gchunks, kBThreads, 0, st>>>(C, k, Vb, ldv, w, pn, V, 1);
    k_b_step<<<gsys, 128, 0, st>>>(nsys, k, C, pn, V);
    k_b_flags<<<1, 256, 0, st>>>(nsys, V, flags.p);
    k_b_scale<<<gchunks, kBThreads, 0, st>>>(C, V, w, w, k);
  }
  k_b_solve_small<<<gsys, 128, 0, st>>>(nsys, V);
  k_b_flags<<<1, 256, 0, st>>>(nsys, V, flags.p);
  if(flexible)
    k_b_combine<1><<<gchunks, kBThreads, 0, st>>>(C, Z, ldv, x, V);
  else {
    k_b_combine<0><<<gchunks, kBThreads, 0, st>>>(C, Vb, ldv, u, V);
    precond_apply(u, zt, flags.p + 2, 1);
    k_b_addto<<<gchunks, kBThreads, 0, st>>>(C, zt, x, V);
  }
  k_b_after<<<gsys, 128, 0, st>>>(nsys, V);
  k_b_flags<<<1, 256, 0, st>>>(nsys, V, flags.p);
  GB_CUDA(cudaStreamEndCapture(st, &graph));
  GB_CUDA(cudaGraphInstantiate(&exec, graph, 0));

  int hf[4] = {0, 1, 0, 0};
  int launches = 0;
  const int max_launches = p->nb_iter_max > 0 ? p->nb_iter_max + 2 : 1 << 30;
  int rc = GB300_OK;
  while(hf[1] && launches < max_launches) {
    if(cudaGraphLaunch(exec, st) != cudaSuccess) {
      rc = GB300_ERR_CUDA;
      break;
    }
    launches++;
    if(cudaMemcpyAsync(hf, flags.p, sizeof(int) * 4, cudaMemcpyDeviceToHost, st) !=
         cudaSuccess ||
       cudaStreamSynchronize(st) != cudaSuccess) {
      rc = GB300_ERR_CUDA;
      break;
    }
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  if(rc != GB300_OK) {
    set_error("batched solve: graph launch failed");
    return rc;
  }

  // per-system results and true residuals
  k_b_residual<2, 1><<<gchunks, kBThreads, 0, st>>>(C, A->rowptr.p, A->col.p, val, x,
                                                    rhs, r, part, part2, V);
  GB_CUDA(cudaGetLastError());
  std::vector<BState> hsys(nsys);
  std::vector<double> hp(nch), hb(nch);
  GB_CUDA(cudaMemcpyAsync(hsys.data(), S.p, sizeof(BState) * nsys, cudaMemcpyDeviceToHost, st));
  if(nch > 0) {
    GB_CUDA(cudaMemcpyAsync(hp.data(), part, sizeof(double) * nch, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaMemcpyAsync(hb.data(), part2, sizeof(double) * nch, cudaMemcpyDeviceToHost, st));
  }
  GB_CUDA(cudaStreamSynchronize(st));
  for(int q = 0; q < nsys; q++) {
    gb300_solve_info &f = infos[q];
    memset(&f, 0, sizeof(f));
    const BState &s = hsys[q];
    f.status = s.active ? -1 : s.status;
    f.iterations = s.its;
    f.residual_estimate = s.res6;
    double rr = 0., bb = 0.;
    for(int c = hcb[q]; c < hcb[q + 1]; c++) {
      rr += hp[c];
      bb += hb[c];
    }
    f.true_residual = sqrt(rr);
    f.rhs_norm = sqrt(bb);
  }
  return GB300_OK;
}

// checks that every row's entries lie in its block
int check_blocks(const gb300_matrix *A, int nsys, const int *off)
{
  cudaStream_t st = A->ctx->stream;
  const int n = A->n;
  DevBuf<int> doff, lo, hi, bad;
  GB_TRY(doff.alloc(nsys + 1));
  GB_TRY(lo.alloc(n > 0 ? n : 1));
  GB_TRY(hi.alloc(n > 0 ? n : 1));
  GB_TRY(bad.alloc(1));
  GB_CUDA(cudaMemcpyAsync(doff.p, off, sizeof(int) * (nsys + 1), cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  if(n > 0) {
    k_b_row_range<<<nsys, 256, 0, st>>>(nsys, doff.p, lo.p, hi.p);
    k_b_check_blocks<<<grid_for(n, 256), 256, 0, st>>>(n, A->rowptr.p, A->col.p, lo.p,
                                                       hi.p, bad.p);
  }
  int hb = 0;
  GB_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  GB_CUDA(cudaGetLastError());
  return hb ? GB300_ERR_ARG : GB300_OK;
}

}  // namespace gb
