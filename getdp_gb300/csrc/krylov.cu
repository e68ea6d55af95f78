// Solve[A] on the GPU: the work of solve_matrix
// (contrib/Sparskit/Sparskit.cpp:108-634) with the Krylov methods of
// contrib/Sparskit/iters.f.
//
// Every scalar of a Krylov iteration (dot products, step lengths, the
// stopping test of stopbis, iters.f:3275-3331) lives in device memory and is
// computed on the device (one-block control kernels, or the last CTA of the
// kernel that produced the partial sums), so iterations run back to back
// without host round trips.  A fixed batch of iterations is captured once
// in a CUDA graph and replayed; kernels after convergence see the device
// flag `active == 0` and return at once.  The host reads one status word
// per graph launch.
//
// Dot products use fixed-size partial-sum grids summed in a fixed order, so
// a solve is bit-reproducible run to run.
#include "krylov.cuh"

namespace gb {

// ---------------------------------------------------------------------------
// scaling (scale_matrix DIAG_SCALING, Sparskit.cpp:978-1001: rowscal =
// colscal = 1/sqrt(|a_ii|), A <- D A D applied as (a*s_i)*s_j, b <- D b,
// x <- D y at the end)
// ---------------------------------------------------------------------------
__global__ void k_diag_scal(int n, const int *__restrict__ rowptr,
                            const int *__restrict__ col,
                            const double *__restrict__ val,
                            double *__restrict__ s, int *__restrict__ zero)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n) return;
  double d = 0.;
  for(int k = rowptr[i]; k < rowptr[i + 1]; k++)
    if(col[k] == i) {
      d = val[k];
      break;
    }
  if(d != 0.)
    s[i] = 1. / sqrt(fabs(d));
  else {
    s[i] = 1.;
    atomicExch(zero, 1);
  }
}

__global__ void k_scale_vals(int n, const int *__restrict__ rowptr,
                             const int *__restrict__ col,
                             const double *__restrict__ val,
                             const double *__restrict__ s,
                             double *__restrict__ out)
{
  int i = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if(i >= n) return;
  double si = s[i];
  for(int k = rowptr[i] + (threadIdx.x & 31); k < rowptr[i + 1]; k += 32)
    out[k] = (val[k] * si) * s[col[k]];
}

__global__ void k_mul(int n, const double *a, const double *s, double *out)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) out[i] = a[i] * s[i];
}

template <typename TO, typename TI>
__global__ void k_convert(long long n, const TI *__restrict__ in,
                          TO *__restrict__ out)
{
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) out[i] = (TO)in[i];
}

// ---------------------------------------------------------------------------
// CG (iters.f:379-564, no preconditioner: Ml = Mr = I)
// ---------------------------------------------------------------------------
struct CgState {
  double rho;    // <r, r> of the previous step (fpar(7))
  double alpha;  // step length
  double beta;
  double tol;    // fpar(4) = rtol * ||r0|| + atol
  double res;    // fpar(5) = fpar(6) = ||r||
  double res0;   // fpar(3)
  int active;
  int status;    // ipar(1) at exit
  int its;       // ipar(7)
  int maxit;     // ipar(6)
  // mixed precision (reliable updates)
  double maxrr;  // largest FP32 ||r||^2 since the last update
  double delta2; // update when ||r32||^2 < delta2 * maxrr
  int update;    // this iteration replaces the residual in FP64
  int convert;   // r32 <- r64 pending
  int final_;    // the iteration cap was reached: last update then stop
  int updates;   // residual replacements done
  // fused control: go = active && !update guards the iteration kernels;
  // pq = <p, Ap> written by the SpMV's last CTA; arrival counters
  int go;
  double pq;
  unsigned tick_dot, tick_step;
};

__global__ void k_cg_start(CgState *S, const double *__restrict__ part_rr,
                           double rtol, int maxit)
{
  double rr = 0.;
  for(int i = threadIdx.x; i < kReduceBlocks; i += blockDim.x) rr += part_rr[i];
  rr = block_sum<double, 256>(rr);
  if(threadIdx.x == 0) {
    S->rho = rr;
    S->res0 = sqrt(rr);
    S->res = S->res0;
    S->tol = rtol * S->res0 + 0.0;
    S->its = 1;  // the initial residual's matrix-vector product
    S->maxit = maxit;
    S->status = 1;
    S->active = 1;
    S->alpha = S->beta = 0.;
    S->update = S->convert = S->final_ = S->updates = 0;
    S->tick_dot = S->tick_step = 0u;
    // no test before the first step, as in iters.f's cg: a zero or
    // abnormal right-hand side stops there at brkdn (-3 / -9), x = 0
    S->go = S->active;
  }
}

// four consecutive entries through one 16-byte (float) or two 16-byte
// (double) accesses; i4 indexes groups of four
__device__ __forceinline__ void ld4(const float *p, long long i4, float (&v)[4])
{
  float4 t = reinterpret_cast<const float4 *>(p)[i4];
  v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w;
}
__device__ __forceinline__ void st4(float *p, long long i4, const float (&v)[4])
{
  reinterpret_cast<float4 *>(p)[i4] = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void ld4(const double *p, long long i4, double (&v)[4])
{
  double2 a = reinterpret_cast<const double2 *>(p)[2 * i4];
  double2 b = reinterpret_cast<const double2 *>(p)[2 * i4 + 1];
  v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
}
__device__ __forceinline__ void st4(double *p, long long i4, const double (&v)[4])
{
  reinterpret_cast<double2 *>(p)[2 * i4] = make_double2(v[0], v[1]);
  reinterpret_cast<double2 *>(p)[2 * i4 + 1] = make_double2(v[2], v[3]);
}

// brkdn (iters.f:3368-3402) on <p, Ap>: 0, or the ipar(1) code
__device__ __forceinline__ int cg_breakdown(double pq)
{
  if(pq > 0.) {
    double b = 1. / pq;
    return (b > 0.) ? 0 : -9;
  }
  if(pq < 0.) {
    double b = 1. / pq;
    return (b < 0.) ? 0 : -9;
  }
  if(pq == 0.) return -3;
  return -9;
}

// the stopping test of the FP64 CG (stopbis: the iteration cap first, then
// the residual test)
__device__ void cg_check_tail(CgState *S, double rr)
{
  if(S->maxit > 0 && S->its >= S->maxit) {
    S->status = -1;
    S->active = 0;
    S->res = sqrt(rr);
    return;
  }
  S->res = sqrt(rr);
  if(!(S->res > S->tol)) {
    S->status = (S->res == S->res) ? 0 : -10;
    S->active = 0;
    return;
  }
  S->beta = S->res * S->res / S->rho;
  S->rho = S->res * S->res;
}

// the reliable-update test of the mixed CG: replace the residual when the
// FP32 one has dropped by delta since the last update, claims convergence,
// or the iteration cap is reached
__device__ void rcg_check_tail(CgState *S, double rr)
{
  S->convert = 0;
  double tol2 = S->tol * S->tol;
  bool cap = (S->maxit > 0 && S->its >= S->maxit);
  if(cap || !(rr > tol2) || rr < S->delta2 * S->maxrr) {
    S->update = 1;
    S->final_ = cap ? 1 : 0;
    S->res = sqrt(rr);
    return;
  }
  S->update = 0;
  if(rr > S->maxrr) S->maxrr = rr;
  S->beta = rr / S->rho;
  S->rho = rr;
  S->res = sqrt(rr);
}

// One CG step after the SpMV: alpha = rho / <p, Ap> (from S->pq), x += alpha
// p, r -= alpha Ap with the partials of ||r||^2; the last CTA then counts
// the iteration, applies brkdn and the stopping (or update) test.
template <typename T, bool MIXED>
__global__ void __launch_bounds__(256)
k_cg_step(int n, CgState *__restrict__ S, T *__restrict__ x, T *__restrict__ r,
          const T *__restrict__ p, const T *__restrict__ q, double *__restrict__ part)
{
  if(!S->go) return;
  // alpha and the breakdown test once per CTA: FP64 divisions in every
  // thread would keep the FP64 pipe busier than the vector traffic
  __shared__ T s_alpha;
  __shared__ int s_bad;
  const double pq = S->pq, rho = S->rho;
  if(threadIdx.x == 0) {
    s_bad = cg_breakdown(pq);
    s_alpha = s_bad ? (T)0 : (T)(rho / pq);
  }
  __syncthreads();
  const int bad = s_bad;
  typename Acc<T>::type v = 0;
  if(!bad) {
    // vectors are cudaMalloc'ed (256-byte aligned): groups of four, then
    // the n % 4 remainder
    const T a = s_alpha;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long n4 = n / 4;
    for(long long i4 = (long long)blockIdx.x * blockDim.x + threadIdx.x; i4 < n4;
        i4 += stride) {
      T xv[4], rv[4], pv[4], qv[4];
      ld4(x, i4, xv);
      ld4(r, i4, rv);
      ld4(p, i4, pv);
      ld4(q, i4, qv);
#pragma unroll
      for(int c = 0; c < 4; c++) {
        xv[c] += a * pv[c];
        rv[c] = rv[c] - a * qv[c];
        v += rv[c] * rv[c];
      }
      st4(x, i4, xv);
      st4(r, i4, rv);
    }
    for(long long i = 4 * n4 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
        i < n; i += stride) {
      x[i] += a * p[i];
      T ri = r[i] - a * q[i];
      r[i] = ri;
      v += ri * ri;
    }
  }
  double s = block_sum<double, 256>((double)v);
  if(threadIdx.x == 0) part[blockIdx.x] = s;
  if(blockIdx.x == 0)
    for(int b = gridDim.x + threadIdx.x; b < kReduceBlocks; b += blockDim.x) part[b] = 0.;
  if(!arrive_last(&S->tick_step)) return;
  double rr = sum_partials_l2<256>(part);
  if(threadIdx.x == 0) {
    S->its += 1;
    if(bad) {
      S->status = bad;
      S->active = 0;
      S->alpha = 0.;
    }
    else {
      S->alpha = rho / pq;
      if(MIXED)
        rcg_check_tail(S, rr);
      else
        cg_check_tail(S, rr);
    }
    S->go = S->active && !S->update;
  }
}

template <typename T>
__global__ void k_cg_p(int n, const CgState *__restrict__ S, T *__restrict__ p,
                       const T *__restrict__ r)
{
  if(!S->go) return;
  T b = (T)S->beta;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long n4 = n / 4;
  for(long long i4 = (long long)blockIdx.x * blockDim.x + threadIdx.x; i4 < n4;
      i4 += stride) {
    T rv[4], pv[4];
    ld4(r, i4, rv);
    ld4(p, i4, pv);
#pragma unroll
    for(int c = 0; c < 4; c++) pv[c] = rv[c] + b * pv[c];
    st4(p, i4, pv);
  }
  for(long long i = 4 * n4 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
      i < n; i += stride)
    p[i] = r[i] + b * p[i];
}

template <typename T>
__global__ void k_copy(long long n, const T *__restrict__ a, T *__restrict__ b)
{
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) b[i] = a[i];
}

// SpMV with the CG dot fused, guarded by the active flag
template <int TPR, typename V, typename XT>
__global__ void __launch_bounds__(256)
k_cg_spmv(int n, const int *__restrict__ rowptr, const int *__restrict__ col,
          const V *__restrict__ val, const XT *__restrict__ p,
          XT *__restrict__ q, double *__restrict__ part, CgState *S)
{
  if(!S->go) return;
  const int rows_per_block = 256 / TPR;
  int lane = threadIdx.x % TPR;
  int sub = threadIdx.x / TPR;
  typename Acc<XT>::type red = 0;
  for(long long rb = (long long)blockIdx.x * rows_per_block; rb < n;
      rb += (long long)gridDim.x * rows_per_block) {
    long long row = rb + sub;
    XT sum = 0;
    if(row < n) {
      int s = rowptr[row], e = rowptr[row + 1];
      sum = csr_row_dot<TPR, (TPR >= 16 ? 4 : 2), XT>(s, e, lane, col, val, p);
    }
#pragma unroll
    for(int o = TPR / 2; o > 0; o >>= 1)
      sum += __shfl_down_sync(0xffffffffu, sum, o, TPR);
    if(lane == 0 && row < n) {
      q[row] = sum;
      red += p[row] * sum;
    }
  }
  double s = block_sum<double, 256>((double)red);
  if(threadIdx.x == 0) part[blockIdx.x] = s;
  if(arrive_last(&S->tick_dot)) {
    double d = sum_partials_l2<256>(part);
    if(threadIdx.x == 0) S->pq = d;
  }
}

template <typename V, typename XT>
static void cg_spmv(const gb300_matrix *A, const V *val, const XT *p, XT *q,
                    double *part, CgState *S, cudaStream_t st)
{
  int n = A->n;
  switch(A->tpr) {
  case 2: k_cg_spmv<2><<<kReduceBlocks, 256, 0, st>>>(n, A->rowptr.p, A->col.p, val, p, q, part, S); break;
  case 4: k_cg_spmv<4><<<kReduceBlocks, 256, 0, st>>>(n, A->rowptr.p, A->col.p, val, p, q, part, S); break;
  case 8: k_cg_spmv<8><<<kReduceBlocks, 256, 0, st>>>(n, A->rowptr.p, A->col.p, val, p, q, part, S); break;
  case 16: k_cg_spmv<16><<<kReduceBlocks, 256, 0, st>>>(n, A->rowptr.p, A->col.p, val, p, q, part, S); break;
  default: k_cg_spmv<32><<<kReduceBlocks, 256, 0, st>>>(n, A->rowptr.p, A->col.p, val, p, q, part, S); break;
  }
}

// Runs CG on the operator applied by spmv_dot(p, q, part, S, stream)
// (q = A p with the partials of <p, q>), y = rhs from y = 0, to
// ||r|| <= rtol ||rhs||.  T is the vector type, n the vector length.
// Returns the final state in *hs.
template <typename T, typename SPMV>
static int cg_core(cudaStream_t st, int n, SPMV spmv_dot, const T *rhs, T *y,
                   double rtol, int maxit, CgState *hs, Work &W)
{
  T *r = (T *)W.vec(0, n * sizeof(T));
  T *p = (T *)W.vec(1, n * sizeof(T));
  T *q = (T *)W.vec(2, n * sizeof(T));
  if(!r || !p || !q) return GB300_ERR_CUDA;
  CgState *S = (CgState *)W.state(sizeof(CgState));
  double *part = W.part();
  if(!S || !part) return GB300_ERR_CUDA;
  int gl = grid_for(n, 256);
  // x0 = 0 (Sparskit.cpp:226); r = rhs - A*0 = rhs, p = r
  GB_CUDA(cudaMemsetAsync(y, 0, n * sizeof(T), st));
  k_copy<T><<<gl, 256, 0, st>>>(n, rhs, r);
  k_copy<T><<<gl, 256, 0, st>>>(n, rhs, p);
  if(sizeof(T) == 8)
    dot_part64(n, (const double *)r, (const double *)r, part, st);
  else
    dot_part32(n, (const float *)r, (const float *)r, part, st);
  k_cg_start<<<1, 256, 0, st>>>(S, part, rtol, maxit);
  GB_CUDA(cudaGetLastError());

  // capture a batch of iterations once
  const int batch = n > 200000 ? 16 : 32;
  const int step_grid = resident_grid(k_cg_step<T, false>, 256, 0);
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  GB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  for(int it = 0; it < batch; it++) {
    spmv_dot(p, q, part, S, st);
    k_cg_step<T, false><<<step_grid, 256, 0, st>>>(n, S, y, r, p, q, part);
    k_cg_p<T><<<grid_for((n + 3) / 4, 256, kReduceBlocks * 4), 256, 0, st>>>(n, S, p, r);
  }
  GB_CUDA(cudaStreamEndCapture(st, &graph));
  GB_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  int active = 1;
  int launches = 0;
  int max_launches = (maxit > 0 ? maxit / batch + 2 : 1 << 30);
  while(active && launches < max_launches) {
    GB_CUDA(cudaGraphLaunch(exec, st));
    launches++;
    GB_CUDA(cudaMemcpyAsync(&active, &S->active, sizeof(int),
                            cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  GB_CUDA(cudaMemcpyAsync(hs, S, sizeof(CgState), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  return GB300_OK;
}

// timed launches of the CG SpMV kernel (used for the roofline figure)
int bench_spmv(gb300_matrix *A, int precision, int reps, double *ms)
{
  cudaStream_t st = A->ctx->stream;
  int n = A->n;
  Work W;
  CgState h;
  memset(&h, 0, sizeof(h));
  h.active = 1;
  h.go = 1;
  CgState *S = (CgState *)W.state(sizeof(CgState));
  double *part = W.part();
  if(!S || !part) return GB300_ERR_CUDA;
  GB_CUDA(cudaMemcpyAsync(S, &h, sizeof(h), cudaMemcpyHostToDevice, st));
  cudaEvent_t e0, e1;
  GB_CUDA(cudaEventCreate(&e0));
  GB_CUDA(cudaEventCreate(&e1));
  float t = 0.f;
  Bsr3 B;
  if(A->block3 &&
     bsr_build(A, A->val.p, precision == 0, precision != 0, B) == GB300_OK &&
     bsr_tune(A, B, st, precision == 0) == GB300_OK) {
    // the kernel the CG runs on a 3-component system: 3x3 blocks
    int n4 = 4 * B.nn;
    if(precision == 0) {
      double *p = (double *)W.vec(0, sizeof(double) * n4);
      double *q = (double *)W.vec(1, sizeof(double) * n4);
      if(!p || !q) return GB300_ERR_CUDA;
      k_copy<double><<<grid_for(n4, 256), 256, 0, st>>>(n4, B.val64.p, p);
      for(int i = 0; i < 3; i++)
        bsr_spmv_dot64(B, p, q, part, &S->go, &S->pq, &S->tick_dot, st);
      GB_CUDA(cudaEventRecord(e0, st));
      for(int i = 0; i < reps; i++)
        bsr_spmv_dot64(B, p, q, part, &S->go, &S->pq, &S->tick_dot, st);
      GB_CUDA(cudaEventRecord(e1, st));
    }
    else {
      float *p = (float *)W.vec(0, sizeof(float) * n4);
      float *q = (float *)W.vec(1, sizeof(float) * n4);
      if(!p || !q) return GB300_ERR_CUDA;
      k_copy<float><<<grid_for(n4, 256), 256, 0, st>>>(n4, B.val32.p, p);
      for(int i = 0; i < 3; i++)
        bsr_spmv_dot32(B, p, q, part, &S->go, &S->pq, &S->tick_dot, st);
      GB_CUDA(cudaEventRecord(e0, st));
      for(int i = 0; i < reps; i++)
        bsr_spmv_dot32(B, p, q, part, &S->go, &S->pq, &S->tick_dot, st);
      GB_CUDA(cudaEventRecord(e1, st));
    }
  }
  else if(precision == 0) {
    double *p = (double *)W.vec(0, sizeof(double) * n);
    double *q = (double *)W.vec(1, sizeof(double) * n);
    if(!p || !q) return GB300_ERR_CUDA;
    k_copy<double><<<grid_for(n, 256), 256, 0, st>>>(n, A->val.p, p);  // any data
    for(int i = 0; i < 3; i++) cg_spmv<double, double>(A, A->val.p, p, q, part, S, st);
    GB_CUDA(cudaEventRecord(e0, st));
    for(int i = 0; i < reps; i++) cg_spmv<double, double>(A, A->val.p, p, q, part, S, st);
    GB_CUDA(cudaEventRecord(e1, st));
  }
  else {
    DevBuf<float> v32;
    GB_TRY(v32.alloc(A->nnz));
    k_convert<float, double><<<grid_for(A->nnz, 256), 256, 0, st>>>(A->nnz, A->val.p, v32.p);
    float *p = (float *)W.vec(0, sizeof(float) * n);
    float *q = (float *)W.vec(1, sizeof(float) * n);
    if(!p || !q) return GB300_ERR_CUDA;
    k_convert<float, double><<<grid_for(n, 256), 256, 0, st>>>(n, A->val.p, p);
    for(int i = 0; i < 3; i++) cg_spmv<float, float>(A, v32.p, p, q, part, S, st);
    GB_CUDA(cudaEventRecord(e0, st));
    for(int i = 0; i < reps; i++) cg_spmv<float, float>(A, v32.p, p, q, part, S, st);
    GB_CUDA(cudaEventRecord(e1, st));
  }
  GB_CUDA(cudaEventSynchronize(e1));
  GB_CUDA(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = (double)t / (reps > 0 ? reps : 1);
  return GB300_OK;
}

// ---------------------------------------------------------------------------
// Mixed precision CG: FP32 matrix, vectors and SpMV, with FP64 reliable
// updates.  The FP32 iterate accumulates a correction x32; whenever the FP32
// residual has dropped by delta since the last update (or claims
// convergence), the correction is folded into the FP64 solution, the true
// residual b - A x is recomputed in FP64 and replaces the FP32 residual,
// and the search direction is kept.  Convergence is only ever declared on
// the FP64 residual.  This is iterative refinement whose inner solves share
// one Krylov sequence, so the iteration count stays close to the FP64 one.
// ---------------------------------------------------------------------------
__global__ void k_rcg_start(CgState *S, const double *__restrict__ part_rr,
                            double rtol, int maxit, double delta)
{
  double rr = 0.;
  for(int i = threadIdx.x; i < kReduceBlocks; i += blockDim.x) rr += part_rr[i];
  rr = block_sum<double, 256>(rr);
  if(threadIdx.x == 0) {
    S->rho = rr;
    S->res0 = sqrt(rr);
    S->res = S->res0;
    S->tol = rtol * S->res0;
    S->its = 1;
    S->maxit = maxit;
    S->status = 1;
    S->active = 1;
    S->maxrr = rr;
    S->delta2 = delta * delta;
    S->update = S->convert = S->final_ = 0;
    S->updates = 0;
    S->tick_dot = S->tick_step = 0u;
    S->go = S->active;  // no test before the first step (see k_cg_start)
  }
}

__global__ void k_rcg_fold(int n, const CgState *__restrict__ S,
                           double *__restrict__ x, float *__restrict__ x32)
{
  if(!S->active || !S->update) return;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (long long)gridDim.x * blockDim.x) {
    x[i] += (double)x32[i];
    x32[i] = 0.f;
  }
}

__global__ void k_rcg_after(CgState *S, const double *__restrict__ part_rr)
{
  if(!S->active || !S->update) return;
  double rr = 0.;
  for(int i = threadIdx.x; i < kReduceBlocks; i += blockDim.x) rr += part_rr[i];
  rr = block_sum<double, 256>(rr);
  if(threadIdx.x == 0) {
    S->updates += 1;
    S->res = sqrt(rr);
    S->update = 0;
    if(!(S->res > S->tol)) {
      S->status = (S->res == S->res) ? 0 : -10;
      S->active = 0;
      return;
    }
    if(S->final_) {
      S->status = -1;
      S->active = 0;
      return;
    }
    S->beta = rr / S->rho;
    S->rho = rr;
    S->maxrr = rr;
    S->convert = 1;
    S->go = 1;
  }
}

__global__ void k_rcg_convert(int n, const CgState *__restrict__ S,
                              const double *__restrict__ r, float *__restrict__ r32)
{
  if(!S->active || !S->convert) return;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (long long)gridDim.x * blockDim.x)
    r32[i] = (float)r[i];
}

__global__ void k_fold_all(int n, double *__restrict__ x, const float *__restrict__ x32)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) x[i] += (double)x32[i];
}

// the FP32 residual reduction between two FP64 residual replacements
static double reliable_delta(const gb300_solver_params *p)
{
  double d = p->inner_tolerance;
  return (d > 0. && d < 1.) ? d : 0.3;
}

// spmv32(p, q, part, S, st): FP32 q = A p with partial <p, q>;
// res64(x, b, r, part, flag, st): FP64 r = b - A x with partial ||r||^2
template <typename SPMV32, typename RES64>
static int cg_mixed_core(cudaStream_t st, int n, SPMV32 spmv32, RES64 res64,
                         const double *rhs, double *x, double rtol, int maxit,
                         double delta, CgState *hs, Work &W)
{
  float *r32 = (float *)W.vec(0, n * sizeof(float));
  float *p32 = (float *)W.vec(1, n * sizeof(float));
  float *q32 = (float *)W.vec(2, n * sizeof(float));
  float *x32 = (float *)W.vec(3, n * sizeof(float));
  double *r64 = (double *)W.vec(4, n * sizeof(double));
  CgState *S = (CgState *)W.state(sizeof(CgState));
  double *part = W.part();
  if(!r32 || !p32 || !q32 || !x32 || !r64 || !S || !part) return GB300_ERR_CUDA;
  int gl = grid_for(n, 256);
  int gs = grid_for((n + 3) / 4, 256, kReduceBlocks * 4);
  GB_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), st));
  GB_CUDA(cudaMemsetAsync(x32, 0, n * sizeof(float), st));
  k_convert<float, double><<<gl, 256, 0, st>>>(n, rhs, r32);
  k_copy<float><<<gl, 256, 0, st>>>(n, r32, p32);
  dot_part64(n, rhs, rhs, part, st);
  k_rcg_start<<<1, 256, 0, st>>>(S, part, rtol, maxit, delta);
  GB_CUDA(cudaGetLastError());

  // Main graph: a batch of FP32 iterations (SpMV, step, direction).  When a
  // step asks for a reliable update, go drops to 0 and the rest of the
  // batch returns at once; the host then replays the update graph (fold the
  // correction, FP64 residual, restart the FP32 residual, direction) and
  // resumes.  The iterations and their arithmetic are those of the one-graph
  // sequence; only the place where the update kernels run moves.
  const int batch = n > 200000 ? 16 : 32;
  const int step_grid = resident_grid(k_cg_step<float, true>, 256, 0);
  cudaGraph_t graph, ugraph;
  cudaGraphExec_t exec, uexec;
  GB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  for(int it = 0; it < batch; it++) {
    spmv32(p32, q32, part, S, st);
    k_cg_step<float, true><<<step_grid, 256, 0, st>>>(n, S, x32, r32, p32, q32, part);
    k_cg_p<float><<<gs, 256, 0, st>>>(n, S, p32, r32);
  }
  GB_CUDA(cudaStreamEndCapture(st, &graph));
  GB_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  GB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  k_rcg_fold<<<kReduceBlocks, 256, 0, st>>>(n, S, x, x32);
  res64(x, rhs, r64, part, &S->update, st);
  k_rcg_after<<<1, 256, 0, st>>>(S, part);
  k_rcg_convert<<<kReduceBlocks, 256, 0, st>>>(n, S, r64, r32);
  k_cg_p<float><<<gs, 256, 0, st>>>(n, S, p32, r32);
  GB_CUDA(cudaStreamEndCapture(st, &ugraph));
  GB_CUDA(cudaGraphInstantiate(&uexec, ugraph, 0));
  struct Flags {
    int active, update;
  } f = {1, 0};
  long long launches = 0;
  const long long max_launches =
    maxit > 0 ? 2LL * (maxit / batch + 3) + 64 : (1LL << 40);
  auto read_flags = [&]() -> int {
    GB_CUDA(cudaMemcpyAsync(&f.active, &S->active, sizeof(int),
                            cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaMemcpyAsync(&f.update, &S->update, sizeof(int),
                            cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    return GB300_OK;
  };
  int rc = GB300_OK;
  while(f.active && launches < max_launches) {
    if(cudaGraphLaunch(exec, st) != cudaSuccess) {
      rc = GB300_ERR_CUDA;
      break;
    }
    launches++;
    if((rc = read_flags()) != GB300_OK) break;
    if(f.active && f.update) {
      if(cudaGraphLaunch(uexec, st) != cudaSuccess) {
        rc = GB300_ERR_CUDA;
        break;
      }
      if((rc = read_flags()) != GB300_OK) break;
    }
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  cudaGraphExecDestroy(uexec);
  cudaGraphDestroy(ugraph);
  if(rc != GB300_OK) {
    set_error("mixed CG: graph launch failed");
    return rc;
  }
  int active = f.active;
  // anything not folded yet (a break-down stop) joins the FP64 solution
  k_fold_all<<<gl, 256, 0, st>>>(n, x, x32);
  GB_CUDA(cudaMemcpyAsync(hs, S, sizeof(CgState), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(active) hs->status = -1;
  return GB300_OK;
}

// ---------------------------------------------------------------------------
// work space owned by a solve
// ---------------------------------------------------------------------------
void *Work::vec(int slot, size_t bytes)
{
  if(slot < 0 || slot >= kSlots) {
    set_error("work slot %d out of range", slot);
    return nullptr;
  }
  if(vecs[slot].alloc(bytes) != GB300_OK) return nullptr;
  return vecs[slot].p;
}
void *Work::state(size_t bytes)
{
  if(st.alloc(bytes) != GB300_OK) return nullptr;
  return st.p;
}
double *Work::part()
{
  if(parts.alloc(kReduceBlocks * 64) != GB300_OK) return nullptr;
  return parts.p;
}

// ---------------------------------------------------------------------------
// FP64 residual ||b - A x|| (fused), used by the refinement loop and for
// the reported true residual
// ---------------------------------------------------------------------------
int true_residual(const gb300_matrix *A, const double *val, const double *x,
                  const double *b, double *r, double *res, Work &W)
{
  cudaStream_t st = A->ctx->stream;
  double *part = W.part();
  double *d_out = (double *)W.vec(kScratchScalar, sizeof(double) * 2);
  residual64(A, val, x, b, r, part, st);
  sum_partials(part, d_out, st);
  double h = 0.;
  GB_CUDA(cudaMemcpyAsync(&h, d_out, sizeof(double), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  *res = sqrt(h);
  return GB300_OK;
}

int norm2_dev(int n, const double *v, double *out, Work &W, cudaStream_t st)
{
  double *part = W.part();
  double *d_out = (double *)W.vec(kScratchScalar, sizeof(double) * 2);
  dot_part64(n, v, v, part, st);
  sum_partials(part, d_out, st);
  double h = 0.;
  GB_CUDA(cudaMemcpyAsync(&h, d_out, sizeof(double), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  *out = sqrt(h);
  return GB300_OK;
}

__global__ void k_axpy_scaled(int n, double a, const float *__restrict__ d,
                              double *__restrict__ x)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) x[i] += a * (double)d[i];
}

__global__ void k_to32_scaled(int n, double s, const double *__restrict__ r,
                              float *__restrict__ o)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) o[i] = (float)(r[i] * s);
}

// ---------------------------------------------------------------------------
// solve_matrix
// ---------------------------------------------------------------------------
int solve(gb300_matrix *A, const gb300_vector *bvec,
          const gb300_solver_params *p, gb300_vector *xvec,
          gb300_solve_info *info)
{
  gb300_solve_info dummy;
  if(!info) info = &dummy;
  memset(info, 0, sizeof(*info));
  if(!A->csr_valid) {
    set_error("matrix not assembled");
    return GB300_ERR_ARG;
  }
  int n = A->n;
  if(bvec->n != n || xvec->n != n) {
    set_error("vector sizes do not match the matrix");
    return GB300_ERR_ARG;
  }
  if(n == 0) return GB300_OK;  // "No equations in linear system"
  cudaStream_t st = A->ctx->stream;
  Work W;

  // zero-row check (Sparskit.cpp:220-223)
  {
    std::vector<int> rp(n + 1);
    GB_CUDA(cudaMemcpyAsync(rp.data(), A->rowptr.p, sizeof(int) * (n + 1),
                            cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    for(int i = 0; i < n; i++)
      if(rp[i + 1] - rp[i] <= 0) {
        set_error("Zero row in matrix (row %d)", i + 1);
        return GB300_ERR_ZERO_ROW;
      }
  }

  // the system actually solved: scaled copies when Scaling = 1
  const double *val = A->val.p;
  const double *rhs = bvec->d.p;
  DevBuf<double> sval, srhs, s;
  bool scaled = false;
  if(p->scaling == 1) {
    DevBuf<int> zero;
    GB_TRY(zero.alloc(1));
    GB_TRY(s.alloc(n));
    GB_CUDA(cudaMemsetAsync(zero.p, 0, sizeof(int), st));
    k_diag_scal<<<grid_for(n, 256), 256, 0, st>>>(n, A->rowptr.p, A->col.p,
                                                   A->val.p, s.p, zero.p);
    int hz = 0;
    GB_CUDA(cudaMemcpyAsync(&hz, zero.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if(!hz) {  // else "Diagonal scaling aborted because of zero diagonal"
      GB_TRY(sval.alloc(A->nnz));
      GB_TRY(srhs.alloc(n));
      k_scale_vals<<<grid_for(n, 8), 256, 0, st>>>(n, A->rowptr.p, A->col.p,
                                                    A->val.p, s.p, sval.p);
      k_mul<<<grid_for(n, 256), 256, 0, st>>>(n, bvec->d.p, s.p, srhs.p);
      val = sval.p;
      rhs = srhs.p;
      scaled = true;
    }
  }
  else if(p->scaling != 0) {
    set_error("Scaling %d is not supported by this backend", p->scaling);
    return GB300_ERR_UNSUPPORTED;
  }

  double *x = xvec->d.p;
  int rc = GB300_OK;
  if(p->algorithm == 1 && p->preconditioner != 6) {
    // CG; Preconditioner 0 and 8 (DIAGONAL stores alu = 1: the identity,
    // Sparskit.cpp:338-354) both leave the operator unchanged
    // (Precision 2 concerns the ILU factor's storage only: FP64 CG here)
    bool mixed = (p->precision == 1);
    CgState hs;
    Bsr3 B;
    bool blocked = A->block3 &&
                   bsr_build(A, val, true, mixed, B) == GB300_OK &&
                   bsr_tune(A, B, st, !mixed) == GB300_OK;
    if(blocked) {
      // node-major 3x3 blocks: vectors of 4 entries per node
      int nn = B.nn, n4 = 4 * nn;
      double *rhs4 = (double *)W.vec(20, sizeof(double) * n4);
      double *x4 = (double *)W.vec(21, sizeof(double) * n4);
      if(!rhs4 || !x4) return GB300_ERR_CUDA;
      to_nodes64(nn, rhs, rhs4, st);
      if(!mixed) {
        auto spmv = [&](const double *pp, double *qq, double *part,
                        CgState *S, cudaStream_t s) {
          bsr_spmv_dot64(B, pp, qq, part, &S->go, &S->pq, &S->tick_dot, s);
        };
        GB_TRY(cg_core<double>(st, n4, spmv, rhs4, x4, p->stopping_test,
                               p->nb_iter_max, &hs, W));
      }
      else {
        auto spmv = [&](const float *pp, float *qq, double *part,
                        CgState *S, cudaStream_t s) {
          bsr_spmv_dot32(B, pp, qq, part, &S->go, &S->pq, &S->tick_dot, s);
        };
        auto res = [&](const double *xx, const double *bb, double *rr,
                       double *part, const int *flag, cudaStream_t s) {
          bsr_residual64(B, xx, bb, rr, part, flag, s);
        };
        GB_TRY(cg_mixed_core(st, n4, spmv, res, rhs4, x4, p->stopping_test,
                             p->nb_iter_max, reliable_delta(p), &hs, W));
      }
      from_nodes64(nn, x4, x, st);
      GB_TRY(bsr_check(B, st));
    }
    else if(!mixed) {
      auto spmv = [&](const double *pp, double *qq, double *part,
                      CgState *S, cudaStream_t s) {
        cg_spmv<double, double>(A, val, pp, qq, part, S, s);
      };
      GB_TRY(cg_core<double>(st, n, spmv, rhs, x, p->stopping_test,
                             p->nb_iter_max, &hs, W));
    }
    else {
      DevBuf<float> v32;
      GB_TRY(v32.alloc(A->nnz > 0 ? A->nnz : 1));
      k_convert<float, double><<<grid_for(A->nnz, 256), 256, 0, st>>>(A->nnz, val, v32.p);
      const float *v32p = v32.p;
      auto spmv = [&](const float *pp, float *qq, double *part,
                      CgState *S, cudaStream_t s) {
        cg_spmv<float, float>(A, v32p, pp, qq, part, S, s);
      };
      auto res = [&](const double *xx, const double *bb, double *rr,
                     double *part, const int *flag, cudaStream_t s) {
        residual64_guarded(A, val, xx, bb, rr, part, flag, s);
      };
      GB_TRY(cg_mixed_core(st, n, spmv, res, rhs, x, p->stopping_test,
                           p->nb_iter_max, reliable_delta(p), &hs, W));
    }
    info->status = hs.status;
    info->iterations = hs.its;
    info->residual_estimate = hs.res;
    if(mixed) {
      info->inner_iterations = hs.its - 1;
      info->refinement_steps = hs.updates;
    }
  }
  else if(p->algorithm == 8 || p->algorithm == 9 ||
          (p->algorithm == 1 && (p->preconditioner == 6 ||
                                 p->preconditioner == kPrecondLearned))) {
    // the two-level cycles without aggregates from the caller: from A's graph
    if(precond_two_level(p->preconditioner) && !coarse_valid(A))
      GB_TRY(coarse_auto(A, std::min(kAutoAggregates, std::max(1, A->n / 16))));
    // Renumbering_Technique 1 (RCMK in Sparskit): this backend's own
    // renumbering, a multicolour ordering, for the ILU(0) solves
    bool used = false;
    // Renumbering_Technique 2 (no Sparskit value): the reference's RCMK
    // order itself, for its default iteration trajectory
    if((p->renumbering_technique == 1 || p->renumbering_technique == 2) &&
       (p->preconditioner == 6 || p->preconditioner == kPrecondLearned ||
        p->preconditioner == kPrecondCoarse || p->preconditioner == kPrecondLearnedCoarse ||
        p->preconditioner == kPrecondLearnedCoarsePre)) {
      // (24 has no triangular sweeps: it keeps GetDP's order)
      rc = gmres_solve_coloured(A, val, rhs, x, p, info, W, &used);
      if(rc != GB300_OK) return rc;
    }
    if(!used) {
      rc = gmres_solve(A, val, rhs, x, p, info, W);
      if(rc != GB300_OK) return rc;
    }
  }
  else {
    set_error("Algorithm %d is not supported by this backend", p->algorithm);
    return GB300_ERR_UNSUPPORTED;
  }

  // the reported true residual, on the system solved
  {
    double *r = (double *)W.vec(kScratchRes, sizeof(double) * n);
    double res = 0., bn = 0.;
    GB_TRY(true_residual(A, val, x, rhs, r, &res, W));
    GB_TRY(norm2_dev(n, rhs, &bn, W, st));
    info->true_residual = res;
    info->rhs_norm = bn;
  }
  if(scaled)  // x <- D y (scale_vector COLUMN, Sparskit.cpp:631-632)
    k_mul<<<grid_for(n, 256), 256, 0, st>>>(n, x, s.p, x);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(st));
  if(info->status != 0) {
    set_error("Iterative solver terminated (code = %d) after %d iterations",
              info->status, info->iterations);
    return GB300_ERR_SOLVER;
  }
  return rc;
}

// ---------------------------------------------------------------------------
// independent systems held as the diagonal blocks of A: the batched form of
// solve() (same scaling, renumbering and Krylov methods, one per block)
// ---------------------------------------------------------------------------
int solve_batch(gb300_matrix *A, const gb300_vector *bvec,
                const gb300_solver_params *p, gb300_vector *xvec, int nsys,
                const int *off, gb300_solve_info *infos)
{
  if(!A->csr_valid) {
    set_error("matrix not assembled");
    return GB300_ERR_ARG;
  }
  const int n = A->n;
  if(bvec->n != n || xvec->n != n) {
    set_error("vector sizes do not match the matrix");
    return GB300_ERR_ARG;
  }
  if(nsys < 1 || !off || !infos || off[0] != 0 || off[nsys] != n) {
    set_error("batched solve: offsets must run from 0 to the matrix size");
    return GB300_ERR_ARG;
  }
  for(int q = 0; q < nsys; q++)
    if(off[q + 1] < off[q]) {
      set_error("batched solve: offsets must not decrease (system %d)", q);
      return GB300_ERR_ARG;
    }
  if(n == 0) {
    for(int q = 0; q < nsys; q++) memset(&infos[q], 0, sizeof(infos[q]));
    return GB300_OK;
  }
  if(check_blocks(A, nsys, off) != GB300_OK) {
    set_error("batched solve: an entry couples two systems");
    return GB300_ERR_ARG;
  }
  cudaStream_t st = A->ctx->stream;
  Work W;
  {
    std::vector<int> rp(n + 1);
    GB_CUDA(cudaMemcpyAsync(rp.data(), A->rowptr.p, sizeof(int) * (n + 1),
                            cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    for(int i = 0; i < n; i++)
      if(rp[i + 1] - rp[i] <= 0) {
        set_error("Zero row in matrix (row %d)", i + 1);
        return GB300_ERR_ZERO_ROW;
      }
  }
  const double *val = A->val.p;
  const double *rhs = bvec->d.p;
  DevBuf<double> sval, srhs, s;
  bool scaled = false;
  if(p->scaling == 1) {
    DevBuf<int> zero;
    GB_TRY(zero.alloc(1));
    GB_TRY(s.alloc(n));
    GB_CUDA(cudaMemsetAsync(zero.p, 0, sizeof(int), st));
    k_diag_scal<<<grid_for(n, 256), 256, 0, st>>>(n, A->rowptr.p, A->col.p, A->val.p,
                                                   s.p, zero.p);
    int hz = 0;
    GB_CUDA(cudaMemcpyAsync(&hz, zero.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if(!hz) {
      GB_TRY(sval.alloc(A->nnz));
      GB_TRY(srhs.alloc(n));
      k_scale_vals<<<grid_for(n, 8), 256, 0, st>>>(n, A->rowptr.p, A->col.p, A->val.p,
                                                    s.p, sval.p);
      k_mul<<<grid_for(n, 256), 256, 0, st>>>(n, bvec->d.p, s.p, srhs.p);
      val = sval.p;
      rhs = srhs.p;
      scaled = true;
    }
  }
  double *x = xvec->d.p;
  bool coloured = false;
  if(p->renumbering_technique == 1 && p->preconditioner == 6) {
    int rc = colour_build(A, nsys, off);
    if(rc != GB300_OK && rc != GB300_ERR_UNSUPPORTED) return rc;
    coloured = (rc == GB300_OK);
  }
  if(coloured) {
    Colouring *C = A->mc;
    gb300_matrix *B = C->B;
    DevBuf<double> rb, yb;
    GB_TRY(rb.alloc(n));
    GB_TRY(yb.alloc(n));
    permute_system(C, A->nnz, val, rhs, B->val.p, rb.p, st);
    bool used = false;
    GB_TRY(gmres_solve_batch_cluster(B, B->val.p, rb.p, yb.p, p, nsys, off, infos, W, &used,
                                     C));
    if(!used) GB_TRY(gmres_solve_batch(B, B->val.p, rb.p, yb.p, p, nsys, off, infos, W));
    unpermute_solution(C, yb.p, x, st);
  }
  else {
    bool used = false;
    GB_TRY(gmres_solve_batch_cluster(A, val, rhs, x, p, nsys, off, infos, W, &used));
    if(!used) GB_TRY(gmres_solve_batch(A, val, rhs, x, p, nsys, off, infos, W));
  }
  if(scaled) k_mul<<<grid_for(n, 256), 256, 0, st>>>(n, x, s.p, x);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(st));
  int failed = 0, first = -1;
  for(int q = 0; q < nsys; q++)
    if(infos[q].status != 0) {
      failed++;
      if(first < 0) first = q;
    }
  if(failed) {
    set_error("Iterative solver terminated in %d of %d systems (first: system %d, "
              "code = %d after %d iterations)",
              failed, nsys, first, infos[first].status, infos[first].iterations);
    return GB300_ERR_SOLVER;
  }
  return GB300_OK;
}

}  // namespace gb
