// Two-level preconditioning on aggregates (Preconditioners 21 and 22; no
// counterpart in Sparskit, whose preconditioners are one-level).
//
// The unknowns are grouped into aggregates (gb300_matrix_set_aggregates:
// one aggregate number per row, given by the caller; geometric cells of the
// mesh, for instance).  P0 is the piecewise-constant prolongation (row i has
// a single 1 in column agg[i]); the coarse matrix Ac = P0^T A P0 sums A's
// entries by (aggregate of the row, aggregate of the column) and is inverted
// densely on the device.  One application of the preconditioner is the
// symmetric two-level cycle
//
//   z  = S v                          ILU(0) smoothing (+ the learned correction)
//   z += P0 Ac^-1 P0^T (v - A z)      exact coarse correction
//   z += S (v - A z)                  second smoothing
//
// ILU(0) alone removes the oscillating part of the error and leaves the
// smooth part, which costs one-level preconditioned Krylov methods a number
// of steps that grows with the mesh size; the coarse correction removes the
// smooth part on the aggregates.
//
// Everything here is deterministic:
//   * Ac is summed in 64-bit fixed point (integer atomic adds are exact and
//     associative), with a power-of-two quantum chosen from max|a_ij| and
//     the largest number of entries one coarse entry can receive, so that
//     no sum can overflow; each term is rounded once, by at most half a
//     quantum, 2^(h-62) of max|a_ij| with h - 1 the bits of the largest
//     number of entries one coarse entry receives (2^-51 for 1,000);
//   * the dense inverse is Gauss-Jordan elimination without pivoting, one
//     launch per pivot (Ac is symmetric positive definite when A is and no
//     aggregate is empty; a pivot <= 0 is reported as an error);
//   * restriction and the coarse product are warp sums in a fixed order.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <functional>
#include <vector>

#include "common.cuh"
#include "krylov.cuh"
#include "sparse.cuh"

namespace gb {

void coarse_free(Coarse *c) { delete c; }

void coarse_values_changed(gb300_matrix *A)
{
  if(A->coarse) A->coarse->ready = false;
}

bool coarse_valid(const gb300_matrix *A)
{
  return A->coarse && A->coarse->version == A->pattern_version && A->coarse->nc > 0 &&
         A->nnz > 0;
}

int coarse_set(gb300_matrix *A, const int *agg, int nc)
{
  const int n = A->n;
  if(nc < 1 || nc > kMaxCoarse) {
    set_error("aggregates: %d aggregates (1 to %d supported)", nc, kMaxCoarse);
    return GB300_ERR_ARG;
  }
  if(!A->csr_valid || A->nnz <= 0) {
    set_error("aggregates: the matrix has no assembled pattern");
    return GB300_ERR_ARG;
  }
  std::vector<int> cnt(nc + 1, 0);
  for(int i = 0; i < n; i++) {
    if(agg[i] < 0 || agg[i] >= nc) {
      set_error("aggregates: row %d has aggregate %d, outside 0..%d", i, agg[i], nc - 1);
      return GB300_ERR_ARG;
    }
    cnt[agg[i] + 1]++;
  }
  for(int k = 0; k < nc; k++)
    if(cnt[k + 1] == 0) {
      set_error("aggregates: aggregate %d has no row", k);
      return GB300_ERR_ARG;
    }
  for(int k = 0; k < nc; k++) cnt[k + 1] += cnt[k];
  std::vector<int> perm(n), pos(cnt.begin(), cnt.end() - 1);
  for(int i = 0; i < n; i++) perm[pos[agg[i]]++] = i;
  // headroom of the fixed-point sums: the entries summed into one coarse
  // entry come from the rows of one aggregate
  std::vector<int> rp(n + 1);
  cudaStream_t st = A->ctx->stream;
  GB_CUDA(cudaMemcpyAsync(rp.data(), A->rowptr.p, sizeof(int) * (n + 1),
                          cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  long long most = 0;
  for(int k = 0; k < nc; k++) {
    long long s = 0;
    for(int q = cnt[k]; q < cnt[k + 1]; q++) s += rp[perm[q] + 1] - rp[perm[q]];
    most = std::max(most, s);
  }
  int head = 1;
  while((1LL << (head - 1)) < most + 1) head++;
  if(!A->coarse) A->coarse = new Coarse();
  Coarse *c = A->coarse;
  c->n = n;
  c->nc = nc;
  c->headroom = head;
  c->stamp++;
  c->ready = false;
  GB_TRY(c->agg.alloc(n));
  GB_TRY(c->aperm.alloc(n));
  GB_TRY(c->aptr.alloc(nc + 1));
  GB_TRY(c->inv.alloc((size_t)nc * nc));
  GB_TRY(c->rbuf.alloc(2 * (size_t)nc));
  GB_TRY(c->cbuf.alloc(2 * (size_t)nc));
  GB_TRY(c->rc.alloc(nc));
  GB_TRY(c->ec.alloc(nc));
  GB_TRY(c->err.alloc(1));
  GB_TRY(c->amax.alloc(1));
  GB_CUDA(cudaMemcpyAsync(c->agg.p, agg, sizeof(int) * n, cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaMemcpyAsync(c->aperm.p, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice,
                          st));
  GB_CUDA(cudaMemcpyAsync(c->aptr.p, cnt.data(), sizeof(int) * (nc + 1),
                          cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaStreamSynchronize(st));
  c->version = A->pattern_version;
  return GB300_OK;
}

// ---------------------------------------------------------------------------
// aggregates from A's graph alone (when the caller has no mesh to give):
// greedy breadth-first aggregation -- from the first row not yet taken,
// take rows breadth-first over A's pattern until the aggregate holds
// ceil(n / target) rows; then rows of aggregates below a quarter of that
// size join the neighbouring aggregate they have most entries with.  On
// the 2D nonlinear Jacobian at 128^2 (ILU(0) smoothing, GMRES(50) to
// 1e-10) these took 96 steps against 121 with square cells of the mesh.

int coarse_auto(gb300_matrix *A, int target)
{
  const int n = A->n;
  if(!A->csr_valid || A->nnz <= 0 || n <= 0) {
    set_error("aggregates: the matrix has no assembled pattern");
    return GB300_ERR_ARG;
  }
  target = std::max(1, std::min(target, kMaxCoarse));
  std::vector<int> rp(n + 1), ci(A->nnz);
  cudaStream_t st = A->ctx->stream;
  GB_CUDA(cudaMemcpyAsync(rp.data(), A->rowptr.p, sizeof(int) * (n + 1),
                          cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaMemcpyAsync(ci.data(), A->col.p, sizeof(int) * A->nnz,
                          cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  std::vector<int> agg(n), queue(n), cnt;
  long long size = (n + target - 1) / target;
  int nc = 0;
  for(;;) {
    std::fill(agg.begin(), agg.end(), -1);
    nc = 0;
    for(int seed = 0; seed < n; seed++) {
      if(agg[seed] >= 0) continue;
      int head = 0, tail = 0;
      long long got = 1;
      agg[seed] = nc;
      queue[tail++] = seed;
      while(head < tail && got < size) {
        const int i = queue[head++];
        for(int k = rp[i]; k < rp[i + 1] && got < size; k++) {
          const int j = ci[k];
          if(agg[j] < 0) {
            agg[j] = nc;
            queue[tail++] = j;
            got++;
          }
        }
      }
      nc++;
    }
    cnt.assign(nc, 0);
    for(int i = 0; i < n; i++) cnt[agg[i]]++;
    const long long small = size / 4;
    std::vector<std::pair<int, int>> seen;
    for(int i = 0; i < n; i++) {
      if(cnt[agg[i]] >= small) continue;
      seen.clear();
      for(int k = rp[i]; k < rp[i + 1]; k++) {
        const int a = agg[ci[k]];
        if(cnt[a] < small) continue;
        bool found = false;
        for(auto &pr : seen)
          if(pr.first == a) {
            pr.second++;
            found = true;
            break;
          }
        if(!found) seen.push_back({a, 1});
      }
      int best = -1, bc = 0;
      for(auto &pr : seen)
        if(pr.second > bc) {
          best = pr.first;
          bc = pr.second;
        }
      if(best >= 0) agg[i] = best;  // (counts stay those of the first pass)
    }
    // compact the numbering (aggregates emptied by the merge disappear)
    std::vector<int> id(nc, -1);
    int m = 0;
    for(int i = 0; i < n; i++) {
      if(id[agg[i]] < 0) id[agg[i]] = m++;
      agg[i] = id[agg[i]];
    }
    nc = m;
    if(nc <= kMaxCoarse) break;
    size *= 2;  // too many aggregates: grow them
  }
  return coarse_set(A, agg.data(), nc);
}

// ---------------------------------------------------------------------------
// a permuted copy of A (the multicolour ordering) follows A's aggregates

__global__ void k_follow_agg(int n, const int *__restrict__ old_of,
                             const int *__restrict__ agg, const int *__restrict__ new_of,
                             const int *__restrict__ aperm, int *__restrict__ bagg,
                             int *__restrict__ baperm)
{
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    bagg[i] = agg[old_of[i]];       // new row i is old row old_of[i]
    baperm[i] = new_of[aperm[i]];   // same aggregate order, rows renamed
  }
}

int coarse_follow(const gb300_matrix *A, gb300_matrix *B, const Colouring *C,
                  cudaStream_t st)
{
  const Coarse *a = A->coarse;
  if(!B->coarse) B->coarse = new Coarse();
  Coarse *c = B->coarse;
  if(c->followed == a->stamp && c->version == B->pattern_version && c->nc == a->nc)
    return GB300_OK;
  const int n = A->n, nc = a->nc;
  c->n = n;
  c->nc = nc;
  c->headroom = a->headroom;
  c->ready = false;
  GB_TRY(c->agg.alloc(n));
  GB_TRY(c->aperm.alloc(n));
  GB_TRY(c->aptr.alloc(nc + 1));
  GB_TRY(c->inv.alloc((size_t)nc * nc));
  GB_TRY(c->rbuf.alloc(2 * (size_t)nc));
  GB_TRY(c->cbuf.alloc(2 * (size_t)nc));
  GB_TRY(c->rc.alloc(nc));
  GB_TRY(c->ec.alloc(nc));
  GB_TRY(c->err.alloc(1));
  GB_TRY(c->amax.alloc(1));
  k_follow_agg<<<grid_for(n, 256), 256, 0, st>>>(n, C->old_of.p, a->agg.p, C->new_of.p,
                                                 a->aperm.p, c->agg.p, c->aperm.p);
  GB_CUDA(cudaMemcpyAsync(c->aptr.p, a->aptr.p, sizeof(int) * (nc + 1),
                          cudaMemcpyDeviceToDevice, st));
  GB_CUDA(cudaGetLastError());
  c->followed = a->stamp;
  c->version = B->pattern_version;
  return GB300_OK;
}

// ---------------------------------------------------------------------------
// set-up: Ac = P0^T A P0 in fixed point, then its inverse

// max |val| (non-negative doubles order like their bit patterns; a NaN
// orders above +Inf and is caught by the scatter)
__global__ void k_abs_max(long long nnz, const double *__restrict__ val,
                          unsigned long long *out)
{
  unsigned long long m = 0;
  for(long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
      k += (long long)gridDim.x * blockDim.x)
    m = max(m, (unsigned long long)__double_as_longlong(fabs(val[k])));
  for(int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// every row's entries, summed by the aggregate of their column (one atomic
// add per run of equal aggregates), into acc[agg(row) * nc + agg(col)]
__global__ void k_coarse_scatter(int n, const int *__restrict__ rowptr,
                                 const int *__restrict__ col, const double *__restrict__ val,
                                 const int *__restrict__ agg, const int *__restrict__ aperm,
                                 int nc, int headroom, const unsigned long long *amax_bits,
                                 unsigned long long *acc, int *err)
{
  const double am = __longlong_as_double((long long)*amax_bits);
  if(!(am <= 1.7976931348623157e308) || am == 0.) {  // NaN, Inf or a zero matrix
    if(blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(err, 0, -1);
    return;
  }
  int e = 0;
  frexp(am, &e);  // am < 2^e
  const double s = ldexp(1.0, 62 - headroom - e);
  for(int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int i = aperm[q];
    const size_t base = (size_t)agg[i] * nc;
    int run = -1;
    long long sum = 0;
    for(int k = rowptr[i]; k < rowptr[i + 1]; k++) {
      const int l = agg[col[k]];
      if(l != run) {
        if(run >= 0) atomicAdd(acc + base + run, (unsigned long long)sum);
        run = l;
        sum = 0;
      }
      sum += llrint(val[k] * s);
    }
    if(run >= 0) atomicAdd(acc + base + run, (unsigned long long)sum);
  }
}

__global__ void k_coarse_to_double(long long m, int headroom,
                                   const unsigned long long *amax_bits, double *a)
{
  const double am = __longlong_as_double((long long)*amax_bits);
  int e = 0;
  frexp(am, &e);
  const double qnt = ldexp(1.0, e + headroom - 62);
  unsigned long long *acc = reinterpret_cast<unsigned long long *>(a);
  for(long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < m;
      k += (long long)gridDim.x * blockDim.x) {
    const long long v = (long long)acc[k];
    a[k] = (double)v * qnt;
  }
}

__global__ void k_gj_init(int nc, const double *__restrict__ a, double *rbuf, double *cbuf)
{
  for(int j = blockIdx.x * blockDim.x + threadIdx.x; j < nc; j += gridDim.x * blockDim.x) {
    rbuf[j] = a[j];                 // row 0
    cbuf[j] = a[(size_t)j * nc];    // column 0
  }
}

// pivot step k of the in-place Gauss-Jordan inversion; row k and column k of
// the matrix before the step come from the buffers of parity k, and the step
// writes row and column k + 1 of its result to the other parity
__global__ void k_gj_step(int nc, int k, double *a, double *rbuf, double *cbuf, int *err)
{
  if(*err) return;
  const double *R = rbuf + (size_t)(k & 1) * nc;
  const double *Cc = cbuf + (size_t)(k & 1) * nc;
  double *Rn = rbuf + (size_t)((k + 1) & 1) * nc;
  double *Cn = cbuf + (size_t)((k + 1) & 1) * nc;
  const double piv = R[k];
  if(!(piv > 0.) || !(piv <= 1.7976931348623157e308)) {
    if(blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(err, 0, k + 1);
    return;
  }
  const double p = 1.0 / piv;
  const long long m = (long long)nc * nc;
  for(long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < m;
      idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / nc), j = (int)(idx - (long long)i * nc);
    double v;
    if(i == k)
      v = (j == k) ? p : R[j] * p;
    else if(j == k)
      v = -Cc[i] * p;
    else
      v = fma(-Cc[i] * p, R[j], a[idx]);
    a[idx] = v;
    if(i == k + 1) Rn[j] = v;
    if(j == k + 1) Cn[i] = v;
  }
}

int coarse_setup(gb300_matrix *A, const double *val, bool reuse)
{
  Coarse *c = A->coarse;
  if(reuse && c->ready) return GB300_OK;
  cudaStream_t st = A->ctx->stream;
  const int nc = c->nc, n = A->n;
  const long long m = (long long)nc * nc;
  unsigned long long *amax = reinterpret_cast<unsigned long long *>(c->amax.p);
  GB_CUDA(cudaMemsetAsync(amax, 0, sizeof(unsigned long long), st));
  GB_CUDA(cudaMemsetAsync(c->err.p, 0, sizeof(int), st));
  GB_CUDA(cudaMemsetAsync(c->inv.p, 0, sizeof(double) * m, st));
  k_abs_max<<<grid_for(A->nnz, 256, kReduceBlocks), 256, 0, st>>>(A->nnz, val, amax);
  k_coarse_scatter<<<grid_for(n, 128), 128, 0, st>>>(
      n, A->rowptr.p, A->col.p, val, c->agg.p, c->aperm.p, nc, c->headroom, amax,
      reinterpret_cast<unsigned long long *>(c->inv.p), c->err.p);
  k_coarse_to_double<<<grid_for(m, 256, kReduceBlocks), 256, 0, st>>>(m, c->headroom, amax,
                                                                      c->inv.p);
  GB_CUDA(cudaGetLastError());
  const void *key[4] = {c->inv.p, c->rbuf.p, c->cbuf.p, c->err.p};
  if(!c->gj_exec || c->gj_nc != nc || memcmp(key, c->gj_key, sizeof(key)) != 0) {
    if(c->gj_exec) cudaGraphExecDestroy(c->gj_exec);
    c->gj_exec = nullptr;
    cudaGraph_t graph;
    GB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    k_gj_init<<<grid_for(nc, 256), 256, 0, st>>>(nc, c->inv.p, c->rbuf.p, c->cbuf.p);
    const int g = grid_for(m, 256, kReduceBlocks * 2);
    for(int k = 0; k < nc; k++)
      k_gj_step<<<g, 256, 0, st>>>(nc, k, c->inv.p, c->rbuf.p, c->cbuf.p, c->err.p);
    GB_CUDA(cudaStreamEndCapture(st, &graph));
    cudaError_t e = cudaGraphInstantiate(&c->gj_exec, graph, 0);
    cudaGraphDestroy(graph);
    if(e != cudaSuccess) {
      c->gj_exec = nullptr;
      set_error("coarse matrix: graph instantiation failed: %s", cudaGetErrorString(e));
      return GB300_ERR_CUDA;
    }
    c->gj_nc = nc;
    memcpy(c->gj_key, key, sizeof(key));
  }
  GB_CUDA(cudaGraphLaunch(c->gj_exec, st));
  int err = 0;
  GB_CUDA(cudaMemcpyAsync(&err, c->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(err < 0) {
    set_error("coarse matrix: the matrix values are zero or not finite");
    return GB300_ERR_ARG;
  }
  if(err > 0) {
    set_error("coarse matrix P^T A P is not positive definite (pivot %d of %d)", err, nc);
    return GB300_ERR_ZERO_PIVOT;
  }
  c->ready = true;
  return GB300_OK;
}

// ---------------------------------------------------------------------------
// application

__global__ void k_add_into(int n, const double *__restrict__ t, double *__restrict__ z,
                           const int *flag)
{
  if(flag && !*flag) return;
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    z[i] += t[i];
}

// rc = P0^T t: one warp per aggregate, its rows in a fixed order
__global__ void k_restrict(int nc, const int *__restrict__ aptr, const int *__restrict__ aperm,
                           const double *__restrict__ t, double *__restrict__ rc,
                           const int *flag)
{
  if(flag && !*flag) return;
  const int lane = threadIdx.x & 31;
  for(int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < nc;
      k += (gridDim.x * blockDim.x) >> 5) {
    double s = 0.;
    for(int q = aptr[k] + lane; q < aptr[k + 1]; q += 32) s += t[aperm[q]];
    s = warp_sum(s);
    if(lane == 0) rc[k] = s;
  }
}

// ec = Ainv rc: one warp per row
__global__ void k_coarse_gemv(int nc, const double *__restrict__ inv,
                              const double *__restrict__ rc, double *__restrict__ ec,
                              const int *flag)
{
  if(flag && !*flag) return;
  const int lane = threadIdx.x & 31;
  for(int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nc;
      i += (gridDim.x * blockDim.x) >> 5) {
    const double *row = inv + (size_t)i * nc;
    double s = 0.;
    for(int j = lane; j < nc; j += 32) s = fma(row[j], rc[j], s);
    s = warp_sum(s);
    if(lane == 0) ec[i] = s;
  }
}

// z += P0 ec
__global__ void k_prolong(int n, const int *__restrict__ agg, const double *__restrict__ ec,
                          double *__restrict__ z, const int *flag)
{
  if(flag && !*flag) return;
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    z[i] += ec[agg[i]];
}

void coarse_correct(const gb300_matrix *A, const double *val, const double *v, double *z,
                    double *t, const int *flag, cudaStream_t st)
{
  const Coarse *c = A->coarse;
  const int n = A->n, nc = c->nc;
  const int g = grid_for(n, 256, kReduceBlocks * 4);
  resid_guarded(A, val, z, v, t, flag, st);  // t = v - A z
  k_restrict<<<grid_for((long long)nc * 32, 256), 256, 0, st>>>(nc, c->aptr.p, c->aperm.p,
                                                                t, c->rc.p, flag);
  k_coarse_gemv<<<grid_for((long long)nc * 32, 256), 256, 0, st>>>(nc, c->inv.p, c->rc.p,
                                                                   c->ec.p, flag);
  k_prolong<<<g, 256, 0, st>>>(n, c->agg.p, c->ec.p, z, flag);
}

// one block: out = rc . ec over the nc coarse entries, in a fixed order
__global__ void k_coarse_dot(int nc, const double *__restrict__ a,
                             const double *__restrict__ b, double *out)
{
  __shared__ double sh[32];
  double s = 0.;
  for(int k = threadIdx.x; k < nc; k += blockDim.x) s = fma(a[k], b[k], s);
  s = warp_sum(s);
  if((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if(threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.;
    s = warp_sum(s);
    if(threadIdx.x == 0) *out = s;
  }
}

__global__ void k_prolong_set(int n, const int *__restrict__ agg, const double *__restrict__ ec,
                              double *__restrict__ t)
{
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    t[i] = ec[agg[i]];
}

__global__ void k_sub_into(int n, const double *__restrict__ q, double *__restrict__ w)
{
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    w[i] -= q[i];
}

int coarse_energy_project(gb300_matrix *A, double *w, double *t, double *q, double *wcw,
                          cudaStream_t st)
{
  GB_TRY(coarse_setup(A, A->val.p, true));
  const Coarse *c = A->coarse;
  const int n = A->n, nc = c->nc;
  const int g = grid_for(n, 256, kReduceBlocks * 4);
  k_restrict<<<grid_for((long long)nc * 32, 256), 256, 0, st>>>(nc, c->aptr.p, c->aperm.p,
                                                                w, c->rc.p, nullptr);
  k_coarse_gemv<<<grid_for((long long)nc * 32, 256), 256, 0, st>>>(nc, c->inv.p, c->rc.p,
                                                                   c->ec.p, nullptr);
  k_coarse_dot<<<1, 1024, 0, st>>>(nc, c->rc.p, c->ec.p, wcw);
  k_prolong_set<<<g, 256, 0, st>>>(n, c->agg.p, c->ec.p, t);
  spmv_plain(A, A->val.p, t, q, st);
  k_sub_into<<<g, 256, 0, st>>>(n, q, w);
  GB_CUDA(cudaGetLastError());
  return GB300_OK;
}

int coarse_energy(gb300_matrix *A, const double *u, double *ucu_dev, cudaStream_t st)
{
  GB_TRY(coarse_setup(A, A->val.p, true));
  const Coarse *c = A->coarse;
  const int nc = c->nc;
  k_restrict<<<grid_for((long long)nc * 32, 256), 256, 0, st>>>(nc, c->aptr.p, c->aperm.p,
                                                                u, c->rc.p, nullptr);
  k_coarse_gemv<<<grid_for((long long)nc * 32, 256), 256, 0, st>>>(nc, c->inv.p, c->rc.p,
                                                                   c->ec.p, nullptr);
  k_coarse_dot<<<1, 1024, 0, st>>>(nc, c->rc.p, c->ec.p, ucu_dev);
  GB_CUDA(cudaGetLastError());
  return GB300_OK;
}

void two_level_apply(const gb300_matrix *A, const double *val, const double *v, double *z,
                     double *t3, double *t4, const int *flag, cudaStream_t st,
                     const std::function<void(const double *, double *)> &smooth,
                     const std::function<void(const double *, double *)> &smooth_post)
{
  const int n = A->n;
  const int g = grid_for(n, 256, kReduceBlocks * 4);
  smooth(v, z);
  coarse_correct(A, val, v, z, t3, flag, st);
  resid_guarded(A, val, z, v, t3, flag, st);  // t3 = v - A z
  smooth_post(t3, t4);
  k_add_into<<<g, 256, 0, st>>>(n, t4, z, flag);
}

}  // namespace gb
