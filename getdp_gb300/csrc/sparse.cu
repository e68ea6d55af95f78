// CSR construction and the sparse kernels of the solver.
//
// * pattern from element tables: the rows of unknowns each element couples,
//   merged and sorted -- the pattern GetDP's per-column linked lists end up
//   with after csr_format (contrib/Sparskit/Sparskit.cpp:809-862, :2186-2217);
// * COO -> CSR for LinAlg-style scalar adds, duplicates summed in call order
//   (the a[iptr] += val accumulation of add_matrix_double);
// * CSR SpMV (amux, contrib/Sparskit/matvec.f:35) with a fixed number of
//   threads per row and deterministic fused reductions.
#include "sparse.cuh"

namespace gb {

// ---------------------------------------------------------------------------
// exclusive scan of int counts into int64 offsets (three phases, fixed order)
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 1024;

__global__ void k_scan_blocks(const int *__restrict__ in, long long n,
                              long long *__restrict__ out,
                              long long *__restrict__ block_sums)
{
  __shared__ long long s[kScanThreads];
  long long i = (long long)blockIdx.x * kScanThreads + threadIdx.x;
  long long v = (i < n) ? in[i] : 0;
  s[threadIdx.x] = v;
  __syncthreads();
  for(int o = 1; o < kScanThreads; o <<= 1) {
    long long t = (threadIdx.x >= o) ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  if(i < n) out[i] = s[threadIdx.x] - v;
  if(threadIdx.x == kScanThreads - 1) block_sums[blockIdx.x] = s[threadIdx.x];
}

__global__ void k_scan_sums(long long *sums, int nb, long long *total)
{
  // single block: sequential carry over chunks of 1024
  __shared__ long long s[kScanThreads];
  __shared__ long long carry;
  if(threadIdx.x == 0) carry = 0;
  __syncthreads();
  for(int base = 0; base < nb; base += kScanThreads) {
    int i = base + threadIdx.x;
    long long v = (i < nb) ? sums[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for(int o = 1; o < kScanThreads; o <<= 1) {
      long long t = (threadIdx.x >= o) ? s[threadIdx.x - o] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if(i < nb) sums[i] = carry + s[threadIdx.x] - v;
    __syncthreads();
    if(threadIdx.x == kScanThreads - 1) carry += s[threadIdx.x];
    __syncthreads();
  }
  if(threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(long long *out, long long n, const long long *sums)
{
  long long i = (long long)blockIdx.x * kScanThreads + threadIdx.x;
  if(i < n) out[i] += sums[blockIdx.x];
}

int exclusive_scan(const int *in, long long n, long long *out, long long *total,
                   DevBuf<long long> &tmp, cudaStream_t st)
{
  int nb = grid_for(n, kScanThreads);
  GB_TRY(tmp.alloc(nb + 1));
  k_scan_blocks<<<nb, kScanThreads, 0, st>>>(in, n, out, tmp.p);
  k_scan_sums<<<1, kScanThreads, 0, st>>>(tmp.p, nb, tmp.p + nb);
  k_scan_add<<<nb, kScanThreads, 0, st>>>(out, n, tmp.p);
  GB_CUDA(cudaGetLastError());
  if(total)
    GB_CUDA(cudaMemcpyAsync(total, tmp.p + nb, sizeof(long long),
                            cudaMemcpyDeviceToHost, st));
  return GB300_OK;
}

__global__ void k_i64_to_i32(const long long *in, long long n, int *out)
{
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) out[i] = (int)in[i];
}

// ---------------------------------------------------------------------------
// bitonic sort of a power-of-two array in shared memory
// ---------------------------------------------------------------------------
template <typename K>
__device__ void smem_bitonic_sort(K *s, int P)
{
  for(int k = 2; k <= P; k <<= 1) {
    for(int j = k >> 1; j > 0; j >>= 1) {
      for(int t = threadIdx.x; t < P / 2; t += blockDim.x) {
        int i = 2 * j * (t / j) + (t % j);
        int l = i + j;
        bool up = ((i & k) == 0);
        K a = s[i], b = s[l];
        if((a > b) == up) {
          s[i] = b;
          s[l] = a;
        }
      }
      __syncthreads();
    }
  }
}

__device__ __forceinline__ int next_pow2(int v)
{
  int p = 1;
  while(p < v) p <<= 1;
  return p;
}

// ---------------------------------------------------------------------------
// pattern from element tables
// ---------------------------------------------------------------------------
// rows of the complex (two-harmonic) layout are (2*base + h); the element
// table holds the harmonic-0 number 2*base of each local DOF
// rows >= lim are not built from their own adjacency (copies of row
// r - k lim, see rep below)
__global__ void k_adj_count(const int *__restrict__ edofs, long long total,
                            int shift, int lim, int *__restrict__ cnt)
{
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= total) return;
  int d = edofs[t];
  if(d >= 0 && d < lim) atomicAdd(&cnt[d >> shift], 1);
}

__global__ void k_adj_fill(const int *__restrict__ edofs, long long total,
                           int nloc, int shift, int lim,
                           const long long *__restrict__ ptr,
                           int *__restrict__ cursor, int *__restrict__ adj)
{
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= total) return;
  int d = edofs[t];
  if(d < 0 || d >= lim) return;
  int b = d >> shift;
  int pos = atomicAdd(&cursor[b], 1);
  adj[ptr[b] + pos] = (int)(t / nloc);
}

constexpr int kPatThreads = 128;
constexpr int kPatCap = 4096;

// one block per row: gather the columns of every element touching the row,
// sort, count (mode 0) or write (mode 1) the distinct ones; with rep > 1
// the n rows built are also those of rows r + k n (k < rep), which have the
// same elements (the components of a vector field's node)
template <int WRITE>
__global__ void __launch_bounds__(kPatThreads)
k_pattern_rows(int n, int rep, int nloc, int complex_mode, const int *__restrict__ edofs,
               const unsigned char *__restrict__ cflag,
               const long long *__restrict__ adj_ptr,
               const int *__restrict__ adj, int *__restrict__ row_cnt,
               const long long *__restrict__ rowptr, int *__restrict__ col,
               int *__restrict__ err)
{
  __shared__ int s[kPatCap];
  __shared__ int wsum[kPatThreads / 32];
  int r = blockIdx.x;
  if(r >= n) return;
  int shift = complex_mode ? 1 : 0;
  int h = complex_mode ? (r & 1) : 0;
  int base = r >> shift;
  long long a0 = adj_ptr[base], a1 = adj_ptr[base + 1];
  int per = complex_mode ? 2 * nloc : nloc;
  long long total = (a1 - a0) * per;
  if(total > kPatCap) {
    if(threadIdx.x == 0) {
      atomicMax(err, (int)total);
      if(!WRITE)
        for(int k = 0; k < rep; k++) row_cnt[r + (long long)k * n] = 0;
    }
    return;
  }
  int P = next_pow2((int)total < 2 ? 2 : (int)total);
  for(int t = threadIdx.x; t < P; t += blockDim.x) {
    int v = 0x7fffffff;
    if(t < total) {
      int a = t / per, k = t % per;
      int e = adj[a0 + a];
      if(!complex_mode) {
        int c = edofs[(long long)e * nloc + k];
        if(c >= 0) v = c;
      }
      else {
        int kk = k >> 1, second = k & 1;
        int c = edofs[(long long)e * nloc + kk];
        if(c >= 0) {
          if(!second)
            v = c + h;  // real block: (r, c + h)
          else if(cflag && cflag[e])
            v = c + (1 - h);  // imaginary coupling
        }
      }
    }
    s[t] = v;
  }
  __syncthreads();
  smem_bitonic_sort(s, P);
  // distinct flags, then a block prefix sum to place them
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int running = 0;
  for(int base_t = 0; base_t < P; base_t += blockDim.x) {
    int t = base_t + threadIdx.x;
    int f = 0;
    if(t < P) {
      int v = s[t];
      f = (v != 0x7fffffff) && (t == 0 || s[t - 1] != v);
    }
    unsigned m = __ballot_sync(0xffffffffu, f);
    int wpre = __popc(m & ((1u << lane) - 1));
    if(lane == 0) wsum[w] = __popc(m);
    __syncthreads();
    int off = running;
    for(int q = 0; q < w; q++) off += wsum[q];
    if(WRITE && f)
      for(int k = 0; k < rep; k++) col[rowptr[r + (long long)k * n] + off + wpre] = s[t];
    int chunk = 0;
    for(int q = 0; q < kPatThreads / 32; q++) chunk += wsum[q];
    running += chunk;
    __syncthreads();
  }
  if(!WRITE && threadIdx.x == 0)
    for(int k = 0; k < rep; k++) row_cnt[r + (long long)k * n] = running;
}

int build_pattern_from_elements(gb300_matrix *A, int ne, int nloc,
                                const int *d_edofs,
                                const unsigned char *d_cflag, int complex_mode,
                                int rep)
{
  cudaStream_t st = A->ctx->stream;
  int n = A->n;
  if(rep < 1 || n % rep || complex_mode) rep = 1;
  const int nb = n / rep;  // rows built; the others are copies
  int shift = complex_mode ? 1 : 0;
  int nbase = complex_mode ? n / 2 : nb;
  long long total = (long long)ne * nloc;
  DevBuf<int> cnt, cursor, adj, err;
  DevBuf<long long> adj_ptr, tmp, rp64;
  GB_TRY(cnt.alloc(nbase + 1));
  GB_TRY(cursor.alloc(nbase + 1));
  GB_TRY(adj_ptr.alloc(nbase + 1));
  GB_TRY(err.alloc(1));
  GB_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * (nbase + 1), st));
  GB_CUDA(cudaMemsetAsync(cursor.p, 0, sizeof(int) * (nbase + 1), st));
  GB_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  k_adj_count<<<grid_for(total, 256), 256, 0, st>>>(d_edofs, total, shift,
                                                     rep > 1 ? nb : n, cnt.p);
  long long nadj = 0;
  GB_TRY(exclusive_scan(cnt.p, nbase + 1, adj_ptr.p, &nadj, tmp, st));
  GB_CUDA(cudaStreamSynchronize(st));
  GB_TRY(adj.alloc(nadj > 0 ? nadj : 1));
  k_adj_fill<<<grid_for(total, 256), 256, 0, st>>>(d_edofs, total, nloc, shift,
                                                    rep > 1 ? nb : n, adj_ptr.p,
                                                    cursor.p, adj.p);
  // count pass
  DevBuf<int> row_cnt;
  GB_TRY(row_cnt.alloc(n + 1));
  GB_CUDA(cudaMemsetAsync(row_cnt.p + n, 0, sizeof(int), st));
  k_pattern_rows<0><<<nb, kPatThreads, 0, st>>>(nb, rep, nloc, complex_mode, d_edofs,
                                                d_cflag, adj_ptr.p, adj.p,
                                                row_cnt.p, nullptr, nullptr,
                                                err.p);
  GB_TRY(rp64.alloc(n + 1));
  long long nnz = 0;
  GB_TRY(exclusive_scan(row_cnt.p, n + 1, rp64.p, &nnz, tmp, st));
  int herr = 0;
  GB_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(herr) {
    set_error("pattern: a row gathers %d candidate columns (capacity %d)", herr,
              kPatCap);
    return GB300_ERR_CAPACITY;
  }
  if(nnz >= (1LL << 31)) {
    set_error("pattern: %lld nonzeros exceed 32-bit CSR indexing", nnz);
    return GB300_ERR_CAPACITY;
  }
  GB_TRY(A->rowptr.alloc(n + 1));
  GB_TRY(A->col.alloc(nnz > 0 ? nnz : 1));
  GB_TRY(A->val.alloc(nnz > 0 ? nnz : 1));
  k_i64_to_i32<<<grid_for(n + 1, 256), 256, 0, st>>>(rp64.p, n + 1, A->rowptr.p);
  k_pattern_rows<1><<<nb, kPatThreads, 0, st>>>(nb, rep, nloc, complex_mode, d_edofs,
                                                d_cflag, adj_ptr.p, adj.p,
                                                nullptr, rp64.p, A->col.p, err.p);
  GB_CUDA(cudaMemsetAsync(A->val.p, 0, sizeof(double) * (nnz > 0 ? nnz : 1), st));
  GB_CUDA(cudaGetLastError());
  A->nnz = nnz;
  A->csr_valid = true;
  A->pattern_version++;
  A->val32_valid = false;
  gb::coarse_values_changed(A);
  A->block3 = false;
  A->node_blocks = false;
  A->bsr_var32 = A->bsr_var64 = -1;
  choose_tpr(A);
  GB_CUDA(cudaStreamSynchronize(st));
  return GB300_OK;
}

// ---------------------------------------------------------------------------
// COO (call order) -> CSR, duplicates summed in call order
// ---------------------------------------------------------------------------
__global__ void k_coo_count(const int *__restrict__ r, long long m, int n,
                            int *__restrict__ cnt, int *__restrict__ err)
{
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= m) return;
  int i = r[t];
  if(i < 0 || i >= n) {
    atomicExch(err, 1);
    return;
  }
  atomicAdd(&cnt[i], 1);
}

__global__ void k_coo_fill(const int *__restrict__ r, const int *__restrict__ c,
                           long long m, int n, const long long *__restrict__ ptr,
                           int *__restrict__ cursor,
                           unsigned long long *__restrict__ keys,
                           int *__restrict__ err)
{
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= m) return;
  int i = r[t], j = c[t];
  if(i < 0 || i >= n || j < 0 || j >= n) {
    atomicExch(err, 1);
    return;
  }
  int pos = atomicAdd(&cursor[i], 1);
  keys[ptr[i] + pos] = ((unsigned long long)(unsigned)j << 32) |
                       (unsigned long long)(t & 0xffffffffULL);
}

constexpr int kCooCap = 4096;

template <int WRITE>
__global__ void __launch_bounds__(kPatThreads)
k_coo_rows(int n, const long long *__restrict__ ptr,
           const unsigned long long *__restrict__ keys,
           const double *__restrict__ v, int *__restrict__ row_cnt,
           const long long *__restrict__ rowptr, int *__restrict__ col,
           double *__restrict__ val, int *__restrict__ err)
{
  __shared__ unsigned long long s[kCooCap];
  __shared__ int wsum[kPatThreads / 32];
  int r = blockIdx.x;
  if(r >= n) return;
  long long a0 = ptr[r], a1 = ptr[r + 1];
  int total = (int)(a1 - a0);
  if(a1 - a0 > kCooCap) {
    if(threadIdx.x == 0) {
      atomicMax(err, total);
      if(!WRITE) row_cnt[r] = 0;
    }
    return;
  }
  int P = next_pow2(total < 2 ? 2 : total);
  for(int t = threadIdx.x; t < P; t += blockDim.x)
    s[t] = (t < total) ? keys[a0 + t] : ~0ULL;
  __syncthreads();
  smem_bitonic_sort(s, P);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int running = 0;
  for(int base_t = 0; base_t < P; base_t += blockDim.x) {
    int t = base_t + threadIdx.x;
    int f = 0;
    if(t < total) f = (t == 0) || ((s[t - 1] >> 32) != (s[t] >> 32));
    unsigned m = __ballot_sync(0xffffffffu, f);
    int wpre = __popc(m & ((1u << lane) - 1));
    if(lane == 0) wsum[w] = __popc(m);
    __syncthreads();
    int off = running;
    for(int q = 0; q < w; q++) off += wsum[q];
    if(WRITE && f) {
      // sum the group in call order (keys sorted by (col, call index))
      unsigned cj = (unsigned)(s[t] >> 32);
      double acc = v[s[t] & 0xffffffffULL];
      for(int u = t + 1; u < total && (unsigned)(s[u] >> 32) == cj; u++)
        acc += v[s[u] & 0xffffffffULL];
      long long o = rowptr[r] + off + wpre;
      col[o] = (int)cj;
      val[o] = acc;
    }
    int chunk = 0;
    for(int q = 0; q < kPatThreads / 32; q++) chunk += wsum[q];
    running += chunk;
    __syncthreads();
  }
  if(!WRITE && threadIdx.x == 0) row_cnt[r] = running;
}

int build_csr_from_coo(gb300_matrix *A, long long m, const int *d_r,
                       const int *d_c, const double *d_v)
{
  cudaStream_t st = A->ctx->stream;
  int n = A->n;
  if(m >= (1LL << 32)) {
    set_error("too many staged entries (%lld)", m);
    return GB300_ERR_CAPACITY;
  }
  DevBuf<int> cnt, cursor, err, row_cnt;
  DevBuf<long long> ptr, tmp, rp64;
  DevBuf<unsigned long long> keys;
  GB_TRY(cnt.alloc(n + 1));
  GB_TRY(cursor.alloc(n + 1));
  GB_TRY(err.alloc(1));
  GB_TRY(ptr.alloc(n + 1));
  GB_TRY(keys.alloc(m > 0 ? m : 1));
  GB_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * (n + 1), st));
  GB_CUDA(cudaMemsetAsync(cursor.p, 0, sizeof(int) * (n + 1), st));
  GB_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  if(m > 0)
    k_coo_count<<<grid_for(m, 256), 256, 0, st>>>(d_r, m, n, cnt.p, err.p);
  GB_TRY(exclusive_scan(cnt.p, n + 1, ptr.p, nullptr, tmp, st));
  if(m > 0)
    k_coo_fill<<<grid_for(m, 256), 256, 0, st>>>(d_r, d_c, m, n, ptr.p,
                                                  cursor.p, keys.p, err.p);
  int herr = 0;
  GB_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(herr) {
    set_error("matrix entry index out of range [0, %d)", n);
    return GB300_ERR_ARG;
  }
  GB_TRY(row_cnt.alloc(n + 1));
  GB_CUDA(cudaMemsetAsync(row_cnt.p + n, 0, sizeof(int), st));
  k_coo_rows<0><<<n, kPatThreads, 0, st>>>(n, ptr.p, keys.p, d_v, row_cnt.p,
                                            nullptr, nullptr, nullptr, err.p);
  GB_TRY(rp64.alloc(n + 1));
  long long nnz = 0;
  GB_TRY(exclusive_scan(row_cnt.p, n + 1, rp64.p, &nnz, tmp, st));
  GB_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(herr) {
    set_error("a matrix row holds %d staged entries (capacity %d)", herr,
              kCooCap);
    return GB300_ERR_CAPACITY;
  }
  GB_TRY(A->rowptr.alloc(n + 1));
  GB_TRY(A->col.alloc(nnz > 0 ? nnz : 1));
  GB_TRY(A->val.alloc(nnz > 0 ? nnz : 1));
  k_i64_to_i32<<<grid_for(n + 1, 256), 256, 0, st>>>(rp64.p, n + 1, A->rowptr.p);
  k_coo_rows<1><<<n, kPatThreads, 0, st>>>(n, ptr.p, keys.p, d_v, nullptr,
                                            rp64.p, A->col.p, A->val.p, err.p);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(st));
  A->nnz = nnz;
  A->csr_valid = true;
  A->pattern_version++;
  A->val32_valid = false;
  gb::coarse_values_changed(A);
  A->block3 = false;
  A->node_blocks = false;
  A->bsr_var32 = A->bsr_var64 = -1;
  choose_tpr(A);
  return GB300_OK;
}

void choose_tpr(gb300_matrix *A)
{
  double avg = A->n ? (double)A->nnz / A->n : 0.0;
  // few lanes per row: GB300's FP64 pipe (about two FMAs per SM per clock)
  // makes the lanes left idle on a short row, and the shuffle-add tree of
  // the row sum, cost more than the row's memory traffic
  A->tpr = avg > 128 ? 32 : avg > 64 ? 16 : avg > 32 ? 8 : avg > 16 ? 4 : 2;
}

// ---------------------------------------------------------------------------
// SpMV family.  MODE 0: y = A x.  MODE 1: y = b - A x, partial ||y||^2.
// MODE 2: y = A x, partial <p, y> with p = x (CG: q = A p, <p, q>).
// Rows are distributed grid-stride over a fixed grid so that the partial
// sums (one per block) are formed in a fixed order.
// ---------------------------------------------------------------------------
template <int TPR, int MODE, typename V, typename XT>
__global__ void __launch_bounds__(256)
k_spmv(int n, const int *__restrict__ rowptr, const int *__restrict__ col,
       const V *__restrict__ val, const XT *__restrict__ x,
       const XT *__restrict__ b, XT *__restrict__ y, double *__restrict__ part,
       const int *flag)
{
  if(flag && !*flag) return;
  using ACC = XT;
  const int rows_per_block = 256 / TPR;
  int lane = threadIdx.x % TPR;
  int sub = threadIdx.x / TPR;
  typename Acc<XT>::type red = 0;
  for(long long rb = (long long)blockIdx.x * rows_per_block; rb < n;
      rb += (long long)gridDim.x * rows_per_block) {
    long long row = rb + sub;
    ACC sum = 0;
    if(row < n) {
      int s = rowptr[row], e = rowptr[row + 1];
      sum = csr_row_dot<TPR, (TPR >= 16 ? 4 : 2), ACC>(s, e, lane, col, val, x);
    }
#pragma unroll
    for(int o = TPR / 2; o > 0; o >>= 1)
      sum += __shfl_down_sync(0xffffffffu, sum, o, TPR);
    if(lane == 0 && row < n) {
      if(MODE == 1) {
        ACC r = b[row] - sum;
        y[row] = r;
        red += r * r;
      }
      else if(MODE == 3)  // y += A x
        y[row] += sum;
      else if(MODE == 4)  // y = b - A x, no partial sums
        y[row] = b[row] - sum;
      else {
        y[row] = sum;
        if(MODE == 2) red += x[row] * sum;
      }
    }
  }
  if(MODE == 1 || MODE == 2) {
    double s = block_sum<double, 256>((double)red);
    if(threadIdx.x == 0) part[blockIdx.x] = s;
  }
}

template <int MODE, typename V, typename XT>
static void launch_spmv(const gb300_matrix *A, const V *val, const XT *x,
                        const XT *b, XT *y, double *part, cudaStream_t st,
                        const int *flag = nullptr)
{
  int n = A->n;
  int rows_per_block_64 = 256 / A->tpr;
  // modes with partial sums (1, 2) run on the fixed reduction grid
  constexpr bool kFree = (MODE == 0 || MODE == 3 || MODE == 4);
  int blocks = kFree ? grid_for(n, rows_per_block_64, 1 << 30) : kReduceBlocks;
  if(kFree && blocks > 152 * 64) blocks = 152 * 64;
  switch(A->tpr) {
  case 2:
    k_spmv<2, MODE><<<blocks, 256, 0, st>>>(n, A->rowptr.p, A->col.p, val, x, b, y, part, flag);
    break;
  case 4:
    k_spmv<4, MODE><<<blocks, 256, 0, st>>>(n, A->rowptr.p, A->col.p, val, x, b, y, part, flag);
    break;
  case 8:
    k_spmv<8, MODE><<<blocks, 256, 0, st>>>(n, A->rowptr.p, A->col.p, val, x, b, y, part, flag);
    break;
  case 16:
    k_spmv<16, MODE><<<blocks, 256, 0, st>>>(n, A->rowptr.p, A->col.p, val, x, b, y, part, flag);
    break;
  default:
    k_spmv<32, MODE><<<blocks, 256, 0, st>>>(n, A->rowptr.p, A->col.p, val, x, b, y, part, flag);
    break;
  }
}

void spmv64(const gb300_matrix *A, const double *x, double *y, cudaStream_t st)
{
  launch_spmv<0, double, double>(A, A->val.p, x, nullptr, y, nullptr, st);
}
void residual64(const gb300_matrix *A, const double *val, const double *x,
                const double *b, double *r, double *part, cudaStream_t st)
{
  launch_spmv<1, double, double>(A, val, x, b, r, part, st);
}
void residual64_guarded(const gb300_matrix *A, const double *val,
                        const double *x, const double *b, double *r,
                        double *part, const int *flag, cudaStream_t st)
{
  launch_spmv<1, double, double>(A, val, x, b, r, part, st, flag);
}
void spmv_dot64(const gb300_matrix *A, const double *val, const double *p,
                double *q, double *part, cudaStream_t st)
{
  launch_spmv<2, double, double>(A, val, p, nullptr, q, part, st);
}
void spmv_dot32(const gb300_matrix *A, const float *val, const float *p,
                float *q, double *part, cudaStream_t st)
{
  launch_spmv<2, float, float>(A, val, p, nullptr, q, part, st);
}
void spmv_plain(const gb300_matrix *A, const double *val, const double *x,
                double *y, cudaStream_t st)
{
  launch_spmv<0, double, double>(A, val, x, nullptr, y, nullptr, st);
}
void spmv_guarded(const gb300_matrix *A, const double *val, const double *x,
                  double *y, const int *flag, cudaStream_t st)
{
  launch_spmv<0, double, double>(A, val, x, nullptr, y, nullptr, st, flag);
}
void spmv_add_guarded(const gb300_matrix *A, const double *val, const double *x,
                      double *y, const int *flag, cudaStream_t st)
{
  launch_spmv<3, double, double>(A, val, x, nullptr, y, nullptr, st, flag);
}
void resid_guarded(const gb300_matrix *A, const double *val, const double *x,
                   const double *b, double *r, const int *flag, cudaStream_t st)
{
  launch_spmv<4, double, double>(A, val, x, b, r, nullptr, st, flag);
}

// sum of the fixed-size partial array, in a fixed order, into *out
__global__ void k_sum_partials(const double *__restrict__ part, int np,
                               double *__restrict__ out)
{
  double v = 0.0;
  for(int i = threadIdx.x; i < np; i += blockDim.x) v += part[i];
  double s = block_sum<double, 256>(v);
  if(threadIdx.x == 0) *out = s;
}

void sum_partials(const double *part, double *out, cudaStream_t st)
{
  k_sum_partials<<<1, 256, 0, st>>>(part, kReduceBlocks, out);
}

// partial sums of <x, y> over a fixed grid
template <typename T>
__global__ void k_dot_part(int n, const T *__restrict__ x,
                           const T *__restrict__ y, double *__restrict__ part)
{
  typename Acc<T>::type v = 0;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (long long)gridDim.x * blockDim.x)
    v += x[i] * y[i];
  double s = block_sum<double, 256>((double)v);
  if(threadIdx.x == 0) part[blockIdx.x] = s;
}

void dot_part64(int n, const double *x, const double *y, double *part,
                cudaStream_t st)
{
  k_dot_part<double><<<kReduceBlocks, 256, 0, st>>>(n, x, y, part);
}
void dot_part32(int n, const float *x, const float *y, double *part,
                cudaStream_t st)
{
  k_dot_part<float><<<kReduceBlocks, 256, 0, st>>>(n, x, y, part);
}

}  // namespace gb
