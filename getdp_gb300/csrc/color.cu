// Multicolour ordering for the ILU(0) preconditioner.
//
// Sparskit reorders the system before its ILU(0) with reverse Cuthill-McKee
// (Renumbering_Technique 1, Sparskit.cpp:255-300): on a CPU that shortens
// the profile and improves locality.  On a GPU the same ordering makes the
// triangular solves nearly sequential (a row depends on the row before it),
// and even GetDP's own DOF order leaves about 2n dependency levels on an
// n x n grid.  This backend's renumbering is a multicolour ordering instead:
// rows of one colour share no matrix entry, so after a symmetric
// permutation by colour the ILU(0) factorisation and both triangular
// sweeps have one dependency level per colour, each a fully parallel pass.
// As with RCMK, the preconditioner (and so the iteration count) depends on
// the ordering; the solution is the solution of the same system.
//
// Colouring: Jones-Plassmann rounds.  An uncoloured row whose hash is the
// largest among its uncoloured neighbours takes the smallest colour none
// of its coloured neighbours has.  Rows coloured in the same round are
// never neighbours, and a stale read of a neighbour's colour can only
// prevent a row from taking a colour this round, so no round races.  Each
// round colours at least the uncoloured row of largest hash: at most n
// rounds.  The order within a colour is the original order (stable), so the
// permutation, and every result computed with it, is deterministic.
#include "krylov.cuh"

namespace gb {

__device__ __forceinline__ unsigned row_hash(unsigned x)
{
  // 32-bit integer mix: C. Wellons' "lowbias32" (hash-prospector, public
  // domain), xor-shift / multiply rounds
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ bool beats(unsigned hj, int j, unsigned hi, int i)
{
  return hj > hi || (hj == hi && j > i);
}

// one round; *left counts the rows still uncoloured afterwards
__global__ void k_jp_round(int n, const int *__restrict__ rowptr,
                           const int *__restrict__ col, int *color,
                           int *__restrict__ left, int *__restrict__ too_many)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n || color[i] >= 0) return;
  const unsigned hi = row_hash((unsigned)i);
  const int s = rowptr[i], e = rowptr[i + 1];
  for(int k = s; k < e; k++) {
    int j = col[k];
    if(j == i) continue;
    if(color[j] < 0 && beats(row_hash((unsigned)j), j, hi, i)) {
      atomicAdd(left, 1);
      return;
    }
  }
  // smallest colour unused by the coloured neighbours, 64 colours a window
  for(int base = 0; base < 1024; base += 64) {
    unsigned long long used = 0ull;
    for(int k = s; k < e; k++) {
      int j = col[k];
      if(j == i) continue;
      int c = color[j] - base;
      if(c >= 0 && c < 64) used |= 1ull << c;
    }
    if(~used) {
      color[i] = base + __ffsll((long long)~used) - 1;
      return;
    }
  }
  atomicExch(too_many, 1);
  color[i] = 1023;  // never reached for a pattern of fewer than 1024 per row
}

__global__ void k_colour_flag(int n, const int *__restrict__ color, int c,
                              int *__restrict__ flag)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) flag[i] = (color[i] == c);
}

__global__ void k_colour_place(int n, const int *__restrict__ color, int c,
                               const long long *__restrict__ pos, long long base,
                               int *__restrict__ new_of, int *__restrict__ old_of)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n || color[i] != c) return;
  int ni = (int)(base + pos[i]);
  new_of[i] = ni;
  old_of[ni] = i;
}

__global__ void k_perm_len(int n, const int *__restrict__ rowptr,
                           const int *__restrict__ old_of, int *__restrict__ len)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) len[i] = rowptr[old_of[i] + 1] - rowptr[old_of[i]];
  if(i == n) len[n] = 0;
}

// one warp per new row: entries of the old row with columns renumbered,
// sorted by the new column (bitonic network in shared memory)
constexpr int kPermWarps = 4;
constexpr int kPermCap = 256;

__global__ void __launch_bounds__(32 * kPermWarps)
k_perm_rows(int n, const int *__restrict__ rowptr, const int *__restrict__ col,
            const int *__restrict__ new_of, const int *__restrict__ old_of,
            const long long *__restrict__ browptr, int *__restrict__ bcol,
            int *__restrict__ src, int *__restrict__ too_long)
{
  __shared__ int key[kPermWarps][kPermCap];
  __shared__ int idx[kPermWarps][kPermCap];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int i = blockIdx.x * kPermWarps + w;
  if(i >= n) return;  // warp-uniform
  int o = old_of[i];
  int s = rowptr[o], len = rowptr[o + 1] - s;
  if(len > kPermCap) {
    if(lane == 0) atomicExch(too_long, 1);
    return;
  }
  int P = 1;
  while(P < len) P <<= 1;
  for(int t = lane; t < P; t += 32) {
    key[w][t] = t < len ? new_of[col[s + t]] : 0x7fffffff;
    idx[w][t] = t < len ? s + t : -1;
  }
  __syncwarp();
  for(int k = 2; k <= P; k <<= 1)
    for(int j = k >> 1; j > 0; j >>= 1) {
      for(int t = lane; t < P; t += 32) {
        int l = t ^ j;
        if(l > t) {
          bool up = ((t & k) == 0);
          int a = key[w][t], b = key[w][l];
          if((a > b) == up) {
            key[w][t] = b;
            key[w][l] = a;
            int ia = idx[w][t];
            idx[w][t] = idx[w][l];
            idx[w][l] = ia;
          }
        }
      }
      __syncwarp();
    }
  long long d = browptr[i];
  for(int t = lane; t < len; t += 32) {
    bcol[d + t] = key[w][t];
    src[d + t] = idx[w][t];
  }
}

__global__ void k_i64_to_i32_rows(const long long *__restrict__ in, int n,
                                  int *__restrict__ out)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) out[i] = (int)in[i];
}

__global__ void k_gather_vals(long long nnz, const int *__restrict__ src,
                              const double *__restrict__ in, double *__restrict__ out)
{
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(k < nnz) out[k] = in[src[k]];
}

__global__ void k_gather_rows(int n, const int *__restrict__ old_of,
                              const double *__restrict__ in, double *__restrict__ out)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) out[i] = in[old_of[i]];
}

__global__ void k_scatter_rows(int n, const int *__restrict__ old_of,
                               const double *__restrict__ in, double *__restrict__ out)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) out[old_of[i]] = in[i];
}

void colour_free(Colouring *c)
{
  if(!c) return;
  if(c->B) {
    if(c->B->ilu) ilu_free(c->B->ilu);
    delete c->B;
  }
  delete c;
}

// builds (or reuses) the multicolour ordering of A's pattern and the
// permuted matrix structure; GB300_ERR_UNSUPPORTED when the pattern does
// not allow it (the caller then keeps GetDP's order)
static int colour_build(gb300_matrix *A)
{
  if(A->mc && A->mc->version == A->pattern_version && A->mc->n == A->n)
    return GB300_OK;
  colour_free(A->mc);
  A->mc = nullptr;
  cudaStream_t st = A->ctx->stream;
  const int n = A->n;
  Colouring *C = new Colouring();
  C->n = n;
  C->version = A->pattern_version;
  auto fail = [&](int rc) {
    colour_free(C);
    return rc;
  };
  DevBuf<int> color, left, flag, len, err;
  DevBuf<long long> pos, tmp, brp;
  if(color.alloc(n) || left.alloc(1) || err.alloc(1) || flag.alloc(n + 1) ||
     pos.alloc(n + 1) || C->new_of.alloc(n) || C->old_of.alloc(n))
    return fail(GB300_ERR_CUDA);
  if(cudaMemsetAsync(color.p, 0xff, sizeof(int) * n, st) != cudaSuccess ||
     cudaMemsetAsync(err.p, 0, sizeof(int), st) != cudaSuccess)
    return fail(GB300_ERR_CUDA);
  int remaining = n, rounds = 0;
  while(remaining > 0 && rounds <= n) {
    if(cudaMemsetAsync(left.p, 0, sizeof(int), st) != cudaSuccess) return fail(GB300_ERR_CUDA);
    k_jp_round<<<grid_for(n, 256), 256, 0, st>>>(n, A->rowptr.p, A->col.p, color.p,
                                                  left.p, err.p);
    if(cudaMemcpyAsync(&remaining, left.p, sizeof(int), cudaMemcpyDeviceToHost, st) !=
         cudaSuccess ||
       cudaStreamSynchronize(st) != cudaSuccess)
      return fail(GB300_ERR_CUDA);
    rounds++;
  }
  int herr = 0;
  if(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
     cudaStreamSynchronize(st) != cudaSuccess)
    return fail(GB300_ERR_CUDA);
  if(remaining > 0 || herr) return fail(GB300_ERR_UNSUPPORTED);
  // number of colours
  {
    std::vector<int> hc(n);
    if(cudaMemcpyAsync(hc.data(), color.p, sizeof(int) * n, cudaMemcpyDeviceToHost, st) !=
         cudaSuccess ||
       cudaStreamSynchronize(st) != cudaSuccess)
      return fail(GB300_ERR_CUDA);
    int mx = -1;
    for(int v : hc) mx = v > mx ? v : mx;
    C->ncolors = mx + 1;
  }
  // stable placement, colour by colour
  long long base = 0;
  for(int c = 0; c < C->ncolors; c++) {
    k_colour_flag<<<grid_for(n, 256), 256, 0, st>>>(n, color.p, c, flag.p);
    long long cnt = 0;
    int rc = exclusive_scan(flag.p, n, pos.p, &cnt, tmp, st);
    if(rc != GB300_OK) return fail(rc);
    k_colour_place<<<grid_for(n, 256), 256, 0, st>>>(n, color.p, c, pos.p, base,
                                                      C->new_of.p, C->old_of.p);
    base += cnt;
  }
  if(base != n) return fail(GB300_ERR_UNSUPPORTED);
  // the permuted structure
  gb300_matrix *B = new gb300_matrix();
  C->B = B;
  B->ctx = A->ctx;
  B->n = n;
  B->nnz = A->nnz;
  if(len.alloc(n + 1) || brp.alloc(n + 1) || B->rowptr.alloc(n + 1) ||
     B->col.alloc(A->nnz > 0 ? A->nnz : 1) || B->val.alloc(A->nnz > 0 ? A->nnz : 1) ||
     C->src.alloc(A->nnz > 0 ? A->nnz : 1))
    return fail(GB300_ERR_CUDA);
  k_perm_len<<<grid_for(n + 1, 256), 256, 0, st>>>(n, A->rowptr.p, C->old_of.p, len.p);
  long long total = 0;
  int rc = exclusive_scan(len.p, n + 1, brp.p, &total, tmp, st);
  if(rc != GB300_OK) return fail(rc);
  if(total != A->nnz) return fail(GB300_ERR_UNSUPPORTED);
  k_i64_to_i32_rows<<<grid_for(n + 1, 256), 256, 0, st>>>(brp.p, n + 1, B->rowptr.p);
  if(cudaMemsetAsync(err.p, 0, sizeof(int), st) != cudaSuccess) return fail(GB300_ERR_CUDA);
  k_perm_rows<<<grid_for(n, kPermWarps), 32 * kPermWarps, 0, st>>>(
    n, A->rowptr.p, A->col.p, C->new_of.p, C->old_of.p, brp.p, B->col.p, C->src.p, err.p);
  if(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
     cudaStreamSynchronize(st) != cudaSuccess)
    return fail(GB300_ERR_CUDA);
  if(herr) return fail(GB300_ERR_UNSUPPORTED);
  B->csr_valid = true;
  choose_tpr(B);
  A->mc = C;
  return GB300_OK;
}

// the Krylov solve of A x = rhs (values val) on the multicolour-permuted
// system; *used = false when the ordering is not available (nothing done)
int gmres_solve_coloured(gb300_matrix *A, const double *val, const double *rhs,
                         double *x, const gb300_solver_params *p,
                         gb300_solve_info *info, Work &W, bool *used)
{
  *used = false;
  int rc = colour_build(A);
  if(rc == GB300_ERR_UNSUPPORTED) return GB300_OK;
  if(rc != GB300_OK) return rc;
  *used = true;
  Colouring *C = A->mc;
  gb300_matrix *B = C->B;
  cudaStream_t st = A->ctx->stream;
  const int n = A->n;
  DevBuf<double> rb, yb;
  GB_TRY(rb.alloc(n));
  GB_TRY(yb.alloc(n));
  k_gather_vals<<<grid_for(A->nnz, 256), 256, 0, st>>>(A->nnz, C->src.p, val, B->val.p);
  k_gather_rows<<<grid_for(n, 256), 256, 0, st>>>(n, C->old_of.p, rhs, rb.p);
  GB_CUDA(cudaGetLastError());
  rc = gmres_solve(B, B->val.p, rb.p, yb.p, p, info, W);
  if(rc != GB300_OK) return rc;
  k_scatter_rows<<<grid_for(n, 256), 256, 0, st>>>(n, C->old_of.p, yb.p, x);
  GB_CUDA(cudaGetLastError());
  return GB300_OK;
}

}  // namespace gb
