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
// A complex system (two real rows per unknown, harmonic-interleaved) is
// coloured by unknown: the two rows of an unknown keep adjacent places and
// one colour, so the 2 x 2 coupling j*omega*sigma stays inside the ILU's
// diagonal blocks (colouring the real rows apart left the high-frequency
// eddy-current systems without convergence in 3000 GMRES steps, against
// ~100 steps this way).
//
// Colouring: Jones-Plassmann rounds with the reverse of the original order
// as priority.  An uncoloured row whose uncoloured neighbours all come
// before it takes the smallest colour none of its coloured neighbours has.
// A row is coloured once every neighbour after it is, and then sees all of
// their colours, so the result is the sequential first-fit colouring from
// the last row to the first (whatever a round reads of a neighbour coloured
// in the same round), and rows coloured in one round are never neighbours.
// Each round colours at least the last uncoloured row: at most n rounds; on
// a mesh numbered GetDP's way it takes about as many rounds as the ILU(0)
// has levels in the original order (~2n on an n x n grid), launched 32 at a
// time.  Measured with the oracle's ILU(0)-(F)GMRES on the permuted systems
// (steps, colours), against hash priorities and the first-to-last order:
// 2D P1 magnetostatics 128^2 (1e-10): 287, 4 | 314, 7 | 278, 4;
// 3D edge curl-curl 6^3 (1e-8): 732, 8 | 1265, 11 | 902, 8; the kappa ~ 3e11
// edge system of 4^3 (1e-10): 369 | 328 | no convergence in 5000 steps.
// Fewer colours also mean fewer launches per triangular solve.  The order
// within a colour is the original order (stable), so the permutation, and
// every result computed with it, is deterministic.  For a
// batch of independent systems (diagonal blocks) the rows are reordered
// within each block only, so every block keeps its row range.
#include "krylov.cuh"

namespace gb {

// one round over vertices (groups of bs consecutive rows); with left
// non-null, *left counts the vertices still uncoloured after this round
__global__ void k_jp_round(int nv, int bs, const int *__restrict__ rowptr,
                           const int *__restrict__ col, int *color,
                           int *__restrict__ left, int *__restrict__ too_many)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= nv || color[i] >= 0) return;
  const int s = rowptr[i * bs], e = rowptr[i * bs + bs];
  for(int k = s; k < e; k++) {
    int j = col[k] / bs;
    if(j > i && color[j] < 0) {  // an uncoloured row after this one
      if(left) atomicAdd(left, 1);
      return;
    }
  }
  // smallest colour unused by the coloured neighbours, 64 colours a window
  for(int base = 0; base < 1024; base += 64) {
    unsigned long long used = 0ull;
    for(int k = s; k < e; k++) {
      int j = col[k] / bs;
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

// block of each row (offsets of nseg diagonal blocks)
__global__ void k_row_block(int n, int nseg, const int *__restrict__ off,
                            int *__restrict__ blk)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n) return;
  int lo = 0, hi = nseg - 1;  // last block with off[b] <= i
  while(lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if(off[mid] <= i)
      lo = mid;
    else
      hi = mid - 1;
  }
  blk[i] = lo;
}

// rows of colour c: position = block start + rows of smaller colours in the
// block + rank among the block's colour-c rows (pos: exclusive scan of the
// colour-c flags over all rows)
__global__ void k_colour_place(int nv, int bs, const int *__restrict__ color, int c,
                               const long long *__restrict__ pos,
                               const int *__restrict__ off, const int *__restrict__ blk,
                               const long long *__restrict__ base,
                               int *__restrict__ new_of, int *__restrict__ old_of)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= nv || color[i] != c) return;
  int b = blk[i];
  int ni = (int)(off[b] + base[b] + (pos[i] - pos[off[b]]));
  for(int t = 0; t < bs; t++) {
    new_of[i * bs + t] = ni * bs + t;
    old_of[ni * bs + t] = i * bs + t;
  }
}

__global__ void k_colour_base(int nseg, const int *__restrict__ off,
                              const long long *__restrict__ pos, long long *base)
{
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if(b < nseg) base[b] += pos[off[b + 1]] - pos[off[b]];
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

void colour_drop_factor(gb300_matrix *A)
{
  if(A->mc && A->mc->B && A->mc->B->ilu) {
    ilu_free(A->mc->B->ilu);
    A->mc->B->ilu = nullptr;
  }
}

void colour_free(Colouring *c)
{
  if(!c) return;
  if(c->B) {
    if(c->B->ilu) ilu_free(c->B->ilu);
    coarse_free(c->B->coarse);
    delete c->B;
  }
  delete c;
}

// builds (or reuses) the multicolour ordering of A's pattern, within the
// diagonal blocks off[0..nseg] (nseg = 1: the whole matrix), by groups of
// A->block_rows rows, and the permuted matrix structure;
// GB300_ERR_UNSUPPORTED when the pattern does not allow it (the caller then
// keeps GetDP's order)
static int permuted_structure(gb300_matrix *A, Colouring *C, cudaStream_t st);

int colour_build(gb300_matrix *A, int nseg, const int *off)
{
  const int n = A->n;
  std::vector<int> seg(off, off + nseg + 1);
  int bs = A->block_rows > 1 ? A->block_rows : 1;
  for(int v : seg)
    if(v % bs) bs = 1;
  if(n % bs) bs = 1;
  if(A->mc && A->mc->kind == 0 && A->mc->version == A->pattern_version && A->mc->n == n &&
     A->mc->seg == seg && A->mc->bs == bs)
    return GB300_OK;
  colour_free(A->mc);
  A->mc = nullptr;
  cudaStream_t st = A->ctx->stream;
  Colouring *C = new Colouring();
  C->n = n;
  C->version = A->pattern_version;
  C->seg = seg;
  C->bs = bs;
  const int nv = n / bs;
  std::vector<int> vseg(seg.size());
  for(size_t q = 0; q < seg.size(); q++) vseg[q] = seg[q] / bs;
  auto fail = [&](int rc) {
    colour_free(C);
    return rc;
  };
  DevBuf<int> color, left, flag, len, err, doff, blk;
  DevBuf<long long> pos, tmp, brp, base;
  if(color.alloc(nv) || left.alloc(1) || err.alloc(1) || flag.alloc(nv + 1) ||
     pos.alloc(nv + 1) || C->new_of.alloc(n) || C->old_of.alloc(n) ||
     doff.alloc(nseg + 1) || blk.alloc(nv) || base.alloc(nseg))
    return fail(GB300_ERR_CUDA);
  if(cudaMemcpyAsync(doff.p, vseg.data(), sizeof(int) * (nseg + 1), cudaMemcpyHostToDevice,
                     st) != cudaSuccess ||
     cudaMemsetAsync(base.p, 0, sizeof(long long) * nseg, st) != cudaSuccess ||
     cudaMemsetAsync(flag.p + nv, 0, sizeof(int), st) != cudaSuccess)
    return fail(GB300_ERR_CUDA);
  k_row_block<<<grid_for(nv, 256), 256, 0, st>>>(nv, nseg, doff.p, blk.p);
  if(cudaMemsetAsync(color.p, 0xff, sizeof(int) * nv, st) != cudaSuccess ||
     cudaMemsetAsync(err.p, 0, sizeof(int), st) != cudaSuccess)
    return fail(GB300_ERR_CUDA);
  // rounds in groups of 32; the last of a group counts what is left
  constexpr int kGroup = 32;
  int remaining = nv, rounds = 0;
  while(remaining > 0 && rounds <= nv) {
    if(cudaMemsetAsync(left.p, 0, sizeof(int), st) != cudaSuccess) return fail(GB300_ERR_CUDA);
    for(int g = 0; g < kGroup; g++)
      k_jp_round<<<grid_for(nv, 256), 256, 0, st>>>(nv, bs, A->rowptr.p, A->col.p, color.p,
                                                     g == kGroup - 1 ? left.p : nullptr,
                                                     err.p);
    if(cudaMemcpyAsync(&remaining, left.p, sizeof(int), cudaMemcpyDeviceToHost, st) !=
         cudaSuccess ||
       cudaStreamSynchronize(st) != cudaSuccess)
      return fail(GB300_ERR_CUDA);
    rounds += kGroup;
  }
  int herr = 0;
  if(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
     cudaStreamSynchronize(st) != cudaSuccess)
    return fail(GB300_ERR_CUDA);
  if(remaining > 0 || herr) return fail(GB300_ERR_UNSUPPORTED);
  // number of colours
  {
    std::vector<int> hc(nv);
    if(cudaMemcpyAsync(hc.data(), color.p, sizeof(int) * nv, cudaMemcpyDeviceToHost, st) !=
         cudaSuccess ||
       cudaStreamSynchronize(st) != cudaSuccess)
      return fail(GB300_ERR_CUDA);
    int mx = -1;
    for(int v : hc) mx = v > mx ? v : mx;
    C->ncolors = mx + 1;
  }
  // stable placement, colour by colour, within each block; base[b] counts
  // the vertices of block b placed so far, so after colour c it closes the
  // block's colour-c range
  long long placed = 0;
  const int nc1 = C->ncolors + 1;
  C->voff.assign((size_t)nseg * nc1, 0);
  std::vector<long long> hbase(nseg);
  for(int b = 0; b < nseg; b++) C->voff[(size_t)b * nc1] = vseg[b];
  for(int c = 0; c < C->ncolors; c++) {
    k_colour_flag<<<grid_for(nv, 256), 256, 0, st>>>(nv, color.p, c, flag.p);
    long long cnt = 0;
    int rc = exclusive_scan(flag.p, nv + 1, pos.p, &cnt, tmp, st);
    if(rc != GB300_OK) return fail(rc);
    k_colour_place<<<grid_for(nv, 256), 256, 0, st>>>(nv, bs, color.p, c, pos.p, doff.p,
                                                       blk.p, base.p, C->new_of.p,
                                                       C->old_of.p);
    k_colour_base<<<grid_for(nseg, 256), 256, 0, st>>>(nseg, doff.p, pos.p, base.p);
    placed += cnt;
    if(cudaMemcpyAsync(hbase.data(), base.p, sizeof(long long) * nseg,
                       cudaMemcpyDeviceToHost, st) != cudaSuccess ||
       cudaStreamSynchronize(st) != cudaSuccess)
      return fail(GB300_ERR_CUDA);
    for(int b = 0; b < nseg; b++)
      C->voff[(size_t)b * nc1 + c + 1] = vseg[b] + (int)hbase[b];
  }
  if(placed != nv) return fail(GB300_ERR_UNSUPPORTED);
  const int rc_ = permuted_structure(A, C, st);
  if(rc_ != GB300_OK) return fail(rc_);
  A->mc = C;
  return GB300_OK;
}

// B = P A P^T for the row permutation C->new_of / C->old_of (rows sorted by
// the new column index, as Sparskit's sortcol leaves them), with C->src the
// position in A of each of B's entries; GB300_ERR_UNSUPPORTED when a row is
// longer than the sort's capacity
static int permuted_structure(gb300_matrix *A, Colouring *C, cudaStream_t st)
{
  const int n = A->n;
  DevBuf<int> len, err;
  DevBuf<long long> brp, tmp;
  gb300_matrix *B = new gb300_matrix();
  C->B = B;
  B->ctx = A->ctx;
  B->n = n;
  B->nnz = A->nnz;
  GB_TRY(len.alloc(n + 1));
  GB_TRY(err.alloc(1));
  GB_TRY(brp.alloc(n + 1));
  GB_TRY(B->rowptr.alloc(n + 1));
  GB_TRY(B->col.alloc(A->nnz > 0 ? A->nnz : 1));
  GB_TRY(B->val.alloc(A->nnz > 0 ? A->nnz : 1));
  GB_TRY(C->src.alloc(A->nnz > 0 ? A->nnz : 1));
  k_perm_len<<<grid_for(n + 1, 256), 256, 0, st>>>(n, A->rowptr.p, C->old_of.p, len.p);
  long long total = 0;
  GB_TRY(exclusive_scan(len.p, n + 1, brp.p, &total, tmp, st));
  if(total != A->nnz) return GB300_ERR_UNSUPPORTED;
  k_i64_to_i32_rows<<<grid_for(n + 1, 256), 256, 0, st>>>(brp.p, n + 1, B->rowptr.p);
  GB_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  k_perm_rows<<<grid_for(n, kPermWarps), 32 * kPermWarps, 0, st>>>(
    n, A->rowptr.p, A->col.p, C->new_of.p, C->old_of.p, brp.p, B->col.p, C->src.p, err.p);
  int herr = 0;
  GB_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(herr) return GB300_ERR_UNSUPPORTED;
  B->csr_valid = true;
  choose_tpr(B);
  return GB300_OK;
}

// The reverse Cuthill-McKee order of Sparskit's cmkreord (cmkreord.f:3-30,
// with perphn, BFS, add_lvst and rversp of reordering.f:15-380), as
// Renumbering_Technique 1 runs it before the ILU (Sparskit.cpp:245-256):
// a breadth-first search from row 0 lists the rows level by level (a row's
// unlisted neighbours appended in the order its CSR row holds them; when a
// connected component is exhausted, the next unlisted row by index starts
// the next level); while the search from a row of the last level with the
// fewest entries (the first such row) yields more levels, it is repeated
// from there (a pseudo-peripheral start); the listing of the last search,
// reversed, is the new order.  new_of[i] is the new index of row i.
void rcmk_order(int n, const int *rowptr, const int *col, int *new_of)
{
  if(n <= 0) return;
  std::vector<int> order(n), lev;
  std::vector<char> seen(n);
  auto search = [&](int start) {
    std::fill(seen.begin(), seen.end(), 0);
    lev.clear();
    int head = 0, tail = 0, next = 0;
    order[tail++] = start;
    seen[start] = 1;
    for(;;) {
      lev.push_back(head);
      const int end = tail;
      for(int t = head; t < end; t++) {
        const int i = order[t];
        for(int k = rowptr[i]; k < rowptr[i + 1]; k++) {
          const int j = col[k];
          if(!seen[j]) {
            seen[j] = 1;
            order[tail++] = j;
          }
        }
      }
      head = end;
      if(head < tail) continue;
      while(next < n && seen[next]) next++;
      if(next >= n) break;
      seen[next] = 1;
      order[tail++] = next;
    }
    lev.push_back(tail);
    return (int)lev.size() - 1;  // levels
  };
  int start = 0, best = 0;
  for(;;) {
    const int nl = search(start);
    if(nl <= best) break;
    best = nl;
    // the first row of the last level with the fewest entries (fewer than
    // the number of rows listed)
    int mindeg = lev[nl];
    for(int t = lev[nl - 1]; t < lev[nl]; t++) {
      const int i = order[t], deg = rowptr[i + 1] - rowptr[i];
      if(deg < mindeg) {
        start = i;
        mindeg = deg;
      }
    }
  }
  for(int t = 0; t < n; t++) new_of[order[n - 1 - t]] = t;
}

// The RCMK order of A's pattern (Renumbering_Technique 2 of this backend:
// the reference's Renumbering_Technique 1) and the permuted structure,
// cached with A's pattern version like the multicolour ordering
int rcmk_build(gb300_matrix *A)
{
  const int n = A->n;
  if(A->mc && A->mc->kind == 1 && A->mc->version == A->pattern_version && A->mc->n == n)
    return GB300_OK;
  colour_free(A->mc);
  A->mc = nullptr;
  cudaStream_t st = A->ctx->stream;
  std::vector<int> rp(n + 1), ci(A->nnz > 0 ? A->nnz : 1), no(n), oo(n);
  GB_CUDA(cudaMemcpyAsync(rp.data(), A->rowptr.p, sizeof(int) * (n + 1),
                          cudaMemcpyDeviceToHost, st));
  if(A->nnz > 0)
    GB_CUDA(cudaMemcpyAsync(ci.data(), A->col.p, sizeof(int) * A->nnz,
                            cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  rcmk_order(n, rp.data(), ci.data(), no.data());
  for(int i = 0; i < n; i++) oo[no[i]] = i;
  Colouring *C = new Colouring();
  C->n = n;
  C->version = A->pattern_version;
  C->kind = 1;
  int rc = C->new_of.alloc(n);
  if(rc == GB300_OK) rc = C->old_of.alloc(n);
  if(rc == GB300_OK &&
     (cudaMemcpyAsync(C->new_of.p, no.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st) !=
        cudaSuccess ||
      cudaMemcpyAsync(C->old_of.p, oo.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st) !=
        cudaSuccess))
    rc = GB300_ERR_CUDA;
  if(rc == GB300_OK) rc = permuted_structure(A, C, st);
  if(rc != GB300_OK) {
    colour_free(C);
    return rc;
  }
  A->mc = C;
  return GB300_OK;
}

void permute_system(const Colouring *C, long long nnz, const double *val,
                    const double *rhs, double *bval, double *brhs, cudaStream_t st)
{
  k_gather_vals<<<grid_for(nnz, 256), 256, 0, st>>>(nnz, C->src.p, val, bval);
  k_gather_rows<<<grid_for(C->n, 256), 256, 0, st>>>(C->n, C->old_of.p, rhs, brhs);
}

void unpermute_solution(const Colouring *C, const double *y, double *x, cudaStream_t st)
{
  k_scatter_rows<<<grid_for(C->n, 256), 256, 0, st>>>(C->n, C->old_of.p, y, x);
}

// the Krylov solve of A x = rhs (values val) on the multicolour-permuted
// system; *used = false when the ordering is not available (nothing done)
int gmres_solve_coloured(gb300_matrix *A, const double *val, const double *rhs,
                         double *x, const gb300_solver_params *p,
                         gb300_solve_info *info, Work &W, bool *used)
{
  *used = false;
  const int whole[2] = {0, A->n};
  int rc = p->renumbering_technique == 2 ? rcmk_build(A) : colour_build(A, 1, whole);
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
  permute_system(C, A->nnz, val, rhs, B->val.p, rb.p, st);
  if(correction_valid(A)) {  // the learned correction follows the rows
    GB_TRY(B->corr.alloc(A->nnz));
    k_gather_vals<<<grid_for(A->nnz, 256), 256, 0, st>>>(A->nnz, C->src.p, A->corr.p,
                                                          B->corr.p);
    B->corr_version = B->pattern_version;
  }
  if(coarse_valid(A)) GB_TRY(coarse_follow(A, B, C, st));  // the aggregates too
  GB_CUDA(cudaGetLastError());
  rc = gmres_solve(B, B->val.p, rb.p, yb.p, p, info, W);
  if(rc != GB300_OK) return rc;
  unpermute_solution(C, yb.p, x, st);
  GB_CUDA(cudaGetLastError());
  return GB300_OK;
}

// z = M^-1 v for the preconditioner a solve with parameters p would use
// (ILU(0) in GetDP's order or the multicolour order, plus the learned
// correction for Preconditioner 20), on A's unscaled values
int precond_apply(gb300_matrix *A, const gb300_solver_params *p, const double *v,
                  double *z)
{
  cudaStream_t st = A->ctx->stream;
  const int n = A->n;
  const bool learned = precond_learned(p->preconditioner);
  const bool coarse = precond_two_level(p->preconditioner);
  const bool learned_post = learned && p->preconditioner != kPrecondLearnedCoarsePre;
  const bool sai = (p->preconditioner == kPrecondLearnedSai ||
                    p->preconditioner == kPrecondSai);
  if(p->preconditioner != 6 && !learned && !coarse) {
    set_error("preconditioner apply: Preconditioner %d is not an ILU(0)", p->preconditioner);
    return GB300_ERR_UNSUPPORTED;
  }
  if(learned && !correction_valid(A)) {
    set_error("Preconditioner %d needs a correction on the matrix pattern", p->preconditioner);
    return GB300_ERR_ARG;
  }
  if(coarse && !coarse_valid(A)) {
    set_error("Preconditioner %d needs aggregates on the matrix pattern", p->preconditioner);
    return GB300_ERR_ARG;
  }
  const bool fp32 = (p->precision != 0);
  gb300_matrix *M = A;
  DevBuf<double> vb, zb, t1, t2, t3, t4;
  DevBuf<float> t32;
  GB_TRY(t1.alloc(n));
  GB_TRY(t2.alloc(n));
  if(coarse) {
    GB_TRY(t3.alloc(n));
    GB_TRY(t4.alloc(n));
  }
  if(fp32) GB_TRY(t32.alloc(n));
  const double *vin = v;
  double *zout = z;
  Colouring *C = nullptr;
  if((p->renumbering_technique == 1 || p->renumbering_technique == 2) && !sai) {
    const int whole[2] = {0, n};
    int rc = p->renumbering_technique == 2 ? rcmk_build(A) : colour_build(A, 1, whole);
    if(rc != GB300_OK && rc != GB300_ERR_UNSUPPORTED) return rc;
    if(rc == GB300_OK) {
      C = A->mc;
      M = C->B;
      GB_TRY(vb.alloc(n));
      GB_TRY(zb.alloc(n));
      permute_system(C, A->nnz, A->val.p, v, M->val.p, vb.p, st);
      if(learned) {
        GB_TRY(M->corr.alloc(A->nnz));
        k_gather_vals<<<grid_for(A->nnz, 256), 256, 0, st>>>(A->nnz, C->src.p, A->corr.p,
                                                              M->corr.p);
        M->corr_version = M->pattern_version;
      }
      if(coarse) GB_TRY(coarse_follow(A, M, C, st));
      vin = vb.p;
      zout = zb.p;
    }
  }
  int zr = 0;
  // Re_Use_LU: keep the factor of the previous call (same pattern)
  if(!sai) GB_TRY(ilu_factor(M, M->val.p, fp32, &zr, p->re_use_lu != 0));
  if(zr) {
    set_error("Zero pivot on line %d in ILU", zr);
    return GB300_ERR_ZERO_PIVOT;
  }
  auto smooth = [&](const double *vv, double *zz, bool corr) {
    if(sai) {  // z = G v
      spmv_guarded(M, M->corr.p, vv, zz, nullptr, st);
      return;
    }
    ilu_apply(M, ilu_mode(p), vv, zz, fp32 ? t32.p : nullptr, nullptr, st);
    if(corr) correction_apply(M, M->val.p, vv, zz, t1.p, t2.p, nullptr, st);
  };
  if(p->preconditioner == kPrecondSai) GB_TRY(spai1(M, M->val.p));
  if(coarse) {
    GB_TRY(coarse_setup(M, M->val.p, p->re_use_lu != 0));
    two_level_apply(M, M->val.p, vin, zout, t3.p, t4.p, nullptr, st,
                    [&](const double *vv, double *zz) { smooth(vv, zz, learned); },
                    [&](const double *vv, double *zz) { smooth(vv, zz, learned_post); });
  }
  else
    smooth(vin, zout, learned);
  if(C) unpermute_solution(C, zout, z, st);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(st));
  return GB300_OK;
}

}  // namespace gb
