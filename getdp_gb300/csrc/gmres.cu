// ILU(0) and the GMRES family on the GPU.
//
// ILU(0) (ilu0, contrib/Sparskit/ilut.F:1818-1941) keeps A's pattern; the
// factor is stored in a copy of A's values (L multipliers left of the
// diagonal, U right of it) plus the inverted pivots, as Sparskit's MSR
// layout does.  Rows are factored and solved level by level: a level holds
// rows whose lower (resp. upper) neighbours all belong to earlier levels,
// so its rows are independent.  Narrow levels (<= kNarrow rows) run back to
// back inside one thread block separated by __syncthreads; a wide level gets
// its own grid launch.  For the solves, each wide level also keeps its rows'
// L (resp. U) entries in a sliced-ELL copy (32 rows per slice, entry j of
// the slice's rows side by side), so that a warp reads them coalesced and
// without the row-pointer indirection.  The triangular solves follow lusol
// (ilut.F:2297-2347) row by row in the same accumulation order.
//
// GMRES(m) and FGMRES(m) follow iters.f:1912-2219 / :2522-2806 with right
// preconditioning (Preconditioner_Position 2): restart residual, Arnoldi
// steps, Givens rotations (iters.f:3235-3273), the stopping test on the
// Givens residual estimate, and the triangular solve + update at the end of
// a cycle.  The orthogonalisation is classical Gram-Schmidt with block dot
// products, which parallelises over the basis, in place of the reference's
// sequential modified Gram-Schmidt; like mgsro (iters.f:3475) it
// re-orthogonalises selectively (a second pass when the first removed more
// than 98 % of ||w||^2), and both return an orthonormal basis to working
// precision.
#include <algorithm>
#include <memory>

#include "krylov.cuh"

namespace gb {

constexpr int kNarrow = 2048;
constexpr int kNarrowThreads = 1024;

struct Segment {
  int l0, l1;  // levels [l0, l1)
  bool narrow;
  int width;   // rows of the (single) wide level
  int r0;      // first index in the level-row list
};

// sliced-ELL copy of one triangular part, wide levels only: slice s holds
// 32 rows x width[s] entries at 32 * wscan[s], entry j of lane l at
// + 32 j + l; src is the entry's position in the CSR factor (-1: padding,
// col = the row itself with value 0)
struct EllPart {
  std::vector<int> slice0;  // per segment: its first slice (wide segments)
  int nslices = 0;
  long long entries = 0;
  DevBuf<int> width, col, src;
  DevBuf<long long> wscan;
  DevBuf<double> v64;
  DevBuf<float> v32;
};

struct ilu_data {
  int n = 0;
  EllPart lell, uell;
  DevBuf<int> diag;                 // position of a_ii in each row
  DevBuf<int> lrows, urows;         // rows grouped by level
  DevBuf<int> lptr, uptr;           // level offsets (device copies)
  std::vector<int> hlptr, huptr;    // level offsets (host)
  std::vector<Segment> lseg, useg;
  DevBuf<double> lu64, inv64;
  DevBuf<float> lu32, inv32;
  bool fact64 = false, fact32 = false;  // a factor of that precision is held
  unsigned version = ~0u;               // the matrix pattern it was set up for
  std::unique_ptr<SysLevels> sys;       // the schedule cut into a batch's blocks
};

void ilu_free(ilu_data *d) { delete d; }

// ---------------------------------------------------------------------------
// level schedule
// ---------------------------------------------------------------------------
__global__ void k_ilu_prep(int n, const int *__restrict__ rowptr,
                           const int *__restrict__ col, int *__restrict__ diag,
                           int *__restrict__ indl, int *__restrict__ indu,
                           int *__restrict__ err)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n) return;
  int s = rowptr[i], e = rowptr[i + 1];
  int dpos = -1, nl = 0, nu = 0;
  for(int k = s; k < e; k++) {
    int c = col[k];
    if(c < i)
      nl++;
    else if(c > i)
      nu++;
    else
      dpos = k;
    // structural symmetry: (c, i) must exist
    if(c != i && find_col(col, rowptr[c], rowptr[c + 1], i) < 0)
      atomicOr(err, 2);
  }
  if(dpos < 0) atomicOr(err, 1);
  diag[i] = dpos;
  indl[i] = nl;
  indu[i] = nu;
}

__global__ void k_level0(int n, const int *__restrict__ indeg,
                         int *__restrict__ rows, int *__restrict__ cnt)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n && indeg[i] == 0) rows[atomicAdd(cnt, 1)] = i;
}

// release the dependants of one level; UPPER = 0 walks the lower
// triangular DAG (dependants of i are j > i in row i), UPPER = 1 the upper
template <int UPPER>
__global__ void k_level_next(int p0, int p1, const int *__restrict__ rowptr,
                             const int *__restrict__ col,
                             const int *__restrict__ diag,
                             int *__restrict__ indeg, int *__restrict__ rows,
                             int *__restrict__ cnt)
{
  int t = p0 + blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= p1) return;
  int i = rows[t];
  int s = UPPER ? rowptr[i] : diag[i] + 1;
  int e = UPPER ? diag[i] : rowptr[i + 1];
  for(int k = s; k < e; k++) {
    int j = col[k];
    if(atomicSub(&indeg[j], 1) == 1) rows[p1 + atomicAdd(cnt, 1)] = j;
  }
}

template <int UPPER>
static int make_levels(gb300_matrix *A, ilu_data *L, int *d_indeg,
                       DevBuf<int> &rows, DevBuf<int> &dptr,
                       std::vector<int> &hptr, std::vector<Segment> &seg)
{
  cudaStream_t st = A->ctx->stream;
  int n = A->n;
  DevBuf<int> cnt;
  GB_TRY(cnt.alloc(1));
  GB_TRY(rows.alloc(n));
  GB_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int), st));
  k_level0<<<grid_for(n, 256), 256, 0, st>>>(n, d_indeg, rows.p, cnt.p);
  int c = 0;
  GB_CUDA(cudaMemcpyAsync(&c, cnt.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  hptr.assign(1, 0);
  hptr.push_back(c);
  int p0 = 0, p1 = c;
  while(p1 < n) {
    if(p1 == p0) {
      set_error("ILU level schedule: dependency cycle");
      return GB300_ERR_ARG;
    }
    GB_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int), st));
    k_level_next<UPPER><<<grid_for(p1 - p0, 256), 256, 0, st>>>(
      p0, p1, A->rowptr.p, A->col.p, L->diag.p, d_indeg, rows.p, cnt.p);
    GB_CUDA(cudaMemcpyAsync(&c, cnt.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    p0 = p1;
    p1 += c;
    hptr.push_back(p1);
  }
  int nl = (int)hptr.size() - 1;
  GB_TRY(dptr.alloc(nl + 1));
  GB_CUDA(cudaMemcpyAsync(dptr.p, hptr.data(), sizeof(int) * (nl + 1),
                          cudaMemcpyHostToDevice, st));
  seg.clear();
  for(int l = 0; l < nl;) {
    int w = hptr[l + 1] - hptr[l];
    if(w > kNarrow) {
      seg.push_back({l, l + 1, false, w, hptr[l]});
      l++;
    }
    else {
      int l1 = l;
      while(l1 < nl && hptr[l1 + 1] - hptr[l1] <= kNarrow) l1++;
      seg.push_back({l, l1, true, 0, hptr[l]});
      l = l1;
    }
  }
  GB_CUDA(cudaStreamSynchronize(st));
  return GB300_OK;
}

// entries of row i's strictly lower (UPPER = 0) or upper part
template <int UPPER>
__device__ __forceinline__ void part_range(int i, const int *rowptr, const int *diag,
                                           int &k0, int &cnt)
{
  k0 = UPPER ? diag[i] + 1 : rowptr[i];
  cnt = UPPER ? rowptr[i + 1] - diag[i] - 1 : diag[i] - rowptr[i];
}

template <int UPPER>
__global__ void k_ell_width(int r0, int w, int nsl, int slice0, const int *__restrict__ rows,
                            const int *__restrict__ rowptr, const int *__restrict__ diag,
                            int *__restrict__ width)
{
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= nsl * 32) return;  // whole warps: nsl * 32 is a multiple of 32
  int cnt = 0;
  if(t < w) {
    int k0;
    part_range<UPPER>(rows[r0 + t], rowptr, diag, k0, cnt);
  }
  cnt = __reduce_max_sync(0xffffffffu, cnt);
  if((t & 31) == 0) width[slice0 + (t >> 5)] = cnt;
}

template <int UPPER>
__global__ void k_ell_fill(int r0, int w, int nsl, int slice0, const int *__restrict__ rows,
                           const int *__restrict__ rowptr, const int *__restrict__ col,
                           const int *__restrict__ diag, const int *__restrict__ width,
                           const long long *__restrict__ wscan, int *__restrict__ ecol,
                           int *__restrict__ esrc)
{
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= nsl * 32) return;
  int s = slice0 + (t >> 5), lane = t & 31;
  long long base = 32 * wscan[s] + lane;
  int W = width[s];
  int i = 0, k0 = 0, cnt = 0;
  if(t < w) {
    i = rows[r0 + t];
    part_range<UPPER>(i, rowptr, diag, k0, cnt);
  }
  for(int j = 0; j < W; j++) {
    bool in = j < cnt;
    ecol[base + 32LL * j] = in ? col[k0 + j] : i;
    esrc[base + 32LL * j] = in ? k0 + j : -1;
  }
}

template <typename T>
__global__ void k_ell_vals(long long m, const int *__restrict__ src, const T *__restrict__ lu,
                           T *__restrict__ v)
{
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(e < m) v[e] = src[e] >= 0 ? lu[src[e]] : (T)0;
}

template <int UPPER>
static int build_ell(gb300_matrix *A, const std::vector<Segment> &seg, const int *rows,
                     const int *diag, EllPart &E, cudaStream_t st)
{
  E.slice0.assign(seg.size(), -1);
  E.nslices = 0;
  for(size_t q = 0; q < seg.size(); q++)
    if(!seg[q].narrow) {
      E.slice0[q] = E.nslices;
      E.nslices += (seg[q].width + 31) / 32;
    }
  E.entries = 0;
  if(E.nslices == 0) return GB300_OK;
  GB_TRY(E.width.alloc(E.nslices));
  GB_TRY(E.wscan.alloc(E.nslices));
  for(size_t q = 0; q < seg.size(); q++)
    if(!seg[q].narrow) {
      int nsl = (seg[q].width + 31) / 32;
      k_ell_width<UPPER><<<grid_for((long long)nsl * 32, 256), 256, 0, st>>>(
        seg[q].r0, seg[q].width, nsl, E.slice0[q], rows, A->rowptr.p, diag, E.width.p);
    }
  DevBuf<long long> tmp;
  long long total = 0;
  GB_TRY(exclusive_scan(E.width.p, E.nslices, E.wscan.p, &total, tmp, st));
  E.entries = 32 * total;
  GB_TRY(E.col.alloc(E.entries > 0 ? E.entries : 1));
  GB_TRY(E.src.alloc(E.entries > 0 ? E.entries : 1));
  for(size_t q = 0; q < seg.size(); q++)
    if(!seg[q].narrow) {
      int nsl = (seg[q].width + 31) / 32;
      k_ell_fill<UPPER><<<grid_for((long long)nsl * 32, 256), 256, 0, st>>>(
        seg[q].r0, seg[q].width, nsl, E.slice0[q], rows, A->rowptr.p, A->col.p, diag,
        E.width.p, E.wscan.p, E.col.p, E.src.p);
    }
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(st));
  return GB300_OK;
}

// the factor's values in the ELL copies (after each factorisation)
template <typename T>
static int ell_values(EllPart &E, const T *lu, DevBuf<T> &v, cudaStream_t st)
{
  if(E.entries == 0) return GB300_OK;
  GB_TRY(v.alloc(E.entries));
  k_ell_vals<T><<<grid_for(E.entries, 256), 256, 0, st>>>(E.entries, E.src.p, lu, v.p);
  GB_CUDA(cudaGetLastError());
  return GB300_OK;
}

static int ilu_setup(gb300_matrix *A)
{
  // the level schedule and diagonal positions belong to one pattern
  if(A->ilu && A->ilu->n == A->n && A->ilu->version == A->pattern_version) return GB300_OK;
  if(A->ilu) ilu_free(A->ilu);
  A->ilu = new ilu_data();
  ilu_data *L = A->ilu;
  L->n = A->n;
  L->version = A->pattern_version;
  cudaStream_t st = A->ctx->stream;
  int n = A->n;
  DevBuf<int> indl, indu, err;
  GB_TRY(L->diag.alloc(n));
  GB_TRY(indl.alloc(n));
  GB_TRY(indu.alloc(n));
  GB_TRY(err.alloc(1));
  GB_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  k_ilu_prep<<<grid_for(n, 256), 256, 0, st>>>(n, A->rowptr.p, A->col.p,
                                                L->diag.p, indl.p, indu.p, err.p);
  int herr = 0;
  GB_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(herr & 1) {
    set_error("ILU(0): a row has no diagonal entry");
    ilu_free(A->ilu);
    A->ilu = nullptr;
    return GB300_ERR_ZERO_PIVOT;
  }
  if(herr & 2) {
    set_error("ILU(0): the level schedule needs a structurally symmetric pattern");
    ilu_free(A->ilu);
    A->ilu = nullptr;
    return GB300_ERR_UNSUPPORTED;
  }
  int rc = make_levels<0>(A, L, indl.p, L->lrows, L->lptr, L->hlptr, L->lseg);
  if(rc == GB300_OK)
    rc = make_levels<1>(A, L, indu.p, L->urows, L->uptr, L->huptr, L->useg);
  if(rc == GB300_OK) rc = build_ell<0>(A, L->lseg, L->lrows.p, L->diag.p, L->lell, st);
  if(rc == GB300_OK) rc = build_ell<1>(A, L->useg, L->urows.p, L->diag.p, L->uell, st);
  if(rc != GB300_OK) {
    ilu_free(A->ilu);
    A->ilu = nullptr;
  }
  return rc;
}

// ---------------------------------------------------------------------------
// per-row work of the three level-scheduled sweeps
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void row_fact(int i, const int *__restrict__ rowptr,
                                         const int *__restrict__ col,
                                         const int *__restrict__ diag, T *lu,
                                         T *inv, int *zero_row)
{
  int s = rowptr[i], e = rowptr[i + 1], di = diag[i];
  for(int k = s; k < di; k++) {
    int kr = col[k];
    T l = lu[k] * inv[kr];  // tl = alu(j) * alu(jrow)
    lu[k] = l;
    int ks = diag[kr] + 1, ke = rowptr[kr + 1];
    int lo = k + 1;  // columns of row i beyond kr
    for(int kk = ks; kk < ke; kk++) {
      int c = col[kk];
      int pos = find_col(col, lo, e, c);
      if(pos >= 0) {
        lu[pos] = lu[pos] - l * lu[kk];
        lo = pos + 1;
      }
    }
  }
  T piv = lu[di];
  if(piv == (T)0) {
    atomicMin(zero_row, i + 1);
    inv[i] = (T)0;
  }
  else
    inv[i] = (T)(1.0 / (double)piv);
}

// T: the factor's storage type; X: the vectors' (and the arithmetic's) type
template <typename T, typename X = T>
__device__ __forceinline__ void row_fwd(int i, const int *__restrict__ rowptr,
                                        const int *__restrict__ col,
                                        const int *__restrict__ diag,
                                        const T *__restrict__ lu, const X *src, X *x)
{
  X s = src[i];  // the right-hand side's entry (src may be x itself)
  for(int k = rowptr[i]; k < diag[i]; k++) s = s - (X)lu[k] * x[col[k]];
  x[i] = s;
}

template <typename T, typename X = T>
__device__ __forceinline__ void row_bwd(int i, const int *__restrict__ rowptr,
                                        const int *__restrict__ col,
                                        const int *__restrict__ diag,
                                        const T *__restrict__ lu,
                                        const T *__restrict__ inv, X *x)
{
  X s = x[i];
  for(int k = diag[i] + 1; k < rowptr[i + 1]; k++) s = s - (X)lu[k] * x[col[k]];
  x[i] = (X)inv[i] * s;
}

// MODE 0 factor, 1 forward solve, 2 backward solve
template <int MODE, typename T, typename X = T>
__global__ void __launch_bounds__(kNarrowThreads)
k_levels_narrow(int l0, int l1, const int *__restrict__ lptr,
                const int *__restrict__ rows, const int *__restrict__ rowptr,
                const int *__restrict__ col, const int *__restrict__ diag,
                T *lu, T *inv, X *x, int *zero_row, const int *flag,
                const unsigned char *__restrict__ rmask, const X *src)
{
  if(flag && !*flag) return;
  for(int l = l0; l < l1; l++) {
    int a = lptr[l], b = lptr[l + 1];
    for(int t = a + threadIdx.x; t < b; t += blockDim.x) {
      int i = rows[t];
      if(MODE != 0 && rmask && !rmask[i]) continue;
      if(MODE == 0)
        row_fact<T>(i, rowptr, col, diag, lu, inv, zero_row);
      else if(MODE == 1)
        row_fwd<T, X>(i, rowptr, col, diag, lu, src, x);
      else
        row_bwd<T, X>(i, rowptr, col, diag, lu, inv, x);
    }
    __syncthreads();
  }
}

template <int MODE, typename T, typename X = T>
__global__ void __launch_bounds__(256)
k_level_wide(int r0, int width, const int *__restrict__ rows,
             const int *__restrict__ rowptr, const int *__restrict__ col,
             const int *__restrict__ diag, T *lu, T *inv, X *x, int *zero_row,
             const int *flag, const unsigned char *__restrict__ rmask, const X *src)
{
  if(flag && !*flag) return;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= width) return;
  int i = rows[r0 + t];
  if(MODE != 0 && rmask && !rmask[i]) return;
  if(MODE == 0)
    row_fact<T>(i, rowptr, col, diag, lu, inv, zero_row);
  else if(MODE == 1)
    row_fwd<T, X>(i, rowptr, col, diag, lu, src, x);
  else
    row_bwd<T, X>(i, rowptr, col, diag, lu, inv, x);
}

// one wide level of a triangular solve from the sliced-ELL copy: entry j
// of the warp's 32 rows is one coalesced load (the row's entries stay in
// CSR order, the accumulation order of lusol)
template <int MODE, typename T, typename X = T>
__global__ void __launch_bounds__(256)
k_level_ell(int r0, int w, int slice0, const int *__restrict__ rows,
            const int *__restrict__ width, const long long *__restrict__ wscan,
            const int *__restrict__ ecol, const T *__restrict__ ev,
            const T *__restrict__ inv, X *x, const int *flag,
            const unsigned char *__restrict__ rmask, const X *src)
{
  if(flag && !*flag) return;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= w) return;
  int i = rows[r0 + t];
  if(rmask && !rmask[i]) return;
  int s = slice0 + (t >> 5);
  long long e = 32 * wscan[s] + (t & 31);
  int W = width[s];
  X acc = (MODE == 1) ? src[i] : x[i];
  for(int j = 0; j < W; j++, e += 32) acc = acc - (X)ev[e] * x[ecol[e]];
  x[i] = (MODE == 2) ? (X)inv[i] * acc : acc;
}

template <typename T> const T *ell_vals(const EllPart &E);
template <> const double *ell_vals<double>(const EllPart &E) { return E.v64.p; }
template <> const float *ell_vals<float>(const EllPart &E) { return E.v32.p; }

// rmask (sweeps only): rows with rmask[i] == 0 are skipped (the rows of
// systems of a batch that have stopped)
template <int MODE, typename T, typename X = T>
// MODE 1 reads the right-hand side from src (x when null) and writes x
static void run_levels(const gb300_matrix *A, const ilu_data *L, T *lu, T *inv,
                       X *x, int *zero_row, const int *flag, cudaStream_t st,
                       const unsigned char *rmask = nullptr, const X *src = nullptr)
{
  if(!src) src = x;
  bool upper = (MODE == 2);
  const std::vector<Segment> &seg = upper ? L->useg : L->lseg;
  const int *rows = upper ? L->urows.p : L->lrows.p;
  const int *lptr = upper ? L->uptr.p : L->lptr.p;
  const EllPart &E = upper ? L->uell : L->lell;
  for(size_t q = 0; q < seg.size(); q++) {
    const Segment &s = seg[q];
    if(MODE != 0 && !s.narrow && E.entries > 0) {
      k_level_ell<MODE, T, X><<<grid_for(s.width, 256), 256, 0, st>>>(
        s.r0, s.width, E.slice0[q], rows, E.width.p, E.wscan.p, E.col.p,
        ell_vals<T>(E), inv, x, flag, rmask, src);
      continue;
    }
    if(s.narrow)
      k_levels_narrow<MODE, T, X><<<1, kNarrowThreads, 0, st>>>(
        s.l0, s.l1, lptr, rows, A->rowptr.p, A->col.p, L->diag.p, lu, inv, x,
        zero_row, flag, rmask, src);
    else
      k_level_wide<MODE, T, X><<<grid_for(s.width, 256), 256, 0, st>>>(
        s.r0, s.width, rows, A->rowptr.p, A->col.p, L->diag.p, lu, inv, x,
        zero_row, flag, rmask, src);
  }
}

template <typename TO, typename TI>
__global__ void k_cvt(long long n, const TI *__restrict__ in, TO *__restrict__ out,
                      const int *flag)
{
  if(flag && !*flag) return;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) out[i] = (TO)in[i];
}

// factor A's values (val) into the ILU(0) of the requested precision; with
// reuse, a factor of that precision already held for A's pattern is kept
// (Re_Use_LU, as LinAlg_SolveAgain sets it: LinAlg_SPARSKIT.cpp:578-585)
int ilu_factor(gb300_matrix *A, const double *val, bool fp32, int *zero_row_out,
               bool reuse, int *factorized)
{
  GB_TRY(ilu_setup(A));
  ilu_data *L = A->ilu;
  if(factorized) *factorized = 0;
  if(reuse && (fp32 ? L->fact32 : L->fact64)) {
    *zero_row_out = 0;
    return GB300_OK;
  }
  if(factorized) *factorized = 1;
  L->fact32 = L->fact64 = false;
  cudaStream_t st = A->ctx->stream;
  int n = A->n;
  DevBuf<int> zr;
  GB_TRY(zr.alloc(1));
  int big = 0x7fffffff;
  GB_CUDA(cudaMemcpyAsync(zr.p, &big, sizeof(int), cudaMemcpyHostToDevice, st));
  if(!fp32) {
    GB_TRY(L->lu64.alloc(A->nnz));
    GB_TRY(L->inv64.alloc(n));
    GB_CUDA(cudaMemcpyAsync(L->lu64.p, val, sizeof(double) * A->nnz,
                            cudaMemcpyDeviceToDevice, st));
    run_levels<0, double>(A, L, L->lu64.p, L->inv64.p, (double *)nullptr, zr.p,
                          nullptr, st);
    GB_TRY(ell_values<double>(L->lell, L->lu64.p, L->lell.v64, st));
    GB_TRY(ell_values<double>(L->uell, L->lu64.p, L->uell.v64, st));
  }
  else {
    GB_TRY(L->lu32.alloc(A->nnz));
    GB_TRY(L->inv32.alloc(n));
    k_cvt<float, double><<<grid_for(A->nnz, 256), 256, 0, st>>>(A->nnz, val,
                                                                L->lu32.p, nullptr);
    run_levels<0, float>(A, L, L->lu32.p, L->inv32.p, (float *)nullptr, zr.p,
                         nullptr, st);
    GB_TRY(ell_values<float>(L->lell, L->lu32.p, L->lell.v32, st));
    GB_TRY(ell_values<float>(L->uell, L->lu32.p, L->uell.v32, st));
  }
  int hz = 0;
  GB_CUDA(cudaMemcpyAsync(&hz, zr.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  GB_CUDA(cudaGetLastError());
  *zero_row_out = (hz == big) ? 0 : hz;
  if(!*zero_row_out) (fp32 ? L->fact32 : L->fact64) = true;
  return GB300_OK;
}

// z = M^-1 v for the ILU(0) factor: mode 0 FP64 factor and sweeps; 1 FP32
// factor, sweeps on FP32 vectors in FP32 arithmetic; 2 FP32 factor, sweeps
// in FP64 (the reference built with HAVE_ILU_FLOAT: lusol's float alu
// against double x, ilut.F:2297-2347)
void ilu_apply(const gb300_matrix *A, int mode, const double *v, double *z,
               float *t32, const int *flag, cudaStream_t st,
               const unsigned char *rmask)
{
  const ilu_data *L = A->ilu;
  int n = A->n;
  if(mode == 0) {
    // the forward sweep reads v and writes z (no copy of v first); rows a
    // mask leaves out are not written
    run_levels<1, double>(A, L, (double *)L->lu64.p, (double *)L->inv64.p, z,
                          nullptr, flag, st, rmask, v);
    run_levels<2, double>(A, L, (double *)L->lu64.p, (double *)L->inv64.p, z,
                          nullptr, flag, st, rmask);
  }
  else if(mode == 2) {
    run_levels<1, float, double>(A, L, (float *)L->lu32.p, (float *)L->inv32.p, z, nullptr,
                                 flag, st, rmask, v);
    run_levels<2, float, double>(A, L, (float *)L->lu32.p, (float *)L->inv32.p, z, nullptr,
                                 flag, st, rmask);
  }
  else {
    k_cvt<float, double><<<grid_for(n, 256), 256, 0, st>>>(n, v, t32, flag);
    run_levels<1, float>(A, L, (float *)L->lu32.p, (float *)L->inv32.p, t32,
                         nullptr, flag, st, rmask);
    run_levels<2, float>(A, L, (float *)L->lu32.p, (float *)L->inv32.p, t32,
                         nullptr, flag, st, rmask);
    k_cvt<double, float><<<grid_for(n, 256), 256, 0, st>>>(n, t32, z, flag);
  }
}

// one sweep's levels cut into the diagonal blocks off[0..nsys]: the rows of
// each level go, in level order, to their system's range of out, and each
// system records where its levels begin (a system's rows occupy the same
// range [off[p], off[p+1]) in out as in the matrix)
static void cut_levels(int n, int nsys, const int *off, const std::vector<int> &rows,
                       const std::vector<int> &lptr, std::vector<int> &out,
                       std::vector<int> &lev, std::vector<int> &lb, int *max_levels)
{
  std::vector<int> sys_of(n), fill(nsys), last(nsys, -1);
  std::vector<std::vector<int>> starts(nsys);
  for(int q = 0; q < nsys; q++) {
    fill[q] = off[q];
    for(int i = off[q]; i < off[q + 1]; i++) sys_of[i] = q;
  }
  out.assign(n, 0);
  const int nl = (int)lptr.size() - 1;
  for(int l = 0; l < nl; l++)
    for(int t = lptr[l]; t < lptr[l + 1]; t++) {
      int i = rows[t], q = sys_of[i];
      if(last[q] != l) {
        starts[q].push_back(fill[q]);
        last[q] = l;
      }
      out[fill[q]++] = i;
    }
  lev.clear();
  lb.assign(nsys + 1, 0);
  for(int q = 0; q < nsys; q++) {
    lb[q] = (int)lev.size();
    lev.insert(lev.end(), starts[q].begin(), starts[q].end());
    lev.push_back(off[q + 1]);
    *max_levels = std::max(*max_levels, (int)starts[q].size());
  }
  lb[nsys] = (int)lev.size();
}

int ilu_sys_levels(gb300_matrix *A, int nsys, const int *off, const SysLevels **out)
{
  GB_TRY(ilu_setup(A));
  ilu_data *L = A->ilu;
  if(L->sys && (int)L->sys->off.size() == nsys + 1 &&
     std::equal(off, off + nsys + 1, L->sys->off.begin())) {
    *out = L->sys.get();
    return GB300_OK;
  }
  cudaStream_t st = A->ctx->stream;
  const int n = A->n;
  std::vector<int> lr(n), ur(n);
  if(n > 0) {
    GB_CUDA(cudaMemcpyAsync(lr.data(), L->lrows.p, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaMemcpyAsync(ur.data(), L->urows.p, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
  }
  GB_CUDA(cudaStreamSynchronize(st));
  auto S = std::make_unique<SysLevels>();
  S->off.assign(off, off + nsys + 1);
  std::vector<int> lo, uo, llev, ulev, llb, ulb;
  cut_levels(n, nsys, off, lr, L->hlptr, lo, llev, llb, &S->max_levels);
  cut_levels(n, nsys, off, ur, L->huptr, uo, ulev, ulb, &S->max_levels);
  auto up = [&](DevBuf<int> &d, const std::vector<int> &h) -> int {
    GB_TRY(d.alloc(h.size() > 0 ? h.size() : 1));
    if(!h.empty())
      GB_CUDA(cudaMemcpyAsync(d.p, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice, st));
    return GB300_OK;
  };
  GB_TRY(up(S->lrows, lo));
  GB_TRY(up(S->urows, uo));
  GB_TRY(up(S->llev, llev));
  GB_TRY(up(S->ulev, ulev));
  GB_TRY(up(S->llb, llb));
  GB_TRY(up(S->ulb, ulb));
  GB_CUDA(cudaStreamSynchronize(st));  // the host vectors go out of scope
  L->sys = std::move(S);
  *out = L->sys.get();
  return GB300_OK;
}

// the factor held for A (after ilu_factor): values, inverted pivots and the
// position of each diagonal entry
void ilu_factor_arrays(const gb300_matrix *A, bool fp32, const void **lu, const void **inv,
                       const int **diag)
{
  const ilu_data *L = A->ilu;
  *lu = fp32 ? (const void *)L->lu32.p : (const void *)L->lu64.p;
  *inv = fp32 ? (const void *)L->inv32.p : (const void *)L->inv64.p;
  *diag = L->diag.p;
}

// ---------------------------------------------------------------------------
// GMRES device state and kernels
// ---------------------------------------------------------------------------
constexpr int kMaxKrylov = 128;

struct GmState {
  int active;       // whole solve still running
  int cycle;        // current restart cycle still extending the basis
  int did_cycle;    // the cycle took >= 1 Arnoldi step (solution update due)
  int k;            // Arnoldi steps taken in the cycle
  int its;          // ipar(7)
  int maxit;        // ipar(6)
  int status;       // ipar(1)
  int breakdown;    // ipar(12) (-3: linear combination, -1/-2 bad vector)
  int first;        // first restart still to come
  double tol;       // fpar(4)
  double res0;      // fpar(3)
  double res;       // fpar(5)
  double res6;      // fpar(6)
  double rtol;
  double scale;     // 1 / h(k+1,k) for the new basis vector
  double H[(kMaxKrylov + 1) * kMaxKrylov];  // column-major, (m+1) x m
  double cs[kMaxKrylov], sn[kMaxKrylov], g[kMaxKrylov + 1], y[kMaxKrylov];
  double h1[kMaxKrylov + 1], h2[kMaxKrylov + 1];
  double nrm0;      // ||w||^2 before the Gram-Schmidt pass of this step
  int reorth;       // this step takes a second Gram-Schmidt pass
  int reorths;      // second passes taken so far
  // arrival counters of the kernels whose last CTA finishes a reduction
  unsigned tick_dots0, tick_dots1, tick_upd0, tick_upd1;
};

// restart: r = rhs - A x was computed with its partial norms
__global__ void k_gm_restart(GmState *S, const double *__restrict__ part, int m)
{
  if(!S->active) return;
  double rr = 0.;
  for(int i = threadIdx.x; i < kReduceBlocks; i += blockDim.x) rr += part[i];
  rr = block_sum<double, 256>(rr);
  if(threadIdx.x) return;
  S->its += 1;
  double alpha = sqrt(rr);
  if(S->first) {
    S->tol = S->rtol * alpha + 0.0;
    S->res0 = alpha;
    S->first = 0;
  }
  S->res = alpha;
  S->g[0] = alpha;
  S->k = 0;
  S->did_cycle = 0;
  S->breakdown = 0;
  // iters.f's restart test: converged when alpha <= tol (also for a zero
  // right-hand side); a NaN residual goes on to the Arnoldi step, where the
  // abnormal norm ends the solve as a break-down
  if(alpha <= S->tol) {
    S->status = 0;
    S->res6 = alpha;
    S->active = 0;
    S->cycle = 0;
    return;
  }
  S->scale = 1. / alpha;
  S->cycle = 1;
}

// y = s * x, guarded by the cycle flag
__global__ void k_gm_scale(int n, const GmState *__restrict__ S,
                           const double *__restrict__ x, double *__restrict__ y)
{
  if(!S->cycle) return;
  double s = S->scale;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (long long)gridDim.x * blockDim.x)
    y[i] = s * x[i];
}

// partial dots <V_j, w>, j < k, over a fixed grid; part[j * B + block].
// PASS 0 also forms <w, w> (as column k), the norm the selective
// re-orthogonalisation compares with; PASS 1 runs only when this step
// takes the second Gram-Schmidt pass.
// the partial dots of columns [j0, j0 + CNT) over this CTA's share of rows
template <int CNT>
__device__ __forceinline__ void dots_group(int n, int j0, const double *__restrict__ V,
                                           size_t ldv, const double *__restrict__ w,
                                           double *__restrict__ part)
{
  double acc[8];
#pragma unroll
  for(int u = 0; u < 8; u++) acc[u] = 0.;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (long long)gridDim.x * blockDim.x) {
    double wi = w[i];
#pragma unroll
    for(int u = 0; u < CNT; u++) acc[u] += V[(size_t)(j0 + u) * ldv + i] * wi;
  }
  double s = block_sum8<256>(acc);
  if(threadIdx.x < CNT) part[(size_t)(j0 + threadIdx.x) * kReduceBlocks + blockIdx.x] = s;
}

// end of one Arnoldi step (thread 0), with rr = ||w||^2 after the
// Gram-Schmidt pass: h(k+1,k), Givens rotations, stopping test
__device__ void gm_step_tail(GmState *S, int k, int m, double rr)
{
  S->its += 1;
  double *Hc = S->H + (size_t)(k - 1) * (kMaxKrylov + 1);  // column k
  double nrm = sqrt(rr);
  Hc[k] = nrm;
  S->k = k;
  S->did_cycle = 1;
  if(!(nrm > 0.)) {  // mgsro ierr -3: the new vector depends on the others
    S->breakdown = -3;
    S->cycle = 0;
    return;
  }
  // previous rotations on the new column, then a new one
  for(int i = 0; i < k - 1; i++) {
    double a = Hc[i], c = S->cs[i], s = S->sn[i];
    Hc[i] = c * a + s * Hc[i + 1];
    Hc[i + 1] = c * Hc[i + 1] - s * a;
  }
  double c, s;
  givens_dev(&Hc[k - 1], &Hc[k], &c, &s);
  S->cs[k - 1] = c;
  S->sn[k - 1] = s;
  double alpha = -s * S->g[k - 1];
  S->g[k - 1] = c * S->g[k - 1];
  S->g[k] = alpha;
  alpha = fabs(alpha);
  S->res = alpha;
  S->scale = 1. / nrm;
  if(!(k < m && !(alpha <= S->tol) && (S->maxit <= 0 || S->its < S->maxit)))
    S->cycle = 0;  // end of this cycle after the scaling below is skipped
}

// Partial dots <V_j, w>, j < k, over a fixed grid (part[j * B + block]);
// blockIdx.y selects a group of (at most) eight columns, so the groups run
// side by side and each FMA issued is needed.  PASS 0 also forms <w, w>
// (column k: V_k is w), the norm the selective re-orthogonalisation
// compares with; PASS 1 runs only when this step takes the second pass.
// The last CTA to finish sums the partials in a fixed order (one warp per
// column): PASS 0 stores h1 (and the column of H) and ||w||^2, PASS 1
// stores h2 and adds it to the column.
template <int PASS>
__global__ void __launch_bounds__(256)
k_gm_dots(int n, int k, const double *__restrict__ V, size_t ldv,
          const double *__restrict__ w, double *__restrict__ part, GmState *S, int nb)
{
  if(!S->cycle || (PASS == 1 && !S->reorth)) return;  // the same in every CTA
  const int kk = PASS == 0 ? k + 1 : k;  // column k: V_k = w itself
  const int j0 = blockIdx.y * 8;
  switch(j0 >= kk ? 0 : kk - j0 < 8 ? kk - j0 : 8) {
  case 0: break;
  case 1: dots_group<1>(n, j0, V, ldv, w, part); break;
  case 2: dots_group<2>(n, j0, V, ldv, w, part); break;
  case 3: dots_group<3>(n, j0, V, ldv, w, part); break;
  case 4: dots_group<4>(n, j0, V, ldv, w, part); break;
  case 5: dots_group<5>(n, j0, V, ldv, w, part); break;
  case 6: dots_group<6>(n, j0, V, ldv, w, part); break;
  case 7: dots_group<7>(n, j0, V, ldv, w, part); break;
  default: dots_group<8>(n, j0, V, ldv, w, part); break;
  }
  if(!arrive_last(PASS == 0 ? &S->tick_dots0 : &S->tick_dots1)) return;
  __shared__ double sums[kMaxKrylov + 1];
  __shared__ int abnormal;
  int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for(int j = wp; j < kk; j += blockDim.x / 32) {
    double v = 0.;
    for(int b = lane; b < nb; b += 32) v += __ldcg(part + (size_t)j * kReduceBlocks + b);
    v = warp_sum(v);
    if(lane == 0) sums[j] = v;
  }
  __syncthreads();
  if(threadIdx.x == 0) {
    abnormal = 0;
    if(PASS == 0) {
      // mgsro's checks on ||w||^2 before it orthogonalises (iters.f:
      // 3475-3600): zero (ierr -1) or abnormal (-2) leaves the column
      // unwritten and ends the cycle; gmres then reports a break-down
      const double nrm0 = sums[k];
      S->nrm0 = nrm0;
      if(!(nrm0 > 0. && 1. / nrm0 > 0.)) {
        abnormal = 1;
        S->its += 1;  // the Arnoldi step's product was formed
        S->breakdown = (nrm0 <= 0.) ? -1 : -2;
        S->cycle = 0;
      }
    }
  }
  __syncthreads();
  if(abnormal) return;
  for(int j = threadIdx.x; j < k; j += blockDim.x) {
    if(PASS == 0) {
      S->h1[j] = sums[j];
      S->H[(size_t)(k - 1) * (kMaxKrylov + 1) + j] = sums[j];
    }
    else {
      S->h2[j] = sums[j];
      S->H[(size_t)(k - 1) * (kMaxKrylov + 1) + j] = S->h1[j] + sums[j];
    }
  }
}

// w -= sum_j h_j V_j (h of pass `pass`) with the partials of ||w||^2 in pn.
// The last CTA to finish sums them.  After pass 0 it applies the selective
// re-orthogonalisation test with mgsro's constant (iters.f:3475-3600,
// reorth = 0.98: mgsro repeats the projection on one basis vector when it
// removed more than 98 % of the squared norm left; here the second
// classical Gram-Schmidt pass runs when the first pass removed more than
// 98 % of ||w||^2, ||w'|| < 0.14 ||w||; the loss of orthogonality of one
// pass grows like eps ||w|| / ||w'||, so a pass that keeps more than 2 %
// leaves w' orthogonal to within ~10 eps) and, without a second pass, ends
// the Arnoldi step; after pass 1 it ends the step.
__global__ void __launch_bounds__(256)
k_gm_update(int n, int k, int m, const double *__restrict__ V, size_t ldv,
            double *__restrict__ w, double *__restrict__ pn, GmState *S, int pass, int nb)
{
  if(!S->cycle || (pass == 1 && !S->reorth)) return;  // the same in every CTA
  __shared__ double h[kMaxKrylov];
  for(int j = threadIdx.x; j < k; j += blockDim.x)
    h[j] = pass == 0 ? S->h1[j] : S->h2[j];
  __syncthreads();
  double v = 0.;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (long long)gridDim.x * blockDim.x) {
    // four partial sums of h_j V_j: four independent FMA chains instead of
    // one (the FP64 FMA latency otherwise serialises the k terms)
    double s0 = 0., s1 = 0., s2 = 0., s3 = 0.;
    int j = 0;
    for(; j + 3 < k; j += 4) {
      s0 += h[j] * V[(size_t)j * ldv + i];
      s1 += h[j + 1] * V[(size_t)(j + 1) * ldv + i];
      s2 += h[j + 2] * V[(size_t)(j + 2) * ldv + i];
      s3 += h[j + 3] * V[(size_t)(j + 3) * ldv + i];
    }
    for(; j < k; j++) s0 += h[j] * V[(size_t)j * ldv + i];
    double wi = w[i] - ((s0 + s1) + (s2 + s3));
    w[i] = wi;
    v += wi * wi;
  }
  double s = block_sum<double, 256>(v);
  if(threadIdx.x == 0) pn[blockIdx.x] = s;
  if(!arrive_last(pass == 0 ? &S->tick_upd0 : &S->tick_upd1)) return;
  double rr = 0.;
  for(int i = threadIdx.x; i < nb; i += blockDim.x) rr += __ldcg(pn + i);
  rr = block_sum<double, 256>(rr);
  if(threadIdx.x) return;
  if(pass == 0) {
    S->reorth = !(rr >= 0.02 * S->nrm0);
    if(S->reorth) {
      S->reorths += 1;
      return;  // the step ends after the second pass
    }
  }
  gm_step_tail(S, k, m, rr);
}

// scale the new basis vector (runs only while the cycle continues)
__global__ void k_gm_scale_next(int n, const GmState *__restrict__ S,
                                double *__restrict__ w, int k)
{
  if(!S->cycle || S->k != k) return;
  double s = S->scale;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (long long)gridDim.x * blockDim.x)
    w[i] *= s;
}

// end of a cycle: solve H y = g (upper triangular, k x k) on one thread
__global__ void k_gm_solve_small(GmState *S)
{
  if(!S->active || !S->did_cycle || threadIdx.x) return;
  int k = S->k;
  const int ld = kMaxKrylov + 1;
  while(k > 0 && S->H[(size_t)(k - 1) * ld + (k - 1)] == 0.) k--;  // iters.f:2141-2155
  if(k == 0) {
    S->status = -3;
    S->breakdown = -4;
    S->active = 0;
    S->did_cycle = 0;
    return;
  }
  S->k = k;
  for(int i = k - 1; i >= 0; i--) {
    double t = S->g[i];
    for(int j = i + 1; j < k; j++) t -= S->H[(size_t)j * ld + i] * S->y[j];
    S->y[i] = t / S->H[(size_t)i * ld + i];
  }
}

// u = sum_j y_j Vj (GMRES) or x += sum_j y_j Z_j (FGMRES, ADD = 1)
template <int ADD>
__global__ void __launch_bounds__(256)
k_gm_combine(int n, const double *__restrict__ V, size_t ldv,
             double *__restrict__ out, const GmState *__restrict__ S)
{
  if(!S->active || !S->did_cycle) return;
  __shared__ double y[kMaxKrylov];
  int k = S->k;
  for(int j = threadIdx.x; j < k; j += blockDim.x) y[j] = S->y[j];
  __syncthreads();
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (long long)gridDim.x * blockDim.x) {
    double s = ADD ? out[i] : 0.;
    for(int j = 0; j < k; j++) s += y[j] * V[(size_t)j * ldv + i];
    out[i] = s;
  }
}

__global__ void k_gm_addto(int n, const double *__restrict__ u,
                           double *__restrict__ x, const GmState *__restrict__ S)
{
  if(!S->active || !S->did_cycle) return;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
      i += (long long)gridDim.x * blockDim.x)
    x[i] += u[i];
}

// after the update: the restart decision of iters.f:2196-2218
__global__ void k_gm_after(GmState *S)
{
  if(!S->active || threadIdx.x) return;
  S->res6 = S->res;
  if(S->breakdown != 0) {
    S->status = -3;
    S->active = 0;
    return;
  }
  bool more = (S->its < S->maxit || S->maxit <= 0) && (S->res6 > S->tol);
  if(!more) {
    if(S->res6 <= S->tol)
      S->status = 0;
    else if(S->its >= S->maxit && S->maxit > 0)
      S->status = -1;
    else
      S->status = -10;
    S->active = 0;
  }
}

// flag pointer for the preconditioner inside a cycle: S->cycle
static const int *cycle_flag(GmState *S) { return &S->cycle; }

__global__ void k_gm_apply_ok(GmState *S, int *ok)
{
  // the update's preconditioner runs when a solution update is due
  if(threadIdx.x == 0) *ok = (S->active && S->did_cycle) ? 1 : 0;
}

bool correction_valid(const gb300_matrix *A)
{
  return A->corr_version == A->pattern_version && A->corr.p && A->nnz > 0;
}

// z <- z + G (v - A z): the learned correction after the ILU(0) step (two
// fused products: t1 = v - A z, then z += G t1; t2 is not needed)
void correction_apply(const gb300_matrix *A, const double *val, const double *v,
                      double *z, double *t1, double *t2, const int *flag, cudaStream_t st)
{
  (void)t2;
  resid_guarded(A, val, z, v, t1, flag, st);
  spmv_add_guarded(A, A->corr.p, t1, z, flag, st);
}

int gmres_solve(gb300_matrix *A, const double *val, const double *rhs,
                double *x, const gb300_solver_params *p, gb300_solve_info *info,
                Work &W)
{
  cudaStream_t st = A->ctx->stream;
  int n = A->n;
  bool flexible = (p->algorithm == 9);
  if(p->algorithm != 8 && p->algorithm != 9) {
    set_error("Algorithm %d with Preconditioner %d is not supported", p->algorithm,
              p->preconditioner);
    return GB300_ERR_UNSUPPORTED;
  }
  int m = p->krylov_size <= 1 ? 15 : p->krylov_size;
  if(m > kMaxKrylov) {
    set_error("Krylov_Size %d exceeds this backend's maximum %d", m, kMaxKrylov);
    return GB300_ERR_UNSUPPORTED;
  }
  // 20: ILU(0) followed by the learned correction on A's pattern; 21, 22:
  // the two-level cycle on aggregates around ILU(0) (22: and the correction)
  const bool learned = precond_learned(p->preconditioner);
  const bool coarse = precond_two_level(p->preconditioner);
  const bool learned_post = learned && p->preconditioner != kPrecondLearnedCoarsePre;
  // 24: G alone smooths, no ILU(0); 25: with G the SPAI-1 made here
  const bool sai = (p->preconditioner == kPrecondLearnedSai ||
                    p->preconditioner == kPrecondSai);
  if(p->preconditioner == kPrecondSai && !(p->re_use_lu && correction_valid(A)))
    GB_TRY(spai1(A, val));
  bool precond = ((p->preconditioner == 6) || learned || coarse) && !sai;
  if(p->preconditioner != 0 && p->preconditioner != 6 && p->preconditioner != 8 &&
     !learned && !coarse) {
    set_error("Preconditioner %d is not supported by this backend", p->preconditioner);
    return GB300_ERR_UNSUPPORTED;
  }
  if(learned && !correction_valid(A)) {
    set_error("Preconditioner %d needs a correction on the matrix pattern "
              "(gb300_matrix_set_correction)", p->preconditioner);
    return GB300_ERR_ARG;
  }
  if(coarse && !coarse_valid(A)) {
    set_error("Preconditioner %d needs aggregates on the matrix pattern "
              "(gb300_matrix_set_aggregates)", p->preconditioner);
    return GB300_ERR_ARG;
  }
  bool fp32 = (p->precision != 0);
  const int imode = ilu_mode(p);
  if(precond) {
    int zr = 0;
    // the factor is on A's values as given to the solver (scaled if needed)
    GB_TRY(ilu_factor(A, val, fp32, &zr, p->re_use_lu != 0, &info->ilu_factorized));
    if(zr) {
      info->status = zr;
      set_error("Zero pivot on line %d in ILU", zr);
      return GB300_ERR_ZERO_PIVOT;
    }
  }
  if(coarse) GB_TRY(coarse_setup(A, val, p->re_use_lu != 0));
  size_t ldv = (size_t)n;
  double *V = (double *)W.vec(0, sizeof(double) * ldv * (m + 1));
  double *Z = flexible ? (double *)W.vec(1, sizeof(double) * ldv * m) : nullptr;
  double *r = (double *)W.vec(2, sizeof(double) * n);
  double *u = (double *)W.vec(3, sizeof(double) * n);
  double *zt = (double *)W.vec(4, sizeof(double) * n);
  float *t32 = fp32 ? (float *)W.vec(5, sizeof(float) * n) : nullptr;
  double *part = (double *)W.vec(6, sizeof(double) * kReduceBlocks * (m + 1));
  double *pn = (double *)W.vec(12, sizeof(double) * kReduceBlocks);
  GmState *S = (GmState *)W.state(sizeof(GmState));
  int *okflag = (int *)W.vec(7, sizeof(int));
  double *t1 = learned ? (double *)W.vec(8, sizeof(double) * n) : nullptr;
  double *t2 = learned ? (double *)W.vec(9, sizeof(double) * n) : nullptr;
  double *t3 = coarse ? (double *)W.vec(13, sizeof(double) * n) : nullptr;
  double *t4 = coarse ? (double *)W.vec(14, sizeof(double) * n) : nullptr;
  if(!V || (flexible && !Z) || !r || !u || !zt || (fp32 && !t32) || !part || !pn || !S ||
     (learned && (!t1 || !t2)) || (coarse && (!t3 || !t4)))
    return GB300_ERR_CUDA;
  GmState h0;
  memset(&h0, 0, sizeof(h0));
  h0.active = 1;
  h0.first = 1;
  h0.maxit = p->nb_iter_max;
  h0.rtol = p->stopping_test;
  h0.status = 1;
  GB_CUDA(cudaMemcpyAsync(S, &h0, sizeof(GmState), cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, st));  // sol = 0

  int gs = grid_for(n, 256, kReduceBlocks * 4);
  // partial-sum blocks of the Arnoldi dot products: one per SM at least,
  // one per 2048 rows up to kReduceBlocks (small systems keep the
  // one-block reductions short); fixed for a given n, so deterministic
  const int nb = std::min(kReduceBlocks, std::max(152, (n + 2047) / 2048));
  auto smooth = [&](const double *v, double *z, const int *flag, bool corr) {
    if(sai) {  // z = G v
      spmv_guarded(A, A->corr.p, v, z, flag, st);
      return;
    }
    if(precond)
      ilu_apply(A, imode, v, z, t32, flag, st);
    else
      k_cvt<double, double><<<grid_for(n, 256), 256, 0, st>>>(n, v, z, flag);
    if(corr) correction_apply(A, val, v, z, t1, t2, flag, st);
  };
  auto precond_apply = [&](const double *v, double *z, const int *flag) {
    if(!coarse) {
      smooth(v, z, flag, learned);
      return;
    }
    two_level_apply(A, val, v, z, t3, t4, flag, st,
                    [&](const double *vv, double *zz) { smooth(vv, zz, flag, learned); },
                    [&](const double *vv, double *zz) { smooth(vv, zz, flag, learned_post); });
  };

  cudaGraph_t graph;
  cudaGraphExec_t exec;
  GB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  // restart: r = rhs - A x, its norm, v1 = r / ||r||
  residual64(A, val, x, rhs, r, part, st);
  k_gm_restart<<<1, 256, 0, st>>>(S, part, m);
  k_gm_scale<<<gs, 256, 0, st>>>(n, S, r, V);
  for(int k = 1; k <= m; k++) {
    double *vk = V + (size_t)(k - 1) * ldv;
    double *w = V + (size_t)k * ldv;
    double *z = flexible ? Z + (size_t)(k - 1) * ldv : zt;
    precond_apply(vk, z, cycle_flag(S));
    spmv_guarded(A, val, z, w, &S->cycle, st);
    // classical Gram-Schmidt, a second pass only when the test after the
    // first asks for it; the reductions, the test and the end of the step
    // run in the last CTA of each kernel
    k_gm_dots<0><<<dim3(nb, (k + 1 + 7) / 8), 256, 0, st>>>(n, k, V, ldv, w, part, S, nb);
    k_gm_update<<<nb, 256, 0, st>>>(n, k, m, V, ldv, w, pn, S, 0, nb);
    k_gm_dots<1><<<dim3(nb, (k + 7) / 8), 256, 0, st>>>(n, k, V, ldv, w, part, S, nb);
    k_gm_update<<<nb, 256, 0, st>>>(n, k, m, V, ldv, w, pn, S, 1, nb);
    k_gm_scale_next<<<gs, 256, 0, st>>>(n, S, w, k);
  }
  k_gm_solve_small<<<1, 32, 0, st>>>(S);
  if(flexible)
    k_gm_combine<1><<<gs, 256, 0, st>>>(n, Z, ldv, x, S);
  else {
    k_gm_combine<0><<<gs, 256, 0, st>>>(n, V, ldv, u, S);
    k_gm_apply_ok<<<1, 32, 0, st>>>(S, okflag);
    precond_apply(u, zt, okflag);
    k_gm_addto<<<gs, 256, 0, st>>>(n, zt, x, S);
  }
  k_gm_after<<<1, 32, 0, st>>>(S);
  GB_CUDA(cudaStreamEndCapture(st, &graph));
  GB_CUDA(cudaGraphInstantiate(&exec, graph, 0));

  int active = 1, launches = 0;
  int max_launches = p->nb_iter_max > 0 ? p->nb_iter_max + 2 : 1 << 30;
  while(active && launches < max_launches) {
    GB_CUDA(cudaGraphLaunch(exec, st));
    launches++;
    GB_CUDA(cudaMemcpyAsync(&active, &S->active, sizeof(int),
                            cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  GB_CUDA(cudaMemcpyAsync(&h0, S, sizeof(GmState), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  info->status = active ? -1 : h0.status;
  info->iterations = h0.its;
  info->residual_estimate = h0.res6;
  return GB300_OK;
}

}  // namespace gb
