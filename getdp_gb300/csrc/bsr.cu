// Node-blocked (3 x 3 BSR) form of a vector-valued system for the CG solver.
//
// GetDP numbers the unknowns of a three-component field component by
// component (all ux, then uy, then uz: its DOF tree is keyed first by the
// basis function, DofData.cpp:36-45), so a CSR row of (node a, component i)
// holds three segments, one per component, each listing the same neighbour
// nodes.  The solver keeps the assembled CSR in that numbering and, for its
// own iterations, builds a node-major copy: one block row per node, one
// column index per 3 x 3 block, values in nine coalesced planes, vectors
// padded to four entries per node (16/32-byte gathers).  It is a private
// reordering of the solver, as Sparskit's RCMK renumbering is; results are
// permuted back.  The structure is verified while converting; a matrix that
// does not have it is solved in CSR.
#include <map>
#include <mutex>
#include <tuple>

#include "krylov.cuh"

namespace gb {

// one warp per block row a: rows a + c*nn (c = 0..2) of the CSR
__global__ void __launch_bounds__(256)
k_bsr_build(int nn, const int *__restrict__ rowptr, const int *__restrict__ col,
            const double *__restrict__ val, int *__restrict__ bcol,
            double *__restrict__ bval64, float *__restrict__ bval32,
            long long nblk, int *__restrict__ bad)
{
  int a = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if(a >= nn) return;
  int s0 = rowptr[a];
  int len = rowptr[a + 1] - s0;
  if(len % 3) {
    if(lane == 0) atomicExch(bad, 1);
    return;
  }
  int L = len / 3;
  int bs = s0 / 3;
  for(int c = 0; c < 3; c++) {
    int r = a + c * nn;
    if(rowptr[r + 1] - rowptr[r] != len) {
      if(lane == 0) atomicExch(bad, 1);
      return;
    }
  }
  for(int k = lane; k < L; k += 32) {
    int b = col[s0 + k];
    if(b < 0 || b >= nn) {
      atomicExch(bad, 1);
      continue;
    }
    bcol[bs + k] = b;
#pragma unroll
    for(int c = 0; c < 3; c++) {
      int rs = rowptr[a + c * nn];
#pragma unroll
      for(int cc = 0; cc < 3; cc++) {
        int pos = rs + cc * L + k;
        if(col[pos] != b + cc * nn) atomicExch(bad, 1);
        double v = val[pos];
        long long o = (long long)(c * 3 + cc) * nblk + bs + k;
        if(bval64) bval64[o] = v;
        if(bval32) bval32[o] = (float)v;
      }
    }
  }
}

__global__ void k_bsr_ptr(int nn, const int *__restrict__ rowptr,
                          int *__restrict__ bptr)
{
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if(a <= nn) bptr[a] = rowptr[a] / 3;
}

int bsr_build(const gb300_matrix *A, const double *val, bool want64,
              bool want32, Bsr3 &B)
{
  cudaStream_t st = A->ctx->stream;
  if(A->n % 3 || A->n == 0) return GB300_ERR_UNSUPPORTED;
  int nn = A->n / 3;
  long long nnz_c0 = 0;
  int h = 0;
  GB_CUDA(cudaMemcpyAsync(&h, A->rowptr.p + nn, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  nnz_c0 = h;  // entries of the component-0 rows
  if(nnz_c0 % 3 || nnz_c0 * 3 != A->nnz) return GB300_ERR_UNSUPPORTED;
  long long nblk = nnz_c0 / 3;
  B.nn = nn;
  B.nblk = nblk;
  // plane stride: a multiple of 4 entries plus slack, so that every bulk
  // copy of a 4-aligned block range starts and ends on 16 bytes
  B.pstride = ((nblk + 3) & ~3LL) + 4;
  GB_TRY(B.ptr.alloc(nn + 1));
  GB_TRY(B.col.alloc(B.pstride));
  if(want64) GB_TRY(B.val64.alloc(9 * B.pstride));
  if(want32) GB_TRY(B.val32.alloc(9 * B.pstride));
  GB_TRY(B.err.alloc(1));
  GB_CUDA(cudaMemsetAsync(B.err.p, 0, sizeof(int), st));
  DevBuf<int> bad;
  GB_TRY(bad.alloc(1));
  GB_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  k_bsr_ptr<<<grid_for(nn + 1, 256), 256, 0, st>>>(nn, A->rowptr.p, B.ptr.p);
  k_bsr_build<<<grid_for(nn, 8), 256, 0, st>>>(nn, A->rowptr.p, A->col.p, val,
                                                B.col.p, want64 ? B.val64.p : nullptr,
                                                want32 ? B.val32.p : nullptr, B.pstride,
                                                bad.p);
  GB_CUDA(cudaGetLastError());
  int hb = 0;
  GB_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  return hb ? GB300_ERR_UNSUPPORTED : GB300_OK;
}

// component-major (length 3 nn) <-> node-major padded (length 4 nn)
template <typename TO, typename TI>
__global__ void k_to_nodes(int nn, const TI *__restrict__ in, TO *__restrict__ out)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= nn) return;
  out[4 * i] = (TO)in[i];
  out[4 * i + 1] = (TO)in[i + nn];
  out[4 * i + 2] = (TO)in[i + 2 * nn];
  out[4 * i + 3] = (TO)0;
}

template <typename TO, typename TI>
__global__ void k_from_nodes(int nn, const TI *__restrict__ in, TO *__restrict__ out)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= nn) return;
  out[i] = (TO)in[4 * i];
  out[i + nn] = (TO)in[4 * i + 1];
  out[i + 2 * nn] = (TO)in[4 * i + 2];
}

void to_nodes64(int nn, const double *in, double *out, cudaStream_t st)
{
  k_to_nodes<double, double><<<grid_for(nn, 256), 256, 0, st>>>(nn, in, out);
}
void from_nodes64(int nn, const double *in, double *out, cudaStream_t st)
{
  k_from_nodes<double, double><<<grid_for(nn, 256), 256, 0, st>>>(nn, in, out);
}

template <typename T> struct Vec4;
template <> struct Vec4<float> {
  __device__ static float4 load(const float *p) { return __ldg((const float4 *)p); }
};
struct D4 {
  double x, y, z, w;
};
template <> struct Vec4<double> {
  __device__ static D4 load(const double *p)
  {
    double2 a = __ldg((const double2 *)p), b = __ldg((const double2 *)(p + 2));
    return D4{a.x, a.y, b.x, b.y};
  }
};

// y = A p over block rows, LPR lanes per block row (LPR consecutive blocks
// of a row are one 32-byte sector per value plane); MODE 2: partial
// <p, y>; MODE 1: y = b - A p with partial ||y||^2.  Guarded by *flag.
// matrix loads: CS = 1 streams them (evict-first), CS = 0 reads them through
// the read-only path with the default L2 policy, so that the other half of
// a DRAM burst is still cached when the next block of the row needs it
template <int CS, typename U> __device__ __forceinline__ U mload(const U *p)
{
  if(CS) return __ldcs(p);
  return __ldg(p);
}

template <typename T, int CS>
__device__ __forceinline__ void bsr_block(const int *__restrict__ col,
                                          const T *__restrict__ val,
                                          long long nblk, const T *__restrict__ p,
                                          int k, T &y0, T &y1, T &y2)
{
  int b = mload<CS>(col + k);
  auto xb = Vec4<T>::load(p + 4 * (size_t)b);
  if constexpr(sizeof(T) == 8) {
    // FP64: nine chained FMAs per block.  `y += a x + b y + c z` compiles to
    // a multiply, two FMAs and an add per row (12 FP64 instructions per
    // block instead of 9), and GB300's FP64 pipe (2 FMAs per SM per cycle)
    // bounds the FP64 product
    y0 = fma(mload<CS>(val + k), xb.x, y0);
    y1 = fma(mload<CS>(val + 3 * nblk + k), xb.x, y1);
    y2 = fma(mload<CS>(val + 6 * nblk + k), xb.x, y2);
    y0 = fma(mload<CS>(val + nblk + k), xb.y, y0);
    y1 = fma(mload<CS>(val + 4 * nblk + k), xb.y, y1);
    y2 = fma(mload<CS>(val + 7 * nblk + k), xb.y, y2);
    y0 = fma(mload<CS>(val + 2 * nblk + k), xb.z, y0);
    y1 = fma(mload<CS>(val + 5 * nblk + k), xb.z, y1);
    y2 = fma(mload<CS>(val + 8 * nblk + k), xb.z, y2);
  }
  else {
    // FP32 (memory bound): each row's three products first, then one add
    // (measured faster than the chained form: 0.2036 against 0.2096 ms per
    // launch at 48^3)
    y0 += mload<CS>(val + k) * xb.x + mload<CS>(val + nblk + k) * xb.y +
          mload<CS>(val + 2 * nblk + k) * xb.z;
    y1 += mload<CS>(val + 3 * nblk + k) * xb.x + mload<CS>(val + 4 * nblk + k) * xb.y +
          mload<CS>(val + 5 * nblk + k) * xb.z;
    y2 += mload<CS>(val + 6 * nblk + k) * xb.x + mload<CS>(val + 7 * nblk + k) * xb.y +
          mload<CS>(val + 8 * nblk + k) * xb.z;
  }
}

// MINB: CTAs per SM the register allocation must allow (0 = the compiler's
// own choice).  The grid is the number of CTAs that are resident at once
// (resident_grid), so no CTA waits for a second wave.
template <int MODE, typename T, int LPR, int UNR, int CS, int MINB = 0>
__global__ void __launch_bounds__(256, MINB)
k_bsr_spmv(int nn, const int *__restrict__ ptr, const int *__restrict__ col,
           const T *__restrict__ val, long long nblk, const T *__restrict__ p,
           const T *__restrict__ bvec, T *__restrict__ y,
           double *__restrict__ part, const int *flag, double *dot_out,
           unsigned *counter)
{
  if(flag && !*flag) return;
  const int rows_per_block = 256 / LPR;
  int lane = threadIdx.x % LPR, sub = threadIdx.x / LPR;
  typename Acc<T>::type red = 0;
  for(long long a0 = (long long)blockIdx.x * rows_per_block; a0 < nn;
      a0 += (long long)gridDim.x * rows_per_block) {
    long long a = a0 + sub;
    T y0 = 0, y1 = 0, y2 = 0;
    if(a < nn) {
      int s = ptr[a], e = ptr[a + 1];
      int k = s + lane;
      for(; k + (UNR - 1) * LPR < e; k += UNR * LPR) {  // UNR blocks in flight
#pragma unroll
        for(int u = 0; u < UNR; u++)
          bsr_block<T, CS>(col, val, nblk, p, k + u * LPR, y0, y1, y2);
      }
      for(; k < e; k += LPR) bsr_block<T, CS>(col, val, nblk, p, k, y0, y1, y2);
    }
#pragma unroll
    for(int o = LPR / 2; o > 0; o >>= 1) {
      y0 += __shfl_down_sync(0xffffffffu, y0, o, LPR);
      y1 += __shfl_down_sync(0xffffffffu, y1, o, LPR);
      y2 += __shfl_down_sync(0xffffffffu, y2, o, LPR);
    }
    if(lane == 0 && a < nn) {
      size_t o = 4 * (size_t)a;
      if(MODE == 1) {
        T r0 = bvec[o] - y0, r1 = bvec[o + 1] - y1, r2 = bvec[o + 2] - y2;
        y[o] = r0;
        y[o + 1] = r1;
        y[o + 2] = r2;
        y[o + 3] = 0;
        red += r0 * r0 + r1 * r1 + r2 * r2;
      }
      else {
        y[o] = y0;
        y[o + 1] = y1;
        y[o + 2] = y2;
        y[o + 3] = 0;
        if(MODE == 2)
          red += p[o] * y0 + p[o + 1] * y1 + p[o + 2] * y2;
      }
    }
  }
  if(MODE != 0) {
    double s = block_sum<double, 256>((double)red);
    if(threadIdx.x == 0) part[blockIdx.x] = s;
    // the consumers sum a fixed number of partials
    if(blockIdx.x == 0)
      for(int b = gridDim.x + threadIdx.x; b < kReduceBlocks; b += blockDim.x)
        part[b] = 0.;
    // MODE 2 with dot_out: the last block to finish sums <p, y> itself
    if(MODE == 2 && dot_out && arrive_last(counter)) {
      double d = sum_partials_l2<256>(part);
      if(threadIdx.x == 0) *dot_out = d;
    }
  }
}

// Column indices one step ahead: in k_bsr_spmv a lane waits for a block's
// column index before it can gather x, then for the gather, so each group
// of blocks costs two memory latencies.  Here the column indices of a
// lane's next UNR blocks are loaded while the current blocks' values and x
// gathers are in flight (their columns were loaded the step before), and
// the next block row's bounds while the current row runs: one latency per
// group of blocks.  Same arithmetic and order as k_bsr_spmv.
template <int MODE, typename T, int LPR, int UNR, int MINB = 0>
__global__ void __launch_bounds__(256, MINB)
k_bsr_spmv_pf(int nn, const int *__restrict__ ptr, const int *__restrict__ col,
              const T *__restrict__ val, long long nblk, const T *__restrict__ p,
              const T *__restrict__ bvec, T *__restrict__ y,
              double *__restrict__ part, const int *flag, double *dot_out,
              unsigned *counter)
{
  if(flag && !*flag) return;
  const int rows_per_block = 256 / LPR;
  const long long stride = (long long)gridDim.x * rows_per_block;
  int lane = threadIdx.x % LPR, sub = threadIdx.x / LPR;
  typename Acc<T>::type red = 0;
  long long a0 = (long long)blockIdx.x * rows_per_block;
  int s = 0, e = 0;
  if(a0 + sub < nn) {
    s = __ldg(ptr + a0 + sub);
    e = __ldg(ptr + a0 + sub + 1);
  }
  for(; a0 < nn; a0 += stride) {
    long long a = a0 + sub;
    // the next row's bounds
    int sn = 0, en = 0;
    if(a + stride < nn) {
      sn = __ldg(ptr + a + stride);
      en = __ldg(ptr + a + stride + 1);
    }
    T y0 = 0, y1 = 0, y2 = 0;
    if(a < nn) {
      int k = s + lane;
      int c[UNR];
#pragma unroll
      for(int u = 0; u < UNR; u++) {
        int kk = k + u * LPR;
        c[u] = kk < e ? __ldg(col + kk) : 0;
      }
      for(; k < e; k += UNR * LPR) {
        int cn[UNR];
#pragma unroll
        for(int u = 0; u < UNR; u++) {
          int kk = k + (UNR + u) * LPR;
          cn[u] = kk < e ? __ldg(col + kk) : 0;
        }
#pragma unroll
        for(int u = 0; u < UNR; u++) {
          int kk = k + u * LPR;
          if(kk < e) {
            auto xb = Vec4<T>::load(p + 4 * (size_t)c[u]);
            if constexpr(sizeof(T) == 8) {
              y0 = fma(__ldg(val + kk), xb.x, y0);
              y1 = fma(__ldg(val + 3 * nblk + kk), xb.x, y1);
              y2 = fma(__ldg(val + 6 * nblk + kk), xb.x, y2);
              y0 = fma(__ldg(val + nblk + kk), xb.y, y0);
              y1 = fma(__ldg(val + 4 * nblk + kk), xb.y, y1);
              y2 = fma(__ldg(val + 7 * nblk + kk), xb.y, y2);
              y0 = fma(__ldg(val + 2 * nblk + kk), xb.z, y0);
              y1 = fma(__ldg(val + 5 * nblk + kk), xb.z, y1);
              y2 = fma(__ldg(val + 8 * nblk + kk), xb.z, y2);
            }
            else {
              y0 += __ldg(val + kk) * xb.x + __ldg(val + nblk + kk) * xb.y +
                    __ldg(val + 2 * nblk + kk) * xb.z;
              y1 += __ldg(val + 3 * nblk + kk) * xb.x + __ldg(val + 4 * nblk + kk) * xb.y +
                    __ldg(val + 5 * nblk + kk) * xb.z;
              y2 += __ldg(val + 6 * nblk + kk) * xb.x + __ldg(val + 7 * nblk + kk) * xb.y +
                    __ldg(val + 8 * nblk + kk) * xb.z;
            }
          }
        }
#pragma unroll
        for(int u = 0; u < UNR; u++) c[u] = cn[u];
      }
    }
    s = sn;
    e = en;
#pragma unroll
    for(int o = LPR / 2; o > 0; o >>= 1) {
      y0 += __shfl_down_sync(0xffffffffu, y0, o, LPR);
      y1 += __shfl_down_sync(0xffffffffu, y1, o, LPR);
      y2 += __shfl_down_sync(0xffffffffu, y2, o, LPR);
    }
    if(lane == 0 && a < nn) {
      size_t o = 4 * (size_t)a;
      if(MODE == 1) {
        T r0 = bvec[o] - y0, r1 = bvec[o + 1] - y1, r2 = bvec[o + 2] - y2;
        y[o] = r0;
        y[o + 1] = r1;
        y[o + 2] = r2;
        y[o + 3] = 0;
        red += r0 * r0 + r1 * r1 + r2 * r2;
      }
      else {
        y[o] = y0;
        y[o + 1] = y1;
        y[o + 2] = y2;
        y[o + 3] = 0;
        if(MODE == 2) red += p[o] * y0 + p[o + 1] * y1 + p[o + 2] * y2;
      }
    }
  }
  if(MODE != 0) {
    double sm = block_sum<double, 256>((double)red);
    if(threadIdx.x == 0) part[blockIdx.x] = sm;
    if(blockIdx.x == 0)
      for(int b = gridDim.x + threadIdx.x; b < kReduceBlocks; b += blockDim.x)
        part[b] = 0.;
    if(MODE == 2 && dot_out && arrive_last(counter)) {
      double d = sum_partials_l2<256>(part);
      if(threadIdx.x == 0) *dot_out = d;
    }
  }
}

// ---------------------------------------------------------------------------
// TMA-staged variant: each CTA walks tiles of kTileRows block rows; one
// elected thread copies a tile's nine value planes and column indices from
// HBM to shared memory with cp.async.bulk (completion counted on an
// mbarrier), two tiles in flight; all threads compute from shared memory,
// so only the x gathers (L2-resident vectors) still wait on memory.
// Bulk copies need 16-byte aligned addresses and sizes: tile ranges are
// widened to multiples of four blocks (planes are padded accordingly).
// Every wait is bounded; on time-out the CTA records an error, waits
// (bounded) for its own copies and returns.
// ---------------------------------------------------------------------------
constexpr int kTileRows = 16;
constexpr int kTileCap = 1024;  // blocks per tile (+4 alignment slack)
constexpr int kTmaThreads = 256;
constexpr long long kWaitLimit = 1LL << 26;

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, int count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar,
                                               unsigned bytes)
{
  asm volatile(
    "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
    "r"(bytes)
    : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src,
                                         unsigned bytes, unsigned long long *bar)
{
  asm volatile(
    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
    "[%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
    "l"(src), "r"(bytes), "r"(smem_addr(bar))
    : "memory");
}

// true when the phase with the given parity has completed
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar,
                                              unsigned parity)
{
  unsigned ok;
  asm volatile(
    "{\n .reg .pred p;\n"
    " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
    " selp.u32 %0, 1, 0, p;\n}"
    : "=r"(ok)
    : "r"(smem_addr(bar)), "r"(parity)
    : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar,
                                                  unsigned parity)
{
  for(long long i = 0; i < kWaitLimit; i++)
    if(mbar_try_wait(bar, parity)) return true;
  return false;
}

template <typename T> struct TmaTile {
  T val[9][kTileCap + 4];
  int col[kTileCap + 4];
};

template <int MODE, typename T, int LPR>
__global__ void __launch_bounds__(kTmaThreads)
k_bsr_spmv_tma(int nn, const int *__restrict__ ptr, const int *__restrict__ col,
               const T *__restrict__ val, long long pstride,
               const T *__restrict__ p, const T *__restrict__ bvec,
               T *__restrict__ y, double *__restrict__ part, const int *flag,
               int *__restrict__ err, double *dot_out, unsigned *counter)
{
  if(flag && !*flag) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TmaTile<T> *stage = (TmaTile<T> *)smem_raw;
  __shared__ __align__(8) unsigned long long bar[2];
  __shared__ int tile_k0[2], tile_n[2];  // aligned first block, blocks copied
  __shared__ int in_flight[2];  // a copy into the stage has not been waited for
  const int ntiles = (nn + kTileRows - 1) / kTileRows;
  const int tid = threadIdx.x;

  if(tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    in_flight[0] = in_flight[1] = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  // thread 0 issues the copies of tile t into stage s (or marks it direct)
  auto issue = [&](int t, int s) {
    int r0 = t * kTileRows;
    int r1 = min(r0 + kTileRows, nn);
    int k0 = ptr[r0], k1 = ptr[r1];
    int k0a = k0 & ~3, k1a = (k1 + 3) & ~3;
    int nb = k1a - k0a;
    tile_k0[s] = k0a;
    if(nb > kTileCap + 4 || nb <= 0) {
      tile_n[s] = -1;  // too long for the stage: read this tile directly
      return;
    }
    tile_n[s] = nb;
    in_flight[s] = 1;
    unsigned bytes = (unsigned)(9 * nb * sizeof(T) + nb * sizeof(int));
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&bar[s], bytes);
    for(int c = 0; c < 9; c++)
      bulk_g2s(stage[s].val[c], val + c * pstride + k0a, nb * sizeof(T), &bar[s]);
    bulk_g2s(stage[s].col, col + k0a, nb * sizeof(int), &bar[s]);
  };

  int t0 = blockIdx.x;
  if(tid == 0) {
    if(t0 < ntiles) issue(t0, 0);
    if(t0 + gridDim.x < ntiles) issue(t0 + gridDim.x, 1);
  }
  __syncthreads();

  const int lane = tid % LPR, sub = tid / LPR;
  const int rows_per_pass = kTmaThreads / LPR;
  double red = 0.;
  unsigned phase[2] = {0u, 0u};
  int i = 0;
  bool failed = false;
  for(int t = t0; t < ntiles; t += gridDim.x, i++) {
    int s = i & 1;
    bool direct = tile_n[s] < 0;
    if(!direct) {
      bool ok = mbar_wait_bounded(&bar[s], phase[s]);
      if(__syncthreads_or(!ok)) {
        failed = true;
        break;
      }
      phase[s] ^= 1u;
      if(tid == 0) in_flight[s] = 0;  // read again only after the next issue
    }
    int k0a = tile_k0[s];
    const T *sv = stage[s].val[0];
    int r0 = t * kTileRows, r1 = min(r0 + kTileRows, nn);
    for(int a = r0 + sub; a - sub < r1; a += rows_per_pass) {
      T y0 = 0, y1 = 0, y2 = 0;
      if(a < r1) {
        int s0 = ptr[a], e0 = ptr[a + 1];
        for(int k = s0 + lane; k < e0; k += LPR) {
          int b;
          T v[9];
          if(!direct) {
            int kk = k - k0a;
            b = stage[s].col[kk];
#pragma unroll
            for(int c = 0; c < 9; c++) v[c] = sv[c * (kTileCap + 4) + kk];
          }
          else {
            b = __ldg(col + k);
#pragma unroll
            for(int c = 0; c < 9; c++) v[c] = __ldg(val + c * pstride + k);
          }
          auto xb = Vec4<T>::load(p + 4 * (size_t)b);
          y0 = fma(v[0], xb.x, y0);
          y1 = fma(v[3], xb.x, y1);
          y2 = fma(v[6], xb.x, y2);
          y0 = fma(v[1], xb.y, y0);
          y1 = fma(v[4], xb.y, y1);
          y2 = fma(v[7], xb.y, y2);
          y0 = fma(v[2], xb.z, y0);
          y1 = fma(v[5], xb.z, y1);
          y2 = fma(v[8], xb.z, y2);
        }
      }
#pragma unroll
      for(int o = LPR / 2; o > 0; o >>= 1) {
        y0 += __shfl_down_sync(0xffffffffu, y0, o, LPR);
        y1 += __shfl_down_sync(0xffffffffu, y1, o, LPR);
        y2 += __shfl_down_sync(0xffffffffu, y2, o, LPR);
      }
      if(lane == 0 && a < r1) {
        size_t o = 4 * (size_t)a;
        if(MODE == 1) {
          T q0 = bvec[o] - y0, q1 = bvec[o + 1] - y1, q2 = bvec[o + 2] - y2;
          y[o] = q0;
          y[o + 1] = q1;
          y[o + 2] = q2;
          y[o + 3] = 0;
          red += (double)q0 * q0 + (double)q1 * q1 + (double)q2 * q2;
        }
        else {
          y[o] = y0;
          y[o + 1] = y1;
          y[o + 2] = y2;
          y[o + 3] = 0;
          if(MODE == 2)
            red += (double)p[o] * y0 + (double)p[o + 1] * y1 + (double)p[o + 2] * y2;
        }
      }
    }
    __syncthreads();  // every thread is done with stage s
    if(tid == 0 && t + 2 * (int)gridDim.x < ntiles) issue(t + 2 * gridDim.x, s);
    __syncthreads();
  }
  if(failed) {
    // record, then let the copies still in flight land before leaving (only
    // stages with a copy issued and not yet waited for: a stage whose tile
    // was consumed has no phase left to complete)
    if(tid == 0) {
      atomicExch(err, 1);
      for(int s = 0; s < 2; s++)
        if(in_flight[s]) mbar_wait_bounded(&bar[s], phase[s]);
    }
    __syncthreads();
    red = 0.;  // the result is void (err is set); keep the reduction whole
  }
  if(MODE != 0) {
    double s = block_sum<double, kTmaThreads>(red);
    if(tid == 0) part[blockIdx.x] = s;
    // the consumers sum a fixed number of partials
    if(blockIdx.x == 0)
      for(int b = gridDim.x + tid; b < kReduceBlocks; b += blockDim.x) part[b] = 0.;
    if(MODE == 2 && dot_out && arrive_last(counter)) {
      double d = sum_partials_l2<kTmaThreads>(part);
      if(tid == 0) *dot_out = d;
    }
  }
}

// launch shapes the tuner chooses from, as (lanes per block row, blocks in
// flight per lane, streaming loads, CTAs per SM the registers must allow):
// 0 (8,2,cs) 1 (8,2,ldg) 2 (16,2,cs) 3 (16,2,ldg) 4 (8,4,ldg) 5 (32,2,ldg);
// 6 and 7: the TMA-staged kernel with 16 and 8 lanes per block row;
// 8 (8,2,ldg,8 CTAs) 9 (8,4,ldg,4 CTAs) 10 (8,2,ldg,4 CTAs); fewer lanes
// per block row, for the FP64 product whose shuffle-add tree and idle lanes
// load GB300's FP64 pipe: 11 (4,2,ldg) 12 (4,4,ldg) 13 (2,4,ldg); column
// indices one step ahead (k_bsr_spmv_pf): 14 (8,2) 15 (8,4) 16 (4,4)
// 17 (4,2) 18 (8,2,8 CTAs)
constexpr int kBsrVariants = 19;

template <int MODE, typename T, int LPR>
static void launch_tma(const Bsr3 &B, const T *val, const T *p, const T *b,
                       T *y, double *part, const int *flag, double *dot_out,
                       unsigned *counter, cudaStream_t st)
{
  size_t smem = 2 * sizeof(TmaTile<T>);
  static int grid = 0;  // per instantiation
  if(!grid) {
    cudaFuncSetAttribute(k_bsr_spmv_tma<MODE, T, LPR>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    grid = resident_grid(k_bsr_spmv_tma<MODE, T, LPR>, kTmaThreads, smem);
  }
  k_bsr_spmv_tma<MODE, T, LPR><<<grid, kTmaThreads, smem, st>>>(
    B.nn, B.ptr.p, B.col.p, val, B.pstride, p, b, y, part, flag, B.err.p,
    dot_out, counter);
}

template <int MODE, typename T, int L, int U, int C, int M>
static void launch_plain(const Bsr3 &B, const T *val, const T *p, const T *b,
                         T *y, double *part, const int *flag, double *dot_out,
                         unsigned *counter, cudaStream_t st)
{
  static int grid = 0;  // per instantiation
  if(!grid) grid = resident_grid(k_bsr_spmv<MODE, T, L, U, C, M>, 256, 0);
  k_bsr_spmv<MODE, T, L, U, C, M><<<grid, 256, 0, st>>>(
    B.nn, B.ptr.p, B.col.p, val, B.pstride, p, b, y, part, flag, dot_out, counter);
}

template <int MODE, typename T, int L, int U, int M>
static void launch_pf(const Bsr3 &B, const T *val, const T *p, const T *b, T *y,
                      double *part, const int *flag, double *dot_out, unsigned *counter,
                      cudaStream_t st)
{
  static int grid = 0;  // per instantiation
  if(!grid) grid = resident_grid(k_bsr_spmv_pf<MODE, T, L, U, M>, 256, 0);
  k_bsr_spmv_pf<MODE, T, L, U, M><<<grid, 256, 0, st>>>(
    B.nn, B.ptr.p, B.col.p, val, B.pstride, p, b, y, part, flag, dot_out, counter);
}

template <int MODE, typename T>
static void launch_bsr(int variant, const Bsr3 &B, const T *val, const T *p,
                       const T *b, T *y, double *part, const int *flag,
                       cudaStream_t st, double *dot_out = nullptr,
                       unsigned *counter = nullptr)
{
#define GB_BSR(L, U, C, M) \
  launch_plain<MODE, T, L, U, C, M>(B, val, p, b, y, part, flag, dot_out, counter, st)
  switch(variant) {
  case 6: launch_tma<MODE, T, 16>(B, val, p, b, y, part, flag, dot_out, counter, st); break;
  case 7: launch_tma<MODE, T, 8>(B, val, p, b, y, part, flag, dot_out, counter, st); break;
  case 1: GB_BSR(8, 2, 0, 0); break;
  case 2: GB_BSR(16, 2, 1, 0); break;
  case 3: GB_BSR(16, 2, 0, 0); break;
  case 4: GB_BSR(8, 4, 0, 0); break;
  case 5: GB_BSR(32, 2, 0, 0); break;
  case 8: GB_BSR(8, 2, 0, 8); break;
  case 9: GB_BSR(8, 4, 0, 4); break;
  case 10: GB_BSR(8, 2, 0, 4); break;
  case 11: GB_BSR(4, 2, 0, 0); break;
  case 12: GB_BSR(4, 4, 0, 0); break;
  case 13: GB_BSR(2, 4, 0, 0); break;
  case 14: launch_pf<MODE, T, 8, 2, 0>(B, val, p, b, y, part, flag, dot_out, counter, st); break;
  case 15: launch_pf<MODE, T, 8, 4, 0>(B, val, p, b, y, part, flag, dot_out, counter, st); break;
  case 16: launch_pf<MODE, T, 4, 4, 0>(B, val, p, b, y, part, flag, dot_out, counter, st); break;
  case 17: launch_pf<MODE, T, 4, 2, 0>(B, val, p, b, y, part, flag, dot_out, counter, st); break;
  case 18: launch_pf<MODE, T, 8, 2, 8>(B, val, p, b, y, part, flag, dot_out, counter, st); break;
  default: GB_BSR(8, 2, 1, 0); break;
  }
#undef GB_BSR
}

void bsr_spmv_dot32(const Bsr3 &B, const float *p, float *q, double *part,
                    const int *flag, double *dot_out, unsigned *counter,
                    cudaStream_t st)
{
  launch_bsr<2, float>(B.var32, B, B.val32.p, p, nullptr, q, part, flag, st,
                       dot_out, counter);
}
void bsr_spmv_dot64(const Bsr3 &B, const double *p, double *q, double *part,
                    const int *flag, double *dot_out, unsigned *counter,
                    cudaStream_t st)
{
  launch_bsr<2, double>(B.var64, B, B.val64.p, p, nullptr, q, part, flag, st,
                        dot_out, counter);
}
void bsr_residual64(const Bsr3 &B, const double *x, const double *b, double *r,
                    double *part, const int *flag, cudaStream_t st)
{
  launch_bsr<1, double>(B.var64, B, B.val64.p, x, b, r, part, flag, st);
}

// The staged (TMA) variants report a bulk copy that did not complete within
// its bounded wait through B.err, leaving that product incomplete; a solve
// that ran one of them checks the flag once at its end.
int bsr_check(const Bsr3 &B, cudaStream_t st)
{
  bool staged = (B.val32.p && (B.var32 == 6 || B.var32 == 7)) ||
                (B.val64.p && (B.var64 == 6 || B.var64 == 7));
  if(!staged || !B.err.p) return GB300_OK;
  int he = 0;
  GB_CUDA(cudaMemcpyAsync(&he, B.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(he) {
    set_error("block SpMV: a staged copy did not complete within its wait limit");
    return GB300_ERR_CUDA;
  }
  return GB300_OK;
}

template <typename T>
__global__ void k_tune_fill(size_t n4, T *a, T *b)
{
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n4) return;
  bool pad = (i & 3) == 3;
  a[i] = pad ? (T)0 : (T)(1.0 + 0.125 * (double)(i % 7));
  b[i] = pad ? (T)0 : (T)(0.5 - 0.0625 * (double)(i % 5));
}

// flags a result that differs from the reference beyond tol * max|ref|
template <typename T>
__global__ void k_tune_check(size_t n4, const T *q, const T *ref, double scale,
                             double tol, int *bad)
{
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n4) return;
  double d = fabs((double)q[i] - (double)ref[i]);
  if(!(d <= tol * scale)) atomicExch(bad, 1);
}

// max |q_i| (bits of a non-negative double): grid stride, warp shuffles,
// one atomic per warp
template <typename T>
__global__ void k_absmax(size_t n4, const T *q, unsigned long long *out)
{
  unsigned long long m = 0;
  for(size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4;
      i += (size_t)gridDim.x * blockDim.x) {
    const unsigned long long b =
      (unsigned long long)__double_as_longlong(fabs((double)q[i]));
    m = b > m ? b : m;
  }
  for(int o = 16; o > 0; o >>= 1) {
    const unsigned long long u = __shfl_down_sync(0xffffffffu, m, o);
    m = u > m ? u : m;
  }
  if((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// Times every launch shape on this matrix (alternating between two input
// vectors, as in a CG where p changes every step) and keeps the fastest of
// those whose result matches the plain kernel's (a variant that disagrees,
// or whose staged copies time out, is never chosen).
template <typename T>
static int tune_one(Bsr3 &B, const T *val, int *out, cudaStream_t st)
{
  size_t n4 = 4 * (size_t)B.nn;
  DevBuf<T> pa, pb, q, qref;
  DevBuf<double> part;
  DevBuf<int> bad;
  DevBuf<unsigned long long> amax;
  GB_TRY(pa.alloc(n4));
  GB_TRY(pb.alloc(n4));
  GB_TRY(q.alloc(n4));
  GB_TRY(qref.alloc(n4));
  GB_TRY(part.alloc(kReduceBlocks));
  GB_TRY(bad.alloc(1));
  GB_TRY(amax.alloc(1));
  k_tune_fill<T><<<grid_for((long long)n4, 256), 256, 0, st>>>(n4, pa.p, pb.p);
  // the reference: the plain (non-staged) kernel, variant 1
  launch_bsr<2, T>(1, B, val, pa.p, nullptr, qref.p, part.p, nullptr, st);
  GB_CUDA(cudaMemsetAsync(amax.p, 0, sizeof(unsigned long long), st));
  k_absmax<T><<<grid_for((long long)n4, 256, kReduceBlocks * 4), 256, 0, st>>>(n4, qref.p,
                                                                                amax.p);
  unsigned long long hmax = 0;
  GB_CUDA(cudaMemcpyAsync(&hmax, amax.p, sizeof(hmax), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  double scale;
  memcpy(&scale, &hmax, sizeof(scale));
  double tol = sizeof(T) == 4 ? 1e-4 : 1e-12;
  cudaEvent_t e0, e1;
  GB_CUDA(cudaEventCreate(&e0));
  GB_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int bestv = 1;
  for(int v = 0; v < kBsrVariants; v++) {
    GB_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
    GB_CUDA(cudaMemsetAsync(B.err.p, 0, sizeof(int), st));
    launch_bsr<2, T>(v, B, val, pa.p, nullptr, q.p, part.p, nullptr, st);
    k_tune_check<T><<<grid_for((long long)n4, 256), 256, 0, st>>>(n4, q.p, qref.p,
                                                                 scale, tol, bad.p);
    int hb = 0, he = 0;
    GB_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaMemcpyAsync(&he, B.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    GB_CUDA(cudaGetLastError());
    if(hb || he) {
      if(getenv("GB300_TUNE_VERBOSE"))
        fprintf(stderr, "bsr spmv variant %d rejected (%s)\n", v,
                hb ? "result differs" : "staged copy timed out");
      continue;
    }
    GB_CUDA(cudaEventRecord(e0, st));
    for(int r = 0; r < 6; r++)
      launch_bsr<2, T>(v, B, val, (r & 1) ? pb.p : pa.p, nullptr, q.p, part.p,
                       nullptr, st);
    GB_CUDA(cudaEventRecord(e1, st));
    GB_CUDA(cudaEventSynchronize(e1));
    float t = 0.f;
    GB_CUDA(cudaEventElapsedTime(&t, e0, e1));
    if(getenv("GB300_TUNE_VERBOSE"))
      fprintf(stderr, "bsr spmv %s variant %d: %.4f ms\n",
              sizeof(T) == 4 ? "fp32" : "fp64", v, t / 6);
    if(t < best) {
      best = t;
      bestv = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *out = bestv;
  return GB300_OK;
}

// launch shapes already chosen, by (device, block rows, blocks, value size):
// a matrix re-generated with the same structure is not tuned again
static std::mutex g_tune_mutex;
static std::map<std::tuple<int, int, long long, int>, int> g_tuned;

template <typename T>
static int tune_cached(Bsr3 &B, const T *val, int *out, cudaStream_t st)
{
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  auto key = std::make_tuple(dev, B.nn, B.nblk, (int)sizeof(T));
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tuned.find(key);
    if(it != g_tuned.end()) {
      *out = it->second;
      return GB300_OK;
    }
  }
  GB_TRY(tune_one<T>(B, val, out, st));
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  g_tuned[key] = *out;
  return GB300_OK;
}

int bsr_tune(gb300_matrix *A, Bsr3 &B, cudaStream_t st, bool tune64)
{
  if(B.val32.p) {
    if(A->bsr_var32 < 0) GB_TRY(tune_cached<float>(B, B.val32.p, &A->bsr_var32, st));
    B.var32 = A->bsr_var32;
  }
  if(B.val64.p) {
    // FP64 products that only recompute a residual now and then keep the
    // default shape (4 lanes per block row: the FP64 pipe, not the memory,
    // limits wider lane groups); tuning them would cost more than it saves
    if(A->bsr_var64 < 0 && tune64)
      GB_TRY(tune_cached<double>(B, B.val64.p, &A->bsr_var64, st));
    B.var64 = A->bsr_var64 < 0 ? 11 : A->bsr_var64;
  }
  return GB300_OK;
}

}  // namespace gb
