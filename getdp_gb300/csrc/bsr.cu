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
  GB_TRY(B.ptr.alloc(nn + 1));
  GB_TRY(B.col.alloc(nblk > 0 ? nblk : 1));
  if(want64) GB_TRY(B.val64.alloc(9 * (nblk > 0 ? nblk : 1)));
  if(want32) GB_TRY(B.val32.alloc(9 * (nblk > 0 ? nblk : 1)));
  DevBuf<int> bad;
  GB_TRY(bad.alloc(1));
  GB_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  k_bsr_ptr<<<grid_for(nn + 1, 256), 256, 0, st>>>(nn, A->rowptr.p, B.ptr.p);
  k_bsr_build<<<grid_for(nn, 8), 256, 0, st>>>(nn, A->rowptr.p, A->col.p, val,
                                                B.col.p, want64 ? B.val64.p : nullptr,
                                                want32 ? B.val32.p : nullptr, nblk,
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
  y0 += mload<CS>(val + k) * xb.x + mload<CS>(val + nblk + k) * xb.y +
        mload<CS>(val + 2 * nblk + k) * xb.z;
  y1 += mload<CS>(val + 3 * nblk + k) * xb.x + mload<CS>(val + 4 * nblk + k) * xb.y +
        mload<CS>(val + 5 * nblk + k) * xb.z;
  y2 += mload<CS>(val + 6 * nblk + k) * xb.x + mload<CS>(val + 7 * nblk + k) * xb.y +
        mload<CS>(val + 8 * nblk + k) * xb.z;
}

template <int MODE, typename T, int LPR, int UNR, int CS>
__global__ void __launch_bounds__(256)
k_bsr_spmv(int nn, const int *__restrict__ ptr, const int *__restrict__ col,
           const T *__restrict__ val, long long nblk, const T *__restrict__ p,
           const T *__restrict__ bvec, T *__restrict__ y,
           double *__restrict__ part, const int *flag)
{
  if(flag && !*flag) return;
  const int rows_per_block = 256 / LPR;
  int lane = threadIdx.x % LPR, sub = threadIdx.x / LPR;
  double red = 0.;
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
        red += (double)r0 * r0 + (double)r1 * r1 + (double)r2 * r2;
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
  if(MODE != 0) {
    double s = block_sum<double, 256>(red);
    if(threadIdx.x == 0) part[blockIdx.x] = s;
  }
}

// launch shapes the tuner chooses from, as (lanes per block row, blocks in
// flight per lane, streaming loads): 0 (8,2,cs) 1 (8,2,ldg) 2 (16,2,cs)
// 3 (16,2,ldg) 4 (8,4,ldg) 5 (32,2,ldg)
constexpr int kBsrVariants = 6;

template <int MODE, typename T>
static void launch_bsr(int variant, const Bsr3 &B, const T *val, const T *p,
                       const T *b, T *y, double *part, const int *flag,
                       cudaStream_t st)
{
#define GB_BSR(L, U, C)                                                       \
  k_bsr_spmv<MODE, T, L, U, C><<<kReduceBlocks, 256, 0, st>>>(               \
    B.nn, B.ptr.p, B.col.p, val, B.nblk, p, b, y, part, flag)
  switch(variant) {
  case 1: GB_BSR(8, 2, 0); break;
  case 2: GB_BSR(16, 2, 1); break;
  case 3: GB_BSR(16, 2, 0); break;
  case 4: GB_BSR(8, 4, 0); break;
  case 5: GB_BSR(32, 2, 0); break;
  default: GB_BSR(8, 2, 1); break;
  }
#undef GB_BSR
}

void bsr_spmv_dot32(const Bsr3 &B, const float *p, float *q, double *part,
                    const int *flag, cudaStream_t st)
{
  launch_bsr<2, float>(B.var32, B, B.val32.p, p, nullptr, q, part, flag, st);
}
void bsr_spmv_dot64(const Bsr3 &B, const double *p, double *q, double *part,
                    const int *flag, cudaStream_t st)
{
  launch_bsr<2, double>(B.var64, B, B.val64.p, p, nullptr, q, part, flag, st);
}
void bsr_residual64(const Bsr3 &B, const double *x, const double *b, double *r,
                    double *part, const int *flag, cudaStream_t st)
{
  launch_bsr<1, double>(B.var64, B, B.val64.p, x, b, r, part, flag, st);
}

// Times every launch shape on this matrix (alternating between two input
// vectors, as in a CG where p changes every step) and keeps the fastest.
template <typename T>
static int tune_one(Bsr3 &B, const T *val, int *out, cudaStream_t st)
{
  size_t n4 = 4 * (size_t)B.nn;
  DevBuf<T> pa, pb, q;
  DevBuf<double> part;
  GB_TRY(pa.alloc(n4));
  GB_TRY(pb.alloc(n4));
  GB_TRY(q.alloc(n4));
  GB_TRY(part.alloc(kReduceBlocks));
  GB_CUDA(cudaMemsetAsync(pa.p, 0, n4 * sizeof(T), st));
  GB_CUDA(cudaMemsetAsync(pb.p, 0, n4 * sizeof(T), st));
  cudaEvent_t e0, e1;
  GB_CUDA(cudaEventCreate(&e0));
  GB_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int bestv = 0;
  for(int v = 0; v < kBsrVariants; v++) {
    launch_bsr<2, T>(v, B, val, pa.p, nullptr, q.p, part.p, nullptr, st);
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

int bsr_tune(gb300_matrix *A, Bsr3 &B, cudaStream_t st)
{
  if(B.val32.p) {
    if(A->bsr_var32 < 0) GB_TRY(tune_one<float>(B, B.val32.p, &A->bsr_var32, st));
    B.var32 = A->bsr_var32;
  }
  if(B.val64.p) {
    if(A->bsr_var64 < 0) GB_TRY(tune_one<double>(B, B.val64.p, &A->bsr_var64, st));
    B.var64 = A->bsr_var64;
  }
  return GB300_OK;
}

}  // namespace gb
