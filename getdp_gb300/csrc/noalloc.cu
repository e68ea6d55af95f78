// Residual r = b - A x and ||r||_2 without any device allocation.
//
// Some callers of this library cannot allocate GPU memory while they run:
// a host application that reserves all device memory up front and forbids
// later cudaMalloc (cudaMalloc can also synchronize the device, which a
// time-stepping or Newton loop with a hard latency budget must avoid), or a
// caller that hands its memory to another allocator.  For them this file
// provides a variant of the solver's residual kernel (k_spmv in sparse.cu,
// MODE 1) whose scratch memory -- one partial sum per block plus the final
// sum -- lives in a file-scope device array instead of a per-call buffer.
//
// Limit: one partial sum per block of kRowsPerBlock rows, at most
// kMaxBlocks blocks, so n <= kMaxBlocks * kRowsPerBlock = 33,554,432 rows;
// the array takes (kMaxBlocks + 1) * 8 bytes = 128 KiB + 8 bytes on every GPU
// that loads the library, until the process exits.
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress (with that device current) and caches it; make
// that first call before any stream capture.  Every call returns the norm
// on the host, so it waits for the context's stream to finish its work
// before it returns.  Every call shares the array:
// each call overwrites all the partial sums it reads, so nothing needs
// clearing, but calls that overlap on the GPU (two streams, two threads,
// two contexts on the same device) race on it and must be serialized by the
// caller.
#include <mutex>

#include "sparse.cuh"

namespace gb {

constexpr int kNoAllocThreads = 256;
constexpr int kRowsPerBlock = 2048;
constexpr int kMaxBlocks = 16384;
constexpr long long kNoAllocMaxRows = (long long)kMaxBlocks * kRowsPerBlock;

static __device__ __align__(256) double g_residual_scratch[kMaxBlocks + 1];

// device address of g_residual_scratch, per device (set up on first use)
static double *g_scratch_ptr[64];
static std::mutex g_scratch_mutex;

static int scratch_for_device(int device, double **out)
{
  if(device < 0 || device >= 64) {
    set_error("device %d out of range for the no-allocation entry point", device);
    return GB300_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if(!g_scratch_ptr[device]) {
    int cur = -1;
    GB_CUDA(cudaGetDevice(&cur));
    GB_CUDA(cudaSetDevice(device));
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_residual_scratch);
    cudaSetDevice(cur);
    if(e != cudaSuccess || !p) {
      set_error("cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return GB300_ERR_CUDA;
    }
    g_scratch_ptr[device] = (double *)p;
  }
  *out = g_scratch_ptr[device];
  return GB300_OK;
}

// TPR threads per row; block b handles rows [b*kRowsPerBlock, ...) and
// writes the partial sum of r_i^2 over them to part[b]
template <int TPR>
__global__ void __launch_bounds__(kNoAllocThreads)
k_residual_noalloc(int n, const int *__restrict__ rowptr,
                   const int *__restrict__ col, const double *__restrict__ val,
                   const double *__restrict__ x, const double *__restrict__ b,
                   double *__restrict__ r, double *__restrict__ part)
{
  const int rows_per_iter = kNoAllocThreads / TPR;
  int lane = threadIdx.x % TPR;
  int sub = threadIdx.x / TPR;
  long long r0 = (long long)blockIdx.x * kRowsPerBlock;
  long long r1 = r0 + kRowsPerBlock < n ? r0 + kRowsPerBlock : n;
  double red = 0.0;
  for(long long rb = r0; rb < r1; rb += rows_per_iter) {
    long long row = rb + sub;
    double sum = 0.0;
    if(row < r1) {
      int s = rowptr[row], e = rowptr[row + 1];
      for(int k = s + lane; k < e; k += TPR) sum += ld_stream(val + k) * x[ld_stream(col + k)];
    }
#pragma unroll
    for(int o = TPR / 2; o > 0; o >>= 1)
      sum += __shfl_down_sync(0xffffffffu, sum, o, TPR);
    if(lane == 0 && row < r1) {
      double ri = b[row] - sum;
      r[row] = ri;
      red += ri * ri;
    }
  }
  double s = block_sum<double, kNoAllocThreads>(red);
  if(threadIdx.x == 0) part[blockIdx.x] = s;
}

// fixed-order sum of the nb partials into part[kMaxBlocks]
__global__ void k_residual_noalloc_sum(int nb, double *part)
{
  double v = 0.0;
  for(int i = threadIdx.x; i < nb; i += blockDim.x) v += part[i];
  double s = block_sum<double, kNoAllocThreads>(v);
  if(threadIdx.x == 0) part[kMaxBlocks] = s;
}

}  // namespace gb

using namespace gb;

extern "C" int gb300_residual_noalloc(gb300_matrix *A, const gb300_vector *x,
                                      const gb300_vector *b, gb300_vector *r,
                                      double *norm)
{
  if(!A || !x || !b || !r || !norm) {
    set_error("gb300_residual_noalloc: NULL argument");
    return GB300_ERR_ARG;
  }
  if((long long)A->n > kNoAllocMaxRows) {
    set_error("gb300_residual_noalloc: %d rows exceed the maximum of %lld "
              "(fixed scratch of %d partial sums)", A->n, kNoAllocMaxRows,
              kMaxBlocks);
    return GB300_ERR_CAPACITY;
  }
  if(!A->csr_valid || !A->hr.empty()) {
    set_error("gb300_residual_noalloc: the matrix must be assembled first "
              "(assembling would allocate)");
    return GB300_ERR_ARG;
  }
  if(x->n != A->n || b->n != A->n || r->n != A->n) {
    set_error("gb300_residual_noalloc: vector sizes do not match the matrix");
    return GB300_ERR_ARG;
  }
  if(x == r || b == r) {
    set_error("gb300_residual_noalloc: r must not alias x or b");
    return GB300_ERR_ARG;
  }
  double *scratch = nullptr;
  GB_TRY(scratch_for_device(A->ctx->device, &scratch));
  cudaStream_t st = A->ctx->stream;
  int n = A->n;
  int nb = n > 0 ? (int)((n + kRowsPerBlock - 1) / kRowsPerBlock) : 0;
  if(nb > 0) {
    switch(A->tpr) {
    case 2: k_residual_noalloc<2><<<nb, kNoAllocThreads, 0, st>>>(n, A->rowptr.p, A->col.p, A->val.p, x->d.p, b->d.p, r->d.p, scratch); break;
    case 4: k_residual_noalloc<4><<<nb, kNoAllocThreads, 0, st>>>(n, A->rowptr.p, A->col.p, A->val.p, x->d.p, b->d.p, r->d.p, scratch); break;
    case 8: k_residual_noalloc<8><<<nb, kNoAllocThreads, 0, st>>>(n, A->rowptr.p, A->col.p, A->val.p, x->d.p, b->d.p, r->d.p, scratch); break;
    case 16: k_residual_noalloc<16><<<nb, kNoAllocThreads, 0, st>>>(n, A->rowptr.p, A->col.p, A->val.p, x->d.p, b->d.p, r->d.p, scratch); break;
    default: k_residual_noalloc<32><<<nb, kNoAllocThreads, 0, st>>>(n, A->rowptr.p, A->col.p, A->val.p, x->d.p, b->d.p, r->d.p, scratch); break;
    }
  }
  k_residual_noalloc_sum<<<1, kNoAllocThreads, 0, st>>>(nb, scratch);
  GB_CUDA(cudaGetLastError());
  double h = 0.0;
  GB_CUDA(cudaMemcpyAsync(&h, scratch + kMaxBlocks, sizeof(double),
                          cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  *norm = sqrt(h);
  return GB300_OK;
}
