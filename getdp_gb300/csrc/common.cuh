// Shared infrastructure of the GB300 backend: error reporting, the context
// (one device, one stream), device buffers and small device helpers.
#pragma once

#include <nvtx3/nvToolsExt.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/getdp_gb300.h"

namespace gb {

// NVTX range over a scope: the C ABI's phases (Generate, solve, batched
// solve, post-processing, network) show up by name in ncu / Nsight captures
// (ncu --nvtx --nvtx-include "gb300_solve/"); a no-op without a tool
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};


struct ilu_data;
struct Colouring;
struct Coarse;
// A's values changed: a coarse inverse made from the old ones is stale
void coarse_values_changed(gb300_matrix *A);

// last error message, per thread (read through gb300_last_error)
void set_error(const char *fmt, ...);

#define GB_CUDA(x)                                                           \
  do {                                                                       \
    cudaError_t e_ = (x);                                                    \
    if(e_ != cudaSuccess) {                                                  \
      ::gb::set_error("%s:%d: %s failed: %s", __FILE__, __LINE__, #x,        \
                      cudaGetErrorString(e_));                               \
      return GB300_ERR_CUDA;                                                 \
    }                                                                        \
  } while(0)

#define GB_TRY(...)                                                          \
  do {                                                                       \
    int r_ = (__VA_ARGS__);                                                  \
    if(r_ != GB300_OK) return r_;                                            \
  } while(0)

// number of SMs on GB300 and the partial-sum grid used by every
// deterministic reduction (fixed, so results do not depend on timing)
constexpr int kReduceBlocks = 1216;  // 152 SMs x 8
constexpr int kReduceThreads = 256;

template <typename T> struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release()
  {
    if(p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  int alloc(size_t count)
  {
    if(count <= n && p) return GB300_OK;
    release();
    if(count == 0) return GB300_OK;
    cudaError_t e = cudaMalloc((void **)&p, count * sizeof(T));
    if(e != cudaSuccess) {
      set_error("cudaMalloc(%zu bytes) failed: %s", count * sizeof(T),
                cudaGetErrorString(e));
      p = nullptr;
      return GB300_ERR_CUDA;
    }
    n = count;
    return GB300_OK;
  }
};

__device__ __forceinline__ double warp_sum(double v)
{
  for(int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v)
{
  for(int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Per-thread accumulator of a reduction over vector entries of type T:
// float for FP32 vectors (a thread sums a few dozen terms at most, FP64
// takes over at the block sum), double otherwise.  GB300's FP64 pipe
// retires about two FMAs (or conversions) per SM per clock, so FP64
// arithmetic on every entry of an FP32 vector costs more time than the
// entry's memory traffic.
template <typename T> struct Acc {
  using type = double;
};
template <> struct Acc<float> {
  using type = float;
};

// block-wide sum in a fixed order; result valid in thread 0
template <typename T, int NT> __device__ __forceinline__ T block_sum(T v)
{
  __shared__ T red[NT / 32];
  v = warp_sum(v);
  if((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  T s = 0;
  if(threadIdx.x == 0)
    for(int w = 0; w < NT / 32; w++) s += red[w];
  __syncthreads();
  return s;
}

// Block-wide sums of eight per-thread accumulators, in a fixed order.
// Within a warp a transposing butterfly halves the accumulators a lane
// carries at each of the first three exchanges (offsets 16, 8, 4) and then
// adds across the remaining lane pairs: 9 FP64 additions per lane instead
// of 8 x 5 for eight separate warp sums (GB300's FP64 pipe makes the
// difference visible).  Afterwards lane l of each warp holds the warp total
// of accumulator (l >> 2) & 7.  out[j] is valid in thread j (j < 8).
template <int NT> __device__ __forceinline__ double block_sum8(const double (&a)[8])
{
  __shared__ double red[NT / 32][8];
  const int lane = threadIdx.x & 31;
  double b[4], c[2], d;
  {
    const bool hi = lane & 16;
#pragma unroll
    for(int m = 0; m < 4; m++) {
      double keep = hi ? a[m + 4] : a[m], send = hi ? a[m] : a[m + 4];
      b[m] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
  }
  {
    const bool hi = lane & 8;
#pragma unroll
    for(int m = 0; m < 2; m++) {
      double keep = hi ? b[m + 2] : b[m], send = hi ? b[m] : b[m + 2];
      c[m] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
  }
  {
    const bool hi = lane & 4;
    double keep = hi ? c[1] : c[0], send = hi ? c[0] : c[1];
    d = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  d += __shfl_xor_sync(0xffffffffu, d, 2);
  d += __shfl_xor_sync(0xffffffffu, d, 1);
  if((lane & 3) == 0) red[threadIdx.x >> 5][lane >> 2] = d;
  __syncthreads();
  double s = 0.;
  if(threadIdx.x < 8)
    for(int w = 0; w < NT / 32; w++) s += red[w][threadIdx.x];
  __syncthreads();
  return s;
}

// Completion of a grid-wide reduction inside the kernel that produces the
// partials: every block calls arrive_last after its partials are stored;
// exactly one block, the last to arrive, gets true and then sees every
// partial (read them with __ldcg).  It resets the counter for the next
// launch.  Needs no co-residency and never waits.
__device__ __forceinline__ bool arrive_last(unsigned *counter)
{
  __shared__ int last;
  __threadfence();
  __syncthreads();
  if(threadIdx.x == 0) {
    unsigned t = atomicAdd(counter, 1u);
    last = (t == gridDim.x * gridDim.y * gridDim.z - 1);
    if(last) *counter = 0u;
  }
  __syncthreads();
  if(last) __threadfence();
  return last != 0;
}

// the kReduceBlocks partials summed in the fixed order of the one-block
// control kernels (NT threads), read through L2
template <int NT> __device__ __forceinline__ double sum_partials_l2(const double *part)
{
  double s = 0.;
  for(int i = threadIdx.x; i < kReduceBlocks; i += NT) s += __ldcg(part + i);
  return block_sum<double, NT>(s);
}

// streaming loads for data read once per pass (matrix values and indices)
template <typename T> __device__ __forceinline__ T ld_stream(const T *p)
{
  return __ldcs(p);
}

// Partial dot product of one CSR row with x for the TPR lanes that share
// the row: each lane first issues U independent (column, value) loads, then
// the U gathers of x through the read-only path, then the multiply-adds, so
// a warp keeps U memory requests in flight instead of one dependent chain.
template <int TPR, int U, typename ACC, typename V, typename XT>
__device__ __forceinline__ ACC csr_row_dot(int s, int e, int lane,
                                           const int *__restrict__ col,
                                           const V *__restrict__ val,
                                           const XT *__restrict__ x)
{
  ACC sum = 0;
  for(int k0 = s + lane; k0 < e; k0 += TPR * U) {
    int c[U];
    V v[U];
#pragma unroll
    for(int u = 0; u < U; u++) {
      int k = k0 + u * TPR;
      bool in = k < e;
      c[u] = in ? __ldcs(col + k) : 0;
      v[u] = in ? __ldcs(val + k) : (V)0;
    }
    XT xv[U];
#pragma unroll
    for(int u = 0; u < U; u++) xv[u] = __ldg(x + c[u]);
#pragma unroll
    for(int u = 0; u < U; u++) sum += (ACC)v[u] * (ACC)xv[u];
  }
  return sum;
}

// position of column c in the sorted row [lo, hi) of col[], or -1
__device__ __forceinline__ int find_col(const int *__restrict__ col, int lo,
                                        int hi, int c)
{
  const int end = hi;
  while(lo < hi) {
    int mid = (lo + hi) >> 1;
    int v = col[mid];
    if(v < c)
      lo = mid + 1;
    else
      hi = mid;
  }
  return (lo < end && col[lo] == c) ? lo : -1;
}

inline int grid_for(long long work, int threads, int max_blocks = 1 << 30)
{
  long long b = (work + threads - 1) / threads;
  if(b < 1) b = 1;
  if(b > max_blocks) b = max_blocks;
  return (int)b;
}

// CTAs of `kernel` that fit on the device at once (at most kReduceBlocks):
// a grid-stride kernel launched this wide runs in one wave
template <typename K> int resident_grid(K kernel, int threads, size_t smem)
{
  int dev = 0, sms = 0, per_sm = 0;
  if(cudaGetDevice(&dev) != cudaSuccess ||
     cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
     cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) !=
       cudaSuccess ||
     per_sm < 1 || sms < 1)
    return kReduceBlocks;
  return per_sm * sms < kReduceBlocks ? per_sm * sms : kReduceBlocks;
}

}  // namespace gb

namespace gb {
struct GenCache;  // the pattern of the last Generate (assemble.cu)
void gen_cache_free(GenCache *c);
}  // namespace gb

// the objects behind the opaque handles of the C ABI
struct gb300_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 152;
  // CSR pattern, scatter positions and element colouring of the element
  // table last generated on this context: a Generate of the same table
  // (GetDP's ZeroMatrix recreates A before every Generate) reuses them
  gb::GenCache *gen = nullptr;
};

struct gb300_vector {
  gb300_ctx *ctx = nullptr;
  int n = 0;
  gb::DevBuf<double> d;
};

struct gb300_matrix {
  gb300_ctx *ctx = nullptr;
  int n = 0;
  // host staging of LinAlg-style scalar adds, in call order
  std::vector<int> hr, hc;
  std::vector<double> hv;
  // device CSR (0-based, rows sorted by column)
  gb::DevBuf<int> rowptr, col;
  gb::DevBuf<double> val;
  gb::DevBuf<float> val32;  // fp32 copy for mixed-precision inner solves
  long long nnz = 0;
  bool csr_valid = false;
  bool val32_valid = false;
  int tpr = 32;  // threads per row for the CSR kernels
  // three-component system in GetDP's component-major numbering (set by the
  // elasticity Generate hook): the CG may iterate on a 3x3-blocked copy
  bool block3 = false;
  // the pattern has been verified to hold 3 x 3 node blocks (elasticity
  // Generate: one search per node pair); reset by every pattern build
  bool node_blocks = false;
  int bsr_var32 = -1, bsr_var64 = -1;  // tuned SpMV launch shapes (-1: not yet)
  // ILU(0) state, created on demand by the solver
  gb::ilu_data *ilu = nullptr;
  // bumped whenever the pattern is rebuilt; the multicolour ordering of the
  // ILU solves (created on demand) remembers the version it was made for
  unsigned pattern_version = 0;
  gb::Colouring *mc = nullptr;
  // rows per unknown (2: complex system in real form, harmonic-interleaved)
  int block_rows = 1;
  // learned preconditioner correction on the pattern (valid while
  // corr_version == pattern_version)
  gb::DevBuf<double> corr;
  unsigned corr_version = ~0u;
  // aggregates and coarse operator of the two-level preconditioners
  // (gb300_matrix_set_aggregates; valid while their version is pattern_version)
  gb::Coarse *coarse = nullptr;
  // the pattern came from the context's Generate cache entry gen_tag while
  // pattern_version was gen_pv (a later change of the pattern bumps the
  // version and so invalidates the link)
  unsigned gen_tag = 0, gen_pv = ~0u;
};
