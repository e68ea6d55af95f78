// The C ABI (include/getdp_gb300.h): handles, parameters, vectors,
// matrices, the batched element loop and the solve entry point.
#include <cctype>
#include <cstring>
#include <string>

#include "krylov.cuh"

namespace gb {

static thread_local std::string g_error;

void set_error(const char *fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_error = buf;
}

template <typename T> static int check(T *p, const char *what)
{
  if(!p) {
    set_error("%s is NULL", what);
    return GB300_ERR_ARG;
  }
  return GB300_OK;
}

__global__ void k_add_values(int count, const int *__restrict__ idx,
                             const double *__restrict__ val, int n,
                             double *__restrict__ v)
{
  // entries added in order: one thread walks them (LinAlg adds are
  // sequential; duplicates must accumulate in call order)
  if(blockIdx.x || threadIdx.x) return;
  for(int k = 0; k < count; k++) {
    int i = idx[k];
    if(i >= 0 && i < n) v[i] += val[k];
  }
}

__global__ void k_add_diag(int n, const int *__restrict__ rowptr,
                           const int *__restrict__ col, int *__restrict__ missing)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n) return;
  if(find_col(col, rowptr[i], rowptr[i + 1], i) < 0) atomicExch(missing, 1);
}

}  // namespace gb

using namespace gb;

extern "C" {

const char *gb300_last_error(void) { return g_error.c_str(); }
int gb300_version(void) { return 10000; }

int gb300_ctx_create(int device, gb300_ctx **out)
{
  GB_TRY(check(out, "out"));
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if(e != cudaSuccess || count == 0) {
    set_error("no CUDA device available (%s)", cudaGetErrorString(e));
    return GB300_ERR_CUDA;
  }
  if(device < 0 || device >= count) {
    set_error("device %d out of range (%d devices)", device, count);
    return GB300_ERR_ARG;
  }
  GB_CUDA(cudaSetDevice(device));
  gb300_ctx *c = new gb300_ctx();
  c->device = device;
  cudaDeviceProp prop;
  if(cudaGetDeviceProperties(&prop, device) == cudaSuccess)
    c->num_sms = prop.multiProcessorCount;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if(e != cudaSuccess) {
    delete c;
    set_error("cudaStreamCreate failed: %s", cudaGetErrorString(e));
    return GB300_ERR_CUDA;
  }
  *out = c;
  return GB300_OK;
}

int gb300_ctx_destroy(gb300_ctx *ctx)
{
  if(!ctx) return GB300_OK;
  cudaStreamSynchronize(ctx->stream);
  gb::gen_cache_free(ctx->gen);
  ctx->gen = nullptr;
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return GB300_OK;
}

int gb300_ctx_synchronize(gb300_ctx *ctx)
{
  GB_TRY(check(ctx, "ctx"));
  GB_CUDA(cudaStreamSynchronize(ctx->stream));
  return GB300_OK;
}

int gb300_host_alloc(size_t bytes, void **out)
{
  GB_TRY(check(out, "out"));
  GB_CUDA(cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault));
  return GB300_OK;
}

int gb300_host_free(void *p)
{
  if(p) GB_CUDA(cudaFreeHost(p));
  return GB300_OK;
}

int gb300_device_alloc(gb300_ctx *ctx, size_t bytes, void **out)
{
  GB_TRY(check(ctx, "ctx"));
  GB_TRY(check(out, "out"));
  GB_CUDA(cudaMalloc(out, bytes ? bytes : 1));
  return GB300_OK;
}

int gb300_device_free(gb300_ctx *ctx, void *p)
{
  GB_TRY(check(ctx, "ctx"));
  if(p) {
    GB_CUDA(cudaStreamSynchronize(ctx->stream));
    GB_CUDA(cudaFree(p));
  }
  return GB300_OK;
}

int gb300_copy_to_device(gb300_ctx *ctx, void *dst, const void *src, size_t bytes)
{
  GB_TRY(check(ctx, "ctx"));
  if(!bytes) return GB300_OK;
  GB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  GB_CUDA(cudaStreamSynchronize(ctx->stream));
  return GB300_OK;
}

int gb300_copy_to_host(gb300_ctx *ctx, void *dst, const void *src, size_t bytes)
{
  GB_TRY(check(ctx, "ctx"));
  if(!bytes) return GB300_OK;
  GB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  GB_CUDA(cudaStreamSynchronize(ctx->stream));
  return GB300_OK;
}

// ---------------------------------------------------------------- params
void gb300_solver_params_default(gb300_solver_params *p)
{
  if(!p) return;
  memset(p, 0, sizeof(*p));
  // Sparskit.cpp:1847-1868
  p->matrix_format = 1;
  p->matrix_printing = 0;
  p->matrix_storage = 0;
  p->scaling = 0;
  p->renumbering_technique = 1;
  p->preconditioner = 2;
  p->preconditioner_position = 2;
  p->nb_fill = 20;
  p->permutation_tolerance = 5.e-2;
  p->dropping_tolerance = 0.;
  p->diagonal_compensation = 0.;
  p->re_use_ilu = 0;
  p->algorithm = 8;
  p->krylov_size = 40;
  p->ic_acceleration = 1.;
  p->re_use_lu = 0;
  p->iterative_improvement = 0;
  p->nb_iter_max = 1000;
  p->stopping_test = 1.e-10;
  p->precision = 0;
  p->inner_tolerance = 0.3;
  p->inner_iter_max = 1000;
  p->batch_kernel = 4;
}

struct ParamKey {
  const char *name;
  int is_real;
  size_t off;
};
#define PK(n, r, f) {n, r, offsetof(gb300_solver_params, f)}
static const ParamKey kKeys[] = {
  PK("Matrix_Format", 0, matrix_format),
  PK("Matrix_Printing", 0, matrix_printing),
  PK("Matrix_Storage", 0, matrix_storage),
  PK("Scaling", 0, scaling),
  PK("Renumbering_Technique", 0, renumbering_technique),
  PK("Preconditioner", 0, preconditioner),
  PK("Preconditioner_Position", 0, preconditioner_position),
  PK("Nb_Fill", 0, nb_fill),
  PK("Permutation_Tolerance", 1, permutation_tolerance),
  PK("Dropping_Tolerance", 1, dropping_tolerance),
  PK("Diagonal_Compensation", 1, diagonal_compensation),
  PK("Re_Use_ILU", 0, re_use_ilu),
  PK("Algorithm", 0, algorithm),
  PK("Krylov_Size", 0, krylov_size),
  PK("IC_Acceleration", 1, ic_acceleration),
  PK("Re_Use_LU", 0, re_use_lu),
  PK("Iterative_Improvement", 0, iterative_improvement),
  PK("Nb_Iter_Max", 0, nb_iter_max),
  PK("Stopping_Test", 1, stopping_test),
  PK("Precision", 0, precision),
  PK("Inner_Tolerance", 1, inner_tolerance),
  PK("Inner_Iter_Max", 0, inner_iter_max),
  PK("Batch_Kernel", 0, batch_kernel),
};
#undef PK

static const ParamKey *find_key(const char *name)
{
  for(const ParamKey &k : kKeys)
    if(!strcmp(k.name, name)) return &k;
  return nullptr;
}

static void set_key(gb300_solver_params *p, const ParamKey *k, double v)
{
  char *base = (char *)p;
  if(k->is_real)
    *(double *)(base + k->off) = v;
  else
    *(int *)(base + k->off) = (int)v;
}

int gb300_solver_params_set(gb300_solver_params *p, const char *name,
                            const char *value)
{
  GB_TRY(check(p, "params"));
  GB_TRY(check(name, "name"));
  GB_TRY(check(value, "value"));
  const ParamKey *k = find_key(name);
  if(!k) {
    set_error("Unknown solver parameter '%s'", name);
    return GB300_ERR_ARG;
  }
  // init_solver_option passes reals through a float (Sparskit.cpp:2019-2027)
  if(k->is_real)
    set_key(p, k, (double)(float)atof(value));
  else
    set_key(p, k, (double)atoi(value));
  return GB300_OK;
}

int gb300_solver_params_read(gb300_solver_params *p, const char *path)
{
  GB_TRY(check(p, "params"));
  GB_TRY(check(path, "path"));
  FILE *f = fopen(path, "r");
  if(!f) {
    set_error("could not open solver parameter file '%s'", path);
    return GB300_ERR_ARG;
  }
  char buf[256];
  while(fscanf(f, "%255s", buf) == 1) {
    if(buf[0] == '/' && buf[1] == '*') {
      // skip a comment up to "*/" (the token itself may close it)
      if(strstr(buf + 2, "*/")) continue;
      int c, prev = 0;
      while((c = getc(f)) != EOF) {
        if(prev == '*' && c == '/') break;
        prev = c;
      }
      continue;
    }
    const ParamKey *k = find_key(buf);
    if(!k) {  // "Unknown solver parameter": skip its value
      if(fscanf(f, "%255s", buf) != 1) break;
      continue;
    }
    if(k->is_real) {
      double v;
      if(fscanf(f, "%lf", &v) == 1) set_key(p, k, v);
    }
    else {
      int v;
      if(fscanf(f, "%d", &v) == 1) set_key(p, k, (double)v);
    }
  }
  fclose(f);
  return GB300_OK;
}

// --------------------------------------------------------------- vectors
int gb300_vector_create(gb300_ctx *ctx, int n, gb300_vector **out)
{
  GB_TRY(check(ctx, "ctx"));
  GB_TRY(check(out, "out"));
  if(n < 0) {
    set_error("negative vector size");
    return GB300_ERR_ARG;
  }
  gb300_vector *v = new gb300_vector();
  v->ctx = ctx;
  v->n = n;
  int rc = v->d.alloc(n > 0 ? n : 1);
  if(rc != GB300_OK) {
    delete v;
    return rc;
  }
  GB_CUDA(cudaMemsetAsync(v->d.p, 0, sizeof(double) * (n > 0 ? n : 1), ctx->stream));
  *out = v;
  return GB300_OK;
}

int gb300_vector_destroy(gb300_vector *v)
{
  if(v) {
    cudaStreamSynchronize(v->ctx->stream);
    delete v;
  }
  return GB300_OK;
}

int gb300_vector_zero(gb300_vector *v)
{
  GB_TRY(check(v, "vector"));
  GB_CUDA(cudaMemsetAsync(v->d.p, 0, sizeof(double) * (v->n > 0 ? v->n : 1),
                          v->ctx->stream));
  return GB300_OK;
}

int gb300_vector_set(gb300_vector *v, const double *host)
{
  GB_TRY(check(v, "vector"));
  GB_TRY(check(host, "host"));
  GB_CUDA(cudaMemcpyAsync(v->d.p, host, sizeof(double) * v->n,
                          cudaMemcpyHostToDevice, v->ctx->stream));
  GB_CUDA(cudaStreamSynchronize(v->ctx->stream));
  return GB300_OK;
}

int gb300_vector_get(const gb300_vector *v, double *host)
{
  GB_TRY(check(v, "vector"));
  GB_TRY(check(host, "host"));
  GB_CUDA(cudaMemcpyAsync(host, v->d.p, sizeof(double) * v->n,
                          cudaMemcpyDeviceToHost, v->ctx->stream));
  GB_CUDA(cudaStreamSynchronize(v->ctx->stream));
  return GB300_OK;
}

int gb300_vector_size(const gb300_vector *v, int *n)
{
  GB_TRY(check(v, "vector"));
  GB_TRY(check(n, "n"));
  *n = v->n;
  return GB300_OK;
}

int gb300_vector_norm2(const gb300_vector *v, double *norm)
{
  GB_TRY(check(v, "vector"));
  GB_TRY(check(norm, "norm"));
  Work W;
  return norm2_dev(v->n, v->d.p, norm, W, v->ctx->stream);
}

__global__ void k_axpby(int n, double a, const double *x, double b, double *y)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i < n) y[i] = (b == 0. ? 0. : b * y[i]) + a * x[i];
}

int gb300_vector_axpby(double a, const gb300_vector *x, double b, gb300_vector *y)
{
  GB_TRY(check(x, "x"));
  GB_TRY(check(y, "y"));
  if(x->n != y->n) {
    set_error("vector sizes %d and %d differ", x->n, y->n);
    return GB300_ERR_ARG;
  }
  if(y->n == 0) return GB300_OK;
  cudaStream_t st = y->ctx->stream;
  k_axpby<<<grid_for(y->n, 256), 256, 0, st>>>(y->n, a, x->d.p, b, y->d.p);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(st));
  return GB300_OK;
}

int gb300_vector_add_values(gb300_vector *v, int count, const int *idx,
                            const double *val)
{
  GB_TRY(check(v, "vector"));
  if(count <= 0) return GB300_OK;
  GB_TRY(check(idx, "idx"));
  GB_TRY(check(val, "val"));
  cudaStream_t st = v->ctx->stream;
  DevBuf<int> di;
  DevBuf<double> dv;
  GB_TRY(di.alloc(count));
  GB_TRY(dv.alloc(count));
  GB_CUDA(cudaMemcpyAsync(di.p, idx, sizeof(int) * count, cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaMemcpyAsync(dv.p, val, sizeof(double) * count, cudaMemcpyHostToDevice, st));
  k_add_values<<<1, 32, 0, st>>>(count, di.p, dv.p, v->n, v->d.p);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(st));
  return GB300_OK;
}

// -------------------------------------------------------------- matrices
int gb300_matrix_create(gb300_ctx *ctx, int n, gb300_matrix **out)
{
  GB_TRY(check(ctx, "ctx"));
  GB_TRY(check(out, "out"));
  if(n < 0) {
    set_error("negative matrix size");
    return GB300_ERR_ARG;
  }
  gb300_matrix *A = new gb300_matrix();
  A->ctx = ctx;
  A->n = n;
  *out = A;
  return GB300_OK;
}

int gb300_matrix_destroy(gb300_matrix *A)
{
  if(!A) return GB300_OK;
  cudaStreamSynchronize(A->ctx->stream);
  if(A->ilu) ilu_free(A->ilu);
  colour_free(A->mc);
  coarse_free(A->coarse);
  delete A;
  return GB300_OK;
}

int gb300_matrix_reset(gb300_matrix *A)
{
  GB_TRY(check(A, "matrix"));
  A->hr.clear();
  A->hc.clear();
  A->hv.clear();
  A->csr_valid = false;
  A->val32_valid = false;
  gb::coarse_values_changed(A);
  A->nnz = 0;
  A->block_rows = 1;
  if(A->ilu) {
    ilu_free(A->ilu);
    A->ilu = nullptr;
  }
  return GB300_OK;
}

int gb300_matrix_add_double(gb300_matrix *A, double d, int i, int j)
{
  GB_TRY(check(A, "matrix"));
  if(i < 0 || i >= A->n || j < 0 || j >= A->n) {
    set_error("entry (%d, %d) out of range [0, %d)", i, j, A->n);
    return GB300_ERR_ARG;
  }
  A->hr.push_back(i);
  A->hc.push_back(j);
  A->hv.push_back(d);
  return GB300_OK;
}

int gb300_matrix_add_complex(gb300_matrix *A, double d1, double d2, int i,
                             int j, int k, int l)
{
  GB_TRY(check(A, "matrix"));
  // GetDP's complex unknowns are row pairs (2m, 2m + 1), k = i + 1
  if(k == i + 1 && i % 2 == 0) A->block_rows = 2;
  if(d1) {
    GB_TRY(gb300_matrix_add_double(A, d1, i, j));
    GB_TRY(gb300_matrix_add_double(A, d1, k, l));
  }
  if(d2) {
    GB_TRY(gb300_matrix_add_double(A, -d2, i, l));
    GB_TRY(gb300_matrix_add_double(A, d2, k, j));
  }
  return GB300_OK;
}

int gb300_matrix_add_coo(gb300_matrix *A, long long count, const int *i,
                         const int *j, const double *v)
{
  GB_TRY(check(A, "matrix"));
  if(count <= 0) return GB300_OK;
  GB_TRY(check(i, "i"));
  GB_TRY(check(j, "j"));
  GB_TRY(check(v, "v"));
  for(long long k = 0; k < count; k++)
    if(i[k] < 0 || i[k] >= A->n || j[k] < 0 || j[k] >= A->n) {
      set_error("entry %lld (%d, %d) out of range [0, %d)", k, i[k], j[k], A->n);
      return GB300_ERR_ARG;
    }
  A->hr.insert(A->hr.end(), i, i + count);
  A->hc.insert(A->hc.end(), j, j + count);
  A->hv.insert(A->hv.end(), v, v + count);
  return GB300_OK;
}

int gb300_matrix_assemble(gb300_matrix *A)
{
  gb::NvtxRange nvtx_range("gb300_matrix_assemble");
  GB_TRY(check(A, "matrix"));
  if(A->hr.empty() && A->csr_valid) return GB300_OK;
  cudaStream_t st = A->ctx->stream;
  long long m = (long long)A->hr.size();
  // existing device entries come first: they were added before
  std::vector<int> r, c;
  std::vector<double> v;
  if(A->csr_valid && A->nnz > 0) {
    std::vector<int> rp(A->n + 1), cc(A->nnz);
    std::vector<double> vv(A->nnz);
    GB_CUDA(cudaMemcpyAsync(rp.data(), A->rowptr.p, sizeof(int) * (A->n + 1), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaMemcpyAsync(cc.data(), A->col.p, sizeof(int) * A->nnz, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaMemcpyAsync(vv.data(), A->val.p, sizeof(double) * A->nnz, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    for(int row = 0; row < A->n; row++)
      for(int k = rp[row]; k < rp[row + 1]; k++) {
        r.push_back(row);
        c.push_back(cc[k]);
        v.push_back(vv[k]);
      }
  }
  r.insert(r.end(), A->hr.begin(), A->hr.end());
  c.insert(c.end(), A->hc.begin(), A->hc.end());
  v.insert(v.end(), A->hv.begin(), A->hv.end());
  m = (long long)r.size();
  DevBuf<int> dr, dc;
  DevBuf<double> dv;
  GB_TRY(dr.alloc(m > 0 ? m : 1));
  GB_TRY(dc.alloc(m > 0 ? m : 1));
  GB_TRY(dv.alloc(m > 0 ? m : 1));
  if(m > 0) {
    GB_CUDA(cudaMemcpyAsync(dr.p, r.data(), sizeof(int) * m, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(dc.p, c.data(), sizeof(int) * m, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(dv.p, v.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st));
  }
  if(A->ilu) {
    ilu_free(A->ilu);
    A->ilu = nullptr;
  }
  GB_TRY(build_csr_from_coo(A, m, dr.p, dc.p, dv.p));
  A->hr.clear();
  A->hc.clear();
  A->hv.clear();
  return GB300_OK;
}

int gb300_matrix_zero(gb300_matrix *A)
{
  GB_TRY(check(A, "matrix"));
  GB_TRY(gb300_matrix_assemble(A));
  cudaStream_t st = A->ctx->stream;
  if(A->nnz > 0) GB_CUDA(cudaMemsetAsync(A->val.p, 0, sizeof(double) * A->nnz, st));
  // every row gets its diagonal (LinAlg_SPARSKIT.cpp:168-169)
  DevBuf<int> missing;
  GB_TRY(missing.alloc(1));
  GB_CUDA(cudaMemsetAsync(missing.p, 0, sizeof(int), st));
  int hm = A->n > 0 ? 1 : 0;
  if(A->csr_valid && A->n > 0) {
    k_add_diag<<<grid_for(A->n, 256), 256, 0, st>>>(A->n, A->rowptr.p, A->col.p,
                                                     missing.p);
    GB_CUDA(cudaMemcpyAsync(&hm, missing.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
  }
  if(hm) {
    for(int i = 0; i < A->n; i++) GB_TRY(gb300_matrix_add_double(A, 0.0, i, i));
    GB_TRY(gb300_matrix_assemble(A));
  }
  A->val32_valid = false;
  gb::coarse_values_changed(A);
  return GB300_OK;
}

int gb300_matrix_size(const gb300_matrix *A, int *n)
{
  GB_TRY(check(A, "matrix"));
  GB_TRY(check(n, "n"));
  *n = A->n;
  return GB300_OK;
}

int gb300_matrix_nnz(const gb300_matrix *A, long long *nnz)
{
  GB_TRY(check(A, "matrix"));
  GB_TRY(check(nnz, "nnz"));
  *nnz = A->csr_valid ? A->nnz : 0;
  return GB300_OK;
}

int gb300_matrix_get_csr(const gb300_matrix *A, int *rowptr, int *col, double *val)
{
  GB_TRY(check(A, "matrix"));
  if(!A->csr_valid) {
    set_error("matrix not assembled");
    return GB300_ERR_ARG;
  }
  cudaStream_t st = A->ctx->stream;
  if(rowptr)
    GB_CUDA(cudaMemcpyAsync(rowptr, A->rowptr.p, sizeof(int) * (A->n + 1), cudaMemcpyDeviceToHost, st));
  if(col && A->nnz)
    GB_CUDA(cudaMemcpyAsync(col, A->col.p, sizeof(int) * A->nnz, cudaMemcpyDeviceToHost, st));
  if(val && A->nnz)
    GB_CUDA(cudaMemcpyAsync(val, A->val.p, sizeof(double) * A->nnz, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  return GB300_OK;
}

int gb300_matrix_set_csr(gb300_matrix *A, long long nnz, const int *rowptr,
                         const int *col, const double *val)
{
  GB_TRY(check(A, "matrix"));
  GB_TRY(check(rowptr, "rowptr"));
  if(nnz > 0) {
    GB_TRY(check(col, "col"));
    GB_TRY(check(val, "val"));
  }
  if(rowptr[0] != 0 || rowptr[A->n] != nnz) {
    set_error("inconsistent CSR row pointers");
    return GB300_ERR_ARG;
  }
  cudaStream_t st = A->ctx->stream;
  GB_TRY(A->rowptr.alloc(A->n + 1));
  GB_TRY(A->col.alloc(nnz > 0 ? nnz : 1));
  GB_TRY(A->val.alloc(nnz > 0 ? nnz : 1));
  GB_CUDA(cudaMemcpyAsync(A->rowptr.p, rowptr, sizeof(int) * (A->n + 1), cudaMemcpyHostToDevice, st));
  if(nnz > 0) {
    GB_CUDA(cudaMemcpyAsync(A->col.p, col, sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(A->val.p, val, sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
  }
  GB_CUDA(cudaStreamSynchronize(st));
  A->nnz = nnz;
  A->csr_valid = true;
  A->pattern_version++;
  A->val32_valid = false;
  gb::coarse_values_changed(A);
  A->block3 = false;
  A->node_blocks = false;
  A->bsr_var32 = A->bsr_var64 = -1;
  A->hr.clear();
  A->hc.clear();
  A->hv.clear();
  if(A->ilu) {
    ilu_free(A->ilu);
    A->ilu = nullptr;
  }
  choose_tpr(A);
  return GB300_OK;
}

int gb300_matrix_mult(gb300_matrix *A, const gb300_vector *x, gb300_vector *y)
{
  GB_TRY(check(A, "matrix"));
  GB_TRY(check(x, "x"));
  GB_TRY(check(y, "y"));
  if(x == y) {
    set_error("Wrong arguments in 'LinAlg_ProdMatrixVector'");
    return GB300_ERR_ARG;
  }
  GB_TRY(gb300_matrix_assemble(A));
  if(x->n != A->n || y->n != A->n) {
    set_error("size mismatch in matrix-vector product");
    return GB300_ERR_ARG;
  }
  spmv64(A, x->d.p, y->d.p, A->ctx->stream);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(A->ctx->stream));
  return GB300_OK;
}

// -------------------------------------------------------------- generate
int gb300_generate_pattern(gb300_matrix *A, const gb300_term_batch *t)
{
  gb::NvtxRange nvtx_range("gb300_generate_pattern");
  GB_TRY(check(A, "matrix"));
  GB_TRY(check(t, "term batch"));
  // a Generate makes a new matrix (GetDP's ZeroMatrix): no factor survives it
  if(A->ilu) {
    ilu_free(A->ilu);
    A->ilu = nullptr;
  }
  colour_drop_factor(A);
  return generate_pattern(A, t);
}

int gb300_generate_values(gb300_matrix *A, gb300_vector *b,
                          const gb300_term_batch *t)
{
  gb::NvtxRange nvtx_range("gb300_generate_values");
  GB_TRY(check(A, "matrix"));
  GB_TRY(check(b, "rhs"));
  GB_TRY(check(t, "term batch"));
  return generate_values(A, b, t, nullptr);
}

int gb300_generate_values_at(gb300_matrix *A, gb300_vector *b,
                             const gb300_term_batch *t, const gb300_vector *x)
{
  gb::NvtxRange nvtx_range("gb300_generate_values_at");
  GB_TRY(check(A, "matrix"));
  GB_TRY(check(b, "rhs"));
  GB_TRY(check(t, "term batch"));
  GB_TRY(check(x, "solution"));
  return generate_values(A, b, t, x);
}

// ----------------------------------------------------------- measurement
static cudaEvent_t g_events[16];

int gb300_event_record(gb300_ctx *ctx, int slot)
{
  GB_TRY(check(ctx, "ctx"));
  if(slot < 0 || slot >= 16) {
    set_error("event slot %d out of range [0, 16)", slot);
    return GB300_ERR_ARG;
  }
  if(!g_events[slot]) {
    GB_CUDA(cudaEventCreate(&g_events[slot]));
  }
  GB_CUDA(cudaEventRecord(g_events[slot], ctx->stream));
  return GB300_OK;
}

int gb300_event_elapsed(gb300_ctx *ctx, int slot0, int slot1, float *ms)
{
  GB_TRY(check(ctx, "ctx"));
  GB_TRY(check(ms, "ms"));
  if(slot0 < 0 || slot0 >= 16 || slot1 < 0 || slot1 >= 16 || !g_events[slot0] ||
     !g_events[slot1]) {
    set_error("event slots not recorded");
    return GB300_ERR_ARG;
  }
  GB_CUDA(cudaEventSynchronize(g_events[slot1]));
  GB_CUDA(cudaEventElapsedTime(ms, g_events[slot0], g_events[slot1]));
  return GB300_OK;
}

// FP64 FMA throughput: eight independent dependency chains per thread, so
// the FP64 pipe, not the FMA latency, limits the rate; the result is
// consumed so that no chain is removed.
__global__ void __launch_bounds__(256) k_fp64_fma(int iters, double a, double c,
                                                  double *sink)
{
  double v[8];
#pragma unroll
  for(int k = 0; k < 8; k++) v[k] = 1.0 + 1e-3 * (threadIdx.x + k);
  for(int i = 0; i < iters; i++) {
#pragma unroll
    for(int k = 0; k < 8; k++) v[k] = fma(v[k], a, c);
  }
  double s = 0.;
#pragma unroll
  for(int k = 0; k < 8; k++) s += v[k];
  if(s == 1234.5678) sink[0] = s;  // never true for these inputs; keeps the chains
}

int gb300_bench_fp64_peak(gb300_ctx *ctx, double *tflops)
{
  GB_TRY(check(ctx, "ctx"));
  GB_TRY(check(tflops, "tflops"));
  cudaStream_t st = ctx->stream;
  int sms = 0, per_sm = 0;
  GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fp64_fma, 256, 0));
  const int grid = sms * (per_sm > 0 ? per_sm : 1);
  const int iters = 4096;
  DevBuf<double> sink;
  GB_TRY(sink.alloc(1));
  cudaEvent_t e0, e1;
  GB_CUDA(cudaEventCreate(&e0));
  GB_CUDA(cudaEventCreate(&e1));
  k_fp64_fma<<<grid, 256, 0, st>>>(iters, 0.9999999, 1e-7, sink.p);  // warm-up
  GB_CUDA(cudaEventRecord(e0, st));
  const int reps = 5;
  for(int r = 0; r < reps; r++)
    k_fp64_fma<<<grid, 256, 0, st>>>(iters, 0.9999999, 1e-7, sink.p);
  GB_CUDA(cudaEventRecord(e1, st));
  GB_CUDA(cudaEventSynchronize(e1));
  GB_CUDA(cudaGetLastError());
  float ms = 0.f;
  GB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  double flops = 2.0 * 8.0 * iters * 256.0 * grid * reps;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return GB300_OK;
}

// FP64 tensor-core (DMMA) throughput: each warp keeps four independent
// m8n8k4 accumulators (D = A B + D, 512 flops per warp instruction)
__global__ void __launch_bounds__(256) k_fp64_dmma(int iters, double *sink)
{
  const int lane = threadIdx.x & 31;
  double a = 1.0 + 1e-3 * lane, b = 1.0 - 1e-3 * lane;
  double acc[4][2];
#pragma unroll
  for(int k = 0; k < 4; k++) acc[k][0] = acc[k][1] = 0.;
  for(int i = 0; i < iters; i++) {
#pragma unroll
    for(int k = 0; k < 4; k++)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 "
                   "{%0, %1}, {%2}, {%3}, {%0, %1};"
                   : "+d"(acc[k][0]), "+d"(acc[k][1])
                   : "d"(a), "d"(b));
  }
  double s = 0.;
#pragma unroll
  for(int k = 0; k < 4; k++) s += acc[k][0] + acc[k][1];
  if(s == 1234.5678) sink[0] = s;  // never true for these inputs
}

int gb300_bench_dmma_peak(gb300_ctx *ctx, double *tflops)
{
  GB_TRY(check(ctx, "ctx"));
  GB_TRY(check(tflops, "tflops"));
  cudaStream_t st = ctx->stream;
  int sms = 0, per_sm = 0;
  GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fp64_dmma, 256, 0));
  const int grid = sms * (per_sm > 0 ? per_sm : 1);
  const int iters = 1024;
  DevBuf<double> sink;
  GB_TRY(sink.alloc(1));
  cudaEvent_t e0, e1;
  GB_CUDA(cudaEventCreate(&e0));
  GB_CUDA(cudaEventCreate(&e1));
  k_fp64_dmma<<<grid, 256, 0, st>>>(iters, sink.p);  // warm-up
  GB_CUDA(cudaEventRecord(e0, st));
  const int reps = 5;
  for(int r = 0; r < reps; r++) k_fp64_dmma<<<grid, 256, 0, st>>>(iters, sink.p);
  GB_CUDA(cudaEventRecord(e1, st));
  GB_CUDA(cudaEventSynchronize(e1));
  GB_CUDA(cudaGetLastError());
  float ms = 0.f;
  GB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double warps = grid * 256.0 / 32.0;
  const double flops = 512.0 * 4.0 * iters * warps * reps;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return GB300_OK;
}

int gb300_bench_spmv(gb300_matrix *A, int precision, int reps, double *ms)
{
  GB_TRY(check(A, "matrix"));
  GB_TRY(check(ms, "ms"));
  GB_TRY(gb300_matrix_assemble(A));
  return bench_spmv(A, precision, reps, ms);
}

// ----------------------------------------------------------------- solve
int gb300_solve(gb300_matrix *A, const gb300_vector *b,
                const gb300_solver_params *p, gb300_vector *x,
                gb300_solve_info *info)
{
  gb::NvtxRange nvtx_range("gb300_solve");
  GB_TRY(check(A, "matrix"));
  GB_TRY(check(b, "rhs"));
  GB_TRY(check(p, "params"));
  GB_TRY(check(x, "solution"));
  GB_TRY(gb300_matrix_assemble(A));
  return solve(A, b, p, x, info);
}

int gb300_matrix_set_correction(gb300_matrix *A, const double *values, int on_device)
{
  GB_TRY(check(A, "matrix"));
  GB_TRY(gb300_matrix_assemble(A));
  if(A->nnz > 0) {
    GB_TRY(check(values, "values"));
    GB_TRY(A->corr.alloc(A->nnz));
    GB_CUDA(cudaMemcpyAsync(A->corr.p, values, sizeof(double) * A->nnz,
                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                            A->ctx->stream));
    GB_CUDA(cudaStreamSynchronize(A->ctx->stream));
  }
  A->corr_version = A->pattern_version;
  return GB300_OK;
}

int gb300_matrix_set_aggregates(gb300_matrix *A, const int *agg, int n_agg)
{
  GB_TRY(check(A, "matrix"));
  GB_TRY(gb300_matrix_assemble(A));
  if(A->n > 0) GB_TRY(check(agg, "aggregates"));
  return coarse_set(A, agg, n_agg);
}

int gb300_matrix_aggregate_graph(gb300_matrix *A, int n_agg)
{
  GB_TRY(check(A, "matrix"));
  GB_TRY(gb300_matrix_assemble(A));
  if(n_agg < 1 || n_agg > kMaxCoarse) {
    set_error("aggregates: %d aggregates asked (1 to %d supported)", n_agg, kMaxCoarse);
    return GB300_ERR_ARG;
  }
  return coarse_auto(A, n_agg);
}

int gb300_matrix_coarse_energy(gb300_matrix *A, const gb300_vector *u, double *ucu)
{
  GB_TRY(check(A, "matrix"));
  GB_TRY(check(u, "vector"));
  GB_TRY(check(ucu, "result"));
  GB_TRY(gb300_matrix_assemble(A));
  if(u->n != A->n) {
    set_error("coarse energy: vector size %d, matrix size %d", u->n, A->n);
    return GB300_ERR_ARG;
  }
  if(!coarse_valid(A)) {
    set_error("coarse energy: the matrix has no aggregates on its current pattern");
    return GB300_ERR_ARG;
  }
  cudaStream_t st = A->ctx->stream;
  DevBuf<double> d;
  GB_TRY(d.alloc(1));
  GB_TRY(coarse_energy(A, u->d.p, d.p, st));
  GB_CUDA(cudaMemcpyAsync(ucu, d.p, sizeof(double), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  return GB300_OK;
}

int gb300_matrix_scale_correction(gb300_matrix *A, double s)
{
  GB_TRY(check(A, "matrix"));
  if(!correction_valid(A)) {
    set_error("the matrix has no correction on its current pattern");
    return GB300_ERR_ARG;
  }
  cudaStream_t st = A->ctx->stream;
  for(long long o = 0; o < A->nnz; o += (1LL << 30)) {
    int m = (int)((A->nnz - o) < (1LL << 30) ? (A->nnz - o) : (1LL << 30));
    k_axpby<<<grid_for(m, 256), 256, 0, st>>>(m, 0., A->corr.p + o, s, A->corr.p + o);
  }
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(st));
  return GB300_OK;
}

int gb300_precond_apply(gb300_matrix *A, const gb300_solver_params *p,
                        const gb300_vector *v, gb300_vector *z)
{
  gb::NvtxRange nvtx_range("gb300_precond_apply");
  GB_TRY(check(A, "matrix"));
  GB_TRY(check(p, "params"));
  GB_TRY(check(v, "v"));
  GB_TRY(check(z, "z"));
  GB_TRY(gb300_matrix_assemble(A));
  if(v->n != A->n || z->n != A->n || v == z) {
    set_error("preconditioner apply: sizes or aliasing");
    return GB300_ERR_ARG;
  }
  return precond_apply(A, p, v->d.p, z->d.p);
}

int gb300_post_elements(const gb300_term_batch *t, const gb300_vector *x,
                        double *out)
{
  gb::NvtxRange nvtx_range("gb300_post_elements");
  GB_TRY(check(t, "term batch"));
  GB_TRY(check(x, "solution"));
  GB_TRY(check(out, "out"));
  return post_elements(t, x, out);
}

int gb300_post_points(const gb300_term_batch *t, const gb300_vector *x, int npts,
                      const double *xyz, double *field, double *curl, int *elem)
{
  gb::NvtxRange nvtx_range("gb300_post_points");
  GB_TRY(check(t, "term batch"));
  GB_TRY(check(x, "solution"));
  if(npts > 0) GB_TRY(check(xyz, "xyz"));
  return post_points(t, x, npts, xyz, field, curl, elem);
}

int gb300_rcmk_order(int n, const int *rowptr, const int *col, int *new_of)
{
  GB_TRY(check(rowptr, "rowptr"));
  GB_TRY(check(col, "col"));
  GB_TRY(check(new_of, "new_of"));
  if(n < 0 || rowptr[0] != 0) {
    set_error("gb300_rcmk_order: bad pattern");
    return GB300_ERR_ARG;
  }
  for(int i = 0; i < n; i++) {
    if(rowptr[i + 1] < rowptr[i]) {
      set_error("gb300_rcmk_order: row pointers decrease at row %d", i);
      return GB300_ERR_ARG;
    }
    for(int k = rowptr[i]; k < rowptr[i + 1]; k++)
      if(col[k] < 0 || col[k] >= n) {
        set_error("gb300_rcmk_order: column %d out of range in row %d", col[k], i);
        return GB300_ERR_ARG;
      }
  }
  gb::rcmk_order(n, rowptr, col, new_of);
  return GB300_OK;
}

int gb300_solve_batch(gb300_matrix *A, const gb300_vector *b,
                      const gb300_solver_params *p, gb300_vector *x, int nsys,
                      const int *offsets, gb300_solve_info *infos)
{
  gb::NvtxRange nvtx_range("gb300_solve_batch");
  GB_TRY(check(A, "matrix"));
  GB_TRY(check(b, "rhs"));
  GB_TRY(check(p, "params"));
  GB_TRY(check(x, "solution"));
  GB_TRY(check(offsets, "offsets"));
  GB_TRY(check(infos, "infos"));
  GB_TRY(gb300_matrix_assemble(A));
  return solve_batch(A, b, p, x, nsys, offsets, infos);
}

}  // extern "C"
