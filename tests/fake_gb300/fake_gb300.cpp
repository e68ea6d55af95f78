// Test double of libgetdp_gb300 -- test infrastructure only, never shipped.
//
// GetDP linked with the GB300 backend stops at its first CUDA call on a host
// without a GPU.  To check the GetDP side of the batched Generate hook
// (getdp_gb300/getdp_backend/Generate_GB300.cpp) on such a host, the tests
// link the same GetDP objects against this library instead: the C-ABI entry
// points the backend calls, kept in host memory (matrix entries as triplets,
// vectors as arrays), with gb300_generate_* accepting the batch (the hook
// dumps it before submitting) and gb300_solve reporting "unsupported".
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "getdp_gb300.h"

struct gb300_ctx {
  int device;
};
struct gb300_vector {
  std::vector<double> v;
};
struct gb300_matrix {
  int n;
  std::vector<int> r, c;
  std::vector<double> v;
};

static const char *g_err = "";

extern "C" {

const char *gb300_last_error(void) { return g_err; }
int gb300_ctx_create(int device, gb300_ctx **out)
{
  *out = new gb300_ctx{device};
  return GB300_OK;
}
int gb300_ctx_destroy(gb300_ctx *ctx)
{
  delete ctx;
  return GB300_OK;
}
void gb300_solver_params_default(gb300_solver_params *p)
{
  memset(p, 0, sizeof(*p));
  p->algorithm = 8;
  p->preconditioner = 2;
  p->krylov_size = 40;
  p->nb_iter_max = 1000;
  p->stopping_test = 1e-10;
}
int gb300_solver_params_set(gb300_solver_params *, const char *, const char *) { return GB300_OK; }
int gb300_solver_params_read(gb300_solver_params *, const char *) { return GB300_OK; }
int gb300_vector_create(gb300_ctx *, int n, gb300_vector **out)
{
  *out = new gb300_vector();
  (*out)->v.assign(n > 0 ? n : 0, 0.);
  return GB300_OK;
}
int gb300_vector_destroy(gb300_vector *v)
{
  delete v;
  return GB300_OK;
}
int gb300_vector_set(gb300_vector *v, const double *h)
{
  memcpy(v->v.data(), h, v->v.size() * sizeof(double));
  return GB300_OK;
}
int gb300_vector_get(const gb300_vector *v, double *h)
{
  memcpy(h, v->v.data(), v->v.size() * sizeof(double));
  return GB300_OK;
}
int gb300_matrix_create(gb300_ctx *, int n, gb300_matrix **out)
{
  *out = new gb300_matrix();
  (*out)->n = n;
  return GB300_OK;
}
int gb300_matrix_destroy(gb300_matrix *A)
{
  delete A;
  return GB300_OK;
}
int gb300_matrix_zero(gb300_matrix *A)
{
  for(auto &x : A->v) x = 0.;
  return GB300_OK;
}
int gb300_matrix_add_double(gb300_matrix *A, double d, int i, int j)
{
  A->r.push_back(i);
  A->c.push_back(j);
  A->v.push_back(d);
  return GB300_OK;
}
int gb300_matrix_add_complex(gb300_matrix *A, double d1, double d2, int i, int j, int k, int l)
{
  gb300_matrix_add_double(A, d1, i, j);
  return GB300_OK;
}
int gb300_matrix_add_coo(gb300_matrix *A, long long m, const int *i, const int *j, const double *v)
{
  for(long long k = 0; k < m; k++) gb300_matrix_add_double(A, v[k], i[k], j[k]);
  return GB300_OK;
}
int gb300_matrix_assemble(gb300_matrix *) { return GB300_OK; }
int gb300_matrix_size(const gb300_matrix *A, int *n)
{
  *n = A->n;
  return GB300_OK;
}
int gb300_matrix_nnz(const gb300_matrix *A, long long *nnz)
{
  *nnz = 0;
  return GB300_OK;
}
int gb300_matrix_get_csr(const gb300_matrix *A, int *rowptr, int *, double *)
{
  for(int i = 0; i <= A->n; i++) rowptr[i] = 0;
  return GB300_OK;
}
int gb300_matrix_set_csr(gb300_matrix *, long long, const int *, const int *, const double *)
{
  return GB300_OK;
}
int gb300_matrix_mult(gb300_matrix *, const gb300_vector *, gb300_vector *y)
{
  for(auto &x : y->v) x = 0.;
  return GB300_OK;
}
int gb300_generate_pattern(gb300_matrix *, const gb300_term_batch *) { return GB300_OK; }
int gb300_generate_values(gb300_matrix *, gb300_vector *, const gb300_term_batch *)
{
  return GB300_OK;
}
int gb300_solve(gb300_matrix *, const gb300_vector *, const gb300_solver_params *,
                gb300_vector *, gb300_solve_info *info)
{
  if(info) memset(info, 0, sizeof(*info));
  g_err = "test double: no solver";
  return GB300_ERR_UNSUPPORTED;
}

}  // extern "C"
