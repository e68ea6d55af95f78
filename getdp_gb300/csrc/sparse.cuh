// Declarations shared by the sparse, assembly and solver translation units.
#pragma once

#include "common.cuh"

namespace gb {

int exclusive_scan(const int *in, long long n, long long *out, long long *total,
                   DevBuf<long long> &tmp, cudaStream_t st);
void choose_tpr(gb300_matrix *A);
// rep > 1: rows r + k n/rep (k < rep) have row r's elements (checked by
// the caller), so only the first n/rep rows are built and copied
int build_pattern_from_elements(gb300_matrix *A, int ne, int nloc,
                                const int *d_edofs, const unsigned char *d_cflag,
                                int complex_mode, int rep = 1);
int build_csr_from_coo(gb300_matrix *A, long long m, const int *d_r,
                       const int *d_c, const double *d_v);

void spmv64(const gb300_matrix *A, const double *x, double *y, cudaStream_t st);
void spmv_plain(const gb300_matrix *A, const double *val, const double *x,
                double *y, cudaStream_t st);
void spmv_guarded(const gb300_matrix *A, const double *val, const double *x,
                  double *y, const int *flag, cudaStream_t st);
// y += A x, and r = b - A x without partial sums (guarded by *flag)
void spmv_add_guarded(const gb300_matrix *A, const double *val, const double *x,
                      double *y, const int *flag, cudaStream_t st);
void resid_guarded(const gb300_matrix *A, const double *val, const double *x,
                   const double *b, double *r, const int *flag, cudaStream_t st);
void residual64(const gb300_matrix *A, const double *val, const double *x,
                const double *b, double *r, double *part, cudaStream_t st);
void residual64_guarded(const gb300_matrix *A, const double *val,
                        const double *x, const double *b, double *r,
                        double *part, const int *flag, cudaStream_t st);
void spmv_dot64(const gb300_matrix *A, const double *val, const double *p,
                double *q, double *part, cudaStream_t st);
void spmv_dot32(const gb300_matrix *A, const float *val, const float *p,
                float *q, double *part, cudaStream_t st);
void sum_partials(const double *part, double *out, cudaStream_t st);
void dot_part64(int n, const double *x, const double *y, double *part,
                cudaStream_t st);
void dot_part32(int n, const float *x, const float *y, double *part,
                cudaStream_t st);

int generate_values(gb300_matrix *A, gb300_vector *b, const gb300_term_batch *t,
                    const gb300_vector *x);
int generate_pattern(gb300_matrix *A, const gb300_term_batch *t);

struct ilu_data;
void ilu_free(ilu_data *d);

int solve(gb300_matrix *A, const gb300_vector *b, const gb300_solver_params *p,
          gb300_vector *x, gb300_solve_info *info);
int precond_apply(gb300_matrix *A, const gb300_solver_params *p, const double *v,
                  double *z);
int post_elements(const gb300_term_batch *t, const gb300_vector *x, double *out);
int post_points(const gb300_term_batch *t, const gb300_vector *x, int np,
                const double *xyz, double *field, double *curl, int *elem);
int solve_batch(gb300_matrix *A, const gb300_vector *b, const gb300_solver_params *p,
                gb300_vector *x, int nsys, const int *off, gb300_solve_info *infos);
// GB300_ERR_ARG unless every negative entry e of the device table edofs (n
// entries) names a fixed DOF of the table: -n_fixed <= e
int check_fixed_table(cudaStream_t st, const int *edofs, long long n, int n_fixed);

}  // namespace gb
