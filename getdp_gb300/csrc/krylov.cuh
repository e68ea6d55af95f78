// Solver-internal declarations (work space, ILU(0), GMRES).
#pragma once

#include <cstring>

#include "sparse.cuh"

namespace gb {

constexpr int kScratchRes = 10;
constexpr int kScratchScalar = 11;

// work space of one solve: numbered device vectors, a state block and the
// partial-sum array of the deterministic reductions
struct Work {
  static constexpr int kSlots = 32;
  DevBuf<char> vecs[kSlots];
  DevBuf<char> st;
  DevBuf<double> parts;
  void *vec(int slot, size_t bytes);
  void *state(size_t bytes);
  double *part();
};

int true_residual(const gb300_matrix *A, const double *val, const double *x,
                  const double *b, double *r, double *res, Work &W);
int norm2_dev(int n, const double *v, double *out, Work &W, cudaStream_t st);

int bench_spmv(gb300_matrix *A, int precision, int reps, double *ms);

int gmres_solve(gb300_matrix *A, const double *val, const double *rhs,
                double *x, const gb300_solver_params *p, gb300_solve_info *info,
                Work &W);

}  // namespace gb
