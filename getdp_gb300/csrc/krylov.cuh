// Solver-internal declarations (work space, ILU(0), GMRES).
#pragma once

#include <functional>

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

// node-blocked 3 x 3 copy of a three-component system (bsr.cu)
struct Bsr3 {
  int nn = 0;          // block rows (nodes)
  long long nblk = 0;  // blocks
  long long pstride = 0;  // stride between value planes (padded)
  DevBuf<int> ptr, col;
  DevBuf<double> val64;  // 9 planes of nblk values
  DevBuf<float> val32;
  int var32 = 0, var64 = 0;  // SpMV launch shapes chosen by bsr_tune
  DevBuf<int> err;           // set by a staged SpMV whose copies timed out
};
int bsr_build(const gb300_matrix *A, const double *val, bool want64,
              bool want32, Bsr3 &B);
// pick the fastest SpMV launch shape for this matrix (cached in A and by
// structure); the FP64 product is tuned only when tune64
int bsr_tune(gb300_matrix *A, Bsr3 &B, cudaStream_t st, bool tune64);
void to_nodes64(int nn, const double *in, double *out, cudaStream_t st);
void from_nodes64(int nn, const double *in, double *out, cudaStream_t st);
// q = A p with the partials of <p, q>; with dot_out, the last CTA also
// writes the sum <p, q> there (counter: a zeroed word owned by the caller)
void bsr_spmv_dot32(const Bsr3 &B, const float *p, float *q, double *part,
                    const int *flag, double *dot_out, unsigned *counter,
                    cudaStream_t st);
void bsr_spmv_dot64(const Bsr3 &B, const double *p, double *q, double *part,
                    const int *flag, double *dot_out, unsigned *counter,
                    cudaStream_t st);
void bsr_residual64(const Bsr3 &B, const double *x, const double *b, double *r,
                    double *part, const int *flag, cudaStream_t st);
// GB300_ERR_CUDA if a staged SpMV variant timed out during the solve
int bsr_check(const Bsr3 &B, cudaStream_t st);

// Preconditioner 20 (not a Sparskit value): ILU(0), then z += G (v - A z)
// with G the learned correction on A's pattern (gb300_matrix_set_correction)
constexpr int kPrecondLearned = 20;
// Preconditioners 21 and 22 (not Sparskit values): the two-level cycle
// z = S v; z += P0 Ac^-1 P0^T (v - A z); z += S (v - A z) on the aggregates
// of gb300_matrix_set_aggregates, with S = ILU(0) (21) or ILU(0) followed by
// the learned correction (22) (coarse.cu)
constexpr int kPrecondCoarse = 21;
constexpr int kPrecondLearnedCoarse = 22;
// 23: as 22 with the correction in the first smoothing only (the half of
// the cycle its loss is trained on; half its cost)
constexpr int kPrecondLearnedCoarsePre = 23;
// 24: the two-level cycle smoothed by the learned sparse approximate inverse
// G alone (z = G v: one product per smoothing, no ILU(0) factor)
constexpr int kPrecondLearnedSai = 24;
// 25: as 24 with G the SPAI-1 of A computed by the solver (spai.cu)
constexpr int kPrecondSai = 25;
inline bool precond_two_level(int p)
{
  return p == kPrecondCoarse || p == kPrecondLearnedCoarse || p == kPrecondLearnedCoarsePre ||
         p == kPrecondLearnedSai || p == kPrecondSai;
}
// G = SPAI-1 of A on its pattern, into A->corr (A symmetric, rows <= 16)
int spai1(gb300_matrix *A, const double *val);
inline bool precond_learned(int p)
{
  return p == kPrecondLearned || p == kPrecondLearnedCoarse || p == kPrecondLearnedCoarsePre ||
         p == kPrecondLearnedSai;
}
constexpr int kMaxCoarse = 2048;  // dense coarse inverse: at most 32 MiB
struct Coarse {
  int n = 0, nc = 0;
  unsigned version = ~0u;   // the owner's pattern_version when set
  unsigned stamp = 0;       // bumped by every new set of aggregates
  unsigned followed = ~0u;  // on a permuted copy: the source's stamp it follows
  int headroom = 0;         // bits kept free in the fixed-point sums
  bool ready = false;       // inv holds the inverse for the last values
  DevBuf<int> agg, aperm, aptr;   // aggregate of each row; rows by aggregate
  DevBuf<double> inv;             // nc x nc, row-major
  DevBuf<double> rbuf, cbuf;      // Gauss-Jordan pivot rows and columns
  DevBuf<double> rc, ec;          // coarse residual and correction
  DevBuf<int> err;
  DevBuf<double> amax;
  // the nc pivot launches of the inversion, captured once in a CUDA graph
  // (replayed while nc and the buffers stay the same)
  cudaGraphExec_t gj_exec = nullptr;
  const void *gj_key[4] = {nullptr, nullptr, nullptr, nullptr};
  int gj_nc = 0;
  ~Coarse()
  {
    if(gj_exec) cudaGraphExecDestroy(gj_exec);
  }
};
void coarse_free(Coarse *c);
bool coarse_valid(const gb300_matrix *A);
int coarse_set(gb300_matrix *A, const int *agg, int nc);
// aggregates of about n / target rows from A's graph (greedy breadth-first)
int coarse_auto(gb300_matrix *A, int target);
constexpr int kAutoAggregates = 1024;
int coarse_follow(const gb300_matrix *A, gb300_matrix *B, const Colouring *C,
                  cudaStream_t st);
int coarse_setup(gb300_matrix *A, const double *val, bool reuse);
void coarse_correct(const gb300_matrix *A, const double *val, const double *v, double *z,
                    double *t, const int *flag, cudaStream_t st);
// w <- (I - A C) w and *wcw = w^T C w (device scalar), C = P0 Ac^-1 P0^T on
// A's own values (the coarse inverse made once and then reused; t, q: n
// doubles of scratch) -- the two-level form of the learned correction's loss
int coarse_energy_project(gb300_matrix *A, double *w, double *t, double *q, double *wcw,
                          cudaStream_t st);
// *ucu_dev = u^T C u (same coarse inverse as coarse_energy_project)
int coarse_energy(gb300_matrix *A, const double *u, double *ucu_dev, cudaStream_t st);
// smooth: the first smoothing, smooth_post: the second
void two_level_apply(const gb300_matrix *A, const double *val, const double *v, double *z,
                     double *t3, double *t4, const int *flag, cudaStream_t st,
                     const std::function<void(const double *, double *)> &smooth,
                     const std::function<void(const double *, double *)> &smooth_post);
bool correction_valid(const gb300_matrix *A);
void correction_apply(const gb300_matrix *A, const double *val, const double *v,
                      double *z, double *t1, double *t2, const int *flag, cudaStream_t st);

// ILU(0) of A's pattern on the values val (FP64, or FP32 storage), and its
// application z = M^-1 v guarded by *flag (gmres.cu)
int ilu_factor(gb300_matrix *A, const double *val, bool fp32, int *zero_row_out,
               bool reuse = false, int *factorized = nullptr);
// drop the factor held by the multicolour copy of A (a new Generate)
void colour_drop_factor(gb300_matrix *A);
// mode (ilu_mode): 0 FP64; 1 FP32 factor and FP32 sweeps; 2 FP32 factor,
// FP64 sweeps (the reference's HAVE_ILU_FLOAT build); rmask (optional): rows
// with rmask[i] == 0 are left out of the sweeps
void ilu_apply(const gb300_matrix *A, int mode, const double *v, double *z,
               float *t32, const int *flag, cudaStream_t st,
               const unsigned char *rmask = nullptr);
// Precision 0: FP64 ILU(0); 1: FP32 factor and FP32 sweeps (the mixed form);
// 2: FP32 factor with FP64 sweeps, as the reference built with
// HAVE_ILU_FLOAT (Sparskit.h:48-52) applies it
inline int ilu_mode(const gb300_solver_params *p)
{
  return p->precision == 2 ? 2 : (p->precision != 0 ? 1 : 0);
}

// the Givens rotation of iters.f's givens (3235-3273): zeroes y against x;
// x becomes the norm, (c, s) the rotation
__device__ inline void givens_dev(double *x, double *y, double *c, double *s)
{
  if(*x == 0. && *y == 0.) {
    *c = 1.;
    *s = 0.;
  }
  else if(fabs(*y) > fabs(*x)) {
    double t = *x / *y;
    *x = sqrt(1. + t * t);
    *s = copysign(1. / *x, *y);
    *c = t * *s;
  }
  else if(fabs(*y) <= fabs(*x)) {
    double t = *y / *x;
    *y = sqrt(1. + t * t);
    *c = copysign(1. / *y, *x);
    *s = t * *c;
  }
  else {
    *x = 0.;
    *y = 0.;
    *c = 1.;
    *s = 0.;
  }
  *x = fabs(*x * *y);
}

int gmres_solve(gb300_matrix *A, const double *val, const double *rhs,
                double *x, const gb300_solver_params *p, gb300_solve_info *info,
                Work &W);

// batched GMRES/FGMRES over the diagonal blocks off[0..nsys] of A
// (gmres_batch.cu); infos[p] per system
int gmres_solve_batch(gb300_matrix *A, const double *val, const double *rhs,
                      double *x, const gb300_solver_params *p, int nsys,
                      const int *off, gb300_solve_info *infos, Work &W);

// The ILU(0) level schedule cut into the diagonal blocks of a batch: system
// p's rows are lrows[off[p] .. off[p+1]) grouped by forward-sweep level, its
// levels bounded by llev[llb[p] .. llb[p+1]] (positions in lrows, so
// llb[p+1] - llb[p] - 1 levels); the same for the backward sweep (u*).
struct SysLevels {
  std::vector<int> off;  // the block offsets it was made for
  DevBuf<int> lrows, urows, llev, ulev, llb, ulb;
  int max_levels = 0;    // most levels of one system in either sweep
};
// made (once per pattern and offsets) from A's ILU(0) schedule (gmres.cu)
int ilu_sys_levels(gb300_matrix *A, int nsys, const int *off, const SysLevels **out);
// the ILU(0) factor held for A after ilu_factor: values (double or float),
// inverted pivots and the position of each row's diagonal entry
void ilu_factor_arrays(const gb300_matrix *A, bool fp32, const void **lu, const void **inv,
                       const int **diag);

// batched GMRES/FGMRES with one thread-block cluster per system and the
// whole solve in one launch (gmres_cluster.cu); *used is false, and nothing
// is done, where that form does not apply (then gmres_solve_batch does)
// mc: the multicolour ordering A is permuted by (A = mc->B), or null: with
// it the ILU(0) sweeps go colour by colour, a vertex's rows in one thread
struct Colouring;
int gmres_solve_batch_cluster(gb300_matrix *A, const double *val, const double *rhs,
                              double *x, const gb300_solver_params *p, int nsys,
                              const int *off, gb300_solve_info *infos, Work &W,
                              bool *used, const Colouring *mc = nullptr);
int check_blocks(const gb300_matrix *A, int nsys, const int *off);

// multicolour ordering of a pattern for the ILU(0) solves (color.cu)
struct Colouring {
  int kind = 0;  // 0 multicolour ordering, 1 the RCMK order (rcmk_build)
  int n = 0, ncolors = 0;
  unsigned version = 0;        // pattern version it was built for
  std::vector<int> seg;        // diagonal blocks it was built for
  int bs = 1;                  // rows per coloured vertex
  // per block b, the vertices of colour c are [voff[b (ncolors + 1) + c],
  // voff[b (ncolors + 1) + c + 1]) in the permuted order
  std::vector<int> voff;
  DevBuf<int> new_of, old_of;  // row permutation and its inverse
  DevBuf<int> src;             // entry k of the permuted matrix = entry src[k] of A
  gb300_matrix *B = nullptr;   // permuted structure (+ its ILU state)
};
void colour_free(Colouring *c);
int colour_build(gb300_matrix *A, int nseg, const int *off);
// Sparskit's reverse Cuthill-McKee order (host) and A permuted by it
void rcmk_order(int n, const int *rowptr, const int *col, int *new_of);
int rcmk_build(gb300_matrix *A);
void permute_system(const Colouring *C, long long nnz, const double *val,
                    const double *rhs, double *bval, double *brhs, cudaStream_t st);
void unpermute_solution(const Colouring *C, const double *y, double *x, cudaStream_t st);
int gmres_solve_coloured(gb300_matrix *A, const double *val, const double *rhs,
                         double *x, const gb300_solver_params *p,
                         gb300_solve_info *info, Work &W, bool *used);

}  // namespace gb
