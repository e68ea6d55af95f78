/*
 * getdp_gb300 — C ABI of the GB300 (sm_103a) backend for GetDP's
 * Generate/Solve hot path.
 *
 * GetDP talks to its linear-algebra backend through the LinAlg_* functions
 * of src/kernel/LinAlg.h:90-213 (implemented for Sparskit in
 * src/kernel/LinAlg_SPARSKIT.cpp).  This library provides the device-side
 * objects and operations behind a drop-in replacement of that file
 * (getdp_gb300/getdp_backend/LinAlg_GB300.cpp) plus one batched entry point
 * for the element loop of Treatment_FemFormulation
 * (src/kernel/Treatment_Formulation.cpp:413-618), which per-entry
 * LinAlg_AddDoubleInMatrix calls cannot carry to a GPU.
 *
 * Conventions: plain C types only; indices are 0-based as in GetDP's calls
 * (DofData.cpp:1478-1486); every function returns GB300_OK or an error code
 * and the message is available from gb300_last_error().  Nothing here
 * aborts the process: device-side failures are reported as status codes.
 */
#ifndef GETDP_GB300_H
#define GETDP_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GB300_OK 0
#define GB300_ERR_ARG 1          /* invalid argument */
#define GB300_ERR_CUDA 2         /* CUDA runtime error (or no device) */
#define GB300_ERR_UNSUPPORTED 3  /* option not implemented by this backend */
#define GB300_ERR_SOLVER 4       /* Krylov solver did not converge (info) */
#define GB300_ERR_ZERO_PIVOT 5   /* ILU(0) met a zero pivot (info.status) */
#define GB300_ERR_CAPACITY 6     /* a row exceeds a fixed work capacity */
#define GB300_ERR_ZERO_ROW 7     /* empty matrix row (Sparskit.cpp:220-223) */

typedef struct gb300_ctx gb300_ctx;
typedef struct gb300_vector gb300_vector;
typedef struct gb300_matrix gb300_matrix;

/* Message of the last error on the calling thread ("" if none). */
const char *gb300_last_error(void);
int gb300_version(void);

/* ---- context: one device, one stream -------------------------------- */
int gb300_ctx_create(int device, gb300_ctx **out);
int gb300_ctx_destroy(gb300_ctx *ctx);
int gb300_ctx_synchronize(gb300_ctx *ctx);
/* page-locked host memory for fast host<->device copies */
int gb300_host_alloc(size_t bytes, void **out);
int gb300_host_free(void *p);
/* raw device buffers (e.g. element tables kept resident between calls)
   and copies on the context's stream (synchronous on return) */
int gb300_device_alloc(gb300_ctx *ctx, size_t bytes, void **out);
int gb300_device_free(gb300_ctx *ctx, void *p);
int gb300_copy_to_device(gb300_ctx *ctx, void *dst, const void *src, size_t bytes);
int gb300_copy_to_host(gb300_ctx *ctx, void *dst, const void *src, size_t bytes);

/* ---- solver parameters --------------------------------------------- */
/* The fields are the keys of Sparskit's solver.par, same meaning and
   defaults (contrib/Sparskit/Sparskit.h:83-103 Solver_Params,
   Sparskit.cpp:1847-1868 Tab_Params).  Codes: Algorithm 1 CG, 8 GMRES,
   9 FGMRES; Preconditioner 0 none, 6 ILU0, 8 DIAGONAL; Scaling 0 none,
   1 diagonal (D^-1/2 A D^-1/2).  The last four fields are extensions of
   this backend (keys Sparskit would reject as unknown). */
typedef struct gb300_solver_params {
  int matrix_format;
  int matrix_printing;
  int matrix_storage;
  int scaling;
  int renumbering_technique; /* 1 (Sparskit's RCMK): this backend's multicolour
                                order for the ILU(0) sweeps; 2 (no Sparskit
                                value): the reference's RCMK order itself
                                (its default iteration trajectory, serial
                                level schedule); 0 GetDP's order */
  int preconditioner;
  int preconditioner_position;
  int nb_fill;
  double permutation_tolerance;
  double dropping_tolerance;
  double diagonal_compensation;
  int re_use_ilu;
  int algorithm;
  int krylov_size;
  double ic_acceleration;
  int re_use_lu;
  int iterative_improvement;
  int nb_iter_max;
  double stopping_test;
  /* extensions */
  int precision;          /* Precision: 0 FP64, 1 FP32 inner solves in FP64
                             refinement (CG) / the ILU(0) factor applied in
                             FP32 (GMRES, FGMRES); 2 the ILU(0) factor stored
                             in FP32 and applied in FP64, as the reference
                             built with HAVE_ILU_FLOAT (Sparskit.h:48-52) */
  double inner_tolerance; /* Inner_Tolerance: mixed CG, reduction of the FP32
                             residual between two FP64 residual replacements
                             (default 0.3) */
  int inner_iter_max;     /* Inner_Iter_Max */
  int batch_kernel;       /* Batch_Kernel: form of gb300_solve_batch: c = 1, 2,
                             4 (default), 8 or 16: one launch for the whole
                             batch, a thread-block cluster of c CTAs per
                             system (GMRES/FGMRES, Nb_Iter_Max > 0,
                             Krylov_Size <= 64, at most 64 ILU(0) levels per
                             system, e.g. Renumbering_Technique 1); 0, or
                             where that does not apply: one launch per Krylov
                             kernel for all systems in step */
} gb300_solver_params;

/* Replaces Sparskit's init_solver defaults (Sparskit.cpp:1847-1868). */
void gb300_solver_params_default(gb300_solver_params *p);
/* One "-Name value" override (init_solver_option, Sparskit.cpp:2016-2043):
   GB300_ERR_ARG for an unknown name, like "Unknown solver parameter". */
int gb300_solver_params_set(gb300_solver_params *p, const char *name,
                            const char *value);
/* Reads a solver.par file ("Name value" pairs and C comments,
   init_solver Sparskit.cpp:1895-2013); unknown names are skipped. */
int gb300_solver_params_read(gb300_solver_params *p, const char *path);

typedef struct gb300_solve_info {
  int status;            /* Sparskit ipar(1): 0 converged, -1 too many
                            iterations, -3 break-down, -9/-10 abnormal
                            numbers; for a zero pivot: its row (1-based) */
  int iterations;        /* ipar(7): matrix-vector products counted as
                            Sparskit counts them */
  double residual_estimate; /* fpar(6) of the (last) Krylov solve */
  double true_residual;  /* ||b - A x||_2 of the returned x, in FP64, on the
                            system actually solved (scaled if Scaling=1) */
  double rhs_norm;       /* ||b||_2 of that system */
  int refinement_steps;  /* FP64 refinement steps (Precision 1) */
  int inner_iterations;  /* FP32 inner iterations (Precision 1) */
  int ilu_factorized;    /* 1: this solve computed an ILU(0) factorisation;
                            0: none, or the previous one was reused
                            (Re_Use_LU, as LinAlg_SolveAgain sets it) */
  int batch_form;        /* gb300_solve_batch: 1 the one-launch form (a
                            thread-block cluster per system) ran, 0 the
                            per-kernel form; 0 for single solves */
} gb300_solve_info;

/* ---- vectors (device resident, FP64) -------------------------------- */
/* LinAlg_CreateVector / DestroyVector / ZeroVector / SetVector /
   GetDoubleInVector (LinAlg_SPARSKIT.cpp:115-127, :160, :285-300). */
int gb300_vector_create(gb300_ctx *ctx, int n, gb300_vector **out);
int gb300_vector_destroy(gb300_vector *v);
int gb300_vector_zero(gb300_vector *v);
int gb300_vector_set(gb300_vector *v, const double *host);
int gb300_vector_get(const gb300_vector *v, double *host);
int gb300_vector_size(const gb300_vector *v, int *n);
/* LinAlg_VectorNorm2 (norm2_vector) */
int gb300_vector_norm2(const gb300_vector *v, double *norm);
/* y = a x + b y on the device (x and y of the same size, x may be y):
   LinAlg_CopyVector (a = 1, b = 0), LinAlg_ProdVectorDouble (x = y, b = 0)
   and LinAlg_AddVectorProdVectorDouble (b = 1), LinAlg.h:159-175 */
int gb300_vector_axpby(double a, const gb300_vector *x, double b, gb300_vector *y);
/* LinAlg_AddScalarInVector / AddDoubleInVector for a batch of entries
   (host arrays), added in order */
int gb300_vector_add_values(gb300_vector *v, int count, const int *idx,
                            const double *val);

/* ---- matrices (device CSR, rows sorted by column) -------------------- */
/* LinAlg_CreateMatrix / DestroyMatrix (LinAlg_SPARSKIT.cpp:121-134). */
int gb300_matrix_create(gb300_ctx *ctx, int n, gb300_matrix **out);
int gb300_matrix_destroy(gb300_matrix *A);
/* Forget all entries (the Generate path's ZeroMatrix: destroy+create,
   SolvingOperations.cpp:175-184). */
int gb300_matrix_reset(gb300_matrix *A);
/* LinAlg_ZeroMatrix (LinAlg_SPARSKIT.cpp:163-170): keep the pattern, zero
   the values, and make sure every diagonal entry exists. */
int gb300_matrix_zero(gb300_matrix *A);
/* LinAlg_AddDoubleInMatrix (LinAlg_SPARSKIT.cpp:392-400): staged on the
   host in call order; duplicates are summed in that order. */
int gb300_matrix_add_double(gb300_matrix *A, double d, int i, int j);
/* LinAlg_AddComplexInMatrix (LinAlg_SPARSKIT.cpp:402-413): the 2x2 real
   block [[d1, -d2], [d2, d1]] at rows i,k and columns j,l; zero parts are
   skipped exactly as the reference skips them. */
int gb300_matrix_add_complex(gb300_matrix *A, double d1, double d2, int i,
                             int j, int k, int l);
/* Bulk form of add_double (host arrays). */
int gb300_matrix_add_coo(gb300_matrix *A, long long count, const int *i,
                         const int *j, const double *v);
/* LinAlg_AssembleMatrix: merge the staged entries into the device CSR
   (the csr_format step, Sparskit.cpp:2186-2217, done on the GPU). */
int gb300_matrix_assemble(gb300_matrix *A);
int gb300_matrix_size(const gb300_matrix *A, int *n);
int gb300_matrix_nnz(const gb300_matrix *A, long long *nnz);
/* copy the CSR to host arrays (rowptr n+1, col nnz, val nnz) */
int gb300_matrix_get_csr(const gb300_matrix *A, int *rowptr, int *col,
                         double *val);
/* replace the matrix by a host CSR (sorted rows) */
int gb300_matrix_set_csr(gb300_matrix *A, long long nnz, const int *rowptr,
                         const int *col, const double *val);
/* LinAlg_ProdMatrixVector (prod_matrix_vector, Sparskit.cpp:1080-1122) */
int gb300_matrix_mult(gb300_matrix *A, const gb300_vector *x, gb300_vector *y);

/* ---- the batched element loop (Generate) ---------------------------- */
/* One canonical formulation = the Galerkin terms GetDP's element loop
   would evaluate one element at a time (Cal_GalerkinTermOfFemEquation.cpp
   :531-1014) for all elements at once. */
#define GB300_TERM_TRI3_MAGNETOSTATIC 1
/*   2D a_z, BF_PerpendicularEdge on 3-node triangles, 3-point Gauss:
     [coef * Dof{d a}, {d a}] + [-source, {a}]; coef = nu, source = J_z */
#define GB300_TERM_TRI3_EDDY_COMPLEX 2
/*   as above with Type Complex (two harmonics, interleaved unknowns) plus
     DtDof[coef2 * Dof{a}, {a}] (coef2 = sigma) times j*omega, omega = p0 */
#define GB300_TERM_TET10_ELASTICITY 3
/*   3D linear elasticity on 10-node tets, 4-point Gauss: the nine terms
     [-C_ij * Dof{d u_j}, {d u_i}] (Lib_Elasticity_u.pro C tensors with
     E = coef, Poisson = p0) + [f_z, {u_z}] with f_z = p1.  elem_dofs holds
     30 entries per element: ux nodes 1..10, uy nodes, uz nodes */
#define GB300_TERM_TET4_EDGE_CURLCURL 4
/*   3D Whitney edges (BF_Edge) on 4-node tets, 4-point Gauss:
     [coef * Dof{d a}, {d a}] + [p0 * coef * Dof{a}, {a}] + [-js, {a}],
     js constant per element: source holds 3 values per element
     (js_x, js_y, js_z; all zero = no source term) */
#define GB300_TERM_TRI3_MAGNETOSTATIC_NL 5
/*   2D a_z as TRI3_MAGNETOSTATIC with a field-dependent reluctivity, the
     Newton-Raphson terms of templates/Lib_Magnetostatics_a_phi.pro:186-193
     at the current solution (gb300_generate_values_at):
     [nu(b) b, {d a}] + [dhdb(b) Dof{d a}, {d a}] + [-dhdb(b) b, {d a}]
     + [-source, {a}], b = {d a}, nu(b) = coef / (1 + p0 exp(-|b|^2 / p1)),
     dhdb = nu I + 2 dnu/d|b|^2 b b^T */

typedef struct gb300_term_batch {
  int kind;
  int n_nodes;
  int n_elems;
  const double *nodes;           /* n_nodes x 3 */
  const int *elems;              /* n_elems x vertices, 0-based */
  const int *elem_dofs;          /* n_elems x local DOFs: unknown or -1 */
  const signed char *elem_sign;  /* n_elems x local DOFs (edges) or NULL */
  const double *coef;            /* per element */
  const double *source;          /* per element (3 per element for
                                    TET4_EDGE_CURLCURL), or NULL */
  const double *coef2;           /* per element, or NULL */
  const double *coef3;           /* per element, or NULL: TRI3_EDDY_COMPLEX
                                    angular frequency (overrides p0), so one
                                    batch can carry a frequency sweep */
  double p0, p1, p2;
  int on_device;                 /* 1: the arrays above are device pointers */
  /* Fixed DOFs with values (the Dirichlet elimination of Dof_AssembleInMat,
     DofData.cpp:1489-1542): NULL when every fixed DOF is 0 (any negative
     elem_dofs entry is then a fixed zero).  Otherwise a negative entry e
     names fixed DOF -e-1 of value fixed_values[-e-1] (TRI3_EDDY_COMPLEX: two
     values per fixed DOF, real and imaginary part), and every unknown row i
     of the element gets b_i += (g_j * 1) * -Ek_ij.  Supported by the TRI3
     kinds and TET10_ELASTICITY (the nonlinear kind also evaluates {d a}
     with them). */
  const double *fixed_values;
  int n_fixed;
  /* How element contributions are added into A and b (GB300_SCATTER_*):
     DEFAULT is TABLE where one exists, else SEARCH.  SEARCH finds each
     entry by a binary search in its sorted row and adds with FP64 atomics;
     TABLE (node-blocked P2 elasticity on a pattern this context's
     gb300_generate_pattern built) reads the offsets from a table made once
     per pattern and adds with atomics; COLOURED launches the elements colour
     by colour (no two elements of a colour share an unknown; the colouring
     is made once per pattern) and adds without atomics, so that A and b are
     the same to the last bit on every run.  Atomics make the order of the
     additions into one entry vary between runs (rounding only). */
  int scatter;
} gb300_term_batch;

#define GB300_SCATTER_DEFAULT 0
#define GB300_SCATTER_SEARCH 1
#define GB300_SCATTER_TABLE 2
#define GB300_SCATTER_COLOURED 3

/* Build the CSR pattern of A from the element tables (rows of unknowns
   touched by each element, sorted, no duplicates: the pattern the
   reference's linked lists end up with) and zero A and b. */
int gb300_generate_pattern(gb300_matrix *A, const gb300_term_batch *t);
/* Evaluate every element matrix and add it into A and b (A's pattern must
   contain the element pairs: gb300_generate_pattern). */
int gb300_generate_values(gb300_matrix *A, gb300_vector *b,
                          const gb300_term_batch *t);
/* The same at the current solution x (Generate of a nonlinear problem
   evaluates its coefficients from Current.DofData->CurrentSolution);
   formulations that do not depend on x ignore it. */
int gb300_generate_values_at(gb300_matrix *A, gb300_vector *b,
                             const gb300_term_batch *t, const gb300_vector *x);

/* ---- post-processing ------------------------------------------------- */
/* PostOperation Print[ {d a}, OnElementsOf ... ] (Pos_Print.cpp,
   Pos_FemInterpolation.cpp, Cal_PostQuantity.cpp): the curl of the solution
   x on every element of the term batch t, for the formulations
   TRI3_MAGNETOSTATIC, TRI3_EDDY_COMPLEX and TET4_EDGE_CURLCURL (fixed
   unknowns are zero), into the host array out: 2D (bx, by) per element and
   harmonic (2 or 4 values per element), 3D (bx, by, bz). */
int gb300_post_elements(const gb300_term_batch *t, const gb300_vector *x,
                        double *out);
/* Print[ {a}, OnPoint {x,y,z} ] and Print[ {d a}, OnPoint ... ] (the point
   located as Pos_Search.cpp does) for npts points given as host xyz triples:
   field receives a_z per harmonic (2D: 1 or 2 values per point) or the
   vector a (3D, 3 values); curl as gb300_post_elements; elem the 0-based
   element holding the point, or -1 outside the mesh (values 0).  A point on
   a face shared by several elements takes the lowest-numbered one.  NULL
   outputs are skipped. */
int gb300_post_points(const gb300_term_batch *t, const gb300_vector *x, int npts,
                      const double *xyz, double *field, double *curl, int *elem);

/* ---- mesh input (Gmsh MSH 2.2) ----------------------------------------- */
/* The mesh file GetDP reads (Geo_ReadFileWithGmsh, GeoData.cpp), parsed on
   the host at memory speed, ASCII or binary: nodes with their Gmsh numbers,
   and elements grouped by (Gmsh type, tag count) in file order with their
   numbers, tags (physical, elementary, ...) and Gmsh node numbers.  The
   pointers returned stay valid until gb300_msh_free. */
typedef struct gb300_msh gb300_msh;
int gb300_msh_read(const char *path, gb300_msh **out);
int gb300_msh_free(gb300_msh *m);
int gb300_msh_nodes(const gb300_msh *m, long long *n, const long long **numbers,
                    const double **xyz);
int gb300_msh_group_count(const gb300_msh *m, int *count);
int gb300_msh_group(const gb300_msh *m, int g, int *type, long long *n_elems,
                    int *n_tags, int *nodes_per_elem, const long long **numbers,
                    const int **tags, const long long **nodes);

/* ---- measurement ---------------------------------------------------- */
/* CUDA events on the context's stream (slots 0..15), for timing calls
   made through this library on the device. */
int gb300_event_record(gb300_ctx *ctx, int slot);
int gb300_event_elapsed(gb300_ctx *ctx, int slot0, int slot1, float *ms);
/* Average device time of one launch of the solver's CSR SpMV kernel (the
   CG form q = A p with <p, q> fused; precision 0 FP64, 1 FP32 values and
   vectors) over `reps` launches timed with CUDA events after a warm-up. */
int gb300_bench_spmv(gb300_matrix *A, int precision, int reps, double *ms);
/* Measured FP64 FMA throughput of the context's device in TFLOP/s (two
   flops per FMA): the denominator of the FP64-bound element kernels'
   roofline. */
int gb300_bench_fp64_peak(gb300_ctx *ctx, double *tflops);
/* The same for FP64 tensor-core instructions (mma.sync m8n8k4 f64): whether
   DMMA would raise the FP64-bound element kernels' ceiling. */
int gb300_bench_dmma_peak(gb300_ctx *ctx, double *tflops);

/* ---- residual without device allocation ------------------------------ */
/* No counterpart in the reference: an entry point for callers that cannot
   allocate GPU memory once they are running (an application that reserves
   all device memory at start-up, or a latency-bound loop in which
   cudaMalloc's implicit synchronisation is not acceptable).  Computes
   r = b - A x (device vectors, r distinct from x and b) and *norm =
   ||r||_2 in FP64 with scratch in a fixed device array: A must already be
   assembled and have at most 33,554,432 rows (GB300_ERR_CAPACITY
   otherwise).  The array (128 KiB) is held on every GPU that loads the
   library until the process exits.  The first call on a device looks up
   the array's address; make it before any stream capture.  Each call
   returns the norm on the host and so waits for the context's stream to
   finish before it returns.  All calls share
   the array, so calls that overlap on the GPU race and must be serialized
   by the caller. */
int gb300_residual_noalloc(gb300_matrix *A, const gb300_vector *x,
                           const gb300_vector *b, gb300_vector *r,
                           double *norm);

/* ---- learned preconditioner ------------------------------------------ */
/* No counterpart in the reference.  Preconditioner 20 (not a Sparskit
   value) is ILU(0) followed by a correction z += G (v - A z), G a sparse
   matrix on A's pattern.  gb300_matrix_set_correction attaches G (values in
   A's CSR order, host or device pointer); a pattern change drops it. */
int gb300_matrix_set_correction(gb300_matrix *A, const double *values, int on_device);
/* G <- s G for the attached correction (a per-system step length) */
int gb300_matrix_scale_correction(gb300_matrix *A, double s);
/* No counterpart in the reference (Sparskit's preconditioners are one-level).
   Preconditioners 21 and 22 (not Sparskit values) are a two-level cycle:
   z = S v; z += P0 Ac^-1 P0^T (v - A z); z += S (v - A z), with S = ILU(0)
   (21) or ILU(0) followed by the learned correction (22; 23: in the first
   smoothing only), or the learned sparse approximate inverse alone
   (24: z = G v, no ILU(0) factor), P0 the
   piecewise-constant prolongation on aggregates of unknowns and
   Ac = P0^T A P0 inverted densely on the device at every solve (with
   Re_Use_LU, once).  gb300_matrix_set_aggregates gives the aggregate (0 ..
   n_agg - 1) of each of A's n rows, host array; every aggregate must hold a
   row; 1 <= n_agg <= 2048; a pattern change drops them.  A must be symmetric
   positive definite for Ac to be (a non-positive pivot of Ac is an error). */
int gb300_matrix_set_aggregates(gb300_matrix *A, const int *agg, int n_agg);
/* Aggregates from A's graph alone, about n / n_agg rows each (greedy
   breadth-first over A's pattern, small leftovers joined to a neighbour);
   a solve with Preconditioner 21-23 on a matrix without aggregates makes
   them so, with n_agg = min(1024, n / 16). */
int gb300_matrix_aggregate_graph(gb300_matrix *A, int n_agg);
/* u^T P0 Ac^-1 P0^T u for A's aggregates and its own values (the part of
   the energy of an error e with A e = u that the coarse correction removes);
   the coarse inverse is made at the first call and then reused. */
int gb300_matrix_coarse_energy(gb300_matrix *A, const gb300_vector *u, double *ucu);
/* z = M^-1 v with the preconditioner the solver would use for p
   (Preconditioner 6 or 20-24; Renumbering_Technique selects the
   ordering) on A's unscaled values; with p->re_use_lu the factor (and
   coarse inverse) of the previous call on A's pattern is kept. */
int gb300_precond_apply(gb300_matrix *A, const gb300_solver_params *p,
                        const gb300_vector *v, gb300_vector *z);
/* The network that predicts G: 3 message-passing layers of width 32 over the
   matrix graph, BF16 weights, FP32 accumulation (getdp_gb300/csrc/learned.cu).
   gb300_mpnn_infer computes G for A and attaches it (set_correction).
   gb300_mpnn_loss_grad runs the forward and backward passes for one system
   with the energy-norm loss 1 + (y^T A y - 2 r1^T y) / S, y = G r1, which
   is (G r1 - e1)^T A (G r1 - e1) / e1^T A e1 for e1 = A^-1 r1 (A symmetric
   positive definite; r1 = v - A z1, z1 = ILU^-1 v): S = e1^T A e1 when e1
   (x* - z1 for a solved right-hand side) is given, r1^T diag(A)^-1 r1 for a
   probe without solution (e1 NULL); it adds the weight gradients to the
   network's gradient
   (zeroed first unless accumulate); grad_host (param_count floats) may be
   NULL.  gb300_mpnn_adam_step applies grad_scale * gradient with Adam. */
typedef struct gb300_mpnn gb300_mpnn;
int gb300_mpnn_param_count(void);
int gb300_mpnn_create(gb300_ctx *ctx, unsigned seed, gb300_mpnn **out);
int gb300_mpnn_destroy(gb300_mpnn *net);
int gb300_mpnn_set_params(gb300_mpnn *net, const float *host);
int gb300_mpnn_get_params(const gb300_mpnn *net, float *host);
int gb300_mpnn_infer(gb300_mpnn *net, gb300_matrix *A);
int gb300_mpnn_loss_grad(gb300_mpnn *net, gb300_matrix *A, const gb300_vector *r1,
                         const gb300_vector *e1, int accumulate, double *loss,
                         float *grad_host);
int gb300_mpnn_adam_step(gb300_mpnn *net, float lr, float grad_scale);
/* The loss of gb300_mpnn_loss_grad: mode 0 (default) as above; mode 1, for
   the correction inside the two-level cycle (Preconditioner 22), the energy
   of the error left after the coarse correction on A's aggregates,
   (e1 - y)^T (A - A C A) (e1 - y) / S with C = P0 Ac^-1 P0^T (the matrix
   needs gb300_matrix_set_aggregates; its coarse inverse is made at the
   first call and reused). */
int gb300_mpnn_set_loss(gb300_mpnn *net, int mode);

/* ---- solve ------------------------------------------------------------ */
/* LinAlg_Solve -> solve_matrix (Sparskit.cpp:108-634) on the GPU.  A and b
   are not modified (Sparskit scales them in place; here scaling acts on
   private copies).  x receives the solution. */
int gb300_solve(gb300_matrix *A, const gb300_vector *b,
                const gb300_solver_params *p, gb300_vector *x,
                gb300_solve_info *info);

/* Text of the two bulky blocks of a .pre file, into a caller's buffer of
   cap bytes (*len: bytes written; GB300_ERR_CAPACITY if cap is too small);
   host only.  gb300_format_dof_records: the $DofData records of
   Dof_WriteFilePRE (DofData.cpp:363-462), rec5[5 i..5 i+4] = (NumType,
   Entity, Harmonic, Type, NumDof): "NumType Entity Harmonic 1 NumDof 1" for
   Type 1 (unknown), else "NumType Entity Harmonic 2 val[i] 0" with val[i]
   as "%.16g" (LinAlg_PrintScalar).  gb300_format_int_rows: the
   $ElementsXEdges rows of Geo_WriteFilePRE (GeoEntity.cpp:526-552),
   "index width v_1 .. v_width" for rows numbered from first_index. */
int gb300_format_dof_records(long long n, const long long *rec5, const double *val,
                             char *out, long long cap, long long *len);
int gb300_format_int_rows(long long nrows, int width, const long long *vals,
                          long long first_index, char *out, long long cap, long long *len);

/* The reverse Cuthill-McKee order Sparskit computes for Renumbering_Technique
   1 (cmkreord, contrib/Sparskit/cmkreord.f:3-30, called at
   Sparskit.cpp:247-250): new_of[i] is the new index of row i of the n x n
   pattern (0-based CSR, host arrays; structurally symmetric patterns as the
   ILU needs).  Host only; gb300_solve uses it for Renumbering_Technique 2. */
int gb300_rcmk_order(int n, const int *rowptr, const int *col, int *new_of);

/* Batched LinAlg_Solve (Sparskit.cpp:108-634 once per system): the nsys
   independent systems are the diagonal blocks of A, system k owning rows
   [offsets[k], offsets[k+1]) (offsets[0] = 0, offsets[nsys] = n, host
   array); an entry coupling two blocks is an error.  Each system is solved
   as gb300_solve would solve it alone (GMRES or FGMRES, Preconditioner 0 or
   6; Renumbering_Technique 1 reorders within each block), with its own
   convergence test, iteration count and status in infos[k] (nsys entries).
   By default the whole batch is one launch, a thread-block cluster per
   system (Batch_Kernel, infos[k].batch_form = 1); otherwise every Krylov
   kernel launch serves all systems.  Returns GB300_ERR_SOLVER (with the
   solutions and infos filled) if any system did not converge. */
int gb300_solve_batch(gb300_matrix *A, const gb300_vector *b,
                      const gb300_solver_params *p, gb300_vector *x, int nsys,
                      const int *offsets, gb300_solve_info *infos);

#ifdef __cplusplus
}
#endif
#endif
