// GetDP linear-algebra backend on the GB300 library: the functions of
// src/kernel/LinAlg.h:90-213, compiled into GetDP in place of
// src/kernel/LinAlg_SPARSKIT.cpp when HAVE_GB300 is defined (build_getdp.sh
// adds the HAVE_GB300 branch of LinAlg.h and the configuration define).
//
// Types (declared in the HAVE_GB300 branch of LinAlg.h):
//   gMatrix { gb300_matrix *M; }            device CSR, adds staged in order
//   gVector { int N; double *V; gb300_vector *D; int state; }
//            a host mirror V (per-entry access, as GetDP does everywhere)
//            and a device copy D for the solver; `state` says which is
//            current (1 host, 2 device, 3 both)
//   gSolver { gb300_solver_params Params; }
//   gScalar { double s; }
// Semantics follow LinAlg_SPARSKIT.cpp function by function; errors are
// reported through Message::Error with the library's message.

#include <math.h>
#include <string.h>

#include <set>

#include "DofData.h"
#include "GetDPConfig.h"
#include "LinAlg.h"
#include "MallocUtils.h"
#include "Message.h"
#include "ProData.h"

#if defined(HAVE_GB300)

extern struct CurrentData Current;
extern char *Name_Path;

static gb300_ctx *g_ctx = nullptr;
static const char *Name_SolverFile = nullptr;
static const char *Name_DefaultSolverFile = "solver.par";
static char *SolverOptions[100];

enum { HOST = 1, DEV = 2, BOTH = 3 };

static gb300_ctx *ctx()
{
  if(!g_ctx && gb300_ctx_create(0, &g_ctx) != GB300_OK)
    Message::Error("GB300 backend: %s", gb300_last_error());
  return g_ctx;
}

static void ok(int rc)
{
  if(rc != GB300_OK) Message::Error("GB300 backend: %s", gb300_last_error());
}

// the host mirror is current (pull from the device if needed)
static void host(gVector *V)
{
  if(V->state == DEV) {
    ok(gb300_vector_get(V->D, V->V));
    V->state = BOTH;
  }
}
static void host_w(gVector *V)
{
  host(V);
  V->state = HOST;
}
// the device copy is current (push the host mirror if needed)
static void dev(gVector *V)
{
  if(V->state == HOST) {
    ok(gb300_vector_set(V->D, V->V));
    V->state = BOTH;
  }
}

// matrices something has been added to since they were created or zeroed
// (the Generate hook, Generate_GB300.cpp, takes only an untouched matrix)
static std::set<gb300_matrix *> g_touched;
static void touched(gMatrix *M) { g_touched.insert(M->M); }
int GB300_MatrixUntouched(gMatrix *M) { return M->M && !g_touched.count(M->M); }
void GB300_VectorOnDevice(gVector *V) { dev(V); }
void GB300_VectorDeviceWritten(gVector *V) { V->state = DEV; }

void LinAlg_InitializeSolver(int *sargc, char ***sargv)
{
  int i = 1, argc = *sargc, iopt = 0;
  char **argv = *sargv;
  SolverOptions[0] = nullptr;
  while(i < argc) {
    if(argv[i][0] == '-') {
      if(!strcmp(argv[i] + 1, "solver") || !strcmp(argv[i] + 1, "s")) {
        i++;
        if(i < argc && argv[i][0] != '-')
          Name_SolverFile = argv[i++];
        else
          Message::Error("Missing file name");
      }
      else {
        i++;
        if(i < argc && argv[i][0] != '-') {
          SolverOptions[iopt++] = argv[i - 1] + 1;
          SolverOptions[iopt++] = argv[i];
          SolverOptions[iopt] = nullptr;
          i++;
        }
        else
          Message::Error("Missing number");
      }
    }
    else
      Message::Info("Unknown option: '%s'", argv[i++]);
  }
}

void LinAlg_FinalizeSolver()
{
  if(g_ctx) gb300_ctx_destroy(g_ctx);
  g_ctx = nullptr;
}
void LinAlg_SetCommSelf() {}
void LinAlg_SetCommWorld() {}

void LinAlg_CreateSolver(gSolver *Solver, const char *SolverDataFileName)
{
  char FileName[256];
  strcpy(FileName, Name_Path);
  if(SolverDataFileName) {
    if(SolverDataFileName[0] == '/' || SolverDataFileName[0] == '\\')
      strcpy(FileName, SolverDataFileName);
    else
      strcat(FileName, SolverDataFileName);
  }
  else if(Name_SolverFile)
    strcpy(FileName, Name_SolverFile);
  else
    strcat(FileName, Name_DefaultSolverFile);
  gb300_solver_params_default(&Solver->Params);
  FILE *f = fopen(FileName, "r");
  if(f) {
    fclose(f);
    Message::Info("Loading parameter file '%s'", FileName);
    ok(gb300_solver_params_read(&Solver->Params, FileName));
  }
  else
    Message::Info("Parameter file '%s' not found: using defaults", FileName);
  for(int i = 0; SolverOptions[i] && SolverOptions[i + 1]; i += 2) {
    if(gb300_solver_params_set(&Solver->Params, SolverOptions[i],
                               SolverOptions[i + 1]) != GB300_OK)
      Message::Error("Unknown solver parameter '%s'", SolverOptions[i]);
    else
      Message::Info("Overriding parameter '%s': %s", SolverOptions[i],
                    SolverOptions[i + 1]);
  }
}

void LinAlg_SetGlobalSolverOptions(const std::string &opt) {}

void LinAlg_CreateVector(gVector *V, gSolver *Solver, int n)
{
  V->N = n;
  V->V = (double *)Malloc((n > 0 ? n : 1) * sizeof(double));
  V->D = nullptr;
  ok(gb300_vector_create(ctx(), n, &V->D));
  V->state = HOST;
}

void LinAlg_CreateMatrix(gMatrix *M, gSolver *Solver, int n, int m)
{
  ok(gb300_matrix_create(ctx(), n, &M->M));
  g_touched.erase(M->M);
}

void LinAlg_DestroySolver(gSolver *Solver) {}

void LinAlg_DestroyVector(gVector *V)
{
  Free(V->V);
  gb300_vector_destroy(V->D);
  V->D = nullptr;
}

void LinAlg_DestroyMatrix(gMatrix *M)
{
  g_touched.erase(M->M);
  gb300_matrix_destroy(M->M);
  M->M = nullptr;
}

void LinAlg_CopyScalar(gScalar *S1, gScalar *S2) { S2->s = S1->s; }

void LinAlg_CopyVector(gVector *V1, gVector *V2)
{
  host(V1);
  host_w(V2);
  memcpy(V2->V, V1->V, V1->N * sizeof(double));
}

void LinAlg_SwapVector(gVector *V1, gVector *V2)
{
  if(V1->N != V2->N) {
    Message::Error("Cannot swap vectors of different size");
    return;
  }
  host_w(V1);
  host_w(V2);
  for(int i = 0; i < V1->N; i++) {
    double t = V1->V[i];
    V1->V[i] = V2->V[i];
    V2->V[i] = t;
  }
}

void LinAlg_CopyMatrix(gMatrix *M1, gMatrix *M2)
{
  Message::Error("'LinAlg_CopyMatrix' not yet implemented");
}

void LinAlg_ZeroScalar(gScalar *S) { S->s = 0.; }

void LinAlg_ZeroVector(gVector *V)
{
  for(int i = 0; i < V->N; i++) V->V[i] = 0.;
  V->state = HOST;
}

void LinAlg_ZeroMatrix(gMatrix *M)
{
  ok(gb300_matrix_zero(M->M));
  g_touched.erase(M->M);
}

void LinAlg_ScanScalar(FILE *file, gScalar *S) { fscanf(file, "%lf", &S->s); }

void LinAlg_ScanVector(FILE *file, gVector *V)
{
  host_w(V);
  for(int i = 0; i < V->N; i++) fscanf(file, "%lf", &V->V[i]);
}

void LinAlg_ScanMatrix(FILE *file, gMatrix *M)
{
  Message::Error("'LinAlg_ScanMatrix' not yet implemented");
}

void LinAlg_ReadScalar(FILE *file, gScalar *S)
{
  Message::Error("'LinAlg_ReadScalar' not yet implemented");
}

void LinAlg_ReadVector(FILE *file, gVector *V)
{
  host_w(V);
  fread(V->V, sizeof(double), V->N, file);
}

void LinAlg_ReadMatrix(FILE *file, gMatrix *M)
{
  Message::Error("'LinAlg_ReadMatrix' not yet implemented");
}

void LinAlg_PrintScalar(FILE *file, gScalar *S) { fprintf(file, "%.16g", S->s); }

void LinAlg_PrintVector(FILE *file, gVector *V, bool matlab,
                        const char *fileName, const char *varName)
{
  host(V);
  for(int i = 0; i < V->N; i++) fprintf(file, "%.16g\n", V->V[i]);
}

// the KUL format of Sparskit's formatted_write_matrix: "row  col  value"
void LinAlg_PrintMatrix(FILE *file, gMatrix *M, bool matlab,
                        const char *fileName, const char *varName)
{
  ok(gb300_matrix_assemble(M->M));
  int n = 0;
  long long nnz = 0;
  gb300_matrix_size(M->M, &n);
  gb300_matrix_nnz(M->M, &nnz);
  int *rp = (int *)Malloc((n + 1) * sizeof(int));
  int *ci = (int *)Malloc((nnz ? nnz : 1) * sizeof(int));
  double *v = (double *)Malloc((nnz ? nnz : 1) * sizeof(double));
  ok(gb300_matrix_get_csr(M->M, rp, ci, v));
  for(int i = 0; i < n; i++)
    for(int k = rp[i]; k < rp[i + 1]; k++)
      fprintf(file, "%d  %d  %.16g\n", i + 1, ci[k] + 1, v[k]);
  Free(rp);
  Free(ci);
  Free(v);
}

void LinAlg_WriteScalar(FILE *file, gScalar *S)
{
  Message::Error("'LinAlg_WriteScalar' not yet implemented");
}

void LinAlg_WriteVector(FILE *file, gVector *V)
{
  host(V);
  fwrite(V->V, sizeof(double), V->N, file);
  fprintf(file, "\n");
}

void LinAlg_WriteMatrix(FILE *file, gMatrix *M)
{
  LinAlg_PrintMatrix(file, M, false, nullptr, nullptr);
}

void LinAlg_GetVectorSize(gVector *V, int *i) { *i = V->N; }

void LinAlg_GetLocalVectorRange(gVector *V, int *low, int *high)
{
  *low = 0;
  *high = V->N;
}

void LinAlg_GetMatrixSize(gMatrix *M, int *i, int *j)
{
  gb300_matrix_size(M->M, i);
  *j = *i;
}

void LinAlg_GetLocalMatrixRange(gMatrix *M, int *low, int *high)
{
  *low = 0;
  gb300_matrix_size(M->M, high);
}

void LinAlg_GetDoubleInScalar(double *d, gScalar *S) { *d = S->s; }

void LinAlg_GetComplexInScalar(double *d1, double *d2, gScalar *S)
{
  Message::Error("'LinAlg_GetComplexInScalar' not available with this Solver");
}

void LinAlg_GetScalarInVector(gScalar *S, gVector *V, int i)
{
  host(V);
  S->s = V->V[i];
}

void LinAlg_GetDoubleInVector(double *d, gVector *V, int i)
{
  host(V);
  *d = V->V[i];
}

void LinAlg_GetAbsDoubleInVector(double *d, gVector *V, int i)
{
  host(V);
  *d = fabs(V->V[i]);
}

void LinAlg_GetComplexInVector(double *d1, double *d2, gVector *V, int i, int j)
{
  host(V);
  *d1 = V->V[i];
  *d2 = V->V[j];
}

void LinAlg_GetScalarInMatrix(gScalar *S, gMatrix *M, int i, int j)
{
  Message::Error("'LinAlg_GetScalarInMatrix' not yet implemented");
}

void LinAlg_GetDoubleInMatrix(double *d, gMatrix *M, int i, int j)
{
  ok(gb300_matrix_assemble(M->M));
  int n = 0;
  long long nnz = 0;
  gb300_matrix_size(M->M, &n);
  gb300_matrix_nnz(M->M, &nnz);
  int *rp = (int *)Malloc((n + 1) * sizeof(int));
  int *ci = (int *)Malloc((nnz ? nnz : 1) * sizeof(int));
  double *v = (double *)Malloc((nnz ? nnz : 1) * sizeof(double));
  ok(gb300_matrix_get_csr(M->M, rp, ci, v));
  *d = 0.;
  for(int k = rp[i]; k < rp[i + 1]; k++)
    if(ci[k] == j) *d = v[k];
  Free(rp);
  Free(ci);
  Free(v);
}

void LinAlg_GetComplexInMatrix(double *d1, double *d2, gMatrix *M, int i, int j,
                               int k, int l)
{
  Message::Error("'LinAlg_GetComplexInMatrix' not yet implemented");
}

void LinAlg_GetColumnInMatrix(gMatrix *M, int col, gVector *V1)
{
  ok(gb300_matrix_assemble(M->M));
  int n = 0;
  long long nnz = 0;
  gb300_matrix_size(M->M, &n);
  gb300_matrix_nnz(M->M, &nnz);
  int *rp = (int *)Malloc((n + 1) * sizeof(int));
  int *ci = (int *)Malloc((nnz ? nnz : 1) * sizeof(int));
  double *v = (double *)Malloc((nnz ? nnz : 1) * sizeof(double));
  ok(gb300_matrix_get_csr(M->M, rp, ci, v));
  host_w(V1);
  for(int i = 0; i < n; i++) {
    V1->V[i] = 0.;
    for(int k = rp[i]; k < rp[i + 1]; k++)
      if(ci[k] == col) V1->V[i] = v[k];
  }
  Free(rp);
  Free(ci);
  Free(v);
}

void LinAlg_SetScalar(gScalar *S, double *d) { S->s = d[0]; }

void LinAlg_SetVector(gVector *V, double *v)
{
  for(int i = 0; i < V->N; i++) V->V[i] = *v;
  V->state = HOST;
}

void LinAlg_SetScalarInVector(gScalar *S, gVector *V, int i)
{
  host_w(V);
  V->V[i] = S->s;
}

void LinAlg_SetDoubleInVector(double d, gVector *V, int i)
{
  host_w(V);
  V->V[i] = d;
}

void LinAlg_SetComplexInVector(double d1, double d2, gVector *V, int i, int j)
{
  host_w(V);
  V->V[i] = d1;
  V->V[j] = d2;
}

void LinAlg_SetScalarInMatrix(gScalar *S, gMatrix *M, int i, int j)
{
  Message::Error("'LinAlg_SetScalarInMatrix' not yet implemented");
}

void LinAlg_SetDoubleInMatrix(double d, gMatrix *M, int i, int j)
{
  Message::Error("'LinAlg_SetDoubleInMatrix' not yet implemented");
}

void LinAlg_SetComplexInMatrix(double d1, double d2, gMatrix *M, int i, int j,
                               int k, int l)
{
  Message::Error("'LinAlg_SetComplexInMatrix' not yet implemented");
}

void LinAlg_AddScalarScalar(gScalar *S1, gScalar *S2, gScalar *S3)
{
  S3->s = S1->s + S2->s;
}

void LinAlg_DummyVector(gVector *V)
{
  int *DummyDof = Current.DofData->DummyDof;
  if(!DummyDof) return;
  host_w(V);
  for(int i = 0; i < V->N; i++)
    if(DummyDof[i] == 1) V->V[i] = 0;
}

void LinAlg_AddScalarInVector(gScalar *S, gVector *V, int i)
{
  int *DummyDof;
  if((DummyDof = Current.DofData->DummyDof))
    if(DummyDof[i] == 1) return;
  host_w(V);
  V->V[i] += S->s;
}

void LinAlg_AddDoubleInVector(double d, gVector *V, int i)
{
  int *DummyDof;
  if((DummyDof = Current.DofData->DummyDof))
    if(DummyDof[i] == 1) return;
  host_w(V);
  V->V[i] += d;
}

void LinAlg_AddComplexInVector(double d1, double d2, gVector *V, int i, int j)
{
  int *DummyDof, iok = 1, jok = 1;
  if((DummyDof = Current.DofData->DummyDof)) {
    if(DummyDof[i] == 1) iok = 0;
    if(DummyDof[j] == 1) jok = 0;
  }
  host_w(V);
  if(iok) V->V[i] += d1;
  if(jok) V->V[j] += d2;
}

void LinAlg_AddScalarInMatrix(gScalar *S, gMatrix *M, int i, int j)
{
  LinAlg_AddDoubleInMatrix(S->s, M, i, j);
}

void LinAlg_AddDoubleInMatrix(double d, gMatrix *M, int i, int j)
{
  int *DummyDof;
  if((DummyDof = Current.DofData->DummyDof))
    if((DummyDof[i] == 1 || DummyDof[j] == 1) && (i != j)) return;
  touched(M);
  ok(gb300_matrix_add_double(M->M, d, i, j));
}

void LinAlg_AddComplexInMatrix(double d1, double d2, gMatrix *M, int i, int j,
                               int k, int l)
{
  touched(M);
  ok(gb300_matrix_add_complex(M->M, d1, d2, i, j, k, l));
}

void LinAlg_AddVectorVector(gVector *V1, gVector *V2, gVector *V3)
{
  if(V3 != V1) {
    Message::Error("Wrong arguments in 'LinAlg_AddVectorVector'");
    return;
  }
  host(V2);
  host_w(V1);
  for(int i = 0; i < V1->N; i++) V1->V[i] += V2->V[i];
}

void LinAlg_AddVectorProdVectorDouble(gVector *V1, gVector *V2, double d,
                                      gVector *V3)
{
  if(V3 != V1) {
    Message::Error("Wrong arguments in 'LinAlg_AddVectorProdVectorDouble'");
    return;
  }
  host(V2);
  host_w(V1);
  for(int i = 0; i < V1->N; i++) V1->V[i] += d * V2->V[i];
}

void LinAlg_AddProdVectorDoubleProdVectorDouble(double alpha, gVector *V1,
                                                double beta, gVector *V2,
                                                gVector *V3)
{
  Message::Error(
    "'LinAlg_AddProdVectorDoubleProdVectorDouble' not yet implemented");
}

// M1 <- M1 + d * M2 through the staged adds (entries of M2 in row order)
static void add_scaled(gMatrix *M1, gMatrix *M2, double d)
{
  ok(gb300_matrix_assemble(M2->M));
  int n = 0;
  long long nnz = 0;
  gb300_matrix_size(M2->M, &n);
  gb300_matrix_nnz(M2->M, &nnz);
  int *rp = (int *)Malloc((n + 1) * sizeof(int));
  int *ci = (int *)Malloc((nnz ? nnz : 1) * sizeof(int));
  int *ri = (int *)Malloc((nnz ? nnz : 1) * sizeof(int));
  double *v = (double *)Malloc((nnz ? nnz : 1) * sizeof(double));
  ok(gb300_matrix_get_csr(M2->M, rp, ci, v));
  for(int i = 0; i < n; i++)
    for(int k = rp[i]; k < rp[i + 1]; k++) {
      ri[k] = i;
      v[k] *= d;
    }
  touched(M1);
  ok(gb300_matrix_add_coo(M1->M, nnz, ri, ci, v));
  Free(rp);
  Free(ci);
  Free(ri);
  Free(v);
}

void LinAlg_AddMatrixMatrix(gMatrix *M1, gMatrix *M2, gMatrix *M3)
{
  if(M3 == M1)
    add_scaled(M1, M2, 1.);
  else if(M3 == M2)
    add_scaled(M2, M1, 1.);
  else
    Message::Error("Wrong arguments in 'LinAlg_AddMatrixMatrix'");
}

void LinAlg_AddMatrixProdMatrixDouble(gMatrix *M1, gMatrix *M2, double d,
                                      gMatrix *M3)
{
  if(M3 == M1)
    add_scaled(M1, M2, d);
  else
    Message::Error("Wrong arguments in 'LinAlg_AddMatrixProdMatrixDouble'");
}

void LinAlg_SubScalarScalar(gScalar *S1, gScalar *S2, gScalar *S3)
{
  S3->s = S1->s - S2->s;
}

void LinAlg_SubVectorVector(gVector *V1, gVector *V2, gVector *V3)
{
  host(V1);
  host(V2);
  if(V3 == V1) {
    host_w(V1);
    for(int i = 0; i < V1->N; i++) V1->V[i] -= V2->V[i];
  }
  else if(V3 == V2) {
    host_w(V2);
    for(int i = 0; i < V1->N; i++) V2->V[i] = V1->V[i] - V2->V[i];
  }
  else
    Message::Error("Wrong arguments in 'LinAlg_SubVectorVector'");
}

void LinAlg_SubMatrixMatrix(gMatrix *M1, gMatrix *M2, gMatrix *M3)
{
  Message::Error("'LinAlg_SubMatrixMatrix' not yet implemented");
}

void LinAlg_ProdScalarScalar(gScalar *S1, gScalar *S2, gScalar *S3)
{
  S3->s = S1->s * S2->s;
}

void LinAlg_ProdScalarDouble(gScalar *S1, double d, gScalar *S2)
{
  S2->s = S1->s * d;
}

void LinAlg_ProdScalarComplex(gScalar *S, double d1, double d2, double *d3,
                              double *d4)
{
  *d3 = S->s * d1;
  *d4 = S->s * d2;
}

void LinAlg_ProdVectorScalar(gVector *V1, gScalar *S, gVector *V2)
{
  Message::Error("'LinAlg_ProdVectorScalar' not yet implemented");
}

void LinAlg_ProdVectorDouble(gVector *V1, double d, gVector *V2)
{
  if(V2 != V1) {
    Message::Error("Wrong arguments in 'LinAlg_ProdVectorDouble'");
    return;
  }
  host_w(V1);
  for(int i = 0; i < V1->N; i++) V1->V[i] *= d;
}

void LinAlg_ProdVectorComplex(gVector *V1, double d1, double d2, gVector *V2)
{
  Message::Error("'LinAlg_ProdVectorComplex' not yet implemented");
}

void LinAlg_ProdVectorVector(gVector *V1, gVector *V2, double *d)
{
  host(V1);
  host(V2);
  *d = 0.;
  for(int i = 0; i < V1->N; i++) *d += V1->V[i] * V2->V[i];
}

void LinAlg_ProdMatrixVector(gMatrix *M, gVector *V1, gVector *V2)
{
  if(V2 == V1) {
    Message::Error("Wrong arguments in 'LinAlg_ProdMatrixVector'");
    return;
  }
  dev(V1);
  ok(gb300_matrix_mult(M->M, V1->D, V2->D));
  V2->state = DEV;
}

static void scale_matrix(gMatrix *M, double d)
{
  ok(gb300_matrix_assemble(M->M));
  int n = 0;
  long long nnz = 0;
  gb300_matrix_size(M->M, &n);
  gb300_matrix_nnz(M->M, &nnz);
  int *rp = (int *)Malloc((n + 1) * sizeof(int));
  int *ci = (int *)Malloc((nnz ? nnz : 1) * sizeof(int));
  double *v = (double *)Malloc((nnz ? nnz : 1) * sizeof(double));
  ok(gb300_matrix_get_csr(M->M, rp, ci, v));
  for(long long k = 0; k < nnz; k++) v[k] *= d;
  ok(gb300_matrix_set_csr(M->M, nnz, rp, ci, v));
  Free(rp);
  Free(ci);
  Free(v);
}

void LinAlg_ProdMatrixScalar(gMatrix *M1, gScalar *S, gMatrix *M2)
{
  if(M2 == M1)
    scale_matrix(M1, S->s);
  else
    Message::Error("Wrong arguments in 'LinAlg_ProdMatrixScalar'");
}

void LinAlg_ProdMatrixDouble(gMatrix *M1, double d, gMatrix *M2)
{
  if(M2 == M1)
    scale_matrix(M1, d);
  else
    Message::Error("Wrong arguments in 'LinAlg_ProdMatrixDouble'");
}

void LinAlg_ProdMatrixComplex(gMatrix *M1, double d1, double d2, gMatrix *M2)
{
  Message::Error("'LinAlg_ProdMatrixComplex' not yet implemented");
}

void LinAlg_DivScalarScalar(gScalar *S1, gScalar *S2, gScalar *S3)
{
  S3->s = S1->s / S2->s;
}

void LinAlg_DivScalarDouble(gScalar *S1, double d, gScalar *S2)
{
  S2->s = S1->s / d;
}

void LinAlg_VectorNorm2(gVector *V1, double *norm)
{
  host(V1);
  double s = 0.;
  for(int i = 0; i < V1->N; i++) s += V1->V[i] * V1->V[i];
  *norm = sqrt(s);
}

void LinAlg_VectorNormInf(gVector *V1, double *norm)
{
  host(V1);
  *norm = 0.;
  for(int i = 0; i < V1->N; i++)
    if(fabs(V1->V[i]) > *norm) *norm = fabs(V1->V[i]);
}

void LinAlg_AssembleMatrix(gMatrix *M) { ok(gb300_matrix_assemble(M->M)); }

void LinAlg_AssembleVector(gVector *V) {}

// Sparskit's threshold and level-of-fill ILUs (Preconditioner 1 ILUT,
// 2 ILUTP -- the default of Sparskit.cpp:1854 --, 3 ILUD, 4 ILUDP, 5 ILUK,
// 7 MILU0) have no GPU counterpart here: the solve runs with ILU(0)
// (Preconditioner 6) and says so once per run.
static gb300_solver_params gpu_params(const gb300_solver_params &p)
{
  gb300_solver_params q = p;
  if((p.preconditioner >= 1 && p.preconditioner <= 5) || p.preconditioner == 7) {
    static int warned = 0;
    if(!warned) {
      Message::Warning("GB300 backend: Preconditioner %d is not available on the GPU; "
                       "ILU(0) (Preconditioner 6) is used instead", p.preconditioner);
      warned = 1;
    }
    q.preconditioner = 6;
  }
  return q;
}

void LinAlg_Solve(gMatrix *A, gVector *B, gSolver *Solver, gVector *X,
                  int solverIndex)
{
  gb300_solve_info info;
  dev(B);
  gb300_solver_params params = gpu_params(Solver->Params);
  int rc = gb300_solve(A->M, B->D, &params, X->D, &info);
  X->state = DEV;
  if(rc == GB300_ERR_SOLVER)  // Sparskit only warns when iterations fail
    Message::Warning("Iterative solver terminated (code = %d)", info.status);
  else
    ok(rc);
  Message::Info("%d Iterations / Residual: %g", info.iterations,
                info.true_residual);
}

// the factorisation of the previous solve of A is reused, as the reference
// sets Re_Use_LU for this call (LinAlg_SPARSKIT.cpp:578-585)
void LinAlg_SolveAgain(gMatrix *A, gVector *B, gSolver *Solver, gVector *X,
                       int solverIndex)
{
  int tmp = Solver->Params.re_use_lu;
  Solver->Params.re_use_lu = 1;
  LinAlg_Solve(A, B, Solver, X, solverIndex);
  Solver->Params.re_use_lu = tmp;
}

void LinAlg_SolveNL(gMatrix *A, gVector *B, gMatrix *J, gVector *R,
                    gSolver *Solver, gVector *X, int solverIndex)
{
  Message::Error("'LinAlg_SolveNL' not yet implemented for GB300");
}

#endif
