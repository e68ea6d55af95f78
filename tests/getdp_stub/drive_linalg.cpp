// GetDP's linear-algebra call sequence, through the unchanged backend file
// getdp_gb300/getdp_backend/LinAlg_GB300.cpp and the real library, without
// GetDP itself: the calls Generate / Solve / SolveAgain / GetResidual make
// (SolvingOperations.cpp: ZeroMatrix, one LinAlg_AddDoubleInMatrix per
// entry in the element loop's order, AssembleMatrix, LinAlg_Solve ...).
// Test infrastructure.
//
// usage: drive_linalg SYSTEM OUT [-Name value ...]
//   SYSTEM: int32 n, int64 m, int32 rows[m], int32 cols[m], float64 vals[m],
//           float64 rhs[n] (the entries in the order GetDP would add them)
//   OUT:    float64 x[n] (LinAlg_Solve), float64 x2[n] (a second Generate of
//           the same system, LinAlg_SolveAgain with 2 b), float64 ||b - A x||
//   options: passed to LinAlg_InitializeSolver as on GetDP's command line
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "LinAlg.h"
#include "Message.h"

static void need(bool c, const char *what)
{
  if(!c) Message::Error("drive_linalg: %s", what);
}

int main(int argc, char **argv)
{
  need(argc >= 3, "usage: drive_linalg SYSTEM OUT [-Name value ...]");
  FILE *f = fopen(argv[1], "rb");
  need(f != nullptr, "cannot open the system file");
  int n = 0;
  long long m = 0;
  need(fread(&n, sizeof(int), 1, f) == 1 && fread(&m, sizeof(long long), 1, f) == 1,
       "short system file");
  need(n > 0 && m > 0, "empty system");
  std::vector<int> ri(m), ci(m);
  std::vector<double> v(m), rhs(n);
  need(fread(ri.data(), sizeof(int), m, f) == (size_t)m &&
         fread(ci.data(), sizeof(int), m, f) == (size_t)m &&
         fread(v.data(), sizeof(double), m, f) == (size_t)m &&
         fread(rhs.data(), sizeof(double), n, f) == (size_t)n,
       "short system file");
  fclose(f);

  // the solver options, as GetDP hands its command line over
  int sargc = argc - 2;
  std::vector<char *> sargv(argv + 2, argv + argc);
  sargv[0] = argv[0];
  char **pargv = sargv.data();
  LinAlg_InitializeSolver(&sargc, &pargv);

  gSolver S;
  gMatrix A;
  gVector b, x, r, b2, x2;
  LinAlg_CreateSolver(&S, nullptr);
  LinAlg_CreateMatrix(&A, &S, n, n);
  LinAlg_CreateVector(&b, &S, n);
  LinAlg_CreateVector(&x, &S, n);
  LinAlg_CreateVector(&r, &S, n);
  LinAlg_CreateVector(&b2, &S, n);
  LinAlg_CreateVector(&x2, &S, n);

  for(int pass = 0; pass < 2; pass++) {
    // Generate: ZeroMatrix / ZeroVector, then the element loop's adds
    LinAlg_ZeroMatrix(&A);
    LinAlg_ZeroVector(&b);
    for(long long k = 0; k < m; k++) LinAlg_AddDoubleInMatrix(v[k], &A, ri[k], ci[k]);
    for(int i = 0; i < n; i++) LinAlg_AddDoubleInVector(rhs[i], &b, i);
    LinAlg_AssembleMatrix(&A);
    LinAlg_AssembleVector(&b);
    if(pass == 0) {
      LinAlg_Solve(&A, &b, &S, &x, 0);
      // GetResidual: r = b - A x, ||r||
      LinAlg_ProdMatrixVector(&A, &x, &r);
      LinAlg_SubVectorVector(&b, &r, &r);
    }
    else {
      // b2 = 2 b (ProdVectorDouble scales in place, as in Sparskit's backend)
      LinAlg_CopyVector(&b, &b2);
      LinAlg_ProdVectorDouble(&b2, 2., &b2);
      LinAlg_SolveAgain(&A, &b2, &S, &x2, 0);
    }
  }
  double rn = 0.;
  LinAlg_VectorNorm2(&r, &rn);

  std::vector<double> hx(n), hx2(n);
  for(int i = 0; i < n; i++) {
    LinAlg_GetDoubleInVector(&hx[i], &x, i);
    LinAlg_GetDoubleInVector(&hx2[i], &x2, i);
  }
  FILE *o = fopen(argv[2], "wb");
  need(o != nullptr, "cannot write the output file");
  fwrite(hx.data(), sizeof(double), n, o);
  fwrite(hx2.data(), sizeof(double), n, o);
  fwrite(&rn, sizeof(double), 1, o);
  fclose(o);
  LinAlg_DestroyVector(&b);
  LinAlg_DestroyVector(&x);
  LinAlg_DestroyVector(&r);
  LinAlg_DestroyVector(&b2);
  LinAlg_DestroyVector(&x2);
  LinAlg_DestroyMatrix(&A);
  LinAlg_DestroySolver(&S);
  LinAlg_FinalizeSolver();
  return 0;
}
