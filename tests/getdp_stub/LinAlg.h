/* Stand-in for GetDP's src/kernel/LinAlg.h with the GB300 branch only: the
   backend's types (the same bodies getdp_backend/build_getdp.sh adds to the
   real header) and the prototypes of the functions LinAlg_GB300.cpp defines,
   generated from that file (linalg_protos.h, made by the test that builds
   the driver).  Test infrastructure. */
#ifndef LINALG_STUB_H
#define LINALG_STUB_H
#include <stdio.h>

#include <string>

#include "getdp_gb300.h"
#define gSCALAR_SIZE 1
#define gCOMPLEX_INCREMENT 2
typedef struct {
  double s;
} gScalar;
typedef struct {
  gb300_matrix *M;
} gMatrix;
typedef struct {
  int N;
  double *V;
  gb300_vector *D;
  int state;
} gVector;
typedef struct {
  gb300_solver_params Params;
} gSolver;

#include "linalg_protos.h"
#endif
