/* Stand-in for GetDP's generated configuration header: the GB300 backend
   alone (no Sparskit, no PETSc).  Test infrastructure: it lets the backend
   file getdp_gb300/getdp_backend/LinAlg_GB300.cpp compile and run on a
   machine without GetDP's sources. */
#ifndef GETDP_CONFIG_H
#define GETDP_CONFIG_H
#define HAVE_GB300
#endif
