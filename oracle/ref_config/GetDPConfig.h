/* Configuration header for compiling the reference GetDP 3.5.0 from its own
   sources without its CMake system: kernel + Sparskit backend, no Fortran,
   no PETSc/GSL/Gmsh/BLAS.  Used only by oracle/build_ref.sh. */
#ifndef GETDP_CONFIG_H
#define GETDP_CONFIG_H
#define HAVE_KERNEL
#define HAVE_SPARSKIT
#define HAVE_NO_FORTRAN
#define GETDP_CONFIG_OPTIONS "64Bit Kernel Sparskit(C restatement) NoFortran"
#endif
