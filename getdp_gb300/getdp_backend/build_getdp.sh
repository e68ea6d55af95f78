#!/bin/bash
# Build GetDP with the GB300 linear-algebra backend (LinAlg_GB300.cpp) from
# a GetDP source tree, without CMake, the way a maintainer would wire it:
#   * LinAlg.h gains a HAVE_GB300 branch declaring the backend's types (the
#     source tree is not modified: a patched copy goes to the build folder
#     and comes first on the include path);
#   * the dummy backend LinAlg.cpp and the Sparskit/PETSc backends are left
#     out; LinAlg_GB300.cpp is compiled instead;
#   * Treatment_Formulation.cpp gains the batched Generate hook
#     (Generate_GB300.cpp): a patched copy in the build folder, as for LinAlg.h;
#   * the program links against getdp_gb300/_build/libgetdp_gb300.so.
# Usage: build_getdp.sh GETDP_SOURCE_DIR [OUT_DIR]
set -euo pipefail
SRC=${1:?GetDP source directory}
HERE=$(cd "$(dirname "$0")" && pwd)
PKG=$(dirname "$HERE")
ROOT=$(dirname "$PKG")
OUT=${2:-$PKG/_build/getdp_backend}
OBJ=$OUT/obj
mkdir -p "$OBJ" "$OUT/include"

# configuration: kernel + GB300 backend
cat > "$OUT/include/GetDPConfig.h" <<'EOF'
#ifndef GETDP_CONFIG_H
#define GETDP_CONFIG_H
#define HAVE_KERNEL
#define HAVE_GB300
#define HAVE_NO_FORTRAN
#define GETDP_CONFIG_OPTIONS "64Bit Kernel GB300 NoFortran"
#endif
EOF
cp "$ROOT/oracle/ref_config/GetDPVersion.h" "$OUT/include/GetDPVersion.h"

# LinAlg.h with the GB300 branch in front of the Sparskit one
python3 - "$SRC/src/kernel/LinAlg.h" "$OUT/include/LinAlg.h" <<'EOF'
import sys
src, dst = sys.argv[1], sys.argv[2]
s = open(src).read()
branch = '''#if defined(HAVE_GB300)

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

#elif defined(HAVE_SPARSKIT)'''
assert s.count("#if defined(HAVE_SPARSKIT)") == 1
open(dst, "w").write(s.replace("#if defined(HAVE_SPARSKIT)", branch))
EOF

# a shadow tree of symbolic links, so that every quoted #include "LinAlg.h"
# (searched first in the including file's folder) finds the patched copy
SH=$OUT/shadow
rm -rf "$SH"
for d in common kernel functions interface numeric main; do
  mkdir -p "$SH/$d"
  for f in "$SRC/src/$d"/*; do ln -s "$f" "$SH/$d/$(basename "$f")"; done
done
rm "$SH/kernel/LinAlg.h"
cp "$OUT/include/LinAlg.h" "$SH/kernel/LinAlg.h"
rm "$OUT/include/LinAlg.h"

# Treatment_Formulation.cpp with the batched Generate hook (Generate_GB300.cpp):
# before the element loop of a Generate the hook gathers the terms the GPU
# kernels evaluate and submits them as one batch; the loop then skips those
# (term, element) pairs
rm "$SH/kernel/Treatment_Formulation.cpp"
python3 - "$SRC/src/kernel/Treatment_Formulation.cpp" "$SH/kernel/Treatment_Formulation.cpp" <<'HOOKEOF'
import sys
src, dst = sys.argv[1], sys.argv[2]
s = open(src).read()
decl = """#if defined(HAVE_GB300)
int GB300_Generate_Begin(struct EquationTerm *EquationTerm_P0, int Nbr_EquationTerm,
                         struct QuantityStorage *QuantityStorage_P0,
                         struct Group *Generate_Group);
int GB300_Generate_Skip(int i_EquTerm, int element_num);
#endif

void Treatment_FemFormulation(struct Formulation *Formulation_P)
"""
a = "void Treatment_FemFormulation(struct Formulation *Formulation_P)\n"
assert s.count(a) == 1
s = s.replace(a, decl)
b = "  /*     Treatment of eventual GALERKIN terms                   */\n"
assert s.count(b) == 1
s = s.replace(b, b + """#if defined(HAVE_GB300)
  const int gb300_hook =
    (TreatmentStatus == STATUS_CAL) ?
      GB300_Generate_Begin(EquationTerm_P0, Nbr_EquationTerm, QuantityStorage_P0,
                           Generate_Group) :
      0;
#endif
""")
c = """                Cal_GalerkinTermOfFemEquation(&Element, EquationTerm_P,
                                              QuantityStorage_P0);

                /* if multiple candidate Trace elements"""
assert s.count(c) == 1
s = s.replace(c, """#if defined(HAVE_GB300)
                if(!gb300_hook || !GB300_Generate_Skip(i_EquTerm, Element.Num))
#endif
""" + c)
open(dst, "w").write(s)
HOOKEOF

INC="-I$OUT/include -I$ROOT/include -I$SH/common -I$SH/kernel \
 -I$SH/functions -I$SH/interface -I$SH/numeric"
CXXFLAGS="-O2 -std=c++11 -w -fno-strict-aliasing"
SRCS=$(ls $SH/kernel/*.cpp $SH/functions/*.cpp $SH/interface/*.cpp \
          $SH/numeric/*.cpp $SH/common/*.cpp $SH/main/Main.cpp |
       grep -v -e '/LinAlg.cpp$' -e '/LinAlg_SPARSKIT.cpp$' -e '/LinAlg_PETSC.cpp$')
SRCS="$SRCS $HERE/LinAlg_GB300.cpp $HERE/Generate_GB300.cpp"
printf '%s\n' $SRCS | xargs -P "${JOBS:-$(nproc)}" -I{} bash -c '
  s={}; o='"$OBJ"'/$(echo "$s" | sed "s|/|_|g; s|\.cpp$|.o|")
  if [ ! -f "$o" ] || [ "$s" -nt "$o" ]; then g++ '"$CXXFLAGS $INC"' -c "$s" -o "$o"; fi'
LIB=$PKG/_build
g++ -o "$OUT/getdp" $OBJ/*.o -L"$LIB" -lgetdp_gb300 -Wl,-rpath,"$LIB" -lm
echo "built $OUT/getdp"
