#!/bin/bash
# Compile the reference GetDP 3.5.0 (read-only sources) into oracle/_ref/
# without its CMake system: every kernel/functions/interface/numeric/common
# source plus contrib/Sparskit/Sparskit.cpp, compiled directly with g++ and
# linked against oracle/sparskit_port.c (the C restatement of the Sparskit
# Fortran routines; no Fortran compiler exists in this image).
#
# Two binaries are produced:
#   oracle/_ref/getdp_ilu32  -- HAVE_ILU_FLOAT, as the official build
#   oracle/_ref/getdp_ilu64  -- double-precision ILU, the strict FP64 oracle
#
# The path of the sources it compiled is recorded in oracle/_ref/source_dir,
# where the tests that read the reference's own files (examples/, src/) find
# it (oracle/refsrc.py).
#
# Usage: oracle/build_ref.sh [--optional] [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $GETDP_SOURCE_DIR, else /root/reference (the
#   development container); --optional exits 0 without building when the
#   sources are absent (the GPU hosts, which get no reference sources).
set -euo pipefail
OPTIONAL=0
if [ "${1:-}" = "--optional" ]; then OPTIONAL=1; shift; fi
REF=${1:-${GETDP_SOURCE_DIR:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/_ref
OBJ=$OUT/obj
if [ ! -d "$REF/src/kernel" ]; then
  [ $OPTIONAL = 1 ] && exit 0
  echo "reference sources not found at $REF" >&2; exit 1
fi
mkdir -p "$OBJ"
echo "$REF" > "$OUT/source_dir"
INC="-I$HERE/ref_config -I$REF/src/common -I$REF/src/kernel -I$REF/src/functions \
 -I$REF/src/interface -I$REF/src/numeric -I$REF/contrib/Sparskit"
CXXFLAGS="-O2 -std=c++11 -w -fno-strict-aliasing"
SRCS=$(ls $REF/src/kernel/*.cpp $REF/src/functions/*.cpp $REF/src/interface/*.cpp \
          $REF/src/numeric/*.cpp $REF/src/common/*.cpp $REF/src/main/Main.cpp)
JOBS=${JOBS:-$(nproc)}
# compile the shared objects in parallel, skipping up-to-date ones
printf '%s\n' $SRCS | xargs -P "$JOBS" -I{} bash -c '
  src={}; o='"$OBJ"'/$(echo "$src" | sed "s|'"$REF"'/||; s|/|_|g; s|\.cpp$|.o|")
  if [ ! -f "$o" ] || [ "$src" -nt "$o" ]; then g++ '"$CXXFLAGS $INC"' -c "$src" -o "$o"; fi'
for prec in 32 64; do
  DEF=""; [ $prec = 32 ] && DEF="-DHAVE_ILU_FLOAT"
  g++ $CXXFLAGS $INC $DEF -c $REF/contrib/Sparskit/Sparskit.cpp -o $OBJ/Sparskit_ilu$prec.o
  gcc -O2 -w $DEF -c $HERE/sparskit_port.c -o $OBJ/sparskit_port_ilu$prec.o
  g++ -o $OUT/getdp_ilu$prec $(ls $OBJ/src_*.o) $OBJ/Sparskit_ilu$prec.o \
      $OBJ/sparskit_port_ilu$prec.o -lm
done
echo "built $OUT/getdp_ilu32 $OUT/getdp_ilu64"
