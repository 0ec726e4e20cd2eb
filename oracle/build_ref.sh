#!/bin/sh
# Builds the reference's own quasi-static shear step, its general multigrid
# on the poisson_fd problem class and the coord_transforms variant of the
# step from their sources, read in place under the reference tree, into
# oracle/_ref/libstzref.so, libtgmgref.so and libctref.so (test-only).
#
#   oracle/build_ref.sh [REFERENCE_ROOT]
#   oracle/build_ref.sh --root     prints the reference tree it would use and
#                                  exits 0, or exits 2 when it is absent
#
# REFERENCE_ROOT defaults to $STZ_REFERENCE_ROOT, else /root/reference.
#
# Recipe (the reference's own make files are not used):
#   1. esim/tgmg/tgmg_compile.pl expands tgmg.in.cc into tgmg.cc.  The script
#      reads ./tgmg.in.cc and writes ./tgmg.cc, so it runs in a scratch
#      directory under oracle/_ref/ holding a symlink to tgmg.in.cc; the
#      scratch directory is deleted after compiling.
#   2. g++ compiles esim/sb/main/{shear_sim,qs_multi,common}.cc and
#      esim/shared/mat.cc with the reference's flags (esim/config/
#      config.mk.linux:4: -Wall -ansi -pedantic -fopenmp -O3) plus -fPIC,
#      together with oracle/ref_driver.cc, into one shared library;
#   3. g++ compiles esim/tgmg/poisson_fd.cc (which includes the generated
#      tgmg.cc and instantiates tgmg<poisson_fd,double,double>) with
#      oracle/ref_tgmg_driver.cc into a second one;
#   4. g++ compiles esim/coord_transforms/simple_shear/{shear_sim,qs_multi,
#      common,extra,bi_interp}.cc and esim/shared/mat.cc with
#      oracle/ref_ct_driver.cc into a third one (that directory first on the
#      include path: its headers share names with esim/sb/main's).
# Only x86/Arm-neutral flags are used; nothing here runs on the GPU.
set -e
DEFAULT_REF=${STZ_REFERENCE_ROOT:-/root/reference}
if [ "$1" = "--root" ]; then
    [ -f "$DEFAULT_REF/esim/tgmg/tgmg.in.cc" ] || exit 2
    echo "$DEFAULT_REF"
    exit 0
fi
REF=${1:-$DEFAULT_REF}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
ESIM="$REF/esim"
if [ ! -f "$ESIM/tgmg/tgmg.in.cc" ]; then
    echo "build_ref: reference sources not found under $REF" >&2
    exit 2
fi
mkdir -p "$OUT"
GEN="$OUT/gen"
rm -rf "$GEN"
mkdir -p "$GEN"
ln -s "$ESIM/tgmg/tgmg.in.cc" "$GEN/tgmg.in.cc"
(cd "$GEN" && perl "$ESIM/tgmg/tgmg_compile.pl")
CXX=${CXX:-g++}
FLAGS="-Wall -ansi -pedantic -fopenmp -O3 -fPIC -Wno-unused-variable -Wno-unused-but-set-variable"
INC="-I$GEN -I$ESIM/tgmg -I$ESIM/shared -I$ESIM/sb/main"
OBJ="$OUT/obj"
mkdir -p "$OBJ"
$CXX $FLAGS $INC -c "$ESIM/sb/main/shear_sim.cc" -o "$OBJ/shear_sim.o" &
$CXX $FLAGS $INC -c "$ESIM/sb/main/qs_multi.cc" -o "$OBJ/qs_multi.o" &
$CXX $FLAGS $INC -c "$ESIM/sb/main/common.cc" -o "$OBJ/common.o" &
$CXX $FLAGS $INC -c "$ESIM/shared/mat.cc" -o "$OBJ/mat.o" &
$CXX $FLAGS $INC -c "$HERE/ref_driver.cc" -o "$OBJ/ref_driver.o" &
TG="$OUT/objtg"
mkdir -p "$TG"
$CXX $FLAGS $INC -c "$ESIM/tgmg/poisson_fd.cc" -o "$TG/poisson_fd.o" &
$CXX $FLAGS $INC -c "$HERE/ref_tgmg_driver.cc" -o "$TG/ref_tgmg_driver.o" &
CT="$OUT/objct"
CTD="$ESIM/coord_transforms/simple_shear"
CTINC="-I$CTD -I$GEN -I$ESIM/tgmg -I$ESIM/shared"
mkdir -p "$CT"
for f in shear_sim qs_multi common extra bi_interp; do
    $CXX $FLAGS $CTINC -c "$CTD/$f.cc" -o "$CT/$f.o" &
done
$CXX $FLAGS $CTINC -c "$ESIM/shared/mat.cc" -o "$CT/mat.o" &
$CXX $FLAGS $CTINC -c "$HERE/ref_ct_driver.cc" -o "$CT/ref_ct_driver.o" &
wait
$CXX -shared -fopenmp -o "$OUT/libstzref.so" "$OBJ"/*.o
$CXX -shared -fopenmp -o "$OUT/libtgmgref.so" "$TG"/*.o
$CXX -shared -fopenmp -o "$OUT/libctref.so" "$CT"/*.o
rm -rf "$GEN" "$OBJ" "$TG" "$CT"
echo "build_ref: wrote $OUT/libstzref.so $OUT/libtgmgref.so $OUT/libctref.so"
