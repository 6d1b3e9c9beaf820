#!/usr/bin/env bash
# Builds the reference's own gather-scatter library (NekCEM src/jl, C99) from
# the reference source tree into oracle/_ref/libjlgs.so, with the test shim
# oracle/jlgs_driver.c.  Single process: no -DMPI, so jl's comm.h uses its
# serial branch.  Only the sources the gs path needs are compiled.  Test
# infrastructure only; outputs go to oracle/_ref/ (git-ignored).
#
# usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $NEKCEM_REFERENCE_ROOT, else /root/reference.
#   Exit status 3 (nothing built) when the reference tree is not there: the
#   GPU machines carry the built library in oracle/_ref/ instead.
set -euo pipefail
REF="${1:-${NEKCEM_REFERENCE_ROOT:-/root/reference}}"
JL="$REF/src/jl"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$JL/gs.c" ]; then
  echo "reference jl sources not found under $JL: nothing built" >&2
  exit 3
fi
mkdir -p "$OUT"
OBJ="$(mktemp -d)"
trap 'rm -rf "$OBJ"' EXIT
CFLAGS="-std=gnu99 -O2 -fPIC -DUNDERSCORE -DGLOBAL_LONG_LONG -w"
for f in gs gs_local sort sarray_sort sarray_transfer crystal comm tensor fail; do
  gcc $CFLAGS -I"$JL" -c "$JL/$f.c" -o "$OBJ/$f.o"
done
gcc -std=c99 -O2 -fPIC -c "$HERE/jlgs_driver.c" -o "$OBJ/jlgs_driver.o"
gcc -shared -o "$OUT/libjlgs.so.tmp" "$OBJ"/*.o -lm
mv "$OUT/libjlgs.so.tmp" "$OUT/libjlgs.so"
echo "built $OUT/libjlgs.so"
