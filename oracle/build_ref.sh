#!/usr/bin/env bash
# Builds the reference's own gather-scatter library (NekCEM src/jl, C99) from
# the reference source tree into oracle/_ref/libjlgs.so, with the test shim
# oracle/jlgs_driver.c.  Single process: no -DMPI, so jl's comm.h uses its
# serial branch.  Only the sources the gs path needs are compiled.  Test
# infrastructure only; outputs go to oracle/_ref/ (git-ignored).
#
# usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -euo pipefail
REF="${1:-/root/reference}"
JL="$REF/src/jl"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$JL/gs.c" ]; then
  echo "reference jl sources not found under $JL" >&2
  exit 2
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
