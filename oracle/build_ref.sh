#!/bin/sh
# Build the ALiS reference library from its own sources into oracle/_ref/
# (checker only: pins the oracle restatement; never linked into the
# engine).  HDF5 and libpng are replaced by the stand-in headers in
# oracle/stubs.  FMA contraction is disabled so results do not depend on
# the host ISA.
#
# This recipe is the one place that knows where the read-only reference
# checkout lies: the first argument, else $ALIS_REFERENCE, else the
# checkout of the build container (/root/reference).
#   usage: oracle/build_ref.sh [REFERENCE_ROOT]   build oracle/_ref/libalis_ref.a
#          oracle/build_ref.sh --locate           print the checkout's path (exit 1: none)
set -e
if [ "$1" = "--locate" ]; then
  REF=${ALIS_REFERENCE:-/root/reference}
  [ -d "$REF/src" ] || exit 1
  echo "$REF"
  exit 0
fi
REF=${1:-${ALIS_REFERENCE:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -d "$REF/src" ] || { echo "reference sources not found at $REF/src" >&2; exit 1; }
mkdir -p "$OUT"
for f in world object shapes source update output slices fields phaser farfld; do
  gcc -std=c99 -O3 -fopenmp -ffp-contract=off -fPIC -w -I"$HERE/stubs" -I"$REF/src" \
      -c "$REF/src/$f.c" -o "$OUT/$f.o" &
done
wait
rm -f "$OUT/libalis_ref.a"
ar rcs "$OUT/libalis_ref.a" "$OUT"/world.o "$OUT"/object.o "$OUT"/shapes.o "$OUT"/source.o \
    "$OUT"/update.o "$OUT"/output.o "$OUT"/slices.o "$OUT"/fields.o "$OUT"/phaser.o "$OUT"/farfld.o
echo "built $OUT/libalis_ref.a"
