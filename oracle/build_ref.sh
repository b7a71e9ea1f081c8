#!/bin/bash
# Builds the unmodified reference (akohta/bem3_emf_b2) from its own sources,
# where they lie, into oracle/_ref/ -- test infrastructure only.
#  * MKL is replaced by numpy's bundled ILP64 OpenBLAS through the four shim
#    headers in oracle/ref_shim/.
#  * Outputs: oracle/_ref/libbem3ref.so and the executables d3b2_create_matrix,
#    d3b2_bv_solver, example1, example2, example4 (example3 needs libpng, which
#    is absent), bem3_analysis (this repository's driver, reference API only) and
#    the two probes ref_point and ref_beam.
# Usage: oracle/build_ref.sh [reference_dir]
#        oracle/build_ref.sh --where   (print the reference directory; exit 2 if absent)
# The reference directory is the argument, else $BEM3_REFERENCE_DIR, else the
# location this container mounts it at.  This recipe is the one place that
# names that location; the Python side asks it (oracle.reference_dir()).
set -euo pipefail
WHERE=0
if [ "${1:-}" = "--where" ]; then WHERE=1; shift; fi
REF=${1:-${BEM3_REFERENCE_DIR:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -d "$REF/d3b2_src" ] || { [ $WHERE = 1 ] || echo "reference sources not found at $REF" >&2; exit 2; }
if [ $WHERE = 1 ]; then echo "$REF"; exit 0; fi
mkdir -p "$OUT"
BLASDIR=$(python3 -c "import numpy,os;print(os.path.join(os.path.dirname(numpy.__file__)+'.libs'))")
BLAS=$(ls "$BLASDIR"/libscipy_openblas64_*.so | head -1)
CFLAGS="-O3 -fopenmp -fPIC -w -I$HERE/ref_shim -I$REF/d3b2_src -I$REF/mfb_src -I$REF/com_src"
SRCS=$(ls "$REF"/d3b2_src/*.c "$REF"/mfb_src/*.c "$REF"/com_src/*.c | grep -v -e d3b2_create_matrix.c -e d3b2_bv_solver.c)
OBJS=""
for s in $SRCS; do
  o="$OUT/$(basename "$s" .c).o"
  gcc $CFLAGS -c "$s" -o "$o" &
  OBJS="$OBJS $o"
done
wait
gcc -shared -fopenmp -o "$OUT/libbem3ref.so" $OBJS "$BLAS" -Wl,-rpath,"$BLASDIR" -lm
for m in d3b2_src/d3b2_create_matrix d3b2_src/d3b2_bv_solver example1 example4 example2; do
  gcc $CFLAGS -o "$OUT/$(basename $m)" "$REF/$m.c" -L"$OUT" -lbem3ref -Wl,-rpath,"$OUT" "$BLAS" -Wl,-rpath,"$BLASDIR" -lm
done
# the repository's own analysis driver, compiled against the reference API, so
# that both libraries print the same quantities with full precision
APPS="$HERE/../bem3_emf_b2_gb300/apps"
gcc $CFLAGS -o "$OUT/bem3_analysis" "$APPS/bem3_analysis.c" -L"$OUT" -lbem3ref -Wl,-rpath,"$OUT" "$BLAS" -Wl,-rpath,"$BLASDIR" -lm
gcc $CFLAGS -o "$OUT/ref_point" "$HERE/ref_point.c" -L"$OUT" -lbem3ref -Wl,-rpath,"$OUT" "$BLAS" -Wl,-rpath,"$BLASDIR" -lm
gcc $CFLAGS -o "$OUT/ref_beam" "$HERE/ref_beam.c" -L"$OUT" -lbem3ref -Wl,-rpath,"$OUT" "$BLAS" -Wl,-rpath,"$BLASDIR" -lm
rm -f "$OUT"/*.o
echo "built $OUT"
