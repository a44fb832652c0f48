#!/usr/bin/env bash
# Builds the reference's own SRC/orth.c and SRC/util.c, unmodified, into
# oracle/_ref/liborth_ref.so for use as a CPU oracle (test infrastructure only).
#
# The reference needs MPI, Trilinos TSQR and BLAS/LAPACK. They are supplied by:
#   ref_stubs/include/mpi.h           single-rank MPI (allreduce == copy)
#   ref_stubs/tpetra/include/*.hpp    TSQR::factorExplicit as LAPACK dgeqrf+dorgqr
#   scipy's bundled LP64 OpenBLAS     dgemm_ -> scipy_dgemm_ etc. via -D renames
# orth.c includes "../tpetra/include/Tsqr.hpp"; with -I ref_stubs/include that
# path resolves to ref_stubs/tpetra/include/Tsqr.hpp.
#
# Usage: oracle/build_ref.sh REFERENCE_ROOT   (or set BCGS_REFERENCE_ROOT)
# Does nothing (exit 0) when the reference sources are absent.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${BCGS_REFERENCE_ROOT:-}}"
if [ -z "$REF" ]; then
    echo "build_ref: give the reference's root as an argument or in BCGS_REFERENCE_ROOT; skipping" >&2
    exit 0
fi
OUT="$HERE/_ref"
if [ ! -f "$REF/SRC/orth.c" ] || [ ! -f "$REF/SRC/util.c" ]; then
    echo "build_ref: reference sources not found under $REF; skipping" >&2
    exit 0
fi
OPENBLAS="$(python3 - <<'PY'
import glob, os, scipy
d = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
c = [p for p in glob.glob(os.path.join(d, "libscipy_openblas-*.so")) if "openblas64" not in p]
print(c[0] if c else "")
PY
)"
if [ -z "$OPENBLAS" ]; then
    echo "build_ref: scipy's LP64 OpenBLAS not found" >&2
    exit 1
fi
mkdir -p "$OUT"
RENAMES=""
for f in dgemm dtrsm dpotrf dlacpy dlaset daxpy dnrm2 dcopy dscal; do
    RENAMES="$RENAMES -D${f}_=scipy_${f}_"
done
CFLAGS="-O2 -fPIC -w -I$HERE/ref_stubs/include $RENAMES"
g++ $CFLAGS -x c++ -c "$REF/SRC/orth.c" -o "$OUT/orth.o"
gcc $CFLAGS -x c -c "$REF/SRC/util.c" -o "$OUT/util.o"
g++ -shared -o "$OUT/liborth_ref.so" "$OUT/orth.o" "$OUT/util.o" \
    "$OPENBLAS" -Wl,-rpath,"$(dirname "$OPENBLAS")" -lm
rm -f "$OUT/orth.o" "$OUT/util.o"
echo "build_ref: built $OUT/liborth_ref.so against $OPENBLAS"
