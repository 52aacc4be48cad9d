#!/bin/sh
# Compile the reference's CPU programs from their own sources into oracle/_ref/
# (test infrastructure: used to pin the oracle; never part of the product).
#   seq_ref        <- seq/seq.cpp + seq/TYPES.h + seq/GraphRP.h (max-heap path decomposition)
#   cpu_reference  <- workingPad/cpu_reference.cpp (single-edge factoring, float p)
# Usage: oracle/build_ref.sh [reference_root]
# The reference root is the argument, else $NR_REFERENCE_ROOT, else the
# read-only mount of the build container this recipe was written for.
set -e
REF="${1:-${NR_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/seq/seq.cpp" ]; then
    echo "reference sources not found under $REF" >&2
    exit 2
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
"$CXX" -O2 -std=c++17 -w -I"$REF/seq" -o "$OUT/seq_ref" "$REF/seq/seq.cpp"
"$CXX" -O2 -std=c++17 -w -o "$OUT/cpu_reference" "$REF/workingPad/cpu_reference.cpp"
echo "built $OUT/seq_ref $OUT/cpu_reference"
