#!/usr/bin/env bash
# Builds the reference harness (test infrastructure) from the reference's own
# sources where they lie.  Output goes to oracle/_ref/ only (git-ignored).
# The reference is compiled at its default -O2 with default (SSE2) Eigen
# packets: its Mersenne-Twister noise stream depends on the packet width.
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   (default: $MD_REFERENCE_ROOT, else /root/reference).  The root it used is
#   recorded in oracle/_ref/reference_root for the tests that read the
#   reference's own files.
set -euo pipefail
REF="${1:-${MD_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/simulation.cpp" ]; then
  echo "reference sources not found under $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS="-O2 -std=c++14 -w -I$REF/src/lib -I$REF/src"
pids=()
for f in interaction configuration postprocessing mathFun; do
  $CXX $FLAGS -c "$REF/src/$f.cpp" -o "$OUT/$f.o" & pids+=($!)
done
$CXX $FLAGS -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
$CXX -o "$OUT/ref_harness" "$OUT/ref_harness.o" "$OUT/interaction.o" \
  "$OUT/configuration.o" "$OUT/postprocessing.o" "$OUT/mathFun.o"
echo "$REF" > "$OUT/reference_root"
echo "built $OUT/ref_harness"
