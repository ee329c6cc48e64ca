#!/usr/bin/env bash
# Compiles the reference's own kernel code for the host CPU into
# oracle/_ref/libref_kernels.so, straight from the reference sources (read in
# place, streamed through the compiler; no source text is written anywhere).
#
# The anonymous-namespace kernel sections of voro_optimizer.cu and
# poisson_disk.cu are wrapped in namespaces k12 (as shipped), k16 (kLossK
# patched to 16, the 1M-site config's k) and pd, behind shim_pre.h, followed
# by harness.cpp. -ffp-contract=off keeps a*b+c as two roundings, i.e. the
# reference built with nvcc --fmad=false.
#
# It also compiles the reference's Canvas (src/voromesh/canvas.cpp and
# shape2d.cpp, in place, with -I on its include/) and canvas_harness.cpp into
# oracle/_ref/libref_canvas.so.
#
# Usage: REF=/path/to/reference bash oracle/ref_shim/build_ref.sh
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${REF:?set REF to the root of the reference project sources}"
OUT="$HERE/../_ref"
VORO="$REF/src/voromesh/voro_optimizer.cu"
POIS="$REF/src/poisson/poisson_disk.cu"
if [[ ! -f "$VORO" || ! -f "$POIS" ]]; then
  echo "build_ref: reference sources not found under $REF" >&2
  exit 2
fi
mkdir -p "$OUT"
section() { sed -n '/^namespace {$/,/^} \/\/ namespace$/p' "$1"; }
{
  cat "$HERE/shim_pre.h"
  echo 'namespace k12 {'
  section "$VORO"
  echo '}'
  echo 'namespace k16 {'
  section "$VORO" | sed 's/\(constexpr int kLossK *= *\)12;/\116;/'
  echo '}'
  echo 'namespace pd {'
  section "$POIS"
  echo '}'
  cat "$HERE/harness.cpp"
} | ${CXX:-g++} -std=c++17 -O2 -fPIC -shared -ffp-contract=off -fno-fast-math -w -x c++ - \
    -o "$OUT/libref_kernels.so"
echo "built $OUT/libref_kernels.so"
${CXX:-g++} -std=c++20 -O2 -fPIC -shared -ffp-contract=off -fno-fast-math -w -I"$REF/include" \
    "$REF/src/voromesh/canvas.cpp" "$REF/src/voromesh/shape2d.cpp" "$HERE/canvas_harness.cpp" \
    -o "$OUT/libref_canvas.so"
echo "built $OUT/libref_canvas.so"
