#!/usr/bin/env bash
# Build the reference's own CPU path (mikekatz04/EOBGPU) as a host shared
# library, oracle/_ref/libeobref.so, straight from the reference checkout.
#
# Test infrastructure only: it pins the oracle and generates the golden
# fixtures under tests/golden/.  Nothing is copied into this repository: the
# sources are compiled where they lie (src/interpolate.cu is fed through a pipe
# because only its lines 1-308, the spline build, compile on a host).
#
# Usage: oracle/ref/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/../_ref"
mkdir -p "$OUT"
if [ ! -f "$REF/src/EOB.cu" ]; then
  echo "reference sources not found under $REF" >&2
  exit 2
fi
CXX="${CXX:-g++}"
FLAGS=(-x c++ -std=c++11 -O2 -fPIC -ffp-contract=off -w -include "$HERE/ref_shim.h" -I"$REF/include")
"$CXX" "${FLAGS[@]}" -c "$REF/src/EOB.cu" -o "$OUT/EOB.o" &
"$CXX" "${FLAGS[@]}" -c "$REF/src/DOPR853.cu" -o "$OUT/DOPR853.o" &
sed -n '1,308p' "$REF/src/interpolate.cu" | "$CXX" "${FLAGS[@]}" -I"$REF/src" -c - -o "$OUT/interpolate.o" &
"$CXX" -std=c++11 -O2 -fPIC -ffp-contract=off -w -include "$HERE/ref_shim.h" -I"$REF/include" \
  -c "$HERE/ref_abi.cpp" -o "$OUT/ref_abi.o" &
wait
"$CXX" -shared -o "$OUT/libeobref.so" "$OUT/EOB.o" "$OUT/DOPR853.o" "$OUT/interpolate.o" "$OUT/ref_abi.o"
rm -f "$OUT"/*.o
echo "built $OUT/libeobref.so"
