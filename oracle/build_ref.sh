#!/usr/bin/env bash
# Compile the reference tuna CLI from its own sources, one binary per (k, m),
# into oracle/_ref/. Test infrastructure only: the binaries pin the oracle and
# generate golden fixtures; nothing in the product links or runs them.
#
# The reference's CMake fetches kff-cpp-api and zlib-ng over the network, so it
# is not used: the two translation units are compiled directly with system zlib
# and the KFF stand-in in oracle/ref_stub/ (TSV output only).
#
# Usage: oracle/build_ref.sh [REF_ROOT] [k:m ...]
# REF_ROOT defaults to $TUNA_REFERENCE, else a "reference" directory beside the
# repository.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${TUNA_REFERENCE:-}}"
if [ -z "$REF" ]; then
  REF="$(cd "$HERE/../.." && pwd)/reference"
fi
shift || true
PAIRS=("$@")
if [ ${#PAIRS[@]} -eq 0 ]; then
  PAIRS=(31:21 31:23 63:21 21:17 25:21 15:9 33:21)
fi
if [ ! -f "$REF/src/main.cpp" ]; then
  echo "reference sources not found at $REF" >&2
  exit 1
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
build_one() {
  local k="$1" m="$2" bin="$OUT/tuna_k${1}_m${2}"
  if [ -x "$bin" ] && [ "$bin" -nt "$REF/src/main.cpp" ]; then return 0; fi
  g++ -std=c++20 -O3 -march=native -funroll-loops -fconstexpr-ops-limit=99000100 \
      -DL1_CACHE_LINE_SIZE=64 -DTUNA_VERSION='"reference"' \
      -DFIXED_K="$k" -DFIXED_M="$m" \
      -I"$HERE/ref_stub" -I"$REF/include" -I"$REF/src" -I"$REF/include/helicase_cpp" \
      "$REF/src/main.cpp" "$REF/src/CLI.cpp" -x c -std=c11 "$REF/external/xxHash/xxhash.c" -x none \
      -lz -lpthread -o "$bin.tmp"
  mv "$bin.tmp" "$bin"
}
pids=()
for p in "${PAIRS[@]}"; do
  build_one "${p%%:*}" "${p##*:}" &
  pids+=($!)
done
rc=0
for pid in "${pids[@]}"; do wait "$pid" || rc=1; done
exit $rc
