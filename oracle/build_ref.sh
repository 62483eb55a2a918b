#!/bin/sh
# TEST INFRASTRUCTURE ONLY.  Compiles the reference's own C++ programs (from
# their sources where they lie; nothing is copied) around the wrapper mains in
# oracle/ref/ into oracle/_ref/, with the reference's flags (g++ -O3 -pthread,
# scripts/run_codes.py:105).  Needs the reference tree; skipped without it.
# usage: oracle/build_ref.sh [reference_root]
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${INDIGO_REFERENCE:-/root/reference}}
if [ ! -d "$REF/include" ] || [ ! -d "$REF/codes/cpp" ]; then
  echo "reference tree not found at $REF; oracle/_ref not built"
  exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
CXX=${CXX:-g++}
for a in bfs sssp cc mis pr tc; do
  $CXX -O3 -pthread -w -I"$REF/include" -I"$REF/codes/cpp" -I"$HERE/ref" \
      "$HERE/ref/ref_$a.cpp" -o "$OUT/ref_$a" &
done
wait
ls "$OUT"
