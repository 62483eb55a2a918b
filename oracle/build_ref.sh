#!/bin/sh
# TEST INFRASTRUCTURE ONLY.  Compiles the reference's own C++ programs
# around the wrapper mains in oracle/ref/ into oracle/_ref/, with the
# reference's flags (g++ -O3 -pthread, scripts/run_codes.py:105):
#   ref_<algo>   run one variant + the driver's serial verifier, dump results
#                (golden fixtures, oracle pins);
#   time_<algo>  run the best-published variant per request (CPU arm of the
#                benchmark).
# The sources come from oracle/_ref/src/ (staged unmodified by
# oracle/stage_ref.sh; git-ignored), so this also runs on machines without
# the reference tree.  Skipped when nothing is staged.  Rebuilds when the
# programs were built for another machine architecture.
# usage: oracle/build_ref.sh
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
SRC="$HERE/_ref/src"
OUT="$HERE/_ref"
if [ ! -f "$SRC/include/ECLgraph.h" ]; then
  echo "no staged reference sources in $SRC; oracle/_ref not built"
  exit 0
fi
ARCH=$(uname -m)
if [ -f "$OUT/ARCH" ] && [ "$(cat "$OUT/ARCH")" != "$ARCH" ]; then
  rm -f "$OUT"/ref_* "$OUT"/time_*
fi
CXX=${CXX:-g++}
for p in ref_bfs ref_sssp ref_cc ref_mis ref_pr ref_tc time_bfs time_sssp time_cc time_mis time_pr time_tc; do
  if [ ! -x "$OUT/$p" ] || [ "$HERE/ref/$p.cpp" -nt "$OUT/$p" ]; then
    $CXX -O3 -pthread -w -I"$SRC/include" -I"$SRC/codes/cpp" -I"$HERE/ref" "$HERE/ref/$p.cpp" -o "$OUT/$p" &
  fi
done
wait
echo "$ARCH" > "$OUT/ARCH"
ls "$OUT"
