#!/bin/sh
# TEST INFRASTRUCTURE ONLY.  Stages the reference files that the CPU oracle
# programs and the drop-in driver programs compile against -- its include/
# headers and the C++ variant files named below, unmodified -- into
# oracle/_ref/src/, mirroring their paths in the reference tree.  That folder
# is git-ignored (nothing of the reference is committed) and travels with the
# working tree to machines without the reference tree, where
# oracle/build_ref.sh and the package's build_shims compile from it.
# usage: oracle/stage_ref.sh [reference_root]
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${INDIGO_REFERENCE:-/root/reference}}
DST="$HERE/_ref/src"
if [ ! -d "$REF/include" ] || [ ! -d "$REF/codes/cpp" ]; then
  echo "reference tree not found at $REF; nothing staged"
  exit 0
fi
mkdir -p "$DST/include"
cp "$REF"/include/*.h "$DST/include/"
while read -r f; do
  [ -z "$f" ] && continue
  mkdir -p "$DST/$(dirname "$f")"
  cp "$REF/$f" "$DST/$f"
done <<LIST
codes/cpp/bfs-cpp/BFS_CPP_V_Topo_Push_IntType_ReadWrite_NoFieldBug_Block_Atomic_Determ_NoBoundsBug_NoRangeBug.cpp
codes/cpp/sssp-cpp/SSSP_CPP_V_Topo_Push_IntType_ReadModifyWrite_NonDeterm_NoBoundsBug_Block_Atomic_NoRangeBug.cpp
codes/cpp/cc-cpp/CC_CPP_V_Topo_Push_IntType_ReadModifyWrite_Determ_NoBoundsBug_Block_Atomic.cpp
codes/cpp/cc-cpp/CC_CPP_V_Topo_Push_IntType_ReadWrite_NonDeterm_NoBoundsBug_Block_Atomic.cpp
codes/cpp/mis-cpp/MIS_CPP_V_Topo_Push_IntType_Atomic_CopyDeterm_Block.cpp
codes/cpp/mis-cpp/MIS_CPP_V_Topo_Push_IntType_Atomic_NonDeterm_Block.cpp
codes/cpp/pr-cpp/PR_CPP_Pull_FloatType_Reduction_Block_Determin.cpp
codes/cpp/pr-cpp/PR_CPP_Pull_FloatType_AtomicAdd_Block_Determin.cpp
codes/cpp/tc-cpp/TC_CPP_V_IntType_Critical_Cyclic.cpp
LIST
echo "staged $(find "$DST" -type f | wc -l) reference files in $DST"
