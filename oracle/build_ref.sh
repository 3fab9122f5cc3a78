#!/usr/bin/env bash
# build_ref.sh -- compile the reference graph-utils CPU checkers from their
# sources, where they lie, into oracle/_ref/ref_oracle.
#
# Test infrastructure only (pins oracle/gu_oracle.c and makes tests/golden/).
# Needs the reference tree (default /root/reference, or $GU_REFERENCE); it is
# absent on GPU machines, where this script exits 0 without building.
# Nothing is copied out of the reference tree; objects go to oracle/_ref/.
set -euo pipefail
REF="${GU_REFERENCE:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF" ]; then
  echo "build_ref: reference tree not present; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
NVCC="${NVCC:-nvcc}"
INC="-I$REF -I$REF/graph-utils -I$REF/graph-utils/multi_search"
# Device code of the reference headers only has to parse; one sm_100a target is enough.
CUFLAGS="-std=c++17 -O2 -rdc=true -gencode arch=compute_100a,code=sm_100a -include $HERE/ref_shim.h $INC -w"
CXXFLAGS="-std=c++17 -O2 -ffp-contract=off $INC -w"

g++ $CXXFLAGS -c "$REF/parse.cpp" -o "$OUT/parse.o" &
g++ $CXXFLAGS -c "$REF/util.cpp" -o "$OUT/util.o" &
g++ $CXXFLAGS -c "$REF/graph-utils/reverse.cpp" -o "$OUT/reverse.o" &
g++ $CXXFLAGS -c "$REF/graph-utils/dag_reachability.cpp" -o "$OUT/dag_reachability.o" &
$NVCC $CUFLAGS -Dmain=ms_main -Dsequential=ms_sequential -c "$REF/examples/multi_search/multi_search_test.cu" -o "$OUT/ms.o" &
$NVCC $CUFLAGS -Dmain=bc_main -Dsequential=bc_sequential -c "$REF/examples/betweenness_centrality/bc.cu" -o "$OUT/bc.o" &
$NVCC $CUFLAGS -Dmain=sp_main -Dsequential=sp_sequential -Dverify=sp_verify -c "$REF/examples/counting_shortest_paths/shortest_paths.cu" -o "$OUT/sp.o" &
$NVCC $CUFLAGS -Dmain=ds_main -Dsequential=ds_sequential -c "$REF/examples/diameter_sampling/diameter_sampling_test.cu" -o "$OUT/ds.o" &
$NVCC $CUFLAGS -Dmain=tc_main -Dsequential=tc_sequential -Dverify=tc_verify -c "$REF/examples/transitive_closure/reachability.cu" -o "$OUT/tc.o" &
$NVCC $CUFLAGS -Dmain=lbs_main -c "$REF/examples/load_balanced_search/lbs.cu" -o "$OUT/lbs.o" &
g++ $CXXFLAGS -c "$HERE/ref_driver.cpp" -o "$OUT/ref_driver.o" &
g++ $CXXFLAGS -c "$HERE/ref_stubs.cpp" -o "$OUT/ref_stubs.o" &
wait
# The example main()s (renamed, never called) reference the reference's GPU
# entry points, which are not built here; leave those symbols unresolved.
$NVCC -rdc=true -gencode arch=compute_100a,code=sm_100a -o "$OUT/ref_oracle" \
  "$OUT"/ref_driver.o "$OUT"/ref_stubs.o "$OUT"/parse.o "$OUT"/util.o "$OUT"/reverse.o "$OUT"/dag_reachability.o \
  "$OUT"/ms.o "$OUT"/bc.o "$OUT"/sp.o "$OUT"/ds.o "$OUT"/tc.o "$OUT"/lbs.o \
  -Xlinker --unresolved-symbols=ignore-all
echo "build_ref: built $OUT/ref_oracle"
