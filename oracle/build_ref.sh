#!/bin/sh
# Builds oracle/_ref/ref_partition_harness from the reference's own partitioner
# sources (Xilinx/HPC L2/sparse + utils), compiled where they lie.  Test
# infrastructure only: the binary is used to pin the oracle's and the product's
# format conversion and to generate the committed fixtures in tests/golden/.
# Usage: oracle/build_ref.sh <reference-root>   (or XJPCG_REFERENCE_ROOT set)
set -e
REF=${1:-$XJPCG_REFERENCE_ROOT}
if [ -z "$REF" ]; then
    echo "usage: $0 <reference-root> (or set XJPCG_REFERENCE_ROOT)" >&2
    exit 2
fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/L2/sparse/src/sw/c++/gen_signature.cpp" ]; then
    echo "reference partitioner sources not found under $REF" >&2
    exit 1
fi
mkdir -p "$OUT"
g++ -O2 -std=c++11 -pthread -fopenmp \
    -DSPARSE_dataType=double -DSPARSE_maxRows=4096 -DSPARSE_maxCols=4096 \
    -DSPARSE_hbmChannels=16 -DSPARSE_parEntries=4 -DSPARSE_accLatency=8 \
    -DSPARSE_hbmMemBits=256 \
    -I"$REF/L2/sparse/include/sw/fp64" -I"$REF/utils/include/sw" \
    "$REF/L2/sparse/src/sw/c++/gen_signature.cpp" "$HERE/ref_partition_harness.cpp" \
    -o "$OUT/ref_partition_harness"
echo "$OUT/ref_partition_harness"
