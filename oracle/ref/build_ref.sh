#!/bin/sh
# Compiles the reference's device code (Program/src/chrsim.cu, sugrid.cu,
# chrana.cu, read where they lie under the reference checkout) into
# oracle/_ref/ccp_ref.cubin for sm_103a. Device code only: the cubin is loaded
# on a GB300 through the CUDA driver API by tests/golden/make_golden.py.
# Usage: oracle/ref/build_ref.sh [reference_root]   (default /root/reference)
set -e
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/../_ref"
mkdir -p "$OUT"
nvcc -cubin -gencode arch=compute_103a,code=sm_103a -O3 \
  -I "$REF/Program/src" "$HERE/ref_kernels.cu" -o "$OUT/ccp_ref.cubin"
echo "$OUT/ccp_ref.cubin"
