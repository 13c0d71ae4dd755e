#!/bin/sh
# Compiles the reference's device code (Program/src/chrsim.cu, sugrid.cu,
# chrana.cu, read where they lie under the reference checkout) into
# oracle/_ref/ccp_ref.cubin for sm_103a. Device code only: the cubin is loaded
# on a GB300 through the CUDA driver API by tests/golden/make_golden.py.
# Usage: oracle/ref/build_ref.sh [reference_root]
#   reference_root: argument, else $CCP_REFERENCE_ROOT, else /root/reference;
#   exits 3 when no checkout is there (build() then keeps the prebuilt files)
set -e
REF=${1:-${CCP_REFERENCE_ROOT:-/root/reference}}
[ -d "$REF/Program/src" ] || { echo "no reference checkout at $REF" >&2; exit 3; }
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/../_ref"
mkdir -p "$OUT"
nvcc -cubin -gencode arch=compute_103a,code=sm_103a -O3 \
  -I "$REF/Program/src" "$HERE/ref_kernels.cu" -o "$OUT/ccp_ref.cubin"
echo "$OUT/ccp_ref.cubin"
