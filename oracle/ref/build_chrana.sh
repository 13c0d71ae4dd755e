#!/bin/sh
# Builds oracle/_ref/chrana_driver (host code only, runs without a GPU) from
# the reference's analysis sources (Program/src/chrana.cu, chrdat.cu,
# sostat.cu, util.cu, read where they lie under the reference checkout),
# oracle/ref/chrana_driver.cu and the host stand-ins of the CUDA runtime in
# oracle/ref/host_cuda_stub.c (no CUDA runtime is linked).
# Usage: oracle/ref/build_chrana.sh [reference_root]
#   reference_root: argument, else $CCP_REFERENCE_ROOT, else /root/reference;
#   exits 3 when no checkout is there (build() then keeps the prebuilt files)
set -e
REF=${1:-${CCP_REFERENCE_ROOT:-/root/reference}}
[ -d "$REF/Program/src" ] || { echo "no reference checkout at $REF" >&2; exit 3; }
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/../_ref"
TMP=$(mktemp -d)
trap 'rm -rf "$TMP"' EXIT
mkdir -p "$OUT"
gcc -O2 -std=gnu11 -c "$HERE/host_cuda_stub.c" -o "$TMP/host_cuda_stub.o"
nvcc -O2 -std=c++17 -cudart none -gencode arch=compute_103a,code=sm_103a \
  -I "$REF/Program/src" "$HERE/chrana_driver.cu" "$REF/Program/src/chrana.cu" \
  "$REF/Program/src/chrdat.cu" "$REF/Program/src/sostat.cu" "$REF/Program/src/util.cu" \
  "$TMP/host_cuda_stub.o" -o "$OUT/chrana_driver"
echo "$OUT/chrana_driver"
