#!/bin/sh
# Builds oracle/_ref/sostat_driver (host code only, no GPU needed) from the
# reference's statistics and utilities (Program/src/sostat.cu, util.cu, read
# where they lie under the reference checkout) and oracle/ref/sostat_driver.cu.
# Usage: oracle/ref/build_sostat.sh [reference_root]
#   reference_root: argument, else $CCP_REFERENCE_ROOT, else /root/reference;
#   exits 3 when no checkout is there (build() then keeps the prebuilt files)
set -e
REF=${1:-${CCP_REFERENCE_ROOT:-/root/reference}}
[ -d "$REF/Program/src" ] || { echo "no reference checkout at $REF" >&2; exit 3; }
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/../_ref"
mkdir -p "$OUT"
nvcc -O2 -std=c++17 -I "$REF/Program/src" "$HERE/sostat_driver.cu" \
  "$REF/Program/src/sostat.cu" "$REF/Program/src/util.cu" -o "$OUT/sostat_driver"
echo "$OUT/sostat_driver"
