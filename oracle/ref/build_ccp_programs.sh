#!/bin/sh
# Builds the reference's own ccp-perform and ccp-profile, unchanged, against
# the engine as INTEGRATION.md section 2 tells a maintainer to: a copy of the
# reference's Program/src as symbolic links to its files (read where they
# lie under the reference checkout) in a temporary directory, with
# chrsim.cuh replaced by a header that includes chrdat.cuh and
# include/ccpgpu_chrsim.hpp; chrsim.cu and sugrid.cu are left out of the link
# and tfm_gb300/libccpgpu.so linked instead. Only the two programs are kept,
# in oracle/_ref/ccp_programs/bin (host binaries of this machine).
# Usage: oracle/ref/build_ccp_programs.sh [reference_root]
#   reference_root: argument, else $CCP_REFERENCE_ROOT, else /root/reference;
#   exits 3 when no checkout is there
set -e
REF=${1:-${CCP_REFERENCE_ROOT:-/root/reference}}
[ -d "$REF/Program/src" ] || { echo "no reference checkout at $REF" >&2; exit 3; }
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/../.." && pwd)
OUT="$HERE/../_ref/ccp_programs"
TREE=$(mktemp -d)
trap 'rm -rf "$TREE"' EXIT
rm -rf "$OUT"
mkdir -p "$TREE/src" "$OUT/bin"
for f in "$REF"/Program/src/*; do ln -s "$f" "$TREE/src/"; done
rm "$TREE/src/chrsim.cuh"
cat > "$TREE/src/chrsim.cuh" <<'HDR'
#ifndef MMC_CHRSIM_H
#define MMC_CHRSIM_H
#include "chrdat.cuh"
#include "ccpgpu_chrsim.hpp"
#endif
HDR
NV="nvcc -O2 -std=c++17 -gencode arch=compute_103a,code=sm_103a -I $ROOT/include"
for u in util chrdat ccp-perform ccp-profile; do
  $NV -c "$TREE/src/$u.cu" -o "$TREE/$u.o"
done
for p in ccp-perform ccp-profile; do
  $NV "$TREE/util.o" "$TREE/chrdat.o" "$TREE/$p.o" -o "$OUT/bin/$p" \
    -L "$ROOT/tfm_gb300" -lccpgpu -Xlinker -rpath="$ROOT/tfm_gb300"
done
echo "$OUT/bin"
