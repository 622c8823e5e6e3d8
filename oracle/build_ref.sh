#!/usr/bin/env bash
# Compiles the reference's own CUDA kernels (PCR-Penta kernel.cu, unmodified,
# read in place from the reference checkout) to PTX for sm_103a, into
# oracle/_ref/.  Test infrastructure: the PTX is loaded by oracle/refrun.c on
# the GPU to produce golden outputs of the reference itself.
#   kernel_nofma.ptx  built with -fmad=false (every product and sum rounded)
#   kernel_fma.ptx    built with nvcc's default FMA contraction
# Usage: oracle/build_ref.sh [reference_dir]
#   (default: $PCRP_REFERENCE_DIR, else the read-only checkout at /root/reference)
set -euo pipefail
REF=${1:-${PCRP_REFERENCE_DIR:-/root/reference}}
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
mkdir -p "$OUT"
if [ ! -f "$REF/kernel.cu" ]; then
    echo "build_ref.sh: $REF/kernel.cu not found; nothing built" >&2
    exit 0
fi
NVCC=${NVCC:-nvcc}
for mode in nofma fma; do
    flag=""
    [ "$mode" = nofma ] && flag="-fmad=false"
    if [ ! -f "$OUT/kernel_$mode.ptx" ] || [ "$REF/kernel.cu" -nt "$OUT/kernel_$mode.ptx" ]; then
        "$NVCC" -ptx -arch=compute_103a -O3 $flag -I"$REF" "$REF/kernel.cu" -o "$OUT/kernel_$mode.ptx"
    fi
done
