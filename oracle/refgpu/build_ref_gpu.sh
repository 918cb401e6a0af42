#!/bin/sh
# Compiles the reference's CUDA kernels (GraphCut.h + GraphCutKernels.cu,
# read from the reference checkout, unmodified) for sm_103a into
# oracle/_ref/gc_ref_kernels.cubin, and with NEIGHBORHOOD 8 into
# oracle/_ref/gc_ref_kernels8.cubin, and the data-term kernels
# (DataTermKernels.cu) into oracle/_ref/gc_ref_dt_kernels.cubin.  A cubin
# holds device code only; the
# host side that launches the kernels is ref_gpu.cpp (this repository's
# restatement of GC_Init / GC_SetGraph / GC_Optimize / GC_End), built on
# whichever machine runs it.  Nothing from the reference is written anywhere
# but oracle/_ref/.
set -e
REF=${GCFG_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/../_ref"
NVCC=${NVCC:-nvcc}
if [ ! -f "$REF/GraphCutKernels.cu" ]; then
  echo "reference checkout not found at $REF" >&2
  exit 3
fi
mkdir -p "$OUT"
"$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -O3 -w \
  -I "$HERE" -I "$REF" -o "$OUT/gc_ref_kernels.cubin.tmp" "$HERE/ref_kernels.cu"
mv "$OUT/gc_ref_kernels.cubin.tmp" "$OUT/gc_ref_kernels.cubin"
# the same kernels with the NEIGHBORHOOD switch (GraphCut.h:22) set to 8: the
# header, switched on the fly, is streamed ahead of the kernels' source (no
# modified copy is written anywhere)
N8='s/^#define NEIGHBORHOOD 4/#define NEIGHBORHOOD 8/'
{ sed "$N8" "$REF/GraphCut.h"; cat "$REF/GraphCutKernels.cu"; } |
  "$NVCC" -x cu -cubin -gencode arch=compute_103a,code=sm_103a -O3 -w \
    -I "$HERE" -I "$REF" -o "$OUT/gc_ref_kernels8.cubin.tmp" /dev/stdin
mv "$OUT/gc_ref_kernels8.cubin.tmp" "$OUT/gc_ref_kernels8.cubin"
# the data-term kernels (DataTermKernels.cu) as a third cubin
"$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -O3 -w \
  -I "$HERE" -I "$REF" -o "$OUT/gc_ref_dt_kernels.cubin.tmp" "$HERE/ref_dt_kernels.cu"
mv "$OUT/gc_ref_dt_kernels.cubin.tmp" "$OUT/gc_ref_dt_kernels.cubin"
echo "$OUT/gc_ref_kernels.cubin"
