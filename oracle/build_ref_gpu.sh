#!/usr/bin/env bash
# Compiles the reference's own CUDA kernels -- the UNMODIFIED kernel.cu (which
# includes IDIC.h and data.h), as the reference's project builds it: nvcc -O3,
# default floating-point options -- into a cubin for sm_103a, in oracle/_ref/
# (git-ignored).  Device code only: the cubin is loaded by oracle/ref_gpu.c,
# which restates the reference's host loop around these kernels, for the
# reference-GPU baseline.  Baseline infrastructure; the product never uses it.
# Needs the reference tree, named by DS_REFERENCE_DIR (there is no default);
# exits 3 when the variable is unset or the sources are not there.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ -z "${DS_REFERENCE_DIR:-}" ]; then
  echo "DS_REFERENCE_DIR is not set: point it at the reference tree (kernel.cu, IDIC.h, data.h)" >&2
  exit 3
fi
REF="$DS_REFERENCE_DIR"
OUT="$HERE/_ref"
if [ ! -f "$REF/kernel.cu" ] || [ ! -f "$REF/IDIC.h" ] || [ ! -f "$REF/data.h" ]; then
  echo "reference sources not found under $REF" >&2
  exit 3
fi
mkdir -p "$OUT"
nvcc -cubin -O3 -gencode arch=compute_103a,code=sm_103a -w -I "$REF" \
  -o "$OUT/ref_kernels.cubin.tmp" "$REF/kernel.cu"
mv "$OUT/ref_kernels.cubin.tmp" "$OUT/ref_kernels.cubin"
echo "$OUT/ref_kernels.cubin"
