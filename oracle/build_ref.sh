#!/usr/bin/env bash
# Builds the UNMODIFIED reference program (kernel.cu, IDIC.h, data.h) for the
# host CPU from the sources where they lie, into oracle/_ref/ (git-ignored).
# Test infrastructure for pinning the oracle; the product never uses it.
#
# Two textual changes are made, both to syntax g++ rejects:
#   Name << <grid, block >> > (args)   ->   ds_ref_launch(grid, block, Name) (args)
#   the "\Nn" escape in one snapshot header string (kernel.cu:455; MSVC reads an
#   unknown escape as the bare letter, g++ refuses it)  ->  "Nn"
# everything else compiles as written against oracle/ref_include/cuda_runtime.h.
# Needs the reference tree (default /root/reference); exits 3 when it is absent.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${DS_REFERENCE_DIR:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF/kernel.cu" ] || [ ! -f "$REF/IDIC.h" ] || [ ! -f "$REF/data.h" ]; then
  echo "reference sources not found under $REF" >&2
  exit 3
fi
mkdir -p "$OUT"
# the rewritten text is piped straight into the compiler (no copy is written)
sed -E -e 's/([A-Za-z_][A-Za-z_0-9]*)[[:space:]]*<<[[:space:]]*<([^>]*)>>[[:space:]]*>/ds_ref_launch(\2, \1)/g' \
  -e 's/\\Nn /Nn /g' \
  "$REF/kernel.cu" |
  g++ -O2 -fopenmp -ffp-contract=off -w -std=c++17 \
    -I "$HERE/ref_include" -I "$REF" -x c++ - -o "$OUT/dustyshock_ref" -lm
echo "$OUT/dustyshock_ref"
