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
# the rewritten text is piped straight into the compiler (no copy is written)
sed -E -e 's/([A-Za-z_][A-Za-z_0-9]*)[[:space:]]*<<[[:space:]]*<([^>]*)>>[[:space:]]*>/ds_ref_launch(\2, \1)/g' \
  -e 's/\\Nn /Nn /g' \
  "$REF/kernel.cu" |
  g++ -O2 -fopenmp -ffp-contract=off -w -std=c++17 \
    -I "$HERE/ref_include" -I "$REF" -x c++ - -o "$OUT/dustyshock_ref" -lm
echo "$OUT/dustyshock_ref"
