#!/usr/bin/env bash
# Rebuild the reference's device code for sm_103a, for oracle pinning only.
#
# Reads the reference headers where they lie (REF_DIR, default
# /root/reference) and writes ONLY into oracle/_ref/ (git-ignored):
#   qcuref.cubin   sm_103a machine code of oracle/ref_shim.cu
#   qcuref.ptx     the same module as PTX (loaded by the driver when the cubin
#                  is not usable on the machine that runs it)
#   names.txt      mangled names of the reference's storage kernels
#   expected       marker: the sources were present, so the module must exist
# The reference's CMake build targets sm_70, which CUDA 13 rejects, so the
# sources are compiled directly with nvcc.  Nothing here runs the reference.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF_DIR="${REF_DIR:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -d "$REF_DIR/include" ]; then
  echo "build_ref.sh: reference sources not found at $REF_DIR; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
# the sources are here, so the module is expected: the GPU tests that compare
# against the reference kernel fail (instead of skipping) if it is missing
echo "reference sources present at build time" > "$OUT/expected"
NVCC="${NVCC:-nvcc}"
FLAGS=(-std=c++17 -O3 -I"$REF_DIR/include" -gencode arch=compute_103a,code=sm_103a -w -static-global-template-stub=false)
"$NVCC" "${FLAGS[@]}" -cubin -o "$OUT/qcuref.cubin.tmp" "$HERE/ref_shim.cu"
"$NVCC" "${FLAGS[@]}" -ptx -o "$OUT/qcuref.ptx.tmp" "$HERE/ref_shim.cu"
# host stubs carry the same mangled names as the device kernels
"$NVCC" "${FLAGS[@]}" -c -o "$OUT/ref_shim.o.tmp" "$HERE/ref_shim.cu"
nm "$OUT/ref_shim.o.tmp" | awk '($2 == "T" || $2 == "W") && $3 ~ /store(Vector|Gauge)(NonCoalesced|Coalesced)/ {print $3}' \
  | sort -u > "$OUT/names.txt.tmp"
rm -f "$OUT/ref_shim.o.tmp"
mv "$OUT/qcuref.cubin.tmp" "$OUT/qcuref.cubin"
mv "$OUT/qcuref.ptx.tmp" "$OUT/qcuref.ptx"
mv "$OUT/names.txt.tmp" "$OUT/names.txt"
echo "build_ref.sh: wrote $OUT/{qcuref.cubin,qcuref.ptx,names.txt}"
