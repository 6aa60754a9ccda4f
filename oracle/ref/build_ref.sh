#!/usr/bin/env bash
# Builds oracle/_ref/libotfem_ref.so: the UNMODIFIED OpenTissue FEM headers
# (read in place from the reference tree) behind the oracle C interface.
# Test infrastructure only.  Usage: build_ref.sh [reference_root]
# reference_root: the OpenTissue source tree; default $OTFEM_REFERENCE_ROOT,
# else /root/reference (the default location of oracle/build.py).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
oracle="$(dirname "$here")"
ref="${1:-${OTFEM_REFERENCE_ROOT:-/root/reference}}"
out="$oracle/_ref"
if [ ! -f "$ref/OpenTissue/dynamics/fem/fem.h" ]; then
  echo "reference tree not found at $ref" >&2
  exit 2
fi
mkdir -p "$out/include/OpenTissue"
# configuration.h is generated from the reference's configuration.h.in
sed -e 's/@OpenTissue_VERSION@/0.994/g' \
    -e 's/@OpenTissue_VERSION_MAJOR@/0/g' \
    -e 's/@OpenTissue_VERSION_MINOR@/994/g' \
    -e "s#@PROJECT_SOURCE_DIR@#$ref#g" \
    "$ref/OpenTissue/configuration.h.in" > "$out/include/OpenTissue/configuration.h"
# Pinned parity flags: no FMA contraction, so the FP64 arithmetic is the
# plain IEEE sequence written in the headers.
${CXX:-g++} -std=c++11 -O2 -ffp-contract=off -DNDEBUG -fPIC -shared -w \
  -I"$out/include" -I"$ref" -I"$here/boost_shim" \
  "$here/ref_capi.cpp" "$here/ref_coupling.cpp" -o "$out/libotfem_ref.so"
echo "built $out/libotfem_ref.so"
