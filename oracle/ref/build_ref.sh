#!/usr/bin/env bash
# Builds oracle/_ref/ref_fixtures and oracle/_ref/ref_partition from the
# reference's own headers (host code only; nvcc is used because the
# reference's headers include the CUDA runtime and thrust). Needs the reference sources at $LOOPS_REF (default
# /root/reference); outputs go only to oracle/_ref/ (git-ignored).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${LOOPS_REF:-/root/reference}"
out="$here/../_ref"
[ -d "$ref/include/loops" ] || { echo "reference sources not found at $ref" >&2; exit 3; }
mkdir -p "$out"
nvcc -std=c++17 -O1 --expt-extended-lambda --expt-relaxed-constexpr -w \
  -I"$ref/include" -x cu "$ref/include/loops/container/detail/mmio.cpp" \
  -dc -o "$out/mmio.o"
nvcc -std=c++17 -O1 --expt-extended-lambda --expt-relaxed-constexpr -w \
  -I"$ref/include" "$here/ref_fixtures.cu" -dc -o "$out/ref_fixtures.o"
nvcc "$out/ref_fixtures.o" "$out/mmio.o" -o "$out/ref_fixtures"
nvcc -std=c++17 -O1 --expt-extended-lambda --expt-relaxed-constexpr -w \
  -I"$ref/include" "$here/ref_partition.cu" -o "$out/ref_partition"
echo "built $out/ref_fixtures $out/ref_partition"
