#!/usr/bin/env bash
# Builds oracle/_ref/ref_fixtures and oracle/_ref/ref_partition from the
# reference's own headers (host code only; nvcc is used because the
# reference's headers include the CUDA runtime and thrust). Needs the reference sources at $LOOPS_REF
# (default: a `reference` folder beside this repository's folder); outputs go only to oracle/_ref/
# (git-ignored).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${LOOPS_REF:-$here/../../../reference}"
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
# the reference's CPU SpMV (cpu::reference) with thrust's device system on
# the host, so that it runs without a GPU; cxxopts replaced by a stand-in
nvcc -std=c++17 -O3 --expt-extended-lambda --expt-relaxed-constexpr -w \
  -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP -I"$here/stub" -I"$ref/include" \
  -I"$ref/examples/spmv" "$here/ref_cpu.cu" -o "$out/ref_cpu"
# the reference's SpMV kernels as a cubin, the names of its entry functions
# (as ptxas prints them) and the launch-parameter layout the host compiler
# sees (a host program run here, no GPU needed)
nvcc -std=c++17 -O3 --expt-extended-lambda --expt-relaxed-constexpr -w \
  -I"$ref/include" -cubin -gencode arch=compute_103a,code=sm_103a -Xptxas -v \
  "$here/ref_kernels.cu" -o "$out/ref_kernels.cubin" 2> "$out/ref_kernels.ptxas.log"
nvcc -std=c++17 -O1 --expt-extended-lambda --expt-relaxed-constexpr -w \
  -I"$ref/include" -gencode arch=compute_103a,code=sm_103a \
  "$here/ref_kernels.cu" -o "$out/ref_kernels_layout"
python3 - "$out" <<'PY'
import json, os, re, subprocess, sys
out = sys.argv[1]
names = re.findall(r"Compiling entry function '([^']+)'",
                   open(os.path.join(out, "ref_kernels.ptxas.log")).read())
kernels = {}
for key, tag in (("merge_path_flat", "__merge_path_flat"), ("thread_mapped", "__thread_mapped"),
                 ("group_mapped", "__group_mapped"), ("work_oriented", "__work_oriented"),
                 ("original", "__original"), ("spmm_thread_mapped", "__thread_mapped")):
    pre = "4spmm" if key.startswith("spmm") else "4spmv"
    hit = [n for n in names if pre + str(len(tag)) + tag in n]
    assert len(hit) == 1, (key, hit)
    kernels[key] = hit[0]
layout = json.loads(subprocess.check_output([os.path.join(out, "ref_kernels_layout")]))
layout["kernels"] = kernels
json.dump(layout, open(os.path.join(out, "ref_kernels.json"), "w"), indent=1)
PY
echo "built $out/ref_fixtures $out/ref_partition $out/ref_cpu $out/ref_kernels.cubin"
