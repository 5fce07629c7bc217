#!/usr/bin/env bash
# Builds the reference's own CPU early-break path, its -normalize /
# -translate preprocessing and the host side of its statistics grid from its
# sources where they lie (read-only) into oracle/_ref/ (ref_eb and, in the
# double instantiation, ref_eb64; ref_prep; ref_stats).  Test infrastructure: used to pin
# the oracle restatement and to generate tests/golden/.  Needs nvcc (the
# reference header mixes host code with thrust/CUDA device lambdas).  The
# shims in oracle/shim/ stand in for glog, nlohmann::json, HdrHistogram and
# OptiX, none of which the CPU path calls at run time.
#
# Usage: build_ref.sh <reference src directory>   (or HD_REFERENCE_SRC=<dir>)
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ref="${1:-${HD_REFERENCE_SRC:-}}"
if [ -z "$ref" ]; then
  echo "usage: $0 <reference src directory> (or set HD_REFERENCE_SRC)" >&2
  exit 2
fi
if [ ! -f "$ref/hd_impl/hausdorff_distance_early_break.h" ]; then
  echo "reference sources not found at $ref; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$here/_ref"
# --fmad=false and -ffp-contract=off: the reference builds with fmad off
# (CMakeLists.txt:122) and its squared distances must not be contracted.
nvcc -std=c++17 -O2 --extended-lambda --expt-relaxed-constexpr --fmad=false \
  -Xcompiler -ffp-contract=off -Xcompiler -pthread \
  -gencode arch=compute_103a,code=sm_103a \
  -I "$here/shim" -I "$ref" -include "$here/shim/prelude.h" \
  "$here/ref_eb_main.cu" -o "$here/_ref/ref_eb"
echo "built $here/_ref/ref_eb"
# The same early-break in the reference's double instantiation.
nvcc -std=c++17 -O2 --extended-lambda --expt-relaxed-constexpr --fmad=false \
  -Xcompiler -ffp-contract=off -Xcompiler -pthread -DREF_COORD=double \
  -gencode arch=compute_103a,code=sm_103a \
  -I "$here/shim" -I "$ref" -include "$here/shim/prelude.h" \
  "$here/ref_eb_main.cu" -o "$here/_ref/ref_eb64"
echo "built $here/_ref/ref_eb64"
# The reference's -normalize / -translate preprocessing (translate_points.h),
# for the golden vectors of hd_exec's same options.
nvcc -std=c++17 -O2 --extended-lambda --expt-relaxed-constexpr --fmad=false \
  -Xcompiler -ffp-contract=off \
  -gencode arch=compute_103a,code=sm_103a \
  -I "$here/shim" -I "$ref" -include "$here/shim/prelude.h" \
  "$here/ref_prep_main.cu" -o "$here/_ref/ref_prep"
echo "built $here/_ref/ref_prep"
# The host-side grid shape of the reference's per-file statistics.
nvcc -std=c++17 -O2 --extended-lambda --expt-relaxed-constexpr --fmad=false \
  -Xcompiler -ffp-contract=off \
  -gencode arch=compute_103a,code=sm_103a \
  -I "$here/shim" -I "$ref" -include "$here/shim/prelude.h" \
  "$here/ref_stats_main.cu" -o "$here/_ref/ref_stats"
echo "built $here/_ref/ref_stats"
