#!/usr/bin/env bash
# Builds the reference implementation (qognitive/fast-pauli, header-only C++)
# from its own headers where they lie, unmodified, into oracle/_ref/.
# Test infrastructure only.  Needs: g++ >= 13 with OpenMP, fmt headers (the
# copy bundled in torch/include, header-only), CCCL's cuda::std::mdspan (CUDA
# toolkit) and the small shim in oracle/shim.  The reference's CMake cannot run
# offline (it fetches its dependencies), so it is not used.
# The reference tree is FP_REFERENCE_ROOT, by default the checkout this recipe
# was written against; where it is absent the recipe builds nothing.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${FP_REFERENCE_ROOT:-/root/reference}"
INC="$REF/fast_pauli/cpp/include"
if [ ! -d "$INC" ]; then
  echo "reference headers not found at $INC; oracle/_ref not built" >&2
  exit 3
fi
TORCH_INC="$(python3 -c 'import torch, os; print(os.path.join(os.path.dirname(torch.__file__), "include"))')"
CCCL="$(ls -d /usr/local/cuda/targets/*/include/cccl | head -1)"
mkdir -p "$HERE/_ref"
g++ -std=c++20 -O3 -fopenmp -fPIC -shared -DFMT_HEADER_ONLY \
  -I"$HERE/shim" -I"$CCCL" -I"$TORCH_INC" -I"$INC" \
  "$HERE/ref_driver.cpp" -o "$HERE/_ref/libfpref.so"
echo "built $HERE/_ref/libfpref.so"
