#!/bin/sh
# Builds oracle/_ref/libshoccs_ref.so from the reference's OWN stencil and sphere
# translation units (compiled unmodified from the reference tree) plus oracle/ref_driver.cpp.
# Runs only where the reference tree exists; the product never loads the result.
set -e
REF=${SHOCCS_REFERENCE_ROOT:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
[ -d "$REF/src" ] || { echo "reference tree not found at $REF; skipping oracle/_ref"; exit 0; }
FMT_INC=$(python3 -c "import torch, os; print(os.path.join(os.path.dirname(torch.__file__), 'include'))")
mkdir -p "$HERE/_ref"
g++ -std=c++20 -O2 -fPIC -shared -ffp-contract=off -DNDEBUG -DFMT_HEADER_ONLY \
    -I"$HERE/ref_stubs" -I"$REF/src" -I"$FMT_INC" \
    "$REF/src/stencils/E2_2.cpp" "$REF/src/stencils/E4_2.cpp" "$REF/src/stencils/E4_1.cpp" "$REF/src/stencils/E4u_1.cpp" \
    "$REF/src/mesh/sphere.cpp" "$HERE/ref_driver.cpp" \
    -o "$HERE/_ref/libshoccs_ref.so"
echo "built $HERE/_ref/libshoccs_ref.so"
