#!/bin/sh
# Builds oracle/_ref/libshoccs_ref.so from the reference's OWN hot-path translation units
# (stencils, mesh, matrices, operators, the heat and scalar-wave systems, the RK4 integrator,
# manufactured solutions), compiled unmodified from the reference tree, plus
# oracle/ref_driver.cpp and oracle/ref_unbuilt.cpp, against the
# serial Kokkos / sol / spdlog stand-ins in oracle/ref_stubs and fmt's header-only build
# (shipped inside torch's include directory).
#
# TEST INFRASTRUCTURE ONLY: the product never loads the result.  The reference tree is
# found through SHOCCS_REFERENCE_ROOT, else as the directory `reference` beside this
# repository; where neither exists the script does nothing.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${SHOCCS_REFERENCE_ROOT:-$(dirname "$(dirname "$HERE")")/reference}
[ -d "$REF/src" ] || { echo "reference tree not found at $REF; skipping oracle/_ref"; exit 0; }
FMT_INC=$(python3 -c "import torch, os; print(os.path.join(os.path.dirname(torch.__file__), 'include'))")
OBJ="$HERE/_ref/obj"
mkdir -p "$OBJ"
TUS="stencils/E2_2 stencils/E4_2 stencils/E4_1 stencils/E4u_1 stencils/polyE2_1 stencils/E6u_1 stencils/E8u_1 stencils/stencil
     mesh/sphere mesh/rect mesh/cartesian mesh/object_geometry mesh/mesh
     matrices/csr matrices/inner_block matrices/circulant matrices/dense
     matrices/coefficient_visitor matrices/unit_stride_visitor
     operators/boundaries operators/derivative operators/laplacian operators/gradient
     systems/heat systems/scalar_wave systems/system systems/empty_system
     systems/inviscid_vortex systems/hyperbolic_eigenvalues
     temporal/rk4 temporal/euler temporal/integrator temporal/step_controller
     mms/mms mms/gauss1d mms/gauss2d mms/gauss3d mms/lua_mms
     io/logging io/field_io io/field_data"
FLAGS="-std=c++20 -O2 -fPIC -ffp-contract=off -DNDEBUG -DFMT_HEADER_ONLY -w
       -I$HERE/ref_stubs -I$REF/src -I$FMT_INC"
pids=""
objs=""
for tu in $TUS; do
    o="$OBJ/$(echo "$tu" | tr / _).o"
    objs="$objs $o"
    if [ ! -f "$o" ] || [ "$REF/src/$tu.cpp" -nt "$o" ] || [ "$HERE/ref_stubs/Kokkos_Core.hpp" -nt "$o" ]; then
        g++ $FLAGS -c "$REF/src/$tu.cpp" -o "$o" &
        pids="$pids $!"
    fi
done
g++ $FLAGS -c "$HERE/ref_driver.cpp" -o "$OBJ/ref_driver.o" &
pids="$pids $!"
g++ $FLAGS -c "$HERE/ref_unbuilt.cpp" -o "$OBJ/ref_unbuilt.o" &
pids="$pids $!"
for p in $pids; do wait "$p"; done
g++ -shared -fPIC -Wl,--no-undefined $objs "$OBJ/ref_driver.o" "$OBJ/ref_unbuilt.o" -o "$HERE/_ref/libshoccs_ref.so"
echo "built $HERE/_ref/libshoccs_ref.so"
