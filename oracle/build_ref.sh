#!/usr/bin/env bash
# ORACLE build recipe (test infrastructure).  Compiles the reference's own,
# unmodified C++ translation units for the solid transfer path and the
# stabilized fluid assembly plus
# oracle/ref_harness.cpp into oracle/_ref/libmpmref.so, against the
# single-rank stubs in oracle/ref_stubs/.  Reads the reference sources where
# they lie; copies nothing.  The checkout is named by the first argument or,
# failing that, by MPM_REFERENCE_DIR; the recipe exits 0 without building when
# neither names a checkout (it is only present in the development container):
#     oracle/build_ref.sh <reference checkout>
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${MPM_REFERENCE_DIR:-}}"
OUT="$HERE/_ref"
if [ -z "$REF" ] || [ ! -d "$REF/module" ]; then
    echo "build_ref: no reference checkout given (argument or MPM_REFERENCE_DIR); skipping oracle/_ref" >&2
    exit 0
fi
mkdir -p "$OUT/obj"
TUS="shape_function mesh material_point map_and_interpolate nonlinear_time_integration bc data_io mpi_data
     solid/constitutive_model solid/solid_material_point solid/solid_data_io
     solid/implicit/var_trans_solid_implicit solid/implicit/solve_solid_implicit
     solver/crsmat solver/solver
     fluid/MPM/solve_ns_mpm fluid/MPM/var_trans_fluid fluid/MPM/fluid_material_point
     fluid/MPM/fluid_mpm_data_io fluid/MPM/fluid_point_inflow"
CXX="${CXX:-g++}"
FLAGS="-std=c++17 -O3 -fPIC -w -I$HERE/ref_stubs -I$REF/module"
pids=()
objs=()
for tu in $TUS; do
    o="$OUT/obj/$(echo "$tu" | tr / _).o"
    objs+=("$o")
    $CXX $FLAGS -c "$REF/module/$tu.cpp" -o "$o" &
    pids+=($!)
done
$CXX $FLAGS -c "$HERE/ref_harness.cpp" -o "$OUT/obj/ref_harness.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
$CXX -shared -o "$OUT/libmpmref.so" "${objs[@]}" "$OUT/obj/ref_harness.o"
echo "build_ref: wrote $OUT/libmpmref.so"
