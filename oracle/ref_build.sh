#!/bin/bash
# Recipe for the reference's own 2-D build, used to make golden vectors and to
# time the reference's GPU step (test infrastructure; nothing in the product
# links it).
#
#   ref_build.sh sources   copy src/ and third_party/ of the reference checkout
#                          into oracle/_ref/ and patch the COPY so the D2Q9
#                          path compiles (the checkout is never modified)
#   ref_build.sh build     compile oracle/ref_harness.cu against the patched
#                          copy, one binary per golden case, into oracle/_ref/bin/
#   ref_build.sh timers    compile oracle/ref_timer.cu the same way, one binary
#                          per timed configuration (oracle/_ref/bin/time_*), to
#                          time the reference's own GPU step
#   ref_build.sh validators  compile oracle/ref_validate.cu the same way, once per
#                          unchanged 2-D scenario header (oracle/_ref/bin/validate_*),
#                          to record the scenarios' own compute_error
#
# oracle/_ref/ is git-ignored; it travels with the working tree, so `build`
# also works where the reference checkout is absent.  The patches are the
# minimum that makes the shipped 2-D path build:
#   defines.hpp            D2Q9 on, D3Q27 off; NX/NY/periodicity come from -D flags
#   boundaries.cuh:11      `float rho` -> `float* rho` (its launch passes d_rho)
#   zeroGradientOutflow:13 arrays sized 3 (a dim=2 instantiation initialises 3 values)
#   scenario.cuh           include IBM_generators.cuh (create_cylinder)
#   lbm_constants.cuh:298  drop `#define SOA`: the 2-D functors index AoS
#                          (u[2*node], get_node_index(node)+q)
#   lbm.cuh:35             `private:` -> `public:` so the harness can read d_f
#   adapters.cuh:101       silence the per-node OptimalAdapter printf
#   flowPastCylinderScenario.cuh:12  `BGK` -> `BGK<2>` (the header names the
#                          template without its argument and builds nowhere as shipped)
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${LBMX_REFERENCE:-/root/reference}
OUT=$HERE/_ref
NVCC=${NVCC:-nvcc}

sources() {
    rm -rf "$OUT/src" "$OUT/third_party"
    mkdir -p "$OUT"
    cp -r "$REF/src" "$OUT/src"
    cp -r "$REF/third_party" "$OUT/third_party"
    chmod -R u+w "$OUT"
    local S=$OUT/src
    cat > "$S/defines.hpp" <<'EOF'
#ifndef DEFINES_H
#define DEFINES_H
/* written by oracle/ref_build.sh: 2-D lattice, sizes from the command line */
#define D2Q9
#ifndef SCALE
#define SCALE 1
#endif
#ifndef NZ
#define NZ 1
#endif
#define BLOCK_SIZE 16
#endif
EOF
    sed -i '11s/float\* u, float rho, int\* boundary_flags/float* u, float* rho, int* boundary_flags/' \
        "$S/core/boundaries/boundaries.cuh"
    sed -i 's/int normal\[dim\] = {0};/int normal[3] = {0};/; s/int interior_node_coord\[dim\] = {x, y, z};/int interior_node_coord[3] = {x, y, z};/' \
        "$S/functors/boundaryConditions/zeroGradientOutflow.cuh"
    sed -i 's|#include "IBM/IBMBody.cuh"|#include "IBM/IBMBody.cuh"\n#include "IBM/IBM_generators.cuh"|' \
        "$S/scenarios/scenario.cuh"
    sed -i '298s|^#define SOA$|// #define SOA|' "$S/core/lbm_constants.cuh"
    sed -i '35s/^private:/public:/' "$S/core/lbm.cuh"
    sed -i '101s/if (fabsf(tau_star_old) > 0.5f || fabsf(tau_star_old) < 0.1f){/if (false) {/' \
        "$S/core/collision/adapters.cuh"
    sed -i -E 's/^([[:space:]]*)BGK(\r?)$/\1BGK<2>\2/' "$S/scenarios/flowPastCylinder/flowPastCylinderScenario.cuh"
    grep -q 'BGK<2>' "$S/scenarios/flowPastCylinder/flowPastCylinderScenario.cuh"
    grep -q 'float\* rho, int\* boundary_flags' "$S/core/boundaries/boundaries.cuh"
    grep -q '^// #define SOA' "$S/core/lbm_constants.cuh"
    grep -q '^public:' "$S/core/lbm.cuh"
    echo "patched reference sources in $OUT/src"
}

# case name | -D flags (see ref_scenarios.cuh)
CASES=(
  "tg_bgk|-DNX=32 -DNY=32 -DPERIODIC_X -DPERIODIC_Y -DLBX_CASE=1 -DLBX_OPID=0 -DLBX_NU=0.01f"
  "tg_mrt|-DNX=32 -DNY=32 -DPERIODIC_X -DPERIODIC_Y -DLBX_CASE=1 -DLBX_OPID=1 -DLBX_NU=0.01f"
  "tg_cm|-DNX=32 -DNY=32 -DPERIODIC_X -DPERIODIC_Y -DLBX_CASE=1 -DLBX_OPID=2 -DLBX_NU=0.01f"
  "tg_cmopt|-DNX=32 -DNY=32 -DPERIODIC_X -DPERIODIC_Y -DLBX_CASE=1 -DLBX_OPID=3 -DLBX_NU=0.01f"
  "cavity_bgk|-DNX=32 -DNY=24 -DLBX_CASE=2 -DLBX_OPID=0 -DLBX_NU=0.02f"
  "cavity_mrt|-DNX=32 -DNY=24 -DLBX_CASE=2 -DLBX_OPID=1 -DLBX_NU=0.02f"
  "poiseuille_ibm_bgk|-DNX=48 -DNY=24 -DPERIODIC_X -DLBX_CASE=3 -DLBX_OPID=0 -DLBX_NU=0.1666667f"
  "poiseuille_mrt|-DNX=48 -DNY=24 -DPERIODIC_X -DLBX_CASE=3 -DLBX_OPID=1 -DLBX_NU=0.1666667f -DLBX_NO_MARKERS"
  "channel_zg_bgk|-DNX=48 -DNY=24 -DLBX_CASE=4 -DLBX_OPID=0 -DLBX_NU=0.04f"
  "channel_pressure_cm|-DNX=48 -DNY=24 -DLBX_CASE=5 -DLBX_OPID=2 -DLBX_NU=0.04f"
)

# timed configurations | -D flags: the 1024^2 lid-driven cavity (MRT, Re 1000,
# the reference's regularized walls) and the 256^2 Taylor-Green vortex (BGK)
TIMERS=(
  "time_cavity1024_mrt|-DNX=1024 -DNY=1024 -DLBX_CASE=2 -DLBX_OPID=1 -DLBX_NU=0.1024f"
  "time_tg256_bgk|-DNX=256 -DNY=256 -DPERIODIC_X -DPERIODIC_Y -DLBX_CASE=1 -DLBX_OPID=0 -DLBX_NU=0.01f"
)

# unchanged scenario headers | struct | their as-shipped lattice and periodicity
# (src/defines.hpp:20-35; periodic where the flow is: Taylor-Green in x and y,
# the Poiseuille channel in x)
VALIDATORS=(
  "validate_tg|scenarios/taylorGreen/taylorGreenScenario.cuh|TaylorGreenScenario|-DNX=256 -DNY=256 -DSCALE=2 -DPERIODIC_X -DPERIODIC_Y"
  "validate_ldc|scenarios/lidDrivenCavity/lidDrivenCavityScenario.cuh|LidDrivenScenario|-DNX=129 -DNY=129"
  "validate_poiseuille|scenarios/poiseuille/poiseuilleScenario.cuh|PoiseuilleScenario|-DNX=150 -DNY=100 -DPERIODIC_X"
  "validate_cylinder|scenarios/flowPastCylinder/flowPastCylinderScenario.cuh|FlowPastCylinderScenario|-DNX=256 -DNY=128 -DLBX_DEFINE_CURRENT_VELOCITY"
)

build() {
    local S=$OUT/src
    [ -d "$S" ] || { echo "no patched sources in $OUT/src (run: ref_build.sh sources)"; exit 1; }
    mkdir -p "$OUT/bin" "$OUT/obj"
    local FLAGS="-gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -rdc=true -w -I$S -I$OUT/third_party -I$HERE"
    local SRCS="$S/core/lbm.cu $S/core/streaming/streaming.cu $S/core/macroscopics/macroscopics.cu \
$S/core/equilibrium/equilibrium.cu $S/core/collision/MRT/MRT.cu $S/core/collision/CM/CM.cu \
$S/IBM/IBM_impl.cu $S/IBM/IBM_generators.cu $S/util/utility.cu"
    local pids=()
    local driver=$HERE/ref_harness.cu
    local list=("${CASES[@]}")
    if [ "${1:-}" = timers ]; then driver=$HERE/ref_timer.cu; list=("${TIMERS[@]}"); fi
    if [ "${1:-}" = validators ]; then
        driver=$HERE/ref_validate.cu
        list=()
        for v in "${VALIDATORS[@]}"; do
            IFS='|' read -r vn vh vs vd <<< "$v"
            list+=("$vn|-DLBX_SCENARIO_HEADER=\"$vh\" -DLBX_SCENARIO=$vs $vd")
        done
    fi
    for c in "${list[@]}"; do
        local name=${c%%|*} defs=${c#*|}
        ( $NVCC $FLAGS $defs "$driver" $SRCS -o "$OUT/bin/$name" > "$OUT/obj/$name.log" 2>&1 \
          || { echo "build of $name failed:"; tail -30 "$OUT/obj/$name.log"; exit 1; } ) &
        pids+=($!)
    done
    local rc=0
    for p in "${pids[@]}"; do wait "$p" || rc=1; done
    [ $rc -eq 0 ] && echo "built ${#list[@]} reference binaries in $OUT/bin"
    return $rc
}

list() { for c in "${CASES[@]}"; do echo "${c%%|*}|${c#*|}"; done; }
validators_list() { for v in "${VALIDATORS[@]}"; do echo "$v"; done; }

case "${1:-}" in
    sources) sources ;;
    build) build ;;
    timers) build timers ;;
    validators) build validators ;;
    list) list ;;
    validators-list) validators_list ;;
    *) echo "usage: $0 sources|build|timers|validators|list|validators-list"; exit 2 ;;
esac
