// ref_validate.cu -- runs one of the reference's own, unchanged 2-D scenario
// headers on the patched reference build and records its validator.  Test
// infrastructure: the numbers it prints are the golden values the lbmx run of
// the same header (tests/compat/scenario_runner.cu) is held to.  Built by
// oracle/ref_build.sh (`validators`) with
//   -DLBX_SCENARIO_HEADER="scenarios/<dir>/<name>Scenario.cuh"
//   -DLBX_SCENARIO=<ScenarioStruct>
// and the scenario's as-shipped NX / NY / SCALE / periodicity
// (src/defines.hpp:20-35, src/core/streaming/streaming.cuh:8-11).
//
// One step is the call sequence of the reference's main loop
// (src/main.cu:96-114).  At each requested step it does what the main loop's
// save branch does (src/main.cu:144-156): update_macroscopics() and
// Scenario::compute_error(lbm).
//
// usage: <binary> <out_dir> <dump steps...>
// Prints one line per dump step, "<t> <compute_error>", and writes
// <out_dir>/u<t>.bin: the force-corrected velocity h_u (AoS, u[2*node + c]).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "core/lbm.cuh"
#include LBX_SCENARIO_HEADER

using Scenario = LBX_SCENARIO;

#ifdef LBX_DEFINE_CURRENT_VELOCITY
// declared by FlowPastCylinderScenario (flowPastCylinderScenario.cuh:27) and
// defined nowhere in the reference; a linked program needs one definition
float Scenario::current_velocity = 0.0f;
#endif

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s <out_dir> <dump steps...>\n", argv[0]);
        return 2;
    }
    const char* dir = argv[1];
    std::vector<int> at;
    for (int i = 2; i < argc; i++) at.push_back(atoi(argv[i]));
    LBM<2> lbm;
    lbm.allocate<Scenario>();
    lbm.init<Scenario>();
    int t = 0;
    for (int t_dump : at) {
        for (; t < t_dump; t++) {
            lbm.increase_ts<Scenario>();
            lbm.stream();
            lbm.swap_buffers();
            lbm.apply_boundaries<Scenario>();
            lbm.uncorrected_macroscopics();
            lbm.reset_forces<Scenario>();
            lbm.ibm_step();
            lbm.correct_macroscopics();
            lbm.compute_equilibrium();
            lbm.collide<Scenario::CollisionOp>();
        }
        lbm.update_macroscopics();
        const float err = Scenario::compute_error(lbm);
        printf("%d %.9g\n", t, err);
        char path[1024];
        snprintf(path, sizeof(path), "%s/u%d.bin", dir, t);
        FILE* fp = fopen(path, "wb");
        if (!fp) {
            fprintf(stderr, "cannot write %s\n", path);
            return 4;
        }
        fwrite(lbm.h_u.data(), sizeof(float), lbm.h_u.size(), fp);
        fclose(fp);
    }
    cudaDeviceSynchronize();
    return cudaGetLastError() == cudaSuccess ? 0 : 5;
}
