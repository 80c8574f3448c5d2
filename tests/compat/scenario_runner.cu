// scenario_runner.cu -- test harness: runs one of the reference's own 2-D
// scenario headers, unchanged, on lbmx through the compat layer and
// evaluates the header's own compute_error validator on the lbmx solver, at
// the steps where the reference's main loop would (src/main.cu:144-156).
// Built by tests/test_compat.py with the same -D flags as the reference's
// validator binaries (oracle/ref_validate.cu, `ref_build.sh validators`).
#include "lbmx_scenario.cuh"
#include LBX_SCENARIO_HEADER

using Scenario = LBX_SCENARIO;

#ifdef LBX_DEFINE_CURRENT_VELOCITY
float Scenario::current_velocity = 0.0f;
#endif

extern "C" void scenario_lattice(int* nx, int* ny) {
    *nx = NX;
    *ny = NY;
}

// Steps to each of the ndump (increasing) step indices; after each, the
// scenario's compute_error into err_out[k] and the force-corrected velocity
// the validator read (AoS, u[2*node + c]) into u_out + k * 2 * NX * NY.
extern "C" int run_validation(const int* dump_steps, int ndump, float* err_out, float* u_out) {
    lbmx_compat::Solver<Scenario> sim;
    if (lbmx_compat::create<Scenario>(&sim.h) != LBMX_OK) return -1;
    const size_t n2 = 2 * (size_t)NX * NY;
    for (int k = 0; k < ndump; k++) {
        if (sim.step(dump_steps[k] - sim.timestep) != LBMX_OK) return -2;
        sim.update_macroscopics();
        if (sim.h_u.size() != n2) return -3;
        err_out[k] = Scenario::compute_error(sim);
        for (size_t i = 0; i < n2; i++) u_out[k * n2 + i] = sim.h_u[i];
    }
    return 0;
}
