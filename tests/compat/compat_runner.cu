// compat_runner.cu -- test harness: runs the golden scenarios of
// oracle/ref_scenarios.cuh (written against the reference's scenario
// contract) on lbmx through the compat layer, with the same -D flags the
// reference harness was built with.  Loaded by tests/test_compat.py.
#include "lbmx_scenario.cuh"
#include "ref_scenarios.cuh"

// Steps the scenario to each of the ndump (increasing) step indices and
// writes populations [9][n], density [n] and velocity [2][n] after each.
extern "C" int run_scenario(const int* dump_steps, int ndump, float* f_out, float* rho_out, float* u_out) {
    lbmx_compat::Solver<GoldenScenario> sim;
    if (lbmx_compat::create<GoldenScenario>(&sim.h) != LBMX_OK) return -1;
    const int n = NX * NY;
    for (int k = 0; k < ndump; k++) {
        if (sim.step(dump_steps[k] - sim.timestep) != LBMX_OK) return -2;
        if (lbmx_get_populations(sim.h, f_out + (size_t)k * 9 * n) != LBMX_OK) return -3;
        if (lbmx_moments(sim.h, rho_out + (size_t)k * n, u_out + (size_t)k * 2 * n, nullptr) != LBMX_OK) return -4;
    }
    return 0;
}

// the unchanged scenario's other contract members compile against the layer
extern "C" int scenario_lattice(int* nx, int* ny) {
    *nx = NX;
    *ny = NY;
    return GoldenScenario::CollisionOp::lbmx_op;
}
