// ref_timer.cu -- times the patched reference build's own D2Q9 step on the
// GPU.  Test infrastructure: a measurement of the reference (the
// kernel-for-kernel bar), never linked into the product.  Built by
// oracle/ref_build.sh (`timers`) against the same patched copy as the golden
// harness, with a scenario from ref_scenarios.cuh.
//
// One step is the call sequence of the reference's main loop
// (src/main.cu:96-114), on its default stream.  CUDA events bracket `steps`
// back-to-back steps after `warmup` untimed ones.
//
// usage: <binary> [warmup=50] [steps=1000]   -> one JSON line on stdout
#include <cstdio>
#include <cstdlib>

#include "core/lbm.cuh"
#include "ref_scenarios.cuh"

using Golden = GoldenScenario;

static void step(LBM<2>& lbm) {
    lbm.increase_ts<Golden>();
    lbm.stream();
    lbm.swap_buffers();
    lbm.apply_boundaries<Golden>();
    lbm.uncorrected_macroscopics();
    lbm.reset_forces<Golden>();
    lbm.ibm_step();
    lbm.correct_macroscopics();
    lbm.compute_equilibrium();
    lbm.collide<Golden::CollisionOp>();
}

int main(int argc, char** argv) {
    const int warmup = argc > 1 ? atoi(argv[1]) : 50;
    const int steps = argc > 2 ? atoi(argv[2]) : 1000;
    if (warmup < 0 || steps < 1) {
        fprintf(stderr, "usage: %s [warmup] [steps]\n", argv[0]);
        return 2;
    }
    LBM<2> lbm;
    lbm.allocate<Golden>();
    lbm.init<Golden>();
    for (int i = 0; i < warmup; i++) step(lbm);
    cudaDeviceSynchronize();
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    cudaEventRecord(t0, 0);
    for (int i = 0; i < steps; i++) step(lbm);
    cudaEventRecord(t1, 0);
    cudaEventSynchronize(t1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        fprintf(stderr, "ref_timer: %s\n", cudaGetErrorString(err));
        return 5;
    }
    const double per_step = (double)ms / steps;
    printf("{\"nx\": %d, \"ny\": %d, \"case\": %d, \"op\": %d, \"warmup\": %d, \"steps\": %d, "
           "\"ms_per_step\": %.5f, \"mlups\": %.1f}\n",
           NX, NY, LBX_CASE, LBX_OPID, warmup, steps, per_step, (double)NX * NY / (per_step * 1e3));
    return 0;
}
