// ref_harness.cu -- golden-dump driver for the patched reference build.
// Test infrastructure: it runs the reference's own LBM<2> through the exact
// call sequence of its main loop (src/main.cu:96-114) and writes the device
// state at requested steps.  Built by oracle/ref_build.sh.
//
// usage: <binary> <out_dir> <nsteps> <dump steps...>
// Each dump <out_dir>/t<step>.bin holds, little-endian:
//   int32 magic 0x4658424c, nx, ny, t, nmarkers
//   float32 f[nx*ny*9] (AoS, node*9+q, as the patched build stores it)
//   float32 rho[nx*ny], u[nx*ny*2] (AoS), force[nx*ny*2] (AoS)
//   float32 marker xy[nmarkers*2]
//   int32 boundary flags[nx*ny]
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "core/lbm.cuh"
#include "ref_scenarios.cuh"

using Golden = GoldenScenario;

static void dump(LBM<2>& lbm, const char* dir, int t) {
    const int n = NX * NY;
    std::vector<float> f(9 * (size_t)n), rho(n), u(2 * (size_t)n), F(2 * (size_t)n);
    cudaDeviceSynchronize();
    cudaMemcpy(f.data(), lbm.d_f, f.size() * sizeof(float), cudaMemcpyDeviceToHost);
    cudaMemcpy(rho.data(), lbm.d_rho, rho.size() * sizeof(float), cudaMemcpyDeviceToHost);
    cudaMemcpy(u.data(), lbm.d_u, u.size() * sizeof(float), cudaMemcpyDeviceToHost);
    cudaMemcpy(F.data(), lbm.d_force, F.size() * sizeof(float), cudaMemcpyDeviceToHost);
    const int nm = lbm.IBM.num_points;
    std::vector<float> xy(2 * (size_t)nm);
    if (nm > 0) cudaMemcpy(xy.data(), lbm.IBM.d_lag_points, xy.size() * sizeof(float), cudaMemcpyDeviceToHost);
    std::vector<int> flags(n);
    cudaMemcpy(flags.data(), lbm.d_boundary_flags, flags.size() * sizeof(int), cudaMemcpyDeviceToHost);
    if (cudaGetLastError() != cudaSuccess) {
        fprintf(stderr, "dump: CUDA error\n");
        exit(3);
    }
    char path[1024];
    snprintf(path, sizeof(path), "%s/t%06d.bin", dir, t);
    FILE* fp = fopen(path, "wb");
    if (!fp) {
        fprintf(stderr, "cannot write %s\n", path);
        exit(4);
    }
    const int hdr[5] = {0x4658424c, NX, NY, t, nm};
    fwrite(hdr, sizeof(int), 5, fp);
    fwrite(f.data(), sizeof(float), f.size(), fp);
    fwrite(rho.data(), sizeof(float), rho.size(), fp);
    fwrite(u.data(), sizeof(float), u.size(), fp);
    fwrite(F.data(), sizeof(float), F.size(), fp);
    fwrite(xy.data(), sizeof(float), xy.size(), fp);
    fwrite(flags.data(), sizeof(int), flags.size(), fp);
    fclose(fp);
}

int main(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s <out_dir> <nsteps> <dump steps...>\n", argv[0]);
        return 2;
    }
    const char* dir = argv[1];
    const int nsteps = atoi(argv[2]);
    std::vector<int> at;
    for (int i = 3; i < argc; i++) at.push_back(atoi(argv[i]));
    auto wanted = [&](int t) {
        for (int v : at)
            if (v == t) return true;
        return false;
    };
    LBM<2> lbm;
    lbm.allocate<Golden>();
    lbm.init<Golden>();
    if (wanted(0)) dump(lbm, dir, 0);
    for (int t = 1; t <= nsteps; t++) {
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
        if (wanted(t)) dump(lbm, dir, t);
    }
    cudaDeviceSynchronize();
    return cudaGetLastError() == cudaSuccess ? 0 : 5;
}
