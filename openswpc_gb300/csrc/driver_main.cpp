// driver_main.cpp -- swpc_3d_gpu: command-line drop-in for swpc_3d's driver
// (src/swpc_3d/main.f90:48-158): swpc_3d_gpu -i input.inf
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/swpc_gpu.h"

extern "C" int swpc_host_nt(swpc_sim* sim);

static int fail(const char* what) {
    char buf[1024];
    swpc_gpu_last_error(buf, sizeof buf);
    std::fprintf(stderr, "swpc_3d_gpu: %s: %s\n", what, buf);
    return 1;
}

int main(int argc, char** argv) {
    std::string inf = "./in/input.inf";
    std::string odir;
    for (int a = 1; a < argc; ++a) {
        if ((!std::strcmp(argv[a], "-i")) && a + 1 < argc) inf = argv[++a];
        else if ((!std::strcmp(argv[a], "-o")) && a + 1 < argc) odir = argv[++a];
        else if (!std::strcmp(argv[a], "-v") || !std::strcmp(argv[a], "--version")) {
            std::printf("swpc_3d_gpu (GB300 swpc_3d time loop)\n");
            return 0;
        }
    }
    swpc_sim* sim = nullptr;
    if (swpc_host_prepare(inf.c_str(), &sim)) return fail("set-up");
    int ntw = 0, nst = 0;
    swpc_gpu_query(sim, &ntw, &nst, nullptr, nullptr, nullptr);
    int nt = 0;
    // the number of steps is carried by the simulation's dims; run them all
    nt = swpc_host_nt(sim);
    auto t0 = std::chrono::steady_clock::now();
    if (swpc_gpu_run(sim, 1, nt)) return fail("time loop");
    if (swpc_gpu_sync(sim)) return fail("time loop");
    auto t1 = std::chrono::steady_clock::now();
    double s = std::chrono::duration<double>(t1 - t0).count();
    std::fprintf(stderr, "  time loop: %d steps in %.3f s (%.3f ms/step)\n", nt, s, 1e3 * s / nt);
    if (nst > 0 && swpc_host_write_sac(sim, odir.empty() ? nullptr : odir.c_str())) return fail("waveform output");
    if (swpc_host_write_snp(sim, odir.empty() ? nullptr : odir.c_str())) return fail("snapshot output");
    if (swpc_host_write_green(sim, odir.empty() ? nullptr : odir.c_str())) return fail("Green's-function output");
    swpc_gpu_destroy(sim);
    return 0;
}
