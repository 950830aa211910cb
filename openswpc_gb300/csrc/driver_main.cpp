// driver_main.cpp -- swpc_3d_gpu: command-line drop-in for swpc_3d's driver
// (src/swpc_3d/main.f90:48-158): swpc_3d_gpu -i input.inf
//
// Like the reference it prints the run banner (report__setup,
// src/swpc_3d/m_report.f90:64-88) and, every ntdec_r steps, a progress line
// with the max |V| at the ocean bottom (report__progress,
// m_report.f90:120-181), to standard error.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/swpc_gpu.h"

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
    {
        char buf[2048];
        if (swpc_host_banner(sim, buf, sizeof buf) > 0) std::fputs(buf, stderr);
    }
    const int nt = swpc_host_nt(sim);
    const int ntdec_r = swpc_host_ntdec_r(sim);
    // the loop runs in pieces of ntdec_r steps (graph replay inside each
    // piece); after each piece the report step's max |V| is read back
    const int piece = ntdec_r > 0 ? ntdec_r : nt;
    auto t0 = std::chrono::steady_clock::now();
    for (int it0 = 1; it0 <= nt; it0 += piece) {
        const int it1 = std::min(nt, it0 + piece - 1);
        if (swpc_gpu_run(sim, it0, it1)) return fail("time loop");
        if (swpc_gpu_sync(sim)) return fail("time loop");
        if (ntdec_r > 0 && it1 % ntdec_r == 0) {
            float v[3];
            if (swpc_gpu_vmax(sim, v)) return fail("time loop");
            const double tt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            double eta = (double)(nt - it1) / it1 * tt;
            const int eh = (int)(eta / 3600);
            eta -= eh * 3600;
            const int em = (int)(eta / 60);
            eta -= em * 60;
            std::fprintf(stderr, "  it=%07d,%6.3f s/loop, eta %03d:%02d:%02d, (%9.2E %9.2E %9.2E )\n", it1, tt / it1, eh, em,
                         (int)eta, v[0], v[1], v[2]);
        }
    }
    auto t1 = std::chrono::steady_clock::now();
    double s = std::chrono::duration<double>(t1 - t0).count();
    std::fprintf(stderr, "\n ------------------------------------------------------------------------------\n\n");
    std::fprintf(stderr, "  Total time             : %15.3f s\n\n", s);
    std::fprintf(stderr, " ------------------------------------------------------------------------------\n");
    std::fprintf(stderr, "  time loop: %d steps in %.3f s (%.3f ms/step)\n", nt, s, 1e3 * s / nt);
    int nst = 0;
    swpc_gpu_query(sim, nullptr, &nst, nullptr, nullptr, nullptr);
    if (nst > 0 && swpc_host_write_sac(sim, odir.empty() ? nullptr : odir.c_str())) return fail("waveform output");
    if (swpc_host_write_snp(sim, odir.empty() ? nullptr : odir.c_str())) return fail("snapshot output");
    if (swpc_host_write_green(sim, odir.empty() ? nullptr : odir.c_str())) return fail("Green's-function output");
    swpc_gpu_destroy(sim);
    return 0;
}
