// tile_cover.cu -- host check of the tile lists of the TMA sweep kernels.
//
// Built and run by tests/test_tile_cover.py on the CPU (no GPU needed): for a
// grid and a tile shape it enumerates the tiles of the interior kernels
// (interior_tiles, chunks of kc planes over the interior's planes) and of the
// shell-tile kernels (shell_tile_count / shell_tile), replays which lanes of
// each tile update which points (the rules of stress_tma_tile and
// vel_tma_tile: an interior lane of an interior tile, an interior lane of a
// shell tile on the interior's planes, a shell lane), and checks that every
// grid point is updated exactly once, that every tile lies in the sweep grid
// and that no chunk is empty.  It also checks the interior-only view (the
// shell in launches of its own): every interior point exactly once.
// Arguments: nx ny nz na rows kc.  Prints "ok" or the first failure.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../openswpc_gb300/csrc/kernels_tma.cuh"

using namespace swpc;

static int fail(const char* what, int a, int b, int c) {
    std::printf("FAIL %s %d %d %d\n", what, a, b, c);
    return 1;
}

int main(int argc, char** argv) {
    if (argc != 7) {
        std::printf("usage: tile_cover nx ny nz na rows kc\n");
        return 2;
    }
    const int nx = std::atoi(argv[1]), ny = std::atoi(argv[2]), nz = std::atoi(argv[3]);
    const int na = std::atoi(argv[4]), TY = std::atoi(argv[5]), kc = std::atoi(argv[6]);
    static const float dummy_prof[4] = {0, 0, 0, 0};
    for (int shell_view = 1; shell_view >= 0; --shell_view) {
        ZArgs a{};
        a.x0 = na; a.y0 = na;
        a.nxi = nx - 2 * na; a.nyi = ny - 2 * na; a.nzi = nz - na;
        a.g.nx = nx; a.g.ny = ny; a.g.nz = nz;
        if (shell_view) {  // as Sim::fill_zargs with the shell swept by the tile kernels
            a.kz_end = nz;
            a.tx0 = a.x0 - 32 * ((a.x0 + 31) / 32);
            a.ty0 = 0;
            a.sx = nx - a.tx0;
            a.sy = ny;
            a.sh.prof = dummy_prof;
        } else {
            a.kz_end = a.nzi;
            a.tx0 = a.x0;
            a.ty0 = a.y0;
            a.sx = a.nxi;
            a.sy = a.nyi;
        }
        std::vector<unsigned char> hits((size_t)nx * ny * nz, 0);
        auto at = [&](int i, int j, int k) -> unsigned char& { return hits[((size_t)k * ny + j) * nx + i]; };
        const int ntx = (a.sx + 31) / 32, nty = (a.sy + TY - 1) / TY;
        // one tile over one chunk: the lanes that update a point
        auto visit = [&](int bx, int by, int kz0, bool shell_tile_kernel) -> int {
            if (bx < 0 || bx >= ntx || by < 0 || by >= nty) return fail("tile outside the sweep grid", bx, by, kz0);
            const int kz1 = chunk_end(a, kz0, kc);
            if (kz0 < 0 || kz0 >= kz1 || kz1 > a.kz_end) return fail("empty or out-of-range chunk", bx, by, kz0);
            for (int ty = 0; ty < TY; ++ty)
                for (int tx = 0; tx < 32; ++tx) {
                    const int ix = a.tx0 + bx * 32 + tx, jy = a.ty0 + by * TY + ty;
                    const bool interior = ix >= a.x0 && ix < a.x0 + a.nxi && jy >= a.y0 && jy < a.y0 + a.nyi;
                    const bool shell_col = a.sh.prof && !interior && ix >= 0 && ix < nx && jy >= 0 && jy < ny;
                    const bool shl = shell_tile_kernel && (shell_col || (interior && kz0 >= a.nzi));
                    for (int k = kz0; k < kz1; ++k) {
                        if (interior && !shl) {
                            if (k >= a.nzi) return fail("interior lane below the interior", ix, jy, k);
                            ++at(ix, jy, k);
                        } else if (shl) {
                            ++at(ix, jy, k);
                        }
                    }
                }
            return 0;
        };
        int bxl, bxh, byl, byh;
        interior_tiles(a, TY, bxl, bxh, byl, byh);
        for (int c = 0; c * kc < a.nzi; ++c)
            for (int by = byl; by < byh; ++by)
                for (int bx = bxl; bx < bxh; ++bx)
                    if (visit(bx, by, c * kc, false)) return 1;
        const int ns = shell_tile_count(a, TY, kc);
        if (!shell_view && ns != 0) return fail("shell tiles without a shell sweep", ns, 0, 0);
        for (int L = 0; L < ns; ++L) {
            int bx, by, kz0;
            shell_tile(a, TY, kc, L, bx, by, kz0);
            if (bx >= bxl && bx < bxh && by >= byl && by < byh && kz0 < a.nzi)
                return fail("shell list holds an interior tile", bx, by, kz0);
            if (visit(bx, by, kz0, true)) return 1;
        }
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const bool interior = i >= a.x0 && i < a.x0 + a.nxi && j >= a.y0 && j < a.y0 + a.nyi && k < a.nzi;
                    const int want = (shell_view || interior) ? 1 : 0;
                    if (at(i, j, k) != want) return fail(shell_view ? "point updated not once" : "interior point", i, j, k);
                }
    }
    std::printf("ok\n");
    return 0;
}
