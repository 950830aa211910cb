"""The tile lists of the TMA sweep kernels cover the grid exactly once (CPU).

tests/tile_cover.cu includes the kernels' own host/device tile functions
(interior_tiles, chunk_end, shell_tile_count, shell_tile of
openswpc_gb300/csrc/kernels_tma.cuh), replays which lanes of every tile update
which points, and checks that with the shell swept by the tile kernels every
grid point is updated exactly once per phase (and with the shell in launches
of its own every interior point), for odd interior widths, PML widths other
than 20, every tile height and chunk depths that do not divide the interior.
The program is built for the host with nvcc (PTX only for the device side,
nothing runs on a GPU)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc) and not shutil.which(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("tile_cover") / "tile_cover")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=compute_103a", "-O1", "-std=c++17",
                    "--expt-relaxed-constexpr", "-o", exe, os.path.join(HERE, "tile_cover.cu")],
                   check=True, capture_output=True)
    return exe


@pytest.mark.parametrize("nx,ny,nz,na,rows,kc", [
    (96, 80, 64, 20, 8, 8), (100, 84, 70, 13, 8, 8), (100, 84, 70, 20, 8, 5), (64, 96, 72, 20, 8, 8),
    (96, 80, 64, 20, 16, 16), (130, 70, 50, 20, 8, 3), (60, 60, 40, 20, 8, 8), (72, 72, 48, 20, 16, 7),
    (100, 84, 70, 20, 12, 5), (288, 288, 144, 20, 12, 33), (384, 384, 192, 20, 8, 58), (200, 96, 80, 40, 8, 8),
])
def test_tiles_cover_every_point_once(checker, nx, ny, nz, na, rows, kc):
    r = subprocess.run([checker, str(nx), str(ny), str(nz), str(na), str(rows), str(kc)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout
