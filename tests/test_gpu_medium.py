"""The medium the host layer uploads (read back from the device) equals the
oracle's medium after medium__setup, with and without the absorber
conditioning of stabilize_pml (m_medium.f90:273-337)."""
import os

import numpy as np
import pytest

from openswpc_gb300 import configs, gpu
from oracle import pyoracle

# a slow top layer (Vs 1.5 km/s < 0.4 x 6.5) and a 4-cell low-velocity zone
LAYERS = [(0, 2.3, 2.8, 1.5, 100, 50), (2, 2.7, 6.0, 3.5, 300, 150), (4, 2.6, 5.0, 2.9, 300, 150),
          (6, 2.9, 6.5, 3.7, 600, 300)]


def _medium_case(d, stabilize):
    inf = configs.write_plain_small(str(d), nt=5, stabilize_pml=stabilize)
    configs.write_lhm(os.path.join(str(d), "lhm.dat"), LAYERS)
    return inf


@pytest.mark.gpu
@pytest.mark.parametrize("stabilize", [False, True])
def test_uploaded_medium_matches_oracle(tmp_path, stabilize):
    inf = _medium_case(tmp_path, stabilize)
    o = pyoracle.Oracle(inf, "fp32")
    s = gpu.Simulation.from_inf(inf)
    for name in ("rho", "lam", "mu", "taup", "taus"):
        ref = o.medium(name)[3:-3, 3:-3, 3:-3].astype(np.float64)  # (ny, nx, nz) physical cells
        got = s.field(name)
        assert got.shape == ref.shape
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err < 2e-6, (name, err)
    s.close()


def test_stabilize_pml_changes_the_absorber_only(tmp_path):
    """Oracle-side check that runs without a GPU: the conditioning raises the
    slow layer's Vs inside the absorber and leaves the interior alone."""
    a = pyoracle.Oracle(_medium_case(tmp_path / "a", False), "fp32")
    b = pyoracle.Oracle(_medium_case(tmp_path / "b", True), "fp32")
    mu_a, mu_b, rho = a.medium("mu"), b.medium("mu"), b.medium("rho")
    vs_b = np.sqrt(mu_b / np.where(rho > 0, rho, 1))
    na = 20
    # interior column (i, j) = (64, 64): unchanged
    assert np.array_equal(mu_a[64 + 2, 64 + 2], mu_b[64 + 2, 64 + 2])
    # absorber column (i, j) = (5, 64): no solid cell slower than 0.4 x max Vp
    col = vs_b[64 + 2, 5 + 2, 3:-3]
    solid = col[col > 1e-3]
    assert solid.min() >= 0.4 * 6.5 * 0.97  # 0.4 x the largest (relaxed) Vp
    assert vs_b[64 + 2, 64 + 2, 3:-3][vs_b[64 + 2, 64 + 2, 3:-3] > 1e-3].min() < 2.0  # slow layer kept inside
    assert not np.array_equal(mu_a[64 + 2, 5 + 2], mu_b[64 + 2, 5 + 2])
    assert na == b.na
