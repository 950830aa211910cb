"""Parity of the CUDA time loop with the CPU oracle (FP32 restatement of the
reference, MP = SP) on identical inputs.

Tolerance: relative L2 misfit <= 1e-5 of receiver waveforms (the stated
bar), and of the full wavefields after a few steps.  The GPU evaluates the
same formulas in FP32 with fused multiply-adds; the oracle does not fuse."""
import os

import numpy as np
import pytest

from openswpc_gb300 import configs, gpu
from oracle import pyoracle
from tests.helpers import misfit, sim_from_oracle

TOL = 1e-5


@pytest.fixture(scope="module")
def small_inf(tmp_path_factory):
    d = tmp_path_factory.mktemp("plain_small")
    return configs.write_plain_small(str(d), nt=240)


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [0, 1])
def test_fields_after_few_steps(small_inf, variant):
    o = pyoracle.Oracle(small_inf, "fp32")
    s = sim_from_oracle(o, variant=variant)
    # 40 steps: the source (rise time 1 s, dt 0.02 s) is still injecting
    o.run(40)
    s.run(1, 40)
    s.sync()
    for name in pyoracle.FIELDS:
        a, b = s.field(name), o.field(name)
        assert misfit(a, b) < TOL, (name, misfit(a, b))
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [0, 1])
def test_waveforms_match_oracle(small_inf, variant):
    o = pyoracle.Oracle(small_inf, "fp32")
    s = sim_from_oracle(o, variant=variant)
    o.run(240)
    s.run(1, 240)
    w_gpu = s.waveforms()
    w_ref = o.waveforms()
    assert w_gpu.shape == w_ref.shape
    m = misfit(w_gpu, w_ref)
    assert m < TOL, m
    # every station saw signal
    assert np.all(np.abs(w_ref).max(axis=2) > 0)
    s.close()


@pytest.mark.gpu
def test_full_length_small_configuration(tmp_path):
    """The small plain configuration over its whole nt = 1000 steps: receiver
    traces within 1e-5 of the fp32 oracle (the error against the fp64 oracle
    is stated)."""
    inf = configs.write_plain_small(str(tmp_path), nt=1000)
    o = pyoracle.Oracle(inf, "fp32")
    s = sim_from_oracle(o)
    o.run(1000)
    s.run(1, 1000)
    w, w32 = s.waveforms(), o.waveforms()
    s.close()
    o.close()
    o64 = pyoracle.Oracle(inf, "fp64")
    o64.run(1000)
    w64 = o64.waveforms()
    o64.close()
    m32, m64 = misfit(w, w32), misfit(w, w64)
    print("small configuration, 1000 steps: misfit vs fp32 oracle %.3e, vs fp64 oracle %.3e" % (m32, m64))
    assert m32 <= TOL, m32
    assert m64 <= TOL, m64


@pytest.mark.gpu
def test_vmax_matches_oracle(small_inf):
    """max |V| at the ocean bottom every ntdec_r steps (kernel__vmax,
    m_kernel.f90:350-374, as report__progress prints it, m_report.f90:157)
    equals the oracle's."""
    o = pyoracle.Oracle(small_inf, "fp32")
    assert o.ntdec_r > 0
    s = sim_from_oracle(o, ntdec_r=o.ntdec_r)
    nrep = 240 // o.ntdec_r
    got = []
    for q in range(nrep):
        s.run(q * o.ntdec_r + 1, (q + 1) * o.ntdec_r)
        got.append(s.vmax())
    o.run(nrep * o.ntdec_r)
    ref = o.vmax_log()
    s.close()
    assert ref.shape[0] == len(got) == nrep
    assert np.array_equal(ref[:, 0], np.arange(1, len(got) + 1) * o.ntdec_r)
    ref_v = ref[:, 1:].astype(np.float64) * o.UC * o.M0
    got = np.array(got, np.float64)
    assert np.all(ref_v > 0)
    assert misfit(got, ref_v) <= TOL, misfit(got, ref_v)
    assert np.allclose(got, ref_v, rtol=1e-4, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("rows", [(16, 8), (8, 16), (16, 16), (8, 12), (16, 12)])
def test_tile_shapes_give_identical_fields(small_inf, rows):
    """Every tile shape evaluates the same expressions on the same values:
    the fields after 60 steps equal those of the default 8-row tiles bit
    for bit."""
    o = pyoracle.Oracle(small_inf, "fp32")
    a = sim_from_oracle(o)
    b = sim_from_oracle(o)
    b.set_tiles(*rows)
    assert b.tiles() == rows
    a.run(1, 60)
    b.run(1, 60)
    for name in pyoracle.FIELDS:
        assert np.array_equal(a.field(name), b.field(name)), name
    assert np.array_equal(a.waveforms(), b.waveforms())
    a.close()
    b.close()


@pytest.mark.gpu
def test_step_by_step_equals_graph_replay(small_inf):
    o = pyoracle.Oracle(small_inf, "fp32")
    a = sim_from_oracle(o)
    b = sim_from_oracle(o)
    a.run(1, 37)
    for it in range(1, 38):
        b.step(it)
    a.sync(); b.sync()
    for name in ("Vx", "Szz", "Sxy"):
        assert np.array_equal(a.field(name), b.field(name))
    a.close(); b.close()


@pytest.mark.gpu
def test_drop_in_path_matches_golden_traces(tmp_path):
    """input.inf -> host set-up (swpc_host_prepare) -> GPU -> receiver traces,
    against the committed oracle traces: relative L2 <= 1e-5 against the
    fp32 build, and the error against the fp64 build is stated."""
    from tests.golden import make_golden
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "plain_small_nt200.npz"))
    inf = make_golden.write_inputs(str(tmp_path))
    s = gpu.Simulation.from_inf(inf)
    s.run(1, int(g["nt"]))
    s.sync()
    w = s.waveforms()
    s.close()
    m32, m64 = misfit(w, g["fp32"]), misfit(w, g["fp64"])
    print("drop-in path: misfit vs fp32 oracle %.3e, vs fp64 oracle %.3e" % (m32, m64))
    assert m32 <= 1e-5
    assert m64 <= 1e-5


@pytest.mark.gpu
def test_simulations_driven_from_two_threads(tmp_path):
    """One host thread per simulation (each with its own streams): two
    simulations stepped concurrently from two threads give the same traces,
    bit for bit, as the same simulations run one after the other."""
    import threading
    infs = [configs.write_plain_small(str(tmp_path / n), nt=120, nx=n2, ny=n2, nz=48, xbeg=-n2 / 4, ybeg=-n2 / 4)
            for n, n2 in (("a", 96), ("b", 112))]

    def run(inf):
        s = gpu.Simulation.from_inf(inf)
        s.run(1, 120)
        s.sync()
        w = s.waveforms()
        s.close()
        return w

    alone = [run(f) for f in infs]
    out = [None, None]

    def worker(q):
        out[q] = run(infs[q])

    th = [threading.Thread(target=worker, args=(q,)) for q in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for q in range(2):
        assert out[q] is not None and np.array_equal(out[q], alone[q])
