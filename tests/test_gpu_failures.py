"""Failure detection without faulting the GPU: the bounded device wait gives
up and reports, a numerically unstable run is caught by the divergence check
(m_report.f90:142-151) and reported as an error code instead of stopping the
process, and the serving loop isolates a failing request from the others."""
import ctypes

import numpy as np
import pytest

from openswpc_gb300 import configs, gpu

NT = 100


@pytest.mark.gpu
def test_bounded_wait_gives_up_and_device_stays_usable(tmp_path):
    sec = ctypes.c_double()
    rc = gpu.lib().swpc_gpu_selftest_wait(ctypes.byref(sec))
    assert rc == -7, gpu.last_error()  # SWPC_E_TIMEOUT: the wait ran out and said so
    assert 0 < sec.value < 60
    inf = configs.write_plain_small(str(tmp_path), nt=40)
    s = gpu.Simulation.from_inf(inf)
    s.run(1, 40)
    s.sync()
    s.close()


def _unstable(d):
    # dt far above the CFL limit (Vp dt / dx = 2.6): the wavefield grows
    # without bound and the max |V| check at every ntdec_r steps trips
    return configs.write_plain_small(str(d), nt=NT, dt=0.2, ntdec_r=10)


@pytest.mark.gpu
def test_divergence_is_reported_not_fatal(tmp_path):
    s = gpu.Simulation.from_inf(_unstable(tmp_path))
    s.run(1, NT)
    with pytest.raises(gpu.SwpcError) as e:
        s.sync()
    assert e.value.code == -5  # SWPC_E_DIVERGED
    s.close()


@pytest.mark.gpu
def test_serving_isolates_failed_requests(tmp_path):
    good = configs.write_layered(str(tmp_path / "good"), 96, 96, 96, 31, nt=NT, n_station=8, src_depth_max=4.0)
    bad = _unstable(tmp_path / "bad")
    s = gpu.Simulation.from_inf(good)
    s.run(1, NT)
    s.sync()
    alone = s.waveforms()
    s.close()
    with gpu.Server(quantum=20, prep_threads=2) as srv:
        rb, rg = srv.submit(bad), srv.submit(good)
        with pytest.raises(gpu.SwpcError):
            srv.wait(rb, 120.0)
        assert srv.state(rb) == -5
        assert srv.wait(rg, 120.0) == gpu.REQ_DONE
        assert np.array_equal(srv.result(rg), alone)
    # a request larger than the whole budget is refused, the server goes on
    need = gpu.Request(good).device_bytes
    with gpu.Server(hbm_budget=need // 2, prep_threads=1) as srv:
        r = srv.submit(good)
        with pytest.raises(gpu.SwpcError):
            srv.wait(r, 60.0)
        assert srv.state(r) == -3  # SWPC_E_NOMEM
        assert "budget" in srv.error(r)
