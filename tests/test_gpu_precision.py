"""Precision form: the 18 memory-variable arrays stored in FP16 or BF16
(arithmetic FP32).  The waveform misfit against the FP32 path and against the
FP64 oracle is measured on the small plain workload.

Tolerances (relative L2 over all receivers, components and samples):
FP16 storage within 1e-3 of the FP32 path, BF16 within 1e-2; both within the
same distance of the FP64 oracle plus the FP32 path's own error."""
import numpy as np
import pytest

from openswpc_gb300 import configs
from oracle import pyoracle
from tests.helpers import misfit, sim_from_oracle

NT = 300


@pytest.fixture(scope="module")
def runs(tmp_path_factory):
    inf = configs.write_plain_small(str(tmp_path_factory.mktemp("prec")), nt=NT)
    o = pyoracle.Oracle(inf, "fp32")
    w = {}
    for store in ("fp32", "fp16", "bf16"):
        s = sim_from_oracle(o, store=store)
        s.run(1, NT)
        w[store] = s.waveforms()
        s.close()
    o64 = pyoracle.Oracle(inf, "fp64")
    o64.run(NT)
    w["fp64"] = o64.waveforms()
    return w


@pytest.mark.gpu
def test_fp16_memory_variables(runs):
    m32 = misfit(runs["fp16"], runs["fp32"])
    m64 = misfit(runs["fp16"], runs["fp64"])
    base = misfit(runs["fp32"], runs["fp64"])
    print("fp16 storage: misfit vs fp32 %.3e, vs fp64 %.3e (fp32 vs fp64 %.3e)" % (m32, m64, base))
    assert m32 < 1e-3
    assert m64 < 1e-3 + base


@pytest.mark.gpu
def test_bf16_memory_variables(runs):
    m32 = misfit(runs["bf16"], runs["fp32"])
    m64 = misfit(runs["bf16"], runs["fp64"])
    base = misfit(runs["fp32"], runs["fp64"])
    print("bf16 storage: misfit vs fp32 %.3e, vs fp64 %.3e (fp32 vs fp64 %.3e)" % (m32, m64, base))
    assert m32 < 1e-2
    assert m64 < 1e-2 + base


@pytest.mark.gpu
@pytest.mark.parametrize("store", ["fp16", "bf16"])
def test_16bit_batch_equals_alone(tmp_path, store):
    """The batched kernels with 16-bit memory variables give each member
    exactly (bit for bit) the traces of the same simulation run alone."""
    from openswpc_gb300 import gpu
    infs = [configs.write_plain_small(str(tmp_path / n), nt=120, nx=n2, ny=n2, nz=48, xbeg=-n2 / 4, ybeg=-n2 / 4)
            for n, n2 in (("a", 96), ("b", 128))]
    orc = [pyoracle.Oracle(f, "fp32") for f in infs]
    alone = []
    for o in orc:
        s = sim_from_oracle(o, store=store)
        s.run(1, 120)
        alone.append(s.waveforms())
        s.close()
    sims = [sim_from_oracle(o, store=store) for o in orc]
    b = gpu.Batch(sims)
    b.run(120)
    b.sync()
    for s, w in zip(sims, alone):
        assert np.array_equal(s.waveforms(), w)
    b.close()
    for s in sims:
        s.close()
