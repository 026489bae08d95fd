"""The single large instance at full size (2^24 cells, 64M macroparticles, Kerr slab over the
middle half, FP32): properties that do not depend on size -- particles stay on the grid and
inside the periodic beam domain, fields stay finite, and two runs are bit-identical (exact
integer deposits make the result independent of atomic and scheduling order)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DZ = 0.015


def _run(steps):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fdtdpic.pic import large_case
    run = large_case(1 << 24, 64 << 20, 20000, dz=DZ, nzsrc=100)
    run.step(steps)
    torch.cuda.synchronize()
    return run


def test_large_instance_properties_and_bit_stability():
    import torch
    steps = 40  # crosses a re-binning (every 32 steps)
    runs = []
    for _ in range(2):
        run = _run(steps)
        st = run.status()
        assert int(st[0]) == 0 and int(st[1]) == 0
        cell = run.d_cell.cpu().numpy()
        frac = run.d_frac.float().cpu().numpy()
        assert cell.min() >= 50 and cell.max() < (1 << 24) - 51
        assert frac.min() >= 0.0 and frac.max() < 1.0
        ex = run.d_state[: (1 << 24) + 1].float()
        assert bool(torch.isfinite(ex).all())
        jx, _ = run.currents()
        assert np.isfinite(jx).all() and np.abs(jx).max() > 0
        runs.append((run.d_state.clone(), run.d_jx.clone(), run.probes().copy(),
                     run.particles()))
        del run
        torch.cuda.empty_cache()
    (s0, j0, p0, q0), (s1, j1, p1, q1) = runs
    assert torch.equal(s0, s1) and torch.equal(j0, j1)
    np.testing.assert_array_equal(p0, p1)
    for a, b in zip(q0, q1):
        np.testing.assert_array_equal(a, b)
