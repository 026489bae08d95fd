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
    import scipy.constants as sc
    from fdtdpic.grid import lorentz_kerr_grid
    from fdtdpic.pic import PicRun, make_beam
    nz, npart = 1 << 24, 64 << 20
    g = lorentz_kerr_grid(nz, 20000, front=nz // 4, rear=3 * nz // 4, nzsrc=100,
                          probes=(50, nz - 50), chi3=1e-2)
    beam = make_beam(npart, 50, nz - 51, DZ, seed=7, sort=False)
    run = PicRun(g, beam, DZ, 0.5 * DZ / 299792458.0, sc.mu_0, precision="f32")
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
