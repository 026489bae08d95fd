"""The temporally blocked beam path (PicRun path="pass", fdtdpic_run path mode 3): several whole
steps per launch over tiles held in shared memory, against the streaming kernels on the same
run, bit for bit -- fields (every state array), Hy one half step back, currents, probe traces,
particles (by id) and status words -- in FP32 and FP64, on Kerr and Lorentz grids and with a
TF/SF source; a run in several calls equals one call; pass lengths 4, 8 (the default) and 16."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

DZ = 0.015
DT = 0.5 * DZ / O.C0
NZ, T, NPART, CLO, CHI = 6000, 300, 12000, 40, 5959


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _grid(mode, tfsf=False):
    from fdtdpic.grid import MODE_KERR, MODE_LINLOR, lorentz_kerr_grid
    g = lorentz_kerr_grid(NZ, T, front=2500, rear=3500, nzsrc=60, probes=(50, 3200), chi3=1e-2,
                          mode={"kerr": MODE_KERR, "linlor": MODE_LINLOR}[mode])
    if tfsf:
        g.tfsf = True
        g.hys = 0.5 * g.exs
    # move the source next to the slab so the beam and the slab both see the pulse in 300 steps
    g.nzsrc = 2440
    return g


def _run(precision, path, mode="kerr", tfsf=False, steps=(T,), **kw):
    torch = _torch()
    import scipy.constants as sc
    from fdtdpic.pic import PicRun, make_beam
    g = _grid(mode, tfsf)
    beam = make_beam(NPART, CLO, CHI, DZ, v_spread=0.05)
    run = PicRun(g, beam, DZ, DT, sc.mu_0, precision=precision, path=path, **kw)
    for s in steps:
        run.step(s)
    torch.cuda.synchronize()
    jx, jz = run.currents()
    return dict(state=run.d_state.cpu().numpy(), hyp=run.d_hyp.cpu().numpy(), jx=jx, jz=jz,
                probes=run.probes(), parts=run.particles(), status=run.status())


def _equal(got, want):
    assert int(got["status"][0]) == 0 and int(got["status"][1]) == 0, got["status"]
    for k in ("state", "hyp", "jx", "jz", "probes"):
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    for a, b in zip(got["parts"], want["parts"]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("precision,mode,tfsf", [("f32", "kerr", False), ("f64", "kerr", False),
                                                 ("f32", "linlor", False), ("f64", "kerr", True)])
def test_pass_path_equals_streaming_kernels_bitwise(precision, mode, tfsf):
    # FP64 holds twice the bytes a cell and a particle: 256-cell tiles keep the CTA that runs
    # both wrap tiles inside shared memory
    kw = dict(tile_cells=256) if precision == "f64" else {}
    want = _run(precision, "streaming", mode, tfsf)
    got = _run(precision, "pass", mode, tfsf, **kw)
    assert np.abs(want["jx"]).max() > 0  # the beam carries a current by the last step
    _equal(got, want)


@pytest.mark.parametrize("pass_steps", [4, 16])
def test_pass_length_changes_no_bits(pass_steps):
    want = _run("f32", "pass")
    got = _run("f32", "pass", pass_steps=pass_steps)
    _equal(got, want)


def test_pass_path_resumes_across_calls():
    want = _run("f32", "pass")
    got = _run("f32", "pass", steps=(101, 3, 196))
    _equal(got, want)


def test_pass_path_refuses_what_it_cannot_run():
    """A beam outside its domain, or tiles too narrow for the pass's halo: fdtdpic_run refuses
    (FDTDPIC_ERR_ARG) instead of running something else."""
    _torch()
    import scipy.constants as sc
    from fdtdpic._lib import FdtdPicError
    from fdtdpic.pic import PicRun, make_beam
    g = _grid("kerr")
    beam = make_beam(1000, CLO, CHI, DZ)
    beam.cell[0] = CHI + 5  # outside [clo, chi): no FDTDPIC_PATH_CELLS_INSIDE
    run = PicRun(g, beam, DZ, DT, sc.mu_0, precision="f32", path="pass")
    with pytest.raises(FdtdPicError):
        run.step(10)
    run = PicRun(g, make_beam(1000, CLO, CHI, DZ), DZ, DT, sc.mu_0, precision="f32", path="pass",
                 pass_steps=32, tile_cells=128)  # halo 100 cells > half a 128-cell tile
    with pytest.raises(FdtdPicError):
        run.step(10)


def test_pass_path_long_grid_equals_streaming():
    """2^21 cells and 2^23 particles (4 a cell, the large instance's density; 513-cell tiles
    with an odd number of loaded cells): the pass path gives the streaming kernels' bits through
    a call's last step (Jz deposited too)."""
    torch = _torch()
    import scipy.constants as sc
    from fdtdpic.grid import lorentz_kerr_grid
    from fdtdpic.pic import PicRun, make_beam
    nz, steps, npart = 1 << 21, 64, 1 << 23
    out = []
    for path in ("streaming", "pass"):
        g = lorentz_kerr_grid(nz, steps, front=nz // 4, rear=3 * nz // 4, nzsrc=100,
                              probes=(50, nz - 50), chi3=1e-2)
        beam = make_beam(npart, 50, nz - 51, DZ, seed=11, sort=False)
        beam.ux[:] = 0.01  # transverse momentum from the start: every step deposits Jx
        run = PicRun(g, beam, DZ, DT, sc.mu_0, precision="f32", path=path)
        run.step(steps)
        torch.cuda.synchronize()
        jx, jz = run.currents()
        out.append(dict(state=run.d_state.cpu().numpy(), hyp=run.d_hyp.cpu().numpy(), jx=jx,
                        jz=jz, probes=run.probes(), parts=run.particles(), status=run.status()))
        del run
    want, got = out
    assert np.abs(want["jx"]).max() > 0
    _equal(got, want)


@pytest.mark.parametrize("precision,tile", [("f32", 0), ("f64", 256)])
def test_pass_plan_sizes_the_run(precision, tile):
    """The host planner (fdtdpic_pass_plan at GB300's 227 KiB of opt-in shared memory) and a run
    on this device take the same tiling: PicRun(path="pass") sizes the scratch the plan reports."""
    _torch()
    import scipy.constants as sc
    from fdtdpic.pic import PicRun, make_beam, pass_plan
    g = _grid("kerr")
    beam = make_beam(NPART, CLO, CHI, DZ, v_spread=0.05)
    plan = pass_plan(g, beam, precision=precision, tile_cells=tile)
    assert plan is not None
    run = PicRun(g, beam, DZ, DT, sc.mu_0, precision=precision, path="pass", tile_cells=tile)
    assert run.scratch_bytes == plan["scratch_bytes"]
