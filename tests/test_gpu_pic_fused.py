"""The streaming PIC step whose push launch carries the previous step's H phase
(FDTDPIC_PATH_CELLS_INSIDE) against the same run with separate push, E and H launches: fields,
particles, currents and probes equal bit for bit, in FP32 and FP64, over graph blocks, re-binning
steps and an eager tail, with the source cell inside the beam domain, with TF/SF on (the on-the-fly
H takes the source correction at nzsrc-1) and in the free-space mode (the slab's own H
coefficient).  Grids above 1024 cells: smaller ones take the one-CTA field kernel instead.  The
FP64 fused run also matches the CPU oracle."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

NZ, T, NPART = 2048, 300, 30000
DZ = 0.015
DT = 0.5 * DZ / O.C0
CLO, CHI = 40, 2000
FRONT, REAR, NZSRC = 900, 1100, 60


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _grid(tfsf=False, mode=None):
    from fdtdpic._lib import MODE_KERR
    from fdtdpic.grid import lorentz_kerr_grid
    g = lorentz_kerr_grid(NZ, T, front=FRONT, rear=REAR, nzsrc=NZSRC, probes=(50, 1500),
                          chi3=1e-2, mode=MODE_KERR if mode is None else mode)
    if tfsf:
        g.tfsf = True
        g.hys = 0.5 * g.exs / 376.73
    if mode is not None:
        # a slab with its own coefficients, as epsRe = 2.5, muRe = 1.5 give the free-space
        # integrator (UpExMat / epsRe, UpHyMat / muRe)
        g.ue_slab = g.ue / 2.5
        g.uh_slab = g.uh / 1.5
    return g


def _run(precision, fused, tfsf=False, mode=None, steps=(T,)):
    torch = _torch()
    import scipy.constants as sc
    from fdtdpic.pic import PicRun, make_beam
    g = _grid(tfsf, mode)
    beam = make_beam(NPART, CLO, CHI, DZ)
    run = PicRun(g, beam, DZ, DT, sc.mu_0, precision=precision, sort_every=32)
    if not fused:
        run.pb.path = run.path_mode  # no cells-inside guarantee: separate launches
    else:
        assert run.pb.path & 16
    for s in steps:
        run.step(s)
    torch.cuda.synchronize()
    return g, beam, run


def _path_taken(precision, fused, **kw):
    """The path (FdtdPicTiming.path) a fresh run of this case takes, on a few timed steps."""
    import scipy.constants as sc
    from fdtdpic.pic import FdtdPicTiming, PicRun, make_beam
    run = PicRun(_grid(**kw), make_beam(NPART, CLO, CHI, DZ), DZ, DT, sc.mu_0,
                 precision=precision, sort_every=32)
    if not fused:
        run.pb.path = run.path_mode
    tm = FdtdPicTiming()
    run.step(3, timing=tm)
    return tm.path


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_fused_form_is_taken_only_with_the_guarantee(precision):
    _torch()
    assert _path_taken(precision, True) == 3
    assert _path_taken(precision, False) == 1


def _same(a, b):
    fa, fb = a.fields(), b.fields()
    for k in ("Ex", "Hy", "Dx"):
        np.testing.assert_array_equal(fa[k], fb[k], err_msg=k)
    for x, y in zip(a.particles(), b.particles()):
        np.testing.assert_array_equal(x, y)
    for x, y in zip(a.currents(), b.currents()):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(a.probes(), b.probes())
    assert list(a.status()) == list(b.status())


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_fused_h_equals_separate_launches(precision):
    _, _, a = _run(precision, True)
    _, _, b = _run(precision, False)
    _same(a, b)


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_fused_h_equals_separate_launches_tfsf(precision):
    _, _, a = _run(precision, True, tfsf=True)
    _, _, b = _run(precision, False, tfsf=True)
    assert np.abs(a.fields()["Hy"]).max() > 0
    _same(a, b)


def test_fused_h_equals_separate_launches_free_space():
    from fdtdpic._lib import MODE_FREESPACE
    _, _, a = _run("f32", True, mode=MODE_FREESPACE)
    _, _, b = _run("f32", False, mode=MODE_FREESPACE)
    _same(a, b)


def test_fused_h_resumed_in_pieces_equals_one_call():
    _, _, a = _run("f32", True, steps=(T,))
    _, _, b = _run("f32", True, steps=(97, 64, 139))
    _same(a, b)


def test_fused_h_fp64_matches_oracle():
    import scipy.constants as sc
    g, beam, run = _run("f64", True)
    P = O.RefParams(Nz=NZ, timeSteps=T, dz=DZ, delT=DT, courantNo=O.f32(0.5),
                    materialFrontEdge=FRONT, materialRearEdge=REAR, pmlWidth=20, nzsrc=NZSRC,
                    freq_in=1e9, permit_0=g.eps0, permea_0=sc.mu_0, nonLinMed=True,
                    FreeSpace=False, plasmaFreqE=np.sqrt(2.0) * 2 * np.pi * 1.5e9,
                    omega_0E=2 * np.pi * 1.5e9, gammaE=2 * np.pi * 0.1e9, chi3Stat=1e-2,
                    sigmaOpt=O.sigma_opt(DZ, g.eps0, sc.mu_0))
    cell, frac = beam.cell.copy(), beam.frac.copy()
    ux, uz = beam.ux.copy(), beam.uz.copy()
    k = O.pic_constants(DZ, DT, beam.weight, sc.mu_0)
    r = O.integrate_pic(P, O.KERR, g.exs, np.zeros(T), cell, frac, ux, uz, k, CLO, CHI,
                        probe_cells=(50, 1500))
    f = run.fields()
    gc, gf, gux, guz = run.particles()[:4]
    assert run.status()[0] == 0 and r["lost"] == 0
    for key in ("Ex", "Hy", "Dx"):
        assert O.rel_l2(f[key], r[key]) <= 1e-12, key
    assert O.rel_l2(run.probes()[:, 1], r["probes"][:, 1]) <= 1e-12
    assert np.array_equal(gc, cell)
    assert np.abs(gf - frac).max() <= 1e-12
    assert O.rel_l2(guz, uz) <= 1e-14
