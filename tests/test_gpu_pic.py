"""GPU PIC (fdtdpic_run through the C ABI) against the FP64 CPU oracle's beam model."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

NZ, T, NPART = 512, 600, 20000
DZ = 0.015
DT = 0.5 * DZ / O.C0
CLO, CHI = 40, 480


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _case(precision, sort_every=32, chunk=0, steps=(T,), path="auto"):
    torch = _torch()
    import scipy.constants as sc
    from fdtdpic.grid import lorentz_kerr_grid
    from fdtdpic.pic import PicRun, make_beam
    g = lorentz_kerr_grid(NZ, T, front=300, rear=400, nzsrc=60, probes=(50, 350), chi3=1e-2)
    beam = make_beam(NPART, CLO, CHI, DZ)
    run = PicRun(g, beam, DZ, DT, sc.mu_0, precision=precision, sort_every=sort_every, chunk=chunk,
                 path=path)
    snaps = []
    for s in steps:
        run.step(s)
        torch.cuda.synchronize()
        snaps.append((run.fields(), run.particles(), run.currents()))
    return g, beam, run, snaps


def _oracle(g, beam, n_steps=T):
    import scipy.constants as sc
    P = O.RefParams(Nz=NZ, timeSteps=T, dz=DZ, delT=DT, courantNo=O.f32(0.5),
                    materialFrontEdge=300, materialRearEdge=400, pmlWidth=20, nzsrc=60,
                    freq_in=1e9, permit_0=g.eps0, permea_0=sc.mu_0, nonLinMed=True,
                    FreeSpace=False, plasmaFreqE=np.sqrt(2.0) * 2 * np.pi * 1.5e9,
                    omega_0E=2 * np.pi * 1.5e9, gammaE=2 * np.pi * 0.1e9, chi3Stat=1e-2,
                    sigmaOpt=O.sigma_opt(DZ, g.eps0, sc.mu_0))
    cell, frac = beam.cell.copy(), beam.frac.copy()
    ux, uz = beam.ux.copy(), beam.uz.copy()
    k = O.pic_constants(DZ, DT, beam.weight, sc.mu_0)
    r = O.integrate_pic(P, O.KERR, g.exs, np.zeros(T), cell, frac, ux, uz, k, CLO, CHI,
                        n_steps=n_steps, probe_cells=(50, 350))
    return r, (cell, frac, ux, uz)


def _zeta(cell, frac):
    return cell + frac


@pytest.mark.parametrize("path", ["streaming", "tiled"])
def test_pic_fp64_matches_oracle(path):
    g, beam, run, snaps = _case("f64", path=path)
    f, (cell, frac, ux, uz), (jx, jz) = snaps[-1]
    r, (oc, of, oux, ouz) = _oracle(g, beam)
    assert run.status()[0] == 0 and r["lost"] == 0
    for key, want in (("Ex", r["Ex"]), ("Hy", r["Hy"]), ("Dx", r["Dx"])):
        assert O.rel_l2(f[key], want) <= 1e-12, key
    assert O.rel_l2(run.probes()[:, 1], r["probes"][:, 1]) <= 1e-12
    assert O.rel_l2(jx, r["Jx"]) <= 1e-11
    assert O.rel_l2(jz, r["Jz"]) <= 1e-12
    assert np.array_equal(cell, oc)
    assert np.abs(frac - of).max() <= 1e-12
    assert O.rel_l2(ux, oux) <= 1e-11
    assert O.rel_l2(uz, ouz) <= 1e-14


@pytest.mark.parametrize("path", ["streaming", "tiled"])
def test_pic_fp32_error_vs_fp64_oracle(path):
    g, beam, run, snaps = _case("f32", path=path)
    f, (cell, frac, ux, uz), (jx, jz) = snaps[-1]
    r, (oc, of, oux, ouz) = _oracle(g, beam)
    assert run.status()[0] == 0
    # stated FP32 bounds against the FP64 oracle after 600 coupled steps
    e = dict(Ex=O.rel_l2(f["Ex"], r["Ex"]), Hy=O.rel_l2(f["Hy"], r["Hy"]),
             trace=O.rel_l2(run.probes()[:, 1], r["probes"][:, 1]),
             zeta=float(np.abs(_zeta(cell, frac) - _zeta(oc, of)).max()),
             ux=O.rel_l2(ux, oux), uz=O.rel_l2(uz, ouz))
    print(f"\nbeam FP32 ({path}) vs oracle: " + ", ".join(f"{k} {v:.3e}" for k, v in e.items()))
    assert e["Ex"] <= 1e-5 and e["Hy"] <= 1e-5, e
    assert e["trace"] <= 5e-5, e
    assert e["zeta"] <= 1e-4, e
    assert e["ux"] <= 1e-4, e
    assert e["uz"] <= 1e-6, e


@pytest.mark.parametrize("precision,path", [("f32", "streaming"), ("f64", "streaming"),
                                            ("f32", "tiled"), ("f64", "tiled")])
def test_pic_run_to_run_bit_stable(precision, path):
    _, _, run1, s1 = _case(precision, sort_every=16, path=path)
    _, _, run2, s2 = _case(precision, sort_every=16, path=path)
    for k in ("Ex", "Hy", "Dx"):
        np.testing.assert_array_equal(s1[-1][0][k], s2[-1][0][k])
    for a, b in zip(s1[-1][1], s2[-1][1]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(s1[-1][2][0], s2[-1][2][0])


def test_pic_result_independent_of_binning_and_chunking():
    """Deposits are exact integer sums: re-binning cadence and CTA chunking change nothing."""
    _, _, _, a = _case("f32", sort_every=0, chunk=512, path="streaming")
    _, _, _, b = _case("f32", sort_every=7, chunk=2048, path="streaming")
    np.testing.assert_array_equal(a[-1][0]["Ex"], b[-1][0]["Ex"])
    np.testing.assert_array_equal(a[-1][2][0], b[-1][2][0])
    for x, y in zip(a[-1][1], b[-1][1]):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("path", ["streaming", "tiled"])
def test_pic_resume_in_chunks_equals_one_call(path):
    _, _, _, whole = _case("f64", steps=(T,), path=path)
    _, _, _, parts = _case("f64", steps=(250, 200, 150), path=path)
    for k in ("Ex", "Hy", "Dx"):
        np.testing.assert_array_equal(whole[-1][0][k], parts[-1][0][k])


@pytest.mark.parametrize("path", ["streaming", "tiled"])
def test_pic_gpu_jz_conserves_charge(path):
    g, beam, run, snaps = _case("f64", steps=(T - 1, 1), path=path)
    (_, (c0, f0, _, _), _), (_, (c1, f1, _, _), (jx, jz)) = snaps
    qw = O.Q_E * beam.weight

    def charge(c, f):
        Q = np.zeros(NZ + 1)
        np.add.at(Q, c, qw * (1 - f))
        np.add.at(Q, c + 1, qw * f)
        return Q

    h = np.arange(CLO + 2, CHI - 2)
    resid = (charge(c1, f1)[h] - charge(c0, f0)[h]) / DT + (jz[h] - jz[h - 1]) / DZ
    assert np.abs(resid).max() <= 1e-9 * np.abs(jz).max() / DZ


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_tiled_kernel_equals_streaming_kernels_bitwise(precision):
    """Same arithmetic per cell and per particle, exact integer deposits: identical bits, although
    one path is a single persistent launch with neighbour handshakes and the other three
    launches per step."""
    _, _, r1, a = _case(precision, path="streaming")
    _, _, r2, b = _case(precision, path="tiled")
    assert r1.status()[0] == 0 and r2.status()[0] == 0 and r2.status()[1] == 0
    for k in ("Ex", "Hy", "Dx", "psiE", "psiH", "A"):
        np.testing.assert_array_equal(a[-1][0][k], b[-1][0][k], err_msg=k)
    np.testing.assert_array_equal(a[-1][2][0], b[-1][2][0])
    np.testing.assert_array_equal(a[-1][2][1], b[-1][2][1])
    np.testing.assert_array_equal(r1.probes(), r2.probes())
    for x, y in zip(a[-1][1], b[-1][1]):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("nz,clo,chi", [(512, 40, 480), (1536, 40, 1480)])
def test_push_chunk_changes_no_bits(nz, clo, chi):
    """The FP32 push with the default particles-per-CTA and with 1022 (a ragged split of the
    warps' particles) gives the same bits: fields, currents (Jz deposited on the last step),
    probes and particles, since deposits are integer sums whose grouping does not matter; on
    the 1536-cell grid the push launches carry the previous step's H phase."""
    torch = _torch()
    import scipy.constants as sc
    from fdtdpic.grid import lorentz_kerr_grid
    from fdtdpic.pic import PicRun, make_beam
    out = []
    for chunk in (0, 1022):
        g = lorentz_kerr_grid(nz, T, front=300, rear=400, nzsrc=60, probes=(50, 350), chi3=1e-2)
        beam = make_beam(NPART + 3, clo, chi, DZ)  # a ragged last warp
        run = PicRun(g, beam, DZ, DT, sc.mu_0, precision="f32", chunk=chunk, path="streaming")
        run.step(T)
        torch.cuda.synchronize()
        assert run.status()[0] == 0
        out.append((run.fields(), run.currents(), run.probes(), run.particles()))
    (fa, ja, pa, qa), (fb, jb, pb, qb) = out
    for k in ("Ex", "Hy", "Dx", "A"):
        np.testing.assert_array_equal(fa[k], fb[k], err_msg=k)
    np.testing.assert_array_equal(ja[0], jb[0])
    np.testing.assert_array_equal(ja[1], jb[1])
    np.testing.assert_array_equal(pa, pb)
    for x, y in zip(qa, qb):
        np.testing.assert_array_equal(x, y)
