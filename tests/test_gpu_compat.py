"""The drop-in modules (fdtdpic.compat) on the GPU against the reference's own outputs
(tests/golden), and the batched sweep against one-at-a-time runs."""
import numpy as np
import pytest

from helpers import RUN_CASES, acubic_bound, compat_objects, integrator_of, load

from oracle import oracle as O

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12


def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _controller(g, monkeypatch):
    from fdtdpic.compat import MasterController as MC
    from fdtdpic.compat import Solver_Engine as SE
    V, P, C_V, C_P = compat_objects(g)
    if bool(g["source_supplied"]):
        monkeypatch.setattr(SE, "SourceManager",
                            lambda V_, P_, C_V_, C_P_: (g["Exs"].copy(), g["Hys"].copy()))
    return MC.Controller(V, P, C_V, C_P)


@pytest.mark.parametrize("name", RUN_CASES)
def test_controller_matches_reference(name, monkeypatch):
    _cuda()
    g = load(name)
    V, P, C_V, C_P, Exs, Hys = _controller(g, monkeypatch)
    for got, key in ((V.Ex, "Ex"), (V.Hy, "Hy"), (C_V.psi_Ex, "psi_Ex"), (C_V.psi_Hy, "psi_Hy"),
                     (V.x1ColBe, "x1ColBe"), (V.x1ColAf, "x1ColAf"), (V.Port1, "Port1"),
                     (V.Port2, "Port2"), (V.polarisationCurr, "polarisationCurr")):
        assert O.rel_l2(got, g[key]) <= F64_TOL, key
    assert O.rel_l2(V.Dx, g["Dx"]) <= 1e-11
    if integrator_of(g) == "IntegratorNL1D":
        # per cell: the closed form's conditioning and the run's Dx difference (helpers)
        from fdtdpic import physics_setup as ps
        bound = acubic_bound(g["Acubic"], ps.kerr_coefficients(P, V, V.plasmaFreqE))
        assert np.all(np.abs(np.asarray(V.Acubic) - g["Acubic"]) <= bound)
    if "Ex_History" in g.files:
        assert V.Ex_History.shape == g["Ex_History"].shape
        assert O.rel_l2(V.Ex_History, g["Ex_History"]) <= F64_TOL
    np.testing.assert_allclose(np.asarray(Exs, float), g["Exs"], rtol=1e-13, atol=1e-300)
    assert V.plasmaFreqE == pytest.approx(float(g["plasmaFreqE_out"]), rel=1e-14)


@pytest.mark.parametrize("name", ["lorentz_nz1000", "lorentz_sinecont_tfsf"])
def test_results_refco_matches_fft_peak_ratio(name, monkeypatch):
    from fdtdpic.compat import MasterController as MC
    from fdtdpic.compat import TransformHandler as TH
    _cuda()
    g = load(name)
    V, P, C_V, C_P, _, _ = _controller(g, monkeypatch)
    R = MC.results(V, P, C_V, C_P, None, RefCo=True)

    def peak(y):
        Y = 2 * np.abs(np.fft.fft(y)) / P.timeSteps
        return Y[np.argmax(Y)]
    want = peak(g["x1ColAf"]) / peak(g["x1ColBe"])
    assert R == pytest.approx(want, rel=1e-6)
    bob, fr, val = TH.RefTester(V, P, g["x1ColAf"], 1)
    N = len(g["x1ColAf"])
    Y = np.abs(np.fft.fft(g["x1ColAf"]))
    np.testing.assert_allclose(bob, (Y[N // 2 + 10:N - 500] * 2) / N, rtol=1e-5,
                               atol=1e-6 * Y.max() / N)
    np.testing.assert_allclose(fr, np.fft.fftfreq(N, P.delT)[N // 2 + 10:N - 500])


def test_looped_sim_batch_equals_one_at_a_time():
    """LoopedSim(loop=True) steps its 20 points in one batched launch; the same points run one
    Controller call at a time, in the reference's loop order, give identical results."""
    _cuda()
    from fdtdpic.compat import Environment_Setup as envDef
    from fdtdpic.compat import MasterController as MC
    dom, lo, hi, f0, step = 0.2, 400, 600, 3e9, 1e8

    def start():
        P = MC.Params(*envDef.envSetup(f0, dom, lo, hi), False, dom, f0, 20, LorentzMed=True,
                      SineCont=True, TFSF=True)
        V = MC.Variables(P.Nz, P.timeSteps, P.vidInterval, 1)
        return V, P, MC.CPML_Variables(P.Nz, P.timeSteps), MC.CPML_Params(P.dz)

    V, P, C_V, C_P = start()
    rng, ref_b, anal_b = MC.LoopedSim(None, V, P, C_V, C_P, False, dom, lo, hi, loop=True,
                                      Low=f0, Interval=step)
    V, P, C_V, C_P = start()
    ref_s, anal_s = np.zeros(20), np.zeros(20)
    for i in range(20):
        setup = envDef.envSetup(P.freq_in, dom, lo, hi, VExists=True, V=V, P=P)
        P = MC.Params(*setup, P.MORmode, dom, P.freq_in, 20, LorentzMed=True, SineCont=True,
                      TFSF=True)
        V = MC.Variables(P.Nz, P.timeSteps, P.vidInterval, 1)
        C_P, C_V = MC.CPML_Params(P.dz), MC.CPML_Variables(P.Nz, P.timeSteps)
        V, P, C_V, C_P, _, _ = MC.Controller(V, P, C_V, C_P)
        t = np.arange(len(V.x1ColBe)) * P.delT
        ref_s[i] = MC.results(V, P, C_V, C_P, t, RefCo=True)
        anal_s[i] = MC.results(V, P, C_V, C_P, t, AnalRefCo=True)
        P.freq_in = P.freq_in + step
    np.testing.assert_array_equal(ref_b, ref_s)
    np.testing.assert_array_equal(anal_b, anal_s)
    assert np.all(np.isfinite(ref_b)) and np.all(ref_b > 0)
    np.testing.assert_allclose(rng, f0 + step * np.arange(20))
