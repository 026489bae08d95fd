"""fdtdpic.compat on the host: the state classes' declared types, the set-up each integrator
call performs before any GPU work (coefficient arrays, plasma-frequency rescale, sources,
grids), and the reference's error behaviour."""
import numpy as np
import pytest

from helpers import RUN_CASES, compat_objects, integrator_of, load


def test_state_classes_keep_declared_types():
    from fdtdpic.compat import MasterController as MC
    from fdtdpic.compat import Environment_Setup as envDef
    setup = envDef.envSetup(9e9, 0.7, 7000, 8000, nonLinMed=True)
    P = MC.Params(*setup, False, 0.7, 9e9, 20, LorentzMed=True)
    assert (P.Nz, P.timeSteps, P.pmlWidth) == (11555, 19250, 2100)
    assert P.courantNo == float(np.float32(0.95)) and P.courantNo != 0.95
    assert isinstance(P.Nz, int) and isinstance(P.timeSteps, int)
    assert P.FreeSpace and P.CPMLXp and P.vidInterval == 50
    V = MC.Variables(P.Nz, P.timeSteps, P.vidInterval, 1)
    assert V.alpha3 == float(np.float32(0.7))
    assert V.Ex_History.shape == (int(P.timeSteps / 50), P.Nz + 1)
    assert V.cubPoly.dtype == np.complex128 and V.cubPoly.shape == (P.Nz + 1, 4)
    C_P = MC.CPML_Params(P.dz)
    assert C_P.alphaMax == float(np.float32(0.05)) and C_P.r_scale == 4.0
    assert C_P.sigmaOpt == C_P.sigmaEMax == C_P.sigmaHMax
    C_V = MC.CPML_Variables(P.Nz, P.timeSteps)
    assert C_V.psi_Ex.shape == (P.Nz + 1,) and C_V.psi_Ex_Old.shape == (P.timeSteps,)


@pytest.mark.parametrize("name", RUN_CASES)
def test_prepare_matches_reference_setup(name, monkeypatch):
    from fdtdpic.compat import Solver_Engine as SE
    g = load(name)
    V, P, C_V, C_P = compat_objects(g)
    if bool(g["source_supplied"]):
        monkeypatch.setattr(SE, "SourceManager",
                            lambda V_, P_, C_V_, C_P_: (g["Exs"].copy(), g["Hys"].copy()))
    T = P.timeSteps
    job = SE.prepare(integrator_of(g), V, P, C_V, C_P, int(T * 0.7), int(T * 0.05))
    assert V.plasmaFreqE == pytest.approx(float(g["plasmaFreqE_out"]), rel=1e-14)
    for k in ("beX", "ceX", "bmY", "cmY", "Cb", "C2", "den_Exdz", "den_Hydz"):
        np.testing.assert_allclose(getattr(C_V, k), g[k], rtol=1e-13, atol=0, err_msg=k)
    np.testing.assert_allclose(np.asarray(job.Exs, float), g["Exs"], rtol=1e-13, atol=1e-300)
    n_grids = 2 if integrator_of(g) == "IntegratorLinLor1D" else 1
    assert len(job.grids) == n_grids
    assert job.grids[-1].hist_rows == V.Ex_History.shape[0]


def test_missing_source_fails_like_the_reference():
    from fdtdpic.compat import Solver_Engine as SE
    g = load("kerr_nz1000")
    V, P, C_V, C_P = compat_objects(g)  # neither SineCont nor Gaussian: SourceManager -> []
    with pytest.raises(IndexError):
        SE.prepare("IntegratorNL1D", V, P, C_V, C_P, 10, 1)


def test_field_init_checks_exit_like_the_reference():
    from fdtdpic.compat import BaseFDTD11
    from types import SimpleNamespace
    V = SimpleNamespace()
    with pytest.raises(SystemExit):
        BaseFDTD11.FieldInit(V, SimpleNamespace(Nz=25001, timeSteps=10))
    with pytest.raises(SystemExit):
        BaseFDTD11.FieldInit(V, SimpleNamespace(Nz=100, timeSteps=0))
    with pytest.raises(TypeError):
        BaseFDTD11.FieldInit(V, SimpleNamespace(Nz=100.0, timeSteps=10))
    BaseFDTD11.FieldInit(V, SimpleNamespace(Nz=100, timeSteps=10))
    assert V.Ex.shape == (101,) and not V.Ex.any()


def test_analytical_reflection_is_fresnel():
    from fdtdpic.compat import BaseFDTD11
    from types import SimpleNamespace
    w0 = 2 * np.pi * 20e9
    V = SimpleNamespace(plasmaFreqE=np.sqrt(1.5) * w0, omega_0E=w0, gammaE=0.1 * w0)
    P = SimpleNamespace(freq_in=9e9)
    w = 2 * np.pi * 9e9
    eps = 1 + V.plasmaFreqE ** 2 / (w0 ** 2 - w ** 2 + 1j * V.gammaE * w)
    n2 = np.sqrt(eps).real
    assert BaseFDTD11.AnalyticalReflectionE(V, P) == pytest.approx(abs((n2 - 1) / (n2 + 1)))
