"""GPU parity: the sm_103a kernels through the C ABI against the reference's own outputs
(tests/golden) and the FP64 CPU oracle."""
import numpy as np
import pytest

from helpers import RUN_CASES, acubic_bound, integrator_of, load, ref_objects, sources_of

from oracle import oracle as O

pytestmark = pytest.mark.gpu

# FP64 parity bound (relative L2), as the reference's precision allows
F64_TOL = 1e-12


def _engine():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fdtdpic import engine
    return engine


def _run_golden(name, precision="f64", force_global=False):
    engine = _engine()
    from fdtdpic.grid import grids_from_reference
    g = load(name)
    P, V, C_P = ref_objects(g)
    grids = grids_from_reference(P, V, C_P, integrator_of(g), *sources_of(g))
    p = engine.upload(grids, precision)
    if force_global:
        p.global_idx, p.resident = list(range(len(grids))), []
    engine.launch(p)
    import torch
    torch.cuda.synchronize()
    return g, grids, engine.download(p)


def _compare(g, grids, res, tol):
    last = res[-1]
    integ = integrator_of(g)
    assert O.rel_l2(last.Ex, g["Ex"]) <= tol
    assert O.rel_l2(last.Hy, g["Hy"]) <= tol
    assert O.rel_l2(last.psi_Ex, g["psi_Ex"]) <= tol
    assert O.rel_l2(last.psi_Hy, g["psi_Hy"]) <= tol
    assert O.rel_l2(last.Dx, g["Dx"]) <= max(tol, 1e-11)
    assert O.rel_l2(last.P, g["polarisationCurr"]) <= tol
    if integ == "IntegratorNL1D":
        assert O.rel_l2(last.probes[:, 0], g["Port1"]) <= tol
        assert O.rel_l2(last.probes[:, 1], g["Port2"]) <= tol
        # per cell: the closed form's conditioning and the run's Dx difference (helpers)
        bound = acubic_bound(g["Acubic"], grids[-1].kerr)
        assert np.all(np.abs(last.Acubic - g["Acubic"]) <= bound)
    elif integ == "IntegratorLinLor1D":
        assert O.rel_l2(res[0].probes[:, 0], g["x1ColBe"]) <= tol
        assert O.rel_l2(res[1].probes[:, 1], g["x1ColAf"]) <= tol
    else:
        assert O.rel_l2(last.probes[:, 0], g["x1ColBe"]) <= tol
        assert O.rel_l2(last.probes[:, 1], g["x1ColAf"]) <= tol
    if "Ex_History" in g.files and last.hist is not None:
        assert O.rel_l2(last.hist, g["Ex_History"]) <= tol
    for r in res:
        assert r.status == 0


@pytest.mark.parametrize("name", RUN_CASES)
def test_fp64_resident_matches_reference(name):
    g, grids, res = _run_golden(name)
    _compare(g, grids, res, F64_TOL)


@pytest.mark.parametrize("name", ["kerr_sinecont_tfsf", "lorentz_sinecont_tfsf",
                                  "freespace_gauss_tfsf", "kerr_kappa3"])
def test_fp64_global_path_matches_reference(name):
    g, grids, res = _run_golden(name, force_global=True)
    _compare(g, grids, res, F64_TOL)


def test_fp64_matches_oracle_bitwise_close():
    """Same inputs to the GPU and the oracle: differences only from libm vs CUDA ulps."""
    g, grids, res = _run_golden("kerr_nz1000")
    P = O.params_from_golden(g)
    r = O.integrate(P, Exs=g["Exs"], Hys=g["Hys"])
    assert O.rel_l2(res[0].Ex, r.Ex) <= 1e-13
    assert O.rel_l2(res[0].probes[:, 1], r.Port2) <= 1e-13


def test_batch_equals_alone_and_is_deterministic():
    engine = _engine()
    from fdtdpic.grid import grids_from_reference
    grids, alone = [], []
    for name in RUN_CASES:
        g = load(name)
        P, V, C_P = ref_objects(g)
        gg = grids_from_reference(P, V, C_P, integrator_of(g), *sources_of(g))
        grids += gg
    for prec in ("f64", "f32"):
        mixed = engine.run(grids, prec)
        again = engine.run(grids, prec)
        for i, gr in enumerate(grids):
            one = engine.run([gr], prec)[0]
            for a, b, c in ((mixed[i].Ex, one.Ex, again[i].Ex), (mixed[i].Hy, one.Hy, again[i].Hy),
                            (mixed[i].probes, one.probes, again[i].probes)):
                np.testing.assert_array_equal(a, b)
                np.testing.assert_array_equal(a, c)


def test_fp32_error_vs_fp64_oracle():
    """FP32 state (FP64 only for near-degenerate cubics) against the reference's FP64 outputs
    over 4096 steps.  Kerr: 1e-5 relative L2 on the final fields.  Lorentz (two passes, the
    second with the polarisation on): 2e-5, because its E = (Dx - P)/eps0 subtracts two values
    about (1 + d_eps) = 3 and d_eps = 2 times E, so FP32 rounding of Dx and P reaches E three
    times larger.  Probe traces 5e-5."""
    for name, bound in (("kerr_nz1000", 1e-5), ("lorentz_nz1000", 2e-5)):
        g, grids, res = _run_golden(name, "f32")
        last = res[-1]
        want = g["Port2"] if name.startswith("kerr") else g["x1ColAf"]
        e = dict(Ex=O.rel_l2(last.Ex, g["Ex"]), Hy=O.rel_l2(last.Hy, g["Hy"]),
                 trace=O.rel_l2(last.probes[:, 1], want))
        print(f"\n{name} FP32 vs reference: " + ", ".join(f"{k} {v:.3e}" for k, v in e.items()))
        assert e["Ex"] <= bound and e["Hy"] <= bound, (name, e)
        assert e["trace"] <= 5e-5, (name, e)


def test_cubic_root0_on_gpu_matches_reference_answers():
    engine = _engine()
    g = load("cubic_solve")
    co = g["coeffs"][~g["complex_input"]]
    want = g["roots_re"][~g["complex_input"]][:, 0]
    got = engine.cubic_root0(co)
    # the closed form returns x1 = 2 j cos(k/3) - b/(3a): its absolute error scales with the
    # size of the terms it cancels, not with the root itself
    with np.errstate(divide="ignore", invalid="ignore"):
        shift = np.where(co[:, 0] != 0, np.abs(co[:, 1] / (3 * co[:, 0])), 0.0)
    scale = np.maximum.reduce([np.ones_like(want), np.abs(want), shift])
    # the near-triple root case is ill-conditioned in any implementation
    ok = np.abs(got - want) <= 1e-12 * scale
    ill = np.isclose(co[:, 3], -1 + 1e-12, atol=1e-16, rtol=0)
    assert np.all(ok | ill)
