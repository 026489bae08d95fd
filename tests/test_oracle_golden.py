"""The CPU oracle against outputs of the reference itself (tests/golden/*.npz).

The fixtures were produced by ``tests/golden/make_golden.py``, which runs the reference's own
integrators (Solver_Engine.py:142-371) with inert stand-ins for its missing imports.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
               if os.path.basename(p) not in ("cubic_solve.npz", "setup.npz", "variants.npz",
                                              "stepops.npz"))

# FP64 end-state fields and probe traces: the reference itself, to rounding.
FIELD_TOL = 1e-12
# Acubic is a difference of two numbers ~b/(3a) far larger than the root (the reference's own
# closed form); its last digits are cancellation noise, so it gets a looser bound.
ACUBIC_TOL = 1e-6


def _run(path):
    g = np.load(path)
    P = O.params_from_golden(g)
    user = bool(g["source_supplied"])
    extra = tuple(int(k.split("_")[1]) for k in g.files if k.startswith("probe_"))
    r = O.integrate(P, Exs=g["Exs"] if user else None, Hys=g["Hys"] if user else None,
                    extra_probes=extra)
    return g, r, extra


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p) for p in CASES])
def test_oracle_matches_reference_run(path):
    g, r, extra = _run(path)
    for k in ("Ex", "Hy", "psi_Ex", "psi_Hy", "Dx", "polarisationCurr", "Port1", "Port2",
              "x1ColBe", "x1ColAf", "Exs", "Hys"):
        assert O.rel_l2(getattr(r, k), g[k]) <= FIELD_TOL, k
    assert O.rel_l2(r.Acubic, g["Acubic"]) <= ACUBIC_TOL
    if "Ex_History" in g:
        assert O.rel_l2(r.Ex_History, g["Ex_History"]) <= FIELD_TOL
    for j, c in enumerate(extra):
        assert O.rel_l2(r.probes[:, j], g[f"probe_{c}"]) <= FIELD_TOL
    for k in ("beX", "ceX", "bmY", "cmY", "Cb", "C2", "den_Exdz", "den_Hydz"):
        assert O.rel_l2(r.coef[k], g[k]) <= 1e-15, k
    assert abs(r.plasmaFreqE - float(g["plasmaFreqE_out"])) <= 1e-14 * float(g["plasmaFreqE_out"])


def test_cpml_quirks_visible_in_golden():
    g = np.load(os.path.join(GOLDEN, "kerr_nz1000.npz"))
    nz, pml = int(g["P_Nz"]), int(g["P_pmlWidth"])
    # Cb and C2 stay zero at Nz+1-pml (BaseFDTD11.py:312,326)
    assert g["Cb"][nz + 1 - pml] == 0.0 and g["C2"][nz + 1 - pml] == 0.0
    assert g["Cb"][nz + 2 - pml] != 0.0
    # Hy recursion coefficients alias the Ex ones (BaseFDTD11.py:266-268)
    np.testing.assert_array_equal(g["bmY"], g["beX"])


def test_cubic_known_answers():
    g = np.load(os.path.join(GOLDEN, "cubic_solve.npz"))
    for co, re, im, n, cplx in zip(g["coeffs"], g["roots_re"], g["roots_im"], g["n_roots"],
                                   g["complex_input"]):
        want = (re + 1j * im)[:n]
        for got in (O.cubic_solve(*co), O.cubic_solve_py(*[float(x) for x in co])):
            assert len(got) == n
            scale = max(1.0, float(np.max(np.abs(want))))
            # real-typed inputs reproduce the reference bit for bit up to libm; complex-typed
            # inputs (as Nonlin_Cubic_Solver passes them) differ by a few ulp in the powers
            tol = 1e-13 if cplx else 1e-15
            # the near-triple root (1,-3,3,-1+1e-12) is ill-conditioned: cube-root sensitivity
            if abs(co[3] + 1 - 1e-12) < 1e-15 and co[0] == 1:
                tol = 1e-4
            np.testing.assert_allclose(got, want, rtol=0, atol=tol * scale)


def test_named_cubic_answers():
    assert np.allclose(O.cubic_solve(1, -6, 11, -6), [3, 1, 2])
    assert np.allclose(O.cubic_solve(1, -3, 3, -1), [1, 1, 1])
    assert np.allclose(O.cubic_solve(0, 0, 2, -4), [2])
    assert np.allclose(O.cubic_solve(0, 1, 0, -4), [2, -2])
    r = O.cubic_solve(2, 0, 0, -16)
    assert np.allclose(r, [2, -1 + 1.7320508075688772j, -1 - 1.7320508075688772j])
    assert abs(O.cubic_solve(4.9e-7, 2e-3, 4, -1)[0] - 0.249968756) < 1e-9


def test_benchmark_cubic_of_the_reference():
    """The Kerr-type cubic the reference times in benchmarkTests.py (-81 x^3 + 4 x^2 + 2e-5 x +
    2e-16, solved there with np.roots, taking the first real root >= 0): roots[0] of the
    restated closed form is that root."""
    co = (-81.0, 4.0, 2e-5, 2e-16)
    want = next(x for x in np.roots(co) if x >= 0 and np.imag(x) == 0).real
    for got in (complex(O.cubic_solve(*co)[0]), complex(O.cubic_solve_py(*co)[0])):
        assert got.imag == 0.0
        assert abs(got.real - want) <= 1e-15 * want, (got, want)


def test_env_and_mat_setup_match_reference():
    g = np.load(os.path.join(GOLDEN, "setup.npz"))
    for args, want in zip(g["env_in"], g["env_out"]):
        f, dom, lo, hi, nl = args
        got = O.env_setup(f, dom, int(lo), int(hi), nonLinMed=bool(nl))
        np.testing.assert_allclose(np.array(got, float), want, rtol=1e-15, atol=0)
    for args, want in zip(g["mat_in"], g["mat_out"]):
        got = O.mat_setup(args[0], args[1], int(args[2]), int(args[3]))
        np.testing.assert_allclose(np.array(got, float), want, rtol=1e-15, atol=0)
    for args, want in zip(g["stab_in"], g["stab_out"]):
        got = O.spatial_stab(*[a.item() for a in args])
        np.testing.assert_allclose(np.real(np.array(got, complex)), want, rtol=1e-14, atol=0)


def test_env_setup_reference_default_geometry():
    # __Main__'s call (MasterController.py:636): Nz=11555, T=19250, pml=2100
    r = O.env_setup(9e9, 0.7, 7000, 8000, nonLinMed=True)
    assert (r[0], r[1], r[12]) == (11555, 19250, 2100)
    assert abs(r[15] - 9.5172e-5) < 1e-8 and abs(r[16] - 3.0159e-13) < 1e-16
