"""Set-up on the device (fdtdpic_setup_batch) against the host restatement of the reference's
set-up: the coefficient fields and PML tables agree to the last few places (the kernel's pow,
exp and hypot may round differently from the host library's in the last place), for the sweep's
batch and for CPML configurations the sweep does not use (kappaMax > 1, other grading powers,
one-sided and absent CPML, grids narrower than two PML widths, the free-space slab); and a sweep
set up on the device gives the host-set-up sweep's probe traces and |R(f)|."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COEF = ["ue", "ue_slab", "uh", "uh_slab", "dtdz", "eps0", "sc", "pol_a", "pol_b", "pol_c",
        "kerr_a", "kerr_b", "kerr_c", "nl_e0", "nl_e0chi"]


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _close(a, b, rel=1e-14):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = np.maximum(np.abs(a), np.abs(b))
    bad = np.abs(a - b) > rel * np.where(scale > 0, scale, 1.0)
    assert not bad.any(), (np.flatnonzero(bad)[:5], a[bad][:5], b[bad][:5])


def test_sweep_batch_matches_host_setup():
    _torch()
    from fdtdpic import device_setup as ds, sweep
    from fdtdpic.grid import pack
    spec = sweep.SweepSpec(n_inst=96, n_steps=1024)
    packed, dt = ds.sweep_batch(spec, "f32")
    grids, _ = sweep.make_sweep_grids(spec)
    pk = pack(grids, 4)
    for f in COEF:
        _close(packed.desc_host[f], pk["desc"][f])
    _close(packed.d_table.cpu().numpy()[:pk["table"].size], pk["table"])


@pytest.mark.parametrize("case", [
    dict(nz=500, pml=20, lo=1, hi=1, kappa_max=3.0, r_scale=3.0, r_a_scale=2.0),
    dict(nz=500, pml=25, lo=1, hi=0, kappa_max=2.0),
    dict(nz=500, pml=25, lo=0, hi=1, kappa_max=2.0),
    dict(nz=500, pml=10, lo=0, hi=0),
    dict(nz=30, pml=20, lo=1, hi=1, kappa_max=3.0),
    dict(nz=30, pml=20, lo=0, hi=1, kappa_max=3.0),
    dict(nz=400, pml=16, lo=1, hi=1, free_space=True, eps_re=4.0, mu_re=1.5),
])
def test_setup_kernel_matches_host_tables(case):
    torch = _torch()
    from types import SimpleNamespace

    import scipy.constants as sc

    from fdtdpic import _lib, device_setup as ds, physics_setup as ps
    nz, pml = case["nz"], case["pml"]
    dz, courant = 0.015, ps.f32(0.5)
    dt = 0.5 * dz / ps.C0
    eps0, mu0 = sc.epsilon_0, sc.mu_0
    kappa_max = case.get("kappa_max", 1.0)
    r_scale, r_a_scale = case.get("r_scale", 4.0), case.get("r_a_scale", 1.0)
    free = case.get("free_space", False)
    eps_re, mu_re = case.get("eps_re", 1.0), case.get("mu_re", 1.0)
    w0 = 2 * np.pi * 1.5e9
    pf = np.float64(np.sqrt(2.0) * w0)
    P = SimpleNamespace(Nz=nz, pmlWidth=pml, CPMLXm=bool(case["lo"]), CPMLXp=bool(case["hi"]),
                        delT=dt, permit_0=eps0, permea_0=mu0, dz=dz, kappaMax=kappa_max,
                        r_scale=r_scale, r_a_scale=r_a_scale, sigmaOpt=ps.sigma_opt(dz, eps0, mu0),
                        alphaMax=ps.f32(0.05), CharImp=ps.CHAR_IMP, courantNo=courant,
                        epsRe=eps_re, muRe=mu_re, freq_in=1e9)
    V = SimpleNamespace(omega_0E=w0, gammaE=2 * np.pi * 0.1e9, chi3Stat=1e-2, alpha3=ps.f32(0.7))
    ue, ue_s, uh, uh_s = ps.update_coefficients(P, free)
    table = ps.pml_table(P, ps.cpml_arrays(P, ue))
    kerr = ps.kerr_coefficients(P, V, pf)
    pol = ps.lorentz_coefficients(P, V, pf)

    desc = np.zeros(1, _lib.INSTANCE_DTYPE)
    desc["nz"], desc["pml"], desc["cpml_lo"], desc["cpml_hi"] = nz, pml, case["lo"], case["hi"]
    rec = ds.setup_records(1, dz=dz, dt=dt, courant=courant, eps0=eps0, mu0=mu0, plasma_freq=pf,
                           omega0=w0, gamma=V.gammaE, chi3=V.chi3Stat, freq_in=1e9,
                           kappa_max=kappa_max, r_scale=r_scale, r_a_scale=r_a_scale,
                           eps_re=eps_re, mu_re=mu_re, free_space=free)
    d_desc, d_tab = ds.run_setup(desc, rec)
    torch.cuda.synchronize()
    got = d_desc.cpu().numpy().view(_lib.INSTANCE_DTYPE)[0]
    _close(d_tab.cpu().numpy()[:table.size].reshape(table.shape), table)
    _close([got["ue"], got["ue_slab"], got["uh"], got["uh_slab"]], [ue, ue_s, uh, uh_s])
    _close([got["kerr_a"], got["kerr_b"], got["kerr_c"], got["nl_e0"], got["nl_e0chi"]], kerr)
    _close([got["pol_a"], got["pol_b"], got["pol_c"]], pol)
    _close([got["dtdz"], got["eps0"], got["sc"]], [dt / dz, eps0, courant])


def test_sweep_set_up_on_device_runs_as_host_set_up():
    _torch()
    from fdtdpic import sweep
    spec = sweep.SweepSpec(n_inst=48, n_steps=768)
    a = sweep.Sweep.from_spec(spec, "f32", device_setup=True)
    b = sweep.Sweep.from_spec(spec, "f32", device_setup=False)
    a.run()
    b.run()
    pa, pb = a.probes(), b.probes()
    scale = np.abs(pb).max(axis=(1, 2), keepdims=True)
    assert np.abs(pa - pb).max() <= 1e-6 * scale.max()
    ra, rb = a.reflection(), b.reflection()
    np.testing.assert_allclose(ra, rb, rtol=1e-5, atol=1e-9)
    assert a.cell_steps() == b.cell_steps()
