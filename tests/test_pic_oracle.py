"""The beam model's own checks, on the CPU oracle (no GPU): analytic Boris orbits and exact
discrete charge conservation of the Jz deposit."""
import numpy as np

from oracle import oracle as O


def _step(cell, frac, ux, uz, Ex, Hy, Hyp, scal, nz):
    Jx, Jz = np.zeros(nz + 1), np.zeros(nz + 1)
    lost = O.lib().or_pic_step(len(cell), O._p(cell), O._p(frac), O._p(ux), O._p(uz), O._p(Ex),
                               O._p(Hy), O._p(Hyp), O._p(Jx), O._p(Jz), nz, O._p(scal), 1)
    return Jx, Jz, lost


def test_boris_gyration_in_uniform_magnetic_field():
    """Pure B: |u| is conserved exactly and u rotates by 2*atan(t) per step."""
    nz = 400
    Ex = np.zeros(nz + 1)
    H0 = 50.0  # A/m in the reference's Hy convention
    Hy = np.full(nz + 1, H0)
    dz, dt = 0.015, 0.5 * 0.015 / O.C0
    k = O.pic_constants(dz, dt, 1.0, 1.25663706127e-06)
    scal = np.array([10, 390, k["kE"], k["kH"], k["sc"], k["kJ"], k["kJz"]])
    cell = np.array([200], np.int32)
    frac = np.array([0.25])
    ux, uz = np.array([0.2]), np.array([0.0])
    g = np.sqrt(1 + 0.04)
    ty = k["kH"] * H0 / g
    angle = 2 * np.arctan(ty)
    u0 = np.hypot(ux[0], uz[0])
    for n in range(1, 51):
        _step(cell, frac, ux, uz, Ex, Hy, Hy, scal, nz)
        assert abs(np.hypot(ux[0], uz[0]) - u0) < 1e-15
        phi = np.arctan2(uz[0], ux[0])
        want = np.angle(np.exp(1j * (n * angle)))
        assert abs(np.angle(np.exp(1j * (phi - want)))) < 1e-12


def test_uniform_electric_field_momentum_gain():
    """Pure E: ux grows by 2*kE*E per step, exactly linear."""
    nz = 400
    E0 = 1e3
    Ex = np.full(nz + 1, E0)
    Hy = np.zeros(nz + 1)
    dz, dt = 0.015, 0.5 * 0.015 / O.C0
    k = O.pic_constants(dz, dt, 1.0, 1.25663706127e-06)
    scal = np.array([10, 390, k["kE"], k["kH"], k["sc"], k["kJ"], k["kJz"]])
    cell, frac = np.array([100], np.int32), np.array([0.5])
    ux, uz = np.array([0.0]), np.array([0.3])
    for n in range(1, 21):
        _step(cell, frac, ux, uz, Ex, Hy, Hy, scal, nz)
        assert abs(ux[0] - n * 2 * k["kE"] * E0) <= 1e-13 * abs(n * 2 * k["kE"] * E0)
        assert uz[0] == 0.3


def _charge(cell, frac, nz, qw):
    Q = np.zeros(nz + 1)
    np.add.at(Q, cell, qw * (1 - frac))
    np.add.at(Q, cell + 1, qw * frac)
    return Q


def test_jz_deposit_conserves_charge_exactly():
    nz = 300
    rng = np.random.Generator(np.random.PCG64(7))
    Ex = rng.normal(0, 50, nz + 1)
    Hy = rng.normal(0, 0.1, nz + 1)
    dz, dt = 0.015, 0.5 * 0.015 / O.C0
    w = 1e10
    k = O.pic_constants(dz, dt, w, 1.25663706127e-06)
    clo, chi = 20, 280
    scal = np.array([clo, chi, k["kE"], k["kH"], k["sc"], k["kJ"], k["kJz"]])
    cell, frac, ux, uz = O.beam(5000, clo, chi, v_mean=0.3, v_spread=0.1)
    qw = O.Q_E * w
    for _ in range(5):
        Q0 = _charge(cell, frac, nz, qw)
        Jx, Jz, lost = _step(cell, frac, ux, uz, Ex, Hy, Hy, scal, nz)
        assert lost == 0
        Q1 = _charge(cell, frac, nz, qw)
        # (Q1-Q0)/dt + (Jz[h]-Jz[h-1])/dz = 0 away from the wrap seam
        h = np.arange(clo + 2, chi - 2)
        resid = (Q1[h] - Q0[h]) / dt + (Jz[h] - Jz[h - 1]) / dz
        scale = np.abs(Jz).max() / dz
        assert np.abs(resid).max() <= 1e-9 * scale
