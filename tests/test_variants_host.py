"""The reference's uncalled per-step variants (MUR1DEx, ADE_JxUpdate, Varin's three ADE
updates; BaseFDTD11.py:543-607, 769-788) on the host: the oracle reproduces the reference's own
outputs (tests/golden/variants.npz, made by running those functions) bit for bit, the C ABI
accepts and refuses row sets as documented, and the compat ADE_JxUpdate raises as the
reference's does when the state has no omega_0.  No GPU needed."""
import numpy as np
import pytest

from oracle import oracle as o
from helpers import load

TAGS = ["v60", "v200", "v6", "v8", "v10"]


def _g(tag):
    g = load("variants")
    return lambda k: g[f"{tag}_{k}"]


def _f(G, k):
    return float(G(k))


@pytest.mark.parametrize("tag", TAGS)
def test_oracle_matches_reference_bit_for_bit(tag):
    G = _g(tag)
    Nz, fr, rr = int(G("Nz")), int(G("front")), int(G("rear"))
    ex = G("mur_Ex_in").copy()
    o.mur1d_ex(ex, G("mur_E2"), Nz, _f(G, "c0"), _f(G, "delT"), _f(G, "dz"))
    assert np.array_equal(ex, G("mur_Ex_out"))
    jx = G("jx_in").copy()
    o.ade_jx_update(jx, G("jx_pc"), G("jx_p1"), G("jx_p2"), fr, rr, _f(G, "permit_0"),
                    _f(G, "plasmaFreqE"), _f(G, "omega_0E"), _f(G, "omega_0"), _f(G, "gammaE"),
                    _f(G, "delT"))
    assert np.array_equal(jx, G("jx_out"))
    assert bool(G("jx_raises"))
    pb = np.zeros_like(G("pbar_Ex"))
    o.varin_pbar(pb, G("pbar_Ex"), G("pbar_Q"), fr, rr, _f(G, "permit_0"), _f(G, "chi1Stat"),
                 _f(G, "chi3Stat"), _f(G, "alpha3"))
    assert np.array_equal(pb, G("pbar_out"))
    J, P = G("jp_J").copy(), G("jp_P").copy()
    o.varin_jp(J, P, G("pbar_out"), fr, rr, _f(G, "omega_0E"), _f(G, "gammaE"), _f(G, "delT"))
    assert np.array_equal(J, G("jp_J_out")) and np.array_equal(P, G("jp_P_out"))
    Gx, Q = G("qg_G").copy(), G("qg_Q").copy()
    o.varin_qg(Gx, Q, G("qg_Ex"), fr, rr, _f(G, "nonLin3gammaE"), _f(G, "nonLin3Omega_0E"),
               _f(G, "delT"))
    assert np.array_equal(Gx, G("qg_G_out")) and np.array_equal(Q, G("qg_Q_out"))


def test_golden_mur_bands_overlap_on_short_grids():
    # on 6-10 cell grids the right loop reads cells the left loop rewrote
    for tag in ("v6", "v8"):
        G = _g(tag)
        assert int(G("Nz")) - 6 < 5


def _rows(**kw):
    from fdtdpic import variants
    base = dict(n=61, nz=60, front=20, rear=45, dt=1e-12, dz=1e-3, eps0=8.854e-12)
    base.update(kw)
    return variants.make_rows(**base)


def test_variant_row_checks():
    from fdtdpic import _lib, variants
    ok = variants.check_rows
    assert ok(_lib.VAR_MUR_EX, _rows(), 61)
    assert ok(_lib.VAR_MUR_EX, _rows(n=6, nz=6, front=1, rear=5), 8)
    assert not ok(_lib.VAR_MUR_EX, _rows(n=6, nz=5, front=1, rear=5), 8)    # Nz < 6
    assert not ok(_lib.VAR_MUR_EX, _rows(nz=62), 61)                       # Nz > n
    assert not ok(_lib.VAR_MUR_EX, _rows(), 60)                            # n > stride
    assert ok(_lib.VAR_ADE_JX, _rows(front=1, rear=61), 61)
    assert not ok(_lib.VAR_ADE_JX, _rows(front=0), 61)                     # cell -1
    assert not ok(_lib.VAR_ADE_JX, _rows(rear=62), 64)
    for op in (_lib.VAR_VARIN_PBAR, _lib.VAR_VARIN_JP, _lib.VAR_VARIN_QG, _lib.VAR_VARIN_STEP):
        assert ok(op, _rows(front=0, rear=61), 61)
        assert ok(op, _rows(front=50, rear=10), 61)                        # empty range
        assert not ok(op, _rows(front=-1), 61)
        assert not ok(op, _rows(rear=62), 64)
    assert not ok(99, _rows(), 61)
    big = 2 ** 31 - 1
    assert ok(_lib.VAR_VARIN_PBAR, _rows(front=big, rear=10), 61)          # empty, far out
    assert ok(_lib.VAR_ADE_JX, _rows(front=big, rear=10), 61)
    assert not ok(_lib.VAR_ADE_JX, _rows(front=-big - 1, rear=10), 61)
    two = np.concatenate([_rows(), _rows(n=30, nz=29, front=5, rear=25)])
    assert ok(_lib.VAR_VARIN_STEP, two, 61)
    two["rear"][1] = 31
    assert not ok(_lib.VAR_VARIN_STEP, two, 61)


def test_variant_run_refuses_bad_arguments_before_any_device_work():
    import ctypes

    from fdtdpic import _lib
    L = _lib.lib()
    rec = _rows()
    ptrs = (ctypes.c_void_p * 6)()
    # precision, row checks and null arrays are refused on the host
    assert L.fdtdpic_variant_run(_lib.VAR_MUR_EX, 2, 1, rec.ctypes.data, None, 61,
                                 ctypes.cast(ptrs, ctypes.c_void_p), None) == -1
    assert L.fdtdpic_variant_run(_lib.VAR_MUR_EX, 8, 1, rec.ctypes.data, None, 60,
                                 ctypes.cast(ptrs, ctypes.c_void_p), None) == -1
    assert L.fdtdpic_variant_run(_lib.VAR_MUR_EX, 8, 1, rec.ctypes.data, rec.ctypes.data, 61,
                                 ctypes.cast(ptrs, ctypes.c_void_p), None) == -1
    assert L.fdtdpic_variant_run(_lib.VAR_MUR_EX, 8, 0, None, None, 61, None, None) == 0


def test_compat_jx_update_raises_without_omega_0():
    from types import SimpleNamespace

    from fdtdpic.compat import BaseFDTD11 as B
    V = SimpleNamespace(Jx=np.zeros(11), polarisationCurr=np.zeros(11), tempVarPol=np.zeros(11),
                        tempTempVarPol=np.zeros(11), plasmaFreqE=1.0, omega_0E=1.0, gammaE=0.1)
    P = SimpleNamespace(Nz=10, materialFrontEdge=2, materialRearEdge=8, c0=3e8, delT=1e-12,
                        dz=1e-3, permit_0=8.854e-12)
    with pytest.raises(AttributeError):
        B.ADE_JxUpdate(V, P, None, None)
