"""The reference's uncalled per-step variants on the GPU (fdtdpic_variant_run) against the
reference's own outputs (tests/golden/variants.npz) and the oracle: FP64 bit for bit, single
rows and ragged batches (rows of different sizes in one launch); FP32 within 1e-5 of the FP64
values (relative to each array's largest magnitude); the one-pass Varin step equal to the three
separate updates; the compat wrappers (reference names, (V, P) arguments) equal to the
reference."""
import numpy as np
import pytest

from helpers import load
from oracle import oracle as o

pytestmark = pytest.mark.gpu

TAGS = ["v60", "v200", "v6", "v8", "v10"]
FP32_TOL = 1e-5


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _case(tag):
    g = load("variants")
    G = lambda k: g[f"{tag}_{k}"]  # noqa: E731
    return G


def _row_of(G):
    from fdtdpic import variants
    return variants.make_rows(
        len(G("mur_Ex_in")), int(G("Nz")), int(G("front")), int(G("rear")), c0=float(G("c0")),
        dt=float(G("delT")), dz=float(G("dz")), eps0=float(G("permit_0")),
        plasma_freq=float(G("plasmaFreqE")), omega0=float(G("omega_0E")),
        gamma=float(G("gammaE")), omega0_j=float(G("omega_0")), chi1=float(G("chi1Stat")),
        chi3=float(G("chi3Stat")), alpha3=float(G("alpha3")), nl_gamma=float(G("nonLin3gammaE")),
        nl_omega0=float(G("nonLin3Omega_0E")))


def _stack(torch, arrs, stride, dtype):
    out = np.zeros((len(arrs), stride))
    for i, a in enumerate(arrs):
        out[i, :len(a)] = a
    return torch.from_numpy(out).to("cuda", dtype)


def _run_all(torch, tags, dtype):
    """Every operation over the rows of `tags` in one launch each; returns host results."""
    from fdtdpic import variants
    Gs = [_case(t) for t in tags]
    rec = np.concatenate([_row_of(G) for G in Gs])
    rows = variants.Rows(rec)
    stride = int(rec["n"].max()) + 3
    S = lambda k: _stack(torch, [G(k) for G in Gs], stride, dtype)  # noqa: E731
    ex, e2 = S("mur_Ex_in"), S("mur_E2")
    variants.mur_ex(ex, e2, rows)
    jx = S("jx_in")
    variants.ade_jx(jx, S("jx_pc"), S("jx_p1"), S("jx_p2"), rows)
    pb = torch.zeros_like(jx)
    variants.varin_pbar(pb, S("pbar_Ex"), S("pbar_Q"), rows)
    J, P = S("jp_J"), S("jp_P")
    variants.varin_jp(J, P, S("pbar_out"), rows)
    Gx, Q = S("qg_G"), S("qg_Q")
    variants.varin_qg(Gx, Q, S("qg_Ex"), rows)
    torch.cuda.synchronize()
    res = dict(mur_Ex_out=ex, jx_out=jx, pbar_out=pb, jp_J_out=J, jp_P_out=P, qg_G_out=Gx,
               qg_Q_out=Q)
    return Gs, {k: v.double().cpu().numpy() for k, v in res.items()}


@pytest.mark.parametrize("tag", TAGS)
def test_fp64_single_row_equals_reference(tag):
    torch = _torch()
    Gs, res = _run_all(torch, [tag], torch.float64)
    G = Gs[0]
    for k, v in res.items():
        ref = G(k)
        assert np.array_equal(v[0, :len(ref)], ref), k


def test_fp64_ragged_batch_equals_reference():
    torch = _torch()
    Gs, res = _run_all(torch, TAGS, torch.float64)
    for i, G in enumerate(Gs):
        for k, v in res.items():
            ref = G(k)
            assert np.array_equal(v[i, :len(ref)], ref), (TAGS[i], k)
            assert not v[i, len(ref):].any(), "padding beyond a row's n was written"


def test_fp32_within_tolerance():
    torch = _torch()
    Gs, res = _run_all(torch, TAGS, torch.float32)
    for i, G in enumerate(Gs):
        for k, v in res.items():
            ref = G(k)
            got = v[i, :len(ref)]
            scale = np.abs(ref).max()
            assert np.abs(got - ref).max() <= FP32_TOL * scale, (TAGS[i], k)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_varin_step_equals_three_updates(dtype):
    torch = _torch()
    from fdtdpic import variants
    td = torch.float64 if dtype == "f64" else torch.float32
    rng = np.random.Generator(np.random.PCG64(5))
    n_rows, stride = 7, 4099
    n = rng.integers(100, stride + 1, n_rows)
    front = rng.integers(0, 50, n_rows)
    rear = np.minimum(n, front + rng.integers(10, 4000, n_rows))
    rec = variants.make_rows(n, n - 1, front, rear, dt=1.6e-12, dz=1e-3, eps0=8.854e-12,
                             omega0=2 * np.pi * 1.5e9, gamma=2 * np.pi * 1e8, chi1=0.2,
                             chi3=1e-3, alpha3=0.699999988079071, nl_gamma=2 * np.pi * 3e8,
                             nl_omega0=2 * np.pi * 4e9)
    rows = variants.Rows(rec)
    mk = lambda s: torch.from_numpy(s * rng.standard_normal((n_rows, stride))).to("cuda", td)  # noqa: E731
    a = dict(pb=mk(0.0), jx=mk(1.0), pc=mk(1e-11), g=mk(1.0), q=mk(1.0) ** 2, ex=mk(1.0))
    b = {k: v.clone() for k, v in a.items()}
    init = {k: v.double().cpu().numpy().copy() for k, v in a.items()}
    variants.varin_step(a["pb"], a["jx"], a["pc"], a["g"], a["q"], a["ex"], rows)
    variants.varin_pbar(b["pb"], b["ex"], b["q"], rows)
    variants.varin_jp(b["jx"], b["pc"], b["pb"], rows)
    variants.varin_qg(b["g"], b["q"], b["ex"], rows)
    torch.cuda.synchronize()
    for k in a:
        assert torch.equal(a[k], b[k]), k
    # and the FP64 values are the oracle's, row by row (cells outside [front, rear) untouched)
    if dtype == "f64":
        h = {k: v.cpu().numpy() for k, v in b.items()}
        for r in range(n_rows):
            fr, rr = int(front[r]), int(rear[r])
            x = {k: v[r].copy() for k, v in init.items()}
            o.varin_pbar(x["pb"], x["ex"], x["q"], fr, rr, 8.854e-12, 0.2, 1e-3,
                         0.699999988079071)
            o.varin_jp(x["jx"], x["pc"], x["pb"], fr, rr, 2 * np.pi * 1.5e9, 2 * np.pi * 1e8,
                       1.6e-12)
            o.varin_qg(x["g"], x["q"], x["ex"], fr, rr, 2 * np.pi * 3e8, 2 * np.pi * 4e9, 1.6e-12)
            for k in x:
                assert np.array_equal(h[k][r], x[k]), (r, k)


def test_compat_wrappers_equal_reference():
    _torch()
    from types import SimpleNamespace

    from fdtdpic.compat import BaseFDTD11 as B
    for tag in TAGS:
        G = _case(tag)
        P = SimpleNamespace(Nz=int(G("Nz")), materialFrontEdge=int(G("front")),
                            materialRearEdge=int(G("rear")), c0=float(G("c0")),
                            delT=float(G("delT")), dz=float(G("dz")),
                            permit_0=float(G("permit_0")))
        V = SimpleNamespace(plasmaFreqE=float(G("plasmaFreqE")), omega_0E=float(G("omega_0E")),
                            gammaE=float(G("gammaE")), chi1Stat=float(G("chi1Stat")),
                            chi3Stat=float(G("chi3Stat")), alpha3=float(G("alpha3")),
                            nonLin3gammaE=float(G("nonLin3gammaE")),
                            nonLin3Omega_0E=float(G("nonLin3Omega_0E")))
        V.Ex, V.tempTempVarE = G("mur_Ex_in").copy(), G("mur_E2").copy()
        ex_obj = V.Ex
        out = B.MUR1DEx(V, P, None, None)
        assert out is ex_obj and np.array_equal(out, G("mur_Ex_out"))
        V.Jx, V.polarisationCurr = G("jx_in").copy(), G("jx_pc").copy()
        V.tempVarPol, V.tempTempVarPol = G("jx_p1").copy(), G("jx_p2").copy()
        with pytest.raises(AttributeError):
            B.ADE_JxUpdate(V, P, None, None)
        V.omega_0 = float(G("omega_0"))
        assert np.array_equal(B.ADE_JxUpdate(V, P, None, None), G("jx_out"))
        V.Pbar3 = np.zeros_like(G("pbar_Ex"))
        V.Ex, V.Qx3 = G("pbar_Ex").copy(), G("pbar_Q").copy()
        assert np.array_equal(B.ADE_NonLin_Pol_Ex_Pbar(V, P), G("pbar_out"))
        V.Jx, V.polarisationCurr = G("jp_J").copy(), G("jp_P").copy()
        J, Pc = B.ADE_Lin_Curr_And_Pol_Varin(V, P)
        assert np.array_equal(J, G("jp_J_out")) and np.array_equal(Pc, G("jp_P_out"))
        V.Gx3, V.Qx3, V.Ex = G("qg_G").copy(), G("qg_Q").copy(), G("qg_Ex").copy()
        Gx, Q, _ = B.ADE_Nonlin_Q_and_G(V, P)
        assert np.array_equal(Gx, G("qg_G_out")) and np.array_equal(Q, G("qg_Q_out"))


def test_fp64_large_rows_equal_oracle():
    """Rows of 2^20 cells (many CTAs' worth of cells per row, grid-stride over rows)."""
    torch = _torch()
    from fdtdpic import variants
    rng = np.random.Generator(np.random.PCG64(11))
    n_rows, n = 3, 1 << 20
    rec = variants.make_rows(n, n - 1, [1, 100, 5000], [n, n - 7, 600000], dt=1.6e-12, dz=1e-3,
                             eps0=8.854e-12, plasma_freq=2 * np.pi * 2e9,
                             omega0=2 * np.pi * 1.5e9, gamma=2 * np.pi * 1e8,
                             omega0_j=2 * np.pi * 3e9)
    rows = variants.Rows(rec)
    h = [1e-11 * rng.standard_normal((n_rows, n)) for _ in range(3)]
    jx0 = rng.standard_normal((n_rows, n))
    jx = torch.from_numpy(jx0).cuda()
    variants.ade_jx(jx, *[torch.from_numpy(x).cuda() for x in h], rows)
    got = jx.cpu().numpy()
    for r in range(n_rows):
        ref = jx0[r].copy()
        o.ade_jx_update(ref, h[0][r], h[1][r], h[2][r], int(rec["front"][r]), int(rec["rear"][r]),
                        8.854e-12, 2 * np.pi * 2e9, 2 * np.pi * 1.5e9, 2 * np.pi * 3e9,
                        2 * np.pi * 1e8, 1.6e-12)
        assert np.array_equal(got[r], ref), r
