"""Batched sweep (one persistent launch over ragged instances) and the batched probe DFT,
against the FP64 CPU oracle and a float64 numpy DFT."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _np_dft(x, freqs, dt):
    n = np.arange(x.shape[-1])
    W = np.exp(-2j * np.pi * np.outer(freqs * dt, n))
    return x @ W.T


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_dft_matches_numpy_strided(precision):
    torch = _torch()
    import ctypes
    from fdtdpic import engine
    from fdtdpic._lib import check, lib
    L = lib()
    rng = np.random.default_rng(7)
    n_pairs, S, F = 45, 1000, 77  # ragged against the 32 x 64 x 64 tiles
    dt = 2.5e-11
    freqs = np.sort(rng.uniform(0.1e9, 3.1e9, F))  # off the FFT bins
    x = rng.standard_normal((n_pairs, S, 2))
    tdt = torch.float32 if precision == "f32" else torch.float64
    d_x = torch.from_numpy(x).to(tdt).cuda().contiguous()
    d_f = torch.from_numpy(freqs).cuda()
    d_tw = torch.empty(int(L.fdtdpic_dft_twiddle_bytes(F, S)), dtype=torch.uint8, device="cuda")
    d_out = torch.empty(2 * n_pairs * F * 2, dtype=torch.float64, device="cuda")
    d_R = torch.empty(n_pairs * F, dtype=torch.float64, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    check(L.fdtdpic_dft_twiddles(engine._ptr(d_f), F, S, dt, engine._ptr(d_tw), st))
    prec = 4 if precision == "f32" else 8
    check(L.fdtdpic_dft_probes(prec, engine._ptr(d_x), 2 * n_pairs, S, 2, 2 * S, 1, 2,
                               engine._ptr(d_tw), F, engine._ptr(d_out), st))
    check(L.fdtdpic_reflection_ratio(engine._ptr(d_out), n_pairs, F, engine._ptr(d_R), st))
    torch.cuda.synchronize()
    got = d_out.cpu().numpy().reshape(2 * n_pairs, F, 2)
    got = got[..., 0] + 1j * got[..., 1]
    xin = d_x.double().cpu().numpy()  # the values the kernel read
    traces = xin.transpose(0, 2, 1).reshape(2 * n_pairs, S)
    want = _np_dft(traces, freqs, dt)
    # FP32 twiddles and FP32 products inside 64-step chunks, FP64 across chunks
    err = np.abs(got - want).max() / np.abs(traces).sum(axis=1).max()
    assert err < 2e-7, err
    ratio = d_R.cpu().numpy().reshape(n_pairs, F)
    want_r = np.abs(want[1::2]) / np.abs(want[0::2])
    np.testing.assert_allclose(ratio, want_r, rtol=1e-4)


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_dft_tensor_cores_match_numpy(precision):
    """tcgen05 split-BF16x3 form: each product carries ~16 significant bits, so the error is
    bounded by ~3 * 2^-17 of the sum of |terms|; FP64 sums across 64-step chunks."""
    torch = _torch()
    import ctypes
    from fdtdpic import engine
    from fdtdpic._lib import check, lib
    L = lib()
    rng = np.random.default_rng(11)
    n_pairs, S, F = 70, 1000, 77  # 140 traces: two row tiles, the second ragged
    dt = 2.5e-11
    freqs = np.sort(rng.uniform(0.1e9, 3.1e9, F))
    x = rng.standard_normal((n_pairs, S, 2))
    tdt = torch.float32 if precision == "f32" else torch.float64
    d_x = torch.from_numpy(x).to(tdt).cuda().contiguous()
    d_f = torch.from_numpy(freqs).cuda()
    d_tw = torch.empty(int(L.fdtdpic_dft_twiddle_bytes(F, S)), dtype=torch.uint8, device="cuda")
    d_out = torch.full((2 * n_pairs * F * 2,), float("nan"), dtype=torch.float64, device="cuda")
    d_err = torch.zeros(1, dtype=torch.int32, device="cuda")
    nb = int(L.fdtdpic_dft_tc_scratch_bytes(2 * n_pairs, S, F))
    d_scr = torch.empty(nb, dtype=torch.uint8, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    check(L.fdtdpic_dft_twiddles(engine._ptr(d_f), F, S, dt, engine._ptr(d_tw), st))
    prec = 4 if precision == "f32" else 8
    assert L.fdtdpic_dft_probes_tc(prec, engine._ptr(d_x), 2 * n_pairs, S, 2, 2 * S, 1, 2,
                                   engine._ptr(d_tw), F, engine._ptr(d_out), engine._ptr(d_scr),
                                   nb - 16, engine._ptr(d_err), st) != 0  # scratch too small
    check(L.fdtdpic_dft_probes_tc(prec, engine._ptr(d_x), 2 * n_pairs, S, 2, 2 * S, 1, 2,
                                  engine._ptr(d_tw), F, engine._ptr(d_out), engine._ptr(d_scr), nb,
                                  engine._ptr(d_err), st))
    torch.cuda.synchronize()
    assert int(d_err.item()) == 0
    got = d_out.cpu().numpy().reshape(2 * n_pairs, F, 2)
    got = got[..., 0] + 1j * got[..., 1]
    traces = d_x.double().cpu().numpy().transpose(0, 2, 1).reshape(2 * n_pairs, S)
    want = _np_dft(traces, freqs, dt)
    err = np.abs(got - want).max() / np.abs(traces).sum(axis=1).max()
    assert err < 5e-5, err


def test_dft_rejects_bad_arguments():
    torch = _torch()
    from fdtdpic._lib import lib
    L = lib()
    d = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = d.data_ptr()
    assert L.fdtdpic_dft_probes(4, p, 2, 0, 2, 0, 1, 2, p, 4, p, None) != 0  # S = 0
    assert L.fdtdpic_dft_probes(3, p, 2, 8, 2, 16, 1, 2, p, 4, p, None) != 0  # precision
    assert L.fdtdpic_dft_twiddles(p, 4, 8, -1.0, p, None) != 0                 # dt <= 0
    assert L.fdtdpic_dft_twiddle_bytes(512, 8192) == 512 * 8192 * 8


SMALL = dict(n_inst=10, n_steps=2048, nz_lo=500, nz_hi=1400, n_freqs=96, seed=11)


def _oracle_probes(spec, p, src):
    import scipy.constants as sc
    from fdtdpic import sweep
    dt = sweep.SC * sweep.DZ / O.C0
    w0 = 2 * np.pi * p["f0"]
    P = O.RefParams(Nz=p["nz"], timeSteps=spec.n_steps, dz=sweep.DZ, delT=dt,
                    courantNo=O.f32(sweep.SC), materialFrontEdge=p["front"],
                    materialRearEdge=p["rear"], pmlWidth=spec.pml, nzsrc=spec.nzsrc,
                    freq_in=spec.freq_in, permit_0=sc.epsilon_0, permea_0=sc.mu_0,
                    nonLinMed=True, FreeSpace=False, plasmaFreqE=np.sqrt(p["d_eps"]) * w0,
                    omega_0E=w0, gammaE=2 * np.pi * 0.1e9, chi3Stat=p["chi3"],
                    sigmaOpt=O.sigma_opt(sweep.DZ, sc.epsilon_0, sc.mu_0))
    r = O.integrate(P, O.KERR, src, np.zeros(spec.n_steps), extra_probes=p["probes"])
    return r


@pytest.fixture(scope="module", params=["tc", "cuda"])
def small_sweep(request):
    _torch()
    import torch
    from fdtdpic import sweep
    spec = sweep.SweepSpec(**SMALL)
    grids, dt = sweep.make_sweep_grids(spec)
    sw = sweep.Sweep(grids, dt, spec.freqs(), precision="f32", dft=request.param)
    sw.run()
    torch.cuda.synchronize()
    assert sw.dft_error() == 0
    return spec, grids, dt, sw


def test_sweep_fp32_matches_fp64_oracle(small_sweep):
    from fdtdpic import engine, sweep
    spec, grids, dt, sw = small_sweep
    params = sweep.sweep_parameters(spec)
    res = engine.download(sw.packed)
    R = sw.reflection()
    X = sw.spectra()
    freqs = spec.freqs()
    worst_f, worst_p, worst_r = 0.0, 0.0, 0.0
    for i, p in enumerate(params):
        assert res[i].status == 0
        r = _oracle_probes(spec, p, grids[i].exs)
        worst_f = max(worst_f, O.rel_l2(res[i].Ex, r.Ex), O.rel_l2(res[i].Hy, r.Hy))
        for j in (0, 1):
            worst_p = max(worst_p, O.rel_l2(res[i].probes[:, j], r.probes[:, j]))
        want = _np_dft(r.probes.T, freqs, dt)
        # spectra of the GPU traces vs the oracle's traces
        assert np.abs(X[2 * i:2 * i + 2] - want).max() <= 1e-4 * np.abs(want).max()
        # |R(f)| in the source band: where the incident spectrum is within 40 dB of its peak
        # (further out the ratio divides FP32 rounding by a vanishing incident amplitude)
        band = np.abs(want[0]) >= 1e-2 * np.abs(want[0]).max()
        want_r = np.abs(want[1]) / np.abs(want[0])
        worst_r = max(worst_r, np.abs(R[i][band] - want_r[band]).max() / max(want_r[band].max(), 1e-30))
    # stated FP32 error against the FP64 oracle (2048 steps): final Ex/Hy 1e-5 rel L2, probe
    # traces 5e-5 rel L2 (a trace also holds the low-amplitude tail after the pulse has
    # passed, where FP32 rounding is a larger share), |R(f)| 1e-4 relative to its largest
    # value in the source band
    print(f"sweep fp32 vs oracle: fields {worst_f:.3e} traces {worst_p:.3e} |R| {worst_r:.3e}")
    assert worst_f <= 1e-5, worst_f
    assert worst_p <= 5e-5, worst_p
    assert worst_r <= 1e-4, worst_r


def test_sweep_graph_replay_and_alone_equal_batch(small_sweep):
    torch = _torch()
    from fdtdpic import engine, sweep
    spec, grids, dt, sw = small_sweep
    base_p = sw.d_probe_view().copy()
    base_R = sw.reflection().copy()
    sw2 = sweep.Sweep(grids, dt, spec.freqs(), precision="f32", threads=512, dft=sw.dft)
    sw2.capture()
    for _ in range(2):
        sw2.run()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(sw2.d_probe_view(), base_p)
    np.testing.assert_array_equal(sw2.reflection(), base_R)
    for k in (0, len(grids) - 1):
        one = sweep.Sweep([grids[k]], dt, spec.freqs(), precision="f32", dft=sw.dft)
        one.run()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(one.d_probe_view()[0], base_p[k])
        np.testing.assert_array_equal(one.reflection()[0], base_R[k])


def test_autotune_picks_a_candidate(tmp_path, monkeypatch):
    _torch()
    from fdtdpic import sweep
    monkeypatch.setattr(sweep, "_CACHE", str(tmp_path / "autotune.json"))
    spec = sweep.SweepSpec(n_inst=24, n_steps=256, seed=3)
    grids, dt = sweep.make_sweep_grids(spec)
    res = sweep.autotune(grids, probe_steps=64, candidates=(128, 256))
    assert res["threads"] in (128, 256)
    again = sweep.autotune(grids, probe_steps=64, candidates=(128, 256))
    assert again == res  # served from the cache file
