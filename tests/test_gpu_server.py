"""Served requests (continuous batching over slots) on the GPU: a beam request equals the
streaming PIC run bit for bit, a field-only request equals the batch engine (FP64 bit for bit),
and every request's result is the same alone and in a mix with staggered arrivals."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DZ = 0.015


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _grid(nz, steps, front, rear, nzsrc=60, chi3=1e-2, seed=None):
    from fdtdpic.grid import lorentz_kerr_grid
    return lorentz_kerr_grid(nz, steps, front=front, rear=rear, nzsrc=nzsrc,
                             probes=(50, nz - 50), chi3=chi3)


def _serve(reqs, precision="f32", **kw):
    from fdtdpic.server import Server
    srv = Server(precision=precision, keep_state=True, **kw)
    for r in reqs:
        srv.submit(r)
    done = srv.drain()
    return {d.rid: d for d in done}


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_beam_request_equals_streaming_pic_run(precision):
    torch = _torch()
    import scipy.constants as sc
    from fdtdpic.pic import PicRun, make_beam
    from fdtdpic.server import Request
    nz, T, npart = 512, 600, 20000
    dt = 0.5 * DZ / 299792458.0
    g = _grid(nz, T, 300, 400)
    beam = make_beam(npart, 40, 480, DZ)
    run = PicRun(g, beam, DZ, dt, sc.mu_0, precision=precision, path="streaming")
    run.step(T)
    torch.cuda.synchronize()
    probes_ref = run.probes()
    cell_ref, frac_ref, ux_ref, uz_ref = run.particles()
    Ex_ref, Hy_ref = run.fields()["Ex"], run.fields()["Hy"]
    Jx_ref, Jz_ref = run.currents()
    # small chunks so the request crosses many rounds
    got = _serve([Request(grid=g, beam=beam, dz=DZ, dt=dt, mu0=sc.mu_0, rid=0)],
                 precision=precision, chunk_ms=0.05)[0]
    np.testing.assert_array_equal(got.probes, probes_ref)
    assert got.status[0] == 0 and got.status[1] == 0
    p = got.particles  # never re-ordered: index == id
    np.testing.assert_array_equal(p["cell"], cell_ref)
    for k, ref in (("frac", frac_ref), ("ux", ux_ref), ("uz", uz_ref)):
        np.testing.assert_array_equal(np.asarray(p[k], np.float64), ref, err_msg=k)
    np.testing.assert_array_equal(got.fields["Ex"], Ex_ref)
    np.testing.assert_array_equal(got.fields["Hy"], Hy_ref)
    np.testing.assert_array_equal(got.fields["Jx"], Jx_ref)
    np.testing.assert_array_equal(got.fields["Jz"], Jz_ref)


def test_field_only_requests_equal_batch_engine_fp64():
    """Both forms (shared-memory fields, and global-memory fields for a grid too large for the
    server's shared-memory budget) against engine.run in FP64."""
    _torch()
    from fdtdpic import engine
    from fdtdpic.server import Request
    grids = [_grid(900, 700, 400, 500, nzsrc=100), _grid(6000, 300, 2000, 3000, nzsrc=100)]
    want = engine.run(grids, "f64")
    got = _serve([Request(grid=g, rid=i) for i, g in enumerate(grids)], precision="f64",
                 chunk_ms=0.05, smem_bytes=48 * 1024)
    for i in range(len(grids)):
        np.testing.assert_array_equal(got[i].probes, want[i].probes)
        np.testing.assert_array_equal(got[i].fields["Ex"], want[i].Ex)
        np.testing.assert_array_equal(got[i].fields["Hy"], want[i].Hy)


def test_results_same_alone_and_in_the_mix():
    """Requests of mixed sizes (field-only, beams, grids past the shared-memory budget) arrive
    while others run; each result equals the same request served alone."""
    torch = _torch()
    import scipy.constants as sc
    from fdtdpic.pic import make_beam
    from fdtdpic.server import Request, Server
    dt = 0.5 * DZ / 299792458.0
    rng = np.random.default_rng(3)
    specs = []
    for i in range(14):
        nz = int(rng.choice([300, 700, 2500, 9000]))
        T = int(rng.integers(200, 900))
        npart = int(rng.choice([0, 0, 3000, 40000]))
        specs.append((nz, T, npart))

    def req(i):
        nz, T, npart = specs[i]
        g = _grid(nz, T, nz // 2 - nz // 10, nz // 2 + nz // 10, nzsrc=60)
        b = make_beam(npart, 40, nz - 41, DZ, seed=100 + i) if npart else None
        return Request(grid=g, beam=b, dz=DZ, dt=dt, mu0=sc.mu_0, rid=i)

    alone = {}
    for i in range(len(specs)):
        alone.update(_serve([req(i)], chunk_ms=0.2))
    srv = Server(precision="f32", keep_state=True, chunk_ms=0.2)
    pending = [req(i) for i in range(len(specs))]
    # staggered admission: a few requests join after rounds have started
    for r in pending[:5]:
        srv.submit(r)
    srv.poll()
    srv.poll()
    for r in pending[5:10]:
        srv.submit(r)
    srv.poll()
    for r in pending[10:]:
        srv.submit(r)
    mixed = {d.rid: d for d in srv.drain()}
    assert sorted(mixed) == list(range(len(specs)))
    assert srv.rounds > 3
    for i in range(len(specs)):
        np.testing.assert_array_equal(mixed[i].probes, alone[i].probes, err_msg=str(specs[i]))
        np.testing.assert_array_equal(mixed[i].fields["Ex"], alone[i].fields["Ex"])
        if specs[i][2]:
            np.testing.assert_array_equal(mixed[i].particles["uz"], alone[i].particles["uz"])
        assert mixed[i].status[1] == 0


def test_hbm_budget_limits_admission():
    _torch()
    from fdtdpic.server import Request, Server
    grids = [_grid(2000, 400, 900, 1100, nzsrc=100) for _ in range(6)]
    srv = Server(precision="f32", hbm_budget=1.0, chunk_ms=0.2)  # room for one at a time
    for i, g in enumerate(grids):
        srv.submit(Request(grid=g, rid=i))
    peak = 0
    while srv.pending or srv.active or srv.inflight:
        srv.poll()
        peak = max(peak, len(srv.active))
    assert peak == 1 and len(srv.done) == 6


def test_streaming_side_path_equals_rounds():
    """Beam requests sent to the streaming kernels (big_ms=0: every beam request) give the slot
    rounds' results (big_ms=None) bit for bit, mixed with field-only requests."""
    _torch()
    import scipy.constants as sc
    from fdtdpic.pic import make_beam
    from fdtdpic.server import Request
    dt = 0.5 * DZ / 299792458.0

    def reqs():
        return [Request(grid=_grid(700, 500, 300, 400), beam=make_beam(20000, 40, 660, DZ, seed=5),
                        dz=DZ, dt=dt, mu0=sc.mu_0, rid=0),
                Request(grid=_grid(900, 400, 400, 500, nzsrc=100), rid=1),
                Request(grid=_grid(2500, 300, 1000, 1500), beam=make_beam(3000, 40, 2460, DZ, seed=6),
                        dz=DZ, dt=dt, mu0=sc.mu_0, rid=2)]

    side = _serve(reqs(), big_ms=0.0, chunk_ms=0.2)
    rounds = _serve(reqs(), big_ms=None, chunk_ms=0.2)
    assert sorted(side) == sorted(rounds) == [0, 1, 2]
    for i in range(3):
        np.testing.assert_array_equal(side[i].probes, rounds[i].probes)
        np.testing.assert_array_equal(side[i].fields["Ex"], rounds[i].fields["Ex"])
        assert side[i].status[0] == rounds[i].status[0] and side[i].status[1] == 0
    for i in (0, 2):
        np.testing.assert_array_equal(side[i].fields["Jx"], rounds[i].fields["Jx"])
        for k in ("cell", "frac", "ux", "uz"):
            np.testing.assert_array_equal(np.asarray(side[i].particles[k], np.float64),
                                          np.asarray(rounds[i].particles[k], np.float64),
                                          err_msg=k)
