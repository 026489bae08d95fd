"""Failures in the served stream, made on the host: a request cancelled before admission, one
cancelled while its chunks run, one whose preparation raises, one whose source holds a NaN (its
kernel raises the non-finite status bit), and an out-of-memory raised by the admission
allocator (through the server's fault hook).  Each failed request is retired with its error;
every other request's result equals the same request served alone, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DZ = 0.015
DT = 0.5 * DZ / 299792458.0


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _req(i, nz, T, npart, nan_source=False):
    import scipy.constants as sc
    from fdtdpic.grid import lorentz_kerr_grid
    from fdtdpic.pic import make_beam
    from fdtdpic.server import Request
    g = lorentz_kerr_grid(nz, T, front=nz // 2 - nz // 10, rear=nz // 2 + nz // 10, nzsrc=60,
                          probes=(50, nz - 50), chi3=1e-2)
    if nan_source:
        g.exs = g.exs.copy()
        g.exs[5] = np.nan
    b = make_beam(npart, 40, nz - 41, DZ, seed=200 + i) if npart else None
    return Request(grid=g, beam=b, dz=DZ, dt=DT, mu0=sc.mu_0, rid=i)


SPECS = {0: (700, 400, 0), 1: (2500, 300, 3000), 2: (300, 800, 0), 3: (900, 500, 20000),
         4: (9000, 200, 0), 5: (600, 300, 0), 6: (800, 300, 0), 7: (1200, 6000, 0)}


def _alone(i):
    from fdtdpic.server import Server
    srv = Server(precision="f32", keep_state=True, chunk_ms=0.2)
    srv.submit(_req(i, *SPECS[i]))
    (d,) = srv.drain()
    srv.close()
    return d


def test_faults_are_retired_and_the_rest_is_unchanged():
    torch = _torch()
    from fdtdpic.server import Request, Server
    ok_ids = (0, 1, 2, 3, 4)
    alone = {i: _alone(i) for i in ok_ids}
    failed_once = []

    def hook(stage, req):
        # request 3 meets an out-of-memory on its first allocation, while others are resident
        if stage == "alloc" and req.rid == 3 and not failed_once:
            failed_once.append(req.rid)
            raise torch.cuda.OutOfMemoryError("injected")

    srv = Server(precision="f32", keep_state=True, chunk_ms=0.2, fault_hook=hook)
    for i in (0, 1, 2):
        srv.submit(_req(i, *SPECS[i]))
    srv.submit(_req(6, *SPECS[6]))
    srv.cancel(6)  # cancelled before it is admitted
    srv.submit(_req(7, *SPECS[7]))  # 6000 steps: many rounds
    srv.poll()
    srv.poll()
    srv.submit(_req(3, *SPECS[3]))
    srv.submit(_req(5, *SPECS[5], nan_source=True))

    def bad_grid():
        raise ValueError("no such material")

    srv.submit(Request(grid_fn=bad_grid, rid=8, nz=500, n_steps=100))
    srv.submit(_req(4, *SPECS[4]))
    for _ in range(3):
        srv.poll()
    srv.cancel(7)  # while its chunks run
    done = {d.rid: d for d in srv.drain()}
    srv.close()
    assert sorted(done) == [0, 1, 2, 3, 4, 5, 6, 7, 8]
    assert failed_once == [3] and srv.oom_retries >= 1
    assert done[6].error == "cancelled" and done[6].probes.shape[0] == 0
    assert done[7].error == "cancelled"
    assert done[8].error.startswith("prepare: ValueError")
    assert done[5].error is not None and "non-finite" in done[5].error
    for i in ok_ids:
        assert done[i].error is None, (i, done[i].error)
        np.testing.assert_array_equal(done[i].probes, alone[i].probes, err_msg=str(i))
        np.testing.assert_array_equal(done[i].fields["Ex"], alone[i].fields["Ex"])
        np.testing.assert_array_equal(done[i].fields["Hy"], alone[i].fields["Hy"])
        if SPECS[i][2]:
            for k in ("cell", "frac", "ux", "uz"):
                np.testing.assert_array_equal(done[i].particles[k], alone[i].particles[k])
    # everything was handed back
    assert srv.bytes_in_use == 0 and not srv.active and len(srv.free) == srv.max_active


def test_out_of_memory_with_nothing_resident_fails_the_request():
    _torch()
    import torch
    from fdtdpic.server import Server

    def hook(stage, req):
        raise torch.cuda.OutOfMemoryError("injected")

    srv = Server(precision="f32", chunk_ms=0.2, fault_hook=hook)
    srv.submit(_req(0, *SPECS[0]))
    srv.submit(_req(1, 2500, 300, 3000))
    done = {d.rid: d for d in srv.drain()}
    srv.close()
    assert done[0].error.startswith("out of device memory")
    assert done[1].error.startswith("out of device memory")
    assert srv.bytes_in_use == 0 and len(srv.free) == srv.max_active


def test_streaming_run_cancelled_is_discarded():
    """A beam request on the streaming kernels (big_ms=0) cancelled after admission runs out on
    its stream and is reported cancelled; a field-only request beside it is unaffected."""
    _torch()
    from fdtdpic.server import Server
    want = _alone(0)
    srv = Server(precision="f32", keep_state=True, chunk_ms=0.2, big_ms=0.0)
    srv.submit(_req(3, *SPECS[3]))
    srv.submit(_req(0, *SPECS[0]))
    srv.poll()
    srv.cancel(3)
    done = {d.rid: d for d in srv.drain()}
    srv.close()
    assert done[3].error == "cancelled" and done[3].particles is None
    assert done[0].error is None
    np.testing.assert_array_equal(done[0].probes, want.probes)
    assert srv.bytes_in_use == 0


def test_preempted_streaming_runs_resume_bit_for_bit():
    """Streaming runs advance a segment at a time; two of three are parked on the host at a
    segment's end (PicRun.snapshot, device memory released) and resumed later (restore): every
    result equals the same request run without interruption, bit for bit."""
    _torch()
    from fdtdpic.server import Server

    def serve(preempt):
        srv = Server(precision="f32", keep_state=True, big_ms=0.0, big_segment=64)
        srv.submit(_req(1, 2500, 1500, 3000))  # 24 segments of 64 steps
        srv.submit(_req(3, *SPECS[3]))
        srv.submit(_req(9, 700, 2000, 20000))   # 32 segments
        srv.poll()
        while len(srv.big) < 3 and srv.pending:  # the preparation thread hands them over
            srv.poll()
        if preempt:
            assert srv.preempt(1) and srv.preempt(9)
        done = {d.rid: d for d in srv.drain()}
        srv.close()
        return srv, done

    srv0, want = serve(False)
    srv1, got = serve(True)
    assert srv0.preemptions == 0 and srv1.preemptions >= 2
    for i in (1, 3, 9):
        assert got[i].error is None
        np.testing.assert_array_equal(got[i].probes, want[i].probes)
        np.testing.assert_array_equal(got[i].fields["Ex"], want[i].fields["Ex"])
        np.testing.assert_array_equal(got[i].fields["Jx"], want[i].fields["Jx"])
        for k in ("cell", "frac", "ux", "uz"):
            np.testing.assert_array_equal(got[i].particles[k], want[i].particles[k])
    assert srv1.bytes_in_use == 0 and not srv1.parked
