"""Checkpoint and resume of a beam run: run(N) equals run(k), snapshot to the host, restore into
a fresh run of the same grid and beam, run(N - k), bit for bit (fields, psi, P, Acubic, Hy one
half step back, probe traces, currents, particles), in FP32 and FP64, on the streaming kernels
(with and without the fused push-with-H launches) and on the persistent tiled kernel.

The reference keeps only in-memory histories (Ex_History every vidInterval steps,
MasterController.py:160-166, Solver_Engine.py:57-68); nothing there resumes a run."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

T, NPART, DZ = 600, 20000, 0.015
DT = 0.5 * DZ / O.C0
# (nz, clo, chi, path): the one-CTA field kernel, the fused push-with-H launches, the tiled kernel
CASES = {"nz512": (512, 40, 480, "streaming"), "nz1536_fused": (1536, 40, 1480, "auto"),
         "nz1536_tiled": (1536, 40, 1480, "tiled")}


def _run(precision, case):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import scipy.constants as sc
    from fdtdpic.grid import lorentz_kerr_grid
    from fdtdpic.pic import PicRun, make_beam
    nz, clo, chi, path = CASES[case]
    g = lorentz_kerr_grid(nz, T, front=300, rear=400, nzsrc=60, probes=(50, 350), chi3=1e-2)
    beam = make_beam(NPART, clo, chi, DZ)
    return torch, PicRun(g, beam, DZ, DT, sc.mu_0, precision=precision, sort_every=32, path=path)


def _all(run):
    import torch
    torch.cuda.synchronize()
    jx, jz = run.currents()
    return dict(state=run.d_state.cpu().numpy(), hyp=run.d_hyp.cpu().numpy(), jx=jx, jz=jz,
                probes=run.probes(), parts=run.particles(), status=run.status())


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_snapshot_restore_equals_uninterrupted_run(precision, case):
    torch, whole = _run(precision, case)
    whole.step(T)
    want = _all(whole)
    del whole
    _, first = _run(precision, case)
    first.step(250)
    snap = first.snapshot()
    first.step(100)  # the source run moves on; the snapshot keeps step 250
    del first
    _, second = _run(precision, case)
    second.restore(snap)
    assert second.step_done == 250
    second.step(T - 250)
    got = _all(second)
    assert int(got["status"][0]) == 0 and int(got["status"][1]) == 0
    for k in ("state", "hyp", "jx", "jz", "probes"):
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    for a, b in zip(got["parts"], want["parts"]):
        np.testing.assert_array_equal(a, b)
    assert snap.nbytes() > 0


@pytest.mark.parametrize("case", ["nz512", "nz1536_fused"])
def test_calls_on_a_side_stream_equal_one_call(case):
    """step(n, stream=s) calls queued back to back on a stream other than the current one, with
    no host wait between them: each call's descriptor (its step range) goes in on s, behind the
    previous call's kernels, so the run equals one call on the current stream bit for bit."""
    torch, whole = _run("f32", case)
    whole.step(T)
    want = _all(whole)
    del whole
    _, run = _run("f32", case)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())  # the run's buffers were set up on this one
    for n in (100, 37, 200, 263):
        run.step(n, stream=s)
    assert run.step_done == T
    got = _all(run)
    for k in ("state", "hyp", "jx", "jz", "probes"):
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    for a, b in zip(got["parts"], want["parts"]):
        np.testing.assert_array_equal(a, b)


def test_restore_refuses_another_shape():
    torch, a = _run("f32", "nz512")
    _, b = _run("f64", "nz512")
    with pytest.raises(ValueError):
        b.restore(a.snapshot())
