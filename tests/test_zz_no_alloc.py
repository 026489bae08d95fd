"""fdtdpic_run_noalloc: the beam + field step for callers that cannot allocate device memory
(code inside another framework's memory pool, plug-ins in a host that reserved the device).

It must give what fdtdpic_run gives with caller scratch, call after call (the compiled-in
scratch array keeps the previous call's contents), and refuse runs larger than its 24 MiB.
This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

NZ, T, NPART = 512, 400, 20000
DZ = 0.015
DT = 0.5 * DZ / O.C0


def _setup(precision):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import scipy.constants as sc
    from fdtdpic.grid import lorentz_kerr_grid
    from fdtdpic.pic import PicRun, make_beam
    g = lorentz_kerr_grid(NZ, T, front=300, rear=400, nzsrc=60, probes=(50, 350), chi3=1e-2)
    beam = make_beam(NPART, 40, 480, DZ)
    return torch, PicRun(g, beam, DZ, DT, sc.mu_0, precision=precision, sort_every=32)


def _noalloc_run(run):
    """One whole run through the no-allocation entry point, on run's own buffers."""
    from fdtdpic.engine import _ptr
    run.reset()
    d = run.desc.copy()
    d["step_begin"], d["step_end"], d["resume"] = 0, run.grid.n_steps, 0
    run.d_desc.copy_(torch_from(d))
    L = run.L
    rc = L.fdtdpic_run_noalloc(
        run.prec, d.ctypes.data, _ptr(run.d_desc), _ptr(run.d_table), _ptr(run.d_src),
        _ptr(run.d_state), _ptr(run.d_probe), ctypes.byref(run.pb), _ptr(run.d_cell),
        _ptr(run.d_frac), _ptr(run.d_ux), _ptr(run.d_uz), _ptr(run.d_id), _ptr(run.d_jx),
        _ptr(run.d_jz), _ptr(run.d_hyp), _ptr(run.d_status),
        ctypes.c_void_p(__import__("torch").cuda.current_stream().cuda_stream))
    assert rc == 0, L.fdtdpic_strerror(rc)
    return _snapshot(run)


def torch_from(d):
    import torch
    return torch.from_numpy(d.view(np.uint8).copy())


def _snapshot(run):
    import torch
    torch.cuda.synchronize()
    f = run.fields()
    jx, jz = run.currents()
    return dict(Ex=f["Ex"], Hy=f["Hy"], Dx=f["Dx"], probes=run.probes(), jx=jx, jz=jz,
                parts=run.particles(), status=run.status().copy())


def _compare(a, b, tol):
    for k in ("Ex", "Hy", "Dx", "probes", "jx", "jz"):
        assert O.rel_l2(a[k], b[k]) <= tol, k
    for x, y in zip(a["parts"], b["parts"]):
        assert O.rel_l2(x, y) <= tol
    assert a["status"][0] == 0 and b["status"][0] == 0


@pytest.mark.parametrize("precision,tol", [("f32", 1e-6), ("f64", 1e-12)])
def test_noalloc_matches_scratch_entry_point_twice(precision, tol):
    torch, run = _setup(precision)
    run.reset()
    run.step(T)
    want = _snapshot(run)
    first = _noalloc_run(run)
    second = _noalloc_run(run)
    _compare(first, want, tol)
    _compare(second, want, tol)


def test_noalloc_rejects_runs_beyond_its_scratch():
    torch, run = _setup("f32")
    from fdtdpic.engine import _ptr
    need = run.L.fdtdpic_scratch_bytes(4, NZ, 2_000_000)
    assert need > 24 << 20
    pb = type(run.pb).from_buffer_copy(run.pb)
    pb.n_part = 2_000_000
    d = run.desc.copy()
    rc = run.L.fdtdpic_run_noalloc(
        run.prec, d.ctypes.data, _ptr(run.d_desc), _ptr(run.d_table), _ptr(run.d_src),
        _ptr(run.d_state), _ptr(run.d_probe), ctypes.byref(pb), _ptr(run.d_cell),
        _ptr(run.d_frac), _ptr(run.d_ux), _ptr(run.d_uz), _ptr(run.d_id), _ptr(run.d_jx),
        _ptr(run.d_jz), _ptr(run.d_hyp), _ptr(run.d_status), None)
    assert rc == -2  # FDTDPIC_ERR_OOM, before anything is launched
