"""fdtdpic_run_noalloc: the beam + field step for callers that cannot allocate device memory
(code inside another framework's memory pool, plug-ins in a host that reserved the device).

It must give what fdtdpic_run gives with caller scratch, bit for bit, call after call (the
compiled-in scratch array keeps the previous call's contents), on the one-CTA field kernel and
on the fused push-with-H launches, and refuse runs larger than its 24 MiB or on the tiled path.
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
# (nz, clo, chi): a 512-cell grid (one-CTA field kernel) and a 1536-cell grid with the beam
# inside its domain, whose push launches carry the previous step's H phase
CASES = {"nz512": (512, 40, 480), "nz1536_fused": (1536, 40, 1480)}


def _setup(precision, case="nz512"):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import scipy.constants as sc
    from fdtdpic.grid import lorentz_kerr_grid
    from fdtdpic.pic import PicRun, make_beam
    nz, clo, chi = CASES[case]
    g = lorentz_kerr_grid(nz, T, front=300, rear=400, nzsrc=60, probes=(50, 350), chi3=1e-2)
    beam = make_beam(NPART, clo, chi, DZ)
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


def _compare(a, b):
    """Both entry points run the same kernels with exact integer deposits: equal bits."""
    for k in ("Ex", "Hy", "Dx", "probes", "jx", "jz"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    for x, y in zip(a["parts"], b["parts"]):
        np.testing.assert_array_equal(x, y)
    assert a["status"][0] == 0 and b["status"][0] == 0


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_noalloc_matches_scratch_entry_point_twice(precision, case):
    torch, run = _setup(precision, case)
    run.reset()
    run.step(T)
    want = _snapshot(run)
    first = _noalloc_run(run)
    second = _noalloc_run(run)
    _compare(first, want)
    _compare(second, want)


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
    pb = type(run.pb).from_buffer_copy(run.pb)
    pb.path = 2  # the tiled path's scratch is not sized against the array
    rc = run.L.fdtdpic_run_noalloc(
        run.prec, d.ctypes.data, _ptr(run.d_desc), _ptr(run.d_table), _ptr(run.d_src),
        _ptr(run.d_state), _ptr(run.d_probe), ctypes.byref(pb), _ptr(run.d_cell),
        _ptr(run.d_frac), _ptr(run.d_ux), _ptr(run.d_uz), _ptr(run.d_id), _ptr(run.d_jx),
        _ptr(run.d_jz), _ptr(run.d_hyp), _ptr(run.d_status), None)
    assert rc == -1  # FDTDPIC_ERR_ARG
