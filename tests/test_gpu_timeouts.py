"""Bounded device-side waits give up, report, and leave the context usable.

* The tiled kernel's neighbour-flag wait and the tensor-core DFT's mbarrier wait, each run alone
  on something nothing completes (fdtdpic_wait_selftest): both report FDTDPIC_ERR_TIMEOUT.
* A whole persistent tiled run given a deadline of one microsecond (fdtdpic_set_run_deadline):
  its CTAs stop at their first wait, the call returns, the status word carries
  FDTD_STATUS_TIMEOUT, and the next run with the default deadline gives the same bits as a run
  that never met a timeout."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

ERR_TIMEOUT = -3
STATUS_TIMEOUT = 4


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _selftest(which, limit):
    torch = _torch()
    from fdtdpic._lib import check, lib
    L = lib()
    out = torch.full((2,), 7, dtype=torch.int32, device="cuda")
    scr = torch.ones(2, dtype=torch.int32, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    check(L.fdtdpic_wait_selftest(which, limit, ctypes.c_void_p(out.data_ptr()),
                                  ctypes.c_void_p(scr.data_ptr()), st))
    torch.cuda.synchronize()
    return [int(v) for v in out.cpu()]


def test_neighbour_flag_wait_gives_up_at_its_deadline():
    code, us = _selftest(0, 2_000_000)  # 2 ms
    assert code == ERR_TIMEOUT
    assert 2000 <= us < 1_000_000


def test_mbarrier_wait_gives_up_after_its_polls():
    code, _ = _selftest(1, 4096)
    assert code == ERR_TIMEOUT


def test_selftest_refuses_long_waits():
    """Limits above 2 s or 2^26 polls are refused before anything is launched."""
    torch = _torch()
    from fdtdpic._lib import lib
    L = lib()
    out = torch.zeros(2, dtype=torch.int32, device="cuda")
    scr = torch.zeros(2, dtype=torch.int32, device="cuda")
    p, q = ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(scr.data_ptr())
    assert L.fdtdpic_wait_selftest(0, 10_000_000_000, p, q, None) != 0
    assert L.fdtdpic_wait_selftest(1, 1 << 30, p, q, None) != 0
    assert L.fdtdpic_wait_selftest(2, 10, p, q, None) != 0
    assert L.fdtdpic_wait_selftest(0, 1000, p, None, None) != 0


def _tiled_run():
    import scipy.constants as sc
    from fdtdpic.grid import lorentz_kerr_grid
    from fdtdpic.pic import PicRun, make_beam
    nz, T = 1536, 300
    dz = 0.015
    g = lorentz_kerr_grid(nz, T, front=300, rear=400, nzsrc=60, probes=(50, 350), chi3=1e-2)
    beam = make_beam(20000, 40, 1480, dz)
    return PicRun(g, beam, dz, 0.5 * dz / O.C0, sc.mu_0, precision="f32", path="tiled")


def test_tiled_run_past_its_deadline_reports_timeout_and_recovers():
    torch = _torch()
    from fdtdpic._lib import check, lib
    L = lib()
    want = _tiled_run()
    want.step(300)
    torch.cuda.synchronize()
    assert int(want.status()[1]) == 0
    try:
        check(L.fdtdpic_set_run_deadline(1000))  # 1 us: gone before the first handshake
        late = _tiled_run()
        late.step(300)
        torch.cuda.synchronize()  # the call returned and its kernels finished
        assert int(late.status()[1]) & STATUS_TIMEOUT
    finally:
        check(L.fdtdpic_set_run_deadline(0))
    again = _tiled_run()
    again.step(300)
    torch.cuda.synchronize()
    assert int(again.status()[1]) == 0
    np.testing.assert_array_equal(again.fields()["Ex"], want.fields()["Ex"])
    np.testing.assert_array_equal(again.probes(), want.probes())
    for a, b in zip(again.particles(), want.particles()):
        np.testing.assert_array_equal(a, b)
