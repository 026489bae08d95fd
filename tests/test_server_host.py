"""Serving layer on the host: the slot descriptor layout, the slot check, the request stream."""
import ctypes

import numpy as np


def test_slot_layout_matches_header():
    from fdtdpic import server
    server.check_slot_layout()


def _slot(nz=300, n_part=0):
    from fdtdpic import server
    from fdtdpic.grid import lorentz_kerr_grid, pack
    g = lorentz_kerr_grid(nz, 64, front=150, rear=200, nzsrc=60, probes=(50, 250))
    s = np.zeros(1, server.SLOT_DTYPE)
    s["inst"] = pack([g], 4)["desc"][0]
    for k in ("pml_tab", "src", "state", "probe"):
        s[k] = 4096
    if n_part:
        s["n_part"], s["clo"], s["chi"] = n_part, 40, nz - 40
        for k in ("cell", "frac", "ux", "uz", "hyp", "jx", "jz", "acc"):
            s[k] = 4096
        s["jscale"], s["sc"] = 2.0 ** 40, 0.5
    return s


def test_slot_check_accepts_and_rejects():
    from fdtdpic._lib import lib
    L = lib()
    assert L.fdtdpic_slot_check(4, _slot().ctypes.data) == 0
    assert L.fdtdpic_slot_check(4, _slot(n_part=100).ctypes.data) == 0
    s = _slot(n_part=100)
    s["chi"] = 299  # beam domain must end by nz - 2
    assert L.fdtdpic_slot_check(4, s.ctypes.data) != 0
    s = _slot(n_part=100)
    s["acc"] = 0
    assert L.fdtdpic_slot_check(4, s.ctypes.data) != 0
    s = _slot()
    s["probe"] = 0
    assert L.fdtdpic_slot_check(4, s.ctypes.data) != 0
    assert L.fdtdpic_slot_check(3, _slot().ctypes.data) != 0
    # size limits (FDTDPIC_MAX_PARTICLES, FDTDPIC_MAX_CELLS = 2^30)
    assert L.fdtdpic_slot_check(4, _slot(n_part=(1 << 30) + 1).ctypes.data) == -1
    assert L.fdtdpic_slot_check(4, _slot(n_part=1 << 30).ctypes.data) == 0
    s = _slot()
    s["inst"]["nz"] = (1 << 30) + 1
    assert L.fdtdpic_slot_check(4, s.ctypes.data) == -1
    # shared memory: field-only slots need their resident arrays, beam slots their accumulators
    assert L.fdtdpic_slot_smem_bytes(4, _slot(n_part=100).ctypes.data) == 2 * 301 * 8
    assert L.fdtdpic_slot_smem_bytes(8, _slot(n_part=100).ctypes.data) == 4 * 301 * 8
    assert L.fdtdpic_slot_smem_bytes(4, _slot().ctypes.data) > 2 * 301 * 4


def test_request_stream_shapes():
    from fdtdpic import server
    reqs = server.make_request_stream(rate=2000.0, duration=2.0, seed=5)
    assert 3700 < len(reqs) < 4300  # Poisson(4000)
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) > 0) and arr[-1] < 2.0
    nz = np.array([r.nz for r in reqs])
    steps = np.array([r.n_steps for r in reqs])
    npart = np.array([r.n_part for r in reqs])
    assert nz.min() >= 256 and nz.max() <= 65536
    assert steps.min() >= 1000 and steps.max() <= 50000
    assert npart.min() == 0 and npart.max() <= 2_000_000
    # log-uniform sizes: median near the geometric mean of the range
    assert 2500 < np.median(nz) < 6500
    assert 0.02 < np.mean(npart == 0) < 0.09
    g = reqs[0].grid_fn()  # grids are built on admission
    assert g.nz == reqs[0].nz and g.n_steps == reqs[0].n_steps
    assert g.front >= 102 and g.rear <= g.nz - 22


def test_streaming_limit_drops_while_requests_wait():
    from fdtdpic.server import streaming_limit
    # an idle server lets big requests use the GPU with many streaming runs ...
    assert streaming_limit(False, True, 8, 2) == 8
    # ... but while prepared requests wait for a slot, or every slot is taken, the slot rounds
    # need the SMs
    assert streaming_limit(True, True, 8, 2) == 2
    assert streaming_limit(False, False, 8, 2) == 2
    assert streaming_limit(True, False, 8, 2) == 2


def test_streaming_request_budget_counts_its_scratch():
    """A 2M-particle request run on the streaming kernels holds its re-binning copies and
    deposit accumulators besides its own buffers: admission counts them, so with other requests
    resident a budget between the two totals refuses it."""
    from fdtdpic._lib import lib
    from fdtdpic.server import fits_budget, slot_request_bytes, streaming_request_bytes
    L = lib()
    nz, T, n_part = 65536, 50000, 2_000_000
    for prec in (4, 8):
        slot = slot_request_bytes(prec, nz, T, n_part, 20)
        full = streaming_request_bytes(prec, nz, T, n_part, 20, L)
        scratch = int(L.fdtdpic_scratch_bytes(prec, nz, n_part))
        assert scratch >= n_part * (8 + 3 * prec)  # a second copy of every particle array
        assert full >= slot + scratch
        budget = (slot + full) // 2
        assert fits_budget(0, slot, budget, True)
        assert not fits_budget(0, full, budget, True)
        # a request larger than the whole budget still runs when nothing else is resident
        assert fits_budget(0, full, budget, False)
        assert not fits_budget(budget - 10, 11, budget, True)


def test_status_words_map_to_errors():
    from fdtdpic.server import status_error
    assert status_error(np.zeros(4, np.int32)) is None
    assert status_error(np.array([0, 0, 7, 0])) is None  # FP64 cubic re-solves are no error
    assert "non-finite" in status_error(np.array([0, 1, 0, 0]))
    assert "bounded wait" in status_error(np.array([0, 4, 0, 0]))
    assert "3 particles left" in status_error(np.array([3, 0, 0, 0]))
