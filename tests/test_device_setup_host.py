"""Host side of the device set-up (fdtdpic.device_setup): the batch layout equals what
fdtdpic.grid.pack makes of the per-grid host set-up, the batched plasma-frequency correction
equals the per-grid one to the last place, and the FdtdSetup layout matches the header."""
import numpy as np

from fdtdpic import _lib, device_setup as ds, sweep
from fdtdpic.grid import pack

GEOMETRY = ["nz", "n_steps", "step_begin", "step_end", "pml", "cpml_lo", "cpml_hi", "front",
            "rear", "nzsrc", "tfsf", "mode", "pol_active", "resume", "hist_interval",
            "hist_rows", "probe_cell", "probe_lo", "probe_hi", "pml_offset", "src_offset",
            "probe_offset", "state_offset", "hist_offset", "srcs_offset"]


def test_sweep_layout_matches_host_pack():
    spec = sweep.SweepSpec(n_inst=300, n_steps=1024)
    lay = ds.sweep_layout(spec)
    grids, dt = sweep.make_sweep_grids(spec)
    pk = pack(grids, 4)
    for f in GEOMETRY:
        np.testing.assert_array_equal(lay["desc"][f], pk["desc"][f], err_msg=f)
    np.testing.assert_array_equal(lay["src"], pk["src"])
    assert lay["n_state"] == pk["n_state"] and lay["n_probe"] == pk["n_probe"]
    assert lay["dt"] == dt
    np.testing.assert_array_equal(lay["records"]["plasma_freq"],
                                  np.array([g.plasma_freq for g in grids]))
    assert [s.cost() for s in lay["shapes"]] == [g.cost() for g in grids]


def test_setup_layout_matches_header():
    L = _lib.lib()
    n = L.fdtdpic_setup_layout(None, 0)
    out = np.zeros(n, np.int64)
    L.fdtdpic_setup_layout(out.ctypes.data, n)
    dt = _lib.SETUP_DTYPE
    assert out[0] == dt.itemsize
    assert list(out[1:]) == [dt.fields[f][1] for f in dt.names]
