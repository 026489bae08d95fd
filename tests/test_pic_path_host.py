"""Host side of the beam step's path selection (no GPU): PicRun sets FDTDPIC_PATH_CELLS_INSIDE
exactly when every cell of its host beam lies in [clo, chi), and fdtdpic_run refuses path words
with unknown bits or an unknown path, and temporally blocked passes (mode 3) whose tiling does not
apply, before any device work (its device pointers here are placeholders that a refused call never
reads)."""
import ctypes
from types import SimpleNamespace

import numpy as np


def test_cells_inside_flag_follows_the_host_beam():
    from fdtdpic.pic import PATH_CELLS_INSIDE, PicBeam, PicRun, make_beam
    b = make_beam(500, 40, 480, 0.015)
    for mode in (0, 1, 2):
        obj = SimpleNamespace(pb=PicBeam(), path_mode=mode)
        PicRun._set_inside(obj, b)
        assert obj.pb.path == mode | PATH_CELLS_INSIDE
    obj = SimpleNamespace(pb=PicBeam(), path_mode=1)
    for bad in (39, 480, -5, 10_000):
        c = b.cell.copy()
        c[7] = bad
        PicRun._set_inside(obj, SimpleNamespace(cell=c, clo=b.clo, chi=b.chi))
        assert obj.pb.path == 1, bad
    PicRun._set_inside(obj, SimpleNamespace(cell=np.zeros(0, np.int32), clo=40, chi=480))
    assert obj.pb.path == 1 | PATH_CELLS_INSIDE


def test_run_refuses_unknown_path_bits():
    from fdtdpic import _lib
    from fdtdpic.grid import lorentz_kerr_grid, pack
    from fdtdpic.pic import PicBeam
    L = _lib.lib()
    g = lorentz_kerr_grid(512, 64, front=300, rear=400, nzsrc=60, probes=(50, 350))
    desc = pack([g], 4)["desc"]
    fake = ctypes.c_void_p(256)  # never dereferenced: every call below is refused first

    def run(path, scratch_bytes):
        pb = PicBeam()
        pb.n_part, pb.clo, pb.chi, pb.sort_every = 0, 40, 480, 32
        pb.sc, pb.jscale, pb.path = 0.5, 1.0, path
        return L.fdtdpic_run(_lib.F32, desc.ctypes.data, fake, fake, fake, fake, fake,
                             ctypes.byref(pb), None, None, None, None, None, fake, fake, fake,
                             fake, scratch_bytes, fake, None, None)

    # 32, 15, -1: bits outside the mode and the CELLS_INSIDE flag; 3: passes without the flag;
    # 16 | 3: passes over an empty beam, which have no tiling
    for path in (32, 3, 15, 16 | 3, -1):
        assert run(path, 0) == -1, path  # FDTDPIC_ERR_ARG
    # accepted path words get past that check to the scratch-size check (FDTDPIC_ERR_OOM),
    # which also comes before any device work
    for path in (0, 1, 16, 16 | 1):
        assert run(path, 0) == -2, path


def test_run_refuses_sizes_beyond_the_limits():
    """FDTDPIC_MAX_PARTICLES and FDTDPIC_MAX_CELLS (2^30 each): larger beams and grids are
    refused with FDTDPIC_ERR_ARG before any device work; at the limits the call gets on to the
    scratch-size check."""
    from fdtdpic import _lib
    from fdtdpic.grid import lorentz_kerr_grid, pack
    from fdtdpic.pic import PicBeam
    L = _lib.lib()
    g = lorentz_kerr_grid(512, 64, front=300, rear=400, nzsrc=60, probes=(50, 350))
    desc = pack([g], 4)["desc"]
    fake = ctypes.c_void_p(256)  # never dereferenced: every call below stops at a host check

    def run(d, n_part):
        pb = PicBeam()
        pb.n_part, pb.clo, pb.chi, pb.sort_every = n_part, 40, 480, 32
        pb.sc, pb.jscale, pb.path = 0.5, 1.0, 1
        return L.fdtdpic_run(_lib.F32, d.ctypes.data, fake, fake, fake, fake, fake,
                             ctypes.byref(pb), fake, fake, fake, fake, fake, fake, fake, fake,
                             fake, 0, fake, None, None)

    assert run(desc, (1 << 30) + 1) == -1
    assert run(desc, 1 << 30) == -2
    big = desc.copy()
    big["nz"] = (1 << 30) + 1
    assert run(big, 100) == -1
    big["nz"] = 1 << 30
    assert run(big, 100) == -2


def _plan(nz=8191, clo=40, chi=8189, ppc=4, **kw):
    from fdtdpic.grid import lorentz_kerr_grid
    from fdtdpic.pic import make_beam, pass_plan
    g = lorentz_kerr_grid(nz, 64, front=nz // 4, rear=3 * nz // 4, nzsrc=60, probes=(50, nz // 2))
    beam = make_beam(ppc * (chi - clo), clo, chi, 0.015)
    return pass_plan(g, beam, **kw)


def test_pass_plan_tiles_a_long_grid():
    """fdtdpic_pass_plan on the host: 8192 nodes in 512-cell tiles, 8 steps a pass (halo
    3 x 8 + 4 = 28 cells), the FP32 Kerr CTA holding both wrap tiles within GB300's 227 KiB of
    shared memory; the defaults (0, 0) are 8 steps and 512 cells; longer passes are cut to 32."""
    p = _plan(pass_steps=8, tile_cells=512)
    assert p is not None
    assert (p["steps"], p["halo"], p["tiles"], p["wmin"], p["wmax"]) == (8, 28, 16, 512, 512)
    assert p["loaded"] == 512 + 2 * 28
    assert p["particles_per_range"] >= 4 * p["loaded"]
    assert 0 < p["smem_one_tile"] < p["smem_wrap_pair"] <= 232448 - 1024
    assert p["scratch_bytes"] > 0
    assert _plan() == p
    assert _plan(pass_steps=64, tile_cells=512)["steps"] == 32


def test_pass_plan_refusals():
    """The conditions under which the pass path refuses a run, each alone."""
    assert _plan(pass_steps=8, tile_cells=512) is not None
    assert _plan(ppc=0) is None                                  # an empty beam
    assert _plan(pass_steps=8, tile_cells=40) is None            # tiles narrower than 2H = 56
    assert _plan(nz=2047, chi=2045) is None                      # four tiles: fewer than five
    assert _plan(clo=500) is None                                # clo 12 cells from its tile's edge
    assert _plan(chi=700) is None                                # the wrap tiles 2H apart at most
    assert _plan(smem_optin=48 * 1024) is None                   # shared memory too small
    # FP64 state and particles take twice the room: 256-cell tiles fit, 512-cell ones do not
    assert _plan(precision="f64") is None
    assert _plan(precision="f64", tile_cells=256) is not None
