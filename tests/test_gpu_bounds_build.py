"""The index-checking debug build (libfdtdpic_bounds.so, FDTDPIC_BOUNDS_CHECK): every
data-dependent index of the beam kernels is checked before use and a failed check raises
FDTD_STATUS_BOUNDS instead of touching memory.  Beam runs on the streaming kernels (with a
ragged chunk, and with the push launches carrying the H phase), on the persistent
tiled kernel, and in FP64, run in a child process on that build: no check fails, and every
result equals the release build's bit for bit (the checks change no arithmetic)."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
STATUS_BOUNDS = 16
CASES = [("f32", 512, 40, 480, "streaming", 1022), ("f32", 1536, 40, 1480, "auto", 0),
         ("f32", 1536, 40, 1480, "tiled", 0), ("f64", 512, 40, 480, "streaming", 0)]


def run_cases():
    """The beam runs of CASES on whichever library this process loads."""
    import scipy.constants as sc
    import torch

    from fdtdpic.grid import lorentz_kerr_grid
    from fdtdpic.pic import PicRun, make_beam
    out = {}
    dz = 0.015
    for i, (prec, nz, clo, chi, path, chunk) in enumerate(CASES):
        g = lorentz_kerr_grid(nz, 300, front=300, rear=400, nzsrc=60, probes=(50, 350),
                              chi3=1e-2)
        beam = make_beam(20003, clo, chi, dz)
        run = PicRun(g, beam, dz, 0.5 * dz / 299792458.0, sc.mu_0, precision=prec, chunk=chunk,
                     path=path)
        run.step(300)
        torch.cuda.synchronize()
        f = run.fields()
        cell, frac, ux, uz = run.particles()
        out.update({f"{i}_Ex": f["Ex"], f"{i}_Hy": f["Hy"], f"{i}_cell": cell, f"{i}_frac": frac,
                    f"{i}_ux": ux, f"{i}_status": run.status()})
    return out


def test_bounds_checked_build_finds_nothing_and_changes_nothing(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    out = tmp_path / "bounds.npz"
    child = (f"import sys; sys.path[:0] = [{HERE!r}, {ROOT!r}, {os.path.join(ROOT, 'py-fdtd_pic_gb300')!r}]\n"
             "import numpy as np, test_gpu_bounds_build as t\n"
             f"np.savez({str(out)!r}, **t.run_cases())\n")
    env = dict(os.environ, FDTDPIC_LIBRARY_VARIANT="bounds")
    r = subprocess.run([sys.executable, "-c", child], env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    got = np.load(out)
    want = run_cases()
    for i in range(len(CASES)):
        assert (int(got[f"{i}_status"][1]) & STATUS_BOUNDS) == 0, CASES[i]
        assert int(got[f"{i}_status"][0]) == 0
    for k, v in want.items():
        np.testing.assert_array_equal(got[k], v, err_msg=k)
    from fdtdpic import _lib
    assert _lib.VARIANT == ""  # this process used the release build
