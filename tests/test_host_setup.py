"""Host-side set-up of the product (fdtdpic.physics_setup / fdtdpic.grid) against the
reference's own outputs, and the C-ABI library's exports.  No GPU needed."""
import ctypes
import os
import re

import numpy as np
import pytest

from helpers import RUN_CASES, integrator_of, load, ref_objects, sources_of

from fdtdpic import _lib
from fdtdpic import physics_setup as ps
from fdtdpic.grid import grids_from_reference, pack

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("name", RUN_CASES)
def test_pml_table_and_scalars_match_reference(name):
    g = load(name)
    P, V, C_P = ref_objects(g)
    Exs, Hys = sources_of(g)
    grids = grids_from_reference(P, V, C_P, integrator_of(g), Exs=Exs, Hys=Hys)
    n, pml = P.Nz + 1, P.pmlWidth
    cols = np.r_[0:pml + 1, n - pml:n]
    rows = ("beX", "ceX", "Cb", "bmY", "cmY", "C2", "den_Exdz", "den_Hydz")
    for gr in grids:
        for r, key in enumerate(rows):
            np.testing.assert_array_equal(gr.table[r], g[key][cols], err_msg=key)
        # outside the table columns the reference arrays are the bulk values
        mask = np.ones(n, bool)
        mask[cols] = False
        for key, bulk in (("beX", 0), ("ceX", 0), ("Cb", 0), ("C2", 0), ("den_Exdz", 1),
                          ("den_Hydz", 1)):
            assert np.all(g[key][mask] == bulk), key
    # plasma frequency after the spatialStab rescale(s) the integrator applies
    assert grids[-1].plasma_freq == pytest.approx(float(g["plasmaFreqE_out"]), rel=1e-15)
    if not bool(g["source_supplied"]):
        np.testing.assert_allclose(grids[-1].exs, g["Exs"], rtol=0, atol=1e-13)
        np.testing.assert_allclose(grids[-1].hys, g["Hys"], rtol=0, atol=1e-13)


def test_env_mat_setup_match_reference():
    g = load("setup")
    for args, want in zip(g["env_in"], g["env_out"]):
        f, dom, lo, hi, nl = args
        got = ps.env_setup(f, dom, int(lo), int(hi), nonLinMed=bool(nl))
        np.testing.assert_allclose(np.array(got, float), want, rtol=1e-15, atol=0)
    for args, want in zip(g["mat_in"], g["mat_out"]):
        got = ps.mat_setup(None, None, None, None, args[0], args[1], int(args[2]), int(args[3]))
        np.testing.assert_allclose(np.array(got, float), want, rtol=1e-15, atol=0)
    for args, want in zip(g["stab_in"], g["stab_out"]):
        got = ps.spatial_stab(*[a.item() for a in args])
        np.testing.assert_allclose(np.real(np.array(got, complex)), want, rtol=1e-14, atol=0)


def test_stability_exit_like_reference():
    # a step that resolves the frequency too coarsely: the reference prints and sys.exit()s
    with pytest.raises(SystemExit):
        ps.spatial_stab(100, 1000, 0.015, 1e9, 1e-9, 1e10, 1e10, 1e9)


def test_library_loads_and_exports_header_symbols():
    L = _lib.lib()
    header = open(os.path.join(ROOT, "include", "fdtdpic.h")).read()
    # every function the header declares, whatever it returns
    names = re.findall(r"^\s*[A-Za-z_][\w ]*?[\w*]\s+\**\s*((?:fdtdpic|fdtd1d)_\w+)\s*\(",
                       header, re.M)
    assert len(names) >= 34 and "fdtdpic_pic_jscale" in names
    for n in names:
        assert hasattr(L, n), n
    assert L.fdtdpic_abi_version() == 2
    assert L.fdtdpic_strerror(-1) == b"invalid argument"


def test_instance_layout_matches_numpy():
    L = _lib.lib()
    n = L.fdtdpic_instance_layout(None, 0)
    out = np.zeros(n, np.int64)
    L.fdtdpic_instance_layout(out.ctypes.data, n)
    assert out[0] == _lib.INSTANCE_DTYPE.itemsize


def test_resident_smem_sizes():
    g = load("kerr_nz1000")
    P, V, C_P = ref_objects(g)
    gr = grids_from_reference(P, V, C_P, "IntegratorNL1D", *sources_of(g))[0]
    d = pack([gr], 8)["desc"]
    L = _lib.lib()
    b64 = L.fdtd1d_resident_smem_bytes(d.ctypes.data, 8)
    b32 = L.fdtd1d_resident_smem_bytes(d.ctypes.data, 4)
    W = 2 * 20 + 1
    assert b64 == 8 * (2 * 1001 + 200 + 2 * W + 8 * W)
    assert b32 * 2 == b64
    # invalid precision and out-of-range geometry are rejected, not run
    assert L.fdtd1d_resident_smem_bytes(d.ctypes.data, 3) == 0
    bad = d.copy()
    bad["rear"] = 5000
    assert L.fdtd1d_resident_smem_bytes(bad.ctypes.data, 8) == 0


def _prototypes(header):
    """name -> number of parameters, for every function declared in a C header."""
    src = re.sub(r"/\*.*?\*/", "", header, flags=re.S)
    out = {}
    for m in re.finditer(r"^\s*(?:const\s+)?\w+\s*\**\s*(\w+)\s*\(([^;{]*?)\)\s*;", src, re.M):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_bindings_match_header_arity():
    L = _lib.lib()
    protos = {}
    for h in os.listdir(os.path.join(ROOT, "include")):
        protos.update(_prototypes(open(os.path.join(ROOT, "include", h)).read()))
    assert protos
    for name, nargs in protos.items():
        fn = getattr(L, name)
        assert fn.argtypes is not None, f"{name} has no ctypes binding"
        assert len(fn.argtypes) == nargs, f"{name}: binding {len(fn.argtypes)} vs header {nargs}"
