"""Build and load libfdtdpic.so, the C-ABI library of hand-written sm_103a kernels.

There is no CPU fallback: if the library is missing or cannot be loaded, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes
import fcntl
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
# FDTDPIC_LIBRARY_VARIANT=bounds selects the index-checking debug build (libfdtdpic_bounds.so,
# compiled with FDTDPIC_BOUNDS_CHECK: data-dependent indices are checked before use and a failed
# check raises FDTD_STATUS_BOUNDS instead of touching memory); unset: the release build
VARIANT = os.environ.get("FDTDPIC_LIBRARY_VARIANT", "")
if VARIANT not in ("", "bounds"):
    raise RuntimeError(f"FDTDPIC_LIBRARY_VARIANT={VARIANT!r}: expected 'bounds' or unset")
_SUFFIX = "_bounds" if VARIANT == "bounds" else ""
BUILD_DIR = os.path.join(ROOT, "_build" + _SUFFIX)
LIB_PATH = os.path.join(PKG_DIR, f"libfdtdpic{_SUFFIX}.so")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
# translation unit -> extra nvcc flags
UNITS = {
    "capi.cu": [],
    "fdtd1d_f64.cu": ["-fmad=false"],
    "fdtd1d_f32.cu": [],
    "pic_f64.cu": ["-fmad=false"],
    "pic_f32.cu": ["-fmad=false"],  # PIC paths agree bit for bit (explicit fmaf in the push)
    "dft.cu": [],
    "dft_tc.cu": [],
    "slot.cu": ["-fmad=false"],  # beam requests round as fdtdpic_run's step
    "noalloc.cu": [],
    "setup.cu": ["-fmad=false"],  # set-up products and sums round one by one, as numpy's
    "variants.cu": ["-fmad=false"],  # the uncalled ADE variants, rounded as the reference's
    "stepops.cu": ["-fmad=false"],  # per-step module functions, rounded as the reference's
    "selftest.cu": [],  # the bounded waits' self-test
}


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _sources():
    return [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    deps.append(os.path.abspath(__file__))  # the units' nvcc flags
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every translation unit for sm_103a (in parallel) and link libfdtdpic.so.
    Processes building at once take turns (a lock file in the build folder): the object files
    have fixed names."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    with open(os.path.join(BUILD_DIR, ".lock"), "w") as lock:
        try:
            fcntl.flock(lock, fcntl.LOCK_EX)
        except OSError:  # a file system without locks: build unlocked, as a single process
            pass
        if not force and not _stale():  # another process built it meanwhile
            return LIB_PATH
        return _build_locked(verbose)


def _build_locked(verbose: bool) -> str:
    nvcc = _nvcc()
    common = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-I", INCLUDE, "-I", CSRC]
    if VARIANT == "bounds":
        common.append("-DFDTDPIC_BOUNDS_CHECK")

    def compile_one(unit):
        obj = os.path.join(BUILD_DIR, unit.replace(".cu", ".o"))
        cmd = [nvcc] + common + UNITS[unit] + ["-c", os.path.join(CSRC, unit), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    units = _sources()
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(compile_one, units))
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = [nvcc, ARCH, "-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


# ------------------------------------------------------------------------------------------
# FdtdInstance layout (include/fdtdpic.h)
# ------------------------------------------------------------------------------------------
_I4 = [("nz", "<i4"), ("n_steps", "<i4"), ("step_begin", "<i4"), ("step_end", "<i4"),
       ("pml", "<i4"), ("cpml_lo", "<i4"), ("cpml_hi", "<i4"), ("front", "<i4"),
       ("rear", "<i4"), ("nzsrc", "<i4"), ("tfsf", "<i4"), ("mode", "<i4"),
       ("pol_active", "<i4"), ("resume", "<i4"), ("hist_interval", "<i4"),
       ("hist_rows", "<i4"), ("probe_cell", "<i4", (2,)), ("probe_lo", "<i4", (2,)),
       ("probe_hi", "<i4", (2,))]
_F8 = [(n, "<f8") for n in ("ue", "ue_slab", "uh", "uh_slab", "dtdz", "eps0", "sc", "pol_a",
                            "pol_b", "pol_c", "kerr_a", "kerr_b", "kerr_c", "nl_e0", "nl_e0chi")]
_I8 = [(n, "<i8") for n in ("pml_offset", "src_offset", "probe_offset", "state_offset",
                            "hist_offset", "srcs_offset")]
INSTANCE_DTYPE = np.dtype(_I4 + _F8 + _I8, align=True)
INSTANCE_FIELDS = [f[0] for f in _I4 + _F8 + _I8]

# FdtdSetup (include/fdtdpic.h): the per-grid inputs of fdtdpic_setup_batch
SETUP_FIELDS = ["dz", "dt", "courant", "eps0", "mu0", "char_imp", "eps_re", "mu_re", "kappa_max",
                "sigma_opt", "alpha_max", "r_scale", "r_a_scale", "plasma_freq", "omega0",
                "gamma", "chi3", "alpha3", "freq_in"]
SETUP_DTYPE = np.dtype([(n, "<f8") for n in SETUP_FIELDS] + [("free_space", "<i4"),
                                                            ("reserved", "<i4")], align=True)

# FdtdVariantRow (include/fdtdpic.h): one row of fdtdpic_variant_run
VARIANT_FIELDS = ["c0", "dt", "dz", "eps0", "plasma_freq", "omega0", "gamma", "omega0_j", "chi1",
                  "chi3", "alpha3", "nl_gamma", "nl_omega0"]
VARIANT_DTYPE = np.dtype([(n, "<i4") for n in ("n", "nz", "front", "rear")] +
                         [(n, "<f8") for n in VARIANT_FIELDS], align=True)
VAR_MUR_EX, VAR_ADE_JX, VAR_VARIN_PBAR, VAR_VARIN_JP, VAR_VARIN_QG, VAR_VARIN_STEP = range(6)

MODE_FREESPACE, MODE_LINLOR, MODE_KERR = 0, 1, 2
F64, F32 = 8, 4
TAB_ROWS = 8
STATE_ARRAYS = 8
ST = dict(Ex=0, Hy=1, Dx=2, P=3, Pprev=4, psiE=5, psiH=6, A=7)
STATUS_NONFINITE, STATUS_SKIPPED = 1, 2

_lock = threading.Lock()
_lib = None


class FdtdPicError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        msg = _lib.fdtdpic_strerror(code).decode() if _lib is not None else str(code)
        super().__init__(f"{what}: {msg} ({code})" if what else f"{msg} ({code})")


def _declare(L):
    c_int, c_i64, P = ctypes.c_int, ctypes.c_int64, ctypes.c_void_p
    L.fdtdpic_abi_version.restype = c_int
    L.fdtdpic_abi_version.argtypes = []
    L.fdtdpic_strerror.restype = ctypes.c_char_p
    L.fdtdpic_strerror.argtypes = [c_int]
    L.fdtdpic_instance_layout.restype = c_int
    L.fdtdpic_instance_layout.argtypes = [P, c_int]
    L.fdtdpic_device_sms.restype = c_int
    L.fdtdpic_device_sms.argtypes = [P]
    L.fdtd1d_resident_smem_bytes.restype = c_i64
    L.fdtd1d_resident_smem_bytes.argtypes = [P, c_int]
    L.fdtd1d_run_batch.restype = c_int
    L.fdtd1d_run_batch.argtypes = [c_int, c_int] + [P] * 10 + [c_i64, c_int, c_int, P]
    L.fdtd1d_run_global.restype = c_int
    L.fdtd1d_run_global.argtypes = [c_int] + [P] * 9 + [P]
    L.fdtdpic_cubic_root0.restype = c_int
    L.fdtdpic_cubic_root0.argtypes = [c_int, P, P, P]
    L.fdtdpic_scratch_bytes.restype = c_i64
    L.fdtdpic_scratch_bytes.argtypes = [c_int, c_int, c_int]
    L.fdtdpic_pic_jscale.restype = ctypes.c_double
    L.fdtdpic_pic_jscale.argtypes = [P]
    L.fdtdpic_run.restype = c_int
    L.fdtdpic_run.argtypes = [c_int] + [P] * 16 + [c_i64, P, P, P]
    L.fdtdpic_pic_scratch_bytes.restype = c_i64
    L.fdtdpic_pic_scratch_bytes.argtypes = [c_int, P, P]
    L.fdtdpic_pass_plan.restype = c_int
    L.fdtdpic_pass_plan.argtypes = [c_int, P, P, c_i64, P, c_int]
    L.fdtdpic_dft_twiddle_bytes.restype = c_i64
    L.fdtdpic_dft_twiddle_bytes.argtypes = [c_int, c_int]
    L.fdtdpic_dft_twiddles.restype = c_int
    L.fdtdpic_dft_twiddles.argtypes = [P, c_int, c_int, ctypes.c_double, P, P]
    L.fdtdpic_dft_probes.restype = c_int
    L.fdtdpic_dft_probes.argtypes = [c_int, P, c_int, c_int, c_int, c_i64, c_i64, c_i64, P,
                                     c_int, P, P]
    L.fdtdpic_dft_tc_scratch_bytes.restype = c_i64
    L.fdtdpic_dft_tc_scratch_bytes.argtypes = [c_int, c_int, c_int]
    L.fdtdpic_dft_probes_tc.restype = c_int
    L.fdtdpic_dft_probes_tc.argtypes = [c_int, P, c_int, c_int, c_int, c_i64, c_i64, c_i64, P,
                                        c_int, P, P, c_i64, P, P]
    L.fdtdpic_reflection_ratio.restype = c_int
    L.fdtdpic_reflection_ratio.argtypes = [P, c_int, c_int, P, P]
    L.fdtdpic_slot_layout.restype = c_int
    L.fdtdpic_slot_layout.argtypes = [P, c_int]
    L.fdtdpic_setup_layout.restype = c_int
    L.fdtdpic_setup_layout.argtypes = [P, c_int]
    L.fdtdpic_setup_batch.restype = c_int
    L.fdtdpic_setup_batch.argtypes = [c_int, P, P, P, P]
    L.fdtdpic_variant_layout.restype = c_int
    L.fdtdpic_variant_layout.argtypes = [P, c_int]
    L.fdtdpic_variant_check.restype = c_int
    L.fdtdpic_variant_check.argtypes = [c_int, c_int, P, c_i64]
    L.fdtdpic_variant_run.restype = c_int
    L.fdtdpic_variant_run.argtypes = [c_int, c_int, c_int, P, P, c_i64, P, P]
    L.fdtdpic_slot_check.restype = c_int
    L.fdtdpic_slot_check.argtypes = [c_int, P]
    L.fdtdpic_slot_smem_bytes.restype = c_i64
    L.fdtdpic_slot_smem_bytes.argtypes = [c_int, P]
    L.fdtdpic_slots_grid.restype = c_int
    L.fdtdpic_slots_grid.argtypes = [c_int, c_i64, c_int]
    L.fdtdpic_slots_run.restype = c_int
    L.fdtdpic_slots_run.argtypes = [c_int, P, c_int, P, c_int, P, c_i64, c_int, c_int, P]
    L.fdtdpic_run_noalloc.restype = c_int
    L.fdtdpic_run_noalloc.argtypes = [c_int] + [P] * 17
    L.fdtdpic_step_op_layout.restype = c_int
    L.fdtdpic_step_op_layout.argtypes = [P, c_int]
    L.fdtdpic_step_op_check.restype = c_int
    L.fdtdpic_step_op_check.argtypes = [P, P, c_i64]
    L.fdtdpic_step_op.restype = c_int
    L.fdtdpic_step_op.argtypes = [P, P, c_i64, P]
    L.fdtdpic_set_run_deadline.restype = c_int
    L.fdtdpic_set_run_deadline.argtypes = [c_i64]
    L.fdtdpic_wait_selftest.restype = c_int
    L.fdtdpic_wait_selftest.argtypes = [c_int, c_i64, P, P, P]
    for name, argt in _EXTRA_DECLS.items():
        if hasattr(L, name):
            fn = getattr(L, name)
            fn.restype, fn.argtypes = argt


# filled by the modules that bind further entry points: name -> (restype, argtypes)
_EXTRA_DECLS: dict = {}


def declare(name, restype, argtypes):
    _EXTRA_DECLS[name] = (restype, argtypes)
    if _lib is not None and hasattr(_lib, name):
        fn = getattr(_lib, name)
        fn.restype, fn.argtypes = restype, argtypes


def lib(build_if_missing: bool = True):
    """Load libfdtdpic.so (building it first if it is missing or stale)."""
    global _lib
    with _lock:
        if _lib is None:
            if build_if_missing:
                build()
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"libfdtdpic.so not found at {LIB_PATH}; run build()")
            L = ctypes.CDLL(LIB_PATH)
            _declare(L)
            _check_layout(L)
            _lib = L
    return _lib


def _check_layout(L):
    n = L.fdtdpic_instance_layout(None, 0)
    out = np.zeros(n, np.int64)
    L.fdtdpic_instance_layout(out.ctypes.data, n)
    want = [INSTANCE_DTYPE.itemsize] + [INSTANCE_DTYPE.fields[f][1] for f in INSTANCE_FIELDS]
    if list(out) != want:
        raise RuntimeError(f"FdtdInstance layout mismatch: C {list(out)} vs numpy {want}")
    n = L.fdtdpic_variant_layout(None, 0)
    out = np.zeros(n, np.int64)
    L.fdtdpic_variant_layout(out.ctypes.data, n)
    want = [VARIANT_DTYPE.itemsize] + [VARIANT_DTYPE.fields[f][1] for f in VARIANT_DTYPE.names]
    if list(out) != want:
        raise RuntimeError(f"FdtdVariantRow layout mismatch: C {list(out)} vs numpy {want}")


def check(rc, what=""):
    if rc != 0:
        raise FdtdPicError(rc, what)
    return rc
