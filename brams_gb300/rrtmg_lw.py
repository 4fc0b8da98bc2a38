"""Python front end of the GB300 RRTMG_LW library (ctypes over include/gb_rrtmg_lw.h).

Mirrors the reference's routines with the same names, argument meaning and
Fortran layouts:

* ``rrtmg_lw_ini(cpdair)``       -- rrtmg_lw_init.f90:47
* ``rrtmg_lw(...)``              -- rrtmg_lw_rad.f90:99-108 (host numpy arrays)
* ``rrtmg_lw_device(...)``       -- same on device pointers (e.g. torch CUDA tensors)
* ``mcica_subcol_lw(...)``       -- mcica_subcol_gen_lw.f90:183-185

Arrays are numpy arrays in Fortran order with the reference's shapes, e.g.
``play`` is (ncol, nlay), ``cldfmcl`` is (140, ncol, nlay).  Reference STOP
conditions raise ``RrtmgLwError`` carrying the reference's message.  There is
no CPU fallback: if the CUDA library cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgb_rrtmg_lw.so")
DATA_DIR = os.path.join(HERE, "data")

STATE_ORDER = ["play", "plev", "tlay", "tlev", "tsfc", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr",
               "n2ovmr", "o2vmr", "cfc11vmr", "cfc12vmr", "cfc22vmr", "ccl4vmr", "emis"]
CLOUD_ORDER = ["cldfmcl", "taucmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl"]
OUT_ORDER = ["uflx", "dflx", "hr", "uflxc", "dflxc", "hrc", "duflx_dt", "duflxc_dt"]

# C prototypes (see include/gb_rrtmg_lw.h)
EXPORTS = [
    "gb_rrtmg_lw_ini", "gb_rrtmg_lw_free", "gb_rrtmg_lw", "gb_rrtmg_lw_device",
    "gb_rrtmg_lw_sync_status", "gb_mcica_subcol_lw", "gb_mcica_subcol_lw_device",
    "gb_rrtmg_lw_strerror", "gb_rrtmg_lw_last_error", "gb_rrtmg_lw_gas_optics_diag",
    "gb_mcica_subcol_lw_noalloc",
]


class RrtmgLwError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"rrtmg_lw status {code}: {msg}")
        self.code = code


_lib = None
_lock = threading.Lock()


def load_library(path: str = LIB_PATH):
    """Load the CUDA library; raises if it is missing (there is no fallback)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(f"GB300 RRTMG_LW library not built: {path} (run brams_gb300/build.py)")
        L = C.CDLL(path)
        P, I, D, LL = C.c_void_p, C.c_int, C.c_double, C.c_int64
        IP = C.POINTER(C.c_int)
        L.gb_rrtmg_lw_ini.argtypes = [D, C.c_char_p, I, C.POINTER(P)]
        L.gb_rrtmg_lw_free.argtypes = [P]
        L.gb_rrtmg_lw.argtypes = [P, I, I, IP, I] + [P] * 16 + [I, I, I] + [P] * 7 + [P] * 8 + [LL, LL]
        L.gb_rrtmg_lw_device.argtypes = [P, P, I, I, IP, I] + [P] * 16 + [I, I, I] + [P] * 7 + [P] * 8 + [LL, LL, P]
        L.gb_rrtmg_lw_sync_status.argtypes = [P, P]
        L.gb_mcica_subcol_lw.argtypes = [P, I, I, I, I, IP] + [P] * 8 + [P] * 6 + [LL, I]
        L.gb_mcica_subcol_lw_device.argtypes = [P, P, I, I, I, I, IP] + [P] * 8 + [P] * 6 + [LL, I]
        L.gb_rrtmg_lw_gas_optics_diag.argtypes = [P, I, I] + [P] * 17 + [P, P]
        L.gb_mcica_subcol_lw_noalloc.argtypes = [P, I, I, I, I, IP] + [P] * 8 + [P] * 6 + [LL, I, P]
        L.gb_rrtmg_lw_strerror.restype = C.c_char_p
        L.gb_rrtmg_lw_strerror.argtypes = [I]
        L.gb_rrtmg_lw_last_error.restype = C.c_char_p
        L.gb_rrtmg_lw_last_error.argtypes = [P]
        _lib = L
        return L


def _check(L, ctx, rc: int):
    if rc != 0:
        detail = L.gb_rrtmg_lw_last_error(ctx).decode() if ctx else ""
        raise RrtmgLwError(rc, L.gb_rrtmg_lw_strerror(rc).decode() + (f" ({detail})" if detail else ""))


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return C.c_void_p(a)
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(a.ctypes.data)


def _f64(a):
    return np.asfortranarray(a, dtype=np.float64)


class Context:
    """rrtmg_lw_ini + the device state the calls share (tables, buffers, streams)."""

    def __init__(self, cpdair: float = 1004.0, device: int = 0, table_dir: str | None = None):
        self.L = load_library()
        h = C.c_void_p()
        rc = self.L.gb_rrtmg_lw_ini(cpdair, (table_dir or DATA_DIR).encode(), device, C.byref(h))
        _check(self.L, None, rc)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.gb_rrtmg_lw_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ rrtmg_lw
    def rrtmg_lw(self, state: dict, mc: dict | None, icld: int = 3, idrv: int = 1, inflglw: int = 2,
                 iceflglw: int = 3, liqflglw: int = 1, out: dict | None = None) -> dict:
        """rrtmg_lw on host arrays; returns uflx, dflx, hr, uflxc, dflxc, hrc, duflx_dt, duflxc_dt."""
        ncol, nlay = state["play"].shape
        st = [_f64(state[k]) for k in STATE_ORDER]
        tauaer = _f64(state.get("tauaer", np.zeros((ncol, nlay, 16))))
        cl = [_f64(mc[k]) if mc is not None else None for k in CLOUD_ORDER]
        if out is None:
            out = {k: np.zeros((ncol, nlay + 1), order="F") for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt")}
            out["hr"] = np.zeros((ncol, nlay), order="F")
            out["hrc"] = np.zeros((ncol, nlay), order="F")
        ic = C.c_int(icld)
        args = [self.h, ncol, nlay, C.byref(ic), idrv] + [_ptr(a) for a in st] + [inflglw, iceflglw, liqflglw]
        args += [_ptr(a) for a in cl] + [_ptr(tauaer)] + [_ptr(out[k]) for k in OUT_ORDER] + [ncol, ncol]
        _check(self.L, self.h, self.L.gb_rrtmg_lw(*args))
        out["icld"] = ic.value
        return out

    def rrtmg_lw_host_ptrs(self, ncol: int, nlay: int, ptrs: dict, icld: int = 3, idrv: int = 1,
                           inflglw: int = 2, iceflglw: int = 3, liqflglw: int = 1,
                           ld_in: int | None = None, ld_out: int | None = None) -> int:
        """rrtmg_lw on raw host pointers (e.g. pinned buffers); returns the status."""
        ic = C.c_int(icld)
        args = [self.h, ncol, nlay, C.byref(ic), idrv] + [_ptr(ptrs[k]) for k in STATE_ORDER]
        args += [inflglw, iceflglw, liqflglw] + [_ptr(ptrs.get(k)) for k in CLOUD_ORDER] + [_ptr(ptrs["tauaer"])]
        args += [_ptr(ptrs.get(k)) for k in OUT_ORDER] + [ld_in or ncol, ld_out or ncol]
        return self.L.gb_rrtmg_lw(*args)

    def rrtmg_lw_device(self, ncol: int, nlay: int, ptrs: dict, stream=None, icld: int = 3, idrv: int = 1,
                        inflglw: int = 2, iceflglw: int = 3, liqflglw: int = 1,
                        ld_in: int | None = None, ld_out: int | None = None, col_status=None) -> None:
        """rrtmg_lw on device pointers/tensors (Fortran layout), enqueued on `stream` (int handle)."""
        ic = C.c_int(icld)
        args = [self.h, _ptr(stream or 0), ncol, nlay, C.byref(ic), idrv] + [_ptr(ptrs[k]) for k in STATE_ORDER]
        args += [inflglw, iceflglw, liqflglw] + [_ptr(ptrs.get(k)) for k in CLOUD_ORDER] + [_ptr(ptrs["tauaer"])]
        args += [_ptr(ptrs.get(k)) for k in OUT_ORDER] + [ld_in or ncol, ld_out or ncol, _ptr(col_status)]
        _check(self.L, self.h, self.L.gb_rrtmg_lw_device(*args))

    def sync_status(self, stream=None) -> int:
        return self.L.gb_rrtmg_lw_sync_status(self.h, _ptr(stream or 0))

    def gas_optics_diag(self, state: dict):
        """taut and Planck fractions per (column, layer, g) from the column kernel."""
        ncol, nlay = state["play"].shape
        st = [_f64(state[k]) for k in STATE_ORDER]
        tauaer = _f64(state.get("tauaer", np.zeros((ncol, nlay, 16))))
        taut = np.zeros((ncol, nlay, 140), dtype=np.float32)
        fracs = np.zeros((ncol, nlay, 140), dtype=np.float32)
        rc = self.L.gb_rrtmg_lw_gas_optics_diag(self.h, ncol, nlay, *[_ptr(a) for a in st], _ptr(tauaer),
                                                _ptr(taut), _ptr(fracs))
        _check(self.L, self.h, rc)
        return taut, fracs

    # ------------------------------------------------------------ McICA
    def mcica_subcol_lw(self, state: dict, tauc: np.ndarray, icld: int, permuteseed: int, irng: int = 1,
                        alpha: np.ndarray | None = None, seed_per_column: bool = False) -> dict:
        ncol, nlay = state["play"].shape
        o = {k: np.zeros((140, ncol, nlay), order="F") for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl")}
        o["reicmcl"] = np.zeros((ncol, nlay), order="F")
        o["relqmcl"] = np.zeros((ncol, nlay), order="F")
        ir = C.c_int(irng)
        ins = [_f64(state[k]) for k in ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")]
        rc = self.L.gb_mcica_subcol_lw(self.h, ncol, nlay, icld, permuteseed, C.byref(ir), *[_ptr(a) for a in ins],
                                       _ptr(_f64(tauc)), _ptr(_f64(alpha) if alpha is not None else None),
                                       _ptr(o["cldfmcl"]), _ptr(o["ciwpmcl"]), _ptr(o["clwpmcl"]),
                                       _ptr(o["reicmcl"]), _ptr(o["relqmcl"]), _ptr(o["taucmcl"]), ncol,
                                       1 if seed_per_column else 0)
        _check(self.L, self.h, rc)
        return o

    def mcica_subcol_lw_device(self, ncol: int, nlay: int, ptrs: dict, icld: int, permuteseed: int, irng: int = 1,
                               seed_per_column: bool = True, stream=None, ld: int | None = None) -> None:
        ir = C.c_int(irng)
        rc = self.L.gb_mcica_subcol_lw_device(
            self.h, _ptr(stream or 0), ncol, nlay, icld, permuteseed, C.byref(ir),
            *[_ptr(ptrs.get(k)) for k in ("play", "cldfrac", "ciwp", "clwp", "rei", "rel", "tauc", "alpha")],
            *[_ptr(ptrs[k]) for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl")],
            ld or ncol, 1 if seed_per_column else 0)
        _check(self.L, self.h, rc)
