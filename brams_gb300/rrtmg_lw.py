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
BAND_ORDER = ["cldfrac", "tauc_band", "ciwp", "clwp", "rei", "rel"]  # non-McICA clouds (device keys)
SW_STATE = ["play", "plev", "tlay", "tlev", "tsfc", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "n2ovmr", "o2vmr",
            "asdir", "asdif", "aldir", "aldif", "coszen"]
SW_CLOUD = ["cldfmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl"]
SW_OUT = ["swuflx", "swdflx", "swhr", "swuflxc", "swdflxc", "swhrc"]
OUT_ORDER = ["uflx", "dflx", "hr", "uflxc", "dflxc", "hrc", "duflx_dt", "duflxc_dt"]

# C prototypes (see include/gb_rrtmg_lw.h)
EXPORTS = [
    "gb_rrtmg_lw_ini", "gb_rrtmg_lw_free", "gb_rrtmg_lw", "gb_rrtmg_lw_device",
    "gb_rrtmg_lw_sync_status", "gb_mcica_subcol_lw", "gb_mcica_subcol_lw_device",
    "gb_rrtmg_lw_strerror", "gb_rrtmg_lw_last_error", "gb_rrtmg_lw_gas_optics_diag",
    "gb_mcica_subcol_lw_noalloc", "gb_rrtmg_lw_batch_device", "gb_rrtmg_lw_autotune",
    "gb_rrtmg_lw_tuning_get", "gb_rrtmg_lw_batch_graph_create", "gb_rrtmg_lw_graph_launch",
    "gb_rrtmg_lw_graph_destroy", "gb_rrtmg_lw_tuning_set", "gb_rrtmg_lw_num_variants",
    "gb_lw_mlp_create", "gb_lw_mlp_destroy", "gb_lw_mlp_save", "gb_lw_mlp_load", "gb_lw_mlp_get_params",
    "gb_lw_mlp_set_params", "gb_lw_mlp_set_loss_weights", "gb_lw_mlp_samples", "gb_lw_mlp_fit_norm",
    "gb_lw_mlp_prepare", "gb_lw_mlp_gradients", "gb_lw_mlp_train_step", "gb_lw_mlp_forward", "gb_lw_mlp_infer",
    "gb_rrtmg_lw_batch_surrogate", "gb_lw_mlp_set_engine", "gb_rrtmg_lw_autotune_report",
    "gb_cldprop_lw_device", "gb_rtm_pack_lw_device", "gb_rtm_unpack_lw_device",
    "gb_rtm_ozone_load", "gb_rtm_ozone_free", "gb_rtm_ozone_lw",
    "gb_rrtmg_lw_shard_plan", "gb_rrtmg_lw_grid_slice", "gb_rrtmg_lw_nomcica", "gb_rrtmg_lw_nomcica_device",
    "gb_rrtmg_sw_ini", "gb_rrtmg_sw_set_precision", "gb_rrtmg_sw", "gb_rrtmg_sw_device", "gb_mcica_subcol_sw", "gb_mcica_subcol_sw_device",
    "gb_cldprop_sw_device", "gb_rtm_pack_sw_device", "gb_rtm_unpack_sw_device",
]
MLP_MMA_SYNC, MLP_TCGEN05 = 0, 1
MLP_NPARAM = 72352
MLP_NNORM = 626

CLOUD_SUBCOL, CLOUD_FUSED = 0, 1
KIND_FUSED, KIND_LEARNED = 1, 2
MAX_GRIDS = 32

_GRID_PTRS = ["play", "plev", "tlay", "tlev", "tsfc", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "n2ovmr",
              "o2vmr", "cfc11vmr", "cfc12vmr", "cfc22vmr", "ccl4vmr", "emis", "tauaer",
              "cldfmcl", "taucmcl", "ciwpmcl", "clwpmcl", "cldfrac", "ciwp", "clwp", "tauc",
              "reicmcl", "relqmcl", "uflx", "dflx", "hr", "uflxc", "dflxc", "hrc", "duflx_dt", "duflxc_dt",
              "d_col_status", "sur_tau", "sur_frac", "sur_flag"]


class GridDesc(C.Structure):
    """gb_lw_grid: one grid of a batched call (device arrays, Fortran layouts)."""
    _fields_ = ([(k, C.c_int) for k in ("ncol", "nlay", "icld", "idrv", "inflglw", "iceflglw", "liqflglw",
                                        "cloud_mode")]
                + [("seed0", C.c_uint32), ("ld_in", C.c_int64), ("ld_out", C.c_int64)]
                + [(k, C.c_void_p) for k in _GRID_PTRS])


class Tuning(C.Structure):
    """gb_lw_tuning: launch shape of the batched kernel."""
    _fields_ = [(k, C.c_int) for k in ("variant", "threads", "min_blocks", "blocks_per_sm", "blocks")] + \
        [("ms", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def grid_desc(ncol: int, nlay: int, arrays: dict, icld: int = 3, idrv: int = 1, inflglw: int = 2,
              iceflglw: int = 3, liqflglw: int = 1, cloud_mode: int = CLOUD_SUBCOL, seed0: int = 0,
              ld_in: int | None = None, ld_out: int | None = None) -> GridDesc:
    """Descriptor of one grid from device arrays (torch tensors or raw pointers) keyed by argument name.
    In CLOUD_FUSED mode the layer radii go under "reicmcl"/"relqmcl" (or "rei"/"rel")."""
    g = GridDesc()
    g.ncol, g.nlay, g.icld, g.idrv = ncol, nlay, icld, idrv
    g.inflglw, g.iceflglw, g.liqflglw, g.cloud_mode = inflglw, iceflglw, liqflglw, cloud_mode
    g.seed0 = seed0 & 0xFFFFFFFF
    g.ld_in = ld_in or ncol
    g.ld_out = ld_out or ncol
    alias = {"reicmcl": "rei", "relqmcl": "rel"}
    for k in _GRID_PTRS:
        a = arrays.get(k)
        if a is None and k in alias:
            a = arrays.get(alias[k])
        p = _ptr(a)
        setattr(g, k, p.value if p is not None else None)
    return g


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
        L.gb_rrtmg_lw_nomcica.argtypes = [P, I, I, IP, I] + [P] * 16 + [I, I, I] + [P] * 7 + [P] * 8 + [LL, LL]
        L.gb_rrtmg_lw_nomcica_device.argtypes = [P, P, I, I, IP, I] + [P] * 16 + [I, I, I] + [P] * 7 + [P] * 8 + \
            [LL, LL, P]
        L.gb_mcica_subcol_lw.argtypes = [P, I, I, I, I, IP] + [P] * 8 + [P] * 6 + [LL, I]
        L.gb_mcica_subcol_lw_device.argtypes = [P, P, I, I, I, I, IP] + [P] * 8 + [P] * 6 + [LL, I]
        L.gb_rrtmg_lw_gas_optics_diag.argtypes = [P, I, I] + [P] * 17 + [P, P]
        L.gb_cldprop_lw_device.argtypes = [P, P, I, I, I, I, I] + [P] * 7 + [LL, P]
        L.gb_rtm_pack_lw_device.argtypes = [P, P] + [I] * 9 + [P] * 31 + [LL]
        L.gb_rtm_unpack_lw_device.argtypes = [P, P] + [I] * 7 + [P] * 3 + [LL, LL, P, P]
        L.gb_rtm_pack_sw_device.argtypes = [P, P] + [I] * 7 + [P] * 7
        L.gb_rtm_unpack_sw_device.argtypes = [P, P] + [I] * 6 + [P] * 2
        L.gb_rtm_ozone_load.argtypes = [C.c_char_p, C.POINTER(P)]
        L.gb_rtm_ozone_free.argtypes = [P]
        L.gb_rtm_ozone_lw.argtypes = [P, I, I, P, LL, P, I, P, LL]
        L.gb_mcica_subcol_lw_noalloc.argtypes = [P, I, I, I, I, IP] + [P] * 8 + [P] * 6 + [LL, I, P]
        GP = C.POINTER(GridDesc)
        L.gb_rrtmg_lw_batch_device.argtypes = [P, P, I, GP]
        L.gb_rrtmg_lw_autotune.argtypes = [P, P, I, GP, I, I, C.POINTER(Tuning)]
        L.gb_rrtmg_lw_tuning_get.argtypes = [P, I, I, C.POINTER(Tuning)]
        L.gb_rrtmg_lw_batch_graph_create.argtypes = [P, I, GP, C.POINTER(P)]
        L.gb_rrtmg_lw_graph_launch.argtypes = [P, P]
        L.gb_rrtmg_lw_graph_destroy.argtypes = [P]
        L.gb_rrtmg_lw_tuning_set.argtypes = [P, I, I, C.POINTER(Tuning)]
        L.gb_rrtmg_lw_num_variants.argtypes = []
        SWA = [P] * 16 + [D, I, D, I, I, I, I] + [P] * 9 + [P] * 4 + [P] * 6
        L.gb_rrtmg_sw_ini.argtypes = [P, D, C.c_char_p]
        L.gb_rrtmg_sw_set_precision.argtypes = [P, I]
        L.gb_rrtmg_sw.argtypes = [P, I, I, IP, IP] + SWA + [LL, LL]
        L.gb_rrtmg_sw_device.argtypes = [P, P, I, I, IP, IP] + SWA + [LL, LL, P]
        L.gb_mcica_subcol_sw.argtypes = [P, I, I, I, I, IP] + [P] * 11 + [P] * 9 + [LL, I]
        L.gb_mcica_subcol_sw_device.argtypes = [P, P, I, I, I, I, IP] + [P] * 11 + [P] * 9 + [LL, I]
        L.gb_cldprop_sw_device.argtypes = [P, P, I, I, I, I, I] + [P] * 9 + [P] * 4 + [LL, P]
        L.gb_rrtmg_lw_shard_plan.argtypes = [I, IP, IP, I, I, C.POINTER(LL), C.POINTER(LL)]
        L.gb_rrtmg_lw_grid_slice.argtypes = [GP, LL, LL, GP]
        U64, F = C.c_uint64, C.c_float
        L.gb_lw_mlp_create.argtypes = [P, U64, C.POINTER(P)]
        L.gb_lw_mlp_destroy.argtypes = [P]
        L.gb_lw_mlp_save.argtypes = [P, C.c_char_p]
        L.gb_lw_mlp_load.argtypes = [P, C.c_char_p, C.POINTER(P)]
        L.gb_lw_mlp_get_params.argtypes = [P, P, P]
        L.gb_lw_mlp_set_params.argtypes = [P, P, P]
        L.gb_lw_mlp_set_loss_weights.argtypes = [P, P]
        L.gb_lw_mlp_samples.argtypes = [P, P, GP, P, P, P]
        L.gb_lw_mlp_fit_norm.argtypes = [P, P, LL, P, P, P]
        L.gb_lw_mlp_prepare.argtypes = [P, P, LL, P, P, P, P, P]
        L.gb_lw_mlp_gradients.argtypes = [P, P, LL, P, P, P, P]
        L.gb_lw_mlp_train_step.argtypes = [P, P, LL, P, P, F, P]
        L.gb_lw_mlp_forward.argtypes = [P, P, LL, P, P]
        L.gb_lw_mlp_infer.argtypes = [P, P, GP, P, P, P]
        L.gb_rrtmg_lw_batch_surrogate.argtypes = [P, P, I, GP, P]
        L.gb_lw_mlp_set_engine.argtypes = [P, I]
        L.gb_rrtmg_lw_autotune_report.argtypes = [P, C.POINTER(Tuning), I]
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

    # ------------------------------------------------------------ non-McICA rrtmg_lw
    def rrtmg_lw_nomcica(self, state: dict, icld: int = 2, idrv: int = 1, inflglw: int = 2, iceflglw: int = 3,
                         liqflglw: int = 1, out: dict | None = None) -> dict:
        """rrtmg_lw of the non-McICA driver on host arrays: band-level clouds
        state['cldfrac'], 'ciwp', 'clwp', 'rei', 'rel' (ncol, nlay) and
        optional 'tauc_band' (16, ncol, nlay).  icld 1: random overlap;
        0, 2, 3: maximum/random (0 without clouds)."""
        ncol, nlay = state["play"].shape
        st = [_f64(state[k]) for k in STATE_ORDER]
        tauaer = _f64(state.get("tauaer", np.zeros((ncol, nlay, 16))))
        tb = state.get("tauc_band")
        cl = [_f64(state["cldfrac"]), _f64(np.zeros((16, ncol, nlay)) if tb is None else tb)]
        cl += [_f64(state[k]) for k in ("ciwp", "clwp", "rei", "rel")]
        if out is None:
            out = {k: np.zeros((ncol, nlay + 1), order="F") for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt")}
            out["hr"] = np.zeros((ncol, nlay), order="F")
            out["hrc"] = np.zeros((ncol, nlay), order="F")
        ic = C.c_int(icld)
        args = [self.h, ncol, nlay, C.byref(ic), idrv] + [_ptr(a) for a in st] + [inflglw, iceflglw, liqflglw]
        args += [_ptr(a) for a in cl] + [_ptr(tauaer)] + [_ptr(out[k]) for k in OUT_ORDER] + [ncol, ncol]
        _check(self.L, self.h, self.L.gb_rrtmg_lw_nomcica(*args))
        out["icld"] = ic.value
        return out

    def rrtmg_lw_nomcica_device(self, ncol: int, nlay: int, ptrs: dict, stream=None, icld: int = 2, idrv: int = 1,
                                inflglw: int = 2, iceflglw: int = 3, liqflglw: int = 1,
                                ld_in: int | None = None, ld_out: int | None = None, col_status=None) -> int:
        """The non-McICA driver on device pointers/tensors (Fortran layout)
        keyed as rrtmg_lw_nomcica's state; returns icld after the clamp."""
        ic = C.c_int(icld)
        args = [self.h, _ptr(stream or 0), ncol, nlay, C.byref(ic), idrv] + [_ptr(ptrs[k]) for k in STATE_ORDER]
        args += [inflglw, iceflglw, liqflglw] + [_ptr(ptrs.get(k)) for k in BAND_ORDER] + [_ptr(ptrs["tauaer"])]
        args += [_ptr(ptrs.get(k)) for k in OUT_ORDER] + [ld_in or ncol, ld_out or ncol, _ptr(col_status)]
        _check(self.L, self.h, self.L.gb_rrtmg_lw_nomcica_device(*args))
        return ic.value

    # ------------------------------------------------------------ RRTMG_SW
    def sw_ini(self, cpdair: float = 1004.0, table_dir: str | None = None) -> None:
        """gb_rrtmg_sw_ini: the shortwave tables into this context."""
        _check(self.L, self.h, self.L.gb_rrtmg_sw_ini(self.h, cpdair, table_dir.encode() if table_dir else None))

    def sw_set_precision(self, bits: int) -> None:
        """gb_rrtmg_sw_set_precision: 32 (fp32 solution, fp64 sums) or 64."""
        _check(self.L, self.h, self.L.gb_rrtmg_sw_set_precision(self.h, bits))

    def rrtmg_sw(self, state: dict, mc: dict | None, icld: int = 3, iaer: int = 10, adjes: float = 1.0,
                 dyofyr: int = 0, scon: float = 1368.22, isolvar: int = -1, inflgsw: int = 2, iceflgsw: int = 3,
                 liqflgsw: int = 1) -> dict:
        """rrtmg_sw on host arrays (keys as oracle/pyoracle.py rrtmg_sw);
        returns swuflx, swdflx, swhr, swuflxc, swdflxc, swhrc, icld, iaer."""
        ncol, nlay = state["play"].shape
        st = [_f64(state[k]) for k in SW_STATE]
        cl = [_f64(mc[k]) if mc is not None else None for k in SW_CLOUD]
        aer = [_f64(state[k]) if k in state else None for k in ("tauaer_sw", "ssaaer_sw", "asmaer_sw")]
        out = {k: np.zeros((ncol, nlay + 1), order="F") for k in ("swuflx", "swdflx", "swuflxc", "swdflxc")}
        out["swhr"] = np.zeros((ncol, nlay), order="F")
        out["swhrc"] = np.zeros((ncol, nlay), order="F")
        ic, ia = C.c_int(icld), C.c_int(iaer)
        args = [self.h, ncol, nlay, C.byref(ic), C.byref(ia)] + [_ptr(a) for a in st]
        args += [adjes, dyofyr, scon, isolvar, inflgsw, iceflgsw, liqflgsw] + [_ptr(a) for a in cl]
        args += [_ptr(a) for a in aer] + [None] + [_ptr(out[k]) for k in SW_OUT] + [ncol, ncol]
        _check(self.L, self.h, self.L.gb_rrtmg_sw(*args))
        out["icld"], out["iaer"] = ic.value, ia.value
        return out

    def mcica_subcol_sw(self, state: dict, band: dict, icld: int, permuteseed: int, irng: int = 1,
                        seed_per_column: bool = False) -> dict:
        """mcica_subcol_sw on host arrays: state['play', 'cldfrac', 'ciwp',
        'clwp', 'rei', 'rel'] (ncol, nlay), band['tauc', 'ssac', 'asmc',
        'fsfc'] (14, ncol, nlay), optional state['alpha']."""
        ncol, nlay = state["play"].shape
        ins = [_f64(state[k]) for k in ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")]
        ins += [_f64(band[k]) for k in ("tauc", "ssac", "asmc", "fsfc")]
        alpha = _f64(state["alpha"]) if "alpha" in state else None
        o = {k: np.zeros((112, ncol, nlay), order="F") for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl",
                                                                 "ssacmcl", "asmcmcl", "fsfcmcl")}
        o["reicmcl"] = np.zeros((ncol, nlay), order="F")
        o["relqmcl"] = np.zeros((ncol, nlay), order="F")
        ir = C.c_int(irng)
        outs = [o[k] for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl",
                               "asmcmcl", "fsfcmcl")]
        rc = self.L.gb_mcica_subcol_sw(self.h, ncol, nlay, icld, permuteseed, C.byref(ir), *[_ptr(a) for a in ins],
                                       _ptr(alpha), *[_ptr(a) for a in outs], ncol, int(seed_per_column))
        _check(self.L, self.h, rc)
        return o

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

    def cldprop_lw_device(self, ncol: int, nlay: int, ptrs: dict, inflag: int = 2, iceflag: int = 3,
                          liqflag: int = 1, ld: int | None = None, stream=None) -> None:
        """cldprop (rrtmg_lw_cldprop.f90:50) on device arrays: ptrs holds cldfrac, ciwp, clwp, rei,
        rel ((ld, nlay) memory order), optional tauc (16, ld, nlay), taucloud (16, ld, nlay) out and
        optional d_col_status (ncol int32)."""
        g = lambda k: _ptr(ptrs.get(k))
        _check(self.L, self.h, self.L.gb_cldprop_lw_device(
            self.h, _ptr(stream or 0), ncol, nlay, inflag, iceflag, liqflag, g("cldfrac"), g("tauc"), g("ciwp"),
            g("clwp"), g("rei"), g("rel"), g("taucloud"), ld if ld is not None else ncol, g("d_col_status")))

    def cldprop_sw_device(self, ncol: int, nlay: int, ptrs: dict, inflag: int = 2, iceflag: int = 3,
                          liqflag: int = 1, ld: int | None = None, stream=None) -> None:
        """cldprop_sw (rrtmg_sw_cldprop.f90:53) on device arrays: ptrs holds cldfrac, ciwp, clwp, rei,
        rel ((ld, nlay) memory order), optional tauc, ssac, asmc, fsfc (14, ld, nlay), outputs
        taucloud, ssacloud, asmcloud and optional taucldorig (14, ld, nlay), optional d_col_status
        (ncol int32)."""
        g = lambda k: _ptr(ptrs.get(k))
        _check(self.L, self.h, self.L.gb_cldprop_sw_device(
            self.h, _ptr(stream or 0), ncol, nlay, inflag, iceflag, liqflag, g("cldfrac"), g("tauc"), g("ssac"),
            g("asmc"), g("fsfc"), g("ciwp"), g("clwp"), g("rei"), g("rel"), g("taucloud"), g("ssacloud"),
            g("asmcloud"), g("taucldorig"), ld if ld is not None else ncol, g("d_col_status")))

    PACK_IN = ("pi0", "pp", "theta", "rv", "rlongup", "albedt", "cldf", "lwl", "iwl", "rel", "rei")
    PACK_OUT = ("play", "plev", "tlay", "tlev", "tsfc", "h2ovmr", "co2vmr", "ch4vmr", "n2ovmr", "o2vmr", "cfc11vmr",
                "cfc12vmr", "cfc22vmr", "ccl4vmr", "emis", "cldfrac", "ciwp", "clwp", "reic", "relq")

    def rtm_pack_lw_device(self, mzp: int, mxp: int, myp: int, box, ptrs: dict, iceflgsw: int = 3,
                           firsttime: bool = False, ld: int | None = None, stream=None) -> None:
        """gb_rtm_pack_lw_device: BRAMS fields (PACK_IN, float32 device arrays in
        Fortran order) of the 1-based box (ia, iz, ja, jz) into the rrtmg_lw
        inputs (PACK_OUT, float64, leading dimension ld)."""
        ia, iz, ja, jz = box
        ncol = (iz - ia + 1) * (jz - ja + 1)
        args = [_ptr(ptrs[k]) for k in self.PACK_IN] + [_ptr(ptrs[k]) for k in self.PACK_OUT]
        _check(self.L, self.h, self.L.gb_rtm_pack_lw_device(
            self.h, _ptr(stream or 0), mzp, mxp, myp, ia, iz, ja, jz, iceflgsw, 1 if firsttime else 0, *args,
            ld if ld is not None else ncol))

    def rtm_unpack_lw_device(self, mzp: int, mxp: int, myp: int, box, hr, dflx, fthrd, rlong, swhr=None,
                             ld_hr: int | None = None, ld_flx: int | None = None, stream=None) -> None:
        """gb_rtm_unpack_lw_device: heating rates into BRAMS's theta tendency
        fthrd (mzp, mxp, myp) and dflx(:, 1) into rlong (mxp, myp), float32."""
        ia, iz, ja, jz = box
        ncol = (iz - ia + 1) * (jz - ja + 1)
        _check(self.L, self.h, self.L.gb_rtm_unpack_lw_device(
            self.h, _ptr(stream or 0), mzp, mxp, myp, ia, iz, ja, jz, _ptr(hr), _ptr(swhr), _ptr(dflx),
            ld_hr if ld_hr is not None else ncol, ld_flx if ld_flx is not None else ncol, _ptr(fthrd),
            _ptr(rlong)))

    def rtm_pack_sw_device(self, mxp: int, myp: int, box, cosz, albedt, out: dict, firsttime: bool = False,
                           stream=None) -> None:
        """gb_rtm_pack_sw_device: BRAMS's cosz and albedt (float32 (mxp, myp)) into coszen and
        the albedos asdir, asdif, aldir, aldif (float64 (ncol) device arrays in out)."""
        ia, iz, ja, jz = box
        _check(self.L, self.h, self.L.gb_rtm_pack_sw_device(
            self.h, _ptr(stream or 0), mxp, myp, ia, iz, ja, jz, 1 if firsttime else 0, _ptr(cosz), _ptr(albedt),
            *[_ptr(out[k]) for k in ("coszen", "asdir", "asdif", "aldir", "aldif")]))

    def rtm_unpack_sw_device(self, mxp: int, myp: int, box, swdflx, rshort, stream=None) -> None:
        """gb_rtm_unpack_sw_device: the surface downward shortwave flux (the first ncol values of
        swdflx) into BRAMS's rshort (float32 (mxp, myp)), 0 below 0.5 W m-2."""
        ia, iz, ja, jz = box
        _check(self.L, self.h, self.L.gb_rtm_unpack_sw_device(
            self.h, _ptr(stream or 0), mxp, myp, ia, iz, ja, jz, _ptr(swdflx), _ptr(rshort)))

    def mcica_subcol_lw_device(self, ncol: int, nlay: int, ptrs: dict, icld: int, permuteseed: int, irng: int = 1,
                               seed_per_column: bool = True, stream=None, ld: int | None = None) -> None:
        ir = C.c_int(irng)
        rc = self.L.gb_mcica_subcol_lw_device(
            self.h, _ptr(stream or 0), ncol, nlay, icld, permuteseed, C.byref(ir),
            *[_ptr(ptrs.get(k)) for k in ("play", "cldfrac", "ciwp", "clwp", "rei", "rel", "tauc", "alpha")],
            *[_ptr(ptrs[k]) for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl")],
            ld or ncol, 1 if seed_per_column else 0)
        _check(self.L, self.h, rc)

    # ------------------------------------------------------------ batched grids
    @staticmethod
    def _grids(grids) -> tuple:
        n = len(grids)
        if not 1 <= n <= MAX_GRIDS:
            raise ValueError(f"1..{MAX_GRIDS} grids per batch, got {n}")
        arr = (GridDesc * n)(*grids)
        return n, arr

    def rrtmg_lw_batch_device(self, grids, stream=None) -> None:
        """All grids (GridDesc list) in one persistent launch on `stream`."""
        n, arr = self._grids(grids)
        _check(self.L, self.h, self.L.gb_rrtmg_lw_batch_device(self.h, _ptr(stream or 0), n, arr))

    def autotune(self, grids, sample_cols: int = 0, reps: int = 3, stream=None) -> dict:
        """Time every kernel variant and grid size on a sample of the batch; keeps and returns the best."""
        n, arr = self._grids(grids)
        t = Tuning()
        _check(self.L, self.h, self.L.gb_rrtmg_lw_autotune(self.h, _ptr(stream or 0), n, arr, sample_cols, reps,
                                                           C.byref(t)))
        return t.as_dict()

    def autotune_report(self) -> list:
        """Every candidate of the last autotune call: shape and time per launch (ms)."""
        n = self.L.gb_rrtmg_lw_autotune_report(self.h, None, 0)
        arr = (Tuning * max(n, 1))()
        self.L.gb_rrtmg_lw_autotune_report(self.h, arr, n)
        return [arr[i].as_dict() for i in range(n)]

    def tuning(self, nlay: int, kind: int = KIND_FUSED) -> dict:
        """Shape used for batches of this largest nlay and kind (KIND_FUSED | KIND_LEARNED bits)."""
        t = Tuning()
        _check(self.L, self.h, self.L.gb_rrtmg_lw_tuning_get(self.h, nlay, kind, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, nlay: int, variant: int, blocks_per_sm: int, kind: int = KIND_FUSED) -> None:
        t = Tuning(variant, 0, 0, blocks_per_sm, 0, 0.0)
        _check(self.L, self.h, self.L.gb_rrtmg_lw_tuning_set(self.h, nlay, kind, C.byref(t)))

    def num_variants(self) -> int:
        return self.L.gb_rrtmg_lw_num_variants()

    def batch_graph(self, grids) -> "BatchGraph":
        """CUDA graph of one batched launch (inputs updated in place between replays)."""
        n, arr = self._grids(grids)
        h = C.c_void_p()
        _check(self.L, self.h, self.L.gb_rrtmg_lw_batch_graph_create(self.h, n, arr, C.byref(h)))
        return BatchGraph(self, h)


class BatchGraph:
    def __init__(self, ctx: Context, h):
        self.ctx, self.h = ctx, h

    def launch(self, stream=None) -> None:
        _check(self.ctx.L, self.ctx.h, self.ctx.L.gb_rrtmg_lw_graph_launch(self.h, _ptr(stream or 0)))

    def close(self) -> None:
        if getattr(self, "h", None):
            self.ctx.L.gb_rrtmg_lw_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Mlp:
    """The learned stand-in for taumol (gb_lw_mlp_*): training and inference on device buffers."""

    def __init__(self, ctx: Context, seed: int = 1, path: str | None = None):
        self.ctx, self.L = ctx, ctx.L
        h = C.c_void_p()
        if path is not None:
            rc = self.L.gb_lw_mlp_load(ctx.h, path.encode(), C.byref(h))
        else:
            rc = self.L.gb_lw_mlp_create(ctx.h, seed, C.byref(h))
        _check(self.L, ctx.h, rc)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.gb_lw_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, rc):
        _check(self.L, self.ctx.h, rc)

    def save(self, path: str) -> None:
        self._ok(self.L.gb_lw_mlp_save(self.h, path.encode()))

    def set_engine(self, engine: int) -> None:
        """MLP_TCGEN05 (tensor-memory MMAs) or MLP_MMA_SYNC (warp MMAs) for inference."""
        self._ok(self.L.gb_lw_mlp_set_engine(self.h, engine))

    def params(self):
        p = np.zeros(MLP_NPARAM, dtype=np.float32)
        n = np.zeros(MLP_NNORM, dtype=np.float32)
        self._ok(self.L.gb_lw_mlp_get_params(self.h, _ptr(p), _ptr(n)))
        return p, n

    def set_params(self, params=None, norm=None) -> None:
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        n = None if norm is None else np.ascontiguousarray(norm, dtype=np.float32)
        self._ok(self.L.gb_lw_mlp_set_params(self.h, _ptr(p), _ptr(n)))

    def set_loss_weights(self, w) -> None:
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._ok(self.L.gb_lw_mlp_set_loss_weights(self.h, _ptr(w)))

    def samples(self, grid: GridDesc, feat, tau, frac, stream=None) -> None:
        self._ok(self.L.gb_lw_mlp_samples(self.ctx.h, _ptr(stream or 0), C.byref(grid), _ptr(feat), _ptr(tau),
                                          _ptr(frac)))

    def fit_norm(self, rows: int, feat, tau, frac, stream=None) -> None:
        self._ok(self.L.gb_lw_mlp_fit_norm(self.h, _ptr(stream or 0), rows, _ptr(feat), _ptr(tau), _ptr(frac)))

    def prepare(self, rows: int, feat, tau, frac, x, t, stream=None) -> None:
        self._ok(self.L.gb_lw_mlp_prepare(self.h, _ptr(stream or 0), rows, _ptr(feat), _ptr(tau), _ptr(frac),
                                          _ptr(x), _ptr(t)))

    def gradients(self, rows: int, x, t, grad, loss, stream=None) -> None:
        self._ok(self.L.gb_lw_mlp_gradients(self.h, _ptr(stream or 0), rows, _ptr(x), _ptr(t), _ptr(grad),
                                            _ptr(loss)))

    def train_step(self, rows: int, x, t, lr: float, loss=None, stream=None) -> None:
        self._ok(self.L.gb_lw_mlp_train_step(self.h, _ptr(stream or 0), rows, _ptr(x), _ptr(t), lr, _ptr(loss)))

    def forward(self, rows: int, x, y, stream=None) -> None:
        self._ok(self.L.gb_lw_mlp_forward(self.h, _ptr(stream or 0), rows, _ptr(x), _ptr(y)))

    def infer(self, grid: GridDesc, tau, frac, flag, stream=None) -> None:
        """gb_lw_mlp_infer: tau and frac are float16 device arrays of
        ncol*nlay*140 values (8-byte aligned), flag uint8 of ncol*nlay."""
        self._ok(self.L.gb_lw_mlp_infer(self.h, _ptr(stream or 0), C.byref(grid), _ptr(tau), _ptr(frac), _ptr(flag)))

    def batch(self, grids, stream=None) -> None:
        """gb_rrtmg_lw_batch_surrogate: all grids with learned gas optics."""
        n, arr = Context._grids(grids)
        self._ok(self.L.gb_rrtmg_lw_batch_surrogate(self.ctx.h, _ptr(stream or 0), n, arr, self.h))


class Ozone:
    """gb_rtm_ozone_*: BRAMS's zonal ozone climatology for packed columns, on
    host arrays (no GPU needed)."""

    def __init__(self, table_dir: str | None = None):
        self.L = load_library()
        h = C.c_void_p()
        rc = self.L.gb_rtm_ozone_load((table_dir or DATA_DIR).encode(), C.byref(h))
        if rc != 0:
            raise RrtmgLwError(rc, self.L.gb_rrtmg_lw_strerror(rc).decode())
        self.h = h

    def o3vmr(self, plev: np.ndarray, glat: np.ndarray, doy: int) -> np.ndarray:
        """plev (ncol, mzp) interface pressures, glat (ncol,) degrees ->
        o3vmr (ncol, mzp - 1)."""
        plev = np.asfortranarray(plev, dtype=np.float64)
        glat = np.ascontiguousarray(glat, dtype=np.float32)
        ncol, mzp = plev.shape
        out = np.zeros((ncol, mzp - 1), order="F")
        rc = self.L.gb_rtm_ozone_lw(self.h, ncol, mzp, plev.ctypes.data, ncol, glat.ctypes.data, int(doy),
                                    out.ctypes.data, ncol)
        if rc != 0:
            raise RrtmgLwError(rc, self.L.gb_rrtmg_lw_strerror(rc).decode())
        return out

    def close(self) -> None:
        if self.h:
            self.L.gb_rtm_ozone_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
