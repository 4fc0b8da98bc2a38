"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module; the product library never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DATA = os.path.join(ROOT, "brams_gb300", "data")
_lib = {}

_D = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")


def build(tuned: bool = False) -> str:
    target = "tuned" if tuned else "all"
    subprocess.run(["make", "-s", "-C", HERE, target], check=True)
    return os.path.join(HERE, "_build", "liblworacle_tuned.so" if tuned else "liblworacle.so")


def lib(tuned: bool = False):
    key = "tuned" if tuned else "portable"
    if key in _lib:
        return _lib[key]
    path = os.path.join(HERE, "_build", "liblworacle_tuned.so" if tuned else "liblworacle.so")
    src = os.path.join(HERE, "lw_oracle.cpp")
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        build(tuned)
    L = C.CDLL(path)
    L.ora_init.restype = C.c_int
    L.ora_init.argtypes = [C.c_double, C.c_char_p, C.c_char_p]
    L.ora_error_string.restype = C.c_char_p
    rc = L.ora_init(1004.0, os.path.join(DATA, "lw_ref_tables.gblw").encode(),
                    os.path.join(DATA, "lw_ktables.gblw").encode())
    if rc != 0:
        raise RuntimeError(f"oracle init failed: {rc}")
    _lib[key] = L
    return L


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _f(a):
    return np.asfortranarray(a, dtype=np.float64)


STATE_ORDER = ["play", "plev", "tlay", "tlev", "tsfc", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr",
               "n2ovmr", "o2vmr", "cfc11vmr", "cfc12vmr", "cfc22vmr", "ccl4vmr", "emis"]
CLOUD_ORDER = ["cldfmcl", "taucmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl"]


def rrtmg_lw(state: dict, mc: dict, icld: int = 3, idrv: int = 1, inflglw: int = 2,
             iceflglw: int = 3, liqflglw: int = 1, nthreads: int = 1, tuned: bool = False) -> dict:
    """Reference-order FP64 rrtmg_lw on Fortran-ordered arrays; returns the outputs."""
    L = lib(tuned)
    ncol, nlay = state["play"].shape
    st = [_f(state[k]) for k in STATE_ORDER]
    cl = [_f(mc[k]) for k in CLOUD_ORDER]
    tauaer = _f(state["tauaer"])
    out = {k: np.zeros((ncol, nlay + 1), order="F") for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt")}
    out["hr"] = np.zeros((ncol, nlay), order="F")
    out["hrc"] = np.zeros((ncol, nlay), order="F")
    ic = C.c_int(icld)
    args = [C.c_int(ncol), C.c_int(nlay), C.byref(ic), C.c_int(idrv)] + [_p(a) for a in st]
    args += [C.c_int(inflglw), C.c_int(iceflglw), C.c_int(liqflglw)] + [_p(a) for a in cl] + [_p(tauaer)]
    args += [_p(out[k]) for k in ("uflx", "dflx", "hr", "uflxc", "dflxc", "hrc", "duflx_dt", "duflxc_dt")]
    args += [C.c_int(nthreads)]
    rc = L.ora_rrtmg_lw(*args)
    if rc != 0:
        raise RuntimeError(f"oracle rrtmg_lw: {L.ora_error_string(rc).decode()}")
    out["icld"] = ic.value
    return out


def rrtmg_lw_rtrn(state: dict, idrv: int = 1, inflglw: int = 2, iceflglw: int = 3,
                  liqflglw: int = 1) -> dict:
    """The non-McICA driver with random cloud overlap (icld 1, rtrn)."""
    return rrtmg_lw_nomcica(state, 1, idrv, inflglw, iceflglw, liqflglw)


def rrtmg_lw_nomcica(state: dict, icld: int = 2, idrv: int = 1, inflglw: int = 2, iceflglw: int = 3,
                     liqflglw: int = 1, tuned: bool = False) -> dict:
    """rrtmg_lw of the non-McICA driver (rrtmg_lw_rad.nomcica.f90) on
    band-level clouds: state['cldfrac'], 'ciwp', 'clwp', 'rei', 'rel' (ncol,
    nlay) and optional 'tauc_band' (16, ncol, nlay, read for inflag 0).
    icld 1: random overlap (rtrn); 0, 2, 3: maximum/random overlap (rtrnmr);
    other values become 2 (returned in out['icld'])."""
    L = lib(tuned)
    ncol, nlay = state["play"].shape
    st = [_f(state[k]) for k in STATE_ORDER]
    tb = state.get("tauc_band")
    tb = _f(np.zeros((16, ncol, nlay)) if tb is None else tb)
    cl = [_f(state["cldfrac"]), tb] + [_f(state[k]) for k in ("ciwp", "clwp", "rei", "rel")]
    out = {k: np.zeros((ncol, nlay + 1), order="F") for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt")}
    out["hr"] = np.zeros((ncol, nlay), order="F")
    out["hrc"] = np.zeros((ncol, nlay), order="F")
    ic = C.c_int(icld)
    args = [C.c_int(ncol), C.c_int(nlay), C.byref(ic), C.c_int(idrv)] + [_p(a) for a in st]
    args += [C.c_int(inflglw), C.c_int(iceflglw), C.c_int(liqflglw)] + [_p(a) for a in cl] + [_p(_f(state["tauaer"]))]
    args += [_p(out[k]) for k in ("uflx", "dflx", "hr", "uflxc", "dflxc", "hrc", "duflx_dt", "duflxc_dt")]
    rc = L.ora_rrtmg_lw_nomcica(*args)
    if rc != 0:
        raise RuntimeError(f"oracle rrtmg_lw (non-McICA): {L.ora_error_string(rc).decode()}")
    out["icld"] = ic.value
    return out


def column_intermediates(state: dict, mc: dict, icol: int, icld: int = 3, inflglw: int = 2,
                         iceflglw: int = 3, liqflglw: int = 1) -> dict:
    L = lib()
    ncol, nlay = state["play"].shape
    st = [_f(state[k]) for k in STATE_ORDER]
    cl = [_f(mc[k]) for k in CLOUD_ORDER]
    o = {"taug": np.zeros((nlay, 140), order="F"), "fracs": np.zeros((nlay, 140), order="F"),
         "taut": np.zeros((nlay, 140), order="F"), "planklay": np.zeros((nlay, 16), order="F"),
         "planklev": np.zeros((nlay + 1, 16), order="F"), "plankbnd": np.zeros(16),
         "taucmc": np.zeros((140, nlay), order="F")}
    lt = C.c_int(0)
    args = [C.c_int(ncol), C.c_int(nlay), C.c_int(icol), C.c_int(icld)] + [_p(a) for a in st]
    args += [C.c_int(inflglw), C.c_int(iceflglw), C.c_int(liqflglw)] + [_p(a) for a in cl]
    args += [_p(_f(state["tauaer"]))]
    args += [_p(o[k]) for k in ("taug", "fracs", "taut", "planklay", "planklev", "plankbnd", "taucmc")]
    args += [C.byref(lt)]
    rc = L.ora_column_intermediates(*args)
    if rc != 0:
        raise RuntimeError(f"oracle intermediates: {L.ora_error_string(rc).decode()}")
    o["laytrop"] = lt.value
    return o


def cldprop_columns(state: dict, inflag: int = 2, iceflag: int = 3, liqflag: int = 1) -> np.ndarray:
    """BRAMS's per-column cldprop call (rtm_driver.f90:1250-1258): tauc (16, ncol, nlay)."""
    L = lib()
    ncol, nlay = state["play"].shape
    tauc_in = np.zeros((16, nlay), order="F")
    out = np.zeros((16, ncol, nlay), order="F")
    tc = np.zeros((nlay, 16), order="F")
    nb = C.c_int(0)
    for i in range(ncol):
        cf = np.ascontiguousarray(state["cldfrac"][i, :])
        ci = np.ascontiguousarray(state["ciwp"][i, :])
        cw = np.ascontiguousarray(state["clwp"][i, :])
        re = np.ascontiguousarray(state["rei"][i, :])
        rl = np.ascontiguousarray(state["rel"][i, :])
        rc = L.ora_cldprop(C.c_int(nlay), C.c_int(inflag), C.c_int(iceflag), C.c_int(liqflag),
                           _p(cf), _p(tauc_in), _p(ci), _p(cw), _p(re), _p(rl), C.byref(nb), _p(tc))
        if rc != 0:
            raise RuntimeError(f"oracle cldprop: {L.ora_error_string(rc).decode()}")
        out[:, i, :] = tc.T
    return out


def mcica_subcol_lw(state: dict, tauc: np.ndarray, icld: int, permuteseed: int, irng: int = 1,
                    alpha: np.ndarray | None = None) -> dict:
    """One call of mcica_subcol_lw over all columns (BRAMS draw order)."""
    L = lib()
    ncol, nlay = state["play"].shape
    o = {k: np.zeros((140, ncol, nlay), order="F") for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl")}
    o["reicmcl"] = np.zeros((ncol, nlay), order="F")
    o["relqmcl"] = np.zeros((ncol, nlay), order="F")
    ir = C.c_int(irng)
    rc = L.ora_mcica_subcol_lw(C.c_int(ncol), C.c_int(nlay), C.c_int(icld), C.c_int(permuteseed), C.byref(ir),
                               _p(_f(state["play"])), _p(_f(state["cldfrac"])), _p(_f(state["ciwp"])),
                               _p(_f(state["clwp"])), _p(_f(state["rei"])), _p(_f(state["rel"])),
                               _p(_f(tauc)), _p(_f(alpha) if alpha is not None else None),
                               _p(o["cldfmcl"]), _p(o["ciwpmcl"]), _p(o["clwpmcl"]), _p(o["reicmcl"]),
                               _p(o["relqmcl"]), _p(o["taucmcl"]))
    if rc != 0:
        raise RuntimeError(f"oracle mcica: {L.ora_error_string(rc).decode()}")
    return o


def mcica_per_column(state: dict, tauc: np.ndarray, icld: int, base_seed: int, irng: int = 1) -> dict:
    """Per-column seeding (seed = base + column index, 0-based): the reference
    generator called with ncol = 1 for each column."""
    ncol, nlay = state["play"].shape
    o = {k: np.zeros((140, ncol, nlay), order="F") for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl")}
    o["reicmcl"] = np.asfortranarray(state["rei"].copy())
    o["relqmcl"] = np.asfortranarray(state["rel"].copy())
    for i in range(ncol):
        sub = {k: np.asfortranarray(state[k][i:i + 1, :]) for k in ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")}
        r = mcica_subcol_lw(sub, np.asfortranarray(tauc[:, i:i + 1, :]), icld, base_seed + i, irng)
        for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl"):
            o[k][:, i, :] = r[k][:, 0, :]
    return o


def mt_draws(seed: int, n: int):
    L = lib()
    ints = np.zeros(n, dtype=np.uint32)
    reals = np.zeros(n)
    L.ora_mt_draws(C.c_int32(seed), C.c_int(n), ints.ctypes.data_as(C.POINTER(C.c_uint32)), _p(reals))
    return ints, reals


def kiss_draws(s1: int, s2: int, s3: int, s4: int, n: int) -> np.ndarray:
    L = lib()
    reals = np.zeros(n)
    L.ora_kiss_draws(C.c_int32(s1), C.c_int32(s2), C.c_int32(s3), C.c_int32(s4), C.c_int(n), _p(reals))
    return reals


def lookup_tables():
    L = lib()
    tau, ex, tfn = np.zeros(10001), np.zeros(10001), np.zeros(10001)
    hf, ff = C.c_double(0), C.c_double(0)
    L.ora_get_tables(_p(tau), _p(ex), _p(tfn), C.byref(hf), C.byref(ff))
    return tau, ex, tfn, hf.value, ff.value


def flops_per_column(state: dict, mc: dict, icld: int = 3, idrv: int = 1) -> dict:
    """Floating-point operations (additions, subtractions, multiplications,
    divisions) the restatement executes per column, by phase: a copy of the
    oracle built with a counting number type (flop_count.h) runs rrtmg_lw
    single-threaded on these columns."""
    path = os.path.join(HERE, "_build", "liblworacle_count.so")
    src = os.path.join(HERE, "lw_oracle.cpp")
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    L = C.CDLL(path)
    L.ora_init.restype = C.c_int
    L.ora_init.argtypes = [C.c_double, C.c_char_p, C.c_char_p]
    L.ora_flops.restype = C.c_uint64
    L.ora_flops.argtypes = [C.c_int]
    if L.ora_init(1004.0, os.path.join(DATA, "lw_ref_tables.gblw").encode(),
                  os.path.join(DATA, "lw_ktables.gblw").encode()) != 0:
        raise RuntimeError("oracle init failed")
    ncol, nlay = state["play"].shape
    st = [_f(state[k]) for k in STATE_ORDER]
    cl = [_f(mc[k]) for k in CLOUD_ORDER]
    out = {k: np.zeros((ncol, nlay + 1), order="F") for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt")}
    out["hr"] = np.zeros((ncol, nlay), order="F")
    out["hrc"] = np.zeros((ncol, nlay), order="F")
    ic = C.c_int(icld)
    args = [C.c_int(ncol), C.c_int(nlay), C.byref(ic), C.c_int(idrv)] + [_p(a) for a in st]
    args += [C.c_int(2), C.c_int(3), C.c_int(1)] + [_p(a) for a in cl] + [_p(_f(state["tauaer"]))]
    args += [_p(out[k]) for k in ("uflx", "dflx", "hr", "uflxc", "dflxc", "hrc", "duflx_dt", "duflxc_dt")]
    args += [C.c_int(1)]
    L.ora_flops_reset()
    rc = L.ora_rrtmg_lw(*args)
    if rc != 0:
        raise RuntimeError(f"counting oracle: status {rc}")
    names = ("inatm", "cldprmc", "setcoef", "taumol", "rtrnmc")
    res = {n: L.ora_flops(i) / ncol for i, n in enumerate(names)}
    res["total"] = L.ora_flops(-1) / ncol
    res["outputs"] = out
    return res


# ---------------------------------------------------------------- RRTMG_SW
SW_STATE = ["play", "plev", "tlay", "tlev", "tsfc", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "n2ovmr", "o2vmr",
            "asdir", "asdif", "aldir", "aldif", "coszen"]
SW_CLOUD = ["cldfmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl"]
SW_OUT = ["swuflx", "swdflx", "swhr", "swuflxc", "swdflxc", "swhrc"]


def sw_lib(tuned: bool = False, count: bool = False):
    """The SW oracle (sw_oracle.cpp), built on first use and initialised with
    cpdair 1004; count=True: the copy whose arithmetic counts its operations
    (flop_count.h, single-threaded use)."""
    key = "sw_count" if count else ("sw_tuned" if tuned else "sw")
    if key in _lib:
        return _lib[key]
    name = "libsworacle_count.so" if count else ("libsworacle_tuned.so" if tuned else "libsworacle.so")
    path = os.path.join(HERE, "_build", name)
    src = os.path.join(HERE, "sw_oracle.cpp")
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, os.path.join("_build", os.path.basename(path))], check=True)
    L = C.CDLL(path)
    if count:
        L.ora_flops.restype = C.c_uint64
        L.ora_flops.argtypes = [C.c_int]
    L.ora_sw_init.restype = C.c_int
    L.ora_sw_init.argtypes = [C.c_double, C.c_char_p]
    if L.ora_sw_init(1004.0, os.path.join(DATA, "sw_tables.gbsw").encode()) != 0:
        raise RuntimeError("SW oracle init failed")
    _lib[key] = L
    return L


def rrtmg_sw(state: dict, mc: dict | None, icld: int = 3, iaer: int = 10, adjes: float = 1.0, dyofyr: int = 0,
             scon: float = 1368.22, isolvar: int = -1, inflgsw: int = 2, iceflgsw: int = 3, liqflgsw: int = 1,
             nthreads: int = 1, tuned: bool = False, _count: bool = False) -> dict:
    """rrtmg_sw (rrtmg_sw_rad.f90:243) on Fortran-ordered arrays: state keys
    SW_STATE ((ncol, nlay), (ncol, nlay+1), (ncol,)), aerosols 'tauaer_sw',
    'ssaaer_sw', 'asmaer_sw' (ncol, nlay, 14), McICA arrays SW_CLOUD ((112,
    ncol, nlay); reicmcl/relqmcl (ncol, nlay)).  Returns the outputs, icld,
    iaer."""
    L = sw_lib(tuned, count=_count)
    ncol, nlay = state["play"].shape
    st = [_f(state[k]) for k in SW_STATE]
    z3 = np.zeros((112, ncol, nlay), order="F")
    z2 = np.zeros((ncol, nlay), order="F")
    cl = [_f(mc[k]) if mc is not None else (z2 if k in ("reicmcl", "relqmcl") else z3) for k in SW_CLOUD]
    aer = [_f(state.get(k, np.zeros((ncol, nlay, 14)) if k != "ssaaer_sw" else np.ones((ncol, nlay, 14))))
           for k in ("tauaer_sw", "ssaaer_sw", "asmaer_sw")]
    out = {k: np.zeros((ncol, nlay + 1), order="F") for k in ("swuflx", "swdflx", "swuflxc", "swdflxc")}
    out["swhr"] = np.zeros((ncol, nlay), order="F")
    out["swhrc"] = np.zeros((ncol, nlay), order="F")
    ic, ia = C.c_int(icld), C.c_int(iaer)
    args = [C.c_int(ncol), C.c_int(nlay), C.byref(ic), C.byref(ia)] + [_p(a) for a in st]
    args += [C.c_double(adjes), C.c_int(dyofyr), C.c_double(scon), C.c_int(isolvar), C.c_int(inflgsw),
             C.c_int(iceflgsw), C.c_int(liqflgsw)] + [_p(a) for a in cl] + [_p(a) for a in aer]
    args += [_p(out[k]) for k in SW_OUT] + [C.c_int(nthreads)]
    rc = L.ora_rrtmg_sw(*args)
    if rc != 0:
        raise RuntimeError(f"SW oracle status {rc}")
    out["icld"], out["iaer"] = ic.value, ia.value
    return out


def sw_flops_per_column(state: dict, mc: dict | None, **kw) -> float:
    """Floating-point operations (additions, subtractions, multiplications,
    divisions) the SW restatement executes per column: the counting copy of
    the oracle (flop_count.h) runs rrtmg_sw single-threaded on these columns."""
    L = sw_lib(count=True)
    L.ora_flops_reset()
    rrtmg_sw(state, mc, nthreads=1, _count=True, **kw)
    return L.ora_flops(-1) / state["play"].shape[0]


SW_CLDPROP_OUT = ["taucldorig", "taucloud", "ssacloud", "asmcloud"]


def cldprop_sw_columns(state: dict, band_in: dict | None = None, inflag: int = 2, iceflag: int = 3,
                       liqflag: int = 1) -> tuple[dict, np.ndarray]:
    """BRAMS's per-column cldprop_sw call (rtm_driver.f90:1356-1368): state
    cldfrac ciwp clwp rei rel (ncol, nlay); band_in tauc ssac asmc fsfc
    (14, ncol, nlay) (None: zeros, as the driver passes for inflag 2).
    Returns taucldorig taucloud ssacloud asmcloud (14, ncol, nlay) -- the
    layout mcica_subcol_sw takes -- and the status of each column (0, or
    the code of the STOP the reference reaches; that column's outputs are
    then left 0)."""
    L = sw_lib()
    ncol, nlay = state["cldfrac"].shape
    z = np.zeros((14, ncol, nlay))
    bi = {k: (band_in[k] if band_in is not None and k in band_in else z) for k in ("tauc", "ssac", "asmc", "fsfc")}
    out = {k: np.zeros((14, ncol, nlay), order="F") for k in SW_CLDPROP_OUT}
    status = np.zeros(ncol, dtype=np.int64)
    tmp = {k: np.zeros((nlay, 14), order="F") for k in SW_CLDPROP_OUT}
    col = lambda a, i: np.ascontiguousarray(a[i, :], dtype=np.float64)  # noqa: E731
    for i in range(ncol):
        ins = [np.asfortranarray(bi[k][:, i, :], dtype=np.float64) for k in ("tauc", "ssac", "asmc", "fsfc")]
        rc = L.ora_cldprop_sw(C.c_int(nlay), C.c_int(inflag), C.c_int(iceflag), C.c_int(liqflag),
                              _p(col(state["cldfrac"], i)), *[_p(a) for a in ins],
                              *[_p(col(state[k], i)) for k in ("ciwp", "clwp", "rei", "rel")],
                              *[_p(tmp[k]) for k in SW_CLDPROP_OUT])
        status[i] = rc
        if rc == 0:
            for k in SW_CLDPROP_OUT:
                out[k][:, i, :] = tmp[k].T
    return out, status


def mcica_subcol_sw(state: dict, band: dict, icld: int, permuteseed: int, irng: int = 1) -> dict:
    """mcica_subcol_sw (mcica_subcol_gen_sw.f90:181): one call over all columns."""
    L = lib()
    ncol, nlay = state["play"].shape
    ins = [_f(state[k]) for k in ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")]
    ins += [_f(band[k]) for k in ("tauc", "ssac", "asmc", "fsfc")]
    alpha = _f(state["alpha"]) if "alpha" in state else None
    o = {k: np.zeros((112, ncol, nlay), order="F") for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl", "ssacmcl",
                                                             "asmcmcl", "fsfcmcl")}
    o["reicmcl"] = np.zeros((ncol, nlay), order="F")
    o["relqmcl"] = np.zeros((ncol, nlay), order="F")
    ir = C.c_int(irng)
    outs = [o[k] for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl", "ssacmcl", "asmcmcl",
                           "fsfcmcl")]
    rc = L.ora_mcica_subcol_sw(C.c_int(ncol), C.c_int(nlay), C.c_int(icld), C.c_int(permuteseed), C.byref(ir),
                               *[_p(a) for a in ins], _p(alpha), *[_p(a) for a in outs])
    if rc != 0:
        raise RuntimeError(f"oracle mcica_subcol_sw: {L.ora_error_string(rc).decode()}")
    return o
