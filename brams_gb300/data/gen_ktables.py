"""Seeded synthetic k-distribution tables for RRTMG_LW, reduced 256 -> 140 g-points.

The reference's absorption-coefficient data module (``rrtmg_lw_k_g.f90``,
AER RRTMG_LW v5.0, ``lw_kgb01..16``) is not distributed with the reference
tree, so the solver is exercised on tables that this script generates.  They
have exactly the array shapes of the reference's 16-point ("o") tables in
``src/rrtmg/RRTMG_LW/modules/rrlw_kg01.f90 .. rrlw_kg16.f90`` and are reduced
to the 140-g-point tables the solver uses with the reference's own reduction
(``rrtmg_lw_init.f90:144-192`` for ``rwgt`` and ``cmbgb1..16`` at
``rrtmg_lw_init.f90:385-2034``): every absorption-type table is summed over
the original g-points of each reduced interval with weights
``rwgt = wt(ig)/sum(wt over the interval)``, and every Planck-fraction table
is summed without weights.

The values are smooth functions of the table coordinates (pressure level,
temperature column, binary-species mixing index, g-point) times a seeded
multiplicative perturbation, so that any index transposition changes the
result.  Magnitudes are chosen per absorber so that column optical depths
span roughly 1e-2 .. 1e3 across the g-points of a band, which puts
broadband fluxes of standard profiles in the physical 150-450 W m-2 range.
No values of the AER data are reproduced.

Usage:  python brams_gb300/data/gen_ktables.py   (writes lw_ktables.gblw)
"""
from __future__ import annotations

import os
import sys
from collections import OrderedDict

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from brams_gb300.tables_io import read_tables, write_tables  # noqa: E402

SEED = 0x5EED_1E57_0B57  # fixed: the tables are part of the test contract
NG16 = 16
NSPA = (1, 1, 9, 9, 9, 1, 9, 1, 9, 1, 1, 9, 9, 1, 9, 9)
NSPB = (1, 1, 5, 5, 5, 0, 1, 1, 1, 1, 1, 0, 0, 1, 0, 0)

# Original (16-point) table inventory per band: name -> (shape without g, g-axis position)
# "g_last" tables have g as the last Fortran index, "g_first" (fracref) as the first.
def _band_tables(b: int) -> "OrderedDict[str, tuple]":
    """Shapes of the 16-point tables of band b, from modules/rrlw_kgNN.f90."""
    t: "OrderedDict[str, tuple]" = OrderedDict()
    na, nb = NSPA[b - 1], NSPB[b - 1]
    lower_binary = na > 1
    # major absorbers
    t["kao"] = ((9, 5, 13) if lower_binary else (5, 13), "k")
    has_kb = b not in (6, 12, 13, 15)
    if has_kb:
        t["kbo"] = ((5, 5, 47) if nb > 1 else (5, 47), "k")
    # planck fractions
    t["fracrefao"] = ((9,) if lower_binary else (), "f")
    if b not in (6, 12, 15):
        upper_binary = nb > 1
        t["fracrefbo"] = ((5,) if upper_binary else (), "f")
    t["selfrefo"] = ((10,), "k")
    t["forrefo"] = ((4,), "k")
    minors = {
        1: [("kao_mn2", (19,)), ("kbo_mn2", (19,))],
        3: [("kao_mn2o", (9, 19)), ("kbo_mn2o", (5, 19))],
        5: [("kao_mo3", (9, 19)), ("ccl4o", ())],
        6: [("kao_mco2", (19,)), ("cfc11adjo", ()), ("cfc12o", ())],
        7: [("kao_mco2", (9, 19)), ("kbo_mco2", (19,))],
        8: [("kao_mco2", (19,)), ("kao_mn2o", (19,)), ("kao_mo3", (19,)),
            ("kbo_mco2", (19,)), ("kbo_mn2o", (19,)), ("cfc12o", ()), ("cfc22adjo", ())],
        9: [("kao_mn2o", (9, 19)), ("kbo_mn2o", (19,))],
        11: [("kao_mo2", (19,)), ("kbo_mo2", (19,))],
        13: [("kao_mco2", (9, 19)), ("kao_mco", (9, 19)), ("kbo_mo3", (19,))],
        15: [("kao_mn2", (9, 19))],
    }
    for name, shp in minors.get(b, []):
        t[name] = (shp, "k")
    return t


# Key-absorber magnitude class per band, lower and upper atmosphere:
# (log10 of the weakest-g coefficient, decades spanned across the 16 g-points)
_MAJOR = {
    1: ((-5.0, 5.5), (-5.0, 5.0)), 2: ((-5.0, 5.0), (-5.0, 4.5)),
    3: ((-5.0, 5.5), (-4.5, 5.0)), 4: ((-5.5, 5.0), (-1.5, 4.0)),
    5: ((-5.5, 5.0), (-1.5, 4.0)), 6: ((-5.5, 4.0), None),
    7: ((-5.5, 5.0), (-1.0, 3.5)), 8: ((-6.0, 4.5), (-1.0, 3.5)),
    9: ((-5.5, 5.0), (-2.0, 4.0)), 10: ((-5.0, 5.0), (-5.0, 4.5)),
    11: ((-5.0, 5.0), (-5.0, 4.5)), 12: ((-5.5, 4.5), None),
    13: ((-5.5, 4.5), None), 14: ((-4.0, 5.0), (-4.0, 4.5)),
    15: ((-2.0, 4.0), None), 16: ((-5.0, 5.0), (-2.0, 4.0)),
}
# minor-gas magnitude (log10 weakest g, decades)
_MINOR = {
    "mn2": (-7.5, 2.0), "mn2o": (-1.0, 3.0), "mo3": (-1.0, 3.0), "mco2": (-4.0, 3.0),
    "mo2": (-7.5, 3.0), "mco": (0.0, 2.0), "ccl4o": (2.5, 1.0), "cfc11adjo": (3.0, 1.0),
    "cfc12o": (3.0, 1.0), "cfc22adjo": (2.5, 1.0),
}


def _gprof(lo: float, span: float) -> np.ndarray:
    g = np.arange(NG16, dtype=np.float64)
    return 10.0 ** (lo + span * g / (NG16 - 1))


def _noise(rng: np.random.Generator, shape, amp: float = 0.25) -> np.ndarray:
    u = rng.random(shape)
    return np.exp(amp * (u - 0.5))


def make_original_tables(ref: dict) -> "OrderedDict[str, np.ndarray]":
    """All 16-point tables for the 16 bands, keyed 'bNN.<name>' (Fortran order arrays)."""
    rng = np.random.Generator(np.random.PCG64(SEED))
    pref, tref = ref["pref"], ref["tref"]
    wt = ref["wt"]
    out: "OrderedDict[str, np.ndarray]" = OrderedDict()
    for b in range(1, 17):
        for name, (shp, kind) in _band_tables(b).items():
            key = f"b{b:02d}.{name}"
            if kind == "f":
                # planck fractions: shape (16, neta); ~wt with smooth eta/g modulation, sum 1 over g
                neta = shp[0] if shp else 1
                g = np.arange(NG16)[:, None]
                eta = (np.arange(neta)[None, :] / max(neta - 1, 1))
                v = wt[:, None] * (1.0 + 0.35 * np.sin(0.7 * g + 2.3 * eta + 0.4 * b)) * _noise(rng, (NG16, neta), 0.1)
                v = v / v.sum(axis=0, keepdims=True)
                out[key] = v if shp else v[:, 0]
                continue
            full = tuple(shp) + (NG16,)
            if name in ("kao", "kbo"):
                upper = name == "kbo"
                mag = _MAJOR[b][1 if upper else 0]
                gp = _gprof(*mag)
                binary = len(shp) == 3
                if binary:
                    nsp, _, njp = shp
                else:
                    nsp, njp = 1, shp[1]
                jp0 = 13 if upper else 1
                jp = np.arange(jp0, jp0 + njp)
                p = pref[jp - 1]
                t = tref[jp - 1][None, :] + 15.0 * (np.arange(5)[:, None] - 2.0)  # (5, njp)
                alpha = 0.55 + 0.25 * np.linspace(0.0, 1.0, NG16)
                pf = (p[None, :, None] / 1013.25) ** alpha[None, None, :]  # (1, njp, g)
                beta = -1.2 + 0.9 * np.sin(np.arange(NG16) * 0.9 + b)
                tf = (t[:, :, None] / 250.0) ** beta[None, None, :]  # (5, njp, g)
                base = gp[None, None, :] * pf * tf  # (5, njp, g)
                if binary:
                    eta = np.arange(nsp) / (nsp - 1)
                    ratio = 10.0 ** (0.8 * np.cos(0.5 * np.arange(NG16) + b))
                    mix = eta[:, None] + (1.0 - eta[:, None]) * ratio[None, :]  # (nsp, g)
                    v = mix[:, None, None, :] * base[None, :, :, :]
                else:
                    v = base
                out[key] = v * _noise(rng, v.shape)
            elif name == "selfrefo":
                tcol = 188.0 + 7.2 * (np.arange(10) + 7.0)
                v = (2e-2 * 10.0 ** (0.8 * np.arange(NG16) / 15.0))[None, :] * (296.0 / tcol[:, None]) ** 4.5
                out[key] = v * _noise(rng, v.shape, 0.1)
            elif name == "forrefo":
                v = np.tile((1.5e-3 * 10.0 ** (0.8 * np.arange(NG16) / 15.0))[None, :], (4, 1))
                v = v * (1.0 + 0.1 * np.arange(4))[:, None]
                out[key] = v * _noise(rng, v.shape, 0.1)
            else:
                gas = name.split("_")[1] if "_" in name else name
                lo, span = _MINOR[gas]
                gp = _gprof(lo, span)
                if shp == ():
                    v = gp.copy()
                else:
                    tcol = np.arange(19)
                    tf = (1.0 + 0.03 * (tcol - 9.0))[:, None]
                    v = tf * gp[None, :]
                    if len(shp) == 2:
                        eta = np.arange(shp[0]) / (shp[0] - 1)
                        v = (0.5 + eta)[:, None, None] * v[None, :, :]
                out[key] = v * _noise(rng, v.shape, 0.2)
    return out


def rwgt_table(ref: dict) -> np.ndarray:
    """rwgt(256) exactly as rrtmg_lw_ini builds it (rrtmg_lw_init.f90:144-173)."""
    ngc, ngn, ngm, wt = ref["ngc"], ref["ngn"], ref["ngm"], ref["wt"]
    rwgt = np.zeros(256)
    igcsm = 0
    for ibnd in range(16):
        iprsm = 0
        if ngc[ibnd] < NG16:
            wtsm = np.zeros(NG16)
            for igc in range(ngc[ibnd]):
                igcsm += 1
                wtsum = 0.0
                for _ in range(ngn[igcsm - 1]):
                    iprsm += 1
                    wtsum = wtsum + wt[iprsm - 1]
                wtsm[igc] = wtsum
            for ig in range(NG16):
                ind = ibnd * NG16 + ig
                rwgt[ind] = wt[ig] / wtsm[ngm[ind] - 1]
        else:
            for ig in range(NG16):
                igcsm += 1
                rwgt[ibnd * NG16 + ig] = 1.0
    return rwgt


def reduce_tables(orig: dict, ref: dict) -> "OrderedDict[str, np.ndarray]":
    """cmbgb1..16: combine the 16 original g-points into ngc(b) reduced ones."""
    ngc, ngs, ngn = ref["ngc"], ref["ngs"], ref["ngn"]
    rwgt = rwgt_table(ref)
    out: "OrderedDict[str, np.ndarray]" = OrderedDict()
    for key, arr in orig.items():
        b = int(key[1:3])
        name = key.split(".")[1]
        rname = name[:-1] if name.endswith("o") else name.replace("o_", "_")
        if name.startswith("ka") or name.startswith("kb"):
            rname = name[:2] + name[3:]  # kao -> ka, kao_mn2 -> ka_mn2
        nred = int(ngc[b - 1])
        g0 = 0 if b == 1 else int(ngs[b - 2])
        is_frac = name.startswith("fracref")
        a = np.asarray(arr, dtype=np.float64)
        if is_frac:
            a = np.moveaxis(a, 0, -1) if a.ndim == 2 else a  # g to last for the loop
        red = np.zeros(a.shape[:-1] + (nred,))
        iprsm = 0
        for igc in range(nred):
            s = np.zeros(a.shape[:-1])
            for _ in range(int(ngn[g0 + igc])):
                iprsm += 1
                if is_frac:
                    s = s + a[..., iprsm - 1]
                else:
                    s = s + a[..., iprsm - 1] * rwgt[(b - 1) * NG16 + iprsm - 1]
            red[..., igc] = s
        if is_frac and red.ndim == 2:
            red = np.moveaxis(red, -1, 0)  # back to (ng, neta)
        out[f"b{b:02d}.{rname}"] = red
    return out


def main() -> None:
    ref = read_tables(os.path.join(HERE, "lw_ref_tables.gblw"))
    orig = make_original_tables(ref)
    red = reduce_tables(orig, ref)
    dst = os.path.join(HERE, "lw_ktables.gblw")
    write_tables(dst, red)
    n = sum(v.size for v in red.values())
    print(f"wrote {dst}: {len(red)} tables, {n} values")


if __name__ == "__main__":
    main()
