"""Extract the RRTMG_SW tables from the reference source and reduce them to 112 g-points.

RRTMG_SW carries all of its data in its source:

* ``src/rrtmg/RRTMG_SW/src/rrtmg_sw_k_g.f90``  sw_kgb16..29: the 16-point
  k-distribution tables of every band (kao, kbo, selfrefo, forrefo,
  sfluxrefo, Rayleigh and minor-absorber coefficients);
* ``src/rrtmg/RRTMG_SW/src/rrtmg_sw_init.f90:174-260`` swdatinit (band
  limits, nspa/nspb, physical constants), ``:262-386`` swcmbdat (the
  16 -> 112 g-point maps and weights), ``:1692-3514`` swcldpr (cloud
  optics of liquid and ice);
* ``src/rrtmg/RRTMG_SW/src/rrtmg_sw_setcoef.f90`` swatmref (pref,
  preflog, tref);
* ``src/rrtmg/RRTMG_SW/modules/parrrsw.f90`` rrsw_scon.

The reduction is rrtmg_sw_ini's (rrtmg_sw_init.f90:99-172 for the weights
rwgt, :492-1689 cmbgb16s..cmbgb29): every table with a g-point axis is
combined as sum(table * rwgt) over the original g-points of each reduced
one, except the solar source sfluxref, which is a plain sum; sums run in
the reference's order, starting from 0.  Values with the ``_rb`` suffix are
double precision, values without it default (single precision) reals.

Output ``sw_tables.gbsw`` (container format of ``brams_gb300/tables_io.py``):
constants under their module names, band tables as ``bNN.<name>`` with the
reference's reduced shapes (``absa`` (nspa*65, ng) and ``absb`` (nspb*235,
ng), the equivalenced views taumol indexes).

Usage:  python -m brams_gb300.data.extract_sw_tables <luflarois/brams source tree>
"""
from __future__ import annotations

import os
import re
import sys
from collections import OrderedDict

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from brams_gb300.data.extract_ref_tables import _literal, _statements  # noqa: E402
from brams_gb300.tables_io import write_tables  # noqa: E402

SW = "src/rrtmg/RRTMG_SW"
NG = {16: 6, 17: 12, 18: 8, 19: 8, 20: 10, 21: 10, 22: 2, 23: 10, 24: 8, 25: 6, 26: 6, 27: 8, 28: 6, 29: 12}

# per band: name -> shape of the 16-point array as ((lower, upper) per dimension);
# "G" marks the g-point axis (16 values)
G = (1, 16)
_KA9 = ((1, 9), (1, 5), (1, 13), G)
_KA1 = ((1, 5), (1, 13), G)
_KB1 = ((1, 5), (13, 59), G)
_KB5 = ((1, 5), (1, 5), (13, 59), G)
BANDS = {
    16: {"kao": _KA9, "kbo": _KB1, "selfrefo": ((1, 10), G), "forrefo": ((1, 3), G), "sfluxrefo": (G,), "rayl": ()},
    17: {"kao": _KA9, "kbo": _KB5, "selfrefo": ((1, 10), G), "forrefo": ((1, 4), G), "sfluxrefo": (G, (1, 5)), "rayl": ()},
    18: {"kao": _KA9, "kbo": _KB1, "selfrefo": ((1, 10), G), "forrefo": ((1, 3), G), "sfluxrefo": (G, (1, 9)), "rayl": ()},
    19: {"kao": _KA9, "kbo": _KB1, "selfrefo": ((1, 10), G), "forrefo": ((1, 3), G), "sfluxrefo": (G, (1, 9)), "rayl": ()},
    20: {"kao": _KA1, "kbo": _KB1, "selfrefo": ((1, 10), G), "forrefo": ((1, 4), G), "sfluxrefo": (G,), "absch4o": (G,),
         "rayl": ()},
    21: {"kao": _KA9, "kbo": _KB5, "selfrefo": ((1, 10), G), "forrefo": ((1, 4), G), "sfluxrefo": (G, (1, 9)), "rayl": ()},
    22: {"kao": _KA9, "kbo": _KB1, "selfrefo": ((1, 10), G), "forrefo": ((1, 3), G), "sfluxrefo": (G, (1, 9)), "rayl": ()},
    23: {"kao": _KA1, "selfrefo": ((1, 10), G), "forrefo": ((1, 3), G), "sfluxrefo": (G,), "raylo": (G,)},
    24: {"kao": _KA9, "kbo": _KB1, "selfrefo": ((1, 10), G), "forrefo": ((1, 3), G), "sfluxrefo": (G, (1, 9)),
         "abso3ao": (G,), "abso3bo": (G,), "raylao": (G, (1, 9)), "raylbo": (G,)},
    25: {"kao": _KA1, "sfluxrefo": (G,), "abso3ao": (G,), "abso3bo": (G,), "raylo": (G,)},
    26: {"sfluxrefo": (G,), "raylo": (G,)},
    27: {"kao": _KA1, "kbo": _KB1, "sfluxrefo": (G,), "raylo": (G,)},
    28: {"kao": _KA9, "kbo": _KB5, "sfluxrefo": (G, (1, 5)), "rayl": ()},
    29: {"kao": _KA1, "kbo": _KB1, "selfrefo": ((1, 10), G), "forrefo": ((1, 4), G), "sfluxrefo": (G,),
         "absh2oo": (G,), "absco2o": (G,), "rayl": ()},
}

# constants: name -> (shape, kind, source file, subroutine)
CONSTS = OrderedDict([
    ("pref", ((59,), "f")), ("preflog", ((59,), "f")), ("tref", ((59,), "f")),
    ("wavenum1", ((14,), "f")), ("wavenum2", ((14,), "f")), ("delwave", ((14,), "f")),
    ("nspa", ((14,), "i")), ("nspb", ((14,), "i")),
    ("grav", ((), "f")), ("avogad", ((), "f")), ("secdy", ((), "f")),
    ("ngc", ((14,), "i")), ("ngs", ((14,), "i")), ("ngm", ((224,), "i")), ("ngn", ((112,), "i")),
    ("ngb", ((112,), "i")), ("wt", ((16,), "f")),
    ("extliq1", ((58, 14), "f")), ("ssaliq1", ((58, 14), "f")), ("asyliq1", ((58, 14), "f")),
    ("extice2", ((43, 14), "f")), ("ssaice2", ((43, 14), "f")), ("asyice2", ((43, 14), "f")),
    ("extice3", ((46, 14), "f")), ("ssaice3", ((46, 14), "f")), ("asyice3", ((46, 14), "f")),
    ("fdlice3", ((46, 14), "f")),
    ("abari", ((5,), "f")), ("bbari", ((5,), "f")), ("cbari", ((5,), "f")), ("dbari", ((5,), "f")),
    ("ebari", ((5,), "f")), ("fbari", ((5,), "f")),
])
CONST_SOURCES = [
    (f"{SW}/src/rrtmg_sw_setcoef.f90", ("swatmref",)),
    (f"{SW}/src/rrtmg_sw_init.f90", ("swdatinit", "swcmbdat", "swcldpr")),
]
# the cloud tables are declared (58, 16:29) etc.: band subscripts start at 16
LOWER = {k: (1, 16) for k in ("extliq1", "ssaliq1", "asyliq1", "extice2", "ssaice2", "asyice2", "extice3",
                              "ssaice3", "asyice3", "fdlice3")}


def _subscript(sub: str, dims):
    """Fortran subscript text -> numpy index for an array with (lower, upper) dims."""
    parts = [p.strip() for p in sub.split(",")]
    if len(parts) != len(dims):
        raise ValueError(f"subscript {sub} vs {dims}")
    idx = []
    for p, (lo, hi) in zip(parts, dims):
        if p == ":":
            idx.append(slice(0, hi - lo + 1))
        elif ":" in p:
            a, b = p.split(":")
            idx.append(slice(int(a) - lo, int(b) - lo + 1))
        else:
            idx.append(int(p) - lo)
    return tuple(idx)


def _assign(statements, want, arrays, filled):
    for st in statements:
        m = re.match(r"([A-Za-z_][A-Za-z0-9_]*)\s*(\(([^=]*)\))?\s*=\s*(.*)$", st)
        if not m:
            continue
        name = m.group(1).lower()
        if name not in want:
            continue
        dims = want[name]
        rhs = m.group(4).strip()
        if rhs.startswith("(/"):
            body = rhs[2:rhs.rindex("/)")]
            vals = [_literal(t)[0] for t in body.split(",") if t.strip()]
        else:
            try:
                vals = [_literal(rhs)[0]]
            except ValueError:
                continue
        shape = tuple(hi - lo + 1 for lo, hi in dims)
        idx = _subscript(m.group(3), dims) if m.group(3) else tuple(slice(0, n) for n in shape)
        tgt = arrays[name][idx]
        if np.size(tgt) != len(vals):
            raise ValueError(f"{name}({m.group(3)}): {len(vals)} values for {np.size(tgt)} slots")
        arrays[name][idx] = np.array(vals, dtype=np.float64).reshape(np.shape(tgt), order="F")
        filled[name][idx] = True


def extract_constants(root: str) -> "OrderedDict[str, np.ndarray]":
    want = {}
    for k, (shape, _) in CONSTS.items():
        lo = LOWER.get(k, (1,) * len(shape))
        want[k] = tuple((l, l + n - 1) for l, n in zip(lo, shape))
    arrays = {k: np.full(CONSTS[k][0], np.nan) for k in CONSTS}
    filled = {k: np.zeros(CONSTS[k][0], dtype=bool) for k in CONSTS}
    for rel, subs in CONST_SOURCES:
        text = open(os.path.join(root, rel)).read()
        for sub in subs:
            _assign(_statements(text, sub), want, arrays, filled)
    out = OrderedDict()
    for k, (shape, kind) in CONSTS.items():
        if not filled[k].all():
            raise ValueError(f"{k}: {int((~filled[k]).sum())} entries not found")
        out[k] = arrays[k].astype(np.int32) if kind == "i" else arrays[k]
    # parrrsw.f90: rrsw_scon = 1.36822e+03, a default (single precision) real
    txt = open(os.path.join(root, SW, "modules", "parrrsw.f90")).read()
    m = re.search(r"rrsw_scon\s*=\s*([0-9.eE+-]+(?:_rb)?)", txt)
    out["rrsw_scon"] = np.float64(_literal(m.group(1))[0])
    return out


def extract_bands(root: str) -> "dict[int, dict[str, np.ndarray]]":
    text = open(os.path.join(root, SW, "src", "rrtmg_sw_k_g.f90")).read()
    bands = {}
    for b, spec in BANDS.items():
        arrays = {k: np.full(tuple(hi - lo + 1 for lo, hi in d), np.nan) for k, d in spec.items()}
        filled = {k: np.zeros(a.shape, dtype=bool) for k, a in arrays.items()}
        _assign(_statements(text, f"sw_kgb{b}"), spec, arrays, filled)
        for k in spec:
            if not filled[k].all():
                raise ValueError(f"band {b} {k}: {int((~filled[k]).sum())} entries not found")
        bands[b] = arrays
    return bands


def reduction_weights(c) -> np.ndarray:
    """rwgt(224) of rrtmg_sw_ini (rrtmg_sw_init.f90:146-172)."""
    ngc, ngn, ngm, wt = c["ngc"], c["ngn"], c["ngm"], c["wt"]
    rwgt = np.zeros(224)
    igcsm = 0
    for ibnd in range(14):
        iprsm = 0
        wtsm = np.zeros(16)
        for igc in range(ngc[ibnd]):
            igcsm += 1
            wtsum = 0.0
            for _ in range(ngn[igcsm - 1]):
                iprsm += 1
                wtsum = wtsum + wt[iprsm - 1]
            wtsm[igc] = wtsum
        for ig in range(16):
            ind = ibnd * 16 + ig
            rwgt[ind] = wt[ig] / wtsm[ngm[ind] - 1]
    return rwgt


def _combine(a: np.ndarray, gaxis: int, counts, w) -> np.ndarray:
    """Sum runs of the g axis: run j takes counts[j] original g-points, each
    multiplied by w (None: a plain sum), accumulated from 0 in order."""
    a = np.moveaxis(a, gaxis, -1)
    out = np.zeros(a.shape[:-1] + (len(counts),))
    ipr = 0
    for j, n in enumerate(counts):
        s = np.zeros(a.shape[:-1])
        for _ in range(n):
            s = s + (a[..., ipr] * w[ipr] if w is not None else a[..., ipr])
            ipr += 1
        out[..., j] = s
    return np.moveaxis(out, -1, gaxis)


def reduce_bands(c, bands) -> "OrderedDict[str, np.ndarray]":
    rwgt = reduction_weights(c)
    out = OrderedDict()
    gs = 0
    for b in range(16, 30):
        ib = b - 16
        counts = [int(x) for x in c["ngn"][gs:gs + NG[b]]]
        gs += NG[b]
        w = rwgt[ib * 16:(ib + 1) * 16]
        for name, arr in bands[b].items():
            dims = BANDS[b][name]
            if not dims:  # a scalar Rayleigh coefficient, used as is
                out[f"b{b}.rayl"] = np.float64(arr)
                continue
            gaxis = dims.index(G)
            red = _combine(arr, gaxis, counts, None if name == "sfluxrefo" else w)
            base = name[:-1] if name.endswith("o") else name
            if base == "ka":
                out[f"b{b}.absa"] = red.reshape((-1, NG[b]), order="F")
            elif base == "kb":
                out[f"b{b}.absb"] = red.reshape((-1, NG[b]), order="F")
            else:
                out[f"b{b}.{base}"] = red
    return out


def extract(root: str) -> "OrderedDict[str, np.ndarray]":
    c = extract_constants(root)
    out = OrderedDict(c)
    out.update(reduce_bands(c, extract_bands(root)))
    return out


def main() -> None:
    if len(sys.argv) != 2:
        sys.exit(f"usage: python -m brams_gb300.data.{os.path.basename(__file__)[:-3]} <luflarois/brams source tree>")
    tabs = extract(sys.argv[1])
    dst = os.path.join(HERE, "sw_tables.gbsw")
    write_tables(dst, tabs)
    print(f"wrote {dst}: {len(tabs)} tables, " + ", ".join(f"{k}{tuple(np.shape(v))}" for k, v in list(tabs.items())[:8]))


if __name__ == "__main__":
    main()
