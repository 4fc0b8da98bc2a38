"""Extract the RRTMG_LW constant tables that the reference carries in its source.

The reference initialises its longwave tables with Fortran array-constructor
assignments inside ``rrtmg_lw_ini`` and ``setcoef``'s data routines:

* ``src/rrtmg/RRTMG_LW/src/rrtmg_lw_setcoef.f90:437-597``  lwatmref
  (pref, preflog, tref, chi_mls)
* ``src/rrtmg/RRTMG_LW/src/rrtmg_lw_setcoef.f90:600-1303`` lwavplank
  (totplnk, totplk16)
* ``src/rrtmg/RRTMG_LW/src/rrtmg_lw_setcoef.f90:1306-2009`` lwavplankderiv
  (totplnkderiv, totplk16deriv)
* ``src/rrtmg/RRTMG_LW/src/rrtmg_lw_init.f90:197-300``  lwdatinit
  (wavenumber bounds, delwave, nspa/nspb, physical constants)
* ``src/rrtmg/RRTMG_LW/src/rrtmg_lw_init.f90:303-382``  lwcmbdat
  (ngc, ngs, ngm, ngn, ngb, wt: the 256 -> 140 g-point reduction maps)
* ``src/rrtmg/RRTMG_LW/src/rrtmg_lw_init.f90:2037-2675`` lwcldpr
  (abscld1, absice0..3, absliq0..1 cloud absorption tables)

These are numeric tables whose values must be identical to the reference's
for parity, so this script reads them out of the Fortran source and writes
them into ``lw_ref_tables.gblw`` (format: ``brams_gb300/tables_io.py``).
Literals with the ``_rb`` kind suffix are double precision; literals without
it are default (single precision) reals in Fortran and are rounded through
float32, exactly as the Fortran compiler stores them.

Usage:  python brams_gb300/data/extract_ref_tables.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import os
import re
import sys
from collections import OrderedDict

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from brams_gb300.tables_io import write_tables  # noqa: E402

# name -> (shape, dtype); every array starts at Fortran index 1.
WANTED = OrderedDict(
    [
        ("pref", ((59,), "f")),
        ("preflog", ((59,), "f")),
        ("tref", ((59,), "f")),
        ("chi_mls", ((7, 59), "f")),
        ("totplnk", ((181, 16), "f")),
        ("totplk16", ((181,), "f")),
        ("totplnkderiv", ((181, 16), "f")),
        ("totplk16deriv", ((181,), "f")),
        ("wavenum1", ((16,), "f")),
        ("wavenum2", ((16,), "f")),
        ("delwave", ((16,), "f")),
        ("nspa", ((16,), "i")),
        ("nspb", ((16,), "i")),
        ("grav", ((), "f")),
        ("avogad", ((), "f")),
        ("sbcnst", ((), "f")),
        ("secdy", ((), "f")),
        ("ngc", ((16,), "i")),
        ("ngs", ((16,), "i")),
        ("ngm", ((256,), "i")),
        ("ngn", ((140,), "i")),
        ("ngb", ((140,), "i")),
        ("wt", ((16,), "f")),
        ("abscld1", ((), "f")),
        ("absice0", ((2,), "f")),
        ("absice1", ((2, 5), "f")),
        ("absice2", ((43, 16), "f")),
        ("absice3", ((46, 16), "f")),
        ("absliq0", ((), "f")),
        ("absliq1", ((58, 16), "f")),
    ]
)

SOURCES = [
    ("src/rrtmg/RRTMG_LW/src/rrtmg_lw_setcoef.f90", ("lwatmref", "lwavplank", "lwavplankderiv")),
    ("src/rrtmg/RRTMG_LW/src/rrtmg_lw_init.f90", ("lwdatinit", "lwcmbdat", "lwcldpr")),
]

_NUM = re.compile(r"[+-]?(?:\d+\.\d*|\.\d+|\d+)(?:[eEdD][+-]?\d+)?(?:_rb|_im)?")


def _strip_comment(line: str) -> str:
    # No character literals appear in the data routines except version
    # strings of the form '$Revision$', which contain no '!'.
    i = line.find("!")
    return line if i < 0 else line[:i]


def _statements(text: str, subroutine: str) -> list[str]:
    lines = text.splitlines()
    start = None
    for i, ln in enumerate(lines):
        if re.match(rf"\s*subroutine\s+{subroutine}\b", ln, re.I):
            start = i
            break
    if start is None:
        raise ValueError(f"subroutine {subroutine} not found")
    out, cur = [], ""
    for ln in lines[start + 1:]:
        if re.match(r"\s*end\s+subroutine", ln, re.I):
            break
        s = _strip_comment(ln).rstrip()
        if not s.strip():
            continue
        s = s.strip()
        if s.startswith("&"):
            s = s[1:]
        if s.endswith("&"):
            cur += s[:-1] + " "
            continue
        out.append(cur + s)
        cur = ""
    return out


def _literal(tok: str):
    tok = tok.strip()
    if tok.endswith("_im"):
        return int(tok[:-3]), "i"
    if tok.endswith("_rb"):
        return float(tok[:-3].replace("d", "e").replace("D", "e")), "f"
    if re.fullmatch(r"[+-]?\d+", tok):
        return int(tok), "i"
    # default real literal: single precision in Fortran
    return float(np.float32(float(tok.replace("d", "e").replace("D", "e")))), "f"


def _index(sub: str, shape: tuple[int, ...]):
    parts = [p.strip() for p in sub.split(",")]
    if len(parts) != len(shape):
        raise ValueError(f"subscript {sub} vs shape {shape}")
    idx = []
    for p, n in zip(parts, shape):
        if p == ":":
            idx.append(slice(0, n))
        elif ":" in p:
            a, b = p.split(":")
            idx.append(slice(int(a) - 1, int(b)))
        else:
            idx.append(int(p) - 1)
    return tuple(idx)


def extract(ref_root: str) -> "OrderedDict[str, np.ndarray]":
    arrays = {k: np.full(v[0], np.nan) for k, v in WANTED.items()}
    filled = {k: np.zeros(v[0], dtype=bool) for k, v in WANTED.items()}
    for rel, subs in SOURCES:
        with open(os.path.join(ref_root, rel)) as f:
            text = f.read()
        for sub in subs:
            for st in _statements(text, sub):
                m = re.match(r"([A-Za-z_][A-Za-z0-9_]*)\s*(\(([^=]*)\))?\s*=\s*(.*)$", st)
                if not m:
                    continue
                name = m.group(1).lower()
                if name not in WANTED:
                    continue
                shape, kind = WANTED[name]
                rhs = m.group(4).strip()
                if rhs.startswith("(/"):
                    body = rhs[2:rhs.rindex("/)")]
                    vals = [_literal(t) for t in body.split(",") if t.strip()]
                else:
                    # scalar constant or an expression of constants we skip
                    toks = _NUM.fullmatch(rhs)
                    if not toks:
                        continue
                    vals = [_literal(rhs)]
                idx = _index(m.group(3), shape) if m.group(3) else tuple(slice(0, n) for n in shape)
                target = arrays[name][idx]
                if np.size(target) != len(vals):
                    raise ValueError(f"{name}{m.group(2) or ''}: {len(vals)} values for {np.size(target)} slots")
                arr_vals = np.array([v for v, _ in vals], dtype=np.float64).reshape(np.shape(target), order="F")
                arrays[name][idx] = arr_vals
                filled[name][idx] = True
    out: "OrderedDict[str, np.ndarray]" = OrderedDict()
    for name, (shape, kind) in WANTED.items():
        if not filled[name].all():
            raise ValueError(f"{name}: {int((~filled[name]).sum())} entries not found")
        a = arrays[name]
        out[name] = a.astype(np.int32) if kind == "i" else a
    return out


def main() -> None:
    if len(sys.argv) != 2:
        sys.exit(f"usage: python -m brams_gb300.data.{os.path.basename(__file__)[:-3]} <luflarois/brams source tree>")
    tabs = extract(sys.argv[1])
    dst = os.path.join(HERE, "lw_ref_tables.gblw")
    write_tables(dst, tabs)
    print(f"wrote {dst}: " + ", ".join(f"{k}{tuple(v.shape)}" for k, v in tabs.items()))


if __name__ == "__main__":
    main()
