"""Extract BRAMS's zonal ozone climatology for the radiation driver.

``InitGetoz_rrtm`` (``src/brams/radiate/rtm_driver.f90:2062-2636``) fills
``ozone(18, 37, 4)`` (18 sigma levels, 37 latitudes from 90 N to 90 S every
5 degrees, 4 seasons) and ``ozsig(18)`` with Fortran array constructors;
``getoz_rrtm`` (``:2638-2823``) interpolates them.  The values must be the
driver's, so this script reads the constructors out of the Fortran source
and writes ``brams_ozone.gblw`` (format: ``brams_gb300/tables_io.py``).  All
literals carry the ``_r8`` kind suffix (double precision).

Usage:  python brams_gb300/data/extract_ozone.py [REFERENCE_ROOT]
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

NLEV, NLAT, NSEA = 18, 37, 4


def _numbers(text: str) -> list:
    return [float(t.replace("_r8", "")) for t in re.findall(r"[-+]?\d*\.\d+(?:e[-+]?\d+)?_r8", text)]


def extract(ref_root: str) -> "OrderedDict[str, np.ndarray]":
    path = os.path.join(ref_root, "src", "brams", "radiate", "rtm_driver.f90")
    src = open(path).read()
    i0 = src.index("subroutine InitGetoz_rrtm")
    i1 = src.index("END SUBROUTINE InitGetoz_rrtm")
    body = re.sub(r"&\s*\n\s*", " ", src[i0:i1])  # join continuation lines
    oz = np.full((NLEV, NLAT, NSEA), np.nan)
    # ozone(1:18, a:b, s) = RESHAPE( (/ ... /), (/18,n/))  or  ozone(1:18, a, s) = (/ ... /)
    pat = re.compile(r"ozone\(1:18,\s*(\d+)(?::(\d+))?,\s*(\d)\)\s*=\s*(?:RESHAPE\(\s*)?\(/(.*?)/\)")
    for m in pat.finditer(body):
        a, b, s = int(m.group(1)), int(m.group(2) or m.group(1)), int(m.group(3))
        vals = _numbers(m.group(4))
        n = b - a + 1
        if len(vals) != NLEV * n:
            raise ValueError(f"ozone(1:18,{a}:{b},{s}): {len(vals)} values")
        oz[:, a - 1:b, s - 1] = np.array(vals).reshape(n, NLEV).T  # Fortran order: level fastest
    if np.isnan(oz).any():
        raise ValueError(f"{int(np.isnan(oz).sum())} ozone entries not found")
    m = re.search(r"ozsig\(:\)\s*=\s*\(/(.*?)/\)", body)
    sig = np.array(_numbers(m.group(1)))
    if sig.size != NLEV:
        raise ValueError(f"ozsig: {sig.size} values")
    return OrderedDict([("ozone", oz), ("ozsig", sig)])


def main() -> None:
    if len(sys.argv) != 2:
        sys.exit(f"usage: python -m brams_gb300.data.{os.path.basename(__file__)[:-3]} <luflarois/brams source tree>")
    tabs = extract(sys.argv[1])
    dst = os.path.join(HERE, "brams_ozone.gblw")
    write_tables(dst, tabs)
    print(f"wrote {dst}: " + ", ".join(f"{k}{tuple(v.shape)}" for k, v in tabs.items()))


if __name__ == "__main__":
    main()
