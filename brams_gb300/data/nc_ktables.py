"""The solver's k-distribution tables from the netCDF table file of AER
RRTMG_LW (``rrtmg_lw.nc``), and that file's layout written from tables.

The reference can take its absorption coefficients from ``rrtmg_lw.nc``
instead of the compiled data module (``src/rrtmg/RRTMG_LW/src/rrtmg_lw_read_nc.f90``,
subroutines ``lw_kgb01 .. lw_kgb16``; dimensions in
``src/rrtmg/RRTMG_LW/modules/rrlw_ncpar.f90:12-44``).  Each subroutine reads, for
its band and g-point set 1, the 16-point ("o") tables of ``rrlw_kgNN``:

* Planck fractions from ``PlanckFraction{Lower,Upper}Atmos``
  (Fortran dims: g-point, key-species mix, band, g-point set);
* key-species coefficients from ``KeySpeciesAbsorptionCoefficients{Lower,Upper}Atmos``
  (key-species mix, temperature difference, pressure, g-point, band, set);
* water-vapour self and foreign continua from ``H20{Self,Foreign}AbsorptionCoefficients``
  (temperature, g-point, band, set);
* minor gases from ``AbsorptionCoefficients{Lower,Upper}Atmos`` at the gas's
  index in the absorber list (key-species mix, temperature, g-point,
  absorber, band, set).

:func:`read_original` takes those hyperslabs (netCDF's C order is the
Fortran order reversed) into the same 16-point tables that ``gen_ktables``
makes, so :func:`build` reduces them to 140 g-points with the reference's
``cmbgb`` weights and writes the solver's ``.gblw`` file.
:func:`write_original` writes 16-point tables in the same layout, so the
reference's own reader can load the tables this project generates.
netCDF classic files (CDF-1/CDF-2) only: scipy reads no HDF5-based netCDF-4.

Usage:  python -m brams_gb300.data.nc_ktables rrtmg_lw.nc <table dir>
        (then gb_rrtmg_lw_ini(cpdair, "<table dir>", ...))
"""
from __future__ import annotations

import os
import sys
from collections import OrderedDict

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from brams_gb300.data.gen_ktables import NG16, _band_tables, reduce_tables  # noqa: E402
from brams_gb300.tables_io import read_tables, write_tables  # noqa: E402

# rrlw_ncpar.f90:12-25 (absorber order of the minor-gas variables) and :31-44
ABSORBERS = ("N2", "CCL4", "CFC11", "CFC12", "CFC22", "H2O", "CO2", "O3", "N2O", "CO", "CH4", "O2")
DIMS = OrderedDict([("GPointSet", 2), ("Band", 16), ("Absorber", 12), ("GPoint", 16), ("PressureLower", 13),
                    ("PressureUpper", 47), ("TemperatureDiff", 5), ("Temperature", 19), ("TempSelf", 10),
                    ("TempForeign", 4), ("KeySpeciesLower", 9), ("KeySpeciesUpper", 5)])
GPOINT_SET = 1  # every lw_kgbNN reads g-point set 1

# variable names and their dimensions in netCDF (C) order
VARS = OrderedDict([
    ("PlanckFractionLowerAtmos", ("GPointSet", "Band", "KeySpeciesLower", "GPoint")),
    ("PlanckFractionUpperAtmos", ("GPointSet", "Band", "KeySpeciesUpper", "GPoint")),
    ("KeySpeciesAbsorptionCoefficientsLowerAtmos",
     ("GPointSet", "Band", "GPoint", "PressureLower", "TemperatureDiff", "KeySpeciesLower")),
    ("KeySpeciesAbsorptionCoefficientsUpperAtmos",
     ("GPointSet", "Band", "GPoint", "PressureUpper", "TemperatureDiff", "KeySpeciesUpper")),
    ("H20SelfAbsorptionCoefficients", ("GPointSet", "Band", "GPoint", "TempSelf")),
    ("H20ForeignAbsorptionCoefficients", ("GPointSet", "Band", "GPoint", "TempForeign")),
    ("AbsorptionCoefficientsLowerAtmos", ("GPointSet", "Band", "Absorber", "GPoint", "Temperature", "KeySpeciesLower")),
    ("AbsorptionCoefficientsUpperAtmos", ("GPointSet", "Band", "Absorber", "GPoint", "Temperature", "KeySpeciesUpper")),
])
# minor-gas tables that are not named ka?_m<gas>: (absorber, lower atmosphere)
_NAMED_MINOR = {"ccl4o": ("CCL4", True), "cfc11adjo": ("CFC11", True), "cfc12o": ("CFC12", True),
                "cfc22adjo": ("CFC22", True)}


def _slot(name: str, shp: tuple):
    """(variable, index in netCDF order after the set and band, axes that
    turn the hyperslab into the reference's index order) of one 16-point
    table: the start/count of the table's nf90_get_var in lw_kgbNN."""
    g = slice(0, NG16)
    if name in ("kao", "kbo"):
        lower = name == "kao"
        nkey = shp[0] if len(shp) == 3 else 1
        var = "KeySpeciesAbsorptionCoefficients" + ("LowerAtmos" if lower else "UpperAtmos")
        npr = DIMS["PressureLower" if lower else "PressureUpper"]
        return var, (g, slice(0, npr), slice(0, 5), slice(0, nkey)), (3, 2, 1, 0)
    if name.startswith("fracref"):
        nkey = shp[0] if shp else 1
        var = "PlanckFraction" + ("LowerAtmos" if name == "fracrefao" else "UpperAtmos")
        return var, (slice(0, nkey), g), (1, 0)
    if name in ("selfrefo", "forrefo"):
        var = "H20SelfAbsorptionCoefficients" if name == "selfrefo" else "H20ForeignAbsorptionCoefficients"
        return var, (g, slice(0, shp[0])), (1, 0)
    if name in _NAMED_MINOR:
        gas, lower = _NAMED_MINOR[name]
    else:  # kao_m<gas> / kbo_m<gas>
        gas, lower = name.split("_m")[1].upper(), name.startswith("kao")
    ab = ABSORBERS.index(gas)
    nkey = shp[0] if len(shp) == 2 else 1
    nt = shp[-1] if shp else 1
    var = "AbsorptionCoefficients" + ("LowerAtmos" if lower else "UpperAtmos")
    return var, (ab, g, slice(0, nt), slice(0, nkey)), (2, 1, 0)


def _to_fortran(a: np.ndarray, axes: tuple, shp: tuple, kind: str) -> np.ndarray:
    """A hyperslab in netCDF order -> the table with the reference's index order."""
    t = np.transpose(a, axes)
    want = (NG16,) + tuple(shp) if kind == "f" else tuple(shp) + (NG16,)
    return np.asarray(t, dtype=np.float64).reshape(want)


def read_original(path: str) -> "OrderedDict[str, np.ndarray]":
    """All 16-point tables of the 16 bands from a netCDF table file, keyed
    'bNN.<name>' like gen_ktables.make_original_tables."""
    from scipy.io import netcdf_file

    out: "OrderedDict[str, np.ndarray]" = OrderedDict()
    with netcdf_file(path, "r", mmap=False) as f:
        for b in range(1, 17):
            for name, (shp, kind) in _band_tables(b).items():
                var, idx, axes = _slot(name, shp)
                if var not in f.variables:
                    raise KeyError(f"{path}: no variable {var} (band {b}, {name})")
                a = np.asarray(f.variables[var][(GPOINT_SET - 1, b - 1) + idx])
                out[f"b{b:02d}.{name}"] = _to_fortran(a, axes, shp, kind)
    return out


def write_original(path: str, orig: dict) -> None:
    """16-point tables (keyed like read_original) into a netCDF classic file
    with the reference reader's variables; entries no band uses stay 0."""
    from scipy.io import netcdf_file

    data = {v: np.zeros(tuple(DIMS[d] for d in dims)) for v, dims in VARS.items()}
    for key, arr in orig.items():
        b, name = int(key[1:3]), key.split(".")[1]
        shp, kind = _band_tables(b)[name]
        var, idx, axes = _slot(name, shp)
        block = data[var][(GPOINT_SET - 1, b - 1) + idx]  # a view
        fshape = tuple(block.shape[i] for i in axes)    # with the singleton axes the table drops
        block[...] = np.transpose(np.asarray(arr, dtype=np.float64).reshape(fshape), np.argsort(axes))
    with netcdf_file(path, "w", version=2) as f:
        for d, n in DIMS.items():
            f.createDimension(d, n)
        for v, dims in VARS.items():
            f.createVariable(v, "d", dims)[:] = data[v]


def build(nc_path: str, out_dir: str) -> str:
    """Reduce the file's tables to the solver's 140 g-points (the reference's
    cmbgb1..16) into out_dir/lw_ktables.gblw, beside a copy of the constant
    tables, so that out_dir is a table directory for gb_rrtmg_lw_ini.  The
    shipped synthetic tables are left as they are."""
    import shutil

    os.makedirs(out_dir, exist_ok=True)
    ref_path = os.path.join(HERE, "lw_ref_tables.gblw")
    red = reduce_tables(read_original(nc_path), read_tables(ref_path))
    dst = os.path.join(out_dir, "lw_ktables.gblw")
    if os.path.abspath(dst) == os.path.abspath(os.path.join(HERE, "lw_ktables.gblw")):
        raise ValueError("out_dir must not be the directory of the shipped tables")
    write_tables(dst, red)
    if os.path.abspath(out_dir) != HERE:
        shutil.copyfile(ref_path, os.path.join(out_dir, "lw_ref_tables.gblw"))
    return dst


if __name__ == "__main__":
    if len(sys.argv) != 3:
        sys.exit(__doc__)
    print(build(sys.argv[1], sys.argv[2]))
