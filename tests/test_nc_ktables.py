"""The netCDF table reader (brams_gb300/data/nc_ktables.py) against the
reference reader's hyperslabs (rrtmg_lw_read_nc.f90, lw_kgb01..16): element
placement checked on a file whose values encode their own netCDF index, a
write/read round trip of the 16-point tables, and the reduced tables built
from such a file equal to the shipped ones."""
import os

import numpy as np
import pytest

pytest.importorskip("scipy")

from brams_gb300.data import gen_ktables as G  # noqa: E402
from brams_gb300.data import nc_ktables as N  # noqa: E402
from brams_gb300.tables_io import read_tables  # noqa: E402

DATA = os.path.dirname(os.path.abspath(G.__file__))


def _index_file(path):
    """Every variable holds 1 + its C-order linear index (so each value names its place)."""
    from scipy.io import netcdf_file

    with netcdf_file(path, "w", version=2) as f:
        for d, n in N.DIMS.items():
            f.createDimension(d, n)
        for v, dims in N.VARS.items():
            shape = tuple(N.DIMS[d] for d in dims)
            f.createVariable(v, "d", dims)[:] = 1.0 + np.arange(np.prod(shape), dtype=np.float64).reshape(shape)
    return {v: tuple(N.DIMS[d] for d in dims) for v, dims in N.VARS.items()}


def _at(shapes, var, *idx):
    return 1.0 + np.ravel_multi_index(idx, shapes[var])


def test_hyperslabs_follow_the_reference_reader(tmp_path):
    p = str(tmp_path / "idx.nc")
    shapes = _index_file(p)
    t = N.read_original(p)
    s = 0  # g-point set 1
    # band 3 kao(key, Tdiff, p, g) <- KeySpecies...LowerAtmos(key, Tdiff, p, g, band 3, set 1) in Fortran order
    assert t["b03.kao"][1, 2, 3, 4] == _at(shapes, "KeySpeciesAbsorptionCoefficientsLowerAtmos", s, 2, 4, 3, 2, 1)
    # band 1 kao(Tdiff, p, g): key-species index 1
    assert t["b01.kao"][2, 5, 7] == _at(shapes, "KeySpeciesAbsorptionCoefficientsLowerAtmos", s, 0, 7, 5, 2, 0)
    # band 4 kbo(key, Tdiff, p 13:59, g)
    assert t["b04.kbo"][4, 0, 46, 15] == _at(shapes, "KeySpeciesAbsorptionCoefficientsUpperAtmos", s, 3, 15, 46, 0, 4)
    # fracrefao(g, key) of band 9; fracrefbo(g) of band 7 (key index 1)
    assert t["b09.fracrefao"][6, 8] == _at(shapes, "PlanckFractionLowerAtmos", s, 8, 8, 6)
    assert t["b07.fracrefbo"][3] == _at(shapes, "PlanckFractionUpperAtmos", s, 6, 0, 3)
    # selfrefo(T, g), forrefo(T, g) of band 12
    assert t["b12.selfrefo"][9, 2] == _at(shapes, "H20SelfAbsorptionCoefficients", s, 11, 2, 9)
    assert t["b12.forrefo"][3, 15] == _at(shapes, "H20ForeignAbsorptionCoefficients", s, 11, 15, 3)
    # minor gases at their absorber index: kao_mco2(key, T, g) band 13, kbo_mo3(T, g) band 13, ccl4o(g) band 5
    co2, o3, ccl4 = N.ABSORBERS.index("CO2"), N.ABSORBERS.index("O3"), N.ABSORBERS.index("CCL4")
    assert t["b13.kao_mco2"][7, 18, 1] == _at(shapes, "AbsorptionCoefficientsLowerAtmos", s, 12, co2, 1, 18, 7)
    assert t["b13.kbo_mo3"][5, 0] == _at(shapes, "AbsorptionCoefficientsUpperAtmos", s, 12, o3, 0, 5, 0)
    assert t["b05.ccl4o"][11] == _at(shapes, "AbsorptionCoefficientsLowerAtmos", s, 4, ccl4, 11, 0, 0)


def test_round_trip_and_reduced_tables_equal_the_shipped_ones(tmp_path):
    ref = read_tables(os.path.join(DATA, "lw_ref_tables.gblw"))
    orig = G.make_original_tables(ref)
    p = str(tmp_path / "synthetic_rrtmg_lw.nc")
    N.write_original(p, orig)
    back = N.read_original(p)
    assert list(back) == list(orig)
    for k in orig:
        assert back[k].shape == np.asarray(orig[k]).shape, k
        assert np.array_equal(back[k], orig[k]), k
    dst = N.build(p, str(tmp_path / "tables"))
    assert os.path.exists(str(tmp_path / "tables" / "lw_ref_tables.gblw"))
    built, shipped = read_tables(dst), read_tables(os.path.join(DATA, "lw_ktables.gblw"))
    assert list(built) == list(shipped)
    for k in shipped:
        assert np.array_equal(built[k], shipped[k]), k
