"""The oracle against golden vectors written by the reference's own GetHI
sources (compiled with project shims; tests/golden/make_golden.py).  Every
stage must be bit-identical: both sides run the same arithmetic in the same
order, so any difference is a restatement bug."""
import numpy as np
import pytest

from conftest import load_case, oracle_for_case

CASES = ["case_irr32", "case_reg24"]


def real_cells(a, n):
    return a.reshape(n, n, 2 * (n // 2 + 1))[:, :, :n]


@pytest.fixture(scope="module", params=CASES)
def case(request, oracle_lib):
    oracle_lib.set_threads(1)
    c = load_case(request.param)
    return c, oracle_for_case(c)


def test_derived_parameters(case):
    g, o = case
    d = o.d
    for key, val in [("fgrowth_0", d.fgrowth_0), ("hubble_0", d.hubble_0), ("z_min", d.z_min),
                     ("z_max", d.z_max), ("r_min", d.r_min), ("r_max", d.r_max), ("l_box", d.l_box),
                     ("glob_idr", d.glob_idr), ("r2_smooth", d.r2_smooth), ("idlogk", d.idlogk)]:
        assert g["p_" + key] == val, key
    np.testing.assert_array_equal(o.pk, g["pk"])
    np.testing.assert_array_equal(o.logk, g["logk"])
    if "tables" in g:
        np.testing.assert_array_equal(o.tables(), g["tables"])


def test_modes_mt_bitexact(case):
    g, o = case
    dk, vk = o.modes_mt(nthreads=1)
    np.testing.assert_array_equal(dk.view(np.float32).reshape(-1), g["dens_k"])
    np.testing.assert_array_equal(vk.view(np.float32).reshape(-1), g["vpot_k"])


def test_modes_mt_thread_partition(oracle_lib):
    g = load_case("case_irr32_t3")
    o = oracle_for_case(g)
    dk, vk = o.modes_mt(nthreads=int(g["cfg_n_threads"]))
    np.testing.assert_array_equal(dk.view(np.float32).reshape(-1), g["dens_k"])
    np.testing.assert_array_equal(vk.view(np.float32).reshape(-1), g["vpot_k"])
    # and it really differs from the single-thread draw
    d1, _ = o.modes_mt(nthreads=1)
    assert not np.array_equal(d1, dk)


def test_fields_bitexact(case):
    g, o = case
    n = o.n
    dk = g["dens_k"].view(np.complex64).reshape(o.spec_shape())
    vk = g["vpot_k"].view(np.complex64).reshape(o.spec_shape())
    dens = o.normalize(o.c2r(dk))
    vpot = o.normalize(o.c2r(vk))
    np.testing.assert_array_equal(real_cells(dens, n), real_cells(g["dens_real"], n))
    np.testing.assert_array_equal(real_cells(vpot, n), real_cells(g["vpot_real"], n))
    rv = o.radial_velocity_fd(vpot)
    np.testing.assert_array_equal(real_cells(rv, n), real_cells(g["rvel"], n))
    _, s2 = o.sigma(dens)
    assert s2 == g["p_sigma2_gauss"]
    mass, dz = o.get_hi(dens, rv, s2)
    np.testing.assert_array_equal(real_cells(mass, n), real_cells(g["mass"], n))
    np.testing.assert_array_equal(real_cells(dz, n), real_cells(g["dz"], n))


def test_maps_bitexact(case):
    g, o = case
    maps = o.mk_T_maps(g["mass"], g["dz"])
    np.testing.assert_array_equal(maps.reshape(-1), g["maps"])
    assert np.count_nonzero(maps) > 0.5 * maps.size


# ---- point sources (src/psources.c, grid_tools.c:24-101, pixelize.c:58-148)
@pytest.fixture(scope="module")
def ps_case(oracle_lib):
    oracle_lib.set_threads(1)
    g = load_case("case_ps32")
    return g, oracle_for_case(g)


def test_psources_tables_bitexact(ps_case):
    g, o = ps_case
    nz, mp, gdz = o.setup_psources()
    assert gdz == g["p_glob_dz"]
    np.testing.assert_array_equal(nz, g["ps_nz"])
    np.testing.assert_array_equal(mp, g["ps_maxpdf"])


@pytest.mark.parametrize("nthreads,name", [(1, "case_ps32"), (3, "case_ps32_t3")])
def test_point_source_counts_bitexact(ps_case, nthreads, name):
    _, o = ps_case
    g = load_case(name)  # the 3-thread run draws other modes, so its own density field
    ns = o.point_sources(g["dens_real"], float(g["p_sigma2_gauss"]), nthreads=nthreads)
    ref = g["nsources"]
    np.testing.assert_array_equal(ns.reshape(-1), ref)
    assert ref.sum() > 1000 and ref.max() >= 2


def test_psources_maps_bitexact(ps_case):
    g, o = ps_case
    maps = o.psources_maps(g["nsources"], g["dz"], nthreads=1)
    np.testing.assert_array_equal(maps.reshape(-1), g["maps_ps"])
    assert maps.sum() > 0
    # the catalogue form of the same sum (FP64) agrees to rounding
    n = o.n
    ns = g["nsources"].reshape(n, n, 2 * (n // 2 + 1))[:, :, :n]
    assert (ns > 0).sum() > 100
