"""Host side of the GB300 JoinT (include/joint_gpu.h, no GPU needed): FITS map
reading in RING, NESTED and multi-element-row layouts (src/healpix_extra.c:166-224),
the frequency table and .ini (src/io_jt.c), the instrument table
(src/main_jt.c:28-72), against the golden vectors of the reference's JoinT."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from fits_io import read_map as py_read_map
from fits_io import write_map
from oracle import orc


@pytest.fixture(scope="session")
def jt():
    from crime_gb300 import build
    build.build()
    from crime_gb300 import joint
    return joint


def test_read_map_layouts(jt, tmp_path):
    g = dict(np.load(os.path.join(GOLDEN, "joint_merge.npz")))
    nside = int(g["cfg_nside_in"])
    t, q = g["in_synchrotron"][0], g["in_synchrotron_q"][0]
    write_map(tmp_path / "ring.fits", [t, q], nside)
    m, ns = jt.read_map(str(tmp_path / "ring.fits"), 0)
    assert ns == nside and np.array_equal(m, t)
    m, _ = jt.read_map(str(tmp_path / "ring.fits"), 1)
    assert np.array_equal(m, q)
    nest = np.array([t[orc.nest2ring(nside, p)] for p in range(t.size)], np.float32)
    write_map(tmp_path / "nest.fits", [nest], nside, ordering="NESTED", repeat=64)
    m, _ = jt.read_map(str(tmp_path / "nest.fits"), 0)
    assert np.array_equal(m, t)  # NESTED files come back in RING order
    with pytest.raises(Exception):
        jt.read_map(str(tmp_path / "ring.fits"), 2)
    with pytest.raises(Exception):
        jt.read_map(str(tmp_path / "missing.fits"), 0)


def test_write_maps_round_trip(jt, tmp_path):
    rng = np.random.default_rng(1)
    maps = rng.standard_normal((2, 12 * 16)).astype(np.float32)
    # write_maps needs no device: the host entry point directly
    from crime_gb300.gethi import _check
    _check(jt.lib().joint_host_write_maps(os.fsencode(str(tmp_path / "o")), 4, 2, maps.ctypes.data))
    for i in range(2):
        h, d = py_read_map(str(tmp_path / ("o_%03d.fits" % (i + 1))))
        assert h["ORDERING"] == "RING" and int(h["NSIDE"]) == 4 and h["TTYPE1"] == "T"
        assert np.array_equal(d, maps[i])
        m, ns = jt.read_map(str(tmp_path / ("o_%03d.fits" % (i + 1))))
        assert ns == 4 and np.array_equal(m, maps[i])


@pytest.mark.parametrize("name", ["joint_merge", "joint_beam", "joint_t3"])
def test_instrument_table_matches_reference(jt, tmp_path, name):
    import ctypes as C
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    nu0, nuf = np.ascontiguousarray(g["nu0"]), np.ascontiguousarray(g["nuf"])
    p = jt.JointParams(nside=int(g["cfg_nside"]), n_nu=nu0.size, nu0=nu0.ctypes.data, nuf=nuf.ctypes.data,
                       dish_diameter=float(g["cfg_dish"]), n_dish=int(g["cfg_n_dish"]), tsys=float(g["cfg_tsys"]),
                       time_tot=float(g["cfg_time_tot"]))
    mask = g.get("mask")
    fsky = 1.0 if mask is None else np.count_nonzero(mask) / mask.size
    from crime_gb300.gethi import _check
    _check(jt.lib().joint_host_write_instrument(os.fsencode(str(tmp_path / "o")), C.byref(p), fsky))
    rows = np.loadtxt(str(tmp_path / "o_instrument.dat"), ndmin=2)
    np.testing.assert_array_equal(rows, g["instrument"])  # the same %lE text


def test_nutable_and_ini(jt, tmp_path, capfd):
    nt = tmp_path / "nu.dat"
    nt.write_text("1 700.0 710.5 1.0 1.1\n2 710.5 721.0 0.9 1.0\n")
    nu0, nuf = jt.read_nutable(str(nt))
    assert list(nu0) == [700.0, 710.5] and list(nuf) == [710.5, 721.0]
    import ctypes as C
    ini = tmp_path / "p.ini"
    ini.write_text("# c\nprefix_cosmo= a\nnside= 8\nseed= 5\ndish_diameter= 30.\nn_dishes= 4\n"
                   "t_system= 1000.\ntime_total= 10.\nbogus= 1\nrng= mt_validation\n")
    L = jt.lib()

    class Ini(C.Structure):
        _fields_ = [(n, C.c_char * 256) for n in (
            "prefix_cosmo", "prefix_synchrotron", "prefix_galactic_freefree", "prefix_extragalactic_freefree",
            "prefix_point_sources", "prefix_custom", "prefix_out", "fname_nutable", "fname_mask")] + [
            ("seed_signed", C.c_int), ("nside", C.c_int), ("do_polarization", C.c_int),
            ("polarization_leakage", C.c_double), ("dish_diameter", C.c_double), ("tsys", C.c_double),
            ("time_tot", C.c_double), ("n_dish", C.c_int), ("rng", C.c_int), ("omp_threads_for_noise", C.c_int)]
    L.joint_host_read_ini.argtypes = [C.c_char_p, C.POINTER(Ini)]
    o = Ini()
    assert L.joint_host_read_ini(os.fsencode(str(ini)), C.byref(o)) == 0
    assert o.prefix_cosmo == b"a" and o.prefix_custom == b"custom" and o.prefix_out == b"default"
    assert (o.nside, o.seed_signed, o.dish_diameter, o.n_dish, o.tsys, o.time_tot, o.rng) == \
        (8, 5, 30.0, 4, 1000.0, 10.0, 1)
    assert "unknown param bogus=" in capfd.readouterr().err  # warned, as src/io_jt.c:165-168
    ini.write_text("nside= 8\ndo_polarization= 1\npolarization_leakage= 2.0\n")
    assert L.joint_host_read_ini(os.fsencode(str(ini)), C.byref(o)) != 0  # src/io_jt.c:172-177
    ini.write_text("nside=8\n")
    assert L.joint_host_read_ini(os.fsencode(str(ini)), C.byref(o)) != 0  # one token: error_read_line
