"""The JoinT oracle (oracle/orc_joint.c, oracle/orc.py `joint`) against golden
vectors of the reference's own JoinT (src/main_jt.c and helpers, compiled with
the test shims; tests/golden/make_golden_joint.py), and the HEALPix helpers
against their defining properties.  CPU only."""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import orc

# the order in which src/main_jt.c:98-200 adds the components
ORDER = ["cosmo", "extragalactic_freefree", "galactic_freefree", "point_sources", "synchrotron", "custom"]


def joint_inputs(g):
    comps = []
    for c in ORDER:
        if "in_" + c not in g:
            continue
        if c == "synchrotron" and float(g["cfg_leakage"]) > 0:
            comps.append((g["in_synchrotron_q"], float(g["cfg_leakage"])))
        comps.append((g["in_" + c], None))
    mask = g["mask"] if "mask" in g else None
    return comps, mask


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.mark.parametrize("name", ["joint_merge", "joint_beam", "joint_t3"])
def test_oracle_joint_matches_reference(name):
    g = load(name)
    comps, mask = joint_inputs(g)
    out = orc.joint(comps, int(g["cfg_nside_in"]), int(g["cfg_nside"]), g["nu0"], g["nuf"],
                    dish=float(g["cfg_dish"]), n_dish=int(g["cfg_n_dish"]), tsys=float(g["cfg_tsys"]),
                    time_tot=float(g["cfg_time_tot"]), seed=int(g["cfg_seed"]), mask=mask,
                    nthreads=int(g["cfg_n_threads"]))
    np.testing.assert_array_equal(out, g["maps"])  # bit-exact
    fsky = 1.0 if mask is None else np.count_nonzero(mask) / mask.size
    inst = orc.joint_instrument(int(g["cfg_nside"]), g["nu0"], g["nuf"], float(g["cfg_dish"]),
                                int(g["cfg_n_dish"]), float(g["cfg_tsys"]), float(g["cfg_time_tot"]), fsky)
    np.testing.assert_allclose(inst, g["instrument"], rtol=1e-6)  # printed with %lE


def test_nest_ring_round_trip_and_nesting():
    """NESTED <-> RING is a bijection and the four NESTED children of a pixel lie
    inside it (their centres within ~0.55 pixel sizes of the parent's)."""
    for nside in (1, 2, 4, 8, 16):
        npix = 12 * nside * nside
        r = np.array([orc.nest2ring(nside, p) for p in range(npix)])
        assert sorted(r) == list(range(npix))
        assert all(orc.ring2nest(nside, int(r[p])) == p for p in range(npix))
    for nside in (4, 8):
        npix = 12 * nside * nside
        worst = 0.0
        for p in range(npix):
            t, f = orc.pix2ang_ring(nside, orc.nest2ring(nside, p))
            v = np.array([math.sin(t) * math.cos(f), math.sin(t) * math.sin(f), math.cos(t)])
            for c in range(4):
                t2, f2 = orc.pix2ang_ring(2 * nside, orc.nest2ring(2 * nside, 4 * p + c))
                w = np.array([math.sin(t2) * math.cos(f2), math.sin(t2) * math.sin(f2), math.cos(t2)])
                worst = max(worst, math.acos(min(1.0, float(v @ w))))
        assert worst < 0.55 * math.sqrt(4 * math.pi / npix)


def test_ring_geometry_matches_pixel_centres():
    nside = 8
    for r in range(4 * nside - 1):
        first, nph, z, sth, phi0 = orc.ring_info(nside, r)
        for j in (0, nph - 1):
            t, f = orc.pix2ang_ring(nside, first + j)
            assert abs(math.cos(t) - z) < 1e-12 and abs(math.sin(t) - sth) < 1e-12
            assert abs(f - (phi0 + 2 * math.pi * j / nph)) < 1e-12


def test_sht_known_answers():
    """a_00 of a constant map is c sqrt(4 pi); Y_10 and Y_11 synthesise their
    closed forms; lambda_lm matches scipy's spherical harmonics."""
    nside = 8
    lmax = 3 * nside - 1
    npix = 12 * nside * nside
    a = orc.map2alm(nside, lmax, np.full(npix, 2.0))
    assert abs(a[0].real - 2 * math.sqrt(4 * math.pi)) < 1e-12
    ang = [orc.pix2ang_ring(nside, p) for p in range(npix)]
    alm = np.zeros(orc.nalms(lmax), np.complex128)
    alm[1] = 1.0  # (l, m) = (1, 0)
    m = orc.alm2map(nside, lmax, alm)
    np.testing.assert_allclose(m, [math.sqrt(3 / (4 * math.pi)) * math.cos(t) for t, _ in ang], atol=1e-14)
    alm[:] = 0
    alm[lmax + 1] = 1.0  # (1, 1): index l + m lmax - m(m-1)/2
    m = orc.alm2map(nside, lmax, alm)
    np.testing.assert_allclose(m, [-2 * math.sqrt(3 / (8 * math.pi)) * math.sin(t) * math.cos(f) for t, f in ang],
                               atol=1e-14)
    sp = pytest.importorskip("scipy.special")
    if not hasattr(sp, "sph_harm_y"):
        pytest.skip("scipy without sph_harm_y")
    lm = 200
    for mm, th in [(0, 0.3), (40, 0.7), (150, 1.2), (199, 2.9)]:
        out = np.zeros(lm - mm + 1)
        orc.lib().orc_lambda_m(lm, mm, math.cos(th), math.sin(th), out)
        ref = np.real(sp.sph_harm_y(np.arange(mm, lm + 1), mm, th, 0.0))
        assert np.abs(out - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1e-300)


def test_udgrade_degrade_is_nested_mean():
    rng = np.random.default_rng(3)
    m = rng.standard_normal(12 * 16 * 16).astype(np.float32)
    d = orc.udgrade(m, 16, 4)
    for p in range(12 * 16):
        pn = orc.ring2nest(4, p)
        kids = [m[orc.nest2ring(16, 16 * pn + j)] for j in range(16)]
        assert d[p] == np.float32(np.sum(np.array(kids, np.float64)) / 16)
    u = orc.udgrade(d, 4, 16)
    assert np.array_equal(orc.udgrade(u, 16, 4), d)
