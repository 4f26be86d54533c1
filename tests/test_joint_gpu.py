"""GPU parity of the GB300 JoinT (include/joint_gpu.h) with the oracle and the
reference's JoinT golden vectors (tests/golden/joint_*.npz):

* merge (FP32 sums in the reference's component order) + he_udgrade + the
  reference's MT19937 noise + mask: bit-exact;
* the beam (map2alm -> exp(-l(l+1) sigma^2/2) -> alm2map, lmax = 3 nside - 1)
  in FP32 on the GPU against the FP64 transform: relative L2 <= 2e-6 of the map,
  max error <= 1e-5 of the map's largest value;
* map2alm / alm2map separately against the oracle;
* the Philox noise: variance s2/2 per channel (the law of src/main_jt.c:304-311);
* the device hand-off from a GetHI context and the JoinT_gpu command line."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, REPO
from fits_io import read_map, write_map
from oracle import orc
from test_joint_oracle import ORDER, joint_inputs

pytestmark = pytest.mark.gpu
BEAM_L2 = 2e-6
BEAM_MAX = 1e-5


@pytest.fixture(scope="module")
def jt():
    from crime_gb300 import build
    build.build()
    from crime_gb300 import joint
    return joint


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def joint_for(jt, g, rng="mt_validation"):
    mask = g.get("mask")
    return jt.JoinT(int(g["cfg_nside"]), g["nu0"], g["nuf"], seed=int(g["cfg_seed"]), dish_diameter=float(g["cfg_dish"]),
                    n_dish=int(g["cfg_n_dish"]), tsys=float(g["cfg_tsys"]), time_tot=float(g["cfg_time_tot"]),
                    mask=mask, rng=rng, omp_threads_for_noise=int(g["cfg_n_threads"]))


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("name", ["joint_merge", "joint_beam", "joint_t3"])
def test_joint_matches_reference_golden(jt, name):
    g = load(name)
    j = joint_for(jt, g)
    comps, _ = joint_inputs(g)
    for maps, fac in comps:
        j.add_maps(maps, int(g["cfg_nside_in"]), 1.0 if fac is None else fac)
    out = j.run()
    if float(g["cfg_dish"]) <= 0:
        np.testing.assert_array_equal(out, g["maps"])
    else:
        ref = g["maps"]
        assert rel_l2(out, ref) <= BEAM_L2
        assert np.abs(out - ref).max() <= BEAM_MAX * np.abs(ref).max()
        if "mask" in g:
            assert np.all(out[:, g["mask"] == 0] == 0)
    # a second run of the same combination gives the same maps
    np.testing.assert_array_equal(j.run(), out)
    j.close()


@pytest.mark.parametrize("precision", ["auto", "fp32"])
@pytest.mark.parametrize("nside,dish", [(16, 1.0), (32, 4.0), (64, 8.0)])
def test_beam_matches_oracle(jt, nside, dish, precision):
    """the beam with the Legendre sums on the tensor cores (3xTF32, 'auto' at these
    sizes) and on the FP32 CUDA cores"""
    rng = np.random.default_rng(nside)
    nu0 = np.array([600.0, 800.0, 1000.0])
    nuf = nu0 + 10.0
    maps = (rng.standard_normal((3, 12 * nside * nside)) * 3 + 1).astype(np.float32)
    j = jt.JoinT(nside, nu0, nuf, dish_diameter=dish, sht_precision=precision)
    j.add_maps(maps, nside)
    out = j.run()
    assert j.uses_tensor_cores == (precision == "auto")
    ref = orc.apply_beam(maps, nside, orc.joint_fwhm(nu0, nuf, dish))
    assert rel_l2(out, ref) <= BEAM_L2
    assert np.abs(out - ref).max() <= BEAM_MAX * np.abs(ref).max()
    assert rel_l2(out, maps) > 0.05  # the beam did smooth


@pytest.mark.parametrize("nside", [4, 16, 32, 128])
def test_map2alm_alm2map_match_oracle(jt, nside):
    """against the oracle's FP64 transform; Nside 128 takes the compile-time ring-FFT
    plans (512-point equatorial rings, 1024-point Bluestein convolutions)"""
    rng = np.random.default_rng(7 + nside)
    lmax = 3 * nside - 1
    maps = rng.standard_normal((2, 12 * nside * nside)).astype(np.float32)
    j = jt.JoinT(nside, [700.0], [710.0])
    alm = j.map2alm(maps)
    for i in range(2):
        ref = orc.map2alm(nside, lmax, maps[i].astype(np.float64))
        assert np.linalg.norm(alm[i] - ref) <= 2e-6 * np.linalg.norm(ref)
    syn = j.alm2map(alm)
    for i in range(2):
        ref = orc.alm2map(nside, lmax, alm[i].astype(np.complex128))
        assert np.linalg.norm(syn[i] - ref) <= 2e-6 * np.linalg.norm(ref)
    # known answers: constant map -> a_00 = c sqrt(4 pi); Y_10 -> sqrt(3/4pi) cos(theta)
    # (FP32 quadrature over 12 nside^2 pixels: 5e-6 relative)
    a = j.map2alm(np.full(12 * nside * nside, 2.0, np.float32))
    assert abs(a[0, 0].real - 2 * np.sqrt(4 * np.pi)) < 5e-6 * 2 * np.sqrt(4 * np.pi)
    y = np.zeros(orc.nalms(lmax), np.complex64)
    y[1] = 1.0
    m = j.alm2map(y)[0]
    th = np.array([orc.pix2ang_ring(nside, p)[0] for p in range(12 * nside * nside)])
    np.testing.assert_allclose(m, np.sqrt(3 / (4 * np.pi)) * np.cos(th), atol=1e-6)


def test_udgrade_both_ways_bit_exact(jt):
    rng = np.random.default_rng(2)
    for nin, nout in ((32, 8), (8, 32), (16, 16)):
        maps = rng.standard_normal((2, 12 * nin * nin)).astype(np.float32)
        j = jt.JoinT(nout, [700.0, 710.0], [710.0, 720.0])
        j.add_maps(maps, nin)
        out = j.run()
        for i in range(2):
            np.testing.assert_array_equal(out[i], orc.udgrade(maps[i], nin, nout))


def test_philox_noise_statistics(jt):
    nside = 128
    nu0 = np.array([700.0, 800.0])
    nuf = nu0 + np.array([1.0, 4.0])
    kw = dict(tsys=20000.0, time_tot=100.0, n_dish=10, seed=42)
    j = jt.JoinT(nside, nu0, nuf, **kw)
    out = j.run()  # no component: zero maps plus noise
    npix = 12 * nside * nside
    for i in range(2):
        s2 = npix * kw["tsys"] ** 2 / (orc.PREFAC_TNU * (nuf[i] - nu0[i]) * kw["time_tot"] * kw["n_dish"])
        var = float(np.var(out[i].astype(np.float64)))
        assert abs(var / (s2 / 2) - 1) < 0.02, (var, s2 / 2)
        assert abs(float(np.mean(out[i]))) < 5 * np.sqrt(s2 / 2 / npix)
    np.testing.assert_array_equal(jt.JoinT(nside, nu0, nuf, **kw).run(), out)  # counter-based: reproducible
    assert not np.array_equal(jt.JoinT(nside, nu0, nuf, **dict(kw, seed=43)).run(), out)


def test_run_fuses_noise_and_mask_exactly(jt):
    """run() applies the Philox noise and the mask in one pass; the maps equal those of
    the stages called one by one (merge, add_noise, apply_mask), bit for bit"""
    nside = 64
    rng = np.random.default_rng(7)
    nu0 = np.array([700.0, 800.0, 900.0])
    nuf = nu0 + 2.0
    npix = 12 * nside * nside
    mask = (rng.random(npix) > 0.3).astype(np.int32)
    maps = rng.standard_normal((3, npix)).astype(np.float32)
    kw = dict(tsys=20000.0, time_tot=100.0, n_dish=10, seed=9, mask=mask)
    j = jt.JoinT(nside, nu0, nuf, **kw)
    j.add_maps(maps, nside)
    fused = j.run()
    j2 = jt.JoinT(nside, nu0, nuf, **kw)
    j2.add_maps(maps, nside)
    j2.merge_maps()
    j2.add_noise()
    j2.apply_mask()
    np.testing.assert_array_equal(j2.maps(), fused)
    assert np.all(fused[:, mask == 0] == 0) and np.all(fused[:, mask == 1] != maps[:, mask == 1])


def test_beam_independent_of_the_channel_batching(jt):
    """the beam of 7 channels in batches of 3 (odd column counts: single-channel E/O
    stores, blocks with channels beyond the batch) equals the one-batch beam bit for
    bit on the FP32 path, where every output column depends on its own channel only"""
    nside = 16
    rng = np.random.default_rng(21)
    nu0 = np.linspace(600.0, 900.0, 7)
    maps = rng.standard_normal((7, 12 * nside * nside)).astype(np.float32)
    outs = []
    for chunk in (0, 3):
        j = jt.JoinT(nside, nu0, nu0 + 4.0, dish_diameter=2.0, sht_precision="fp32", sht_chunk=chunk)
        j.add_maps(maps, nside)
        outs.append(j.run())
        j.close()
    np.testing.assert_array_equal(outs[0], outs[1])
    assert rel_l2(outs[0], maps) > 0.05


def test_run_with_device_components_equals_the_stages(jt):
    """run() with device components (summed in one pass at the merge) equals merge,
    apply_beam, add_noise and apply_mask called one by one, bit for bit, also on a
    repeated run; the same components from the host give the same maps"""
    torch = pytest.importorskip("torch")
    nside = 32
    rng = np.random.default_rng(11)
    nu0 = np.array([600.0, 750.0, 900.0])
    nuf = nu0 + 3.0
    npix = 12 * nside * nside
    comps = [(rng.standard_normal((3, npix)) * s).astype(np.float32) for s in (1.0, 100.0, 0.01)]
    dev = [torch.from_numpy(m).cuda() for m in comps]
    kw = dict(dish_diameter=4.0, tsys=20000.0, time_tot=100.0, n_dish=10, seed=3,
              mask=(rng.random(npix) > 0.2).astype(np.int32))
    j = jt.JoinT(nside, nu0, nuf, **kw)
    for d in dev:
        j.add_maps_device(d.data_ptr(), nside)
    fused = j.run()
    j2 = jt.JoinT(nside, nu0, nuf, **kw)
    for d in dev:
        j2.add_maps_device(d.data_ptr(), nside)
    j2.merge_maps()
    j2.apply_beam()
    j2.add_noise()
    j2.apply_mask()
    np.testing.assert_array_equal(j2.maps(), fused)
    np.testing.assert_array_equal(j.run(), fused)  # a repeated run sums the components again
    j3 = jt.JoinT(nside, nu0, nuf, **kw)
    for m in comps:
        j3.add_maps(m, nside)
    np.testing.assert_array_equal(j3.run(), fused)


def test_gethi_maps_handed_over_on_the_device(jt):
    import crime_gb300 as cg
    p = cg.make_params(n_grid=32, n_side=16, pk_filename="EH", frequencies_filename="", nu_min=700.0, nu_max=800.0,
                       n_nu=4, seed=11)
    gh = cg.GetHI(p)
    host = np.empty((4, 12 * 16 * 16), np.float32)
    gh.run(host)
    kw = dict(dish_diameter=3.0, tsys=500.0, time_tot=10.0, n_dish=4, seed=3)
    nu0 = np.linspace(700.0, 775.0, 4)
    a = jt.JoinT(8, nu0, nu0 + 25.0, **kw)
    a.add_gethi(gh)
    out_dev = a.run()
    b = jt.JoinT(8, nu0, nu0 + 25.0, **kw)
    b.add_maps(host, 16)
    np.testing.assert_array_equal(out_dev, b.run())


def test_stage_errors(jt):
    import crime_gb300 as cg
    j = jt.JoinT(8, [700.0], [710.0])
    j.add_maps(np.zeros(12 * 64, np.float32), 8)
    with pytest.raises(cg.GetHIError):
        j.add_maps(np.zeros(12 * 16 * 16, np.float32), 16)  # nside differs from the first component
    with pytest.raises(cg.GetHIError):
        jt.JoinT(8, [700.0], [710.0]).apply_beam()  # before the merge
    j.merge_maps()
    with pytest.raises(cg.GetHIError):
        j.apply_beam()  # dish_diameter <= 0
    with pytest.raises(cg.GetHIError):
        jt.JoinT(2048, [700.0], [710.0], dish_diameter=10.0).run()  # SHT limited to nside <= 1024


def test_cli_matches_reference_golden(jt, tmp_path):
    g = load("joint_merge")
    n_nu = int(g["cfg_n_nu"])
    nside_in = int(g["cfg_nside_in"])
    edges = list(g["nu0"]) + [g["nuf"][-1]]
    with open(tmp_path / "nu.dat", "w") as f:
        for i in range(n_nu):
            f.write("%d %.17g %.17g 0 0\n" % (i + 1, edges[i], edges[i + 1]))
    keys = {"fname_nutable": tmp_path / "nu.dat", "prefix_out": tmp_path / "out", "nside": int(g["cfg_nside"]),
            "seed": int(g["cfg_seed"]), "do_polarization": 1, "polarization_leakage": float(g["cfg_leakage"]),
            "dish_diameter": float(g["cfg_dish"]), "n_dishes": int(g["cfg_n_dish"]), "t_system": float(g["cfg_tsys"]),
            "time_total": float(g["cfg_time_tot"]), "rng": "mt_validation", "omp_threads_for_noise": 1}
    for comp in ORDER:
        if "in_" + comp not in g:
            keys["prefix_" + comp] = "none"
            continue
        keys["prefix_" + comp] = tmp_path / comp
        for i in range(n_nu):
            cols = [g["in_" + comp][i]] + ([g["in_synchrotron_q"][i]] if comp == "synchrotron" else [])
            write_map(tmp_path / ("%s_%03d.fits" % (comp, i + 1)), cols, nside_in)
    write_map(tmp_path / "mask.fits", [g["mask"].astype(np.float32)], int(g["cfg_nside"]))
    keys["fname_mask"] = tmp_path / "mask.fits"
    with open(tmp_path / "p.ini", "w") as f:
        for k, v in keys.items():
            f.write("%s= %s\n" % (k, v))
    exe = os.path.join(REPO, "crime_gb300", "lib", "JoinT_gpu")
    subprocess.run([exe, str(tmp_path / "p.ini")], check=True)
    for i in range(n_nu):
        h, d = read_map(str(tmp_path / ("out_%03d.fits" % (i + 1))))
        assert int(h["NSIDE"]) == int(g["cfg_nside"]) and h["ORDERING"] == "RING"
        np.testing.assert_array_equal(d, g["maps"][i])
    np.testing.assert_array_equal(np.loadtxt(tmp_path / "out_instrument.dat", ndmin=2), g["instrument"])


def _bandlimited(jt, j, nside, lmax_in, seed):
    """a map synthesised from random a_lm with l <= lmax_in (HEALPix order) and those a_lm"""
    lmax = 3 * nside - 1
    rng = np.random.default_rng(seed)
    alm = np.zeros(orc.nalms(lmax), np.complex64)
    for m in range(lmax_in + 1):
        i0 = m * (2 * lmax + 1 - m) // 2 + m  # index of (l = m, m): l + m lmax - m(m-1)/2
        cnt = lmax_in - m + 1
        alm[i0:i0 + cnt] = rng.standard_normal(cnt) + (1j * rng.standard_normal(cnt) if m else 0)
    return j.alm2map(alm)[0], alm


@pytest.mark.parametrize("nside", [512, 1024])
def test_beam_of_bandlimited_map_large_nside(jt, nside):
    """At Nside 512 (tensor cores) and 1024 (FP32 CUDA cores: 2-channel equatorial
    FFT blocks, 1-channel Bluestein at M = 8192): the beam of a band-limited map
    (l <= 48) equals the synthesis of b_l a_lm, to the HEALPix quadrature error."""
    lmax = 3 * nside - 1
    nu = np.array([800.0])
    j = jt.JoinT(nside, nu, nu + 10.0, dish_diameter=15.0)
    m, alm = _bandlimited(jt, j, nside, 48, nside)
    j.add_maps(m[None, :], nside)
    out = j.run()[0]
    assert j.uses_tensor_cores == (nside <= 512)
    b = orc.beam_window(lmax, orc.joint_fwhm([800.0], [810.0], 15.0)[0])
    l_of = np.concatenate([np.arange(mm, lmax + 1) for mm in range(lmax + 1)])
    ref = j.alm2map((alm * b[l_of]).astype(np.complex64))[0]
    assert rel_l2(out, ref) < 1e-4
    assert rel_l2(out, m) > 1e-3  # the beam changed the map


def test_tensor_and_fp32_legendre_agree_at_nside_512(jt):
    """the two Legendre paths on white-noise maps at Nside 512 (1024-term ring-pair
    sums, 2048-point ring FFTs): both FP32-accumulated, each within ~2-3e-6 of the
    exact beam, so they agree to 1e-5"""
    rng = np.random.default_rng(5)
    nu0 = np.array([700.0, 900.0])
    maps = rng.standard_normal((2, 12 * 512 * 512)).astype(np.float32)
    outs = []
    for prec in ("auto", "fp32"):
        j = jt.JoinT(512, nu0, nu0 + 5.0, dish_diameter=20.0, sht_precision=prec)
        j.add_maps(maps, 512)
        outs.append(j.run())
        j.close()
    assert rel_l2(outs[0], outs[1]) < 1e-5


def test_tensor_core_column_tiles_match_fp32(jt):
    """150 channels with 150 beam widths: the tensor-core path takes them as one batch
    of three 64-channel column tiles (the last padded), the FP32 path in batches of 64;
    per channel the two agree, and channels of each column tile match the oracle"""
    nside = 32
    rng = np.random.default_rng(150)
    nu0 = np.linspace(500.0, 1300.0, 150)
    nuf = nu0 + 5.0
    maps = (rng.standard_normal((150, 12 * nside * nside)) * 2 + 1).astype(np.float32)
    outs = []
    for prec in ("auto", "fp32"):
        j = jt.JoinT(nside, nu0, nuf, dish_diameter=6.0, sht_precision=prec)
        j.add_maps(maps, nside)
        outs.append(j.run())
        assert j.uses_tensor_cores == (prec == "auto")
        j.close()
    for ch in range(150):
        assert rel_l2(outs[0][ch], outs[1][ch]) < 1e-5, ch
    sel = [0, 70, 149]
    ref = orc.apply_beam(maps[sel], nside, orc.joint_fwhm(nu0[sel], nuf[sel], 6.0))
    assert rel_l2(outs[0][sel], ref) <= BEAM_L2
