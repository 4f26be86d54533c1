"""GPU path against the oracle and the reference's golden vectors, through the C ABI.

Tolerances: integer work (per-sample pixel and shell keys) is bit-exact;
FP32 fields against FP64 references are compared by relative L2 norm
(FFT: 2e-6, finite-difference velocity: 2e-5), HI mass/dz element-wise to
2e-5 relative, maps element-wise to 1e-5 relative (FP32 sums in a different
order than the reference's atomics)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_case, oracle_for_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gh():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crime_gb300 import build
    build.build()
    import crime_gb300
    return crime_gb300


def params_for_case(gh, case, **extra):
    kw = dict(omega_M=0.315, omega_L=0.685, omega_B=0.049, h=0.67, w=-1.0, ns=0.96, sigma_8=0.83,
              pk_filename=os.path.join(GOLDEN, "pk_eh_nowiggle.txt"), n_grid=int(case["cfg_n_grid"]),
              n_side=int(case["cfg_n_side"]), seed=int(case["cfg_seed"]),
              r_smooth=float(case["cfg_r_smooth"]) if "cfg_r_smooth" in case else 2.0)
    if int(case["cfg_regular_nu"]):
        kw.update(frequencies_filename="", nu_min=float(case["cfg_nu_min"]), nu_max=float(case["cfg_nu_max"]),
                  n_nu=int(case["cfg_n_nu"]))
    else:
        kw.update(frequencies_filename=os.path.join(GOLDEN, "nutable_8.txt"))
    kw.update(extra)
    return gh.make_params(**kw)


def cells(a, n):
    """real cells of a padded reference grid -> compact [z][y][x]"""
    return np.asarray(a).reshape(n, n, 2 * (n // 2 + 1))[:, :, :n]


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


CASES = ["case_irr32", "case_reg24"]


@pytest.fixture(scope="module", params=CASES)
def run(request, gh):
    g = load_case(request.param)
    n = int(g["cfg_n_grid"])
    ctx = gh.GetHI(params_for_case(gh, g))
    modes = g["dens_k"].view(np.complex64).reshape(n, n, n // 2 + 1)
    ctx.create_d_and_vr_fields(modes)
    yield g, ctx, n
    ctx.free()


def test_fields_vs_reference(run):
    g, ctx, n = run
    dens, vr = ctx.grids()
    assert rel_l2(dens, cells(g["dens_real"], n)) < 2e-6
    assert rel_l2(vr, cells(g["rvel"], n)) < 2e-5
    d = ctx.derived()
    assert abs(d.sigma2_gauss / g["p_sigma2_gauss"] - 1) < 2e-6


def test_get_hi_vs_reference(run):
    g, ctx, n = run
    ctx.upload_grids(cells(g["dens_real"], n), cells(g["rvel"], n), stage=1)
    ctx.get_HI()
    mass, dz = ctx.grids()
    np.testing.assert_allclose(mass, cells(g["mass"], n), rtol=2e-5, atol=0)
    ref_dz = cells(g["dz"], n)
    np.testing.assert_allclose(dz, ref_dz, rtol=2e-5, atol=2e-5 * np.abs(ref_dz).max())


@pytest.mark.parametrize("exact", [True, False], ids=["fp64", "fp32_certified"])
def test_sample_keys_bitexact(run, exact):
    g, ctx, n = run
    ctx.upload_grids(cells(g["mass"], n), cells(g["dz"], n), stage=2)
    keys = ctx.sample_keys(exact=exact)
    o = oracle_for_case(g)
    _, okeys = o.mk_T_maps(g["mass"], g["dz"], want_keys=True)
    assert np.count_nonzero(okeys != 0xFFFFFFFF) > 0.3 * okeys.size
    np.testing.assert_array_equal(keys, okeys)


def test_maps_vs_reference(run):
    g, ctx, n = run
    ctx.upload_grids(cells(g["mass"], n), cells(g["dz"], n), stage=2)
    maps = ctx.mk_T_maps()
    ref = g["maps"].reshape(maps.shape)
    np.testing.assert_allclose(maps, ref, rtol=1e-5, atol=1e-6 * np.abs(ref).max())


def test_philox_modes_vs_oracle(gh):
    g = load_case("case_irr32")
    ctx = gh.GetHI(params_for_case(gh, g))
    dm = ctx.device_modes()
    ctx.free()
    om = oracle_for_case(g).modes_philox()
    amp = np.abs(om)
    assert np.all(np.abs(dm - om) <= 3e-5 * amp + 1e-30)


@pytest.mark.parametrize("l_box,effect", [(None, 1e-3), (400.0, 0.1)])
def test_gaussianised_modes_vs_oracle(gh, l_box, effect):
    """gaussianise=1: P_G from xi_G = ln(1 + xi) on the grid (FP32 FFTs, FP64 log)
    against the all-FP64 oracle; the modes share the Philox draws, so they
    differ only through P_G.  The 400 Mpc/h box has xi(0) = 0.82."""
    g = load_case("case_irr32")
    extra = {} if l_box is None else dict(l_box=l_box)
    ctx = gh.GetHI(params_for_case(gh, g, gaussianise=1, **extra))
    dm = ctx.device_modes()
    ctx.free()
    orc = oracle_for_case(g, **({} if l_box is None else dict(l_box_override=l_box)))
    om = orc.modes_philox_gaussianised()
    assert np.linalg.norm(dm - om) / np.linalg.norm(om) < 1e-4
    # P_G differs from P(k) by more than the tolerance at this variance
    pm = orc.modes_philox()
    assert np.linalg.norm(om - pm) / np.linalg.norm(pm) > effect


def test_spectral_velocity_vs_oracle(gh):
    g = load_case("case_irr32")
    n = int(g["cfg_n_grid"])
    ctx = gh.GetHI(params_for_case(gh, g, velocity_mode="spectral"))
    modes = g["dens_k"].view(np.complex64).reshape(n, n, n // 2 + 1)
    ctx.create_d_and_vr_fields(modes)
    _, vr = ctx.grids()
    ctx.free()
    ref = cells(oracle_for_case(g).radial_velocity_spectral(modes), n)
    assert rel_l2(vr, ref) < 2e-6


def test_stage_order_and_errors(gh):
    g = load_case("case_reg24")
    ctx = gh.GetHI(params_for_case(gh, g))
    with pytest.raises(gh.GetHIError) as e:
        ctx.get_HI()
    assert e.value.code == -6
    with pytest.raises(gh.GetHIError) as e:
        ctx.mk_T_maps()
    assert e.value.code == -6
    ctx.free()
    with pytest.raises(gh.GetHIError) as e:
        gh.GetHI(params_for_case(gh, g, n_grid=48))
    assert e.value.code == -1


@pytest.mark.parametrize("vmode", ["fd", "spectral"])
def test_production_run_vs_oracle(gh, vmode):
    """Philox modes end to end (run() fuses get_HI into the projection) against
    the oracle fed with the same modes: FP64 FFTs, FP64 lognormal, reference binning."""
    g = load_case("case_irr32")
    n = int(g["cfg_n_grid"])
    ctx = gh.GetHI(params_for_case(gh, g, velocity_mode=vmode))
    maps = ctx.run()
    modes = ctx.device_modes()
    ctx.free()
    o = oracle_for_case(g)
    dens = o.normalize(o.c2r(modes))
    if vmode == "fd":
        k = np.fft.fftfreq(n, 1.0 / n) * (2 * np.pi / o.d.l_box)
        kx = np.abs(k[: n // 2 + 1])
        kx[n // 2] = n // 2 * 2 * np.pi / o.d.l_box
        kz, ky = k.copy(), k.copy()
        kz[n // 2] = ky[n // 2] = n // 2 * 2 * np.pi / o.d.l_box
        k2 = kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2
        k2[0, 0, 0] = 1
        vk = (modes.astype(np.complex128) * (o.d.fgrowth_0 * o.d.hubble_0) / k2).astype(np.complex64)
        rv = o.radial_velocity_fd(o.normalize(o.c2r(vk)))
    else:
        rv = o.radial_velocity_spectral(modes)
    _, s2 = o.sigma(dens)
    mass, dz = o.get_hi(dens, rv, s2)
    ref = o.mk_T_maps(mass, dz)
    assert rel_l2(maps, ref) < 1e-4
    close = np.isclose(maps, ref, rtol=1e-5, atol=1e-6 * np.abs(ref).max())
    assert close.mean() > 0.995


def synthetic_params(gh, **kw):
    nu21 = 1420.40575177
    base = dict(omega_M=0.315, omega_L=0.685, omega_B=0.049, h=0.67, w=-1.0, ns=0.96, sigma_8=0.83,
                pk_filename=os.path.join(GOLDEN, "pk_eh_nowiggle.txt"), frequencies_filename="",
                nu_min=nu21 / 3.0, nu_max=nu21 / 1.3, n_nu=150, seed=11)
    base.update(kw)
    return gh.make_params(**base)


def test_fast_keys_certified_high_nside(gh):
    """FP32 keys with margins == FP64 keys on 21M samples at Nside=512, random dz."""
    n = 128
    ctx = gh.GetHI(synthetic_params(gh, n_grid=n, n_side=512, l_box=2000.0))
    rng = np.random.default_rng(5)
    mass = rng.lognormal(0, 1, (n, n, n)).astype(np.float32)
    dz = rng.normal(0, 3e-3, (n, n, n)).astype(np.float32)
    ctx.upload_grids(mass, dz, stage=2)
    exact = ctx.sample_keys(exact=True)
    fast = ctx.sample_keys(exact=False)
    ctx.free()
    assert np.count_nonzero(exact != 0xFFFFFFFF) > 0.5 * exact.size
    np.testing.assert_array_equal(fast, exact)


def test_projection_many_keys_per_tile(gh):
    """Small box, high Nside: every sample of a tile is its own pixel, so the
    per-tile key table overflows; maps must still match the oracle."""
    from oracle import orc
    n, nside = 32, 1024
    nu21 = 1420.40575177
    p = synthetic_params(gh, n_grid=n, n_side=nside, l_box=300.0, nu_min=nu21 / 1.12, nu_max=nu21 / 1.02, n_nu=4)
    ctx = gh.GetHI(p)
    rng = np.random.default_rng(9)
    mass = rng.lognormal(0, 1, (n, n, n)).astype(np.float32)
    dz = rng.normal(0, 1e-3, (n, n, n)).astype(np.float32)
    ctx.upload_grids(mass, dz, stage=2)
    maps = ctx.mk_T_maps()
    ctx.free()
    k, pk = orc.load_pk(os.path.join(GOLDEN, "pk_eh_nowiggle.txt"))
    o = orc.Oracle(dict(OmegaM=0.315, OmegaL=0.685, OmegaB=0.049, hhub=0.67, weos=-1.0, n_scal=0.96, sig8=0.83,
                        n_grid=n, n_side=nside, seed=11, regular_nu=1, nu_min=p.nu_min, nu_max=p.nu_max, n_nu=4,
                        l_box_override=300.0), k, pk)
    pad = np.zeros((n, n, 2 * (n // 2 + 1)), np.float32)
    padz = np.zeros_like(pad)
    pad[:, :, :n] = mass
    padz[:, :, :n] = dz
    ref = o.mk_T_maps(pad, padz)
    assert np.count_nonzero(ref) > 10000
    np.testing.assert_allclose(maps, ref, rtol=1e-5, atol=1e-6 * np.abs(ref).max())


def test_fast_keys_certified_nside1024(gh):
    """The 2048^3 workload's geometry (box 6000 Mpc/h, 256 shells over z 0.2-2.5,
    Nside 1024) at 128^3: certified FP32 keys == FP64 keys on 21M samples."""
    nu21 = 1420.40575177
    n = 128
    ctx = gh.GetHI(synthetic_params(gh, n_grid=n, n_side=1024, l_box=6000.0, nu_min=nu21 / 3.5, nu_max=nu21 / 1.2,
                                    n_nu=256))
    rng = np.random.default_rng(6)
    mass = rng.lognormal(0, 1, (n, n, n)).astype(np.float32)
    dz = rng.normal(0, 3e-3, (n, n, n)).astype(np.float32)
    ctx.upload_grids(mass, dz, stage=2)
    exact = ctx.sample_keys(exact=True)
    fast = ctx.sample_keys(exact=False)
    ctx.free()
    assert np.count_nonzero(exact != 0xFFFFFFFF) > 0.5 * exact.size
    np.testing.assert_array_equal(fast, exact)


def test_c1_shaped_run_vs_oracle(gh):
    """The 512^3 workload's shells at 128^3 (box 2500 Mpc/h, 150 shells over z
    0.3-2.0, Nside 256, spectral RSD, Gaussianised P(k), Philox modes): the fused
    run() against the oracle on the same modes, with the tolerances of
    test_production_run_vs_oracle; then the validation path, the oracle's own
    mass and dz uploaded: FP32 keys == FP64 keys, maps element-wise within 1e-5."""
    from oracle import orc
    nu21 = 1420.40575177
    n, nside = 128, 256
    p = synthetic_params(gh, n_grid=n, n_side=nside, l_box=2500.0, nu_min=nu21 / 3.0, nu_max=nu21 / 1.3, n_nu=150,
                         velocity_mode="spectral", gaussianise=1, seed=2001)
    ctx = gh.GetHI(p)
    maps = ctx.run()
    modes = ctx.device_modes()
    k, pk = orc.load_pk(os.path.join(GOLDEN, "pk_eh_nowiggle.txt"))
    o = orc.Oracle(dict(OmegaM=0.315, OmegaL=0.685, OmegaB=0.049, hhub=0.67, weos=-1.0, n_scal=0.96, sig8=0.83,
                        n_grid=n, n_side=nside, seed=2001, regular_nu=1, nu_min=p.nu_min, nu_max=p.nu_max,
                        n_nu=150, l_box_override=2500.0), k, pk)
    dens = o.normalize(o.c2r(modes))
    rv = o.radial_velocity_spectral(modes)
    _, s2 = o.sigma(dens)
    mass, dz = o.get_hi(dens, rv, s2)
    ref = o.mk_T_maps(mass, dz)
    assert np.count_nonzero(ref) > 100000
    assert rel_l2(maps, ref) < 1e-4
    close = np.isclose(maps, ref, rtol=1e-5, atol=1e-6 * np.abs(ref).max())
    assert close.mean() > 0.995
    # validation path on the oracle's grids
    ctx.upload_grids(np.ascontiguousarray(cells(mass, n)), np.ascontiguousarray(cells(dz, n)), stage=2)
    np.testing.assert_array_equal(ctx.sample_keys(exact=False), ctx.sample_keys(exact=True))
    vmaps = ctx.mk_T_maps()
    ctx.free()
    np.testing.assert_allclose(vmaps, ref, rtol=1e-5, atol=1e-6 * np.abs(ref).max())


def test_tma_and_bulk_passes_match_register_passes(gh):
    """At 512^3 the Y passes run from TMA-staged tiles and the X passes from
    bulk-copied rows by default; the same Philox realisation with every pass
    loading through registers (gethi_gpu_set_launch col_variant=2) gives the same
    delta, v_r and sigma^2 to FP32 rounding (the compiler fuses products into
    FMAs differently in the kernels)."""
    nu21 = 1420.40575177
    n = 512
    ctx = gh.GetHI(synthetic_params(gh, n_grid=n, n_side=64, l_box=2500.0, nu_min=nu21 / 3.0, nu_max=nu21 / 1.3,
                                    n_nu=8, velocity_mode="spectral", seed=77))
    ctx.create_d_and_vr_fields()
    d_tma, v_tma = ctx.grids()
    s_tma = ctx.derived().sigma2_gauss
    ctx.set_launch(0, 2)
    ctx.create_d_and_vr_fields()
    d_reg, v_reg = ctx.grids()
    s_reg = ctx.derived().sigma2_gauss
    ctx.free()
    assert np.isfinite(d_tma).all() and np.abs(d_tma).max() > 0
    # each path is ~2e-7 from FP64; the FFT bound against FP64 is 2e-6
    assert rel_l2(d_tma, d_reg) < 1e-6
    assert rel_l2(v_tma, v_reg) < 1e-6
    assert abs(s_tma - s_reg) < 1e-6 * s_reg
