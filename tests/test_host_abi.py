"""Host side of the GB300 library, no GPU needed: the C ABI exports, the .ini
parser (keys and defaults of src/io_gh.c:133-253), and the FP64 setup and
validation-mode draws against the golden vectors of the reference."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, REPO, load_case, oracle_for_case


@pytest.fixture(scope="session")
def gh():
    from crime_gb300 import build
    build.build()
    import crime_gb300
    return crime_gb300


def header_symbols():
    syms = set()
    for h in sorted(os.listdir(os.path.join(REPO, "include"))):
        src = open(os.path.join(REPO, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        syms |= set(re.findall(r"\b((?:gethi|joint)_\w+)\s*\(", src))
    return sorted(syms)


def test_library_exports_every_declared_symbol(gh):
    lib = ctypes.CDLL(gh.gethi.LIB_PATH)
    syms = header_symbols()
    assert len(syms) >= 40 and "joint_gpu_apply_beam" in syms
    for s in syms:
        assert hasattr(lib, s), s


def test_defaults_are_the_reference_defaults(gh):
    p = gh.default_params()
    # src/io_gh.c:137-172
    assert (p.omega_M, p.omega_L, p.omega_B, p.h, p.w, p.ns, p.sigma_8) == (0.3, 0.7, 0.05, 0.7, -1.0, 0.96, 0.83)
    assert (p.r_smooth, p.seed, p.n_side, p.nu_max, p.nu_min, p.n_nu, p.n_grid) == (2.0, 1234, 128, 1050., 350., 150, 512)
    assert p.prefix_out == b"default" and p.pk_filename == b"default"
    assert (p.do_rsd, p.velocity_mode, p.rng, p.bias_model) == (1, 0, 0, 0)


def test_ini_parser_keys(gh, tmp_path, capfd):
    ini = tmp_path / "p.ini"
    ini.write_text("""###File names
prefix_out= out/test
pk_filename= data/pk.dat
omega_M= 0.31
omega_L= 0.69
omega_B= 0.048
h= 0.68
w= -0.9
ns= 0.97
sigma_8= 0.81
r_smooth= 3.
frequencies_filename= data/nu.txt
nu_min= 355.
nu_max= 945.
n_nu= 150.
n_side= 512
n_grid= 2048
seed= 1001
do_psources= 0

velocity_mode= spectral
rng= mt_validation
bias_model= const
b_HI= 1.5
l_box= 4000
not_a_key= 3
""")
    p = gh.read_params(str(ini))
    assert p.prefix_out == b"out/test" and p.pk_filename == b"data/pk.dat"
    assert p.frequencies_filename == b"data/nu.txt"
    assert (p.omega_M, p.omega_L, p.omega_B, p.h, p.w, p.ns, p.sigma_8, p.r_smooth) == \
        (0.31, 0.69, 0.048, 0.68, -0.9, 0.97, 0.81, 3.0)
    assert (p.nu_min, p.nu_max, p.n_nu, p.n_side, p.n_grid, p.seed) == (355., 945., 150, 512, 2048, 1001)
    assert (p.velocity_mode, p.rng, p.bias_model, p.b_HI, p.l_box) == (1, 1, 1, 1.5, 4000.)
    assert "Unknown parameter not_a_key=" in capfd.readouterr().err


def test_ini_errors(gh, tmp_path):
    with pytest.raises(gh.GetHIError) as e:
        gh.read_params(str(tmp_path / "missing.ini"))
    assert e.value.code == -2
    bad = tmp_path / "bad.ini"
    bad.write_text("n_grid=\n")
    with pytest.raises(gh.GetHIError):
        gh.read_params(str(bad))
    bad.write_text("rng= sobol\n")
    with pytest.raises(gh.GetHIError) as e:
        gh.read_params(str(bad))
    assert e.value.code == -1


def params_for_case(gh, case):
    kw = dict(omega_M=0.315, omega_L=0.685, omega_B=0.049, h=0.67, w=-1.0, ns=0.96, sigma_8=0.83,
              pk_filename=os.path.join(GOLDEN, "pk_eh_nowiggle.txt"), n_grid=int(case["cfg_n_grid"]),
              n_side=int(case["cfg_n_side"]), seed=int(case["cfg_seed"]),
              r_smooth=float(case["cfg_r_smooth"]) if "cfg_r_smooth" in case else 2.0)
    if int(case["cfg_regular_nu"]):
        kw.update(frequencies_filename="", nu_min=float(case["cfg_nu_min"]), nu_max=float(case["cfg_nu_max"]),
                  n_nu=int(case["cfg_n_nu"]))
    else:
        kw.update(frequencies_filename=os.path.join(GOLDEN, "nutable_8.txt"))
    return gh.make_params(**kw)


@pytest.mark.parametrize("name", ["case_irr32", "case_reg24"])
def test_host_setup_matches_reference(gh, name):
    g = load_case(name)
    s = gh.host_setup(params_for_case(gh, g))
    d = s["derived"]
    for key in ("fgrowth_0", "hubble_0", "z_min", "z_max", "r_min", "r_max", "l_box", "glob_idr", "r2_smooth",
                "idlogk", "logkmin", "logkmax"):
        assert getattr(d, key) == g["p_" + key], key
    np.testing.assert_array_equal(s["pk"], g["pk"])
    np.testing.assert_array_equal(s["logk"], g["logk"])
    if "tables" in g:
        np.testing.assert_array_equal(s["tables"], g["tables"])
    o = oracle_for_case(g)
    xs, ys, zs = o.subsample_offsets()
    np.testing.assert_array_equal(s["offsets"], np.stack([xs, ys, zs], axis=1))
    np.testing.assert_array_equal(s["prefac"], o.prefactors())


@pytest.mark.parametrize("name", ["case_irr32", "case_reg24", "case_irr32_t3"])
def test_host_mt_modes_match_reference(gh, name):
    g = load_case(name)
    nthr = int(g["cfg_n_threads"])
    modes = gh.host_modes_mt(params_for_case(gh, g), nthr)
    np.testing.assert_array_equal(modes.view(np.float32).reshape(-1), g["dens_k"])


def test_host_psources_tables_match_reference(gh):
    g = load_case("case_ps32")
    t = gh.host_psources(params_for_case(gh, g))
    assert t["glob_dz"] == g["p_glob_dz"]
    np.testing.assert_array_equal(t["nz"], g["ps_nz"])
    np.testing.assert_array_equal(t["maxpdf"], g["ps_maxpdf"])
    # inverse CDF of log10 L: endpoints, monotone, and its median is the density's
    icdf = t["icdf"]
    assert icdf[0] == -5.0 and icdf[-1] == 6.0 and np.all(np.diff(icdf) > 0)
    x = np.linspace(-5, 6, 400001)
    L = 10 ** x
    f = (L / 2.11) ** 0.367 * np.exp(-L / 2.11)
    cdf = np.concatenate([[0], np.cumsum(0.5 * (f[1:] + f[:-1]))])
    cdf /= cdf[-1]
    for q in (0.1, 0.5, 0.9):
        assert abs(np.interp(q, cdf, x) - np.interp(q * 4096, np.arange(4097), icdf)) < 2e-3


def test_setup_rejects_bad_configs(gh):
    with pytest.raises(gh.GetHIError):
        gh.host_setup(gh.make_params(n_grid=33, pk_filename="EH", frequencies_filename=""))
    gh.host_setup(gh.make_params(do_psources=1, pk_filename="EH", frequencies_filename=""))  # point sources: built
    with pytest.raises(gh.GetHIError) as e:  # Gaussianised draws are Philox draws
        gh.host_setup(gh.make_params(gaussianise=1, rng="mt_validation", pk_filename="EH", frequencies_filename=""))
    assert e.value.code == -1
    gh.host_setup(gh.make_params(gaussianise=1, n_grid=16, pk_filename="EH", frequencies_filename=""))
    with pytest.raises(gh.GetHIError) as e:  # the tensor-core column transform is 1024-point
        gh.host_setup(gh.make_params(fft_precision="tc_split", n_grid=512, pk_filename="EH", frequencies_filename=""))
    assert e.value.code == -1
    gh.host_setup(gh.make_params(fft_precision="tc_split", n_grid=1024, pk_filename="EH", frequencies_filename=""))
    with pytest.raises(gh.GetHIError) as e:
        gh.host_setup(gh.make_params(pk_filename="/nonexistent", frequencies_filename=""))
    assert e.value.code == -2
    with pytest.raises(gh.GetHIError) as e:
        gh.host_setup(gh.make_params(omega_M=-0.1, pk_filename="EH", frequencies_filename=""))
    assert e.value.code == -3


def test_eh_table_and_filled_fraction(gh):
    s = gh.host_setup(gh.make_params(pk_filename="EH", frequencies_filename="", nu_min=NU21 / 2.0,
                                     nu_max=NU21 / 1.5, n_nu=30, n_grid=128, n_side=64, l_box=1500.0))
    d = s["derived"]
    assert d.numk == 1000 and abs(d.logkmin + 4) < 1e-12 and abs(d.logkmax - 1) < 1e-12
    assert d.l_box == 1500.0
    # shells at r > 1300 Mpc/h lie outside a 1500 Mpc/h box centred on the observer
    assert d.filled_fraction == 0.0


NU21 = 1420.40575177


def test_gpu_calls_fail_cleanly_without_device(gh):
    import torch
    if torch.cuda.is_available():
        pytest.skip("device present")
    with pytest.raises(gh.GetHIError) as e:
        gh.GetHI(gh.make_params(n_grid=32, n_side=8, pk_filename="EH", frequencies_filename=""))
    assert e.value.code in (-4, -5)
