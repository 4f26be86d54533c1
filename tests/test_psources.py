"""Point sources on the GPU (do_psources=1) against the oracle.

The GPU draws with counter-based Philox streams, so its sources are compared in
two ways: (1) its own catalogue (cells, positions, luminosities, dz_rsd) run
through the oracle's FP64 restatement of mk_psources_maps must give the same
pixel for every source and the same maps; (2) its draws must follow the
reference's distributions: the number of sources against the sum of the cells'
Poisson means (computed by the oracle from the same Gaussian field), and the
luminosities against the luminosity function of src/psources.c:39-52."""
import numpy as np
import pytest

from conftest import load_case, oracle_for_case
from test_gpu_parity import gh, params_for_case  # noqa: F401  (fixture)


def _padded(a, n):
    out = np.zeros((n, n, 2 * (n // 2 + 1)), np.float32)
    out[:, :, :n] = np.asarray(a).reshape(n, n, n)
    return out


@pytest.fixture(scope="module")
def run(gh):  # noqa: F811
    g = load_case("case_ps32")
    ctx = gh.GetHI(params_for_case(gh, g, do_psources=1, seed=91))
    ctx.create_d_and_vr_fields()
    maps, ns = ctx.psources_maps()
    cat = ctx.psources_catalogue()
    d, _ = ctx.grids()
    s2 = ctx.derived().sigma2_gauss
    ctx.free()
    return dict(g=g, maps=maps, ns=ns, cat=cat, dens=d, sigma2=s2)


@pytest.mark.gpu
def test_catalogue_pixels_and_maps_vs_oracle(run):
    g, cat = run["g"], run["cat"]
    # the catalogue holds the sources that contribute: sources of a cell below z_max whose
    # own position lies beyond it get no luminosity (src/psources.c:130)
    assert 1000 < cat["count"] <= run["ns"] and run["ns"] - cat["count"] < 0.1 * run["ns"]
    assert len(cat["cell"]) == cat["count"]
    o = oracle_for_case(g)
    ref, pix = o.psources_maps_catalogue(cat["cell"], cat["u"], cat["L0"], cat["dz"])
    # the pixel of every source is the FP64 RING pixel of its position (bit-exact)
    np.testing.assert_array_equal(cat["pix"], pix)
    # maps: FP32 sums of the two per-pixel factors against FP64 per-channel sums
    got = run["maps"].astype(np.float64)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5
    assert np.abs(got - ref).max() < 1e-5 * np.abs(ref).max()


@pytest.mark.gpu
def test_source_statistics(run):
    g, cat = run["g"], run["cat"]
    o = oracle_for_case(g)
    n = o.n
    lam = o.ps_lambda(_padded(run["dens"], n), run["sigma2"])
    mu = lam.sum()
    # the count is Poisson with mean sum(lambda) (cells beyond z_max have no sources)
    assert abs(run["ns"] - mu) < 5 * np.sqrt(mu)
    occupied = np.bincount(cat["cell"], minlength=n ** 3)
    assert np.all(occupied[lam.reshape(-1) == 0] == 0)
    # positions uniform in the cell
    u = cat["u"].astype(np.float64)
    assert np.all((u >= 0) & (u < 1)) and np.all(np.abs(u.mean(axis=0) - 0.5) < 0.05)
    # log10 L follows dn/dlog10 L (z factor cancels): Kolmogorov-Smirnov at 99.9%
    x = np.sort(np.log10(cat["L0"].astype(np.float64)))
    grid = np.linspace(-5, 6, 400001)
    L = 10 ** grid
    f = (L / 2.11) ** 0.367 * np.exp(-L / 2.11)
    cdf = np.concatenate([[0], np.cumsum(0.5 * (f[1:] + f[:-1]))])
    cdf /= cdf[-1]
    model = np.interp(x, grid, cdf)
    emp_hi = np.arange(1, len(x) + 1) / len(x)
    emp_lo = np.arange(len(x)) / len(x)
    D = max(np.max(emp_hi - model), np.max(model - emp_lo))
    assert D < 1.95 / np.sqrt(len(x))


@pytest.mark.gpu
def test_psources_run_and_outputs(gh, tmp_path):  # noqa: F811
    """The fused run draws the same sources as the staged path; write_maps adds
    <prefix>_ps_%03d.fits; batches refuse point sources."""
    g = load_case("case_ps32")
    p = params_for_case(gh, g, do_psources=1, seed=91, prefix_out=str(tmp_path / "out"))
    ctx = gh.GetHI(p)
    maps = ctx.run()
    ps, ns = ctx.psources_maps()
    ctx.create_d_and_vr_fields()
    ps2, ns2 = ctx.psources_maps()
    assert ns == ns2 > 0
    assert np.linalg.norm(ps - ps2) <= 1e-6 * np.linalg.norm(ps2)
    ctx.write_maps(maps)
    for i in range(1, int(g["cfg_n_nu"]) + 1):
        assert (tmp_path / ("out_%03d.fits" % i)).exists()
        assert (tmp_path / ("out_ps_%03d.fits" % i)).exists()
    with pytest.raises(gh.GetHIError):
        gh.run_batch([ctx], [(0, 5)])
    ctx.free()
