"""Statistics of the Philox production draws (gaussianise=1) at 128^3 in a 600 Mpc/h
box, over four seeds:

* the Gaussian field's power spectrum is the drawn spectrum P_G, within the
  sample variance of its modes, and its one-point PDF is Gaussian with mean 0;
* the lognormal field exp(delta - sigma^2/2) has mean 1 and the power spectrum
  V/N^3 DFT[exp(xi_G) - 1] of the field's own correlation function, which equals
  the grid-sampled, smoothed input P(k) wherever the Gaussianisation is exact.

Only modes with 0 < kx < N/2 enter the spectra: the c2r keeps the real part of
the kx = 0 and N/2 planes, whose independently drawn modes then carry half the power
(the reference's own draw, src/fourier.c:275-299).  The expectation includes that
halving."""
import os

import numpy as np
import pytest

from conftest import COSMO, GOLDEN
from test_gpu_parity import gh  # noqa: F401  (fixture)

N = 128
L_BOX = 600.0
SEEDS = (7001, 7002, 7003, 7004)


def _oracle():
    from oracle import orc
    k, pk = orc.load_pk(os.path.join(GOLDEN, "pk_eh_nowiggle.txt"))
    cfg = dict(COSMO, r_smooth=2.0, n_grid=N, n_side=16, seed=1, regular_nu=1, nu_min=700.0, nu_max=900.0,
               n_nu=4, l_box_override=L_BOX)
    return orc.Oracle(cfg, k, pk)


def _power(field):
    """|DFT|^2 V / N^6 on the half grid (kx <= N/2)"""
    f = np.fft.rfftn(np.asarray(field, np.float64))
    return np.abs(f) ** 2 * L_BOX ** 3 / float(N) ** 6


def _bins():
    i = np.fft.fftfreq(N, 1.0 / N)
    kx = np.arange(N // 2 + 1)
    kk = np.sqrt(i[:, None, None] ** 2 + i[None, :, None] ** 2 + kx[None, None, :] ** 2)
    use = (kx[None, None, :] > 0) & (kx[None, None, :] < N // 2) & (kk >= 2) & (kk < N // 2)
    b = np.floor(kk).astype(int)
    return b, use


def _binned(p, b, use):
    nb = N // 2
    s = np.bincount(b[use], weights=p[use], minlength=nb)
    c = np.bincount(b[use], minlength=nb)
    return s, c


@pytest.mark.gpu
def test_philox_gaussianised_statistics(gh):  # noqa: F811
    orc = _oracle()
    pg = np.maximum(orc.gaussianised_pk(), 0.0)  # [kz][ky][kx] full grid, FP64
    ptil = orc.pk_grid()
    # the Gaussian field's spectrum as drawn: P_G, half power on the kx = 0 and N/2 planes
    pg_eff = pg.copy()
    pg_eff[:, :, 0] *= 0.5
    pg_eff[:, :, N // 2] *= 0.5
    vol = L_BOX ** 3
    xi_g = np.fft.ifftn(pg_eff / vol).real * N ** 3
    p_ln = np.fft.rfftn(np.expm1(xi_g)).real * vol / N ** 3  # the lognormal field's spectrum
    b, use = _bins()

    p = gh.make_params(pk_filename=os.path.join(GOLDEN, "pk_eh_nowiggle.txt"), frequencies_filename="",
                       nu_min=700.0, nu_max=900.0, n_nu=4, n_side=16, n_grid=N, l_box=L_BOX, do_rsd=0,
                       gaussianise=1, r_smooth=2.0, omega_M=0.315, omega_L=0.685, omega_B=0.049, h=0.67,
                       w=-1.0, ns=0.96, sigma_8=0.83)
    ctx = gh.GetHI(p)
    sg = np.zeros(N // 2)
    sl = np.zeros(N // 2)
    cnt = None
    for seed in SEEDS:
        ctx.set_seed(seed)
        ctx.create_d_and_vr_fields()
        d, _ = ctx.grids()
        d = d.astype(np.float64)
        s2 = ctx.derived().sigma2_gauss
        # one-point statistics of the Gaussian field
        assert abs(d.mean()) < 1e-6 * np.sqrt(s2)
        assert abs(d.var() / s2 - 1) < 1e-4  # sigma^2 of the GPU is the field's own variance
        z = d / np.sqrt(s2)
        assert abs((z ** 3).mean()) < 0.05 and abs((z ** 4).mean() - 3) < 0.1
        rho = np.exp(d - 0.5 * s2)
        assert abs(rho.mean() - 1) < 0.05
        x, cnt = _binned(_power(d), b, use)
        sg += x
        x, _ = _binned(_power(rho - rho.mean()), b, use)
        sl += x
    ctx.free()
    nr = len(SEEDS)
    eg, _ = _binned(np.broadcast_to(pg_eff[:, :, :N // 2 + 1], (N, N, N // 2 + 1)), b, use)
    el, _ = _binned(p_ln, b, use)
    ok = cnt > 0
    mg, ml = sg[ok] / (cnt[ok] * nr), sl[ok] / (cnt[ok] * nr)
    eg, el = eg[ok] / cnt[ok], el[ok] / cnt[ok]
    sig = 1.0 / np.sqrt(cnt[ok] * nr)  # relative error of a bin mean for Gaussian modes
    # Gaussian field: every bin within 5 sigma, chi^2 per bin near 1
    rg = (mg / eg - 1) / sig
    assert np.all(np.abs(rg) < 5), rg
    assert np.mean(rg ** 2) < 2.0
    # lognormal field: modes are not Gaussian (larger scatter), so 8 sigma per bin, and
    # the spectrum-weighted mean ratio within 1%
    rl = (ml / el - 1) / sig
    assert np.all(np.abs(rl) < 8), rl
    assert abs(np.sum(ml * cnt[ok]) / np.sum(el * cnt[ok]) - 1) < 0.01
    # and that spectrum is the input P(k) where the Gaussianisation is exact (low k)
    pt, _ = _binned(np.broadcast_to(ptil[:, :, :N // 2 + 1], (N, N, N // 2 + 1)), b, use)
    pt = pt[ok] / cnt[ok]
    low = slice(0, 10)
    assert np.all(np.abs(el[low] / pt[low] - 1) < 0.02)
