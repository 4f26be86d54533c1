"""Certification bounds of the projection's per-cell expansions, checked on the CPU.

The projection keys a cell's ten sub-samples from per-cell expansions
(crime_gb300/csrc/stages.cu: cell_shell, cell_pix, key_lin):
  * the shell coordinate u (channel coordinate of a regular table) is linear in
    the sub-sample radius, u_c + s (R - Rc), with the FP64 table's deviation from
    the centre interval's line taken from a per-interval bound;
  * in the equatorial zone the two RING floor arguments n (0.5 + tt) -/+ 0.75 n cos
    theta are quadratics in the sub-sample offset.
A key is certified when its FP32 value lies farther than the margin from every
decision boundary, so the margins must bound the distance to the exact (FP64)
value, which follows the reference (src/pixelize.c:206-222, src/cosmo.c:52-62).
These tests restate the kernels' FP32 arithmetic in numpy (every operation
rounded to FP32, approximate reciprocals and the centre's azimuth perturbed to
their error budgets) on random cells of the bench geometries and check the error
against the margins, with the redshift tables and sub-sample offsets of the
oracle.
"""
import numpy as np
import pytest

from oracle import orc

NU21 = 1420.40575177
f32 = np.float32


def r32(x):
    return np.asarray(x, np.float64).astype(np.float32)


def fma(a, b, c):
    return r32(np.float64(a) * np.float64(b) + np.float64(c))


def geometry(n, box, nside, zmin, zmax, n_nu):
    nu_min, nu_max = NU21 / (1 + zmax), NU21 / (1 + zmin)
    cfg = dict(OmegaM=0.315, OmegaL=0.685, OmegaB=0.049, hhub=0.67, n_scal=0.96, sig8=0.83, nu_min=nu_min,
               nu_max=nu_max, l_box_override=box, n_grid=n, n_nu=n_nu, n_side=nside, regular_nu=1, do_rsd=1)
    k = np.logspace(-4, 2, 200)
    o = orc.Oracle(cfg, k, 1e4 * k / (1 + (k / 0.02) ** 3))
    dx = o.d.l_box / n
    xs, ys, zs = o.subsample_offsets()
    return o, dx, xs, ys, zs, nu_min, nu_max


def exact_positions(X, Y, Z, xs, ys, zs, dx, j):
    return (X.astype(np.float64) + xs[j] / dx, Y.astype(np.float64) + ys[j] / dx, Z.astype(np.float64) + zs[j] / dx)


GEOMETRIES = [  # n, box (Mpc/h), Nside, zmin, zmax, shells: the bench's 512^3, 1024^3 and 2048^3 workloads
    (512, 2500.0, 256, 0.3, 2.0, 150),
    (1024, 4000.0, 512, 0.3, 2.0, 150),
    (2048, 6000.0, 1024, 0.2, 2.5, 256),
]


@pytest.mark.parametrize("regular", [1, 0], ids=["regular", "frequency_file"])
@pytest.mark.parametrize("n,box,nside,zmin,zmax,n_nu", GEOMETRIES)
def test_shell_line_bound(n, box, nside, zmin, zmax, n_nu, regular):
    """u is the channel coordinate of a regular table, or the frequency itself
    (compared with FP32 edges) for a frequency file."""
    rng = np.random.default_rng(n + regular)
    o, dx, xs, ys, zs, nu_min, nu_max = geometry(n, box, nside, zmin, zmax, n_nu)
    zt = np.ctypeslib.as_array(o.d.z_r2z).copy()
    gi = o.d.glob_idr
    nz = len(zt)
    # the line table (shell_line_entry): slope per cell and deviation bound per interval
    rho_d = np.max(np.sqrt(xs ** 2 + ys ** 2 + zs ** 2)) / dx
    h = 1.0 / (gi * dx)
    Rn = np.arange(nz) * h
    g = np.diff(zt) * gi * dx
    E = np.zeros(nz - 1)
    for i in range(nz - 1):
        a, b = i * h, (i + 1) * h
        eps = 1e-3 + 1e-6 * b
        lo, hi = max(0.0, a - rho_d - eps), min(Rn[-1], b + rho_d + eps)
        kk = np.arange(max(0, int(lo / h) + 1), min(nz - 1, int(hi / h)) + 1)
        pts = np.concatenate([[lo, hi], Rn[kk]])
        E[i] = np.max(np.abs(np.interp(pts, Rn, zt) - zt[i] - g[i] * (pts - a)))
    E = r32(E * (1 + 1e-5) + 1e-12)
    gf, ztf = r32(g), r32(zt)
    rho = f32(rho_d * (1 + 1e-5) + 1e-6)
    idr_cell = f32(gi * dx)
    inv_dnu = n_nu / (nu_max - nu_min)
    sc, off = (f32(inv_dnu), f32(nu_min)) if regular else (f32(1), f32(0))
    ncell = 60000
    ix, iy, iz = (rng.integers(0, n, ncell) for _ in range(3))
    dzc = r32(rng.normal(0, 1.5e-3, ncell))
    Xc, Yc, Zc = r32(ix - n // 2), r32(iy - n // 2), r32(iz - n // 2)
    X, Y, Z = Xc + f32(0.5), Yc + f32(0.5), Zc + f32(0.5)
    R2 = fma(Z, Z, fma(Y, Y, r32(X * X)))
    Rc = r32(np.sqrt(np.float64(R2)))
    tr = r32(Rc * idr_cell)
    ok = (r32(tr + r32(rho * idr_cell * f32(1.0001))) < nz - 3) & (Rc > r32(2 * rho + 2))
    trs = np.where(ok, tr, f32(0))
    ir = trs.astype(np.int64)
    z0, z1 = ztf[ir], ztf[ir + 1]
    dzt = r32(z1 - z0)
    zz = r32(1 + r32(fma(dzt, r32(trs - ir), z0) + dzc))
    izz = r32(1 / np.float64(zz) * (1 + rng.uniform(-1.2e-7, 1.2e-7, ncell)))
    nu = r32(f32(NU21) * izz)
    u = r32(r32(nu - off) * sc) if regular else nu
    mnu = r32(2 * nu * r32(np.abs(dzt) * trs * f32(1.8e-7) * izz + f32(4.8e-7) + f32(2.7e-7)))
    mc = r32(r32(mnu + f32(1.2e-7) * nu) * sc + f32(4e-7) * np.abs(u) + f32(1e-6)) if regular else mnu
    gg, e = gf[ir], E[ir]
    d1 = r32(f32(NU21) * sc * izz * izz)
    s = r32(-d1 * gg)
    dZ = r32(np.abs(gg) * rho + e)
    zlo = r32(zz - dZ)
    ok &= zlo > 0.25
    izlo = r32(1 / np.float64(zlo))
    common = d1 * e + f32(2e-6) * np.abs(s) * rho + f32(NU21) * sc * dZ * dZ * izlo ** 3 + \
        f32(2e-7) * (np.abs(u) + np.abs(s) * rho)
    m_old = mc + f32(1.5) * (np.abs(s) * (f32(3.7e-7) * (Rc + rho) + f32(1.8e-7) * Rc) + common)
    m_lin = mc + f32(1.5) * (np.abs(s) * (rho * rho / (2 * (Rc - rho)) + f32(3e-7) * rho + f32(1e-7)) + common)
    sr = r32(s / np.float64(Rc))
    gx, gy, gz = r32(sr * X), r32(sr * Y), r32(sr * Z)
    rt = np.ctypeslib.as_array(o.d.r_r2z)
    worst_old = worst_lin = 0.0
    for j in range(10):
        # per-sample radius form (key_fast)
        tx, ty, tz = f32(0.5 + xs[j] / dx), f32(0.5 + ys[j] / dx), f32(0.5 + zs[j] / dx)
        Xs, Ys, Zs = r32(Xc + tx), r32(Yc + ty), r32(Zc + tz)
        R2s = fma(Zs, Zs, fma(Ys, Ys, r32(Xs * Xs)))
        Rs = r32(R2s * r32(1 / np.sqrt(np.float64(R2s)) * (1 + rng.uniform(-1.3e-7, 1.3e-7, ncell))))
        u_old = fma(s, r32(Rs - Rc), u)
        # offset form (key_lin)
        ox, oy, oz = r32(tx - f32(0.5)), r32(ty - f32(0.5)), r32(tz - f32(0.5))
        u_lin = fma(gz, oz, fma(gy, oy, fma(gx, ox, u)))
        px, py, pz = exact_positions(X, Y, Z, xs, ys, zs, dx, j)
        r = np.sqrt(px * px + py * py + pz * pz) * dx  # Mpc/h
        k = (r * gi).astype(np.int64)
        ze = zt[k] + (zt[k + 1] - zt[k]) * (r - rt[k]) * gi
        nue = NU21 / (1 + (ze + dzc.astype(np.float64)))
        te = inv_dnu * (nue - nu_min) if regular else nue
        worst_old = max(worst_old, np.max(np.abs(u_old[ok] - te[ok]) / m_old[ok]))
        worst_lin = max(worst_lin, np.max(np.abs(u_lin[ok] - te[ok]) / m_lin[ok]))
    assert ok.mean() > 0.99
    # each term is a worst case taken x1.5 (the FP32 centre's terms x2), so where one term
    # dominates (the second-order radius term of the offset form, near the observer) the
    # error may approach 1/1.5 of the margin; it must never reach it
    assert worst_old < 0.7 and worst_lin < 0.7, (worst_old, worst_lin)


@pytest.mark.parametrize("n,box,nside,zmin,zmax,n_nu", GEOMETRIES)
def test_equatorial_quadratic_bound(n, box, nside, zmin, zmax, n_nu):
    rng = np.random.default_rng(n + 1)
    o, dx, xs, ys, zs, _, _ = geometry(n, box, nside, zmin, zmax, n_nu)
    tox = r32(r32(0.5 + xs / dx) - f32(0.5))
    toy = r32(r32(0.5 + ys / dx) - f32(0.5))
    toz = r32(r32(0.5 + zs / dx) - f32(0.5))
    rho = f32(np.max(np.sqrt(xs ** 2 + ys ** 2 + zs ** 2)) / dx * (1 + 1e-5) + 1e-6)
    fn = f32(nside)
    K, L = r32(fn * f32(0.63661977)), r32(f32(0.75) * fn)
    ncell = 60000
    ix, iy, iz = (rng.integers(0, n, ncell) for _ in range(3))
    X, Y, Z = r32(ix - n // 2 + 0.5), r32(iy - n // 2 + 0.5), r32(iz - n // 2 + 0.5)
    rxy2 = r32(np.float64(X) * X + np.float64(Y) * Y)
    R2 = r32(rxy2 + np.float64(Z) * Z)
    Rc, rxy = r32(np.sqrt(np.float64(R2))), r32(np.sqrt(np.float64(rxy2)))
    cth = r32(np.float64(Z) / np.float64(Rc))
    tt = np.arctan2(np.float64(Y), np.float64(X)) / (np.pi / 2)
    tt = np.where(tt < 0, tt + 4, tt)
    q = np.floor(tt).astype(np.int64)
    w = r32(tt - q + rng.uniform(-2.05e-7, 2.05e-7, ncell))  # the FP32 azimuth within its budget

    def approx_inv(x):
        return r32(1 / np.float64(x) * (1 + rng.uniform(-1.2e-7, 1.2e-7, np.shape(x))))

    irxy2, iR = approx_inv(rxy2), approx_inv(Rc)
    Kr = r32(K * irxy2)
    Kr2 = r32(Kr * irxy2)
    a = [r32(-Kr * Y), r32(Kr * X), r32(Kr2 * r32(X * Y)), r32(Kr2 * r32(r32(Y * Y) - r32(X * X)))]
    Lr3 = r32(L * iR * iR * iR)
    hh = r32(f32(0.5) * Lr3)
    sx, sy, c2 = r32(X * iR), r32(Y * iR), r32(cth * cth)
    t3 = r32(3 * c2 - 1)
    b = [r32(-Lr3 * r32(X * Z)), r32(-Lr3 * r32(Y * Z)), r32(Lr3 * rxy2),
         r32(hh * Z * r32(3 * sx * sx - 1)), r32(hh * Z * r32(3 * sy * sy - 1)), r32(3 * hh * Z * r32(c2 - 1)),
         r32(3 * Lr3 * Z * sx * sy), r32(Lr3 * X * t3), r32(Lr3 * Y * t3)]
    base = r32(fn * r32(f32(0.5) + w))
    Lc = r32(L * cth)
    V1c, V2c = r32(base - Lc), r32(base + Lc)
    sa = sum(np.abs(v) for v in a[:2]) + sum(np.abs(v) for v in b[:3])
    sq = sum(np.abs(v) for v in a[2:]) + sum(np.abs(v) for v in b[3:])
    rmin, rxymin = Rc - rho, rxy - rho
    i1, i2 = rho / rxymin, rho / rmin
    third = K * i1 ** 3 / 3 + L * i2 ** 3
    mu = f32(2) * (fn * f32(2.05e-7 + 3e-7 + 1.2e-7) + L * f32(2.4e-7) + f32(1e-6) * (sa * rho + sq * rho * rho) +
                   f32(1e-7) * sa + third)
    dT = f32(0.63661977) * i1 + 1e-5
    lin = (rxymin > 1) & (np.abs(cth) + i2 + 1e-5 < 0.66666) & ~(((q == 0) & (w < dT)) | ((q == 3) & (w > 1 - dT)))
    worst = 0.0
    for j in range(10):
        ox, oy, oz = tox[j], toy[j], toz[j]
        dP = r32(np.float64(a[0]) * ox)
        for c, m in zip(a[1:], [oy, r32(ox * ox - oy * oy), r32(ox * oy)]):
            dP = fma(c, m, dP)
        dQ = r32(np.float64(b[0]) * ox)
        for c, m in zip(b[1:], [oy, oz, r32(ox * ox), r32(oy * oy), r32(oz * oz), r32(ox * oy), r32(ox * oz),
                                r32(oy * oz)]):
            dQ = fma(c, m, dQ)
        v1, v2 = r32(V1c + r32(dP - dQ)), r32(V2c + r32(dP + dQ))
        px, py, pz = exact_positions(X, Y, Z, xs, ys, zs, dx, j)
        ce = pz / np.sqrt(px * px + py * py + pz * pz)
        te = np.arctan2(py, px) / (np.pi / 2)
        te = np.where(te < 0, te + 4, te)
        V1e = nside * (0.5 + te) - 0.75 * nside * ce - nside * q
        V2e = nside * (0.5 + te) + 0.75 * nside * ce - nside * q
        err = np.maximum(np.abs(v1 - V1e), np.abs(v2 - V2e))
        worst = max(worst, np.max(err[lin] / mu[lin]))
    assert 0.6 < lin.mean() < 0.72  # the equatorial zone, less the cells at its edges
    assert worst < 0.5, worst
