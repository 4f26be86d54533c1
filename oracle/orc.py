"""ctypes wrapper of the oracle (oracle/_build/liborc.so) -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg.  Grids use the reference's padded layout: real [z][y][2(N/2+1)] float32,
half spectra [kz][ky][N/2+1] complex64.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liborc.so")
NZ = 5001
NU21 = 1420.40575177


def build():
    subprocess.run(["make", "-C", HERE, "all"], check=True, stdout=subprocess.DEVNULL)


class Config(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("OmegaM", "OmegaL", "OmegaB", "hhub", "weos", "n_scal", "sig8",
                                          "r_smooth", "nu_min", "nu_max", "l_box_override", "b_HI")] + [
        ("n_side", C.c_long), ("n_grid", C.c_int), ("n_nu", C.c_int), ("seed", C.c_uint),
        ("regular_nu", C.c_int), ("bias_const", C.c_int), ("do_rsd", C.c_int), ("pad_", C.c_int)]


class Derived(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("fgrowth_0", "hubble_0", "z_min", "z_max", "r_min", "r_max",
                                          "l_box")] + [("pos_obs", C.c_double * 3)] + [
        (n, C.c_double) for n in ("r2_smooth", "glob_idr", "logkmin", "logkmax", "idlogk", "n_scal",
                                  "sigma8_in", "pk_norm")] + [
        ("do_smoothing", C.c_int), ("numk", C.c_int)] + [
        (n, C.c_double * NZ) for n in ("z_z2r", "r_z2r", "z_r2z", "r_r2z", "gd", "gv")]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
        L.orc_cosmo_set.argtypes = [P(Config), C.c_int, f64p, f64p, f64p, f64p, P(Derived)]
        L.orc_cosmo_set.restype = C.c_int
        for fn in ("orc_z_of_r", "orc_r_of_z", "orc_dgrowth_of_r", "orc_vgrowth_of_r"):
            getattr(L, fn).argtypes = [P(Derived), C.c_double]
            getattr(L, fn).restype = C.c_double
        L.orc_modes_mt.argtypes = [P(Config), P(Derived), f64p, f64p, C.c_int, f32p, C.c_void_p]
        L.orc_modes_philox.argtypes = [P(Config), P(Derived), f64p, f64p, f32p]
        L.orc_modes_philox_pg.argtypes = [P(Config), P(Derived), f64p, f64p, f64p, f32p]
        L.orc_pk_grid.argtypes = [P(Config), P(Derived), f64p, f64p, f64p]
        L.orc_c2r_inplace.argtypes = [C.c_int, f32p]
        L.orc_c2r_to_double.argtypes = [C.c_int, f32p, f64p]
        L.orc_normalize.argtypes = [C.c_int, C.c_double, f32p]
        L.orc_radial_velocity_fd.argtypes = [P(Config), P(Derived), f32p, f32p]
        L.orc_radial_velocity_spectral.argtypes = [P(Config), P(Derived), f32p, f32p]
        L.orc_sigma_dens.argtypes = [C.c_int, f32p, P(C.c_double), P(C.c_double)]
        L.orc_get_hi.argtypes = [P(Config), P(Derived), C.c_double, f32p, f32p]
        L.orc_subsample_offsets.argtypes = [C.c_uint, C.c_double, f64p, f64p, f64p]
        L.orc_vec2pix_ring.argtypes = [C.c_long, f64p]
        L.orc_vec2pix_ring.restype = C.c_long
        L.orc_pix2ang_ring.argtypes = [C.c_long, C.c_long, P(C.c_double), P(C.c_double)]
        L.orc_mk_T_maps.argtypes = [P(Config), P(Derived), f64p, f64p, f32p, f32p, f32p, C.c_void_p]
        L.orc_channel_prefactors.argtypes = [P(Config), P(Derived), f64p, f64p, f64p]
        L.orc_philox4x32_10.argtypes = [u32p, u32p, u32p]
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
        L.orc_setup_psources.argtypes = [C.c_double, f64p, f64p, P(C.c_double)]
        L.orc_point_sources.argtypes = [P(Config), P(Derived), f64p, C.c_double, f32p, C.c_double, C.c_int, i32p]
        L.orc_point_sources.restype = C.c_long
        L.orc_psources_maps.argtypes = [P(Config), P(Derived), f64p, f64p, f64p, f64p, C.c_double, i32p, f32p,
                                        C.c_int, f32p]
        L.orc_psources_maps_catalogue.argtypes = [P(Config), P(Derived), f64p, f64p, C.c_long, i64p, f64p, f64p,
                                                  f64p, f64p, i64p]
        L.orc_n_of_z_psources.argtypes = [f64p, C.c_double, C.c_double]
        L.orc_ps_lambda.argtypes = [P(Config), P(Derived), f64p, C.c_double, f32p, C.c_double, f64p]
        L.orc_n_of_z_psources.restype = C.c_double
        for fn in ("orc_nest2ring", "orc_ring2nest"):
            getattr(L, fn).argtypes = [C.c_long, C.c_long]
            getattr(L, fn).restype = C.c_long
        L.orc_ring_info.argtypes = [C.c_long, C.c_long, P(C.c_long), P(C.c_long), P(C.c_double), P(C.c_double),
                                    P(C.c_double)]
        L.orc_lambda_m.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, f64p]
        L.orc_map2alm.argtypes = [C.c_long, C.c_int, f64p, f64p]
        L.orc_alm2map.argtypes = [C.c_long, C.c_int, f64p, f64p]
        L.orc_udgrade.argtypes = [f32p, C.c_long, f32p, C.c_long]
        L.orc_beam_window.argtypes = [C.c_int, C.c_double, f64p]
        L.orc_apply_beam.argtypes = [C.c_long, C.c_int, f64p, f32p]
        L.orc_add_noise.argtypes = [C.c_long, C.c_int, f64p, f64p, C.c_double, C.c_double, C.c_double, C.c_int,
                                    C.c_uint, C.c_int, f32p]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_num_threads.restype = C.c_int
        _lib = L
    return _lib


class Oracle:
    """One GetHI configuration evaluated by the oracle, stage by stage."""

    def __init__(self, cfg: dict, k, pk, nu0=None, nuf=None):
        self.c = Config()
        defaults = dict(OmegaM=0.3, OmegaL=0.7, OmegaB=0.05, hhub=0.7, weos=-1.0, n_scal=0.96, sig8=0.83,
                        r_smooth=2.0, nu_min=350.0, nu_max=1050.0, l_box_override=-1.0, b_HI=1.0,
                        n_side=128, n_grid=512, n_nu=150, seed=1234, regular_nu=0, bias_const=0, do_rsd=1)
        defaults.update(cfg)
        for kk, v in defaults.items():
            setattr(self.c, kk, v)
        if not self.c.regular_nu:
            self.nu0 = np.ascontiguousarray(nu0, dtype=np.float64)
            self.nuf = np.ascontiguousarray(nuf, dtype=np.float64)
            self.c.n_nu = len(self.nu0)
            self.c.nu_min = float(self.nu0[0])
            self.c.nu_max = float(self.nuf[-1])
        else:
            self.nu0 = np.zeros(1)
            self.nuf = np.zeros(1)
        self.d = Derived()
        k = np.ascontiguousarray(k, dtype=np.float64)
        pk = np.ascontiguousarray(pk, dtype=np.float64)
        self.logk = np.zeros_like(k)
        self.pk = np.zeros_like(pk)
        rc = lib().orc_cosmo_set(C.byref(self.c), len(k), k, pk, self.logk, self.pk, C.byref(self.d))
        if rc != 0:
            raise ValueError("orc_cosmo_set failed: %d" % rc)
        self.n = self.c.n_grid

    # ---- shapes
    def spec_shape(self):
        return (self.n, self.n, self.n // 2 + 1)

    def real_pad_shape(self):
        return (self.n, self.n, 2 * (self.n // 2 + 1))

    # ---- stages
    def modes_mt(self, nthreads=1, with_vpot=True):
        dk = np.zeros(self.spec_shape(), np.complex64)
        vk = np.zeros(self.spec_shape(), np.complex64) if with_vpot else None
        lib().orc_modes_mt(C.byref(self.c), C.byref(self.d), self.logk, self.pk, nthreads,
                           dk.view(np.float32), vk.view(np.float32).ctypes.data if with_vpot else None)
        return dk, vk

    def modes_philox(self):
        dk = np.zeros(self.spec_shape(), np.complex64)
        lib().orc_modes_philox(C.byref(self.c), C.byref(self.d), self.logk, self.pk, dk.view(np.float32))
        return dk

    def pk_grid(self):
        out = np.zeros((self.n,) * 3, np.float64)
        lib().orc_pk_grid(C.byref(self.c), C.byref(self.d), self.logk, self.pk, out.reshape(-1))
        return out

    def gaussianised_pk(self):
        """P_G on the grid, all in FP64: xi = sum_k P(k)/V e^{ikx}, xi_G = ln(1 + xi),
        P_G = V/N^3 sum_x xi_G e^{-ikx} (the periodic-box form of the lognormal
        Gaussianisation, e.g. Coles & Jones 1991; Agrawal et al. 2017, sec. 2)."""
        n, vol = self.n, self.d.l_box ** 3
        xi = np.fft.ifftn(self.pk_grid() / vol).real * n ** 3
        xg = np.log1p(np.maximum(xi, -1 + 1e-12))
        return np.ascontiguousarray(np.fft.fftn(xg).real * (vol / n ** 3))

    def modes_philox_gaussianised(self, pg=None):
        pg = self.gaussianised_pk() if pg is None else np.ascontiguousarray(pg, np.float64)
        dk = np.zeros(self.spec_shape(), np.complex64)
        lib().orc_modes_philox_pg(C.byref(self.c), C.byref(self.d), self.logk, self.pk, pg.reshape(-1),
                                  dk.view(np.float32))
        return dk

    # ---- point sources (src/psources.c, grid_tools.c:24-101, pixelize.c:58-148)
    def setup_psources(self):
        nz, mp, gdz = np.zeros(256), np.zeros(256), C.c_double()
        lib().orc_setup_psources(self.d.z_max, nz, mp, C.byref(gdz))
        return nz, mp, gdz.value

    def point_sources(self, dens_padded, sigma2, nthreads=1):
        nz, _, gdz = self.setup_psources()
        ns = np.zeros(self.real_pad_shape(), np.int32)
        tot = lib().orc_point_sources(C.byref(self.c), C.byref(self.d), nz, gdz,
                                      np.ascontiguousarray(dens_padded, np.float32).reshape(-1), sigma2, nthreads,
                                      ns.reshape(-1))
        if tot < 0:
            raise ValueError("a cell's Poisson mean exceeds the restated range (<= 10)")
        return ns

    def ps_lambda(self, dens_padded, sigma2):
        """Poisson mean of every cell, compact [z][y][x]."""
        nz, _, gdz = self.setup_psources()
        lam = np.zeros((self.n,) * 3)
        lib().orc_ps_lambda(C.byref(self.c), C.byref(self.d), nz, gdz,
                            np.ascontiguousarray(dens_padded, np.float32).reshape(-1), sigma2, lam.reshape(-1))
        return lam

    def psources_maps(self, nsources_padded, dz_padded, nthreads=1):
        nz, mp, gdz = self.setup_psources()
        npix = 12 * self.c.n_side ** 2
        maps = np.zeros((self.c.n_nu, npix), np.float32)
        lib().orc_psources_maps(C.byref(self.c), C.byref(self.d), self.nu0, self.nuf, nz, mp, gdz,
                                np.ascontiguousarray(nsources_padded, np.int32).reshape(-1),
                                np.ascontiguousarray(dz_padded, np.float32).reshape(-1), nthreads, maps.reshape(-1))
        return maps

    def psources_maps_catalogue(self, cells, u, L0, dz):
        """FP64 maps and pixels of a given source catalogue."""
        ns = len(cells)
        npix = 12 * self.c.n_side ** 2
        maps = np.zeros((self.c.n_nu, npix))
        pix = np.zeros(ns, np.int64)
        lib().orc_psources_maps_catalogue(C.byref(self.c), C.byref(self.d), self.nu0, self.nuf, ns,
                                          np.ascontiguousarray(cells, np.int64),
                                          np.ascontiguousarray(u, np.float64).reshape(-1),
                                          np.ascontiguousarray(L0, np.float64),
                                          np.ascontiguousarray(dz, np.float64), maps.reshape(-1), pix)
        return maps, pix

    def c2r(self, spec):
        """In-place padded c2r of a half spectrum, float32 result (FFTW layout)."""
        buf = np.ascontiguousarray(spec, np.complex64).copy()
        flat = buf.view(np.float32).reshape(self.real_pad_shape())
        lib().orc_c2r_inplace(self.n, flat.reshape(-1))
        return flat

    def c2r_double(self, spec):
        out = np.zeros((self.n, self.n, self.n), np.float64)
        lib().orc_c2r_to_double(self.n, np.ascontiguousarray(spec, np.complex64).view(np.float32).reshape(-1),
                                out.reshape(-1))
        return out

    def normalize(self, grid):
        lib().orc_normalize(self.n, self.d.l_box, grid.reshape(-1))
        return grid

    def radial_velocity_fd(self, vpot_real):
        rv = np.zeros(self.real_pad_shape(), np.float32)
        lib().orc_radial_velocity_fd(C.byref(self.c), C.byref(self.d),
                                     np.ascontiguousarray(vpot_real, np.float32).reshape(-1), rv.reshape(-1))
        return rv

    def radial_velocity_spectral(self, dens_k):
        rv = np.zeros(self.real_pad_shape(), np.float32)
        lib().orc_radial_velocity_spectral(C.byref(self.c), C.byref(self.d),
                                           np.ascontiguousarray(dens_k, np.complex64).view(np.float32).reshape(-1),
                                           rv.reshape(-1))
        return rv

    def sigma(self, dens):
        m, s = C.c_double(), C.c_double()
        lib().orc_sigma_dens(self.n, np.ascontiguousarray(dens, np.float32).reshape(-1), C.byref(m), C.byref(s))
        return m.value, s.value

    def get_hi(self, dens, rvel, sigma2):
        d = np.ascontiguousarray(dens, np.float32).copy()
        r = np.ascontiguousarray(rvel, np.float32).copy()
        lib().orc_get_hi(C.byref(self.c), C.byref(self.d), sigma2, d.reshape(-1), r.reshape(-1))
        return d, r

    def subsample_offsets(self):
        xs, ys, zs = np.zeros(10), np.zeros(10), np.zeros(10)
        lib().orc_subsample_offsets(self.c.seed, self.d.l_box / self.n, xs, ys, zs)
        return xs, ys, zs

    def mk_T_maps(self, mass, dz, want_keys=False):
        npix = 12 * self.c.n_side ** 2
        maps = np.zeros((self.c.n_nu, npix), np.float32)
        keys = np.zeros(self.n ** 3 * 10, np.uint32) if want_keys else None
        lib().orc_mk_T_maps(C.byref(self.c), C.byref(self.d), self.nu0, self.nuf,
                            np.ascontiguousarray(mass, np.float32).reshape(-1),
                            np.ascontiguousarray(dz, np.float32).reshape(-1), maps.reshape(-1),
                            keys.ctypes.data if want_keys else None)
        return (maps, keys) if want_keys else maps

    def prefactors(self):
        out = np.zeros(self.c.n_nu)
        lib().orc_channel_prefactors(C.byref(self.c), C.byref(self.d), self.nu0, self.nuf, out)
        return out

    def tables(self):
        d = self.d
        return np.concatenate([np.ctypeslib.as_array(getattr(d, n)) for n in
                               ("z_z2r", "r_z2r", "z_r2z", "r_r2z", "gd", "gv")])


def vec2pix_ring(nside, v):
    return lib().orc_vec2pix_ring(nside, np.ascontiguousarray(v, np.float64))


def pix2ang_ring(nside, ipix):
    th, ph = C.c_double(), C.c_double()
    lib().orc_pix2ang_ring(nside, ipix, C.byref(th), C.byref(ph))
    return th.value, ph.value


def philox(ctr, key):
    out = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(np.asarray(ctr, np.uint32), np.asarray(key, np.uint32), out)
    return out


def set_threads(t):
    lib().orc_set_threads(int(t))


def load_pk(path):
    a = np.loadtxt(path)
    return a[:, 0], a[:, 1]


# ---------------------------------------------------------------------------
# JoinT (src/main_jt.c:98-372; src/healpix_extra.c:31-43, 318-421)
# ---------------------------------------------------------------------------
PREFAC_FWHM = 1030610.55  # src/main_jt.c:26, arcmin for nu in MHz and the dish in m
PREFAC_TNU = 3.6e9        # src/main_jt.c:25


def nest2ring(nside, ipnest):
    return lib().orc_nest2ring(nside, int(ipnest))


def ring2nest(nside, ipring):
    return lib().orc_ring2nest(nside, int(ipring))


def ring_info(nside, ring):
    a, b = C.c_long(), C.c_long()
    z, s, p = C.c_double(), C.c_double(), C.c_double()
    lib().orc_ring_info(nside, ring, C.byref(a), C.byref(b), C.byref(z), C.byref(s), C.byref(p))
    return a.value, b.value, z.value, s.value, p.value


def nalms(lmax):
    return (lmax + 1) * (lmax + 2) // 2


def map2alm(nside, lmax, m):
    """HEALPix a_lm (m-major triangular, complex128) of one FP64 map"""
    out = np.zeros(2 * nalms(lmax))
    lib().orc_map2alm(nside, lmax, np.ascontiguousarray(m, np.float64), out)
    return out.view(np.complex128)


def alm2map(nside, lmax, alm):
    out = np.zeros(12 * nside * nside)
    lib().orc_alm2map(nside, lmax, np.ascontiguousarray(np.asarray(alm, np.complex128).view(np.float64)), out)
    return out


def udgrade(map_in, nside_in, nside_out):
    out = np.zeros(12 * nside_out * nside_out, np.float32)
    lib().orc_udgrade(np.ascontiguousarray(map_in, np.float32), nside_in, out, nside_out)
    return out


def beam_window(lmax, fwhm_amin):
    out = np.zeros(lmax + 1)
    lib().orc_beam_window(lmax, fwhm_amin, out)
    return out


def joint_fwhm(nu0, nuf, dish):
    """per channel FWHM in arcmin at the channel centre (src/main_jt.c:224-226)"""
    return PREFAC_FWHM / (0.5 * (np.asarray(nu0) + np.asarray(nuf)) * dish)


def apply_beam(maps, nside, fwhm_amin):
    out = np.ascontiguousarray(maps, np.float32).copy()
    lib().orc_apply_beam(nside, out.shape[0], np.ascontiguousarray(fwhm_amin, np.float64), out)
    return out


def add_noise(maps, nside, nu0, nuf, fsky, tsys, time_tot, n_dish, seed, nthreads=1):
    out = np.ascontiguousarray(maps, np.float32).copy()
    lib().orc_add_noise(nside, out.shape[0], np.ascontiguousarray(nu0, np.float64),
                        np.ascontiguousarray(nuf, np.float64), fsky, tsys, time_tot, n_dish, seed, nthreads, out)
    return out


def joint(components, nside_in, nside, nu0, nuf, dish=-1.0, n_dish=1, tsys=-1.0, time_tot=1.0, seed=1,
          mask=None, nthreads=1):
    """The JoinT pipeline: merge_maps (src/main_jt.c:98-200, float sums in the
    component order, then he_udgrade), apply_beam when dish > 0, add_noise when
    tsys > 0, apply_mask.  components: [(maps [n_nu][12 nside_in^2], factor or
    None)], the factor (polarisation leakage) applied as float * double -> float."""
    n_nu = len(nu0)
    acc = np.zeros((n_nu, 12 * nside_in * nside_in), np.float32)
    for maps, fac in components:
        m = np.asarray(maps, np.float32)
        if fac is not None:
            m = (m.astype(np.float64) * fac).astype(np.float32)
        acc = acc + m
    out = np.stack([udgrade(acc[i], nside_in, nside) for i in range(n_nu)])
    if dish > 0:
        out = apply_beam(out, nside, joint_fwhm(nu0, nuf, dish))
    npix = 12 * nside * nside
    fsky = 1.0 if mask is None else float(np.count_nonzero(mask)) / npix
    if tsys > 0:
        out = add_noise(out, nside, nu0, nuf, fsky, tsys, time_tot, n_dish, seed, nthreads)
    if mask is not None:
        out[:, np.asarray(mask) == 0] = 0
    return out


def joint_instrument(nside, nu0, nuf, dish, n_dish, tsys, time_tot, fsky):
    """Rows of <prefix_out>_instrument.dat (src/main_jt.c:28-72): nu, FWHM in
    degrees, noise rms per pointing, noise rms per pixel."""
    rows = []
    npix = 12 * nside * nside
    for a, b in zip(nu0, nuf):
        nu, dnu = 0.5 * (a + b), b - a
        n_pix = fsky * npix
        if dish > 0:
            fwhm_rad = PREFAC_FWHM / (nu * dish) * np.pi / (180 * 60)
            n_point = fsky * 4 * np.pi / (1.1330900354567985 * fwhm_rad * fwhm_rad)
        else:
            fwhm_rad, n_point = 0.0, fsky * npix
        if tsys > 0:
            s2p = n_point * tsys * tsys / (PREFAC_TNU * dnu * time_tot * n_dish)
            s2x = n_pix * tsys * tsys / (PREFAC_TNU * dnu * time_tot * n_dish)
        else:
            s2p = s2x = 0.0
        rows.append((nu, 180 * fwhm_rad / np.pi, np.sqrt(s2p), np.sqrt(s2x)))
    return np.array(rows)
