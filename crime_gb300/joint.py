"""Host-side mirror of JoinT's stage interface over the GB300 C ABI.

The reference combines the per-channel maps as (src/main_jt.c:326-389)

    pars = read_input_params_JoinT(fname)  # src/io_jt.c:86
    merge_maps(pars, maps_out)             # src/main_jt.c:98 (sum + he_udgrade)
    apply_beam(pars, maps_out)             # src/main_jt.c:202 (dish_diameter > 0)
    add_noise(pars, maps_out)              # src/main_jt.c:263 (t_system > 0)
    apply_mask(pars, maps_out)             # src/main_jt.c:240
    write_maps(...); write_arrays(pars)    # src/io_jt.c:25, src/main_jt.c:28

and this module keeps those names on a ``JoinT`` object whose work runs in
libgethi_gpu.so (include/joint_gpu.h).  There is no CPU fallback.

    python -m crime_gb300.joint param_JoinT.ini     # the command-line drop-in
"""
import ctypes as C
import os
import sys

import numpy as np

from .gethi import _check, _ptr, lib as _gethi_lib

RNG = {"philox": 0, "mt_validation": 1}


class JointParams(C.Structure):
    """joint_params of include/joint_gpu.h"""
    _fields_ = [("nside", C.c_int), ("n_nu", C.c_int), ("nu0", C.c_void_p), ("nuf", C.c_void_p),
                ("seed", C.c_uint), ("dish_diameter", C.c_double), ("n_dish", C.c_int), ("tsys", C.c_double),
                ("time_tot", C.c_double), ("mask", C.c_void_p), ("rng", C.c_int),
                ("omp_threads_for_noise", C.c_int), ("sht_chunk", C.c_int), ("sht_precision", C.c_int)]


_bound = False


def lib():
    global _bound
    L = _gethi_lib()
    if not _bound:
        vp = C.c_void_p
        L.joint_gpu_init.argtypes = [C.POINTER(JointParams), C.c_int, C.POINTER(vp)]
        L.joint_gpu_free.argtypes = [vp]
        L.joint_gpu_free.restype = None
        L.joint_gpu_set_stream.argtypes = [vp, vp]
        L.joint_gpu_add_maps.argtypes = [vp, vp, C.c_long, C.c_double]
        L.joint_gpu_add_maps_device.argtypes = [vp, vp, C.c_long, C.c_double]
        for fn in ("joint_gpu_merge", "joint_gpu_apply_beam", "joint_gpu_add_noise", "joint_gpu_apply_mask"):
            getattr(L, fn).argtypes = [vp]
        L.joint_gpu_get_maps.argtypes = [vp, vp]
        L.joint_gpu_device_maps.argtypes = [vp, C.POINTER(vp)]
        L.joint_gpu_run.argtypes = [vp, vp]
        L.joint_gpu_fsky.argtypes = [vp]
        L.joint_gpu_fsky.restype = C.c_double
        L.joint_gpu_map2alm.argtypes = [vp, vp, C.c_int, vp]
        L.joint_gpu_alm2map.argtypes = [vp, vp, C.c_int, vp]
        L.joint_gpu_stage_times.argtypes = [vp, vp]
        L.joint_gpu_profile.argtypes = [vp, C.c_int]
        L.joint_gpu_uses_tensor_cores.argtypes = [vp]
        L.joint_gpu_kernel_times.argtypes = [vp, vp, vp]
        L.joint_host_read_map.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_long), vp]
        L.joint_host_read_nutable.argtypes = [C.c_char_p, C.POINTER(C.c_int), vp, vp]
        L.joint_host_write_maps.argtypes = [C.c_char_p, C.c_long, C.c_int, vp]
        L.joint_host_write_instrument.argtypes = [C.c_char_p, C.POINTER(JointParams), C.c_double]
        L.joint_host_run.argtypes = [C.c_char_p, C.c_int]
        L.gethi_gpu_device_maps.argtypes = [vp, C.POINTER(vp), C.POINTER(vp)]
        _bound = True
    return L


def nalms(lmax):
    return (lmax + 1) * (lmax + 2) // 2


def read_map(path, column=0):
    """one column of a HEALPix FITS map in RING order (src/healpix_extra.c:166-224)"""
    ns = C.c_long()
    _check(lib().joint_host_read_map(os.fsencode(path), column, C.byref(ns), None))
    out = np.empty(12 * ns.value * ns.value, np.float32)
    _check(lib().joint_host_read_map(os.fsencode(path), column, C.byref(ns), out.ctypes.data))
    return out, ns.value


def read_nutable(path):
    """(nu0, nuf) of a frequency table (src/io_jt.c:215-241)"""
    n = C.c_int()
    _check(lib().joint_host_read_nutable(os.fsencode(path), C.byref(n), None, None))
    nu0, nuf = np.empty(n.value), np.empty(n.value)
    _check(lib().joint_host_read_nutable(os.fsencode(path), C.byref(n), nu0.ctypes.data, nuf.ctypes.data))
    return nu0, nuf


def run_ini(path, device=0):
    """The whole JoinT run of a param_JoinT .ini (src/main_jt.c:326-389)"""
    _check(lib().joint_host_run(os.fsencode(path), device))


class JoinT:
    """One JoinT configuration on one GPU (include/joint_gpu.h)."""

    def __init__(self, nside, nu0, nuf, seed=1, dish_diameter=-1.0, n_dish=1, tsys=-1.0, time_tot=1.0, mask=None,
                 rng="philox", omp_threads_for_noise=1, sht_chunk=0, sht_precision="auto", device=0):
        self.nu0 = np.ascontiguousarray(nu0, np.float64)
        self.nuf = np.ascontiguousarray(nuf, np.float64)
        self.mask = None if mask is None else np.ascontiguousarray(mask, np.int32)
        p = JointParams(nside=nside, n_nu=len(self.nu0), nu0=self.nu0.ctypes.data, nuf=self.nuf.ctypes.data,
                        seed=seed, dish_diameter=dish_diameter, n_dish=n_dish, tsys=tsys, time_tot=time_tot,
                        mask=None if self.mask is None else self.mask.ctypes.data,
                        rng=RNG[rng] if isinstance(rng, str) else rng, omp_threads_for_noise=omp_threads_for_noise,
                        sht_chunk=sht_chunk,
                        sht_precision={"auto": 0, "fp32": 1}[sht_precision] if isinstance(sht_precision, str)
                        else sht_precision)
        self.params = p
        self.nside, self.n_nu = nside, len(self.nu0)
        self.npix = 12 * nside * nside
        self.lmax = 3 * nside - 1
        self._ctx = C.c_void_p()
        _check(lib().joint_gpu_init(C.byref(p), device, C.byref(self._ctx)))

    def close(self):
        if self._ctx:
            lib().joint_gpu_free(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def uses_tensor_cores(self):
        return bool(lib().joint_gpu_uses_tensor_cores(self._ctx))

    @property
    def fsky(self):
        return lib().joint_gpu_fsky(self._ctx)

    # merge_maps (src/main_jt.c:98-200)
    def add_maps(self, maps, nside_in, factor=1.0):
        m = np.ascontiguousarray(maps, np.float32)
        assert m.size == self.n_nu * 12 * nside_in * nside_in
        _check(lib().joint_gpu_add_maps(self._ctx, m.ctypes.data, nside_in, factor))

    def add_maps_device(self, dev_ptr, nside_in, factor=1.0):
        _check(lib().joint_gpu_add_maps_device(self._ctx, C.c_void_p(dev_ptr), nside_in, factor))

    def add_gethi(self, gh, factor=1.0, point_sources=False):
        """the maps a GetHI context left on the device (no host round trip)"""
        m, ps = C.c_void_p(), C.c_void_p()
        _check(lib().gethi_gpu_device_maps(gh._ctx, C.byref(m), C.byref(ps)))
        ptr = ps if point_sources else m
        if not ptr.value:
            raise ValueError("the GetHI context has no such maps")
        self.add_maps_device(ptr.value, int(gh.params.n_side), factor)

    def merge_maps(self):
        _check(lib().joint_gpu_merge(self._ctx))

    def apply_beam(self):
        _check(lib().joint_gpu_apply_beam(self._ctx))

    def add_noise(self):
        _check(lib().joint_gpu_add_noise(self._ctx))

    def apply_mask(self):
        _check(lib().joint_gpu_apply_mask(self._ctx))

    def maps(self):
        out = np.empty((self.n_nu, self.npix), np.float32)
        _check(lib().joint_gpu_get_maps(self._ctx, out.ctypes.data))
        return out

    def run(self, copy_out=True):
        out = np.empty((self.n_nu, self.npix), np.float32) if copy_out else None
        _check(lib().joint_gpu_run(self._ctx, _ptr(out)))
        return out

    def stage_times(self):
        """device ms of the last run: merge, beam, noise, mask"""
        t = np.zeros(4, np.float32)
        _check(lib().joint_gpu_stage_times(self._ctx, t.ctypes.data))
        return dict(zip(("merge", "beam", "noise", "mask"), t.tolist()))

    BEAM_KERNELS = ("ring_analysis", "legendre_analysis", "legendre_synthesis", "ring_synthesis", "legendre_pack")

    def profile(self, on=True):
        _check(lib().joint_gpu_profile(self._ctx, 1 if on else 0))

    def kernel_times(self):
        """{class: (device ms, launches)} of the beam while profiling"""
        ms, n = np.zeros(5), np.zeros(5, np.int64)
        _check(lib().joint_gpu_kernel_times(self._ctx, ms.ctypes.data, n.ctypes.data))
        return {k: (float(a), int(b)) for k, a, b in zip(self.BEAM_KERNELS, ms, n)}

    # he_map2alm / he_alm2map (src/healpix_extra.c:44-130)
    def map2alm(self, maps):
        m = np.ascontiguousarray(np.atleast_2d(maps), np.float32)
        out = np.empty((m.shape[0], nalms(self.lmax)), np.complex64)
        _check(lib().joint_gpu_map2alm(self._ctx, m.ctypes.data, m.shape[0], out.ctypes.data))
        return out

    def alm2map(self, alms):
        a = np.ascontiguousarray(np.atleast_2d(alms), np.complex64)
        out = np.empty((a.shape[0], self.npix), np.float32)
        _check(lib().joint_gpu_alm2map(self._ctx, a.ctypes.data, a.shape[0], out.ctypes.data))
        return out

    def write_maps(self, prefix, maps):
        m = np.ascontiguousarray(maps, np.float32)
        _check(lib().joint_host_write_maps(os.fsencode(prefix), self.nside, self.n_nu, m.ctypes.data))

    def write_arrays(self, prefix):
        _check(lib().joint_host_write_instrument(os.fsencode(prefix), C.byref(self.params), self.fsky))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("Usage: python -m crime_gb300.joint file_name")
    run_ini(sys.argv[1])
