"""Host-side mirror of GetHI's stage interface over the GB300 C ABI.

The reference drives one realisation as (src/main_gh.c:34-74)

    par = read_run_params(fname)      # src/io_gh.c:188
    create_d_and_vr_fields(par)       # src/fourier.c:375
    get_HI(par)                       # src/grid_tools.c:103
    mk_T_maps(par)                    # src/pixelize.c:150
    write_maps(par)                   # src/io_gh.c:109
    param_gethi_free(par)             # src/io_gh.c:298

and this module keeps those names on a ``GetHI`` object whose work runs in
libgethi_gpu.so (include/gethi_gpu.h).  There is no CPU fallback: without the
built library every call raises.
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libgethi_gpu.so")
NZ = 5001

GETHI_ERRORS = {-1: "GETHI_E_ARG", -2: "GETHI_E_IO", -3: "GETHI_E_COSMO", -4: "GETHI_E_CUDA",
                -5: "GETHI_E_NOMEM", -6: "GETHI_E_STATE", -7: "GETHI_E_DEVICE"}


class GetHIError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (GETHI_ERRORS.get(code, "?"), code, msg))
        self.code = code


class Params(C.Structure):
    """gethi_params of include/gethi_gpu.h (the .ini keys of src/io_gh.c:211-249 + new keys)."""
    _fields_ = [("prefix_out", C.c_char * 256), ("pk_filename", C.c_char * 256),
                ("frequencies_filename", C.c_char * 256)] + \
        [(n, C.c_double) for n in ("omega_M", "omega_L", "omega_B", "h", "w", "ns", "sigma_8", "r_smooth",
                                   "nu_min", "nu_max")] + \
        [("n_nu", C.c_int), ("n_grid", C.c_int), ("n_side", C.c_long), ("seed", C.c_uint),
         ("do_psources", C.c_int), ("l_box", C.c_double), ("bias_model", C.c_int), ("b_HI", C.c_double)] + \
        [(n, C.c_int) for n in ("do_rsd", "velocity_mode", "gaussianise", "fft_precision", "rng",
                                "omp_threads_for_modes", "write_maps")]


class Derived(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("fgrowth_0", "hubble_0", "z_min", "z_max", "r_min", "r_max", "l_box",
                                          "pos_obs", "r2_smooth", "glob_idr", "logkmin", "logkmax", "idlogk",
                                          "pk_norm", "sigma8_in", "sigma2_gauss", "mean_gauss")] + \
        [(n, C.c_int) for n in ("do_smoothing", "numk", "n_nu", "regular_nu")] + [("filled_fraction", C.c_double)]


_CHOICES = {"bias_model": ("fit", "const"), "velocity_mode": ("fd", "spectral"),
            "fft_precision": ("fp32", "tc_split"), "rng": ("philox", "mt_validation")}

_lib = None


def lib():
    """Load libgethi_gpu.so (raises if it was not built: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libgethi_gpu.so is not built (%s); run `python -m crime_gb300.build`" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        vp = C.c_void_p
        L.gethi_params_default.argtypes = [P(Params)]
        L.gethi_read_params.argtypes = [C.c_char_p, P(Params)]
        L.gethi_host_setup.argtypes = [P(Params), P(Derived), vp, vp, vp, vp, vp]
        L.gethi_host_modes_mt.argtypes = [P(Params), C.c_int, vp]
        L.gethi_gpu_init.argtypes = [P(Params), C.c_int, P(vp)]
        L.gethi_gpu_free.argtypes = [vp]
        L.gethi_gpu_free.restype = None
        L.gethi_gpu_set_stream.argtypes = [vp, vp]
        L.gethi_gpu_get_derived.argtypes = [vp, P(Derived)]
        L.gethi_last_error.restype = C.c_char_p
        L.gethi_gpu_make_fields.argtypes = [vp, vp]
        L.gethi_gpu_get_hi.argtypes = [vp]
        L.gethi_gpu_make_maps.argtypes = [vp, vp]
        L.gethi_gpu_write_maps.argtypes = [vp, vp]
        L.gethi_gpu_run.argtypes = [vp, vp]
        L.gethi_gpu_download_grids.argtypes = [vp, vp, vp]
        L.gethi_gpu_upload_grids.argtypes = [vp, vp, vp, C.c_int]
        L.gethi_gpu_sample_keys.argtypes = [vp, vp, C.c_int]
        L.gethi_gpu_download_modes.argtypes = [vp, vp]
        L.gethi_gpu_stage_times.argtypes = [vp, vp, C.c_int]
        L.gethi_gpu_profile.argtypes = [vp, C.c_int]
        L.gethi_gpu_set_seed.argtypes = [vp, C.c_uint]
        L.gethi_gpu_upload_inputs.argtypes = [vp]
        L.gethi_gpu_upload_inputs.restype = C.c_long
        L.gethi_gpu_kernel_times.argtypes = [vp, vp, vp, vp]
        L.gethi_gpu_fallback_count.argtypes = [vp, vp]
        L.gethi_gpu_wait_selftest.argtypes = [vp, C.c_long]
        L.gethi_gpu_run_batch.argtypes = [vp, C.c_int, vp, vp, C.c_int, vp, C.c_int, vp]
        L.gethi_gpu_autotune.argtypes = [vp, vp, vp]
        L.gethi_gpu_set_launch.argtypes = [vp, C.c_int, C.c_int]
        L.gethi_gpu_run_async.argtypes = [vp, vp]
        L.gethi_gpu_wait.argtypes = [vp]
        L.gethi_gpu_psources_maps.argtypes = [vp, vp, vp]
        L.gethi_gpu_psources_catalogue.argtypes = [vp, C.c_long, vp, vp, vp, vp, vp]
        L.gethi_host_psources.argtypes = [P(Params), vp, vp, vp, vp]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise GetHIError(rc, lib().gethi_last_error().decode(errors="replace"))
    return rc


def _ptr(a):
    return None if a is None else a.ctypes.data


def default_params():
    p = Params()
    _check(lib().gethi_params_default(C.byref(p)))
    return p


def make_params(**kw):
    """Reference defaults (src/io_gh.c:133-186) overridden by keyword arguments
    named like the .ini keys (n_grid=..., omega_M=..., velocity_mode="spectral")."""
    p = default_params()
    for k, v in kw.items():
        if k in _CHOICES and isinstance(v, str):
            v = _CHOICES[k].index(v)
        if isinstance(getattr(p, k), bytes):
            v = str(v).encode()
        setattr(p, k, v)
    return p


def read_params(fname):
    p = Params()
    _check(lib().gethi_read_params(os.fsencode(fname), C.byref(p)))
    return p


def host_setup(p):
    """FP64 host setup without a GPU: derived values, tables, P(k), offsets, prefactors."""
    d = Derived()
    _check(lib().gethi_host_setup(C.byref(p), C.byref(d), None, None, None, None, None))
    tables = np.zeros(6 * NZ)
    logk, pk = np.zeros(d.numk), np.zeros(d.numk)
    offs, pref = np.zeros(30), np.zeros(d.n_nu)
    _check(lib().gethi_host_setup(C.byref(p), C.byref(d), _ptr(tables), _ptr(logk), _ptr(pk), _ptr(offs),
                                  _ptr(pref)))
    return dict(derived=d, tables=tables, logk=logk, pk=pk, offsets=offs.reshape(10, 3), prefac=pref)


def host_psources(p):
    """Point-source tables of the host setup: n(z), rejection bounds, glob_dz, log10 L inverse CDF."""
    nz, mp, icdf = np.zeros(256), np.zeros(256), np.zeros(4097)
    gdz = np.zeros(1)
    _check(lib().gethi_host_psources(C.byref(p), _ptr(nz), _ptr(mp), _ptr(gdz), _ptr(icdf)))
    return dict(nz=nz, maxpdf=mp, glob_dz=float(gdz[0]), icdf=icdf)


def host_modes_mt(p, nthreads=1):
    n = p.n_grid
    out = np.zeros((n, n, n // 2 + 1), np.complex64)
    _check(lib().gethi_host_modes_mt(C.byref(p), int(nthreads), out.ctypes.data))
    return out


class GetHI:
    """One GetHI configuration on one GPU (the ParamGetHI of src/common_gh.h:58-129)."""

    def __init__(self, params, device=0):
        self.params = params
        self._ctx = C.c_void_p()
        _check(lib().gethi_gpu_init(C.byref(params), int(device), C.byref(self._ctx)))
        self.n = params.n_grid
        self.npix = 12 * params.n_side ** 2
        self.n_nu = self.derived().n_nu

    # -- lifecycle
    def free(self):
        if self._ctx:
            lib().gethi_gpu_free(self._ctx)
            self._ctx = C.c_void_p()

    param_gethi_free = free

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def set_stream(self, stream_handle):
        _check(lib().gethi_gpu_set_stream(self._ctx, C.c_void_p(stream_handle)))

    def derived(self):
        d = Derived()
        _check(lib().gethi_gpu_get_derived(self._ctx, C.byref(d)))
        return d

    # -- stages, named as in the reference
    def create_d_and_vr_fields(self, modes_k=None):
        m = None if modes_k is None else np.ascontiguousarray(modes_k, np.complex64)
        _check(lib().gethi_gpu_make_fields(self._ctx, _ptr(m)))

    def get_HI(self):
        _check(lib().gethi_gpu_get_hi(self._ctx))

    def mk_T_maps(self, download=True):
        maps = np.zeros((self.n_nu, self.npix), np.float32) if download else None
        _check(lib().gethi_gpu_make_maps(self._ctx, _ptr(maps)))
        return maps

    def write_maps(self, maps):
        _check(lib().gethi_gpu_write_maps(self._ctx, _ptr(np.ascontiguousarray(maps, np.float32))))

    def run(self, maps=None):
        """All stages, get_HI fused into the projection. Returns the maps (host)."""
        if maps is None:
            maps = np.zeros((self.n_nu, self.npix), np.float32)
        _check(lib().gethi_gpu_run(self._ctx, _ptr(maps)))
        return maps

    def set_seed(self, seed):
        _check(lib().gethi_gpu_set_seed(self._ctx, int(seed) & 0xFFFFFFFF))

    def upload_inputs(self):
        r = lib().gethi_gpu_upload_inputs(self._ctx)
        if r < 0:
            _check(int(r))
        return int(r)

    def run_async(self, maps_ptr=None):
        """Enqueue a realisation and the copy of its maps to maps_ptr (an address of
        page-locked host or device memory); returns at once (see gethi_gpu_run_async)."""
        _check(lib().gethi_gpu_run_async(self._ctx, C.c_void_p(maps_ptr) if maps_ptr else None))

    def wait(self):
        _check(lib().gethi_gpu_wait(self._ctx))

    def run_into(self, maps_ptr):
        """All stages into an existing host buffer given as an address (pinned memory)."""
        _check(lib().gethi_gpu_run(self._ctx, C.c_void_p(maps_ptr)))

    # -- inspection
    def grids(self):
        n = self.n
        d = np.zeros((n, n, n), np.float32)
        v = np.zeros((n, n, n), np.float32)
        _check(lib().gethi_gpu_download_grids(self._ctx, _ptr(d), _ptr(v)))
        return d, v

    def upload_grids(self, dens, rvel, stage):
        n = self.n
        d = np.ascontiguousarray(dens, np.float32).reshape(n, n, n)
        v = np.ascontiguousarray(rvel, np.float32).reshape(n, n, n)
        _check(lib().gethi_gpu_upload_grids(self._ctx, _ptr(d), _ptr(v), int(stage)))

    def sample_keys(self, exact=True):
        keys = np.zeros(self.n ** 3 * 10, np.uint32)
        _check(lib().gethi_gpu_sample_keys(self._ctx, _ptr(keys), int(bool(exact))))
        return keys

    def device_modes(self):
        n = self.n
        out = np.zeros((n, n, n // 2 + 1), np.complex64)
        _check(lib().gethi_gpu_download_modes(self._ctx, _ptr(out)))
        return out

    KERNEL_CLASSES = ("zpass", "ypass", "xpass", "xpass_vel", "nyq", "sigma", "fd_vel", "get_hi", "project",
                      "scale", "zpass_raw", "fixup", "psources")

    # -- point sources (do_psources=1)
    def psources_maps(self):
        """Point-source maps [n_nu, 12 n_side^2] (mK) and the number of sources."""
        maps = np.zeros((self.n_nu, self.npix), np.float32)
        ns = np.zeros(1, np.int64)
        _check(lib().gethi_gpu_psources_maps(self._ctx, _ptr(maps), _ptr(ns)))
        return maps, int(ns[0])

    def psources_catalogue(self, cap=1 << 22):
        """The sources of the current fields: cell index, (ux, uy, uz), L0 [1e22 W/Hz], dz_rsd, pixel."""
        cell = np.zeros(cap, np.int64)
        ul = np.zeros((cap, 4), np.float32)
        dz = np.zeros(cap, np.float32)
        pix = np.zeros(cap, np.int32)
        cnt = np.zeros(1, np.int64)
        _check(lib().gethi_gpu_psources_catalogue(self._ctx, cap, _ptr(cell), _ptr(ul), _ptr(dz), _ptr(pix),
                                                  _ptr(cnt)))
        k = min(int(cnt[0]), cap)
        return dict(cell=cell[:k], u=ul[:k, :3], L0=ul[:k, 3], dz=dz[:k], pix=pix[:k], count=int(cnt[0]))

    def profile(self, on=True):
        _check(lib().gethi_gpu_profile(self._ctx, int(on)))

    def kernel_times(self):
        ms = np.zeros(len(self.KERNEL_CLASSES))
        cnt = np.zeros(len(self.KERNEL_CLASSES), np.int64)
        launches = np.zeros(1, np.int64)
        lib().gethi_gpu_kernel_times(self._ctx, _ptr(ms), _ptr(cnt), _ptr(launches))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.KERNEL_CLASSES)}, int(launches[0])

    def wait_selftest(self, limit_us=20000):
        """Run the bounded-wait expiry path once (gethi_gpu_wait_selftest); returns its status code."""
        return lib().gethi_gpu_wait_selftest(self._ctx, int(limit_us))

    def fallback_count(self):
        v = np.zeros(1, np.int64)
        _check(lib().gethi_gpu_fallback_count(self._ctx, _ptr(v)))
        return int(v[0])

    def set_launch(self, proj_zsteps=0, col_variant=0):
        """Launch shapes by hand (gethi_gpu_set_launch)."""
        _check(lib().gethi_gpu_set_launch(self._ctx, int(proj_zsteps), int(col_variant)))

    def autotune(self):
        """Pick the fastest projection tile depth / column tile width for this
        configuration (kept for the context's later work)."""
        ch = np.zeros(2, np.int32)
        ms = np.zeros(1, np.float32)
        _check(lib().gethi_gpu_autotune(self._ctx, _ptr(ch), _ptr(ms)))
        return {"tile_depth": 4 * int(ch[0]), "column_variant": int(ch[1]), "ms_per_realisation": float(ms[0])}

    def stage_times(self):
        ms = np.zeros(8, np.float32)
        k = lib().gethi_gpu_stage_times(self._ctx, _ptr(ms), 8)
        return ms[:max(k, 0)]


def run_batch(contexts, jobs, download=True, graph=True):
    """A batch of Philox realisations: jobs = [(context index, seed), ...].  Jobs of
    one context run in order, contexts run concurrently; graph=True captures the
    whole batch into one CUDA graph.  Returns (maps per job or None, stats dict)."""
    nctx = len(contexts)
    ctx_arr = (C.c_void_p * nctx)(*[c._ctx.value for c in contexts])
    job_ctx = np.ascontiguousarray([j[0] for j in jobs], np.int32)
    seeds = np.ascontiguousarray([j[1] & 0xFFFFFFFF for j in jobs], np.uint32)
    maps = None
    ptrs = None
    if download:
        sizes = [contexts[j[0]].n_nu * contexts[j[0]].npix for j in jobs]
        buf = np.empty(sum(sizes), np.float32)
        offs = np.concatenate([[0], np.cumsum(sizes)])
        maps = [buf[offs[i]:offs[i + 1]].reshape(contexts[j[0]].n_nu, contexts[j[0]].npix)
                for i, j in enumerate(jobs)]
        ptrs = (C.c_void_p * len(jobs))(*[m.ctypes.data for m in maps])
    st = np.zeros(4)
    _check(lib().gethi_gpu_run_batch(ctx_arr, nctx, _ptr(job_ctx), _ptr(seeds), len(jobs), ptrs, int(bool(graph)),
                                     _ptr(st)))
    return maps, {"capture_ms": float(st[0]), "device_ms": float(st[1]), "graph_nodes": int(st[2]),
                  "kernel_launches": int(st[3])}


def read_run_params(fname, device=0):
    """src/io_gh.c:188: parse the .ini and set the run up (on the GPU)."""
    return GetHI(read_params(fname), device)
