"""gethi_project_noalloc: the projection entry point that allocates no device
memory, for callers that own all device memory themselves and cannot let a
library call cudaMalloc.  Called through the C ABI with caller-owned device
grids and maps, twice in a row, and compared with the maps of the allocating
entry point (gethi_gpu_make_maps) on the same grids.  Collected last on
purpose: the arrays it uses are shared by all calls in the process."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


COSMO = dict(omega_M=0.315, omega_L=0.685, omega_B=0.049, h=0.67, w=-1.0, ns=0.96, sigma_8=0.83,
             pk_filename=os.path.join(GOLDEN, "pk_eh_nowiggle.txt"))


def _setup(p):
    """gethi_host_setup outputs the entry point takes (derived values, tables, offsets, prefactors)."""
    from crime_gb300.gethi import Derived, lib
    L = lib()
    d = Derived()
    assert L.gethi_host_setup(C.byref(p), C.byref(d), None, None, None, None, None) == 0
    tables, offsets, prefac = np.zeros(6 * 5001), np.zeros(30), np.zeros(d.n_nu)
    assert L.gethi_host_setup(C.byref(p), C.byref(d), tables.ctypes.data, None, None, offsets.ctypes.data,
                              prefac.ctypes.data) == 0
    return d, tables, offsets, prefac


def _compare(torch, gh, p, edges, mass, dz, calls=2):
    """Maps of the allocating entry point (gethi_gpu_make_maps on an uploaded
    context) against `calls` calls in a row of gethi_project_noalloc on
    caller-owned device arrays.  Returns the allocating path's count of
    samples whose FP32 key was uncertain."""
    from crime_gb300.gethi import Derived, lib
    L = lib()
    d, tables, offsets, prefac = _setup(p)
    ctx = gh.GetHI(p)
    ctx.upload_grids(mass, dz, stage=2)
    ref = ctx.mk_T_maps()
    uncertain = ctx.fallback_count()
    ctx.free()
    assert np.count_nonzero(ref) > 1000

    dev_mass = torch.from_numpy(mass).cuda()
    dev_dz = torch.from_numpy(dz).cuda()
    dev_maps = torch.empty(ref.shape, dtype=torch.float32, device="cuda")
    vp = C.c_void_p
    L.gethi_project_noalloc.argtypes = [C.POINTER(type(p)), C.POINTER(Derived), vp, vp, vp, vp, vp, vp, vp, vp]
    stream = torch.cuda.current_stream()
    for _ in range(calls):
        dev_maps.fill_(7.0)  # stale contents must not leak into the result
        rc = L.gethi_project_noalloc(C.byref(p), C.byref(d), tables.ctypes.data, offsets.ctypes.data,
                                     prefac.ctypes.data, None if edges is None else edges.ctypes.data,
                                     dev_mass.data_ptr(), dev_dz.data_ptr(), dev_maps.data_ptr(), stream.cuda_stream)
        assert rc == 0, L.gethi_last_error()
        torch.cuda.synchronize()
        np.testing.assert_allclose(dev_maps.cpu().numpy(), ref, rtol=1e-5, atol=1e-6 * np.abs(ref).max())
    return uncertain


def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crime_gb300 import build
    build.build()
    import crime_gb300 as gh
    return torch, gh


def test_project_noalloc_matches_make_maps():
    torch, gh = _cuda()
    from crime_gb300.gethi import Derived, lib
    L = lib()
    n, nside = 64, 64
    nut = os.path.join(GOLDEN, "nutable_8.txt")
    p = gh.make_params(frequencies_filename=nut, n_grid=n, n_side=nside, seed=21, **COSMO)
    edges = np.ascontiguousarray(np.loadtxt(nut), np.float64)
    rng = np.random.default_rng(3)
    mass = rng.lognormal(0.0, 1.0, (n, n, n)).astype(np.float32)
    dz = rng.normal(0.0, 2e-3, (n, n, n)).astype(np.float32)
    _compare(torch, gh, p, edges, mass, dz)
    d, tables, offsets, prefac = _setup(p)
    dev_mass = torch.from_numpy(mass).cuda()
    dev_dz = torch.from_numpy(dz).cuda()
    dev_maps = torch.empty((d.n_nu, 12 * nside * nside), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    # a request beyond the entry point's stated maximum is refused
    big = gh.make_params(pk_filename="EH", frequencies_filename="", n_nu=5000, n_grid=n, n_side=4)
    dbig = Derived()
    assert L.gethi_host_setup(C.byref(big), C.byref(dbig), None, None, None, None, None) == 0
    tb, ob, pb = np.zeros(6 * 5001), np.zeros(30), np.zeros(dbig.n_nu)
    assert L.gethi_host_setup(C.byref(big), C.byref(dbig), tb.ctypes.data, None, None, ob.ctypes.data,
                              pb.ctypes.data) == 0
    rc = L.gethi_project_noalloc(C.byref(big), C.byref(dbig), tb.ctypes.data, ob.ctypes.data, pb.ctypes.data, None,
                                 dev_mass.data_ptr(), dev_dz.data_ptr(), dev_maps.data_ptr(), stream.cuda_stream)
    assert rc == -1 and b"maximum" in L.gethi_last_error()


def test_project_noalloc_regular_table():
    """Shells from nu_min, nu_max, n_nu (no frequency file): the entry point builds
    the edges itself and bins by the reference's (int) truncation."""
    torch, gh = _cuda()
    n = 64
    p = gh.make_params(frequencies_filename="", nu_min=900.0, nu_max=1100.0, n_nu=5, n_grid=n, n_side=32, seed=5,
                       **COSMO)
    rng = np.random.default_rng(8)
    mass = rng.lognormal(0.0, 1.0, (n, n, n)).astype(np.float32)
    dz = rng.normal(0.0, 2e-3, (n, n, n)).astype(np.float32)
    _compare(torch, gh, p, None, mass, dz)


def test_project_noalloc_queue_overflow():
    """More uncertain samples than the entry point's fixed queue holds (2^20):
    those beyond it are decided inside the projection kernel in FP64, and the
    maps still equal the allocating path's."""
    torch, gh = _cuda()
    n = 384
    # a box inside the outer shell (corner at 2165 Mpc/h, z = 1.03 at 2340 Mpc/h): nearly every sample is in a shell
    p = gh.make_params(frequencies_filename="", nu_min=700.0, nu_max=1300.0, n_nu=8, n_grid=n, n_side=1024,
                       l_box=2500.0, seed=9, **COSMO)
    rng = np.random.default_rng(11)
    mass = rng.lognormal(0.0, 1.0, (n, n, n)).astype(np.float32)
    dz = rng.normal(0.0, 2e-3, (n, n, n)).astype(np.float32)
    uncertain = _compare(torch, gh, p, None, mass, dz, calls=1)
    assert uncertain > (1 << 20), "the case must overflow the entry point's queue (%d uncertain samples)" % uncertain
