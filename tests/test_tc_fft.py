"""Tensor-core split-precision column transforms (fft_precision=tc_split, n_grid=1024)
against the FP32 CUDA-core transforms on the same Philox modes and against an
FP64 evaluation of delta on whole z planes.

The FP64 plane z0 is delta(x, y, z0) = norm * sum_k modes(k) e^{i k.x}, evaluated
separably from the downloaded modes (sum over kz at z0, then an FP64 inverse FFT
over ky and the c2r over kx with the real-part semantics of the path)."""
import numpy as np
import pytest

from test_gpu_parity import gh  # noqa: F401  (fixture)

NU21 = 1420.40575177
COSMO = dict(omega_M=0.315, omega_L=0.685, omega_B=0.049, h=0.67, w=-1.0, ns=0.96, sigma_8=0.83)
N = 1024
L_BOX = 4000.0


def _params(gh, prec):
    return gh.make_params(pk_filename="EH", frequencies_filename="", nu_min=NU21 / 3.0, nu_max=NU21 / 1.3,
                          n_nu=8, n_side=64, n_grid=N, l_box=L_BOX, seed=3001, do_rsd=1,
                          velocity_mode="spectral", fft_precision=prec, gaussianise=1, **COSMO)


def _fields(gh, prec, with_modes=False):
    ctx = gh.GetHI(_params(gh, prec))
    ctx.create_d_and_vr_fields()
    d, v = ctx.grids()
    m = ctx.device_modes() if with_modes else None
    ctx.free()
    return d, v, m


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _fp64_plane(modes, z0):
    n = modes.shape[0]
    ph = np.exp(2j * np.pi * np.arange(n) * z0 / n)
    s = np.zeros((n, n // 2 + 1), np.complex128)
    for a in range(0, n, 32):
        s += np.tensordot(ph[a:a + 32], modes[a:a + 32].astype(np.complex128), axes=(0, 0))
    t = np.fft.ifft(s, axis=0) * n
    norm = (np.sqrt(2 * np.pi) / L_BOX) ** 3
    return np.fft.irfft(t, n=n, axis=1) * n * norm


@pytest.mark.gpu
def test_tc_split_fields_vs_fp32_and_fp64(gh):  # noqa: F811
    d32, v32, modes = _fields(gh, "fp32", with_modes=True)
    dtc, vtc, _ = _fields(gh, "tc_split")
    # same modes, both precisions: delta and the spectral v_r
    assert _rel(dtc, d32) < 2e-6
    assert _rel(vtc, v32) < 2e-6
    # error of each against FP64 on two z planes: tensor-core path <= 2e-6
    for z0 in (0, 517):
        ref = _fp64_plane(modes, z0)
        e32, etc = _rel(d32[z0], ref), _rel(dtc[z0], ref)
        assert e32 < 1e-6
        assert etc < 2e-6
