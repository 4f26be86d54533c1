"""Failure detection on the GPU without a fault: every device-side wait of the
library is bounded by time and reports through the context's error flag.  The
self-test makes one such wait run out (an mbarrier nothing arrives on, nothing
asynchronous in flight); the call must report GETHI_E_CUDA once, within the
bound, and the context must then run a realisation as before."""
import os
import time

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def test_wait_expiry_reported_and_context_recovers():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crime_gb300 import build
    build.build()
    import crime_gb300 as gh
    from crime_gb300.gethi import lib
    p = gh.make_params(omega_M=0.315, omega_L=0.685, omega_B=0.049, h=0.67, w=-1.0, ns=0.96, sigma_8=0.83,
                       pk_filename=os.path.join(GOLDEN, "pk_eh_nowiggle.txt"),
                       frequencies_filename=os.path.join(GOLDEN, "nutable_8.txt"), n_grid=32, n_side=16, seed=3)
    ctx = gh.GetHI(p)
    before = ctx.run()
    for _ in range(2):  # reported by each expiry, and cleared after it
        t0 = time.perf_counter()
        rc = ctx.wait_selftest(20000)  # 20 ms bound
        dt = time.perf_counter() - t0
        assert rc == -4, rc  # GETHI_E_CUDA
        assert b"expired" in lib().gethi_last_error()
        assert dt < 5.0
    after = ctx.run()
    ctx.free()
    np.testing.assert_allclose(after, before, rtol=1e-5, atol=1e-6 * np.abs(before).max())
