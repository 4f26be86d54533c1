"""The command-line drop-in: `GetHI_gpu param.ini` (for `./GetHI param.ini`,
src/main_gh.c:24-80) reads a reference .ini and writes <prefix_out>_%03d.fits,
one RING BINTABLE per shell with the column T in mK (src/io_gh.c:69-82,
src/healpix_extra.c:132-164), and <prefix_out>_ps_%03d.fits for point sources."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, REPO
from test_gpu_parity import gh  # noqa: F401  (fixture)

EXE = os.path.join(REPO, "crime_gb300", "lib", "GetHI_gpu")


def read_fits_map(path):
    """(header cards of the table extension, big-endian float column)"""
    raw = open(path, "rb").read()
    assert len(raw) % 2880 == 0

    def header(off):
        cards = {}
        while True:
            block = raw[off:off + 2880]
            off += 2880
            for i in range(36):
                c = block[80 * i:80 * i + 80].decode("ascii")
                key = c[:8].strip()
                if key == "END":
                    return cards, off
                if c[8:10] == "= ":
                    cards[key] = c[10:].split("/")[0].strip().strip("'").strip()

    h0, off = header(0)
    assert h0["SIMPLE"] == "T" and h0["EXTEND"] == "T"
    h1, off = header(off)
    n = int(h1["NAXIS2"])
    data = np.frombuffer(raw[off:off + 4 * n], dtype=">f4").astype(np.float32)
    return h1, data


@pytest.mark.gpu
def test_cli_writes_reference_fits(gh, tmp_path):  # noqa: F811
    ini = tmp_path / "param.ini"
    prefix = tmp_path / "run"
    keys = dict(prefix_out=str(prefix), pk_filename=os.path.join(GOLDEN, "pk_eh_nowiggle.txt"), r_smooth=2.0,
                n_grid=32, n_side=16, seed=505, do_psources=1, omega_M=0.315, omega_L=0.685, omega_B=0.049,
                h=0.67, w=-1.0, ns=0.96, sigma_8=0.83, nu_min=1388.0, nu_max=1410.0, n_nu=4)
    with open(ini, "w") as f:
        f.write("# reference-style parameter file\n")
        for k, v in keys.items():
            f.write("%s= %s\n" % (k, v))
    out = subprocess.run([EXE, str(ini)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    ctx = gh.GetHI(gh.read_params(str(ini)))
    ref = ctx.run()
    ref_ps, _ = ctx.psources_maps()
    ctx.free()
    for i in range(4):
        h, t = read_fits_map("%s_%03d.fits" % (prefix, i + 1))
        assert h["XTENSION"] == "BINTABLE" and h["TTYPE1"] == "T" and h["TFORM1"] == "1E"
        assert h["TUNIT1"] == "mK" and h["PIXTYPE"] == "HEALPIX" and h["ORDERING"] == "RING"
        assert int(h["NSIDE"]) == 16 and h["COORDSYS"] == "G" and int(h["NAXIS2"]) == 12 * 16 ** 2
        assert np.abs(ref[i]).max() > 0
        # the same realisation: only the FP32 accumulation order may differ
        assert np.linalg.norm(t - ref[i]) <= 1e-6 * np.linalg.norm(ref[i])
        _, tps = read_fits_map("%s_ps_%03d.fits" % (prefix, i + 1))
        assert np.linalg.norm(tps - ref_ps[i]) <= 1e-6 * np.linalg.norm(ref_ps[i])
