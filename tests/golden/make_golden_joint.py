"""Golden vectors for the JoinT map combination: runs the reference's own JoinT
(src/main_jt.c, io_jt.c, common_jt.c, common.c, healpix_extra.c compiled in
place against the test shims, oracle/Makefile target `ref`) on small seeded
inputs written as HEALPix FITS files, and stores inputs and outputs as
tests/golden/joint_*.npz.  Needs the reference sources; run from the repo root:
    python tests/golden/make_golden_joint.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))
from fits_io import read_map, write_map  # noqa: E402

NU21 = 1420.40575177
COMPONENTS = ["cosmo", "extragalactic_freefree", "galactic_freefree", "point_sources", "synchrotron", "custom"]


def nest_order(ring_map, nside):
    """the same sky in NESTED order (for inputs written NESTED)"""
    sys.path.insert(0, REPO)
    from oracle import orc
    out = np.empty_like(ring_map)
    for p in range(ring_map.size):
        out[p] = ring_map[orc.nest2ring(nside, p)]
    return out


def make_case(td, name, nside_in, nside, n_nu, seed, present, leakage, dish, tsys, nthreads, masked,
              nest_inputs=(), repeat_inputs=()):
    rng = np.random.default_rng(seed)
    npix_in, npix = 12 * nside_in ** 2, 12 * nside ** 2
    edges = np.linspace(NU21 / 2.0, NU21 / 1.6, n_nu + 1)
    nutab = os.path.join(td, name + "_nuTable.dat")
    with open(nutab, "w") as f:
        for i in range(n_nu):  # the 5-column table GetHI writes (src/io_gh.c:84-107)
            f.write("%d %.17g %.17g %.17g %.17g\n" % (i + 1, edges[i], edges[i + 1], NU21 / edges[i + 1] - 1,
                                                       NU21 / edges[i] - 1))
    keys = {"fname_nutable": nutab, "prefix_out": os.path.join(td, name + "_out"), "nside": nside,
            "seed": seed, "do_polarization": 1 if leakage > 0 else 0, "polarization_leakage": leakage,
            "dish_diameter": dish, "n_dishes": 16, "t_system": tsys, "time_total": 1000.0}
    arrays = {}
    for comp in COMPONENTS:
        if comp not in present:
            keys["prefix_" + comp] = "none"
            continue
        prefix = os.path.join(td, name + "_" + comp)
        keys["prefix_" + comp] = prefix
        t = (rng.standard_normal((n_nu, npix_in)) * 10 + 5).astype(np.float32)
        arrays["in_" + comp] = t
        cols = [t]
        if comp == "synchrotron":
            q = (rng.standard_normal((n_nu, npix_in)) * 50).astype(np.float32)
            arrays["in_synchrotron_q"] = q
            cols = [t, q]
        for i in range(n_nu):
            c = [x[i] for x in cols]
            order = "RING"
            if comp in nest_inputs:
                c = [nest_order(x, nside_in) for x in c]
                order = "NESTED"
            write_map("%s_%03d.fits" % (prefix, i + 1), c, nside_in, ordering=order,
                      repeat=64 if comp in repeat_inputs else 1)
    if masked:
        mask = (rng.random(npix) > 0.3).astype(np.float32)
        write_map(os.path.join(td, name + "_mask.fits"), [mask], nside)
        keys["fname_mask"] = os.path.join(td, name + "_mask.fits")
        arrays["mask"] = mask.astype(np.int32)
    else:
        keys["fname_mask"] = "none"
    ini = os.path.join(td, name + ".ini")
    with open(ini, "w") as f:
        for k, v in keys.items():
            f.write("%s= %s\n" % (k, v))
    exe = os.path.join(REPO, "oracle", "_ref", "joint_ref")
    env = dict(os.environ, OMP_NUM_THREADS=str(nthreads))
    subprocess.run([exe, ini], check=True, env=env, stdout=subprocess.DEVNULL)
    out = np.stack([read_map("%s_out_%03d.fits" % (os.path.join(td, name), i + 1))[1] for i in range(n_nu)])
    inst = np.loadtxt(os.path.join(td, name + "_out_instrument.dat"), ndmin=2)
    cfg = dict(nside_in=nside_in, nside=nside, n_nu=n_nu, seed=seed, leakage=leakage, dish=dish, n_dish=16,
               tsys=tsys, time_tot=1000.0, n_threads=nthreads)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), maps=out, instrument=inst, nu0=edges[:-1],
                        nuf=edges[1:], present=np.array(present), **arrays,
                        **{"cfg_" + k: np.asarray(v) for k, v in cfg.items()})
    print(name, out.shape, sorted(arrays))


def main():
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "ref"], check=True, stdout=subprocess.DEVNULL)
    with tempfile.TemporaryDirectory() as td:
        # merge of five components (one NESTED, one with 64-element rows), polarisation
        # leakage, degrade 8 -> 4, noise, mask; no beam
        make_case(td, "joint_merge", 8, 4, 3, 1234, ["cosmo", "extragalactic_freefree", "point_sources",
                                                     "synchrotron", "galactic_freefree"], 0.01, -1.0, 800.0, 1,
                  True, nest_inputs=("point_sources",), repeat_inputs=("galactic_freefree",))
        # upgrade 4 -> 8, beam of a 2 m dish (FWHM ~ 11 deg), noise, no mask
        make_case(td, "joint_beam", 4, 8, 2, 99, ["cosmo", "point_sources"], -1.0, 2.0, 500.0, 1, False)
        # same resolution, beam, noise drawn by 3 OpenMP threads, mask
        make_case(td, "joint_t3", 8, 8, 4, 7, ["cosmo"], -1.0, 3.0, 900.0, 3, True)


if __name__ == "__main__":
    sys.exit(main())
