"""Generate the golden vectors under tests/golden/ from the reference itself.

Runs the reference's own GetHI sources, compiled with project shims by
``make -C oracle ref`` (oracle/_ref/gethi_ref_{irr,reg}), on small configs and
stores every stage's buffers as compressed .npz fixtures.  Only this script
needs the reference tree; the fixtures it writes travel with the repository.

    python tests/golden/make_golden.py            # rebuild all fixtures
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
NU21 = 1420.40575177

# Cosmology of the synthetic configs: Planck-like, EH no-wiggle P(k).
COSMO = dict(omega_M=0.315, omega_L=0.685, omega_B=0.049, h=0.67, w=-1.0, ns=0.96, sigma_8=0.83)


def eh_nowiggle(k, om, ob, h, ns, tcmb=2.7255):
    """Eisenstein & Hu (1998, ApJ 496:605) zero-baryon-oscillation transfer
    function times k^ns (amplitude arbitrary: GetHI renormalises to sigma_8)."""
    theta = tcmb / 2.7
    omh2, obh2 = om * h * h, ob * h * h
    fb = ob / om
    s = 44.5 * np.log(9.83 / omh2) / np.sqrt(1 + 10 * obh2 ** 0.75)
    alpha = 1 - 0.328 * np.log(431 * omh2) * fb + 0.38 * np.log(22.3 * omh2) * fb * fb
    gamma = om * h * (alpha + (1 - alpha) / (1 + (0.43 * k * h * s) ** 4))
    q = k * theta * theta / gamma
    l0 = np.log(2 * np.e + 1.8 * q)
    c0 = 14.2 + 731.0 / (1 + 62.5 * q)
    t = l0 / (l0 + c0 * q * q)
    return k ** ns * t * t


def write_pk(path, nk=1000, kmin=1e-4, kmax=10.0):
    k = np.logspace(np.log10(kmin), np.log10(kmax), nk)
    p = eh_nowiggle(k, COSMO["omega_M"], COSMO["omega_B"], COSMO["h"], COSMO["ns"]) * 2e4
    with open(path, "w") as f:
        for a, b in zip(k, p):
            f.write("%.6E %.6E\n" % (a, b))


def write_ini(path, pk, extra):
    kv = dict(prefix_out="golden", pk_filename=pk, r_smooth=2.0, n_grid=32, n_side=16, seed=1001,
              do_psources=0)
    kv.update({k: v for k, v in COSMO.items()})
    kv.update(extra)
    with open(path, "w") as f:
        f.write("# golden-vector config\n")
        for k, v in kv.items():
            f.write("%s= %s\n" % (k, v))


def run_case(binary, ini, nthreads, outdir):
    env = dict(os.environ, OMP_NUM_THREADS=str(nthreads))
    subprocess.run([binary, ini, outdir], check=True, env=env, stdout=subprocess.DEVNULL)
    out = {}
    with open(os.path.join(outdir, "params.txt")) as f:
        for line in f:
            k, v = line.split()
            out["p_" + k] = np.float64(v)
    for fn in os.listdir(outdir):
        stem, ext = os.path.splitext(fn)
        if ext == ".f64":
            out[stem] = np.fromfile(os.path.join(outdir, fn), dtype=np.float64)
        elif ext == ".f32":
            out[stem] = np.fromfile(os.path.join(outdir, fn), dtype=np.float32)
        elif ext == ".i32":
            out[stem] = np.fromfile(os.path.join(outdir, fn), dtype=np.int32)
    return out


def main():
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "ref"], check=True,
                   stdout=subprocess.DEVNULL)
    ref_irr = os.path.join(REPO, "oracle", "_ref", "gethi_ref_irr")
    ref_reg = os.path.join(REPO, "oracle", "_ref", "gethi_ref_reg")
    pk = os.path.join(HERE, "pk_eh_nowiggle.txt")
    write_pk(pk)
    # irregular table: 8 channels uniform in nu between z=1.0 and z=0.5
    nutab = os.path.join(HERE, "nutable_8.txt")
    edges = np.linspace(NU21 / 2.0, NU21 / 1.5, 9)
    np.savetxt(nutab, edges, fmt="%.6f")

    cases = {
        # name: (binary, n_threads, ini keys)
        "case_irr32": (ref_irr, 1, dict(frequencies_filename=nutab, n_grid=32, n_side=16, seed=1001)),
        "case_reg24": (ref_reg, 1, dict(nu_min=600.0, nu_max=900.0, n_nu=6, n_grid=24, n_side=8,
                                        seed=77, r_smooth=-1.0)),
        "case_irr32_t3": (ref_irr, 3, dict(frequencies_filename=nutab, n_grid=32, n_side=16, seed=1001)),
        # point sources: z <= 0.023 keeps the derived box small (cells ~6 Mpc/h, Poisson means < 10)
        "case_ps32": (ref_reg, 1, dict(nu_min=1388.0, nu_max=1410.0, n_nu=4, n_grid=32, n_side=16, seed=505,
                                       do_psources=1)),
        "case_ps32_t3": (ref_reg, 3, dict(nu_min=1388.0, nu_max=1410.0, n_nu=4, n_grid=32, n_side=16, seed=505,
                                          do_psources=1)),
    }
    with tempfile.TemporaryDirectory() as td:
        for name, (binary, nthr, keys) in cases.items():
            ini = os.path.join(td, name + ".ini")
            write_ini(ini, pk, keys)
            od = os.path.join(td, name)
            os.makedirs(od)
            out = run_case(binary, ini, nthr, od)
            if name == "case_ps32_t3":  # atomic float sums: only the counts are thread-order independent
                out = {k: v for k, v in out.items() if k in ("nsources", "dens_real") or k.startswith("p_")}
            elif name.endswith("_t3"):
                out = {k: v for k, v in out.items() if k in ("dens_k", "vpot_k") or k.startswith("p_")}
            elif name == "case_ps32":
                out = {k: v for k, v in out.items() if k not in ("dens_k", "vpot_k", "vpot_real", "tables")}
            elif name != "case_irr32":
                out.pop("tables", None)
            cfg = {k: np.asarray(v) for k, v in keys.items() if k != "frequencies_filename"}
            cfg["n_threads"] = np.asarray(nthr)
            cfg["regular_nu"] = np.asarray(int("nu_min" in keys))
            np.savez_compressed(os.path.join(HERE, name + ".npz"),
                                **out, **{"cfg_" + k: v for k, v in cfg.items()})
            print(name, sorted(out.keys()))


if __name__ == "__main__":
    sys.exit(main())
