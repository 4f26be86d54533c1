"""CPU baseline timing (test infrastructure): the reference's own GetHI stages,
compiled from its sources with the project shims (`make -C oracle ref`: GSL,
chealpix, cfitsio and FFTW calls answered by the shims; the FFT is the shim's
FP64 transform, not FFTW), run on all host cores with one workload's
cosmology, shells and Nside.  The reference derives its box from the outer
shell (src/cosmo.c:361), so the box here is 2 r_max (1 + 2/N) whatever the
workload states.

    python -m oracle.time_ref --n-grid 128 --zmin 0.5 --zmax 1.0 --n-nu 30 --n-side 64 --seed 1001

prints one JSON line: seconds per stage, voxels/s and the thread count."""
import argparse
import json
import os
import subprocess
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
NU21 = 1420.40575177
COSMO = dict(omega_M=0.315, omega_L=0.685, omega_B=0.049, h=0.67, w=-1.0, ns=0.96, sigma_8=0.83)


def time_reference(n_grid, zmin, zmax, n_nu, n_side, seed, threads=None):
    binary = os.path.join(HERE, "_ref", "gethi_ref_reg")
    if not os.path.exists(binary):
        raise RuntimeError("oracle/_ref/gethi_ref_reg is not built (make -C oracle ref, needs the reference tree)")
    threads = threads or os.cpu_count()
    with tempfile.TemporaryDirectory() as td:
        ini = os.path.join(td, "param.ini")
        kv = dict(prefix_out=os.path.join(td, "out"), pk_filename=os.path.join(REPO, "tests", "golden",
                                                                               "pk_eh_nowiggle.txt"),
                  r_smooth=2.0, n_grid=n_grid, n_side=n_side, seed=seed, do_psources=0,
                  frequencies_filename="default", nu_min=NU21 / (1 + zmax), nu_max=NU21 / (1 + zmin), n_nu=n_nu,
                  **COSMO)
        with open(ini, "w") as f:
            for k, v in kv.items():
                f.write("%s= %s\n" % (k, v))
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        t0 = time.perf_counter()
        out = subprocess.run([binary, ini, "-"], check=True, env=env, capture_output=True, text=True).stdout
        wall = time.perf_counter() - t0
    stages = {}
    for line in out.splitlines():
        f = line.split()
        if len(f) == 3 and f[0] == "stage" and f[1] != "dumps":
            stages[f[1]] = stages.get(f[1], 0.0) + float(f[2])
    work = sum(v for k, v in stages.items() if k != "setup")
    return {"n_grid": n_grid, "threads": threads, "stage_s": {k: round(v, 3) for k, v in stages.items()},
            "realisation_s": round(work, 3), "voxels_per_s": n_grid ** 3 / work, "wall_s": round(wall, 3)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-grid", type=int, required=True)
    ap.add_argument("--zmin", type=float, required=True)
    ap.add_argument("--zmax", type=float, required=True)
    ap.add_argument("--n-nu", type=int, required=True)
    ap.add_argument("--n-side", type=int, required=True)
    ap.add_argument("--seed", type=int, default=1001)
    ap.add_argument("--threads", type=int, default=0)
    a = ap.parse_args()
    print(json.dumps(time_reference(a.n_grid, a.zmin, a.zmax, a.n_nu, a.n_side, a.seed, a.threads or None)))


if __name__ == "__main__":
    main()
