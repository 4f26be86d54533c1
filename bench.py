"""Throughput of the GB300 GetHI realisation path (one JSON line on rank 0).

Workload (default): a 1024^3 realisation in a 4000 Mpc/h box with redshift-
space distortions (spectral velocity, three c2r FFTs of i k_j/k^2 delta_k),
Philox modes from an Eisenstein-Hu no-wiggle P(k), 150 frequency shells over
z 0.3-2.0 and Nside=512 maps.  A step is one whole realisation: modes ->
4 c2r FFTs -> sigma^2 -> fused lognormal/HI/RSD -> projection -> channel scaling.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config c2]

`value` is voxels/s with everything resident in HBM; `e2e` is the same metric
through the public C ABI with the per-realisation host inputs copied in from
pinned memory and the maps copied back to pinned host memory every step.
Under torchrun each rank runs an independent replica (its own seed) on its own
GPU; there is no data-path collective.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
NU21 = 1420.40575177

# Synthetic configurations (seeded; the P(k) is the built-in EH no-wiggle table).
CONFIGS = {
    "c0": dict(n_grid=128, l_box=1500.0, zmin=0.5, zmax=1.0, n_nu=30, n_side=64, seed=1001, do_rsd=0,
               bias_model="const", b_HI=1.0, velocity_mode="spectral", gaussianise=1),
    "c1": dict(n_grid=512, l_box=2500.0, zmin=0.3, zmax=2.0, n_nu=150, n_side=256, seed=2001, do_rsd=1,
               velocity_mode="spectral", gaussianise=1),
    "c2": dict(n_grid=1024, l_box=4000.0, zmin=0.3, zmax=2.0, n_nu=150, n_side=512, seed=3001, do_rsd=1,
               velocity_mode="spectral", gaussianise=1),
    "c4": dict(n_grid=2048, l_box=6000.0, zmin=0.2, zmax=2.5, n_nu=256, n_side=1024, seed=5001, do_rsd=1,
               velocity_mode="spectral", gaussianise=1),
}
COSMO = dict(omega_M=0.315, omega_L=0.685, omega_B=0.049, h=0.67, w=-1.0, ns=0.96, sigma_8=0.83)
# ensemble: (n_grid, box, realisations, lanes = concurrent contexts of that size); seeds 4000.. in order
ENSEMBLE = dict(members=[(128, 1000.0, 32, 4), (256, 2000.0, 24, 3), (384, 3000.0, 8, 2)], seed=4000, zmin=0.5,
                zmax=1.5, n_nu=64, n_side=128, do_rsd=1, velocity_mode="spectral", gaussianise=1)


def params_for(cfg, seed_offset=0):
    import crime_gb300 as gh
    c = dict(cfg)
    zmin, zmax = c.pop("zmin"), c.pop("zmax")
    c["seed"] = c["seed"] + seed_offset
    return gh.make_params(pk_filename="EH", frequencies_filename="", nu_min=NU21 / (1 + zmax),
                          nu_max=NU21 / (1 + zmin), **COSMO, **c)


def replica_seed(base, rank, step, stride=7919):
    """Seed of realisation `step` on rank `rank` (replicas: every rank runs its own
    realisations; distinct for ranks < stride)."""
    return base + rank + stride * step


def max_over_ranks(x, ws, device="cuda"):
    """The slowest rank's value (replicas finish when the last one does)."""
    if ws == 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_step, steps, ws, ms):
    """Units processed by all ranks over the slowest rank's time (per second)."""
    return units_per_step * steps * ws / (ms / 1e3)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def read_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region (clocks and throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_bytes(cls, n, npix, n_nu, zfields=3, gaussianised=True):
    """Minimum HBM bytes of one launch of a kernel class (FP32 data; a mode is one
    complex of the N^3/2-mode half spectrum, a cell one of N^3)."""
    n3 = float(n) ** 3
    return {
        # the drawing Z pass writes zfields transformed fields (delta; + phi; + i kz phi for the
        # spectral velocity) at 8 B/mode each and reads P_G (4 B/mode) when the spectrum is Gaussianised
        "zpass": 4 * zfields * n3 + (2 * n3 if gaussianised else 0),
        "zpass_raw": 8 * n3,        # read the raw modes, write the transformed column
        "ypass": 8 * n3,            # read + write 8 B/mode
        "xpass": 8 * n3,            # read 8 B/mode, write 4 B/cell
        "xpass_vel": 16 * n3,       # read v_x, v_y, v_z (8 B/mode each), write v_r 4 B/cell
        "project": 8 * n3 + 4.0 * npix * n_nu,  # read delta, v_r; write the maps once
        "scale": 8.0 * npix * n_nu,
    }.get(cls)


def fp64_planes(modes, zs, n, l_box, vfac, pos_obs):
    """delta(x, y, z0) and v_r(x, y, z0) on whole z planes in FP64 from a half spectrum
    [kz][ky][kx <= n/2]: separable sums (kz at z0, an FP64 inverse FFT over ky, the
    c2r over kx taking Re of the kx = 0 and n/2 terms), the spectral velocity
    v_j = c2r(i k_j delta_k f0 H0 / k^2) with derivatives of Nyquist indices set to
    zero, and v_r = v . (x - x_obs)/|x - x_obs| at cell centres."""
    m = n // 2
    dk = 2 * np.pi / l_box
    idx = np.arange(n)
    kv = np.where(2 * idx <= n, idx, idx - n) * dk
    kd = kv.copy()
    kd[m] = 0.0
    kx, kdx = kv[:m + 1], kd[:m + 1]
    norm = (np.sqrt(2 * np.pi) / l_box) ** 3
    cc = (idx + 0.5) * (l_box / n) - pos_obs
    out = []
    for z0 in zs:
        ph = np.exp(2j * np.pi * idx * z0 / n)
        acc = [np.zeros((n, m + 1), np.complex128) for _ in range(4)]
        for a in range(0, n, 16):
            blk = modes[a:a + 16].astype(np.complex128)
            k2 = kv[a:a + 16, None, None] ** 2 + kv[None, :, None] ** 2 + kx[None, None, :] ** 2
            with np.errstate(divide="ignore", invalid="ignore"):
                phi = blk * np.where(k2 > 0, vfac / k2, 0.0)
            p = ph[a:a + 16]
            acc[0] += np.tensordot(p, blk, axes=(0, 0))
            acc[1] += np.tensordot(p, phi, axes=(0, 0)) * (1j * kdx[None, :])
            acc[2] += np.tensordot(p, phi, axes=(0, 0)) * (1j * kd[:, None])
            acc[3] += np.tensordot(p * (1j * kd[a:a + 16]), phi, axes=(0, 0))
        pl = [np.fft.irfft(np.fft.ifft(s, axis=0) * n, n=n, axis=1) * n * norm for s in acc]
        x, y, z = cc[None, :], cc[:, None], cc[z0]
        r = np.sqrt(x * x + y * y + z * z)
        out.append((pl[0], (pl[1] * x + pl[2] * y + pl[3] * z) / r))
    return out


def fft_precision_compare(args, cfg, ctx32, stream, local, steps, ms32, ktimes32):
    """The same workload with the tensor-core split-precision column passes: time per
    realisation, column-pass time, and the error of delta and v_r of both paths against
    FP64 on two z planes (same Philox seed)."""
    import torch

    import crime_gb300 as gh
    n = cfg["n_grid"]
    ctx = gh.GetHI(params_for(dict(cfg, fft_precision="tc_split")), device=local)
    ctx.set_stream(stream.cuda_stream)
    for i in range(2):
        ctx.set_seed(cfg["seed"] + 1000 * (i + 1))
        ctx.run_into(0)
    torch.cuda.synchronize()
    ctx.profile(True)
    ctx.kernel_times()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for i in range(steps):
        ctx.set_seed(cfg["seed"] + 7919 * i)
        ctx.run_into(0)
    b.record(stream)
    torch.cuda.synchronize()
    mstc = a.elapsed_time(b)
    kttc, _ = ctx.kernel_times()
    ctx.profile(False)

    def col_ms(kt):
        return sum(kt[k][0] for k in ("zpass", "ypass", "nyq") if k in kt) / steps

    # errors on one seed
    seed = cfg["seed"]
    npix, n_nu = ctx.npix, ctx.n_nu
    res = {}
    maps = {}
    for name, c in (("fp32", ctx32), ("tc_split", ctx)):
        c.set_seed(seed)
        maps[name] = c.run()
        c.create_d_and_vr_fields()
        res[name] = c.grids()
    modes = ctx32.device_modes()
    d = ctx32.derived()
    zs = (0, 517 % n)
    planes = fp64_planes(modes, zs, n, d.l_box, d.fgrowth_0 * d.hubble_0, d.pos_obs)
    del modes

    def rel(x, y):
        x = np.asarray(x, np.float64)
        y = np.asarray(y, np.float64)
        return float(np.linalg.norm(x - y) / np.linalg.norm(y))

    out = {"fft": "column passes (Z, Y) of the 1024-point c2r; the X (row) passes are FP32 in both",
           "error_vs_fp64": "relative L2 on the z planes %s against an FP64 separable evaluation of the same "
                            "modes" % (list(zs),)}
    for name, ms_, kt in (("fp32", ms32, ktimes32), ("tc_split", mstc, kttc)):
        dd, vv = res[name]
        out[name] = {"ms_per_step": round(ms_ / steps, 3), "voxels_per_s": float(n) ** 3 * steps / (ms_ / 1e3),
                     "column_pass_ms_per_step": round(col_ms(kt), 3),
                     "delta_rel_l2_vs_fp64": max(rel(dd[z], p[0]) for z, p in zip(zs, planes)),
                     "v_r_rel_l2_vs_fp64": max(rel(vv[z], p[1]) for z, p in zip(zs, planes))}
    out["maps_rel_l2_tc_vs_fp32"] = rel(maps["tc_split"], maps["fp32"])
    out["speedup_tc_over_fp32"] = round(out["fp32"]["ms_per_step"] / out["tc_split"]["ms_per_step"], 3)
    out["column_pass_speedup_tc_over_fp32"] = round(out["fp32"]["column_pass_ms_per_step"] /
                                                    out["tc_split"]["column_pass_ms_per_step"], 3)
    ctx.free()
    return out


def bench_ensemble(args):
    """The batched ensemble: every member's realisations in one CUDA-graph launch per
    step (run_batch), contexts of one size run as concurrent lanes, launch shapes
    from the autotuner.  value = voxels/s of the device-resident batch; e2e = the
    same through run_batch with the maps copied to host memory and the graph
    captured and instantiated inside the timed region."""
    import torch

    import crime_gb300 as gh
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    E = ENSEMBLE
    ctxs, jobs, tuned, filled = [], [], {}, {}
    seed = E["seed"] + 1000 * rank
    for n, box, count, lanes in E["members"]:
        first = len(ctxs)
        for ln in range(lanes):
            cfg = dict(n_grid=n, l_box=box, zmin=E["zmin"], zmax=E["zmax"], n_nu=E["n_nu"], n_side=E["n_side"],
                       seed=seed, do_rsd=E["do_rsd"], velocity_mode=E["velocity_mode"], gaussianise=E["gaussianise"])
            c = gh.GetHI(params_for(cfg), device=local)
            t = c.autotune()
            tuned.setdefault(n, []).append(t)
            ctxs.append(c)
        filled[n] = ctxs[first].derived().filled_fraction
        for i in range(count):
            jobs.append((first + i % lanes, seed))
            seed += 1
    voxels = float(sum(float(n) ** 3 * count for n, _, count, _ in E["members"]))
    for _ in range(args.warmup):
        gh.run_batch(ctxs, jobs, download=False, graph=True)
    torch.cuda.synchronize()
    dev_ms, stats = [], None
    clk = ClockSampler(local)
    with clk:
        for _ in range(args.steps):
            _, stats = gh.run_batch(ctxs, jobs, download=False, graph=True)
            dev_ms.append(stats["device_ms"])
    ms = max_over_ranks(sum(dev_ms), ws)
    # end to end: capture + instantiate + run + maps to the host, wall clock
    if ws > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        maps, st_e2e = gh.run_batch(ctxs, jobs, download=True, graph=True)
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws)
    assert all(np.isfinite(m).all() for m in maps)
    d2h = int(sum(4 * m.size for m in maps))
    # the same batch without the graph, and one realisation at a time through gethi_gpu_run
    _, st_ng = gh.run_batch(ctxs, jobs, download=False, graph=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k, s in jobs:
        ctxs[k].set_seed(s)
        ctxs[k].run_into(0)
    torch.cuda.synchronize()
    seq_s = time.perf_counter() - t0
    line = {
        "metric": "GetHI batched ensemble throughput (voxels/s): %s" % " + ".join(
            "%dx%d^3" % (cnt, n) for n, _, cnt, _ in E["members"]),
        "value": whole_job_rate(voxels, args.steps, ws, ms), "unit": "voxels/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic (Philox modes from an EH no-wiggle P(k))",
        "realisations_per_s": whole_job_rate(len(jobs), args.steps, ws, ms),
        "config": {"workload": "c3: " + ", ".join("%d x %d^3 (box %g Mpc/h, %d lanes)" % (cnt, n, box, ln)
                                                  for n, box, cnt, ln in E["members"]) +
                   "; seeds %d-%d; Nside %d x %d shells, z %.1f-%.1f; spectral RSD; Gaussianised P(k)" % (
                       E["seed"], E["seed"] + len(jobs) - 1, E["n_side"], E["n_nu"], E["zmin"], E["zmax"]),
                   "graph_nodes": stats["graph_nodes"], "kernel_launches_per_step": stats["kernel_launches"],
                   "autotuned": {str(n): v[0] for n, v in tuned.items()},
                   "filled_fraction": {str(n): f for n, f in filled.items()},
                   "l2": "the batch's working set (%.1f GB of fields) exceeds L2" % (
                       sum(6 * 4 * float(n) ** 3 * ln for n, _, _, ln in E["members"]) / 1e9)},
        "e2e": {"value": whole_job_rate(voxels, args.steps, ws, 1e3 * e2e_s), "unit": "voxels/s",
                "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": d2h, "includes": "graph capture + instantiate (%.1f ms) + run + maps to "
                                                      "host" % st_e2e["capture_ms"]},
        "gpu_launches": stats["kernel_launches"] * args.steps,
        "compare": {"batch_no_graph_ms": round(st_ng["device_ms"], 3),
                    "one_at_a_time_ms": round(1e3 * seq_s, 3),
                    "graph_ms": round(ms / args.steps, 3)},
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    for c in ctxs:
        c.free()
    if ws > 1:
        torch.distributed.destroy_process_group()


JOINT = dict(n_side=512, n_nu=150, zmin=0.3, zmax=2.0, dish_diameter=30.0, n_dish=64, tsys=25000.0,
             time_tot=10000.0, seed=6001, b_cut_deg=10.0)


def joint_workload(E=JOINT):
    edges = np.linspace(NU21 / (1 + E["zmax"]), NU21 / (1 + E["zmin"]), E["n_nu"] + 1)
    nside = E["n_side"]
    npix = 12 * nside * nside
    # galactic-plane cut |b| < b_cut (the RING pixel heights: z = cos(theta) per ring)
    z = np.empty(npix)
    ncap = 2 * nside * (nside - 1)
    for i in range(1, 4 * nside):
        north = i if i <= 2 * nside else 4 * nside - i
        if north < nside:
            zz, nph, first = 1 - north * north / (3.0 * nside * nside), 4 * north, 2 * north * (north - 1)
        else:
            zz, nph, first = (2 * nside - north) * 2.0 / (3 * nside), 4 * nside, ncap + (north - nside) * 4 * nside
        if north != i:
            zz, first = -zz, npix - nph - first
        z[first:first + nph] = zz
    mask = (np.abs(z) >= np.sin(np.radians(E["b_cut_deg"]))).astype(np.int32)
    return edges[:-1], edges[1:], mask


def bench_joint(args):
    """The JoinT combination of a c2-sized set of maps (Nside 512 x 150 channels):
    two components (HI and a foreground) summed, beam of a 30 m dish through the
    spherical harmonic transform (lmax 1535), Philox noise, |b| < 10 deg mask.
    value = map pixels (channels x 12 Nside^2) per second with the components
    resident in HBM; e2e = the same through the C ABI with the components copied in
    from pinned host memory and the maps copied back every step."""
    import torch

    from crime_gb300 import joint as jt
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    E = dict(JOINT)
    if args.joint_nside:
        E["n_side"] = args.joint_nside
    if args.joint_nnu:
        E["n_nu"] = args.joint_nnu
    nu0, nuf, mask = joint_workload(E)
    nside, n_nu = E["n_side"], E["n_nu"]
    npix = 12 * nside * nside
    g = torch.Generator(device="cuda").manual_seed(E["seed"] + rank)
    comp = [torch.randn((n_nu, npix), device="cuda", generator=g) * s for s in (0.1, 1000.0)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    j = jt.JoinT(nside, nu0, nuf, seed=E["seed"] + rank, dish_diameter=E["dish_diameter"], n_dish=E["n_dish"],
                 tsys=E["tsys"], time_tot=E["time_tot"], mask=mask, device=local)

    def step():
        for c in comp:
            j.add_maps_device(c.data_ptr(), nside)
        j.run(copy_out=False)

    step()  # builds the Legendre table (once per context)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    stages = np.zeros(4)
    with ClockSampler(local) as clk:
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        start.record()
        for _ in range(args.steps):
            step()
            st = j.stage_times()
            stages += [st["merge"], st["beam"], st["noise"], st["mask"]]
        end.record()
        torch.cuda.synchronize()
    ms = max_over_ranks(start.elapsed_time(end), ws)
    units = float(npix) * n_nu
    # end to end: pinned host components in, maps out
    host = [c.cpu().pin_memory() for c in comp]
    out = torch.empty((n_nu, npix), dtype=torch.float32, pin_memory=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for h in host:
            jt.lib().joint_gpu_add_maps(j._ctx, h.data_ptr(), nside, 1.0)
        jt._check(jt.lib().joint_gpu_run(j._ctx, out.data_ptr()))
    e2e_ms = max_over_ranks(1e3 * (time.perf_counter() - t0), ws)
    assert np.isfinite(out.numpy()).all()
    # channels per spherical-harmonic batch: every channel at once on the tensor-core path
    # (column tiles of 64 channels, up to 256), batches of 64 on the CUDA cores
    batch = min(256, 64 * -(-n_nu // 64)) if j.uses_tensor_cores else 64
    chunks = -(-n_nu // batch)
    # per-kernel-class device time of the beam over one more profiled step
    j.profile(True)
    step()
    kt = j.kernel_times()
    j.profile(False)
    lmax, R, N2 = 3 * nside - 1, 2 * nside, 2 * min(batch, n_nu)  # N2: real columns of the first batch
    nalm = (lmax + 1) * (lmax + 2) // 2
    gemm_bytes = 4.0 * (nalm * R + 2 * (lmax + 1) * R * N2 + nalm * N2)  # Legendre table + E/O + a_lm per batch
    gemm_flops = 2.0 * nalm * R * N2
    peak_hbm, peak_kind = read_peaks()
    if j.uses_tensor_cores:
        # the analysis GEMM alone (class "legendre_analysis" includes the E/O pack)
        ms_tc = (kt["legendre_analysis"][0] - kt["legendre_pack"][0]) / kt["legendre_analysis"][1]
        nkq = -(-R // 32)
        tiles = sum(-(-((lmax - m) // 2 + 1 if p == 0 else (lmax - m + 1) // 2) // 128) * nkq
                    for m in range(lmax + 1) for p in (0, 1))
        # columns used per 64-channel column tile (the last one cut to a multiple of 16)
        used = sum(min(128, -(-(N2 - 128 * ct) // 16) * 16) for ct in range(-(-N2 // 128)))
        # lambda tiles read once (their column tiles share them through L2), the used rows
        # of the E/O tiles read, the packed a_lm written
        packed = 32768.0 * (tiles + 2 * (lmax + 1) * nkq * used / 128) + 8.0 * nalm * used
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            bf16 = float(json.load(f)["bf16_tflops"])
        achieved = gemm_bytes / (ms_tc / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": "tc_legendre_analysis", "achieved": round(achieved, 1),
                "peak": peak_hbm, "unit": "GB/s", "frac": round(achieved / peak_hbm, 3), "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": gemm_bytes, "avg_launch_ms": round(ms_tc, 3),
                "traffic": packed,
                "traffic_source": "bytes of the packed operands per launch (hi and lo TF32 tiles of the Legendre "
                                  "table read once and of the used E/O rows of every 64-channel column tile, "
                                  "padded to 128 x 16 tiles, plus the packed a_lm written)",
                "batch_channels": batch,
                "traffic_gbs": round(packed / (ms_tc / 1e3) / 1e9, 1),
                "traffic_frac": round(packed / (ms_tc / 1e3) / 1e9 / peak_hbm, 3),
                "tensor": {"tflops": round(3 * gemm_flops / (ms_tc / 1e3) / 1e12, 1),
                           "peak_tflops": round(bf16 / 2, 1),
                           "peak_source": "half the measured dense bf16 burst (TF32 runs at half the bf16 rate)",
                           "frac": round(3 * gemm_flops / (ms_tc / 1e3) / 1e12 / (bf16 / 2), 3),
                           "note": "3 TF32 MMAs per product (hi*hi, hi*lo, lo*hi)"}}
    else:
        dom = max(("legendre_analysis", "legendre_synthesis"), key=lambda k: kt[k][0])
        per_launch = kt[dom][0] / kt[dom][1]
        fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12  # TFLOP/s: SMs x FP32 lanes x 2 x max clock (nominal)
        tflops = gemm_flops / (per_launch / 1e3) / 1e12
        roof = {"bound": "fp32", "kernel": dom, "achieved": round(tflops, 2), "peak": round(fp32_peak, 1),
                "unit": "TFLOP/s", "frac": round(tflops / fp32_peak, 3),
                "peak_source": "nominal FP32 CUDA-core rate (152 SMs x 128 lanes x 2 x 2.07 GHz); no measured figure",
                "flops_per_launch": gemm_flops, "avg_launch_ms": round(per_launch, 3), "traffic": None}
    line = {
        "metric": "JoinT map combination throughput (map pixels/s): Nside %d x %d channels, beam + noise + mask" % (
            nside, n_nu),
        "value": whole_job_rate(units, args.steps, ws, ms), "unit": "pixels/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic (Gaussian component maps, seeded)",
        "config": {"workload": "joint: Nside %d, %d channels over z %.1f-%.1f, 2 components, %g m dish "
                               "(lmax %d), Philox noise (t_sys %g mK, %g h, %d dishes), |b| < %g deg mask" % (
                                   nside, n_nu, E["zmin"], E["zmax"], E["dish_diameter"], 3 * nside - 1, E["tsys"],
                                   E["time_tot"], E["n_dish"], E["b_cut_deg"]),
                   "fsky": j.fsky, "legendre_table_gb": round(4.0 * (3 * nside) * (3 * nside + 1) / 2 * 2 * nside / 1e9, 2),
                   "setup_s_incl_legendre_table": round(setup_s, 3),
                   "l2": "inputs larger than L2 (maps %.1f GB, Legendre table above)" % (4 * units / 1e9)},
        "stage_ms": dict(zip(("merge", "beam", "noise", "mask"), np.round(stages / args.steps, 3).tolist())),
        "beam_kernels_ms": {k: round(v[0], 3) for k, v in kt.items()},
        "legendre": "tensor cores (3xTF32, tcgen05)" if j.uses_tensor_cores else "FP32 CUDA cores",
        "roofline": roof,
        "e2e": {"value": whole_job_rate(units, args.steps, ws, e2e_ms), "unit": "pixels/s",
                "h2d_bytes_per_step": int(4 * units * len(comp)), "d2h_bytes_per_step": int(4 * units)},
        # per step: one sum of the device components, per batch the ring analysis and synthesis and
        # the two Legendre kernels (+ the E/O pack on the tensor-core path), noise and mask in one pass
        "gpu_launches": args.steps * (1 + (5 if j.uses_tensor_cores else 4) * chunks + 1),
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_joint()
    if rank == 0:
        print(json.dumps(line), flush=True)
    j.close()


def cpu_baseline_joint(nside=64, n_nu=16):
    """The oracle's JoinT (FP64 transforms, one host thread) on a bounded sample:
    Nside 64, 16 channels, the same beam, noise and mask law."""
    from oracle import orc
    E = JOINT
    edges = np.linspace(NU21 / (1 + E["zmax"]), NU21 / (1 + E["zmin"]), n_nu + 1)
    rng = np.random.default_rng(1)
    npix = 12 * nside * nside
    comps = [(rng.standard_normal((n_nu, npix)).astype(np.float32), None) for _ in range(2)]
    mask = (rng.random(npix) > 0.17).astype(np.int32)
    t0 = time.perf_counter()
    orc.joint(comps, nside, nside, edges[:-1], edges[1:], dish=E["dish_diameter"] / 8, n_dish=E["n_dish"],
              tsys=E["tsys"], time_tot=E["time_tot"], seed=1, mask=mask)
    dt = time.perf_counter() - t0
    return {"value": npix * n_nu / dt, "unit": "pixels/s", "cores": 1, "kind": "port",
            "sample": "oracle JoinT (merge, FP64 map2alm/alm2map beam, MT noise, mask) at Nside %d x %d channels, "
                      "%.1f s" % (nside, n_nu, dt)}


def bench_ours(args):
    import torch

    import crime_gb300 as gh

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    cfg = CONFIGS[args.config]
    n = cfg["n_grid"]
    p = params_for(cfg, seed_offset=rank)
    ctx = gh.GetHI(p, device=local)
    stream = torch.cuda.Stream(device=local)
    ctx.set_stream(stream.cuda_stream)
    npix, n_nu = ctx.npix, ctx.n_nu

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    # ---- device-resident throughput
    for i in range(args.warmup):
        ctx.set_seed(replica_seed(cfg["seed"], rank, i + 1, stride=1000))
        ctx.run_into(0)
    barrier()
    ctx.profile(True)
    _, launches0 = ctx.kernel_times()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        start.record(stream)
        t0 = time.perf_counter()
        for i in range(args.steps):
            ctx.set_seed(replica_seed(cfg["seed"], rank, i))
            ctx.run_into(0)
        end.record(stream)
        barrier()
        wall = time.perf_counter() - t0
    ms = max_over_ranks(start.elapsed_time(end), ws)
    ktimes, launches1 = ctx.kernel_times()
    ctx.profile(False)
    fallbacks = ctx.fallback_count()

    # ---- end to end through the C ABI: host inputs in (pinned staging), maps out to
    # pinned host memory every step, pipelined (gethi_gpu_run_async: realisation i+1
    # computes while the maps of i are copied), wall clock around the whole loop
    maps_host = [torch.empty((n_nu, npix), dtype=torch.float32, pin_memory=True) for _ in range(2)]
    h2d = ctx.upload_inputs()
    ctx.run_async(maps_host[0].data_ptr())
    ctx.wait()
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        ctx.set_seed(replica_seed(cfg["seed"], rank, i + 1, stride=104729))
        h2d = ctx.upload_inputs()
        ctx.run_async(maps_host[i % 2].data_ptr())
    ctx.wait()
    e2e_ms = max_over_ranks(1e3 * (time.perf_counter() - t0), ws)
    barrier()
    assert all(np.isfinite(m.numpy()).all() for m in maps_host)

    voxels = float(n) ** 3
    value = whole_job_rate(voxels, args.steps, ws, ms)
    e2e = whole_job_rate(voxels, args.steps, ws, e2e_ms)

    # ---- roofline of the dominant kernel class
    peak, peak_kind = read_peaks()
    dom = max(((k, v) for k, v in ktimes.items() if v[1] > 0 and algorithmic_bytes(k, n, npix, n_nu)),
              key=lambda kv: kv[1][0])
    cls, (tot_ms, cnt) = dom
    per_launch_ms = tot_ms / cnt
    zf = (3 if cfg.get("velocity_mode") == "spectral" else 2) if cfg["do_rsd"] else 1
    gz = bool(cfg.get("gaussianise"))
    abytes = algorithmic_bytes(cls, n, npix, n_nu, zf, gz)
    achieved = abytes / (per_launch_ms / 1e3) / 1e9
    traffic = None
    tf = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(tf):
        with open(tf) as f:
            t = json.load(f)
        if cls in t:
            traffic = float(t[cls]["bytes_per_cell"]) * voxels if "bytes_per_cell" in t[cls] else None
    roof = {"bound": "hbm", "kernel": cls, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
            "algorithmic_bytes_per_launch": abytes, "avg_launch_ms": round(per_launch_ms, 4)}
    kernels = {k: {"ms_per_step": round(v[0] / args.steps, 4), "launches_per_step": v[1] / args.steps}
               for k, v in ktimes.items() if v[1] > 0}
    for k in kernels:
        b = algorithmic_bytes(k, n, npix, n_nu, zf, gz)
        if b:
            kernels[k]["GBps"] = round(b / (ktimes[k][0] / ktimes[k][1] / 1e3) / 1e9, 1)

    line = {
        "metric": "GetHI %d^3 realisation throughput (voxels/s), FP32 FFT path" % n,
        "value": value, "unit": "voxels/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic (Philox modes from an EH no-wiggle P(k))",
        "realisations_per_s": args.steps * ws / (ms / 1e3),
        "config": {"workload": "%s: %d^3 grid, box %g Mpc/h, RSD (spectral velocity), z %.1f-%.1f in %d shells, "
                               "Nside=%d" % (args.config, n, cfg["l_box"], cfg["zmin"], cfg["zmax"], cfg["n_nu"],
                                             cfg["n_side"]),
                   "n_grid": n, "n_side": cfg["n_side"], "n_nu": cfg["n_nu"], "l_box": cfg["l_box"],
                   "fft_precision": "fp32", "parallelism": "replicas" if ws > 1 else "single",
                   "l2": "inputs larger than L2 (each field is %.1f GB)" % (4 * voxels / 1e9)},
        "e2e": {"value": e2e, "unit": "voxels/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(4 * npix * n_nu)},
        "gpu_launches": int((launches1 - launches0)),
        "roofline": roof,
        "kernels": kernels,
        "fp64_fallback_samples_last_step": fallbacks,
        "clocks": clk.summary(),
        "wall_s": wall,
        "filled_fraction": ctx.derived().filled_fraction,
    }
    if ws == 1 and n == 1024 and not args.no_fft_compare:
        line["fft_precision_compare"] = fft_precision_compare(args, cfg, ctx, stream, local, args.steps, ms, ktimes)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.free()
    if ws > 1:
        torch.distributed.destroy_process_group()


def cpu_pipeline(cfg_name, n_sample):
    """The oracle (C restatement of the reference, OpenMP on all host cores) on a
    realisation of the workload's box, shells and Nside at n_sample^3 cells.
    Returns seconds per stage."""
    from oracle import orc
    cfg = dict(CONFIGS[cfg_name])
    k, pk = orc.load_pk(os.path.join(REPO, "tests", "golden", "pk_eh_nowiggle.txt"))
    o = orc.Oracle(dict(OmegaM=COSMO["omega_M"], OmegaL=COSMO["omega_L"], OmegaB=COSMO["omega_B"],
                        hhub=COSMO["h"], weos=-1.0, n_scal=COSMO["ns"], sig8=COSMO["sigma_8"], n_grid=n_sample,
                        n_side=cfg["n_side"], seed=cfg["seed"], regular_nu=1, nu_min=NU21 / (1 + cfg["zmax"]),
                        nu_max=NU21 / (1 + cfg["zmin"]), n_nu=cfg["n_nu"], l_box_override=cfg["l_box"],
                        do_rsd=cfg["do_rsd"]), k, pk)
    t = {}
    t0 = time.perf_counter()
    dk, _ = o.modes_mt(nthreads=orc.lib().orc_num_threads(), with_vpot=False)
    t["modes"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    dens = o.normalize(o.c2r(dk))
    t["fft_density"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    rv = o.radial_velocity_spectral(dk) if cfg["do_rsd"] else np.zeros_like(dens)
    t["velocity_3fft"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    _, s2 = o.sigma(dens)
    mass, dz = o.get_hi(dens, rv, s2)
    t["sigma_get_hi"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    o.mk_T_maps(mass, dz)
    t["mk_T_maps"] = time.perf_counter() - t0
    return t


def cpu_baseline(args):
    from oracle import orc
    orc.build()
    n_sample = args.cpu_sample
    t = cpu_pipeline(args.config, n_sample)
    tot = sum(t.values())
    return {"value": n_sample ** 3 / tot, "unit": "voxels/s", "cores": orc.lib().orc_num_threads(), "kind": "port",
            "sample": "oracle pipeline (modes, 4 FP64 c2r FFTs, sigma, get_HI, mk_T_maps) at %d^3 with the "
                      "workload's box, shells and Nside; %.1f s" % (n_sample, tot),
            "stage_s": {k: round(v, 3) for k, v in t.items()}}


def bench_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import orc
    orc.build()
    n_sample = args.cpu_sample
    for _ in range(args.warmup):
        cpu_pipeline(args.config, 32)
    times = []
    for _ in range(args.steps):
        t = cpu_pipeline(args.config, n_sample)
        times.append(sum(t.values()))
    tot = sum(times)
    value = n_sample ** 3 * args.steps / tot
    cores = orc.lib().orc_num_threads()
    cfg = CONFIGS[args.config]
    line = {"impl": "reference", "metric": "GetHI %d^3 realisation throughput (voxels/s), FP32 FFT path"
            % cfg["n_grid"], "value": value, "unit": "voxels/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp64 (FFT), fp32 grids", "data": "synthetic",
            "config": {"workload": args.config, "sample_n_grid": n_sample},
            "cpu_baseline": {"value": value, "unit": "voxels/s", "cores": cores, "kind": "port",
                             "sample": "oracle pipeline at %d^3 per step with the workload's box, shells and "
                                       "Nside (the reference does not build on this host without its libraries; "
                                       "the oracle is its C restatement, pinned bit-exact against it)" % n_sample},
            "e2e": {"value": value, "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=sorted(CONFIGS) + ["c3", "joint"])
    ap.add_argument("--cpu-sample", type=int, default=256)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--joint-nside", type=int, default=0, help="joint: Nside (default 512; smaller for profiling)")
    ap.add_argument("--joint-nnu", type=int, default=0, help="joint: channels (default 150)")
    ap.add_argument("--no-fft-compare", action="store_true",
                    help="skip the tensor-core split-precision FFT comparison (1024^3 workloads)")
    args = ap.parse_args()
    if args.impl == "reference":
        bench_reference(args)
    elif args.config == "c3":
        bench_ensemble(args)
    elif args.config == "joint":
        bench_joint(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
