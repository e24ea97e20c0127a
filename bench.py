"""Benchmark of the standard-lattice evolution path on GB300.

Metric: lattice site-updates per second of the fused leapfrog step (one step
of one site: psi1, psi2, pi1, pi2 read and written once), with the fraction
of the measured HBM copy bandwidth it represents.

Headline workload: 3D N=1024^3, FP32 fields (FP64 time bookkeeping),
7-point stencil, lambda=1, dx=0.5, dt=0.1, the reference's PRS step (prs=1,
T0=0: coupling lambda/tau^2, stable at every tau; the unrescaled coupling,
prs=0, runs the same kernels at the same speed but its radial mode outgrows
dt = 0.1 past tau ~ 13, within a 200-step timed region), flat k_cut=1
Gaussian start (seed 1). The state (2 x 8.6 GB
psi buffers + 8.6 GB pi) is far larger than L2 (129 MB), so every step
streams from HBM; no L2 flush is needed between steps.

Also reported (extra keys): the plain FP64 step on the same lattice and
start, the 96-member uneven batched ensemble (with the kernel its tuner
kept), the reference CPU path, and the wall time of the per-output analysis
calls on the headline lattice (`analysis_ms`: string finder, 128-bin axion
spectrum, background means, energies) and on the ensemble.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

For N > 1 (torchrun), each rank runs an independent replica on its own GPU
(the single lattice does not shard without a halo exchange per step) and rank 0 prints
the aggregate.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "axion-strings_gb300")

N_MAIN = 1024
# per site and pass of the step kernel: psi1, psi2, pi1, pi2 read once and
# written once; a two-step pass (halo depth 2) advances every site twice
BYTES_PER_SITE = {32: 32, 64: 64}
ENSEMBLE_SIZES = (64, 96, 128, 160, 192)
# The end-to-end leg runs one output interval of the reference's run loop:
# strings are searched every 20 steps (s_run.cpp cadence), so a user's host
# round trip covers 20 steps whatever --steps times on the device.
E2E_STEPS = 20


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "of measured"
    except Exception:
        return 6800.0, "of fallback"


# --------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------- dist
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


# --------------------------------------------------------------------- CPU baseline
# What the CPU legs time, and how it compares with the reference's own code
# (oracle/cpu_calibration.py on an 8-core x86 host, 256^3: 1.6-1.9x the
# reference's FP64 step compiled from its sources with the project's COO SpMV
# in place of MKL; the direct-stencil port was 0.73-0.81x).
CPU_KIND = ("oracle port of vvsl_field_rescaled in the reference's six passes, Laplacian as a sparse "
            "matrix-vector product over build_coefficient_matrix's matrix (CSR), float data_t, OpenMP")
CPU_CALIBRATION = ("1.6-1.9x the reference's own FP64 step built from its sources with the project's SpMV shim "
                   "(8-core x86, 256^3; profiles/cpu_baseline_calibration.md)")


def cpu_port_rate(n=256, target_s=10.0, max_steps=200, min_steps=2):
    """The oracle's timing port of vvsl_field_rescaled (the reference's six
    passes, its Laplacian as a sparse matrix-vector product, FP32 data_t,
    OpenMP on all host cores) on an n^3 sample; site-updates/s."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    orc = oracle_lib.load()
    p = oracle_lib.make_params(NDIMS=3, N=n, lam=1.0, T0=0.0, dx=0.5, dt=0.1, prs=1)
    rng = np.random.default_rng(1)
    f = [rng.standard_normal((n, n, n)).astype(np.float32) * 0.5 for _ in range(2)] + \
        [np.zeros((n, n, n), dtype=np.float32) for _ in range(2)]
    k = [np.zeros((n, n, n), dtype=np.float32) for _ in range(4)]
    t = ctypes.c_float(1.0)
    ptr = [a.ctypes.data for a in f + k]
    A = orc.lib.orc_csr_build(ctypes.byref(p))     # build_coefficient_matrix: once, not timed
    if not A:
        raise MemoryError("CPU leg: no memory for the %d^3 sparse matrix" % n)
    step = lambda: orc.lib.orc_ref_step_f32(ctypes.byref(p), A, *ptr, ctypes.byref(t))
    try:
        step()
        t0 = time.perf_counter()
        step()
        one = time.perf_counter() - t0
        steps = int(max(min_steps, min(max_steps, target_s / max(one, 1e-6))))
        t0 = time.perf_counter()
        for _ in range(steps):
            step()
        dt = time.perf_counter() - t0
    finally:
        orc.lib.orc_csr_free(A)
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return n ** 3 * steps / dt, steps, dt, threads


# --------------------------------------------------------------------- GPU legs
def load_axs():
    sys.path.insert(0, PKG)
    if not os.path.exists(os.path.join(PKG, "libaxs.so")):
        sys.path.insert(0, ROOT)
        import __graft_entry__
        __graft_entry__.build()
    import axs
    return axs


def main_params(axs, precision, n, stencil=0):
    return axs.default_params(NDIMS=3, N=n, lambda_=1.0, T_initial=0.0, space_step=0.5, time_step=0.1,
                              precision=precision, prs=1, thr=1, stencil_setting=stencil)


def run_lattice(axs, dist, precision, steps, warmup, with_e2e, sampler=None, n=N_MAIN, stencil=0):
    p = main_params(axs, precision, n, stencil)
    L = axs.Lattice(p)
    L.init_flat(1, 1.0)
    L.evolve(warmup)                       # includes autotuning (dt = 0 trials) and graph capture
    L.evolve_timed(steps)                  # captures the graph for `steps`
    dist.barrier()
    if sampler:
        sampler.start()
    launches0 = axs.kernel_launches()
    ms = L.evolve_timed(steps)             # CUDA events on the lattice's stream, synchronised
    launches = axs.kernel_launches() - launches0
    clocks = sampler.stop() if sampler else None
    dist.barrier()
    ms_max = dist.max(ms)
    rec = {"ms": ms_max, "launches": launches, "desc": L.describe(), "clocks": clocks,
           "sites": p.N ** 3, "finite": L.check_finite()}
    # per-output analysis on the same lattice (wall time of the synchronising calls)
    L.find_strings()
    t0 = time.perf_counter()
    for _ in range(3):
        L.find_strings()
    t_str = (time.perf_counter() - t0) / 3
    L.axion_spectrum(128)
    t0 = time.perf_counter()
    L.axion_spectrum(128)
    t_spec = time.perf_counter() - t0
    rec["analysis_ms"] = {"find_strings": 1e3 * t_str, "axion_spectrum_128": 1e3 * t_spec}
    for name, fn in (("background", L.background), ("energies", L.energies)):
        fn()
        t0 = time.perf_counter()
        for _ in range(3):
            fn()
        rec["analysis_ms"][name] = 1e3 * (time.perf_counter() - t0) / 3
    if with_e2e:
        rec["e2e"] = e2e_leg(axs, L, dist, E2E_STEPS)
    L.close()
    return rec


def e2e_leg(axs, L, dist, steps):
    """The user's call sequence with host buffers, one output interval: upload
    the state from pinned host memory, evolve `steps` steps through
    axs_evolve, read the interval's result (the string count) and psi back to
    pinned host memory. Two untimed rehearsals first: a production run repeats
    the interval, so its CUDA graphs (one per buffer parity) are already
    captured when the timed one runs."""
    shape = L.shape
    ins = [axs.PinnedBuffer(shape, np.float32) for _ in range(4)]
    outs = [axs.PinnedBuffer(shape, np.float32) for _ in range(2)]
    f = L.download(dtype=np.float32)
    for b, a in zip(ins, f):
        b.array[...] = a
    del f

    split = {}

    def interval():
        # upload, find_strings and download return after their stream has
        # synchronised, so the split points cost no extra synchronisation
        t = time.perf_counter()
        L.upload(*[b.array for b in ins], dtype=np.float32)
        t1 = time.perf_counter()
        L.evolve(steps)
        n, _, _ = L.find_strings()
        t2 = time.perf_counter()
        axs._check(axs._lib.axs_download_f32(L._h, outs[0].array.ctypes.data, outs[1].array.ctypes.data, None, None))
        t3 = time.perf_counter()
        split.update(upload_s=t1 - t, evolve_and_strings_s=t2 - t1, download_s=t3 - t2)
        return n

    for _ in range(2):
        interval()
    dist.barrier()
    t0 = time.perf_counter()
    n = interval()
    wall = time.perf_counter() - t0
    dist.barrier()
    wall = dist.max(wall)
    for b in ins + outs:
        b.free()
    sites = L.length
    h2d = 4 * 4 * sites
    d2h = 2 * 4 * sites + 16
    return {"wall_s": wall, "h2d_bytes_per_step": h2d / steps, "d2h_bytes_per_step": d2h / steps,
            "string_count": int(n), "site_updates_per_s": sites * steps / wall,
            "split_s": {k: round(v, 6) for k, v in split.items()},
            "h2d_gbs": h2d / split["upload_s"] / 1e9, "d2h_gbs": d2h / split["download_s"] / 1e9}


def ensemble_shard(n_total, rank, world):
    """Realisations owned by `rank`: round-robin, disjoint, covering all."""
    return [i for i in range(n_total) if i % world == rank]


def run_ensemble(axs, dist, steps, warmup, master_seed=2026):
    rng = np.random.default_rng(master_seed)
    n_total = 96
    mine = ensemble_shard(n_total, dist.rank, dist.world)   # no data-path collective between ranks
    sizes = rng.choice(ENSEMBLE_SIZES, size=n_total)
    lams = np.exp(rng.uniform(np.log(0.5), np.log(4.0), size=n_total))
    seeds = rng.integers(1, 2 ** 31, size=n_total)
    plist = [axs.default_params(NDIMS=3, N=int(sizes[i]), lambda_=float(lams[i]), T_initial=0.0, space_step=0.5,
                                time_step=0.1, precision=32, prs=1, thr=1) for i in mine]
    E = axs.Ensemble(plist)
    for m, i in zip(E.members, mine):
        m.init_flat(int(seeds[i]), 1.0)
    E.evolve(warmup)
    E.evolve_timed(steps)
    dist.barrier()
    l0 = axs.kernel_launches()
    ms = E.evolve_timed(steps)
    launches = axs.kernel_launches() - l0
    dist.barrier()
    sites = sum(int(p.N) ** 3 for p in plist)
    sites_all = dist.sum(sites)
    ms_max = dist.max(ms)
    # per-output analysis of every member, batched (wall time of the
    # synchronising calls; the first call of a binning plans the transforms)
    E.find_strings()
    E.axion_spectrum(128)
    t0 = time.perf_counter()
    E.find_strings()
    t1 = time.perf_counter()
    E.axion_spectrum(128)
    t2 = time.perf_counter()
    desc = E.describe()
    E.close()
    return {"members": n_total, "sites": int(sites_all), "ms": ms_max, "launches": launches, "desc": desc,
            "sizes": [int(s) for s in sizes], "master_seed": master_seed,
            "analysis_ms": {"find_strings_all_members": 1e3 * (t1 - t0), "axion_spectrum_128_all_members": 1e3 * (t2 - t1)}}


# --------------------------------------------------------------------- arms
def workload_name(n, precision, stencil=0):
    """The workload both arms measure (the reference arm on a sample of it)."""
    return ("3D %d^3 FP%d leapfrog step, %d-point stencil, prs=1, lambda=1, dx=0.5, dt=0.1, flat k_cut=1 start"
            % (n, precision, 1 + 6 * (stencil + 1)))


def reference_arm(args, dist):
    """The reference's CPU path on the host cores: the oracle's port of
    vvsl_field_rescaled in the reference's structure (the reference's own
    sources are not on the GPU machines, so oracle/_ref cannot be built
    there)."""
    if dist.rank != 0:
        return
    n = 256
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    # about 10 s of CPU work (up to 600 steps of the 256^3 sample)
    rate, steps_done, secs, threads = cpu_port_rate(n=n, target_s=10.0, max_steps=600)
    line = {"metric": "site-updates/s", "value": rate, "unit": "site-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * n ** 3 / rate,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": workload_name(args.n, 32), "N": args.n, "precision": "fp32 fields",
                       "sample": "%d^3 lattice, %d steps" % (n, steps_done)},
            "cpu_baseline": {"value": rate, "unit": "site-updates/s", "cores": threads, "kind": "port",
                             "sample": "%d^3 FP32, %d steps (%.1f s)" % (n, steps_done, secs),
                             "code": CPU_KIND, "calibration": CPU_CALIBRATION},
            "e2e": {"value": rate, "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def gpu_arm(args, dist):
    axs = load_axs()
    axs.set_device(dist.local)
    hbm, peak_note = peaks()
    sampler = ClockSampler(dist.local)
    main = run_lattice(axs, dist, args.precision, args.steps, args.warmup, with_e2e=not args.no_e2e, sampler=sampler,
                       n=args.n, stencil=args.stencil)
    sites_all = dist.sum(main["sites"])
    value = sites_all * args.steps / (main["ms"] * 1e-3)
    launches = max(1, main["launches"])
    # steps per launch: 3 or 2 for the multi-step kernels (an interval's last
    # one or two steps run on their partners, each pass moving the same bytes)
    steps_per_launch = args.steps / launches
    per_launch_ms = main["ms"] / launches
    achieved = BYTES_PER_SITE[args.precision] * main["sites"] / (per_launch_ms * 1e-3) / 1e9
    two_step = "two steps per pass" in main["desc"]
    three_step = "three steps per pass" in main["desc"]
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "k_zmarch_traffic.txt")
    if three_step:
        tkey = "zmarch_3step_fp32_1024_per_launch_bytes:"
    elif two_step:
        tkey = ("zmarch_2step_lean_fp32_1024_per_launch_bytes:" if "lean" in main["desc"] else
                "zmarch_2step_fp32_1024_per_launch_bytes:")
    else:
        tkey = "zmarch_fp32_1024_per_launch_bytes:"
    if args.precision == 32 and args.n == N_MAIN and args.stencil == 0 and os.path.exists(tfile):
        for line in open(tfile):
            if line.startswith(tkey):
                traffic = float(line.split(":", 1)[1]) / 1e9     # GB per launch, like `achieved`'s bytes
    fp64 = ens = None
    if not args.quick:
        f64 = run_lattice(axs, dist, 64, max(3, args.steps // 2), args.warmup, with_e2e=False, n=args.n)
        r64 = dist.sum(f64["sites"]) * max(3, args.steps // 2) / (f64["ms"] * 1e-3)
        fp64 = {"value": r64, "unit": "site-updates/s", "ms_per_step": f64["ms"] / max(3, args.steps // 2),
                "hbm_frac": r64 / dist.world * 64 * f64["launches"] / max(3, args.steps // 2) / 1e9 / hbm,
                "kernel": f64["desc"],
                "fp32_over_fp64": value / r64}
        e = run_ensemble(axs, dist, args.steps, args.warmup)
        re = e["sites"] * args.steps / (e["ms"] * 1e-3)
        ens = {"value": re, "unit": "site-updates/s", "members": e["members"], "sites": e["sites"],
               "ms_per_step": e["ms"] / args.steps,
               "hbm_frac": re / dist.world * 32 * e["launches"] / args.steps / 1e9 / hbm,
               "master_seed": e["master_seed"], "launches_per_step": e["launches"] / args.steps, "kernel": e["desc"],
               "analysis_ms": e["analysis_ms"]}
    cpu = None
    if dist.rank == 0 and not args.no_cpu:
        rate, steps_done, secs, threads = cpu_port_rate(n=256, target_s=10.0, max_steps=600)
        cpu = {"value": rate, "unit": "site-updates/s", "cores": threads, "kind": "port",
               "sample": "256^3 FP32, %d steps (%.1f s)" % (steps_done, secs),
               "code": CPU_KIND, "calibration": CPU_CALIBRATION}
    e2e = main.get("e2e")
    e2e_line = None
    if e2e:
        e2e_line = {"value": sites_all * E2E_STEPS / e2e["wall_s"],      # wall_s is already the max over ranks
                    "unit": "site-updates/s", "h2d_bytes_per_step": e2e["h2d_bytes_per_step"],
                    "d2h_bytes_per_step": e2e["d2h_bytes_per_step"], "wall_s": e2e["wall_s"],
                    "steps": E2E_STEPS, "split_s": e2e["split_s"],   # rank 0's upload / evolve + strings / download
                    "h2d_gbs": e2e["h2d_gbs"], "d2h_gbs": e2e["d2h_gbs"]}
    if dist.rank != 0:
        return
    # state held on the device: two psi buffers, pi and the spare (complex)
    state_bytes = 4 * 2 * (args.precision // 8) * main["sites"]
    big = state_bytes > 129e6
    l2_note = ("state %.3g GB %s 129 MB L2: %s" %
               (state_bytes / 1e9, ">" if big else "<=",
                "every pass streams from HBM, no flush needed" if big else
                "the state fits in L2; figures are L2-resident, not HBM"))
    # 32 B (FP32) per site-update is the algorithmic minimum of one step per
    # pass; a two-step pass moves those bytes once for two site-updates
    per_step_achieved = BYTES_PER_SITE[args.precision] * value / dist.world / 1e9
    line = {
        "metric": "site-updates/s", "value": value, "unit": "site-updates/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": main["ms"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == 32 else "f64", "data": "synthetic",
        "config": {"workload": workload_name(args.n, args.precision, args.stencil),
                   "N": args.n, "precision": "fp32 fields, fp64 tau",
                   "parallelism": "replicas" if dist.world > 1 else "single",
                   "l2": l2_note, "kernel": main["desc"]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "frac_per_pass": achieved / hbm,
                     "effective_bytes_per_step_frac": per_step_achieved / hbm,
                     "effective_note": ("%d B per site-update (one step per pass) x site-updates/s over the peak; "
                                        "above 1 because the kernel takes %g steps per pass (temporal blocking), "
                                        "bit-identical to one-step passes" % (BYTES_PER_SITE[args.precision],
                                                                               steps_per_launch))
                                       if steps_per_launch > 1 else "one step per pass: equals frac_per_pass",
                     "traffic": traffic, "traffic_unit": "GB per launch (ncu dram read+write)",
                     "traffic_source": ("profiles/k_zmarch_traffic.txt: dram__bytes_read.sum + dram__bytes_write.sum "
                                        "of this kernel in an ncu launch list of this bench command")
                                       if traffic else None,
                     "algorithmic_gb_per_launch": BYTES_PER_SITE[args.precision] * main["sites"] / 1e9,
                     "peak_source": peak_note,
                     "algorithmic_bytes_per_site_update": BYTES_PER_SITE[args.precision] / steps_per_launch,
                     "steps_per_launch": steps_per_launch, "ms_per_launch": per_launch_ms},
        "cpu_baseline": cpu,
        "e2e": e2e_line,
        "gpu_launches": main["launches"],
        "analysis_ms": main.get("analysis_ms"),
        "state_finite": bool(main.get("finite")),   # no NaN/Inf in the fields after the timed steps
        "clocks": main["clocks"],
        "fp64": fp64,
        "ensemble": ens,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="axs", choices=["axs", "reference"])
    ap.add_argument("--quick", action="store_true", help="headline only (no FP64 / ensemble legs)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer end-to-end leg")
    ap.add_argument("--n", type=int, default=N_MAIN, help="lattice side (profiling cases use smaller N)")
    ap.add_argument("--precision", type=int, default=32, choices=[32, 64],
                    help="headline leg precision (64 only for profiling the FP64 step)")
    ap.add_argument("--stencil", type=int, default=0, choices=[0, 1, 2, 3],
                    help="stencil_setting of the headline leg (1-3, radius 2-4, only for profiling those kernels)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    dist = Dist()
    try:
        if args.impl == "reference":
            reference_arm(args, dist)
        else:
            gpu_arm(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
