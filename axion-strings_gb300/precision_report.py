"""FP32 (compensated reductions) against plain FP64 on the GPU, from the same
seeded start: the errors by which the precision form is assessed.

  1. field relative error after 10 steps of the physical equation (prs = 0)
     from the flat k_cut = 1 start: ||x32 - x64|| / ||x64|| per field;
  2. xi(tau) along a full PRS run (the reference's integrator) to
     tau_end = N dx / 2, string count every `--interval` steps;
  3. the axion kinetic-energy spectrum (128 log bins) at a few times:
     per-bin relative error.

Prints one JSON object. Usage (on a GPU):
    python axion-strings_gb300/precision_report.py --n 1024 [--interval 20]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import axs  # noqa: E402


def params(n, precision, prs, lam=1.0):
    return axs.default_params(NDIMS=3, N=n, lambda_=lam, T_initial=0.0, space_step=0.5, time_step=0.1,
                              precision=precision, prs=prs, thr=1)


def field_error(n, steps=10, seed=1):
    a = axs.Lattice(params(n, 32, 0))
    b = axs.Lattice(params(n, 64, 0))
    a.init_flat(seed, 1.0)
    b.init_flat(seed, 1.0)
    a.evolve(steps)
    b.evolve(steps)
    err = axs.field_distance(a, b)
    a.close()
    b.close()
    return {"steps": steps, "equation": "physical (prs=0)", "rel_l2": dict(zip(["phi1", "phi2", "phidot1", "phidot2"],
                                                                                [float(e) for e in err]))}


def xi_run(n, interval, spec_every, seed=1, nbins=128):
    pa, pb = params(n, 32, 1), params(n, 64, 1)
    a, b = axs.Lattice(pa), axs.Lattice(pb)
    a.init_flat(seed, 1.0)
    b.init_flat(seed, 1.0)
    lct = np.float32(0.5) * np.float32(n) * np.float32(0.5)
    final_step = int(round(float(lct / np.float32(0.1))) - round(float(np.float32(0.5) / np.float32(0.1))) + 1)
    rows, spectra = [], []
    t = 0
    t0 = time.time()
    while t <= final_step:
        tau, _ = a.time
        na, ca, _ = a.find_strings()
        nb, cb, _ = b.find_strings()
        rows.append({"step": t, "tau": tau, "n32": na, "n64": nb, "xi32": axs.xi(pa, na, ca, tau),
                     "xi64": axs.xi(pb, nb, cb, tau)})
        if spec_every and (t // interval) % spec_every == 0 and t > 0:
            ka, pka, cnt = a.axion_spectrum(nbins)
            kb, pkb, _ = b.axion_spectrum(nbins)
            ok = (cnt > 0) & (pkb > 0)
            rel = np.abs(pka[ok] - pkb[ok]) / pkb[ok]
            spectra.append({"step": t, "tau": tau, "max_bin_rel_err": float(rel.max()),
                            "median_bin_rel_err": float(np.median(rel))})
        if t == final_step:
            break
        step = min(interval, final_step - t)
        a.evolve(step)
        b.evolve(step)
        t += step
    a.close()
    b.close()
    return {"equation": "PRS (prs=1)", "final_step": final_step, "interval": interval, "wall_s": time.time() - t0,
            "xi_summary": xi_summary(rows), "samples": rows, "spectra": spectra}


def xi_summary(rows):
    """xi(tau) of FP32 against FP64 over every sample with strings (n64 > 0):
    the largest relative difference and the sample it occurs at, the same
    over samples with n64 >= 1000, and the plaquette-count differences in
    units of sqrt(n64) (the Poisson scatter of a count, to judge whether a
    large relative difference at a low count is more than one or two cells)."""
    def rel(r):
        return abs(r["xi32"] - r["xi64"]) / r["xi64"]
    live = [r for r in rows if r["n64"] > 0]
    big = [r for r in live if r["n64"] >= 1000]
    worst = max(live, key=rel, default=None)
    return {
        "samples_with_strings": len(live),
        "samples_identical_count": sum(r["n32"] == r["n64"] for r in live),
        "xi_max_rel_diff": rel(worst) if worst else None,
        "xi_worst_sample": worst,
        "xi_max_rel_diff_where_n64>=1000": max((rel(r) for r in big), default=None),
        "count_max_abs_diff": max((abs(r["n32"] - r["n64"]) for r in live), default=None),
        "count_max_diff_over_sqrt_n64": max((abs(r["n32"] - r["n64"]) / np.sqrt(r["n64"]) for r in live), default=None),
        "samples_within_1pct": sum(rel(r) <= 0.01 for r in live),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--interval", type=int, default=20)
    ap.add_argument("--spec-every", type=int, default=25, help="spectrum every this many string intervals")
    ap.add_argument("--no-xi", action="store_true")
    args = ap.parse_args()
    out = {"N": args.n, "field_error_10_steps": field_error(args.n)}
    if not args.no_xi:
        out["xi_run"] = xi_run(args.n, args.interval, args.spec_every)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
