"""Production-shape run and its statistical check.

  A. 3D N^3 FP32 lattice (default 1536^3, ~116 GB of device state), PRS
     equation, lambda = 1, dx = 0.5, dt = 0.1, flat k_cut = 1 start, to
     tau_end = N dx / 2; string count (xi) every `--strings-every` steps and
     the axion kinetic-energy spectrum (`--bins` log bins) every
     `--spectra-every` steps.
  B. `--seeds` FP64 runs at `--ref-n`^3 (default 8 x 512^3) with the same
     physics and cadences.
  C. Check: over the common tau range, the fraction of xi(tau) samples of A
     within 2 and 3 standard errors of the mean of B, and the spectrum shape
     (A interpolated in log k onto B's bins, both normalised by their total)
     against B's seed scatter.

Prints one JSON object (per-sample series included). Usage (on a GPU):
    python axion-strings_gb300/production_run.py [--n 1536] [--ref-n 512] [--seeds 8]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import axs  # noqa: E402


def final_step(n, dx=0.5, dt=0.1):   # s_run.cpp:82 with physics.cpp:29 in float
    lct = np.float32(0.5) * np.float32(n) * np.float32(dx)
    return int(round(float(lct / np.float32(dt))) - round(float(np.float32(dx) / np.float32(dt))) + 1)


def run(n, precision, seed, strings_every, spectra_every, bins):
    p = axs.default_params(NDIMS=3, N=n, lambda_=1.0, T_initial=0.0, space_step=0.5, time_step=0.1,
                           precision=precision, prs=1, thr=1)
    L = axs.Lattice(p)
    t0 = time.time()
    L.init_flat(seed, 1.0)
    t_init = time.time() - t0
    fs = final_step(n)
    xi, spec = [], []
    t = 0
    t_evolve = t_strings = t_spec = 0.0
    while True:
        tau, _ = L.time
        if t % strings_every == 0:
            a = time.time()
            nplaq, ncores, _ = L.find_strings()
            t_strings += time.time() - a
            xi.append((t, tau, int(nplaq), axs.xi(p, nplaq, ncores, tau)))
        if t % spectra_every == 0 and t > 0:
            a = time.time()
            k, pk, cnt = L.axion_spectrum(bins)
            t_spec += time.time() - a
            spec.append((t, tau, k.tolist(), pk.tolist(), cnt.tolist()))
        if t >= fs:
            break
        nxt = min(fs, (t // strings_every + 1) * strings_every)
        a = time.time()
        L.evolve(nxt - t)
        L.time   # host bookkeeping only; evolve is asynchronous
        t_evolve += time.time() - a
        t = nxt
    finite = L.check_finite()
    L.close()
    return {"N": n, "precision": precision, "seed": seed, "final_step": fs, "finite": finite,
            "seconds": {"init": t_init, "evolve_and_sync": t_evolve, "strings": t_strings, "spectra": t_spec},
            "xi": xi, "spectra": spec}


def compare(big, refs):
    ref_xi = {}
    for r in refs:
        for (t, tau, n, x) in r["xi"]:
            ref_xi.setdefault(round(tau, 6), []).append(x)
    within2 = within3 = total = 0
    rows = []
    for (t, tau, n, x) in big["xi"]:
        v = ref_xi.get(round(tau, 6))
        if not v or len(v) < 2:
            continue
        m, se = float(np.mean(v)), float(np.std(v, ddof=1) / np.sqrt(len(v)))
        if m <= 0:
            continue
        total += 1
        z = abs(x - m) / se if se > 0 else (0.0 if x == m else np.inf)
        within2 += z <= 2
        within3 += z <= 3
        rows.append({"tau": tau, "xi_big": x, "xi_ref_mean": m, "xi_ref_se": se, "z": z})
    spec_rows = []
    ref_spec = {}
    for r in refs:
        for (t, tau, k, pk, cnt) in r["spectra"]:
            ref_spec.setdefault(round(tau, 6), []).append((np.array(k), np.array(pk), np.array(cnt)))
    for (t, tau, k, pk, cnt) in big["spectra"]:
        v = ref_spec.get(round(tau, 6))
        if not v:
            continue
        kb, pkb = np.array(k), np.array(pk)
        okb = (np.array(cnt) > 0) & (pkb > 0)
        kr = v[0][0]
        okr = np.all([(c > 0) & (p > 0) for (_, p, c) in v], axis=0)
        sel = okr & (kr >= kb[okb].min()) & (kr <= kb[okb].max())
        if sel.sum() < 4:
            continue
        shape_big = np.exp(np.interp(np.log(kr[sel]), np.log(kb[okb]), np.log(pkb[okb])))
        shape_big /= shape_big.sum()
        refs_n = np.array([p[sel] / p[sel].sum() for (_, p, _) in v])
        m = refs_n.mean(axis=0)
        sd = refs_n.std(axis=0, ddof=1) if len(v) > 1 else np.zeros_like(m)
        z = np.abs(shape_big - m) / np.where(sd > 0, sd, np.inf)
        spec_rows.append({"tau": tau, "bins": int(sel.sum()), "frac_within_2sd": float(np.mean(z <= 2)),
                          "frac_within_3sd": float(np.mean(z <= 3)), "max_rel_dev": float(np.max(np.abs(shape_big - m) / m))})
    return {"xi_samples_compared": total, "xi_frac_within_2se": within2 / total if total else None,
            "xi_frac_within_3se": within3 / total if total else None, "xi_rows": rows, "spectrum_shape": spec_rows}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1536)
    ap.add_argument("--ref-n", type=int, default=512)
    ap.add_argument("--seeds", type=int, default=8)
    ap.add_argument("--strings-every", type=int, default=10)
    ap.add_argument("--spectra-every", type=int, default=100)
    ap.add_argument("--bins", type=int, default=256)
    args = ap.parse_args()
    big = run(args.n, 32, 1, args.strings_every, args.spectra_every, args.bins)
    refs = [run(args.ref_n, 64, 100 + s, args.strings_every, args.spectra_every, args.bins) for s in range(args.seeds)]
    out = {"big": {k: v for k, v in big.items() if k not in ("spectra",)},
           "refs": [{k: v for k, v in r.items() if k not in ("spectra", "xi")} for r in refs],
           "check": compare(big, refs)}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
