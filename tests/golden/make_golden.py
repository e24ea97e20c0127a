"""Generate the golden fixtures of tests/golden/ from the reference's own
hot-path sources, compiled from the reference tree against the project's
MKL/FFTW shims by `make -C oracle ref` (needs the reference checkout).

Fixtures (all small):
  fdm_matrix_n4.txt     the exact 16x16 matrix golden of src/tests/fdm_matrix.cpp:47-64
  strings_*.npz         theta snapshots and the reference's cores2/cores3 masks
  step_*.npz            thermal initial state and the reference's state after 1 / 10
                        vvsl_field_rescaled steps
  pk_*.npz              output_powerspec of a stepped field

The reference's random numbers come from the shim (Philox + Box-Muller), not
MKL, so the initial states pin the restatement of init.cpp's arithmetic, not
MKL's bitstream.

Usage: python tests/golden/make_golden.py  (from the repository root)
"""
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))
import oracle_lib  # noqa: E402
from strings_util import accept_value, near_threshold_theta, num_cores2_ascending  # noqa: E402

REF_SRC = os.environ.get("REF_SRC", "/root/reference/src")


def fdm_matrix():
    text = open(os.path.join(REF_SRC, "tests", "fdm_matrix.cpp")).read()
    body = re.search(r"correct_matrix\[\]\s*=\s*\{(.*?)\};", text, re.S).group(1)
    vals = [int(v) for v in re.findall(r"-?\d+", body)]
    assert len(vals) == 256
    np.savetxt(os.path.join(HERE, "fdm_matrix_n4.txt"), np.array(vals).reshape(16, 16), fmt="%d")


def strings(ref):
    rng = np.random.default_rng(20240601)
    for nd, N, thr in [(2, 64, 1), (3, 16, 1), (3, 16, 30)]:
        p = oracle_lib.make_params(NDIMS=nd, N=N, thr=thr)
        for kind in ("uniform", "near"):
            if kind == "uniform":
                theta = rng.uniform(-np.pi, np.pi, (N,) * nd)
            else:
                theta = near_threshold_theta(rng, nd, N, accept_value(thr))
            n, pos = ref.cores(p, theta)
            if nd == 2:
                offs = pos[:, 0] + N * pos[:, 1]
            else:
                offs = (pos[:, 0].astype(np.int64) * N + pos[:, 1]) * N + pos[:, 2]
            mask = np.zeros(theta.size, dtype=np.uint8)
            mask[offs] = 1
            extra = {}
            if nd == 2:
                extra["num_cores_serial"] = num_cores2_ascending(N, offs)
            np.savez_compressed(os.path.join(HERE, "strings_%dd%d_thr%d_%s.npz" % (nd, N, thr, kind)),
                                nd=nd, N=N, thr=thr, theta=theta, n=n, mask_bits=np.packbits(mask), **extra)


def steps(ref):
    for nd, N, seed, lam, T0 in [(2, 32, 5, 1.0, 4.0), (3, 16, 6, 1.0, 4.0)]:
        p = oracle_lib.make_params(NDIMS=nd, N=N, lam=lam, T0=T0, dx=0.5, dt=0.1)
        f0 = ref.gaussian_thermal(p, seed)
        f1 = ref.evolve(p, *f0, 1)
        f10 = ref.evolve(p, *f0, 10)
        np.savez_compressed(os.path.join(HERE, "step_%dd%d.npz" % (nd, N)), nd=nd, N=N, seed=seed, lam=lam, T0=T0,
                            dx=0.5, dt=0.1, s0=np.stack(f0), s1=np.stack(f1[:4]), s10=np.stack(f10[:4]),
                            tau1=f1[4], tau10=f10[4])
        pk, ks, cnt = ref.powerspec(p, f10[1])
        np.savez_compressed(os.path.join(HERE, "pk_%dd%d.npz" % (nd, N)), pk=pk, ks=ks, count=cnt)


def main():
    if not os.path.isdir(REF_SRC):
        raise SystemExit("reference sources not found at " + REF_SRC)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "REF_SRC=" + REF_SRC], check=True)
    ref = oracle_lib.load_ref(64)
    fdm_matrix()
    strings(ref)
    steps(ref)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
