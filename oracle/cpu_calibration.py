"""CPU calibration of the timed baseline: the reference's own step against the
oracle ports on the same host, same lattice, same thread count.

  ref f64   vvsl_field_rescaled of the reference's sources (oracle/_ref,
            USE_DOUBLE_PRECISION build: the reference's default), Laplacian
            by the COO matrix of build_coefficient_matrix through the project
            shim of mkl_sparse_d_mv (symmetric/upper, expanded to CSR)
  ref f32   the same sources built with data_t = float
  port f64  orc_vvsl_step: the reference's six passes, direct stencil
  port f32  orc_vvsl_step_f32: the same in float
  port f32 sparse   orc_ref_step_f32: float, the six passes with the
            Laplacian as a sparse matrix-vector product over the same matrix
            (the benchmark's CPU legs)

Needs oracle/_ref (built next to a reference checkout). Prints a Markdown
table of site-updates/s and the ratios. Test infrastructure: nothing in the
product runs this.

    OMP_NUM_THREADS=8 python oracle/cpu_calibration.py [--n 256] [--steps 10]
"""
import argparse
import ctypes
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "tests"))
import oracle_lib  # noqa: E402


def _state(n, dtype):
    rng = np.random.default_rng(1)
    return [rng.standard_normal((n, n, n)).astype(dtype) * 0.5 for _ in range(2)] + \
        [np.zeros((n, n, n), dtype=dtype) for _ in range(2)]


def time_ref(precision, n, steps):
    ref = oracle_lib.load_ref(precision)
    if ref is None:
        return None
    p = oracle_lib.make_params(NDIMS=3, N=n, T0=0.0, dx=0.5, dt=0.1)

    class P:
        pass
    q = P()
    for k, v in dict(NDIMS=3, N=n, lambda_=1.0, T_initial=0.0, space_step=0.5, time_step=0.1,
                     stencil_setting=0, thr=1).items():
        setattr(q, k, v)
    ref.set_params(q)
    f = _state(n, ref.dtype)
    k = [np.zeros_like(f[0]) for _ in range(4)]
    ptr = [a.ctypes.data for a in f + k]
    ref.lib.ref_steps(*ptr, 1)          # builds the COO matrix (serial, not timed) and warms up
    t0 = time.perf_counter()
    ref.lib.ref_steps(*ptr, steps)
    return n ** 3 * steps / (time.perf_counter() - t0)


def time_port(precision, n, steps, sparse=False):
    orc = oracle_lib.load()
    p = oracle_lib.make_params(NDIMS=3, N=n, T0=0.0, dx=0.5, dt=0.1)
    dt = np.float64 if precision == 64 else np.float32
    f = _state(n, dt)
    k = [np.zeros_like(f[0]) for _ in range(4)]
    ptr = [a.ctypes.data for a in f + k]
    A = None
    if sparse:
        A = orc.lib.orc_csr_build(ctypes.byref(p))
        t = ctypes.c_float(1.0)
        step = lambda: orc.lib.orc_ref_step_f32(ctypes.byref(p), A, *ptr, ctypes.byref(t))
    elif precision == 64:
        t = ctypes.c_double(1.0)
        step = lambda: orc.lib.orc_vvsl_step(ctypes.byref(p), *ptr, ctypes.byref(t))
    else:
        t = ctypes.c_float(1.0)
        step = lambda: orc.lib.orc_vvsl_step_f32(ctypes.byref(p), *ptr, ctypes.byref(t))
    step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    rate = n ** 3 * steps / (time.perf_counter() - t0)
    if A:
        orc.lib.orc_csr_free(A)
    return rate


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--steps", type=int, default=10)
    args = ap.parse_args()
    threads = os.environ.get("OMP_NUM_THREADS", str(os.cpu_count()))
    r = {"ref f64": time_ref(64, args.n, args.steps), "ref f32": time_ref(32, args.n, args.steps),
         "port f64": time_port(64, args.n, args.steps), "port f32": time_port(32, args.n, args.steps),
         "port f32 sparse": time_port(32, args.n, args.steps, sparse=True)}
    print("host: %s, %s cores, OMP_NUM_THREADS=%s; %d^3 lattice, %d timed steps after one warm-up step"
          % (platform.processor() or platform.machine(), os.cpu_count(), threads, args.n, args.steps))
    print()
    print("| code | site-updates/s | / ref f64 |")
    print("|---|---|---|")
    base = r["ref f64"]
    for name, v in r.items():
        if v is None:
            print("| %s | not built | — |" % name)
        else:
            print("| %s | %.3g | %s |" % (name, v, "%.2f" % (v / base) if base else "—"))


if __name__ == "__main__":
    main()
