"""ctypes binding of the CPU oracle (oracle/liboracle.so) and, where it was
built, of the reference's own sources compiled against the project's MKL/FFTW
shims (oracle/_ref/libaxsref_*.so). Test infrastructure only."""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
REF_DIR = os.path.join(ORACLE_DIR, "_ref")


def reference_checkout():
    """The reference checkout's root folder, or None where there is none:
    $AXS_REFERENCE_DIR when set, else a folder named `reference` beside this
    repository (the layout of the development container; the GPU machines
    have no checkout)."""
    d = os.environ.get("AXS_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")
    return d if os.path.isdir(os.path.join(d, "src")) else None

_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)


class OrcParams(ctypes.Structure):
    _fields_ = [("NDIMS", ctypes.c_int), ("N", ctypes.c_int), ("lambda_", ctypes.c_float),
                ("T_initial", ctypes.c_float), ("space_step", ctypes.c_float), ("time_step", ctypes.c_float),
                ("stencil_setting", ctypes.c_int), ("thr", ctypes.c_int), ("prs", ctypes.c_int),
                ("laplacian", ctypes.c_int)]


def make_params(NDIMS=3, N=32, lam=1.0, T0=0.0, dx=0.5, dt=0.1, stencil=0, thr=1, prs=1, laplacian=0):
    return OrcParams(NDIMS, N, lam, T0, dx, dt, stencil, thr, prs, laplacian)


def from_axs(p):
    """OrcParams from an axs.Params."""
    return OrcParams(p.NDIMS, p.N, p.lambda_, p.T_initial, p.space_step, p.time_step, p.stencil_setting, p.thr, p.prs,
                     getattr(p, "laplacian", 0))


def _ptr(a):
    return None if a is None else a.ctypes.data


class Oracle:
    def __init__(self, lib):
        self.lib = lib
        P = ctypes.POINTER(OrcParams)
        sig = {
            "orc_fft_nd": ([_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int], None),
            "orc_normal_draw": ([ctypes.c_uint64, ctypes.c_int, ctypes.c_int64], ctypes.c_double),
            "orc_laplacian": ([P, _vp, _vp], None),
            "orc_vvsl_step": ([P, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _dp], None),
            "orc_vvsl_step_f32": ([P, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.POINTER(ctypes.c_float)], None),
            "orc_csr_build": ([P], _vp),
            "orc_csr_free": ([_vp], None),
            "orc_ref_step_f32": ([P, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.POINTER(ctypes.c_float)],
                                 None),
            "orc_vvsl_hamiltonian_step": ([P, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _dp], None),
            "orc_cores": ([P, _vp, _vp], ctypes.c_int64),
            "orc_num_cores2": ([ctypes.c_int, _vp], ctypes.c_int64),
            "orc_xi": ([P, ctypes.c_int64, ctypes.c_int64, ctypes.c_double], ctypes.c_float),
            "orc_powerspec": ([P, _vp, _vp, _vp, _vp, _vp], None),
            "orc_gaussian_thermal": ([P, ctypes.c_uint64, _vp, _vp, _vp, _vp], None),
            "orc_init_flat": ([P, ctypes.c_uint64, ctypes.c_double, _vp, _vp, _vp, _vp], None),
            "orc_background": ([P, _vp, _vp, _vp, _vp, _vp], None),
            "orc_energies": ([P, _vp, _vp, _vp, _vp, ctypes.c_double, _vp], None),
            "orc_axion_spectrum": ([P, _vp, _vp, _vp, _vp, ctypes.c_double, ctypes.c_int, _vp, _vp, _vp], None),
        }
        for name, (args, res) in sig.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = res

    @staticmethod
    def shape(p):
        return (p.N, p.N) if p.NDIMS == 2 else (p.N, p.N, p.N)

    def fftn(self, x, sign):
        a = np.ascontiguousarray(x, dtype=np.complex128).copy()
        d = (ctypes.c_int * a.ndim)(*a.shape)
        self.lib.orc_fft_nd(_ptr(a), a.ndim, d, int(sign))
        return a

    def normal(self, seed, a, m):
        return self.lib.orc_normal_draw(int(seed), int(a), int(m))

    def laplacian(self, p, phi):
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        out = np.empty_like(phi)
        self.lib.orc_laplacian(ctypes.byref(p), _ptr(phi), _ptr(out))
        return out

    def evolve(self, p, phi1, phi2, pi1, pi2, nsteps, tau=1.0, ker=None, form=0, return_ker=False):
        """Reference-structured velocity-Verlet steps (form 0: vvsl_field_rescaled,
        form 1: vvsl_hamiltonian_form); returns the new state. `ker` is the
        pair (ker1_curr, ker2_curr) to continue from (zero, as after the
        reference's calloc, when None); with return_ker the pair after the
        last step is returned too."""
        f = [np.array(a, dtype=np.float64, copy=True, order="C") for a in (phi1, phi2, pi1, pi2)]
        k = [np.zeros_like(f[0]) for _ in range(4)] if ker is None else [np.array(a, copy=True) for a in ker] + [np.zeros_like(f[0]), np.zeros_like(f[0])]
        t = ctypes.c_double(tau)
        step = self.lib.orc_vvsl_hamiltonian_step if form == 1 else self.lib.orc_vvsl_step
        for _ in range(nsteps):
            step(ctypes.byref(p), *[_ptr(a) for a in f], _ptr(k[0]), _ptr(k[1]), _ptr(k[2]), _ptr(k[3]), ctypes.byref(t))
        if return_ker:
            return f[0], f[1], f[2], f[3], t.value, (k[0], k[1])
        return f[0], f[1], f[2], f[3], t.value

    def evolve_f32(self, p, phi1, phi2, pi1, pi2, nsteps, tau=1.0):
        f = [np.array(a, dtype=np.float32, copy=True, order="C") for a in (phi1, phi2, pi1, pi2)]
        k = [np.zeros_like(f[0]) for _ in range(4)]
        t = ctypes.c_float(tau)
        for _ in range(nsteps):
            self.lib.orc_vvsl_step_f32(ctypes.byref(p), *[_ptr(a) for a in f], *[_ptr(a) for a in k], ctypes.byref(t))
        return f[0], f[1], f[2], f[3], t.value

    def cores(self, p, theta):
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        mask = np.empty(theta.shape, dtype=np.uint8)
        n = self.lib.orc_cores(ctypes.byref(p), _ptr(theta), _ptr(mask))
        return n, mask

    def num_cores2(self, N, mask):
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        return self.lib.orc_num_cores2(int(N), _ptr(mask))

    def xi(self, p, n_plaq, n_cores, tau):
        return self.lib.orc_xi(ctypes.byref(p), int(n_plaq), int(n_cores), float(tau))

    def powerspec(self, p, re, im=None):
        nb = p.N // 2
        pk, ks, cnt = np.empty(nb), np.empty(nb), np.empty(nb, dtype=np.int32)
        re = np.ascontiguousarray(re, dtype=np.float64)
        im = None if im is None else np.ascontiguousarray(im, dtype=np.float64)
        self.lib.orc_powerspec(ctypes.byref(p), _ptr(re), _ptr(im), _ptr(pk), _ptr(ks), _ptr(cnt))
        return pk, ks, cnt

    def init_thermal(self, p, seed):
        out = [np.empty(self.shape(p)) for _ in range(4)]
        self.lib.orc_gaussian_thermal(ctypes.byref(p), int(seed), *[_ptr(a) for a in out])
        return tuple(out)

    def init_flat(self, p, seed, kcut):
        out = [np.empty(self.shape(p)) for _ in range(4)]
        self.lib.orc_init_flat(ctypes.byref(p), int(seed), float(kcut), *[_ptr(a) for a in out])
        return tuple(out)

    def background(self, p, phi1, phi2, pi1, pi2):
        out = np.empty(6)
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (phi1, phi2, pi1, pi2)]
        self.lib.orc_background(ctypes.byref(p), *[_ptr(a) for a in arrs], _ptr(out))
        return out

    def energies(self, p, psi1, psi2, pi1, pi2, tau):
        out = np.empty(3)
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (psi1, psi2, pi1, pi2)]
        self.lib.orc_energies(ctypes.byref(p), *[_ptr(a) for a in arrs], float(tau), _ptr(out))
        return out

    def axion_spectrum(self, p, psi1, psi2, pi1, pi2, tau, nbins):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (psi1, psi2, pi1, pi2)]
        k, pk, cnt = np.empty(nbins), np.empty(nbins), np.empty(nbins, dtype=np.int64)
        self.lib.orc_axion_spectrum(ctypes.byref(p), *[_ptr(a) for a in arrs], float(tau), int(nbins), _ptr(k), _ptr(pk), _ptr(cnt))
        return k, pk, cnt


def build():
    """Build oracle/liboracle.so if missing or stale."""
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "liboracle.so"], check=True)


_ORACLE = None


def load():
    global _ORACLE
    if _ORACLE is None:
        build()
        _ORACLE = Oracle(ctypes.CDLL(os.path.join(ORACLE_DIR, "liboracle.so")))
    return _ORACLE


class RefLib:
    """The reference's own hot-path functions, compiled with the project shims."""

    def __init__(self, path):
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.ref_sizeof_data_t.restype = ctypes.c_int
        self.dtype = np.float64 if L.ref_sizeof_data_t() == 8 else np.float32
        L.ref_set_params.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_uint]
        L.ref_get_tau.restype = ctypes.c_double
        L.ref_set_tau.argtypes = [ctypes.c_double]
        L.ref_gaussian_thermal.argtypes = [_vp] * 4
        L.ref_steps.argtypes = [_vp] * 8 + [ctypes.c_int]
        L.ref_steps_hamiltonian.argtypes = [_vp] * 8 + [ctypes.c_int]
        L.ref_laplacian_fft.argtypes = [_vp, _vp]
        L.ref_cores.argtypes = [_vp, _vp, ctypes.c_int]
        L.ref_cores.restype = ctypes.c_int
        L.ref_powerspec.argtypes = [_vp, _vp, _vp, _vp]

    def set_params(self, p, seed=1):
        self.lib.ref_set_params(p.NDIMS, p.N, p.lambda_, p.T_initial, p.space_step, p.time_step, p.stencil_setting,
                                p.thr, seed)

    def shape(self, p):
        return (p.N, p.N) if p.NDIMS == 2 else (p.N, p.N, p.N)

    def gaussian_thermal(self, p, seed):
        self.set_params(p, seed)
        out = [np.zeros(self.shape(p), dtype=self.dtype) for _ in range(4)]
        self.lib.ref_gaussian_thermal(*[_ptr(a) for a in out])
        return tuple(out)

    def laplacian_fft(self, p, field):
        self.set_params(p)
        f = np.ascontiguousarray(field, dtype=self.dtype).copy()
        out = np.zeros_like(f)
        self.lib.ref_laplacian_fft(_ptr(out), _ptr(f))
        return out

    def evolve(self, p, phi1, phi2, pi1, pi2, nsteps, form=0):
        self.set_params(p)
        f = [np.array(a, dtype=self.dtype, copy=True, order="C") for a in (phi1, phi2, pi1, pi2)]
        k = [np.zeros_like(f[0]) for _ in range(4)]
        step = self.lib.ref_steps_hamiltonian if form == 1 else self.lib.ref_steps
        step(*[_ptr(a) for a in f + k], int(nsteps))
        return f[0], f[1], f[2], f[3], self.lib.ref_get_tau()

    def cores(self, p, theta):
        self.set_params(p)
        theta = np.ascontiguousarray(theta, dtype=self.dtype)
        cap = theta.size
        pos = np.empty((cap, p.NDIMS), dtype=np.int32)
        n = self.lib.ref_cores(_ptr(theta), _ptr(pos), cap)
        return n, pos[:n]

    def powerspec(self, p, field):
        self.set_params(p)
        nb = p.N // 2
        pk, ks, cnt = np.empty(nb), np.empty(nb), np.empty(nb, dtype=np.int32)
        f = np.ascontiguousarray(field, dtype=self.dtype)
        self.lib.ref_powerspec(_ptr(f), _ptr(pk), _ptr(ks), _ptr(cnt))
        return pk, ks, cnt


def load_ref(precision=64):
    path = os.path.join(REF_DIR, "libaxsref_f%d.so" % precision)
    if not os.path.exists(path):
        return None
    return RefLib(path)
