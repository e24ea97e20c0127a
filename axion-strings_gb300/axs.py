"""Python mirror of the C ABI in include/axs.h (ctypes over libaxs.so).

The reference drives its hot path from C++ (src/standard/s_run.cpp); this
module exposes the same operations to Python for tests, benches and notebooks:
one Lattice per GPU-resident lattice, numpy arrays in the reference's layout
(2D: a[j, i] = phi(i, j), i fastest; 3D: a[i, j, k], k fastest).

There is no fallback: if libaxs.so is missing or cannot load, importing this
module raises.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBPATH = os.path.join(_HERE, "libaxs.so")

if not os.path.exists(_LIBPATH):
    raise ImportError("libaxs.so not built: run `python -c 'import __graft_entry__ as g; g.build()'` "
                      "or `python axion-strings_gb300/build.py` first (" + _LIBPATH + ")")
_lib = ctypes.CDLL(_LIBPATH)

OK, ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_STATE, ERR_NONFINITE, ERR_TIMEOUT, ERR_PARSE = 0, -1, -2, -3, -4, -5, -6, -7
F32, F64 = 32, 64
PHI1, PHI2, PHIDOT1, PHIDOT2 = 0, 1, 2, 3


class Params(ctypes.Structure):
    """axs_params: the reference's struct parameters subset plus additions."""
    _fields_ = [
        ("lambda_", ctypes.c_float),
        ("enable_PRS", ctypes.c_int),
        ("T_initial", ctypes.c_float),
        ("NDIMS", ctypes.c_int),
        ("N", ctypes.c_int),
        ("space_step", ctypes.c_float),
        ("time_step", ctypes.c_float),
        ("stencil_setting", ctypes.c_int),
        ("seed", ctypes.c_uint),
        ("thr", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("prs", ctypes.c_int),
        ("tau_initial", ctypes.c_double),
        ("form", ctypes.c_int),
        ("laplacian", ctypes.c_int),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class AxsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("axs error %d: %s" % (code, msg))
        self.code = code


_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_dp = ctypes.POINTER(ctypes.c_double)


def _sig(name, args, res=ctypes.c_int):
    f = getattr(_lib, name)
    f.argtypes = args
    f.restype = res
    return f


_sig("axs_default_params", [ctypes.POINTER(Params)], None)
_sig("axs_last_error", [ctypes.c_char_p, ctypes.c_size_t])
_sig("axs_create", [ctypes.POINTER(Params), ctypes.POINTER(_vp)])
_sig("axs_destroy", [_vp])
_sig("axs_upload", [_vp, _vp, _vp, _vp, _vp])
_sig("axs_upload_f32", [_vp, _vp, _vp, _vp, _vp])
_sig("axs_download", [_vp, _vp, _vp, _vp, _vp])
_sig("axs_download_f32", [_vp, _vp, _vp, _vp, _vp])
_sig("axs_get_time", [_vp, _dp, ctypes.POINTER(_i64)])
_sig("axs_set_time", [_vp, ctypes.c_double, _i64])
_sig("axs_init_gaussian_thermal", [_vp, ctypes.c_uint64])
_sig("axs_init_flat", [_vp, ctypes.c_uint64, ctypes.c_double])
_sig("axs_evolve", [_vp, ctypes.c_int])
_sig("axs_evolve_timed", [_vp, ctypes.c_int, _dp])
_sig("axs_laplacian", [_vp, ctypes.c_int, _vp])
_sig("axs_find_strings", [_vp, _vp, _vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64)])
_sig("axs_string_positions", [_vp, _vp, _i64, ctypes.POINTER(_i64)])
_sig("axs_xi", [ctypes.POINTER(Params), _i64, _i64, ctypes.c_double, ctypes.POINTER(ctypes.c_float)])
_sig("axs_powerspec", [_vp, ctypes.c_int, _vp, _vp, _vp])
_sig("axs_axion_spectrum", [_vp, ctypes.c_int, _vp, _vp, _vp])
_sig("axs_background", [_vp, _vp])
_sig("axs_energies", [_vp, _vp])
_sig("axs_check_finite", [_vp, ctypes.POINTER(ctypes.c_int)])
_sig("axs_field_distance", [_vp, _vp, _vp])
_sig("axs_checkpoint_size", [_vp, ctypes.POINTER(ctypes.c_size_t)])
_sig("axs_checkpoint", [_vp, _vp, ctypes.c_size_t])
_sig("axs_restore", [_vp, _vp, ctypes.c_size_t])
_sig("axs_ensemble_create", [ctypes.POINTER(Params), ctypes.c_int, ctypes.POINTER(_vp)])
_sig("axs_ensemble_destroy", [_vp])
_sig("axs_ensemble_member", [_vp, ctypes.c_int, ctypes.POINTER(_vp)])
_sig("axs_ensemble_evolve", [_vp, ctypes.c_int])
_sig("axs_ensemble_evolve_timed", [_vp, ctypes.c_int, _dp])
_sig("axs_ensemble_find_strings", [_vp, ctypes.c_void_p, ctypes.c_void_p])
_sig("axs_ensemble_axion_spectrum", [_vp, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p])
_sig("axs_inject_wait_timeout", [_vp])
_sig("axs_autotune", [_vp])
_sig("axs_describe", [_vp, ctypes.c_char_p, ctypes.c_size_t])
_sig("axs_ensemble_describe", [_vp, ctypes.c_char_p, ctypes.c_size_t])
_sig("axs_kernel_launches", [], ctypes.c_int64)
_sig("axs_powerspec_noalloc", [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, _vp, _vp, _vp, _vp])
_sig("axs_set_device", [ctypes.c_int])
_sig("axs_host_alloc", [ctypes.c_size_t, ctypes.POINTER(_vp)])
_sig("axs_host_free", [_vp])


def _check(rc):
    if rc != OK:
        buf = ctypes.create_string_buffer(512)
        _lib.axs_last_error(buf, 512)
        raise AxsError(rc, buf.value.decode(errors="replace"))
    return rc


def lib_path():
    return _LIBPATH


def default_params(**kw):
    """Params with the reference's default.param values, then overrides."""
    p = Params()
    _lib.axs_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if k == "lambda":
            k = "lambda_"
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def xi(params, n_plaquettes, num_cores, tau):
    out = ctypes.c_float()
    _check(_lib.axs_xi(ctypes.byref(params), int(n_plaquettes), int(num_cores), float(tau), ctypes.byref(out)))
    return out.value


def field_distance(a, b):
    """Relative L2 distance per field (phi1, phi2, phidot1, phidot2) of lattice
    a from lattice b: sqrt(sum (a-b)^2 / sum b^2), computed on the device."""
    out = np.empty(8)
    _check(_lib.axs_field_distance(a._h, b._h, _ptr(out)))
    return np.sqrt(out[0::2] / np.where(out[1::2] > 0, out[1::2], 1.0))


def kernel_launches():
    return int(_lib.axs_kernel_launches())


def set_device(device):
    _check(_lib.axs_set_device(int(device)))


def powerspec_noalloc(spectrum_ptr, ndims, n, precision, space_step, pk_ptr, ks_ptr, count_ptr, stream=0):
    """axs_powerspec_noalloc on caller-owned device buffers (raw device
    addresses); asynchronous on `stream` (a cudaStream_t value, 0 = default)."""
    _check(_lib.axs_powerspec_noalloc(_vp(spectrum_ptr), int(ndims), int(n), int(precision), float(space_step),
                                      _vp(pk_ptr), _vp(ks_ptr), _vp(count_ptr), _vp(stream or None)))


def _ptr(a):
    return None if a is None else a.ctypes.data


class Lattice:
    """One lattice resident on the GPU (axs_lattice)."""

    def __init__(self, params=None, _handle=None, _owner=None, **kw):
        if _handle is not None:
            self._h = _handle
            self._owner = _owner
            self.params = params
            return
        p = params if params is not None else default_params(**kw)
        if params is not None and kw:
            for k, v in kw.items():
                setattr(p, "lambda_" if k == "lambda" else k, v)
        self.params = p
        self._owner = None
        h = _vp()
        _check(_lib.axs_create(ctypes.byref(p), ctypes.byref(h)))
        self._h = h

    # lifetime
    def close(self):
        if self._h and self._owner is None:
            _check(_lib.axs_destroy(self._h))
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def shape(self):
        n = self.params.N
        return (n, n) if self.params.NDIMS == 2 else (n, n, n)

    @property
    def length(self):
        return int(np.prod(self.shape))

    # state transfer
    def _prep(self, a, dt):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dt)
        if a.size != self.length:
            raise ValueError("array has %d values, lattice has %d" % (a.size, self.length))
        return a

    def upload(self, phi1=None, phi2=None, phidot1=None, phidot2=None, dtype=np.float64):
        arrs = [self._prep(a, dtype) for a in (phi1, phi2, phidot1, phidot2)]
        fn = _lib.axs_upload if np.dtype(dtype) == np.float64 else _lib.axs_upload_f32
        _check(fn(self._h, *[_ptr(a) for a in arrs]))

    def download(self, dtype=np.float64, fields=(True, True, True, True)):
        outs = [np.empty(self.shape, dtype=dtype) if want else None for want in fields]
        fn = _lib.axs_download if np.dtype(dtype) == np.float64 else _lib.axs_download_f32
        _check(fn(self._h, *[_ptr(a) for a in outs]))
        return tuple(outs)

    @property
    def time(self):
        t = ctypes.c_double()
        s = _i64()
        _check(_lib.axs_get_time(self._h, ctypes.byref(t), ctypes.byref(s)))
        return t.value, s.value

    def set_time(self, tau, steps=0):
        _check(_lib.axs_set_time(self._h, float(tau), int(steps)))

    # initial conditions
    def init_thermal(self, seed):
        _check(_lib.axs_init_gaussian_thermal(self._h, int(seed)))

    def init_flat(self, seed, kcut=1.0):
        _check(_lib.axs_init_flat(self._h, int(seed), float(kcut)))

    # evolution
    def evolve(self, nsteps):
        _check(_lib.axs_evolve(self._h, int(nsteps)))

    def evolve_timed(self, nsteps):
        ms = ctypes.c_double()
        _check(_lib.axs_evolve_timed(self._h, int(nsteps), ctypes.byref(ms)))
        return ms.value

    def laplacian(self, field=PHI1):
        out = np.empty(self.shape, dtype=np.float64)
        _check(_lib.axs_laplacian(self._h, int(field), _ptr(out)))
        return out

    # strings
    def find_strings(self, theta=None, want_mask=False):
        th = self._prep(theta, np.float64)
        mask = np.empty(self.shape, dtype=np.uint8) if want_mask else None
        n = _i64()
        c = _i64()
        _check(_lib.axs_find_strings(self._h, _ptr(th), _ptr(mask), ctypes.byref(n), ctypes.byref(c)))
        return n.value, c.value, mask

    def string_positions(self):
        n = _i64()
        _check(_lib.axs_string_positions(self._h, None, 0, ctypes.byref(n)))
        out = np.empty((n.value, self.params.NDIMS), dtype=np.int32)
        if n.value:
            _check(_lib.axs_string_positions(self._h, _ptr(out), n.value, ctypes.byref(n)))
        return out

    # spectra and reductions
    def powerspec(self, field=PHI2):
        nb = self.params.N // 2
        pk = np.empty(nb)
        ks = np.empty(nb)
        cnt = np.empty(nb, dtype=np.int32)
        _check(_lib.axs_powerspec(self._h, int(field), _ptr(pk), _ptr(ks), _ptr(cnt)))
        return pk, ks, cnt

    def axion_spectrum(self, nbins=128):
        k = np.empty(nbins)
        pk = np.empty(nbins)
        cnt = np.empty(nbins, dtype=np.int64)
        _check(_lib.axs_axion_spectrum(self._h, int(nbins), _ptr(k), _ptr(pk), _ptr(cnt)))
        return k, pk, cnt

    def background(self):
        out = np.empty(6)
        _check(_lib.axs_background(self._h, _ptr(out)))
        return out

    def energies(self):
        out = np.empty(3)
        _check(_lib.axs_energies(self._h, _ptr(out)))
        return out

    def check_finite(self):
        f = ctypes.c_int()
        rc = _lib.axs_check_finite(self._h, ctypes.byref(f))
        if rc not in (OK, ERR_NONFINITE):
            _check(rc)
        return bool(f.value)

    # checkpoint
    def checkpoint(self):
        n = ctypes.c_size_t()
        _check(_lib.axs_checkpoint_size(self._h, ctypes.byref(n)))
        buf = np.empty(n.value, dtype=np.uint8)
        _check(_lib.axs_checkpoint(self._h, _ptr(buf), n.value))
        return buf

    def restore(self, buf):
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        _check(_lib.axs_restore(self._h, _ptr(buf), buf.size))

    def inject_wait_timeout(self):
        """Test-only: make the next step's device-side waits run out."""
        _check(_lib.axs_inject_wait_timeout(self._h))

    # tuning
    def autotune(self):
        _check(_lib.axs_autotune(self._h))

    def describe(self):
        b = ctypes.create_string_buffer(256)
        _check(_lib.axs_describe(self._h, b, 256))
        return b.value.decode()


class Ensemble:
    """Independent lattices stepped by one persistent launch per step."""

    def __init__(self, params_list):
        arr = (Params * len(params_list))(*params_list)
        h = _vp()
        _check(_lib.axs_ensemble_create(arr, len(params_list), ctypes.byref(h)))
        self._h = h
        self.members = []
        for i, p in enumerate(params_list):
            mh = _vp()
            _check(_lib.axs_ensemble_member(h, i, ctypes.byref(mh)))
            self.members.append(Lattice(params=p, _handle=mh, _owner=self))

    def evolve(self, nsteps):
        _check(_lib.axs_ensemble_evolve(self._h, int(nsteps)))

    def evolve_timed(self, nsteps):
        ms = ctypes.c_double()
        _check(_lib.axs_ensemble_evolve_timed(self._h, int(nsteps), ctypes.byref(ms)))
        return ms.value

    def describe(self):
        b = ctypes.create_string_buffer(256)
        _check(_lib.axs_ensemble_describe(self._h, b, 256))
        return b.value.decode()

    def find_strings(self):
        """(n_plaquettes, num_cores) per member, one batched call."""
        n = len(self.members)
        npl, nco = np.zeros(n, np.int64), np.zeros(n, np.int64)
        _check(_lib.axs_ensemble_find_strings(self._h, npl.ctypes.data, nco.ctypes.data))
        return npl, nco

    def axion_spectrum(self, nbins=128):
        """(kmean, pk, count), each (members, nbins), one batched call."""
        n = len(self.members)
        k, pk = np.zeros((n, nbins)), np.zeros((n, nbins))
        cnt = np.zeros((n, nbins), np.int64)
        _check(_lib.axs_ensemble_axion_spectrum(self._h, int(nbins), k.ctypes.data, pk.ctypes.data, cnt.ctypes.data))
        return k, pk, cnt

    def close(self):
        if self._h:
            for m in self.members:
                m._h = None
            _check(_lib.axs_ensemble_destroy(self._h))
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class PinnedBuffer:
    """Page-locked host array (cudaMallocHost) viewed as numpy."""

    def __init__(self, shape, dtype=np.float64):
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = _vp()
        _check(_lib.axs_host_alloc(self.nbytes, ctypes.byref(p)))
        self._p = p
        buf = (ctypes.c_char * self.nbytes).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if self._p:
            self.array = None
            _check(_lib.axs_host_free(self._p))
            self._p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
