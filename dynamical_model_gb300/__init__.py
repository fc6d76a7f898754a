"""GB300-native MOLOCH dynamical-core step.

Python mirror of the reference module `mod_moloch` (nompi/mod_moloch.F90):
``Moloch`` holds one domain on the GPU and offers the reference's three
entry points -- ``allocate_moloch`` (constructor), ``init_moloch`` (upload +
init) and ``moloch(istep, lprint)`` -- over the C ABI in
include/moloch_gb300.h.  There is no CPU fallback: the native library must
load, and every step runs the CUDA kernels in csrc/.
"""
import ctypes
import os

import numpy as np

from .build import LIB as _LIB_PATH, build as _build

__all__ = ["Moloch", "Ensemble", "MolochError", "Params", "Grid", "Diag", "Ideal", "lib", "FIELD",
           "FP64", "FP64_EXACT", "FP32_MIXED", "field_bounds"]

FP64, FP64_EXACT, FP32_MIXED = 0, 1, 2
_MODES = {"fp64": FP64, "fp64_exact": FP64_EXACT, "fp32_mixed": FP32_MIXED, "mixed": FP32_MIXED}

# field ids, same order as enum moloch_field
_FIELD_NAMES = ["u", "v", "w", "pai", "t", "tetav", "qv", "qc", "qi", "qr", "qs", "qx",
                "p", "tvirt", "qsat", "rho", "ps", "zeta", "fmz", "fmzf", "ht",
                "msfx", "msfu", "msfv", "hx", "hy", "ulat", "vlat", "zita", "zitah", "s", "deltaw"]
FIELD = {n: i for i, n in enumerate(_FIELD_NAMES)}

ERRORS = {0: "ok", 1: "bad argument", 2: "bounds mismatch", 3: "CUDA error", 4: "CFL violation",
          5: "call out of order", 6: "device wait timed out", 7: "out of device memory"}


class MolochError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Grid(ctypes.Structure):
    _fields_ = [("jx", ctypes.c_int), ("iy", ctypes.c_int), ("kz", ctypes.c_int)]


class Params(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("dx", ctypes.c_double), ("mo_ztop", ctypes.c_double),
                ("mo_h", ctypes.c_double), ("mo_a0", ctypes.c_double), ("mo_anu2", ctypes.c_double),
                ("mo_nadv", ctypes.c_int), ("mo_nsound", ctypes.c_int), ("mode", ctypes.c_int),
                ("mo_divfilter", ctypes.c_int), ("do_filterpai", ctypes.c_int),
                ("do_filtertheta", ctypes.c_int), ("rotllr", ctypes.c_int)]


class Diag(ctypes.Structure):
    _fields_ = [("maxps", ctypes.c_double), ("minps", ctypes.c_double), ("maxu", ctypes.c_double),
                ("minu", ctypes.c_double), ("maxv", ctypes.c_double), ("minv", ctypes.c_double),
                ("mass", ctypes.c_double), ("energy", ctypes.c_double),
                ("status", ctypes.c_int), ("nonfinite", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class Ideal(ctypes.Structure):
    _fields_ = [("nhills", ctypes.c_int), ("hill_h", ctypes.c_double * 4), ("hill_j", ctypes.c_double * 4),
                ("hill_i", ctypes.c_double * 4), ("hill_r", ctypes.c_double * 4),
                ("pert_amp", ctypes.c_double), ("pert_levels", ctypes.c_int),
                ("seed", ctypes.c_ulonglong), ("u0", ctypes.c_double), ("v0", ctypes.c_double)]


# exported symbols and their prototypes (must cover every function of the header)
_PROTOS = {
    "moloch_gpu_create": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(Params), ctypes.c_void_p,
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "moloch_gpu_default_params": (None, [ctypes.POINTER(Params)]),
    "moloch_gpu_upload": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "moloch_gpu_init": (ctypes.c_int, [ctypes.c_void_p]),
    "moloch_gpu_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(Diag)]),
    "moloch_gpu_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "moloch_gpu_download": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "moloch_gpu_sync": (ctypes.c_int, [ctypes.c_void_p]),
    "moloch_gpu_set_wait_limit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int]),
    "moloch_gpu_check_division": (ctypes.c_int, [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.c_void_p]),
    "moloch_gpu_check_division_f64": (ctypes.c_int, [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.c_void_p]),
    "moloch_gpu_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "moloch_gpu_kernel_count": (ctypes.c_longlong, [ctypes.c_void_p]),
    "moloch_gpu_phase": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "moloch_gpu_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "moloch_gpu_last_error": (ctypes.c_char_p, []),
    "moloch_gpu_setup_idealized": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Ideal)]),
    "moloch_gpu_setup_idealized_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Ideal)]),
    "moloch_gpu_profile_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                               ctypes.POINTER(ctypes.c_int), ctypes.c_int]),
    "moloch_gpu_kernel_kinds": (ctypes.c_int, []),
    "moloch_gpu_host_direct": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "moloch_gpu_host_register": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "moloch_gpu_host_unregister": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "moloch_gpu_kernel_name": (ctypes.c_char_p, [ctypes.c_int]),
    "moloch_gpu_tuning_count": (ctypes.c_int, []),
    "moloch_gpu_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_double), ctypes.c_int]),
    "moloch_gpu_set_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int]),
    "moloch_gpu_ensemble_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                                  ctypes.POINTER(ctypes.c_void_p)]),
    "moloch_gpu_ensemble_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "moloch_gpu_ensemble_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                                    ctypes.POINTER(ctypes.c_double), ctypes.c_int]),
    "moloch_gpu_ensemble_set_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int]),
    "moloch_gpu_ensemble_kernel_count": (ctypes.c_longlong, [ctypes.c_void_p]),
    "moloch_gpu_ensemble_set_persistent": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "moloch_gpu_ensemble_persistent": (ctypes.c_int, [ctypes.c_void_p]),
    "moloch_gpu_ensemble_set_wait_limit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int,
                                                          ctypes.c_int]),
    "moloch_gpu_ensemble_sync": (ctypes.c_int, [ctypes.c_void_p]),
    "moloch_gpu_ensemble_profile_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                                        ctypes.POINTER(ctypes.c_int), ctypes.c_int]),
    "moloch_gpu_ensemble_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "moloch_tc_gemm": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                      ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                      ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_void_p]),
    "moloch_tc_status": (ctypes.c_int, []),
    "moloch_tc_set_wait_limit": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_int, ctypes.c_int]),
    "moloch_gpu_wafone_noalloc": (ctypes.c_int, [ctypes.c_void_p] * 9 + [ctypes.c_int] * 3 +
                                  [ctypes.c_double] * 3 + [ctypes.c_int, ctypes.c_void_p]),
    "moloch_gpu_output_start": (ctypes.c_int, [ctypes.c_void_p]),
    "moloch_gpu_output_finish": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                                ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int),
                                                ctypes.POINTER(ctypes.c_int)]),
    "moloch_sur_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong,
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "moloch_sur_collect": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_ulonglong]),
    "moloch_sur_pairs": (ctypes.c_int, [ctypes.c_void_p]),
    "moloch_sur_pair_data": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                            ctypes.c_void_p]),
    "moloch_sur_prepare": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_ulonglong]),
    "moloch_sur_train": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_ulonglong,
                                        ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "moloch_sur_attach": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_int,
                                         ctypes.c_float]),
    "moloch_sur_counts": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong),
                                         ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "moloch_sur_param": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "moloch_sur_gradients": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.c_void_p,
                                            ctypes.c_void_p]),
    "moloch_sur_dims": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "moloch_sur_stats": (ctypes.c_int, [ctypes.c_void_p] * 5 + [ctypes.c_int]),
    "moloch_sur_profile": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                          ctypes.c_int]),
    "moloch_sur_destroy": (ctypes.c_int, [ctypes.c_void_p]),
}

_lib = None


def lib(build_if_missing=True):
    """Load libmoloch_gb300.so (building it first when it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build()
    if not os.path.exists(_LIB_PATH):
        raise ImportError(f"native library {_LIB_PATH} is missing; run dynamical_model_gb300.build.build()")
    L = ctypes.CDLL(_LIB_PATH)
    for name, (res, args) in _PROTOS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise MolochError(rc, lib().moloch_gpu_last_error().decode())


def field_bounds(name, jx, iy, kz):
    """Fortran (lower, upper) bounds of a reference array (nompi/mod_atmosphere.F90:104-169)."""
    nj, ni = jx, iy
    b = {
        "u": ((-1, nj + 2), (0, ni + 1), (1, kz)),
        "v": ((0, nj + 1), (-1, ni + 2), (1, kz)),
        "w": ((1, nj), (1, ni), (1, kz + 1)),
        "zeta": ((-1, nj + 2), (-1, ni + 2), (1, kz)),
        "fmzf": ((1, nj), (1, ni), (1, kz + 1)),
        "s": ((1, nj), (1, ni), (1, kz + 1)),
        "deltaw": ((0, nj + 1), (0, ni + 1), (1, kz + 1)),
        "ps": ((0, nj + 1), (0, ni + 1)),
        "ht": ((-1, nj + 2), (-1, ni + 2)),
        "msfx": ((1, nj), (1, ni)), "ulat": ((1, nj), (1, ni)), "vlat": ((1, nj), (1, ni)),
        "msfu": ((0, nj + 1), (1, ni)), "hx": ((0, nj + 1), (1, ni)),
        "msfv": ((1, nj), (0, ni + 1)), "hy": ((1, nj), (0, ni + 1)),
        "zita": ((1, kz + 1),), "zitah": ((1, kz),),
        "qx": ((0, nj + 1), (0, ni + 1), (1, kz), (1, 5)),
    }
    if name in b:
        return b[name]
    if name in ("pai", "t", "tetav", "fmz", "qv", "qc", "qi", "qr", "qs"):
        return ((0, nj + 1), (0, ni + 1), (1, kz))
    if name in ("p", "tvirt", "qsat", "rho"):
        return ((1, nj), (1, ni), (1, kz))
    raise KeyError(name)


class Moloch:
    """One MOLOCH domain resident on the GPU.

    ``Moloch(jx, iy, kz, mode=...)`` is allocate_moloch; ``setup_idealized``
    runs the reference driver's param()+init() and init_moloch;
    ``moloch(istep, lprint)`` is one dt step.  ``get(name)`` returns the
    interior of a field as a (nk, iy, jx) float64 array (C order: the last
    axis is the reference's contiguous j index).
    """

    def __init__(self, jx, iy, kz, mode="fp64", stream=None, **opts):
        self.L = lib()
        self.jx, self.iy, self.kz = jx, iy, kz
        self.grid = Grid(jx, iy, kz)
        self.params = Params()
        self.L.moloch_gpu_default_params(ctypes.byref(self.params))
        self.params.mode = _MODES[mode] if isinstance(mode, str) else int(mode)
        for k, v in opts.items():
            if not hasattr(self.params, k):
                raise TypeError(f"unknown option {k}")
            setattr(self.params, k, v)
        h = ctypes.c_void_p()
        _check(self.L.moloch_gpu_create(ctypes.byref(self.grid), ctypes.byref(self.params),
                                        ctypes.c_void_p(stream) if stream else None, ctypes.byref(h)))
        self.h = h
        self._pinned = {}  # registered host arrays, kept alive while pinned

    # -- init_moloch ----------------------------------------------------------
    def setup_idealized(self, hills=(), pert_amp=0.5, pert_levels=10, seed=1234, u0=1.0, v0=1.0, device=False):
        """param() + init() + init_moloch.  device=True computes the state on
        the GPU (moloch_gpu_setup_idealized_device) instead of on the host."""
        z = Ideal()
        z.nhills = len(hills)
        for n, (hh, cj, ci, r) in enumerate(hills):
            z.hill_h[n], z.hill_j[n], z.hill_i[n], z.hill_r[n] = hh, cj, ci, r
        z.pert_amp, z.pert_levels, z.seed, z.u0, z.v0 = pert_amp, pert_levels, seed, u0, v0
        fn = self.L.moloch_gpu_setup_idealized_device if device else self.L.moloch_gpu_setup_idealized
        _check(fn(self.h, ctypes.byref(z)))

    def upload(self, name, arr):
        """Upload a reference-layout array (Fortran order, with its halo)."""
        bnds = field_bounds(name, self.jx, self.iy, self.kz)
        a = np.asfortranarray(arr, dtype=np.float64)
        shape = tuple(u - l + 1 for l, u in bnds)
        if a.shape != shape:
            raise ValueError(f"{name}: shape {a.shape}, expected {shape}")
        lb = (ctypes.c_int * 4)(*[l for l, _ in bnds])
        ub = (ctypes.c_int * 4)(*[u for _, u in bnds])
        _check(self.L.moloch_gpu_upload(self.h, FIELD[name], a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                        lb, ub))

    def init(self):
        _check(self.L.moloch_gpu_init(self.h))

    # -- moloch ---------------------------------------------------------------
    def moloch(self, istep=1, lprint=False):
        d = Diag()
        _check(self.L.moloch_gpu_step(self.h, istep, int(lprint), ctypes.byref(d)))
        return d if lprint else None

    step = moloch

    def run(self, nsteps, graph=True):
        _check(self.L.moloch_gpu_run(self.h, nsteps, int(graph)))

    def phase(self, p):
        _check(self.L.moloch_gpu_phase(self.h, p))

    def sync(self):
        _check(self.L.moloch_gpu_sync(self.h))

    def set_wait_limit(self, cycles=0, skip_job=-1):
        """Limit (SM clock cycles, 0: default) of the staged column kernel's
        bounded waits; skip_job >= 0 is a test hook that leaves that staged
        chunk unissued so a wait runs out (moloch_gpu_set_wait_limit)."""
        _check(self.L.moloch_gpu_set_wait_limit(self.h, int(cycles), int(skip_job)))

    def profile_step(self):
        """One step with CUDA events around every kernel: {kernel: (ms, launches)}."""
        n = self.L.moloch_gpu_kernel_kinds()
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_int * n)()
        _check(self.L.moloch_gpu_profile_step(self.h, ms, cnt, n))
        return {self.L.moloch_gpu_kernel_name(k).decode(): (ms[k], cnt[k]) for k in range(n) if cnt[k]}

    def autotune(self):
        """Time the tunable launch shapes on this handle (advances the state)
        and keep the fastest; returns the chosen values."""
        n = self.L.moloch_gpu_tuning_count()
        ch = (ctypes.c_int * n)()
        ms = (ctypes.c_double * n)()
        _check(self.L.moloch_gpu_autotune(self.h, ch, ms, n))
        return list(ch)

    def set_tuning(self, choice):
        arr = (ctypes.c_int * len(choice))(*choice)
        _check(self.L.moloch_gpu_set_tuning(self.h, arr, len(choice)))

    @property
    def stream(self):
        return self.L.moloch_gpu_stream(self.h)

    @property
    def host_direct(self):
        """True when uploads read the host arrays with a kernel through the
        host page tables (see moloch_gpu_host_direct)."""
        rc = self.L.moloch_gpu_host_direct(self.h, -1)
        _check(min(rc, 0))
        return bool(rc)

    @host_direct.setter
    def host_direct(self, enable):
        rc = self.L.moloch_gpu_host_direct(self.h, 1 if enable else 0)
        _check(min(rc, 0))

    def host_register(self, arr):
        """Pin a host array that will be uploaded repeatedly: its uploads
        become DMA copies overlapping the steps already issued.  The array
        is kept alive until host_unregister or close."""
        _check(self.L.moloch_gpu_host_register(self.h, arr.ctypes.data, arr.nbytes))
        self._pinned[arr.ctypes.data] = arr

    def host_unregister(self, arr):
        _check(self.L.moloch_gpu_host_unregister(self.h, arr.ctypes.data))
        self._pinned.pop(arr.ctypes.data, None)

    @property
    def kernel_count(self):
        return self.L.moloch_gpu_kernel_count(self.h)

    def download(self, name):
        """The reference-layout array (Fortran order, halo rings included)."""
        bnds = field_bounds(name, self.jx, self.iy, self.kz)
        shape = tuple(u - l + 1 for l, u in bnds)
        a = np.zeros(shape, dtype=np.float64, order="F")
        lb = (ctypes.c_int * 4)(*[l for l, _ in bnds])
        ub = (ctypes.c_int * 4)(*[u for _, u in bnds])
        _check(self.L.moloch_gpu_download(self.h, FIELD[name], a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                          lb, ub))
        return a

    def output_start(self):
        """Snapshot t and ps now (in stream order) and start their copy to
        the host; the next steps overlap the copy."""
        _check(self.L.moloch_gpu_output_start(self.h))

    def output_finish(self, t=None, ps=None):
        """(t, ps) of the last output_start, reference layout with halos;
        filled into the given arrays (for instance registered ones, which the
        device then writes directly) or into new ones."""
        arrs, args = [], []
        for name, given in (("t", t), ("ps", ps)):
            bnds = field_bounds(name, self.jx, self.iy, self.kz)
            shape = tuple(u - l + 1 for l, u in bnds)
            if given is None:
                a = np.zeros(shape, dtype=np.float64, order="F")
            else:
                if given.shape != shape or given.dtype != np.float64 or not given.flags.f_contiguous:
                    raise ValueError(f"{name}: need a Fortran-ordered float64 array of shape {shape}")
                a = given
            arrs.append(a)
            args += [a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                     (ctypes.c_int * 4)(*[l for l, _ in bnds]), (ctypes.c_int * 4)(*[u for _, u in bnds])]
        _check(self.L.moloch_gpu_output_finish(self.h, *args))
        return arrs[0], arrs[1]

    def get_1d(self, name):
        """A 1-D level table (zita, zitah) as uploaded."""
        return np.array(self.download(name))

    def get(self, name):
        """Interior of a field as (nk, iy, jx) float64 (or (iy, jx) for 2-D)."""
        a = self.download(name)
        bnds = field_bounds(name, self.jx, self.iy, self.kz)
        sl = tuple(slice(1 - l, 1 - l + n) for (l, _), n in zip(bnds[:2], (self.jx, self.iy)))
        if len(bnds) == 2:
            return np.ascontiguousarray(a[sl].T)
        k0 = 1 - bnds[2][0]
        return np.ascontiguousarray(a[sl + (slice(k0, None),)].transpose(2, 1, 0))

    def close(self):
        if getattr(self, "h", None):
            self.L.moloch_gpu_destroy(self.h)  # also unregisters the pinned arrays
            self.h = None
            self._pinned = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Ensemble:
    """Members (Moloch handles on one stream) advanced together, one CUDA
    graph per ensemble step: one batched launch per kernel over all members,
    or (persistent mode) one cooperative launch per step whose blocks walk
    the step's kernels as phases between grid barriers, taking (member,
    tile) items from a device-side work queue."""

    def __init__(self, members):
        self.L = lib()
        self.members = list(members)
        arr = (ctypes.c_void_p * len(self.members))(*[m.h.value for m in self.members])
        h = ctypes.c_void_p()
        _check(self.L.moloch_gpu_ensemble_create(len(self.members), arr, ctypes.byref(h)))
        self.h = h

    def run(self, nsteps, graph=True):
        _check(self.L.moloch_gpu_ensemble_run(self.h, nsteps, int(graph)))

    def autotune(self):
        n = self.L.moloch_gpu_tuning_count()
        ch = (ctypes.c_int * n)()
        ms = (ctypes.c_double * n)()
        _check(self.L.moloch_gpu_ensemble_autotune(self.h, ch, ms, n))
        return list(ch)

    def set_tuning(self, choice):
        arr = (ctypes.c_int * len(choice))(*choice)
        _check(self.L.moloch_gpu_ensemble_set_tuning(self.h, arr, len(choice)))

    @property
    def kernel_count(self):
        return self.L.moloch_gpu_ensemble_kernel_count(self.h)

    def profile_step(self):
        """One step timed per kernel kind: {kernel: (ms, launches or phases)}."""
        n = self.L.moloch_gpu_kernel_kinds()
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_int * n)()
        _check(self.L.moloch_gpu_ensemble_profile_step(self.h, ms, cnt, n))
        return {self.L.moloch_gpu_kernel_name(k).decode(): (ms[k], cnt[k]) for k in range(n) if cnt[k]}

    def set_persistent(self, on=True):
        """on: False/0 off; True/1 on; 2, 3, 4: on, with the kernel built for
        that many resident blocks per SM."""
        _check(self.L.moloch_gpu_ensemble_set_persistent(self.h, int(on)))

    @property
    def persistent(self):
        """0 when off, else the resident blocks per SM of the build in use."""
        return self.L.moloch_gpu_ensemble_persistent(self.h)

    def set_wait_limit(self, cycles=0, skip_block=-1, skip_barrier=-1):
        """Limit of the persistent kernel's grid-barrier waits (SM cycles,
        0: default); skip_block/skip_barrier make that block leave at that
        barrier without arriving (test hook)."""
        _check(self.L.moloch_gpu_ensemble_set_wait_limit(self.h, int(cycles), int(skip_block), int(skip_barrier)))

    def sync(self):
        """Wait for the stream; MolochError (MOLOCH_ERR_TIMEOUT) when a
        barrier wait of the persistent kernel gave up."""
        _check(self.L.moloch_gpu_ensemble_sync(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.L.moloch_gpu_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Surrogate:
    """Learned acoustic-cycle surrogate (per-column MLP on tcgen05): collect
    training pairs from plain steps of an FP32-storage handle, train, attach.
    While attached, every sound() call runs the MLP first and falls back to
    the plain acoustic substeps when the on-device check rejects it."""

    def __init__(self, kz, capacity=65536, batch=256, seed=1):
        self.L = lib()
        h = ctypes.c_void_p()
        _check(self.L.moloch_sur_create(kz, capacity, batch, seed, ctypes.byref(h)))
        self.h = h
        self.attached = None

    def dims(self):
        d = (ctypes.c_int * 9)()
        _check(self.L.moloch_sur_dims(self.h, d))
        keys = ("kz", "nin", "kin", "nout", "nop", "hidden", "batch", "pairs", "ntrain")
        return dict(zip(keys, list(d)))

    def collect(self, model, nsteps, cols_per_cycle=512, seed=3):
        _check(self.L.moloch_sur_collect(self.h, model.h, nsteps, cols_per_cycle, seed))
        return self.L.moloch_sur_pairs(self.h)

    def pair_data(self, first=0, count=None):
        """Collected pairs as (X [count][45 kz] raw features, T [count][5 kz]
        raw increments), in collection order."""
        d = self.dims()
        if count is None:
            count = d["pairs"] - first
        X = np.empty((count, d["nin"]), np.float32)
        T = np.empty((count, d["nout"]), np.float32)
        _check(self.L.moloch_sur_pair_data(self.h, first, count, X.ctypes.data, T.ctypes.data))
        return X, T

    def prepare(self, val_fraction=0.1, seed=5):
        _check(self.L.moloch_sur_prepare(self.h, val_fraction, seed))

    def train(self, iters, lr=1e-3, seed=7):
        tl, vl = ctypes.c_float(), ctypes.c_float()
        _check(self.L.moloch_sur_train(self.h, iters, lr, seed, ctypes.byref(tl), ctypes.byref(vl)))
        return tl.value, vl.value

    def attach(self, model, threshold=4.0, judge_every=6, tol=0.3):
        """threshold: multiple of the training envelope an increment may
        reach; judge_every: plain-loop judge every n-th sound() call (0:
        never); tol: largest relative RMS error of the increments the judge
        accepts."""
        _check(self.L.moloch_sur_attach(model.h, self.h, threshold, judge_every, tol))
        self.attached = model

    def detach(self):
        if self.attached is not None and getattr(self.attached, "h", None):
            _check(self.L.moloch_sur_attach(self.attached.h, None, 0.0, 0, 0.0))
        self.attached = None

    def counts(self):
        """(sound() calls, calls run by the plain loop)."""
        return self.stats_counts()["cycles"], self.stats_counts()["plain"]

    def stats_counts(self):
        c = (ctypes.c_longlong * 4)()
        r, e = ctypes.c_float(), ctypes.c_float()
        _check(self.L.moloch_sur_counts(self.h, c, ctypes.byref(r), ctypes.byref(e)))
        return {"cycles": c[0], "plain": c[1], "judged": c[2], "judge_rejections": c[3],
                "max_ratio": r.value, "last_judge_error": e.value}

    def param(self, layer):
        io = (ctypes.c_int * 2)()
        _check(self.L.moloch_sur_param(self.h, layer, None, None, 0, io))
        W = np.empty((io[1], io[0]), np.float32)
        b = np.empty(io[1], np.float32)
        _check(self.L.moloch_sur_param(self.h, layer, W.ctypes.data, b.ctypes.data, 0, io))
        return W, b

    def set_param(self, layer, W, b):
        W = np.ascontiguousarray(W, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        io = (ctypes.c_int * 2)()
        _check(self.L.moloch_sur_param(self.h, layer, None, None, 0, io))
        if W.shape != (io[1], io[0]) or b.shape != (io[1],):
            raise ValueError(f"layer {layer} is {io[1]}x{io[0]}")
        _check(self.L.moloch_sur_param(self.h, layer, W.ctypes.data, b.ctypes.data, 1, io))

    def profile(self, model):
        """CUDA-event ms of the inference stages of one cycle on the model's
        state (changes no field)."""
        ms = (ctypes.c_double * 6)()
        _check(self.L.moloch_sur_profile(self.h, model.h, ms, 6))
        return dict(zip(("features", "layer1", "layer2", "layer3", "layer4", "check"), list(ms)))

    def stats(self):
        """(xmean, xstd, ymean, ystd), each [5, kz] (u, v, w, pai, tetav)."""
        kz = self.dims()["kz"]
        a = [np.empty((5, kz), np.float32) for _ in range(4)]
        _check(self.L.moloch_sur_stats(self.h, *[x.ctypes.data for x in a], 0))
        return tuple(a)

    def set_stats(self, xmean, xstd, ymean, ystd):
        kz = self.dims()["kz"]
        a = [np.ascontiguousarray(np.broadcast_to(np.asarray(x, np.float32), (5, kz))) for x in
             (xmean, xstd, ymean, ystd)]
        _check(self.L.moloch_sur_stats(self.h, *[x.ctypes.data for x in a], 1))

    def gradients(self, X, T, layer):
        """(summed squared error, dW, db) of one forward+backward pass."""
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        W, _ = self.param(layer)
        gW = np.empty_like(W)
        gb = np.empty(W.shape[0], np.float32)
        loss = ctypes.c_float()
        _check(self.L.moloch_sur_gradients(self.h, X.ctypes.data, T.ctypes.data, X.shape[0], ctypes.byref(loss),
                                           layer, gW.ctypes.data, gb.ctypes.data))
        return loss.value, gW, gb

    def close(self):
        if getattr(self, "h", None):
            try:
                self.detach()
            finally:
                self.L.moloch_sur_destroy(self.h)
                self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
