"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker.  The product never imports it.

The oracle restates the reference's serial (nompi) MOLOCH step; see the
header of moloch_oracle.c for what it follows and why parity is unpinned.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {}


class OracleCfg(ctypes.Structure):
    _fields_ = [
        ("jx", ctypes.c_int), ("iy", ctypes.c_int), ("kz", ctypes.c_int),
        ("nhills", ctypes.c_int),
        ("hill_h", ctypes.c_double * 4), ("hill_j", ctypes.c_double * 4),
        ("hill_i", ctypes.c_double * 4), ("hill_r", ctypes.c_double * 4),
        ("pert_amp", ctypes.c_double), ("pert_levels", ctypes.c_int),
        ("seed", ctypes.c_ulonglong),
        ("u0", ctypes.c_double), ("v0", ctypes.c_double),
        ("divfilter", ctypes.c_int), ("filterpai", ctypes.c_int),
        ("filtertheta", ctypes.c_int), ("rotllr", ctypes.c_int),
    ]


def build():
    """Compile the oracle with its Makefile (gcc, OpenMP, no FMA contraction)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib(checked=False):
    name = "liboracle_moloch_chk.so" if checked else "liboracle_moloch.so"
    if name in _LIBS:
        return _LIBS[name]
    path = os.path.join(_HERE, "build", name)
    if not os.path.exists(path):
        build()
    L = ctypes.CDLL(path)
    L.oracle_create.restype = ctypes.c_void_p
    L.oracle_create.argtypes = [ctypes.POINTER(OracleCfg)]
    L.oracle_step.restype = ctypes.c_int
    L.oracle_step.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                              ctypes.POINTER(ctypes.c_double)]
    L.oracle_phase.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.oracle_stagger.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.oracle_divdamp.argtypes = [ctypes.c_void_p]
    L.oracle_filter.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.oracle_set_map_factors.argtypes = [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_double)] * 3
    L.oracle_wafone.restype = ctypes.c_int
    L.oracle_wafone.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    L.oracle_get.restype = ctypes.c_int
    L.oracle_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]
    L.oracle_set.restype = ctypes.c_int
    L.oracle_set.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]
    L.oracle_get_bounded.restype = ctypes.c_int
    L.oracle_get_bounded.argtypes = [ctypes.c_void_p, ctypes.c_char_p,
                                     ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.oracle_destroy.argtypes = [ctypes.c_void_p]
    for fn in ("oracle_pfesat", "oracle_pfwsat"):
        getattr(L, fn).restype = ctypes.c_double
        getattr(L, fn).argtypes = [ctypes.c_double, ctypes.c_double]
    L.oracle_gzita.restype = ctypes.c_double
    L.oracle_gzita.argtypes = [ctypes.c_double] * 3
    for fn in ("oracle_md_zeta", "oracle_md_fmz"):
        getattr(L, fn).restype = ctypes.c_double
        getattr(L, fn).argtypes = [ctypes.c_double] * 5
    L.oracle_superbee.restype = ctypes.c_double
    L.oracle_superbee.argtypes = [ctypes.c_double]
    L.oracle_splitmix_u01.restype = ctypes.c_double
    L.oracle_splitmix_u01.argtypes = [ctypes.c_ulonglong, ctypes.c_ulonglong]
    L.oracle_constants.argtypes = [ctypes.POINTER(ctypes.c_double)]
    L.oracle_scalars.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    L.oracle_xknu.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    L.oracle_set_threads.argtypes = [ctypes.c_int]
    _LIBS[name] = L
    return L


def make_cfg(jx, iy, kz, *, hills=(), pert_amp=0.5, pert_levels=10, seed=1234,
             u0=1.0, v0=1.0, divfilter=False, filterpai=False, filtertheta=False,
             rotllr=True):
    c = OracleCfg()
    c.jx, c.iy, c.kz = jx, iy, kz
    c.nhills = len(hills)
    for n, (h, cj, ci, r) in enumerate(hills):
        c.hill_h[n], c.hill_j[n], c.hill_i[n], c.hill_r[n] = h, cj, ci, r
    c.pert_amp, c.pert_levels, c.seed = pert_amp, pert_levels, seed
    c.u0, c.v0 = u0, v0
    c.divfilter, c.filterpai, c.filtertheta = int(divfilter), int(filterpai), int(filtertheta)
    c.rotllr = int(rotllr)
    return c


FIELDS_3D = ("u", "v", "w", "pai", "t", "tetav", "qv", "qc", "qi", "qr", "qs",
             "p", "rho", "tvirt", "qsat", "s", "deltaw", "zdiv2", "fmz", "fmzf",
             "zeta", "ux", "vx", "wx", "qwltot", "qwitot")
FIELDS_KZP1 = ("w", "s", "deltaw", "fmzf")


class Oracle:
    """One oracle domain.  Fields come back as (nk, ni, nj) float64 arrays
    (C order, so the last axis is the reference's contiguous j index)."""

    def __init__(self, cfg, checked=False):
        self.L = lib(checked)
        self.cfg = cfg
        self.h = self.L.oracle_create(ctypes.byref(cfg))
        self.nj, self.ni, self.kz = cfg.jx, cfg.iy, cfg.kz

    def step(self, istep=1, lprint=False):
        d = (ctypes.c_double * 6)()
        bad = self.L.oracle_step(self.h, istep, int(lprint), d)
        return bad, list(d)

    def phase(self, p):
        self.L.oracle_phase(self.h, p)

    def stagger(self, to_x):
        self.L.oracle_stagger(self.h, int(to_x))

    def set_map_factors(self, msfu, msfv, msfx):
        """Whole bounded arrays in the layout get_bounded returns."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (msfu, msfv, msfx)]
        self.L.oracle_set_map_factors(self.h, *[a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for a in arrs])

    def filter(self, which):
        self.L.oracle_filter(self.h, int(which))

    def divdamp(self):
        self.L.oracle_divdamp(self.h)

    def wafone(self, name):
        if self.L.oracle_wafone(self.h, name.encode()) < 0:
            raise KeyError(name)

    def get(self, name):
        nk = self.kz + 1 if name in FIELDS_KZP1 else self.kz
        if name in FIELDS_3D:
            out = np.empty((nk, self.ni, self.nj))
        else:
            out = np.empty((self.ni, self.nj))
        r = self.L.oracle_get(self.h, name.encode(), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        if r < 0:
            raise KeyError(name)
        return out

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        r = self.L.oracle_set(self.h, name.encode(), a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        if r < 0:
            raise KeyError(name)

    def get_bounded(self, name):
        lb = (ctypes.c_int * 3)()
        ub = (ctypes.c_int * 3)()
        nd = self.L.oracle_get_bounded(self.h, name.encode(), None, lb, ub)
        if nd < 0:
            raise KeyError(name)
        shape = [ub[d] - lb[d] + 1 for d in range(3)]
        out = np.empty(shape[::-1])
        self.L.oracle_get_bounded(self.h, name.encode(),
                                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), lb, ub)
        return out, tuple(lb), tuple(ub)

    def close(self):
        if self.h:
            self.L.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
