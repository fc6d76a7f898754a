"""The C-ABI library loads and exports every function include/ declares;
host-side argument checks that run before any CUDA call."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(moloch_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_reference_entry_points():
    names = declared_functions()
    for n in ("moloch_gpu_create", "moloch_gpu_upload", "moloch_gpu_init", "moloch_gpu_step",
              "moloch_gpu_download", "moloch_gpu_destroy"):
        assert n in names


def test_library_exports_every_declared_symbol(gpu_lib):
    L = gpu_lib.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    # the Python binding covers every declared function too
    assert set(declared_functions()) <= set(gpu_lib._PROTOS)


def test_default_params_match_reference_param(gpu_lib):
    p = gpu_lib.Params()
    gpu_lib.lib().moloch_gpu_default_params(ctypes.byref(p))
    # nompi/regcm_dynamical_core.F90:99-113
    assert (p.dt, p.dx, p.mo_ztop, p.mo_h, p.mo_a0, p.mo_anu2) == (30.0, 3000.0, 36000.0, 12000.0, 0.0, 0.6)
    assert (p.mo_nadv, p.mo_nsound, p.rotllr) == (3, 5, 1)
    assert (p.mo_divfilter, p.do_filterpai, p.do_filtertheta) == (0, 0, 0)


def test_create_rejects_bad_arguments_before_touching_the_gpu(gpu_lib):
    L = gpu_lib.lib()
    p = gpu_lib.Params()
    L.moloch_gpu_default_params(ctypes.byref(p))
    h = ctypes.c_void_p()
    g = gpu_lib.Grid(3, 10, 10)
    assert L.moloch_gpu_create(ctypes.byref(g), ctypes.byref(p), None, ctypes.byref(h)) == 1
    assert b"too small" in L.moloch_gpu_last_error()
    g = gpu_lib.Grid(10, 10, 10)
    p.mode = 7
    assert L.moloch_gpu_create(ctypes.byref(g), ctypes.byref(p), None, ctypes.byref(h)) == 1
    p.mode = 0
    p.mo_nsound = 0
    assert L.moloch_gpu_create(ctypes.byref(g), ctypes.byref(p), None, ctypes.byref(h)) == 1
    assert L.moloch_gpu_create(None, ctypes.byref(p), None, ctypes.byref(h)) == 1
    assert L.moloch_gpu_step(None, 1, 0, None) == 1
    assert L.moloch_gpu_destroy(None) == 0


def test_field_bounds_follow_reference_allocations(gpu_lib):
    b = gpu_lib.field_bounds
    # nompi/mod_atmosphere.F90:107-126
    assert b("u", 100, 90, 30) == ((-1, 102), (0, 91), (1, 30))
    assert b("v", 100, 90, 30) == ((0, 101), (-1, 92), (1, 30))
    assert b("w", 100, 90, 30) == ((1, 100), (1, 90), (1, 31))
    assert b("qx", 100, 90, 30) == ((0, 101), (0, 91), (1, 30), (1, 5))
    assert b("zeta", 100, 90, 30) == ((-1, 102), (-1, 92), (1, 30))
