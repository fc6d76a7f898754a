"""moloch_gpu_wafone_noalloc: WAF advection of one field for callers that
own all device memory and cannot let a library call cudaMalloc (a Fortran
model with its own CUDA/OpenACC data regions, a framework with its own
memory pool).  Its work arrays live in a fixed device array inside the
library instead of being allocated.

The tests call it through the C ABI on device buffers the test itself
allocates before the first call:
  * against the advection phase of the existing entry point
    (moloch_gpu_phase, exact FP64 build) on the same state, for three calls
    in a row; the device's free memory (cudaMemGetInfo) is the same after
    the second and third calls as after the first, which is where the CUDA
    runtime may load the code and reserve the fixed array;
  * against the oracle's wafone on a state with map factors within 5 % of 1
    (periodic rings), in both map-factor branches (rotllr 1 and 0), for two
    calls in a row.
Tolerance: relative L2 <= 1e-13 (the same FP64 expressions without
multiply-add contraction on both sides).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def _dev(torch):
    dev = torch.device("cuda", 0)

    def T(a):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)

    def P(t):
        return ctypes.c_void_p(t.data_ptr())

    return T, P


def _call(L, P, pp, ro, jx, iy, kz, dta, dx, dzita, rotllr):
    return L.moloch_gpu_wafone_noalloc(P(pp), P(ro["s"]), P(ro["u"]), P(ro["v"]), P(ro["fmz"]), P(ro["fmzf"]),
                                       P(ro["msfu"]), P(ro["msfv"]), P(ro["msfx"]), jx, iy, kz,
                                       dta, dx, dzita, rotllr, None)


def test_wafone_noalloc_matches_advection_phase(gpu_lib):
    torch = pytest.importorskip("torch")
    dm = gpu_lib
    L = dm.lib()
    jx, iy, kz = 40, 33, 16
    g = dm.Moloch(jx, iy, kz, mode="fp64_exact")
    g.setup_idealized(hills=((400.0, 20.0, 16.0, 5.0),), u0=5.0, v0=-3.0)
    g.phase(0)
    g.phase(1)  # the state advection() starts from: sound() done, s complete
    names = ("tetav", "pai", "qv")
    before = {n: g.get(n) for n in names + ("s", "u", "v", "fmz", "fmzf", "msfu", "msfv", "msfx")}
    dzita = g.get_1d("zita")[kz - 1]  # mo_dzita = zita(kz)
    g.phase(2)  # advection() through the existing entry point
    after = {n: g.get(n) for n in names}

    T, P = _dev(torch)
    ro = {n: T(before[n]) for n in ("s", "u", "v", "fmz", "fmzf", "msfu", "msfv", "msfx")}
    pps = {n: T(before[n]) for n in names}
    big = T(before["qv"])
    torch.cuda.synchronize()
    dta = g.params.dt / g.params.mo_nadv
    free = []
    for name in names:  # calls in a row share the fixed work arrays
        rc = _call(L, P, pps[name], ro, jx, iy, kz, dta, g.params.dx, dzita, 1)
        assert rc == 0, L.moloch_gpu_last_error()
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        e = _rel_l2(pps[name].cpu().numpy(), after[name])
        assert e <= 1e-13, (name, e)
    # nothing was reserved after the first call (which may load the code)
    assert free[1] == free[0] and free[2] == free[0], free

    # sizes beyond the fixed work arrays, and kz beyond a grid dimension,
    # are refused before any launch
    rc = _call(L, P, big, ro, 512, 512, 60, dta, g.params.dx, dzita, 1)
    assert rc == 1 and b"exceeds" in L.moloch_gpu_last_error()
    rc = _call(L, P, big, ro, 4, 4, 70000, dta, g.params.dx, dzita, 1)
    assert rc == 1 and b"kz" in L.moloch_gpu_last_error()
    g.close()


@pytest.mark.parametrize("rotllr", [1, 0])
def test_wafone_noalloc_matches_oracle_with_map_factors(oracle_mod, gpu_lib, rotllr):
    torch = pytest.importorskip("torch")
    from tests.test_gpu_parity_production import periodic_map_factors
    L = gpu_lib.lib()
    jx, iy, kz = 36, 28, 12
    o = oracle_mod.Oracle(oracle_mod.make_cfg(jx, iy, kz, hills=((400.0, 18.0, 14.0, 4.0),), u0=5.0, v0=-3.0,
                                              rotllr=bool(rotllr)))
    msfu, msfv, msfx = periodic_map_factors(jx, iy, 11)
    o.set_map_factors(msfu[None], msfv[None], msfx[None])
    o.phase(0)
    o.phase(1)
    # advection() refreshes the u, v rings in uvstagtox (:1389-1417) before
    # its wafone calls; wafone reads u along j and v along i, which that
    # refresh makes periodic images of the interior
    o.stagger(1)
    scal = (ctypes.c_double * 9)()
    oracle_mod.lib().oracle_scalars(o.h, scal)
    dt, dx, dzita, nadv = scal[0], scal[1], scal[2], scal[6]
    T, P = _dev(torch)
    ro = {n: T(o.get(n)) for n in ("s", "u", "v", "fmz", "fmzf")}
    ro.update(msfu=T(msfu[:, 1:-1]), msfv=T(msfv[1:-1, :]), msfx=T(msfx))
    for name in ("tetav", "qv"):
        pp = T(o.get(name))
        torch.cuda.synchronize()
        rc = _call(L, P, pp, ro, jx, iy, kz, dt / nadv, dx, dzita, rotllr)
        assert rc == 0, L.moloch_gpu_last_error()
        o.wafone(name)
        e = _rel_l2(pp.cpu().numpy(), o.get(name))
        assert e <= 1e-13, (name, rotllr, e)
    o.close()
