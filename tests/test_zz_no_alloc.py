"""moloch_gpu_wafone_noalloc: WAF advection of one field for callers that
own all device memory and cannot let a library call cudaMalloc (a Fortran
model with its own CUDA/OpenACC data regions, a framework with its own
memory pool).  Its work arrays live in a fixed device array inside the
library instead of being allocated.

The test calls it through the C ABI on device buffers the test itself
allocates, and compares it with the advection phase of the existing entry
point (moloch_gpu_phase, exact FP64 build) on the same state, for two calls
in a row.  Tolerance: relative L2 <= 1e-13 (both paths evaluate the same
FP64 expressions without multiply-add contraction).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def test_wafone_noalloc_matches_advection_phase(gpu_lib):
    torch = pytest.importorskip("torch")
    dm = gpu_lib
    L = dm.lib()
    jx, iy, kz = 40, 33, 16
    g = dm.Moloch(jx, iy, kz, mode="fp64_exact")
    g.setup_idealized(hills=((400.0, 20.0, 16.0, 5.0),), u0=5.0, v0=-3.0)
    g.phase(0)
    g.phase(1)  # the state advection() starts from: sound() done, s complete
    before = {n: g.get(n) for n in ("tetav", "pai", "qv", "s", "u", "v", "fmz", "fmzf", "msfu", "msfv", "msfx")}
    dzita = g.get_1d("zita")[kz - 1]  # mo_dzita = zita(kz)
    g.phase(2)  # advection() through the existing entry point
    after = {n: g.get(n) for n in ("tetav", "pai", "qv")}

    dev = torch.device("cuda", 0)

    def T(a):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)

    def P(t):
        return ctypes.c_void_p(t.data_ptr())

    ro = {n: T(before[n]) for n in ("s", "u", "v", "fmz", "fmzf", "msfu", "msfv", "msfx")}
    dta = g.params.dt / g.params.mo_nadv
    for name in ("tetav", "pai"):  # two calls in a row share the fixed work arrays
        pp = T(before[name])
        rc = L.moloch_gpu_wafone_noalloc(P(pp), P(ro["s"]), P(ro["u"]), P(ro["v"]), P(ro["fmz"]), P(ro["fmzf"]),
                                         P(ro["msfu"]), P(ro["msfv"]), P(ro["msfx"]), jx, iy, kz,
                                         dta, g.params.dx, dzita, 1, None)
        assert rc == 0, L.moloch_gpu_last_error()
        torch.cuda.synchronize()
        e = _rel_l2(pp.cpu().numpy(), after[name])
        assert e <= 1e-13, (name, e)

    # sizes beyond the fixed work arrays are refused before any launch
    pp = T(before["qv"])
    rc = L.moloch_gpu_wafone_noalloc(P(pp), P(ro["s"]), P(ro["u"]), P(ro["v"]), P(ro["fmz"]), P(ro["fmzf"]),
                                     P(ro["msfu"]), P(ro["msfv"]), P(ro["msfx"]), 512, 512, 60,
                                     dta, g.params.dx, dzita, 1, None)
    assert rc == 1 and b"exceeds" in L.moloch_gpu_last_error()
    g.close()
