"""FP32 storage with the FP64 tridiagonal solve (MOLOCH_FP32_MIXED) against
the FP64 oracle, through the C ABI.

Tolerances (stated error of the FP32 path):
  * 100 steps at the reference defaults 100 x 100 x 30 with the seeded
    +-0.5 K theta noise: RMSE of theta <= 0.01 K, of u, v, w <= 0.01 m/s,
    relative L2 of pai, t, qv <= 5e-5 (measured on GB300: theta 1.1e-3 K,
    u/v 1.2e-4 m/s, w 5.6e-5 m/s, pai 7.0e-6, t 8.6e-6, qv 1.5e-5);
  * the FP64 column sums of the lprint diagnostics (mass, energy) of the
    FP32 path agree with those of the FP64 path to 1e-6 relative, and the
    printed max/min of ps, u, v to 1e-4 relative.
"""
import numpy as np
import pytest

from tests.conftest import rel_l2
from tests.test_gpu_parity import pair

pytestmark = pytest.mark.gpu


def rmse(a, b):
    return float(np.sqrt(np.mean((np.asarray(a) - np.asarray(b)) ** 2)))


@pytest.mark.parametrize("tuning", [[1, 0], [32, 11], [32, 24], [32, 56], [32, 184], [32, 312]])
def test_mixed_100_steps_vs_oracle(oracle_mod, gpu_lib, tuning):
    """Default kernels, and the FP32 variants the autotuner picks on GB300
    (warp strips for the horizontal WAF and the momentum, k-marching or
    fused warp-strip divergence and damping, the column solve staged by
    TMA with its state in TMEM, the momentum update and the fused
    divergence/damping staged by TMA)."""
    o, g = pair(oracle_mod, gpu_lib, 100, 100, 30, mode="fp32_mixed")
    g.set_tuning(tuning)
    for s in range(1, 101):
        o.step(s)
        g.moloch(s)
    th_g = g.get("t") / g.get("pai")
    th_o = o.get("t") / o.get("pai")
    err = {"theta_K": rmse(th_g, th_o), "u": rmse(g.get("u"), o.get("u")), "v": rmse(g.get("v"), o.get("v")),
           "w": rmse(g.get("w"), o.get("w"))}
    rel = {n: rel_l2(g.get(n), o.get(n)) for n in ("pai", "t", "qv")}
    print("fp32_mixed after 100 steps:", {k: f"{v:.2e}" for k, v in {**err, **rel}.items()})
    assert err["theta_K"] <= 0.01 and err["u"] <= 0.01 and err["v"] <= 0.01 and err["w"] <= 0.01, err
    assert all(v <= 5e-5 for v in rel.values()), rel


def test_mixed_column_sums_vs_fp64(gpu_lib):
    a = gpu_lib.Moloch(64, 48, 20, mode="fp64")
    b = gpu_lib.Moloch(64, 48, 20, mode="fp32_mixed")
    for g in (a, b):
        g.setup_idealized(hills=((400.0, 32.0, 24.0, 5.0),), u0=5.0)
    for s in range(1, 6):
        da = a.moloch(s, lprint=(s == 5))
        db = b.moloch(s, lprint=(s == 5))
    assert abs(db.mass - da.mass) <= 1e-6 * abs(da.mass)
    assert abs(db.energy - da.energy) <= 1e-6 * abs(da.energy)
    for f in ("maxps", "minps", "maxu", "minu", "maxv", "minv"):
        x, y = getattr(db, f), getattr(da, f)
        assert abs(x - y) <= 1e-4 * max(abs(y), 1.0), (f, x, y)
