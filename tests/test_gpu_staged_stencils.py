"""The stencils of sound() staged by TMA (FP32 storage: tiles of 32 x 8
columns marching down the levels, each level's neighbourhood one TMA box
per array, cells outside the domain patched from periodic images and the
stale-halo edge buffers) against the warp-strip kernels they replace:
  * k_momentum_tm (tuning bit 64) against k_momentum_strip;
  * k_divdamp_tm (bits 16 + 128) against k_divdamp_strip.

The arithmetic per point is that of the strip kernels in the same order;
multiply-add contraction may differ where an expression has two products
(a*b + c*d), and in FP32 the WAF limiter turns a last-bit difference into
one of the size of the FP32 error itself, so the bound is 1e-6 relative L2
for the momentum kernel (measured: printed) and 1e-3 for the
divergence/damping kernel, the bound of the other FP32 variant tests.
Sizes: partial tiles in j and i, a domain one tile wide (all four edges in
one tile), the benchmark's proportions, both map-factor branches.
tests/test_gpu_mixed.py runs both kernels 100 steps against the oracle
(tunings [32, 120] and [32, 240]).
"""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "w", "pai", "t", "qv", "qc", "tetav", "s", "deltaw")


@pytest.mark.parametrize("jx,iy,kz,base", [(64, 44, 30, 24), (24, 20, 9, 24), (36, 29, 13, 56), (96, 37, 60, 56),
                                           (128, 64, 16, 16)])
def test_staged_momentum_matches_strips(gpu_lib, jx, iy, kz, base):
    a = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
    b = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
    for g in (a, b):
        g.setup_idealized(hills=((500.0, jx / 2, iy / 2, 5.0),), u0=6.0, v0=-4.0)
    a.set_tuning([16, base | 8])
    b.set_tuning([16, base | 64])
    for s in (1, 2, 3):
        a.moloch(s)
        b.moloch(s)
    a.run(2, graph=True)
    b.run(2, graph=True)
    b.sync()
    worst = {n: rel_l2(b.get(n), a.get(n)) for n in FIELDS}
    print(f"{jx}x{iy}x{kz} staged momentum vs strips:", {k: f"{v:.1e}" for k, v in worst.items()})
    assert all(v <= 1e-6 for v in worst.values()), worst
    a.close()
    b.close()


def test_staged_momentum_needs_aligned_rows(gpu_lib):
    """jx not a multiple of 4 (no TMA row stride): the bit is ignored and the
    strips run, with identical results."""
    a = gpu_lib.Moloch(37, 20, 10, mode="fp32_mixed")
    b = gpu_lib.Moloch(37, 20, 10, mode="fp32_mixed")
    for g in (a, b):
        g.setup_idealized(hills=((300.0, 18.0, 10.0, 4.0),), u0=3.0)
    a.set_tuning([16, 24])
    b.set_tuning([16, 24 | 64])
    for s in (1, 2):
        a.moloch(s)
        b.moloch(s)
    for n in FIELDS:
        assert np.array_equal(a.get(n), b.get(n)), n
    a.close()
    b.close()


@pytest.mark.parametrize("jx,iy,kz,rotllr", [(64, 44, 30, 1), (24, 20, 9, 1), (36, 29, 13, 0), (96, 37, 60, 1),
                                             (128, 64, 16, 0)])
def test_staged_divdamp_matches_strips(gpu_lib, jx, iy, kz, rotllr):
    a = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed", rotllr=rotllr)
    b = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed", rotllr=rotllr)
    for g in (a, b):
        g.setup_idealized(hills=((500.0, jx / 2, iy / 2, 5.0),), u0=6.0, v0=-4.0)
    a.set_tuning([16, 16 | 8])
    b.set_tuning([16, 16 | 128 | 8])
    for s in (1, 2, 3):
        a.moloch(s)
        b.moloch(s)
    a.run(2, graph=True)
    b.run(2, graph=True)
    b.sync()
    worst = {n: rel_l2(b.get(n), a.get(n)) for n in FIELDS}
    print(f"{jx}x{iy}x{kz} rotllr={rotllr} staged divergence/damping vs strips:",
          {k: f"{v:.1e}" for k, v in worst.items()})
    assert all(v <= 1e-3 for v in worst.values()), worst
    a.close()
    b.close()
