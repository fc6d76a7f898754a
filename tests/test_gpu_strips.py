"""Warp-strip kernels with two columns per lane against the one-column
strips (FP32 storage): the same expressions in the same order, so the
results are bit-identical.  Momentum (tuning bit 64 with 8): 62 output
columns per warp; sizes cover one strip across the whole domain (jx = 24),
strips ending inside and at the seam (jx = 62, 64, 126, 128, 130), the
non-ROTLLR branch with map factors other than 1, and odd jx (the tuning
falls back to the one-column strips)."""
import numpy as np
import pytest

from tests.test_gpu_parity_production import periodic_map_factors

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "w", "pai", "t", "qv", "tetav")


def run(dm, jx, iy, kz, tuning, rotllr=True, steps=3):
    g = dm.Moloch(jx, iy, kz, mode="fp32_mixed", rotllr=rotllr)
    g.setup_idealized(hills=((400.0, jx / 2.0, iy / 2.0, 4.0),), u0=6.0, v0=-3.0, pert_amp=0.5, pert_levels=kz)
    if not rotllr:
        msfu, msfv, msfx = periodic_map_factors(jx, iy, 9)
        for name, a in (("msfu", msfu), ("msfv", msfv), ("msfx", msfx)):
            g.upload(name, a.T)
        g.init()
    g.set_tuning(tuning)
    for s in range(1, steps + 1):
        g.moloch(s)
    out = {f: g.get(f) for f in FIELDS}
    g.close()
    return out


@pytest.mark.parametrize("jx,iy,kz", [(24, 20, 8), (62, 40, 10), (64, 48, 12), (126, 40, 10), (128, 33, 10),
                                      (130, 64, 6), (37, 29, 8)])
@pytest.mark.parametrize("sound", [8, 24])  # momentum strips; with the fused divergence/damping strips
def test_momentum_pair_strips_match_one_column_strips(gpu_lib, jx, iy, kz, sound):
    a = run(gpu_lib, jx, iy, kz, [4, sound])
    b = run(gpu_lib, jx, iy, kz, [4, sound | 64])
    for f in FIELDS:
        assert np.array_equal(a[f], b[f]), (f, float(np.max(np.abs(a[f] - b[f]))))


@pytest.mark.parametrize("jx,iy,kz", [(64, 40, 10), (128, 33, 8)])
def test_momentum_pair_strips_non_rotllr(gpu_lib, jx, iy, kz):
    a = run(gpu_lib, jx, iy, kz, [4, 24], rotllr=False)
    b = run(gpu_lib, jx, iy, kz, [4, 88], rotllr=False)
    for f in FIELDS:
        assert np.array_equal(a[f], b[f]), (f, float(np.max(np.abs(a[f] - b[f]))))
