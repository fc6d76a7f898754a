"""The implicit-w column solve staged by TMA with its column state in TMEM
(k_sound_column_tm, tuning bit 32, FP32 storage; k_sound_column_tw with
bit 128 or 256) against the one-thread-per-column kernel and the oracle,
and its bounded waits.

  * Against k_sound_column<float> on the same state: the same FP32/FP64
    arithmetic per level in the same order, so the steps agree to the last
    bit when the compiler contracts both alike; bound 1e-6 relative L2
    (printed: the measured difference).  Sizes cover partial tiles (jx not a
    multiple of 32, iy not a multiple of 4), kz from 13 to the largest the
    TMEM columns hold (64) and the last-substep path.
  * Against the oracle: tests/test_gpu_mixed.py runs 100 steps with this
    kernel (tuning [32, 56]).
  * A bounded wait that runs out: a test hook leaves one staged chunk
    unissued, the wait on it gives up after about a millisecond,
    moloch_gpu_sync returns MOLOCH_ERR_TIMEOUT (6), and the next steps on a
    fresh state are correct again (the context stays usable).
"""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "w", "pai", "t", "qv", "qc", "tetav", "s", "deltaw")


def _pair(dm, jx, iy, kz, base, hills, **kw):
    a = dm.Moloch(jx, iy, kz, mode="fp32_mixed")
    b = dm.Moloch(jx, iy, kz, mode="fp32_mixed")
    for g in (a, b):
        g.setup_idealized(hills=hills, **kw)
    a.set_tuning([16, base])
    b.set_tuning([16, base | 32])
    return a, b


@pytest.mark.parametrize("jx,iy,kz", [(64, 44, 30), (36, 29, 13), (96, 37, 60), (128, 64, 64), (40, 33, 40)])
def test_staged_column_matches_column_kernel(gpu_lib, jx, iy, kz):
    a, b = _pair(gpu_lib, jx, iy, kz, 24, ((500.0, jx / 2, iy / 2, 5.0),), u0=6.0, v0=-4.0)
    for s in (1, 2, 3):
        a.moloch(s)
        b.moloch(s)
    b.run(2, graph=True)
    a.run(2, graph=True)
    worst = {n: rel_l2(b.get(n), a.get(n)) for n in FIELDS}
    print(f"{jx}x{iy}x{kz} staged vs one-thread column solve:", {k: f"{v:.1e}" for k, v in worst.items()})
    assert all(v <= 1e-6 for v in worst.values()), worst
    a.close()
    b.close()


@pytest.mark.parametrize("rows_bit", [128, 256])
@pytest.mark.parametrize("jx,iy,kz", [(64, 44, 30), (36, 29, 13), (96, 37, 60), (128, 64, 64), (40, 33, 41)])
def test_two_word_staged_column_matches_staged(gpu_lib, jx, iy, kz, rows_bit):
    """k_sound_column_tw (tuning bit 128: 12 compute warps, bit 256: 16;
    two words of column state a level in TMEM, the old w and zdiv2b staged
    again for the back-substitution, chunks of 4 levels) against
    k_sound_column_tm: the same arithmetic per level, so the same bits.
    Sizes cover partial tiles in both directions, kz not a multiple of the
    chunk and the largest kz the TMEM columns hold (64)."""
    a, b = _pair(gpu_lib, jx, iy, kz, 24, ((500.0, jx / 2, iy / 2, 5.0),), u0=6.0, v0=-4.0)
    a.set_tuning([16, 56])
    b.set_tuning([16, 56 | rows_bit])
    for s in (1, 2, 3):
        a.moloch(s)
        b.moloch(s)
    b.run(2, graph=True)
    a.run(2, graph=True)
    worst = {n: rel_l2(b.get(n), a.get(n)) for n in FIELDS}
    same = all(np.array_equal(b.get(n), a.get(n)) for n in FIELDS)
    print(f"{jx}x{iy}x{kz} two-word ({rows_bit}) vs four-word staged solve: bit-identical {same}",
          {k: f"{v:.1e}" for k, v in worst.items()})
    assert all(v <= 1e-6 for v in worst.values()), worst
    a.close()
    b.close()


def test_staged_column_is_used_only_where_it_fits(gpu_lib):
    """jx not a multiple of 4 (no TMA row stride) and kz > 64 (TMEM full)
    fall back to the one-thread kernel: results identical to it."""
    for jx, iy, kz in ((37, 20, 12), (32, 16, 70)):
        a, b = _pair(gpu_lib, jx, iy, kz, 24, ((300.0, jx / 2, iy / 2, 4.0),), u0=3.0)
        for s in (1, 2):
            a.moloch(s)
            b.moloch(s)
        for n in FIELDS:
            assert np.array_equal(a.get(n), b.get(n)), (jx, kz, n)
        a.close()
        b.close()


@pytest.mark.parametrize("variant", [56, 56 | 128, 56 | 256])
def test_staged_column_wait_runs_out(gpu_lib, variant):
    jx, iy, kz = 64, 48, 20
    hills = ((400.0, 32.0, 24.0, 4.0),)
    g = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
    ref = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
    for x in (g, ref):
        x.setup_idealized(hills=hills, u0=4.0)
        x.set_tuning([16, variant])
    # each CTA's staged chunk 3 is never issued: the compute warps' wait on
    # it and the loader's wait for that stage to drain both give up after
    # 2e6 cycles (about 1 ms); the kernel reports, drains and returns
    g.set_wait_limit(2_000_000, 3)
    g.moloch(1)
    with pytest.raises(gpu_lib.MolochError) as ei:
        g.sync()
    assert ei.value.code == 6
    g.sync()  # the flag is cleared once reported
    # back to the default limit, a fresh state: the context is usable and the
    # steps are correct again
    g.set_wait_limit(0, -1)
    g.setup_idealized(hills=hills, u0=4.0)
    for s in (1, 2, 3):
        g.moloch(s)
        ref.moloch(s)
    g.sync()
    for n in FIELDS:
        assert np.array_equal(g.get(n), ref.get(n)), n
    g.close()
    ref.close()


def test_corrected_quotient_within_one_ulp(gpu_lib):
    """The FP32 Exner/theta update divides with a reciprocal estimate and one
    residual correction (no slow path).  Against CUDA's IEEE quotient on
    2^20 seeded values: at most 1 ulp apart, over the range the update sees
    (denominator 1 + 0.96 qv + 4.8 qc in [1, 1.2]) and over a wide one."""
    torch = pytest.importorskip("torch")
    import ctypes
    L = gpu_lib.lib()
    rng = np.random.default_rng(17)
    n = 1 << 20
    dev = torch.device("cuda", 0)
    for lo, hi in ((1.0, 1.2), (1e-3, 1e3)):
        a = (rng.uniform(-1.0, 1.0, n) * 10.0 ** rng.uniform(-6, 3, n)).astype(np.float32)
        b = rng.uniform(lo, hi, n).astype(np.float32)
        ta, tb = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
        qc, qi = torch.empty_like(ta), torch.empty_like(ta)
        P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        assert L.moloch_gpu_check_division(P(ta), P(tb), P(qc), P(qi), n, None) == 0
        torch.cuda.synchronize()
        c, i = qc.cpu().numpy().view(np.int32), qi.cpu().numpy().view(np.int32)
        ulps = np.abs(c.astype(np.int64) - i.astype(np.int64))
        print(f"b in [{lo}, {hi}]: {float(np.mean(ulps == 0)):.6f} identical, max {ulps.max()} ulp")
        assert ulps.max() <= 1


def test_fp64_limiter_quotient_within_one_ulp(gpu_lib):
    """The contracting build's FP64 WAF limiter divides by an FP32
    reciprocal estimate refined by two Newton-Raphson steps with one
    residual correction.  Against CUDA's IEEE FP64 quotient on 2^20 seeded
    values: at most 1 ulp apart, for the denominators the limiter sees
    (|b| from its floor 1e-30 up, both signs, field differences of many
    magnitudes) and for denominators outside the FP32 range (the IEEE path)."""
    torch = pytest.importorskip("torch")
    import ctypes
    L = gpu_lib.lib()
    rng = np.random.default_rng(23)
    n = 1 << 20
    dev = torch.device("cuda", 0)
    sign = lambda: np.where(rng.random(n) < 0.5, -1.0, 1.0)  # noqa: E731
    cases = ((-30, 3), (-8, 8), (-300, -40))
    for lo, hi in cases:
        a = sign() * rng.uniform(0.5, 1.0, n) * 10.0 ** rng.uniform(-12, 6, n)
        b = sign() * rng.uniform(0.5, 1.0, n) * 10.0 ** rng.uniform(lo, hi, n)
        ta, tb = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
        qn, qi = torch.empty_like(ta), torch.empty_like(ta)
        P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        assert L.moloch_gpu_check_division_f64(P(ta), P(tb), P(qn), P(qi), n, None) == 0
        torch.cuda.synchronize()
        c, i = qn.cpu().numpy().view(np.int64), qi.cpu().numpy().view(np.int64)
        ulps = np.abs(c - i)
        print(f"|b| in 1e{lo}..1e{hi}: {float(np.mean(ulps == 0)):.6f} identical, max {ulps.max()} ulp")
        assert ulps.max() <= 1
