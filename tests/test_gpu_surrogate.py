"""The learned acoustic-cycle surrogate on the GPU, through the C ABI.

* gradients: one forward+backward pass of the tcgen05 MLP against the NumPy
  oracle with the same BF16 roundings -- relative L2 <= 5e-3 per gradient
  (only the FP32 summation order differs, which can move a stored BF16
  activation by one unit in the last place);
* inference + commit: one sound() call replaced by the surrogate, every
  committed field and s against the oracle -- relative L2 of the increment
  <= 5e-3;
* fallback: a surrogate whose check rejects every cycle leaves the step
  bit-identical to the plain FP32 step (graph and stepwise);
* judge: judge cycles run the plain loop; a judge with tol 0 keeps the
  surrogate off with a doubling interval (bit-identical to the plain step),
  a judge with an infinite tol enables it between judge cycles (schedule
  and counts checked);
* training: collect, prepare, train on a small hilly domain; the validation
  loss falls and the surrogate run stays within a stated error of the FP64
  run (see the test for the bound).
"""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

STATE = ("u", "v", "w", "pai", "tetav")


def _random_params(sur, rng, scale=1.0):
    P = []
    for l in range(4):
        W, b = sur.param(l)
        fan = W.shape[1]
        W = rng.normal(0, scale / np.sqrt(fan), W.shape).astype(np.float32)
        b = rng.normal(0, 0.1, b.shape).astype(np.float32)
        sur.set_param(l, W, b)
        P.append((W.astype(np.float64), b.astype(np.float64)))
    return P


def test_sur_gradients_match_oracle(gpu_lib):
    from oracle import mlp_oracle as mo
    kz, B = 8, 128
    sur = gpu_lib.Surrogate(kz, capacity=256, batch=B, seed=3)
    d = sur.dims()
    rng = np.random.default_rng(11)
    P = _random_params(sur, rng, scale=1.5)
    X = np.zeros((B, d["kin"]), np.float32)
    X[:, :d["nin"]] = rng.normal(size=(B, d["nin"]))
    T = np.zeros((B, d["nop"]), np.float32)
    T[:, :d["nout"]] = rng.normal(size=(B, d["nout"]))
    loss_ref, grads = mo.backward(P, X, T, d["nout"])
    for l in range(4):
        loss, gW, gb = sur.gradients(X, T, l)
        assert abs(loss - loss_ref) <= 1e-4 * loss_ref, (loss, loss_ref)
        assert rel_l2(gW, grads[l][0]) <= 5e-3, (l, rel_l2(gW, grads[l][0]))
        assert rel_l2(gb, grads[l][1]) <= 5e-3, (l, rel_l2(gb, grads[l][1]))
    sur.close()


def _state(g):
    return {f: g.get(f) for f in STATE}


@pytest.mark.parametrize("jx,iy,kz,tuning", [(24, 20, 8, [1, 0]), (37, 29, 12, [1, 0]), (37, 29, 12, [32, 11]),
                                             (24, 20, 8, [16, 7]), (37, 29, 12, [32, 24]), (24, 20, 8, [16, 39])])
def test_sur_cycle_matches_oracle(gpu_lib, jx, iy, kz, tuning):
    """tuning: the plain kernel variants that must all stand aside on a
    committed cycle (one level per thread, strips, k-marching, the fused
    divergence/damping strips, which flip the u/v buffers twice a substep,
    and the column solve staged by TMA with its state in TMEM)."""
    from oracle import mlp_oracle as mo
    g = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
    g.setup_idealized(hills=((400.0, jx / 2, iy / 2, 3.0),), u0=5.0, v0=-3.0)
    g.set_tuning(tuning)
    g.phase(0)
    pre = _state(g)
    sur = gpu_lib.Surrogate(kz, capacity=256, batch=128, seed=5)
    d = sur.dims()
    rng = np.random.default_rng(jx)
    P = _random_params(sur, rng)
    feats = mo.features(pre)
    x5 = feats.reshape(-1, 5, kz, 9)
    xmean = x5.mean(axis=(0, 3)).astype(np.float32)
    xstd = (x5.std(axis=(0, 3)) + 1e-3).astype(np.float32)
    ymean = rng.normal(0, 0.05, (5, kz)).astype(np.float32)
    ystd = rng.uniform(0.2, 0.5, (5, kz)).astype(np.float32)
    sur.set_stats(xmean, xstd, ymean, ystd)
    sur.attach(g, threshold=1e30, judge_every=0)
    g.phase(1)
    assert sur.counts() == (1, 0)
    post = _state(g)
    post["s"] = g.get("s")
    Xn = mo.normalise(feats, xmean.astype(np.float64), xstd.astype(np.float64), d["kin"])
    Y, _, _ = mo.forward(P, Xn.astype(np.float32))
    inc = Y[:, :5 * kz].reshape(-1, 5, kz) * ystd + ymean
    inc = inc.transpose(1, 2, 0).reshape(5, kz, iy, jx)
    zita = g.get_1d("zita")
    gz = mo.gzita(zita, g.params.mo_ztop, g.params.mo_a0)
    want = mo.apply(pre, inc, g.params.mo_nsound, g.get("hx"), g.get("hy"), gz, g.get("fmzf"))
    for f in STATE:
        e = rel_l2(post[f] - pre[f], want[f] - pre[f])
        assert e <= 5e-3, (f, e)
    assert rel_l2(post["s"], want["s"]) <= 5e-3, rel_l2(post["s"], want["s"])
    sur.close()
    g.close()


def _splitmix(seed, n):
    """The collector's column sampler: splitmix64 draws."""
    m = (1 << 64) - 1
    st, out = seed, []
    for _ in range(n):
        st = (st + 0x9E3779B97F4A7C15) & m
        z = st
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
        out.append(z ^ (z >> 31))
    return out


@pytest.mark.parametrize("tuning", [[1, 0], [32, 24]])
def test_sur_collected_pairs_match_oracle(gpu_lib, tuning):
    """Training pairs of the first collected cycle against the feature
    layout of the oracle and the increments of a twin domain run through
    the same phases: bit for bit (the features are copies of state values,
    the increments one FP32 subtraction)."""
    from oracle import mlp_oracle as mo
    jx, iy, kz, take, seed = 37, 29, 8, 96, 11
    a = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
    b = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
    for g in (a, b):
        g.setup_idealized(hills=((400.0, jx / 2, iy / 2, 3.0),), u0=5.0, v0=-3.0)
        g.set_tuning(tuning)
    sur = gpu_lib.Surrogate(kz, capacity=1024, batch=128)
    n = sur.collect(a, 1, cols_per_cycle=take, seed=seed)
    assert n == take * a.params.mo_nadv
    X, T = sur.pair_data(0, take)
    b.phase(0)
    pre = _state(b)
    b.phase(1)
    post = _state(b)
    cols = np.array([z % (jx * iy) for z in _splitmix(seed, take)])
    assert np.array_equal(X, mo.features(pre)[cols].astype(np.float32))
    def lv(st, f):  # the field's kz levels as FP32 (w: levels 2..kz+1)
        return (st[f][1:kz + 1] if f == "w" else st[f]).astype(np.float32)
    inc = np.stack([lv(post, f) - lv(pre, f) for f in STATE])  # [5][kz][iy][jx], FP32 differences
    want = inc.reshape(5 * kz, iy * jx)[:, cols].T
    assert np.array_equal(T, want)
    sur.close()
    a.close()
    b.close()


@pytest.mark.parametrize("tuning", [[1, 0], [32, 24], [32, 56]])
def test_sur_fallback_is_bit_identical(gpu_lib, tuning):
    jx, iy, kz = 32, 24, 10
    a = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
    b = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
    for g in (a, b):
        g.setup_idealized(hills=((300.0, 16.0, 12.0, 3.0),), u0=4.0)
        g.set_tuning(tuning)
    sur = gpu_lib.Surrogate(kz, capacity=256, batch=128)
    _random_params(sur, np.random.default_rng(2))
    sur.set_stats(np.zeros((5, kz)), np.ones((5, kz)), np.zeros((5, kz)), np.ones((5, kz)))
    sur.attach(b, threshold=0.0, judge_every=0)  # nothing passes: every cycle falls back
    for s in range(1, 3):
        a.moloch(s)
        b.moloch(s)
    a.run(2, graph=True)
    b.run(2, graph=True)
    nadv = a.params.mo_nadv
    assert sur.counts() == (4 * nadv, 4 * nadv)
    for f in ("u", "v", "w", "pai", "t", "qv", "ps", "s"):
        assert np.array_equal(a.get(f), b.get(f)), f
    sur.close()
    a.close()
    b.close()


@pytest.mark.parametrize("tol,judge_every", [(0.0, 2), (1e30, 3)])
def test_sur_judge(gpu_lib, tol, judge_every):
    jx, iy, kz = 32, 24, 10
    a = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
    b = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
    for g in (a, b):
        g.setup_idealized(hills=((300.0, 16.0, 12.0, 3.0),), u0=4.0)
    sur = gpu_lib.Surrogate(kz, capacity=256, batch=128)
    _random_params(sur, np.random.default_rng(4), scale=0.3)
    sur.set_stats(np.zeros((5, kz)), np.ones((5, kz)), np.zeros((5, kz)), np.full((5, kz), 1e-4))
    sur.attach(b, threshold=1e30, judge_every=judge_every, tol=tol)
    a.run(2, graph=True)
    b.run(2, graph=True)
    a.moloch(3)
    b.moloch(3)
    n = 3 * a.params.mo_nadv
    c = sur.stats_counts()
    # judge schedule: first cycle, then judge_every later after a pass,
    # doubling (up to 16 x judge_every) after a failure
    judged, nxt, iv = 0, 0, judge_every
    for cyc in range(n):
        if cyc == nxt:
            judged += 1
            iv = judge_every if tol > 0 else min(2 * iv, 16 * judge_every)
            nxt = cyc + iv
    assert c["cycles"] == n and c["judged"] == judged, (c, judged)
    if tol == 0.0:
        assert c["judge_rejections"] == judged and c["plain"] == n
        for f in ("u", "v", "w", "pai", "t", "ps"):
            assert np.array_equal(a.get(f), b.get(f)), f
    else:
        assert c["judge_rejections"] == 0 and c["plain"] == judged
        assert np.isfinite(c["last_judge_error"])
        assert not np.array_equal(a.get("pai"), b.get("pai"))
    sur.close()
    a.close()
    b.close()


def test_sur_train_and_run(gpu_lib):
    """Train on 6 plain steps of a 64 x 64 x 12 hilly domain, then run 6
    steps with the surrogate from the same initial state.  Error measure:
    RMS difference of tetav from the FP64 run.  Bound: the surrogate run
    stays within 0.05 K of FP64 after 6 steps, and the validation loss
    drops below 0.5 of its untrained value."""
    jx, iy, kz = 64, 64, 12
    setup = dict(hills=((500.0, 32.0, 32.0, 5.0),), u0=6.0, v0=2.0, pert_amp=0.5, pert_levels=6)
    col = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
    col.setup_idealized(**setup)
    sur = gpu_lib.Surrogate(kz, capacity=16384, batch=256, seed=1)
    n = sur.collect(col, 6, cols_per_cycle=512)
    assert n == 6 * col.params.mo_nadv * 512
    sur.prepare(0.1)
    _, v0 = sur.train(0)
    tl, vl = sur.train(2000, lr=1e-3)
    print(f"surrogate: val loss {v0:.4g} -> {vl:.4g} (train {tl:.4g})")
    assert np.isfinite(vl) and vl < 0.5 * v0
    ref = gpu_lib.Moloch(jx, iy, kz, mode="fp64")
    pl = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
    run = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
    for g in (ref, pl, run):
        g.setup_idealized(**setup)
    sur.attach(run)
    for g in (ref, pl, run):
        g.run(6, graph=True)
    c = sur.stats_counts()
    e_pl = np.sqrt(np.mean((pl.get("tetav") - ref.get("tetav")) ** 2))
    e_sur = np.sqrt(np.mean((run.get("tetav") - ref.get("tetav")) ** 2))
    print(f"surrogate: {c}, tetav rms vs fp64: plain fp32 {e_pl:.3g}, surrogate {e_sur:.3g}")
    assert c["cycles"] == 6 * run.params.mo_nadv
    assert np.isfinite(e_sur) and e_sur <= 0.05
    sur.close()
    for g in (col, ref, pl, run):
        g.close()


def test_sur_training_and_judged_run_are_deterministic(gpu_lib):
    """Two identical collect / train / judged-run sequences from the same
    seeds give bit-identical weights, the same judge verdicts and
    bit-identical states: every reduction on the training and judging path
    has a fixed order (GEMM tiles over the full K, serial column sums, the
    judge's two-level sum), so two runs of one configuration cannot end at
    different errors."""
    jx, iy, kz = 48, 40, 10
    setup = dict(hills=((500.0, 24.0, 20.0, 4.0),), u0=6.0, v0=2.0, pert_amp=0.5, pert_levels=5)

    def once():
        col = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
        col.setup_idealized(**setup)
        sur = gpu_lib.Surrogate(kz, capacity=8192, batch=128, seed=3)
        sur.collect(col, 4, cols_per_cycle=256)
        sur.prepare(0.1)
        tl, vl = sur.train(300, lr=1e-3)
        weights = [sur.param(layer) for layer in range(4)]
        run = gpu_lib.Moloch(jx, iy, kz, mode="fp32_mixed")
        run.setup_idealized(**setup)
        sur.attach(run, judge_every=2, tol=0.3)
        run.run(6, graph=True)
        state = {f: run.get(f) for f in ("u", "v", "w", "pai", "t")}
        counts = sur.stats_counts()
        sur.close()
        col.close()
        run.close()
        return tl, vl, weights, state, counts

    a, b = once(), once()
    assert a[0] == b[0] and a[1] == b[1], (a[:2], b[:2])
    for (wa, ba), (wb, bb) in zip(a[2], b[2]):
        assert np.array_equal(wa, wb) and np.array_equal(ba, bb)
    assert a[4] == b[4], (a[4], b[4])
    for f in a[3]:
        assert np.array_equal(a[3][f], b[3][f]), f
