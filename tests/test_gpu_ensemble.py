"""Batched ensembles: members of uneven size advanced by one launch per
kernel (and one graph per step) must match the same members advanced one
at a time through their own handles.  Both paths run the same kernel bodies
(FP64: rel. L2 <= 1e-13; FP32 storage: <= 1e-6)."""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

SHAPES = [(40, 33, 16, 3.0, 11), (24, 20, 12, 7.5, 12), (37, 29, 10, 0.5, 13), (64, 48, 20, 5.0, 14)]
FIELDS = ("u", "v", "w", "pai", "t", "qv", "ps", "tetav")


def members(dm, mode, stream=None):
    out = []
    for jx, iy, kz, u0, seed in SHAPES:
        m = dm.Moloch(jx, iy, kz, mode=mode, stream=stream)
        m.setup_idealized(pert_amp=1.0, pert_levels=kz, seed=seed, u0=u0, v0=0.5 * u0,
                          hills=((300.0, jx / 2.0, iy / 2.0, 4.0),))
        out.append(m)
    return out


@pytest.fixture
def stream():
    torch = pytest.importorskip("torch")
    s = torch.cuda.Stream()
    yield s
    torch.cuda.synchronize()


@pytest.mark.parametrize("mode,tol", [("fp64", 1e-13), ("fp32_mixed", 1e-6)])
@pytest.mark.parametrize("graph", [False, True])
def test_ensemble_matches_members(gpu_lib, stream, mode, tol, graph):
    dm = gpu_lib
    single = members(dm, mode)
    for m in single:
        for s in range(1, 4):
            m.moloch(s)
    ens_members = members(dm, mode, stream=stream.cuda_stream)
    ens = dm.Ensemble(ens_members)
    ens.run(3, graph=graph)
    for a, b in zip(ens_members, single):
        a.sync()
        for f in FIELDS:
            e = rel_l2(a.get(f), b.get(f))
            assert e <= tol, (f, e, a.jx, a.iy, a.kz)
    assert ens.kernel_count > 0
    # the members keep working as single handles after the ensemble run
    ens_members[0].moloch(4)
    single[0].moloch(4)
    assert rel_l2(ens_members[0].get("t"), single[0].get("t")) <= tol
    ens.close()
    for m in ens_members + single:
        m.close()


def test_ensemble_autotune(gpu_lib, stream):
    ms = members(gpu_lib, "fp32_mixed", stream=stream.cuda_stream)
    ens = gpu_lib.Ensemble(ms)
    choice = ens.autotune()
    assert choice[0] in (1, 2, 4, 8, 16, 32, 64) and choice[2] in (1, 2, 5, 10), choice
    ens.run(1)
    for m in ms:
        assert np.isfinite(m.get("t")).all()
    ens.close()
    for m in ms:
        m.close()


@pytest.mark.parametrize("tuning", [[32, 11], [32, 7], [32, 24, 5], [32, 24, 1, 8], [32, 536, 1]])
def test_ensemble_strip_shape_matches_members(gpu_lib, stream, tuning):
    """Ensemble with the warp-strip horizontal WAF, the k-marching,
    warp-strip or fused divergence/damping sound kernels, five fields per
    thread in the vertical WAF (third case), momentum strips of 8 rows
    (fourth) and the fused strips over two levels per warp (last) against
    the same members run alone with the tile kernel and the
    one-level-per-thread kernels.
    Different kernels contract different multiply-adds in the FP64 build,
    so the bound is 1e-12 rather than the 1e-13 of identical kernels."""
    ms = members(gpu_lib, "fp64", stream=stream.cuda_stream)
    solo = members(gpu_lib, "fp64", stream=stream.cuda_stream)
    e = gpu_lib.Ensemble(ms)
    e.set_tuning(tuning)
    e.run(2, graph=True)
    for m in solo:
        m.set_tuning([1, 0])
        m.run(2, graph=True)
    for m, s in zip(ms, solo):
        for n in ("u", "v", "w", "pai", "t", "qv"):
            assert rel_l2(m.get(n), s.get(n)) <= 1e-12, n
    e.close()
    for m in ms + solo:
        m.close()


# ---- persistent mode: one cooperative launch per ensemble step ------------
# FP32: default shapes; horizontal tiles of 2 levels with the fused
# divergence/damping and momentum strips and 2 vertical fields per thread;
# the k-marching divergence and damping.  FP64: default; k-marching
# divergence, damping and momentum with 8-level horizontal tiles.
PERSIST_CASES = [("fp32_mixed", [4, 0, 1]), ("fp32_mixed", [2, 24, 2]), ("fp32_mixed", [8, 3, 1]),
                 ("fp64", [4, 0, 1]), ("fp64", [8, 7, 1])]


@pytest.mark.parametrize("mode,tuning", PERSIST_CASES)
@pytest.mark.parametrize("graph", [False, True])
def test_persistent_matches_per_kernel(gpu_lib, stream, mode, tuning, graph):
    """The persistent kernel runs the per-kernel launches' bodies in the
    same order on the same tiles (column tiles 8 rows high, 8 strips per
    item), so the two modes agree bit for bit."""
    per_kernel = members(gpu_lib, mode, stream=stream.cuda_stream)
    pers = members(gpu_lib, mode, stream=stream.cuda_stream)
    e0 = gpu_lib.Ensemble(per_kernel)
    e0.set_tuning(tuning)
    e1 = gpu_lib.Ensemble(pers)
    e1.set_tuning(tuning)
    e1.set_persistent(True)
    assert e1.persistent and not e0.persistent
    e0.run(3, graph=graph)
    k0 = e1.kernel_count
    e1.run(3, graph=graph)
    e1.sync()
    assert e1.kernel_count - k0 == 3  # one launch per step
    for a, b in zip(pers, per_kernel):
        for f in FIELDS:
            x, y = a.get(f), b.get(f)
            assert np.array_equal(x, y), (f, float(np.max(np.abs(x - y))), a.jx, a.iy, a.kz)
    e0.close()
    e1.close()
    for m in per_kernel + pers:
        m.close()


def test_persistent_rejects_variants_it_does_not_carry(gpu_lib, stream):
    ms = members(gpu_lib, "fp32_mixed", stream=stream.cuda_stream)
    e = gpu_lib.Ensemble(ms)
    for tuning in ([32, 0, 1], [4, 4, 1], [4, 0, 5]):  # strips, k-marching momentum, 5 fields
        e.set_tuning(tuning)
        with pytest.raises(gpu_lib.MolochError):
            e.set_persistent(True)
        assert not e.persistent
    e.close()
    for m in ms:
        m.close()


def test_persistent_barrier_wait_runs_out(gpu_lib, stream):
    """Block 0 leaves at the fourth grid barrier without arriving: every
    other block's wait gives up after its limit (about 1 ms here), the step
    is abandoned and sync reports MOLOCH_ERR_TIMEOUT; launches made while
    the flag is set return at once.  With the hook off, steps run again."""
    ms = members(gpu_lib, "fp32_mixed", stream=stream.cuda_stream)
    e = gpu_lib.Ensemble(ms)
    e.set_persistent(True)
    e.set_wait_limit(cycles=2_000_000, skip_block=0, skip_barrier=3)
    e.run(2, graph=False)
    with pytest.raises(gpu_lib.MolochError) as err:
        e.sync()
    assert err.value.code == 6, err.value  # MOLOCH_ERR_TIMEOUT
    e.set_wait_limit()
    e.run(1, graph=False)
    e.sync()
    e.close()
    for m in ms:
        m.close()


def test_persistent_autotune_picks_a_mode(gpu_lib, stream):
    ms = members(gpu_lib, "fp32_mixed", stream=stream.cuda_stream)
    e = gpu_lib.Ensemble(ms)
    e.autotune()
    e.run(2, graph=True)
    e.sync()
    for m in ms:
        assert np.isfinite(m.get("t")).all()
    print("persistent" if e.persistent else "per kernel")
    e.close()
    for m in ms:
        m.close()


# ---- the staged column solve over all members' tiles ----------------------
SHAPES_TW = [(40, 33, 16, 3.0, 11), (24, 20, 12, 7.5, 12), (36, 29, 10, 0.5, 13), (64, 48, 61, 5.0, 14)]


def members_tw(dm, stream=None):
    out = []
    for jx, iy, kz, u0, seed in SHAPES_TW:
        m = dm.Moloch(jx, iy, kz, mode="fp32_mixed", stream=stream)
        m.setup_idealized(pert_amp=1.0, pert_levels=kz, seed=seed, u0=u0, v0=0.5 * u0,
                          hills=((300.0, jx / 2.0, iy / 2.0, 4.0),))
        out.append(m)
    return out


@pytest.mark.parametrize("graph", [False, True])
def test_ensemble_staged_column_matches_members(gpu_lib, stream, graph):
    """kb_sound_column_tw (tuning bit 32 in an ensemble: one persistent
    launch over the 32 x 12 column tiles of every member, each member's
    tensor maps read from device memory) against the members run alone
    with the single-domain two-word staged solve (bits 32 + 128): the same
    arithmetic, so the same bits.  Members of uneven jx, iy and kz (partial
    tiles, kz 10 to 61), four steps (every substep parity and the
    last-substep path)."""
    ms = members_tw(gpu_lib, stream=stream.cuda_stream)
    solo = members_tw(gpu_lib)
    e = gpu_lib.Ensemble(ms)
    e.set_tuning([16, 56, 1])
    e.run(4, graph=graph)
    e.sync()
    for m in solo:
        m.set_tuning([16, 56 | 128, 1])
        m.run(4, graph=graph)
        m.sync()
    same = True
    for m, s in zip(ms, solo):
        for f in FIELDS + ("s", "deltaw"):
            a, b = m.get(f), s.get(f)
            same = same and np.array_equal(a, b)
            assert rel_l2(a, b) <= 1e-6, (f, m.jx, m.iy, m.kz)
    print("batched staged column solve bit-identical to the members alone:", same)
    e.close()
    for m in ms + solo:
        m.close()


def test_ensemble_autotune_may_pick_staged_column(gpu_lib, stream):
    """The ensemble autotuner offers the batched staged column solve when
    every member has tensor maps, and the chosen tuning runs."""
    ms = members_tw(gpu_lib, stream=stream.cuda_stream)
    e = gpu_lib.Ensemble(ms)
    choice = e.autotune()
    print("ensemble autotune:", choice)
    e.run(2)
    e.sync()
    for m in ms:
        assert np.isfinite(m.get("t")).all()
    e.close()
    for m in ms:
        m.close()
