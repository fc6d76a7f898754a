"""Parity of the CUDA step against the CPU oracle, through the C ABI.

Tolerances (floating point, FP64):
  * initial state and static terms: bit-identical (same host code path);
  * one phase / one step, FP64_EXACT build: relative L2 <= 1e-13 (only the
    transcendental calls pow/exp differ between CUDA and the host libm);
  * 100 steps at the reference defaults (100 x 100 x 30): relative L2 <= 1e-9
    per prognostic field, for the FP64 (contracting) and FP64_EXACT builds;
  * FP32 storage with FP64 solve: tests/test_gpu_mixed.py.
"""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

PROG = ("u", "v", "w", "pai", "t", "qv", "qc")
DIAG = ("ps", "p", "rho", "qsat", "tvirt", "tetav")


def pair(oracle_mod, dm, jx, iy, kz, mode="fp64_exact", hills=(), pert_amp=0.5, pert_levels=10,
         seed=1234, u0=1.0, v0=1.0, **opts):
    cfg_opts = {}
    prm = {}
    for k, v in opts.items():
        if k == "divfilter":
            cfg_opts["divfilter"] = v; prm["mo_divfilter"] = int(v)
        elif k == "filterpai":
            cfg_opts["filterpai"] = v; prm["do_filterpai"] = int(v)
        elif k == "filtertheta":
            cfg_opts["filtertheta"] = v; prm["do_filtertheta"] = int(v)
        elif k == "rotllr":
            cfg_opts["rotllr"] = v; prm["rotllr"] = int(v)
        else:
            raise TypeError(k)
    o = oracle_mod.Oracle(oracle_mod.make_cfg(jx, iy, kz, hills=hills, pert_amp=pert_amp,
                                              pert_levels=pert_levels, seed=seed, u0=u0, v0=v0, **cfg_opts))
    g = dm.Moloch(jx, iy, kz, mode=mode, **prm)
    g.setup_idealized(hills=hills, pert_amp=pert_amp, pert_levels=pert_levels, seed=seed, u0=u0, v0=v0)
    return o, g


def compare(o, g, names, tol):
    worst = {}
    for n in names:
        e = rel_l2(g.get(n), o.get(n))
        worst[n] = e
    bad = {n: e for n, e in worst.items() if not e <= tol}
    assert not bad, f"relative L2 above {tol}: {bad}"
    return worst


def test_initial_state_bit_identical(oracle_mod, gpu_lib):
    o, g = pair(oracle_mod, gpu_lib, 17, 13, 9, hills=((400.0, 8.0, 6.0, 3.0),))
    for n in ("u", "v", "w", "pai", "t", "qv", "fmz", "fmzf", "zeta", "hx", "hy"):
        a, b = g.get(n), o.get(n)
        assert np.array_equal(a, b), n


@pytest.mark.parametrize("jx,iy,kz", [(13, 11, 7), (40, 33, 16)])
def test_phases_exact(oracle_mod, gpu_lib, jx, iy, kz):
    """Each phase of one step separately (odd sizes exercise the edge paths)."""
    o, g = pair(oracle_mod, gpu_lib, jx, iy, kz)
    o.phase(0); g.phase(0)
    compare(o, g, ("tetav", "tvirt"), 0.0)
    compare(o, g, ("p", "qsat"), 1e-15)
    o.phase(1); g.phase(1)
    compare(o, g, ("u", "v", "w", "pai", "tetav", "s", "deltaw"), 1e-13)
    o.phase(2); g.phase(2)
    compare(o, g, ("u", "v", "w", "pai", "tetav", "qv", "qc"), 1e-13)
    for _ in range(2):
        o.phase(1); g.phase(1)
        o.phase(2); g.phase(2)
    o.phase(3); g.phase(3)
    compare(o, g, PROG + DIAG, 1e-13)


@pytest.mark.parametrize("mode", ["fp64_exact", "fp64"])
def test_steps_small(oracle_mod, gpu_lib, mode):
    o, g = pair(oracle_mod, gpu_lib, 24, 20, 12)
    for s in range(1, 6):
        o.step(s)
        g.moloch(s)
    compare(o, g, PROG + DIAG, 1e-12)


@pytest.mark.parametrize("opts", [
    dict(divfilter=True),
    dict(filterpai=True, filtertheta=True),
    dict(rotllr=False),
    dict(divfilter=True, filterpai=True, filtertheta=True, rotllr=False),
])
def test_options(oracle_mod, gpu_lib, opts):
    o, g = pair(oracle_mod, gpu_lib, 19, 16, 10, hills=((300.0, 9.0, 8.0, 3.0),), **opts)
    for s in range(1, 4):
        o.step(s)
        g.moloch(s)
    compare(o, g, PROG + DIAG, 1e-12)


@pytest.mark.parametrize("opts", [dict(divfilter=True), dict(rotllr=False),
                                  dict(divfilter=True, filterpai=True, filtertheta=True, rotllr=False)])
@pytest.mark.parametrize("variant", [7, 11, 24])
def test_options_with_sound_variants(oracle_mod, gpu_lib, variant, opts):
    """The divergence filter path (the column kernel leaves zdiv2b and pai to
    the filter kernels) and the non-rotated map factors with the k-marching,
    warp-strip and fused divergence/damping sound kernels, against the
    oracle."""
    o, g = pair(oracle_mod, gpu_lib, 19, 16, 10, hills=((300.0, 9.0, 8.0, 3.0),), **opts)
    g.set_tuning([1, variant])
    for s in range(1, 4):
        o.step(s)
        g.moloch(s)
    compare(o, g, PROG + DIAG, 1e-12)


def test_hill_and_wind(oracle_mod, gpu_lib):
    """Gaussian hill (500 m, radius 20 gp as in the 512 x 512 x 60 workload,
    scaled to the grid) and a 7 m/s background wind."""
    o, g = pair(oracle_mod, gpu_lib, 48, 40, 20, hills=((500.0, 24.5, 20.5, 6.0),), u0=7.0, v0=-2.0)
    for s in range(1, 4):
        o.step(s)
        g.moloch(s)
    compare(o, g, PROG + DIAG, 1e-12)


@pytest.mark.parametrize("mode", ["fp64", "fp64_exact"])
def test_reference_defaults_100_steps(oracle_mod, gpu_lib, mode):
    """The reference's own defaults (namelist.in: 100 x 100 x 30) with the
    seeded +-0.5 K theta noise on the lowest 10 levels: 100 steps."""
    o, g = pair(oracle_mod, gpu_lib, 100, 100, 30, mode=mode)
    diag_o = diag_g = None
    for s in range(1, 101):
        lp = s % 20 == 0
        bad, diag_o = o.step(s, lp)
        d = g.moloch(s, lp)
        if lp:
            diag_g = d
            assert bad == 0 and d.status == 0
    worst = compare(o, g, PROG + DIAG, 1e-9)
    print(mode, {k: f"{v:.2e}" for k, v in worst.items()})
    # lprint max/min printout (mod_moloch.F90:396-401)
    gd = [diag_g.maxps, diag_g.minps, diag_g.maxu, diag_g.minu, diag_g.maxv, diag_g.minv]
    assert np.allclose(gd, diag_o, rtol=1e-9, atol=0)


def test_graph_replay_matches_stepwise(gpu_lib):
    a = gpu_lib.Moloch(32, 24, 12)
    b = gpu_lib.Moloch(32, 24, 12)
    a.setup_idealized()
    b.setup_idealized()
    for s in range(4):
        a.moloch(s + 1)
    b.run(4, graph=True)
    b.sync()
    for n in PROG + DIAG:
        assert np.array_equal(a.get(n), b.get(n)), n
    assert b.kernel_count > 0


def test_cfl_violation_is_reported(gpu_lib):
    """A non-finite state is reported like the reference's fatal('CFL VIOLATION')."""
    g = gpu_lib.Moloch(16, 12, 8)
    g.setup_idealized()
    t = g.download("t")
    t[5, 5, 3] = np.nan
    g.upload("t", t)
    g.moloch(1)
    with pytest.raises(gpu_lib.MolochError) as ei:
        g.moloch(2, lprint=True)
    assert ei.value.code == 4


@pytest.mark.parametrize("direct", [True, False])
def test_upload_download_roundtrip_and_bounds(gpu_lib, direct):
    """Host arrays with halo rings through upload and download, with direct
    (a kernel reading the host arrays) and staged uploads."""
    g = gpu_lib.Moloch(12, 10, 6)
    g.setup_idealized()
    g.host_direct = direct
    assert g.host_direct == direct or not direct
    rng = np.random.default_rng(0)
    for name in ("u", "v", "w", "pai", "t", "qv", "qc", "qi", "qr", "qs"):
        a = g.download(name)
        interior = rng.standard_normal(g.get(name).shape)
        b = a.copy()
        (l1, _), (l2, _) = gpu_lib.field_bounds(name, 12, 10, 6)[:2]
        b[1 - l1:1 - l1 + 12, 1 - l2:1 - l2 + 10, :] = interior.transpose(2, 1, 0)
        g.upload(name, b)
        assert np.array_equal(g.get(name), interior)
        full = g.download(name)
        # halo positions hold periodic images of the interior
        assert np.array_equal(full[0 - l1], full[12 - l1]) if l1 <= 0 else True
    import ctypes
    L = gpu_lib.lib()
    lb = (ctypes.c_int * 3)(0, 0, 1)
    ub = (ctypes.c_int * 3)(13, 11, 6)
    buf = np.zeros(14 * 12 * 6)
    rc = L.moloch_gpu_upload(g.h, gpu_lib.FIELD["u"], buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), lb, ub)
    assert rc == 2  # u has bounds (-1:nj+2, 0:ni+1, 1:kz)


@pytest.mark.parametrize("mode", ["fp64", "fp32_mixed"])
@pytest.mark.parametrize("registered", [False, True])
def test_output_path_overlaps_steps(gpu_lib, mode, registered):
    """output_start after step 2, two more steps, output_finish: the arrays
    hold t and ps of step 2 (with periodic halos), and the run itself is
    not disturbed; into new arrays (host threads) or into registered ones
    (kernels writing them from the device snapshot)."""
    a = gpu_lib.Moloch(40, 28, 12, mode=mode)
    b = gpu_lib.Moloch(40, 28, 12, mode=mode)
    for g in (a, b):
        g.setup_idealized(hills=((300.0, 20.0, 14.0, 4.0),), u0=3.0)
    a.run(2, graph=True)
    b.run(2, graph=True)
    a.output_start()
    a.run(2, graph=True)
    if registered:
        t_out, ps_out = np.full_like(a.download("t"), np.nan), np.full_like(a.download("ps"), np.nan)
        a.host_register(t_out)
        a.host_register(ps_out)
        t2, ps2 = a.output_finish(t_out, ps_out)
        assert t2 is t_out and ps2 is ps_out
    else:
        t2, ps2 = a.output_finish()
    assert np.array_equal(t2, b.download("t"))
    assert np.array_equal(ps2, b.download("ps"))
    b.run(2, graph=True)
    for n in ("t", "ps", "u", "pai"):
        assert np.array_equal(a.get(n), b.get(n)), n
    with pytest.raises(gpu_lib.MolochError):
        a.output_finish()


@pytest.mark.parametrize("mode", ["fp64", "fp32_mixed"])
def test_direct_and_staged_transfers_agree(gpu_lib, mode):
    """Uploads through the direct path (a kernel reading the host arrays),
    the staged path and DMA from registered (pinned) arrays give identical
    device states: identical downloads (halo rings included) and identical
    steps afterwards."""
    if not gpu_lib.Moloch(8, 8, 4).host_direct:
        pytest.skip("device without pageable host memory access")
    a = gpu_lib.Moloch(37, 29, 9, mode=mode)
    b = gpu_lib.Moloch(37, 29, 9, mode=mode)
    for g in (a, b):
        g.setup_idealized(hills=((300.0, 18.0, 14.0, 4.0),), u0=3.0)
        g.run(2, graph=True)
    a.host_direct = True
    b.host_direct = False
    names = ("u", "v", "w", "pai", "t", "qx", "ps", "tetav", "p", "rho", "qsat")
    for n in names:
        da, db = a.download(n), b.download(n)
        assert np.array_equal(da, db), n
    c = gpu_lib.Moloch(37, 29, 9, mode=mode)  # uploads from registered (pinned) arrays: DMA
    c.setup_idealized(hills=((300.0, 18.0, 14.0, 4.0),), u0=3.0)
    c.run(2, graph=True)
    for n in ("u", "v", "w", "pai", "t", "qx"):
        host = a.download(n) * (1.0 + 1e-3)  # a state the device does not hold yet
        a.upload(n, host)
        b.upload(n, host)
        pinned = np.asfortranarray(host.copy())
        c.host_register(pinned)
        c.upload(n, pinned)
        pinned[...] = np.nan  # the upload has read the array when it returns
        c.host_unregister(pinned)
    for g in (a, b, c):
        g.run(1, graph=True)
    for n in names:
        assert np.array_equal(a.download(n), b.download(n)), n
        assert np.array_equal(a.download(n), c.download(n)), n


@pytest.mark.parametrize("mode", ["fp64", "fp32_mixed"])
def test_setup_on_device_matches_host(gpu_lib, mode):
    """The idealized state computed on the device against the host
    restatement: static and prognostic fields to 1e-13 relative (FP64; only
    exp/pow/sqrt roundings differ) or to the FP32 rounding, and 5 steps from
    each to 1e-11 / 1e-5."""
    kw = dict(hills=((500.0, 30.5, 20.5, 6.0), (300.0, 10.0, 33.0, 3.0)), u0=4.0, v0=-1.5, pert_amp=0.5,
              pert_levels=7, seed=99)
    a = gpu_lib.Moloch(61, 41, 17, mode=mode)
    b = gpu_lib.Moloch(61, 41, 17, mode=mode)
    a.setup_idealized(**kw)
    b.setup_idealized(device=True, **kw)
    tol0 = 1e-13 if mode == "fp64" else 1e-7
    for n in ("zeta", "fmz", "fmzf", "hx", "hy", "u", "v", "w", "t", "pai", "qv", "qc"):
        e = rel_l2(b.get(n), a.get(n))
        assert e <= tol0, (n, e)
    for s in range(1, 6):
        a.moloch(s)
        b.moloch(s)
    tol = 1e-11 if mode == "fp64" else 1e-5
    for n in PROG + DIAG:
        e = rel_l2(b.get(n), a.get(n))
        assert e <= tol, (n, e)


@pytest.mark.parametrize("mode,tol", [("fp64_exact", 0.0), ("fp64", 1e-11), ("fp32_mixed", 1e-3)])
@pytest.mark.parametrize("shape", [16, 32, 64])
def test_horizontal_waf_strips_match_tiles(gpu_lib, mode, tol, shape):
    """The warp-strip horizontal WAF kernel (launch shape >= 16 rows per
    strip) against the tile kernel (shape 1): the same arithmetic, so the
    exact build agrees bit for bit.  The contracting builds fuse
    multiply-adds differently in the two kernels, and in FP32 the limiter
    turns last-bit differences into differences of the size of the FP32
    error itself (w: 8e-5 relative after 3 steps), hence 1e-3 there; odd
    sizes exercise partial strips."""
    a = gpu_lib.Moloch(61, 45, 9, mode=mode)
    b = gpu_lib.Moloch(61, 45, 9, mode=mode)
    for g in (a, b):
        g.setup_idealized(hills=((400.0, 30.0, 22.0, 4.0),), u0=6.0, v0=-4.0)
    a.set_tuning([1])
    b.set_tuning([shape])
    for s in range(1, 4):
        a.moloch(s)
        b.moloch(s)
    for n in PROG:
        e = rel_l2(b.get(n), a.get(n))
        assert e <= tol, (n, e)


@pytest.mark.parametrize("mode,tol", [("fp64_exact", 0.0), ("fp64", 1e-11), ("fp32_mixed", 1e-3)])
@pytest.mark.parametrize("fields", [2, 5, 10])
def test_vertical_waf_fields_per_thread_match(gpu_lib, mode, tol, fields):
    """The vertical WAF kernel with 2, 5 or 10 advected fields per thread
    (shared velocity loads and terms) against one field per thread: the
    same arithmetic per field, bit for bit in the exact build."""
    a = gpu_lib.Moloch(45, 37, 11, mode=mode)
    b = gpu_lib.Moloch(45, 37, 11, mode=mode)
    for g in (a, b):
        g.setup_idealized(hills=((400.0, 22.0, 18.0, 4.0),), u0=6.0, v0=-4.0)
    a.set_tuning([1, 0, 1])
    b.set_tuning([1, 0, fields])
    for s in range(1, 4):
        a.moloch(s)
        b.moloch(s)
    for n in PROG:
        e = rel_l2(b.get(n), a.get(n))
        assert e <= tol, (n, e)


@pytest.mark.parametrize("mode", ["fp64_exact", "fp32_mixed"])
@pytest.mark.parametrize("variant", [24, 536, 88])
@pytest.mark.parametrize("rows", [4, 8, 24])
def test_sound_strip_rows_match(gpu_lib, mode, variant, rows):
    """The momentum strips with 4, 8 or 24 rows per warp (tuning slot 3)
    against 32: the same arithmetic at every point, only the partition into
    strips differs, so the same bits; iy not a multiple of the rows, jx
    even (the two-column strips of variant 88)."""
    a = gpu_lib.Moloch(46, 37, 11, mode=mode)
    b = gpu_lib.Moloch(46, 37, 11, mode=mode)
    for g in (a, b):
        g.setup_idealized(hills=((400.0, 22.0, 18.0, 4.0),), u0=6.0, v0=-4.0)
    a.set_tuning([16, variant, 1, 32])
    b.set_tuning([16, variant, 1, rows])
    for s in range(1, 4):
        a.moloch(s)
        b.moloch(s)
    for n in PROG + ("s", "deltaw"):
        assert np.array_equal(b.get(n), a.get(n)), n


@pytest.mark.parametrize("mode,tol", [("fp64_exact", 0.0), ("fp64", 1e-11), ("fp32_mixed", 1e-3)])
@pytest.mark.parametrize("kz,variant", [(9, 7), (13, 7), (9, 11), (13, 8), (9, 16), (13, 24), (10, 20),
                                          (9, 528), (10, 536), (13, 536)])
def test_kmarching_sound_kernels_match(gpu_lib, mode, tol, kz, variant):
    """The k-marching divergence/damping/momentum kernels (chunks of 4
    levels, the next level prefetched), the warp-strip momentum kernel
    (30 columns x 32 rows, neighbours by shuffles, stale-halo edge buffers
    on the boundary lanes and rows) and the fused divergence/damping strips
    (variant bit 16: 29 columns x 32 rows, damped u, v to the other buffer;
    with bit 512 over two levels per warp) against the one-level-per-thread
    kernels: bit for bit in the exact build; kz not a multiple of the
    chunk (nor of the two levels), jx and iy not multiples of the strips."""
    a = gpu_lib.Moloch(45, 37, kz, mode=mode)
    b = gpu_lib.Moloch(45, 37, kz, mode=mode)
    for g in (a, b):
        g.setup_idealized(hills=((400.0, 22.0, 18.0, 4.0),), u0=6.0, v0=-4.0)
    a.set_tuning([1, 0])
    b.set_tuning([1, variant])
    for s in range(1, 4):
        a.moloch(s)
        b.moloch(s)
    for n in PROG + ("s", "deltaw"):
        e = rel_l2(b.get(n), a.get(n))
        assert e <= tol, (n, e)


def test_tuning_arguments_are_checked(gpu_lib):
    """set_tuning refuses what no kernel runs, with MOLOCH_ERR_ARG (1) and
    the handle's tuning unchanged (every slot is checked before any is
    applied): both two-word staged variants at once, rows per momentum
    strip outside 4..64, fields per thread other than 1, 2, 5, 10, bits
    beyond the variants, a staggering variant other than 0 and 1; the
    tuning count has five slots; a valid tuning runs."""
    g = gpu_lib.Moloch(32, 24, 10, mode="fp32_mixed")
    g.setup_idealized(device=True)
    assert g.L.moloch_gpu_tuning_count() == 5
    g.set_tuning([16, 24, 1, 32])
    a = g.get("t")
    for bad in ([32, 32 | 128 | 256], [32, 56, 1, 3], [32, 56, 1, 65], [32, 56, 3], [32, 1024], [0],
                [32, 56, 1, 8, 2]):
        with pytest.raises(gpu_lib.MolochError) as ei:
            g.set_tuning(bad)
        assert ei.value.code == 1, bad
    # the refused calls left [16, 24, 1, 32]: a step matches a second
    # handle set to it
    h = gpu_lib.Moloch(32, 24, 10, mode="fp32_mixed")
    h.setup_idealized(device=True)
    h.set_tuning([16, 24, 1, 32])
    g.moloch(1)
    h.moloch(1)
    for n in ("u", "v", "w", "t"):
        assert np.array_equal(g.get(n), h.get(n)), n
    h.close()
    assert np.isfinite(a).all()
    g.set_tuning([16, 760, 1, 8])
    g.moloch(1)
    g.sync()
    assert np.isfinite(g.get("t")).all()
    g.close()


@pytest.mark.parametrize("jx", [48, 46])
def test_staggering_four_columns_per_thread_matches(gpu_lib, jx):
    """The staggering back from the cross points with four columns per
    thread (tuning slot 4, FP32, jx a multiple of 4; 16-byte loads and
    stores, the neighbouring quads wrapped whole at the periodic edges)
    against one column per thread: the same expression per column, so the
    same bits; jx = 46 falls back to the one-column kernel."""
    a = gpu_lib.Moloch(jx, 37, 11, mode="fp32_mixed")
    b = gpu_lib.Moloch(jx, 37, 11, mode="fp32_mixed")
    for g in (a, b):
        g.setup_idealized(hills=((400.0, jx / 2.0, 18.0, 4.0),), u0=6.0, v0=-4.0)
    a.set_tuning([16, 24, 1, 32, 0])
    b.set_tuning([16, 24, 1, 32, 1])
    for s in range(1, 4):
        a.moloch(s)
        b.moloch(s)
    for n in PROG:
        assert np.array_equal(b.get(n), a.get(n)), n
