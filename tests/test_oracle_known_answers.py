"""Known-answer checks of the CPU oracle, written from the reference's
equations (the reference ships no tests or golden data)."""
import math

import numpy as np
import pytest


def test_constants(oracle_mod):
    L = oracle_mod.lib()
    import ctypes
    c = (ctypes.c_double * 11)()
    L.oracle_constants(c)
    rgas, rwat, cpd, cvd, rdrcv, cpovr, rovcp, ep1, ep2, eomeg2, degrad = list(c)
    # mod_constants.F90 comments: rgas 287.05661, rwat 461.52281, cpd 1004.69813, cvd 717.64152
    assert abs(rgas - 287.05661) < 1e-5
    assert abs(rwat - 461.52281) < 1e-5
    assert abs(cpd - 1004.69813) < 1e-5
    assert abs(cvd - 717.64152) < 1e-5
    assert rdrcv == rgas / cvd and cpovr == cpd / rgas and rovcp == rgas * (1.0 / cpd)
    assert abs(ep1 - 0.6077762876) < 1e-9 and abs(ep2 - 0.6219770795) < 1e-9
    assert eomeg2 == 2.0 * 7.2921159e-5


def test_gzita_and_zeta(oracle_mod):
    L = oracle_mod.lib()
    ztop, h = 36000.0, 12000.0
    assert L.oracle_gzita(0.0, ztop, 0.0) == 1.0
    assert abs(L.oracle_gzita(ztop, ztop, 0.0)) < 1e-15
    # zeta(zita=0) = 0 on flat ground and over a hill (mod_zita.F90:145-150)
    assert L.oracle_md_zeta(0.0, 0.0, ztop, h, 0.0) == 0.0
    assert abs(L.oracle_md_zeta(0.0, 500.0 * 9.80665, ztop, h, 0.0)) < 1e-9
    # zeta is the height above the orography: bzita(ztop) = ztop and
    # gzita(ztop) = 0, so zeta(ztop) = ztop - orog
    assert abs(L.oracle_md_zeta(ztop, 0.0, ztop, h, 0.0) - ztop) < 1e-7
    assert abs(L.oracle_md_zeta(ztop, 1000.0 * 9.80665, ztop, h, 0.0) - (ztop - 1000.0)) < 1e-7
    # fmz = 1 / (d zeta / d zita) > 0
    for z in np.linspace(0, ztop, 7):
        f = L.oracle_md_fmz(z, 0.0, ztop, h, 0.0)
        dz = 1e-3
        dzeta = (L.oracle_md_zeta(z + dz, 0.0, ztop, h, 0.0) - L.oracle_md_zeta(z - dz, 0.0, ztop, h, 0.0)) / (2 * dz)
        assert abs(f * dzeta - 1.0) < 1e-6


def test_pfesat(oracle_mod):
    L = oracle_mod.lib()
    # at 0 C both branches give their zeroth coefficient (mod_moloch.F90:128,140)
    assert L.oracle_pfesat(273.15, 1e5) == 0.611213476e+03
    assert abs(L.oracle_pfesat(273.15 - 1e-9, 1e5) - 0.611123516e+03) < 1e-3
    # clipped at 0.15 p
    assert L.oracle_pfesat(373.15, 1000.0) == 150.0
    # temperature clamped to [-75, 100] C
    assert L.oracle_pfesat(500.0, 1e9) == L.oracle_pfesat(373.15, 1e9)
    assert L.oracle_pfesat(100.0, 1e9) == L.oracle_pfesat(190.0, 1e9)
    es = L.oracle_pfesat(300.0, 1e5)
    assert L.oracle_pfwsat(300.0, 1e5) == 0.6219770795 * (es / (1e5 - es)) or \
        abs(L.oracle_pfwsat(300.0, 1e5) - 28.96454 ** -1 * 18.01528 * es / (1e5 - es)) < 1e-15


def test_superbee(oracle_mod):
    L = oracle_mod.lib()
    # superbee: 0 for r <= 0, 2r on [0, 1/2], 1 on [1/2, 1], r on [1, 2], 2 beyond
    for r, b in [(-3.0, 0.0), (0.0, 0.0), (0.25, 0.5), (0.5, 1.0), (0.75, 1.0), (1.0, 1.0),
                 (1.5, 1.5), (2.0, 2.0), (7.0, 2.0)]:
        assert L.oracle_superbee(r) == b


def test_xknu_profile(oracle_mod):
    o = oracle_mod.Oracle(oracle_mod.make_cfg(8, 8, 10))
    import ctypes
    x = (ctypes.c_double * 10)()
    o.L.oracle_xknu(o.h, x)
    x = list(x)
    assert x[0] == 1.0  # xdamp + (1 - xdamp) * sin(pi/2)
    assert abs(x[-1] - 0.0625) < 1e-15  # sin(0)
    assert all(a > b for a, b in zip(x, x[1:]))


def test_splitmix_uniform(oracle_mod):
    L = oracle_mod.lib()
    u = np.array([L.oracle_splitmix_u01(1234, i) for i in range(20000)])
    assert u.min() >= 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.01 and abs(u.std() - math.sqrt(1 / 12)) < 0.01


def test_initial_state_hydrostatic(oracle_mod):
    """fill_atmosphere: pai integrates the hydrostatic equation, so the
    discrete balance used by the implicit solver holds on the initial state:
    cpd * tv_avg * (pai(k-1) - pai(k)) = g * dzita / fmzf(k) to round-off."""
    o = oracle_mod.Oracle(oracle_mod.make_cfg(12, 10, 12, pert_amp=0.0))
    t, pai, qv, fmzf = o.get("t"), o.get("pai"), o.get("qv"), o.get("fmzf")
    tv = t * (1 + 0.6077762876 * qv)
    import ctypes
    s = (ctypes.c_double * 9)()
    o.L.oracle_scalars(o.h, s)
    dzita = s[2]
    cpd = 3.5 * (6.02214076e23 * 1.3806490e-23 / 28.96454 * 1000.0)
    # zb/zdelta quadratic in fill_atmosphere solves
    # (k = 1 is the top level) (tv1/pai(k) + tv2/pai(k+1)) * cpd*(pai(k+1)-pai(k))/2 = g*dzita/fmzf(k+1)
    for k in range(0, 11):
        lhs = 0.5 * cpd * (tv[k] / pai[k] + tv[k + 1] / pai[k + 1]) * (pai[k + 1] - pai[k])
        rhs = 9.80665 * dzita / fmzf[k + 1]
        assert np.max(np.abs(lhs - rhs) / rhs) < 1e-9


def test_constant_field_advection(oracle_mod):
    """wafone keeps a spatially constant tracer constant for any velocity:
    the zdv term cancels the flux divergence (mod_moloch.F90:1013,1124,1180)."""
    o = oracle_mod.Oracle(oracle_mod.make_cfg(14, 12, 10))
    o.set("qc", np.full((10, 12, 14), 1.0e-3))
    o.step(1)
    qc = o.get("qc")
    assert np.max(np.abs(qc - 1.0e-3)) < 1e-15


def test_oracle_bounds_checked_run(oracle_mod):
    """The bounds-checked oracle build runs a step with filters and both
    map-factor branches without touching memory outside the reference's
    declared bounds (it aborts on any out-of-bounds index)."""
    for rot in (True, False):
        o = oracle_mod.Oracle(oracle_mod.make_cfg(9, 7, 6, divfilter=True, filterpai=True,
                                                  filtertheta=True, rotllr=rot,
                                                  hills=((300.0, 4.0, 3.0, 2.0),)), checked=True)
        bad, _ = o.step(1, True)
        assert bad == 0
        assert np.isfinite(o.get("u")).all()
