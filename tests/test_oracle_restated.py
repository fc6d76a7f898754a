"""A second restatement of parts of the step, in NumPy and written from the
reference's source alone, against the C oracle: the pointwise diagnostics
of moloch() (the oracle's phases 0, reset + pre-diagnostics, and 3,
post-diagnostics), sound() (phase 1), the staggering of advection(),
wafone, divdamp and the 3-D filters (the oracle's stagger, wafone, divdamp
and filter hooks), the lprint printout, one whole step composed from those
pieces, and the initial state of param() and fill_atmosphere.  Together they cover the routines of the step; wafone and
sound() in both map-factor branches, the
non-ROTLLR one with map factors other than 1 (oracle_set_map_factors).

Reference: nompi/mod_moloch.F90:289-323 (p, qsat, tvirt, qwltot, qwitot,
tetav before the advection loop), :355-391 (tvirt, t, p, rho, the
hypsometric ps and qsat after it), :119-181 (pfesat / pfwsat, the Flatau
polynomials); constants of nompi/mod_constants.F90 (p00 :225, lrate :231,
tzero :193, egrav :81).  Tolerance: relative 1e-13 (both evaluate the same
FP64 expressions; NumPy's vectorised exp/pow may differ from libm in the
last bit)."""
import ctypes

import numpy as np
import pytest

P00 = 1.0e5
LRATE = 0.00649
TZERO = 273.15
EGRAV = 9.80665

# Flatau et al. (1992) polynomial coefficients as the reference lists them
# (pfesat, nompi/mod_moloch.F90:128-147): water 0..100 C, ice -75..0 C
A_W = (0.611213476e+03, 0.444007856e+02, 0.143064234e+01, 0.264461437e-01, 0.305903558e-03,
       0.196237241e-05, 0.892344772e-08, -0.373208410e-10, 0.209339997e-13)
C_I = (0.611123516e+03, 0.503109514e+02, 0.188369801e+01, 0.420547422e-01, 0.614396778e-03,
       0.602780717e-05, 0.387940929e-07, 0.149436277e-09, 0.262655803e-12)


def constants(oracle_mod):
    c = (ctypes.c_double * 11)()
    oracle_mod.lib().oracle_constants(c)
    rgas, rwat, cpd, cvd, rdrcv, cpovr, rovcp, ep1, ep2, eomeg2, degrad = list(c)
    return {"rgas": rgas, "cpovr": cpovr, "ep1": ep1, "ep2": ep2}


def horner(coef, td):
    # a0 + td*(a1 + td*(a2 + ... + td*a8)), innermost first
    acc = np.full_like(td, coef[8])
    for a in coef[7::-1]:
        acc = a + td * acc
    return acc


def pfwsat(t, p, ep2):
    td = np.clip(t - TZERO, -75.0, 100.0)
    esat = np.where(td >= 0.0, horner(A_W, td), horner(C_I, td))
    es = np.minimum(esat, 0.15 * p)
    return ep2 * (es / (p - es))


def rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def make(oracle_mod, names, rotllr=True):
    """A developed state (one step: moisture, winds and theta no longer the
    initial profiles), then the inputs of the phase under test perturbed by
    a seeded relative 1e-3, so that the phase's outputs cannot be left over
    from the step's own diagnostics."""
    cfg = oracle_mod.make_cfg(13, 11, 9, hills=((300.0, 6.5, 5.5, 3.0),), pert_amp=0.5, pert_levels=9,
                              seed=42, u0=3.0, v0=-2.0, rotllr=rotllr)
    o = oracle_mod.Oracle(cfg)
    o.step(1)
    rng = np.random.default_rng(5)
    for n in names:
        a = o.get(n)
        o.set(n, a * (1.0 + 1e-3 * rng.uniform(-1.0, 1.0, a.shape)))
    return o


def test_prediagnostics_restated(oracle_mod):
    c = constants(oracle_mod)
    o = make(oracle_mod, ("pai", "t", "qv", "qc"))
    pai, t = o.get("pai"), o.get("t")
    qv, qc, qi, qr, qs = (o.get(n) for n in ("qv", "qc", "qi", "qr", "qs"))
    o.phase(0)
    p = (pai ** c["cpovr"]) * P00
    qsat = pfwsat(t, p, c["ep2"])
    tvirt = t * (1.0 + c["ep1"] * qv - qc - qi - qr - qs)
    expect = {"p": p, "qsat": qsat, "tvirt": tvirt, "tetav": tvirt / pai,
              "qwltot": qc + qr, "qwitot": qi + qs}
    for n, v in expect.items():
        assert rel(o.get(n), v) <= 1e-13, (n, rel(o.get(n), v))
    o.close()


def test_postdiagnostics_restated(oracle_mod):
    c = constants(oracle_mod)
    o = make(oracle_mod, ("tetav", "pai", "qv"))
    tetav, pai, zeta = o.get("tetav"), o.get("pai"), o.get("zeta")
    qv, qc, qi, qr, qs = (o.get(n) for n in ("qv", "qc", "qi", "qr", "qs"))
    o.phase(3)
    tvirt = tetav * pai
    t = tvirt / (1.0 + c["ep1"] * qv - qc - qi - qr - qs)
    p = (pai ** c["cpovr"]) * P00
    rho = p / (c["rgas"] * t)
    # hypsometric surface pressure from the lowest level (k = kz, the last
    # index here): lapse rate from the two lowest levels blended with lrate
    zdgz = zeta[-1] * EGRAV
    lrt = (tvirt[-2] - tvirt[-1]) / (zeta[-2] - zeta[-1])
    lrt = 0.65 * lrt - 0.35 * LRATE
    tv = tvirt[-1] - 0.5 * zeta[-1] * lrt
    ps = p[-1] * np.exp(zdgz / (c["rgas"] * tv))
    expect = {"tvirt": tvirt, "t": t, "p": p, "rho": rho, "ps": ps, "qsat": pfwsat(t, p, c["ep2"])}
    for n, v in expect.items():
        assert rel(o.get(n), v) <= 1e-13, (n, rel(o.get(n), v))
    o.close()


# ---- staggering (nompi/mod_moloch.F90:1327-1417) ---------------------------
# Arrays are (levels, i, j): the last axis is j.  The domain is periodic, so
# the reference's width-2 halo copies before each stencil are index wraps.
def uv_to_x(u, v):
    ux = 0.5625 * (np.roll(u, -1, 2) + u) - 0.0625 * (np.roll(u, -2, 2) + np.roll(u, 1, 2))
    vx = 0.5625 * (np.roll(v, -1, 1) + v) - 0.0625 * (np.roll(v, -2, 1) + np.roll(v, 1, 1))
    return ux, vx


def w_to_x(w):
    """w has kz+1 levels (Fortran 1..kz+1), wx kz; index = Fortran level - 1."""
    kz = w.shape[0] - 1
    wx = np.empty((kz,) + w.shape[1:])
    k = np.arange(1, kz - 1)
    wx[k] = 0.5625 * (w[k + 1] + w[k]) - 0.0625 * (w[k + 2] + w[k - 1])
    wx[0] = 0.5 * (w[1] + w[0])
    wx[kz - 1] = 0.5 * (w[kz] + w[kz - 1])
    return wx


def x_to_uv(ux, vx):
    u = 0.5625 * (ux + np.roll(ux, 1, 2)) - 0.0625 * (np.roll(ux, -1, 2) + np.roll(ux, 2, 2))
    v = 0.5625 * (vx + np.roll(vx, 1, 1)) - 0.0625 * (np.roll(vx, -1, 1) + np.roll(vx, 2, 1))
    return u, v


def x_to_w(wx, w_old):
    """Fortran levels 3..kz-1 fourth order, 2 and kz two-point; levels 1 and
    kz+1 keep their values."""
    kz = wx.shape[0]
    w = w_old.copy()
    k = np.arange(2, kz - 1)  # Fortran 3 .. kz-1
    w[k] = 0.5625 * (wx[k] + wx[k - 1]) - 0.0625 * (wx[k + 1] + wx[k - 2])
    w[1] = 0.5 * (wx[1] + wx[0])
    w[kz - 1] = 0.5 * (wx[kz - 1] + wx[kz - 2])
    return w


def test_staggering_restated(oracle_mod):
    o = make(oracle_mod, ("u", "v", "w"))
    u, v, w = o.get("u"), o.get("v"), o.get("w")
    o.stagger(True)
    ux, vx = uv_to_x(u, v)
    for n, want in (("ux", ux), ("vx", vx), ("wx", w_to_x(w))):
        got = o.get(n)
        assert np.max(np.abs(got - want)) <= 1e-15 * np.max(np.abs(want)), n
    # back, from perturbed cross-point values (not a round trip of the above)
    rng = np.random.default_rng(9)
    for n in ("ux", "vx", "wx"):
        a = o.get(n)
        o.set(n, a + 0.1 * rng.standard_normal(a.shape))
    ux, vx, wx = o.get("ux"), o.get("vx"), o.get("wx")
    w_before = o.get("w")
    o.stagger(False)
    u2, v2 = x_to_uv(ux, vx)
    for n, want in (("u", u2), ("v", v2), ("w", x_to_w(wx, w_before))):
        got = o.get(n)
        assert np.max(np.abs(got - want)) <= 1e-15 * np.max(np.abs(want)), n
    o.close()


# ---- wafone, ROTLLR branch (nompi/mod_moloch.F90:929-1187) -----------------
MINDEN = 1.0e-30  # :95


def superbee(r):
    # b = max(wlow, min(whigh, max(r, min(2 r, 1)))), wlow = 0, whigh = 2
    return np.maximum(0.0, np.minimum(2.0, np.maximum(r, np.minimum(2.0 * r, 1.0))))


def safe_den(z):
    # sign(max(abs(z), minden), z)
    return np.copysign(np.maximum(np.abs(z), MINDEN), z)


class Bounded:
    """A reference array with its Fortran bounds: a[j, i, k] -> data[k-lk, i-li, j-lj]."""

    def __init__(self, o, name):
        self.data, self.lb, _ = o.get_bounded(name)

    def ji(self, j0, j1, i0, i1, k=None):
        """Fortran ranges j0..j1, i0..i1 (inclusive) of level k (or a 2-D field)."""
        d = self.data[0] if k is None else self.data[k - self.lb[2]]  # a 2-D field has one level
        return d[..., i0 - self.lb[1]:i1 - self.lb[1] + 1, j0 - self.lb[0]:j1 - self.lb[0] + 1]


def wafone_np(pp, s, fmz, fmzf, u, v, msfu, msfv, msfx, dta, dx, dzita, rotllr=True):
    """pp: interior (kz, ni, nj) of the advected field; s, fmzf: interior
    (kz+1, ni, nj); fmz, u, v, msfu, msfv, msfx: Bounded.  Returns the new
    interior of pp.  rotllr False: the map-factor branch (:1189-1298)."""
    kz, ni, nj = pp.shape
    dtrdx = dta / dx
    dtrdy = dta / dx
    dtrdz = 0.5 * (dta / dzita)  # do_vadvtwice
    P = {k: pp[k - 1] for k in range(1, kz + 1)}  # Fortran level -> (ni, nj)
    S = {k: s[k - 1] for k in range(1, kz + 2)}
    FZ = {k: fmz.ji(1, nj, 1, ni, k) for k in range(1, kz + 1)}
    FF = {k: fmzf[k - 1] for k in range(1, kz + 2)}

    def vertical(src):
        wfw = {1: np.zeros((ni, nj)), kz + 1: np.zeros((ni, nj))}
        for k in range(1, kz):
            zamu = S[k + 1] * dtrdz
            pos = zamu >= 0.0
            is_ = np.where(pos, 1.0, -1.0)
            num = np.where(pos, src[k + 1] - src[min(k + 2, kz)], src[max(k - 1, 1)] - src[k])
            r = num / safe_den(src[k] - src[k + 1])
            b = superbee(r)
            zphi = (is_ + zamu * b) - is_ * b
            wfw[k + 1] = (0.5 * S[k + 1]) * ((1.0 + zphi) * src[k + 1] + (1.0 - zphi) * src[k])
        out = {}
        for k in range(1, kz + 1):
            zrfmu = (dtrdz * FZ[k]) / FF[k]
            zrfmd = (dtrdz * FZ[k]) / FF[k + 1]
            zdv = (S[k] * zrfmu - S[k + 1] * zrfmd) * src[k]
            out[k] = ((src[k] - wfw[k] * zrfmu) + wfw[k + 1] * zrfmd) + zdv
        return out

    wz = vertical(vertical(P))  # two passes at dt/2 (do_vadvtwice, :1022-1073)
    new = np.empty_like(pp)
    for k in range(1, kz + 1):
        # meridional: wz with its periodic ring of two rows, Fortran i = -1 .. ni+2
        w2 = wz[k]
        ext = np.concatenate([w2[ni - 2:ni], w2, w2[0:2]], axis=0)  # row q <-> i = q - 1

        def WZ(i):
            return ext[i + 1]

        imin, imax = -1, ni + 2
        vk = v.ji(1, nj, 0, ni + 2, k)  # rows i = 0 .. ni+2

        def V(i):
            return vk[i]

        rmv = 1.0 / msfv.ji(1, nj, 0, ni + 1)   # rows i = 0 .. ni+1
        mx = msfx.ji(1, nj, 1, ni)
        mx2 = mx * mx
        zpby = {}
        for i in range(1, ni + 2):
            zamu = V(i) * dtrdy if rotllr else (V(i) * rmv[i]) * dtrdy
            pos = zamu > 0.0
            is_ = np.where(pos, 1.0, -1.0)
            ihp = min(i + 1, imax)
            num = np.where(pos, WZ(i - 1) - WZ(max(i - 2, imin)), WZ(ihp) - WZ(max(ihp - 1, imin)))
            r = num / safe_den(WZ(i) - WZ(i - 1))
            b = superbee(r)
            zphi = (is_ + zamu * b) - is_ * b
            vh = 0.5 * V(i) if rotllr else (0.5 * V(i)) * rmv[i]
            zpby[i] = vh * ((1.0 + zphi) * WZ(i - 1) + (1.0 - zphi) * WZ(i))
        fzk = fmz.ji(0, nj + 1, 0, ni + 1, k)  # rows i = 0 .. ni+1, columns j = 0 .. nj+1
        p0 = np.empty((ni, nj))
        for i in range(1, ni + 1):
            fc = fzk[i, 1:nj + 1]
            if rotllr:
                zhxvtn = (dtrdy * rmv[i + 1]) * mx[i - 1]
                zhxvts = (dtrdy * rmv[i]) * mx[i - 1]
                zrfmn = ((zhxvtn * 2.0) * fc) / (fc + fzk[i + 1, 1:nj + 1])
                zrfms = ((zhxvts * 2.0) * fc) / (fc + fzk[i - 1, 1:nj + 1])
                zdv = (V(i + 1) * zrfmn - V(i) * zrfms) * P[k][i - 1]
                p0[i - 1] = ((WZ(i) + zpby[i] * zrfms) - zpby[i + 1] * zrfmn) + zdv
            else:
                zrfmn = ((dtrdy * 2.0) * fc) / (fc + fzk[i + 1, 1:nj + 1])
                zrfms = ((dtrdy * 2.0) * fc) / (fc + fzk[i - 1, 1:nj + 1])
                zdv = ((V(i + 1) * rmv[i + 1]) * zrfmn - (V(i) * rmv[i]) * zrfms) * P[k][i - 1]
                p0[i - 1] = WZ(i) + mx2[i - 1] * ((zpby[i] * zrfms - zpby[i + 1] * zrfmn) + zdv)
        # zonal: p0 with its periodic ring of two columns, Fortran j = -1 .. nj+2
        pext = np.concatenate([p0[:, nj - 2:nj], p0, p0[:, 0:2]], axis=1)  # column q <-> j = q - 1

        def P0(j):
            return pext[:, j + 1]

        jmin, jmax = -1, nj + 2
        uk = u.ji(0, nj + 2, 1, ni, k)  # columns j = 0 .. nj+2
        mu = msfu.ji(0, nj + 1, 1, ni)  # columns j = 0 .. nj+1
        rmu = 1.0 / mu
        zpbw = {}
        for j in range(1, nj + 2):
            zamu = (uk[:, j] * mu[:, j]) * dtrdx if rotllr else (uk[:, j] * rmu[:, j]) * dtrdx
            pos = zamu > 0.0
            is_ = np.where(pos, 1.0, -1.0)
            jhp = min(j + 1, jmax)
            num = np.where(pos, P0(j - 1) - P0(max(j - 2, jmin)), P0(jhp) - P0(max(jhp - 1, jmin)))
            r = num / safe_den(P0(j) - P0(j - 1))
            b = superbee(r)
            zphi = (is_ + zamu * b) - is_ * b
            uh = 0.5 * uk[:, j] if rotllr else (0.5 * uk[:, j]) * rmu[:, j]
            zpbw[j] = uh * ((1.0 + zphi) * P0(j - 1) + (1.0 - zphi) * P0(j))
        for j in range(1, nj + 1):
            fc = fzk[1:ni + 1, j]
            if rotllr:
                zcostx = dtrdx * mu[:, j]
                zrfme = ((zcostx * 2.0) * fc) / (fc + fzk[1:ni + 1, j + 1])
                zrfmw = ((zcostx * 2.0) * fc) / (fc + fzk[1:ni + 1, j - 1])
                zdv = (uk[:, j + 1] * zrfme - uk[:, j] * zrfmw) * P[k][:, j - 1]
                new[k - 1][:, j - 1] = ((P0(j) + zpbw[j] * zrfmw) - zpbw[j + 1] * zrfme) + zdv
            else:
                zrfme = ((dtrdx * 2.0) * fc) / (fc + fzk[1:ni + 1, j + 1])
                zrfmw = ((dtrdx * 2.0) * fc) / (fc + fzk[1:ni + 1, j - 1])
                zdv = ((uk[:, j + 1] * rmu[:, j + 1]) * zrfme - (uk[:, j] * rmu[:, j]) * zrfmw) * P[k][:, j - 1]
                new[k - 1][:, j - 1] = P0(j) + mx2[:, j - 1] * ((zpbw[j] * zrfmw - zpbw[j + 1] * zrfme) + zdv)
    return new


@pytest.mark.parametrize("rotllr", [True, False])
def test_wafone_restated(oracle_mod, rotllr):
    """After the staggering has filled the u, v rings (as advection() does
    before its wafone calls), wafone of theta and of the cross-point u."""
    o = make(oracle_mod, ("u", "v", "tetav"), rotllr=rotllr)
    if not rotllr:
        skew_map_factors(o, 23)
    rng = np.random.default_rng(3)
    for n in ("u", "v"):  # winds of both signs, so both upwind branches run
        a = o.get(n)
        o.set(n, a * np.where(rng.uniform(size=a.shape) < 0.5, -1.0, 1.0))
    o.stagger(True)
    for n in ("u", "v", "s"):
        a = o.get(n)
        assert (a > 0).any() and (a < 0).any(), n
    sc = (ctypes.c_double * 9)()
    oracle_mod.lib().oracle_scalars(o.h, sc)
    dt, dx, dzita, nadv = sc[0], sc[1], sc[2], sc[6]
    args = dict(s=o.get("s"), fmz=Bounded(o, "fmz"), fmzf=o.get("fmzf"), u=Bounded(o, "u"),
                v=Bounded(o, "v"), msfu=Bounded(o, "msfu"), msfv=Bounded(o, "msfv"),
                msfx=Bounded(o, "msfx"), dta=dt / nadv, dx=dx, dzita=dzita, rotllr=rotllr)
    for name in ("tetav", "ux"):
        want = wafone_np(o.get(name), **args)
        before = o.get(name)
        o.wafone(name)
        got = o.get(name)
        assert np.max(np.abs(got - before)) > 1e-6 * np.max(np.abs(before)), name  # it moved
        err = np.max(np.abs(got - want)) / np.max(np.abs(want))
        assert err <= 1e-14, (name, err)
    o.close()


# ---- divdamp, ROTLLR branch (nompi/mod_moloch.F90:853-895) -----------------
XDAMP = 0.0625  # :96


def divdamp_np(u, v, zdiv2, xknu, mu, dx, dts, mv=None):
    """u, v, zdiv2: interiors (kz, ni, nj); xknu (kz,); mu: msfu interior
    (ni, nj); mv: msfv interior for the non-ROTLLR form (:874-881), None
    for ROTLLR.  The width-1 ring of zdiv2 is its periodic image
    (:858-861).  Returns the new u, v, zdiv2."""
    ddamp = 0.125 * (dx / dts)
    zw = np.roll(zdiv2, 1, 2)  # zdiv2(j-1)
    zs = np.roll(zdiv2, 1, 1)  # zdiv2(i-1)
    c = (xknu * ddamp)[:, None, None]
    u2 = u + ((c * mu[None]) * (zdiv2 - zw))
    v2 = v + (c * (zdiv2 - zs)) if mv is None else v + ((c * mv[None]) * (zdiv2 - zs))
    ddamp = (XDAMP * 0.015625) / dts
    p2d = 0.125 * (((zw + np.roll(zdiv2, -1, 2)) + zs) + np.roll(zdiv2, -1, 1)) - 0.5 * zdiv2
    return u2, v2, zdiv2 + ddamp * p2d


def test_divdamp_restated(oracle_mod):
    o = make(oracle_mod, ("u", "v"))
    rng = np.random.default_rng(11)
    z = o.get("zdiv2")
    o.set("zdiv2", z + 1e-4 * rng.standard_normal(z.shape))  # a divergence field of both signs
    sc = (ctypes.c_double * 9)()
    oracle_mod.lib().oracle_scalars(o.h, sc)
    dt, dx, nadv, nsound = sc[0], sc[1], sc[6], sc[7]
    xk = (ctypes.c_double * o.kz)()
    oracle_mod.lib().oracle_xknu(o.h, xk)
    xknu = np.array(list(xk))
    mu = Bounded(o, "msfu").ji(1, o.nj, 1, o.ni)
    u2, v2, z2 = divdamp_np(o.get("u"), o.get("v"), o.get("zdiv2"), xknu, mu, dx, dt / nadv / nsound)
    o.divdamp()
    for n, want in (("u", u2), ("v", v2), ("zdiv2", z2)):
        got = o.get(n)
        assert np.max(np.abs(got - want)) <= 1e-15 * np.max(np.abs(want)), n
    o.close()


# ---- sound(), ROTLLR branch (nompi/mod_moloch.F90:483-851) -----------------
WLHV = 2500610.0  # mod_constants.F90:167


def pad1(a):
    """The width-1 periodic ring (corners included) around (levels, i, j)."""
    return np.pad(a, ((0, 0), (1, 1), (1, 1)), mode="wrap")


def gzita_np(zita, ztop, a0):
    # nompi/mod_zita.F90:109-120; ratio**2 = r r, ratio**3 = (r r) r
    r = zita / ztop
    r2 = r * r
    return (((0.0 - 1.0 * a0) * r - (3.0 - 2.0 * a0) * r2) + (2.0 - 1.0 * a0) * (r2 * r)) + 1.0


def zita_levels(kz, ztop):
    # model_zitaf / model_zitah (nompi/mod_zita.F90:57-85), accumulated from the ground
    dz = ztop / float(kz)
    zf = np.zeros(kz + 1)
    for k in range(kz - 1, -1, -1):
        zf[k] = zf[k + 1] + dz
    zh = np.zeros(kz)
    zh[kz - 1] = dz * 0.5
    for k in range(kz - 2, -1, -1):
        zh[k] = zh[k + 1] + dz
    return zf, zh


def sound_np(st, sc, c, dts, nsub, rotllr=True):
    """One sound() call: nsub substeps of dts.  st: interiors (levels, i, j)
    of the state and the diagnostics; sc: Bounded statics and the 1-D level
    tables; c: constants.  Returns the new u, v, w, pai, tetav, s, deltaw,
    zdiv2."""
    u, v, w = st["u"].copy(), st["v"].copy(), st["w"].copy()
    pai, tet, s, dw = st["pai"].copy(), st["tetav"].copy(), st["s"].copy(), st["deltaw"].copy()
    kz, ni, nj = u.shape
    cpd, rdrcv, rwat, egrav = c["cpd"], c["rdrcv"], c["rwat"], EGRAV
    dtrdx = dts / sc["dx"]
    dtrdy = dts / sc["dx"]
    dtrdz = dts / sc["dzita"]
    zcs2 = (dtrdz * dtrdz) * rdrcv
    F = sc["fmz"].data  # (kz, ni+2, nj+2): rings i, j = 0 .. n+1
    FI = F[:, 1:ni + 1, 1:nj + 1]
    fmzf, qv, qc, qs_, t = st["fmzf"], st["qv"], st["qc"], st["qsat"], st["t"]
    qwl, qwi = st["qwltot"], st["qwitot"]
    hx = sc["hx"].ji(1, nj + 1, 1, ni)   # columns j = 1 .. nj+1
    hy = sc["hy"].ji(1, nj, 1, ni + 1)   # rows i = 1 .. ni+1
    mx = sc["msfx"].ji(1, nj, 1, ni)
    mu = sc["msfu"].ji(1, nj, 1, ni)
    rmv = 1.0 / sc["msfv"].ji(1, nj, 1, ni + 1)  # rows i = 1 .. ni+1
    rmu = 1.0 / sc["msfu"].ji(1, nj + 1, 1, ni)  # columns j = 1 .. nj+1
    mv = sc["msfv"].ji(1, nj, 1, ni)
    coru = sc["coru"].ji(1, nj, 1, ni)
    corv = sc["corv"].ji(1, nj, 1, ni)
    gk, gkh = sc["gzitak"], sc["gzitakh"]  # Fortran level k -> index k-1
    I, J = slice(1, ni + 1), slice(1, nj + 1)
    wwkw = np.zeros((kz + 1, ni, nj))
    for n in range(1, nsub + 1):
        U, V = pad1(u), pad1(v)  # rings and corners at the start of the substep (:512-527)
        # surface w and s (:529-565)
        zuh = U[kz - 1][I, J] * hx[:, 0:nj] + U[kz - 1][I, 2:nj + 2] * hx[:, 1:nj + 1]
        zvh = V[kz - 1][I, J] * hy[0:ni] + V[kz - 1][2:ni + 2, J] * hy[1:ni + 1]
        w[kz] = 0.5 * (zuh + zvh)
        s[kz] = -w[kz]
        for k in range(2, kz + 1):
            uu, vv = U[k - 1] + U[k - 2], V[k - 1] + V[k - 2]
            zuh = uu[I, J] * hx[:, 0:nj] + uu[I, 2:nj + 2] * hx[:, 1:nj + 1]
            zvh = vv[I, J] * hy[0:ni] + vv[2:ni + 2, J] * hy[1:ni + 1]
            s[k - 1] = -((0.25 * (zuh + zvh)) * gk[k - 1])
        # Equation 16 (:575-597)
        zdiv2 = np.empty((kz, ni, nj))
        for k in range(1, kz + 1):
            f = F[k - 1]
            fc = f[I, J]
            zrfmzum = 2.0 / (fc + f[I, 0:nj])
            zrfmzvm = 2.0 / (fc + f[0:ni, J])
            zrfmzup = 2.0 / (fc + f[I, 2:nj + 2])
            zrfmzvp = 2.0 / (fc + f[2:ni + 2, J])
            if rotllr:
                zum = (dtrdx * U[k - 1][I, J]) * zrfmzum
                zup = (dtrdx * U[k - 1][I, 2:nj + 2]) * zrfmzup
                zvm = ((dtrdy * V[k - 1][I, J]) * zrfmzvm) * rmv[0:ni]
                zvp = ((dtrdy * V[k - 1][2:ni + 2, J]) * zrfmzvp) * rmv[1:ni + 1]
                zdiv2[k - 1] = (fc * mx) * ((zup - zum) + (zvp - zvm))
            else:  # :598-621
                zum = ((dtrdx * U[k - 1][I, J]) * rmu[:, 0:nj]) * zrfmzum
                zup = ((dtrdx * U[k - 1][I, 2:nj + 2]) * rmu[:, 1:nj + 1]) * zrfmzup
                zvm = ((dtrdy * V[k - 1][I, J]) * rmv[0:ni]) * zrfmzvm
                zvp = ((dtrdy * V[k - 1][2:ni + 2, J]) * rmv[1:ni + 1]) * zrfmzvp
                zdiv2[k - 1] = ((mx * mx) * fc) * ((zup - zum) + (zvp - zvm))
        u, v, zdiv2 = divdamp_np(u, v, zdiv2, sc["xknu"], mu, sc["dx"], dts, None if rotllr else mv)
        for k in range(1, kz + 1):
            zdiv2[k - 1] = zdiv2[k - 1] + (FI[k - 1] * dtrdz) * (s[k - 1] - s[k])
        # implicit w (:634-679)
        wwkw[kz] = 0.0
        for k in range(kz, 1, -1):
            a, b = k - 1, k - 2  # indices of levels k and k-1
            dw[a] = -w[a]
            zrom1w = ((0.5 * cpd) * fmzf[a]) * (tet[b] + tet[a])
            zrom1w = zrom1w - (((((cpd * w[a]) * fmzf[a]) * fmzf[a]) * float(n)) * dtrdz) * (tet[b] - tet[a])
            moist = (qv[a] > 0.96 * qs_[a]) & (w[a] > 0.1)
            zqs = 0.5 * (qs_[a] + qs_[b])
            zdth = ((((((egrav * w[a]) * float(n - 1)) * dts) * WLHV) * WLHV) * zqs) / \
                ((((cpd * pai[b]) * rwat) * t[b]) * t[b])
            zrom1w = np.where(moist, zrom1w + zdth * fmzf[a], zrom1w)
            zwexpl = (w[a] - (zrom1w * dtrdz) * (pai[b] - pai[a])) - egrav * dts
            zwexpl = zwexpl + ((rdrcv * zrom1w) * dtrdz) * (pai[b] * zdiv2[b] - pai[a] * zdiv2[a])
            zu = ((zcs2 * FI[b]) * zrom1w) * pai[b] + 0.0  # + ffilt(k), zero
            zd = ((zcs2 * FI[a]) * zrom1w) * pai[a] + 0.0
            zrapp = 1.0 / (((1.0 + zd) + zu) - zd * wwkw[a + 1])
            w[a] = zrapp * (zwexpl + zd * w[a + 1])
            wwkw[a] = zrapp * zu
        for k in range(2, kz + 1):
            a = k - 1
            w[a] = w[a] + wwkw[a] * w[a - 1]
            dw[a] = dw[a] + w[a]
        # new Exner function and theta (:683-712)
        for k in range(1, kz + 1):
            a = k - 1
            zdiv2[a] = zdiv2[a] + (dtrdz * FI[a]) * (w[a] - w[a + 1])
        zdiv2 = (zdiv2 * ((1.0 + 0.86 * qv) + 3.2 * qc)) / ((1.0 + 0.96 * qv) + 4.8 * qc)
        tet = tet * (1.0 + (rdrcv * zdiv2) * ((0.25 * qv + 4.2 * qwl) + 2.1 * qwi))
        TET = pad1(tet)
        # the pai ring is filled before the update (:716-728), the deltaw ring after the solve
        PAI = pad1(pai)
        pai = pai * (1.0 - rdrcv * zdiv2)
        PAI[:, I, J] = pai
        DW = pad1(dw)
        # ud, vd: the rings keep the values from the start of the substep (:730-735)
        UD, VD = U.copy(), V.copy()
        UD[:, I, J] = u
        VD[:, I, J] = v
        # Equations 17 and 18 (:737-787)
        un = np.empty_like(u)
        vn = np.empty_like(v)
        for k in range(1, kz + 1):
            a = k - 1
            zcx = dtrdx * mu
            zfz = egrav * dts + 0.25 * (((DW[a][I, 0:nj] + DW[a + 1][I, 0:nj]) + DW[a][I, J]) + DW[a + 1][I, J])
            zrom1u = (0.5 * cpd) * (TET[a][I, 0:nj] + TET[a][I, J])
            zcor1u = ((coru * dts) * 0.25) * (((VD[a][I, J] + VD[a][I, 0:nj]) + VD[a][2:ni + 2, 0:nj]) +
                                               VD[a][2:ni + 2, J])
            un[a] = ((u[a] + zcor1u) - ((zfz * hx[:, 0:nj]) * gkh[a])) - \
                ((zcx * zrom1u) * (PAI[a][I, J] - PAI[a][I, 0:nj]))
            zcy = dtrdy if rotllr else dtrdy * mv  # :797 non-ROTLLR
            zfz = egrav * dts + 0.25 * (((DW[a][0:ni, J] + DW[a + 1][0:ni, J]) + DW[a][I, J]) + DW[a + 1][I, J])
            zrom1v = (0.5 * cpd) * (TET[a][0:ni, J] + TET[a][I, J])
            zcor1v = ((corv * dts) * 0.25) * (((UD[a][I, J] + UD[a][0:ni, J]) + UD[a][I, 2:nj + 2]) +
                                               UD[a][0:ni, 2:nj + 2])
            vn[a] = ((v[a] - zcor1v) - ((zfz * hy[0:ni]) * gkh[a])) - \
                ((zcy * zrom1v) * (PAI[a][I, J] - PAI[a][0:ni, J]))
        u, v = un, vn
    # complete Equation 10 (:841-849)
    for k in range(2, kz + 1):
        s[k - 1] = (w[k - 1] + s[k - 1]) * fmzf[k - 1]
    s[0] = 0.0
    s[kz] = 0.0
    return {"u": u, "v": v, "w": w, "pai": pai, "tetav": tet, "s": s, "deltaw": dw, "zdiv2": zdiv2}


def skew_map_factors(o, seed):
    """Map factors within 5 % of 1 instead of the idealized grid's 1, so the
    non-ROTLLR branches' factors change the result."""
    rng = np.random.default_rng(seed)
    arrs = [o.get_bounded(n)[0] for n in ("msfu", "msfv", "msfx")]
    o.set_map_factors(*[a * (1.0 + 0.05 * rng.uniform(-1.0, 1.0, a.shape)) for a in arrs])


@pytest.mark.parametrize("rotllr", [True, False])
def test_sound_restated(oracle_mod, rotllr):
    """One sound() call (five substeps) from a developed state with a moist,
    rising region, so the latent-heat branch of the explicit w runs.  The
    non-ROTLLR case runs with map factors other than 1."""
    o = make(oracle_mod, ("u", "v", "pai", "tetav"), rotllr=rotllr)
    if not rotllr:
        skew_map_factors(o, 21)
    w = o.get("w")
    rng = np.random.default_rng(13)
    w[1:-1] = 0.3 * rng.standard_normal(w[1:-1].shape)  # w(1) = 0 and the surface w stay
    o.set("w", w)
    qv, qsat = o.get("qv"), o.get("qsat")
    qv[:, 2:6, 3:8] = 0.98 * qsat[:, 2:6, 3:8]
    o.set("qv", qv)
    cst = (ctypes.c_double * 11)()
    oracle_mod.lib().oracle_constants(cst)
    c = {"rwat": cst[1], "cpd": cst[2], "rdrcv": cst[4]}
    scal = (ctypes.c_double * 9)()
    oracle_mod.lib().oracle_scalars(o.h, scal)
    dt, dx, dzita, ztop, a0, nadv, nsound = scal[0], scal[1], scal[2], scal[3], scal[5], scal[6], scal[7]
    xk = (ctypes.c_double * o.kz)()
    oracle_mod.lib().oracle_xknu(o.h, xk)
    zf, zh = zita_levels(o.kz, ztop)
    sc = {n: Bounded(o, n) for n in ("fmz", "hx", "hy", "coru", "corv", "msfu", "msfv", "msfx")}
    sc.update(dx=dx, dzita=dzita, xknu=np.array(list(xk)), gzitak=gzita_np(zf, ztop, a0),
              gzitakh=gzita_np(zh, ztop, a0))
    st = {n: o.get(n) for n in ("u", "v", "w", "pai", "tetav", "s", "deltaw", "fmzf", "qv", "qc", "qsat",
                                "t", "qwltot", "qwitot")}
    moist = (st["qv"][1:] > 0.96 * st["qsat"][1:]) & (st["w"][1:-1] > 0.1)
    assert moist.any()  # the latent-heat branch is taken somewhere
    want = sound_np(st, sc, c, dt / nadv / nsound, int(nsound), rotllr)
    o.phase(1)
    for n, v in want.items():
        got = o.get(n)
        err = np.max(np.abs(got - v)) / max(np.max(np.abs(v)), 1e-300)
        assert err <= 1e-13, (n, err)
    o.close()


# ---- the 3-D filters (nompi/mod_moloch.F90:423-481) ------------------------
NUPAITQ = 0.05  # :106


def lap_filter_np(a, coef):
    """a + coef(k) (0.125 (aW + aE + aS + aN) - 0.5 a), ring periodic; coef
    per level (kz,)."""
    p2d = 0.125 * (((np.roll(a, 1, 2) + np.roll(a, -1, 2)) + np.roll(a, 1, 1)) + np.roll(a, -1, 1)) - 0.5 * a
    return a + coef[:, None, None] * p2d


def test_filters_restated(oracle_mod):
    o = make(oracle_mod, ("pai", "tetav"))
    rng = np.random.default_rng(17)
    z = o.get("zdiv2")
    o.set("zdiv2", z + 1e-4 * rng.standard_normal(z.shape))
    scal = (ctypes.c_double * 9)()
    oracle_mod.lib().oracle_scalars(o.h, scal)
    anu2 = scal[8]
    xk = (ctypes.c_double * o.kz)()
    oracle_mod.lib().oracle_xknu(o.h, xk)
    xknu = np.array(list(xk))
    for which, name, coef in ((0, "zdiv2", anu2 * xknu), (1, "pai", np.full(o.kz, NUPAITQ)),
                              (2, "tetav", np.full(o.kz, NUPAITQ))):
        want = lap_filter_np(o.get(name), coef)
        o.filter(which)
        got = o.get(name)
        assert np.max(np.abs(got - want)) <= 1e-15 * np.max(np.abs(want)), name
    o.close()


# ---- the lprint printout (nompi/mod_moloch.F90:395-411) --------------------
def test_lprint_restated(oracle_mod):
    """maxval/minval of ps over the interior and of u, v over the interior
    columns and all levels, as moloch(istep, .true.) prints them."""
    o = make(oracle_mod, ())
    bad, d = o.step(2, lprint=True)
    ps, u, v = o.get("ps"), o.get("u"), o.get("v")
    assert bad == 0
    assert d == [ps.max(), ps.min(), u.max(), u.min(), v.max(), v.min()]
    o.close()


# ---- the initial state: fill_atmosphere (nompi/mod_atmosphere.F90:171-235) -
def test_fill_atmosphere_restated(oracle_mod):
    """qv, t (with the warm bubble on the lowest level) and the hydrostatic
    pai of the idealized state over a hill, from the oracle's zeta and
    fmzf.  The bubble radius mixes default-REAL and FP64 arithmetic (:199:
    real(iy)/5_rkx is a default-REAL division, and md is a default-REAL
    sqrt), restated here with float32."""
    jx, iy, kz = 23, 19, 12
    cfg = oracle_mod.make_cfg(jx, iy, kz, hills=((600.0, 9.0, 11.0, 4.0),), pert_amp=0.0)
    o = oracle_mod.Oracle(cfg)
    cst = (ctypes.c_double * 11)()
    oracle_mod.lib().oracle_constants(cst)
    rgas, cpd, rovcp, ep1 = cst[0], cst[2], cst[6], cst[7]
    scal = (ctypes.c_double * 9)()
    oracle_mod.lib().oracle_scalars(o.h, scal)
    dzita = scal[2]
    zeta, fmzf = o.get("zeta"), o.get("fmzf")
    ts, qs, ps, tropoh = 300.0, 0.01865, 101480.0, 15000.0
    tvs = ts * (1.0 + ep1 * qs)
    tvt = tvs - LRATE * tropoh
    low = zeta < tropoh
    qi = (qs * np.exp(-zeta / 4000.0)) * np.exp((-zeta / 7500.0) ** 2)
    qv = np.where(low, qi, 1.0e-8)
    t = np.where(low, (tvs - LRATE * zeta) / (1.0 + qi), tvt)
    mx, my = jx // 2, iy // 2
    bi = np.float32(np.float32(iy) / np.float32(5))
    mr = np.sqrt((float(np.float32(jx)) / 5.0) ** 2 + float(bi * bi)) / 2.0
    j = np.arange(1, jx + 1)[None, :]
    i = np.arange(1, iy + 1)[:, None]
    fj, fi = (j - mx).astype(np.float32), (i - my).astype(np.float32)
    md = np.sqrt(fj * fj + fi * fi).astype(np.float64)  # float32 sqrt, widened
    t[kz - 1] = np.where(md < mr, t[kz - 1] + (mr - md) / mr, t[kz - 1])
    pai = np.empty_like(t)
    zdelta = zeta[kz - 1] * EGRAV
    tv1 = t[kz - 1] * (1.0 + ep1 * qv[kz - 1])
    tv2 = t[kz - 2] * (1.0 + ep1 * qv[kz - 2])
    lrt = (tv2 - tv1) / (zeta[kz - 2] - zeta[kz - 1])
    lrt = 0.65 * lrt - 0.35 * LRATE
    tv = tv1 - (0.5 * zeta[kz - 1]) * lrt
    zz = 1.0 / (rgas * tv)
    p = ps * np.exp(-zdelta * zz)
    pai[kz - 1] = (p / P00) ** rovcp
    for k in range(kz - 1, 0, -1):  # Fortran k = kz-1 .. 1; index k-1
        a = k - 1
        tv1 = t[a] * (1.0 + ep1 * qv[a])
        tv2 = t[a + 1] * (1.0 + ep1 * qv[a + 1])
        zb = (((2.0 * EGRAV) * dzita) / (fmzf[a + 1] * cpd) + tv1) - tv2
        zd = np.sqrt(zb * zb + (4.0 * tv2) * tv1)
        pai[a] = -((pai[a + 1] / (2.0 * tv2)) * (zb - zd))
    assert (md < mr).any() and (md >= mr).any()  # the bubble covers part of the level
    for n, want in (("qv", qv), ("t", t), ("pai", pai)):
        got = o.get(n)
        err = np.max(np.abs(got - want) / np.abs(want))
        assert err <= 1e-14, (n, err)
    assert np.all(o.get("u") == 1.0) and np.all(o.get("v") == 1.0)
    o.close()


# ---- param(): orography terms and the zita metric (regcm_dynamical_core.F90:93-194,
# ---- nompi/mod_zita.F90:88-179) --------------------------------------------
def zfz_np(ztop, zh):
    return ztop / (np.exp(ztop / zh) - 1.0)


def md_zeta_np(zita, geopot, ztop, zh, a0):
    orog = geopot * (1.0 / EGRAV)  # geopot * regrav
    return orog * (gzita_np(zita, ztop, a0) - 1.0) + zfz_np(ztop, zh) * (np.exp(zita / zh) - 1.0)


def md_fmz_np(zita, geopot, ztop, zh, a0):
    orog = geopot * (1.0 / EGRAV)
    r = zita / ztop
    gzp = (((0.0 - 1.0 * a0) * 1.0 - (6.0 - 4.0 * a0) * r) + (6.0 - 3.0 * a0) * (r * r)) / ztop
    bzp = (zfz_np(ztop, zh) * np.exp(zita / zh)) / zh
    return 1.0 / (gzp * orog + bzp)


def test_param_restated(oracle_mod):
    """hx, hy from the orography (with the ghosts of ht at 0, never set by
    the reference), zeta, fmz and fmzf on the zita levels, and their
    periodic rings, for hills that reach the domain's edges."""
    jx, iy, kz = 17, 14, 10
    cfg = oracle_mod.make_cfg(jx, iy, kz, hills=((700.0, 2.0, 3.0, 3.0), (400.0, 15.0, 12.0, 2.5)))
    o = oracle_mod.Oracle(cfg)
    scal = (ctypes.c_double * 9)()
    oracle_mod.lib().oracle_scalars(o.h, scal)
    dx, ztop, zh, a0 = scal[1], scal[3], scal[4], scal[5]
    ht_b = Bounded(o, "ht")
    assert ht_b.lb[:2] == (-1, -1)
    full = ht_b.data[0]
    ring = full.copy()
    ring[2:iy + 2, 2:jx + 2] = 0.0
    assert np.all(ring == 0.0)  # the ghosts stay 0
    ht = np.zeros((iy + 2, jx + 2))  # i, j = 0 .. n+1, ghosts 0
    ht[1:iy + 1, 1:jx + 1] = full[2:iy + 2, 2:jx + 2]
    rdx, regrav = 1.0 / dx, 1.0 / EGRAV
    hx = np.empty((iy, jx + 2))
    hx[:, 1:jx + 1] = (((ht[1:iy + 1, 1:jx + 1] - ht[1:iy + 1, 0:jx]) * 1.0) * rdx) * regrav  # msfu = 1
    hx[:, 0], hx[:, jx + 1] = hx[:, jx], hx[:, 1]
    hy = np.empty((iy + 2, jx))
    hy[1:iy + 1] = ((ht[1:iy + 1, 1:jx + 1] - ht[0:iy, 1:jx + 1]) * rdx) * regrav
    hy[0], hy[iy + 1] = hy[iy], hy[1]
    assert np.array_equal(Bounded(o, "hx").data[0], hx)
    assert np.array_equal(Bounded(o, "hy").data[0], hy)
    assert hx[:, 1].any() and hy[1].any()  # the hills reach the first row and column
    zf, zhf = zita_levels(kz, ztop)
    g = ht[1:iy + 1, 1:jx + 1]
    zeta = np.stack([md_zeta_np(zhf[k], g, ztop, zh, a0) for k in range(kz)])
    fmz = np.stack([md_fmz_np(zhf[k], g, ztop, zh, a0) for k in range(kz)])
    fmzf = np.stack([md_fmz_np(zf[k], g, ztop, zh, a0) for k in range(kz + 1)])
    zeta_b = np.pad(zeta, ((0, 0), (2, 2), (2, 2)), mode="wrap")
    fmz_b = np.pad(fmz, ((0, 0), (1, 1), (1, 1)), mode="wrap")
    for n, want, tol in (("zeta", zeta_b, 1e-14), ("fmz", fmz_b, 1e-14)):
        got = Bounded(o, n).data
        # the rings' corners are not filled by the reference (never read)
        mask = np.ones(want.shape[1:], bool)
        w = 2 if n == "zeta" else 1
        mask[:w, :w] = mask[:w, -w:] = mask[-w:, :w] = mask[-w:, -w:] = False
        err = np.max(np.abs(got[:, mask] - want[:, mask]) / np.abs(want[:, mask]))
        assert err <= tol, (n, err)
    err = np.max(np.abs(o.get("fmzf") - fmzf) / np.abs(fmzf))
    assert err <= 1e-14, ("fmzf", err)
    o.close()


# ---- one whole moloch() step from the pieces above (nompi/mod_moloch.F90:272-421)
class Padded(Bounded):
    """A periodic field with a ring of width w on the j and i sides."""

    def __init__(self, a, w):
        self.data = np.pad(a, ((0, 0), (w, w), (w, w)), mode="wrap")
        self.lb = (1 - w, 1 - w, 1)


def test_whole_step_restated(oracle_mod):
    """reset_tendencies, the pre-diagnostics, three times sound() and
    advection() (ten fields), the post-diagnostics, composed in the order of
    moloch() from the restatements above, against one oracle step."""
    o = make(oracle_mod, ("u", "v", "t", "pai"))
    cst = (ctypes.c_double * 11)()
    oracle_mod.lib().oracle_constants(cst)
    c = {"rgas": cst[0], "rwat": cst[1], "cpd": cst[2], "rdrcv": cst[4], "cpovr": cst[5], "ep1": cst[7],
         "ep2": cst[8]}
    scal = (ctypes.c_double * 9)()
    oracle_mod.lib().oracle_scalars(o.h, scal)
    dt, dx, dzita, ztop, a0, nadv, nsound = scal[0], scal[1], scal[2], scal[3], scal[5], int(scal[6]), int(scal[7])
    xk = (ctypes.c_double * o.kz)()
    oracle_mod.lib().oracle_xknu(o.h, xk)
    zf, zh = zita_levels(o.kz, ztop)
    sc = {n: Bounded(o, n) for n in ("fmz", "hx", "hy", "coru", "corv", "msfu", "msfv", "msfx")}
    sc.update(dx=dx, dzita=dzita, xknu=np.array(list(xk)), gzitak=gzita_np(zf, ztop, a0),
              gzitakh=gzita_np(zh, ztop, a0))
    f = {n: o.get(n) for n in ("u", "v", "w", "pai", "t", "qv", "qc", "qi", "qr", "qs", "fmzf", "zeta")}
    kz = o.kz
    # reset_tendencies (:1313-1325) and the pre-diagnostics (:289-323)
    s = np.zeros((kz + 1,) + f["u"].shape[1:])
    dw = np.zeros_like(s)
    p = (f["pai"] ** c["cpovr"]) * P00
    qsat = pfwsat(f["t"], p, c["ep2"])
    tvirt = f["t"] * (1.0 + c["ep1"] * f["qv"] - f["qc"] - f["qi"] - f["qr"] - f["qs"])
    qwl, qwi = f["qc"] + f["qr"], f["qi"] + f["qs"]
    tet = tvirt / f["pai"]
    u, v, w, pai = f["u"], f["v"], f["w"], f["pai"]
    q = {n: f[n] for n in ("qv", "qc", "qi", "qr", "qs")}
    dta = dt / nadv
    for _ in range(nadv):
        st = {"u": u, "v": v, "w": w, "pai": pai, "tetav": tet, "s": s, "deltaw": dw, "fmzf": f["fmzf"],
              "qv": q["qv"], "qc": q["qc"], "qsat": qsat, "t": f["t"], "qwltot": qwl, "qwitot": qwi}
        r = sound_np(st, sc, c, dta / nsound, nsound)
        u, v, w, pai, tet, s, dw = r["u"], r["v"], r["w"], r["pai"], r["tetav"], r["s"], r["deltaw"]
        # advection (:897-927)
        ux, vx = uv_to_x(u, v)
        wx = w_to_x(w)
        args = dict(s=s, fmz=sc["fmz"], fmzf=f["fmzf"], u=Padded(u, 2), v=Padded(v, 2), msfu=sc["msfu"],
                    msfv=sc["msfv"], msfx=sc["msfx"], dta=dta, dx=dx, dzita=dzita)
        tet, pai, ux, vx, wx = (wafone_np(a, **args) for a in (tet, pai, ux, vx, wx))
        q = {n: wafone_np(a, **args) for n, a in q.items()}
        u, v = x_to_uv(ux, vx)
        w = x_to_w(wx, w)
    # the post-diagnostics (:355-391)
    tvirt = tet * pai
    t = tvirt / (1.0 + c["ep1"] * q["qv"] - q["qc"] - q["qi"] - q["qr"] - q["qs"])
    p = (pai ** c["cpovr"]) * P00
    rho = p / (c["rgas"] * t)
    zeta = f["zeta"]
    lrt = 0.65 * ((tvirt[-2] - tvirt[-1]) / (zeta[-2] - zeta[-1])) - 0.35 * LRATE
    ps = p[-1] * np.exp((zeta[-1] * EGRAV) / (c["rgas"] * (tvirt[-1] - 0.5 * zeta[-1] * lrt)))
    want = {"u": u, "v": v, "w": w, "pai": pai, "tetav": tet, "t": t, "p": p, "rho": rho, "ps": ps,
            "qsat": pfwsat(t, p, c["ep2"]), "s": s, **q}
    o.step(2)
    for n, x in want.items():
        err = np.max(np.abs(o.get(n) - x)) / max(np.max(np.abs(x)), 1e-300)
        assert err <= 1e-13, (n, err)
    o.close()
