"""A second restatement of parts of the step, in NumPy and written from the
reference's source alone, against the C oracle: the pointwise diagnostics
of moloch() (the oracle's phases 0, reset + pre-diagnostics, and 3,
post-diagnostics), the staggering of advection(), wafone and divdamp (the
oracle's stagger, wafone and divdamp hooks).

Reference: nompi/mod_moloch.F90:289-323 (p, qsat, tvirt, qwltot, qwitot,
tetav before the advection loop), :355-391 (tvirt, t, p, rho, the
hypsometric ps and qsat after it), :119-181 (pfesat / pfwsat, the Flatau
polynomials); constants of nompi/mod_constants.F90 (p00 :225, lrate :231,
tzero :193, egrav :81).  Tolerance: relative 1e-13 (both evaluate the same
FP64 expressions; NumPy's vectorised exp/pow may differ from libm in the
last bit)."""
import ctypes

import numpy as np

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


def make(oracle_mod, names):
    """A developed state (one step: moisture, winds and theta no longer the
    initial profiles), then the inputs of the phase under test perturbed by
    a seeded relative 1e-3, so that the phase's outputs cannot be left over
    from the step's own diagnostics."""
    cfg = oracle_mod.make_cfg(13, 11, 9, hills=((300.0, 6.5, 5.5, 3.0),), pert_amp=0.5, pert_levels=9,
                              seed=42, u0=3.0, v0=-2.0)
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


def wafone_np(pp, s, fmz, fmzf, u, v, msfu, msfv, msfx, dta, dx, dzita):
    """pp: interior (kz, ni, nj) of the advected field; s, fmzf: interior
    (kz+1, ni, nj); fmz, u, v, msfu, msfv, msfx: Bounded.  Returns the new
    interior of pp."""
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

        zpby = {}
        for i in range(1, ni + 2):
            zamu = V(i) * dtrdy
            pos = zamu > 0.0
            is_ = np.where(pos, 1.0, -1.0)
            ihp = min(i + 1, imax)
            num = np.where(pos, WZ(i - 1) - WZ(max(i - 2, imin)), WZ(ihp) - WZ(max(ihp - 1, imin)))
            r = num / safe_den(WZ(i) - WZ(i - 1))
            b = superbee(r)
            zphi = (is_ + zamu * b) - is_ * b
            zpby[i] = (0.5 * V(i)) * ((1.0 + zphi) * WZ(i - 1) + (1.0 - zphi) * WZ(i))
        fzk = fmz.ji(0, nj + 1, 0, ni + 1, k)  # rows i = 0 .. ni+1, columns j = 0 .. nj+1
        rmv = 1.0 / msfv.ji(1, nj, 0, ni + 1)   # rows i = 0 .. ni+1
        mx = msfx.ji(1, nj, 1, ni)
        p0 = np.empty((ni, nj))
        for i in range(1, ni + 1):
            fc = fzk[i, 1:nj + 1]
            zhxvtn = (dtrdy * rmv[i + 1]) * mx[i - 1]
            zhxvts = (dtrdy * rmv[i]) * mx[i - 1]
            zrfmn = ((zhxvtn * 2.0) * fc) / (fc + fzk[i + 1, 1:nj + 1])
            zrfms = ((zhxvts * 2.0) * fc) / (fc + fzk[i - 1, 1:nj + 1])
            zdv = (V(i + 1) * zrfmn - V(i) * zrfms) * P[k][i - 1]
            p0[i - 1] = ((WZ(i) + zpby[i] * zrfms) - zpby[i + 1] * zrfmn) + zdv
        # zonal: p0 with its periodic ring of two columns, Fortran j = -1 .. nj+2
        pext = np.concatenate([p0[:, nj - 2:nj], p0, p0[:, 0:2]], axis=1)  # column q <-> j = q - 1

        def P0(j):
            return pext[:, j + 1]

        jmin, jmax = -1, nj + 2
        uk = u.ji(0, nj + 2, 1, ni, k)  # columns j = 0 .. nj+2
        mu = msfu.ji(0, nj + 1, 1, ni)  # columns j = 0 .. nj+1
        zpbw = {}
        for j in range(1, nj + 2):
            zamu = (uk[:, j] * mu[:, j]) * dtrdx
            pos = zamu > 0.0
            is_ = np.where(pos, 1.0, -1.0)
            jhp = min(j + 1, jmax)
            num = np.where(pos, P0(j - 1) - P0(max(j - 2, jmin)), P0(jhp) - P0(max(jhp - 1, jmin)))
            r = num / safe_den(P0(j) - P0(j - 1))
            b = superbee(r)
            zphi = (is_ + zamu * b) - is_ * b
            zpbw[j] = (0.5 * uk[:, j]) * ((1.0 + zphi) * P0(j - 1) + (1.0 - zphi) * P0(j))
        for j in range(1, nj + 1):
            fc = fzk[1:ni + 1, j]
            zcostx = dtrdx * mu[:, j]
            zrfme = ((zcostx * 2.0) * fc) / (fc + fzk[1:ni + 1, j + 1])
            zrfmw = ((zcostx * 2.0) * fc) / (fc + fzk[1:ni + 1, j - 1])
            zdv = (uk[:, j + 1] * zrfme - uk[:, j] * zrfmw) * P[k][:, j - 1]
            new[k - 1][:, j - 1] = ((P0(j) + zpbw[j] * zrfmw) - zpbw[j + 1] * zrfme) + zdv
    return new


def test_wafone_restated(oracle_mod):
    """After the staggering has filled the u, v rings (as advection() does
    before its wafone calls), wafone of theta and of the cross-point u."""
    o = make(oracle_mod, ("u", "v", "tetav"))
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
                msfx=Bounded(o, "msfx"), dta=dt / nadv, dx=dx, dzita=dzita)
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


def divdamp_np(u, v, zdiv2, xknu, mu, dx, dts):
    """u, v, zdiv2: interiors (kz, ni, nj); xknu (kz,); mu: msfu interior
    (ni, nj).  The width-1 ring of zdiv2 is its periodic image
    (:858-861).  Returns the new u, v, zdiv2."""
    ddamp = 0.125 * (dx / dts)
    zw = np.roll(zdiv2, 1, 2)  # zdiv2(j-1)
    zs = np.roll(zdiv2, 1, 1)  # zdiv2(i-1)
    c = (xknu * ddamp)[:, None, None]
    u2 = u + ((c * mu[None]) * (zdiv2 - zw))
    v2 = v + (c * (zdiv2 - zs))
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
