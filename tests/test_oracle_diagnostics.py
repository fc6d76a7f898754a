"""A second restatement of the pointwise diagnostics of moloch(), in NumPy
and written from the reference's source alone, against the C oracle's
phases 0 (reset + pre-diagnostics) and 3 (post-diagnostics).

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
