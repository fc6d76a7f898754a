/*
 * moloch_oracle.c -- CPU restatement of the MOLOCH dynamical-core step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: it is linked
 * by the tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg
 * as the checker.  The product (dynamical_model_gb300/) never links it.
 *
 * PARITY UNPINNED: the reference is Fortran and no Fortran compiler exists
 * on any machine this project runs on, so the reference itself cannot be
 * run and it ships no golden vectors or tests.  This restatement is checked
 * by known-answer checks written from the equations
 * (tests/test_oracle_known_answers.py), by a second restatement of its
 * routines in NumPy written from the reference's source alone
 * (tests/test_oracle_restated.py, through the oracle_stagger,
 * oracle_wafone, oracle_divdamp, oracle_filter and oracle_set_map_factors
 * hooks and the phases), and by golden
 * fixtures it generated itself (tests/golden/).  These catch slips and
 * regressions, not a misreading of the reference that both restatements
 * share.
 *
 * What it restates (paths relative to the reference project):
 *   nompi/mod_moloch.F90            moloch(), sound(), divdamp(), advection(),
 *                                   wafone(), filters, staggering, pfesat/pfwsat
 *   nompi/regcm_dynamical_core.F90  param()  (grid, metric, Coriolis)
 *   nompi/mod_atmosphere.F90        fill_atmosphere() (idealized state)
 *   nompi/mod_zita.F90              zita levels, gzita, bzita, fmz, zeta
 *   nompi/mod_constants.F90         physical constants
 * Additions that are not in the reference (input generator only): a seeded
 * splitmix64 theta perturbation, Gaussian hills in ht, a background wind.
 *
 * Arithmetic rules: every expression keeps the reference's evaluation order
 * (Fortran evaluates a*b*c as (a*b)*c); compile with -ffp-contract=off so
 * no multiply-add is fused; Fortran SIGN -> copysign, ** integer -> repeated
 * multiplication, ** real -> pow.  Arrays keep the reference's lower and
 * upper bounds (halo rings included), column-major with j fastest.
 * Loops over independent points carry OpenMP pragmas; results do not depend
 * on the thread count (no floating-point reductions).
 */
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ---- constants: nompi/mod_constants.F90 ------------------------------- */
#define EGRAV 9.80665                               /* :81  */
#define NAVGDR 6.02214076e23                        /* :90  */
#define BOLTZK 1.3806490e-23                        /* :88  */
#define AMD 28.96454                                /* :103 */
#define AMW 18.01528                                /* :105 */
#define RGASMOL (NAVGDR * BOLTZK)                   /* :126 */
#define RGAS ((RGASMOL / AMD) * 1000.0)             /* :130 */
#define RWAT ((RGASMOL / AMW) * 1000.0)             /* :131 */
#define CPD (3.5 * RGAS)                            /* :141 */
#define CVD (2.5 * RGAS)                            /* :145 */
#define WLHV 2500610.0                              /* :167 */
#define REGRAV (1.0 / EGRAV)                        /* :178 */
#define RCPD (1.0 / CPD)                            /* :179 */
#define ROVCP (RGAS * RCPD)                         /* :180 */
#define RDRCV (RGAS / CVD)                          /* :181 */
#define CPOVR (CPD / RGAS)                          /* :182 */
#define TZERO 273.15                                /* :193 */
#define P00 1.000000e5                              /* :225 */
#define LRATE 0.00649                               /* :231 */
#define MATHPI 3.1415926535897932384626433832795029 /* :247 */
#define DEGRAD (MATHPI / 180.0)                     /* :254 */
#define RADDEG (180.0 / MATHPI)                     /* :255 */
#define EARTHRAD 6.371229e6                         /* :275 */
#define EOMEG 7.2921159e-5                          /* :279 */
#define EOMEG2 (2.0 * EOMEG)                        /* :280 */
#define EP1 (AMD / AMW - 1.0)                       /* :296 */
#define EP2 (AMW / AMD)                             /* :299 */

/* nompi/mod_moloch.F90:95-106 */
#define MINDEN 1.0e-30
#define XDAMP 0.0625
#define NUPAITQ 0.05

/* ---- bounded arrays ---------------------------------------------------- */
typedef struct {
  double *p;
  int l1, u1, l2, u2, l3, u3;
  long n1, n12;
} A3;
typedef struct {
  double *p;
  int l1, u1, l2, u2;
  long n1;
} A2;

static A3 a3(int l1, int u1, int l2, int u2, int l3, int u3) {
  A3 a;
  a.l1 = l1; a.u1 = u1; a.l2 = l2; a.u2 = u2; a.l3 = l3; a.u3 = u3;
  a.n1 = u1 - l1 + 1;
  a.n12 = a.n1 * (u2 - l2 + 1);
  a.p = (double *)calloc((size_t)(a.n12 * (u3 - l3 + 1)), sizeof(double));
  return a; /* getmem zero-fills: nompi/mod_memutil.F90:1249 */
}
static A2 a2(int l1, int u1, int l2, int u2) {
  A2 a;
  a.l1 = l1; a.u1 = u1; a.l2 = l2; a.u2 = u2;
  a.n1 = u1 - l1 + 1;
  a.p = (double *)calloc((size_t)(a.n1 * (u2 - l2 + 1)), sizeof(double));
  return a;
}

#ifdef ORACLE_BOUNDS_CHECK
static double *chk3(const A3 *a, int j, int i, int k, const char *f, int l) {
  if (j < a->l1 || j > a->u1 || i < a->l2 || i > a->u2 || k < a->l3 || k > a->u3) {
    fprintf(stderr, "oracle bounds: (%d,%d,%d) outside (%d:%d,%d:%d,%d:%d) at %s:%d\n",
            j, i, k, a->l1, a->u1, a->l2, a->u2, a->l3, a->u3, f, l);
    abort();
  }
  return &a->p[(long)(k - a->l3) * a->n12 + (long)(i - a->l2) * a->n1 + (j - a->l1)];
}
static double *chk2(const A2 *a, int j, int i, const char *f, int l) {
  if (j < a->l1 || j > a->u1 || i < a->l2 || i > a->u2) {
    fprintf(stderr, "oracle bounds: (%d,%d) outside (%d:%d,%d:%d) at %s:%d\n", j, i,
            a->l1, a->u1, a->l2, a->u2, f, l);
    abort();
  }
  return &a->p[(long)(i - a->l2) * a->n1 + (j - a->l1)];
}
#define E3(a, j, i, k) (*chk3(&(a), (j), (i), (k), __FILE__, __LINE__))
#define E2(a, j, i) (*chk2(&(a), (j), (i), __FILE__, __LINE__))
#else
#define E3(a, j, i, k) \
  ((a).p[(long)((k) - (a).l3) * (a).n12 + (long)((i) - (a).l2) * (a).n1 + ((j) - (a).l1)])
#define E2(a, j, i) ((a).p[(long)((i) - (a).l2) * (a).n1 + ((j) - (a).l1)])
#endif

/* ---- configuration (mirrors oracle_cfg in oracle/moloch_oracle.h) ------- */
typedef struct {
  int jx, iy, kz;
  int nhills;
  double hill_h[4], hill_j[4], hill_i[4], hill_r[4]; /* height m, centre, radius (gp) */
  double pert_amp;                                  /* half-width of U(-a,+a) K theta noise */
  int pert_levels;                                  /* lowest levels perturbed */
  unsigned long long seed;
  double u0, v0; /* background wind (reference: 1, 1) */
  int divfilter, filterpai, filtertheta, rotllr;
} oracle_cfg;

typedef struct {
  int nj, ni, kz;
  /* runparams / dynparam */
  double dt, dx, rdx, mo_dzita, mo_anu2, mo_ztop, mo_h, mo_a0;
  int mo_nadv, mo_nsound, divfilter, filterpai, filtertheta, lrotllr;
  double *zita, *zitah, *ffilt; /* 1-based */
  /* mddom */
  A2 ht, xlat, msfx, msfu, msfv, hx, hy, ulat, vlat;
  /* mo_atm */
  A3 u, v, ux, vx, t, tetav, w, pai, qv, qc, qi, qr, qsn, zeta, rho, p, tvirt, qsat, fmz,
      fmzf, zetaf, dz;
  A2 ps;
  /* mod_moloch private (allocate_moloch :183-217) */
  double *gzitak, *gzitakh, *xknu;
  A2 p2d, mx2, rmu, rmv, coru, corv;
  A3 deltaw, s, wx, zdiv2, wz, p0, ud, vd, qwltot, qwitot, pf, tf;
  /* automatic arrays of sound() and wafone() */
  A3 wwkw, wfw, zpby, zpbw;
  double dzita;
  int jmin, jmax, imin, imax;
} Moloch;

/* ---- splitmix64 seeded noise (input generator, not in the reference) --- */
static double splitmix_u01(unsigned long long seed, unsigned long long idx) {
  uint64_t z = (uint64_t)seed + (idx + 1ULL) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z = z ^ (z >> 31);
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

/* ---- nompi/mod_zita.F90 ------------------------------------------------ */
static void model_zitaf(double *zitaf, int kz, double ztop) { /* :57-71 */
  double dz = ztop / (double)kz;
  zitaf[kz + 1] = 0.0;
  for (int k = kz; k >= 1; k--) zitaf[k] = zitaf[k + 1] + dz;
}
static void model_zitah(double *zitah, int kz, double ztop) { /* :73-85 */
  double dz = ztop / (double)kz;
  zitah[kz] = dz * 0.5;
  for (int k = kz - 1; k >= 1; k--) zitah[k] = zitah[k + 1] + dz;
}
static double zfz(double ztop, double zh) { return ztop / (exp(ztop / zh) - 1.0); } /* :88-93 */
static double bzita(double zita, double ztop, double zh) {                           /* :95-100 */
  return zfz(ztop, zh) * (exp(zita / zh) - 1.0);
}
static double bzitap(double zita, double ztop, double zh) { /* :102-107 */
  return zfz(ztop, zh) * exp(zita / zh) / zh;
}
static double gzita(double zita, double ztop, double a0) { /* :109-120 */
  double ratio = zita / ztop;
  double r2 = ratio * ratio, r3 = r2 * ratio;
  return (((0.0 - 1.0 * a0) * ratio - (3.0 - 2.0 * a0) * r2) + (2.0 - 1.0 * a0) * r3) + 1.0;
}
static double gzitap(double zita, double ztop, double a0) { /* :122-132 */
  double ratio = zita / ztop;
  double r2 = ratio * ratio;
  return (((0.0 - 1.0 * a0) * 1.0 - (6.0 - 4.0 * a0) * ratio) + (6.0 - 3.0 * a0) * r2) / ztop;
}
static double md_fmz_h(double zita, double orog, double ztop, double zh, double a0) { /* :135-142 */
  return 1.0 / (gzitap(zita, ztop, a0) * orog + bzitap(zita, ztop, zh));
}
static double md_zeta_h(double zita, double orog, double ztop, double zh, double a0) { /* :144-150 */
  return orog * (gzita(zita, ztop, a0) - 1.0) + bzita(zita, ztop, zh);
}
static double md_fmz(double zita, double geopot, double ztop, double zh, double a0) { /* :166-171 */
  return md_fmz_h(zita, geopot * REGRAV, ztop, zh, a0);
}
static double md_zeta(double zita, double geopot, double ztop, double zh, double a0) { /* :173-179 */
  return md_zeta_h(zita, geopot * REGRAV, ztop, zh, a0);
}

/* ---- nompi/mod_moloch.F90:119-181 saturation --------------------------- */
static double pfesat(double t, double p) {
  const double a0 = 0.611213476e+03, a1 = 0.444007856e+02, a2 = 0.143064234e+01,
               a3_ = 0.264461437e-01, a4 = 0.305903558e-03, a5 = 0.196237241e-05,
               a6 = 0.892344772e-08, a7 = -0.373208410e-10, a8 = 0.209339997e-13;
  const double c0 = 0.611123516e+03, c1 = 0.503109514e+02, c2 = 0.188369801e+01,
               c3 = 0.420547422e-01, c4 = 0.614396778e-03, c5 = 0.602780717e-05,
               c6 = 0.387940929e-07, c7 = 0.149436277e-09, c8 = 0.262655803e-12;
  double t_limit = t - TZERO, td, esat;
  if (t_limit > 100.0) t_limit = 100.0;
  if (t_limit < -75.0) t_limit = -75.0;
  td = t_limit;
  if (td >= 0.0) {
    esat = a0 + td * (a1 + td * (a2 + td * (a3_ + td * (a4 + td * (a5 + td * (a6 + td * (a7 + td * a8)))))));
  } else {
    esat = c0 + td * (c1 + td * (c2 + td * (c3 + td * (c4 + td * (c5 + td * (c6 + td * (c7 + td * c8)))))));
  }
  double lim = 0.15 * p;
  return esat < lim ? esat : lim; /* min(esat, 0.15p) */
}
static double pfwsat(double t, double p) {
  double es = pfesat(t, p);
  return EP2 * (es / (p - es));
}

/* Fortran MAX/MIN on two reals (no NaN handling needed by the algorithm) */
static inline double fmax2(double a, double b) { return a > b ? a : b; }
static inline double fmin2(double a, double b) { return a < b ? a : b; }
/* superbee limiter: b = max(0, min(2, max(r, min(2r, 1)))) */
static inline double superbee(double r) {
  return fmax2(0.0, fmin2(2.0, fmax2(r, fmin2(2.0 * r, 1.0))));
}

/* ---- setup: param (regcm_dynamical_core.F90:93-194) ------------------- */
static void param(Moloch *m, const oracle_cfg *c) {
  int nj = m->nj, ni = m->ni, kz = m->kz;
  double ds = 3.0;
  m->dx = ds * 1000.0;
  m->rdx = 1.0 / m->dx;
  m->dt = 30.0;
  m->mo_ztop = 36000.0;
  m->mo_h = 12000.0;
  m->mo_a0 = 0.0;
  m->mo_nadv = 3;
  m->mo_nsound = 5;
  m->mo_anu2 = 0.6;
  m->zita = (double *)calloc(kz + 2, sizeof(double));
  m->zitah = (double *)calloc(kz + 2, sizeof(double));
  m->ffilt = (double *)calloc(kz + 2, sizeof(double)); /* allocated, zero, never set */
  model_zitaf(m->zita, kz, m->mo_ztop);
  model_zitah(m->zitah, kz, m->mo_ztop);
  m->mo_dzita = m->zita[kz];

  /* mddom%ht = 0 (all, ghosts included); optional hills on the interior */
  for (int h = 0; h < c->nhills; h++) {
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) {
        double dj = (double)j - c->hill_j[h], di = (double)i - c->hill_i[h];
        double rr = (dj * dj + di * di) / (c->hill_r[h] * c->hill_r[h]);
        E2(m->ht, j, i) += c->hill_h[h] * EGRAV * exp(-rr);
      }
  }
  for (long q = 0; q < m->msfx.n1 * (m->msfx.u2 - m->msfx.l2 + 1); q++) m->msfx.p[q] = 1.0;
  for (long q = 0; q < m->msfu.n1 * (m->msfu.u2 - m->msfu.l2 + 1); q++) m->msfu.p[q] = 1.0;
  for (long q = 0; q < m->msfv.n1 * (m->msfv.u2 - m->msfv.l2 + 1); q++) m->msfv.p[q] = 1.0;

  double dl = RADDEG * m->dx / EARTHRAD;
  double clat = 0.0;
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++) {
      E2(m->xlat, j, i) = clat + dl * (((double)i - (double)ni * 0.5) - 0.5);
      E2(m->ulat, j, i) = E2(m->xlat, j, i);
      E2(m->vlat, j, i) = clat + dl * ((double)i - (double)ni * 0.5);
    }
  for (int i = 1; i <= ni; i++) {
    E2(m->msfu, 0, i) = E2(m->msfu, nj, i);
    E2(m->msfu, nj + 1, i) = E2(m->msfu, 1, i);
  }
  for (int j = 1; j <= nj; j++) {
    E2(m->msfv, j, 0) = E2(m->msfv, j, ni);
    E2(m->msfv, j, ni + 1) = E2(m->msfv, j, 1);
  }
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++)
      E2(m->hx, j, i) = (((E2(m->ht, j, i) - E2(m->ht, j - 1, i)) * E2(m->msfu, j, i)) * m->rdx) * REGRAV;
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++) {
      if (m->lrotllr)
        E2(m->hy, j, i) = ((E2(m->ht, j, i) - E2(m->ht, j, i - 1)) * m->rdx) * REGRAV;
      else
        E2(m->hy, j, i) = (((E2(m->ht, j, i) - E2(m->ht, j, i - 1)) * E2(m->msfv, j, i)) * m->rdx) * REGRAV;
    }
  for (int i = 1; i <= ni; i++) {
    E2(m->hx, 0, i) = E2(m->hx, nj, i);
    E2(m->hx, nj + 1, i) = E2(m->hx, 1, i);
  }
  for (int j = 1; j <= nj; j++) {
    E2(m->hy, j, 0) = E2(m->hy, j, ni);
    E2(m->hy, j, ni + 1) = E2(m->hy, j, 1);
  }
  for (int k = 1; k <= kz; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) {
        E3(m->zeta, j, i, k) = md_zeta(m->zitah[k], E2(m->ht, j, i), m->mo_ztop, m->mo_h, m->mo_a0);
        E3(m->fmz, j, i, k) = md_fmz(m->zitah[k], E2(m->ht, j, i), m->mo_ztop, m->mo_h, m->mo_a0);
      }
  for (int k = 1; k <= kz; k++) {
    for (int i = 1; i <= ni; i++) {
      E3(m->fmz, 0, i, k) = E3(m->fmz, nj, i, k);
      E3(m->fmz, nj + 1, i, k) = E3(m->fmz, 1, i, k);
    }
    for (int j = 1; j <= nj; j++) {
      E3(m->fmz, j, 0, k) = E3(m->fmz, j, ni, k);
      E3(m->fmz, j, ni + 1, k) = E3(m->fmz, j, 1, k);
    }
    for (int i = 1; i <= ni; i++) {
      E3(m->zeta, 0, i, k) = E3(m->zeta, nj, i, k);
      E3(m->zeta, nj + 1, i, k) = E3(m->zeta, 1, i, k);
      E3(m->zeta, -1, i, k) = E3(m->zeta, nj - 1, i, k);
      E3(m->zeta, nj + 2, i, k) = E3(m->zeta, 2, i, k);
    }
    for (int j = 1; j <= nj; j++) {
      E3(m->zeta, j, 0, k) = E3(m->zeta, j, ni, k);
      E3(m->zeta, j, ni + 1, k) = E3(m->zeta, j, 1, k);
      E3(m->zeta, j, -1, k) = E3(m->zeta, j, ni - 1, k);
      E3(m->zeta, j, ni + 2, k) = E3(m->zeta, j, 2, k);
    }
  }
  for (int k = 1; k <= kz + 1; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) {
        E3(m->fmzf, j, i, k) = md_fmz(m->zita[k], E2(m->ht, j, i), m->mo_ztop, m->mo_h, m->mo_a0);
        E3(m->zetaf, j, i, k) = md_zeta(m->zita[k], E2(m->ht, j, i), m->mo_ztop, m->mo_h, m->mo_a0);
      }
  for (int k = 1; k <= kz; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++)
        E3(m->dz, j, i, k) = E3(m->zetaf, j, i, k) - E3(m->zetaf, j, i, k + 1);
}

/* ---- fill_atmosphere (nompi/mod_atmosphere.F90:171-235) ---------------- */
static void fill_atmosphere(Moloch *m, const oracle_cfg *c) {
  int nj = m->nj, ni = m->ni, kz = m->kz;
  const double ts = 300.0, qs = 0.01865, ps = 101480.0, tropoh = 15000.0;
  double tvs = ts * (1.0 + EP1 * qs);
  double tvt = tvs - LRATE * tropoh;
  for (long q = 0; q < m->ps.n1 * (m->ps.u2 - m->ps.l2 + 1); q++) m->ps.p[q] = ps;
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++)
      for (int k = 1; k <= kz; k++) {
        if (E3(m->zeta, j, i, k) < tropoh) {
          double zi = E3(m->zeta, j, i, k);
          double xq = -(zi / 7500.0);
          double qi = (qs * exp(-(zi / 4000.0))) * exp(xq * xq);
          E3(m->qv, j, i, k) = qi;
          E3(m->t, j, i, k) = (tvs - LRATE * zi) / (1.0 + qi);
        } else {
          E3(m->qv, j, i, k) = 1.0e-8;
          E3(m->t, j, i, k) = tvt;
        }
        E3(m->qc, j, i, k) = 0.0;
        E3(m->qi, j, i, k) = 0.0;
        E3(m->qr, j, i, k) = 0.0;
        E3(m->qsn, j, i, k) = 0.0;
      }
  int mx = m->nj / 2, my = m->ni / 2;
  /* mr = sqrt((real(jx)/5.0_rkx)**2+(real(iy)/5_rkx)**2)/2.0_rkx : the second
     quotient is default REAL (single precision) because 5_rkx is an integer. */
  double aj = (double)(float)nj / 5.0;
  float bi = (float)ni / 5.0f;
  float bi2 = bi * bi;
  double mr = sqrt(aj * aj + (double)bi2) / 2.0;
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++) {
      float fj = (float)(j - mx), fi = (float)(i - my);
      double md = (double)sqrtf(fj * fj + fi * fi); /* single-precision sqrt */
      if (md < mr) E3(m->t, j, i, kz) = E3(m->t, j, i, kz) + (mr - md) / mr;
    }
  for (long q = 0; q < m->u.n12 * (m->u.u3 - m->u.l3 + 1); q++) m->u.p[q] = c->u0;
  for (long q = 0; q < m->v.n12 * (m->v.u3 - m->v.l3 + 1); q++) m->v.p[q] = c->v0;
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++) {
      double zdelta = E3(m->zeta, j, i, kz) * EGRAV;
      double tv1 = E3(m->t, j, i, kz) * (1.0 + EP1 * E3(m->qv, j, i, kz));
      double tv2 = E3(m->t, j, i, kz - 1) * (1.0 + EP1 * E3(m->qv, j, i, kz - 1));
      double lrt = (tv2 - tv1) / (E3(m->zeta, j, i, kz - 1) - E3(m->zeta, j, i, kz));
      lrt = 0.65 * lrt - 0.35 * LRATE;
      double tv = tv1 - (0.5 * E3(m->zeta, j, i, kz)) * lrt;
      double zz = 1.0 / (RGAS * tv);
      double p = E2(m->ps, j, i) * exp(-(zdelta * zz));
      E3(m->pai, j, i, kz) = pow(p / P00, ROVCP);
    }
  for (int k = kz - 1; k >= 1; k--)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) {
        double tv1 = E3(m->t, j, i, k) * (1.0 + EP1 * E3(m->qv, j, i, k));
        double tv2 = E3(m->t, j, i, k + 1) * (1.0 + EP1 * E3(m->qv, j, i, k + 1));
        double zb = (((2.0 * EGRAV) * m->mo_dzita) / (E3(m->fmzf, j, i, k + 1) * CPD) + tv1) - tv2;
        double zdelta = sqrt(zb * zb + (4.0 * tv2) * tv1);
        E3(m->pai, j, i, k) = -((E3(m->pai, j, i, k + 1) / (2.0 * tv2)) * (zb - zdelta));
      }
  /* seeded theta perturbation on the lowest pert_levels levels (not in the
     reference): t += a*(2u-1)*pai, i.e. a uniform theta offset in [-a, a] K */
  if (c->pert_amp != 0.0) {
    int k0 = kz - c->pert_levels + 1;
    if (k0 < 1) k0 = 1;
    for (int k = k0; k <= kz; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++) {
          unsigned long long idx =
              (unsigned long long)(j - 1) +
              (unsigned long long)nj * ((unsigned long long)(i - 1) + (unsigned long long)ni * (k - 1));
          double d = c->pert_amp * (2.0 * splitmix_u01(c->seed, idx) - 1.0);
          E3(m->t, j, i, k) = E3(m->t, j, i, k) + d * E3(m->pai, j, i, k);
        }
  }
}

/* ---- allocate_moloch / init_moloch (nompi/mod_moloch.F90:183-268) ------ */
static void allocate_all(Moloch *m) {
  int nj = m->nj, ni = m->ni, kz = m->kz;
  /* mod_atmosphere.F90:104-169 */
  m->u = a3(-1, nj + 2, 0, ni + 1, 1, kz);
  m->v = a3(0, nj + 1, -1, ni + 2, 1, kz);
  m->ux = a3(-1, nj + 2, 0, ni + 1, 1, kz);
  m->vx = a3(0, nj + 1, -1, ni + 2, 1, kz);
  m->t = a3(0, nj + 1, 0, ni + 1, 1, kz);
  m->tetav = a3(0, nj + 1, 0, ni + 1, 1, kz);
  m->w = a3(1, nj, 1, ni, 1, kz + 1);
  m->pai = a3(0, nj + 1, 0, ni + 1, 1, kz);
  m->qv = a3(0, nj + 1, 0, ni + 1, 1, kz);
  m->qc = a3(0, nj + 1, 0, ni + 1, 1, kz);
  m->qi = a3(0, nj + 1, 0, ni + 1, 1, kz);
  m->qr = a3(0, nj + 1, 0, ni + 1, 1, kz);
  m->qsn = a3(0, nj + 1, 0, ni + 1, 1, kz);
  m->zeta = a3(-1, nj + 2, -1, ni + 2, 1, kz);
  m->rho = a3(1, nj, 1, ni, 1, kz);
  m->p = a3(1, nj, 1, ni, 1, kz);
  m->tvirt = a3(1, nj, 1, ni, 1, kz);
  m->zetaf = a3(1, nj, 1, ni, 1, kz + 1);
  m->dz = a3(1, nj, 1, ni, 1, kz);
  m->qsat = a3(1, nj, 1, ni, 1, kz);
  m->fmz = a3(0, nj + 1, 0, ni + 1, 1, kz);
  m->fmzf = a3(1, nj, 1, ni, 1, kz + 1);
  m->ht = a2(-1, nj + 2, -1, ni + 2);
  m->xlat = a2(0, nj + 1, 0, ni + 1);
  m->msfx = a2(1, nj, 1, ni);
  m->msfu = a2(0, nj + 1, 1, ni);
  m->msfv = a2(1, nj, 0, ni + 1);
  m->hx = a2(0, nj + 1, 1, ni);
  m->hy = a2(1, nj, 0, ni + 1);
  m->ulat = a2(1, nj, 1, ni);
  m->vlat = a2(1, nj, 1, ni);
  m->ps = a2(0, nj + 1, 0, ni + 1);
  /* mod_moloch.F90:183-217 */
  m->gzitak = (double *)calloc(kz + 2, sizeof(double));
  m->gzitakh = (double *)calloc(kz + 2, sizeof(double));
  m->xknu = (double *)calloc(kz + 2, sizeof(double));
  m->p2d = a2(1, nj, 1, ni);
  m->deltaw = a3(0, nj + 1, 0, ni + 1, 1, kz + 1);
  m->s = a3(1, nj, 1, ni, 1, kz + 1);
  m->wx = a3(1, nj, 1, ni, 1, kz);
  m->zdiv2 = a3(0, nj + 1, 0, ni + 1, 1, kz);
  m->wz = a3(1, nj, -1, ni + 2, 1, kz);
  m->p0 = a3(-1, nj + 2, 1, ni, 1, kz);
  m->mx2 = a2(1, nj, 1, ni);
  m->rmu = a2(0, nj + 1, 1, ni);
  m->rmv = a2(1, nj, 0, ni + 1);
  m->coru = a2(1, nj, 1, ni);
  m->corv = a2(1, nj, 1, ni);
  m->ud = a3(0, nj + 1, 0, ni + 1, 1, kz);
  m->vd = a3(0, nj + 1, 0, ni + 1, 1, kz);
  m->qwltot = a3(1, nj, 1, ni, 1, kz);
  m->qwitot = a3(1, nj, 1, ni, 1, kz);
  m->pf = a3(1, nj, 1, ni, 1, kz);
  m->tf = a3(1, nj, 1, ni, 1, kz);
  for (int k = 1; k <= kz; k++) /* :207-210 */
    m->xknu[k] = XDAMP + (1.0 - XDAMP) * sin((0.5 * MATHPI) * (1.0 - (double)(k - 1) / (double)(kz - 1)));
  /* automatic arrays */
  m->wwkw = a3(1, nj, 1, ni, 2, kz + 1);
  m->wfw = a3(1, nj, 1, ni, 1, kz + 1);
  m->zpby = a3(1, nj, 1, ni + 1, 1, kz);
  m->zpbw = a3(1, nj + 1, 1, ni, 1, kz);
}

static void init_moloch(Moloch *m) { /* :219-268 */
  int nj = m->nj, ni = m->ni, kz = m->kz;
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++) {
      E2(m->coru, j, i) = EOMEG2 * sin(E2(m->ulat, j, i) * DEGRAD);
      E2(m->corv, j, i) = EOMEG2 * sin(E2(m->vlat, j, i) * DEGRAD);
      E2(m->mx2, j, i) = E2(m->msfx, j, i) * E2(m->msfx, j, i);
    }
  for (int i = 1; i <= ni; i++)
    for (int j = 0; j <= nj + 1; j++) E2(m->rmu, j, i) = 1.0 / E2(m->msfu, j, i);
  for (int i = 0; i <= ni + 1; i++)
    for (int j = 1; j <= nj; j++) E2(m->rmv, j, i) = 1.0 / E2(m->msfv, j, i);
  for (int k = 1; k <= kz + 1; k++) m->gzitak[k] = gzita(m->zita[k], m->mo_ztop, m->mo_a0);
  for (int k = 1; k <= kz; k++) m->gzitakh[k] = gzita(m->zitah[k], m->mo_ztop, m->mo_a0);
  m->dzita = m->mo_dzita;
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++) E3(m->w, j, i, 1) = 0.0;
  m->jmin = 1 - 2;
  m->jmax = nj + 2;
  m->imin = 1 - 2;
  m->imax = ni + 2;
}

/* ---- halo fills (inline array-section copies in the reference) --------- */
/* width-1 fill of a (0:nj+1, 0:ni+1) array, no corners (e.g. :708-711) */
static void halo1(Moloch *m, A3 *a, int k1, int k2) {
  int nj = m->nj, ni = m->ni;
#pragma omp parallel for
  for (int k = k1; k <= k2; k++) {
    for (int i = 1; i <= ni; i++) {
      E3(*a, 0, i, k) = E3(*a, nj, i, k);
      E3(*a, nj + 1, i, k) = E3(*a, 1, i, k);
    }
    for (int j = 1; j <= nj; j++) {
      E3(*a, j, 0, k) = E3(*a, j, ni, k);
      E3(*a, j, ni + 1, k) = E3(*a, j, 1, k);
    }
  }
}

/* ---- filters :423-481 -------------------------------------------------- */
static void lap_filter(Moloch *m, A3 *a, const double *coef_k, double coef) {
  int nj = m->nj, ni = m->ni, kz = m->kz;
  halo1(m, a, 1, kz);
  for (int k = 1; k <= kz; k++) {
    double c = coef_k ? (m->mo_anu2 * coef_k[k]) : coef;
#pragma omp parallel for
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++)
        E2(m->p2d, j, i) = 0.125 * (((E3(*a, j - 1, i, k) + E3(*a, j + 1, i, k)) + E3(*a, j, i - 1, k)) +
                                    E3(*a, j, i + 1, k)) -
                           0.5 * E3(*a, j, i, k);
#pragma omp parallel for
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) E3(*a, j, i, k) = E3(*a, j, i, k) + c * E2(m->p2d, j, i);
  }
}
/* divergence_filter: zdiv2 += mo_anu2*xknu(k)*p2d ; filtpai/filttheta: += nupaitq*p2d */
static void divergence_filter(Moloch *m) { lap_filter(m, &m->zdiv2, m->xknu, 0.0); }
static void filtpai(Moloch *m) { lap_filter(m, &m->pai, NULL, NUPAITQ); }
static void filttheta(Moloch *m) { lap_filter(m, &m->tetav, NULL, NUPAITQ); }

/* ---- divdamp :853-895 -------------------------------------------------- */
static void divdamp(Moloch *m, double dts) {
  int nj = m->nj, ni = m->ni, kz = m->kz;
  halo1(m, &m->zdiv2, 1, kz);
  double ddamp = 0.125 * (m->dx / dts);
#pragma omp parallel for
  for (int k = 1; k <= kz; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) {
        E3(m->u, j, i, k) = E3(m->u, j, i, k) + ((m->xknu[k] * ddamp) * E2(m->msfu, j, i)) *
                                                    (E3(m->zdiv2, j, i, k) - E3(m->zdiv2, j - 1, i, k));
      }
#pragma omp parallel for
  for (int k = 1; k <= kz; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) {
        if (m->lrotllr)
          E3(m->v, j, i, k) = E3(m->v, j, i, k) +
                              (m->xknu[k] * ddamp) * (E3(m->zdiv2, j, i, k) - E3(m->zdiv2, j, i - 1, k));
        else
          E3(m->v, j, i, k) = E3(m->v, j, i, k) + ((m->xknu[k] * ddamp) * E2(m->msfv, j, i)) *
                                                      (E3(m->zdiv2, j, i, k) - E3(m->zdiv2, j, i - 1, k));
      }
  double ddamp2 = (XDAMP * 0.015625) / dts;
  for (int k = 1; k <= kz; k++) {
#pragma omp parallel for
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++)
        E2(m->p2d, j, i) = 0.125 * (((E3(m->zdiv2, j - 1, i, k) + E3(m->zdiv2, j + 1, i, k)) +
                                     E3(m->zdiv2, j, i - 1, k)) +
                                    E3(m->zdiv2, j, i + 1, k)) -
                           0.5 * E3(m->zdiv2, j, i, k);
#pragma omp parallel for
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) E3(m->zdiv2, j, i, k) = E3(m->zdiv2, j, i, k) + ddamp2 * E2(m->p2d, j, i);
  }
}

/* ---- sound :483-851 ---------------------------------------------------- */
static void sound(Moloch *m, double dts) {
  int nj = m->nj, ni = m->ni, kz = m->kz;
  double dtrdx = dts / m->dx, dtrdy = dts / m->dx, dtrdz = dts / m->dzita;
  double zcs2 = (dtrdz * dtrdz) * RDRCV;
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++) E3(m->wwkw, j, i, kz + 1) = 0.0;
  /* (do_fulleq is .true.: no tetav halo fill here, :505-510) */
  for (int nsound = 1; nsound <= m->mo_nsound; nsound++) {
    /* u, v halos incl. corners :514-529 */
    for (int k = 1; k <= kz; k++) {
      for (int i = 1; i <= ni; i++) {
        E3(m->u, 0, i, k) = E3(m->u, nj, i, k);
        E3(m->u, nj + 1, i, k) = E3(m->u, 1, i, k);
      }
      for (int j = 1; j <= nj; j++) {
        E3(m->u, j, 0, k) = E3(m->u, j, ni, k);
        E3(m->u, j, ni + 1, k) = E3(m->u, j, 1, k);
      }
      E3(m->u, nj + 1, ni + 1, k) = E3(m->u, 1, 1, k);
      E3(m->u, 0, ni + 1, k) = E3(m->u, nj, 1, k);
      E3(m->u, 0, 0, k) = E3(m->u, nj, ni, k);
      E3(m->u, nj + 1, 0, k) = E3(m->u, 1, ni, k);
      for (int i = 1; i <= ni; i++) {
        E3(m->v, 0, i, k) = E3(m->v, nj, i, k);
        E3(m->v, nj + 1, i, k) = E3(m->v, 1, i, k);
      }
      for (int j = 1; j <= nj; j++) {
        E3(m->v, j, 0, k) = E3(m->v, j, ni, k);
        E3(m->v, j, ni + 1, k) = E3(m->v, j, 1, k);
      }
      E3(m->v, nj + 1, ni + 1, k) = E3(m->v, 1, 1, k);
      E3(m->v, 0, ni + 1, k) = E3(m->v, nj, 1, k);
      E3(m->v, 0, 0, k) = E3(m->v, nj, ni, k);
      E3(m->v, nj + 1, 0, k) = E3(m->v, 1, ni, k);
    }
    /* surface w and s(kz+1) :536-549 */
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) {
        double zuh = E3(m->u, j, i, kz) * E2(m->hx, j, i) + E3(m->u, j + 1, i, kz) * E2(m->hx, j + 1, i);
        double zvh = E3(m->v, j, i, kz) * E2(m->hy, j, i) + E3(m->v, j, i + 1, kz) * E2(m->hy, j, i + 1);
        E3(m->w, j, i, kz + 1) = 0.5 * (zuh + zvh);
      }
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) E3(m->s, j, i, kz + 1) = -E3(m->w, j, i, kz + 1);
    /* Equation 10 :557-570 */
#pragma omp parallel for
    for (int k = 2; k <= kz; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++) {
          double zuh = (E3(m->u, j, i, k) + E3(m->u, j, i, k - 1)) * E2(m->hx, j, i) +
                       (E3(m->u, j + 1, i, k) + E3(m->u, j + 1, i, k - 1)) * E2(m->hx, j + 1, i);
          double zvh = (E3(m->v, j, i, k) + E3(m->v, j, i, k - 1)) * E2(m->hy, j, i) +
                       (E3(m->v, j, i + 1, k) + E3(m->v, j, i + 1, k - 1)) * E2(m->hy, j, i + 1);
          E3(m->s, j, i, k) = -((0.25 * (zuh + zvh)) * m->gzitak[k]);
        }
    /* Equation 16 :575-621 */
#pragma omp parallel for
    for (int k = 1; k <= kz; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++) {
          double f = E3(m->fmz, j, i, k);
          double zrfmzum = 2.0 / (f + E3(m->fmz, j - 1, i, k));
          double zrfmzvm = 2.0 / (f + E3(m->fmz, j, i - 1, k));
          double zrfmzup = 2.0 / (f + E3(m->fmz, j + 1, i, k));
          double zrfmzvp = 2.0 / (f + E3(m->fmz, j, i + 1, k));
          if (m->lrotllr) {
            double zum = (dtrdx * E3(m->u, j, i, k)) * zrfmzum;
            double zup = (dtrdx * E3(m->u, j + 1, i, k)) * zrfmzup;
            double zvm = ((dtrdy * E3(m->v, j, i, k)) * zrfmzvm) * E2(m->rmv, j, i);
            double zvp = ((dtrdy * E3(m->v, j, i + 1, k)) * zrfmzvp) * E2(m->rmv, j, i + 1);
            E3(m->zdiv2, j, i, k) = (f * E2(m->msfx, j, i)) * ((zup - zum) + (zvp - zvm));
          } else {
            double zum = ((dtrdx * E3(m->u, j, i, k)) * E2(m->rmu, j, i)) * zrfmzum;
            double zup = ((dtrdx * E3(m->u, j + 1, i, k)) * E2(m->rmu, j + 1, i)) * zrfmzup;
            double zvm = ((dtrdy * E3(m->v, j, i, k)) * E2(m->rmv, j, i)) * zrfmzvm;
            double zvp = ((dtrdy * E3(m->v, j, i + 1, k)) * E2(m->rmv, j, i + 1)) * zrfmzvp;
            E3(m->zdiv2, j, i, k) = (E2(m->mx2, j, i) * f) * ((zup - zum) + (zvp - zvm));
          }
        }
    divdamp(m, dts); /* do_divdamp */
#pragma omp parallel for
    for (int k = 1; k <= kz; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++)
          E3(m->zdiv2, j, i, k) = E3(m->zdiv2, j, i, k) +
                                  (E3(m->fmz, j, i, k) * dtrdz) * (E3(m->s, j, i, k) - E3(m->s, j, i, k + 1));
    /* implicit w, Thomas down-sweep :634-678 */
    for (int k = kz; k >= 2; k--) {
#pragma omp parallel for
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++) {
          double wk = E3(m->w, j, i, k);
          double fz = E3(m->fmzf, j, i, k);
          E3(m->deltaw, j, i, k) = -wk;
          double zrom1w = ((0.5 * CPD) * fz) * (E3(m->tetav, j, i, k - 1) + E3(m->tetav, j, i, k));
          zrom1w = zrom1w - (((((CPD * wk) * fz) * fz) * (double)nsound) * dtrdz) *
                                (E3(m->tetav, j, i, k - 1) - E3(m->tetav, j, i, k));
          if (E3(m->qv, j, i, k) > 0.96 * E3(m->qsat, j, i, k) && wk > 0.1) {
            double zqs = 0.5 * (E3(m->qsat, j, i, k) + E3(m->qsat, j, i, k - 1));
            double tkm = E3(m->t, j, i, k - 1);
            double zdth = ((((((EGRAV * wk) * (double)(nsound - 1)) * dts) * WLHV) * WLHV) * zqs) /
                          ((((CPD * E3(m->pai, j, i, k - 1)) * RWAT) * tkm) * tkm);
            zrom1w = zrom1w + zdth * fz;
          }
          double pkm = E3(m->pai, j, i, k - 1), pk = E3(m->pai, j, i, k);
          double zwexpl = (wk - (zrom1w * dtrdz) * (pkm - pk)) - EGRAV * dts;
          zwexpl = zwexpl + ((RDRCV * zrom1w) * dtrdz) *
                                (pkm * E3(m->zdiv2, j, i, k - 1) - pk * E3(m->zdiv2, j, i, k));
          double zu = ((zcs2 * E3(m->fmz, j, i, k - 1)) * zrom1w) * pkm + m->ffilt[k];
          double zd = ((zcs2 * E3(m->fmz, j, i, k)) * zrom1w) * pk + m->ffilt[k];
          double zrapp = 1.0 / (((1.0 + zd) + zu) - zd * E3(m->wwkw, j, i, k + 1));
          E3(m->w, j, i, k) = zrapp * (zwexpl + zd * E3(m->w, j, i, k + 1));
          E3(m->wwkw, j, i, k) = zrapp * zu;
        }
    }
    /* back-substitution :681-686 */
    for (int k = 2; k <= kz; k++) {
#pragma omp parallel for
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++) {
          E3(m->w, j, i, k) = E3(m->w, j, i, k) + E3(m->wwkw, j, i, k) * E3(m->w, j, i, k - 1);
          E3(m->deltaw, j, i, k) = E3(m->deltaw, j, i, k) + E3(m->w, j, i, k);
        }
    }
    /* new Exner function :690-712 */
#pragma omp parallel for
    for (int k = 1; k <= kz; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++)
          E3(m->zdiv2, j, i, k) = E3(m->zdiv2, j, i, k) +
                                  (dtrdz * E3(m->fmz, j, i, k)) * (E3(m->w, j, i, k) - E3(m->w, j, i, k + 1));
#pragma omp parallel for
    for (int k = 1; k <= kz; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++) {
          double qv = E3(m->qv, j, i, k), qc = E3(m->qc, j, i, k);
          E3(m->zdiv2, j, i, k) =
              (E3(m->zdiv2, j, i, k) * ((1.0 + 0.86 * qv) + 3.2 * qc)) / ((1.0 + 0.96 * qv) + 4.8 * qc);
          E3(m->tetav, j, i, k) =
              E3(m->tetav, j, i, k) *
              (1.0 + (RDRCV * E3(m->zdiv2, j, i, k)) *
                         ((0.25 * qv + 4.2 * E3(m->qwltot, j, i, k)) + 2.1 * E3(m->qwitot, j, i, k)));
        }
    halo1(m, &m->tetav, 1, kz);
    if (m->divfilter) divergence_filter(m);
    /* nompi order: pai and deltaw halos BEFORE the pai update (:716-728) */
    halo1(m, &m->pai, 1, kz);
    halo1(m, &m->deltaw, 1, kz + 1);
#pragma omp parallel for
    for (int k = 1; k <= kz; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++)
          E3(m->pai, j, i, k) = E3(m->pai, j, i, k) * (1.0 - RDRCV * E3(m->zdiv2, j, i, k));
    /* ud, vd copies including the halo ring :730-735 */
#pragma omp parallel for
    for (int k = 1; k <= kz; k++)
      for (int i = 0; i <= ni + 1; i++)
        for (int j = 0; j <= nj + 1; j++) {
          E3(m->ud, j, i, k) = E3(m->u, j, i, k);
          E3(m->vd, j, i, k) = E3(m->v, j, i, k);
        }
    /* Equations 17, 18 :737-837 */
#pragma omp parallel for
    for (int k = 1; k <= kz; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++) {
          double zcx = dtrdx * E2(m->msfu, j, i);
          double zfz = EGRAV * dts + 0.25 * (((E3(m->deltaw, j - 1, i, k) + E3(m->deltaw, j - 1, i, k + 1)) +
                                              E3(m->deltaw, j, i, k)) +
                                             E3(m->deltaw, j, i, k + 1));
          double zrom1u = (0.5 * CPD) * (E3(m->tetav, j - 1, i, k) + E3(m->tetav, j, i, k));
          double zcor1u = ((E2(m->coru, j, i) * dts) * 0.25) *
                          (((E3(m->vd, j, i, k) + E3(m->vd, j - 1, i, k)) + E3(m->vd, j - 1, i + 1, k)) +
                           E3(m->vd, j, i + 1, k));
          E3(m->u, j, i, k) = ((E3(m->u, j, i, k) + zcor1u) - (zfz * E2(m->hx, j, i)) * m->gzitakh[k]) -
                              (zcx * zrom1u) * (E3(m->pai, j, i, k) - E3(m->pai, j - 1, i, k));
        }
#pragma omp parallel for
    for (int k = 1; k <= kz; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++) {
          double zcy = m->lrotllr ? dtrdy : dtrdy * E2(m->msfv, j, i);
          double zfz = EGRAV * dts + 0.25 * (((E3(m->deltaw, j, i - 1, k) + E3(m->deltaw, j, i - 1, k + 1)) +
                                              E3(m->deltaw, j, i, k)) +
                                             E3(m->deltaw, j, i, k + 1));
          double zrom1v = (0.5 * CPD) * (E3(m->tetav, j, i - 1, k) + E3(m->tetav, j, i, k));
          double zcor1v = ((E2(m->corv, j, i) * dts) * 0.25) *
                          (((E3(m->ud, j, i, k) + E3(m->ud, j, i - 1, k)) + E3(m->ud, j + 1, i, k)) +
                           E3(m->ud, j + 1, i - 1, k));
          E3(m->v, j, i, k) = ((E3(m->v, j, i, k) - zcor1v) - (zfz * E2(m->hy, j, i)) * m->gzitakh[k]) -
                              (zcy * zrom1v) * (E3(m->pai, j, i, k) - E3(m->pai, j, i - 1, k));
        }
  } /* sound loop */
  /* complete Equation 10 :843-849 */
#pragma omp parallel for
  for (int k = 2; k <= kz; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++)
        E3(m->s, j, i, k) = (E3(m->w, j, i, k) + E3(m->s, j, i, k)) * E3(m->fmzf, j, i, k);
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++) {
      E3(m->s, j, i, 1) = 0.0;
      E3(m->s, j, i, kz + 1) = 0.0;
    }
}

/* ---- wafone :929-1311 -------------------------------------------------- */
static void wafone(Moloch *m, A3 *ppa, double dta) {
  int nj = m->nj, ni = m->ni, kz = m->kz;
  A3 pp = *ppa;
  double dtrdx = dta / m->dx, dtrdy = dta / m->dx, dtrdz = dta / m->dzita;
  dtrdz = 0.5 * dtrdz; /* do_vadvtwice */
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++) {
      E3(m->wfw, j, i, 1) = 0.0;
      E3(m->wfw, j, i, kz + 1) = 0.0;
    }
  for (int pass = 0; pass < 2; pass++) {
    A3 src = pass == 0 ? pp : m->wz; /* first pass reads pp, second wz */
#pragma omp parallel for
    for (int k = 1; k <= kz - 1; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++) {
          double zamu = E3(m->s, j, i, k + 1) * dtrdz, is;
          int k1, k1p1;
          if (zamu >= 0.0) {
            is = 1.0; k1 = k + 1; k1p1 = k1 + 1;
            if (k1p1 > kz) k1p1 = kz;
          } else {
            is = -1.0; k1 = k - 1; k1p1 = k;
            if (k1 < 1) k1 = 1;
          }
          double zzden = E3(src, j, i, k) - E3(src, j, i, k + 1);
          zzden = copysign(fmax2(fabs(zzden), MINDEN), zzden);
          double r = (E3(src, j, i, k1) - E3(src, j, i, k1p1)) / zzden;
          double b = superbee(r);
          double zphi = (is + zamu * b) - is * b;
          E3(m->wfw, j, i, k + 1) = (0.5 * E3(m->s, j, i, k + 1)) *
                                    ((1.0 + zphi) * E3(src, j, i, k + 1) + (1.0 - zphi) * E3(src, j, i, k));
        }
#pragma omp parallel for
    for (int k = 1; k <= kz; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++) {
          double zrfmu = (dtrdz * E3(m->fmz, j, i, k)) / E3(m->fmzf, j, i, k);
          double zrfmd = (dtrdz * E3(m->fmz, j, i, k)) / E3(m->fmzf, j, i, k + 1);
          double c = E3(src, j, i, k);
          double zdv = (E3(m->s, j, i, k) * zrfmu - E3(m->s, j, i, k + 1) * zrfmd) * c;
          E3(m->wz, j, i, k) = ((c - E3(m->wfw, j, i, k) * zrfmu) + E3(m->wfw, j, i, k + 1) * zrfmd) + zdv;
        }
  }
  /* wz halo in i, width 2 :1075-1078 */
  for (int k = 1; k <= kz; k++)
    for (int j = 1; j <= nj; j++) {
      E3(m->wz, j, 0, k) = E3(m->wz, j, ni, k);
      E3(m->wz, j, ni + 1, k) = E3(m->wz, j, 1, k);
      E3(m->wz, j, -1, k) = E3(m->wz, j, ni - 1, k);
      E3(m->wz, j, ni + 2, k) = E3(m->wz, j, 2, k);
    }
  /* meridional fluxes :1087-1111 (ROTLLR) / :1197-1221 */
#pragma omp parallel for
  for (int k = 1; k <= kz; k++)
    for (int i = 1; i <= ni + 1; i++)
      for (int j = 1; j <= nj; j++) {
        double vv = E3(m->v, j, i, k), zamu, is;
        int ih, ihm1;
        if (m->lrotllr)
          zamu = vv * dtrdy;
        else
          zamu = (vv * E2(m->rmv, j, i)) * dtrdy;
        if (zamu > 0.0) {
          is = 1.0; ih = i - 1;
        } else {
          is = -1.0; ih = i + 1 < m->imax ? i + 1 : m->imax;
        }
        ihm1 = ih - 1 > m->imin ? ih - 1 : m->imin;
        double zzden = E3(m->wz, j, i, k) - E3(m->wz, j, i - 1, k);
        zzden = copysign(fmax2(fabs(zzden), MINDEN), zzden);
        double r = (E3(m->wz, j, ih, k) - E3(m->wz, j, ihm1, k)) / zzden;
        double b = superbee(r);
        double zphi = (is + zamu * b) - is * b;
        double fl = (1.0 + zphi) * E3(m->wz, j, i - 1, k) + (1.0 - zphi) * E3(m->wz, j, i, k);
        if (m->lrotllr)
          E3(m->zpby, j, i, k) = (0.5 * vv) * fl;
        else
          E3(m->zpby, j, i, k) = ((0.5 * vv) * E2(m->rmv, j, i)) * fl;
      }
#pragma omp parallel for
  for (int k = 1; k <= kz; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) {
        double f = E3(m->fmz, j, i, k);
        if (m->lrotllr) {
          double zhxvtn = (dtrdy * E2(m->rmv, j, i + 1)) * E2(m->msfx, j, i);
          double zhxvts = (dtrdy * E2(m->rmv, j, i)) * E2(m->msfx, j, i);
          double zrfmn = ((zhxvtn * 2.0) * f) / (f + E3(m->fmz, j, i + 1, k));
          double zrfms = ((zhxvts * 2.0) * f) / (f + E3(m->fmz, j, i - 1, k));
          double zdv = (E3(m->v, j, i + 1, k) * zrfmn - E3(m->v, j, i, k) * zrfms) * E3(pp, j, i, k);
          E3(m->p0, j, i, k) = ((E3(m->wz, j, i, k) + E3(m->zpby, j, i, k) * zrfms) -
                                E3(m->zpby, j, i + 1, k) * zrfmn) +
                               zdv;
        } else {
          double zrfmn = ((dtrdy * 2.0) * f) / (f + E3(m->fmz, j, i + 1, k));
          double zrfms = ((dtrdy * 2.0) * f) / (f + E3(m->fmz, j, i - 1, k));
          double zdv = ((E3(m->v, j, i + 1, k) * E2(m->rmv, j, i + 1)) * zrfmn -
                        (E3(m->v, j, i, k) * E2(m->rmv, j, i)) * zrfms) *
                       E3(pp, j, i, k);
          E3(m->p0, j, i, k) =
              E3(m->wz, j, i, k) +
              E2(m->mx2, j, i) * (((E3(m->zpby, j, i, k) * zrfms) - E3(m->zpby, j, i + 1, k) * zrfmn) + zdv);
        }
      }
  /* p0 halo in j, width 2 :1133-1136 */
  for (int k = 1; k <= kz; k++)
    for (int i = 1; i <= ni; i++) {
      E3(m->p0, 0, i, k) = E3(m->p0, nj, i, k);
      E3(m->p0, nj + 1, i, k) = E3(m->p0, 1, i, k);
      E3(m->p0, -1, i, k) = E3(m->p0, nj - 1, i, k);
      E3(m->p0, nj + 2, i, k) = E3(m->p0, 2, i, k);
    }
  /* zonal fluxes :1144-1168 */
#pragma omp parallel for
  for (int k = 1; k <= kz; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj + 1; j++) {
        double uu = E3(m->u, j, i, k), zamu, is;
        int jh, jhm1;
        if (m->lrotllr)
          zamu = (uu * E2(m->msfu, j, i)) * dtrdx;
        else
          zamu = (uu * E2(m->rmu, j, i)) * dtrdx;
        if (zamu > 0.0) {
          is = 1.0; jh = j - 1;
        } else {
          is = -1.0; jh = j + 1 < m->jmax ? j + 1 : m->jmax;
        }
        jhm1 = jh - 1 > m->jmin ? jh - 1 : m->jmin;
        double zzden = E3(m->p0, j, i, k) - E3(m->p0, j - 1, i, k);
        zzden = copysign(fmax2(fabs(zzden), MINDEN), zzden);
        double r = (E3(m->p0, jh, i, k) - E3(m->p0, jhm1, i, k)) / zzden;
        double b = superbee(r);
        double zphi = (is + zamu * b) - is * b;
        double fl = (1.0 + zphi) * E3(m->p0, j - 1, i, k) + (1.0 - zphi) * E3(m->p0, j, i, k);
        if (m->lrotllr)
          E3(m->zpbw, j, i, k) = (0.5 * uu) * fl;
        else
          E3(m->zpbw, j, i, k) = ((0.5 * uu) * E2(m->rmu, j, i)) * fl;
      }
#pragma omp parallel for
  for (int k = 1; k <= kz; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) {
        double f = E3(m->fmz, j, i, k);
        if (m->lrotllr) {
          double zcostx = dtrdx * E2(m->msfu, j, i);
          double zrfme = ((zcostx * 2.0) * f) / (f + E3(m->fmz, j + 1, i, k));
          double zrfmw = ((zcostx * 2.0) * f) / (f + E3(m->fmz, j - 1, i, k));
          double zdv = (E3(m->u, j + 1, i, k) * zrfme - E3(m->u, j, i, k) * zrfmw) * E3(pp, j, i, k);
          E3(pp, j, i, k) =
              ((E3(m->p0, j, i, k) + E3(m->zpbw, j, i, k) * zrfmw) - E3(m->zpbw, j + 1, i, k) * zrfme) + zdv;
        } else {
          double zrfme = ((dtrdx * 2.0) * f) / (f + E3(m->fmz, j + 1, i, k));
          double zrfmw = ((dtrdx * 2.0) * f) / (f + E3(m->fmz, j - 1, i, k));
          double zdv = ((E3(m->u, j + 1, i, k) * E2(m->rmu, j + 1, i)) * zrfme -
                        (E3(m->u, j, i, k) * E2(m->rmu, j, i)) * zrfmw) *
                       E3(pp, j, i, k);
          E3(pp, j, i, k) =
              E3(m->p0, j, i, k) +
              E2(m->mx2, j, i) * (((E3(m->zpbw, j, i, k) * zrfmw) - E3(m->zpbw, j + 1, i, k) * zrfme) + zdv);
        }
      }
}

/* ---- staggering :1327-1417 --------------------------------------------- */
static void uvstagtox(Moloch *m) {
  int nj = m->nj, ni = m->ni, kz = m->kz;
  for (int k = 1; k <= kz; k++) {
    for (int i = 1; i <= ni; i++) {
      E3(m->u, 0, i, k) = E3(m->u, nj, i, k);
      E3(m->u, nj + 1, i, k) = E3(m->u, 1, i, k);
      E3(m->u, -1, i, k) = E3(m->u, nj - 1, i, k);
      E3(m->u, nj + 2, i, k) = E3(m->u, 2, i, k);
    }
    for (int j = 1; j <= nj; j++) {
      E3(m->v, j, 0, k) = E3(m->v, j, ni, k);
      E3(m->v, j, ni + 1, k) = E3(m->v, j, 1, k);
      E3(m->v, j, -1, k) = E3(m->v, j, ni - 1, k);
      E3(m->v, j, ni + 2, k) = E3(m->v, j, 2, k);
    }
  }
#pragma omp parallel for
  for (int k = 1; k <= kz; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) {
        E3(m->ux, j, i, k) = 0.5625 * (E3(m->u, j + 1, i, k) + E3(m->u, j, i, k)) -
                             0.0625 * (E3(m->u, j + 2, i, k) + E3(m->u, j - 1, i, k));
        E3(m->vx, j, i, k) = 0.5625 * (E3(m->v, j, i + 1, k) + E3(m->v, j, i, k)) -
                             0.0625 * (E3(m->v, j, i + 2, k) + E3(m->v, j, i - 1, k));
      }
}
static void wstagtox(Moloch *m) {
  int nj = m->nj, ni = m->ni, kz = m->kz;
#pragma omp parallel for
  for (int k = 2; k <= kz - 1; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++)
        E3(m->wx, j, i, k) = 0.5625 * (E3(m->w, j, i, k + 1) + E3(m->w, j, i, k)) -
                             0.0625 * (E3(m->w, j, i, k + 2) + E3(m->w, j, i, k - 1));
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++) {
      E3(m->wx, j, i, 1) = 0.5 * (E3(m->w, j, i, 2) + E3(m->w, j, i, 1));
      E3(m->wx, j, i, kz) = 0.5 * (E3(m->w, j, i, kz + 1) + E3(m->w, j, i, kz));
    }
}
static void xtowstag(Moloch *m) {
  int nj = m->nj, ni = m->ni, kz = m->kz;
#pragma omp parallel for
  for (int k = 3; k <= kz - 1; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++)
        E3(m->w, j, i, k) = 0.5625 * (E3(m->wx, j, i, k) + E3(m->wx, j, i, k - 1)) -
                            0.0625 * (E3(m->wx, j, i, k + 1) + E3(m->wx, j, i, k - 2));
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++) {
      E3(m->w, j, i, 2) = 0.5 * (E3(m->wx, j, i, 2) + E3(m->wx, j, i, 1));
      E3(m->w, j, i, kz) = 0.5 * (E3(m->wx, j, i, kz) + E3(m->wx, j, i, kz - 1));
    }
}
static void xtouvstag(Moloch *m) {
  int nj = m->nj, ni = m->ni, kz = m->kz;
  for (int k = 1; k <= kz; k++) {
    for (int i = 1; i <= ni; i++) {
      E3(m->ux, 0, i, k) = E3(m->ux, nj, i, k);
      E3(m->ux, nj + 1, i, k) = E3(m->ux, 1, i, k);
      E3(m->ux, -1, i, k) = E3(m->ux, nj - 1, i, k);
      E3(m->ux, nj + 2, i, k) = E3(m->ux, 2, i, k);
    }
    for (int j = 1; j <= nj; j++) {
      E3(m->vx, j, 0, k) = E3(m->vx, j, ni, k);
      E3(m->vx, j, ni + 1, k) = E3(m->vx, j, 1, k);
      E3(m->vx, j, -1, k) = E3(m->vx, j, ni - 1, k);
      E3(m->vx, j, ni + 2, k) = E3(m->vx, j, 2, k);
    }
  }
#pragma omp parallel for
  for (int k = 1; k <= kz; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) {
        E3(m->u, j, i, k) = 0.5625 * (E3(m->ux, j, i, k) + E3(m->ux, j - 1, i, k)) -
                            0.0625 * (E3(m->ux, j + 1, i, k) + E3(m->ux, j - 2, i, k));
        E3(m->v, j, i, k) = 0.5625 * (E3(m->vx, j, i, k) + E3(m->vx, j, i - 1, k)) -
                            0.0625 * (E3(m->vx, j, i + 1, k) + E3(m->vx, j, i - 2, k));
      }
}

/* ---- advection :897-927 ------------------------------------------------ */
static void advection(Moloch *m, double dta) {
  uvstagtox(m);
  wstagtox(m);
  wafone(m, &m->tetav, dta);
  wafone(m, &m->pai, dta);
  wafone(m, &m->ux, dta);
  wafone(m, &m->vx, dta);
  wafone(m, &m->wx, dta);
  wafone(m, &m->qv, dta);
  wafone(m, &m->qc, dta);
  wafone(m, &m->qi, dta);
  wafone(m, &m->qr, dta);
  wafone(m, &m->qsn, dta);
  xtouvstag(m);
  xtowstag(m);
}

static void reset_tendencies(Moloch *m) { /* :1313-1325 */
  memset(m->s.p, 0, sizeof(double) * m->s.n12 * (m->s.u3 - m->s.l3 + 1));
  memset(m->zdiv2.p, 0, sizeof(double) * m->zdiv2.n12 * (m->zdiv2.u3 - m->zdiv2.l3 + 1));
  memset(m->deltaw.p, 0, sizeof(double) * m->deltaw.n12 * (m->deltaw.u3 - m->deltaw.l3 + 1));
}

/* ---- moloch :272-421 --------------------------------------------------- */
static void prediag(Moloch *m) { /* :289-323 */
  int nj = m->nj, ni = m->ni, kz = m->kz;
#pragma omp parallel for
  for (int k = 1; k <= kz; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) {
        E3(m->p, j, i, k) = pow(E3(m->pai, j, i, k), CPOVR) * P00;
        E3(m->qsat, j, i, k) = pfwsat(E3(m->t, j, i, k), E3(m->p, j, i, k));
        E3(m->tvirt, j, i, k) = E3(m->t, j, i, k) * ((((1.0 + EP1 * E3(m->qv, j, i, k)) - E3(m->qc, j, i, k)) -
                                                      E3(m->qi, j, i, k)) -
                                                     E3(m->qr, j, i, k) - E3(m->qsn, j, i, k));
        E3(m->qwltot, j, i, k) = E3(m->qc, j, i, k) + E3(m->qr, j, i, k);
        E3(m->qwitot, j, i, k) = E3(m->qi, j, i, k) + E3(m->qsn, j, i, k);
        E3(m->tetav, j, i, k) = E3(m->tvirt, j, i, k) / E3(m->pai, j, i, k);
        if (m->filterpai) E3(m->pf, j, i, k) = E3(m->pai, j, i, k);
        if (m->filtertheta) E3(m->tf, j, i, k) = E3(m->tetav, j, i, k);
      }
}

static void postdiag(Moloch *m) { /* :333-391 */
  int nj = m->nj, ni = m->ni, kz = m->kz;
  if (m->filterpai) {
    for (int k = 1; k <= kz; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++) E3(m->pai, j, i, k) = E3(m->pai, j, i, k) - E3(m->pf, j, i, k);
    filtpai(m);
    for (int k = 1; k <= kz; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++) E3(m->pai, j, i, k) = E3(m->pai, j, i, k) + E3(m->pf, j, i, k);
  }
  if (m->filtertheta) {
    for (int k = 1; k <= kz; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++) E3(m->tetav, j, i, k) = E3(m->tetav, j, i, k) - E3(m->tf, j, i, k);
    filttheta(m);
    for (int k = 1; k <= kz; k++)
      for (int i = 1; i <= ni; i++)
        for (int j = 1; j <= nj; j++) E3(m->tetav, j, i, k) = E3(m->tetav, j, i, k) + E3(m->tf, j, i, k);
  }
#pragma omp parallel for
  for (int k = 1; k <= kz; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) {
        E3(m->tvirt, j, i, k) = E3(m->tetav, j, i, k) * E3(m->pai, j, i, k);
        E3(m->t, j, i, k) = E3(m->tvirt, j, i, k) /
                            ((((1.0 + EP1 * E3(m->qv, j, i, k)) - E3(m->qc, j, i, k)) - E3(m->qi, j, i, k)) -
                             E3(m->qr, j, i, k) - E3(m->qsn, j, i, k));
        E3(m->p, j, i, k) = pow(E3(m->pai, j, i, k), CPOVR) * P00;
        E3(m->rho, j, i, k) = E3(m->p, j, i, k) / (RGAS * E3(m->t, j, i, k));
      }
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++) {
      double zdgz = E3(m->zeta, j, i, kz) * EGRAV;
      double lrt = (E3(m->tvirt, j, i, kz - 1) - E3(m->tvirt, j, i, kz)) /
                   (E3(m->zeta, j, i, kz - 1) - E3(m->zeta, j, i, kz));
      lrt = 0.65 * lrt - 0.35 * LRATE;
      double tv = E3(m->tvirt, j, i, kz) - (0.5 * E3(m->zeta, j, i, kz)) * lrt;
      E2(m->ps, j, i) = E3(m->p, j, i, kz) * exp(zdgz / (RGAS * tv));
    }
#pragma omp parallel for
  for (int k = 1; k <= kz; k++)
    for (int i = 1; i <= ni; i++)
      for (int j = 1; j <= nj; j++) E3(m->qsat, j, i, k) = pfwsat(E3(m->t, j, i, k), E3(m->p, j, i, k));
}

/* ======================================================================= */
/* exported oracle API (ctypes)                                            */
/* ======================================================================= */
void *oracle_create(const oracle_cfg *c) {
  Moloch *m = (Moloch *)calloc(1, sizeof(Moloch));
  m->nj = c->jx;
  m->ni = c->iy;
  m->kz = c->kz;
  m->divfilter = c->divfilter;
  m->filterpai = c->filterpai;
  m->filtertheta = c->filtertheta;
  m->lrotllr = c->rotllr;
  allocate_all(m);
  param(m, c);
  fill_atmosphere(m, c);
  init_moloch(m);
  return m;
}

/* one moloch() call; diag[0..5] = max/min ps, u, v over the interior;
   returns 1 if ps is NaN/Inf ("CFL VIOLATION", :402-411), else 0 */
int oracle_step(void *h, int istep, int lprint, double *diag) {
  Moloch *m = (Moloch *)h;
  (void)istep;
  double dtstepa = m->dt / (double)m->mo_nadv;
  double dtsound = dtstepa / (double)m->mo_nsound;
  reset_tendencies(m);
  prediag(m);
  for (int nadv = 1; nadv <= m->mo_nadv; nadv++) {
    sound(m, dtsound);
    advection(m, dtstepa);
  }
  postdiag(m);
  int bad = 0;
  if (lprint && diag) {
    double mxp = -INFINITY, mnp = INFINITY, mxu = -INFINITY, mnu = INFINITY, mxv = -INFINITY, mnv = INFINITY;
    for (int i = 1; i <= m->ni; i++)
      for (int j = 1; j <= m->nj; j++) {
        double x = E2(m->ps, j, i);
        if (x > mxp || isnan(x)) mxp = x;
        if (x < mnp || isnan(x)) mnp = x;
      }
    for (int k = 1; k <= m->kz; k++)
      for (int i = 1; i <= m->ni; i++)
        for (int j = 1; j <= m->nj; j++) {
          double x = E3(m->u, j, i, k), y = E3(m->v, j, i, k);
          mxu = x > mxu ? x : mxu;
          mnu = x < mnu ? x : mnu;
          mxv = y > mxv ? y : mxv;
          mnv = y < mnv ? y : mnv;
        }
    diag[0] = mxp; diag[1] = mnp; diag[2] = mxu; diag[3] = mnu; diag[4] = mxv; diag[5] = mnv;
    if (isnan(mxp) || isnan(mnp) || isinf(mxp) || isinf(mnp)) bad = 1;
  }
  return bad;
}

/* the staggering of advection() alone, for the cross-check of
   tests/test_oracle_restated.py: to_x = 1 runs uvstagtox + wstagtox
   (u, v, w -> ux, vx, wx), 0 runs xtouvstag + xtowstag (back) */
void oracle_stagger(void *h, int to_x) {
  Moloch *m = (Moloch *)h;
  if (to_x) {
    uvstagtox(m);
    wstagtox(m);
  } else {
    xtouvstag(m);
    xtowstag(m);
  }
}

/* phases, for per-phase parity tests: 0 reset+prediag, 1 sound, 2 advection, 3 postdiag */
void oracle_phase(void *h, int phase) {
  Moloch *m = (Moloch *)h;
  double dtstepa = m->dt / (double)m->mo_nadv;
  double dtsound = dtstepa / (double)m->mo_nsound;
  switch (phase) {
    case 0: reset_tendencies(m); prediag(m); break;
    case 1: sound(m, dtsound); break;
    case 2: advection(m, dtstepa); break;
    case 3: postdiag(m); break;
    default: break;
  }
}

static const A3 *field3(Moloch *m, const char *name) {
#define F(n, a) if (!strcmp(name, n)) return &m->a
  F("u", u); F("v", v); F("w", w); F("pai", pai); F("t", t); F("tetav", tetav);
  F("qv", qv); F("qc", qc); F("qi", qi); F("qr", qr); F("qs", qsn);
  F("p", p); F("rho", rho); F("tvirt", tvirt); F("qsat", qsat); F("s", s);
  F("deltaw", deltaw); F("zdiv2", zdiv2); F("fmz", fmz); F("fmzf", fmzf);
  F("zeta", zeta); F("ux", ux); F("vx", vx); F("wx", wx); F("qwltot", qwltot); F("qwitot", qwitot);
#undef F
  return NULL;
}
static const A2 *field2(Moloch *m, const char *name) {
#define F(n, a) if (!strcmp(name, n)) return &m->a
  F("ps", ps); F("ht", ht); F("hx", hx); F("hy", hy); F("coru", coru); F("corv", corv);
  F("msfu", msfu); F("msfv", msfv); F("msfx", msfx); F("ulat", ulat); F("vlat", vlat);
#undef F
  return NULL;
}

/* copy the interior (1:nj, 1:ni, 1:nk) of a field into a dense j-fastest
   buffer; nk = kz or kz+1.  Returns the number of levels, or -1. */
int oracle_get(void *h, const char *name, double *out) {
  Moloch *m = (Moloch *)h;
  const A3 *a = field3(m, name);
  if (a) {
    int nk = a->u3;
    long q = 0;
    for (int k = 1; k <= nk; k++)
      for (int i = 1; i <= m->ni; i++)
        for (int j = 1; j <= m->nj; j++) out[q++] = E3(*a, j, i, k);
    return nk;
  }
  const A2 *b = field2(m, name);
  if (b) {
    long q = 0;
    for (int i = 1; i <= m->ni; i++)
      for (int j = 1; j <= m->nj; j++) out[q++] = E2(*b, j, i);
    return 0;
  }
  return -1;
}

/* overwrite the interior of a prognostic field (for planted-error tests and
   for starting the oracle from a state produced elsewhere) */
int oracle_set(void *h, const char *name, const double *in) {
  Moloch *m = (Moloch *)h;
  A3 *a = (A3 *)field3(m, name);
  if (!a) return -1;
  int nk = a->u3;
  long q = 0;
  for (int k = 1; k <= nk; k++)
    for (int i = 1; i <= m->ni; i++)
      for (int j = 1; j <= m->nj; j++) E3(*a, j, i, k) = in[q++];
  return nk;
}

/* replace the map factors msfu, msfv, msfx (whole bounded arrays, as
   oracle_get_bounded returns them) and redo the terms init_moloch derives
   from them (mx2, rmu, rmv; :254-256), so the cross-check of
   tests/test_oracle_restated.py can run the non-ROTLLR branches with map
   factors other than 1 */
void oracle_set_map_factors(void *h, const double *msfu, const double *msfv, const double *msfx) {
  Moloch *m = (Moloch *)h;
  int nj = m->nj, ni = m->ni;
  memcpy(m->msfu.p, msfu, sizeof(double) * m->msfu.n1 * (m->msfu.u2 - m->msfu.l2 + 1));
  memcpy(m->msfv.p, msfv, sizeof(double) * m->msfv.n1 * (m->msfv.u2 - m->msfv.l2 + 1));
  memcpy(m->msfx.p, msfx, sizeof(double) * m->msfx.n1 * (m->msfx.u2 - m->msfx.l2 + 1));
  for (int i = 1; i <= ni; i++)
    for (int j = 1; j <= nj; j++) E2(m->mx2, j, i) = E2(m->msfx, j, i) * E2(m->msfx, j, i);
  for (int i = 1; i <= ni; i++)
    for (int j = 0; j <= nj + 1; j++) E2(m->rmu, j, i) = 1.0 / E2(m->msfu, j, i);
  for (int i = 0; i <= ni + 1; i++)
    for (int j = 1; j <= nj; j++) E2(m->rmv, j, i) = 1.0 / E2(m->msfv, j, i);
}

/* one 3-D filter for the cross-check of tests/test_oracle_restated.py:
   0 divergence_filter, 1 filtpai, 2 filttheta */
void oracle_filter(void *h, int which) {
  Moloch *m = (Moloch *)h;
  if (which == 0) divergence_filter(m);
  else if (which == 1) filtpai(m);
  else if (which == 2) filttheta(m);
}

/* divdamp with the step's dts = dt / mo_nadv / mo_nsound, for the
   cross-check of tests/test_oracle_restated.py */
void oracle_divdamp(void *h) {
  Moloch *m = (Moloch *)h;
  divdamp(m, m->dt / (double)m->mo_nadv / (double)m->mo_nsound);
}

/* wafone on one named field with the step's dta = dt / mo_nadv, for the
   cross-check of tests/test_oracle_restated.py; -1 for an unknown name */
int oracle_wafone(void *h, const char *name) {
  Moloch *m = (Moloch *)h;
  A3 *a = (A3 *)field3(m, name);
  if (!a) return -1;
  wafone(m, a, m->dt / (double)m->mo_nadv);
  return 0;
}

/* the full bounded array (halo included), for layout-contract tests */
int oracle_get_bounded(void *h, const char *name, double *out, int *lb, int *ub) {
  Moloch *m = (Moloch *)h;
  const A3 *a = field3(m, name);
  if (a) {
    lb[0] = a->l1; ub[0] = a->u1; lb[1] = a->l2; ub[1] = a->u2; lb[2] = a->l3; ub[2] = a->u3;
    if (out) memcpy(out, a->p, sizeof(double) * a->n12 * (a->u3 - a->l3 + 1));
    return 3;
  }
  const A2 *b = field2(m, name);
  if (b) {
    lb[0] = b->l1; ub[0] = b->u1; lb[1] = b->l2; ub[1] = b->u2; lb[2] = 1; ub[2] = 1;
    if (out) memcpy(out, b->p, sizeof(double) * b->n1 * (b->u2 - b->l2 + 1));
    return 2;
  }
  return -1;
}

/* OpenMP threads used by the oracle's loops (results do not depend on it) */
void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* known-answer hooks */
double oracle_pfesat(double t, double p) { return pfesat(t, p); }
double oracle_pfwsat(double t, double p) { return pfwsat(t, p); }
double oracle_gzita(double z, double ztop, double a0) { return gzita(z, ztop, a0); }
double oracle_md_zeta(double z, double geopot, double ztop, double zh, double a0) {
  return md_zeta(z, geopot, ztop, zh, a0);
}
double oracle_md_fmz(double z, double geopot, double ztop, double zh, double a0) {
  return md_fmz(z, geopot, ztop, zh, a0);
}
double oracle_superbee(double r) { return superbee(r); }
double oracle_splitmix_u01(unsigned long long seed, unsigned long long idx) { return splitmix_u01(seed, idx); }
void oracle_constants(double *c) {
  c[0] = RGAS; c[1] = RWAT; c[2] = CPD; c[3] = CVD; c[4] = RDRCV; c[5] = CPOVR; c[6] = ROVCP;
  c[7] = EP1; c[8] = EP2; c[9] = EOMEG2; c[10] = DEGRAD;
}
void oracle_scalars(void *h, double *s) {
  Moloch *m = (Moloch *)h;
  s[0] = m->dt; s[1] = m->dx; s[2] = m->mo_dzita; s[3] = m->mo_ztop; s[4] = m->mo_h; s[5] = m->mo_a0;
  s[6] = m->mo_nadv; s[7] = m->mo_nsound; s[8] = m->mo_anu2;
}
void oracle_xknu(void *h, double *out) {
  Moloch *m = (Moloch *)h;
  for (int k = 1; k <= m->kz; k++) out[k - 1] = m->xknu[k];
}

static void free3(A3 *a) { free(a->p); a->p = NULL; }
static void free2(A2 *a) { free(a->p); a->p = NULL; }
void oracle_destroy(void *h) {
  Moloch *m = (Moloch *)h;
  if (!m) return;
  A3 *a3s[] = {&m->u, &m->v, &m->ux, &m->vx, &m->t, &m->tetav, &m->w, &m->pai, &m->qv, &m->qc, &m->qi,
               &m->qr, &m->qsn, &m->zeta, &m->rho, &m->p, &m->tvirt, &m->qsat, &m->fmz, &m->fmzf,
               &m->zetaf, &m->dz, &m->deltaw, &m->s, &m->wx, &m->zdiv2, &m->wz, &m->p0, &m->ud, &m->vd,
               &m->qwltot, &m->qwitot, &m->pf, &m->tf, &m->wwkw, &m->wfw, &m->zpby, &m->zpbw};
  for (size_t q = 0; q < sizeof(a3s) / sizeof(a3s[0]); q++) free3(a3s[q]);
  A2 *a2s[] = {&m->ht, &m->xlat, &m->msfx, &m->msfu, &m->msfv, &m->hx, &m->hy, &m->ulat, &m->vlat,
               &m->ps, &m->p2d, &m->mx2, &m->rmu, &m->rmv, &m->coru, &m->corv};
  for (size_t q = 0; q < sizeof(a2s) / sizeof(a2s[0]); q++) free2(a2s[q]);
  free(m->zita); free(m->zitah); free(m->ffilt); free(m->gzitak); free(m->gzitakh); free(m->xknu);
  free(m);
}
