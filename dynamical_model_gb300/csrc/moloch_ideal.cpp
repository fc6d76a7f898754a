// Idealized initial state: host restatement of the reference driver's
// param() and init() (nompi/regcm_dynamical_core.F90:93-201) and of
// fill_atmosphere() (nompi/mod_atmosphere.F90:171-235), followed by the
// uploads and moloch_gpu_init() -- the sequence the Fortran program runs
// before its time loop.  Arrays are built with the reference's bounds so
// they travel through exactly the same moloch_gpu_upload() path a Fortran
// caller uses.  Compiled with -ffp-contract=off (FP64 as the reference).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/moloch_gb300.h"
#include "moloch_constants.h"

using namespace moloch;

namespace {

// a Fortran-style array with explicit lower/upper bounds, zero-filled
struct Arr {
  int nd = 0;
  int lb[4] = {1, 1, 1, 1}, ub[4] = {1, 1, 1, 1};
  std::vector<double> a;
  Arr() = default;
  Arr(std::initializer_list<int> b) {
    nd = (int)b.size() / 2;
    int n = 0;
    for (auto it = b.begin(); it != b.end(); it += 2, ++n) { lb[n] = it[0]; ub[n] = it[1]; }
    size_t tot = 1;
    for (int d = 0; d < nd; ++d) tot *= (size_t)(ub[d] - lb[d] + 1);
    a.assign(tot, 0.0);
  }
  size_t n(int d) const { return (size_t)(ub[d] - lb[d] + 1); }
  double& operator()(int j) { return a[(size_t)(j - lb[0])]; }
  double& operator()(int j, int i) { return a[(size_t)(j - lb[0]) + n(0) * (size_t)(i - lb[1])]; }
  double& operator()(int j, int i, int k) {
    return a[(size_t)(j - lb[0]) + n(0) * ((size_t)(i - lb[1]) + n(1) * (size_t)(k - lb[2]))];
  }
  void fill(double x) { for (auto& y : a) y = x; }
};

// splitmix64 of the linear index -> U[0,1)  (input generator, not in the reference)
double u01(uint64_t seed, uint64_t idx) {
  uint64_t z = seed + (idx + 1ULL) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z = z ^ (z >> 31);
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// vertical coordinate, nompi/mod_zita.F90
double zfz(double ztop, double zh) { return ztop / (std::exp(ztop / zh) - 1.0); }
double bzita(double z, double ztop, double zh) { return zfz(ztop, zh) * (std::exp(z / zh) - 1.0); }
double bzitap(double z, double ztop, double zh) { return zfz(ztop, zh) * std::exp(z / zh) / zh; }
double gzita(double z, double ztop, double a0) {
  double r = z / ztop, r2 = r * r, r3 = r2 * r;
  return (((0.0 - 1.0 * a0) * r - (3.0 - 2.0 * a0) * r2) + (2.0 - 1.0 * a0) * r3) + 1.0;
}
double gzitap(double z, double ztop, double a0) {
  double r = z / ztop, r2 = r * r;
  return (((0.0 - 1.0 * a0) * 1.0 - (6.0 - 4.0 * a0) * r) + (6.0 - 3.0 * a0) * r2) / ztop;
}
double fmz_of(double z, double geopot, double ztop, double zh, double a0) {  // md_fmz, Eq. 9
  double orog = geopot * kRegrav;
  return 1.0 / (gzitap(z, ztop, a0) * orog + bzitap(z, ztop, zh));
}
double zeta_of(double z, double geopot, double ztop, double zh, double a0) {  // md_zeta
  double orog = geopot * kRegrav;
  return orog * (gzita(z, ztop, a0) - 1.0) + bzita(z, ztop, zh);
}

int up(moloch_handle_t* h, int f, Arr& x) { return moloch_gpu_upload(h, f, x.a.data(), x.lb, x.ub); }

}  // namespace

// grid and parameters of a handle (defined in moloch_api.cpp, not exported in the header)
extern "C" int moloch_internal_describe(moloch_handle_t* h, moloch_grid_t* g, moloch_params_t* p);

extern "C" int moloch_gpu_setup_idealized(moloch_handle_t* h, const moloch_ideal_t* ideal) {
  if (!h || !ideal) return MOLOCH_ERR_ARG;
  // the grid and parameters the handle was created with
  moloch_grid_t g;
  moloch_params_t P;
  int rc = moloch_internal_describe(h, &g, &P);
  if (rc) return rc;
  const int nj = g.jx, ni = g.iy, kz = g.kz;

  // ---- param() ----
  std::vector<double> zita(kz + 2), zitah(kz + 2);
  {
    double dz = P.mo_ztop / (double)kz;  // model_zitaf / model_zitah
    zita[kz + 1] = 0.0;
    for (int k = kz; k >= 1; --k) zita[k] = zita[k + 1] + dz;
    zitah[kz] = dz * 0.5;
    for (int k = kz - 1; k >= 1; --k) zitah[k] = zitah[k + 1] + dz;
  }
  const double dzita = zita[kz];
  const double rdx = 1.0 / P.dx;
  Arr ht{-1, nj + 2, -1, ni + 2};
  for (int n = 0; n < ideal->nhills && n < 4; ++n)
    for (int i = 1; i <= ni; ++i)
      for (int j = 1; j <= nj; ++j) {
        double dj = (double)j - ideal->hill_j[n], di = (double)i - ideal->hill_i[n];
        double rr = (dj * dj + di * di) / (ideal->hill_r[n] * ideal->hill_r[n]);
        ht(j, i) += ideal->hill_h[n] * kEgrav * std::exp(-rr);
      }
  Arr msfx{1, nj, 1, ni}, msfu{0, nj + 1, 1, ni}, msfv{1, nj, 0, ni + 1};
  msfx.fill(1.0); msfu.fill(1.0); msfv.fill(1.0);
  Arr ulat{1, nj, 1, ni}, vlat{1, nj, 1, ni};
  const double dl = kRaddeg * P.dx / kEarthrad;
  const double clat = 0.0;
  for (int i = 1; i <= ni; ++i)
    for (int j = 1; j <= nj; ++j) {
      ulat(j, i) = clat + dl * (((double)i - (double)ni * 0.5) - 0.5);  // xlat, ulat = xlat
      vlat(j, i) = clat + dl * ((double)i - (double)ni * 0.5);
    }
  Arr hx{0, nj + 1, 1, ni}, hy{1, nj, 0, ni + 1};
  for (int i = 1; i <= ni; ++i)
    for (int j = 1; j <= nj; ++j) hx(j, i) = (((ht(j, i) - ht(j - 1, i)) * msfu(j, i)) * rdx) * kRegrav;
  for (int i = 1; i <= ni; ++i)
    for (int j = 1; j <= nj; ++j)
      hy(j, i) = P.rotllr ? ((ht(j, i) - ht(j, i - 1)) * rdx) * kRegrav
                          : (((ht(j, i) - ht(j, i - 1)) * msfv(j, i)) * rdx) * kRegrav;
  for (int i = 1; i <= ni; ++i) { hx(0, i) = hx(nj, i); hx(nj + 1, i) = hx(1, i); }
  for (int j = 1; j <= nj; ++j) { hy(j, 0) = hy(j, ni); hy(j, ni + 1) = hy(j, 1); }
  Arr zeta{-1, nj + 2, -1, ni + 2, 1, kz}, fmz{0, nj + 1, 0, ni + 1, 1, kz}, fmzf{1, nj, 1, ni, 1, kz + 1};
  for (int k = 1; k <= kz; ++k)
    for (int i = 1; i <= ni; ++i)
      for (int j = 1; j <= nj; ++j) {
        zeta(j, i, k) = zeta_of(zitah[k], ht(j, i), P.mo_ztop, P.mo_h, P.mo_a0);
        fmz(j, i, k) = fmz_of(zitah[k], ht(j, i), P.mo_ztop, P.mo_h, P.mo_a0);
      }
  for (int k = 1; k <= kz + 1; ++k)
    for (int i = 1; i <= ni; ++i)
      for (int j = 1; j <= nj; ++j) fmzf(j, i, k) = fmz_of(zita[k], ht(j, i), P.mo_ztop, P.mo_h, P.mo_a0);

  // ---- fill_atmosphere() ----
  const double ts = 300.0, qs0 = 0.01865, ps0 = 101480.0, tropoh = 15000.0;
  const double tvs = ts * (1.0 + kEp1 * qs0);
  const double tvt = tvs - kLrate * tropoh;
  Arr t{0, nj + 1, 0, ni + 1, 1, kz}, pai{0, nj + 1, 0, ni + 1, 1, kz};
  Arr qx{0, nj + 1, 0, ni + 1, 1, kz, 1, 5};
  auto QV = [&](int j, int i, int k) -> double& {
    return qx.a[(size_t)(j - qx.lb[0]) + qx.n(0) * ((size_t)(i - qx.lb[1]) + qx.n(1) * (size_t)(k - 1))];
  };
  for (int i = 1; i <= ni; ++i)
    for (int j = 1; j <= nj; ++j)
      for (int k = 1; k <= kz; ++k) {
        double zi = zeta(j, i, k);
        if (zi < tropoh) {
          double xq = -(zi / 7500.0);
          double qi = (qs0 * std::exp(-(zi / 4000.0))) * std::exp(xq * xq);
          QV(j, i, k) = qi;
          t(j, i, k) = (tvs - kLrate * zi) / (1.0 + qi);
        } else {
          QV(j, i, k) = 1.0e-8;
          t(j, i, k) = tvt;
        }
      }
  // warm bubble on the lowest level; the radius mixes default-REAL (single)
  // and FP64 arithmetic exactly as written in the reference
  {
    const int mx = nj / 2, my = ni / 2;
    double aj = (double)(float)nj / 5.0;
    float bi = (float)ni / 5.0f;
    float bi2 = bi * bi;
    double mr = std::sqrt(aj * aj + (double)bi2) / 2.0;
    for (int i = 1; i <= ni; ++i)
      for (int j = 1; j <= nj; ++j) {
        float fj = (float)(j - mx), fi = (float)(i - my);
        double md = (double)std::sqrt(fj * fj + fi * fi);
        if (md < mr) t(j, i, kz) = t(j, i, kz) + (mr - md) / mr;
      }
  }
  Arr u{-1, nj + 2, 0, ni + 1, 1, kz}, v{0, nj + 1, -1, ni + 2, 1, kz}, w{1, nj, 1, ni, 1, kz + 1};
  u.fill(ideal->u0);
  v.fill(ideal->v0);
  for (int i = 1; i <= ni; ++i)  // hydrostatic pai, top-down (lowest level first)
    for (int j = 1; j <= nj; ++j) {
      double zdelta = zeta(j, i, kz) * kEgrav;
      double tv1 = t(j, i, kz) * (1.0 + kEp1 * QV(j, i, kz));
      double tv2 = t(j, i, kz - 1) * (1.0 + kEp1 * QV(j, i, kz - 1));
      double lrt = (tv2 - tv1) / (zeta(j, i, kz - 1) - zeta(j, i, kz));
      lrt = 0.65 * lrt - 0.35 * kLrate;
      double tv = tv1 - (0.5 * zeta(j, i, kz)) * lrt;
      double zz = 1.0 / (kRgas * tv);
      double p = ps0 * std::exp(-(zdelta * zz));
      pai(j, i, kz) = std::pow(p / kP00, kRovcp);
    }
  for (int k = kz - 1; k >= 1; --k)
    for (int i = 1; i <= ni; ++i)
      for (int j = 1; j <= nj; ++j) {
        double tv1 = t(j, i, k) * (1.0 + kEp1 * QV(j, i, k));
        double tv2 = t(j, i, k + 1) * (1.0 + kEp1 * QV(j, i, k + 1));
        double zb = (((2.0 * kEgrav) * dzita) / (fmzf(j, i, k + 1) * kCpd) + tv1) - tv2;
        double zdelta = std::sqrt(zb * zb + (4.0 * tv2) * tv1);
        pai(j, i, k) = -((pai(j, i, k + 1) / (2.0 * tv2)) * (zb - zdelta));
      }
  if (ideal->pert_amp != 0.0) {
    int k0 = kz - ideal->pert_levels + 1;
    if (k0 < 1) k0 = 1;
    for (int k = k0; k <= kz; ++k)
      for (int i = 1; i <= ni; ++i)
        for (int j = 1; j <= nj; ++j) {
          uint64_t idx = (uint64_t)(j - 1) + (uint64_t)nj * ((uint64_t)(i - 1) + (uint64_t)ni * (uint64_t)(k - 1));
          double dth = ideal->pert_amp * (2.0 * u01(ideal->seed, idx) - 1.0);
          t(j, i, k) = t(j, i, k) + dth * pai(j, i, k);
        }
  }
  // ---- uploads (init_moloch aliases these arrays) and init_moloch ----
  Arr zz{1, kz + 1}, zh{1, kz};
  for (int k = 1; k <= kz + 1; ++k) zz(k) = zita[k];
  for (int k = 1; k <= kz; ++k) zh(k) = zitah[k];
  // periodic ghosts of fmz and zeta as param() fills them
  for (int k = 1; k <= kz; ++k) {
    for (int i = 1; i <= ni; ++i) {
      fmz(0, i, k) = fmz(nj, i, k); fmz(nj + 1, i, k) = fmz(1, i, k);
      zeta(0, i, k) = zeta(nj, i, k); zeta(nj + 1, i, k) = zeta(1, i, k);
      zeta(-1, i, k) = zeta(nj - 1, i, k); zeta(nj + 2, i, k) = zeta(2, i, k);
    }
    for (int j = 1; j <= nj; ++j) {
      fmz(j, 0, k) = fmz(j, ni, k); fmz(j, ni + 1, k) = fmz(j, 1, k);
      zeta(j, 0, k) = zeta(j, ni, k); zeta(j, ni + 1, k) = zeta(j, 1, k);
      zeta(j, -1, k) = zeta(j, ni - 1, k); zeta(j, ni + 2, k) = zeta(j, 2, k);
    }
  }
  for (int i = 1; i <= ni; ++i) { msfu(0, i) = msfu(nj, i); msfu(nj + 1, i) = msfu(1, i); }
  for (int j = 1; j <= nj; ++j) { msfv(j, 0) = msfv(j, ni); msfv(j, ni + 1) = msfv(j, 1); }
  if ((rc = up(h, MOLOCH_F_ZITA, zz)) || (rc = up(h, MOLOCH_F_ZITAH, zh)) || (rc = up(h, MOLOCH_F_HT, ht)) ||
      (rc = up(h, MOLOCH_F_MSFX, msfx)) || (rc = up(h, MOLOCH_F_MSFU, msfu)) || (rc = up(h, MOLOCH_F_MSFV, msfv)) ||
      (rc = up(h, MOLOCH_F_HX, hx)) || (rc = up(h, MOLOCH_F_HY, hy)) || (rc = up(h, MOLOCH_F_ULAT, ulat)) ||
      (rc = up(h, MOLOCH_F_VLAT, vlat)) || (rc = up(h, MOLOCH_F_ZETA, zeta)) || (rc = up(h, MOLOCH_F_FMZ, fmz)) ||
      (rc = up(h, MOLOCH_F_FMZF, fmzf)) || (rc = up(h, MOLOCH_F_U, u)) || (rc = up(h, MOLOCH_F_V, v)) ||
      (rc = up(h, MOLOCH_F_W, w)) || (rc = up(h, MOLOCH_F_T, t)) || (rc = up(h, MOLOCH_F_PAI, pai)) ||
      (rc = up(h, MOLOCH_F_QX, qx)))
    return rc;
  return moloch_gpu_init(h);
}
