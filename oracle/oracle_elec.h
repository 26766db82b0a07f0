// TEST INFRASTRUCTURE ONLY — the oracle of the storm's electrification and lightning (see oracle_core.h).
// Restates src/core/charge.ts (the non-inductive charging of the Takahashi and Saunders-Peck schemes, the inductive
// charging, the transfer of charge with the water between its carriers), src/core/takahashi.ts (the table lookup),
// src/core/electric.ts (ElectricSolver) and src/core/lightning.ts (Lightning: the conduction and corona, the field
// solve, the breakdown search, the branched channel growth and its charge deposit). FP64 throughout, JS evaluation
// order; Float32Array stores go through Cell<float>.
#pragma once
#include <cstdint>
#include <memory>
#include "oracle_solvers.h"
#include "../meteolab_gb300/csrc/sg_takahashi.h"

namespace orc {

constexpr double EPSILON0 = 8.8541878128e-12;  // src/core/electric.ts:6

// ---------------------------------------------------------------- src/core/charge.ts
constexpr double CHARGING_COLDEST = -33, MAX_COLLISION_CHARGE = 20e-15, COLLECTION_EFFICIENCY = .6, CHARGING_SPEED = 6;  // :13,:29,:34,:42
constexpr double CRYSTAL_SIZE = 100e-6, MAX_CRYSTALS = 150e3, CRYSTAL_LO = 20e-6, CRYSTAL_HI = 300e-6;               // :81,:86,:88
constexpr double RIMER_CD = .6, TAK_RATE_MAX = 3e-9;                                                                   // :107,:154
constexpr double DROPLET_REBOUND = .01, DROPLET_SIZE = 20e-6, CONTACT_COS = .5;                                        // :184
constexpr int AIR_CARRIER = 3;                                                                                         // :206

inline double criticalRar(double tc) {  // :50-53
  double t = jmin(-7.35, jmax(-23.7, tc));
  return 1 + 7.9262e-2 * t + 4.4847e-2 * std::pow(t, 2) + 7.4754e-3 * std::pow(t, 3) + 5.4686e-4 * std::pow(t, 4) + 1.6737e-5 * std::pow(t, 5) +
         1.7613e-7 * std::pow(t, 6);
}
inline double collisionCharge(double tc, double rar, double d, double v, bool signedCoefficients = false) {  // :62-70
  if (tc >= 0 || tc < CHARGING_COLDEST || d <= 0 || v <= 0) return 0;
  double c = criticalRar(tc);
  double q = rar > c ? 6.74 * (rar - c) : rar > .1 ? 3.9 * (c - .1) * (4 * std::pow((rar - (c + .1) / 2) / (c - .1), 2) - 1) : 0;
  double scale = signedCoefficients && q < 0 ? (d < 253e-6 ? 5.24e8 * std::pow(d, 2.54) : 24 * std::pow(d, .5)) * std::pow(v, 2.8)
                                             : (d < 155e-6 ? 4.92e13 * std::pow(d, 3.76) : d < 452e-6 ? 4.04e6 * std::pow(d, 1.9) : 52.8 * std::pow(d, .44)) * std::pow(v, 2.5);
  double dq = scale * q * 1e-15;
  return jmax(-MAX_COLLISION_CHARGE, jmin(MAX_COLLISION_CHARGE, dq));
}
inline double crystalNumber(double tc, double qi = 0, double rho = 1) {  // :97-100
  double cooper = jmin(MAX_CRYSTALS, 5 * std::exp(.304 * jmax(0, -tc))), fromMass = rho * qi / (PI / 6 * 900 * std::pow(CRYSTAL_SIZE, 3));
  return jmin(MAX_CRYSTALS, jmax(cooper, fromMass));
}
inline double crystalDiameter(double qi, double rho, double tc) {  // :103-105
  return qi > 0 ? jmin(CRYSTAL_HI, jmax(CRYSTAL_LO, std::cbrt(6 * rho * qi / (PI * 900 * crystalNumber(tc, qi, rho))))) : 0;
}

struct RimerMoments { double n, d1, d2, fall, d2v; };
inline RimerMoments exponentialMoments(double n0, double density, double q, double rho) {  // :118-121
  double lambda = std::pow(PI * density * n0 / (rho * q), .25), a = std::sqrt(4 * G * density / (3 * RIMER_CD * rho));
  return {n0 / lambda, n0 / (lambda * lambda), 2 * n0 / std::pow(lambda, 3), a * GAMMA_45 / 6 / std::sqrt(lambda), a * n0 * GAMMA_35 / std::pow(lambda, 3.5)};
}

// src/core/takahashi.ts:43-54: bilinear in the temperature (1 K columns) and between the neighbouring cloud-water rows.
inline double takahashiCharge(double tc, double lwc) {
  static const double LWC[SG_TAKAHASHI_ROWS] = SG_TAKAHASHI_LWC;
  static const double TABLE[SG_TAKAHASHI_ROWS][SG_TAKAHASHI_COLS] = SG_TAKAHASHI_TABLE;
  if (tc >= 0 || tc <= -40 || lwc < .01) return 0;
  double w = jmin(30, lwc);
  int row = 0;
  while (row < SG_TAKAHASHI_ROWS - 2 && w >= LWC[row + 1]) row++;
  double t = jmin(30, -jmax(-30, tc));
  int col = (int)jmin(29, std::floor(t));
  double f = t - col;
  auto at = [&](const double* r) { return r[col] + f * (r[col + 1] - r[col]); };
  double a = at(TABLE[row]), b = at(TABLE[row + 1]), g = jmin(1, (w - LWC[row]) / (LWC[row + 1] - LWC[row]));
  double cold = tc < -30 ? 1 - std::pow((tc + 30) / 10, 2) : 1;
  return cold * (a + g * (b - a));
}
inline double takahashiScaled(double table, double d, double dv) {  // charge.ts:229-233
  double q = table * jmin(5 * std::pow(d / 100e-6, 2) * std::fabs(dv) / 8, 10) * 1e-15;
  return jmax(-500e-15, jmin(500e-15, q));
}

inline double rimerRate(const RimerMoments& m, double tc, double water, double rebound, double ni, double di, double ns, double ds, double vs,
                        double table, bool tak) {  // :157-168
  double fall = m.fall, impact = jmin(fall, CHARGING_SPEED), rar = COLLECTION_EFFICIENCY * water * impact, k = PI / 4 * rebound;
  auto swept = [&](double d) { return m.d2 + 2 * d * m.d1 + d * d * m.n; };
  auto pair = [&](double r) { return tak ? jmax(-TAK_RATE_MAX, jmin(TAK_RATE_MAX, r)) : r; };
  double rate = 0;
  if (ni > 0) rate += pair(ni * k * swept(di) * fall * (tak ? takahashiScaled(table, di, fall) : collisionCharge(tc, rar, di, impact)));
  if (ns > 0) {
    double v = std::fabs(fall - vs);
    rate += pair(ns * k * swept(ds) * v * (tak ? takahashiScaled(table, ds, v) : collisionCharge(tc, rar, ds, std::fabs(impact - vs))));
  }
  return rate;
}

// :136-151. `crystals` < 0 stands for "not given" (the reference's undefined): the number is then estimated from the mass.
// `twoMoment` (ice2m.ts rimerMoments of graupel and hail, a null pointer or a false flag for "none") replaces the
// exponential moments of a rimer that has them (:153-155; a missing entry falls back to the fixed intercept's).
inline double chargingRate(double tc, double rho, double cloud, double ice, double snow, double graupel, double hail, double snowFall, bool wetGraupel = false,
                           bool wetHail = false, double crystals = -1, bool tak = true, const RimerMoments* twoMoment = nullptr, const bool* twoHas = nullptr) {
  if (tc >= 0 || tc < (tak ? -40 : CHARGING_COLDEST) || cloud <= 0 || ice + snow <= 0 || graupel + hail <= 0) return 0;
  double rebound = tak ? .5 * (1 - .1 * std::exp(.1 * tc)) : 1 - std::exp(.09 * tc), water = rho * cloud * 1000;
  bool given = crystals >= 0;
  double ni = ice <= 0 ? 0 : given ? crystals : crystalNumber(tc, ice, rho);
  auto size = [&](double m) { return tak ? .1871 * std::pow(m, .3429) : plateSize(m); };
  double di = ice <= 0 ? 0 : (given && crystals != 0) ? jmin(CRYSTAL_HI, jmax(CRYSTAL_LO, size(rho * ice / crystals))) : crystalDiameter(ice, rho, tc);
  double snowSlope = snow > 0 ? std::pow(PI * RHO_S * N0S / (rho * snow), .25) : 0, ns = snow > 0 ? N0S / snowSlope : 0,
         ds = snow > 0 ? (tak ? 1.8171 : 1) / snowSlope : 0;
  double rate = 0, table = tak ? takahashiCharge(tc, water) : 0;
  auto momentsOf = [&](int j, double n0, double dens, double q) { return twoMoment && twoHas[j] ? twoMoment[j] : exponentialMoments(n0, dens, q, rho); };
  if (graupel > 0 && !wetGraupel) rate += rimerRate(momentsOf(0, N0G, RHO_G, graupel), tc, water, rebound, ni, di, ns, ds, snowFall, table, tak);
  if (hail > 0 && !wetHail) rate += rimerRate(momentsOf(1, N0H, RHO_H, hail), tc, water, rebound, ni, di, ns, ds, snowFall, table, tak);
  return rate;
}

inline double inductiveRate(double tc, double rho, double cloud, double graupel, double hail, double ez, double rimerCharge, bool wetGraupel = false,
                            bool wetHail = false, const RimerMoments* twoMoment = nullptr, const bool* twoHas = nullptr) {  // :187-200
  if (tc >= 0 || cloud <= 0) return 0;
  double d = DROPLET_SIZE, droplets = rho * cloud / (PI / 6 * 1000 * std::pow(d, 3)), k = COLLECTION_EFFICIENCY * DROPLET_REBOUND * droplets;
  double polarize = 0, mass = 0, massFall = 0;
  const double n0[2] = {N0G, N0H}, dens[2] = {RHO_G, RHO_H}, q[2] = {graupel, hail};
  const bool wet[2] = {wetGraupel, wetHail};
  for (int j = 0; j < 2; j++) {
    if (q[j] <= 1e-9 || wet[j]) continue;
    RimerMoments m = twoMoment && twoHas[j] ? twoMoment[j] : exponentialMoments(n0[j], dens[j], q[j], rho);
    polarize += std::pow(PI, 4) / 8 * EPSILON0 * ez * CONTACT_COS * d * d * m.d2v;
    mass += q[j]; massFall += q[j] * m.fall;
  }
  if (mass == 0) return 0;
  return k * (polarize - std::pow(PI, 3) / 24 * d * d * (massFall / mass) * rimerCharge);
}

// :216-226: charge moves with the mass between [ice-snow, graupel-hail, rain, droplets and ions]; in place, conservative.
inline void transferCharge(double* charge, const double* before, const double* after) {
  double pool = 0, lost = 0, gained = 0;
  for (int k = 0; k < 4; k++) {
    if (after[k] < before[k]) {
      double share = before[k] > 0 ? (before[k] - after[k]) / before[k] : 1, out = charge[k] * share;
      charge[k] -= out; pool += out; lost += before[k] - after[k];
    } else gained += after[k] - before[k];
    if (k != AIR_CARRIER && after[k] <= 0 && charge[k] != 0) { pool += charge[k]; charge[k] = 0; }
  }
  if (pool == 0) return;
  double moved = gained > 0 ? jmin(1, lost > 0 ? gained / lost : 1) : 0;
  if (moved > 0) for (int k = 0; k < 4; k++) if (after[k] > before[k]) charge[k] += pool * moved * (after[k] - before[k]) / gained;
  charge[AIR_CARRIER] += pool * (1 - moved);
}

// ---------------------------------------------------------------- src/core/electric.ts:15-60
struct ElectricSolver {
  const GridSpec* g = nullptr;
  HorizontalDFT dft; DftScratch scr;
  std::vector<double> lambda, cp, dRe, dIm;
  ElectricSolver() {}
  explicit ElectricSolver(const GridSpec& grid) : g(&grid), dft(grid.nx, grid.ny, grid.nz - 2), scr(grid.nx, grid.ny) {
    int nx = grid.nx, ny = grid.ny;
    lambda.resize((size_t)nx * ny);
    for (int n = 0; n < ny; n++) for (int m = 0; m < nx; m++)
      lambda[m + nx * n] = 4 * std::pow(std::sin(PI * m / nx), 2) / (grid.dx * grid.dx) + 4 * std::pow(std::sin(PI * n / ny), 2) / (grid.dy * grid.dy);
    cp.assign(grid.nz, 0); dRe.assign(grid.nz, 0); dIm.assign(grid.nz, 0);
  }
  void solve(const double* rho, double* phi) {
    const GridSpec& G_ = *g;
    int nx = G_.nx, ny = G_.ny, nz = G_.nz, layer = G_.layer, ni = nz - 2, cl = nx * ny;
    std::vector<double> inner((size_t)cl * ni);
    for (size_t i = 0; i < inner.size(); i++) inner[i] = -rho[i + layer] / EPSILON0;
    dft.forwardLayers([&](size_t i) { return inner[i]; }, 0, ni, scr);
    double *re = dft.re.data(), *im = dft.im.data();
    for (int n = 0; n < ny; n++) for (int m = 0; m <= dft.mh; m++) {
      int mode = m + nx * n; double lam = lambda[mode];
      for (int j = 0; j < ni; j++) {
        int k = j + 1; double lo = 1 / (G_.hz[k] * G_.dzs[k - 1]), up = 1 / (G_.hz[k] * G_.dzs[k]), di = -lo - up - lam;
        double a = j > 0 ? lo : 0, c = j < ni - 1 ? up : 0, r = re[mode + (size_t)j * cl], s = im[mode + (size_t)j * cl];
        double piv = j == 0 ? di : di - a * cp[j - 1];
        cp[j] = c / piv;
        dRe[j] = (r - (j == 0 ? 0 : a * dRe[j - 1])) / piv;
        dIm[j] = (s - (j == 0 ? 0 : a * dIm[j - 1])) / piv;
      }
      for (int j = ni - 1; j >= 0; j--) {
        if (j < ni - 1) { dRe[j] -= cp[j] * dRe[j + 1]; dIm[j] -= cp[j] * dIm[j + 1]; }
        re[mode + (size_t)j * cl] = dRe[j]; im[mode + (size_t)j * cl] = dIm[j];
      }
    }
    dft.inverseLayers([&](size_t i, double v) { inner[i] = v; }, 0, ni, scr);
    for (int i = 0; i < layer; i++) { phi[i] = 0; phi[i + (size_t)(nz - 1) * layer] = 0; }
    for (size_t i = 0; i < inner.size(); i++) phi[i + layer] = inner[i];
  }
};

// ---------------------------------------------------------------- src/core/math.ts:7-14
struct Mulberry32 {
  uint32_t s;
  explicit Mulberry32(uint32_t seed = 0) : s(seed) {}
  double operator()() {
    s += 0x6D2B79F5u;
    uint32_t t = (s ^ (s >> 15)) * (1u | s);
    t = (t + (t ^ (t >> 7)) * (61u | t)) ^ t;
    return (double)(t ^ (t >> 14)) / 4294967296.0;
  }
};

// ---------------------------------------------------------------- src/core/lightning.ts
constexpr double E_INIT = 2.84e5, RHO_STANDARD = 1.225, F_CRIT = .43, RHO_MIN = 1e-10, CHANNEL_RADIUS = 1, SHIELDING = .25;  // :13-29
constexpr int MAX_CHANNEL = 3000, STROKES = 4, MAX_FLASHES = 10;                                                           // :31,:36,:43
constexpr double FLASH_WINDOW = 3, SIGMA_GROUND = 2e-14, SIGMA_SCALE = 6000, CLOUD_SIGMA = .1, CLOUDY = 1e-5;                // :43,:51,:58
constexpr double CORONA_FIELD = 5e3, CORONA_RATE = 5e-13;                                                                  // :67
inline int flashLimit(double dt) { return (int)jmax(1, std::floor(MAX_FLASHES * dt / FLASH_WINDOW + .5)); }               // :45

struct Flash {
  double time = 0; bool cg = false; int start = -1, ground = -1;
  std::vector<int> nodes, parent, polarity;
  double potential = 0, charge = 0, moment = 0;
  std::vector<double> strokes;
};

// Lightning (:135-420). Carriers are fields (C/kg) of the model's storage S, changed in place through Cell<S>.
struct Lightning {
  const GridSpec* g; std::vector<double> air;
  ElectricSolver solver;
  std::vector<double> rho, phi, change, sigma, eInit, capacitance, weight, scale;
  std::vector<int> mark, failed, frontier, seen, link;
  std::vector<float> cloudy; bool hasCloud = false;
  double fromGround = 0, moment = 0, conducted = 0; bool corona = true;
  int flashId = 0, size = 0; uint32_t seed; Mulberry32 rng;

  Lightning(const GridSpec& grid, const double* airDensity, int seed_ = 1) : g(&grid), air(airDensity, airDensity + grid.nz), solver(grid),
      seed((uint32_t)seed_), rng((uint32_t)seed_) {
    int n = grid.n, nz = grid.nz;
    rho.assign(n, 0); phi.assign(n, 0); change.assign(n, 0); sigma.assign(n, 0); weight.assign(n, 0); scale.assign(n, 0);
    mark.assign(n, 0); failed.assign(n, 0); frontier.assign(n, 0); seen.assign(n, 0); link.assign(n, 0);
    eInit.resize(nz); capacitance.resize(nz);
    for (int z = 0; z < nz; z++) {
      eInit[z] = E_INIT * air[z] / RHO_STANDARD;
      double L = std::cbrt(grid.dx * grid.dy * grid.hz[z]);
      capacitance[z] = SHIELDING * 2 * PI * EPSILON0 * L / std::log(L / CHANNEL_RADIUS);
    }
  }

  // :185-223 the ion current sigma E over dt and the corona; returns the charge the air lost.
  template <class S> double conduct(Arr<S> ions, double dt) {
    const GridSpec& G_ = *g;
    int nx = G_.nx, ny = G_.ny, nz = G_.nz, layer = G_.layer; double dx = G_.dx, dy = G_.dy;
    for (int z = 0, i = 0; z < nz; z++) {
      double clear = SIGMA_GROUND * std::exp(G_.zs[z] / SIGMA_SCALE);
      for (int e = i + layer; i < e; i++) sigma[i] = hasCloud && (double)cloudy[i] > CLOUDY ? clear * CLOUD_SIGMA : clear;
    }
    std::fill(change.begin(), change.end(), 0.0);
    auto series = [](double a, double b) { return 2 * a * b / (a + b); };
    double lost = 0;
    for (int z = 0; z < nz - 1; z++) {
      double across = dy * G_.hz[z] * dt / dx, along = dx * G_.hz[z] * dt / dy, up = dx * dy * dt / G_.dzs[z];
      for (int y = 0; y < ny; y++) for (int x = 0; x < nx; x++) {
        int i = x + y * nx + z * layer;
        if (z > 0) {
          int ix = G_.xp[x] + y * nx + z * layer, iy = x + G_.yp[y] + z * layer;
          double qx = series(sigma[i], sigma[ix]) * (phi[i] - phi[ix]) * across, qy = series(sigma[i], sigma[iy]) * (phi[i] - phi[iy]) * along;
          change[i] -= qx + qy; change[ix] += qx; change[iy] += qy;
        }
        int j = i + layer; double q = series(sigma[i], sigma[j]) * (phi[i] - phi[j]) * up;
        if (z == 0) { change[j] += q; lost -= q; } else if (z == nz - 2) { change[i] -= q; lost += q; } else { change[i] -= q; change[j] += q; }
      }
    }
    if (corona) for (int c = 0; c < layer; c++) {
      double e0 = -phi[c + layer] / G_.dzs[0], over = std::fabs(e0) - CORONA_FIELD;
      if (over <= 0) continue;
      double q = (e0 > 0 ? 1 : e0 < 0 ? -1 : 0) * CORONA_RATE * over * dx * dy * dt;
      change[c + layer] += q; lost -= q;
    }
    for (int z = 1; z < nz - 1; z++) {
      double perKg = 1 / (air[z] * dx * dy * G_.hz[z]);
      for (int i = z * layer, e = i + layer; i < e; i++) if (change[i] != 0) ions[i] += change[i] * perKg;
    }
    conducted += lost;
    return lost;
  }

  template <class S> void solve(Arr<S>* carriers, int count) {  // :226-230
    int nz = g->nz, layer = g->layer;
    for (int z = 0, i = 0; z < nz; z++) for (int e = i + layer; i < e; i++) {
      double s = 0; for (int c = 0; c < count; c++) s += carriers[c][i];
      rho[i] = s * air[z];
    }
    solver.solve(rho.data(), phi.data());
  }

  std::pair<int, double> strongest(int stamp = -1) const {  // :233-246
    const GridSpec& G_ = *g;
    int nx = G_.nx, ny = G_.ny, nz = G_.nz, layer = G_.layer, best = -1; double ratio = 0;
    for (int z = 1; z < nz - 1; z++) {
      double dz = G_.zs[z + 1] - G_.zs[z - 1], limit2 = eInit[z] * eInit[z];
      for (int y = 0; y < ny; y++) for (int x = 0; x < nx; x++) {
        int i = x + y * nx + z * layer, row = y * nx + z * layer;
        double ex = (phi[G_.xp[x] + row] - phi[G_.xm[x] + row]) / (2 * G_.dx), ey = (phi[x + G_.yp[y] + z * layer] - phi[x + G_.ym[y] + z * layer]) / (2 * G_.dy),
               ez = (phi[i + layer] - phi[i - layer]) / dz;
        double r = (ex * ex + ey * ey + ez * ez) / limit2;
        if (r > ratio && failed[i] != stamp) { ratio = r; best = i; }
      }
    }
    return {best, std::sqrt(ratio)};
  }

  template <class S> void cloud(Arr<S>* fields, int count) {  // :249-253
    cloudy.assign(g->n, 0.f); hasCloud = true;
    for (int f = 0; f < count; f++) for (int i = 0; i < g->n; i++) cloudy[i] = (float)((double)cloudy[i] + (double)fields[f][i]);
  }

  // :259-275
  template <class S> std::vector<Flash> discharge(Arr<S>* carriers, int count, double time, int limit = MAX_FLASHES) {
    std::vector<Flash> flashes; int stamp = ++flashId;
    int32_t tenths = (int32_t)(int64_t)std::floor(time * 10 + .5);
    rng = Mulberry32(seed ^ (uint32_t)((uint32_t)tenths * 0x9E3779B1u));
    for (int k = 0; k <= limit; k++) {
      solve(carriers, count);
      if (k == limit) break;
      auto [start, ratio] = strongest(stamp);
      if (ratio <= 1) break;
      Flash f = flash(start, carriers, count, time);
      if (f.charge == 0) { failed[start] = stamp; continue; }
      flashes.push_back(std::move(f));
    }
    return flashes;
  }

  bool clear(int i) const { return std::fabs(rho[i]) < RHO_MIN || (hasCloud && (double)cloudy[i] <= CLOUDY); }  // :343

  // :287-340
  template <class S> Flash flash(int start, Arr<S>* carriers, int count, double time) {
    int layer = g->layer, id = ++flashId;
    std::vector<int> nodes, parent, polarity; std::vector<double> strokeCharges;
    double sum = 0, potential = 0, before = 0, neutralized = 0, lowered = 0;
    int ground = -1, strokes = 0; bool touched = false, left = false;
    size = 0; moment = 0;
    auto add = [&](int j, int from) {
      mark[j] = id; nodes.push_back(j); parent.push_back(from);
      if (j < layer) { ground = j; before = potential; potential = 0; touched = true; return; }
      if (ground < 0) { sum += phi[j]; potential = sum / (double)nodes.size(); }
      extend(j, (int)nodes.size() - 1, id);
    };
    add(start, -1);
    for (;;) {
      size_t grown = nodes.size(); bool event = false;
      while (nodes.size() < (size_t)MAX_CHANNEL) {
        double total = 0;
        for (int f = 0; f < size; f++) {
          int j = frontier[f];
          bool zero = (ground >= 0 && (j < layer || phi[j] * before <= 0)) || (clear(j) && (phi[j] - potential) * potential >= 0);
          double w = zero ? 0 : std::fabs(potential - phi[j]) / scale[j] - 1;
          weight[f] = w > 0 ? w : 0; total += weight[f];
        }
        if (total == 0) break;
        double pick = rng() * total; int n = 0;
        while (n < size - 1 && (pick -= weight[n]) > 0) n++;
        int j = frontier[n], from = link[j];
        if (!left && ground < 0 && clear(j)) { left = true; event = true; break; }
        frontier[n] = frontier[--size];
        if (clear(nodes[from])) for (int f = size - 1; f >= 0; f--) if (link[frontier[f]] == from) frontier[f] = frontier[--size];
        add(j, from);
        if (touched) { touched = false; event = true; break; }
      }
      if (ground >= 0) { double q = deposit(nodes, polarity, potential, true, carriers, count); lowered += q; strokeCharges.push_back(q); }
      else neutralized += deposit(nodes, polarity, potential, false, carriers, count);
      if (ground >= 0 && (++strokes >= STROKES || (!event && nodes.size() == grown))) break;
      if (ground < 0 && !event) break;
      if (nodes.size() >= (size_t)MAX_CHANNEL) break;
      solve(carriers, count);
      if (ground < 0) { sum = 0; for (int i : nodes) sum += phi[i]; potential = sum / (double)nodes.size(); }
    }
    Flash f; f.time = time; f.cg = ground >= 0; f.start = start; f.nodes = nodes; f.parent = parent; f.polarity = polarity;
    f.potential = ground >= 0 ? before : potential; f.charge = ground >= 0 ? lowered : neutralized; f.ground = ground; f.moment = ground >= 0 ? moment : 0;
    if (ground >= 0) f.strokes = strokeCharges;
    return f;
  }

  // :352-381
  template <class S> double deposit(const std::vector<int>& nodes, std::vector<int>& polarity, double V, bool grounded, Arr<S>* carriers, int count) {
    const GridSpec& G_ = *g; int layer = G_.layer; std::vector<double> dep(nodes.size(), 0.0);
    double positive = 0, negative = 0;
    for (size_t c = 0; c < nodes.size(); c++) {
      int i = nodes[c], z = i / layer;
      if (z == 0) { if (c >= polarity.size()) polarity.push_back(0); continue; }
      double q = capacitance[z] * (V - phi[i]), here = rho[i] * G_.dx * G_.dy * G_.hz[z];
      if (c >= polarity.size()) polarity.push_back(q > 0 ? 1 : q < 0 ? -1 : 0);
      if (q * here >= 0) continue;
      double d = (q > 0 ? 1 : -1) * jmin(std::fabs(q), std::fabs(here));
      dep[c] = d;
      if (d > 0) positive += d; else negative -= d;
    }
    double charge;
    if (!grounded) {
      double both = jmin(positive, negative);
      for (size_t c = 0; c < nodes.size(); c++) dep[c] *= dep[c] > 0 ? (positive > 0 ? both / positive : 0) : (negative > 0 ? both / negative : 0);
      charge = both;
    } else {
      charge = negative - positive;
      fromGround -= charge;
      for (size_t c = 0; c < nodes.size(); c++) if (dep[c] != 0) moment -= dep[c] * G_.zs[nodes[c] / layer];
    }
    for (size_t c = 0; c < nodes.size(); c++) if (dep[c] != 0) neutralize(carriers, count, nodes[c], dep[c]);
    return charge;
  }

  // :389-404
  void extend(int i, int c, int id) {
    const GridSpec& G_ = *g; int nx = G_.nx, ny = G_.ny, nz = G_.nz, layer = G_.layer;
    int z = i / layer, y = (i - z * layer) / nx, x = i - z * layer - y * nx;
    for (int k = std::max(0, z - 1); k <= std::min(nz - 2, z + 1); k++) {
      double hz = G_.zs[k] - G_.zs[z], threshold = F_CRIT * .5 * (eInit[z] + eInit[k]);
      for (int dj = -1; dj <= 1; dj++) for (int di = -1; di <= 1; di++) {
        if (x + di < 0 || x + di >= nx || y + dj < 0 || y + dj >= ny) continue;
        int j = x + di + (y + dj) * nx + k * layer;
        if (mark[j] == id || (k >= z && std::fabs(rho[j]) < RHO_MIN)) continue;
        double s = std::sqrt(std::pow(di * G_.dx, 2) + std::pow(dj * G_.dy, 2) + hz * hz) * threshold;
        if (seen[j] != id) { seen[j] = id; frontier[size++] = j; }
        else if (s >= scale[j]) continue;
        scale[j] = s; link[j] = c;
      }
    }
  }

  // :410-418
  template <class S> void neutralize(Arr<S>* carriers, int count, int i, double q) {
    const GridSpec& G_ = *g; int z = i / G_.layer;
    double perKg = q / (air[z] * G_.dx * G_.dy * G_.hz[z]), sq = q > 0 ? 1 : -1, opposite = 0;
    for (int c = 0; c < count; c++) if ((double)carriers[c][i] * q < 0) opposite -= (double)carriers[c][i] * sq;
    if (opposite <= 0) return;
    for (int c = 0; c < count; c++) if ((double)carriers[c][i] * q < 0) carriers[c][i] += perKg * std::fabs((double)carriers[c][i]) / opposite;
  }
};

}  // namespace orc
