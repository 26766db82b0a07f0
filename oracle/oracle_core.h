// TEST INFRASTRUCTURE ONLY — the oracle. A CPU restatement of the reference's StormLab model step
// (Bandananor/MeteoLAB, TypeScript, src/core/*.ts) used by tests/, __graft_entry__.smoke() and bench.py's
// cpu_baseline / --impl reference leg as the checker. The product (meteolab_gb300) never links or calls it.
//
// Semantics follow the reference as JavaScript runs it: every arithmetic operation in double precision, every store
// into a Float32Array rounded to float (Math.fround). `Cell<S>` reproduces that: reading converts to double, every
// assignment (=, +=, -=, *=) rounds to S. S = float gives the reference's own storage ("faithful"); S = double gives
// the pure FP64 oracle. Evaluation order is the reference's order as written.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace orc {

// src/core/constants.ts:1-6
constexpr double G = 9.81, CP = 1004, LV = 2.5e6, KAPPA = .286, RD = 287.05, RV = 461.5, EPS = .622, OMEGA = 7.2921e-5;
// src/core/ice.ts:92-125
constexpr double LF = 3.34e5, LS = LV + LF, T0 = 273.15, T_HOMOGENEOUS = 235.15, CW = 4187;
constexpr double NUCLEATION_START = -5, MAX_NUCLEATED = 250e3, CRYSTAL_MASS = 1e-12, MAX_CRYSTAL_MASS = 9.4e-10;
constexpr double RHO_I = 900;
constexpr double SPLINTERS = 3.5e8;
constexpr double KA = 2.43e-2, PSI = 2.26e-5, NU = 1.51e-5, SC = .6;
constexpr double N0S = 3e6, RHO_S = 100, D_S = .25;
constexpr double GAMMA_3D = 2.5493, GAMMA_4D = 8.2850, GAMMA_5D2 = 1.4569;
constexpr double ICE_AUTOCONVERSION_THRESHOLD = .001;
// src/core/microphysics.ts:9-15
constexpr double AUTOCONVERSION_THRESHOLD = .001, AUTOCONVERSION_RATE = .001, N0_MP = 8e6;
// src/core/graupel.ts:6-13
constexpr double N0G = 4e4, RHO_G = 400, CD_G = .6, N0R = 8e6, RHO_W = 1000, BIGG_B = 100, BIGG_A = .66;
constexpr double GAMMA_45 = 11.6317, GAMMA_35 = 3.3234, GAMMA_275 = 1.6084;
constexpr double SNOW_TO_GRAUPEL_THRESHOLD = 6e-4;
// src/core/hail.ts:84-90
constexpr double N0H = 4e4, RHO_H = 900, CD_H = .6, CI = 2106, HAIL_CONVERSION_TIME = 60, HAIL_SAMPLE_VOLUME = 10;
// src/core/model.ts:71, :110
constexpr double TINY_WATER = 1e-10, U_LIMIT = 120, W_LIMIT = 100;
// src/core/turbulence.ts:11-13
constexpr double SMAGORINSKY = .18, PRANDTL = 1.0 / 3;
constexpr double PI = 3.141592653589793;

inline double C_S() { return 152.93 * std::pow(.01, .75); }  // src/core/ice.ts:122
inline double DROPLET_MASS() { return PI / 6 * 1000 * std::pow(20e-6, 3); }  // src/core/ice.ts:102

// JavaScript Math.max / Math.min (NaN in, NaN out).
inline double jmax(double a, double b) { if (a != a || b != b) return NAN; return a >= b ? a : b; }
inline double jmin(double a, double b) { if (a != a || b != b) return NAN; return a <= b ? a : b; }
inline double jmax3(double a, double b, double c) { return jmax(jmax(a, b), c); }
inline double jmin3(double a, double b, double c) { return jmin(jmin(a, b), c); }
// src/core/math.ts:1-3
inline double clamp(double x, double a = 0, double b = 1) { return jmax(a, jmin(b, x)); }
inline double lerp(double a, double b, double t) { return a + (b - a) * clamp(t); }
inline double jmod(double x, double n) { return std::fmod(std::fmod(x, n) + n, n); }

// One element of a typed array: reads as double, stores rounded to S.
template <class S> struct Cell {
  S v;
  operator double() const { return (double)v; }
  Cell& operator=(double x) { v = (S)x; return *this; }
  Cell& operator=(const Cell& o) = default;
  Cell& operator+=(double x) { v = (S)((double)v + x); return *this; }
  Cell& operator-=(double x) { v = (S)((double)v - x); return *this; }
  Cell& operator*=(double x) { v = (S)((double)v * x); return *this; }
};
template <class S> using Arr = Cell<S>*;

// ---------------------------------------------------------------- microphysics (src/core/microphysics.ts)
inline double qsatP(double t, double p) {  // :5
  double es = 611.2 * std::exp(17.67 * t / (t + 243.5));
  return clamp(EPS * es / jmax(1000, p - es), 0, .045);
}
inline double fallSpeed(double rain, double rho, double rhoGround) {  // :37-39 (Marshall-Palmer intercept)
  return rain > 0 ? 36.34 * std::pow(.001 * rho * rain, .1364) * std::sqrt(rhoGround / rho) * 1 : 0;
}
// :48-60 with the fixed intercept; returns the evaporated rain.
template <class S> double rainProcesses(Arr<S> q, Arr<S> cloud, Arr<S> rain, int i, double tk, double p, double rho, double dt, bool evaporate) {
  double qc = cloud[i], qr = rain[i];
  double rate = AUTOCONVERSION_RATE * jmax(0, qc - AUTOCONVERSION_THRESHOLD) + (qr > 0 ? 2.2 * qc * std::pow(qr, .875) * 1 : 0);
  double production = jmin(qc, rate * dt);
  cloud[i] -= production; rain[i] += production;
  double qs = qsatP(tk - 273.15, p);
  if (!evaporate || (double)rain[i] <= 0 || (double)q[i] >= qs) return 0;
  double rq = .001 * rho * (double)rain[i], ventilation = 1.6 + 124.9 * std::pow(rq, .2046);
  double er = (1 - (double)q[i] / qs) * ventilation * std::pow(rq, .525) / (.001 * rho * (5.4e5 + 2.55e6 / (p / 100 * qs)));
  double evaporation = jmin3(rain[i], er * dt, (qs - (double)q[i]) / (1 + LV * LV * qs / (CP * RV * tk * tk)));
  rain[i] -= evaporation; q[i] += evaporation;
  return evaporation;
}
// :67-77
template <class S> double saturationAdjust(Arr<S> theta, Arr<S> q, Arr<S> cloud, int i, double exner, double p) {
  double total = 0;
  for (int k = 0; k < 2; k++) {
    double tk = (double)theta[i] * exner, qs = qsatP(tk - 273.15, p);
    double d = ((double)q[i] - qs) / (1 + LV * LV * qs / (CP * RV * tk * tk));
    if (d < 0) d = jmax(d, -(double)cloud[i]);
    if (d == 0) break;
    q[i] -= d; cloud[i] += d; theta[i] += LV / (CP * exner) * d; total += d;
  }
  return total;
}

// ---------------------------------------------------------------- ice (src/core/ice.ts)
inline double splintering(double tc) { return tc >= -3 || tc <= -8 ? 0 : tc > -5 ? (-3 - tc) / 2 : (tc + 8) / 3; }  // :108
inline double fragmentsPerKg(double lambda) { return 2.5e13 * 7 / (lambda * 1000 * PI / 6); }  // :116
inline double qsatIce(double t, double p) {  // :130-134
  if (t >= 0) return qsatP(t, p);
  double es = 611.21 * std::exp(22.587 * t / (t + 273.86));
  return clamp(EPS * es / jmax(1000, p - es), 0, .045);
}
inline double cooperCrystals(double tc) { return tc >= NUCLEATION_START ? 0 : jmin(MAX_NUCLEATED, 5 * std::exp(.304 * -tc)); }  // :137
inline double snowSlope(double snow, double rho) { return std::pow(PI * RHO_S * N0S / (rho * snow), .25); }  // :140
inline double snowFallSpeed(double snow, double rho, double rhoGround) {  // :143-145
  return snow > 1e-9 ? C_S() * GAMMA_4D / 6 * std::pow(snowSlope(snow, rho), -D_S) * std::sqrt(rhoGround / rho) : 0;
}
// :154-176
template <class S> double saturationAdjustMixed(Arr<S> theta, Arr<S> q, Arr<S> cloud, Arr<S> ice, int i, double exner, double p, Arr<S> number) {
  double heat = LF / (CP * exner);
  if ((double)theta[i] * exner >= T_HOMOGENEOUS) {
    if ((double)ice[i] > 0 && (double)theta[i] * exner > T0) {
      double melt = jmin(ice[i], ((double)theta[i] * exner - T0) * CP / LF);
      if (number) number[i] *= 1 - melt / (double)ice[i];
      ice[i] -= melt; cloud[i] += melt; theta[i] -= heat * melt;
    }
    return saturationAdjust<S>(theta, q, cloud, i, exner, p);
  }
  if ((double)cloud[i] > 0) { if (number) number[i] += (double)cloud[i] / DROPLET_MASS(); ice[i] += (double)cloud[i]; theta[i] += heat * (double)cloud[i]; cloud[i] = 0.0; }
  double total = 0;
  for (int k = 0; k < 2; k++) {
    double tk = (double)theta[i] * exner, qs = qsatIce(tk - T0, p);
    double d = ((double)q[i] - qs) / (1 + LS * LS * qs / (CP * RV * tk * tk));
    if (d < 0) d = jmax(d, -(double)ice[i]);
    if (d == 0) break;
    q[i] -= d; ice[i] += d; theta[i] += LS / (CP * exner) * d; total += d;
  }
  return total;
}
// :179-183
template <class S> void freezeRain(Arr<S> theta, Arr<S> rain, Arr<S> graupel, int i, double exner) {
  double r = rain[i];
  if (r <= 0 || (double)theta[i] * exner >= T_HOMOGENEOUS) return;
  rain[i] = 0.0; graupel[i] += r; theta[i] += LF / (CP * exner) * r;
}
inline double crystalSize(double qi, double n, double rho) { return std::cbrt(6 * rho * qi / (PI * RHO_I * n)); }  // :186
inline double plateSize(double m) { return .01 * std::pow(m * 1000 / .00739, 1 / 2.45); }  // :192
// :197-206 (Koenig 1971 growth table of the reference)
static const double KOENIG_A1[31] = {.7939e-7, .7841e-6, .3369e-5, .4336e-5, .5285e-5, .3728e-5, .1852e-5, .2991e-6, .4248e-6, .7434e-6, .1812e-5, .4394e-5, .9145e-5, .1725e-4, .3348e-4,
  .1725e-4, .9175e-5, .4412e-5, .2252e-5, .9115e-6, .4876e-6, .3473e-6, .4758e-6, .6306e-6, .8573e-6, .7868e-6, .7192e-6, .6513e-6, .5956e-6, .5333e-6, .4834e-6};
static const double KOENIG_A2[31] = {.4006, .4831, .5320, .5307, .5319, .5249, .4888, .3894, .4047, .4318, .4771, .5183, .5463, .5651, .5813,
  .5655, .5478, .5203, .4906, .4447, .4126, .3960, .4149, .4320, .4506, .4483, .4460, .4433, .4413, .4382, .4361};
inline double koenigGrowth(double tc, double m) {
  double x = clamp(-tc, 1, 31) - 1; int k = (int)jmin(29, std::floor(x)); double f = x - k, g = m * 1000;
  return 1e-3 * ((1 - f) * KOENIG_A1[k] * std::pow(g, KOENIG_A2[k]) + f * KOENIG_A1[k + 1] * std::pow(g, KOENIG_A2[k + 1]));
}
// :223-242
template <class S> double iceProcesses(Arr<S> theta, Arr<S> q, Arr<S> ice, Arr<S> snow, Arr<S> number, int i, double exner, double p, double rho, double dt) {
  double tk = (double)theta[i] * exner, tc = tk - T0;
  if (tc >= 0 || tk < T_HOMOGENEOUS) return 0;
  double qsi = qsatIce(tc, p), limit = ((double)q[i] - qsi) / (1 + LS * LS * qsi / (CP * RV * tk * tk)), heat = LS / (CP * exner), lacking = cooperCrystals(tc) / rho - (double)number[i];
  double change = 0;
  if (limit > 0 && lacking > 0) { change = jmin(limit, lacking * CRYSTAL_MASS); number[i] += change / CRYSTAL_MASS; }
  double qi = (double)ice[i] + change, n = number[i];
  if (qi > 1e-12 && n > 0) {
    if ((double)q[i] > qsi) change += jmin(n * koenigGrowth(tc, qi / n) * ((double)q[i] - qsi) / (qsatP(tc, p) - qsi) * dt, limit - change);
    else {
      double a = LS * LS / (KA * RV * tk * tk), b = 1 / (rho * qsi * PSI);
      double lost = jmin(qi, n * 2 * PI * crystalSize(qi, n * rho, rho) * (1 - (double)q[i] / qsi) / (a + b) * dt);
      change -= lost; number[i] *= 1 - lost / qi;
    }
  }
  ice[i] += change; q[i] -= change; theta[i] += heat * change;
  double excess = (double)ice[i] - (double)number[i] * MAX_CRYSTAL_MASS;
  if (excess > 0) { ice[i] -= excess; snow[i] += excess; }
  return change < 0 ? -heat * change : 0;
}
// :245-248
template <class S> void settleCrystals(Arr<S> ice, Arr<S> number, int i) {
  double qi = ice[i];
  number[i] = qi > 1e-12 ? jmin(qi / CRYSTAL_MASS, jmax(qi / MAX_CRYSTAL_MASS, number[i])) : 0;
}
// :266-303 (RIMED_SNOW_TO_GRAUPEL off, the default)
template <class S> double snowProcesses(Arr<S> theta, Arr<S> q, Arr<S> cloud, Arr<S> ice, Arr<S> snow, Arr<S> rain, int i, double exner, double p, double rho, double rhoGround, double dt) {
  double tk = (double)theta[i] * exner, tc = tk - T0, qs = snow[i];
  if (tc < 0 && (double)ice[i] > 0) {
    double aut = 1e-3 * std::exp(.025 * tc) * jmax(0, (double)ice[i] - ICE_AUTOCONVERSION_THRESHOLD);
    double moved = jmin(ice[i], aut * dt); ice[i] -= moved; snow[i] += moved;
  }
  if (qs <= 1e-9) return 0;
  double lambda = snowSlope(qs, rho), fall = std::sqrt(rhoGround / rho), cs = C_S();
  double sweep = PI * N0S * cs * GAMMA_3D / (4 * std::pow(lambda, 3 + D_S)) * fall;
  double vent = N0S * (.78 / (lambda * lambda) + .31 * std::pow(SC, 1.0 / 3) * GAMMA_5D2 * std::sqrt(cs) * std::pow(fall, .5) / std::sqrt(NU) * std::pow(lambda, -(D_S + 5) / 2));
  double cooling = 0;
  if (tc < 0) {
    double saci = jmin(ice[i], sweep * std::exp(.025 * tc) * (double)ice[i] * dt); ice[i] -= saci; snow[i] += saci;
    double sacw = jmin(cloud[i], sweep * (double)cloud[i] * dt); cloud[i] -= sacw; snow[i] += sacw;
    theta[i] += LF / (CP * exner) * sacw;
    double qsi = qsatIce(tc, p), a = LS * LS / (KA * RV * tk * tk), b = 1 / (rho * qsi * PSI);
    double rate = 2 * PI * ((double)q[i] / qsi - 1) * vent / (rho * (a + b));
    double dep = rate > 0 ? jmin(rate * dt, ((double)q[i] - qsi) / (1 + LS * LS * qsi / (CP * RV * tk * tk))) : -jmin(snow[i], -rate * dt);
    snow[i] += dep; q[i] -= dep; theta[i] += LS / (CP * exner) * dep;
    if (dep < 0) cooling -= LS / (CP * exner) * dep;
  } else {
    double sacw = jmin(cloud[i], sweep * (double)cloud[i] * dt); cloud[i] -= sacw; rain[i] += sacw;
    double rate = 2 * PI * KA * tc * vent / (rho * LF) + CW * tc / LF * sweep * (double)cloud[i];
    double melt = jmin3(snow[i], rate * dt, CP * tc / LF);
    snow[i] -= melt; rain[i] += melt; theta[i] -= LF / (CP * exner) * melt; cooling += LF / (CP * exner) * melt;
  }
  return cooling;
}

// ---------------------------------------------------------------- graupel (src/core/graupel.ts)
inline double graupelSlope(double graupel, double rho) { return std::pow(PI * RHO_G * N0G / (rho * graupel), .25); }  // :16
inline double graupelFallCoefficient(double rho) { return std::sqrt(4 * G * RHO_G / (3 * CD_G * rho)); }  // :18
inline double graupelFallSpeed(double graupel, double rho) {  // :21-23
  return graupel > 1e-9 ? graupelFallCoefficient(rho) * GAMMA_45 / 6 * std::pow(graupelSlope(graupel, rho), -.5) : 0;
}
// :34-72
template <class S> double graupelProcesses(Arr<S> theta, Arr<S> q, Arr<S> cloud, Arr<S> ice, Arr<S> snow, Arr<S> rain, Arr<S> graupel, int i, double exner, double p, double rho, double dt) {
  double tk = (double)theta[i] * exner, tc = tk - T0, heat = 1 / (CP * exner);
  double cooling = 0;
  if (tc < 0) {
    if ((double)rain[i] > 1e-9) {
      double lambdaR = std::pow(PI * RHO_W * N0R / (rho * (double)rain[i]), .25);
      double rate = 20 * PI * PI * BIGG_B * N0R * RHO_W / rho * (std::exp(-BIGG_A * tc) - 1) / std::pow(lambdaR, 7);
      double frozen = jmin(rain[i], rate * dt); rain[i] -= frozen; graupel[i] += frozen; theta[i] += LF * heat * frozen;
    }
    double aut = jmin(snow[i], 1e-3 * std::exp(.09 * tc) * jmax(0, (double)snow[i] - SNOW_TO_GRAUPEL_THRESHOLD) * dt);
    snow[i] -= aut; graupel[i] += aut;
  }
  double qg = graupel[i];
  if (qg <= 1e-9) return 0;
  double lambda = graupelSlope(qg, rho), a = graupelFallCoefficient(rho);
  double sweep = PI * N0G * a * GAMMA_35 / (4 * std::pow(lambda, 3.5));
  double vent = N0G * (.78 / (lambda * lambda) + .31 * std::pow(SC, 1.0 / 3) * GAMMA_275 * std::sqrt(a / NU) * std::pow(lambda, -2.75));
  if (tc < 0) {
    double gacw = jmin(cloud[i], sweep * (double)cloud[i] * dt), gacr = jmin(rain[i], sweep * (double)rain[i] * dt);
    double gaci = jmin(ice[i], sweep * .1 * (double)ice[i] * dt), gacs = jmin(snow[i], sweep * std::exp(.09 * tc) * (double)snow[i] * dt);
    cloud[i] -= gacw; rain[i] -= gacr; ice[i] -= gaci; snow[i] -= gacs; graupel[i] += gacw + gacr + gaci + gacs;
    theta[i] += LF * heat * (gacw + gacr);
    double qsi = qsatIce(tc, p);
    if ((double)q[i] < qsi) {
      double aa = LS * LS / (KA * RV * tk * tk), b = 1 / (rho * qsi * PSI);
      double sub = jmin3(graupel[i], 2 * PI * (1 - (double)q[i] / qsi) * vent / (rho * (aa + b)) * dt, (qsi - (double)q[i]) / (1 + LS * LS * qsi / (CP * RV * tk * tk)));
      graupel[i] -= sub; q[i] += sub; theta[i] -= LS * heat * sub; cooling += LS * heat * sub;
    }
  } else {
    double gacw = jmin(cloud[i], sweep * (double)cloud[i] * dt); cloud[i] -= gacw; rain[i] += gacw;
    double rate = 2 * PI * KA * tc * vent / (rho * LF) + CW * tc / LF * sweep * ((double)cloud[i] + (double)rain[i]);
    double melt = jmin3(graupel[i], rate * dt, CP * tc / LF);
    graupel[i] -= melt; rain[i] += melt; theta[i] -= LF * heat * melt; cooling += LF * heat * melt;
  }
  return cooling;
}

// ---------------------------------------------------------------- hail (src/core/hail.ts)
inline double slopeOf(double q, double rho, double n0, double rhoX) { return std::pow(PI * rhoX * n0 / (rho * q), .25); }  // :93
inline double fallCoefficientOf(double rho, double rhoX) { return std::sqrt(4 * G * rhoX / (3 * CD_H * rho)); }  // :95
inline double sweepOf(double lambda, double a, double n0) { return PI * n0 * a * GAMMA_35 / (4 * std::pow(lambda, 3.5)); }  // :97
inline double ventilationOf(double lambda, double a, double n0) { return n0 * (.78 / (lambda * lambda) + .31 * std::pow(SC, 1.0 / 3) * GAMMA_275 * std::sqrt(a / NU) * std::pow(lambda, -2.75)); }  // :99
inline double hailFallSpeed(double hail, double rho) {  // :102-104
  return hail > 1e-9 ? fallCoefficientOf(rho, RHO_H) * GAMMA_45 / 6 * std::pow(slopeOf(hail, rho, N0H, RHO_H), -.5) : 0;
}
inline double hailMaxDiameter(double hail, double rho) {  // :107-111
  if (!(hail > 1e-9)) return 0;
  double lambda = slopeOf(hail, rho, N0H, RHO_H);
  return jmax(0, std::log(N0H * HAIL_SAMPLE_VOLUME / lambda) / lambda);
}
inline double wetGrowth(double lambda, double a, double n0, double tc, double qv, double p, double rho, double iceRate) {  // :118-121
  double heat = KA * -tc + LV * PSI * rho * (qsatP(0, p) - qv);
  return jmax(0, 2 * PI * ventilationOf(lambda, a, n0) * heat / (rho * (LF + CW * tc))) + iceRate * (1 - CI * tc / (LF + CW * tc));
}
inline bool wetGrowing(double q, double n0, double rhoX, double tc, double qv, double p, double rho, double cloud, double rain, double ice, double snow) {  // :127-131
  if (tc >= 0 || q <= 1e-9) return false;
  double lambda = slopeOf(q, rho, n0, rhoX), a = fallCoefficientOf(rho, rhoX), k = sweepOf(lambda, a, n0);
  return k * (cloud + rain + .1 * ice + std::exp(.09 * tc) * snow) > wetGrowth(lambda, a, n0, tc, qv, p, rho, k * (ice + snow));
}
// :140-175
template <class S> double hailProcesses(Arr<S> theta, Arr<S> q, Arr<S> cloud, Arr<S> ice, Arr<S> snow, Arr<S> rain, Arr<S> graupel, Arr<S> hail, int i, double exner, double p, double rho, double dt) {
  double tk = (double)theta[i] * exner, tc = tk - T0, heat = 1 / (CP * exner);
  double cooling = 0;
  if (wetGrowing(graupel[i], N0G, RHO_G, tc, q[i], p, rho, cloud[i], rain[i], ice[i], snow[i])) {
    double turned = (double)graupel[i] * (1 - std::exp(-dt / HAIL_CONVERSION_TIME)); graupel[i] -= turned; hail[i] += turned;
  }
  double qh = hail[i];
  if (qh <= 1e-9) return 0;
  double lambda = slopeOf(qh, rho, N0H, RHO_H), a = fallCoefficientOf(rho, RHO_H), k = sweepOf(lambda, a, N0H), vent = ventilationOf(lambda, a, N0H);
  if (tc < 0) {
    double hacw = jmin(cloud[i], k * (double)cloud[i] * dt), hacr = jmin(rain[i], k * (double)rain[i] * dt), liquid = hacw + hacr;
    double haci = jmin(ice[i], k * .1 * (double)ice[i] * dt), hacs = jmin(snow[i], k * std::exp(.09 * tc) * (double)snow[i] * dt), frozen = liquid;
    double wet = wetGrowth(lambda, a, N0H, tc, q[i], p, rho, k * ((double)ice[i] + (double)snow[i])) * dt;
    if (liquid + haci + hacs > wet) {
      haci = jmin(ice[i], k * (double)ice[i] * dt); hacs = jmin(snow[i], k * (double)snow[i] * dt);
      frozen = jmin(liquid, jmax(0, wet - haci - hacs));
    }
    cloud[i] -= hacw; rain[i] += liquid - frozen - hacr; ice[i] -= haci; snow[i] -= hacs; hail[i] += frozen + haci + hacs;
    theta[i] += LF * heat * frozen;
    double qsi = qsatIce(tc, p);
    if ((double)q[i] < qsi) {
      double aa = LS * LS / (KA * RV * tk * tk), b = 1 / (rho * qsi * PSI);
      double sub = jmin3(hail[i], 2 * PI * (1 - (double)q[i] / qsi) * vent / (rho * (aa + b)) * dt, (qsi - (double)q[i]) / (1 + LS * LS * qsi / (CP * RV * tk * tk)));
      hail[i] -= sub; q[i] += sub; theta[i] -= LS * heat * sub; cooling += LS * heat * sub;
    }
  } else {
    double hacw = jmin(cloud[i], k * (double)cloud[i] * dt); cloud[i] -= hacw; rain[i] += hacw;
    double rate = 2 * PI * KA * tc * vent / (rho * LF) + CW * tc / LF * k * ((double)cloud[i] + (double)rain[i]);
    double melt = jmin3(hail[i], rate * dt, CP * tc / LF);
    hail[i] -= melt; rain[i] += melt; theta[i] -= LF * heat * melt; cooling += LF * heat * melt;
  }
  return cooling;
}

}  // namespace orc
