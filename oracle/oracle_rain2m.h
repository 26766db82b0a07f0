// TEST INFRASTRUCTURE ONLY — the oracle of two-moment rain (see oracle_core.h): restates src/core/rain2m.ts (the NSSL
// warm-rain processes of rain mass and drop number, the drops' fall speeds, the number's bookkeeping when the ice
// processes take or give rain). FP64 arithmetic in JS order; Float32Array stores through Cell<S>.
#pragma once
#include "oracle_core.h"

namespace orc {
namespace r2m {

constexpr double RHO_W2 = 1000, RHO_00 = 1.225;                                                                 // rain2m.ts:11
const double XV_MIN = PI / 6 * std::pow(80e-6, 3), XV_MAX = PI / 6 * std::pow(6e-3, 3) / (64.0 / 6);              // :13
constexpr double CLOUD_DROPLETS = .6e9, AA1 = 9.44e15, AA2 = 5.78e3, G1 = 120.0 / 6, VT_A = 10, VT_B = 516.575;   // :15-21
constexpr double RAIN_BREAK_FACTOR = 1e6, RAIN_MIN = 1e-12, NUMBER_MIN = 1e-8;                                    // :32-35
enum Breakup { NONE = 0, NSSL = 1, MORRISON = 2 };

inline double meanVolume(double q, double n) { return jmin(XV_MAX, jmax(XV_MIN, q / (RHO_W2 * n))); }           // :38
inline double dnOf(double xv) { return std::cbrt(xv / PI); }                                                     // :41
inline double boundedNumber(double q, double n, double rho) {                                                    // :47-51
  if (!(q > RAIN_MIN)) return 0;
  if (!(n > NUMBER_MIN)) { double lambda = std::pow(PI * RHO_W2 * 8e6 / (rho * q), .25); n = 8e6 / lambda / rho; }
  return q / (RHO_W2 * meanVolume(q, n));
}
inline void fallSpeeds(double q, double n, double rho, double& vm, double& vn) {                                 // :57-61
  if (!(q > RAIN_MIN) || !(n > NUMBER_MIN)) { vm = vn = 0; return; }
  double dn = dnOf(meanVolume(q, n)), r = std::sqrt(RHO_00 / jmax(.05, rho)), x = 1 + VT_B * dn;
  vm = r * VT_A * (1 - std::pow(x, -4)); vn = r * VT_A * (1 - std::pow(x, -1));
}
inline double fallSpeedZ(double q, double n, double rho) {                                                       // :64-67
  if (!(q > RAIN_MIN) || !(n > NUMBER_MIN)) return 0;
  return std::sqrt(RHO_00 / jmax(.05, rho)) * VT_A * (1 - std::pow(1 + VT_B * dnOf(meanVolume(q, n)), -7));
}

// rain2mProcesses (:76-146): autoconversion, accretion, self-collection (and breakup), evaporation; the number bounded.
template <class S>
double processes(Arr<S> q, Arr<S> cloud, Arr<S> rain, Arr<S> number, int i, double tk, double p, double rho, double dt, int breakup, bool evaporate) {
  double qc = cloud[i], qr = rain[i];
  double nr = qr > RAIN_MIN ? boundedNumber(qr, number[i], rho) * rho : 0;
  double autoM = 0, autoN = 0, accretion = 0;
  const double nc = CLOUD_DROPLETS * rho / RHO_00;
  const double xvc = qc > 1e-9 ? jmin(PI / 6 * std::pow(120e-6, 3), jmax(PI / 6 * std::pow(4e-6, 3), rho * qc / (RHO_W2 * nc))) : 0;
  const double dc = std::cbrt(6 * xvc / PI), rb = .5 * dc;
  if (qc > 1e-9 && tk > 237.15) {
    double xl2p = jmax(0, 2.7e-2 * rho * qc * (.5e20 * std::pow(rb, 3) * dc - .4));
    if (rb > 7.51e-6 && xl2p > 0) {
      double t2s = 3.72 / (1e6 * (rb - 7.5e-6) * rho * qc);
      autoM = xl2p / (t2s * rho);
      double cautn = jmin(.1 * nc / dt, 2 * AA1 * nc * nc * xvc * xvc);
      autoN = jmax(0, jmin(3.5e9 * xl2p / t2s, .5 * cautn));
      if (rho * qr > 1.2 * xl2p && nr > NUMBER_MIN) autoN = nr / (rho * qr) * autoM * rho;
    }
  }
  const double xvr = nr > 0 ? rho * qr / (RHO_W2 * nr) : 0, dv = std::cbrt(6 * xvr / PI), rwrad = dv / 2;
  if (qc > 1e-9 && nr > 0) {
    double rh = rb > 3.5e-6 ? jmax(41e-6, 6.3e-4 / (1e6 * (rb - 3.5e-6))) : 41e-6;
    if (rwrad > rh) {
      accretion = rwrad > 50e-6 ? AA2 * nr * nc * RHO_W2 * xvc * (2 * xvc + xvr) / rho : AA1 * nr * qc * (6 * xvc * xvc + G1 * xvr * xvr);
      accretion = jmin(accretion, .1 * qc / dt);
    }
  }
  double take = (autoM + accretion) * dt;
  if (take > qc) { double s = qc / take; autoM *= s; autoN *= s; accretion *= s; }
  double selfN = 0;
  if (breakup == MORRISON) {
    if (nr > 0) { double dn = dnOf(xvr), ec = dn < 300e-6 ? 1 : 2 - std::exp(2300 * (dn - 300e-6)); selfN = 5.78 * ec * nr * qr * rho; }
  } else {
    bool big = !(dv - 1e-4 <= 1.9e-3);
    double ec0 = big ? 0 : dv < 6.1e-4 ? 1 : std::exp(-2500 * (dv - 6e-4));
    if (nr > 0 && !big) selfN = rwrad >= 50e-6 ? ec0 * AA2 * nr * nr * xvr : ec0 * AA1 * std::pow(nr * xvr, 2) * G1;
    if (breakup == NSSL && nr > 0) selfN -= RAIN_BREAK_FACTOR * (1 - ec0) * std::pow(rho * qr, 2);
  }
  cloud[i] = qc - (autoM + accretion) * dt;
  double qrNew = qr + (autoM + accretion) * dt;
  nr = nr + (autoN - selfN) * dt;
  if (nr < 0) nr = 0;
  double evaporation = 0;
  const double qs = qsatP(tk - 273.15, p);
  if (evaporate && qrNew > RAIN_MIN && nr > 0 && (double)q[i] < qs) {
    double l = 2500837.367 * std::pow(273.15 / tk, .167 + 3.67e-4 * tk), dvap = 2.11e-5 * std::pow(tk / 273.15, 1.94) * (101325 / p);
    double mu = 1.832e-5 * (416.16 / (tk + 120)) * std::pow(tk / 296, 1.5), ka = 2.43e-2 * mu / 1.718e-5, nuKin = mu / rho;
    double fvent = std::cbrt(nuKin / dvap) / std::sqrt(nuKin);
    double fav = l * l / (ka * 461.5 * tk * tk), fbv = 1 / (rho * dvap * qs);
    double fvce = 4 * PI / rho * ((double)q[i] / qs - 1) / (fav + fbv);
    double dn = dnOf(meanVolume(qrNew, nr / rho)), rhovt = std::sqrt(RHO_00 / jmax(.05, rho));
    double vent = .78 + .308 * 1.8273551 * fvent * std::sqrt(841.99666 * rhovt) * std::pow(dn, .9);
    double rate = -fvce * nr * vent * .5 * dn;
    evaporation = jmin(jmin(rate * dt, .1 * qrNew), ((qs - (double)q[i]) / (1 + LV * LV * qs / (CP * 461.5 * tk * tk))));
    if (evaporation > 0) { nr -= nr * evaporation / qrNew; qrNew -= evaporation; q[i] += evaporation; } else evaporation = 0;
  }
  rain[i] = qrNew;
  number[i] = qrNew > RAIN_MIN ? boundedNumber(qrNew, nr / rho, rho) : 0;
  if (!(qrNew > RAIN_MIN)) rain[i] = jmax(0, qrNew);
  return evaporation;
}

// rainNumberChange (:152-159): a loss keeps the mean drop mass; a gain arrives as drops of `meanMass`.
template <class S> void numberChange(Arr<S> rain, Arr<S> number, int i, double before, double rho, double meanMass) {
  double after = rain[i];
  if (!(after > RAIN_MIN)) { number[i] = 0.0; return; }
  double n = number[i];
  if (after < before) number[i] = before > 0 ? n * after / before : n;
  else if (after > before) number[i] = n + (after - before) / jmax(meanMass, RHO_W2 * XV_MIN);
  number[i] = boundedNumber(after, number[i], rho);
}

// exponentialMeanMass (:165-169)
inline double exponentialMeanMass(double q, double n0, double rhoX, double rho) {
  if (!(q > 0)) return 0;
  double lambda = std::pow(PI * rhoX * n0 / (rho * q), .25);
  return rho * q * lambda / n0;
}

}  // namespace r2m
}  // namespace orc
