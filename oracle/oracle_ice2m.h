// TEST INFRASTRUCTURE ONLY — the oracle of two-moment graupel and hail (see oracle_core.h): restates src/core/ice2m.ts
// (after the NSSL scheme: mass, number and particle volume of graupel and of hail; gamma size distributions, the
// Milbrandt-Morrison fall law, Seifert-Beheng collection, wet growth and shedding, melting, graupel into hail, Bigg
// freezing, deposition and sublimation). FP64 arithmetic in JS order; Float32Array stores through Cell<S>.
#pragma once
#include "oracle_core.h"
#include "oracle_rain2m.h"

namespace orc {
namespace i2m {

// gammaFn (:23-30): Lanczos, g 7, nine terms; reflection below 1/2.
inline double gammaFn(double x) {
  if (x < .5) return PI / (std::sin(PI * x) * gammaFn(1 - x));
  static const double c[9] = {.99999999999980993, 676.5203681218851, -1259.1392167224028, 771.32342877765313, -176.61502916214059,
                              12.507343278686905, -.13857109526572012, 9.9843695780195716e-6, 1.5056327351493116e-7};
  x -= 1;
  double a = c[0]; const double t = x + 7.5;
  for (int k = 1; k < 9; k++) a += c[k] / (x + k);
  return std::sqrt(2 * PI) * std::pow(t, x + .5) * std::exp(-t) * a;
}
// upperGamma (:33-38): Q(n, x) = e^-x sum_{k<n} x^k / k!
inline double upperGamma(int n, double x) {
  if (x <= 0) return 1;
  double term = 1, sum = 1;
  for (int k = 1; k < n; k++) { term *= x / k; sum += term; }
  return std::exp(-x) * sum;
}

struct IceClass { double alpha, rhoMin, rhoMax, rhoNone, dMin, dMax; };                    // :41
const IceClass GRAUPEL_2M = {0, 170, 900, 500, .3e-3, 20e-3}, HAIL_2M = {1, 500, 900, 800, .3e-3, 40e-3};  // :42-43
constexpr double HAIL_TIME = 3, SNOW_GRAUPEL = 6e-4, SNOW_GRAUPEL_DENSITY = 250, ICE2M_MIN = 1e-12;  // :47-53

inline double shape3(double a) { return (3 + a) * (2 + a) * (1 + a); }                  // :56
inline double reflectivityFactor(double a) { return (6 + a) * (5 + a) * (4 + a) / shape3(a); }  // :57
inline double densityOf(const IceClass& c, double q, double vol) { return vol > 0 && q > 0 ? jmin(c.rhoMax, jmax(c.rhoMin, q / vol)) : c.rhoNone; }  // :60
inline double meanVolumeOf(const IceClass& c, double q, double n, double rhoX) {          // :63-66
  double lo = PI / 6 * std::pow(c.dMin, 3), hi = PI / 6 * std::pow(c.dMax, 3) / (std::pow(4 + c.alpha, 3) / shape3(c.alpha));
  return jmin(hi, jmax(lo, q / (rhoX * jmax(n, 1e-30))));
}
inline double boundedIceNumber(const IceClass& c, double q, double n, double vol) {         // :69-74
  if (!(q > ICE2M_MIN)) return 0;
  double rhoX = densityOf(c, q, vol);
  if (!(n > 0)) n = q / (rhoX * PI / 6 * 1e-9);
  return q / (rhoX * meanVolumeOf(c, q, n, rhoX));
}
inline double characteristic(const IceClass& c, double xv) { return std::cbrt(6 * xv / PI) / std::cbrt(shape3(c.alpha)); }  // :77

// fallLaw (:80-86): V = a D^b by density, the table interpolated (and extrapolated past its last row).
inline void fallLaw(double rhoX, double& a, double& b) {
  static const double R[9] = {50, 150, 250, 350, 450, 550, 650, 750, 850};
  static const double A[9] = {62.923, 94.122, 114.74, 131.21, 145.26, 157.71, 168.98, 179.36, 189.02};
  static const double B[9] = {.67819, .63789, .62197, .61240, .60572, .60066, .59663, .59330, .59048};
  int k = (int)jmin(7, jmax(0, std::floor((rhoX - 50) / 100)));
  double f = jmax(0, (rhoX - R[k]) / 100);
  a = A[k] + f * (A[k + 1] - A[k]); b = B[k] + f * (B[k + 1] - B[k]);
}
// momentSpeed (:89-93): the k-th-moment-weighted fall speed, at most 70 m/s.
inline double momentSpeed(const IceClass& c, double q, double n, double vol, double rho, int k) {
  if (!(q > ICE2M_MIN) || !(n > 0)) return 0;
  double rhoX = densityOf(c, q, vol), dn = characteristic(c, meanVolumeOf(c, q, n, rhoX)), a, b; fallLaw(rhoX, a, b);
  return jmin(70, std::sqrt(r2m::RHO_00 / jmax(.05, rho)) * a * std::pow(dn, b) * gammaFn(k + 1 + c.alpha + b) / gammaFn(k + 1 + c.alpha));
}
// largestDiameter (:98-105): the diameter past which 5e-4 particles per m3 remain, by bisection of the tail's share.
inline double largestDiameter(const IceClass& c, double q, double n, double vol, double rho) {
  const double thresh = 5e-4, nm3 = rho * n;
  if (!(q > 1e-9) || !(nm3 > thresh)) return 0;
  double rhoX = densityOf(c, q, vol), dn = characteristic(c, meanVolumeOf(c, q, n, rhoX)), target = thresh / nm3;
  double lo = 0, hi = 200;
  for (int k = 0; k < 60; k++) { double mid = (lo + hi) / 2; if (upperGamma(1 + (int)c.alpha, mid) > target) lo = mid; else hi = mid; }
  return (lo + hi) / 2 * dn;
}
// rimerMoments (:111-117): the charging's moments of a class at a node (RimerMoments of charge.ts); false without it.
inline bool rimerMoments(const IceClass& c, double q, double n, double vol, double rho, RimerMoments& m) {
  if (!(q > 1e-9) || !(n > 0)) return false;
  double rhoX = densityOf(c, q, vol), nb = boundedIceNumber(c, q, n, vol), dn = characteristic(c, meanVolumeOf(c, q, nb, rhoX)), a, b;
  fallLaw(rhoX, a, b);
  double nm3 = rho * nb, g = gammaFn(1 + c.alpha), rhovt = std::sqrt(r2m::RHO_00 / jmax(.05, rho));
  m.n = nm3; m.d1 = nm3 * dn * gammaFn(2 + c.alpha) / g; m.d2 = nm3 * dn * dn * gammaFn(3 + c.alpha) / g;
  m.fall = momentSpeed(c, q, nb, vol, rho, 3); m.d2v = rhovt * a * nm3 * std::pow(dn, 2 + b) * gammaFn(3 + c.alpha + b) / g;
  return true;
}

// Seifert-Beheng collection coefficients (:119-141): a class in mass space by (nu, mu); bb = 1/3.
struct MassShape { double nu, mu; };
inline MassShape diameterShape(double alpha) { return {(alpha - 2) / 3, 1.0 / 3}; }
const MassShape DROPLETS = {0, 1};
constexpr double BB = 1.0 / 3;
inline double delbk(MassShape s, int k) {
  double x1 = gammaFn((1 + s.nu) / s.mu), x2 = gammaFn((2 + s.nu) / s.mu), x3 = gammaFn((1 + 2 * BB + k + s.nu) / s.mu);
  return std::pow(x1 / x2, 2 * BB + k) * x3 / x1;
}
inline double delabk(MassShape a, MassShape b, int k) {
  double g1a = gammaFn((1 + a.nu) / a.mu), g2a = gammaFn((2 + a.nu) / a.mu), g1b = gammaFn((1 + b.nu) / b.mu), g2b = gammaFn((2 + b.nu) / b.mu);
  return 2 * std::pow(g1a / g2a, BB) * gammaFn((1 + BB + a.nu) / a.mu) * std::pow(g1b / g2b, BB + k) * gammaFn((1 + BB + k + b.nu) / b.mu) / (g1a * g1b);
}
inline double sweepFactor(MassShape x, MassShape y, double dx, double dy, int k) {
  return delbk(x, 0) * dx * dx + delabk(x, y, k) * dx * dy + delbk(y, k) * dy * dy;
}

// air (:144-151): NSSL's thermodynamic properties.
struct Air { double tc, lv, lf, ls, dv, ka, nuKin, fvent, cw, ci, qss0; };
inline Air air(double tk, double p, double rho) {
  Air t; t.tc = tk - T0;
  t.lv = 2500837.367 * std::pow(T0 / tk, .167 + 3.67e-4 * tk); t.dv = 2.11e-5 * std::pow(tk / T0, 1.94) * (101325 / p);
  double mu = 1.832e-5 * (416.16 / (tk + 120)) * std::pow(tk / 296, 1.5); t.ka = 2.43e-2 * mu / 1.718e-5; t.nuKin = mu / rho;
  t.lf = 333690.6098 + 2030.61425 * t.tc - 10.46708312 * t.tc * t.tc;
  t.cw = t.tc < 0 ? 4203.1548 + 1.30572e-2 * std::pow(t.tc - 35, 2) : 4187; t.ci = (2.118636 + .007371 * t.tc) * 1e3;
  t.ls = t.lv + t.lf; t.fvent = std::cbrt(t.nuKin / t.dv) / std::sqrt(t.nuKin); t.qss0 = 380 / p;
  return t;
}

// rimerAt (:164-169)
struct Rimer { const IceClass* c; double q, n, v, rhoX, xv, dv, dn, vm, a, b; MassShape shape; };
inline bool rimerAt(const IceClass& c, double q, double n, double v, double rho, Rimer& r) {
  if (!(q > ICE2M_MIN)) return false;
  double rhoX = densityOf(c, q, v), nb = boundedIceNumber(c, q, n, v), xv = meanVolumeOf(c, q, nb, rhoX), a, b;
  fallLaw(rhoX, a, b);
  r.c = &c; r.q = q; r.n = nb; r.v = v > 0 ? v : q / rhoX; r.rhoX = rhoX; r.xv = xv; r.dv = std::cbrt(6 * xv / PI);
  r.dn = characteristic(c, xv); r.vm = momentSpeed(c, q, nb, v, rho, 3); r.a = a; r.b = b; r.shape = diameterShape(c.alpha);
  return true;
}
// ventilation (:172-175)
inline double ventilation(const Rimer& r, double fvent, double rho) {
  double al = r.c->alpha;
  return .78 * (1 + al) + .308 * fvent * std::pow(r.dn, .5 + .5 * r.b) * std::sqrt(r.a * std::sqrt(r2m::RHO_00 / jmax(.05, rho))) * gammaFn(2.5 + al + .5 * r.b) / gammaFn(1 + al);
}
// wetOnsetDiameter (:181-193): the Farley-Orville onset of wet growth, fixed point from 5 mm.
inline double wetOnsetDiameter(const Rimer& r, const Air& t, double rho, double qv, double ql, double iceSwept) {
  double h1 = -t.ka * t.tc - t.lv * t.dv * rho * (qv - t.qss0);
  if (!(h1 > 0) || !(ql > 0)) return 0;
  double d = 5e-3;
  for (int k = 0; k < 10; k++) {
    double vth = std::sqrt(r2m::RHO_00 / rho) * r.a * std::pow(d, r.b), x2 = std::cbrt(t.nuKin / t.dv) * std::sqrt(vth * d / t.nuKin);
    double ah = x2 > 1.4 ? .78 + .308 * x2 : 1 + .108 * x2 * x2;
    double den = vth * rho * ((t.lf + t.cw * t.tc) * ql + t.ci * t.tc * iceSwept);
    if (!(den > 0)) return 0;
    d = jmax(5e-3, 8 * ah * h1 / den);
  }
  return d;
}
// shedVolume (:196-205)
inline double shedVolume(const Rimer& r, bool melt) {
  double big = (3 + r.c->alpha) * r.dn, three = PI / 6 * std::pow(3e-3, 3);
  if (melt) {
    double own = jmin(r2m::RHO_W2 * r2m::XV_MAX * 64 / 6, r.rhoX * r.xv) / r2m::RHO_W2, w = jmin(1, jmax(0, (r.dv - 8e-3) / 12e-3));
    return 1 / ((1 - w) / own + w / three);
  }
  const double fac = 4.5;
  return big > 20e-3 ? PI / 6 * std::pow(1.5e-3, 3) / fac : big > 8e-3 ? three / fac : jmin(r2m::XV_MAX * 64 / 6, PI / 6 * r.rhoX / r2m::RHO_W2 * std::pow(big, 3)) / fac;
}

// The node's fields ice2mProcesses reads and writes (Ice2mFields, :154-160).
template <class S> struct Fields {
  Arr<S> theta, q, cloud, ice, iceNumber, snow, rain, rainNumber, graupel, graupelNumber, graupelVolume, hail, hailNumber, hailVolume;
};
struct Result { double cooling; bool wetG, wetH; };

// ice2mProcesses (:211-333)
template <class S> Result processes(const Fields<S>& f, int i, double exner, double p, double rho, double dt) {
  const double tk = (double)f.theta[i] * exner, heat = 1 / (CP * exner);
  const Air t = air(tk, p, rho);
  double cooling = 0; bool wetG = false, wetH = false;
  if (t.tc < 0) {
    if ((double)f.rain[i] > r2m::RAIN_MIN && (double)f.rainNumber[i] > 0) {  // Bigg freezing into graupel (:217-226)
      double nr = f.rainNumber[i], xv = r2m::meanVolume(f.rain[i], nr), k = BIGG_B * (std::exp(-BIGG_A * t.tc) - 1);
      double qf = jmin(f.rain[i], (double)f.rain[i] * k * 20 * xv * dt), nf = jmin(nr, nr * k * xv * dt);
      if (qf > 0) {
        f.rain[i] -= qf; f.rainNumber[i] -= nf;
        f.graupel[i] += qf; f.graupelNumber[i] += nf; f.graupelVolume[i] += qf / 900;
        f.theta[i] += LF * heat * qf;
      }
    }
    if ((double)f.snow[i] > SNOW_GRAUPEL) {  // rimed snow into graupel (:228-234)
      double m = jmin(f.snow[i], 1e-3 * std::exp(.09 * t.tc) * ((double)f.snow[i] - SNOW_GRAUPEL) * dt);
      if (m > 0) {
        double lambda = std::pow(PI * RHO_S * N0S / (rho * (double)f.snow[i]), .25), mean = rho * (double)f.snow[i] * lambda / N0S;
        f.snow[i] -= m; f.graupel[i] += m; f.graupelNumber[i] += m / mean; f.graupelVolume[i] += m / SNOW_GRAUPEL_DENSITY;
      }
    }
  }
  const double nc = r2m::CLOUD_DROPLETS * rho / r2m::RHO_00, dc = (double)f.cloud[i] > 1e-9 ? std::cbrt(6 * rho * (double)f.cloud[i] / (PI * r2m::RHO_W2 * nc)) : 0;
  const double rc = dc / 2, ehw = dc < 2.4e-6 ? 0 : jmin(.9, jmax(0, -.27544 + rc * (.26249e6 + rc * (-1.8896e10 + rc * 4.4626e14))));
  double toHail = 0, toHailN = 0, toHailV = 0, meltLeft = t.tc > 0 ? CP * t.tc / LF : 0;
  const MassShape EXPONENTIAL = diameterShape(0);
  for (int kind = 0; kind < 2; kind++) {
    const bool graupel = kind == 0; const IceClass& c = graupel ? GRAUPEL_2M : HAIL_2M;
    Arr<S> qa = graupel ? f.graupel : f.hail, na = graupel ? f.graupelNumber : f.hailNumber, va = graupel ? f.graupelVolume : f.hailVolume;
    Rimer r;
    if (!rimerAt(c, qa[i], na[i], va[i], rho, r)) { qa[i] = jmax(0, qa[i]); na[i] = 0.0; va[i] = 0.0; continue; }
    const double nm3 = rho * r.n, vent = ventilation(r, t.fvent, rho);
    double qacw = 0, qacr = 0, cacr = 0, qaci = 0, qacs = 0;
    if ((double)f.cloud[i] > 1e-9 && ehw > 0) qacw = jmin(.5 * (double)f.cloud[i] / dt, .25 * PI * ehw * nm3 * (double)f.cloud[i] * r.vm * sweepFactor(r.shape, DROPLETS, r.dv, dc, 1));
    const double nr = f.rainNumber[i];
    if ((double)f.rain[i] > r2m::RAIN_MIN && nr > 0) {
      double xvr = r2m::meanVolume(f.rain[i], nr), dr = std::cbrt(6 * xvr / PI), vr, vrn; r2m::fallSpeeds(f.rain[i], nr, rho, vr, vrn);
      double vt = std::sqrt(std::pow(r.vm - vr, 2) + .04 * r.vm * vr), er = graupel ? jmin(1, std::exp(-40e-6 / dr) * std::exp(-40e-6 / r.dv)) : 1;
      qacr = jmin(.1 * (double)f.rain[i] / dt, .25 * PI * er * nm3 * (double)f.rain[i] * vt * sweepFactor(r.shape, EXPONENTIAL, r.dv, dr, 1));
      cacr = jmin(.1 * nr / dt, .25 * PI * er * nm3 * nr * vt * sweepFactor(r.shape, EXPONENTIAL, r.dv, dr, 0));
    }
    if (t.tc < 0) {
      if ((double)f.ice[i] > 1e-12 && (double)f.iceNumber[i] > 0) {
        double di = std::cbrt(6 * (double)f.ice[i] / (PI * 900 * (double)f.iceNumber[i])), e = graupel ? jmin(1, .1 * std::exp(.1 * t.tc)) : .2;
        qaci = jmin(.1 * (double)f.ice[i] / dt, e * .25 * PI * nm3 * (double)f.ice[i] * r.vm * sweepFactor(r.shape, DROPLETS, r.dv, di, 1));
      }
      if ((double)f.snow[i] > 1e-12) {
        double lambda = std::pow(PI * RHO_S * N0S / (rho * (double)f.snow[i]), .25), ns = N0S / lambda, ds = std::cbrt(6 * rho * (double)f.snow[i] / (PI * RHO_S * ns));
        double e = .5 * std::exp(.09 * t.tc) * (graupel ? jmin(1, jmax(0, r.rhoX - 300) / 300) : 1);
        qacs = jmin(.1 * (double)f.snow[i] / dt, e * .25 * PI * nm3 * (double)f.snow[i] * r.vm * sweepFactor(r.shape, EXPONENTIAL, r.dv, ds, 1));
      }
    }
    double dq = 0, dn = 0, dvol = 0, toRain = 0, toRainN = 0;
    if (t.tc < 0) {
      auto rime = [&](double d, double v) { return jmin(900, jmax(graupel ? 170 : 500, 300 * std::pow(-(.5e6 * d) * (.6 * v) / t.tc, .44))); };
      const double dry = qacw + qacr + qaci + qacs;
      double wet = dry;
      if (tk > 243.15) {
        double fwet1 = 2 * PI * (t.lv * t.dv * rho * (t.qss0 - (double)f.q[i]) - t.ka * t.tc) / (rho * (t.lf + t.cw * t.tc)), fwet2 = 1 - t.ci * t.tc / (t.lf + t.cw * t.tc);
        wet = jmax(0, r.dn * vent * nm3 * fwet1 + fwet2 * (qaci + qacs));
      }
      const double shed = jmin(0, wet - dry); const bool isWet = shed < 0;
      if (graupel) wetG = isWet; else wetH = isWet;
      dq += (dry + shed) * dt;
      toRainN -= cacr * dt;
      if (isWet) {
        dvol += wet / 900 * dt - jmin((1 - r.rhoX / 900) * r.v, wet / 900 * dt);
        toRain += -shed * dt; toRainN += -shed * dt / (r2m::RHO_W2 * shedVolume(r, false));
      } else {
        double rhoCloud = rime(dc, r.vm), rhoRain = rime((double)f.rain[i] > r2m::RAIN_MIN && nr > 0 ? std::cbrt(6 * r2m::meanVolume(f.rain[i], nr) / PI) : 1e-3, r.vm);
        dvol += (qacw / rhoCloud + qacr / rhoRain + (qaci + qacs) / jmax(rhoCloud, 170)) * dt;
      }
      f.cloud[i] -= qacw * dt; f.rain[i] -= qacr * dt; f.ice[i] -= qaci * dt; f.snow[i] -= qacs * dt;
      f.theta[i] += LF * heat * jmax(0, (qacw + qacr) * dt + shed * dt);
      if (graupel && tk > 242 && tk <= 271.15 && r.q > 1e-4 && qacw * dt > 1e-12) {  // graupel into hail (:292-300)
        double d0 = wetOnsetDiameter(r, t, rho, f.q[i], ehw * (double)f.cloud[i] + (double)f.rain[i], jmin(1, .1 * std::exp(.1 * t.tc)) * (double)f.ice[i]);
        if (d0 > 0 && d0 < .15) {
          double ratio = jmin(100, d0 / r.dn), share = jmin(.1, upperGamma(4, ratio) * dt / HAIL_TIME);
          double shareN = upperGamma(4, ratio) > 0 ? share * upperGamma(1, ratio) / upperGamma(4, ratio) : 0;
          double m = share * r.q, nn = jmin(r.n, shareN * r.n);
          if (m > 0) { dq -= m; dn -= nn; dvol -= m / r.rhoX; toHail += m; toHailN += nn; toHailV += m / r.rhoX; }
        }
      }
      const double qsi = qsatIce(t.tc, p), fai = t.ls * t.ls / (t.ka * 461.5 * tk * tk), fbi = 1 / (rho * t.dv * qsi);
      const double rate = 4 * PI / rho * ((double)f.q[i] / qsi - 1) / (fai + fbi) * nm3 * vent * .5 * r.dn;
      if (rate > 0) {
        double m = jmin(rate * dt, jmax(0, ((double)f.q[i] - qsi) / (1 + LS * LS * qsi / (CP * 461.5 * tk * tk))));
        dq += m; dvol += m / r.rhoX; f.q[i] -= m; f.theta[i] += LS * heat * m;
      } else if (rate < 0) {
        double m = jmin3(-rate * dt, .1 * r.q, (qsi - (double)f.q[i]) / (1 + LS * LS * qsi / (CP * 461.5 * tk * tk)));
        if (m > 0) { dq -= m; dn -= r.n * m / r.q; dvol -= m / r.rhoX; f.q[i] += m; f.theta[i] -= LS * heat * m; cooling += LS * heat * m; }
      }
    } else {
      f.cloud[i] -= qacw * dt; toRain += qacw * dt; toRainN += qacw * dt / (r2m::RHO_W2 * shedVolume(r, false));
      double fmlt1 = 2 * PI * (t.lv * t.dv * (t.qss0 - (double)f.q[i]) - t.ka * t.tc / rho) / t.lf, fmlt2 = -t.cw * t.tc / t.lf;
      double rate = jmin(0, fmlt1 * nm3 * vent * r.dn + fmlt2 * (qacr + qacw));
      double m = jmin3(r.q, -rate * dt, meltLeft);
      if (m > 0) {
        meltLeft -= m;
        dq -= m; dn -= jmin(.95 * r.n, r.n * m / r.q); dvol -= m / r.rhoX + (r.rhoX < 900 ? jmin((1 - r.rhoX / 900) * r.v, m / 900) : 0);
        toRain += m; toRainN += m / (r2m::RHO_W2 * shedVolume(r, true));
        f.theta[i] -= LF * heat * m; cooling += LF * heat * m;
      }
    }
    qa[i] = jmax(0, r.q + dq); na[i] = jmax(0, r.n + dn); va[i] = jmax(0, r.v + dvol);
    f.rain[i] += toRain; f.rainNumber[i] = jmax(0, (double)f.rainNumber[i] + toRainN);
  }
  if (toHail > 0) { f.hail[i] += toHail; f.hailNumber[i] += toHailN; f.hailVolume[i] += toHailV; }
  for (int kind = 0; kind < 2; kind++) {  // BOUNDED (:322-325)
    const IceClass& c = kind == 0 ? GRAUPEL_2M : HAIL_2M;
    Arr<S> qa = kind == 0 ? f.graupel : f.hail, na = kind == 0 ? f.graupelNumber : f.hailNumber, va = kind == 0 ? f.graupelVolume : f.hailVolume;
    if (!((double)qa[i] > ICE2M_MIN)) { qa[i] = jmax(0, qa[i]); na[i] = 0.0; va[i] = 0.0; continue; }
    double rhoX = densityOf(c, qa[i], va[i]); va[i] = (double)qa[i] / rhoX; na[i] = boundedIceNumber(c, qa[i], na[i], va[i]);
  }
  if ((double)f.ice[i] < 0) f.ice[i] = 0.0;
  if ((double)f.snow[i] < 0) f.snow[i] = 0.0;
  if ((double)f.cloud[i] < 0) f.cloud[i] = 0.0;
  f.rainNumber[i] = r2m::boundedNumber(f.rain[i], f.rainNumber[i], rho);
  return {cooling, wetG, wetH};
}

}  // namespace i2m
}  // namespace orc
