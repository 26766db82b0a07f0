// Two-moment graupel and hail of one node in FP32 (src/core/ice2m.ts, after the NSSL scheme): mass, number and particle
// volume per kg of air for each class; gamma size distributions in diameter (alpha 0 graupel, 1 hail) with the bounded
// mean particle; the Milbrandt-Morrison fall law a(rho) D^b(rho); collection with the Seifert-Beheng coefficients; wet
// growth and shedding; melting into drops; graupel turning into hail; Bigg freezing of the drops; deposition and
// sublimation. Each function names the routine it follows and keeps its order of operations. The gamma function of a
// run-time argument is CUDA's tgammaf; the Seifert-Beheng coefficients (fixed per pair of classes) are made on the host
// in FP64 and kept in constant memory.
#pragma once
#include "sg_charge.cuh"
#include "sg_rain2m.cuh"

namespace sg {
namespace i2m {

using namespace phys;

// A class (ice2m.ts:41-43): its shape alpha, density bounds and the density without a volume, the bounds of its mean
// particle volume (pi/6 dMin^3 and the mass-weighted diameter dMax, :63-66), (3+a)(2+a)(1+a) and its cube root, the
// reflectivity factor (:57), Gamma(1+a), Gamma(2+a), Gamma(3+a) and Gamma(k+1+a) for k 0, 3, 6 (factorials).
struct IceClass {
  float alpha, rhoMin, rhoMax, rhoNone, xvLo, xvHi, shape3, cbrtShape3, g1, gamma1, gamma2, gamma3, gammaK0, gammaK3, gammaK6;
};
// pi/6 (0.3 mm)^3; pi/6 (20 mm)^3 / (4^3 / 6); pi/6 (40 mm)^3 / (5^3 / 24); cube roots of 6 and 24 (FP64 values)
SG_HD constexpr IceClass GRAUPEL_2M() { return {0.f, 170.f, 900.f, 500.f, 1.41371669e-11f, 3.92699082e-7f, 6.f, 1.81712059f, 20.f, 1.f, 1.f, 2.f, 1.f, 6.f, 720.f}; }
SG_HD constexpr IceClass HAIL_2M() { return {1.f, 500.f, 900.f, 800.f, 1.41371669e-11f, 6.43398175e-6f, 24.f, 2.88449914f, 8.75f, 1.f, 2.f, 6.f, 1.f, 24.f, 5040.f}; }
constexpr float ICE2M_MIN = 1e-12f, HAIL_TIME = 3.f, SNOW_GRAUPEL = 6e-4f, SNOW_GRAUPEL_DENSITY = 250.f;  // :44-53
constexpr float BIGG_B = 100.f, BIGG_A = .66f;                                                         // :45
constexpr float RV_NSSL = 461.5f;

// The Seifert-Beheng sweep coefficients (delbk(x, 0), delabk(x, y, k), delbk(y, k), ice2m.ts:124-141) of graupel and
// hail (class 0, 1) with the cloud droplets for the mass (pair 0), an exponential class for the mass (pair 1) and for
// the number (pair 2).
struct SweepTable { float a[2][3], b[2][3], c[2][3]; };
inline SweepTable sweep_table() {
  struct Shape { double nu, mu; };
  const double bb = 1.0 / 3;
  auto delbk = [&](Shape s, int k) {
    const double x1 = std::tgamma((1 + s.nu) / s.mu), x2 = std::tgamma((2 + s.nu) / s.mu), x3 = std::tgamma((1 + 2 * bb + k + s.nu) / s.mu);
    return std::pow(x1 / x2, 2 * bb + k) * x3 / x1;
  };
  auto delabk = [&](Shape a, Shape b, int k) {
    const double g1a = std::tgamma((1 + a.nu) / a.mu), g2a = std::tgamma((2 + a.nu) / a.mu), g1b = std::tgamma((1 + b.nu) / b.mu), g2b = std::tgamma((2 + b.nu) / b.mu);
    return 2 * std::pow(g1a / g2a, bb) * std::tgamma((1 + bb + a.nu) / a.mu) * std::pow(g1b / g2b, bb + k) * std::tgamma((1 + bb + k + b.nu) / b.mu) / (g1a * g1b);
  };
  SweepTable t{};
  const Shape droplets = {0, 1}, exponential = {-2.0 / 3, bb};
  for (int c = 0; c < 2; c++) {
    const Shape x = {(c - 2.0) / 3, bb};
    const Shape ys[3] = {droplets, exponential, exponential};
    const int ks[3] = {1, 1, 0};
    for (int p = 0; p < 3; p++) { t.a[c][p] = (float)delbk(x, 0); t.b[c][p] = (float)delabk(x, ys[p], ks[p]); t.c[c][p] = (float)delbk(ys[p], ks[p]); }
  }
  return t;
}
#ifdef __CUDACC__
__constant__ SweepTable c_sweep;
#endif
static const SweepTable h_sweep = sweep_table();
SG_HD float sweepFactor(int cls, int pair, float dx, float dy) {  // sweepFactor (:143-149)
#ifdef __CUDA_ARCH__
  const SweepTable& t = c_sweep;
#else
  const SweepTable& t = h_sweep;
#endif
  return t.a[cls][pair] * dx * dx + t.b[cls][pair] * dx * dy + t.c[cls][pair] * dy * dy;
}

SG_HD float densityOf(const IceClass& c, float q, float vol) { return vol > 0.f && q > 0.f ? fminf(c.rhoMax, fmaxf(c.rhoMin, q / vol)) : c.rhoNone; }  // :60
SG_HD float meanVolumeOf(const IceClass& c, float q, float n, float rhoX) { return fminf(c.xvHi, fmaxf(c.xvLo, q / (rhoX * fmaxf(n, 1e-30f)))); }  // :63-66
SG_HD float boundedIceNumber(const IceClass& c, float q, float n, float vol) {  // :69-74
  if (!(q > ICE2M_MIN)) return 0.f;
  const float rhoX = densityOf(c, q, vol);
  if (!(n > 0.f)) n = q / (rhoX * (PI / 6.f * 1e-9f));
  return q / (rhoX * meanVolumeOf(c, q, n, rhoX));
}
SG_HD float characteristic(const IceClass& c, float xv) { return cbrtf(6.f * xv / PI) / c.cbrtShape3; }  // :77
// fallLaw (:80-86): the table (Milbrandt-Morrison's a and b at 50, 150, ... 850 kg/m3) interpolated by density (and
// extrapolated past its last row).
#define SG_MM_A {62.923f, 94.122f, 114.74f, 131.21f, 145.26f, 157.71f, 168.98f, 179.36f, 189.02f}
#define SG_MM_B {.67819f, .63789f, .62197f, .61240f, .60572f, .60066f, .59663f, .59330f, .59048f}
#ifdef __CUDACC__
__constant__ float c_mmA[9] = SG_MM_A, c_mmB[9] = SG_MM_B;
#endif
static const float h_mmA[9] = SG_MM_A, h_mmB[9] = SG_MM_B;
SG_HD void fallLaw(float rhoX, float& a, float& b) {
#ifdef __CUDA_ARCH__
  const float *A = c_mmA, *B = c_mmB;
#else
  const float *A = h_mmA, *B = h_mmB;
#endif
  const int k = (int)fminf(7.f, fmaxf(0.f, floorf((rhoX - 50.f) / 100.f)));
  const float f = fmaxf(0.f, (rhoX - (50.f + 100.f * (float)k)) / 100.f);
  a = A[k] + f * (A[k + 1] - A[k]); b = B[k] + f * (B[k + 1] - B[k]);
}
SG_HD float gammaK(const IceClass& c, int k) { return k == 0 ? c.gammaK0 : k == 3 ? c.gammaK3 : c.gammaK6; }
// momentSpeed (:89-93): the k-th-moment-weighted fall speed (k 0, 3 or 6), at most 70 m/s.
SG_HD float momentSpeed(const IceClass& c, float q, float n, float vol, float rho, int k) {
  if (!(q > ICE2M_MIN) || !(n > 0.f)) return 0.f;
  const float rhoX = densityOf(c, q, vol), dn = characteristic(c, meanVolumeOf(c, q, n, rhoX));
  float a, b; fallLaw(rhoX, a, b);
  return fminf(70.f, sqrtf(r2m::RHO_00 / fmaxf(.05f, rho)) * a * pow_small(dn, b) * tgammaf((float)k + 1.f + c.alpha + b) / gammaK(c, k));
}
// The mass-, number- and reflectivity-weighted speeds together (the three momentSpeed calls of one node).
SG_HD void momentSpeeds(const IceClass& c, float q, float n, float vol, float rho, float& vm, float& vn, float& vz) {
  vm = vn = vz = 0.f;
  if (!(q > ICE2M_MIN) || !(n > 0.f)) return;
  const float rhoX = densityOf(c, q, vol), dn = characteristic(c, meanVolumeOf(c, q, n, rhoX));
  float a, b; fallLaw(rhoX, a, b);
  const float base = sqrtf(r2m::RHO_00 / fmaxf(.05f, rho)) * a * pow_small(dn, b), ab = 1.f + c.alpha + b;
  vn = fminf(70.f, base * tgammaf(ab) / c.gammaK0);
  vm = fminf(70.f, base * tgammaf(ab + 3.f) / c.gammaK3);
  vz = fminf(70.f, base * tgammaf(ab + 6.f) / c.gammaK6);
}
// upperGamma (:33-38) for whole n
SG_HD float upperGamma(int n, float x) {
  if (x <= 0.f) return 1.f;
  float term = 1.f, sum = 1.f;
  for (int k = 1; k < n; k++) { term *= x / (float)k; sum += term; }
  return expf(-x) * sum;
}
// largestDiameter (:98-105): the diameter past which 5e-4 particles per m3 remain (bisection of the tail's share).
SG_HD float largestDiameter(const IceClass& c, float q, float n, float vol, float rho) {
  const float thresh = 5e-4f, nm3 = rho * n;
  if (!(q > 1e-9f) || !(nm3 > thresh)) return 0.f;
  const float rhoX = densityOf(c, q, vol), dn = characteristic(c, meanVolumeOf(c, q, n, rhoX)), target = thresh / nm3;
  float lo = 0.f, hi = 200.f;
  for (int k = 0; k < 60; k++) { const float mid = (lo + hi) / 2.f; if (upperGamma(1 + (int)c.alpha, mid) > target) lo = mid; else hi = mid; }
  return (lo + hi) / 2.f * dn;
}

// rimerMoments (:111-117) as the charging's moments; false without the class (the one-moment moments are taken then).
SG_HD bool rimerMoments(const IceClass& c, float q, float n, float vol, float rho, charge::Moments& m) {
  if (!(q > 1e-9f) || !(n > 0.f)) return false;
  const float rhoX = densityOf(c, q, vol), nb = boundedIceNumber(c, q, n, vol), dn = characteristic(c, meanVolumeOf(c, q, nb, rhoX));
  float a, b; fallLaw(rhoX, a, b);
  const float nm3 = rho * nb, rhovt = sqrtf(r2m::RHO_00 / fmaxf(.05f, rho)), db = pow_small(dn, b);
  m.n = nm3; m.d1 = nm3 * dn * c.gamma2 / c.gamma1; m.d2 = nm3 * dn * dn * c.gamma3 / c.gamma1;
  m.fall = fminf(70.f, rhovt * a * db * tgammaf(4.f + c.alpha + b) / c.gammaK3);
  m.d2v = rhovt * a * nm3 * (dn * dn * db) * tgammaf(3.f + c.alpha + b) / c.gamma1;
  return true;
}

// air (:144-151): NSSL's thermodynamic properties at the node's temperature.
struct Air { float tc, tk, lv, lf, ls, dv, ka, nuKin, fvent, cw, ci, qss0; };
SG_HD Air air(float tc, float p, float rho) {
  Air t; t.tc = tc; const float tk = tc + T0; t.tk = tk;
  t.lv = 2500837.367f * pow_small(T0 / tk, .167f + 3.67e-4f * tk); t.dv = 2.11e-5f * powf(tk / T0, 1.94f) * (101325.f / p);
  const float r = tk / 296.f, mu = 1.832e-5f * (416.16f / (tk + 120.f)) * (r * sqrtf(r));
  t.ka = 2.43e-2f * mu / 1.718e-5f; t.nuKin = mu / rho;
  t.lf = 333690.6098f + 2030.61425f * tc - 10.46708312f * tc * tc;
  t.cw = tc < 0.f ? 4203.1548f + 1.30572e-2f * (tc - 35.f) * (tc - 35.f) : 4187.f; t.ci = (2.118636f + .007371f * tc) * 1e3f;
  t.ls = t.lv + t.lf; t.fvent = cbrtf(t.nuKin / t.dv) / sqrtf(t.nuKin); t.qss0 = 380.f / p;
  return t;
}

// rimerAt (:164-169): a class's state at the node and its derived sizes and speeds.
struct Rimer { float q, n, v, rhoX, xv, dv, dn, vm, a, b; };
SG_HD bool rimerAt(const IceClass& c, float q, float n, float v, float rho, Rimer& r) {
  if (!(q > ICE2M_MIN)) return false;
  const float rhoX = densityOf(c, q, v), nb = boundedIceNumber(c, q, n, v), xv = meanVolumeOf(c, q, nb, rhoX);
  fallLaw(rhoX, r.a, r.b);
  r.q = q; r.n = nb; r.v = v > 0.f ? v : q / rhoX; r.rhoX = rhoX; r.xv = xv; r.dv = cbrtf(6.f * xv / PI);
  r.dn = characteristic(c, xv);
  r.vm = fminf(70.f, sqrtf(r2m::RHO_00 / fmaxf(.05f, rho)) * r.a * pow_small(r.dn, r.b) * tgammaf(4.f + c.alpha + r.b) / c.gammaK3);
  return true;
}
// ventilation (:172-175)
SG_HD float ventilation(const IceClass& c, const Rimer& r, float fvent, float rho) {
  return .78f * (1.f + c.alpha) + .308f * fvent * pow_small(r.dn, .5f + .5f * r.b) * sqrtf(r.a * sqrtf(r2m::RHO_00 / fmaxf(.05f, rho))) *
         tgammaf(2.5f + c.alpha + .5f * r.b) / c.gamma1;
}
// wetOnsetDiameter (:181-193): the Farley-Orville onset of wet growth of one particle, by fixed point from 5 mm.
SG_HD float wetOnsetDiameter(const Rimer& r, const Air& t, float rho, float qv, float ql, float iceSwept) {
  const float h1 = -t.ka * t.tc - t.lv * t.dv * rho * (qv - t.qss0);
  if (!(h1 > 0.f) || !(ql > 0.f)) return 0.f;
  float d = 5e-3f;
  for (int k = 0; k < 10; k++) {
    const float vth = sqrtf(r2m::RHO_00 / rho) * r.a * pow_small(d, r.b), x2 = cbrtf(t.nuKin / t.dv) * sqrtf(vth * d / t.nuKin);
    const float ah = x2 > 1.4f ? .78f + .308f * x2 : 1.f + .108f * x2 * x2;
    const float den = vth * rho * ((t.lf + t.cw * t.tc) * ql + t.ci * t.tc * iceSwept);
    if (!(den > 0.f)) return 0.f;
    d = fmaxf(5e-3f, 8.f * ah * h1 / den);
  }
  return d;
}
// shedVolume (:196-205): the volume of the drops shed (or melted) water falls as.
SG_HD float shedVolume(const IceClass& c, const Rimer& r, bool melt) {
  const float big = (3.f + c.alpha) * r.dn, three = PI / 6.f * 27e-9f;
  if (melt) {
    const float own = fminf(RHO_W * r2m::XV_MAX * 64.f / 6.f, r.rhoX * r.xv) / RHO_W, w = fminf(1.f, fmaxf(0.f, (r.dv - 8e-3f) / 12e-3f));
    return 1.f / ((1.f - w) / own + w / three);
  }
  const float fac = 4.5f;
  return big > 20e-3f ? PI / 6.f * 3.375e-9f / fac : big > 8e-3f ? three / fac : fminf(r2m::XV_MAX * 64.f / 6.f, PI / 6.f * r.rhoX / RHO_W * (big * big * big)) / fac;
}

// The node's number and volume of graupel and hail (their masses are the node's own).
struct Fields { float gn, gv, hn, hv; };

// ice2mProcesses (:211-333): returns the cooling (melting and sublimation, for the cold-pool indicator) and whether
// graupel and hail are in wet growth. The ice saturation is the one at the node's temperature when the call began (the
// reference evaluates everything temperature-dependent once, from that temperature), about the level's base state.
SG_HD float processes(phys::Node& s, float& rn, Fields& f, const phys::Level& L, float dt, bool& wetG, bool& wetH) {
  const float exner = L.exner, rho = L.rho, p = L.p, heat = 1.f / (CP * exner);
  const Air t = air(tcOf(s, exner), p, rho);
  const Sat si = satIce(s, L);
  const float tk = t.tk;
  float cooling = 0.f;
  wetG = wetH = false;
  if (t.tc < 0.f) {
    if (s.rain > r2m::RAIN_MIN && rn > 0.f) {  // Bigg freezing into graupel of 900 kg/m3 (:217-226)
      const float nr = rn, xv = r2m::meanVolume(s.rain, nr), k = BIGG_B * (expf(-BIGG_A * t.tc) - 1.f);
      const float qf = fminf(s.rain, s.rain * k * 20.f * xv * dt), nf = fminf(nr, nr * k * xv * dt);
      if (qf > 0.f) {
        s.rain -= qf; rn -= nf;
        s.graupel += qf; f.gn += nf; f.gv += qf / 900.f;
        s.thp += LF * heat * qf;
      }
    }
    if (s.snow > SNOW_GRAUPEL) {  // rimed snow into graupel (:228-234)
      const float m = fminf(s.snow, 1e-3f * expf(.09f * t.tc) * (s.snow - SNOW_GRAUPEL) * dt);
      if (m > 0.f) {
        const float lambda = root4(PI * RHO_S * N0S / (rho * s.snow)), mean = rho * s.snow * lambda / N0S;
        s.snow -= m; s.graupel += m; f.gn += m / mean; f.gv += m / SNOW_GRAUPEL_DENSITY;
      }
    }
  }
  const float nc = r2m::CLOUD_DROPLETS * rho / r2m::RHO_00, dc = s.cloud > 1e-9f ? cbrtf(6.f * rho * s.cloud / (PI * RHO_W * nc)) : 0.f;
  const float rc = dc / 2.f, ehw = dc < 2.4e-6f ? 0.f : fminf(.9f, fmaxf(0.f, -.27544f + rc * (.26249e6f + rc * (-1.8896e10f + rc * 4.4626e14f))));
  float toHail = 0.f, toHailN = 0.f, toHailV = 0.f, meltLeft = t.tc > 0.f ? CP * t.tc / LF : 0.f;
#pragma unroll 1
  for (int kind = 0; kind < 2; kind++) {
    const bool graupel = kind == 0;
    const IceClass c = graupel ? GRAUPEL_2M() : HAIL_2M();
    float& qa = graupel ? s.graupel : s.hail;
    float& na = graupel ? f.gn : f.hn;
    float& va = graupel ? f.gv : f.hv;
    Rimer r;
    if (!rimerAt(c, qa, na, va, rho, r)) { qa = fmaxf(0.f, qa); na = 0.f; va = 0.f; continue; }
    const float nm3 = rho * r.n, vent = ventilation(c, r, t.fvent, rho);
    float qacw = 0.f, qacr = 0.f, cacr = 0.f, qaci = 0.f, qacs = 0.f;
    if (s.cloud > 1e-9f && ehw > 0.f) qacw = fminf(.5f * s.cloud / dt, .25f * PI * ehw * nm3 * s.cloud * r.vm * sweepFactor(kind, 0, r.dv, dc));
    const float nr = rn;
    if (s.rain > r2m::RAIN_MIN && nr > 0.f) {
      const float xvr = r2m::meanVolume(s.rain, nr), dr = cbrtf(6.f * xvr / PI);
      float vr, vrn, vrz; r2m::fallSpeeds(s.rain, nr, rho, vr, vrn, vrz);
      const float dvr = r.vm - vr, vt = sqrtf(dvr * dvr + .04f * r.vm * vr);
      const float er = graupel ? fminf(1.f, expf(-40e-6f / dr) * expf(-40e-6f / r.dv)) : 1.f;
      qacr = fminf(.1f * s.rain / dt, .25f * PI * er * nm3 * s.rain * vt * sweepFactor(kind, 1, r.dv, dr));
      cacr = fminf(.1f * nr / dt, .25f * PI * er * nm3 * nr * vt * sweepFactor(kind, 2, r.dv, dr));
    }
    if (t.tc < 0.f) {
      if (s.ice > 1e-12f && s.inum > 0.f) {
        const float di = cbrtf(6.f * s.ice / (PI * 900.f * s.inum)), e = graupel ? fminf(1.f, .1f * expf(.1f * t.tc)) : .2f;
        qaci = fminf(.1f * s.ice / dt, e * .25f * PI * nm3 * s.ice * r.vm * sweepFactor(kind, 0, r.dv, di));
      }
      if (s.snow > 1e-12f) {
        const float lambda = root4(PI * RHO_S * N0S / (rho * s.snow)), ns = N0S / lambda, ds = cbrtf(6.f * rho * s.snow / (PI * RHO_S * ns));
        const float e = .5f * expf(.09f * t.tc) * (graupel ? fminf(1.f, fmaxf(0.f, r.rhoX - 300.f) / 300.f) : 1.f);
        qacs = fminf(.1f * s.snow / dt, e * .25f * PI * nm3 * s.snow * r.vm * sweepFactor(kind, 1, r.dv, ds));
      }
    }
    float dq = 0.f, dn = 0.f, dvol = 0.f, toRain = 0.f, toRainN = 0.f;
    if (t.tc < 0.f) {
      const float rimeMin = graupel ? 170.f : 500.f;
      auto rime = [&](float d, float v) { return fminf(900.f, fmaxf(rimeMin, 300.f * pow_small(-(.5e6f * d) * (.6f * v) / t.tc, .44f))); };
      const float dry = qacw + qacr + qaci + qacs;
      float wet = dry;
      if (tk > 243.15f) {
        const float fwet1 = 2.f * PI * (t.lv * t.dv * rho * (t.qss0 - s.q) - t.ka * t.tc) / (rho * (t.lf + t.cw * t.tc)), fwet2 = 1.f - t.ci * t.tc / (t.lf + t.cw * t.tc);
        wet = fmaxf(0.f, r.dn * vent * nm3 * fwet1 + fwet2 * (qaci + qacs));
      }
      const float shed = fminf(0.f, wet - dry);
      const bool isWet = shed < 0.f;
      if (graupel) wetG = isWet; else wetH = isWet;
      dq += (dry + shed) * dt;
      toRainN -= cacr * dt;
      if (isWet) {
        dvol += wet / 900.f * dt - fminf((1.f - r.rhoX / 900.f) * r.v, wet / 900.f * dt);
        toRain += -shed * dt; toRainN += -shed * dt / (RHO_W * shedVolume(c, r, false));
      } else {
        const float rhoCloud = rime(dc, r.vm), rhoRain = rime(s.rain > r2m::RAIN_MIN && nr > 0.f ? cbrtf(6.f * r2m::meanVolume(s.rain, nr) / PI) : 1e-3f, r.vm);
        dvol += (qacw / rhoCloud + qacr / rhoRain + (qaci + qacs) / fmaxf(rhoCloud, 170.f)) * dt;
      }
      s.cloud -= qacw * dt; s.rain -= qacr * dt; s.ice -= qaci * dt; s.snow -= qacs * dt;
      s.thp += LF * heat * fmaxf(0.f, (qacw + qacr) * dt + shed * dt);
      if (graupel && tk > 242.f && tk <= 271.15f && r.q > 1e-4f && qacw * dt > 1e-12f) {  // graupel into hail (:292-300)
        const float d0 = wetOnsetDiameter(r, t, rho, s.q, ehw * s.cloud + s.rain, fminf(1.f, .1f * expf(.1f * t.tc)) * s.ice);
        if (d0 > 0.f && d0 < .15f) {
          const float ratio = fminf(100.f, d0 / r.dn), q4 = upperGamma(4, ratio), share = fminf(.1f, q4 * dt / HAIL_TIME);
          const float shareN = q4 > 0.f ? share * upperGamma(1, ratio) / q4 : 0.f;
          const float m = share * r.q, nn = fminf(r.n, shareN * r.n);
          if (m > 0.f) { dq -= m; dn -= nn; dvol -= m / r.rhoX; toHail += m; toHailN += nn; toHailV += m / r.rhoX; }
        }
      }
      // deposition and sublimation over ice (:302-311); q - qsi about the level's base state
      const float qsi = satv(si), fai = t.ls * t.ls / (t.ka * RV_NSSL * tk * tk), fbi = 1.f / (rho * t.dv * qsi);
      const float rate = 4.f * PI / rho * (excess(s.q, si) / qsi) / (fai + fbi) * nm3 * vent * .5f * r.dn;
      const float lim = 1.f + LS * LS * qsi / (CP * RV_NSSL * tk * tk);
      if (rate > 0.f) {
        const float m = fminf(rate * dt, fmaxf(0.f, excess(s.q, si) / lim));
        dq += m; dvol += m / r.rhoX; s.q -= m; s.thp += LS * heat * m;
      } else if (rate < 0.f) {
        const float m = fminf(fminf(-rate * dt, .1f * r.q), -excess(s.q, si) / lim);
        if (m > 0.f) { dq -= m; dn -= r.n * m / r.q; dvol -= m / r.rhoX; s.q += m; s.thp -= LS * heat * m; cooling += LS * heat * m; }
      }
    } else {
      s.cloud -= qacw * dt; toRain += qacw * dt; toRainN += qacw * dt / (RHO_W * shedVolume(c, r, false));
      const float fmlt1 = 2.f * PI * (t.lv * t.dv * (t.qss0 - s.q) - t.ka * t.tc / rho) / t.lf, fmlt2 = -t.cw * t.tc / t.lf;
      const float rate = fminf(0.f, fmlt1 * nm3 * vent * r.dn + fmlt2 * (qacr + qacw));
      const float m = fminf(fminf(r.q, -rate * dt), meltLeft);
      if (m > 0.f) {
        meltLeft -= m;
        dq -= m; dn -= fminf(.95f * r.n, r.n * m / r.q); dvol -= m / r.rhoX + (r.rhoX < 900.f ? fminf((1.f - r.rhoX / 900.f) * r.v, m / 900.f) : 0.f);
        toRain += m; toRainN += m / (RHO_W * shedVolume(c, r, true));
        s.thp -= LF * heat * m; cooling += LF * heat * m;
      }
    }
    qa = fmaxf(0.f, r.q + dq); na = fmaxf(0.f, r.n + dn); va = fmaxf(0.f, r.v + dvol);
    s.rain += toRain; rn = fmaxf(0.f, rn + toRainN);
  }
  if (toHail > 0.f) { s.hail += toHail; f.hn += toHailN; f.hv += toHailV; }
  // BOUNDED (:322-325): the volume at the bounded density, the number bounded
  if (!(s.graupel > ICE2M_MIN)) { s.graupel = fmaxf(0.f, s.graupel); f.gn = 0.f; f.gv = 0.f; }
  else { f.gv = s.graupel / densityOf(GRAUPEL_2M(), s.graupel, f.gv); f.gn = boundedIceNumber(GRAUPEL_2M(), s.graupel, f.gn, f.gv); }
  if (!(s.hail > ICE2M_MIN)) { s.hail = fmaxf(0.f, s.hail); f.hn = 0.f; f.hv = 0.f; }
  else { f.hv = s.hail / densityOf(HAIL_2M(), s.hail, f.hv); f.hn = boundedIceNumber(HAIL_2M(), s.hail, f.hn, f.hv); }
  if (s.ice < 0.f) s.ice = 0.f;
  if (s.snow < 0.f) s.snow = 0.f;
  if (s.cloud < 0.f) s.cloud = 0.f;
  rn = r2m::boundedNumber(s.rain, rn, rho);
  return cooling;
}

// The microphysics of physics(z) with two-moment rain, graupel and hail (src/core/model.ts:1391-1452): the two-moment
// rain processes, the freezing (its frozen drops become as many graupel particles of 900 kg/m3, :1404), the crystals,
// the snow, then the two-moment graupel and hail processes instead of the one-moment ones (:1421-1426); the drop number
// follows the freezing and the snow (:1405-1418). The one-moment snow makes no graupel (RIMED_SNOW_TO_GRAUPEL off), so
// :1417 never applies.
SG_HD void microphysics(phys::Node& s, float& rn, Fields& f, const phys::Level& L, float dt, int flags, int breakup, float& evapOut, bool& wetG, bool& wetH) {
  const float exner = L.exner, rho = L.rho;
  float evap = (flags & RF_RAINFORM) ? r2m::processes(s, rn, L, dt, breakup, (flags & RF_EVAP) != 0) : 0.f;
  if (evap > 0.f) { const float cool = LV / CP / exner * evap; s.thp -= cool; s.cold += cool; }
  float rainMark = s.rain;
  const float frozenDrops = rn, graupelMark = s.graupel;
  freezeRain(s, exner);
  if (s.graupel > graupelMark) { f.gn += rainMark > 0.f ? frozenDrops * (1.f - s.rain / rainMark) : 0.f; f.gv += (s.graupel - graupelMark) / 900.f; }
  r2m::numberChange(s, rn, rainMark, rho, 0.f); rainMark = s.rain;
  settleCrystals(s);
  s.cold += iceProcesses(s, L, dt);
  const float iceBefore = s.ice, cloudBefore = s.cloud;
  const float snowMass = r2m::exponentialMeanMass(s.snow, N0S, RHO_S, rho);
  s.cold += snowProcesses(s, L, dt);
  r2m::numberChange(s, rn, rainMark, rho, snowMass);
  const float rainBefore = s.rain;
  s.cold += processes(s, rn, f, L, dt, wetG, wetH);
  const float rainFrozen = tcOf(s, exner) < 0.f ? fmaxf(0.f, rainBefore - s.rain) : 0.f;
  if (iceBefore > 0.f) s.inum *= s.ice / iceBefore;
  const float splinters = splintering(tcOf(s, exner)) * SPLINTERS * fmaxf(0.f, cloudBefore - s.cloud)
    + (rainFrozen > 0.f ? fragmentsPerKg(root4(PI * RHO_W * N0R / (rho * rainBefore))) * rainFrozen : 0.f);
  if (splinters > 0.f) {
    const float fromG = fminf(s.graupel, splinters * CRYSTAL_MASS), fromS = fminf(s.snow, splinters * CRYSTAL_MASS - fromG);
    s.graupel -= fromG; s.snow -= fromS; s.ice += fromG + fromS; s.inum += (fromG + fromS) / CRYSTAL_MASS;
  }
  const float cond = saturationAdjustMixed(s, L);
  settleCrystals(s);
  if (cond < 0.f) s.cold -= LV / CP / exner * cond * .14f;
  evapOut = evap;
}

}  // namespace i2m
}  // namespace sg
