// Bulk microphysics of one node in FP32: warm rain (Kessler), one-moment Lin ice, snow, graupel and hail, the
// saturation adjustment, secondary ice; each function follows the reference routine it names (file:line) and
// updates the node in the reference's order. theta is held as its departure `thp` from the level's base value `thb`.
// Where the reference reads theta * exner, the Celsius temperature is formed as tcb + thp * exner, tcb = thb * exner
// - 273.15 of the level from FP64: FP32 resolves it to ~1e-6 K (an FP32 kelvin value near 290 K only to 3e-5 K,
// which moves the saturation mixing ratio by ~2e-6 of itself and small condensation amounts by up to a percent).
#pragma once
#include <math.h>
#include <algorithm>
#include <cmath>
#include "sg_common.cuh"

namespace sg {
namespace phys {

constexpr float G = 9.81f, CP = 1004.f, LV = 2.5e6f, RD = 287.05f, RV = 461.5f, EPS = .622f;
constexpr float LF = 3.34e5f, LS = 2.5e6f + 3.34e5f, T0 = 273.15f, T_HOM = 235.15f, CW = 4187.f;
constexpr float CRYSTAL_MASS = 1e-12f, MAX_CRYSTAL_MASS = 9.4e-10f, SPLINTERS = 3.5e8f, MAX_NUCLEATED = 250e3f;
constexpr float KA = 2.43e-2f, PSI = 2.26e-5f, NU = 1.51e-5f;
constexpr float N0S = 3e6f, RHO_S = 100.f, N0G = 4e4f, RHO_G = 400.f, N0R = 8e6f, RHO_W = 1000.f, N0H = 4e4f, RHO_H = 900.f;
constexpr float PI = 3.14159265358979f;
constexpr float GAMMA_3D = 2.5493f, GAMMA_4D = 8.2850f, GAMMA_5D2 = 1.4569f, GAMMA_45 = 11.6317f, GAMMA_35 = 3.3234f, GAMMA_275 = 1.6084f;
// C_S = 152.93 * 0.01^0.75 (src/core/ice.ts:122) and the droplet mass pi/6 * 1000 * (20 um)^3 (:102), evaluated in FP64.
constexpr float C_S = 4.8360712f;
constexpr float SQRT_C_S = 2.1991069f;
constexpr float DROPLET_MASS = 4.18879020e-12f;
constexpr float SC13 = 0.84343267f;  // 0.6^(1/3)

SG_HD float fclamp(float x, float a, float b) { return fmaxf(a, fminf(b, x)); }

struct Node { float thp, thb, tcb, q, cloud, rain, ice, inum, snow, graupel, hail, cold; };
SG_HD float tcOf(const Node& s, float exner) { return s.tcb + s.thp * exner; }

// Saturation about the level's base state. With t = tb + t' (tb = theta_b exner - 273.15 of the level in FP64,
// t' = theta' exner at the node), es(t) = es(tb) (1 + x), x = expm1(A (t - tb) / ((t + B)(tb + B))) for the Bolton
// (A = 17.67 * 243.5, B = 243.5) and Alduchov-Eskridge (A = 22.587 * 273.86, B = 273.86) fits, and
// qs(t) = eps es / (p - es) = qs(tb) (1 + g), g = x (1 + beta) / (1 - beta x), beta = es(tb) / (p - es(tb)): exact
// identities of the reference's formulas. qs(tb) is an FP32 pair hi + lo from FP64, so q - qs = (q - hi) - (lo + hi g)
// keeps the digits that matter near saturation (q - qs ~ 1e-6 of q ~ 1e-2) without FP64 on the device.
struct Level { float exner, p, rho, fallsq, tcb, qw_hi, qw_lo, bw, qi_hi, qi_lo, bi, q0_hi, q0_lo; };
struct Sat { float hi, corr; };                 // qs = hi + corr
SG_HD float satv(Sat a) { return a.hi + a.corr; }
SG_HD float excess(float q, Sat a) { return (q - a.hi) - a.corr; }  // q - qs
SG_HD float satDiff(Sat a, Sat b) { return (a.hi - b.hi) + (a.corr - b.corr); }  // qs_a - qs_b

SG_HD float qsatP(float t, float p) {  // src/core/microphysics.ts:5
  float es = 611.2f * expf(17.67f * t / (t + 243.5f));
  return fclamp(EPS * es / fmaxf(1000.f, p - es), 0.f, .045f);
}
SG_HD float qsatIce(float t, float p) {  // src/core/ice.ts:130-134
  if (t >= 0.f) return qsatP(t, p);
  float es = 611.21f * expf(22.587f * t / (t + 273.86f));
  return fclamp(EPS * es / fmaxf(1000.f, p - es), 0.f, .045f);
}
SG_HD Sat satExpand(float hi, float lo, float beta, float A, float B, float dT, float t, float tcb) {
  const float x = expm1f(A * dT / ((t + B) * (tcb + B)));
  const float g = x * (1.f + beta) / (1.f - beta * x);
  const float v = hi + (lo + hi * g);
  if (!(v < .045f)) return Sat{.045f, 0.f};   // the reference's upper clamp
  return Sat{hi, lo + hi * g};
}
// Water saturation at the node (qsatP of its temperature); the level's base must be valid (hi >= 0), else direct.
SG_HD Sat satWater(const Node& s, const Level& L) {
  const float dT = s.thp * L.exner, t = L.tcb + dT;
  if (!(L.qw_hi >= 0.f)) return Sat{qsatP(t, L.p), 0.f};
  return satExpand(L.qw_hi, L.qw_lo, L.bw, 17.67f * 243.5f, 243.5f, dT, t, L.tcb);
}
// Ice saturation (qsatIce: over water at and above 0 C).
SG_HD Sat satIce(const Node& s, const Level& L) {
  const float dT = s.thp * L.exner, t = L.tcb + dT;
  if (t >= 0.f) return satWater(s, L);
  if (!(L.qi_hi >= 0.f)) return Sat{qsatIce(t, L.p), 0.f};
  return satExpand(L.qi_hi, L.qi_lo, L.bi, 22.587f * 273.86f, 273.86f, dT, t, L.tcb);
}

// Powers with dyadic exponents from correctly rounded square roots and products: within a few ulp of powf at a fraction
// of its cost (the processes below evaluate several a node). x^(1/4), x^(1/8), x^(1/16).
SG_HD float root4(float x) { return sqrtf(sqrtf(x)); }
SG_HD float root8(float x) { return sqrtf(root4(x)); }
SG_HD float root16(float x) { return sqrtf(root8(x)); }
// x^y for x > 0 and a small exponent |y| < 1 (the rain laws, Koenig's growth): exp2(y log2 x). log2f's error (1 ulp of log2 x) enters
// scaled by |y|, so the result stays within ~3e-7 of x^y, at a fraction of powf's cost.
SG_HD float pow_small(float x, float y) { return exp2f(y * log2f(x)); }

// Fall speeds (src/core/microphysics.ts:37, ice.ts:143, graupel.ts:21, hail.ts:102); fallsq = sqrt(rho_ground / rho).
SG_HD float rainFall(float rain, float rho, float fallsq) { return rain > 0.f ? 36.34f * pow_small(.001f * rho * rain, .1364f) * fallsq : 0.f; }
SG_HD float snowFall(float snow, float rho, float fallsq) {
  return snow > 1e-9f ? C_S * GAMMA_4D / 6.f * (1.f / root16(PI * RHO_S * N0S / (rho * snow))) * fallsq : 0.f;
}
SG_HD float fallCoef(float rho, float rhoX) { return sqrtf(4.f * G * rhoX / (3.f * .6f * rho)); }
SG_HD float graupelFall(float x, float rho) { return x > 1e-9f ? fallCoef(rho, RHO_G) * GAMMA_45 / 6.f * (1.f / root8(PI * RHO_G * N0G / (rho * x))) : 0.f; }
SG_HD float hailFall(float x, float rho) { return x > 1e-9f ? fallCoef(rho, RHO_H) * GAMMA_45 / 6.f * (1.f / root8(PI * RHO_H * N0H / (rho * x))) : 0.f; }
SG_HD float hailMaxDiameter(float hail, float rho) {  // src/core/hail.ts:107-111
  if (!(hail > 1e-9f)) return 0.f;
  float lambda = root4(PI * RHO_H * N0H / (rho * hail));
  return fmaxf(0.f, logf(N0H * 10.f / lambda) / lambda);
}

// src/core/microphysics.ts:48-60 (Marshall-Palmer intercept). Returns the evaporated rain.
SG_HD float rainProcesses(Node& s, const Level& L, float dt, bool evaporate) {
  const float tk = tcOf(s, L.exner) + 273.15f, rho = L.rho, p = L.p;
  float qc = s.cloud, qr = s.rain;
  float rate = .001f * fmaxf(0.f, qc - .001f) + (qr > 0.f ? 2.2f * qc * (qr / root8(qr)) : 0.f);
  float production = fminf(qc, rate * dt);
  s.cloud -= production; s.rain += production;
  if (!evaporate || s.rain <= 0.f) return 0.f;         // (the saturation below is only needed to evaporate rain)
  const Sat sw = satWater(s, L);
  const float qs = satv(sw), ex = excess(s.q, sw);     // ex = q - qs
  if (ex >= 0.f) return 0.f;
  float rq = .001f * rho * s.rain, vent = 1.6f + 124.9f * pow_small(rq, .2046f);
  float er = (-ex / qs) * vent * pow_small(rq, .525f) / (.001f * rho * (5.4e5f + 2.55e6f / (p / 100.f * qs)));
  float ev = fminf(fminf(s.rain, er * dt), -ex / (1.f + LV * LV * qs / (CP * RV * tk * tk)));
  s.rain -= ev; s.q += ev;
  return ev;
}
// src/core/microphysics.ts:67-77
SG_HD float saturationAdjust(Node& s, const Level& L) {
  float total = 0.f;
  for (int k = 0; k < 2; k++) {
    const float tk = tcOf(s, L.exner) + 273.15f;
    const Sat sw = satWater(s, L);
    float d = excess(s.q, sw) / (1.f + LV * LV * satv(sw) / (CP * RV * tk * tk));
    if (d < 0.f) d = fmaxf(d, -s.cloud);
    if (d == 0.f) break;
    s.q -= d; s.cloud += d; s.thp += LV / (CP * L.exner) * d; total += d;
  }
  return total;
}
SG_HD float cooperCrystals(float tc) { return tc >= -5.f ? 0.f : fminf(MAX_NUCLEATED, 5.f * expf(.304f * -tc)); }  // src/core/ice.ts:137
// src/core/ice.ts:154-176 (number = the crystal count)
SG_HD float saturationAdjustMixed(Node& s, const Level& L) {
  const float exner = L.exner, heat = LF / (CP * exner);
  if (tcOf(s, exner) >= T_HOM - T0) {
    if (s.ice > 0.f && tcOf(s, exner) > 0.f) {
      float melt = fminf(s.ice, tcOf(s, exner) * CP / LF);
      s.inum *= 1.f - melt / s.ice;
      s.ice -= melt; s.cloud += melt; s.thp -= heat * melt;
    }
    return saturationAdjust(s, L);
  }
  if (s.cloud > 0.f) { s.inum += s.cloud / DROPLET_MASS; s.ice += s.cloud; s.thp += heat * s.cloud; s.cloud = 0.f; }
  float total = 0.f;
  for (int k = 0; k < 2; k++) {
    const float tk = tcOf(s, exner) + T0;
    const Sat si = satIce(s, L);
    float d = excess(s.q, si) / (1.f + LS * LS * satv(si) / (CP * RV * tk * tk));
    if (d < 0.f) d = fmaxf(d, -s.ice);
    if (d == 0.f) break;
    s.q -= d; s.ice += d; s.thp += LS / (CP * exner) * d; total += d;
  }
  return total;
}
SG_HD void freezeRain(Node& s, float exner) {  // src/core/ice.ts:179-183
  float r = s.rain;
  if (r <= 0.f || tcOf(s, exner) >= T_HOM - T0) return;
  s.rain = 0.f; s.graupel += r; s.thp += LF / (CP * exner) * r;
}
SG_HD void settleCrystals(Node& s) {  // src/core/ice.ts:245-248
  float qi = s.ice;
  s.inum = qi > 1e-12f ? fminf(qi / CRYSTAL_MASS, fmaxf(qi / MAX_CRYSTAL_MASS, s.inum)) : 0.f;
}
// Koenig (1971) crystal growth table of the reference (src/core/ice.ts:197-200), as coded there; a device copy in
// constant memory and a host copy for the CPU build of these functions.
#define SG_KOENIG_A1 {.7939e-7f, .7841e-6f, .3369e-5f, .4336e-5f, .5285e-5f, .3728e-5f, .1852e-5f, .2991e-6f, .4248e-6f, .7434e-6f, .1812e-5f, .4394e-5f, .9145e-5f, .1725e-4f, .3348e-4f, \
  .1725e-4f, .9175e-5f, .4412e-5f, .2252e-5f, .9115e-6f, .4876e-6f, .3473e-6f, .4758e-6f, .6306e-6f, .8573e-6f, .7868e-6f, .7192e-6f, .6513e-6f, .5956e-6f, .5333e-6f, .4834e-6f}
#define SG_KOENIG_A2 {.4006f, .4831f, .5320f, .5307f, .5319f, .5249f, .4888f, .3894f, .4047f, .4318f, .4771f, .5183f, .5463f, .5651f, .5813f, \
  .5655f, .5478f, .5203f, .4906f, .4447f, .4126f, .3960f, .4149f, .4320f, .4506f, .4483f, .4460f, .4433f, .4413f, .4382f, .4361f}
#ifdef __CUDACC__
__constant__ float KOENIG_A1_D[31] = SG_KOENIG_A1;
__constant__ float KOENIG_A2_D[31] = SG_KOENIG_A2;
#endif
static const float KOENIG_A1_H[31] = SG_KOENIG_A1;
static const float KOENIG_A2_H[31] = SG_KOENIG_A2;
#ifdef __CUDA_ARCH__
#define KOENIG_A1 KOENIG_A1_D
#define KOENIG_A2 KOENIG_A2_D
#else
#define KOENIG_A1 KOENIG_A1_H
#define KOENIG_A2 KOENIG_A2_H
#endif
SG_HD float koenigGrowth(float tc, float m) {  // src/core/ice.ts:203-206
  float x = fclamp(-tc, 1.f, 31.f) - 1.f; int k = (int)fminf(29.f, floorf(x)); float f = x - (float)k, g = m * 1000.f;
  return 1e-3f * ((1.f - f) * KOENIG_A1[k] * pow_small(g, KOENIG_A2[k]) + f * KOENIG_A1[k + 1] * pow_small(g, KOENIG_A2[k + 1]));
}
// src/core/ice.ts:223-242
SG_HD float iceProcesses(Node& s, const Level& L, float dt) {
  const float exner = L.exner, rho = L.rho;
  float tc = tcOf(s, exner), tk = tc + T0;
  if (tc >= 0.f || tc < T_HOM - T0) return 0.f;
  const Sat si = satIce(s, L);
  const float qsi = satv(si), exi = excess(s.q, si);
  float limit = exi / (1.f + LS * LS * qsi / (CP * RV * tk * tk)), heat = LS / (CP * exner), lacking = cooperCrystals(tc) / rho - s.inum;
  float change = 0.f;
  if (limit > 0.f && lacking > 0.f) { change = fminf(limit, lacking * CRYSTAL_MASS); s.inum += change / CRYSTAL_MASS; }
  float qi = s.ice + change, n = s.inum;
  if (qi > 1e-12f && n > 0.f) {
    if (exi > 0.f) change += fminf(n * koenigGrowth(tc, qi / n) * exi / satDiff(satWater(s, L), si) * dt, limit - change);
    else {
      float a = LS * LS / (KA * RV * tk * tk), b = 1.f / (rho * qsi * PSI);
      float size = cbrtf(6.f * rho * qi / (PI * 900.f * (n * rho)));
      float lost = fminf(qi, n * 2.f * PI * size * (-exi / qsi) / (a + b) * dt);
      change -= lost; s.inum *= 1.f - lost / qi;
    }
  }
  s.ice += change; s.q -= change; s.thp += heat * change;
  float excessIce = s.ice - s.inum * MAX_CRYSTAL_MASS;
  if (excessIce > 0.f) { s.ice -= excessIce; s.snow += excessIce; }
  return change < 0.f ? -heat * change : 0.f;
}
// src/core/ice.ts:266-303 (riming of snow into graupel off, the reference default)
SG_HD float snowProcesses(Node& s, const Level& L, float dt) {
  const float exner = L.exner, rho = L.rho, fallsq = L.fallsq;
  const float tc = tcOf(s, exner), tk = tc + T0, qs = s.snow;
  if (tc < 0.f && s.ice > 0.f) {
    float aut = 1e-3f * expf(.025f * tc) * fmaxf(0.f, s.ice - .001f);
    float moved = fminf(s.ice, aut * dt); s.ice -= moved; s.snow += moved;
  }
  if (qs <= 1e-9f) return 0.f;
  // at the temperature the routine starts with, as the reference evaluates it (the conversion above leaves it)
  const Sat si = tc < 0.f ? satIce(s, L) : Sat{0.f, 0.f};
  float lambda = root4(PI * RHO_S * N0S / (rho * qs));
  float sweep = PI * N0S * C_S * GAMMA_3D / (4.f * (lambda * lambda * lambda * root4(lambda))) * fallsq;
  float vent = N0S * (.78f / (lambda * lambda) + .31f * SC13 * GAMMA_5D2 * SQRT_C_S * sqrtf(fallsq) / sqrtf(NU) * (1.f / (lambda * lambda * sqrtf(lambda) * root8(lambda))));
  float cooling = 0.f;
  if (tc < 0.f) {
    float saci = fminf(s.ice, sweep * expf(.025f * tc) * s.ice * dt); s.ice -= saci; s.snow += saci;
    float sacw = fminf(s.cloud, sweep * s.cloud * dt); s.cloud -= sacw; s.snow += sacw;
    s.thp += LF / (CP * exner) * sacw;
    const float qsi = satv(si), exi = excess(s.q, si);
    float a = LS * LS / (KA * RV * tk * tk), b = 1.f / (rho * qsi * PSI);
    float rate = 2.f * PI * (exi / qsi) * vent / (rho * (a + b));
    float dep = rate > 0.f ? fminf(rate * dt, exi / (1.f + LS * LS * qsi / (CP * RV * tk * tk))) : -fminf(s.snow, -rate * dt);
    s.snow += dep; s.q -= dep; s.thp += LS / (CP * exner) * dep;
    if (dep < 0.f) cooling -= LS / (CP * exner) * dep;
  } else {
    float sacw = fminf(s.cloud, sweep * s.cloud * dt); s.cloud -= sacw; s.rain += sacw;
    float rate = 2.f * PI * KA * tc * vent / (rho * LF) + CW * tc / LF * sweep * s.cloud;
    float melt = fminf(fminf(s.snow, rate * dt), CP * tc / LF);
    s.snow -= melt; s.rain += melt; s.thp -= LF / (CP * exner) * melt; cooling += LF / (CP * exner) * melt;
  }
  return cooling;
}
// src/core/graupel.ts:34-72
SG_HD float graupelProcesses(Node& s, const Level& L, float dt) {
  const float exner = L.exner, rho = L.rho;
  const float tc = tcOf(s, exner), tk = tc + T0, heat = 1.f / (CP * exner);
  // at the starting temperature (the reference's qsatIce(tc, p)); needed only below 0 C when graupel is or becomes
  // present (frozen rain, autoconverted snow)
  const bool needSi = tc < 0.f && (s.graupel > 1e-9f || s.rain > 1e-9f || s.snow > 6e-4f);
  const Sat si = needSi ? satIce(s, L) : Sat{0.f, 0.f};
  float cooling = 0.f;
  if (tc < 0.f) {
    if (s.rain > 1e-9f) {
      float lambdaR = root4(PI * RHO_W * N0R / (rho * s.rain));
      float l2 = lambdaR * lambdaR, l7 = l2 * l2 * l2 * lambdaR;
      float rate = 20.f * PI * PI * 100.f * N0R * RHO_W / rho * (expf(-.66f * tc) - 1.f) / l7;
      float frozen = fminf(s.rain, rate * dt); s.rain -= frozen; s.graupel += frozen; s.thp += LF * heat * frozen;
    }
    float aut = fminf(s.snow, 1e-3f * expf(.09f * tc) * fmaxf(0.f, s.snow - 6e-4f) * dt);
    s.snow -= aut; s.graupel += aut;
  }
  float qg = s.graupel;
  if (qg <= 1e-9f) return 0.f;
  float lambda = root4(PI * RHO_G * N0G / (rho * qg)), a = fallCoef(rho, RHO_G);
  float sweep = PI * N0G * a * GAMMA_35 / (4.f * (lambda * lambda * lambda * sqrtf(lambda)));
  float vent = N0G * (.78f / (lambda * lambda) + .31f * SC13 * GAMMA_275 * sqrtf(a / NU) * (1.f / (lambda * lambda * sqrtf(lambda) * root4(lambda))));
  if (tc < 0.f) {
    float gacw = fminf(s.cloud, sweep * s.cloud * dt), gacr = fminf(s.rain, sweep * s.rain * dt);
    float gaci = fminf(s.ice, sweep * .1f * s.ice * dt), gacs = fminf(s.snow, sweep * expf(.09f * tc) * s.snow * dt);
    s.cloud -= gacw; s.rain -= gacr; s.ice -= gaci; s.snow -= gacs; s.graupel += gacw + gacr + gaci + gacs;
    s.thp += LF * heat * (gacw + gacr);
    const float qsi = satv(si), exi = excess(s.q, si);
    if (exi < 0.f) {
      float aa = LS * LS / (KA * RV * tk * tk), b = 1.f / (rho * qsi * PSI);
      float sub = fminf(fminf(s.graupel, 2.f * PI * (-exi / qsi) * vent / (rho * (aa + b)) * dt), -exi / (1.f + LS * LS * qsi / (CP * RV * tk * tk)));
      s.graupel -= sub; s.q += sub; s.thp -= LS * heat * sub; cooling += LS * heat * sub;
    }
  } else {
    float gacw = fminf(s.cloud, sweep * s.cloud * dt); s.cloud -= gacw; s.rain += gacw;
    float rate = 2.f * PI * KA * tc * vent / (rho * LF) + CW * tc / LF * sweep * (s.cloud + s.rain);
    float melt = fminf(fminf(s.graupel, rate * dt), CP * tc / LF);
    s.graupel -= melt; s.rain += melt; s.thp -= LF * heat * melt; cooling += LF * heat * melt;
  }
  return cooling;
}
// src/core/hail.ts:99, :118-131
SG_HD float ventilationOf(float lambda, float a, float n0) { return n0 * (.78f / (lambda * lambda) + .31f * SC13 * GAMMA_275 * sqrtf(a / NU) * (1.f / (lambda * lambda * sqrtf(lambda) * root4(lambda)))); }
SG_HD float wetGrowth(float lambda, float a, float n0, float tc, float qv, const Level& L, float iceRate) {
  const float rho = L.rho;
  float heat = KA * -tc + LV * PSI * rho * ((L.q0_hi - qv) + L.q0_lo);   // qsatP(0, p) - qv
  return fmaxf(0.f, 2.f * PI * ventilationOf(lambda, a, n0) * heat / (rho * (LF + CW * tc))) + iceRate * (1.f - 2106.f * tc / (LF + CW * tc));
}
// src/core/hail.ts:140-175
SG_HD float hailProcesses(Node& s, const Level& L, float dt) {
  const float exner = L.exner, rho = L.rho;
  const float tc = tcOf(s, exner), tk = tc + T0, heat = 1.f / (CP * exner);
  float cooling = 0.f;
  // wetGrowing(graupel, N0G, RHO_G, ...) (src/core/hail.ts:127-131)
  if (tc < 0.f && s.graupel > 1e-9f) {
    float lambda = root4(PI * RHO_G * N0G / (rho * s.graupel)), a = fallCoef(rho, RHO_G);
    float k = PI * N0G * a * GAMMA_35 / (4.f * (lambda * lambda * lambda * sqrtf(lambda)));
    if (k * (s.cloud + s.rain + .1f * s.ice + expf(.09f * tc) * s.snow) > wetGrowth(lambda, a, N0G, tc, s.q, L, k * (s.ice + s.snow))) {
      float turned = s.graupel * (1.f - expf(-dt / 60.f)); s.graupel -= turned; s.hail += turned;
    }
  }
  float qh = s.hail;
  if (qh <= 1e-9f) return 0.f;
  // at the starting temperature (the reference's qsatIce(tc, p)): the conversion above leaves it
  const Sat si = tc < 0.f ? satIce(s, L) : Sat{0.f, 0.f};
  float lambda = root4(PI * RHO_H * N0H / (rho * qh)), a = fallCoef(rho, RHO_H);
  float k = PI * N0H * a * GAMMA_35 / (4.f * (lambda * lambda * lambda * sqrtf(lambda))), vent = ventilationOf(lambda, a, N0H);
  if (tc < 0.f) {
    float hacw = fminf(s.cloud, k * s.cloud * dt), hacr = fminf(s.rain, k * s.rain * dt), liquid = hacw + hacr;
    float haci = fminf(s.ice, k * .1f * s.ice * dt), hacs = fminf(s.snow, k * expf(.09f * tc) * s.snow * dt), frozen = liquid;
    float wet = wetGrowth(lambda, a, N0H, tc, s.q, L, k * (s.ice + s.snow)) * dt;
    if (liquid + haci + hacs > wet) {
      haci = fminf(s.ice, k * s.ice * dt); hacs = fminf(s.snow, k * s.snow * dt);
      frozen = fminf(liquid, fmaxf(0.f, wet - haci - hacs));
    }
    s.cloud -= hacw; s.rain += liquid - frozen - hacr; s.ice -= haci; s.snow -= hacs; s.hail += frozen + haci + hacs;
    s.thp += LF * heat * frozen;
    const float qsi = satv(si), exi = excess(s.q, si);
    if (exi < 0.f) {
      float aa = LS * LS / (KA * RV * tk * tk), b = 1.f / (rho * qsi * PSI);
      float sub = fminf(fminf(s.hail, 2.f * PI * (-exi / qsi) * vent / (rho * (aa + b)) * dt), -exi / (1.f + LS * LS * qsi / (CP * RV * tk * tk)));
      s.hail -= sub; s.q += sub; s.thp -= LS * heat * sub; cooling += LS * heat * sub;
    }
  } else {
    float hacw = fminf(s.cloud, k * s.cloud * dt); s.cloud -= hacw; s.rain += hacw;
    float rate = 2.f * PI * KA * tc * vent / (rho * LF) + CW * tc / LF * k * (s.cloud + s.rain);
    float melt = fminf(fminf(s.hail, rate * dt), CP * tc / LF);
    s.hail -= melt; s.rain += melt; s.thp -= LF * heat * melt; cooling += LF * heat * melt;
  }
  return cooling;
}
SG_HD float splintering(float tc) { return tc >= -3.f || tc <= -8.f ? 0.f : tc > -5.f ? (-3.f - tc) * .5f : (tc + 8.f) * (1.f / 3.f); }
SG_HD float fragmentsPerKg(float lambda) { return 2.5e13f * 7.f / (lambda * 1000.f * PI / 6.f); }

// The microphysics part of physics(z) (src/core/model.ts:1384-1471), ice or warm. Returns evap (for the water
// budget) through `evapOut`.
SG_HD void microphysics(Node& s, const Level& L, float dt, int flags, float& evapOut) {
  const float exner = L.exner, rho = L.rho;
  float evap = (flags & RF_RAINFORM) ? rainProcesses(s, L, dt, (flags & RF_EVAP) != 0) : 0.f;
  if (evap > 0.f) { float cool = LV / CP / exner * evap; s.thp -= cool; s.cold += cool; }
  float cond;
  if (flags & RF_ICE) {
    freezeRain(s, exner);
    settleCrystals(s);
    s.cold += iceProcesses(s, L, dt);
    float iceBefore = s.ice, cloudBefore = s.cloud;
    s.cold += snowProcesses(s, L, dt);
    float rainBefore = s.rain;
    s.cold += graupelProcesses(s, L, dt);
    float rainFrozen = tcOf(s, exner) < 0.f ? fmaxf(0.f, rainBefore - s.rain) : 0.f;
    s.cold += hailProcesses(s, L, dt);
    if (iceBefore > 0.f) s.inum *= s.ice / iceBefore;
    float splinters = splintering(tcOf(s, exner)) * SPLINTERS * fmaxf(0.f, cloudBefore - s.cloud)
      + (rainFrozen > 0.f ? fragmentsPerKg(root4(PI * RHO_W * N0R / (rho * rainBefore))) * rainFrozen : 0.f);
    if (splinters > 0.f) {
      float fromG = fminf(s.graupel, splinters * CRYSTAL_MASS), fromS = fminf(s.snow, splinters * CRYSTAL_MASS - fromG);
      s.graupel -= fromG; s.snow -= fromS; s.ice += fromG + fromS; s.inum += (fromG + fromS) / CRYSTAL_MASS;
    }
    cond = saturationAdjustMixed(s, L);
    settleCrystals(s);
  } else cond = saturationAdjust(s, L);
  if (cond < 0.f) s.cold -= LV / CP / exner * cond * .14f;
  evapOut = evap;
}

// The per-level saturation bases in FP64 (host side, when a run is created; the CPU tests use the same).
inline Level makeLevel(double thb, double exner, double p, double rho, double rho0) {
  auto split = [](double x, float& hi, float& lo) { hi = (float)x; lo = (float)(x - (double)hi); };
  Level L{};
  L.exner = (float)exner; L.p = (float)p; L.rho = (float)rho; L.fallsq = (float)std::sqrt(rho0 / rho);
  const double tb = thb * exner - 273.15;
  L.tcb = (float)tb;
  auto base = [&](double es, float& hi, float& lo, float& beta) {
    double den = p - es;
    if (!(den > 1000.0)) { hi = -1.f; lo = 0.f; beta = 0.f; return; }   // the reference's floor binds: direct formula
    double qs = .622 * es / den;
    if (!(qs < .045 * 0.999)) { hi = -1.f; lo = 0.f; beta = 0.f; return; }
    split(qs, hi, lo); beta = (float)(es / den);
  };
  base(611.2 * std::exp(17.67 * tb / (tb + 243.5)), L.qw_hi, L.qw_lo, L.bw);
  base(611.21 * std::exp(22.587 * tb / (tb + 273.86)), L.qi_hi, L.qi_lo, L.bi);
  const double es0 = 611.2, q0 = std::min(.045, std::max(0.0, .622 * es0 / std::max(1000.0, p - es0)));
  split(q0, L.q0_hi, L.q0_lo);
  return L;
}

}  // namespace phys
}  // namespace sg
