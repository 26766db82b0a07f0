// Two-moment rain of one node in FP32 (src/core/rain2m.ts, after the NSSL scheme): rain mass and drop number per kg,
// the drops' fall speeds, the warm-rain processes (autoconversion, accretion, self-collection and its breakup,
// evaporation) and the number's bookkeeping when the ice processes take or give rain, in the reference's order
// (src/core/model.ts:1391-1435). Each function names the routine it follows.
#pragma once
#include "sg_physics.cuh"

namespace sg {
namespace r2m {

using namespace phys;
// rain2m.ts:11-35, the volumes evaluated in FP64: pi/6 (80 um)^3 and pi/6 (6 mm)^3 / (64/6)
constexpr float RHO_00 = 1.225f, XV_MIN = 2.68082573e-13f, XV_MAX = 1.06028752e-8f;
constexpr float CLOUD_DROPLETS = .6e9f, AA1 = 9.44e15f, AA2 = 5.78e3f, G1 = 20.f, VT_A = 10.f, VT_B = 516.575f;
constexpr float RAIN_BREAK_FACTOR = 1e6f, RAIN_MIN = 1e-12f, NUMBER_MIN = 1e-8f;
// pi/6 (120 um)^3 and pi/6 (4 um)^3 (the cloud droplet's volume bounds, :82), (6 / (pi rho_w))^2 (:963)
constexpr float XVC_MAX = 9.04778684e-13f, XVC_MIN = 3.35103216e-17f, K6 = 3.64756353e-6f;
enum Breakup { NONE = 0, NSSL = 1, MORRISON = 2 };

SG_HD float meanVolume(float q, float n) { return fminf(XV_MAX, fmaxf(XV_MIN, q / (RHO_W * n))); }   // :38
SG_HD float dnOf(float xv) { return cbrtf(xv / PI); }                                                 // :41
SG_HD float boundedNumber(float q, float n, float rho) {                                              // :47-51
  if (!(q > RAIN_MIN)) return 0.f;
  if (!(n > NUMBER_MIN)) { const float lambda = root4(PI * RHO_W * 8e6f / (rho * q)); n = 8e6f / lambda / rho; }
  return q / (RHO_W * meanVolume(q, n));
}
// fallSpeeds and fallSpeedZ (:57-67): mass-, number- and reflectivity-weighted speeds, 10 (1 - (1 + 516.575 Dn)^-k).
SG_HD void fallSpeeds(float q, float n, float rho, float& vm, float& vn, float& vz) {
  if (!(q > RAIN_MIN) || !(n > NUMBER_MIN)) { vm = vn = vz = 0.f; return; }
  const float dn = dnOf(meanVolume(q, n)), r = sqrtf(RHO_00 / fmaxf(.05f, rho)), x = 1.f + VT_B * dn, ix = 1.f / x;
  const float ix2 = ix * ix, ix4 = ix2 * ix2;
  vm = r * VT_A * (1.f - ix4); vn = r * VT_A * (1.f - ix); vz = r * VT_A * (1.f - ix4 * ix2 * ix);
}

// rain2mProcesses (:76-146) on the node; returns the evaporated rain (the caller cools the air).
SG_HD float processes(phys::Node& s, float& number, const phys::Level& L, float dt, int breakup, bool evaporate) {
  const float rho = L.rho, tk = tcOf(s, L.exner) + T0, qc = s.cloud, qr = s.rain;
  // neither cloud water nor rain: nothing forms, collects or evaporates; the reference's arithmetic leaves the rain as
  // it is (negative tails to zero) and the number zero
  if (!(qc > 1e-9f) && !(qr > RAIN_MIN)) { s.rain = fmaxf(0.f, qr); number = 0.f; return 0.f; }
  float nr = qr > RAIN_MIN ? boundedNumber(qr, number, rho) * rho : 0.f;
  float autoM = 0.f, autoN = 0.f, accretion = 0.f;
  const float nc = CLOUD_DROPLETS * rho / RHO_00;
  const float xvc = qc > 1e-9f ? fminf(XVC_MAX, fmaxf(XVC_MIN, rho * qc / (RHO_W * nc))) : 0.f;
  const float dc = cbrtf(6.f * xvc / PI), rb = .5f * dc;
  if (qc > 1e-9f && tk > 237.15f) {
    const float xl2p = fmaxf(0.f, 2.7e-2f * rho * qc * (.5e20f * rb * rb * rb * dc - .4f));
    if (rb > 7.51e-6f && xl2p > 0.f) {
      const float t2s = 3.72f / (1e6f * (rb - 7.5e-6f) * rho * qc);
      autoM = xl2p / (t2s * rho);
      const float cautn = fminf(.1f * nc / dt, 2.f * AA1 * nc * nc * xvc * xvc);
      autoN = fmaxf(0.f, fminf(3.5e9f * xl2p / t2s, .5f * cautn));
      if (rho * qr > 1.2f * xl2p && nr > NUMBER_MIN) autoN = nr / (rho * qr) * autoM * rho;
    }
  }
  const float xvr = nr > 0.f ? rho * qr / (RHO_W * nr) : 0.f, dv = cbrtf(6.f * xvr / PI), rwrad = dv / 2.f;
  if (qc > 1e-9f && nr > 0.f) {
    const float rh = rb > 3.5e-6f ? fmaxf(41e-6f, 6.3e-4f / (1e6f * (rb - 3.5e-6f))) : 41e-6f;
    if (rwrad > rh) {
      accretion = rwrad > 50e-6f ? AA2 * nr * nc * RHO_W * xvc * (2.f * xvc + xvr) / rho : AA1 * nr * qc * (6.f * xvc * xvc + G1 * xvr * xvr);
      accretion = fminf(accretion, .1f * qc / dt);
    }
  }
  const float take = (autoM + accretion) * dt;
  if (take > qc) { const float f = qc / take; autoM *= f; autoN *= f; accretion *= f; }
  float selfN = 0.f;
  if (breakup == MORRISON) {
    if (nr > 0.f) { const float dn = dnOf(xvr), ec = dn < 300e-6f ? 1.f : 2.f - expf(2300.f * (dn - 300e-6f)); selfN = 5.78f * ec * nr * qr * rho; }
  } else {
    const bool big = !(dv - 1e-4f <= 1.9e-3f);
    const float ec0 = big ? 0.f : dv < 6.1e-4f ? 1.f : expf(-2500.f * (dv - 6e-4f));
    if (nr > 0.f && !big) selfN = rwrad >= 50e-6f ? ec0 * AA2 * nr * nr * xvr : ec0 * AA1 * (nr * xvr) * (nr * xvr) * G1;
    if (breakup == NSSL && nr > 0.f) selfN -= RAIN_BREAK_FACTOR * (1.f - ec0) * (rho * qr) * (rho * qr);
  }
  s.cloud = qc - (autoM + accretion) * dt;
  float qrNew = qr + (autoM + accretion) * dt;
  nr = nr + (autoN - selfN) * dt;
  if (nr < 0.f) nr = 0.f;
  float evaporation = 0.f;
  const float qs = qsatP(tk - T0, L.p);
  if (evaporate && qrNew > RAIN_MIN && nr > 0.f && s.q < qs) {
    const float l = 2500837.367f * powf(T0 / tk, .167f + 3.67e-4f * tk), dvap = 2.11e-5f * powf(tk / T0, 1.94f) * (101325.f / L.p);
    const float mu = 1.832e-5f * (416.16f / (tk + 120.f)) * powf(tk / 296.f, 1.5f), ka = 2.43e-2f * mu / 1.718e-5f, nuKin = mu / rho;
    const float fvent = cbrtf(nuKin / dvap) / sqrtf(nuKin);
    const float fav = l * l / (ka * RV * tk * tk), fbv = 1.f / (rho * dvap * qs);
    const float fvce = 4.f * PI / rho * (s.q / qs - 1.f) / (fav + fbv);
    const float dn = dnOf(meanVolume(qrNew, nr / rho)), rhovt = sqrtf(RHO_00 / fmaxf(.05f, rho));
    const float vent = .78f + .308f * 1.8273551f * fvent * sqrtf(841.99666f * rhovt) * powf(dn, .9f);
    const float rate = -fvce * nr * vent * .5f * dn;
    evaporation = fminf(fminf(rate * dt, .1f * qrNew), (qs - s.q) / (1.f + LV * LV * qs / (CP * RV * tk * tk)));
    if (evaporation > 0.f) { nr -= nr * evaporation / qrNew; qrNew -= evaporation; s.q += evaporation; } else evaporation = 0.f;
  }
  s.rain = qrNew;
  number = qrNew > RAIN_MIN ? boundedNumber(qrNew, nr / rho, rho) : 0.f;
  if (!(qrNew > RAIN_MIN)) s.rain = fmaxf(0.f, qrNew);
  return evaporation;
}

// rainNumberChange (:152-159): a loss keeps the mean drop mass, a gain arrives as drops of meanMass.
SG_HD void numberChange(const phys::Node& s, float& number, float before, float rho, float meanMass) {
  const float after = s.rain;
  if (!(after > RAIN_MIN)) { number = 0.f; return; }
  if (after < before) number = before > 0.f ? number * after / before : number;
  else if (after > before) number = number + (after - before) / fmaxf(meanMass, RHO_W * XV_MIN);
  number = boundedNumber(after, number, rho);
}
// exponentialMeanMass (:165-169)
SG_HD float exponentialMeanMass(float q, float n0, float rhoX, float rho) {
  if (!(q > 0.f)) return 0.f;
  const float lambda = root4(PI * rhoX * n0 / (rho * q));
  return rho * q * lambda / n0;
}

// The microphysics of physics(z) with two-moment rain (src/core/model.ts:1391-1471): its processes instead of Kessler's,
// the drop number following the rain the freezing, snow, graupel and hail take or give; the rest as phys::microphysics.
SG_HD void microphysics(phys::Node& s, float& number, const phys::Level& L, float dt, int flags, int breakup, float& evapOut) {
  const float exner = L.exner, rho = L.rho;
  float evap = (flags & RF_RAINFORM) ? processes(s, number, L, dt, breakup, (flags & RF_EVAP) != 0) : 0.f;
  if (evap > 0.f) { float cool = LV / CP / exner * evap; s.thp -= cool; s.cold += cool; }
  float cond;
  if (flags & RF_ICE) {
    float rainMark = s.rain;
    freezeRain(s, exner);
    numberChange(s, number, rainMark, rho, 0.f); rainMark = s.rain;
    settleCrystals(s);
    s.cold += iceProcesses(s, L, dt);
    float iceBefore = s.ice, cloudBefore = s.cloud;
    const float snowMass = exponentialMeanMass(s.snow, N0S, RHO_S, rho);
    s.cold += snowProcesses(s, L, dt);
    numberChange(s, number, rainMark, rho, snowMass); rainMark = s.rain;
    float rainBefore = s.rain;
    const float graupelMass = exponentialMeanMass(s.graupel, N0G, RHO_G, rho);
    s.cold += graupelProcesses(s, L, dt);
    numberChange(s, number, rainMark, rho, graupelMass); rainMark = s.rain;
    float rainFrozen = tcOf(s, exner) < 0.f ? fmaxf(0.f, rainBefore - s.rain) : 0.f;
    const float hailMass = exponentialMeanMass(s.hail, N0H, RHO_H, rho);
    s.cold += hailProcesses(s, L, dt);
    numberChange(s, number, rainMark, rho, hailMass);
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

}  // namespace r2m
}  // namespace sg
