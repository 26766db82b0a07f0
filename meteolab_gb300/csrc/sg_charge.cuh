// Electrification of one node in FP32 (src/core/charge.ts, src/core/takahashi.ts): the charge moved with the water
// between its four carriers, the non-inductive graupel-crystal charging of the Takahashi scheme (the reference's default,
// CHARGING_SCHEME 'tak') and the inductive charging in the vertical field. Each function follows the reference routine
// it names (file:line) in the reference's order of operations; the physics kernel calls them after the microphysics.
#pragma once
#include "sg_physics.cuh"
#include "sg_takahashi.h"

namespace sg {
namespace charge {

using namespace phys;
constexpr float EPSILON0 = 8.8541878128e-12f;       // src/core/electric.ts:6
constexpr float COLLECTION_EFFICIENCY = .6f, CHARGING_SPEED = 6.f, CRYSTAL_LO = 20e-6f, CRYSTAL_HI = 300e-6f;  // charge.ts:34,42,88
constexpr float TAK_RATE_MAX = 3e-9f, DROPLET_REBOUND = .01f, DROPLET_SIZE = 20e-6f, CONTACT_COS = .5f;     // :154,:184
// pi^4 / 8 and pi^3 / 24 (charge.ts:195, :199), evaluated in FP64
constexpr float PI4_8 = 12.176136f, PI3_24 = 1.2919282f;
// the droplet volume pi/6 (20 um)^3 times the water density (charge.ts:189)
constexpr float DROPLET_KG = 4.18879020e-12f;

#ifdef __CUDACC__
__constant__ float c_takLwc[SG_TAKAHASHI_ROWS] = SG_TAKAHASHI_LWC;
__constant__ float c_takTable[SG_TAKAHASHI_ROWS][SG_TAKAHASHI_COLS] = SG_TAKAHASHI_TABLE;
#endif
static const float h_takLwc[SG_TAKAHASHI_ROWS] = SG_TAKAHASHI_LWC;
static const float h_takTable[SG_TAKAHASHI_ROWS][SG_TAKAHASHI_COLS] = SG_TAKAHASHI_TABLE;
SG_HD float takLwc(int r) {
#ifdef __CUDA_ARCH__
  return c_takLwc[r];
#else
  return h_takLwc[r];
#endif
}
SG_HD float takEntry(int r, int c) {
#ifdef __CUDA_ARCH__
  return c_takTable[r][c];
#else
  return h_takTable[r][c];
#endif
}

// takahashiCharge (takahashi.ts:43-54), fC: bilinear over 1 K columns and the two neighbouring cloud-water rows.
SG_HD float takahashi(float tc, float lwc) {
  if (tc >= 0.f || tc <= -40.f || lwc < .01f) return 0.f;
  const float w = fminf(30.f, lwc);
  int row = 0;
  while (row < SG_TAKAHASHI_ROWS - 2 && w >= takLwc(row + 1)) row++;
  const float t = fminf(30.f, -fmaxf(-30.f, tc));
  const int col = (int)fminf(29.f, floorf(t));
  const float f = t - (float)col;
  const float a0 = takEntry(row, col), a = a0 + f * (takEntry(row, col + 1) - a0);
  const float b0 = takEntry(row + 1, col), b = b0 + f * (takEntry(row + 1, col + 1) - b0);
  const float l0 = takLwc(row), g = fminf(1.f, (w - l0) / (takLwc(row + 1) - l0));
  const float cold = tc < -30.f ? 1.f - ((tc + 30.f) / 10.f) * ((tc + 30.f) / 10.f) : 1.f;
  return cold * (a + g * (b - a));
}
// takahashiScaled (charge.ts:229-233), C: the table's charge for a crystal of size d at relative speed dv.
SG_HD float takScaled(float table, float d, float dv) {
  const float r = d / 100e-6f;
  const float q = table * fminf(5.f * r * r * fabsf(dv) / 8.f, 10.f) * 1e-15f;
  return fmaxf(-500e-15f, fminf(500e-15f, q));
}

// exponentialMoments (charge.ts:118-121): number, n<D>, n<D^2>, mass-weighted fall speed, the integral of D^2 V n.
struct Moments { float n, d1, d2, fall, d2v; };
SG_HD Moments moments(float n0, float density, float q, float rho) {
  const float lambda = root4(PI * density * n0 / (rho * q)), a = fallCoef(rho, density), sl = sqrtf(lambda);
  const float l3 = lambda * lambda * lambda;
  return {n0 / lambda, n0 / (lambda * lambda), 2.f * n0 / l3, a * GAMMA_45 / 6.f / sl, a * n0 * GAMMA_35 / (l3 * sl)};
}

// rimerRate (charge.ts:157-168) of the Takahashi scheme: a rimer's collisions with the cloud ice (at rest) and the snow.
SG_HD float rimerRate(const Moments& m, float table, float rebound, float ni, float di, float ns, float ds, float vs) {
  const float fall = m.fall, k = PI / 4.f * rebound;
  float rate = 0.f;
  if (ni > 0.f) {
    const float swept = m.d2 + 2.f * di * m.d1 + di * di * m.n;
    rate += fmaxf(-TAK_RATE_MAX, fminf(TAK_RATE_MAX, ni * k * swept * fall * takScaled(table, di, fall)));
  }
  if (ns > 0.f) {
    const float v = fabsf(fall - vs), swept = m.d2 + 2.f * ds * m.d1 + ds * ds * m.n;
    rate += fmaxf(-TAK_RATE_MAX, fminf(TAK_RATE_MAX, ns * k * swept * v * takScaled(table, ds, v)));
  }
  return rate;
}

// chargingRate (charge.ts:136-151), Takahashi scheme, the model's own crystals (`crystals` per m3): the charge
// separation rate, C m^-3 s^-1, gained by the graupel-hail carrier. `two` (graupel's, hail's) with the bits of `has`:
// two-moment classes' own moments (ice2m.ts rimerMoments), taken instead of the fixed intercept's where given (:153-155).
SG_HD float chargingRate(float tc, float rho, float cloud, float ice, float snow, float graupel, float hail, float snowFall, bool wetG, bool wetH,
                         float crystals, const Moments* two = nullptr, int has = 0) {
  if (tc >= 0.f || tc < -40.f || cloud <= 0.f || ice + snow <= 0.f || graupel + hail <= 0.f) return 0.f;
  const float rebound = .5f * (1.f - .1f * expf(.1f * tc)), water = rho * cloud * 1000.f;
  const float ni = ice <= 0.f ? 0.f : crystals;
  // the column length of a crystal of the mean mass, .1871 m^.3429 (charge.ts:142-143); no crystals: none charge
  const float di = (ice <= 0.f || crystals == 0.f) ? 0.f : fminf(CRYSTAL_HI, fmaxf(CRYSTAL_LO, .1871f * powf(rho * ice / crystals, .3429f)));
  float ns = 0.f, ds = 0.f;
  if (snow > 0.f) { const float slope = root4(PI * RHO_S * N0S / (rho * snow)); ns = N0S / slope; ds = 1.8171f / slope; }
  const float table = takahashi(tc, water);
  float rate = 0.f;
  if (graupel > 0.f && !wetG) rate += rimerRate((has & 1) ? two[0] : moments(N0G, RHO_G, graupel, rho), table, rebound, ni, di, ns, ds, snowFall);
  if (hail > 0.f && !wetH) rate += rimerRate((has & 2) ? two[1] : moments(N0H, RHO_H, hail, rho), table, rebound, ni, di, ns, ds, snowFall);
  return rate;
}

// inductiveRate (charge.ts:187-200): C m^-3 s^-1 gained by the graupel-hail carrier (the droplets get the opposite).
SG_HD float inductiveRate(float tc, float rho, float cloud, float graupel, float hail, float ez, float rimerCharge, bool wetG, bool wetH,
                          const Moments* two = nullptr, int has = 0) {
  if (tc >= 0.f || cloud <= 0.f) return 0.f;
  const float d = DROPLET_SIZE, droplets = rho * cloud / DROPLET_KG, k = COLLECTION_EFFICIENCY * DROPLET_REBOUND * droplets;
  float polarize = 0.f, mass = 0.f, massFall = 0.f;
  if (graupel > 1e-9f && !wetG) {
    const Moments m = (has & 1) ? two[0] : moments(N0G, RHO_G, graupel, rho);
    polarize += PI4_8 * EPSILON0 * ez * CONTACT_COS * d * d * m.d2v; mass += graupel; massFall += graupel * m.fall;
  }
  if (hail > 1e-9f && !wetH) {
    const Moments m = (has & 2) ? two[1] : moments(N0H, RHO_H, hail, rho);
    polarize += PI4_8 * EPSILON0 * ez * CONTACT_COS * d * d * m.d2v; mass += hail; massFall += hail * m.fall;
  }
  if (mass == 0.f) return 0.f;
  return k * (polarize - PI3_24 * d * d * (massFall / mass) * rimerCharge);
}

// transferCharge (charge.ts:216-226): the charge moved with the mass between [ice-snow, graupel-hail, rain, droplets
// and ions]; what went to vapour stays on the ions (the last carrier). The sum of the four is kept.
SG_HD void transferCharge(float (&c)[4], const float (&before)[4], const float (&after)[4]) {
  float pool = 0.f, lost = 0.f, gained = 0.f;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    if (after[k] < before[k]) {
      const float share = before[k] > 0.f ? (before[k] - after[k]) / before[k] : 1.f, out = c[k] * share;
      c[k] -= out; pool += out; lost += before[k] - after[k];
    } else gained += after[k] - before[k];
    if (k != 3 && after[k] <= 0.f && c[k] != 0.f) { pool += c[k]; c[k] = 0.f; }
  }
  if (pool == 0.f) return;
  const float moved = gained > 0.f ? fminf(1.f, lost > 0.f ? gained / lost : 1.f) : 0.f;
  if (moved > 0.f) {
#pragma unroll
    for (int k = 0; k < 4; k++) if (after[k] > before[k]) c[k] += pool * moved * (after[k] - before[k]) / gained;
  }
  c[3] += pool * (1.f - moved);
}

// wetGrowing (src/core/hail.ts:127-131): the rimer population sweeps out more water than its surface can freeze.
SG_HD bool wetGrowing(float q, float n0, float rhoX, float tc, const phys::Node& s, const phys::Level& L) {
  if (tc >= 0.f || q <= 1e-9f) return false;
  const float rho = L.rho, lambda = root4(PI * rhoX * n0 / (rho * q)), a = fallCoef(rho, rhoX);
  const float k = PI * n0 * a * GAMMA_35 / (4.f * (lambda * lambda * lambda * sqrtf(lambda)));
  return k * (s.cloud + s.rain + .1f * s.ice + expf(.09f * tc) * s.snow) > wetGrowth(lambda, a, n0, tc, s.q, L, k * (s.ice + s.snow));
}

}  // namespace charge
}  // namespace sg
