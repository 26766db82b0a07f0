// Test harness: the device step's per-node functions (meteolab_gb300/csrc/sg_physics.cuh, sg_common.cuh,
// sg_fft.cuh) compiled for the host, so their logic can be checked against the oracle on the CPU. Built by
// tests/test_device_code_on_cpu.py with g++; not part of the library.
#include <vector_types.h>
#include <vector_functions.h>
#include <cmath>
#include <vector>
#include "../../meteolab_gb300/csrc/sg_common.cuh"
#include "../../meteolab_gb300/csrc/sg_fft.cuh"
#include "../../meteolab_gb300/csrc/sg_physics.cuh"
#include "../../meteolab_gb300/csrc/sg_tile_copies.cuh"
#include "../../meteolab_gb300/csrc/sg_charge.cuh"
#include "../../meteolab_gb300/csrc/sg_rain2m.cuh"
#include "../../meteolab_gb300/csrc/sg_ice2m.cuh"

using namespace sg;

extern "C" {

// two-moment rain of the physics kernel (sg_rain2m.cuh), FP32: v = [q, cloud, rain, number] in place at temperature
// tk (K), pressure p, density rho; returns the evaporated rain
float ht_r2m_processes(float* v, double tk, double p, double rho, float dt, int breakup, int evaporate) {
  phys::Level L = phys::makeLevel(tk, 1.0, p, rho, rho);
  phys::Node s{0.f, (float)tk, L.tcb, v[0], v[1], v[2], 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  float number = v[3];
  const float evap = r2m::processes(s, number, L, dt, breakup, evaporate != 0);
  v[0] = s.q; v[1] = s.cloud; v[2] = s.rain; v[3] = number;
  return evap;
}
void ht_r2m_fall(float q, float n, float rho, float* out) { r2m::fallSpeeds(q, n, rho, out[0], out[1], out[2]); }

// two-moment graupel and hail (sg_ice2m.cuh), FP32; class c 0 graupel, 1 hail
static i2m::IceClass cls(int c) { return c == 0 ? i2m::GRAUPEL_2M() : i2m::HAIL_2M(); }
void ht_i2m_speeds(int c, float q, float n, float vol, float rho, float* out3) { i2m::momentSpeeds(cls(c), q, n, vol, rho, out3[0], out3[1], out3[2]); }
float ht_i2m_largest(int c, float q, float n, float vol, float rho) { return i2m::largestDiameter(cls(c), q, n, vol, rho); }
int ht_i2m_rimer(int c, float q, float n, float vol, float rho, float* out5) {
  charge::Moments m;
  if (!i2m::rimerMoments(cls(c), q, n, vol, rho, m)) return 0;
  out5[0] = m.n; out5[1] = m.d1; out5[2] = m.d2; out5[3] = m.fall; out5[4] = m.d2v;
  return 1;
}
void ht_i2m_sweep(int c, int pair, float* out3) { out3[0] = i2m::h_sweep.a[c][pair]; out3[1] = i2m::h_sweep.b[c][pair]; out3[2] = i2m::h_sweep.c[c][pair]; }
// the node's microphysics with two-moment rain, graupel and hail: v = thp, thb, q, cloud, rain, ice, inum, snow, graupel,
// hail, cold, rainNumber, graupelNumber, graupelVolume, hailNumber, hailVolume (in place); wet2 = wet growth
float ht_microphysics_2m(float* v, double exner, double p, double rho, double rho0, float dt, int flags, int* wet2) {
  phys::Level L = phys::makeLevel((double)v[1], exner, p, rho, rho0);
  phys::Node s{v[0], v[1], L.tcb, v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9], v[10]};
  float rn = v[11], evap = 0.f;
  i2m::Fields f = {v[12], v[13], v[14], v[15]};
  bool wg = false, wh = false;
  i2m::microphysics(s, rn, f, L, dt, flags, 0, evap, wg, wh);
  v[0] = s.thp; v[2] = s.q; v[3] = s.cloud; v[4] = s.rain; v[5] = s.ice; v[6] = s.inum; v[7] = s.snow; v[8] = s.graupel; v[9] = s.hail; v[10] = s.cold;
  v[11] = rn; v[12] = f.gn; v[13] = f.gv; v[14] = f.hn; v[15] = f.hv;
  wet2[0] = wg; wet2[1] = wh;
  return evap;
}
float ht_charging_2m(float tc, float rho, float cloud, float ice, float snow, float graupel, float hail, float snowFall, float crystals,
                     const float* m10, int has) {
  charge::Moments two[2];
  for (int j = 0; j < 2; j++) two[j] = {m10[5 * j], m10[5 * j + 1], m10[5 * j + 2], m10[5 * j + 3], m10[5 * j + 4]};
  return charge::chargingRate(tc, rho, cloud, ice, snow, graupel, hail, snowFall, false, false, crystals, two, has);
}

// the charging of the physics kernel (sg_charge.cuh), FP32
float ht_takahashi(float tc, float lwc) { return charge::takahashi(tc, lwc); }
float ht_charging(float tc, float rho, float cloud, float ice, float snow, float graupel, float hail, float snowFall, int wetG, int wetH, float crystals) {
  return charge::chargingRate(tc, rho, cloud, ice, snow, graupel, hail, snowFall, wetG != 0, wetH != 0, crystals);
}
float ht_inductive(float tc, float rho, float cloud, float graupel, float hail, float ez, float rimerCharge, int wetG, int wetH) {
  return charge::inductiveRate(tc, rho, cloud, graupel, hail, ez, rimerCharge, wetG != 0, wetH != 0);
}
void ht_transfer(float* c, const float* before, const float* after) {
  float cc[4] = {c[0], c[1], c[2], c[3]};
  const float b[4] = {before[0], before[1], before[2], before[3]}, a[4] = {after[0], after[1], after[2], after[3]};
  charge::transferCharge(cc, b, a);
  for (int k = 0; k < 4; k++) c[k] = cc[k];
}

float ht_weno(float a, float b, float c, float d, float e) { return weno5(a, b, c, d, e); }
float ht_upwind(float a, float b, float c, float d, float e) { return upwind5(a, b, c, d, e); }

// v = [thp, thb, q, cloud, rain, ice, inum, snow, graupel, hail, cold] in/out; returns evap. The level's constants
// (the Celsius base temperature, the saturation bases) come from thb, exner, p, rho in FP64, as when a run is created.
float ht_microphysics(float* v, double exner, double p, double rho, double rho0, float dt, int flags) {
  phys::Level L = phys::makeLevel((double)v[1], exner, p, rho, rho0);
  phys::Node s{v[0], v[1], L.tcb, v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9], v[10]};
  float evap = 0;
  phys::microphysics(s, L, dt, flags, evap);
  v[0] = s.thp; v[2] = s.q; v[3] = s.cloud; v[4] = s.rain; v[5] = s.ice; v[6] = s.inum; v[7] = s.snow; v[8] = s.graupel; v[9] = s.hail; v[10] = s.cold;
  return evap;
}
void ht_fall(float rain, float snow, float graupel, float hail, float rho, float fallsq, float* out) {
  out[0] = phys::rainFall(rain, rho, fallsq); out[1] = phys::snowFall(snow, rho, fallsq);
  out[2] = phys::graupelFall(graupel, rho); out[3] = phys::hailFall(hail, rho);
}
// Forward FFT of one row with the device's Stockham stages (x in/out as interleaved re, im).
int ht_fft(int n, float* x) {
  int rad[8]; int nf = fft_plan_factors(n, rad);
  if (nf < 0) return -1;
  std::vector<float2> tw(n), a(n), b(n);
  for (int t = 0; t < n; t++) { double ang = -2 * M_PI * t / n; tw[t] = make_float2((float)cos(ang), (float)sin(ang)); }
  for (int i = 0; i < n; i++) a[i] = make_float2(x[2 * i], x[2 * i + 1]);
  float2 *src = a.data(), *dst = b.data();
  int Ns = 1;
  for (int s = 0; s < nf; s++) {
    int r = rad[s];
    for (int j = 0; j < n / r; j++) fft_butterfly(src, dst, n, r, Ns, j, tw.data());
    std::swap(src, dst); Ns *= r;
  }
  for (int i = 0; i < n; i++) { x[2 * i] = src[i].x; x[2 * i + 1] = src[i].y; }
  return nf;
}

double ht_widen(float f) { return widen(f); }
float ht_narrow(double d) { return narrow(d); }
int ht_fft_factors(int n, int* rad) { return fft_plan_factors(n, rad); }
int ht_fft_count(int n) { return fft_count(n); }
int ht_fft_radix(int n, int s) { return fft_radix_at(n, s); }


// The bulk-copy transport's packet plan of one tile (sg_tile_copies.cuh): every ring copy of one plane and every
// auxiliary copy, as rows (kind, smem float offset, source offset, bytes): kind 0 a ring piece (source: float offset
// in a field's level), 1 a face-flux copy (float4 offset in the level), 2 + g a step-start row of field g (float
// offset). Returns the number of rows (at most cap); *bytes gets the announced bytes of a one-plane packet, *covered
// the window columns the pieces fill.
int ht_tile_copies(int nx, int ny, int TX, int TY, int x0, int y0, int G, int s0, int* out, int cap, unsigned* bytes, int* covered) {
  TileCopies T{nx, ny, nx * ny, TX, TY, x0, y0, G, s0 != 0};
  int cov = 0;
  const int nseg = T.pieces(cov);
  int k = 0;
  for (int j = 0; j < T.PH() * nseg && k < cap; j++, k++) {
    int soff, goff, len;
    T.ring(j, nseg, soff, goff, len);
    out[4 * k] = 0; out[4 * k + 1] = soff; out[4 * k + 2] = goff; out[4 * k + 3] = 4 * len;
  }
  for (int j = 0; j < T.naux() && k < cap; j++, k++) {
    int soff, src, which, b;
    T.aux(j, soff, src, which, b);
    out[4 * k] = which == 0 ? 1 : 1 + which; out[4 * k + 1] = soff; out[4 * k + 2] = src; out[4 * k + 3] = b;
  }
  *bytes = T.bytes(1);
  *covered = cov;
  return k;
}
}  // extern "C"
