// TEST INFRASTRUCTURE ONLY — the oracle's restatement of the reference's per-run diagnostics: the rotation tracking
// run after every step (updateRotation, src/core/model.ts:1609-1648, with zeta :1597-1601), the domain diagnostics a
// sample reads (diagnostics, :1672-1696; countCores :1650-1670; precipitationFlux, src/core/surfaceflux.ts:31-36;
// outflowDeficit / deficitNear, src/core/rkw.ts:72-90) and the ensemble's swaths (addSwaths,
// src/ensemble/member.ts:71-89). Plain loops in FP64 in the reference's order.
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>
#include "oracle_model.h"

namespace orc {

constexpr double CORE_ROTATION_W = 10;          // model.ts:112
constexpr double MESO_CORE_ZETA = 3e-3;         // model.ts:120
constexpr double MESO_GRID = 1200;              // model.ts:127
constexpr double OUTFLOW_WARM = .75, OUTFLOW_NEAR = 2000;  // rkw.ts:57-59
inline double mesoCoreZeta(double dx) { return MESO_CORE_ZETA * std::max(1.0, MESO_GRID / dx); }  // model.ts:129

struct Rotation {
  double uh = 0, x = 0, y = 0, anticyclonic = 0, persisted = 0, uh01 = 0, uh03 = 0, low = 0, coreZeta = 0, coreUH = 0, coreAnti = 0;
};

// The 2-5 km levels (model.ts:389) and the last levels at or below 1 and 3 km (:1612).
inline void uh_levels(const GridSpec& g, int& z0, int& z1, int& top1, int& top3) {
  z0 = -1; z1 = -1; top1 = -1; top3 = -1;
  for (int z = 0; z < g.nz; z++) {
    if (z0 < 0 && g.zs[z] >= 2000) z0 = z;
    if (g.zs[z] <= 5000) z1 = z;
    if (g.zs[z] <= 1000) top1 = z;
    if (g.zs[z] <= 3000) top3 = z;
  }
}

template <class S> double zeta(const Model<S>& m, int x, int y, int z) {  // model.ts:1597-1601
  const GridSpec& g = m.g;
  const int nx = g.nx, l = z * g.layer;
  const auto& u = m.f[F_U]; const auto& v = m.f[F_V];
  return ((double)v[g.xp[x] + nx * y + l] - (double)v[g.xm[x] + nx * y + l]) / (2 * g.dx) -
         ((double)u[x + g.yp[y] + l] - (double)u[x + g.ym[y] + l]) / (2 * g.dy);
}

// updateRotation (model.ts:1609-1648) on the model's fields: the UH column (col, FP32 values as the reference's
// Float32Array), the rotation summary into r.
template <class S> void updateRotation(const Model<S>& m, double dt, Rotation& r, std::vector<double>& col) {
  const GridSpec& g = m.g;
  const int nx = g.nx, ny = g.ny, layer = g.layer;
  int z0, z1, top1, top3;
  uh_levels(g, z0, z1, top1, top3);
  const auto& w = m.f[F_W];
  double max = 0, min = 0, bx = 0, by = 0, max01 = 0, max03 = 0, low01 = 0;
  std::vector<double> coreW(layer), coreWZ(layer);
  col.assign(layer, 0);
  for (int y = 0; y < ny; y++) for (int x = 0; x < nx; x++) {
    double uh = 0, low = 0, sw = 0, swz = 0;
    for (int z = 1; z <= top3; z++) {
      low += (double)w[x + nx * y + z * layer] * zeta(m, x, y, z) * g.hz[z];
      if (z == top1 && low > max01) { max01 = low; low01 = x + nx * y; }
    }
    max03 = std::max(max03, low);
    for (int z = z0; z <= z1; z++) {
      const double wv = w[x + nx * y + z * layer], wz = wv * zeta(m, x, y, z) * g.hz[z];
      uh += wz;
      if (wv > CORE_ROTATION_W) { sw += wv * g.hz[z]; swz += wz; }
    }
    col[x + nx * y] = (float)uh; coreW[x + nx * y] = sw; coreWZ[x + nx * y] = swz;  // uhColumn is a Float32Array (:384)
    if (uh > max) { max = uh; bx = x; by = y; }
    min = std::min(min, uh);
  }
  // updraught cores: connected columns (8 neighbours, periodic) with 2-5 km nodes above CORE_ROTATION_W
  std::vector<unsigned char> label(layer, 0);
  std::vector<int> stack;
  double coreZeta = 0, coreUH = 0, coreAnti = 0;
  for (int start = 0; start < layer; start++) {
    if (coreW[start] <= 0 || label[start]) continue;
    double sw = 0, swz = 0, peak = 0;
    label[start] = 1; stack.push_back(start);
    while (!stack.empty()) {
      const int a = stack.back(); stack.pop_back();
      const int x = a % nx, y = (a - x) / nx;
      sw += coreW[a]; swz += coreWZ[a]; peak = std::max(peak, col[a]);
      for (int oy = -1; oy <= 1; oy++) for (int ox = -1; ox <= 1; ox++) {
        const int b = (x + ox + nx) % nx + nx * ((y + oy + ny) % ny);
        if (coreW[b] > 0 && !label[b]) { label[b] = 1; stack.push_back(b); }
      }
    }
    if (swz / sw > coreZeta) { coreZeta = swz / sw; coreUH = peak; }
    coreAnti = std::max(coreAnti, -swz / sw);
  }
  r.coreZeta = coreZeta; r.coreUH = coreUH; r.coreAnti = coreAnti;
  r.uh = max; r.anticyclonic = -min; r.uh01 = max01; r.uh03 = max03; r.low = low01; r.x = bx; r.y = by;
  r.persisted = coreZeta >= mesoCoreZeta(g.dx) ? r.persisted + dt : 0;
}

struct Diagnostics {
  double updraft, downdraft, rainRate, rainTotal, cloudTop, thermalTop, maxCloud, coldMax, cores, outflow, outflowLow, gust, hail, clipped;
};

// countCores (model.ts:1650-1670): cloudy updraught columns (w > 2 m/s, cloud + ice > 7e-5 between 1.9 and 6.6 km),
// 4-connected, periodic.
template <class S> int countCores(const Model<S>& m) {
  const GridSpec& g = m.g;
  const int nx = g.nx, ny = g.ny, nz = g.nz, layer = g.layer;
  int lo = -1, last = -1;
  for (int z = 0; z < nz; z++) { if (lo < 0 && g.zs[z] >= 1900) lo = z; if (g.zs[z] <= 6600) last = z; }
  const int hi = std::min(nz - 3, last);
  std::vector<unsigned char> mask(layer, 0);
  for (int y = 0; y < ny; y++) for (int x = 0; x < nx; x++) {
    bool active = false;
    for (int z = lo; z <= hi && lo >= 0; z++) {
      const int i = x + nx * y + z * layer;
      if ((double)m.f[F_W][i] > 2 && (double)m.f[F_CLOUD][i] + (double)m.f[F_ICE][i] > .00007) { active = true; break; }
    }
    mask[x + nx * y] = active ? 1 : 0;
  }
  int cores = 0;
  std::vector<int> stack;
  for (int i = 0; i < layer; i++) {
    if (mask[i] != 1) continue;
    cores++; mask[i] = 2; stack.push_back(i);
    while (!stack.empty()) {
      const int a = stack.back(); stack.pop_back();
      const int x = a % nx, y = a / nx;
      const int nb[4] = {(x + 1) % nx + nx * y, (x - 1 + nx) % nx + nx * y, x + nx * ((y + 1) % ny), x + nx * ((y - 1 + ny) % ny)};
      for (int b : nb) if (mask[b] == 1) { mask[b] = 2; stack.push_back(b); }
    }
  }
  return cores;
}

// diagnostics (model.ts:1672-1696) without the environment's shear06 (a property of the sounding), no terrain:
// every column's ground node is level 0, the surface density rho[0].
template <class S> Diagnostics diagnostics(const Model<S>& m, const Rotation& r) {
  const GridSpec& g = m.g;
  const int nx = g.nx, ny = g.ny, nz = g.nz, layer = g.layer;
  Diagnostics d{};
  double up = 0, down = 0, top = 0, coldMax = 0, thermalTop = 0, maxCloud = 0;
  for (int z = 0, i = 0; z < nz; z++) for (int y = 0; y < ny; y++) for (int x = 0; x < nx; x++, i++) {
    const double alt = g.zs[z], wv = m.f[F_W][i], ci = (double)m.f[F_CLOUD][i] + (double)m.f[F_ICE][i];
    up = std::max(up, wv); down = std::max(down, -wv); maxCloud = std::max(maxCloud, ci);
    if (ci > .00007) top = std::max(top, alt / 1000);
    if (wv > .6) thermalTop = std::max(thermalTop, alt / 1000);
    if (alt < 1500) coldMax = std::max(coldMax, (double)m.f[F_COLD][i]);
  }
  const double rho0 = m.rho[0], fu = m.sw.frameU, fv = m.sw.frameV;
  double rainRate = 0, rainTotal = 0, gust = 0, hail = 0;
  for (int c = 0; c < layer; c++) gust = std::max(gust, std::hypot((double)m.f[F_U][c] + fu, (double)m.f[F_V][c] + fv));
  for (int c = 0; c < layer; c++) {
    // precipitationFlux (surfaceflux.ts:31-36) with the one-moment fall speeds, mm/h of water
    const double r_ = m.f[F_RAIN][c], s = m.f[F_SNOW][c], gr = m.f[F_GRAUPEL][c], h = m.f[F_HAIL][c];
    const double vg = gr > 0 ? graupelFallSpeed(gr, rho0) : 0, vh = h > 0 ? hailFallSpeed(h, rho0) : 0;
    const double flux = rho0 * r_ * fallSpeed(r_, rho0, rho0) + rho0 * (s * snowFallSpeed(s, rho0, rho0) + gr * vg + h * vh);
    rainRate = std::max(rainRate, flux * 3600);
    rainTotal = std::max(rainTotal, (double)m.precipitation[c]);
    hail = std::max(hail, hailMaxDiameter(h, rho0) * 1000);
  }
  // outflowDeficit (rkw.ts:72-80): the ground air's theta_v below the 75th percentile of the columns
  std::vector<float> thv(layer);
  for (int c = 0; c < layer; c++) thv[c] = (float)((double)m.f[F_THETA][c] * (1 + .61 * (double)m.f[F_Q][c]));
  std::vector<float> sorted = thv;
  std::sort(sorted.begin(), sorted.end());
  const double warm = sorted[(size_t)std::floor((layer - 1) * OUTFLOW_WARM)];
  std::vector<float> deficit(layer);
  double omax = 0;
  for (int c = 0; c < layer; c++) { deficit[c] = (float)std::max(0.0, warm - (double)thv[c]); omax = std::max(omax, (double)deficit[c]); }
  // deficitNear (rkw.ts:82-90) around the low-level rotation's column
  const int c0 = (int)r.low, x0 = c0 % nx, y0 = c0 / nx, rx = (int)std::floor(OUTFLOW_NEAR / g.dx), ry = (int)std::floor(OUTFLOW_NEAR / g.dy);
  double near = 0;
  for (int j = -ry; j <= ry; j++) for (int i = -rx; i <= rx; i++) {
    if (std::pow(i * g.dx, 2) + std::pow(j * g.dy, 2) > OUTFLOW_NEAR * OUTFLOW_NEAR) continue;
    near = std::max(near, (double)deficit[((x0 + i) % nx + nx) % nx + nx * (((y0 + j) % ny + ny) % ny)]);
  }
  d.updraft = up; d.downdraft = down; d.rainRate = rainRate; d.rainTotal = rainTotal; d.cloudTop = top; d.thermalTop = thermalTop;
  d.maxCloud = maxCloud; d.coldMax = coldMax; d.cores = countCores(m); d.outflow = omax; d.outflowLow = near; d.gust = gust;
  d.hail = hail; d.clipped = m.clipped;
  return d;
}

// addSwaths (member.ts:71-89) for a periodic domain: the surface wind and the UH column folded into the per-ground-
// column maxima, the domain shifted by its motion so far (whole columns).
template <class S> void addSwaths(const Model<S>& m, double time, const std::vector<double>& uhColumn, std::vector<float>& gustMax,
                                  std::vector<float>& uhMax) {
  const GridSpec& g = m.g;
  const int nx = g.nx, ny = g.ny;
  const double fu = m.sw.frameU, fv = m.sw.frameV;
  const long sx = (long)std::floor(fu * time / g.dx + .5), sy = (long)std::floor(fv * time / g.dy + .5);  // Math.round
  for (int y = 0; y < ny; y++) {
    const int gy = (int)((((y + sy) % ny) + ny) % ny);
    for (int x = 0; x < nx; x++) {
      const int gx = (int)((((x + sx) % nx) + nx) % nx);
      const int c = x + nx * y, gc = gx + nx * gy;
      const float wind = (float)std::hypot((double)m.f[F_U][c] + fu, (double)m.f[F_V][c] + fv);
      if (wind > gustMax[gc]) gustMax[gc] = wind;
      if ((float)uhColumn[c] > uhMax[gc]) uhMax[gc] = (float)uhColumn[c];
    }
  }
}

}  // namespace orc
