// TEST INFRASTRUCTURE ONLY — the oracle's terrain (see oracle_core.h): the checker the device's masked projection is
// compared with, never linked into the product. Restates src/core/terrain.ts: the ground heights of a terrain form
// (terrainHeights :37-63), the cut-cell geometry (volumeTop :72, solidMask :80-84, groundLevels :87-91, nodeHeights
// :101-105, faceApertures :119-134, slopeArea :141-150) and MaskedProjection (:168-363), the cut-cell projection
// solved by preconditioned conjugate gradients around the flat spectral solve (PressureSolver, oracle_solvers.h); and
// the transport's faces with terrain (src/core/advection.ts:78-184, MaskedFaces: setTerrain, setVelocityMasked).
// JS semantics: doubles, Float32Array stores rounded to float, sums in the reference's order.
#pragma once
#include <cstdint>
#include "oracle_solvers.h"

namespace orc {
namespace terrain {

// A terrain form (terrain.ts:16-27): kind 0 hill, 1 ridge, 2 plateau, 3 schar; heights and widths in km; an absent
// centre, heading or wavelength is NaN (the reference's `??` defaults).
struct Form { int kind; double height, width, x, y, heading, wavelength; };

inline double jsRound(double x) { double r = std::floor(x); return x - r >= 0.5 ? r + 1 : r; }  // Math.round

// terrain.ts:37-63: the form's height per column, two 1-2-1 passes in x then y, the lowest column moved to 0.
inline std::vector<float> heights(const Form& t, const GridSpec& g) {
  const int nx = g.nx, ny = g.ny;
  std::vector<float> h((size_t)nx * ny), tmp((size_t)nx * ny);
  const double cx = (std::isnan(t.x) ? g.width / 2000 : t.x) * 1000, cy = (std::isnan(t.y) ? g.depth / 2000 : t.y) * 1000;
  const double a = std::max(t.width * 1000, 2 * std::max(g.dx, g.dy)), top = t.height * 1000;
  const double axis = (std::isnan(t.heading) ? 0 : t.heading) * PI / 180, ax = std::sin(axis), ay = std::cos(axis);
  auto wrap = [](double d, double size) { return d - size * jsRound(d / size); };
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      const double ex = wrap((i + .5) * g.dx - cx, g.width), ey = wrap((j + .5) * g.dy - cy, g.depth);
      double v;
      if (t.kind == 0) v = top / std::pow(1 + (ex * ex + ey * ey) / (a * a), 1.5);
      else if (t.kind == 1) { const double across = ex * ay - ey * ax; v = top / (1 + across * across / (a * a)); }
      else if (t.kind == 3) {
        const double across = ex * ay - ey * ax, c = std::cos(PI * across / ((std::isnan(t.wavelength) ? 4 : t.wavelength) * 1000));
        v = top * std::exp(-across * across / (a * a)) * (c * c);
      } else { const double r = std::max(std::fabs(ex), std::fabs(ey)); v = top / (1 + std::exp((r - a) / (.25 * a))); }
      h[i + (size_t)nx * j] = (float)v;
    }
  for (int pass = 0; pass < 2; pass++) {
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++)
        tmp[i + (size_t)nx * j] = (float)(((double)h[(i + nx - 1) % nx + (size_t)nx * j] + 2 * (double)h[i + (size_t)nx * j] + (double)h[(i + 1) % nx + (size_t)nx * j]) / 4);
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++)
        h[i + (size_t)nx * j] = (float)(((double)tmp[i + (size_t)nx * ((j + ny - 1) % ny)] + 2 * (double)tmp[i + (size_t)nx * j] + (double)tmp[i + (size_t)nx * ((j + 1) % ny)]) / 4);
  }
  double low = INFINITY;
  for (float v : h) low = std::min(low, (double)v);
  for (float& v : h) v = (float)((double)v - low);
  return h;
}

constexpr double LEAST_SHARE = .2;  // terrain.ts:69

inline double volumeTop(const GridSpec& g, int k) { return k < g.nz - 1 ? g.zs[k] + g.dzs[k] / 2 : g.zs[k]; }  // :72

// :80-84: solid where the ground leaves less than LEAST_SHARE of the node's control volume; the top two levels fluid.
template <class H> std::vector<uint8_t> solidMask(const GridSpec& g, const H* h) {
  std::vector<uint8_t> solid((size_t)g.n, 0);
  for (int c = 0; c < g.layer; c++)
    for (int z = 0; z < g.nz - 2 && volumeTop(g, z) - (double)h[c] < LEAST_SHARE * g.hz[z]; z++) solid[c + (size_t)z * g.layer] = 1;
  return solid;
}

inline std::vector<int> groundLevels(const GridSpec& g, const uint8_t* solid) {  // :87-91
  std::vector<int> lv(g.layer);
  for (int c = 0; c < g.layer; c++) { int z = 0; while (z < g.nz - 1 && solid[c + (size_t)z * g.layer]) z++; lv[c] = z; }
  return lv;
}

// :101-105: the ground node owns its volume above the ground, solid nodes nothing, the rest their level's hz.
template <class H> std::vector<double> nodeHeights(const GridSpec& g, const uint8_t* solid, const H* ground) {
  std::vector<double> h((size_t)g.n);
  std::vector<int> lv = groundLevels(g, solid);
  for (int z = 0, i = 0; z < g.nz; z++)
    for (int c = 0; c < g.layer; c++, i++)
      h[i] = solid[i] ? 0 : z == lv[c] ? volumeTop(g, z) - (ground ? (double)ground[c] : g.zs[z]) : g.hz[z];
  return h;
}

// :119-134: the open height of each node's faces to x + 1 and y + 1, the ground on the face the mean of its columns'.
template <class H> void faceApertures(const GridSpec& g, const uint8_t* solid, const H* ground, std::vector<double>& ax, std::vector<double>& ay) {
  const int nx = g.nx, ny = g.ny, nz = g.nz, layer = g.layer;
  ax.assign((size_t)g.n, 0); ay.assign((size_t)g.n, 0);
  auto shave = [&](std::vector<double>& out, int c, int other) {
    const double face = ((double)ground[c] + (double)ground[other]) / 2;
    double carry = 0;
    for (int k = 0; k < nz; k++) {
      const double bottom = k > 0 ? volumeTop(g, k - 1) : 0, top = volumeTop(g, k);
      const double open = face <= bottom ? g.hz[k] : std::max(0.0, top - face);
      const size_t i = c + (size_t)k * layer;
      if (solid[i] || solid[other + (size_t)k * layer]) { carry += open; continue; }
      out[i] = open + carry; carry = 0;
    }
  };
  for (int j = 0, c = 0; j < ny; j++)
    for (int i = 0; i < nx; i++, c++) { shave(ax, c, (i + 1) % nx + j * nx); shave(ay, c, i + ((j + 1) % ny) * nx); }
}

template <class H> std::vector<float> slopeArea(const GridSpec& g, const H* h) {  // :141-150
  const int nx = g.nx, ny = g.ny;
  std::vector<float> area((size_t)nx * ny);
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      const double hx = ((double)h[(i + 1) % nx + nx * j] - (double)h[(i + nx - 1) % nx + nx * j]) / (2 * g.dx);
      const double hy = ((double)h[i + nx * ((j + 1) % ny)] - (double)h[i + nx * ((j + ny - 1) % ny)]) / (2 * g.dy);
      area[i + (size_t)nx * j] = (float)std::sqrt(1 + hx * hx + hy * hy);
    }
  return area;
}

// :168-363: the cut-cell projection of the node mass flux rho0 u over the dual cells, by PCG on -D M (rho0 H)^-1 D^T
// with the flat solve as the preconditioner.
struct MaskedProjection {
  const GridSpec& g;
  PressureSolver& solver;
  double tolerance; int maxIterations;
  int iterations = 0; double residual = 0;
  bool any = false;
  std::vector<uint8_t> solid, wall, dropped;
  std::vector<double> inverseMass, low, high;
  std::vector<double> tu, tv, tw, work, out, z, b, q, r, d, phi;
  DftScratch ds; ModeScratch ms;

  template <class H>
  MaskedProjection(const GridSpec& grid, PressureSolver& s, const H* ground, double tol = 1e-6, int maxIt = 200)
      : g(grid), solver(s), tolerance(tol), maxIterations(maxIt), ds(grid.nx, grid.ny), ms(grid.nz) {
    const int nx = g.nx, ny = g.ny, nz = g.nz, layer = g.layer; const size_t n = g.n, cells = s.cells;
    solid = solidMask(g, ground);
    std::vector<double> heights = nodeHeights(g, solid.data(), ground);
    for (uint8_t v : solid) any = any || v == 1;
    for (int c = 0; c < layer; c++) any = any || (double)ground[c] > 0;
    for (auto* a : {&tu, &tv, &tw}) a->assign(n, 0);
    for (auto* a : {&work, &out, &z, &b, &q, &r, &d, &phi, &low, &high}) a->assign(cells, 0);
    wall.assign(n, 0); inverseMass.assign(n, 0); dropped.assign(cells, 0);
    for (int k = 0, i = 0; k < nz; k++)
      for (int c = 0; c < layer; c++, i++) {
        if (solid[i]) continue;
        if (g.zs[k] <= (double)ground[c]) wall[i] = 1;
        inverseMass[i] = 1 / (s.rho[k] * heights[i]);
      }
    auto clamp = [](double x) { return std::min(1.0, std::max(0.0, x)); };
    for (int k = 0; k < nz - 1; k++)
      for (int c = 0; c < layer; c++) {
        const double half = g.dzs[k] / 2, middle = g.zs[k] + half, h = (double)ground[c];
        low[c + (size_t)k * layer] = clamp((middle - std::max(h, g.zs[k])) / half);
        high[c + (size_t)k * layer] = clamp((g.zs[k + 1] - std::max(h, middle)) / half);
      }
    for (int k = 0, c = 0; k < nz - 1; k++)
      for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++, c++) {
          const int i1 = (i + 1) % nx, j1 = ((j + 1) % ny) * nx, j0 = j * nx; const size_t l = (size_t)k * layer;
          if (high[i + j0 + l] == 0 && high[i1 + j0 + l] == 0 && high[i + j1 + l] == 0 && high[i1 + j1 + l] == 0) dropped[c] = 1;
        }
  }

  // :240-264: the cut cells' divergence of cell layer k.
  template <class S> void divergencePart(const S* u, const S* v, const S* w, double* o, int k) const {
    const int nx = g.nx, ny = g.ny, layer = g.layer; const double r0 = solver.rho[k] / 4, r1 = solver.rho[k + 1] / 4;
    const size_t l = (size_t)k * layer;
    for (int j = 0, c = (int)l; j < ny; j++) {
      const int j0 = j * nx, j1 = ((j + 1) % ny) * nx;
      for (int i = 0; i < nx; i++, c++) {
        if (dropped[c]) { o[c] = 0; continue; }
        const int i1 = (i + 1) % nx;
        double ddx = 0, ddy = 0, ddz = 0;
        for (int corner = 0; corner < 4; corner++) {
          const size_t col = (corner & 1 ? i1 : i) + (corner & 2 ? j1 : j0), lo = col + l, up = lo + layer;
          if (high[lo] > 0) {
            const double a = solid[lo] ? 0 : r0 * low[lo], bb = r1 * (high[lo] + (solid[lo] ? low[lo] : 0));
            const double fu = a * (double)u[lo] + bb * (double)u[up], fv = a * (double)v[lo] + bb * (double)v[up];
            ddx += corner & 1 ? fu : -fu; ddy += corner & 2 ? fv : -fv;
          }
          ddz += r1 * (double)w[up] - r0 * (double)w[lo];
        }
        o[c] = ddx / g.dx + ddy / g.dy + ddz / g.dzs[k];
      }
    }
  }
  template <class S> void divergence(const S* u, const S* v, const S* w, double* o) const {
    for (int k = 0; k < g.nz - 1; k++) divergencePart(u, v, w, o, k);
  }

  // :270-300: the operator's adjoint over each node's mass, of `work` times the cells' heights, into tu, tv, tw.
  void gradientPart(int k) {
    const int nx = g.nx, ny = g.ny, nz = g.nz, layer = g.layer;
    const bool below = k > 0, above = k < nz - 1; const double rr = solver.rho[k] / 4;
    for (int j = 0, i = k * layer; j < ny; j++) {
      const int jm = ((j + ny - 1) % ny) * nx, j0 = j * nx;
      for (int x = 0; x < nx; x++, i++) {
        if (solid[i]) { tu[i] = tv[i] = tw[i] = 0; continue; }
        const int xm = (x + nx - 1) % nx, col = x + j0;
        double gu = 0, gv = 0, gw = 0;
        if (above) {
          const size_t l = (size_t)k * layer; const double f = low[col + l] * rr, h = g.dzs[k];
          const double a = h * work[xm + jm + l], b_ = h * work[x + jm + l], c = h * work[xm + j0 + l], d_ = h * work[x + j0 + l];
          gu += f * (a - b_ + c - d_) / g.dx; gv += f * (a + b_ - c - d_) / g.dy; gw -= rr * (a + b_ + c + d_) / h;
        }
        if (below) {
          const size_t l = (size_t)(k - 1) * layer; const double f = rr * (high[col + l] + (solid[col + l] ? low[col + l] : 0)), h = g.dzs[k - 1];
          const double a = h * work[xm + jm + l], b_ = h * work[x + jm + l], c = h * work[xm + j0 + l], d_ = h * work[x + j0 + l];
          gu += f * (a - b_ + c - d_) / g.dx; gv += f * (a + b_ - c - d_) / g.dy; gw += rr * (a + b_ + c + d_) / h;
        }
        const double m = inverseMass[i];
        tu[i] = gu * m; tv[i] = gv * m; tw[i] = wall[i] || !below || !above ? 0 : gw * m;
      }
    }
  }

  template <class S> void mask(S* u, S* v, S* w) const {  // :229-234
    const size_t n = g.n, layer = g.layer;
    for (size_t i = 0; i < n; i++) if (solid[i]) { u[i] = v[i] = w[i] = 0; } else if (wall[i]) w[i] = 0;
    for (size_t c = 0; c < layer; c++) { w[c] = 0; w[n - layer + c] = 0; }
  }

  void apply(const double* x) {  // :341-345
    const size_t cl = g.layer; const size_t cells = solver.cells;
    for (size_t c = 0; c < cells; c++) work[c] = dropped[c] ? 0 : x[c] / g.dzs[c / cl];
    for (int k = 0; k < g.nz; k++) gradientPart(k);
    for (int k = 0; k < g.nz - 1; k++) divergencePart(tu.data(), tv.data(), tw.data(), out.data(), k);
  }

  void precondition(const double* rv) {  // :351-356
    const size_t cl = g.layer, cells = solver.cells;
    for (size_t c = 0; c < cells; c++) work[c] = -rv[c];
    solver.transform(work.data(), 0, g.nz - 1, ds); solver.modes(0, g.ny, ms); solver.back(z.data(), 0, g.nz - 1, ds);
    for (size_t c = 0; c < cells; c++) z[c] = dropped[c] ? 0 : z[c] * g.dzs[c / cl];
  }

  // :303-333: projects (u, v, w) in place over dt; `pressure` (per cell) is the first guess and gets the result.
  void project(float* u, float* v, float* w, double dt, double* pressure) {
    const size_t cl = g.layer, cells = solver.cells;
    mask(u, v, w);
    if (!any) {
      iterations = 0; residual = 0;
      Arr<float> U = (Arr<float>)u, V = (Arr<float>)v, W = (Arr<float>)w;
      solver.divergence<float>(U, V, W, dt, b.data(), 0, g.nz - 1);
      solver.transform(b.data(), 0, g.nz - 1, ds); solver.modes(0, g.ny, ms); solver.back(pressure, 0, g.nz - 1, ds);
      solver.correct<float>(pressure, U, V, W, dt, 0, g.nz);
      return;
    }
    divergence(u, v, w, b.data());
    double bb = 0;
    for (size_t c = 0; c < cells; c++) bb += b[c] * b[c];
    if (!(bb > 0)) { iterations = 0; residual = 0; return; }
    for (size_t c = 0; c < cells; c++) q[c] = dropped[c] ? 0 : pressure[c] * dt * g.dzs[c / cl];
    apply(q.data());
    for (size_t c = 0; c < cells; c++) r[c] = -b[c] - out[c];
    precondition(r.data());
    double rz = 0;
    for (size_t c = 0; c < cells; c++) { d[c] = z[c]; rz += r[c] * z[c]; }
    int k = 0; double rr = 0;
    for (; k < maxIterations; k++) {
      rr = 0;
      for (size_t c = 0; c < cells; c++) rr += r[c] * r[c];
      if (rr <= tolerance * tolerance * bb) break;
      apply(d.data());
      double dsd = 0;
      for (size_t c = 0; c < cells; c++) dsd += d[c] * out[c];
      if (!(dsd > 0)) break;
      const double alpha = rz / dsd;
      for (size_t c = 0; c < cells; c++) { q[c] += alpha * d[c]; r[c] -= alpha * out[c]; }
      precondition(r.data());
      double rzNew = 0;
      for (size_t c = 0; c < cells; c++) rzNew += r[c] * z[c];
      const double beta = rzNew / rz;
      rz = rzNew;
      for (size_t c = 0; c < cells; c++) d[c] = z[c] + beta * d[c];
    }
    iterations = k; residual = std::sqrt(rr / bb);
    for (size_t c = 0; c < cells; c++) { phi[c] = q[c] / g.dzs[c / cl]; pressure[c] = phi[c] / dt; }
    work = phi;
    for (int kk = 0; kk < g.nz; kk++) gradientPart(kk);
    for (size_t i = 0; i < (size_t)g.n; i++) { u[i] = (float)((double)u[i] + tu[i]); v[i] = (float)((double)v[i] + tv[i]); w[i] = (float)((double)w[i] + tw[i]); }
    mask(u, v, w);
  }
};

// src/core/advection.ts:78-90, :96-105, :115-184: the transport's face fluxes with terrain. setTerrain's open faces
// (bit 1 to x + 1, 2 to y + 1, 4 to z + 1: both nodes fluid) and node heights (1 in the ground), the apertures'
// divergence, and setVelocityMasked: the faces of the node velocity, shut next to the ground, made divergence-free over
// the fluid nodes by PCG on S phi = -h div(M rho0 grad phi) with the flat face solve as the preconditioner.
struct MaskedFaces {
  const GridSpec& g;
  FluxTransport& t;
  std::vector<uint8_t> open;
  std::vector<double> hn, ax, ay, q, r, zz, d, sd, b, fx, fy, fz;
  int iterations = 0; double residual = 0;
  DftScratch ds; ModeScratch ms;

  MaskedFaces(const GridSpec& grid, FluxTransport& tr, const uint8_t* solid, const double* heights, const std::vector<double>& apX,
              const std::vector<double>& apY)
      : g(grid), t(tr), ax(apX), ay(apY), ds(grid.nx, grid.ny), ms(grid.nz) {
    const size_t n = g.n;
    open.assign(n, 0); hn.assign(n, 0);
    for (auto* a : {&q, &r, &zz, &d, &sd, &b, &fx, &fy, &fz}) a->assign(n, 0);
    for (size_t i = 0; i < n; i++) hn[i] = solid[i] ? 1 : heights[i];
    for (int z = 0, i = 0; z < g.nz; z++)
      for (int y = 0; y < g.ny; y++)
        for (int x = 0; x < g.nx; x++, i++) {
          if (solid[i]) continue;
          const int l = z * g.layer, e = g.xo[3][x] + y * g.nx + l, north = x + g.yo[3][y] + l;
          if (!solid[e]) open[i] |= 1;
          if (!solid[north]) open[i] |= 2;
          if (z < g.nz - 1 && !solid[i + g.layer]) open[i] |= 4;
        }
  }

  void terrainDivergence(double* out, const double* gx, const double* gy, const double* gz) const {  // :96-105
    for (int z = 0, i = 0; z < g.nz; z++) {
      const int l = z * g.layer;
      for (int y = 0; y < g.ny; y++)
        for (int x = 0; x < g.nx; x++, i++) {
          const int w = g.xo[1][x] + y * g.nx + l, s = x + g.yo[1][y] + l;
          out[i] = (ax[i] * gx[i] - ax[w] * gx[w]) / g.dx + (ay[i] * gy[i] - ay[s] * gy[s]) / g.dy + (gz[i] - (z > 0 ? gz[i - g.layer] : 0));
        }
    }
  }

  void maskedGradient(const double* phi, double sign, double* gx, double* gy, double* gz) const {  // :156-167
    for (int z = 0, i = 0; z < g.nz; z++) {
      const int l = z * g.layer; const double rr = t.rho[z], rUp = z < g.nz - 1 ? (t.rho[z] + t.rho[z + 1]) / 2 : 0;
      for (int y = 0; y < g.ny; y++)
        for (int x = 0; x < g.nx; x++, i++) {
          const uint8_t o = open[i];
          gx[i] += o & 1 ? sign * rr * (phi[g.xo[3][x] + y * g.nx + l] - phi[i]) / g.dx : 0;
          gy[i] += o & 2 ? sign * rr * (phi[x + g.yo[3][y] + l] - phi[i]) / g.dy : 0;
          gz[i] += o & 4 ? sign * rUp * (phi[i + g.layer] - phi[i]) / g.dzs[z] : 0;
        }
    }
  }

  void applyMasked(const double* dd, double* out) {  // :170-176
    std::fill(fx.begin(), fx.end(), 0.0); std::fill(fy.begin(), fy.end(), 0.0); std::fill(fz.begin(), fz.end(), 0.0);
    maskedGradient(dd, 1, fx.data(), fy.data(), fz.data());
    terrainDivergence(out, fx.data(), fy.data(), fz.data());
    for (size_t i = 0; i < (size_t)g.n; i++) out[i] = -out[i];
  }

  void flatSolve(const double* rv, double* out) {  // :179-184
    for (size_t i = 0; i < (size_t)g.n; i++) t.div[i] = -rv[i] / g.hz[i / g.layer];
    t.forward(0, g.nz, ds); t.modes(0, g.ny, ms); t.inverse(0, g.nz, ds);
    std::copy(t.phi.begin(), t.phi.end(), out);
  }

  template <class S> void setVelocityMasked(Arr<S> u, Arr<S> v, Arr<S> w, double tolerance = 1e-10, int maxIterations = 400) {  // :115-153
    const size_t n = g.n;
    t.faces<S>(u, v, w, 0, g.nz);
    for (size_t i = 0; i < n; i++) { if (!(open[i] & 1)) t.mx[i] = 0; if (!(open[i] & 2)) t.my[i] = 0; if (!(open[i] & 4)) t.mz[i] = 0; }
    terrainDivergence(b.data(), t.mx.data(), t.my.data(), t.mz.data());
    double bb = 0;
    for (size_t i = 0; i < n; i++) { b[i] = -b[i]; bb += b[i] * b[i]; }
    std::fill(q.begin(), q.end(), 0.0);
    if (bb > 0) {
      r = b;
      flatSolve(r.data(), zz.data());
      double rz = 0;
      for (size_t i = 0; i < n; i++) { d[i] = zz[i]; rz += r[i] * zz[i]; }
      int k = 0; double rr = bb;
      for (; k < maxIterations && rr > tolerance * tolerance * bb; k++) {
        applyMasked(d.data(), sd.data());
        double dsd = 0;
        for (size_t i = 0; i < n; i++) dsd += d[i] * sd[i];
        if (!(dsd > 0)) break;
        const double alpha = rz / dsd;
        rr = 0;
        for (size_t i = 0; i < n; i++) { q[i] += alpha * d[i]; r[i] -= alpha * sd[i]; rr += r[i] * r[i]; }
        flatSolve(r.data(), zz.data());
        double rzNew = 0;
        for (size_t i = 0; i < n; i++) rzNew += r[i] * zz[i];
        const double beta = rzNew / rz;
        rz = rzNew;
        for (size_t i = 0; i < n; i++) d[i] = zz[i] + beta * d[i];
      }
      iterations = k; residual = std::sqrt(rr / bb);
    } else { iterations = 0; residual = 0; }
    maskedGradient(q.data(), -1, t.mx.data(), t.my.data(), t.mz.data());
    terrainDivergence(t.div.data(), t.mx.data(), t.my.data(), t.mz.data());
    for (size_t i = 0; i < n; i++) t.div[i] /= hn[i];
  }
};

}  // namespace terrain
}  // namespace orc
