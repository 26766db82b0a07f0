// TEST INFRASTRUCTURE ONLY — the oracle's elliptic solvers, transport and turbulence (see oracle_core.h).
// Restates src/core/spectral.ts (FFT, HorizontalDFT), src/core/pressure.ts (PressureSolver),
// src/core/advection.ts (FluxTransport, weno, upwind5) and src/core/turbulence.ts (Turbulence).
#pragma once
#include "oracle_core.h"

namespace orc {

struct GridSpec {
  int nx, ny, nz, n, layer;
  double dx, dy, dz, width, depth, height;
  std::vector<double> zs, dzs, hz;
  std::vector<int> xp, xm, yp, ym;     // src/core/grid.ts:125-128
  std::vector<int> xo[6], yo[6];       // offsets -2..3 (src/core/advection.ts:41-42)
  void finish() {
    n = nx * ny * nz; layer = nx * ny;
    xp.resize(nx); xm.resize(nx); yp.resize(ny); ym.resize(ny);
    for (int x = 0; x < nx; x++) { xp[x] = (x + 1) % nx; xm[x] = (x + nx - 1) % nx; }
    for (int y = 0; y < ny; y++) { yp[y] = (y + 1) % ny * nx; ym[y] = (y + ny - 1) % ny * nx; }
    for (int o = 0; o < 6; o++) {
      xo[o].resize(nx); yo[o].resize(ny);
      for (int x = 0; x < nx; x++) xo[o][x] = (x + (o - 2) + 2 * nx) % nx;
      for (int y = 0; y < ny; y++) yo[o][y] = ((y + (o - 2) + 2 * ny) % ny) * nx;
    }
  }
};

// ---------------------------------------------------------------- src/core/spectral.ts:8-73
struct FFT {
  int n = 0;
  std::vector<double> twRe, twIm, outRe, outIm, scrRe, scrIm;
  std::vector<int> factors;
  FFT() {}
  explicit FFT(int n_) : n(n_) {
    twRe.resize(n); twIm.resize(n);
    for (int k = 0; k < n; k++) { twRe[k] = std::cos(2 * PI * k / n); twIm[k] = -std::sin(2 * PI * k / n); }
    int rest = n, p = 4, largest = 1;
    while (rest > 1) {
      while (rest % p) { p = p == 4 ? 2 : p == 2 ? 3 : p + 2; if (p * p > rest) p = rest; }
      rest /= p; factors.push_back(p); factors.push_back(rest); largest = std::max(largest, p);
    }
    outRe.assign(n, 0); outIm.assign(n, 0); scrRe.assign(largest, 0); scrIm.assign(largest, 0);
  }
  void transform(double* re, double* im, int sign) {
    if (n == 1) return;
    if (sign > 0) for (int k = 0; k < n; k++) im[k] = -im[k];
    work(0, re, im, 0, 1, 0);
    for (int k = 0; k < n; k++) { re[k] = outRe[k]; im[k] = sign > 0 ? -outIm[k] : outIm[k]; }
  }
  void work(int out, const double* re, const double* im, int src, int stride, int f) {
    int p = factors[f], m = factors[f + 1];
    double *oRe = outRe.data(), *oIm = outIm.data();
    if (m == 1) for (int k = 0; k < p; k++) { oRe[out + k] = re[src + k * stride]; oIm[out + k] = im[src + k * stride]; }
    else for (int k = 0; k < p; k++) work(out + k * m, re, im, src + k * stride, stride * p, f + 2);
    const double *tr = twRe.data(), *ti = twIm.data();
    if (p == 2) {
      for (int u = 0, t = 0; u < m; u++, t += stride) {
        int a = out + u, b = a + m; double c = tr[t], s = ti[t], xr = oRe[b] * c - oIm[b] * s, xi = oRe[b] * s + oIm[b] * c;
        oRe[b] = oRe[a] - xr; oIm[b] = oIm[a] - xi; oRe[a] += xr; oIm[a] += xi;
      }
      return;
    }
    if (p == 4) {
      for (int u = 0, t = 0; u < m; u++, t += stride) {
        int a = out + u, b = a + m, c = b + m, d = c + m, t2 = 2 * t, t3 = 3 * t;
        double r0 = oRe[b] * tr[t] - oIm[b] * ti[t], i0 = oRe[b] * ti[t] + oIm[b] * tr[t];
        double r1 = oRe[c] * tr[t2] - oIm[c] * ti[t2], i1 = oRe[c] * ti[t2] + oIm[c] * tr[t2];
        double r2 = oRe[d] * tr[t3] - oIm[d] * ti[t3], i2 = oRe[d] * ti[t3] + oIm[d] * tr[t3];
        double r5 = oRe[a] - r1, i5 = oIm[a] - i1, ra = oRe[a] + r1, ia = oIm[a] + i1, r3 = r0 + r2, i3 = i0 + i2, r4 = r0 - r2, i4 = i0 - i2;
        oRe[c] = ra - r3; oIm[c] = ia - i3; oRe[a] = ra + r3; oIm[a] = ia + i3;
        oRe[b] = r5 + i4; oIm[b] = i5 - r4; oRe[d] = r5 - i4; oIm[d] = i5 + r4;
      }
      return;
    }
    double *sRe = scrRe.data(), *sIm = scrIm.data();
    for (int u = 0; u < m; u++) {
      for (int q = 0; q < p; q++) { sRe[q] = oRe[out + u + q * m]; sIm[q] = oIm[out + u + q * m]; }
      for (int q1 = 0, k = u; q1 < p; q1++, k += m) {
        double a = sRe[0], b = sIm[0]; int t = 0; int step = stride * k;
        for (int q = 1; q < p; q++) { t += step; if (t >= n) t -= n; double c = tr[t], s = ti[t]; a += sRe[q] * c - sIm[q] * s; b += sRe[q] * s + sIm[q] * c; }
        oRe[out + k] = a; oIm[out + k] = b;
      }
    }
  }
};

// Per-thread scratch of a 2-D transform (the reference keeps one per model/helper thread).
struct DftScratch {
  FFT fx, fy; std::vector<double> rowRe, rowIm;
  DftScratch() {}
  DftScratch(int nx, int ny) : fx(nx), fy(ny), rowRe(std::max(nx, ny)), rowIm(std::max(nx, ny)) {}
};

// src/core/spectral.ts:81-152: spectra at [layer*nx*ny + n*nx + m], m <= nx/2.
struct HorizontalDFT {
  int nx, ny, mh; std::vector<double> re, im;
  HorizontalDFT() : nx(0), ny(0), mh(0) {}
  HorizontalDFT(int nx_, int ny_, int layers) : nx(nx_), ny(ny_), mh(nx_ / 2), re((size_t)nx_ * ny_ * layers), im((size_t)nx_ * ny_ * layers) {}
  template <class Src> void forwardLayers(const Src& src, int k0, int k1, DftScratch& s) {
    int cl = nx * ny; double *rowRe = s.rowRe.data(), *rowIm = s.rowIm.data();
    for (int k = k0; k < k1; k++) {
      size_t base = (size_t)k * cl;
      for (int j = 0; j < ny; j += 2) {
        size_t row = base + (size_t)j * nx, row2 = row + nx; bool pair = j + 1 < ny;
        for (int i = 0; i < nx; i++) { rowRe[i] = src(row + i); rowIm[i] = pair ? (double)src(row2 + i) : 0; }
        s.fx.transform(rowRe, rowIm, -1);
        for (int m = 0; m <= mh; m++) {
          int c = m ? nx - m : 0; double zr = rowRe[m], zi = rowIm[m], cr = rowRe[c], ci = rowIm[c];
          re[row + m] = (zr + cr) / 2; im[row + m] = (zi - ci) / 2;
          if (pair) { re[row2 + m] = (zi + ci) / 2; im[row2 + m] = (cr - zr) / 2; }
        }
      }
      for (int m = 0; m <= mh; m++) {
        for (int j = 0; j < ny; j++) { rowRe[j] = re[base + (size_t)j * nx + m]; rowIm[j] = im[base + (size_t)j * nx + m]; }
        s.fy.transform(rowRe, rowIm, -1);
        for (int n = 0; n < ny; n++) { re[base + (size_t)n * nx + m] = rowRe[n]; im[base + (size_t)n * nx + m] = rowIm[n]; }
      }
    }
  }
  template <class Dst> void inverseLayers(Dst dst, int k0, int k1, DftScratch& s) {
    int cl = nx * ny; double *rowRe = s.rowRe.data(), *rowIm = s.rowIm.data();
    for (int k = k0; k < k1; k++) {
      size_t base = (size_t)k * cl;
      for (int m = 0; m <= mh; m++) {
        for (int n = 0; n < ny; n++) { rowRe[n] = re[base + (size_t)n * nx + m]; rowIm[n] = im[base + (size_t)n * nx + m]; }
        s.fy.transform(rowRe, rowIm, 1);
        for (int j = 0; j < ny; j++) { re[base + (size_t)j * nx + m] = rowRe[j]; im[base + (size_t)j * nx + m] = rowIm[j]; }
      }
      for (int j = 0; j < ny; j += 2) {
        size_t row = base + (size_t)j * nx, row2 = row + nx; bool pair = j + 1 < ny;
        for (int m = 0; m < nx; m++) {
          int c = m <= mh ? m : nx - m; double sg = m <= mh ? 1 : -1; bool real = c == 0 || 2 * c == nx;
          double ar = re[row + c], ai = real ? 0 : sg * im[row + c], br = pair ? re[row2 + c] : 0, bi = pair && !real ? sg * im[row2 + c] : 0;
          rowRe[m] = ar - bi; rowIm[m] = ai + br;
        }
        s.fx.transform(rowRe, rowIm, 1);
        for (int i = 0; i < nx; i++) { dst(row + i, rowRe[i] / cl); if (pair) dst(row2 + i, rowIm[i] / cl); }
      }
    }
  }
};

struct ModeScratch { std::vector<double> cp, dRe, dIm; explicit ModeScratch(int nz = 0) : cp(nz), dRe(nz), dIm(nz) {} };

// ---------------------------------------------------------------- src/core/pressure.ts:18-141
struct PressureSolver {
  const GridSpec* g; int cells; HorizontalDFT dft; std::vector<double> alpha, beta, rho;
  PressureSolver() : g(nullptr), cells(0) {}
  PressureSolver(const GridSpec& grid, const double* density) : g(&grid), cells(grid.nx * grid.ny * (grid.nz - 1)), dft(grid.nx, grid.ny, grid.nz - 1) {
    int nx = grid.nx, ny = grid.ny;
    rho.resize(grid.nz);
    for (int k = 0; k < grid.nz; k++) rho[k] = density ? density[k] : 1;
    alpha.resize((size_t)nx * ny); beta.resize((size_t)nx * ny);
    auto exact = [](double x) { return x < 1e-12 ? 0 : x > 1 - 1e-12 ? 1 : x; };
    for (int n = 0; n < ny; n++) for (int m = 0; m < nx; m++) {
      double sx = exact(std::pow(std::sin(PI * m / nx), 2)), cx = exact(std::pow(std::cos(PI * m / nx), 2));
      double sy = exact(std::pow(std::sin(PI * n / ny), 2)), cy = exact(std::pow(std::cos(PI * n / ny), 2));
      alpha[m + nx * n] = 4 * (sx * cy / (grid.dx * grid.dx) + cx * sy / (grid.dy * grid.dy));
      beta[m + nx * n] = cx * cy;
    }
  }
  template <class S> void divergence(Arr<S> u, Arr<S> v, Arr<S> w, double dt, double* out, int k0, int k1) const {
    const GridSpec& G_ = *g; int nx = G_.nx, ny = G_.ny, layer = G_.layer;
    for (int k = k0; k < k1; k++) {
      size_t c = (size_t)k * nx * ny;
      int l0 = k * layer, l1 = l0 + layer; double r0 = rho[k] / 4, r1 = rho[k + 1] / 4, dz = G_.dzs[k];
      for (int j = 0; j < ny; j++) {
        int y0 = j * nx, y1 = ((j + 1) % ny) * nx;
        for (int i = 0; i < nx; i++, c++) {
          int i1 = (i + 1) % nx;
          int a = i + y0 + l0, b = i1 + y0 + l0, e = i + y1 + l0, f = i1 + y1 + l0, gg = i + y0 + l1, h = i1 + y0 + l1, s = i + y1 + l1, t = i1 + y1 + l1;
          double ddx = (r0 * ((double)u[b] + (double)u[f] - (double)u[a] - (double)u[e]) + r1 * ((double)u[h] + (double)u[t] - (double)u[gg] - (double)u[s])) / G_.dx;
          double ddy = (r0 * ((double)v[e] + (double)v[f] - (double)v[a] - (double)v[b]) + r1 * ((double)v[s] + (double)v[t] - (double)v[gg] - (double)v[h])) / G_.dy;
          double ddz = (r1 * ((double)w[gg] + (double)w[h] + (double)w[s] + (double)w[t]) - r0 * ((double)w[a] + (double)w[b] + (double)w[e] + (double)w[f])) / dz;
          out[c] = (ddx + ddy + ddz) / dt;
        }
      }
    }
  }
  template <class S> void correct(const double* p, Arr<S> u, Arr<S> v, Arr<S> w, double dt, int k0, int k1) const {
    const GridSpec& G_ = *g; int nx = G_.nx, ny = G_.ny, nz = G_.nz, layer = G_.layer, cl = nx * ny;
    for (int k = k0; k < k1; k++) {
      size_t lo = (size_t)std::max(0, k - 1) * cl, hi = (size_t)std::min(nz - 2, k) * cl;
      double wLo = k > 0 ? G_.dzs[k - 1] / G_.hz[k] : 0, wHi = k < nz - 1 ? G_.dzs[k] / G_.hz[k] : 0;
      for (int j = 0; j < ny; j++) {
        int jm = ((j + ny - 1) % ny) * nx, j0 = j * nx;
        for (int i = 0; i < nx; i++) {
          int im = (i + nx - 1) % nx, node = i + j * nx + k * layer;
          auto P = [&](int ii, int jj, size_t base) { return p[base + ii + jj]; };
          double gx = (wLo * (P(i, jm, lo) + P(i, j0, lo) - P(im, jm, lo) - P(im, j0, lo)) + wHi * (P(i, jm, hi) + P(i, j0, hi) - P(im, jm, hi) - P(im, j0, hi))) / (4 * G_.dx);
          double gy = (wLo * (P(im, j0, lo) + P(i, j0, lo) - P(im, jm, lo) - P(i, jm, lo)) + wHi * (P(im, j0, hi) + P(i, j0, hi) - P(im, jm, hi) - P(i, jm, hi))) / (4 * G_.dy);
          u[node] -= dt * gx; v[node] -= dt * gy;
          if (k > 0 && k < nz - 1) {
            size_t below = (size_t)(k - 1) * cl, above = (size_t)k * cl;
            double gz = (P(im, jm, above) + P(i, jm, above) + P(im, j0, above) + P(i, j0, above) - P(im, jm, below) - P(i, jm, below) - P(im, j0, below) - P(i, j0, below)) / (4 * G_.hz[k]);
            w[node] -= dt * gz;
          }
        }
      }
    }
  }
  void transform(const double* rhs, int k0, int k1, DftScratch& s) { dft.forwardLayers([rhs](size_t i) { return rhs[i]; }, k0, k1, s); }
  void back(double* p, int k0, int k1, DftScratch& s) { dft.inverseLayers([p](size_t i, double v) { p[i] = v; }, k0, k1, s); }
  void modes(int n0, int n1, ModeScratch& ms) {
    const GridSpec& G_ = *g; int nx = G_.nx, cl = nx * G_.ny, nc = G_.nz - 1, mh = dft.mh;
    for (int n = n0; n < n1; n++) for (int m = 0; m <= mh; m++) {
      int mode = m + nx * n; double a = alpha[mode], b = beta[mode];
      if ((a == 0 && b == 0) || (nc == 1 && a == 0)) { for (int k = 0; k < nc; k++) dft.re[mode + (size_t)k * cl] = dft.im[mode + (size_t)k * cl] = 0; continue; }
      tridiagonal(mode, a, b, nc, cl, ms);
    }
  }
  void tridiagonal(int mode, double a, double b, int nc, int cl, ModeScratch& ms) {
    const GridSpec& G_ = *g; const double *dzs = G_.dzs.data(), *hz = G_.hz.data();
    double *cp = ms.cp.data(), *dRe = ms.dRe.data(), *dIm = ms.dIm.data();
    bool pinned = a == 0;
    for (int k = 0; k < nc; k++) {
      double di = -a / 2 * (rho[k] * dzs[k] / (2 * hz[k]) + rho[k + 1] * dzs[k] / (2 * hz[k + 1])), lo = 0, up = 0;
      if (k > 0) { lo = -a / 2 * rho[k] * dzs[k - 1] / (2 * hz[k]); double v = b * rho[k] / (hz[k] * dzs[k]); lo += v; di -= v; }
      if (k < nc - 1) { up = -a / 2 * rho[k + 1] * dzs[k + 1] / (2 * hz[k + 1]); double v = b * rho[k + 1] / (hz[k + 1] * dzs[k]); up += v; di -= v; }
      double r = dft.re[mode + (size_t)k * cl], s = dft.im[mode + (size_t)k * cl];
      if (pinned && k == 0) { lo = 0; di = 1; up = 0; r = 0; s = 0; }
      if (pinned && k == 1) lo = 0;
      double m = k == 0 ? di : di - lo * cp[k - 1];
      cp[k] = up / m;
      dRe[k] = (r - lo * (k == 0 ? 0 : dRe[k - 1])) / m;
      dIm[k] = (s - lo * (k == 0 ? 0 : dIm[k - 1])) / m;
    }
    for (int k = nc - 1; k >= 0; k--) {
      if (k < nc - 1) { dRe[k] -= cp[k] * dRe[k + 1]; dIm[k] -= cp[k] * dIm[k + 1]; }
      dft.re[mode + (size_t)k * cl] = dRe[k]; dft.im[mode + (size_t)k * cl] = dIm[k];
    }
  }
};

// ---------------------------------------------------------------- src/core/advection.ts:385-399
inline double upwind5(double a, double b, double c, double d, double e) { return (2 * a - 13 * b + 47 * c + 27 * d - 3 * e) / 60; }
inline double weno(double a, double b, double c, double d, double e) {
  if (a == 0 && b == 0 && c == 0 && d == 0 && e == 0) return 0;
  double p0 = (2 * a - 7 * b + 11 * c) / 6, p1 = (-b + 5 * c + 2 * d) / 6, p2 = (2 * c + 5 * d - e) / 6;
  double s0 = a - 2 * b + c, t0 = a - 4 * b + 3 * c, s1 = b - 2 * c + d, t1 = b - d, s2 = c - 2 * d + e, t2 = 3 * c - 4 * d + e;
  double eps = 2e-7 * (a * a + b * b + c * c + d * d + e * e) + 1e-40;
  double b0 = eps + 13.0 / 12 * s0 * s0 + .25 * t0 * t0, b1 = eps + 13.0 / 12 * s1 * s1 + .25 * t1 * t1, b2 = eps + 13.0 / 12 * s2 * s2 + .25 * t2 * t2;
  double c0 = b0 * b0, c1 = b1 * b1, c2 = b2 * b2, w0 = .1 * c1 * c2, w1 = .6 * c0 * c2, w2 = .3 * c0 * c1;
  return (w0 * p0 + w1 * p1 + w2 * p2) / (w0 + w1 + w2);
}
constexpr double RK3[3] = {1.0 / 3, 1.0 / 2, 1.0};

// Per-thread scratch of one field's transport tendency.
struct TendScratch {
  std::vector<double> fx, fy, fz; std::vector<uint8_t> rowNonzero, rowActive;
  TendScratch() {}
  TendScratch(int n, int rows) : fx(n), fy(n), fz(n), rowNonzero(rows), rowActive(rows) {}
};

// ---------------------------------------------------------------- src/core/advection.ts:17-379 (flat ground)
struct FluxTransport {
  const GridSpec* g; std::vector<double> rho, mx, my, mz, div, phi, lambda; HorizontalDFT dft;
  FluxTransport() : g(nullptr) {}
  FluxTransport(const GridSpec& grid, const double* density) : g(&grid), rho(density, density + grid.nz), mx(grid.n), my(grid.n), mz(grid.n), div(grid.n), phi(grid.n),
      lambda((size_t)grid.nx * grid.ny), dft(grid.nx, grid.ny, grid.nz) {
    for (int mode = 0; mode < grid.nx * grid.ny; mode++) {
      int m = mode % grid.nx, n = mode / grid.nx;
      lambda[mode] = m == 0 && n == 0 ? 0 : 4 * std::pow(std::sin(PI * m / grid.nx), 2) / (grid.dx * grid.dx) + 4 * std::pow(std::sin(PI * n / grid.ny), 2) / (grid.dy * grid.dy);
    }
  }
  template <class S> void faces(Arr<S> u, Arr<S> v, Arr<S> w, int z0, int z1) {  // :190-200
    const GridSpec& G_ = *g; int nx = G_.nx, ny = G_.ny, nz = G_.nz, layer = G_.layer;
    for (int z = z0; z < z1; z++) {
      size_t i = (size_t)z * layer; int l = z * layer; double r = rho[z], rUp = z < nz - 1 ? (rho[z] + rho[z + 1]) / 2 : 0;
      for (int y = 0; y < ny; y++) for (int x = 0; x < nx; x++, i++) {
        mx[i] = r * ((double)u[i] + (double)u[G_.xo[3][x] + y * nx + l]) / 2;
        my[i] = r * ((double)v[i] + (double)v[x + G_.yo[3][y] + l]) / 2;
        mz[i] = z < nz - 1 ? rUp * ((double)w[i] + (double)w[i + layer]) / 2 : 0;
      }
    }
  }
  void divergence(int z0, int z1) {  // :203-211
    const GridSpec& G_ = *g; int nx = G_.nx, ny = G_.ny, layer = G_.layer;
    for (int z = z0; z < z1; z++) {
      size_t i = (size_t)z * layer; int l = z * layer;
      for (int y = 0; y < ny; y++) for (int x = 0; x < nx; x++, i++)
        div[i] = (mx[i] - mx[G_.xo[1][x] + y * nx + l]) / G_.dx + (my[i] - my[x + G_.yo[1][y] + l]) / G_.dy + (mz[i] - (z > 0 ? mz[i - layer] : 0)) / G_.hz[z];
    }
  }
  void forward(int z0, int z1, DftScratch& s) { const double* d = div.data(); dft.forwardLayers([d](size_t i) { return d[i]; }, z0, z1, s); }
  void inverse(int z0, int z1, DftScratch& s) { double* p = phi.data(); dft.inverseLayers([p](size_t i, double v) { p[i] = v; }, z0, z1, s); }
  void modes(int n0, int n1, ModeScratch& ms) {  // :222-241
    const GridSpec& G_ = *g; int nx = G_.nx, nz = G_.nz, layer = G_.layer; const double *h = G_.hz.data(), *dzs = G_.dzs.data();
    double *cp = ms.cp.data(), *dRe = ms.dRe.data(), *dIm = ms.dIm.data();
    auto face = [&](int k) { return k < 0 || k >= nz - 1 ? 0.0 : (rho[k] + rho[k + 1]) / 2; };
    for (int n = n0; n < n1; n++) for (int m = 0; m <= dft.mh; m++) {
      int mode = m + nx * n; double lam = lambda[mode]; bool pinned = lam == 0;
      for (int k = 0; k < nz; k++) {
        double lo = k > 0 ? face(k - 1) / dzs[k - 1] : 0, up = k < nz - 1 ? face(k) / dzs[k] : 0, di = -rho[k] * h[k] * lam - lo - up;
        double rr = h[k] * dft.re[mode + (size_t)k * layer], ri = h[k] * dft.im[mode + (size_t)k * layer];
        if (pinned && k == 0) { lo = 0; di = 1; up = 0; rr = 0; ri = 0; }
        if (pinned && k == 1) lo = 0;
        double piv = k == 0 ? di : di - lo * cp[k - 1];
        cp[k] = up / piv;
        dRe[k] = (rr - (k == 0 ? 0 : lo * dRe[k - 1])) / piv;
        dIm[k] = (ri - (k == 0 ? 0 : lo * dIm[k - 1])) / piv;
      }
      for (int k = nz - 1; k >= 0; k--) {
        if (k < nz - 1) { dRe[k] -= cp[k] * dRe[k + 1]; dIm[k] -= cp[k] * dIm[k + 1]; }
        dft.re[mode + (size_t)k * layer] = dRe[k]; dft.im[mode + (size_t)k * layer] = dIm[k];
      }
    }
  }
  void correctFaces(int z0, int z1) {  // :244-255
    const GridSpec& G_ = *g; int nx = G_.nx, ny = G_.ny, nz = G_.nz, layer = G_.layer;
    auto face = [&](int k) { return k < 0 || k >= nz - 1 ? 0.0 : (rho[k] + rho[k + 1]) / 2; };
    for (int z = z0; z < z1; z++) {
      size_t i = (size_t)z * layer; int l = z * layer; double r = rho[z], rUp = face(z);
      for (int y = 0; y < ny; y++) for (int x = 0; x < nx; x++, i++) {
        mx[i] -= r * (phi[G_.xo[3][x] + y * nx + l] - phi[i]) / G_.dx;
        my[i] -= r * (phi[x + G_.yo[3][y] + l] - phi[i]) / G_.dy;
        if (z < nz - 1) mz[i] -= rUp * (phi[i + layer] - phi[i]) / G_.dzs[z];
      }
    }
  }
  // setVelocity (:55-60) with a single scratch.
  template <class S> void setVelocity(Arr<S> u, Arr<S> v, Arr<S> w, DftScratch& s, ModeScratch& ms) {
    int nz = g->nz, ny = g->ny;
    faces<S>(u, v, w, 0, nz); divergence(0, nz); forward(0, nz, s); modes(0, ny, ms); inverse(0, nz, s); correctFaces(0, nz); divergence(0, nz);
  }
  template <class S> int markActiveRows(Arr<S> q, int z0, int z1, TendScratch& ts) {  // :282-292
    const GridSpec& G_ = *g; int nx = G_.nx, ny = G_.ny, nz = G_.nz; uint8_t *rows = ts.rowNonzero.data(), *active = ts.rowActive.data();
    for (int r = std::max(0, z0 - 3) * ny; r < std::min(nz, z1 + 3) * ny; r++) {
      size_t b = (size_t)r * nx; uint8_t any = 0; for (int x = 0; x < nx; x++) if ((double)q[b + x] != 0) { any = 1; break; } rows[r] = any;
    }
    int count = 0;
    for (int z = z0; z < z1; z++) for (int y = 0; y < ny; y++) {
      uint8_t any = 0;
      for (int dz = -3; dz <= 3 && !any; dz++) { int zz = z + dz; if (zz < 0 || zz >= nz) continue; for (int dy = -3; dy <= 3; dy++) if (rows[zz * ny + (y + dy + ny) % ny]) { any = 1; break; } }
      active[z * ny + y] = any; count += any;
    }
    return count;
  }
  // :274-378 (flat ground): monotone = WENO5 with the empty-row skip, else linear fifth-order upwind.
  template <class S> void tendency(Arr<S> q, double* tend, int z0, int z1, bool monotone, TendScratch& ts) {
    const GridSpec& G_ = *g; int nx = G_.nx, ny = G_.ny, nz = G_.nz, layer = G_.layer;
    double *fx = ts.fx.data(), *fy = ts.fy.data(), *fz = ts.fz.data();
    const int *xm2 = G_.xo[0].data(), *xm1 = G_.xo[1].data(), *xp1 = G_.xo[3].data(), *xp2 = G_.xo[4].data(), *xp3 = G_.xo[5].data();
    const int *ym2 = G_.yo[0].data(), *ym1 = G_.yo[1].data(), *yp1 = G_.yo[3].data(), *yp2 = G_.yo[4].data(), *yp3 = G_.yo[5].data();
    uint8_t* active = ts.rowActive.data();
    int below = std::max(0, z0 - 1);
    if (monotone && markActiveRows<S>(q, below, z1, ts) == 0) { for (size_t i = (size_t)z0 * layer; i < (size_t)z1 * layer; i++) tend[i] = 0; return; }
    auto rec = [monotone](double a, double b, double c, double d, double e) { return monotone ? weno(a, b, c, d, e) : upwind5(a, b, c, d, e); };
    for (int z = below; z < z1; z++) {
      size_t i = (size_t)z * layer; int l = z * layer; bool top = z == nz - 1;
      int zm2 = std::max(0, z - 2) * layer, zm1 = std::max(0, z - 1) * layer, zp1 = std::min(nz - 1, z + 1) * layer, zp2 = std::min(nz - 1, z + 2) * layer, zp3 = std::min(nz - 1, z + 3) * layer;
      for (int y = 0; y < ny; y++) {
        int row = y * nx + l, c0 = y * nx;
        if (monotone && !active[z * ny + y]) { for (int x = 0; x < nx; x++) fx[i + x] = fy[i + x] = fz[i + x] = 0; i += nx; continue; }
        for (int x = 0; x < nx; x++, i++) {
          double m1 = mx[i];
          fx[i] = m1 >= 0 ? m1 * rec(q[xm2[x] + row], q[xm1[x] + row], q[i], q[xp1[x] + row], q[xp2[x] + row]) : m1 * rec(q[xp3[x] + row], q[xp2[x] + row], q[xp1[x] + row], q[i], q[xm1[x] + row]);
          double m2 = my[i];
          fy[i] = m2 >= 0 ? m2 * rec(q[x + ym2[y] + l], q[x + ym1[y] + l], q[i], q[x + yp1[y] + l], q[x + yp2[y] + l]) : m2 * rec(q[x + yp3[y] + l], q[x + yp2[y] + l], q[x + yp1[y] + l], q[i], q[x + ym1[y] + l]);
          double m3 = mz[i]; int c = x + c0;
          fz[i] = top ? 0 : m3 >= 0 ? m3 * rec(q[c + zm2], q[c + zm1], q[i], q[c + zp1], q[c + zp2]) : m3 * rec(q[c + zp3], q[c + zp2], q[c + zp1], q[i], q[c + zm1]);
        }
      }
    }
    for (int z = z0; z < z1; z++) {
      size_t i = (size_t)z * layer; int l = z * layer; double r = rho[z], hz = G_.hz[z];
      for (int y = 0; y < ny; y++) {
        if (monotone && !active[z * ny + y]) { for (int x = 0; x < nx; x++) tend[i + x] = 0; i += nx; continue; }
        for (int x = 0; x < nx; x++, i++) {
          double flux = (fx[i] - fx[xm1[x] + y * nx + l]) / G_.dx + (fy[i] - fy[x + ym1[y] + l]) / G_.dy + (fz[i] - (z > 0 ? fz[i - layer] : 0)) / hz;
          tend[i] = -(flux - (double)q[i] * div[i]) / r;
        }
      }
    }
  }
  // advect (:261-268), for the transport tests.
  template <class S> void advect(Arr<S> a, double dt, bool monotone, TendScratch& ts, std::vector<double>& tend) {
    std::vector<S> start(g->n); for (int i = 0; i < g->n; i++) start[i] = a[i].v;
    for (double fraction : RK3) {
      tendency<S>(a, tend.data(), 0, g->nz, monotone, ts);
      for (int i = 0; i < g->n; i++) a[i] = (double)start[i] + fraction * dt * tend[i];
    }
  }
};

// ---------------------------------------------------------------- src/core/turbulence.ts:21-209 (flat ground)
struct Turbulence {
  const GridSpec* g; std::vector<double> rho, km, kh;
  bool anisotropic = false, verticalDz = false, implicitVertical = false, durranKlemp = false;
  Turbulence() : g(nullptr) {}
  Turbulence(const GridSpec& grid, const double* density) : g(&grid), rho(density, density + grid.nz), km(grid.n), kh(grid.n) {}
  // :87-137. moistQ/condensate null: dry N^2.
  template <class S> void viscosity(Arr<S> u, Arr<S> v, Arr<S> w, Arr<S> theta, const double* thetaEnv, double cs, double dt, Arr<S> moistQ, Arr<S> condensate, const double* exner, int z0, int z1) {
    const GridSpec& G_ = *g; int nx = G_.nx, ny = G_.ny, nz = G_.nz, layer = G_.layer; double dx = G_.dx, dy = G_.dy;
    double lenH2 = std::pow(cs * std::sqrt(dx * dy), 2), capH = .05 * std::pow(std::min(dx, dy), 2) / dt;
    bool implicit = implicitVertical && anisotropic;
    for (int z = z0; z < z1; z++) {
      size_t i = (size_t)z * layer;
      double local = z == 0 ? G_.dzs[0] : z == nz - 1 ? G_.dzs[nz - 2] : G_.hz[z];
      double len2 = std::pow(cs * (anisotropic && verticalDz ? local : std::cbrt(dx * dy * local)), 2);
      double cap = implicit ? INFINITY : .05 * std::pow(jmin(jmin(dx, dy), jmin(z > 0 ? G_.dzs[z - 1] : INFINITY, z < nz - 1 ? G_.dzs[z] : INFINITY)), 2) / dt;
      int up = z < nz - 1 ? layer : 0, below = z > 0 ? -layer : 0;
      double levelSpan = G_.zs[z + (up ? 1 : 0)] - G_.zs[z - (below ? 1 : 0)];
      for (int y = 0; y < ny; y++) {
        int row = y * nx + z * layer;
        for (int x = 0; x < nx; x++, i++) {
          int e = G_.xp[x] + row, wst = G_.xm[x] + row, n = x + G_.yp[y] + z * layer, s = x + G_.ym[y] + z * layer; double hx = 2 * dx, hy = 2 * dy, span = levelSpan; int down = below;
          double dudx = ((double)u[e] - (double)u[wst]) / hx, dvdy = ((double)v[n] - (double)v[s]) / hy, dwdz = ((double)w[i + up] - (double)w[i + down]) / span;
          double dudy = ((double)u[n] - (double)u[s]) / hy, dvdx = ((double)v[e] - (double)v[wst]) / hx;
          double dudz = ((double)u[i + up] - (double)u[i + down]) / span, dwdx = ((double)w[e] - (double)w[wst]) / hx;
          double dvdz = ((double)v[i + up] - (double)v[i + down]) / span, dwdy = ((double)w[n] - (double)w[s]) / hy;
          double s2 = 2 * (dudx * dudx + dvdy * dvdy + dwdz * dwdz) + std::pow(dudy + dvdx, 2) + std::pow(dudz + dwdx, 2) + std::pow(dvdz + dwdy, 2);
          double n2 = G / thetaEnv[z] * ((double)theta[i + up] - (double)theta[i + down]) / span;
          if (moistQ && (double)condensate[i] > 1e-5 && durranKlemp && (double)condensate[i + up] > 1e-5 && (double)condensate[i + down] > 1e-5) {
            size_t a = i + up, b = i + down; double t = (double)theta[i] * exner[z], qs = moistQ[i];
            double factor = (1 + LV * qs / (RD * t)) / (1 + EPS * LV * LV * qs / (CP * RD * t * t));
            n2 = G * (factor * (((double)theta[a] - (double)theta[b]) / (double)theta[i] + LV / (CP * t) * ((double)moistQ[a] - (double)moistQ[b])) - ((double)moistQ[a] + (double)condensate[a] - (double)moistQ[b] - (double)condensate[b])) / span;
          } else if (moistQ && (double)condensate[i] > 1e-5) {
            auto te = [&](size_t k, int level) { return (double)theta[k] * std::exp(LV * (double)moistQ[k] / (CP * (double)theta[k] * exner[level])); };
            n2 = G / te(i, z) * (te(i + up, z + (up ? 1 : 0)) - te(i + down, z - (down ? 1 : 0))) / span;
          }
          double rate = std::sqrt(jmax(0, s2 - n2 / PRANDTL));
          km[i] = jmin(cap, len2 * rate); kh[i] = anisotropic ? jmin(capH, lenH2 * rate) : km[i];
        }
      }
    }
  }
  // :143-185 (explicit, flat ground). `tmp` is the reference's Float32Array accumulator.
  template <class S> void mix(Arr<S> a, const double* base, double factor, double dt, std::vector<S>& tmpStore) {
    const GridSpec& G_ = *g; int nx = G_.nx, ny = G_.ny, nz = G_.nz, layer = G_.layer; const double* h = G_.hz.data();
    Arr<S> t = reinterpret_cast<Arr<S>>(tmpStore.data());
    for (int i = 0; i < G_.n; i++) t[i] = 0.0;
    bool implicit = implicitVertical && anisotropic;
    auto dev = [&](size_t i, int z) { return (double)a[i] - (base ? base[z] : 0); };
    size_t i = 0;
    for (int z = 0; z < nz; z++) {
      double rUp = z < nz - 1 ? (rho[z] + rho[z + 1]) / 2 : 0;
      for (int y = 0; y < ny; y++) {
        int row = y * nx + z * layer;
        for (int x = 0; x < nx; x++, i++) {
          double here = dev(i, z);
          int e = G_.xp[x] + row, n = x + G_.yp[y] + z * layer;
          { double fx = factor * (kh[i] + kh[e]) / 2 * (dev(e, z) - here) / G_.dx; t[i] += fx / G_.dx; t[e] -= fx / G_.dx; }
          { double fy = factor * (kh[i] + kh[n]) / 2 * (dev(n, z) - here) / G_.dy; t[i] += fy / G_.dy; t[n] -= fy / G_.dy; }
          if (z < nz - 1 && !implicit) {
            double fz = factor * rUp * (km[i] + km[i + layer]) / 2 * (dev(i + layer, z + 1) - here) / G_.dzs[z];
            t[i] += fz / (rho[z] * h[z]); t[i + layer] -= fz / (rho[z + 1] * h[z + 1]);
          }
        }
      }
    }
    for (int k = 0; k < G_.n; k++) a[k] += dt * (double)t[k];
    if (implicit) mixVertical<S>(a, base, factor, dt);
  }
  // :191-208
  template <class S> void mixVertical(Arr<S> a, const double* base, double factor, double dt) {
    const GridSpec& G_ = *g; int nz = G_.nz, layer = G_.layer; const double *h = G_.hz.data(), *dzs = G_.dzs.data();
    std::vector<double> lo(nz), up(nz), dg(nz), r(nz);
    for (int c = 0; c < layer; c++) {
      for (int z = 0; z < nz; z++) { lo[z] = 0; up[z] = 0; r[z] = (double)a[c + (size_t)z * layer] - (base ? base[z] : 0); }
      for (int z = 0; z < nz - 1; z++) {
        size_t i = c + (size_t)z * layer; double face = dt * factor * (rho[z] + rho[z + 1]) / 2 * (km[i] + km[i + layer]) / 2 / dzs[z];
        up[z] = face / (rho[z] * h[z]); lo[z + 1] = face / (rho[z + 1] * h[z + 1]);
      }
      for (int z = 0; z < nz; z++) dg[z] = 1 + lo[z] + up[z];
      for (int z = 1; z < nz; z++) { double f = lo[z] / dg[z - 1]; dg[z] -= f * up[z - 1]; r[z] += f * r[z - 1]; }
      r[nz - 1] /= dg[nz - 1];
      for (int z = nz - 2; z >= 0; z--) r[z] = (r[z] + up[z] * r[z + 1]) / dg[z];
      for (int z = 0; z < nz; z++) a[c + (size_t)z * layer] = r[z] + (base ? base[z] : 0);
    }
  }
};

}  // namespace orc
