// The storm's electric potential on the device (src/core/electric.ts:15-60): Laplacian(phi) = -rho/eps0 at the nodes,
// phi = 0 on the ground and top levels, periodic in x and y. A 2-D DFT of each interior level's right-hand side, one
// stretched vertical tridiagonal per horizontal mode with fixed ends (Thomas, the reference's rows and pivots), the
// inverse DFT. All in FP64: the reference's own tests hold the solution to 1e-9 of the discrete Poisson equation and
// the plate field to 5e-7. The DFTs are direct sums over exact FP64 twiddle tables, one output a thread: x (real to
// half-complex) per row, then y per level and x-mode; the inverse in the opposite order. Used by the standalone solver
// (sg_electric.cu) and by the lightning of an electrified run (sg_lightning.cu), each on its own buffers.
#pragma once
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <vector>

namespace {

constexpr double EPSILON0 = 8.8541878128e-12;  // src/core/electric.ts:6
constexpr double PI = 3.14159265358979323846;

// Forward x-DFT of one interior level's row: S1[j][m][y] = sum_x (-rho / eps0) e^{-2 pi i m x / nx}, m <= nx / 2.
__global__ void k_elec_xdft(const double* __restrict__ rho, double2* __restrict__ S1, const double2* __restrict__ twx, int nx, int ny, int mh) {
  extern __shared__ double row[];
  const int y = blockIdx.x, j = blockIdx.y, layer = nx * ny;
  const double* src = rho + (size_t)(j + 1) * layer + (size_t)y * nx;
  for (int x = threadIdx.x; x < nx; x += blockDim.x) row[x] = -src[x] / EPSILON0;
  __syncthreads();
  for (int m = threadIdx.x; m <= mh; m += blockDim.x) {
    double re = 0, im = 0;
    int t = 0;
    for (int x = 0; x < nx; x++) {
      const double2 w = twx[t];
      re = fma(row[x], w.x, re);
      im = fma(-row[x], w.y, im);
      t += m;
      if (t >= nx) t -= nx;
    }
    S1[((size_t)j * (mh + 1) + m) * ny + y] = make_double2(re, im);
  }
}

// y-DFT of one (level, x-mode) column: out[j][m][n] = sum_y in[j][m][y] e^{sign 2 pi i n y / ny}.
__global__ void k_elec_ydft(const double2* __restrict__ in, double2* __restrict__ out, const double2* __restrict__ twy, int ny, int mh, double sign) {
  extern __shared__ double2 col[];
  const int m = blockIdx.x, j = blockIdx.y;
  const size_t base = ((size_t)j * (mh + 1) + m) * ny;
  for (int y = threadIdx.x; y < ny; y += blockDim.x) col[y] = in[base + y];
  __syncthreads();
  for (int n = threadIdx.x; n < ny; n += blockDim.x) {
    double re = 0, im = 0;
    int t = 0;
    for (int y = 0; y < ny; y++) {
      const double2 w = twy[t], v = col[y];
      const double s = sign * w.y;
      re = fma(v.x, w.x, fma(-v.y, s, re));
      im = fma(v.y, w.x, fma(v.x, s, im));
      t += n;
      if (t >= ny) t -= ny;
    }
    out[base + n] = make_double2(re, im);
  }
}

// One horizontal mode (thread) over the interior levels, in place in S2[j][mode]: row j is node level k = j + 1,
// lo phi_{k-1} + di phi_k + up phi_{k+1} = rhs with phi = 0 at both ends (src/core/electric.ts:41-56). The pivots
// depend on the grid alone: cp = up / pivot and 1 / pivot come from the host (FP64), so a level costs two FMAs a lane.
// The right-hand sides arrive eight levels ahead of the recurrence; the forward values wait in a per-thread column.
constexpr int ELEC_MAXNI = 128;
__global__ void k_elec_thomas(double2* __restrict__ S2, const double* __restrict__ cp, const double* __restrict__ ipiv,
                              const double* __restrict__ lo_, int ni, int modes) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= modes) return;
  double2 col[ELEC_MAXNI];
  double2 d = make_double2(0, 0);
  for (int j0 = 0; j0 < ni; j0 += 8) {
    double2 r[8];
    double ip[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int j = min(j0 + q, ni - 1);
      r[q] = S2[(size_t)j * modes + g];
      ip[q] = ipiv[(size_t)j * modes + g];
    }
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int j = j0 + q;
      if (j < ni) {
        const double a = j > 0 ? lo_[j + 1] : 0;
        d = make_double2((r[q].x - a * d.x) * ip[q], (r[q].y - a * d.y) * ip[q]);
        col[j] = d;
      }
    }
  }
  S2[(size_t)(ni - 1) * modes + g] = d;
  for (int j1 = ni - 2; j1 >= 0; j1 -= 8) {
    double c[8];
#pragma unroll
    for (int q = 0; q < 8; q++) c[q] = cp[(size_t)max(j1 - q, 0) * modes + g];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int j = j1 - q;
      if (j >= 0) {
        const double2 v = col[j];
        d = make_double2(v.x - c[q] * d.x, v.y - c[q] * d.y);
        S2[(size_t)j * modes + g] = d;
      }
    }
  }
}

// Inverse x-DFT of one interior level's row from its half spectrum (the other half by Hermitian symmetry), over nx * ny.
__global__ void k_elec_xidft(const double2* __restrict__ S1, double* __restrict__ phi, const double2* __restrict__ twx, int nx, int ny, int mh) {
  extern __shared__ double2 z[];
  const int y = blockIdx.x, j = blockIdx.y, layer = nx * ny;
  for (int m = threadIdx.x; m <= mh; m += blockDim.x) z[m] = S1[((size_t)j * (mh + 1) + m) * ny + y];
  __syncthreads();
  const double scale = 1.0 / ((double)nx * ny);
  for (int x = threadIdx.x; x < nx; x += blockDim.x) {
    double v = z[0].x;
    int t = 0;
    for (int m = 1; m <= mh; m++) {
      t += x;
      if (t >= nx) t -= nx;
      const double2 w = twx[t];
      const double term = fma(z[m].x, w.x, -z[m].y * w.y);
      v = fma(2 * m == nx ? 1.0 : 2.0, term, v);
    }
    phi[(size_t)(j + 1) * layer + (size_t)y * nx + x] = v * scale;
  }
}

}  // namespace

namespace sg {

// The grid's tables of a solve and its two spectrum buffers, all device pointers.
struct ElecSolve {
  int nx = 0, ny = 0, nz = 0, mh = 0;
  double *cp = nullptr, *ipiv = nullptr, *lo = nullptr;
  double2 *S1 = nullptr, *S2 = nullptr, *twx = nullptr, *twy = nullptr;
  size_t spec() const { return (size_t)(nz - 2) * (mh + 1) * ny; }
};

// The host tables of a grid: minus the eigenvalue of the 5-point horizontal Laplacian per mode (electric.ts:29), the
// rows' off-diagonals 1/(hz dzs) below and above each level (:45), and every mode's elimination in the reference's
// order (:46-48): piv = di - lo cp_{j-1}, cp = up / piv; the twiddles exp(2 pi i t / n).
inline void elec_host_tables(int nx, int ny, int nz, double dx, double dy, const double* dzs, const double* hz, std::vector<double>& lo,
                             std::vector<double>& cpv, std::vector<double>& ipv, std::vector<double2>& tx, std::vector<double2>& ty) {
  const double PI_ = 3.14159265358979323846;
  const int mh = nx / 2, ni = nz - 2, modes = (mh + 1) * ny;
  const size_t spec = (size_t)ni * modes;
  std::vector<double> up(nz, 0.0);
  lo.assign(nz, 0.0); cpv.assign(spec, 0.0); ipv.assign(spec, 0.0);
  for (int k = 1; k < nz - 1; k++) { lo[k] = 1 / (hz[k] * dzs[k - 1]); up[k] = 1 / (hz[k] * dzs[k]); }
  for (int m = 0; m <= mh; m++)
    for (int q = 0; q < ny; q++) {
      const double lam = 4 * std::pow(std::sin(PI_ * m / nx), 2) / (dx * dx) + 4 * std::pow(std::sin(PI_ * q / ny), 2) / (dy * dy);
      const size_t mode = (size_t)m * ny + q;
      double cprev = 0;
      for (int j = 0; j < ni; j++) {
        const int k = j + 1;
        const double di = -lo[k] - up[k] - lam, a = j > 0 ? lo[k] : 0, c = j < ni - 1 ? up[k] : 0;
        const double piv = j == 0 ? di : di - a * cprev;
        cprev = c / piv;
        cpv[(size_t)j * modes + mode] = cprev;
        ipv[(size_t)j * modes + mode] = 1 / piv;
      }
    }
  tx.resize(nx); ty.resize(ny);
  for (int t = 0; t < nx; t++) tx[t] = make_double2(std::cos(2 * PI_ * t / nx), std::sin(2 * PI_ * t / nx));
  for (int t = 0; t < ny; t++) ty[t] = make_double2(std::cos(2 * PI_ * t / ny), std::sin(2 * PI_ * t / ny));
}

// phi (device, n) of rho (device, n); phi's ground and top levels are left as they are (zero: the caller clears them once).
inline void elec_solve_launch(const ElecSolve& s, const double* rho, double* phi, cudaStream_t st) {
  const int nx = s.nx, ny = s.ny, nz = s.nz, mh = s.mh, ni = nz - 2, modes = (mh + 1) * ny;
  const int tx = std::min(256, std::max(32, (mh + 1 + 31) / 32 * 32)), tyb = std::min(256, std::max(32, (ny + 31) / 32 * 32));
  const int txi = std::min(256, std::max(32, (nx + 31) / 32 * 32));
  k_elec_xdft<<<dim3(ny, ni), tx, (size_t)nx * 8, st>>>(rho, s.S1, s.twx, nx, ny, mh);
  k_elec_ydft<<<dim3(mh + 1, ni), tyb, (size_t)ny * 16, st>>>(s.S1, s.S2, s.twy, ny, mh, -1.0);
  k_elec_thomas<<<(modes + 31) / 32, 32, 0, st>>>(s.S2, s.cp, s.ipiv, s.lo, ni, modes);
  k_elec_ydft<<<dim3(mh + 1, ni), tyb, (size_t)ny * 16, st>>>(s.S2, s.S1, s.twy, ny, mh, 1.0);
  k_elec_xidft<<<dim3(ny, ni), txi, (size_t)(mh + 1) * 16, st>>>(s.S1, phi, s.twx, nx, ny, mh);
}

}  // namespace sg
