// The storm's electric potential on the device: the reference's ElectricSolver (src/core/electric.ts:15-60), which
// the lightning re-solves for every flash (Lightning.discharge, src/core/lightning.ts:231). Laplacian(phi) = -rho/eps0
// at the nodes, phi = 0 on the ground and top levels, periodic in x and y: a 2-D DFT of each interior level's right-hand
// side, one stretched vertical tridiagonal per horizontal mode with fixed ends (Thomas, the reference's rows and
// pivots), the inverse DFT. All in FP64: the reference's own tests hold the solution to 1e-9 of the discrete Poisson
// equation and the plate field to 5e-7, and a solve is small (the standard grid's is 60 thousand nodes). The DFTs are
// direct sums over exact FP64 twiddle tables, one output a thread: x (real to half-complex) per row, then y per level
// and x-mode; the inverse in the opposite order.
#include <cuda_runtime.h>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "sg_kernels.h"
#include "stormgpu.h"

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

struct sg_electric {
  sg_context* ctx = nullptr;
  int nx = 0, ny = 0, nz = 0, mh = 0;
  char* mem = nullptr;
  double *rho = nullptr, *phi = nullptr, *cp = nullptr, *ipiv = nullptr, *lo = nullptr;
  double2 *S1 = nullptr, *S2 = nullptr, *twx = nullptr, *twy = nullptr;
};

extern "C" {

int sg_electric_create(sg_context* ctx, const sg_grid* g, sg_electric** out) {
  if (!ctx || !out) return SG_ERR_INVALID;
  *out = nullptr;
  if (!g || !g->dzs || !g->hz || g->nx < 1 || g->ny < 1 || !(g->dx > 0) || !(g->dy > 0))
    return sg_context_fail(ctx, SG_ERR_INVALID, "electric solver: a grid with nx, ny >= 1, dx, dy > 0 and its level arrays");
  if (g->nz < 3) return sg_context_fail(ctx, SG_ERR_INVALID, "the electric solver needs an interior level");
  if (g->nz - 2 > ELEC_MAXNI) return sg_context_fail(ctx, SG_ERR_INVALID, "electric solver: at most 130 levels");
  // (a row, a column and a half spectrum in shared memory: at most 32 KB)
  if (g->nx > 2048 || g->ny > 2048) return sg_context_fail(ctx, SG_ERR_INVALID, "electric solver: nx and ny at most 2048");
  const int nx = g->nx, ny = g->ny, nz = g->nz, mh = nx / 2, ni = nz - 2, modes = (mh + 1) * ny;
  for (int k = 0; k < nz; k++)
    if (!(g->hz[k] > 0) || (k < nz - 1 && !(g->dzs[k] > 0))) return sg_context_fail(ctx, SG_ERR_INVALID, "electric solver: level spacings must be positive");
  if (cudaSetDevice(sg_context_device(ctx)) != cudaSuccess) return sg_context_fail(ctx, SG_ERR_DEVICE, "electric solver: cudaSetDevice");
  const size_t n = (size_t)nx * ny * nz, spec = (size_t)ni * modes;
  // one allocation: rho, phi [n]; S1, S2 [ni][mh + 1][ny] complex; cp, 1/pivot [ni][modes]; lo [nz]; twiddles
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t oRho = 0, oPhi = oRho + al(n * 8), oS1 = oPhi + al(n * 8), oS2 = oS1 + al(spec * 16), oCp = oS2 + al(spec * 16),
               oIp = oCp + al(spec * 8), oLo = oIp + al(spec * 8), oTx = oLo + al((size_t)nz * 8), oTy = oTx + al((size_t)nx * 16),
               total = oTy + al((size_t)ny * 16);
  auto* s = new sg_electric;
  s->ctx = ctx; s->nx = nx; s->ny = ny; s->nz = nz; s->mh = mh;
  cudaError_t e = cudaMalloc(&s->mem, total);
  if (e != cudaSuccess) { delete s; cudaGetLastError(); return sg_context_fail(ctx, SG_ERR_BUDGET, "electric solver: device memory"); }
  s->rho = (double*)(s->mem + oRho); s->phi = (double*)(s->mem + oPhi); s->S1 = (double2*)(s->mem + oS1); s->S2 = (double2*)(s->mem + oS2);
  s->cp = (double*)(s->mem + oCp); s->ipiv = (double*)(s->mem + oIp); s->lo = (double*)(s->mem + oLo);
  s->twx = (double2*)(s->mem + oTx); s->twy = (double2*)(s->mem + oTy);
  // minus the eigenvalue of the 5-point horizontal Laplacian per mode (src/core/electric.ts:29), the rows'
  // off-diagonals 1/(hz dzs) below and above each level (:45), and every mode's elimination in the reference's order
  // (:46-48): piv = di - lo cp_{j-1}, cp = up / piv
  std::vector<double> lo(nz, 0.0), up(nz, 0.0), cpv(spec), ipv(spec);
  for (int k = 1; k < nz - 1; k++) { lo[k] = 1 / (g->hz[k] * g->dzs[k - 1]); up[k] = 1 / (g->hz[k] * g->dzs[k]); }
  for (int m = 0; m <= mh; m++)
    for (int q = 0; q < ny; q++) {
      const double lam = 4 * std::pow(std::sin(PI * m / nx), 2) / (g->dx * g->dx) + 4 * std::pow(std::sin(PI * q / ny), 2) / (g->dy * g->dy);
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
  std::vector<double2> tx(nx), ty(ny);
  for (int t = 0; t < nx; t++) tx[t] = make_double2(std::cos(2 * PI * t / nx), std::sin(2 * PI * t / nx));
  for (int t = 0; t < ny; t++) ty[t] = make_double2(std::cos(2 * PI * t / ny), std::sin(2 * PI * t / ny));
  cudaStream_t st = sg_context_stream(ctx);
  if ((e = cudaMemcpyAsync(s->cp, cpv.data(), cpv.size() * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(s->ipiv, ipv.data(), ipv.size() * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(s->lo, lo.data(), lo.size() * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(s->twx, tx.data(), tx.size() * 16, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(s->twy, ty.data(), ty.size() * 16, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess) {
    cudaFree(s->mem); delete s;
    return sg_context_fail(ctx, SG_ERR_DEVICE, (std::string("electric solver: ") + cudaGetErrorString(e)).c_str());
  }
  *out = s;
  return SG_OK;
}

int sg_electric_solve(sg_electric* s, const double* rho, double* phi) {
  if (!s) return SG_ERR_INVALID;
  if (!rho || !phi) return sg_context_fail(s->ctx, SG_ERR_INVALID, "electric solver: rho and phi buffers");
  cudaSetDevice(sg_context_device(s->ctx));
  const int nx = s->nx, ny = s->ny, nz = s->nz, mh = s->mh, ni = nz - 2, modes = (mh + 1) * ny;
  const size_t n = (size_t)nx * ny * nz;
  cudaStream_t st = sg_context_stream(s->ctx);
  cudaError_t e;
  if ((e = cudaMemcpyAsync(s->rho, rho, n * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(s->phi, 0, n * 8, st)) != cudaSuccess)
    return sg_context_fail(s->ctx, SG_ERR_DEVICE, (std::string("electric solver: ") + cudaGetErrorString(e)).c_str());
  const int tx = std::min(256, std::max(32, (mh + 1 + 31) / 32 * 32)), tyb = std::min(256, std::max(32, (ny + 31) / 32 * 32));
  const int txi = std::min(256, std::max(32, (nx + 31) / 32 * 32));
  k_elec_xdft<<<dim3(ny, ni), tx, (size_t)nx * 8, st>>>(s->rho, s->S1, s->twx, nx, ny, mh);
  k_elec_ydft<<<dim3(mh + 1, ni), tyb, (size_t)ny * 16, st>>>(s->S1, s->S2, s->twy, ny, mh, -1.0);
  k_elec_thomas<<<(modes + 31) / 32, 32, 0, st>>>(s->S2, s->cp, s->ipiv, s->lo, ni, modes);
  k_elec_ydft<<<dim3(mh + 1, ni), tyb, (size_t)ny * 16, st>>>(s->S2, s->S1, s->twy, ny, mh, 1.0);
  k_elec_xidft<<<dim3(ny, ni), txi, (size_t)(mh + 1) * 16, st>>>(s->S1, s->phi, s->twx, nx, ny, mh);
  if ((e = cudaMemcpyAsync(phi, s->phi, n * 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess || (e = cudaStreamSynchronize(st)) != cudaSuccess ||
      (e = cudaGetLastError()) != cudaSuccess)
    return sg_context_fail(s->ctx, SG_ERR_DEVICE, (std::string("electric solver: ") + cudaGetErrorString(e)).c_str());
  return SG_OK;
}

int sg_electric_destroy(sg_electric* s) {
  if (!s) return SG_ERR_INVALID;
  cudaSetDevice(sg_context_device(s->ctx));
  cudaStreamSynchronize(sg_context_stream(s->ctx));
  cudaFree(s->mem);
  delete s;
  return SG_OK;
}

}  // extern "C"
