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
#include "sg_elec_solve.cuh"
#include "sg_kernels.h"
#include "stormgpu.h"

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
  std::vector<double> lo, cpv, ipv;
  std::vector<double2> tx, ty;
  sg::elec_host_tables(nx, ny, nz, g->dx, g->dy, g->dzs, g->hz, lo, cpv, ipv, tx, ty);
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
  const int nx = s->nx, ny = s->ny, nz = s->nz, mh = s->mh;
  const size_t n = (size_t)nx * ny * nz;
  cudaStream_t st = sg_context_stream(s->ctx);
  cudaError_t e;
  if ((e = cudaMemcpyAsync(s->rho, rho, n * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(s->phi, 0, n * 8, st)) != cudaSuccess)
    return sg_context_fail(s->ctx, SG_ERR_DEVICE, (std::string("electric solver: ") + cudaGetErrorString(e)).c_str());
  sg::ElecSolve es;
  es.nx = nx; es.ny = ny; es.nz = nz; es.mh = mh; es.cp = s->cp; es.ipiv = s->ipiv; es.lo = s->lo; es.S1 = s->S1; es.S2 = s->S2;
  es.twx = s->twx; es.twy = s->twy;
  sg::elec_solve_launch(es, s->rho, s->phi, st);
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
