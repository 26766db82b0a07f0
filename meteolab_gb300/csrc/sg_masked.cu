// Terrain on GB300 (src/core/terrain.ts): the ground heights of a terrain form and the cut-cell geometry on the host
// (terrainHeights :37-63, solidMask :80-84, groundLevels :87-91, nodeHeights :101-105, faceApertures :119-134,
// slopeArea :141-150), and MaskedProjection (:168-363) on the device: the node mass flux rho0 u made divergence-free
// over the dual cells cut by the ground. The masked operator S = -D M (rho0 H)^-1 D^T is solved by preconditioned
// conjugate gradients with the flat operator's spectral inverse (PressureSolver.solve, src/core/pressure.ts:95-140) as
// the preconditioner, all in FP64 as the reference. The transport's faces with terrain (FluxTransport.setTerrain and
// setVelocityMasked, src/core/advection.ts:78-184) are solved the same way over node vectors, with the flat face solve
// as the preconditioner (sg_faces_*).
//
// Layout: velocities FP32 [n] (node x + nx (y + ny z)); the cells' vectors FP64 [nc * nx * ny], nc = nz - 1 (cell
// x + nx (y + ny k) between node levels k and k + 1); spectra FP64 complex [nc][nx/2 + 1][ny]. One CG iteration is
// twelve launches: the cut cells' gradient of the search direction (a thread per node), its divergence fused with the
// d.Sd partial sums (a thread per cell), the q/r update fused with the r.r partials, the preconditioner (x-DFT per row,
// y-DFT per column, a Thomas sweep per mode over the levels, y- and x-inverse, the last fused with the r.z partials),
// the direction update, and one-block reductions that finish each dot product in a fixed order (the result does not
// depend on scheduling) and keep alpha, beta and the stopping test on the device. Eight iterations are one CUDA graph,
// replayed until the device's stop flag is set: the host reads one int per eight iterations; every kernel of an
// iteration after the stop returns at once, so the iterations done, the residual and the result are exactly those
// of the reference's loop (:313-329), which stops at the first top-of-loop test it passes.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "sg_kernels.h"
#include "stormgpu.h"

namespace {

constexpr double PI_ = 3.141592653589793;  // Math.PI
constexpr double LEAST_SHARE = .2;         // terrain.ts:69

// ---------------------------------------------------------------- host geometry

struct HostGrid {
  int nx, ny, nz, layer;
  size_t n;
  double dx, dy, width, depth;
  const double *zs, *dzs, *hz;
  double volumeTop(int k) const { return k < nz - 1 ? zs[k] + dzs[k] / 2 : zs[k]; }  // terrain.ts:72
};

bool host_grid(const sg_grid* g, HostGrid& h) {
  if (!g || !g->zs || !g->dzs || !g->hz || g->nx < 1 || g->ny < 1 || g->nz < 3 || !(g->dx > 0) || !(g->dy > 0)) return false;
  h.nx = g->nx; h.ny = g->ny; h.nz = g->nz; h.layer = g->nx * g->ny; h.n = (size_t)h.layer * g->nz;
  h.dx = g->dx; h.dy = g->dy; h.width = g->dx * g->nx; h.depth = g->dy * g->ny;
  h.zs = g->zs; h.dzs = g->dzs; h.hz = g->hz;
  return true;
}

double js_round(double x) { const double f = std::floor(x); return x - f >= 0.5 ? f + 1 : f; }  // Math.round

// terrainHeights: the form's height per column (periodic distances), two 1-2-1 passes (x, then y), lowest column at 0.
void terrain_heights(const HostGrid& g, const sg_terrain& t, float* h) {
  const int nx = g.nx, ny = g.ny;
  const double cx = (std::isnan(t.x) ? g.width / 2000 : t.x) * 1000, cy = (std::isnan(t.y) ? g.depth / 2000 : t.y) * 1000;
  const double a = std::max(t.width * 1000, 2 * std::max(g.dx, g.dy)), top = t.height * 1000, a2 = a * a;
  const double axis = (std::isnan(t.heading) ? 0 : t.heading) * PI_ / 180, sx = std::sin(axis), sy = std::cos(axis);
  const double lambda = (std::isnan(t.wavelength) ? 4 : t.wavelength) * 1000;
  for (int j = 0; j < ny; j++) {
    double ey = (j + .5) * g.dy - cy;
    ey -= g.depth * js_round(ey / g.depth);
    for (int i = 0; i < nx; i++) {
      double ex = (i + .5) * g.dx - cx;
      ex -= g.width * js_round(ex / g.width);
      const double across = ex * sy - ey * sx;
      double v;
      switch (t.kind) {
        case SG_TERRAIN_HILL: v = top / std::pow(1 + (ex * ex + ey * ey) / a2, 1.5); break;
        case SG_TERRAIN_RIDGE: v = top / (1 + across * across / a2); break;
        case SG_TERRAIN_SCHAR: { const double c = std::cos(PI_ * across / lambda); v = top * std::exp(-across * across / a2) * (c * c); break; }
        default: v = top / (1 + std::exp((std::max(std::fabs(ex), std::fabs(ey)) - a) / (.25 * a)));
      }
      h[i + (size_t)nx * j] = (float)v;
    }
  }
  std::vector<float> tmp((size_t)nx * ny);
  for (int pass = 0; pass < 2; pass++) {
    for (int j = 0; j < ny; j++) {
      const float* row = h + (size_t)nx * j;
      for (int i = 0; i < nx; i++) tmp[i + (size_t)nx * j] = (float)(((double)row[(i + nx - 1) % nx] + 2 * (double)row[i] + (double)row[(i + 1) % nx]) / 4);
    }
    for (int j = 0; j < ny; j++) {
      const float *s = tmp.data() + (size_t)nx * ((j + ny - 1) % ny), *c = tmp.data() + (size_t)nx * j, *nn = tmp.data() + (size_t)nx * ((j + 1) % ny);
      for (int i = 0; i < nx; i++) h[i + (size_t)nx * j] = (float)(((double)s[i] + 2 * (double)c[i] + (double)nn[i]) / 4);
    }
  }
  double low = INFINITY;
  for (size_t c = 0; c < (size_t)nx * ny; c++) low = std::min(low, (double)h[c]);
  for (size_t c = 0; c < (size_t)nx * ny; c++) h[c] = (float)((double)h[c] - low);
}

// solidMask and groundLevels: a column is solid from level 0 up while the ground leaves less than LEAST_SHARE of the
// level's volume above it (never the top two levels); its ground node is the first level that is not.
void solid_levels(const HostGrid& g, const float* ground, uint8_t* solid, int32_t* levels) {
  std::fill(solid, solid + g.n, (uint8_t)0);
  for (int c = 0; c < g.layer; c++) {
    int z = 0;
    while (z < g.nz - 2 && g.volumeTop(z) - (double)ground[c] < LEAST_SHARE * g.hz[z]) { solid[c + (size_t)z * g.layer] = 1; z++; }
    levels[c] = z;
  }
}

// nodeHeights: the ground node's volume above the ground, nothing in the ground, the level's hz elsewhere.
void node_heights(const HostGrid& g, const uint8_t* solid, const int32_t* levels, const float* ground, double* h) {
  for (int z = 0; z < g.nz; z++)
    for (int c = 0; c < g.layer; c++) {
      const size_t i = c + (size_t)z * g.layer;
      h[i] = solid[i] ? 0 : z == levels[c] ? g.volumeTop(z) - (double)ground[c] : g.hz[z];
    }
}

// faceApertures: each face to x + 1 (ax) or y + 1 (ay) open above the mean ground of its two columns in each level's
// layer of volume; a layer's open part next to a solid node carried up to the first face with both nodes fluid.
void face_apertures(const HostGrid& g, const uint8_t* solid, const float* ground, double* ax, double* ay) {
  std::fill(ax, ax + g.n, 0.0);
  std::fill(ay, ay + g.n, 0.0);
  auto shave = [&](double* out, int c, int other) {
    const double face = ((double)ground[c] + (double)ground[other]) / 2;
    double carry = 0;
    for (int k = 0; k < g.nz; k++) {
      const double bottom = k > 0 ? g.volumeTop(k - 1) : 0, open = face <= bottom ? g.hz[k] : std::max(0.0, g.volumeTop(k) - face);
      const size_t i = c + (size_t)k * g.layer;
      if (solid[i] || solid[other + (size_t)k * g.layer]) carry += open;
      else { out[i] = open + carry; carry = 0; }
    }
  };
  for (int j = 0; j < g.ny; j++)
    for (int i = 0; i < g.nx; i++) {
      const int c = i + j * g.nx;
      shave(ax, c, (i + 1) % g.nx + j * g.nx);
      shave(ay, c, i + ((j + 1) % g.ny) * g.nx);
    }
}

void slope_area(const HostGrid& g, const float* h, float* area) {
  const int nx = g.nx, ny = g.ny;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      const double hx = ((double)h[(i + 1) % nx + nx * j] - (double)h[(i + nx - 1) % nx + nx * j]) / (2 * g.dx);
      const double hy = ((double)h[i + nx * ((j + 1) % ny)] - (double)h[i + nx * ((j + ny - 1) % ny)]) / (2 * g.dy);
      area[i + (size_t)nx * j] = (float)std::sqrt(1 + hx * hx + hy * hy);
    }
}

// ---------------------------------------------------------------- device

// The solve's scalars on the device. done: 0 iterating, 1 stopped (converged, no descent, or out of iterations),
// 2 a zero right-hand side (nothing to project).
struct MpState {
  double bb, tol2bb, rz, rr, alpha, beta, tolerance;
  int k, done, maxIt, keepBB;
};
enum { STOP = 1, ZERO = 2, ANY = 3 };
enum { R_BB, R_RZ0, R_RR, R_DSD, R_RZN, R_RR_KEEP, R_TEST };

struct Geo {
  const uint8_t *solid, *wall, *dropped;
  const double *invMass, *low, *high, *rho, *dzs, *hz;
  int nx, ny, nz, layer, nc;
  size_t n, cells;
  double dx, dy;
};

constexpr int TPB = 256;

// Sum over the block (valid in thread 0); every thread of the block calls it.
__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  v = 0;
  if (wid == 0) {
    v = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;
}

// mask (terrain.ts:229-234): the solid nodes at rest, w zero at the wall nodes and on the ground and top levels.
__global__ void k_mp_mask(float* __restrict__ u, float* __restrict__ v, float* __restrict__ w, Geo g) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  if (g.solid[i]) { u[i] = 0; v[i] = 0; w[i] = 0; }
  else if (g.wall[i] || i < (size_t)g.layer || i >= g.n - g.layer) w[i] = 0;
}

// divergencePart (:240-264) of every cell; DOT 1 adds the partial sums of out . with, DOT 2 of out . out.
template <class S, int DOT>
__global__ void __launch_bounds__(TPB) k_mp_div(const S* __restrict__ u, const S* __restrict__ v, const S* __restrict__ w,
                                                double* __restrict__ out, const double* __restrict__ with, double* __restrict__ part,
                                                Geo g, const MpState* __restrict__ st, int skip) {
  __shared__ double sh[32];
  if (st && (st->done & skip)) return;
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double dot = 0;
  if (c < g.cells) {
    double val = 0;
    if (!g.dropped[c]) {
      const int k = (int)(c / g.layer), rem = (int)(c - (size_t)k * g.layer), j = rem / g.nx, i = rem - j * g.nx;
      const int i1 = i + 1 == g.nx ? 0 : i + 1, j0 = j * g.nx, j1 = (j + 1 == g.ny ? 0 : j + 1) * g.nx;
      const size_t l = (size_t)k * g.layer;
      const double r0 = g.rho[k] / 4, r1 = g.rho[k + 1] / 4;
      double ddx = 0, ddy = 0, ddz = 0;
#pragma unroll
      for (int corner = 0; corner < 4; corner++) {
        const size_t lo = (size_t)((corner & 1 ? i1 : i) + (corner & 2 ? j1 : j0)) + l, up = lo + g.layer;
        const double hi = g.high[lo];
        if (hi > 0) {
          const bool s = g.solid[lo] != 0;
          const double lw = g.low[lo], a = s ? 0 : r0 * lw, b = r1 * (hi + (s ? lw : 0));
          const double fu = a * (double)u[lo] + b * (double)u[up], fv = a * (double)v[lo] + b * (double)v[up];
          ddx += corner & 1 ? fu : -fu;
          ddy += corner & 2 ? fv : -fv;
        }
        ddz += r1 * (double)w[up] - r0 * (double)w[lo];
      }
      val = ddx / g.dx + ddy / g.dy + ddz / g.dzs[k];
    }
    out[c] = val;
    if (DOT == 1) dot = val * with[c];
    if (DOT == 2) dot = val * val;
  }
  if (DOT) {
    const double s = block_sum(dot, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
  }
}

// gradientPart (:270-300) of every node: the operator's adjoint over the node's mass of phi = q / dzs (zero in the
// dropped cells), times the cells' heights.
__global__ void __launch_bounds__(TPB) k_mp_grad(const double* __restrict__ q, double* __restrict__ tu, double* __restrict__ tv,
                                                 double* __restrict__ tw, Geo g, const MpState* __restrict__ st, int skip) {
  if (st->done & skip) return;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  if (g.solid[i]) { tu[i] = 0; tv[i] = 0; tw[i] = 0; return; }
  const int k = (int)(i / g.layer), rem = (int)(i - (size_t)k * g.layer), j = rem / g.nx, x = rem - j * g.nx;
  const int xm = x == 0 ? g.nx - 1 : x - 1, jm = (j == 0 ? g.ny - 1 : j - 1) * g.nx, j0 = j * g.nx, col = x + j0;
  const bool below = k > 0, above = k < g.nz - 1;
  const double r = g.rho[k] / 4;
  auto phi = [&](size_t cell, double dz) { return g.dropped[cell] ? 0.0 : q[cell] / dz; };
  double gu = 0, gv = 0, gw = 0;
  if (above) {
    const size_t l = (size_t)k * g.layer;
    const double f = g.low[col + l] * r, h = g.dzs[k];
    const double a = h * phi(xm + jm + l, h), b = h * phi(x + jm + l, h), c = h * phi(xm + j0 + l, h), d = h * phi(x + j0 + l, h);
    gu += f * (a - b + c - d) / g.dx; gv += f * (a + b - c - d) / g.dy; gw -= r * (a + b + c + d) / h;
  }
  if (below) {
    const size_t l = (size_t)(k - 1) * g.layer;
    const double f = r * (g.high[col + l] + (g.solid[col + l] ? g.low[col + l] : 0)), h = g.dzs[k - 1];
    const double a = h * phi(xm + jm + l, h), b = h * phi(x + jm + l, h), c = h * phi(xm + j0 + l, h), d = h * phi(x + j0 + l, h);
    gu += f * (a - b + c - d) / g.dx; gv += f * (a + b - c - d) / g.dy; gw += r * (a + b + c + d) / h;
  }
  const double m = g.invMass[i];
  tu[i] = gu * m; tv[i] = gv * m; tw[i] = g.wall[i] || !below || !above ? 0 : gw * m;
}

// The first guess q = V phi from the last pressure (:311).
__global__ void k_mp_start(const double* __restrict__ p, double* __restrict__ q, double dt, Geo g, const MpState* __restrict__ st) {
  if (st->done & ZERO) return;
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < g.cells) q[c] = g.dropped[c] ? 0 : p[c] * dt * g.dzs[c / g.layer];
}

// r = -b - S q with the r.r partials (:313).
__global__ void __launch_bounds__(TPB) k_mp_resid(const double* __restrict__ b, const double* __restrict__ sq, double* __restrict__ r,
                                                  double* __restrict__ part, Geo g, const MpState* __restrict__ st) {
  __shared__ double sh[32];
  if (st->done & ZERO) return;
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0;
  if (c < g.cells) { v = -b[c] - sq[c]; r[c] = v; }
  const double s = block_sum(v * v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// q += alpha d, r -= alpha S d, with the r.r partials of the next top-of-loop test (:324).
__global__ void __launch_bounds__(TPB) k_mp_update(double* __restrict__ q, double* __restrict__ r, const double* __restrict__ d,
                                                   const double* __restrict__ sd, double* __restrict__ part, Geo g, const MpState* __restrict__ st) {
  __shared__ double sh[32];
  if (st->done) return;
  const double alpha = st->alpha;
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0;
  if (c < g.cells) { q[c] += alpha * d[c]; v = r[c] - alpha * sd[c]; r[c] = v; }
  const double s = block_sum(v * v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// d = z (first) or d = z + beta d (:331, :328).
__global__ void k_mp_dir(double* __restrict__ d, const double* __restrict__ z, Geo g, const MpState* __restrict__ st, int first) {
  if (st->done & (first ? ZERO : ANY)) return;
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < g.cells) d[c] = first ? z[c] : z[c] + st->beta * d[c];
}

// One block finishes a dot product from the partials in a fixed order and acts on it (the scalars of :306-329).
template <int OP>
__global__ void __launch_bounds__(TPB) k_mp_reduce(MpState* __restrict__ st, const double* __restrict__ part, int nparts, int skip) {
  __shared__ double sh[32];
  if (st->done & skip) return;
  double v = 0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) v += part[i];
  const double s = block_sum(v, sh);
  if (threadIdx.x != 0) return;
  if (OP == R_BB) {
    st->bb = s; st->tol2bb = st->tolerance * st->tolerance * s; st->rr = st->keepBB ? s : 0; st->k = 0;
    if (!(s > 0)) st->done = ZERO;
  } else if (OP == R_RZ0) {
    st->rz = s;
    if (st->maxIt <= 0) st->done = STOP;
  } else if (OP == R_RR) {
    st->rr = s;
    if (s <= st->tol2bb) st->done = STOP;
  } else if (OP == R_RR_KEEP) {
    st->rr = s;
  } else if (OP == R_TEST) {
    if (!(st->rr > st->tol2bb)) st->done = STOP;
  } else if (OP == R_DSD) {
    if (!(s > 0)) st->done = STOP;
    else st->alpha = st->rz / s;
  } else {
    st->beta = s / st->rz; st->rz = s; st->k++;
    if (st->k >= st->maxIt) st->done = STOP;
  }
}

// Forward x-DFT of each cell row of scale * src: S1[k][m][y], m <= nx / 2.
// With `per` (the face solve): row = scale * src / per[k], the right-hand side over each level's height.
__global__ void k_mp_xdft(const double* __restrict__ src, double scale, const double* __restrict__ per, double2* __restrict__ S1,
                          const double2* __restrict__ twx, Geo g, int mh, const MpState* __restrict__ st, int skip) {
  extern __shared__ double row[];
  if (st && (st->done & skip)) return;
  const int y = blockIdx.x, k = blockIdx.y, nx = g.nx;
  const double* s = src + (size_t)k * g.layer + (size_t)y * nx;
  for (int x = threadIdx.x; x < nx; x += blockDim.x) row[x] = per ? scale * s[x] / per[k] : scale * s[x];
  __syncthreads();
  for (int m = threadIdx.x; m <= mh; m += blockDim.x) {
    double re = 0, im = 0;
    int t = 0;
    for (int x = 0; x < nx; x++) {
      const double2 tw = twx[t];
      re = fma(row[x], tw.x, re);
      im = fma(-row[x], tw.y, im);
      t += m;
      if (t >= nx) t -= nx;
    }
    S1[((size_t)k * (mh + 1) + m) * g.ny + y] = make_double2(re, im);
  }
}

// y-DFT of each (cell layer, x-mode) column, sign -1 forward and +1 inverse (unnormalised).
__global__ void k_mp_ydft(const double2* __restrict__ in, double2* __restrict__ out, const double2* __restrict__ twy, int ny, int mh, double sign,
                          const MpState* __restrict__ st, int skip) {
  extern __shared__ double2 colv[];
  if (st && (st->done & skip)) return;
  const size_t base = ((size_t)blockIdx.y * (mh + 1) + blockIdx.x) * ny;
  for (int y = threadIdx.x; y < ny; y += blockDim.x) colv[y] = in[base + y];
  __syncthreads();
  for (int nn = threadIdx.x; nn < ny; nn += blockDim.x) {
    double re = 0, im = 0;
    int t = 0;
    for (int y = 0; y < ny; y++) {
      const double2 tw = twy[t], v = colv[y];
      const double s = sign * tw.y;
      re = fma(v.x, tw.x, fma(-v.y, s, re));
      im = fma(v.y, tw.x, fma(v.x, s, im));
      t += nn;
      if (t >= ny) t -= ny;
    }
    out[base + nn] = make_double2(re, im);
  }
}

// One mode a thread, the reference's Thomas sweep over the cell layers (pressure.ts:118-140) with the rows' lower
// coefficients and pivots from the host (the face solve's right-hand sides times each level's height, rs); the forward
// values kept in place for the back substitution. A mode the
// reference zeroes, and the pinned lowest cell of the uniform mode, have an infinite pivot. The recurrence is a
// dependent chain of FP64 divides: each eight layers' coefficients and right-hand sides are loaded before their eight
// steps, so a step waits on the divide, not on memory.
constexpr int THOMAS_AHEAD = 8;
__global__ void k_mp_thomas(double2* __restrict__ S2, const double* __restrict__ lo, const double* __restrict__ cp,
                            const double* __restrict__ piv, const double* __restrict__ rs, int nc, int modes, const MpState* __restrict__ st,
                            int skip) {
  if (st && (st->done & skip)) return;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= modes) return;
  double2 d = make_double2(0, 0);
  for (int k0 = 0; k0 < nc; k0 += THOMAS_AHEAD) {
    double2 r[THOMAS_AHEAD];
    double a[THOMAS_AHEAD], m[THOMAS_AHEAD];
#pragma unroll
    for (int q = 0; q < THOMAS_AHEAD; q++) {
      const size_t at = (size_t)min(k0 + q, nc - 1) * modes + g;
      r[q] = S2[at]; a[q] = lo[at]; m[q] = piv[at];
      if (rs) { const double h = rs[min(k0 + q, nc - 1)]; r[q] = make_double2(h * r[q].x, h * r[q].y); }
    }
#pragma unroll
    for (int q = 0; q < THOMAS_AHEAD; q++)
      if (k0 + q < nc) {
        d = make_double2((r[q].x - a[q] * d.x) / m[q], (r[q].y - a[q] * d.y) / m[q]);
        S2[(size_t)(k0 + q) * modes + g] = d;
      }
  }
  for (int k1 = nc - 2; k1 >= 0; k1 -= THOMAS_AHEAD) {
    double2 v[THOMAS_AHEAD];
    double c[THOMAS_AHEAD];
#pragma unroll
    for (int q = 0; q < THOMAS_AHEAD; q++) {
      const size_t at = (size_t)max(k1 - q, 0) * modes + g;
      v[q] = S2[at]; c[q] = cp[at];
    }
#pragma unroll
    for (int q = 0; q < THOMAS_AHEAD; q++)
      if (k1 - q >= 0) {
        d = make_double2(v[q].x - c[q] * d.x, v[q].y - c[q] * d.y);
        S2[(size_t)(k1 - q) * modes + g] = d;
      }
  }
}

// Inverse x-DFT of each cell row from its half spectrum, / (nx ny). MODE 1: the preconditioner's z = V phi, zero in the
// dropped cells (:355), with the r.z partials; 2: the plain solution with the r.z partials (the face solve's); 0: the
// plain solution (the flat solve's pressure).
template <int MODE>
__global__ void k_mp_xidft(const double2* __restrict__ S1, double* __restrict__ out, const double* __restrict__ r, double* __restrict__ part,
                           const double2* __restrict__ twx, Geo g, int mh, const MpState* __restrict__ st, int skip) {
  extern __shared__ double2 zs[];
  __shared__ double sh[32];
  if (st && (st->done & skip)) return;
  const int y = blockIdx.x, k = blockIdx.y, nx = g.nx;
  for (int m = threadIdx.x; m <= mh; m += blockDim.x) zs[m] = S1[((size_t)k * (mh + 1) + m) * g.ny + y];
  __syncthreads();
  const double scale = 1.0 / ((double)nx * g.ny);
  double dot = 0;
  for (int x = threadIdx.x; x < nx; x += blockDim.x) {
    double v = zs[0].x;
    int t = 0;
    for (int m = 1; m <= mh; m++) {
      t += x;
      if (t >= nx) t -= nx;
      const double2 tw = twx[t];
      v = 2 * m == nx ? fma(zs[m].x, tw.x, v) : fma(2.0, fma(zs[m].x, tw.x, -zs[m].y * tw.y), v);
    }
    const size_t c = (size_t)k * g.layer + (size_t)y * nx + x;
    double val = v * scale;
    if (MODE == 1) val = g.dropped[c] ? 0 : val * g.dzs[k];
    if (MODE) dot += r[c] * val;
    out[c] = val;
  }
  if (MODE) {
    const double s = block_sum(dot, sh);
    if (threadIdx.x == 0) part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = s;
  }
}

// The potential phi = q / V and the pressure kept, phi / dt (:332).
__global__ void k_mp_finish(const double* __restrict__ q, double* __restrict__ p, double dt, Geo g, const MpState* __restrict__ st) {
  if (st->done & ZERO) return;
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < g.cells) p[c] = q[c] / g.dzs[c / g.layer] / dt;
}

// u = M (u* - G phi): the correction added in FP32 stores, then masked (:334-336).
__global__ void k_mp_correct(float* __restrict__ u, float* __restrict__ v, float* __restrict__ w, const double* __restrict__ tu,
                             const double* __restrict__ tv, const double* __restrict__ tw, Geo g, const MpState* __restrict__ st) {
  if (st->done & ZERO) return;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  if (g.solid[i]) { u[i] = 0; v[i] = 0; w[i] = 0; return; }
  u[i] = (float)((double)u[i] + tu[i]);
  v[i] = (float)((double)v[i] + tv[i]);
  const float wn = (float)((double)w[i] + tw[i]);
  w[i] = g.wall[i] || i < (size_t)g.layer || i >= g.n - g.layer ? 0.0f : wn;
}

// Flat ground (:336-339): PressureSolver.divergence (pressure.ts:50-66), per unit time dt.
__global__ void k_mp_flat_div(const float* __restrict__ u, const float* __restrict__ v, const float* __restrict__ w, double* __restrict__ out,
                              double dt, Geo g) {
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.cells) return;
  const int k = (int)(c / g.layer), rem = (int)(c - (size_t)k * g.layer), j = rem / g.nx, i = rem - j * g.nx;
  const int i1 = i + 1 == g.nx ? 0 : i + 1, y0 = j * g.nx, y1 = (j + 1 == g.ny ? 0 : j + 1) * g.nx;
  const size_t l0 = (size_t)k * g.layer, l1 = l0 + g.layer;
  const size_t a = i + y0 + l0, b = i1 + y0 + l0, e = i + y1 + l0, f = i1 + y1 + l0, gg = i + y0 + l1, h = i1 + y0 + l1, s = i + y1 + l1,
               t = i1 + y1 + l1;
  const double r0 = g.rho[k] / 4, r1 = g.rho[k + 1] / 4;
  const double ddx = (r0 * ((double)u[b] + (double)u[f] - (double)u[a] - (double)u[e]) + r1 * ((double)u[h] + (double)u[t] - (double)u[gg] - (double)u[s])) / g.dx;
  const double ddy = (r0 * ((double)v[e] + (double)v[f] - (double)v[a] - (double)v[b]) + r1 * ((double)v[s] + (double)v[t] - (double)v[gg] - (double)v[h])) / g.dy;
  const double ddz = (r1 * ((double)w[gg] + (double)w[h] + (double)w[s] + (double)w[t]) - r0 * ((double)w[a] + (double)w[b] + (double)w[e] + (double)w[f])) / g.dzs[k];
  out[c] = (ddx + ddy + ddz) / dt;
}

// PressureSolver.correct (pressure.ts:69-92): u -= dt G p; w only at the interior levels.
__global__ void k_mp_flat_correct(const double* __restrict__ p, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w, double dt, Geo g) {
  const size_t node = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (node >= g.n) return;
  const int k = (int)(node / g.layer), rem = (int)(node - (size_t)k * g.layer), j = rem / g.nx, i = rem - j * g.nx, nz = g.nz;
  const int im = i == 0 ? g.nx - 1 : i - 1, jm = (j == 0 ? g.ny - 1 : j - 1) * g.nx, j0 = j * g.nx;
  const size_t lo = (size_t)(k > 0 ? k - 1 : 0) * g.layer, hi = (size_t)(k < nz - 2 ? k : nz - 2) * g.layer;
  const double wLo = k > 0 ? g.dzs[k - 1] / g.hz[k] : 0, wHi = k < nz - 1 ? g.dzs[k] / g.hz[k] : 0;
  auto P = [&](int ii, int jj, size_t base) { return p[base + ii + jj]; };
  const double gx = (wLo * (P(i, jm, lo) + P(i, j0, lo) - P(im, jm, lo) - P(im, j0, lo)) + wHi * (P(i, jm, hi) + P(i, j0, hi) - P(im, jm, hi) - P(im, j0, hi))) / (4 * g.dx);
  const double gy = (wLo * (P(im, j0, lo) + P(i, j0, lo) - P(im, jm, lo) - P(i, jm, lo)) + wHi * (P(im, j0, hi) + P(i, j0, hi) - P(im, jm, hi) - P(i, jm, hi))) / (4 * g.dy);
  u[node] = (float)((double)u[node] - dt * gx);
  v[node] = (float)((double)v[node] - dt * gy);
  if (k > 0 && k < nz - 1) {
    const size_t below = (size_t)(k - 1) * g.layer, above = (size_t)k * g.layer;
    const double gz = (P(im, jm, above) + P(i, jm, above) + P(im, j0, above) + P(i, j0, above) - P(im, jm, below) - P(i, jm, below) - P(im, j0, below) -
                       P(i, j0, below)) / (4 * g.hz[k]);
    w[node] = (float)((double)w[node] - dt * gz);
  }
}

// ---------------------------------------------------------------- the transport's faces with terrain
// (FluxTransport.setTerrain and setVelocityMasked, src/core/advection.ts:78-184): node vectors [n].

struct FaceGeo {
  const uint8_t* open;  // bit 1 the face to x + 1, 2 to y + 1, 4 to z + 1: both nodes fluid
  const double *ax, *ay, *hn, *rho, *dzs;
  int nx, ny, nz, layer;
  size_t n;
  double dx, dy;
};

struct Node {
  int x, y, z;
  size_t l, e, w, no, so;
};
__device__ __forceinline__ Node node_of(size_t i, const FaceGeo& g) {
  Node a;
  a.z = (int)(i / g.layer);
  const int rem = (int)(i - (size_t)a.z * g.layer);
  a.y = rem / g.nx; a.x = rem - a.y * g.nx;
  a.l = (size_t)a.z * g.layer;
  a.e = (size_t)(a.x + 1 == g.nx ? 0 : a.x + 1) + (size_t)a.y * g.nx + a.l;
  a.w = (size_t)(a.x == 0 ? g.nx - 1 : a.x - 1) + (size_t)a.y * g.nx + a.l;
  a.no = (size_t)a.x + (size_t)(a.y + 1 == g.ny ? 0 : a.y + 1) * g.nx + a.l;
  a.so = (size_t)a.x + (size_t)(a.y == 0 ? g.ny - 1 : a.y - 1) * g.nx + a.l;
  return a;
}

// faces (advection.ts:190-200) of the node velocity, shut where a face is not open (:120).
__global__ void k_tm_faces(const float* __restrict__ u, const float* __restrict__ v, const float* __restrict__ w, double* __restrict__ mx,
                           double* __restrict__ my, double* __restrict__ mz, FaceGeo g) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const Node a = node_of(i, g);
  const uint8_t o = g.open[i];
  const double r = g.rho[a.z];
  mx[i] = o & 1 ? r * ((double)u[i] + (double)u[a.e]) / 2 : 0;
  my[i] = o & 2 ? r * ((double)v[i] + (double)v[a.no]) / 2 : 0;
  mz[i] = o & 4 ? (g.rho[a.z] + g.rho[a.z + 1]) / 2 * ((double)w[i] + (double)w[i + g.layer]) / 2 : 0;
}

// The apertures' divergence of the face fluxes (:96-105): MODE 0 b = -(h div) with the b.b partials, 1 div = h div / hn.
template <int MODE>
__global__ void __launch_bounds__(TPB) k_tm_tdiv(const double* __restrict__ mx, const double* __restrict__ my, const double* __restrict__ mz,
                                                 double* __restrict__ out, double* __restrict__ part, FaceGeo g) {
  __shared__ double sh[32];
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double dot = 0;
  if (i < g.n) {
    const Node a = node_of(i, g);
    double v = (g.ax[i] * mx[i] - g.ax[a.w] * mx[a.w]) / g.dx + (g.ay[i] * my[i] - g.ay[a.so] * my[a.so]) / g.dy +
               (mz[i] - (a.z > 0 ? mz[i - g.layer] : 0));
    if (MODE == 0) { v = -v; dot = v * v; }
    else v = v / g.hn[i];
    out[i] = v;
  }
  if (MODE == 0) {
    const double s = block_sum(dot, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
  }
}

// S d = -h div(M rho0 grad d) (:170-176) at each node from d at it and its six neighbours (each face flux as the
// reference forms it), with the d.Sd partials.
__global__ void __launch_bounds__(TPB) k_tm_apply(const double* __restrict__ d, double* __restrict__ out, double* __restrict__ part, FaceGeo g,
                                                  const MpState* __restrict__ st) {
  __shared__ double sh[32];
  if (st->done) return;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double dot = 0;
  if (i < g.n) {
    const Node a = node_of(i, g);
    const double r = g.rho[a.z], di = d[i];
    const uint8_t oi = g.open[i];
    const double fxi = oi & 1 ? r * (d[a.e] - di) / g.dx : 0, fxw = g.open[a.w] & 1 ? r * (di - d[a.w]) / g.dx : 0;
    const double fyi = oi & 2 ? r * (d[a.no] - di) / g.dy : 0, fys = g.open[a.so] & 2 ? r * (di - d[a.so]) / g.dy : 0;
    const double fzi = oi & 4 ? (g.rho[a.z] + g.rho[a.z + 1]) / 2 * (d[i + g.layer] - di) / g.dzs[a.z] : 0;
    const double fzb = a.z > 0 && (g.open[i - g.layer] & 4) ? (g.rho[a.z - 1] + g.rho[a.z]) / 2 * (di - d[i - g.layer]) / g.dzs[a.z - 1] : 0;
    const double v = -((g.ax[i] * fxi - g.ax[a.w] * fxw) / g.dx + (g.ay[i] * fyi - g.ay[a.so] * fys) / g.dy + (fzi - fzb));
    out[i] = v;
    dot = di * v;
  }
  const double s = block_sum(dot, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// The fluxes lose M rho0 grad(q) (:150).
__global__ void k_tm_correct(const double* __restrict__ q, double* __restrict__ mx, double* __restrict__ my, double* __restrict__ mz, FaceGeo g,
                             const MpState* __restrict__ st) {
  if (st->done & ZERO) return;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const Node a = node_of(i, g);
  const uint8_t o = g.open[i];
  const double r = g.rho[a.z], qi = q[i];
  mx[i] += o & 1 ? -r * (q[a.e] - qi) / g.dx : 0;
  my[i] += o & 2 ? -r * (q[a.no] - qi) / g.dy : 0;
  mz[i] += o & 4 ? -((g.rho[a.z] + g.rho[a.z + 1]) / 2) * (q[i + g.layer] - qi) / g.dzs[a.z] : 0;
}

int blocks(size_t count) { return (int)((count + TPB - 1) / TPB); }
int threads_for(int count) { return std::min(256, std::max(32, (count + 31) / 32 * 32)); }

}  // namespace

struct sg_masked {
  sg_context* ctx = nullptr;
  HostGrid hg{};
  Geo geo{};
  int mh = 0, modes = 0, maxIt = 200;
  double tolerance = 1e-6;
  bool any = false;
  char* mem = nullptr;
  float *u = nullptr, *v = nullptr, *w = nullptr;
  double *p = nullptr, *b = nullptr, *q = nullptr, *r = nullptr, *z = nullptr, *d = nullptr, *sd = nullptr, *tu = nullptr, *tv = nullptr,
         *tw = nullptr, *pDot = nullptr, *pRR = nullptr, *lo = nullptr, *cp = nullptr, *piv = nullptr;
  double2 *S1 = nullptr, *S2 = nullptr, *twx = nullptr, *twy = nullptr;
  MpState* st = nullptr;
  std::vector<uint8_t> dropped;
  cudaGraphExec_t chunk = nullptr;
  int iterations = 0;
  double residual = 0;
};

struct sg_faces {
  sg_context* ctx = nullptr;
  FaceGeo fg{};
  Geo geo{};  // the node vectors as the shared kernels see them: cells = n, nc = nz
  int mh = 0, modes = 0, maxIt = 400;
  double tolerance = 1e-10;
  char* mem = nullptr;
  float *u = nullptr, *v = nullptr, *w = nullptr;
  double *mx = nullptr, *my = nullptr, *mz = nullptr, *div = nullptr, *b = nullptr, *q = nullptr, *r = nullptr, *z = nullptr, *d = nullptr,
         *sd = nullptr, *pDot = nullptr, *pRR = nullptr, *lo = nullptr, *cp = nullptr, *piv = nullptr, *hz = nullptr;
  double2 *S1 = nullptr, *S2 = nullptr, *twx = nullptr, *twy = nullptr;
  MpState* st = nullptr;
  cudaGraphExec_t chunk = nullptr;
  int iterations = 0;
  double residual = 0;
};

namespace {

constexpr int CHUNK = 8;

// The face solve's preconditioner (flatSolve, advection.ts:179-184): div = -r / h, the flat face solve (forward,
// modes with the right-hand sides times h, inverse) into z, with the r.z partials.
void enqueue_face_precondition(sg_faces* f, cudaStream_t s, int skip) {
  const Geo& g = f->geo;
  const int nx = g.nx, ny = g.ny, nz = g.nc, mh = f->mh;
  k_mp_xdft<<<dim3(ny, nz), threads_for(mh + 1), (size_t)nx * 8, s>>>(f->r, -1.0, f->hz, f->S1, f->twx, g, mh, f->st, skip);
  k_mp_ydft<<<dim3(mh + 1, nz), threads_for(ny), (size_t)ny * 16, s>>>(f->S1, f->S2, f->twy, ny, mh, -1.0, f->st, skip);
  k_mp_thomas<<<(f->modes + 63) / 64, 64, 0, s>>>(f->S2, f->lo, f->cp, f->piv, f->hz, nz, f->modes, f->st, skip);
  k_mp_ydft<<<dim3(mh + 1, nz), threads_for(ny), (size_t)ny * 16, s>>>(f->S2, f->S1, f->twy, ny, mh, 1.0, f->st, skip);
  k_mp_xidft<2><<<dim3(ny, nz), threads_for(nx), (size_t)(mh + 1) * 16, s>>>(f->S1, f->z, f->r, f->pDot, f->twx, g, mh, f->st, skip);
}

// One iteration of setVelocityMasked's loop (:127-145): the test on the last update's r.r, S d and d.Sd, alpha, the
// update with its r.r kept, the preconditioner, beta, the new direction.
void enqueue_face_iteration(sg_faces* f, cudaStream_t s) {
  const Geo& g = f->geo;
  const int nb = blocks(g.cells);
  k_mp_reduce<R_TEST><<<1, TPB, 0, s>>>(f->st, f->pRR, 0, ANY);
  k_tm_apply<<<nb, TPB, 0, s>>>(f->d, f->sd, f->pDot, f->fg, f->st);
  k_mp_reduce<R_DSD><<<1, TPB, 0, s>>>(f->st, f->pDot, nb, ANY);
  k_mp_update<<<nb, TPB, 0, s>>>(f->q, f->r, f->d, f->sd, f->pRR, g, f->st);
  k_mp_reduce<R_RR_KEEP><<<1, TPB, 0, s>>>(f->st, f->pRR, nb, ANY);
  enqueue_face_precondition(f, s, ANY);
  k_mp_reduce<R_RZN><<<1, TPB, 0, s>>>(f->st, f->pDot, g.ny * g.nc, ANY);
  k_mp_dir<<<nb, TPB, 0, s>>>(f->d, f->z, g, f->st, 0);
}

// The preconditioner z = P S0^-1 P r (:351-356): the flat solve of -r, z = V phi, with the r.z partials.
void enqueue_precondition(sg_masked* m, cudaStream_t s, int skip) {
  const Geo& g = m->geo;
  const int nx = g.nx, ny = g.ny, nc = g.nc, mh = m->mh;
  k_mp_xdft<<<dim3(ny, nc), threads_for(mh + 1), (size_t)nx * 8, s>>>(m->r, -1.0, nullptr, m->S1, m->twx, g, mh, m->st, skip);
  k_mp_ydft<<<dim3(mh + 1, nc), threads_for(ny), (size_t)ny * 16, s>>>(m->S1, m->S2, m->twy, ny, mh, -1.0, m->st, skip);
  k_mp_thomas<<<(m->modes + 63) / 64, 64, 0, s>>>(m->S2, m->lo, m->cp, m->piv, nullptr, nc, m->modes, m->st, skip);
  k_mp_ydft<<<dim3(mh + 1, nc), threads_for(ny), (size_t)ny * 16, s>>>(m->S2, m->S1, m->twy, ny, mh, 1.0, m->st, skip);
  k_mp_xidft<1><<<dim3(ny, nc), threads_for(nx), (size_t)(mh + 1) * 16, s>>>(m->S1, m->z, m->r, m->pDot, m->twx, g, mh, m->st, skip);
}

// One iteration of the loop (:314-329).
void enqueue_iteration(sg_masked* m, cudaStream_t s) {
  const Geo& g = m->geo;
  const int cb = blocks(g.cells), nb = blocks(g.n);
  k_mp_reduce<R_RR><<<1, TPB, 0, s>>>(m->st, m->pRR, cb, ANY);
  k_mp_grad<<<nb, TPB, 0, s>>>(m->d, m->tu, m->tv, m->tw, g, m->st, ANY);
  k_mp_div<double, 1><<<cb, TPB, 0, s>>>(m->tu, m->tv, m->tw, m->sd, m->d, m->pDot, g, m->st, ANY);
  k_mp_reduce<R_DSD><<<1, TPB, 0, s>>>(m->st, m->pDot, cb, ANY);
  k_mp_update<<<cb, TPB, 0, s>>>(m->q, m->r, m->d, m->sd, m->pRR, g, m->st);
  enqueue_precondition(m, s, ANY);
  k_mp_reduce<R_RZN><<<1, TPB, 0, s>>>(m->st, m->pDot, g.ny * g.nc, ANY);
  k_mp_dir<<<cb, TPB, 0, s>>>(m->d, m->z, g, m->st, 0);
}

int fail(sg_masked* m, const char* what, cudaError_t e) {
  return sg_context_fail(m->ctx, SG_ERR_DEVICE, (std::string("masked projection: ") + what + ": " + cudaGetErrorString(e)).c_str());
}

}  // namespace

extern "C" {

int sg_terrain_heights(const sg_grid* grid, const sg_terrain* form, float* out) {
  HostGrid g;
  if (!host_grid(grid, g) || !form || !out) return SG_ERR_INVALID;
  if (form->kind < SG_TERRAIN_HILL || form->kind > SG_TERRAIN_SCHAR || !std::isfinite(form->height) || !std::isfinite(form->width)) return SG_ERR_INVALID;
  terrain_heights(g, *form, out);
  return SG_OK;
}

int sg_terrain_geometry(const sg_grid* grid, const float* ground, uint8_t* solid, int32_t* levels, double* heights, double* ax, double* ay,
                        float* slope) {
  HostGrid g;
  if (!host_grid(grid, g) || !ground) return SG_ERR_INVALID;
  std::vector<uint8_t> s(g.n);
  std::vector<int32_t> lv(g.layer);
  solid_levels(g, ground, s.data(), lv.data());
  if (solid) std::memcpy(solid, s.data(), g.n);
  if (levels) std::memcpy(levels, lv.data(), (size_t)g.layer * 4);
  if (heights) node_heights(g, s.data(), lv.data(), ground, heights);
  if (ax && ay) face_apertures(g, s.data(), ground, ax, ay);
  else if (ax || ay) {
    std::vector<double> tx(g.n), ty(g.n);
    face_apertures(g, s.data(), ground, tx.data(), ty.data());
    if (ax) std::memcpy(ax, tx.data(), g.n * 8);
    if (ay) std::memcpy(ay, ty.data(), g.n * 8);
  }
  if (slope) slope_area(g, ground, slope);
  return SG_OK;
}

int sg_masked_create(sg_context* ctx, const sg_grid* grid, const double* rho, const float* ground, double tolerance, int max_iterations,
                     sg_masked** out) {
  if (!ctx || !out) return SG_ERR_INVALID;
  *out = nullptr;
  HostGrid g;
  if (!host_grid(grid, g) || !rho || !ground)
    return sg_context_fail(ctx, SG_ERR_INVALID, "masked projection: a grid with nx, ny >= 1, nz >= 3, dx, dy > 0, its level arrays, rho and the ground");
  if (g.nx > 2048 || g.ny > 2048) return sg_context_fail(ctx, SG_ERR_INVALID, "masked projection: nx and ny at most 2048");
  if (g.n > (size_t)1 << 30) return sg_context_fail(ctx, SG_ERR_INVALID, "masked projection: at most 2^30 nodes");
  if (!(tolerance >= 0) || max_iterations < 0) return sg_context_fail(ctx, SG_ERR_INVALID, "masked projection: tolerance >= 0, max_iterations >= 0");
  for (int k = 0; k < g.nz; k++)
    if (!(g.hz[k] > 0) || (k < g.nz - 1 && !(g.dzs[k] > 0)) || !(rho[k] > 0))
      return sg_context_fail(ctx, SG_ERR_INVALID, "masked projection: level spacings and densities must be positive");
  for (int c = 0; c < g.layer; c++)
    if (!std::isfinite(ground[c])) return sg_context_fail(ctx, SG_ERR_INVALID, "masked projection: finite ground heights");
  if (cudaSetDevice(sg_context_device(ctx)) != cudaSuccess) return sg_context_fail(ctx, SG_ERR_DEVICE, "masked projection: cudaSetDevice");
  const int nx = g.nx, ny = g.ny, nz = g.nz, nc = nz - 1, layer = g.layer, mh = nx / 2, modes = (mh + 1) * ny;
  const size_t n = g.n, cells = (size_t)layer * nc, spec = (size_t)nc * modes;

  // The constructor (:190-218): solid and wall nodes, 1 / (rho0 hn), the columns' shares of each cell layer, dropped cells.
  std::vector<uint8_t> solid(n), wall(n, 0), dropped(cells, 0);
  std::vector<int32_t> levels(layer);
  std::vector<double> heights(n), inv(n, 0.0), low(cells), high(cells);
  solid_levels(g, ground, solid.data(), levels.data());
  node_heights(g, solid.data(), levels.data(), ground, heights.data());
  bool any = false;
  for (size_t i = 0; i < n; i++) any = any || solid[i];
  for (int c = 0; c < layer; c++) any = any || ground[c] > 0;
  for (int k = 0; k < nz; k++)
    for (int c = 0; c < layer; c++) {
      const size_t i = c + (size_t)k * layer;
      if (solid[i]) continue;
      if (g.zs[k] <= (double)ground[c]) wall[i] = 1;
      inv[i] = 1 / (rho[k] * heights[i]);
    }
  for (int k = 0; k < nc; k++)
    for (int c = 0; c < layer; c++) {
      const double half = g.dzs[k] / 2, middle = g.zs[k] + half, h = (double)ground[c];
      low[c + (size_t)k * layer] = std::min(1.0, std::max(0.0, (middle - std::max(h, g.zs[k])) / half));
      high[c + (size_t)k * layer] = std::min(1.0, std::max(0.0, (g.zs[k + 1] - std::max(h, middle)) / half));
    }
  for (int k = 0; k < nc; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const size_t l = (size_t)k * layer;
        const int i1 = (i + 1) % nx, j0 = j * nx, j1 = ((j + 1) % ny) * nx;
        if (high[i + j0 + l] == 0 && high[i1 + j0 + l] == 0 && high[i + j1 + l] == 0 && high[i1 + j1 + l] == 0) dropped[i + j0 + l] = 1;
      }

  // The flat solve's rows per mode (pressure.ts:36-44, :118-140): lower coefficient, pivot and cp = up / pivot of each
  // cell layer in the reference's elimination order. Modes it zeroes and the uniform mode's pinned lowest cell get an
  // infinite pivot (their values come out zero).
  std::vector<double> tlo(spec, 0.0), tcp(spec, 0.0), tpiv(spec, 0.0);
  auto exact = [](double x) { return x < 1e-12 ? 0 : x > 1 - 1e-12 ? 1 : x; };
  for (int m = 0; m <= mh; m++)
    for (int q = 0; q < ny; q++) {
      const double sx = exact(std::pow(std::sin(PI_ * m / nx), 2)), cx = exact(std::pow(std::cos(PI_ * m / nx), 2));
      const double sy = exact(std::pow(std::sin(PI_ * q / ny), 2)), cy = exact(std::pow(std::cos(PI_ * q / ny), 2));
      const double a = 4 * (sx * cy / (g.dx * g.dx) + cx * sy / (g.dy * g.dy)), b = cx * cy;
      const size_t mode = (size_t)m * ny + q;
      if ((a == 0 && b == 0) || (nc == 1 && a == 0)) {
        for (int k = 0; k < nc; k++) tpiv[(size_t)k * modes + mode] = INFINITY;
        continue;
      }
      const bool pinned = a == 0;
      double cprev = 0;
      for (int k = 0; k < nc; k++) {
        double di = -a / 2 * (rho[k] * g.dzs[k] / (2 * g.hz[k]) + rho[k + 1] * g.dzs[k] / (2 * g.hz[k + 1])), lo = 0, up = 0;
        if (k > 0) { lo = -a / 2 * rho[k] * g.dzs[k - 1] / (2 * g.hz[k]); const double v = b * rho[k] / (g.hz[k] * g.dzs[k]); lo += v; di -= v; }
        if (k < nc - 1) { up = -a / 2 * rho[k + 1] * g.dzs[k + 1] / (2 * g.hz[k + 1]); const double v = b * rho[k + 1] / (g.hz[k + 1] * g.dzs[k]); up += v; di -= v; }
        bool zero = false;
        if (pinned && k == 0) { lo = 0; di = 1; up = 0; zero = true; }
        if (pinned && k == 1) lo = 0;
        const double piv = k == 0 ? di : di - lo * cprev;
        cprev = up / piv;
        const size_t at = (size_t)k * modes + mode;
        tlo[at] = lo; tcp[at] = cprev; tpiv[at] = zero ? INFINITY : piv;
      }
    }
  std::vector<double2> tx(nx), ty(ny);
  for (int t = 0; t < nx; t++) tx[t] = make_double2(std::cos(2 * PI_ * t / nx), std::sin(2 * PI_ * t / nx));
  for (int t = 0; t < ny; t++) ty[t] = make_double2(std::cos(2 * PI_ * t / ny), std::sin(2 * PI_ * t / ny));

  // One allocation, 256-byte aligned parts.
  auto al = [](size_t bytes) { return (bytes + 255) / 256 * 256; };
  const size_t nparts = std::max((size_t)blocks(cells), (size_t)ny * nc);
  size_t off = 0;
  auto take = [&](size_t bytes) { const size_t o = off; off += al(bytes); return o; };
  const size_t oU = take(n * 4), oV = take(n * 4), oW = take(n * 4), oP = take(cells * 8), oB = take(cells * 8), oQ = take(cells * 8), oR = take(cells * 8),
               oZ = take(cells * 8), oD = take(cells * 8), oSd = take(cells * 8), oTu = take(n * 8), oTv = take(n * 8), oTw = take(n * 8),
               oPd = take(nparts * 8), oPr = take(nparts * 8), oLo = take(spec * 8), oCp = take(spec * 8), oPv = take(spec * 8),
               oS1 = take(spec * 16), oS2 = take(spec * 16), oTx = take((size_t)nx * 16), oTy = take((size_t)ny * 16), oSt = take(sizeof(MpState)),
               oSol = take(n), oWal = take(n), oDr = take(cells), oInv = take(n * 8), oLow = take(cells * 8), oHigh = take(cells * 8),
               oRho = take((size_t)nz * 8), oDz = take((size_t)nz * 8), oHz = take((size_t)nz * 8), total = off;
  auto* s = new sg_masked;
  s->ctx = ctx; s->hg = g; s->mh = mh; s->modes = modes; s->maxIt = max_iterations; s->tolerance = tolerance; s->any = any;
  s->dropped = dropped;
  cudaError_t e = cudaMalloc(&s->mem, total);
  if (e != cudaSuccess) { delete s; cudaGetLastError(); return sg_context_fail(ctx, SG_ERR_BUDGET, "masked projection: device memory"); }
  char* M = s->mem;
  s->u = (float*)(M + oU); s->v = (float*)(M + oV); s->w = (float*)(M + oW);
  s->p = (double*)(M + oP); s->b = (double*)(M + oB); s->q = (double*)(M + oQ); s->r = (double*)(M + oR); s->z = (double*)(M + oZ);
  s->d = (double*)(M + oD); s->sd = (double*)(M + oSd); s->tu = (double*)(M + oTu); s->tv = (double*)(M + oTv); s->tw = (double*)(M + oTw);
  s->pDot = (double*)(M + oPd); s->pRR = (double*)(M + oPr); s->lo = (double*)(M + oLo); s->cp = (double*)(M + oCp); s->piv = (double*)(M + oPv);
  s->S1 = (double2*)(M + oS1); s->S2 = (double2*)(M + oS2); s->twx = (double2*)(M + oTx); s->twy = (double2*)(M + oTy); s->st = (MpState*)(M + oSt);
  Geo& G = s->geo;
  G.solid = (const uint8_t*)(M + oSol); G.wall = (const uint8_t*)(M + oWal); G.dropped = (const uint8_t*)(M + oDr);
  G.invMass = (const double*)(M + oInv); G.low = (const double*)(M + oLow); G.high = (const double*)(M + oHigh);
  G.rho = (const double*)(M + oRho); G.dzs = (const double*)(M + oDz); G.hz = (const double*)(M + oHz);
  G.nx = nx; G.ny = ny; G.nz = nz; G.layer = layer; G.nc = nc; G.n = n; G.cells = cells; G.dx = g.dx; G.dy = g.dy;
  cudaStream_t st = sg_context_stream(ctx);
  std::vector<double> dz(nz, 0.0);
  std::copy(g.dzs, g.dzs + nz - 1, dz.begin());
  struct Up { size_t off; const void* src; size_t bytes; };
  const Up ups[] = {{oLo, tlo.data(), spec * 8}, {oCp, tcp.data(), spec * 8}, {oPv, tpiv.data(), spec * 8}, {oTx, tx.data(), (size_t)nx * 16},
                    {oTy, ty.data(), (size_t)ny * 16}, {oSol, solid.data(), n}, {oWal, wall.data(), n}, {oDr, dropped.data(), cells},
                    {oInv, inv.data(), n * 8}, {oLow, low.data(), cells * 8}, {oHigh, high.data(), cells * 8}, {oRho, rho, (size_t)nz * 8},
                    {oDz, dz.data(), (size_t)nz * 8}, {oHz, g.hz, (size_t)nz * 8}};
  for (const Up& up : ups)
    if ((e = cudaMemcpyAsync(M + up.off, up.src, up.bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
  if (e == cudaSuccess) e = cudaMemsetAsync(s->d, 0, cells * 8, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaFree(s->mem); delete s;
    return sg_context_fail(ctx, SG_ERR_DEVICE, (std::string("masked projection: ") + cudaGetErrorString(e)).c_str());
  }
  *out = s;
  return SG_OK;
}

int sg_masked_mask(sg_masked* m, float* u, float* v, float* w) {
  if (!m) return SG_ERR_INVALID;
  if (!u || !v || !w) return sg_context_fail(m->ctx, SG_ERR_INVALID, "masked projection: u, v and w buffers");
  cudaSetDevice(sg_context_device(m->ctx));
  cudaStream_t s = sg_context_stream(m->ctx);
  const size_t n = m->geo.n;
  cudaError_t e;
  float* host[3] = {u, v, w};
  float* dev[3] = {m->u, m->v, m->w};
  for (int f = 0; f < 3; f++)
    if ((e = cudaMemcpyAsync(dev[f], host[f], n * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess) return fail(m, "copy in", e);
  k_mp_mask<<<blocks(n), TPB, 0, s>>>(m->u, m->v, m->w, m->geo);
  for (int f = 0; f < 3; f++)
    if ((e = cudaMemcpyAsync(host[f], dev[f], n * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return fail(m, "copy out", e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) return fail(m, "mask", e);
  return SG_OK;
}

int sg_masked_divergence(sg_masked* m, const float* u, const float* v, const float* w, double* out) {
  if (!m) return SG_ERR_INVALID;
  if (!u || !v || !w || !out) return sg_context_fail(m->ctx, SG_ERR_INVALID, "masked projection: u, v, w and out buffers");
  cudaSetDevice(sg_context_device(m->ctx));
  cudaStream_t s = sg_context_stream(m->ctx);
  const size_t n = m->geo.n, cells = m->geo.cells;
  cudaError_t e;
  const float* host[3] = {u, v, w};
  float* dev[3] = {m->u, m->v, m->w};
  for (int f = 0; f < 3; f++)
    if ((e = cudaMemcpyAsync(dev[f], host[f], n * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess) return fail(m, "copy in", e);
  k_mp_div<float, 0><<<blocks(cells), TPB, 0, s>>>(m->u, m->v, m->w, m->b, nullptr, nullptr, m->geo, nullptr, 0);
  if ((e = cudaMemcpyAsync(out, m->b, cells * 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess || (e = cudaStreamSynchronize(s)) != cudaSuccess ||
      (e = cudaGetLastError()) != cudaSuccess)
    return fail(m, "divergence", e);
  return SG_OK;
}

int sg_masked_project(sg_masked* m, float* u, float* v, float* w, double dt, double* pressure) {
  if (!m) return SG_ERR_INVALID;
  if (!u || !v || !w || !pressure) return sg_context_fail(m->ctx, SG_ERR_INVALID, "masked projection: u, v, w and pressure buffers");
  if (!(dt > 0) || !std::isfinite(dt)) return sg_context_fail(m->ctx, SG_ERR_INVALID, "masked projection: dt > 0");
  cudaSetDevice(sg_context_device(m->ctx));
  cudaStream_t s = sg_context_stream(m->ctx);
  const Geo& g = m->geo;
  const size_t n = g.n, cells = g.cells;
  const int nb = blocks(n), cb = blocks(cells), nx = g.nx, ny = g.ny, nc = g.nc, mh = m->mh;
  cudaError_t e;
  float* host[3] = {u, v, w};
  float* dev[3] = {m->u, m->v, m->w};
  for (int f = 0; f < 3; f++)
    if ((e = cudaMemcpyAsync(dev[f], host[f], n * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess) return fail(m, "copy in", e);
  if ((e = cudaMemcpyAsync(m->p, pressure, cells * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess) return fail(m, "copy in", e);
  k_mp_mask<<<nb, TPB, 0, s>>>(m->u, m->v, m->w, g);
  m->iterations = 0; m->residual = 0;
  if (!m->any) {
    // No terrain at all: the flat projection exactly (:336-339); the pressure is the flat solve's, not a first guess.
    k_mp_flat_div<<<cb, TPB, 0, s>>>(m->u, m->v, m->w, m->b, dt, g);
    k_mp_xdft<<<dim3(ny, nc), threads_for(mh + 1), (size_t)nx * 8, s>>>(m->b, 1.0, nullptr, m->S1, m->twx, g, mh, nullptr, 0);
    k_mp_ydft<<<dim3(mh + 1, nc), threads_for(ny), (size_t)ny * 16, s>>>(m->S1, m->S2, m->twy, ny, mh, -1.0, nullptr, 0);
    k_mp_thomas<<<(m->modes + 63) / 64, 64, 0, s>>>(m->S2, m->lo, m->cp, m->piv, nullptr, nc, m->modes, nullptr, 0);
    k_mp_ydft<<<dim3(mh + 1, nc), threads_for(ny), (size_t)ny * 16, s>>>(m->S2, m->S1, m->twy, ny, mh, 1.0, nullptr, 0);
    k_mp_xidft<0><<<dim3(ny, nc), threads_for(nx), (size_t)(mh + 1) * 16, s>>>(m->S1, m->p, nullptr, nullptr, m->twx, g, mh, nullptr, 0);
    k_mp_flat_correct<<<nb, TPB, 0, s>>>(m->p, m->u, m->v, m->w, dt, g);
  } else {
    MpState init{};
    init.tolerance = m->tolerance; init.maxIt = m->maxIt;
    if ((e = cudaMemcpyAsync(m->st, &init, sizeof(MpState), cudaMemcpyHostToDevice, s)) != cudaSuccess) return fail(m, "state", e);
    // b = D R M u*, bb; q from the first guess, r = -b - S q, z = P S0^-1 P r, d = z, rz (:306-312).
    k_mp_div<float, 2><<<cb, TPB, 0, s>>>(m->u, m->v, m->w, m->b, nullptr, m->pDot, g, m->st, 0);
    k_mp_reduce<R_BB><<<1, TPB, 0, s>>>(m->st, m->pDot, cb, 0);
    k_mp_start<<<cb, TPB, 0, s>>>(m->p, m->q, dt, g, m->st);
    k_mp_grad<<<nb, TPB, 0, s>>>(m->q, m->tu, m->tv, m->tw, g, m->st, ZERO);
    k_mp_div<double, 0><<<cb, TPB, 0, s>>>(m->tu, m->tv, m->tw, m->sd, nullptr, nullptr, g, m->st, ZERO);
    k_mp_resid<<<cb, TPB, 0, s>>>(m->b, m->sd, m->r, m->pRR, g, m->st);
    enqueue_precondition(m, s, ZERO);
    k_mp_reduce<R_RZ0><<<1, TPB, 0, s>>>(m->st, m->pDot, ny * nc, ZERO);
    k_mp_dir<<<cb, TPB, 0, s>>>(m->d, m->z, g, m->st, 1);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(m, "launch", e);
    if (!m->chunk) {
      // Eight iterations as one graph (the buffers are the object's own, so one capture serves every call).
      cudaGraph_t graph = nullptr;
      if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return fail(m, "capture", e);
      for (int it = 0; it < CHUNK; it++) enqueue_iteration(m, s);
      e = cudaStreamEndCapture(s, &graph);
      if (e == cudaSuccess) e = cudaGraphInstantiate(&m->chunk, graph, 0);
      if (graph) cudaGraphDestroy(graph);
      if (e != cudaSuccess) { m->chunk = nullptr; return fail(m, "graph", e); }
    }
    // Every iteration either counts or stops, so maxIt / CHUNK + 1 replays always reach the stop.
    int done = 0;
    for (int c = 0;; c++) {
      if ((e = cudaMemcpyAsync(&done, &m->st->done, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess || (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail(m, "solve", e);
      if (done || c > m->maxIt / CHUNK + 1) break;
      if ((e = cudaGraphLaunch(m->chunk, s)) != cudaSuccess) return fail(m, "graph launch", e);
    }
    if (!done) return sg_context_fail(m->ctx, SG_ERR_DEVICE, "masked projection: the iterations did not stop");
    // u = M (u* - G phi); the pressure kept is phi / dt (:332-336).
    k_mp_finish<<<cb, TPB, 0, s>>>(m->q, m->p, dt, g, m->st);
    k_mp_grad<<<nb, TPB, 0, s>>>(m->q, m->tu, m->tv, m->tw, g, m->st, ZERO);
    k_mp_correct<<<nb, TPB, 0, s>>>(m->u, m->v, m->w, m->tu, m->tv, m->tw, g, m->st);
    MpState fin{};
    if ((e = cudaMemcpyAsync(&fin, m->st, sizeof(MpState), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return fail(m, "state", e);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(m, "solve", e);
    if (fin.done != ZERO) { m->iterations = fin.k; m->residual = std::sqrt(fin.rr / fin.bb); }
  }
  for (int f = 0; f < 3; f++)
    if ((e = cudaMemcpyAsync(host[f], dev[f], n * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return fail(m, "copy out", e);
  if ((e = cudaMemcpyAsync(pressure, m->p, cells * 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return fail(m, "copy out", e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) return fail(m, "project", e);
  return SG_OK;
}

int sg_masked_stats(sg_masked* m, int32_t* iterations, double* residual) {
  if (!m) return SG_ERR_INVALID;
  if (iterations) *iterations = m->iterations;
  if (residual) *residual = m->residual;
  return SG_OK;
}

int sg_masked_dropped(sg_masked* m, uint8_t* dropped) {
  if (!m || !dropped) return SG_ERR_INVALID;
  std::memcpy(dropped, m->dropped.data(), m->dropped.size());
  return SG_OK;
}

int sg_faces_create(sg_context* ctx, const sg_grid* grid, const double* rho, const float* ground, double tolerance, int max_iterations,
                    sg_faces** out) {
  if (!ctx || !out) return SG_ERR_INVALID;
  *out = nullptr;
  HostGrid g;
  if (!host_grid(grid, g) || !rho || !ground)
    return sg_context_fail(ctx, SG_ERR_INVALID, "masked faces: a grid with nx, ny >= 1, nz >= 3, dx, dy > 0, its level arrays, rho and the ground");
  if (g.nx > 2048 || g.ny > 2048) return sg_context_fail(ctx, SG_ERR_INVALID, "masked faces: nx and ny at most 2048");
  if (g.n > (size_t)1 << 30) return sg_context_fail(ctx, SG_ERR_INVALID, "masked faces: at most 2^30 nodes");
  if (!(tolerance >= 0) || max_iterations < 0) return sg_context_fail(ctx, SG_ERR_INVALID, "masked faces: tolerance >= 0, max_iterations >= 0");
  for (int k = 0; k < g.nz; k++)
    if (!(g.hz[k] > 0) || (k < g.nz - 1 && !(g.dzs[k] > 0)) || !(rho[k] > 0))
      return sg_context_fail(ctx, SG_ERR_INVALID, "masked faces: level spacings and densities must be positive");
  for (int c = 0; c < g.layer; c++)
    if (!std::isfinite(ground[c])) return sg_context_fail(ctx, SG_ERR_INVALID, "masked faces: finite ground heights");
  if (cudaSetDevice(sg_context_device(ctx)) != cudaSuccess) return sg_context_fail(ctx, SG_ERR_DEVICE, "masked faces: cudaSetDevice");
  const int nx = g.nx, ny = g.ny, nz = g.nz, layer = g.layer, mh = nx / 2, modes = (mh + 1) * ny;
  const size_t n = g.n, spec = (size_t)nz * modes;

  // setTerrain (advection.ts:78-90) with the model's geometry (model.ts:366-377): open faces, node heights (1 in the
  // ground), the faces' open heights.
  std::vector<uint8_t> solid(n), open(n, 0);
  std::vector<int32_t> levels(layer);
  std::vector<double> heights(n), hn(n), ax(n), ay(n);
  solid_levels(g, ground, solid.data(), levels.data());
  node_heights(g, solid.data(), levels.data(), ground, heights.data());
  face_apertures(g, solid.data(), ground, ax.data(), ay.data());
  for (size_t i = 0; i < n; i++) hn[i] = solid[i] ? 1 : heights[i];
  for (int z = 0; z < nz; z++)
    for (int y = 0; y < ny; y++)
      for (int x = 0; x < nx; x++) {
        const size_t i = x + (size_t)nx * y + (size_t)layer * z, l = (size_t)layer * z;
        if (solid[i]) continue;
        if (!solid[(x + 1) % nx + (size_t)nx * y + l]) open[i] |= 1;
        if (!solid[x + (size_t)nx * ((y + 1) % ny) + l]) open[i] |= 2;
        if (z < nz - 1 && !solid[i + layer]) open[i] |= 4;
      }

  // The flat face solve's rows per mode (advection.ts:222-241): each level's lower coefficient, pivot and cp in the
  // reference's order; the uniform mode's pinned lowest level with an infinite pivot.
  std::vector<double> tlo(spec, 0.0), tcp(spec, 0.0), tpiv(spec, 0.0);
  auto face = [&](int k) { return k < 0 || k >= nz - 1 ? 0.0 : (rho[k] + rho[k + 1]) / 2; };
  for (int m = 0; m <= mh; m++)
    for (int q = 0; q < ny; q++) {
      const double lam = m == 0 && q == 0 ? 0
                                          : 4 * std::pow(std::sin(PI_ * m / nx), 2) / (g.dx * g.dx) + 4 * std::pow(std::sin(PI_ * q / ny), 2) / (g.dy * g.dy);
      const bool pinned = lam == 0;
      const size_t mode = (size_t)m * ny + q;
      double cprev = 0;
      for (int k = 0; k < nz; k++) {
        double lo = k > 0 ? face(k - 1) / g.dzs[k - 1] : 0, up = k < nz - 1 ? face(k) / g.dzs[k] : 0, di = -rho[k] * g.hz[k] * lam - lo - up;
        bool zero = false;
        if (pinned && k == 0) { lo = 0; di = 1; up = 0; zero = true; }
        if (pinned && k == 1) lo = 0;
        const double piv = k == 0 ? di : di - lo * cprev;
        cprev = up / piv;
        const size_t at = (size_t)k * modes + mode;
        tlo[at] = lo; tcp[at] = cprev; tpiv[at] = zero ? INFINITY : piv;
      }
    }
  std::vector<double2> tx(nx), ty(ny);
  for (int t = 0; t < nx; t++) tx[t] = make_double2(std::cos(2 * PI_ * t / nx), std::sin(2 * PI_ * t / nx));
  for (int t = 0; t < ny; t++) ty[t] = make_double2(std::cos(2 * PI_ * t / ny), std::sin(2 * PI_ * t / ny));

  auto al = [](size_t bytes) { return (bytes + 255) / 256 * 256; };
  const size_t nparts = std::max((size_t)blocks(n), (size_t)ny * nz);
  size_t off = 0;
  auto take = [&](size_t bytes) { const size_t o = off; off += al(bytes); return o; };
  const size_t oU = take(n * 4), oV = take(n * 4), oW = take(n * 4), oMx = take(n * 8), oMy = take(n * 8), oMz = take(n * 8), oDiv = take(n * 8),
               oB = take(n * 8), oQ = take(n * 8), oR = take(n * 8), oZ = take(n * 8), oD = take(n * 8), oSd = take(n * 8), oPd = take(nparts * 8),
               oPr = take(nparts * 8), oLo = take(spec * 8), oCp = take(spec * 8), oPv = take(spec * 8), oS1 = take(spec * 16), oS2 = take(spec * 16),
               oTx = take((size_t)nx * 16), oTy = take((size_t)ny * 16), oSt = take(sizeof(MpState)), oOpen = take(n), oAx = take(n * 8),
               oAy = take(n * 8), oHn = take(n * 8), oRho = take((size_t)nz * 8), oDz = take((size_t)nz * 8), oHz = take((size_t)nz * 8), total = off;
  auto* f = new sg_faces;
  f->ctx = ctx; f->mh = mh; f->modes = modes; f->maxIt = max_iterations; f->tolerance = tolerance;
  cudaError_t e = cudaMalloc(&f->mem, total);
  if (e != cudaSuccess) { delete f; cudaGetLastError(); return sg_context_fail(ctx, SG_ERR_BUDGET, "masked faces: device memory"); }
  char* M = f->mem;
  f->u = (float*)(M + oU); f->v = (float*)(M + oV); f->w = (float*)(M + oW);
  f->mx = (double*)(M + oMx); f->my = (double*)(M + oMy); f->mz = (double*)(M + oMz); f->div = (double*)(M + oDiv); f->b = (double*)(M + oB);
  f->q = (double*)(M + oQ); f->r = (double*)(M + oR); f->z = (double*)(M + oZ); f->d = (double*)(M + oD); f->sd = (double*)(M + oSd);
  f->pDot = (double*)(M + oPd); f->pRR = (double*)(M + oPr); f->lo = (double*)(M + oLo); f->cp = (double*)(M + oCp); f->piv = (double*)(M + oPv);
  f->S1 = (double2*)(M + oS1); f->S2 = (double2*)(M + oS2); f->twx = (double2*)(M + oTx); f->twy = (double2*)(M + oTy); f->st = (MpState*)(M + oSt);
  f->hz = (double*)(M + oHz);
  FaceGeo& F = f->fg;
  F.open = (const uint8_t*)(M + oOpen); F.ax = (const double*)(M + oAx); F.ay = (const double*)(M + oAy); F.hn = (const double*)(M + oHn);
  F.rho = (const double*)(M + oRho); F.dzs = (const double*)(M + oDz);
  F.nx = nx; F.ny = ny; F.nz = nz; F.layer = layer; F.n = n; F.dx = g.dx; F.dy = g.dy;
  Geo& G = f->geo;
  G.nx = nx; G.ny = ny; G.nz = nz; G.layer = layer; G.nc = nz; G.n = n; G.cells = n; G.dx = g.dx; G.dy = g.dy;
  cudaStream_t st = sg_context_stream(ctx);
  std::vector<double> dz(nz, 0.0);
  std::copy(g.dzs, g.dzs + nz - 1, dz.begin());
  struct Up { size_t off; const void* src; size_t bytes; };
  const Up ups[] = {{oLo, tlo.data(), spec * 8}, {oCp, tcp.data(), spec * 8}, {oPv, tpiv.data(), spec * 8}, {oTx, tx.data(), (size_t)nx * 16},
                    {oTy, ty.data(), (size_t)ny * 16}, {oOpen, open.data(), n}, {oAx, ax.data(), n * 8}, {oAy, ay.data(), n * 8},
                    {oHn, hn.data(), n * 8}, {oRho, rho, (size_t)nz * 8}, {oDz, dz.data(), (size_t)nz * 8}, {oHz, g.hz, (size_t)nz * 8}};
  for (const Up& up : ups)
    if ((e = cudaMemcpyAsync(M + up.off, up.src, up.bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
  if (e == cudaSuccess) e = cudaMemsetAsync(f->d, 0, n * 8, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaFree(f->mem); delete f;
    return sg_context_fail(ctx, SG_ERR_DEVICE, (std::string("masked faces: ") + cudaGetErrorString(e)).c_str());
  }
  *out = f;
  return SG_OK;
}

int sg_faces_set_velocity(sg_faces* f, const float* u, const float* v, const float* w, double* mx, double* my, double* mz, double* div) {
  if (!f) return SG_ERR_INVALID;
  if (!u || !v || !w) return sg_context_fail(f->ctx, SG_ERR_INVALID, "masked faces: u, v and w buffers");
  cudaSetDevice(sg_context_device(f->ctx));
  cudaStream_t s = sg_context_stream(f->ctx);
  const Geo& g = f->geo;
  const size_t n = g.n;
  const int nb = blocks(n);
  auto fail_f = [&](const char* what, cudaError_t e) {
    return sg_context_fail(f->ctx, SG_ERR_DEVICE, (std::string("masked faces: ") + what + ": " + cudaGetErrorString(e)).c_str());
  };
  cudaError_t e;
  const float* host[3] = {u, v, w};
  float* dev[3] = {f->u, f->v, f->w};
  for (int k = 0; k < 3; k++)
    if ((e = cudaMemcpyAsync(dev[k], host[k], n * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess) return fail_f("copy in", e);
  MpState init{};
  init.tolerance = f->tolerance; init.maxIt = f->maxIt; init.keepBB = 1;
  if ((e = cudaMemcpyAsync(f->st, &init, sizeof(MpState), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
      (e = cudaMemsetAsync(f->q, 0, n * 8, s)) != cudaSuccess)
    return fail_f("state", e);
  // faces, shut next to the ground; b = -h div, bb (= the first rr); r = b; z = S0^-1 r, rz; d = z (:117-126).
  k_tm_faces<<<nb, TPB, 0, s>>>(f->u, f->v, f->w, f->mx, f->my, f->mz, f->fg);
  k_tm_tdiv<0><<<nb, TPB, 0, s>>>(f->mx, f->my, f->mz, f->b, f->pRR, f->fg);
  k_mp_reduce<R_BB><<<1, TPB, 0, s>>>(f->st, f->pRR, nb, 0);
  if ((e = cudaMemcpyAsync(f->r, f->b, n * 8, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return fail_f("copy", e);
  enqueue_face_precondition(f, s, ZERO);
  k_mp_reduce<R_RZ0><<<1, TPB, 0, s>>>(f->st, f->pDot, g.ny * g.nc, ZERO);
  k_mp_dir<<<nb, TPB, 0, s>>>(f->d, f->z, g, f->st, 1);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail_f("launch", e);
  if (!f->chunk) {
    cudaGraph_t graph = nullptr;
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return fail_f("capture", e);
    for (int it = 0; it < CHUNK; it++) enqueue_face_iteration(f, s);
    e = cudaStreamEndCapture(s, &graph);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&f->chunk, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) { f->chunk = nullptr; return fail_f("graph", e); }
  }
  int done = 0;
  for (int c = 0;; c++) {
    if ((e = cudaMemcpyAsync(&done, &f->st->done, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess || (e = cudaStreamSynchronize(s)) != cudaSuccess)
      return fail_f("solve", e);
    if (done || c > f->maxIt / CHUNK + 1) break;
    if ((e = cudaGraphLaunch(f->chunk, s)) != cudaSuccess) return fail_f("graph launch", e);
  }
  if (!done) return sg_context_fail(f->ctx, SG_ERR_DEVICE, "masked faces: the iterations did not stop");
  // The fluxes lose M rho0 grad(q); div the apertures' divergence over the node heights (:150-152).
  k_tm_correct<<<nb, TPB, 0, s>>>(f->q, f->mx, f->my, f->mz, f->fg, f->st);
  k_tm_tdiv<1><<<nb, TPB, 0, s>>>(f->mx, f->my, f->mz, f->div, nullptr, f->fg);
  MpState fin{};
  if ((e = cudaMemcpyAsync(&fin, f->st, sizeof(MpState), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return fail_f("state", e);
  double* outs[4] = {mx, my, mz, div};
  const double* devs[4] = {f->mx, f->my, f->mz, f->div};
  for (int k = 0; k < 4; k++)
    if (outs[k] && (e = cudaMemcpyAsync(outs[k], devs[k], n * 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return fail_f("copy out", e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) return fail_f("faces", e);
  if (fin.done == ZERO) { f->iterations = 0; f->residual = 0; }
  else { f->iterations = fin.k; f->residual = std::sqrt(fin.rr / fin.bb); }
  return SG_OK;
}

int sg_faces_stats(sg_faces* f, int32_t* iterations, double* residual) {
  if (!f) return SG_ERR_INVALID;
  if (iterations) *iterations = f->iterations;
  if (residual) *residual = f->residual;
  return SG_OK;
}

int sg_faces_destroy(sg_faces* f) {
  if (!f) return SG_ERR_INVALID;
  cudaSetDevice(sg_context_device(f->ctx));
  cudaStreamSynchronize(sg_context_stream(f->ctx));
  if (f->chunk) cudaGraphExecDestroy(f->chunk);
  cudaFree(f->mem);
  delete f;
  return SG_OK;
}

int sg_masked_destroy(sg_masked* m) {
  if (!m) return SG_ERR_INVALID;
  cudaSetDevice(sg_context_device(m->ctx));
  cudaStreamSynchronize(sg_context_stream(m->ctx));
  if (m->chunk) cudaGraphExecDestroy(m->chunk);
  cudaFree(m->mem);
  delete m;
  return SG_OK;
}

}  // extern "C"
