// Per-run diagnostics on the device, for runs with the rotation switch: the rotation tracking the reference runs after
// every step (afterStep -> updateRotation, src/core/model.ts:1130-1131, :1609-1648) together with the ensemble's swaths
// (addSwaths, src/ensemble/member.ts:71-89), and the domain diagnostics a sample reads (diagnostics, :1672-1696).
// The per-step part stays on the device (two launches, no host copy); a sample copies a few scalars and five ground
// columns to the host, which counts the cores and takes the outflow's quantile on those (sg_run_diagnostics).
#include <cuda_runtime.h>
#include <math.h>
#include "sg_common.cuh"
#include "sg_physics.cuh"
#include "sg_kernels.h"
#include "sg_device.cuh"

namespace sg {

namespace {

constexpr float CORE_ROTATION_W = 10.f;   // src/core/model.ts:112
constexpr int ROT_COLS = 64;              // columns per block of the column kernel (the COLS work items)

__device__ __forceinline__ unsigned long long* key(const RunDesc& R, int slot) { return reinterpret_cast<unsigned long long*>(R.rot + slot); }
// A non-negative value with the first column on ties: larger keys for larger values, then for smaller columns.
__device__ __forceinline__ unsigned long long argmax_key(float v, int c) {
  return ((unsigned long long)__float_as_uint(v) << 32) | (unsigned long long)(0xffffffffu - (unsigned)c);
}
__device__ __forceinline__ float key_value(unsigned long long k) { return __uint_as_float((unsigned)(k >> 32)); }
__device__ __forceinline__ int key_column(unsigned long long k) { return (int)(0xffffffffu - (unsigned)(k & 0xffffffffu)); }

// Vertical vorticity dv/dx - du/dy at a node (zeta, src/core/model.ts:1597-1601).
__device__ __forceinline__ float zeta_at(const RunDesc& R, const float* __restrict__ u, const float* __restrict__ v, int x, int y, int z) {
  const int nx = R.nx, ny = R.ny, l = z * R.layer;
  const int xp = x + 1 == nx ? 0 : x + 1, xm = x == 0 ? nx - 1 : x - 1;
  const int yp = (y + 1 == ny ? 0 : y + 1) * nx, ym = (y == 0 ? ny - 1 : y - 1) * nx;
  return (v[xp + nx * y + l] - v[xm + nx * y + l]) * (.5f * R.inv_dx) - (u[x + yp + l] - u[x + ym + l]) * (.5f * R.inv_dy);
}

}  // namespace

// updateRotation's column loop (:1616-1630), ROT_COLS columns a block with ROT_SLICES threads per column, each
// summing every ROT_SLICES-th level (the slices combined in shared memory in a fixed order): the 0-1 and 0-3 km sums of
// w zeta hz, the 2-5 km UH column and the core sums of its nodes above CORE_ROTATION_W; the maxima with their columns
// and the minimum as 64-bit keys for k_rotation_summary. Unless `refresh`, the surface wind and the UH column folded
// into the swaths of the ground under the moving domain (addSwaths: the shift is the domain's motion to the end of
// this step, whole columns).
constexpr int ROT_SLICES = 4;
__global__ void __launch_bounds__(ROT_COLS * ROT_SLICES) k_rotation_columns(const RunDesc* __restrict__ runs, const int4* items, int nitems, int refresh) {
  __shared__ float part[5][ROT_SLICES][ROT_COLS];
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED] || !(R.flags & RF_ROTATION)) continue;
    const double dt = R.dt;
    const int layer = R.layer, nx = R.nx, ny = R.ny, lc = threadIdx.x % ROT_COLS, sl = threadIdx.x / ROT_COLS;
    const int c = items[it].y * ROT_COLS + lc;
    const bool on = c < layer;
    const int x = on ? c % nx : 0, y = on ? c / nx : 0;
    const float* __restrict__ u = field(R, 0, U);
    const float* __restrict__ v = field(R, 0, V);
    const float* __restrict__ w = field(R, 0, W);
    float low1 = 0.f, low3 = 0.f, uh = 0.f, sw = 0.f, swz = 0.f;  // levels 1..top1, top1+1..top3, 2-5 km
    if (on) {
      for (int z = 1 + sl; z <= R.uh_top3; z += ROT_SLICES) {
        const float t = w[c + z * layer] * zeta_at(R, u, v, x, y, z) * lvl(R, L_HZ, z);
        if (z <= R.uh_top1) low1 += t; else low3 += t;
      }
      for (int z = R.uh_z0 + sl; z <= R.uh_z1 && R.uh_z0 >= 0; z += ROT_SLICES) {
        const float wv = w[c + z * layer], wz = wv * zeta_at(R, u, v, x, y, z) * lvl(R, L_HZ, z);
        uh += wz;
        if (wv > CORE_ROTATION_W) { sw += wv * lvl(R, L_HZ, z); swz += wz; }
      }
    }
    part[0][sl][lc] = low1; part[1][sl][lc] = low3; part[2][sl][lc] = uh; part[3][sl][lc] = sw; part[4][sl][lc] = swz;
    __syncthreads();
    if (sl == 0) {  // (the first ROT_COLS threads: whole warps)
      for (int k = 1; k < ROT_SLICES; k++) { low1 += part[0][k][lc]; low3 += part[1][k][lc]; uh += part[2][k][lc]; sw += part[3][k][lc]; swz += part[4][k][lc]; }
      const float low01 = R.uh_top1 >= 1 ? low1 : 0.f, low = low1 + low3;
      // the keys of this column (0: none), reduced over the warp before one atomic per warp
      unsigned long long kq[4] = {on && uh > 0.f ? argmax_key(uh, c) : 0ull, on && uh < 0.f ? (unsigned long long)__float_as_uint(-uh) : 0ull,
                                  on && low01 > 0.f ? argmax_key(low01, c) : 0ull, on && low > 0.f ? (unsigned long long)__float_as_uint(low) : 0ull};
#pragma unroll
      for (int q = 0; q < 4; q++) {
        for (int o = 16; o > 0; o >>= 1) { const unsigned long long other = __shfl_xor_sync(0xffffffffu, kq[q], o); kq[q] = other > kq[q] ? other : kq[q]; }
        if ((threadIdx.x & 31) == 0 && kq[q]) atomicMax(key(R, q == 0 ? K_UH : q == 1 ? K_MIN : q == 2 ? K_01 : K_03), kq[q]);
      }
    }
    if (sl == 0 && on) {
      R.diag[DG_UH * layer + c] = uh;
      R.diag[DG_COREW * layer + c] = sw;
      R.diag[DG_COREWZ * layer + c] = swz;
      if (!refresh) {
        const double time = R.rot[R_TIME] + dt;
        const long sx = (long)floor((double)R.frame_u * time / R.dx + .5), sy = (long)floor((double)R.frame_v * time / R.dy + .5);
        const int gx = (int)(((x + sx) % nx + nx) % nx), gy = (int)(((y + sy) % ny + ny) % ny), g = gx + nx * gy;
        const float ug = u[c] + R.frame_u, vg = v[c] + R.frame_v, wind = sqrtf(ug * ug + vg * vg);
        float* gust = R.diag + DG_GUST_MAX * layer;
        float* uhm = R.diag + DG_UH_MAX * layer;
        if (wind > gust[g]) gust[g] = wind;
        if (uh > uhm[g]) uhm[g] = uh;
      }
    }
    __syncthreads();
  }
}

// One block per run (updateRotation's cores and summary, :1631-1647): the columns with core nodes are labelled by
// their component's smallest column (8 neighbours, periodic) by repeated minimum passes; the components, in the order
// of those columns, give the core vorticity (sum of w zeta hz / sum of w hz, FP64 sums in a fixed order), the UH
// peak of the most rotating one and the strongest anticyclonic one; then the rotation state from the step's keys, the
// time the rotation has held (unless `refresh`, which keeps it and the model time), and the keys cleared.
__global__ void k_rotation_summary(const RunDesc* __restrict__ runs, const int4* items, int nitems, int refresh) {
  __shared__ int roots[256];
  __shared__ int nroots;
  __shared__ double red[3][32];
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED] || !(R.flags & RF_ROTATION)) continue;
    const int layer = R.layer, nx = R.nx, ny = R.ny, t = threadIdx.x, NT = blockDim.x;
    const float* coreW = R.diag + DG_COREW * layer;
    const float* coreWZ = R.diag + DG_COREWZ * layer;
    const float* col = R.diag + DG_UH * layer;
    int* label = reinterpret_cast<int*>(R.diag + DG_LABEL * layer);
    int any = 0;
    for (int c = t; c < layer; c += NT) { const bool core = coreW[c] > 0.f; label[c] = core ? c : -1; any |= core; }
    const bool hasCores = __syncthreads_or(any);  // (no core column: no labels, no components)
    // labels only decrease, so the passes end (at most one per column)
    for (int pass = 0; pass < layer && hasCores && __syncthreads_or(any); pass++) {
      int changed = 0;
      for (int c = t; c < layer; c += NT) {
        const int l0 = label[c];
        if (l0 < 0) continue;
        int m = min(l0, label[l0]);
        const int x = c % nx, y = c / nx;
        for (int oy = -1; oy <= 1; oy++) {
          const int yy = (y + oy + ny) % ny;
          for (int ox = -1; ox <= 1; ox++) {
            const int lb = label[(x + ox + nx) % nx + nx * yy];
            if (lb >= 0 && lb < m) m = lb;
          }
        }
        if (m < l0) { label[c] = m; changed = 1; }
      }
      any = changed;
    }
    __syncthreads();
    double coreZeta = 0, coreUH = 0, coreAnti = 0;  // meaningful in thread 0
    // the components in the order of their smallest columns (the roots), a block of columns at a time: the block's
    // roots are compacted in column order by warp ballots
    for (int start = 0; start < layer && hasCores; start += NT) {
      const int c = start + t;
      const bool isRoot = c < layer && label[c] == c;
      const unsigned ballot = __ballot_sync(0xffffffffu, isRoot);
      if ((t & 31) == 0) red[0][t >> 5] = (double)__popc(ballot);
      __syncthreads();
      if (t == 0) {
        int acc = 0;
        for (int wi = 0; wi < (NT + 31) / 32; wi++) { const int k = (int)red[0][wi]; red[1][wi] = (double)acc; acc += k; }
        nroots = acc;
      }
      __syncthreads();
      if (isRoot) roots[(int)red[1][t >> 5] + __popc(ballot & ((1u << (t & 31)) - 1u))] = c;
      __syncthreads();
      const int nr = nroots;
      for (int k = 0; k < nr; k++) {
        const int r = roots[k];
        double sw = 0, swz = 0, peak = 0;
        for (int c = t; c < layer; c += NT)
          if (label[c] == r) { sw += coreW[c]; swz += coreWZ[c]; peak = fmax(peak, (double)col[c]); }
        for (int o = 16; o > 0; o >>= 1) {
          sw += __shfl_xor_sync(0xffffffffu, sw, o);
          swz += __shfl_xor_sync(0xffffffffu, swz, o);
          peak = fmax(peak, __shfl_xor_sync(0xffffffffu, peak, o));
        }
        if ((t & 31) == 0) { red[0][t >> 5] = sw; red[1][t >> 5] = swz; red[2][t >> 5] = peak; }
        __syncthreads();
        if (t == 0) {
          double a = 0, b = 0, p = 0;
          for (int wi = 0; wi < (NT + 31) / 32; wi++) { a += red[0][wi]; b += red[1][wi]; p = fmax(p, red[2][wi]); }
          const double ratio = b / a;
          if (ratio > coreZeta) { coreZeta = ratio; coreUH = p; }
          coreAnti = fmax(coreAnti, -ratio);
        }
        __syncthreads();
      }
      __syncthreads();
    }
    if (t == 0) {
      const unsigned long long kuh = *key(R, K_UH), k01 = *key(R, K_01), kmin = *key(R, K_MIN), k03 = *key(R, K_03);
      double* rot = R.rot;
      rot[R_UH] = kuh ? (double)key_value(kuh) : 0.0;
      rot[R_X] = kuh ? (double)(key_column(kuh) % nx) : 0.0;
      rot[R_Y] = kuh ? (double)(key_column(kuh) / nx) : 0.0;
      rot[R_ANTI] = (double)__uint_as_float((unsigned)kmin);
      rot[R_UH01] = k01 ? (double)key_value(k01) : 0.0;
      rot[R_LOW] = k01 ? (double)key_column(k01) : 0.0;
      rot[R_UH03] = (double)__uint_as_float((unsigned)k03);
      rot[R_CZETA] = coreZeta; rot[R_CUH] = coreUH; rot[R_CANTI] = coreAnti;
      if (!refresh) {
        rot[R_PERSISTED] = coreZeta >= (double)R.meso_zeta ? rot[R_PERSISTED] + (double)R.dt : 0.0;
        rot[R_TIME] += (double)R.dt;
      }
      *key(R, K_UH) = 0; *key(R, K_01) = 0; *key(R, K_MIN) = 0; *key(R, K_03) = 0;
    }
    __syncthreads();
  }
}

// A sample's domain maxima (diagnostics, :1676-1683) over node chunks of one run, into the run's M_* keys (non-negative
// values as their bits); thread per ground column of the chunk: the precipitation rate (precipitationFlux with the
// one-moment fall speeds at the ground density, src/core/surfaceflux.ts:31-36, mm/h), the largest hail (mm), the
// surface wind, the ground theta_v (rkw.ts:73-74) and whether the column holds a cloudy updraught core (countCores'
// test, :1655-1658).
__global__ void k_diag_sample(const RunDesc* __restrict__ runs, const int4* items, int nitems) {
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (!(R.flags & RF_ROTATION)) continue;
    const int layer = R.layer, i0 = items[it].y * CHUNK, i1 = min(R.n, i0 + CHUNK);
    const float* __restrict__ w = field(R, 0, W);
    const float* __restrict__ cl = field(R, 0, CLOUD);
    const float* __restrict__ ic = field(R, 0, ICE);
    const float* __restrict__ cold = field(R, 0, COLD);
    float up = 0.f, down = 0.f, cloud = 0.f, top = 0.f, thermal = 0.f, cmax = 0.f;
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      const int z = i / layer;
      const float alt = lvl(R, L_ZS, z) * 1e-3f, wv = w[i], ci = cl[i] + ic[i];
      up = fmaxf(up, wv); down = fmaxf(down, -wv); cloud = fmaxf(cloud, ci);
      if (ci > .00007f) top = fmaxf(top, alt);
      if (wv > .6f) thermal = fmaxf(thermal, alt);
      if (lvl(R, L_ZS, z) < 1500.f) cmax = fmaxf(cmax, cold[i]);
      if (z == 0) {
        const int c = i;
        const float rho0 = R.rho0;
        const float r_ = field(R, 0, RAIN)[c], s = field(R, 0, SNOW)[c], gr = field(R, 0, GRAUPEL)[c], h = field(R, 0, HAIL)[c];
        const float flux = rho0 * r_ * phys::rainFall(r_, rho0, 1.f) +
                           rho0 * (s * phys::snowFall(s, rho0, 1.f) + gr * (gr > 0.f ? phys::graupelFall(gr, rho0) : 0.f) +
                                   h * (h > 0.f ? phys::hailFall(h, rho0) : 0.f));
        const float ug = field(R, 0, U)[c] + R.frame_u, vg = field(R, 0, V)[c] + R.frame_v;
        bool active = false;
        for (int k = R.core_lo; k <= R.core_hi && R.core_lo >= 0 && !active; k++)
          active = w[c + k * layer] > 2.f && cl[c + k * layer] + ic[c + k * layer] > .00007f;
        R.diag[DG_RATE * layer + c] = flux * 3600.f;
        R.diag[DG_HAIL * layer + c] = phys::hailMaxDiameter(h, rho0) * 1000.f;
        R.diag[DG_GUST * layer + c] = sqrtf(ug * ug + vg * vg);
        // theta as the run reads it back (the FP32 rounding of theta_b + theta'), then theta (1 + 0.61 q) stored as FP32
        const float th = (float)((double)field(R, 0, THETA)[c] + R.lv64[D_THB * R.nz]);
        R.diag[DG_THV * layer + c] = (float)((double)th * (1.0 + .61 * (double)field(R, 0, Q)[c]));
        R.diag[DG_MASK * layer + c] = active ? 1.f : 0.f;
      }
    }
    const float v[6] = {up, down, cloud, top, thermal, cmax};
#pragma unroll
    for (int k = 0; k < 6; k++) {
      float m = v[k];
      for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
      if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(key(R, M_UP + k), (unsigned long long)__float_as_uint(m));
    }
  }
}

void launch_rotation_columns(const Launch& cols, int refresh) {
  if (cols.n) k_rotation_columns<<<GRID(cols.n, cols.cap), ROT_COLS * ROT_SLICES, 0, cols.stream>>>(cols.runs, cols.items, cols.n, refresh);
}
void launch_rotation_summary(const Launch& runs, int refresh) {
  if (runs.n) k_rotation_summary<<<GRID(runs.n, runs.cap), 256, 0, runs.stream>>>(runs.runs, runs.items, runs.n, refresh);
}
void launch_diag_sample(const Launch& L) { k_diag_sample<<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n); }

}  // namespace sg
