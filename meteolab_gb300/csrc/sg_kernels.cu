// The StormLab step as sm_103a kernels. Every kernel is a grid-stride loop over a list of work items
// (run slot, a, b, c): one launch advances every run of a batch, whatever its size, and the same launch sequence
// captured once replays as a CUDA graph. No kernel waits on another block, so nothing here can spin.
//
// Step order (AtmosphereModel.step, src/core/model.ts:873-877, with the reference's phases):
//   fall_courant  -> sediment                     beginStep: fall speeds, hail swath, CFL-split sedimentation (:893-932)
//   face projection (div+xfft, modes, xifft, correct)   FluxTransport.setVelocity in phases (:1039, advection.ts:190-255)
//   3 x transport stage (+ pressure projection after stages 0, 1)  RK3 with buoyancy and rigid w (:1042-1049)
//   fill_partial -> fill_final                    positivity fix sums (:1116-1121, :606-617)
//   physics                                       per-node physics (:1347-1531) + fill apply + cold decay
//   viscosity -> mix                              Turbulence.viscosity / mix, drag, rigid walls (:1161-1195)
//   final pressure projection with the wind clip  project(dt) (:1575-1595)
//   step_end                                      budgets and counters
#include <cuda_runtime.h>
#include <math.h>
#include <algorithm>
#include "sg_common.cuh"
#include "sg_fft.cuh"
#include "sg_physics.cuh"
#include "sg_charge.cuh"
#include "sg_rain2m.cuh"
#include "sg_ice2m.cuh"
#include "sg_kernels.h"
#include "sg_device.cuh"

namespace sg {

__device__ __forceinline__ void atomicMaxPos(float* addr, float v) {
  // Non-negative floats order like their bit patterns.
  atomicMax(reinterpret_cast<int*>(addr), __float_as_int(v));
}

template <class T>
__device__ __forceinline__ T warpSum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warpMax(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
// Block sum of `count` doubles per thread into out[] (fixed order: warp shuffles, then warps in order).
template <int COUNT>
__device__ void blockSums(double (&v)[COUNT], double* out, double* sh /* >= 32*COUNT */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int c = 0; c < COUNT; c++) v[c] = warpSum(v[c]);
  __syncthreads();
  if (lane == 0)
    for (int c = 0; c < COUNT; c++) sh[warp * COUNT + c] = v[c];
  __syncthreads();
  if (threadIdx.x < COUNT) {
    double s = 0;
    for (int w = 0; w < nw; w++) s += sh[w * COUNT + threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

// Compensated FP32 sums: a partial sum is kept as hi + lo (two FP32 words, about 48 significant bits) and terms are
// added with TwoSum (Knuth), so the per-thread sums of the positivity fix and the water budget keep FP64-like accuracy
// on the FP32 pipes (GB300 runs FP64 at a small fraction of its FP32 rate); warps combine them the same way and the
// sums across warps and blocks are FP64. Every step is an explicitly rounded operation, so the sums do not depend on
// compiler contraction.
__device__ __forceinline__ void df_add(float& hi, float& lo, float a) {
  const float s = __fadd_rn(hi, a), bp = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(a, bp));
  hi = s; lo = __fadd_rn(lo, e);
}
// (hi, lo) += (whi + wlo) x, the product's rounding error included.
__device__ __forceinline__ void df_add_prod(float& hi, float& lo, float whi, float wlo, float x) {
  const float p = __fmul_rn(whi, x);
  const float pe = __fmaf_rn(wlo, x, __fmaf_rn(whi, x, -p));
  df_add(hi, lo, p);
  lo = __fadd_rn(lo, pe);
}
__device__ __forceinline__ void df_norm(float& hi, float& lo) {
  const float s = __fadd_rn(hi, lo);
  lo = __fsub_rn(lo, __fsub_rn(s, hi)); hi = s;
}
// Block sums of `count` compensated sums per thread into out[] (FP64, a fixed order). Within a warp the sums are
// reduced by halving exchanges: partner lanes swap halves of their (zero-padded) value lists and each keeps the sum of
// one half, so after log2(P) exchanges lane v * 32 / P holds value v; the offsets left over add the one value per lane
// as a plain butterfly. Then the warps' sums are added in warp order.
template <int COUNT>
__device__ void blockSumsDF(float (&hi)[COUNT], float (&lo)[COUNT], double* out, double* sh /* >= 32*COUNT */) {
  static_assert(COUNT >= 1 && COUNT <= 32, "at most 32 sums");
  constexpr int P = COUNT <= 1 ? 1 : COUNT <= 2 ? 2 : COUNT <= 4 ? 4 : COUNT <= 8 ? 8 : COUNT <= 16 ? 16 : 32;
  constexpr int LOGP = P == 1 ? 0 : P == 2 ? 1 : P == 4 ? 2 : P == 8 ? 3 : P == 16 ? 4 : 5;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  float h[P], l[P];
#pragma unroll
  for (int i = 0; i < P; i++) {
    h[i] = i < COUNT ? hi[i] : 0.f; l[i] = i < COUNT ? lo[i] : 0.f;
    df_norm(h[i], l[i]);
  }
#pragma unroll
  for (int j = 0; j < LOGP; j++) {
    const int m = P >> j, o = 16 >> j;
    const bool up = lane & o;
#pragma unroll
    for (int i = 0; i < m / 2; i++) {
      const float sendH = up ? h[i] : h[i + m / 2], sendL = up ? l[i] : l[i + m / 2];
      float kh = up ? h[i + m / 2] : h[i], kl = up ? l[i + m / 2] : l[i];
      const float rh = __shfl_xor_sync(0xffffffffu, sendH, o), rl = __shfl_xor_sync(0xffffffffu, sendL, o);
      df_add(kh, kl, rh);
      kl = __fadd_rn(kl, rl);
      df_norm(kh, kl);
      h[i] = kh; l[i] = kl;
    }
  }
#pragma unroll
  for (int o = 16 >> LOGP; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(0xffffffffu, h[0], o), l2 = __shfl_xor_sync(0xffffffffu, l[0], o);
    df_add(h[0], l[0], h2);
    l[0] = __fadd_rn(l[0], l2);
    df_norm(h[0], l[0]);
  }
  __syncthreads();
  if ((lane & (32 / P - 1)) == 0 && lane / (32 / P) < COUNT) sh[warp * COUNT + lane / (32 / P)] = (double)h[0] + (double)l[0];
  __syncthreads();
  if (threadIdx.x < COUNT) {
    double s = 0;
    for (int w = 0; w < nw; w++) s += sh[w * COUNT + threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

// ==================================================================== conversion at the ABI boundary
// theta' = theta - theta_b(z) (FP64 difference) and back.
__global__ void k_theta_in(const RunDesc* __restrict__ runs, const int4* items, int nitems, const float* src) {
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    int i0 = items[it].y * CHUNK, i1 = min(R.n, i0 + CHUNK);
    float* th = field(R, 0, THETA);
    const float* s = src ? src : field(R, 1, THETA);  // null: each run's own staging slot (set B)
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) th[i] = (float)((double)s[i] - R.lv64[D_THB * R.nz + i / R.layer]);
  }
}
__global__ void k_theta_out(const RunDesc* __restrict__ runs, const int4* items, int nitems, float* dst) {
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    int i0 = items[it].y * CHUNK, i1 = min(R.n, i0 + CHUNK);
    const float* th = field(R, 0, THETA);
    float* d = dst ? dst : field(R, 1, THETA);
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) d[i] = (float)((double)th[i] + R.lv64[D_THB * R.nz + i / R.layer]);
  }
}

// ==================================================================== beginStep
// Fall speeds of the four falling fields and the largest Courant number dt Vt / h of each over its non-zero nodes
// (fallParts, src/core/model.ts:575-580): the sedimentation's sub-step count.
__global__ void k_fall_courant(const RunDesc* __restrict__ runs, const int4* items, int nitems) {
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    int i0 = items[it].y * CHUNK, i1 = min(R.n, i0 + CHUNK);
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    const float *rain = field(R, 0, RAIN), *snow = field(R, 0, SNOW), *graupel = field(R, 0, GRAUPEL), *hail = field(R, 0, HAIL);
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      int z = i / R.layer;
      float rho = lvl(R, L_RHO, z), fsq = lvl(R, L_FALLSQ, z), k = R.dt * lvl(R, L_INV_HZ, z);
      float a = rain[i], b = snow[i], g = graupel[i], h = hail[i];
      if (a != 0.f) c[0] = fmaxf(c[0], k * phys::rainFall(a, rho, fsq));
      if (b != 0.f) c[1] = fmaxf(c[1], k * phys::snowFall(b, rho, fsq));
      if (g != 0.f) c[2] = fmaxf(c[2], k * phys::graupelFall(g, rho));
      if (h != 0.f) c[3] = fmaxf(c[3], k * phys::hailFall(h, rho));
    }
    for (int f = 0; f < 4; f++) {
      float m = warpMax(c[f]);
      if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMaxPos(R.scr + S_COURANT + f, m);
    }
    if (R.flags & RF_EXTRA) {
      // the charge carriers' fall speeds (:1230-1234) from the step-start water, with rain's and snow's own (the
      // charge on rain falls with it; the charging reads the snow's), and the charges' Courant numbers; two-moment
      // rain's mass-, number- and reflectivity-weighted speeds from both moments (:1224) and its Courant number (:973);
      // two-moment graupel's and hail's from their moments and density (:1226-1229), which the graupel-hail carrier
      // falls with too
      const size_t n = R.n;
      const bool elec = R.flags & RF_ELEC, two = R.flags & RF_RAIN2M, ice2 = R.flags & RF_ICE2M;
      const float *ice = field(R, 0, ICE), *num = field(R, 0, RAIN_NUMBER);
      const float *cI = field(R, 0, CHARGE_ICE), *cG = field(R, 0, CHARGE_GRAUPEL), *cR = field(R, 0, CHARGE_RAIN);
      const float *gn = field(R, 0, GRAUPEL_NUMBER), *gv = field(R, 0, GRAUPEL_VOLUME), *hn = field(R, 0, HAIL_NUMBER), *hv = field(R, 0, HAIL_VOLUME);
      float cc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const int z = i / R.layer;
        const float rho = lvl(R, L_RHO, z), fsq = lvl(R, L_FALLSQ, z), k = R.dt * lvl(R, L_INV_HZ, z);
        const float a = rain[i], b = snow[i], g = graupel[i], h = hail[i], ic = ice[i];
        float vr, vn = 0.f, vz = 0.f;
        if (two) r2m::fallSpeeds(a, num[i], rho, vr, vn, vz); else vr = phys::rainFall(a, rho, fsq);
        const float vs = phys::snowFall(b, rho, fsq);
        float vg, vh;
        if (ice2) {
          float vgn, vgz, vhn, vhz;
          i2m::momentSpeeds(i2m::GRAUPEL_2M(), g, gn[i], gv[i], rho, vg, vgn, vgz);
          i2m::momentSpeeds(i2m::HAIL_2M(), h, hn[i], hv[i], rho, vh, vhn, vhz);
          R.vfall[V_GRAUPEL * n + i] = vg; R.vfall[V_GRAUPEL_N * n + i] = vgn; R.vfall[V_GRAUPEL_Z * n + i] = vgz;
          R.vfall[V_HAIL * n + i] = vh; R.vfall[V_HAIL_N * n + i] = vhn; R.vfall[V_HAIL_Z * n + i] = vhz;
          cc[4] = fmaxf(cc[4], k * fmaxf(vgz, vg)); cc[5] = fmaxf(cc[5], k * fmaxf(vhz, vh));
        } else { vg = phys::graupelFall(g, rho); vh = phys::hailFall(h, rho); }
        const float is = ic + b, gh = g + h;
        const float vi = is > 0.f ? b * vs / is : 0.f, vgh = gh > 0.f ? (g * vg + h * vh) / gh : 0.f;
        R.vfall[V_CHG_ICE * n + i] = vi; R.vfall[V_CHG_GRAUPEL * n + i] = vgh; R.vfall[V_RAIN * n + i] = vr; R.vfall[V_SNOW * n + i] = vs;
        if (two) { R.vfall[V_RAIN_N * n + i] = vn; R.vfall[V_RAIN_Z * n + i] = vz; cc[3] = fmaxf(cc[3], k * fmaxf(vz, vr)); }
        if (elec) {
          if (cI[i] != 0.f) cc[0] = fmaxf(cc[0], k * vi);
          if (cG[i] != 0.f) cc[1] = fmaxf(cc[1], k * vgh);
          if (cR[i] != 0.f) cc[2] = fmaxf(cc[2], k * vr);
        }
      }
      for (int f = 0; f < 6; f++) {
        float m = warpMax(cc[f]);
        if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMaxPos(R.scr + (f < 3 ? S_CCOURANT + f : f == 3 ? S_R2M : f == 4 ? S_G2M : S_H2M), m);
      }
    }
  }
}

// One thread per column: the hail swath (collectHail, :697-706), then for rain, snow, graupel and hail the upwind
// flux-form fall in ceil(courant / 0.8) sub-steps (sediment/sedimentPart, :565-598), bottom-up so each face uses the
// values above from before the sub-step, the ground flux into the rain gauge. Fall speeds are those of the step's
// start. Columns stay in shared memory; a column of zeros stays zero and is left alone.
constexpr int SED_COLS = 64;
__global__ void k_sediment(const RunDesc* __restrict__ runs, const int4* items, int nitems) {
  extern __shared__ float sm[];
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    const int nz = R.nz, layer = R.layer, t = threadIdx.x;
    float* sq = sm;                     // [nz][SED_COLS]
    float* sv = sq + nz * SED_COLS;     // [nz][SED_COLS]
    float* lrho = sv + nz * SED_COLS;   // [nz] rho0, 1/(rho0 h), fall-speed density factor
    float* lk = lrho + nz;
    float* lfs = lk + nz;
    for (int z = t; z < nz; z += blockDim.x) {
      lrho[z] = lvl(R, L_RHO, z); lk[z] = lvl(R, L_INV_RHO, z) * lvl(R, L_INV_HZ, z); lfs[z] = lvl(R, L_FALLSQ, z);
    }
    __syncthreads();
    const int c = items[it].y * SED_COLS + t;
    const bool on = t < SED_COLS && c < layer;
    const float rho0 = R.rho0;
    float* precip = R.cols;
    float* hailGround = R.cols + layer;
    float* hailSize = R.cols + 2 * layer;
    // sedimented(): two-moment rain, graupel and hail fall on their own (:907-911)
    const int fEnd = (R.flags & RF_ICE2M) ? GRAUPEL : 4;
    for (int f = (R.flags & RF_RAIN2M) ? 1 : 0; f < fEnd; f++) {
      float* a = field(R, 0, f);
      const float courant = R.scr[S_COURANT + f];
      const int parts = max(1, (int)ceilf(courant / .8f));
      if (!on) continue;
      bool any = false;
#pragma unroll 8
      for (int z = 0; z < nz; z++) {
        const float q = a[c + z * layer];
        sq[z * SED_COLS + t] = q;
        any |= q != 0.f;
      }
      if (!any) continue;
      for (int z = 0; z < nz; z++) {
        const float q = sq[z * SED_COLS + t], rho = lrho[z], fsq = lfs[z];
        sv[z * SED_COLS + t] = f == 0 ? phys::rainFall(q, rho, fsq) : f == 1 ? phys::snowFall(q, rho, fsq) : f == 2 ? phys::graupelFall(q, rho) : phys::hailFall(q, rho);
      }
      if (f == HAIL && (R.flags & RF_ICE)) {
        const float h = sq[t];
        if (h > 1e-9f) {
          hailGround[c] += rho0 * h * sv[t] * R.dt;
          hailSize[c] = fmaxf(hailSize[c], phys::hailMaxDiameter(h, rho0) * 1000.f);
        }
      }
      if (f == RAIN || (R.flags & RF_ICE)) {
        const float dts = R.dt / (float)parts;
        for (int p = 0; p < parts; p++) {
          precip[c] += rho0 * sq[t] * sv[t] * dts;
          float inflowAbove = 0.f;  // the flux into level z from above, from the values before this sub-step
          for (int z = nz - 1; z >= 0; z--) {
            const float q = sq[z * SED_COLS + t], out = lrho[z] * q * sv[z * SED_COLS + t];
            sq[z * SED_COLS + t] = q + dts * (inflowAbove - out) * lk[z];
            inflowAbove = out;
          }
        }
        for (int z = 0; z < nz; z++) a[c + z * layer] = sq[z * SED_COLS + t];
      }
    }
    if (R.flags & RF_ELEC) {
      // The charge on the falling carriers (sediment(field, vt, dt, false), :931, :582-598) with the carriers' step-start
      // fall speeds: what falls through the ground is the ground's charge, C (:588-591), summed per work item.
      __shared__ double gsum[SED_COLS];
      double ground = 0;
      const float dxy = R.dx * R.dy;
      for (int j = 0; j < 3; j++) {
        float* a = field(R, 0, CHARGE_ICE + j);
        const float* vt = R.vfall + (size_t)(j == 2 ? V_RAIN : j) * R.n;
        const int parts = max(1, (int)ceilf(R.scr[S_CCOURANT + j] / .8f));
        if (!on) continue;
        bool any = false;
        for (int z = 0; z < nz; z++) {
          const float q = a[c + z * layer];
          sq[z * SED_COLS + t] = q; sv[z * SED_COLS + t] = vt[c + z * layer];
          any |= q != 0.f;
        }
        if (!any) continue;
        const float dts = R.dt / (float)parts;
        for (int p = 0; p < parts; p++) {
          ground += (double)rho0 * (double)(sq[t] * sv[t]) * (double)dts * (double)dxy;
          float inflowAbove = 0.f;
          for (int z = nz - 1; z >= 0; z--) {
            const float q = sq[z * SED_COLS + t], out = lrho[z] * q * sv[z * SED_COLS + t];
            sq[z * SED_COLS + t] = q + dts * (inflowAbove - out) * lk[z];
            inflowAbove = out;
          }
        }
        for (int z = 0; z < nz; z++) a[c + z * layer] = sq[z * SED_COLS + t];
      }
      gsum[t] = ground;
      __syncthreads();
      if (t == 0) {
        double s = 0;
        for (int k = 0; k < SED_COLS; k++) s += gsum[k];
        R.cpart[items[it].y] = s;
      }
    }
    __syncthreads();  // the level tables are restaged for the block's next item
  }
}

// Two-moment fall (sedimentRain2m / sedimentIce2m / sediment2m, :898-988; NSSL sediment1d, infall 4) for two-moment
// rain and then two-moment graupel and hail: the mass with its mass-weighted speed, the number with its number-weighted
// one, an ice class's particle volume with the mass, a reflectivity and a number carried at the mass's speed beside
// them; every sub-step the number is kept between what those two imply. A warp a column, level z in lane z % 32 (slot
// z / 32, K slots), every value in registers: a level's update reads only its own and the level above's values from
// before the sub-step (the reference's bottom-up loop), so the level above's out-fluxes come by one warp shuffle. The
// ground flux into the rain gauge (lane 0, level 0, in sub-step order). Sub-steps by the faster of the reflectivity's
// and the mass's speed over the run. Before two-moment hail falls, the hail reaching the ground and its largest stones
// (collectHail, :697-711, with the two-moment speed and tail).
constexpr int SED2_WARPS = 8;
template <int K>
__global__ void __launch_bounds__(SED2_WARPS * 32) k_sediment_2m(const RunDesc* __restrict__ runs, const int4* items, int nitems) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr unsigned FULL = 0xffffffffu;
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED] || !(R.flags & RF_RAIN2M)) continue;
    const int nz = R.nz, layer = R.layer;
    const size_t n = R.n;
    const int classes = (R.flags & RF_ICE2M) ? 3 : 1;
    float rho[K], lk[K], lh[K];
#pragma unroll
    for (int j = 0; j < K; j++) {
      const int z = lane + 32 * j;
      rho[j] = z < nz ? lvl(R, L_RHO, z) : 0.f;
      lk[j] = z < nz ? lvl(R, L_INV_RHO, z) * lvl(R, L_INV_HZ, z) : 0.f;
      lh[j] = z < nz ? lvl(R, L_INV_HZ, z) : 0.f;
    }
    for (int cc = wid; cc < SED_COLS; cc += SED2_WARPS) {
      const int c = items[it].y * SED_COLS + cc;
      if (c >= layer) break;
      for (int k = 0; k < classes; k++) {
        // class k: rain (the drops' density, reflectivity factor G1), graupel, hail (their own density, bounded to
        // 170-900 kg/m3 for the reflectivity, :920, and factor)
        const bool ice = k > 0;
        const i2m::IceClass cl = k == 1 ? i2m::GRAUPEL_2M() : i2m::HAIL_2M();
        float* Q = field(R, 0, k == 0 ? RAIN : k == 1 ? GRAUPEL : HAIL);
        float* N = field(R, 0, k == 0 ? RAIN_NUMBER : k == 1 ? GRAUPEL_NUMBER : HAIL_NUMBER);
        float* V = ice ? field(R, 0, k == 1 ? GRAUPEL_VOLUME : HAIL_VOLUME) : nullptr;
        const float* FM = R.vfall + (size_t)(k == 0 ? V_RAIN : k == 1 ? V_GRAUPEL : V_HAIL) * n;
        const float* FN = R.vfall + (size_t)(k == 0 ? V_RAIN_N : k == 1 ? V_GRAUPEL_N : V_HAIL_N) * n;
        const float* FZ = R.vfall + (size_t)(k == 0 ? V_RAIN_Z : k == 1 ? V_GRAUPEL_Z : V_HAIL_Z) * n;
        const float g1 = ice ? cl.g1 : r2m::G1;
        auto k6 = [&](float qq, float vv) {
          if (!ice) return r2m::K6;
          const float d = 6.f / (phys::PI * fminf(900.f, fmaxf(170.f, i2m::densityOf(cl, qq, vv))));
          return d * d;
        };
        if (k == 2 && lane == 0) {
          const float h = Q[c];
          if (h > 1e-9f) {
            R.cols[layer + c] += R.rho0 * h * FM[c] * R.dt;
            R.cols[2 * layer + c] = fmaxf(R.cols[2 * layer + c], i2m::largestDiameter(i2m::HAIL_2M(), h, N[c], V[c], R.rho0) * 1000.f);
          }
        }
        float q[K], num[K], vol[K], vm[K], vn[K], vz[K];
        bool any = false;
#pragma unroll
        for (int j = 0; j < K; j++) {
          const int z = lane + 32 * j, i = c + z * layer;
          const bool in = z < nz;
          q[j] = in ? Q[i] : 0.f; num[j] = in ? N[i] : 0.f; vol[j] = in && ice ? V[i] : 0.f;
          vm[j] = in ? FM[i] : 0.f; vn[j] = in ? FN[i] : 0.f; vz[j] = in ? FZ[i] : 0.f;
          any |= q[j] != 0.f || num[j] != 0.f || vol[j] != 0.f;
        }
        if (!__any_sync(FULL, any)) continue;
        const int parts = max(1, (int)ceilf(R.scr[k == 0 ? S_R2M : k == 1 ? S_G2M : S_H2M] / .8f));
        const float step = R.dt / (float)parts;
        for (int p = 0; p < parts; p++) {
          float refl[K], carried[K];
#pragma unroll
          for (int j = 0; j < K; j++) {
            const float rq = rho[j] * q[j], rn = rho[j] * num[j];
            refl[j] = rq > 0.f && rn > 0.f ? g1 * k6(q[j], vol[j]) * rq * rq / rn : 0.f;
            carried[j] = num[j];
          }
          if (lane == 0) R.cols[c] += R.rho0 * q[0] * vm[0] * step;
          // each level's out-fluxes from before the sub-step; the level above's into this one (none past the top)
          float oq[K], on[K], oc[K], orr[K], ov[K];
#pragma unroll
          for (int j = 0; j < K; j++) {
            oq[j] = rho[j] * q[j] * vm[j]; on[j] = rho[j] * num[j] * vn[j]; oc[j] = rho[j] * carried[j] * vm[j];
            orr[j] = refl[j] * vz[j]; ov[j] = rho[j] * vol[j] * vm[j];
          }
          auto above = [&](const float (&o)[K], int j) {
            const float next = __shfl_down_sync(FULL, o[j], 1);
            const float wrap = __shfl_sync(FULL, j + 1 < K ? o[j + 1 < K ? j + 1 : j] : 0.f, 0);
            return lane < 31 ? next : (j + 1 < K ? wrap : 0.f);
          };
#pragma unroll
          for (int j = 0; j < K; j++) {
            const float iq = above(oq, j), in_ = above(on, j), ic = above(oc, j), ir = above(orr, j), iv = above(ov, j);
            q[j] += step * (iq - oq[j]) * lk[j];
            vol[j] += step * (iv - ov[j]) * lk[j];
            num[j] += step * (in_ - on[j]) * lk[j];
            carried[j] += step * (ic - oc[j]) * lk[j];
            refl[j] += step * (ir - orr[j]) * lh[j];
          }
#pragma unroll
          for (int j = 0; j < K; j++) {
            if (!(q[j] > r2m::RAIN_MIN)) { if (q[j] < 0.f) q[j] = 0.f; num[j] = 0.f; vol[j] = 0.f; continue; }
            const float rq = rho[j] * q[j];
            num[j] = refl[j] > 0.f ? fmaxf(fminf(g1 * k6(q[j], vol[j]) * rq * rq / refl[j] / rho[j], carried[j]), num[j]) : fmaxf(carried[j], num[j]);
          }
        }
#pragma unroll
        for (int j = 0; j < K; j++) {
          const int z = lane + 32 * j, i = c + z * layer;
          if (z < nz) { Q[i] = q[j]; N[i] = num[j]; if (ice) V[i] = vol[j]; }
        }
      }
    }
  }
}

// ==================================================================== elliptic solves
// Exact row index of element e of a row-major block with rows of length `len` (e < 2^20, len <= 640; checked
// exhaustively for the grid widths in use): one multiply by the reciprocal instead of an integer division.
__device__ __forceinline__ int row_of(int e, float inv_len) { return __float2int_rz(((float)e + .5f) * inv_len); }

// Divergence rows of one layer and their forward x-transform (real rows paired into complex ones, the reference's
// trick, src/core/spectral.ts:246-255), written m-major: spec[(m * nzc + k) * ny + y].
//  FACE: node divergence of the unprojected face mass fluxes rho0 * mean(u) (src/core/advection.ts:190-211).
//  PRES: dual-cell divergence of rho0 u from the 8 corner nodes, over dt (src/core/pressure.ts:50-66).
__global__ void k_proj_div_xfft(const RunDesc* __restrict__ runs, const int4* items, int nitems, int mode, int set, int yc) {
  extern __shared__ float2 smc[];
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    const int k = items[it].y, y0 = items[it].z, nx = R.nx, ny = R.ny, layer = R.layer, nz = R.nz;
    const int rows = min(yc, ny - y0), pairs = (rows + 1) / 2, nzc = mode == PROJ_FACE ? nz : nz - 1;
    const float inv_nx = 1.f / (float)nx;
    float2* Z = smc;                   // [pairs][nx]
    float2* T = smc + pairs * nx;      // scratch
    const float *u = field(R, set, U), *v = field(R, set, V), *w = field(R, set, W);
    const float idx = R.inv_dx, idy = R.inv_dy;
    if (mode == PROJ_FACE) {
      const float rho = lvl(R, L_RHO, k), ihz = lvl(R, L_INV_HZ, k);
      const float rup = k < nz - 1 ? .5f * lvl(R, L_RUP, k) : 0.f, rdn = k > 0 ? .5f * lvl(R, L_RUP, k - 1) : 0.f;
      const int l = k * layer, lu = k < nz - 1 ? l + layer : l, ld = k > 0 ? l - layer : l;
#pragma unroll 4
      for (int e = threadIdx.x; e < pairs * 2 * nx; e += blockDim.x) {
        const int r = row_of(e, inv_nx), x = e - r * nx, y = y0 + r;
        float d = 0.f;
        if (r < rows) {
          const int c = x + y * nx;
          const int ce = (x + 1 == nx ? 0 : x + 1) + y * nx, cw = (x == 0 ? nx - 1 : x - 1) + y * nx;
          const int cn = x + (y + 1 == ny ? 0 : y + 1) * nx, cs = x + (y == 0 ? ny - 1 : y - 1) * nx;
          const float ddx = .5f * rho * (u[ce + l] - u[cw + l]);
          const float ddy = .5f * rho * (v[cn + l] - v[cs + l]);
          const float wc = w[c + l];
          const float up = rup * (wc + w[c + lu]), dn = rdn * (w[c + ld] + wc);
          d = ddx * idx + ddy * idy + (up - dn) * ihz;
        }
        reinterpret_cast<float*>(&Z[(r >> 1) * nx + x])[r & 1] = d;
      }
    } else if (mode == PROJ_GIVEN) {
      const float* rhs = R.phi + (size_t)k * layer;
      for (int e = threadIdx.x; e < pairs * 2 * nx; e += blockDim.x) {
        const int r = row_of(e, inv_nx), x = e - r * nx, y = y0 + r;
        reinterpret_cast<float*>(&Z[(r >> 1) * nx + x])[r & 1] = r < rows ? rhs[x + y * nx] : 0.f;
      }
    } else {
      const float r0 = .25f * lvl(R, L_RHO, k), r1 = .25f * lvl(R, L_RHO, k + 1), idz = lvl(R, L_INV_DZS, k), idt = 1.f / R.dt;
      const int l0 = k * layer, l1 = l0 + layer;
#pragma unroll 4
      for (int e = threadIdx.x; e < pairs * 2 * nx; e += blockDim.x) {
        const int r = row_of(e, inv_nx), x = e - r * nx, y = y0 + r;
        float d = 0.f;
        if (r < rows) {
          const int x1 = x + 1 == nx ? 0 : x + 1, y1 = (y + 1 == ny ? 0 : y + 1) * nx, yy = y * nx;
          const int a = x + yy, b = x1 + yy, ee = x + y1, f = x1 + y1;
          const float ddx = (r0 * ((u[b + l0] - u[a + l0]) + (u[f + l0] - u[ee + l0])) + r1 * ((u[b + l1] - u[a + l1]) + (u[f + l1] - u[ee + l1]))) * idx;
          const float ddy = (r0 * ((v[ee + l0] - v[a + l0]) + (v[f + l0] - v[b + l0])) + r1 * ((v[ee + l1] - v[a + l1]) + (v[f + l1] - v[b + l1]))) * idy;
          const float ddz = (r1 * ((w[a + l1] + w[b + l1]) + (w[ee + l1] + w[f + l1])) - r0 * ((w[a + l0] + w[b + l0]) + (w[ee + l0] + w[f + l0]))) * idz;
          d = (ddx + ddy + ddz) * idt;
        }
        reinterpret_cast<float*>(&Z[(r >> 1) * nx + x])[r & 1] = d;
      }
    }
    __syncthreads();
    FftPlan P{nx, R.fx_nf, R.fx_rad, R.twx};
    const float2* Zf = fft_rows_any(Z, T, nx, pairs, P);
    const int nm = R.nm;
    const float inv_rows = 1.f / (float)rows;
    for (int e = threadIdx.x; e < nm * rows; e += blockDim.x) {
      const int m = row_of(e, inv_rows), r = e - m * rows, pr = r >> 1, c = m ? nx - m : 0;
      const float2 zm = Zf[pr * nx + m], zc = Zf[pr * nx + c];
      float2 out;
      if ((r & 1) == 0) out = make_float2(.5f * (zm.x + zc.x), .5f * (zm.y - zc.y));
      else out = make_float2(.5f * (zm.y + zc.y), .5f * (zc.x - zm.x));
      R.spec[((size_t)m * nzc + k) * ny + y0 + r] = out;
    }
    __syncthreads();
  }
}

// One x-wavenumber m per item: the y-transform of every layer, one tridiagonal solve per y-wavenumber n along the
// vertical in FP64, the inverse y-transform. The solve is Thomas' algorithm with the LU factors made on the host in
// FP64 (the k = 0 uniform mode pinned at the ground, the null modes zero): per level the forward sweep
// d_k = A_k r_k - B_k d_(k-1) and the back substitution x_k = d_k - C_k x_(k+1), one real recurrence per
// (n, real/imaginary part), the two parts sharing the coefficients. FACE: rows -rho h lambda + vertical faces
// (src/core/advection.ts:222-241); PRES: the density-weighted consistent Laplacian (src/core/pressure.ts:104-140).
// The inverse transform is the forward one of the conjugate, conjugated: the back substitution stores conj(x).
// Transform of `rows` rows at S (stride n) with a scratch of `cap` rows; the result ends in S.
__device__ void fft_rows_grouped(float2* S, float2* T, int n, int rows, int cap, const FftPlan& P) {
  for (int k0 = 0; k0 < rows; k0 += cap) {
    const int g = min(cap, rows - k0);
    float2* r = fft_rows_any(S + k0 * n, T, n, g, P);
    if (r != S + k0 * n) {
      for (int e = threadIdx.x; e < g * n; e += blockDim.x) S[k0 * n + e] = r[e];
      __syncthreads();
    }
  }
}

// `group`: layers the scratch holds (all of them: the transforms ping-pong between the two buffers; fewer, for tall
// or wide grids: the layers go through the scratch in groups).
__global__ void k_proj_modes(const RunDesc* __restrict__ runs, const int4* items, int nitems, int mode, int group) {
  extern __shared__ float2 smc[];
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    const int m = items[it].y, ny = R.ny, nz = R.nz, nzc = mode == PROJ_FACE ? nz : nz - 1;
    const bool whole = group >= nzc;
    float2* S = smc;                   // [nzc][ny]
    float2* T = smc + nzc * ny;        // [group][ny] scratch
    float2* g = R.spec + (size_t)m * nzc * ny;
    for (int e = threadIdx.x; e < nzc * ny; e += blockDim.x) S[e] = g[e];
    __syncthreads();
    FftPlan P{ny, R.fy_nf, R.fy_rad, R.twy};
    float2* F = S;
    if (whole) F = fft_rows_any(S, T, ny, nzc, P);
    else fft_rows_grouped(S, T, ny, nzc, group, P);
    float2* Fo = F == S ? T : S;       // the other buffer (whole slab case)
    const TriAB* AB = (mode == PROJ_FACE ? R.tri_face : R.tri_pres) + (size_t)m * nzc * ny;
    const double* Cc = reinterpret_cast<const double*>((mode == PROJ_FACE ? R.tri_face : R.tri_pres) + (size_t)R.nm * nzc * ny) + (size_t)m * nzc * ny;
    // one FP64 recurrence per (n, real/imaginary part); values enter and leave FP64 through the integer-pipe
    // conversions
    float* Ff = reinterpret_cast<float*>(F);
    for (int u = threadIdx.x; u < 2 * ny; u += blockDim.x) {
      const int n = u >> 1, c = u & 1;
      double d[MAXNZ];
      double prev = 0;
#pragma unroll 4
      for (int k = 0; k < nzc; k++) {
        const TriAB ab = AB[(size_t)k * ny + n];
        prev = fma(-ab.b, prev, widen(__fmul_rn(ab.a, Ff[2 * (k * ny + n) + c])));
        d[k] = prev;
      }
      double x = d[nzc - 1];
      Ff[2 * ((nzc - 1) * ny + n) + c] = c ? -narrow(x) : narrow(x);
#pragma unroll 4
      for (int k = nzc - 2; k >= 0; k--) {
        x = fma(-Cc[(size_t)k * ny + n], x, d[k]);
        Ff[2 * (k * ny + n) + c] = c ? -narrow(x) : narrow(x);
      }
    }
    __syncthreads();
    const float2* G = F;
    if (whole) G = fft_rows_any(F, Fo, ny, nzc, P);
    else fft_rows_grouped(S, T, ny, nzc, group, P);
    for (int e = threadIdx.x; e < nzc * ny; e += blockDim.x) { const float2 z = G[e]; g[e] = make_float2(z.x, -z.y); }
    __syncthreads();
  }
}

// Inverse x-transform of one layer's rows (Hermitian rows rebuilt from the half spectrum, two real rows per complex
// transform, src/core/spectral.ts:281-290; the inverse as the conjugate of the forward transform of the conjugate),
// normalised by nx*ny, into phi (FACE) or the pressure (PRES).
__global__ void k_proj_xifft(const RunDesc* __restrict__ runs, const int4* items, int nitems, int mode, int yc) {
  extern __shared__ float2 smc[];
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    const int k = items[it].y, y0 = items[it].z, nx = R.nx, ny = R.ny, nz = R.nz, mh = R.mh, nm = R.nm;
    const int rows = min(yc, ny - y0), pairs = (rows + 1) / 2, nzc = mode == PROJ_FACE ? nz : nz - 1;
    float2* H = smc;                    // [rows][nm] half spectra
    float2* Z = smc + yc * nm;          // [pairs][nx]
    float2* T = Z + pairs * nx;
    const float inv_rows = 1.f / (float)rows, inv_nx = 1.f / (float)nx;
#pragma unroll 4
    for (int e = threadIdx.x; e < nm * rows; e += blockDim.x) {
      const int m = row_of(e, inv_rows), r = e - m * rows;
      H[r * nm + m] = R.spec[((size_t)m * nzc + k) * ny + y0 + r];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < pairs * nx; e += blockDim.x) {
      const int pr = row_of(e, inv_nx), m = e - pr * nx, c = m <= mh ? m : nx - m;
      const float sg = m <= mh ? 1.f : -1.f;
      const bool real = c == 0 || 2 * c == nx, pair = 2 * pr + 1 < rows;
      const float2 A = H[(2 * pr) * nm + c];
      const float ar = A.x, ai = real ? 0.f : sg * A.y;
      float br = 0.f, bi = 0.f;
      if (pair) { const float2 B = H[(2 * pr + 1) * nm + c]; br = B.x; bi = real ? 0.f : sg * B.y; }
      Z[pr * nx + m] = make_float2(ar - bi, -(ai + br));  // conj(A + iB)
    }
    __syncthreads();
    FftPlan P{nx, R.fx_nf, R.fx_rad, R.twx};
    const float2* Zf = fft_rows_any(Z, T, nx, pairs, P);
    const float norm = 1.f / (float)(nx * ny);
    float* out = (mode == PROJ_FACE ? R.phi : mode == PROJ_GIVEN ? R.pres2 : R.pres) + (size_t)k * nx * ny;
    for (int e = threadIdx.x; e < rows * nx; e += blockDim.x) {
      const int r = row_of(e, inv_nx), x = e - r * nx;
      const float2 z = Zf[(r >> 1) * nx + x];
      out[(y0 + r) * nx + x] = ((r & 1) ? -z.y : z.x) * norm;
    }
    __syncthreads();
  }
}


// ---- the whole-layer path (grids whose layer spectrum fits in shared memory: the benchmark's 40x32 and 80x64):
// the divergence kernel transforms each layer along x and y, the mode kernel is a pure FP64 sweep without
// transforms or barriers, and the inverse kernel transforms back along y and x.

// Builds the half spectrum X[m][y] (m <= nx/2) of the real rows held in pairs in Zf (spectral.ts:246-255).
__device__ __forceinline__ void unpack_rows(const float2* Zf, float2* X, int nx, int ny, int rows, int nm) {
  for (int e = threadIdx.x; e < nm * rows; e += blockDim.x) {
    const int m = e / rows, r = e - m * rows, pr = r >> 1, c = m ? nx - m : 0;
    const float2 zm = Zf[pr * nx + m], zc = Zf[pr * nx + c];
    X[m * ny + r] = (r & 1) == 0 ? make_float2(.5f * (zm.x + zc.x), .5f * (zm.y - zc.y))
                                 : make_float2(.5f * (zm.y + zc.y), .5f * (zc.x - zm.x));
  }
  __syncthreads();
}

// The layer transforms done by warps (sg_fft.cuh): 1 for the 40 x 32 grid, 2 for 80 x 64, 0 the block-wide stages.
__device__ __forceinline__ int layer_fast(int nx, int ny) { return nx == 40 && ny == 32 ? 1 : nx == 80 && ny == 64 ? 2 : 0; }

// The source of one layer's forward transform on a grid of NX * NY = 256 * PER nodes (the 40 x 32 grid), by a block of
// 256 threads: the level planes it needs are read once, coalesced, and combined per node into three staged planes P
// (FACE: u, v and the vertical flux difference; PRES: u, v and w weighted by the levels' densities), then each node's
// divergence takes its horizontal neighbours from P; into the pair rows of Z (row stride NX + 1). The same
// divergences as the block-wide path, summed in another order. Ends with the block synchronised.
template <int NX, int NY>
__device__ __forceinline__ void layer_source_staged(const RunDesc& R, int mode, int set, int k, float2* Z, float* P) {
  constexpr int N = NX * NY, PER = N / 256, ZS = NX + 1;
  static_assert(PER * 256 == N, "a whole number of nodes a thread");
  const int t = threadIdx.x, nz = R.nz;
  float* Zf = reinterpret_cast<float*>(Z);
  auto put = [&](int e, float d) { const int r = e / NX, x = e - r * NX; Zf[2 * ((r >> 1) * ZS + x) + (r & 1)] = d; };
  if (mode == PROJ_GIVEN) {
    const float* rhs = R.phi + (size_t)k * N;
    float d[PER];
#pragma unroll
    for (int j = 0; j < PER; j++) d[j] = rhs[t + 256 * j];
#pragma unroll
    for (int j = 0; j < PER; j++) put(t + 256 * j, d[j]);
    __syncthreads();
    return;
  }
  const float *u = field(R, set, U), *v = field(R, set, V), *w = field(R, set, W);
  const float idx = R.inv_dx, idy = R.inv_dy;
  if (mode == PROJ_FACE) {
    const float rho = lvl(R, L_RHO, k), ihz = lvl(R, L_INV_HZ, k);
    const float rup = k < nz - 1 ? .5f * lvl(R, L_RUP, k) : 0.f, rdn = k > 0 ? .5f * lvl(R, L_RUP, k - 1) : 0.f;
    const int l = k * N, lu = k < nz - 1 ? l + N : l, ld = k > 0 ? l - N : l;
#pragma unroll
    for (int j = 0; j < PER; j++) {
      const int e = t + 256 * j;
      const float wc = w[l + e];
      P[e] = u[l + e]; P[N + e] = v[l + e];
      P[2 * N + e] = (rup * (wc + w[lu + e]) - rdn * (w[ld + e] + wc)) * ihz;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; j++) {
      const int e = t + 256 * j, y = e / NX, x = e - y * NX, row = y * NX;
      const int ce = (x + 1 == NX ? 0 : x + 1) + row, cw = (x == 0 ? NX - 1 : x - 1) + row;
      const int cn = x + (y + 1 == NY ? 0 : y + 1) * NX, cs = x + (y == 0 ? NY - 1 : y - 1) * NX;
      const float ddx = .5f * rho * (P[ce] - P[cw]), ddy = .5f * rho * (P[N + cn] - P[N + cs]);
      put(e, ddx * idx + ddy * idy + P[2 * N + e]);
    }
  } else {
    const float r0 = .25f * lvl(R, L_RHO, k), r1 = .25f * lvl(R, L_RHO, k + 1), idz = lvl(R, L_INV_DZS, k), idt = 1.f / R.dt;
    const int l0 = k * N, l1 = l0 + N;
#pragma unroll
    for (int j = 0; j < PER; j++) {
      const int e = t + 256 * j;
      P[e] = r0 * u[l0 + e] + r1 * u[l1 + e];
      P[N + e] = r0 * v[l0 + e] + r1 * v[l1 + e];
      P[2 * N + e] = r1 * w[l1 + e] - r0 * w[l0 + e];
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; j++) {
      const int e = t + 256 * j, y = e / NX, x = e - y * NX;
      const int x1 = x + 1 == NX ? 0 : x + 1, y1 = (y + 1 == NY ? 0 : y + 1) * NX, yy = y * NX;
      const int a = x + yy, b = x1 + yy, c = x + y1, f = x1 + y1;
      const float ddx = ((P[b] - P[a]) + (P[f] - P[c])) * idx;
      const float ddy = ((P[N + c] - P[N + a]) + (P[N + f] - P[N + b])) * idy;
      const float ddz = ((P[2 * N + a] + P[2 * N + b]) + (P[2 * N + c] + P[2 * N + f])) * idz;
      put(e, (ddx + ddy + ddz) * idt);
    }
  }
  __syncthreads();
}

// The 2-D forward transform of one layer whose pair rows (real rows 2p and 2p + 1 as one complex row) are in Z (row
// stride NX + 1; the block synchronised): the rows by warps in place, then per x-wavenumber m a warp unpacks the two
// real rows' spectra (from Z[m] and conj Z[NX - m]) for every y and transforms the column, into
// spec[(m * nzc + k) * NY + n].
template <int NX, int NY>
__device__ __forceinline__ void layer_forward_fast(const RunDesc& R, float2* Z, const float2* TW, int k, int nzc) {
  constexpr int PAIRS = NY / 2, NM = NX / 2 + 1, ZS = NX + 1;
  warp_rows_fft<NX, ZS>(Z, PAIRS, TW);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const float2* twy = TW + NX;
  for (int m = warp; m < NM; m += nw) {
    const int c = m ? NX - m : 0;
    float2 x[2];
#pragma unroll
    for (int s = 0; s < NY / 32; s++) {
      const int r = lane + 32 * s;
      const float2 zm = Z[(r >> 1) * ZS + m], zc = Z[(r >> 1) * ZS + c];
      x[s] = (r & 1) == 0 ? make_float2(.5f * (zm.x + zc.x), .5f * (zm.y - zc.y)) : make_float2(.5f * (zm.y + zc.y), .5f * (zc.x - zm.x));
    }
    float2 out[2];
    warp_column_fft<NY>(x[0], x[NY / 32 - 1], twy, lane, out);
    float2* gm = R.spec + ((size_t)m * nzc + k) * NY;
    const int b = bitrev<5>(lane);
    if (NY == 32) gm[b] = out[0];
    else { gm[2 * b] = out[0]; gm[2 * b + 1] = out[1]; }
  }
  __syncthreads();
}

// The 2-D inverse of one layer by warps: per x-wavenumber m a warp transforms the conjugated column
// (G[m][y] = conj of the y-inverse) into X (row stride NY + 1); then each pair row is rebuilt from the Hermitian half
// spectrum, transformed along x, and its conjugate gives the two real rows, normalised, into out.
// A block of 256 threads; the twiddles' staging in TW is synchronised here (after the spectrum's loads are issued).
template <int NX, int NY>
__device__ __forceinline__ void layer_inverse_fast(const RunDesc& R, float2* X, const float2* TW, int k, int nzc, float* out) {
  constexpr int PAIRS = NY / 2, NM = NX / 2 + 1, MH = NX / 2, XS = NY + 1, G = NX / 5, RPW = 32 / G, NW = 8, ROUNDS = (NM + NW - 1) / NW;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = NW;
  const float2* twy = TW + NX;
  float2 sp[ROUNDS][NY / 32];  // every column of this warp, loaded before any is transformed
#pragma unroll
  for (int q = 0; q < ROUNDS; q++) {
    const int m = warp + NW * q;
    const float2* gm = R.spec + ((size_t)(m < NM ? m : 0) * nzc + k) * NY;
#pragma unroll
    for (int s = 0; s < NY / 32; s++) sp[q][s] = gm[lane + 32 * s];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < ROUNDS; q++) {
    const int m = warp + NW * q;
    if (m >= NM) break;
    float2 x[2];
#pragma unroll
    for (int s = 0; s < NY / 32; s++) x[s] = make_float2(sp[q][s].x, -sp[q][s].y);
    float2 o[2];
    warp_column_fft<NY>(x[0], x[NY / 32 - 1], twy, lane, o);
    const int b = bitrev<5>(lane);
    if (NY == 32) X[m * XS + b] = o[0];
    else { X[m * XS + 2 * b] = o[0]; X[m * XS + 2 * b + 1] = o[1]; }
  }
  __syncthreads();
  const int l = lane % G, gi = lane / G;
  const float norm = 1.f / (float)(NX * NY);
  for (int rw = warp; rw * RPW < PAIRS; rw += nw) {
    const int pr = rw * RPW + gi;
    float2 v[5];
#pragma unroll
    for (int q = 0; q < 5; q++) {
      const int j = l + G * q, c = j <= MH ? j : NX - j;
      const float sg = j <= MH ? 1.f : -1.f;
      const bool real = c == 0 || 2 * c == NX;
      const float2 A = X[c * XS + 2 * pr], B = X[c * XS + 2 * pr + 1];
      const float ar = A.x, ai = real ? 0.f : -sg * A.y, br = B.x, bi = real ? 0.f : -sg * B.y;
      v[q] = make_float2(ar - bi, -(ai + br));  // conj(A + iB)
    }
    dft5(v[0], v[1], v[2], v[3], v[4]);
#pragma unroll
    for (int q = 1; q < 5; q++) v[q] = cmul(v[q], TW[l * q]);
#pragma unroll
    for (int q = 0; q < 5; q++) v[q] = lane_dft<G>(v[q], TW, 5, l);
    const int x0 = 5 * bitrev<ilog2(G)>(l);
    float* o0 = out + (size_t)(2 * pr) * NX + x0;
    float* o1 = o0 + NX;
#pragma unroll
    for (int q = 0; q < 5; q++) { o0[q] = v[q].x * norm; o1[q] = -v[q].y * norm; }
  }
  __syncthreads();
}

// Divergence of one layer (FACE or PRES, as k_proj_div_xfft) and its 2-D forward transform, written
// spec[(m * nzc + k) * ny + n].
__global__ void __launch_bounds__(256, 5) k_proj_div_fft2(const RunDesc* __restrict__ runs, const int4* items, int nitems, int mode, int set) {
  extern __shared__ float2 smc[];
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    const int k = items[it].y, nx = R.nx, ny = R.ny, layer = R.layer, nz = R.nz, nm = R.nm;
    const int pairs = (ny + 1) / 2, nzc = mode == PROJ_FACE ? nz : nz - 1;
    const float inv_nx = 1.f / (float)nx;
    const int fast = layer_fast(nx, ny), zs = fast ? nx + 1 : nx;  // Z's row stride (padded for the warp transforms)
    float2* TW = smc;                       // the twiddles of x then y, staged once per layer
    float2* Z = TW + nx + ny;               // [pairs][zs]
    for (int e = threadIdx.x; e < nx + ny; e += blockDim.x) TW[e] = e < nx ? R.twx[e] : R.twy[e - nx];
    if (fast == 1) {  // the 40 x 32 grid: staged source, warp transforms
      layer_source_staged<40, 32>(R, mode, set, k, Z, reinterpret_cast<float*>(Z + pairs * zs));
      layer_forward_fast<40, 32>(R, Z, TW, k, nzc);
      continue;
    }
    const float *u = field(R, set, U), *v = field(R, set, V), *w = field(R, set, W);
    const float idx = R.inv_dx, idy = R.inv_dy;
    if (mode == PROJ_FACE) {
      const float rho = lvl(R, L_RHO, k), ihz = lvl(R, L_INV_HZ, k);
      const float rup = k < nz - 1 ? .5f * lvl(R, L_RUP, k) : 0.f, rdn = k > 0 ? .5f * lvl(R, L_RUP, k - 1) : 0.f;
      const int l = k * layer, lu = k < nz - 1 ? l + layer : l, ld = k > 0 ? l - layer : l;
#pragma unroll 4
      for (int e = threadIdx.x; e < pairs * 2 * nx; e += blockDim.x) {
        const int r = row_of(e, inv_nx), x = e - r * nx, y = r;
        float d = 0.f;
        if (r < ny) {
          const int c = x + y * nx;
          const int ce = (x + 1 == nx ? 0 : x + 1) + y * nx, cw = (x == 0 ? nx - 1 : x - 1) + y * nx;
          const int cn = x + (y + 1 == ny ? 0 : y + 1) * nx, cs = x + (y == 0 ? ny - 1 : y - 1) * nx;
          const float ddx = .5f * rho * (u[ce + l] - u[cw + l]);
          const float ddy = .5f * rho * (v[cn + l] - v[cs + l]);
          const float wc = w[c + l];
          const float up = rup * (wc + w[c + lu]), dn = rdn * (w[c + ld] + wc);
          d = ddx * idx + ddy * idy + (up - dn) * ihz;
        }
        reinterpret_cast<float*>(&Z[(r >> 1) * zs + x])[r & 1] = d;
      }
    } else if (mode == PROJ_GIVEN) {
      const float* rhs = R.phi + (size_t)k * layer;
      for (int e = threadIdx.x; e < pairs * 2 * nx; e += blockDim.x) {
        const int r = row_of(e, inv_nx), x = e - r * nx, y = r;
        reinterpret_cast<float*>(&Z[(r >> 1) * zs + x])[r & 1] = r < ny ? rhs[x + y * nx] : 0.f;
      }
    } else {
      const float r0 = .25f * lvl(R, L_RHO, k), r1 = .25f * lvl(R, L_RHO, k + 1), idz = lvl(R, L_INV_DZS, k), idt = 1.f / R.dt;
      const int l0 = k * layer, l1 = l0 + layer;
#pragma unroll 4
      for (int e = threadIdx.x; e < pairs * 2 * nx; e += blockDim.x) {
        const int r = row_of(e, inv_nx), x = e - r * nx, y = r;
        float d = 0.f;
        if (r < ny) {
          const int x1 = x + 1 == nx ? 0 : x + 1, y1 = (y + 1 == ny ? 0 : y + 1) * nx, yy = y * nx;
          const int a = x + yy, b = x1 + yy, ee = x + y1, f = x1 + y1;
          const float ddx = (r0 * ((u[b + l0] - u[a + l0]) + (u[f + l0] - u[ee + l0])) + r1 * ((u[b + l1] - u[a + l1]) + (u[f + l1] - u[ee + l1]))) * idx;
          const float ddy = (r0 * ((v[ee + l0] - v[a + l0]) + (v[f + l0] - v[b + l0])) + r1 * ((v[ee + l1] - v[a + l1]) + (v[f + l1] - v[b + l1]))) * idy;
          const float ddz = (r1 * ((w[a + l1] + w[b + l1]) + (w[ee + l1] + w[f + l1])) - r0 * ((w[a + l0] + w[b + l0]) + (w[ee + l0] + w[f + l0]))) * idz;
          d = (ddx + ddy + ddz) * idt;
        }
        reinterpret_cast<float*>(&Z[(r >> 1) * zs + x])[r & 1] = d;
      }
    }
    __syncthreads();
    if (fast == 2) { layer_forward_fast<80, 64>(R, Z, TW, k, nzc); continue; }
    float2* T = Z + pairs * nx;
    float2* X = T + pairs * nx;             // [nm][ny]
    float2* Xs = X + nm * ny;
    FftPlan Px{nx, R.fx_nf, R.fx_rad, TW}, Py{ny, R.fy_nf, R.fy_rad, TW + nx};
    const float2* Zf = fft_rows_any(Z, T, nx, pairs, Px);
    unpack_rows(Zf, X, nx, ny, ny, nm);
    const float2* Xf = fft_rows_any(X, Xs, ny, nm, Py);
    float2* g = R.spec + (size_t)k * ny;
    for (int e = threadIdx.x; e < nm * ny; e += blockDim.x) {
      const int m = e / ny, n = e - m * ny;
      g[(size_t)m * nzc * ny + n] = Xf[e];
    }
    __syncthreads();
  }
}

// One x-wavenumber m of one run per block, thread (n, real/imaginary): the FP64 sweeps of k_proj_modes on the 2-D
// spectrum in place (the input and the output stay in global memory; no transform, no barrier).
__global__ void k_proj_sweep(const RunDesc* __restrict__ runs, const int4* items, int nitems, int mode) {
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    const int m = items[it].y, ny = R.ny, nz = R.nz, nzc = mode == PROJ_FACE ? nz : nz - 1;
    const int u = threadIdx.x;
    if (u >= 2 * ny) continue;
    const int n = u >> 1, c = u & 1;
    float* g = reinterpret_cast<float*>(R.spec + (size_t)m * nzc * ny) + c;
    const TriAB* AB = (mode == PROJ_FACE ? R.tri_face : R.tri_pres) + (size_t)m * nzc * ny;
    const double* Cc = reinterpret_cast<const double*>((mode == PROJ_FACE ? R.tri_face : R.tri_pres) + (size_t)R.nm * nzc * ny) + (size_t)m * nzc * ny;
    double d[MAXNZ];
    double prev = 0;
    // levels in blocks of 8: the block's coefficients and values are loaded before its recurrence steps
    for (int k0 = 0; k0 < nzc; k0 += 8) {
      TriAB ab[8];
      float r[8];
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int k = min(k0 + j, nzc - 1);
        ab[j] = AB[(size_t)k * ny + n];
        r[j] = g[2 * ((size_t)k * ny + n)];
      }
#pragma unroll
      for (int j = 0; j < 8; j++) {
        if (k0 + j < nzc) { prev = fma(-ab[j].b, prev, widen(__fmul_rn(ab[j].a, r[j]))); d[k0 + j] = prev; }
      }
    }
    double x = d[nzc - 1];
    g[2 * ((size_t)(nzc - 1) * ny + n)] = narrow(x);
    for (int k1 = nzc - 2; k1 >= 0; k1 -= 8) {
      double cc[8];
#pragma unroll
      for (int j = 0; j < 8; j++) cc[j] = Cc[(size_t)max(k1 - j, 0) * ny + n];
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int k = k1 - j;
        if (k >= 0) { x = fma(-cc[j], x, d[k]); g[2 * ((size_t)k * ny + n)] = narrow(x); }
      }
    }
  }
}

// The 2-D inverse transform of one layer (y, then x with the Hermitian rows rebuilt two real rows per complex
// transform), normalised by nx*ny, into phi (FACE) or the pressure (PRES). Each inverse is the conjugate of the
// forward transform of the conjugate.
__global__ void __launch_bounds__(256, 5) k_proj_ifft2(const RunDesc* __restrict__ runs, const int4* items, int nitems, int mode) {
  extern __shared__ float2 smc[];
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    const int k = items[it].y, nx = R.nx, ny = R.ny, nz = R.nz, mh = R.mh, nm = R.nm;
    const int pairs = (ny + 1) / 2, nzc = mode == PROJ_FACE ? nz : nz - 1;
    float2* TW = smc;                       // the twiddles of x then y, staged once per layer
    for (int e = threadIdx.x; e < nx + ny; e += blockDim.x) TW[e] = e < nx ? R.twx[e] : R.twy[e - nx];
    float* out = (mode == PROJ_FACE ? R.phi : mode == PROJ_GIVEN ? R.pres2 : R.pres) + (size_t)k * nx * ny;
    if (const int fast = layer_fast(nx, ny)) {
      if (fast == 1) layer_inverse_fast<40, 32>(R, TW + nx + ny, TW, k, nzc, out);
      else layer_inverse_fast<80, 64>(R, TW + nx + ny, TW, k, nzc, out);
      continue;
    }
    float2* X = TW + nx + ny;               // [nm][ny]
    float2* Xs = X + nm * ny;
    float2* Z = Xs + nm * ny;               // [pairs][nx]
    float2* T = Z + pairs * nx;
    const float2* g = R.spec + (size_t)k * ny;
    for (int e = threadIdx.x; e < nm * ny; e += blockDim.x) {
      const int m = e / ny, n = e - m * ny;
      const float2 v = g[(size_t)m * nzc * ny + n];
      X[e] = make_float2(v.x, -v.y);
    }
    __syncthreads();
    FftPlan Px{nx, R.fx_nf, R.fx_rad, TW}, Py{ny, R.fy_nf, R.fy_rad, TW + nx};
    const float2* G = fft_rows_any(X, Xs, ny, nm, Py);   // conj of the y-inverse: H[m][y] = conj(G[m][y])
    const float inv_nx = 1.f / (float)nx;
    for (int e = threadIdx.x; e < pairs * nx; e += blockDim.x) {
      const int pr = row_of(e, inv_nx), m = e - pr * nx, c = m <= mh ? m : nx - m;
      const float sg = m <= mh ? 1.f : -1.f;
      const bool real = c == 0 || 2 * c == nx, pair = 2 * pr + 1 < ny;
      const float2 A = G[c * ny + 2 * pr];
      const float ar = A.x, ai = real ? 0.f : -sg * A.y;
      float br = 0.f, bi = 0.f;
      if (pair) { const float2 B = G[c * ny + 2 * pr + 1]; br = B.x; bi = real ? 0.f : -sg * B.y; }
      Z[pr * nx + m] = make_float2(ar - bi, -(ai + br));  // conj(A + iB)
    }
    __syncthreads();
    const float2* Zf = fft_rows_any(Z, T, nx, pairs, Px);
    const float norm = 1.f / (float)(nx * ny);
    for (int e = threadIdx.x; e < ny * nx; e += blockDim.x) {
      const int r = row_of(e, inv_nx), x = e - r * nx;
      const float2 z = Zf[(r >> 1) * nx + x];
      out[r * nx + x] = ((r & 1) ? -z.y : z.x) * norm;
    }
    __syncthreads();
  }
}

// Projected face mass fluxes and their divergence (FluxTransport.correctFaces + divergence, advection.ts:203-255):
// mx = rho (u + u_e)/2 - rho (phi_e - phi)/dx, and so on; div of the corrected faces at the node. Each thread takes
// nodes in passes of NB, their loads issued together.
constexpr int NB = 4;
__global__ void k_face_correct(const RunDesc* __restrict__ runs, const int4* items, int nitems, int set) {
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    const int nx = R.nx, ny = R.ny, nz = R.nz, layer = R.layer, i0 = items[it].y * CHUNK, i1 = min(R.n, i0 + CHUNK);
    const float* __restrict__ u = field(R, set, U);
    const float* __restrict__ v = field(R, set, V);
    const float* __restrict__ w = field(R, set, W);
    const float* __restrict__ phi = R.phi;
    float4* F4 = reinterpret_cast<float4*>(R.faces);
    const float inv_nx = 1.f / (float)nx, idx = R.inv_dx, idy = R.inv_dy;
    const int B = blockDim.x;
    int z = (i0 + threadIdx.x) / layer;
    for (int base = i0 + threadIdx.x; base < i1; base += NB * B) {
      float uc[NB], ue[NB], uw[NB], vc[NB], vn[NB], vs[NB], wc[NB], wu[NB], wd[NB];
      float pc[NB], pe[NB], pw[NB], pn[NB], ps[NB], pu[NB], pd[NB];
      int zz[NB];
#pragma unroll
      for (int j = 0; j < NB; j++) {
        const int i = min(base + j * B, i1 - 1);
        while (i >= (z + 1) * layer) z++;
        zz[j] = z;
        const int c = i - z * layer, y = row_of(c, inv_nx), x = c - y * nx, l = z * layer;
        const int ie = (x + 1 == nx ? 0 : x + 1) + y * nx + l, iw = (x == 0 ? nx - 1 : x - 1) + y * nx + l;
        const int in = x + (y + 1 == ny ? 0 : y + 1) * nx + l, is = x + (y == 0 ? ny - 1 : y - 1) * nx + l;
        const int iu = z < nz - 1 ? i + layer : i, id = z > 0 ? i - layer : i;
        uc[j] = u[i]; ue[j] = u[ie]; uw[j] = u[iw]; vc[j] = v[i]; vn[j] = v[in]; vs[j] = v[is];
        wc[j] = w[i]; wu[j] = w[iu]; wd[j] = w[id];
        pc[j] = phi[i]; pe[j] = phi[ie]; pw[j] = phi[iw]; pn[j] = phi[in]; ps[j] = phi[is]; pu[j] = phi[iu]; pd[j] = phi[id];
      }
#pragma unroll
      for (int j = 0; j < NB; j++) {
        const int i = base + j * B;
        if (i >= i1) break;
        const int k = zz[j];
        const float rho = lvl(R, L_RHO, k), p0 = pc[j];
        const float fxE = rho * (.5f * (uc[j] + ue[j]) - (pe[j] - p0) * idx);
        const float fxW = rho * (.5f * (uw[j] + uc[j]) - (p0 - pw[j]) * idx);
        const float fyN = rho * (.5f * (vc[j] + vn[j]) - (pn[j] - p0) * idy);
        const float fyS = rho * (.5f * (vs[j] + vc[j]) - (p0 - ps[j]) * idy);
        const float fzU = k < nz - 1 ? lvl(R, L_RUP, k) * (.5f * (wc[j] + wu[j]) - (pu[j] - p0) * lvl(R, L_INV_DZS, k)) : 0.f;
        const float fzD = k > 0 ? lvl(R, L_RUP, k - 1) * (.5f * (wd[j] + wc[j]) - (p0 - pd[j]) * lvl(R, L_INV_DZS, k - 1)) : 0.f;
        F4[i] = make_float4(fxE, fyN, fzU, (fxE - fxW) * idx + (fyN - fyS) * idy + (fzU - fzD) * lvl(R, L_INV_HZ, k));
      }
    }
  }
}

// u -= dt G p at the nodes of one set (PressureSolver.correct, src/core/pressure.ts:69-92); in the final projection
// the wind limits act and count (clipWind, src/core/model.ts:1586-1595). Nodes in passes of NB, as above.
// MODE: 0 a stage projection; 1 the final projection of the runs without its refinement (the refined runs are skipped);
// 2 the final velocity of the refined runs, u - dt G p1 - dt G p2 in FP32 (p2 from the refinement's solve: the
// correction of mode 1, then that of p2, a few 1e-6 of it).
template <int MODE>
__global__ void k_pres_correct(const RunDesc* __restrict__ runs, const int4* items, int nitems, int set) {
  constexpr bool final_ = MODE > 0, two = MODE == 2;
  constexpr int nb = two ? 2 : NB;  // two pressures: fewer nodes a pass
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    if (final_ && (bool)(R.flags & RF_REFINE) != two) continue;
    const int nx = R.nx, ny = R.ny, nz = R.nz, layer = R.layer, i0 = items[it].y * CHUNK, i1 = min(R.n, i0 + CHUNK);
    float *u = field(R, set, U), *v = field(R, set, V), *w = field(R, set, W);
    const float* __restrict__ p = R.pres;
    const float* __restrict__ p2 = R.pres2;
    const float dt = R.dt, inv_nx = 1.f / (float)nx;
    const int B = blockDim.x;
    int clipped = 0;
    int z = (i0 + threadIdx.x) / layer;
    for (int base = i0 + threadIdx.x; base < i1; base += nb * B) {
      float lo[nb][4], hi[nb][4], lo2[two ? nb : 1][4], hi2[two ? nb : 1][4], uu[nb], vv[nb], ww[nb];
      int zz[nb];
#pragma unroll
      for (int j = 0; j < nb; j++) {
        const int i = min(base + j * B, i1 - 1);
        while (i >= (z + 1) * layer) z++;
        zz[j] = z;
        const int c = i - z * layer, jy = row_of(c, inv_nx), x = c - jy * nx;
        const int im = x == 0 ? nx - 1 : x - 1, jm = (jy == 0 ? ny - 1 : jy - 1) * nx, j0 = jy * nx;
        const size_t lz = (size_t)max(0, z - 1) * layer, hz_ = (size_t)min(nz - 2, z) * layer;
        const float* L = p + lz;
        const float* H = p + hz_;
        // corners (im, jm), (x, jm), (im, j0), (x, j0) of the dual cells below and above
        lo[j][0] = L[im + jm]; lo[j][1] = L[x + jm]; lo[j][2] = L[im + j0]; lo[j][3] = L[x + j0];
        hi[j][0] = H[im + jm]; hi[j][1] = H[x + jm]; hi[j][2] = H[im + j0]; hi[j][3] = H[x + j0];
        if (two) {
          const float* L2 = p2 + lz;
          const float* H2 = p2 + hz_;
          lo2[j][0] = L2[im + jm]; lo2[j][1] = L2[x + jm]; lo2[j][2] = L2[im + j0]; lo2[j][3] = L2[x + j0];
          hi2[j][0] = H2[im + jm]; hi2[j][1] = H2[x + jm]; hi2[j][2] = H2[im + j0]; hi2[j][3] = H2[x + j0];
        }
        uu[j] = u[i]; vv[j] = v[i]; ww[j] = w[i];
      }
#pragma unroll
      for (int j = 0; j < nb; j++) {
        const int i = base + j * B;
        if (i >= i1) break;
        const int k = zz[j];
        // dzs(k-1)/hz and dzs(k)/hz, rounded once from FP64 (zero at the ground and the top)
        const float wLo = lvl(R, L_WLO, k), wHi = lvl(R, L_WHI, k);
        const float qx = .25f * R.inv_dx, qy = .25f * R.inv_dy, qz = .25f * lvl(R, L_INV_HZ, k);
        const bool inner = k > 0 && k < nz - 1;
        auto grad = [&](const float* l, const float* h, float& gx, float& gy, float& gz) {
          gx = (wLo * ((l[1] - l[0]) + (l[3] - l[2])) + wHi * ((h[1] - h[0]) + (h[3] - h[2]))) * qx;
          gy = (wLo * ((l[2] - l[0]) + (l[3] - l[1])) + wHi * ((h[2] - h[0]) + (h[3] - h[1]))) * qy;
          // the gradient between the dual cells below (k - 1) and above (k)
          gz = ((h[0] - l[0]) + (h[1] - l[1]) + (h[2] - l[2]) + (h[3] - l[3])) * qz;
        };
        float gx, gy, gz;
        grad(lo[j], hi[j], gx, gy, gz);
        float un = __fmaf_rn(-dt, gx, uu[j]), vn = __fmaf_rn(-dt, gy, vv[j]), wn = inner ? __fmaf_rn(-dt, gz, ww[j]) : ww[j];
        if (two) {
          grad(lo2[j], hi2[j], gx, gy, gz);
          un = __fmaf_rn(-dt, gx, un); vn = __fmaf_rn(-dt, gy, vn);
          if (inner) wn = __fmaf_rn(-dt, gz, wn);
        }
        if (final_) {
          const float UL = 120.f, WL = 100.f;
          if (un < -UL || un > UL) { un = fmaxf(-UL, fminf(UL, un)); clipped++; }
          if (vn < -UL || vn > UL) { vn = fmaxf(-UL, fminf(UL, vn)); clipped++; }
          if (wn < -WL || wn > WL) { wn = fmaxf(-WL, fminf(WL, wn)); clipped++; }
        }
        u[i] = un; v[i] = vn; w[i] = wn;
      }
    }
    if (final_) {
      clipped = warpSum(clipped);
      if ((threadIdx.x & 31) == 0 && clipped) atomicAdd(&R.cnt[C_CLIPPED], (unsigned long long)clipped);
    }
  }
}

// ---- refinement of the final projection (runs with RF_REFINE). The solve above works in FP32 transforms and an FP32
// pressure, which leaves a residual divergence of a few 1e-6 of the one it removed. One refinement step brings it to
// rounding level: the projected velocity v = u - dt G p1 and its divergence are formed in double-FP32 arithmetic
// (hi + lo pairs, error-free sums and products: about 44 significant bits on the FP32 pipes), the residual r = D v / dt
// is solved again (p2) and the velocity becomes u - dt G p1 - dt G p2 in FP32 (two corrections of a few rounding
// errors of v each: the storage of v in FP32 bounds its divergence either way). The projection's pressure is p1 + p2.
struct DF { float hi, lo; };
__device__ __forceinline__ DF df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b), bp = __fsub_rn(s, a);
  return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp))};
}
__device__ __forceinline__ DF df_fast(float s, float e) {  // |s| >= |e|
  const float h = __fadd_rn(s, e);
  return DF{h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  const DF s = df_two_sum(a.hi, b.hi);
  return df_fast(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ DF df_sub(DF a, DF b) { return df_add(a, DF{-b.hi, -b.lo}); }
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.hi, -p)));
  return df_fast(p, e);
}
__device__ __forceinline__ DF df_diff(float a, float b) { return df_two_sum(a, -b); }  // a - b exactly

// The same operations on two independent values at once (the x and y lanes) on the packed FP32 pipes: per lane the
// bits of the scalar functions above (a - b is formed as fma(b, -1, a), the same rounded difference).
struct DF2 { float2 hi, lo; };
__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f, -1.f), a); }
__device__ __forceinline__ DF2 df2_two_sum(float2 a, float2 b) {
  const float2 s = add2(a, b), bp = sub2(s, a);
  return DF2{s, add2(sub2(a, sub2(s, bp)), sub2(b, bp))};
}
__device__ __forceinline__ DF2 df2_fast(float2 s, float2 e) {
  const float2 h = add2(s, e);
  return DF2{h, sub2(e, sub2(h, s))};
}
__device__ __forceinline__ DF2 df2_add(DF2 a, DF2 b) {
  const DF2 s = df2_two_sum(a.hi, b.hi);
  return df2_fast(s.hi, add2(s.lo, add2(a.lo, b.lo)));
}
__device__ __forceinline__ DF2 df2_mul(DF2 a, DF2 b) {
  const float2 p = __fmul2_rn(a.hi, b.hi);
  const float2 e = __ffma2_rn(a.hi, b.lo, __ffma2_rn(a.lo, b.hi, __ffma2_rn(a.hi, b.hi, f2(-p.x, -p.y))));
  return df2_fast(p, e);
}
__device__ __forceinline__ DF2 df2_diff(float2 a, float2 b) { return df2_two_sum(a, f2(-b.x, -b.y)); }
__device__ __forceinline__ DF2 df2_splat(DF a) { return DF2{f2(a.hi, a.hi), f2(a.lo, a.lo)}; }

// G p1 at a node of level k in double-FP32 (the gradient of k_pres_correct) from the pressure of the four dual cells
// around it below (l: (x-1, y-1), (x, y-1), (x-1, y), (x, y)) and above (h, the same order).
__device__ __forceinline__ void df_gradient_of(const RunDesc& R, int k, float l0, float l1, float l2, float l3, float h0, float h1,
                                               float h2, float h3, DF& gx, DF& gy, DF& gz) {
  const int nz = R.nz;
  const DF wlo = k > 0 ? DF{lvl(R, L_WLO, k), lvl(R, L_WLO_LO, k)} : DF{0.f, 0.f};
  const DF whi = k < nz - 1 ? DF{lvl(R, L_WHI, k), lvl(R, L_WHI_LO, k)} : DF{0.f, 0.f};
  const DF qx{.25f * R.inv_dx, .25f * R.inv_dx_lo}, qy{.25f * R.inv_dy, .25f * R.inv_dy_lo};
  // gx and gy as the two lanes of one packed evaluation
  const DF2 W0 = df2_splat(wlo), W1 = df2_splat(whi), Q{f2(qx.hi, qy.hi), f2(qx.lo, qy.lo)};
  const DF2 g = df2_mul(df2_add(df2_mul(W0, df2_add(df2_diff(f2(l1, l2), f2(l0, l0)), df2_diff(f2(l3, l3), f2(l2, l1)))),
                                df2_mul(W1, df2_add(df2_diff(f2(h1, h2), f2(h0, h0)), df2_diff(f2(h3, h3), f2(h2, h1))))), Q);
  gx = DF{g.hi.x, g.lo.x};
  gy = DF{g.hi.y, g.lo.y};
  gz = DF{0.f, 0.f};
  if (k > 0 && k < nz - 1) {
    const DF s = df_add(df_add(df_diff(h0, l0), df_diff(h1, l1)), df_add(df_diff(h2, l2), df_diff(h3, l3)));
    gz = df_mul(s, DF{.25f * lvl(R, L_INV_HZ, k), .25f * lvl(R, L_INV_HZ_LO, k)});
  }
}

// The residual of the refined runs' final projection in one tiled march over the item's levels (run, tile, z0, z1),
// a thread per node of the tile and its halo:
// per node level, v = u - dt G p1 in double-FP32 for the tile's nodes and a one-node halo on the high x and y sides
// (into a pair of shared-memory planes); per dual layer, r = D v / dt rounded once into phi: D of the hi parts in double-FP32 (their differences
// are exact), D of the lo parts (a few 1e-8 of them) in FP32. The pressure planes (dual levels k - 1 and k, with a
// one-cell halo on the low sides) arrive by asynchronous copies a level ahead.
// CTX x CTY: the tile as compile-time constants (20 x 8, the refinement tile of grids 40 wide), or 0 x 0 for a tile
// given at run time.
template <int CTX, int CTY>
__global__ void __launch_bounds__(192, 4) k_refine_residual(const RunDesc* __restrict__ runs, const int4* items, int nitems, int set,
                                                         int TXr, int TYr) {
  extern __shared__ float rsm[];
  const int TX = CTX ? CTX : TXr, TY = CTY ? CTY : TYr;
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED] || !(R.flags & RF_REFINE)) continue;
    const int tile = items[it].y, z0 = items[it].z, z1 = items[it].w;
    const int nx = R.nx, ny = R.ny, nz = R.nz, layer = R.layer;
    const int PW = TX + 2, PP = PW * (TY + 2), NW = TX + 1, NN = NW * (TY + 1), t = threadIdx.x;
    const int NT = CTX ? ((CTX + 1) * (CTY + 1) + 31) / 32 * 32 : (int)blockDim.x;
    float* pp = rsm;                 // [2][PP]: p1 of dual level d in slot d & 1, columns x0 - 1 .. x0 + TX
    float* nv = rsm + 2 * PP;        // [2][6][NN]: node level k in slot k & 1; u hi, u lo, v hi, v lo, w hi, w lo
    const int tilesX = (nx + TX - 1) / TX, x0 = (tile % tilesX) * TX, y0 = (tile / tilesX) * TY;
    const float* __restrict__ u = field(R, set, U);
    const float* __restrict__ v = field(R, set, V);
    const float* __restrict__ w = field(R, set, W);
    const float* __restrict__ p = R.pres;
    const DF dt{R.dt, 0.f};
    const int kTop = min(z1, nz - 1);  // node levels z0 .. kTop; dual layers z0 .. kTop - 1
    auto load_plane = [&](int d, bool async) {
      float* dst = pp + (d & 1) * PP;
      const float* src = p + (size_t)d * layer;
      for (int e = t; e < PP; e += NT) {
        const int hy = e / PW, hx = e - hy * PW;
        const int gx = wrap(x0 - 1 + hx, nx), gy = wrap(y0 - 1 + hy, ny);
        if (async) cp_async4(dst + e, src + gx + gy * nx); else dst[e] = src[gx + gy * nx];
      }
    };
    load_plane(max(0, z0 - 1), false);
    load_plane(min(nz - 2, z0), false);
    const int lx = t % TX, ly = t / TX, cx = x0 + lx, cy = y0 + ly;  // the dual cell of thread t < TX * TY
    const bool on = t < TX * TY && cx < nx && cy < ny;
    const DF idx{R.inv_dx, R.inv_dx_lo}, idy{R.inv_dy, R.inv_dy_lo}, idt{R.inv_dt, R.inv_dt_lo};
    for (int k = z0; k <= kTop; k++) {
      cp_async_wait_all();
      __syncthreads();
      // node velocities of level k
      const float* L = pp + (max(0, k - 1) & 1) * PP;
      const float* H = pp + (min(nz - 2, k) & 1) * PP;
      float* V = nv + (k & 1) * 6 * NN;
      for (int e = t; e < NN; e += NT) {
        const int ny_ = e / NW, nx_ = e - ny_ * NW;
        if (x0 + nx_ > nx || y0 + ny_ > ny) continue;  // past the last cell of a partial tile
        const int gx = x0 + nx_ == nx ? 0 : x0 + nx_, gy = y0 + ny_ == ny ? 0 : y0 + ny_;
        const int a = ny_ * PW + nx_;  // p plane cell (x - 1, y - 1)
        DF g[3];
        df_gradient_of(R, k, L[a], L[a + 1], L[a + PW], L[a + PW + 1], H[a], H[a + 1], H[a + PW], H[a + PW + 1], g[0], g[1], g[2]);
        const size_t i = (size_t)k * layer + gx + gy * nx;
        const float uin[3] = {u[i], v[i], w[i]};
        DF r[3];
        {  // u and v as the lanes of one packed evaluation (df_sub(a, b) = df_add(a, -b))
          const DF2 m = df2_mul(df2_splat(dt), DF2{f2(g[0].hi, g[1].hi), f2(g[0].lo, g[1].lo)});
          const DF2 uv = df2_add(DF2{f2(uin[0], uin[1]), f2(0.f, 0.f)}, DF2{f2(-m.hi.x, -m.hi.y), f2(-m.lo.x, -m.lo.y)});
          r[0] = DF{uv.hi.x, uv.lo.x}; r[1] = DF{uv.hi.y, uv.lo.y};
        }
        r[2] = df_sub(DF{uin[2], 0.f}, df_mul(dt, g[2]));
#pragma unroll
        for (int d = 0; d < 3; d++) {
          V[(2 * d) * NN + e] = r[d].hi;
          V[(2 * d + 1) * NN + e] = r[d].lo;
        }
      }
      __syncthreads();
      // the pressure of dual level k + 1 for the next node level (its slot held dual level k - 1, read above)
      if (k + 1 <= kTop && k + 1 <= nz - 2) load_plane(k + 1, true);
      // the residual of dual layer k - 1 (node levels k - 1 and k)
      if (k > z0 && on) {
        const int kc = k - 1;
        const float* B0 = nv + (kc & 1) * 6 * NN;
        const float* B1 = V;
        const int a = ly * NW + lx, b = a + 1, e = a + NW, f = e + 1;
        const DF r0{.25f * lvl(R, L_RHO, kc), .25f * lvl(R, L_RHO_LO, kc)}, r1{.25f * lvl(R, L_RHO, kc + 1), .25f * lvl(R, L_RHO_LO, kc + 1)};
        const DF idz{lvl(R, L_INV_DZS, kc), lvl(R, L_INV_DZS_LO, kc)};
        const float *hu0 = B0, *hv0 = B0 + 2 * NN, *hw0 = B0 + 4 * NN, *hu1 = B1, *hv1 = B1 + 2 * NN, *hw1 = B1 + 4 * NN;
        // ddx and ddy as the two lanes of one packed evaluation
        const DF2 dxy = df2_mul(df2_add(df2_mul(df2_splat(r0), df2_add(df2_diff(f2(hu0[b], hv0[e]), f2(hu0[a], hv0[a])), df2_diff(f2(hu0[f], hv0[f]), f2(hu0[e], hv0[b])))),
                                        df2_mul(df2_splat(r1), df2_add(df2_diff(f2(hu1[b], hv1[e]), f2(hu1[a], hv1[a])), df2_diff(f2(hu1[f], hv1[f]), f2(hu1[e], hv1[b]))))),
                                DF2{f2(idx.hi, idy.hi), f2(idx.lo, idy.lo)});
        const DF ddx{dxy.hi.x, dxy.lo.x}, ddy{dxy.hi.y, dxy.lo.y};
        const DF up = df_add(df_add(DF{hw1[a], 0.f}, DF{hw1[b], 0.f}), df_add(DF{hw1[e], 0.f}, DF{hw1[f], 0.f}));
        const DF dn = df_add(df_add(DF{hw0[a], 0.f}, DF{hw0[b], 0.f}), df_add(DF{hw0[e], 0.f}, DF{hw0[f], 0.f}));
        const DF ddz = df_mul(df_sub(df_mul(r1, up), df_mul(r0, dn)), idz);
        const float *lu0 = B0 + NN, *lv0 = B0 + 3 * NN, *lw0 = B0 + 5 * NN, *lu1 = B1 + NN, *lv1 = B1 + 3 * NN, *lw1 = B1 + 5 * NN;
        const float rr0 = r0.hi, rr1 = r1.hi;
        const float lox = (rr0 * ((lu0[b] - lu0[a]) + (lu0[f] - lu0[e])) + rr1 * ((lu1[b] - lu1[a]) + (lu1[f] - lu1[e]))) * idx.hi;
        const float loy = (rr0 * ((lv0[e] - lv0[a]) + (lv0[f] - lv0[b])) + rr1 * ((lv1[e] - lv1[a]) + (lv1[f] - lv1[b]))) * idy.hi;
        const float loz = (rr1 * ((lw1[a] + lw1[b]) + (lw1[e] + lw1[f])) - rr0 * ((lw0[a] + lw0[b]) + (lw0[e] + lw0[f]))) * idz.hi;
        const DF dd = df_mul(df_add(df_add(df_add(ddx, ddy), ddz), DF{(lox + loy) + loz, 0.f}), idt);
        R.phi[(size_t)kc * layer + cx + cy * nx] = dd.hi + dd.lo;
      }
    }
    cp_async_wait_all();
    __syncthreads();
  }
}

// ==================================================================== endStep
// Sums of the positivity fix over one chunk of the final RK3 values (fillNegative, src/core/model.ts:606-617):
// per conserve field, (removed, kept, negative) weighted by the level weight, FP64, in a fixed order.
__global__ void k_fill_partial(const RunDesc* __restrict__ runs, const int4* items, int nitems, int set) {
  __shared__ double sh[32 * NCONS * 3];
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    const int chunk = items[it].y, i0 = chunk * CHUNK, i1 = min(R.n, i0 + CHUNK);
    // per conserve field: removed (the tiny values the fix zeroes), kept (the rest), negative (-sum of the negatives)
    float hi[NCONS * 3], lo[NCONS * 3];
#pragma unroll
    for (int k = 0; k < NCONS * 3; k++) hi[k] = lo[k] = 0.f;
    const float* fp[NCONS];
#pragma unroll
    for (int k = 0; k < NCONS; k++) fp[k] = field(R, set, cons_field(k));
    const int layer = R.layer, B = blockDim.x;
    int z = (i0 + threadIdx.x) / layer;
    // four nodes per pass: their 28 loads are issued together
    for (int base = i0 + threadIdx.x; base < i1; base += 4 * B) {
      float x[4][NCONS];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int i = base + j * B;
#pragma unroll
        for (int k = 0; k < NCONS; k++) x[j][k] = i < i1 ? fp[k][i] : 0.f;
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int i = base + j * B;
        while (i >= (z + 1) * layer) z++;
        const float whi = lvl(R, L_LW, z), wlo = lvl(R, L_LW_LO, z);
#pragma unroll
        for (int k = 0; k < NCONS; k++) {
          const float v = x[j][k];
          if (v < 1e-10f) {
            if (v != 0.f) {
              df_add_prod(hi[3 * k], lo[3 * k], whi, wlo, v);
              if (v < 0.f) df_add_prod(hi[3 * k + 2], lo[3 * k + 2], whi, wlo, -v);
            }
          } else {
            df_add_prod(hi[3 * k + 1], lo[3 * k + 1], whi, wlo, v);
          }
        }
      }
    }
    blockSumsDF<NCONS * 3>(hi, lo, R.part + (size_t)chunk * NCONS * 3, sh);
  }
}
// Per run: the scale of each conserve field, kept as delta = scale - 1 so a * scale rounds once (fma). Thread k sums
// field k's block partials (FP64, in chunk order).
__global__ void k_fill_final(const RunDesc* __restrict__ runs, const int4* items, int nitems) {
  __shared__ double negs[NCONS];
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    const int nch = (R.n + CHUNK - 1) / CHUNK, k = threadIdx.x;
    if (k < NCONS) {
      double removed = 0, kept = 0, negative = 0;
      for (int c = 0; c < nch; c++) {
        const double* p = R.part + ((size_t)c * NCONS + k) * 3;
        removed += p[0]; kept += p[1]; negative += p[2];
      }
      double delta = 0;
      if (!(removed == 0 && negative == 0)) delta = kept > 0 ? fmax(-1.0, removed / kept) : -1.0;
      R.scr[S_FILL + k] = (float)delta;
      negs[k] = negative;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double neg = 0;
      for (int j = 0; j < NCONS; j++) neg += negs[j];
      R.acc[A_NEG] += neg;
    }
    __syncthreads();
  }
}

// Per node: the positivity fix and the cold decay ('finish', :1253-1258), then physics(z) (:1347-1531): microphysics,
// Coriolis and wind relaxation, surface fluxes (none in the single-storm mode), cold clamp, Rayleigh sponge.
// In: set `in` (final RK3 values). Out: rain, snow, graupel, hail, cold -> set A; the mixed fields -> set `mid`.
// A variant for each kind of run, so each runs only its own code (the plan launches each on its runs' items): ELEC, an
// electrified run's, which also moves the charge with the water and charges the graupel and crystals after the
// microphysics (:1454-1469; the charges go to set A, they are not mixed); MOM 1 one-moment microphysics, 2 two-moment
// rain, 3 two-moment rain, graupel and hail (their numbers and volumes to set A).
template <bool ELEC, int MOM>
__global__ void __launch_bounds__(256, (ELEC || MOM == 3) ? 2 : 3) k_physics(const RunDesc* __restrict__ runs, const int4* items, int nitems, int in, int mid) {
  __shared__ double sh[32 * 4];
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    const int chunk = items[it].y, i0 = chunk * CHUNK, i1 = min(R.n, i0 + CHUNK);
    const float dt = R.dt, keepCold = __powf(.9992f, dt);
    float fill[NCONS];
#pragma unroll
    for (int k = 0; k < NCONS; k++) fill[k] = R.scr[S_FILL + k];
    constexpr int NW = ELEC ? 4 : 3;  // the water budget's three sums, and the charge separated
    float whi[NW], wlo[NW];
#pragma unroll
    for (int k = 0; k < NW; k++) whi[k] = wlo[k] = 0.f;
    bool bad = false;
    constexpr bool elec = ELEC;
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      const int z = i / R.layer;
      auto fixed = [&](int kc, float x) { return x < 1e-10f ? 0.f : fmaf(x, fill[kc], x); };
      phys::Node s;
      s.rain = fixed(0, field(R, in, RAIN)[i]); s.snow = fixed(1, field(R, in, SNOW)[i]);
      s.graupel = fixed(2, field(R, in, GRAUPEL)[i]); s.hail = fixed(3, field(R, in, HAIL)[i]);
      s.q = fixed(4, field(R, in, Q)[i]); s.cloud = fixed(5, field(R, in, CLOUD)[i]); s.ice = fixed(6, field(R, in, ICE)[i]);
      s.inum = field(R, in, ICENUM)[i];
      s.cold = field(R, in, COLD)[i] * keepCold;
      s.thp = field(R, in, THETA)[i]; s.thb = lvl(R, L_THB, z); s.tcb = lvl(R, L_TCB, z);
      float u = field(R, in, U)[i], v = field(R, in, V)[i], w = field(R, in, W)[i];
      phys::Level pl;
      pl.exner = lvl(R, L_EXNER, z); pl.p = lvl(R, L_P, z); pl.rho = lvl(R, L_RHO, z); pl.fallsq = lvl(R, L_FALLSQ, z); pl.tcb = s.tcb;
      pl.qw_hi = lvl(R, L_QW_HI, z); pl.qw_lo = lvl(R, L_QW_LO, z); pl.bw = lvl(R, L_BW, z);
      pl.qi_hi = lvl(R, L_QI_HI, z); pl.qi_lo = lvl(R, L_QI_LO, z); pl.bi = lvl(R, L_BI, z);
      pl.q0_hi = lvl(R, L_Q0_HI, z); pl.q0_lo = lvl(R, L_Q0_LO, z);
      const float q0 = s.q;
      float before[4];
      if constexpr (ELEC) if (elec) { before[0] = s.ice + s.snow; before[1] = s.graupel + s.hail; before[2] = s.rain; before[3] = s.cloud; }
      float evap, rnum = 0.f;
      i2m::Fields f2m = {0.f, 0.f, 0.f, 0.f};
      bool wet2G = false, wet2H = false;
      if constexpr (MOM == 3) {
        rnum = field(R, in, RAIN_NUMBER)[i];
        f2m = {field(R, in, GRAUPEL_NUMBER)[i], field(R, in, GRAUPEL_VOLUME)[i], field(R, in, HAIL_NUMBER)[i], field(R, in, HAIL_VOLUME)[i]};
        i2m::microphysics(s, rnum, f2m, pl, dt, R.flags, R.breakup, evap, wet2G, wet2H);
      } else if constexpr (MOM == 2) {
        rnum = field(R, in, RAIN_NUMBER)[i];
        r2m::microphysics(s, rnum, pl, dt, R.flags, R.breakup, evap);
      } else phys::microphysics(s, pl, dt, R.flags, evap);
      if constexpr (ELEC) if (elec) {
        const float after[4] = {s.ice + s.snow, s.graupel + s.hail, s.rain, s.cloud};
        float c[4] = {field(R, in, CHARGE_ICE)[i], field(R, in, CHARGE_GRAUPEL)[i], field(R, in, CHARGE_RAIN)[i], field(R, in, CHARGE_AIR)[i]};
        if (c[0] != 0.f || c[1] != 0.f || c[2] != 0.f || c[3] != 0.f) charge::transferCharge(c, before, after);
        const float tc = phys::tcOf(s, pl.exner), rho = pl.rho;
        // two-moment graupel and hail: their wet growth from their processes, their charging by their own moments
        // (:1461-1466; a class without particles charges by the fixed intercept's)
        bool wetG, wetH;
        charge::Moments two[2];
        int has = 0;
        if constexpr (MOM == 3) {
          wetG = wet2G; wetH = wet2H;
          if (i2m::rimerMoments(i2m::GRAUPEL_2M(), s.graupel, f2m.gn, f2m.gv, rho, two[0])) has |= 1;
          if (i2m::rimerMoments(i2m::HAIL_2M(), s.hail, f2m.hn, f2m.hv, rho, two[1])) has |= 2;
        } else {
          wetG = charge::wetGrowing(s.graupel, phys::N0G, phys::RHO_G, tc, s, pl); wetH = charge::wetGrowing(s.hail, phys::N0H, phys::RHO_H, tc, s, pl);
        }
        const float separated = charge::chargingRate(tc, rho, s.cloud, s.ice, s.snow, s.graupel, s.hail, R.vfall[V_SNOW * (size_t)R.n + i], wetG, wetH, s.inum * rho, two, has) * dt / rho;
        const float induced = charge::inductiveRate(tc, rho, s.cloud, s.graupel, s.hail, R.ez[i], (c[1] + separated) * rho, wetG, wetH, two, has) * dt / rho;
        field(R, 0, CHARGE_ICE)[i] = c[0] - separated; field(R, 0, CHARGE_GRAUPEL)[i] = c[1] + separated + induced;
        field(R, 0, CHARGE_RAIN)[i] = c[2]; field(R, 0, CHARGE_AIR)[i] = c[3] - induced;
        df_add_prod(whi[NW - 1], wlo[NW - 1], lvl(R, L_NODEMASS, z), lvl(R, L_NODEMASS_LO, z), fabsf(separated) + fabsf(induced));
      }
      if (!(R.flags & RF_STAGES)) {
        float num = s.thp + .61f * ((s.thb + s.thp) * (s.q - lvl(R, L_QB, z)) + lvl(R, L_QB, z) * s.thp);
        float loaded = s.cloud + s.ice + ((R.flags & RF_LOADING) ? s.rain + s.snow + s.graupel + s.hail : 0.f);
        w += 9.81f * (num / lvl(R, L_THVENV, z) - loaded) * dt;
      }
      // Coriolis on the departure from the environmental wind, relaxed towards it (:1478).
      const float ue = lvl(R, L_UENV, z), ve = lvl(R, L_VENV, z);
      float du = (u - ue) * R.keep, dvv = (v - ve) * R.keep;
      u = ue + du + R.coriolis * dvv * dt; v = ve + dvv - R.coriolis * du * dt;
      const float nmh = lvl(R, L_NODEMASS, z), nml = lvl(R, L_NODEMASS_LO, z);
      {
        const float dq = s.q - q0;
        if (dq < 0.f) df_add_prod(whi[0], wlo[0], nmh, nml, -dq); else df_add_prod(whi[1], wlo[1], nmh, nml, dq);
        if (evap > 0.f) df_add_prod(whi[2], wlo[2], nmh, nml, evap);
      }
      s.cold = s.cold < 1e-3f ? 0.f : fminf(s.cold, 15.f);
      const float sp = lvl(R, L_SPONGE, z);
      if (sp > 0.f) { w *= 1.f - sp; u += (ue - u) * sp; v += (ve - v) * sp; s.thp += (0.f - s.thp) * sp; }
      bad |= !(isfinite(s.thp) && isfinite(s.q) && isfinite(u) && isfinite(v) && isfinite(w) && isfinite(s.rain) && isfinite(s.cloud));
      field(R, 0, RAIN)[i] = s.rain; field(R, 0, SNOW)[i] = s.snow; field(R, 0, GRAUPEL)[i] = s.graupel; field(R, 0, HAIL)[i] = s.hail;
      field(R, 0, COLD)[i] = s.cold;
      field(R, mid, U)[i] = u; field(R, mid, V)[i] = v; field(R, mid, W)[i] = w; field(R, mid, THETA)[i] = s.thp;
      field(R, mid, Q)[i] = s.q; field(R, mid, CLOUD)[i] = s.cloud; field(R, mid, ICE)[i] = s.ice; field(R, mid, ICENUM)[i] = s.inum;
      if constexpr (MOM >= 2) field(R, 0, RAIN_NUMBER)[i] = rnum;  // not mixed: straight to set A
      if constexpr (MOM == 3) {
        field(R, 0, GRAUPEL_NUMBER)[i] = f2m.gn; field(R, 0, GRAUPEL_VOLUME)[i] = f2m.gv; field(R, 0, HAIL_NUMBER)[i] = f2m.hn; field(R, 0, HAIL_VOLUME)[i] = f2m.hv;
      }
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(&R.cnt[C_FAILED], 1ull);
    size_t nch = (R.n + CHUNK - 1) / CHUNK;
    blockSumsDF<NW>(whi, wlo, R.part + nch * NCONS * 3 + (size_t)chunk * 4, sh);
  }
}

// Smagorinsky-Lilly eddy viscosities (Turbulence.viscosity, src/core/turbulence.ts:87-137): anisotropic horizontal
// width, cube-root (or dz) vertical width with the per-level explicit cap, dry N^2 or the saturated one in cloud
// (theta-e form; Durran-Klemp when switched on).
__global__ void k_viscosity(const RunDesc* __restrict__ runs, const int4* items, int nitems, int set) {
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    const int nx = R.nx, ny = R.ny, nz = R.nz, layer = R.layer, i0 = items[it].y * CHUNK, i1 = min(R.n, i0 + CHUNK);
    const float* __restrict__ u = field(R, set, U);
    const float* __restrict__ v = field(R, set, V);
    const float* __restrict__ w = field(R, set, W);
    const float* __restrict__ th = field(R, set, THETA);
    const float* __restrict__ qv = field(R, set, Q);
    const float* __restrict__ cl = field(R, set, CLOUD);
    const float* __restrict__ ic = field(R, set, ICE);
    float* __restrict__ km = R.kmkh;
    float* __restrict__ kh = R.kmkh + R.n;
    const bool ice = R.flags & RF_ICE;
    // (the outputs do not alias the inputs, so the loads of two nodes can be issued together)
#pragma unroll 2
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      int z = i / layer, c = i - z * layer, y = c / nx, x = c - y * nx, l = z * layer;
      int e = wrap(x + 1, nx) + y * nx + l, wst = wrap(x - 1, nx) + y * nx + l, n = x + wrap(y + 1, ny) * nx + l, s = x + wrap(y - 1, ny) * nx + l;
      int up = z < nz - 1 ? layer : 0, dn = z > 0 ? -layer : 0;
      float ihx = .5f * R.inv_dx, ihy = .5f * R.inv_dy, isp = lvl(R, L_INV_SPAN, z);
      float dudx = (u[e] - u[wst]) * ihx, dvdy = (v[n] - v[s]) * ihy, dwdz = (w[i + up] - w[i + dn]) * isp;
      float dudy = (u[n] - u[s]) * ihy, dvdx = (v[e] - v[wst]) * ihx;
      float dudz = (u[i + up] - u[i + dn]) * isp, dwdx = (w[e] - w[wst]) * ihx;
      float dvdz = (v[i + up] - v[i + dn]) * isp, dwdy = (w[n] - w[s]) * ihy;
      float a1 = dudy + dvdx, a2 = dudz + dwdx, a3 = dvdz + dwdy;
      float s2 = 2.f * (dudx * dudx + dvdy * dvdy + dwdz * dwdz) + a1 * a1 + a2 * a2 + a3 * a3;
      float n2 = lvl(R, L_G_OVER_THB, z) * ((th[i + up] - th[i + dn]) + lvl(R, L_DTHB, z)) * isp;
      float cond = ice ? cl[i] + ic[i] : cl[i];
      if (cond > 1e-5f) {
        const int zu = z + (up ? 1 : 0), zd = z - (dn ? 1 : 0);
        float condU = ice ? cl[i + up] + ic[i + up] : cl[i + up], condD = ice ? cl[i + dn] + ic[i + dn] : cl[i + dn];
        float Ti = lvl(R, L_THB, z) + th[i], Tu = lvl(R, L_THB, zu) + th[i + up], Td = lvl(R, L_THB, zd) + th[i + dn];
        if ((R.flags & RF_DK) && condU > 1e-5f && condD > 1e-5f) {
          const float LV = 2.5e6f, RD = 287.05f, CP = 1004.f, EPS = .622f;
          float t = Ti * lvl(R, L_EXNER, z), qs = qv[i];
          float factor = (1.f + LV * qs / (RD * t)) / (1.f + EPS * LV * LV * qs / (CP * RD * t * t));
          float dT = (th[i + up] - th[i + dn]) + lvl(R, L_DTHB, z);
          n2 = 9.81f * (factor * (dT / Ti + LV / (CP * t) * (qv[i + up] - qv[i + dn])) - ((qv[i + up] - qv[i + dn]) + (condU - condD))) * isp;
        } else {
          // g / theta_e d theta_e / dz with theta_e = theta exp(L q / (cp theta pi)). The difference of the two
          // theta_e values (~330 K) is formed without cancellation: (theta_u - theta_d) e^xu + theta_d e^xd expm1(xu - xd),
          // theta_u - theta_d from the departures and the base profile's own difference.
          const float L_CP = 2.5e6f / 1004.f;
          float xi = L_CP * qv[i] / (Ti * lvl(R, L_EXNER, z));
          float xu = L_CP * qv[i + up] / (Tu * lvl(R, L_EXNER, zu));
          float xd = L_CP * qv[i + dn] / (Td * lvl(R, L_EXNER, zd));
          float dT = (th[i + up] - th[i + dn]) + lvl(R, L_DTHB, z);
          float eu = expf(xu), ed = expf(xd);
          float dte = dT * eu + Td * ed * expm1f(xu - xd);
          n2 = 9.81f / (Ti * expf(xi)) * dte * isp;
        }
      }
      float rate = sqrtf(fmaxf(0.f, s2 - 3.f * n2));
      float kmv = fminf(lvl(R, L_CAP, z), lvl(R, L_LEN2, z) * rate);
      km[i] = kmv;
      kh[i] = (R.flags & RF_ANISO) ? fminf(R.capH, R.lenH2 * rate) : kmv;
    }
  }
}

// Explicit flux-form diffusion of each mixed field's departure (Turbulence.mix, src/core/turbulence.ts:143-185),
// then the ground drag balanced against the environment's own and rigid w at the ground and top (mixStep, :1179-1194).
// In: set `in`; out: set A. A block takes one tile of columns of one run and a range of levels [z0, z1), marching up:
// per level the planes of the mixed fields and of K_h (1-node periodic halo) arrive in shared memory by asynchronous
// copies issued a level ahead, the vertical neighbours and K_m stay in registers, one barrier per level.
constexpr int MIX_MAXC = 2;  // plane cells per thread: (TX + 2)(TY + 2) <= MIX_MAXC * TX * TY
template <int NM>
__device__ __forceinline__ void mix_item(const RunDesc& R, int tile, int z0, int z1, int in, int TX, int TY, float* sm) {
  const int nx = R.nx, ny = R.ny, nz = R.nz, layer = R.layer;
  const int PW = TX + 2, PH = TY + 2, NCELL = PW * PH, NP = NM + 1;  // planes: the NM fields, then K_h
  const int t = threadIdx.x, lx = t % TX, ly = t / TX;
  const int tilesX = (nx + TX - 1) / TX, x0 = (tile % tilesX) * TX, y0 = (tile / tilesX) * TY;
  const int x = x0 + lx, y = y0 + ly;
  const bool on = x < nx && y < ny;
  const int col = on ? x + y * nx : 0;
  // the fields as 32-bit element offsets from the run's field block (fewer live registers than pointers); plane NM
  // is K_h
  const float* const fld = R.fld;
  const float* const kh = R.kmkh + R.n;
  int so[NM];
#pragma unroll
  for (int k = 0; k < NM; k++) so[k] = (in * NF + mix_field(k)) * (int)R.n;
#define SRC(p) ((p) < NM ? fld + so[(p) < NM ? (p) : 0] : kh)
  const float* km = R.kmkh;
  int off[MIX_MAXC], cell[MIX_MAXC];
#pragma unroll
  for (int j = 0; j < MIX_MAXC; j++) {
    const int e = t + j * blockDim.x;
    cell[j] = e < NCELL ? e : -1;
    const int hy = e / PW, hx = e - hy * PW;
    int gx = x0 + hx - 1, gy = y0 + hy - 1;
    gx = gx < 0 ? gx + nx : (gx >= nx ? gx - nx : gx);
    gy = gy < 0 ? gy + ny : (gy >= ny ? gy - ny : gy);
    off[j] = e < NCELL ? gx + gy * nx : 0;
  }
  // plane z0 into buffer 0; the centre values of z0 - 1, z0, z0 + 1 into registers
#pragma unroll
  for (int p = 0; p < NP; p++)
#pragma unroll
    for (int j = 0; j < MIX_MAXC; j++) if (cell[j] >= 0) sm[p * NCELL + cell[j]] = SRC(p)[off[j] + z0 * layer];
  float below[NM], cur[NM], above[NM];
#pragma unroll
  for (int k = 0; k < NM; k++) {
    cur[k] = SRC(k)[col + z0 * layer];
    below[k] = z0 > 0 ? SRC(k)[col + (z0 - 1) * layer] : 0.f;
    above[k] = z0 + 1 < nz ? SRC(k)[col + (z0 + 1) * layer] : 0.f;
  }
  float kmD = z0 > 0 ? km[col + (z0 - 1) * layer] : 0.f, kmC = km[col + z0 * layer], kmU = z0 + 1 < nz ? km[col + (z0 + 1) * layer] : 0.f;
  __syncthreads();
  const float ix2 = R.inv_dx * R.inv_dx, iy2 = R.inv_dy * R.inv_dy, dt = R.dt;
  const int cc = (ly + 1) * PW + lx + 1;
  for (int z = z0; z < z1; z++) {
    const int buf = (z - z0) & 1;
    const float* P = sm + buf * NP * NCELL;
    // a level ahead: plane z + 1 (asynchronous copies into the other buffer), the centre values of z + 2
    if (z + 1 < z1) {
      float* Q = sm + (buf ^ 1) * NP * NCELL;
#pragma unroll
      for (int p = 0; p < NP; p++)
#pragma unroll
        for (int j = 0; j < MIX_MAXC; j++) if (cell[j] >= 0) cp_async4(Q + p * NCELL + cell[j], SRC(p) + off[j] + (z + 1) * layer);
    }
    float nextv[NM];
    float kmN = 0.f;
    const bool more = z + 2 < nz;
#pragma unroll
    for (int k = 0; k < NM; k++) nextv[k] = more ? SRC(k)[col + (z + 2) * layer] : 0.f;
    if (more) kmN = km[col + (z + 2) * layer];
    if (on) {
      const float* KH = P + NM * NCELL + cc;
      const float khi = KH[0];
      const float hE = .5f * (khi + KH[1]), hW = .5f * (KH[-1] + khi), hN = .5f * (khi + KH[PW]), hS = .5f * (KH[-PW] + khi);
      const float vU = z < nz - 1 ? .5f * (kmC + kmU) * lvl(R, L_MIXUP, z) * lvl(R, L_INV_DZS, z) : 0.f;
      const float vD = z > 0 ? .5f * (kmD + kmC) * lvl(R, L_MIXDN, z) * lvl(R, L_INV_DZS, z - 1) : 0.f;
      float uu = 0.f, vv = 0.f;
      const int i = col + z * layer;
#pragma unroll
      for (int k = 0; k < NM; k++) {
        const int f = mix_field(k);
        const float factor = k < 3 ? 1.f : 3.f;
        const float* A = P + k * NCELL + cc;
        const float ai = cur[k];
        // vertical departures: the base differences to the level above / below (u, v, q carry a base profile;
        // theta' is already a departure; w, cloud, ice, number have none)
        float bu = 0.f, bd = 0.f;
        if (f == U) { bu = z < nz - 1 ? lvl(R, L_DUENV, z) : 0.f; bd = z > 0 ? lvl(R, L_DUENV, z - 1) : 0.f; }
        else if (f == V) { bu = z < nz - 1 ? lvl(R, L_DVENV, z) : 0.f; bd = z > 0 ? lvl(R, L_DVENV, z - 1) : 0.f; }
        else if (f == Q) { bu = z < nz - 1 ? lvl(R, L_DQB, z) : 0.f; bd = z > 0 ? lvl(R, L_DQB, z - 1) : 0.f; }
        const float tx = (hE * (A[1] - ai) - hW * (ai - A[-1])) * ix2;
        const float ty = (hN * (A[PW] - ai) - hS * (ai - A[-PW])) * iy2;
        const float tz = (z < nz - 1 ? vU * ((above[k] - ai) - bu) : 0.f) - (z > 0 ? vD * ((ai - below[k]) - bd) : 0.f);
        float out = ai + dt * factor * (tx + ty + tz);
        if (f == U) uu = out;
        else if (f == V) vv = out;
        else {
          if (f == W && (z == 0 || z == nz - 1)) out = 0.f;
          field(R, 0, f)[i] = out;
        }
      }
      if (z == 0 && R.drag != 0.f) {
        const float ug = uu + R.frame_u, vg = vv + R.frame_v, speed = sqrtf(ug * ug + vg * vg);
        uu -= R.drag * (speed * ug - R.env_speed * R.ue0);
        vv -= R.drag * (speed * vg - R.env_speed * R.ve0);
      }
      field(R, 0, U)[i] = uu; field(R, 0, V)[i] = vv;
    }
#pragma unroll
    for (int k = 0; k < NM; k++) { below[k] = cur[k]; cur[k] = above[k]; above[k] = nextv[k]; }
    kmD = kmC; kmC = kmU; kmU = kmN;
    cp_async_wait_all();
    __syncthreads();
  }
#undef SRC
}

// Work item (run, tile, z0, z1); `TX` x `TY` threads.
__global__ void __launch_bounds__(320, 2) k_mix_tile(const RunDesc* __restrict__ runs, const int4* items, int nitems, int in, int TX, int TY) {
  extern __shared__ float sm[];
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    if (R.flags & RF_ICE) mix_item<NMIX>(R, items[it].y, items[it].z, items[it].w, in, TX, TY, sm);
    else mix_item<6>(R, items[it].y, items[it].z, items[it].w, in, TX, TY, sm);
  }
}

// Per run, once a step: the water budget and negative mass of this step added in a fixed order, the step count,
// the scratch reset for the next step.
__global__ void k_step_end(const RunDesc* __restrict__ runs, const int4* items, int nitems) {
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (threadIdx.x == 0 && !R.cnt[C_FAILED]) {
      const size_t nch = (R.n + CHUNK - 1) / CHUNK;
      double w[3] = {0, 0, 0};
      for (size_t c = 0; c < nch; c++) for (int j = 0; j < 3; j++) w[j] += R.part[nch * NCONS * 3 + c * 4 + j];
      for (int j = 0; j < 3; j++) R.acc[A_WATER + j] += w[j];
      if (R.flags & RF_ELEC) {
        // the charge separated this step (:1126), and the sedimentation's charge reaching the ground (:590)
        double sep = 0, ground = 0;
        for (size_t c = 0; c < nch; c++) sep += R.part[nch * NCONS * 3 + c * 4 + 3];
        const int sedItems = (R.layer + SED_COLS - 1) / SED_COLS;
        for (int c = 0; c < sedItems; c++) ground += R.cpart[c];
        R.acc[A_CHG_SEPARATED] += sep; R.acc[A_CHG_GROUND] += ground; R.acc[A_CHG_PRECIP] += ground;
      }
      R.cnt[C_STEPS] += 1;
    }
    __syncthreads();
    if (threadIdx.x < S_COUNT + 16) R.scr[threadIdx.x] = 0.f;
    __syncthreads();
  }
}

// FP64 max |D R u| over the dual cells of a set (the divergence check).
__global__ void k_divergence_max(const RunDesc* __restrict__ runs, const int4* items, int nitems, int set, double* out) {
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    const int nx = R.nx, ny = R.ny, layer = R.layer, i0 = items[it].y * CHUNK, i1 = min(R.ncells, i0 + CHUNK);
    const float *u = field(R, set, U), *v = field(R, set, V), *w = field(R, set, W);
    double m = 0;
    for (int cidx = i0 + threadIdx.x; cidx < i1; cidx += blockDim.x) {
      int k = cidx / layer, c = cidx - k * layer, y = c / nx, x = c - y * nx;
      int l0 = k * layer, x1 = wrap(x + 1, nx), y1 = wrap(y + 1, ny);
      int a = x + y * nx + l0, b = x1 + y * nx + l0, ee = x + y1 * nx + l0, f = x1 + y1 * nx + l0, g = a + layer, h = b + layer, s = ee + layer, tt = f + layer;
      double r0 = lvl(R, L_RHO, k) / 4.0, r1 = lvl(R, L_RHO, k + 1) / 4.0;
      double ddx = (r0 * ((double)u[b] + u[f] - u[a] - u[ee]) + r1 * ((double)u[h] + u[tt] - u[g] - u[s])) / R.dx;
      double ddy = (r0 * ((double)v[ee] + v[f] - v[a] - v[b]) + r1 * ((double)v[s] + v[tt] - v[g] - v[h])) / R.dy;
      double ddz = (r1 * ((double)w[g] + w[h] + w[s] + w[tt]) - r0 * ((double)w[a] + w[b] + w[ee] + w[f])) / lvl(R, L_DZS, k);
      const double d = fabs(ddx + ddy + ddz);
      m = (d > m || d != d) ? d : m;  // a NaN wins (fmax would drop it)
    }
    for (int o = 16; o > 0; o >>= 1) { const double a = __shfl_xor_sync(0xffffffffu, m, o); m = (a > m || a != a) ? a : m; }
    // the bits of a non-negative double order as unsigned integers; a NaN with its sign cleared orders above +inf
    if ((threadIdx.x & 31) == 0)
      atomicMax(reinterpret_cast<unsigned long long*>(out), (unsigned long long)__double_as_longlong(m) & 0x7fffffffffffffffull);
  }
}

// ==================================================================== packed field transfer
// Moves fields between the runs and one staging buffer that holds, run after run, the selected fields in field
// order (the host copies the whole buffer at once). Item (slot, field, chunk, staging offset of the chunk); theta
// crosses as the full potential temperature (FP64 difference with the base profile).
__global__ void k_pack(const RunDesc* __restrict__ runs, const int4* items, int nitems, float* staging, int write) {
  FOR_ITEMS {
    const int4 w = items[it];
    const RunDesc& R = runs[w.x];
    const int i0 = w.z * CHUNK, i1 = min(R.n, i0 + CHUNK);
    float* f = field(R, 0, w.y);
    float* s = staging + (size_t)(unsigned)w.w;
    const double* thb = R.lv64 + (size_t)D_THB * R.nz;
    if (write) {
      if (w.y == THETA) for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) f[i] = (float)((double)s[i - i0] - thb[i / R.layer]);
      else for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) f[i] = s[i - i0];
    } else {
      if (w.y == THETA) for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) s[i - i0] = (float)((double)f[i] + thb[i / R.layer]);
      else for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) s[i - i0] = f[i];
    }
  }
}

// ==================================================================== launchers

void launch_pack(const Launch& L, float* staging, int write) { k_pack<<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, staging, write); }
void launch_theta_in(const Launch& L, const float* src) { k_theta_in<<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, src); }
void launch_theta_out(const Launch& L, float* dst) { k_theta_out<<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, dst); }
void launch_fall_courant(const Launch& L) { k_fall_courant<<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n); }
void launch_sediment(const Launch& L, int maxnz) {
  k_sediment<<<GRID(L.n, L.cap), SED_COLS, (2 * maxnz * SED_COLS + 3 * maxnz) * sizeof(float), L.stream>>>(L.runs, L.items, L.n);
}
void launch_proj_div_xfft(const Launch& L, int mode, int set, int yc, int maxnx) {
  size_t smem = (size_t)2 * ((yc + 1) / 2) * maxnx * sizeof(float2);
  k_proj_div_xfft<<<GRID(L.n, L.cap), 256, smem, L.stream>>>(L.runs, L.items, L.n, mode, set, yc);
}
void launch_proj_modes(const Launch& L, int mode, int maxnz, int maxny, int threads, int smem_budget) {
  // the column slab [nz][ny] plus a scratch of `group` layers, all of them when they fit
  const size_t slab = (size_t)maxnz * maxny * sizeof(float2);
  int group = (int)std::min<size_t>(maxnz, (smem_budget - slab) / ((size_t)maxny * sizeof(float2)));
  group = std::max(group, 1);
  const size_t smem = slab + (size_t)group * maxny * sizeof(float2);
  k_proj_modes<<<GRID(L.n, L.cap), threads, smem, L.stream>>>(L.runs, L.items, L.n, mode, group);
}
size_t layer_fft_smem(int maxnx, int maxny) {
  return ((size_t)2 * ((maxny + 1) / 2) * maxnx + (size_t)2 * (maxnx / 2 + 1) * maxny + maxnx + maxny) * sizeof(float2);
}
size_t layer_fft_smem_run(int nx, int ny) {
  const bool fast = (nx == 40 && ny == 32) || (nx == 80 && ny == 64);
  if (!fast) return layer_fft_smem(nx, ny);
  // the forward's pair rows (and on 40 x 32 its three staged planes, 1.5 complex words a node), the inverse's columns
  const size_t fwd = (size_t)(ny / 2) * (nx + 1) + (nx == 40 ? (size_t)3 * nx * ny / 2 : 0), inv = (size_t)(nx / 2 + 1) * (ny + 1);
  return ((size_t)nx + ny + std::max(fwd, inv)) * sizeof(float2);
}
void launch_proj_div_fft2(const Launch& L, int mode, int set, size_t smem) {
  k_proj_div_fft2<<<GRID(L.n, L.cap), 256, smem, L.stream>>>(L.runs, L.items, L.n, mode, set);
}
void launch_proj_sweep(const Launch& L, int mode, int maxny) {
  k_proj_sweep<<<GRID(L.n, L.cap), (2 * maxny + 31) / 32 * 32, 0, L.stream>>>(L.runs, L.items, L.n, mode);
}
void launch_proj_ifft2(const Launch& L, int mode, size_t smem) {
  k_proj_ifft2<<<GRID(L.n, L.cap), 256, smem, L.stream>>>(L.runs, L.items, L.n, mode);
}
void launch_proj_xifft(const Launch& L, int mode, int yc, int maxnx) {
  size_t smem = ((size_t)yc * (maxnx / 2 + 1) + (size_t)2 * ((yc + 1) / 2) * maxnx) * sizeof(float2);
  k_proj_xifft<<<GRID(L.n, L.cap), 256, smem, L.stream>>>(L.runs, L.items, L.n, mode, yc);
}
void launch_face_correct(const Launch& L, int set) { k_face_correct<<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, set); }
size_t refine_smem(int TX, int TY) { return ((size_t)2 * (TX + 2) * (TY + 2) + (size_t)12 * (TX + 1) * (TY + 1)) * sizeof(float); }
void launch_refine_residual(const Launch& L, int set, int TX, int TY) {
  if (L.n == 0) return;
  const int threads = ((TX + 1) * (TY + 1) + 31) / 32 * 32;  // a thread per node of the tile and its halo
  if (TX == 20 && TY == 8) k_refine_residual<20, 8><<<GRID(L.n, L.cap), threads, refine_smem(TX, TY), L.stream>>>(L.runs, L.items, L.n, set, TX, TY);
  else k_refine_residual<0, 0><<<GRID(L.n, L.cap), threads, refine_smem(TX, TY), L.stream>>>(L.runs, L.items, L.n, set, TX, TY);
}
void launch_refine_correct(const Launch& L, int set) { k_pres_correct<2><<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, set); }
void launch_pres_correct(const Launch& L, int set, int final_) {
  if (final_) k_pres_correct<1><<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, set);
  else k_pres_correct<0><<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, set);
}

void launch_fill_partial(const Launch& L, int set) { k_fill_partial<<<GRID(L.n, L.cap), 128, 0, L.stream>>>(L.runs, L.items, L.n, set); }
void launch_fill_final(const Launch& L) { k_fill_final<<<GRID(L.n, L.cap), 32, 0, L.stream>>>(L.runs, L.items, L.n); }
void launch_sediment_2m(const Launch& L, int maxnz) {
  const int K = (maxnz + 31) / 32;  // level slots a lane (nz <= 128)
  if (K <= 1) k_sediment_2m<1><<<GRID(L.n, L.cap), SED2_WARPS * 32, 0, L.stream>>>(L.runs, L.items, L.n);
  else if (K == 2) k_sediment_2m<2><<<GRID(L.n, L.cap), SED2_WARPS * 32, 0, L.stream>>>(L.runs, L.items, L.n);
  else if (K == 3) k_sediment_2m<3><<<GRID(L.n, L.cap), SED2_WARPS * 32, 0, L.stream>>>(L.runs, L.items, L.n);
  else k_sediment_2m<4><<<GRID(L.n, L.cap), SED2_WARPS * 32, 0, L.stream>>>(L.runs, L.items, L.n);
}
void launch_physics(const Launch& L, int in, int mid, int variant) {
  if (L.n == 0) return;
  switch (variant) {  // (electrified ? 3 : 0) + moments - 1
    case 0: k_physics<false, 1><<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, in, mid); break;
    case 1: k_physics<false, 2><<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, in, mid); break;
    case 2: k_physics<false, 3><<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, in, mid); break;
    case 3: k_physics<true, 1><<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, in, mid); break;
    case 4: k_physics<true, 2><<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, in, mid); break;
    default: k_physics<true, 3><<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, in, mid); break;
  }
}
void launch_viscosity(const Launch& L, int set) { k_viscosity<<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, set); }
size_t mix_smem(int TX, int TY) { return (size_t)2 * (NMIX + 1) * (TX + 2) * (TY + 2) * sizeof(float); }
void launch_mix(const Launch& L, int in, int TX, int TY) {
  k_mix_tile<<<GRID(L.n, L.cap), TX * TY, mix_smem(TX, TY), L.stream>>>(L.runs, L.items, L.n, in, TX, TY);
}
void launch_step_end(const Launch& L) { k_step_end<<<GRID(L.n, L.cap), 64, 0, L.stream>>>(L.runs, L.items, L.n); }
void launch_divergence_max(const Launch& L, int set, double* out) { k_divergence_max<<<GRID(L.n, L.cap), 256, 0, L.stream>>>(L.runs, L.items, L.n, set, out); }

// The constant tables the kernels read that are made on the host: the Seifert-Beheng sweep coefficients of two-moment
// graupel and hail (FP64, then rounded).
cudaError_t upload_tables() { return cudaMemcpyToSymbol(i2m::c_sweep, &i2m::h_sweep, sizeof(i2m::SweepTable)); }

cudaError_t set_smem_limits(int bytes) {
  cudaError_t e;
  if ((e = smem_limit(k_proj_modes, bytes)) != cudaSuccess) return e;
  if ((e = smem_limit(k_proj_div_xfft, bytes)) != cudaSuccess) return e;
  if ((e = smem_limit(k_proj_xifft, bytes)) != cudaSuccess) return e;
  if ((e = smem_limit(k_sediment, bytes)) != cudaSuccess) return e;
  if ((e = smem_limit(k_proj_div_fft2, bytes)) != cudaSuccess) return e;
  if ((e = smem_limit(k_proj_ifft2, bytes)) != cudaSuccess) return e;
  if ((e = smem_limit(k_refine_residual<0, 0>, bytes)) != cudaSuccess) return e;
  if ((e = smem_limit(k_refine_residual<20, 8>, bytes)) != cudaSuccess) return e;
  return set_transport_smem_limits(bytes);
}

}  // namespace sg
