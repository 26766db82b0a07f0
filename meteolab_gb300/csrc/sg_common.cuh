// Device data layout of the step and the small numerical building blocks shared by the kernels.
//
// HBM layout of one run (all FP32 unless noted, n = nx*ny*nz nodes, node i = x + nx*(y + ny*z)):
//   fld   3 sets x 13 fields x n      set A = the state between steps, B and C = RK3 stage / mixing scratch
//   faces 4 x n                       projected face mass fluxes mx, my, mz and their divergence
//   kmkh  2 x n                       eddy viscosities (vertical km, horizontal kh)
//   phi   n                           face-projection potential
//   pres  nx*ny*(nz-1)                projection pressure (dual cells between node levels)
//   spec  (nx/2+1) x nzc x ny complex x-spectrum of one projection, m-major so a mode slab is contiguous
//   cols  3 x nx*ny                   precipitation, hail on the ground, largest hail
//   lv    L_COUNT x nz                per-level constants (FP32); lv64: per-level FP64 (tridiagonal coefficients)
//   tri_face/tri_pres  (invpiv, cp) FP64 per (m, k, n) of the two tridiagonal factorisations
// theta is carried as its departure from the base profile theta_b(z) (the full value only at the ABI boundary).
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define SG_HD __host__ __device__ __forceinline__
#define SG_D __device__ __forceinline__
#else
#define SG_HD inline
#define SG_D inline
#endif

namespace sg {

constexpr int NF = 13;  // carried fields
enum Field { RAIN = 0, SNOW, GRAUPEL, HAIL, U, V, W, THETA, Q, CLOUD, ICE, ICENUM, COLD };
// WENO5 for the water species and the cold-pool indicator, linear fifth-order upwind for u, v, w, theta
// (src/core/model.ts:1320-1328).
SG_HD bool monotone(int f) { return !(f == U || f == V || f == W || f == THETA); }
// The positivity fix applies to rain, snow, graupel, hail, vapour, cloud water, cloud ice (`water(...)`).
constexpr int NCONS = 7;
__host__ __device__ constexpr int cons_field(int k) { return k < 4 ? k : (k == 4 ? Q : k == 5 ? CLOUD : ICE); }
// The fields the turbulence mixes (src/core/model.ts:1338-1344), in mixed() order.
constexpr int NMIX = 8;
__host__ __device__ constexpr int mix_field(int k) { return k < 3 ? U + k : (k == 3 ? THETA : k == 4 ? Q : k == 5 ? CLOUD : k == 6 ? ICE : ICENUM); }

// Per-level FP32 constants (host-computed in FP64).
enum Level {
  L_RHO, L_INV_RHO, L_HZ, L_INV_HZ, L_DZS, L_INV_DZS, L_RUP, L_EXNER, L_P, L_THB, L_QB, L_UENV, L_VENV, L_THVENV, L_ZS,
  L_TH_UP_POS, L_TH_UP_NEG, L_TH_DN_POS, L_TH_DN_NEG,   // base-theta face values minus theta_b(z) (profile tendency)
  L_LEN2, L_CAP, L_INV_SPAN, L_DTHB, L_G_OVER_THB,      // turbulence: filter width^2, cap, 1/span, theta_b(up)-theta_b(down)
  L_MIXUP, L_MIXDN,                                     // rUp/(rho h) above, rUp(below)/(rho h)
  L_DUENV, L_DVENV, L_DQB,                              // base differences to the level above (mixing)
  L_FALLSQ,                                             // sqrt(rho_ground / rho)
  L_SPONGE,                                             // sponge rate * dt share (0 below the sponge)
  L_NODEMASS,                                           // dx dy hz rho (water budget)
  L_LW,                                                 // level weight hz/dz rho (positivity fix)
  L_SURF,                                               // surface flux share per metre (sharesAbove)
  L_TCB,                                                // theta_b exner - 273.15 (Celsius base temperature)
  L_QW_HI, L_QW_LO, L_BW, L_QI_HI, L_QI_LO, L_BI, L_Q0_HI, L_Q0_LO,  // saturation bases (sg_physics.cuh Level)
  L_COUNT
};
// Per-level FP64 constants.
enum Level64 { D_FLO, D_FHZ, D_PL1, D_PL2, D_THB, D_COUNT };

struct RunDesc {
  int nx, ny, nz, layer, n, nm, mh, ncells;
  int fx_nf, fy_nf, fx_rad[8], fy_rad[8];  // FFT radix plans of nx and ny
  int slot, flags, pad0, pad1;
  float dx, dy, inv_dx, inv_dy, dt, height;
  float coriolis, keep, sponge_start, cs, drag, frame_u, frame_v, ue0, ve0, env_speed, lenH2, capH, rho0;
  float* fld;
  float* faces;
  float* kmkh;
  float* phi;
  float* pres;
  float2* spec;
  float* cols;
  const float* lv;
  const double* lv64;
  const double2* tri_face;
  const double2* tri_pres;
  const double2* ab;       // pressure symbols (alpha, beta) per mode [m][n]
  const float2* twx;       // exp(-2 pi i t / nx), t < nx
  const float2* twy;       // exp(-2 pi i t / ny)
  float* scr;              // per-step scratch: courant[4], fill delta[7], ...
  double* part;            // FP64 partial sums (positivity fix, water budget)
  double* acc;             // FP64 running totals: negativeFilled, water[4]
  unsigned long long* cnt; // counters: clipped, steps, failed flag
};
enum RunFlags { RF_LOADING = 1, RF_EVAP = 2, RF_RAINFORM = 4, RF_ANISO = 8, RF_VDZ = 16, RF_DK = 32, RF_STAGES = 64, RF_ICE = 128 };
// scr layout
enum Scratch { S_COURANT = 0, S_FILL = 4, S_COUNT = 16 };
// cnt layout
enum Counter { C_CLIPPED = 0, C_STEPS = 1, C_FAILED = 2, C_COUNT = 4 };
// acc layout
enum Acc { A_NEG = 0, A_WATER = 1, A_COUNT = 8 };
// partial-sum layout (per run): fill partials [chunk][7][3], then water partials [chunk][4].
constexpr int CHUNK = 4096;   // nodes per pointwise work item

SG_HD float lvl(const RunDesc& R, int which, int z) { return R.lv[which * R.nz + z]; }
SG_HD float* field(const RunDesc& R, int set, int f) { return R.fld + ((size_t)set * NF + f) * R.n; }

// ---------------------------------------------------------------- reconstructions (src/core/advection.ts:385-399)
// Linear fifth-order upwind value at the face between c and d for flow from a towards e.
SG_HD float upwind5(float a, float b, float c, float d, float e) {
  return (2.f * a - 13.f * b + 47.f * c + 27.f * d - 3.f * e) * (1.f / 60.f);
}

// WENO5 (Jiang & Shu weights with the reference's scale-aware epsilon 2e-7 * sum q^2). The five values are first
// scaled by an exact power of two that brings the largest to [1, 2): the weights are scale-free, so this changes
// nothing in exact arithmetic, and in FP32 it keeps the squared products of water contents of 1e-6 kg/kg away from
// underflow. All-zero input gives 0 exactly (the reference's early return).
SG_HD float weno5(float a, float b, float c, float d, float e) {
  float s = fmaxf(fmaxf(fabsf(a), fabsf(b)), fmaxf(fmaxf(fabsf(c), fabsf(d)), fabsf(e)));
#ifdef __CUDA_ARCH__
  int ex = (__float_as_int(s) >> 23) & 0xff;
#else
  int ex; { union { float f; int i; } u; u.f = s; ex = (u.i >> 23) & 0xff; }
#endif
  if (ex == 0) return 0.f;  // all zero (or below 1.2e-38)
  float down, up;
#ifdef __CUDA_ARCH__
  down = __int_as_float((254 - ex) << 23); up = __int_as_float(ex << 23);
#else
  { union { float f; int i; } u; u.i = (254 - ex) << 23; down = u.f; u.i = ex << 23; up = u.f; }
#endif
  a *= down; b *= down; c *= down; d *= down; e *= down;
  const float sixth = 1.f / 6.f;
  float p0 = (2.f * a - 7.f * b + 11.f * c) * sixth, p1 = (-b + 5.f * c + 2.f * d) * sixth, p2 = (2.f * c + 5.f * d - e) * sixth;
  float s0 = a - 2.f * b + c, t0 = a - 4.f * b + 3.f * c, s1 = b - 2.f * c + d, t1 = b - d, s2 = c - 2.f * d + e, t2 = 3.f * c - 4.f * d + e;
  float eps = 2e-7f * (a * a + b * b + c * c + d * d + e * e);
  const float k13 = 13.f / 12.f;
  float b0 = eps + k13 * s0 * s0 + .25f * t0 * t0, b1 = eps + k13 * s1 * s1 + .25f * t1 * t1, b2 = eps + k13 * s2 * s2 + .25f * t2 * t2;
  float c0 = b0 * b0, c1 = b1 * b1, c2 = b2 * b2;
  float w0 = .1f * c1 * c2, w1 = .6f * c0 * c2, w2 = .3f * c0 * c1;
  float num = w0 * p0 + w1 * p1 + w2 * p2, den = w0 + w1 + w2;
#ifdef __CUDA_ARCH__
  return __fdividef(num, den) * up;
#else
  return num / den * up;
#endif
}

SG_HD int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
SG_HD int clampi(int i, int lo, int hi) { return i < lo ? lo : (i > hi ? hi : i); }

}  // namespace sg
