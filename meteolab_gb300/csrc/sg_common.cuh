// Device data layout of the step and the small numerical building blocks shared by the kernels.
//
// HBM layout of one run (all FP32 unless noted, n = nx*ny*nz nodes, node i = x + nx*(y + ny*z)):
//   fld   3 sets x 13 fields x n      set A = the state between steps, B and C = RK3 stage / mixing scratch; an
//                                     electrified or two-moment run's 3 sets x 5 extra fields x n after them
//   faces 4 x n                       projected face mass fluxes mx, my, mz and their divergence
//   kmkh  2 x n                       eddy viscosities (vertical km, horizontal kh)
//   phi   n                           face-projection potential
//   pres  nx*ny*(nz-1)                projection pressure (dual cells between node levels)
//   spec  (nx/2+1) x nzc x ny complex x-spectrum of one projection, m-major so a mode slab is contiguous
//   cols  3 x nx*ny                   precipitation, hail on the ground, largest hail
//   lv    L_COUNT x nz                per-level constants (FP32); lv64: per-level FP64 (tridiagonal coefficients)
//   tri_face/tri_pres  (TriAB, then cp in FP64) per (m, k, n) of the two tridiagonal factorisations
// theta is carried as its departure from the base profile theta_b(z) (the full value only at the ABI boundary).
#pragma once
#include <stdint.h>
#include <cmath>
#include <cstring>

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
// An electrified run also carries the charge on the ice-snow, graupel-hail, rain and droplet-ion carriers (C/kg,
// src/core/model.ts:210), a two-moment run the raindrop number (per kg, :194) and with two-moment graupel and hail
// their number and particle volume (:202): WENO fields without the positivity fix, not mixed (:1323-1324, :1331,
// :1338-1344). Such a run's sets hold all nine extra fields (NXE) after the 13 base fields'.
constexpr int NXE = 9, NFE = NF + NXE;
enum ExtraField { CHARGE_ICE = 13, CHARGE_GRAUPEL, CHARGE_RAIN, CHARGE_AIR, RAIN_NUMBER, GRAUPEL_NUMBER, GRAUPEL_VOLUME, HAIL_NUMBER, HAIL_VOLUME };
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
  L_NODEMASS_LO, L_LW_LO,                               // their FP32 rounding errors (compensated sums)
  L_SURF,                                               // surface flux share per metre (sharesAbove)
  L_TCB,                                                // theta_b exner - 273.15 (Celsius base temperature)
  L_QW_HI, L_QW_LO, L_BW, L_QI_HI, L_QI_LO, L_BI, L_Q0_HI, L_Q0_LO,  // saturation bases (sg_physics.cuh Level)
  L_RHO_LO, L_INV_DZS_LO, L_INV_HZ_LO,                 // FP32 rounding errors of rho, 1/dzs, 1/hz (refinement)
  L_WLO, L_WLO_LO, L_WHI, L_WHI_LO,                     // dzs(k-1)/hz, dzs(k)/hz as FP32 pairs (refinement)
  L_COUNT
};
// Per-level FP64 constants.
enum Level64 { D_FLO, D_FHZ, D_PL1, D_PL2, D_THB, D_COUNT };

// One mode's forward-sweep coefficients at one level: d_k = a r_k - b d_(k-1), a = (row scale) / pivot in FP32 (it
// multiplies the FP32 right-hand side, rounded once like that value itself), b = lower / pivot in FP64.
struct TriAB { double b; float a; float pad; };
static_assert(sizeof(TriAB) == 16, "one 16-byte load a level");

struct RunDesc {
  int nx, ny, nz, layer, n, nm, mh, ncells;
  int fx_nf, fy_nf, fx_rad[8], fy_rad[8];  // FFT radix plans of nx and ny
  int slot, flags, nf, breakup;  // nf: the run's field ids (NF, or NFE with the extra fields); breakup: two-moment rain's
  float dx, dy, inv_dx, inv_dy, dt, height;
  float inv_dx_lo, inv_dy_lo, inv_dt, inv_dt_lo;      // FP32 rounding errors of 1/dx, 1/dy; 1/dt as a pair
  float coriolis, keep, sponge_start, cs, drag, frame_u, frame_v, ue0, ve0, env_speed, lenH2, capH, rho0;
  float* fld;
  float* faces;
  float* kmkh;
  float* phi;
  float* pres;
  float* pres2;            // the refinement's pressure correction (the projection's pressure is pres + pres2)
  float2* spec;
  float* cols;
  const float* lv;
  const double* lv64;
  const TriAB* tri_face;
  const TriAB* tri_pres;
  const double2* ab;       // pressure symbols (alpha, beta) per mode [m][n]
  const float2* twx;       // exp(-2 pi i t / nx), t < nx
  const float2* twy;       // exp(-2 pi i t / ny)
  float* scr;              // per-step scratch: courant[4], fill delta[7], ...
  double* part;            // FP64 partial sums (positivity fix, water budget)
  double* acc;             // FP64 running totals: negativeFilled, water[4]
  unsigned long long* cnt; // counters: clipped, steps, failed flag
  // per-run diagnostics (RF_ROTATION): columns [DG_COUNT][layer] and the rotation state and accumulators
  float* diag;
  double* rot;
  int uh_z0, uh_z1, uh_top1, uh_top3;  // 2-5 km levels, the last levels at or below 1 and 3 km (src/core/model.ts:389, :1612)
  int core_lo, core_hi;                // the cloudy-core levels of countCores (:1653)
  float meso_zeta;                     // mesoCoreZeta(dx) (:129)
  float pad2;
  // electrified or two-moment runs: the step-start fall speeds [6][n] (ice-snow and graupel-hail charge carriers, rain,
  // snow, rain's number- and reflectivity-weighted), with two-moment graupel and hail [12][n] (then also graupel's mass-,
  // number- and reflectivity-weighted, and hail's: V_MASS_G...), the vertical field of the last solve [n] (V/m, for the
  // inductive charging), the sedimentation's charge reaching the ground per work item
  float* vfall;
  float* ez;
  double* cpart;
};
enum RunFlags { RF_LOADING = 1, RF_EVAP = 2, RF_RAINFORM = 4, RF_ANISO = 8, RF_VDZ = 16, RF_DK = 32, RF_STAGES = 64, RF_ICE = 128,
                RF_REFINE = 256, RF_ROTATION = 512, RF_ELEC = 1024, RF_RAIN2M = 2048, RF_ICE2M = 4096 };
constexpr int RF_EXTRA = RF_ELEC | RF_RAIN2M | RF_ICE2M;  // a run with the extra fields
// vfall rows: the charge carriers', rain's mass-, snow's, rain's number- and reflectivity-weighted speeds; then
// two-moment graupel's and hail's mass-, number- and reflectivity-weighted ones
enum FallRow { V_CHG_ICE = 0, V_CHG_GRAUPEL, V_RAIN, V_SNOW, V_RAIN_N, V_RAIN_Z, V_GRAUPEL, V_GRAUPEL_N, V_GRAUPEL_Z, V_HAIL, V_HAIL_N, V_HAIL_Z };
// diag columns: the UH column, the core sums, the swaths, the core labels; then the ground columns of a sample
enum DiagColumn { DG_UH = 0, DG_COREW, DG_COREWZ, DG_GUST_MAX, DG_UH_MAX, DG_LABEL, DG_RATE, DG_HAIL, DG_GUST, DG_THV, DG_MASK, DG_COUNT };
// rot layout (doubles): the rotation state (src/core/model.ts:263), the run's model time, then the step's keys and the
// sample's maxima (stored as 64-bit keys: non-negative values order as their bits)
enum RotSlot { R_UH = 0, R_X, R_Y, R_ANTI, R_PERSISTED, R_UH01, R_UH03, R_LOW, R_CZETA, R_CUH, R_CANTI, R_TIME,
               K_UH = 12, K_01, K_MIN, K_03,
               M_UP = 16, M_DOWN, M_CLOUD, M_TOP, M_THERMAL, M_COLD, R_COUNT = 24 };
// scr layout
// S_CCOURANT: the three falling charges; S_R2M, S_G2M, S_H2M: two-moment rain's, graupel's and hail's fall (mass and
// reflectivity speeds)
enum Scratch { S_COURANT = 0, S_FILL = 4, S_CCOURANT = 11, S_R2M = 14, S_G2M = 15, S_H2M = 16, S_COUNT = 18 };
// cnt layout
// C_TIMEOUT: a kernel's bounded wait for its own asynchronous copies ran out (the run is then failed too)
enum Counter { C_CLIPPED = 0, C_STEPS = 1, C_FAILED = 2, C_TIMEOUT = 3, C_COUNT = 4 };
// acc layout
// A_CHG_*: the charge budget (AtmosphereModel.chargeGround and .charge, src/core/model.ts:218-224), C; A_FLASH_*: counts
enum Acc { A_NEG = 0, A_WATER = 1, A_CHG_GROUND = 8, A_CHG_SEPARATED, A_CHG_IC, A_CHG_CG_NEG, A_CHG_CG_POS, A_CHG_PRECIP, A_CHG_CONDUCTION,
           A_FLASH_IC, A_FLASH_CG, A_COUNT = 24 };
// partial-sum layout (per run): fill partials [chunk][7][3], then water partials [chunk][4].
constexpr int CHUNK = 4096;   // nodes per pointwise work item

SG_HD float lvl(const RunDesc& R, int which, int z) { return R.lv[which * R.nz + z]; }
// Set s of the 13 base fields is fld[s * 13 n ...]; an electrified run's charge carriers follow the three sets,
// four fields a set, so the base fields keep their offsets (and the hot kernels their constant strides).
SG_HD float* field(const RunDesc& R, int set, int f) {
  return f < NF ? R.fld + ((size_t)set * NF + f) * R.n : R.fld + ((size_t)3 * NF + (size_t)set * NXE + (f - NF)) * R.n;
}

// ---- face reconstruction. Every operation is an explicitly rounded one (no contraction left to the compiler), so
// a face gets the same bits whether it is computed alone (Op1, here and on the host) or paired with another face on
// Blackwell's packed FP32 pipes (Op2, in the transport kernel).
struct Op1 {
  using T = float;
#ifdef __CUDA_ARCH__
  static __device__ __forceinline__ T mul(T a, T b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ T fma(T a, T b, T c) { return __fmaf_rn(a, b, c); }
  static __device__ __forceinline__ T add(T a, T b) { return __fadd_rn(a, b); }
#else
  static T mul(T a, T b) { return a * b; }
  static T fma(T a, T b, T c) { return std::fma(a, b, c); }
  static T add(T a, T b) { return a + b; }
#endif
  SG_HD static T k(float v) { return v; }
};

// WENO5 on values already scaled so the largest is in [1, 2) (the Jiang-Shu weights with the reference's scale-aware
// epsilon 2e-7 sum q^2, src/core/advection.ts:388-399), written about the centre value c: the face value is
// c + num / den, where num / den is the weighted average of the three candidates' departures from c. In exact
// arithmetic this is the reference's sum w_k p_k / sum w_k; in FP32 a uniform stencil gives c exactly (all departures
// are 0) and smooth data keep the rounding of the small correction only. alpha_k = d_k / beta_k^2 is multiplied
// through by the three beta^2, so one division remains.
template <class O>
SG_HD void weno_core(typename O::T a, typename O::T b, typename O::T c, typename O::T d, typename O::T e, typename O::T& num,
                     typename O::T& den) {
  using T = typename O::T;
  const T m1 = O::k(-1.f), two = O::k(2.f), m2 = O::k(-2.f), m4 = O::k(-4.f);
  const T da = O::fma(c, m1, a), db = O::fma(c, m1, b), dd = O::fma(c, m1, d), de = O::fma(c, m1, e);
  // six times the candidates' departures from c: p0 = (2a - 7b + 11c)/6, p1 = (-b + 5c + 2d)/6, p2 = (2c + 5d - e)/6
  const T p0 = O::fma(O::k(-7.f), db, O::mul(two, da));
  const T p1 = O::fma(two, dd, O::mul(m1, db));
  const T p2 = O::fma(m1, de, O::mul(O::k(5.f), dd));
  // smoothness: s0 = a - 2b + c, t0 = a - 4b + 3c, s1 = b - 2c + d, t1 = b - d, s2 = c - 2d + e, t2 = 3c - 4d + e
  const T s0 = O::fma(m2, db, da), t0 = O::fma(m4, db, da);
  const T s1 = O::add(db, dd), t1 = O::fma(m1, dd, db);
  const T s2 = O::fma(m2, dd, de), t2 = O::fma(m4, dd, de);
  const T eps = O::mul(O::k(2e-7f), O::fma(e, e, O::fma(d, d, O::fma(c, c, O::fma(b, b, O::mul(a, a))))));
  const T k13 = O::k(13.f / 12.f), q4 = O::k(.25f);
  const T b0 = O::fma(O::mul(k13, s0), s0, O::fma(O::mul(q4, t0), t0, eps));
  const T b1 = O::fma(O::mul(k13, s1), s1, O::fma(O::mul(q4, t1), t1, eps));
  const T b2 = O::fma(O::mul(k13, s2), s2, O::fma(O::mul(q4, t2), t2, eps));
  const T c0 = O::mul(b0, b0), c1 = O::mul(b1, b1), c2 = O::mul(b2, b2);
  const T w0 = O::mul(O::mul(O::k(.1f), c1), c2), w1 = O::mul(O::mul(O::k(.6f), c0), c2), w2 = O::mul(O::mul(O::k(.3f), c0), c1);
  num = O::fma(w2, p2, O::fma(w1, p1, O::mul(w0, p0)));
  den = O::mul(O::k(6.f), O::add(O::add(w0, w1), w2));
}

SG_HD int float_bits(float v) {
#ifdef __CUDA_ARCH__
  return __float_as_int(v);
#else
  union { float f; int i; } u; u.f = v; return u.i;
#endif
}
SG_HD float bits_float(int v) {
#ifdef __CUDA_ARCH__
  return __int_as_float(v);
#else
  union { float f; int i; } u; u.i = v; return u.f;
#endif
}
SG_HD float div_fast(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdividef(a, b);
#else
  return a / b;
#endif
}
// FP32 <-> FP64 conversions on the integer pipes (GB300 runs FP64, conversions included, at a small fraction of its
// FP32 rate; the tridiagonal solves convert every value in and out). Bit manipulation of the IEEE 754 formats:
// exact widening, and narrowing with round-to-nearest-even, for normal FP32 values and zeros; anything else (FP32
// subnormals, out-of-range, Inf, NaN) takes the hardware conversion.
SG_HD uint32_t dbl_hi(double d) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__double2hiint(d);
#else
  uint64_t u; std::memcpy(&u, &d, 8); return (uint32_t)(u >> 32);
#endif
}
SG_HD uint32_t dbl_lo(double d) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__double2loint(d);
#else
  uint64_t u; std::memcpy(&u, &d, 8); return (uint32_t)u;
#endif
}
SG_HD double dbl_make(uint32_t hi, uint32_t lo) {
#ifdef __CUDA_ARCH__
  return __hiloint2double((int)hi, (int)lo);
#else
  uint64_t u = ((uint64_t)hi << 32) | lo; double d; std::memcpy(&d, &u, 8); return d;
#endif
}
SG_HD double widen(float f) {
  const uint32_t b = (uint32_t)float_bits(f), mag = b & 0x7fffffffu;
  if (mag == 0) return dbl_make(b, 0);                                    // signed zero
  if (mag - 0x00800000u >= 0x7f000000u) return (double)f;                 // subnormal, Inf, NaN
  return dbl_make((b & 0x80000000u) | ((mag >> 3) + (896u << 20)), mag << 29);  // exponent rebias 127 -> 1023
}
SG_HD float narrow(double d) {
  const uint32_t hi = dbl_hi(d), lo = dbl_lo(d), e = (hi >> 20) & 0x7ffu;
  if (((hi & 0x7fffffffu) | lo) == 0) return bits_float((int)(hi & 0x80000000u));  // signed zero
  if (e - 897u > 253u) return (float)d;                                   // outside the normal FP32 range
  const uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29), rest = lo & 0x1fffffffu;
  uint32_t bits = (hi & 0x80000000u) | ((e - 896u) << 23) | m;
  if (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) bits += 1;  // a carry moves into the exponent
  return bits_float((int)bits);
}

// Biased exponent of the largest magnitude of a stencil; the values are scaled by the exact power of two that brings
// it to [1, 2). The weights are scale-free, so this changes nothing in exact arithmetic, and in FP32 it keeps the
// eighth powers inside the weights away from underflow for water contents of 1e-6 kg/kg.
// The exponent is kept in place (the bits of 2^(e - 127)): the scale down is 2^(127 - e) = bits 0x7f000000 - those, the
// scale back up those bits themselves.
SG_HD int weno_exponent(float a, float b, float c, float d, float e) {
  const float s = fmaxf(fmaxf(fabsf(a), fabsf(b)), fmaxf(fmaxf(fabsf(c), fabsf(d)), fabsf(e)));
  return float_bits(s) & 0x7f800000;
}
SG_HD float weno_down(int m) { return bits_float((int)(0x7f000000u - (uint32_t)m)); }
// WENO5 of one face. All-zero input (or all below 1.2e-38) gives 0, the reference's early return.
SG_HD float weno5(float a, float b, float c, float d, float e) {
  const int ex = weno_exponent(a, b, c, d, e);
  if (ex == 0) return 0.f;
  const float down = weno_down(ex), up = bits_float(ex);
  float num, den;
  weno_core<Op1>(Op1::mul(a, down), Op1::mul(b, down), Op1::mul(c, down), Op1::mul(d, down), Op1::mul(e, down), num, den);
  return Op1::fma(div_fast(num, den), up, c);
}
// Linear fifth-order upwind (advection.ts:385): (2a - 13b + 47c + 27d - 3e) / 60.
template <class O>
SG_HD typename O::T upwind_core(typename O::T a, typename O::T b, typename O::T c, typename O::T d, typename O::T e) {
  return O::mul(O::fma(O::k(-3.f), e, O::fma(O::k(27.f), d, O::fma(O::k(47.f), c, O::fma(O::k(-13.f), b, O::mul(O::k(2.f), a))))),
                O::k(1.f / 60.f));
}
SG_HD float upwind5(float a, float b, float c, float d, float e) { return upwind_core<Op1>(a, b, c, d, e); }

SG_HD int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
SG_HD int clampi(int i, int lo, int hi) { return i < lo ? lo : (i > hi ? hi : i); }

}  // namespace sg
