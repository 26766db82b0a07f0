// The RK3 transport kernels of the StormLab step (FluxTransport.tendency and the RK3 update) for sm_103a, in their own
// translation unit: one kernel per field kind, group size and register budget, each compiled for the autotuner's
// candidate tiles with constant strides and once for a tile given at run time.
#include <cuda_runtime.h>
#include <math.h>
#include "sg_common.cuh"
#include "sg_kernels.h"
#include "sg_device.cuh"
#include "sg_tile_copies.cuh"

namespace sg {

// ==================================================================== RK3 transport
// A group of G fields of one run on a TX x TY tile of columns, marching up the column: the tendency
// -(div F - q div)/rho0 of the flux-form WENO5 (monotone fields) or linear fifth-order upwind reconstruction on the
// projected face fluxes (FluxTransport.tendency, src/core/advection.ts:274-378), w with the stage buoyancy
// (stageBuoyancy, model.ts:1204), theta' with the base profile's own vertical flux tendency, then the RK3 update
// a = start + f dt tend (:1250) and, before a stage projection, w = 0 on the ground and the top (:1045).
// Each field's planes z-3..z+3 (clamped at the ground and top, with a 3-node periodic halo) sit in a 7-slot ring in
// shared memory; per level one new plane per field arrives by asynchronous copies issued before the level's
// arithmetic, every thread reconstructs the east and north faces of its own cell (as one packed pair) and the top face,
// threads 0..TY-1 and TY..TY+TX-1 reconstruct the tile's west and south edge faces, the x and y faces are exchanged
// through shared memory (double-buffered), and one barrier separates the levels. The group shares the face-flux loads.
constexpr int TMAXC = 4;  // plane cells per thread: (TX + 6)(TY + 6) <= TMAXC * TX * TY
// Per-level constants staged in shared memory, rows of MAXNZ: 1/hz, 1/rho (both kinds), theta's four base-profile
// face values, thb, qb, thv_env (dynamics).
constexpr int tlv_rows(int kind) { return kind == TK_DYN ? 9 : 2; }
// Field groups of the transport work items: 0-2 the WENO fields in threes, 3 the dynamics {u, v, w, theta'}, 4-12
// the WENO fields one by one, 13-16 the charge carriers of an electrified run, 17 the raindrop number of a two-moment
// run and 18-21 the graupel and hail numbers and volumes of a two-moment ice run, one by one; 22-24 extra fields in
// threes (the first three charge carriers; the drop number with graupel's number and volume; hail's number and volume
// with the ions' charge).
constexpr int TGROUPS = 25;
__constant__ int TGROUP[TGROUPS][4] = {{RAIN, SNOW, GRAUPEL, -1}, {HAIL, Q, CLOUD, -1}, {ICE, ICENUM, COLD, -1}, {U, V, W, THETA},
                                       {RAIN, -1, -1, -1}, {SNOW, -1, -1, -1}, {GRAUPEL, -1, -1, -1}, {HAIL, -1, -1, -1},
                                       {Q, -1, -1, -1}, {CLOUD, -1, -1, -1}, {ICE, -1, -1, -1}, {ICENUM, -1, -1, -1}, {COLD, -1, -1, -1},
                                       {CHARGE_ICE, -1, -1, -1}, {CHARGE_GRAUPEL, -1, -1, -1}, {CHARGE_RAIN, -1, -1, -1}, {CHARGE_AIR, -1, -1, -1},
                                       {RAIN_NUMBER, -1, -1, -1}, {GRAUPEL_NUMBER, -1, -1, -1}, {GRAUPEL_VOLUME, -1, -1, -1},
                                       {HAIL_NUMBER, -1, -1, -1}, {HAIL_VOLUME, -1, -1, -1},
                                       {CHARGE_ICE, CHARGE_GRAUPEL, CHARGE_RAIN, -1}, {RAIN_NUMBER, GRAUPEL_NUMBER, GRAUPEL_VOLUME, -1},
                                       {HAIL_NUMBER, HAIL_VOLUME, CHARGE_AIR, -1}};

// Two faces at once on the packed FP32 pipes (bit-identical per face to the scalar weno5 / upwind5).
struct Op2 {
  using T = float2;
  static __device__ __forceinline__ T mul(T a, T b) { return __fmul2_rn(a, b); }
  static __device__ __forceinline__ T fma(T a, T b, T c) { return __ffma2_rn(a, b, c); }
  static __device__ __forceinline__ T add(T a, T b) { return __fadd2_rn(a, b); }
  static __device__ __forceinline__ T k(float v) { return make_float2(v, v); }
};
__device__ __forceinline__ float2 weno2(float2 a, float2 b, float2 c, float2 d, float2 e) {
  const int ex = weno_exponent(a.x, b.x, c.x, d.x, e.x), ey = weno_exponent(a.y, b.y, c.y, d.y, e.y);
  if ((ex | ey) == 0) return make_float2(0.f, 0.f);  // a warp of empty stencils skips the weights
  const float2 down = make_float2(weno_down(ex), weno_down(ey));
  float2 num, den;
  weno_core<Op2>(__fmul2_rn(a, down), __fmul2_rn(b, down), __fmul2_rn(c, down), __fmul2_rn(d, down), __fmul2_rn(e, down), num, den);
  return make_float2(ex ? __fmaf_rn(__fdividef(num.x, den.x), __int_as_float(ex), c.x) : 0.f,
                     ey ? __fmaf_rn(__fdividef(num.y, den.y), __int_as_float(ey), c.y) : 0.f);
}
template <int KIND>
__device__ __forceinline__ float recon1(float a, float b, float c, float d, float e) {
  if (KIND == TK_WENO) return weno5(a, b, c, d, e);
  return upwind5(a, b, c, d, e);
}
template <int KIND>
__device__ __forceinline__ float2 recon2(float2 a, float2 b, float2 c, float2 d, float2 e) {
  if (KIND == TK_WENO) return weno2(a, b, c, d, e);
  return upwind_core<Op2>(a, b, c, d, e);
}

// The upwind stencil of a face along one axis (stride s) whose low-side cell is at P[-1] and high-side cell at P[0]:
// for flow towards +axis the cells -3..1, else 2..-2 (mirrored).
__device__ __forceinline__ void face_stencil(const float* P, int s, bool pos, float& a, float& b, float& c, float& d, float& e) {
  if (pos) { a = P[-3 * s]; b = P[-2 * s]; c = P[-s]; d = P[0]; e = P[s]; }
  else { a = P[2 * s]; b = P[s]; c = P[0]; d = P[-s]; e = P[-2 * s]; }
}

// CTX x CTY: the tile as compile-time constants (every plane stride and stencil offset an immediate), or 0 x 0 for a
// tile given at run time (TXr x TYr). EW: the block has two more warps, whose 64 lanes take the tile's west and south
// edge faces (one face a lane) while the TX x TY column threads take only their own cells' faces; without it the
// first TY + TX column threads take the edges too, and their warps do up to 40% more reconstructions than the rest
// of the block waits for at every level's barrier.
constexpr int TEDGE = 64;  // edge threads of an EW block
template <int KIND, int G, int CTX, int CTY, bool EW>
__device__ __forceinline__ void transport_item(const RunDesc& Rg, int group, int tile, int in_set, int out_set, float frac, int stage,
                                               int TXr, int TYr, float* sm) {
  const int TX = CTX ? CTX : TXr, TY = CTY ? CTY : TYr;
  const int nx = Rg.nx, ny = Rg.ny, nz = Rg.nz, layer = Rg.layer;
  const size_t n = Rg.n;
  const float inv_dx = Rg.inv_dx, inv_dy = Rg.inv_dy, fdt = frac * Rg.dt;
  const int flags = Rg.flags;
  const float4* __restrict__ F4 = reinterpret_cast<const float4*>(Rg.faces);
  const float* __restrict__ inb = Rg.fld + (size_t)in_set * NF * n;   // the input set (buoyancy)
  // the group's fields as 32-bit element offsets from the run's field block (input set, step-start set A, output
  // set): fewer live registers than a pointer per field and set
  float* const fld = Rg.fld;
  int fo[G];
#pragma unroll
  // an extra field's sets follow the base fields' three, NXE fields a set: its offsets are shifted by `so` so the same
  // set arithmetic addresses it
  // (extra fields come one an item, or three an item without the edge warps: the base kernels keep compile-time offsets)
  const bool chg = (G == 1 || !EW) && group >= 13;
  const int so = chg ? (3 * NF - NF) * (int)n : 0, ss = chg ? NXE * (int)n : NF * (int)n;
  for (int g = 0; g < G; g++) fo[g] = TGROUP[group][g] * (int)n + so;
  const int qo = in_set * ss, oo = out_set * ss;
#define QP(g) (fld + qo + fo[g])
#define SP(g) (fld + fo[g])
#define OP(g) (fld + oo + fo[g])
  const int PW = TX + 6, PH = TY + 6, NCELL = PW * PH;
  const int NT = CTX ? CTX * CTY : (EW ? (int)blockDim.x - TEDGE : (int)blockDim.x);  // one thread a column of the tile
  // plane cells a thread copies: exact for a compile-time tile, the bound TMAXC otherwise
  constexpr int CJ = CTX ? ((CTX + 6) * (CTY + 6) + CTX * CTY - 1) / (CTX * CTY) : TMAXC;
  static_assert(CJ <= TMAXC, "the tile's halo plane fits in TMAXC cells a thread");
  float* lv = sm;                                   // [tlv_rows][MAXNZ]
  float4* fcs = reinterpret_cast<float4*>(lv + tlv_rows(KIND) * MAXNZ);  // [2][NT]: the face fluxes of levels z, z + 1
  float* ring = reinterpret_cast<float*>(fcs + 2 * NT);  // [G][7][NCELL]
  float* fxs = ring + G * 7 * NCELL;                // [2][G][TY][TX + 1]: x faces, west edge at column 0
  float* fys = fxs + 2 * G * TY * (TX + 1);         // [2][G][TY + 1][TX]: y faces, south edge at row 0
  const int FXS = TY * (TX + 1), FYS = (TY + 1) * TX;
  const int t = threadIdx.x, lx = t % TX, ly = t / TX;
  const bool column = !EW || t < NT;  // a column thread (else an edge thread of an EW block)
  const int tilesX = (nx + TX - 1) / TX, x0 = (tile % tilesX) * TX, y0 = (tile / tilesX) * TY;
  const int x = x0 + lx, y = y0 + ly;
  const bool on = column && x < nx && y < ny;
  const int col = on ? x + y * nx : 0;
  // edge lanes: e < TY the west face of row e, TY <= e < TY + TX the south face of column e - TY (e = t, or the edge
  // thread's index in an EW block)
  const int e = EW ? t - NT : t;
  const bool edgeW = e >= 0 && e < TY && y0 + e < ny, edgeS = e >= TY && e < TY + TX && x0 + e - TY < nx;
  const int eoff = edgeW ? wrap(x0 - 1, nx) + (y0 + e) * nx : edgeS ? (x0 + e - TY) + wrap(y0 - 1, ny) * nx : 0;
  const int ecell = edgeW ? (e + 3) * PW + 3 : (3 * PW + e - TY + 3);  // plane index of the cell on the edge's high side
  const int estride = edgeW ? 1 : PW;
  float* const edst = edgeW ? fxs + e * (TX + 1) : fys + (e - TY);
  for (int z = t; z < nz; z += blockDim.x) {
    lv[0 * MAXNZ + z] = lvl(Rg, L_INV_HZ, z);
    lv[1 * MAXNZ + z] = lvl(Rg, L_INV_RHO, z);
    if (KIND == TK_DYN) {
      lv[2 * MAXNZ + z] = lvl(Rg, L_TH_UP_POS, z); lv[3 * MAXNZ + z] = lvl(Rg, L_TH_UP_NEG, z);
      lv[4 * MAXNZ + z] = lvl(Rg, L_TH_DN_POS, z); lv[5 * MAXNZ + z] = lvl(Rg, L_TH_DN_NEG, z);
      lv[6 * MAXNZ + z] = lvl(Rg, L_THB, z); lv[7 * MAXNZ + z] = lvl(Rg, L_QB, z); lv[8 * MAXNZ + z] = lvl(Rg, L_THVENV, z);
    }
  }
  // plane cell t + j * NT of this thread: its column offset (periodic), -1 past the plane
  int off[CJ];
#pragma unroll
  for (int j = 0; j < CJ; j++) {
    int c = t + j * NT;
    int hy = c / PW, hx = c - hy * PW;
    int gx = x0 + hx - 3, gy = y0 + hy - 3;
    gx = ((gx % nx) + nx) % nx; gy = ((gy % ny) + ny) % ny;
    off[j] = column && c < NCELL ? gx + gy * nx : -1;
  }
  const bool loadBuoy = KIND == TK_DYN && (flags & RF_STAGES);
  const bool loading = flags & RF_LOADING;
  // prologue: ring slots of the virtual levels -3..3 (clamped), level 0's inputs
  for (int v = -3; v <= 3; v++) {
    const int lev = clampi(v, 0, nz - 1), slot = (v + 7) % 7;
#pragma unroll
    for (int g = 0; g < G; g++)
#pragma unroll
      for (int j = 0; j < CJ; j++) if (off[j] >= 0) ring[(g * 7 + slot) * NCELL + t + j * NT] = QP(g)[off[j] + lev * layer];
  }
  if (on) cp_async16(fcs + t, F4 + col);
  float me = edgeW ? F4[eoff].x : edgeS ? F4[eoff].y : 0.f;
  float s0[G];
#pragma unroll
  for (int g = 0; g < G; g++) s0[g] = on && stage > 0 ? SP(g)[col] : 0.f;
  // buoyancy inputs of the level (dynamics): the vapour and the condensate load (theta' is the ring's centre value)
  float bQ = 0.f, bL = 0.f;
  if (loadBuoy && on) {
    bQ = inb[Q * n + col];
    bL = inb[CLOUD * n + col] + inb[ICE * n + col] +
         (loading ? (inb[RAIN * n + col] + inb[SNOW * n + col]) + (inb[GRAUPEL * n + col] + inb[HAIL * n + col]) : 0.f);
  }
  cp_async_wait_all();
  __syncthreads();
  float fzD[G];
#pragma unroll
  for (int g = 0; g < G; g++) fzD[g] = 0.f;
  float mzD = 0.f;
  const int cidx = (ly + 3) * PW + (lx + 3);
  for (int z = 0; z < nz; z++) {
    const int buf = z & 1, l = z * layer;
    const bool more = z + 1 < nz;
    const int ln = l + layer;
    // loads for later levels, issued before this level's arithmetic: the plane z + 4 into the ring slot of z - 3
    // (read last by the previous level, before its barrier) by asynchronous copies; level z + 1's faces, start values
    // and buoyancy inputs into registers
    const int levNext = min(z + 4, nz - 1) * layer, s_new = (z + 4) % 7;
#pragma unroll
    for (int g = 0; g < G; g++)
#pragma unroll
      for (int j = 0; j < CJ; j++) if (off[j] >= 0) cp_async4(ring + (g * 7 + s_new) * NCELL + t + j * NT, QP(g) + off[j] + levNext);
    float men = 0.f, s0n[G], bn[7];
#pragma unroll
    for (int g = 0; g < G; g++) s0n[g] = 0.f;
#pragma unroll
    for (int j = 0; j < 7; j++) bn[j] = 0.f;
    if (more) {
      if (edgeW) men = F4[eoff + ln].x;
      if (edgeS) men = F4[eoff + ln].y;
      if (on) {
        cp_async16(fcs + (buf ^ 1) * NT + t, F4 + col + ln);
        if (stage > 0) {
#pragma unroll
          for (int g = 0; g < G; g++) s0n[g] = SP(g)[col + ln];
        }
        if (loadBuoy) { bn[0] = inb[Q * n + col + ln]; bn[1] = inb[CLOUD * n + col + ln]; bn[2] = inb[ICE * n + col + ln];
          if (loading) { bn[3] = inb[RAIN * n + col + ln]; bn[4] = inb[SNOW * n + col + ln]; bn[5] = inb[GRAUPEL * n + col + ln]; bn[6] = inb[HAIL * n + col + ln]; } }
      }
    }
    // faces of level z (slot buf is read only before this level's barrier and rewritten after it, by the next
    // level's copies)
    const float4 fc = on ? fcs[buf * NT + t] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float m1 = fc.x, m2 = fc.y, m3 = fc.z;
    const bool px = m1 >= 0.f, py = m2 >= 0.f, pz = m3 >= 0.f, top = z == nz - 1;
    const int s_m2 = (z + 5) % 7, s_m1 = (z + 6) % 7, s_0 = z % 7, s_p1 = (z + 1) % 7, s_p2 = (z + 2) % 7, s_p3 = (z + 3) % 7;
    float fzU[G], qc[G];
    if (on) {
#pragma unroll
      for (int g = 0; g < G; g++) {
        // east and north faces of this cell as one pair
        const float* P = ring + (g * 7 + s_0) * NCELL + cidx;
        qc[g] = P[0];
        float2 A, B, C, D, E;
        face_stencil(P + 1, 1, px, A.x, B.x, C.x, D.x, E.x);
        face_stencil(P + PW, PW, py, A.y, B.y, C.y, D.y, E.y);
        const float2 r = recon2<KIND>(A, B, C, D, E);
        fxs[(buf * G + g) * FXS + ly * (TX + 1) + lx + 1] = m1 * r.x;
        fys[(buf * G + g) * FYS + (ly + 1) * TX + lx] = m2 * r.y;
      }
      // top faces, fields in pairs
#pragma unroll
      for (int g = 0; g < G; g += 2) {
        const int g2 = g + 1 < G ? g + 1 : g;
        const float* R = ring + g * 7 * NCELL + cidx;
        const float* S = ring + g2 * 7 * NCELL + cidx;
        const float2 a2 = make_float2(R[s_m2 * NCELL], S[s_m2 * NCELL]), a1 = make_float2(R[s_m1 * NCELL], S[s_m1 * NCELL]);
        const float2 c0 = make_float2(qc[g], qc[g2]), b1 = make_float2(R[s_p1 * NCELL], S[s_p1 * NCELL]);
        const float2 b2 = make_float2(R[s_p2 * NCELL], S[s_p2 * NCELL]), b3 = make_float2(R[s_p3 * NCELL], S[s_p3 * NCELL]);
        const float2 A = pz ? a2 : b3, B = pz ? a1 : b2, C = pz ? c0 : b1, D = pz ? b1 : c0, E = pz ? b2 : a1;
        if (g + 1 < G) {
          const float2 r = recon2<KIND>(A, B, C, D, E);
          fzU[g] = top ? 0.f : m3 * r.x;
          fzU[g + 1] = top ? 0.f : m3 * r.y;
        } else {
          fzU[g] = top ? 0.f : m3 * recon1<KIND>(A.x, B.x, C.x, D.x, E.x);
        }
      }
    }
    // the tile's west and south edge faces
    if (edgeW || edgeS) {
      const bool pe = me >= 0.f;
      const int es = edgeW ? FXS : FYS;
#pragma unroll
      for (int g = 0; g < G; g += 2) {  // fields in pairs, as the top faces
        float2 A, B, C, D, E;
        face_stencil(ring + (g * 7 + s_0) * NCELL + ecell, estride, pe, A.x, B.x, C.x, D.x, E.x);
        if (g + 1 < G) {
          face_stencil(ring + ((g + 1) * 7 + s_0) * NCELL + ecell, estride, pe, A.y, B.y, C.y, D.y, E.y);
          const float2 r = recon2<KIND>(A, B, C, D, E);
          edst[(buf * G + g) * es] = me * r.x;
          edst[(buf * G + g + 1) * es] = me * r.y;
        } else {
          edst[(buf * G + g) * es] = me * recon1<KIND>(A.x, B.x, C.x, D.x, E.x);
        }
      }
    }
    // the next level's buoyancy inputs reduced to two values before the barrier
    const float bnQ = bn[0], bnL = bn[1] + bn[2] + (loading ? (bn[3] + bn[4]) + (bn[5] + bn[6]) : 0.f);
    cp_async_wait_all();
    __syncthreads();
    if (on) {
      const float ihz = lv[z], irho = lv[MAXNZ + z];
#pragma unroll
      for (int g = 0; g < G; g++) {
        const float* FX = fxs + (buf * G + g) * FXS + ly * (TX + 1) + lx;
        const float* FY = fys + (buf * G + g) * FYS + ly * TX + lx;
        float flux = (FX[1] - FX[0]) * inv_dx + (FY[TX] - FY[0]) * inv_dy + (fzU[g] - fzD[g]) * ihz;
        float tend = -(flux - qc[g] * fc.w) * irho;
        if (KIND == TK_DYN && g == 3) {  // theta': the base profile's own vertical flux
          float up = m3 * (m3 >= 0.f ? lv[2 * MAXNZ + z] : lv[3 * MAXNZ + z]);
          float dn = mzD * (mzD >= 0.f ? lv[4 * MAXNZ + z] : lv[5 * MAXNZ + z]);
          tend -= (up - dn) * ihz * irho;
        }
        if (KIND == TK_DYN && g == 2 && loadBuoy) {
          // g B with theta' and the base state (stageBuoyancy): theta_v - theta_v,env from small differences.
          const float Rb = lv[6 * MAXNZ + z], Qb = lv[7 * MAXNZ + z];
          float dth = qc[3], num = dth + .61f * ((Rb + dth) * (bQ - Qb) + Qb * dth);
          tend += 9.81f * (num / lv[8 * MAXNZ + z] - bL);
        }
        float a = (stage == 0 ? qc[g] : s0[g]) + fdt * tend;
        if (KIND == TK_DYN && g == 2 && stage < 2 && (flags & RF_STAGES) && (z == 0 || z == nz - 1)) a = 0.f;
        OP(g)[col + l] = a;
        fzD[g] = fzU[g];
      }
    }
    mzD = m3;
    me = men;
#pragma unroll
    for (int g = 0; g < G; g++) s0[g] = s0n[g];
    bQ = bnQ; bL = bnL;
  }
  __syncthreads();
#undef QP
#undef SP
#undef OP
}

// MINB: resident blocks per SM the register budget is cut for (2: up to 96 registers a thread, 80 with the edge warps;
// 3: 64).
template <int KIND, int G, int MINB, int CTX, int CTY, bool EW>
__global__ void __launch_bounds__(EW ? 320 + TEDGE : 320, MINB) k_transport(const RunDesc* __restrict__ runs, const int4* items, int nitems,
                                                                             int in_set, int out_set, float frac, int stage, int TX, int TY) {
  extern __shared__ float sm[];
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    transport_item<KIND, G, CTX, CTY, EW>(R, items[it].y, items[it].z, in_set, out_set, frac, stage, TX, TY, sm);
  }
}

// ==================================================================== RK3 transport, bulk-copy tiles
// The same arithmetic as transport_item (the same bits for every face), with the tile's inputs moved by the TMA
// engine: the block is TX x TY consumer threads (one per column) and two producer warps. Per level the producer warps
// issue cp.async.bulk row copies of the next input packet into shared memory - the G field planes of level z + 4
// (rows of the periodic window [x0 - 4, x0 + TX + 4) x [y0 - 3, y0 + TY + 3), one copy per piece of a row between
// wraps, so the halo needs no wrapped index arithmetic), the tile's face fluxes of level z + 1 (one row copy per tile
// row), the face fluxes of the west and south edges and, for the WENO fields, their step-start values - completing on
// one of two mbarriers (the packet of level L on barrier L & 1), from a table of copy descriptors made once per tile;
// they then reconstruct the tile's west and south edge faces, one a lane. The consumer threads wait on the packet's
// mbarrier, reconstruct the east, north and top faces of their own cells, and after the level's block barrier form
// the tendency and the RK3 update. The edge faces, which made two warps of every block do 40% more reconstructions
// than the rest, are all on the producer warps.
// Needs nx and TX multiples of 4 (16-byte rows and pieces), TX <= nx (at most three pieces a row), TX + TY <= 64.
constexpr int TPROD = 64;  // producer threads per block (two warps; named barrier 1 is theirs)

// Entries of the copy-descriptor table of a tile (ring pieces, at most three a window row, then auxiliary rows).
__host__ __device__ constexpr int copy_table_entries(int kind, int G, int TY) {
  return (TY + 6) * 3 + 2 * TY + 1 + (kind == TK_WENO ? G * TY : 0);
}

template <int KIND, int G>
__host__ __device__ constexpr int aux_floats(int TX, int TY) {
  // per buffer: faces [TY][TX] float4, edges [TY + TX] float4, step-start values [G][TY][TX] (WENO)
  return 4 * (TY * TX + TY + TX) + (KIND == TK_WENO ? G * TY * TX : 0);
}

template <int KIND, int G, int CTX, int CTY>
__device__ __forceinline__ void transport_item_bulk(const RunDesc& Rg, int group, int tile, int in_set, int out_set, float frac, int stage,
                                                    int TXr, int TYr, float* sm, unsigned long long* bars, unsigned& phase,
                                                    bool& timed_out) {
  const int TX = CTX ? CTX : TXr, TY = CTY ? CTY : TYr;
  const int nx = Rg.nx, ny = Rg.ny, nz = Rg.nz, layer = Rg.layer;
  const size_t n = Rg.n;
  const float inv_dx = Rg.inv_dx, inv_dy = Rg.inv_dy, fdt = frac * Rg.dt;
  const int flags = Rg.flags;
  const float4* __restrict__ F4 = reinterpret_cast<const float4*>(Rg.faces);
  const float* __restrict__ inb = Rg.fld + (size_t)in_set * NF * n;
  float* const fld = Rg.fld;
  int fo[G];
#pragma unroll
  // an extra field's sets follow the base fields' three, NXE fields a set: its offsets are shifted by `so` so the same
  // set arithmetic addresses it
  const bool chg = G == 1 && group >= 13;  // (the bulk kernels carry no extra fields: only G == 1 could)
  const int so = chg ? (3 * NF - NF) * (int)n : 0, ss = chg ? NXE * (int)n : NF * (int)n;
  for (int g = 0; g < G; g++) fo[g] = TGROUP[group][g] * (int)n + so;
  const int qo = in_set * ss, oo = out_set * ss;
  constexpr bool AUX_S0 = KIND == TK_WENO;
  const int PW = TX + 8, PH = TY + 6, NCELL = PW * PH;
  const int NT = CTX ? CTX * CTY : TXr * TYr;
  const int AUXF = aux_floats<KIND, G>(TX, TY);
  float* lv = sm;                                     // [tlv_rows][MAXNZ]
  float* ring = lv + tlv_rows(KIND) * MAXNZ;          // [G][7][PH][PW], cell (x0 - 4 + c, y0 - 3 + r) at r PW + c
  float* aux = ring + G * 7 * NCELL;                  // [2][AUXF]
  float* fxs = aux + 2 * AUXF;                        // [2][G][TY][TX + 1]: x faces, west edge at column 0
  float* fys = fxs + 2 * G * TY * (TX + 1);           // [2][G][TY + 1][TX]: y faces, south edge at row 0
  // the copy descriptors: ring pieces (smem offset, global offset, bytes), then auxiliary rows (smem offset, source
  // offset, source, bytes); each producer lane fills and reads only its own entries
  int4* const tab = reinterpret_cast<int4*>(sm + (((fys + 2 * G * (TY + 1) * TX) - sm + 3) & ~3));
  const int FXS = TY * (TX + 1), FYS = (TY + 1) * TX;
  const int t = threadIdx.x;
  const bool producer = t >= NT;
  const int lane = t - NT;
  const int tilesX = (nx + TX - 1) / TX, x0 = (tile % tilesX) * TX, y0 = (tile / tilesX) * TY;
  const int rows_on = min(TY, ny - y0), ncols = min(TX, nx - x0);  // tile rows and columns inside the grid
  const int lx = producer ? 0 : t % TX, ly = producer ? 0 : t / TX;
  const int x = x0 + lx, y = y0 + ly;
  const bool on = !producer && x < nx && y < ny;
  const int col = on ? x + y * nx : 0;
  for (int z = t; z < nz; z += blockDim.x) {
    lv[0 * MAXNZ + z] = lvl(Rg, L_INV_HZ, z);
    lv[1 * MAXNZ + z] = lvl(Rg, L_INV_RHO, z);
    if (KIND == TK_DYN) {
      lv[2 * MAXNZ + z] = lvl(Rg, L_TH_UP_POS, z); lv[3 * MAXNZ + z] = lvl(Rg, L_TH_UP_NEG, z);
      lv[4 * MAXNZ + z] = lvl(Rg, L_TH_DN_POS, z); lv[5 * MAXNZ + z] = lvl(Rg, L_TH_DN_NEG, z);
      lv[6 * MAXNZ + z] = lvl(Rg, L_THB, z); lv[7 * MAXNZ + z] = lvl(Rg, L_QB, z); lv[8 * MAXNZ + z] = lvl(Rg, L_THVENV, z);
    }
  }
  const TileCopies TC{nx, ny, layer, TX, TY, x0, y0, G, AUX_S0 && stage > 0};
  int covered;
  const int nseg = TC.pieces(covered), nrs = PH * nseg, na = TC.naux();
  const unsigned auxBytes = TC.bytes(0), planeBytes = TC.bytes(1) - auxBytes;
  int4* const rtab = tab;
  int4* const atab = tab + nrs;
  if (producer) {
    for (int j = lane; j < nrs; j += TPROD) { int so, go, len; TC.ring(j, nseg, so, go, len); rtab[j] = make_int4(so, go, 4 * len, 0); }
    for (int j = lane; j < na; j += TPROD) { int so, src, which, b; TC.aux(j, so, src, which, b); atab[j] = make_int4(so, src, which, b); }
  }
  // The packet of level L (issued by the producer warp): the plane L + 3 (for L = 0 the six planes of virtual levels
  // -2..3, clamped, that level 0 reads; the seventh slot is the one the packet of level 1, issued before this one has
  // landed, fills with plane 4, so no two packets in flight write the same slot) and the level's faces, edges and
  // step-start values; its bytes announced on barrier L & 1 first.
  auto issue = [&](int L) {
    unsigned long long* bar = bars + (L & 1);
    const int v0 = L == 0 ? -2 : L + 3, v1 = L + 3;
    if (lane == 0) mbar_arrive_expect_tx(bar, auxBytes + (unsigned)(v1 - v0 + 1) * planeBytes);
    asm volatile("bar.sync 1, %0;\n" ::"n"(TPROD) : "memory");  // the bytes are announced before any copy lands
    for (int v = v0; v <= v1; v++) {
      const int lev = clampi(v, 0, nz - 1), slot = (v + 7) % 7;
      float* const rs = ring + slot * NCELL;
      const float* const gs = fld + qo + lev * layer;
      for (int j = lane; j < nrs; j += TPROD) {
        const int4 d = rtab[j];
#pragma unroll
        for (int g = 0; g < G; g++) bulk_g2s(rs + g * 7 * NCELL + d.x, gs + fo[g] + d.y, (unsigned)d.z, bar);
      }
    }
    float* A = aux + (L & 1) * AUXF;
    const int l = L * layer;
    for (int j = lane; j < na; j += TPROD) {
      const int4 d = atab[j];
      const void* from = d.z == 0 ? static_cast<const void*>(F4 + l + d.y)
                                  : static_cast<const void*>(fld + TGROUP[group][d.z - 1] * (int)n + l + d.y);
      bulk_g2s(A + d.x, from, (unsigned)d.w, bar);
    }
  };
  // the packet of level L has landed (all threads); a wait that runs out is recorded and ends the item
  auto await = [&](int L) {
    const int b = L & 1;
    if (!mbar_wait(bars + b, (phase >> b) & 1u)) timed_out = true;
    phase ^= 1u << b;
  };
  __syncthreads();  // the level table; the previous item's reads of the ring and the packets are done
  if (producer) { fence_proxy_async(); issue(0); }
  // edge faces: producer lane e (e < TY: the west face of tile row e; TY <= e < TY + TX: the south face of tile column
  // e - TY)
  constexpr int EROUNDS = 1;
  const bool loadBuoy = KIND == TK_DYN && (flags & RF_STAGES);
  const bool loading = flags & RF_LOADING;
  float s0[G];
#pragma unroll
  for (int g = 0; g < G; g++) s0[g] = !AUX_S0 && on && stage > 0 ? fld[fo[g] + col] : 0.f;
  float bQ = 0.f, bL = 0.f;
  if (loadBuoy && on) {
    bQ = inb[Q * n + col];
    bL = inb[CLOUD * n + col] + inb[ICE * n + col] +
         (loading ? (inb[RAIN * n + col] + inb[SNOW * n + col]) + (inb[GRAUPEL * n + col] + inb[HAIL * n + col]) : 0.f);
  }
  float fzD[G];
#pragma unroll
  for (int g = 0; g < G; g++) fzD[g] = 0.f;
  float mzD = 0.f;
  const int cidx = (ly + 3) * PW + (lx + 4);
  for (int z = 0; z < nz; z++) {
    const int buf = z & 1, l = z * layer;
    const bool more = z + 1 < nz;
    const int ln = l + layer;
    if (producer && more) { fence_proxy_async(); issue(z + 1); }
    // the next level's start values (dynamics) and buoyancy inputs into registers, a level ahead
    float s0n[G], bn[7];
#pragma unroll
    for (int g = 0; g < G; g++) s0n[g] = 0.f;
#pragma unroll
    for (int j = 0; j < 7; j++) bn[j] = 0.f;
    if (more && on) {
      if (!AUX_S0 && stage > 0) {
#pragma unroll
        for (int g = 0; g < G; g++) s0n[g] = fld[fo[g] + col + ln];
      }
      if (loadBuoy) { bn[0] = inb[Q * n + col + ln]; bn[1] = inb[CLOUD * n + col + ln]; bn[2] = inb[ICE * n + col + ln];
        if (loading) { bn[3] = inb[RAIN * n + col + ln]; bn[4] = inb[SNOW * n + col + ln]; bn[5] = inb[GRAUPEL * n + col + ln]; bn[6] = inb[HAIL * n + col + ln]; } }
    }
    await(z);
    const float* A = aux + buf * AUXF;
    const int s_m2 = (z + 5) % 7, s_m1 = (z + 6) % 7, s_0 = z % 7, s_p1 = (z + 1) % 7, s_p2 = (z + 2) % 7, s_p3 = (z + 3) % 7;
    const bool top = z == nz - 1;
    float4 fc = make_float4(0.f, 0.f, 0.f, 0.f);
    float fzU[G], qc[G];
    if (on) {
      fc = reinterpret_cast<const float4*>(A)[ly * TX + lx];
      if (AUX_S0 && stage > 0) {
#pragma unroll
        for (int g = 0; g < G; g++) s0[g] = A[4 * (TY * TX + TY + TX) + (g * TY + ly) * TX + lx];
      }
      const float m1 = fc.x, m2 = fc.y, m3 = fc.z;
      const bool px = m1 >= 0.f, py = m2 >= 0.f, pz = m3 >= 0.f;
#pragma unroll
      for (int g = 0; g < G; g++) {
        // east and north faces of this cell as one pair
        const float* P = ring + (g * 7 + s_0) * NCELL + cidx;
        qc[g] = P[0];
        float2 Av, Bv, Cv, Dv, Ev;
        face_stencil(P + 1, 1, px, Av.x, Bv.x, Cv.x, Dv.x, Ev.x);
        face_stencil(P + PW, PW, py, Av.y, Bv.y, Cv.y, Dv.y, Ev.y);
        const float2 r = recon2<KIND>(Av, Bv, Cv, Dv, Ev);
        fxs[(buf * G + g) * FXS + ly * (TX + 1) + lx + 1] = m1 * r.x;
        fys[(buf * G + g) * FYS + (ly + 1) * TX + lx] = m2 * r.y;
      }
      // top faces, fields in pairs
#pragma unroll
      for (int g = 0; g < G; g += 2) {
        const int g2 = g + 1 < G ? g + 1 : g;
        const float* R = ring + g * 7 * NCELL + cidx;
        const float* S = ring + g2 * 7 * NCELL + cidx;
        const float2 a2 = make_float2(R[s_m2 * NCELL], S[s_m2 * NCELL]), a1 = make_float2(R[s_m1 * NCELL], S[s_m1 * NCELL]);
        const float2 c0v = make_float2(qc[g], qc[g2]), b1 = make_float2(R[s_p1 * NCELL], S[s_p1 * NCELL]);
        const float2 b2 = make_float2(R[s_p2 * NCELL], S[s_p2 * NCELL]), b3 = make_float2(R[s_p3 * NCELL], S[s_p3 * NCELL]);
        const float2 Av = pz ? a2 : b3, Bv = pz ? a1 : b2, Cv = pz ? c0v : b1, Dv = pz ? b1 : c0v, Ev = pz ? b2 : a1;
        if (g + 1 < G) {
          const float2 r = recon2<KIND>(Av, Bv, Cv, Dv, Ev);
          fzU[g] = top ? 0.f : m3 * r.x;
          fzU[g + 1] = top ? 0.f : m3 * r.y;
        } else {
          fzU[g] = top ? 0.f : m3 * recon1<KIND>(Av.x, Bv.x, Cv.x, Dv.x, Ev.x);
        }
      }
    }
    if (producer) {
#pragma unroll
      for (int rd = 0; rd < EROUNDS; rd++) {
        const int e = lane + rd * TPROD;
        const bool edgeW = e < TY && e < rows_on, edgeS = e >= TY && e < TY + ncols;
        if (!(edgeW || edgeS)) continue;
        const float4 ef = reinterpret_cast<const float4*>(A)[TY * TX + e];  // west faces, then the south ones
        const float me = edgeW ? ef.x : ef.y;
        const bool pe = me >= 0.f;
        const int ecell = edgeW ? (e + 3) * PW + 4 : 3 * PW + (e - TY) + 4;  // the cell on the edge's high side
        const int estride = edgeW ? 1 : PW, es = edgeW ? FXS : FYS;
        float* const edst = edgeW ? fxs + e * (TX + 1) : fys + (e - TY);
#pragma unroll
        for (int g = 0; g < G; g += 2) {  // fields in pairs, as the top faces
          float2 Av, Bv, Cv, Dv, Ev;
          face_stencil(ring + (g * 7 + s_0) * NCELL + ecell, estride, pe, Av.x, Bv.x, Cv.x, Dv.x, Ev.x);
          if (g + 1 < G) {
            face_stencil(ring + ((g + 1) * 7 + s_0) * NCELL + ecell, estride, pe, Av.y, Bv.y, Cv.y, Dv.y, Ev.y);
            const float2 r = recon2<KIND>(Av, Bv, Cv, Dv, Ev);
            edst[(buf * G + g) * es] = me * r.x;
            edst[(buf * G + g + 1) * es] = me * r.y;
          } else {
            edst[(buf * G + g) * es] = me * recon1<KIND>(Av.x, Bv.x, Cv.x, Dv.x, Ev.x);
          }
        }
      }
    }
    const float bnQ = bn[0], bnL = bn[1] + bn[2] + (loading ? (bn[3] + bn[4]) + (bn[5] + bn[6]) : 0.f);
    if (__syncthreads_or(timed_out)) {
      // a packet never landed: record it on the run, give the copies in flight a last bounded wait (this level's
      // packet, whose phase bit await has already flipped, and the next one's), and end the item and the kernel
      timed_out = true;
      if (t == 0) { atomicAdd(Rg.cnt + C_TIMEOUT, 1ull); atomicExch(Rg.cnt + C_FAILED, 1ull); }
      mbar_wait(bars + (z & 1), ((phase >> (z & 1)) & 1u) ^ 1u);
      if (more) mbar_wait(bars + ((z + 1) & 1), (phase >> ((z + 1) & 1)) & 1u);
      return;
    }
    if (on) {
      const float ihz = lv[z], irho = lv[MAXNZ + z];
#pragma unroll
      for (int g = 0; g < G; g++) {
        const float* FX = fxs + (buf * G + g) * FXS + ly * (TX + 1) + lx;
        const float* FY = fys + (buf * G + g) * FYS + ly * TX + lx;
        float flux = (FX[1] - FX[0]) * inv_dx + (FY[TX] - FY[0]) * inv_dy + (fzU[g] - fzD[g]) * ihz;
        float tend = -(flux - qc[g] * fc.w) * irho;
        if (KIND == TK_DYN && g == 3) {  // theta': the base profile's own vertical flux
          const float m3 = fc.z;
          float up = m3 * (m3 >= 0.f ? lv[2 * MAXNZ + z] : lv[3 * MAXNZ + z]);
          float dn = mzD * (mzD >= 0.f ? lv[4 * MAXNZ + z] : lv[5 * MAXNZ + z]);
          tend -= (up - dn) * ihz * irho;
        }
        if (KIND == TK_DYN && g == 2 && loadBuoy) {
          const float Rb = lv[6 * MAXNZ + z], Qb = lv[7 * MAXNZ + z];
          float dth = qc[3], num = dth + .61f * ((Rb + dth) * (bQ - Qb) + Qb * dth);
          tend += 9.81f * (num / lv[8 * MAXNZ + z] - bL);
        }
        float a = (stage == 0 ? qc[g] : s0[g]) + fdt * tend;
        if (KIND == TK_DYN && g == 2 && stage < 2 && (flags & RF_STAGES) && (z == 0 || z == nz - 1)) a = 0.f;
        fld[oo + fo[g] + col + l] = a;
        fzD[g] = fzU[g];
      }
    }
    mzD = fc.z;
    if (!AUX_S0) {
#pragma unroll
      for (int g = 0; g < G; g++) s0[g] = s0n[g];
    }
    bQ = bnQ; bL = bnL;
  }
  __syncthreads();
}

template <int KIND, int G, int MINB, int CTX, int CTY>
__global__ void __launch_bounds__(320 + TPROD, MINB) k_transport_bulk(const RunDesc* __restrict__ runs, const int4* items, int nitems, int in_set,
                                                                       int out_set, float frac, int stage, int TX, int TY) {
  extern __shared__ __align__(16) float sm[];
  __shared__ __align__(8) unsigned long long bars[2];
  if (threadIdx.x == 0) { mbar_init(bars, 1); mbar_init(bars + 1, 1); fence_mbar_init(); fence_proxy_async(); }
  __syncthreads();
  unsigned phase = 0;
  bool timed_out = false;
  FOR_ITEMS {
    const RunDesc& R = runs[items[it].x];
    if (R.cnt[C_FAILED]) continue;
    transport_item_bulk<KIND, G, CTX, CTY>(R, items[it].y, items[it].z, in_set, out_set, frac, stage, TX, TY, sm, bars, phase, timed_out);
    if (timed_out) return;
  }
}

// ==================================================================== launchers
size_t transport_smem(int kind, int G, int TX, int TY) {
  return ((size_t)tlv_rows(kind) * MAXNZ + 2 * 4 * (size_t)TX * TY + (size_t)G * 7 * (TX + 6) * (TY + 6) + 2 * (size_t)G * TY * (TX + 1) + 2 * (size_t)G * (TY + 1) * TX) * sizeof(float);
}
size_t transport_smem_bulk(int kind, int G, int TX, int TY) {
  const size_t auxf = kind == TK_WENO ? (G == 3 ? aux_floats<TK_WENO, 3>(TX, TY) : aux_floats<TK_WENO, 1>(TX, TY)) : aux_floats<TK_DYN, 4>(TX, TY);
  const size_t floats = (size_t)tlv_rows(kind) * MAXNZ + (size_t)G * 7 * (TX + 8) * (TY + 6) + 2 * auxf + 2 * (size_t)G * TY * (TX + 1) +
                        2 * (size_t)G * (TY + 1) * TX;
  return ((floats + 3) / 4 * 4 + 4 * (size_t)copy_table_entries(kind, G, TY)) * sizeof(float);
}
bool transport_bulk_ok(int TX, int TY, int min_nx, bool all_nx4) {
  return all_nx4 && TX % 4 == 0 && TX <= min_nx && (TX * TY) % 32 == 0 && TX * TY <= 320 && TX + TY <= TPROD;
}

namespace {
// The tiles compiled with constant strides (the autotuner's candidates); any other tile takes the run-time variant.
template <int KIND, int G, int MINB, int CTX, int CTY, bool EW>
void tlaunch(const Launch& L, int in_set, int out_set, float frac, int stage, int TX, int TY) {
  k_transport<KIND, G, MINB, CTX, CTY, EW><<<GRID(L.n, L.cap), TX * TY + (EW ? TEDGE : 0), transport_smem(KIND, G, TX, TY), L.stream>>>(
      L.runs, L.items, L.n, in_set, out_set, frac, stage, TX, TY);
}
template <int KIND, int G, int CTX, int CTY>
void tlaunch_ew(const Launch& L, int in_set, int out_set, float frac, int stage, int TX, int TY, bool ew) {
  if (ew) tlaunch<KIND, G, 2, CTX, CTY, true>(L, in_set, out_set, frac, stage, TX, TY);
  else tlaunch<KIND, G, 2, CTX, CTY, false>(L, in_set, out_set, frac, stage, TX, TY);
}
template <int KIND, int G, int CTX, int CTY>
void tlaunch_bulk(const Launch& L, int in_set, int out_set, float frac, int stage, int TX, int TY) {
  k_transport_bulk<KIND, G, 2, CTX, CTY><<<GRID(L.n, L.cap), TX * TY + TPROD, transport_smem_bulk(KIND, G, TX, TY), L.stream>>>(
      L.runs, L.items, L.n, in_set, out_set, frac, stage, TX, TY);
}
template <int KIND, int G>
void tlaunch_tile_bulk(const Launch& L, int in_set, int out_set, float frac, int stage, int TX, int TY) {
  if (TX == 40 && TY == 8) return tlaunch_bulk<KIND, G, 40, 8>(L, in_set, out_set, frac, stage, TX, TY);
  if (TX == 32 && TY == 8) return tlaunch_bulk<KIND, G, 32, 8>(L, in_set, out_set, frac, stage, TX, TY);
  if (TX == 20 && TY == 8) return tlaunch_bulk<KIND, G, 20, 8>(L, in_set, out_set, frac, stage, TX, TY);
  if (TX == 16 && TY == 16) return tlaunch_bulk<KIND, G, 16, 16>(L, in_set, out_set, frac, stage, TX, TY);
  if (TX == 40 && TY == 4) return tlaunch_bulk<KIND, G, 40, 4>(L, in_set, out_set, frac, stage, TX, TY);
  tlaunch_bulk<KIND, G, 0, 0>(L, in_set, out_set, frac, stage, TX, TY);
}
template <int KIND, int G>
cudaError_t tlimits_bulk(int bytes) {
  cudaError_t e;
  if ((e = smem_limit(k_transport_bulk<KIND, G, 2, 0, 0>, bytes)) != cudaSuccess) return e;
  if ((e = smem_limit(k_transport_bulk<KIND, G, 2, 40, 8>, bytes)) != cudaSuccess) return e;
  if ((e = smem_limit(k_transport_bulk<KIND, G, 2, 32, 8>, bytes)) != cudaSuccess) return e;
  if ((e = smem_limit(k_transport_bulk<KIND, G, 2, 20, 8>, bytes)) != cudaSuccess) return e;
  if ((e = smem_limit(k_transport_bulk<KIND, G, 2, 16, 16>, bytes)) != cudaSuccess) return e;
  return smem_limit(k_transport_bulk<KIND, G, 2, 40, 4>, bytes);
}
// ew: the compile-time tiles (all with a multiple of 32 columns) with the two edge warps
template <int KIND, int G, int MINB>
void tlaunch_tile(const Launch& L, int in_set, int out_set, float frac, int stage, int TX, int TY, bool ew) {
  if constexpr (MINB == 2) {
    if (TX == 40 && TY == 8) return tlaunch_ew<KIND, G, 40, 8>(L, in_set, out_set, frac, stage, TX, TY, ew);
    if (TX == 32 && TY == 8) return tlaunch_ew<KIND, G, 32, 8>(L, in_set, out_set, frac, stage, TX, TY, ew);
    if (TX == 20 && TY == 8) return tlaunch_ew<KIND, G, 20, 8>(L, in_set, out_set, frac, stage, TX, TY, ew);
    if (TX == 16 && TY == 16) return tlaunch_ew<KIND, G, 16, 16>(L, in_set, out_set, frac, stage, TX, TY, ew);
    if (TX == 40 && TY == 4) return tlaunch_ew<KIND, G, 40, 4>(L, in_set, out_set, frac, stage, TX, TY, ew);
  }
  tlaunch<KIND, G, MINB, 0, 0, false>(L, in_set, out_set, frac, stage, TX, TY);
}
template <int KIND, int G, int CTX, int CTY>
cudaError_t tlimits_ew(int bytes) {
  cudaError_t e;
  if ((e = smem_limit(k_transport<KIND, G, 2, CTX, CTY, false>, bytes)) != cudaSuccess) return e;
  return smem_limit(k_transport<KIND, G, 2, CTX, CTY, true>, bytes);
}
template <int KIND, int G, int MINB>
cudaError_t tlimits(int bytes) {
  cudaError_t e;
  if ((e = smem_limit(k_transport<KIND, G, MINB, 0, 0, false>, bytes)) != cudaSuccess) return e;
  if constexpr (MINB == 2) {
    if ((e = tlimits_ew<KIND, G, 40, 8>(bytes)) != cudaSuccess) return e;
    if ((e = tlimits_ew<KIND, G, 32, 8>(bytes)) != cudaSuccess) return e;
    if ((e = tlimits_ew<KIND, G, 20, 8>(bytes)) != cudaSuccess) return e;
    if ((e = tlimits_ew<KIND, G, 16, 16>(bytes)) != cudaSuccess) return e;
    if ((e = tlimits_ew<KIND, G, 40, 4>(bytes)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}
}  // namespace

void launch_transport(const Launch& L, int kind, int group, int minb, int in_set, int out_set, float frac, int stage, int TX, int TY,
                      bool bulk, bool ew) {
  if (L.n == 0) return;
  if (bulk && minb == 2) {
    if (kind == TK_WENO) {
      if (group == 3) tlaunch_tile_bulk<TK_WENO, 3>(L, in_set, out_set, frac, stage, TX, TY);
      else tlaunch_tile_bulk<TK_WENO, 1>(L, in_set, out_set, frac, stage, TX, TY);
    } else {
      tlaunch_tile_bulk<TK_DYN, 4>(L, in_set, out_set, frac, stage, TX, TY);
    }
    return;
  }
  switch (kind) {
    case TK_WENO:
      if (group == 3) { if (minb == 3) tlaunch_tile<TK_WENO, 3, 3>(L, in_set, out_set, frac, stage, TX, TY, false); else tlaunch_tile<TK_WENO, 3, 2>(L, in_set, out_set, frac, stage, TX, TY, ew); }
      else { if (minb == 3) tlaunch_tile<TK_WENO, 1, 3>(L, in_set, out_set, frac, stage, TX, TY, false); else tlaunch_tile<TK_WENO, 1, 2>(L, in_set, out_set, frac, stage, TX, TY, ew); }
      break;
    // the dynamics kernel without the edge warps: at their 80-register budget it spills, and measured slower
    default: tlaunch_tile<TK_DYN, 4, 2>(L, in_set, out_set, frac, stage, TX, TY, false); break;
  }
}

cudaError_t set_transport_smem_limits(int bytes) {
  cudaError_t e;
  if ((e = tlimits<TK_WENO, 3, 2>(bytes)) != cudaSuccess) return e;
  if ((e = tlimits<TK_WENO, 3, 3>(bytes)) != cudaSuccess) return e;
  if ((e = tlimits<TK_WENO, 1, 2>(bytes)) != cudaSuccess) return e;
  if ((e = tlimits<TK_WENO, 1, 3>(bytes)) != cudaSuccess) return e;
  if ((e = tlimits_bulk<TK_WENO, 3>(bytes)) != cudaSuccess) return e;
  if ((e = tlimits_bulk<TK_WENO, 1>(bytes)) != cudaSuccess) return e;
  if ((e = tlimits_bulk<TK_DYN, 4>(bytes)) != cudaSuccess) return e;
  return tlimits<TK_DYN, 4, 2>(bytes);
}

}  // namespace sg
