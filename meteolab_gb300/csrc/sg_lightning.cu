// Lightning of an electrified run on the device (src/core/lightning.ts:135-420, driven by AtmosphereModel.discharge,
// src/core/model.ts:1537-1552): after every step, while the storm's field somewhere exceeds the breakdown threshold
// (and at most flashLimit(dt) times), one flash there; then the conduction of the small ions and the corona from the
// ground; then the vertical field for the next step's inductive charging.
//
// The work splits by its shape. Whole-grid passes (the charge density of the four carriers, the FP64 potential solve,
// the search for the strongest field, the conduction) are ordinary grid-wide kernels. A flash's channel grows one node
// at a time with a random pick among the links that exceed the propagation threshold, each pick depending on the last:
// one block grows it (k_lgt_grow), its threads weighting the growth front and finding the picked link in parallel and
// one thread doing the reference's sequential bookkeeping (the front's order, the neighbours appended in the
// reference's order, the running potential sum), so the channel is the reference's own for the same potential. The
// deposit of a stage is one block over the channel. The host steps through the flash's stages (a stage ends when the
// channel leaves the cloud, touches the ground or stops; the field is solved again between stages), reading a small
// state record after each: the control flow of Lightning.flash, with every array on the device.
//
// Every loop is bounded: a grow launch adds at most MAX_CHANNEL nodes, a flash has at most STROKES + 2 stages, a step
// at most flashLimit(dt) flashes.
#include <cuda_runtime.h>
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "sg_common.cuh"
#include "sg_elec_solve.cuh"
#include "sg_lightning.h"

namespace sg {

namespace {

constexpr double EPS0 = 8.8541878128e-12;                                                     // src/core/electric.ts:6
constexpr double E_INIT = 2.84e5, RHO_STANDARD = 1.225, F_CRIT = .43, RHO_MIN = 1e-10, CHANNEL_RADIUS = 1, SHIELDING = .25;  // lightning.ts:13-29
constexpr double SIGMA_GROUND = 2e-14, SIGMA_SCALE = 6000, CLOUD_SIGMA = .1, CLOUDY = 1e-5, CORONA_FIELD = 5e3, CORONA_RATE = 5e-13;  // :51-67
constexpr int GROW_THREADS = 256, DEP_THREADS = 256;

SG_D double mulberry(uint32_t& s) {  // src/core/math.ts:7-14
  s += 0x6D2B79F5u;
  uint32_t t = (s ^ (s >> 15)) * (1u | s);
  t = (t + (t ^ (t >> 7)) * (61u | t)) ^ t;
  return (double)(t ^ (t >> 14)) / 4294967296.0;
}
SG_D double lt(const LgtDev& L, int which, int z) { return L.lv[(size_t)which * L.nz + z]; }
SG_D double dmul(double a, double b) { return __dmul_rn(a, b); }
SG_D double dadd(double a, double b) { return __dadd_rn(a, b); }
SG_D double series(double a, double b) { return __ddiv_rn(dmul(dmul(2.0, a), b), dadd(a, b)); }  // conductances in series
SG_D bool clearAt(const LgtDev& L, int i) { return fabs(L.rho[i]) < RHO_MIN || (double)L.cloudy[i] <= CLOUDY; }  // :343

// ---------------------------------------------------------------- grid-wide passes
// cloud(): the cloud water, ice and snow summed at each node as FP32 (:249-253).
__global__ void k_lgt_cloudy(const RunDesc R, const LgtDev L) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= R.n) return;
  L.cloudy[i] = __fadd_rn(__fadd_rn(field(R, 0, CLOUD)[i], field(R, 0, ICE)[i]), field(R, 0, SNOW)[i]);
}
// solve()'s charge density (:226-230): the four carriers summed in FP64, times the level's air density.
__global__ void k_lgt_rho(const RunDesc R, const LgtDev L) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= R.n) return;
  double s = (double)field(R, 0, CHARGE_ICE)[i];
  s = dadd(s, (double)field(R, 0, CHARGE_GRAUPEL)[i]);
  s = dadd(s, (double)field(R, 0, CHARGE_RAIN)[i]);
  s = dadd(s, (double)field(R, 0, CHARGE_AIR)[i]);
  L.rho[i] = dmul(s, lt(L, LT_AIR, i / R.layer));
}
// strongest() (:233-246): |E|^2 / Einit^2 of the interior nodes not failed at this step; the largest, first in node order.
SG_D double fieldRatio2(const RunDesc& R, const LgtDev& L, int i) {
  const int nx = R.nx, ny = R.ny, layer = R.layer, z = i / layer, y = (i - z * layer) / nx, x = i - z * layer - y * nx, row = y * nx + z * layer;
  const double* phi = L.phi;
  const int xp = x + 1 == nx ? 0 : x + 1, xm = x == 0 ? nx - 1 : x - 1, yp = y + 1 == ny ? 0 : y + 1, ym = y == 0 ? ny - 1 : y - 1;
  const double ex = (phi[xp + row] - phi[xm + row]) / (2 * L.dx), ey = (phi[x + yp * nx + z * layer] - phi[x + ym * nx + z * layer]) / (2 * L.dy);
  const double ez = (phi[i + layer] - phi[i - layer]) / lt(L, LT_SPAN, z);
  return dadd(dadd(dmul(ex, ex), dmul(ey, ey)), dmul(ez, ez)) / lt(L, LT_EINIT2, z);
}
__global__ void k_lgt_strongest(const RunDesc R, const LgtDev L, int stamp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + R.layer;
  if (i >= R.n - R.layer) return;
  if (L.failed[i] == stamp) return;
  const double r = fieldRatio2(R, L, i);
  if (r > 0) atomicMax(&L.st->maxBits, (unsigned long long)__double_as_longlong(r));  // non-negative: bits order as values
}
__global__ void k_lgt_pick(const RunDesc R, const LgtDev L, int stamp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + R.layer;
  if (i >= R.n - R.layer) return;
  const unsigned long long m = L.st->maxBits;
  if (m == 0 || L.failed[i] == stamp) return;
  if ((unsigned long long)__double_as_longlong(fieldRatio2(R, L, i)) == m) atomicMin(&L.st->best, i);
}

// ---------------------------------------------------------------- the channel
// extend() (:389-404) by one warp: lane l takes the l-th candidate of the reference's loop (level k from z - 1 up,
// then dj, then di); the candidates are distinct nodes, so each lane keeps its node's shorter link on its own, and the
// new links go on the growth front in the reference's order (a ballot over the lanes). All 32 lanes call it.
SG_D void extendWarp(const RunDesc& R, const LgtDev& L, volatile LgtState& V, int i, int c, int id) {
  const int lane = threadIdx.x & 31;
  const int nx = R.nx, ny = R.ny, nz = R.nz, layer = R.layer, z = i / layer, y = (i - z * layer) / nx, x = i - z * layer - y * nx;
  const int k0 = max(0, z - 1), k1 = min(nz - 2, z + 1);
  bool fresh = false;
  int j = -1;
  if (lane < 27) {
    const int k = k0 + lane / 9, dj = (lane % 9) / 3 - 1, di = lane % 3 - 1;
    if (k <= k1 && x + di >= 0 && x + di < nx && y + dj >= 0 && y + dj < ny) {
      j = x + di + (y + dj) * nx + k * layer;
      if (!(L.mark[j] == id || (k >= z && fabs(L.rho[j]) < RHO_MIN))) {
        const double hz = lt(L, LT_ZS, k) - lt(L, LT_ZS, z), threshold = dmul(F_CRIT * .5, dadd(lt(L, LT_EINIT, z), lt(L, LT_EINIT, k)));
        const double a = dmul((double)di, L.dx), b = dmul((double)dj, L.dy);
        const double s = dmul(__dsqrt_rn(dadd(dadd(dmul(a, a), dmul(b, b)), dmul(hz, hz))), threshold);
        if (L.seen[j] != id) { L.seen[j] = id; fresh = true; L.scale[j] = s; L.link[j] = c; }
        else if (s < L.scale[j]) { L.scale[j] = s; L.link[j] = c; }
      }
    }
  }
  const unsigned mask = __ballot_sync(0xffffffffu, fresh);
  const int size = V.size;
  if (fresh) L.frontier[size + __popc(mask & ((1u << lane) - 1))] = j;
  __syncwarp();
  if (lane == 0) V.size = size + __popc(mask);
  __syncwarp();
}
// add() of Lightning.flash (:294-304) by one warp (lane 0 the bookkeeping, all lanes the extension), on the block's
// copy of the state record.
SG_D void addNodeWarp(const RunDesc& R, const LgtDev& L, volatile LgtState& V, int j, int from, int id) {
  if ((threadIdx.x & 31) == 0) {
    const int nn = V.nnodes;
    L.mark[j] = id; L.nodes[nn] = j; L.parent[nn] = from; V.nnodes = nn + 1;
    if (j < R.layer) { V.ground = j; V.before = V.potential; V.potential = 0; V.touched = 1; }
    else if (V.ground < 0) { const double sum = dadd(V.sum, L.phi[j]); V.sum = sum; V.potential = sum / (double)(nn + 1); }
  }
  __syncwarp();
  if (j >= R.layer) extendWarp(R, L, V, j, V.nnodes - 1, id);
}

// The state record in shared memory for a kernel's run (a copy in, its changes out): the channel's bookkeeping reads
// and writes it every node, a round trip to L2 each time in global memory.
static_assert(sizeof(LgtState) % 4 == 0, "the state record copies as words");
SG_D void stateIn(LgtState& sh, const LgtDev& L, int t, int threads) {
  for (int k = t; k < (int)(sizeof(LgtState) / 4); k += threads) reinterpret_cast<int*>(&sh)[k] = reinterpret_cast<const int*>(L.st)[k];
}
SG_D void stateOut(const LgtState& sh, const LgtDev& L, int t, int threads) {
  for (int k = t; k < (int)(sizeof(LgtState) / 4); k += threads) reinterpret_cast<int*>(L.st)[k] = reinterpret_cast<const int*>(&sh)[k];
}

__global__ void k_lgt_flash_begin(const RunDesc R, const LgtDev L, int start, int id) {
  __shared__ LgtState sh;
  if (blockIdx.x || threadIdx.x >= 32) return;
  stateIn(sh, L, threadIdx.x, 32);
  __syncwarp();
  if (threadIdx.x == 0) {
    LgtState& S = sh;
    S.size = 0; S.nnodes = 0; S.npol = 0; S.ground = -1; S.touched = 0; S.left = 0; S.event = 0; S.strokes = 0; S.nstrokes = 0;
    S.sum = 0; S.potential = 0; S.before = 0; S.moment = 0; S.lowered = 0; S.neutralized = 0; S.stage = 0; S.needPotential = 0;
    S.start = start; S.id = id;
  }
  __syncwarp();
  addNodeWarp(R, L, sh, start, -1, id);
  __syncwarp();
  stateOut(sh, L, threadIdx.x, 32);
}

// One stage's growth (:309-331): until no link exceeds the threshold, the channel leaves the cloud (the first time),
// touches the ground, or has MAX_CHANNEL nodes. First, after a re-solve, the neutral channel's potential (:338).
// A pick: every thread weights a contiguous part of the front; the parts' exclusive sums (warp scans, in order) and
// the total; one random number; the part holding the first position where the pick less the weights before it is no
// longer positive finds it; then warp 0 removes the link from the front, prunes the clear-air leader's other links (the
// reference's swap-with-last order, its match flags formed by the block) and adds the node.
constexpr int PRUNE_FLAGS = 16384;
__global__ void __launch_bounds__(GROW_THREADS) k_lgt_grow(const RunDesc R, const LgtDev L, int id) {
  __shared__ double wsum[GROW_THREADS / 32], wpre[GROW_THREADS / 32];
  __shared__ double pick;
  __shared__ int pickN, stop, sJ, sFrom, sPrune;
  __shared__ unsigned char flag[PRUNE_FLAGS];
  __shared__ LgtState sh;
  volatile LgtState& V = sh;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5, layer = R.layer;
  stateIn(sh, L, t, GROW_THREADS);
  __syncthreads();
  if (t == 0) {
    V.grown = V.nnodes; V.event = 0;
    if (V.needPotential) {
      double sum = 0;
      const int nn = V.nnodes;
      for (int c = 0; c < nn; c++) sum = dadd(sum, L.phi[L.nodes[c]]);
      V.sum = sum; V.potential = sum / (double)nn; V.needPotential = 0;
    }
  }
  __syncthreads();
  for (int iter = 0; iter < MAX_CHANNEL; iter++) {
    if (V.nnodes >= MAX_CHANNEL) break;
    const int size = V.size, ground = V.ground;
    const double before = V.before, potential = V.potential;
    const int C = (size + GROW_THREADS - 1) / GROW_THREADS, f0 = min(size, t * C), f1 = min(size, f0 + C);
    double acc = 0;
    for (int f = f0; f < f1; f++) {
      const int j = L.frontier[f];
      const double pj = L.phi[j];
      const bool zero = (ground >= 0 && (j < layer || dmul(pj, before) <= 0)) || (clearAt(L, j) && dmul(pj - potential, potential) >= 0);
      const double w = zero ? 0.0 : fabs(potential - pj) / L.scale[j] - 1;
      const double wp = w > 0 ? w : 0.0;
      L.weight[f] = wp; acc = dadd(acc, wp);
    }
    // exclusive sums of the parts in thread order: a shuffle scan in each warp, then over the warps' sums
    double inc = acc;
    for (int o = 1; o < 32; o <<= 1) { const double u = __shfl_up_sync(0xffffffffu, inc, o); if (lane >= o) inc = dadd(inc, u); }
    double exc = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane == 0) exc = 0;
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (t == 0) {
      double s = 0;
      for (int w = 0; w < GROW_THREADS / 32; w++) { wpre[w] = s; s = dadd(s, wsum[w]); }
      pickN = INT_MAX; sPrune = -1;
      stop = s == 0;
      if (!stop) { uint32_t r = V.rng; pick = dmul(mulberry(r), s); V.rng = r; }
    }
    __syncthreads();
    if (stop) break;
    if (f0 < f1) {
      double p = pick - dadd(wpre[warp], exc);
      if (p > 0)
        for (int f = f0; f < f1; f++) {
          p -= L.weight[f];
          if (p <= 0) { atomicMin(&pickN, f); break; }
        }
    }
    __syncthreads();
    if (t == 0) {
      int sz = V.size;
      const int n = min(pickN, sz - 1), j = L.frontier[n], from = L.link[j];
      if (!V.left && V.ground < 0 && clearAt(L, j)) { V.left = 1; V.event = 1; stop = 1; }  // the first step out of the cloud
      else {
        L.frontier[n] = L.frontier[--sz];
        V.size = sz;
        sJ = j; sFrom = from;
        // through clear air a leader does not branch: the other links from the same clear-air node leave the front
        sPrune = clearAt(L, L.nodes[from]) ? from : -1;
      }
    }
    __syncthreads();
    if (stop) break;
    if (sPrune >= 0) {
      const int sz = V.size;
      if (sz <= PRUNE_FLAGS) {
        for (int f = t; f < sz; f += GROW_THREADS) flag[f] = L.link[L.frontier[f]] == sPrune;
        __syncthreads();
        if (t == 0) {
          int m = sz;
          for (int f = sz - 1; f >= 0; f--) if (flag[f]) L.frontier[f] = L.frontier[--m];
          V.size = m;
        }
      } else if (t == 0) {
        int m = sz;
        for (int f = sz - 1; f >= 0; f--) if (L.link[L.frontier[f]] == sPrune) L.frontier[f] = L.frontier[--m];
        V.size = m;
      }
      __syncthreads();
    }
    if (warp == 0) {
      addNodeWarp(R, L, sh, sJ, sFrom, id);
      if (lane == 0 && V.touched) { V.touched = 0; V.event = 1; stop = 1; }
    }
    __syncthreads();
    if (stop) break;
  }
  __syncthreads();
  stateOut(sh, L, t, GROW_THREADS);
}

// deposit() (:352-381) and neutralize() (:410-418) of one stage, one block: each channel node gets its capacitance
// times the potential difference, limited to neutralizing the charge there; before the ground contact both signs are
// scaled to the smaller (the channel stays neutral), after it the ground supplies the difference.
__global__ void __launch_bounds__(DEP_THREADS) k_lgt_deposit(const RunDesc R, const LgtDev L) {
  __shared__ double pos[DEP_THREADS], neg[DEP_THREADS], mom[DEP_THREADS];
  __shared__ double scaleP, scaleN;
  LgtState& S = *L.st;
  const int t = threadIdx.x, layer = R.layer, nn = S.nnodes, npol = S.npol;
  const bool grounded = S.ground >= 0;
  const double V = S.potential;
  const int C = (nn + DEP_THREADS - 1) / DEP_THREADS, c0 = min(nn, t * C), c1 = min(nn, c0 + C);
  double p = 0, q_ = 0, m = 0;
  for (int c = c0; c < c1; c++) {
    const int i = L.nodes[c], z = i / layer;
    double d = 0;
    if (z == 0) { if (c >= npol) L.polarity[c] = 0; }
    else {
      const double q = dmul(lt(L, LT_CAP, z), V - L.phi[i]), here = dmul(dmul(dmul(L.rho[i], L.dx), L.dy), lt(L, LT_HZ, z));
      if (c >= npol) L.polarity[c] = q > 0 ? 1 : q < 0 ? -1 : 0;
      if (dmul(q, here) < 0) {
        d = (q > 0 ? 1.0 : -1.0) * fmin(fabs(q), fabs(here));
        if (d > 0) p = dadd(p, d); else q_ = dadd(q_, -d);
      }
    }
    L.dep[c] = d;
  }
  pos[t] = p; neg[t] = q_;
  __syncthreads();
  if (t == 0) {
    double P = 0, N = 0;
    for (int k = 0; k < DEP_THREADS; k++) { P = dadd(P, pos[k]); N = dadd(N, neg[k]); }
    if (!grounded) {
      const double both = fmin(P, N);
      scaleP = P > 0 ? both / P : 0; scaleN = N > 0 ? both / N : 0;
      S.stage = both; S.neutralized = dadd(S.neutralized, both);
    } else {
      const double charge = N - P;
      scaleP = scaleN = 1;
      S.stage = charge; S.fromGround -= charge; S.lowered = dadd(S.lowered, charge);
      if (S.nstrokes < STROKES) S.strokeQ[S.nstrokes++] = charge;
    }
  }
  __syncthreads();
  for (int c = c0; c < c1; c++) {
    double d = L.dep[c];
    if (d == 0) continue;
    if (!grounded) d = dmul(d, d > 0 ? scaleP : scaleN);
    const int i = L.nodes[c], z = i / layer;
    if (grounded) m = dadd(m, dmul(d, lt(L, LT_ZS, z)));
    if (d == 0) continue;
    // neutralize: taken from the carriers of the opposite sign, in proportion to their charge
    const double perKg = d / lt(L, LT_NODEAIR, z), sq = d > 0 ? 1.0 : -1.0;
    float* cr[4] = {field(R, 0, CHARGE_ICE), field(R, 0, CHARGE_GRAUPEL), field(R, 0, CHARGE_RAIN), field(R, 0, CHARGE_AIR)};
    double opposite = 0;
    for (int k = 0; k < 4; k++) { const double v = cr[k][i]; if (dmul(v, d) < 0) opposite -= dmul(v, sq); }
    if (opposite <= 0) continue;
    for (int k = 0; k < 4; k++) {
      const double v = cr[k][i];
      if (dmul(v, d) < 0) cr[k][i] = (float)dadd(v, dmul(perKg, fabs(v)) / opposite);
    }
  }
  mom[t] = m;
  __syncthreads();
  if (t == 0) {
    if (grounded) { double M = 0; for (int k = 0; k < DEP_THREADS; k++) M = dadd(M, mom[k]); S.moment -= M; S.strokes++; }
    S.npol = nn;
    S.needPotential = !grounded;  // after the next solve the neutral channel's potential is the mean of its nodes' (:338)
  }
}

// The end of a flash: the run's counts and charge budget (:1543), or, for a breakdown that neutralized nothing, the node
// left out for the rest of the step (:270).
__global__ void k_lgt_flash_end(const RunDesc R, const LgtDev L, int stamp) {
  if (threadIdx.x || blockIdx.x) return;
  LgtState& S = *L.st;
  const bool cg = S.ground >= 0;
  const double charge = cg ? S.lowered : S.neutralized;
  S.charge = charge;
  if (charge == 0) { L.failed[S.start] = stamp; return; }
  if (cg) {
    R.acc[A_CHG_GROUND] += charge; R.acc[A_FLASH_CG] += 1;
    if (charge < 0) R.acc[A_CHG_CG_NEG] += charge; else R.acc[A_CHG_CG_POS] += charge;
  } else { R.acc[A_FLASH_IC] += 1; R.acc[A_CHG_IC] += fabs(charge); }
}

// ---------------------------------------------------------------- conduction and corona (:185-223)
__global__ void k_lgt_sigma(const RunDesc R, const LgtDev L) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= R.n) return;
  const double clear = lt(L, LT_SIGMA, i / R.layer);
  L.sigma[i] = (double)L.cloudy[i] > CLOUDY ? dmul(clear, CLOUD_SIGMA) : clear;
}
// Per interior node, the charge through its six faces over dt (a face's conductance the harmonic mean of its two nodes'
// in series; the ground and top take what reaches them) and, on the lowest interior level, the corona from the ground;
// the ion carrier takes it. The charge the air lost to the ground, the top and the corona goes to per-block sums.
__global__ void __launch_bounds__(256) k_lgt_conduct(const RunDesc R, const LgtDev L, int corona, double dt) {
  __shared__ double red[256];
  const int nx = R.nx, ny = R.ny, nz = R.nz, layer = R.layer;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + layer;
  double lost = 0;
  if (i < R.n - layer) {
    const int z = i / layer, y = (i - z * layer) / nx, x = i - z * layer - y * nx;
    const int xp = x + 1 == nx ? 0 : x + 1, xm = x == 0 ? nx - 1 : x - 1, yp = y + 1 == ny ? 0 : y + 1, ym = y == 0 ? ny - 1 : y - 1;
    const double* s = L.sigma;
    const double* phi = L.phi;
    const int ixp = xp + y * nx + z * layer, ixm = xm + y * nx + z * layer, iyp = x + yp * nx + z * layer, iym = x + ym * nx + z * layer;
    const double across = lt(L, LT_ACROSS, z), along = lt(L, LT_ALONG, z);
    const double qxo = dmul(dmul(series(s[i], s[ixp]), phi[i] - phi[ixp]), across), qyo = dmul(dmul(series(s[i], s[iyp]), phi[i] - phi[iyp]), along);
    const double qxi = dmul(dmul(series(s[ixm], s[i]), phi[ixm] - phi[i]), across), qyi = dmul(dmul(series(s[iym], s[i]), phi[iym] - phi[i]), along);
    const double qb = dmul(dmul(series(s[i - layer], s[i]), phi[i - layer] - phi[i]), lt(L, LT_UP, z - 1));
    const double qa = dmul(dmul(series(s[i], s[i + layer]), phi[i] - phi[i + layer]), lt(L, LT_UP, z));
    double change = -dadd(qxo, qyo);
    change = dadd(dadd(change, qxi), qyi);
    change = dadd(dadd(change, qb), -qa);
    if (z == 1) {
      lost -= qb;
      if (corona) {
        const double e0 = -phi[i] / lt(L, LT_DZS, 0), over = fabs(e0) - CORONA_FIELD;
        if (over > 0) {
          const double qc = dmul(dmul(dmul(dmul((e0 > 0 ? 1.0 : -1.0) * CORONA_RATE, over), L.dx), L.dy), dt);
          change = dadd(change, qc); lost -= qc;
        }
      }
    }
    if (z == nz - 2) lost += qa;
    if (change != 0) {
      float* air = field(R, 0, CHARGE_AIR);
      air[i] = (float)dadd((double)air[i], dmul(change, lt(L, LT_PERKG, z)));
    }
  }
  red[threadIdx.x] = lost;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int k = 0; k < (int)blockDim.x; k++) s = dadd(s, red[k]);
    L.part[blockIdx.x] = s;
  }
}
// The conduction's total (in block order) into the run's budget, and the vertical field of the last solve (:1550-1551).
__global__ void k_lgt_conduct_end(const RunDesc R, const LgtDev L, int blocks) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double lost = 0;
    for (int b = 0; b < blocks; b++) lost = dadd(lost, L.part[b]);
    L.st->conducted += lost; R.acc[A_CHG_GROUND] += lost; R.acc[A_CHG_CONDUCTION] += lost;
  }
}
__global__ void k_lgt_fieldz(const RunDesc R, const LgtDev L) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + R.layer;
  if (i >= R.n - R.layer) return;
  const int z = i / R.layer;
  R.ez[i] = (float)(-(L.phi[i + R.layer] - L.phi[i - R.layer]) / lt(L, LT_SPAN, z));
}

__global__ void k_lgt_seed(const LgtDev L, uint32_t rng) {
  if (threadIdx.x == 0 && blockIdx.x == 0) { L.st->rng = rng; L.st->maxBits = 0; L.st->best = INT_MAX; }
}
__global__ void k_lgt_search_reset(const LgtDev L) {
  if (threadIdx.x == 0 && blockIdx.x == 0) { L.st->maxBits = 0; L.st->best = INT_MAX; }
}

inline int blocks(int n, int t) { return (n + t - 1) / t; }

}  // namespace

// ---------------------------------------------------------------- host side
size_t lightning_bytes(int nx, int ny, int nz) {
  const size_t n = (size_t)nx * ny * nz, mh = nx / 2, spec = (size_t)(nz - 2) * (mh + 1) * ny;
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  return al(sizeof(LgtState)) + 6 * al(n * 8) + al(n * 4) + 5 * al(n * 4) + 4 * al((size_t)MAX_CHANNEL * 8) +
         al((size_t)LT_COUNT * nz * 8) + al(((n + 255) / 256 + 1) * 8) + 2 * al(spec * 16) + 2 * al(spec * 8) + al((size_t)nz * 8) +
         al((size_t)nx * 16) + al((size_t)ny * 16);
}

void lightning_bind(char* base, int nx, int ny, int nz, LgtDev& L) {
  const size_t n = (size_t)nx * ny * nz, mh = nx / 2, spec = (size_t)(nz - 2) * (mh + 1) * ny;
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  size_t o = 0;
  auto take = [&](size_t b) { char* p = base + o; o += al(b); return p; };
  L.nz = nz;
  L.st = (LgtState*)take(sizeof(LgtState));
  L.rho = (double*)take(n * 8); L.phi = (double*)take(n * 8); L.sigma = (double*)take(n * 8);
  L.weight = (double*)take(n * 8); L.scale = (double*)take(n * 8); double* spare = (double*)take(n * 8); (void)spare;
  L.cloudy = (float*)take(n * 4);
  L.mark = (int*)take(n * 4); L.seen = (int*)take(n * 4); L.link = (int*)take(n * 4); L.failed = (int*)take(n * 4); L.frontier = (int*)take(n * 4);
  L.nodes = (int*)take(MAX_CHANNEL * 8); L.parent = (int*)take(MAX_CHANNEL * 8); L.polarity = (int*)take(MAX_CHANNEL * 8);
  L.dep = (double*)take(MAX_CHANNEL * 8);
  L.lv = (double*)take((size_t)LT_COUNT * nz * 8);
  L.part = (double*)take(((n + 255) / 256 + 1) * 8);
  L.es.nx = nx; L.es.ny = ny; L.es.nz = nz; L.es.mh = (int)mh;
  L.es.S1 = (double2*)take(spec * 16); L.es.S2 = (double2*)take(spec * 16);
  L.es.cp = (double*)take(spec * 8); L.es.ipiv = (double*)take(spec * 8); L.es.lo = (double*)take((size_t)nz * 8);
  L.es.twx = (double2*)take((size_t)nx * 16); L.es.twy = (double2*)take((size_t)ny * 16);
}

int lightning_init(cudaStream_t st, const sg_grid* g, const double* rho, LgtHost& H) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  LgtDev& L = H.dev;
  L.dx = g->dx; L.dy = g->dy;
  // per-level tables in FP64, each the reference's expression
  std::vector<double> lv((size_t)LT_COUNT * nz, 0.0);
  auto T = [&](int w, int z, double v) { lv[(size_t)w * nz + z] = v; };
  const double dx = g->dx, dy = g->dy;
  for (int z = 0; z < nz; z++) {
    const double h = g->hz[z], e = E_INIT * rho[z] / RHO_STANDARD, Lc = std::cbrt(dx * dy * h);
    T(LT_EINIT, z, e); T(LT_EINIT2, z, std::pow(e, 2)); T(LT_AIR, z, rho[z]); T(LT_ZS, z, g->zs[z]);
    T(LT_CAP, z, SHIELDING * 2 * 3.14159265358979323846 * EPS0 * Lc / std::log(Lc / CHANNEL_RADIUS));        // :179
    T(LT_VOLUME, z, dx * dy * h); T(LT_NODEAIR, z, rho[z] * dx * dy * h); T(LT_PERKG, z, 1 / (rho[z] * dx * dy * h));
    T(LT_SIGMA, z, SIGMA_GROUND * std::exp(g->zs[z] / SIGMA_SCALE));
    T(LT_DZS, z, z < nz - 1 ? g->dzs[z] : 0);
    T(LT_SPAN, z, z > 0 && z < nz - 1 ? g->zs[z + 1] - g->zs[z - 1] : 1);
    T(LT_HZ, z, h);
  }
  H.conductDt = 0;
  H.tables = lv;
  std::vector<double> lo, cpv, ipv;
  std::vector<double2> tx, ty;
  elec_host_tables(nx, ny, nz, dx, dy, g->dzs, g->hz, lo, cpv, ipv, tx, ty);
  cudaError_t e;
  if ((e = cudaMemcpyAsync(L.lv, lv.data(), lv.size() * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(L.es.cp, cpv.data(), cpv.size() * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(L.es.ipiv, ipv.data(), ipv.size() * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(L.es.lo, lo.data(), lo.size() * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(L.es.twx, tx.data(), tx.size() * 16, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(L.es.twy, ty.data(), ty.size() * 16, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return (int)e;
  H.dxy = dx * dy;
  return 0;
}

// The conduction tables depend on dt (across = dy hz dt / dx, along, up = dx dy dt / dzs: :192).
static cudaError_t conduct_tables(cudaStream_t st, const sg_grid* g, LgtHost& H, double dt) {
  if (H.conductDt == dt) return cudaSuccess;
  const int nz = g->nz;
  const double dx = g->dx, dy = g->dy;
  for (int z = 0; z < nz; z++) {
    H.tables[(size_t)LT_ACROSS * nz + z] = dy * g->hz[z] * dt / dx;
    H.tables[(size_t)LT_ALONG * nz + z] = dx * g->hz[z] * dt / dy;
    H.tables[(size_t)LT_UP * nz + z] = z < nz - 1 ? dx * dy * dt / g->dzs[z] : 0;
  }
  H.conductDt = dt;
  return cudaMemcpyAsync(H.dev.lv, H.tables.data(), H.tables.size() * 8, cudaMemcpyHostToDevice, st);
}

static cudaError_t read_state(cudaStream_t st, const LgtHost& H, LgtState& S) {
  cudaError_t e = cudaMemcpyAsync(&S, H.dev.st, sizeof(LgtState), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(st);
}

int lightning_state(cudaStream_t st, LgtHost& H, double* out) {
  LgtState S{};
  if (read_state(st, H, S) != cudaSuccess) return SG_ERR_DEVICE;
  const double v[16] = {(double)S.id, (double)S.start, (double)S.size, (double)S.nnodes, (double)S.ground, (double)S.event, (double)S.left,
                        (double)S.strokes, (double)S.grown, S.potential, S.sum, S.neutralized, S.lowered, S.stage, S.charge, (double)H.flashId};
  for (int k = 0; k < 16; k++) out[k] = v[k];
  return SG_OK;
}

int lightning_probe(cudaStream_t st, const RunDesc& R, LgtHost& H, double* phi, double* rho, int* best, double* ratio) {
  const LgtDev& L = H.dev;
  const int nb = blocks(R.n, 256), ni = blocks(R.n - 2 * R.layer, 256);
  k_lgt_cloudy<<<nb, 256, 0, st>>>(R, L);
  k_lgt_rho<<<nb, 256, 0, st>>>(R, L);
  elec_solve_launch(L.es, L.rho, L.phi, st);
  k_lgt_search_reset<<<1, 32, 0, st>>>(L);
  k_lgt_strongest<<<ni, 256, 0, st>>>(R, L, -1);
  k_lgt_pick<<<ni, 256, 0, st>>>(R, L, -1);
  LgtState S{};
  cudaError_t e;
  if (read_state(st, H, S) != cudaSuccess) return SG_ERR_DEVICE;
  if (phi && (e = cudaMemcpyAsync(phi, L.phi, (size_t)R.n * 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return SG_ERR_DEVICE;
  if (rho && (e = cudaMemcpyAsync(rho, L.rho, (size_t)R.n * 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return SG_ERR_DEVICE;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) return SG_ERR_DEVICE;
  double r2;
  std::memcpy(&r2, &S.maxBits, sizeof(double));
  *best = S.maxBits ? S.best : -1;
  *ratio = S.maxBits ? std::sqrt(r2) : 0;
  return SG_OK;
}

LgtHost::~LgtHost() {
  if (st) { cudaStreamSynchronize(st); cudaStreamDestroy(st); }
  if (hs) cudaFreeHost(hs);
  if (hchan) cudaFreeHost(hchan);
}

int lightning_host_buffers(LgtHost& H) {
  if (!H.st && cudaStreamCreateWithFlags(&H.st, cudaStreamNonBlocking) != cudaSuccess) return SG_ERR_DEVICE;
  if (!H.hs && cudaMallocHost(&H.hs, sizeof(LgtState)) != cudaSuccess) return SG_ERR_DEVICE;
  if (!H.hchan && cudaMallocHost(&H.hchan, 3 * (size_t)MAX_CHANNEL * sizeof(int)) != cudaSuccess) return SG_ERR_DEVICE;
  return SG_OK;
}

namespace {

// The search of pass k of Discharge (:264-268): the charge density and its field, then the strongest field; at the pass
// after the last flash allowed, the conduction and the vertical field instead (:1547-1551).
void launch_finish(const LgtJob& J) {
  const LgtDev& L = J.H->dev;
  const int nb = blocks(J.R.n, 256), ni = blocks(J.R.n - 2 * J.R.layer, 256);
  k_lgt_sigma<<<nb, 256, 0, J.H->st>>>(J.R, L);
  k_lgt_conduct<<<ni, 256, 0, J.H->st>>>(J.R, L, J.H->corona ? 1 : 0, J.dt);
  k_lgt_conduct_end<<<1, 32, 0, J.H->st>>>(J.R, L, ni);
  k_lgt_fieldz<<<ni, 256, 0, J.H->st>>>(J.R, L);
}
void launch_search(LgtJob& J) {
  const LgtDev& L = J.H->dev;
  const int nb = blocks(J.R.n, 256), ni = blocks(J.R.n - 2 * J.R.layer, 256);
  cudaStream_t st = J.H->st;
  k_lgt_rho<<<nb, 256, 0, st>>>(J.R, L);
  elec_solve_launch(L.es, L.rho, L.phi, st);
  if (J.k == J.limit) { launch_finish(J); J.phase = LgtJob::FINISHING; return; }
  k_lgt_search_reset<<<1, 32, 0, st>>>(L);
  k_lgt_strongest<<<ni, 256, 0, st>>>(J.R, L, J.stamp);
  k_lgt_pick<<<ni, 256, 0, st>>>(J.R, L, J.stamp);
  J.phase = LgtJob::SEARCH;
}
void launch_stage(LgtJob& J) {
  k_lgt_grow<<<1, GROW_THREADS, 0, J.H->st>>>(J.R, J.H->dev, J.id);
  k_lgt_deposit<<<1, DEP_THREADS, 0, J.H->st>>>(J.R, J.H->dev);
  J.stage++;
}

// Advances a job by what its last round's state record says (Lightning.discharge and .flash, :259-340).
cudaError_t advance(LgtJob& J) {
  LgtHost& H = *J.H;
  const LgtState& S = *H.hs;
  cudaError_t e = cudaSuccess;
  if (J.pending) {  // the flash that ended last round: its record (its channel was copied behind flash_end)
    J.pending = false;
    if (S.charge != 0) {
      FlashRecord f;
      f.time = J.time; f.cg = S.ground >= 0; f.start = J.start; f.ground = S.ground; f.charge = S.charge;
      f.potential = S.ground >= 0 ? S.before : S.potential; f.moment = S.ground >= 0 ? S.moment : 0;
      f.strokes.assign(S.strokeQ, S.strokeQ + (S.ground >= 0 ? S.nstrokes : 0));
      const int m = J.copied;
      f.nodes.assign(H.hchan, H.hchan + m); f.parent.assign(H.hchan + MAX_CHANNEL, H.hchan + MAX_CHANNEL + m);
      f.polarity.assign(H.hchan + 2 * MAX_CHANNEL, H.hchan + 2 * MAX_CHANNEL + m);
      H.last.push_back(std::move(f));
    }
  }
  switch (J.phase) {
    case LgtJob::SEARCH: {
      double r2;
      std::memcpy(&r2, &S.maxBits, sizeof(double));
      if (S.maxBits == 0 || !(std::sqrt(r2) > 1)) { launch_finish(J); J.phase = LgtJob::DONE; break; }
      J.start = S.best; J.id = ++H.flashId; J.stage = 0;
      k_lgt_flash_begin<<<1, 32, 0, H.st>>>(J.R, H.dev, J.start, J.id);
      launch_stage(J);
      J.phase = LgtJob::FLASH;
      break;
    }
    case LgtJob::FLASH: {
      const bool end = (S.ground >= 0 && (S.strokes >= STROKES || (!S.event && S.nnodes == S.grown))) || (S.ground < 0 && !S.event) ||
                       S.nnodes >= MAX_CHANNEL || J.stage >= STROKES + 8;
      if (!end) {
        // the field of the charge as it now stands; before the contact the channel stays neutral on it
        k_lgt_rho<<<blocks(J.R.n, 256), 256, 0, H.st>>>(J.R, H.dev);
        elec_solve_launch(H.dev.es, H.dev.rho, H.dev.phi, H.st);
        launch_stage(J);
        break;
      }
      k_lgt_flash_end<<<1, 32, 0, H.st>>>(J.R, H.dev, J.stamp);
      J.copied = S.nnodes;
      if ((e = cudaMemcpyAsync(H.hchan, H.dev.nodes, (size_t)S.nnodes * 4, cudaMemcpyDeviceToHost, H.st)) != cudaSuccess ||
          (e = cudaMemcpyAsync(H.hchan + MAX_CHANNEL, H.dev.parent, (size_t)S.nnodes * 4, cudaMemcpyDeviceToHost, H.st)) != cudaSuccess ||
          (e = cudaMemcpyAsync(H.hchan + 2 * MAX_CHANNEL, H.dev.polarity, (size_t)S.nnodes * 4, cudaMemcpyDeviceToHost, H.st)) != cudaSuccess)
        return e;
      J.pending = true;
      J.k++;
      launch_search(J);
      break;
    }
    case LgtJob::FINISHING: J.phase = LgtJob::DONE; break;
    case LgtJob::DONE: break;
  }
  return e;
}

}  // namespace

// The discharges of several runs in lockstep, each on its own stream: a round launches every run's next piece of
// work (a search, a flash stage, the end of a flash and the next search, the conduction), then reads every run's state
// record once; the runs' single-block channel growths run side by side on the SMs.
int lightning_discharge_many(LgtJob* jobs, int n, std::string* err) {
  cudaError_t e = cudaSuccess;
  for (int j = 0; j < n; j++) {
    LgtJob& J = jobs[j];
    LgtHost& H = *J.H;
    if ((e = conduct_tables(H.st, J.g, H, J.dt)) != cudaSuccess) { *err = cudaGetErrorString(e); return SG_ERR_DEVICE; }
    H.last.clear();
    J.stamp = ++H.flashId; J.k = 0; J.pending = false;
    // the random numbers start afresh from the seed and the model time (:263)
    const int32_t tenths = (int32_t)(int64_t)std::floor(J.time * 10 + .5);
    k_lgt_seed<<<1, 32, 0, H.st>>>(H.dev, H.seed ^ (uint32_t)((uint32_t)tenths * 0x9E3779B1u));
    k_lgt_cloudy<<<blocks(J.R.n, 256), 256, 0, H.st>>>(J.R, H.dev);
    launch_search(J);
  }
  int bound = 8;  // rounds: every flash at most STROKES + 9 stages and its end, every pass a search
  for (int j = 0; j < n; j++) bound = std::max(bound, (jobs[j].limit + 2) * (STROKES + 12));
  for (int round = 0; round < bound; round++) {
    bool any = false;
    for (int j = 0; j < n; j++) {
      if (jobs[j].phase == LgtJob::DONE) continue;
      any = true;
      if ((e = cudaMemcpyAsync(jobs[j].H->hs, jobs[j].H->dev.st, sizeof(LgtState), cudaMemcpyDeviceToHost, jobs[j].H->st)) != cudaSuccess) break;
    }
    if (!any || e != cudaSuccess) break;
    for (int j = 0; j < n && e == cudaSuccess; j++)
      if (jobs[j].phase != LgtJob::DONE) e = cudaStreamSynchronize(jobs[j].H->st);
    for (int j = 0; j < n && e == cudaSuccess; j++)
      if (jobs[j].phase != LgtJob::DONE) e = advance(jobs[j]);
    if (e != cudaSuccess) break;
  }
  for (int j = 0; j < n && e == cudaSuccess; j++) e = cudaStreamSynchronize(jobs[j].H->st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) { *err = cudaGetErrorString(e); return SG_ERR_DEVICE; }
  for (int j = 0; j < n; j++)
    if (jobs[j].phase != LgtJob::DONE) { *err = "a discharge did not end within its bound of rounds"; return SG_ERR_DEVICE; }
  return SG_OK;
}

int lightning_discharge(cudaStream_t, const sg_grid* g, const RunDesc& R, LgtHost& H, double time, double dt, int limit, std::string* err) {
  LgtJob J;
  J.g = g; J.R = R; J.H = &H; J.time = time; J.dt = dt; J.limit = limit;
  return lightning_discharge_many(&J, 1, err);
}

}  // namespace sg
