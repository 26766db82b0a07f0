// Host runtime of the device step: context, runs, batch plans, CUDA graphs, the C ABI (include/stormgpu.h) and the
// serving loop. Everything a run needs beyond its fields is precomputed here in FP64 when the run is created: the
// per-level constants, the FP64 LU factorisations of the two vertical tridiagonal families (face projection,
// src/core/advection.ts:222-241; pressure, src/core/pressure.ts:104-140), the FFT twiddles and radix plans.
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <array>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <vector>
#include "../../include/stormgpu.h"
#include "sg_common.cuh"
#include "sg_fft.cuh"
#include "sg_kernels.h"
#include "sg_state.h"
#include "sg_physics.cuh"
#include "sg_lightning.h"

using namespace sg;

namespace {

constexpr int MAX_SLOTS = 4096;
constexpr size_t ALIGN = 256;
const double RK3[3] = {1.0 / 3, 1.0 / 2, 1.0};

size_t align(size_t x) { return (x + ALIGN - 1) / ALIGN * ALIGN; }

struct Layout {
  size_t fld, faces, kmkh, phi, pres, pres2, spec, cols, lv, lv64, triF, triP, ab, twx, twy, scr, part, acc, cnt, items, diag, rot;
  size_t vfall = 0, ez = 0, cpart = 0, lgt = 0, total;  // electrified runs only
};
// One run's allocation (flags: its RF_ELEC / RF_RAIN2M); such a run's sets hold the extra fields too, and it has its
// fall speeds and the vertical field after the rest, an electrified one also the lightning's buffers (sg_lightning.cu).
Layout layout(int nx, int ny, int nz, int flags = 0) {
  const bool extra = flags & RF_EXTRA, elec = flags & RF_ELEC;
  Layout L; size_t n = (size_t)nx * ny * nz, layer = (size_t)nx * ny, nm = nx / 2 + 1, nch = (n + CHUNK - 1) / CHUNK, o = 0;
  auto take = [&](size_t bytes) { size_t at = o; o += align(bytes); return at; };
  L.fld = take(3 * (size_t)(extra ? NFE : NF) * n * 4); L.faces = take(4 * n * 4); L.kmkh = take(2 * n * 4); L.phi = take(n * 4);
  L.pres = take(layer * (nz - 1) * 4); L.pres2 = take(layer * (nz - 1) * 4); L.spec = take(nm * nz * ny * 8); L.cols = take(3 * layer * 4);
  L.lv = take((size_t)L_COUNT * nz * 4); L.lv64 = take((size_t)D_COUNT * nz * 8);
  L.triF = take(nm * nz * ny * 24); L.triP = take(nm * (nz - 1) * ny * 24); L.ab = take(nm * ny * 16);
  L.twx = take(nx * 8); L.twy = take(ny * 8); L.scr = take(64 * 4); L.part = take((nch * NCONS * 3 + nch * 4) * 8);
  L.acc = take(A_COUNT * 8); L.cnt = take(C_COUNT * 8);
  L.items = take(nch * 16);  // the run's own per-node work items (field conversions outside a batch plan)
  L.diag = take((size_t)DG_COUNT * layer * 4); L.rot = take(R_COUNT * 8);
  if (extra) { L.vfall = take(((flags & RF_ICE2M) ? 12 : 6) * n * 4); L.ez = take(n * 4); L.cpart = take(((layer + 63) / 64) * 8); }
  if (elec) L.lgt = take(lightning_bytes(nx, ny, nz));
  L.total = o;
  return L;
}

struct Run {
  bool live = false;
  int slot = -1;
  int nx = 0, ny = 0, nz = 0;
  size_t bytes = 0;
  char* mem = nullptr;
  RunDesc desc{};
  int4* nodeItems = nullptr;  // inside mem
  int nNode = 0;
  double waterStart = 0;      // the water reservoirs' sum when the run began (AtmosphereModel.water.start), kg
  // an electrified run: its lightning, the model time it has reached (the flashes' time and random numbers), its step
  // length, and its grid (the lightning's tables and solve)
  std::unique_ptr<LgtHost> lgt;
  double time = 0, dt = 0;
  std::vector<double> zs, dzs, hz;
  sg_grid grid{};
};

struct Plan {
  std::vector<int> slots;
  int4* items = nullptr;  // device
  int off[24] = {0}, cnt[24] = {0};
  int maxnx = 0, maxny = 0, maxnz = 0, TX = 40, TY = 8, wenoG = 3;  // transport tile and WENO fields per item
  int minb = 2;                                                       // WENO transport blocks per SM (register budget)
  int minnx = 1 << 30;                                                // the narrowest grid of the plan
  bool nx4 = true;                                                    // every grid width a multiple of 4
  bool bulk = false;                                                  // transport inputs by TMA bulk copies (producer warp)
  int yc = 32;                                                        // layer rows per x-transform item
  int mixTX = 32, mixTY = 8;                                          // mixing tile
  int refTX = 16, refTY = 8;                                          // refinement tile
  bool layerAny = false, rowAny = false;                              // some run takes the 2-D layer transforms / the row path
  int rowMaxnx = 0, rowMaxny = 0;                                     // the widest grid of the row path
  size_t fftSmem = 0;                                                 // their shared memory: the largest over the runs
  bool refine = false;                                                // some run refines its final projection
  bool unrefined = false;                                             // some run does not (k_pres_correct<1> has work)
  bool rotation = false;                                              // some run tracks its rotation and swaths
  bool elec = false;                                                  // some run is electrified (charges, lightning)
  bool extra = false;                                                 // some run has the extra fields (electrified or two-moment)
  bool rain2m = false;                                                // some run has two-moment rain
  bool tuned = false;                                                 // TX, TY, wenoG chosen by timing
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~Plan() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (items) cudaFree(items);
  }
};
enum Family { FAM_NODE, FAM_COLS, FAM_ROWS_FACE, FAM_ROWS_PRES, FAM_MODES, FAM_RUNS, FAM_CELLS, FAM_T_WENO, FAM_T_DYN, FAM_MIX,
              FAM_REFINE, FAM_T_CHG, FAM_T_CHG3, FAM_PHYS, FAM_PHYS_LAST = FAM_PHYS + 5, FAM_LROWS_FACE, FAM_LROWS_PRES, FAM_LMODES, FAM_COUNT };

}  // namespace

struct sg_context {
  int device = 0, sms = 0, maxSmem = 0;
  uint64_t budget = 0, used = 0;
  cudaStream_t stream = nullptr;
  RunDesc* d_runs = nullptr;
  std::vector<Run> runs;
  std::vector<int> freeSlots;
  std::map<std::vector<int>, std::unique_ptr<Plan>> plans;
  std::multimap<size_t, char*> pool;   // retired run allocations kept for reuse
  uint64_t pooled = 0;
  std::string error;
  double* d_scalar = nullptr;           // scratch for reductions read back by the host
  // Independent chains of the step (sedimentation, the WENO transport) run on a side stream as parallel branches
  // of the step's graph; dep[] are the events between the branches.
  cudaStream_t side[2] = {nullptr, nullptr};
  cudaEvent_t dep[8] = {};
  bool autotune = true;
  bool tuneLog = false;                 // SG_AUTOTUNE_LOG=1: the tuner prints every candidate's time to stderr
  bool bulk = true;                     // the bulk-copy transport kernels where a plan allows them (SG_TRANSPORT_BULK=0: never)
  bool edgeWarps = true;                // per-thread transport with two edge warps (SG_TRANSPORT_EDGE_WARPS=0: the column threads take the edges)
  bool rowsOnly = false;                // row-transform spectral path for every grid (SG_SPECTRAL_ROWS=1)
  int pinned[4] = {0, 0, 0, 2};         // transport tile, WENO group, blocks per SM fixed by the caller (TX = 0: tune)
  std::map<std::vector<int>, std::array<int, 5>> tuning;  // batch signature -> (TX, TY, wenoG, minb, bulk)
  // packed transfers: a device staging buffer (grown on demand) and the item lists per (runs, mask)
  float* staging = nullptr;
  size_t stagingBytes = 0;
  std::map<std::vector<int>, std::pair<int4*, int>> packs;
  // the groups of sg_batch_step_io: a stream each, the event that ends each group's work, and the event their work
  // starts after (created on first use)
  static constexpr int IO_GROUPS = 8;
  cudaStream_t io[IO_GROUPS] = {};
  cudaEvent_t ioEv[IO_GROUPS + 1] = {};
};

namespace {

int fail(sg_context* ctx, int code, const std::string& msg) { if (ctx) ctx->error = msg; return code; }
int cudaFail(sg_context* ctx, cudaError_t e, const char* where) {
  return fail(ctx, SG_ERR_DEVICE, std::string(where) + ": " + cudaGetErrorString(e));
}
#define CK(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return cudaFail(ctx, e_, #call); } while (0)

// ------------------------------------------------------------------ host precomputation
// triF / triP: the Thomas coefficients of every mode, [m][k][n] TriAB (b, a) followed by [m][k][n] C values.
struct HostTables { std::vector<float> lv; std::vector<double> lv64; std::vector<TriAB> triF, triP; std::vector<double2> ab; std::vector<double> triFc, triPc; std::vector<float2> twx, twy; };

void twiddles(int n, std::vector<float2>& tw) {
  tw.resize(n);
  for (int t = 0; t < n; t++) { double a = -2 * M_PI * t / n; tw[t] = make_float2((float)std::cos(a), (float)std::sin(a)); }
}

// Per-level constants (FP64 -> FP32), the turbulence widths and caps (src/core/turbulence.ts:91-99), the base-theta
// face values for the profile tendency, the mixing coefficients, sponge shares (src/core/model.ts:1369, :1495).
void build_tables(const sg_grid* g, const sg_base_state* b, const sg_switches* sw, HostTables& T, RunDesc& d) {
  const int nx = g->nx, ny = g->ny, nz = g->nz, nm = nx / 2 + 1;
  const double dx = g->dx, dy = g->dy, dt = sw->dt;
  const double* zs = g->zs; const double* dzs = g->dzs; const double* hz = g->hz; const double* rho = b->rho;
  T.lv.assign((size_t)L_COUNT * nz, 0.f); T.lv64.assign((size_t)D_COUNT * nz, 0.0);
  auto L = [&](int w, int z, double v) { T.lv[(size_t)w * nz + z] = (float)v; };
  auto D = [&](int w, int z, double v) { T.lv64[(size_t)w * nz + z] = v; };
  const double G = 9.81, dzMean = g->height / (nz - 1);
  const double* thb = b->theta;
  auto thc = [&](int k) { return thb[std::max(0, std::min(nz - 1, k))]; };
  auto up5 = [](double a, double bb, double c, double dd, double e) { return (2 * a - 13 * bb + 47 * c + 27 * dd - 3 * e) / 60; };
  double cs = sw->cs;
  for (int z = 0; z < nz; z++) {
    double rUp = z < nz - 1 ? (rho[z] + rho[z + 1]) / 2 : 0;
    L(L_RHO, z, rho[z]); L(L_INV_RHO, z, 1 / rho[z]); L(L_HZ, z, hz[z]); L(L_INV_HZ, z, 1 / hz[z]);
    L(L_DZS, z, z < nz - 1 ? dzs[z] : 0); L(L_INV_DZS, z, z < nz - 1 ? 1 / dzs[z] : 0); L(L_RUP, z, rUp);
    // FP32 pairs (value and rounding error) for the refinement's double-FP32 arithmetic
    auto lo = [](double v) { return v - (double)(float)v; };
    L(L_RHO_LO, z, lo(rho[z])); L(L_INV_HZ_LO, z, lo(1 / hz[z])); L(L_INV_DZS_LO, z, z < nz - 1 ? lo(1 / dzs[z]) : 0);
    const double wlo = z > 0 ? dzs[z - 1] / hz[z] : 0, whi = z < nz - 1 ? dzs[z] / hz[z] : 0;
    L(L_WLO, z, wlo); L(L_WLO_LO, z, lo(wlo)); L(L_WHI, z, whi); L(L_WHI_LO, z, lo(whi));
    L(L_EXNER, z, b->exner[z]); L(L_P, z, b->p[z]); L(L_THB, z, thb[z]); L(L_QB, z, b->q[z]);
    double ue = b->u[z] - sw->frame_u, ve = b->v[z] - sw->frame_v;
    L(L_UENV, z, ue); L(L_VENV, z, ve); L(L_THVENV, z, thb[z] * (1 + .61 * b->q[z])); L(L_ZS, z, zs[z]);
    // The base profile's vertical faces minus theta_b(z): the face above (k = z) and below (k = z - 1), each for
    // both flow directions, with the reference's clamped stencils (src/core/advection.ts:356, :366).
    double r0 = thb[z];
    L(L_TH_UP_POS, z, up5(thc(z - 2), thc(z - 1), thc(z), thc(z + 1), thc(z + 2)) - r0);
    L(L_TH_UP_NEG, z, up5(thc(z + 3), thc(z + 2), thc(z + 1), thc(z), thc(z - 1)) - r0);
    L(L_TH_DN_POS, z, up5(thc(z - 3), thc(z - 2), thc(z - 1), thc(z), thc(z + 1)) - r0);
    L(L_TH_DN_NEG, z, up5(thc(z + 2), thc(z + 1), thc(z), thc(z - 1), thc(z - 2)) - r0);
    double local = z == 0 ? dzs[0] : z == nz - 1 ? dzs[nz - 2] : hz[z];
    double len = sw->anisotropic && sw->vertical_dz ? local : std::cbrt(dx * dy * local);
    L(L_LEN2, z, (cs * len) * (cs * len));
    double mn = std::min(dx, dy);
    if (z > 0) mn = std::min(mn, dzs[z - 1]);
    if (z < nz - 1) mn = std::min(mn, dzs[z]);
    L(L_CAP, z, .05 * mn * mn / dt);
    int zu = z < nz - 1 ? z + 1 : z, zd = z > 0 ? z - 1 : z;
    L(L_INV_SPAN, z, 1 / (zs[zu] - zs[zd]));
    L(L_DTHB, z, thb[zu] - thb[zd]);
    L(L_G_OVER_THB, z, G / thb[z]);
    L(L_MIXUP, z, z < nz - 1 ? rUp / (rho[z] * hz[z]) : 0);
    L(L_MIXDN, z, z > 0 ? (rho[z - 1] + rho[z]) / 2 / (rho[z] * hz[z]) : 0);
    L(L_DUENV, z, z < nz - 1 ? (b->u[z + 1] - sw->frame_u) - ue : 0);
    L(L_DVENV, z, z < nz - 1 ? (b->v[z + 1] - sw->frame_v) - ve : 0);
    L(L_DQB, z, z < nz - 1 ? b->q[z + 1] - b->q[z] : 0);
    L(L_FALLSQ, z, std::sqrt(rho[0] / rho[z]));
    double alt = zs[z], H = g->height;
    double sp = alt > sw->sponge_start ? std::max(0.0, std::min(1.0, (alt - sw->sponge_start) / (H - sw->sponge_start))) * sw->sponge_rate * dt : 0;
    L(L_SPONGE, z, sp);
    L(L_NODEMASS, z, dx * dy * hz[z] * rho[z]);
    L(L_LW, z, hz[z] / dzMean * rho[z]);
    L(L_NODEMASS_LO, z, dx * dy * hz[z] * rho[z] - (double)(float)(dx * dy * hz[z] * rho[z]));
    L(L_LW_LO, z, hz[z] / dzMean * rho[z] - (double)(float)(hz[z] / dzMean * rho[z]));
    L(L_SURF, z, 0);
    L(L_TCB, z, thb[z] * b->exner[z] - 273.15);
    {
      phys::Level pl = phys::makeLevel(thb[z], b->exner[z], b->p[z], rho[z], rho[0]);
      T.lv[(size_t)L_QW_HI * nz + z] = pl.qw_hi; T.lv[(size_t)L_QW_LO * nz + z] = pl.qw_lo; T.lv[(size_t)L_BW * nz + z] = pl.bw;
      T.lv[(size_t)L_QI_HI * nz + z] = pl.qi_hi; T.lv[(size_t)L_QI_LO * nz + z] = pl.qi_lo; T.lv[(size_t)L_BI * nz + z] = pl.bi;
      T.lv[(size_t)L_Q0_HI * nz + z] = pl.q0_hi; T.lv[(size_t)L_Q0_LO * nz + z] = pl.q0_lo;
      T.lv[(size_t)L_TCB * nz + z] = pl.tcb;
    }
    double face = z > 0 ? (rho[z - 1] + rho[z]) / 2 : 0;
    D(D_FLO, z, z > 0 ? face / dzs[z - 1] : 0);
    D(D_FHZ, z, hz[z]);
    D(D_PL1, z, z > 0 && z < nz - 1 ? -rho[z] * dzs[z - 1] / (4 * hz[z]) : 0);
    D(D_PL2, z, z > 0 && z < nz - 1 ? rho[z] / (hz[z] * dzs[z]) : 0);
    D(D_THB, z, thb[z]);
  }
  // Face projection factorisation [m][k][n] (src/core/advection.ts:222-241): rows -rho h lambda - lo - up.
  T.triF.assign((size_t)nm * nz * ny, TriAB{0, 0.f, 0.f}); T.triFc.assign((size_t)nm * nz * ny, 0.0);
  std::vector<double> cp(nz);
  auto faceRho = [&](int k) { return k < 0 || k >= nz - 1 ? 0.0 : (rho[k] + rho[k + 1]) / 2; };
  for (int m = 0; m < nm; m++) for (int n = 0; n < ny; n++) {
    double lam = (m == 0 && n == 0) ? 0 : 4 * std::pow(std::sin(M_PI * m / nx), 2) / (dx * dx) + 4 * std::pow(std::sin(M_PI * n / ny), 2) / (dy * dy);
    bool pinned = lam == 0;
    for (int k = 0; k < nz; k++) {
      double lo = k > 0 ? faceRho(k - 1) / dzs[k - 1] : 0, up = k < nz - 1 ? faceRho(k) / dzs[k] : 0, di = -rho[k] * hz[k] * lam - lo - up;
      if (pinned && k == 0) { lo = 0; di = 1; up = 0; }
      if (pinned && k == 1) lo = 0;
      double piv = k == 0 ? di : di - lo * cp[k - 1];
      cp[k] = up / piv;
      // forward sweep d_k = a r_k - b d_(k-1) with a = h_k / pivot (the rows are scaled by h), b = lower / pivot
      const double ip = pinned && k == 0 ? 0.0 : 1 / piv, lower = k > 0 ? faceRho(k - 1) / dzs[k - 1] : 0;
      T.triF[((size_t)m * nz + k) * ny + n] = TriAB{ip * lower, (float)(ip * hz[k]), 0.f};
      T.triFc[((size_t)m * nz + k) * ny + n] = cp[k];
    }
  }
  // Pressure factorisation [m][k][n] (src/core/pressure.ts:37-44, :104-140), the symbols snapped as there.
  const int nc = nz - 1;
  T.triP.assign((size_t)nm * nc * ny, TriAB{0, 0.f, 0.f}); T.triPc.assign((size_t)nm * nc * ny, 0.0);
  T.ab.assign((size_t)nm * ny, make_double2(0, 0));
  auto exact = [](double x) { return x < 1e-12 ? 0 : x > 1 - 1e-12 ? 1 : x; };
  for (int m = 0; m < nm; m++) for (int n = 0; n < ny; n++) {
    double sx = exact(std::pow(std::sin(M_PI * m / nx), 2)), cx = exact(std::pow(std::cos(M_PI * m / nx), 2));
    double sy = exact(std::pow(std::sin(M_PI * n / ny), 2)), cy = exact(std::pow(std::cos(M_PI * n / ny), 2));
    double a = 4 * (sx * cy / (dx * dx) + cx * sy / (dy * dy)), bb = cx * cy;
    T.ab[(size_t)m * ny + n] = make_double2(a, bb);
    if ((a == 0 && bb == 0) || (nc == 1 && a == 0)) continue;  // null modes: zero
    bool pinned = a == 0;
    for (int k = 0; k < nc; k++) {
      double di = -a / 2 * (rho[k] * dzs[k] / (2 * hz[k]) + rho[k + 1] * dzs[k] / (2 * hz[k + 1])), lo = 0, up = 0;
      if (k > 0) { lo = a * T.lv64[(size_t)D_PL1 * nz + k] + bb * T.lv64[(size_t)D_PL2 * nz + k]; di -= bb * rho[k] / (hz[k] * dzs[k]); }
      if (k < nc - 1) { up = -a / 2 * rho[k + 1] * dzs[k + 1] / (2 * hz[k + 1]); double v = bb * rho[k + 1] / (hz[k + 1] * dzs[k]); up += v; di -= v; }
      if (pinned && k == 0) { lo = 0; di = 1; up = 0; }
      if (pinned && k == 1) lo = 0;
      double piv = k == 0 ? di : di - lo * cp[k - 1];
      cp[k] = up / piv;
      const double ip = pinned && k == 0 ? 0.0 : 1 / piv;
      T.triP[((size_t)m * nc + k) * ny + n] = TriAB{ip * lo, (float)ip, 0.f};
      T.triPc[((size_t)m * nc + k) * ny + n] = cp[k];
    }
  }
  twiddles(nx, T.twx); twiddles(ny, T.twy);
  d.nx = nx; d.ny = ny; d.nz = nz; d.layer = nx * ny; d.n = nx * ny * nz; d.nm = nm; d.mh = nx / 2; d.ncells = nx * ny * (nz - 1);
  d.fx_nf = fft_plan_factors(nx, d.fx_rad); d.fy_nf = fft_plan_factors(ny, d.fy_rad);
  d.dx = (float)dx; d.dy = (float)dy; d.inv_dx = (float)(1 / dx); d.inv_dy = (float)(1 / dy); d.dt = (float)dt; d.height = (float)g->height;
  d.inv_dx_lo = (float)(1 / dx - (double)d.inv_dx); d.inv_dy_lo = (float)(1 / dy - (double)d.inv_dy);
  d.inv_dt = (float)(1 / (double)d.dt); d.inv_dt_lo = (float)(1 / (double)d.dt - (double)d.inv_dt);
  d.coriolis = (float)sw->coriolis; d.keep = (float)std::exp(-sw->wind_relaxation * dt); d.sponge_start = (float)sw->sponge_start; d.cs = (float)cs;
  d.drag = (float)(sw->drag_cd * dt / hz[0]); d.frame_u = (float)sw->frame_u; d.frame_v = (float)sw->frame_v;
  d.ue0 = (float)b->u[0]; d.ve0 = (float)b->v[0]; d.env_speed = (float)std::hypot(b->u[0], b->v[0]);
  d.lenH2 = (float)std::pow(cs * std::sqrt(dx * dy), 2); d.capH = (float)(.05 * std::pow(std::min(dx, dy), 2) / dt); d.rho0 = (float)rho[0];
  d.flags = (sw->loading ? RF_LOADING : 0) | (sw->evaporation ? RF_EVAP : 0) | (sw->rain_formation ? RF_RAINFORM : 0) | (sw->anisotropic ? RF_ANISO : 0) |
            (sw->vertical_dz ? RF_VDZ : 0) | (sw->durran_klemp ? RF_DK : 0) | (sw->pressure_in_stages ? RF_STAGES : 0) | (sw->ice ? RF_ICE : 0) |
            (sw->refine_projection ? RF_REFINE : 0) | (sw->rotation ? RF_ROTATION : 0);
  // the rotation tracking's levels (src/core/model.ts:389, :1612) and countCores' (:1653), its threshold (:129)
  const double* zl = g->zs;
  d.uh_z0 = -1; d.uh_z1 = -1; d.uh_top1 = -1; d.uh_top3 = -1; d.core_lo = -1;
  int coreLast = -1;
  for (int z = 0; z < nz; z++) {
    if (d.uh_z0 < 0 && zl[z] >= 2000) d.uh_z0 = z;
    if (zl[z] <= 5000) d.uh_z1 = z;
    if (zl[z] <= 1000) d.uh_top1 = z;
    if (zl[z] <= 3000) d.uh_top3 = z;
    if (d.core_lo < 0 && zl[z] >= 1900) d.core_lo = z;
    if (zl[z] <= 6600) coreLast = z;
  }
  d.core_hi = std::min(nz - 3, coreLast);
  d.meso_zeta = (float)(3e-3 * std::max(1.0, 1200.0 / dx));
}

int validate(sg_context* ctx, const sg_grid* g, const sg_base_state* b, const sg_switches* sw) {
  if (!g || !b || !sw) return fail(ctx, SG_ERR_INVALID, "null grid, base state or switches");
  if (g->nx < 1 || g->ny < 1 || g->nz < 3) return fail(ctx, SG_ERR_INVALID, "grid needs nx, ny >= 1 and nz >= 3");
  if (g->nz > 128) return fail(ctx, SG_ERR_UNSUPPORTED, "nz > 128 levels");
  if (g->nx > 4096 || g->ny > 4096) return fail(ctx, SG_ERR_UNSUPPORTED, "nx or ny > 4096");
  // the kernels index a run's field sets with 32-bit element offsets
  if ((size_t)g->nx * g->ny * g->nz * 3 * ((sw->lightning || sw->rain_moments == 2) ? NFE : NF) >= (1ull << 31))
    return fail(ctx, SG_ERR_UNSUPPORTED, "grid beyond 55 million nodes");
  if (sw->rain_moments != 1 && sw->rain_moments != 2) return fail(ctx, SG_ERR_INVALID, "rain_moments must be 1 or 2");
  if (sw->rain_breakup < 0 || sw->rain_breakup > 2) return fail(ctx, SG_ERR_INVALID, "rain_breakup must be 0 (none), 1 (NSSL) or 2 (Morrison)");
  if (sw->ice_moments != 1 && sw->ice_moments != 2) return fail(ctx, SG_ERR_INVALID, "ice_moments must be 1 or 2");
  int rad[8];
  if (fft_plan_factors(g->nx, rad) < 0 || fft_plan_factors(g->ny, rad) < 0) return fail(ctx, SG_ERR_UNSUPPORTED, "nx or ny has more than 8 prime factors");
  if (!(g->dx > 0 && g->dy > 0 && g->height > 0) || !g->zs || !g->dzs || !g->hz) return fail(ctx, SG_ERR_INVALID, "bad grid spacing or levels");
  if (!b->p || !b->exner || !b->theta || !b->q || !b->u || !b->v || !b->rho) return fail(ctx, SG_ERR_INVALID, "null base-state array");
  for (int z = 0; z < g->nz; z++) if (!(b->rho[z] > 0) || !(b->theta[z] > 0) || !(g->hz[z] > 0)) return fail(ctx, SG_ERR_INVALID, "non-positive rho, theta or hz");
  if (!(sw->dt > 0)) return fail(ctx, SG_ERR_INVALID, "dt must be positive");
  if (!sw->pressure_in_stages) return fail(ctx, SG_ERR_UNSUPPORTED, "the device step needs the pressure in the RK3 stages");
  // the lightning's potential solve holds a row, a column and a half spectrum of a level in shared memory
  if (sw->lightning && sw->ice && (g->nx > 2048 || g->ny > 2048)) return fail(ctx, SG_ERR_UNSUPPORTED, "lightning: nx and ny at most 2048");
  // The shared memory of the mode kernel: (nz + 8) * ny complex values.
  size_t smem = (size_t)(g->nz + 8) * g->ny * 8;
  if ((int)smem > ctx->maxSmem) return fail(ctx, SG_ERR_UNSUPPORTED, "(nz + 8) * ny too large for one block's shared memory");
  return SG_OK;
}

Run* find(sg_context* ctx, sg_run run) {
  if (run < 0 || run >= (int)ctx->runs.size() || !ctx->runs[run].live) return nullptr;
  return &ctx->runs[run];
}

// ------------------------------------------------------------------ plans
// Transport work items (run, field group, tile) of a plan for a tile shape and WENO group size: groups 0-2 are the
// WENO fields in threes, 4-12 one by one, 3 the dynamics {u, v, w, theta'}.
void transport_items(sg_context* ctx, const std::vector<int>& slots, int TX, int TY, int wenoG, std::vector<int4>* fam) {
  for (int s : slots) {
    const Run& r = ctx->runs[s];
    const int tiles = ((r.nx + TX - 1) / TX) * ((r.ny + TY - 1) / TY);
    const int grp0 = wenoG == 3 ? 0 : 4, ngrp = wenoG == 3 ? 3 : 9;
    for (int g = grp0; g < grp0 + ngrp; g++) for (int t = 0; t < tiles; t++) fam[0].push_back(make_int4(s, g, t, 0));
    for (int t = 0; t < tiles; t++) fam[1].push_back(make_int4(s, 3, t, 0));
  }
}

// The extra fields of the plan's runs, one WENO field an item on the plan's tile: the charge carriers of the
// electrified runs (groups 13-16), the raindrop number of the two-moment ones (group 17).
// The extra fields' transport items: three fields an item where a run carries a whole triple (groups 22: the first
// three charge carriers, 23: the drop number with graupel's number and volume, 24: hail's number and volume with the
// ions' charge), the rest one an item (groups 13-21).
void charge_items(sg_context* ctx, const std::vector<int>& slots, int TX, int TY, std::vector<int4>& out, std::vector<int4>& out3) {
  out.clear(); out3.clear();
  for (int s : slots) {
    const Run& r = ctx->runs[s];
    const int tiles = ((r.nx + TX - 1) / TX) * ((r.ny + TY - 1) / TY);
    const bool elec = r.desc.flags & RF_ELEC, rain2 = r.desc.flags & RF_RAIN2M, ice2 = r.desc.flags & RF_ICE2M;
    std::vector<int> ones, threes;
    if (elec) threes.push_back(22);
    if (ice2) threes.push_back(23); else if (rain2) ones.push_back(17);
    if (elec && ice2) threes.push_back(24);
    else {
      if (elec) ones.push_back(16);
      if (ice2) { ones.push_back(20); ones.push_back(21); }
    }
    for (int g : threes) for (int t = 0; t < tiles; t++) out3.push_back(make_int4(s, g, t, 0));
    for (int g : ones) for (int t = 0; t < tiles; t++) out.push_back(make_int4(s, g, t, 0));
  }
}

// The physics kernel variant of a run: (electrified ? 3 : 0) + its moments - 1 (k_physics<ELEC, MOM>).
int physics_variant(int flags) {
  return ((flags & RF_ELEC) ? 3 : 0) + ((flags & RF_ICE2M) ? 2 : (flags & RF_RAIN2M) ? 1 : 0);
}

int upload_items(sg_context* ctx, Plan& P, std::vector<int4>* all) {
  std::vector<int4> flat;
  for (int f = 0; f < FAM_COUNT; f++) { P.off[f] = (int)flat.size(); P.cnt[f] = (int)all[f].size(); flat.insert(flat.end(), all[f].begin(), all[f].end()); }
  if (P.items) { cudaFree(P.items); P.items = nullptr; }
  CK(cudaMalloc(&P.items, flat.size() * sizeof(int4)));
  CK(cudaMemcpy(P.items, flat.data(), flat.size() * sizeof(int4), cudaMemcpyHostToDevice));
  return SG_OK;
}

int autotune_transport(sg_context* ctx, Plan& P);

int build_plan(sg_context* ctx, const std::vector<int>& slots, Plan& P) {
  P.slots = slots;
  std::vector<int4> all[FAM_COUNT];
  bool all40 = true;
  for (int s : slots) {
    const Run& r = ctx->runs[s];
    P.maxnx = std::max(P.maxnx, r.nx); P.maxny = std::max(P.maxny, r.ny); P.maxnz = std::max(P.maxnz, r.nz);
    P.minnx = std::min(P.minnx, r.nx); P.nx4 = P.nx4 && r.nx % 4 == 0;
    if (r.nx % 40) all40 = false;
  }
  // Default transport tile: 40 x 8 columns when every grid is a multiple of 40 wide, else 32 x 8 (a tile may be
  // wider than a small grid: its halo wraps periodically and the threads beyond the grid only load); the WENO fields
  // in threes. The autotuner below replaces these by the fastest measured shape.
  P.TX = all40 ? 40 : 32;
  P.TY = 8;
  P.wenoG = 3;
  // Spectral solves, chosen run by run (so a run's bits do not depend on its batch): when a layer's spectrum fits in
  // shared memory (the 40x32 and 80x64 grids), whole layers are transformed in 2-D and the mode kernel is a pure FP64
  // sweep; otherwise rows of 16 or 32 are x-transformed and the mode kernel transforms along y around its sweep.
  auto layerPath = [&](const Run& r) { return !ctx->rowsOnly && layer_fft_smem(r.nx, r.ny) <= (size_t)std::min(ctx->maxSmem, 100 * 1024); };
  for (int s : slots) {
    const Run& r = ctx->runs[s];
    if (layerPath(r)) { P.layerAny = true; P.fftSmem = std::max(P.fftSmem, layer_fft_smem_run(r.nx, r.ny)); }
    else { P.rowAny = true; P.rowMaxnx = std::max(P.rowMaxnx, r.nx); P.rowMaxny = std::max(P.rowMaxny, r.ny); }
  }
  P.yc = P.rowAny ? std::min(P.rowMaxnx > 128 ? 16 : 32, (P.rowMaxny + 1) / 2 * 2) : 32;
  for (int s : slots) {
    const Run& r = ctx->runs[s];
    int n = r.nx * r.ny * r.nz, nch = (n + CHUNK - 1) / CHUNK, layer = r.nx * r.ny;
    for (int c = 0; c < nch; c++) all[FAM_NODE].push_back(make_int4(s, c, 0, 0));
    // the physics' node chunks by kernel variant: a run takes the same physics code whatever batch it is in
    for (int c = 0; c < nch; c++) all[FAM_PHYS + physics_variant(r.desc.flags)].push_back(make_int4(s, c, 0, 0));
    int ncc = (r.nx * r.ny * (r.nz - 1) + CHUNK - 1) / CHUNK;
    for (int c = 0; c < ncc; c++) all[FAM_CELLS].push_back(make_int4(s, c, 0, 0));
    for (int c = 0; c < (layer + 63) / 64; c++) all[FAM_COLS].push_back(make_int4(s, c, 0, 0));
    if (layerPath(r)) {  // a layer an item
      for (int k = 0; k < r.nz; k++) all[FAM_LROWS_FACE].push_back(make_int4(s, k, 0, 0));
      for (int k = 0; k < r.nz - 1; k++) all[FAM_LROWS_PRES].push_back(make_int4(s, k, 0, 0));
      for (int m = 0; m < r.nx / 2 + 1; m++) all[FAM_LMODES].push_back(make_int4(s, m, 0, 0));
    } else {
      for (int k = 0; k < r.nz; k++) for (int y = 0; y < r.ny; y += P.yc) all[FAM_ROWS_FACE].push_back(make_int4(s, k, y, 0));
      for (int k = 0; k < r.nz - 1; k++) for (int y = 0; y < r.ny; y += P.yc) all[FAM_ROWS_PRES].push_back(make_int4(s, k, y, 0));
      for (int m = 0; m < r.nx / 2 + 1; m++) all[FAM_MODES].push_back(make_int4(s, m, 0, 0));
    }
    all[FAM_RUNS].push_back(make_int4(s, 0, 0, 0));
    if (r.desc.flags & RF_REFINE) P.refine = true; else P.unrefined = true;
    if (r.desc.flags & RF_ROTATION) P.rotation = true;
    if (r.desc.flags & RF_ELEC) P.elec = true;
    if (r.desc.flags & RF_EXTRA) P.extra = true;
    if (r.desc.flags & RF_RAIN2M) P.rain2m = true;
  }
  // mixing items: (run, tile, z0, z1), the column in four level ranges
  P.mixTX = all40 ? 40 : 32; P.mixTY = 8;
  for (int s : slots) {
    const Run& r = ctx->runs[s];
    const int tiles = ((r.nx + P.mixTX - 1) / P.mixTX) * ((r.ny + P.mixTY - 1) / P.mixTY), zc = (r.nz + 3) / 4;
    for (int t = 0; t < tiles; t++)
      for (int z0 = 0; z0 < r.nz; z0 += zc) all[FAM_MIX].push_back(make_int4(s, t, z0, std::min(r.nz, z0 + zc)));
  }
  // refinement items (refined runs only): (run, tile, z0, z1) on tiles whose nodes, halo included, fit one block
  P.refTX = all40 ? 20 : 16; P.refTY = 8;
  for (int s : slots) {
    const Run& r = ctx->runs[s];
    if (!(r.desc.flags & RF_REFINE)) continue;
    const int tiles = ((r.nx + P.refTX - 1) / P.refTX) * ((r.ny + P.refTY - 1) / P.refTY), zc = (r.nz + 3) / 4;
    for (int t = 0; t < tiles; t++)
      for (int z0 = 0; z0 < r.nz; z0 += zc) all[FAM_REFINE].push_back(make_int4(s, t, z0, std::min(r.nz, z0 + zc)));
  }
  if (ctx->pinned[0]) { P.TX = ctx->pinned[0]; P.TY = ctx->pinned[1]; P.wenoG = ctx->pinned[2]; P.minb = ctx->pinned[3]; }
  P.bulk = P.minb == 2 && ctx->bulk && transport_bulk_ok(P.TX, P.TY, P.minnx, P.nx4) &&
           std::max(transport_smem_bulk(TK_WENO, P.wenoG, P.TX, P.TY), transport_smem_bulk(TK_DYN, 4, P.TX, P.TY)) <= (size_t)ctx->maxSmem;
  transport_items(ctx, slots, P.TX, P.TY, P.wenoG, all + FAM_T_WENO);
  charge_items(ctx, slots, P.TX, P.TY, all[FAM_T_CHG], all[FAM_T_CHG3]);
  int st = upload_items(ctx, P, all);
  if (st != SG_OK) return st;
  return ctx->autotune && !ctx->pinned[0] ? autotune_transport(ctx, P) : SG_OK;
}

Launch lx(sg_context* ctx, const Plan& P, int fam, int capPerSm = 8) {
  return Launch{ctx->d_runs, P.items + P.off[fam], P.cnt[fam], ctx->sms * capPerSm, ctx->stream};
}

// The extra fields' WENO transport of one RK3 stage (electrified and two-moment runs; per-thread copies): the items of
// three fields, then those of one.
void launch_charges(sg_context* ctx, const Plan& P, int in, int out, float frac, int stage, cudaStream_t stream) {
  Launch C3 = lx(ctx, P, FAM_T_CHG3);
  C3.cap = C3.n; C3.stream = stream;
  if (C3.n) launch_transport(C3, TK_WENO, 3, P.minb, in, out, frac, stage, P.TX, P.TY, false, false);  // (no edge warps: see the kernel)
  Launch C = lx(ctx, P, FAM_T_CHG);
  C.cap = C.n; C.stream = stream;
  if (C.n) launch_transport(C, TK_WENO, 1, P.minb, in, out, frac, stage, P.TX, P.TY, false, ctx->edgeWarps);
}

// Transport launches: one block per item, so the hardware block scheduler balances items of uneven cost (tiles of
// empty air skip their WENO weights) across the SMs.
void launch_transport_kinds(sg_context* ctx, const Plan& P, int in, int out, float frac, int stage, int hookBase,
                            const std::function<void(int)>& hook) {
  const int fams[2] = {FAM_T_WENO, FAM_T_DYN};
  for (int k = 0; k < 2; k++) {
    Launch L = lx(ctx, P, fams[k]);
    L.cap = L.n;
    if (L.n) launch_transport(L, k, P.wenoG, P.minb, in, out, frac, stage, P.TX, P.TY, P.bulk, ctx->edgeWarps);
    hook(hookBase + k);
    if (k == 0 && P.extra) { launch_charges(ctx, P, in, out, frac, stage, ctx->stream); hook(29); }
  }
}

// Picks the transport tile (TX x TY columns) and WENO fields per item by timing every candidate on the plan's own
// runs: the two transport kinds of one RK3 stage (set A in, set C out; C is scratch between steps), best of three
// after a warm-up. Results are cached per batch signature (the sorted grid shapes, and the run count to a power of
// two), so a serving loop whose batch changes run by run tunes each kind of batch once.
int autotune_transport(sg_context* ctx, Plan& P) {
  std::vector<int> sig;
  for (int s : P.slots) { const Run& r = ctx->runs[s]; sig.push_back(r.nx); sig.push_back(r.ny); sig.push_back(r.nz); }
  {
    std::vector<std::array<int, 3>> dims;
    for (size_t i = 0; i < sig.size(); i += 3) dims.push_back({sig[i], sig[i + 1], sig[i + 2]});
    std::sort(dims.begin(), dims.end());
    dims.erase(std::unique(dims.begin(), dims.end()), dims.end());
    sig.clear();
    for (auto& d : dims) sig.insert(sig.end(), d.begin(), d.end());
    int c = 1; while (c < (int)P.slots.size()) c *= 2;
    sig.push_back(c);
  }
  std::array<int, 5> best{P.TX, P.TY, P.wenoG, P.minb, P.bulk ? 1 : 0};
  auto it = ctx->tuning.find(sig);
  if (it != ctx->tuning.end()) {
    best = it->second;
  } else {
    static const int shapes[][2] = {{40, 8}, {32, 8}, {20, 8}, {16, 16}, {16, 8}, {40, 4}, {32, 4}, {8, 8}};
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    float bestMs = 1e30f;
    Plan T;  // candidate items only
    T.slots = P.slots; T.maxnx = P.maxnx; T.maxny = P.maxny; T.maxnz = P.maxnz; T.minnx = P.minnx; T.nx4 = P.nx4;
    for (auto& sh : shapes) {
      const int TX = sh[0], TY = sh[1];
      if (TX > 2 * P.maxnx || TY > 2 * P.maxny) continue;
      // variants: per-thread copies at 2 or 3 blocks an SM, and (where the shape allows them) the bulk copies at 2
      for (int G : {3, 1}) for (int V : {0, 1, 2}) {
        const int MB = V == 1 ? 3 : 2;
        const bool bulk = V == 2;
        if (bulk && !(ctx->bulk && transport_bulk_ok(TX, TY, P.minnx, P.nx4))) continue;
        const size_t need = bulk ? std::max(transport_smem_bulk(TK_WENO, G, TX, TY), transport_smem_bulk(TK_DYN, 4, TX, TY))
                                 : transport_smem(TK_WENO, G, TX, TY);
        if (need > (size_t)ctx->maxSmem) continue;
        std::vector<int4> all[FAM_COUNT];
        transport_items(ctx, P.slots, TX, TY, G, all + FAM_T_WENO);
        int st = upload_items(ctx, T, all);
        if (st != SG_OK) { cudaEventDestroy(e0); cudaEventDestroy(e1); return st; }
        T.TX = TX; T.TY = TY; T.wenoG = G; T.minb = MB; T.bulk = bulk;
        float ms = 1e30f;
        for (int rep = 0; rep < 4; rep++) {
          cudaEventRecord(e0, ctx->stream);
          launch_transport_kinds(ctx, T, 0, 2, 1.f / 3.f, 0, 0, [](int) {});
          cudaEventRecord(e1, ctx->stream);
          CK(cudaEventSynchronize(e1));
          float t = 0; cudaEventElapsedTime(&t, e0, e1);
          if (rep) ms = std::min(ms, t);
        }
        CK(cudaGetLastError());
        if (ctx->tuneLog) fprintf(stderr, "stormgpu tuner: tile %dx%d, %d WENO fields an item, %d blocks an SM, %s: %.4f ms\n", TX, TY, G, MB,
                                  bulk ? "bulk copies" : "per-thread copies", ms);
        if (ms < bestMs) { bestMs = ms; best = {TX, TY, G, MB, bulk ? 1 : 0}; }
      }
    }
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    ctx->tuning[sig] = best;
  }
  P.TX = best[0]; P.TY = best[1]; P.wenoG = best[2]; P.minb = best[3]; P.bulk = best[4] != 0; P.tuned = true;
  std::vector<int4> all[FAM_COUNT];
  for (int f = 0; f < FAM_COUNT; f++) {  // keep the other families, rebuild the transport ones
    if (f == FAM_T_WENO || f == FAM_T_DYN || f == FAM_T_CHG || f == FAM_T_CHG3) continue;
    all[f].resize(P.cnt[f]);
    if (P.cnt[f]) CK(cudaMemcpy(all[f].data(), P.items + P.off[f], P.cnt[f] * sizeof(int4), cudaMemcpyDeviceToHost));
  }
  transport_items(ctx, P.slots, P.TX, P.TY, P.wenoG, all + FAM_T_WENO);
  charge_items(ctx, P.slots, P.TX, P.TY, all[FAM_T_CHG], all[FAM_T_CHG3]);
  return upload_items(ctx, P, all);
}

// The three stages of a spectral solve (divergence and forward transform, mode solves, inverse transform) on the
// plan's rows and modes, on the stream of `rows`.
template <class Hook>
void enqueue_solve(sg_context* ctx, const Plan& P, int mode, int set, cudaStream_t stream, Hook hook) {
  const int h = mode == PROJ_FACE ? 2 : mode == PROJ_PRES ? 7 : 22;  // profile ids of the three stages
  if (P.layerAny) {  // the runs whose layers transform in 2-D
    Launch rows = lx(ctx, P, mode == PROJ_FACE ? FAM_LROWS_FACE : FAM_LROWS_PRES), modes = lx(ctx, P, FAM_LMODES);
    rows.cap = rows.n;
    modes.cap = modes.n;  // one block per wavenumber: its column solves are serial in z, so spread them over the SMs
    rows.stream = modes.stream = stream;
    launch_proj_div_fft2(rows, mode, set, P.fftSmem); hook(h);
    launch_proj_sweep(modes, mode, P.maxny); hook(h + 1);
    launch_proj_ifft2(rows, mode, P.fftSmem); hook(h + 2);
  }
  if (P.rowAny) {  // the runs of the row path
    Launch rows = lx(ctx, P, mode == PROJ_FACE ? FAM_ROWS_FACE : FAM_ROWS_PRES), modes = lx(ctx, P, FAM_MODES);
    rows.cap = rows.n;
    modes.cap = modes.n;
    rows.stream = modes.stream = stream;
    const int mthreads = std::min(512, std::max(64, (2 * P.rowMaxny + 31) / 32 * 32));
    const int mbudget = std::min(ctx->maxSmem, 200 * 1024);
    launch_proj_div_xfft(rows, mode, set, P.yc, P.rowMaxnx); hook(h);
    launch_proj_modes(modes, mode, P.maxnz, P.rowMaxny, mthreads, mbudget); hook(h + 1);
    launch_proj_xifft(rows, mode, P.yc, P.rowMaxnx); hook(h + 2);
  }
}

// The pressure projection of one set (a stage projection, or the final one with the wind limits and, for refined
// runs, the refinement pass).
template <class Hook>
void enqueue_project(sg_context* ctx, const Plan& P, int set, int final_, cudaStream_t stream, Hook hook) {
  Launch node = lx(ctx, P, FAM_NODE), cells = lx(ctx, P, FAM_CELLS);
  node.stream = cells.stream = stream;
  enqueue_solve(ctx, P, PROJ_PRES, set, stream, hook);
  // the final correction of unrefined runs (refined runs take theirs from both pressures below): not launched when
  // every run of the plan refines
  if (!final_ || P.unrefined) { launch_pres_correct(node, set, final_); hook(final_ ? 16 : 10); }
  if (final_ && P.refine) {
    Launch rr = lx(ctx, P, FAM_REFINE);
    rr.cap = rr.n; rr.stream = stream;
    launch_refine_residual(rr, set, P.refTX, P.refTY); hook(20);
    enqueue_solve(ctx, P, PROJ_GIVEN, set, stream, hook);
    launch_refine_correct(node, set); hook(25);
  }
}

// The step's launch sequence for a plan in five parts (the oracle's partition of AtmosphereModel.step):
// 1 beginStep (fall speeds, sedimentation), 2 dynamics (face projection, RK3 stages with their projections),
// 3 physicsStep (positivity fix, physics), 4 mixStep (viscosity, mixing, drag), 5 the final projection and the
// end-of-step counters. `hook(k)` is called after each launch (profiling). Everything runs in order on the context's
// stream.
template <class Hook>
void enqueue_part(sg_context* ctx, const Plan& P, int part, Hook hook) {
  const int A = 0, B = 1, C = 2;
  cudaStream_t st = ctx->stream;
  Launch node = lx(ctx, P, FAM_NODE), cols = lx(ctx, P, FAM_COLS), runs = lx(ctx, P, FAM_RUNS);
  if (part == 1) {
    launch_fall_courant(node); hook(0);
    launch_sediment(cols, P.maxnz); hook(1);
    if (P.rain2m) { launch_sediment_2m(cols, P.maxnz); hook(28); }
  } else if (part == 2) {
    enqueue_solve(ctx, P, PROJ_FACE, A, st, hook);
    launch_face_correct(node, A); hook(5);
    const int in[3] = {A, B, C}, out[3] = {B, C, B};
    for (int s = 0; s < 3; s++) {
      launch_transport_kinds(ctx, P, in[s], out[s], (float)RK3[s], s, 18, hook);
      if (s < 2) enqueue_project(ctx, P, out[s], 0, st, hook);
    }
  } else if (part == 3) {
    launch_fill_partial(node, B); hook(11);
    launch_fill_final(runs); hook(12);
    for (int v = 0; v < 6; v++) launch_physics(lx(ctx, P, FAM_PHYS + v), B, C, v);
    hook(13);
  } else if (part == 4) {
    launch_viscosity(node, C); hook(14);
    Launch mx = lx(ctx, P, FAM_MIX);
    mx.cap = mx.n;
    launch_mix(mx, C, P.mixTX, P.mixTY); hook(15);
  } else if (part == 5) {
    enqueue_project(ctx, P, A, 1, st, hook);
    launch_step_end(runs); hook(17);
    if (P.rotation) {  // afterStep (src/core/model.ts:1130-1131): the rotation tracking, and the swaths
      launch_rotation_columns(cols, 0); hook(26);
      launch_rotation_summary(runs, 0); hook(27);
    }
  }
}

// Parts 1 and 2 for a graph, with their independent chains on parallel branches (the same launches and the same
// results as the serial order):
//  * sedimentation (the falling fields of set A) alongside the face projection (u, v, w of set A);
//  * the WENO transport of the three RK3 stages as one chain, alongside the chain of the dynamics transport
//    (u, v, w, theta') and the stage projections. A WENO stage needs only the face fluxes, the step-start values and
//    its input scalars; the dynamics stage 0 reads the step-start precipitation after the sedimentation (its
//    buoyancy's condensate load), stage s > 0 the scalars WENO stage s - 1 wrote, and WENO stage 2 overwrites the
//    scalars of set B only after dynamics stage 1 has read them.
void enqueue_dynamics_graph(sg_context* ctx, const Plan& P) {
  const int A = 0, B = 1, C = 2;
  auto none = [](int) {};
  cudaStream_t main = ctx->stream, side = ctx->side[1];
  cudaEvent_t* ev = ctx->dep;
  Launch node = lx(ctx, P, FAM_NODE), cols = lx(ctx, P, FAM_COLS);
  Launch nodeS = node, colsS = cols;
  nodeS.stream = colsS.stream = side;
  cudaEventRecord(ev[0], main);
  cudaStreamWaitEvent(side, ev[0], 0);
  launch_fall_courant(nodeS);
  launch_sediment(colsS, P.maxnz);
  if (P.rain2m) launch_sediment_2m(colsS, P.maxnz);
  cudaEventRecord(ev[6], side);  // the sedimented precipitation (the dynamics' stage-0 buoyancy loads it)
  enqueue_solve(ctx, P, PROJ_FACE, A, main, none);
  launch_face_correct(node, A);
  cudaEventRecord(ev[1], main);
  cudaStreamWaitEvent(side, ev[1], 0);  // the face fluxes
  Launch W = lx(ctx, P, FAM_T_WENO), D = lx(ctx, P, FAM_T_DYN);
  W.cap = W.n; D.cap = D.n; W.stream = side;
  const int in[3] = {A, B, C}, out[3] = {B, C, B};
  // ev[2 + s]: WENO stage s done; ev[5]: dynamics stage 1 done; ev[6]: the sedimentation done
  for (int s = 0; s < 3; s++) {
    if (s == 2) cudaStreamWaitEvent(side, ev[5], 0);     // dynamics stage 1 has read set B's scalars
    if (W.n) launch_transport(W, TK_WENO, P.wenoG, P.minb, in[s], out[s], (float)RK3[s], s, P.TX, P.TY, P.bulk, ctx->edgeWarps);
    launch_charges(ctx, P, in[s], out[s], (float)RK3[s], s, side);
    cudaEventRecord(ev[2 + s], side);
    // the stage's input scalars: for stage 0 the step-start fields after the sedimentation, later the WENO stage's
    cudaStreamWaitEvent(main, s == 0 ? ev[6] : ev[1 + s], 0);
    if (D.n) launch_transport(D, TK_DYN, P.wenoG, P.minb, in[s], out[s], (float)RK3[s], s, P.TX, P.TY, P.bulk, ctx->edgeWarps);
    if (s == 1) cudaEventRecord(ev[5], main);
    if (s < 2) enqueue_project(ctx, P, out[s], 0, main, none);
  }
  cudaStreamWaitEvent(main, ev[4], 0);
}

template <class Hook>
void enqueue_step(sg_context* ctx, const Plan& P, Hook hook) {
  for (int part = 1; part <= 5; part++) enqueue_part(ctx, P, part, hook);
}
// The same step with parallel branches, for graph capture.
void enqueue_step_graph(sg_context* ctx, const Plan& P) {
  auto none = [](int) {};
  enqueue_dynamics_graph(ctx, P);
  for (int part = 3; part <= 5; part++) enqueue_part(ctx, P, part, none);
}
const int NKERNELS = 30;
const char* KERNEL_NAMES[NKERNELS] = {"fall_courant", "sediment", "face_div_xfft", "face_modes", "face_xifft", "face_correct", "transport",
                                      "pres_div_xfft", "pres_modes", "pres_xifft", "pres_correct", "fill_partial", "fill_final", "physics",
                                      "viscosity", "mix", "pres_correct_final", "step_end", "transport_weno", "transport_dynamics",
                                      "refine_residual", "refine_unused", "refine_div_xfft", "refine_modes", "refine_xifft", "refine_correct",
                                      "rotation_columns", "rotation_summary", "sediment_2m", "transport_extra"};

Plan* get_plan(sg_context* ctx, const std::vector<int>& slots, int* status) {
  auto it = ctx->plans.find(slots);
  if (it != ctx->plans.end()) { *status = SG_OK; return it->second.get(); }
  if (ctx->plans.size() > 256) ctx->plans.clear();
  auto P = std::make_unique<Plan>();
  *status = build_plan(ctx, slots, *P);
  if (*status != SG_OK) return nullptr;
  Plan* raw = P.get();
  ctx->plans[slots] = std::move(P);
  return raw;
}

int ensure_graph(sg_context* ctx, Plan& P) {
  if (P.exec) return SG_OK;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_step_graph(ctx, P);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &P.graph);
  if (e != cudaSuccess) return cudaFail(ctx, e, "cudaStreamEndCapture");
  CK(cudaGraphInstantiate(&P.exec, P.graph, 0));
  return SG_OK;
}

void drop_packs_with(sg_context* ctx, int slot) {
  for (auto it = ctx->packs.begin(); it != ctx->packs.end();) {
    if (std::find(it->first.begin(), it->first.end() - 1, slot) != it->first.end() - 1) { cudaFree(it->second.first); it = ctx->packs.erase(it); }
    else ++it;
  }
}

void drop_plans_with(sg_context* ctx, int slot) {
  for (auto it = ctx->plans.begin(); it != ctx->plans.end();) {
    if (std::find(it->first.begin(), it->first.end(), slot) != it->first.end()) it = ctx->plans.erase(it);
    else ++it;
  }
}

int slots_of(sg_context* ctx, const sg_run* runs, int n, std::vector<int>& slots) {
  if (n < 1 || !runs) return fail(ctx, SG_ERR_INVALID, "empty batch");
  for (int k = 0; k < n; k++) {
    if (!find(ctx, runs[k])) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(runs[k]));
    slots.push_back(runs[k]);
  }
  std::vector<int> s = slots; std::sort(s.begin(), s.end());
  if (std::adjacent_find(s.begin(), s.end()) != s.end()) return fail(ctx, SG_ERR_INVALID, "a run appears twice in the batch");
  return SG_OK;
}

// The lightning of a batch's electrified runs after their step (afterStep, src/core/model.ts:1130-1133), all of them
// together: the flash time is the step's end (time + dt, :1542), so each run's time moves by its dt first. Runs that
// failed are left alone.
int discharge_batch(sg_context* ctx, const std::vector<int>& slots) {
  std::vector<Run*> elec;
  for (int s : slots) if (ctx->runs[s].lgt) elec.push_back(&ctx->runs[s]);
  if (elec.empty()) return SG_OK;
  std::vector<unsigned long long> failed(elec.size(), 0);
  for (size_t k = 0; k < elec.size(); k++)
    CK(cudaMemcpyAsync(&failed[k], elec[k]->desc.cnt + C_FAILED, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  std::vector<LgtJob> jobs;
  for (size_t k = 0; k < elec.size(); k++) {
    Run& r = *elec[k];
    r.time += r.dt;
    if (failed[k]) continue;
    LgtJob J;
    J.g = &r.grid; J.R = r.desc; J.H = r.lgt.get(); J.time = r.time; J.dt = r.dt; J.limit = flash_limit(r.dt);
    jobs.push_back(J);
  }
  if (jobs.empty()) return SG_OK;
  std::string err;
  const int st = lightning_discharge_many(jobs.data(), (int)jobs.size(), &err);
  if (st != SG_OK) return fail(ctx, st, "lightning: " + err);
  return SG_OK;
}

int batch_step(sg_context* ctx, const sg_run* runs, int n, int nsteps, bool wait) {
  if (nsteps < 0) return fail(ctx, SG_ERR_INVALID, "negative step count");
  std::vector<int> slots;
  int st = slots_of(ctx, runs, n, slots);
  if (st) return st;
  Plan* P = get_plan(ctx, slots, &st);
  if (!P) return st;
  if ((st = ensure_graph(ctx, *P))) return st;
  if (P->elec) {
    // electrified runs: after each step their lightning (host-stepped flash stages, src/core/model.ts:1130-1133)
    for (int s = 0; s < nsteps; s++) {
      CK(cudaGraphLaunch(P->exec, ctx->stream));
      if ((st = discharge_batch(ctx, P->slots)) != SG_OK) return st;
    }
  } else {
    for (int s = 0; s < nsteps; s++) CK(cudaGraphLaunch(P->exec, ctx->stream));
  }
  if (wait) CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaGetLastError());
  return SG_OK;
}

// A plan over one run for the boundary kernels (theta conversion).
Launch node_launch(sg_context* ctx, const Run& r) { return Launch{ctx->d_runs, r.nodeItems, r.nNode, ctx->sms * 8, ctx->stream}; }
Plan* single_plan(sg_context* ctx, int slot, int* st) { return get_plan(ctx, std::vector<int>{slot}, st); }

}  // namespace

// waterReservoirs (src/core/water.ts:27-46) of initial fields on the host, FP64 in the reference's order: per level the
// vapour above the environment's profile, the condensate (cloud water, ice) and the precipitation aloft, each weighted
// by the level's air mass; nothing on the ground yet.
static double water_reservoirs(const sg_grid* g, const sg_base_state* b, const float* const* f) {
  const size_t layer = (size_t)g->nx * g->ny;
  double vapour = 0, condensate = 0, aloft = 0;
  for (int z = 0; z < g->nz; z++) {
    const double mass = b->rho[z] * g->dx * g->dy * g->hz[z], q0 = b->q[z];
    double v = 0, c = 0, a = 0;
    for (size_t i = z * layer, e = i + layer; i < e; i++) {
      v += f[Q][i] - q0;
      c += (double)f[CLOUD][i] + f[ICE][i];
      a += (double)f[RAIN][i] + f[SNOW][i] + f[GRAUPEL][i] + f[HAIL][i];
    }
    vapour += v * mass; condensate += c * mass; aloft += a * mass;
  }
  return vapour + condensate + aloft;
}

// ==================================================================== C ABI
extern "C" {

int sg_context_create(int device, uint64_t hbm_budget_bytes, sg_context** out) {
  if (!out) return SG_ERR_INVALID;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return SG_ERR_DEVICE;
  if (device < 0 || device >= count) return SG_ERR_INVALID;
  auto* ctx = new sg_context;
  ctx->device = device;
  cudaError_t e = cudaSuccess;
  if ((e = cudaSetDevice(device)) != cudaSuccess) { delete ctx; return SG_ERR_DEVICE; }
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, device);
  ctx->sms = prop.multiProcessorCount; ctx->maxSmem = (int)prop.sharedMemPerBlockOptin;
  size_t freeB = 0, totalB = 0; cudaMemGetInfo(&freeB, &totalB);
  ctx->budget = hbm_budget_bytes ? hbm_budget_bytes : (uint64_t)(freeB * 0.9);
  if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaMalloc(&ctx->d_runs, MAX_SLOTS * sizeof(RunDesc))) != cudaSuccess ||
      (e = cudaMalloc(&ctx->d_scalar, 64 * sizeof(double))) != cudaSuccess ||
      (e = set_smem_limits(ctx->maxSmem)) != cudaSuccess || (e = upload_tables()) != cudaSuccess) {
    delete ctx; return SG_ERR_DEVICE;
  }
  for (int k = 0; k < 2; k++)
    if ((e = cudaStreamCreateWithFlags(&ctx->side[k], cudaStreamNonBlocking)) != cudaSuccess) { delete ctx; return SG_ERR_DEVICE; }
  for (int k = 0; k < 8; k++)
    if ((e = cudaEventCreateWithFlags(&ctx->dep[k], cudaEventDisableTiming)) != cudaSuccess) { delete ctx; return SG_ERR_DEVICE; }
  // the no-allocation divergence check's module (its code and static scratch) loads now, while the context is made
  if (static_prepare(device) != 0) { cudaGetLastError(); delete ctx; return SG_ERR_DEVICE; }
  if (const char* a = getenv("SG_AUTOTUNE")) ctx->autotune = atoi(a) != 0;
  if (const char* a = getenv("SG_SPECTRAL_ROWS")) ctx->rowsOnly = atoi(a) != 0;
  if (const char* a = getenv("SG_TRANSPORT_BULK")) ctx->bulk = atoi(a) != 0;
  if (const char* a = getenv("SG_AUTOTUNE_LOG")) ctx->tuneLog = atoi(a) != 0;
  if (const char* a = getenv("SG_TRANSPORT_EDGE_WARPS")) ctx->edgeWarps = atoi(a) != 0;
  *out = ctx;
  return SG_OK;
}

int sg_context_destroy(sg_context* ctx) {
  if (!ctx) return SG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->plans.clear();
  for (auto& r : ctx->runs) if (r.live) cudaFree(r.mem);
  for (auto& p : ctx->pool) cudaFree(p.second);
  cudaFree(ctx->d_runs); cudaFree(ctx->d_scalar);
  cudaStreamDestroy(ctx->stream);
  for (int k = 0; k < 2; k++) cudaStreamDestroy(ctx->side[k]);
  for (int k = 0; k < 8; k++) cudaEventDestroy(ctx->dep[k]);
  for (int k = 0; k < sg_context::IO_GROUPS; k++) if (ctx->io[k]) cudaStreamDestroy(ctx->io[k]);
  for (int k = 0; k <= sg_context::IO_GROUPS; k++) if (ctx->ioEv[k]) cudaEventDestroy(ctx->ioEv[k]);
  for (auto& p : ctx->packs) cudaFree(p.second.first);
  if (ctx->staging) cudaFree(ctx->staging);
  delete ctx;
  return SG_OK;
}

const char* sg_last_error(sg_context* ctx) { return ctx ? ctx->error.c_str() : "no context"; }

}  // extern "C"
int sg_context_device(sg_context* ctx) { return ctx->device; }
cudaStream_t sg_context_stream(sg_context* ctx) { return ctx->stream; }
int sg_context_fail(sg_context* ctx, int code, const char* message) { return fail(ctx, code, message); }
extern "C" {

}  // extern "C"
// The extra-field flags of a run: electrified() (src/core/model.ts:1316), rain2m() (:905), ice2m() (:914).
static int run_flags(const sg_switches* sw) {
  const bool two = sw->rain_moments == 2;
  return (sw->lightning && sw->ice ? RF_ELEC : 0) | (two ? RF_RAIN2M : 0) | (two && sw->ice && sw->ice_moments == 2 ? RF_ICE2M : 0);
}
extern "C" {

uint64_t sg_run_bytes(const sg_grid* grid) { return grid ? layout(grid->nx, grid->ny, grid->nz).total : 0; }
uint64_t sg_run_bytes_for(const sg_grid* grid, const sg_switches* sw) {
  if (!grid || !sw) return 0;
  return layout(grid->nx, grid->ny, grid->nz, run_flags(sw)).total;
}

int sg_run_create(sg_context* ctx, const sg_grid* g, const sg_base_state* b, const sg_switches* sw, const float* const* init, sg_run* out) {
  if (!ctx || !out) return SG_ERR_INVALID;
  int st = validate(ctx, g, b, sw);
  if (st) return st;
  cudaSetDevice(ctx->device);
  const int xflags = run_flags(sw);
  const bool elec = xflags & RF_ELEC, two = xflags & RF_RAIN2M;
  Layout Lo = layout(g->nx, g->ny, g->nz, xflags);
  // Admission by the HBM budget (pooled allocations of a retired run count as free).
  char* mem = nullptr;
  auto pit = ctx->pool.find(Lo.total);
  if (pit != ctx->pool.end()) { mem = pit->second; ctx->pool.erase(pit); ctx->pooled -= Lo.total; }
  else {
    while (ctx->used + ctx->pooled + Lo.total > ctx->budget && !ctx->pool.empty()) {
      auto last = std::prev(ctx->pool.end()); cudaFree(last->second); ctx->pooled -= last->first; ctx->pool.erase(last);
    }
    if (ctx->used + Lo.total > ctx->budget) return fail(ctx, SG_ERR_BUDGET, "run needs " + std::to_string(Lo.total) + " bytes beyond the HBM budget");
    cudaError_t e = cudaMalloc(&mem, Lo.total);
    if (e != cudaSuccess) { cudaGetLastError(); return fail(ctx, SG_ERR_BUDGET, std::string("cudaMalloc: ") + cudaGetErrorString(e)); }
  }
  ctx->used += Lo.total;
  int slot;
  if (!ctx->freeSlots.empty()) { slot = ctx->freeSlots.back(); ctx->freeSlots.pop_back(); }
  else {
    slot = (int)ctx->runs.size();
    if (slot >= MAX_SLOTS) { cudaFree(mem); ctx->used -= Lo.total; return fail(ctx, SG_ERR_BUDGET, "too many runs"); }
    ctx->runs.emplace_back();
  }
  Run& r = ctx->runs[slot];
  r.live = true; r.slot = slot; r.nx = g->nx; r.ny = g->ny; r.nz = g->nz; r.bytes = Lo.total; r.mem = mem;
  HostTables T; RunDesc& d = r.desc; d = RunDesc{};
  build_tables(g, b, sw, T, d);
  d.slot = slot;
  d.nf = elec || two ? NFE : NF;
  d.flags |= xflags;
  d.breakup = sw->rain_breakup;
  d.fld = (float*)(mem + Lo.fld); d.faces = (float*)(mem + Lo.faces); d.kmkh = (float*)(mem + Lo.kmkh); d.phi = (float*)(mem + Lo.phi);
  d.pres = (float*)(mem + Lo.pres); d.pres2 = (float*)(mem + Lo.pres2); d.spec = (float2*)(mem + Lo.spec); d.cols = (float*)(mem + Lo.cols);
  d.lv = (const float*)(mem + Lo.lv); d.lv64 = (const double*)(mem + Lo.lv64); d.tri_face = (const TriAB*)(mem + Lo.triF);
  d.tri_pres = (const TriAB*)(mem + Lo.triP); d.ab = (const double2*)(mem + Lo.ab); d.twx = (const float2*)(mem + Lo.twx);
  d.twy = (const float2*)(mem + Lo.twy); d.scr = (float*)(mem + Lo.scr); d.part = (double*)(mem + Lo.part); d.acc = (double*)(mem + Lo.acc);
  d.cnt = (unsigned long long*)(mem + Lo.cnt);
  d.diag = (float*)(mem + Lo.diag); d.rot = (double*)(mem + Lo.rot);
  r.lgt.reset();
  if (elec || two) { d.vfall = (float*)(mem + Lo.vfall); d.ez = (float*)(mem + Lo.ez); d.cpart = (double*)(mem + Lo.cpart); }
  if (elec) {
    r.lgt = std::make_unique<LgtHost>();
    lightning_bind(mem + Lo.lgt, g->nx, g->ny, g->nz, r.lgt->dev);
    r.lgt->seed = (uint32_t)sw->lightning_seed; r.lgt->corona = sw->corona != 0;
    r.zs.assign(g->zs, g->zs + g->nz); r.dzs.assign(g->dzs, g->dzs + g->nz - 1); r.hz.assign(g->hz, g->hz + g->nz);
    r.grid = *g; r.grid.zs = r.zs.data(); r.grid.dzs = r.dzs.data(); r.grid.hz = r.hz.data();
  }
  r.time = 0; r.dt = sw->dt;
  auto H2D = [&](size_t off, const void* src, size_t bytes) { return cudaMemcpyAsync(mem + off, src, bytes, cudaMemcpyHostToDevice, ctx->stream); };
  CK(cudaMemsetAsync(mem, 0, Lo.total, ctx->stream));
  CK(H2D(Lo.lv, T.lv.data(), T.lv.size() * 4)); CK(H2D(Lo.lv64, T.lv64.data(), T.lv64.size() * 8));
  CK(H2D(Lo.triF, T.triF.data(), T.triF.size() * 16)); CK(H2D(Lo.triF + T.triF.size() * 16, T.triFc.data(), T.triFc.size() * 8));
  CK(H2D(Lo.triP, T.triP.data(), T.triP.size() * 16)); CK(H2D(Lo.triP + T.triP.size() * 16, T.triPc.data(), T.triPc.size() * 8));
  CK(H2D(Lo.ab, T.ab.data(), T.ab.size() * 16)); CK(H2D(Lo.twx, T.twx.data(), T.twx.size() * 8)); CK(H2D(Lo.twy, T.twy.data(), T.twy.size() * 8));
  CK(cudaMemcpyAsync(ctx->d_runs + slot, &d, sizeof(RunDesc), cudaMemcpyHostToDevice, ctx->stream));
  if (elec) {
    const int e = lightning_init(ctx->stream, &r.grid, b->rho, *r.lgt);
    if (e) return fail(ctx, SG_ERR_DEVICE, std::string("lightning tables: ") + cudaGetErrorString((cudaError_t)e));
    if (lightning_host_buffers(*r.lgt) != SG_OK) return fail(ctx, SG_ERR_DEVICE, "lightning stream and pinned buffers");
  }
  {
    const size_t n = (size_t)g->nx * g->ny * g->nz;
    r.nNode = (int)((n + CHUNK - 1) / CHUNK);
    std::vector<int4> items(r.nNode);
    for (int c = 0; c < r.nNode; c++) items[c] = make_int4(slot, c, 0, 0);
    r.nodeItems = (int4*)(mem + Lo.items);
    CK(H2D(Lo.items, items.data(), items.size() * sizeof(int4)));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  *out = slot;
  if (init) {
    int s2 = sg_run_write_fields(ctx, slot, SG_ALL_FIELDS, init);
    if (s2) { sg_run_retire(ctx, slot); return s2; }
    r.waterStart = water_reservoirs(g, b, init);
  }
  return SG_OK;
}

// Whether a field mask names only fields the run carries.
static bool mask_fits(const Run& r, uint32_t mask) {
  const int f = r.desc.flags;
  return !(mask >> r.desc.nf) && !((mask & SG_CHARGE_FIELDS) && !(f & RF_ELEC)) && !((mask & (1u << SG_RAIN_NUMBER)) && !(f & RF_RAIN2M)) &&
         !((mask & SG_ICE2M_FIELDS) && !(f & RF_ICE2M));
}

int sg_run_write_fields(sg_context* ctx, sg_run run, uint32_t mask, const float* const* host) {
  if (!ctx || !host) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  cudaSetDevice(ctx->device);
  size_t n = (size_t)r->nx * r->ny * r->nz;
  const int nf = r->desc.nf;
  if (!mask_fits(*r, mask))
    return fail(ctx, SG_ERR_INVALID, "field mask beyond the run's fields (the charges need an electrified run, the drop number two-moment rain, "
                                     "the graupel and hail numbers and volumes two-moment ice)");
  for (int f = 0; f < nf; f++) {
    if (!(mask & (1u << f))) continue;
    if (!host[f]) return fail(ctx, SG_ERR_INVALID, "null field pointer");
    // theta arrives full; it is staged in set B and converted to its departure in set A.
    float* dst = field(r->desc, f == THETA ? 1 : 0, f);
    CK(cudaMemcpyAsync(dst, host[f], n * 4, cudaMemcpyHostToDevice, ctx->stream));
  }
  if (mask & (1u << THETA)) launch_theta_in(node_launch(ctx, *r), field(r->desc, 1, THETA));
  CK(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

int sg_run_read_fields(sg_context* ctx, sg_run run, uint32_t mask, float* const* host) {
  if (!ctx || !host) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  cudaSetDevice(ctx->device);
  size_t n = (size_t)r->nx * r->ny * r->nz;
  const int nf = r->desc.nf;
  if (!mask_fits(*r, mask))
    return fail(ctx, SG_ERR_INVALID, "field mask beyond the run's fields (the charges need an electrified run, the drop number two-moment rain, "
                                     "the graupel and hail numbers and volumes two-moment ice)");
  if (mask & (1u << THETA)) launch_theta_out(node_launch(ctx, *r), field(r->desc, 1, THETA));
  for (int f = 0; f < nf; f++) {
    if (!(mask & (1u << f))) continue;
    if (!host[f]) return fail(ctx, SG_ERR_INVALID, "null field pointer");
    const float* src = field(r->desc, f == THETA ? 1 : 0, f);
    CK(cudaMemcpyAsync(host[f], src, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

// Fields of many runs in one call: all copies on the library's stream, one theta conversion launch for the batch,
// one synchronisation at the end. host[k * 13 + f] is run k's field f (by the mask).
int batch_fields(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, float* const* host, bool write) {
  if (!ctx || !host) return SG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  std::vector<int> slots;
  int st = slots_of(ctx, runs, n, slots);
  if (st != SG_OK) return st;
  Plan* P = nullptr;
  if (mask & (1u << THETA)) { P = get_plan(ctx, slots, &st); if (!P) return st; }
  if (!write && P) launch_theta_out(lx(ctx, *P, FAM_NODE), nullptr);
  for (int k = 0; k < n; k++) {
    Run* r = find(ctx, runs[k]);
    const size_t nn = (size_t)r->nx * r->ny * r->nz;
    for (int f = 0; f < NF; f++) {
      if (!(mask & (1u << f))) continue;
      float* h = host[(size_t)k * NF + f];
      if (!h) return fail(ctx, SG_ERR_INVALID, "null field pointer");
      float* dev = field(r->desc, f == THETA ? 1 : 0, f);  // theta staged in set B
      if (write) CK(cudaMemcpyAsync(dev, h, nn * 4, cudaMemcpyHostToDevice, ctx->stream));
      else CK(cudaMemcpyAsync(h, dev, nn * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
  }
  if (write && P) launch_theta_in(lx(ctx, *P, FAM_NODE), nullptr);
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaGetLastError());
  return SG_OK;
}

// The placing items of a packed batch (run after run in the caller's order, the mask's fields in field order, n
// nodes each; item w = the chunk's offset in the packed buffer) and the buffer's length in floats, cached per
// (runs, mask).
static int pack_items(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, std::pair<int4*, int>& out, size_t& total) {
  std::vector<int> key;
  int st = slots_of(ctx, runs, n, key);
  if (st != SG_OK) return st;
  key.push_back((int)mask);
  total = 0;
  for (int k = 0; k < n; k++) {
    const Run* r = find(ctx, runs[k]);
    for (int f = 0; f < NF; f++) if (mask & (1u << f)) total += (size_t)r->nx * r->ny * r->nz;
  }
  if (total >= (1ull << 31)) return fail(ctx, SG_ERR_INVALID, "packed batch too large");
  auto it = ctx->packs.find(key);
  if (it == ctx->packs.end()) {
    std::vector<int4> items;
    size_t off = 0;
    for (int k = 0; k < n; k++) {
      const Run* r = find(ctx, runs[k]);
      const int nn = r->nx * r->ny * r->nz;
      for (int f = 0; f < NF; f++) {
        if (!(mask & (1u << f))) continue;
        for (int c = 0; c * CHUNK < nn; c++) items.push_back(make_int4(runs[k], f, c, (int)(off + (size_t)c * CHUNK)));
        off += nn;
      }
    }
    int4* d = nullptr;
    CK(cudaMalloc(&d, items.size() * sizeof(int4)));
    CK(cudaMemcpy(d, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice));
    if (ctx->packs.size() > 64) { for (auto& p : ctx->packs) cudaFree(p.second.first); ctx->packs.clear(); }
    it = ctx->packs.emplace(key, std::make_pair(d, (int)items.size())).first;
  }
  out = it->second;
  return SG_OK;
}

// The context's staging buffer, grown to at least `floats` values.
static int ensure_staging(sg_context* ctx, size_t floats) {
  if (ctx->stagingBytes < floats * 4) {
    if (ctx->staging) cudaFree(ctx->staging);
    ctx->staging = nullptr; ctx->stagingBytes = 0;
    CK(cudaMalloc(&ctx->staging, floats * 4));
    ctx->stagingBytes = floats * 4;
  }
  return SG_OK;
}

// Fields of many runs packed run after run (the mask's fields in field order, n nodes each) through one staging
// buffer: one host copy, one kernel, one synchronisation. The packing follows the caller's order of the runs.
static int batch_packed(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, float* host, bool write) {
  if (!ctx || !host) return SG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  std::pair<int4*, int> items;
  size_t total = 0;
  int st = pack_items(ctx, runs, n, mask, items, total);
  if (st != SG_OK) return st;
  if ((st = ensure_staging(ctx, total)) != SG_OK) return st;
  Launch L{ctx->d_runs, items.first, items.second, ctx->sms * 8, ctx->stream};
  if (write) {
    CK(cudaMemcpyAsync(ctx->staging, host, total * 4, cudaMemcpyHostToDevice, ctx->stream));
    launch_pack(L, ctx->staging, 1);
  } else {
    launch_pack(L, ctx->staging, 0);
    CK(cudaMemcpyAsync(host, ctx->staging, total * 4, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaGetLastError());
  return SG_OK;
}

// Steps with the state moved through host memory around them, as the reference's GPU engine moves it every step
// (src/gpu/dynamics.ts:446-450, :488-497): the mask's fields of every run are written from `host` (the packed layout),
// the runs advance `nsteps`, and the fields are read back into `host`. The runs are cut into `groups` consecutive
// groups, each with a stream, a part of the staging buffer and a graph of its own, so one group's copies overlap the
// other groups' steps. Each group's runs step exactly as in any other batch (a run's results do not depend on the
// runs beside it).
// each_step: nsteps round trips (every step written from host, stepped once, read back into host; a group's next
// write reads what its last read wrote), else one round trip around nsteps steps.
static int batch_step_io(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, float* host, int nsteps, int groups,
                         bool each_step = false) {
  if (!ctx || !host) return SG_ERR_INVALID;
  if (nsteps < 0) return fail(ctx, SG_ERR_INVALID, "negative step count");
  cudaSetDevice(ctx->device);
  std::vector<int> all;
  int st = slots_of(ctx, runs, n, all);
  if (st != SG_OK) return st;
  groups = std::max(1, std::min(std::min(groups, n), sg_context::IO_GROUPS));
  // the plan and item-list caches drop everything when full: make room first, so no group's plan or items are dropped
  // while the others are set up
  if (ctx->plans.size() + groups > 256) ctx->plans.clear();
  if (ctx->packs.size() + groups > 64) { for (auto& p : ctx->packs) cudaFree(p.second.first); ctx->packs.clear(); }
  // set-up before any group's work is queued: plans, graphs (captured on the context's stream), item lists, staging
  struct Group { int first = 0, count = 0; Plan* P = nullptr; std::pair<int4*, int> items; size_t off = 0, total = 0; };
  std::vector<Group> gs(groups);
  size_t total = 0;
  for (int g = 0; g < groups; g++) {
    Group& x = gs[g];
    x.first = (int)((int64_t)n * g / groups);
    x.count = (int)((int64_t)n * (g + 1) / groups) - x.first;
    const std::vector<int> slots(all.begin() + x.first, all.begin() + x.first + x.count);
    if (!(x.P = get_plan(ctx, slots, &st))) return st;
    if (x.P->elec) return fail(ctx, SG_ERR_UNSUPPORTED, "host round trips of electrified runs: step them with sg_batch_step (the lightning is host-stepped)");
    if ((st = ensure_graph(ctx, *x.P)) != SG_OK) return st;
    if ((st = pack_items(ctx, runs + x.first, x.count, mask, x.items, x.total)) != SG_OK) return st;
    x.off = total;
    total += x.total;
  }
  if ((st = ensure_staging(ctx, total)) != SG_OK) return st;
  for (int g = 0; g <= groups; g++) {
    if (g < groups && !ctx->io[g]) CK(cudaStreamCreateWithFlags(&ctx->io[g], cudaStreamNonBlocking));
    const int e = g < groups ? g : sg_context::IO_GROUPS;
    if (!ctx->ioEv[e]) CK(cudaEventCreateWithFlags(&ctx->ioEv[e], cudaEventDisableTiming));
  }
  // the groups start after the work already on the context's stream; the stream's later work waits for them all
  CK(cudaEventRecord(ctx->ioEv[sg_context::IO_GROUPS], ctx->stream));
  for (int g = 0; g < groups; g++) {
    const Group& x = gs[g];
    cudaStream_t s = ctx->io[g];
    float* dev = ctx->staging + x.off;
    const Launch L{ctx->d_runs, x.items.first, x.items.second, ctx->sms * 8, s};
    CK(cudaStreamWaitEvent(s, ctx->ioEv[sg_context::IO_GROUPS], 0));
    const int trips = each_step ? nsteps : 1, inner = each_step ? 1 : nsteps;
    for (int r = 0; r < trips; r++) {
      CK(cudaMemcpyAsync(dev, host + x.off, x.total * 4, cudaMemcpyHostToDevice, s));
      launch_pack(L, dev, 1);
      for (int k = 0; k < inner; k++) CK(cudaGraphLaunch(x.P->exec, s));
      launch_pack(L, dev, 0);
      CK(cudaMemcpyAsync(host + x.off, dev, x.total * 4, cudaMemcpyDeviceToHost, s));
    }
    CK(cudaEventRecord(ctx->ioEv[g], s));
    CK(cudaStreamWaitEvent(ctx->stream, ctx->ioEv[g], 0));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaGetLastError());
  return SG_OK;
}

int sg_run_read_columns(sg_context* ctx, sg_run run, float* precipitation, float* hail_ground, float* hail_size) {
  if (!ctx) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  size_t layer = (size_t)r->nx * r->ny;
  float* dst[3] = {precipitation, hail_ground, hail_size};
  for (int k = 0; k < 3; k++) if (dst[k]) CK(cudaMemcpyAsync(dst[k], r->desc.cols + k * layer, layer * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

int sg_run_write_columns(sg_context* ctx, sg_run run, const float* precipitation, const float* hail_ground, const float* hail_size) {
  if (!ctx) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  size_t layer = (size_t)r->nx * r->ny;
  const float* src[3] = {precipitation, hail_ground, hail_size};
  for (int k = 0; k < 3; k++) if (src[k]) CK(cudaMemcpyAsync(r->desc.cols + k * layer, src[k], layer * 4, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

int sg_run_shape(sg_context* ctx, sg_run run, int32_t* nx, int32_t* ny, int32_t* nz) {
  if (!ctx) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  if (nx) *nx = r->nx;
  if (ny) *ny = r->ny;
  if (nz) *nz = r->nz;
  return SG_OK;
}

// saveState (src/core/state.ts:43-53): the carried fields gathered by the packed transfer (one kernel, one copy),
// placed in STATE_FIELDS order on the host, the fields the step does not carry written as zeros.
int sg_run_save_state(sg_context* ctx, sg_run run, const char* config_json, double time, double persisted, uint8_t* out,
                      size_t cap, size_t* size) {
  if (!ctx || !size) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  if (!state::json_valid(config_json)) return fail(ctx, SG_ERR_INVALID, "config_json is not one JSON value");
  sg_run_counters c;
  int st = sg_run_status(ctx, run, &c);
  if (st != SG_OK && st != SG_ERR_NONFINITE) return st;
  const double water[5] = {c.water_condensed, c.water_evaporated, c.water_rain_evaporated, c.water_surface, r->waterStart};
  sg_charge_state cs;
  if ((st = sg_run_charge(ctx, run, &cs)) != SG_OK) return st;
  const double charge9[9] = {cs.ground, (double)cs.flashes_ic, (double)cs.flashes_cg, cs.separated, cs.ic, cs.cg_negative, cs.cg_positive,
                             cs.precipitation, cs.conduction};
  const std::string json = state::header_json(config_json, time, persisted, r->nx, r->ny, r->nz, water, r->lgt ? charge9 : nullptr);
  const size_t need = state::image_bytes(json.size(), state::VERSION, r->nx, r->ny, r->nz);
  *size = need;
  if (!out) return SG_OK;
  if (cap < need) return fail(ctx, SG_ERR_INVALID, "the buffer holds " + std::to_string(cap) + " bytes, the image needs " + std::to_string(need));
  const size_t n = (size_t)r->nx * r->ny * r->nz, layer = (size_t)r->nx * r->ny, off = state::data_offset(json.size());
  std::vector<float> fields((size_t)SG_NFIELDS * n), cols(3 * layer);
  if ((st = sg_batch_read_packed(ctx, &run, 1, SG_ALL_FIELDS, fields.data())) != SG_OK) return st;
  // the extra fields the run carries (an electrified run's charges, a two-moment run's drop number, graupel and hail
  // numbers and volumes)
  constexpr int NX = SG_NFIELDS_EXTRA - SG_CHARGE_ICE;
  std::vector<float> extra(NX * n, 0.f);
  const uint32_t xmask = (r->lgt ? SG_CHARGE_FIELDS : 0u) | ((r->desc.flags & RF_RAIN2M) ? 1u << SG_RAIN_NUMBER : 0u) |
                         ((r->desc.flags & RF_ICE2M) ? SG_ICE2M_FIELDS : 0u);
  if (xmask) {
    float* ptr[SG_NFIELDS_EXTRA] = {};
    for (int k = 0; k < NX; k++) ptr[SG_CHARGE_ICE + k] = extra.data() + (size_t)k * n;
    if ((st = sg_run_read_fields(ctx, run, xmask, ptr)) != SG_OK) return st;
  }
  if ((st = sg_run_read_columns(ctx, run, cols.data(), cols.data() + layer, cols.data() + 2 * layer)) != SG_OK) return st;
  std::memset(out, 0, off);
  std::memcpy(out, "MLAB", 4);
  const uint32_t jl = (uint32_t)json.size();
  const uint8_t len4[4] = {(uint8_t)jl, (uint8_t)(jl >> 8), (uint8_t)(jl >> 16), (uint8_t)(jl >> 24)};
  std::memcpy(out + 4, len4, 4);
  std::memcpy(out + 8, json.data(), json.size());
  for (int k = 0; k < state::NSTATE; k++) {
    uint8_t* dst = out + off + (size_t)k * n * 4;
    const int f = state::carried_of(k);
    if (f >= SG_CHARGE_ICE) std::memcpy(dst, extra.data() + (size_t)(f - SG_CHARGE_ICE) * n, n * 4);
    else if (f >= 0 && f < SG_NFIELDS) std::memcpy(dst, fields.data() + (size_t)f * n, n * 4);
    else std::memset(dst, 0, n * 4);
  }
  std::memcpy(out + off + (size_t)state::NSTATE * n * 4, cols.data(), 3 * layer * 4);
  return SG_OK;
}

// readState + applyState (src/core/state.ts:55-83) into a run of the same grid: the file's fields (those an older
// version lacks as zeros, state.ts:70), the columns; the packed transfer scatters them (one copy, one kernel).
int sg_run_load_state(sg_context* ctx, sg_run run, const uint8_t* image, size_t len, sg_state_info* info) {
  if (!ctx) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  state::Info h;
  const std::string msg = state::parse(image, len, h);
  if (!msg.empty()) return fail(ctx, SG_ERR_INVALID, msg);
  if (h.nx != r->nx || h.ny != r->ny || h.nz != r->nz)
    return fail(ctx, SG_ERR_INVALID, "the file's grid is " + std::to_string(h.nx) + "x" + std::to_string(h.ny) + "x" + std::to_string(h.nz) +
                                         ", the run's " + std::to_string(r->nx) + "x" + std::to_string(r->ny) + "x" + std::to_string(r->nz));
  const size_t n = (size_t)r->nx * r->ny * r->nz, layer = (size_t)r->nx * r->ny;
  std::vector<float> fields((size_t)SG_NFIELDS * n, 0.f), cols(3 * layer), extra((size_t)(SG_NFIELDS_EXTRA - SG_CHARGE_ICE) * n, 0.f);
  for (int k = 0; k < h.nfields; k++) {
    const int f = state::carried_of(k);
    if (f >= 0 && f < SG_NFIELDS) std::memcpy(fields.data() + (size_t)f * n, image + h.data_offset + (size_t)k * n * 4, n * 4);
    else if (f >= SG_CHARGE_ICE) std::memcpy(extra.data() + (size_t)(f - SG_CHARGE_ICE) * n, image + h.data_offset + (size_t)k * n * 4, n * 4);
  }
  std::memcpy(cols.data(), image + h.data_offset + (size_t)h.nfields * n * 4, 3 * layer * 4);
  int st = sg_batch_write_packed(ctx, &run, 1, SG_ALL_FIELDS, fields.data());
  if (st != SG_OK) return st;
  if ((st = sg_run_write_columns(ctx, run, cols.data(), cols.data() + layer, cols.data() + 2 * layer)) != SG_OK) return st;
  if (r->desc.flags & RF_RAIN2M) {
    // a two-moment run: the file's drop number (none before version 4; the first step rebuilds it from the rain, as
    // the reference's boundedNumber does for rain without a number, state.ts:13)
    const float* ptr[SG_NFIELDS_EXTRA] = {};
    ptr[SG_RAIN_NUMBER] = extra.data() + (size_t)(SG_RAIN_NUMBER - SG_CHARGE_ICE) * n;
    if ((st = sg_run_write_fields(ctx, run, 1u << SG_RAIN_NUMBER, ptr)) != SG_OK) return st;
  }
  if (r->desc.flags & RF_ICE2M) {
    // two-moment graupel and hail: the file's numbers and volumes (none before version 5: the first step's bounding
    // rebuilds them from the mass, as boundedIceNumber and the class's density without a volume do, state.ts:14)
    const float* ptr[SG_NFIELDS_EXTRA] = {};
    for (int k = SG_GRAUPEL_NUMBER; k <= SG_HAIL_VOLUME; k++) ptr[k] = extra.data() + (size_t)(k - SG_CHARGE_ICE) * n;
    if ((st = sg_run_write_fields(ctx, run, SG_ICE2M_FIELDS, ptr)) != SG_OK) return st;
  }
  if (r->lgt) {
    // an electrified run: the file's charge (none in a version-1 file), its ground charge, flash counts and charge budget
    // (state.ts:78-81); the flashes after the file's time forgotten (:82), the vertical field as a new model's (zero)
    const float* ptr[SG_NFIELDS_EXTRA] = {};
    for (int k = 0; k < 4; k++) ptr[SG_CHARGE_ICE + k] = extra.data() + (size_t)k * n;
    if ((st = sg_run_write_fields(ctx, run, SG_CHARGE_FIELDS, ptr)) != SG_OK) return st;
    const double acc[9] = {h.charge[0], h.charge[3], h.charge[4], h.charge[5], h.charge[6], h.charge[7], h.charge[8], h.charge[1], h.charge[2]};
    static_assert(A_CHG_SEPARATED == A_CHG_GROUND + 1 && A_FLASH_CG == A_CHG_GROUND + 8, "the charge budget's slots in order");
    CK(cudaMemcpyAsync(r->desc.acc + A_CHG_GROUND, acc, sizeof(acc), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(r->desc.ez, 0, n * 4, ctx->stream));
    r->lgt->last.clear();
  }
  // the water budget goes on from the file's flows and start (state.ts:77)
  CK(cudaMemcpyAsync(r->desc.acc + A_WATER, h.water, 3 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  r->waterStart = h.water[4];
  // the model time and the time the rotation has held; the rotation recomputed from the fields (state.ts:74-76)
  const double tp[2] = {h.time, h.persisted};
  r->time = h.time;
  CK(cudaMemcpyAsync(r->desc.rot + R_TIME, &tp[0], sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(r->desc.rot + R_PERSISTED, &tp[1], sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if ((r->desc.flags & RF_ROTATION) && (st = sg_run_refresh_rotation(ctx, run)) != SG_OK) return st;
  if (info) {
    info->version = h.version; info->nx = h.nx; info->ny = h.ny; info->nz = h.nz; info->nfields = h.nfields;
    info->time = h.time; info->persisted = h.persisted; info->data_offset = (uint64_t)h.data_offset;
  }
  return SG_OK;
}

int sg_run_rotation(sg_context* ctx, sg_run run, sg_rotation* out, float* uh_column) {
  if (!ctx || !out) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  if (!(r->desc.flags & RF_ROTATION)) return fail(ctx, SG_ERR_INVALID, "the run does not track its rotation (switches.rotation = 0)");
  double rot[R_COUNT];
  CK(cudaMemcpyAsync(rot, r->desc.rot, sizeof rot, cudaMemcpyDeviceToHost, ctx->stream));
  if (uh_column) CK(cudaMemcpyAsync(uh_column, r->desc.diag + (size_t)DG_UH * r->nx * r->ny, (size_t)r->nx * r->ny * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  out->uh = rot[R_UH]; out->x = rot[R_X]; out->y = rot[R_Y]; out->anticyclonic = rot[R_ANTI]; out->persisted = rot[R_PERSISTED];
  out->uh01 = rot[R_UH01]; out->uh03 = rot[R_UH03]; out->low = rot[R_LOW]; out->core_zeta = rot[R_CZETA]; out->core_uh = rot[R_CUH];
  out->core_anti = rot[R_CANTI]; out->time = rot[R_TIME];
  return SG_OK;
}

int sg_run_refresh_rotation(sg_context* ctx, sg_run run) {
  if (!ctx) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  if (!(r->desc.flags & RF_ROTATION)) return fail(ctx, SG_ERR_INVALID, "the run does not track its rotation (switches.rotation = 0)");
  int st;
  Plan* P = single_plan(ctx, run, &st);
  if (!P) return st;
  launch_rotation_columns(lx(ctx, *P, FAM_COLS), 1);
  launch_rotation_summary(lx(ctx, *P, FAM_RUNS), 1);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

int sg_run_read_swaths(sg_context* ctx, sg_run run, float* gust_max, float* uh_max) {
  if (!ctx) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  const size_t layer = (size_t)r->nx * r->ny;
  if (gust_max) CK(cudaMemcpyAsync(gust_max, r->desc.diag + DG_GUST_MAX * layer, layer * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (uh_max) CK(cudaMemcpyAsync(uh_max, r->desc.diag + DG_UH_MAX * layer, layer * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

int sg_run_reset_swaths(sg_context* ctx, sg_run run) {
  if (!ctx) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  const size_t layer = (size_t)r->nx * r->ny;
  CK(cudaMemsetAsync(r->desc.diag + DG_GUST_MAX * layer, 0, 2 * layer * 4, ctx->stream));  // gustMax, uhMax
  CK(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

// diagnostics() (src/core/model.ts:1672-1696): the device's maxima and ground columns, then countCores (:1650-1670,
// 4-connected), outflowDeficit and deficitNear (src/core/rkw.ts:72-90) on the host, from those columns.
int sg_run_diagnostics(sg_context* ctx, sg_run run, sg_diagnostics* out) {
  if (!ctx || !out) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  if (!(r->desc.flags & RF_ROTATION)) return fail(ctx, SG_ERR_INVALID, "the run does not track its rotation (switches.rotation = 0)");
  const int nx = r->nx, ny = r->ny;
  const size_t layer = (size_t)nx * ny;
  CK(cudaMemsetAsync(r->desc.rot + M_UP, 0, 6 * sizeof(double), ctx->stream));
  launch_diag_sample(node_launch(ctx, *r));
  CK(cudaGetLastError());
  double rot[R_COUNT];
  std::vector<float> cols(5 * layer);
  CK(cudaMemcpyAsync(rot, r->desc.rot, sizeof rot, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(cols.data(), r->desc.diag + DG_RATE * layer, 5 * layer * 4, cudaMemcpyDeviceToHost, ctx->stream));
  std::vector<float> precip(layer);
  CK(cudaMemcpyAsync(precip.data(), r->desc.cols, layer * 4, cudaMemcpyDeviceToHost, ctx->stream));
  sg_run_counters c;
  int st = sg_run_status(ctx, run, &c);  // (synchronises the stream)
  if (st != SG_OK && st != SG_ERR_NONFINITE) return st;
  auto keyed = [&](int slot) { uint64_t k; std::memcpy(&k, &rot[slot], 8); uint32_t b = (uint32_t)k; float v; std::memcpy(&v, &b, 4); return (double)v; };
  const float *rate = cols.data(), *hail = rate + layer, *gust = hail + layer, *thv = gust + layer, *mask = thv + layer;
  double rainRate = 0, rainTotal = 0, gmax = 0, hmax = 0;
  for (size_t k = 0; k < layer; k++) {
    rainRate = std::max(rainRate, (double)rate[k]); rainTotal = std::max(rainTotal, (double)precip[k]);
    gmax = std::max(gmax, (double)gust[k]); hmax = std::max(hmax, (double)hail[k]);
  }
  // countCores: 4-connected components of the flagged columns, periodic
  std::vector<unsigned char> m(layer);
  for (size_t k = 0; k < layer; k++) m[k] = mask[k] > 0.f ? 1 : 0;
  int cores = 0;
  std::vector<int> stack;
  for (size_t i = 0; i < layer; i++) {
    if (m[i] != 1) continue;
    cores++; m[i] = 2; stack.push_back((int)i);
    while (!stack.empty()) {
      const int a = stack.back(); stack.pop_back();
      const int x = a % nx, y = a / nx;
      const int nb[4] = {(x + 1) % nx + nx * y, (x - 1 + nx) % nx + nx * y, x + nx * ((y + 1) % ny), x + nx * ((y - 1 + ny) % ny)};
      for (int b : nb) if (m[b] == 1) { m[b] = 2; stack.push_back(b); }
    }
  }
  // outflowDeficit: theta_v of the ground columns below their 75th percentile; deficitNear around the low-level rotation
  std::vector<float> sorted(thv, thv + layer);
  std::sort(sorted.begin(), sorted.end());
  const double warm = sorted[(size_t)std::floor((layer - 1) * .75)];
  std::vector<float> deficit(layer);
  double omax = 0;
  for (size_t k = 0; k < layer; k++) { deficit[k] = (float)std::max(0.0, warm - (double)thv[k]); omax = std::max(omax, (double)deficit[k]); }
  const int c0 = (int)rot[R_LOW], x0 = c0 % nx, y0 = c0 / nx;
  const double dx = r->desc.dx, dy = r->desc.dy, radius = 2000;
  const int rx = (int)std::floor(radius / dx), ry = (int)std::floor(radius / dy);
  double near = 0;
  for (int j = -ry; j <= ry; j++) for (int i = -rx; i <= rx; i++) {
    if ((i * dx) * (i * dx) + (j * dy) * (j * dy) > radius * radius) continue;
    near = std::max(near, (double)deficit[((x0 + i) % nx + nx) % nx + nx * (((y0 + j) % ny + ny) % ny)]);
  }
  out->updraft = keyed(M_UP); out->downdraft = keyed(M_DOWN); out->max_cloud = keyed(M_CLOUD); out->cloud_top = keyed(M_TOP);
  out->thermal_top = keyed(M_THERMAL); out->cold_max = keyed(M_COLD);
  out->rain_rate = rainRate; out->rain_total = rainTotal; out->gust = gmax; out->hail = hmax; out->cores = cores;
  out->outflow = omax; out->outflow_low = near; out->clipped = (double)c.clipped;
  return SG_OK;
}

int sg_run_read_pressure(sg_context* ctx, sg_run run, double* p) {
  if (!ctx || !p) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  size_t cells = (size_t)r->nx * r->ny * (r->nz - 1);
  std::vector<float> tmp(cells), tmp2(cells, 0.f);
  CK(cudaMemcpyAsync(tmp.data(), r->desc.pres, cells * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (r->desc.flags & RF_REFINE) CK(cudaMemcpyAsync(tmp2.data(), r->desc.pres2, cells * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (size_t i = 0; i < cells; i++) p[i] = (double)tmp[i] + (double)tmp2[i];  // p1 + p2 of a refined projection
  return SG_OK;
}

int sg_run_status(sg_context* ctx, sg_run run, sg_run_counters* out) {
  if (!ctx || !out) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  double acc[A_COUNT]; unsigned long long cnt[C_COUNT];
  CK(cudaMemcpyAsync(acc, r->desc.acc, sizeof(acc), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(cnt, r->desc.cnt, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  out->steps = (int64_t)cnt[C_STEPS]; out->clipped = (int64_t)cnt[C_CLIPPED]; out->reserved = 0;
  out->failed = cnt[C_TIMEOUT] ? 2 : cnt[C_FAILED] ? 1 : 0;
  out->negative_filled = acc[A_NEG]; out->water_condensed = acc[A_WATER]; out->water_evaporated = acc[A_WATER + 1];
  out->water_rain_evaporated = acc[A_WATER + 2]; out->water_surface = 0;
  if (out->failed == 2) return fail(ctx, SG_ERR_TIMEOUT, "a bounded device wait for the transport's copies ran out; the run is failed");
  return out->failed ? SG_ERR_NONFINITE : SG_OK;
}

int sg_batch_write_fields(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, const float* const* host) {
  return batch_fields(ctx, runs, n, mask, const_cast<float* const*>(host), true);
}
int sg_batch_read_fields(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, float* const* host) {
  return batch_fields(ctx, runs, n, mask, host, false);
}
int sg_batch_write_packed(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, const float* host) {
  return batch_packed(ctx, runs, n, mask, const_cast<float*>(host), true);
}
int sg_batch_read_packed(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, float* host) {
  return batch_packed(ctx, runs, n, mask, host, false);
}
int sg_batch_step_io(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, float* host, int nsteps, int groups) {
  return batch_step_io(ctx, runs, n, mask, host, nsteps, groups);
}
int sg_batch_step_round_trips(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, float* host, int nsteps, int groups) {
  return batch_step_io(ctx, runs, n, mask, host, nsteps, groups, true);
}

int sg_run_retire(sg_context* ctx, sg_run run) {
  if (!ctx) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  cudaStreamSynchronize(ctx->stream);
  drop_plans_with(ctx, run);
  drop_packs_with(ctx, run);
  ctx->used -= r->bytes;
  ctx->pool.emplace(r->bytes, r->mem); ctx->pooled += r->bytes;
  r->live = false; r->mem = nullptr; r->lgt.reset();
  ctx->freeSlots.push_back(run);
  return SG_OK;
}

int sg_run_step(sg_context* ctx, sg_run run, int nsteps) { return sg_batch_step(ctx, &run, 1, nsteps); }

int sg_batch_step(sg_context* ctx, const sg_run* runs, int n, int nsteps) {
  if (!ctx) return SG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  return batch_step(ctx, runs, n, nsteps, true);
}
int sg_batch_step_async(sg_context* ctx, const sg_run* runs, int n, int nsteps) {
  if (!ctx) return SG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  return batch_step(ctx, runs, n, nsteps, false);
}
int sg_synchronize(sg_context* ctx) {
  if (!ctx) return SG_ERR_INVALID;
  CK(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

int sg_time_steps(sg_context* ctx, const sg_run* runs, int n, int nsteps, int use_graph, double* ms) {
  if (!ctx || !ms || nsteps < 1) return SG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  std::vector<int> slots;
  int st = slots_of(ctx, runs, n, slots);
  if (st) return st;
  Plan* P = get_plan(ctx, slots, &st);
  if (!P) return st;
  if (use_graph && (st = ensure_graph(ctx, *P))) return st;
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a)); CK(cudaEventCreate(&b));
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaEventRecord(a, ctx->stream));
  for (int s = 0; s < nsteps; s++) {
    if (use_graph) CK(cudaGraphLaunch(P->exec, ctx->stream));
    else enqueue_step(ctx, *P, [](int) {});
    if (P->elec && (st = discharge_batch(ctx, P->slots)) != SG_OK) return st;
  }
  CK(cudaEventRecord(b, ctx->stream));
  CK(cudaEventSynchronize(b));
  float t = 0; CK(cudaEventElapsedTime(&t, a, b));
  cudaEventDestroy(a); cudaEventDestroy(b);
  CK(cudaGetLastError());
  *ms = t;
  return SG_OK;
}

int sg_profile_kernels(sg_context* ctx, const sg_run* runs, int n, int nsteps, const char** names, double* ms, int64_t* launches, int cap) {
  if (!ctx || !names || !ms || !launches) return SG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  std::vector<int> slots;
  int st = slots_of(ctx, runs, n, slots);
  if (st) return -st;
  Plan* P = get_plan(ctx, slots, &st);
  if (!P) return -st;
  const int K = NKERNELS;
  std::vector<double> total(K, 0); std::vector<int64_t> count(K, 0);
  cudaEvent_t ev[64];
  for (int e = 0; e < 64; e++) cudaEventCreate(&ev[e]);
  for (int s = 0; s < nsteps; s++) {
    int k = 0; int which[64];
    cudaEventRecord(ev[k++], ctx->stream);
    enqueue_step(ctx, *P, [&](int id) { which[k] = id; cudaEventRecord(ev[k++], ctx->stream); });
    cudaStreamSynchronize(ctx->stream);
    for (int e = 1; e < k; e++) { float t; cudaEventElapsedTime(&t, ev[e - 1], ev[e]); total[which[e]] += t; count[which[e]]++; }
  }
  for (int e = 0; e < 64; e++) cudaEventDestroy(ev[e]);
  if (cudaGetLastError() != cudaSuccess) return -SG_ERR_DEVICE;
  int w = 0;
  for (int k = 0; k < K && w < cap; k++) if (count[k]) { names[w] = KERNEL_NAMES[k]; ms[w] = total[k] / count[k]; launches[w] = count[k]; w++; }
  return w;
}

int sg_run_divergence(sg_context* ctx, sg_run run, double* max_abs_div) {
  if (!ctx || !max_abs_div) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  int st; Plan* P = single_plan(ctx, run, &st);
  if (!P) return st;
  CK(cudaMemsetAsync(ctx->d_scalar, 0, 8, ctx->stream));
  launch_divergence_max(lx(ctx, *P, FAM_CELLS), 0, ctx->d_scalar);
  CK(cudaMemcpyAsync(max_abs_div, ctx->d_scalar, 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (!std::isfinite(*max_abs_div)) return fail(ctx, SG_ERR_NONFINITE, "the run's velocities hold a non-finite value");
  return SG_OK;
}

int sg_run_charge(sg_context* ctx, sg_run run, sg_charge_state* out) {
  if (!ctx || !out) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  cudaSetDevice(ctx->device);
  std::memset(out, 0, sizeof(*out));
  if (!r->lgt) return SG_OK;
  double acc[A_COUNT];
  CK(cudaMemcpyAsync(acc, r->desc.acc, sizeof(acc), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  out->ground = acc[A_CHG_GROUND]; out->separated = acc[A_CHG_SEPARATED]; out->ic = acc[A_CHG_IC];
  out->cg_negative = acc[A_CHG_CG_NEG]; out->cg_positive = acc[A_CHG_CG_POS]; out->precipitation = acc[A_CHG_PRECIP];
  out->conduction = acc[A_CHG_CONDUCTION]; out->flashes_ic = (int64_t)acc[A_FLASH_IC]; out->flashes_cg = (int64_t)acc[A_FLASH_CG];
  out->last_flashes = (int32_t)r->lgt->last.size(); out->electrified = 1;
  return SG_OK;
}

int sg_run_flashes(sg_context* ctx, sg_run run, sg_flash* out, int cap, int* count) {
  if (!ctx || !count || cap < 0 || (cap > 0 && !out)) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  *count = r->lgt ? (int)r->lgt->last.size() : 0;
  for (int k = 0; k < *count && k < cap; k++) {
    const FlashRecord& f = r->lgt->last[k];
    sg_flash& o = out[k];
    std::memset(&o, 0, sizeof(o));
    o.time = f.time; o.potential = f.potential; o.charge = f.charge; o.moment = f.moment;
    for (size_t j = 0; j < f.strokes.size() && j < 4; j++) o.stroke_charge[j] = f.strokes[j];
    o.cg = f.cg ? 1 : 0; o.start = f.start; o.ground = f.ground; o.nodes = (int32_t)f.nodes.size(); o.strokes = (int32_t)f.strokes.size();
  }
  return SG_OK;
}

int sg_run_flash_channel(sg_context* ctx, sg_run run, int k, int32_t* nodes, int32_t* parent, int32_t* polarity, int cap) {
  if (!ctx || cap < 0) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  if (!r->lgt || k < 0 || k >= (int)r->lgt->last.size()) return fail(ctx, SG_ERR_INVALID, "no flash " + std::to_string(k) + " in the last step");
  const FlashRecord& f = r->lgt->last[k];
  const int m = std::min(cap, (int)f.nodes.size());
  for (int c = 0; c < m; c++) {
    if (nodes) nodes[c] = f.nodes[c];
    if (parent) parent[c] = f.parent[c];
    if (polarity) polarity[c] = f.polarity[c];
  }
  return SG_OK;
}

int sg_debug_lightning(sg_context* ctx, sg_run run, double* phi, double* rho, int32_t* best, double* ratio, double* last16) {
  if (!ctx || !best || !ratio) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  if (!r->lgt) return fail(ctx, SG_ERR_INVALID, "the run is not electrified");
  cudaSetDevice(ctx->device);
  if (last16 && lightning_state(ctx->stream, *r->lgt, last16) != SG_OK) return fail(ctx, SG_ERR_DEVICE, "lightning state");
  int b = -1;
  const int st = lightning_probe(ctx->stream, r->desc, *r->lgt, phi, rho, &b, ratio);
  *best = b;
  return st == SG_OK ? SG_OK : fail(ctx, st, "lightning probe");
}

int sg_run_discharge(sg_context* ctx, sg_run run, double time, double dt) {
  if (!ctx || !(dt > 0) || !std::isfinite(time)) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run " + std::to_string(run));
  if (!r->lgt) return fail(ctx, SG_ERR_INVALID, "the run is not electrified");
  cudaSetDevice(ctx->device);
  std::string err;
  const int st = lightning_discharge(ctx->stream, &r->grid, r->desc, *r->lgt, time, dt, flash_limit(dt), &err);
  if (st != SG_OK) return fail(ctx, st, "lightning: " + err);
  CK(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ diagnostics
extern "C" {
int sg_set_transport_shape(sg_context* ctx, int tile_x, int tile_y, int weno_group) {
  if (!ctx) return SG_ERR_INVALID;
  if (tile_x == 0) { ctx->pinned[0] = 0; ctx->tuning.clear(); }  // back to tuning, on the runs as they are from now on
  else {
    if (tile_x < 1 || tile_y < 1 || tile_x * tile_y > 320 || tile_x * tile_y < tile_x + tile_y ||
        (tile_x + 6) * (tile_y + 6) > 4 * tile_x * tile_y || (weno_group != 1 && weno_group != 3) ||
        transport_smem(TK_WENO, weno_group, tile_x, tile_y) > (size_t)ctx->maxSmem)
      return fail(ctx, SG_ERR_INVALID, "transport shape out of range");
    ctx->pinned[0] = tile_x; ctx->pinned[1] = tile_y; ctx->pinned[2] = weno_group;
  }
  cudaStreamSynchronize(ctx->stream);
  ctx->plans.clear();
  return SG_OK;
}
int sg_batch_transport_shape(sg_context* ctx, const sg_run* runs, int n, int* shape4) {
  int* shape3 = shape4;
  if (!ctx || !shape3) return SG_ERR_INVALID;
  std::vector<int> slots;
  int st = slots_of(ctx, runs, n, slots);
  if (st != SG_OK) return st;
  Plan* P = get_plan(ctx, slots, &st);
  if (!P) return st;
  shape3[0] = P->TX; shape3[1] = P->TY; shape3[2] = P->wenoG; shape3[3] = P->minb;
  return SG_OK;
}
int sg_batch_transport_copies(sg_context* ctx, const sg_run* runs, int n, int* bulk) {
  if (!ctx || !bulk) return SG_ERR_INVALID;
  std::vector<int> slots;
  int st = slots_of(ctx, runs, n, slots);
  if (st != SG_OK) return st;
  Plan* P = get_plan(ctx, slots, &st);
  if (!P) return st;
  *bulk = P->bulk ? 1 : 0;
  return SG_OK;
}
int sg_debug_step_part(sg_context* ctx, sg_run run, int part) {
  if (!ctx || part < 1 || part > 5) return SG_ERR_INVALID;
  if (!find(ctx, run)) return fail(ctx, SG_ERR_NOT_FOUND, "no run");
  int st; Plan* P = single_plan(ctx, run, &st);
  if (!P) return st;
  enqueue_part(ctx, *P, part, [](int) {});
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaGetLastError());
  return SG_OK;
}
int sg_debug_read_set(sg_context* ctx, sg_run run, int set, int field, float* host) {
  if (!ctx || !host || set < 0 || set > 2 || field < 0) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run");
  size_t n = (size_t)r->nx * r->ny * r->nz;
  if (field >= r->desc.nf) return fail(ctx, SG_ERR_INVALID, "no such field in this run");
  CK(cudaMemcpyAsync(host, sg::field(r->desc, set, field), n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}
int sg_debug_read_faces(sg_context* ctx, sg_run run, float* faces4) {
  if (!ctx || !faces4) return SG_ERR_INVALID;
  Run* r = find(ctx, run);
  if (!r) return fail(ctx, SG_ERR_NOT_FOUND, "no run");
  size_t n = (size_t)r->nx * r->ny * r->nz;
  CK(cudaMemcpyAsync(faces4, r->desc.faces, 4 * n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}
}  // extern "C"

// ==================================================================== serving
namespace {
struct Request {
  sg_grid grid; std::vector<double> zs, dzs, hz;
  std::vector<double> base[7]; sg_switches sw;
  std::vector<std::vector<float>> init;
  int64_t steps, tag;
};
struct Active { sg_run run; int64_t left, tag; };
}  // namespace

struct sg_server {
  sg_context* ctx;
  int maxActive;
  int quantum = 1;      // steps per iteration at most (an iteration stops where the first active run finishes)
  int lastSteps = 0;
  std::deque<Request> queue;
  std::vector<Active> active;
  std::map<int64_t, sg_run> finished;  // done, resident until collected
};

extern "C" {

int sg_server_create(sg_context* ctx, int max_active, sg_server** out) {
  if (!ctx || !out || max_active < 1) return SG_ERR_INVALID;
  *out = new sg_server{ctx, max_active};
  return SG_OK;
}

int sg_server_destroy(sg_server* srv) {
  if (!srv) return SG_ERR_INVALID;
  for (auto& a : srv->active) sg_run_retire(srv->ctx, a.run);
  for (auto& f : srv->finished) sg_run_retire(srv->ctx, f.second);
  delete srv;
  return SG_OK;
}

int sg_server_submit(sg_server* srv, const sg_grid* grid, const sg_base_state* base, const sg_switches* sw, const float* const* init, int64_t steps, int64_t tag) {
  if (!srv || !grid || !base || !sw || !init || steps < 1) return SG_ERR_INVALID;
  int st = validate(srv->ctx, grid, base, sw);
  if (st) return st;
  Request r; r.grid = *grid; int nz = grid->nz;
  r.zs.assign(grid->zs, grid->zs + nz); r.dzs.assign(grid->dzs, grid->dzs + nz - 1); r.hz.assign(grid->hz, grid->hz + nz);
  const double* src[7] = {base->p, base->exner, base->theta, base->q, base->u, base->v, base->rho};
  for (int k = 0; k < 7; k++) r.base[k].assign(src[k], src[k] + nz);
  r.sw = *sw;
  size_t n = (size_t)grid->nx * grid->ny * nz;
  r.init.resize(NF);
  for (int f = 0; f < NF; f++) r.init[f].assign(init[f], init[f] + n);
  r.steps = steps; r.tag = tag;
  srv->queue.push_back(std::move(r));
  return SG_OK;
}

int sg_server_iterate(sg_server* srv, int64_t* done_tags, int* done_count, int cap, int* active, int* queued) {
  if (!srv) return SG_ERR_INVALID;
  sg_context* ctx = srv->ctx;
  // Admit in arrival order while slots and HBM allow.
  while (!srv->queue.empty() && (int)srv->active.size() < srv->maxActive) {
    Request& q = srv->queue.front();
    q.grid.zs = q.zs.data(); q.grid.dzs = q.dzs.data(); q.grid.hz = q.hz.data();
    sg_base_state b{q.base[0].data(), q.base[1].data(), q.base[2].data(), q.base[3].data(), q.base[4].data(), q.base[5].data(), q.base[6].data()};
    std::vector<const float*> init(NF);
    for (int f = 0; f < NF; f++) init[f] = q.init[f].data();
    sg_run run;
    int st = sg_run_create(ctx, &q.grid, &b, &q.sw, init.data(), &run);
    if (st == SG_ERR_BUDGET) break;  // wait for a retirement
    if (st) return st;
    srv->active.push_back(Active{run, q.steps, q.tag});
    srv->queue.pop_front();
  }
  int done = 0;
  srv->lastSteps = 0;
  if (!srv->active.empty()) {
    std::vector<sg_run> ids;
    int64_t q = srv->quantum;
    for (auto& a : srv->active) { ids.push_back(a.run); q = std::min(q, a.left); }
    int st = sg_batch_step(ctx, ids.data(), (int)ids.size(), (int)q);
    if (st) return st;
    srv->lastSteps = (int)q;
    std::vector<Active> keep;
    for (auto& a : srv->active) {
      if ((a.left -= q) > 0) { keep.push_back(a); continue; }
      if (done < cap && done_tags) done_tags[done] = a.tag;
      done++;
      srv->finished[a.tag] = a.run;
    }
    srv->active.swap(keep);
  }
  if (done_count) *done_count = std::min(done, cap);
  if (active) *active = (int)srv->active.size();
  if (queued) *queued = (int)srv->queue.size();
  return SG_OK;
}


int sg_server_set_quantum(sg_server* srv, int steps) {
  if (!srv || steps < 1) return SG_ERR_INVALID;
  srv->quantum = steps;
  return SG_OK;
}
int sg_server_last_steps(sg_server* srv) { return srv ? srv->lastSteps : 0; }

int sg_server_collect(sg_server* srv, int64_t tag, uint32_t mask, float* const* host, float* precipitation) {
  if (!srv) return SG_ERR_INVALID;
  auto it = srv->finished.find(tag);
  if (it == srv->finished.end()) return fail(srv->ctx, SG_ERR_NOT_FOUND, "no finished run with tag " + std::to_string(tag));
  int st = SG_OK;
  if (mask && host) st = sg_run_read_fields(srv->ctx, it->second, mask, host);
  if (!st && precipitation) st = sg_run_read_columns(srv->ctx, it->second, precipitation, nullptr, nullptr);
  if (st) return st;
  sg_run_retire(srv->ctx, it->second);
  srv->finished.erase(it);
  return SG_OK;
}
}  // extern "C"
