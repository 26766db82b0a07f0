// TEST INFRASTRUCTURE ONLY — C entry points of the oracle (a CPU restatement of the reference's StormLab step,
// see oracle_core.h). Loaded by oracle/pyoracle.py for tests/, __graft_entry__.smoke() and bench.py's CPU legs.
#include "oracle_model.h"
#include "oracle_diag.h"
#include "oracle_terrain.h"

using namespace orc;

namespace {
struct LightningHandle {
  GridSpec g; std::unique_ptr<Lightning> l; std::vector<Flash> flashes;
};

void copyFlash(const Flash& f, double* out, int* nodes, int* parent, int* polarity, double* strokes, int cap) {
  const double v[9] = {f.time, f.cg ? 1.0 : 0.0, (double)f.start, (double)f.ground, f.potential, f.charge, f.moment, (double)f.nodes.size(), (double)f.strokes.size()};
  for (int k = 0; k < 9; k++) out[k] = v[k];
  for (int c = 0; c < (int)f.nodes.size() && c < cap; c++) { if (nodes) nodes[c] = f.nodes[c]; if (parent) parent[c] = f.parent[c]; if (polarity) polarity[c] = f.polarity[c]; }
  if (strokes) for (size_t k = 0; k < f.strokes.size() && k < 8; k++) strokes[k] = f.strokes[k];
}

struct Handle {
  bool fp64;
  Model<float>* m32 = nullptr;
  Model<double>* m64 = nullptr;
  // afterStep's rotation tracking (src/core/model.ts:1130-1131) and runMember's swaths (src/ensemble/member.ts:103)
  Rotation rot;
  std::vector<double> uhColumn;
  std::vector<float> gustMax, uhMax;
};

GridSpec makeGrid(int nx, int ny, int nz, double dx, double dy, double dz, double height, const double* zs, const double* dzs, const double* hz) {
  GridSpec g; g.nx = nx; g.ny = ny; g.nz = nz; g.dx = dx; g.dy = dy; g.dz = dz; g.width = dx * nx; g.depth = dy * ny; g.height = height;
  g.zs.assign(zs, zs + nz); g.dzs.assign(dzs, dzs + nz - 1); g.hz.assign(hz, hz + nz); g.finish();
  return g;
}

Switches makeSwitches(const double* s) {
  Switches w;
  w.coriolis = s[0]; w.windRelaxation = s[1]; w.spongeRate = s[2]; w.spongeStart = s[3]; w.cs = s[4]; w.dragCd = s[5];
  w.frameU = s[6]; w.frameV = s[7]; w.loading = s[8] != 0; w.evaporation = s[9] != 0; w.rainFormation = s[10] != 0;
  w.anisotropic = s[11] != 0; w.verticalDz = s[12] != 0; w.durranKlemp = s[13] != 0; w.pressureInStages = s[14] != 0;
  w.ice = s[15] != 0; w.sensible = s[16]; w.latent = s[17]; w.surfaceOn = s[18] != 0; w.slabs = (int)s[19];
  return w;
}

template <class S> std::vector<S>* extraField(Model<S>* m, int id) {
  switch (id) {
    case 100: return &m->precipitation; case 101: return &m->hailGround; case 102: return &m->hailSize;
    case 103: return &m->fallRain; case 104: return &m->fallSnow; case 105: return &m->fallGraupel; case 106: return &m->fallHail;
    case 107: return &m->condensate;
    case 108: return &m->fallChargeIce; case 109: return &m->fallChargeGraupel; case 110: return &m->fieldZ;
    case 111: return &m->rainFallNumber;
    case 112: return &m->graupelFallNumber; case 113: return &m->hailFallNumber;
  }
  return (id >= 0 && id < N_CARRIED) ? &m->f[id] : nullptr;
}
}  // namespace

extern "C" {

// Model. env7 = p, exner, theta, q, u, v, rho (each nz, FP64). sw = 20 switches (makeSwitches).
void* orc_create(int fp64, int nx, int ny, int nz, double dx, double dy, double dz, double height, const double* zs, const double* dzs,
                 const double* hz, const double* env7, const double* sw, int threads) {
  Handle* h = new Handle; h->fp64 = fp64 != 0;
  GridSpec g = makeGrid(nx, ny, nz, dx, dy, dz, height, zs, dzs, hz); Switches s = makeSwitches(sw);
  if (h->fp64) h->m64 = new Model<double>(g, env7, s, threads); else h->m32 = new Model<float>(g, env7, s, threads);
  h->uhColumn.assign(g.layer, 0); h->gustMax.assign(g.layer, 0); h->uhMax.assign(g.layer, 0);
  return h;
}
void orc_destroy(void* p) { Handle* h = (Handle*)p; delete h->m32; delete h->m64; delete h; }
void orc_set_threads(void* p, int threads) {
  Handle* h = (Handle*)p;
  if (h->m32) h->m32->nthreads = std::min(threads, (int)h->m32->dscr.size());
  if (h->m64) h->m64->nthreads = std::min(threads, (int)h->m64->dscr.size());
}
// Field ids: 0..21 carried (rain, snow, graupel, hail, u, v, w, theta, q, cloud, ice, iceNumber, cold, chargeIce,
// chargeGraupel, chargeRain, chargeAir, rainNumber, graupelNumber, graupelVolume, hailNumber, hailVolume); 100
// precipitation, 101 hailGround, 102 hailSize, 103-106 fall speeds, 107 condensate, 108-109 the charge carriers' fall
// speeds, 110 the vertical field (fieldZ), 111-113 the number-weighted fall speeds of rain, graupel and hail.
int orc_set_field(void* p, int id, const double* src, long count) {
  Handle* h = (Handle*)p;
  if (h->m32) { auto* v = extraField(h->m32, id); if (!v || (long)v->size() != count) return -1; for (long i = 0; i < count; i++) (*v)[i] = (float)src[i]; }
  else { auto* v = extraField(h->m64, id); if (!v || (long)v->size() != count) return -1; for (long i = 0; i < count; i++) (*v)[i] = src[i]; }
  return 0;
}
int orc_get_field(void* p, int id, double* dst, long count) {
  Handle* h = (Handle*)p;
  if (h->m32) { auto* v = extraField(h->m32, id); if (!v || (long)v->size() != count) return -1; for (long i = 0; i < count; i++) dst[i] = (*v)[i]; }
  else { auto* v = extraField(h->m64, id); if (!v || (long)v->size() != count) return -1; for (long i = 0; i < count; i++) dst[i] = (*v)[i]; }
  return 0;
}
// Steps with time += dt after each (src/core/fixtures.ts:28-30); each step ends with the rotation tracking
// (afterStep, src/core/model.ts:1130-1131) and, after the time moves, the swaths (runMember, src/ensemble/member.ts:102-103).
void orc_step(void* p, double dt, int steps) {
  Handle* h = (Handle*)p;
  auto go = [&](auto* m) {
    m->step(dt);
    updateRotation(*m, dt, h->rot, h->uhColumn);
    m->time += dt;
    addSwaths(*m, m->time, h->uhColumn, h->gustMax, h->uhMax);
  };
  for (int s = 0; s < steps; s++) { if (h->m32) go(h->m32); else go(h->m64); }
}
// The rotation tracking on the fields as they are (refreshRotation with dt, src/core/model.ts:1607-1609).
void orc_update_rotation(void* p, double dt) {
  Handle* h = (Handle*)p;
  if (h->m32) updateRotation(*h->m32, dt, h->rot, h->uhColumn); else updateRotation(*h->m64, dt, h->rot, h->uhColumn);
}
// out[11]: uh, x, y, anticyclonic, persisted, uh01, uh03, low, coreZeta, coreUH, coreAnti; uhColumn[layer] (nullable).
void orc_rotation(void* p, double* out, double* uhColumn) {
  Handle* h = (Handle*)p;
  const Rotation& r = h->rot;
  const double v[11] = {r.uh, r.x, r.y, r.anticyclonic, r.persisted, r.uh01, r.uh03, r.low, r.coreZeta, r.coreUH, r.coreAnti};
  for (int k = 0; k < 11; k++) out[k] = v[k];
  if (uhColumn) for (size_t c = 0; c < h->uhColumn.size(); c++) uhColumn[c] = h->uhColumn[c];
}
void orc_set_persisted(void* p, double persisted) { ((Handle*)p)->rot.persisted = persisted; }
// out[14]: updraft, downdraft, rainRate, rainTotal, cloudTop, thermalTop, maxCloud, coldMax, cores, outflow, outflowLow,
// gust, hail, clipped (diagnostics, src/core/model.ts:1672-1696, without shear06).
void orc_diagnostics(void* p, double* out) {
  Handle* h = (Handle*)p;
  const Diagnostics d = h->m32 ? diagnostics(*h->m32, h->rot) : diagnostics(*h->m64, h->rot);
  const double v[14] = {d.updraft, d.downdraft, d.rainRate, d.rainTotal, d.cloudTop, d.thermalTop, d.maxCloud, d.coldMax, d.cores,
                        d.outflow, d.outflowLow, d.gust, d.hail, d.clipped};
  for (int k = 0; k < 14; k++) out[k] = v[k];
}
// addSwaths on the fields as they are, at model time `time`, with the given UH column (member.ts:71-89).
void orc_add_swaths(void* p, double time, const double* uhColumn) {
  Handle* h = (Handle*)p;
  std::vector<double> col(uhColumn, uhColumn + h->uhColumn.size());
  if (h->m32) addSwaths(*h->m32, time, col, h->gustMax, h->uhMax); else addSwaths(*h->m64, time, col, h->gustMax, h->uhMax);
}
void orc_swaths(void* p, float* gustMax, float* uhMax) {
  Handle* h = (Handle*)p;
  for (size_t c = 0; c < h->gustMax.size(); c++) { gustMax[c] = h->gustMax[c]; uhMax[c] = h->uhMax[c]; }
}
// Stages of one step, for stage-wise parity: 1 = beginStep, 2 = dynamics, 3 = physicsStep, 4 = mixStep, 5 = final project.
void orc_step_part(void* p, double dt, int part) {
  Handle* h = (Handle*)p;
  auto go = [&](auto* m) {
    switch (part) {
      case 1: m->beginStep(dt); break; case 2: m->dynamics(dt); break; case 3: m->physicsStep(dt); break;
      case 4: m->mixStep(dt); break; case 5: m->project(dt, true); m->time += dt; break;
    }
  };
  if (h->m32) go(h->m32); else go(h->m64);
}
int orc_get_pressure(void* p, double* dst, long count) {
  Handle* h = (Handle*)p; auto& v = h->m32 ? h->m32->pressure : h->m64->pressure;
  if ((long)v.size() != count) return -1;
  std::memcpy(dst, v.data(), count * sizeof(double));
  return 0;
}
int orc_get_faces(void* p, double* mx, double* my, double* mz, double* dv, long count) {
  Handle* h = (Handle*)p; FluxTransport& f = h->m32 ? h->m32->flux : h->m64->flux;
  if ((long)f.mx.size() != count) return -1;
  std::memcpy(mx, f.mx.data(), count * 8); std::memcpy(my, f.my.data(), count * 8); std::memcpy(mz, f.mz.data(), count * 8); std::memcpy(dv, f.div.data(), count * 8);
  return 0;
}
// counters: clipped, negativeFilled, water condensed, evaporated, rainEvaporated, surface, time.
void orc_counters(void* p, double* out) {
  Handle* h = (Handle*)p;
  auto fill = [&](auto* m) { out[0] = m->clipped; out[1] = m->negativeFilled; for (int k = 0; k < 4; k++) out[2 + k] = m->water[k]; out[6] = m->time; };
  if (h->m32) fill(h->m32); else fill(h->m64);
}

// Electrification and lightning (SimConfig.lightning; with ice only). seed: the lightning's (config.seed + 1).
void orc_set_lightning(void* p, int on, int corona, int seed) {
  Handle* h = (Handle*)p;
  auto set = [&](auto* m) { m->sw.lightning = on != 0; m->sw.corona = corona != 0; m->sw.lightningSeed = seed; };
  if (h->m32) set(h->m32); else set(h->m64);
}
// Two-moment rain (AtmosphereModel.rainMoments, src/core/model.ts:842) and its breakup: 0 none, 1 NSSL, 2 Morrison.
void orc_set_rain2m(void* p, int moments, int breakup) {
  Handle* h = (Handle*)p;
  auto set = [&](auto* m) { m->sw.rainMoments = moments; m->sw.rainBreakup = breakup; };
  if (h->m32) set(h->m32); else set(h->m64);
}
// Two-moment graupel and hail (AtmosphereModel.iceMoments, src/core/model.ts:839-840; with two-moment rain and ice only).
void orc_set_ice2m(void* p, int moments) {
  Handle* h = (Handle*)p;
  auto set = [&](auto* m) { m->sw.iceMoments = moments; };
  if (h->m32) set(h->m32); else set(h->m64);
}
// out[11]: chargeGround, separated, ic, cgNegative, cgPositive, precipitation, conduction, flashes IC, flashes CG,
// totalCharge, flashes of the last step.
void orc_charge_state(void* p, double* out) {
  Handle* h = (Handle*)p;
  auto fill = [&](auto* m) {
    const double v[11] = {m->chargeGround, m->chargeSeparated, m->chargeIC, m->chargeCgNegative, m->chargeCgPositive, m->chargePrecipitation,
                          m->chargeConduction, (double)m->flashesIC, (double)m->flashesCG, m->totalCharge(), (double)m->lastFlashes.size()};
    for (int k = 0; k < 11; k++) out[k] = v[k];
  };
  if (h->m32) fill(h->m32); else fill(h->m64);
}
// Flash k of the last step: out[9] = time, cg, start, ground, potential, charge, moment, nodes, strokes; the channel
// (nodes, parent, polarity; up to cap) and the strokes' charges (up to 8). Returns -1 past the end.
int orc_flash(void* p, int k, double* out, int* nodes, int* parent, int* polarity, double* strokes, int cap) {
  Handle* h = (Handle*)p;
  const std::vector<Flash>& f = h->m32 ? h->m32->lastFlashes : h->m64->lastFlashes;
  if (k < 0 || k >= (int)f.size()) return -1;
  copyFlash(f[k], out, nodes, parent, polarity, strokes, cap);
  return 0;
}

// ---------------------------------------------------------------- Lightning on its own (src/core/lightning.test.ts)
void* orc_lightning_create(int nx, int ny, int nz, double dx, double dy, double dz, double height, const double* zs, const double* dzs, const double* hz,
                           const double* air, int seed) {
  auto* L = new LightningHandle;
  L->g = makeGrid(nx, ny, nz, dx, dy, dz, height, zs, dzs, hz);
  L->l = std::make_unique<Lightning>(L->g, air, seed);
  return L;
}
void orc_lightning_destroy(void* p) { delete (LightningHandle*)p; }
void orc_lightning_set_corona(void* p, int on) { ((LightningHandle*)p)->l->corona = on != 0; }
// cloud(): the sum of `count` FP32 fields of n nodes each (fields[k] points to field k).
void orc_lightning_cloud(void* p, float** fields, int count) {
  auto* L = (LightningHandle*)p; std::vector<Arr<float>> a(count);
  for (int k = 0; k < count; k++) a[k] = (Arr<float>)fields[k];
  L->l->cloud(a.data(), count);
}
void orc_lightning_solve(void* p, float** carriers) {
  auto* L = (LightningHandle*)p; Arr<float> a[4] = {(Arr<float>)carriers[0], (Arr<float>)carriers[1], (Arr<float>)carriers[2], (Arr<float>)carriers[3]};
  L->l->solve(a, 4);
}
int orc_lightning_strongest(void* p, int stamp, double* ratio) { auto r = ((LightningHandle*)p)->l->strongest(stamp); *ratio = r.second; return r.first; }
int orc_lightning_discharge(void* p, float** carriers, double time, int limit) {
  auto* L = (LightningHandle*)p; Arr<float> a[4] = {(Arr<float>)carriers[0], (Arr<float>)carriers[1], (Arr<float>)carriers[2], (Arr<float>)carriers[3]};
  L->flashes = L->l->discharge(a, 4, time, limit);
  return (int)L->flashes.size();
}
int orc_lightning_flash(void* p, int k, double* out, int* nodes, int* parent, int* polarity, double* strokes, int cap) {
  auto* L = (LightningHandle*)p;
  if (k < 0 || k >= (int)L->flashes.size()) return -1;
  copyFlash(L->flashes[k], out, nodes, parent, polarity, strokes, cap);
  return 0;
}
double orc_lightning_conduct(void* p, float* ions, double dt) { return ((LightningHandle*)p)->l->conduct((Arr<float>)ions, dt); }
// phi (n), rho (n) of the last solve; state[2] = fromGround, conducted.
void orc_lightning_fields(void* p, double* phi, double* rho, double* state) {
  auto* L = (LightningHandle*)p;
  if (phi) std::memcpy(phi, L->l->phi.data(), L->l->phi.size() * 8);
  if (rho) std::memcpy(rho, L->l->rho.data(), L->l->rho.size() * 8);
  if (state) { state[0] = L->l->fromGround; state[1] = L->l->conducted; }
}
int orc_flash_limit(double dt) { return flashLimit(dt); }

// ---------------------------------------------------------------- two-moment rain (src/core/rain2m.test.ts)
double orc_r2m_bounded(double q, double n, double rho) { return r2m::boundedNumber(q, n, rho); }
double orc_r2m_mean_volume(double q, double n) { return r2m::meanVolume(q, n); }
double orc_r2m_dn(double xv) { return r2m::dnOf(xv); }
void orc_r2m_fall(double q, double n, double rho, double* out3) { r2m::fallSpeeds(q, n, rho, out3[0], out3[1]); out3[2] = r2m::fallSpeedZ(q, n, rho); }
double orc_r2m_limits(int which) { return which == 0 ? r2m::XV_MIN : which == 1 ? r2m::XV_MAX : r2m::RAIN_MIN; }
// v = [q, cloud, rain, number] FP32 cells, in place; returns the evaporated rain.
double orc_r2m_processes(float* v, double tk, double p, double rho, double dt, int breakup, int evaporate) {
  Arr<float> a = (Arr<float>)v;
  return r2m::processes<float>(a, a + 1, a + 2, a + 3, 0, tk, p, rho, dt, breakup, evaporate != 0);
}
// v = [rain, number] FP32 cells, in place.
void orc_r2m_number_change(float* v, double before, double rho, double meanMass) {
  Arr<float> a = (Arr<float>)v;
  r2m::numberChange<float>(a, a + 1, 0, before, rho, meanMass);
}

// ---------------------------------------------------------------- two-moment graupel and hail (src/core/ice2m.test.ts)
double orc_i2m_gamma(double x) { return i2m::gammaFn(x); }
double orc_i2m_upper_gamma(int n, double x) { return i2m::upperGamma(n, x); }
static const i2m::IceClass& i2mClass(int c) { return c == 0 ? i2m::GRAUPEL_2M : i2m::HAIL_2M; }
void orc_i2m_fall_law(double rhoX, double* ab) { i2m::fallLaw(rhoX, ab[0], ab[1]); }
double orc_i2m_density(int c, double q, double vol) { return i2m::densityOf(i2mClass(c), q, vol); }
double orc_i2m_bounded(int c, double q, double n, double vol) { return i2m::boundedIceNumber(i2mClass(c), q, n, vol); }
double orc_i2m_moment_speed(int c, double q, double n, double vol, double rho, int k) { return i2m::momentSpeed(i2mClass(c), q, n, vol, rho, k); }
double orc_i2m_largest(int c, double q, double n, double vol, double rho) { return i2m::largestDiameter(i2mClass(c), q, n, vol, rho); }
double orc_i2m_reflectivity_factor(int c) { return i2m::reflectivityFactor(i2mClass(c).alpha); }
// out5 = n, d1, d2, fall, d2v; returns 0 without the class (null in the reference).
int orc_i2m_rimer_moments(int c, double q, double n, double vol, double rho, double* out5) {
  RimerMoments m;
  if (!i2m::rimerMoments(i2mClass(c), q, n, vol, rho, m)) return 0;
  out5[0] = m.n; out5[1] = m.d1; out5[2] = m.d2; out5[3] = m.fall; out5[4] = m.d2v;
  return 1;
}
// The Seifert-Beheng sweep coefficients of a class (0 graupel, 1 hail) with the droplets (y 0) or an exponential class
// (y 1) for moment k: out3 = delbk(x, 0), delabk(x, y, k), delbk(y, k).
void orc_i2m_sweep_coefficients(int c, int y, int k, double* out3) {
  i2m::MassShape x = i2m::diameterShape(i2mClass(c).alpha), ys = y == 0 ? i2m::DROPLETS : i2m::diameterShape(0);
  out3[0] = i2m::delbk(x, 0); out3[1] = i2m::delabk(x, ys, k); out3[2] = i2m::delbk(ys, k);
}
// v = 14 FP32 cells in Ice2mFields order (theta, q, cloud, ice, iceNumber, snow, rain, rainNumber, graupel, graupelNumber,
// graupelVolume, hail, hailNumber, hailVolume), in place; out3 = cooling, wetG, wetH.
void orc_i2m_processes(float* v, double exner, double p, double rho, double dt, double* out3) {
  Arr<float> a = (Arr<float>)v;
  i2m::Fields<float> f = {a, a + 1, a + 2, a + 3, a + 4, a + 5, a + 6, a + 7, a + 8, a + 9, a + 10, a + 11, a + 12, a + 13};
  i2m::Result r = i2m::processes<float>(f, 0, exner, p, rho, dt);
  out3[0] = r.cooling; out3[1] = r.wetG; out3[2] = r.wetH;
}
// chargingRate with optional two-moment moments (m10 = graupel's five then hail's five; has2 flags which are given).
double orc_charging_rate_2m(double tc, double rho, double cloud, double ice, double snow, double graupel, double hail, double snowFall, int wetG, int wetH,
                            double crystals, const double* m10, const int* has2) {
  RimerMoments m[2]; bool has[2] = {has2[0] != 0, has2[1] != 0};
  for (int j = 0; j < 2; j++) m[j] = {m10[5 * j], m10[5 * j + 1], m10[5 * j + 2], m10[5 * j + 3], m10[5 * j + 4]};
  return chargingRate(tc, rho, cloud, ice, snow, graupel, hail, snowFall, wetG != 0, wetH != 0, crystals, true, m, has);
}

// ---------------------------------------------------------------- charging (src/core/charge.test.ts)
double orc_critical_rar(double tc) { return criticalRar(tc); }
double orc_collision_charge(double tc, double rar, double d, double v, int signedCoefficients) { return collisionCharge(tc, rar, d, v, signedCoefficients != 0); }
double orc_crystal_number(double tc, double qi, double rho) { return crystalNumber(tc, qi, rho); }
double orc_crystal_diameter(double qi, double rho, double tc) { return crystalDiameter(qi, rho, tc); }
double orc_takahashi(double tc, double lwc) { return takahashiCharge(tc, lwc); }
// crystals < 0: not given (estimated from the mass); tak 1: the Takahashi scheme, 0: Saunders-Peck.
double orc_charging_rate(double tc, double rho, double cloud, double ice, double snow, double graupel, double hail, double snowFall, int wetG, int wetH,
                         double crystals, int tak) {
  return chargingRate(tc, rho, cloud, ice, snow, graupel, hail, snowFall, wetG != 0, wetH != 0, crystals, tak != 0);
}
double orc_inductive_rate(double tc, double rho, double cloud, double graupel, double hail, double ez, double rimerCharge, int wetG, int wetH) {
  return inductiveRate(tc, rho, cloud, graupel, hail, ez, rimerCharge, wetG != 0, wetH != 0);
}
void orc_transfer_charge(double* charge, const double* before, const double* after) { transferCharge(charge, before, after); }

// ---------------------------------------------------------------- known-answer hooks (reference unit tests)
double orc_weno(double a, double b, double c, double d, double e) { return weno(a, b, c, d, e); }
double orc_upwind5(double a, double b, double c, double d, double e) { return upwind5(a, b, c, d, e); }
double orc_qsat(double t, double p) { return qsatP(t, p); }
double orc_qsat_ice(double t, double p) { return qsatIce(t, p); }
double orc_fall_speed(double rain, double rho, double rhoGround) { return fallSpeed(rain, rho, rhoGround); }
double orc_snow_fall_speed(double snow, double rho, double rhoGround) { return snowFallSpeed(snow, rho, rhoGround); }
double orc_graupel_fall_speed(double x, double rho) { return graupelFallSpeed(x, rho); }
double orc_hail_fall_speed(double x, double rho) { return hailFallSpeed(x, rho); }
double orc_hail_max_diameter(double x, double rho) { return hailMaxDiameter(x, rho); }
double orc_cooper(double tc) { return cooperCrystals(tc); }
double orc_splintering(double tc) { return splintering(tc); }
double orc_fragments(double lambda) { return fragmentsPerKg(lambda); }
double orc_koenig(double tc, double m) { return koenigGrowth(tc, m); }
double orc_plate_size(double m) { return plateSize(m); }
double orc_crystal_size(double qi, double n, double rho) { return crystalSize(qi, n, rho); }

// Cell processes on float32 cells (the reference tests use Float32Array.of): v = [theta, q, cloud, ice, snow, rain, graupel, hail, number].
double orc_cell(int which, float* v, double exner, double p, double rho, double dt, double aux) {
  Arr<float> th = (Arr<float>)&v[0], q = (Arr<float>)&v[1], cl = (Arr<float>)&v[2], ic = (Arr<float>)&v[3], sn = (Arr<float>)&v[4];
  Arr<float> rn = (Arr<float>)&v[5], gr = (Arr<float>)&v[6], ha = (Arr<float>)&v[7], nb = (Arr<float>)&v[8];
  switch (which) {
    case 0: return rainProcesses<float>(q, cl, rn, 0, aux, p, rho, dt, true);          // aux = tk
    case 1: return saturationAdjust<float>(th, q, cl, 0, exner, p);
    case 2: return saturationAdjustMixed<float>(th, q, cl, ic, 0, exner, p, aux != 0 ? nb : nullptr);
    case 3: freezeRain<float>(th, rn, gr, 0, exner); return 0;
    case 4: return iceProcesses<float>(th, q, ic, sn, nb, 0, exner, p, rho, dt);
    case 5: return snowProcesses<float>(th, q, cl, ic, sn, rn, 0, exner, p, rho, aux, dt);  // aux = rhoGround
    case 6: return graupelProcesses<float>(th, q, cl, ic, sn, rn, gr, 0, exner, p, rho, dt);
    case 7: return hailProcesses<float>(th, q, cl, ic, sn, rn, gr, ha, 0, exner, p, rho, dt);
    case 8: settleCrystals<float>(ic, nb, 0); return 0;
  }
  return NAN;
}

// The per-node microphysics sequence of physics(z) on float32 cells: v = [theta, q, cloud, rain, ice, iceNumber,
// snow, graupel, hail, cold]; flags bit 0 ice, bit 1 evaporation, bit 2 rain formation. Returns the evaporated rain.
double orc_microphysics(float* v, double exner, double p, double rho, double rhoGround, double dt, int flags) {
  Switches sw; sw.ice = flags & 1; sw.evaporation = (flags & 2) != 0; sw.rainFormation = (flags & 4) != 0;
  Arr<float> a = (Arr<float>)v;
  return microphysicsNode<float>(a, a + 1, a + 2, a + 3, a + 9, a + 4, a + 5, a + 6, a + 7, a + 8, 0, exner, p, rho, rhoGround, dt, sw);
}

// The microphysics of a node with two-moment rain, graupel and hail: v = theta, q, cloud, rain, ice, iceNumber, snow,
// graupel, hail, cold, rainNumber, graupelNumber, graupelVolume, hailNumber, hailVolume (FP32 cells, in place); flags as
// orc_microphysics (ice on); wet2 = graupel's and hail's wet growth. Returns the evaporated rain.
double orc_microphysics_2m(float* v, double exner, double p, double rho, double rhoGround, double dt, int flags, int* wet2) {
  Switches sw; sw.ice = true; sw.evaporation = (flags & 2) != 0; sw.rainFormation = (flags & 4) != 0; sw.rainMoments = 2; sw.iceMoments = 2;
  Arr<float> a = (Arr<float>)v;
  i2m::Fields<float> f = {a, a + 1, a + 2, a + 4, a + 5, a + 6, a + 3, a + 10, a + 7, a + 11, a + 12, a + 8, a + 13, a + 14};
  i2m::Result r = {0, false, false};
  double e = microphysicsNode<float>(a, a + 1, a + 2, a + 3, a + 9, a + 4, a + 5, a + 6, a + 7, a + 8, 0, exner, p, rho, rhoGround, dt, sw, a + 10, &f, &r);
  wet2[0] = r.wetG; wet2[1] = r.wetH;
  return e;
}

// The same on FP64 cells (the pure FP64 oracle's arithmetic and storage).
double orc_microphysics64(double* v, double exner, double p, double rho, double rhoGround, double dt, int flags) {
  Switches sw; sw.ice = flags & 1; sw.evaporation = (flags & 2) != 0; sw.rainFormation = (flags & 4) != 0;
  Arr<double> a = (Arr<double>)v;
  return microphysicsNode<double>(a, a + 1, a + 2, a + 3, a + 9, a + 4, a + 5, a + 6, a + 7, a + 8, 0, exner, p, rho, rhoGround, dt, sw);
}

// FFT of length n in place (sign -1 forward, +1 unnormalised inverse).
void orc_fft(int n, double* re, double* im, int sign) { FFT f(n); f.transform(re, im, sign); }
// HorizontalDFT forward of `layers` layers of src; spectra into re/im (nx*ny*layers); then inverse into out.
void orc_hdft(int nx, int ny, int layers, const double* src, double* re, double* im, double* out) {
  HorizontalDFT d(nx, ny, layers); DftScratch s(nx, ny);
  d.forwardLayers([src](size_t i) { return src[i]; }, 0, layers, s);
  std::memcpy(re, d.re.data(), d.re.size() * 8); std::memcpy(im, d.im.data(), d.im.size() * 8);
  d.inverseLayers([out](size_t i, double v) { out[i] = v; }, 0, layers, s);
}
// Pressure projection on float velocities: divergence before/after into div0/div1 (cells), pressure into p.
void orc_pressure_project(int nx, int ny, int nz, double dx, double dy, double dz, double height, const double* zs, const double* dzs, const double* hz,
                          const double* rho, float* u, float* v, float* w, double dt, double* div0, double* div1, double* pOut) {
  GridSpec g = makeGrid(nx, ny, nz, dx, dy, dz, height, zs, dzs, hz);
  PressureSolver s(g, rho); DftScratch ds(nx, ny); ModeScratch ms(nz);
  Arr<float> U = (Arr<float>)u, V = (Arr<float>)v, W = (Arr<float>)w;
  s.divergence<float>(U, V, W, dt, div0, 0, nz - 1);
  s.transform(div0, 0, nz - 1, ds); s.modes(0, ny, ms); s.back(pOut, 0, nz - 1, ds);
  s.correct<float>(pOut, U, V, W, dt, 0, nz);
  s.divergence<float>(U, V, W, dt, div1, 0, nz - 1);
}
// Transport: face fluxes of (u, v, w) projected, then `steps` advect() calls on q (float) with dt. Faces out (may be null).
void orc_transport(int nx, int ny, int nz, double dx, double dy, double dz, double height, const double* zs, const double* dzs, const double* hz,
                   const double* rho, const float* u, const float* v, const float* w, float* q, double dt, int steps, int monotone,
                   double* mx, double* my, double* mz, double* div) {
  GridSpec g = makeGrid(nx, ny, nz, dx, dy, dz, height, zs, dzs, hz);
  FluxTransport t(g, rho); DftScratch ds(nx, ny); ModeScratch ms(nz); TendScratch ts(g.n, nz * ny); std::vector<double> tend(g.n);
  t.setVelocity<float>((Arr<float>)u, (Arr<float>)v, (Arr<float>)w, ds, ms);
  if (mx) { std::memcpy(mx, t.mx.data(), g.n * 8); std::memcpy(my, t.my.data(), g.n * 8); std::memcpy(mz, t.mz.data(), g.n * 8); std::memcpy(div, t.div.data(), g.n * 8); }
  for (int s = 0; s < steps; s++) t.advect<float>((Arr<float>)q, dt, monotone != 0, ts, tend);
}
// Turbulence: viscosity into km/kh (dry when q null), then `steps` mix() calls on a with base/factor when a is not null.
void orc_turbulence(int nx, int ny, int nz, double dx, double dy, double dz, double height, const double* zs, const double* dzs, const double* hz,
                    const double* rho, const float* u, const float* v, const float* w, const float* theta, const double* thetaEnv, double cs, double dt,
                    const float* q, const float* cond, const double* exner, int anisotropic, int verticalDz, int implicitV, int durranKlemp,
                    const double* kmIn, const double* khIn, double* km, double* kh, float* a, const double* base, double factor, int steps) {
  GridSpec g = makeGrid(nx, ny, nz, dx, dy, dz, height, zs, dzs, hz);
  Turbulence t(g, rho); t.anisotropic = anisotropic; t.verticalDz = verticalDz; t.implicitVertical = implicitV; t.durranKlemp = durranKlemp;
  if (kmIn) { std::memcpy(t.km.data(), kmIn, g.n * 8); std::memcpy(t.kh.data(), khIn, g.n * 8); }
  else t.viscosity<float>((Arr<float>)u, (Arr<float>)v, (Arr<float>)w, (Arr<float>)theta, thetaEnv, cs, dt, (Arr<float>)q, (Arr<float>)cond, exner, 0, nz);
  if (km) { std::memcpy(km, t.km.data(), g.n * 8); std::memcpy(kh, t.kh.data(), g.n * 8); }
  std::vector<float> tmp(g.n);
  if (a) for (int s = 0; s < steps; s++) t.mix<float>((Arr<float>)a, base, factor, dt, tmp);
}

// Terrain (terrain.ts): the heights of a form (kind 0 hill, 1 ridge, 2 plateau, 3 schar; NaN for an absent option).
void orc_terrain_heights(int nx, int ny, int nz, double dx, double dy, double dz, double height, const double* zs, const double* dzs, const double* hz,
                         int kind, double top, double width, double x, double y, double heading, double wavelength, float* out) {
  GridSpec g = makeGrid(nx, ny, nz, dx, dy, dz, height, zs, dzs, hz);
  std::vector<float> h = terrain::heights(terrain::Form{kind, top, width, x, y, heading, wavelength}, g);
  std::memcpy(out, h.data(), h.size() * 4);
}
// The cut-cell geometry of ground heights: solid mask, ground levels, node heights, face apertures, slope areas.
void orc_terrain_geometry(int nx, int ny, int nz, double dx, double dy, double dz, double height, const double* zs, const double* dzs, const double* hz,
                          const float* ground, uint8_t* solid, int* levels, double* heights, double* ax, double* ay, float* slope) {
  GridSpec g = makeGrid(nx, ny, nz, dx, dy, dz, height, zs, dzs, hz);
  std::vector<uint8_t> s = terrain::solidMask(g, ground);
  std::memcpy(solid, s.data(), s.size());
  std::vector<int> lv = terrain::groundLevels(g, s.data());
  std::memcpy(levels, lv.data(), lv.size() * 4);
  std::vector<double> h = terrain::nodeHeights(g, s.data(), ground);
  std::memcpy(heights, h.data(), h.size() * 8);
  std::vector<double> a, b;
  terrain::faceApertures(g, s.data(), ground, a, b);
  std::memcpy(ax, a.data(), a.size() * 8); std::memcpy(ay, b.data(), b.size() * 8);
  std::vector<float> sl = terrain::slopeArea(g, ground);
  std::memcpy(slope, sl.data(), sl.size() * 4);
}
// MaskedProjection over ground heights: mask, the cut cells' divergence before, project, the divergence after.
// stats = {iterations, residual}; dropped (cells) the cells without a row.
void orc_masked_project(int nx, int ny, int nz, double dx, double dy, double dz, double height, const double* zs, const double* dzs, const double* hz,
                        const double* rho, const float* ground, double tolerance, int maxIterations, float* u, float* v, float* w, double dt,
                        double* pressure, double* before, double* after, double* stats, uint8_t* dropped) {
  GridSpec g = makeGrid(nx, ny, nz, dx, dy, dz, height, zs, dzs, hz);
  PressureSolver s(g, rho);
  terrain::MaskedProjection m(g, s, ground, tolerance, maxIterations);
  m.mask(u, v, w);
  m.divergence(u, v, w, before);
  m.project(u, v, w, dt, pressure);
  m.divergence(u, v, w, after);
  stats[0] = m.iterations; stats[1] = m.residual;
  std::memcpy(dropped, m.dropped.data(), m.dropped.size());
}

// FluxTransport.setTerrain + setVelocityMasked (advection.ts:78-153) of float velocities over ground heights (the
// model's set-up, model.ts:366-377: nodeHeights and faceApertures of the ground); faces and their divergence out,
// stats = {iterations, residual}.
void orc_masked_faces(int nx, int ny, int nz, double dx, double dy, double dz, double height, const double* zs, const double* dzs, const double* hz,
                      const double* rho, const float* ground, double tolerance, int maxIterations, const float* u, const float* v, const float* w,
                      double* mx, double* my, double* mz, double* div, double* stats) {
  GridSpec g = makeGrid(nx, ny, nz, dx, dy, dz, height, zs, dzs, hz);
  FluxTransport t(g, rho);
  std::vector<uint8_t> solid = terrain::solidMask(g, ground);
  std::vector<double> heights = terrain::nodeHeights(g, solid.data(), ground), ax, ay;
  terrain::faceApertures(g, solid.data(), ground, ax, ay);
  terrain::MaskedFaces m(g, t, solid.data(), heights.data(), ax, ay);
  m.setVelocityMasked<float>((Arr<float>)u, (Arr<float>)v, (Arr<float>)w, tolerance, maxIterations);
  std::memcpy(mx, t.mx.data(), g.n * 8); std::memcpy(my, t.my.data(), g.n * 8); std::memcpy(mz, t.mz.data(), g.n * 8);
  std::memcpy(div, t.div.data(), g.n * 8);
  stats[0] = m.iterations; stats[1] = m.residual;
}

}  // extern "C"
