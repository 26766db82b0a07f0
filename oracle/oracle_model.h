// TEST INFRASTRUCTURE ONLY — the oracle's model step (see oracle_core.h).
// Restates AtmosphereModel.step (src/core/model.ts:873-877) for the configuration of the device path: flat ground,
// WENO transport with the pressure and buoyancy in the RK3 stages, one-moment microphysics (ice or warm), no
// lightning, no budget tracers, no zones/fronts/large-scale forcing, no nudging, periodic edges. Phases run on
// OpenMP threads over the reference's own task split (src/core/threads.ts:44-48): every task writes only its own
// outputs and every sum is taken in task order afterwards, so results are bit-identical for any thread count.
#pragma once
#include <omp.h>
#include "oracle_solvers.h"
#include "oracle_elec.h"
#include "oracle_rain2m.h"
#include "oracle_ice2m.h"

namespace orc {

struct Switches {
  double coriolis = 0, windRelaxation = 1e-4, spongeRate = .06, spongeStart = 14000, cs = SMAGORINSKY, dragCd = 0;
  double frameU = 0, frameV = 0, sensible = 0, latent = 0;
  bool loading = true, evaporation = true, rainFormation = true, anisotropic = true, verticalDz = false, durranKlemp = false;
  bool pressureInStages = true, ice = true, surfaceOn = true;
  int slabs = 1;
  // Electrification and lightning (SimConfig.lightning, with the ice microphysics only: electrified(), model.ts:1316);
  // the lightning's random numbers are seeded with config.seed + 1 (:1538); corona over land (:1539).
  bool lightning = false, corona = true;
  int lightningSeed = 43;
  // Two-moment rain (AtmosphereModel.rainMoments 2, src/core/model.ts:842; rain2m(), :905) and its breakup (:843).
  int rainMoments = 1, rainBreakup = r2m::NONE;
  // Two-moment graupel and hail (iceMoments 2, :839-840; ice2m(), :914: with the ice microphysics and two-moment rain).
  int iceMoments = 1;
};

enum FieldId { F_RAIN, F_SNOW, F_GRAUPEL, F_HAIL, F_U, F_V, F_W, F_THETA, F_Q, F_CLOUD, F_ICE, F_ICENUMBER, F_COLD,
               F_CHARGE_ICE, F_CHARGE_GRAUPEL, F_CHARGE_RAIN, F_CHARGE_AIR,  // charges: src/core/model.ts:210
               F_RAIN_NUMBER,                                                // raindrops per kg (two-moment rain): :194
               F_GRAUPEL_NUMBER, F_GRAUPEL_VOLUME, F_HAIL_NUMBER, F_HAIL_VOLUME,  // two-moment graupel and hail: :202
               N_CARRIED };

// The microphysics part of physics(z) for node i (src/core/model.ts:1391-1471): Kessler rain, then with ice the
// freezing, crystals, snow, graupel, hail, secondary ice and the mixed-phase saturation adjustment, else the warm
// adjustment; the cold-pool indicator's share of the cooling. Returns the evaporated rain.
// With two-moment rain (`rainNumber` given), its processes replace Kessler's and the drop number follows the rain the
// ice processes take or give (:1391, :1402-1435). With two-moment graupel and hail as well (`ice2m` given, its
// rainNumber the same array), their processes replace the one-moment graupel and hail ones (:1420-1426) and `wet2m`
// receives their cooling and wet growth.
template <class S>
double microphysicsNode(Arr<S> theta, Arr<S> q, Arr<S> cloud, Arr<S> rain, Arr<S> cold, Arr<S> ice, Arr<S> iceNumber, Arr<S> snow, Arr<S> graupel,
                        Arr<S> hail, int i, double ex, double pz, double rhoZ, double rhoGround, double dt, const Switches& sw, Arr<S> rainNumber = nullptr,
                        const i2m::Fields<S>* ice2m = nullptr, i2m::Result* wet2m = nullptr) {
  const bool two = rainNumber != nullptr;
  double evap = !sw.rainFormation ? 0
               : two ? r2m::processes<S>(q, cloud, rain, rainNumber, i, (double)theta[i] * ex, pz, rhoZ, dt, sw.rainBreakup, sw.evaporation)
                     : rainProcesses<S>(q, cloud, rain, i, (double)theta[i] * ex, pz, rhoZ, dt, sw.evaporation);
  if (evap > 0) { double cool = LV / CP / ex * evap; theta[i] -= cool; cold[i] += cool; }
  double cond;
  if (sw.ice) {
    double rainMark = rain[i];
    const double frozenDrops = two ? (double)rainNumber[i] : 0, graupelMark = graupel[i];
    freezeRain<S>(theta, rain, graupel, i, ex);
    // two-moment graupel: the drops frozen at once become as many particles of 900 kg/m3 (:1404)
    if (ice2m && (double)graupel[i] > graupelMark) {
      ice2m->graupelNumber[i] += rainMark > 0 ? frozenDrops * (1 - (double)rain[i] / rainMark) : 0; ice2m->graupelVolume[i] += ((double)graupel[i] - graupelMark) / 900;
    }
    if (two) { r2m::numberChange<S>(rain, rainNumber, i, rainMark, rhoZ, 0); rainMark = rain[i]; }
    settleCrystals<S>(ice, iceNumber, i);
    cold[i] += iceProcesses<S>(theta, q, ice, snow, iceNumber, i, ex, pz, rhoZ, dt);
    double iceBefore = ice[i], cloudBefore = cloud[i];
    const double snowMass = two ? r2m::exponentialMeanMass(snow[i], N0S, RHO_S, rhoZ) : 0;
    cold[i] += snowProcesses<S>(theta, q, cloud, ice, snow, rain, i, ex, pz, rhoZ, rhoGround, dt);
    if (two) { r2m::numberChange<S>(rain, rainNumber, i, rainMark, rhoZ, snowMass); rainMark = rain[i]; }
    // (the one-moment snow gives no graupel with RIMED_SNOW_TO_GRAUPEL off, so :1417 never applies)
    double rainBefore = rain[i], rainFrozen;
    if (ice2m) {  // :1421-1426
      i2m::Result r = i2m::processes<S>(*ice2m, i, ex, pz, rhoZ, dt); cold[i] += r.cooling;
      if (wet2m) *wet2m = r;
      rainFrozen = (double)theta[i] * ex < 273.15 ? jmax(0, rainBefore - (double)rain[i]) : 0;
    } else {
      const double graupelMass = two ? r2m::exponentialMeanMass(graupel[i], N0G, RHO_G, rhoZ) : 0;
      cold[i] += graupelProcesses<S>(theta, q, cloud, ice, snow, rain, graupel, i, ex, pz, rhoZ, dt);
      if (two) { r2m::numberChange<S>(rain, rainNumber, i, rainMark, rhoZ, graupelMass); rainMark = rain[i]; }
      rainFrozen = (double)theta[i] * ex < 273.15 ? jmax(0, rainBefore - (double)rain[i]) : 0;
      const double hailMass = two ? r2m::exponentialMeanMass(hail[i], N0H, RHO_H, rhoZ) : 0;
      cold[i] += hailProcesses<S>(theta, q, cloud, ice, snow, rain, graupel, hail, i, ex, pz, rhoZ, dt);
      if (two) r2m::numberChange<S>(rain, rainNumber, i, rainMark, rhoZ, hailMass);
    }
    if (iceBefore > 0) iceNumber[i] *= (double)ice[i] / iceBefore;
    double splinters = splintering((double)theta[i] * ex - 273.15) * SPLINTERS * jmax(0, cloudBefore - (double)cloud[i])
      + (rainFrozen > 0 ? fragmentsPerKg(std::pow(PI * RHO_W * N0R / (rhoZ * rainBefore), .25)) * rainFrozen : 0);
    if (splinters > 0) {
      double fromG = jmin(graupel[i], splinters * CRYSTAL_MASS), fromS = jmin(snow[i], splinters * CRYSTAL_MASS - fromG);
      graupel[i] -= fromG; snow[i] -= fromS; ice[i] += fromG + fromS; iceNumber[i] += (fromG + fromS) / CRYSTAL_MASS;
    }
    cond = saturationAdjustMixed<S>(theta, q, cloud, ice, i, ex, pz, iceNumber);
    settleCrystals<S>(ice, iceNumber, i);
  } else cond = saturationAdjust<S>(theta, q, cloud, i, ex, pz);
  if (cond < 0) cold[i] -= LV / CP / ex * cond * .14;
  return evap;
}

template <class S> struct Model {
  GridSpec g;
  std::vector<double> p, exner, thetaEnv, qEnv, uGround, vGround, rho, uEnv, vEnv, levelWeight, surfaceShare;
  Switches sw;
  std::vector<S> f[N_CARRIED];
  std::vector<S> fallRain, fallSnow, fallGraupel, fallHail, condensate, precipitation, hailGround, hailSize, levelWater;
  // electrification (src/core/model.ts:205-245): the carriers' fall speeds, the vertical field of the last solve, the
  // charge separated per level; the ground's charge, the budget, the flash counts and this step's flashes
  std::vector<S> fallChargeIce, fallChargeGraupel, fieldZ, levelCharge;
  std::vector<S> rainFallNumber;  // two-moment rain: the number-weighted fall speed (:1224)
  std::vector<S> graupelFallNumber, hailFallNumber;  // two-moment graupel and hail: their number-weighted fall speeds (:1227-1228)
  double chargeGround = 0, chargeSeparated = 0, chargeIC = 0, chargeCgNegative = 0, chargeCgPositive = 0, chargePrecipitation = 0, chargeConduction = 0;
  long flashesIC = 0, flashesCG = 0;
  std::vector<Flash> lastFlashes;
  std::unique_ptr<Lightning> lightning;
  std::vector<S> stageStart[N_CARRIED]; std::vector<double> stageTend[N_CARRIED];
  FluxTransport flux; PressureSolver solver; Turbulence turb;
  std::vector<double> pressure, divergence;
  double negativeFilled = 0, time = 0; double clipped = 0;
  double water[4] = {0, 0, 0, 0};
  double taskNegative[N_CARRIED] = {0};
  std::vector<int> groundCell; std::vector<double> groundWeight;
  int nthreads;
  std::vector<DftScratch> dscr; std::vector<ModeScratch> mscr; std::vector<TendScratch> tscr; std::vector<std::vector<S>> mixTmp;

  Arr<S> F(int k) { return reinterpret_cast<Arr<S>>(f[k].data()); }
  static Arr<S> A(std::vector<S>& v) { return reinterpret_cast<Arr<S>>(v.data()); }

  Model(const GridSpec& grid, const double* env7, const Switches& s, int threads) : g(grid), sw(s), nthreads(threads) {
    int nz = g.nz, n = g.n, layer = g.layer;
    auto lvl = [&](int k) { return std::vector<double>(env7 + k * nz, env7 + (k + 1) * nz); };
    p = lvl(0); exner = lvl(1); thetaEnv = lvl(2); qEnv = lvl(3); uGround = lvl(4); vGround = lvl(5); rho = lvl(6);
    uEnv.resize(nz); vEnv.resize(nz);
    for (int z = 0; z < nz; z++) { uEnv[z] = uGround[z] - sw.frameU; vEnv[z] = vGround[z] - sw.frameV; }
    for (int k = 0; k < N_CARRIED; k++) { f[k].assign(n, 0); stageStart[k].assign(n, 0); stageTend[k].assign(n, 0); }
    fallRain.assign(n, 0); fallSnow.assign(n, 0); fallGraupel.assign(n, 0); fallHail.assign(n, 0); condensate.assign(n, 0);
    precipitation.assign(layer, 0); hailGround.assign(layer, 0); hailSize.assign(layer, 0); levelWater.assign(nz * 4, 0);
    fallChargeIce.assign(n, 0); fallChargeGraupel.assign(n, 0); fieldZ.assign(n, 0); levelCharge.assign(nz, 0); rainFallNumber.assign(n, 0);
    graupelFallNumber.assign(n, 0); hailFallNumber.assign(n, 0);
    flux = FluxTransport(g, rho.data()); solver = PressureSolver(g, rho.data()); turb = Turbulence(g, rho.data());
    flux.g = &g; solver.g = &g; turb.g = &g;
    turb.anisotropic = sw.anisotropic; turb.verticalDz = sw.verticalDz; turb.durranKlemp = sw.durranKlemp;
    pressure.assign(solver.cells, 0); divergence.assign(solver.cells, 0);
    levelWeight.resize(nz);
    for (int z = 0; z < nz; z++) levelWeight[z] = g.hz[z] / g.dz * rho[z];  // src/core/model.ts:386
    // sharesAbove(0) (src/core/model.ts:762-767)
    int first500 = -1; for (int z = 0; z < nz; z++) if (g.zs[z] - g.zs[0] >= 500) { first500 = z; break; }
    int low = std::max(2, first500); double total = 0; surfaceShare.assign(low, 0);
    for (int z = 0; z < low; z++) { surfaceShare[z] = std::exp(-(g.zs[z] - g.zs[0]) / 300); total += surfaceShare[z] * g.hz[z]; }
    for (int z = 0; z < low; z++) surfaceShare[z] /= total;
    groundCell.assign(layer * 4, 0); groundWeight.assign(layer * 4, 0);
    dscr.resize(threads); mscr.resize(threads); tscr.resize(threads); mixTmp.resize(threads);
    for (int t = 0; t < threads; t++) { dscr[t] = DftScratch(g.nx, g.ny); mscr[t] = ModeScratch(nz); tscr[t] = TendScratch(n, nz * g.ny); mixTmp[t].assign(n, 0); }
  }

  template <class Fn> void run(int tasks, Fn fn) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int k = 0; k < tasks; k++) fn(k, omp_get_thread_num());
  }

  struct Carried { int k; bool monotone, conserve; double decay; };
  std::vector<Carried> carried() const {  // src/core/model.ts:1319-1335
    std::vector<Carried> c;
    c.push_back({F_RAIN, true, true, 1});
    if (sw.ice) { c.push_back({F_SNOW, true, true, 1}); c.push_back({F_GRAUPEL, true, true, 1}); c.push_back({F_HAIL, true, true, 1}); }
    if (rain2m()) c.push_back({F_RAIN_NUMBER, true, false, 1});  // :1323
    if (ice2m()) for (int k : {F_GRAUPEL_NUMBER, F_GRAUPEL_VOLUME, F_HAIL_NUMBER, F_HAIL_VOLUME}) c.push_back({k, true, false, 1});  // :1324
    for (int k : {F_U, F_V, F_W, F_THETA}) c.push_back({k, false, false, 1});
    c.push_back({F_Q, true, true, 1}); c.push_back({F_CLOUD, true, true, 1});
    if (sw.ice) { c.push_back({F_ICE, true, true, 1}); c.push_back({F_ICENUMBER, true, false, 1}); }
    c.push_back({F_COLD, true, false, .9992});
    if (electrified()) for (int k : {F_CHARGE_ICE, F_CHARGE_GRAUPEL, F_CHARGE_RAIN, F_CHARGE_AIR}) c.push_back({k, true, false, 1});  // :1331
    return c;
  }
  bool electrified() const { return sw.ice && sw.lightning; }  // :1316
  bool rain2m() const { return sw.rainMoments == 2; }             // :905 (the WENO transport is the only one here)
  bool ice2m() const { return sw.iceMoments == 2 && sw.ice && rain2m(); }  // :914
  i2m::Fields<S> fields2m() {
    return {F(F_THETA), F(F_Q), F(F_CLOUD), F(F_ICE), F(F_ICENUMBER), F(F_SNOW), F(F_RAIN), F(F_RAIN_NUMBER), F(F_GRAUPEL), F(F_GRAUPEL_NUMBER),
            F(F_GRAUPEL_VOLUME), F(F_HAIL), F(F_HAIL_NUMBER), F(F_HAIL_VOLUME)};
  }

  // ---------------------------------------------------------- beginStep (src/core/model.ts:893-902)
  void updateGround() {  // :644-657 (the surface pattern, city and zones are zero in the device's configuration)
    int nx = g.nx, ny = g.ny; double ox = sw.frameU * time, oy = sw.frameV * time;
    double sx = jmod(ox / g.dx, nx), sy = jmod(oy / g.dy, ny);
    int x0 = (int)std::floor(sx), y0 = (int)std::floor(sy); double fx = sx - x0, fy = sy - y0;
    for (int y = 0; y < ny; y++) for (int x = 0; x < nx; x++) {
      int i = x + nx * y, ax = (x + x0) % nx, bx = (ax + 1) % nx, ay = (y + y0) % ny * nx, by = (ay / nx + 1) % ny * nx, k = i * 4;
      groundCell[k] = ax + ay; groundCell[k + 1] = bx + ay; groundCell[k + 2] = ax + by; groundCell[k + 3] = bx + by;
      groundWeight[k] = (1 - fx) * (1 - fy); groundWeight[k + 1] = fx * (1 - fy); groundWeight[k + 2] = (1 - fx) * fy; groundWeight[k + 3] = fx * fy;
    }
  }
  void deposit(int i, double mm, std::vector<S>& target) {  // :691-694
    Arr<S> t = A(target); int k = i * 4;
    for (int j = 0; j < 4; j++) if (groundWeight[k + j] > 0) t[groundCell[k + j]] += groundWeight[k + j] * mm;
  }
  void fall(int k) {  // 'fall' task (:1220-1235), one-moment
    int layer = g.layer; Arr<S> rain = F(F_RAIN), snow = F(F_SNOW), graupel = F(F_GRAUPEL), hail = F(F_HAIL);
    Arr<S> fr = A(fallRain), fs = A(fallSnow), fg = A(fallGraupel), fh = A(fallHail);
    for (int i = k * layer, end = i + layer; i < end; i++) {
      fr[i] = fallSpeed(rain[i], rho[k], rho[0]); fs[i] = snowFallSpeed(snow[i], rho[k], rho[0]);
      fg[i] = graupelFallSpeed(graupel[i], rho[k]); fh[i] = hailFallSpeed(hail[i], rho[k]);
    }
    if (rain2m()) {  // :1224
      Arr<S> num = F(F_RAIN_NUMBER), rfn = A(rainFallNumber);
      for (int i = k * layer, end = i + layer; i < end; i++) { double vm, vn; r2m::fallSpeeds(rain[i], num[i], rho[k], vm, vn); fr[i] = vm; rfn[i] = vn; }
    }
    if (ice2m()) {  // :1226-1229
      Arr<S> gn = F(F_GRAUPEL_NUMBER), gv = F(F_GRAUPEL_VOLUME), hn = F(F_HAIL_NUMBER), hv = F(F_HAIL_VOLUME), gfn = A(graupelFallNumber), hfn = A(hailFallNumber);
      for (int i = k * layer, end = i + layer; i < end; i++) {
        fg[i] = i2m::momentSpeed(i2m::GRAUPEL_2M, graupel[i], gn[i], gv[i], rho[k], 3); gfn[i] = i2m::momentSpeed(i2m::GRAUPEL_2M, graupel[i], gn[i], gv[i], rho[k], 0);
        fh[i] = i2m::momentSpeed(i2m::HAIL_2M, hail[i], hn[i], hv[i], rho[k], 3); hfn[i] = i2m::momentSpeed(i2m::HAIL_2M, hail[i], hn[i], hv[i], rho[k], 0);
      }
    }
    if (electrified()) {  // :1230-1234
      Arr<S> ice = F(F_ICE), ci = A(fallChargeIce), cg = A(fallChargeGraupel);
      for (int i = k * layer, end = i + layer; i < end; i++) {
        double is = (double)ice[i] + (double)snow[i], gh = (double)graupel[i] + (double)hail[i];
        ci[i] = is > 0 ? (double)snow[i] * (double)fs[i] / is : 0;
        cg[i] = gh > 0 ? ((double)graupel[i] * (double)fg[i] + (double)hail[i] * (double)fh[i]) / gh : 0;
      }
    }
  }
  void collectHail(double dt) {  // :697-706
    int layer = g.layer; Arr<S> hail = F(F_HAIL), fh = A(fallHail), hs = A(hailSize);
    for (int b = 0; b < layer; b++) {
      int i = b; double h = hail[i];
      if (!(h > 1e-9)) continue;
      deposit(b, rho[0] * h * (double)fh[i] * dt, hailGround);
      double size = (ice2m() ? i2m::largestDiameter(i2m::HAIL_2M, hail[i], F(F_HAIL_NUMBER)[i], F(F_HAIL_VOLUME)[i], rho[0]) : hailMaxDiameter(hail[i], rho[0])) * 1000;  // largestHail :709-711
      for (int j = 0; j < 4; j++) if (groundWeight[b * 4 + j] > 0) { int c = groundCell[b * 4 + j]; hs[c] = jmax(hs[c], size); }
    }
  }
  int fallParts(Arr<S> rain, Arr<S> vt, double dt) {  // :575-580
    int nz = g.nz, layer = g.layer; double courant = 0;
    for (int z = 0; z < nz; z++) { double c = dt * rho[z] / (levelWeight[z] * g.dz); for (int i = z * layer; i < (z + 1) * layer; i++) if ((double)rain[i] != 0) courant = jmax(courant, c * (double)vt[i] / 1); }
    return (int)jmax(1, std::ceil(courant / .8));
  }
  void sedimentPart(Arr<S> rain, Arr<S> vt, double dt, bool water = true) {  // :582-598 (flat ground)
    int nz = g.nz, layer = g.layer;
    if (water) for (int c = 0; c < layer; c++) deposit(c, rho[0] * (double)rain[c] * (double)vt[c] * dt, precipitation);
    else {  // a charge carrier: what falls through the ground goes to the ground's charge (:588-591)
      double out = 0;
      for (int i = 0; i < layer; i++) out += (double)rain[i] * (double)vt[i];
      out *= rho[0];
      double q = out * dt * g.dx * g.dy; chargeGround += q; chargePrecipitation += q;
    }
    run(64, [&](int part, int) {
      int c0 = (int)((long)part * layer / 64), c1 = (int)((long)(part + 1) * layer / 64);
      for (int z = 0; z < nz; z++) {
        int l = z * layer; double inflow = z < nz - 1 ? rho[z + 1] : 0;
        for (int i = l + c0; i < l + c1; i++)
          rain[i] += dt * (inflow * (z < nz - 1 ? (double)rain[i + layer] * (double)vt[i + layer] : 0) - rho[z] * (double)rain[i] * (double)vt[i]) / (levelWeight[z] * g.dz * 1);
      }
    });
  }
  void sedimentStep(double dt) {  // :928-932
    std::pair<int, std::vector<S>*> falls[4] = {{F_RAIN, &fallRain}, {F_SNOW, &fallSnow}, {F_GRAUPEL, &fallGraupel}, {F_HAIL, &fallHail}};
    for (int j = rain2m() ? 1 : 0; j < (sw.ice ? 4 : 1); j++) {  // sedimented(): two-moment rain falls on its own (:907-911)
      if (ice2m() && j >= 2) continue;                            // and so do two-moment graupel and hail
      Arr<S> field = F(falls[j].first), vt = A(*falls[j].second);
      int parts = fallParts(field, vt, dt);
      for (int q = 0; q < parts; q++) sedimentPart(field, vt, dt / parts);
    }
    if (electrified()) {  // chargeFalls (:562), :931
      std::pair<int, std::vector<S>*> charges[3] = {{F_CHARGE_ICE, &fallChargeIce}, {F_CHARGE_GRAUPEL, &fallChargeGraupel}, {F_CHARGE_RAIN, &fallRain}};
      for (auto& cf : charges) {
        Arr<S> field = F(cf.first), vt = A(*cf.second);
        int parts = fallParts(field, vt, dt);
        for (int q = 0; q < parts; q++) sedimentPart(field, vt, dt / parts, false);
      }
    }
  }
  void beginStep(double dt) {
    updateGround();
    run(g.nz, [&](int k, int) { fall(k); });
    if (sw.ice) collectHail(dt);
    if (rain2m()) sedimentRain2m(dt);  // :899
    if (ice2m()) {                     // :900
      sediment2m(dt, F(F_GRAUPEL), F(F_GRAUPEL_NUMBER), F(F_GRAUPEL_VOLUME), A(fallGraupel), A(graupelFallNumber), &i2m::GRAUPEL_2M);
      sediment2m(dt, F(F_HAIL), F(F_HAIL_NUMBER), F(F_HAIL_VOLUME), A(fallHail), A(hailFallNumber), &i2m::HAIL_2M);
    }
    sedimentStep(dt);
  }
  // sedimentRain2m / sedimentIce2m / sediment2m (:916-988; NSSL sediment1d, infall 4): mass with its mass-weighted speed,
  // number with its number-weighted one, a two-moment ice class's volume with the mass, and each sub-step the number
  // kept between what the reflectivity (at its own speed) and a number carried at the mass's speed imply. Flat ground.
  void sedimentRain2m(double dt) { sediment2m(dt, F(F_RAIN), F(F_RAIN_NUMBER), nullptr, A(fallRain), A(rainFallNumber), nullptr); }
  void sediment2m(double dt, Arr<S> q, Arr<S> num, Arr<S> vol, Arr<S> vm, Arr<S> vn, const i2m::IceClass* c) {
    int nz = g.nz, layer = g.layer, n = g.n;
    const double qMin = c ? i2m::ICE2M_MIN : r2m::RAIN_MIN, g1 = c ? i2m::reflectivityFactor(c->alpha) : r2m::G1;
    // the reflectivity's particle density: water's, or the class's own now, bounded to 170-900 kg/m3 (:920)
    auto k6of = [&](int i) { double rx = c ? jmin(900, jmax(170, i2m::densityOf(*c, q[i], vol[i]))) : r2m::RHO_W2; return std::pow(6 / (PI * rx), 2); };
    std::vector<double> refl(n), carriedN(n); std::vector<float> vzv(n);
    double courant = 0;
    for (int z = 0; z < nz; z++) for (int i = z * layer; i < (z + 1) * layer; i++) {
      vzv[i] = (float)(c ? ((double)q[i] > qMin ? i2m::momentSpeed(*c, q[i], num[i], vol[i], rho[z], 6) : 0)
                         : ((double)q[i] > qMin ? r2m::fallSpeedZ(q[i], num[i], rho[z]) : 0));
      double h = g.hz[z];
      courant = jmax(courant, jmax(dt * (double)vzv[i] / h, dt * (double)vm[i] / h));
    }
    const int parts = (int)jmax(1, std::ceil(courant / .8));
    const double step = dt / parts;
    for (int p = 0; p < parts; p++) {
      for (int z = 0; z < nz; z++) for (int i = z * layer; i < (z + 1) * layer; i++) {
        double rq = rho[z] * (double)q[i], rn = rho[z] * (double)num[i], k6 = k6of(i);
        refl[i] = rq > 0 && rn > 0 ? g1 * k6 * rq * rq / rn : 0;
        carriedN[i] = num[i];
      }
      for (int c = 0; c < layer; c++) deposit(c, rho[0] * (double)q[c] * (double)vm[c] * step, precipitation);
      for (int z = 0; z < nz; z++) {
        bool top = z < nz - 1; double level = rho[z] * g.hz[z];
        for (int i = z * layer; i < (z + 1) * layer; i++) {
          int a = i + layer; double m = level;
          q[i] += step * ((top ? rho[z + 1] * (double)q[a] * (double)vm[a] : 0) - rho[z] * (double)q[i] * (double)vm[i]) / m;
          if (vol) vol[i] += step * ((top ? rho[z + 1] * (double)vol[a] * (double)vm[a] : 0) - rho[z] * (double)vol[i] * (double)vm[i]) / m;
          num[i] += step * ((top ? rho[z + 1] * (double)num[a] * (double)vn[a] : 0) - rho[z] * (double)num[i] * (double)vn[i]) / m;
          carriedN[i] += step * ((top ? rho[z + 1] * carriedN[a] * (double)vm[a] : 0) - rho[z] * carriedN[i] * (double)vm[i]) / m;
          refl[i] += step * ((top ? refl[a] * (double)vzv[a] : 0) - refl[i] * (double)vzv[i]) / g.hz[z];
        }
      }
      for (int z = 0; z < nz; z++) for (int i = z * layer; i < (z + 1) * layer; i++) {
        if (!((double)q[i] > qMin)) { if ((double)q[i] < 0) q[i] = 0.0; num[i] = 0.0; if (vol) vol[i] = 0.0; continue; }
        double rq = rho[z] * (double)q[i], k6 = k6of(i), fromZ = refl[i] > 0 ? g1 * k6 * rq * rq / refl[i] / rho[z] : INFINITY;
        num[i] = refl[i] > 0 ? jmax(jmin(fromZ, carriedN[i]), (double)num[i]) : jmax(carriedN[i], (double)num[i]);
      }
    }
  }

  // ---------------------------------------------------------- dynamics (src/core/model.ts:1029-1051)
  void stageBuoyancy(double* tend, int z0, int z1) {  // :1204-1214 (no zones)
    int layer = g.layer; Arr<S> theta = F(F_THETA), q = F(F_Q), cloud = F(F_CLOUD), ice = F(F_ICE), rain = F(F_RAIN), snow = F(F_SNOW), graupel = F(F_GRAUPEL), hail = F(F_HAIL);
    for (int z = z0; z < z1; z++) {
      double thEnv = thetaEnv[z], qE = qEnv[z], thvEnv = thEnv * (1 + .61 * qE);
      for (int i = z * layer, c = 0; c < layer; i++, c++) {
        double ref = thvEnv;
        double loaded = (double)cloud[i] + (double)ice[i] + (sw.loading ? (double)rain[i] + (double)snow[i] + (double)graupel[i] + (double)hail[i] : 0);
        tend[i] += G * (((double)theta[i] * (1 + .61 * (double)q[i]) - ref) / ref - loaded);
      }
    }
  }
  void project(double dt, bool limit) {  // :1575-1583
    int nz = g.nz, ny = g.ny;
    Arr<S> u = F(F_U), v = F(F_V), w = F(F_W);
    run(nz - 1, [&](int k, int) { solver.divergence<S>(u, v, w, dt, divergence.data(), k, k + 1); });
    run(nz - 1, [&](int k, int t) { solver.transform(divergence.data(), k, k + 1, dscr[t]); });
    run(ny, [&](int n, int t) { solver.modes(n, n + 1, mscr[t]); });
    run(nz - 1, [&](int k, int t) { solver.back(pressure.data(), k, k + 1, dscr[t]); });
    run(nz, [&](int k, int) { solver.correct<S>(pressure.data(), u, v, w, dt, k, k + 1); });
    if (limit) clipWind();
  }
  void clipWind() {  // :1586-1595
    Arr<S> u = F(F_U), v = F(F_V), w = F(F_W); double c = 0;
    for (int i = 0; i < g.n; i++) {
      if ((double)u[i] < -U_LIMIT || (double)u[i] > U_LIMIT) { u[i] = clamp(u[i], -U_LIMIT, U_LIMIT); c++; }
      if ((double)v[i] < -U_LIMIT || (double)v[i] > U_LIMIT) { v[i] = clamp(v[i], -U_LIMIT, U_LIMIT); c++; }
      if ((double)w[i] < -W_LIMIT || (double)w[i] > W_LIMIT) { w[i] = clamp(w[i], -W_LIMIT, W_LIMIT); c++; }
    }
    clipped += c;
  }
  void faceProjection() {  // the 'faces' .. 'faceDivergence' phases (:1039)
    int nz = g.nz, ny = g.ny; Arr<S> u = F(F_U), v = F(F_V), w = F(F_W);
    run(nz, [&](int k, int) { flux.faces<S>(u, v, w, k, k + 1); });
    run(nz, [&](int k, int) { flux.divergence(k, k + 1); });
    run(nz, [&](int k, int t) { flux.forward(k, k + 1, dscr[t]); });
    run(ny, [&](int n, int t) { flux.modes(n, n + 1, mscr[t]); });
    run(nz, [&](int k, int t) { flux.inverse(k, k + 1, dscr[t]); });
    run(nz, [&](int k, int) { flux.correctFaces(k, k + 1); });
    run(nz, [&](int k, int) { flux.divergence(k, k + 1); });
  }
  void dynamics(double dt) {
    int nz = g.nz, layer = g.layer;
    faceProjection();
    std::vector<Carried> c = carried(); int slabs = std::max(1, std::min(sw.slabs, nz)); int tasks = (int)c.size() * slabs;
    for (int stage = 0; stage < 3; stage++) {
      run(tasks, [&](int k, int t) {  // 'tendency{s}' (:1237-1249)
        int fi = k / slabs, j = k % slabs; const Carried& cc = c[fi];
        int z0 = (int)std::floor((double)j * nz / slabs), z1 = (int)std::floor((double)(j + 1) * nz / slabs);
        Arr<S> a = F(cc.k);
        if (stage == 0) for (size_t i = (size_t)z0 * layer; i < (size_t)z1 * layer; i++) stageStart[cc.k][i] = f[cc.k][i];
        flux.tendency<S>(a, stageTend[cc.k].data(), z0, z1, cc.monotone, tscr[t]);
        if (cc.k == F_W && sw.pressureInStages) stageBuoyancy(stageTend[cc.k].data(), z0, z1);
      });
      double fraction = RK3[stage] * dt;
      run(tasks, [&](int k, int) {  // 'update{s}' (:1250)
        int fi = k / slabs, j = k % slabs; const Carried& cc = c[fi];
        int z0 = (int)std::floor((double)j * nz / slabs), z1 = (int)std::floor((double)(j + 1) * nz / slabs);
        Arr<S> a = F(cc.k); const S* start = stageStart[cc.k].data(); const double* tend = stageTend[cc.k].data();
        for (size_t i = (size_t)z0 * layer; i < (size_t)z1 * layer; i++) a[i] = (double)start[i] + fraction * tend[i];
      });
      if (sw.pressureInStages && stage < 2) {
        Arr<S> w = F(F_W); int top = (nz - 1) * layer;
        for (int b = 0; b < layer; b++) { w[b] = 0.0; w[b + top] = 0.0; }
        project(dt, false);
      }
    }
  }

  // ---------------------------------------------------------- endStep (src/core/model.ts:1103-1195)
  double fillNegative(Arr<S> a) {  // :606-617 (flat ground)
    int nz = g.nz, layer = g.layer; double removed = 0, kept = 0, negative = 0;
    for (int z = 0, i = 0; z < nz; z++) {
      double level = levelWeight[z];
      for (int e = i + layer; i < e; i++) { double x = a[i], wz = level; if (x < TINY_WATER) { if (x != 0) { removed += wz * x; if (x < 0) negative -= wz * x; } } else kept += wz * x; }
    }
    if (removed == 0 && negative == 0) return 0;
    double scale = kept > 0 ? jmax(0, 1 + removed / kept) : 0;
    for (int i = 0; i < g.n; i++) a[i] = (double)a[i] < TINY_WATER ? 0 : (double)a[i] * scale;
    return negative;
  }
  void physics(int z, double dt) {  // :1347-1531 for the device configuration
    int nx = g.nx, ny = g.ny, layer = g.layer;
    double nodeMass = g.dx * g.dy * g.hz[z] * rho[z]; double wCond = 0, wEvap = 0, wRain = 0, wSurf = 0;
    Arr<S> u = F(F_U), v = F(F_V), w = F(F_W), theta = F(F_THETA), q = F(F_Q), cloud = F(F_CLOUD), rain = F(F_RAIN), cold = F(F_COLD);
    Arr<S> ice = F(F_ICE), iceNumber = F(F_ICENUMBER), snow = F(F_SNOW), graupel = F(F_GRAUPEL), hail = F(F_HAIL);
    double rhoGround = rho[0], f = sw.coriolis, keep = std::exp(-sw.windRelaxation * dt), H = g.height;
    double alt = g.zs[z], pz = p[z], rhoZ = rho[z], ex = exner[z], ue = uEnv[z], ve = vEnv[z], thEnv = thetaEnv[z];
    const bool electric = electrified(), two2m = ice2m(); double wCharge = 0;
    const i2m::Fields<S> f2m = fields2m();
    Arr<S> cI = F(F_CHARGE_ICE), cG = F(F_CHARGE_GRAUPEL), cR = F(F_CHARGE_RAIN), cA = F(F_CHARGE_AIR), snowFall = A(fallSnow), ez = A(fieldZ);
    for (int y = 0; y < ny; y++) for (int x = 0, i = z * layer + y * nx; x < nx; x++, i++) {
      double q0 = q[i];
      double before[4] = {0, 0, 0, 0};
      if (electric) { before[0] = (double)ice[i] + (double)snow[i]; before[1] = (double)graupel[i] + (double)hail[i]; before[2] = rain[i]; before[3] = cloud[i]; }
      i2m::Result wet2m = {0, false, false};
      double evap = microphysicsNode<S>(theta, q, cloud, rain, cold, ice, iceNumber, snow, graupel, hail, i, ex, pz, rhoZ, rhoGround, dt, sw,
                                        rain2m() ? F(F_RAIN_NUMBER) : nullptr, two2m ? &f2m : nullptr, &wet2m);
      if (electric) {  // :1454-1469 (after the microphysics' last change to the carriers; only cold changes after it there)
        double after[4] = {(double)ice[i] + (double)snow[i], (double)graupel[i] + (double)hail[i], (double)rain[i], (double)cloud[i]};
        double now[4] = {cI[i], cG[i], cR[i], cA[i]};
        if (now[0] != 0 || now[1] != 0 || now[2] != 0 || now[3] != 0) transferCharge(now, before, after);
        double tc = (double)theta[i] * ex - 273.15;
        bool wetG = two2m ? wet2m.wetG : wetGrowing(graupel[i], N0G, RHO_G, tc, q[i], pz, rhoZ, cloud[i], rain[i], ice[i], snow[i]);
        bool wetH = two2m ? wet2m.wetH : wetGrowing(hail[i], N0H, RHO_H, tc, q[i], pz, rhoZ, cloud[i], rain[i], ice[i], snow[i]);
        // two-moment graupel and hail charge by their own distributions (:1462-1466)
        RimerMoments mom[2]; bool has[2] = {false, false};
        if (two2m) {
          has[0] = i2m::rimerMoments(i2m::GRAUPEL_2M, graupel[i], f2m.graupelNumber[i], f2m.graupelVolume[i], rhoZ, mom[0]);
          has[1] = i2m::rimerMoments(i2m::HAIL_2M, hail[i], f2m.hailNumber[i], f2m.hailVolume[i], rhoZ, mom[1]);
        }
        double separated = chargingRate(tc, rhoZ, cloud[i], ice[i], snow[i], graupel[i], hail[i], snowFall[i], wetG, wetH, (double)iceNumber[i] * rhoZ, true,
                                        two2m ? mom : nullptr, has) * dt / rhoZ;
        double induced = inductiveRate(tc, rhoZ, cloud[i], graupel[i], hail[i], ez[i], (now[1] + separated) * rhoZ, wetG, wetH, two2m ? mom : nullptr, has) * dt / rhoZ;
        cI[i] = now[0] - separated; cG[i] = now[1] + separated + induced; cR[i] = now[2]; cA[i] = now[3] - induced;
        wCharge += std::fabs(separated) + std::fabs(induced);
      }
      if (!sw.pressureInStages) {
        double thvEnv = thEnv * (1 + .61 * qEnv[z]);
        double buoy = ((double)theta[i] * (1 + .61 * (double)q[i]) - thvEnv) / thvEnv - (double)cloud[i] - (double)ice[i] - (sw.loading ? (double)rain[i] + (double)snow[i] + (double)graupel[i] + (double)hail[i] : 0);
        w[i] += G * buoy * dt;
      }
      double du = ((double)u[i] - ue) * keep, dv = ((double)v[i] - ve) * keep; u[i] = ue + du + f * dv * dt; v[i] = ve + dv - f * du * dt;
      { double dq = (double)q[i] - q0; if (dq < 0) wCond -= dq; else wEvap += dq; if (evap > 0) wRain += evap; }
      double share = z < (int)surfaceShare.size() ? surfaceShare[z] : 0;
      if (sw.surfaceOn && share > 0) {
        double per = 1 * share * dt / rhoZ;
        double heat = sw.sensible * per / (CP * ex), vapour = sw.latent * per / LV;
        theta[i] += heat; q[i] += vapour; wSurf += vapour;
      }
      cold[i] = (double)cold[i] < 1e-3 ? 0 : jmin(cold[i], 15);
      if (alt > sw.spongeStart) {
        double s = clamp((alt - sw.spongeStart) / (H - sw.spongeStart)) * sw.spongeRate * dt;
        w[i] *= 1 - s; u[i] = lerp(u[i], ue, s); v[i] = lerp(v[i], ve, s); theta[i] = lerp(theta[i], thEnv, s);
      }
    }
    Arr<S> cnd = A(condensate);
    if (sw.ice) for (int i = z * layer, e = i + layer; i < e; i++) cnd[i] = (double)cloud[i] + (double)ice[i];
    Arr<S> lw = A(levelWater); int l4 = z * 4;
    lw[l4] = wCond * nodeMass; lw[l4 + 1] = wEvap * nodeMass; lw[l4 + 2] = wRain * nodeMass; lw[l4 + 3] = wSurf * nodeMass;
    A(levelCharge)[z] = wCharge * nodeMass;
  }
  void physicsStep(double dt) {  // :1116-1127
    std::vector<Carried> c = carried();
    run((int)c.size(), [&](int k, int) {
      const Carried& cc = c[k]; Arr<S> a = F(cc.k);
      taskNegative[k] = cc.conserve ? fillNegative(a) : 0;
      if (cc.decay != 1) { double keep = std::pow(cc.decay, dt); for (int i = 0; i < g.n; i++) a[i] *= keep; }
    });
    for (size_t k = 0; k < c.size(); k++) if (c[k].conserve) negativeFilled += taskNegative[k];
    run(g.nz, [&](int z, int) { physics(z, dt); });
    for (int k = 0; k < g.nz * 4; k += 4) { water[0] += (double)levelWater[k]; water[1] += (double)levelWater[k + 1]; water[2] += (double)levelWater[k + 2]; water[3] += (double)levelWater[k + 3]; }
    for (int z = 0; z < g.nz; z++) chargeSeparated += (double)levelCharge[z];  // :1126
  }
  void mixStep(double dt) {  // :1161-1195 (flat ground)
    int nz = g.nz, layer = g.layer;
    Arr<S> u = F(F_U), v = F(F_V), w = F(F_W);
    Arr<S> moistCond = sw.ice ? A(condensate) : F(F_CLOUD);
    run(nz, [&](int k, int) { turb.viscosity<S>(u, v, w, F(F_THETA), thetaEnv.data(), sw.cs, dt, F(F_Q), moistCond, exner.data(), k, k + 1); });
    struct Mixed { int k; const double* base; double factor; };
    std::vector<Mixed> mixed = {{F_U, uEnv.data(), 1}, {F_V, vEnv.data(), 1}, {F_W, nullptr, 1}, {F_THETA, thetaEnv.data(), 3}, {F_Q, qEnv.data(), 3}, {F_CLOUD, nullptr, 3}};
    if (sw.ice) { mixed.push_back({F_ICE, nullptr, 3}); mixed.push_back({F_ICENUMBER, nullptr, 3}); }
    run((int)mixed.size(), [&](int k, int t) { turb.mix<S>(F(mixed[k].k), mixed[k].base, mixed[k].factor, dt, mixTmp[t]); });
    double cd = sw.dragCd * dt, drag = cd / g.hz[0], ue0 = uGround[0], ve0 = vGround[0], envSpeed = std::hypot(ue0, ve0), fu = sw.frameU, fv = sw.frameV;
    for (int b = 0; b < layer; b++) {
      double ug = (double)u[b] + fu, vg = (double)v[b] + fv, speed = std::hypot(ug, vg);
      u[b] -= drag * (speed * ug - envSpeed * ue0); v[b] -= drag * (speed * vg - envSpeed * ve0);
      w[b] = 0.0; w[b + (nz - 1) * layer] = 0.0;
    }
  }
  void endStep(double dt) {
    physicsStep(dt);
    mixStep(dt);
    project(dt, true);
    if (electrified()) discharge(dt);  // afterStep (:1130-1133): the rotation tracking there changes no field
  }
  // :1537-1552: flashes where the field exceeds the breakdown threshold, then the ion conduction and the corona, then
  // the vertical field of the last solve for the next step's inductive charging.
  void discharge(double dt) {
    if (!lightning) lightning = std::make_unique<Lightning>(g, rho.data(), sw.lightningSeed);
    lightning->corona = sw.corona;
    Arr<S> clouds[3] = {F(F_CLOUD), F(F_ICE), F(F_SNOW)};
    lightning->cloud(clouds, 3);
    Arr<S> carriers[4] = {F(F_CHARGE_ICE), F(F_CHARGE_GRAUPEL), F(F_CHARGE_RAIN), F(F_CHARGE_AIR)};
    lastFlashes = lightning->discharge(carriers, 4, time + dt, flashLimit(dt));
    for (const Flash& f : lastFlashes) {
      if (f.cg) { chargeGround += f.charge; flashesCG++; if (f.charge < 0) chargeCgNegative += f.charge; else chargeCgPositive += f.charge; }
      else { flashesIC++; chargeIC += std::fabs(f.charge); }
    }
    double conducted = lightning->conduct(F(F_CHARGE_AIR), dt);
    chargeGround += conducted; chargeConduction += conducted;
    int nz = g.nz, layer = g.layer; Arr<S> ez = A(fieldZ); const double* phi = lightning->phi.data();
    for (int z = 1; z < nz - 1; z++) {
      double h = g.zs[z + 1] - g.zs[z - 1];
      for (int c = 0, i = z * layer; c < layer; c++, i++) ez[i] = -(phi[i + layer] - phi[i - layer]) / h;
    }
  }
  // Total charge, C (:1555-1560): the four carriers summed with each node's air mass.
  double totalCharge() {
    int nz = g.nz, layer = g.layer; double total = 0;
    Arr<S> a = F(F_CHARGE_ICE), b = F(F_CHARGE_GRAUPEL), c = F(F_CHARGE_RAIN), d = F(F_CHARGE_AIR);
    for (int z = 0, i = 0; z < nz; z++) {
      double s = 0;
      for (int e = i + layer; i < e; i++) s += (double)a[i] + (double)b[i] + (double)c[i] + (double)d[i];
      total += s * rho[z] * g.dx * g.dy * g.hz[z];
    }
    return total;
  }
  void step(double dt) { beginStep(dt); dynamics(dt); endStep(dt); }
};

}  // namespace orc
