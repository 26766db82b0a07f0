/*
 * N-API addon over the stormgpu C ABI, for the reference's Node host (its physics worker, src/simulation.worker.ts,
 * and the ensemble/series runners). Each stepping call runs on the libuv thread pool (napi_async_work) and resolves
 * a Promise, as the reference awaits GpuDynamics.step (src/gpu/step.ts:16). Build where node_api.h exists:
 *   cc -O2 -shared -fPIC -I<node>/include/node stormgpu_napi.c -L.. -lstormgpu -o stormgpu.node
 *
 * JS surface:
 *   createContext(device = 0, hbmBudget = 0) -> ctx
 *   createRun(ctx, grid, base, switches, fields) -> run      grid {nx, ny, nz, dx, dy, height, zs, dzs, hz: Float64Array}
 *                                                             base {p, exner, theta, q, u, v, rho: Float64Array}
 *                                                             switches {dt, coriolis, ...}, fields: Float32Array[13]
 *   step(ctx, runs: Int32Array, steps) -> Promise<void>
 *   readFields(ctx, run, fields: Float32Array[13]) / writeFields(ctx, run, fields)
 *   status(ctx, run) -> {steps, clipped, negativeFilled, failed}
 *   retire(ctx, run), destroyContext(ctx)
 *   saveState(ctx, run, configJson: string, time, persisted) -> ArrayBuffer      (saveState, src/core/state.ts:43)
 *   loadState(ctx, run, image: ArrayBuffer) -> {version, time, persisted}        (readState + applyState, :55-83)
 *   two-moment runs: switches.rainMoments 2 (and rainBreakup), switches.iceMoments 2 (with ice and two-moment rain):
 *   readMoments(ctx, run, fields: Float32Array[1 or 5]) / writeMoments(ctx, run, fields)   rainNumber, then graupelNumber,
 *                                                             graupelVolume, hailNumber, hailVolume (src/core/model.ts:194-202)
 *   electrified runs (switches.lightning, with ice; switches.corona, switches.lightningSeed = config.seed + 1):
 *   readCharges(ctx, run, charges: Float32Array[4]) / writeCharges(ctx, run, charges)   chargeIce, chargeGraupel,
 *                                                             chargeRain, chargeAir (src/core/model.ts:210)
 *   charge(ctx, run) -> {ground, separated, ic, cgNegative, cgPositive, precipitation, conduction, flashCount: {ic, cg}}
 *   flashes(ctx, run) -> [{time, kind: 'IC'|'CG', start, ground, potential, charge, moment, strokes: number[],
 *                          nodes, parent, polarity: Int32Array}]               (the last step's Flash records)
 *   discharge(ctx, run, time, dt)                             (AtmosphereModel.discharge, :1537-1552, on the charge
 *                                                             as it stands)
 */
#include <math.h>
#include <node_api.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "../../../include/stormgpu.h"

#define CHECK(env, call)                                                    \
  do {                                                                      \
    if ((call) != napi_ok) { napi_throw_error(env, NULL, #call); return NULL; } \
  } while (0)

static napi_value throw_status(napi_env env, sg_context* ctx, int st) {
  char msg[256];
  snprintf(msg, sizeof msg, "stormgpu error %d: %s", st, ctx ? sg_last_error(ctx) : "");
  napi_throw_error(env, NULL, msg);
  return NULL;
}

static double get_num(napi_env env, napi_value obj, const char* key) {
  napi_value v; double d = 0;
  if (napi_get_named_property(env, obj, key, &v) == napi_ok) napi_get_value_double(env, v, &d);
  return d;
}

/* A number property, or `otherwise` where the object has none (an optional setting). */
static double get_num_or(napi_env env, napi_value obj, const char* key, double otherwise) {
  napi_value v; double d;
  if (napi_get_named_property(env, obj, key, &v) != napi_ok || napi_get_value_double(env, v, &d) != napi_ok) return otherwise;
  return d;
}

static void* typed_data(napi_env env, napi_value obj, const char* key, size_t* length) {
  napi_value v; napi_typedarray_type type; size_t len; void* data; napi_value buf; size_t off;
  if (napi_get_named_property(env, obj, key, &v) != napi_ok) return NULL;
  if (napi_get_typedarray_info(env, v, &type, &len, &data, &buf, &off) != napi_ok) return NULL;
  if (length) *length = len;
  return data;
}

static napi_value create_context(napi_env env, napi_callback_info info) {
  size_t argc = 2; napi_value argv[2]; int32_t device = 0; double budget = 0;
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  if (argc > 0) napi_get_value_int32(env, argv[0], &device);
  if (argc > 1) napi_get_value_double(env, argv[1], &budget);
  sg_context* ctx = NULL;
  int st = sg_context_create(device, (uint64_t)budget, &ctx);
  if (st) return throw_status(env, NULL, st);
  napi_value ext;
  CHECK(env, napi_create_external(env, ctx, NULL, NULL, &ext));
  return ext;
}

static sg_context* ctx_of(napi_env env, napi_value v) { void* p = NULL; napi_get_value_external(env, v, &p); return (sg_context*)p; }

static int fields_of(napi_env env, napi_value arr, float** out) {
  for (uint32_t k = 0; k < SG_NFIELDS; k++) {
    napi_value el; napi_typedarray_type type; size_t len; void* data; napi_value buf; size_t off;
    if (napi_get_element(env, arr, k, &el) != napi_ok) return 0;
    if (napi_get_typedarray_info(env, el, &type, &len, &data, &buf, &off) != napi_ok || type != napi_float32_array) return 0;
    out[k] = (float*)data;
  }
  return 1;
}

static napi_value create_run(napi_env env, napi_callback_info info) {
  size_t argc = 5; napi_value argv[5];
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  sg_context* ctx = ctx_of(env, argv[0]);
  sg_grid g; memset(&g, 0, sizeof g);
  g.nx = (int32_t)get_num(env, argv[1], "nx"); g.ny = (int32_t)get_num(env, argv[1], "ny"); g.nz = (int32_t)get_num(env, argv[1], "nz");
  g.dx = get_num(env, argv[1], "dx"); g.dy = get_num(env, argv[1], "dy"); g.height = get_num(env, argv[1], "height");
  g.zs = typed_data(env, argv[1], "zs", NULL); g.dzs = typed_data(env, argv[1], "dzs", NULL); g.hz = typed_data(env, argv[1], "hz", NULL);
  sg_base_state b = {typed_data(env, argv[2], "p", NULL), typed_data(env, argv[2], "exner", NULL), typed_data(env, argv[2], "theta", NULL),
                     typed_data(env, argv[2], "q", NULL), typed_data(env, argv[2], "u", NULL), typed_data(env, argv[2], "v", NULL),
                     typed_data(env, argv[2], "rho", NULL)};
  sg_switches s; memset(&s, 0, sizeof s);
  s.dt = get_num(env, argv[3], "dt"); s.coriolis = get_num(env, argv[3], "coriolis"); s.wind_relaxation = get_num(env, argv[3], "windRelaxation");
  s.sponge_rate = get_num(env, argv[3], "spongeRate"); s.sponge_start = get_num(env, argv[3], "spongeStart"); s.cs = get_num(env, argv[3], "cs");
  s.drag_cd = get_num(env, argv[3], "dragCd"); s.frame_u = get_num(env, argv[3], "frameU"); s.frame_v = get_num(env, argv[3], "frameV");
  s.loading = (int32_t)get_num(env, argv[3], "loading"); s.evaporation = (int32_t)get_num(env, argv[3], "evaporation");
  s.rain_formation = (int32_t)get_num(env, argv[3], "rainFormation"); s.anisotropic = (int32_t)get_num(env, argv[3], "anisotropic");
  s.vertical_dz = (int32_t)get_num(env, argv[3], "verticalDz"); s.durran_klemp = (int32_t)get_num(env, argv[3], "durranKlemp");
  s.pressure_in_stages = (int32_t)get_num(env, argv[3], "pressureInStages"); s.ice = (int32_t)get_num(env, argv[3], "ice");
  s.refine_projection = (int32_t)get_num(env, argv[3], "refineProjection");
  s.rotation = (int32_t)get_num(env, argv[3], "rotation");
  s.lightning = (int32_t)get_num(env, argv[3], "lightning"); s.corona = (int32_t)get_num(env, argv[3], "corona");
  s.lightning_seed = (int32_t)get_num(env, argv[3], "lightningSeed");
  /* the model's moments (AtmosphereModel.rainMoments / iceMoments, rainBreakup 0 none, 1 NSSL, 2 Morrison; 1, 1, 0 when
   * not given) */
  s.rain_moments = (int32_t)get_num_or(env, argv[3], "rainMoments", 1); s.ice_moments = (int32_t)get_num_or(env, argv[3], "iceMoments", 1);
  s.rain_breakup = (int32_t)get_num_or(env, argv[3], "rainBreakup", 0);
  float* init[SG_NFIELDS];
  if (!fields_of(env, argv[4], init)) { napi_throw_type_error(env, NULL, "fields: 13 Float32Array"); return NULL; }
  sg_run run;
  int st = sg_run_create(ctx, &g, &b, &s, (const float* const*)init, &run);
  if (st) return throw_status(env, ctx, st);
  napi_value out;
  CHECK(env, napi_create_int32(env, run, &out));
  return out;
}

/* host: the packed buffer of stepIo (NULL for step), held by `keep` while the work runs. */
typedef struct { sg_context* ctx; sg_run* runs; int n, steps, groups, status; float* host; napi_ref keep; napi_deferred deferred; napi_async_work work; } StepJob;

static void step_execute(napi_env env, void* data) {
  StepJob* j = (StepJob*)data;
  j->status = j->host ? sg_batch_step_io(j->ctx, j->runs, j->n, SG_ALL_FIELDS, j->host, j->steps, j->groups)
                      : sg_batch_step(j->ctx, j->runs, j->n, j->steps);
}
static void step_complete(napi_env env, napi_status status, void* data) {
  StepJob* j = (StepJob*)data;
  if (j->status == SG_OK) { napi_value u; napi_get_undefined(env, &u); napi_resolve_deferred(env, j->deferred, u); }
  else {
    napi_value msg, err; char text[256];
    snprintf(text, sizeof text, "stormgpu error %d: %s", j->status, sg_last_error(j->ctx));
    napi_create_string_utf8(env, text, NAPI_AUTO_LENGTH, &msg); napi_create_error(env, NULL, msg, &err);
    napi_reject_deferred(env, j->deferred, err);
  }
  napi_delete_async_work(env, j->work);
  if (j->keep) napi_delete_reference(env, j->keep);
  free(j->runs); free(j);
}

static napi_value step(napi_env env, napi_callback_info info) {
  size_t argc = 3; napi_value argv[3];
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  StepJob* j = (StepJob*)calloc(1, sizeof(StepJob));
  j->ctx = ctx_of(env, argv[0]);
  napi_typedarray_type type; size_t len; void* data; napi_value buf; size_t off;
  if (napi_get_typedarray_info(env, argv[1], &type, &len, &data, &buf, &off) != napi_ok || type != napi_int32_array) {
    free(j); napi_throw_type_error(env, NULL, "runs: Int32Array"); return NULL;
  }
  j->n = (int)len; j->runs = (sg_run*)malloc(len * sizeof(sg_run)); memcpy(j->runs, data, len * sizeof(sg_run));
  napi_get_value_int32(env, argv[2], &j->steps);
  napi_value promise, name;
  CHECK(env, napi_create_promise(env, &j->deferred, &promise));
  CHECK(env, napi_create_string_utf8(env, "stormgpu.step", NAPI_AUTO_LENGTH, &name));
  CHECK(env, napi_create_async_work(env, NULL, name, step_execute, step_complete, j, &j->work));
  CHECK(env, napi_queue_async_work(env, j->work));
  return promise;
}

/* stepIo(ctx, runs: Int32Array, packed: Float32Array, steps, groups) -> Promise: every run's fields written from
 * `packed` (run after run, the 13 fields in sg_field order), `steps` steps, the fields read back into `packed`
 * (sg_batch_step_io) -- the per-step round trip of GpuDynamics.step (src/gpu/dynamics.ts:446-450, :488-497) for a
 * whole batch, its copies overlapping the steps of the other groups. */
static napi_value step_io(napi_env env, napi_callback_info info) {
  size_t argc = 5; napi_value argv[5];
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  StepJob* j = (StepJob*)calloc(1, sizeof(StepJob));
  j->ctx = ctx_of(env, argv[0]);
  napi_typedarray_type type; size_t len; void* data; napi_value buf; size_t off;
  if (napi_get_typedarray_info(env, argv[1], &type, &len, &data, &buf, &off) != napi_ok || type != napi_int32_array) {
    free(j); napi_throw_type_error(env, NULL, "runs: Int32Array"); return NULL;
  }
  j->n = (int)len; j->runs = (sg_run*)malloc(len * sizeof(sg_run)); memcpy(j->runs, data, len * sizeof(sg_run));
  if (napi_get_typedarray_info(env, argv[2], &type, &len, &data, &buf, &off) != napi_ok || type != napi_float32_array) {
    free(j->runs); free(j); napi_throw_type_error(env, NULL, "packed: Float32Array"); return NULL;
  }
  j->host = (float*)data;
  napi_get_value_int32(env, argv[3], &j->steps);
  napi_get_value_int32(env, argv[4], &j->groups);
  CHECK(env, napi_create_reference(env, argv[2], 1, &j->keep));
  napi_value promise, name;
  CHECK(env, napi_create_promise(env, &j->deferred, &promise));
  CHECK(env, napi_create_string_utf8(env, "stormgpu.stepIo", NAPI_AUTO_LENGTH, &name));
  CHECK(env, napi_create_async_work(env, NULL, name, step_execute, step_complete, j, &j->work));
  CHECK(env, napi_queue_async_work(env, j->work));
  return promise;
}

/* electricCreate(ctx, grid) -> solver: `new ElectricSolver(grid)` (src/core/electric.ts:24) on the device. */
static napi_value electric_create(napi_env env, napi_callback_info info) {
  size_t argc = 2; napi_value argv[2];
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  sg_context* ctx = ctx_of(env, argv[0]);
  sg_grid g; memset(&g, 0, sizeof g);
  g.nx = (int32_t)get_num(env, argv[1], "nx"); g.ny = (int32_t)get_num(env, argv[1], "ny"); g.nz = (int32_t)get_num(env, argv[1], "nz");
  g.dx = get_num(env, argv[1], "dx"); g.dy = get_num(env, argv[1], "dy"); g.height = get_num(env, argv[1], "height");
  g.zs = typed_data(env, argv[1], "zs", NULL); g.dzs = typed_data(env, argv[1], "dzs", NULL); g.hz = typed_data(env, argv[1], "hz", NULL);
  sg_electric* solver = NULL;
  int st = sg_electric_create(ctx, &g, &solver);
  if (st) return throw_status(env, ctx, st);
  napi_value ext;
  CHECK(env, napi_create_external(env, solver, NULL, NULL, &ext));
  return ext;
}

/* electricSolve(ctx, solver, rho: Float64Array, phi: Float64Array): ElectricSolver.solve(rho, phi) (:33-60), synchronous
 * (a solve is a fraction of a millisecond), as the reference's Lightning calls it for each flash. */
static napi_value electric_solve(napi_env env, napi_callback_info info) {
  size_t argc = 4; napi_value argv[4];
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  sg_context* ctx = ctx_of(env, argv[0]);
  void* solver = NULL; napi_get_value_external(env, argv[1], &solver);
  napi_typedarray_type type; size_t len; void* rho; void* phi; napi_value buf; size_t off;
  if (napi_get_typedarray_info(env, argv[2], &type, &len, &rho, &buf, &off) != napi_ok || type != napi_float64_array ||
      napi_get_typedarray_info(env, argv[3], &type, &len, &phi, &buf, &off) != napi_ok || type != napi_float64_array) {
    napi_throw_type_error(env, NULL, "rho, phi: Float64Array"); return NULL;
  }
  int st = sg_electric_solve((sg_electric*)solver, (const double*)rho, (double*)phi);
  if (st) return throw_status(env, ctx, st);
  return NULL;
}

static napi_value electric_destroy(napi_env env, napi_callback_info info) {
  size_t argc = 1; napi_value argv[1];
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  void* solver = NULL; napi_get_value_external(env, argv[0], &solver);
  sg_electric_destroy((sg_electric*)solver);
  return NULL;
}

static void read_grid(napi_env env, napi_value obj, sg_grid* g) {
  memset(g, 0, sizeof *g);
  g->nx = (int32_t)get_num(env, obj, "nx"); g->ny = (int32_t)get_num(env, obj, "ny"); g->nz = (int32_t)get_num(env, obj, "nz");
  g->dx = get_num(env, obj, "dx"); g->dy = get_num(env, obj, "dy"); g->height = get_num(env, obj, "height");
  g->zs = typed_data(env, obj, "zs", NULL); g->dzs = typed_data(env, obj, "dzs", NULL); g->hz = typed_data(env, obj, "hz", NULL);
}

/* terrainHeights(grid, form) -> Float32Array: terrainHeights(form, grid) (src/core/terrain.ts:37-63); form as
 * SimConfig.terrain: {kind: 'hill'|'ridge'|'plateau'|'schar', height, width, x?, y?, heading?, wavelength?}. */
static napi_value terrain_heights_js(napi_env env, napi_callback_info info) {
  size_t argc = 2; napi_value argv[2];
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  sg_grid g; read_grid(env, argv[0], &g);
  sg_terrain t; memset(&t, 0, sizeof t);
  napi_value kind; char name[16] = {0}; size_t len = 0;
  if (napi_get_named_property(env, argv[1], "kind", &kind) != napi_ok || napi_get_value_string_utf8(env, kind, name, sizeof name, &len) != napi_ok) {
    napi_throw_type_error(env, NULL, "terrain: kind"); return NULL;
  }
  t.kind = !strcmp(name, "hill") ? SG_TERRAIN_HILL : !strcmp(name, "ridge") ? SG_TERRAIN_RIDGE : !strcmp(name, "plateau") ? SG_TERRAIN_PLATEAU
         : !strcmp(name, "schar") ? SG_TERRAIN_SCHAR : -1;
  t.height = get_num(env, argv[1], "height"); t.width = get_num(env, argv[1], "width");
  t.x = get_num_or(env, argv[1], "x", NAN); t.y = get_num_or(env, argv[1], "y", NAN);
  t.heading = get_num_or(env, argv[1], "heading", NAN); t.wavelength = get_num_or(env, argv[1], "wavelength", NAN);
  const size_t columns = (size_t)(g.nx > 0 ? g.nx : 0) * (size_t)(g.ny > 0 ? g.ny : 0);
  void* data = NULL; napi_value ab, out;
  CHECK(env, napi_create_arraybuffer(env, columns * 4, &data, &ab));
  CHECK(env, napi_create_typedarray(env, napi_float32_array, columns, ab, 0, &out));
  if (sg_terrain_heights(&g, &t, (float*)data)) { napi_throw_error(env, NULL, "terrain: an invalid grid or form"); return NULL; }
  return out;
}

/* maskedCreate(ctx, grid, rho: Float64Array, ground: Float32Array, tolerance = 1e-6, maxIterations = 200) -> handle:
 * `new MaskedProjection(grid, new PressureSolver(grid, rho), ground, tolerance, maxIterations)` (terrain.ts:190). */
static napi_value masked_create(napi_env env, napi_callback_info info) {
  size_t argc = 6; napi_value argv[6];
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  if (argc < 4) { napi_throw_type_error(env, NULL, "maskedCreate(ctx, grid, rho, ground, tolerance?, maxIterations?)"); return NULL; }
  sg_context* ctx = ctx_of(env, argv[0]);
  sg_grid g; read_grid(env, argv[1], &g);
  napi_typedarray_type type; size_t len; void* rho; void* ground; napi_value buf; size_t off;
  if (napi_get_typedarray_info(env, argv[2], &type, &len, &rho, &buf, &off) != napi_ok || type != napi_float64_array ||
      napi_get_typedarray_info(env, argv[3], &type, &len, &ground, &buf, &off) != napi_ok || type != napi_float32_array) {
    napi_throw_type_error(env, NULL, "rho: Float64Array, ground: Float32Array"); return NULL;
  }
  double tolerance = 1e-6, iterations = 200;
  if (argc > 4) napi_get_value_double(env, argv[4], &tolerance);
  if (argc > 5) napi_get_value_double(env, argv[5], &iterations);
  sg_masked* m = NULL;
  int st = sg_masked_create(ctx, &g, (const double*)rho, (const float*)ground, tolerance, (int)iterations, &m);
  if (st) return throw_status(env, ctx, st);
  napi_value ext;
  CHECK(env, napi_create_external(env, m, NULL, NULL, &ext));
  return ext;
}

/* maskedProject(ctx, m, u, v, w: Float32Array, dt, pressure: Float64Array) -> {iterations, residual}:
 * MaskedProjection.project(u, v, w, dt, pressure) (terrain.ts:303-337), synchronous as the reference's. */
static napi_value masked_project(napi_env env, napi_callback_info info) {
  size_t argc = 7; napi_value argv[7];
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  if (argc < 7) { napi_throw_type_error(env, NULL, "maskedProject(ctx, m, u, v, w, dt, pressure)"); return NULL; }
  sg_context* ctx = ctx_of(env, argv[0]);
  void* m = NULL; napi_get_value_external(env, argv[1], &m);
  void* f[3]; void* p; napi_typedarray_type type; size_t len; napi_value buf; size_t off;
  for (int k = 0; k < 3; k++)
    if (napi_get_typedarray_info(env, argv[2 + k], &type, &len, &f[k], &buf, &off) != napi_ok || type != napi_float32_array) {
      napi_throw_type_error(env, NULL, "u, v, w: Float32Array"); return NULL;
    }
  if (napi_get_typedarray_info(env, argv[6], &type, &len, &p, &buf, &off) != napi_ok || type != napi_float64_array) {
    napi_throw_type_error(env, NULL, "pressure: Float64Array"); return NULL;
  }
  double dt = 0;
  napi_get_value_double(env, argv[5], &dt);
  int st = sg_masked_project((sg_masked*)m, (float*)f[0], (float*)f[1], (float*)f[2], dt, (double*)p);
  if (st) return throw_status(env, ctx, st);
  int32_t iterations = 0; double residual = 0;
  sg_masked_stats((sg_masked*)m, &iterations, &residual);
  napi_value out, a, b;
  CHECK(env, napi_create_object(env, &out));
  CHECK(env, napi_create_int32(env, iterations, &a));
  CHECK(env, napi_create_double(env, residual, &b));
  CHECK(env, napi_set_named_property(env, out, "iterations", a));
  CHECK(env, napi_set_named_property(env, out, "residual", b));
  return out;
}

static napi_value masked_destroy(napi_env env, napi_callback_info info) {
  size_t argc = 1; napi_value argv[1];
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  void* m = NULL; napi_get_value_external(env, argv[0], &m);
  sg_masked_destroy((sg_masked*)m);
  return NULL;
}

static napi_value fields_io(napi_env env, napi_callback_info info, int write) {
  size_t argc = 3; napi_value argv[3]; int32_t run;
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  sg_context* ctx = ctx_of(env, argv[0]);
  napi_get_value_int32(env, argv[1], &run);
  float* f[SG_NFIELDS];
  if (!fields_of(env, argv[2], f)) { napi_throw_type_error(env, NULL, "fields: 13 Float32Array"); return NULL; }
  int st = write ? sg_run_write_fields(ctx, run, SG_ALL_FIELDS, (const float* const*)f) : sg_run_read_fields(ctx, run, SG_ALL_FIELDS, f);
  if (st) return throw_status(env, ctx, st);
  return NULL;
}
static napi_value read_fields(napi_env env, napi_callback_info info) { return fields_io(env, info, 0); }
static napi_value write_fields(napi_env env, napi_callback_info info) { return fields_io(env, info, 1); }

/* The extra fields first .. first + count - 1 (a JS array of that many Float32Arrays; `most` of them at most, `least`
 * at least) from or into the run. */
static napi_value extras_io(napi_env env, napi_callback_info info, int write, int first, uint32_t least, uint32_t most, const char* what) {
  size_t argc = 3; napi_value argv[3]; int32_t run; uint32_t count = 0;
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  sg_context* ctx = ctx_of(env, argv[0]);
  napi_get_value_int32(env, argv[1], &run);
  if (napi_get_array_length(env, argv[2], &count) != napi_ok || count < least || count > most) { napi_throw_type_error(env, NULL, what); return NULL; }
  float* f[SG_NFIELDS_EXTRA] = {0};
  uint32_t mask = 0;
  for (uint32_t k = 0; k < count; k++) {
    napi_value el; napi_typedarray_type type; size_t len; void* data; napi_value buf; size_t off;
    if (napi_get_element(env, argv[2], k, &el) != napi_ok || napi_get_typedarray_info(env, el, &type, &len, &data, &buf, &off) != napi_ok ||
        type != napi_float32_array) { napi_throw_type_error(env, NULL, what); return NULL; }
    f[first + k] = (float*)data;
    mask |= 1u << (first + k);
  }
  int st = write ? sg_run_write_fields(ctx, run, mask, (const float* const*)f) : sg_run_read_fields(ctx, run, mask, f);
  if (st) return throw_status(env, ctx, st);
  return NULL;
}
static napi_value charges_io(napi_env env, napi_callback_info info, int write) {
  return extras_io(env, info, write, SG_CHARGE_ICE, 4, 4, "charges: 4 Float32Array");
}
static napi_value moments_io(napi_env env, napi_callback_info info, int write) {
  return extras_io(env, info, write, SG_RAIN_NUMBER, 1, 5, "moments: 1 or 5 Float32Array (rainNumber, then graupelNumber, graupelVolume, hailNumber, hailVolume)");
}
static napi_value read_moments(napi_env env, napi_callback_info info) { return moments_io(env, info, 0); }
static napi_value write_moments(napi_env env, napi_callback_info info) { return moments_io(env, info, 1); }
static napi_value read_charges(napi_env env, napi_callback_info info) { return charges_io(env, info, 0); }
static napi_value write_charges(napi_env env, napi_callback_info info) { return charges_io(env, info, 1); }

static void set_num(napi_env env, napi_value o, const char* key, double x) { napi_value v; napi_create_double(env, x, &v); napi_set_named_property(env, o, key, v); }

static napi_value charge(napi_env env, napi_callback_info info) {
  size_t argc = 2; napi_value argv[2]; int32_t run;
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  sg_context* ctx = ctx_of(env, argv[0]);
  napi_get_value_int32(env, argv[1], &run);
  sg_charge_state c;
  int st = sg_run_charge(ctx, run, &c);
  if (st) return throw_status(env, ctx, st);
  napi_value o, fc;
  CHECK(env, napi_create_object(env, &o));
  set_num(env, o, "ground", c.ground); set_num(env, o, "separated", c.separated); set_num(env, o, "ic", c.ic);
  set_num(env, o, "cgNegative", c.cg_negative); set_num(env, o, "cgPositive", c.cg_positive); set_num(env, o, "precipitation", c.precipitation);
  set_num(env, o, "conduction", c.conduction);
  CHECK(env, napi_create_object(env, &fc));
  set_num(env, fc, "ic", (double)c.flashes_ic); set_num(env, fc, "cg", (double)c.flashes_cg);
  napi_set_named_property(env, o, "flashCount", fc);
  return o;
}

static napi_value int32_array(napi_env env, const int32_t* src, int n) {
  napi_value ab, arr; void* data;
  if (napi_create_arraybuffer(env, (size_t)n * 4, &data, &ab) != napi_ok) return NULL;
  memcpy(data, src, (size_t)n * 4);
  if (napi_create_typedarray(env, napi_int32_array, (size_t)n, ab, 0, &arr) != napi_ok) return NULL;
  return arr;
}

static napi_value flashes(napi_env env, napi_callback_info info) {
  size_t argc = 2; napi_value argv[2]; int32_t run;
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  sg_context* ctx = ctx_of(env, argv[0]);
  napi_get_value_int32(env, argv[1], &run);
  int count = 0;
  int st = sg_run_flashes(ctx, run, NULL, 0, &count);
  if (st) return throw_status(env, ctx, st);
  sg_flash* recs = (sg_flash*)calloc(count > 0 ? count : 1, sizeof(sg_flash));
  int32_t* chan = (int32_t*)malloc(3 * 3000 * sizeof(int32_t));
  st = sg_run_flashes(ctx, run, recs, count, &count);
  napi_value list;
  napi_create_array_with_length(env, (size_t)count, &list);
  for (int k = 0; st == 0 && k < count; k++) {
    const sg_flash* f = &recs[k];
    st = sg_run_flash_channel(ctx, run, k, chan, chan + 3000, chan + 6000, 3000);
    if (st) break;
    napi_value o, kind, strokes, v;
    napi_create_object(env, &o);
    set_num(env, o, "time", f->time);
    napi_create_string_utf8(env, f->cg ? "CG" : "IC", NAPI_AUTO_LENGTH, &kind); napi_set_named_property(env, o, "kind", kind);
    set_num(env, o, "start", f->start); set_num(env, o, "ground", f->ground); set_num(env, o, "potential", f->potential);
    set_num(env, o, "charge", f->charge); set_num(env, o, "moment", f->moment);
    napi_create_array_with_length(env, (size_t)f->strokes, &strokes);
    for (int j = 0; j < f->strokes && j < 4; j++) { napi_create_double(env, f->stroke_charge[j], &v); napi_set_element(env, strokes, (uint32_t)j, v); }
    napi_set_named_property(env, o, "strokes", strokes);
    napi_set_named_property(env, o, "nodes", int32_array(env, chan, f->nodes));
    napi_set_named_property(env, o, "parent", int32_array(env, chan + 3000, f->nodes));
    napi_set_named_property(env, o, "polarity", int32_array(env, chan + 6000, f->nodes));
    napi_set_element(env, list, (uint32_t)k, o);
  }
  free(recs); free(chan);
  if (st) return throw_status(env, ctx, st);
  return list;
}

static napi_value discharge(napi_env env, napi_callback_info info) {
  size_t argc = 4; napi_value argv[4]; int32_t run; double time = 0, dt = 0;
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  sg_context* ctx = ctx_of(env, argv[0]);
  napi_get_value_int32(env, argv[1], &run);
  napi_get_value_double(env, argv[2], &time);
  napi_get_value_double(env, argv[3], &dt);
  int st = sg_run_discharge(ctx, run, time, dt);
  if (st) return throw_status(env, ctx, st);
  return NULL;
}

static napi_value status(napi_env env, napi_callback_info info) {
  size_t argc = 2; napi_value argv[2]; int32_t run;
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  sg_context* ctx = ctx_of(env, argv[0]);
  napi_get_value_int32(env, argv[1], &run);
  sg_run_counters c;
  int st = sg_run_status(ctx, run, &c);
  if (st && st != SG_ERR_NONFINITE) return throw_status(env, ctx, st);
  napi_value o, v;
  CHECK(env, napi_create_object(env, &o));
  napi_create_double(env, (double)c.steps, &v); napi_set_named_property(env, o, "steps", v);
  napi_create_double(env, (double)c.clipped, &v); napi_set_named_property(env, o, "clipped", v);
  napi_create_double(env, c.negative_filled, &v); napi_set_named_property(env, o, "negativeFilled", v);
  napi_get_boolean(env, c.failed != 0, &v); napi_set_named_property(env, o, "failed", v);
  return o;
}

static napi_value retire(napi_env env, napi_callback_info info) {
  size_t argc = 2; napi_value argv[2]; int32_t run;
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  sg_context* ctx = ctx_of(env, argv[0]);
  napi_get_value_int32(env, argv[1], &run);
  int st = sg_run_retire(ctx, run);
  if (st) return throw_status(env, ctx, st);
  return NULL;
}

static napi_value save_state(napi_env env, napi_callback_info info) {
  size_t argc = 5; napi_value argv[5]; int32_t run; double time = 0, persisted = 0; size_t jl = 0, size = 0;
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  sg_context* ctx = ctx_of(env, argv[0]);
  napi_get_value_int32(env, argv[1], &run);
  CHECK(env, napi_get_value_string_utf8(env, argv[2], NULL, 0, &jl));
  char* config = (char*)malloc(jl + 1);
  if (!config) { napi_throw_error(env, NULL, "out of memory"); return NULL; }
  napi_get_value_string_utf8(env, argv[2], config, jl + 1, &jl);
  if (argc > 3) napi_get_value_double(env, argv[3], &time);
  if (argc > 4) napi_get_value_double(env, argv[4], &persisted);
  int st = sg_run_save_state(ctx, run, config, time, persisted, NULL, 0, &size);
  napi_value ab; void* data = NULL;
  if (!st && napi_create_arraybuffer(env, size, &data, &ab) != napi_ok) { free(config); napi_throw_error(env, NULL, "arraybuffer"); return NULL; }
  if (!st) st = sg_run_save_state(ctx, run, config, time, persisted, (uint8_t*)data, size, &size);
  free(config);
  if (st) return throw_status(env, ctx, st);
  return ab;
}

static napi_value load_state(napi_env env, napi_callback_info info) {
  size_t argc = 3; napi_value argv[3]; int32_t run; void* data; size_t len;
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  sg_context* ctx = ctx_of(env, argv[0]);
  napi_get_value_int32(env, argv[1], &run);
  CHECK(env, napi_get_arraybuffer_info(env, argv[2], &data, &len));
  sg_state_info h;
  int st = sg_run_load_state(ctx, run, (const uint8_t*)data, len, &h);
  if (st) return throw_status(env, ctx, st);
  napi_value o, v;
  CHECK(env, napi_create_object(env, &o));
  napi_create_int32(env, h.version, &v); napi_set_named_property(env, o, "version", v);
  napi_create_double(env, h.time, &v); napi_set_named_property(env, o, "time", v);
  napi_create_double(env, h.persisted, &v); napi_set_named_property(env, o, "persisted", v);
  return o;
}

static napi_value destroy_context(napi_env env, napi_callback_info info) {
  size_t argc = 1; napi_value argv[1];
  CHECK(env, napi_get_cb_info(env, info, &argc, argv, NULL, NULL));
  sg_context_destroy(ctx_of(env, argv[0]));
  return NULL;
}

static napi_value init(napi_env env, napi_value exports) {
  napi_property_descriptor d[] = {
    {"createContext", 0, create_context, 0, 0, 0, napi_default, 0}, {"createRun", 0, create_run, 0, 0, 0, napi_default, 0},
    {"step", 0, step, 0, 0, 0, napi_default, 0}, {"readFields", 0, read_fields, 0, 0, 0, napi_default, 0},
    {"writeFields", 0, write_fields, 0, 0, 0, napi_default, 0}, {"status", 0, status, 0, 0, 0, napi_default, 0},
    {"retire", 0, retire, 0, 0, 0, napi_default, 0}, {"destroyContext", 0, destroy_context, 0, 0, 0, napi_default, 0},
    {"saveState", 0, save_state, 0, 0, 0, napi_default, 0}, {"loadState", 0, load_state, 0, 0, 0, napi_default, 0},
    {"stepIo", 0, step_io, 0, 0, 0, napi_default, 0},
    {"electricCreate", 0, electric_create, 0, 0, 0, napi_default, 0}, {"electricSolve", 0, electric_solve, 0, 0, 0, napi_default, 0},
    {"electricDestroy", 0, electric_destroy, 0, 0, 0, napi_default, 0},
    {"terrainHeights", 0, terrain_heights_js, 0, 0, 0, napi_default, 0}, {"maskedCreate", 0, masked_create, 0, 0, 0, napi_default, 0},
    {"maskedProject", 0, masked_project, 0, 0, 0, napi_default, 0}, {"maskedDestroy", 0, masked_destroy, 0, 0, 0, napi_default, 0},
    {"readCharges", 0, read_charges, 0, 0, 0, napi_default, 0}, {"writeCharges", 0, write_charges, 0, 0, 0, napi_default, 0},
    {"readMoments", 0, read_moments, 0, 0, 0, napi_default, 0}, {"writeMoments", 0, write_moments, 0, 0, 0, napi_default, 0},
    {"charge", 0, charge, 0, 0, 0, napi_default, 0}, {"flashes", 0, flashes, 0, 0, 0, napi_default, 0},
    {"discharge", 0, discharge, 0, 0, 0, napi_default, 0},
  };
  napi_define_properties(env, exports, sizeof d / sizeof d[0], d);
  return exports;
}

NAPI_MODULE(NODE_GYP_MODULE_NAME, init)
