/*
 * stormgpu — the StormLab model time step on one GB300 (sm_103a), behind a plain C ABI.
 *
 * The step replaces AtmosphereModel.step (src/core/model.ts:873-877 of Bandananor/MeteoLAB) for the reference's
 * GPU-eligible configuration (AtmosphereModel.gpuDynamics/gpuMixing, src/core/model.ts:882, :1136: WENO transport with
 * the pressure and buoyancy in the RK3 stages, flat ground, explicit Smagorinsky mixing), with the one-moment ice
 * microphysics, no lightning, single-storm surface (no sun). The whole step runs on the device; a run's state stays
 * resident in HBM between calls. Many independent runs of uneven sizes advance together in one set of launches
 * (sg_batch_step), and a serving loop admits, steps and retires runs (sg_server_*).
 *
 * Conventions: every call returns an sg_status (0 = ok); no exception crosses the ABI. Host buffers belong to the
 * caller; device state belongs to the library; handles are opaque. Fields are FP32 arrays of n = nx*ny*nz values,
 * node i = x + nx*(y + ny*z) (x fastest), as the reference's Float32Array fields. One context per host thread, or
 * serialise calls on a context.
 */
#ifndef STORMGPU_H
#define STORMGPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum sg_status {
  SG_OK = 0,
  SG_ERR_INVALID = 1,      /* a bad argument or configuration */
  SG_ERR_BUDGET = 2,       /* the run does not fit the context's HBM budget */
  SG_ERR_DEVICE = 3,       /* a CUDA error (sg_last_error says which) */
  SG_ERR_TIMEOUT = 4,      /* a bounded wait ran out */
  SG_ERR_NONFINITE = 5,    /* the run's state went non-finite; the run is marked failed */
  SG_ERR_NOT_FOUND = 6,    /* no such run */
  SG_ERR_UNSUPPORTED = 7   /* a configuration the device step does not implement */
} sg_status;

/* The carried fields in the reference's transport order (src/core/model.ts:1319-1335, ice, no lightning). */
enum sg_field {
  SG_RAIN = 0, SG_SNOW, SG_GRAUPEL, SG_HAIL, SG_U, SG_V, SG_W, SG_THETA, SG_Q, SG_CLOUD, SG_ICE, SG_ICE_NUMBER, SG_COLD,
  SG_NFIELDS
};
#define SG_ALL_FIELDS ((1u << SG_NFIELDS) - 1u)
/* An electrified run (sg_switches.lightning with ice) also carries the charge on the ice-snow, graupel-hail, rain and
 * droplet-ion carriers, C per kg of air (AtmosphereModel.chargeIce, chargeGraupel, chargeRain, chargeAir,
 * src/core/model.ts:210), fields 13-16 of sg_run_read_fields / sg_run_write_fields (host[f] by field id). */
/* A two-moment run (sg_switches.rain_moments 2) also carries the raindrops per kg of air (AtmosphereModel.rainNumber,
 * :194), field 17; with two-moment graupel and hail (sg_switches.ice_moments 2) also their particles per kg of air and
 * their particle volume, m3 per kg (graupelNumber, graupelVolume, hailNumber, hailVolume, :202), fields 18-21. */
enum sg_extra_field {
  SG_CHARGE_ICE = 13, SG_CHARGE_GRAUPEL, SG_CHARGE_RAIN, SG_CHARGE_AIR, SG_RAIN_NUMBER,
  SG_GRAUPEL_NUMBER, SG_GRAUPEL_VOLUME, SG_HAIL_NUMBER, SG_HAIL_VOLUME, SG_NFIELDS_EXTRA
};
#define SG_CHARGE_FIELDS (0xFu << SG_CHARGE_ICE)
#define SG_ICE2M_FIELDS (0xFu << SG_GRAUPEL_NUMBER)
#define SG_NFIELDS_ELECTRIFIED SG_NFIELDS_EXTRA

typedef struct sg_context sg_context;
typedef int32_t sg_run;

/* A grid as createGrid builds it (src/core/grid.ts:99-121): levels zs[nz], spacings dzs[nz-1], control volumes hz[nz]. */
typedef struct sg_grid {
  int32_t nx, ny, nz, reserved;
  double dx, dy, height;
  const double* zs;
  const double* dzs;
  const double* hz;
} sg_grid;

/* The base state per level, FP64 (Environment, src/core/environment.ts:34-37): ground-relative wind u, v. */
typedef struct sg_base_state {
  const double* p;
  const double* exner;
  const double* theta;
  const double* q;
  const double* u;
  const double* v;
  const double* rho;
} sg_base_state;

/* Scalar settings of a run (AtmosphereModel's switches, src/core/model.ts:747-844, and SimConfig). */
typedef struct sg_switches {
  double dt;               /* step length, s (DT = 3, src/core/constants.ts:6) */
  double coriolis;         /* f = 2 Omega sin(latitude), 1/s; 0 switches it off */
  double wind_relaxation;  /* 1/s (windRelaxation, 1e-4) */
  double sponge_rate;      /* 1/s (spongeRate, .06) */
  double sponge_start;     /* m: max(tropopause + 2.5 km, 14 km) */
  double cs;               /* Smagorinsky constant times the turbulence slider (SMAGORINSKY * turbulence / .55) */
  double drag_cd;          /* neutral drag coefficient of the ground node (dragCoefficient), 0 = no drag */
  double frame_u, frame_v; /* velocity of the domain over the ground, m/s */
  int32_t loading, evaporation, rain_formation, anisotropic, vertical_dz, durran_klemp, pressure_in_stages, ice;
  /* 1: the final projection is refined once (the residual divergence formed in double-FP32 and solved again), so the
   * projected velocity's divergence before its FP32 rounding is at rounding level as with the reference's FP64 solve;
   * 0: one FP32-transform solve (residual a few 1e-6 of the divergence removed). No counterpart switch in the reference. */
  int32_t refine_projection;
  /* 1: after every step the rotation tracking (updateRotation, src/core/model.ts:1609-1648, which the reference's step
   * runs in afterStep) and the run's swaths (addSwaths, src/ensemble/member.ts:71-89) on the device; read with
   * sg_run_rotation / sg_run_read_swaths. 0: neither (two launches a step fewer). */
  int32_t rotation;
  /* 1 with ice: electrification and lightning (SimConfig.lightning; electrified(), src/core/model.ts:1316): the four
   * charge carriers transported and sedimented with their carriers, the non-inductive (Takahashi) and inductive
   * charging and the charge transfer in the physics, and after every step the flashes (Lightning.discharge,
   * src/core/lightning.ts:259-275), the ion conduction and the corona. 0: none of it (the step of the configurations
   * the throughput is quoted on). */
  int32_t lightning;
  int32_t corona;          /* 1: the ground gives corona (over land; surfaceType 'water': 0, :1539) */
  int32_t lightning_seed;  /* the lightning's random numbers: config.seed + 1 (:1538) */
  /* 2: two-moment rain after NSSL (AtmosphereModel.rainMoments, :842; src/core/rain2m.ts): the drop number carried,
   * transported and falling with the rain (sedimentRain2m, :944-988), the NSSL warm-rain processes instead of Kessler's
   * and the number following the rain the ice processes take or give; 1: one-moment rain (the configured step). */
  int32_t rain_moments;
  int32_t rain_breakup;    /* two-moment rain's collisional breakup (rainBreakup, :843): 0 none, 1 NSSL's, 2 Morrison's */
  /* 2: two-moment graupel and hail after NSSL (AtmosphereModel.iceMoments, :839-840; src/core/ice2m.ts), with the ice
   * microphysics and two-moment rain only (ice2m(), :914; SimConfig.moments 2 sets both, :331): their number and
   * particle volume carried, transported and falling with the mass (sedimentIce2m, :916-921), their processes instead
   * of the one-moment graupel and hail ones, the charging by their own distributions; 1: one-moment graupel and hail. */
  int32_t ice_moments;
} sg_switches;

/* The charge budget of an electrified run since it began (AtmosphereModel.chargeGround, .charge, .flashCount,
 * src/core/model.ts:218-241), C and counts. */
typedef struct sg_charge_state {
  double ground;           /* chargeGround: what the precipitation, the flashes and the conduction gave the ground */
  double separated;        /* charge separated by the charging (both signs, |non-inductive| + |inductive|) */
  double ic;               /* neutralized by IC flashes (each sign) */
  double cg_negative, cg_positive;  /* lowered to the ground by -CG and +CG flashes */
  double precipitation;    /* carried to the ground by the falling carriers */
  double conduction;       /* lost to the ground and the top by the ion current and the corona */
  int64_t flashes_ic, flashes_cg;
  int32_t last_flashes;    /* flashes of the last step (sg_run_flashes) */
  int32_t electrified;
} sg_charge_state;

/* One flash of the last step (Flash, src/core/lightning.ts:69-106, without its drawing and transient event). */
typedef struct sg_flash {
  double time;             /* model time of the step's end, s */
  double potential;        /* the channel's potential when it stopped growing (a CG's before its ground contact), V */
  double charge;           /* IC: charge neutralized of each sign (> 0); CG: charge lowered to the ground, signed */
  double moment;           /* CG: charge moment change, C m */
  double stroke_charge[4]; /* CG: each stroke's charge (at most 4) */
  int32_t cg;              /* 1: a cloud-to-ground flash */
  int32_t start, ground;   /* initiation node; the ground contact node (-1 for IC) */
  int32_t nodes, strokes;  /* channel nodes; CG strokes */
  int32_t reserved;
} sg_flash;

/* Per-run counters (AtmosphereModel.clipped, negativeFilled, water, src/core/model.ts:236, :269-271). */
typedef struct sg_run_counters {
  int64_t steps;
  int64_t clipped;
  double negative_filled;
  double water_condensed, water_evaporated, water_rain_evaporated, water_surface;
  int32_t failed;          /* 1: the state went non-finite; 2: a bounded device wait ran out (SG_ERR_TIMEOUT); either
                            * way the run is skipped by later steps */
  int32_t reserved;
} sg_run_counters;

/* ---- context (replaces GpuDynamics.create / destroy / errors, src/gpu/dynamics.ts:250-282, :404) */
int sg_context_create(int device, uint64_t hbm_budget_bytes, sg_context** out);
int sg_context_destroy(sg_context* ctx);
const char* sg_last_error(sg_context* ctx);
/* Bytes of HBM one run of this grid takes (state, scratch, solver tables); a run with these switches (electrified:
 * its charge carriers and lightning buffers; two-moment rain: its drop number). */
uint64_t sg_run_bytes(const sg_grid* grid);
uint64_t sg_run_bytes_for(const sg_grid* grid, const sg_switches* sw);

/* ---- runs (replace `new AtmosphereModel(config, grid, profile)`, src/core/model.ts:329; fields as its arrays) */
/* init[SG_NFIELDS] host arrays in sg_field order (theta is the full potential temperature, K). */
int sg_run_create(sg_context* ctx, const sg_grid* grid, const sg_base_state* base, const sg_switches* sw,
                  const float* const* init, sg_run* out);
int sg_run_write_fields(sg_context* ctx, sg_run run, uint32_t mask, const float* const* host);
int sg_run_read_fields(sg_context* ctx, sg_run run, uint32_t mask, float* const* host);
/* The same for n runs at once (host[k * SG_NFIELDS + f] is run k's field f): all copies queued on the library's
 * stream, one synchronisation at the end, so pinned host buffers move at full link speed. The batch of an ensemble
 * runner that reads every member between samples (src/ensemble/member.ts:101-107). */
int sg_batch_write_fields(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, const float* const* host);
int sg_batch_read_fields(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, float* const* host);
/* The same with one host buffer: `host` holds, run after run in the order of `runs`, the mask's fields in sg_field
 * order, nx*ny*nz FP32 values each (theta as the full potential temperature). One host<->device copy of the whole
 * buffer through a device staging buffer the context keeps, one kernel placing or gathering the fields, one
 * synchronisation: the fastest way to move a batch's state (pinned host memory moves at link speed). */
int sg_batch_write_packed(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, const float* host);
int sg_batch_read_packed(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, float* host);
/* Steps with the state moved through host memory around them, as the reference's GPU engine moves all fields in and
 * out every step (src/gpu/dynamics.ts:446-450, :488-497; GpuDynamics.step, :404): the mask's fields of every run are
 * written from `host` (the layout of sg_batch_write_packed), the runs advance `nsteps`, and the fields are read back
 * into `host`. The runs are cut into `groups` (1..8, at most n) consecutive groups with a stream, a part of the staging
 * buffer and a CUDA graph each, so one group's host copies overlap the other groups' steps; a run's results are the
 * same as with sg_batch_write_packed, sg_batch_step and sg_batch_read_packed. Returns when every group is done. */
int sg_batch_step_io(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, float* host, int nsteps, int groups);
/* The engine's round trip every step for nsteps steps in one call: each step writes the mask's fields of every run from
 * `host`, advances one step and reads them back into `host`, so a step's inputs are the host buffer as the previous
 * step left it (GpuDynamics.step, src/gpu/dynamics.ts:446-450, :488-497, called nsteps times). The groups (as in
 * sg_batch_step_io) run as independent pipelines: one group's copies overlap the other groups' steps within and across
 * steps, and the call pays its first write and last read once instead of every step. The same bits as nsteps calls
 * of sg_batch_step_io with one step each. */
int sg_batch_step_round_trips(sg_context* ctx, const sg_run* runs, int n, uint32_t mask, float* host, int nsteps, int groups);
/* precipitation, hailGround, hailSize: nx*ny each (nullable); src/core/model.ts:253, :262. */
int sg_run_read_columns(sg_context* ctx, sg_run run, float* precipitation, float* hail_ground, float* hail_size);
/* The same columns written (each pointer nullable: that column is left as it is). */
int sg_run_write_columns(sg_context* ctx, sg_run run, const float* precipitation, const float* hail_ground, const float* hail_size);
/* The run's grid size. */
int sg_run_shape(sg_context* ctx, sg_run run, int32_t* nx, int32_t* ny, int32_t* nz);

/* ---- the storm's electric potential (ElectricSolver, src/core/electric.ts:15-60; re-solved by Lightning.discharge for
 * every flash, src/core/lightning.ts:231). Laplacian(phi) = -rho/eps0 at the nodes of `grid`, phi = 0 on the ground and
 * top levels, periodic in x and y; FP64 throughout (the reference's tests hold it to 1e-9 of the discrete equation).
 * sg_electric_create replaces `new ElectricSolver(grid)` ("the electric solver needs an interior level" for nz < 3;
 * nx, ny <= 2048); sg_electric_solve replaces `solve(rho, phi)`: rho (C/m^3) and phi (V) are host arrays of
 * nx*ny*nz doubles, node x + nx*(y + ny*z). Errors are reported on the context (sg_last_error). */
typedef struct sg_electric sg_electric;
int sg_electric_create(sg_context* ctx, const sg_grid* grid, sg_electric** out);
int sg_electric_solve(sg_electric* solver, const double* rho, double* phi);
int sg_electric_destroy(sg_electric* solver);

/* ---- terrain (src/core/terrain.ts): the ground as cut cells in the flat grid, and the projection that keeps the air
 * out of it. A form (TerrainConfig, terrain.ts:16-27): heights and widths in km, the centre in km from the domain's
 * south-west corner, the ridge's heading in degrees clockwise from north, the Schar ridges' wavelength in km; NaN for
 * an absent option (the reference's defaults: the middle, north-south, 4 km). */
enum sg_terrain_kind { SG_TERRAIN_HILL = 0, SG_TERRAIN_RIDGE = 1, SG_TERRAIN_PLATEAU = 2, SG_TERRAIN_SCHAR = 3 };
typedef struct sg_terrain {
  int32_t kind, reserved;
  double height, width, x, y, heading, wavelength;
} sg_terrain;
/* terrainHeights (terrain.ts:37-63): the ground height of every column, m, into out[nx*ny]. Host arithmetic only. */
int sg_terrain_heights(const sg_grid* grid, const sg_terrain* form, float* out);
/* The cut-cell geometry of ground heights ground[nx*ny] (m), host arithmetic only; every output nullable:
 * solidMask (:80-84) solid[n], groundLevels (:87-91) levels[nx*ny], nodeHeights (:101-105) heights[n],
 * faceApertures (:119-134) ax[n] and ay[n], slopeArea (:141-150) slope[nx*ny]. */
int sg_terrain_geometry(const sg_grid* grid, const float* ground, uint8_t* solid, int32_t* levels, double* heights, double* ax,
                        double* ay, float* slope);
/* MaskedProjection (terrain.ts:168-363) on the device: the node mass flux rho0 u made divergence-free over the dual
 * cells cut by the ground, by preconditioned conjugate gradients (the flat spectral solve as the preconditioner) to
 * `tolerance` of the first residual in at most `max_iterations`, FP64 throughout. sg_masked_create replaces
 * `new MaskedProjection(grid, new PressureSolver(grid, rho), ground, tolerance, maxIterations)` (rho: nz base-state
 * densities; ground: nx*ny heights, m); sg_masked_project replaces `project(u, v, w, dt, pressure)`: u, v, w host
 * arrays of n floats projected in place, pressure the host array of nx*ny*(nz-1) cell values, the first guess in and
 * the result out; sg_masked_mask and sg_masked_divergence replace `mask` and `divergence` (out: nx*ny*(nz-1));
 * sg_masked_stats gives `iterations` and `residual` of the last projection and sg_masked_dropped the cells without a
 * row (`dropped`, nullable outputs). */
typedef struct sg_masked sg_masked;
int sg_masked_create(sg_context* ctx, const sg_grid* grid, const double* rho, const float* ground, double tolerance, int max_iterations,
                     sg_masked** out);
int sg_masked_project(sg_masked* m, float* u, float* v, float* w, double dt, double* pressure);
int sg_masked_mask(sg_masked* m, float* u, float* v, float* w);
int sg_masked_divergence(sg_masked* m, const float* u, const float* v, const float* w, double* out);
int sg_masked_stats(sg_masked* m, int32_t* iterations, double* residual);
int sg_masked_dropped(sg_masked* m, uint8_t* dropped);
int sg_masked_destroy(sg_masked* m);
/* The transport's face fluxes with terrain (FluxTransport.setTerrain and setVelocityMasked, src/core/advection.ts:78-184)
 * on the device: the face mass fluxes of the node velocity, shut next to the ground and made divergence-free over the
 * fluid nodes with the faces' open heights, by preconditioned conjugate gradients (the flat face solve as the
 * preconditioner) to `tolerance` of the first residual in at most `max_iterations` (the reference's 1e-10 and 400), FP64.
 * sg_faces_create replaces `new FluxTransport(grid, rho)` with `setTerrain(solid, nodeHeights, faceApertures)` of the
 * ground heights (as the model sets it up, src/core/model.ts:366-377); sg_faces_set_velocity replaces
 * `setVelocityMasked(u, v, w)` and reading `mx`, `my`, `mz`, `div` (host arrays of n doubles, each nullable);
 * sg_faces_stats gives `maskedIterations` and `maskedResidual`. */
typedef struct sg_faces sg_faces;
int sg_faces_create(sg_context* ctx, const sg_grid* grid, const double* rho, const float* ground, double tolerance, int max_iterations,
                    sg_faces** out);
int sg_faces_set_velocity(sg_faces* f, const float* u, const float* v, const float* w, double* mx, double* my, double* mz, double* div);
int sg_faces_stats(sg_faces* f, int32_t* iterations, double* residual);
int sg_faces_destroy(sg_faces* f);

/* ---- per-run diagnostics (runs with switches.rotation). The rotation state after the last step (RotationState,
 * src/core/model.ts:263; the reference's field names) and the model time the device keeps for the swaths' ground shift. */
typedef struct sg_rotation {
  double uh, x, y, anticyclonic, persisted, uh01, uh03, low, core_zeta, core_uh, core_anti, time;
} sg_rotation;
/* uh_column: nx*ny floats (nullable), the 2-5 km updraught helicity of every column (model.uhColumn). */
int sg_run_rotation(sg_context* ctx, sg_run run, sg_rotation* out, float* uh_column);
/* refreshRotation (src/core/model.ts:1607): the rotation state from the fields as they are (after fields were written
 * or a state loaded), the time the rotation has held and the model time kept, the swaths untouched. */
int sg_run_refresh_rotation(sg_context* ctx, sg_run run);
/* The swaths since the run began or since the last reset (MemberResult.gustMax / uhMax, src/ensemble/member.ts:20-21):
 * per ground column the strongest surface wind (m/s) and the strongest UH 2-5 km (m2/s2); nullable outputs. */
int sg_run_read_swaths(sg_context* ctx, sg_run run, float* gust_max, float* uh_max);
int sg_run_reset_swaths(sg_context* ctx, sg_run run);
/* diagnostics() (src/core/model.ts:1672-1696) without shear06 (a property of the sounding the host has): the domain
 * maxima on the device, then on the host the cores (countCores, 4-connected) and the outflow deficit (rkw.ts:72-90) from
 * five ground columns copied once. */
typedef struct sg_diagnostics {
  double updraft, downdraft, rain_rate, rain_total, cloud_top, thermal_top, max_cloud, cold_max, cores, outflow, outflow_low, gust,
      hail, clipped;
} sg_diagnostics;
int sg_run_diagnostics(sg_context* ctx, sg_run run, sg_diagnostics* out);

/* ---- saved state (.meteolab files: saveState / readState / applyState, src/core/state.ts:43-83). The image is 'MLAB',
 * the JSON header's length (uint32 LE), the JSON header, zero padding to 4 bytes, the fields as float32 in the file's
 * STATE_FIELDS order (state.ts:9; the charge fields and two-moment moments, which the configured step does not carry,
 * are written as zeros and ignored on loading) and the ground columns (precipitation, hailGround, hailSize). */
typedef struct sg_state_info {
  int32_t version, nx, ny, nz, nfields, reserved;
  double time, persisted;
  uint64_t data_offset;
} sg_state_info;
/* readState's checks alone (no context, no device): SG_OK and the header's values, or SG_ERR_INVALID with the
 * reference's message in err ("this is not a MeteoLab state file", "the file is truncated", "the file's header is
 * damaged", "unknown file format or version", "the file's size does not match the grid"). */
int sg_state_parse(const uint8_t* image, size_t len, sg_state_info* out, char* err, size_t err_len);
/* saveState of one run (version 5): config_json is the run's SimConfig as JSON text (nullable), time the model time
 * and persisted how long the rotation has held (the host keeps both). out == NULL or cap too small: *size gets the
 * bytes needed and nothing is written (SG_OK, or SG_ERR_INVALID when cap is too small). One gather on the device and
 * one copy to the host. */
int sg_run_save_state(sg_context* ctx, sg_run run, const char* config_json, double time, double persisted, uint8_t* out,
                      size_t cap, size_t* size);
/* readState + applyState into a run of the same grid: the fields a file of its version holds (the others zero, as
 * the reference fills them) and the columns, one copy to the device and one scatter; info gets the header's values
 * (time, persisted: the host's to keep). A different grid: SG_ERR_INVALID, "the file's grid is AxBxC, the run's DxExF". */
int sg_run_load_state(sg_context* ctx, sg_run run, const uint8_t* image, size_t len, sg_state_info* info);
/* The projection pressure of the last final projection, nx*ny*(nz-1) values (AtmosphereModel.pressure, :247). */
int sg_run_read_pressure(sg_context* ctx, sg_run run, double* p);
int sg_run_status(sg_context* ctx, sg_run run, sg_run_counters* out);
int sg_run_retire(sg_context* ctx, sg_run run);

/* ---- electrification and lightning (an electrified run; replace AtmosphereModel.chargeGround / charge / flashCount /
 * flashes, src/core/model.ts:218-241, and Lightning, src/core/lightning.ts:135) */
int sg_run_charge(sg_context* ctx, sg_run run, sg_charge_state* out);
/* The flashes of the run's last step, oldest first: up to cap records, *count = how many there were. */
int sg_run_flashes(sg_context* ctx, sg_run run, sg_flash* out, int cap, int* count);
/* Flash k's channel: nodes in growth order, the index of the node each grew from (-1 for the first), the leader
 * polarity (+1, -1, 0), up to cap each (a flash has at most 3000 nodes). */
int sg_run_flash_channel(sg_context* ctx, sg_run run, int k, int32_t* nodes, int32_t* parent, int32_t* polarity, int cap);
/* The discharge of the run's charge as it stands (AtmosphereModel.discharge, src/core/model.ts:1537-1552: the flashes
 * at model time `time`, at most flashLimit(dt) of them, then the conduction and corona over dt and the vertical field),
 * without a step: the seam of a caller that orders the step itself. The run's own time is not moved. */
int sg_run_discharge(sg_context* ctx, sg_run run, double time, double dt);
/* Diagnostics (no counterpart in the reference): the discharge's first search on the run's charge as it stands --
 * the charge density (C/m3) and its potential (V), n FP64 values each (either may be null), the node of the strongest
 * field and |E| / Einit there (-1 and 0: no field); last16 (nullable): the last flash's state record before the
 * search (id, start node, front size, nodes, ground node, event, left the cloud, strokes, nodes before the last stage,
 * potential, potential sum, neutralized, lowered, last stage's charge, flash charge, flash counter). Changes no field. */
int sg_debug_lightning(sg_context* ctx, sg_run run, double* phi, double* rho, int32_t* best, double* ratio, double* last16);

/* ---- stepping (replaces AtmosphereModel.step(dt) + time += dt, src/core/model.ts:873; gpuStep, src/gpu/step.ts:12) */
int sg_run_step(sg_context* ctx, sg_run run, int nsteps);
/* All runs advance together, one set of launches per stage for the whole batch, replayed from a CUDA graph. */
int sg_batch_step(sg_context* ctx, const sg_run* runs, int n, int nsteps);
/* Enqueue without waiting; sg_synchronize waits for the context's stream. */
int sg_batch_step_async(sg_context* ctx, const sg_run* runs, int n, int nsteps);
int sg_synchronize(sg_context* ctx);

/* ---- measurement: mean device time (ms) per launch of each kernel class over `nsteps` eager steps of a batch.
 * names[k] receives a static string; returns the number of classes written (<= cap). */
int sg_profile_kernels(sg_context* ctx, const sg_run* runs, int n, int nsteps, const char** names, double* ms_per_launch,
                       int64_t* launches, int cap);
/* Advance a batch `nsteps` steps (from its CUDA graph, or eagerly) between two CUDA events on the context's stream;
 * *ms receives the device time. */
int sg_time_steps(sg_context* ctx, const sg_run* runs, int n, int nsteps, int use_graph, double* ms);
/* Max |D R u| of the run's current velocities (FP64 on the device), for the divergence check. A NaN or infinite
 * velocity gives a non-finite maximum and SG_ERR_NONFINITE. */
int sg_run_divergence(sg_context* ctx, sg_run run, double* max_abs_div);

/* ---- transport tile: the RK3 transport works on tiles of tile_x x tile_y columns, each work item carrying 1 or 3 of
 * the nine WENO fields (weno_group). By default a batch's shape is picked by timing the candidates on the batch itself
 * when its plan is first built (the autotuner; SG_AUTOTUNE=0 in the environment keeps the default 40x8 or 32x8, 3).
 * The tuner also picks the WENO kernel's register budget. sg_set_transport_shape pins one shape for every later plan
 * (tile_x = 0 returns to tuning and forgets earlier results, so the next plan of a batch is tuned on its runs as they are
 * then, e.g. developed storms after a spin-up; register budget for 2 blocks per SM); results are the same bits
 * for every shape. sg_batch_transport_shape reports the shape a batch runs with. No counterpart in the reference (its
 * CPU transport has no tiles). */
int sg_set_transport_shape(sg_context* ctx, int tile_x, int tile_y, int weno_group);
/* shape4 = (tile_x, tile_y, weno_group, blocks per SM the WENO kernel's register budget is cut for: 2 or 3). */
int sg_batch_transport_shape(sg_context* ctx, const sg_run* runs, int n, int* shape4);
/* *bulk = 1 when the batch's transport tiles get their inputs by TMA bulk copies that two producer warps issue, 0 when
 * every thread copies its own plane cells (the tuner times both; SG_TRANSPORT_BULK=0 keeps the bulk copies out). No
 * counterpart in the reference. */
int sg_batch_transport_copies(sg_context* ctx, const sg_run* runs, int n, int* bulk);

/* ---- divergence check without allocation. No counterpart in the reference (its check, PressureSolver.divergence,
 * src/core/pressure.ts:50-66, runs on its own CPU arrays).
 * Max |D rho0 u| over the dual cells of velocities the caller holds in device memory (u, v, w: nx*ny*nz FP32 nodes,
 * x fastest; rho: nz and dzs: nz-1 host FP64 values), the same FP64 arithmetic as sg_run_divergence, on `stream` (NULL: the
 * default stream; a stream of another device is refused), synchronised before it returns. The call allocates nothing:
 * its scratch is a static device array of 256 bytes, so callers that must not allocate at that point (HBM fully
 * committed, or device memory owned by another allocator) can still check a projection. The array and the kernel
 * belong to the library's module: sg_context_create loads them for its device; without a context on the device, the
 * first call loads them (under lazy module loading, the default, that takes a little device memory), so make that
 * first call before HBM is committed or set CUDA_MODULE_LOADING=EAGER, and before any stream capture. nz is at most
 * SG_STATIC_MAX_NZ; a larger grid, or a bad argument, returns SG_ERR_INVALID with the reason in err (err_len bytes,
 * nullable). A NaN or infinite velocity returns SG_ERR_NONFINITE (*max_abs_div non-finite). Calls that overlap on one
 * device race on the scratch: serialise them. The calling thread's current device is the same after the call. */
#define SG_STATIC_MAX_NZ 128
int sg_divergence_max_static(int device, const float* u, const float* v, const float* w, int nx, int ny, int nz,
                             double dx, double dy, const double* rho, const double* dzs, void* stream,
                             double* max_abs_div, char* err, size_t err_len);

/* ---- diagnostics: one part of the step (1 beginStep, 2 dynamics, 3 physicsStep, 4 mixStep, 5 final projection),
 * and the raw device buffers (set 0 = state, 1 and 2 = stage scratch; theta of a set is its departure from the base
 * profile; faces4 = (mx, my, mz, div) per node, interleaved). For stage-wise parity tests against the oracle. */
int sg_debug_step_part(sg_context* ctx, sg_run run, int part);
int sg_debug_read_set(sg_context* ctx, sg_run run, int set, int field, float* host);
int sg_debug_read_faces(sg_context* ctx, sg_run run, float* faces4);

/* ---- serving: a request loop with HBM-budget admission, device-resident runs and mid-batch retirement ---- */
typedef struct sg_server sg_server;
int sg_server_create(sg_context* ctx, int max_active, sg_server** out);
int sg_server_destroy(sg_server* srv);
/* Queue a request: the run (created by sg_run_create or queued lazily) and its number of steps. */
int sg_server_submit(sg_server* srv, const sg_grid* grid, const sg_base_state* base, const sg_switches* sw,
                     const float* const* init, int64_t steps, int64_t tag);
/* One iteration: admit what fits, advance every active run one step in one batch, retire finished runs.
 * done_tags/done_count receive the tags of runs finished in this iteration (cap entries). */
int sg_server_iterate(sg_server* srv, int64_t* done_tags, int* done_count, int cap, int* active, int* queued);
/* Steps an iteration may advance (default 1): each iteration advances every active run by min(quantum, the fewest
 * steps any active run has left), so no run overshoots and new requests join at the next iteration boundary. */
int sg_server_set_quantum(sg_server* srv, int steps);
/* Steps the last sg_server_iterate advanced. */
int sg_server_last_steps(sg_server* srv);
/* Read a finished run's fields (mask/host as sg_run_read_fields; precipitation nullable) and retire it. Finished runs
 * stay resident, and are no longer stepped, until collected. */
int sg_server_collect(sg_server* srv, int64_t tag, uint32_t mask, float* const* host, float* precipitation);

#ifdef __cplusplus
}
#endif
#endif /* STORMGPU_H */
