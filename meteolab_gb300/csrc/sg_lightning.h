// Lightning of an electrified run (sg_lightning.cu): its device buffers, the small state record a flash's stages
// share, and the host side that steps through the stages.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>
#include "sg_common.cuh"
#include "sg_elec_solve.cuh"
#include "stormgpu.h"

namespace sg {

constexpr int MAX_CHANNEL = 3000, STROKES = 4, MAX_FLASHES = 10;  // src/core/lightning.ts:31, :36, :43
inline int flash_limit(double dt) {                               // flashLimit (:45): 10 per 3 s of model time, at least 1
  const double v = std::floor(MAX_FLASHES * dt / 3 + .5);
  return v < 1 ? 1 : (int)v;
}

// Per-level FP64 tables of the lightning (each the reference's expression): the breakdown field and its square, the air
// density, the height, a channel node's capacitance, the cell's volume and air mass and its inverse, the clear air's
// conductivity, the level spacing, the centred span zs[z+1] - zs[z-1], and the conduction's face factors for dt.
enum LgtTable { LT_EINIT, LT_EINIT2, LT_AIR, LT_ZS, LT_CAP, LT_VOLUME, LT_NODEAIR, LT_PERKG, LT_SIGMA, LT_DZS, LT_SPAN, LT_HZ,
                LT_ACROSS, LT_ALONG, LT_UP, LT_COUNT };

// The state a flash's kernels share (device memory; read by the host after each stage).
struct LgtState {
  unsigned long long maxBits;  // the largest |E|^2 / Einit^2 of the breakdown search, as bits
  int best;                    // its node
  int id, start, size, nnodes, npol, ground, touched, left, event, grown, strokes, nstrokes, needPotential;
  uint32_t rng;
  double sum, potential, before, moment, fromGround, conducted, lowered, neutralized, stage, charge;
  double strokeQ[STROKES];
};

struct LgtDev {
  int nz = 0;
  double dx = 0, dy = 0;
  LgtState* st = nullptr;
  double *rho = nullptr, *phi = nullptr, *sigma = nullptr, *weight = nullptr, *scale = nullptr, *dep = nullptr, *lv = nullptr, *part = nullptr;
  float* cloudy = nullptr;
  int *mark = nullptr, *seen = nullptr, *link = nullptr, *failed = nullptr, *frontier = nullptr, *nodes = nullptr, *parent = nullptr, *polarity = nullptr;
  ElecSolve es;
};

// One flash (the reference's Flash record, src/core/lightning.ts:69-106, without the drawing and the TLE).
struct FlashRecord {
  double time = 0, potential = 0, charge = 0, moment = 0;
  bool cg = false;
  int start = -1, ground = -1;
  std::vector<int> nodes, parent, polarity;
  std::vector<double> strokes;
};

struct LgtHost {
  LgtDev dev;
  int flashId = 0;
  uint32_t seed = 0;     // config.seed + 1 (src/core/model.ts:1538)
  bool corona = true;    // over land (:1539)
  double dxy = 0, conductDt = 0;
  std::vector<double> tables;
  std::vector<FlashRecord> last;   // the flashes of the last discharge
  cudaStream_t st = nullptr;       // the run's lightning stream
  LgtState* hs = nullptr;          // pinned: the state record read each round
  int* hchan = nullptr;            // pinned: a finished flash's channel (nodes, parents, polarities)
  LgtHost() = default;
  LgtHost(const LgtHost&) = delete;
  LgtHost& operator=(const LgtHost&) = delete;
  ~LgtHost();
};

// One run's discharge as the batch driver steps it.
struct LgtJob {
  const sg_grid* g = nullptr;
  RunDesc R{};
  LgtHost* H = nullptr;
  double time = 0, dt = 0;
  int limit = 0, k = 0, stamp = 0, stage = 0, start = -1, id = 0, copied = 0;
  bool pending = false;            // a flash ended in the previous discharge round; its record is read in this one
  enum Phase { SEARCH, FLASH, FINISHING, DONE } phase = SEARCH;
};

size_t lightning_bytes(int nx, int ny, int nz);
void lightning_bind(char* base, int nx, int ny, int nz, LgtDev& L);
int lightning_init(cudaStream_t st, const sg_grid* g, const double* rho, LgtHost& H);
// The run's lightning stream and pinned host buffers (once).
int lightning_host_buffers(LgtHost& H);
// The discharges of n runs together (lockstep rounds, a stream a run); each job's time is its flashes' model time.
int lightning_discharge_many(LgtJob* jobs, int n, std::string* err);
// The discharge after a step at model time `time` (the step's end) with step length dt: at most `limit` flashes, then
// the conduction and corona over dt, then the vertical field. SG_OK, or SG_ERR_DEVICE with *err set.
int lightning_discharge(cudaStream_t st, const sg_grid* g, const RunDesc& R, LgtHost& H, double time, double dt, int limit, std::string* err);
// The discharge's first search alone (no flash): the charge density, its potential, the strongest field's node and
// |E| / Einit there (-1 and 0 when there is no field) -- the diagnostics of sg_debug_lightning.
int lightning_probe(cudaStream_t st, const RunDesc& R, LgtHost& H, double* phi, double* rho, int* best, double* ratio);
// The last flash's state record: id, start, front size, nodes, ground, event, left, strokes, grown, potential, sum,
// neutralized, lowered, the last stage's charge, the flash's charge, the flash counter.
int lightning_state(cudaStream_t st, LgtHost& H, double* out16);

}  // namespace sg
