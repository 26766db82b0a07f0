// Host-side launchers of the step's kernels (sg_kernels.cu). Each launch covers a list of work items of a batch.
#pragma once
#include <cuda_runtime.h>
#include "sg_common.cuh"

namespace sg {

// FACE: the face projection; PRES: the pressure projection of a set's velocities; GIVEN: the pressure solve of the
// right-hand side held in phi (the refinement), its result into pres2.
enum ProjMode { PROJ_FACE = 0, PROJ_PRES = 1, PROJ_GIVEN = 2 };

struct Launch {
  const RunDesc* runs;   // device array of run descriptors
  const int4* items;     // device work items (slot, a, b, c)
  int n;                 // number of items
  int cap;               // grid cap (blocks)
  cudaStream_t stream;
};

// Packed field transfer between the runs and a staging buffer (write = 1: staging -> runs); items (slot, field, chunk,
// staging offset).
void launch_pack(const Launch& L, float* staging, int write);
void launch_theta_in(const Launch& L, const float* src);
void launch_theta_out(const Launch& L, float* dst);
void launch_fall_courant(const Launch& L);
void launch_sediment(const Launch& L, int maxnz);
void launch_proj_div_xfft(const Launch& L, int mode, int set, int yc, int maxnx);
void launch_proj_modes(const Launch& L, int mode, int maxnz, int maxny, int threads, int smem_budget);
// The whole-layer path: 2-D transforms per layer, FP64 sweeps per (m, n) in global memory.
size_t layer_fft_smem(int maxnx, int maxny);
size_t layer_fft_smem_run(int nx, int ny);  // the layer transforms' shared memory for one run's grid
void launch_proj_div_fft2(const Launch& L, int mode, int set, size_t smem);
void launch_proj_sweep(const Launch& L, int mode, int maxny);
void launch_proj_ifft2(const Launch& L, int mode, size_t smem);
void launch_proj_xifft(const Launch& L, int mode, int yc, int maxnx);
void launch_face_correct(const Launch& L, int set);
// Refinement of the final projection: node pairs v = u - dt G p1 (nodes), their divergence into phi (cells), and
// the corrected velocity from pres2 (nodes).
void launch_refine_residual(const Launch& L, int set, int TX, int TY);
void launch_refine_correct(const Launch& L, int set);
void launch_pres_correct(const Launch& L, int set, int final_);
// kind: 0 WENO fields, 1 u and v, 2 w, 3 theta (the item list of that kind)
enum TKind { TK_WENO = 0, TK_DYN = 1 };
// Transport of one field kind (0: the WENO fields, 1: the dynamics u, v, w, theta'); for WENO `group` is the fields
// per item (1 or 3)
// and `minb` the blocks per SM its register budget is cut for (2 or 3).
// bulk: the bulk-copy kernels (two producer warps move each level's inputs with TMA bulk copies; only with minb 2 and
// when transport_bulk_ok holds for the plan), else the kernels whose threads copy their own plane cells; ew: those
// with two edge warps that take the tile's edge faces (minb 2, the compile-time tiles).
void launch_transport(const Launch& L, int kind, int group, int minb, int in_set, int out_set, float frac, int stage, int TX, int TY,
                      bool bulk, bool ew);
size_t transport_smem(int kind, int G, int TX, int TY);
size_t transport_smem_bulk(int kind, int G, int TX, int TY);
// Whether a tile shape can take the bulk-copy kernels on a plan whose narrowest grid is min_nx wide (all_nx4: every
// grid width a multiple of 4).
bool transport_bulk_ok(int TX, int TY, int min_nx, bool all_nx4);
void launch_fill_partial(const Launch& L, int set);
void launch_fill_final(const Launch& L);
// variant: (electrified ? 3 : 0) + moments - 1 (1 one-moment, 2 two-moment rain, 3 two-moment rain, graupel and hail)
void launch_physics(const Launch& L, int in, int mid, int variant);
void launch_sediment_2m(const Launch& L, int maxnz);
void launch_viscosity(const Launch& L, int set);
// Mixing on (run, tile of TX x TY columns, z0, z1) items.
void launch_mix(const Launch& L, int in, int TX, int TY);
size_t mix_smem(int TX, int TY);
void launch_step_end(const Launch& L);
void launch_divergence_max(const Launch& L, int set, double* out);
// Per-run diagnostics (sg_diag.cu): the rotation tracking after a step (or a refresh that keeps the held time and the
// model time) on COLS and RUNS items; a sample's domain maxima and ground columns on node items of one run.
void launch_rotation_columns(const Launch& cols, int refresh);
void launch_rotation_summary(const Launch& runs, int refresh);
void launch_diag_sample(const Launch& L);
cudaError_t set_smem_limits(int bytes);
cudaError_t upload_tables();
// With `device` current: loads the module of sg_divergence_max_static and resolves its static scratch (sg_static.cu).
int static_prepare(int device);
cudaError_t set_transport_smem_limits(int bytes);  // (sg_transport.cu)

}  // namespace sg

// The context's device, stream and error message, for the entry points in other translation units (sg_runtime.cu).
struct sg_context;
int sg_context_device(sg_context* ctx);
cudaStream_t sg_context_stream(sg_context* ctx);
int sg_context_fail(sg_context* ctx, int code, const char* message);
