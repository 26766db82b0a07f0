// sg_divergence_max_static: the dual-cell divergence check of sg_run_divergence for velocity fields the caller
// already holds in device memory, without allocating anything.
//
// The scratch it needs (the FP64 maximum the blocks combine into) is a file-scope static device array; host code
// learns its device address once per device with cudaGetSymbolAddress. The per-level density and spacing travel as
// kernel parameters. The call makes no cudaMalloc, cudaFree or other allocating call. It is for callers that cannot
// allocate device memory at that point: a process whose HBM is fully committed (the serving loop's budget admits
// runs up to the last byte), or one whose device memory belongs to another allocator (a framework's caching
// allocator that must own every allocation), and that still want to check the projection on their own buffers.
//
// Where the array and the kernel's code come from: they are part of this translation unit's module, which the CUDA
// runtime loads into the device's context. Under lazy module loading (the default) that happens at the first use of
// the module, so sg_context_create resolves the address and loads the kernel for its device (sg::static_prepare).
// A caller that never creates a context gets the load at its first call on a device: that first call can then
// need a little device memory for the module (the code and the 256-byte array), so make it before HBM is fully
// committed, or set CUDA_MODULE_LOADING=EAGER so every module loads with the context.
//
// Limits: nz <= SG_STATIC_MAX_NZ (the level table in the parameters); larger grids are rejected with an error message.
// One scratch per device and process: calls that overlap on the same device (two host threads, or two streams in
// flight) race on it. The calling thread's current device is restored before the call returns. A NaN or an infinity
// in the velocities gives a non-finite maximum and SG_ERR_NONFINITE.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <mutex>
#include "../../include/stormgpu.h"

namespace {

constexpr int MAX_NZ = SG_STATIC_MAX_NZ;
constexpr int MAX_DEVICES = 64;

// [0]: the maximum |D rho u| as the bits of a non-negative double (starts at zero for every call; a NaN, its sign
// cleared, orders above +inf and so survives the maximum); the rest is reserved padding, 256 bytes in all.
__device__ __align__(256) unsigned long long g_scratch[32];

// The larger of m and a where a NaN wins (fmax drops a NaN and would report a finite maximum for broken fields).
__device__ __forceinline__ double nan_max(double m, double a) { return (a > m || a != a) ? a : m; }

struct Levels {
  float rho_quarter[MAX_NZ];  // rho0 / 4, rounded to FP32 as the device step's level table holds it
  float dzs[MAX_NZ];          // node spacing to the level above (nz - 1 of them), FP32
};

// The same arithmetic, in the same order, as the device step's k_divergence_max (FP64 from the FP32 fields and the
// FP32 level values), over all dual cells with a grid-stride loop.
__global__ void k_divergence_max_static(const float* __restrict__ u, const float* __restrict__ v, const float* __restrict__ w,
                                        int nx, int ny, int nz, float dx, float dy, Levels lv, unsigned long long* out) {
  const int layer = nx * ny;
  const long long ncells = (long long)layer * (nz - 1);
  double m = 0;
  for (long long cidx = (long long)blockIdx.x * blockDim.x + threadIdx.x; cidx < ncells; cidx += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(cidx / layer), c = (int)(cidx - (long long)k * layer), y = c / nx, x = c - y * nx;
    const long long l0 = (long long)k * layer;
    const int x1 = x + 1 == nx ? 0 : x + 1, y1 = y + 1 == ny ? 0 : y + 1;
    const long long a = x + y * nx + l0, b = x1 + y * nx + l0, ee = x + y1 * nx + l0, f = x1 + y1 * nx + l0;
    const long long g = a + layer, h = b + layer, s = ee + layer, tt = f + layer;
    const double r0 = lv.rho_quarter[k], r1 = lv.rho_quarter[k + 1];
    const double ddx = (r0 * ((double)u[b] + u[f] - u[a] - u[ee]) + r1 * ((double)u[h] + u[tt] - u[g] - u[s])) / dx;
    const double ddy = (r0 * ((double)v[ee] + v[f] - v[a] - v[b]) + r1 * ((double)v[s] + v[tt] - v[g] - v[h])) / dy;
    const double ddz = (r1 * ((double)w[g] + w[h] + w[s] + w[tt]) - r0 * ((double)w[a] + w[b] + w[ee] + w[f])) / lv.dzs[k];
    m = nan_max(m, fabs(ddx + ddy + ddz));
  }
  for (int o = 16; o > 0; o >>= 1) m = nan_max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m) & 0x7fffffffffffffffull);
}

unsigned long long* g_addr[MAX_DEVICES];  // the scratch's device address, per device (resolved once)
int g_sms[MAX_DEVICES];
std::mutex g_mutex;

int fail(char* err, size_t len, int code, const char* msg) {
  if (err && len) snprintf(err, len, "%s", msg);
  return code;
}

// With `device` current: the scratch's address and the SM count, resolved once per device. The symbol lookup and the
// attribute query of the kernel load this module's code and array into the context if lazy loading has not yet.
cudaError_t resolve(int device, unsigned long long** addr, int* sms) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return e;
    cudaFuncAttributes attr;
    if ((e = cudaFuncGetAttributes(&attr, k_divergence_max_static)) != cudaSuccess) return e;
    int count = 0;
    if ((e = cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) return e;
    g_sms[device] = count;
    g_addr[device] = static_cast<unsigned long long*>(p);
  }
  *addr = g_addr[device];
  *sms = g_sms[device];
  return cudaSuccess;
}

// Puts the calling thread's current device back when the entry point returns, on every path.
struct DeviceGuard {
  int saved = -1;
  ~DeviceGuard() { if (saved >= 0) cudaSetDevice(saved); }
};

}  // namespace

namespace sg {
// Called by sg_context_create with `device` current: loads the module and resolves the scratch while the context is
// made, so later calls of the entry point need no module load.
int static_prepare(int device) {
  if (device < 0 || device >= MAX_DEVICES) return 0;
  unsigned long long* addr = nullptr;
  int sms = 0;
  return resolve(device, &addr, &sms) == cudaSuccess ? 0 : -1;
}
}  // namespace sg

extern "C" int sg_divergence_max_static(int device, const float* u, const float* v, const float* w, int nx, int ny, int nz,
                                        double dx, double dy, const double* rho, const double* dzs, void* stream_,
                                        double* max_abs_div, char* err, size_t err_len) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  if (!u || !v || !w || !rho || !dzs || !max_abs_div) return fail(err, err_len, SG_ERR_INVALID, "null pointer argument");
  if (nx < 1 || ny < 1 || nz < 2) return fail(err, err_len, SG_ERR_INVALID, "grid needs nx, ny >= 1 and nz >= 2");
  if (nz > MAX_NZ) {
    char msg[96];
    snprintf(msg, sizeof msg, "nz = %d is beyond the static level table (at most %d levels)", nz, MAX_NZ);
    return fail(err, err_len, SG_ERR_INVALID, msg);
  }
  if (device < 0 || device >= MAX_DEVICES) return fail(err, err_len, SG_ERR_INVALID, "device index out of range");
  DeviceGuard guard;
  cudaError_t e = cudaGetDevice(&guard.saved);
  if (e != cudaSuccess) { guard.saved = -1; return fail(err, err_len, SG_ERR_DEVICE, cudaGetErrorString(e)); }
  if (guard.saved == device) guard.saved = -1;  // nothing to put back
  else if ((e = cudaSetDevice(device)) != cudaSuccess) return fail(err, err_len, SG_ERR_DEVICE, cudaGetErrorString(e));
  if (stream) {  // a stream of another device would run the kernel there, on this device's pointers
    int sdev = -1;
    if ((e = cudaStreamGetDevice(stream, &sdev)) != cudaSuccess) return fail(err, err_len, SG_ERR_INVALID, cudaGetErrorString(e));
    if (sdev != device) return fail(err, err_len, SG_ERR_INVALID, "the stream belongs to another device");
  }
  unsigned long long* out = nullptr;
  int sms = 0;
  if ((e = resolve(device, &out, &sms)) != cudaSuccess) return fail(err, err_len, SG_ERR_DEVICE, cudaGetErrorString(e));
  Levels lv;
  for (int k = 0; k < nz; k++) lv.rho_quarter[k] = (float)rho[k] / 4.0f;
  for (int k = 0; k < nz - 1; k++) lv.dzs[k] = (float)dzs[k];
  // the maximum starts at zero (a non-negative double's bits order as unsigned integers)
  if ((e = cudaMemsetAsync(out, 0, sizeof(unsigned long long), stream)) != cudaSuccess) return fail(err, err_len, SG_ERR_DEVICE, cudaGetErrorString(e));
  const long long ncells = (long long)nx * ny * (nz - 1);
  const long long want = (ncells + 255) / 256, cap = 8LL * sms;
  const int blocks = (int)(want < cap ? want : cap);
  k_divergence_max_static<<<blocks, 256, 0, stream>>>(u, v, w, nx, ny, nz, (float)dx, (float)dy, lv, out);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(err, err_len, SG_ERR_DEVICE, cudaGetErrorString(e));
  unsigned long long bits = 0;
  if ((e = cudaMemcpyAsync(&bits, out, sizeof bits, cudaMemcpyDeviceToHost, stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(stream)) != cudaSuccess)
    return fail(err, err_len, SG_ERR_DEVICE, cudaGetErrorString(e));
  memcpy(max_abs_div, &bits, sizeof bits);
  if (!isfinite(*max_abs_div)) return fail(err, err_len, SG_ERR_NONFINITE, "the velocities hold a non-finite value");
  return SG_OK;
}
