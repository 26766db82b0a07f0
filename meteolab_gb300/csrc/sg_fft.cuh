// Complex FFTs of short rows held in shared memory: the horizontal transforms of the two elliptic solves
// (lengths 40, 32, 80, 64, 320, 256 in the benchmark grids; any length whose prime factors are handled below).
// Self-sorting Stockham stages (no bit reversal): stage s with radix r reads src[j + q*n/r] and writes
// dst[(j / Ns) * Ns * r + j % Ns + q * Ns], the inputs turned by exp(-2 pi i q (j % Ns) / (Ns r)); Ns is the product
// of the radices already applied. Radix 4, 2, 3, 5 butterflies are written out; any other prime p uses a direct
// p-point sum. Twiddles exp(-2 pi i t / n) come from a per-length FP32 table computed in FP64 on the host.
#pragma once
#include "sg_common.cuh"

namespace sg {

struct FftPlan { int n, nf; const int* rad; const float2* tw; };

SG_HD float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
SG_HD float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
SG_HD float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// One butterfly group: j in [0, n/r) of one row, from x (stage input) into y (stage output).
SG_HD void fft_butterfly(const float2* x, float2* y, int n, int r, int Ns, int j, const float2* tw) {
  const int nb = n / r, k = j % Ns, t = k * (n / (Ns * r)), out = (j / Ns) * Ns * r + k;
  if (r == 4) {
    float2 v0 = x[j], v1 = cmul(x[j + nb], tw[t]), v2 = cmul(x[j + 2 * nb], tw[2 * t]), v3 = cmul(x[j + 3 * nb], tw[3 * t]);
    float2 a0 = cadd(v0, v2), a1 = csub(v0, v2), b0 = cadd(v1, v3), b1 = csub(v1, v3);
    y[out] = cadd(a0, b0);
    y[out + Ns] = make_float2(a1.x + b1.y, a1.y - b1.x);
    y[out + 2 * Ns] = csub(a0, b0);
    y[out + 3 * Ns] = make_float2(a1.x - b1.y, a1.y + b1.x);
  } else if (r == 2) {
    float2 v0 = x[j], v1 = cmul(x[j + nb], tw[t]);
    y[out] = cadd(v0, v1); y[out + Ns] = csub(v0, v1);
  } else if (r == 3) {
    const float s3 = 0.86602540378443865f;
    float2 v0 = x[j], v1 = cmul(x[j + nb], tw[t]), v2 = cmul(x[j + 2 * nb], tw[2 * t]);
    float2 s = cadd(v1, v2), d = csub(v1, v2);
    float2 m = make_float2(v0.x - .5f * s.x, v0.y - .5f * s.y);
    y[out] = cadd(v0, s);
    y[out + Ns] = make_float2(m.x + s3 * d.y, m.y - s3 * d.x);
    y[out + 2 * Ns] = make_float2(m.x - s3 * d.y, m.y + s3 * d.x);
  } else if (r == 5) {
    const float c1 = 0.30901699437494742f, s1 = 0.95105651629515357f, c2 = -0.80901699437494742f, s2 = 0.58778525229247313f;
    float2 v0 = x[j], v1 = cmul(x[j + nb], tw[t]), v2 = cmul(x[j + 2 * nb], tw[2 * t]), v3 = cmul(x[j + 3 * nb], tw[3 * t]), v4 = cmul(x[j + 4 * nb], tw[4 * t]);
    float2 t1 = cadd(v1, v4), t2 = cadd(v2, v3), d1 = csub(v1, v4), d2 = csub(v2, v3);
    float2 a = make_float2(v0.x + c1 * t1.x + c2 * t2.x, v0.y + c1 * t1.y + c2 * t2.y);
    float2 b = make_float2(v0.x + c2 * t1.x + c1 * t2.x, v0.y + c2 * t1.y + c1 * t2.y);
    float2 e = make_float2(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y);   // -i e goes to X1, +i e to X4
    float2 f = make_float2(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y);   // -i f goes to X2, +i f to X3
    y[out] = make_float2(v0.x + t1.x + t2.x, v0.y + t1.y + t2.y);
    y[out + Ns] = make_float2(a.x + e.y, a.y - e.x);
    y[out + 4 * Ns] = make_float2(a.x - e.y, a.y + e.x);
    y[out + 2 * Ns] = make_float2(b.x + f.y, b.y - f.x);
    y[out + 3 * Ns] = make_float2(b.x - f.y, b.y + f.x);
  } else {
    const int base = n / r;  // exp(-2 pi i / r) = tw[n / r]
    for (int q1 = 0; q1 < r; q1++) {
      float2 acc = make_float2(0.f, 0.f);
      for (int q = 0; q < r; q++) {
        float2 v = q ? cmul(x[j + q * nb], tw[q * t]) : x[j];
        acc = cadd(acc, cmul(v, tw[((q * q1) % r) * base]));
      }
      y[out + q1 * Ns] = acc;
    }
  }
}

// The radix sequence of a length, known at compile time (the same order as fft_plan_factors below).
constexpr int fft_count(int n) {
  int nf = 0;
  while (n % 4 == 0 && n > 1) { nf++; n /= 4; }
  while (n % 2 == 0) { nf++; n /= 2; }
  while (n % 3 == 0) { nf++; n /= 3; }
  while (n % 5 == 0) { nf++; n /= 5; }
  return n == 1 ? nf : -1;
}
constexpr int fft_radix_at(int n, int s) {
  int nf = 0;
  while (n % 4 == 0 && n > 1) { if (nf++ == s) return 4; n /= 4; }
  while (n % 2 == 0) { if (nf++ == s) return 2; n /= 2; }
  while (n % 3 == 0) { if (nf++ == s) return 3; n /= 3; }
  while (n % 5 == 0) { if (nf++ == s) return 5; n /= 5; }
  return 0;
}

#ifdef __CUDACC__
// Forward transform of `rows` rows of a compile-time length N (stride `stride`), ping-ponging between `src` and `dst`:
// every index division is by a constant. Returns the buffer that holds the result. Ends with the block synchronised.
template <int N, int S = 0, int NS = 1>
__device__ __forceinline__ float2* fft_rows_t(float2* src, float2* dst, int stride, int rows, const float2* tw) {
  if constexpr (S >= fft_count(N)) {
    return src;
  } else {
    constexpr int R = fft_radix_at(N, S), NB = N / R;
    for (int u = threadIdx.x; u < rows * NB; u += blockDim.x) {
      const int row = u / NB, j = u - row * NB;
      fft_butterfly(src + row * stride, dst + row * stride, N, R, NS, j, tw);
    }
    __syncthreads();
    return fft_rows_t<N, S + 1, NS * R>(dst, src, stride, rows, tw);
  }
}

// Forward transform (exp(-i)) of `rows` rows of length P.n, row stride `stride`, in place in `a`, with scratch `b`
// (same shape). All threads of the block take part; ends with the block synchronised.
__device__ inline void fft_rows(float2* a, float2* b, int stride, int rows, const FftPlan& P) {
  const int tid = threadIdx.x, nth = blockDim.x, n = P.n;
  float2 *src = a, *dst = b;
  int Ns = 1;
  for (int s = 0; s < P.nf; s++) {
    const int r = P.rad[s], nb = n / r, total = rows * nb;
    for (int u = tid; u < total; u += nth) {
      int row = u / nb, j = u - row * nb;
      fft_butterfly(src + row * stride, dst + row * stride, n, r, Ns, j, P.tw);
    }
    __syncthreads();
    float2* t = src; src = dst; dst = t; Ns *= r;
  }
  if (src != a) {
    for (int u = tid; u < rows * n; u += nth) { int row = u / n, i = u - row * n; a[row * stride + i] = src[row * stride + i]; }
    __syncthreads();
  }
}
// Forward transform of rows of any supported length: the compile-time path for the grid widths in use (32, 40, 64,
// 80, 128, 160, 256, 320), the runtime plan for the others. Returns the buffer that holds the result (a or b).
__device__ inline float2* fft_rows_any(float2* a, float2* b, int stride, int rows, const FftPlan& P) {
  switch (P.n) {
    case 32: return fft_rows_t<32>(a, b, stride, rows, P.tw);
    case 40: return fft_rows_t<40>(a, b, stride, rows, P.tw);
    case 64: return fft_rows_t<64>(a, b, stride, rows, P.tw);
    case 80: return fft_rows_t<80>(a, b, stride, rows, P.tw);
    case 128: return fft_rows_t<128>(a, b, stride, rows, P.tw);
    case 160: return fft_rows_t<160>(a, b, stride, rows, P.tw);
    case 256: return fft_rows_t<256>(a, b, stride, rows, P.tw);
    case 320: return fft_rows_t<320>(a, b, stride, rows, P.tw);
    default: fft_rows(a, b, stride, rows, P); return a;
  }
}
// Unnormalised inverse (exp(+i)): conj, forward, conj.
__device__ inline void ifft_rows(float2* a, float2* b, int stride, int rows, const FftPlan& P) {
  const int tid = threadIdx.x, nth = blockDim.x, n = P.n;
  for (int u = tid; u < rows * n; u += nth) { int row = u / n, i = u - row * n; a[row * stride + i].y = -a[row * stride + i].y; }
  __syncthreads();
  fft_rows(a, b, stride, rows, P);
  for (int u = tid; u < rows * n; u += nth) { int row = u / n, i = u - row * n; a[row * stride + i].y = -a[row * stride + i].y; }
  __syncthreads();
}
#endif

#ifdef __CUDACC__
// ---- Warp-level transforms (no block barrier inside): the layer transforms of the grids 40 x 32 and 80 x 64.
// A length N = 5 G row (G = 8 or 16 lanes) is one 5-point DFT in registers per lane (its elements l + G q, q = 0..4),
// a turn by exp(-2 pi i l k2 / N), then a G-point DFT across the lanes for each register k2 (the index map
// n = l + G q, k = 5 k1 + k2); a length 32 or 64 column is a 32-point DFT across the lanes (after one radix-2 stage in
// registers for 64). The lane DFTs are decimation in frequency: lane l ends with output bitrev(l).

// The forward 5-point DFT of five values (the radix-5 butterfly above without its turns).
__device__ __forceinline__ void dft5(float2& v0, float2& v1, float2& v2, float2& v3, float2& v4) {
  const float c1 = 0.30901699437494742f, s1 = 0.95105651629515357f, c2 = -0.80901699437494742f, s2 = 0.58778525229247313f;
  const float2 t1 = cadd(v1, v4), t2 = cadd(v2, v3), d1 = csub(v1, v4), d2 = csub(v2, v3);
  const float2 a = make_float2(v0.x + c1 * t1.x + c2 * t2.x, v0.y + c1 * t1.y + c2 * t2.y);
  const float2 b = make_float2(v0.x + c2 * t1.x + c1 * t2.x, v0.y + c2 * t1.y + c1 * t2.y);
  const float2 e = make_float2(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y);
  const float2 f = make_float2(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y);
  v0 = make_float2(v0.x + t1.x + t2.x, v0.y + t1.y + t2.y);
  v1 = make_float2(a.x + e.y, a.y - e.x);
  v4 = make_float2(a.x - e.y, a.y + e.x);
  v2 = make_float2(b.x + f.y, b.y - f.x);
  v3 = make_float2(b.x - f.y, b.y + f.x);
}
// G-point forward DFT across the aligned group of G lanes holding one value each (l = lane within the group), the
// twiddles exp(-2 pi i t / T) in tw with T = G * tstep. All 32 lanes of the warp take part.
template <int G>
__device__ __forceinline__ float2 lane_dft(float2 a, const float2* tw, int tstep, int l) {
#pragma unroll
  for (int h = G / 2; h >= 1; h >>= 1) {
    const float2 b = make_float2(__shfl_xor_sync(0xffffffffu, a.x, h), __shfl_xor_sync(0xffffffffu, a.y, h));
    if (l & h) a = cmul(csub(b, a), tw[(l & (h - 1)) * (G / (2 * h)) * tstep]);
    else a = cadd(a, b);
  }
  return a;
}
template <int BITS>
__device__ __forceinline__ int bitrev(int l) { return (int)(__brev((unsigned)l) >> (32 - BITS)); }
constexpr int ilog2(int v) { return v <= 1 ? 0 : 1 + ilog2(v / 2); }

// Forward transform of the length-NX rows of Z (row stride ZS) in place, by warps of the block.
template <int NX, int ZS>
__device__ __forceinline__ void warp_rows_fft(float2* Z, int rows, const float2* twx) {
  constexpr int G = NX / 5, RPW = 32 / G;
  static_assert(G * 5 == NX && (G == 8 || G == 16), "rows of 40 or 80");
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, l = lane % G, gi = lane / G, nw = blockDim.x >> 5;
  for (int rw = warp; rw * RPW < rows; rw += nw) {
    const int row = rw * RPW + gi;
    float2* Zr = Z + (row < rows ? row : rows - 1) * ZS;
    float2 v[5];
#pragma unroll
    for (int q = 0; q < 5; q++) v[q] = Zr[l + G * q];
    dft5(v[0], v[1], v[2], v[3], v[4]);
#pragma unroll
    for (int q = 1; q < 5; q++) v[q] = cmul(v[q], twx[l * q]);
#pragma unroll
    for (int q = 0; q < 5; q++) v[q] = lane_dft<G>(v[q], twx, 5, l);
    __syncwarp();
    if (row < rows) {
      const int k1 = bitrev<ilog2(G)>(l);
#pragma unroll
      for (int q = 0; q < 5; q++) Zr[5 * k1 + q] = v[q];
    }
  }
}
// Forward transform of one length-NY column held one value a lane (NY = 32) or two (NY = 64: x0 = element lane,
// x1 = element lane + 32); out[s] is the output 2 * bitrev(lane) + s (NY = 64) or bitrev(lane) (NY = 32, s = 0).
template <int NY>
__device__ __forceinline__ void warp_column_fft(float2 x0, float2 x1, const float2* twy, int lane, float2 out[2]) {
  static_assert(NY == 32 || NY == 64, "columns of 32 or 64");
  if constexpr (NY == 32) {
    out[0] = lane_dft<32>(x0, twy, 1, lane);
  } else {
    const float2 top = cadd(x0, x1), bot = cmul(csub(x0, x1), twy[lane]);
    out[0] = lane_dft<32>(top, twy, 2, lane);
    out[1] = lane_dft<32>(bot, twy, 2, lane);
  }
}
#endif

// Host reference of the same stages (used to build plans and by the CPU tests of the plan).
inline int fft_plan_factors(int n, int* rad) {
  int nf = 0, rest = n;
  while (rest % 4 == 0 && rest > 1) { rad[nf++] = 4; rest /= 4; }
  while (rest % 2 == 0) { rad[nf++] = 2; rest /= 2; }
  while (rest % 3 == 0) { rad[nf++] = 3; rest /= 3; }
  while (rest % 5 == 0) { rad[nf++] = 5; rest /= 5; }
  for (int p = 7; rest > 1; p += 2) while (rest % p == 0) { if (nf >= 8) return -1; rad[nf++] = p; rest /= p; }
  return nf <= 8 ? nf : -1;
}

}  // namespace sg
