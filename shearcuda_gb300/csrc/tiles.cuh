// Tile shapes and shared-memory staging helpers of the 2-D row and column
// FFT kernels (k_directional.cu, k_dct.cu).
#pragma once
#include "fft_core.cuh"
#include "internal.h"

namespace nsst {

// Tile shapes: a row CTA owns RS rows, a column CTA owns CS columns, each as two
// ping-pong shared buffers [index][sequence] (dense, see block_fft_pp).  They keep a thread's share of a tile at <= 16 complex values and the
// shared memory low enough for 2-3 resident CTAs per SM: the kernels are bound
// by global-memory latency, so resident CTAs are what hides it.
template <int N>
struct RowCfg {  // N = W/2 complex points per row
  static constexpr int RS = N >= 1024 ? 4 : 8;
  // 256 = 16 x 16: a radix-16 pass has 16 butterflies per row, one per thread
  static constexpr int T = N == 256 ? 128 : 256;
  static constexpr int MINB = 1024 / T;  // <= 64 registers: at least 32 warps per SM
  static constexpr int LD = RS;
  static constexpr size_t smem() { return 2 * (size_t)N * LD * sizeof(float2); }
  // one tile staged row-major with rows padded to N + 2 (holds the dense layout too)
  static constexpr size_t smem_rm() { return (size_t)RS * (N + 2) * sizeof(float2); }
};
template <int N>
struct ColCfg {  // N = H points per column
  static constexpr int CS = N >= 768 ? 4 : 8;  // 768 x 8 float2 per plane would leave one CTA per SM
  static constexpr int T = N >= 2048 ? 512 : 256;
  static constexpr int LD = CS;
  static constexpr int MINB = 1024 / T;  // in-place column passes: 4 CTAs of 256 threads per SM
  static constexpr size_t smem() { return 2 * (size_t)N * LD * sizeof(float2); }
};

// The synthesis CTA keeps its running band sum in shared memory next to the
// transform buffer and the next band's staging buffer.
template <int N>
struct SynCfg : ColCfg<N> {
  // two column buffers (transform, running sum), the DC column and the
  // staging buffer that the next band streams into (cp.async) while the
  // current one is transformed
  static constexpr size_t smem() {
    return (2 * (size_t)N * ColCfg<N>::LD + N + (size_t)N * ColCfg<N>::CS) * sizeof(float2);
  }
  // the column kernels' thread count; shared memory allows two CTAs per SM below 2048 points
  static constexpr int T = ColCfg<N>::T;
  static constexpr int MINB = N >= 2048 ? 1 : 2;
};

// The multi-band analysis CTA keeps its column group of the level spectrum,
// a staging buffer for the next band's filter spectrum and the transform.
template <int N>
struct AnaCfg : ColCfg<N> {
  static constexpr size_t smem() { return 3 * (size_t)N * ColCfg<N>::CS * sizeof(float2); }
  // the column kernels' thread count (every thread busy in the radix-16
  // passes); shared memory allows two CTAs per SM below 2048 points.  The
  // 3 x 16 x 16 and 3 x 16 x 8 plans (768 and 384 points) have 192
  // radix-16 butterflies per column group: 192 threads, three CTAs per SM
  // (their planes take 72 KB), where 256 threads left a quarter of the
  // warps waiting at the barrier in those passes
  static constexpr bool ODD3 = N == 768 || N == 384;
  static constexpr int T = ODD3 ? 192 : ColCfg<N>::T;
  static constexpr int MINB = N >= 2048 ? 1 : ODD3 ? 3 : 2;
};

// Split-complex column pairs (cpx2): columns 2p and 2p + 1 of a group share a
// thread's registers; the staging buffers keep global memory's [row][column]
// float2 layout.
// a * b and a * conj(b) for two independent products
__device__ __forceinline__ cpx2 cmul_pp(cpx2 a, cpx2 b) {
  return {__ffma2_rn(a.re, b.re, neg2(__fmul2_rn(a.im, b.im))), __ffma2_rn(a.re, b.im, __fmul2_rn(a.im, b.re))};
}
__device__ __forceinline__ cpx2 cmulc_pp(cpx2 a, cpx2 b) {
  return {__ffma2_rn(a.re, b.re, __fmul2_rn(a.im, b.im)), __ffma2_rn(a.im, b.re, neg2(__fmul2_rn(a.re, b.im)))};
}
__device__ __forceinline__ cpx2 ld_pair(const float2* p) {  // two adjacent float2 (16-byte aligned)
  const float4 q = *reinterpret_cast<const float4*>(p);
  return pair(make_float2(q.x, q.y), make_float2(q.z, q.w));
}
__device__ __forceinline__ void st_pair(float2* p, cpx2 v) {
  *reinterpret_cast<float4*>(p) = make_float4(v.re.x, v.im.x, v.re.y, v.im.y);
}


// DCT-II post-processing of the FFT V of a column group (dense [row][column]
// in A, CS = ColCfg<H>::CS columns, T threads):
// C[k] = (wd[k] V[k] + conj(wd[k]) V[H-k]) / 2, stored down the columns
template <int H, int T>
__device__ __forceinline__ void dct2_cols_store(const float2* A, float2* dst, int WH, const float2* __restrict__ wd) {
  constexpr int CS = ColCfg<H>::CS;
  for (int e = threadIdx.x; e < H * CS; e += T) {
    const int s = e % CS, k = e / CS;
    const float2 w = __ldg(&wd[k]);
    const float2 a = A[k * CS + s], b = A[((H - k) % H) * CS + s];
    dst[(size_t)k * WH + s] = cscale(cadd(cmul(w, a), cmulc(b, w)), 0.5f);
  }
}

// transform lengths with row / column kernels
#define NSST_ROW_SIZES(X) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(1024)
#define NSST_COL_SIZES(X) X(128) X(192) X(256) X(384) X(512) X(768) X(1024) X(2048)

// The threshold rule of nsst_HT.m:34-46 (hard: |v| > th keeps v) and
// soft thresholding (sign(v) max(|v| - th, 0)).
__device__ __forceinline__ float apply_thresh(float v, float th, int mode) {
  if (mode == THRESH_HARD) return fabsf(v) > th ? v : 0.0f;
  float a = fabsf(v) - th;  // soft: sign(v) * max(|v| - th, 0)
  return a > 0.0f ? copysignf(a, v) : 0.0f;
}

// threshold of both real values of a packed element, stored dense [i][s]
template <int NSEQ>
struct ThreshSt {
  float2* p;
  float th;
  int mode;
  __device__ __forceinline__ void operator()(int i, int s, float2 v) const {
    v.x = apply_thresh(v.x, th, mode);
    v.y = apply_thresh(v.y, th, mode);
    p[i * NSEQ + s] = v;
  }
};

// ThreshSt that also records whether this thread kept any nonzero value
// (*kept, a thread-local flag; the caller reduces it over the block).
template <int NSEQ>
struct ThreshStKept {
  float2* p;
  float th;
  int mode;
  bool* kept;
  __device__ __forceinline__ void operator()(int i, int s, float2 v) const {
    v.x = apply_thresh(v.x, th, mode);
    v.y = apply_thresh(v.y, th, mode);
    *kept |= (v.x != 0.0f) | (v.y != 0.0f);
    p[i * NSEQ + s] = v;
  }
};

// FFT hooks (see block_fft_hook).
template <int NSEQ>
struct SmemLd {
  const float2* p;
  __device__ __forceinline__ float2 operator()(int i, int s) const { return p[i * NSEQ + s]; }
};
template <int NSEQ>
struct SmemSt {
  float2* p;
  __device__ __forceinline__ void operator()(int i, int s, float2 v) const { p[i * NSEQ + s] = v; }
};

// Row-major staging of a CTA's RS rows with rows padded to WH + 2 elements:
// the tile's global loads and stores then run along the rows (each warp a
// contiguous 256-byte stretch), and the FFT's first and last passes, which
// reach it through the functors below, see no bank conflicts.
template <int WH, int RS, int T>
__device__ __forceinline__ void fetch_rows_rm(float2* P, const float2* src) {
  constexpr int WHP = WH + 2, CH = WH / 2;  // 16-byte chunks per row
  for (int e = threadIdx.x; e < RS * CH; e += T) {
    const int s = e / CH, c = e - s * CH;
    cp_async16(P + s * WHP + 2 * c, src + (size_t)s * WH + 2 * c);
  }
  cp_async_commit();
}
template <int WH>
struct C2RPreLdRM {  // C2RPreLd reading the padded row-major staging
  const float2* X;
  const float2* twW;
  __device__ __forceinline__ float2 operator()(int k, int s) const {
    const float2* row = X + s * (WH + 2);
    const float2 xk = row[k];
    if (k == 0) return make_float2(xk.x + xk.y, xk.x - xk.y);
    const float2 xmc = cconj(row[WH - k]);
    const float2 E = cadd(xk, xmc);
    const float2 O = cmulc(csub(xk, xmc), __ldg(&twW[k]));
    return make_float2(E.x - O.y, E.y + O.x);
  }
};
template <int WH>
struct SmemStRM {  // element (i, s) -> padded row-major
  float2* p;
  __device__ __forceinline__ void operator()(int i, int s, float2 v) const { p[s * (WH + 2) + i] = v; }
};
template <int WH>
struct SmemLdRM {  // element (i, s) <- padded row-major
  const float2* p;
  __device__ __forceinline__ float2 operator()(int i, int s) const { return p[s * (WH + 2) + i]; }
};
// padded row-major rows -> global rows, 16 bytes per thread and step
template <int WH, int RS, int T>
__device__ __forceinline__ void store_rows_rm(float2* __restrict__ dst, const float2* P) {
  constexpr int CH = WH / 2;
  for (int e = threadIdx.x; e < RS * CH; e += T) {
    const int s = e / CH, c = e - s * CH;
    *reinterpret_cast<float4*>(dst + (size_t)s * WH + 2 * c) =
        *reinterpret_cast<const float4*>(P + s * (WH + 2) + 2 * c);
  }
}
// RS rows of WH zero float2 (the packed R2C of all-zero rows), 16 bytes per
// thread and step
template <int WH, int RS, int T>
__device__ __forceinline__ void store_zero_rows(float2* __restrict__ dst) {
  constexpr int CH = WH / 2;
  for (int e = threadIdx.x; e < RS * CH; e += T) {
    const int s = e / CH, c = e - s * CH;
    *reinterpret_cast<float4*>(dst + (size_t)s * WH + 2 * c) = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}
// packed-real post-processing of every index k (see r2c_post) fused with the
// store of the CTA's rows, from the padded row-major layout along the rows:
// X[k] = E + w^k O, E = (Z[k] + conj(Z[WH-k]))/2, O = (Z[k] - conj(Z[WH-k]))/(2i);
// k = 0 packs the two real bins.
template <int WH, int RS, int T>
__device__ __forceinline__ void r2c_post_store_rm(float2* __restrict__ dst, const float2* Z,
                                                  const float2* __restrict__ twW) {
#pragma unroll 4
  for (int e = threadIdx.x; e < WH * RS; e += T) {
    const int k = e % WH, s = e / WH;
    const float2* row = Z + s * (WH + 2);
    const float2 zk = row[k];
    float2 out;
    if (k == 0) {
      out = make_float2(zk.x + zk.y, zk.x - zk.y);
    } else {
      const float2 zmc = cconj(row[WH - k]);
      const float2 E = cscale(cadd(zk, zmc), 0.5f);
      const float2 d = cscale(csub(zk, zmc), 0.5f);
      const float2 To = cmul(__ldg(&twW[k]), make_float2(d.y, -d.x));
      out = cadd(E, To);
    }
    dst[(size_t)s * WH + k] = out;
  }
}


// Column hooks: element (i, s) of the CTA's column group is image element
// (row i, column col0 + s) of an H x WH packed array.
struct ColGlobalLd {
  const float2* src;
  int WH;
  __device__ __forceinline__ float2 operator()(int i, int s) const { return src[(size_t)i * WH + s]; }
};
struct ColGlobalSt {
  float2* dst;
  int WH;
  __device__ __forceinline__ void operator()(int i, int s, float2 v) const { dst[(size_t)i * WH + s] = v; }
};

}  // namespace nsst
