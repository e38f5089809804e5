// Undecimated (redundant) 2-D wavelet transform and the image-separation
// helpers, for n images per launch.
//
// mrdwt (shearcuda/src/mrdwt_r.h:104-209) filters each level's lowpass along
// rows and then columns with the level's dilation sf = 2^(l-1), periodically;
// mirdwt (mirdwt_r.h:115-219) undoes it columns first.  The filters are
// separable, so a level here runs in the other order -- columns, then rows --
// which lets the row pass (one CTA per image row, the whole row staged in
// shared memory) write its outputs over its inputs: an analysis level needs no
// scratch beyond its own output planes.  Per level:
//   analysis   columns: cur -> (C_lo, C_hi) in yh planes 1 and 0
//              rows:    C_lo -> LL (yl), HL (plane 1); C_hi -> LH (plane 0), HH (plane 2)
//   synthesis  rows:    (LL, HL) -> tl, (LH, HH) -> th
//              columns: (tl, th) -> x
// The column passes read their taps straight from global memory (each warp a
// 128-byte row segment, re-reads served by L1/L2); the row passes from shared
// memory.  All passes are HBM- or L2-bound stencils of at most 32 taps.
#include "internal.h"

namespace nsst {

constexpr int kWvRowThreads = 256;
constexpr int kWvMaxW = 8192;

__device__ __forceinline__ float hard_keep(float v, float t) { return fabsf(v) > t ? v : 0.0f; }
__device__ __forceinline__ float soft(float v, float t) {
  const float r = fabsf(v) - t;  // SoftThresh.m: sign(y) (|y| - t)_+
  return r > 0.0f ? copysignf(r, v) : 0.0f;
}

// ---------------------------------------------------------------- analysis
// C_lo[r][c] = sum_j a[j] cur[(r + j sf) mod H][c] -> yh plane 1; C_hi with b -> plane 0
__global__ void __launch_bounds__(256) k_rdwt_cols_fwd(const float* __restrict__ cur, size_t s_cur,
                                                       float* __restrict__ yh, size_t s_yh, int H, int W, int sf,
                                                       WvTaps t) {
  const int c = blockIdx.x * 32 + threadIdx.x, r = blockIdx.y * 8 + threadIdx.y, item = blockIdx.z;
  if (c >= W || r >= H) return;
  const float* x = cur + item * s_cur + c;
  float lo = 0.0f, hi = 0.0f;
  int rr = r;
  for (int j = 0; j < t.lh; j++) {
    const float v = __ldg(x + (size_t)rr * W);
    lo = fmaf(t.a[j], v, lo);
    hi = fmaf(t.b[j], v, hi);
    rr += sf;
    if (rr >= H) rr -= H;
  }
  const size_t HW = (size_t)H * W;
  float* out = yh + item * s_yh + (size_t)r * W + c;
  out[HW] = lo;
  out[0] = hi;
}

// one CTA per (row, item): LL = rows_a(C_lo), HL = rows_b(C_lo), LH = rows_a(C_hi), HH = rows_b(C_hi)
__global__ void __launch_bounds__(kWvRowThreads) k_rdwt_rows_fwd(float* yl, size_t s_yl, float* yh, size_t s_yh,
                                                                 int H, int W, int sf, WvTaps t,
                                                                 const float* __restrict__ thr) {
  extern __shared__ float sm[];
  float* slo = sm;
  float* shi = sm + W;
  const int r = blockIdx.x, item = blockIdx.y;
  const size_t HW = (size_t)H * W;
  float* p0 = yh + item * s_yh + (size_t)r * W;  // C_hi in, LH out
  float* p1 = p0 + HW;                           // C_lo in, HL out
  float* p2 = p1 + HW;                           // HH out
  for (int c = threadIdx.x; c < W; c += kWvRowThreads) {
    slo[c] = p1[c];
    shi[c] = p0[c];
  }
  __syncthreads();
  const float th = thr ? thr[item] : -1.0f;
  float* ylr = yl + item * s_yl + (size_t)r * W;
  for (int c = threadIdx.x; c < W; c += kWvRowThreads) {
    float ll = 0.0f, hl = 0.0f, lh = 0.0f, hh = 0.0f;
    int cc = c;
    for (int j = 0; j < t.lh; j++) {
      const float vl = slo[cc], vh = shi[cc];
      ll = fmaf(t.a[j], vl, ll);
      hl = fmaf(t.b[j], vl, hl);
      lh = fmaf(t.a[j], vh, lh);
      hh = fmaf(t.b[j], vh, hh);
      cc += sf;
      if (cc >= W) cc -= W;
    }
    if (th >= 0.0f) {
      hl = hard_keep(hl, th);
      lh = hard_keep(lh, th);
      hh = hard_keep(hh, th);
    }
    ylr[c] = ll;
    p0[c] = lh;
    p1[c] = hl;
    p2[c] = hh;
  }
}

// --------------------------------------------------------------- synthesis
// one CTA per (row, item): tl = a * LL + b * HL, th = a * LH + b * HH along the row (taps at c - t sf)
__global__ void __launch_bounds__(kWvRowThreads) k_rdwt_rows_inv(const float* ll, size_t s_ll, const float* yh,
                                                                 size_t s_yh, float* tl, float* th, size_t s_t,
                                                                 int H, int W, int sf, WvTaps t) {
  extern __shared__ float sm[];
  float* sll = sm;
  float* shl = sm + W;
  float* slh = sm + 2 * W;
  float* shh = sm + 3 * W;
  const int r = blockIdx.x, item = blockIdx.y;
  const size_t HW = (size_t)H * W;
  const float* q0 = yh + item * s_yh + (size_t)r * W;
  const float* q = ll + item * s_ll + (size_t)r * W;
  for (int c = threadIdx.x; c < W; c += kWvRowThreads) {
    sll[c] = q[c];
    slh[c] = q0[c];
    shl[c] = q0[HW + c];
    shh[c] = q0[2 * HW + c];
  }
  __syncthreads();
  float* outl = tl + item * s_t + (size_t)r * W;
  float* outh = th + item * s_t + (size_t)r * W;
  for (int c = threadIdx.x; c < W; c += kWvRowThreads) {
    float a = 0.0f, b = 0.0f;
    int cc = c;
    for (int k = 0; k < t.lh; k++) {
      a = fmaf(t.a[k], sll[cc], a);
      a = fmaf(t.b[k], shl[cc], a);
      b = fmaf(t.a[k], slh[cc], b);
      b = fmaf(t.b[k], shh[cc], b);
      cc -= sf;
      if (cc < 0) cc += W;
    }
    outl[c] = a;
    outh[c] = b;
  }
}

// x[r][c] = sum_t a[t] tl[(r - t sf) mod H][c] + b[t] th[(r - t sf) mod H][c]
__global__ void __launch_bounds__(256) k_rdwt_cols_inv(const float* __restrict__ tl, const float* __restrict__ th,
                                                       size_t s_t, float* __restrict__ x, size_t s_x, int H, int W,
                                                       int sf, WvTaps t) {
  const int c = blockIdx.x * 32 + threadIdx.x, r = blockIdx.y * 8 + threadIdx.y, item = blockIdx.z;
  if (c >= W || r >= H) return;
  const float* pl = tl + item * s_t + c;
  const float* ph = th + item * s_t + c;
  float acc = 0.0f;
  int rr = r;
  for (int k = 0; k < t.lh; k++) {
    acc = fmaf(t.a[k], __ldg(pl + (size_t)rr * W), acc);
    acc = fmaf(t.b[k], __ldg(ph + (size_t)rr * W), acc);
    rr -= sf;
    if (rr < 0) rr += H;
  }
  x[item * s_x + (size_t)r * W + c] = acc;
}

// ----------------------------------------------------- TV correction (Haar)
// y = mirdwt(LL, soft(yh, gamma)) with (LL, yh) = mrdwt(x) at one level and
// the Haar pair (analysis lo = a x[c] + a x[c+1], hi = a x[c] - a x[c+1];
// synthesis x = a/2 (lo[c] + lo[c-1]) + a/2 (hi[c] - hi[c-1]), a = 1/sqrt 2):
// an output pixel reads the 3 x 3 neighbourhood x[r-1..r+1][c-1..c+1].
constexpr int kTvTx = 32, kTvTy = 8;
__global__ void __launch_bounds__(kTvTx* kTvTy) k_tv_haar(const float* __restrict__ x, float* __restrict__ y,
                                                          size_t stride, int H, int W, WvTaps ta, WvTaps ts,
                                                          float gamma) {
  __shared__ float tile[kTvTy + 2][kTvTx + 2];  // rows r0-1 .. r0+8, cols c0-1 .. c0+32
  const int c0 = blockIdx.x * kTvTx, r0 = blockIdx.y * kTvTy, item = blockIdx.z;
  const float* xi = x + item * stride;
  for (int e = threadIdx.y * kTvTx + threadIdx.x; e < (kTvTy + 2) * (kTvTx + 2); e += kTvTx * kTvTy) {
    const int i = e / (kTvTx + 2), j = e % (kTvTx + 2);
    const int rr = ((r0 - 1 + i) % H + H) % H, cc = ((c0 - 1 + j) % W + W) % W;  // periodic, any H, W >= 1
    tile[i][j] = __ldg(xi + (size_t)rr * W + cc);
  }
  __syncthreads();
  const int r = r0 + threadIdx.y, c = c0 + threadIdx.x;
  if (r >= H || c >= W) return;
  // coefficients at (r - dr, c - dc), dr, dc in {0, 1}; tile index of x[r'][c'] is [r' - r0 + 1][c' - c0 + 1]
  float LL[2][2], LH[2][2], HL[2][2], HH[2][2];
#pragma unroll
  for (int dr = 0; dr < 2; dr++) {
#pragma unroll
    for (int dc = 0; dc < 2; dc++) {
      const int ti = threadIdx.y + 1 - dr, tj = threadIdx.x + 1 - dc;
      // rows first (mrdwt_r.h:157-177), then columns (:180-206)
      const float lr0 = ta.a[0] * tile[ti][tj] + ta.a[1] * tile[ti][tj + 1];
      const float hr0 = ta.b[0] * tile[ti][tj] + ta.b[1] * tile[ti][tj + 1];
      const float lr1 = ta.a[0] * tile[ti + 1][tj] + ta.a[1] * tile[ti + 1][tj + 1];
      const float hr1 = ta.b[0] * tile[ti + 1][tj] + ta.b[1] * tile[ti + 1][tj + 1];
      LL[dr][dc] = ta.a[0] * lr0 + ta.a[1] * lr1;
      LH[dr][dc] = soft(ta.b[0] * lr0 + ta.b[1] * lr1, gamma);
      HL[dr][dc] = soft(ta.a[0] * hr0 + ta.a[1] * hr1, gamma);
      HH[dr][dc] = soft(ta.b[0] * hr0 + ta.b[1] * hr1, gamma);
    }
  }
  // columns (mirdwt_r.h:163-189): x1 = a LL + b LH, xh = a HL + b HH over rows r, r-1
  float x1[2], xh[2];
#pragma unroll
  for (int dc = 0; dc < 2; dc++) {
    x1[dc] = ts.a[0] * LL[0][dc] + ts.b[0] * LH[0][dc] + ts.a[1] * LL[1][dc] + ts.b[1] * LH[1][dc];
    xh[dc] = ts.a[0] * HL[0][dc] + ts.b[0] * HH[0][dc] + ts.a[1] * HL[1][dc] + ts.b[1] * HH[1][dc];
  }
  // rows (:192-213) over columns c, c-1
  y[item * stride + (size_t)r * W + c] = ts.a[0] * x1[0] + ts.b[0] * xh[0] + ts.a[1] * x1[1] + ts.b[1] * xh[1];
}

// ---------------------------------------------------- decimated HH (FP64)
struct DTaps {
  double b[kMaxQmf];
  int lh;
};
__global__ void __launch_bounds__(256) k_dwt_hh(const float* __restrict__ xb, size_t stride, int H, int W, DTaps t,
                                                double* __restrict__ hhb) {
  const int l = blockIdx.x * 32 + threadIdx.x, k = blockIdx.y * 8 + threadIdx.y;
  if (l >= W / 2 || k >= H / 2) return;
  const float* x = xb + blockIdx.z * stride;
  double* hh = hhb + (size_t)blockIdx.z * (H / 2) * (W / 2);
  double acc = 0.0;
  int rr = 2 * k;
  for (int i = 0; i < t.lh; i++) {
    double row = 0.0;
    int cc = 2 * l;
    const float* xr = x + (size_t)rr * W;
    for (int j = 0; j < t.lh; j++) {
      row = fma(t.b[j], (double)__ldg(xr + cc), row);
      if (++cc >= W) cc -= W;
    }
    acc = fma(t.b[i], row, acc);
    if (++rr >= H) rr -= H;
  }
  hh[(size_t)k * (W / 2) + l] = acc;
}

// ------------------------------------------------------------- separation
__global__ void k_sep_residual(const float* __restrict__ img, const float* __restrict__ p1,
                               const float* __restrict__ p2, float* __restrict__ ra1, float* __restrict__ ra2,
                               size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float a = p1[i], b = p2[i];
    const float r = (img[i] - a) - b;  // GPUminus twice (separate.m:146-148)
    ra1[i] = a + r;
    ra2[i] = b + r;
  }
}

// ----------------------------------------------------------------- launchers
bool rdwt_width_supported(int W) { return W >= 2 && W <= kWvMaxW; }

static cudaError_t set_row_smem() {
  static cudaError_t once = [] {
    cudaError_t e = cudaFuncSetAttribute(k_rdwt_rows_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         2 * kWvMaxW * (int)sizeof(float));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_rdwt_rows_inv, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               4 * kWvMaxW * (int)sizeof(float));
    return e;
  }();
  return once;
}

cudaError_t launch_rdwt_level(const WvPlanes& P, int n, int H, int W, int sf, const WvTaps& t, const float* thr,
                              cudaStream_t st) {
  if (!rdwt_width_supported(W) || t.lh < 1 || t.lh > kMaxQmf || n < 1 || n > 65535) return cudaErrorInvalidValue;
  const cudaError_t e = set_row_smem();
  if (e != cudaSuccess) return e;
  const dim3 cb(32, 8), cg((W + 31) / 32, (H + 7) / 8, n);
  count_launch(2);
  k_rdwt_cols_fwd<<<cg, cb, 0, st>>>(P.cur, P.s_cur, P.yh, P.s_yh, H, W, sf, t);
  k_rdwt_rows_fwd<<<dim3(H, n), kWvRowThreads, 2 * W * sizeof(float), st>>>(P.yl, P.s_yl, P.yh, P.s_yh, H, W, sf,
                                                                             t, thr);
  return cudaGetLastError();
}

cudaError_t launch_irdwt_level(const float* ll, size_t s_ll, const float* yh, size_t s_yh, float* tl, float* th,
                               size_t s_t, float* x, size_t s_x, int n, int H, int W, int sf, const WvTaps& t,
                               cudaStream_t st) {
  if (!rdwt_width_supported(W) || t.lh < 1 || t.lh > kMaxQmf || n < 1 || n > 65535) return cudaErrorInvalidValue;
  const cudaError_t e = set_row_smem();
  if (e != cudaSuccess) return e;
  count_launch(2);
  k_rdwt_rows_inv<<<dim3(H, n), kWvRowThreads, 4 * W * sizeof(float), st>>>(ll, s_ll, yh, s_yh, tl, th, s_t, H, W,
                                                                             sf, t);
  const dim3 cb(32, 8), cg((W + 31) / 32, (H + 7) / 8, n);
  k_rdwt_cols_inv<<<cg, cb, 0, st>>>(tl, th, s_t, x, s_x, H, W, sf, t);
  return cudaGetLastError();
}

cudaError_t launch_tv_haar(const float* x, float* y, size_t stride, int n, int H, int W, float a, float gamma,
                           cudaStream_t st) {
  if (n < 1 || n > 65535) return cudaErrorInvalidValue;
  const std::vector<double> haar = {(double)a, (double)a};
  const WvTaps ta = analysis_taps(haar), ts = synthesis_taps(haar);
  count_launch();
  k_tv_haar<<<dim3((W + kTvTx - 1) / kTvTx, (H + kTvTy - 1) / kTvTy, n), dim3(kTvTx, kTvTy), 0, st>>>(
      x, y, stride, H, W, ta, ts, gamma);
  return cudaGetLastError();
}

cudaError_t launch_dwt_hh(const float* x, size_t stride, int n, int H, int W, const double* b, int lh, double* hh,
                          cudaStream_t st) {
  if (lh < 1 || lh > kMaxQmf || n < 1 || n > 65535) return cudaErrorInvalidValue;
  DTaps t{};
  t.lh = lh;
  for (int i = 0; i < lh; i++) t.b[i] = b[i];
  count_launch();
  k_dwt_hh<<<dim3((W / 2 + 31) / 32, (H / 2 + 7) / 8, n), dim3(32, 8), 0, st>>>(x, stride, H, W, t, hh);
  return cudaGetLastError();
}

cudaError_t launch_sep_residual(const float* img, const float* p1, const float* p2, float* ra1, float* ra2,
                                size_t n, cudaStream_t st) {
  const int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
  count_launch();
  k_sep_residual<<<blocks, 256, 0, st>>>(img, p1, p2, ra1, ra2, n);
  return cudaGetLastError();
}

}  // namespace nsst
