// À trous (dilated) pyramid filtering on sm_103a: the "direct" pyramid path.
//
// One call computes, for every output pixel,
//     out[r][c] = sum_{a,b} hf[a][b] * xe[r - M*c0 + M*a][c - M*c0 + M*b]
//               (+ the same with a second input / filter, summed),
// where hf is the filter flipped in both axes, c0 = (F-1)/2 and xe is the
// half-sample symmetric extension of x.  That is exactly one
// atrousc(symext(x, upsample2df(h, log2 M), shift), h, M) call of the
// reference (atrousc.cpp:43-73 with symext.m:18-31 and the shifts of
// atrousdec.m:33,44 / atrousrec.m:33,40; for every level those shifts centre
// the dilated filter, so the extension is a mirror with the edge sample
// repeated).  The GPU reference materialises the extension (symExt kernel,
// shear_cuda.cu:828-883) and a polyphase copy (atrousSubsample, :330-361)
// before convolving (atrousConvolution, :462-585); here the mirror is applied
// while the halo tile is staged into shared memory, so each launch reads its
// input once and writes its output once.
//
// Tiling: a CTA owns 64 columns x 64 rows of one polyphase row class
// (rows r = phase + M*t); with that split every tap row of the dilated filter
// is a neighbouring tile row.  Each thread keeps 8 vertically adjacent
// outputs of two columns 32 apart in registers, as float2 pairs, and streams
// one tap column at a time: 2(8+F-1) conflict-free shared loads feed 8F
// packed FP32 FMAs (FFMA2, two outputs per instruction).
#include <mutex>

#include "internal.h"

namespace nsst {

constexpr int kAtTX = 64;   // tile width (columns)
constexpr int kAtHX = kAtTX / 2;  // threads across: columns tx and tx + 32
constexpr int kAtP = 8;     // outputs per thread and column (poly rows)
constexpr int kAtTY = 8;    // thread rows
constexpr int kAtRows = kAtP * kAtTY;  // poly rows per tile
constexpr int kAtThreads = kAtHX * kAtTY;
// Launches whose 64-row grid would not fill the GPU (a single image, a few
// small images) use tiles of half the height: P = 4 outputs per thread.
constexpr int kAtPSmall = 4;

__device__ __forceinline__ int mirror_index(int i, int n) {
  if (i < 0) i = -1 - i;
  if (i >= n) i = 2 * n - 1 - i;
  // Only outputs that are never stored can reach past one reflection.
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

// out[r][c] += sum_{a,b} taps[a][b] * X[r + M(a - ORG)][c + M(b - ORG)] for this
// thread's 16 rows.  Forward steps: ORG = (F-1)/2 and X mirror-extended;
// adjoint steps (ZERO): ORG = F-1 and X zero-extended.
// ZR: tap rows 1 and F-2 are zero and symmetric columns (tap column b equals
// column F-1-b) -- the mirrored-quadrant filters of atrousfilters.m
// ('maxflat').  The zero rows are skipped at compile time, and each pair of
// mirrored input columns is added once (FADD2) before the shared taps
// multiply it: half the packed FMAs of the column pairs.
template <int F, bool ZERO, int P, bool ZR = false>
__device__ __forceinline__ void atrous_accumulate(const float* __restrict__ x, int H, int W, int M, int phase,
                                                  int prow0, int col0, const float* __restrict__ taps,
                                                  const int* __restrict__ tapcols, int ntapcols, float* tile,
                                                  float2 (&acc)[P]) {
  constexpr int C0 = ZERO ? F - 1 : (F - 1) / 2;
  constexpr int TR = P * kAtTY + F - 1;
  const int TC = kAtTX + M * (F - 1);
  const int tid = threadIdx.x;
  // halo tile: one warp per tile row at a time (the row's source index and
  // mirror are computed once), lanes across the row
  const int lane = tid & 31, warp = tid >> 5;
  for (int tr = warp; tr < TR; tr += kAtThreads / 32) {
    const int r = phase + M * (prow0 + tr - C0);
    float* trow = tile + tr * TC;
    const int cbase = col0 - M * C0;
    if (ZERO) {
      const bool rin = r >= 0 && r < H;
      const float* src = x + (size_t)(rin ? r : 0) * W;
      for (int tc = lane; tc < TC; tc += 32) {
        const int c = cbase + tc;
        trow[tc] = (rin && c >= 0 && c < W) ? __ldg(&src[c]) : 0.0f;
      }
    } else {
      const float* src = x + (size_t)mirror_index(r, H) * W;
      for (int tc = lane; tc < TC; tc += 32) trow[tc] = __ldg(&src[mirror_index(cbase + tc, W)]);
    }
  }
  __syncthreads();
  const int tx = tid % kAtHX, ty = tid / kAtHX;
  const float* base = tile + (ty * P) * TC + tx;
  for (int ib = 0; ib < ntapcols; ib++) {
    const int b = tapcols[ib];
    if (ZR && b > (F - 1) / 2) break;  // tapcols ascend; the mirrored half came with its partner
    float2 col[P + F - 1];
    if (ZR && b < (F - 1) / 2) {
      const int bm = F - 1 - b;
#pragma unroll
      for (int t = 0; t < P + F - 1; t++) {
        const float* q = base + t * TC + M * b;
        const float* qm = base + t * TC + M * bm;
        col[t] = __fadd2_rn(make_float2(q[0], q[kAtHX]), make_float2(qm[0], qm[kAtHX]));
      }
    } else {
#pragma unroll
      for (int t = 0; t < P + F - 1; t++) {
        const float* q = base + t * TC + M * b;
        col[t] = make_float2(q[0], q[kAtHX]);
      }
    }
#pragma unroll
    for (int a = 0; a < F; a++) {
      if (ZR && (a == 1 || a == F - 2)) continue;
      const float w = taps[a * F + b];
      const float2 w2 = make_float2(w, w);
#pragma unroll
      for (int p = 0; p < P; p++) acc[p] = __ffma2_rn(w2, col[p + a], acc[p]);
    }
  }
  __syncthreads();
}

// out = conv(xa, filter A) [+ conv(xb, filter B)].  grid = (W/64, M * ceil(ceil(H/M)/(8 P)), njobs)
template <int FA, int FB, bool ZERO = false, int P = kAtP, bool ZR = false>
__global__ void __launch_bounds__(kAtThreads, (FA <= 13 && FB == 0) ? 4 : 3) k_atrous(const __grid_constant__ AtrousJobs jobs, int M,
                                                        const __grid_constant__ AtrousTaps<FA> ta,
                                                        const __grid_constant__ AtrousTaps<FB> tb) {
  extern __shared__ float at_smem[];
  __shared__ float s_taps[(FA > FB ? FA * FA : FB * FB)];
  __shared__ int s_cols[(FA > FB ? FA : FB)];
  const AtrousJob& job = jobs.j[blockIdx.z];
  const int H = job.H, W = job.W;
  const int Ho = job.Ho > 0 ? job.Ho : H, Wo = job.Wo > 0 ? job.Wo : W;  // 0: same as the input
  const int col0 = blockIdx.x * kAtTX;
  const int phase = blockIdx.y % M;
  const int prow0 = (blockIdx.y / M) * (P * kAtTY);
  const int nprow = (Ho - phase + M - 1) / M;  // output poly rows of this phase
  if (col0 >= Wo || prow0 >= nprow) return;
  float2 acc[P];
#pragma unroll
  for (int p = 0; p < P; p++) acc[p] = make_float2(0.f, 0.f);

  for (int e = threadIdx.x; e < FA * FA; e += kAtThreads) s_taps[e] = ta.w[e];
  for (int e = threadIdx.x; e < ta.ncols; e += kAtThreads) s_cols[e] = ta.cols[e];
  __syncthreads();
  atrous_accumulate<FA, ZERO, P, ZR>(job.xa, H, W, M, phase, prow0, col0, s_taps, s_cols, ta.ncols, at_smem, acc);
  if (FB > 0 && job.xb != nullptr) {
    for (int e = threadIdx.x; e < FB * FB; e += kAtThreads) s_taps[e] = tb.w[e];
    for (int e = threadIdx.x; e < tb.ncols; e += kAtThreads) s_cols[e] = tb.cols[e];
    __syncthreads();
    atrous_accumulate<(FB > 0 ? FB : 1), ZERO, P, ZR>(job.xb, H, W, M, phase, prow0, col0, s_taps, s_cols,
                                                       tb.ncols, at_smem, acc);
  }
  const int tx = threadIdx.x % kAtHX, ty = threadIdx.x / kAtHX;
  const int c = col0 + tx;
#pragma unroll
  for (int p = 0; p < P; p++) {
    const int pr = prow0 + ty * P + p;
    if (pr < nprow) {
      float* o = job.out + (size_t)(phase + M * pr) * Wo;
      if (c < Wo) o[c] = acc[p].x;
      if (c + kAtHX < Wo) o[c + kAtHX] = acc[p].y;
    }
  }
}

template <int F>
static size_t atrous_smem(int M) {
  return sizeof(float) * (size_t)(kAtRows + F - 1) * (kAtTX + M * (F - 1));
}

template <int FA, int FB>
static size_t atrous_smem_pair(int M) {
  size_t sm = atrous_smem<FA>(M);
  if (FB > 0) sm = std::max(sm, atrous_smem<(FB > 0 ? FB : 1)>(M));
  return sm;
}

// The shared-memory opt-in only ever grows: plans (and the no-allocation
// entry point) with different pyramid depths share these kernels.
template <int FA, int FB>
static cudaError_t prepare_atrous_t(int Mmax) {
  constexpr int kDevs = 64;
  static std::mutex mu;
  static size_t configured[kDevs] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const size_t want = atrous_smem_pair<FA, FB>(Mmax);
  if (want > 227 * 1024) return cudaErrorInvalidValue;
  std::lock_guard<std::mutex> lk(mu);
  if (dev >= 0 && dev < kDevs && configured[dev] >= want) return cudaSuccess;
  e = cudaFuncSetAttribute(k_atrous<FA, FB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_atrous<FA, FB, false, kAtPSmall>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)want);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_atrous<FA, FB, false, kAtP, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)want);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_atrous<FA, FB, false, kAtPSmall, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)want);
  if (e == cudaSuccess && FB == 0)
    e = cudaFuncSetAttribute(k_atrous<FA, FB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want);
  if (e == cudaSuccess && FB == 0)
    e = cudaFuncSetAttribute(k_atrous<FA, FB, true, kAtP, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)want);
  if (e == cudaSuccess && dev >= 0 && dev < kDevs) configured[dev] = want;
  return e;
}

static int sm_count() {
  static const int n = [] {
    int dev = 0, c = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess || c <= 0)
      return 152;
    return c;
  }();
  return n;
}

// rows 1 and F-2 of an F x F filter all zero (F >= 5) and its columns
// mirror-symmetric (column b equals column F-1-b, nonzero together)
static bool zero_rows_1(const float* h, int F) {
  if (!h || F < 5) return false;
  for (int b = 0; b < F; b++)
    if (h[F + b] != 0.0f || h[(F - 2) * F + b] != 0.0f) return false;
  for (int a = 0; a < F; a++)
    for (int b = 0; b < F; b++)
      if (h[a * F + b] != h[a * F + (F - 1 - b)]) return false;
  return true;
}

template <int FA, int FB>
static cudaError_t launch_atrous_t(const AtrousJobs& jobs, int njobs, int maxH, int maxW, int M, const float* ha,
                                   const float* hb, cudaStream_t st) {
  AtrousTaps<FA> ta;
  AtrousTaps<FB> tb;
  fill_taps(ta, ha);
  if (FB > 0) fill_taps(tb, hb);
  const size_t sm = atrous_smem_pair<FA, FB>(M);
  const int nprow_max = (maxH + M - 1) / M;
  dim3 grid((maxW + kAtTX - 1) / kAtTX, M * ((nprow_max + kAtRows - 1) / kAtRows), njobs);
  count_launch();
  const bool zr = zero_rows_1(ha, FA) && (FB == 0 || zero_rows_1(hb, FB));
  if ((size_t)grid.x * grid.y * grid.z < (size_t)2 * sm_count()) {  // half-height tiles: twice the CTAs
    grid.y = M * ((nprow_max + kAtPSmall * kAtTY - 1) / (kAtPSmall * kAtTY));
    if (zr)
      k_atrous<FA, FB, false, kAtPSmall, true><<<grid, kAtThreads, sm, st>>>(jobs, M, ta, tb);
    else
      k_atrous<FA, FB, false, kAtPSmall><<<grid, kAtThreads, sm, st>>>(jobs, M, ta, tb);
  } else {
    if (zr)
      k_atrous<FA, FB, false, kAtP, true><<<grid, kAtThreads, sm, st>>>(jobs, M, ta, tb);
    else
      k_atrous<FA, FB, false><<<grid, kAtThreads, sm, st>>>(jobs, M, ta, tb);
  }
  return cudaGetLastError();
}

template <int F>
static cudaError_t launch_atrous_full_t(const AtrousJobs& jobs, int njobs, int maxHo, int maxWo, int M,
                                        const float* h, cudaStream_t st) {
  AtrousTaps<F> ta;
  AtrousTaps<0> tb;
  fill_taps(ta, h);
  fill_taps(tb, nullptr);
  const size_t sm = atrous_smem<F>(M);
  const int nprow_max = (maxHo + M - 1) / M;
  dim3 grid((maxWo + kAtTX - 1) / kAtTX, M * ((nprow_max + kAtRows - 1) / kAtRows), njobs);
  count_launch();
  if (zero_rows_1(h, F))  // the same filter structure as the forward steps
    k_atrous<F, 0, true, kAtP, true><<<grid, kAtThreads, sm, st>>>(jobs, M, ta, tb);
  else
    k_atrous<F, 0, true><<<grid, kAtThreads, sm, st>>>(jobs, M, ta, tb);
  return cudaGetLastError();
}

#define NSST_AT_PAIRS(X) X(13, 0) X(19, 0) X(19, 13) X(9, 0) X(7, 0) X(5, 0) X(7, 9) X(7, 5) X(7, 7)

cudaError_t prepare_atrous_kernels(int FA, int FB, int Mmax) {
#define NSST_AT(a, b) \
  if (FA == a && FB == b) return prepare_atrous_t<a, b>(Mmax);
  NSST_AT_PAIRS(NSST_AT)
#undef NSST_AT
  return cudaErrorInvalidValue;
}

cudaError_t launch_atrous(const AtrousJobs& jobs, int njobs, int maxH, int maxW, int M, int FA, const float* ha,
                          int FB, const float* hb, cudaStream_t st) {
  if (njobs == 0) return cudaSuccess;
  if (njobs > kMaxAtrousJobs) return cudaErrorInvalidValue;
#define NSST_AT(a, b) \
  if (FA == a && FB == b) return launch_atrous_t<a, b>(jobs, njobs, maxH, maxW, M, ha, hb, st);
  NSST_AT_PAIRS(NSST_AT)
#undef NSST_AT
  return cudaErrorInvalidValue;
}

cudaError_t launch_atrous_full(const AtrousJobs& jobs, int njobs, int maxHo, int maxWo, int M, int F, const float* h,
                               cudaStream_t st) {
  if (njobs == 0) return cudaSuccess;
  if (njobs > kMaxAtrousJobs) return cudaErrorInvalidValue;
  switch (F) {
    case 5: return launch_atrous_full_t<5>(jobs, njobs, maxHo, maxWo, M, h, st);
    case 7: return launch_atrous_full_t<7>(jobs, njobs, maxHo, maxWo, M, h, st);
    case 9: return launch_atrous_full_t<9>(jobs, njobs, maxHo, maxWo, M, h, st);
    case 13: return launch_atrous_full_t<13>(jobs, njobs, maxHo, maxWo, M, h, st);
    case 19: return launch_atrous_full_t<19>(jobs, njobs, maxHo, maxWo, M, h, st);
    default: return cudaErrorInvalidValue;
  }
}

bool atrous_pair_supported(int FA, int FB) {
#define NSST_AT(a, b) \
  if (FA == a && FB == b) return true;
  NSST_AT_PAIRS(NSST_AT)
#undef NSST_AT
  return false;
}

// Elementwise threshold of a band (used for the lowpass band and the
// standalone thresh entry point).  One launch covers nbands bands of n
// values each; band b uses thr[b].
__global__ void k_thresh_bands(float* __restrict__ data, size_t n, int nbands, const float* __restrict__ thr,
                               int mode) {
  size_t total = n * (size_t)nbands;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    float th = thr[i / n];
    float v = data[i];
    float r;
    if (mode == THRESH_HARD) {
      r = fabsf(v) > th ? v : 0.0f;
    } else {
      float a = fabsf(v) - th;
      r = a > 0.0f ? copysignf(a, v) : 0.0f;
    }
    data[i] = r;
  }
}

cudaError_t launch_thresh_bands(float* data, size_t n, int nbands, const float* thr, int mode, cudaStream_t st) {
  size_t total = n * (size_t)nbands;
  if (total == 0) return cudaSuccess;
  int blocks = (int)std::min<size_t>((total + 255) / 256, 152 * 16);
  count_launch();
  k_thresh_bands<<<blocks, 256, 0, st>>>(data, n, nbands, thr, mode);
  return cudaGetLastError();
}

}  // namespace nsst
