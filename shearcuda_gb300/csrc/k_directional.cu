// Directional (shearing) stage of the 2-D NSST on sm_103a.
//
// Replaces the reference's cuFFT + modulate/threshold/sum kernel chain
// (shear_trans_cuda.cpp:220-287, inverse_shear_cuda.cpp:222-286,
//  shear_cuda.cu:39-138 modulate*, :620-822 hard/softThreshold*, :255-291
//  sumVectors*) with hand-written FFT passes that fuse the spectral multiply,
// the threshold and the band sum:
//
//   analysis  c_k = real(ifft2(W_k .* fft2(y)))            (nsst_dec2.m:58)
//   threshold c'_k = T(c_k)                                 (nsst_HT.m:34-46)
//   synthesis y'  = real(ifft2(sum_k conj(W_k) .* fft2(c'_k))) (nsst_rec2.m:27-33)
//
// Data layout ("packed half spectrum"): an H x W real image maps to an
// H x (W/2) array of float2.  Rows hold the W/2+1 non-redundant bins of the
// row transform with the two real bins (DC, Nyquist) packed into slot 0; the
// column transform then runs on all W/2 columns alike, column 0 carrying the
// DC and Nyquist columns as one complex sequence.  Filter spectra are stored
// in the same layout, pre-scaled by 1/(H W); column 0 keeps
// P = (W_0 + W_N)/2 in place and M = (W_0 - W_N)/2 in a side array, because
// the packed column needs Z'[u] = P[u] Z[u] + M[u] conj(Z[-u]).
//
// Every kernel takes a job list (one job per image / level / band) in device
// memory plus a tile index, so one launch covers a whole batch of images of
// one size.
#include "fft_core.cuh"
#include "internal.h"

namespace nsst {

constexpr int kThreads = 256;

template <int N>
struct RowCfg {  // N = W/2 complex points per row
  static constexpr int RS = N >= 1024 ? 8 : 16;
  static constexpr size_t smem() { return (size_t)N * (RS + 1) * sizeof(float2); }
};
template <int N>
struct ColCfg {  // N = H points per column
  static constexpr int CS = N >= 2048 ? 4 : (N >= 768 ? 8 : 16);
  static constexpr size_t smem() { return (size_t)N * (CS + 1) * sizeof(float2); }
};

__device__ __forceinline__ float apply_thresh(float v, float th, int mode) {
  if (mode == THRESH_HARD) return fabsf(v) > th ? v : 0.0f;
  float a = fabsf(v) - th;  // soft: sign(v) * max(|v| - th, 0)
  return a > 0.0f ? copysignf(a, v) : 0.0f;
}

// ---------------------------------------------------------------------------
// Row kernels.  grid = (H / RS, njobs), block = kThreads.
// ---------------------------------------------------------------------------

// real rows -> packed half-spectrum rows (forward R2C along W)
template <int WH>
__global__ void __launch_bounds__(kThreads) k_rows_fwd(const RowJob* __restrict__ jobs, int n_active, const float2* src_base,
                                                        float2* dst_base, const float2* __restrict__ twWh,
                                                        const float2* __restrict__ twW) {
  constexpr int RS = RowCfg<WH>::RS, LD = RS + 1;
  extern __shared__ float2 smem[];
  const RowJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const int row0 = blockIdx.x * RS;
  const float2* src = src_base + job.src + (size_t)row0 * WH;
  for (int e = threadIdx.x; e < WH * RS; e += kThreads) {
    int s = e / WH, i = e % WH;
    smem[i * LD + s] = src[(size_t)s * WH + i];
  }
  __syncthreads();
  block_fft<WH, RS, kThreads, -1>(smem, twWh);
  r2c_post<WH, RS, kThreads>(smem, twW);
  float2* dst = dst_base + job.dst + (size_t)row0 * WH;
  for (int e = threadIdx.x; e < WH * RS; e += kThreads) {
    int s = e / WH, i = e % WH;
    dst[(size_t)s * WH + i] = smem[i * LD + s];
  }
}

// packed rows -> real rows (inverse C2R along W, unnormalised: x W)
template <int WH>
__global__ void __launch_bounds__(kThreads) k_rows_inv(const RowJob* __restrict__ jobs, int n_active, const float2* src_base,
                                                        float2* dst_base, const float2* __restrict__ twWh,
                                                        const float2* __restrict__ twW) {
  constexpr int RS = RowCfg<WH>::RS, LD = RS + 1;
  extern __shared__ float2 smem[];
  const RowJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const int row0 = blockIdx.x * RS;
  const float2* src = src_base + job.src + (size_t)row0 * WH;
  for (int e = threadIdx.x; e < WH * RS; e += kThreads) {
    int s = e / WH, i = e % WH;
    smem[i * LD + s] = src[(size_t)s * WH + i];
  }
  __syncthreads();
  c2r_pre<WH, RS, kThreads>(smem, twW);
  block_fft<WH, RS, kThreads, +1>(smem, twWh);
  float2* dst = dst_base + job.dst + (size_t)row0 * WH;
  for (int e = threadIdx.x; e < WH * RS; e += kThreads) {
    int s = e / WH, i = e % WH;
    dst[(size_t)s * WH + i] = smem[i * LD + s];
  }
}

// packed rows -> C2R -> threshold -> R2C -> packed rows (the fused band round trip)
template <int WH>
__global__ void __launch_bounds__(kThreads) k_rows_thresh(const RowJob* __restrict__ jobs, int n_active, const float2* src_base,
                                                           float2* dst_base, const float2* __restrict__ twWh,
                                                           const float2* __restrict__ twW,
                                                           const float* __restrict__ thr, int mode) {
  constexpr int RS = RowCfg<WH>::RS, LD = RS + 1;
  extern __shared__ float2 smem[];
  const RowJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const float th = thr[job.th_index];
  const int row0 = blockIdx.x * RS;
  const float2* src = src_base + job.src + (size_t)row0 * WH;
  for (int e = threadIdx.x; e < WH * RS; e += kThreads) {
    int s = e / WH, i = e % WH;
    smem[i * LD + s] = src[(size_t)s * WH + i];
  }
  __syncthreads();
  c2r_pre<WH, RS, kThreads>(smem, twW);
  block_fft<WH, RS, kThreads, +1>(smem, twWh);
  for (int e = threadIdx.x; e < WH * RS; e += kThreads) {
    int i = e / RS, s = e % RS;
    float2 v = smem[i * LD + s];
    v.x = apply_thresh(v.x, th, mode);
    v.y = apply_thresh(v.y, th, mode);
    smem[i * LD + s] = v;
  }
  __syncthreads();
  block_fft<WH, RS, kThreads, -1>(smem, twWh);
  r2c_post<WH, RS, kThreads>(smem, twW);
  float2* dst = dst_base + job.dst + (size_t)row0 * WH;
  for (int e = threadIdx.x; e < WH * RS; e += kThreads) {
    int s = e / WH, i = e % WH;
    dst[(size_t)s * WH + i] = smem[i * LD + s];
  }
}

// ---------------------------------------------------------------------------
// Column kernels.  grid = (WH / CS, njobs), block = kThreads.
// ---------------------------------------------------------------------------

// plain column FFT (forward or inverse) src -> dst
template <int H, int DIR>
__global__ void __launch_bounds__(kThreads) k_cols(const ColJob* __restrict__ jobs, int n_active, int WH, const float2* src_base,
                                                    float2* dst_base, const float2* __restrict__ twH) {
  constexpr int CS = ColCfg<H>::CS, LD = CS + 1;
  extern __shared__ float2 smem[];
  const ColJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const int col0 = blockIdx.x * CS;
  for (int e = threadIdx.x; e < H * CS; e += kThreads) {
    int i = e / CS, s = e % CS;
    smem[i * LD + s] = src_base[job.src + (size_t)i * WH + col0 + s];
  }
  __syncthreads();
  block_fft<H, CS, kThreads, DIR>(smem, twH);
  for (int e = threadIdx.x; e < H * CS; e += kThreads) {
    int i = e / CS, s = e % CS;
    dst_base[job.dst + (size_t)i * WH + col0 + s] = smem[i * LD + s];
  }
}

// analysis band: dst = colIFFT( Wk .* src ), src = fully transformed level spectrum
template <int H>
__global__ void __launch_bounds__(kThreads) k_band_analysis(const ColJob* __restrict__ jobs, int n_active, int WH,
                                                             const float2* src_base, float2* dst_base,
                                                             const float2* __restrict__ spec_base,
                                                             const float2* __restrict__ twH) {
  constexpr int CS = ColCfg<H>::CS, LD = CS + 1;
  extern __shared__ float2 smem[];
  const ColJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const int col0 = blockIdx.x * CS;
  for (int e = threadIdx.x; e < H * CS; e += kThreads) {
    int i = e / CS, s = e % CS;
    size_t g = (size_t)i * WH + col0 + s;
    float2 z = src_base[job.src + g];
    float2 p = __ldg(&spec_base[job.spec + g]);
    float2 r = cmul(p, z);
    if (col0 + s == 0) {  // packed DC/Nyquist column
      float2 zm = src_base[job.src + (size_t)((H - i) % H) * WH];
      r = cadd(r, cmul(__ldg(&spec_base[job.m0 + i]), cconj(zm)));
    }
    smem[i * LD + s] = r;
  }
  __syncthreads();
  block_fft<H, CS, kThreads, +1>(smem, twH);
  for (int e = threadIdx.x; e < H * CS; e += kThreads) {
    int i = e / CS, s = e % CS;
    dst_base[job.dst + (size_t)i * WH + col0 + s] = smem[i * LD + s];
  }
}

// synthesis: dst = colIFFT( sum_k conj(Wk) .* colFFT(src_k) ) over job.nbands
// bands stored at src + k * band_stride, spectra at spec + k * band_stride,
// side arrays at m0 + k * H.
template <int H>
__global__ void __launch_bounds__(kThreads) k_band_synthesis(const ColJob* __restrict__ jobs, int n_active, int WH,
                                                              const float2* src_base, float2* dst_base,
                                                              const float2* __restrict__ spec_base,
                                                              size_t band_stride,
                                                              const float2* __restrict__ twH) {
  constexpr int CS = ColCfg<H>::CS, LD = CS + 1;
  constexpr int EPT = H * CS / kThreads;
  static_assert(H * CS % kThreads == 0, "tile must divide evenly");
  extern __shared__ float2 smem[];
  const ColJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const int col0 = blockIdx.x * CS;
  float2 acc[EPT];
#pragma unroll
  for (int it = 0; it < EPT; it++) acc[it] = make_float2(0.f, 0.f);
  for (int k = 0; k < job.nbands; k++) {
    const float2* src = src_base + job.src + k * band_stride;
    const float2* spec = spec_base + job.spec + k * band_stride;
#pragma unroll 4
    for (int it = 0; it < EPT; it++) {
      int e = threadIdx.x + it * kThreads;
      int i = e / CS, s = e % CS;
      smem[i * LD + s] = src[(size_t)i * WH + col0 + s];
    }
    __syncthreads();
    block_fft<H, CS, kThreads, -1>(smem, twH);
#pragma unroll
    for (int it = 0; it < EPT; it++) {
      int e = threadIdx.x + it * kThreads;
      int i = e / CS, s = e % CS;
      float2 z = smem[i * LD + s];
      float2 p = __ldg(&spec[(size_t)i * WH + col0 + s]);
      acc[it] = cadd(acc[it], cmulc(z, p));
      if (col0 + s == 0) {
        float2 zm = smem[((H - i) % H) * LD];
        float2 m = __ldg(&spec_base[job.m0 + (size_t)k * H + i]);
        // conj(M) * conj(z[-u]) = conj(M * z[-u])
        acc[it] = cadd(acc[it], cconj(cmul(m, zm)));
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int it = 0; it < EPT; it++) {
    int e = threadIdx.x + it * kThreads;
    int i = e / CS, s = e % CS;
    smem[i * LD + s] = acc[it];
  }
  __syncthreads();
  block_fft<H, CS, kThreads, +1>(smem, twH);
  for (int e = threadIdx.x; e < H * CS; e += kThreads) {
    int i = e / CS, s = e % CS;
    dst_base[job.dst + (size_t)i * WH + col0 + s] = smem[i * LD + s];
  }
}

// ---------------------------------------------------------------------------
// Host-side launchers, dispatched on the (compile-time) transform lengths.
// The dynamic shared-memory opt-in is done once per device and kernel by the
// prepare_* calls (plan creation), never on the launch path.
// ---------------------------------------------------------------------------
#define NSST_ROW_SIZES(X) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(1024)
#define NSST_COL_SIZES(X) X(128) X(192) X(256) X(384) X(512) X(768) X(1024) X(2048)

bool row_len_supported(int wh) {
  switch (wh) {
#define CASE(n) case n:
    NSST_ROW_SIZES(CASE)
#undef CASE
    return true;
    default:
      return false;
  }
}
bool col_len_supported(int h) {
  switch (h) {
#define CASE(n) case n:
    NSST_COL_SIZES(CASE)
#undef CASE
    return true;
    default:
      return false;
  }
}
int row_tile(int wh) { return wh >= 1024 ? 8 : 16; }
int col_tile(int h) { return h >= 2048 ? 4 : (h >= 768 ? 8 : 16); }

template <typename KernelT>
static cudaError_t opt_in(KernelT k, size_t bytes) {
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

cudaError_t prepare_row_kernels(int wh) {
  switch (wh) {
#define CASE(n)                                                               \
  case n: {                                                                   \
    constexpr size_t sm = RowCfg<n>::smem();                                  \
    cudaError_t e = opt_in(k_rows_fwd<n>, sm);                                \
    if (e == cudaSuccess) e = opt_in(k_rows_inv<n>, sm);                      \
    if (e == cudaSuccess) e = opt_in(k_rows_thresh<n>, sm);                   \
    return e;                                                                 \
  }
    NSST_ROW_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t prepare_col_kernels(int h) {
  switch (h) {
#define CASE(n)                                                               \
  case n: {                                                                   \
    constexpr size_t sm = ColCfg<n>::smem();                                  \
    cudaError_t e = opt_in(k_cols<n, -1>, sm);                                \
    if (e == cudaSuccess) e = opt_in(k_cols<n, 1>, sm);                       \
    if (e == cudaSuccess) e = opt_in(k_band_analysis<n>, sm);                 \
    if (e == cudaSuccess) e = opt_in(k_band_synthesis<n>, sm);                \
    return e;                                                                 \
  }
    NSST_COL_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_rows(RowOp op, const RowJob* jobs, int njobs, int n_active, int H, int W, const void* src_base,
                        void* dst_base, const float2* twWh, const float2* twW, const float* thr, int mode,
                        cudaStream_t st) {
  const int WH = W / 2;
  if (njobs == 0) return cudaSuccess;
  count_launch();
  const float2* sb = static_cast<const float2*>(src_base);
  float2* db = static_cast<float2*>(dst_base);
  switch (WH) {
#define CASE(n)                                                                        \
  case n: {                                                                            \
    constexpr size_t sm = RowCfg<n>::smem();                                           \
    dim3 grid(H / RowCfg<n>::RS, njobs);                                               \
    if (op == RowOp::Fwd)                                                              \
      k_rows_fwd<n><<<grid, kThreads, sm, st>>>(jobs, n_active, sb, db, twWh, twW);              \
    else if (op == RowOp::Inv)                                                         \
      k_rows_inv<n><<<grid, kThreads, sm, st>>>(jobs, n_active, sb, db, twWh, twW);              \
    else                                                                               \
      k_rows_thresh<n><<<grid, kThreads, sm, st>>>(jobs, n_active, sb, db, twWh, twW, thr, mode); \
    return cudaGetLastError();                                                         \
  }
    NSST_ROW_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_cols(ColOp op, const ColJob* jobs, int njobs, int n_active, int H, int W, const float2* src_base,
                        float2* dst_base, const float2* spec_base, size_t band_stride, const float2* twH,
                        cudaStream_t st) {
  const int WH = W / 2;
  if (njobs == 0) return cudaSuccess;
  count_launch();
  switch (H) {
#define CASE(n)                                                                                       \
  case n: {                                                                                           \
    constexpr size_t sm = ColCfg<n>::smem();                                                          \
    dim3 grid(WH / ColCfg<n>::CS, njobs);                                                             \
    if (op == ColOp::Fwd)                                                                             \
      k_cols<n, -1><<<grid, kThreads, sm, st>>>(jobs, n_active, WH, src_base, dst_base, twH);                   \
    else if (op == ColOp::Inv)                                                                        \
      k_cols<n, 1><<<grid, kThreads, sm, st>>>(jobs, n_active, WH, src_base, dst_base, twH);                    \
    else if (op == ColOp::Analysis)                                                                   \
      k_band_analysis<n><<<grid, kThreads, sm, st>>>(jobs, n_active, WH, src_base, dst_base, spec_base, twH);   \
    else                                                                                              \
      k_band_synthesis<n><<<grid, kThreads, sm, st>>>(jobs, n_active, WH, src_base, dst_base, spec_base,        \
                                                      band_stride, twH);                              \
    return cudaGetLastError();                                                                        \
  }
    NSST_COL_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace nsst
