// The à trous pyramid in the DCT-II domain (the spectral pyramid of the fused
// denoise pipeline, its backward, shear_trans / inverse_shear and atrousdec).
//
// Every pyramid step of the reference (atrousc.cpp:43-73 on symext.m's
// extension, atrousdec.m:33-44, atrousrec.m:33-40) filters with a filter that
// is symmetric in both axes (all of atrousfilters.m's sets) on the
// half-sample symmetric extension of its input, reflected once.  On the
// 2H x 2W periodic symmetric extension that is a circular convolution, which
// the 2-D DCT-II diagonalises:
//     DCT2(conv(x, h dilated by M)) = DCT2(x) .* G_h(M k1 / H, M k2 / W),
//     G_h(u, v) = sum_{a,b} h[a][b] cos(pi u (a - c0)) cos(pi v (b - c0)).
// So the whole pyramid is pointwise: band l = IDCT2(X .* R_l) with X =
// DCT2(x), and the reconstruction is IDCT2(sum_l DCT2(band'_l) .* Q_l +
// X .* T), R, Q and T being products of the level responses (FP64 host
// tables, the 1/(H W) of the inverse folded in).  The directional stage needs
// fft2(band l), so the pyramid's transforms merge with the level FFTs:
//     rows    : X .* R_l -> DCT-III -> R2C FFT          (k_dct_rows_ana)
//     columns : DCT-III -> FFT                          (k_dct_cols<H, kDctAna>)
// and on the way back
//     columns : DCT-II of the band sum (after the inverse column FFT)
//     rows    : C2R -> DCT-II -> .* Q_l, summed over the levels, + X .* T,
//               then DCT-III                            (k_dct_rows_syn)
//     columns : DCT-III -> the output image             (k_dct_cols_out)
// A thresholded lowpass leaves the DCT domain once (k_dct_rows_ana<·, true>,
// k_dct_cols<H, kDctThresh>, k_dct_rows_fwd).  Seven launches replace the
// direct pyramid's FFMA-bound convolutions (two launches per analysis level,
// one per synthesis level: twelve at four levels) and the three level-FFT
// launches; with the TMA directional kernels (k_cols_tma.cu) the level
// analysis does the DCT-III + FFT column pass and the register-sum synthesis
// the band sums' DCT-II, leaving five.
//
// DCTs of length N through one N-point FFT (J. Makhoul, "A fast cosine
// transform in one and two dimensions", IEEE Trans. ASSP 28(1), 1980), all
// unnormalised: C[k] = sum_n x[n] cos(pi k (2n + 1) / (2N)) and its inverse
// up to the factor N, with wd[k] = exp(-i pi k / (2N)):
//   DCT-II : v[n] = x[2n], v[N-1-n] = x[2n+1];  V = FFT(v);
//            C[k] = (wd[k] V[k] + conj(wd[k]) V[N-k]) / 2   (= Re(wd[k] V[k]) for real x)
//   DCT-III: Z[k] = conj(wd[k]) (C[k] - i C[N-k]), C[N] = 0;  v = IFFT(Z) (unscaled);
//            x[2n] = v[n], x[2n+1] = v[N-1-n]
// Both forms are complex-linear, so a column group of a packed real plane
// (two real columns per float2) or of a packed half spectrum transforms as
// complex data.  Rows are real: they use the W/2-point packed real FFT
// (c2r / r2c pre- and post-processing) of the directional kernels.
#include "internal.h"
#include "tiles.cuh"

namespace nsst {

namespace {

template <int WH>
__device__ __forceinline__ const float* rowf(const float2* P, int s) {
  return reinterpret_cast<const float*>(P + s * (WH + 2));
}

// DCT-II input order of a real row in the padded row-major staging: element
// m of the W/2-point complex view is (v[2m], v[2m+1]), v[j] = x[2j] for
// j < W/2 and x[2W-1-2j] above.
template <int WH>
struct DctShufLd {
  const float2* P;
  __device__ __forceinline__ float2 operator()(int m, int s) const {
    constexpr int W = 2 * WH;
    const float* x = rowf<WH>(P, s);
    const int j0 = 2 * m, j1 = 2 * m + 1;
    return make_float2(j0 < WH ? x[2 * j0] : x[2 * W - 1 - 2 * j0], j1 < WH ? x[2 * j1] : x[2 * W - 1 - 2 * j1]);
  }
};

// The same order written by the last pass of a C2R whose element m is
// (y[2m], y[2m+1]): v[m] = y[2m], v[W-1-m] = y[2m+1] (stride-1 stores, where
// DctShufLd's reads are four floats apart)
template <int WH>
struct DctShufStRM {
  float2* P;
  __device__ __forceinline__ void operator()(int m, int s, float2 y) const {
    float* v = reinterpret_cast<float*>(P + s * (WH + 2));
    v[m] = y.x;
    v[2 * WH - 1 - m] = y.y;
  }
};

// The DCT-III output order undone: y[2m] = v[m], y[2m+1] = v[W-1-m]; element
// m of y's complex view.
template <int WH>
struct DctUnshufLd {
  const float2* P;
  __device__ __forceinline__ float2 operator()(int m, int s) const {
    const float* v = rowf<WH>(P, s);
    return make_float2(v[m], v[2 * WH - 1 - m]);
  }
};

// Row twiddles, one 16-byte load per index k = 0..W/2: (wd[k], twW[k]) with
// wd[k] = exp(-i pi k / (2W)) and twW[k] = exp(-2 pi i k / W) the packed-real
// twiddle (k < W/2).  wd[W/2 - k] = exp(-i pi / 4) conj(wd[k]).
__device__ __forceinline__ float2 wd_mirror(float2 w) {
  constexpr float c = 0.70710678118654752f;
  return make_float2(c * (w.x - w.y), -c * (w.x + w.y));
}

// Zh[k] = conj(w) (a - i b)
__device__ __forceinline__ float2 dct3_pre(float2 w, float a, float b) {
  return make_float2(w.x * a - w.y * b, -(w.x * b + w.y * a));
}

// DCT-III pre-processing of a real coefficient row c(j), j = 0..W-1, fused
// with the packed-real C2R pre-processing: the half spectrum
// Zh[k] = conj(wd[k]) (C[k] - i C[W-k]), k = 0..W/2, is Hermitian, and the
// W/2-point complex inputs k and W/2-k are built from Zh[k] and Zh[W/2-k]
// (k = 0 unpacks the two real bins).  Written to the padded row-major row
// `out`, which c must not read.
template <int WH, class Coef>
__device__ __forceinline__ void dct3_pre_pair(const Coef& c, int k, const float4* __restrict__ tw, float2* out) {
  const float4 t = __ldg(&tw[k == 0 ? WH : k]);
  const float2 w = make_float2(t.x, t.y);
  if (k == 0) {
    const float cn = c(WH);
    const float dc = c(0), ny = dct3_pre(w, cn, cn).x;
    out[0] = make_float2(dc + ny, dc - ny);
    return;
  }
  const float2 xk = dct3_pre(w, c(k), c(2 * WH - k));
  const float2 xmc = cconj(dct3_pre(wd_mirror(w), c(WH - k), c(WH + k)));
  const float2 E = cadd(xk, xmc);
  const float2 O = cmulc(csub(xk, xmc), make_float2(t.z, t.w));
  out[k] = make_float2(E.x - O.y, E.y + O.x);
  if (k != WH - k) out[WH - k] = make_float2(E.x + O.y, O.x - E.y);  // conj(E) + i conj(O)
}

// DCT-II coefficients of a real row from the forward FFT Z of its shuffled
// complex view (padded row-major): the packed-real post-processing gives V[k],
// then C[k] = Re(wd[k] V[k]) and C[W-k] = -Im(wd[k] V[k]).  For k = 0 the pair
// is (C[0], C[W/2]); otherwise (C[k], C[W-k]).
template <int WH>
__device__ __forceinline__ void dct2_row_pair(const float2* row, int k, const float4* __restrict__ tw, float& ck,
                                              float& cm) {
  const float2 zk = row[k];
  const float4 t = __ldg(&tw[k == 0 ? WH : k]);
  if (k == 0) {
    ck = zk.x + zk.y;
    cm = (zk.x - zk.y) * t.x;
    return;
  }
  const float2 zmc = cconj(row[WH - k]);
  const float2 E = cscale(cadd(zk, zmc), 0.5f);
  const float2 d = cscale(csub(zk, zmc), 0.5f);
  const float2 V = cadd(E, cmul(make_float2(t.z, t.w), make_float2(d.y, -d.x)));
  const float2 U = cmul(make_float2(t.x, t.y), V);
  ck = U.x;
  cm = -U.y;
}

}  // namespace

// Two transforms with DCT pre- and post-processing per kernel need more
// registers than one: 768 threads per SM (at most 80 registers each).
template <int T>
struct DctMinB {
  static constexpr int value = 768 / T;
};

// ---------------------------------------------------------------------------
// Row kernels, grid = (H / RS, jobs); RS rows per CTA staged row-major.
// ---------------------------------------------------------------------------

// real rows (the caller's images) -> DCT-II rows
template <int WH>
__global__ void __launch_bounds__(RowCfg<WH>::T, DctMinB<RowCfg<WH>::T>::value)
    k_dct_rows_fwd(const __grid_constant__ DctIo io, const float2* __restrict__ twWh, const float4* __restrict__ tw) {
  using C = RowCfg<WH>;
  extern __shared__ float2 smem[];
  float2* A = smem;
  const size_t off = (size_t)blockIdx.x * C::RS * WH;  // float2 units
  fetch_rows_rm<WH, C::RS, C::T>(A, reinterpret_cast<const float2*>(io.src[blockIdx.y]) + off);
  cp_async_wait_all();
  __syncthreads();
  block_fft_hook_ip<WH, C::RS, C::T, -1>(A, twWh, DctShufLd<WH>{A}, SmemStRM<WH>{A});
  float* dst = io.dst[blockIdx.y] + 2 * off;
  for (int e = threadIdx.x; e < WH * C::RS; e += C::T) {
    const int k = e % WH, s = e / WH;
    float ck, cm;
    dct2_row_pair<WH>(A + s * (WH + 2), k, tw, ck, cm);
    float* d = dst + (size_t)s * 2 * WH;
    d[k] = ck;
    d[k == 0 ? WH : 2 * WH - k] = cm;
  }
}

// level analysis rows: (X .* R_level) -> DCT-III -> R2C -> packed half
// spectrum rows; REAL: (X .* R) -> DCT-III -> real rows (the lowpass band).
// job.src: X plane, job.dst: output plane, job.th_index: the response plane.
template <int WH, bool REAL>
__global__ void __launch_bounds__(RowCfg<WH>::T, DctMinB<RowCfg<WH>::T>::value)
    k_dct_rows_ana(const RowJob* __restrict__ jobs, int n_active, const float2* src_base, float2* dst_base,
                   const float* __restrict__ resp, size_t resp_stride, const float2* __restrict__ twWh,
                   const float2* __restrict__ twW, const float4* __restrict__ tw) {
  using C = RowCfg<WH>;
  extern __shared__ float2 smem[];
  float2* A = smem;
  const RowJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const size_t off = (size_t)blockIdx.x * C::RS * WH;
  const float* X = reinterpret_cast<const float*>(src_base + job.src + off);
  const float* R = resp + (size_t)job.th_index * resp_stride + 2 * off;
  constexpr int NP = WH / 2 + 1;  // index pairs (k, WH - k) per row
  for (int e = threadIdx.x; e < C::RS * NP; e += C::T) {
    const int s = e / NP, k = e - s * NP;
    const float* xr = X + (size_t)s * 2 * WH;
    const float* rr = R + (size_t)s * 2 * WH;
    dct3_pre_pair<WH>([&](int j) { return xr[j] * __ldg(&rr[j]); }, k, tw, A + s * (WH + 2));
  }
  __syncthreads();
  block_fft_hook_ip<WH, C::RS, C::T, +1>(A, twWh, SmemLdRM<WH>{A}, SmemStRM<WH>{A});
  if (REAL) {
    float2* dst = dst_base + job.dst + off;
    for (int e = threadIdx.x; e < WH * C::RS; e += C::T) {
      const int m = e % WH, s = e / WH;
      const float* v = rowf<WH>(A, s);
      dst[(size_t)s * WH + m] = make_float2(v[m], v[2 * WH - 1 - m]);
    }
    return;
  }
  block_fft_hook_ip<WH, C::RS, C::T, -1>(A, twWh, DctUnshufLd<WH>{A}, SmemStRM<WH>{A});
  r2c_post_store_rm<WH, C::RS, C::T>(dst_base + job.dst + off, A, twW);
}

// synthesis rows of one item: for every level l the band sum's packed half
// spectrum rows (DCT-II down the columns already) -> C2R -> DCT-II -> .* Q_l,
// accumulated with X .* T in shared memory, then DCT-III -> real rows.  With
// REAL the level planes already hold the bands' DCT-II coefficients (real).
// job.src: level 0 of the band sums (level l at + l * lev_stride), job.dst:
// the output plane; X plane of the item at xbase + item * xstride.
template <int WH, bool REAL>
__global__ void __launch_bounds__(RowCfg<WH>::T, DctMinB<RowCfg<WH>::T>::value)
    k_dct_rows_syn(const RowJob* __restrict__ jobs, int n_active, int nlev, size_t lev_stride,
                   const float2* src_base, float2* dst_base, const float* __restrict__ xbase, size_t xstride,
                   const float* __restrict__ resp, size_t resp_stride, const float* __restrict__ tlow,
                   const float2* __restrict__ twWh, const float2* __restrict__ twW, const float4* __restrict__ tw) {
  using C = RowCfg<WH>;
  constexpr int CH = WH / 2;
  constexpr int W = 2 * WH;
  extern __shared__ float2 smem[];
  float2* A = smem;                      // transform tile
  float2* S = smem + C::RS * (WH + 2);   // coefficient sums, same padded layout
  const RowJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const size_t off = (size_t)blockIdx.x * C::RS * WH;
  {
    const float4* X = reinterpret_cast<const float4*>(xbase + (size_t)job.item * xstride + 2 * off);
    const float4* T = reinterpret_cast<const float4*>(tlow + 2 * off);
    for (int e = threadIdx.x; e < C::RS * CH; e += C::T) {
      const int s = e / CH, c = e - s * CH;
      const float4 x = X[(size_t)s * CH + c], t = __ldg(&T[(size_t)s * CH + c]);
      *reinterpret_cast<float4*>(S + s * (WH + 2) + 2 * c) = make_float4(x.x * t.x, x.y * t.y, x.z * t.z, x.w * t.w);
    }
  }
  // (a prefetch of the next level into a third buffer measured no faster:
  // fewer CTAs per SM)
  for (int l = 0; l < nlev && REAL; l++) {
    const float4* Y = reinterpret_cast<const float4*>(src_base + job.src + (size_t)l * lev_stride + off);
    const float4* Q = reinterpret_cast<const float4*>(resp + (size_t)l * resp_stride + 2 * off);
    for (int e = threadIdx.x; e < C::RS * CH; e += C::T) {
      const int s = e / CH, c = e - s * CH;
      const float4 y = Y[(size_t)s * CH + c], q = __ldg(&Q[(size_t)s * CH + c]);
      float4* a = reinterpret_cast<float4*>(S + s * (WH + 2) + 2 * c);
      const float4 v = *a;
      *a = make_float4(v.x + y.x * q.x, v.y + y.y * q.y, v.z + y.z * q.z, v.w + y.w * q.w);
    }
  }
  if (REAL) __syncthreads();
  for (int l = 0; l < nlev && !REAL; l++) {
    fetch_rows_rm<WH, C::RS, C::T>(A, src_base + job.src + (size_t)l * lev_stride + off);
    cp_async_wait_all();
    __syncthreads();
    // C2R stored in the DCT-II input order, then the DCT-II's FFT
    block_fft_hook_ip<WH, C::RS, C::T, +1>(A, twWh, C2RPreLdRM<WH>{A, twW}, DctShufStRM<WH>{A});
    block_fft_hook_ip<WH, C::RS, C::T, -1>(A, twWh, SmemLdRM<WH>{A}, SmemStRM<WH>{A});
    const float* Q = resp + (size_t)l * resp_stride + 2 * off;
    for (int e = threadIdx.x; e < WH * C::RS; e += C::T) {
      const int k = e % WH, s = e / WH;
      float ck, cm;
      dct2_row_pair<WH>(A + s * (WH + 2), k, tw, ck, cm);
      const int km = k == 0 ? WH : W - k;
      float* acc = reinterpret_cast<float*>(S + s * (WH + 2));
      acc[k] += ck * __ldg(&Q[(size_t)s * W + k]);
      acc[km] += cm * __ldg(&Q[(size_t)s * W + km]);
    }
    __syncthreads();
  }
  {
    constexpr int NP = WH / 2 + 1;
    for (int e = threadIdx.x; e < C::RS * NP; e += C::T) {
      const int s = e / NP, k = e - s * NP;
      const float* sr = rowf<WH>(S, s);
      dct3_pre_pair<WH>([&](int j) { return sr[j]; }, k, tw, A + s * (WH + 2));
    }
    __syncthreads();
  }
  block_fft_hook_ip<WH, C::RS, C::T, +1>(A, twWh, SmemLdRM<WH>{A}, SmemStRM<WH>{A});
  float2* dst = dst_base + job.dst + off;
  for (int e = threadIdx.x; e < WH * C::RS; e += C::T) {
    const int m = e % WH, s = e / WH;
    const float* v = rowf<WH>(A, s);
    dst[(size_t)s * WH + m] = make_float2(v[m], v[W - 1 - m]);
  }
}

// ---------------------------------------------------------------------------
// Column kernels, grid = (WH / CS, jobs): CS columns of a packed H x WH array.
// ---------------------------------------------------------------------------
// kDct2: DCT-II; kDct3: DCT-III; kDctAna: DCT-III then the forward FFT;
// kDctThresh: DCT-III, the threshold (th, tmode) of both real columns of each
// element, DCT-II (the DCT-II input order undoes the DCT-III output order, so
// the threshold applies to the inverse FFT's output in place)
template <int H, int MODE>
__device__ __forceinline__ void dct_cols_body(const float2* src, float2* dst, int WH, float2* A,
                                              const float2* __restrict__ twH, const float2* __restrict__ wd,
                                              float th = 0.0f, int tmode = 0) {
  using C = ColCfg<H>;
  auto row_of = [](int i) { return i < H / 2 ? 2 * i : 2 * H - 1 - 2 * i; };
  if (MODE == kDct2) {
    // the column group staged in the DCT-II input order: source row r is
    // element r/2 (r even) or H-1-(r-1)/2 (r odd) of v
    for (int e = threadIdx.x; e < H * (C::CS / 2); e += C::T) {
      const int r = e / (C::CS / 2), c = e - r * (C::CS / 2);
      const int i = (r & 1) ? H - 1 - (r >> 1) : (r >> 1);
      cp_async16(A + i * C::CS + 2 * c, src + (size_t)r * WH + 2 * c);
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    block_fft_hook_ip<H, C::CS, C::T, -1>(A, twH, SmemLd<C::CS>{A}, SmemSt<C::CS>{A});
    dct2_cols_store<H, ColCfg<H>::T>(A, dst, WH, wd);
    return;
  }
  // the column group staged whole (the pre-processing pairs rows k and H-k)
  for (int e = threadIdx.x; e < H * (C::CS / 2); e += C::T) {
    const int i = e / (C::CS / 2), c = e - i * (C::CS / 2);
    cp_async16(A + i * C::CS + 2 * c, src + (size_t)i * WH + 2 * c);
  }
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();
  // Z[k] = conj(wd[k]) (C[k] - i C[H-k]) and Z[H-k] = conj(wd[H-k]) (C[H-k] - i C[k])
  // = i wd[k] (C[H-k] - i C[k]): each pair in place by one thread
  for (int e = threadIdx.x; e < (H / 2 + 1) * C::CS; e += C::T) {
    const int s = e % C::CS, k = e / C::CS;
    if (k == 0) continue;  // Z[0] = C[0]
    const float2 w = __ldg(&wd[k]);
    const float2 a = A[k * C::CS + s], b = A[(H - k) * C::CS + s];
    A[k * C::CS + s] = cmulc(make_float2(a.x + b.y, a.y - b.x), w);
    if (k != H - k) A[(H - k) * C::CS + s] = cmul(make_float2(b.x + a.y, b.y - a.x), make_float2(-w.y, w.x));
  }
  __syncthreads();
  if (MODE == kDct3) {
    block_fft_hook_ip<H, C::CS, C::T, +1>(A, twH, SmemLd<C::CS>{A},
                                          [&](int i, int s, float2 v) { dst[(size_t)row_of(i) * WH + s] = v; });
  } else if (MODE == kDctThresh) {
    block_fft_hook_ip<H, C::CS, C::T, +1>(A, twH, SmemLd<C::CS>{A}, [&](int i, int s, float2 v) {
      A[i * C::CS + s] = make_float2(apply_thresh(v.x, th, tmode), apply_thresh(v.y, th, tmode));
    });
    block_fft_hook_ip<H, C::CS, C::T, -1>(A, twH, SmemLd<C::CS>{A}, SmemSt<C::CS>{A});
    dct2_cols_store<H, ColCfg<H>::T>(A, dst, WH, wd);
  } else {
    block_fft_hook_ip<H, C::CS, C::T, +1>(A, twH, SmemLd<C::CS>{A},
                                          [&](int i, int s, float2 v) { A[row_of(i) * C::CS + s] = v; });
    block_fft_hook_ip<H, C::CS, C::T, -1>(A, twH, SmemLd<C::CS>{A}, ColGlobalSt{dst, WH});
  }
}

template <int H, int MODE>
__global__ void __launch_bounds__(ColCfg<H>::T, DctMinB<ColCfg<H>::T>::value)
    k_dct_cols(const ColJob* __restrict__ jobs, int n_active, int WH, const float2* src_base, float2* dst_base,
               const float2* __restrict__ twH, const float2* __restrict__ wd, const float* __restrict__ thr,
               int th_stride, int tmode) {
  extern __shared__ float2 smem[];
  const ColJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const int col0 = blockIdx.x * ColCfg<H>::CS;
  const float th = MODE == kDctThresh ? thr[(size_t)job.item * th_stride] : 0.0f;
  dct_cols_body<H, MODE>(src_base + job.src + col0, dst_base + job.dst + col0, WH, smem, twH, wd, th, tmode);
}

// DCT-III down the columns into the caller's output images
template <int H>
__global__ void __launch_bounds__(ColCfg<H>::T, DctMinB<ColCfg<H>::T>::value)
    k_dct_cols_out(const __grid_constant__ DctIo io, int WH, const float2* __restrict__ twH,
                   const float2* __restrict__ wd) {
  extern __shared__ float2 smem[];
  const int col0 = blockIdx.x * ColCfg<H>::CS;
  dct_cols_body<H, kDct3>(reinterpret_cast<const float2*>(io.src[blockIdx.y]) + col0,
                          reinterpret_cast<float2*>(io.dst[blockIdx.y]) + col0, WH, smem, twH, wd);
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
#define NSST_DCT_ROW_SIZES(X) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(1024)
#define NSST_DCT_COL_SIZES(X) X(128) X(192) X(256) X(384) X(512) X(768) X(1024) X(2048)

template <typename KernelT>
static cudaError_t dct_opt_in(KernelT k, size_t bytes) {
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

cudaError_t prepare_dct_kernels(int H, int WH) {
  cudaError_t e = cudaErrorInvalidValue;
  switch (WH) {
#define CASE(n)                                                                  \
  case n:                                                                        \
    e = dct_opt_in(k_dct_rows_fwd<n>, RowCfg<n>::smem_rm());                     \
    if (e == cudaSuccess) e = dct_opt_in(k_dct_rows_ana<n, false>, RowCfg<n>::smem_rm()); \
    if (e == cudaSuccess) e = dct_opt_in(k_dct_rows_ana<n, true>, RowCfg<n>::smem_rm()); \
    if (e == cudaSuccess) e = dct_opt_in(k_dct_rows_syn<n, false>, 2 * RowCfg<n>::smem_rm()); \
    if (e == cudaSuccess) e = dct_opt_in(k_dct_rows_syn<n, true>, 2 * RowCfg<n>::smem_rm()); \
    break;
    NSST_DCT_ROW_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess) return e;
  switch (H) {
#define CASE(n)                                                                         \
  case n: {                                                                             \
    constexpr size_t sm = ColCfg<n>::smem() / 2;                                        \
    e = dct_opt_in(k_dct_cols<n, kDct2>, sm);                                           \
    if (e == cudaSuccess) e = dct_opt_in(k_dct_cols<n, kDctAna>, sm);                   \
    if (e == cudaSuccess) e = dct_opt_in(k_dct_cols<n, kDctThresh>, sm);                \
    if (e == cudaSuccess) e = dct_opt_in(k_dct_cols_out<n>, sm);                        \
    return e;                                                                           \
  }
    NSST_DCT_COL_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_dct_rows_fwd(const DctIo& io, int n, int H, int W, const float2* twWh, const float4* twD,
                                cudaStream_t st) {
  if (n <= 0 || n > kMaxAtrousJobs) return n == 0 ? cudaSuccess : cudaErrorInvalidValue;
  count_launch();
  switch (W / 2) {
#define CASE(n_)                                                                                         \
  case n_:                                                                                               \
    k_dct_rows_fwd<n_><<<dim3(H / RowCfg<n_>::RS, n), RowCfg<n_>::T, RowCfg<n_>::smem_rm(), st>>>(io, twWh, \
                                                                                                   twD);      \
    return cudaGetLastError();
    NSST_DCT_ROW_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_dct_rows_ana(const RowJob* jobs, int njobs, int n_active, int H, int W, const void* src_base,
                                void* dst_base, const float* resp, size_t resp_stride, const float2* twWh,
                                const float2* twW, const float4* twD, bool real_out, cudaStream_t st) {
  if (njobs == 0) return cudaSuccess;
  count_launch();
  const float2* sb = static_cast<const float2*>(src_base);
  float2* db = static_cast<float2*>(dst_base);
  switch (W / 2) {
#define CASE(n_)                                                                                            \
  case n_: {                                                                                                \
    const dim3 grid(H / RowCfg<n_>::RS, njobs);                                                             \
    if (real_out)                                                                                           \
      k_dct_rows_ana<n_, true><<<grid, RowCfg<n_>::T, RowCfg<n_>::smem_rm(), st>>>(                          \
          jobs, n_active, sb, db, resp, resp_stride, twWh, twW, twD);                                       \
    else                                                                                                    \
      k_dct_rows_ana<n_, false><<<grid, RowCfg<n_>::T, RowCfg<n_>::smem_rm(), st>>>(                         \
          jobs, n_active, sb, db, resp, resp_stride, twWh, twW, twD);                                       \
    return cudaGetLastError();                                                                              \
  }
    NSST_DCT_ROW_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_dct_rows_syn(const RowJob* jobs, int njobs, int n_active, int nlev, size_t lev_stride, int H,
                                int W, const void* src_base, void* dst_base, const float* xbase, size_t xstride,
                                const float* resp, size_t resp_stride, const float* tlow, const float2* twWh,
                                const float2* twW, const float4* twD, cudaStream_t st, bool real_in) {
  if (njobs == 0) return cudaSuccess;
  count_launch();
  const float2* sb = static_cast<const float2*>(src_base);
  float2* db = static_cast<float2*>(dst_base);
  switch (W / 2) {
#define CASE(n_)                                                                                              \
  case n_: {                                                                                                  \
    const dim3 grid(H / RowCfg<n_>::RS, njobs);                                                               \
    constexpr size_t sm = 2 * RowCfg<n_>::smem_rm();                                                          \
    if (real_in)                                                                                              \
      k_dct_rows_syn<n_, true><<<grid, RowCfg<n_>::T, sm, st>>>(jobs, n_active, nlev, lev_stride, sb, db, xbase, \
                                                               xstride, resp, resp_stride, tlow, twWh, twW, twD); \
    else                                                                                                      \
      k_dct_rows_syn<n_, false><<<grid, RowCfg<n_>::T, sm, st>>>(jobs, n_active, nlev, lev_stride, sb, db, xbase, \
                                                                xstride, resp, resp_stride, tlow, twWh, twW, twD); \
    return cudaGetLastError();                                                                                \
  }
    NSST_DCT_ROW_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_dct_cols(int mode, const ColJob* jobs, int njobs, int n_active, int H, int W, const void* src_base,
                            void* dst_base, const float2* twH, const float2* wdH, cudaStream_t st, const float* thr,
                            int th_stride, int th_mode) {
  if (njobs == 0) return cudaSuccess;
  if (mode != kDct2 && mode != kDctAna && mode != kDctThresh) return cudaErrorInvalidValue;
  if (mode == kDctThresh && !thr) return cudaErrorInvalidValue;
  count_launch();
  const int WH = W / 2;
  const float2* sb = static_cast<const float2*>(src_base);
  float2* db = static_cast<float2*>(dst_base);
  switch (H) {
#define CASE(n_)                                                                                   \
  case n_: {                                                                                       \
    const dim3 grid(WH / ColCfg<n_>::CS, njobs);                                                   \
    constexpr size_t sm = ColCfg<n_>::smem() / 2;                                                  \
    if (mode == kDct2)                                                                             \
      k_dct_cols<n_, kDct2><<<grid, ColCfg<n_>::T, sm, st>>>(jobs, n_active, WH, sb, db, twH, wdH,     \
                                                             thr, th_stride, th_mode);                 \
    else if (mode == kDctAna)                                                                      \
      k_dct_cols<n_, kDctAna><<<grid, ColCfg<n_>::T, sm, st>>>(jobs, n_active, WH, sb, db, twH, wdH,   \
                                                               thr, th_stride, th_mode);               \
    else                                                                                           \
      k_dct_cols<n_, kDctThresh><<<grid, ColCfg<n_>::T, sm, st>>>(jobs, n_active, WH, sb, db, twH,     \
                                                                  wdH, thr, th_stride, th_mode);       \
    return cudaGetLastError();                                                                     \
  }
    NSST_DCT_COL_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_dct_cols_out(const DctIo& io, int n, int H, int W, const float2* twH, const float2* wdH,
                                cudaStream_t st) {
  if (n <= 0 || n > kMaxAtrousJobs) return n == 0 ? cudaSuccess : cudaErrorInvalidValue;
  count_launch();
  const int WH = W / 2;
  switch (H) {
#define CASE(n_)                                                                                                   \
  case n_:                                                                                                         \
    k_dct_cols_out<n_><<<dim3(WH / ColCfg<n_>::CS, n), ColCfg<n_>::T, ColCfg<n_>::smem() / 2, st>>>(io, WH, twH, \
                                                                                                   wdH);           \
    return cudaGetLastError();
    NSST_DCT_COL_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace nsst
