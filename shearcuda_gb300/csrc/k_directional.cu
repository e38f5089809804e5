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
#include "internal.h"
#include "tiles.cuh"

namespace nsst {

// packed-real pre-processing of index k (see c2r_pre) is C2RPreLdRM (tiles.cuh):
// Z[k] = E + iO with E = X[k] + conj(X[WH-k]), O = (X[k] - conj(X[WH-k])) w^-k;
// k = 0 unpacks the two real bins.
// ---------------------------------------------------------------------------
// Row kernels.  grid = (H / RS, njobs).
// ---------------------------------------------------------------------------

// real rows -> packed half-spectrum rows (forward R2C along W)
template <int WH>
__global__ void __launch_bounds__(RowCfg<WH>::T, RowCfg<WH>::MINB) k_rows_fwd(const RowJob* __restrict__ jobs, int n_active,
                                                             const float2* src_base, float2* dst_base,
                                                             const float2* __restrict__ twWh,
                                                             const float2* __restrict__ twW) {
  using C = RowCfg<WH>;
  extern __shared__ float2 smem[];
  float2 *A = smem, *B = smem + (size_t)WH * C::LD;
  const RowJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const size_t off = (size_t)blockIdx.x * C::RS * WH;
  fetch_rows_rm<WH, C::RS, C::T>(A, src_base + job.src + off);
  cp_async_wait_all();
  __syncthreads();
  (void)B;
  block_fft_hook_ip<WH, C::RS, C::T, -1>(A, twWh, SmemLdRM<WH>{A}, SmemStRM<WH>{A});
  r2c_post_store_rm<WH, C::RS, C::T>(dst_base + job.dst + off, A, twW);
}

// packed rows -> real rows (inverse C2R along W, unnormalised: x W)
template <int WH>
__global__ void __launch_bounds__(RowCfg<WH>::T, RowCfg<WH>::MINB) k_rows_inv(const RowJob* __restrict__ jobs, int n_active,
                                                             const float2* src_base, float2* dst_base,
                                                             const float2* __restrict__ twWh,
                                                             const float2* __restrict__ twW) {
  using C = RowCfg<WH>;
  extern __shared__ float2 smem[];
  float2 *A = smem, *B = smem + (size_t)WH * C::LD;
  const RowJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const size_t off = (size_t)blockIdx.x * C::RS * WH;
  fetch_rows_rm<WH, C::RS, C::T>(A, src_base + job.src + off);
  cp_async_wait_all();
  __syncthreads();
  (void)B;
  block_fft_hook_ip<WH, C::RS, C::T, +1>(A, twWh, C2RPreLdRM<WH>{A, twW}, SmemStRM<WH>{A});
  store_rows_rm<WH, C::RS, C::T>(dst_base + job.dst + off, A);
}

// packed rows -> C2R -> threshold -> R2C -> packed rows (the band round trip
// of the split directional stage).  RS rows per CTA: RowCfg's tile, or a
// multiple of it (the autotuner's row-tile candidates) with the threads per
// row unchanged.
template <int WH, int RS>
struct RowTile {
  static constexpr int T = RowCfg<WH>::T / RowCfg<WH>::RS * RS;
  static constexpr int MINB = 1024 / T > 0 ? 1024 / T : 1;
  static constexpr size_t smem() { return (size_t)RS * (WH + 2) * sizeof(float2); }
};
template <int WH, int RS = RowCfg<WH>::RS>
__global__ void __launch_bounds__(RowTile<WH, RS>::T, RowTile<WH, RS>::MINB)
    k_rows_thresh(const RowJob* __restrict__ jobs, int n_active, const float2* src_base, float2* dst_base,
                  const float2* __restrict__ twWh, const float2* __restrict__ twW, const float* __restrict__ thr,
                  int mode) {
  constexpr int T = RowTile<WH, RS>::T;
  extern __shared__ float2 smem[];
  float2* A = smem;
  const RowJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const float th = thr[job.th_index];
  const size_t off = (size_t)blockIdx.x * RS * WH;
  // the tile arrives row-major (padded); the first pass reads it from there
  // and leaves the dense [index][row] layout in the same buffer
  fetch_rows_rm<WH, RS, T>(A, src_base + job.src + off);
  cp_async_wait_all();
  __syncthreads();
  // C2R (pre-processing in the first pass) -> threshold -> R2C, in place on
  // one buffer (every pass reads all of its inputs, the pre-processing's
  // mirrored ones included, before a barrier); the R2C's last pass goes back
  // to the padded row-major layout, the post-processing is fused with a store
  // along the rows.  A tile whose coefficients all threshold to zero has a
  // zero transform: it stores zero rows instead.
  auto thresh = [&](float2 v, bool& kept) {
    v.x = apply_thresh(v.x, th, mode);
    v.y = apply_thresh(v.y, th, mode);
    kept |= (v.x != 0.0f) | (v.y != 0.0f);
    return v;
  };
  using Plan = typename FftPlan<WH>::type;
  if constexpr (FirstRadix<Plan>::value == LastRadix<Plan>::value) {
    // the turn from the C2R to the R2C in registers
    if (!block_fft_inv_op_fwd<WH, RS, T>(A, twWh, C2RPreLdRM<WH>{A, twW}, thresh, SmemStRM<WH>{A})) {
      store_zero_rows<WH, RS, T>(dst_base + job.dst + off);
      return;
    }
  } else {
    bool kept = false;
    block_fft_hook_ip<WH, RS, T, +1>(A, twWh, C2RPreLdRM<WH>{A, twW}, ThreshStKept<RS>{A, th, mode, &kept});
    if (!__syncthreads_or(kept)) {
      store_zero_rows<WH, RS, T>(dst_base + job.dst + off);
      return;
    }
    block_fft_hook_ip<WH, RS, T, -1>(A, twWh, SmemLd<RS>{A}, SmemStRM<WH>{A});
  }
  r2c_post_store_rm<WH, RS, T>(dst_base + job.dst + off, A, twW);
}

// The band row pass on split-complex pairs (cpx2): rows 2p and 2p + 1 of the
// tile share a thread's registers, so the twiddle multiplies, the packed-real
// pre- and post-processing and the index arithmetic serve two rows at once as
// FP32x2 instructions.  Same operations per value as k_rows_thresh.  twWh4 /
// twW4: the row twiddle tables with each entry as its broadcast pairs.
// Radix plans of the paired row transforms: FftPlan's, up to 128 registers
// (sixteen pairs in a radix-16 pass).  A 256-point 8 x 8 x 4 plan at 64
// registers (32 warps per SM) measured slower than radix 16 x 16 at 128
// (4.71 against 4.44 ms for the directional stage of 64 x 512^2).
template <int WH>
struct RowPlanP {
  using type = typename FftPlan<WH>::type;
  static constexpr int R0 = 16;  // largest radix: butterflies per pass = WH / R0 per sequence
  static constexpr int MAXREG = 128;
};
template <int WH, int RS>
struct RowTileP {
  static constexpr int NP = RS / 2;  // row pairs
  static constexpr int T0 = WH / RowPlanP<WH>::R0 * NP;
  static constexpr int T = T0 < 64 ? 64 : T0;
  static constexpr int MINB = 65536 / RowPlanP<WH>::MAXREG / T > 0 ? 65536 / RowPlanP<WH>::MAXREG / T : 1;
  static constexpr size_t smem() { return (size_t)RS * (WH + 2) * sizeof(float2); }
  static_assert(RS % 2 == 0 && T % 32 == 0, "row pairs, whole warps");
};
template <int WH, int RS>
__global__ void __launch_bounds__(RowTileP<WH, RS>::T, RowTileP<WH, RS>::MINB)
    k_rows_thresh_p(const RowJob* __restrict__ jobs, int n_active, const float2* src_base, float2* dst_base,
                    const float2* __restrict__ twWh4, const float4* __restrict__ twW4, const float* __restrict__ thr,
                    int mode) {
  constexpr int NP = RowTileP<WH, RS>::NP, T = RowTileP<WH, RS>::T, RP = WH + 2;
  extern __shared__ float2 smem[];
  float2* A = smem;                         // row-major rows, pitch WH + 2
  cpx2* D = reinterpret_cast<cpx2*>(smem);  // dense [index][pair] between passes
  const RowJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const float th = thr[job.th_index];
  const size_t off = (size_t)blockIdx.x * RS * WH;
  fetch_rows_rm<WH, RS, T>(A, src_base + job.src + off);
  cp_async_wait_all();
  __syncthreads();
  // C2R, pre-processing (see c2r_pre) in the first pass's loads:
  // Z[k] = E + iO, E = X[k] + conj(X[WH-k]), O = (X[k] - conj(X[WH-k])) w^-k
  auto ld = [&](int k, int p) -> cpx2 {
    const float2* r0 = A + 2 * p * RP;
    const cpx2 xk = pair(r0[k], r0[RP + k]);
    if (k == 0) return {cadd(xk.re, xk.im), csub(xk.re, xk.im)};
    const cpx2 xmc = cconj(pair(r0[WH - k], r0[RP + WH - k]));
    const cpx2 E = cadd(xk, xmc);
    const float4 t = __ldg(&twW4[k]);
    const cpx2 O = cmulc_b(csub(xk, xmc), make_float2(t.x, t.y), make_float2(t.z, t.w));
    return {csub(E.re, O.im), cadd(E.im, O.re)};
  };
  bool kept = false;
  auto thr_st = [&](int i, int p, cpx2 v) {
    v.re.x = apply_thresh(v.re.x, th, mode);
    v.re.y = apply_thresh(v.re.y, th, mode);
    v.im.x = apply_thresh(v.im.x, th, mode);
    v.im.y = apply_thresh(v.im.y, th, mode);
    kept |= (v.re.x != 0.0f) | (v.re.y != 0.0f) | (v.im.x != 0.0f) | (v.im.y != 0.0f);
    D[i * NP + p] = v;
  };
  using Plan = typename RowPlanP<WH>::type;
  block_fft_hook_ip_plan<WH, NP, T, +1, Plan>(D, twWh4, ld, thr_st);
  // a tile whose coefficients all threshold to zero has a zero transform
  if (!__syncthreads_or(kept)) {
    store_zero_rows<WH, RS, T>(dst_base + job.dst + off);
    return;
  }
  // R2C of the thresholded rows, the last pass back to the row-major layout
  auto ldd = [&](int i, int p) -> cpx2 { return D[i * NP + p]; };
  auto st_rm = [&](int i, int p, cpx2 v) {
    A[2 * p * RP + i] = lane0(v);
    A[(2 * p + 1) * RP + i] = lane1(v);
  };
  block_fft_hook_ip_plan<WH, NP, T, -1, Plan>(D, twWh4, ldd, st_rm);
  // post-processing (see r2c_post) fused with the store along the rows:
  // X[k] = E + w^k O, E = (Z[k] + conj(Z[WH-k]))/2, O = (Z[k] - conj(Z[WH-k]))/(2i)
  float2* dst = dst_base + job.dst + off;
#pragma unroll 2
  for (int e = threadIdx.x; e < WH * NP; e += T) {
    const int k = e % WH, p = e / WH;
    const float2* r0 = A + 2 * p * RP;
    const cpx2 zk = pair(r0[k], r0[RP + k]);
    cpx2 out;
    if (k == 0) {
      out = {cadd(zk.re, zk.im), csub(zk.re, zk.im)};
    } else {
      const cpx2 zmc = cconj(pair(r0[WH - k], r0[RP + WH - k]));
      const cpx2 E = cscale(cadd(zk, zmc), 0.5f);
      const cpx2 d = cscale(csub(zk, zmc), 0.5f);
      const float4 t = __ldg(&twW4[k]);
      out = cadd(E, cmul_b(cpx2{d.im, neg2(d.re)}, make_float2(t.x, t.y), make_float2(t.z, t.w)));
    }
    dst[(size_t)(2 * p) * WH + k] = lane0(out);
    dst[(size_t)(2 * p + 1) * WH + k] = lane1(out);
  }
}

// Band maxima (thresh.m's opt == 1 maximum with a zero threshold): C2R of the
// CTA's rows of one band, then max |c| over them into bits[job.th_index] as
// the bit pattern of a non-negative float (atomicMax; bits zeroed first).
template <int WH>
__global__ void __launch_bounds__(RowCfg<WH>::T, RowCfg<WH>::MINB) k_rows_max(const RowJob* __restrict__ jobs, int n_active,
                                                             const float2* src_base,
                                                             const float2* __restrict__ twWh,
                                                             const float2* __restrict__ twW,
                                                             unsigned* __restrict__ bits) {
  using C = RowCfg<WH>;
  extern __shared__ float2 smem[];
  float2* A = smem;
  const RowJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const size_t off = (size_t)blockIdx.x * C::RS * WH;
  fetch_rows_rm<WH, C::RS, C::T>(A, src_base + job.src + off);
  cp_async_wait_all();
  __syncthreads();
  block_fft_hook_ip<WH, C::RS, C::T, +1>(A, twWh, C2RPreLdRM<WH>{A, twW}, SmemSt<C::RS>{A});
  __syncthreads();
  float m = 0.0f;
  for (int e = threadIdx.x; e < WH * C::RS; e += C::T) {  // SmemSt wrote (i, s) at i * RS + s
    const float2 v = A[e];
    m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(&bits[job.th_index], __float_as_uint(m));
}

// Backward band row pass (adjoint of the threshold step, rows of one band):
// coefficients c = C2R(Qc) are recomputed, g = C2R(Qg) is the gradient w.r.t.
// the thresholded coefficients; out = R2C(g * 1[|c| > t]) replaces Qg, and
// each CTA writes its share of d loss / d t = -sum g sign(c) 1[|c| > t] (soft).
template <int WH>
__global__ void __launch_bounds__(RowCfg<WH>::T) k_rows_backward(const RowJob* __restrict__ jobs, int n_active,
                                                                  const float2* src_base, float2* dst_base,
                                                                  const float2* __restrict__ twWh,
                                                                  const float2* __restrict__ twW,
                                                                  const float* __restrict__ tau, int mode,
                                                                  float* __restrict__ partials, size_t pstride) {
  using C = RowCfg<WH>;
  extern __shared__ float2 smem[];
  // three buffers of the padded row-major size (the dense layouts fit in them)
  constexpr int BUF = C::RS * (WH + 2);
  float2 *A = smem, *B = smem + BUF, *Cb = smem + 2 * BUF;
  __shared__ float red[32];
  const RowJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const float th = tau[job.th_index];
  const size_t off = (size_t)blockIdx.x * C::RS * WH;
  fetch_rows_rm<WH, C::RS, C::T>(A, src_base + job.src + off);
  fetch_rows_rm<WH, C::RS, C::T>(Cb, dst_base + job.dst + off);
  cp_async_wait_all();
  __syncthreads();
  // coefficients c = C2R(Qc) (pre-processing in the first pass), noting
  // whether any passes the threshold
  float2* const Xc = fft_hook_target<WH>(A, B);
  bool kept = false;
  auto c_st = [&](int i, int sq, float2 c) {
    kept |= (fabsf(c.x) > th) | (fabsf(c.y) > th);
    Xc[i * C::RS + sq] = c;
  };
  block_fft_hook<WH, C::RS, C::T, +1>(A, B, twWh, C2RPreLdRM<WH>{A, twW}, c_st);
  // no coefficient of the tile passes: the masked gradient, its transform and
  // the tile's share of d loss / d t are zero
  if (!__syncthreads_or(kept)) {
    if (threadIdx.x == 0) partials[(size_t)job.th_index * pstride + (size_t)job.item * gridDim.x + blockIdx.x] = 0.0f;
    store_zero_rows<WH, C::RS, C::T>(dst_base + job.dst + off);
    return;
  }
  // gradient g = C2R(Qg), masked by 1[|c| > t] in the last pass, which also
  // accumulates this thread's share of -sum g sign(c) 1[|c| > t] (soft)
  float2* const S = (Xc == A) ? B : A;
  float2* const Xg = fft_hook_target<WH>(Cb, S);
  float part = 0.0f;
  auto mask_st = [&](int i, int sq, float2 g) {
    const float2 c = Xc[i * C::RS + sq];
    const bool kx = fabsf(c.x) > th, ky = fabsf(c.y) > th;
    if (mode == THRESH_SOFT) {
      if (kx) part -= (c.x > 0.0f ? g.x : -g.x);
      if (ky) part -= (c.y > 0.0f ? g.y : -g.y);
    }
    Xg[i * C::RS + sq] = make_float2(kx ? g.x : 0.0f, ky ? g.y : 0.0f);
  };
  block_fft_hook<WH, C::RS, C::T, +1>(Cb, S, twWh, C2RPreLdRM<WH>{Cb, twW}, mask_st);
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (C::T >> 5) ? red[threadIdx.x] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0)
      partials[(size_t)job.th_index * pstride + (size_t)job.item * gridDim.x + blockIdx.x] = v;
  }
  // R2C of the masked gradient; post-processing fused with the store
  float2* const Y = (Xg == Cb) ? S : Cb;
  float2* const Z = fft_hook_target<WH>(Xg, Y);
  block_fft_hook<WH, C::RS, C::T, -1>(Xg, Y, twWh, SmemLd<C::RS>{Xg}, SmemStRM<WH>{Z});
  r2c_post_store_rm<WH, C::RS, C::T>(dst_base + job.dst + off, Z, twW);
}

// ---------------------------------------------------------------------------
// Column kernels.  grid = (WH / CS, njobs).
// ---------------------------------------------------------------------------

// Wk .* Z for the analysis, with the packed DC/Nyquist column's
// Z'[u] = P[u] Z[u] + M[u] conj(Z[-u]) (src, spec: column group origin)
template <int H>
struct AnalysisLd {
  const float2* src;
  const float2* spec;
  const float2* m0;
  int WH;
  bool dc;  // the group holds column 0
  __device__ __forceinline__ float2 operator()(int i, int s) const {
    const size_t g = (size_t)i * WH + s;
    float2 r = cmul(__ldg(&spec[g]), src[g]);
    if (dc && s == 0) {
      const float2 zm = src[(size_t)((H - i) % H) * WH];
      r = cadd(r, cmul(__ldg(&m0[i]), cconj(zm)));
    }
    return r;
  }
};

// plain column FFT (forward or inverse) src -> dst, straight from and to
// global memory through the first and last passes
template <int H, int DIR>
__global__ void __launch_bounds__(ColCfg<H>::T, ColCfg<H>::MINB) k_cols(const ColJob* __restrict__ jobs, int n_active, int WH,
                                                        const float2* src_base, float2* dst_base,
                                                        const float2* __restrict__ twH) {
  using C = ColCfg<H>;
  extern __shared__ float2 smem[];
  float2 *A = smem, *B = smem + (size_t)H * C::LD;
  const ColJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const int col0 = blockIdx.x * C::CS;
  (void)B;
  block_fft_hook_ip<H, C::CS, C::T, DIR>(A, twH, ColGlobalLd{src_base + job.src + col0, WH},
                                         ColGlobalSt{dst_base + job.dst + col0, WH});
}

// analysis band: dst = colIFFT( Wk .* src ), src = fully transformed level spectrum
template <int H>
__global__ void __launch_bounds__(ColCfg<H>::T, ColCfg<H>::MINB) k_band_analysis(const ColJob* __restrict__ jobs, int n_active,
                                                                 int WH, const float2* src_base, float2* dst_base,
                                                                 const float2* __restrict__ spec_base,
                                                                 const float2* __restrict__ twH) {
  using C = ColCfg<H>;
  extern __shared__ float2 smem[];
  float2 *A = smem, *B = smem + (size_t)H * C::LD;
  const ColJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const int col0 = blockIdx.x * C::CS;
  (void)B;
  block_fft_hook_ip<H, C::CS, C::T, +1>(
      A, twH,
      AnalysisLd<H>{src_base + job.src + col0, spec_base + job.spec + col0, spec_base + job.m0, WH, col0 == 0},
      ColGlobalSt{dst_base + job.dst + col0, WH});
}

// analysis of all bands of one level: dst_k = colIFFT( Wk .* Y ) for the
// job.nbands consecutive bands (spectra, side arrays and outputs at k *
// band_stride, k * H, k * band_stride).  The CTA's column group of Y is
// staged once; each band's filter columns stream into a staging buffer with
// cp.async while the previous band is transformed.
template <int H>
__global__ void __launch_bounds__(AnaCfg<H>::T, AnaCfg<H>::MINB) k_band_analysis_ml(const ColJob* __restrict__ jobs, int n_active,
                                                                  int WH, const float2* src_base, float2* dst_base,
                                                                  const float2* __restrict__ spec_base,
                                                                  size_t band_stride,
                                                                  const float2* __restrict__ twH) {
  using C = AnaCfg<H>;
  constexpr int CS = C::CS, CH = CS / 2;  // 16-byte chunks per row of the column group
  extern __shared__ float2 smem[];
  float2* A = smem;            // transform, in place
  float2* Y = A + H * CS;      // level spectrum column group [row][column]
  float2* Wb = Y + H * CS;     // staged filter spectrum of the current band
  const ColJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const int col0 = blockIdx.x * CS;
  const bool dc = col0 == 0;
  auto stage = [&](float2* dst, const float2* src) {
    for (int e = threadIdx.x; e < H * CH; e += C::T) {
      const int i = e / CH, c = e - (e / CH) * CH;
      cp_async16(dst + i * CS + 2 * c, src + (size_t)i * WH + 2 * c);
    }
  };
  stage(Y, src_base + job.src + col0);
  stage(Wb, spec_base + job.spec + col0);
  cp_async_commit();
  for (int k = 0; k < job.nbands; k++) {
    cp_async_wait_all();
    __syncthreads();
    const float2* m0 = spec_base + job.m0 + (size_t)k * H;
    // Wk .* Y, with the packed DC/Nyquist column's M term (see AnalysisLd)
    auto ld = [&](int i, int s) -> float2 {
      float2 r = cmul(Wb[i * CS + s], Y[i * CS + s]);
      if (dc && s == 0) r = cadd(r, cmul(__ldg(&m0[i]), cconj(Y[((H - i) % H) * CS])));
      return r;
    };
    auto next = [&]() {
      if (k + 1 < job.nbands) {
        stage(Wb, spec_base + job.spec + (size_t)(k + 1) * band_stride + col0);
        cp_async_commit();
      }
    };
    block_fft_hook_ip<H, CS, C::T, +1>(A, twH, ld, ColGlobalSt{dst_base + job.dst + (size_t)k * band_stride + col0, WH},
                                      next);
  }
}

// synthesis: dst = colIFFT( sum_k conj(Wk) .* colFFT(src_k) ) over job.nbands
// bands stored at src + k * band_stride, spectra at spec + k * band_stride,
// side arrays at m0 + k * H.  Each band's column FFT runs in place in A; its
// last pass accumulates conj(Wk) .* X straight into the running sum in S
// (each output element has one owner thread per pass, and passes are
// separated by barriers).  The packed DC/Nyquist column also needs X[-u]:
// the CTA holding column 0 keeps that column in D and adds
// conj(M[u] X[-u]) after the transform.
template <int H>
__global__ void __launch_bounds__(SynCfg<H>::T, SynCfg<H>::MINB) k_band_synthesis(const ColJob* __restrict__ jobs, int n_active,
                                                                  int WH, const float2* src_base, float2* dst_base,
                                                                  const float2* __restrict__ spec_base,
                                                                  size_t band_stride,
                                                                  const float2* __restrict__ twH) {
  using C = SynCfg<H>;
  extern __shared__ float2 smem[];
  float2 *A = smem, *S = smem + (size_t)H * C::LD, *D = smem + 2 * (size_t)H * C::LD;
  float2* P = D + H;  // staging: the band's H x CS column group, [row][column]
  const ColJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const int col0 = blockIdx.x * C::CS;
  const bool dc = col0 == 0;
  // band k's column group -> P with 16-byte cp.async (rows are CS float2 = 64 or 32 contiguous bytes)
  auto prefetch = [&](int k) {
    constexpr int CH = C::CS / 2;
    const float2* src = src_base + job.src + (size_t)k * band_stride + col0;
    for (int e = threadIdx.x; e < H * CH; e += C::T) {
      const int i = e / CH, c = e - (e / CH) * CH;
      cp_async16(P + i * C::CS + 2 * c, src + (size_t)i * WH + 2 * c);
    }
    cp_async_commit();
  };
  prefetch(0);
  for (int k = 0; k < job.nbands; k++) {
    const float2* spec = spec_base + job.spec + k * band_stride + col0;
    const bool first = k == 0;
    auto acc_st = [&](int i, int sq, float2 z) {
      const float2 p = cmulc(z, __ldg(&spec[(size_t)i * WH + sq]));
      float2* t = &S[i * C::LD + sq];
      *t = first ? p : cadd(*t, p);
      if (dc && sq == 0) D[i] = z;
    };
    cp_async_wait_all();
    __syncthreads();
    // the first pass reads band k from P; once it has, band k + 1 starts streaming in
    auto next = [&]() {
      if (k + 1 < job.nbands) prefetch(k + 1);
    };
    block_fft_hook_ip<H, C::CS, C::T, -1>(A, twH, SmemLd<C::CS>{P}, acc_st, next);
    if (dc) {
      for (int i = threadIdx.x; i < H; i += C::T) {
        const float2 m = __ldg(&spec_base[job.m0 + (size_t)k * H + i]);
        S[i * C::LD] = cadd(S[i * C::LD], cconj(cmul(m, D[(H - i) % H])));  // conj(M) conj(z[-u])
      }
      __syncthreads();
    }
  }
  block_fft_hook_ip<H, C::CS, C::T, +1>(S, twH, SmemLd<C::CS>{S}, ColGlobalSt{dst_base + job.dst + col0, WH});
}

// ---------------------------------------------------------------------------
// The two column kernels above on split-complex column pairs (cpx2): columns
// 2p and 2p + 1 of the CTA's group share a thread's registers, so the
// spectrum products, twiddle multiplies and index arithmetic run as FP32x2
// instructions for two columns, a thread holds half the butterflies of the
// one-column form (the same registers), and global stores move 16 bytes.
// The staging buffers keep the [row][column] float2 layout of global memory;
// the transform buffers hold [row][pair] cpx2.  twH4: the column twiddle
// table with each entry as its broadcast pairs.
// ---------------------------------------------------------------------------
template <int H>
__global__ void __launch_bounds__(AnaCfg<H>::T, AnaCfg<H>::MINB)
    k_band_analysis_ml_p(const ColJob* __restrict__ jobs, int n_active, int WH, const float2* src_base,
                         float2* dst_base, const float2* __restrict__ spec_base, size_t band_stride,
                         const float2* __restrict__ twH4) {
  using C = AnaCfg<H>;
  constexpr int CS = C::CS, CH = CS / 2, NP = CS / 2;
  extern __shared__ float2 smem[];
  cpx2* A = reinterpret_cast<cpx2*>(smem);  // transform [row][pair], in place
  float2* Y = smem + H * CS;                // level spectrum column group [row][column]
  float2* Wb = Y + H * CS;                  // staged filter spectrum of the current band
  const ColJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const int col0 = blockIdx.x * CS;
  const bool dc = col0 == 0;
  auto stage = [&](float2* dst, const float2* src) {
    for (int e = threadIdx.x; e < H * CH; e += C::T) {
      const int i = e / CH, c = e - (e / CH) * CH;
      cp_async16(dst + i * CS + 2 * c, src + (size_t)i * WH + 2 * c);
    }
  };
  stage(Y, src_base + job.src + col0);
  stage(Wb, spec_base + job.spec + col0);
  cp_async_commit();
  for (int k = 0; k < job.nbands; k++) {
    cp_async_wait_all();
    __syncthreads();
    const float2* m0 = spec_base + job.m0 + (size_t)k * H;
    // Wk .* Y for two columns, the packed DC/Nyquist column's M term on lane 0 of pair 0
    auto ld = [&](int i, int p) -> cpx2 {
      cpx2 r = cmul_pp(ld_pair(Wb + i * CS + 2 * p), ld_pair(Y + i * CS + 2 * p));
      if (dc && p == 0) {
        const float2 a = cmul(__ldg(&m0[i]), cconj(Y[((H - i) % H) * CS]));
        r.re.x += a.x;
        r.im.x += a.y;
      }
      return r;
    };
    auto next = [&]() {
      if (k + 1 < job.nbands) {
        stage(Wb, spec_base + job.spec + (size_t)(k + 1) * band_stride + col0);
        cp_async_commit();
      }
    };
    float2* dst = dst_base + job.dst + (size_t)k * band_stride + col0;
    auto st = [&](int i, int p, cpx2 v) { st_pair(dst + (size_t)i * WH + 2 * p, v); };
    block_fft_hook_ip<H, NP, C::T, +1>(A, twH4, ld, st, next);
  }
}

template <int H>
__global__ void __launch_bounds__(SynCfg<H>::T, SynCfg<H>::MINB)
    k_band_synthesis_p(const ColJob* __restrict__ jobs, int n_active, int WH, const float2* src_base,
                       float2* dst_base, const float2* __restrict__ spec_base, size_t band_stride,
                       const float2* __restrict__ twH4) {
  using C = SynCfg<H>;
  constexpr int CS = C::CS, NP = CS / 2;
  extern __shared__ float2 smem[];
  cpx2* A = reinterpret_cast<cpx2*>(smem);                  // transform [row][pair]
  cpx2* S = reinterpret_cast<cpx2*>(smem + (size_t)H * CS);  // running band sum [row][pair]
  float2* D = smem + 2 * (size_t)H * CS;                     // column 0 of the band's transform
  float2* P = D + H;                                         // staging: the band's column group [row][column]
  const ColJob job = jobs[blockIdx.y];
  if (job.item >= n_active) return;
  const int col0 = blockIdx.x * CS;
  const bool dc = col0 == 0;
  auto prefetch = [&](int k) {
    constexpr int CH = CS / 2;
    const float2* src = src_base + job.src + (size_t)k * band_stride + col0;
    for (int e = threadIdx.x; e < H * CH; e += C::T) {
      const int i = e / CH, c = e - (e / CH) * CH;
      cp_async16(P + i * CS + 2 * c, src + (size_t)i * WH + 2 * c);
    }
    cp_async_commit();
  };
  prefetch(0);
  for (int k = 0; k < job.nbands; k++) {
    const float2* spec = spec_base + job.spec + k * band_stride + col0;
    const bool first = k == 0;
    auto acc_st = [&](int i, int p, cpx2 z) {
      const float4 w = __ldg(reinterpret_cast<const float4*>(spec + (size_t)i * WH + 2 * p));
      const cpx2 q = cmulc_pp(z, pair(make_float2(w.x, w.y), make_float2(w.z, w.w)));
      cpx2* t = &S[i * NP + p];
      *t = first ? q : cadd(*t, q);
      if (dc && p == 0) D[i] = lane0(z);
    };
    cp_async_wait_all();
    __syncthreads();
    auto next = [&]() {
      if (k + 1 < job.nbands) prefetch(k + 1);
    };
    auto ldp = [&](int i, int p) -> cpx2 { return ld_pair(P + i * CS + 2 * p); };
    block_fft_hook_ip<H, NP, C::T, -1>(A, twH4, ldp, acc_st, next);
    if (dc) {
      for (int i = threadIdx.x; i < H; i += C::T) {
        const float2 m = __ldg(&spec_base[job.m0 + (size_t)k * H + i]);
        const float2 a = cconj(cmul(m, D[(H - i) % H]));  // conj(M) conj(z[-u])
        S[i * NP].re.x += a.x;
        S[i * NP].im.x += a.y;
      }
      __syncthreads();
    }
  }
  float2* dst = dst_base + job.dst + col0;
  block_fft_hook_ip<H, NP, C::T, +1>(
      S, twH4, [&](int i, int p) -> cpx2 { return S[i * NP + p]; },
      [&](int i, int p, cpx2 v) { st_pair(dst + (size_t)i * WH + 2 * p, v); });
}

// ---------------------------------------------------------------------------
// Host-side launchers, dispatched on the (compile-time) transform lengths.
// The dynamic shared-memory opt-in is done once per device and kernel by the
// prepare_* calls (plan creation), never on the launch path.
// ---------------------------------------------------------------------------

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
int row_tile(int wh) { return wh >= 1024 ? 4 : 8; }
int col_tile(int h) { return h >= 768 ? 4 : 8; }

template <typename KernelT>
static cudaError_t opt_in(KernelT k, size_t bytes) {
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  return e;
}

cudaError_t prepare_row_kernels(int wh) {
  switch (wh) {
#define CASE(n)                                                               \
  case n: {                                                                   \
    constexpr size_t sm = RowCfg<n>::smem();                                  \
    cudaError_t e = opt_in(k_rows_fwd<n>, sm);                                \
    if (e == cudaSuccess) e = opt_in(k_rows_inv<n>, sm);                      \
    if (e == cudaSuccess) e = opt_in(k_rows_thresh<n>, sm);                   \
    if (e == cudaSuccess) e = opt_in(k_rows_thresh<n, 2 * RowCfg<n>::RS>, RowTile<n, 2 * RowCfg<n>::RS>::smem()); \
    if (e == cudaSuccess) e = opt_in(k_rows_thresh_p<n, RowCfg<n>::RS>, RowTileP<n, RowCfg<n>::RS>::smem()); \
    if (e == cudaSuccess) e = opt_in(k_rows_thresh_p<n, 2 * RowCfg<n>::RS>, RowTileP<n, 2 * RowCfg<n>::RS>::smem()); \
    if (e == cudaSuccess) e = opt_in(k_rows_max<n>, sm);                      \
    if (e == cudaSuccess) e = opt_in(k_rows_backward<n>, 3 * RowCfg<n>::smem_rm()); \
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
    if (e == cudaSuccess) e = opt_in(k_band_analysis_ml<n>, AnaCfg<n>::smem()); \
    if (e == cudaSuccess) e = opt_in(k_band_synthesis<n>, SynCfg<n>::smem());  \
    if (e == cudaSuccess) e = opt_in(k_band_analysis_ml_p<n>, AnaCfg<n>::smem()); \
    if (e == cudaSuccess) e = opt_in(k_band_synthesis_p<n>, SynCfg<n>::smem());  \
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
    constexpr size_t sm = RowCfg<n>::smem() / 2; /* in place: one buffer */            \
    dim3 grid(H / RowCfg<n>::RS, njobs);                                               \
    /* one tile staged row-major, rows padded to WH + 2 */                           \
    constexpr size_t smr = RowCfg<n>::smem_rm();                                       \
    (void)sm;                                                                          \
    if (op == RowOp::Fwd)                                                              \
      k_rows_fwd<n><<<grid, RowCfg<n>::T, smr, st>>>(jobs, n_active, sb, db, twWh, twW);             \
    else if (op == RowOp::Inv)                                                         \
      k_rows_inv<n><<<grid, RowCfg<n>::T, smr, st>>>(jobs, n_active, sb, db, twWh, twW);             \
    else                                                                               \
      k_rows_thresh<n><<<grid, RowCfg<n>::T, smr, st>>>(jobs, n_active, sb, db, twWh, twW, thr, mode); \
    return cudaGetLastError();                                                         \
  }
    NSST_ROW_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_rows_thresh(const RowJob* jobs, int njobs, int n_active, int H, int W, const void* src_base,
                               void* dst_base, const float2* twWh, const float2* twW, const float* thr, int mode,
                               int tile_mult, cudaStream_t st, bool packed, const float4* twWh4,
                               const float4* twW4) {
  if (tile_mult == 1 && !packed)
    return launch_rows(RowOp::Thresh, jobs, njobs, n_active, H, W, src_base, dst_base, twWh, twW, thr, mode, st);
  if (tile_mult != 1 && tile_mult != 2) return cudaErrorInvalidValue;
  const int WH = W / 2;
  if (njobs == 0) return cudaSuccess;
  const float2* sb = static_cast<const float2*>(src_base);
  float2* db = static_cast<float2*>(dst_base);
  if (packed) {
    if (!twWh4 || !twW4) return cudaErrorInvalidValue;
    switch (WH) {
#define CASE(n)                                                                                            \
  case n: {                                                                                                \
    constexpr int R1 = RowCfg<n>::RS, R2 = 2 * RowCfg<n>::RS;                                              \
    if (tile_mult == 1) {                                                                                  \
      using Tl = RowTileP<n, R1>;                                                                          \
      count_launch();                                                                                      \
      k_rows_thresh_p<n, R1><<<dim3(H / R1, njobs), Tl::T, Tl::smem(), st>>>(                              \
          jobs, n_active, sb, db, reinterpret_cast<const float2*>(twWh4), twW4, thr, mode);                \
    } else {                                                                                               \
      if (H % R2 != 0) return cudaErrorInvalidValue;                                                       \
      using Tl = RowTileP<n, R2>;                                                                          \
      count_launch();                                                                                      \
      k_rows_thresh_p<n, R2><<<dim3(H / R2, njobs), Tl::T, Tl::smem(), st>>>(                              \
          jobs, n_active, sb, db, reinterpret_cast<const float2*>(twWh4), twW4, thr, mode);                \
    }                                                                                                      \
    return cudaGetLastError();                                                                             \
  }
      NSST_ROW_SIZES(CASE)
#undef CASE
      default:
        return cudaErrorInvalidValue;
    }
  }
  count_launch();
  switch (WH) {
#define CASE(n)                                                                                         \
  case n: {                                                                                             \
    constexpr int RS2 = 2 * RowCfg<n>::RS;                                                              \
    using Tl = RowTile<n, RS2>;                                                                         \
    if (H % RS2 != 0) return cudaErrorInvalidValue;                                                     \
    k_rows_thresh<n, RS2><<<dim3(H / RS2, njobs), Tl::T, Tl::smem(), st>>>(jobs, n_active, sb, db, twWh, twW, \
                                                                         thr, mode);                    \
    return cudaGetLastError();                                                                          \
  }
    NSST_ROW_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_rows_max(const RowJob* jobs, int njobs, int n_active, int H, int W, const void* src_base,
                            const float2* twWh, const float2* twW, unsigned* bits, cudaStream_t st) {
  const int WH = W / 2;
  if (njobs == 0) return cudaSuccess;
  count_launch();
  const float2* sb = static_cast<const float2*>(src_base);
  switch (WH) {
#define CASE(n)                                                                                   \
  case n: {                                                                                       \
    constexpr size_t sm = RowCfg<n>::smem_rm();                                                   \
    k_rows_max<n><<<dim3(H / RowCfg<n>::RS, njobs), RowCfg<n>::T, sm, st>>>(jobs, n_active, sb, twWh, twW, bits); \
    return cudaGetLastError();                                                                    \
  }
    NSST_ROW_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_rows_backward(const RowJob* jobs, int njobs, int n_active, int H, int W, const void* src_base,
                                 void* dst_base, const float2* twWh, const float2* twW, const float* tau, int mode,
                                 float* partials, size_t pstride, cudaStream_t st) {
  const int WH = W / 2;
  if (njobs == 0) return cudaSuccess;
  count_launch();
  const float2* sb = static_cast<const float2*>(src_base);
  float2* db = static_cast<float2*>(dst_base);
  switch (WH) {
#define CASE(n)                                                                                      \
  case n: {                                                                                          \
    constexpr size_t sm = 3 * RowCfg<n>::smem_rm();                                                  \
    dim3 grid(H / RowCfg<n>::RS, njobs);                                                             \
    k_rows_backward<n><<<grid, RowCfg<n>::T, sm, st>>>(jobs, n_active, sb, db, twWh, twW, tau, mode, \
                                                      partials, pstride);                           \
    return cudaGetLastError();                                                                       \
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
    if (op == ColOp::Fwd)  /* in-place transforms: one buffer */                                     \
      k_cols<n, -1><<<grid, ColCfg<n>::T, sm / 2, st>>>(jobs, n_active, WH, src_base, dst_base, twH);               \
    else if (op == ColOp::Inv)                                                                        \
      k_cols<n, 1><<<grid, ColCfg<n>::T, sm / 2, st>>>(jobs, n_active, WH, src_base, dst_base, twH);                \
    else if (op == ColOp::Analysis)                                                                   \
      k_band_analysis<n><<<grid, ColCfg<n>::T, sm / 2, st>>>(jobs, n_active, WH, src_base, dst_base, spec_base,     \
                                                         twH);                                        \
    else if (op == ColOp::AnalysisLevelPairs)                                                         \
      k_band_analysis_ml_p<n><<<grid, AnaCfg<n>::T, AnaCfg<n>::smem(), st>>>(jobs, n_active, WH, src_base,          \
                                                                          dst_base, spec_base, band_stride, twH); \
    else if (op == ColOp::SynthesisPairs)                                                             \
      k_band_synthesis_p<n><<<grid, SynCfg<n>::T, SynCfg<n>::smem(), st>>>(jobs, n_active, WH, src_base, dst_base, \
                                                                        spec_base, band_stride, twH); \
    else if (op == ColOp::AnalysisLevel)                                                              \
      k_band_analysis_ml<n><<<grid, AnaCfg<n>::T, AnaCfg<n>::smem(), st>>>(jobs, n_active, WH, src_base, dst_base, \
                                                                        spec_base, band_stride, twH); \
    else                                                                                              \
      k_band_synthesis<n><<<grid, SynCfg<n>::T, SynCfg<n>::smem(), st>>>(jobs, n_active, WH, src_base, dst_base,   \
                                                                       spec_base,                     \
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
