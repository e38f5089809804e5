// Kernels of the 3-D path: the Fourier-domain band-pass pyramid
// (PyrNDDec_mm.m / PyrNDRec_mm.m, Pyr_mode 1.5) and the CONVNFFT-based
// directional filtering with threshold and band sum (ShDecThRec_cuda.cpp:178-335,
// convnfft.m 'same', ThresholdShCoeff.m, ShRec.m).
//
// Volumes are complex float2 (or real float) arrays d0 x d1 x d2, axis 2
// contiguous.  Spectra follow the reference literally: full complex FFTs,
// the half spectrum along the last axis (ccsym 'c') for the pyramid steps, and
// an explicit conjugate extension (ccsym 'e') before each inverse.
#include "fft_core.cuh"
#include "internal.h"

namespace nsst {

// ---------------------------------------------------------------------------
// Elementwise volume kernels (grid-stride over one item, blockIdx.y = item)
// ---------------------------------------------------------------------------
#define V3_LOOP(total) \
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < (total); idx += (size_t)gridDim.x * blockDim.x)

// out (complex L0 x L1 x L2) = zero-padded real in (m0 x m1 x m2) at the origin
__global__ void k_pad_real(const float* __restrict__ in, size_t in_stride, float2* __restrict__ out,
                           size_t out_stride, int m0, int m1, int m2, int L0, int L1, int L2) {
  const float* src = in + blockIdx.y * in_stride;
  float2* dst = out + blockIdx.y * out_stride;
  const size_t total = (size_t)L0 * L1 * L2;
  V3_LOOP(total) {
    const int z = (int)(idx % L2);
    const size_t r = idx / L2;
    const int y = (int)(r % L1), x = (int)(r / L1);
    float v = 0.f;
    if (x < m0 && y < m1 && z < m2) v = src[((size_t)x * m1 + y) * m2 + z];
    dst[idx] = make_float2(v, 0.f);
  }
}

// out (complex d0 x d1 x d2) = in (real n0 x n1 x n2) extended by repeating its
// last plane along each axis (MarshalData.m:10-20)
__global__ void k_pad_edge(const float* __restrict__ in, size_t in_stride, float2* __restrict__ out,
                           size_t out_stride, int n0, int n1, int n2, int d0, int d1, int d2) {
  const float* src = in + blockIdx.y * in_stride;
  float2* dst = out + blockIdx.y * out_stride;
  const size_t total = (size_t)d0 * d1 * d2;
  V3_LOOP(total) {
    const int z = (int)(idx % d2);
    const size_t r = idx / d2;
    const int y = (int)(r % d1), x = (int)(r / d1);
    const int xs = x < n0 ? x : n0 - 1, ys = y < n1 ? y : n1 - 1, zs = z < n2 ? z : n2 - 1;
    dst[idx] = make_float2(src[((size_t)xs * n1 + ys) * n2 + zs], 0.f);
  }
}

// out (real m0 x m1 x m2) = real part of in (complex L0 x L1 x L2) at offset o
__global__ void k_crop_real(const float2* __restrict__ in, size_t in_stride, float* __restrict__ out,
                            size_t out_stride, int m0, int m1, int m2, int L1, int L2, int o0, int o1, int o2,
                            float scale) {
  const float2* src = in + blockIdx.y * in_stride;
  float* dst = out + blockIdx.y * out_stride;
  const size_t total = (size_t)m0 * m1 * m2;
  V3_LOOP(total) {
    const int z = (int)(idx % m2);
    const size_t r = idx / m2;
    const int y = (int)(r % m1), x = (int)(r / m1);
    dst[idx] = src[((size_t)(x + o0) * L1 + (y + o1)) * L2 + (z + o2)].x * scale;
  }
}

// ccsym(X, 3, 'c'): half along the last axis, h2 = d2/2 + 1
__global__ void k_half(const float2* __restrict__ in, size_t in_stride, float2* __restrict__ out, size_t out_stride,
                       int d0, int d1, int d2) {
  const float2* src = in + blockIdx.y * in_stride;
  float2* dst = out + blockIdx.y * out_stride;
  const int h2 = d2 / 2 + 1;
  const size_t total = (size_t)d0 * d1 * h2;
  V3_LOOP(total) {
    const int z = (int)(idx % h2);
    const size_t r = idx / h2;
    dst[idx] = src[r * d2 + z];
  }
}

// ccsym(X, 3, 'e'): full spectrum d0 x d1 x d2 from the half, conjugate mirror
// for z > d2/2 at (-x, -y, d2 - z)
__global__ void k_conj_extend(const float2* __restrict__ in, size_t in_stride, float2* __restrict__ out,
                              size_t out_stride, int d0, int d1, int d2) {
  const float2* src = in + blockIdx.y * in_stride;
  float2* dst = out + blockIdx.y * out_stride;
  const int h2 = d2 / 2 + 1;
  const size_t total = (size_t)d0 * d1 * d2;
  V3_LOOP(total) {
    const int z = (int)(idx % d2);
    const size_t r = idx / d2;
    const int y = (int)(r % d1), x = (int)(r / d1);
    float2 v;
    if (z < h2) {
      v = src[((size_t)x * d1 + y) * h2 + z];
    } else {
      const int xm = x ? d0 - x : 0, ym = y ? d1 - y : 0;
      const float2 c = src[((size_t)xm * d1 + ym) * h2 + (d2 - z)];
      v = make_float2(c.x, -c.y);
    }
    dst[idx] = v;
  }
}

// Window factor of one axis at parent index p (nr = FFT length of that axis,
// K = last window index, v = window values 0..K); full axes mirror at nr - p,
// the last (half) axis does not.  Returns -1 outside the window's support.
__device__ __forceinline__ float win_at(const float* __restrict__ v, int K, int nr, int p, bool half_axis) {
  if (p <= K) return v[p];
  if (!half_axis && p >= nr - K) return v[nr - p];
  return -1.0f;
}

// PrySDdec_onestep.m:82-125 on half spectra.  Hp (in place over Xh) and Lp
// (small half spectrum, szLp = szF/D per axis, last axis szLp/2+1).  Lp is
// gathered with the reference's write order: where the positive and the
// negative parts of a full axis land on the same small index, the negative
// part (written last by the subscripted assignment) wins.
__global__ void k_pyr_dec_hp(float2* __restrict__ Xh, size_t stride, int d0, int d1, int h2, PyrWin w) {
  float2* X = Xh + blockIdx.y * stride;
  const size_t total = (size_t)d0 * d1 * h2;
  V3_LOOP(total) {
    const int z = (int)(idx % h2);
    const size_t r = idx / h2;
    const int y = (int)(r % d1), x = (int)(r / d1);
    const float a = win_at(w.v0, w.K[0], w.nr[0], x, false);
    const float b = win_at(w.v1, w.K[1], w.nr[1], y, false);
    const float c = win_at(w.v2, w.K[2], w.nr[2], z, true);
    if (a >= 0.f && b >= 0.f && c >= 0.f) {
      const float lf = a * b * c;
      const float s = sqrtf(fmaxf(1.0f - lf * lf, 0.0f));
      float2 v = X[idx];
      X[idx] = make_float2(v.x * s, v.y * s);
    }
  }
}

__device__ __forceinline__ int small_to_parent(int s, int K, int nr, int nsmall, bool half_axis) {
  if (!half_axis && s >= nsmall - K) return s + nr - nsmall;  // negative part (written last)
  if (s <= K) return s;
  return -1;
}

__global__ void k_pyr_dec_lp(const float2* __restrict__ Xh, size_t in_stride, float2* __restrict__ Lp,
                             size_t out_stride, int d1, int h2, int s0, int s1, int sh2, PyrWin w, float invDN) {
  const float2* X = Xh + blockIdx.y * in_stride;
  float2* L = Lp + blockIdx.y * out_stride;
  const size_t total = (size_t)s0 * s1 * sh2;
  V3_LOOP(total) {
    const int z = (int)(idx % sh2);
    const size_t r = idx / sh2;
    const int y = (int)(r % s1), x = (int)(r / s1);
    const int px = small_to_parent(x, w.K[0], w.nr[0], s0, false);
    const int py = small_to_parent(y, w.K[1], w.nr[1], s1, false);
    const int pz = small_to_parent(z, w.K[2], w.nr[2], 2 * (sh2 - 1), true);
    float2 out = make_float2(0.f, 0.f);
    if (px >= 0 && py >= 0 && pz >= 0) {
      const float lf = win_at(w.v0, w.K[0], w.nr[0], px, false) * win_at(w.v1, w.K[1], w.nr[1], py, false) *
                       win_at(w.v2, w.K[2], w.nr[2], pz, true);
      const float2 v = X[((size_t)px * d1 + py) * h2 + pz];
      out = make_float2(v.x * lf * invDN, v.y * lf * invDN);
    }
    L[idx] = out;
  }
}

// PrySDrec_onestep.m:96-119: rec = Hp with rec(p) = sqrt(1-Lf^2) Hp(p) + Lf D^(N/2) Lp(s(p))
// on the window's support (in place over Hp).
__global__ void k_pyr_rec(float2* __restrict__ Hh, size_t stride, const float2* __restrict__ Lp, size_t lp_stride,
                          int d0, int d1, int h2, int s0, int s1, int sh2, PyrWin w, float DN) {
  float2* Hx = Hh + blockIdx.y * stride;
  const float2* L = Lp + blockIdx.y * lp_stride;
  const size_t total = (size_t)d0 * d1 * h2;
  V3_LOOP(total) {
    const int z = (int)(idx % h2);
    const size_t r = idx / h2;
    const int y = (int)(r % d1), x = (int)(r / d1);
    const float a = win_at(w.v0, w.K[0], w.nr[0], x, false);
    const float b = win_at(w.v1, w.K[1], w.nr[1], y, false);
    const float c = win_at(w.v2, w.K[2], w.nr[2], z, true);
    if (a >= 0.f && b >= 0.f && c >= 0.f) {
      const float lf = a * b * c;
      const float s = sqrtf(fmaxf(1.0f - lf * lf, 0.0f));
      const int sx = x <= w.K[0] ? x : x - w.nr[0] + s0;
      const int sy = y <= w.K[1] ? y : y - w.nr[1] + s1;
      const float2 l = L[((size_t)sx * s1 + sy) * sh2 + z];
      const float2 h = Hx[idx];
      Hx[idx] = make_float2(s * h.x + lf * DN * l.x, s * h.y + lf * DN * l.y);
    }
  }
}

// One axis of the adjoint of k_pad_edge: out (e with e[axis] reduced to n)
// sums, along `axis`, the source planes that replicate each output plane
// (the last plane collects the padded ones).
__global__ void k_fold_axis(const float* __restrict__ g, size_t g_stride, float* __restrict__ out, size_t o_stride,
                            int e0, int e1, int e2, int axis, int n) {
  const float* src = g + blockIdx.y * g_stride;
  float* dst = out + blockIdx.y * o_stride;
  const int f0 = axis == 0 ? n : e0, f1 = axis == 1 ? n : e1, f2 = axis == 2 ? n : e2;
  const int ext = axis == 0 ? e0 : (axis == 1 ? e1 : e2);
  const size_t step = axis == 0 ? (size_t)e1 * e2 : (axis == 1 ? (size_t)e2 : 1);
  const size_t total = (size_t)f0 * f1 * f2;
  V3_LOOP(total) {
    const int z = (int)(idx % f2);
    const size_t r = idx / f2;
    const int y = (int)(r % f1), x = (int)(r / f1);
    const int c = axis == 0 ? x : (axis == 1 ? y : z);
    const float* s0 = src + ((size_t)x * e1 + y) * e2 + z;
    float sum = s0[0];
    if (c == n - 1)
      for (int k = 1; k < ext - c; k++) sum += s0[k * step];
    dst[idx] = sum;
  }
}

static dim3 v3grid(size_t total, int nitems) {
  return dim3((unsigned)std::min<size_t>((total + 255) / 256, 2048), nitems);
}

cudaError_t launch_pad_real(const float* in, size_t in_stride, float2* out, size_t out_stride, int n, int m0, int m1,
                            int m2, int L0, int L1, int L2, cudaStream_t st) {
  count_launch();
  k_pad_real<<<v3grid((size_t)L0 * L1 * L2, n), 256, 0, st>>>(in, in_stride, out, out_stride, m0, m1, m2, L0, L1, L2);
  return cudaGetLastError();
}
cudaError_t launch_pad_edge(const float* in, size_t in_stride, float2* out, size_t out_stride, int n, int n0, int n1,
                            int n2, int d0, int d1, int d2, cudaStream_t st) {
  count_launch();
  k_pad_edge<<<v3grid((size_t)d0 * d1 * d2, n), 256, 0, st>>>(in, in_stride, out, out_stride, n0, n1, n2, d0, d1, d2);
  return cudaGetLastError();
}
cudaError_t launch_crop_real(const float2* in, size_t in_stride, float* out, size_t out_stride, int n, int m0, int m1,
                             int m2, int L1, int L2, int o0, int o1, int o2, float scale, cudaStream_t st) {
  count_launch();
  k_crop_real<<<v3grid((size_t)m0 * m1 * m2, n), 256, 0, st>>>(in, in_stride, out, out_stride, m0, m1, m2, L1, L2,
                                                               o0, o1, o2, scale);
  return cudaGetLastError();
}
cudaError_t launch_half(const float2* in, size_t in_stride, float2* out, size_t out_stride, int n, int d0, int d1,
                        int d2, cudaStream_t st) {
  count_launch();
  k_half<<<v3grid((size_t)d0 * d1 * (d2 / 2 + 1), n), 256, 0, st>>>(in, in_stride, out, out_stride, d0, d1, d2);
  return cudaGetLastError();
}
cudaError_t launch_conj_extend(const float2* in, size_t in_stride, float2* out, size_t out_stride, int n, int d0,
                               int d1, int d2, cudaStream_t st) {
  count_launch();
  k_conj_extend<<<v3grid((size_t)d0 * d1 * d2, n), 256, 0, st>>>(in, in_stride, out, out_stride, d0, d1, d2);
  return cudaGetLastError();
}
cudaError_t launch_pyr_dec(float2* Xh, size_t stride, float2* Lp, size_t lp_stride, int n, int d0, int d1, int d2,
                           int s0, int s1, int s2, const PyrWin& w, float invDN, cudaStream_t st) {
  const int h2 = d2 / 2 + 1, sh2 = s2 / 2 + 1;
  count_launch(2);
  k_pyr_dec_lp<<<v3grid((size_t)s0 * s1 * sh2, n), 256, 0, st>>>(Xh, stride, Lp, lp_stride, d1, h2, s0, s1, sh2, w,
                                                                  invDN);
  k_pyr_dec_hp<<<v3grid((size_t)d0 * d1 * h2, n), 256, 0, st>>>(Xh, stride, d0, d1, h2, w);
  return cudaGetLastError();
}
cudaError_t launch_pyr_rec(float2* Hh, size_t stride, const float2* Lp, size_t lp_stride, int n, int d0, int d1,
                           int d2, int s0, int s1, int s2, const PyrWin& w, float DN, cudaStream_t st) {
  count_launch();
  k_pyr_rec<<<v3grid((size_t)d0 * d1 * (d2 / 2 + 1), n), 256, 0, st>>>(Hh, stride, Lp, lp_stride, d0, d1, d2 / 2 + 1,
                                                                        s0, s1, s2 / 2 + 1, w, DN);
  return cudaGetLastError();
}
// Adjoint of launch_pad_edge: g (d0 x d1 x d2) -> out (n0 x n1 x n2), one
// axis at a time through scratch (>= d0 d1 n2 + d0 n1 n2 floats per item).
cudaError_t launch_fold_edge(const float* g, size_t g_stride, float* out, size_t o_stride, float* scratch,
                             size_t s_stride, int n, int n0, int n1, int n2, int d0, int d1, int d2, cudaStream_t st) {
  float* t1 = scratch;                           // d0 x d1 x n2
  float* t2 = scratch + (size_t)d0 * d1 * n2;    // d0 x n1 x n2
  count_launch(3);
  k_fold_axis<<<v3grid((size_t)d0 * d1 * n2, n), 256, 0, st>>>(g, g_stride, t1, s_stride, d0, d1, d2, 2, n2);
  k_fold_axis<<<v3grid((size_t)d0 * n1 * n2, n), 256, 0, st>>>(t1, s_stride, t2, s_stride, d0, d1, n2, 1, n1);
  k_fold_axis<<<v3grid((size_t)n0 * n1 * n2, n), 256, 0, st>>>(t2, s_stride, out, o_stride, d0, n1, n2, 0, n0);
  return cudaGetLastError();
}

}  // namespace nsst
