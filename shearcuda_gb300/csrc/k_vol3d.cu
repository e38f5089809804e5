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

constexpr int kV3Seq = 8;     // sequences per CTA
constexpr int kV3Threads = 256;

// Batched complex FFT of length N along one axis of a d0 x d1 x d2 volume
// (unnormalised, DIR -1 forward / +1 inverse), in place.  A CTA owns 8
// sequences that are adjacent in memory (axes 0, 1) or 8 adjacent rows (axis 2).
template <int N, int DIR>
__global__ void __launch_bounds__(kV3Threads) k_fft3_axis(float2* __restrict__ vol, V3Axis ax,
                                                          const float2* __restrict__ tw) {
  extern __shared__ float2 smem[];
  float2 *A = smem, *B = smem + (size_t)N * kV3Seq;
  const long long q0 = (long long)blockIdx.x * kV3Seq;  // first sequence of the group
  const long long seq_per_item = ax.nseq;
  float2* base = vol + (size_t)blockIdx.y * ax.item_stride;
  long long off;
  if (ax.axis == 2) {
    off = q0 * N;
  } else if (ax.axis == 1) {
    const long long i0 = q0 / ax.d2, i2 = q0 % ax.d2;
    off = i0 * (long long)N * ax.d2 + i2;
  } else {
    off = q0;
  }
  if (q0 >= seq_per_item) return;
  const long long si = ax.si, ss = ax.ss;
  for (int e = threadIdx.x; e < N * kV3Seq; e += kV3Threads) {
    const int s = e % kV3Seq, i = e / kV3Seq;
    A[i * kV3Seq + s] = base[off + i * si + s * ss];
  }
  __syncthreads();
  float2* X = block_fft_pp<N, kV3Seq, kV3Threads, DIR>(A, B, tw);
  for (int e = threadIdx.x; e < N * kV3Seq; e += kV3Threads) {
    const int s = e % kV3Seq, i = e / kV3Seq;
    base[off + i * si + s * ss] = X[i * kV3Seq + s];
  }
}

#define NSST_V3_SIZES(X) X(16) X(24) X(32) X(48) X(64) X(72) X(96) X(128) X(144) X(192) X(256)

bool fft3_len_supported(int n) {
  switch (n) {
#define CASE(n) case n:
    NSST_V3_SIZES(CASE)
#undef CASE
    return true;
    default:
      return false;
  }
}

cudaError_t prepare_fft3(int n) {
  switch (n) {
#define CASE(n)                                                                                         \
  case n: {                                                                                             \
    const int sm = (int)(2 * (size_t)n * kV3Seq * sizeof(float2));                                     \
    cudaError_t e = cudaFuncSetAttribute(k_fft3_axis<n, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm); \
    if (e == cudaSuccess)                                                                               \
      e = cudaFuncSetAttribute(k_fft3_axis<n, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);     \
    return e;                                                                                           \
  }
    NSST_V3_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

// One axis of a (batched) 3-D FFT.  tw: table of length d_axis.
cudaError_t launch_fft3_axis(float2* vol, int nitems, size_t item_stride, int d0, int d1, int d2, int axis, int dir,
                             const float2* tw, cudaStream_t st) {
  const int N = axis == 0 ? d0 : (axis == 1 ? d1 : d2);
  V3Axis ax;
  ax.axis = axis;
  ax.d2 = d2;
  ax.item_stride = item_stride;
  ax.nseq = (long long)d0 * d1 * d2 / N;
  if (axis == 2) {
    ax.si = 1;
    ax.ss = d2;
  } else if (axis == 1) {
    ax.si = d2;
    ax.ss = 1;
  } else {
    ax.si = (long long)d1 * d2;
    ax.ss = 1;
  }
  if (axis != 2 && d2 % kV3Seq) return cudaErrorInvalidValue;
  if (axis == 2 && (d0 * d1) % kV3Seq) return cudaErrorInvalidValue;
  dim3 grid((unsigned)(ax.nseq / kV3Seq), nitems);
  const size_t sm = 2 * (size_t)N * kV3Seq * sizeof(float2);
  count_launch();
  switch (N) {
#define CASE(n)                                                                 \
  case n:                                                                       \
    if (dir < 0)                                                                \
      k_fft3_axis<n, -1><<<grid, kV3Threads, sm, st>>>(vol, ax, tw);            \
    else                                                                        \
      k_fft3_axis<n, 1><<<grid, kV3Threads, sm, st>>>(vol, ax, tw);             \
    return cudaGetLastError();
    NSST_V3_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

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

// W = F_a .* Y + i (F_b .* Y) for a pair of filter spectra (F_b may be null)
__global__ void k_band_pair(const float2* __restrict__ Y, size_t y_stride, const float2* __restrict__ Fa,
                            const float2* __restrict__ Fb, float2* __restrict__ W, size_t w_stride, size_t n) {
  const float2* y = Y + blockIdx.y * y_stride;
  float2* w = W + blockIdx.y * w_stride;
  V3_LOOP(n) {
    const float2 v = y[idx];
    const float2 a = cmul(Fa[idx], v);
    float2 out = a;
    if (Fb) {
      const float2 b = cmul(Fb[idx], v);
      out = make_float2(a.x - b.y, a.y + b.x);
    }
    w[idx] = out;
  }
}

// acc (m^3) += T(real(W[crop]) * s, ta) + T(imag(W[crop]) * s, tb);
// T zeroes |c| <= t (ThresholdShCoeff.m:7); t = -1 disables the threshold.
// With ma (and mb) set, the keep bits |c| > t of the pair are stored, one
// 32-bit word per 32 consecutive voxels (m^3 is a multiple of 32, so every
// warp of the grid-stride loop is full).
__global__ void k_crop_thresh_acc(const float2* __restrict__ W, size_t w_stride, float* __restrict__ acc,
                                  size_t a_stride, int m0, int m1, int m2, int L1, int L2, int off,
                                  const float* __restrict__ th, int ia, int ib, int nb_item, float scale,
                                  uint32_t* __restrict__ ma, uint32_t* __restrict__ mb, size_t mask_stride) {
  const float2* w = W + blockIdx.y * w_stride;
  float* a = acc + blockIdx.y * a_stride;
  const float ta = th ? th[blockIdx.y * nb_item + ia] : -1.0f;
  const float tb = (th && ib >= 0) ? th[blockIdx.y * nb_item + ib] : -1.0f;
  uint32_t* mka = ma ? ma + blockIdx.y * mask_stride : nullptr;
  uint32_t* mkb = mb ? mb + blockIdx.y * mask_stride : nullptr;
  const size_t total = (size_t)m0 * m1 * m2;
  V3_LOOP(total) {
    const int z = (int)(idx % m2);
    const size_t r = idx / m2;
    const int y = (int)(r % m1), x = (int)(r / m1);
    const float2 v = w[((size_t)(x + off) * L1 + (y + off)) * L2 + (z + off)];
    const float ca = v.x * scale, cb = v.y * scale;
    const bool ka = !(fabsf(ca) <= ta), kb = !(fabsf(cb) <= tb);
    float sum = a[idx];
    sum += ka ? ca : 0.0f;
    if (ib >= 0) sum += kb ? cb : 0.0f;
    a[idx] = sum;
    if (mka) {
      const uint32_t bits_a = __ballot_sync(0xffffffffu, ka);
      const uint32_t bits_b = __ballot_sync(0xffffffffu, kb);
      if ((threadIdx.x & 31) == 0) {
        mka[idx >> 5] = bits_a;
        if (mkb) mkb[idx >> 5] = bits_b;
      }
    }
  }
}

// Adjoint of the pair's crop + threshold: W (L0 x L1 x L2) = zero except the
// crop box at offset `off`, where it holds keep_a * u + i keep_b * u.
__global__ void k_place_masked(const float* __restrict__ u, size_t u_stride, const uint32_t* __restrict__ ma,
                               const uint32_t* __restrict__ mb, size_t mask_stride, float2* __restrict__ W,
                               size_t w_stride, int m0, int m1, int m2, int L0, int L1, int L2, int off) {
  const float* src = u + blockIdx.y * u_stride;
  const uint32_t* mka = ma + blockIdx.y * mask_stride;
  const uint32_t* mkb = mb ? mb + blockIdx.y * mask_stride : nullptr;
  float2* dst = W + blockIdx.y * w_stride;
  const size_t total = (size_t)L0 * L1 * L2;
  V3_LOOP(total) {
    const int z = (int)(idx % L2) - off;
    const size_t r = idx / L2;
    const int y = (int)(r % L1) - off, x = (int)(r / L1) - off;
    float2 o = make_float2(0.f, 0.f);
    if (x >= 0 && x < m0 && y >= 0 && y < m1 && z >= 0 && z < m2) {
      const size_t j = ((size_t)x * m1 + y) * m2 + z;
      const float v = src[j];
      const uint32_t bit = 1u << (j & 31);
      o.x = (mka[j >> 5] & bit) ? v : 0.0f;
      if (mkb) o.y = (mkb[j >> 5] & bit) ? v : 0.0f;
    }
    dst[idx] = o;
  }
}

// S (=, or += unless first) (conj(Fa) - i conj(Fb)) Z: the real part of the
// inverse transform of the sum is the correlation of the real part of Z's
// source with filter a plus that of its imaginary part with filter b.
__global__ void k_spec_acc(const float2* __restrict__ Z, size_t z_stride, const float2* __restrict__ Fa,
                           const float2* __restrict__ Fb, float2* __restrict__ S, size_t s_stride, size_t n,
                           int first) {
  const float2* z = Z + blockIdx.y * z_stride;
  float2* s = S + blockIdx.y * s_stride;
  V3_LOOP(n) {
    const float2 fa = Fa[idx];
    float2 k = make_float2(fa.x, -fa.y);
    if (Fb) {
      const float2 fb = Fb[idx];
      k.x -= fb.y;
      k.y -= fb.x;
    }
    const float2 v = z[idx];
    const float2 prod = make_float2(k.x * v.x - k.y * v.y, k.x * v.y + k.y * v.x);
    if (first) {
      s[idx] = prod;
    } else {
      const float2 o = s[idx];
      s[idx] = make_float2(o.x + prod.x, o.y + prod.y);
    }
  }
}

// Adjoint of k_pad_edge: out (n0 x n1 x n2) gathers the grid voxels that
// replicate it (the last plane of each axis collects the padded planes).
__global__ void k_fold_edge(const float* __restrict__ g, size_t g_stride, float* __restrict__ out, size_t o_stride,
                            int n0, int n1, int n2, int d0, int d1, int d2) {
  const float* src = g + blockIdx.y * g_stride;
  float* dst = out + blockIdx.y * o_stride;
  const size_t total = (size_t)n0 * n1 * n2;
  V3_LOOP(total) {
    const int z = (int)(idx % n2);
    const size_t r = idx / n2;
    const int y = (int)(r % n1), x = (int)(r / n1);
    const int x1 = x == n0 - 1 ? d0 : x + 1, y1 = y == n1 - 1 ? d1 : y + 1, z1 = z == n2 - 1 ? d2 : z + 1;
    float sum = 0.f;
    for (int a = x; a < x1; a++)
      for (int b = y; b < y1; b++)
        for (int c = z; c < z1; c++) sum += src[((size_t)a * d1 + b) * d2 + c];
    dst[idx] = sum;
  }
}

// out_a = real(W[crop]) * s, out_b = imag(W[crop]) * s (out_b may be null)
__global__ void k_crop_pair(const float2* __restrict__ W, size_t w_stride, float* __restrict__ out_a,
                            float* __restrict__ out_b, size_t o_stride, int m0, int m1, int m2, int L1, int L2, int off,
                            float scale) {
  const float2* w = W + blockIdx.y * w_stride;
  float* a = out_a + blockIdx.y * o_stride;
  float* b = out_b ? out_b + blockIdx.y * o_stride : nullptr;
  const size_t total = (size_t)m0 * m1 * m2;
  V3_LOOP(total) {
    const int z = (int)(idx % m2);
    const size_t r = idx / m2;
    const int y = (int)(r % m1), x = (int)(r / m1);
    const float2 v = w[((size_t)(x + off) * L1 + (y + off)) * L2 + (z + off)];
    a[idx] = v.x * scale;
    if (b) b[idx] = v.y * scale;
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
cudaError_t launch_band_pair(const float2* Y, size_t y_stride, const float2* Fa, const float2* Fb, float2* W,
                             size_t w_stride, int n, size_t total, cudaStream_t st) {
  count_launch();
  k_band_pair<<<v3grid(total, n), 256, 0, st>>>(Y, y_stride, Fa, Fb, W, w_stride, total);
  return cudaGetLastError();
}
cudaError_t launch_crop_pair(const float2* W, size_t w_stride, float* out_a, float* out_b, size_t o_stride, int n,
                            int m0, int m1, int m2, int L1, int L2, int off, float scale, cudaStream_t st) {
  count_launch();
  k_crop_pair<<<v3grid((size_t)m0 * m1 * m2, n), 256, 0, st>>>(W, w_stride, out_a, out_b, o_stride, m0, m1, m2, L1, L2,
                                                                off, scale);
  return cudaGetLastError();
}
cudaError_t launch_crop_thresh_acc(const float2* W, size_t w_stride, float* acc, size_t a_stride, int n, int m0,
                                   int m1, int m2, int L1, int L2, int off, const float* th, int ia, int ib,
                                   int nb_item, float scale, uint32_t* ma, uint32_t* mb, size_t mask_stride,
                                   cudaStream_t st) {
  if (ma && ((size_t)m0 * m1 * m2) % 32) return cudaErrorInvalidValue;
  count_launch();
  k_crop_thresh_acc<<<v3grid((size_t)m0 * m1 * m2, n), 256, 0, st>>>(W, w_stride, acc, a_stride, m0, m1, m2, L1, L2,
                                                                      off, th, ia, ib, nb_item, scale, ma, mb,
                                                                      mask_stride);
  return cudaGetLastError();
}
cudaError_t launch_place_masked(const float* u, size_t u_stride, const uint32_t* ma, const uint32_t* mb,
                                size_t mask_stride, float2* W, size_t w_stride, int n, int m0, int m1, int m2, int L0,
                                int L1, int L2, int off, cudaStream_t st) {
  count_launch();
  k_place_masked<<<v3grid((size_t)L0 * L1 * L2, n), 256, 0, st>>>(u, u_stride, ma, mb, mask_stride, W, w_stride, m0,
                                                                   m1, m2, L0, L1, L2, off);
  return cudaGetLastError();
}
cudaError_t launch_spec_acc(const float2* Z, size_t z_stride, const float2* Fa, const float2* Fb, float2* S,
                            size_t s_stride, int n, size_t total, bool first, cudaStream_t st) {
  count_launch();
  k_spec_acc<<<v3grid(total, n), 256, 0, st>>>(Z, z_stride, Fa, Fb, S, s_stride, total, first ? 1 : 0);
  return cudaGetLastError();
}
cudaError_t launch_fold_edge(const float* g, size_t g_stride, float* out, size_t o_stride, int n, int n0, int n1,
                             int n2, int d0, int d1, int d2, cudaStream_t st) {
  count_launch();
  k_fold_edge<<<v3grid((size_t)n0 * n1 * n2, n), 256, 0, st>>>(g, g_stride, out, o_stride, n0, n1, n2, d0, d1, d2);
  return cudaGetLastError();
}

}  // namespace nsst
