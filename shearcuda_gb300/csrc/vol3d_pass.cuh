// One pass of a batched 3-D FFT with fused load prologues and store
// epilogues: the directional stage of the 3-D path runs as three such passes
// per band pair, pruned to the sequences the next pass (or the crop) needs.
//
// A CTA owns 8 sequences along the transformed axis: 8 adjacent y at one x
// (axis 2), or 8 adjacent z at one x (axis 1) or one y (axis 0).  Only the
// index range [in_lo, in_lo + in_n) is loaded (the rest is zero: the
// zero-extension of a padded volume costs no memory traffic) and only
// [out_lo, out_lo + out_n) is stored.  Loads and stores run as separate
// loops over all 256 threads around the shared-memory FFT: these passes are
// bound by global-memory latency, and spreading each sequence group's loads
// over every thread keeps the most of them in flight.
//
// Prologues:  complex buffer | real volume in a box (zero outside) |
//             spectrum product Y .* C | real volume masked by two keep-bit sets
//             (real part: band a, imaginary part: band b).
// Epilogues:  complex buffer | real part * scale into a box |
//             hard threshold of real and imaginary parts, band-sum
//             accumulation and keep bits | S (+)= conj(C) .* X.
#pragma once
#include <cstdint>

#include "fft_core.cuh"
#include "internal.h"

namespace nsst {

namespace {
constexpr int kSeq = 8;
constexpr int kThreads = 256;

__device__ __forceinline__ void pass_coords(int axis, int a, int b, int i, int& x, int& y, int& z) {
  if (axis == 2) {
    x = a, y = b, z = i;
  } else if (axis == 1) {
    x = a, y = i, z = b;
  } else {
    x = i, y = a, z = b;
  }
}
}  // namespace

// Radix plans of the volume passes: radix <= 8, so that with 8 sequences a
// pass keeps most of the CTA's 256 threads busy (a radix-16 pass of a
// 144-point sequence would have 72 butterflies).
template <int N>
struct FftPlan3 {
  using type = typename FftPlan<N>::type;
};
template <> struct FftPlan3<16> { using type = RadixList<4, 4>; };
template <> struct FftPlan3<48> { using type = RadixList<3, 4, 4>; };
template <> struct FftPlan3<128> { using type = RadixList<8, 4, 4>; };
template <> struct FftPlan3<144> { using type = RadixList<3, 3, 4, 4>; };
template <> struct FftPlan3<256> { using type = RadixList<4, 8, 8>; };
// the level sizes of the reference's padded grids (132 = MarshalData of 128, 204 of 192)
template <> struct FftPlan3<22> { using type = RadixList<2, 11>; };
template <> struct FftPlan3<34> { using type = RadixList<2, 17>; };
template <> struct FftPlan3<44> { using type = RadixList<4, 11>; };
template <> struct FftPlan3<68> { using type = RadixList<4, 17>; };
template <> struct FftPlan3<88> { using type = RadixList<8, 11>; };
template <> struct FftPlan3<136> { using type = RadixList<8, 17>; };
template <> struct FftPlan3<132> { using type = RadixList<3, 4, 11>; };
template <> struct FftPlan3<204> { using type = RadixList<3, 4, 17>; };

template <int N, int DIR, int LD, int ST>
__global__ void __launch_bounds__(kThreads) k_v3_pass(float2* __restrict__ out, const float2* __restrict__ in,
                                                     const V3Pass P, const float2* __restrict__ tw) {
  using Plan = typename FftPlan3<N>::type;
  constexpr int NP = N + 2;  // padded row length of the row-major staging
  extern __shared__ float2 smem[];
  float2* A = smem;
  float2* Bf = smem + (size_t)NP * kSeq;
  // sequence groups of kSeq along b; the last may be partial (b_n not a
  // multiple of kSeq): its sequences from nb_valid on load zeros and store nothing
  const int groups_b = (P.b_n + kSeq - 1) / kSeq;
  const int a = P.a_lo + (int)blockIdx.x / groups_b;
  const int b0 = P.b_lo + ((int)blockIdx.x % groups_b) * kSeq;
  const int nb_valid = P.b_lo + P.b_n - b0;
  // keep-bit row pitch: masks index the box with its last dimension padded to a multiple of 8
  const int mr2 = P.m_r2 > 0 ? P.m_r2 : P.r2;
  const size_t item = blockIdx.y;
  size_t off;
  long long si, ss;
  if (P.axis == 2) {
    off = ((size_t)a * P.D1 + b0) * P.D2, si = 1, ss = P.D2;
  } else if (P.axis == 1) {
    off = (size_t)a * P.D1 * P.D2 + b0, si = P.D2, ss = 1;
  } else {
    off = (size_t)a * P.D2 + b0, si = (long long)P.D1 * P.D2, ss = 1;
  }
  const size_t wbase = item * P.item_stride;

  // the prologue for element i of sequence s
  auto load_elem = [&](int i, int s) -> float2 {
    float2 v = make_float2(0.f, 0.f);
    if (s < nb_valid && i >= P.in_lo && i < P.in_lo + P.in_n) {
      const size_t g = off + (size_t)(i * si + s * ss);
      if (LD == V3_LD_CPLX) {
        v = in[wbase + g];
      } else if (LD == V3_LD_PAIR) {
        v = cmul(in[wbase + g], __ldg(&P.spec[g]));
      } else {
        int x, y, z;
        pass_coords(P.axis, a, b0 + s, i, x, y, z);
        const size_t r = ((size_t)(x - P.o0) * P.r1 + (y - P.o1)) * P.r2 + (z - P.o2);
        const float u = P.rsrc[item * P.r_stride + r];
        if (LD == V3_LD_REAL) {
          v.x = u;
        } else {  // V3_LD_MASKED
          const size_t rm = ((size_t)(x - P.o0) * P.r1 + (y - P.o1)) * mr2 + (z - P.o2);
          const size_t mb = item * P.m_stride + (rm >> 3);
          const unsigned bit = 1u << (rm & 7);
          v.x = (P.mka[mb] & bit) ? u : 0.f;
          if (P.mkb) v.y = (P.mkb[mb] & bit) ? u : 0.f;
        }
      }
    }
    return v;
  };
  // the epilogues other than the threshold, for element i of sequence s
  auto store_elem = [&](int i, int s, float2 v) {
    if (s >= nb_valid || i < P.out_lo || i >= P.out_lo + P.out_n) return;
    const size_t g = off + (size_t)(i * si + s * ss);
    if (ST == V3_ST_CPLX) {
      out[wbase + g] = v;
    } else if (ST == V3_ST_SPEC) {
      const float2 c = __ldg(&P.spec[g]);
      const float2 prod = make_float2(c.x * v.x + c.y * v.y, c.x * v.y - c.y * v.x);  // conj(c) * v
      float2 o = prod;
      if (!P.first) {
        const float2 q = out[wbase + g];
        o = make_float2(q.x + prod.x, q.y + prod.y);
      }
      out[wbase + g] = o;
    } else {
      int x, y, z;
      pass_coords(P.axis, a, b0 + s, i, x, y, z);
      const size_t r = ((size_t)(x - P.o0) * P.r1 + (y - P.o1)) * P.r2 + (z - P.o2);
      if (ST == V3_ST_REAL) {
        P.rdst[item * P.r_stride + r] = v.x * P.scale;
      } else if (ST == V3_ST_PAIR) {
        P.rdst[item * P.r_stride + r] = v.x * P.scale;
        if (P.rdst2) P.rdst2[item * P.r_stride + r] = v.y * P.scale;
      }
    }
  };

  // the complex and real prologues stage their elements with asynchronous
  // copies (every thread's loads in flight at once; zeros written outside
  // the loaded range).  (The spectrum product staged its spectrum the same
  // way, into the second buffer, and multiplied after the wait: that moved
  // the 3-D backward identity test's error from below 2e-5 to 1.9e-4, cause
  // not found, so the product keeps its direct loads.)
  constexpr bool kAsync = LD == V3_LD_CPLX || LD == V3_LD_REAL;
  auto stage = [&](int i, int s, float2* dst, float2* dspec) {
    const bool in_range = s < nb_valid && i >= P.in_lo && i < P.in_lo + P.in_n;
    if (LD == V3_LD_REAL) {
      dst->y = 0.f;
      if (in_range) {
        int x, y, z;
        pass_coords(P.axis, a, b0 + s, i, x, y, z);
        const size_t r = ((size_t)(x - P.o0) * P.r1 + (y - P.o1)) * P.r2 + (z - P.o2);
        cp_async4(&dst->x, P.rsrc + item * P.r_stride + r);
      } else {
        dst->x = 0.f;
      }
    } else if (in_range) {
      const size_t g = off + (size_t)(i * si + s * ss);
      cp_async8(dst, in + wbase + g);
      if (LD == V3_LD_PAIR) cp_async8(dspec, P.spec + g);
    } else {
      *dst = make_float2(0.f, 0.f);
      if (LD == V3_LD_PAIR) *dspec = make_float2(0.f, 0.f);
    }
  };
  if (ST != V3_ST_THRESH && P.axis == 2) {
    // z-rows are contiguous in memory: stage them row-major (rows padded to
    // N + 2) with each warp loading consecutive elements of one row, let the
    // FFT's first and last passes read and write that layout, store along the rows
    for (int e = threadIdx.x; e < N * kSeq; e += kThreads) {
      const int s = e / N, i = e - s * N;
      if constexpr (kAsync)
        stage(i, s, &A[s * NP + i], &Bf[s * NP + i]);
      else
        A[s * NP + i] = load_elem(i, s);
    }
    if constexpr (kAsync) {
      cp_async_commit();
      cp_async_wait_all();
      if constexpr (LD == V3_LD_PAIR)  // each thread multiplies the elements it staged
        for (int e = threadIdx.x; e < N * kSeq; e += kThreads) {
          const int s = e / N, i = e - s * N;
          A[s * NP + i] = cmul(A[s * NP + i], Bf[s * NP + i]);
        }
    }
    __syncthreads();
    float2* const Z = plan_target<Plan>(A, Bf);
    block_fft_hook_plan<N, kSeq, kThreads, DIR, Plan>(
        A, Bf, tw, [&](int i, int s) { return A[s * NP + i]; }, [&](int i, int s, float2 v) { Z[s * NP + i] = v; });
    __syncthreads();
    for (int e = threadIdx.x; e < N * kSeq; e += kThreads) {
      const int s = e / N, i = e - s * N;
      store_elem(i, s, Z[s * NP + i]);
    }
    return;
  }

  for (int e = threadIdx.x; e < N * kSeq; e += kThreads) {
    const int s = e & (kSeq - 1), i = e / kSeq;
    if constexpr (kAsync)
      stage(i, s, &A[i * kSeq + s], &Bf[i * kSeq + s]);
    else
      A[i * kSeq + s] = load_elem(i, s);
  }
  if constexpr (kAsync) {
    cp_async_commit();
    cp_async_wait_all();
    if constexpr (LD == V3_LD_PAIR)  // each thread multiplies the elements it staged
      for (int e = threadIdx.x; e < N * kSeq; e += kThreads) {
        const int s = e & (kSeq - 1), i = e / kSeq;
        A[i * kSeq + s] = cmul(A[i * kSeq + s], Bf[i * kSeq + s]);
      }
  }
  __syncthreads();
  float2* X = block_fft_pp_plan<N, kSeq, kThreads, DIR, Plan>(A, Bf, tw);

  if (ST != V3_ST_THRESH) {
    for (int e = threadIdx.x; e < N * kSeq; e += kThreads) {
      const int s = e & (kSeq - 1), i = e / kSeq;
      store_elem(i, s, X[i * kSeq + s]);
    }
    return;
  }
  float ta = -1.f, tb = -1.f;
  if (P.th) {
    ta = P.th[item * P.nb_item + P.ia];
    if (P.ib >= 0) tb = P.th[item * P.nb_item + P.ib];
  }
  for (int e = threadIdx.x; e < N * kSeq; e += kThreads) {
    const int s = e & (kSeq - 1), i = e / kSeq;
    const bool st = s < nb_valid && i >= P.out_lo && i < P.out_lo + P.out_n;
    const float2 v = X[i * kSeq + s];
    int x, y, z;
    pass_coords(P.axis, a, b0 + s, i, x, y, z);
    const size_t r = ((size_t)(x - P.o0) * P.r1 + (y - P.o1)) * P.r2 + (z - P.o2);
    const size_t rm = ((size_t)(x - P.o0) * P.r1 + (y - P.o1)) * mr2 + (z - P.o2);
    // V3_ST_THRESH (ThresholdShCoeff.m:7 zeroes |c| <= t)
    const float ca = v.x * P.scale;
    const float cb = P.ib >= 0 ? v.y * P.scale : 0.f;
    const bool ka = st && !(fabsf(ca) <= ta);
    const bool kb = st && P.ib >= 0 && !(fabsf(cb) <= tb);
    if (st) {
      float* acc = P.rdst + item * P.r_stride + r;
      *acc += (ka ? ca : 0.f) + (kb ? cb : 0.f);
    }
    if (P.mwa) {  // uniform across the grid: every lane reaches the ballots
      const unsigned lane = threadIdx.x & 31;
      const unsigned ba = __ballot_sync(0xffffffffu, ka);
      const unsigned bb = __ballot_sync(0xffffffffu, kb);
      if (st && s == 0) {
        const size_t mb = item * P.m_stride + (rm >> 3);
        P.mwa[mb] = (uint8_t)((ba >> (lane & 24)) & 0xffu);
        if (P.mwb) P.mwb[mb] = (uint8_t)((bb >> (lane & 24)) & 0xffu);
      }
    }
  }
}

// (DIR, LD, ST) combinations the 3-D path uses
#define V3P_COMBOS(X, n)                        \
  X(n, -1, V3_LD_CPLX, V3_ST_CPLX)              \
  X(n, 1, V3_LD_CPLX, V3_ST_CPLX)               \
  X(n, -1, V3_LD_REAL, V3_ST_CPLX)              \
  X(n, 1, V3_LD_CPLX, V3_ST_REAL)               \
  X(n, 1, V3_LD_PAIR, V3_ST_CPLX)               \
  X(n, 1, V3_LD_CPLX, V3_ST_THRESH)             \
  X(n, 1, V3_LD_CPLX, V3_ST_PAIR)               \
  X(n, -1, V3_LD_MASKED, V3_ST_CPLX)            \
  X(n, -1, V3_LD_CPLX, V3_ST_SPEC)

}  // namespace nsst
