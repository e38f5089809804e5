// Block-cooperative FP32 FFTs in shared memory, for the NSST directional stage.
//
// Layout convention used by every kernel: a CTA owns `NSEQ` sequences of
// length N; element (sequence s, index i) lives at buf[i * LD + s] with
// LD = NSEQ + 1 (one float2 of padding per index keeps the row-to-column
// staging and the butterflies free of shared-memory bank conflicts).
//
// The transform is a Stockham auto-sort FFT: every pass reads its R inputs
// at stride N/R, twiddles them, runs an R-point DFT in registers and writes
// the outputs to their sorted positions, so the result is in natural order
// with no bit-reversal pass.  Radices 2, 3, 4 and 8 cover every length of
// the form 2^a * 3^b (b <= 1) that the pyramid sizes need.
//
// Twiddles come from a table tw[t] = exp(-2 pi i t / N) computed in FP64 on
// the host and rounded once to FP32 (no on-device trigonometry).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace nsst {

struct cpx {
  float x, y;
};

// Complex add / subtract as one packed FP32 instruction each (FADD2 / FFMA2
// with -1, both rounded exactly like the two scalar operations).
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by -i (DIR<0) or +i (DIR>0)
template <int DIR>
__device__ __forceinline__ float2 mul_i(float2 a) {
  return DIR < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}
// a + c t (the radix-3 butterfly's mean term)
__device__ __forceinline__ float2 caxc(float2 a, float c, float2 t) { return make_float2(a.x + c * t.x, a.y + c * t.y); }
// a (c + i sg sn)
__device__ __forceinline__ float2 crot(float2 a, float c, float sg, float sn) {
  return make_float2(a.x * c - sg * sn * a.y, a.y * c + sg * sn * a.x);
}
// a W8^1 and a W8^3 (forward: exp(-2 pi i k / 8), inverse: exp(+2 pi i k / 8))
template <int DIR>
__device__ __forceinline__ float2 rot8_1(float2 o, float r) {
  return DIR < 0 ? make_float2((o.x + o.y) * r, (o.y - o.x) * r) : make_float2((o.x - o.y) * r, (o.y + o.x) * r);
}
template <int DIR>
__device__ __forceinline__ float2 rot8_3(float2 o, float r) {
  return DIR < 0 ? make_float2((-o.x + o.y) * r, (-o.y - o.x) * r) : make_float2((-o.x - o.y) * r, (-o.y + o.x) * r);
}

// Two complex values of two sequences at one index, as one 16-byte element
// (float4 = (re0, im0, re1, im1)): the butterflies below then move two
// sequences per shared-memory access and per twiddle load.
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float4 pk4(float2 a, float2 b) { return make_float4(a.x, a.y, b.x, b.y); }
__device__ __forceinline__ float4 cadd(float4 a, float4 b) { return pk4(cadd(lo2(a), lo2(b)), cadd(hi2(a), hi2(b))); }
__device__ __forceinline__ float4 csub(float4 a, float4 b) { return pk4(csub(lo2(a), lo2(b)), csub(hi2(a), hi2(b))); }
__device__ __forceinline__ float4 cmul(float4 a, float2 b) { return pk4(cmul(lo2(a), b), cmul(hi2(a), b)); }
__device__ __forceinline__ float4 cmulc(float4 a, float2 b) { return pk4(cmulc(lo2(a), b), cmulc(hi2(a), b)); }
__device__ __forceinline__ float4 cscale(float4 a, float s) { return pk4(cscale(lo2(a), s), cscale(hi2(a), s)); }
template <int DIR>
__device__ __forceinline__ float4 mul_i(float4 a) {
  return pk4(mul_i<DIR>(lo2(a)), mul_i<DIR>(hi2(a)));
}
__device__ __forceinline__ float4 caxc(float4 a, float c, float4 t) {
  return pk4(caxc(lo2(a), c, lo2(t)), caxc(hi2(a), c, hi2(t)));
}
__device__ __forceinline__ float4 crot(float4 a, float c, float sg, float sn) {
  return pk4(crot(lo2(a), c, sg, sn), crot(hi2(a), c, sg, sn));
}
template <int DIR>
__device__ __forceinline__ float4 rot8_1(float4 o, float r) {
  return pk4(rot8_1<DIR>(lo2(o), r), rot8_1<DIR>(hi2(o), r));
}
template <int DIR>
__device__ __forceinline__ float4 rot8_3(float4 o, float r) {
  return pk4(rot8_3<DIR>(lo2(o), r), rot8_3<DIR>(hi2(o), r));
}

// Two complex values of two sequences at one index in split form: the real
// parts in one register pair, the imaginary parts in another.  Every complex
// operation on the pair is then packed FP32x2 arithmetic (a twiddle multiply
// of both values is two FMUL2 and two FFMA2 instead of eight scalar
// instructions), and a thread's index arithmetic serves two sequences.  Each
// packed lane rounds exactly like the scalar operation it replaces.
struct cpx2 {
  float2 re, im;
};
__device__ __forceinline__ float2 bcast(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ cpx2 cadd(cpx2 a, cpx2 b) { return {cadd(a.re, b.re), cadd(a.im, b.im)}; }
__device__ __forceinline__ cpx2 csub(cpx2 a, cpx2 b) { return {csub(a.re, b.re), csub(a.im, b.im)}; }
__device__ __forceinline__ cpx2 cconj(cpx2 a) { return {a.re, neg2(a.im)}; }
__device__ __forceinline__ cpx2 cscale(cpx2 a, float s) { return {__fmul2_rn(a.re, bcast(s)), __fmul2_rn(a.im, bcast(s))}; }
// a * t for a twiddle given as its broadcast pairs (t.x, t.x), (t.y, t.y)
__device__ __forceinline__ cpx2 cmul_b(cpx2 a, float2 tx, float2 ty) {
  return {__ffma2_rn(a.re, tx, neg2(__fmul2_rn(a.im, ty))), __ffma2_rn(a.im, tx, __fmul2_rn(a.re, ty))};
}
// a * conj(t)
__device__ __forceinline__ cpx2 cmulc_b(cpx2 a, float2 tx, float2 ty) {
  return {__ffma2_rn(a.re, tx, __fmul2_rn(a.im, ty)), __ffma2_rn(a.im, tx, neg2(__fmul2_rn(a.re, ty)))};
}
__device__ __forceinline__ cpx2 cmul(cpx2 a, float2 t) { return cmul_b(a, bcast(t.x), bcast(t.y)); }
__device__ __forceinline__ cpx2 cmulc(cpx2 a, float2 t) { return cmulc_b(a, bcast(t.x), bcast(t.y)); }
template <int DIR>
__device__ __forceinline__ cpx2 mul_i(cpx2 a) {
  return DIR < 0 ? cpx2{a.im, neg2(a.re)} : cpx2{neg2(a.im), a.re};
}
__device__ __forceinline__ cpx2 caxc(cpx2 a, float c, cpx2 t) {
  return {__ffma2_rn(t.re, bcast(c), a.re), __ffma2_rn(t.im, bcast(c), a.im)};
}
// a (c + i sg sn)
__device__ __forceinline__ cpx2 crot(cpx2 a, float c, float sg, float sn) {
  const float2 s2 = bcast(sg * sn);
  return {__ffma2_rn(a.re, bcast(c), neg2(__fmul2_rn(a.im, s2))), __ffma2_rn(a.im, bcast(c), __fmul2_rn(a.re, s2))};
}
template <int DIR>
__device__ __forceinline__ cpx2 rot8_1(cpx2 o, float r) {
  return DIR < 0 ? cpx2{__fmul2_rn(cadd(o.re, o.im), bcast(r)), __fmul2_rn(csub(o.im, o.re), bcast(r))}
                 : cpx2{__fmul2_rn(csub(o.re, o.im), bcast(r)), __fmul2_rn(cadd(o.im, o.re), bcast(r))};
}
template <int DIR>
__device__ __forceinline__ cpx2 rot8_3(cpx2 o, float r) {
  return DIR < 0 ? cpx2{__fmul2_rn(csub(o.im, o.re), bcast(r)), neg2(__fmul2_rn(cadd(o.im, o.re), bcast(r)))}
                 : cpx2{neg2(__fmul2_rn(cadd(o.re, o.im), bcast(r))), __fmul2_rn(csub(o.re, o.im), bcast(r))};
}
// the two values of a pair as ordinary complex numbers, and back
__device__ __forceinline__ float2 lane0(cpx2 a) { return make_float2(a.re.x, a.im.x); }
__device__ __forceinline__ float2 lane1(cpx2 a) { return make_float2(a.re.y, a.im.y); }
__device__ __forceinline__ cpx2 pair(float2 a, float2 b) { return {make_float2(a.x, b.x), make_float2(a.y, b.y)}; }

// Twiddle multiply inside a pass: for cpx2 elements the table holds each
// twiddle as its broadcast pairs (t.x, t.x, t.y, t.y) in one 16-byte entry.
template <int DIR>
__device__ __forceinline__ float2 tw_mul(float2 v, const float2* __restrict__ tw, int idx) {
  const float2 t = __ldg(&tw[idx]);
  return DIR < 0 ? cmul(v, t) : cmulc(v, t);
}
template <int DIR>
__device__ __forceinline__ float4 tw_mul(float4 v, const float2* __restrict__ tw, int idx) {
  const float2 t = __ldg(&tw[idx]);
  return DIR < 0 ? cmul(v, t) : cmulc(v, t);
}
template <int DIR>
__device__ __forceinline__ cpx2 tw_mul(cpx2 v, const float2* __restrict__ tw, int idx) {
  const float4 t = __ldg(reinterpret_cast<const float4*>(tw) + idx);
  return DIR < 0 ? cmul_b(v, make_float2(t.x, t.y), make_float2(t.z, t.w))
                 : cmulc_b(v, make_float2(t.x, t.y), make_float2(t.z, t.w));
}

// ---------------------------------------------------------------------------
// R-point DFTs in registers.  DIR = -1 forward (exp(-2 pi i ...)), +1 inverse.
// ---------------------------------------------------------------------------
template <int R, int DIR>
struct Dft;

template <int DIR>
struct Dft<2, DIR> {
  template <class E>
  __device__ __forceinline__ static void run(E* v) {
    E a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <int DIR>
struct Dft<3, DIR> {
  template <class E>
  __device__ __forceinline__ static void run(E* v) {
    const float c = -0.5f;
    const float s = 0.86602540378443864676f;  // sin(2 pi / 3)
    E a0 = v[0], a1 = v[1], a2 = v[2];
    E t = cadd(a1, a2);
    E d = csub(a1, a2);
    v[0] = cadd(a0, t);
    E m = caxc(a0, c, t);
    // forward: -i * s * d ; inverse: +i * s * d
    E u = mul_i<DIR>(cscale(d, s));
    v[1] = cadd(m, u);
    v[2] = csub(m, u);
  }
};

template <int DIR>
struct Dft<4, DIR> {
  template <class E>
  __device__ __forceinline__ static void run(E* v) {
    E s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    E s13 = cadd(v[1], v[3]), d13 = mul_i<DIR>(csub(v[1], v[3]));
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, d13);
    v[3] = csub(d02, d13);
  }
};

template <int DIR>
struct Dft<8, DIR> {
  template <class E>
  __device__ __forceinline__ static void run(E* v) {
    const float r = 0.70710678118654752440f;
    E e[4] = {v[0], v[2], v[4], v[6]};
    E o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, DIR>::run(e);
    Dft<4, DIR>::run(o);
    // twiddle o[k] by exp(DIR * 2 pi i k / 8): k=1 (1 + DIR i) r, k=2 DIR i, k=3 (-1 + DIR i) r
    o[1] = rot8_1<DIR>(o[1], r);
    o[2] = mul_i<DIR>(o[2]);
    o[3] = rot8_3<DIR>(o[3], r);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      v[k] = cadd(e[k], o[k]);
      v[k + 4] = csub(e[k], o[k]);
    }
  }
};

// 16 = 4 x 4: 4-point DFTs over n2 of x[n1 + 4 n2], twiddles W16^(n1 k2),
// 4-point DFTs over n1 -> X[k2 + 4 k1].
template <int DIR>
struct Dft<16, DIR> {
  template <class E>
  __device__ __forceinline__ static void run(E* v) {
    const float r = 0.70710678118654752440f;   // cos(pi/4)
    const float c1 = 0.92387953251128675613f;  // cos(pi/8)
    const float s1 = 0.38268343236508977173f;  // sin(pi/8)
    E y[4][4];
#pragma unroll
    for (int n1 = 0; n1 < 4; n1++) {
      E t[4] = {v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]};
      Dft<4, DIR>::run(t);
#pragma unroll
      for (int k2 = 0; k2 < 4; k2++) y[n1][k2] = t[k2];
    }
    // W16^m = exp(DIR * 2 pi i m / 16) for m = n1 * k2 in {1, 2, 3, 4, 6, 9}
    const float sg = DIR < 0 ? -1.f : 1.f;
    auto rot = [&](E a, float c, float sn) { return crot(a, c, sg, sn); };  // a * (c + i sg sn)
    y[1][1] = rot(y[1][1], c1, s1);
    y[1][2] = rot(y[1][2], r, r);
    y[1][3] = rot(y[1][3], s1, c1);
    y[2][1] = rot(y[2][1], r, r);
    y[2][2] = mul_i<DIR>(y[2][2]);
    y[2][3] = rot(y[2][3], -r, r);
    y[3][1] = rot(y[3][1], s1, c1);
    y[3][2] = rot(y[3][2], -r, r);
    y[3][3] = rot(y[3][3], -c1, -s1);
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) {
      E t[4] = {y[0][k2], y[1][k2], y[2][k2], y[3][k2]};
      Dft<4, DIR>::run(t);
#pragma unroll
      for (int k1 = 0; k1 < 4; k1++) v[k2 + 4 * k1] = t[k1];
    }
  }
};

// Odd radices 5, 7, 11, 13, 17 (the 3-D pyramid on the reference's padded
// grids: 132 = 3 * 4 * 11, 204 = 3 * 4 * 17 and their level sizes).  With
// a_j = v[j] + v[R-j], b_j = v[j] - v[R-j] (j = 1 .. h, h = (R-1)/2):
//   X[k]   = v[0] + sum_j a_j cos(2 pi jk/R) + DIR i sum_j b_j sin(2 pi jk/R)
//   X[R-k] = the same with the second sum negated,  X[0] = v[0] + sum_j a_j,
// which is the R-point DFT with exp(DIR 2 pi i jk / R) paired over j and R - j.
// The tables hold cos / sin(2 pi m / R) computed in FP64 and rounded to FP32.
template <int R>
struct OddTab;
template <>
struct OddTab<5> {
  __host__ __device__ static constexpr float c(int m) {
    constexpr float t[5] = {1.000000000e+00f, 3.090169944e-01f, -8.090169944e-01f, -8.090169944e-01f, 3.090169944e-01f};
    return t[m];
  }
  __host__ __device__ static constexpr float s(int m) {
    constexpr float t[5] = {0.000000000e+00f, 9.510565163e-01f, 5.877852523e-01f, -5.877852523e-01f, -9.510565163e-01f};
    return t[m];
  }
};
template <>
struct OddTab<7> {
  __host__ __device__ static constexpr float c(int m) {
    constexpr float t[7] = {1.000000000e+00f, 6.234898019e-01f, -2.225209340e-01f, -9.009688679e-01f, -9.009688679e-01f, -2.225209340e-01f, 6.234898019e-01f};
    return t[m];
  }
  __host__ __device__ static constexpr float s(int m) {
    constexpr float t[7] = {0.000000000e+00f, 7.818314825e-01f, 9.749279122e-01f, 4.338837391e-01f, -4.338837391e-01f, -9.749279122e-01f, -7.818314825e-01f};
    return t[m];
  }
};
template <>
struct OddTab<11> {
  __host__ __device__ static constexpr float c(int m) {
    constexpr float t[11] = {1.000000000e+00f, 8.412535328e-01f, 4.154150130e-01f, -1.423148383e-01f, -6.548607339e-01f, -9.594929736e-01f, -9.594929736e-01f, -6.548607339e-01f, -1.423148383e-01f, 4.154150130e-01f, 8.412535328e-01f};
    return t[m];
  }
  __host__ __device__ static constexpr float s(int m) {
    constexpr float t[11] = {0.000000000e+00f, 5.406408175e-01f, 9.096319954e-01f, 9.898214419e-01f, 7.557495744e-01f, 2.817325568e-01f, -2.817325568e-01f, -7.557495744e-01f, -9.898214419e-01f, -9.096319954e-01f, -5.406408175e-01f};
    return t[m];
  }
};
template <>
struct OddTab<13> {
  __host__ __device__ static constexpr float c(int m) {
    constexpr float t[13] = {1.000000000e+00f, 8.854560257e-01f, 5.680647467e-01f, 1.205366803e-01f, -3.546048870e-01f, -7.485107482e-01f, -9.709418174e-01f, -9.709418174e-01f, -7.485107482e-01f, -3.546048870e-01f, 1.205366803e-01f, 5.680647467e-01f, 8.854560257e-01f};
    return t[m];
  }
  __host__ __device__ static constexpr float s(int m) {
    constexpr float t[13] = {0.000000000e+00f, 4.647231720e-01f, 8.229838659e-01f, 9.927088741e-01f, 9.350162427e-01f, 6.631226582e-01f, 2.393156643e-01f, -2.393156643e-01f, -6.631226582e-01f, -9.350162427e-01f, -9.927088741e-01f, -8.229838659e-01f, -4.647231720e-01f};
    return t[m];
  }
};
template <>
struct OddTab<17> {
  __host__ __device__ static constexpr float c(int m) {
    constexpr float t[17] = {1.000000000e+00f, 9.324722294e-01f, 7.390089172e-01f, 4.457383558e-01f, 9.226835946e-02f, -2.736629901e-01f, -6.026346364e-01f, -8.502171357e-01f, -9.829730997e-01f, -9.829730997e-01f, -8.502171357e-01f, -6.026346364e-01f, -2.736629901e-01f, 9.226835946e-02f, 4.457383558e-01f, 7.390089172e-01f, 9.324722294e-01f};
    return t[m];
  }
  __host__ __device__ static constexpr float s(int m) {
    constexpr float t[17] = {0.000000000e+00f, 3.612416662e-01f, 6.736956436e-01f, 8.951632914e-01f, 9.957341763e-01f, 9.618256432e-01f, 7.980172273e-01f, 5.264321629e-01f, 1.837495178e-01f, -1.837495178e-01f, -5.264321629e-01f, -7.980172273e-01f, -9.618256432e-01f, -9.957341763e-01f, -8.951632914e-01f, -6.736956436e-01f, -3.612416662e-01f};
    return t[m];
  }
};

template <int R, int DIR>
struct DftOdd {
  template <class E>
  __device__ __forceinline__ static void run(E* v) {
    constexpr int h = (R - 1) / 2;
    E a[h], b[h];
#pragma unroll
    for (int j = 1; j <= h; j++) {
      a[j - 1] = cadd(v[j], v[R - j]);
      b[j - 1] = csub(v[j], v[R - j]);
    }
    E x0 = v[0];
#pragma unroll
    for (int j = 0; j < h; j++) x0 = cadd(x0, a[j]);
#pragma unroll
    for (int k = 1; k <= h; k++) {
      E A = caxc(v[0], OddTab<R>::c(k % R), a[0]);
      E Bs = cscale(b[0], OddTab<R>::s(k % R));
#pragma unroll
      for (int j = 2; j <= h; j++) {
        A = caxc(A, OddTab<R>::c((j * k) % R), a[j - 1]);
        Bs = caxc(Bs, OddTab<R>::s((j * k) % R), b[j - 1]);
      }
      // DIR i Bs: forward (DIR = -1) X[k] = A - i Bs, inverse X[k] = A + i Bs
      const E iB = mul_i<DIR>(Bs);
      v[k] = cadd(A, iB);
      v[R - k] = csub(A, iB);
    }
    v[0] = x0;
  }
};
template <int DIR> struct Dft<5, DIR> : DftOdd<5, DIR> {};
template <int DIR> struct Dft<7, DIR> : DftOdd<7, DIR> {};
template <int DIR> struct Dft<11, DIR> : DftOdd<11, DIR> {};
template <int DIR> struct Dft<13, DIR> : DftOdd<13, DIR> {};
template <int DIR> struct Dft<17, DIR> : DftOdd<17, DIR> {};

// ---------------------------------------------------------------------------
// Radix plans per length (product of radices == N).
// ---------------------------------------------------------------------------
template <int... Rs>
struct RadixList {};

template <int N>
struct FftPlan;
template <> struct FftPlan<16> { using type = RadixList<16>; };
template <> struct FftPlan<24> { using type = RadixList<3, 8>; };
template <> struct FftPlan<32> { using type = RadixList<4, 8>; };
template <> struct FftPlan<48> { using type = RadixList<3, 16>; };
template <> struct FftPlan<64> { using type = RadixList<8, 8>; };
template <> struct FftPlan<72> { using type = RadixList<3, 3, 8>; };
template <> struct FftPlan<144> { using type = RadixList<3, 3, 16>; };
template <> struct FftPlan<96> { using type = RadixList<3, 4, 8>; };
template <> struct FftPlan<128> { using type = RadixList<16, 8>; };
template <> struct FftPlan<192> { using type = RadixList<3, 8, 8>; };
template <> struct FftPlan<216> { using type = RadixList<3, 3, 3, 8>; };
template <> struct FftPlan<256> { using type = RadixList<16, 16>; };
template <> struct FftPlan<384> { using type = RadixList<3, 16, 8>; };
template <> struct FftPlan<512> { using type = RadixList<8, 8, 8>; };
template <> struct FftPlan<768> { using type = RadixList<3, 16, 16>; };
template <> struct FftPlan<1024> { using type = RadixList<16, 16, 4>; };
template <> struct FftPlan<2048> { using type = RadixList<16, 16, 8>; };

// One Stockham pass of radix R over NSEQ sequences of length N, in place.
// NS = product of the radices already applied.  All threads participate.
template <int N, int NSEQ, int T, int R, int NS, int DIR>
__device__ __forceinline__ void stockham_pass(float2* buf, const float2* __restrict__ tw) {
  constexpr int LD = NSEQ + 1;
  constexpr int NB = N / R;            // butterflies per sequence
  constexpr int TOTAL = NB * NSEQ;     // butterflies in the CTA
  constexpr int IPT = (TOTAL + T - 1) / T;
  constexpr int STEP = N / (NS * R);   // twiddle index stride
  float2 v[IPT][R];
  const int tid = threadIdx.x;
#pragma unroll
  for (int it = 0; it < IPT; it++) {
    int w = tid + it * T;
    if (TOTAL % T == 0 || w < TOTAL) {
      int s = w % NSEQ;
      int j = w / NSEQ;
#pragma unroll
      for (int r = 0; r < R; r++) v[it][r] = buf[(j + r * NB) * LD + s];
      if (NS > 1) {
        int k = j % NS;
#pragma unroll
        for (int r = 1; r < R; r++) {
          float2 t = __ldg(&tw[r * k * STEP]);
          v[it][r] = DIR < 0 ? cmul(v[it][r], t) : cmulc(v[it][r], t);
        }
      }
      Dft<R, DIR>::run(v[it]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < IPT; it++) {
    int w = tid + it * T;
    if (TOTAL % T == 0 || w < TOTAL) {
      int s = w % NSEQ;
      int j = w / NSEQ;
      int k = j % NS;
      int base = (j / NS) * NS * R + k;
#pragma unroll
      for (int r = 0; r < R; r++) buf[(base + r * NS) * LD + s] = v[it][r];
    }
  }
  __syncthreads();
}

template <int N, int NSEQ, int T, int DIR, int NS>
__device__ __forceinline__ void fft_passes(float2*, const float2* __restrict__, RadixList<>) {}

template <int N, int NSEQ, int T, int DIR, int NS, int R, int... Rest>
__device__ __forceinline__ void fft_passes(float2* buf, const float2* __restrict__ tw, RadixList<R, Rest...>) {
  stockham_pass<N, NSEQ, T, R, NS, DIR>(buf, tw);
  fft_passes<N, NSEQ, T, DIR, NS * R>(buf, tw, RadixList<Rest...>{});
}

// In-place FFT of NSEQ sequences of length N held in shared memory
// (layout buf[i * (NSEQ+1) + s]).  Unnormalised in both directions.
// Caller must __syncthreads() before (data staged) — this routine ends synced.
template <int N, int NSEQ, int T, int DIR>
__device__ __forceinline__ void block_fft(float2* buf, const float2* __restrict__ tw) {
  fft_passes<N, NSEQ, T, DIR, 1>(buf, tw, typename FftPlan<N>::type{});
}

// ---------------------------------------------------------------------------
// Real <-> packed-complex row transforms.
//
// A real row x[0..W) is viewed as W/2 complex z[n] = x[2n] + i x[2n+1].
// Forward: after Z = FFT_{W/2}(z) the packed half spectrum is
//   X[k] = E + w^k O,  X[W/2-k] = conj(E - w^k O),  E = (Z[k]+conj(Z[-k]))/2,
//   O = (Z[k]-conj(Z[-k]))/(2i), w = exp(-2 pi i / W),
// with slot 0 holding the two real bins (X[0], X[W/2]).
// Inverse (before an unnormalised inverse FFT_{W/2}) forms
//   Z[k] = E + iO,  Z[W/2-k] = conj(E - iO),  E = X[k]+conj(X[W/2-k]),
//   O = w^-k (X[k]-conj(X[W/2-k])),
// so that inverse(forward(x)) = W x.
// twW[k] = exp(-2 pi i k / W), k < W/2.
// ---------------------------------------------------------------------------
template <int WH, int NSEQ, int T>
__device__ __forceinline__ void r2c_post(float2* buf, const float2* __restrict__ twW) {
  constexpr int LD = NSEQ + 1;
  constexpr int PAIRS = WH / 2 + 1;  // k = 0 .. WH/2
  constexpr int TOTAL = PAIRS * NSEQ;
  constexpr int IPT = (TOTAL + T - 1) / T;
  float2 a[IPT], b[IPT];
  const int tid = threadIdx.x;
#pragma unroll
  for (int it = 0; it < IPT; it++) {
    int w = tid + it * T;
    if (w < TOTAL) {
      int s = w % NSEQ, k = w / NSEQ;
      float2 zk = buf[k * LD + s];
      if (k == 0) {
        a[it] = make_float2(zk.x + zk.y, zk.x - zk.y);
      } else {
        float2 zm = buf[(WH - k) * LD + s];
        float2 zmc = cconj(zm);
        float2 E = cscale(cadd(zk, zmc), 0.5f);
        float2 d = cscale(csub(zk, zmc), 0.5f);
        float2 O = make_float2(d.y, -d.x);  // d / i
        float2 To = cmul(__ldg(&twW[k]), O);
        a[it] = cadd(E, To);
        b[it] = cconj(csub(E, To));
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < IPT; it++) {
    int w = tid + it * T;
    if (w < TOTAL) {
      int s = w % NSEQ, k = w / NSEQ;
      buf[k * LD + s] = a[it];
      if (k != 0 && k != WH - k) buf[(WH - k) * LD + s] = b[it];
    }
  }
  __syncthreads();
}

template <int WH, int NSEQ, int T>
__device__ __forceinline__ void c2r_pre(float2* buf, const float2* __restrict__ twW) {
  constexpr int LD = NSEQ + 1;
  constexpr int PAIRS = WH / 2 + 1;
  constexpr int TOTAL = PAIRS * NSEQ;
  constexpr int IPT = (TOTAL + T - 1) / T;
  float2 a[IPT], b[IPT];
  const int tid = threadIdx.x;
#pragma unroll
  for (int it = 0; it < IPT; it++) {
    int w = tid + it * T;
    if (w < TOTAL) {
      int s = w % NSEQ, k = w / NSEQ;
      float2 xk = buf[k * LD + s];
      if (k == 0) {
        // X[0] = xk.x, X[W/2] = xk.y (both real)
        a[it] = make_float2(xk.x + xk.y, xk.x - xk.y);
      } else {
        float2 xmc = cconj(buf[(WH - k) * LD + s]);
        float2 E = cadd(xk, xmc);
        float2 O = cmulc(csub(xk, xmc), __ldg(&twW[k]));  // * w^-k
        float2 iO = make_float2(-O.y, O.x);
        a[it] = cadd(E, iO);
        b[it] = cconj(csub(E, iO));
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < IPT; it++) {
    int w = tid + it * T;
    if (w < TOTAL) {
      int s = w % NSEQ, k = w / NSEQ;
      buf[k * LD + s] = a[it];
      if (k != 0 && k != WH - k) buf[(WH - k) * LD + s] = b[it];
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Ping-pong variant: each pass reads buffer `in` and writes buffer `out`, so a
// thread only holds one butterfly's R values at a time (low register use) and
// a pass needs a single barrier.  Returns the buffer that holds the result.
//
// Layout: element (index i, sequence s) at [phi(i) * NSEQ + s] with no padding.
// A warp covers 32/NSEQ consecutive butterflies of NSEQ sequences each, so the
// rows it touches in one access are consecutive (-> alternating bank groups,
// conflict-free) in every pass except where the first pass (NS == 1) writes
// rows R apart; that pass's output is row-swizzled, phi(i) = i ^ ((i / R) & m)
// with m = 16/NSEQ - 1, and the second pass reads it back through the same phi.
// ---------------------------------------------------------------------------
template <int NSEQ, int SWZ>
__device__ __forceinline__ int swz_row(int i) {
  constexpr int M = 16 / NSEQ - 1;
  if (SWZ == 0 || M <= 0) return i;
  return i ^ ((i / SWZ) & M);
}

template <int N, int NSEQ, int T, int R, int NS, int DIR, int SWZ_IN, int SWZ_OUT>
__device__ __forceinline__ void stockham_pp(const float2* __restrict__ in, float2* __restrict__ out,
                                            const float2* __restrict__ tw) {
  constexpr int NB = N / R;
  constexpr int TOTAL = NB * NSEQ;
  constexpr int STEP = N / (NS * R);
#pragma unroll 2
  for (int w = threadIdx.x; w < TOTAL; w += T) {
    const int s = w % NSEQ;
    const int j = w / NSEQ;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = in[swz_row<NSEQ, SWZ_IN>(j + r * NB) * NSEQ + s];
    const int k = j % NS;
    if (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; r++) {
        float2 t = __ldg(&tw[r * k * STEP]);
        v[r] = DIR < 0 ? cmul(v[r], t) : cmulc(v[r], t);
      }
    }
    Dft<R, DIR>::run(v);
    const int base = (j / NS) * NS * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) out[swz_row<NSEQ, SWZ_OUT>(base + r * NS) * NSEQ + s] = v[r];
  }
  __syncthreads();
}

template <int N, int NSEQ, int T, int DIR, int NS, int SWZ_IN>
__device__ __forceinline__ float2* fft_pp_passes(float2* a, float2* b, const float2* __restrict__ tw, RadixList<>) {
  return a;
}

template <int N, int NSEQ, int T, int DIR, int NS, int SWZ_IN, int R, int... Rest>
__device__ __forceinline__ float2* fft_pp_passes(float2* a, float2* b, const float2* __restrict__ tw,
                                                 RadixList<R, Rest...>) {
  // only the first pass (NS == 1, even radix) writes rows R apart
  constexpr int SWZ_OUT = (NS == 1 && R % 2 == 0 && sizeof...(Rest) > 0) ? R : 0;
  stockham_pp<N, NSEQ, T, R, NS, DIR, SWZ_IN, SWZ_OUT>(a, b, tw);
  return fft_pp_passes<N, NSEQ, T, DIR, NS * R, SWZ_OUT>(b, a, tw, RadixList<Rest...>{});
}

// FFT of the data in `a` (layout [i * NSEQ + s]) using `b` as the second
// buffer; returns a or b, holding the result in the same unswizzled layout.
template <int N, int NSEQ, int T, int DIR>
__device__ __forceinline__ float2* block_fft_pp(float2* a, float2* b, const float2* __restrict__ tw) {
  return fft_pp_passes<N, NSEQ, T, DIR, 1, 0>(a, b, tw, typename FftPlan<N>::type{});
}
// Same with an explicit radix plan (a RadixList whose product is N).
template <int N, int NSEQ, int T, int DIR, class Plan>
__device__ __forceinline__ float2* block_fft_pp_plan(float2* a, float2* b, const float2* __restrict__ tw) {
  return fft_pp_passes<N, NSEQ, T, DIR, 1, 0>(a, b, tw, Plan{});
}

// ---------------------------------------------------------------------------
// Ping-pong FFT with hooks: the first pass reads its inputs through `ld`
// (natural index, sequence) and the last pass writes its outputs through
// `st` (natural index, sequence, value) instead of the shared buffers, so a
// prologue (a spectrum product, the packed-real pre-processing, a load from
// global memory) or an epilogue (a threshold, a store to global memory) costs
// no extra shared-memory round trip or barrier.  Intermediate passes use a
// and b alternately (pass 1 writes b).  The first pass ends with a barrier
// like every pass, so `ld` may read the buffer the second pass writes.
// ---------------------------------------------------------------------------
template <typename RL>
struct RadixCount;
template <int... Rs>
struct RadixCount<RadixList<Rs...>> {
  static constexpr int value = sizeof...(Rs);
};
template <int N>
__host__ __device__ constexpr int fft_npasses() {
  return RadixCount<typename FftPlan<N>::type>::value;
}

template <int N, int NSEQ, int T, int R, int NS, int DIR, int SWZ_IN, int SWZ_OUT, class Rd, class Wr>
__device__ __forceinline__ void stockham_hook(const Rd& rd, const Wr& wr, const float2* __restrict__ tw) {
  constexpr int NB = N / R;
  constexpr int TOTAL = NB * NSEQ;
  constexpr int STEP = N / (NS * R);
#pragma unroll 2
  for (int w = threadIdx.x; w < TOTAL; w += T) {
    const int s = w % NSEQ;
    const int j = w / NSEQ;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = rd(swz_row<NSEQ, SWZ_IN>(j + r * NB), s);
    const int k = j % NS;
    if (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; r++) {
        float2 t = __ldg(&tw[r * k * STEP]);
        v[r] = DIR < 0 ? cmul(v[r], t) : cmulc(v[r], t);
      }
    }
    Dft<R, DIR>::run(v);
    const int base = (j / NS) * NS * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) wr(swz_row<NSEQ, SWZ_OUT>(base + r * NS), s, v[r]);
  }
  __syncthreads();
}

template <int N, int NSEQ, int T, int DIR, int NS, int SWZ_IN, class Ld, class St>
__device__ __forceinline__ void fft_hook_passes(float2*, float2*, const float2* __restrict__, const Ld&, const St&,
                                                RadixList<>) {}

template <int N, int NSEQ, int T, int DIR, int NS, int SWZ_IN, class Ld, class St, int R, int... Rest>
__device__ __forceinline__ void fft_hook_passes(float2* a, float2* b, const float2* __restrict__ tw, const Ld& ld,
                                                const St& st, RadixList<R, Rest...>) {
  constexpr bool first = NS == 1;
  constexpr bool last = sizeof...(Rest) == 0;
  constexpr int SWZ_OUT = (first && !last && R % 2 == 0) ? R : 0;
  auto rd = [&](int row, int s) -> float2 {
    if constexpr (first)
      return ld(row, s);
    else
      return a[row * NSEQ + s];
  };
  auto wr = [&](int row, int s, float2 v) {
    if constexpr (last)
      st(row, s, v);
    else
      b[row * NSEQ + s] = v;
  };
  stockham_hook<N, NSEQ, T, R, NS, DIR, SWZ_IN, SWZ_OUT>(rd, wr, tw);
  fft_hook_passes<N, NSEQ, T, DIR, NS * R, SWZ_OUT>(b, a, tw, ld, st, RadixList<Rest...>{});
}

// The buffer the last pass's default target would be (a for an even pass
// count, b for an odd one); an `st` writing shared memory writes there.
template <int N>
__device__ __forceinline__ float2* fft_hook_target(float2* a, float2* b) {
  return (fft_npasses<N>() & 1) ? b : a;
}

template <int N, int NSEQ, int T, int DIR, class Ld, class St>
__device__ __forceinline__ void block_fft_hook(float2* a, float2* b, const float2* __restrict__ tw, const Ld& ld,
                                               const St& st) {
  fft_hook_passes<N, NSEQ, T, DIR, 1, 0>(a, b, tw, ld, st, typename FftPlan<N>::type{});
}

// block_fft_hook with an explicit radix plan; the last pass's default target
// is plan_target<Plan>(a, b)
template <int N, int NSEQ, int T, int DIR, class Plan, class Ld, class St>
__device__ __forceinline__ void block_fft_hook_plan(float2* a, float2* b, const float2* __restrict__ tw,
                                                    const Ld& ld, const St& st) {
  fft_hook_passes<N, NSEQ, T, DIR, 1, 0>(a, b, tw, ld, st, Plan{});
}
template <int... Rs>
__host__ __device__ constexpr int plan_passes(RadixList<Rs...>) {
  return (int)sizeof...(Rs);
}
template <class Plan>
__device__ __forceinline__ float2* plan_target(float2* a, float2* b) {
  return (plan_passes(Plan{}) & 1) ? b : a;
}

// In-place variant of block_fft_hook on one buffer: every pass loads all of
// the thread's butterflies into registers, synchronises, then writes them
// back (two barriers per pass, half the shared memory of the ping-pong form,
// so more CTAs fit on an SM).  `st` of the last pass may write `buf`.
struct NoHook {
  __device__ __forceinline__ void operator()() const {}
};

// after_read runs once every thread has read the pass's inputs (after the
// pass's first barrier): the point from which the source may be overwritten.
// E: the element type, float2 (one sequence) or float4 (two sequences per
// element, NSEQ counting elements); the row swizzle is chosen for the row's
// width in bytes, so both forms place rows in the same banks.
template <int N, int NSEQ, int T, int R, int NS, int DIR, int SWZ_IN, int SWZ_OUT, class Rd, class Wr,
          class Hook = NoHook, class E = float2>
__device__ __forceinline__ void stockham_ip(const Rd& rd, const Wr& wr, const float2* __restrict__ tw,
                                            const Hook& after_read = Hook{}) {
  constexpr int NB = N / R;
  constexpr int TOTAL = NB * NSEQ;
  constexpr int IPT = (TOTAL + T - 1) / T;
  constexpr int STEP = N / (NS * R);
  constexpr int NSW = NSEQ * (int)(sizeof(E) / sizeof(float2));  // row width in float2 units
  E v[IPT][R];
#pragma unroll
  for (int it = 0; it < IPT; it++) {
    const int w = threadIdx.x + it * T;
    if (TOTAL % T == 0 || w < TOTAL) {
      const int s = w % NSEQ, j = w / NSEQ;
#pragma unroll
      for (int r = 0; r < R; r++) v[it][r] = rd(swz_row<NSW, SWZ_IN>(j + r * NB), s);
      const int k = j % NS;
      if (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; r++) v[it][r] = tw_mul<DIR>(v[it][r], tw, r * k * STEP);
      }
      Dft<R, DIR>::run(v[it]);
    }
  }
  __syncthreads();
  after_read();
#pragma unroll
  for (int it = 0; it < IPT; it++) {
    const int w = threadIdx.x + it * T;
    if (TOTAL % T == 0 || w < TOTAL) {
      const int s = w % NSEQ, j = w / NSEQ, k = j % NS;
      const int base = (j / NS) * NS * R + k;
#pragma unroll
      for (int r = 0; r < R; r++) wr(swz_row<NSW, SWZ_OUT>(base + r * NS), s, v[it][r]);
    }
  }
  __syncthreads();
}

template <int N, int NSEQ, int T, int DIR, int NS, int SWZ_IN, class E, class Ld, class St, class Hook>
__device__ __forceinline__ void fft_hook_ip_passes(E*, const float2* __restrict__, const Ld&, const St&,
                                                   const Hook&, RadixList<>) {}

template <int N, int NSEQ, int T, int DIR, int NS, int SWZ_IN, class E, class Ld, class St, class Hook, int R,
          int... Rest>
__device__ __forceinline__ void fft_hook_ip_passes(E* buf, const float2* __restrict__ tw, const Ld& ld,
                                                   const St& st, const Hook& hook, RadixList<R, Rest...>) {
  constexpr bool first = NS == 1;
  constexpr bool last = sizeof...(Rest) == 0;
  constexpr int SWZ_OUT = (first && !last && R % 2 == 0) ? R : 0;
  auto rd = [&](int row, int s) -> E {
    if constexpr (first)
      return ld(row, s);
    else
      return buf[row * NSEQ + s];
  };
  auto wr = [&](int row, int s, E v) {
    if constexpr (last)
      st(row, s, v);
    else
      buf[row * NSEQ + s] = v;
  };
  if constexpr (first)
    stockham_ip<N, NSEQ, T, R, NS, DIR, SWZ_IN, SWZ_OUT, decltype(rd), decltype(wr), Hook, E>(rd, wr, tw, hook);
  else
    stockham_ip<N, NSEQ, T, R, NS, DIR, SWZ_IN, SWZ_OUT, decltype(rd), decltype(wr), NoHook, E>(rd, wr, tw);
  fft_hook_ip_passes<N, NSEQ, T, DIR, NS * R, SWZ_OUT>(buf, tw, ld, st, hook, RadixList<Rest...>{});
}

// ---------------------------------------------------------------------------
// Transforms whose last pass accumulates into registers: acc(it, r, row, s, v)
// receives output (row, s) of the thread's (it, r) slot instead of a store.
// Every thread owns the same (row, s) slots on every call, so a running sum
// over many transforms (the band sum of a synthesis) can stay in registers.
// ---------------------------------------------------------------------------
template <class RL>
struct LastRadix;
template <int R>
struct LastRadix<RadixList<R>> {
  static constexpr int value = R;
};
template <int R, int R2, int... Rs>
struct LastRadix<RadixList<R, R2, Rs...>> {
  static constexpr int value = LastRadix<RadixList<R2, Rs...>>::value;
};

template <int... Rs>
__host__ __device__ constexpr int plan_product(RadixList<Rs...>) {
  return (1 * ... * Rs);
}

// The last pass of an in-place FFT whose outputs go to acc(it, r, row, s, v)
// (registers) instead of the buffer; see stockham_ip for the pass itself.
template <int N, int NSEQ, int T, int R, int NS, int DIR, int SWZ_IN, class Rd, class Acc>
__device__ __forceinline__ void stockham_last_acc(const Rd& rd, Acc& acc, const float2* __restrict__ tw) {
  constexpr int NB = N / R;
  constexpr int TOTAL = NB * NSEQ;
  constexpr int IPT = TOTAL / T;
  constexpr int STEP = N / (NS * R);
#pragma unroll
  for (int it = 0; it < IPT; it++) {
    const int w = threadIdx.x + it * T;
    const int s = w % NSEQ, j = w / NSEQ;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = rd(swz_row<NSEQ, SWZ_IN>(j + r * NB), s);
    const int k = j % NS;
    if (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; r++) {
        const float2 t = __ldg(&tw[r * k * STEP]);
        v[r] = DIR < 0 ? cmul(v[r], t) : cmulc(v[r], t);
      }
    }
    Dft<R, DIR>::run(v);
    const int base = (j / NS) * NS * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) acc(it, r, base + r * NS, s, v[r]);
  }
  __syncthreads();
}

// output row of accumulator (it, r) in the last pass (see stockham_last_acc)
template <int N, int NSEQ, int T, int R>
__device__ __forceinline__ int last_pass_row(int it, int r) {
  constexpr int NS = N / R;
  const int w = threadIdx.x + it * T;
  const int j = w / NSEQ;
  return (j / NS) * NS * R + (j % NS) + r * NS;
}

// The passes of an in-place FFT of NSEQ sequences in buf whose first pass
// reads its inputs through ld (then calls hook, once every thread has read
// them) and whose last pass, entered after pre_last(), accumulates through
// acc (stockham_last_acc).  At least two passes.
template <int N, int NSEQ, int T, int DIR, int NS, int SWZ_IN, class Ld, class Hook, class Pre, class Acc, int R,
          int... Rest>
__device__ __forceinline__ void fft_ld_acc_passes(float2* buf, const float2* __restrict__ tw, const Ld& ld,
                                                  const Hook& hook, const Pre& pre_last, Acc& acc,
                                                  RadixList<R, Rest...>) {
  static_assert(NS > 1 || sizeof...(Rest) > 0, "at least two passes");
  auto rd = [&](int row, int s) -> float2 {
    if constexpr (NS == 1)
      return ld(row, s);
    else
      return buf[row * NSEQ + s];
  };
  if constexpr (sizeof...(Rest) == 0) {
    pre_last();
    stockham_last_acc<N, NSEQ, T, R, NS, DIR, SWZ_IN>(rd, acc, tw);
  } else {
    constexpr int SWZ_OUT = (NS == 1 && R % 2 == 0) ? R : 0;
    auto wr = [&](int row, int s, float2 v) { buf[row * NSEQ + s] = v; };
    if constexpr (NS == 1)
      stockham_ip<N, NSEQ, T, R, NS, DIR, SWZ_IN, SWZ_OUT, decltype(rd), decltype(wr), Hook>(rd, wr, tw, hook);
    else
      stockham_ip<N, NSEQ, T, R, NS, DIR, SWZ_IN, SWZ_OUT>(rd, wr, tw);
    fft_ld_acc_passes<N, NSEQ, T, DIR, NS * R, SWZ_OUT>(buf, tw, ld, hook, pre_last, acc, RadixList<Rest...>{});
  }
}

// ---------------------------------------------------------------------------
// An inverse transform, an elementwise op on its output, and a forward
// transform with the same radix plan, where the plan's first and last radix
// are equal: the inverse transform's last pass leaves each thread exactly the
// values the forward transform's first pass needs (output r of butterfly j is
// index j + r N/R, the first pass's input r of butterfly j), so the turn from
// one transform to the other happens in registers, without a shared-memory
// round trip or a barrier.  op(v, flag) maps each value and may set a
// thread-local flag; the turn returns the block-wide OR of the flags (false:
// the forward transform has not run and buf holds the inverse transform's
// next-to-last pass).
// ---------------------------------------------------------------------------
template <class RL>
struct FirstRadix;
template <int R, int... Rs>
struct FirstRadix<RadixList<R, Rs...>> {
  static constexpr int value = R;
};
template <class RL>
struct TailRadices;
template <int R, int... Rs>
struct TailRadices<RadixList<R, Rs...>> {
  using type = RadixList<Rs...>;
};

// the turn pass: inverse last pass (radix R, NS = N / R), op, forward first pass
template <int N, int NSEQ, int T, int R, int SWZ_IN, int SWZ_OUT, class Op>
__device__ __forceinline__ bool stockham_turn(float2* buf, const float2* __restrict__ tw, const Op& op) {
  constexpr int NB = N / R;
  constexpr int TOTAL = NB * NSEQ;
  constexpr int IPT = (TOTAL + T - 1) / T;
  float2 v[IPT][R];
  bool flag = false;
#pragma unroll
  for (int it = 0; it < IPT; it++) {
    const int w = threadIdx.x + it * T;
    if (TOTAL % T == 0 || w < TOTAL) {
      const int s = w % NSEQ, j = w / NSEQ;
#pragma unroll
      for (int r = 0; r < R; r++) v[it][r] = buf[swz_row<NSEQ, SWZ_IN>(j + r * NB) * NSEQ + s];
#pragma unroll
      for (int r = 1; r < R; r++) v[it][r] = tw_mul<+1>(v[it][r], tw, r * j);  // NS = NB: k = j, STEP = 1
      Dft<R, +1>::run(v[it]);
#pragma unroll
      for (int r = 0; r < R; r++) v[it][r] = op(v[it][r], flag);
      Dft<R, -1>::run(v[it]);  // the forward first pass: no twiddles
    }
  }
  if (!__syncthreads_or(flag)) return false;  // every thread has read its inputs
#pragma unroll
  for (int it = 0; it < IPT; it++) {
    const int w = threadIdx.x + it * T;
    if (TOTAL % T == 0 || w < TOTAL) {
      const int s = w % NSEQ, j = w / NSEQ;
#pragma unroll
      for (int r = 0; r < R; r++) buf[swz_row<NSEQ, SWZ_OUT>(j * R + r) * NSEQ + s] = v[it][r];
    }
  }
  __syncthreads();
  return true;
}

template <int N, int NSEQ, int T, int NS, int SWZ_IN, class Plan, class Ld, class Op, int R, int... Rest>
__device__ __forceinline__ bool fft_inv_turn_passes(float2* buf, const float2* __restrict__ tw, const Ld& ld,
                                                    const Op& op, RadixList<R, Rest...>) {
  if constexpr (sizeof...(Rest) == 0) {
    static_assert(R == FirstRadix<Plan>::value, "the plan's first and last radix must be equal");
    constexpr int SWZ_OUT = R % 2 == 0 ? R : 0;  // the forward transform's first pass (not its last)
    return stockham_turn<N, NSEQ, T, R, SWZ_IN, SWZ_OUT>(buf, tw, op);
  } else {
    constexpr int SWZ_OUT = (NS == 1 && R % 2 == 0) ? R : 0;
    auto rd = [&](int row, int s) -> float2 {
      if constexpr (NS == 1)
        return ld(row, s);
      else
        return buf[row * NSEQ + s];
    };
    auto wr = [&](int row, int s, float2 v) { buf[row * NSEQ + s] = v; };
    stockham_ip<N, NSEQ, T, R, NS, +1, SWZ_IN, SWZ_OUT>(rd, wr, tw);
    return fft_inv_turn_passes<N, NSEQ, T, NS * R, SWZ_OUT, Plan>(buf, tw, ld, op, RadixList<Rest...>{});
  }
}

// inverse FFT (first pass reading through ld) -> op -> forward FFT (last pass
// storing through st), in place on buf; false (and no forward transform)
// when no thread set its flag
template <int N, int NSEQ, int T, class Ld, class Op, class St>
__device__ __forceinline__ bool block_fft_inv_op_fwd(float2* buf, const float2* __restrict__ tw, const Ld& ld,
                                                     const Op& op, const St& st) {
  using Plan = typename FftPlan<N>::type;
  constexpr int RF = FirstRadix<Plan>::value;
  if (!fft_inv_turn_passes<N, NSEQ, T, 1, 0, Plan>(buf, tw, ld, op, Plan{})) return false;
  auto rd = [&](int row, int s) -> float2 { return buf[row * NSEQ + s]; };  // (the passes read buf)
  fft_hook_ip_passes<N, NSEQ, T, -1, RF, RF % 2 == 0 ? RF : 0>(buf, tw, rd, st, NoHook{},
                                                                typename TailRadices<Plan>::type{});
  return true;
}

// An FFT of NSEQ sequences whose inputs are already in registers in the
// layout a last pass of the same radix leaves them (stockham_last_acc: slot
// (it, r) of a thread holds row j + r N/R of column s, w = tid + it T, j =
// w / NSEQ, s = w % NSEQ), which is the first pass's input layout when the
// plan's first radix is R: the first pass runs on the registers and writes
// buf, the rest are the engine's, the last storing through st.
template <int N, int NSEQ, int T, int DIR, int R, int IPT, class St>
__device__ __forceinline__ void block_fft_from_regs(float2* buf, const float2* __restrict__ tw,
                                                    const float2 (&v)[IPT][R], const St& st) {
  using Plan = typename FftPlan<N>::type;
  static_assert(FirstRadix<Plan>::value == R, "the plan's first radix must be the registers' radix");
  constexpr int NB = N / R;
  static_assert(NB * NSEQ == IPT * T, "every thread owns IPT first-pass butterflies");
  constexpr int SWZ = R % 2 == 0 ? R : 0;  // the first pass's output swizzle (as stockham_ip)
#pragma unroll
  for (int it = 0; it < IPT; it++) {
    const int w = threadIdx.x + it * T;
    const int s = w % NSEQ, j = w / NSEQ;
    float2 u[R];
#pragma unroll
    for (int r = 0; r < R; r++) u[r] = v[it][r];
    Dft<R, DIR>::run(u);  // first pass: no twiddles
#pragma unroll
    for (int r = 0; r < R; r++) buf[swz_row<NSEQ, SWZ>(j * R + r) * NSEQ + s] = u[r];
  }
  __syncthreads();
  auto rd = [&](int row, int sq) -> float2 { return buf[row * NSEQ + sq]; };  // (the passes read buf)
  fft_hook_ip_passes<N, NSEQ, T, DIR, R, SWZ>(buf, tw, rd, st, NoHook{}, typename TailRadices<Plan>::type{});
}

// after_first_read: called once the first pass has read all of its inputs
// through ld (e.g. to start refilling the buffer ld reads from).  buf holds
// float2 (NSEQ sequences) or float4 (2 NSEQ sequences, two per element).
template <int N, int NSEQ, int T, int DIR, class E, class Ld, class St, class Hook = NoHook>
__device__ __forceinline__ void block_fft_hook_ip(E* buf, const float2* __restrict__ tw, const Ld& ld,
                                                  const St& st, const Hook& after_first_read = Hook{}) {
  fft_hook_ip_passes<N, NSEQ, T, DIR, 1, 0>(buf, tw, ld, st, after_first_read, typename FftPlan<N>::type{});
}

// block_fft_hook_ip with an explicit radix plan (a RadixList whose product is N)
template <int N, int NSEQ, int T, int DIR, class Plan, class E, class Ld, class St, class Hook = NoHook>
__device__ __forceinline__ void block_fft_hook_ip_plan(E* buf, const float2* __restrict__ tw, const Ld& ld,
                                                       const St& st, const Hook& after_first_read = Hook{}) {
  fft_hook_ip_passes<N, NSEQ, T, DIR, 1, 0>(buf, tw, ld, st, after_first_read, Plan{});
}

// 16-byte asynchronous global -> shared copies (cp.async, sm_80+)
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
// 8-byte asynchronous global -> shared copy (one float2)
__device__ __forceinline__ void cp_async8(void* smem_dst, const void* gmem_src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
// 4-byte asynchronous global -> shared copy (one float)
__device__ __forceinline__ void cp_async4(void* smem_dst, const void* gmem_src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Out-of-place packed-real post-processing (after a forward FFT of the
// W/2-point complex view); see r2c_post for the formulas.
template <int WH, int NSEQ, int LD, int T>
__device__ __forceinline__ void r2c_post_pp(const float2* __restrict__ in, float2* __restrict__ out,
                                            const float2* __restrict__ twW) {
  constexpr int TOTAL = (WH / 2 + 1) * NSEQ;
  for (int w = threadIdx.x; w < TOTAL; w += T) {
    const int s = w % NSEQ, k = w / NSEQ;
    const float2 zk = in[k * LD + s];
    if (k == 0) {
      out[s] = make_float2(zk.x + zk.y, zk.x - zk.y);
    } else {
      const float2 zmc = cconj(in[(WH - k) * LD + s]);
      const float2 E = cscale(cadd(zk, zmc), 0.5f);
      const float2 d = cscale(csub(zk, zmc), 0.5f);
      const float2 O = make_float2(d.y, -d.x);
      const float2 To = cmul(__ldg(&twW[k]), O);
      out[k * LD + s] = cadd(E, To);
      if (k != WH - k) out[(WH - k) * LD + s] = cconj(csub(E, To));
    }
  }
  __syncthreads();
}

// Out-of-place packed-real pre-processing (before an inverse FFT); see c2r_pre.
template <int WH, int NSEQ, int LD, int T>
__device__ __forceinline__ void c2r_pre_pp(const float2* __restrict__ in, float2* __restrict__ out,
                                           const float2* __restrict__ twW) {
  constexpr int TOTAL = (WH / 2 + 1) * NSEQ;
  for (int w = threadIdx.x; w < TOTAL; w += T) {
    const int s = w % NSEQ, k = w / NSEQ;
    const float2 xk = in[k * LD + s];
    if (k == 0) {
      out[s] = make_float2(xk.x + xk.y, xk.x - xk.y);
    } else {
      const float2 xmc = cconj(in[(WH - k) * LD + s]);
      const float2 E = cadd(xk, xmc);
      const float2 O = cmulc(csub(xk, xmc), __ldg(&twW[k]));
      const float2 iO = make_float2(-O.y, O.x);
      out[k * LD + s] = cadd(E, iO);
      if (k != WH - k) out[(WH - k) * LD + s] = cconj(csub(E, iO));
    }
  }
  __syncthreads();
}

}  // namespace nsst
