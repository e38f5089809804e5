// 3-D NSST plan and the C ABI of the volume path declared in include/nsst.h.
//
// The reference runs this path as MATLAB glue around cuFFT
// (shearcuda3d/DenoiseDemo/main.m:80-145, ShDecThRec_cuda.cpp:178-335): every
// call builds cuFFT plans, re-transforms every directional filter, and pads
// and crops through three temporary arrays per band.  Here the plan owns,
// once: the FP64-built Meyer filters' convolution spectra in FP32 on the
// device, the pyramid windows, the twiddle tables, and every work buffer for
// a batch of volumes; an execute call is a fixed sequence of launches on the
// caller's stream over all volumes of the batch at once.
//
// Pipeline of one level of the directional stage (convnfft.m:79-201, 'same'):
//   Y = FFT3(zero-pad(BP_l, Lc))            once per level
//   W = F_a .* Y + i F_b .* Y               two real filters per complex IFFT
//   IFFT3(W); real part -> band a, imaginary part -> band b, cropped at
//   offset ceil((24-1)/2) = 12; hard threshold and band sum (ShRec.m:11-24).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <random>
#include <memory>
#include <thread>

#include "internal.h"

using namespace nsst;

namespace {

constexpr int kCube = 24;          // Meyer filter support (GetMeyerBasedFilter.m:18)
constexpr int kSameOff = 12;       // convnfft 'same' offset: ceil((24 - 1) / 2)
constexpr int kMaxGrid = 192;      // largest padded grid per dimension
const int kFftLens[] = {16, 24, 32, 48, 64, 72, 96, 128, 144, 192, 216, 256};

bool is_fft_len(int n) {
  for (int v : kFftLens)
    if (v == n) return true;
  return false;
}
// Smallest supported circular-convolution length for the 'same' part of a
// linear convolution of m samples with the 24-tap filter: outputs 12 .. m+11
// alias no wrapped tap once N >= m + 12 (taps reach 23 back and 11 ahead of
// the kept range), so the full m + 23 is not needed.
int conv_len(int m) {
  for (int v : kFftLens)
    if (v >= m + kSameOff) return v;
  return -1;
}

nsst_status fail3(nsst_status s, const std::string& msg) {
  set_error(msg);
  return s;
}
nsst_status cuda_fail3(cudaError_t e, const char* what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? NSST_ERR_OUT_OF_MEMORY : NSST_ERR_CUDA;
}
#define V3_CUDA(call)                                    \
  do {                                                   \
    cudaError_t _e = (call);                             \
    if (_e != cudaSuccess) return cuda_fail3(_e, #call); \
  } while (0)
#define V3_TRY(call)              \
  do {                            \
    nsst_status _s = (call);      \
    if (_s != NSST_OK) return _s; \
  } while (0)

// PyrNDDec_mm.m:58-74: w, tbw and D of each level for a pyramid mode
bool pyr_params(double mode, int L, double* w, double* tbw, double* D) {
  double w0, w1, t0, t1, d0, d1;
  if (mode == 1.0) {
    w0 = 0.5, w1 = 0.25, t0 = 1.0 / 6, t1 = 1.0 / 12, d0 = 1.0, d1 = 2.0;
  } else if (mode == 1.5) {
    w0 = 0.5, w1 = 3.0 / 8, t0 = 1.0 / 7, t1 = 1.0 / 9, d0 = 1.5, d1 = 2.0;
  } else if (mode == 2.0) {
    w0 = w1 = 1.0 / 3, t0 = t1 = 1.0 / 7, d0 = d1 = 2.0;
  } else {
    return false;
  }
  for (int l = 0; l < L; l++) {
    w[l] = l ? w1 : w0;
    tbw[l] = l ? t1 : t0;
    D[l] = l ? d1 : d0;
  }
  return true;
}

// Level sizes of a grid g: g, g/D0, g/D0/D1, ...; false if one is not an
// integer supported transform length or its convolution length is missing.
bool level_sizes(int g, int L, const double* D, int* out) {
  double v = g;
  out[0] = g;
  if (!is_fft_len(g) || conv_len(g) < 0) return false;
  for (int l = 0; l < L; l++) {
    v /= D[l];
    const int iv = (int)std::lround(v);
    if (std::fabs(v - iv) > 1e-9 || !is_fft_len(iv) || iv % 8) return false;
    if (l + 1 < L && conv_len(iv) < 0) return false;
    out[l + 1] = iv;
  }
  return true;
}

// The grid of MarshalData.m:3-22 (the reference's any-size demo,
// mainAnySize.m:51): every dimension gains d - rem(n, d) planes, d = 3 2^(L-1)
// (divFactor [3 6 12 24] of the level count), so that Pyr_mode 1.5's level
// sizes g, g/1.5, g/3, ... are integers.  Its level sizes need transform
// lengths with other prime factors (132 = 3 * 4 * 11, 204 = 3 * 4 * 17); the
// pass kernels hold sequence groups that need not divide them.
const int kOddLens[] = {22, 34, 44, 68, 88, 132, 136, 204};
bool is_pyr_len(int n) {
  if (is_fft_len(n)) return true;
  for (int v : kOddLens)
    if (v == n) return true;
  return false;
}
int marshal_grid(int n, int L) {
  const int d = 3 << (L - 1);
  return n + d - n % d;
}
bool marshal_sizes(int g, int L, const double* D, int* out, int* missing) {
  double v = g;
  out[0] = g;
  *missing = 0;
  if (!is_pyr_len(g) || conv_len(g) < 0) {
    *missing = g;
    return false;
  }
  for (int l = 0; l < L; l++) {
    v /= D[l];
    const int iv = (int)std::lround(v);
    if (std::fabs(v - iv) > 1e-9 || !is_pyr_len(iv) || (l + 1 < L && conv_len(iv) < 0)) {
      *missing = iv;
      return false;
    }
    out[l + 1] = iv;
  }
  return true;
}

// Smallest supported grid >= n for which every level size works.
int grid_size(int n, int L, const double* D) {
  int tmp[NSST_MAX_LEVELS + 1];
  for (int g : kFftLens)
    if (g >= n && g <= kMaxGrid && level_sizes(g, L, D, tmp)) return g;
  return -1;
}

// row pitch of the keep bits along the box's last dimension: a multiple of 8,
// so that the eight sequences of a pass group fill whole bytes
int mask_pitch(int m2) { return (m2 + 7) / 8 * 8; }

int host_threads3() {
  unsigned n = std::thread::hardware_concurrency();
  return n == 0 ? 4 : (int)std::min(n, 16u);
}

size_t align_up3(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

struct nsst3_plan {
  nsst3_config cfg{};
  int n[3] = {0, 0, 0};  // volume dims
  int g[3] = {0, 0, 0};  // padded grid
  int L = 0, B = 1, nbands = 0, device = 0;
  double w[NSST_MAX_LEVELS], tbw[NSST_MAX_LEVELS], D[NSST_MAX_LEVELS];

  struct Level {
    int m[3] = {0, 0, 0};   // band-pass dims (level L: lowpass)
    int lc[3] = {0, 0, 0};  // convolution FFT lengths (levels < L)
    int nd = 0, nb = 0, first_band = 0;
    size_t bp_off = 0;      // floats, in the sub-band layout
    size_t xh_off = 0;      // float2, in one volume's half-spectrum block
    size_t spec_off = 0;    // float2, first band's spectrum
    int K[3] = {0, 0, 0};   // window support of the decomposition step (levels < L)
    size_t win_off[3] = {0, 0, 0};
    size_t vol() const { return (size_t)m[0] * m[1] * m[2]; }
    size_t half() const { return (size_t)m[0] * m[1] * (m[2] / 2 + 1); }
    size_t conv() const { return (size_t)lc[0] * lc[1] * lc[2]; }
  };
  std::vector<Level> lev;  // L + 1 entries
  std::vector<int> band_level, band_cone, band_l2, band_l1;

  size_t bp_floats = 0;    // sub-band layout per volume
  size_t vol_elems = 0;    // complex scratch volume per item (grid)
  size_t xh_elems = 0;     // half spectra of every level per item
  size_t conv_elems = 0;   // largest convolution volume
  size_t in_elems = 0;     // n0 n1 n2

  char* arena = nullptr;
  size_t arena_bytes = 0;
  float2* spec = nullptr;
  float* win = nullptr;
  float2* tw = nullptr;
  std::map<int, size_t> tw_off;  // transform length -> offset (float2) in tw
  float2* vol = nullptr;
  float2* xh = nullptr;
  float2* Y = nullptr;
  float2* Wk = nullptr;
  float* bp = nullptr;
  float* rbp = nullptr;
  float* th = nullptr;

  // differentiation: keep bits of every band of the last thresholded forward
  uint8_t* mask = nullptr;
  size_t mask_bytes = 0;            // per item
  std::vector<size_t> mask_off;     // per band, in bytes (bit k = voxel k of the band, linear order)
  int masks_valid_n = 0;            // items covered by the stored masks (0 = none)

  std::vector<double> scalars;
  bool has_scalars = false;
  std::vector<float> th_host;
  std::mutex mu;

  const float2* twid(int len) const { return tw + tw_off.at(len); }
};

namespace {

// Pass descriptors.  A pass transforms `axis`; (a, b) select the sequences
// (axis 2: x, y; axis 1: x, z; axis 0: y, z), `in` the loaded index range and
// `out` the stored one.
struct Range {
  int lo, n;
};
V3Pass make_pass(int axis, const int* D, size_t stride, Range a, Range b, Range in, Range out) {
  V3Pass P;
  P.axis = axis;
  P.D1 = D[1];
  P.D2 = D[2];
  P.a_lo = a.lo, P.a_n = a.n, P.b_lo = b.lo, P.b_n = b.n;
  P.in_lo = in.lo, P.in_n = in.n, P.out_lo = out.lo, P.out_n = out.n;
  P.item_stride = stride;
  return P;
}
void set_box(V3Pass& P, const int* m, int o) {
  P.r1 = m[1];
  P.r2 = m[2];
  P.o0 = P.o1 = P.o2 = o;
}

nsst_status run_pass(nsst3_plan* p, const V3Pass& P, int dir, int ld, int st_mode, float2* out, const float2* in,
                     int D_axis, int n, cudaStream_t st) {
  V3_CUDA(launch_v3_pass(D_axis, dir, ld, st_mode, out, in, P, p->twid(D_axis), n, st));
  return NSST_OK;
}

// Batched full 3-D FFT of n complex volumes d0 x d1 x d2 (item stride
// `stride`), in place: axis 2, then 1, then 0; unnormalised.
nsst_status fft3(nsst3_plan* p, float2* v, size_t stride, int n, const int* d, int dir, cudaStream_t st) {
  V3_TRY(run_pass(p, make_pass(2, d, stride, {0, d[0]}, {0, d[1]}, {0, d[2]}, {0, d[2]}), dir, V3_LD_CPLX, V3_ST_CPLX,
                  v, v, d[2], n, st));
  V3_TRY(run_pass(p, make_pass(1, d, stride, {0, d[0]}, {0, d[2]}, {0, d[1]}, {0, d[1]}), dir, V3_LD_CPLX, V3_ST_CPLX,
                  v, v, d[1], n, st));
  V3_TRY(run_pass(p, make_pass(0, d, stride, {0, d[1]}, {0, d[2]}, {0, d[0]}, {0, d[0]}), dir, V3_LD_CPLX, V3_ST_CPLX,
                  v, v, d[0], n, st));
  return NSST_OK;
}

// Forward FFT of real volumes of dims m (item stride rstride floats) zero
// padded at the origin to the complex buffer v of dims d: the passes read
// only the non-zero part.
nsst_status fft3_real(nsst3_plan* p, const float* x, size_t rstride, const int* m, float2* v, size_t stride,
                      const int* d, int n, cudaStream_t st) {
  V3Pass P = make_pass(2, d, stride, {0, m[0]}, {0, m[1]}, {0, m[2]}, {0, d[2]});
  P.rsrc = x;
  P.r_stride = rstride;
  set_box(P, m, 0);
  V3_TRY(run_pass(p, P, -1, V3_LD_REAL, V3_ST_CPLX, v, v, d[2], n, st));
  V3_TRY(run_pass(p, make_pass(1, d, stride, {0, m[0]}, {0, d[2]}, {0, m[1]}, {0, d[1]}), -1, V3_LD_CPLX, V3_ST_CPLX,
                  v, v, d[1], n, st));
  V3_TRY(run_pass(p, make_pass(0, d, stride, {0, d[1]}, {0, d[2]}, {0, m[0]}, {0, d[0]}), -1, V3_LD_CPLX, V3_ST_CPLX,
                  v, v, d[0], n, st));
  return NSST_OK;
}

// Inverse FFT of the complex buffer v (dims d) whose real part, times scale,
// is wanted only in the box [o, o + m) of each axis: later passes skip the
// sequences outside the box, the last one writes the real box to x.
nsst_status ifft3_real_box(nsst3_plan* p, float2* v, size_t stride, const int* d, const int* m, int o, float* x,
                           size_t rstride, float scale, int n, cudaStream_t st) {
  V3_TRY(run_pass(p, make_pass(2, d, stride, {0, d[0]}, {0, d[1]}, {0, d[2]}, {o, m[2]}), +1, V3_LD_CPLX, V3_ST_CPLX,
                  v, v, d[2], n, st));
  V3_TRY(run_pass(p, make_pass(1, d, stride, {0, d[0]}, {o, m[2]}, {0, d[1]}, {o, m[1]}), +1, V3_LD_CPLX, V3_ST_CPLX,
                  v, v, d[1], n, st));
  V3Pass P = make_pass(0, d, stride, {o, m[1]}, {o, m[2]}, {0, d[0]}, {o, m[0]});
  P.rdst = x;
  P.r_stride = rstride;
  P.scale = scale;
  set_box(P, m, o);
  return run_pass(p, P, +1, V3_LD_CPLX, V3_ST_REAL, v, v, d[0], n, st);
}

PyrWin level_window(const nsst3_plan* p, int l) {
  const nsst3_plan::Level& a = p->lev[l];
  PyrWin w;
  for (int k = 0; k < 3; k++) {
    w.K[k] = a.K[k];
    w.nr[k] = a.m[k];
  }
  w.v0 = p->win + a.win_off[0];
  w.v1 = p->win + a.win_off[1];
  w.v2 = p->win + a.win_off[2];
  return w;
}

// PyrNDDec_mm.m:20-109 (OutD 'S') for n volumes x (dims in[3], padded to the
// grid by edge replication, or by zeros for the adjoint) into the sub-band
// layout bp (item stride bp_floats).
nsst_status run_pyr_dec(nsst3_plan* p, const float* x, const int* in, float* bp, int n, cudaStream_t st,
                        bool zero_pad = false) {
  const size_t xs = (size_t)in[0] * in[1] * in[2];
  const nsst3_plan::Level& l0 = p->lev[0];
  if (zero_pad)
    V3_CUDA(launch_pad_real(x, xs, p->vol, p->vol_elems, n, in[0], in[1], in[2], p->g[0], p->g[1], p->g[2], st));
  else
    V3_CUDA(launch_pad_edge(x, xs, p->vol, p->vol_elems, n, in[0], in[1], in[2], p->g[0], p->g[1], p->g[2], st));
  V3_TRY(fft3(p, p->vol, p->vol_elems, n, p->g, -1, st));
  V3_CUDA(launch_half(p->vol, p->vol_elems, p->xh + l0.xh_off, p->xh_elems, n, p->g[0], p->g[1], p->g[2], st));
  for (int l = 0; l <= p->L; l++) {
    const nsst3_plan::Level& a = p->lev[l];
    if (l < p->L) {
      const nsst3_plan::Level& b = p->lev[l + 1];
      // PrySDdec_onestep.m:82-125: Lp into the next level's block, Hp in place
      V3_CUDA(launch_pyr_dec(p->xh + a.xh_off, p->xh_elems, p->xh + b.xh_off, p->xh_elems, n, a.m[0], a.m[1], a.m[2],
                             b.m[0], b.m[1], b.m[2], level_window(p, l), (float)(1.0 / std::pow(p->D[l], 1.5)), st));
    }
    // subs{l} = real(ifftn(ccsym(Hp, 3, 'e')))   (lowpass: the last Lp)
    V3_CUDA(launch_conj_extend(p->xh + a.xh_off, p->xh_elems, p->vol, p->vol_elems, n, a.m[0], a.m[1], a.m[2], st));
    V3_TRY(ifft3_real_box(p, p->vol, p->vol_elems, a.m, a.m, 0, bp + a.bp_off, p->bp_floats,
                          (float)(1.0 / (double)a.vol()), n, st));
  }
  return NSST_OK;
}

// PyrNDRec_mm.m:20-95 (InD 'S'): bp -> x (dims out[3], the grid cropped).
nsst_status run_pyr_rec(nsst3_plan* p, const float* bp, float* x, const int* out, int n, cudaStream_t st) {
  for (int l = p->L; l >= 0; l--) {
    const nsst3_plan::Level& a = p->lev[l];
    // ccsym(fftn(subs{l}), 3, 'c')
    V3_TRY(fft3_real(p, bp + a.bp_off, p->bp_floats, a.m, p->vol, p->vol_elems, a.m, n, st));
    V3_CUDA(launch_half(p->vol, p->vol_elems, p->xh + a.xh_off, p->xh_elems, n, a.m[0], a.m[1], a.m[2], st));
    if (l < p->L) {
      const nsst3_plan::Level& b = p->lev[l + 1];
      // PrySDrec_onestep.m:96-119, in place over Hp
      V3_CUDA(launch_pyr_rec(p->xh + a.xh_off, p->xh_elems, p->xh + b.xh_off, p->xh_elems, n, a.m[0], a.m[1], a.m[2],
                             b.m[0], b.m[1], b.m[2], level_window(p, l), (float)std::pow(p->D[l], 1.5), st));
    }
  }
  const nsst3_plan::Level& l0 = p->lev[0];
  V3_CUDA(launch_conj_extend(p->xh + l0.xh_off, p->xh_elems, p->vol, p->vol_elems, n, p->g[0], p->g[1], p->g[2], st));
  V3_TRY(fft3(p, p->vol, p->vol_elems, n, p->g, +1, st));
  V3_CUDA(launch_crop_real(p->vol, p->vol_elems, x, (size_t)out[0] * out[1] * out[2], n, out[0], out[1], out[2],
                           p->g[1], p->g[2], 0, 0, 0, (float)(1.0 / (double)l0.vol()), st));
  return NSST_OK;
}

// Directional stage of one level.  Y = FFT3(zero-pad(bp_l)) once; per band
// pair, W = IFFT3(Y .* C) with C = F_a + i F_b, cut to the 'same' box at
// offset 12.  acc != NULL: hard threshold (th, or none when th is NULL) and
// band sum into acc (sub-band layout, level l region, item stride
// bp_floats), with keep bits when record_masks.  acc == NULL: band
// coefficients into coeffs (nb volumes of the level per item).
nsst_status run_sh_level(nsst3_plan* p, const float* bp, int l, float* acc, const float* th, float* coeffs, int n,
                         cudaStream_t st, bool record_masks = false) {
  const nsst3_plan::Level& a = p->lev[l];
  const int* N = a.lc;
  const int* m = a.m;
  const int o = kSameOff;
  const size_t cs = p->conv_elems;
  V3_TRY(fft3_real(p, bp + a.bp_off, p->bp_floats, m, p->Y, cs, N, n, st));
  const float scale = (float)(1.0 / (double)a.conv());
  for (int k = 0; k < a.nb; k += 2) {
    const int ba = a.first_band + k;
    const int bb = k + 1 < a.nb ? ba + 1 : -1;
    const float2* C = p->spec + a.spec_off + (size_t)(k / 2) * a.conv();
    // z rows: the product, stored only where the box needs it
    V3Pass P1 = make_pass(2, N, cs, {0, N[0]}, {0, N[1]}, {0, N[2]}, {o, m[2]});
    P1.spec = C;
    V3_TRY(run_pass(p, P1, +1, V3_LD_PAIR, V3_ST_CPLX, p->Wk, p->Y, N[2], n, st));
    V3_TRY(run_pass(p, make_pass(1, N, cs, {0, N[0]}, {o, m[2]}, {0, N[1]}, {o, m[1]}), +1, V3_LD_CPLX, V3_ST_CPLX,
                    p->Wk, p->Wk, N[1], n, st));
    V3Pass P3 = make_pass(0, N, cs, {o, m[1]}, {o, m[2]}, {0, N[0]}, {o, m[0]});
    set_box(P3, m, o);
    P3.r_stride = p->bp_floats;
    P3.scale = scale;
    if (acc) {
      P3.rdst = acc + a.bp_off;
      P3.th = th;
      P3.ia = ba;
      P3.ib = bb;
      P3.nb_item = p->nbands;
      if (record_masks) {
        P3.m_r2 = mask_pitch(m[2]);
        P3.mwa = p->mask + p->mask_off[ba];
        P3.mwb = bb >= 0 ? p->mask + p->mask_off[bb] : nullptr;
        P3.m_stride = p->mask_bytes;
      }
      V3_TRY(run_pass(p, P3, +1, V3_LD_CPLX, V3_ST_THRESH, p->Wk, p->Wk, N[0], n, st));
    } else {
      P3.rdst = coeffs + (size_t)k * a.vol();
      P3.rdst2 = bb >= 0 ? P3.rdst + a.vol() : nullptr;
      P3.r_stride = (size_t)a.nb * a.vol();
      V3_TRY(run_pass(p, P3, +1, V3_LD_CPLX, V3_ST_PAIR, p->Wk, p->Wk, N[0], n, st));
    }
  }
  return NSST_OK;
}

// th[i * nbands + b] = T[level(b)] * sigma_i * scalars[b]  (ThresholdShCoeff.m:7)
nsst_status upload_th(nsst3_plan* p, int n, const double* sigma, const double* T, const double* scalars,
                      cudaStream_t st) {
  if (!sigma || !T) return fail3(NSST_ERR_INVALID_ARG, "sigma and T are required");
  if (!scalars) {
    if (!p->has_scalars) return fail3(NSST_ERR_INVALID_ARG, "no band scalars given or stored in the plan");
    scalars = p->scalars.data();
  }
  p->th_host.resize((size_t)n * p->nbands);
  for (int i = 0; i < n; i++)
    for (int b = 0; b < p->nbands; b++)
      p->th_host[(size_t)i * p->nbands + b] = (float)(T[p->band_level[b]] * sigma[i] * scalars[b]);
  // pageable source: the copy is staged before the call returns
  V3_CUDA(cudaMemcpyAsync(p->th, p->th_host.data(), p->th_host.size() * sizeof(float), cudaMemcpyHostToDevice, st));
  return NSST_OK;
}

// ShDecThRec_cuda: rec (sub-band layout) = per level sum of thresholded
// bands; lowpass copied from bp.
nsst_status run_dec_thresh_rec(nsst3_plan* p, const float* bp, float* rec, int n, const float* th, cudaStream_t st,
                               bool record_masks = false) {
  V3_CUDA(cudaMemsetAsync(rec, 0, (size_t)n * p->bp_floats * sizeof(float), st));
  for (int l = 0; l < p->L; l++) V3_TRY(run_sh_level(p, bp, l, rec, th, nullptr, n, st, record_masks));
  const nsst3_plan::Level& lp = p->lev[p->L];
  V3_CUDA(cudaMemcpy2DAsync(rec + lp.bp_off, p->bp_floats * sizeof(float), bp + lp.bp_off,
                            p->bp_floats * sizeof(float), lp.vol() * sizeof(float), n, cudaMemcpyDeviceToDevice, st));
  return NSST_OK;
}

nsst_status check_call(nsst3_plan* p, int n, const void* a, const void* b) {
  if (!p) return fail3(NSST_ERR_INVALID_ARG, "NULL plan");
  if (n < 1 || n > p->B) return fail3(NSST_ERR_INVALID_ARG, "n must be in [1, batch capacity]");
  if (!a || !b) return fail3(NSST_ERR_INVALID_ARG, "NULL buffer");
  if (((uintptr_t)a & 3) || ((uintptr_t)b & 3)) return fail3(NSST_ERR_INVALID_ARG, "buffers must be 4-byte aligned");
  if (cudaSetDevice(p->device) != cudaSuccess) return fail3(NSST_ERR_CUDA, "cudaSetDevice failed");
  return NSST_OK;
}

}  // namespace

extern "C" {

int nsst3_meyer_filters(int nlevels, const int* num_dirs, double* out) {
  if (nlevels < 1 || nlevels > NSST_MAX_LEVELS || !num_dirs) return -1;
  int count = 0;
  for (int l = 0; l < nlevels; l++) {
    const int nd = num_dirs[l];
    if (nd < 2 || nd > 12 || kCube % nd) return -1;
    count += 3 * nd * nd;
  }
  if (out) {
    std::vector<double> f = meyer_filters_3d(kCube, nlevels, num_dirs);
    std::memcpy(out, f.data(), f.size() * sizeof(double));
  }
  return count;
}

nsst_status nsst3_plan_create(const nsst3_config* cfg, int n0, int n1, int n2, int batch, nsst3_plan** out) {
  if (!out) return fail3(NSST_ERR_INVALID_ARG, "NULL output pointer");
  *out = nullptr;
  if (!cfg) return fail3(NSST_ERR_INVALID_ARG, "config is NULL");
  if (cfg->nlevels < 1 || cfg->nlevels > 4) return fail3(NSST_ERR_INVALID_ARG, "nlevels must be in [1, 4]");
  if (batch < 1) return fail3(NSST_ERR_INVALID_ARG, "batch must be >= 1");
  if (nsst3_meyer_filters(cfg->nlevels, cfg->num_dirs, nullptr) < 0)
    return fail3(NSST_ERR_INVALID_ARG, "num_dirs must divide 24 and lie in [2, 12]");
  auto p = std::make_unique<nsst3_plan>();
  p->cfg = *cfg;
  p->L = cfg->nlevels;
  p->B = batch;
  if (!pyr_params(cfg->pyr_mode, p->L, p->w, p->tbw, p->D))
    return fail3(NSST_ERR_INVALID_ARG, "pyr_mode must be 1, 1.5 or 2");
  const int dims[3] = {n0, n1, n2};
  int sizes[3][NSST_MAX_LEVELS + 1];
  if (cfg->grid != NSST3_GRID_FAST && cfg->grid != NSST3_GRID_MARSHAL)
    return fail3(NSST_ERR_INVALID_ARG, "grid must be NSST3_GRID_FAST or NSST3_GRID_MARSHAL");
  if (cfg->grid == NSST3_GRID_MARSHAL && cfg->pyr_mode != 1.5)
    return fail3(NSST_ERR_INVALID_ARG, "NSST3_GRID_MARSHAL pads for Pyr_mode 1.5 (MarshalData.m's divFactor)");
  for (int k = 0; k < 3; k++) {
    if (dims[k] < 1) return fail3(NSST_ERR_INVALID_ARG, "volume dims must be positive");
    p->n[k] = dims[k];
    if (cfg->grid == NSST3_GRID_MARSHAL) {
      p->g[k] = marshal_grid(dims[k], p->L);
      int miss = 0;
      if (!marshal_sizes(p->g[k], p->L, p->D, sizes[k], &miss))
        return fail3(NSST_ERR_UNSUPPORTED_SIZE,
                     "MarshalData grid " + std::to_string(p->g[k]) + " of dimension " + std::to_string(dims[k]) +
                         " needs transform length " + std::to_string(miss) +
                         ", not compiled (level sizes of the 132 and 204 grids and the 2^a 3^b lengths are)");
    } else {
      p->g[k] = grid_size(dims[k], p->L, p->D);
      if (p->g[k] < 0 || !level_sizes(p->g[k], p->L, p->D, sizes[k]))
        return fail3(NSST_ERR_UNSUPPORTED_SIZE, "volume dimension too large for this pyramid (grid <= 192)");
    }
  }
  V3_CUDA(cudaGetDevice(&p->device));
  p->in_elems = (size_t)n0 * n1 * n2;

  // level geometry, band tables and layout offsets
  p->lev.resize(p->L + 1);
  size_t bp_off = 0, xh_off = 0, spec_off = 0, win_off = 0;
  for (int l = 0; l <= p->L; l++) {
    nsst3_plan::Level& a = p->lev[l];
    for (int k = 0; k < 3; k++) a.m[k] = sizes[k][l];
    a.bp_off = bp_off;
    bp_off += align_up3(a.vol(), 64);
    a.xh_off = xh_off;
    xh_off += align_up3(a.half(), 32);
    if (l == p->L) break;
    for (int k = 0; k < 3; k++) a.lc[k] = conv_len(a.m[k]);
    a.nd = cfg->num_dirs[l];
    a.nb = 3 * a.nd * a.nd;
    a.first_band = p->nbands;
    for (int c = 0; c < 3; c++)
      for (int l2 = 0; l2 < a.nd; l2++)
        for (int l1 = 0; l1 < a.nd; l1++) {
          p->band_level.push_back(l);
          p->band_cone.push_back(c);
          p->band_l2.push_back(l2);
          p->band_l1.push_back(l1);
        }
    p->nbands += a.nb;
    a.spec_off = spec_off;
    spec_off += (size_t)((a.nb + 1) / 2) * a.conv();  // one spectrum F_a + i F_b per band pair
    p->conv_elems = std::max(p->conv_elems, a.conv());
  }
  p->bp_floats = bp_off;
  p->xh_elems = xh_off;
  p->vol_elems = (size_t)p->g[0] * p->g[1] * p->g[2];

  // pyramid windows (PrySDdec_onestep.m:48-82), FP64 -> FP32
  std::vector<float> win_host;
  for (int l = 0; l < p->L; l++) {
    nsst3_plan::Level& a = p->lev[l];
    for (int k = 0; k < 3; k++) {
      std::vector<double> v;
      pyr_window_1d(a.m[k], p->w[l], p->tbw[l], &a.K[k], &v);
      // the window must fit the level's half spectrum and the next level's
      // grid (full axes: both halves; half axis: its non-negative part)
      const int small = p->lev[l + 1].m[k];
      if (a.K[k] >= a.m[k] / 2 + 1 || (k < 2 && a.K[k] >= small) || (k == 2 && a.K[k] >= small / 2 + 1))
        return fail3(NSST_ERR_UNSUPPORTED_SIZE, "pyramid window wider than the level");
      a.win_off[k] = win_off;
      for (double d : v) win_host.push_back((float)d);
      win_off += v.size();
    }
  }
  // twiddle tables of every transform length in use
  std::vector<float2> tw_host;
  auto add_tw = [&](int len) {
    if (p->tw_off.count(len)) return;
    p->tw_off[len] = tw_host.size();
    std::vector<float2> t = twiddle_table(len);
    tw_host.insert(tw_host.end(), t.begin(), t.end());
  };
  for (int l = 0; l <= p->L; l++)
    for (int k = 0; k < 3; k++) {
      add_tw(p->lev[l].m[k]);
      if (l < p->L) add_tw(p->lev[l].lc[k]);
    }
  for (auto& kv : p->tw_off) {
    cudaError_t e = prepare_v3_pass(kv.first);
    if (e != cudaSuccess) return cuda_fail3(e, "prepare_v3_pass");
  }

  // one device arena
  const size_t B = (size_t)batch;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align_up3(off + bytes, 256);
    return o;
  };
  const size_t o_spec = take(spec_off * sizeof(float2));
  const size_t o_win = take(win_host.size() * sizeof(float));
  const size_t o_tw = take(tw_host.size() * sizeof(float2));
  const size_t o_vol = take(B * p->vol_elems * sizeof(float2));
  const size_t o_xh = take(B * p->xh_elems * sizeof(float2));
  const size_t o_y = take(B * p->conv_elems * sizeof(float2));
  const size_t o_w = take(B * p->conv_elems * sizeof(float2));
  const size_t o_bp = take(B * p->bp_floats * sizeof(float));
  const size_t o_rbp = take(B * p->bp_floats * sizeof(float));
  const size_t o_th = take(B * p->nbands * sizeof(float));
  void* arena = nullptr;
  cudaError_t e = dev_alloc(&arena, off);
  if (e != cudaSuccess) return cuda_fail3(e, "plan arena");
  p->arena = (char*)arena;
  p->arena_bytes = off;
  p->spec = (float2*)(p->arena + o_spec);
  p->win = (float*)(p->arena + o_win);
  p->tw = (float2*)(p->arena + o_tw);
  p->vol = (float2*)(p->arena + o_vol);
  p->xh = (float2*)(p->arena + o_xh);
  p->Y = (float2*)(p->arena + o_y);
  p->Wk = (float2*)(p->arena + o_w);
  p->bp = (float*)(p->arena + o_bp);
  p->rbp = (float*)(p->arena + o_rbp);
  p->th = (float*)(p->arena + o_th);
  nsst3_plan* raw = p.get();
  auto cleanup = [&](nsst_status s) {
    cudaFree(raw->arena);
    raw->arena = nullptr;
    return s;
  };
  if ((e = cudaMemcpy(p->win, win_host.data(), win_host.size() * sizeof(float), cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(p->tw, tw_host.data(), tw_host.size() * sizeof(float2), cudaMemcpyHostToDevice)))
    return cleanup(cuda_fail3(e, "plan tables"));

  // Meyer filters (FP64) and the convolution spectra of each band pair,
  // C = F_a + i F_b, FP64 on host worker threads, converted to FP32 and
  // uploaded as each is finished.
  const std::vector<double> filt = meyer_filters_3d(kCube, p->L, cfg->num_dirs);
  const size_t f3 = (size_t)kCube * kCube * kCube;
  std::vector<int> pair_a;  // first band of every pair
  for (int l = 0; l < p->L; l++)
    for (int k = 0; k < p->lev[l].nb; k += 2) pair_a.push_back(p->lev[l].first_band + k);
  const int npairs = (int)pair_a.size();
  const int nthreads = std::min(host_threads3(), npairs);
  std::vector<cudaError_t> terr(nthreads, cudaSuccess);
  std::vector<std::thread> workers;
  for (int t = 0; t < nthreads; t++) {
    workers.emplace_back([&, t]() {
      if (cudaSetDevice(raw->device) != cudaSuccess) {
        terr[t] = cudaErrorInvalidDevice;
        return;
      }
      std::vector<cd> Sa, Sb;
      std::vector<float2> s32;
      for (int q = t; q < npairs; q += nthreads) {
        const int b = pair_a[q];
        const nsst3_plan::Level& a = raw->lev[raw->band_level[b]];
        const bool has_b = b + 1 < a.first_band + a.nb;
        filter_spectrum_3d(filt.data() + (size_t)b * f3, kCube, a.lc[0], a.lc[1], a.lc[2], &Sa);
        if (has_b) filter_spectrum_3d(filt.data() + (size_t)(b + 1) * f3, kCube, a.lc[0], a.lc[1], a.lc[2], &Sb);
        s32.resize(Sa.size());
        for (size_t i = 0; i < Sa.size(); i++) {
          cd c = Sa[i];
          if (has_b) c += cd(0, 1) * Sb[i];
          s32[i] = make_float2((float)c.real(), (float)c.imag());
        }
        const size_t dst = a.spec_off + (size_t)((b - a.first_band) / 2) * a.conv();
        cudaError_t ce = cudaMemcpy(raw->spec + dst, s32.data(), s32.size() * sizeof(float2), cudaMemcpyHostToDevice);
        if (ce != cudaSuccess) {
          terr[t] = ce;
          return;
        }
      }
    });
  }
  for (auto& w : workers) w.join();
  for (cudaError_t te : terr)
    if (te != cudaSuccess) return cleanup(cuda_fail3(te, "filter spectra upload"));
  *out = p.release();
  return NSST_OK;
}

nsst_status nsst3_plan_destroy(nsst3_plan* p) {
  if (!p) return NSST_OK;
  {
    std::lock_guard<std::mutex> lk(p->mu);
    cudaSetDevice(p->device);
    if (p->arena) cudaFree(p->arena);
    if (p->mask) cudaFree(p->mask);
    p->arena = nullptr;
    p->mask = nullptr;
  }
  delete p;
  return NSST_OK;
}

int nsst3_num_bands(const nsst3_plan* p) { return p ? p->nbands : 0; }
size_t nsst3_subband_floats(const nsst3_plan* p) { return p ? p->bp_floats : 0; }
size_t nsst3_plan_device_bytes(const nsst3_plan* p) { return p ? p->arena_bytes : 0; }

nsst_status nsst3_level_dims(const nsst3_plan* p, int level, int* dims, int* conv) {
  if (!p) return fail3(NSST_ERR_INVALID_ARG, "NULL plan");
  if (level < -1 || level > p->L) return fail3(NSST_ERR_INVALID_ARG, "level out of range");
  for (int k = 0; k < 3; k++) {
    if (dims) dims[k] = level < 0 ? p->g[k] : p->lev[level].m[k];
    if (conv) conv[k] = (level < 0 || level == p->L) ? 0 : p->lev[level].lc[k];
  }
  return NSST_OK;
}

nsst_status nsst3_band_info(const nsst3_plan* p, int b, int* info) {
  if (!p || !info) return fail3(NSST_ERR_INVALID_ARG, "NULL argument");
  if (b < 0 || b >= p->nbands) return fail3(NSST_ERR_INVALID_ARG, "band out of range");
  info[0] = p->band_level[b];
  info[1] = p->band_cone[b];
  info[2] = p->band_l2[b];
  info[3] = p->band_l1[b];
  return NSST_OK;
}

nsst_status nsst3_plan_set_scalars(nsst3_plan* p, const double* s) {
  if (!p || !s) return fail3(NSST_ERR_INVALID_ARG, "NULL argument");
  p->scalars.assign(s, s + p->nbands);
  p->has_scalars = true;
  return NSST_OK;
}

}  // extern "C"

extern "C" {

nsst_status nsst3_pyr_dec(nsst3_plan* p, const float* x, float* bp, int n, void* stream) {
  V3_TRY(check_call(p, n, x, bp));
  std::lock_guard<std::mutex> lk(p->mu);
  return run_pyr_dec(p, x, p->n, bp, n, (cudaStream_t)stream);
}

nsst_status nsst3_pyr_rec(nsst3_plan* p, const float* bp, float* x, int n, void* stream) {
  V3_TRY(check_call(p, n, bp, x));
  std::lock_guard<std::mutex> lk(p->mu);
  return run_pyr_rec(p, bp, x, p->n, n, (cudaStream_t)stream);
}

nsst_status nsst3_sh_dec(nsst3_plan* p, const float* bp, int level, float* coeffs, int n, void* stream) {
  V3_TRY(check_call(p, n, bp, coeffs));
  if (level < 0 || level >= p->L) return fail3(NSST_ERR_INVALID_ARG, "level must be a band-pass level");
  std::lock_guard<std::mutex> lk(p->mu);
  return run_sh_level(p, bp, level, nullptr, nullptr, coeffs, n, (cudaStream_t)stream);
}

nsst_status nsst3_sh_dec_thresh_rec(nsst3_plan* p, const float* bp, float* rec_bp, int n, const double* sigma,
                                    const double* T, const double* scalars, void* stream) {
  V3_TRY(check_call(p, n, bp, rec_bp));
  if (bp == rec_bp) return fail3(NSST_ERR_INVALID_ARG, "bp and rec_bp must not alias");
  std::lock_guard<std::mutex> lk(p->mu);
  const cudaStream_t st = (cudaStream_t)stream;
  V3_TRY(upload_th(p, n, sigma, T, scalars, st));
  return run_dec_thresh_rec(p, bp, rec_bp, n, p->th, st);
}

nsst_status nsst3_denoise_batch(nsst3_plan* p, const float* x, float* out, int n, const double* sigma,
                                const double* T, const double* scalars, void* stream) {
  V3_TRY(check_call(p, n, x, out));
  std::lock_guard<std::mutex> lk(p->mu);
  const cudaStream_t st = (cudaStream_t)stream;
  V3_TRY(upload_th(p, n, sigma, T, scalars, st));
  V3_TRY(run_pyr_dec(p, x, p->n, p->bp, n, st));
  p->masks_valid_n = 0;
  V3_TRY(run_dec_thresh_rec(p, p->bp, p->rbp, n, p->th, st, p->mask != nullptr));
  if (p->mask) p->masks_valid_n = n;
  return run_pyr_rec(p, p->rbp, out, p->n, n, st);
}

nsst_status nsst3_compute_scalars(nsst3_plan* p, uint64_t seed, double* out) {
  if (!p) return fail3(NSST_ERR_INVALID_ARG, "NULL plan");
  if (cudaSetDevice(p->device) != cudaSuccess) return fail3(NSST_ERR_CUDA, "cudaSetDevice failed");
  std::lock_guard<std::mutex> lk(p->mu);
  const size_t G = p->vol_elems;
  // seeded N(0,1) grid volume in FP64 (Box-Muller over a 64-bit Mersenne twister)
  std::mt19937_64 gen(seed);
  std::vector<float> noise(G);
  for (size_t i = 0; i < G; i += 2) {
    double u1 = ((gen() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    double u2 = ((gen() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    double r = std::sqrt(-2.0 * std::log(u1));
    noise[i] = (float)(r * std::cos(2 * M_PI * u2));
    if (i + 1 < G) noise[i + 1] = (float)(r * std::sin(2 * M_PI * u2));
  }
  size_t maxc = 0;
  for (int l = 0; l < p->L; l++) maxc = std::max(maxc, (size_t)p->lev[l].nb * p->lev[l].vol());
  float *dx = nullptr, *dc = nullptr;
  cudaError_t e = dev_alloc((void**)&dx, G * sizeof(float));
  if (e != cudaSuccess) return cuda_fail3(e, "scalar scratch");
  e = dev_alloc((void**)&dc, maxc * sizeof(float));
  if (e != cudaSuccess) {
    cudaFree(dx);
    return cuda_fail3(e, "scalar scratch");
  }
  std::vector<double> sc(p->nbands);
  nsst_status s = NSST_OK;
  std::vector<float> coeffs(maxc);
  e = cudaMemcpy(dx, noise.data(), G * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) s = run_pyr_dec(p, dx, p->g, p->bp, 1, nullptr);
  for (int l = 0; l < p->L && e == cudaSuccess && s == NSST_OK; l++) {
    const nsst3_plan::Level& a = p->lev[l];
    s = run_sh_level(p, p->bp, l, nullptr, nullptr, dc, 1, nullptr);
    if (s != NSST_OK) break;
    e = cudaMemcpy(coeffs.data(), dc, (size_t)a.nb * a.vol() * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) break;
    // MAD / 0.6745 per band (NsstScalars.m:11-15), FP64, bands in parallel
    const int nt = std::min(host_threads3(), a.nb);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++)
      th.emplace_back([&, t]() {
        std::vector<double> v(a.vol());
        auto median = [](std::vector<double>& x) {
          size_t m = x.size(), h = m / 2;
          std::nth_element(x.begin(), x.begin() + h, x.end());
          double hi = x[h];
          if (m % 2) return hi;
          double lo = *std::max_element(x.begin(), x.begin() + h);
          return 0.5 * (lo + hi);
        };
        for (int k = t; k < a.nb; k += nt) {
          const float* c = coeffs.data() + (size_t)k * a.vol();
          for (size_t i = 0; i < v.size(); i++) v[i] = c[i];
          const double med = median(v);
          for (size_t i = 0; i < v.size(); i++) v[i] = std::fabs((double)c[i] - med);
          sc[a.first_band + k] = median(v) / 0.6745;
        }
      });
    for (auto& t : th) t.join();
  }
  cudaFree(dx);
  cudaFree(dc);
  if (e != cudaSuccess) return cuda_fail3(e, "compute scalars");
  if (s != NSST_OK) return s;
  p->scalars = sc;
  p->has_scalars = true;
  if (out) std::copy(sc.begin(), sc.end(), out);
  return NSST_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Differentiation of the 3-D denoise.  The hard threshold's subgradient keeps
// the forward pass's masks; the band-pass pyramid is a Parseval frame, so the
// adjoint of the decomposition is the reconstruction and vice versa; the
// adjoint of each 'same' convolution is a correlation (the conjugate filter
// spectrum) of the masked gradient placed back at offset 12.
// ---------------------------------------------------------------------------
extern "C" {

nsst_status nsst3_plan_enable_grad(nsst3_plan* p) {
  if (!p) return fail3(NSST_ERR_INVALID_ARG, "NULL plan");
  if (p->mask) return NSST_OK;
  if (cudaSetDevice(p->device) != cudaSuccess) return fail3(NSST_ERR_CUDA, "cudaSetDevice failed");
  std::lock_guard<std::mutex> lk(p->mu);
  p->mask_off.assign(p->nbands, 0);
  size_t bytes = 0;
  for (int b = 0; b < p->nbands; b++) {
    p->mask_off[b] = bytes;
    const nsst3_plan::Level& lv = p->lev[p->band_level[b]];
    bytes += align_up3((size_t)lv.m[0] * lv.m[1] * mask_pitch(lv.m[2]) / 8, 256);
  }
  p->mask_bytes = bytes;
  void* m = nullptr;
  cudaError_t e = dev_alloc(&m, (size_t)p->B * bytes);
  if (e != cudaSuccess) return cuda_fail3(e, "mask buffer");
  p->mask = (uint8_t*)m;
  p->masks_valid_n = 0;
  return NSST_OK;
}

nsst_status nsst3_denoise_backward(nsst3_plan* p, const float* gy, float* gx, int n, void* stream) {
  V3_TRY(check_call(p, n, gy, gx));
  std::lock_guard<std::mutex> lk(p->mu);
  if (!p->mask) return fail3(NSST_ERR_INVALID_ARG, "gradients are not enabled on this plan");
  if (p->masks_valid_n != n)
    return fail3(NSST_ERR_INVALID_ARG, "no forward nsst3_denoise_batch of these n volumes since grad was enabled");
  const cudaStream_t st = (cudaStream_t)stream;
  // u = pyr_dec(zero-pad(gy)): the adjoint of crop + pyr_rec
  V3_TRY(run_pyr_dec(p, gy, p->n, p->rbp, n, st, true));
  // per level: bp_bar_l = sum_b corr(mask_b * u_l, f_b).  Per band pair,
  // Z = FFT3(place(mask_a u + i mask_b u)) from the box outwards (the zero
  // outside the box is never read), then S (+)= conj(C) .* Z in the last
  // pass; one inverse transform of S per level, cut to the box at 0.
  for (int l = 0; l < p->L; l++) {
    const nsst3_plan::Level& a = p->lev[l];
    const int* N = a.lc;
    const int* m = a.m;
    const int o = kSameOff;
    const size_t cs = p->conv_elems;
    for (int k = 0; k < a.nb; k += 2) {
      const int ba = a.first_band + k;
      const int bb = k + 1 < a.nb ? ba + 1 : -1;
      V3Pass P1 = make_pass(0, N, cs, {o, m[1]}, {o, m[2]}, {o, m[0]}, {0, N[0]});
      set_box(P1, m, o);
      P1.rsrc = p->rbp + a.bp_off;
      P1.r_stride = p->bp_floats;
      P1.m_r2 = mask_pitch(m[2]);
      P1.mka = p->mask + p->mask_off[ba];
      P1.mkb = bb >= 0 ? p->mask + p->mask_off[bb] : nullptr;
      P1.m_stride = p->mask_bytes;
      V3_TRY(run_pass(p, P1, -1, V3_LD_MASKED, V3_ST_CPLX, p->Wk, p->Wk, N[0], n, st));
      V3_TRY(run_pass(p, make_pass(1, N, cs, {0, N[0]}, {o, m[2]}, {o, m[1]}, {0, N[1]}), -1, V3_LD_CPLX, V3_ST_CPLX,
                      p->Wk, p->Wk, N[1], n, st));
      V3Pass P3 = make_pass(2, N, cs, {0, N[0]}, {0, N[1]}, {o, m[2]}, {0, N[2]});
      P3.spec = p->spec + a.spec_off + (size_t)(k / 2) * a.conv();
      P3.first = k == 0;
      V3_TRY(run_pass(p, P3, -1, V3_LD_CPLX, V3_ST_SPEC, p->Y, p->Wk, N[2], n, st));
    }
    V3_TRY(ifft3_real_box(p, p->Y, cs, N, m, 0, p->bp + a.bp_off, p->bp_floats, (float)(1.0 / (double)a.conv()), n,
                          st));
  }
  // the lowpass passes through unchanged
  const nsst3_plan::Level& lp = p->lev[p->L];
  V3_CUDA(cudaMemcpy2DAsync(p->bp + lp.bp_off, p->bp_floats * sizeof(float), p->rbp + lp.bp_off,
                            p->bp_floats * sizeof(float), lp.vol() * sizeof(float), n, cudaMemcpyDeviceToDevice, st));
  // pyr_rec (the adjoint of pyr_dec) to the full grid, then fold the edge padding
  V3_TRY(run_pyr_rec(p, p->bp, p->rbp, p->g, n, st));
  V3_CUDA(launch_fold_edge(p->rbp, p->vol_elems, gx, p->in_elems, (float*)p->vol, 2 * p->vol_elems, n, p->n[0],
                           p->n[1], p->n[2], p->g[0], p->g[1], p->g[2], st));
  return NSST_OK;
}

}  // extern "C"
