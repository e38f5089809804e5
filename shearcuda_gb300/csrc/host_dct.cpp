// Host (FP64) tables of the DCT-domain pyramid (k_dct.cu).
//
// A pyramid step filters with h (F x F, symmetric in both axes, centre
// c0 = (F-1)/2) dilated by M on the half-sample symmetric extension of its
// input (atrousc.cpp:43-73 on symext.m's extension); in the 2-D DCT-II domain
// of an H x W image that is the pointwise product with
//     G_h,M[k1][k2] = sum_{a,b} h[a][b] cos(pi k1 M (a - c0) / H) cos(pi k2 M (b - c0) / W).
// The tables chain those products the way atrousdec.m:33-48 and
// atrousrec.m:27-40 chain the steps.
#include <cmath>
#include <thread>

#include "internal.h"

namespace nsst {

bool filters_symmetric(const PyramidFilters& pf) {
  for (int f = 0; f < 4; f++) {
    const int F = pf.F[f];
    if (F < 1 || F % 2 == 0 || (int)pf.h[f].size() != F * F) return false;
    const std::vector<double>& h = pf.h[f];
    for (int a = 0; a < F; a++)
      for (int b = 0; b < F; b++)
        if (h[a * F + b] != h[(F - 1 - a) * F + b] || h[a * F + b] != h[a * F + (F - 1 - b)]) return false;
  }
  return true;
}

namespace {

// cos(pi t / n) for an integer t, reduced exactly modulo 2n first
double cos_pi_frac(long long t, int n) {
  long long r = t % (2LL * n);
  if (r < 0) r += 2LL * n;
  return std::cos(M_PI * (double)r / (double)n);
}

// G_h,M as an H x W row-major array: T[a][k2] = sum_b h[a][b] cw[k2][b], then
// G[k1][k2] = sum_a ch[k1][a] T[a][k2]
void level_response(const std::vector<double>& h, int F, int M, int H, int W, std::vector<double>& G) {
  const int c0 = (F - 1) / 2;
  std::vector<double> ch((size_t)H * F), T((size_t)F * W);
  for (int k = 0; k < H; k++)
    for (int a = 0; a < F; a++) ch[(size_t)k * F + a] = cos_pi_frac((long long)k * M * (a - c0), H);
  std::vector<double> cw((size_t)W * F);
  for (int k = 0; k < W; k++)
    for (int b = 0; b < F; b++) cw[(size_t)k * F + b] = cos_pi_frac((long long)k * M * (b - c0), W);
  for (int a = 0; a < F; a++)
    for (int k = 0; k < W; k++) {
      double s = 0;
      for (int b = 0; b < F; b++) s += h[(size_t)a * F + b] * cw[(size_t)k * F + b];
      T[(size_t)a * W + k] = s;
    }
  G.assign((size_t)H * W, 0.0);
  for (int k1 = 0; k1 < H; k1++) {
    double* g = G.data() + (size_t)k1 * W;
    for (int a = 0; a < F; a++) {
      const double c = ch[(size_t)k1 * F + a];
      const double* t = T.data() + (size_t)a * W;
      for (int k2 = 0; k2 < W; k2++) g[k2] += c * t[k2];
    }
  }
}

}  // namespace

void dct_pyramid_tables(const PyramidFilters& pf, int L, int H, int W, std::vector<float>* out) {
  const size_t HW = (size_t)H * W;
  out->assign((size_t)(2 * L + 3) * HW, 0.0f);
  const double s = 1.0 / ((double)H * W);
  std::vector<double> ch(HW, 1.0), cg(HW, 1.0);  // running products of the h0 / g0 responses
  std::vector<double> G[4];
  for (int i = 0; i < L; i++) {  // dilation 2^i: directional level L-1-i
    std::vector<std::thread> th;
    for (int f = 0; f < 4; f++) th.emplace_back([&, f] { level_response(pf.h[f], pf.F[f], 1 << i, H, W, G[f]); });
    for (auto& t : th) t.join();
    const int l = L - 1 - i;
    float* ra = out->data() + (size_t)l * HW;
    float* rs = out->data() + (size_t)(L + l) * HW;
    for (size_t e = 0; e < HW; e++) {
      ra[e] = (float)(s * ch[e] * G[1][e]);  // atrousdec.m: highpass after i lowpass steps
      rs[e] = (float)(s * G[3][e] * cg[e]);  // atrousrec.m: g1 step, then i g0 steps
      ch[e] *= G[0][e];
      cg[e] *= G[2][e];
    }
  }
  float* tl = out->data() + (size_t)2 * L * HW;
  float* rl = tl + HW;
  float* gl = rl + HW;
  for (size_t e = 0; e < HW; e++) {
    tl[e] = (float)(s * ch[e] * cg[e]);  // lowpass round trip: L h0 steps, L g0 steps
    rl[e] = (float)(s * ch[e]);          // lowpass band (atrousdec.m's y{1})
    gl[e] = (float)(s * cg[e]);          // lowpass synthesis (atrousrec.m's L g0 steps)
  }
}

std::vector<float4> dct_row_twiddles(int W) {
  const int WH = W / 2;
  std::vector<float4> t(WH + 1);
  for (int k = 0; k <= WH; k++) {
    const double a = -M_PI * (double)k / (2.0 * W), b = -2.0 * M_PI * (double)k / W;
    t[k] = make_float4((float)std::cos(a), (float)std::sin(a), k < WH ? (float)std::cos(b) : 0.0f,
                       k < WH ? (float)std::sin(b) : 0.0f);
  }
  return t;
}

std::vector<float2> dct_col_twiddles(int H) {
  std::vector<float2> t(H);
  for (int k = 0; k < H; k++) {
    const double a = -M_PI * (double)k / (2.0 * H);
    t[k] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  return t;
}

}  // namespace nsst
