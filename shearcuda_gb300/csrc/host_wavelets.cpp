// Host side of the undecimated wavelets: the orthonormal QMF families of
// MakeONFilter.m and the analysis / synthesis tap sets that the redundant DWT
// kernels use (mrdwt_r.h, mirdwt_r.h, mdwt_r.h of the Rice Wavelet Toolbox as
// the reference ships it in shearcuda/src).
#include <cmath>

#include "internal.h"
#include "wavelet_tables.h"

namespace nsst {

bool on_filter(const std::string& type, int par, std::vector<double>* f) {
  const bool has_par = type == "Coiflet" || type == "Daubechies" || type == "Symmlet" || type == "Battle";
  for (int k = 0; k < kNumOnFilters; k++) {
    const OnFilterTable& t = kOnFilters[k];
    if (type != t.type || (has_par && par != t.par)) continue;
    if (t.half) {
      // MakeONFilter.m:283-286: f(l:2l-1) = g, f(1:l-1) = reverse(g(2:l))
      const int l = t.n;
      f->assign((size_t)(2 * l - 1), 0.0);
      for (int i = 0; i < l; i++) (*f)[(size_t)(l - 1 + i)] = t.v[i];
      for (int i = 1; i < l; i++) (*f)[(size_t)(l - 1 - i)] = t.v[i];
    } else {
      f->assign(t.v, t.v + t.n);
    }
    // MakeONFilter.m:289: f = f ./ norm(f)
    double s = 0.0;
    for (double v : *f) s += v * v;
    const double nrm = std::sqrt(s);
    for (double& v : *f) v /= nrm;
    return true;
  }
  return false;
}

// mrdwt_r.h:118-125: h0[i] = h[lh-1-i]; h1[i] = h[i] with the even entries
// negated; fpconv (:84-101) forms lo[c] = sum_j x[c + j sf] h0[lh-1-j].
WvTaps analysis_taps(const std::vector<double>& h) {
  WvTaps t{};
  const int lh = (int)h.size();
  t.lh = lh;
  for (int j = 0; j < lh; j++) {
    const int i = lh - 1 - j;          // index into h0 / h1
    t.a[j] = (float)h[(size_t)(lh - 1 - i)];
    t.b[j] = (float)((i % 2 == 0) ? -h[(size_t)i] : h[(size_t)i]);
  }
  return t;
}

// mirdwt_r.h:125-130: g0[i] = h[i] / 2; g1[i] = h[lh-1-i] / 2 with the odd
// entries negated; bpconv (:95-112) forms x[c] = sum_t lo[c - t sf] g0[t] +
// hi[c - t sf] g1[t].
WvTaps synthesis_taps(const std::vector<double>& h) {
  WvTaps t{};
  const int lh = (int)h.size();
  t.lh = lh;
  for (int i = 0; i < lh; i++) {
    t.a[i] = (float)(h[(size_t)i] / 2);
    const double g1 = h[(size_t)(lh - 1 - i)] / 2;
    t.b[i] = (float)((i % 2 == 1) ? -g1 : g1);
  }
  return t;
}

}  // namespace nsst
