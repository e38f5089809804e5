// FP64 host-side construction of the NSST filter bank.
//
// The pyramid filters, the Meyer shearing filters and their normalised
// spectra are built here in double precision once per plan and uploaded as
// FP32 (the device never evaluates trigonometry for them).
#include <cmath>
#include <cstring>
#include <thread>

#include "internal.h"
#include "pyramid_tables.h"

namespace nsst {

// --------------------------------------------------------------- pyramid
// atrousfilters.m: for 'maxflat', 'pyr' and 'pyrexc' the table holds one
// quadrant that is mirrored to the full odd-sized filter (:167-175,
// :198-206, :228-236); '9-7' tables are full filters, with h1 and g0 halved
// (:100-104).
static std::vector<double> mirror_quadrant(const double* q, int r, int c, int* F) {
  int R = 2 * r - 1, C = 2 * c - 1;
  std::vector<double> out((size_t)R * C);
  for (int i = 0; i < R; i++) {
    int si = i < r ? i : 2 * r - 2 - i;
    for (int j = 0; j < C; j++) {
      int sj = j < c ? j : 2 * c - 2 - j;
      out[(size_t)i * C + j] = q[(size_t)si * c + sj];
    }
  }
  *F = R;
  return out;
}

bool pyramid_filters(const std::string& name, PyramidFilters* out) {
  for (const PyrTable& t : k_pyr_tables) {
    if (name != t.name) continue;
    out->name = name;
    for (int k = 0; k < 4; k++) {
      if (name == "9-7") {
        out->F[k] = t.rows[k];
        double scale = (k == 1 || k == 2) ? 0.5 : 1.0;
        out->h[k].assign(t.m[k], t.m[k] + (size_t)t.rows[k] * t.cols[k]);
        for (double& v : out->h[k]) v *= scale;
      } else {
        out->h[k] = mirror_quadrant(t.m[k], t.rows[k], t.cols[k], &out->F[k]);
      }
    }
    return true;
  }
  return false;
}

// ------------------------------------------------------ Meyer shearing filters
namespace {

// MATLAB round: half away from zero.
inline double mround(double v) { return v >= 0 ? std::floor(v + 0.5) : -std::floor(-v + 0.5); }

// gen_x_y_cordinates.m:22-80 (1-based index matrices) + avg_pol (:85-110).
struct PolarGrid {
  int n;
  std::vector<int> x1, y1, x2, y2;  // n x n, row-major
  std::vector<double> D;
};

PolarGrid gen_x_y_cordinates(int n0) {
  const int n = n0 + 1;
  std::vector<double> x1((size_t)n * n), y1((size_t)n * n), x2((size_t)n * n), y2((size_t)n * n);
  for (int i = 1; i <= n; i++) {
    const double y0 = 1, x0 = i, x_n = n - i + 1, y_n = n;
    const bool flag = (x_n == x0);
    const double m1 = flag ? 0.0 : (y_n - y0) / (x_n - x0);
    for (int j = 1; j <= n; j++) {
      // linspace(x0, x_n, n)
      double xt = (j == n) ? x_n : x0 + (j - 1) * ((x_n - x0) / (n - 1));
      size_t at = (size_t)(i - 1) * n + (j - 1);
      if (!flag) {
        double yv = mround(m1 * (xt - x0) + y0);
        double xv = mround(xt);
        y1[at] = yv;
        x1[at] = xv;
        x2[at] = yv;
        y2[at] = xv;
      } else {
        x1[at] = (n - 1) / 2.0 + 1;
        y1[at] = j;
        x2[at] = j;
        y2[at] = (n - 1) / 2.0 + 1;
      }
    }
  }
  PolarGrid g;
  g.n = n0;
  const int m = n0;
  g.x1.resize((size_t)m * m);
  g.y1.resize((size_t)m * m);
  g.x2.resize((size_t)m * m);
  g.y2.resize((size_t)m * m);
  for (int i = 0; i < m; i++) {
    for (int j = 0; j < m; j++) {
      // x1n = flipud(x1(1:n,1:n)); y1n = y1(1:n,1:n); x2n/y2n = rows 2..n+1
      g.x1[(size_t)i * m + j] = (int)x1[(size_t)(m - 1 - i) * n + j];
      g.y1[(size_t)i * m + j] = (int)y1[(size_t)i * n + j];
      g.x2[(size_t)i * m + j] = (int)x2[(size_t)(i + 1) * n + j];
      g.y2[(size_t)i * m + j] = (int)y2[(size_t)(i + 1) * n + j];
    }
  }
  g.y2[(size_t)(m - 1) * m + 0] = m;  // y2n(n,1) = n
  g.D.assign((size_t)m * m, 0.0);
  for (int i = 0; i < m; i++)
    for (int j = 0; j < m; j++) g.D[(size_t)(g.y1[i * m + j] - 1) * m + (g.x1[i * m + j] - 1)] += 1;
  for (int i = 0; i < m; i++)
    for (int j = 0; j < m; j++) g.D[(size_t)(g.y2[i * m + j] - 1) * m + (g.x2[i * m + j] - 1)] += 1;
  return g;
}

// meyer_wind.m:11-19
double meyer_wind(double x) {
  if (-1.0 / 3 + 1.0 / 2 < x && x < 1.0 / 3 + 1.0 / 2) return 1.0;
  if ((1.0 / 3 + 1.0 / 2 <= x && x <= 2.0 / 3 + 1.0 / 2) || (-2.0 / 3 + 1.0 / 2 <= x && x <= 1.0 / 3 + 1.0 / 2)) {
    double w = 3 * std::fabs(x - 1.0 / 2) - 1;
    double z = std::pow(w, 4) * (35 - 84 * w + 70 * w * w - 20 * w * w * w);
    double c = std::cos(M_PI / 2 * z);
    return c * c;
  }
  return 0.0;
}

// windowing.m:11-27 applied to ones(N,1): returns N x L (row-major).
std::vector<double> windowing_ones(int N, int L) {
  std::vector<double> y((size_t)N * L, 0.0);
  const double T = (double)N / L;
  const int ng = (int)(2 * T);
  std::vector<double> g(ng);
  for (int j = 1; j <= ng; j++) g[j - 1] = meyer_wind((-1 * T / 2 + j - 1) / T);
  for (int j = 1; j <= L; j++) {
    int index = 0;
    for (double k = -1 * T / 2; k <= 1.5 * T - 1; k += 1) {
      double v = k + (j - 1) * T;
      double md = v - std::floor(v / N) * N;  // MATLAB mod (floor-mod)
      int in_sig = (int)std::floor(md);
      y[(size_t)in_sig * L + (j - 1)] = g[index];
      index++;
    }
  }
  return y;
}

void fftshift2(std::vector<cd>& a, int n) {
  std::vector<cd> b(a.size());
  int h = n / 2;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) b[(size_t)((i + h) % n) * n + (j + h) % n] = a[(size_t)i * n + j];
  a.swap(b);
}

}  // namespace

std::vector<double> shearing_filters_myer(int n1, int level) {
  PolarGrid g = gen_x_y_cordinates(n1);
  const int L = 1 << level;
  std::vector<double> wf = windowing_ones(2 * n1, L);
  std::vector<double> out((size_t)L * n1 * n1);
  std::vector<cd> C((size_t)n1 * n1), row(n1);
  for (int k = 0; k < L; k++) {
    // rec_from_pol.m:16-35 (option 0) with l = wf(:,k) * ones(n1,1)'
    std::vector<double> acc((size_t)n1 * n1, 0.0);
    for (int i = 0; i < n1; i++) {
      for (int j = 0; j < n1; j++) {
        acc[(size_t)(g.y1[i * n1 + j] - 1) * n1 + (g.x1[i * n1 + j] - 1)] += wf[(size_t)i * L + k];
        acc[(size_t)(g.y2[i * n1 + j] - 1) * n1 + (g.x2[i * n1 + j] - 1)] += wf[(size_t)(i + n1) * L + k];
      }
    }
    for (size_t t = 0; t < acc.size(); t++) C[t] = cd(acc[t] / g.D[t], 0.0);
    // real(fftshift(ifft2(fftshift(C)))) / sqrt(n1)   (shearing_filters_Myer.m:26)
    fftshift2(C, n1);
    for (int i = 0; i < n1; i++) fft_inplace(&C[(size_t)i * n1], n1, +1);
    for (int j = 0; j < n1; j++) {
      for (int i = 0; i < n1; i++) row[i] = C[(size_t)i * n1 + j];
      fft_inplace(row.data(), n1, +1);
      for (int i = 0; i < n1; i++) C[(size_t)i * n1 + j] = row[i];
    }
    fftshift2(C, n1);
    const double s = 1.0 / ((double)n1 * n1) / std::sqrt((double)n1);
    for (size_t t = 0; t < C.size(); t++) out[(size_t)k * n1 * n1 + t] = C[t].real() * s;
  }
  return out;
}

// ------------------------------------------------------------ host FFT (FP64)
namespace {
void dit(cd* x, int n, int stride, const cd* w, int N, int wstride, cd* tmp) {
  // in-place decimation-in-time on x[0], x[stride], ... (n points)
  if (n == 1) return;
  int r = n % 4 == 0 ? 4 : (n % 2 == 0 ? 2 : (n % 3 == 0 ? 3 : n));
  int m = n / r;
  // gather the r decimated subsequences contiguously
  for (int q = 0; q < r; q++)
    for (int k = 0; k < m; k++) tmp[q * m + k] = x[(size_t)(k * r + q) * stride];
  for (int q = 0; q < r; q++)
    for (int k = 0; k < m; k++) x[(size_t)(q * m + k) * stride] = tmp[q * m + k];
  for (int q = 0; q < r; q++) dit(x + (size_t)q * m * stride, m, stride, w, N, wstride * r, tmp);
  cd t[64], y[64];
  for (int k = 0; k < m; k++) {
    for (int q = 0; q < r; q++) {
      long idx = ((long)q * k * wstride) % N;
      t[q] = x[(size_t)(q * m + k) * stride] * w[idx];
    }
    for (int p = 0; p < r; p++) {
      cd s = 0;
      for (int q = 0; q < r; q++) s += t[q] * w[((long)q * p * m * wstride) % N];
      y[p] = s;
    }
    for (int p = 0; p < r; p++) x[(size_t)(k + p * m) * stride] = y[p];
  }
}
}  // namespace

void fft_inplace(cd* data, int n, int sign) {
  if (n <= 1) return;
  // per-thread cache of the twiddle table for the last few lengths
  struct Entry {
    int n = 0, sign = 0;
    std::vector<cd> w;
  };
  thread_local Entry cache[4];
  thread_local int next = 0;
  thread_local std::vector<cd> tmp;
  Entry* e = nullptr;
  for (Entry& c : cache)
    if (c.n == n && c.sign == sign) e = &c;
  if (!e) {
    e = &cache[next];
    next = (next + 1) % 4;
    e->n = n;
    e->sign = sign;
    e->w.resize(n);
    for (int t = 0; t < n; t++) {
      double a = 2.0 * M_PI * (double)t / n;
      e->w[t] = cd(std::cos(a), sign * std::sin(a));
    }
  }
  if ((int)tmp.size() < n) tmp.resize(n);
  dit(data, n, 1, e->w.data(), n, 1, tmp.data());
}

bool level_spectra(const std::vector<double>& filters, int ndir, int n1, int H, int W, std::vector<cd>* out,
                   int nthreads) {
  const int WC = W / 2 + 1;
  out->assign((size_t)ndir * H * WC, cd(0, 0));
  auto work = [&](int k) {
    std::vector<cd> row(W), col(H);
    cd* spec = out->data() + (size_t)k * H * WC;
    const double* f = filters.data() + (size_t)k * n1 * n1;
    // rows of the top-left padded filter (rows >= n1 are zero)
    for (int i = 0; i < n1 && i < H; i++) {
      std::fill(row.begin(), row.end(), cd(0, 0));
      for (int j = 0; j < n1 && j < W; j++) row[j] = cd(f[(size_t)i * n1 + j], 0);
      fft_inplace(row.data(), W, -1);
      for (int v = 0; v < WC; v++) spec[(size_t)i * WC + v] = row[v];
    }
    for (int v = 0; v < WC; v++) {
      for (int i = 0; i < H; i++) col[i] = spec[(size_t)i * WC + v];
      fft_inplace(col.data(), H, -1);
      for (int i = 0; i < H; i++) spec[(size_t)i * WC + v] = col[i];
    }
  };
  if (nthreads < 1) nthreads = 1;
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; t++) {
    th.emplace_back([&, t]() {
      for (int k = t; k < ndir; k += nthreads) work(k);
    });
  }
  for (auto& t : th) t.join();
  // d = sqrt(sum_k |W_k|^2); W_k /= d   (nsst_dec2.m:55-57)
  bool ok = true;
  for (size_t p = 0; p < (size_t)H * WC; p++) {
    double s = 0;
    for (int k = 0; k < ndir; k++) s += std::norm((*out)[(size_t)k * H * WC + p]);
    double d = std::sqrt(s);
    if (!(d > 0.0) || !std::isfinite(d)) {
      ok = false;
      d = 1.0;
    }
    for (int k = 0; k < ndir; k++) (*out)[(size_t)k * H * WC + p] /= d;
  }
  return ok;
}

std::vector<float2> twiddle_table(int n) {
  std::vector<float2> t(n);
  for (int i = 0; i < n; i++) {
    double a = -2.0 * M_PI * (double)i / n;
    t[i] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  return t;
}

std::vector<float4> broadcast_table(const std::vector<float2>& tab) {
  std::vector<float4> t(tab.size());
  for (size_t i = 0; i < tab.size(); i++) t[i] = make_float4(tab[i].x, tab[i].x, tab[i].y, tab[i].y);
  return t;
}

std::vector<float2> half_twiddle_table(int n) {
  std::vector<float2> t(n / 2);
  for (int i = 0; i < n / 2; i++) {
    double a = -2.0 * M_PI * (double)i / n;
    t[i] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  return t;
}

}  // namespace nsst
