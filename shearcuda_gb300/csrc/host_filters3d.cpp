// FP64 host-side construction for the 3-D path: the pseudo-polar Meyer
// filters of GetMeyerBasedFilter.m and the separable windows of the
// Fourier-domain band-pass pyramid (PrySDdec_onestep.m / PrySDrec_onestep.m).
#include <cmath>
#include <cstring>
#include <thread>

#include "internal.h"

namespace nsst {

namespace {

inline int u16round(double v) {  // MATLAB double -> uint16 (round half away, saturate)
  double r = std::floor(v + 0.5);
  if (r < 0) r = 0;
  if (r > 65535) r = 65535;
  return (int)r;
}

struct Xyz {
  int n;
  std::vector<int> X, Y, Z;  // n^3, index (i,k,j) -> (i*n + k)*n + j, 1-based values
  int at(int i, int k, int j) const { return (i * n + k) * n + j; }
};

// GenerateXYZ.m:12-54
Xyz generate_xyz(int n) {
  Xyz g;
  g.n = n;
  g.X.assign((size_t)n * n * n, 0);
  g.Y.assign((size_t)n * n * n, 0);
  g.Z.assign((size_t)n * n * n, 0);
  const int mid = (n + 1) / 2;
  for (int j = 1; j <= mid; j++) {
    for (int i = 1; i <= mid; i++) {
      double dL2 = (double)(n - 1) * (n - 1) + (double)(n - i + 1 - i) * (n - i + 1 - i);
      double dL3 = std::sqrt(dL2 + (double)(n - j + 1 - j) * (n - j + 1 - j));
      dL2 = std::sqrt(dL2);
      const double sinA = (n - j + 1 - j) / dL3, cosA = dL2 / dL3;
      const double sinB = (n - i + 1 - i) / dL2, cosB = (n - 1) / dL2;
      const double dl3 = dL3 / (n - 1);
      for (int k = 1; k <= n; k++) {
        const double l = dl3 * (k - 1);
        double temp = l * sinA;
        const int I = i - 1, K = k - 1, J = j - 1, Ii = n - i, Jj = n - j;
        g.Z[g.at(I, K, J)] = u16round(j + temp);
        g.Z[g.at(Ii, K, J)] = g.Z[g.at(I, K, J)];
        g.Z[g.at(I, K, Jj)] = u16round(n - j + 1 - temp);
        g.Z[g.at(Ii, K, Jj)] = u16round(n - j + 1 - temp);
        temp = l * cosA;
        const double t1 = temp * sinB;
        g.Y[g.at(I, K, J)] = u16round(i + t1);
        g.Y[g.at(Ii, K, J)] = u16round(n - i + 1 - t1);
        g.X[g.at(I, K, J)] = u16round(1 + temp * cosB);
        g.X[g.at(Ii, K, J)] = g.X[g.at(I, K, J)];
        g.X[g.at(I, K, Jj)] = g.X[g.at(I, K, J)];
        g.X[g.at(Ii, K, Jj)] = g.X[g.at(I, K, J)];
        g.Y[g.at(I, K, Jj)] = g.Y[g.at(I, K, J)];
        g.Y[g.at(Ii, K, Jj)] = g.Y[g.at(Ii, K, J)];
      }
    }
  }
  return g;
}

struct Cone {
  const std::vector<int>* X;
  const std::vector<int>* Y;
  const std::vector<int>* Z;
};

// PolarToRec.m:10-19 into `out` (n^3, zero-initialised by the caller);
// mRadial is a (a x n x b) block with the given 0-based 1/3 corner (or -1).
void polar_to_rec(const Xyz& g, const Cone& c, int i0, int i1, int j0, int j1, int a, int b, int ca, int cb,
                  std::vector<double>* out) {
  const int n = g.n;
  for (int j = j0; j <= j1; j++)
    for (int i = i0; i <= i1; i++)
      for (int k = 1; k <= n; k++) {
        const int ri = i - i0, rj = j - j0;
        double v = 1.0;
        if (ri == 0 || ri == a - 1 || rj == 0 || rj == b - 1) v = 0.5;
        if (ca >= 0 && ri == ca && rj == cb) v = 1.0 / 3.0;
        const size_t src = (size_t)g.at(i - 1, k - 1, j - 1);
        const int x = (*c.X)[src] - 1, y = (*c.Y)[src] - 1, z = (*c.Z)[src] - 1;
        (*out)[((size_t)x * n + y) * n + z] = v;
      }
}

void fftshift3(std::vector<cd>& a, int n) {
  std::vector<cd> b(a.size());
  const int h = n / 2;
  for (int x = 0; x < n; x++)
    for (int y = 0; y < n; y++)
      for (int z = 0; z < n; z++)
        b[(((size_t)(x + h) % n) * n + (y + h) % n) * n + (z + h) % n] = a[((size_t)x * n + y) * n + z];
  a.swap(b);
}

void fft3_inplace(std::vector<cd>& a, int n, int sign) {
  std::vector<cd> line(n);
  for (int axis = 0; axis < 3; axis++) {
    for (int u = 0; u < n; u++)
      for (int v = 0; v < n; v++) {
        for (int t = 0; t < n; t++) {
          size_t idx = axis == 0 ? (((size_t)t * n + u) * n + v)
                                 : (axis == 1 ? (((size_t)u * n + t) * n + v) : (((size_t)u * n + v) * n + t));
          line[t] = a[idx];
        }
        fft_inplace(line.data(), n, sign);
        for (int t = 0; t < n; t++) {
          size_t idx = axis == 0 ? (((size_t)t * n + u) * n + v)
                                 : (axis == 1 ? (((size_t)u * n + t) * n + v) : (((size_t)u * n + v) * n + t));
          a[idx] = line[t];
        }
      }
  }
}

}  // namespace

// GetMeyerBasedFilter.m:12-150.  Output order: level-major, then cone (after the
// swap of cones 1 and 2 at :148-150), then l2, then l1; each filter cube^3,
// index (x, y, z) -> (x*cube + y)*cube + z.
std::vector<double> meyer_filters_3d(int cube, int nlevels, const int* num_dirs) {
  Xyz g = generate_xyz(cube);
  // GeneratePyramidSection.m:1-14: cone coordinate maps
  Cone cones[3] = {{&g.X, &g.Y, &g.Z}, {&g.Y, &g.X, &g.Z}, {&g.Z, &g.Y, &g.X}};
  const size_t n3 = (size_t)cube * cube * cube;
  std::vector<double> out;
  for (int l = 0; l < nlevels; l++) {
    const int nd = num_dirs[l], s = cube / nd, s1 = s + 1;
    std::vector<std::vector<double>> blk[3];
    for (int c = 0; c < 3; c++) blk[c].assign((size_t)nd * nd, std::vector<double>());
    std::vector<double> A(n3, 0.0);
    auto put = [&](int c, int l2, int l1, int i0, int i1, int j0, int j1, int a, int b, int ca, int cb) {
      std::vector<double> m(n3, 0.0);
      polar_to_rec(g, cones[c], i0, i1, j0, j1, a, b, ca, cb, &m);
      for (size_t t = 0; t < n3; t++) A[t] += m[t];
      blk[c][(size_t)(l2 - 1) * nd + (l1 - 1)] = std::move(m);
    };
    for (int c = 0; c < 3; c++) {
      put(c, 1, 1, 1, s1, 1, s1, s1, s1, 0, 0);
      for (int l2 = 2; l2 <= nd - 1; l2++)
        for (int l1 = 2; l1 <= nd - 1; l1++)
          put(c, l2, l1, (l1 - 1) * s + 1, l1 * s + 1, (l2 - 1) * s + 1, l2 * s + 1, s1, s1, -1, -1);
      put(c, 1, nd, (nd - 1) * s + 1, nd * s, 1, s1, s, s1, s - 1, 0);
      for (int l2 = 2; l2 <= nd - 1; l2++)
        put(c, l2, nd, (nd - 1) * s + 1, nd * s, (l2 - 1) * s + 1, l2 * s + 1, s, s1, -1, -1);
      for (int l2 = 2; l2 <= nd - 1; l2++) put(c, l2, 1, 1, s1, (l2 - 1) * s + 1, l2 * s + 1, s1, s1, -1, -1);
      put(c, nd, 1, 1, s1, (nd - 1) * s + 1, nd * s, s1, s, 0, s - 1);
      for (int l1 = 2; l1 <= nd - 1; l1++)
        put(c, nd, l1, (l1 - 1) * s + 1, l1 * s + 1, (nd - 1) * s + 1, nd * s, s1, s, -1, -1);
      for (int l1 = 2; l1 <= nd - 1; l1++) put(c, 1, l1, (l1 - 1) * s + 1, l1 * s + 1, 1, s1, s1, s1, -1, -1);
      put(c, nd, nd, (nd - 1) * s + 1, nd * s, (nd - 1) * s + 1, nd * s, s, s, s - 1, s - 1);
    }
    const int order[3] = {1, 0, 2};  // F(1,:) <-> F(2,:)
    for (int oc = 0; oc < 3; oc++) {
      const int c = order[oc];
      for (int b = 0; b < nd * nd; b++) {
        std::vector<cd> f(n3);
        for (size_t t = 0; t < n3; t++) f[t] = cd(blk[c][b][t] / A[t], 0.0);
        // real(fftshift(ifftn(fftshift(F))))
        fftshift3(f, cube);
        fft3_inplace(f, cube, +1);
        fftshift3(f, cube);
        const double sc = 1.0 / (double)n3;
        for (size_t t = 0; t < n3; t++) out.push_back(f[t].real() * sc);
      }
    }
  }
  return out;
}

// Spectrum of a cube^3 filter zero-padded (at the end, as fft(B, l) in
// convnfft.m:167-181) to L0 x L1 x L2; full complex, index (u*L1 + v)*L2 + w.
void filter_spectrum_3d(const double* f, int cube, int L0, int L1, int L2, std::vector<cd>* out) {
  out->assign((size_t)L0 * L1 * L2, cd(0, 0));
  std::vector<cd>& S = *out;
  for (int x = 0; x < cube; x++)
    for (int y = 0; y < cube; y++)
      for (int z = 0; z < cube; z++) S[((size_t)x * L1 + y) * L2 + z] = cd(f[((size_t)x * cube + y) * cube + z], 0);
  std::vector<cd> line;
  // axis 2 on the nonzero (x, y) lines, axis 1 on the nonzero x planes, then axis 0 everywhere
  line.resize(L2);
  for (int x = 0; x < cube; x++)
    for (int y = 0; y < cube; y++) {
      cd* p = &S[((size_t)x * L1 + y) * L2];
      fft_inplace(p, L2, -1);
    }
  line.resize(L1);
  for (int x = 0; x < cube; x++)
    for (int w = 0; w < L2; w++) {
      for (int v = 0; v < L1; v++) line[v] = S[((size_t)x * L1 + v) * L2 + w];
      fft_inplace(line.data(), L1, -1);
      for (int v = 0; v < L1; v++) S[((size_t)x * L1 + v) * L2 + w] = line[v];
    }
  // axis 0: gather one (u, w) slab per v so the strided line reads stay in cache
  line.resize(L0);
  std::vector<cd> slab((size_t)L0 * L2);
  for (int v = 0; v < L1; v++) {
    for (int u = 0; u < cube; u++)
      std::memcpy(&slab[(size_t)u * L2], &S[((size_t)u * L1 + v) * L2], sizeof(cd) * L2);
    for (int w = 0; w < L2; w++) {
      for (int u = 0; u < cube; u++) line[u] = slab[(size_t)u * L2 + w];
      for (int u = cube; u < L0; u++) line[u] = cd(0, 0);
      fft_inplace(line.data(), L0, -1);
      for (int u = 0; u < L0; u++) slab[(size_t)u * L2 + w] = line[u];
    }
    for (int u = 0; u < L0; u++)
      std::memcpy(&S[((size_t)u * L1 + v) * L2], &slab[(size_t)u * L2], sizeof(cd) * L2);
  }
}

// rcos.m:1-13
static double rcos(double x) {
  if (x <= 0) return 0.0;
  if (x >= 1) return 1.0;
  return 0.5 * (1 - std::cos(M_PI * x));
}

// PrySDdec_onestep.m:48-82 along one axis of FFT length nr: K and the window
// values v[0..K] (the mirrored negative half uses v[nr - p]).
void pyr_window_1d(int nr, double w, double tbw, int* K, std::vector<double>* v) {
  const int k = (int)std::ceil(nr / 2.0 * (w + tbw));
  const double den = k - std::floor(nr / 2.0 * (w - tbw));
  v->resize(k + 1);
  for (int p = 0; p <= k; p++) (*v)[p] = std::sqrt(rcos((k - p) / den));
  *K = k;
}

}  // namespace nsst
