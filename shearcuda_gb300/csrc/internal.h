// Internal declarations shared by the NSST host library and its kernels.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/nsst.h"

namespace nsst {

enum { THRESH_HARD = NSST_THRESH_HARD, THRESH_SOFT = NSST_THRESH_SOFT };

// ---------------------------------------------------------------- job lists
// Row/column jobs hold element offsets; the launch passes the base pointers.
// That keeps a plan's job lists static in device memory while the caller's
// buffers change from call to call.
struct RowJob {
  size_t src;    // offset (in float2) of the job's first row in the source
  size_t dst;    // offset (in float2) in the destination
  int th_index;  // index into the threshold array (threshold kernels)
  int item;      // batch item; jobs with item >= n_active are skipped
};

struct ColJob {
  size_t src;    // offset (float2) of the packed H x W/2 source
  size_t dst;    // offset (float2) of the destination
  size_t spec;   // offset (float2) of the band spectrum (first band for synthesis)
  size_t m0;     // offset (float2) of the column-0 side array
  int nbands;    // synthesis: number of bands summed
  int item;      // batch item; jobs with item >= n_active are skipped
};

// One (item, level) of the fused directional stage (k_dir_fused.cu).
struct FusedJob {
  size_t dst;     // offset (float2) of the level's band-sum plane (column-IFFT'd, as k_band_synthesis leaves it)
  size_t spec;    // offset (float2) of the level's first band spectrum
  size_t m0;      // offset (float2) of the level's first column-0 side array
  int ymap_row;   // first row of the level spectrum in the tensor map over the level spectra
  int nbands;     // bands of the level
  int th0;        // threshold index of the level's first band
  int item;       // batch item; jobs with item >= n_active are skipped
};

struct AtrousJob {
  const float* xa;
  const float* xb;  // optional second input (synthesis)
  float* out;
  int H, W;         // input image size
  int Ho, Wo;       // output size (0 = same as the input) for the forward
                    // step; the extended domain H + M(F-1) x W + M(F-1) for
                    // the adjoint step
};
constexpr int kMaxAtrousJobs = 64;
struct AtrousJobs {  // passed by value
  AtrousJob j[kMaxAtrousJobs];
};

// Per-item image pointers of the DCT pyramid's first and last passes (the
// caller's buffers), passed by value; rows of W floats, 16-byte aligned.
struct DctIo {
  const float* src[kMaxAtrousJobs];
  float* dst[kMaxAtrousJobs];
};
// column transforms of the DCT pyramid (k_dct.cu): DCT-II, DCT-III, DCT-III
// followed by the forward FFT, and DCT-III -> threshold -> DCT-II
enum { kDct2 = 0, kDct3 = 1, kDctAna = 2, kDctThresh = 3 };

struct FoldJob {
  const float* z1;  // first source (extended domain) / or c for the lowpass mask
  const float* z2;  // optional second source / or g for the lowpass mask
  float* out;
};
struct FoldJobs {  // passed by value
  FoldJob j[kMaxAtrousJobs];
};

template <int F>
struct AtrousTaps {
  float w[F * F];  // filter flipped in both axes, row-major
  int cols[F];     // tap columns that hold a nonzero coefficient
  int ncols;
};
template <>
struct AtrousTaps<0> {
  float w[1];
  int cols[1];
  int ncols;
};

template <int F>
inline void fill_taps(AtrousTaps<F>& t, const float* hflip) {
  t.ncols = 0;
  for (int b = 0; b < F; b++) {
    bool nz = false;
    for (int a = 0; a < F; a++) {
      t.w[a * F + b] = hflip[a * F + b];
      nz |= hflip[a * F + b] != 0.0f;
    }
    if (nz) t.cols[t.ncols++] = b;
  }
}
inline void fill_taps(AtrousTaps<0>& t, const float*) { t.ncols = 0; }

enum class RowOp { Fwd, Inv, Thresh, Backward };
// AnalysisLevel: one job per level (all its bands); *Pairs: the same kernels on
// split-complex column pairs, with twH pointing to the broadcast twiddle table
// SynthesisRegs: the synthesis with the band sum in registers (TMA only);
// SynthesisRegsDct2: the same, the sum leaving as its column DCT-II;
// AnalysisLevelDct: the TMA level analysis finishing the level spectrum's
// columns itself (the spectral pipeline's DCT-III + FFT column pass)
enum class ColOp {
  Fwd,
  Inv,
  Analysis,
  AnalysisLevel,
  Synthesis,
  AnalysisLevelPairs,
  SynthesisPairs,
  SynthesisRegs,
  SynthesisRegsDct2,
  AnalysisLevelDct
};

bool row_len_supported(int wh);
bool col_len_supported(int h);
int row_tile(int wh);
int col_tile(int h);

cudaError_t prepare_row_kernels(int wh);
cudaError_t prepare_col_kernels(int h);
cudaError_t prepare_atrous_kernels(int FA, int FB, int Mmax);
cudaError_t launch_rows(RowOp op, const RowJob* jobs, int njobs, int n_active, int H, int W, const void* src_base,
                        void* dst_base, const float2* twWh, const float2* twW, const float* thr, int mode,
                        cudaStream_t st);
// The band row pass (RowOp::Thresh) with tile_mult (1 or 2) times the rows of
// RowCfg's tile per CTA; packed: on split-complex row pairs, with the row
// twiddle tables twWh4 / twW4 (W/2 entries each) in broadcast form.
cudaError_t launch_rows_thresh(const RowJob* jobs, int njobs, int n_active, int H, int W, const void* src_base,
                               void* dst_base, const float2* twWh, const float2* twW, const float* thr, int mode,
                               int tile_mult, cudaStream_t st, bool packed = false, const float4* twWh4 = nullptr,
                               const float4* twW4 = nullptr);
// twiddle table in broadcast form: entry t = (c.x, c.x, c.y, c.y) of tab[t]
std::vector<float4> broadcast_table(const std::vector<float2>& tab);
cudaError_t launch_cols(ColOp op, const ColJob* jobs, int njobs, int n_active, int H, int W, const float2* src_base,
                        float2* dst_base, const float2* spec_base, size_t band_stride, const float2* twH,
                        cudaStream_t st);
// Fused directional stage (k_dir_fused.cu): W_k .* Y -> column IFFT -> row
// C2R -> threshold -> R2C -> column FFT -> sum conj(W_k) .* X -> column IFFT,
// one thread-block cluster per (item, level) job, bands on chip.
bool dir_fused_supported(int H, int WH);
int dir_fused_cluster(int H, int WH);
// kernel attributes (shared memory, cluster size) and the largest number of
// co-resident clusters (0: the device cannot run them)
cudaError_t prepare_dir_fused(int H, int WH, int* max_clusters);
// tensor map (a 128-byte CUtensorMap at `out`, 64-byte aligned) over `rows`
// rows of WH float2 starting at lev
cudaError_t make_level_tmap(void* out, const float2* lev, int H, int WH, size_t rows);
// tensor map over `rows` rows of `inner` float2 from base (16-byte aligned,
// inner even), box = box_x float2 x box_y rows
cudaError_t make_tmap_2d(void* out, const void* base, int inner, size_t rows, int box_x, int box_y);
// Rows of a column-group tensor-map box: H split into the fewest equal boxes
// of at most 256 rows (the box-dimension limit).
constexpr int tma_box_rows(int H) {
  int n = (H + 255) / 256;
  while (H % n != 0) n++;
  return H / n;
}
// The level analysis and the synthesis column kernels (ColOp AnalysisLevel,
// Synthesis and their *Pairs forms, twH the broadcast table for those) with
// their column groups staged by 2-D TMA (k_cols_tma.cu) from a tensor map
// over the plan's arena (box: col_tile(H) float2 x tma_box_rows(H) rows):
// every job's src and spec offset (spec relative to the arena, as spec_row0
// * WH plus job.spec) is a multiple of WH.  err: the plan's device error word.
// per_level: the jobs come level-major with this many items per level, and
// the CTAs run in chunks of column groups across the items (0: one job per
// grid row); njobs must be a multiple of it.
bool cols_tma_supported(int H, int WH);
cudaError_t prepare_cols_tma(int H);
cudaError_t launch_cols_tma(ColOp op, const void* amap, const ColJob* jobs, int njobs, int n_active, int H, int W,
                            float2* dst_base, const float2* spec_base, size_t spec_row0, size_t band_stride,
                            const float2* twH, int* err, cudaStream_t st, const float2* wd = nullptr,
                            int per_level = 0);
cudaError_t launch_dir_fused(const void* ymap, const FusedJob* jobs, int njobs, int n_active, int nclusters, int H,
                             int W, float2* dst_base, const float2* spec_base, size_t band_stride, const float2* twH,
                             const float2* twWh, const float2* twW, const float* thr, int mode, int* err,
                             cudaStream_t st);
cudaError_t launch_atrous(const AtrousJobs& jobs, int njobs, int maxH, int maxW, int M, int FA, const float* ha,
                          int FB, const float* hb, cudaStream_t st);
// The DCT-domain pyramid of the fused pipeline (k_dct.cu).
cudaError_t prepare_dct_kernels(int H, int WH);
cudaError_t launch_dct_rows_fwd(const DctIo& io, int n, int H, int W, const float2* twWh, const float4* twD,
                                cudaStream_t st);
cudaError_t launch_dct_rows_ana(const RowJob* jobs, int njobs, int n_active, int H, int W, const void* src_base,
                                void* dst_base, const float* resp, size_t resp_stride, const float2* twWh,
                                const float2* twW, const float4* twD, bool real_out, cudaStream_t st);
cudaError_t launch_dct_rows_syn(const RowJob* jobs, int njobs, int n_active, int nlev, size_t lev_stride, int H,
                                int W, const void* src_base, void* dst_base, const float* xbase, size_t xstride,
                                const float* resp, size_t resp_stride, const float* tlow, const float2* twWh,
                                const float2* twW, const float4* twD, cudaStream_t st, bool real_in = false);
cudaError_t launch_dct_cols(int mode, const ColJob* jobs, int njobs, int n_active, int H, int W, const void* src_base,
                            void* dst_base, const float2* twH, const float2* wdH, cudaStream_t st,
                            const float* thr = nullptr, int th_stride = 0, int th_mode = 0);
cudaError_t launch_dct_cols_out(const DctIo& io, int n, int H, int W, const float2* twH, const float2* wdH,
                                cudaStream_t st);
// Adjoint helper: out (Ho x Wo, extended domain) = zero-extended full
// correlation of x with the *unflipped* filter h, Ho = H + M(F-1).
cudaError_t launch_atrous_full(const AtrousJobs& jobs, int njobs, int maxHo, int maxWo, int M, int F, const float* h,
                               cudaStream_t st);
bool atrous_pair_supported(int FA, int FB);
cudaError_t launch_fold(const FoldJobs& jobs, int njobs, int H, int W, int E1, int E2, bool accumulate,
                        cudaStream_t st);
cudaError_t launch_lowpass_backward(const FoldJobs& jobs, int njobs, size_t n, const float* tau, int mode,
                                    float* partials, int slot0, int nblk, cudaStream_t st);
cudaError_t launch_reduce_tau(const float* partials, int count, size_t stride, int nbands, float* grad_tau,
                              bool accumulate, cudaStream_t st);
cudaError_t launch_broadcast_tau(const float* tau, float* th, int nbands, int n, cudaStream_t st);
// Backward band row pass: Qc (coefficients' packed rows, src) and Qg (gradient
// packed rows, dst, in place) -> R2C(C2R(Qg) * 1[|C2R(Qc)| > t]); per-CTA soft
// threshold gradient partials at partials[th_index * pstride + item * (H/RS) + tile].
cudaError_t launch_rows_backward(const RowJob* jobs, int njobs, int n_active, int H, int W, const void* src_base,
                                 void* dst_base, const float2* twWh, const float2* twW, const float* tau, int mode,
                                 float* partials, size_t pstride, cudaStream_t st);
cudaError_t launch_thresh_bands(float* data, size_t n, int nbands, const float* thr, int mode, cudaStream_t st);
// Band row pass without a store: C2R of each band's rows and max |c| into
// bits[th_index] (float bit patterns, atomicMax; bits zeroed first).
cudaError_t launch_rows_max(const RowJob* jobs, int njobs, int n_active, int H, int W, const void* src_base,
                            const float2* twWh, const float2* twW, unsigned* bits, cudaStream_t st);
// per-plane reductions (k_reduce.cu): FP64 partial sums of squares,
// partial[plane * blocks + block]; bit patterns of the largest |x| (maxbits zeroed first)
cudaError_t launch_plane_sumsq(const float* data, size_t n, int nplanes, double* partial, int blocks,
                               cudaStream_t st);
cudaError_t launch_plane_maxabs(const float* data, size_t n, int nplanes, unsigned* maxbits, int blocks,
                                cudaStream_t st);
constexpr int kMaxPlaneWeights = NSST_MAX_LEVELS + 1;
struct PlaneWeights {  // passed by value
  float w[kMaxPlaneWeights];
};
cudaError_t launch_scale_planes(float* data, size_t n, int nplanes, const PlaneWeights& w, cudaStream_t st);

// ------------------------------------------------------------------- 3-D path
struct PyrWin {  // separable pyramid window of one level (device arrays v0..v2)
  int K[3];
  int nr[3];
  const float* v0;
  const float* v1;
  const float* v2;
};
// One pass of a batched 3-D FFT with a fused prologue / epilogue
// (k_vol3d_pass.cu).  Ranges along the two non-transformed axes select the
// CTA's sequences: axis 2 (z rows): a = x, b = y; axis 1: a = x, b = z;
// axis 0: a = y, b = z (b_n need not be a multiple of the 8-sequence group).
enum { V3_LD_CPLX = 0, V3_LD_REAL = 1, V3_LD_PAIR = 2, V3_LD_MASKED = 3 };
enum { V3_ST_CPLX = 0, V3_ST_REAL = 1, V3_ST_THRESH = 2, V3_ST_SPEC = 3, V3_ST_PAIR = 4 };
struct V3Pass {
  int axis = 2;
  int D1 = 0, D2 = 0;             // work buffer dims 1, 2
  int a_lo = 0, a_n = 0, b_lo = 0, b_n = 0;
  int in_lo = 0, in_n = 0;        // loaded range along the axis (zero elsewhere)
  int out_lo = 0, out_n = 0;      // stored range along the axis
  size_t item_stride = 0;         // float2 per item of the work buffers
  const float2* spec = nullptr;   // LD_PAIR / ST_SPEC: filter-pair spectrum (shared by the items)
  const float* rsrc = nullptr;    // LD_REAL / LD_MASKED: real volume of a box
  float* rdst = nullptr;          // ST_REAL / ST_THRESH / ST_PAIR: real volume of a box
  float* rdst2 = nullptr;         // ST_PAIR: second band
  size_t r_stride = 0;            // floats per item of rsrc / rdst
  int r1 = 0, r2 = 0;             // box dims 1, 2
  int o0 = 0, o1 = 0, o2 = 0;     // box origin in work-buffer coordinates
  const uint8_t* mka = nullptr;   // LD_MASKED keep bits (linear bit order over the box)
  const uint8_t* mkb = nullptr;
  uint8_t* mwa = nullptr;         // ST_THRESH keep bits written
  uint8_t* mwb = nullptr;
  size_t m_stride = 0;            // mask bytes per item
  const float* th = nullptr;      // ST_THRESH thresholds [item][nb_item]
  int ia = 0, ib = -1, nb_item = 0;
  float scale = 1.f;
  int first = 0;                  // ST_SPEC: assign instead of accumulate
  int m_r2 = 0;                   // keep-bit row pitch along dim 2 (0: r2), a multiple of 8 when r2 is not
};
bool v3_pass_len_supported(int n);
// the lengths with the factors 11 and 17 (k_vol3d_pass_odd.cu)
bool v3_pass_len_supported_odd(int n);
cudaError_t prepare_v3_pass_odd(int n);
cudaError_t launch_v3_pass_odd(int N, int dir, int ld, int st, float2* out, const float2* in, const V3Pass& P,
                               const float2* tw, int nitems, cudaStream_t stream);
cudaError_t prepare_v3_pass(int n);
cudaError_t launch_v3_pass(int N, int dir, int ld, int st, float2* out, const float2* in, const V3Pass& P,
                           const float2* tw, int nitems, cudaStream_t stream);
cudaError_t launch_pad_real(const float* in, size_t in_stride, float2* out, size_t out_stride, int n, int m0, int m1,
                            int m2, int L0, int L1, int L2, cudaStream_t st);
cudaError_t launch_pad_edge(const float* in, size_t in_stride, float2* out, size_t out_stride, int n, int n0, int n1,
                            int n2, int d0, int d1, int d2, cudaStream_t st);
cudaError_t launch_crop_real(const float2* in, size_t in_stride, float* out, size_t out_stride, int n, int m0, int m1,
                             int m2, int L1, int L2, int o0, int o1, int o2, float scale, cudaStream_t st);
cudaError_t launch_half(const float2* in, size_t in_stride, float2* out, size_t out_stride, int n, int d0, int d1,
                        int d2, cudaStream_t st);
cudaError_t launch_conj_extend(const float2* in, size_t in_stride, float2* out, size_t out_stride, int n, int d0,
                               int d1, int d2, cudaStream_t st);
cudaError_t launch_pyr_dec(float2* Xh, size_t stride, float2* Lp, size_t lp_stride, int n, int d0, int d1, int d2,
                           int s0, int s1, int s2, const PyrWin& w, float invDN, cudaStream_t st);
cudaError_t launch_pyr_rec(float2* Hh, size_t stride, const float2* Lp, size_t lp_stride, int n, int d0, int d1,
                           int d2, int s0, int s1, int s2, const PyrWin& w, float DN, cudaStream_t st);
cudaError_t launch_fold_edge(const float* g, size_t g_stride, float* out, size_t o_stride, float* scratch,
                             size_t s_stride, int n, int n0, int n1, int n2, int d0, int d1, int d2, cudaStream_t st);
std::vector<double> meyer_filters_3d(int cube, int nlevels, const int* num_dirs);
void filter_spectrum_3d(const double* f, int cube, int L0, int L1, int L2, std::vector<std::complex<double>>* out);
void pyr_window_1d(int nr, double w, double tbw, int* K, std::vector<double>* v);

// ------------------------------------------------------- host-side FP64 math
using cd = std::complex<double>;

struct PyramidFilters {
  std::string name;
  int F[4];                       // sizes of h0, h1, g0, g1
  std::vector<double> h[4];       // row-major F x F each: h0, h1, g0, g1
};

// atrousfilters.m tables; returns false for an unknown name.
bool pyramid_filters(const std::string& name, PyramidFilters* out);

// A complete filter bank as the reference's SHFM0002 file holds it
// (host_filterfile.cpp): per level the shearing filters, row-major, and the
// four pyramid filters.
constexpr int kShfmSingle = 0, kShfmDouble = 2;  // the file's data-type codes
struct FilterSet {
  int nlev = 0, dtype = kShfmDouble;
  int dsize[NSST_MAX_LEVELS] = {}, ndir[NSST_MAX_LEVELS] = {};
  std::vector<double> shear[NSST_MAX_LEVELS];  // ndir x dsize x dsize each
  PyramidFilters pf;
};
bool read_filter_file(const char* path, FilterSet* fs, std::string* err);
bool write_filter_file(const char* path, const FilterSet& fs, std::string* err);

// shearing_filters_Myer.m: (2^level) filters of n1 x n1, row-major, FP64.
std::vector<double> shearing_filters_myer(int n1, int level);

// In-place complex FFT of length n (n = 2^a 3^b), sign -1 forward / +1 inverse, unnormalised.
void fft_inplace(cd* data, int n, int sign);

// Spectra of one level: ndir filters zero-padded top-left to H x W, transformed,
// then divided by d = sqrt(sum_k |W_k|^2) (nsst_dec2.m:47-57).  Output: only the
// W/2+1 non-redundant columns, row-major [ndir][H][W/2+1].  Returns false if d
// vanishes somewhere.
bool level_spectra(const std::vector<double>& filters, int ndir, int n1, int H, int W, std::vector<cd>* out,
                   int nthreads);

std::vector<float2> twiddle_table(int n);            // exp(-2 pi i t / n), t < n
std::vector<float2> half_twiddle_table(int n);       // exp(-2 pi i k / n), k < n/2

// DCT-domain pyramid tables (host_dct.cpp): whether all four pyramid filters
// are symmetric in both axes with odd sizes; the (2 L + 3) response planes
// (H x W each, 1/(H W) folded in: analysis per directional level, synthesis
// per directional level, the lowpass round trip, the lowpass analysis, the
// lowpass synthesis); row twiddles (exp(-i pi k / (2W)), exp(-2 pi i k / W)) for
// k = 0..W/2; column twiddles exp(-i pi k / (2H)), k < H.
bool filters_symmetric(const PyramidFilters& pf);
void dct_pyramid_tables(const PyramidFilters& pf, int L, int H, int W, std::vector<float>* out);
std::vector<float4> dct_row_twiddles(int W);
std::vector<float2> dct_col_twiddles(int H);

// -------------------------------------------- undecimated wavelets (k_wavelet.cu)
// MakeONFilter.m: the orthonormal QMF of a family, f / norm(f); false if the
// family / parameter pair is not tabulated.
bool on_filter(const std::string& type, int par, std::vector<double>* f);

constexpr int kMaxQmf = 32;  // longest even-length tabulated QMF is Coiflet 5 (30 taps)
struct WvTaps {              // passed by value; taps multiply x[c + j*sf] (analysis) or x[c - t*sf] (synthesis)
  float a[kMaxQmf];          // lowpass
  float b[kMaxQmf];          // highpass
  int lh;
};
// Analysis taps of mrdwt_r.h:118-125 / mdwt_r.h:113-120 in the form used by
// the kernels: lo = sum_j a[j] x[c + j sf], hi = sum_j b[j] x[c + j sf].
WvTaps analysis_taps(const std::vector<double>& h);
// Synthesis taps of mirdwt_r.h:125-130: x = sum_t a[t] lo[c - t sf] + b[t] hi[c - t sf].
WvTaps synthesis_taps(const std::vector<double>& h);

struct WvPlanes {   // one level of n items (item strides in floats)
  const float* cur; size_t s_cur;   // level input (x, or the previous level's lowpass)
  float* yl; size_t s_yl;           // lowpass output
  float* yh; size_t s_yh;           // this level's three planes [LH, HL, HH]
};
// mrdwt, one level: columns into yh planes 1 (lowpass) and 0 (highpass), then
// rows in place: LL -> yl, HL -> 1, LH -> 0, HH -> 2.  thr (n floats, or
// NULL) hard-thresholds the three highpass planes: c * (|c| > thr[item]).
cudaError_t launch_rdwt_level(const WvPlanes& P, int n, int H, int W, int sf, const WvTaps& t, const float* thr,
                              cudaStream_t st);
// mirdwt, one level: rows (LL, HL) -> tl, (LH, HH) -> th; columns (tl, th) -> x.
// tl / th may be the level's HL / LH planes (the coefficients are then consumed).
cudaError_t launch_irdwt_level(const float* ll, size_t s_ll, const float* yh, size_t s_yh, float* tl, float* th,
                               size_t s_t, float* x, size_t s_x, int n, int H, int W, int sf, const WvTaps& t,
                               cudaStream_t st);
bool rdwt_width_supported(int W);
// TVCorrection (separate.m:268-276): Haar mrdwt of one level, soft threshold
// gamma on the three highpass planes, mirdwt -- fused into one 3 x 3 stencil.
cudaError_t launch_tv_haar(const float* x, float* y, size_t stride, int n, int H, int W, float a, float gamma,
                           cudaStream_t st);
// mdwt_r.h:102-176 with L = 1, HH quadrant only, FP64, for n images (item
// stride `stride` floats): hh[item][k][l] = sum_ij b[i] b[j] x[2k + i][2l + j]
// (periodic), (H/2) x (W/2) per image.
cudaError_t launch_dwt_hh(const float* x, size_t stride, int n, int H, int W, const double* b, int lh, double* hh,
                          cudaStream_t st);
// separate.m:146-155 on n items: r = (img - p1) - p2; ra1 = p1 + r; ra2 = p2 + r.
cudaError_t launch_sep_residual(const float* img, const float* p1, const float* p2, float* ra1, float* ra2,
                                size_t n, cudaStream_t st);

// error reporting
void set_error(const std::string& msg);

// cudaMalloc behind the allocation fault-injection hook
cudaError_t dev_alloc(void** p, size_t bytes);

// launch accounting (every kernel launch site calls this once per launch)
void count_launch(int n = 1);

}  // namespace nsst
