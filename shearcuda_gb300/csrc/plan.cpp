// NSST plan: filter bank construction, device buffers, job lists and the
// C ABI entry points declared in include/nsst.h.
//
// The plan plays the role of the reference's shearing dictionary
// (ShearDictionary.h:18-48 / prepare_shearing_filters_cuda.cpp:234-248):
// it owns the filter spectra, the pyramid filters, the transform tables and
// every work buffer, so execute calls allocate nothing.  Unlike the
// reference it also owns static job lists for each kernel stage, so one call
// is a fixed sequence of launches on the caller's stream.
#include <algorithm>
#include <initializer_list>
#include <numeric>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <random>
#include <thread>

#include "internal.h"

namespace nsst {

// One implementation of the directional stage: the fused cluster kernel, or
// the split kernels with an analysis variant (one CTA per band and column
// group, or per level streaming all its bands) and a row tile (1 or 2 times
// RowCfg's rows per CTA).
struct DirChoice {
  bool fused = false;
  int ana = 0;       // 0: by grid size, 1: per level, 2: per band
  int row_tile = 1;
  bool packed = false;  // row pass on split-complex row pairs (FP32x2 arithmetic)
  bool cols_packed = false;  // analysis (per level) and synthesis on split-complex column pairs
  bool cols_tma = false;     // analysis (per level) and synthesis with column groups staged by TMA
  bool syn_regs = false;     // with cols_tma: the synthesis keeps the band sum in registers
};

// autotuner buckets of the batch size n: bucket b holds 2^b <= n < 2^(b+1)
constexpr int kTuneBuckets = 13;
inline int tune_bucket(int n) {
  int b = 0;
  while (b + 1 < kTuneBuckets && (2 << b) <= n) b++;
  return b;
}

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }

// Host-side fault injection for the allocation path (tests only): the n-th
// device allocation from now fails as if the device were out of memory.
static std::atomic<int> g_fail_alloc_countdown{0};
static std::atomic<uint64_t> g_launches{0};
void count_launch(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }

cudaError_t dev_alloc(void** p, size_t bytes) {
  int c = g_fail_alloc_countdown.load();
  if (c > 0) {
    if (g_fail_alloc_countdown.fetch_sub(1) == 1) {
      *p = nullptr;
      return cudaErrorMemoryAllocation;
    }
  }
  return cudaMalloc(p, bytes);
}

}  // namespace nsst

using namespace nsst;

struct nsst_plan {
  nsst_config cfg{};
  int H = 0, W = 0, WH = 0, nlev = 0, nbands = 0, ndir_total = 0, B = 1;
  std::vector<int> ndir, first_band, band_level;  // per level / per band
  PyramidFilters pf;
  std::vector<std::vector<double>> shear_w;  // FP64 shearing filters per level (ndir x dsize^2, row-major)
  double* red_scratch = nullptr;  // per-plane reduction partials (nbands x kRedBlocks doubles)
  std::vector<float> hflip[4];  // FP32 flipped h0, h1, g0, g1 (forward steps)
  std::vector<float> h32[4];    // FP32 unflipped h0, h1, g0, g1 (adjoint steps)
  int device = 0;

  // one device arena
  char* arena = nullptr;
  size_t arena_bytes = 0;
  float2* spec = nullptr;  // [ndir_total][H][WH] then the column-0 side arrays [ndir_total][H]
  size_t m0_off = 0;       // offset (float2) of the side arrays from spec
  float2 *twH = nullptr, *twWh = nullptr, *twW = nullptr;
  float4 *twWh4 = nullptr, *twW4 = nullptr, *twH4 = nullptr;  // twWh / twW / twH with each entry as broadcast pairs
  // per-item work buffers (item i at base + i * stride)
  float* pyr = nullptr;    // (nlev+1) x H x W   analysis pyramid
  float* tmp = nullptr;    // 2 x H x W          lowpass ping-pong
  float2* lev = nullptr;   // nlev x H x WH      level spectra
  float2* band = nullptr;  // ndir_total x H x WH band scratch
  float2* sum = nullptr;   // nlev x H x WH      synthesis sums
  float* rec = nullptr;    // (nlev+1) x H x W   synthesis pyramid inputs
  size_t s_pyr = 0, s_tmp = 0, s_lev = 0, s_band = 0, s_sum = 0, s_rec = 0;  // strides (elements)
  float* th = nullptr;     // B x nbands thresholds
  float* th_host = nullptr;  // pinned staging for th
  cudaEvent_t th_done = nullptr;
  // separation loop: the wavelet branch runs on a second stream beside the shearlet branch
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  void* sep_host = nullptr;  // pinned staging of the setup's reductions
  size_t sep_host_bytes = 0;

  RowJob* j_rows_lev_fwd = nullptr;   // pyr[1..] -> lev           (B*nlev)
  ColJob* j_cols_lev = nullptr;       // lev in place              (B*nlev)
  ColJob* j_analysis = nullptr;       // lev -> band, band-major in groups of 8 items (B*ndir_total)
  ColJob* j_analysis_lev = nullptr;   // lev -> all bands of the level, level-major (B*nlev)
  RowJob* j_rows_bands = nullptr;     // band in place, same order (B*ndir_total)
  ColJob* j_synthesis = nullptr;      // band -> sum, level-major  (B*nlev)
  RowJob* j_rows_lev_inv = nullptr;   // sum -> rec[1..]           (B*nlev)
  RowJob* j_coeff_fwd = nullptr;      // caller coeffs -> band (item 0)
  RowJob* j_band_to_coeff = nullptr;  // band -> caller coeffs (item 0)

  // DCT-domain pyramid of the fused pipeline (k_dct.cu).  X = DCT2(x) in pyr
  // plane 0, the row-transformed intermediates in pyr plane 1.
  bool dct_ok = false;         // the mode and the filters allow it: tables below allocated
  bool dct_on = false;         // the fused pipeline uses it
  float* dct_ra = nullptr;     // nlev x H x W analysis responses (directional level order)
  float* dct_rs = nullptr;     // nlev x H x W synthesis responses
  float* dct_tl = nullptr;     // H x W lowpass round-trip response
  float* dct_gl = nullptr;     // H x W lowpass synthesis response (after a lowpass threshold)
  int dct_rl_plane = 0;        // plane index of the lowpass analysis response from dct_ra
  float4* twDW = nullptr;      // row twiddles, WH + 1
  float2* wdH = nullptr;       // column twiddles, H
  ColJob* j_dct_x = nullptr;   // pyr plane 1 -> pyr plane 0          (B)
  RowJob* j_dct_ana = nullptr; // pyr plane 0 -> lev, item-major       (B*nlev)
  ColJob* j_dct_sum = nullptr; // sum in place                         (B*nlev)
  RowJob* j_dct_syn = nullptr; // sum (all levels) -> pyr plane 1      (B)
  RowJob* j_dct_low = nullptr; // pyr plane 0 -> tmp plane 0: the lowpass band (B)
  ColJob* j_dct_lowc = nullptr; // tmp plane 0 in place                 (B)
  RowJob* j_dct_rec = nullptr;  // lev (bands' DCT-II planes) -> pyr plane 1 (B)

  // fused directional stage (k_dir_fused.cu): one thread-block cluster per
  // (item, level), the bands kept on chip
  bool fused_ok = false;        // the size has a fused configuration and the device runs its clusters
  int dir_mode = NSST_DIRECTIONAL_AUTO;
  int fused_clusters = 0;       // co-resident clusters of the fused kernel
  alignas(64) unsigned char fused_tmap[128] = {};  // TMA tensor map over the level spectra
  // TMA column staging of the split directional stage (k_cols_tma.cu): a
  // tensor map over the whole arena as rows of WH float2; the filter spectra
  // start at row spec_row0
  alignas(64) unsigned char cols_tmap[128] = {};
  bool cols_tma_ok = false;
  size_t spec_row0 = 0;
  FusedJob* j_fused = nullptr;  // (B*nlev) levels with more bands first, then items
  int* dev_err = nullptr;       // error word of the bounded device waits
  // autotuner record (nsst_plan_autotune): per batch-size bucket the fastest
  // directional-stage candidate, and the candidate under test while tuning
  bool tuned[kTuneBuckets] = {};
  DirChoice tuned_choice[kTuneBuckets];
  bool forcing = false;
  DirChoice forced;

  std::vector<double> scalars;
  bool has_scalars = false;
  std::vector<double> norms;  // exact band norms (nsst_band_norms), computed on first use

  // CUDA graph replay of the batched denoise launch sequence
  bool use_graphs = false;
  cudaStream_t cap_stream = nullptr;
  // a few instantiated graphs, least recently used replaced first: callers
  // that alternate buffer sets (copies of one batch overlapping the compute of
  // the next) replay without re-capturing
  struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    std::vector<const void*> key;
    int n = -1, mode = -1;
    uint64_t used = 0;
  };
  static constexpr int kGraphCache = 4;
  GraphEntry graphs[kGraphCache];
  uint64_t graph_clock = 0;

  // gradient workspace (nsst_plan_enable_grad), one allocation
  char* garena = nullptr;
  size_t garena_bytes = 0;
  float* gyp = nullptr;     // B x (nlev+1) x HW   d loss / d synthesis inputs
  float* gy = nullptr;      // B x (nlev+1) x HW   d loss / d analysis outputs
  float* gtmp = nullptr;    // B x 2 x HW          adjoint pyramid chains
  float* zext = nullptr;    // B x 2 x HWext       extended correlations
  size_t s_zext = 0;        // floats per item (2 slots)
  size_t hwext = 0;         // floats per slot
  float2* lev2 = nullptr;   // B x nlev x HWh
  float2* band2 = nullptr;  // B x ndir_total x HWh
  float2* sum2 = nullptr;   // B x nlev x HWh
  float* partials = nullptr;  // nbands x (B x ntiles)
  int ntiles = 0;             // row tiles per band
  RowJob* gj_rows_lev_fwd = nullptr;   // gyp[1..] -> lev2
  ColJob* gj_cols_lev = nullptr;       // lev2 in place
  ColJob* gj_analysis = nullptr;       // lev2 -> band2
  ColJob* gj_analysis_lev = nullptr;   // lev2 -> all bands of the level in band2, level-major (B*nlev)
  // differentiable forward: thresholded bands go to bandT so that band keeps
  // the coefficients the backward needs (valid for saved_n items)
  float2* bandT = nullptr;
  RowJob* gj_rows_T = nullptr;         // band -> bandT, threshold
  ColJob* gj_synth_T = nullptr;        // bandT -> sum
  int saved_n = 0;
  int sm_count = 152;  // streaming multiprocessors of the plan's device
  RowJob* gj_rows_backward = nullptr;  // band (plan arena) + band2 -> band2
  ColJob* gj_synthesis = nullptr;      // band2 -> sum2
  RowJob* gj_rows_lev_inv = nullptr;   // sum2 -> gy[1..]
  RowJob* gj_coeff_fwd = nullptr;      // caller coeffs -> band2 (item 0)
  RowJob* gj_band_to_coeff = nullptr;  // band2 -> caller coeffs (item 0)
  // the backward on the spectral pyramid (when dct_ok)
  bool saved_dct = false;              // the saved forward ran the spectral pyramid
  ColJob* gj_dct_x = nullptr;          // gtmp plane 0 -> gtmp plane 1 (B)
  RowJob* gj_dct_ana = nullptr;        // gtmp plane 1 -> lev2, Q tables (B*nlev)
  RowJob* gj_dct_low = nullptr;        // gtmp plane 1 -> gtmp plane 0, lowpass synthesis table (B)
  ColJob* gj_dct_gy0 = nullptr;        // gy plane 0 in place (B)
  ColJob* gj_dct_sum = nullptr;        // sum2 in place (B*nlev)
  RowJob* gj_dct_syn = nullptr;        // sum2 -> gy plane 1 (B)

  // stage timers
  bool timing = false;
  static constexpr int kMaxStages = 40;
  cudaEvent_t ev[kMaxStages + 1] = {};
  const char* stage_name[kMaxStages] = {};
  int nstage = 0;
  std::mutex mu;  // serialises calls that share the plan's work buffers
};

namespace {

nsst_status fail(nsst_status s, const std::string& msg) {
  set_error(msg);
  return s;
}

nsst_status cuda_fail(cudaError_t e, const char* what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? NSST_ERR_OUT_OF_MEMORY : NSST_ERR_CUDA;
}

#define NSST_CUDA(call)                                 \
  do {                                                  \
    cudaError_t _e = (call);                            \
    if (_e != cudaSuccess) return cuda_fail(_e, #call); \
  } while (0)
#define NSST_TRY(call)                  \
  do {                                  \
    nsst_status _s = (call);            \
    if (_s != NSST_OK) return _s;       \
  } while (0)

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

constexpr int kRedBlocks = 64;  // blocks per plane of the per-plane reductions

std::vector<float> flip_to_float(const std::vector<double>& h, int F) {
  std::vector<float> out((size_t)F * F);
  for (int a = 0; a < F; a++)
    for (int b = 0; b < F; b++) out[(size_t)a * F + b] = (float)h[(size_t)(F - 1 - a) * F + (F - 1 - b)];
  return out;
}

int host_threads() {
  unsigned n = std::thread::hardware_concurrency();
  return n == 0 ? 4 : (int)std::min(n, 32u);
}

nsst_status validate_config(const nsst_config* cfg, int H, int W) {
  if (!cfg) return fail(NSST_ERR_INVALID_ARG, "config is NULL");
  if (cfg->pyramid != NSST_PYRAMID_AUTO && cfg->pyramid != NSST_PYRAMID_DIRECT &&
      cfg->pyramid != NSST_PYRAMID_SPECTRAL)
    return fail(NSST_ERR_INVALID_ARG, "unknown pyramid mode");
  // the dilated direct convolution stages a (64 + 2^(L-1)(F-1))-wide halo
  // tile in shared memory, which bounds the depth at 6 levels
  if (cfg->nlevels < 1 || cfg->nlevels > 6) return fail(NSST_ERR_INVALID_ARG, "nlevels must be in [1, 6]");
  int nb = 1;
  for (int i = 0; i < cfg->nlevels; i++) {
    if (cfg->dcomp[i] < 0 || cfg->dcomp[i] > 6) return fail(NSST_ERR_INVALID_ARG, "dcomp must be in [0, 6]");
    if (cfg->dsize[i] < 2 || cfg->dsize[i] > 256 || (cfg->dsize[i] & 1))
      return fail(NSST_ERR_INVALID_ARG, "dsize must be even and in [2, 256]");
    if ((2 * cfg->dsize[i]) % (1 << cfg->dcomp[i]) != 0 || (2 * cfg->dsize[i]) / (1 << cfg->dcomp[i]) < 2 ||
        ((2 * cfg->dsize[i]) / (1 << cfg->dcomp[i])) % 2 != 0)
      return fail(NSST_ERR_INVALID_ARG, "2*dsize must be an even multiple of 2^dcomp (Meyer window period)");
    nb += 1 << cfg->dcomp[i];
  }
  if (nb > NSST_MAX_BANDS) return fail(NSST_ERR_INVALID_ARG, "too many bands");
  if (H <= 0 || W <= 0 || (W & 1)) return fail(NSST_ERR_INVALID_ARG, "H and W must be positive, W even");
  if (!col_len_supported(H) || !row_len_supported(W / 2))
    return fail(NSST_ERR_UNSUPPORTED_SIZE,
                "unsupported image size: H must be one of 128,192,256,384,512,768,1024,2048 and W/2 one of "
                "64,96,128,192,256,384,512,1024");
  for (int i = 0; i < cfg->nlevels; i++)
    if (cfg->dsize[i] > H || cfg->dsize[i] > W) return fail(NSST_ERR_INVALID_ARG, "dsize larger than the image");
  return NSST_OK;
}

void timer_begin(nsst_plan* p, cudaStream_t st) {
  p->nstage = 0;
  if (p->timing) cudaEventRecord(p->ev[0], st);
}
void timer_mark(nsst_plan* p, const char* name, cudaStream_t st) {
  if (!p->timing || p->nstage >= nsst_plan::kMaxStages) return;
  p->stage_name[p->nstage] = name;
  cudaEventRecord(p->ev[++p->nstage], st);
}

bool aligned16(const void* ptr) { return ((uintptr_t)ptr & 15) == 0; }

// The spectral pyramid moves 16-byte elements of the caller's images.  Under
// NSST_PYRAMID_AUTO a call with an image that is not 16-byte aligned runs on
// the direct pyramid instead (the same results to FP32 rounding); under
// NSST_PYRAMID_SPECTRAL such a call is an error rather than a silent switch.
nsst_status check_spectral(const nsst_plan* p, std::initializer_list<const void*> ptrs) {
  if (!p->dct_on || p->cfg.pyramid != NSST_PYRAMID_SPECTRAL) return NSST_OK;
  for (const void* q : ptrs)
    if (q && !aligned16(q))
      return fail(NSST_ERR_INVALID_ARG,
                  "NSST_PYRAMID_SPECTRAL needs 16-byte aligned images (NSST_PYRAMID_AUTO runs this call on the "
                  "direct pyramid)");
  return NSST_OK;
}
nsst_status check_spectral_n(const nsst_plan* p, int n, const float* const* a, const float* const* b) {
  for (int i = 0; i < n; i++) NSST_TRY(check_spectral(p, {a ? a[i] : nullptr, b ? b[i] : nullptr}));
  return NSST_OK;
}

// The directional-stage implementation of a denoise call of n items: the
// candidate under test while tuning; else the plan's mode (split or fused),
// with the tuned split settings where the autotuner chose a split candidate;
// else (auto) the tuned choice of n's bucket; else the untuned default: the
// split kernels with the column groups staged by TMA (measured faster than
// the cp.async forms at every size, 2-11 %) and the band sum of the synthesis
// in registers (faster again at every size, 12-28 %), the per-level analysis
// where its grid fills the GPU twice and the per-band analysis below, and the
// row pass on two tiles of row pairs at <= 192 points per row (faster there,
// slower at 256 and up).  The fused kernel measured slower than these at
// every size.
DirChoice dir_choice(const nsst_plan* p, int n) {
  if (p->forcing) return p->forced;
  DirChoice def;
  def.cols_tma = p->cols_tma_ok;
  def.syn_regs = p->cols_tma_ok;
  if (p->WH <= 192 && p->H % (2 * row_tile(p->WH)) == 0) {
    def.packed = true;
    def.row_tile = 2;
  }
  const int b = tune_bucket(n);
  DirChoice c = p->tuned[b] ? p->tuned_choice[b] : def;
  if (p->dir_mode == NSST_DIRECTIONAL_SPLIT && c.fused) c = def;
  if (p->dir_mode == NSST_DIRECTIONAL_FUSED) c.fused = true;
  if (!p->fused_ok) c.fused = false;
  return c;
}
bool use_fused(const nsst_plan* p, int n) { return dir_choice(p, n).fused; }


}  // namespace

// ===================================================================== API
extern "C" {

const char* nsst_last_error(void) { return g_last_error.c_str(); }
const char* nsst_version(void) { return "nsst-gb300 0.2 (sm_103a)"; }

void nsst_debug_fail_next_alloc(int n) { g_fail_alloc_countdown.store(n); }

nsst_status nsst_pyramid_filters(const char* name, int* F, double* taps) {
  if (!name || !F) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  PyramidFilters pf;
  if (!pyramid_filters(name, &pf)) return fail(NSST_ERR_INVALID_ARG, std::string("unknown filter ") + name);
  size_t at = 0;
  for (int k = 0; k < 4; k++) {
    F[k] = pf.F[k];
    if (taps) std::memcpy(taps + at, pf.h[k].data(), pf.h[k].size() * sizeof(double));
    at += pf.h[k].size();
  }
  return NSST_OK;
}

nsst_status nsst_shearing_filters(int n1, int level, double* out) {
  if (!out || n1 < 2 || (n1 & 1) || level < 0 || level > 6) return fail(NSST_ERR_INVALID_ARG, "bad arguments");
  std::vector<double> w = shearing_filters_myer(n1, level);
  std::memcpy(out, w.data(), w.size() * sizeof(double));
  return NSST_OK;
}

}  // extern "C"

namespace {

// Plan construction; ext (optional) supplies the filter bank instead of the
// Meyer construction and the named pyramid filters.
nsst_status create_plan(const nsst_config* cfg, int H, int W, int B, const FilterSet* ext, nsst_plan** out) {
  if (!out) return fail(NSST_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  NSST_TRY(validate_config(cfg, H, W));
  if (B < 1 || B > 4096) return fail(NSST_ERR_INVALID_ARG, "batch capacity must be in [1, 4096]");

  nsst_plan* p = new (std::nothrow) nsst_plan();
  if (!p) return fail(NSST_ERR_OUT_OF_MEMORY, "host allocation failed");
  p->cfg = *cfg;
  p->cfg.lpfilt[sizeof(p->cfg.lpfilt) - 1] = 0;
  p->H = H;
  p->W = W;
  p->WH = W / 2;
  p->B = B;
  p->nlev = cfg->nlevels;
  p->band_level.push_back(0);
  for (int l = 0; l < p->nlev; l++) {
    int nd = 1 << cfg->dcomp[l];
    p->first_band.push_back(p->ndir_total);
    p->ndir.push_back(nd);
    for (int k = 0; k < nd; k++) p->band_level.push_back(l + 1);
    p->ndir_total += nd;
  }
  p->nbands = 1 + p->ndir_total;

  auto destroy = [&](nsst_status s) {
    nsst_plan_destroy(p);
    return s;
  };

  const char* fname = p->cfg.lpfilt[0] ? p->cfg.lpfilt : "maxflat";
  if (ext)
    p->pf = ext->pf;
  else if (!pyramid_filters(fname, &p->pf))
    return destroy(fail(NSST_ERR_INVALID_ARG, "unknown pyramid filter"));
  for (int l = 0; l < p->nlev; l++)
    p->shear_w.push_back(ext ? ext->shear[l] : shearing_filters_myer(cfg->dsize[l], cfg->dcomp[l]));
  if (!atrous_pair_supported(p->pf.F[0], 0) || !atrous_pair_supported(p->pf.F[1], 0) ||
      !atrous_pair_supported(p->pf.F[2], p->pf.F[3]))
    return destroy(fail(NSST_ERR_INVALID_ARG, "pyramid filter sizes not compiled"));
  for (int k = 0; k < 4; k++) {
    p->hflip[k] = flip_to_float(p->pf.h[k], p->pf.F[k]);
    p->h32[k].assign(p->pf.h[k].begin(), p->pf.h[k].end());
  }
  // One reflection must cover the widest dilated filter (symext.m needs
  // p + shift <= image size; the coarsest level dilates by 2^(nlevels-1)).
  const int Mmax = 1 << (p->nlev - 1);
  int Fmax = *std::max_element(p->pf.F, p->pf.F + 4);
  if (Mmax * Fmax + 1 > std::min(H, W))
    return destroy(fail(NSST_ERR_UNSUPPORTED_SIZE, "image too small for the pyramid depth (symmetric extension)"));

  cudaError_t ce = cudaGetDevice(&p->device);
  if (ce != cudaSuccess) return destroy(cuda_fail(ce, "cudaGetDevice"));

  // ---- arena layout
  const size_t HW = (size_t)H * W, HWh = (size_t)H * p->WH;
  p->s_pyr = HW * (p->nlev + 1);
  p->s_tmp = HW * 2;
  p->s_lev = HWh * p->nlev;
  p->s_band = HWh * p->ndir_total;
  p->s_sum = HWh * p->nlev;
  p->s_rec = HW * (p->nlev + 1);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t at = off;
    off = align_up(off + bytes, 256);
    return at;
  };
  // regions that the column kernels stage by TMA start on a row of the
  // arena's tensor map (rows of WH float2)
  const size_t row_pitch = std::lcm((size_t)256, sizeof(float2) * p->WH);
  auto take_rows = [&](size_t bytes) {
    off = align_up(off, row_pitch);
    return take(bytes);
  };
  const size_t NB = (size_t)B;
  size_t o_spec = take_rows(sizeof(float2) * ((size_t)p->ndir_total * HWh + (size_t)p->ndir_total * H));
  size_t o_twH = take(sizeof(float2) * H), o_twWh = take(sizeof(float2) * p->WH),
         o_twW = take(sizeof(float2) * p->WH);
  size_t o_twWh4 = take(sizeof(float4) * p->WH), o_twW4 = take(sizeof(float4) * p->WH),
         o_twH4 = take(sizeof(float4) * H);
  size_t o_pyr = take(sizeof(float) * p->s_pyr * NB);
  size_t o_tmp = take(sizeof(float) * p->s_tmp * NB);
  size_t o_lev = take_rows(sizeof(float2) * p->s_lev * NB);
  size_t o_band = take_rows(sizeof(float2) * p->s_band * NB);
  size_t o_sum = take(sizeof(float2) * p->s_sum * NB);
  size_t o_rec = take(sizeof(float) * p->s_rec * NB);
  size_t o_red = take(sizeof(double) * p->nbands * kRedBlocks);
  size_t o_th = take(sizeof(float) * p->nbands * NB);
  const size_t nL = NB * p->nlev, nD = NB * p->ndir_total;
  size_t o_j1 = take(sizeof(RowJob) * nL), o_j2 = take(sizeof(ColJob) * nL);
  size_t o_j3 = take(sizeof(ColJob) * nD), o_j4 = take(sizeof(RowJob) * nD);
  size_t o_j5 = take(sizeof(ColJob) * nL), o_j6 = take(sizeof(RowJob) * nL);
  size_t o_j7 = take(sizeof(RowJob) * p->ndir_total), o_j8 = take(sizeof(RowJob) * p->ndir_total);
  size_t o_j9 = take(sizeof(ColJob) * nL);
  size_t o_jf = take(sizeof(FusedJob) * nL);
  size_t o_err = take(sizeof(int) * 4);
  p->dct_ok = filters_symmetric(p->pf) && cfg->pyramid != NSST_PYRAMID_DIRECT;
  if (cfg->pyramid == NSST_PYRAMID_SPECTRAL && !p->dct_ok)
    return destroy(fail(NSST_ERR_INVALID_ARG, "the spectral pyramid needs pyramid filters symmetric in both axes"));
  size_t o_dct = 0, o_twDW = 0, o_wdH = 0, o_jd1 = 0, o_jd2 = 0, o_jd3 = 0, o_jd4 = 0, o_jd5 = 0, o_jd6 = 0, o_jd7 = 0;
  if (p->dct_ok) {
    o_dct = take(sizeof(float) * HW * (2 * p->nlev + 3));
    o_twDW = take(sizeof(float4) * (p->WH + 1));
    o_wdH = take(sizeof(float2) * H);
    o_jd1 = take(sizeof(ColJob) * NB);
    o_jd2 = take(sizeof(RowJob) * nL);
    o_jd3 = take(sizeof(ColJob) * nL);
    o_jd4 = take(sizeof(RowJob) * NB);
    o_jd5 = take(sizeof(RowJob) * NB);
    o_jd6 = take(sizeof(ColJob) * NB);
    o_jd7 = take(sizeof(RowJob) * NB);
  }
  p->arena_bytes = off;
  ce = dev_alloc((void**)&p->arena, p->arena_bytes);
  if (ce != cudaSuccess) {
    p->arena = nullptr;
    return destroy(cuda_fail(ce, "device allocation of the plan arena"));
  }
  ce = cudaMallocHost((void**)&p->th_host, sizeof(float) * p->nbands * NB);
  if (ce != cudaSuccess) {
    p->th_host = nullptr;
    return destroy(cuda_fail(ce, "pinned threshold staging"));
  }
  {
    int dev = 0, smc = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&smc, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && smc > 0)
      p->sm_count = smc;
  }
  ce = cudaEventCreateWithFlags(&p->th_done, cudaEventDisableTiming);
  if (ce != cudaSuccess) return destroy(cuda_fail(ce, "cudaEventCreate"));
  char* A = p->arena;
  p->spec = (float2*)(A + o_spec);
  p->m0_off = (size_t)p->ndir_total * HWh;
  p->twH = (float2*)(A + o_twH);
  p->twWh = (float2*)(A + o_twWh);
  p->twW = (float2*)(A + o_twW);
  p->twWh4 = (float4*)(A + o_twWh4);
  p->twW4 = (float4*)(A + o_twW4);
  p->twH4 = (float4*)(A + o_twH4);
  p->pyr = (float*)(A + o_pyr);
  p->tmp = (float*)(A + o_tmp);
  p->lev = (float2*)(A + o_lev);
  p->band = (float2*)(A + o_band);
  p->sum = (float2*)(A + o_sum);
  p->rec = (float*)(A + o_rec);
  p->th = (float*)(A + o_th);
  p->red_scratch = (double*)(A + o_red);
  p->j_rows_lev_fwd = (RowJob*)(A + o_j1);
  p->j_cols_lev = (ColJob*)(A + o_j2);
  p->j_analysis = (ColJob*)(A + o_j3);
  p->j_analysis_lev = (ColJob*)(A + o_j9);
  p->j_rows_bands = (RowJob*)(A + o_j4);
  p->j_synthesis = (ColJob*)(A + o_j5);
  p->j_rows_lev_inv = (RowJob*)(A + o_j6);
  p->j_coeff_fwd = (RowJob*)(A + o_j7);
  p->j_band_to_coeff = (RowJob*)(A + o_j8);
  p->j_fused = (FusedJob*)(A + o_jf);
  p->dev_err = (int*)(A + o_err);
  ce = cudaMemset(p->dev_err, 0, sizeof(int) * 4);
  if (ce != cudaSuccess) return destroy(cuda_fail(ce, "clear the device error word"));

  // ---- filter spectra (FP64 host) -> packed FP32 layout, scaled by 1/(H W)
  {
    std::vector<float2> hspec((size_t)p->ndir_total * HWh + (size_t)p->ndir_total * H);
    const int WC = p->WH + 1;
    const double scale = 1.0 / ((double)H * W);
    for (int l = 0; l < p->nlev; l++) {
      std::vector<cd> S;
      if (!level_spectra(p->shear_w[l], p->ndir[l], cfg->dsize[l], H, W, &S, host_threads()))
        return destroy(fail(NSST_ERR_NUMERIC, "shearing filter normalisation divides by zero"));
      for (int k = 0; k < p->ndir[l]; k++) {
        const int b = p->first_band[l] + k;
        const cd* s = S.data() + (size_t)k * H * WC;
        float2* dst = hspec.data() + (size_t)b * HWh;
        float2* m0 = hspec.data() + p->m0_off + (size_t)b * H;
        for (int u = 0; u < H; u++) {
          for (int v = 1; v < p->WH; v++) {
            cd z = s[(size_t)u * WC + v] * scale;
            dst[(size_t)u * p->WH + v] = make_float2((float)z.real(), (float)z.imag());
          }
          cd w0 = s[(size_t)u * WC + 0] * scale, wn = s[(size_t)u * WC + p->WH] * scale;
          cd P = (w0 + wn) * 0.5, Mm = (w0 - wn) * 0.5;
          dst[(size_t)u * p->WH] = make_float2((float)P.real(), (float)P.imag());
          m0[u] = make_float2((float)Mm.real(), (float)Mm.imag());
        }
      }
    }
    ce = cudaMemcpy(p->spec, hspec.data(), hspec.size() * sizeof(float2), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) return destroy(cuda_fail(ce, "upload spectra"));
  }
  {
    auto tH = twiddle_table(H), tWh = twiddle_table(p->WH), tW = half_twiddle_table(W);
    ce = cudaMemcpy(p->twH, tH.data(), tH.size() * sizeof(float2), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(p->twWh, tWh.data(), tWh.size() * sizeof(float2), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(p->twW, tW.data(), tW.size() * sizeof(float2), cudaMemcpyHostToDevice);
    const auto bWh = broadcast_table(tWh), bW = broadcast_table(tW), bH = broadcast_table(tH);
    if (ce == cudaSuccess) ce = cudaMemcpy(p->twH4, bH.data(), bH.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess)
      ce = cudaMemcpy(p->twWh4, bWh.data(), bWh.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(p->twW4, bW.data(), bW.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) return destroy(cuda_fail(ce, "upload twiddles"));
  }
  // ---- static job lists (offsets in float2 units from the launch bases)
  {
    auto f2 = [&](const void* ptr) { return (size_t)((const char*)ptr - A) / sizeof(float2); };
    std::vector<RowJob> j1, j4, j6, j7, j8;
    std::vector<ColJob> j2, j3, j5;
    for (int i = 0; i < B; i++) {
      const size_t pyr = f2(p->pyr + i * p->s_pyr), lev = f2(p->lev + i * p->s_lev);
      const size_t sum = f2(p->sum + i * p->s_sum), rec = f2(p->rec + i * p->s_rec);
      for (int l = 0; l < p->nlev; l++) {
        j1.push_back(RowJob{pyr + (size_t)(l + 1) * HWh, lev + (size_t)l * HWh, 0, i});
        j2.push_back(ColJob{lev + (size_t)l * HWh, lev + (size_t)l * HWh, 0, 0, 0, i});
        j6.push_back(RowJob{sum + (size_t)l * HWh, rec + (size_t)(l + 1) * HWh, 0, i});
      }
    }
    // groups of 8 items, band-major inside a group: the CTAs running together
    // read the same filter spectrum, and a group's level spectra (8 x 4 B/px)
    // stay in L2 across the bands of their level
    constexpr int kGroup = 8;
    for (int g0 = 0; g0 < B; g0 += kGroup) {
      for (int b = 0; b < p->ndir_total; b++) {
        const int l = p->band_level[1 + b] - 1;
        for (int i = g0; i < std::min(B, g0 + kGroup); i++) {
          const size_t lev = f2(p->lev + i * p->s_lev), band = f2(p->band + i * p->s_band);
          j3.push_back(ColJob{lev + (size_t)l * HWh, band + (size_t)b * HWh, (size_t)b * HWh,
                              p->m0_off + (size_t)b * H, 1, i});
          j4.push_back(RowJob{band + (size_t)b * HWh, band + (size_t)b * HWh, i * p->nbands + 1 + b, i});
        }
      }
    }
    for (int l = 0; l < p->nlev; l++) {
      for (int i = 0; i < B; i++) {
        const size_t band = f2(p->band + i * p->s_band), sum = f2(p->sum + i * p->s_sum);
        j5.push_back(ColJob{band + (size_t)p->first_band[l] * HWh, sum + (size_t)l * HWh,
                            (size_t)p->first_band[l] * HWh, p->m0_off + (size_t)p->first_band[l] * H, p->ndir[l],
                            i});
      }
    }
    // one analysis job per (level, item), level-major: the CTAs running
    // together stream the same filter spectra through L2
    std::vector<ColJob> j9;
    for (int l = 0; l < p->nlev; l++) {
      for (int i = 0; i < B; i++) {
        const size_t lev = f2(p->lev + i * p->s_lev), band = f2(p->band + i * p->s_band);
        j9.push_back(ColJob{lev + (size_t)l * HWh, band + (size_t)p->first_band[l] * HWh,
                            (size_t)p->first_band[l] * HWh, p->m0_off + (size_t)p->first_band[l] * H, p->ndir[l], i});
      }
    }
    for (int b = 0; b < p->ndir_total; b++) {
      const size_t band0 = f2(p->band);
      // coefficient plane 1+b of the caller's buffer <-> band scratch of item 0
      j7.push_back(RowJob{(size_t)(1 + b) * HWh, band0 + (size_t)b * HWh, 1 + b, 0});
      j8.push_back(RowJob{band0 + (size_t)b * HWh, (size_t)(1 + b) * HWh, 1 + b, 0});
    }
    auto up = [&](void* dst, const void* src, size_t bytes) {
      return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    };
    ce = up(p->j_rows_lev_fwd, j1.data(), j1.size() * sizeof(RowJob));
    if (ce == cudaSuccess) ce = up(p->j_cols_lev, j2.data(), j2.size() * sizeof(ColJob));
    if (ce == cudaSuccess) ce = up(p->j_analysis, j3.data(), j3.size() * sizeof(ColJob));
    if (ce == cudaSuccess) ce = up(p->j_analysis_lev, j9.data(), j9.size() * sizeof(ColJob));
    if (ce == cudaSuccess) ce = up(p->j_rows_bands, j4.data(), j4.size() * sizeof(RowJob));
    if (ce == cudaSuccess) ce = up(p->j_synthesis, j5.data(), j5.size() * sizeof(ColJob));
    if (ce == cudaSuccess) ce = up(p->j_rows_lev_inv, j6.data(), j6.size() * sizeof(RowJob));
    if (ce == cudaSuccess) ce = up(p->j_coeff_fwd, j7.data(), j7.size() * sizeof(RowJob));
    if (ce == cudaSuccess) ce = up(p->j_band_to_coeff, j8.data(), j8.size() * sizeof(RowJob));
    if (ce != cudaSuccess) return destroy(cuda_fail(ce, "upload job lists"));
  }
  if (p->dct_ok) {
    p->dct_ra = (float*)(A + o_dct);
    p->dct_rs = p->dct_ra + HW * p->nlev;
    p->dct_tl = p->dct_rs + HW * p->nlev;
    p->dct_rl_plane = 2 * p->nlev + 1;
    p->dct_gl = p->dct_ra + HW * (2 * p->nlev + 2);
    p->twDW = (float4*)(A + o_twDW);
    p->wdH = (float2*)(A + o_wdH);
    p->j_dct_x = (ColJob*)(A + o_jd1);
    p->j_dct_ana = (RowJob*)(A + o_jd2);
    p->j_dct_sum = (ColJob*)(A + o_jd3);
    p->j_dct_syn = (RowJob*)(A + o_jd4);
    p->j_dct_low = (RowJob*)(A + o_jd5);
    p->j_dct_lowc = (ColJob*)(A + o_jd6);
    p->j_dct_rec = (RowJob*)(A + o_jd7);
    std::vector<float> tab;
    dct_pyramid_tables(p->pf, p->nlev, H, W, &tab);
    auto tw = dct_row_twiddles(W);
    auto wh = dct_col_twiddles(H);
    auto f2 = [&](const void* ptr) { return (size_t)((const char*)ptr - A) / sizeof(float2); };
    std::vector<ColJob> jx, js, jlc;
    std::vector<RowJob> ja, jy, jl, jr;
    for (int i = 0; i < B; i++) {
      const size_t p0 = f2(p->pyr + i * p->s_pyr), p1 = f2(p->pyr + i * p->s_pyr + HW);
      const size_t lev = f2(p->lev + i * p->s_lev), sum = f2(p->sum + i * p->s_sum);
      const size_t t0 = f2(p->tmp + i * p->s_tmp);
      jx.push_back(ColJob{p1, p0, 0, 0, 0, i});
      jy.push_back(RowJob{sum, p1, 0, i});
      jl.push_back(RowJob{p0, t0, p->dct_rl_plane, i});
      jlc.push_back(ColJob{t0, t0, 0, 0, 0, i});
      jr.push_back(RowJob{lev, p1, 0, i});
      for (int l = 0; l < p->nlev; l++) {
        ja.push_back(RowJob{p0, lev + (size_t)l * HWh, l, i});
        js.push_back(ColJob{sum + (size_t)l * HWh, sum + (size_t)l * HWh, 0, 0, 0, i});
      }
    }
    ce = cudaMemcpy(p->dct_ra, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(p->twDW, tw.data(), tw.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(p->wdH, wh.data(), wh.size() * sizeof(float2), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(p->j_dct_x, jx.data(), jx.size() * sizeof(ColJob), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(p->j_dct_ana, ja.data(), ja.size() * sizeof(RowJob), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(p->j_dct_sum, js.data(), js.size() * sizeof(ColJob), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(p->j_dct_syn, jy.data(), jy.size() * sizeof(RowJob), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(p->j_dct_low, jl.data(), jl.size() * sizeof(RowJob), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(p->j_dct_lowc, jlc.data(), jlc.size() * sizeof(ColJob), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(p->j_dct_rec, jr.data(), jr.size() * sizeof(RowJob), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = prepare_dct_kernels(H, p->WH);
    if (ce != cudaSuccess) return destroy(cuda_fail(ce, "DCT pyramid tables"));
    p->dct_on = true;
  }
  ce = prepare_row_kernels(p->WH);
  if (ce == cudaSuccess) ce = prepare_col_kernels(H);
  if (ce == cudaSuccess) ce = prepare_atrous_kernels(p->pf.F[0], 0, Mmax);
  if (ce == cudaSuccess) ce = prepare_atrous_kernels(p->pf.F[1], 0, Mmax);
  if (ce == cudaSuccess) ce = prepare_atrous_kernels(p->pf.F[2], p->pf.F[3], Mmax);
  if (ce != cudaSuccess) return destroy(cuda_fail(ce, "kernel attribute setup"));
  // fused directional stage: where the size has a configuration and the
  // device can hold its clusters (else the split kernels run)
  if (dir_fused_supported(H, p->WH)) {
    int ncl = 0;
    ce = prepare_dir_fused(H, p->WH, &ncl);
    if (ce == cudaSuccess && ncl > 0)
      ce = make_level_tmap(p->fused_tmap, p->lev, H, p->WH, (size_t)B * p->nlev * H);
    if (ce == cudaSuccess && ncl > 0) {
      auto f2 = [&](const void* ptr) { return (size_t)((const char*)ptr - A) / sizeof(float2); };
      std::vector<int> order(p->nlev);
      for (int l = 0; l < p->nlev; l++) order[l] = l;
      // levels with more bands first: the long jobs start early
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return p->ndir[a] > p->ndir[b]; });
      std::vector<FusedJob> jf;
      for (int l : order)
        for (int i = 0; i < B; i++)
          jf.push_back(FusedJob{f2(p->sum + i * p->s_sum + (size_t)l * HWh), (size_t)p->first_band[l] * HWh,
                                p->m0_off + (size_t)p->first_band[l] * H, (i * p->nlev + l) * H, p->ndir[l],
                                i * p->nbands + 1 + p->first_band[l], i});
      ce = cudaMemcpy(p->j_fused, jf.data(), jf.size() * sizeof(FusedJob), cudaMemcpyHostToDevice);
      if (ce != cudaSuccess) return destroy(cuda_fail(ce, "upload fused job list"));
      p->fused_ok = true;
      p->fused_clusters = ncl;
    } else {
      (void)cudaGetLastError();  // the split kernels stay; clear a refused attribute or occupancy query
    }
  }
  // TMA column staging (an autotuner candidate): one tensor map over the arena
  {
    const size_t pitch = sizeof(float2) * p->WH, rows = p->arena_bytes / pitch;
    if (cols_tma_supported(H, p->WH) && (size_t)(p->spec - (float2*)A) % p->WH == 0 && rows <= (size_t)INT32_MAX) {
      ce = prepare_cols_tma(H);
      if (ce == cudaSuccess) ce = make_tmap_2d(p->cols_tmap, A, p->WH, rows, col_tile(H), tma_box_rows(H));
      if (ce == cudaSuccess) {
        p->cols_tma_ok = true;
        p->spec_row0 = (size_t)(p->spec - (float2*)A) / p->WH;
      } else {
        (void)cudaGetLastError();  // the cp.async column kernels stay
      }
    }
  }
  *out = p;
  return NSST_OK;
}

}  // namespace

extern "C" {

nsst_status nsst_plan_create_batch(const nsst_config* cfg, int H, int W, int B, nsst_plan** out) {
  return create_plan(cfg, H, W, B, nullptr, out);
}

nsst_status nsst_plan_create_from_file(const char* path, int H, int W, int B, nsst_plan** out) {
  if (!out) return fail(NSST_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if (!path) return fail(NSST_ERR_INVALID_ARG, "path is NULL");
  FilterSet fs;
  std::string err;
  if (!read_filter_file(path, &fs, &err)) return fail(NSST_ERR_INVALID_ARG, err);
  nsst_config cfg{};
  cfg.nlevels = fs.nlev;
  for (int l = 0; l < fs.nlev; l++) {
    int dc = 0;
    while ((1 << dc) < fs.ndir[l]) dc++;
    if ((1 << dc) != fs.ndir[l]) return fail(NSST_ERR_INVALID_ARG, "number of directions must be a power of two");
    cfg.dcomp[l] = dc;
    cfg.dsize[l] = fs.dsize[l];
  }
  std::strcpy(cfg.lpfilt, "file");
  cfg.pyramid = NSST_PYRAMID_AUTO;
  return create_plan(&cfg, H, W, B, &fs, out);
}

nsst_status nsst_filters_save(const char* path, const nsst_config* cfg, int data_type) {
  if (!path || !cfg) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  if (data_type != kShfmSingle && data_type != kShfmDouble)
    return fail(NSST_ERR_INVALID_ARG, "data_type must be 0 (single) or 2 (double)");
  if (cfg->nlevels < 1 || cfg->nlevels > NSST_MAX_LEVELS) return fail(NSST_ERR_INVALID_ARG, "bad nlevels");
  FilterSet fs;
  fs.nlev = cfg->nlevels;
  fs.dtype = data_type;
  for (int l = 0; l < fs.nlev; l++) {
    if (cfg->dcomp[l] < 0 || cfg->dcomp[l] > 6 || cfg->dsize[l] < 2 || cfg->dsize[l] > 256)
      return fail(NSST_ERR_INVALID_ARG, "bad dcomp / dsize");
    fs.dsize[l] = cfg->dsize[l];
    fs.ndir[l] = 1 << cfg->dcomp[l];
    fs.shear[l] = shearing_filters_myer(cfg->dsize[l], cfg->dcomp[l]);
  }
  char name[17] = {0};
  std::memcpy(name, cfg->lpfilt, 16);
  if (!pyramid_filters(name[0] ? name : "maxflat", &fs.pf)) return fail(NSST_ERR_INVALID_ARG, "unknown pyramid filter");
  std::string err;
  if (!write_filter_file(path, fs, &err)) return fail(NSST_ERR_INVALID_ARG, err);
  return NSST_OK;
}

nsst_status nsst_filters_load(const char* path, int* nlevels, int* dsize, int* ndir, int* F, double* shear,
                              double* pyr, int* data_type) {
  if (!path || !nlevels) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  FilterSet fs;
  std::string err;
  if (!read_filter_file(path, &fs, &err)) return fail(NSST_ERR_INVALID_ARG, err);
  *nlevels = fs.nlev;
  if (data_type) *data_type = fs.dtype;
  size_t at = 0;
  for (int l = 0; l < fs.nlev; l++) {
    if (dsize) dsize[l] = fs.dsize[l];
    if (ndir) ndir[l] = fs.ndir[l];
    if (shear) std::memcpy(shear + at, fs.shear[l].data(), fs.shear[l].size() * sizeof(double));
    at += fs.shear[l].size();
  }
  at = 0;
  for (int k = 0; k < 4; k++) {
    if (F) F[k] = fs.pf.F[k];
    if (pyr) std::memcpy(pyr + at, fs.pf.h[k].data(), fs.pf.h[k].size() * sizeof(double));
    at += fs.pf.h[k].size();
  }
  return NSST_OK;
}

nsst_status nsst_plan_create(const nsst_config* cfg, int H, int W, nsst_plan** out) {
  return nsst_plan_create_batch(cfg, H, W, 1, out);
}

nsst_status nsst_plan_destroy(nsst_plan* p) {
  if (!p) return NSST_OK;
  if (p->arena || p->th_host) cudaDeviceSynchronize();  // outstanding work may still use the buffers
  for (cudaEvent_t e : p->ev)
    if (e) cudaEventDestroy(e);
  for (auto& g : p->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  if (p->th_done) cudaEventDestroy(p->th_done);
  if (p->side) cudaStreamDestroy(p->side);
  if (p->fork_ev) cudaEventDestroy(p->fork_ev);
  if (p->join_ev) cudaEventDestroy(p->join_ev);
  if (p->sep_host) cudaFreeHost(p->sep_host);
  if (p->th_host) cudaFreeHost(p->th_host);
  if (p->garena) cudaFree(p->garena);
  if (p->arena) cudaFree(p->arena);
  delete p;
  return NSST_OK;
}

int nsst_plan_num_bands(const nsst_plan* p) { return p ? p->nbands : 0; }
int nsst_plan_batch_capacity(const nsst_plan* p) { return p ? p->B : 0; }

nsst_status nsst_plan_band_levels(const nsst_plan* p, int* out) {
  if (!p || !out) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  std::copy(p->band_level.begin(), p->band_level.end(), out);
  return NSST_OK;
}

size_t nsst_plan_device_bytes(const nsst_plan* p) { return p ? p->arena_bytes : 0; }

nsst_status nsst_level_spectra(int dsize, int dcomp, int H, int W, double* out) {
  if (!out || dsize < 2 || (dsize & 1) || dcomp < 0 || dcomp > 6 || H < dsize || W < dsize || (W & 1))
    return fail(NSST_ERR_INVALID_ARG, "bad arguments");
  std::vector<double> w = shearing_filters_myer(dsize, dcomp);
  std::vector<cd> S;
  if (!level_spectra(w, 1 << dcomp, dsize, H, W, &S, host_threads()))
    return fail(NSST_ERR_NUMERIC, "normalisation divides by zero");
  std::memcpy(out, S.data(), S.size() * sizeof(cd));
  return NSST_OK;
}

nsst_status nsst_plan_level_spectra(const nsst_plan* p, int level, double* out) {
  if (!p || !out || level < 0 || level >= p->nlev) return fail(NSST_ERR_INVALID_ARG, "bad arguments");
  std::vector<cd> S;
  if (!level_spectra(p->shear_w[level], p->ndir[level], p->cfg.dsize[level], p->H, p->W, &S, host_threads()))
    return fail(NSST_ERR_NUMERIC, "shearing filter normalisation divides by zero");
  std::memcpy(out, S.data(), S.size() * sizeof(cd));
  return NSST_OK;
}

nsst_status nsst_plan_set_scalars(nsst_plan* p, const double* s) {
  if (!p || !s) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  for (int b = 0; b < p->nbands; b++)
    if (!std::isfinite(s[b]) || s[b] < 0) return fail(NSST_ERR_INVALID_ARG, "scalars must be finite and >= 0");
  p->scalars.assign(s, s + p->nbands);
  p->has_scalars = true;
  return NSST_OK;
}

nsst_status nsst_plan_use_graphs(nsst_plan* p, int enable) {
  if (!p) return fail(NSST_ERR_INVALID_ARG, "NULL plan");
  std::lock_guard<std::mutex> lk(p->mu);
  if (enable && !p->cap_stream) NSST_CUDA(cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking));
  p->use_graphs = enable != 0;
  return NSST_OK;
}

nsst_status nsst_plan_set_directional(nsst_plan* p, int mode) {
  if (!p) return fail(NSST_ERR_INVALID_ARG, "NULL plan");
  if (mode != NSST_DIRECTIONAL_AUTO && mode != NSST_DIRECTIONAL_SPLIT && mode != NSST_DIRECTIONAL_FUSED)
    return fail(NSST_ERR_INVALID_ARG, "unknown directional mode");
  std::lock_guard<std::mutex> lk(p->mu);
  if (mode == NSST_DIRECTIONAL_FUSED && !p->fused_ok)
    return fail(NSST_ERR_UNSUPPORTED_SIZE,
                "no fused directional configuration for this image size on this device (sizes 256x256, 384x512, "
                "512x512)");
  if (mode != p->dir_mode) {  // captured graphs hold the other kernels
    for (auto& g : p->graphs)
      if (g.exec) {
        cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
        g.key.clear();
      }
  }
  p->dir_mode = mode;
  return NSST_OK;
}

int nsst_plan_directional(const nsst_plan* p, int n) {
  if (!p || n < 1) return -1;
  return use_fused(p, n) ? NSST_DIRECTIONAL_FUSED : NSST_DIRECTIONAL_SPLIT;
}

int nsst_plan_fused_clusters(const nsst_plan* p) { return p && p->fused_ok ? p->fused_clusters : 0; }

nsst_status nsst_plan_check_device(nsst_plan* p) {
  if (!p) return fail(NSST_ERR_INVALID_ARG, "NULL plan");
  std::lock_guard<std::mutex> lk(p->mu);
  int host[4] = {};
  NSST_CUDA(cudaDeviceSynchronize());
  NSST_CUDA(cudaMemcpy(host, p->dev_err, sizeof(host), cudaMemcpyDeviceToHost));
  if (host[0] != 0) {
    NSST_CUDA(cudaMemset(p->dev_err, 0, sizeof(host)));
    return fail(NSST_ERR_TIMEOUT, "a bounded device-side wait (TMA completion) ran out; the outputs of the calls "
                                  "since the last check are invalid");
  }
  return NSST_OK;
}

}  // extern "C"

// ============================================================ stage helpers
namespace {

// atrousdec.m:19-51 on the device for n items: x[i] -> y(i, 0) lowpass,
// y(i, 1..nlev) bandpass coarse -> fine; y(i, k) = ybase[i] + k * HW.
nsst_status run_atrousdec(nsst_plan* p, int n, const float* const* x, float* const* ybase, float* lowpass0,
                          cudaStream_t st, int levels = 0) {
  const int H = p->H, W = p->W, L = levels > 0 ? levels : p->nlev;
  const size_t HW = (size_t)H * W;
  static const char* kHi[] = {"atrous_dec_h1_M1",  "atrous_dec_h1_M2",  "atrous_dec_h1_M4",  "atrous_dec_h1_M8",
                              "atrous_dec_h1_M16", "atrous_dec_h1_M32", "atrous_dec_h1_M64", "atrous_dec_h1_M128"};
  static const char* kLo[] = {"atrous_dec_h0_M1",  "atrous_dec_h0_M2",  "atrous_dec_h0_M4",  "atrous_dec_h0_M8",
                              "atrous_dec_h0_M16", "atrous_dec_h0_M32", "atrous_dec_h0_M64", "atrous_dec_h0_M128"};
  for (int i = 0; i < L; i++) {  // i = 0 is the undilated first level
    const int M = 1 << i;
    for (int c0 = 0; c0 < n; c0 += kMaxAtrousJobs) {
      const int cn = std::min(kMaxAtrousJobs, n - c0);
      AtrousJobs jh{};
      for (int t = 0; t < cn; t++) {
        const int it = c0 + t;
        const float* cur = (i == 0) ? x[it] : p->tmp + it * p->s_tmp + (size_t)((i - 1) & 1) * HW;
        jh.j[t] = AtrousJob{cur, nullptr, ybase[it] + (size_t)(L - i) * HW, H, W};
      }
      cudaError_t e = launch_atrous(jh, cn, H, W, M, p->pf.F[1], p->hflip[1].data(), 0, nullptr, st);
      if (e != cudaSuccess) return cuda_fail(e, "atrous analysis launch");
    }
    timer_mark(p, kHi[i], st);
    for (int c0 = 0; c0 < n; c0 += kMaxAtrousJobs) {
      const int cn = std::min(kMaxAtrousJobs, n - c0);
      AtrousJobs jl{};
      for (int t = 0; t < cn; t++) {
        const int it = c0 + t;
        const float* cur = (i == 0) ? x[it] : p->tmp + it * p->s_tmp + (size_t)((i - 1) & 1) * HW;
        float* lo = (i == L - 1) ? (lowpass0 && it == 0 ? lowpass0 : ybase[it])
                                 : p->tmp + it * p->s_tmp + (size_t)(i & 1) * HW;
        jl.j[t] = AtrousJob{cur, nullptr, lo, H, W};
      }
      cudaError_t e = launch_atrous(jl, cn, H, W, M, p->pf.F[0], p->hflip[0].data(), 0, nullptr, st);
      if (e != cudaSuccess) return cuda_fail(e, "atrous analysis launch");
    }
    timer_mark(p, kLo[i], st);
  }
  return NSST_OK;
}

// atrousrec.m:18-41 on the device for n items: y(i, k) = ybase[i] + k*HW,
// except that low[i] (if given) replaces y(i, 0).
nsst_status run_atrousrec(nsst_plan* p, int n, const float* const* ybase, const float* const* low, float* const* out,
                          cudaStream_t st, int levels = 0) {
  const int H = p->H, W = p->W, L = levels > 0 ? levels : p->nlev;
  const size_t HW = (size_t)H * W;
  static const char* kRec[] = {"atrous_rec_M1",  "atrous_rec_M2",  "atrous_rec_M4",  "atrous_rec_M8",
                               "atrous_rec_M16", "atrous_rec_M32", "atrous_rec_M64", "atrous_rec_M128"};
  for (int i = L - 1; i >= 0; i--) {
    const int M = 1 << i;
    for (int c0 = 0; c0 < n; c0 += kMaxAtrousJobs) {
      const int cn = std::min(kMaxAtrousJobs, n - c0);
      AtrousJobs j{};
      for (int t = 0; t < cn; t++) {
        const int it = c0 + t;
        const float* cur = (i == L - 1) ? (low && low[it] ? low[it] : ybase[it])
                                        : p->tmp + it * p->s_tmp + (size_t)((i + 1) & 1) * HW;
        float* dst = (i == 0) ? out[it] : p->tmp + it * p->s_tmp + (size_t)(i & 1) * HW;
        j.j[t] = AtrousJob{cur, ybase[it] + (size_t)(L - i) * HW, dst, H, W};
      }
      cudaError_t e =
          launch_atrous(j, cn, H, W, M, p->pf.F[2], p->hflip[2].data(), p->pf.F[3], p->hflip[3].data(), st);
      if (e != cudaSuccess) return cuda_fail(e, "atrous synthesis launch");
    }
    timer_mark(p, kRec[i], st);
  }
  return NSST_OK;
}

// Thresholds t[i][b] = K[level(b)] * sigma[i] * scalars[b] -> pinned staging -> device.
nsst_status upload_thresholds(nsst_plan* p, int n, const double* sigma, const double* K, const double* scalars,
                              cudaStream_t st, float* lowpass_max) {
  if (!K || !sigma) return fail(NSST_ERR_INVALID_ARG, "K or sigma is NULL");
  if (!scalars) {
    if (!p->has_scalars) return fail(NSST_ERR_INVALID_ARG, "no scalars given and none stored in the plan");
    scalars = p->scalars.data();
  }
  // the previous call's copy must have consumed the staging buffer
  NSST_CUDA(cudaEventSynchronize(p->th_done));
  float lmax = 0.f;
  for (int i = 0; i < n; i++) {
    if (!std::isfinite(sigma[i]) || sigma[i] < 0) return fail(NSST_ERR_INVALID_ARG, "sigma must be finite and >= 0");
    for (int b = 0; b < p->nbands; b++) {
      double t = K[p->band_level[b]] * sigma[i] * scalars[b];
      if (!std::isfinite(t) || t < 0) return fail(NSST_ERR_INVALID_ARG, "thresholds must be finite and >= 0");
      p->th_host[(size_t)i * p->nbands + b] = (float)t;
    }
    lmax = std::max(lmax, p->th_host[(size_t)i * p->nbands]);
  }
  NSST_CUDA(cudaMemcpyAsync(p->th, p->th_host, sizeof(float) * p->nbands * n, cudaMemcpyHostToDevice, st));
  NSST_CUDA(cudaEventRecord(p->th_done, st));
  if (lowpass_max) *lowpass_max = lmax;
  return NSST_OK;
}

// The band analysis of n active items: one CTA per (level, item) column
// group streams all bands of the level when that grid fills the GPU twice
// (ana 0), or always (ana 1); otherwise (a single image, ana 2) one CTA per
// (band, item) column group, which has ndir times more CTAs.  pairs: the
// level form on split-complex column pairs; tma: the level form with its
// column groups staged by TMA (forward arena only).
bool analysis_per_level(const nsst_plan* p, int n, int ana) {
  const size_t ctas = (size_t)n * p->nlev * (p->WH / col_tile(p->H));
  return ana == 1 || (ana == 0 && ctas >= (size_t)2 * p->sm_count);
}

// Whether the directional stage of n items takes the TMA level analysis that
// finishes the level spectra's columns itself (the spectral pipeline then
// leaves them out of its analysis front), and whether the register-sum
// synthesis hands the band sums on as their column DCT-II.  Measured (stage
// timers, us per megapixel, fused against the two kernels): analysis 256 rows
// 101.2 / 105.1, 384 rows 106.1 / 105.3, 768 rows 121.7 / 119.6; synthesis
// 256 rows 87.9 / 83.9, 384 rows 86.6 / 87.2, 768 rows 91.5 / 94.5; at 512
// rows both sides gain (64 x 512^2: -0.02 and -0.05 ms), at 1024 neither
// side lost.
bool dct_ana_fusion_pays(const nsst_plan* p) { return p->H >= 256 && (p->H & (p->H - 1)) == 0; }
bool dct_syn_fusion_pays(const nsst_plan* p) {
  return p->H == 768 || (p->H >= 512 && (p->H & (p->H - 1)) == 0);
}

bool analysis_takes_dct(const nsst_plan* p, int n) {
  const DirChoice c = dir_choice(p, n);
  return dct_ana_fusion_pays(p) && !c.fused && c.cols_tma && p->cols_tma_ok && !c.cols_packed && p->wdH &&
         analysis_per_level(p, n, c.ana);
}

nsst_status enqueue_band_analysis(nsst_plan* p, int n, bool grad, cudaStream_t st, int ana = 0, bool pairs = false,
                                  bool tma = false, bool dctana = false) {
  float2* base = (float2*)(grad ? p->garena : p->arena);
  const bool level = analysis_per_level(p, n, ana);
  const size_t bs = (size_t)p->H * p->WH;
  const float2* tw = pairs ? (const float2*)p->twH4 : p->twH;
  if (dctana) {  // the level planes' columns are still to be transformed
    if (!(level && tma && !pairs && !grad && p->cols_tma_ok && p->wdH))
      return fail(NSST_ERR_INVALID_ARG, "internal: the level analysis cannot finish the level spectra");
    NSST_CUDA(launch_cols_tma(ColOp::AnalysisLevelDct, p->cols_tmap, p->j_analysis_lev, p->B * p->nlev, n, p->H,
                              p->W, base, p->spec, p->spec_row0, bs, p->twH, p->dev_err, st, p->wdH, p->B));
  } else if (level && tma && !grad && p->cols_tma_ok) {
    NSST_CUDA(launch_cols_tma(pairs ? ColOp::AnalysisLevelPairs : ColOp::AnalysisLevel, p->cols_tmap,
                              p->j_analysis_lev, p->B * p->nlev, n, p->H, p->W, base, p->spec, p->spec_row0, bs, tw,
                              p->dev_err, st, nullptr, p->B));
  } else if (level) {
    NSST_CUDA(launch_cols(pairs ? ColOp::AnalysisLevelPairs : ColOp::AnalysisLevel,
                          grad ? p->gj_analysis_lev : p->j_analysis_lev, p->B * p->nlev, n, p->H, p->W, base, base,
                          p->spec, bs, tw, st));
  } else {
    NSST_CUDA(launch_cols(ColOp::Analysis, grad ? p->gj_analysis : p->j_analysis, p->B * p->ndir_total, n, p->H,
                          p->W, base, base, p->spec, 0, p->twH, st));
  }
  return NSST_OK;
}

// The directional stage of the fused denoise (level spectra in p->lev, band
// sums out in p->sum): one cluster kernel, or the split analysis / row /
// synthesis kernels with the bands in p->band.
// sums_dct2 (the spectral pipeline): where the chosen synthesis can, the band
// sums leave as their column DCT-II (the next step of the spectral synthesis)
// and *sums_dct2 is set; otherwise it is left false.
nsst_status enqueue_directional(nsst_plan* p, int n, int mode, const float* TH, cudaStream_t st,
                                bool* sums_dct2 = nullptr, bool ana_dct = false) {
  const DirChoice c = dir_choice(p, n);
  if (c.fused) {
    const int ncl = std::min(p->fused_clusters, n * p->nlev);
    NSST_CUDA(launch_dir_fused(p->fused_tmap, p->j_fused, p->B * p->nlev, n, ncl, p->H, p->W, (float2*)p->arena,
                               p->spec, (size_t)p->H * p->WH, p->twH, p->twWh, p->twW, TH, mode, p->dev_err, st));
    timer_mark(p, "band_fused", st);
    return NSST_OK;
  }
  char* A = p->arena;
  const bool tma = c.cols_tma && p->cols_tma_ok;
  NSST_TRY(enqueue_band_analysis(p, n, false, st, c.ana, c.cols_packed, tma, ana_dct));
  timer_mark(p, "band_analysis_cols", st);
  NSST_CUDA(launch_rows_thresh(p->j_rows_bands, p->B * p->ndir_total, n, p->H, p->W, A, A, p->twWh, p->twW, TH, mode,
                               c.row_tile, st, c.packed, p->twWh4, p->twW4));
  timer_mark(p, "band_rows_threshold", st);
  const bool dct2 = sums_dct2 && tma && c.syn_regs && !c.cols_packed && p->wdH && dct_syn_fusion_pays(p);
  const ColOp syn = c.cols_packed          ? ColOp::SynthesisPairs
                    : (tma && c.syn_regs) ? (dct2 ? ColOp::SynthesisRegsDct2 : ColOp::SynthesisRegs)
                                          : ColOp::Synthesis;
  const float2* twc = c.cols_packed ? (const float2*)p->twH4 : p->twH;
  if (tma)
    NSST_CUDA(launch_cols_tma(syn, p->cols_tmap, p->j_synthesis, p->B * p->nlev, n, p->H, p->W, (float2*)A, p->spec,
                              p->spec_row0, (size_t)p->H * p->WH, twc, p->dev_err, st, p->wdH, p->B));
  else
    NSST_CUDA(launch_cols(syn, p->j_synthesis, p->B * p->nlev, n, p->H, p->W, (float2*)A, (float2*)A, p->spec,
                          (size_t)p->H * p->WH, twc, st));
  timer_mark(p, "band_synthesis_cols", st);
  if (dct2) *sums_dct2 = true;
  return NSST_OK;
}

// Whether a fused pipeline call can take the DCT-domain pyramid: symmetric
// filters, 16-byte aligned images.
bool dct_path(const nsst_plan* p, int n, const float* const* x, float* const* out) {
  if (!p->dct_on) return false;
  for (int i = 0; i < n; i++)
    if (!aligned16(x[i]) || !aligned16(out[i])) return false;
  return true;
}

// DCT-II of planes given by pointer (rows of the caller's images or arena
// planes; src may equal dst): rows into rows_dst[i], then down the columns
// with the static job list cols (in place on rows_dst or into its target).
nsst_status enqueue_dct_rows_io(nsst_plan* p, int n, const float* const* src, float* const* dst, cudaStream_t st) {
  for (int c0 = 0; c0 < n; c0 += kMaxAtrousJobs) {
    const int cn = std::min(kMaxAtrousJobs, n - c0);
    DctIo io{};
    for (int t = 0; t < cn; t++) {
      io.src[t] = src[c0 + t];
      io.dst[t] = dst[c0 + t];
    }
    NSST_CUDA(launch_dct_rows_fwd(io, cn, p->H, p->W, p->twWh, p->twDW, st));
  }
  return NSST_OK;
}

// DCT-III down the columns of arena planes src[i] into the caller's dst[i]
nsst_status enqueue_dct_cols_out(nsst_plan* p, int n, const float* const* src, float* const* dst, cudaStream_t st) {
  for (int c0 = 0; c0 < n; c0 += kMaxAtrousJobs) {
    const int cn = std::min(kMaxAtrousJobs, n - c0);
    DctIo io{};
    for (int t = 0; t < cn; t++) {
      io.src[t] = src[c0 + t];
      io.dst[t] = dst[c0 + t];
    }
    NSST_CUDA(launch_dct_cols_out(io, cn, p->H, p->W, p->twH, p->wdH, st));
  }
  return NSST_OK;
}

// Spectral analysis front of n items: X = DCT2(x) in pyr plane 0 (through
// plane 1), then every level's spectrum (p->lev) from X .* R_l.
// skip_cols_levels: the directional stage's level analysis finishes the
// level spectra's columns (analysis_takes_dct).
nsst_status enqueue_dct_analysis(nsst_plan* p, int n, const float* const* x, cudaStream_t st,
                                 bool skip_cols_levels = false) {
  char* A = p->arena;
  const int B = p->B, H = p->H, W = p->W;
  const size_t HW = (size_t)H * W;
  std::vector<float*> p1(n);
  for (int i = 0; i < n; i++) p1[i] = p->pyr + (size_t)i * p->s_pyr + HW;
  NSST_TRY(enqueue_dct_rows_io(p, n, x, p1.data(), st));
  timer_mark(p, "dct_rows_image", st);
  NSST_CUDA(launch_dct_cols(kDct2, p->j_dct_x, B, n, H, W, A, A, p->twH, p->wdH, st));
  timer_mark(p, "dct_cols_image", st);
  NSST_CUDA(launch_dct_rows_ana(p->j_dct_ana, B * p->nlev, n, H, W, A, A, p->dct_ra, HW, p->twWh, p->twW, p->twDW,
                                false, st));
  timer_mark(p, "dct_rows_levels", st);
  if (!skip_cols_levels) {
    NSST_CUDA(launch_dct_cols(kDctAna, p->j_cols_lev, B * p->nlev, n, H, W, A, A, p->twH, p->wdH, st));
    timer_mark(p, "dct_cols_levels", st);
  }
  return NSST_OK;
}

// The lowpass band y0 = IDCT2(X .* R_low) of n items as rows DCT-III'd into
// tmp plane 0 (its columns still in the DCT domain).
nsst_status enqueue_dct_lowpass_rows(nsst_plan* p, int n, cudaStream_t st) {
  char* A = p->arena;
  NSST_CUDA(launch_dct_rows_ana(p->j_dct_low, p->B, n, p->H, p->W, A, A, p->dct_ra, (size_t)p->H * p->W, p->twWh,
                                p->twW, p->twDW, true, st));
  return NSST_OK;
}

// Spectral synthesis back end of n items: the band sums (p->sum, from the
// band synthesis) DCT-II'd down the columns, then per row C2R -> DCT-II ->
// .* Q_l summed over the levels with low .* lowtab (low: a DCT-domain plane
// per item at lowbase + i * lowstride), DCT-III (pyr plane 1), and DCT-III down
// the columns into out[i].
nsst_status enqueue_dct_synthesis(nsst_plan* p, int n, const float* lowbase, size_t lowstride, const float* lowtab,
                                  float* const* out, cudaStream_t st, bool sums_dct2 = false) {
  char* A = p->arena;
  const int B = p->B, H = p->H, W = p->W;
  const size_t HW = (size_t)H * W;
  if (!sums_dct2) {  // (else the band synthesis has left the sums' column DCT-II)
    NSST_CUDA(launch_dct_cols(kDct2, p->j_dct_sum, B * p->nlev, n, H, W, A, A, p->twH, p->wdH, st));
    timer_mark(p, "dct_cols_sums", st);
  }
  NSST_CUDA(launch_dct_rows_syn(p->j_dct_syn, B, n, p->nlev, (size_t)H * p->WH, H, W, A, A, lowbase, lowstride,
                                p->dct_rs, HW, lowtab, p->twWh, p->twW, p->twDW, st));
  timer_mark(p, "dct_rows_synthesis", st);
  std::vector<const float*> p1(n);
  for (int i = 0; i < n; i++) p1[i] = p->pyr + (size_t)i * p->s_pyr + HW;
  NSST_TRY(enqueue_dct_cols_out(p, n, p1.data(), out, st));
  timer_mark(p, "dct_cols_image_out", st);
  return NSST_OK;
}

// The fused pipeline with the pyramid in the DCT-II domain (k_dct.cu): the
// pyramid's analysis merges with the level FFTs, its synthesis with the
// inverse level FFTs; the directional stage is the same.  The lowpass band
// stays in the DCT domain unless it is thresholded (lowpass_th): then it is
// transformed back, thresholded and transformed again (three passes).
nsst_status enqueue_denoise_dct(nsst_plan* p, int n, const float* const* x, float* const* out, int mode,
                                bool lowpass_th, const float* TH, cudaStream_t st, bool keep = false) {
  char* A = p->arena;
  float2* A2 = (float2*)A;
  const int B = p->B, H = p->H, W = p->W;
  const bool ana_dct = !keep && analysis_takes_dct(p, n);
  NSST_TRY(enqueue_dct_analysis(p, n, x, st, ana_dct));
  if (lowpass_th) {  // lowpass band -> threshold -> DCT2, in tmp plane 0
    NSST_TRY(enqueue_dct_lowpass_rows(p, n, st));
    NSST_CUDA(launch_dct_cols(kDctThresh, p->j_dct_lowc, B, n, H, W, A, A, p->twH, p->wdH, st, TH, p->nbands, mode));
    std::vector<float*> t0(n);
    for (int i = 0; i < n; i++) t0[i] = p->tmp + (size_t)i * p->s_tmp;
    std::vector<const float*> t0c(t0.begin(), t0.end());
    NSST_TRY(enqueue_dct_rows_io(p, n, t0c.data(), t0.data(), st));
    timer_mark(p, "dct_lowpass_threshold", st);
  }
  if (keep) {  // the thresholded bands to bandT: band keeps the pre-threshold spectra for the backward
    NSST_TRY(enqueue_band_analysis(p, n, false, st));
    timer_mark(p, "band_analysis_cols", st);
    NSST_CUDA(launch_rows(RowOp::Thresh, p->gj_rows_T, B * p->ndir_total, n, H, W, A, p->garena, p->twWh, p->twW, TH,
                          mode, st));
    timer_mark(p, "band_rows_threshold", st);
    NSST_CUDA(launch_cols(ColOp::Synthesis, p->gj_synth_T, B * p->nlev, n, H, W, (float2*)p->garena, A2, p->spec,
                          (size_t)H * p->WH, p->twH, st));
    timer_mark(p, "band_synthesis_cols", st);
  }
  bool sums_dct2 = false;
  if (!keep) NSST_TRY(enqueue_directional(p, n, mode, TH, st, &sums_dct2, ana_dct));
  return lowpass_th ? enqueue_dct_synthesis(p, n, p->tmp, p->s_tmp, p->dct_gl, out, st, sums_dct2)
                    : enqueue_dct_synthesis(p, n, p->pyr, p->s_pyr, p->dct_tl, out, st, sums_dct2);
}

// The fused batched pipeline (no host work, no allocation): capturable.
// keep: the differentiable forward writes the thresholded bands to bandT,
// leaving the pre-threshold band spectra (and the pyramid's lowpass) for
// nsst_denoise_tau_backward_saved.
nsst_status enqueue_denoise(nsst_plan* p, int n, const float* const* x, float* const* out, int mode, bool lowpass_th,
                            cudaStream_t st, bool keep = false, const float* thr = nullptr) {
  const float* TH = thr ? thr : p->th;  // [item][band] thresholds on the device
  char* A = p->arena;
  float2* A2 = (float2*)A;
  const int B = p->B, H = p->H, W = p->W;
  const size_t HW = (size_t)H * W;
  if (keep) p->saved_dct = dct_path(p, n, x, out);
  if (dct_path(p, n, x, out)) return enqueue_denoise_dct(p, n, x, out, mode, lowpass_th, TH, st, keep);
  std::vector<float*> ys(n);
  for (int i = 0; i < n; i++) ys[i] = p->pyr + i * p->s_pyr;
  NSST_TRY(run_atrousdec(p, n, x, ys.data(), nullptr, st));
  NSST_CUDA(launch_rows(RowOp::Fwd, p->j_rows_lev_fwd, B * p->nlev, n, H, W, A, A, p->twWh, p->twW, nullptr, 0, st));
  timer_mark(p, "fft_rows_fwd", st);
  NSST_CUDA(launch_cols(ColOp::Fwd, p->j_cols_lev, B * p->nlev, n, H, W, A2, A2, nullptr, 0, p->twH, st));
  timer_mark(p, "fft_cols_fwd", st);
  if (keep) {
    NSST_TRY(enqueue_band_analysis(p, n, false, st));
    timer_mark(p, "band_analysis_cols", st);
    NSST_CUDA(launch_rows(RowOp::Thresh, p->gj_rows_T, B * p->ndir_total, n, H, W, A, p->garena, p->twWh, p->twW,
                          TH, mode, st));
    timer_mark(p, "band_rows_threshold", st);
    NSST_CUDA(launch_cols(ColOp::Synthesis, p->gj_synth_T, B * p->nlev, n, H, W, (float2*)p->garena, A2, p->spec,
                          (size_t)H * p->WH, p->twH, st));
    timer_mark(p, "band_synthesis_cols", st);
  } else {
    NSST_TRY(enqueue_directional(p, n, mode, TH, st));
  }
  NSST_CUDA(launch_rows(RowOp::Inv, p->j_rows_lev_inv, B * p->nlev, n, H, W, A, A, p->twWh, p->twW, nullptr, 0, st));
  timer_mark(p, "fft_rows_inv", st);
  std::vector<const float*> yr(n), low(n, nullptr);
  for (int i = 0; i < n; i++) {
    yr[i] = p->rec + i * p->s_rec;
    low[i] = p->pyr + i * p->s_pyr;
  }
  if (lowpass_th) {
    // lowpass band: copy into rec plane 0 and threshold there (t > 0 only)
    for (int i = 0; i < n; i++) {
      NSST_CUDA(cudaMemcpyAsync(p->rec + i * p->s_rec, p->pyr + i * p->s_pyr, HW * sizeof(float),
                                cudaMemcpyDeviceToDevice, st));
      NSST_CUDA(launch_thresh_bands(p->rec + i * p->s_rec, HW, 1, TH + (size_t)i * p->nbands, mode, st));
      low[i] = p->rec + i * p->s_rec;
    }
    timer_mark(p, "lowpass_threshold", st);
  }
  return run_atrousrec(p, n, yr.data(), low.data(), out, st);
}

// Per image the largest |c| of every coefficient plane of shear_trans(x_i),
// as float bit patterns in bits[i * nbands + b] (zeroed here): the pyramid
// and the directional analysis of the fused pipeline, then band rows C2R'd
// and reduced without being stored; the lowpass plane reduced directly.  The
// plan must be locked.
nsst_status enqueue_band_maxima(nsst_plan* p, int n, const float* const* x, unsigned* bits, cudaStream_t st) {
  char* A = p->arena;
  float2* A2 = (float2*)A;
  const int B = p->B, H = p->H, W = p->W;
  const size_t HW = (size_t)H * W;
  std::vector<float*> ys(n);
  for (int i = 0; i < n; i++) ys[i] = p->pyr + i * p->s_pyr;
  NSST_CUDA(cudaMemsetAsync(bits, 0, sizeof(unsigned) * n * p->nbands, st));
  bool spectral = p->dct_on;
  for (int i = 0; i < n; i++) spectral = spectral && aligned16(x[i]);
  if (spectral) {
    // level spectra from X = DCT2(x); the spatial lowpass into pyr plane 1
    NSST_TRY(enqueue_dct_analysis(p, n, x, st));
    NSST_TRY(enqueue_dct_lowpass_rows(p, n, st));
    std::vector<const float*> t0(n);
    for (int i = 0; i < n; i++) {
      t0[i] = p->tmp + (size_t)i * p->s_tmp;
      ys[i] += HW;
    }
    NSST_TRY(enqueue_dct_cols_out(p, n, t0.data(), ys.data(), st));
  } else {
    NSST_TRY(run_atrousdec(p, n, x, ys.data(), nullptr, st));
    NSST_CUDA(launch_rows(RowOp::Fwd, p->j_rows_lev_fwd, B * p->nlev, n, H, W, A, A, p->twWh, p->twW, nullptr, 0,
                          st));
    NSST_CUDA(launch_cols(ColOp::Fwd, p->j_cols_lev, B * p->nlev, n, H, W, A2, A2, nullptr, 0, p->twH, st));
  }
  NSST_TRY(enqueue_band_analysis(p, n, false, st));
  NSST_CUDA(launch_rows_max(p->j_rows_bands, B * p->ndir_total, n, H, W, A, p->twWh, p->twW, bits, st));
  for (int i = 0; i < n; i++)
    NSST_CUDA(launch_plane_maxabs(ys[(size_t)i], HW, 1, bits + (size_t)i * p->nbands, kRedBlocks, st));
  return NSST_OK;
}

// shear_trans of one image into nbands caller planes; the plan must be locked.
nsst_status enqueue_shear_trans(nsst_plan* p, const float* x, float* coeffs, cudaStream_t st) {
  char* A = p->arena;
  float2* A2 = (float2*)A;
  float* yb = p->pyr;
  if (p->dct_on && aligned16(x)) {
    // spectral pyramid: the level spectra from X = DCT2(x); the lowpass
    // IDCT2(X .* R_low) straight to coefficient plane 0
    NSST_TRY(enqueue_dct_analysis(p, 1, &x, st));
    NSST_TRY(enqueue_dct_lowpass_rows(p, 1, st));
    const float* t0 = p->tmp;
    NSST_TRY(enqueue_dct_cols_out(p, 1, &t0, &coeffs, st));
    timer_mark(p, "dct_lowpass", st);
  } else {
    // the lowpass goes straight to coefficient plane 0
    NSST_TRY(run_atrousdec(p, 1, &x, &yb, coeffs, st));
    NSST_CUDA(launch_rows(RowOp::Fwd, p->j_rows_lev_fwd, p->nlev, 1, p->H, p->W, A, A, p->twWh, p->twW, nullptr, 0,
                          st));
    NSST_CUDA(launch_cols(ColOp::Fwd, p->j_cols_lev, p->nlev, 1, p->H, p->W, A2, A2, nullptr, 0, p->twH, st));
  }
  // the job list covers every item; n_active = 1 skips the others
  NSST_CUDA(launch_cols(ColOp::Analysis, p->j_analysis, p->B * p->ndir_total, 1, p->H, p->W, A2, A2, p->spec, 0,
                        p->twH, st));
  timer_mark(p, "band_analysis_cols", st);
  NSST_CUDA(launch_rows(RowOp::Inv, p->j_band_to_coeff, p->ndir_total, 1, p->H, p->W, A, coeffs, p->twWh, p->twW,
                        nullptr, 0, st));
  timer_mark(p, "band_rows_inv", st);
  return NSST_OK;
}

}  // namespace

extern "C" {

nsst_status nsst_atrousdec(nsst_plan* p, const float* x, float* y, void* stream) {
  if (!p || !x || !y) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  NSST_TRY(check_spectral(p, {x, y}));
  std::lock_guard<std::mutex> lk(p->mu);
  p->saved_n = 0;  // the arena no longer holds the last differentiable forward
  cudaStream_t st = (cudaStream_t)stream;
  timer_begin(p, st);
  float* yb = y;
  if (p->dct_on && aligned16(x) && aligned16(y)) {
    // spectral pyramid: X = DCT2(x); band l = IDCT2(X .* R_l) (rows into the
    // level planes, then down the columns into y plane l + 1); the lowpass
    const int L = p->nlev;
    const size_t HW = (size_t)p->H * p->W;
    std::vector<float*> p1{p->pyr + HW};
    NSST_TRY(enqueue_dct_rows_io(p, 1, &x, p1.data(), st));
    char* A = p->arena;
    NSST_CUDA(launch_dct_cols(kDct2, p->j_dct_x, p->B, 1, p->H, p->W, A, A, p->twH, p->wdH, st));
    NSST_CUDA(launch_dct_rows_ana(p->j_dct_ana, p->B * L, 1, p->H, p->W, A, A, p->dct_ra, HW, p->twWh, p->twW,
                                  p->twDW, true, st));
    NSST_TRY(enqueue_dct_lowpass_rows(p, 1, st));
    std::vector<const float*> src(L + 1);
    std::vector<float*> dst(L + 1);
    src[0] = p->tmp;
    dst[0] = y;
    for (int l = 0; l < L; l++) {
      src[l + 1] = reinterpret_cast<const float*>(p->lev + (size_t)l * p->H * p->WH);
      dst[l + 1] = y + (size_t)(l + 1) * HW;
    }
    return enqueue_dct_cols_out(p, L + 1, src.data(), dst.data(), st);
  }
  return run_atrousdec(p, 1, &x, &yb, nullptr, st);
}

nsst_status nsst_atrousrec(nsst_plan* p, const float* y, float* x, void* stream) {
  if (!p || !x || !y) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  NSST_TRY(check_spectral(p, {x, y}));
  std::lock_guard<std::mutex> lk(p->mu);
  p->saved_n = 0;  // the arena no longer holds the last differentiable forward
  cudaStream_t st = (cudaStream_t)stream;
  timer_begin(p, st);
  if (p->dct_on && aligned16(x) && aligned16(y)) {
    // spectral pyramid: the DCT-II of every band (into the level planes) and
    // of the lowpass (tmp plane 0), then IDCT2(sum_l Q_l .* Y_l + G_low .* Y_0)
    const int L = p->nlev;
    const size_t HW = (size_t)p->H * p->W, HWh = (size_t)p->H * p->WH;
    char* A = p->arena;
    std::vector<const float*> src(L + 1);
    std::vector<float*> dst(L + 1);
    src[0] = y;
    dst[0] = p->tmp;
    for (int l = 0; l < L; l++) {
      src[l + 1] = y + (size_t)(l + 1) * HW;
      dst[l + 1] = reinterpret_cast<float*>(p->lev + (size_t)l * HWh);
    }
    NSST_TRY(enqueue_dct_rows_io(p, L + 1, src.data(), dst.data(), st));
    NSST_CUDA(launch_dct_cols(kDct2, p->j_cols_lev, p->B * L, 1, p->H, p->W, A, A, p->twH, p->wdH, st));
    NSST_CUDA(launch_dct_cols(kDct2, p->j_dct_lowc, p->B, 1, p->H, p->W, A, A, p->twH, p->wdH, st));
    NSST_CUDA(launch_dct_rows_syn(p->j_dct_rec, p->B, 1, L, HWh, p->H, p->W, A, A, p->tmp, p->s_tmp, p->dct_rs, HW,
                                  p->dct_gl, p->twWh, p->twW, p->twDW, st, true));
    const float* p1 = p->pyr + HW;
    return enqueue_dct_cols_out(p, 1, &p1, &x, st);
  }
  return run_atrousrec(p, 1, &y, nullptr, &x, st);
}

nsst_status nsst_shear_trans(nsst_plan* p, const float* x, float* coeffs, void* stream) {
  if (!p || !x || !coeffs) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  NSST_TRY(check_spectral(p, {x}));
  if (!aligned16(coeffs)) return fail(NSST_ERR_INVALID_ARG, "coeffs must be 16-byte aligned");
  std::lock_guard<std::mutex> lk(p->mu);
  p->saved_n = 0;  // the arena no longer holds the last differentiable forward
  cudaStream_t st = (cudaStream_t)stream;
  timer_begin(p, st);
  return enqueue_shear_trans(p, x, coeffs, st);
}

nsst_status nsst_thresh(nsst_plan* p, float* coeffs, double sigma, const double* K, const double* scalars, int mode,
                        void* stream) {
  if (!p || !coeffs) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  if (mode != NSST_THRESH_HARD && mode != NSST_THRESH_SOFT) return fail(NSST_ERR_INVALID_ARG, "bad mode");
  std::lock_guard<std::mutex> lk(p->mu);
  cudaStream_t st = (cudaStream_t)stream;
  NSST_TRY(upload_thresholds(p, 1, &sigma, K, scalars, st, nullptr));
  NSST_CUDA(launch_thresh_bands(coeffs, (size_t)p->H * p->W, p->nbands, p->th, mode, st));
  return NSST_OK;
}

nsst_status nsst_thresh_max(nsst_plan* p, float* coeffs, double sigma, const double* K, const double* scalars,
                            int mode, double* maxabs, void* stream) {
  if (!maxabs) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  NSST_TRY(nsst_thresh(p, coeffs, sigma, K, scalars, mode, stream));
  if (!scalars && !p->has_scalars) return fail(NSST_ERR_INVALID_ARG, "no scalars");
  const double* sc = scalars ? scalars : p->scalars.data();
  std::lock_guard<std::mutex> lk(p->mu);
  cudaStream_t st = (cudaStream_t)stream;
  unsigned* bits = reinterpret_cast<unsigned*>(p->red_scratch);
  NSST_CUDA(cudaMemsetAsync(bits, 0, sizeof(unsigned) * p->nbands, st));
  NSST_CUDA(launch_plane_maxabs(coeffs, (size_t)p->H * p->W, p->nbands, bits, kRedBlocks, st));
  std::vector<unsigned> hb(p->nbands);
  NSST_CUDA(cudaMemcpyAsync(hb.data(), bits, sizeof(unsigned) * p->nbands, cudaMemcpyDeviceToHost, st));
  NSST_CUDA(cudaStreamSynchronize(st));
  // thresh.m:38-41: max over the bands of max|c_b| / E_b
  double m = 0.0;
  for (int b = 0; b < p->nbands; b++) {
    float v;
    std::memcpy(&v, &hb[b], sizeof(float));
    if (sc[b] > 0) m = std::max(m, (double)v / sc[b]);
  }
  *maxabs = m;
  return NSST_OK;
}

// re_weight_band.m:23-29 / re_weight_band_cuda.cpp:132-183: atrousdec with
// nweights - 1 levels, weight per pyramid band, atrousrec
nsst_status nsst_re_weight_band(nsst_plan* p, const float* x, const double* weights, int nweights, float* out,
                                void* stream) {
  if (!p || !x || !weights || !out) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  // re_weight_band_cuda.cpp:126-127: at least one band-pass level; the plan's
  // pyramid buffers hold up to its own level count
  if (nweights < 2 || nweights > p->nlev + 1)
    return fail(NSST_ERR_INVALID_ARG, "need 2 to nlevels + 1 weights (nweights - 1 pyramid levels)");
  PlaneWeights w{};
  for (int k = 0; k < nweights; k++) {
    if (!std::isfinite(weights[k])) return fail(NSST_ERR_INVALID_ARG, "weights must be finite");
    w.w[k] = (float)weights[k];
  }
  std::lock_guard<std::mutex> lk(p->mu);
  p->saved_n = 0;
  cudaStream_t st = (cudaStream_t)stream;
  timer_begin(p, st);
  float* y = p->pyr;  // item 0's pyramid planes: lowpass, then band-pass coarse -> fine
  NSST_TRY(run_atrousdec(p, 1, &x, &y, nullptr, st, nweights - 1));
  NSST_CUDA(launch_scale_planes(y, (size_t)p->H * p->W, nweights, w, st));
  const float* yc = y;
  return run_atrousrec(p, 1, &yc, nullptr, &out, st, nweights - 1);
}

nsst_status nsst_band_norms(nsst_plan* p, double* E) {
  if (!p || !E) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  {
    std::lock_guard<std::mutex> lk(p->mu);
    if (!p->norms.empty()) {  // deterministic: computed once per plan
      std::copy(p->norms.begin(), p->norms.end(), E);
      return NSST_OK;
    }
  }
  const size_t HW = (size_t)p->H * p->W;
  // com_norm.m:37-40: X = fftshift(real(ifft2(ones))) * sqrt(HW), an impulse
  // of height sqrt(HW) at (H/2, W/2)
  std::vector<float> x(HW, 0.0f);
  x[(size_t)(p->H / 2) * p->W + p->W / 2] = (float)std::sqrt((double)HW);
  float *dx = nullptr, *dc = nullptr;
  cudaError_t e = dev_alloc((void**)&dx, HW * sizeof(float));
  if (e != cudaSuccess) return cuda_fail(e, "norm scratch");
  e = dev_alloc((void**)&dc, HW * sizeof(float) * p->nbands);
  if (e != cudaSuccess) {
    cudaFree(dx);
    return cuda_fail(e, "norm scratch");
  }
  nsst_status s = NSST_OK;
  std::vector<double> part((size_t)p->nbands * kRedBlocks);
  e = cudaMemcpy(dx, x.data(), HW * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) s = nsst_shear_trans(p, dx, dc, nullptr);
  if (e == cudaSuccess && s == NSST_OK) {
    std::lock_guard<std::mutex> lk(p->mu);
    e = launch_plane_sumsq(dc, HW, p->nbands, p->red_scratch, kRedBlocks, nullptr);
    if (e == cudaSuccess)
      e = cudaMemcpy(part.data(), p->red_scratch, part.size() * sizeof(double), cudaMemcpyDeviceToHost);
  }
  cudaFree(dx);
  cudaFree(dc);
  if (e != cudaSuccess) return cuda_fail(e, "band norms");
  if (s != NSST_OK) return s;
  // com_norm.m:45-51: E = sqrt(sum |C_b|^2 / (H W))
  for (int b = 0; b < p->nbands; b++) {
    double t = 0.0;
    for (int k = 0; k < kRedBlocks; k++) t += part[(size_t)b * kRedBlocks + k];
    E[b] = std::sqrt(t / (double)HW);
  }
  std::lock_guard<std::mutex> lk(p->mu);
  p->norms.assign(E, E + p->nbands);
  return NSST_OK;
}

nsst_status nsst_inverse_shear(nsst_plan* p, const float* coeffs, float* x, void* stream) {
  if (!p || !x || !coeffs) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  NSST_TRY(check_spectral(p, {x}));
  if (!aligned16(coeffs)) return fail(NSST_ERR_INVALID_ARG, "coeffs must be 16-byte aligned");
  std::lock_guard<std::mutex> lk(p->mu);
  p->saved_n = 0;  // the arena no longer holds the last differentiable forward
  cudaStream_t st = (cudaStream_t)stream;
  timer_begin(p, st);
  char* A = p->arena;
  float2* A2 = (float2*)A;
  NSST_CUDA(launch_rows(RowOp::Fwd, p->j_coeff_fwd, p->ndir_total, 1, p->H, p->W, coeffs, A, p->twWh, p->twW,
                        nullptr, 0, st));
  timer_mark(p, "band_rows_fwd", st);
  NSST_CUDA(launch_cols(ColOp::Synthesis, p->j_synthesis, p->B * p->nlev, 1, p->H, p->W, A2, A2, p->spec,
                        (size_t)p->H * p->WH, p->twH, st));
  timer_mark(p, "band_synthesis_cols", st);
  if (p->dct_on && aligned16(x)) {
    // spectral pyramid: the lowpass coefficients DCT2'd into tmp plane 0,
    // then the band sums and that plane through the synthesis back end
    float* t0 = p->tmp;
    NSST_TRY(enqueue_dct_rows_io(p, 1, &coeffs, &t0, st));
    NSST_CUDA(launch_dct_cols(kDct2, p->j_dct_lowc, p->B, 1, p->H, p->W, A, A, p->twH, p->wdH, st));
    timer_mark(p, "dct_lowpass", st);
    return enqueue_dct_synthesis(p, 1, p->tmp, p->s_tmp, p->dct_gl, &x, st);
  }
  NSST_CUDA(launch_rows(RowOp::Inv, p->j_rows_lev_inv, p->nlev, 1, p->H, p->W, A, A, p->twWh, p->twW, nullptr, 0,
                        st));
  timer_mark(p, "fft_rows_inv", st);
  const float* yr = p->rec;
  return run_atrousrec(p, 1, &yr, &coeffs, &x, st);
}

nsst_status nsst_denoise_batch(nsst_plan* p, const float* const* x, float* const* out, int n, const double* sigma,
                               const double* K, const double* scalars, int mode, void* stream) {
  if (!p || !x || !out || !sigma) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  if (n < 1 || n > p->B) return fail(NSST_ERR_INVALID_ARG, "item count outside [1, batch capacity]");
  if (mode != NSST_THRESH_HARD && mode != NSST_THRESH_SOFT) return fail(NSST_ERR_INVALID_ARG, "bad mode");
  for (int i = 0; i < n; i++)
    if (!x[i] || !out[i]) return fail(NSST_ERR_INVALID_ARG, "NULL image pointer");
  NSST_TRY(check_spectral_n(p, n, x, out));
  std::lock_guard<std::mutex> lk(p->mu);
  p->saved_n = 0;  // the arena no longer holds the last differentiable forward
  cudaStream_t st = (cudaStream_t)stream;
  float lmax = 0.f;
  NSST_TRY(upload_thresholds(p, n, sigma, K, scalars, st, &lmax));
  const bool lowpass_th = lmax > 0.f;
  if (!p->use_graphs || p->timing) {
    timer_begin(p, st);
    return enqueue_denoise(p, n, x, out, mode, lowpass_th, st);
  }
  // graph replay: the launch sequence depends only on (n, pointers, mode, lowpass_th)
  std::vector<const void*> key;
  for (int i = 0; i < n; i++) {
    key.push_back(x[i]);
    key.push_back(out[i]);
  }
  const int kmode = mode * 2 + (lowpass_th ? 1 : 0);
  nsst_plan::GraphEntry* hit = nullptr;
  for (auto& g : p->graphs)
    if (g.exec && g.n == n && g.mode == kmode && g.key == key) hit = &g;
  if (!hit) {
    hit = &p->graphs[0];
    for (auto& g : p->graphs)
      if (!g.exec || g.used < hit->used) hit = &g;
    if (hit->exec) {
      cudaGraphExecDestroy(hit->exec);
      hit->exec = nullptr;
    }
    NSST_CUDA(cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal));
    nsst_status s = enqueue_denoise(p, n, x, out, mode, lowpass_th, p->cap_stream);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(p->cap_stream, &g);
    if (s != NSST_OK) {
      if (g) cudaGraphDestroy(g);
      return s;
    }
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
    ce = cudaGraphInstantiate(&hit->exec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
      hit->exec = nullptr;
      return cuda_fail(ce, "cudaGraphInstantiate");
    }
    hit->key = key;
    hit->n = n;
    hit->mode = kmode;
  }
  hit->used = ++p->graph_clock;
  count_launch(0);
  NSST_CUDA(cudaGraphLaunch(hit->exec, st));
  return NSST_OK;
}

}  // extern "C"

namespace {

// The directional-stage candidates of a plan: the split kernels with each
// analysis variant and row tile, and the fused cluster kernel where the plan
// has it.
std::vector<std::pair<DirChoice, std::string>> dir_candidates(const nsst_plan* p) {
  std::vector<std::pair<DirChoice, std::string>> c;
  const int rs = row_tile(p->WH);
  // row pass: RowCfg's tile with one complex value per thread, or 1 or 2
  // tiles of split-complex row pairs; columns: one value or column pairs
  // (the pairs' analysis streams all bands of a level per CTA)
  const int rows[3][2] = {{1, 0}, {1, 1}, {2, 1}};
  for (bool tma : {false, true}) {
    if (tma && !p->cols_tma_ok) continue;
    for (int ana : {1, 2})
      for (bool cp : {false, true})
        for (const auto& r : rows) {
          DirChoice d;
          d.ana = ana;
          d.row_tile = r[0];
          d.packed = r[1] != 0;
          d.cols_packed = cp;
          d.cols_tma = tma;
          if (p->H % (rs * r[0]) != 0) continue;
          const std::string cols = std::string(cp ? "-pairs" : "") + (tma ? "-tma" : "");
          c.push_back({d, std::string("split/") + (ana == 1 ? "level" + cols : std::string("band")) + "/rows" +
                              std::to_string(rs * r[0]) + (d.packed ? "-pairs" : "") + "/synthesis" + cols});
        }
  }
  // the TMA synthesis with the band sum in registers
  if (p->cols_tma_ok)
    for (int ana : {1, 2})
      for (const auto& r : rows) {
        DirChoice d;
        d.ana = ana;
        d.row_tile = r[0];
        d.packed = r[1] != 0;
        d.cols_tma = true;
        d.syn_regs = true;
        if (p->H % (rs * r[0]) != 0) continue;
        c.push_back({d, std::string("split/") + (ana == 1 ? "level-tma" : "band") + "/rows" +
                            std::to_string(rs * r[0]) + (d.packed ? "-pairs" : "") + "/synthesis-regs"});
      }
  if (p->fused_ok) {
    DirChoice d;
    d.fused = true;
    c.push_back({d, "fused/cluster" + std::to_string(dir_fused_cluster(p->H, p->WH))});
  }
  return c;
}

// Direct (spatial) directional convolution instead of the FFT path: the
// effective filter of band k is e_k = ifft2(W_k / d), d = sqrt(sum_j |W_j|^2)
// (nsst_dec2.m:47-57), which the normalisation spreads over the whole image.
// For each level the smallest square window around the shearing filter's own
// support [0, dsize)^2 (circularly, with the same margin m on every side) that
// keeps every band's truncation error ||e_k - window(e_k)|| / ||e_k|| <= tol;
// 0 if no window smaller than the image does.  err: the worst band's error
// at the largest window tried.
void direct_support(int nlev, const int* dsize, const int* ndir, const std::vector<double>* shear_w, int H, int W,
                    double tol, int* support, double* err) {
  const int WC = W / 2 + 1;
  for (int l = 0; l < nlev; l++) {
    const int nd = ndir[l], ds = dsize[l];
    std::vector<cd> S;
    support[l] = 0;
    err[l] = 1.0;
    if (!level_spectra(shear_w[l], nd, ds, H, W, &S, host_threads())) continue;
    const int mmax = (std::min(H, W) - ds) / 2 - 1;
    std::vector<int> need(nd, -1);
    std::vector<double> worst(nd, 0.0);
    auto work = [&](int k) {
      // full Hermitian spectrum -> 2-D inverse FFT (rows, then columns) -> e_k
      std::vector<cd> F((size_t)H * W);
      const cd* s = S.data() + (size_t)k * H * WC;
      for (int u = 0; u < H; u++)
        for (int v = 0; v < W; v++)
          F[(size_t)u * W + v] = v < WC ? s[(size_t)u * WC + v] : std::conj(s[(size_t)((H - u) % H) * WC + (W - v)]);
      for (int u = 0; u < H; u++) fft_inplace(F.data() + (size_t)u * W, W, +1);
      std::vector<cd> col(H);
      for (int v = 0; v < W; v++) {
        for (int u = 0; u < H; u++) col[u] = F[(size_t)u * W + v];
        fft_inplace(col.data(), H, +1);
        for (int u = 0; u < H; u++) F[(size_t)u * W + v] = col[u];
      }
      // energy per circular "ring" distance from the filter's support
      double total = 0.0;
      std::vector<double> ring(std::max(H, W), 0.0);
      for (int i = 0; i < H; i++)
        for (int j = 0; j < W; j++) {
          const double e = std::norm(F[(size_t)i * W + j].real());
          total += e;
          auto dist = [&](int a, int n) {  // circular distance of a from [0, ds)
            if (a < ds) return 0;
            return std::min(a - ds + 1, n - a);
          };
          ring[std::max(dist(i, H), dist(j, W))] += e;
        }
      double inside = 0.0;
      for (int m = 0; m <= mmax; m++) {
        inside += ring[m];
        const double rel = std::sqrt(std::max(total - inside, 0.0) / total);
        if (m == mmax) worst[k] = rel;
        if (rel <= tol) {
          need[k] = m;
          worst[k] = rel;
          break;
        }
      }
    };
    std::vector<std::thread> th;
    const int nt = std::min(host_threads(), nd);
    for (int t = 0; t < nt; t++)
      th.emplace_back([&, t]() {
        for (int k = t; k < nd; k += nt) work(k);
      });
    for (auto& t : th) t.join();
    int m = 0;
    double w = 0.0;
    bool ok = true;
    for (int k = 0; k < nd; k++) {
      if (need[k] < 0) ok = false;
      m = std::max(m, need[k]);
      w = std::max(w, worst[k]);
    }
    support[l] = ok ? ds + 2 * m : 0;
    err[l] = w;
  }
}

}  // namespace

extern "C" {

nsst_status nsst_plan_select_directional(nsst_plan* p, int n, int index) {
  if (!p) return fail(NSST_ERR_INVALID_ARG, "NULL plan");
  if (n < 1 || n > p->B) return fail(NSST_ERR_INVALID_ARG, "item count outside [1, batch capacity]");
  std::lock_guard<std::mutex> lk(p->mu);
  const auto cands = dir_candidates(p);
  const int b = tune_bucket(n);
  if (index < 0) {
    p->tuned[b] = false;
  } else {
    if (index >= (int)cands.size()) return fail(NSST_ERR_INVALID_ARG, "candidate index out of range");
    p->tuned[b] = true;
    p->tuned_choice[b] = cands[index].first;
  }
  for (auto& g : p->graphs)
    if (g.exec) {
      cudaGraphExecDestroy(g.exec);
      g.exec = nullptr;
      g.key.clear();
    }
  return NSST_OK;
}

int nsst_plan_directional_candidates(const nsst_plan* p, char* names, size_t len) {
  if (!p) return -1;
  const auto cands = dir_candidates(p);
  std::string all;
  for (const auto& c : cands) all += c.second + "\n";
  if (names && len) {
    const size_t m = std::min(all.size(), len - 1);
    std::memcpy(names, all.data(), m);
    names[m] = 0;
  }
  return (int)cands.size();
}

nsst_status nsst_direct_support(const nsst_config* cfg, int H, int W, double tol, int* support, double* err) {
  if (!cfg || !support || !err) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  NSST_TRY(validate_config(cfg, H, W));
  if (!(tol > 0.0)) return fail(NSST_ERR_INVALID_ARG, "tol must be positive");
  std::vector<std::vector<double>> w(cfg->nlevels);
  std::vector<int> nd(cfg->nlevels);
  for (int l = 0; l < cfg->nlevels; l++) {
    w[l] = shearing_filters_myer(cfg->dsize[l], cfg->dcomp[l]);
    nd[l] = 1 << cfg->dcomp[l];
  }
  direct_support(cfg->nlevels, cfg->dsize, nd.data(), w.data(), H, W, tol, support, err);
  return NSST_OK;
}

nsst_status nsst_plan_autotune(nsst_plan* p, int n, nsst_tune_result* res) {
  if (!p) return fail(NSST_ERR_INVALID_ARG, "NULL plan");
  if (n < 1 || n > p->B) return fail(NSST_ERR_INVALID_ARG, "item count outside [1, batch capacity]");
  std::lock_guard<std::mutex> lk(p->mu);
  const size_t HW = (size_t)p->H * p->W;
  float* buf = nullptr;
  cudaError_t ce = dev_alloc((void**)&buf, sizeof(float) * HW * 2 * (size_t)n);
  if (ce != cudaSuccess) return cuda_fail(ce, "autotune image buffers");
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const bool was_timing = p->timing;
  auto cleanup = [&]() {
    p->forcing = false;
    p->timing = was_timing;
    if (st) cudaStreamSynchronize(st);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cudaFree(buf);
  };
  auto bail = [&](nsst_status s) {
    cleanup();
    return s;
  };
  // a noisy test image (N(128, 40^2)), the same for every item
  {
    std::vector<float> h(HW);
    std::mt19937_64 gen(20261204);
    std::normal_distribution<double> nd(128.0, 40.0);
    for (auto& v : h) v = (float)nd(gen);
    for (int i = 0; i < n; i++) {
      ce = cudaMemcpy(buf + (size_t)i * HW, h.data(), HW * sizeof(float), cudaMemcpyHostToDevice);
      if (ce != cudaSuccess) return bail(cuda_fail(ce, "autotune input upload"));
    }
  }
  ce = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) return bail(cuda_fail(ce, "autotune stream / events"));
  std::vector<const float*> xs(n);
  std::vector<float*> outs(n);
  for (int i = 0; i < n; i++) {
    xs[i] = buf + (size_t)i * HW;
    outs[i] = buf + (size_t)(n + i) * HW;
  }
  std::vector<double> sig(n, 20.0), K(p->nlev + 1, 3.0);
  K[0] = 0.0;
  K[p->nlev] = 4.0;
  std::vector<double> sc = p->has_scalars ? p->scalars : std::vector<double>(p->nbands, 1.0);
  p->timing = false;
  p->forcing = false;
  float lmax = 0.f;
  nsst_status s = upload_thresholds(p, n, sig.data(), K.data(), sc.data(), st, &lmax);
  // one full pass leaves the level spectra that every candidate reads
  if (s == NSST_OK) s = enqueue_denoise(p, n, xs.data(), outs.data(), NSST_THRESH_HARD, false, st);
  if (s != NSST_OK) return bail(s);
  auto cands = dir_candidates(p);
  std::vector<float> med(cands.size());
  for (size_t c = 0; c < cands.size(); c++) {
    p->forcing = true;
    p->forced = cands[c].first;
    std::vector<float> t;
    for (int r = 0; r < 9; r++) {
      ce = cudaEventRecord(e0, st);
      if (ce != cudaSuccess) return bail(cuda_fail(ce, "cudaEventRecord"));
      s = enqueue_directional(p, n, NSST_THRESH_HARD, p->th, st);
      if (s != NSST_OK) return bail(s);
      ce = cudaEventRecord(e1, st);
      if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
      if (ce != cudaSuccess) return bail(cuda_fail(ce, "autotune timing"));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (r >= 2) t.push_back(ms);  // two warm-up passes
    }
    std::sort(t.begin(), t.end());
    med[c] = t[t.size() / 2];
  }
  p->forcing = false;
  {
    int host_err[4] = {};
    ce = cudaMemcpy(host_err, p->dev_err, sizeof(host_err), cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return bail(cuda_fail(ce, "read the device error word"));
    if (host_err[0] != 0) {
      cudaMemset(p->dev_err, 0, sizeof(host_err));
      return bail(fail(NSST_ERR_TIMEOUT, "a bounded device-side wait ran out while tuning"));
    }
  }
  const size_t best = (size_t)(std::min_element(med.begin(), med.end()) - med.begin());
  const int b = tune_bucket(n);
  p->tuned[b] = true;
  p->tuned_choice[b] = cands[best].first;
  for (auto& g : p->graphs)  // captured graphs hold the previous choice
    if (g.exec) {
      cudaGraphExecDestroy(g.exec);
      g.exec = nullptr;
      g.key.clear();
    }
  if (res) {
    std::memset(res, 0, sizeof(*res));
    res->n = n;
    res->ncand = (int)std::min<size_t>(cands.size(), NSST_TUNE_MAX_CANDIDATES);
    res->chosen = (int)best;
    for (int c = 0; c < res->ncand; c++) {
      std::snprintf(res->name[c], sizeof(res->name[c]), "%s", cands[c].second.c_str());
      res->ms[c] = med[c];
    }
    direct_support(p->nlev, p->cfg.dsize, p->ndir.data(), p->shear_w.data(), p->H, p->W, 1e-5, res->direct_support,
                   res->direct_err);
    // A direct convolution with the truncated filters costs support^2 FMAs
    // per pixel and band for the analysis and as many for the synthesis; its
    // lower bound is that work at the FP32 FMA peak (SMs x 128 lanes x clock).
    // It is chosen only if every level has a support (the truncation is
    // proven within 1e-5) and the bound beats the fastest measured candidate.
    int khz = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev);
    const double fma_per_s = (double)p->sm_count * 128.0 * (khz > 0 ? khz * 1e3 : 2.07e9);
    double fmas = 0.0;
    bool all = true;
    for (int l = 0; l < p->nlev; l++) {
      const double s2 = (double)res->direct_support[l] * res->direct_support[l];
      if (res->direct_support[l] == 0) all = false;
      fmas += 2.0 * s2 * (double)HW * p->ndir[l] * n;
    }
    res->direct_bound_ms = all ? (float)(fmas / fma_per_s * 1e3) : -1.0f;
    res->direct_wins = all && res->direct_bound_ms < med[best] ? 1 : 0;
  }
  cleanup();
  return NSST_OK;
}

nsst_status nsst_denoise(nsst_plan* p, const float* x, float* out, double sigma, const double* K,
                         const double* scalars, int mode, void* stream) {
  return nsst_denoise_batch(p, &x, &out, 1, &sigma, K, scalars, mode, stream);
}

nsst_status nsst_timers_enable(nsst_plan* p, int enable) {
  if (!p) return fail(NSST_ERR_INVALID_ARG, "NULL plan");
  std::lock_guard<std::mutex> lk(p->mu);
  if (enable && !p->ev[0]) {
    for (cudaEvent_t& e : p->ev) {
      cudaError_t ce = cudaEventCreate(&e);
      if (ce != cudaSuccess) return cuda_fail(ce, "cudaEventCreate");
    }
  }
  p->timing = enable != 0;
  p->nstage = 0;
  return NSST_OK;
}

int nsst_timers_read(nsst_plan* p, char* names, size_t names_len, float* ms, int max_stages) {
  if (!p || !p->timing || p->nstage == 0) return 0;
  std::lock_guard<std::mutex> lk(p->mu);
  if (cudaEventSynchronize(p->ev[p->nstage]) != cudaSuccess) return -1;
  std::string all;
  int n = std::min(p->nstage, max_stages);
  for (int i = 0; i < n; i++) {
    float t = 0.f;
    cudaEventElapsedTime(&t, p->ev[i], p->ev[i + 1]);
    if (ms) ms[i] = t;
    all += p->stage_name[i];
    all += '\n';
  }
  if (names && names_len) {
    size_t m = std::min(all.size(), names_len - 1);
    std::memcpy(names, all.data(), m);
    names[m] = 0;
  }
  return n;
}

uint64_t nsst_launch_count(void) { return g_launches.load(); }

nsst_status nsst_compute_scalars(nsst_plan* p, uint64_t seed, double* out) {
  if (!p) return fail(NSST_ERR_INVALID_ARG, "NULL plan");
  const size_t HW = (size_t)p->H * p->W;
  // seeded N(0,1) image in FP64 (Box-Muller over a 64-bit Mersenne twister)
  std::mt19937_64 gen(seed);
  std::vector<float> noise(HW);
  for (size_t i = 0; i < HW; i += 2) {
    double u1 = ((gen() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    double u2 = ((gen() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    double r = std::sqrt(-2.0 * std::log(u1));
    noise[i] = (float)(r * std::cos(2 * M_PI * u2));
    if (i + 1 < HW) noise[i + 1] = (float)(r * std::sin(2 * M_PI * u2));
  }
  float *dx = nullptr, *dc = nullptr;
  cudaError_t e = dev_alloc((void**)&dx, HW * sizeof(float));
  if (e != cudaSuccess) return cuda_fail(e, "scalar scratch");
  e = dev_alloc((void**)&dc, HW * sizeof(float) * p->nbands);
  if (e != cudaSuccess) {
    cudaFree(dx);
    return cuda_fail(e, "scalar scratch");
  }
  nsst_status s = NSST_OK;
  std::vector<float> coeffs(HW * p->nbands);
  e = cudaMemcpy(dx, noise.data(), HW * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    s = nsst_shear_trans(p, dx, dc, nullptr);
    if (s == NSST_OK) e = cudaMemcpy(coeffs.data(), dc, coeffs.size() * sizeof(float), cudaMemcpyDeviceToHost);
  }
  cudaFree(dx);
  cudaFree(dc);
  if (e != cudaSuccess) return cuda_fail(e, "compute scalars");
  if (s != NSST_OK) return s;
  // MAD / 0.6745 per band (nsst_scalars.m:36,43), FP64 on the host
  std::vector<double> sc(p->nbands);
  std::vector<double> v(HW);
  auto median = [](std::vector<double>& a) {
    size_t n = a.size(), h = n / 2;
    std::nth_element(a.begin(), a.begin() + h, a.end());
    double hi = a[h];
    if (n % 2) return hi;
    double lo = *std::max_element(a.begin(), a.begin() + h);
    return 0.5 * (lo + hi);
  };
  for (int b = 0; b < p->nbands; b++) {
    for (size_t i = 0; i < HW; i++) v[i] = coeffs[(size_t)b * HW + i];
    double m = median(v);
    for (size_t i = 0; i < HW; i++) v[i] = std::fabs(v[i] - m);
    sc[b] = median(v) / 0.6745;
  }
  p->scalars = sc;
  p->has_scalars = true;
  if (out) std::copy(sc.begin(), sc.end(), out);
  return NSST_OK;
}

}  // extern "C"


// ============================================================ adjoint / gradients
namespace {

// zext slot k of item i
float* zslot(nsst_plan* p, int item, int k) { return p->zext + item * p->s_zext + (size_t)k * p->hwext; }

// g_out = K^T g_in for one dilated filtering step (filter F, dilation M):
// full zero-extended correlation with the unflipped filter, then fold.
nsst_status adjoint_step(nsst_plan* p, int n, const float* const* gin, const std::vector<float>& h, int F, int M,
                         float* const* gout, int slot, cudaStream_t st) {
  const int H = p->H, W = p->W, E = M * (F - 1) / 2;
  const int Ho = H + 2 * E, Wo = W + 2 * E;
  for (int c0 = 0; c0 < n; c0 += kMaxAtrousJobs) {
    const int cn = std::min(kMaxAtrousJobs, n - c0);
    AtrousJobs jz{};
    FoldJobs jf{};
    for (int t = 0; t < cn; t++) {
      jz.j[t] = AtrousJob{gin[c0 + t], nullptr, zslot(p, c0 + t, slot), H, W, Ho, Wo};
      jf.j[t] = FoldJob{zslot(p, c0 + t, slot), nullptr, gout[c0 + t]};
    }
    NSST_CUDA(launch_atrous_full(jz, cn, Ho, Wo, M, F, h.data(), st));
    NSST_CUDA(launch_fold(jf, cn, H, W, E, 0, false, st));
  }
  return NSST_OK;
}

// transpose of atrousrec (atrousrec.m:18-41): g (H x W) -> gyp planes (nlev+1)
nsst_status run_atrousrec_adjoint(nsst_plan* p, int n, const float* const* gout, float* const* gyp_base,
                                  cudaStream_t st) {
  const int L = p->nlev;
  const size_t HW = (size_t)p->H * p->W;
  const std::vector<float>& g0 = p->h32[2];
  const std::vector<float>& g1 = p->h32[3];
  std::vector<const float*> cur(gout, gout + n);
  std::vector<float*> dst_hi(n), dst_lo(n);
  for (int i = 0; i < L; i++) {  // i = 0 is the undilated last synthesis level
    const int M = 1 << i;
    for (int t = 0; t < n; t++) {
      dst_hi[t] = gyp_base[t] + (size_t)(L - i) * HW;
      dst_lo[t] = (i == L - 1) ? gyp_base[t] : p->gtmp + t * 2 * HW + (size_t)(i & 1) * HW;
    }
    NSST_TRY(adjoint_step(p, n, cur.data(), g1, p->pf.F[3], M, dst_hi.data(), 1, st));
    NSST_TRY(adjoint_step(p, n, cur.data(), g0, p->pf.F[2], M, dst_lo.data(), 0, st));
    for (int t = 0; t < n; t++) cur[t] = dst_lo[t];
  }
  timer_mark(p, "adjoint_atrous_rec", st);
  return NSST_OK;
}

// transpose of atrousdec (atrousdec.m:19-51): gy planes -> gx
nsst_status run_atrousdec_adjoint(nsst_plan* p, int n, const float* const* gy_base, float* const* gx,
                                  cudaStream_t st) {
  const int H = p->H, W = p->W, L = p->nlev;
  const size_t HW = (size_t)H * W;
  const std::vector<float>& h0 = p->h32[0];
  const std::vector<float>& h1 = p->h32[1];
  std::vector<const float*> glo(n);
  for (int t = 0; t < n; t++) glo[t] = gy_base[t];  // plane 0: gradient of the final lowpass
  for (int i = L - 1; i >= 0; i--) {
    const int M = 1 << i;
    const int E0 = M * (p->pf.F[0] - 1) / 2, E1 = M * (p->pf.F[1] - 1) / 2;
    for (int c0 = 0; c0 < n; c0 += kMaxAtrousJobs) {
      const int cn = std::min(kMaxAtrousJobs, n - c0);
      AtrousJobs ja{}, jb{};
      FoldJobs jf{};
      for (int t = 0; t < cn; t++) {
        const int it = c0 + t;
        float* out = (i == 0) ? gx[it] : p->gtmp + it * 2 * HW + (size_t)(i & 1) * HW;
        ja.j[t] = AtrousJob{glo[it], nullptr, zslot(p, it, 0), H, W, H + 2 * E0, W + 2 * E0};
        jb.j[t] = AtrousJob{gy_base[it] + (size_t)(L - i) * HW, nullptr, zslot(p, it, 1), H, W, H + 2 * E1,
                            W + 2 * E1};
        jf.j[t] = FoldJob{zslot(p, it, 0), zslot(p, it, 1), out};
      }
      NSST_CUDA(launch_atrous_full(ja, cn, H + 2 * E0, W + 2 * E0, M, p->pf.F[0], h0.data(), st));
      NSST_CUDA(launch_atrous_full(jb, cn, H + 2 * E1, W + 2 * E1, M, p->pf.F[1], h1.data(), st));
      NSST_CUDA(launch_fold(jf, cn, H, W, E0, E1, false, st));
    }
    for (int t = 0; t < n; t++) glo[t] = (i == 0) ? gx[t] : p->gtmp + t * 2 * HW + (size_t)(i & 1) * HW;
  }
  timer_mark(p, "adjoint_atrous_dec", st);
  return NSST_OK;
}

nsst_status need_grad(nsst_plan* p) {
  if (!p->garena) return fail(NSST_ERR_INVALID_ARG, "gradient workspace not enabled (nsst_plan_enable_grad)");
  return NSST_OK;
}

}  // namespace

extern "C" {

nsst_status nsst_plan_enable_grad(nsst_plan* p) {
  if (!p) return fail(NSST_ERR_INVALID_ARG, "NULL plan");
  std::lock_guard<std::mutex> lk(p->mu);
  if (p->garena) return NSST_OK;
  const int H = p->H, W = p->W, B = p->B;
  const size_t HW = (size_t)H * W, HWh = (size_t)H * p->WH, NB = (size_t)B;
  const int Mmax = 1 << (p->nlev - 1);
  const int Fmax = *std::max_element(p->pf.F, p->pf.F + 4);
  const int Emax = Mmax * (Fmax - 1) / 2;
  p->hwext = (size_t)(H + 2 * Emax) * (W + 2 * Emax);
  p->s_zext = 2 * p->hwext;
  p->ntiles = H / row_tile(p->WH);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t at = off;
    off = align_up(off + bytes, 256);
    return at;
  };
  size_t o_gyp = take(sizeof(float) * NB * (p->nlev + 1) * HW), o_gy = take(sizeof(float) * NB * (p->nlev + 1) * HW);
  size_t o_gtmp = take(sizeof(float) * NB * 2 * HW), o_z = take(sizeof(float) * NB * p->s_zext);
  size_t o_lev2 = take(sizeof(float2) * NB * p->nlev * HWh), o_band2 = take(sizeof(float2) * NB * p->ndir_total * HWh);
  size_t o_sum2 = take(sizeof(float2) * NB * p->nlev * HWh);
  size_t o_part = take(sizeof(float) * p->nbands * NB * p->ntiles);
  const size_t nL = NB * p->nlev, nD = NB * p->ndir_total;
  size_t o_j1 = take(sizeof(RowJob) * nL), o_j2 = take(sizeof(ColJob) * nL), o_j3 = take(sizeof(ColJob) * nD);
  size_t o_j4 = take(sizeof(RowJob) * nD), o_j5 = take(sizeof(ColJob) * nL), o_j6 = take(sizeof(RowJob) * nL);
  size_t o_j7 = take(sizeof(RowJob) * p->ndir_total), o_j8 = take(sizeof(RowJob) * p->ndir_total);
  size_t o_bandT = take(sizeof(float2) * NB * p->ndir_total * HWh);
  size_t o_jT = take(sizeof(RowJob) * nD), o_jS = take(sizeof(ColJob) * nL);
  size_t o_jA = take(sizeof(ColJob) * nL);
  size_t o_gd1 = 0, o_gd2 = 0, o_gd3 = 0, o_gd4 = 0, o_gd5 = 0, o_gd6 = 0;
  if (p->dct_ok) {
    o_gd1 = take(sizeof(ColJob) * NB), o_gd2 = take(sizeof(RowJob) * nL), o_gd3 = take(sizeof(RowJob) * NB);
    o_gd4 = take(sizeof(ColJob) * NB), o_gd5 = take(sizeof(ColJob) * nL), o_gd6 = take(sizeof(RowJob) * NB);
  }
  cudaError_t ce = dev_alloc((void**)&p->garena, off);
  if (ce != cudaSuccess) {
    p->garena = nullptr;
    return cuda_fail(ce, "gradient workspace allocation");
  }
  p->garena_bytes = off;
  char* G = p->garena;
  p->gyp = (float*)(G + o_gyp);
  p->gy = (float*)(G + o_gy);
  p->gtmp = (float*)(G + o_gtmp);
  p->zext = (float*)(G + o_z);
  p->lev2 = (float2*)(G + o_lev2);
  p->band2 = (float2*)(G + o_band2);
  p->sum2 = (float2*)(G + o_sum2);
  p->partials = (float*)(G + o_part);
  p->gj_rows_lev_fwd = (RowJob*)(G + o_j1);
  p->gj_cols_lev = (ColJob*)(G + o_j2);
  p->gj_analysis = (ColJob*)(G + o_j3);
  p->gj_rows_backward = (RowJob*)(G + o_j4);
  p->gj_synthesis = (ColJob*)(G + o_j5);
  p->gj_rows_lev_inv = (RowJob*)(G + o_j6);
  p->gj_coeff_fwd = (RowJob*)(G + o_j7);
  p->gj_band_to_coeff = (RowJob*)(G + o_j8);
  p->bandT = (float2*)(G + o_bandT);
  p->gj_rows_T = (RowJob*)(G + o_jT);
  p->gj_synth_T = (ColJob*)(G + o_jS);
  p->gj_analysis_lev = (ColJob*)(G + o_jA);
  auto g2 = [&](const void* ptr) { return (size_t)((const char*)ptr - G) / sizeof(float2); };
  auto a2 = [&](const void* ptr) { return (size_t)((const char*)ptr - p->arena) / sizeof(float2); };
  std::vector<RowJob> j1, j4, j6, j7, j8;
  std::vector<ColJob> j2, j3, j5;
  for (int i = 0; i < B; i++) {
    const size_t gyp = g2(p->gyp + i * (p->nlev + 1) * HW), gy = g2(p->gy + i * (p->nlev + 1) * HW);
    const size_t lev = g2(p->lev2 + i * p->s_lev), sum = g2(p->sum2 + i * p->s_sum);
    for (int l = 0; l < p->nlev; l++) {
      j1.push_back(RowJob{gyp + (size_t)(l + 1) * HWh, lev + (size_t)l * HWh, 0, i});
      j2.push_back(ColJob{lev + (size_t)l * HWh, lev + (size_t)l * HWh, 0, 0, 0, i});
      j6.push_back(RowJob{sum + (size_t)l * HWh, gy + (size_t)(l + 1) * HWh, 0, i});
    }
  }
  for (int b = 0; b < p->ndir_total; b++) {
    const int l = p->band_level[1 + b] - 1;
    for (int i = 0; i < B; i++) {
      const size_t lev = g2(p->lev2 + i * p->s_lev), band2 = g2(p->band2 + i * p->s_band);
      const size_t band = a2(p->band + i * p->s_band);
      j3.push_back(ColJob{lev + (size_t)l * HWh, band2 + (size_t)b * HWh, (size_t)b * HWh, p->m0_off + (size_t)b * H,
                          1, i});
      j4.push_back(RowJob{band + (size_t)b * HWh, band2 + (size_t)b * HWh, 1 + b, i});
    }
  }
  std::vector<ColJob> jA;
  for (int l = 0; l < p->nlev; l++)
    for (int i = 0; i < B; i++) {
      const size_t band2 = g2(p->band2 + i * p->s_band), sum = g2(p->sum2 + i * p->s_sum);
      const size_t lev = g2(p->lev2 + i * p->s_lev);
      j5.push_back(ColJob{band2 + (size_t)p->first_band[l] * HWh, sum + (size_t)l * HWh,
                          (size_t)p->first_band[l] * HWh, p->m0_off + (size_t)p->first_band[l] * H, p->ndir[l], i});
      jA.push_back(ColJob{lev + (size_t)l * HWh, band2 + (size_t)p->first_band[l] * HWh,
                          (size_t)p->first_band[l] * HWh, p->m0_off + (size_t)p->first_band[l] * H, p->ndir[l], i});
    }
  for (int b = 0; b < p->ndir_total; b++) {
    const size_t band20 = g2(p->band2);
    j7.push_back(RowJob{(size_t)(1 + b) * HWh, band20 + (size_t)b * HWh, 1 + b, 0});
    j8.push_back(RowJob{band20 + (size_t)b * HWh, (size_t)(1 + b) * HWh, 1 + b, 0});
  }
  // forward jobs of the differentiable path: the forward's own job order,
  // threshold output to bandT, synthesis reading bandT
  std::vector<RowJob> jT(nD);
  std::vector<ColJob> jS(nL);
  {
    std::vector<RowJob> fr(nD);
    std::vector<ColJob> fs(nL);
    ce = cudaMemcpy(fr.data(), p->j_rows_bands, nD * sizeof(RowJob), cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaMemcpy(fs.data(), p->j_synthesis, nL * sizeof(ColJob), cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return cuda_fail(ce, "read forward job lists");
    const size_t bandA = a2(p->band), bandT = g2(p->bandT);
    for (size_t k = 0; k < nD; k++) {
      jT[k] = fr[k];
      jT[k].dst = fr[k].dst - bandA + bandT;  // same item and band offset inside bandT
    }
    for (size_t k = 0; k < nL; k++) {
      jS[k] = fs[k];
      jS[k].src = fs[k].src - bandA + bandT;
    }
  }
  auto up = [&](void* dst, const void* src, size_t bytes) { return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice); };
  ce = up(p->gj_rows_lev_fwd, j1.data(), j1.size() * sizeof(RowJob));
  if (ce == cudaSuccess) ce = up(p->gj_cols_lev, j2.data(), j2.size() * sizeof(ColJob));
  if (ce == cudaSuccess) ce = up(p->gj_analysis, j3.data(), j3.size() * sizeof(ColJob));
  if (ce == cudaSuccess) ce = up(p->gj_analysis_lev, jA.data(), jA.size() * sizeof(ColJob));
  if (ce == cudaSuccess) ce = up(p->gj_rows_backward, j4.data(), j4.size() * sizeof(RowJob));
  if (ce == cudaSuccess) ce = up(p->gj_synthesis, j5.data(), j5.size() * sizeof(ColJob));
  if (ce == cudaSuccess) ce = up(p->gj_rows_lev_inv, j6.data(), j6.size() * sizeof(RowJob));
  if (ce == cudaSuccess) ce = up(p->gj_coeff_fwd, j7.data(), j7.size() * sizeof(RowJob));
  if (ce == cudaSuccess) ce = up(p->gj_band_to_coeff, j8.data(), j8.size() * sizeof(RowJob));
  if (ce == cudaSuccess) ce = up(p->gj_rows_T, jT.data(), jT.size() * sizeof(RowJob));
  if (ce == cudaSuccess) ce = up(p->gj_synth_T, jS.data(), jS.size() * sizeof(ColJob));
  if (ce != cudaSuccess) return cuda_fail(ce, "upload gradient job lists");
  if (p->dct_ok) {
    p->gj_dct_x = (ColJob*)(G + o_gd1);
    p->gj_dct_ana = (RowJob*)(G + o_gd2);
    p->gj_dct_low = (RowJob*)(G + o_gd3);
    p->gj_dct_gy0 = (ColJob*)(G + o_gd4);
    p->gj_dct_sum = (ColJob*)(G + o_gd5);
    p->gj_dct_syn = (RowJob*)(G + o_gd6);
    std::vector<ColJob> gx, gg, gs;
    std::vector<RowJob> ga, gl, gy1;
    for (int i = 0; i < B; i++) {
      const size_t t0 = g2(p->gtmp + i * 2 * HW), t1 = g2(p->gtmp + i * 2 * HW + HW);
      const size_t gy0 = g2(p->gy + i * (p->nlev + 1) * HW), gyl = g2(p->gy + i * (p->nlev + 1) * HW + HW);
      const size_t lev = g2(p->lev2 + i * p->s_lev), sum = g2(p->sum2 + i * p->s_sum);
      gx.push_back(ColJob{t0, t1, 0, 0, 0, i});
      gl.push_back(RowJob{t1, t0, 2 * p->nlev + 2, i});  // the lowpass synthesis plane from dct_ra
      gg.push_back(ColJob{gy0, gy0, 0, 0, 0, i});
      gy1.push_back(RowJob{sum, gyl, 0, i});
      for (int l = 0; l < p->nlev; l++) {
        ga.push_back(RowJob{t1, lev + (size_t)l * HWh, l, i});
        gs.push_back(ColJob{sum + (size_t)l * HWh, sum + (size_t)l * HWh, 0, 0, 0, i});
      }
    }
    ce = up(p->gj_dct_x, gx.data(), gx.size() * sizeof(ColJob));
    if (ce == cudaSuccess) ce = up(p->gj_dct_ana, ga.data(), ga.size() * sizeof(RowJob));
    if (ce == cudaSuccess) ce = up(p->gj_dct_low, gl.data(), gl.size() * sizeof(RowJob));
    if (ce == cudaSuccess) ce = up(p->gj_dct_gy0, gg.data(), gg.size() * sizeof(ColJob));
    if (ce == cudaSuccess) ce = up(p->gj_dct_sum, gs.data(), gs.size() * sizeof(ColJob));
    if (ce == cudaSuccess) ce = up(p->gj_dct_syn, gy1.data(), gy1.size() * sizeof(RowJob));
    if (ce != cudaSuccess) return cuda_fail(ce, "upload spectral gradient job lists");
  }
  for (int F : {p->pf.F[0], p->pf.F[1], p->pf.F[2], p->pf.F[3]}) {
    ce = prepare_atrous_kernels(F, 0, Mmax);
    if (ce != cudaSuccess) return cuda_fail(ce, "adjoint kernel set-up");
  }
  return NSST_OK;
}

// x = A^T c: adjoint of nsst_shear_trans (directional synthesis with conj
// spectra, then the transpose of the analysis pyramid).
nsst_status nsst_shear_trans_adjoint(nsst_plan* p, const float* coeffs, float* x, void* stream) {
  if (!p || !coeffs || !x) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  NSST_TRY(need_grad(p));
  std::lock_guard<std::mutex> lk(p->mu);
  p->saved_n = 0;  // the arena no longer holds the last differentiable forward
  cudaStream_t st = (cudaStream_t)stream;
  timer_begin(p, st);
  char* G = p->garena;
  float2* G2 = (float2*)G;
  const size_t HW = (size_t)p->H * p->W;
  NSST_CUDA(launch_rows(RowOp::Fwd, p->gj_coeff_fwd, p->ndir_total, 1, p->H, p->W, coeffs, G, p->twWh, p->twW,
                        nullptr, 0, st));
  NSST_CUDA(launch_cols(ColOp::Synthesis, p->gj_synthesis, p->B * p->nlev, 1, p->H, p->W, G2, G2, p->spec,
                        (size_t)p->H * p->WH, p->twH, st));
  NSST_CUDA(launch_rows(RowOp::Inv, p->gj_rows_lev_inv, p->nlev, 1, p->H, p->W, G, G, p->twWh, p->twW, nullptr, 0,
                        st));
  NSST_CUDA(cudaMemcpyAsync(p->gy, coeffs, HW * sizeof(float), cudaMemcpyDeviceToDevice, st));
  const float* gyb = p->gy;
  return run_atrousdec_adjoint(p, 1, &gyb, &x, st);
}

// c = R^T x: adjoint of nsst_inverse_shear (transpose of the synthesis pyramid,
// then the directional analysis).
nsst_status nsst_inverse_shear_adjoint(nsst_plan* p, const float* x, float* coeffs, void* stream) {
  if (!p || !coeffs || !x) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  if (!aligned16(coeffs)) return fail(NSST_ERR_INVALID_ARG, "coeffs must be 16-byte aligned");
  NSST_TRY(need_grad(p));
  std::lock_guard<std::mutex> lk(p->mu);
  p->saved_n = 0;  // the arena no longer holds the last differentiable forward
  cudaStream_t st = (cudaStream_t)stream;
  timer_begin(p, st);
  char* G = p->garena;
  float2* G2 = (float2*)G;
  const size_t HW = (size_t)p->H * p->W;
  float* gypb = p->gyp;
  NSST_TRY(run_atrousrec_adjoint(p, 1, &x, &gypb, st));
  NSST_CUDA(cudaMemcpyAsync(coeffs, p->gyp, HW * sizeof(float), cudaMemcpyDeviceToDevice, st));
  NSST_CUDA(launch_rows(RowOp::Fwd, p->gj_rows_lev_fwd, p->nlev, 1, p->H, p->W, G, G, p->twWh, p->twW, nullptr, 0,
                        st));
  NSST_CUDA(launch_cols(ColOp::Fwd, p->gj_cols_lev, p->nlev, 1, p->H, p->W, G2, G2, nullptr, 0, p->twH, st));
  NSST_CUDA(launch_cols(ColOp::Analysis, p->gj_analysis, p->B * p->ndir_total, 1, p->H, p->W, G2, G2, p->spec, 0,
                        p->twH, st));
  NSST_CUDA(launch_rows(RowOp::Inv, p->gj_band_to_coeff, p->ndir_total, 1, p->H, p->W, G, coeffs, p->twWh, p->twW,
                        nullptr, 0, st));
  return NSST_OK;
}

nsst_status nsst_denoise_tau_batch(nsst_plan* p, const float* const* x, float* const* out, int n, const float* tau,
                                   int mode, void* stream) {
  if (!p || !x || !out || !tau) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  if (n < 1 || n > p->B) return fail(NSST_ERR_INVALID_ARG, "item count outside [1, batch capacity]");
  if (mode != NSST_THRESH_HARD && mode != NSST_THRESH_SOFT) return fail(NSST_ERR_INVALID_ARG, "bad mode");
  for (int i = 0; i < n; i++)
    if (!x[i] || !out[i]) return fail(NSST_ERR_INVALID_ARG, "NULL image pointer");
  NSST_TRY(check_spectral_n(p, n, x, out));
  std::lock_guard<std::mutex> lk(p->mu);
  cudaStream_t st = (cudaStream_t)stream;
  timer_begin(p, st);
  NSST_CUDA(launch_broadcast_tau(tau, p->th, p->nbands, n, st));
  const bool keep = p->garena != nullptr;
  p->saved_n = 0;
  NSST_TRY(enqueue_denoise(p, n, x, out, mode, true, st, keep));
  if (keep) p->saved_n = n;
  return NSST_OK;
}

int nsst_plan_saved_items(const nsst_plan* p) { return p ? p->saved_n : 0; }

}  // extern "C"

namespace {

// The backward of nsst_denoise_tau_batch; x == NULL: the band spectra and the
// pyramid's lowpass of the last differentiable forward are still in the
// arena (saved_n == n), so step 1 is skipped.  Called with the plan locked.
// tau_backward on the spectral pyramid.  Each pyramid operator is symmetric
// (IDCT2 diag(r) DCT2 with the DCT-III the DCT-II's transpose times
// diag(1, 2, 2, ...), and diagonals commute), so the adjoint of the synthesis
// is the analysis front with the synthesis tables and the adjoint of the
// analysis the synthesis back end with the analysis tables.  Images not
// 16-byte aligned pass through gyp plane 1 (unused here).
nsst_status tau_backward_dct(nsst_plan* p, const float* const* x, const float* const* grad_out, float* const* grad_x,
                             int n, const float* tau, float* grad_tau, int accumulate_tau, int mode, cudaStream_t st) {
  char* G = p->garena;
  const int H = p->H, W = p->W, B = p->B, L = p->nlev;
  const size_t HW = (size_t)H * W;
  std::vector<const float*> gout(n), t0c(n), gt0c(n), gy0c(n);
  std::vector<float*> ys(n), gt0(n), gyp0(n), gy0(n), gy1(n), gxo(n), gyp1(n);
  for (int i = 0; i < n; i++) {
    gyp1[i] = p->gyp + (size_t)i * (L + 1) * HW + HW;
    gout[i] = aligned16(grad_out[i]) ? grad_out[i] : gyp1[i];
    if (gout[i] != grad_out[i])
      NSST_CUDA(cudaMemcpyAsync(gyp1[i], grad_out[i], HW * sizeof(float), cudaMemcpyDeviceToDevice, st));
    gxo[i] = aligned16(grad_x[i]) ? grad_x[i] : gyp1[i];
    t0c[i] = p->tmp + (size_t)i * p->s_tmp;
    ys[i] = p->pyr + (size_t)i * p->s_pyr + HW;
    gt0[i] = p->gtmp + (size_t)i * 2 * HW;
    gt0c[i] = gt0[i];
    gyp0[i] = p->gyp + (size_t)i * (L + 1) * HW;
    gy0[i] = p->gy + (size_t)i * (L + 1) * HW;
    gy0c[i] = gy0[i];
    gy1[i] = gy0[i] + HW;
  }
  // 1. the coefficient spectra of x (recomputed unless saved) and the
  //    pre-threshold lowpass band, spatial, in pyr plane 1
  if (x) {
    NSST_TRY(enqueue_dct_analysis(p, n, x, st));
    NSST_TRY(enqueue_band_analysis(p, n, false, st));
    timer_mark(p, "recompute_coefficients", st);
  }
  NSST_TRY(enqueue_dct_lowpass_rows(p, n, st));
  NSST_TRY(enqueue_dct_cols_out(p, n, t0c.data(), ys.data(), st));
  // 2. d loss / d coefficients: level spectra of IDCT2(Q_l .* DCT2(grad_out)),
  //    lowpass IDCT2(G_low .* DCT2(grad_out)) in gyp plane 0
  NSST_TRY(enqueue_dct_rows_io(p, n, gout.data(), gt0.data(), st));
  NSST_CUDA(launch_dct_cols(kDct2, p->gj_dct_x, B, n, H, W, G, G, p->twH, p->wdH, st));
  NSST_CUDA(launch_dct_rows_ana(p->gj_dct_ana, B * L, n, H, W, G, G, p->dct_rs, HW, p->twWh, p->twW, p->twDW, false,
                                st));
  NSST_CUDA(launch_dct_cols(kDctAna, p->gj_cols_lev, B * L, n, H, W, G, G, p->twH, p->wdH, st));
  NSST_CUDA(launch_dct_rows_ana(p->gj_dct_low, B, n, H, W, G, G, p->dct_ra, HW, p->twWh, p->twW, p->twDW, true, st));
  NSST_TRY(enqueue_dct_cols_out(p, n, gt0c.data(), gyp0.data(), st));
  NSST_TRY(enqueue_band_analysis(p, n, true, st));
  timer_mark(p, "gradient_analysis", st);
  // 3. threshold subgradient per band (+ tau partials), then D^T
  const size_t pstride = (size_t)B * p->ntiles;
  NSST_CUDA(launch_rows_backward(p->gj_rows_backward, B * p->ndir_total, n, H, W, p->arena, G, p->twWh, p->twW, tau,
                                 mode, p->partials, pstride, st));
  timer_mark(p, "band_rows_backward", st);
  NSST_CUDA(launch_cols(ColOp::Synthesis, p->gj_synthesis, B * L, n, H, W, (float2*)G, (float2*)G, p->spec,
                        (size_t)H * p->WH, p->twH, st));
  timer_mark(p, "gradient_synthesis", st);
  for (int c0 = 0; c0 < n; c0 += kMaxAtrousJobs) {  // lowpass band mask -> gy plane 0
    const int cn = std::min(kMaxAtrousJobs, n - c0);
    FoldJobs jl{};
    for (int t = 0; t < cn; t++) jl.j[t] = FoldJob{ys[c0 + t], gyp0[c0 + t], gy0[c0 + t]};
    NSST_CUDA(launch_lowpass_backward(jl, cn, HW, tau, mode, p->partials, c0 * p->ntiles, p->ntiles, st));
  }
  // 4. d loss / d x = IDCT2(sum_l R_l .* DCT2(g_l) + R_low .* DCT2(g_0))
  NSST_TRY(enqueue_dct_rows_io(p, n, gy0c.data(), gy0.data(), st));
  NSST_CUDA(launch_dct_cols(kDct2, p->gj_dct_gy0, B, n, H, W, G, G, p->twH, p->wdH, st));
  NSST_CUDA(launch_dct_cols(kDct2, p->gj_dct_sum, B * L, n, H, W, G, G, p->twH, p->wdH, st));
  NSST_CUDA(launch_dct_rows_syn(p->gj_dct_syn, B, n, L, (size_t)H * p->WH, H, W, G, G, p->gy, (size_t)(L + 1) * HW,
                                p->dct_ra, HW, p->dct_ra + (size_t)(2 * L + 1) * HW, p->twWh, p->twW, p->twDW, st));
  std::vector<const float*> gy1c(gy1.begin(), gy1.end());
  NSST_TRY(enqueue_dct_cols_out(p, n, gy1c.data(), gxo.data(), st));
  for (int i = 0; i < n; i++)
    if (gxo[i] != grad_x[i])
      NSST_CUDA(cudaMemcpyAsync(grad_x[i], gxo[i], HW * sizeof(float), cudaMemcpyDeviceToDevice, st));
  timer_mark(p, "gradient_pyramid", st);
  NSST_CUDA(launch_reduce_tau(p->partials, n * p->ntiles, pstride, p->nbands, grad_tau, accumulate_tau != 0, st));
  timer_mark(p, "reduce_tau", st);
  return NSST_OK;
}

nsst_status tau_backward(nsst_plan* p, const float* const* x, const float* const* grad_out, float* const* grad_x,
                         int n, const float* tau, float* grad_tau, int accumulate_tau, int mode, cudaStream_t st) {
  timer_begin(p, st);
  bool spectral = p->saved_dct;
  if (x) {
    spectral = p->dct_on;
    for (int i = 0; i < n; i++) spectral = spectral && aligned16(x[i]);
  }
  if (spectral) return tau_backward_dct(p, x, grad_out, grad_x, n, tau, grad_tau, accumulate_tau, mode, st);
  char* A = p->arena;
  float2* A2 = (float2*)A;
  char* G = p->garena;
  float2* G2 = (float2*)G;
  const int H = p->H, W = p->W, B = p->B;
  const size_t HW = (size_t)H * W;
  // 1. recompute the coefficient spectra of x (they are not stored)
  std::vector<float*> ys(n), gyp(n), gy(n);
  for (int i = 0; i < n; i++) {
    ys[i] = p->pyr + i * p->s_pyr;
    gyp[i] = p->gyp + i * (p->nlev + 1) * HW;
    gy[i] = p->gy + i * (p->nlev + 1) * HW;
  }
  if (x) {
    NSST_TRY(run_atrousdec(p, n, x, ys.data(), nullptr, st));
    NSST_CUDA(launch_rows(RowOp::Fwd, p->j_rows_lev_fwd, B * p->nlev, n, H, W, A, A, p->twWh, p->twW, nullptr, 0,
                          st));
    NSST_CUDA(launch_cols(ColOp::Fwd, p->j_cols_lev, B * p->nlev, n, H, W, A2, A2, nullptr, 0, p->twH, st));
    NSST_TRY(enqueue_band_analysis(p, n, false, st));
    timer_mark(p, "recompute_coefficients", st);
  }
  // 2. d loss / d thresholded coefficients = D P_s^T grad_out
  NSST_TRY(run_atrousrec_adjoint(p, n, grad_out, gyp.data(), st));
  NSST_CUDA(launch_rows(RowOp::Fwd, p->gj_rows_lev_fwd, B * p->nlev, n, H, W, G, G, p->twWh, p->twW, nullptr, 0, st));
  NSST_CUDA(launch_cols(ColOp::Fwd, p->gj_cols_lev, B * p->nlev, n, H, W, G2, G2, nullptr, 0, p->twH, st));
  NSST_TRY(enqueue_band_analysis(p, n, true, st));
  timer_mark(p, "gradient_analysis", st);
  // 3. threshold subgradient per band (+ tau partials), then D^T
  const size_t pstride = (size_t)B * p->ntiles;
  NSST_CUDA(launch_rows_backward(p->gj_rows_backward, B * p->ndir_total, n, H, W, A, G, p->twWh, p->twW, tau, mode,
                                 p->partials, pstride, st));
  timer_mark(p, "band_rows_backward", st);
  NSST_CUDA(launch_cols(ColOp::Synthesis, p->gj_synthesis, B * p->nlev, n, H, W, G2, G2, p->spec, (size_t)H * p->WH,
                        p->twH, st));
  NSST_CUDA(launch_rows(RowOp::Inv, p->gj_rows_lev_inv, B * p->nlev, n, H, W, G, G, p->twWh, p->twW, nullptr, 0, st));
  timer_mark(p, "gradient_synthesis", st);
  // lowpass band
  for (int c0 = 0; c0 < n; c0 += kMaxAtrousJobs) {
    const int cn = std::min(kMaxAtrousJobs, n - c0);
    FoldJobs jl{};
    for (int t = 0; t < cn; t++) jl.j[t] = FoldJob{ys[c0 + t], gyp[c0 + t], gy[c0 + t]};
    NSST_CUDA(launch_lowpass_backward(jl, cn, HW, tau, mode, p->partials, c0 * p->ntiles, p->ntiles, st));
  }
  // 4. d loss / d x = P^T g_y
  std::vector<const float*> gyc(gy.begin(), gy.end());
  NSST_TRY(run_atrousdec_adjoint(p, n, gyc.data(), grad_x, st));
  NSST_CUDA(launch_reduce_tau(p->partials, n * p->ntiles, pstride, p->nbands, grad_tau, accumulate_tau != 0, st));
  timer_mark(p, "reduce_tau", st);
  return NSST_OK;
}

nsst_status tau_backward_check(nsst_plan* p, const float* const* grad_out, float* const* grad_x, int n,
                               const float* tau, float* grad_tau, int mode) {
  if (!p || !grad_out || !grad_x || !tau || !grad_tau) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  if (n < 1 || n > p->B) return fail(NSST_ERR_INVALID_ARG, "item count outside [1, batch capacity]");
  if (mode != NSST_THRESH_HARD && mode != NSST_THRESH_SOFT) return fail(NSST_ERR_INVALID_ARG, "bad mode");
  NSST_TRY(need_grad(p));
  for (int i = 0; i < n; i++)
    if (!grad_out[i] || !grad_x[i]) return fail(NSST_ERR_INVALID_ARG, "NULL image pointer");
  return NSST_OK;
}

}  // namespace

extern "C" {

nsst_status nsst_denoise_tau_backward(nsst_plan* p, const float* const* x, const float* const* grad_out,
                                      float* const* grad_x, int n, const float* tau, float* grad_tau,
                                      int accumulate_tau, int mode, void* stream) {
  NSST_TRY(tau_backward_check(p, grad_out, grad_x, n, tau, grad_tau, mode));
  if (!x) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  for (int i = 0; i < n; i++)
    if (!x[i]) return fail(NSST_ERR_INVALID_ARG, "NULL image pointer");
  NSST_TRY(check_spectral_n(p, n, x, nullptr));
  std::lock_guard<std::mutex> lk(p->mu);
  p->saved_n = 0;  // step 1 rewrites the arena's band spectra
  return tau_backward(p, x, grad_out, grad_x, n, tau, grad_tau, accumulate_tau, mode, (cudaStream_t)stream);
}

nsst_status nsst_denoise_tau_backward_saved(nsst_plan* p, const float* const* grad_out, float* const* grad_x, int n,
                                            const float* tau, float* grad_tau, int accumulate_tau, int mode,
                                            void* stream) {
  NSST_TRY(tau_backward_check(p, grad_out, grad_x, n, tau, grad_tau, mode));
  std::lock_guard<std::mutex> lk(p->mu);
  if (p->saved_n != n)
    return fail(NSST_ERR_INVALID_ARG, "no saved coefficients of n items: the plan ran another call since the forward");
  return tau_backward(p, nullptr, grad_out, grad_x, n, tau, grad_tau, accumulate_tau, mode, (cudaStream_t)stream);
}

}  // extern "C"

// ============================================================ uneven batches
struct nsst_multi {
  std::vector<nsst_plan*> plans;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> done;
  cudaStream_t cap = nullptr;
  cudaEvent_t fork = nullptr, finished = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<const void*> key;
  int key_mode = -1;
  std::mutex mu;
};

extern "C" {

nsst_status nsst_multi_create(nsst_plan* const* plans, int nplans, nsst_multi** out) {
  if (!plans || nplans < 1 || !out) return fail(NSST_ERR_INVALID_ARG, "bad arguments");
  *out = nullptr;
  nsst_multi* m = new (std::nothrow) nsst_multi();
  if (!m) return fail(NSST_ERR_OUT_OF_MEMORY, "host allocation failed");
  m->plans.assign(plans, plans + nplans);
  for (nsst_plan* p : m->plans)
    if (!p) {
      delete m;
      return fail(NSST_ERR_INVALID_ARG, "NULL plan");
    }
  cudaError_t e = cudaStreamCreateWithFlags(&m->cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&m->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&m->finished, cudaEventDisableTiming);
  for (int i = 0; i < nplans && e == cudaSuccess; i++) {
    cudaStream_t s = nullptr;
    cudaEvent_t d = nullptr;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&d, cudaEventDisableTiming);
    m->streams.push_back(s);
    m->done.push_back(d);
  }
  if (e != cudaSuccess) {
    nsst_multi_destroy(m);
    return cuda_fail(e, "multi streams");
  }
  *out = m;
  return NSST_OK;
}

nsst_status nsst_multi_destroy(nsst_multi* m) {
  if (!m) return NSST_OK;
  cudaDeviceSynchronize();
  if (m->exec) cudaGraphExecDestroy(m->exec);
  for (cudaStream_t s : m->streams)
    if (s) cudaStreamDestroy(s);
  for (cudaEvent_t d : m->done)
    if (d) cudaEventDestroy(d);
  if (m->cap) cudaStreamDestroy(m->cap);
  if (m->fork) cudaEventDestroy(m->fork);
  if (m->finished) cudaEventDestroy(m->finished);
  delete m;
  return NSST_OK;
}

nsst_status nsst_multi_denoise(nsst_multi* m, const nsst_item* items, int n, const double* K, int mode,
                               void* stream) {
  if (!m || !items || n < 1 || !K) return fail(NSST_ERR_INVALID_ARG, "bad arguments");
  if (mode != NSST_THRESH_HARD && mode != NSST_THRESH_SOFT) return fail(NSST_ERR_INVALID_ARG, "bad mode");
  std::lock_guard<std::mutex> lk(m->mu);
  const int np = (int)m->plans.size();
  std::vector<std::vector<int>> groups(np);
  for (int i = 0; i < n; i++) {
    if (items[i].plan < 0 || items[i].plan >= np || !items[i].x || !items[i].out)
      return fail(NSST_ERR_INVALID_ARG, "bad item");
    groups[items[i].plan].push_back(i);
  }
  for (int g = 0; g < np; g++) {
    if ((int)groups[g].size() > m->plans[g]->B) return fail(NSST_ERR_INVALID_ARG, "group exceeds plan capacity");
    if (!groups[g].empty() && !m->plans[g]->has_scalars)
      return fail(NSST_ERR_INVALID_ARG, "plan without stored scalars");
  }
  for (nsst_plan* q : m->plans) q->saved_n = 0;  // the replay rewrites the plans' arenas
  // thresholds into every plan's pinned staging; the previous replay must be done with them
  NSST_CUDA(cudaEventSynchronize(m->finished));
  std::vector<char> lowth(np, 0);
  for (int g = 0; g < np; g++) {
    nsst_plan* p = m->plans[g];
    for (size_t t = 0; t < groups[g].size(); t++) {
      const double sg = items[groups[g][t]].sigma;
      if (!std::isfinite(sg) || sg < 0) return fail(NSST_ERR_INVALID_ARG, "sigma must be finite and >= 0");
      for (int b = 0; b < p->nbands; b++) {
        double th = K[p->band_level[b]] * sg * p->scalars[b];
        if (!std::isfinite(th) || th < 0) return fail(NSST_ERR_INVALID_ARG, "thresholds must be finite and >= 0");
        p->th_host[t * p->nbands + b] = (float)th;
      }
      if (p->th_host[t * p->nbands] > 0.f) lowth[g] = 1;
    }
  }
  std::vector<const void*> key;
  for (int i = 0; i < n; i++) {
    key.push_back(items[i].x);
    key.push_back(items[i].out);
    key.push_back((const void*)(intptr_t)items[i].plan);
  }
  for (int g = 0; g < np; g++) key.push_back((const void*)(intptr_t)lowth[g]);
  cudaStream_t st = (cudaStream_t)stream;
  if (!m->exec || key != m->key || mode != m->key_mode) {
    if (m->exec) {
      cudaGraphExecDestroy(m->exec);
      m->exec = nullptr;
    }
    NSST_CUDA(cudaStreamBeginCapture(m->cap, cudaStreamCaptureModeThreadLocal));
    nsst_status s = NSST_OK;
    cudaError_t ce = cudaEventRecord(m->fork, m->cap);
    for (int g = 0; g < np && s == NSST_OK && ce == cudaSuccess; g++) {
      if (groups[g].empty()) continue;
      nsst_plan* p = m->plans[g];
      std::lock_guard<std::mutex> plk(p->mu);
      ce = cudaStreamWaitEvent(m->streams[g], m->fork, 0);
      if (ce != cudaSuccess) break;
      const int cnt = (int)groups[g].size();
      ce = cudaMemcpyAsync(p->th, p->th_host, sizeof(float) * p->nbands * cnt, cudaMemcpyHostToDevice,
                           m->streams[g]);
      if (ce != cudaSuccess) break;
      std::vector<const float*> xs(cnt);
      std::vector<float*> os(cnt);
      for (int t = 0; t < cnt; t++) {
        xs[t] = items[groups[g][t]].x;
        os[t] = items[groups[g][t]].out;
      }
      s = enqueue_denoise(p, cnt, xs.data(), os.data(), mode, lowth[g] != 0, m->streams[g]);
      if (s == NSST_OK) ce = cudaEventRecord(m->done[g], m->streams[g]);
      if (ce == cudaSuccess && s == NSST_OK) ce = cudaStreamWaitEvent(m->cap, m->done[g], 0);
    }
    cudaGraph_t graph = nullptr;
    cudaError_t ce2 = cudaStreamEndCapture(m->cap, &graph);
    if (s != NSST_OK || ce != cudaSuccess || ce2 != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      if (s != NSST_OK) return s;
      return cuda_fail(ce != cudaSuccess ? ce : ce2, "multi capture");
    }
    ce = cudaGraphInstantiate(&m->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
      m->exec = nullptr;
      return cuda_fail(ce, "cudaGraphInstantiate");
    }
    m->key = key;
    m->key_mode = mode;
  }
  NSST_CUDA(cudaGraphLaunch(m->exec, st));
  NSST_CUDA(cudaEventRecord(m->finished, st));
  return NSST_OK;
}

}  // extern "C"

// ============================================ undecimated wavelets, separation
namespace {

bool divisible_pow2(int v, int L) { return L >= 1 && L < 30 && v % (1 << L) == 0; }

nsst_status check_rdwt(int n, int H, int W, int lh, int L) {
  if (n < 1 || n > 65535) return fail(NSST_ERR_INVALID_ARG, "image count outside [1, 65535]");
  if (lh < 1 || lh > kMaxQmf) return fail(NSST_ERR_INVALID_ARG, "filter length outside [1, 32]");
  // mrdwt.cpp:94-112: both dimensions must be multiples of 2^L
  if (H < 1 || W < 1 || !divisible_pow2(H, L) || !divisible_pow2(W, L))
    return fail(NSST_ERR_INVALID_ARG, "L >= 1 and H, W multiples of 2^L required");
  if (!rdwt_width_supported(W)) return fail(NSST_ERR_INVALID_ARG, "W above 8192");
  return NSST_OK;
}

// mrdwt_r.h:135-208 for n images (x item stride s_x; yl item stride HW; yh
// item stride 3 L HW); thr (device, n floats) hard-thresholds every highpass
// plane as it is written (thresh.m:44 with option 1), or NULL.
nsst_status enqueue_mrdwt(const float* x, size_t s_x, int n, int H, int W, const WvTaps& t, int L, float* yl,
                          float* yh, const float* thr, cudaStream_t st) {
  const size_t HW = (size_t)H * W;
  for (int l = 1; l <= L; l++) {
    const WvPlanes P{l == 1 ? x : yl, l == 1 ? s_x : HW, yl, HW, yh + (size_t)3 * (l - 1) * HW, (size_t)3 * L * HW};
    NSST_CUDA(launch_rdwt_level(P, n, H, W, 1 << (l - 1), t, thr, st));
  }
  return NSST_OK;
}

// mirdwt_r.h:148-218 for n images.  scratch == NULL: each level's HL / LH
// planes take the row pass's outputs (yh is consumed); otherwise scratch holds
// two planes per image.
nsst_status enqueue_mirdwt(const float* yl, float* yh, float* scratch, int n, int H, int W, const WvTaps& t, int L,
                           float* x, cudaStream_t st) {
  const size_t HW = (size_t)H * W, s_yh = (size_t)3 * L * HW;
  for (int l = L; l >= 1; l--) {
    float* lev = yh + (size_t)3 * (l - 1) * HW;
    float* tl = scratch ? scratch : lev + HW;
    float* th = scratch ? scratch + HW : lev;
    const size_t s_t = scratch ? 2 * HW : s_yh;
    NSST_CUDA(launch_irdwt_level(l == L ? yl : x, HW, lev, s_yh, tl, th, s_t, x, HW, n, H, W, 1 << (l - 1), t, st));
  }
  return NSST_OK;
}

// MAD.m: median(|x - median(x)|) / 0.6745 over the non-NaN values; MATLAB's
// median averages the two middle values of an even count.
double median_inplace(std::vector<double>& v) {
  const size_t m = v.size(), mid = m / 2;
  std::nth_element(v.begin(), v.begin() + (long)mid, v.end());
  const double hi = v[mid];
  if (m % 2) return hi;
  const double lo = *std::max_element(v.begin(), v.begin() + (long)mid);
  return (lo + hi) / 2;
}

double mad(const std::vector<double>& x) {
  std::vector<double> v;
  v.reserve(x.size());
  for (double t : x)
    if (!std::isnan(t)) v.push_back(t);
  if (v.empty()) return std::nan("");
  const double med = median_inplace(v);
  for (double& t : v) t = std::fabs(t - med);
  return median_inplace(v) / .6745;
}

// Stream-ordered device scratch, released (in stream order) on every exit path.
struct AsyncScratch {
  void* ptr = nullptr;
  cudaStream_t st = nullptr;
  ~AsyncScratch() {
    if (ptr) cudaFreeAsync(ptr, st);
  }
};

nsst_status qmf_vector(const char* type, int par, std::vector<double>* f) {
  if (!on_filter(type, par, f)) return fail(NSST_ERR_INVALID_ARG, std::string("missing QMF table ") + type);
  return NSST_OK;
}

}  // namespace

extern "C" {

nsst_status nsst_onfilter(const char* type, int par, double* out, int* len) {
  if (!type || !out || !len) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  std::vector<double> f;
  if (!on_filter(type, par, &f))
    return fail(NSST_ERR_INVALID_ARG, std::string("no MakeONFilter table for ") + type + " " + std::to_string(par));
  if ((int)f.size() > NSST_MAX_QMF) return fail(NSST_ERR_INVALID_ARG, "QMF longer than NSST_MAX_QMF");
  std::copy(f.begin(), f.end(), out);
  *len = (int)f.size();
  return NSST_OK;
}

nsst_status nsst_mrdwt(const float* x, int n, int H, int W, const double* h, int lh, int L, float* yl, float* yh,
                       void* stream) {
  if (!x || !h || !yl || !yh) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  NSST_TRY(check_rdwt(n, H, W, lh, L));
  const WvTaps t = analysis_taps(std::vector<double>(h, h + lh));
  return enqueue_mrdwt(x, (size_t)H * W, n, H, W, t, L, yl, yh, nullptr, (cudaStream_t)stream);
}

nsst_status nsst_mirdwt(const float* yl, const float* yh, int n, int H, int W, const double* h, int lh, int L,
                        float* x, void* stream) {
  if (!x || !h || !yl || !yh) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  NSST_TRY(check_rdwt(n, H, W, lh, L));
  const WvTaps t = synthesis_taps(std::vector<double>(h, h + lh));
  cudaStream_t st = (cudaStream_t)stream;
  AsyncScratch s;
  s.st = st;
  NSST_CUDA(cudaMallocAsync(&s.ptr, sizeof(float) * 2 * (size_t)n * H * W, st));
  // the scratch variant only reads yh
  return enqueue_mirdwt(yl, const_cast<float*>(yh), (float*)s.ptr, n, H, W, t, L, x, st);
}

nsst_status nsst_tv_correction(const float* x, int n, int H, int W, double gamma, float* y, void* stream) {
  if (!x || !y) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  if (x == y) return fail(NSST_ERR_INVALID_ARG, "y must not be x");
  NSST_TRY(check_rdwt(n, H, W, 2, 1));
  if (!std::isfinite(gamma) || gamma < 0) return fail(NSST_ERR_INVALID_ARG, "gamma must be finite and >= 0");
  std::vector<double> haar;
  NSST_TRY(qmf_vector("Haar", 0, &haar));
  NSST_CUDA(launch_tv_haar(x, y, (size_t)H * W, n, H, W, (float)haar[0], (float)gamma, (cudaStream_t)stream));
  return NSST_OK;
}

// separate.m:41-289 (the GPU branches: re_weight_band_cuda, shear_trans_cuda,
// thresh_cuda, inverse_shear_cuda, TVCorrection_cuda, mrdwt_cuda /
// mirdwt_cuda) for n images at once.  Per iteration the shearlet part is the
// plan's fused dec -> hard threshold -> rec pipeline with thresholds
// 1.4 delta E_b (lowpass included, thresh.m:29-32 with sc = 1), the wavelet
// part a Symmlet-4 mrdwt whose highpass planes are thresholded at 1.4 delta
// as they are written (thresh.m:44), then mirdwt.
nsst_status nsst_separate(nsst_plan* p, const float* img, int n, int level2, int itermax, double stop,
                          double gamma, const double* coeff, int ncoeff, float* C, float* P,
                          nsst_separate_info* info, void* stream) {
  if (!p || !img || !coeff || !C || !P) return fail(NSST_ERR_INVALID_ARG, "NULL argument");
  NSST_TRY(check_spectral(p, {img}));
  if (n < 1 || n > p->B) return fail(NSST_ERR_INVALID_ARG, "image count outside [1, batch capacity]");
  if (itermax < 1) return fail(NSST_ERR_INVALID_ARG, "itermax must be >= 1");
  if (!std::isfinite(stop) || stop <= 0) return fail(NSST_ERR_INVALID_ARG, "stop must be finite and > 0");
  if (!std::isfinite(gamma) || gamma < 0) return fail(NSST_ERR_INVALID_ARG, "gamma must be finite and >= 0");
  const int H = p->H, W = p->W, L = level2, nb = p->nbands;
  const size_t HW = (size_t)H * W;
  NSST_TRY(check_rdwt(n, H, W, 8, L));
  if (ncoeff < 2 || ncoeff > p->nlev + 1) return fail(NSST_ERR_INVALID_ARG, "need 2 to nlevels + 1 band weights");
  cudaStream_t st = (cudaStream_t)stream;

  // separate.m:57-58, 90: Symmlet 4 for the wavelet part, Haar for TV, Daubechies 4 for sigma
  std::vector<double> qmf, haar, d4;
  NSST_TRY(qmf_vector("Symmlet", 4, &qmf));
  NSST_TRY(qmf_vector("Haar", 0, &haar));
  NSST_TRY(qmf_vector("Daubechies", 4, &d4));
  const WvTaps ta = analysis_taps(qmf), ts = synthesis_taps(qmf);
  const int l4 = (int)d4.size();
  std::vector<double> bd4((size_t)l4);  // mdwt_r.h:118-120: the tap on x[2k + j] is h1[lh-1-j]
  for (int j = 0; j < l4; j++) {
    const int i = l4 - 1 - j;
    bd4[(size_t)j] = (i % 2 == 0) ? -d4[(size_t)i] : d4[(size_t)i];
  }
  // separate.m:66: exact band norms (cached in the plan after the first call)
  std::vector<double> E((size_t)nb);
  NSST_TRY(nsst_band_norms(p, E.data()));

  // workspace, 256-byte aligned segments
  auto seg = [](size_t bytes) { return align_up(bytes, 256); };
  const size_t nbits = (size_t)n * (nb + 3 * L);
  const size_t b_plane = seg(sizeof(float) * n * HW), b_yh = seg(sizeof(float) * n * 3 * L * HW),
               b_ths = seg(sizeof(float) * itermax * n * nb),
               b_thw = seg(sizeof(float) * itermax * n), b_bits = seg(sizeof(unsigned) * nbits),
               b_hh = seg(sizeof(double) * n * (HW / 4));
  AsyncScratch ws;
  ws.st = st;
  NSST_CUDA(cudaMallocAsync(&ws.ptr, 5 * b_plane + b_yh + b_ths + b_thw + b_bits + b_hh, st));
  char* q = (char*)ws.ptr;
  auto take = [&q](size_t b) {
    char* r = q;
    q += b;
    return r;
  };
  float* imgw = (float*)take(b_plane);
  float* ra1 = (float*)take(b_plane);
  float* ra2 = (float*)take(b_plane);
  float* S = (float*)take(b_plane);
  float* yl = (float*)take(b_plane);
  float* yh = (float*)take(b_yh);
  float* thS = (float*)take(b_ths);
  float* thW = (float*)take(b_thw);
  unsigned* bits = (unsigned*)take(b_bits);  // [n][nb] shearlet band maxima, then [n][3L] wavelet plane maxima
  double* hh = (double*)take(b_hh);

  std::lock_guard<std::mutex> lk(p->mu);
  p->saved_n = 0;
  timer_begin(p, st);
  if (!p->side) {
    NSST_CUDA(cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking));
    NSST_CUDA(cudaEventCreateWithFlags(&p->fork_ev, cudaEventDisableTiming));
    NSST_CUDA(cudaEventCreateWithFlags(&p->join_ev, cudaEventDisableTiming));
  }
  const size_t host_bytes = sizeof(double) * n * (HW / 4) + sizeof(unsigned) * nbits;
  if (p->sep_host_bytes < host_bytes) {
    if (p->sep_host) cudaFreeHost(p->sep_host);
    p->sep_host = nullptr;
    p->sep_host_bytes = 0;
    NSST_CUDA(cudaMallocHost(&p->sep_host, host_bytes));
    p->sep_host_bytes = host_bytes;
  }
  double* hhh = (double*)p->sep_host;
  unsigned* hb = (unsigned*)(hhh + (size_t)n * (HW / 4));
  std::vector<const float*> xs((size_t)n);
  std::vector<float*> os((size_t)n), ys((size_t)n);
  // separate.m:72-76: band re-weighting of the n images (ncoeff - 1 pyramid levels)
  PlaneWeights w{};
  for (int k = 0; k < ncoeff; k++) {
    if (!std::isfinite(coeff[k])) return fail(NSST_ERR_INVALID_ARG, "band weights must be finite");
    w.w[k] = (float)coeff[k];
  }
  for (int i = 0; i < n; i++) {
    xs[(size_t)i] = img + i * HW;
    os[(size_t)i] = imgw + i * HW;
    ys[(size_t)i] = p->pyr + i * p->s_pyr;
  }
  NSST_TRY(run_atrousdec(p, n, xs.data(), ys.data(), nullptr, st, ncoeff - 1));
  for (int i = 0; i < n; i++) NSST_CUDA(launch_scale_planes(ys[(size_t)i], HW, ncoeff, w, st));
  std::vector<const float*> ysc(ys.begin(), ys.end());
  NSST_TRY(run_atrousrec(p, n, ysc.data(), nullptr, os.data(), st, ncoeff - 1));
  // separate.m:82-102: HH quadrant of a one-level Daubechies-4 mdwt, per image
  NSST_CUDA(launch_dwt_hh(imgw, HW, n, H, W, bd4.data(), l4, hh, st));
  NSST_CUDA(cudaMemcpyAsync(hhh, hh, sizeof(double) * n * (HW / 4), cudaMemcpyDeviceToHost, st));
  NSST_CUDA(cudaEventRecord(p->fork_ev, st));
  // separate.m:104-114: per image the largest |c_b| of every shearlet band (buff(1) = max_b of that / E_b)
  std::vector<const float*> xw((size_t)n);
  for (int i = 0; i < n; i++) xw[(size_t)i] = imgw + i * HW;
  NSST_TRY(enqueue_band_maxima(p, n, xw.data(), bits, st));
  // separate.m:119-126: buff(2) = max |yh| of the Symmlet-4 mrdwt, per image
  NSST_CUDA(cudaMemsetAsync(bits + (size_t)n * nb, 0, sizeof(unsigned) * n * 3 * L, st));
  NSST_TRY(enqueue_mrdwt(imgw, HW, n, H, W, ta, L, yl, yh, nullptr, st));
  NSST_CUDA(launch_plane_maxabs(yh, HW, n * 3 * L, bits + (size_t)n * nb, kRedBlocks, st));
  NSST_CUDA(cudaMemcpyAsync(hb, bits, sizeof(unsigned) * nbits, cudaMemcpyDeviceToHost, st));
  // the noise estimates on the host cores while the maxima are computed
  NSST_CUDA(cudaEventSynchronize(p->fork_ev));
  std::vector<double> sigmas((size_t)n);
  {
    const int nt = std::max(1, std::min(n, host_threads()));
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; t++)
      pool.emplace_back([&, t] {
        for (int i = t; i < n; i += nt)
          sigmas[(size_t)i] = mad(std::vector<double>(hhh + (size_t)i * (HW / 4), hhh + (size_t)(i + 1) * (HW / 4)));
      });
    for (auto& th : pool) th.join();
  }
  NSST_CUDA(cudaStreamSynchronize(st));
  auto as_float = [](unsigned u) {
    float v;
    std::memcpy(&v, &u, sizeof(float));
    return v;
  };

  std::vector<float> hS((size_t)itermax * n * nb), hW((size_t)itermax * n);
  for (int i = 0; i < n; i++) {
    const double sigma = sigmas[(size_t)i], stop_i = stop * sigma;
    double b1 = 0.0;  // thresh.m:38-41 with lambda = 0: max_b max|c_b| / E_b
    for (int b = 0; b < nb; b++)
      if (E[(size_t)b] > 0) b1 = std::max(b1, (double)as_float(hb[(size_t)i * nb + b]) / E[(size_t)b]);
    float m2 = 0.0f;
    for (int k = 0; k < 3 * L; k++) m2 = std::max(m2, as_float(hb[(size_t)n * nb + (size_t)i * 3 * L + k]));
    const double b2 = m2;
    // separate.m:128-131: exponential decrease from deltamax to stop
    const double deltamax = std::min(b1, b2);
    const double lambda = std::pow(deltamax / stop_i, 1.0 / (1.0 - itermax));
    double delta = deltamax;
    for (int k = 0; k < itermax; k++) {
      const double t = 1.4 * delta;  // separate.m:169, 215
      for (int b = 0; b < nb; b++) hS[((size_t)k * n + i) * nb + b] = (float)(1.0 * t * E[(size_t)b]);
      hW[(size_t)k * n + i] = (float)t;
      delta = delta * lambda;  // separate.m:253
    }
    if (info) info[i] = nsst_separate_info{sigma, stop_i, b1, b2, deltamax, lambda};
  }
  NSST_CUDA(cudaMemcpyAsync(thS, hS.data(), sizeof(float) * hS.size(), cudaMemcpyHostToDevice, st));
  NSST_CUDA(cudaMemcpyAsync(thW, hW.data(), sizeof(float) * hW.size(), cudaMemcpyHostToDevice, st));
  NSST_CUDA(cudaStreamSynchronize(st));  // the host tables may go out of scope

  // separate.m:144-256: the relaxation loop, queued without host waits.  The
  // two parts of an iteration only share the residual, so the wavelet branch
  // runs on the plan's second stream (fork after the residual, join before
  // the next one and at the end).
  cudaStream_t sd = p->side;
  for (int i = 0; i < n; i++) {
    xs[(size_t)i] = ra1 + i * HW;
    os[(size_t)i] = S + i * HW;
  }
  NSST_CUDA(cudaMemsetAsync(C, 0, sizeof(float) * n * HW, st));
  NSST_CUDA(cudaMemsetAsync(P, 0, sizeof(float) * n * HW, st));
  for (int k = 0; k < itermax; k++) {
    NSST_CUDA(launch_sep_residual(imgw, C, P, ra1, ra2, n * HW, st));
    NSST_CUDA(cudaEventRecord(p->fork_ev, st));
    NSST_CUDA(cudaStreamWaitEvent(sd, p->fork_ev, 0));
    // points: wavelet hard threshold (second stream)
    NSST_TRY(enqueue_mrdwt(ra2, HW, n, H, W, ta, L, yl, yh, thW + (size_t)k * n, sd));
    NSST_TRY(enqueue_mirdwt(yl, yh, nullptr, n, H, W, ts, L, P, sd));
    NSST_CUDA(cudaEventRecord(p->join_ev, sd));
    // curves: shearlet hard threshold, then TV correction
    NSST_TRY(enqueue_denoise(p, n, xs.data(), os.data(), NSST_THRESH_HARD, true, st, false,
                             thS + (size_t)k * n * nb));
    NSST_CUDA(launch_tv_haar(S, C, HW, n, H, W, (float)haar[0], (float)gamma, st));
    NSST_CUDA(cudaStreamWaitEvent(st, p->join_ev, 0));
  }
  return NSST_OK;
}

}  // extern "C"
