// À trous analysis that allocates nothing: nsst_atrousdec_noalloc.
//
// Some callers cannot call cudaMalloc: a MATLAB MEX host whose GPU array
// runtime already owns the device memory pool, a process running under a
// fixed device-memory budget, or a real-time loop that must not pay
// cudaMalloc's implicit device-wide synchronisation.  For them this entry
// point runs the same pyramid kernels as nsst_atrousdec without a plan: the
// caller passes the input and the (nlevels+1) output planes, and the one
// scratch image the lowpass chain needs lives in the file-scope device array
// below, which every GPU that loads the library holds until the process exits.
#include <cstring>
#include <mutex>

#include "internal.h"
#include "pyramid_tables.h"

namespace nsst {

// Maximum image the scratch array covers: H * W <= 2048 * 2048 pixels (16 MiB).
constexpr size_t kNoAllocMaxPixels = (size_t)2048 * 2048;
static __device__ __align__(256) float g_noalloc_scratch[kNoAllocMaxPixels];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
float* g_scratch_addr[kMaxDevices] = {};

// Mirror one tabulated filter (atrousfilters.m:167-175, or the full '9-7'
// table with the halving of :100-104) and flip it in both axes, into a fixed
// array: no heap use on this path.
void table_filter_flipped(const PyrTable& t, int k, int* F, float* out) {
  const bool full = std::strcmp(t.name, "9-7") == 0;
  const int r = t.rows[k], c = t.cols[k];
  const int n = full ? r : 2 * r - 1;
  const double scale = (full && (k == 1 || k == 2)) ? 0.5 : 1.0;
  for (int a = 0; a < n; a++) {
    for (int b = 0; b < n; b++) {
      int i = n - 1 - a, j = n - 1 - b;  // flip
      int si = full ? i : (i < r ? i : 2 * r - 2 - i);
      int sj = full ? j : (j < c ? j : 2 * c - 2 - j);
      out[a * n + b] = (float)(t.m[k][si * c + sj] * scale);
    }
  }
  *F = n;
}

const PyrTable* find_table(const char* name) {
  for (const PyrTable& t : k_pyr_tables)
    if (std::strcmp(t.name, name) == 0) return &t;
  return nullptr;
}

}  // namespace
}  // namespace nsst

using namespace nsst;

extern "C" nsst_status nsst_atrousdec_noalloc(const float* x, float* y, int H, int W, int nlevels,
                                              const char* lpfilt, void* stream) {
  if (!x || !y) {
    set_error("nsst_atrousdec_noalloc: NULL image pointer");
    return NSST_ERR_INVALID_ARG;
  }
  if (nlevels < 1 || nlevels > 6 || H <= 0 || W <= 0) {
    set_error("nsst_atrousdec_noalloc: nlevels must be in [1, 6] and H, W positive");
    return NSST_ERR_INVALID_ARG;
  }
  if ((size_t)H * (size_t)W > kNoAllocMaxPixels) {
    set_error("nsst_atrousdec_noalloc: H*W exceeds the scratch limit of 4194304 pixels (2048 x 2048, 16 MiB); "
              "use a plan (nsst_plan_create + nsst_atrousdec) for larger images");
    return NSST_ERR_UNSUPPORTED_SIZE;
  }
  {
    // the input must not overlap the (nlevels+1) output planes: level 0
    // writes planes while its kernels still read x
    const uintptr_t xb = (uintptr_t)x, xe = xb + (uintptr_t)H * (uintptr_t)W * sizeof(float);
    const uintptr_t yb = (uintptr_t)y, ye = yb + (uintptr_t)(nlevels + 1) * H * W * sizeof(float);
    if (xb < ye && yb < xe) {
      set_error("nsst_atrousdec_noalloc: x overlaps the output planes y");
      return NSST_ERR_INVALID_ARG;
    }
  }
  const PyrTable* tab = find_table(lpfilt && lpfilt[0] ? lpfilt : "maxflat");
  if (!tab) {
    set_error("nsst_atrousdec_noalloc: unknown pyramid filter name");
    return NSST_ERR_INVALID_ARG;
  }
  float h0[19 * 19], h1[19 * 19];
  int F0 = 0, F1 = 0;
  table_filter_flipped(*tab, 0, &F0, h0);
  table_filter_flipped(*tab, 1, &F1, h1);
  const int Mmax = 1 << (nlevels - 1);
  if (Mmax * (F0 > F1 ? F0 : F1) + 1 > (H < W ? H : W)) {
    set_error("nsst_atrousdec_noalloc: image too small for the pyramid depth (symmetric extension)");
    return NSST_ERR_UNSUPPORTED_SIZE;
  }

  // Per-device set-up on the first call with that device current: resolve the
  // scratch array's device address and opt the kernels into their shared memory.
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_error(std::string("nsst_atrousdec_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return NSST_ERR_CUDA;
  }
  float* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev]) {
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr) {
        set_error(std::string("nsst_atrousdec_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return NSST_ERR_CUDA;
      }
      g_scratch_addr[dev] = static_cast<float*>(ptr);
    }
    scratch = g_scratch_addr[dev];
  }
  // shared-memory opt-in for this depth (idempotent, never shrinks)
  e = prepare_atrous_kernels(F0, 0, Mmax);
  if (e == cudaSuccess) e = prepare_atrous_kernels(F1, 0, Mmax);
  if (e != cudaSuccess) {
    set_error(std::string("nsst_atrousdec_noalloc: kernel set-up: ") + cudaGetErrorString(e));
    return NSST_ERR_CUDA;
  }

  // atrousdec.m:19-51.  The lowpass chain alternates between the caller's
  // plane 0 and the scratch image so that the last lowpass lands in plane 0;
  // each level writes every pixel it later reads, so nothing needs clearing.
  cudaStream_t st = (cudaStream_t)stream;
  const size_t HW = (size_t)H * W;
  const float* cur = x;
  for (int i = 0; i < nlevels; i++) {
    const int M = 1 << i;
    float* lo = ((nlevels - 1 - i) % 2 == 0) ? y : scratch;
    AtrousJobs jh{}, jl{};
    jh.j[0] = AtrousJob{cur, nullptr, y + (size_t)(nlevels - i) * HW, H, W};
    jl.j[0] = AtrousJob{cur, nullptr, lo, H, W};
    e = launch_atrous(jh, 1, H, W, M, F1, h1, 0, nullptr, st);
    if (e == cudaSuccess) e = launch_atrous(jl, 1, H, W, M, F0, h0, 0, nullptr, st);
    if (e != cudaSuccess) {
      set_error(std::string("nsst_atrousdec_noalloc: launch: ") + cudaGetErrorString(e));
      return NSST_ERR_CUDA;
    }
    cur = lo;
  }
  return NSST_OK;
}
