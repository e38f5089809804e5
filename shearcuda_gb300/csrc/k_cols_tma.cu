// The level analysis and the band synthesis column kernels of the split
// directional stage with their column groups staged by 2-D TMA.
//
// Same math, job lists and shared-memory layout as k_band_analysis_ml,
// k_band_synthesis and their split-complex column-pair forms *_p
// (k_directional.cu): c_k = colIFFT(W_k .* Y) for every band
// of a level (nsst_dec2.m:58 on the packed half spectrum), and
// colIFFT(sum_k conj(W_k) .* colFFT(c'_k)) (nsst_rec2.m:27-33).  What changes
// is how a column group (CS columns x H rows, CS * 8 contiguous bytes per
// row) reaches shared memory: instead of every thread issuing 16-byte
// cp.async copies (H * CS / 2 of them per plane, with their address
// arithmetic, then a wait and a block barrier), one thread issues
// H / tma_box_rows(H) tensor-map copies per plane against an mbarrier, and
// every thread waits on the mbarrier's phase.  The tensor map covers the
// plan's whole arena as rows of W/2 float2, so a plane at arena offset o
// (a multiple of W/2) starts at row o / (W/2).
//
// The filter spectrum of band k + 1 (analysis) or band plane k + 1
// (synthesis) is requested as soon as the first FFT pass of band k has read
// the staging buffer (the after-read hook), so the copy overlaps the rest of
// band k's transform, as the cp.async form does.
#include "internal.h"
#include "tiles.cuh"
#include "tma.cuh"

namespace nsst {

// The TMA side of one CTA: H x CS column-group planes requested against one
// mbarrier (a request may hold several planes; the waits take the phases in
// order), the bounded wait, and the drain before exit.
template <int H, int CS>
struct ColTma {
  static constexpr int BH = tma_box_rows(H), NBOX = H / BH;
  static constexpr uint32_t PLANE = (uint32_t)(H * CS * sizeof(float2)), BOX = (uint32_t)(BH * CS * sizeof(float2));
  uint32_t bar;
  int col0;
  uint32_t phase = 0;
  bool ok = true;  // false after a wait gave up: no further requests

  // thread 0, once, before the block barrier that precedes every wait
  __device__ __forceinline__ void init() const {
    mbar_init(bar, 1);
    fence_mbarrier_init();
  }
  // thread 0: the next phase completes when `planes` planes have landed
  __device__ __forceinline__ void expect(int planes) const { mbar_arrive_expect_tx(bar, planes * PLANE); }
  // thread 0: the plane whose first row is row0 of the tensor map -> dst
  __device__ __forceinline__ void load(const CUtensorMap* map, const float2* dst, int row0) const {
#pragma unroll
    for (int q = 0; q < NBOX; q++) tma_load_2d(smem_u32(dst) + q * BOX, map, col0, row0 + q * BH, bar);
  }
  // thread 0, after the block barrier that ends every read of dst: refill it
  __device__ __forceinline__ void refill(const CUtensorMap* map, const float2* dst, int row0) const {
    fence_proxy_async_smem();
    expect(1);
    load(map, dst, row0);
  }
  // every thread: the current phase's planes are in shared memory
  __device__ __forceinline__ void wait(int* err) {
    if (ok) {
      ok = mbar_wait_bounded(bar, phase, err);
      if (ok) phase ^= 1;
    }
  }
  // every thread, last: a copy still in flight after a wait gave up lands
  // before the CTA's shared memory is released
  __device__ __forceinline__ void drain(int* err) const {
    if (!ok) mbar_wait_bounded(bar, phase, err);
  }
};

// Block -> (job, column group).  The job lists come level-major with
// per_level items per level.  Launch order: for each level, for each chunk of
// column groups 512 bytes wide, every item's CTAs of that chunk; so the CTAs
// resident together read the same few column groups of the level's filter
// spectra (from DRAM once for all items of the batch: the spectra of a
// 1024 x 1024 plan, 201 MB, do not stay in the 129 MB L2 between items) and
// still write 512-byte row segments.  per_level == 0: job = blockIdx.y,
// column group = blockIdx.x.
struct ColBlock {
  int job, col0;
};
template <int CS>
__device__ __forceinline__ ColBlock col_block(int per_level) {
  const int G = gridDim.x;
  if (per_level <= 0) return {(int)blockIdx.y, (int)blockIdx.x * CS};
  int cg = 64 / CS;
  while (G % cg) cg >>= 1;
  const long lin = (long)blockIdx.y * G + blockIdx.x;
  const int gi = (int)(lin % cg);
  long t = lin / cg;
  const int i = (int)(t % per_level);
  t /= per_level;
  const int nch = G / cg;
  const int c = (int)(t % nch), l = (int)(t / nch);
  return {l * per_level + i, (c * cg + gi) * CS};
}

// Analysis of all bands of one level (job.nbands consecutive bands): the
// level spectrum's column group Y and band 0's filter group are requested
// together; band k + 1's filter group replaces band k's in Wb.
//
// DCTANA (the spectral pipeline): job.src holds the level plane with only its
// rows transformed (k_dct_rows_ana); the CTA finishes its column group itself
// as k_dct.cu's kDctAna column pass does (DCT-III down the columns, then the
// forward FFT: pre-processing pairs with wd, inverse FFT stored in the
// DCT-III output order, forward FFT), into Y, before the band loop.
template <int H, bool DCTANA>
__global__ void __launch_bounds__(AnaCfg<H>::T, AnaCfg<H>::MINB)
    k_band_analysis_ml_tma(const __grid_constant__ CUtensorMap amap, const ColJob* __restrict__ jobs, int n_active,
                           int WH, float2* dst_base, const float2* __restrict__ spec_base, int spec_row0,
                           size_t band_stride, const float2* __restrict__ twH, const float2* __restrict__ wd,
                           int* err, int per_level) {
  using C = AnaCfg<H>;
  constexpr int CS = C::CS;
  extern __shared__ __align__(1024) float2 tsm[];
  float2* A = tsm;          // transform, in place
  float2* Y = A + H * CS;   // level spectrum column group [row][column]
  float2* Wb = Y + H * CS;  // filter spectrum of the current band
  const ColBlock cb = col_block<CS>(per_level);
  const ColJob job = jobs[cb.job];
  if (job.item >= n_active) return;
  const int col0 = cb.col0;
  const bool dc = col0 == 0;
  const int band_rows = (int)(band_stride / WH);
  const int yrow = (int)(job.src / WH), srow = spec_row0 + (int)(job.spec / WH);
  ColTma<H, CS> tma{smem_u32(Wb + H * CS), col0};
  if (threadIdx.x == 0 && job.nbands > 0) {
    tma.init();
    tma.expect(2);
    tma.load(&amap, Y, yrow);
    tma.load(&amap, Wb, srow);
  }
  __syncthreads();  // the mbarrier is initialised before any thread waits on it
  if (job.nbands > 0) tma.wait(err);  // Y and band 0's filter group
  if constexpr (DCTANA) {
    // the level's column pass, ahead of the band loop (inside it, its
    // registers made the loop spill)
    // Z[k] = conj(wd[k]) (C[k] - i C[H-k]), Z[H-k] = i wd[k] (C[H-k] - i C[k]): each pair by one thread
    for (int e = threadIdx.x; e < (H / 2 + 1) * CS; e += C::T) {
      const int s = e % CS, kk = e / CS;
      if (kk == 0) continue;  // Z[0] = C[0]
      const float2 w = __ldg(&wd[kk]);
      const float2 a = Y[kk * CS + s], b = Y[(H - kk) * CS + s];
      Y[kk * CS + s] = cmulc(make_float2(a.x + b.y, a.y - b.x), w);
      if (kk != H - kk) Y[(H - kk) * CS + s] = cmul(make_float2(b.x + a.y, b.y - a.x), make_float2(-w.y, w.x));
    }
    __syncthreads();
    auto row_of = [](int i) { return i < H / 2 ? 2 * i : 2 * H - 1 - 2 * i; };
    block_fft_hook_ip<H, CS, C::T, +1>(Y, twH, SmemLd<CS>{Y},
                                      [&](int i, int s, float2 v) { A[row_of(i) * CS + s] = v; });
    block_fft_hook_ip<H, CS, C::T, -1>(A, twH, SmemLd<CS>{A}, SmemSt<CS>{Y});
  }
  for (int k = 0; k < job.nbands; k++) {
    if (k > 0) tma.wait(err);
    const float2* m0 = spec_base + job.m0 + (size_t)k * H;
    // Wk .* Y, with the packed DC/Nyquist column's M term
    // Z'[u] = P[u] Z[u] + M[u] conj(Z[-u])
    auto ld = [&](int i, int s) -> float2 {
      float2 r = cmul(Wb[i * CS + s], Y[i * CS + s]);
      if (dc && s == 0) r = cadd(r, cmul(__ldg(&m0[i]), cconj(Y[((H - i) % H) * CS])));
      return r;
    };
    // the hook runs after the first pass's barrier: every thread has read Wb
    auto next = [&]() {
      if (threadIdx.x == 0 && tma.ok && k + 1 < job.nbands) tma.refill(&amap, Wb, srow + (k + 1) * band_rows);
    };
    block_fft_hook_ip<H, CS, C::T, +1>(A, twH, ld, ColGlobalSt{dst_base + job.dst + (size_t)k * band_stride + col0, WH},
                                      next);
  }
  tma.drain(err);
}

// The same on split-complex column pairs (the math of k_band_analysis_ml_p):
// twH4 is the broadcast twiddle table.
template <int H>
__global__ void __launch_bounds__(AnaCfg<H>::T, AnaCfg<H>::MINB)
    k_band_analysis_ml_p_tma(const __grid_constant__ CUtensorMap amap, const ColJob* __restrict__ jobs,
                             int n_active, int WH, float2* dst_base, const float2* __restrict__ spec_base,
                             int spec_row0, size_t band_stride, const float2* __restrict__ twH4, int* err,
                             int per_level) {
  using C = AnaCfg<H>;
  constexpr int CS = C::CS, NP = CS / 2;
  extern __shared__ __align__(1024) float2 tsm[];
  cpx2* A = reinterpret_cast<cpx2*>(tsm);  // transform [row][pair], in place
  float2* Y = tsm + H * CS;                // level spectrum column group [row][column]
  float2* Wb = Y + H * CS;                 // filter spectrum of the current band
  const ColBlock cb = col_block<CS>(per_level);
  const ColJob job = jobs[cb.job];
  if (job.item >= n_active) return;
  const int col0 = cb.col0;
  const bool dc = col0 == 0;
  const int band_rows = (int)(band_stride / WH);
  const int yrow = (int)(job.src / WH), srow = spec_row0 + (int)(job.spec / WH);
  ColTma<H, CS> tma{smem_u32(Wb + H * CS), col0};
  if (threadIdx.x == 0 && job.nbands > 0) {
    tma.init();
    tma.expect(2);
    tma.load(&amap, Y, yrow);
    tma.load(&amap, Wb, srow);
  }
  __syncthreads();
  for (int k = 0; k < job.nbands; k++) {
    tma.wait(err);
    const float2* m0 = spec_base + job.m0 + (size_t)k * H;
    // Wk .* Y for two columns, the packed DC/Nyquist column's M term on lane 0 of pair 0
    auto ld = [&](int i, int p) -> cpx2 {
      cpx2 r = cmul_pp(ld_pair(Wb + i * CS + 2 * p), ld_pair(Y + i * CS + 2 * p));
      if (dc && p == 0) {
        const float2 a = cmul(__ldg(&m0[i]), cconj(Y[((H - i) % H) * CS]));
        r.re.x += a.x;
        r.im.x += a.y;
      }
      return r;
    };
    auto next = [&]() {
      if (threadIdx.x == 0 && tma.ok && k + 1 < job.nbands) tma.refill(&amap, Wb, srow + (k + 1) * band_rows);
    };
    float2* dst = dst_base + job.dst + (size_t)k * band_stride + col0;
    auto st = [&](int i, int p, cpx2 v) { st_pair(dst + (size_t)i * WH + 2 * p, v); };
    block_fft_hook_ip<H, NP, C::T, +1>(A, twH4, ld, st, next);
  }
  tma.drain(err);
}

// Synthesis: dst = colIFFT( sum_k conj(Wk) .* colFFT(src_k) ); band k's
// column group arrives in P by TMA, the transform runs in place in A and its
// last pass accumulates into S; D keeps the DC column's transform for the
// conj(M[u] X[-u]) term.
template <int H>
__global__ void __launch_bounds__(SynCfg<H>::T, SynCfg<H>::MINB)
    k_band_synthesis_tma(const __grid_constant__ CUtensorMap amap, const ColJob* __restrict__ jobs, int n_active,
                         int WH, float2* dst_base, const float2* __restrict__ spec_base, size_t band_stride,
                         const float2* __restrict__ twH, int* err, int per_level) {
  using C = SynCfg<H>;
  constexpr int CS = C::CS;
  static_assert(C::LD == CS, "dense column groups");
  extern __shared__ __align__(1024) float2 tsm[];
  float2 *A = tsm, *S = tsm + (size_t)H * CS, *D = tsm + 2 * (size_t)H * CS;
  float2* P = D + H;  // staging: the band's H x CS column group, [row][column]
  const ColBlock cb = col_block<CS>(per_level);
  const ColJob job = jobs[cb.job];
  if (job.item >= n_active) return;
  const int col0 = cb.col0;
  const bool dc = col0 == 0;
  const int band_rows = (int)(band_stride / WH);
  const int brow = (int)(job.src / WH);
  ColTma<H, CS> tma{smem_u32(P + H * CS), col0};
  if (threadIdx.x == 0 && job.nbands > 0) {
    tma.init();
    tma.expect(1);
    tma.load(&amap, P, brow);
  }
  __syncthreads();  // the mbarrier is initialised before any thread waits on it
  for (int k = 0; k < job.nbands; k++) {
    const float2* spec = spec_base + job.spec + k * band_stride + col0;
    const bool first = k == 0;
    auto acc_st = [&](int i, int sq, float2 z) {
      const float2 p = cmulc(z, __ldg(&spec[(size_t)i * WH + sq]));
      float2* t = &S[i * CS + sq];
      *t = first ? p : cadd(*t, p);
      if (dc && sq == 0) D[i] = z;
    };
    tma.wait(err);
    // the first pass has read band k from P: band k + 1 may come in
    auto next = [&]() {
      if (threadIdx.x == 0 && tma.ok && k + 1 < job.nbands) tma.refill(&amap, P, brow + (k + 1) * band_rows);
    };
    block_fft_hook_ip<H, CS, C::T, -1>(A, twH, SmemLd<CS>{P}, acc_st, next);
    if (dc) {
      for (int i = threadIdx.x; i < H; i += C::T) {
        const float2 m = __ldg(&spec_base[job.m0 + (size_t)k * H + i]);
        S[i * CS] = cadd(S[i * CS], cconj(cmul(m, D[(H - i) % H])));  // conj(M) conj(z[-u])
      }
      __syncthreads();
    }
  }
  block_fft_hook_ip<H, CS, C::T, +1>(S, twH, SmemLd<CS>{S}, ColGlobalSt{dst_base + job.dst + col0, WH});
  tma.drain(err);
}

// The same on split-complex column pairs (the math of k_band_synthesis_p).
template <int H>
__global__ void __launch_bounds__(SynCfg<H>::T, SynCfg<H>::MINB)
    k_band_synthesis_p_tma(const __grid_constant__ CUtensorMap amap, const ColJob* __restrict__ jobs, int n_active,
                           int WH, float2* dst_base, const float2* __restrict__ spec_base, size_t band_stride,
                           const float2* __restrict__ twH4, int* err, int per_level) {
  using C = SynCfg<H>;
  constexpr int CS = C::CS, NP = CS / 2;
  extern __shared__ __align__(1024) float2 tsm[];
  cpx2* A = reinterpret_cast<cpx2*>(tsm);                  // transform [row][pair]
  cpx2* S = reinterpret_cast<cpx2*>(tsm + (size_t)H * CS);  // running band sum [row][pair]
  float2* D = tsm + 2 * (size_t)H * CS;                     // column 0 of the band's transform
  float2* P = D + H;                                        // staging: the band's column group [row][column]
  const ColBlock cb = col_block<CS>(per_level);
  const ColJob job = jobs[cb.job];
  if (job.item >= n_active) return;
  const int col0 = cb.col0;
  const bool dc = col0 == 0;
  const int band_rows = (int)(band_stride / WH);
  const int brow = (int)(job.src / WH);
  ColTma<H, CS> tma{smem_u32(P + H * CS), col0};
  if (threadIdx.x == 0 && job.nbands > 0) {
    tma.init();
    tma.expect(1);
    tma.load(&amap, P, brow);
  }
  __syncthreads();
  for (int k = 0; k < job.nbands; k++) {
    const float2* spec = spec_base + job.spec + k * band_stride + col0;
    const bool first = k == 0;
    auto acc_st = [&](int i, int p, cpx2 z) {
      const float4 w = __ldg(reinterpret_cast<const float4*>(spec + (size_t)i * WH + 2 * p));
      const cpx2 q = cmulc_pp(z, pair(make_float2(w.x, w.y), make_float2(w.z, w.w)));
      cpx2* t = &S[i * NP + p];
      *t = first ? q : cadd(*t, q);
      if (dc && p == 0) D[i] = lane0(z);
    };
    tma.wait(err);
    auto next = [&]() {
      if (threadIdx.x == 0 && tma.ok && k + 1 < job.nbands) tma.refill(&amap, P, brow + (k + 1) * band_rows);
    };
    auto ldp = [&](int i, int p) -> cpx2 { return ld_pair(P + i * CS + 2 * p); };
    block_fft_hook_ip<H, NP, C::T, -1>(A, twH4, ldp, acc_st, next);
    if (dc) {
      for (int i = threadIdx.x; i < H; i += C::T) {
        const float2 m = __ldg(&spec_base[job.m0 + (size_t)k * H + i]);
        const float2 a = cconj(cmul(m, D[(H - i) % H]));  // conj(M) conj(z[-u])
        S[i * NP].re.x += a.x;
        S[i * NP].im.x += a.y;
      }
      __syncthreads();
    }
  }
  float2* dst = dst_base + job.dst + col0;
  block_fft_hook_ip<H, NP, C::T, +1>(
      S, twH4, [&](int i, int p) -> cpx2 { return S[i * NP + p]; },
      [&](int i, int p, cpx2 v) { st_pair(dst + (size_t)i * WH + 2 * p, v); });
  tma.drain(err);
}

// Synthesis with the band sum in registers: the last pass of each band's
// column FFT accumulates conj(W_k) .* X into the thread's own outputs (the
// same (row, column) slots for every band), with W_k's column group staged
// by TMA next to the band's, so the sum needs no shared-memory plane and the
// spectrum no global load.  Shared memory: the transform A, the band's
// column group P, the spectrum's column group Wc, the DC column D.  Two
// mbarriers: P is refilled once the first pass has read it, Wc once the last
// pass has.  Threads per CTA: RaccCfg (every thread owns the same number of
// last-pass outputs).
template <int H>
struct RaccCfg {
  using Plan = typename FftPlan<H>::type;
  static constexpr int CS = ColCfg<H>::CS;
  static constexpr int RL = LastRadix<Plan>::value;
  static constexpr int TOTAL_LAST = (H / RL) * CS;
  // a thread holds IPT * RL sums: 8 at 512 rows (512 threads, 64 registers,
  // two CTAs per SM), 16 elsewhere
  static constexpr int T = H == 2048 ? 512 : H == 1024 ? 256 : H == 768 || H == 384 ? 192 : H == 512 ? 512 : TOTAL_LAST;
  static constexpr int IPT = TOTAL_LAST / T;
  static constexpr int MINB = H == 2048 ? 1 : H <= 256 ? 3 : 2;  // shared memory: one CTA per SM at 2048 rows
  static_assert(TOTAL_LAST % T == 0, "every thread owns the same last-pass outputs");
  static constexpr size_t smem() { return (3 * (size_t)H * CS + H) * sizeof(float2) + 16; }
};

// DCT2: the band sum leaves as its DCT-II down the columns (what the spectral
// pyramid's synthesis takes next, k_dct.cu's kDct2 column pass): the column
// IFFT's last pass stores in the DCT-II's input order, a forward FFT and the
// DCT-II post-processing (wd) follow in shared memory.
template <int H, bool DCT2>
__global__ void __launch_bounds__(RaccCfg<H>::T, RaccCfg<H>::MINB)
    k_band_synthesis_racc(const __grid_constant__ CUtensorMap amap, const ColJob* __restrict__ jobs, int n_active,
                          int WH, float2* dst_base, const float2* __restrict__ spec_base, int spec_row0,
                          size_t band_stride, const float2* __restrict__ twH, const float2* __restrict__ wd,
                          int* err, int per_level) {
  using C = RaccCfg<H>;
  constexpr int CS = C::CS, T = C::T, RL = C::RL, IPT = C::IPT;
  extern __shared__ __align__(1024) float2 tsm[];
  float2* A = tsm;           // transform, in place
  float2* P = A + H * CS;    // the band's column group [row][column]
  float2* Wc = P + H * CS;   // the band's spectrum column group [row][column]
  float2* D = Wc + H * CS;   // column 0 of the band's transform
  const uint32_t bars = smem_u32(D + H);
  const ColBlock cb = col_block<CS>(per_level);
  const ColJob job = jobs[cb.job];
  if (job.item >= n_active) return;
  const int col0 = cb.col0;
  const bool dc = col0 == 0;
  const int band_rows = (int)(band_stride / WH);
  const int brow = (int)(job.src / WH), srow = spec_row0 + (int)(job.spec / WH);
  ColTma<H, CS> tp{bars, col0}, tw{bars + 8, col0};
  if (threadIdx.x == 0 && job.nbands > 0) {
    tp.init();
    tw.init();
    tp.expect(1);
    tp.load(&amap, P, brow);
    tw.expect(1);
    tw.load(&amap, Wc, srow);
  }
  __syncthreads();  // the mbarriers are initialised before any thread waits on them
  float2 acc[IPT][RL];
#pragma unroll
  for (int it = 0; it < IPT; it++)
#pragma unroll
    for (int r = 0; r < RL; r++) acc[it][r] = make_float2(0.0f, 0.0f);
  for (int k = 0; k < job.nbands; k++) {
    tp.wait(err);
    // the first pass has read band k from P: band k + 1 may come in
    auto next = [&]() {
      if (threadIdx.x == 0 && tp.ok && k + 1 < job.nbands) tp.refill(&amap, P, brow + (k + 1) * band_rows);
    };
    auto spec_ready = [&]() { tw.wait(err); };
    auto accf = [&](int it, int r, int row, int s, float2 z) {
      acc[it][r] = cadd(acc[it][r], cmulc(z, Wc[row * CS + s]));
      if (dc && s == 0) D[row] = z;
    };
    fft_ld_acc_passes<H, CS, T, -1, 1, 0>(A, twH, SmemLd<CS>{P}, next, spec_ready, accf, typename C::Plan{});
    // every thread has read Wc (the last pass ends with a barrier)
    if (threadIdx.x == 0 && tw.ok && k + 1 < job.nbands) tw.refill(&amap, Wc, srow + (k + 1) * band_rows);
    if (dc && threadIdx.x % CS == 0) {  // + conj(M[u] X[-u]) on the packed DC/Nyquist column
      const float2* m0 = spec_base + job.m0 + (size_t)k * H;
#pragma unroll
      for (int it = 0; it < IPT; it++)
#pragma unroll
        for (int r = 0; r < RL; r++) {
          const int row = last_pass_row<H, CS, T, RL>(it, r);
          acc[it][r] = cadd(acc[it][r], cconj(cmul(__ldg(&m0[row]), D[(H - row) % H])));
        }
    }
  }
  // the level's band sum: one column IFFT, stored by its last pass; where the
  // plan's first radix is its last, the IFFT's first pass starts from the
  // registers (they hold its inputs), else the sum goes to A first.  With
  // DCT2, row r of the IFFT goes to element r / 2 (r even) or H - 1 - (r - 1)
  // / 2 (r odd) of the DCT-II's FFT input.
  auto st_dct = [&](int i, int sq, float2 v) { A[((i & 1) ? H - 1 - (i >> 1) : (i >> 1)) * CS + sq] = v; };
  const ColGlobalSt st_out{dst_base + job.dst + col0, WH};
  if constexpr (FirstRadix<typename C::Plan>::value == RL) {
    if constexpr (DCT2)
      block_fft_from_regs<H, CS, T, +1>(A, twH, acc, st_dct);
    else
      block_fft_from_regs<H, CS, T, +1>(A, twH, acc, st_out);
  } else {
    const int s = threadIdx.x % CS;
#pragma unroll
    for (int it = 0; it < IPT; it++)
#pragma unroll
      for (int r = 0; r < RL; r++) A[last_pass_row<H, CS, T, RL>(it, r) * CS + s] = acc[it][r];
    __syncthreads();
    if constexpr (DCT2)
      block_fft_hook_ip<H, CS, T, +1>(A, twH, SmemLd<CS>{A}, st_dct);
    else
      block_fft_hook_ip<H, CS, T, +1>(A, twH, SmemLd<CS>{A}, st_out);
  }
  if constexpr (DCT2) {
    block_fft_hook_ip<H, CS, T, -1>(A, twH, SmemLd<CS>{A}, SmemSt<CS>{A});
    dct2_cols_store<H, T>(A, dst_base + job.dst + col0, WH, wd);
  }
  tp.drain(err);
  tw.drain(err);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
constexpr size_t kBarBytes = 16;  // the mbarrier after the shared buffers

template <typename KernelT>
static cudaError_t opt_in_tma(KernelT k, size_t bytes) {
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  return e;
}

bool cols_tma_supported(int H, int WH) { return col_len_supported(H) && WH % col_tile(H) == 0 && WH % 2 == 0; }

cudaError_t prepare_cols_tma(int H) {
  switch (H) {
#define CASE(n)                                                                           \
  case n: {                                                                               \
    cudaError_t e = opt_in_tma(k_band_analysis_ml_tma<n, false>, AnaCfg<n>::smem() + kBarBytes); \
    if (e == cudaSuccess) e = opt_in_tma(k_band_analysis_ml_tma<n, true>, AnaCfg<n>::smem() + kBarBytes); \
    if (e == cudaSuccess) e = opt_in_tma(k_band_synthesis_tma<n>, SynCfg<n>::smem() + kBarBytes); \
    if (e == cudaSuccess) e = opt_in_tma(k_band_analysis_ml_p_tma<n>, AnaCfg<n>::smem() + kBarBytes); \
    if (e == cudaSuccess) e = opt_in_tma(k_band_synthesis_p_tma<n>, SynCfg<n>::smem() + kBarBytes); \
    if (e == cudaSuccess) e = opt_in_tma(k_band_synthesis_racc<n, false>, RaccCfg<n>::smem());       \
    if (e == cudaSuccess) e = opt_in_tma(k_band_synthesis_racc<n, true>, RaccCfg<n>::smem());        \
    return e;                                                                             \
  }
    NSST_COL_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_cols_tma(ColOp op, const void* amap, const ColJob* jobs, int njobs, int n_active, int H, int W,
                            float2* dst_base, const float2* spec_base, size_t spec_row0, size_t band_stride,
                            const float2* twH, int* err, cudaStream_t st, const float2* wd, int per_level) {
  const int WH = W / 2;
  if (njobs == 0) return cudaSuccess;
  if (op != ColOp::AnalysisLevel && op != ColOp::Synthesis && op != ColOp::AnalysisLevelPairs &&
      op != ColOp::SynthesisPairs && op != ColOp::SynthesisRegs && op != ColOp::SynthesisRegsDct2 &&
      op != ColOp::AnalysisLevelDct)
    return cudaErrorInvalidValue;
  if ((op == ColOp::SynthesisRegsDct2 || op == ColOp::AnalysisLevelDct) && !wd) return cudaErrorInvalidValue;
  if (band_stride % (size_t)WH != 0 || spec_row0 > (size_t)INT32_MAX) return cudaErrorInvalidValue;
  if (per_level < 0 || (per_level > 0 && njobs % per_level != 0)) return cudaErrorInvalidValue;
  count_launch();
  const CUtensorMap& m = *reinterpret_cast<const CUtensorMap*>(amap);
  const int sr = (int)spec_row0;
  switch (H) {
#define CASE(n)                                                                                                     \
  case n: {                                                                                                         \
    dim3 grid(WH / ColCfg<n>::CS, njobs);                                                                           \
    constexpr size_t sa = AnaCfg<n>::smem() + kBarBytes, ss = SynCfg<n>::smem() + kBarBytes;                        \
    if (op == ColOp::AnalysisLevel)                                                                                 \
      k_band_analysis_ml_tma<n, false><<<grid, AnaCfg<n>::T, sa, st>>>(m, jobs, n_active, WH, dst_base, spec_base,  \
                                                                       sr, band_stride, twH, wd, err, per_level);   \
    else if (op == ColOp::AnalysisLevelDct)                                                                         \
      k_band_analysis_ml_tma<n, true><<<grid, AnaCfg<n>::T, sa, st>>>(m, jobs, n_active, WH, dst_base, spec_base,   \
                                                                      sr, band_stride, twH, wd, err, per_level);    \
    else if (op == ColOp::AnalysisLevelPairs)                                                                       \
      k_band_analysis_ml_p_tma<n><<<grid, AnaCfg<n>::T, sa, st>>>(m, jobs, n_active, WH, dst_base, spec_base, sr,   \
                                                                  band_stride, twH, err, per_level);                \
    else if (op == ColOp::Synthesis)                                                                                \
      k_band_synthesis_tma<n><<<grid, SynCfg<n>::T, ss, st>>>(m, jobs, n_active, WH, dst_base, spec_base,           \
                                                              band_stride, twH, err, per_level);                    \
    else if (op == ColOp::SynthesisRegs)                                                                            \
      k_band_synthesis_racc<n, false><<<grid, RaccCfg<n>::T, RaccCfg<n>::smem(), st>>>(                             \
          m, jobs, n_active, WH, dst_base, spec_base, sr, band_stride, twH, wd, err, per_level);                    \
    else if (op == ColOp::SynthesisRegsDct2)                                                                        \
      k_band_synthesis_racc<n, true><<<grid, RaccCfg<n>::T, RaccCfg<n>::smem(), st>>>(                              \
          m, jobs, n_active, WH, dst_base, spec_base, sr, band_stride, twH, wd, err, per_level);                    \
    else                                                                                                            \
      k_band_synthesis_p_tma<n><<<grid, SynCfg<n>::T, ss, st>>>(m, jobs, n_active, WH, dst_base, spec_base,         \
                                                                band_stride, twH, err, per_level);                  \
    return cudaGetLastError();                                                                                      \
  }
    NSST_COL_SIZES(CASE)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace nsst
