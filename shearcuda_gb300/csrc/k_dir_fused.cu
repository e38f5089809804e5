// Fused directional stage of the 2-D NSST: one thread-block cluster per
// (image, level) keeps every band on chip.
//
// The split pipeline (k_directional.cu) runs a band through three kernels
// and HBM: the analysis column IFFT writes it, the row pass reads and writes
// it, the synthesis column FFT reads it.  That is the reference's structure
// (shear_trans_cuda.cpp:228-233 materialises all bands of a level,
// inverse_shear_cuda.cpp:222-286 reads them back), with 16 bytes of band
// traffic per packed element and band.  Here a cluster of CL CTAs owns one
// (image, level) job and runs, per band k of the level:
//
//   1. W_k .* Y, column IFFT       each CTA a group of CS = W/2/CL columns;
//                                  Y (the level spectrum's group) staged once
//                                  per job by TMA; the last FFT pass stores
//                                  straight into the peers' row buffers
//                                  (distributed shared memory): the transpose
//   2. row C2R -> threshold -> R2C each CTA RS = H/CL rows; the packed-real
//                                  post-processing stores into the peers'
//                                  column buffers: the transpose back
//   3. column FFT, conj(W_k) .* X  the last pass accumulates into registers
//                                  (each thread owns the same outputs for
//                                  every band), so the band sum never leaves
//                                  the SM either
//
// and after the level's last band one column IFFT of the sum, stored to HBM.
// Per job the only HBM traffic is the level spectrum in (4 B/px) and the sum
// out (4 B/px): the 8N B per level of the fused design.  The filter spectra
// come through L2 (shared by every image of the size).
//
// Math and operation order are those of the split kernels: c_k =
// real(ifft2(W_k .* fft2(y))) (nsst_dec2.m:58), the threshold of
// nsst_HT.m:34-46 (or soft), y' = real(ifft2(sum_k conj(W_k) .* fft2(c'_k)))
// (nsst_rec2.m:27-33), on the packed half-spectrum layout described in
// k_directional.cu.
//
// Synchronisation: two cluster barriers per band (after each transpose);
// a CTA writes into a peer's buffer only after the barrier that ends the
// peer's last read of it.  Every CTA of a cluster runs the same job sequence,
// so every barrier is reached by all of them.  The only wait that is not a
// hardware barrier is the TMA completion wait, bounded by an iteration limit
// after which the kernel records an error code and carries on (its output is
// then invalid, the host reports the error).
#include <cuda.h>

#include "internal.h"
#include "tiles.cuh"
#include "tma.cuh"

namespace nsst {

// ------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_id_x() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t ncluster_x() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
// all threads of all CTAs of the cluster; release/acquire orders the
// distributed-shared-memory stores before it against the loads after it
__device__ __forceinline__ void cluster_barrier() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n"
      "barrier.cluster.wait.acquire.aligned;\n" ::
          : "memory");
}
// address of the same shared-memory location in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t mapa(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ void st_cluster(uint32_t addr, float2 v) {
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(v.x), "f"(v.y) : "memory");
}
// ------------------------------------------------------------ configuration
// H rows, WH packed columns (W/2), CL CTAs per cluster, T threads per CTA;
// the row transforms use radix plan RowPlan (chosen so that every pass gives
// every thread work).
template <int H, int WH, int CL, int T, class RowPlan, class ColPlan>
struct FusedCfg {
  static constexpr int CS = WH / CL;  // columns per CTA (column phases)
  static constexpr int RS = H / CL;   // rows per CTA (row phase)
  static constexpr int RP = WH + 1;   // row pitch of the row buffer (odd: conflict-free column access)
  static constexpr int BH = tma_box_rows(H);  // rows per TMA box (box dims <= 256)
  static constexpr int NBOX = H / BH;
  static constexpr int RL = LastRadix<ColPlan>::value;  // last column pass radix
  static constexpr int TOTAL_LAST = (H / RL) * CS;
  static constexpr int IPT_LAST = TOTAL_LAST / T;
  static_assert(plan_product(RowPlan{}) == WH && plan_product(ColPlan{}) == H, "radix plans must multiply to N");
  static_assert(WH % CL == 0 && H % CL == 0, "cluster must divide the tile");
  static_assert(CS % 2 == 0, "TMA inner extent must be a multiple of 16 bytes");
  static_assert(TOTAL_LAST % T == 0, "last column pass must give every thread the same outputs");
  static_assert(BH <= 256 && H % BH == 0, "TMA box");
  // shared memory (float2 units): Y | column buffer | row buffer | DC column | mbarrier
  static constexpr size_t y_off = 0;
  static constexpr size_t c_off = (size_t)H * CS;
  static constexpr size_t r_off = 2 * (size_t)H * CS;
  static constexpr size_t r_elems = (size_t)RS * RP > (size_t)WH * RS ? (size_t)RS * RP : (size_t)WH * RS;
  static constexpr size_t d_off = r_off + ((r_elems + 15) / 16) * 16;
  static constexpr size_t b_off = d_off + H;
  static constexpr size_t smem() { return (b_off + 2) * sizeof(float2); }
};

// row-major row buffer with pitch RP: C2R pre-processing in the first pass's loads
template <int WH, int RP>
struct C2RPreLdRP {
  const float2* X;
  const float2* twW;
  __device__ __forceinline__ float2 operator()(int k, int s) const {
    const float2* row = X + s * RP;
    const float2 xk = row[k];
    if (k == 0) return make_float2(xk.x + xk.y, xk.x - xk.y);
    const float2 xmc = cconj(row[WH - k]);
    const float2 E = cadd(xk, xmc);
    const float2 O = cmulc(csub(xk, xmc), __ldg(&twW[k]));
    return make_float2(E.x - O.y, E.y + O.x);
  }
};
template <int RP>
struct SmemStRP {  // element (i, s) -> row s, column i
  float2* p;
  __device__ __forceinline__ void operator()(int i, int s, float2 v) const { p[s * RP + i] = v; }
};

template <int N, int NSEQ, int T, int DIR, int NS, int SWZ_IN, class Acc, int R>
__device__ __forceinline__ void fft_ip_acc_passes(float2* buf, const float2* __restrict__ tw, Acc& acc,
                                                  RadixList<R>) {
  auto rd = [&](int row, int s) -> float2 { return buf[row * NSEQ + s]; };
  stockham_last_acc<N, NSEQ, T, R, NS, DIR, SWZ_IN>(rd, acc, tw);
}
template <int N, int NSEQ, int T, int DIR, int NS, int SWZ_IN, class Acc, int R, int R2, int... Rest>
__device__ __forceinline__ void fft_ip_acc_passes(float2* buf, const float2* __restrict__ tw, Acc& acc,
                                                  RadixList<R, R2, Rest...>) {
  constexpr int SWZ_OUT = (NS == 1 && R % 2 == 0) ? R : 0;
  auto rd = [&](int row, int s) -> float2 { return buf[row * NSEQ + s]; };
  auto wr = [&](int row, int s, float2 v) { buf[row * NSEQ + s] = v; };
  stockham_ip<N, NSEQ, T, R, NS, DIR, SWZ_IN, SWZ_OUT>(rd, wr, tw);
  fft_ip_acc_passes<N, NSEQ, T, DIR, NS * R, SWZ_OUT>(buf, tw, acc, RadixList<R2, Rest...>{});
}
// ------------------------------------------------------------------ kernel
template <int H, int WH, int CL, int T, int MINB, class RowPlan, class ColPlan>
__global__ void __launch_bounds__(T, MINB)
    k_dir_fused(const __grid_constant__ CUtensorMap ymap, const FusedJob* __restrict__ jobs, int njobs, int n_active,
                float2* dst_base, const float2* __restrict__ spec_base, size_t band_stride,
                const float2* __restrict__ twH, const float2* __restrict__ twWh, const float2* __restrict__ twW,
                const float* __restrict__ thr, int mode, int* err) {
  using C = FusedCfg<H, WH, CL, T, RowPlan, ColPlan>;
  constexpr int CS = C::CS, RS = C::RS, RP = C::RP, RL = C::RL, IPT = C::IPT_LAST;
  extern __shared__ __align__(128) float2 smem[];
  float2* Y = smem + C::y_off;       // level spectrum, the CTA's column group [row][column]
  float2* colbuf = smem + C::c_off;  // column phases, [row][column], in place
  float2* rowbuf = smem + C::r_off;  // row phase: row-major (pitch RP), dense [index][row] between passes
  float2* D = smem + C::d_off;       // column 0 of the band's column FFT (rank 0)
  const uint32_t rank = cluster_ctarank();
  const int cid = (int)cluster_id_x(), ncl = (int)ncluster_x();
  const int col0 = (int)rank * CS;
  const bool dc = rank == 0;
  const uint32_t bar = smem_u32(smem + C::b_off), y_a = smem_u32(Y), row_a = smem_u32(rowbuf);
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  auto next_active = [&](int j) {
    while (j < njobs && jobs[j].item >= n_active) j += ncl;
    return j;
  };
  // thread 0: the level spectrum's column group of job jj -> Y (NBOX boxes of BH rows)
  bool tma_ok = true;  // false after a timed-out wait: no further TMA is issued
  auto issue = [&](int jj) {
    const int row0 = jobs[jj].ymap_row;
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(bar, (uint32_t)(H * CS * sizeof(float2)));
#pragma unroll
    for (int b = 0; b < C::NBOX; b++)
      tma_load_2d(y_a + (uint32_t)(b * C::BH * CS * sizeof(float2)), &ymap, col0, row0 + b * C::BH, bar);
  };
  uint32_t phase = 0;
  int j = next_active(cid);
  bool inflight = false;
  if (j < njobs && threadIdx.x == 0) issue(j);
  inflight = j < njobs;

  while (j < njobs) {
    const FusedJob job = jobs[j];
    const int jn = next_active(j + ncl);
    if (!mbar_wait_bounded(bar, phase, err)) tma_ok = false;
    phase ^= 1u;
    inflight = false;
    float2 acc[IPT][RL];
#pragma unroll
    for (int it = 0; it < IPT; it++)
#pragma unroll
      for (int r = 0; r < RL; r++) acc[it][r] = make_float2(0.0f, 0.0f);

    for (int k = 0; k < job.nbands; k++) {
      const float2* Wk = spec_base + job.spec + (size_t)k * band_stride + col0;
      const float2* Mk = spec_base + job.m0 + (size_t)k * H;
      // 1. W_k .* Y (packed DC/Nyquist column: + M conj(Y[-u])), column IFFT;
      //    the last pass stores into the owner's row buffer
      auto ld = [&](int i, int s) -> float2 {
        float2 r = cmul(__ldg(&Wk[(size_t)i * WH + s]), Y[i * CS + s]);
        if (dc && s == 0) r = cadd(r, cmul(__ldg(&Mk[i]), cconj(Y[((H - i) % H) * CS])));
        return r;
      };
      auto st = [&](int i, int s, float2 v) {
        const uint32_t local = row_a + (uint32_t)(((i % RS) * RP + col0 + s) * (int)sizeof(float2));
        st_cluster(mapa(local, (uint32_t)(i / RS)), v);
      };
      const bool last_band = k + 1 == job.nbands;
      // once every thread has read Y for the last band, the next job's level spectrum may stream in
      auto after_read = [&]() {
        if (last_band && threadIdx.x == 0 && jn < njobs && tma_ok) issue(jn);
      };
      block_fft_hook_ip_plan<H, CS, T, +1, ColPlan>(colbuf, twH, ld, st, after_read);
      if (last_band) inflight = jn < njobs && tma_ok;
      cluster_barrier();

      // 2. rows: C2R -> threshold -> R2C, post-processing stored into the owner's column buffer
      const float th = thr[job.th0 + k];
      block_fft_hook_ip_plan<WH, RS, T, +1, RowPlan>(rowbuf, twWh, C2RPreLdRP<WH, RP>{rowbuf, twW},
                                                     ThreshSt<RS>{rowbuf, th, mode});
      block_fft_hook_ip_plan<WH, RS, T, -1, RowPlan>(rowbuf, twWh, SmemLd<RS>{rowbuf}, SmemStRP<RP>{rowbuf});
      {
        const uint32_t col_a = smem_u32(colbuf);
#pragma unroll 4
        for (int e = threadIdx.x; e < WH * RS; e += T) {
          const int kk = e % WH, s = e / WH;
          const float2* row = rowbuf + s * RP;
          const float2 zk = row[kk];
          float2 out;
          if (kk == 0) {
            out = make_float2(zk.x + zk.y, zk.x - zk.y);
          } else {
            const float2 zmc = cconj(row[WH - kk]);
            const float2 E = cscale(cadd(zk, zmc), 0.5f);
            const float2 d = cscale(csub(zk, zmc), 0.5f);
            const float2 To = cmul(__ldg(&twW[kk]), make_float2(d.y, -d.x));
            out = cadd(E, To);
          }
          const int grow = (int)rank * RS + s;
          const uint32_t local = col_a + (uint32_t)((grow * CS + kk % CS) * (int)sizeof(float2));
          st_cluster(mapa(local, (uint32_t)(kk / CS)), out);
        }
      }
      cluster_barrier();

      // 3. column FFT; conj(W_k) .* X accumulated in registers
      auto accf = [&](int it, int r, int row, int s, float2 z) {
        acc[it][r] = cadd(acc[it][r], cmulc(z, __ldg(&Wk[(size_t)row * WH + s])));
        if (dc && s == 0) D[row] = z;
      };
      fft_ip_acc_passes<H, CS, T, -1, 1, 0>(colbuf, twH, accf, ColPlan{});
      if (dc && threadIdx.x % CS == 0) {  // + conj(M[u] X[-u]) on the packed DC/Nyquist column
#pragma unroll
        for (int it = 0; it < IPT; it++)
#pragma unroll
          for (int r = 0; r < RL; r++) {
            const int row = last_pass_row<H, CS, T, RL>(it, r);
            acc[it][r] = cadd(acc[it][r], cconj(cmul(__ldg(&Mk[row]), D[(H - row) % H])));
          }
      }
    }
    // the level's band sum: one column IFFT, stored to HBM
    {
      const int s = threadIdx.x % CS;
#pragma unroll
      for (int it = 0; it < IPT; it++)
#pragma unroll
        for (int r = 0; r < RL; r++) colbuf[last_pass_row<H, CS, T, RL>(it, r) * CS + s] = acc[it][r];
    }
    __syncthreads();
    block_fft_hook_ip_plan<H, CS, T, +1, ColPlan>(colbuf, twH, SmemLd<CS>{colbuf},
                                                  ColGlobalSt{dst_base + job.dst + col0, WH});
    j = jn;
  }
  // a copy still in flight (only after a timed-out wait) must land before the CTA exits
  if (inflight) mbar_wait_bounded(bar, phase, err);
  // no CTA leaves while a peer may still address its shared memory
  cluster_barrier();
}

// --------------------------------------------------------------- launchers
// (H, W/2) -> cluster size and threads: see FusedCfg; shared memory per CTA:
// 512 x 512: 196 KB (one CTA per SM), 384 x 512: 147 KB, 256 x 256: 98 KB (two per SM).
using P884 = RadixList<8, 8, 4>;
using P888 = RadixList<8, 8, 8>;
using P168 = RadixList<16, 8>;
using P1616 = RadixList<16, 16>;
using P3448 = RadixList<3, 4, 4, 8>;
#define NSST_FUSED_CONFIGS(X)                                                                         \
  X(512, 256, 16, 512, 1, P1616, P888) X(384, 256, 16, 384, 1, P1616, P3448) \
  X(256, 128, 8, 256, 2, P168, P1616)

bool dir_fused_supported(int H, int WH) {
#define CASE(h, wh, cl, t, mb, rp, cp) \
  if (H == h && WH == wh) return true;
  NSST_FUSED_CONFIGS(CASE)
#undef CASE
  return false;
}

int dir_fused_cluster(int H, int WH) {
#define CASE(h, wh, cl, t, mb, rp, cp) \
  if (H == h && WH == wh) return cl;
  NSST_FUSED_CONFIGS(CASE)
#undef CASE
  return 0;
}

template <int H, int WH, int CL, int T, int MB, class RP, class CP>
static cudaError_t prepare_fused_t(int* max_clusters) {
  using C = FusedCfg<H, WH, CL, T, RP, CP>;
  auto kern = k_dir_fused<H, WH, CL, T, MB, RP, CP>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::smem());
  if (e == cudaSuccess && CL > 8) e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL * 64);
  cfg.blockDim = dim3(T);
  cfg.dynamicSmemBytes = C::smem();
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  e = cudaOccupancyMaxActiveClusters(&n, (const void*)kern, &cfg);
  *max_clusters = e == cudaSuccess ? n : 0;
  return e;
}

cudaError_t prepare_dir_fused(int H, int WH, int* max_clusters) {
  *max_clusters = 0;
#define CASE(h, wh, cl, t, mb, rp, cp) \
  if (H == h && WH == wh) return prepare_fused_t<h, wh, cl, t, mb, rp, cp>(max_clusters);
  NSST_FUSED_CONFIGS(CASE)
#undef CASE
  return cudaErrorInvalidValue;
}

// 2-D tensor map over rows of `inner` 8-byte elements (one float2 each), row
// pitch inner * 8 bytes, starting at base; box = (box_x elements, box_y rows).
cudaError_t make_tmap_2d(void* out, const void* base, int inner, size_t rows, int box_x, int box_y) {
  using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static EncodeFn encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess) return e;
    if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorNotSupported;
    encode = reinterpret_cast<EncodeFn>(fn);
  }
  // 16-byte base and pitch, inner box extent a multiple of 16 bytes, box dims <= 256
  if (((uintptr_t)base & 15) != 0 || inner % 2 != 0 || box_x % 2 != 0 || box_x > 256 || box_y > 256 || box_x < 2 ||
      box_y < 1 || rows == 0)
    return cudaErrorInvalidValue;
  cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)inner * sizeof(float2)};
  cuuint32_t box[2] = {(cuuint32_t)box_x, (cuuint32_t)box_y};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode(reinterpret_cast<CUtensorMap*>(out), CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<void*>(base),
                      dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Tensor map over the level spectra of a plan: rows x WH float2, box = (columns
// of one CTA of the cluster, tma_box_rows(H) rows).
cudaError_t make_level_tmap(void* out, const float2* lev, int H, int WH, size_t rows) {
  const int cl = dir_fused_cluster(H, WH);
  if (cl == 0) return cudaErrorInvalidValue;
  return make_tmap_2d(out, lev, WH, rows, WH / cl, tma_box_rows(H));
}

template <int H, int WH, int CL, int T, int MB, class RP, class CP>
static cudaError_t launch_fused_t(const void* ymap, const FusedJob* jobs, int njobs, int n_active, int nclusters,
                                  float2* dst_base, const float2* spec_base, size_t band_stride, const float2* twH,
                                  const float2* twWh, const float2* twW, const float* thr, int mode, int* err,
                                  cudaStream_t st) {
  using C = FusedCfg<H, WH, CL, T, RP, CP>;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL * nclusters);
  cfg.blockDim = dim3(T);
  cfg.dynamicSmemBytes = C::smem();
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const CUtensorMap& m = *reinterpret_cast<const CUtensorMap*>(ymap);
  return cudaLaunchKernelEx(&cfg, k_dir_fused<H, WH, CL, T, MB, RP, CP>, m, jobs, njobs, n_active, dst_base, spec_base,
                            band_stride, twH, twWh, twW, thr, mode, err);
}

cudaError_t launch_dir_fused(const void* ymap, const FusedJob* jobs, int njobs, int n_active, int nclusters, int H,
                             int W, float2* dst_base, const float2* spec_base, size_t band_stride, const float2* twH,
                             const float2* twWh, const float2* twW, const float* thr, int mode, int* err,
                             cudaStream_t st) {
  if (njobs == 0 || nclusters <= 0) return cudaSuccess;
  count_launch();
  const int WH = W / 2;
#define CASE(h, wh, cl, t, mb, rp, cp)                                                                            \
  if (H == h && WH == wh)                                                                                         \
    return launch_fused_t<h, wh, cl, t, mb, rp, cp>(ymap, jobs, njobs, n_active, nclusters, dst_base, spec_base,         \
                                            band_stride, twH, twWh, twW, thr, mode, err, st);
  NSST_FUSED_CONFIGS(CASE)
#undef CASE
  return cudaErrorInvalidValue;
}

}  // namespace nsst
