// Instantiations and launchers of the volume FFT pass (vol3d_pass.cuh) for
// the 2^a 3^b lengths; the lengths of the reference's padded grids (factors
// 11 and 17) are instantiated in k_vol3d_pass_odd.cu.
#include "vol3d_pass.cuh"

namespace nsst {

#define V3P_SIZES(X) X(16) X(24) X(32) X(48) X(64) X(72) X(96) X(128) X(144) X(192) X(216) X(256)

bool v3_pass_len_supported(int n) {
  switch (n) {
#define CASE(n) case n:
    V3P_SIZES(CASE)
#undef CASE
    return true;
    default:
      return v3_pass_len_supported_odd(n);
  }
}

cudaError_t prepare_v3_pass(int n) {
  const int sm = (int)(2 * (size_t)(n + 2) * kSeq * sizeof(float2));
  cudaError_t e = cudaSuccess;
  switch (n) {
#define ONE(n, d, l, s)                                                                                  \
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_v3_pass<n, d, l, s>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
#define CASE(n)            \
  case n:                  \
    V3P_COMBOS(ONE, n)     \
    return e;
    V3P_SIZES(CASE)
#undef CASE
#undef ONE
    default:
      return prepare_v3_pass_odd(n);
  }
}

cudaError_t launch_v3_pass(int N, int dir, int ld, int st, float2* out, const float2* in, const V3Pass& P,
                           const float2* tw, int nitems, cudaStream_t stream) {
  if (P.b_n <= 0 || P.a_n <= 0) return cudaErrorInvalidValue;
  if (v3_pass_len_supported_odd(N)) return launch_v3_pass_odd(N, dir, ld, st, out, in, P, tw, nitems, stream);
  const dim3 grid((unsigned)(P.a_n * ((P.b_n + kSeq - 1) / kSeq)), (unsigned)nitems);
  const size_t sm = 2 * (size_t)(N + 2) * kSeq * sizeof(float2);
  count_launch();
  switch (N) {
#define ONE(n, d, l, s)                                                 \
  if (dir == d && ld == l && st == s) {                                 \
    k_v3_pass<n, d, l, s><<<grid, kThreads, sm, stream>>>(out, in, P, tw); \
    return cudaGetLastError();                                          \
  }
#define CASE(n)            \
  case n:                  \
    V3P_COMBOS(ONE, n)     \
    return cudaErrorInvalidValue;
    V3P_SIZES(CASE)
#undef CASE
#undef ONE
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace nsst
