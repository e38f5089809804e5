// Instantiations and launchers of the volume FFT pass (vol3d_pass.cuh) for
// the level sizes of the reference's padded grids: MarshalData.m pads 128
// to 132 (levels 132, 88, 44, 22) and 192 to 204 (204, 136, 68, 34), lengths
// with the prime factors 11 and 17.  A separate translation unit so that the
// library's files compile in parallel.
#include "vol3d_pass.cuh"

namespace nsst {

#define V3P_ODD_SIZES(X) X(22) X(34) X(44) X(68) X(88) X(132) X(136) X(204)

bool v3_pass_len_supported_odd(int n) {
  switch (n) {
#define CASE(n) case n:
    V3P_ODD_SIZES(CASE)
#undef CASE
    return true;
    default:
      return false;
  }
}

cudaError_t prepare_v3_pass_odd(int n) {
  const int sm = (int)(2 * (size_t)(n + 2) * kSeq * sizeof(float2));
  cudaError_t e = cudaSuccess;
  switch (n) {
#define ONE(n, d, l, s)                                                                                  \
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_v3_pass<n, d, l, s>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
#define CASE(n)            \
  case n:                  \
    V3P_COMBOS(ONE, n)     \
    return e;
    V3P_ODD_SIZES(CASE)
#undef CASE
#undef ONE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_v3_pass_odd(int N, int dir, int ld, int st, float2* out, const float2* in, const V3Pass& P,
                               const float2* tw, int nitems, cudaStream_t stream) {
  if (P.b_n <= 0 || P.a_n <= 0) return cudaErrorInvalidValue;
  const dim3 grid((unsigned)(P.a_n * ((P.b_n + kSeq - 1) / kSeq)), (unsigned)nitems);
  const size_t sm = 2 * (size_t)(N + 2) * kSeq * sizeof(float2);
  count_launch();
  switch (N) {
#define ONE(n, d, l, s)                                                    \
  if (dir == d && ld == l && st == s) {                                    \
    k_v3_pass<n, d, l, s><<<grid, kThreads, sm, stream>>>(out, in, P, tw); \
    return cudaGetLastError();                                             \
  }
#define CASE(n)            \
  case n:                  \
    V3P_COMBOS(ONE, n)     \
    return cudaErrorInvalidValue;
    V3P_ODD_SIZES(CASE)
#undef CASE
#undef ONE
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace nsst
