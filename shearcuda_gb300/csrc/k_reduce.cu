// Per-plane reductions over coefficient planes: sums of squares in FP64
// partials (exact band norms, com_norm.m:45-51 / norm_cuda.cpp:57-215) and
// the largest magnitude (thresh_cuda's opt == 1, thresh_cuda.cpp:199-205).
// Both are deterministic: fixed-order partials reduced on the host, and a
// maximum of non-negative floats through their bit patterns.
#include "internal.h"

namespace nsst {

constexpr int kRedThreads = 256;

// partial[plane * gridDim.x + block] = sum of x^2 over the block's share of the plane
__global__ void __launch_bounds__(kRedThreads) k_plane_sumsq(const float* __restrict__ data, size_t n,
                                                            double* __restrict__ partial) {
  __shared__ double red[kRedThreads / 32];
  const float* x = data + (size_t)blockIdx.y * n;
  double s = 0.0;
  for (size_t i = (size_t)blockIdx.x * kRedThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kRedThreads) {
    const double v = x[i];
    s += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kRedThreads / 32; w++) t += red[w];
    partial[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = t;
  }
}

// maxbits[plane] = max over the plane of the bit pattern of |x| (monotone for
// non-negative floats); maxbits must start at 0
__global__ void __launch_bounds__(kRedThreads) k_plane_maxabs(const float* __restrict__ data, size_t n,
                                                             unsigned* __restrict__ maxbits) {
  const float* x = data + (size_t)blockIdx.y * n;
  float m = 0.0f;
  for (size_t i = (size_t)blockIdx.x * kRedThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kRedThreads)
    m = fmaxf(m, fabsf(x[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(&maxbits[blockIdx.y], __float_as_uint(m));
}

// data[plane][i] *= w[plane]
__global__ void k_scale_planes(float* __restrict__ data, size_t n, PlaneWeights w) {
  float* x = data + (size_t)blockIdx.y * n;
  const float s = w.w[blockIdx.y];
  for (size_t i = (size_t)blockIdx.x * kRedThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kRedThreads)
    x[i] *= s;
}

cudaError_t launch_scale_planes(float* data, size_t n, int nplanes, const PlaneWeights& w, cudaStream_t st) {
  if (nplanes > kMaxPlaneWeights) return cudaErrorInvalidValue;
  count_launch();
  k_scale_planes<<<dim3(64, nplanes), kRedThreads, 0, st>>>(data, n, w);
  return cudaGetLastError();
}

cudaError_t launch_plane_sumsq(const float* data, size_t n, int nplanes, double* partial, int blocks,
                               cudaStream_t st) {
  count_launch();
  k_plane_sumsq<<<dim3(blocks, nplanes), kRedThreads, 0, st>>>(data, n, partial);
  return cudaGetLastError();
}

cudaError_t launch_plane_maxabs(const float* data, size_t n, int nplanes, unsigned* maxbits, int blocks,
                                cudaStream_t st) {
  count_launch();
  k_plane_maxabs<<<dim3(blocks, nplanes), kRedThreads, 0, st>>>(data, n, maxbits);
  return cudaGetLastError();
}

}  // namespace nsst
