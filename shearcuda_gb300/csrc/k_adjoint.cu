// Adjoint (transpose) building blocks of the NSST for the hand-written
// backward pass.  The reference has no adjoint; these are the exact
// transposes of the forward operators:
//
// * pyramid step: the forward step reads x through a half-sample mirror
//   (symext.m:18-31) at taps r - M c0 + M a; its transpose is a zero-extended
//   full correlation with the unflipped filter over the extended domain
//   (k_atrous<F,0,true>), followed by folding the mirrored margins back onto
//   the image ("transposed extension"): g[i] = Z[i+E] + Z[E-1-i] + Z[2H-1-i+E].
// * threshold: the subgradient mask 1[|c| > t]; for the soft rule the
//   threshold's own gradient is -sum sign(c) g 1[|c| > t] (per band).
#include "internal.h"

namespace nsst {

// out[i][j] (+)= fold(Z1, E1) + fold(Z2, E2), each Z of size (H+2E) x (W+2E).
__global__ void k_fold(const __grid_constant__ FoldJobs jobs, int H, int W, int E1, int E2, int accumulate) {
  const FoldJob& job = jobs.j[blockIdx.y];
  const int W1 = W + 2 * E1, W2 = W + 2 * E2;
  const size_t total = (size_t)H * W;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx / W), j = (int)(idx % W);
    float acc = accumulate ? job.out[idx] : 0.0f;
    const float* zs[2] = {job.z1, job.z2};
    const int Es[2] = {E1, E2}, Ws[2] = {W1, W2};
#pragma unroll
    for (int z = 0; z < 2; z++) {
      const float* Z = zs[z];
      if (!Z) continue;
      const int E = Es[z], Wz = Ws[z], Hz = H + 2 * E;
      int qr[3] = {i + E, E - 1 - i, 2 * H - 1 - i + E};
      int qc[3] = {j + E, E - 1 - j, 2 * W - 1 - j + E};
#pragma unroll
      for (int a = 0; a < 3; a++) {
        if (qr[a] < 0 || qr[a] >= Hz || (a > 0 && (a == 1 ? i >= E : i < H - E))) continue;
#pragma unroll
        for (int b = 0; b < 3; b++) {
          if (qc[b] < 0 || qc[b] >= Wz || (b > 0 && (b == 1 ? j >= E : j < W - E))) continue;
          acc += Z[(size_t)qr[a] * Wz + qc[b]];
        }
      }
    }
    job.out[idx] = acc;
  }
}

cudaError_t launch_fold(const FoldJobs& jobs, int njobs, int H, int W, int E1, int E2, bool accumulate,
                        cudaStream_t st) {
  if (njobs == 0) return cudaSuccess;
  if (njobs > kMaxAtrousJobs) return cudaErrorInvalidValue;
  const size_t total = (size_t)H * W;
  int bx = (int)std::min<size_t>((total + 255) / 256, 1024);
  count_launch();
  k_fold<<<dim3(bx, njobs), 256, 0, st>>>(jobs, H, W, E1, E2, accumulate ? 1 : 0);
  return cudaGetLastError();
}

// Lowpass band: g_c = g * 1[|c| > t]; per-block partial of the soft
// threshold gradient -sum g sign(c) 1[|c| > t] into partials[slot0 + item*nblk + blk].
__global__ void k_lowpass_backward(const __grid_constant__ FoldJobs jobs, size_t n, const float* __restrict__ tau,
                                   int mode, float* __restrict__ partials, int slot0) {
  const FoldJob& job = jobs.j[blockIdx.y];  // z1 = c, z2 = g, out = g_c
  const float t = tau[0];
  float part = 0.0f;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const float c = job.z1[idx], g = job.z2[idx];
    const bool keep = fabsf(c) > t;
    job.out[idx] = keep ? g : 0.0f;
    if (mode == THRESH_SOFT && keep) part -= (c > 0.0f ? g : -g);  // -g sign(c)
  }
  __shared__ float red[32];
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) partials[slot0 + blockIdx.y * gridDim.x + blockIdx.x] = v;
  }
}

cudaError_t launch_lowpass_backward(const FoldJobs& jobs, int njobs, size_t n, const float* tau, int mode,
                                    float* partials, int slot0, int nblk, cudaStream_t st) {
  if (njobs == 0) return cudaSuccess;
  count_launch();
  k_lowpass_backward<<<dim3(nblk, njobs), 256, 0, st>>>(jobs, n, tau, mode, partials, slot0);
  return cudaGetLastError();
}

// grad_tau[b] (+)= sum of partials[b * stride + 0 .. cnt); one block per band,
// fixed summation order (deterministic).
__global__ void k_reduce_tau(const float* __restrict__ partials, int cnt, size_t stride, float* __restrict__ grad_tau,
                             int accumulate) {
  const int b = blockIdx.x;
  double part = 0.0;
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) part += partials[(size_t)b * stride + i];
  __shared__ double red[256];
  red[threadIdx.x] = part;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) grad_tau[b] = (float)(red[0] + (accumulate ? grad_tau[b] : 0.0f));
}

cudaError_t launch_reduce_tau(const float* partials, int count, size_t stride, int nbands, float* grad_tau,
                              bool accumulate, cudaStream_t st) {
  count_launch();
  k_reduce_tau<<<nbands, 256, 0, st>>>(partials, count, stride, grad_tau, accumulate ? 1 : 0);
  return cudaGetLastError();
}

// Copy the shared per-band thresholds into every item's threshold row.
__global__ void k_broadcast_tau(const float* __restrict__ tau, float* __restrict__ th, int nbands, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nbands * n; i += gridDim.x * blockDim.x)
    th[i] = tau[i % nbands];
}

cudaError_t launch_broadcast_tau(const float* tau, float* th, int nbands, int n, cudaStream_t st) {
  count_launch();
  k_broadcast_tau<<<std::max(1, std::min(64, (nbands * n + 255) / 256)), 256, 0, st>>>(tau, th, nbands, n);
  return cudaGetLastError();
}

}  // namespace nsst
