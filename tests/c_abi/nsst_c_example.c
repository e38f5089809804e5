/* A C99 caller of libnsst through include/nsst.h alone: what a MEX gateway or
 * the reference's C++ demo does through the C ABI.  It denoises one seeded
 * synthetic image with the Monte-Carlo noise scalars, runs a Symmlet-4
 * undecimated wavelet round trip, and prints one line:
 *     checksum <sum of the denoised image> rdwt_err <max |x - mirdwt(mrdwt(x))|>
 * Built and run by tests/test_c_abi.py (compile on any machine, run on a GPU).
 * Usage: nsst_c_example H W */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime.h>

#include "nsst.h"

#define CHECK(call)                                                               \
  do {                                                                            \
    nsst_status s_ = (call);                                                      \
    if (s_ != NSST_OK) {                                                          \
      fprintf(stderr, "%s failed: %d %s\n", #call, (int)s_, nsst_last_error()); \
      return 1;                                                                   \
    }                                                                             \
  } while (0)
#define CUDA(call)                                                              \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      fprintf(stderr, "%s failed: %s\n", #call, cudaGetErrorString(e_));        \
      return 1;                                                                 \
    }                                                                           \
  } while (0)

/* the same image as the Python side's seeded ramp: x[r][c] = ((r * 7 + c * 13) % 101) */
static void fill(float* x, int H, int W) {
  for (int r = 0; r < H; r++)
    for (int c = 0; c < W; c++) x[(size_t)r * W + c] = (float)((r * 7 + c * 13) % 101);
}

int main(int argc, char** argv) {
  const int H = argc > 1 ? atoi(argv[1]) : 256, W = argc > 2 ? atoi(argv[2]) : 256;
  const size_t HW = (size_t)H * W;
  nsst_config cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.nlevels = 4;
  const int dcomp[4] = {3, 3, 4, 4}, dsize[4] = {32, 32, 16, 16};
  memcpy(cfg.dcomp, dcomp, sizeof dcomp);
  memcpy(cfg.dsize, dsize, sizeof dsize);
  strcpy(cfg.lpfilt, "maxflat");

  float* h = (float*)malloc(HW * sizeof(float));
  float* o = (float*)malloc(HW * sizeof(float));
  fill(h, H, W);
  float *dx = NULL, *dy = NULL, *yl = NULL, *yh = NULL;
  CUDA(cudaMalloc((void**)&dx, HW * sizeof(float)));
  CUDA(cudaMalloc((void**)&dy, HW * sizeof(float)));
  CUDA(cudaMalloc((void**)&yl, HW * sizeof(float)));
  CUDA(cudaMalloc((void**)&yh, 3 * 3 * HW * sizeof(float)));
  CUDA(cudaMemcpy(dx, h, HW * sizeof(float), cudaMemcpyHostToDevice));

  nsst_plan* plan = NULL;
  CHECK(nsst_plan_create(&cfg, H, W, &plan));
  CHECK(nsst_compute_scalars(plan, 4321, NULL));
  const double K[5] = {0, 3, 3, 3, 4};
  CHECK(nsst_denoise(plan, dx, dy, 20.0, K, NULL, NSST_THRESH_HARD, NULL));
  CUDA(cudaMemcpy(o, dy, HW * sizeof(float), cudaMemcpyDeviceToHost));
  double sum = 0.0;
  for (size_t i = 0; i < HW; i++) sum += o[i];

  double qmf[NSST_MAX_QMF];
  int lq = 0;
  CHECK(nsst_onfilter("Symmlet", 4, qmf, &lq));
  CHECK(nsst_mrdwt(dx, 1, H, W, qmf, lq, 3, yl, yh, NULL));
  CHECK(nsst_mirdwt(yl, yh, 1, H, W, qmf, lq, 3, dy, NULL));
  CUDA(cudaMemcpy(o, dy, HW * sizeof(float), cudaMemcpyDeviceToHost));
  double err = 0.0;
  for (size_t i = 0; i < HW; i++) err = fmax(err, fabs((double)o[i] - (double)h[i]));

  CHECK(nsst_plan_destroy(plan));
  cudaFree(dx);
  cudaFree(dy);
  cudaFree(yl);
  cudaFree(yh);
  free(h);
  free(o);
  printf("checksum %.6f rdwt_err %.3e\n", sum, err);
  return 0;
}
