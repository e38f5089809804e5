/* nsst.h — C ABI of the GB300-native NSST engine (libnsst.so).
 *
 * Drop-in boundary for the 2-D nonsubsampled shearlet transform hot path of
 * ShearCuda: decompose -> hard/soft threshold -> reconstruct.  Each entry point
 * names the reference interface it replaces (paths relative to the ShearCuda
 * tree).  All pointers passed as "device" are CUDA device pointers; `stream`
 * is a cudaStream_t (NULL = legacy default stream).  Images are row-major
 * float32, H rows x W columns, W fastest.  No call aborts the process: every
 * call returns an nsst_status and nsst_last_error() describes the last
 * failure on the calling thread.
 *
 * Coefficient layout (nsst_shear_trans / nsst_thresh / nsst_inverse_shear):
 * nbands = 1 + sum_i 2^dcomp[i] planes of H x W floats; plane 0 is the
 * lowpass image, then level 0 (coarsest) directions 0..2^dcomp[0]-1, level 1,
 * ... — the MATLAB cell {lowpass, L x L x ndir per scale} of
 * shear_trans_cuda.cpp:207-216 flattened level-major, direction-minor.
 */
#ifndef NSST_H
#define NSST_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum nsst_status {
  NSST_OK = 0,
  NSST_ERR_INVALID_ARG = 1,      /* bad pointer, size or parameter */
  NSST_ERR_UNSUPPORTED_SIZE = 2, /* H/W outside the supported transform lengths */
  NSST_ERR_OUT_OF_MEMORY = 3,    /* device or host allocation failed */
  NSST_ERR_CUDA = 4,             /* a CUDA runtime call failed */
  NSST_ERR_TIMEOUT = 5,          /* a bounded device-side wait ran out */
  NSST_ERR_NUMERIC = 6           /* e.g. filter normalisation divides by zero */
} nsst_status;

enum { NSST_THRESH_HARD = 0, NSST_THRESH_SOFT = 1 };
enum { NSST_PYRAMID_AUTO = 0, NSST_PYRAMID_DIRECT = 1, NSST_PYRAMID_SPECTRAL = 2 };
enum { NSST_MAX_LEVELS = 8, NSST_MAX_BANDS = 1 + 8 * 64 };

/* Transform configuration.  Mirrors the reference's shear_parameters struct
 * (nsst_dec2.m:11-20: .dcomp, .dsize) plus the pyramid filter name
 * (atrousfilters.m:26: '9-7' | 'maxflat' | 'pyr' | 'pyrexc'). */
typedef struct nsst_config {
  int nlevels;                  /* length of dcomp/dsize (<= NSST_MAX_LEVELS) */
  int dcomp[NSST_MAX_LEVELS];   /* level i has 2^dcomp[i] directions, coarse -> fine */
  int dsize[NSST_MAX_LEVELS];   /* local support of level i's shearing filter */
  char lpfilt[16];              /* pyramid filter name, NUL-terminated */
  int pyramid;                  /* how nsst_denoise(_batch) runs the pyramid:
                                   _DIRECT: dilated direct convolutions;
                                   _SPECTRAL: in the 2-D DCT-II domain, where each
                                   atrousdec.m / atrousrec.m step is a pointwise
                                   product merged into the directional FFT passes
                                   (same results to FP32 rounding; needs pyramid
                                   filters symmetric in both axes, as all of
                                   atrousfilters.m's sets are, else the plan is
                                   rejected); _AUTO: spectral where the filters
                                   allow it.  nsst_shear_trans,
                                   nsst_inverse_shear, nsst_atrousdec,
                                   nsst_atrousrec, the differentiable denoise
                                   (forward and backward) and the separation
                                   follow the same mode; calls that pass images
                                   not 16-byte aligned, nsst_re_weight_band and
                                   the operator adjoints use the direct pyramid. */
} nsst_config;

typedef struct nsst_plan nsst_plan;

/* Last error message of the calling thread ("" if none). */
const char* nsst_last_error(void);

/* Library version string. */
const char* nsst_version(void);

/* Build a transform plan for H x W images: pyramid filters, Meyer shearing
 * filters and their normalised spectra are constructed in FP64 on the host
 * and uploaded as FP32; work buffers are allocated once here.
 * Replaces prepare_shearing_filters_cuda (prepare_shearing_filters_cuda.cpp:61-249)
 * and the standalone GpuShearDictionary::prepare (demo_denoise/shearcuda/gpusheardictionary.cpp:54-147). */
nsst_status nsst_plan_create(const nsst_config* cfg, int H, int W, nsst_plan** out);

/* Like nsst_plan_create, with work buffers for up to B images of this size
 * processed together by nsst_denoise_batch (the filter spectra are shared). */
nsst_status nsst_plan_create_batch(const nsst_config* cfg, int H, int W, int B, nsst_plan** out);

/* The reference's shearing-filter bank file, "SHFM0002" (little-endian): the
 * magic, uint16 number of scales, uint16 data type (NSST_DATA_SINGLE 0 or
 * NSST_DATA_DOUBLE 2), per scale uint16 filter size n and uint16 number of
 * directions d followed by d n x n filters in MATLAB column-major order, then
 * the four pyramid filters h0, h1, g0, g1 as uint16 size F and F x F values.
 * nsst_filters_save writes the bank of `cfg` (the Meyer shearing filters of
 * shearing_filters_Myer.m and the pyramid filters named in cfg->lpfilt);
 * replaces save_shearing_filters.m:46-84. */
enum { NSST_DATA_SINGLE = 0, NSST_DATA_DOUBLE = 2 };
nsst_status nsst_filters_save(const char* path, const nsst_config* cfg, int data_type);

/* Read an SHFM0002 file: nlevels, and per level dsize / ndir (arrays of
 * NSST_MAX_LEVELS), F[4], the shearing filters (sum_l ndir*dsize^2 doubles,
 * row-major, level after level) and the pyramid filters (sum_k F[k]^2
 * doubles, row-major); every output but nlevels may be NULL.  Replaces
 * ShearConfig::readFromFile (demoImageDenoise/shearconfig.cpp:26-78). */
nsst_status nsst_filters_load(const char* path, int* nlevels, int* dsize, int* ndir, int* F, double* shear,
                              double* pyramid, int* data_type);

/* A plan whose shearing filters and pyramid filters come from an SHFM0002
 * file instead of being constructed (dcomp = log2 of each scale's direction
 * count, dsize = its filter size; the spectra are normalised as
 * nsst_dec2.m:47-57 does).  With the library's own bank saved as doubles the
 * plan is identical to nsst_plan_create_batch's. */
nsst_status nsst_plan_create_from_file(const char* path, int H, int W, int B, nsst_plan** out);

/* Batch capacity B of a plan. */
int nsst_plan_batch_capacity(const nsst_plan* plan);

/* Replay nsst_denoise_batch's launch sequence as a CUDA graph (captured on
 * the first call with a given set of image pointers; thresholds stay a
 * per-call upload).  enable = 0 launches kernels one by one. */
nsst_status nsst_plan_use_graphs(nsst_plan* plan, int enable);

/* How nsst_denoise(_batch) runs the directional stage (analysis W_k .* Y and
 * column IFFT, row C2R -> threshold -> R2C, synthesis column FFT and
 * conj(W_k) sum; nsst_dec2.m:58, nsst_HT.m:34-46, nsst_rec2.m:27-33):
 *   _SPLIT: three kernels, every band plane through device memory, as the
 *           reference's shear_trans_cuda.cpp:228-233 / inverse_shear_cuda.cpp:222-286
 *           materialise them;
 *   _FUSED: one thread-block cluster per (image, level) keeps the bands on
 *           chip (distributed shared memory); sizes 256x256, 384x512, 512x512;
 *   _AUTO:  the autotuner's choice for the call's batch size
 *           (nsst_plan_autotune), fused where untuned and available.
 * The results agree to FP32 rounding.  Setting a mode drops the captured
 * graphs.  NSST_ERR_UNSUPPORTED_SIZE if _FUSED has no configuration here. */
enum { NSST_DIRECTIONAL_AUTO = 0, NSST_DIRECTIONAL_SPLIT = 1, NSST_DIRECTIONAL_FUSED = 2 };
nsst_status nsst_plan_set_directional(nsst_plan* plan, int mode);

/* The implementation (NSST_DIRECTIONAL_SPLIT or _FUSED) a call of n items
 * runs; -1 for a NULL plan or n < 1. */
int nsst_plan_directional(const nsst_plan* plan, int n);

/* Autotuner.  Times every implementation of the directional stage this plan
 * can run on n synthetic images (median of 7 passes after 2 warm-ups, CUDA
 * events): the split kernels with each analysis variant (one CTA per band and
 * column group, or per level streaming all its bands), row tiles, and one
 * complex value per thread or split-complex pairs of rows or columns whose
 * arithmetic runs as FP32x2 instructions ("-pairs"), and
 * the fused cluster kernel where the size has one; the fastest becomes the
 * choice of NSST_DIRECTIONAL_AUTO for batches in n's bucket (2^b <= n <
 * 2^(b+1)) and the captured graphs are dropped.  It also evaluates direct
 * (spatial) directional convolution, the alternative the reference offers
 * nowhere on the GPU: the effective spatial filter of a band is
 * ifft2(W_k / d) (nsst_dec2.m:47-57), which the normalisation by d spreads
 * beyond the shearing filter's dsize support, so per level it finds the
 * smallest square window around that support that keeps every band's
 * truncation error <= 1e-5 relative L2 (0: none smaller than the image), and
 * the lower bound of a direct convolution with it (support^2 FMAs per pixel
 * and band, each way, at the FP32 FMA peak).  direct_wins is the verdict of
 * the rule "every level has a window and the bound beats the fastest measured
 * candidate"; no direct directional kernel is built, so the FFT candidates
 * run whatever it says (at 256^2 .. 512^2 with dsize [32 32 16 16] the
 * windows are 110-204 px and the bound is ~200x the FFT path's time).
 * Synchronous; allocates 2 n images for the run. */
enum { NSST_TUNE_MAX_CANDIDATES = 32 };
typedef struct nsst_tune_result {
  int n;                                     /* batch size timed */
  int ncand;                                 /* candidates timed */
  int chosen;                                /* index of the fastest */
  char name[NSST_TUNE_MAX_CANDIDATES][64];   /* "split/<analysis>/<rows>/<synthesis>" (analysis: level, level-pairs,
                                                level-tma, level-pairs-tma or band; rows: rows8, rows8-pairs,
                                                rows16-pairs; synthesis: synthesis, synthesis-pairs,
                                                synthesis-tma, synthesis-pairs-tma or synthesis-regs; "-tma":
                                                column groups staged by TMA; "-regs": TMA-staged with the band
                                                sum in registers) or "fused/cluster<C>" */
  float ms[NSST_TUNE_MAX_CANDIDATES];        /* median ms of one directional-stage pass over n images */
  int direct_support[NSST_MAX_LEVELS];       /* per level, px (0: no window below the image size) */
  double direct_err[NSST_MAX_LEVELS];        /* per level: the worst band's truncation error at that window */
  float direct_bound_ms;                     /* lower bound of the direct path (-1: some level has no window) */
  int direct_wins;                           /* 1 if the rule above would pick direct convolution */
} nsst_tune_result;
nsst_status nsst_plan_autotune(nsst_plan* plan, int n, nsst_tune_result* out);

/* The directional-stage candidates of a plan, in the autotuner's order, as
 * newline-separated names into `names` (NUL-terminated, truncated to len);
 * returns their count (-1 for a NULL plan). */
int nsst_plan_directional_candidates(const nsst_plan* plan, char* names, size_t len);

/* Make candidate `index` the automatic choice for batches in n's bucket, as if
 * the autotuner had picked it; index -1 returns the bucket to the untuned
 * default.  Drops the captured graphs. */
nsst_status nsst_plan_select_directional(nsst_plan* plan, int n, int index);

/* The autotuner's direct-convolution evaluation alone, on the host (no GPU):
 * per level of cfg at H x W the smallest square window (px) around the
 * shearing filter's support keeping every band's truncation error <= tol
 * relative L2 (0: none below the image size), and the worst band's error
 * there; support and err hold cfg->nlevels entries each. */
nsst_status nsst_direct_support(const nsst_config* cfg, int H, int W, double tol, int* support, double* err);

/* Co-resident clusters of the fused directional kernel (0: not available). */
int nsst_plan_fused_clusters(const nsst_plan* plan);

/* Synchronises the device and reads the plan's device error word:
 * NSST_ERR_TIMEOUT if a bounded device-side wait (the fused kernel's TMA
 * completion wait) ran out since the last check (the word is then cleared and
 * the outputs of those calls are invalid), else NSST_OK.  No counterpart in
 * the reference, whose kernels have no device-side waits. */
nsst_status nsst_plan_check_device(nsst_plan* plan);

/* Release a plan and all its device memory.
 * Replaces clear_shearing_filters_cuda (clear_shearing_filters_cuda.cpp:51-96). */
nsst_status nsst_plan_destroy(nsst_plan* plan);

/* Number of coefficient planes (1 + sum 2^dcomp[i]). */
int nsst_plan_num_bands(const nsst_plan* plan);

/* Level of each band (0 = lowpass, i+1 = directional level i); out has nbands entries. */
nsst_status nsst_plan_band_levels(const nsst_plan* plan, int* out);

/* Device bytes held by the plan (filter spectra + work buffers). */
size_t nsst_plan_device_bytes(const nsst_plan* plan);

/* The pyramid filters (h0, h1, g0, g1 as FP64, row-major, sizes in F[4]);
 * `taps` must hold F0^2+F1^2+F2^2+F3^2 doubles (pass NULL to query sizes).
 * Mirrors atrousfilters.m:26-237. */
nsst_status nsst_pyramid_filters(const char* name, int* F, double* taps);

/* The Meyer shearing filters of one level in FP64 (2^level x n1 x n1).
 * Mirrors shearing_filters_Myer.m:18-26. */
nsst_status nsst_shearing_filters(int n1, int level, double* out);

/* Host-only (no GPU needed): normalised spectra of one directional level,
 * 2^dcomp Meyer filters of support dsize zero-padded top-left to H x W,
 * FP64 [2^dcomp][H][W/2+1] interleaved (re, im).  Mirrors nsst_dec2.m:47-57. */
nsst_status nsst_level_spectra(int dsize, int dcomp, int H, int W, double* out);

/* The normalised spectra of the plan's directional level `level` as FP64,
 * [ndir][H][W/2+1] interleaved (re, im).  Mirrors nsst_dec2.m:47-57. */
nsst_status nsst_plan_level_spectra(const nsst_plan* plan, int level, double* out);

/* À trous analysis: x (H x W, device) -> y ((nlevels+1) x H x W, device):
 * plane 0 lowpass, planes 1..nlevels bandpass from coarse to fine.
 * Replaces atrousdec (atrousdec.cpp:41-131; atrousdec.m:19-51). */
nsst_status nsst_atrousdec(nsst_plan* plan, const float* x, float* y, void* stream);

/* À trous synthesis: y ((nlevels+1) x H x W) -> x (H x W).
 * Replaces atrousrec (atrousrec.cpp:42-132; atrousrec.m:18-41). */
nsst_status nsst_atrousrec(nsst_plan* plan, const float* y, float* x, void* stream);

/* À trous analysis without any device allocation.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc — a MEX host
 * whose GPU array runtime already owns the device memory, a process under a
 * fixed device-memory budget, or a real-time loop that cannot pay cudaMalloc's
 * implicit device synchronisation.  Same result as nsst_atrousdec for the
 * pyramid filter `lpfilt` (NULL = "maxflat") and `nlevels` (1..6) levels, but
 * no plan is needed: the caller passes x (H x W) and y ((nlevels+1) x H x W,
 * plane 0 lowpass, then bandpass coarse -> fine), both device pointers, and
 * the one scratch image the lowpass chain needs lives in a static device array
 * of 2048*2048 floats (16 MiB) that every GPU loading the library holds until
 * exit.  H*W above 2048*2048 is rejected with NSST_ERR_UNSUPPORTED_SIZE,
 * an x that overlaps y with NSST_ERR_INVALID_ARG.  The first call on a device does a one-time set-up for that device (the
 * array's device address, kernel shared-memory limits); make that first call
 * before any stream capture.  All calls share the one array and it keeps the
 * last call's contents (nothing in it needs to start at zero): calls that
 * overlap on the GPU — on different streams or threads — race. */
nsst_status nsst_atrousdec_noalloc(const float* x, float* y, int H, int W, int nlevels, const char* lpfilt,
                                   void* stream);

/* Forward NSST: x (H x W, device) -> coeffs (nbands x H x W, device).
 * Replaces shear_trans_cuda (shear_trans_cuda.cpp:56-287) and
 * Shearcuda::shearTrans (demo_denoise/shearcuda/shearcuda.cpp:273-318). */
nsst_status nsst_shear_trans(nsst_plan* plan, const float* x, float* coeffs, void* stream);

/* Threshold coefficients in place: band b of level l uses
 * t = K[l] * sigma * scalars[b]  (K has nlevels+1 entries, K[0] lowpass);
 * hard keeps c where |c| > t, soft maps c to sign(c) max(|c| - t, 0).
 * Replaces thresh_cuda (thresh_cuda.cpp:57-217) / softth_cuda
 * (softth_cuda.cpp:49-112) / nsst_HT (nsst_HT.m:32-47) /
 * Shearcuda::hardThreshold (shearcuda.cpp:320-358). */
nsst_status nsst_thresh(nsst_plan* plan, float* coeffs, double sigma, const double* K, const double* scalars,
                        int mode, void* stream);

/* Inverse NSST: coeffs (nbands x H x W) -> x (H x W).
 * Replaces inverse_shear_cuda (inverse_shear_cuda.cpp:57-286) and
 * Shearcuda::inverseShear (shearcuda.cpp:360-396). */
nsst_status nsst_inverse_shear(nsst_plan* plan, const float* coeffs, float* x, void* stream);

/* Fused decompose -> threshold -> reconstruct (the coefficients are never
 * materialised).  Same threshold rule as nsst_thresh; scalars may be NULL to
 * use the plan's stored scalars (nsst_plan_set_scalars / nsst_compute_scalars).
 * Replaces the shear_trans_cuda -> thresh -> inverse_shear_cuda sequence of
 * shear_denoise_cuda.m:16-20 and demoImageDenoise mainwindow.cpp:221-234. */
nsst_status nsst_denoise(nsst_plan* plan, const float* x, float* out, double sigma, const double* K,
                         const double* scalars, int mode, void* stream);

/* Fused denoise of n <= B images of the plan's size in one pass: every stage
 * is one launch over all n images; image i uses sigma[i].  x[i], out[i] are
 * device pointers (H x W each). */
nsst_status nsst_denoise_batch(nsst_plan* plan, const float* const* x, float* const* out, int n, const double* sigma,
                               const double* K, const double* scalars, int mode, void* stream);

/* Uneven batches: images of several sizes denoised together.  A multi object
 * groups the items by plan (one plan per distinct size, each with enough
 * batch capacity), runs the groups on forked streams and captures the whole
 * batch (threshold uploads included) as one CUDA graph that is replayed while
 * the item pointers stay the same.  Each plan must hold its scalars
 * (nsst_plan_set_scalars or nsst_compute_scalars). */
typedef struct nsst_item {
  const float* x; /* device, H x W of the item's plan */
  float* out;     /* device, H x W */
  double sigma;
  int plan;       /* index into the plans array */
} nsst_item;
typedef struct nsst_multi nsst_multi;
nsst_status nsst_multi_create(nsst_plan* const* plans, int nplans, nsst_multi** out);
nsst_status nsst_multi_denoise(nsst_multi* m, const nsst_item* items, int n, const double* K, int mode, void* stream);
nsst_status nsst_multi_destroy(nsst_multi* m);

/* ---- Differentiation (no counterpart in the reference).  The adjoint of
 * every stage is hand-written: transposed pyramid steps (zero-extended
 * correlation with the unflipped filter, then the mirrored margins folded
 * back), conjugate-spectrum directional synthesis/analysis, and the threshold
 * subgradient 1[|c| > t] (soft rule: d/dt = -sign(c) 1[|c| > t]). */

/* Allocate the gradient workspace of a plan (once; about twice the plan's
 * own work buffers).  Required by the calls below. */
nsst_status nsst_plan_enable_grad(nsst_plan* plan);

/* x = A^T c, the adjoint of nsst_shear_trans (coeffs: nbands x H x W). */
nsst_status nsst_shear_trans_adjoint(nsst_plan* plan, const float* coeffs, float* x, void* stream);

/* c = R^T x, the adjoint of nsst_inverse_shear. */
nsst_status nsst_inverse_shear_adjoint(nsst_plan* plan, const float* x, float* coeffs, void* stream);

/* Fused denoise with explicit per-band thresholds tau (device, nbands floats,
 * shared by the n images): out_i = R(T(A x_i, tau)). */
nsst_status nsst_denoise_tau_batch(nsst_plan* plan, const float* const* x, float* const* out, int n,
                                   const float* tau, int mode, void* stream);

/* Backward of nsst_denoise_tau_batch: given grad_out_i = d loss / d out_i,
 * writes grad_x_i = d loss / d x_i and grad_tau (device, nbands floats;
 * added to when accumulate_tau != 0) = d loss / d tau summed over the images.
 * Band coefficients are recomputed from x, not stored. */
nsst_status nsst_denoise_tau_backward(nsst_plan* plan, const float* const* x, const float* const* grad_out,
                                      float* const* grad_x, int n, const float* tau, float* grad_tau,
                                      int accumulate_tau, int mode, void* stream);

/* Same as nsst_denoise_tau_backward for the n images of the most recent
 * nsst_denoise_tau_batch on this plan, without recomputing their band
 * coefficients: once nsst_plan_enable_grad has been called, that forward
 * keeps its pre-threshold band spectra and pyramid lowpass in the plan (the
 * thresholded bands go to a separate buffer).  Any other execute call on the
 * plan drops them; nsst_plan_saved_items tells how many images are held (0 =
 * none), and this call fails with NSST_ERR_INVALID_ARG unless it is n.  The
 * caller is responsible for x being unchanged since that forward. */
nsst_status nsst_denoise_tau_backward_saved(nsst_plan* plan, const float* const* grad_out, float* const* grad_x,
                                            int n, const float* tau, float* grad_tau, int accumulate_tau, int mode,
                                            void* stream);
int nsst_plan_saved_items(const nsst_plan* plan);

/* Store per-band noise scalars in the plan (nbands doubles). */
nsst_status nsst_plan_set_scalars(nsst_plan* plan, const double* scalars);

/* nsst_thresh, then the largest thresholded magnitude relative to its band's
 * scalar, max_b max|c_b| / scalars[b] (bands with scalar 0 skipped), into
 * *maxabs; waits for the stream.  Replaces thresh_cuda's opt == 1 output
 * (thresh_cuda.cpp:199-205, thresh.m:38-41). */
nsst_status nsst_thresh_max(nsst_plan* plan, float* coeffs, double sigma, const double* K, const double* scalars,
                            int mode, double* maxabs, void* stream);

/* out = atrousrec(weights .* atrousdec(x, nweights - 1 levels)): the image
 * re-synthesised with weights[0] on the lowpass and weights[1..nweights-1] on
 * the band-pass images, coarse to fine, with the plan's pyramid filters
 * (x, out: H x W device; 2 <= nweights <= nlevels + 1).  Replaces
 * re_weight_band / re_weight_band_cuda (re_weight_band.m:23-29,
 * re_weight_band_cuda.cpp:59-183), which likewise take the level count from
 * the length of the weight vector. */
nsst_status nsst_re_weight_band(nsst_plan* plan, const float* x, const double* weights, int nweights, float* out,
                                void* stream);

/* Exact l2 norm of every band's shearlet (nbands doubles, coefficient plane
 * order): the coefficients of an impulse of height sqrt(H W) at (H/2, W/2),
 * E_b = ||C_b|| / sqrt(H W) — the deterministic alternative to the Monte-Carlo
 * scalars, usable as nsst_thresh's scalars.  Synchronous.  Replaces com_norm.m
 * (com_norm.m:25-55) and norm_cuda (norm_cuda.cpp:57-215). */
nsst_status nsst_band_norms(nsst_plan* plan, double* E);

/* Per-band noise scalars by the Monte-Carlo rule of nsst_scalars.m:28-45:
 * a seeded N(0,1) image (generated in FP64 on the host) is transformed on the
 * GPU and each band's MAD/0.6745 is taken on the host in FP64.  Writes nbands
 * doubles to out and stores them in the plan.  Synchronous.
 * Replaces nsst_scalars.m / Shearcuda::computeShearNorm (shearcuda.cpp:205-271). */
nsst_status nsst_compute_scalars(nsst_plan* plan, uint64_t seed, double* out);

/* Per-stage timing with CUDA events on the call's stream (no device syncs on
 * the execute path).  When enabled, every execute call records one event per
 * stage; nsst_timers_read waits for the last call's final event and returns
 * the stage names ("\n"-separated into `names`, up to names_len bytes) and
 * durations in milliseconds (up to max_stages).  Returns the stage count.
 * Replaces GpuTimes / shear_timers (GpuTimes.h:25-78, shear_timers.cpp:40-85),
 * which synchronised the device around every step. */
nsst_status nsst_timers_enable(nsst_plan* plan, int enable);
int nsst_timers_read(nsst_plan* plan, char* names, size_t names_len, float* ms, int max_stages);

/* ------------------------------------------------------------------------
 * Undecimated wavelets and image separation.
 * ------------------------------------------------------------------------ */
enum { NSST_MAX_QMF = 64 };

/* The orthonormal QMF of MakeONFilter.m (MakeONFilter.m:1-289): type "Haar",
 * "Beylkin", "Coiflet" (par 1-5), "Daubechies" (par 4, 6, ..., 20),
 * "Symmlet" (par 4-10), "Vaidyanathan" or "Battle" (par 1, 3, 5); par is
 * ignored for the families without one.  Writes f / norm(f) to out (up to
 * NSST_MAX_QMF doubles) and its length to *len.  Host only. */
nsst_status nsst_onfilter(const char* type, int par, double* out, int* len);

/* Redundant (undecimated) DWT of n images, L levels, periodic: mrdwt /
 * mrdwt_cuda (src/mrdwt_r.h:104-209, src_cuda/mrdwt_cuda.cpp:55-255).
 * x: n x H x W device; h: lh host doubles (lh <= 32), the scaling filter.
 * yl: n x H x W (the level-L lowpass); yh: n x 3L x H x W, per level the
 * planes LH, HL, HH (first letter: filtering along a row), level 1 first --
 * the reference's m x 3nL yh, block by block.  H and W must be multiples of
 * 2^L, W <= 8192.  x may equal yl.  Asynchronous on stream. */
nsst_status nsst_mrdwt(const float* x, int n, int H, int W, const double* h, int lh, int L, float* yl, float* yh,
                       void* stream);

/* Inverse of nsst_mrdwt: mirdwt / mirdwt_cuda (src/mirdwt_r.h:115-219,
 * src_cuda/mirdwt_cuda.cpp).  yl, yh are left unchanged; x may equal yl.
 * Takes two planes of stream-ordered scratch per image. */
nsst_status nsst_mirdwt(const float* yl, const float* yh, int n, int H, int W, const double* h, int lh, int L,
                        float* x, void* stream);

/* TV correction of n images (x, y: n x H x W device; y != x): one Haar level
 * of nsst_mrdwt, soft threshold gamma on the three highpass planes, nsst_mirdwt
 * -- one fused stencil.  Replaces TVCorrection / TVCorrection_cuda
 * (separate.m:264-285: mrdwt_cuda, softth_cuda, mirdwt_cuda). */
nsst_status nsst_tv_correction(const float* x, int n, int H, int W, double gamma, float* y, void* stream);

/* What nsst_separate derived from each image before its loop (separate.m:72-126). */
typedef struct nsst_separate_info {
  double sigma;          /* MAD / 0.6745 of the HH band of a one-level Daubechies-4 DWT */
  double stop;           /* stop * sigma */
  double buff_shear;     /* thresh opt == 1 max of the shearlet coefficients (buff(1)) */
  double buff_wavelet;   /* max |yh| of the Symmlet-4 mrdwt (buff(2)) */
  double deltamax;       /* min(buff) */
  double lambda;         /* (deltamax / stop)^(1 / (1 - itermax)) */
} nsst_separate_info;

/* Points / curves separation of n images (n <= the plan's batch capacity):
 * separate.m:1-289 with the plan's shearlets and pyramid filters (the
 * reference hard-codes 'maxflat', separate.m:61; a 'maxflat' plan matches it),
 * level2 Symmlet-4 wavelet levels, itermax iterations, the stopping
 * factor stop, the TV soft threshold gamma and the ncoeff band weights coeff
 * (re_weight_band; 2 <= ncoeff <= nlevels + 1).  img: n x H x W device;
 * writes the curve part to C and the point part to P (n x H x W device) and,
 * if info is not NULL, n nsst_separate_info records.  The per-image setup
 * (band norms, MAD, the two maxima) waits for the stream; the iterations are
 * then queued on it without host waits. */
/* The noise estimate uses the HH quadrant (rows H/2.., columns W/2..) of the
 * one-level DWT; for the square images the reference accepts that is its
 * wc(N/2+1:N, N/2+1:N) (separate.m:101). */
nsst_status nsst_separate(nsst_plan* plan, const float* img, int n, int level2, int itermax, double stop,
                          double gamma, const double* coeff, int ncoeff, float* C, float* P,
                          nsst_separate_info* info, void* stream);

/* Number of kernels this library has launched since load (all plans, all threads). */
uint64_t nsst_launch_count(void);

/* Test hook: make the n-th device allocation from now fail with
 * NSST_ERR_OUT_OF_MEMORY (n <= 0 disarms).  Host-side fault injection only. */
void nsst_debug_fail_next_alloc(int n);

/* ------------------------------------------------------------------------
 * 3-D path: Fourier-domain band-pass pyramid (shearcuda3d/3DBP, Pyr_mode 1.5)
 * and 24^3 pseudo-polar Meyer directional filters applied by linear 'same'
 * convolution (shearcuda3d/3DShearTrans, CONVNFFT_Folder/convnfft.m).
 *
 * Volumes are float32 n0 x n1 x n2, index (x*n1 + y)*n2 + z (axis 2 fastest);
 * axis k plays the role of MATLAB dimension k+1, and the pyramid's half
 * spectrum lies along axis 2 as ccsym(X, 3, 'c') does.  The plan pads each
 * dimension by edge replication (MarshalData.m:3-22) to a grid of 96, 144 or
 * 192 so that every level size is a 2^a 3^b transform length, and crops the
 * reconstruction back.
 *
 * Sub-band layout ("bp", per volume): level 0 (finest) band-pass of
 * m_0 = grid dims, level 1 of 2/3 of it, level 2 of 1/3, ..., then the lowpass;
 * concatenated, nsst3_subband_floats() floats per volume.  Directional bands
 * are ordered level-major, then cone (after the swap of cones 1 and 2 of
 * GetMeyerBasedFilter.m:148-150), then l2, then l1.
 * ------------------------------------------------------------------------ */
typedef struct nsst3_plan nsst3_plan;

/* How a volume is padded to the pyramid's grid (edge replication, cropped
 * back after the reconstruction):
 *   NSST3_GRID_FAST:    the smallest grid <= 192 whose level sizes are 2^a 3^b
 *                       lengths (128 -> 144, 192 -> 192): the same result as
 *                       the reference's DenoiseDemo/main.m on volumes whose
 *                       sides divide by 12, and the fastest transforms;
 *   NSST3_GRID_MARSHAL: MarshalData.m:3-22 as the reference's any-size demo
 *                       (mainAnySize.m:51) pads: every side gains
 *                       d - rem(n, d) planes, d = 3 2^(nlevels-1) (128 -> 132,
 *                       192 -> 204), Pyr_mode 1.5 only; its level sizes need
 *                       the lengths 132, 88, 44, 22 and 204, 136, 68, 34,
 *                       which are compiled (others are rejected). */
enum { NSST3_GRID_FAST = 0, NSST3_GRID_MARSHAL = 1 };
typedef struct nsst3_config {
  int nlevels;                   /* pyramid levels, 1..4 (the demo uses 3) */
  int num_dirs[NSST_MAX_LEVELS]; /* numDir per level, finest first; 3*numDir^2 bands per level (numDir | 24) */
  double pyr_mode;               /* 1, 1.5 or 2 (PyrNDDec_mm.m:58-74); 1.5 in the demo */
  int grid;                      /* NSST3_GRID_FAST (0) or NSST3_GRID_MARSHAL */
} nsst3_config;

/* Plan for batches of up to `batch` volumes of n0 x n1 x n2 (each <= 192).
 * Builds the FP64 Meyer filters, their convolution spectra (FP32 on the
 * device) and the pyramid windows; allocates every work buffer.
 * Replaces GetMeyerBasedFilter.m + the per-call cuFFT plans and filter FFTs
 * of ShDecThRec_cuda.cpp:178-335. */
nsst_status nsst3_plan_create(const nsst3_config* cfg, int n0, int n1, int n2, int batch, nsst3_plan** plan);
nsst_status nsst3_plan_destroy(nsst3_plan* plan);
int nsst3_num_bands(const nsst3_plan* plan);           /* directional bands over all levels */
size_t nsst3_subband_floats(const nsst3_plan* plan);   /* floats per volume of the sub-band layout */
size_t nsst3_plan_device_bytes(const nsst3_plan* plan);
/* level -1: dims[0..2] = the padded grid; level l in [0, nlevels]: dims of band-pass l
 * (l = nlevels: lowpass) and conv[0..2] = its convolution FFT lengths. */
nsst_status nsst3_level_dims(const nsst3_plan* plan, int level, int* dims, int* conv);
/* level, cone, l2, l1 of directional band b. */
nsst_status nsst3_band_info(const nsst3_plan* plan, int band, int* info4);

/* FP64 Meyer filters of GetMeyerBasedFilter.m:12-150 (cube 24): writes
 * sum_l 3*num_dirs[l]^2 filters of 24^3 doubles in band order when out is not
 * NULL; returns the filter count (or -1 on a bad argument).  Host only. */
int nsst3_meyer_filters(int nlevels, const int* num_dirs, double* out);

/* Band-pass pyramid of n volumes (device x, n*n0*n1*n2 floats contiguous) into
 * bp (device, n * nsst3_subband_floats).  Replaces MarshalData.m + DoPyrDec.m
 * (PyrNDDec_mm.m:20-109). */
nsst_status nsst3_pyr_dec(nsst3_plan* plan, const float* x, float* bp, int n, void* stream);
/* Inverse: bp -> x (n0 x n1 x n2, the grid cropped).  Replaces DoPyrRec.m
 * (PyrNDRec_mm.m:20-95). */
nsst_status nsst3_pyr_rec(nsst3_plan* plan, const float* bp, float* x, int n, void* stream);

/* Directional coefficients of one pyramid level (ShDec.m:18-34, one level,
 * every cone): coeffs (device) receives, per volume, 3*numDir^2 volumes of
 * that level's band-pass size in band order. */
nsst_status nsst3_sh_dec(nsst3_plan* plan, const float* bp, int level, float* coeffs, int n, void* stream);

/* ShDecThRec_cuda (ShDecThRec_cuda.cpp:57-335): for each level, sum over all
 * bands of the directional coefficients hard-thresholded at
 * T[level] * sigma[i] * scalars[band] (ThresholdShCoeff.m:7 zeroes
 * |c| <= t); the lowpass is copied unchanged.  bp -> rec_bp, same layout.
 * sigma: n doubles (host), T: nlevels doubles, scalars: nsst3_num_bands
 * doubles (NULL = the plan's stored scalars). */
nsst_status nsst3_sh_dec_thresh_rec(nsst3_plan* plan, const float* bp, float* rec_bp, int n, const double* sigma,
                                    const double* T, const double* scalars, void* stream);

/* The whole 3-D denoise of DenoiseDemo/main.m:80-145 for n volumes: pad,
 * pyramid, directional hard threshold + band sum, pyramid reconstruction,
 * crop.  x, out: device, n*n0*n1*n2 floats. */
nsst_status nsst3_denoise_batch(nsst3_plan* plan, const float* x, float* out, int n, const double* sigma,
                                const double* T, const double* scalars, void* stream);

/* NsstScalars.m:1-19: a seeded N(0,1) grid-sized volume (FP64 on the host)
 * is decomposed on the GPU and each band's MAD/0.6745 is taken on the host in
 * FP64.  Writes nsst3_num_bands doubles to out and stores them in the plan.
 * Synchronous. */
nsst_status nsst3_compute_scalars(nsst3_plan* plan, uint64_t seed, double* out);
nsst_status nsst3_plan_set_scalars(nsst3_plan* plan, const double* scalars);

/* Differentiation of nsst3_denoise_batch (no counterpart in the reference).
 * nsst3_plan_enable_grad allocates one keep bit per directional coefficient
 * and batch item; from then on nsst3_denoise_batch records the masks
 * |c| > t of its hard threshold.  nsst3_denoise_backward then maps
 * gy = d loss / d out (device, n volumes) to gx = d loss / d x (device, n
 * volumes) for the n volumes of the most recent nsst3_denoise_batch on this
 * plan (the threshold's subgradient keeps that call's masks).  The adjoint
 * steps: zero-padding of gy, the pyramid decomposition (the band-pass pyramid
 * is a Parseval frame, so it is the reconstruction's adjoint), per band the
 * masked gradient correlated with the filter (conjugate spectrum), the
 * pyramid reconstruction, and the fold of the edge padding. */
nsst_status nsst3_plan_enable_grad(nsst3_plan* plan);
nsst_status nsst3_denoise_backward(nsst3_plan* plan, const float* gy, float* gx, int n, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* NSST_H */
