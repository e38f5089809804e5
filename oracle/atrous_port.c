/* CPU restatement (FP64, plain C) of the reference's à trous building blocks.
 *
 * TEST INFRASTRUCTURE ONLY: this is the oracle's checker and the timed CPU
 * baseline; no product code links it.
 *
 *   atrousc_port    restates shearlet_toolbox_1/atrousc.cpp:43-73
 *                   (convolutionLoop: 'valid' convolution with the filter
 *                   implicitly upsampled by a diagonal matrix M).
 *   symext_port     restates shearlet_toolbox_1/symext.m:18-31.
 *   atrous_level    symext + atrousc for one filter, threaded over output rows;
 *                   that is one call of atrousdec.m:34,46-47 / atrousrec.m:35,41.
 *
 * Arrays are row-major here (MATLAB is column-major); the algorithm is
 * symmetric in the two axes for the square filters and equal shifts the
 * pyramid uses, and the index arithmetic below is written per axis. */
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* out[n1][n2] = sum_{k1,k2} F[Fr-1-k1][Fc-1-k2] * S[n1 + M-1 + k1*M][n2 + M-1 + k2*M]
 * out is (Sr - M*Fr + 1) x (Sc - M*Fc + 1).  Rows [r0, r1) only. */
static void atrousc_rows(const double* S, int Sr, int Sc, const double* F, int Fr, int Fc, int M,
                         double* out, int r0, int r1) {
  (void)Sr;
  int Oc = Sc - M * Fc + 1;
  for (int n1 = r0; n1 < r1; n1++) {
    for (int n2 = 0; n2 < Oc; n2++) {
      double sum = 0.0;
      int kk1 = n1 + M - 1;
      for (int k1 = 0; k1 < Fr; k1++) {
        const double* frow = F + (size_t)(Fr - 1 - k1) * Fc;
        const double* srow = S + (size_t)kk1 * Sc;
        int kk2 = n2 + M - 1;
        for (int k2 = 0; k2 < Fc; k2++) {
          sum += frow[Fc - 1 - k2] * srow[kk2];
          kk2 += M;
        }
        kk1 += M;
      }
      out[(size_t)n1 * Oc + n2] = sum;
    }
  }
}

void atrousc_port(const double* S, int Sr, int Sc, const double* F, int Fr, int Fc, int M,
                  double* out) {
  int Or = Sr - M * Fr + 1;
  atrousc_rows(S, Sr, Sc, F, Fr, Fc, M, out, 0, Or);
}

/* symext.m: x is m x n; filter p x q; shift (s1, s2).  Output (m+p-1) x (n+q-1).
 * Columns are extended by ss = floor(p/2)-s1+1 on the left (mirror including
 * the edge sample) and by p+s1 on the right; rows by rr = floor(q/2)-s2+1 on
 * top and q+s2 at the bottom; the result is cropped to (m+p-1) x (n+q-1).
 * Returns 0, or -1 if the extension would need samples beyond one reflection
 * (MATLAB raises an index error there). */
int symext_port(const double* x, int m, int n, int p, int q, int s1, int s2, double* out) {
  int ss = p / 2 - s1 + 1;
  int rr = q / 2 - s2 + 1;
  int outr = m + p - 1, outc = n + q - 1;
  if (ss > n || p + s1 > n || rr > m || q + s2 > m || ss < 0 || rr < 0) return -1;
  for (int i = 0; i < outr; i++) {
    int t = i - rr;
    int si = t < 0 ? -1 - t : (t >= m ? 2 * m - 1 - t : t);
    for (int j = 0; j < outc; j++) {
      int u = j - ss;
      int sj = u < 0 ? -1 - u : (u >= n ? 2 * n - 1 - u : u);
      out[(size_t)i * outc + j] = x[(size_t)si * n + sj];
    }
  }
  return 0;
}

typedef struct {
  const double* S;
  int Sr, Sc;
  const double* F;
  int Fr, Fc, M;
  double* out;
  int r0, r1;
} job_t;

static void* run_job(void* arg) {
  job_t* j = (job_t*)arg;
  atrousc_rows(j->S, j->Sr, j->Sc, j->F, j->Fr, j->Fc, j->M, j->out, j->r0, j->r1);
  return NULL;
}

/* One pyramid filtering step: out (m x n) = atrousc(symext(x, upsampled F, shift), F, M).
 * The upsampled filter size is M*F (upsample2df.m:4-6).  nthreads >= 1. */
int atrous_level(const double* x, int m, int n, const double* F, int Fs, int M, int shift,
                 double* out, int nthreads) {
  int p = M * Fs;
  int Sr = m + p - 1, Sc = n + p - 1;
  double* S = (double*)malloc(sizeof(double) * (size_t)Sr * Sc);
  if (!S) return -2;
  if (symext_port(x, m, n, p, p, shift, shift, S) != 0) {
    free(S);
    return -1;
  }
  int Or = Sr - M * Fs + 1;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  job_t jobs[256];
  int chunk = (Or + nthreads - 1) / nthreads;
  int started = 0;
  for (int t = 0; t < nthreads; t++) {
    int r0 = t * chunk, r1 = r0 + chunk > Or ? Or : r0 + chunk;
    if (r0 >= r1) break;
    jobs[t] = (job_t){S, Sr, Sc, F, Fs, Fs, M, out, r0, r1};
    if (nthreads == 1) {
      run_job(&jobs[t]);
    } else {
      pthread_create(&th[t], NULL, run_job, &jobs[t]);
      started++;
    }
  }
  for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
  free(S);
  return 0;
}
