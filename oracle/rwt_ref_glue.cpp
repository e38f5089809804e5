/* Glue that exposes the reference's unchanged Rice Wavelet Toolbox templates
 * (shearcuda/src/mrdwt_r.h:84-209, mirdwt_r.h:95-219, mdwt_r.h:81-176) as C
 * functions in double precision, for the oracle's tests.
 *
 * Test infrastructure only.  Built by oracle/build_oracle.py into
 * oracle/_ref/librwt_ref.so; the templates are included where they lie in
 * the reference checkout, nothing of them is copied into this repository.
 * Their scratch comes from mxCalloc and is never released (one small leak per
 * call, as under MATLAB's MEX memory manager without its end-of-call sweep). */
#include <cstdlib>

#include "matrix.h"

void* mxCalloc(size_t n, size_t size) { return std::calloc(n ? n : 1, size ? size : 1); }

#include "mrdwt_r.h"
#undef mat
#undef max
#undef min
#include "mirdwt_r.h"
#undef mat
#undef max
#undef min
#include "mdwt_r.h"

extern "C" {

/* column-major m x n image; yh m x 3nL (mrdwt.cpp:127-154) */
void ref_mrdwt(const double* x, int m, int n, const double* h, int lh, int L, double* yl, double* yh) {
  MRDWT<double>(x, m, n, h, lh, L, yl, yh);
}

void ref_mirdwt(double* x, int m, int n, const double* h, int lh, int L, const double* yl, const double* yh) {
  MIRDWT<double>(x, m, n, h, lh, L, yl, yh);
}

void ref_mdwt(double* x, int m, int n, double* h, int lh, int L, double* y) { MDWT<double>(x, m, n, h, lh, L, y); }

}  // extern "C"
