/* Glue that drives the reference's unchanged atrousc.cpp mexFunction
 * (shearlet_toolbox_1/atrousc.cpp:75-148) from C, for the oracle.
 *
 * Test infrastructure only.  Built by oracle/build_oracle.py into
 * oracle/_ref/libatrousc_ref.so together with the reference source, which is
 * compiled where it lies; nothing of it is copied into this repository. */
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>

#include "mex.h"

struct MexError : std::runtime_error {
  explicit MexError(const std::string& s) : std::runtime_error(s) {}
};

size_t mxGetM(const mxArray* a) { return a->m; }
size_t mxGetN(const mxArray* a) { return a->n; }
bool mxIsDouble(const mxArray* a) { return a->cls == mxDOUBLE_CLASS; }
bool mxIsClass(const mxArray* a, const char* name) {
  if (!strcmp(name, "double")) return a->cls == mxDOUBLE_CLASS;
  if (!strcmp(name, "single")) return a->cls == mxSINGLE_CLASS;
  return false;
}
double* mxGetPr(const mxArray* a) { return static_cast<double*>(a->data); }
void* mxGetData(const mxArray* a) { return a->data; }
mxArray* mxCreateNumericArray(mwSize ndim, const mwSize* dims, mxClassID cls, mxComplexity) {
  mxArray* a = new mxArray;
  a->cls = cls;
  a->m = dims[0];
  a->n = ndim > 1 ? dims[1] : 1;
  size_t esz = cls == mxSINGLE_CLASS ? 4 : 8;
  a->data = calloc(a->m * a->n ? a->m * a->n : 1, esz);
  a->owns = 1;
  return a;
}
void mexErrMsgTxt(const char* msg) { throw MexError(msg); }
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  throw MexError(std::string(id) + ": " + buf);
}

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);

static thread_local std::string g_err;

extern "C" const char* ref_atrousc_error() { return g_err.c_str(); }

/* S: column-major Sm x Sn, F: column-major Fm x Fn, dilation M (diagonal).
 * out: column-major (Sm - M*Fm + 1) x (Sn - M*Fn + 1).  Returns 0 on success. */
extern "C" int ref_atrousc(const double* S, int Sm, int Sn, const double* F, int Fm, int Fn,
                           double M, double* out) {
  mxArray s{mxDOUBLE_CLASS, (size_t)Sm, (size_t)Sn, const_cast<double*>(S), 0};
  mxArray f{mxDOUBLE_CLASS, (size_t)Fm, (size_t)Fn, const_cast<double*>(F), 0};
  double mm[4] = {M, 0.0, 0.0, M};
  mxArray m{mxDOUBLE_CLASS, 2, 2, mm, 0};
  const mxArray* prhs[3] = {&s, &f, &m};
  mxArray* plhs[1] = {nullptr};
  try {
    mexFunction(1, plhs, 3, prhs);
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
  size_t n = plhs[0]->m * plhs[0]->n;
  memcpy(out, plhs[0]->data, n * sizeof(double));
  free(plhs[0]->data);
  delete plhs[0];
  return 0;
}
