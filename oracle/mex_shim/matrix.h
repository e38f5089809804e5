/* Minimal, project-written stand-in for MATLAB's matrix.h.
 *
 * Test infrastructure only: it lets the reference's MEX sources
 * shearlet_toolbox_1/atrousc.cpp and the Rice Wavelet Toolbox templates
 * shearcuda/src/{mrdwt,mirdwt,mdwt}_r.h compile unchanged as plain shared
 * libraries so that their loops can serve as the oracle's ground truth.
 * Only the handful of calls those files make are provided (atrousc.cpp:83-125,
 * mxCalloc in the templates).  Arrays are column-major like MATLAB's. */
#ifndef NSST_ORACLE_MATRIX_H
#define NSST_ORACLE_MATRIX_H
#include <stddef.h>

typedef size_t mwSize;
typedef enum { mxUNKNOWN_CLASS = 0, mxDOUBLE_CLASS = 6, mxSINGLE_CLASS = 7 } mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

typedef struct mxArray_tag {
  mxClassID cls;
  size_t m, n;
  void* data;
  int owns;
} mxArray;

size_t mxGetM(const mxArray* a);
size_t mxGetN(const mxArray* a);
bool mxIsDouble(const mxArray* a);
bool mxIsClass(const mxArray* a, const char* name);
double* mxGetPr(const mxArray* a);
void* mxGetData(const mxArray* a);
mxArray* mxCreateNumericArray(mwSize ndim, const mwSize* dims, mxClassID cls, mxComplexity cplx);
void* mxCalloc(size_t n, size_t size);
#endif
