/* Minimal, project-written stand-in for MATLAB's mex.h (test infrastructure
 * only; see matrix.h).  Errors raised by the MEX source are turned into a
 * C++ exception that the glue in oracle/atrous_ref_glue.cpp catches. */
#ifndef NSST_ORACLE_MEX_H
#define NSST_ORACLE_MEX_H
#include "matrix.h"

void mexErrMsgTxt(const char* msg);
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
#endif
