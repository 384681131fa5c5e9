/*
 * mex.h -- stand-in for the part of MATLAB's mex API that FrameLab's four
 * projector gateways (Ax_fan_mf.cpp, Atx_fan_mf.cpp, Ax_cone_mf.cpp,
 * Atx_cone_mf.cpp) use, so that they compile unmodified outside MATLAB and
 * link against libframelab_gb300.so the way a mex build would.
 *
 * TEST INFRASTRUCTURE ONLY (oracle/Makefile, target `gateways`; tests/).
 * The arrays are plain host buffers: mxArray is defined in mx_standin.cpp.
 */
#pragma once
#include <stddef.h>
#include <stdio.h>

typedef enum {
    mxUNKNOWN_CLASS = 0,
    mxSTRUCT_CLASS = 2,
    mxDOUBLE_CLASS = 6,
    mxSINGLE_CLASS = 7,
    mxINT32_CLASS = 12,
    mxUINT32_CLASS = 13
} mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef size_t mwSize;
typedef size_t mwIndex;
typedef struct mxArray_tag mxArray;

#ifdef __cplusplus
extern "C" {
#endif
/* the gateway's entry point (defined by the gateway source) */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);

mxArray *mxGetField(const mxArray *s, mwIndex i, const char *name);
void *mxGetData(const mxArray *a);
double mxGetScalar(const mxArray *a);
size_t mxGetNumberOfElements(const mxArray *a);
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID c, mxComplexity cx);
#ifdef __cplusplus
}
#endif

#define mexPrintf printf
