/* mex.h -- TEST STUB of the few MATLAB MEX / mx API calls the MEX entry
 * (memd-gpu_gb300/mex/memd_mex.cpp) uses, so that it can be compiled and
 * exercised without MATLAB.  Not MATLAB's header: same names and argument
 * meaning, minimal behaviour (errors become C++ exceptions). */
#ifndef MEMD_TEST_MEX_STUB_H
#define MEMD_TEST_MEX_STUB_H

#include <stddef.h>

typedef size_t mwSize;
typedef enum { mxUNKNOWN_CLASS = 0, mxDOUBLE_CLASS = 6, mxSINGLE_CLASS = 7, mxINT32_CLASS = 12 } mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef struct mxArray_tag mxArray;

#ifdef __cplusplus
extern "C" {
#endif
void* mxGetData(const mxArray* a);
mxClassID mxGetClassID(const mxArray* a);
size_t mxGetNumberOfElements(const mxArray* a);
void mxFree(void* p);
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
int mexAtExit(void (*fn)(void));
/* the MEX loader looks the gateway up by its unmangled name */
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, mxArray const* prhs[]);
#ifdef __cplusplus
}
#endif

#endif
