/* gpu/mxGPUArray.h -- TEST STUB of the mxGPUArray calls used by the MEX
 * entry (see tests/mex_stub/mex.h). */
#ifndef MEMD_TEST_MXGPU_STUB_H
#define MEMD_TEST_MXGPU_STUB_H

#include "mex.h"

typedef enum { MX_GPU_INITIALIZE_VALUES = 0, MX_GPU_DO_NOT_INITIALIZE = 1 } mxGPUInitialize;
typedef struct mxGPUArray_tag mxGPUArray;

#ifdef __cplusplus
extern "C" {
#endif
int mxInitGPU(void);
mxGPUArray const* mxGPUCreateFromMxArray(mxArray const* a);
void const* mxGPUGetDataReadOnly(mxGPUArray const* g);
void* mxGPUGetData(mxGPUArray* g);
mxGPUArray* mxGPUCreateGPUArray(mwSize ndims, mwSize const* dims, mxClassID cid, mxComplexity ccx, mxGPUInitialize init);
mwSize mxGPUGetNumberOfDimensions(mxGPUArray const* g);
mwSize const* mxGPUGetDimensions(mxGPUArray const* g);
mxClassID mxGPUGetClassID(mxGPUArray const* g);
mxComplexity mxGPUGetComplexity(mxGPUArray const* g);
mwSize mxGPUGetNumberOfElements(mxGPUArray const* g);
mxArray* mxGPUCreateMxArrayOnGPU(mxGPUArray const* g);
void mxGPUDestroyGPUArray(mxGPUArray const* g);
#ifdef __cplusplus
}
#endif

#endif
