// memd_internal.h -- host-side helpers shared by the translation units.
#pragma once

#include <cuda_runtime.h>

#include "memd_gb300.h"

namespace memd {

memd_status set_error(memd_status code, const char* msg);
memd_status set_cuda_error(const char* where, cudaError_t e = cudaGetLastError());

}  // namespace memd
