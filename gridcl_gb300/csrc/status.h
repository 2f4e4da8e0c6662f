// Status helpers shared by the C-ABI translation units: the thread-local message returned by
// tlg_last_error().
#pragma once

#include <string>

#include <cuda_runtime.h>

#include "../../include/tlgeom.h"

namespace tlg {

tlg_status fail(tlg_status s, const std::string& msg);
tlg_status ok();
tlg_status cuda_fail(cudaError_t e, const char* what);

}  // namespace tlg
