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
// Whether the strategy settings of a family are valid (false, with the error set, when the
// environment variable is invalid), and the record of a launch for tlg_last_kernel_family /
// tlg_last_launch_family.
bool check_strategy(int family);
void record_launch(int family, int strategy);

}  // namespace tlg
