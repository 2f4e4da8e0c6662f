// f64 instantiations of the evaluation kernels.
#define TLG_F double
#define TLG_LAUNCH launch_eval_f64
#define TLG_WITH_DIRECT
#include "eval_inst.cuh"
