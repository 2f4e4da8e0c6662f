// f64 instantiations of the evaluation kernels.
#define TLG_F double
#define TLG_LAUNCH launch_eval_f64
#include "eval_inst.cuh"
