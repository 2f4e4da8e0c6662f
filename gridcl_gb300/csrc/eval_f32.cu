// f32 instantiations of the evaluation kernels.
#define TLG_F float
#define TLG_LAUNCH launch_eval_f32
#include "eval_inst.cuh"
