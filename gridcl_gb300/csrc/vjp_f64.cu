// f64 instantiations of the adjoint kernel.
#define TLG_VJP_SPLIT false
#define TLG_VJP_LAUNCH launch_vjp_f64
#include "vjp_inst.cuh"
