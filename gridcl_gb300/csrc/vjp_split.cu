// Split-precision instantiations of the adjoint kernel, and the f64 node gather.
#define TLG_VJP_SPLIT true
#define TLG_VJP_LAUNCH launch_vjp_split
#include "vjp_inst.cuh"

namespace tlg {

cudaError_t launch_vjp_gather(const uint32_t* offsets, const uint32_t* entries, int64_t num_nodes, int d,
                              const void* local, int local_dtype, double* grad, cudaStream_t s, bool add) {
  int64_t blocks = (num_nodes + kGatherNodes - 1) / kGatherNodes;
  if (blocks < 1) blocks = 1;
  if (blocks > 152 * 64) blocks = 152 * 64;
#define TLG_GATHER(L, DD) \
  vjp_gather_kernel<L, DD><<<(unsigned)blocks, kGatherNodes, 0, s>>>(offsets, entries, num_nodes, \
                                                            static_cast<const L*>(local), grad, add ? 1 : 0)
  if (local_dtype == 4) {
    if (d == 1) TLG_GATHER(float, 1);
    else if (d == 2) TLG_GATHER(float, 2);
    else TLG_GATHER(float, 3);
  } else {
    if (d == 1) TLG_GATHER(double, 1);
    else if (d == 2) TLG_GATHER(double, 2);
    else TLG_GATHER(double, 3);
  }
#undef TLG_GATHER
  return cudaGetLastError();
}

cudaError_t launch_vjp_tile(bool split, const VjpArgs& a, size_t smem, cudaStream_t s) {
  int group = 1, threads = 32;
  vjp_tile_shape(a.k_runtime, &group, &threads);
  VjpArgs b = a;
  b.group = group;
  auto launch = [&](auto kern) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int grid = persistent_grid(kern, smem, a.padded / 16 * threads, threads);
    kern<<<grid, threads, smem, s>>>(b);
    return cudaGetLastError();
  };
  return split ? launch(vjp_tile_kernel<float>) : launch(vjp_tile_kernel<double>);
}

cudaError_t launch_vjp_gather_blocks(const GatherBlocks& gb, int64_t num_nodes, int d, int local_dtype, double* grad,
                                     cudaStream_t s, bool add) {
  int64_t blocks = (num_nodes + kGatherNodes - 1) / kGatherNodes;
  if (blocks < 1) blocks = 1;
  if (blocks > 152 * 64) blocks = 152 * 64;
#define TLG_GATHER(L, DD) \
  vjp_gather_blocks_kernel<L, DD><<<(unsigned)blocks, kGatherNodes, 0, s>>>(gb, num_nodes, grad, add ? 1 : 0)
  if (local_dtype == 4) {
    if (d == 1) TLG_GATHER(float, 1);
    else if (d == 2) TLG_GATHER(float, 2);
    else TLG_GATHER(float, 3);
  } else {
    if (d == 1) TLG_GATHER(double, 1);
    else if (d == 2) TLG_GATHER(double, 2);
    else TLG_GATHER(double, 3);
  }
#undef TLG_GATHER
  return cudaGetLastError();
}

}  // namespace tlg
