// msx_fast.cu -- FP64 (contracted, simplified algebra) and mixed-precision kernels.
#include "msx_device.cuh"

namespace msx {

void launch_node_fp64(const Problem &p, int parity, cudaStream_t s)
{
    node_kernel<MODE_FP64><<<grid_for(p.nn, kNodeBlock), kNodeBlock, 0, s>>>(p, parity);
}

void launch_elem_fp64(const Problem &p, int parity, cudaStream_t s)
{
    elem_kernel_fp64<false><<<grid_for(p.ne, kElemBlock), kElemBlock, 0, s>>>(p, parity);
}

void launch_internal_force_fp64(const Problem &p, double *fint, cudaStream_t s)
{
    elem_kernel_fp64<true><<<grid_for(p.ne, kElemBlock), kElemBlock, 0, s>>>(p, 0);
    gather_kernel<MODE_FP64><<<grid_for(p.nn, 256), 256, 0, s>>>(p, fint);
}

void launch_node_mixed(const Problem &p, int parity, cudaStream_t s)
{
    node_kernel<MODE_MIXED><<<grid_for(p.nn, kNodeBlock), kNodeBlock, 0, s>>>(p, parity);
}

void launch_elem_mixed(const Problem &p, int parity, cudaStream_t s)
{
    elem_kernel_mixed<false><<<grid_for(p.ne, kElemBlock), kElemBlock, 0, s>>>(p, parity);
}

void launch_internal_force_mixed(const Problem &p, double *fint, cudaStream_t s)
{
    elem_kernel_mixed<true><<<grid_for(p.ne, kElemBlock), kElemBlock, 0, s>>>(p, 0);
    gather_kernel<MODE_MIXED><<<grid_for(p.nn, 256), 256, 0, s>>>(p, fint);
}

}  // namespace msx
