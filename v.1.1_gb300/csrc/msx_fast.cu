// msx_fast.cu -- FP64 (contracted, simplified algebra) and mixed-precision
// kernels.  The tiled step kernels are instantiated here only, so a single
// solve (msx_run) and the pool execute the same machine code.
#include "msx_device.cuh"

namespace msx {

void launch_internal_force_fp64(const Problem &p, double *fint, cudaStream_t s)
{
    elem_force_kernel_fp64<<<grid_for(p.ne, kElemBlock), kElemBlock, 0, s>>>(p, 0);
    gather_kernel<MODE_FP64><<<grid_for(p.nn, 256), 256, 0, s>>>(p, fint);
}

void launch_internal_force_mixed(const Problem &p, double *fint, cudaStream_t s)
{
    elem_force_kernel_mixed<<<grid_for(p.ne, kElemBlock), kElemBlock, 0, s>>>(p, 0);
    gather_kernel<MODE_MIXED><<<grid_for(p.nn, 256), 256, 0, s>>>(p, fint);
}

void launch_tiled_node(const Problem *descs, const Tile *ntiles, const int *counts, int mode, int parity, int grid,
                       int threads, cudaStream_t s)
{
    if (mode == MODE_MIXED)
        pool_node_kernel<MODE_MIXED><<<grid, threads, 0, s>>>(descs, ntiles, counts + 1, parity);
    else
        pool_node_kernel<MODE_FP64><<<grid, threads, 0, s>>>(descs, ntiles, counts + 1, parity);
}

void launch_tiled_elem(const Problem *descs, const Tile *etiles, const int *counts, int mode, int parity, int grid,
                       int threads, cudaStream_t s)
{
    if (mode == MODE_MIXED)
        pool_elem_kernel<MODE_MIXED><<<grid, threads, 0, s>>>(descs, etiles, counts, parity);
    else
        pool_elem_kernel<MODE_FP64><<<grid, threads, 0, s>>>(descs, etiles, counts, parity);
}

int tiled_ctas_per_sm(int mode, int threads, bool node)
{
    int a = 0;
    if (mode == MODE_MIXED)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, node ? (const void *)pool_node_kernel<MODE_MIXED>
                                                               : (const void *)pool_elem_kernel<MODE_MIXED>, threads, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, node ? (const void *)pool_node_kernel<MODE_FP64>
                                                               : (const void *)pool_elem_kernel<MODE_FP64>, threads, 0);
    return a > 0 ? a : 1;
}

}  // namespace msx
