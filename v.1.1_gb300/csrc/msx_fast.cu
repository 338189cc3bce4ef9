// msx_fast.cu -- FP64 (contracted, simplified algebra), double-word and
// mixed-precision kernels.  The tiled step kernels are instantiated here only, so a single
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

void launch_internal_force_dw(const Problem &p, double *fint, cudaStream_t s)
{
    elem_force_kernel_dw<<<grid_for(p.ne, kElemBlock), kElemBlock, 0, s>>>(p, 0);
    gather_kernel<MODE_DW><<<grid_for(p.nn, 256), 256, 0, s>>>(p, fint);
}

void launch_tiled_node(const Problem *descs, const Tile *ntiles, int *counts, int mode, int parity, int grid,
                       int threads, cudaStream_t s)
{
    if (mode == MODE_MIXED)
        pool_node_kernel<MODE_MIXED><<<grid, threads, 0, s>>>(descs, ntiles, counts + 3, parity);
    else if (mode == MODE_DW)
        pool_node_kernel<MODE_DW><<<grid, threads, 0, s>>>(descs, ntiles, counts + 3, parity);
    else
        pool_node_kernel<MODE_FP64><<<grid, threads, 0, s>>>(descs, ntiles, counts + 3, parity);
}

template <int MODE>
static void launch_elem_variant(const Problem *descs, const Tile *etiles, int *counts, int parity, int grid,
                                int threads, size_t smem, cudaStream_t s, bool act, bool visc)
{
    // element birth and bulk viscosity are separate instantiations (never both: the host refuses that)
    if (act)
        pool_elem_kernel<MODE, true><<<grid, threads, smem, s>>>(descs, etiles, counts, parity);
    else if (visc)
        pool_elem_kernel<MODE, false, true><<<grid, threads, smem, s>>>(descs, etiles, counts, parity);
    else
        pool_elem_kernel<MODE><<<grid, threads, smem, s>>>(descs, etiles, counts, parity);
}

void launch_tiled_elem(const Problem *descs, const Tile *etiles, int *counts, int mode, int parity, int grid,
                       int threads, int tile_elems, cudaStream_t s, bool act, bool visc)
{
    (void)tile_elems;
    if (mode == MODE_MIXED)
        launch_elem_variant<MODE_MIXED>(descs, etiles, counts, parity, grid, threads, 0, s, act, visc);
    else if (mode == MODE_DW)
        launch_elem_variant<MODE_DW>(descs, etiles, counts, parity, grid, threads, 0, s, act, visc);
    else
        launch_elem_variant<MODE_FP64>(descs, etiles, counts, parity, grid, threads, 0, s, act, visc);
}

// a32: the mixed mode, whose acceleration is one FP32 per DOF (mixed_a32)
__global__ void state_split_kernel(Problem p, bool a32)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * p.nn) return;
    p.uhl[i] = df_from(p.u[i]);
    p.vhl[i] = df_from(p.v[i]);
    if (a32) mixed_a32(p)[i] = (float)p.a[i];
    else p.ahl[i] = df_from(p.a[i]);
}

__global__ void state_merge_kernel(Problem p, bool a32)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * p.nn) return;
    float2 u = p.uhl[i], v = p.vhl[i];
    p.u[i] = (double)u.x + (double)u.y;
    p.v[i] = (double)v.x + (double)v.y;
    if (a32) {
        p.a[i] = (double)mixed_a32(p)[i];
    } else {
        const float2 a = p.ahl[i];
        p.a[i] = (double)a.x + (double)a.y;
    }
}

__global__ void u4_from_u_kernel(const double *u, double *u4, long long nn)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    reinterpret_cast<double2 *>(u4)[2 * i] = make_double2(u[i], u[nn + i]);
    reinterpret_cast<double2 *>(u4)[2 * i + 1] = make_double2(u[2 * nn + i], 0.0);
}

void launch_u4_from_u(const double *u, double *u4, long long nn, cudaStream_t s)
{
    u4_from_u_kernel<<<grid_for(nn, 256), 256, 0, s>>>(u, u4, nn);
}

__global__ void minv_split_kernel(const double *minv, float2 *minv2, long long nn)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nn) minv2[i] = df_from(minv[i]);
}

void launch_state_split(const Problem &p, bool mixed, cudaStream_t s)
{
    state_split_kernel<<<grid_for(3 * p.nn, 256), 256, 0, s>>>(p, mixed);
}

void launch_state_merge(const Problem &p, bool mixed, cudaStream_t s)
{
    state_merge_kernel<<<grid_for(3 * p.nn, 256), 256, 0, s>>>(p, mixed);
}

void launch_minv_split(const double *minv, float2 *minv2, long long nn, cudaStream_t s)
{
    minv_split_kernel<<<grid_for(nn, 256), 256, 0, s>>>(minv, minv2, nn);
}

__global__ void node_bc_scatter_kernel(int *node_bc, const int2 *nodes, long long n)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) node_bc[nodes[k].x] = nodes[k].y;
}

void launch_node_bc_scatter(int *node_bc, long long nn, const int2 *nodes, long long n, cudaStream_t s)
{
    cudaMemsetAsync(node_bc, 0xFF, sizeof(int) * nn, s);   // -1: no entry
    if (n > 0) node_bc_scatter_kernel<<<grid_for(n, 256), 256, 0, s>>>(node_bc, nodes, n);
}

__global__ void abs_range_kernel(const double *x, long long n, unsigned long long *mm)
{
    unsigned long long lo = ~0ULL, hi = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(fabs(x[i]));
        if (b != 0) {
            lo = b < lo ? b : lo;
            hi = b > hi ? b : hi;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = l2 < lo ? l2 : lo;
        hi = h2 > hi ? h2 : hi;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(mm, lo);
        atomicMax(mm + 1, hi);
    }
}

__global__ void abs_range_init_kernel(unsigned long long *mm)
{
    mm[0] = ~0ULL;
    mm[1] = 0;
}

void launch_abs_range(const double *x, long long n, unsigned long long *mm, cudaStream_t s)
{
    abs_range_init_kernel<<<1, 1, 0, s>>>(mm);
    abs_range_kernel<<<256, 256, 0, s>>>(x, n, mm);
}

int tiled_ctas_per_sm(int mode, int threads, bool node)
{
    int a = 0;
    if (mode == MODE_MIXED)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, node ? (const void *)pool_node_kernel<MODE_MIXED>
                                                               : (const void *)pool_elem_kernel<MODE_MIXED>, threads, 0);
    else if (mode == MODE_DW)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, node ? (const void *)pool_node_kernel<MODE_DW>
                                                               : (const void *)pool_elem_kernel<MODE_DW>, threads, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, node ? (const void *)pool_node_kernel<MODE_FP64>
                                                               : (const void *)pool_elem_kernel<MODE_FP64>, threads, 0);
    return a > 0 ? a : 1;
}

}  // namespace msx
