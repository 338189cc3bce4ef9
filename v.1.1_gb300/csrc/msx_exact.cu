// msx_exact.cu -- kernels in the reference's operation order.
// Built with --fmad=false: every product and sum rounds on its own, as in the
// reference compiled without FMA contraction, so FP64_EXACT results can be
// compared with the reference bit for bit.  Also holds the set-up kernels,
// whose outputs (dphi, wJ, characteristic length, lumped mass) every mode uses.
#define MSX_SETUP_KERNELS
#include "msx_device.cuh"

namespace msx {

void launch_node_exact(const Problem &p, int parity, cudaStream_t s)
{
    node_kernel<MODE_EXACT><<<grid_for(p.nn, kNodeBlock), kNodeBlock, 0, s>>>(p, parity);
}

void launch_elem_exact(const Problem &p, int parity, cudaStream_t s)
{
    if (p.visc)
        elem_kernel_exact_screened<true><<<grid_for(p.ne, kElemBlock), kElemBlock, 0, s>>>(p, parity);
    else
        elem_kernel_exact_screened<false><<<grid_for(p.ne, kElemBlock), kElemBlock, 0, s>>>(p, parity);
}

void launch_setup_elements(const Problem &p, const double *X, cudaStream_t s, long long e0, long long e1)
{
    if (e1 < 0) e1 = p.ne;
    if (e1 <= e0) return;
    setup_elements_kernel<<<grid_for(e1 - e0, 256), 256, 0, s>>>(
        p, X, const_cast<double *>(p.G), const_cast<double *>(p.wJ), const_cast<double *>(p.Lref),
        const_cast<float *>(p.G32), const_cast<float *>(p.wJ32), const_cast<float *>(p.Lref32), e0, e1);
}

void launch_mode_arrays(const Problem &p, float *G32, float *wJ32, float *G32lo, float *wJ32lo, cudaStream_t s)
{
    mode_arrays_kernel<<<grid_for(p.ne, 256), 256, 0, s>>>(p, G32, wJ32, G32lo, wJ32lo);
}

void launch_cnh_arrays(const Problem &p, cudaStream_t s)
{
    cnh_arrays_kernel<<<grid_for(p.ne, 256), 256, 0, s>>>(p);
}

void launch_visc_init(const Problem &p, const double *u, cudaStream_t s)
{
    visc_init_kernel<<<grid_for(p.ne, 256), 256, 0, s>>>(p, u);
}

void launch_setup_mass(const Problem &p, double *mass, double *minv, cudaStream_t s)
{
    setup_mass_kernel<<<grid_for(p.nn, 256), 256, 0, s>>>(p, mass, minv);
}

void launch_initial_cfl(const Problem &p, const double *uK, int slot, cudaStream_t s)
{
    initial_cfl_kernel<<<grid_for(p.ne, kElemBlock), kElemBlock, 0, s>>>(p, uK, slot);
}

void launch_internal_force_exact(const Problem &p, double *fint, cudaStream_t s)
{
    elem_kernel_exact<true><<<grid_for(p.ne, kElemBlock), kElemBlock, 0, s>>>(p, 0);
    gather_kernel<MODE_EXACT><<<grid_for(p.nn, 256), 256, 0, s>>>(p, fint);
}

void launch_node_values(const Problem &p, int mode, int field, int comp, const int *nodes, long long n, double t,
                        double *out, cudaStream_t s)
{
    if (n > 0) node_values_kernel<<<grid_for(n, 128), 128, 0, s>>>(p, mode, field, comp, nodes, n, t, out);
}

void launch_face_loads(const Problem &p, int parity, bool mixed, cudaStream_t s)
{
    if (p.nfaces > 0) face_load_kernel<<<grid_for(p.nfaces, 128), 128, 0, s>>>(p, parity, mixed);
}

void launch_setup_gravity(const Problem &p, double g, double *grav_e, double *grav_n, cudaStream_t s)
{
    setup_gravity_elem_kernel<<<grid_for(p.ne, 256), 256, 0, s>>>(p, g, grav_e);
    setup_gravity_node_kernel<<<grid_for(p.nn, 256), 256, 0, s>>>(p, grav_e, grav_n);
}

void launch_element_fields(const Problem &p, double t, double *cauchy, double *gl, double *vms, cudaStream_t s)
{
    element_fields_kernel<<<grid_for(p.ne, 256), 256, 0, s>>>(p, t, cauchy, gl, vms);
}

void launch_element_values(const Problem &p, int quantity, const int *elems, long long n, double t, double *out,
                           cudaStream_t s)
{
    if (n > 0) element_values_kernel<<<grid_for(n, 128), 128, 0, s>>>(p, quantity, elems, n, t, out);
}

void launch_element_reduce(const Problem &p, int quantity, int op, const int *elems, long long n, double t,
                           double *part, double *out, cudaStream_t s)
{
    element_reduce_kernel<<<kReduceBlocks, kReduceThreads, 0, s>>>(p, quantity, op, elems, n, t, part);
    element_reduce_finish_kernel<<<1, kReduceThreads, 0, s>>>(quantity, op, part, out);
}

long long element_reduce_scratch() { return 2LL * kReduceBlocks + 1; }

}  // namespace msx
