// msx_noalloc.cu -- internal force f_int(u) without any memory allocation.
//
// Built with --fmad=false: the arithmetic is the reference's operation order,
// the same as msx_internal_force on a handle created with MSX_PREC_FP64_EXACT.
//
// The corner forces, which the element pass writes and the node gather reads,
// live in g_corner_scratch below, a fixed array in the library's own device
// memory: every GPU that loads the library holds its 6 MiB until the process
// exits, and the entry point never calls cudaMalloc or cudaFree.
#include <string>

#include "../../include/msx.h"
#include "msx_device.cuh"

using namespace msx;

namespace {

constexpr long long kNoAllocMaxElems = 65536;   // MSX_NOALLOC_MAX_ELEMS in include/msx.h

// Scratch for 12 corner-force components per element.  In host code this name
// is only a stand-in for the device array: its device address comes from
// cudaGetSymbolAddress (set-up below), never from taking its address here.
static __device__ __align__(256) double g_corner_scratch[12 * kNoAllocMaxElems];

// Element pass: the reference's set-up of dphi and wJ from X
// (classLinearTetrahedra.cpp:171-268, classGPs.cpp:27), F (constitutiveManager.cpp:
// 151-164), P (the law) and wJ P dphi (constitutiveAlgorithms.cpp:46-56).
__global__ void noalloc_elem_kernel(const double *__restrict__ X, const int4 *__restrict__ conn, long long nn,
                                    long long ne, MatParams m, const double *__restrict__ u, double *scratch)
{
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int4 cn = conn[e];
    int nd[4] = {cn.x, cn.y, cn.z, cn.w};
    double *fe = scratch + e * 12;
    if (nd[0] < 0 || nd[0] >= nn || nd[1] < 0 || nd[1] >= nn || nd[2] < 0 || nd[2] >= nn || nd[3] < 0 ||
        nd[3] >= nn) {
        // a node id outside the mesh: the element contributes nothing
#pragma unroll
        for (int k = 0; k < 12; k++) fe[k] = 0.0;
        return;
    }
    double xyz[12];
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
        for (int i = 0; i < 3; i++) xyz[i * 4 + k] = X[i * nn + nd[k]];
    const double natDev[12] = {-1.0, -1.0, -1.0, 1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0};
    double Jac[9], iJ[9];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            double c = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) c += xyz[i * 4 + k] * natDev[k * 3 + j];
            Jac[i * 3 + j] = c;
        }
    double J = det3_ref(Jac);
    inv3_ref(Jac, iJ);
    double dphi[12];
#pragma unroll
    for (int k = 0; k < 9; k++) dphi[3 + k] = 0.0 + iJ[k];
#pragma unroll
    for (int j = 0; j < 3; j++) dphi[j] = (-dphi[3 + j] - dphi[6 + j]) - dphi[9 + j];
    double wJ = 0.166666666667 * fabs(J);
    double F[9], P[9];
#pragma unroll
    for (int i = 0; i < 9; i++) F[i] = 0.;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        F[i * 3 + i] += 1.;
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int j = 0; j < 3; j++) F[i * 3 + j] += dphi[a * 3 + j] * u[nd[a] + i * nn];
    }
    stress_ref(m, F, P);
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
            double f = 0;
#pragma unroll
            for (int Jx = 0; Jx < 3; Jx++) f += wJ * P[i * 3 + Jx] * dphi[a * 3 + Jx];
            fe[a * 3 + i] = 0 + f;
        }
}

// Node gather in element order (solverExplicit.cpp:363-379): fint[node + c*nn].
__global__ void noalloc_gather_kernel(const int *__restrict__ node_ptr, const int *__restrict__ node_inc, long long nn,
                                      long long ne, const double *scratch, double *fint)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    double s[3] = {0, 0, 0};
    // incidences outside [0, 4*ne) are skipped, so only this call's entries are read
    const long long ninc = 4 * ne;
    long long k0 = node_ptr[i], k1 = node_ptr[i + 1];
    k0 = k0 < 0 ? 0 : k0;
    k1 = k1 > ninc ? ninc : k1;
    for (long long k = k0; k < k1; k++) {
        long long inc = node_inc[k];
        if (inc < 0 || inc >= ninc) continue;
        const double *f = scratch + inc * 3;
        s[0] += f[0];
        s[1] += f[1];
        s[2] += f[2];
    }
#pragma unroll
    for (int c = 0; c < 3; c++) fint[i + c * nn] = s[c];
}

msx_status nfail(msx_status st, const std::string &m)
{
    msx_set_error(m.c_str());
    return st;
}

// Device address of the scratch array on the current device.  Looked up on
// every call with that device current (the lookup allocates nothing): an
// address kept from an earlier call would go stale if the application reset
// the device, which reloads the library's module at a new address.
msx_status scratch_for_current_device(double **out)
{
    int dev = -1;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return nfail(MSX_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(err));
    void *ptr = nullptr;
    err = cudaGetSymbolAddress(&ptr, g_corner_scratch);
    if (err != cudaSuccess || !ptr)
        return nfail(MSX_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(err));
    *out = (double *)ptr;
    return MSX_OK;
}

bool aligned(const void *p, uintptr_t a) { return (uintptr_t)p % a == 0; }

}  // namespace

extern "C" msx_status msx_internal_force_noalloc(const double *X, const int32_t *conn, int64_t num_nodes,
                                                 int64_t num_elems, const int32_t *node_ptr,
                                                 const int32_t *node_inc, const msx_material *material,
                                                 const double *u, double *fint, void *stream)
{
    if (!X || !conn || !node_ptr || !node_inc || !material || !u || !fint)
        return nfail(MSX_ERR_ARG, "msx_internal_force_noalloc: NULL argument");
    if (num_elems < 1 || num_nodes < 4) return nfail(MSX_ERR_ARG, "msx_internal_force_noalloc: empty mesh");
    if (num_elems > kNoAllocMaxElems)
        return nfail(MSX_ERR_ARG, "msx_internal_force_noalloc: " + std::to_string(num_elems) +
                                      " elements exceed the scratch maximum of " + std::to_string(kNoAllocMaxElems));
    if (num_nodes >= (1LL << 31)) return nfail(MSX_ERR_ARG, "msx_internal_force_noalloc: too many nodes");
    if (!aligned(conn, 16)) return nfail(MSX_ERR_ARG, "msx_internal_force_noalloc: conn must be 16-byte aligned");
    if (!aligned(X, 8) || !aligned(u, 8) || !aligned(fint, 8))
        return nfail(MSX_ERR_ARG, "msx_internal_force_noalloc: X, u and fint must be 8-byte aligned");
    if (!aligned(node_ptr, 4) || !aligned(node_inc, 4))
        return nfail(MSX_ERR_ARG, "msx_internal_force_noalloc: node_ptr and node_inc must be 4-byte aligned");
    // the same law parameters as every other entry point (all four laws)
    MatParams m{};
    if (!material_params(*material, m))
        return nfail(MSX_ERR_ARG, "msx_internal_force_noalloc: material needs law 0..3, E > 0, rho > 0, -1 < nu < 0.5");
    double *scratch = nullptr;
    msx_status st = scratch_for_current_device(&scratch);
    if (st != MSX_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    // every scratch entry the gather reads is written by this call's element
    // pass first, so nothing needs clearing between calls
    noalloc_elem_kernel<<<grid_for(num_elems, 256), 256, 0, s>>>(X, (const int4 *)conn, num_nodes, num_elems, m, u,
                                                                 scratch);
    noalloc_gather_kernel<<<grid_for(num_nodes, 256), 256, 0, s>>>(node_ptr, node_inc, num_nodes, num_elems, scratch, fint);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return nfail(MSX_ERR_CUDA, std::string("msx_internal_force_noalloc launch: ") + cudaGetErrorString(err));
    return MSX_OK;
}
