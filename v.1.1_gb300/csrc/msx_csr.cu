// msx_csr.cu -- node -> (element, corner) lists of a mesh, built on the device.
//
// The list of node i holds the incidences k = 4e + a with conn[k] == i in
// increasing k, that is in element order: the per-node summation order of
// classSolverExplicit::computeInternalForce (solverExplicit.cpp:363-379).
// slot[k] is the position of incidence k in that list (the element kernels
// write corner forces there, so that a node reads its own in one run).
// Integer counts, an exclusive scan, an atomic fill, then each node's list
// sorted: the fill order is arbitrary, the sorted one is not, so the arrays
// are bit for bit those of the sequential construction on the host.  A node
// with more than kCsrMaxDegree incidences is left to the host (the per-node
// insertion sort is quadratic in the degree).
#include <climits>
#include <algorithm>
#include <string>
#include <vector>

#include "../../include/msx.h"
#include "msx_internal.h"

namespace msx {
namespace {

constexpr int kScanThreads = 256, kScanPerThread = 16;
constexpr int kScanChunk = kScanThreads * kScanPerThread;   // counts per scan block
constexpr int kGridStride = 152 * 16;                        // blocks of the grid-stride kernels

__device__ __forceinline__ int warp_incl_scan(int v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    return v;
}

// Exclusive scan of one value per thread over the block (blockDim.x a multiple
// of 32, at most 1024); *total gets the block's sum.
__device__ int block_excl_scan(int v, int *total)
{
    __shared__ int warp_sum[32];
    __shared__ int block_total;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int incl = warp_incl_scan(v);
    if (lane == 31) warp_sum[w] = incl;
    __syncthreads();
    if (w == 0) {
        const int s = lane < nw ? warp_sum[lane] : 0;
        const int si = warp_incl_scan(s);
        if (lane < nw) warp_sum[lane] = si - s;   // exclusive prefix of the warps
        if (lane == 31) block_total = si;         // lanes >= nw add zeros: lane 31 holds the total
    }
    __syncthreads();
    const int r = warp_sum[w] + incl - v;
    const int t = block_total;
    __syncthreads();   // warp_sum and block_total are reused by the next call
    *total = t;
    return r;
}

__global__ void csr_count_kernel(const int *conn, long long n4, long long nn, int *cnt, int *flags)
{
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += (long long)gridDim.x * blockDim.x) {
        const int v = conn[k];
        if (v < 0 || v >= nn) {
            atomicOr(flags, 1);   // connectivity out of range: nothing else runs
            continue;
        }
        atomicAdd(cnt + v, 1);
    }
}

// Sum and largest count of each chunk of kScanChunk counts.
__global__ void csr_chunk_sum_kernel(const int *cnt, long long nn, int *bsum, int *flags)
{
    const long long base = (long long)blockIdx.x * kScanChunk;
    int s = 0, m = 0;
    for (int j = threadIdx.x; j < kScanChunk; j += blockDim.x) {
        const long long i = base + j;
        if (i < nn) {
            const int c = cnt[i];
            s += c;
            m = max(m, c);
        }
    }
    int tot;
    block_excl_scan(s, &tot);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(flags + 1, m);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

// Exclusive scan of the nb chunk sums in place, one block.
__global__ void csr_scan_sums_kernel(int *bsum, long long nb)
{
    int carry = 0;
    for (long long b0 = 0; b0 < nb; b0 += blockDim.x) {
        const long long b = b0 + threadIdx.x;
        const int v = b < nb ? bsum[b] : 0;
        int tot;
        const int ex = block_excl_scan(v, &tot);
        if (b < nb) bsum[b] = carry + ex;
        carry += tot;
    }
}

// node_ptr[i + 1] = counts up to and including node i; node_ptr[0] = 0.
__global__ void csr_scan_chunk_kernel(const int *cnt, long long nn, const int *bsum, int *node_ptr)
{
    const long long base = (long long)blockIdx.x * kScanChunk + (long long)threadIdx.x * kScanPerThread;
    int v[kScanPerThread];
    int run = 0;
#pragma unroll
    for (int j = 0; j < kScanPerThread; j++) {
        const long long i = base + j;
        run += i < nn ? cnt[i] : 0;
        v[j] = run;
    }
    int tot;
    const int off = block_excl_scan(run, &tot) + bsum[blockIdx.x];
#pragma unroll
    for (int j = 0; j < kScanPerThread; j++) {
        const long long i = base + j;
        if (i < nn) node_ptr[i + 1] = off + v[j];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) node_ptr[0] = 0;
}

__global__ void csr_fill_kernel(const int *conn, long long n4, const int *node_ptr, int *fillc, int *inc)
{
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += (long long)gridDim.x * blockDim.x) {
        const int v = conn[k];
        inc[node_ptr[v] + atomicAdd(fillc + v, 1)] = (int)k;
    }
}

// Each node's list in increasing incidence order.  Lists of at most 32 (a
// tet mesh's usual degree is about 24) are sorted in registers by a bitonic
// network, padded with INT_MAX; longer ones (at most kCsrMaxDegree) by
// insertion sort in place.
__global__ void csr_sort_kernel(const int *node_ptr, long long nn, int *inc)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    int *l = inc + node_ptr[i];
    const int d = node_ptr[i + 1] - node_ptr[i];
    if (d <= 32) {
        int v[32];
#pragma unroll
        for (int j = 0; j < 32; j++) v[j] = j < d ? l[j] : INT_MAX;
#pragma unroll
        for (int k = 2; k <= 32; k <<= 1)
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
                for (int a = 0; a < 32; a++) {
                    const int b = a ^ j;
                    if (b > a) {
                        const int lo = min(v[a], v[b]), hi = max(v[a], v[b]);
                        const bool up = (a & k) == 0;
                        v[a] = up ? lo : hi;
                        v[b] = up ? hi : lo;
                    }
                }
#pragma unroll
        for (int j = 0; j < 32; j++)
            if (j < d) l[j] = v[j];
        return;
    }
    for (int x = 1; x < d; x++) {
        const int key = l[x];
        int y = x - 1;
        while (y >= 0 && l[y] > key) {
            l[y + 1] = l[y];
            y--;
        }
        l[y + 1] = key;
    }
}

__global__ void csr_slot_kernel(const int *inc, long long n4, int *slot)
{
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += (long long)gridDim.x * blockDim.x)
        slot[inc[k]] = (int)k;
}

}  // namespace

static void build_node_csr_host(const int *conn, long long ne, long long nn, std::vector<int> &ptr, std::vector<int> &inc,
                                std::vector<int> &slots)
{
    ptr.assign(nn + 1, 0);
    inc.resize(4 * ne);
    slots.resize(4 * ne);
    for (long long k = 0; k < 4 * ne; k++) ptr[conn[k] + 1]++;
    for (long long i = 0; i < nn; i++) ptr[i + 1] += ptr[i];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (long long k = 0; k < 4 * ne; k++) {
        const int pos = fill[conn[k]]++;
        inc[pos] = (int)k;
        slots[k] = pos;
    }
}

msx_status build_node_csr(const int4 *conn4, const int *conn_host, long long ne, long long nn, int *node_ptr,
                          int *node_inc, int4 *slot, cudaStream_t s, std::string &err)
{
    const int *conn = reinterpret_cast<const int *>(conn4);
    const long long n4 = 4 * ne, nb = (nn + kScanChunk - 1) / kScanChunk;
    int *cnt = nullptr, *fillc = nullptr, *bsum = nullptr, *flags = nullptr;
    auto release = [&] {
        for (int *q : {cnt, fillc, bsum, flags})
            if (q) cudaFreeAsync(q, s);
    };
    auto cuda_fail = [&](cudaError_t e) {
        release();
        err = std::string("connectivity lists: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? MSX_ERR_OOM : MSX_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = cudaMallocAsync(&cnt, sizeof(int) * nn, s)) != cudaSuccess ||
        (e = cudaMallocAsync(&fillc, sizeof(int) * nn, s)) != cudaSuccess ||
        (e = cudaMallocAsync(&bsum, sizeof(int) * nb, s)) != cudaSuccess ||
        (e = cudaMallocAsync(&flags, sizeof(int) * 2, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(cnt, 0, sizeof(int) * nn, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(fillc, 0, sizeof(int) * nn, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(flags, 0, sizeof(int) * 2, s)) != cudaSuccess)
        return cuda_fail(e);
    const int gs = (int)std::min<long long>(kGridStride, (n4 + 255) / 256);
    csr_count_kernel<<<gs, 256, 0, s>>>(conn, n4, nn, cnt, flags);
    csr_chunk_sum_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(cnt, nn, bsum, flags);
    int hf[2] = {0, 0};
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaMemcpyAsync(hf, flags, sizeof(hf), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e);
    if (hf[0]) {
        release();
        err = "connectivity index out of range";
        return MSX_ERR_ARG;
    }
    if (hf[1] > kCsrMaxDegree) {   // a node in very many elements: the host builds the lists
        release();
        if (!conn_host) {
            err = "a node is shared by more than the device list builder's limit of elements";
            return MSX_ERR_ARG;
        }
        std::vector<int> ptr, inc, slots;
        build_node_csr_host(conn_host, ne, nn, ptr, inc, slots);
        if ((e = cudaMemcpyAsync(node_ptr, ptr.data(), sizeof(int) * (nn + 1), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
            (e = cudaMemcpyAsync(node_inc, inc.data(), sizeof(int) * n4, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
            (e = cudaMemcpyAsync(slot, slots.data(), sizeof(int) * n4, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess) {
            err = std::string("connectivity lists: ") + cudaGetErrorString(e);
            return MSX_ERR_CUDA;
        }
        return MSX_OK;
    }
    csr_scan_sums_kernel<<<1, 1024, 0, s>>>(bsum, nb);
    csr_scan_chunk_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(cnt, nn, bsum, node_ptr);
    csr_fill_kernel<<<gs, 256, 0, s>>>(conn, n4, node_ptr, fillc, node_inc);
    csr_sort_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(node_ptr, nn, node_inc);
    csr_slot_kernel<<<gs, 256, 0, s>>>(node_inc, n4, reinterpret_cast<int *>(slot));
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e);
    release();
    return MSX_OK;
}

}  // namespace msx
