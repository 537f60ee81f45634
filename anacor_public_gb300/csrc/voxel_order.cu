// Voxel-list packing and ordering at plan creation.
//
// The march is warp-cooperative and a warp's cost is set by its slowest lane,
// so lanes that start close together (similar path lengths, same exit face)
// make it cheaper.  The reference's coordinate list is in np.where order
// (AnACor/utils/utils_rt.py:50-51): 32 consecutive entries form a long row in
// x (128 voxels long at sampling stride 4).  Sorting the packed list by the
// Morton (Z-order) code of (z, y, x) gives each warp a compact 3-D block.
// The absorption factor is a mean over the list, so the order only changes
// the FP32 summation order (results stay deterministic for a given list).
// Blocked orders trade that compactness for fewer 32-byte sectors per warp
// label load: on a crystal sampled at stride s, a Morton block of 32 points
// spans 8 volume rows, a 1 x 2 x 16 block 2 rows of 16 points; the autotuner
// picks the order per sample.
#include <cub/device/device_radix_sort.cuh>
#include <cuda_runtime.h>
#include <stdint.h>

#include "anacor_internal.h"
#include "trace_launch.h"

namespace anacor {
namespace {

__device__ __forceinline__ unsigned long long spread3(unsigned v)
{
    // bits of v (13 used) to every third bit
    unsigned long long x = v & 0x1fffu;
    x = (x | (x << 16)) & 0x0000ff0000ffull;
    x = (x | (x << 8)) & 0x00f00f00f00full;
    x = (x | (x << 4)) & 0x0c30c30c30c3ull;
    x = (x | (x << 2)) & 0x249249249249ull;
    return x;
}

// Sort key of a voxel under voxel order `order` (1: Morton; 2..: blocked)
__device__ __forceinline__ unsigned long long order_key(unsigned z, unsigned y, unsigned x, int lz, int ly, int lx)
{
    const unsigned long long hi =
        (spread3(z >> lz) << 2) | (spread3(y >> ly) << 1) | spread3(x >> lx);
    const unsigned long long lo = ((unsigned long long)(z & ((1u << lz) - 1u)) << (ly + lx)) |
                                  ((unsigned long long)(y & ((1u << ly) - 1u)) << lx) | (x & ((1u << lx) - 1u));
    return (hi << (lz + ly + lx)) | lo;
}

__global__ void pack_keys_kernel(const long long *__restrict__ c, int n, int dz, int dy, int dx, int lz, int ly, int lx,
                                 unsigned long long *__restrict__ keys, unsigned long long *__restrict__ vals,
                                 int *__restrict__ status_word)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    long long z = c[3 * i], y = c[3 * i + 1], x = c[3 * i + 2];
    if (z < 0 || z >= dz || y < 0 || y >= dy || x < 0 || x >= dx) {
        atomicOr(status_word, 1 << kErrArgs);
        z = y = x = 0;
    }
    keys[i] = order_key((unsigned)z, (unsigned)y, (unsigned)x, lz, ly, lx);
    const short4 p = make_short4((short)z, (short)y, (short)x, 0);
    vals[i] = *reinterpret_cast<const unsigned long long *>(&p);
}

__global__ void index_keys_kernel(const long long *__restrict__ c, int n, int dz, int dy, int dx, int lz, int ly,
                                  int lx, unsigned long long *__restrict__ keys, int *__restrict__ idx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    long long z = c[3 * i], y = c[3 * i + 1], x = c[3 * i + 2];
    if (z < 0 || z >= dz || y < 0 || y >= dy || x < 0 || x >= dx)
        z = y = x = 0;
    keys[i] = order_key((unsigned)z, (unsigned)y, (unsigned)x, lz, ly, lx);
    idx[i] = i;
}

// log2 block sizes (z, y, x) of the blocked orders 2, 3, ...: 32 consecutive
// list entries of a crystal sampled on a lattice of stride s cover one block
// of 1 x 2 x 16 or 1 x 4 x 8 lattice points when the block is s times that
constexpr int kOrderShape[kVoxelOrders - 2][3] = {
    {0, 1, 4},   // 1 x 2 x 16 voxels   (stride 1: 1 x 2 x 16 points)
    {0, 2, 3},   // 1 x 4 x 8
    {1, 2, 5},   // 2 x 4 x 32          (stride 2: 1 x 2 x 16)
    {2, 3, 6},   // 4 x 8 x 64          (stride 4: 1 x 2 x 16)
    {2, 4, 5},   // 4 x 16 x 32         (stride 4: 1 x 4 x 8)
    {3, 4, 7},   // 8 x 16 x 128        (stride 8: 1 x 2 x 16)
};

void order_shape(int order, int &lz, int &ly, int &lx)
{
    lz = ly = lx = 0;
    if (order >= 2 && order < kVoxelOrders) {
        lz = kOrderShape[order - 2][0];
        ly = kOrderShape[order - 2][1];
        lx = kOrderShape[order - 2][2];
    }
}

}  // namespace

cudaError_t launch_order_permutation(const long long *d_c, int n, const int *dims, int order, int *d_perm,
                                     cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    int lz, ly, lx;
    order_shape(order, lz, ly, lx);
    unsigned long long *keys = nullptr;
    int *idx = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    cudaError_t e;
    if ((e = lib_malloc_async(reinterpret_cast<void **>(&keys), 2 * sizeof(unsigned long long) * (size_t)n, st)))
        return e;
    if ((e = lib_malloc_async(reinterpret_cast<void **>(&idx), sizeof(int) * (size_t)n, st))) {
        cudaFreeAsync(keys, st);
        return e;
    }
    index_keys_kernel<<<(n + 255) / 256, 256, 0, st>>>(d_c, n, dims[0], dims[1], dims[2], lz, ly, lx, keys, idx);
    e = cudaGetLastError();
    // the same keys, bit range and stable sort as launch_pack_coords_order
    const int bits = 39 + lz + ly + lx;
    if (!e)
        e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys + n, idx, d_perm, n, 0, bits, st);
    if (!e)
        e = lib_malloc_async(reinterpret_cast<void **>(&tmp), tmp_bytes, st);
    if (!e)
        e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys + n, idx, d_perm, n, 0, bits, st);
    if (tmp)
        cudaFreeAsync(tmp, st);
    cudaFreeAsync(keys, st);
    cudaFreeAsync(idx, st);
    return e;
}

cudaError_t launch_pack_coords_order(const long long *d_c, int n, const int *dims, int order, short4 *d_out,
                                     int *d_status, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    if (order <= 0)
        return launch_pack_coords(d_c, n, dims, d_out, d_status, st);
    int lz, ly, lx;
    order_shape(order, lz, ly, lx);
    unsigned long long *keys = nullptr, *vals = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    cudaError_t e;
    if ((e = lib_malloc_async(reinterpret_cast<void **>(&keys), 2 * sizeof(unsigned long long) * (size_t)n, st)))
        return e;
    if ((e = lib_malloc_async(reinterpret_cast<void **>(&vals), sizeof(unsigned long long) * (size_t)n, st))) {
        cudaFreeAsync(keys, st);
        return e;
    }
    unsigned long long *keys2 = keys + n;
    unsigned long long *out = reinterpret_cast<unsigned long long *>(d_out);
    pack_keys_kernel<<<(n + 255) / 256, 256, 0, st>>>(d_c, n, dims[0], dims[1], dims[2], lz, ly, lx, keys, vals,
                                                      d_status);
    e = cudaGetLastError();
    // 39 Morton bits above the in-block bits; the sort is stable, so equal keys
    // keep the list order
    const int bits = 39 + lz + ly + lx;
    if (!e)
        e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys2, vals, out, n, 0, bits, st);
    if (!e)
        e = lib_malloc_async(reinterpret_cast<void **>(&tmp), tmp_bytes, st);
    if (!e)
        e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys2, vals, out, n, 0, bits, st);
    if (tmp)
        cudaFreeAsync(tmp, st);
    cudaFreeAsync(keys, st);
    cudaFreeAsync(vals, st);
    return e;
}

}  // namespace anacor
