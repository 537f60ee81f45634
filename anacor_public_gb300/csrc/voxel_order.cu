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

__global__ void pack_keys_kernel(const long long *__restrict__ c, int n, int dz, int dy, int dx,
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
    keys[i] = (spread3((unsigned)z) << 2) | (spread3((unsigned)y) << 1) | spread3((unsigned)x);
    const short4 p = make_short4((short)z, (short)y, (short)x, 0);
    vals[i] = *reinterpret_cast<const unsigned long long *>(&p);
}

__global__ void index_keys_kernel(const long long *__restrict__ c, int n, int dz, int dy, int dx,
                                  unsigned long long *__restrict__ keys, int *__restrict__ idx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    long long z = c[3 * i], y = c[3 * i + 1], x = c[3 * i + 2];
    if (z < 0 || z >= dz || y < 0 || y >= dy || x < 0 || x >= dx)
        z = y = x = 0;
    keys[i] = (spread3((unsigned)z) << 2) | (spread3((unsigned)y) << 1) | spread3((unsigned)x);
    idx[i] = i;
}

}  // namespace

cudaError_t launch_morton_permutation(const long long *d_c, int n, const int *dims, int *d_perm, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    unsigned long long *keys = nullptr;
    int *idx = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    cudaError_t e;
    if ((e = cudaMallocAsync(&keys, 2 * sizeof(unsigned long long) * (size_t)n, st)))
        return e;
    if ((e = cudaMallocAsync(&idx, sizeof(int) * (size_t)n, st))) {
        cudaFreeAsync(keys, st);
        return e;
    }
    index_keys_kernel<<<(n + 255) / 256, 256, 0, st>>>(d_c, n, dims[0], dims[1], dims[2], keys, idx);
    e = cudaGetLastError();
    // the same keys, bit range and stable sort as launch_pack_coords_morton
    if (!e)
        e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys + n, idx, d_perm, n, 0, 39, st);
    if (!e)
        e = cudaMallocAsync(&tmp, tmp_bytes, st);
    if (!e)
        e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys + n, idx, d_perm, n, 0, 39, st);
    if (tmp)
        cudaFreeAsync(tmp, st);
    cudaFreeAsync(keys, st);
    cudaFreeAsync(idx, st);
    return e;
}

cudaError_t launch_pack_coords_morton(const long long *d_c, int n, const int *dims, short4 *d_out, int *d_status,
                                      cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    unsigned long long *keys = nullptr, *vals = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    cudaError_t e;
    if ((e = cudaMallocAsync(&keys, 2 * sizeof(unsigned long long) * (size_t)n, st)))
        return e;
    if ((e = cudaMallocAsync(&vals, sizeof(unsigned long long) * (size_t)n, st))) {
        cudaFreeAsync(keys, st);
        return e;
    }
    unsigned long long *keys2 = keys + n;
    unsigned long long *out = reinterpret_cast<unsigned long long *>(d_out);
    pack_keys_kernel<<<(n + 255) / 256, 256, 0, st>>>(d_c, n, dims[0], dims[1], dims[2], keys, vals, d_status);
    e = cudaGetLastError();
    // 39 key bits; the sort is stable, so equal keys keep the list order
    if (!e)
        e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys2, vals, out, n, 0, 39, st);
    if (!e)
        e = cudaMallocAsync(&tmp, tmp_bytes, st);
    if (!e)
        e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys2, vals, out, n, 0, 39, st);
    if (tmp)
        cudaFreeAsync(tmp, st);
    cudaFreeAsync(keys, st);
    cudaFreeAsync(vals, st);
    return e;
}

}  // namespace anacor
