// Crystal-voxel sampling on the GPU, so that large volumes are uploaded once
// and never scanned on the host.
//
// The reference samples on the host (AnACor/utils/utils_rt.py:27-253):
// np.where(label == cr) lists the crystal voxels in C order, and the default
// 'even' method keeps entries np.linspace(0, M, num=n, endpoint=False,
// dtype=int) of that list, i.e. entry floor(j * (M / n)) for j < n.  Here a
// stable stream compaction (CUB DeviceSelect over the linear voxel index)
// produces the same C-order list on the device and a gather kernel applies the
// same FP64 index expression.  A stride lattice (z, y, x all multiples of s,
// the benchmark configurations' subsampling) is one more predicate.
#include <cub/device/device_reduce.cuh>
#include <cub/device/device_select.cuh>
#include <cuda_runtime.h>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/iterator/transform_iterator.h>
#include <stdint.h>

#include "trace_launch.h"

namespace anacor {
namespace {

struct IsSampled {
    const int8_t *vol;
    int dy, dx;
    int code;
    int stride;
    __host__ __device__ __forceinline__ bool operator()(const long long &i) const
    {
        if (vol[i] != code)
            return false;
        if (stride <= 1)
            return true;
        const long long yx = (long long)dy * dx;
        const int z = (int)(i / yx);
        const int r = (int)(i - (long long)z * yx);
        const int y = r / dx, x = r - y * dx;
        return z % stride == 0 && y % stride == 0 && x % stride == 0;
    }
};

struct AsCount {
    IsSampled p;
    __host__ __device__ __forceinline__ long long operator()(const long long &i) const { return p(i) ? 1 : 0; }
};

// out[j] = (z, y, x) of list entry k_j: k_j = j when step == 0, else
// numpy.linspace(0, M, n, endpoint=False, dtype=int)[j] = floor(j * (M / n) + 0.0)
__global__ void unravel_kernel(const long long *__restrict__ lin, long long n, double step, int dy, int dx,
                               long long *__restrict__ out)
{
    const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= n)
        return;
    const long long k = step > 0.0 ? (long long)floor(__dadd_rn(__dmul_rn((double)j, step), 0.0)) : j;
    const long long i = lin[k];
    const long long yx = (long long)dy * dx;
    const long long z = i / yx, r = i - z * yx;
    out[3 * j] = z;
    out[3 * j + 1] = r / dx;
    out[3 * j + 2] = r % dx;
}

}  // namespace

cudaError_t count_sampled_voxels(const int8_t *d_vol, const int *dims, int code, int stride, long long *d_count,
                                 cudaStream_t st)
{
    const long long n = (long long)dims[0] * dims[1] * dims[2];
    IsSampled p{d_vol, dims[1], dims[2], code, stride};
    thrust::counting_iterator<long long> idx(0);
    thrust::transform_iterator<AsCount, thrust::counting_iterator<long long>, long long> flags(idx, AsCount{p});
    size_t tmp_bytes = 0;
    void *tmp = nullptr;
    cudaError_t e = cub::DeviceReduce::Sum(nullptr, tmp_bytes, flags, d_count, (int)n, st);
    if (!e)
        e = lib_malloc_async(reinterpret_cast<void **>(&tmp), tmp_bytes, st);
    if (!e)
        e = cub::DeviceReduce::Sum(tmp, tmp_bytes, flags, d_count, (int)n, st);
    if (tmp)
        cudaFreeAsync(tmp, st);
    return e;
}

cudaError_t select_sampled_voxels(const int8_t *d_vol, const int *dims, int code, int stride, long long *d_lin,
                                  long long *d_count, cudaStream_t st)
{
    const long long n = (long long)dims[0] * dims[1] * dims[2];
    IsSampled p{d_vol, dims[1], dims[2], code, stride};
    thrust::counting_iterator<long long> idx(0);
    size_t tmp_bytes = 0;
    void *tmp = nullptr;
    cudaError_t e = cub::DeviceSelect::If(nullptr, tmp_bytes, idx, d_lin, d_count, (int)n, p, st);
    if (!e)
        e = lib_malloc_async(reinterpret_cast<void **>(&tmp), tmp_bytes, st);
    if (!e)
        e = cub::DeviceSelect::If(tmp, tmp_bytes, idx, d_lin, d_count, (int)n, p, st);
    if (tmp)
        cudaFreeAsync(tmp, st);
    return e;
}

cudaError_t unravel_voxels(const long long *d_lin, long long n_out, double step, const int *dims, long long *d_coords,
                           cudaStream_t st)
{
    if (n_out <= 0)
        return cudaSuccess;
    unravel_kernel<<<(unsigned)((n_out + 255) / 256), 256, 0, st>>>(d_lin, n_out, step, dims[1], dims[2], d_coords);
    return cudaGetLastError();
}

}  // namespace anacor
