// Interpolation kernels of the gridding (absorption-map) mode.
//
// The reference's interpolation (AnACor/src/gridding_interpolation.c:100-163)
// takes, per reflection, the two legs' polar angles, reads each voxel's map
// value at both (nearest neighbour, :16-45, or GSL bilinear, :48-76) and
// averages exp(-(z_incident + z_diffracted)) over the voxels.  The host
// computes the grid rows and weights of every reflection exactly as the
// reference does (FP64, same expressions); one CTA per reflection then streams
// the voxels: with the map stored direction-major ([direction][voxel]) the
// two (or eight) rows a reflection reads are contiguous, so the kernel is a
// coalesced read of 2 x 4 bytes per voxel (HBM-bound), four voxels per 16-byte
// load.  For nearest lookups exp runs in FP32 on the FP32 sum of the two map
// values (within 1e-7 relative of the reference's FP64 sum and exp); bilinear
// lookups keep the FP64 weights and an FP64 range reduction.  The mean is a
// compensated FP32 sum, as in the absorption kernel.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "device_math.cuh"
#include "trace_launch.h"

namespace anacor {
namespace {

constexpr int kInterpBlock = 256;

template <class T>
__device__ __forceinline__ double leg_value(const T *mk, const long long *o, const double *w, bool linear)
{
    if (!linear)
        return (double)mk[o[0]];
    // (((w0 z0 + w1 z1) + w2 z2) + w3 z3): the bilinear sum's left-to-right order
    double z = __dmul_rn(w[0], (double)mk[o[0]]);
    z = __dadd_rn(z, __dmul_rn(w[1], (double)mk[o[1]]));
    z = __dadd_rn(z, __dmul_rn(w[2], (double)mk[o[2]]));
    return __dadd_rn(z, __dmul_rn(w[3], (double)mk[o[3]]));
}

template <class T, bool kVec4>
__global__ void __launch_bounds__(kInterpBlock) gridding_interp_kernel(const T *__restrict__ map, long long sK,
                                                                       long long sR, int n_vox,
                                                                       const InterpRow *__restrict__ rows,
                                                                       long long n_refl, int linear,
                                                                       double *__restrict__ out)
{
    __shared__ float red_s[kInterpBlock / 32], red_c[kInterpBlock / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (long long r = blockIdx.x; r < n_refl; r += gridDim.x) {
        long long o0[4], o1[4];
        double w0[4], w1[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            o0[j] = __ldg(&rows[r].row[0][j]) * sR;
            o1[j] = __ldg(&rows[r].row[1][j]) * sR;
            w0[j] = __ldg(&rows[r].w[0][j]);
            w1[j] = __ldg(&rows[r].w[1][j]);
        }
        float s = 0.0f, c = 0.0f;
        int k0 = 0;
        if (kVec4 && !linear) {
            // direction-major float map, nearest lookups: both rows are
            // contiguous, 16-byte aligned (row stride a multiple of 4 floats):
            // four voxels per load, exp in FP32 of the FP32 sum z_0 + z_1
            const float4 *r0 = reinterpret_cast<const float4 *>(map + o0[0]);
            const float4 *r1 = reinterpret_cast<const float4 *>(map + o1[0]);
            const int n4 = n_vox >> 2;
#pragma unroll 2
            for (int q = tid; q < n4; q += kInterpBlock) {
                const float4 a = __ldg(r0 + q), b = __ldg(r1 + q);
                const float t[4] = {expf(-(a.x + b.x)), expf(-(a.y + b.y)), expf(-(a.z + b.z)), expf(-(a.w + b.w))};
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    float ns, e;
                    two_sum(s, t[j], ns, e);
                    s = ns;
                    c += e;
                }
            }
            k0 = n4 << 2;
        }
        for (int k = k0 + tid; k < n_vox; k += kInterpBlock) {
            const T *mk = map + (long long)k * sK;
            const double a = __dadd_rn(leg_value(mk, o0, w0, linear), leg_value(mk, o1, w1, linear));
            float ns, e;
            two_sum(s, exp_neg(a), ns, e);
            s = ns;
            c += e;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float so = __shfl_down_sync(0xffffffffu, s, o);
            const float co = __shfl_down_sync(0xffffffffu, c, o);
            float ns, e;
            two_sum(s, so, ns, e);
            s = ns;
            c = c + co + e;
        }
        if (lane == 0) {
            red_s[warp] = s;
            red_c[warp] = c;
        }
        __syncthreads();
        if (tid == 0) {
            float bs = red_s[0], bc = red_c[0];
            for (int w = 1; w < kInterpBlock / 32; w++) {
                float ns, e;
                two_sum(bs, red_s[w], ns, e);
                bs = ns;
                bc = bc + red_c[w] + e;
            }
            out[r] = ((double)bs + (double)bc) / (double)n_vox;
        }
        __syncthreads();
    }
}

template <class T>
cudaError_t launch_interp(const T *map, long long sK, long long sR, int n_vox, const InterpRow *rows, long long n_refl,
                          int linear, double *out, cudaStream_t st)
{
    if (n_refl <= 0)
        return cudaSuccess;
    int dev = 0, sms = 148;
    if (cudaGetDevice(&dev) == cudaSuccess)
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long grid = std::min<long long>(n_refl, (long long)sms * 8);
    // the vectorised path: float rows (sK == 1) with a stride of whole float4s
    if (sizeof(T) == 4 && sK == 1 && sR % 4 == 0 && ((uintptr_t)map & 15) == 0)
        gridding_interp_kernel<T, true><<<(unsigned)grid, kInterpBlock, 0, st>>>(map, sK, sR, n_vox, rows, n_refl,
                                                                                 linear, out);
    else
        gridding_interp_kernel<T, false><<<(unsigned)grid, kInterpBlock, 0, st>>>(map, sK, sR, n_vox, rows, n_refl,
                                                                                  linear, out);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_gridding_interp_f32(const float *map, long long sK, long long sR, int n_vox, const InterpRow *rows,
                                       long long n_refl, int linear, double *out, cudaStream_t st)
{
    return launch_interp(map, sK, sR, n_vox, rows, n_refl, linear, out, st);
}

cudaError_t launch_gridding_interp_f64(const double *map, long long sK, long long sR, int n_vox,
                                       const InterpRow *rows, long long n_refl, int linear, double *out,
                                       cudaStream_t st)
{
    return launch_interp(map, sK, sR, n_vox, rows, n_refl, linear, out, st);
}

}  // namespace anacor
