// Learned surrogate of the absorption factor: an ensemble of small MLPs that
// map (omega, incident and diffracted unit vectors in the crystal frame) to
// log A_h, trained on the GPU on absorption factors the plain tracer computes.
//
// Network (per ensemble member): 7 inputs -> 64 Fourier features
// [sin 2pi(Bx), cos 2pi(Bx)] with a fixed seeded B (32 x 7; its omega column
// is integer so the features are periodic in omega) -> 4 hidden layers of 256
// with GELU -> 1 output, the standardised log A_h.  Weights are FP32 masters
// with BF16 copies in [out][in] and [in][out] order; every matrix product is a
// tcgen05 BF16 GEMM with FP32 accumulation in tensor memory (umma_gemm.cuh),
// all members in one launch.  Training is Adam on the mean squared error with
// hand-written forward, backward and optimiser kernels; one training step is
// captured in a CUDA graph and replayed.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <random>
#include <vector>

#include "anacor_gb300.h"
#include "anacor_internal.h"
#include "umma_gemm.cuh"

namespace anacor {
int report_status(int st, const char *msg);
}

using namespace anacor;
using bf16 = __nv_bfloat16;

namespace {

constexpr int kIn = 7;        // omega + two unit vectors
constexpr int kFeat = 64;     // Fourier features
constexpr int kWidth = 256;
constexpr int kDepth = 4;     // hidden layers

// parameter offsets of one member (FP32 masters)
__host__ __device__ constexpr long long off_w(int l) { return l == 0 ? 0 : 16640 + (long long)(l - 1) * 65792; }
__host__ __device__ constexpr long long off_b(int l) { return off_w(l) + (long long)kWidth * (l == 0 ? kFeat : kWidth); }
constexpr long long kOffW5 = 214016;
constexpr long long kOffB5 = 214272;
constexpr long long kParams = 214280;   // per member, padded to a multiple of 8
__host__ __device__ constexpr int in_dim(int l) { return l == 0 ? kFeat : kWidth; }
static_assert(off_b(3) + kWidth == kOffW5, "parameter layout");

constexpr int kSplitK = 16;             // K splits of the weight-gradient GEMMs
constexpr int kMaxMembers = 16;
constexpr int kPredictChunk = 1 << 18;  // rows per inference pass

enum Epi { kEpiStoreF32 = 0, kEpiBiasGelu = 1, kEpiGeluBwd = 2 };

struct GemmArgs {
    const bf16 *A;
    long long lda, sA;
    const bf16 *B;
    long long ldb, sB;
    int M, N, K;
    int ksplit;            // z = member * ksplit + split; 0 or 1 = no split
    int mode;
    const float *bias;
    long long sBias;
    float *of;             // fp32 [M][N]  (with ksplit > 1: one slice per z)
    long long ldf, sF;
    bf16 *ob;              // bf16 [M][N]
    long long ldob, sOb;
    bf16 *ot;              // bf16 [N][M]
    long long ldot, sOt;
    const float *aux;      // fp32 [M][N] pre-activation for the GELU derivative
    long long ldaux, sAux;
    int *err;
};

__device__ __forceinline__ float gelu(float x)
{
    return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}

__device__ __forceinline__ float gelu_grad(float x)
{
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.3989422804014327f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

// Stage one K-chunk of 64 of A (128 rows) and B (BN rows) into the canonical
// no-swizzle K-major tile layout with 16-byte cp.async copies.
template <int BN>
__device__ __forceinline__ void load_chunk(uint8_t *As, uint8_t *Bs, const bf16 *A, long long lda, const bf16 *B,
                                           long long ldb, int k0)
{
    for (int c = threadIdx.x; c < umma::kBM * 8; c += umma::kThreads) {
        const int r = c >> 3, kc = c & 7;
        umma::cp_async16(As + umma::tile_off(r, kc * 8), A + (long long)r * lda + k0 + kc * 8);
    }
    for (int c = threadIdx.x; c < BN * 8; c += umma::kThreads) {
        const int r = c >> 3, kc = c & 7;
        umma::cp_async16(Bs + umma::tile_off(r, kc * 8), B + (long long)r * ldb + k0 + kc * 8);
    }
    umma::cp_async_commit();
}

// One 128 x BN tile per CTA, two shared-memory stages: the copy of chunk k+1
// overlaps the tensor-core work on chunk k.  A stage is refilled only after
// the MMAs that read it have signalled their mbarrier.
template <int BN>
__global__ void __launch_bounds__(umma::kThreads, 1) gemm_kernel(GemmArgs g)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    constexpr int kStageA = umma::kBM * umma::kBK * 2, kStageB = BN * umma::kBK * 2;
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ks = g.ksplit > 1 ? g.ksplit : 1;
    const int z = blockIdx.z, e = z / ks, sp = z - e * ks;
    const int Kc = g.K / ks;
    const int m0 = blockIdx.y * umma::kBM, n0 = blockIdx.x * BN;
    const bf16 *A = g.A + e * g.sA + (long long)m0 * g.lda + (long long)sp * Kc;
    const bf16 *B = g.B + e * g.sB + (long long)n0 * g.ldb + (long long)sp * Kc;
    constexpr int kStage = kStageA + kStageB;   // stage s: A at s * kStage, B after it

    if (tid == 0) {
        umma::mbar_init(&bar[0], 1);
        umma::mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0)
        umma::tmem_alloc(&tslot, BN);
    umma::tc_fence_before();
    __syncthreads();
    umma::tc_fence_after();
    const uint32_t tmem = tslot;
    constexpr uint32_t idesc = umma::idesc_bf16_f32(BN);

    const int nk = Kc / umma::kBK;
    uint32_t phase[2] = {0u, 0u};
    bool ok = true;
    load_chunk<BN>(smem, smem + kStageA, A, g.lda, B, g.ldb, 0);
    for (int k = 0; k < nk; k++) {
        const int s = k & 1;
        umma::cp_async_wait_all();
        umma::fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            umma::tc_fence_after();
            const uint32_t a0 = umma::smem_u32(smem + s * kStage), b0 = a0 + kStageA;
#pragma unroll
            for (int kk = 0; kk < umma::kBK / 16; kk++) {
                const uint64_t ad = umma::smem_desc(a0 + kk * 256, 128, 1024);
                const uint64_t bd = umma::smem_desc(b0 + kk * 256, 128, 1024);
                umma::mma_bf16(tmem, ad, bd, idesc, (k > 0 || kk > 0) ? 1u : 0u);
            }
            umma::mma_commit(&bar[s]);
        }
        if (k + 1 < nk) {
            const int t = s ^ 1;
            if (k >= 1) {   // stage t was read by the MMAs of chunk k-1
                ok = umma::mbar_wait(&bar[t], phase[t]) && ok;
                phase[t] ^= 1u;
            }
            load_chunk<BN>(smem + t * kStage, smem + t * kStage + kStageA, A, g.lda, B, g.ldb, (k + 1) * umma::kBK);
        }
    }
    // the last commit covers every MMA issued before it
    ok = umma::mbar_wait(&bar[(nk - 1) & 1], phase[(nk - 1) & 1]) && ok;
    umma::tc_fence_after();
    ok = __all_sync(0xffffffffu, ok);
    if (!ok) {
        if (lane == 0)
            atomicOr(g.err, 1);
    } else {
        const int row = m0 + warp * 32 + lane;
        const long long zo = ks > 1 ? z : e;
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            umma::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            const int n = n0 + c0;
            if (g.mode == kEpiStoreF32) {
                float *o = g.of + zo * g.sF + (long long)row * g.ldf + n;
#pragma unroll
                for (int i = 0; i < 16; i += 4)
                    *reinterpret_cast<float4 *>(o + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                continue;
            }
            if (g.mode == kEpiBiasGelu) {
                const float *bias = g.bias + e * g.sBias + n;
#pragma unroll
                for (int i = 0; i < 16; i++)
                    v[i] += bias[i];
                if (g.of) {
                    float *o = g.of + e * g.sF + (long long)row * g.ldf + n;
#pragma unroll
                    for (int i = 0; i < 16; i += 4)
                        *reinterpret_cast<float4 *>(o + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                }
#pragma unroll
                for (int i = 0; i < 16; i++)
                    v[i] = gelu(v[i]);
            } else {   // kEpiGeluBwd
                const float *h = g.aux + e * g.sAux + (long long)row * g.ldaux + n;
#pragma unroll
                for (int i = 0; i < 16; i++)
                    v[i] *= gelu_grad(h[i]);
            }
            if (g.ob) {
                __align__(16) bf16 t[16];
#pragma unroll
                for (int i = 0; i < 16; i++)
                    t[i] = __float2bfloat16_rn(v[i]);
                bf16 *o = g.ob + e * g.sOb + (long long)row * g.ldob + n;
                *reinterpret_cast<uint4 *>(o) = *reinterpret_cast<const uint4 *>(t);
                *reinterpret_cast<uint4 *>(o + 8) = *reinterpret_cast<const uint4 *>(t + 8);
            }
            if (g.ot) {
                bf16 *o = g.ot + e * g.sOt + row;
#pragma unroll
                for (int i = 0; i < 16; i++)
                    o[(long long)(n + i) * g.ldot] = __float2bfloat16_rn(v[i]);
            }
        }
    }
    umma::tc_fence_before();
    __syncthreads();
    if (warp == 0)
        umma::tmem_dealloc(tmem, BN);
}

constexpr int gemm_smem(int bn) { return 2 * (umma::kBM + bn) * umma::kBK * 2; }

std::once_flag g_gemm_once[64];
cudaError_t g_gemm_init_err[64];

// opt every tile width into its shared-memory size once per device (outside
// any stream capture)
cudaError_t gemm_init()
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e)
        return e;
    if (dev < 0 || dev >= 64)
        return cudaErrorInvalidDevice;
    std::call_once(g_gemm_once[dev], [dev] {
        cudaError_t r = cudaFuncSetAttribute(gemm_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, gemm_smem(256));
        if (!r)
            r = cudaFuncSetAttribute(gemm_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, gemm_smem(128));
        if (!r)
            r = cudaFuncSetAttribute(gemm_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, gemm_smem(64));
        g_gemm_init_err[dev] = r;
    });
    return g_gemm_init_err[dev];
}

// tile width: the widest that still gives at least one CTA per SM
int pick_bn(int M, int N, int zcount)
{
    const int tiles_m = M / umma::kBM;
    for (int bn : {256, 128})
        if (N % bn == 0 && (long long)(N / bn) * tiles_m * zcount >= 148)
            return bn;
    if (N % 128 == 0)
        return 128;
    return N % 64 == 0 ? 64 : 0;
}

cudaError_t gemm(const GemmArgs &g, int members, cudaStream_t st)
{
    const int ks = g.ksplit > 1 ? g.ksplit : 1;
    if (g.M % umma::kBM || g.K % (umma::kBK * ks))
        return cudaErrorInvalidValue;
    const int bn = pick_bn(g.M, g.N, members * ks);
    if (!bn)
        return cudaErrorInvalidValue;
    dim3 grid(g.N / bn, g.M / umma::kBM, members * ks);
    if (bn == 256)
        gemm_kernel<256><<<grid, umma::kThreads, gemm_smem(256), st>>>(g);
    else if (bn == 128)
        gemm_kernel<128><<<grid, umma::kThreads, gemm_smem(128), st>>>(g);
    else
        gemm_kernel<64><<<grid, umma::kThreads, gemm_smem(64), st>>>(g);
    return cudaGetLastError();
}

// ------------------------------------------------------------ small kernels

struct Geometry {
    double xray[3], axis[3], F[9];
};

// x7 = (omega / 2pi wrapped to [0, 1), incident and diffracted unit vectors
// in the crystal frame).  The rotation is T = (R(axis, omega) F)^T as the
// reference builds it (AnACor/src/ray_tracing.c:397-407, matrices.h:49-68).
__global__ void inputs_kernel(const double *__restrict__ omega, const double *__restrict__ s1, long long n,
                              Geometry geo, float *__restrict__ x7)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const double w = omega[i];
    double c, s;
    sincos(w, &s, &c);
    const double x = geo.axis[0], y = geo.axis[1], z = geo.axis[2], k = 1.0 - c;
    const double R[9] = {c + x * x * k,      x * y * k - z * s, y * s + x * z * k,
                         z * s + x * y * k,  c + y * y * k,     -x * s + y * z * k,
                         -y * s + x * z * k, x * s + y * z * k, c + z * z * k};
    double M[9];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int q = 0; q < 3; q++)
            M[r * 3 + q] = R[r * 3 + 0] * geo.F[q] + R[r * 3 + 1] * geo.F[3 + q] + R[r * 3 + 2] * geo.F[6 + q];
    double a[3], b[3];
    const double *sv = s1 + 3 * i;
#pragma unroll
    for (int r = 0; r < 3; r++) {   // T = M^T
        a[r] = M[r] * geo.xray[0] + M[3 + r] * geo.xray[1] + M[6 + r] * geo.xray[2];
        b[r] = M[r] * sv[0] + M[3 + r] * sv[1] + M[6 + r] * sv[2];
    }
    const double na = rsqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    const double nb = rsqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
    float *o = x7 + 7 * i;
    const double turns = w * 0.15915494309189535;
    o[0] = (float)(turns - floor(turns));
#pragma unroll
    for (int r = 0; r < 3; r++) {
        o[1 + r] = (float)(a[r] * na);
        o[4 + r] = (float)(b[r] * nb);
    }
}

// Fourier features of rows 0..n-1 (rows n..rows_pad-1 are written as zeros)
__global__ void features_kernel(const float *__restrict__ x7, const float *__restrict__ Bf, long long n,
                                long long rows_pad, bf16 *__restrict__ out)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long i = t / (kFeat / 2);
    const int j = (int)(t % (kFeat / 2));
    if (i >= rows_pad)
        return;
    float sv = 0.0f, cv = 0.0f;
    if (i < n) {
        const float *x = x7 + 7 * i;
        float p = 0.0f;
#pragma unroll
        for (int q = 0; q < kIn; q++)
            p += Bf[j * kIn + q] * x[q];
        sincospif(2.0f * p, &sv, &cv);
    }
    out[i * kFeat + j] = __float2bfloat16_rn(sv);
    out[i * kFeat + kFeat / 2 + j] = __float2bfloat16_rn(cv);
}

__device__ __forceinline__ uint32_t mix32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

// training batch of every member: rows drawn with replacement by a hash of
// (seed, step, member, row); X0 [E][batch][64], X0T [E][64][batch]
__global__ void gather_kernel(const bf16 *__restrict__ feat, const float *__restrict__ target, long long n_data,
                              int batch, const unsigned *__restrict__ step, uint32_t seed, bf16 *__restrict__ X0,
                              bf16 *__restrict__ X0T, float *__restrict__ tb)
{
    const int e = blockIdx.y;
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= batch)
        return;
    const uint32_t h = mix32(seed ^ mix32(*step * 0x9E3779B9u ^ mix32((uint32_t)e * 0x85EBCA6Bu ^ (uint32_t)b)));
    const long long r = (long long)(((uint64_t)h * (uint64_t)n_data) >> 32);
    const uint4 *src = reinterpret_cast<const uint4 *>(feat + r * kFeat);
    uint4 *dst = reinterpret_cast<uint4 *>(X0 + ((long long)e * batch + b) * kFeat);
#pragma unroll
    for (int q = 0; q < kFeat / 8; q++)
        dst[q] = src[q];
    const bf16 *f = feat + r * kFeat;
    bf16 *t = X0T + (long long)e * kFeat * batch + b;
#pragma unroll 8
    for (int q = 0; q < kFeat; q++)
        t[(long long)q * batch] = f[q];
    tb[(long long)e * batch + b] = target[r];
}

// output layer, one warp per row: y = A4 . w5 + b5; when training also the
// loss and dH4 = bf16((dL/dy) w5 * gelu'(H4)) in [row][256] and [256][row]
__global__ void head_kernel(const bf16 *__restrict__ A4, const float *__restrict__ H4,
                            const float *__restrict__ params, const float *__restrict__ tb, int rows, int train,
                            float *__restrict__ y, float *__restrict__ dy, bf16 *__restrict__ dH, bf16 *__restrict__ dHT,
                            float *__restrict__ loss_acc)
{
    const int e = blockIdx.y;
    const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (r >= rows)
        return;
    const float *P = params + e * kParams;
    const long long base = (long long)e * rows + r;
    const uint4 av = reinterpret_cast<const uint4 *>(A4 + base * kWidth)[lane];
    const bf16 *a = reinterpret_cast<const bf16 *>(&av);
    float acc = 0.0f;
#pragma unroll
    for (int q = 0; q < 8; q++)
        acc += __bfloat162float(a[q]) * P[kOffW5 + lane * 8 + q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
    const float out = acc + P[kOffB5];
    if (lane == 0)
        y[base] = out;
    if (!train)
        return;
    const float diff = out - tb[base];
    const float g = 2.0f * diff / (float)rows;
    if (lane == 0) {
        dy[base] = g;
        atomicAdd(loss_acc + e, diff * diff / (float)rows);
    }
    const float *h = H4 + base * kWidth + lane * 8;
    __align__(16) bf16 t[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
        t[q] = __float2bfloat16_rn(g * P[kOffW5 + lane * 8 + q] * gelu_grad(h[q]));
        dHT[((long long)e * kWidth + lane * 8 + q) * rows + r] = t[q];
    }
    reinterpret_cast<uint4 *>(dH + base * kWidth)[lane] = *reinterpret_cast<const uint4 *>(t);
}

// out[e][n] = sum_b M[e][n][b] * (w ? w[e][b] : 1), one block per (n, e)
__global__ void rowsum_kernel(const bf16 *__restrict__ Mb, const float *__restrict__ w, int len, long long sM,
                              long long sw, float *__restrict__ out, long long sOut)
{
    const int e = blockIdx.y, n = blockIdx.x;
    const bf16 *m = Mb + e * sM + (long long)n * len;
    const float *ww = w ? w + e * sw : nullptr;
    float acc = 0.0f;
    for (int b = threadIdx.x; b < len; b += blockDim.x)
        acc += __bfloat162float(m[b]) * (ww ? ww[b] : 1.0f);
    __shared__ float red[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0)
            out[e * sOut + n] = v;
    }
}

// sum_b v[e][b] (output bias gradient), one block per member
__global__ void vecsum_kernel(const float *__restrict__ v, int len, float *__restrict__ out, long long sOut)
{
    const int e = blockIdx.x;
    float acc = 0.0f;
    for (int b = threadIdx.x; b < len; b += blockDim.x)
        acc += v[(long long)e * len + b];
    __shared__ float red[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        float s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0)
            out[e * sOut] = s;
    }
}

// weight gradient of one layer from its K-split partial products, summed in
// split order: grad[e][i] = sum_s part[e * ks + s][i]
__global__ void splitk_reduce_kernel(const float *__restrict__ part, int ks, long long len, float *__restrict__ grad,
                                     long long sGrad)
{
    const int e = blockIdx.y;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= len)
        return;
    float acc = 0.0f;
    for (int s = 0; s < ks; s++)
        acc += part[((long long)e * ks + s) * len + i];
    grad[e * sGrad + i] = acc;
}

struct AdamArgs {
    float lr_max, lr_min, b1, b2, eps;
    unsigned total;   // cosine decay from lr_max to lr_min over `total` steps
};

// Adam on every member's FP32 masters, step t = *step + 1
__global__ void adam_kernel(float *__restrict__ p, float *__restrict__ m, float *__restrict__ v,
                            const float *__restrict__ g, long long n, const unsigned *__restrict__ step, AdamArgs a)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const unsigned s = *step;
    const float t = (float)(s + 1u);
    const float frac = a.total ? fminf((float)s / (float)a.total, 1.0f) : 0.0f;
    const float lr = a.lr_min + (a.lr_max - a.lr_min) * 0.5f * (1.0f + cospif(frac));
    const float gi = g[i];
    const float mi = a.b1 * m[i] + (1.0f - a.b1) * gi;
    const float vi = a.b2 * v[i] + (1.0f - a.b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.0f - powf(a.b1, t));
    const float vh = vi / (1.0f - powf(a.b2, t));
    p[i] -= lr * mh / (sqrtf(vh) + a.eps);
}

// BF16 copies of layer l's weights: W[e][n][k] and WT[e][k][n]
__global__ void convert_kernel(const float *__restrict__ params, int l, int E, bf16 *__restrict__ W,
                               bf16 *__restrict__ WT)
{
    const int K = in_dim(l);
    const long long per = (long long)kWidth * K;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= per * E)
        return;
    const int e = (int)(i / per);
    const long long r = i - e * per;
    const int n = (int)(r / K), k = (int)(r % K);
    const bf16 w = __float2bfloat16_rn(params[e * kParams + off_w(l) + r]);
    W[i] = w;
    WT[e * per + (long long)k * kWidth + n] = w;
}

__global__ void zero_kernel(float *p, int n)
{
    if ((int)threadIdx.x < n)
        p[threadIdx.x] = 0.0f;
}

__global__ void step_done_kernel(unsigned *step, float *loss_hist, const float *loss_acc, int E, int hist_len)
{
    if (threadIdx.x == 0) {
        const unsigned s = *step;
        if ((int)s < hist_len) {
            float acc = 0.0f;
            for (int e = 0; e < E; e++)
                acc += loss_acc[e];
            loss_hist[s] = acc / (float)E;
        }
        *step = s + 1u;
    }
}

// ensemble mean of A_h = exp(mu + sd * y) and its relative spread (standard
// deviation over members / mean)
__global__ void ensemble_kernel(const float *__restrict__ y, int E, long long rows, long long ld, float mu, float sd,
                                float *__restrict__ mean, float *__restrict__ spread, float *__restrict__ members,
                                long long ldm)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= rows)
        return;
    // two passes (mean, then squared deviations): the members agree to
    // ~1e-3, so a one-pass E[a^2] - E[a]^2 would cancel away the spread
    float a[kMaxMembers];
    float s = 0.0f;
#pragma unroll
    for (int e = 0; e < kMaxMembers; e++) {
        if (e < E) {
            const float la = mu + sd * y[e * ld + i];
            if (members)
                members[e * ldm + i] = la;
            a[e] = expf(la);
            s += a[e];
        }
    }
    const float m = s / E;
    float v = 0.0f;
#pragma unroll
    for (int e = 0; e < kMaxMembers; e++)
        if (e < E)
            v += (a[e] - m) * (a[e] - m);
    mean[i] = m;
    spread[i] = sqrtf(v / E) / m;
}

// audit flags: bit 0 = in the seeded random audit sample, bit 1 = ensemble
// spread above the threshold (or not finite)
__global__ void audit_kernel(const float *__restrict__ spread, long long n, uint32_t seed, uint32_t cut,
                             float threshold, uint8_t *__restrict__ flags)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t h = mix32(seed ^ mix32((uint32_t)i ^ mix32((uint32_t)(i >> 32) + 0x632BE5ABu)));
    const float sp = spread[i];
    flags[i] = (uint8_t)((h < cut ? 1u : 0u) | (!(sp <= threshold) ? 2u : 0u));
}

// ------------------------------------------------- fused inference kernel
//
// The four hidden layers and the head of every member for a 128-row tile in
// one persistent kernel: the tile's Fourier features and each layer's
// activations stay in shared memory, the accumulators in tensor memory, and
// only the weights stream in (from L2: 1.7 MB for four members), as 16 KiB
// K-chunks copied by the bulk-copy engine (cp.async.bulk) into a 4-stage ring
// kept three chunks ahead of the MMAs.
//
// Two members are in flight at a time, on two "streams" with their own
// 256-column TMEM accumulator and 128 x 256 activation tile: while the twelve
// epilogue warps apply bias and GELU to one member's layer (the expensive
// part: an erf per element), the control warp issues the other member's MMAs
// and weight copies.  The streams hand over through mbarriers: acc_full[s]
// (the layer's MMAs are done), act_ready[s] (its epilogue has read the
// accumulator and written the next operand), x0_ready (the tile's features).
// The arithmetic is the layered path's: the same MMAs in the same K order,
// the same epilogue expressions and the head's and ensemble's summation
// orders, so the outputs are the same numbers without the per-layer round
// trips through HBM.

constexpr int kWChunkK = 32;                                          // K per weight chunk
constexpr int kChunkBytes = kWidth * kWChunkK * 2;                    // 256 rows x 32 BF16 = 16 KiB
constexpr int kChunksPerMember = (kFeat + (kDepth - 1) * kWidth) / kWChunkK;   // 2 + 3 * 8 = 26
constexpr int kInferStages = 4;
constexpr int kEpiWarps = 12;                                         // three per TMEM lane quarter
constexpr int kEpiThreads = 32 * kEpiWarps;
constexpr int kInferThreads = kEpiThreads + 32;                       // + the control warp
constexpr int kTileRows = umma::kBM;                                  // 128
constexpr int kActChunk = kTileRows * umma::kBK * 2;                 // 128 rows x 64 BF16 = 16 KiB
constexpr int kActBytes = (kWidth / umma::kBK) * kActChunk;          // 64 KiB
constexpr int kMemberConsts = kDepth * kWidth + kWidth + 2;           // biases, w5, b5, pad
constexpr int kConstBytes = ((kMemberConsts * 4 + 15) / 16) * 16;
constexpr int kGStride = 33;                                          // head partials per row (32 + pad)
constexpr int kInferMaxMembers = 8;
constexpr int kOffInferAct = kInferStages * kChunkBytes;             // two activation tiles
constexpr int kOffInferX0 = kOffInferAct + 2 * kActBytes;
constexpr int kOffInferC = kOffInferX0 + kActChunk;                  // two members' constants
constexpr int kOffInferY = kOffInferC + 2 * kConstBytes;
constexpr int kInferSmem = kOffInferY + kInferMaxMembers * kTileRows * 4;
// the head's partial sums live in the stream's activation tile, which the
// last layer's MMAs have finished reading when the head writes them
static_assert(kTileRows * kGStride * 4 <= kActBytes, "head partials fit the activation tile");
static_assert(kInferSmem + 512 <= 227 * 1024, "fused inference shared memory");

// byte offset of element (r, k) of a rows x 32 K-major weight chunk in the
// canonical no-swizzle layout (8-row groups 512 bytes apart)
__host__ __device__ constexpr uint32_t wchunk_off(int r, int k)
{
    return (uint32_t)(((r >> 3) * (kWChunkK / 8) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// The work of one tile as jobs (stream s, member e, layer l), in the order
// both the control warp and the epilogue warps take them: members in pairs
// (2p on stream 0, 2p + 1 on stream 1), layer by layer, alternating streams;
// an odd last member alone on stream 0.
__host__ __device__ inline void job_of(int j, int E, int &s, int &e, int &l)
{
    const int pairs = E / 2;
    if (j < pairs * 2 * kDepth) {
        const int p = j / (2 * kDepth), r = j % (2 * kDepth);
        l = r / 2;
        s = r % 2;
        e = 2 * p + s;
        return;
    }
    s = 0;
    e = E - 1;
    l = j - pairs * 2 * kDepth;
}

__host__ __device__ constexpr int job_chunks(int l) { return in_dim(l) / kWChunkK; }

// Weight chunk c of the image (the control warp's consumption order):
// member e, layer l, K-chunk kq
__host__ __device__ inline void chunk_of(int c, int E, int &e, int &l, int &kq)
{
    int j = 0;
    int s = 0;
    for (;; j++) {
        job_of(j, E, s, e, l);
        const int n = job_chunks(l);
        if (c < n) {
            kq = c;
            return;
        }
        c -= n;
    }
}

struct WeightPtrs {
    const bf16 *w[kDepth];
};

// The weight image: for every member its 26 K-chunks of W_l [256][K], each in
// the canonical no-swizzle K-major layout of a 256 x 32 tile, in the order the
// fused kernel consumes them.
__global__ void weight_image_kernel(WeightPtrs W, int E, uint8_t *__restrict__ img)
{
    constexpr int kPieces = kChunkBytes / 16;   // 16-byte pieces (8 BF16 along K) per chunk
    const long long total = (long long)E * kChunksPerMember * kPieces;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t / kPieces);
        const int p = (int)(t - (long long)c * kPieces);
        int e, l, kq;
        chunk_of(c, E, e, l, kq);
        const int K = in_dim(l);
        const int r = p >> 2, kc = p & 3;
        const bf16 *src = W.w[l] + (long long)e * kWidth * K + (long long)r * K + kq * kWChunkK + kc * 8;
        *reinterpret_cast<uint4 *>(img + (long long)c * kChunkBytes + wchunk_off(r, kc * 8)) =
            *reinterpret_cast<const uint4 *>(src);
    }
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(umma::smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(umma::smem_u32(bar)) : "memory");
}

// bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from global to this CTA's shared memory, completing on `bar`
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     umma::smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(umma::smem_u32(bar))
                 : "memory");
}

// bounded wait that also gives up once another thread has aborted the CTA;
// a thread whose own wait runs out raises the abort flag
__device__ __forceinline__ bool wait_or_abort(uint64_t *bar, uint32_t parity, volatile int *abort)
{
    const uint32_t addr = umma::smem_u32(bar);
    for (unsigned it = 0; it < umma::kWaitLimit; it++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done)
            return true;
        if ((it & 255u) == 255u && *abort)
            return false;
    }
    *abort = 1;
    return false;
}

// barrier over the epilogue warps (named barrier 1) that also ANDs a
// predicate across them: every epilogue thread takes the same branch after it
__device__ __forceinline__ bool epi_sync_and(bool ok)
{
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, 1, %2, p;\n selp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)ok), "r"(kEpiThreads)
        : "memory");
    return r != 0;
}

struct InferArgs {
    const float *x7;
    long long n;
    const float *Bf;
    const uint8_t *wimg;
    const float *params;
    int E;
    float mu, sd;
    float *mean, *spread, *members;
    long long ldm;
    int *err;
};

// member constant i (biases of the four layers, w5, b5) from the FP32 masters
__device__ __forceinline__ float member_const(const float *P, int i)
{
    if (i < kDepth * kWidth)
        return P[off_b(i / kWidth) + (i % kWidth)];
    if (i < kDepth * kWidth + kWidth)
        return P[kOffW5 + (i - kDepth * kWidth)];
    return i == kDepth * kWidth + kWidth ? P[kOffB5] : 0.0f;
}

__global__ void __launch_bounds__(kInferThreads, 1) infer_kernel(InferArgs a)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t full[kInferStages], empty[kInferStages], acc_full[2], act_ready[2], x0_ready;
    __shared__ uint32_t tslot;
    __shared__ int s_abort;
    uint8_t *Ws = smem;
    uint8_t *X0s = smem + kOffInferX0;
    float *ys = reinterpret_cast<float *>(smem + kOffInferY);
    volatile int *abort = &s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long tiles = (a.n + kTileRows - 1) / kTileRows;
    const long long my_tiles = tiles > (long long)blockIdx.x ? (tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int jobs = kDepth * a.E;

    if (tid == 0) {
        for (int s = 0; s < kInferStages; s++) {
            umma::mbar_init(&full[s], 1);
            umma::mbar_init(&empty[s], 1);
        }
        for (int s = 0; s < 2; s++) {
            umma::mbar_init(&acc_full[s], 1);
            umma::mbar_init(&act_ready[s], kEpiThreads);
        }
        umma::mbar_init(&x0_ready, kEpiThreads);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0)
        umma::tmem_alloc(&tslot, 2 * kWidth);   // one accumulator per stream
    umma::tc_fence_before();
    __syncthreads();
    umma::tc_fence_after();
    const uint32_t tmem = tslot;

    if (warp == kEpiWarps) {
        // ---- control warp: lane 0 issues the weight copies and the MMAs
        if (lane == 0) {
            constexpr uint32_t idesc = umma::idesc_bf16_f32(kWidth);
            const long long per_tile = (long long)a.E * kChunksPerMember;
            const long long total = my_tiles * per_tile;
            long long q_issue = 0, q_use = 0;
            uint32_t kjob[2] = {0u, 0u};
            bool ok = true;
            // load weight chunk q into stage q % kInferStages once the MMAs that
            // read that stage's previous chunk are done
            auto issue = [&](long long q) -> bool {
                const int st = (int)(q % kInferStages);
                if (q >= kInferStages &&
                    !wait_or_abort(&empty[st], (uint32_t)((q / kInferStages - 1) & 1), abort))
                    return false;
                mbar_expect_tx(&full[st], kChunkBytes);
                bulk_g2s(Ws + st * kChunkBytes, a.wimg + (q % per_tile) * kChunkBytes, kChunkBytes, &full[st]);
                return true;
            };
            for (; q_issue < total && q_issue < kInferStages - 1 && ok; q_issue++)
                ok = issue(q_issue);
            for (long long ti = 0; ti < my_tiles && ok; ti++) {
                for (int j = 0; j < jobs && ok; j++) {
                    int s, e, l;
                    job_of(j, a.E, s, e, l);
                    // the operand: the tile's features (layer 0) or the stream's
                    // previous epilogue, which also freed its accumulator
                    if (j == 0)
                        ok = wait_or_abort(&x0_ready, (uint32_t)(ti & 1), abort);
                    if (ok && kjob[s] > 0)
                        ok = wait_or_abort(&act_ready[s], (kjob[s] - 1u) & 1u, abort);
                    if (!ok)
                        break;
                    umma::tc_fence_after();
                    const uint8_t *A = l == 0 ? X0s : smem + kOffInferAct + s * kActBytes;
                    const int nk = job_chunks(l);
                    for (int kc = 0; kc < nk; kc++, q_use++) {
                        const int st = (int)(q_use % kInferStages);
                        if (!wait_or_abort(&full[st], (uint32_t)((q_use / kInferStages) & 1), abort)) {
                            ok = false;
                            break;
                        }
#pragma unroll
                        for (int kk = 0; kk < kWChunkK / 16; kk++) {
                            const int k0 = kc * kWChunkK + kk * 16;
                            const uint32_t a0 = umma::smem_u32(A + (k0 / umma::kBK) * kActChunk) +
                                                (uint32_t)((k0 % umma::kBK) / 16) * 256;
                            const uint32_t b0 = umma::smem_u32(Ws + st * kChunkBytes) + (uint32_t)kk * 256;
                            umma::mma_bf16(tmem + (uint32_t)(s * kWidth), umma::smem_desc(a0, 128, 1024),
                                           umma::smem_desc(b0, 128, 512), idesc, (kc > 0 || kk > 0) ? 1u : 0u);
                        }
                        umma::mma_commit(&empty[st]);
                        if (q_issue < total) {
                            if (!issue(q_issue)) {
                                ok = false;
                                q_use++;
                                break;
                            }
                            q_issue++;
                        }
                    }
                    umma::mma_commit(&acc_full[s]);
                    kjob[s]++;
                }
            }
            // copies still in flight complete before the CTA's shared memory
            // goes away (bounded: a failed copy does not hold the exit)
            for (long long q = q_use; q < q_issue; q++)
                wait_or_abort(&full[q % kInferStages], (uint32_t)((q / kInferStages) & 1), abort);
            if (!ok)
                *abort = 1;
        }
    } else {
        // ---- epilogue warps: features, bias + GELU per layer, head, ensemble
        const int rl = 32 * (warp & 3) + lane;          // this thread's row of the tile (TMEM lane)
        // its accumulator columns: warps 0-3 take 0..95, 4-7 96..175, 8-11 176..255
        const int cb = warp < 4 ? 0 : (warp < 8 ? 96 : 176);
        const int ce = warp < 4 ? 96 : (warp < 8 ? 176 : kWidth);
        uint32_t ejob[2] = {0u, 0u};
        bool ok = true;
        for (long long ti = 0; ti < my_tiles && ok; ti++) {
            const long long row0 = (blockIdx.x + ti * gridDim.x) * kTileRows;
            if (tid < 2 * kTileRows) {
                // Fourier features of the tile (features_kernel's expressions),
                // BF16 into the layer-0 operand tile; rows past n are zeros
                const int r = tid >> 1, h = tid & 1;
                const long long i = row0 + r;
                float sv[16], cv[16];
#pragma unroll
                for (int jj = 0; jj < 16; jj++) {
                    sv[jj] = 0.0f;
                    cv[jj] = 0.0f;
                }
                if (i < a.n) {
                    const float *x = a.x7 + 7 * i;
#pragma unroll
                    for (int jj = 0; jj < 16; jj++) {
                        const int j = 16 * h + jj;
                        float p = 0.0f;
#pragma unroll
                        for (int q = 0; q < kIn; q++)
                            p += a.Bf[j * kIn + q] * x[q];
                        sincospif(2.0f * p, &sv[jj], &cv[jj]);
                    }
                }
#pragma unroll
                for (int part = 0; part < 4; part++) {   // features 16h.. (sin) and 32+16h.. (cos)
                    const float *src = part < 2 ? sv + 8 * part : cv + 8 * (part - 2);
                    const int f0 = (part < 2 ? 0 : kFeat / 2) + 16 * h + 8 * (part & 1);
                    __align__(16) bf16 t[8];
#pragma unroll
                    for (int q = 0; q < 8; q++)
                        t[q] = __float2bfloat16_rn(src[q]);
                    *reinterpret_cast<uint4 *>(X0s + umma::tile_off(r, f0)) = *reinterpret_cast<const uint4 *>(t);
                }
            }
            umma::fence_async_smem();
            mbar_arrive(&x0_ready);
            for (int j = 0; j < jobs; j++) {
                int s, e, l;
                job_of(j, a.E, s, e, l);
                float *cst = reinterpret_cast<float *>(smem + kOffInferC + s * kConstBytes);
                uint8_t *Act = smem + kOffInferAct + s * kActBytes;
                if (l == 0) {
                    // this member's constants (the stream's previous member is done with them)
                    for (int i = tid; i < kMemberConsts; i += kEpiThreads)
                        cst[i] = member_const(a.params + (long long)e * kParams, i);
                }
                ok = wait_or_abort(&acc_full[s], ejob[s] & 1u, abort) && ok;
                ejob[s]++;
                ok = epi_sync_and(ok);   // also publishes the constants
                if (!ok)
                    break;
                umma::tc_fence_after();
                const float *bias = cst + l * kWidth;
                const float *w5 = cst + kDepth * kWidth;
                float *gs = reinterpret_cast<float *>(Act);
                for (int c0 = cb; c0 < ce; c0 += 16) {
                    float v[16];
                    umma::tmem_ld16(tmem + (uint32_t)(s * kWidth) + ((uint32_t)(32 * (warp & 3)) << 16) +
                                        (uint32_t)c0,
                                    v);
#pragma unroll
                    for (int q = 0; q < 16; q++)
                        v[q] = gelu(v[q] + bias[c0 + q]);
                    __align__(16) __nv_bfloat162 t2[8];
#pragma unroll
                    for (int q = 0; q < 8; q++)
                        t2[q] = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
                    const bf16 *t = reinterpret_cast<const bf16 *>(t2);
                    if (l < kDepth - 1) {
                        uint8_t *dst = Act + (c0 / umma::kBK) * kActChunk;
                        const int k = c0 % umma::kBK;
                        *reinterpret_cast<uint4 *>(dst + umma::tile_off(rl, k)) = *reinterpret_cast<const uint4 *>(t);
                        *reinterpret_cast<uint4 *>(dst + umma::tile_off(rl, k + 8)) =
                            *reinterpret_cast<const uint4 *>(t + 8);
                    } else {
                        // the head's per-8-column partial sums, as head_kernel's lanes form them
#pragma unroll
                        for (int g = 0; g < 2; g++) {
                            float acc = 0.0f;
#pragma unroll
                            for (int q = 0; q < 8; q++)
                                acc += __bfloat162float(t[8 * g + q]) * w5[c0 + 8 * g + q];
                            gs[rl * kGStride + (c0 + 8 * g) / 8] = acc;
                        }
                    }
                }
                umma::tc_fence_before();
                umma::fence_async_smem();
                if (l == kDepth - 1) {
                    epi_sync_and(true);
                    if (tid < kTileRows) {
                        // head_kernel's shuffle tree over the 32 partial sums (lane 0's order)
                        float g[32];
#pragma unroll
                        for (int jj = 0; jj < 32; jj++)
                            g[jj] = gs[tid * kGStride + jj];
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                            for (int jj = 0; jj < o; jj++)
                                g[jj] = g[jj] + g[jj + o];
                        ys[e * kTileRows + tid] = g[0] + cst[kDepth * kWidth + kWidth];
                    }
                    epi_sync_and(true);
                }
                mbar_arrive(&act_ready[s]);
            }
            if (!ok)
                break;
            if (tid < kTileRows && row0 + tid < a.n) {
                // ensemble_kernel's statistics (this thread's own row of ys)
                const long long i = row0 + tid;
                float av[kInferMaxMembers];
                float sum = 0.0f;
#pragma unroll
                for (int e = 0; e < kInferMaxMembers; e++) {
                    if (e < a.E) {
                        const float la = a.mu + a.sd * ys[e * kTileRows + tid];
                        if (a.members)
                            a.members[e * a.ldm + i] = la;
                        av[e] = expf(la);
                        sum += av[e];
                    }
                }
                const float m = sum / a.E;
                float var = 0.0f;
#pragma unroll
                for (int e = 0; e < kInferMaxMembers; e++)
                    if (e < a.E)
                        var += (av[e] - m) * (av[e] - m);
                a.mean[i] = m;
                a.spread[i] = sqrtf(var / a.E) / m;
            }
        }
    }
    umma::tc_fence_before();
    __syncthreads();
    if (tid == 0 && s_abort)
        atomicOr(a.err, 1);
    if (warp == 0)
        umma::tmem_dealloc(tmem, 2 * kWidth);
}

// The error path of the tensor-core kernels' bounded waits, on its own: a CTA
// allocates tensor memory as they do, waits for an mbarrier phase that
// nothing completes (an arrival count of 2 with one arrival) with an
// iteration limit, then records the error, releases the tensor memory and
// returns.
__global__ void wait_guard_kernel(unsigned limit, int *err)
{
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    if (threadIdx.x == 0) {
        umma::mbar_init(&bar, 2);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x < 32)
        umma::tmem_alloc(&tslot, 32);
    umma::tc_fence_before();
    __syncthreads();
    umma::tc_fence_after();
    if (threadIdx.x == 0)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(umma::smem_u32(&bar)) : "memory");
    const bool ok = umma::mbar_wait(&bar, 0u, limit);
    if (!__syncthreads_and(ok) && threadIdx.x == 0)
        atomicOr(err, 1);
    umma::tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32)
        umma::tmem_dealloc(tslot, 32);
}

std::once_flag g_infer_once[64];
cudaError_t g_infer_init_err[64];

// opt the fused kernel into its shared-memory size once per device
cudaError_t infer_init(int dev)
{
    if (dev < 0 || dev >= 64)
        return cudaErrorInvalidDevice;
    std::call_once(g_infer_once[dev], [dev] {
        g_infer_init_err[dev] =
            cudaFuncSetAttribute(infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kInferSmem);
    });
    return g_infer_init_err[dev];
}

}  // namespace

// ------------------------------------------------------------------ state

struct anacor_surrogate {
    int E = 4;
    uint32_t seed = 0;
    cudaStream_t st = nullptr;
    float *params = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *part = nullptr;
    bf16 *W[kDepth] = {}, *WT[kDepth] = {};
    float *Bf = nullptr;                    // Fourier matrix [32][7]
    double t_mean = 0.0, t_std = 1.0;       // log A_h = t_mean + t_std * y
    // training data
    long long n_data = 0;
    float *target = nullptr;
    bf16 *feat = nullptr;
    // workspace for `rows` rows per member
    int rows = 0;
    bool train_ws = false;
    bf16 *X0 = nullptr, *X0T = nullptr;
    float *H[kDepth] = {};
    bf16 *A[kDepth] = {}, *AT[kDepth] = {};
    bf16 *dH = nullptr, *dHT = nullptr, *dH2 = nullptr, *dHT2 = nullptr;
    float *tb = nullptr, *y = nullptr, *dy = nullptr, *loss_acc = nullptr;
    unsigned *step = nullptr;
    float *loss_hist = nullptr;
    int hist_len = 0;
    int *err = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_rows = 0;
    AdamArgs adam{1e-3f, 1e-5f, 0.9f, 0.999f, 1e-8f, 0u};
    int fused = 1;                  // inference by the fused kernel (1) or layer by layer (0)
    uint8_t *wimg = nullptr;        // the fused kernel's weight image
};

namespace {

template <class T>
cudaError_t dalloc(T **p, size_t n)
{
    *p = nullptr;
    return cudaMalloc(reinterpret_cast<void **>(p), sizeof(T) * std::max<size_t>(n, 1));
}

template <class T>
void dfree(T *&p)
{
    if (p)
        cudaFree(p);
    p = nullptr;
}

void drop_graph(anacor_surrogate *s)
{
    if (s->exec)
        cudaGraphExecDestroy(s->exec);
    if (s->graph)
        cudaGraphDestroy(s->graph);
    s->exec = nullptr;
    s->graph = nullptr;
    s->graph_rows = 0;
}

void free_work(anacor_surrogate *s)
{
    drop_graph(s);
    dfree(s->X0); dfree(s->X0T);
    for (int l = 0; l < kDepth; l++) {
        dfree(s->H[l]); dfree(s->A[l]); dfree(s->AT[l]);
    }
    dfree(s->dH); dfree(s->dHT); dfree(s->dH2); dfree(s->dHT2);
    dfree(s->tb); dfree(s->y); dfree(s->dy); dfree(s->part);
    s->rows = 0;
    s->train_ws = false;
}

// workspace for exactly `rows` rows per member: inference keeps two
// activation buffers, training every layer's activations in both orders
int ensure_work(anacor_surrogate *s, int rows, bool train)
{
    if (rows <= 0 || rows % umma::kBM)
        return report_status(kErrArgs, "surrogate: rows must be a positive multiple of 128");
    if (train && rows % (umma::kBK * kSplitK))
        return report_status(kErrArgs, "surrogate: the training batch must be a multiple of 1024");
    if (s->rows == rows && s->train_ws == train)
        return kOk;
    free_work(s);
    const size_t E = s->E, R = rows;
    bool ok = !dalloc(&s->X0, E * R * kFeat) && !dalloc(&s->y, E * R) && !dalloc(&s->A[0], E * R * kWidth) &&
              !dalloc(&s->A[1], E * R * kWidth);
    if (ok && train) {
        ok = !dalloc(&s->X0T, E * R * kFeat) && !dalloc(&s->dH, E * R * kWidth) && !dalloc(&s->dHT, E * R * kWidth) &&
             !dalloc(&s->dH2, E * R * kWidth) && !dalloc(&s->dHT2, E * R * kWidth) && !dalloc(&s->tb, E * R) &&
             !dalloc(&s->dy, E * R) && !dalloc(&s->part, E * kSplitK * (size_t)kWidth * kWidth);
        for (int l = 0; l < kDepth && ok; l++)
            ok = !dalloc(&s->H[l], E * R * kWidth) && !dalloc(&s->AT[l], E * R * kWidth) &&
                 (l < 2 || !dalloc(&s->A[l], E * R * kWidth));
    }
    if (!ok) {
        free_work(s);
        return report_status(kErrCuda, "surrogate: device allocation failed");
    }
    s->rows = rows;
    s->train_ws = train;
    return kOk;
}

int cuda_fail(cudaError_t e) { return report_status(kErrCuda, cudaGetErrorString(e)); }

int check_err(anacor_surrogate *s, cudaStream_t st)
{
    int h = 0;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(&h, s->err, sizeof(int), cudaMemcpyDeviceToHost, st)) || (e = cudaStreamSynchronize(st)))
        return cuda_fail(e);
    if (h)
        return report_status(kErrCuda, "surrogate: a tensor-core wait timed out");
    return report_status(kOk, "");
}

cudaError_t convert_all(anacor_surrogate *s, cudaStream_t st)
{
    for (int l = 0; l < kDepth; l++) {
        const long long n = (long long)kWidth * in_dim(l) * s->E;
        convert_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s->params, l, s->E, s->W[l], s->WT[l]);
    }
    return cudaGetLastError();
}

// Forward of every member over `rows` rows of X0 ([E][rows][64], or one
// shared [rows][64] when x_shared).  With keep, every layer's pre-activation
// and both orders of its activation stay for the backward pass.  Returns the
// buffer that holds the last hidden activation.
bf16 *forward(anacor_surrogate *s, int rows, bool x_shared, bool keep, cudaStream_t st, cudaError_t &err)
{
    const long long R = rows;
    const bf16 *in = s->X0;
    bf16 *out = nullptr;
    for (int l = 0; l < kDepth; l++) {
        GemmArgs g{};
        const int K = in_dim(l);
        out = keep ? s->A[l] : s->A[l & 1];
        g.A = in;
        g.lda = K;
        g.sA = (l == 0 && x_shared) ? 0 : R * K;
        g.B = s->W[l];
        g.ldb = K;
        g.sB = (long long)kWidth * K;
        g.M = rows; g.N = kWidth; g.K = K;
        g.mode = kEpiBiasGelu;
        g.bias = s->params + off_b(l);
        g.sBias = kParams;
        g.of = keep ? s->H[l] : nullptr;
        g.ldf = kWidth; g.sF = R * kWidth;
        g.ob = out;
        g.ldob = kWidth; g.sOb = R * kWidth;
        g.ot = keep ? s->AT[l] : nullptr;
        g.ldot = R; g.sOt = R * kWidth;
        g.err = s->err;
        if ((err = gemm(g, s->E, st)))
            return nullptr;
        in = out;
    }
    err = cudaSuccess;
    return out;
}

// backward from the head's dH4 down to every weight and bias gradient
cudaError_t backward(anacor_surrogate *s, int rows, cudaStream_t st)
{
    cudaError_t e;
    const long long R = rows;
    rowsum_kernel<<<dim3(kWidth, s->E), 256, 0, st>>>(s->AT[kDepth - 1], s->dy, rows, R * kWidth, R,
                                                       s->grad + kOffW5, kParams);
    vecsum_kernel<<<s->E, 256, 0, st>>>(s->dy, rows, s->grad + kOffB5, kParams);
    bf16 *dH = s->dH, *dHT = s->dHT, *dH2 = s->dH2, *dHT2 = s->dHT2;
    for (int l = kDepth - 1; l >= 0; l--) {
        const int K = in_dim(l);
        // dW_l = dH_l^T A_{l-1} (A_{-1} = X0): [256][K], K-split over the rows
        GemmArgs g{};
        g.A = dHT; g.lda = R; g.sA = R * kWidth;
        g.B = l == 0 ? s->X0T : s->AT[l - 1]; g.ldb = R; g.sB = R * K;
        g.M = kWidth; g.N = K; g.K = rows;
        g.ksplit = kSplitK;
        g.mode = kEpiStoreF32;
        g.of = s->part; g.ldf = K; g.sF = (long long)kWidth * K;
        g.err = s->err;
        if ((e = gemm(g, s->E, st)))
            return e;
        const long long len = (long long)kWidth * K;
        splitk_reduce_kernel<<<dim3((unsigned)((len + 255) / 256), s->E), 256, 0, st>>>(s->part, kSplitK, len,
                                                                                       s->grad + off_w(l), kParams);
        rowsum_kernel<<<dim3(kWidth, s->E), 256, 0, st>>>(dHT, nullptr, rows, R * kWidth, 0, s->grad + off_b(l),
                                                           kParams);
        if (l == 0)
            break;
        // dH_{l-1} = bf16((dH_l W_l) * gelu'(H_{l-1})): [rows][256]
        GemmArgs b{};
        b.A = dH; b.lda = kWidth; b.sA = R * kWidth;
        b.B = s->WT[l]; b.ldb = kWidth; b.sB = (long long)kWidth * K;
        b.M = rows; b.N = K; b.K = kWidth;
        b.mode = kEpiGeluBwd;
        b.aux = s->H[l - 1]; b.ldaux = kWidth; b.sAux = R * kWidth;
        b.ob = dH2; b.ldob = kWidth; b.sOb = R * kWidth;
        b.ot = dHT2; b.ldot = R; b.sOt = R * kWidth;
        b.err = s->err;
        if ((e = gemm(b, s->E, st)))
            return e;
        std::swap(dH, dH2);
        std::swap(dHT, dHT2);
    }
    return cudaGetLastError();
}

// forward + loss + backward on the batch in X0 / X0T / tb, then (update)
// the Adam step, the BF16 weight copies and the step counter
cudaError_t train_step_body(anacor_surrogate *s, int rows, bool update, cudaStream_t st)
{
    cudaError_t e;
    zero_kernel<<<1, 32, 0, st>>>(s->loss_acc, s->E);
    bf16 *a4 = forward(s, rows, false, true, st, e);
    if (e)
        return e;
    head_kernel<<<dim3((rows * 32 + 255) / 256, s->E), 256, 0, st>>>(a4, s->H[kDepth - 1], s->params, s->tb, rows,
                                                                      1, s->y, s->dy, s->dH, s->dHT, s->loss_acc);
    if ((e = backward(s, rows, st)))
        return e;
    if (update) {
        const long long n = kParams * s->E;
        adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s->params, s->m, s->v, s->grad, n, s->step,
                                                                  s->adam);
        if ((e = convert_all(s, st)))
            return e;
        step_done_kernel<<<1, 32, 0, st>>>(s->step, s->loss_hist, s->loss_acc, s->E, s->hist_len);
    }
    return cudaGetLastError();
}

// He-style initialisation of every member (host RNG, seeded)
void init_params(std::vector<float> &p, int E, uint32_t seed)
{
    std::mt19937 rng(seed);
    for (int e = 0; e < E; e++) {
        float *P = p.data() + e * kParams;
        for (int l = 0; l < kDepth; l++) {
            std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (float)in_dim(l)));
            for (long long i = 0; i < (long long)kWidth * in_dim(l); i++)
                P[off_w(l) + i] = nd(rng);
            for (int i = 0; i < kWidth; i++)
                P[off_b(l) + i] = 0.0f;
        }
        std::normal_distribution<float> nd(0.0f, std::sqrt(1.0f / (float)kWidth));
        for (int i = 0; i < kWidth; i++)
            P[kOffW5 + i] = nd(rng);
        P[kOffB5] = 0.0f;
    }
}

// features of n rows of device x7 into X0 (padded to rows_pad), forward, head
// and ensemble statistics; all on `st`, no synchronisation
cudaError_t predict_pass(anacor_surrogate *s, const float *d_x7, long long n, int rows_pad, float *d_mean,
                         float *d_spread, float *d_members, long long ldm, cudaStream_t st)
{
    cudaError_t e;
    features_kernel<<<(unsigned)(((long long)rows_pad * (kFeat / 2) + 255) / 256), 256, 0, st>>>(d_x7, s->Bf, n,
                                                                                                 rows_pad, s->X0);
    bf16 *a4 = forward(s, rows_pad, true, false, st, e);
    if (e)
        return e;
    head_kernel<<<dim3((rows_pad * 32 + 255) / 256, s->E), 256, 0, st>>>(a4, nullptr, s->params, nullptr, rows_pad,
                                                                          0, s->y, nullptr, nullptr, nullptr, nullptr);
    ensemble_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s->y, s->E, n, rows_pad, (float)s->t_mean,
                                                                 (float)s->t_std, d_mean, d_spread, d_members, ldm);
    return cudaGetLastError();
}

Geometry make_geometry(const double *xray, const double *axis, const double *F)
{
    Geometry g;
    std::memcpy(g.xray, xray, sizeof(g.xray));
    std::memcpy(g.axis, axis, sizeof(g.axis));
    std::memcpy(g.F, F, sizeof(g.F));
    return g;
}

}  // namespace

extern "C" {

anacor_surrogate *anacor_surrogate_create(int n_members, uint32_t seed, float fourier_scale)
{
    if (n_members < 1 || n_members > kMaxMembers || !(fourier_scale > 0.0f)) {
        report_status(kErrArgs, "surrogate: 1..16 members and a positive Fourier scale");
        return nullptr;
    }
    if (cudaError_t e = gemm_init()) {
        cuda_fail(e);
        return nullptr;
    }
    anacor_surrogate *s = new (std::nothrow) anacor_surrogate();
    if (!s) {
        report_status(kErrNoMem, "out of host memory");
        return nullptr;
    }
    s->E = n_members;
    s->seed = seed;
    const size_t np = (size_t)kParams * n_members;
    bool ok = !cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) && !dalloc(&s->params, np) &&
              !dalloc(&s->m, np) && !dalloc(&s->v, np) && !dalloc(&s->grad, np) && !dalloc(&s->Bf, 32 * kIn) &&
              !dalloc(&s->loss_acc, 16) && !dalloc(&s->step, 1) && !dalloc(&s->err, 1);
    for (int l = 0; l < kDepth && ok; l++) {
        const size_t n = (size_t)kWidth * in_dim(l) * n_members;
        ok = !dalloc(&s->W[l], n) && !dalloc(&s->WT[l], n);
    }
    std::vector<float> p(np, 0.0f);
    init_params(p, n_members, seed);
    std::vector<float> B(32 * kIn);
    std::mt19937 rng(seed ^ 0x5bd1e995u);
    std::normal_distribution<float> nd(0.0f, fourier_scale);
    for (int j = 0; j < 32; j++)
        for (int q = 0; q < kIn; q++)   // integer omega frequencies: features periodic in omega
            B[j * kIn + q] = q == 0 ? std::nearbyint(nd(rng)) : nd(rng);
    cudaError_t e = cudaSuccess;
    if (ok && ((e = cudaMemcpy(s->params, p.data(), np * sizeof(float), cudaMemcpyHostToDevice)) ||
               (e = cudaMemset(s->m, 0, np * sizeof(float))) || (e = cudaMemset(s->v, 0, np * sizeof(float))) ||
               (e = cudaMemset(s->grad, 0, np * sizeof(float))) || (e = cudaMemset(s->step, 0, sizeof(unsigned))) ||
               (e = cudaMemset(s->err, 0, sizeof(int))) ||
               (e = cudaMemcpy(s->Bf, B.data(), B.size() * sizeof(float), cudaMemcpyHostToDevice)) ||
               (e = convert_all(s, s->st)) || (e = cudaStreamSynchronize(s->st))))
        ok = false;
    if (!ok) {
        if (e)
            cuda_fail(e);
        else
            report_status(kErrCuda, "surrogate: device allocation failed");
        anacor_surrogate_destroy(s);
        return nullptr;
    }
    report_status(kOk, "");
    return s;
}

void anacor_surrogate_destroy(anacor_surrogate *s)
{
    if (!s)
        return;
    if (s->st)
        cudaStreamSynchronize(s->st);
    free_work(s);
    dfree(s->params); dfree(s->m); dfree(s->v); dfree(s->grad); dfree(s->Bf);
    dfree(s->loss_acc); dfree(s->step); dfree(s->err); dfree(s->loss_hist); dfree(s->wimg);
    dfree(s->target); dfree(s->feat);
    for (int l = 0; l < kDepth; l++) {
        dfree(s->W[l]);
        dfree(s->WT[l]);
    }
    if (s->st)
        cudaStreamDestroy(s->st);
    delete s;
}

int64_t anacor_surrogate_param_count(void) { return kParams; }

int anacor_surrogate_members(const anacor_surrogate *s) { return s ? s->E : 0; }

int anacor_surrogate_params(anacor_surrogate *s, float *host, int to_device)
{
    if (!s || !host)
        return report_status(kErrArgs, "bad arguments");
    const size_t n = (size_t)kParams * s->E * sizeof(float);
    cudaError_t e = cudaStreamSynchronize(s->st);
    if (!e)
        e = to_device ? cudaMemcpy(s->params, host, n, cudaMemcpyHostToDevice)
                      : cudaMemcpy(host, s->params, n, cudaMemcpyDeviceToHost);
    if (!e && to_device)
        e = convert_all(s, s->st);
    if (!e)
        e = cudaStreamSynchronize(s->st);
    return e ? cuda_fail(e) : report_status(kOk, "");
}

int anacor_surrogate_fourier(anacor_surrogate *s, float *host32x7, int to_device)
{
    if (!s || !host32x7)
        return report_status(kErrArgs, "bad arguments");
    cudaError_t e = to_device ? cudaMemcpy(s->Bf, host32x7, 32 * kIn * sizeof(float), cudaMemcpyHostToDevice)
                              : cudaMemcpy(host32x7, s->Bf, 32 * kIn * sizeof(float), cudaMemcpyDeviceToHost);
    return e ? cuda_fail(e) : report_status(kOk, "");
}

int anacor_surrogate_scale(anacor_surrogate *s, double *mean, double *std_dev, int set)
{
    if (!s || !mean || !std_dev || (set && !(*std_dev > 0.0)))
        return report_status(kErrArgs, "bad arguments");
    if (set) {
        s->t_mean = *mean;
        s->t_std = *std_dev;
    } else {
        *mean = s->t_mean;
        *std_dev = s->t_std;
    }
    return report_status(kOk, "");
}

int anacor_surrogate_inputs_device(const double *d_omega, const double *d_s1, int64_t n, const double *xray,
                                   const double *omega_axis, const double *F, float *d_x7, void *stream)
{
    if (n < 0 || (n > 0 && (!d_omega || !d_s1 || !xray || !omega_axis || !F || !d_x7)))
        return report_status(kErrArgs, "bad arguments");
    if (n == 0)
        return report_status(kOk, "");
    inputs_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        d_omega, d_s1, n, make_geometry(xray, omega_axis, F), d_x7);
    cudaError_t e = cudaGetLastError();
    return e ? cuda_fail(e) : report_status(kOk, "");
}

int anacor_surrogate_inputs(const double *omega, const double *s1, int64_t n, const double *xray,
                            const double *omega_axis, const double *F, float *x7_out)
{
    if (n < 0 || (n > 0 && (!omega || !s1 || !xray || !omega_axis || !F || !x7_out)))
        return report_status(kErrArgs, "bad arguments");
    if (n == 0)
        return report_status(kOk, "");
    double *d_om = nullptr, *d_s1 = nullptr;
    float *d_x = nullptr;
    cudaError_t e;
    if (!(e = dalloc(&d_om, n)) && !(e = dalloc(&d_s1, 3 * n)) && !(e = dalloc(&d_x, 7 * n)) &&
        !(e = cudaMemcpy(d_om, omega, n * sizeof(double), cudaMemcpyHostToDevice)) &&
        !(e = cudaMemcpy(d_s1, s1, 3 * n * sizeof(double), cudaMemcpyHostToDevice))) {
        inputs_kernel<<<(unsigned)((n + 255) / 256), 256>>>(d_om, d_s1, n, make_geometry(xray, omega_axis, F), d_x);
        if (!(e = cudaGetLastError()))
            e = cudaMemcpy(x7_out, d_x, 7 * n * sizeof(float), cudaMemcpyDeviceToHost);
    }
    dfree(d_om); dfree(d_s1); dfree(d_x);
    return e ? cuda_fail(e) : report_status(kOk, "");
}

// training set: x7 rows and log A_h targets; the targets are standardised
// with their mean and standard deviation, which become the output scale
int anacor_surrogate_set_data(anacor_surrogate *s, const float *x7, const double *log_ah, int64_t n)
{
    if (!s || n < 2 || !x7 || !log_ah)
        return report_status(kErrArgs, "bad arguments");
    double mu = 0.0, m2 = 0.0;
    for (int64_t i = 0; i < n; i++) {
        if (!std::isfinite(log_ah[i]))
            return report_status(kErrArgs, "surrogate: non-finite training target");
        const double d = log_ah[i] - mu;
        mu += d / (double)(i + 1);
        m2 += d * (log_ah[i] - mu);
    }
    double sd = std::sqrt(m2 / (double)(n - 1));
    if (!(sd > 1e-12))
        sd = 1.0;
    std::vector<float> t(n);
    for (int64_t i = 0; i < n; i++)
        t[i] = (float)((log_ah[i] - mu) / sd);
    cudaStreamSynchronize(s->st);
    drop_graph(s);
    dfree(s->target);
    dfree(s->feat);
    float *d_x = nullptr;
    cudaError_t e;
    if (!(e = dalloc(&d_x, 7 * n)) && !(e = dalloc(&s->target, n)) && !(e = dalloc(&s->feat, n * kFeat)) &&
        !(e = cudaMemcpy(d_x, x7, 7 * n * sizeof(float), cudaMemcpyHostToDevice)) &&
        !(e = cudaMemcpy(s->target, t.data(), n * sizeof(float), cudaMemcpyHostToDevice))) {
        features_kernel<<<(unsigned)((n * (kFeat / 2) + 255) / 256), 256, 0, s->st>>>(d_x, s->Bf, n, n, s->feat);
        if (!(e = cudaGetLastError()))
            e = cudaStreamSynchronize(s->st);
    }
    dfree(d_x);
    if (e) {
        dfree(s->target);
        dfree(s->feat);
        s->n_data = 0;
        return cuda_fail(e);
    }
    s->n_data = n;
    s->t_mean = mu;
    s->t_std = sd;
    return report_status(kOk, "");
}

int anacor_surrogate_train(anacor_surrogate *s, int steps, int batch, float lr_max, float lr_min, int total_steps,
                           float *loss_out)
{
    if (!s || steps < 0 || batch <= 0 || !s->n_data || !(lr_max > 0.0f) || lr_min < 0.0f || total_steps < 0)
        return report_status(kErrArgs, "surrogate: bad training arguments");
    if (int st = ensure_work(s, batch, true))
        return st;
    unsigned start = 0;
    cudaError_t e;
    if ((e = cudaStreamSynchronize(s->st)) || (e = cudaMemcpy(&start, s->step, sizeof(unsigned), cudaMemcpyDeviceToHost)))
        return cuda_fail(e);
    const AdamArgs a{lr_max, lr_min, 0.9f, 0.999f, 1e-8f, (unsigned)total_steps};
    if (std::memcmp(&a, &s->adam, sizeof(a)) != 0) {
        s->adam = a;
        drop_graph(s);   // the graph holds the Adam arguments by value
    }
    const int need = (int)start + steps;
    if (need > s->hist_len) {
        float *h = nullptr;
        if (dalloc(&h, (size_t)need + 1024))
            return report_status(kErrCuda, "surrogate: device allocation failed");
        if (s->loss_hist)
            cudaMemcpy(h, s->loss_hist, s->hist_len * sizeof(float), cudaMemcpyDeviceToDevice);
        dfree(s->loss_hist);
        s->loss_hist = h;
        s->hist_len = need + 1024;
        drop_graph(s);   // ... and the history pointer
    }
    if (!s->exec || s->graph_rows != batch) {
        drop_graph(s);
        if ((e = cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal)))
            return cuda_fail(e);
        gather_kernel<<<dim3((batch + 255) / 256, s->E), 256, 0, s->st>>>(s->feat, s->target, s->n_data, batch,
                                                                          s->step, s->seed, s->X0, s->X0T, s->tb);
        cudaError_t le = train_step_body(s, batch, true, s->st);
        e = cudaStreamEndCapture(s->st, &s->graph);
        if (le || e) {
            drop_graph(s);
            return cuda_fail(le ? le : e);
        }
        if ((e = cudaGraphInstantiate(&s->exec, s->graph, 0))) {
            drop_graph(s);
            return cuda_fail(e);
        }
        s->graph_rows = batch;
    }
    for (int i = 0; i < steps; i++)
        if ((e = cudaGraphLaunch(s->exec, s->st)))
            return cuda_fail(e);
    if (int st = check_err(s, s->st))
        return st;
    if (loss_out && steps > 0 &&
        (e = cudaMemcpy(loss_out, s->loss_hist + start, steps * sizeof(float), cudaMemcpyDeviceToHost)))
        return cuda_fail(e);
    return report_status(kOk, "");
}

int anacor_surrogate_gradients(anacor_surrogate *s, const float *x7, const float *target, int rows,
                               float *grads_out, float *y_out)
{
    if (!s || rows <= 0 || !x7 || !target)
        return report_status(kErrArgs, "bad arguments");
    if (int st = ensure_work(s, rows, true))
        return st;
    const size_t R = rows;
    float *d_x = nullptr, *d_t = nullptr;
    bf16 *d_f = nullptr;
    cudaError_t e;
    std::vector<bf16> hx(R * kFeat), ht(R * kFeat);
    if (!(e = cudaStreamSynchronize(s->st)) && !(e = dalloc(&d_x, 7 * R)) && !(e = dalloc(&d_t, R)) &&
        !(e = dalloc(&d_f, R * kFeat)) && !(e = cudaMemcpy(d_x, x7, 7 * R * sizeof(float), cudaMemcpyHostToDevice)) &&
        !(e = cudaMemcpy(d_t, target, R * sizeof(float), cudaMemcpyHostToDevice))) {
        features_kernel<<<(unsigned)((R * (kFeat / 2) + 255) / 256), 256, 0, s->st>>>(d_x, s->Bf, rows, rows, d_f);
        if (!(e = cudaGetLastError()) &&
            !(e = cudaMemcpyAsync(hx.data(), d_f, hx.size() * sizeof(bf16), cudaMemcpyDeviceToHost, s->st)))
            e = cudaStreamSynchronize(s->st);
    }
    if (!e) {
        for (size_t r = 0; r < R; r++)
            for (int q = 0; q < kFeat; q++)
                ht[(size_t)q * R + r] = hx[r * kFeat + q];
        // the same batch, rows in order, for every member
        for (int m = 0; m < s->E && !e; m++)
            if (!(e = cudaMemcpy(s->X0 + m * R * kFeat, d_f, R * kFeat * sizeof(bf16), cudaMemcpyDeviceToDevice)) &&
                !(e = cudaMemcpy(s->X0T + m * R * kFeat, ht.data(), ht.size() * sizeof(bf16), cudaMemcpyHostToDevice)))
                e = cudaMemcpy(s->tb + m * R, d_t, R * sizeof(float), cudaMemcpyDeviceToDevice);
    }
    if (!e)
        e = train_step_body(s, rows, false, s->st);
    if (!e)
        e = cudaStreamSynchronize(s->st);
    if (!e && grads_out)
        e = cudaMemcpy(grads_out, s->grad, (size_t)kParams * s->E * sizeof(float), cudaMemcpyDeviceToHost);
    if (!e && y_out)
        e = cudaMemcpy(y_out, s->y, R * s->E * sizeof(float), cudaMemcpyDeviceToHost);
    dfree(d_x); dfree(d_t); dfree(d_f);
    if (e)
        return cuda_fail(e);
    return check_err(s, s->st);
}

int anacor_surrogate_predict_device(anacor_surrogate *s, const float *d_x7, int64_t n, float *d_mean,
                                    float *d_spread, float *d_members, void *stream)
{
    if (!s || n < 0 || (n > 0 && (!d_x7 || !d_mean || !d_spread)))
        return report_status(kErrArgs, "bad arguments");
    if (n == 0)
        return report_status(kOk, "");
    cudaStream_t st = stream ? (cudaStream_t)stream : s->st;
    if (s->fused && s->E <= kInferMaxMembers) {
        // one launch over all n rows: no activation workspace
        int dev = 0, sms = 0;
        cudaError_t e;
        if ((e = cudaGetDevice(&dev)) || (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) ||
            (e = infer_init(dev)))
            return cuda_fail(e);
        if (!s->wimg && (e = dalloc(&s->wimg, (size_t)s->E * kChunksPerMember * kChunkBytes)))
            return cuda_fail(e);
        WeightPtrs wp;
        for (int l = 0; l < kDepth; l++)
            wp.w[l] = s->W[l];
        weight_image_kernel<<<2 * sms, 256, 0, st>>>(wp, s->E, s->wimg);
        InferArgs ia;
        ia.x7 = d_x7;
        ia.n = n;
        ia.Bf = s->Bf;
        ia.wimg = s->wimg;
        ia.params = s->params;
        ia.E = s->E;
        ia.mu = (float)s->t_mean;
        ia.sd = (float)s->t_std;
        ia.mean = d_mean;
        ia.spread = d_spread;
        ia.members = d_members;
        ia.ldm = n;
        ia.err = s->err;
        const long long tiles = (n + kTileRows - 1) / kTileRows;
        const int grid = (int)std::min<long long>(tiles, sms);
        infer_kernel<<<grid, kInferThreads, kInferSmem, st>>>(ia);
        if ((e = cudaGetLastError()))
            return cuda_fail(e);
        return report_status(kOk, "");
    }
    const int chunk = (int)std::min<int64_t>(kPredictChunk, (n + umma::kBM - 1) / umma::kBM * umma::kBM);
    if (s->rows != chunk || s->train_ws) {
        // the workspace is about to be replaced: nothing may still use it
        cudaError_t e;
        if ((e = cudaStreamSynchronize(s->st)) || (stream && (e = cudaStreamSynchronize(st))))
            return cuda_fail(e);
        if (int r = ensure_work(s, chunk, false))
            return r;
    }
    for (int64_t i0 = 0; i0 < n; i0 += chunk) {
        const long long m = std::min<int64_t>(chunk, n - i0);
        const int rows = (int)((m + umma::kBM - 1) / umma::kBM * umma::kBM);
        if (cudaError_t e = predict_pass(s, d_x7 + 7 * i0, m, rows, d_mean + i0, d_spread + i0,
                                         d_members ? d_members + i0 : nullptr, n, st))
            return cuda_fail(e);
    }
    return report_status(kOk, "");
}

int anacor_surrogate_set_inference(anacor_surrogate *s, int fused)
{
    if (!s || (fused != 0 && fused != 1))
        return report_status(kErrArgs, "bad arguments");
    if (s->st)
        cudaStreamSynchronize(s->st);
    s->fused = fused;
    return report_status(kOk, "");
}

int anacor_surrogate_predict(anacor_surrogate *s, const float *x7, int64_t n, float *mean_out, float *spread_out,
                             float *members_out)
{
    if (!s || n < 0 || (n > 0 && (!x7 || !mean_out || !spread_out)))
        return report_status(kErrArgs, "bad arguments");
    if (n == 0)
        return report_status(kOk, "");
    float *d_x = nullptr, *d_mean = nullptr, *d_spread = nullptr, *d_mem = nullptr;
    cudaError_t e;
    int st = kOk;
    if (!(e = dalloc(&d_x, 7 * (size_t)n)) && !(e = dalloc(&d_mean, n)) && !(e = dalloc(&d_spread, n)) &&
        !(members_out && (e = dalloc(&d_mem, (size_t)n * s->E))) &&
        !(e = cudaMemcpyAsync(d_x, x7, 7 * (size_t)n * sizeof(float), cudaMemcpyHostToDevice, s->st))) {
        st = anacor_surrogate_predict_device(s, d_x, n, d_mean, d_spread, d_mem, s->st);
        if (!st && !(e = cudaMemcpyAsync(mean_out, d_mean, n * sizeof(float), cudaMemcpyDeviceToHost, s->st)) &&
            !(e = cudaMemcpyAsync(spread_out, d_spread, n * sizeof(float), cudaMemcpyDeviceToHost, s->st)) &&
            !(members_out && (e = cudaMemcpyAsync(members_out, d_mem, (size_t)n * s->E * sizeof(float),
                                                  cudaMemcpyDeviceToHost, s->st))))
            e = cudaStreamSynchronize(s->st);
    }
    dfree(d_x); dfree(d_mean); dfree(d_spread); dfree(d_mem);
    if (st)
        return st;
    if (e)
        return cuda_fail(e);
    return check_err(s, s->st);
}

int anacor_surrogate_audit_flags(const float *d_spread, int64_t n, uint32_t seed, double audit_fraction,
                                 float spread_threshold, uint8_t *d_flags, void *stream)
{
    if (n < 0 || (n > 0 && (!d_spread || !d_flags)) || !(audit_fraction >= 0.0 && audit_fraction <= 1.0))
        return report_status(kErrArgs, "bad arguments");
    if (n == 0)
        return report_status(kOk, "");
    const double c = std::ldexp(audit_fraction, 32);
    const uint32_t cut = c >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)c;
    audit_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(d_spread, n, seed, cut,
                                                                                spread_threshold, d_flags);
    cudaError_t e = cudaGetLastError();
    return e ? cuda_fail(e) : report_status(kOk, "");
}

int anacor_surrogate_save(anacor_surrogate *s, const char *path)
{
    if (!s || !path)
        return report_status(kErrArgs, "bad arguments");
    std::vector<float> p((size_t)kParams * s->E), B(32 * kIn);
    cudaError_t e;
    if ((e = cudaStreamSynchronize(s->st)) ||
        (e = cudaMemcpy(p.data(), s->params, p.size() * sizeof(float), cudaMemcpyDeviceToHost)) ||
        (e = cudaMemcpy(B.data(), s->Bf, B.size() * sizeof(float), cudaMemcpyDeviceToHost)))
        return cuda_fail(e);
    FILE *f = std::fopen(path, "wb");
    if (!f)
        return report_status(kErrArgs, "surrogate: cannot open the checkpoint for writing");
    const uint32_t hdr[4] = {0x41484750u, 1u, (uint32_t)s->E, (uint32_t)kParams};
    const double scale[2] = {s->t_mean, s->t_std};
    bool ok = std::fwrite(hdr, sizeof(hdr), 1, f) == 1 && std::fwrite(scale, sizeof(scale), 1, f) == 1 &&
              std::fwrite(B.data(), sizeof(float), B.size(), f) == B.size() &&
              std::fwrite(p.data(), sizeof(float), p.size(), f) == p.size();
    ok = (std::fclose(f) == 0) && ok;
    return report_status(ok ? kOk : kErrArgs, ok ? "" : "surrogate: checkpoint write failed");
}

int anacor_surrogate_load(anacor_surrogate *s, const char *path)
{
    if (!s || !path)
        return report_status(kErrArgs, "bad arguments");
    FILE *f = std::fopen(path, "rb");
    if (!f)
        return report_status(kErrArgs, "surrogate: cannot open the checkpoint");
    uint32_t hdr[4];
    double scale[2];
    std::vector<float> p((size_t)kParams * s->E), B(32 * kIn);
    bool ok = std::fread(hdr, sizeof(hdr), 1, f) == 1 && hdr[0] == 0x41484750u && hdr[1] == 1u &&
              hdr[2] == (uint32_t)s->E && hdr[3] == (uint32_t)kParams && std::fread(scale, sizeof(scale), 1, f) == 1 &&
              std::fread(B.data(), sizeof(float), B.size(), f) == B.size() &&
              std::fread(p.data(), sizeof(float), p.size(), f) == p.size() && scale[1] > 0.0;
    std::fclose(f);
    if (!ok)
        return report_status(kErrArgs, "surrogate: the checkpoint does not match this network");
    cudaError_t e;
    if ((e = cudaStreamSynchronize(s->st)) ||
        (e = cudaMemcpy(s->params, p.data(), p.size() * sizeof(float), cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(s->Bf, B.data(), B.size() * sizeof(float), cudaMemcpyHostToDevice)) ||
        (e = convert_all(s, s->st)) || (e = cudaStreamSynchronize(s->st)))
        return cuda_fail(e);
    s->t_mean = scale[0];
    s->t_std = scale[1];
    if (s->n_data) {   // the cached training features used the old Fourier matrix
        dfree(s->target);
        dfree(s->feat);
        s->n_data = 0;
        drop_graph(s);
    }
    return report_status(kOk, "");
}

int anacor_wait_guard_check(unsigned iterations, int32_t *status)
{
    if (!status || iterations == 0 || iterations > (1u << 20))
        return report_status(kErrArgs, "iterations must lie in [1, 2^20]");
    int *d_err = nullptr;
    cudaError_t e;
    if ((e = dalloc(&d_err, 1)))
        return cuda_fail(e);
    int h = 0;
    if (!(e = cudaMemset(d_err, 0, sizeof(int)))) {
        wait_guard_kernel<<<1, 128>>>(iterations, d_err);
        if (!(e = cudaGetLastError()) && !(e = cudaDeviceSynchronize()))
            e = cudaMemcpy(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost);
    }
    dfree(d_err);
    if (e)
        return cuda_fail(e);
    *status = h;
    return report_status(kOk, "");
}

int anacor_tc_gemm_check(const float *A, const float *B, int M, int N, int K, int batch, int ksplit, float *C)
{
    if (!A || !B || !C || M <= 0 || N <= 0 || K <= 0 || batch <= 0 || ksplit < 1)
        return report_status(kErrArgs, "bad arguments");
    if (M % umma::kBM || N % 64 || K % (umma::kBK * ksplit))
        return report_status(kErrArgs, "tc_gemm: M % 128, N % 64 and K % (64 * ksplit) must be 0");
    if (cudaError_t e = gemm_init())
        return cuda_fail(e);
    std::vector<bf16> ha((size_t)batch * M * K), hb((size_t)batch * N * K);
    for (size_t i = 0; i < ha.size(); i++)
        ha[i] = __float2bfloat16_rn(A[i]);
    for (size_t i = 0; i < hb.size(); i++)
        hb[i] = __float2bfloat16_rn(B[i]);
    bf16 *da = nullptr, *db = nullptr;
    float *dc = nullptr;
    int *derr = nullptr;
    const size_t nc = (size_t)batch * ksplit * M * N;
    cudaError_t e;
    int herr = 0;
    std::vector<float> part(nc);
    if (!(e = dalloc(&da, ha.size())) && !(e = dalloc(&db, hb.size())) && !(e = dalloc(&dc, nc)) &&
        !(e = dalloc(&derr, 1)) && !(e = cudaMemcpy(da, ha.data(), ha.size() * sizeof(bf16), cudaMemcpyHostToDevice)) &&
        !(e = cudaMemcpy(db, hb.data(), hb.size() * sizeof(bf16), cudaMemcpyHostToDevice)) &&
        !(e = cudaMemset(derr, 0, sizeof(int)))) {
        GemmArgs g{};
        g.A = da; g.lda = K; g.sA = (long long)M * K;
        g.B = db; g.ldb = K; g.sB = (long long)N * K;
        g.M = M; g.N = N; g.K = K;
        g.ksplit = ksplit;
        g.mode = kEpiStoreF32;
        g.of = dc; g.ldf = N; g.sF = (long long)M * N;
        g.err = derr;
        if (!(e = gemm(g, batch, 0)) && !(e = cudaDeviceSynchronize()) &&
            !(e = cudaMemcpy(part.data(), dc, nc * sizeof(float), cudaMemcpyDeviceToHost)))
            e = cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
    }
    dfree(da); dfree(db); dfree(dc); dfree(derr);
    if (e)
        return cuda_fail(e);
    if (herr)
        return report_status(kErrCuda, "tc_gemm: a tensor-core wait timed out");
    const size_t mn = (size_t)M * N;
    for (int z = 0; z < batch; z++)
        for (size_t i = 0; i < mn; i++) {
            float acc = 0.0f;
            for (int sp = 0; sp < ksplit; sp++)
                acc += part[((size_t)z * ksplit + sp) * mn + i];
            C[(size_t)z * mn + i] = acc;
        }
    return report_status(kOk, "");
}

}  // extern "C"
