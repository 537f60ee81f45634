// Chessboard distance field of a label volume, packed with the label.
//
// out[v] = (label & 7) | (min(D(v), 31) << 3), where D(v) is the chessboard
// (L-infinity) distance from voxel v to the nearest voxel of the volume whose
// label differs from v's, and 0 for vacuum voxels (label 0: a ray stops there,
// so their distance is never read).  Every voxel within chessboard distance
// D(v) - 1 of v carries v's label: a march that stands on v may step over the
// increments that provably stay inside that cube.
//
// D is found as the largest uniform cube around v, built from one axis at a
// time (the cube of radius r is uniform iff every row segment of half-width r
// inside it is):
//   rows    d_x(v)   = min(31, distance to the nearest other label along x)
//   planes  d_xy(v)  = 1 + max{ r : all |dy| <= r have v's label and d_x >= r + 1 }
//   volume  D(v)     = 1 + max{ r : all |dz| <= r have v's label and d_xy >= r + 1 }
// Voxels outside the volume do not count (marches never leave it).  The
// labels must fit 3 bits (0..7); the first pass flags any that do not.
//
// Octant fields: the same construction with one-sided scans gives, for each
// of the 8 sign combinations (sz, sy, sx), 1 + the largest r for which the
// corner box v + [0..r]^3 * (sz, sy, sx) holds one label.  A ray whose
// direction has those signs only moves into that box, so behind-the-ray
// boundaries (the one just crossed) do not shorten its skips.  Layout:
// [octant][Z][Y][X] with octant = (sx < 0) | (sy < 0) << 1 | (sz < 0) << 2.
#include "anacor_internal.h"
#include "trace_launch.h"

namespace anacor {
namespace {

constexpr int kFieldCap = 31;
constexpr int kFieldThreads = 256;

// d_x along each row (dir 0: both sides, +1 / -1: ahead / behind only); one
// CTA per (z, y) row
__global__ void __launch_bounds__(kFieldThreads) field_rows(const int8_t *__restrict__ vol, int dx, int dir,
                                                            uint8_t *__restrict__ out, int *__restrict__ bad)
{
    const long long row = (long long)blockIdx.x * dx;
    const int8_t *r = vol + row;
    bool any_bad = false;
    for (int x0 = 0; x0 < dx; x0 += kFieldThreads) {
        const int x = x0 + (int)threadIdx.x;
        if (x < dx) {
            const int lab = r[x];
            uint8_t o = 0;
            if ((unsigned)lab > 7u) {
                any_bad = true;
            } else if (lab != 0) {
                int d = kFieldCap;
                for (int k = 1; k < kFieldCap; k++) {
                    if ((dir >= 0 && x + k < dx && r[x + k] != lab) || (dir <= 0 && x - k >= 0 && r[x - k] != lab)) {
                        d = k;
                        break;
                    }
                }
                o = (uint8_t)(lab | (d << 3));
            }
            out[row + x] = o;
        }
    }
    if (__syncthreads_or(any_bad) && threadIdx.x == 0)
        atomicOr(bad, 1);
}

// One cube-growing pass along an axis of stride `stride` and extent `n`
// (coordinate `c` of the row's voxels on that axis): in holds label | d << 3
// of the previous pass, out receives label | d' << 3.
__global__ void __launch_bounds__(kFieldThreads) field_grow(const uint8_t *__restrict__ in, int dy, int dx,
                                                            int axis, int n, long long stride, int dir,
                                                            uint8_t *__restrict__ out)
{
    const long long row = (long long)blockIdx.x * dx;
    const int c = axis == 1 ? (int)(blockIdx.x % (unsigned)dy) : (int)(blockIdx.x / (unsigned)dy);
    for (int x0 = 0; x0 < dx; x0 += kFieldThreads) {
        const int x = x0 + (int)threadIdx.x;
        if (x >= dx)
            continue;
        const long long v = row + x;
        const uint32_t b = in[v];
        const uint32_t lab = b & 7u;
        if (lab == 0) {
            out[v] = 0;
            continue;
        }
        uint32_t m = b >> 3;
        int d = 1;
        for (int r = 1; r < kFieldCap; r++) {
            if (dir >= 0 && c + r < n) {
                const uint32_t u = in[v + r * stride];
                m = min(m, (u & 7u) == lab ? (u >> 3) : 0u);
            }
            if (dir <= 0 && c - r >= 0) {
                const uint32_t u = in[v - r * stride];
                m = min(m, (u & 7u) == lab ? (u >> 3) : 0u);
            }
            if (m < (uint32_t)(r + 1))
                break;
            d = r + 1;
        }
        out[v] = (uint8_t)(lab | (uint32_t)d << 3);
    }
}

// Octant passes, every sign at once (independent scans interleaved per thread).
// Rows: out[0] looks ahead (+x), out[1] behind (-x).
__global__ void __launch_bounds__(kFieldThreads) octant_rows(const int8_t *__restrict__ vol, int dx, long long nvol,
                                                             uint8_t *__restrict__ out, int *__restrict__ bad)
{
    const long long row = (long long)blockIdx.x * dx;
    const int8_t *r = vol + row;
    bool any_bad = false;
    for (int x0 = 0; x0 < dx; x0 += kFieldThreads) {
        const int x = x0 + (int)threadIdx.x;
        if (x < dx) {
            const int lab = r[x];
            uint8_t o0 = 0, o1 = 0;
            if ((unsigned)lab > 7u) {
                any_bad = true;
            } else if (lab != 0) {
                int d0 = kFieldCap, d1 = kFieldCap;
                for (int k = 1; k < kFieldCap && (d0 == kFieldCap || d1 == kFieldCap); k++) {
                    if (d0 == kFieldCap && x + k < dx && r[x + k] != lab)
                        d0 = k;
                    if (d1 == kFieldCap && x - k >= 0 && r[x - k] != lab)
                        d1 = k;
                }
                o0 = (uint8_t)(lab | (d0 << 3));
                o1 = (uint8_t)(lab | (d1 << 3));
            }
            out[row + x] = o0;
            out[nvol + row + x] = o1;
        }
    }
    if (__syncthreads_or(any_bad) && threadIdx.x == 0)
        atomicOr(bad, 1);
}

// Growth along one axis (stride, extent n) of kIn one-sided inputs at once,
// each toward both signs: result j = 2 * i + s (s = 0 toward +, 1 toward -)
// from in[i], stored as out[j], or (kOctants, i = 2 * bx + by, s = bz) as
// out[bx | by << 1 | bz << 2]; inputs and outputs are volumes nvol apart.
template <int kIn, bool kOctants>
__global__ void __launch_bounds__(kFieldThreads) octant_grow(const uint8_t *__restrict__ in, int dy, int dx,
                                                             int axis, int n, long long stride, long long nvol,
                                                             uint8_t *__restrict__ out)
{
    const long long row = (long long)blockIdx.x * dx;
    const int c = axis == 1 ? (int)(blockIdx.x % (unsigned)dy) : (int)(blockIdx.x / (unsigned)dy);
    for (int x0 = 0; x0 < dx; x0 += kFieldThreads) {
        const int x = x0 + (int)threadIdx.x;
        if (x >= dx)
            continue;
        const long long v = row + x;
        const uint32_t lab = in[v] & 7u;
        if (lab == 0) {
#pragma unroll
            for (int j = 0; j < 2 * kIn; j++)
                out[(kOctants ? ((j >> 2) | (((j >> 1) & 1) << 1) | ((j & 1) << 2)) : j) * nvol + v] = 0;
            continue;
        }
        uint32_t m[2 * kIn];
        int d[2 * kIn];
#pragma unroll
        for (int i = 0; i < kIn; i++) {
            m[2 * i] = m[2 * i + 1] = in[i * nvol + v] >> 3;
            d[2 * i] = d[2 * i + 1] = 1;
        }
        unsigned live = (1u << (2 * kIn)) - 1u;
        for (int r = 1; r < kFieldCap && live; r++) {
            const bool up = c + r < n, down = c - r >= 0;
#pragma unroll
            for (int j = 0; j < 2 * kIn; j++) {
                if (!((live >> j) & 1u))
                    continue;
                const bool plus = (j & 1) == 0;
                if (plus ? up : down) {
                    const uint32_t u = in[(j >> 1) * nvol + v + (plus ? r : -r) * stride];
                    m[j] = min(m[j], (u & 7u) == lab ? (u >> 3) : 0u);
                }
                if (m[j] < (uint32_t)(r + 1))
                    live &= ~(1u << j);
                else
                    d[j] = r + 1;
            }
        }
#pragma unroll
        for (int j = 0; j < 2 * kIn; j++)
            out[(kOctants ? ((j >> 2) | (((j >> 1) & 1) << 1) | ((j & 1) << 2)) : j) * nvol + v] =
                (uint8_t)(lab | (uint32_t)d[j] << 3);
    }
}

}  // namespace

cudaError_t launch_distance_field(const int8_t *d_vol, const int *dims, uint8_t *d_out, uint8_t *d_tmp, int *d_bad,
                                  cudaStream_t st)
{
    const unsigned rows = (unsigned)dims[0] * (unsigned)dims[1];
    if (rows == 0 || dims[2] == 0)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d_bad, 0, sizeof(int), st);
    if (e != cudaSuccess)
        return e;
    const long long plane = (long long)dims[1] * dims[2];
    field_rows<<<rows, kFieldThreads, 0, st>>>(d_vol, dims[2], 0, d_out, d_bad);
    field_grow<<<rows, kFieldThreads, 0, st>>>(d_out, dims[1], dims[2], 1, dims[1], dims[2], 0, d_tmp);
    field_grow<<<rows, kFieldThreads, 0, st>>>(d_tmp, dims[1], dims[2], 0, dims[0], plane, 0, d_out);
    return cudaGetLastError();
}

cudaError_t launch_octant_fields(const int8_t *d_vol, const int *dims, uint8_t *d_out, uint8_t *d_tmp, int *d_bad,
                                 cudaStream_t st)
{
    const unsigned rows = (unsigned)dims[0] * (unsigned)dims[1];
    if (rows == 0 || dims[2] == 0)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d_bad, 0, sizeof(int), st);
    if (e != cudaSuccess)
        return e;
    const long long plane = (long long)dims[1] * dims[2];
    const long long nvol = plane * dims[0];
    // tmp[bx]: rows (bx = 1: -x); tmp[2 + 2*bx + by]: squares; out[bx | by << 1 | bz << 2]
    octant_rows<<<rows, kFieldThreads, 0, st>>>(d_vol, dims[2], nvol, d_tmp, d_bad);
    octant_grow<2, false><<<rows, kFieldThreads, 0, st>>>(d_tmp, dims[1], dims[2], 1, dims[1], dims[2], nvol,
                                                          d_tmp + 2 * nvol);
    octant_grow<4, true><<<rows, kFieldThreads, 0, st>>>(d_tmp + 2 * nvol, dims[1], dims[2], 0, dims[0], plane, nvol,
                                                         d_out);
    return cudaGetLastError();
}

namespace {

// One thread per 16 output bytes (a 4x4 (y, x) slab of one brick row z).
__global__ void brick_fields_kernel(const uint8_t *__restrict__ lin, int dz, int dy, int dx, int nbz, int nby,
                                    int nbx, long long n_fields, uint8_t *__restrict__ out)
{
    const long long nvol = (long long)dz * dy * dx;
    const long long per = (long long)nbz * nby * nbx * 64;
    const long long total = n_fields * (per >> 4);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const long long f = q / (per >> 4);
        const long long r = q - f * (per >> 4);       // 16-byte slab within the field
        const long long brick = r >> 2;
        const int zl = (int)(r & 3);
        const int bx = (int)(brick % nbx);
        const int by = (int)((brick / nbx) % nby);
        const int bz = (int)(brick / ((long long)nbx * nby));
        const int z = bz * 4 + zl;
        uint32_t w[4];
#pragma unroll
        for (int yl = 0; yl < 4; yl++) {
            const int y = by * 4 + yl;
            uint32_t word = 0;
#pragma unroll
            for (int xl = 0; xl < 4; xl++) {
                const int x = bx * 4 + xl;
                const uint32_t b = (z < dz && y < dy && x < dx) ? lin[f * nvol + ((long long)z * dy + y) * dx + x] : 0u;
                word |= b << (8 * xl);
            }
            w[yl] = word;
        }
        reinterpret_cast<uint4 *>(out + f * per)[r] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

}  // namespace

size_t brick_field_bytes(const int *dims)
{
    return (size_t)((dims[0] + 3) / 4) * ((dims[1] + 3) / 4) * ((dims[2] + 3) / 4) * 64;
}

void brick_strides(const int *dims, int *sy, int *sz)
{
    const int nbx = (dims[2] + 3) / 4, nby = (dims[1] + 3) / 4;
    *sy = 64 * nbx;
    *sz = 64 * nbx * nby;
}

cudaError_t launch_brick_fields(const uint8_t *d_lin, const int *dims, int n_fields, uint8_t *d_out,
                                cudaStream_t st)
{
    const int nbz = (dims[0] + 3) / 4, nby = (dims[1] + 3) / 4, nbx = (dims[2] + 3) / 4;
    const long long total = (long long)n_fields * nbz * nby * nbx * 4;
    if (total <= 0)
        return cudaSuccess;
    const int threads = 256;
    const int blocks = (int)std::min<long long>((total + threads - 1) / threads, 152ll * 64);
    brick_fields_kernel<<<blocks, threads, 0, st>>>(d_lin, dims[0], dims[1], dims[2], nbz, nby, nbx, n_fields, d_out);
    return cudaGetLastError();
}

}  // namespace anacor
