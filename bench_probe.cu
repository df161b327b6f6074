// Gather-rate probe: the roofline reference for the CSR kernels.
//
// The single-vector product is bound by the rate at which an SM can serve
// scattered 16-byte loads, not by HBM bandwidth.  This probe measures that
// rate on the matrix at hand: per row, the sum of x[col] over the row's
// column indices (16-byte elements, the float-pair complex layout of B),
// with the row hand-out of the product kernels (G lanes per row, two
// entries in flight per lane) and no values, no arithmetic beyond the sums,
// no epilogue.  Its time is the floor a kernel with this access pattern can
// reach; bench.py reports the Taylor kernel's time against it.  It is a
// measurement helper of bench.py only, built into its own library
// (_build/libqsprobe.so, by __graft_entry__.build) and never linked into
// libqsgpu.so.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

__global__ void __launch_bounds__(256) gather_probe_kernel(int64_t n, int lgG, const int32_t *__restrict__ indptr,
                                                           const int32_t *__restrict__ indices,
                                                           const float4 *__restrict__ x, float4 *__restrict__ y)
{
    const int G = 1 << lgG;
    const int GPW = 32 >> lgG;
    const int lane = threadIdx.x & (G - 1);
    const int gsub = (threadIdx.x & 31) >> lgG;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t rb = warp * GPW; rb < n; rb += nwarps * GPW) {
        const int64_t r = rb + gsub;
        const bool valid = r < n;
        const int32_t k0 = valid ? indptr[r] : 0, k1 = valid ? indptr[r + 1] : 0;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int32_t k = k0 + lane; k < k1; k += 2 * G) {
            const int32_t c0 = __ldcs(indices + k);
            const int32_t c1 = k + G < k1 ? __ldcs(indices + k + G) : -1;
            const float4 v0 = __ldg(x + c0);
            const float4 v1 = c1 >= 0 ? __ldg(x + c1) : make_float4(0.f, 0.f, 0.f, 0.f);
            acc.x += v0.x + v1.x;
            acc.y += v0.y + v1.y;
            acc.z += v0.z + v1.z;
            acc.w += v0.w + v1.w;
        }
        for (int o = G >> 1; o > 0; o >>= 1) {
            acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
            acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
            acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
            acc.w += __shfl_xor_sync(0xffffffffu, acc.w, o);
        }
        if (valid && lane == 0) y[r] = acc;
    }
}

// The same over packed column words (col << 8 | code), read four per
// 16-byte aligned load: a row's groups of four words alternate between its
// G lanes, two gathers in flight per lane (the access pattern of the
// product kernels' four-word form).  words must be readable up to the next
// multiple of four.
__global__ void __launch_bounds__(256) gather_probe_words4_kernel(int64_t n, int lgG,
                                                                  const int32_t *__restrict__ indptr,
                                                                  const uint32_t *__restrict__ words,
                                                                  const float4 *__restrict__ x,
                                                                  float4 *__restrict__ y)
{
    const int G = 1 << lgG;
    const int GPW = 32 >> lgG;
    const int lane = threadIdx.x & (G - 1);
    const int gsub = (threadIdx.x & 31) >> lgG;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t rb = warp * GPW; rb < n; rb += nwarps * GPW) {
        const int64_t r = rb + gsub;
        const bool valid = r < n;
        const int32_t k0 = valid ? indptr[r] : 0, k1 = valid ? indptr[r + 1] : 0;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int32_t c = (k0 & ~3) + 4 * lane; c < k1; c += 4 * G) {
            const uint4 w4 = __ldcs(reinterpret_cast<const uint4 *>(words + c));
            const uint32_t w[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
            for (int h = 0; h < 4; h += 2) {
                const bool in0 = c + h >= k0 && c + h < k1, in1 = c + h + 1 >= k0 && c + h + 1 < k1;
                const float4 v0 = in0 ? __ldg(x + (w[h] >> 8)) : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 v1 = in1 ? __ldg(x + (w[h + 1] >> 8)) : make_float4(0.f, 0.f, 0.f, 0.f);
                acc.x += v0.x + v1.x;
                acc.y += v0.y + v1.y;
                acc.z += v0.z + v1.z;
                acc.w += v0.w + v1.w;
            }
        }
        for (int o = G >> 1; o > 0; o >>= 1) {
            acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
            acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
            acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
            acc.w += __shfl_xor_sync(0xffffffffu, acc.w, o);
        }
        if (valid && lane == 0) y[r] = acc;
    }
}

}  // namespace

// y[r] = sum over row r of x[indices[k]] for an n-row CSR with int32 indptr
// and indices; x, y: 16-byte elements (n of each).  G lanes per row (2, 4, 8);
// blocks_per_sm: grid size in blocks per SM (1..16).  words4 = 1: indices
// holds packed column words (col << 8 | code), padded to a multiple of four
// plus four, read four per load.
extern "C" int bench_gather_probe(int64_t n, const int32_t *indptr, const int32_t *indices, const void *x, void *y,
                               int G, int blocks_per_sm, int words4, void *stream)
{
    if (n < 1 || !indptr || !indices || !x || !y) return -1;
    if ((G != 2 && G != 4 && G != 8) || blocks_per_sm < 1 || blocks_per_sm > 16) return -1;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -2;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) return -2;
    int lg = 0;
    while ((1 << lg) < G) lg++;
    const int64_t rows_pb = 256 / G;
    const int64_t b = (n + rows_pb - 1) / rows_pb, cap = (int64_t)sms * blocks_per_sm;
    if (words4)
        gather_probe_words4_kernel<<<(unsigned)(b > cap ? cap : b), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
            n, lg, indptr, reinterpret_cast<const uint32_t *>(indices), (const float4 *)x, (float4 *)y);
    else
        gather_probe_kernel<<<(unsigned)(b > cap ? cap : b), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
            n, lg, indptr, indices, (const float4 *)x, (float4 *)y);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}
