// Small multilayer perceptron: inference and training kernels.
//
// Used by the learned Taylor-partition predictor (quspin_gb300/learned.py):
// features of an evolution step -> (m*, s).  Layers are dense
// y = x W^T + b with weights held as bfloat16 for the forward and backward
// products (FP32 accumulation) and FP32 master copies updated by Adam.  The
// network is tiny (a few thousand weights), so each kernel maps one thread to
// one output element; no tensor-core path is warranted.
#include "qs_common.cuh"
#include <cuda_bf16.h>

// y[b, o] = act(sum_i x[b, i] w[o, i] + bias[o]); z keeps the pre-activation.
__global__ void mlp_dense_fwd(int B, int din, int dout, const float *__restrict__ x,
                              const __nv_bfloat16 *__restrict__ w, const float *__restrict__ bias,
                              float *__restrict__ z, float *__restrict__ y, int relu)
{
    const int64_t total = (int64_t)B * dout;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)(t / dout), o = (int)(t - (int64_t)b * dout);
        float acc = bias[o];
        const float *xb = x + (int64_t)b * din;
        const __nv_bfloat16 *wo = w + (int64_t)o * din;
        for (int i = 0; i < din; i++) acc = fmaf(xb[i], __bfloat162float(wo[i]), acc);
        if (z) z[t] = acc;
        y[t] = (relu && acc < 0.f) ? 0.f : acc;
    }
}

// dx[b, i] = (sum_o dy[b, o] w[o, i]) * (relu' of zin[b, i] if zin)
__global__ void mlp_dense_bwd_x(int B, int din, int dout, const float *__restrict__ dy,
                                const __nv_bfloat16 *__restrict__ w, const float *__restrict__ zin,
                                float *__restrict__ dx)
{
    const int64_t total = (int64_t)B * din;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)(t / din), i = (int)(t - (int64_t)b * din);
        float acc = 0.f;
        const float *db = dy + (int64_t)b * dout;
        for (int o = 0; o < dout; o++) acc = fmaf(db[o], __bfloat162float(w[(int64_t)o * din + i]), acc);
        if (zin && zin[t] <= 0.f) acc = 0.f;
        dx[t] = acc;
    }
}

// gw[o, i] = sum_b dy[b, o] x[b, i];  gb[o] = sum_b dy[b, o]
__global__ void mlp_dense_bwd_w(int B, int din, int dout, const float *__restrict__ dy,
                                const float *__restrict__ x, float *__restrict__ gw, float *__restrict__ gb)
{
    const int64_t total = (int64_t)dout * (din + 1);
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int o = (int)(t / (din + 1)), i = (int)(t - (int64_t)o * (din + 1));
        float acc = 0.f;
        if (i < din) {
            for (int b = 0; b < B; b++) acc = fmaf(dy[(int64_t)b * dout + o], x[(int64_t)b * din + i], acc);
            gw[(int64_t)o * din + i] = acc;
        } else {
            for (int b = 0; b < B; b++) acc += dy[(int64_t)b * dout + o];
            gb[o] = acc;
        }
    }
}

// mean-squared-error gradient: dy = 2 (y - target) w_col / (B * dout);
// loss partial sums per block into partial[blockIdx.x]
__global__ void mlp_mse(int64_t total, int dout, const float *__restrict__ y, const float *__restrict__ target,
                        const float *__restrict__ colw, float scale, float *__restrict__ dy,
                        float *__restrict__ partial)
{
    __shared__ float sh[32];
    float s = 0.f;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const float cw = colw ? colw[t % dout] : 1.f;
        const float d = y[t] - target[t];
        dy[t] = 2.f * d * cw * scale;
        s += d * d * cw;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
        partial[blockIdx.x] = t * scale;
    }
}

// Adam on FP32 master weights; refreshes the bfloat16 copy.
__global__ void mlp_adam(int64_t n, float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                         float *__restrict__ v, __nv_bfloat16 *__restrict__ wb, float lr, float b1, float b2,
                         float eps, float c1, float c2)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        if (wb) wb[i] = __float2bfloat16_rn(wi);
    }
}

__global__ void mlp_to_bf16(int64_t n, const float *__restrict__ w, __nv_bfloat16 *__restrict__ wb)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        wb[i] = __float2bfloat16_rn(w[i]);
}

static int grid1(int64_t n)
{
    int64_t b = (n + 255) / 256, cap = (int64_t)qs_num_sms() * 8;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

extern "C" int qs_mlp_dense_fwd(int B, int din, int dout, const float *x, const void *w_bf16, const float *bias,
                                float *z, float *y, int relu, void *stream)
{
    if (B < 0 || din < 1 || dout < 1 || !x || !w_bf16 || !bias || !y) return QS_ERR_ARG;
    if (B == 0) return QS_OK;
    mlp_dense_fwd<<<grid1((int64_t)B * dout), 256, 0, qs_stream(stream)>>>(
        B, din, dout, x, (const __nv_bfloat16 *)w_bf16, bias, z, y, relu);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

extern "C" int qs_mlp_dense_bwd(int B, int din, int dout, const float *dy, const void *w_bf16, const float *x,
                                const float *zin, float *dx, float *gw, float *gb, void *stream)
{
    if (B < 1 || din < 1 || dout < 1 || !dy || !w_bf16 || !x || !gw || !gb) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    mlp_dense_bwd_w<<<grid1((int64_t)dout * (din + 1)), 256, 0, st>>>(B, din, dout, dy, x, gw, gb);
    if (dx)
        mlp_dense_bwd_x<<<grid1((int64_t)B * din), 256, 0, st>>>(B, din, dout, dy, (const __nv_bfloat16 *)w_bf16,
                                                                 zin, dx);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

extern "C" int qs_mlp_mse(int64_t total, int dout, const float *y, const float *target, const float *colw,
                          float scale, float *dy, float *partial, int nblocks, void *stream)
{
    if (total < 1 || dout < 1 || !y || !target || !dy || !partial || nblocks < 1) return QS_ERR_ARG;
    mlp_mse<<<nblocks, 256, 0, qs_stream(stream)>>>(total, dout, y, target, colw, scale, dy, partial);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

extern "C" int qs_mlp_adam(int64_t n, float *w, const float *g, float *m, float *v, void *w_bf16, float lr, float b1,
                           float b2, float eps, int step, void *stream)
{
    if (n < 1 || !w || !g || !m || !v || step < 1) return QS_ERR_ARG;
    float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    mlp_adam<<<grid1(n), 256, 0, qs_stream(stream)>>>(n, w, g, m, v, (__nv_bfloat16 *)w_bf16, lr, b1, b2, eps, c1, c2);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

extern "C" int qs_mlp_to_bf16(int64_t n, const float *w, void *w_bf16, void *stream)
{
    if (n < 1 || !w || !w_bf16) return QS_ERR_ARG;
    mlp_to_bf16<<<grid1(n), 256, 0, qs_stream(stream)>>>(n, w, (__nv_bfloat16 *)w_bf16);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}
