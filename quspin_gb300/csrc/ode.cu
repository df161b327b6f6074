// Explicit Runge-Kutta stage arithmetic for hamiltonian.evolve.
//
// The reference integrates the Schroedinger equation with scipy's ode
// wrapper around Hairer's DOP853 (src/quspin/operators/hamiltonian_core.py
// :1499-1630 builds the right-hand side, src/quspin/tools/evolution.py
// :300-345 drives scipy.integrate.ode with rtol = atol = 1e-9 by default).
// On the GPU the right-hand side is the fused hamiltonian.dot (static part
// plus f_k(t) times each dynamic part); these kernels do the rest of a step
// on the device, over the state viewed as 2N real components (the view scipy's
// complex_ode takes):
//
//   qs_rk_combine: out = y + h sum_j c_j K_j       (stage vectors, new state)
//   qs_rk_error:   sum_i (e5_i / sk_i)^2 and sum_i (e3_i / sk_i)^2 with
//                  e5 = sum_j E5_j K_j, e3 = sum_j E3_j K_j and
//                  sk = atol + rtol max(|y_i|, |y_new_i|)  (Hairer's scaled
//                  error of the 5th- and 3rd-order embedded estimates)
//
// K holds the stage derivatives as nk rows of n2 doubles.  Coefficients come
// from the host by value (at most 16), so a step needs no device allocation.
#include "qs_common.cuh"

namespace {

struct Coef16 { double c[16]; };

__global__ void rk_combine_kernel(int64_t n2, const double *__restrict__ y, const double *__restrict__ K, int nk,
                                  Coef16 c, double h, double *__restrict__ out)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int j = 0; j < nk; j++) {
            const double cj = c.c[j];
            if (cj != 0.0) acc = fma(cj, __ldg(K + (int64_t)j * n2 + i), acc);
        }
        out[i] = fma(h, acc, y[i]);
    }
}

__global__ void rk_error_kernel(int64_t n2, const double *__restrict__ y0, const double *__restrict__ y1,
                                const double *__restrict__ K, int nk, Coef16 e5, Coef16 e3, double atol, double rtol,
                                double *__restrict__ partial, unsigned int *__restrict__ arrive,
                                double *__restrict__ out)
{
    double s5 = 0.0, s3 = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
        double a5 = 0.0, a3 = 0.0;
        for (int j = 0; j < nk; j++) {
            const double k = __ldg(K + (int64_t)j * n2 + i);
            a5 = fma(e5.c[j], k, a5);
            a3 = fma(e3.c[j], k, a3);
        }
        const double sk = atol + rtol * fmax(fabs(y0[i]), fabs(y1[i]));
        const double r5 = a5 / sk, r3 = a3 / sk;
        s5 = fma(r5, r5, s5);
        s3 = fma(r3, r3, s3);
    }
    __shared__ double sh5[32], sh3[32];
    __shared__ bool last;
    for (int o = 16; o > 0; o >>= 1) {
        s5 += __shfl_down_sync(0xffffffffu, s5, o);
        s3 += __shfl_down_sync(0xffffffffu, s3, o);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sh5[w] = s5; sh3[w] = s3; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t5 = 0.0, t3 = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) { t5 += sh5[k]; t3 += sh3[k]; }
        partial[2 * blockIdx.x] = t5;
        partial[2 * blockIdx.x + 1] = t3;
        __threadfence();
        last = atomicAdd(arrive, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        // fixed-order sum of the block partials: the result does not depend on block timing
        double t5 = 0.0, t3 = 0.0;
        volatile double *vp = partial;
        for (unsigned int b = 0; b < gridDim.x; b++) { t5 += vp[2 * b]; t3 += vp[2 * b + 1]; }
        out[0] = t5;
        out[1] = t3;
        *arrive = 0u;
    }
}

int grid_of(int64_t n2)
{
    int64_t b = (n2 + 255) / 256, cap = (int64_t)qs_num_sms() * 8;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

// Blocks used by qs_rk_error: its scratch holds 2 doubles per block plus one
// arrival counter (8 bytes).
extern "C" int qs_rk_error_scratch_doubles(int64_t n2) { return 2 * grid_of(n2) + 1; }

// out[i] = y[i] + h * sum_{j < nk} c[j] * K[j * n2 + i]; c: host array of nk
// doubles (nk <= 16).  out may alias y.
extern "C" int qs_rk_combine(int64_t n2, const double *y, const double *K, int nk, const double *c_host, double h,
                             double *out, void *stream)
{
    if (n2 < 0 || nk < 0 || nk > 16 || (nk > 0 && (!K || !c_host)) || (n2 > 0 && (!y || !out))) return QS_ERR_ARG;
    if (n2 == 0) return QS_OK;
    Coef16 c{};
    for (int j = 0; j < nk; j++) c.c[j] = c_host[j];
    rk_combine_kernel<<<grid_of(n2), 256, 0, qs_stream(stream)>>>(n2, y, K, nk, c, h, out);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// out[0] = sum_i (sum_j e5[j] K_j[i] / sk_i)^2, out[1] the same with e3, with
// sk_i = atol + rtol max(|y0_i|, |y1_i|); e5, e3: host arrays of nk doubles
// (nk <= 16).  scratch: qs_rk_error_scratch_doubles(n2) doubles, zeroed once
// before the first call (the counter returns to zero after every call).
extern "C" int qs_rk_error(int64_t n2, const double *y0, const double *y1, const double *K, int nk,
                           const double *e5_host, const double *e3_host, double atol, double rtol, double *scratch,
                           double *out, void *stream)
{
    if (n2 < 1 || nk < 1 || nk > 16 || !y0 || !y1 || !K || !e5_host || !e3_host || !scratch || !out) return QS_ERR_ARG;
    Coef16 a{}, b{};
    for (int j = 0; j < nk; j++) { a.c[j] = e5_host[j]; b.c[j] = e3_host[j]; }
    const int blocks = grid_of(n2);
    unsigned int *arrive = reinterpret_cast<unsigned int *>(scratch + 2 * blocks);
    rk_error_kernel<<<blocks, 256, 0, qs_stream(stream)>>>(n2, y0, y1, K, nk, a, b, atol, rtol, scratch, arrive, out);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// ---------------------------------------------------------------------------
// Adjoint helpers of the Liouville right-hand side -i (H rho - rho H), with
// rho H = (H^dagger rho^dagger)^dagger (hamiltonian_core.py:1394-1420 builds
// the same commutator from transposed products).  Square complex128 n x n
// matrices in C order; 32 x 32 tiles through shared memory so both the read
// and the write are coalesced.

namespace {

__global__ void adjoint_kernel(int64_t n, const cdbl *__restrict__ X, cdbl *__restrict__ out, cdbl alpha, int accumulate)
{
    __shared__ cdbl tile[32][33];
    const int64_t bi = (int64_t)blockIdx.y * 32, bj = (int64_t)blockIdx.x * 32;
    // load X[bi + ty + k, bj + tx]
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int64_t r = bi + k, c = bj + threadIdx.x;
        if (r < n && c < n) tile[k][threadIdx.x] = X[r * n + c];
    }
    __syncthreads();
    // out[bj + ty + k, bi + tx] (+)= alpha conj(X[bi + tx, bj + ty + k])
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int64_t r = bj + k, c = bi + threadIdx.x;
        if (r < n && c < n) {
            const cdbl x = tile[threadIdx.x][k];
            const cdbl v{alpha.x * x.x + alpha.y * x.y, alpha.y * x.x - alpha.x * x.y};   // alpha * conj(x)
            cdbl *o = out + r * n + c;
            if (accumulate) { o->x += v.x; o->y += v.y; }
            else *o = v;
        }
    }
}

}  // namespace

// out = alpha X^dagger (accumulate = 0) or out += alpha X^dagger (accumulate
// = 1) for complex128 n x n matrices; out must not alias X.
extern "C" int qs_adjoint_axpy(int64_t n, const void *X, void *out, double alpha_re, double alpha_im, int accumulate,
                               void *stream)
{
    if (n < 0 || (n > 0 && (!X || !out)) || X == out) return QS_ERR_ARG;
    if (n == 0) return QS_OK;
    const int64_t t = (n + 31) / 32;
    if (t > 65535) return QS_ERR_UNSUPPORTED;
    dim3 grid((unsigned)t, (unsigned)t), block(32, 8);
    adjoint_kernel<<<grid, block, 0, qs_stream(stream)>>>(n, (const cdbl *)X, (cdbl *)out, cdbl{alpha_re, alpha_im},
                                                         accumulate);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}
