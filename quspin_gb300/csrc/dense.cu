// Dense FP64 panels of the Lanczos tools: block inner products
//
//   W[i, j] = sum_r op(Q[i, r]) X[r, j],   i < m, j < k,  op = conj or identity,
//
// with Q the Lanczos vectors as rows ([m, n], row stride ldq) and X either a
// C-order block of k vectors ([n, k], row stride ldx) or, with xrows, k
// vectors stored as rows ([k, n], row stride ldx), real or complex FP64.  These are
// the dense products of the reference's Lanczos tools: the Krylov matrix
// elements <q_j | O q_i> of LTLM (src/quspin/tools/lanczos/_LTLM.py:110-126),
// the overlaps <q_a | O q_0> of FTLM (_FTLM.py:95-105) and the re-projection
// h = Q A Q^H after full_ortho's orthonormalisation (_lanczos_utils.py:206-222).
//
// The contraction runs over n (millions of states) while m and k are the
// Krylov dimensions (tens to a few hundred), so the grid splits n into slices:
// each block owns a 32 x 32 tile of W and one slice, stages 16-row panels of
// Q and X through shared memory (coalesced loads, rows padded against bank
// conflicts) and accumulates in FP64.  Two accumulation forms share the
// staging: FP64 FMAs with a 2 x 4 register tile per thread (block_inner_simt,
// qs_block_inner), and FP64 tensor instructions (mma.sync m8n8k4 .f64, "DMMA";
// each of the 4 warps owns an 8-row strip of the tile, four 8 x 8
// accumulators; block_inner_dmma, qs_block_inner_dmma).  On GB300 both run
// on the FP64 pipe at about the same rate: measured with ncu on a 40 x 40
// panel over 100k rows (two 32 x 32 tiles each way, so 64 x 64 of tile work)
// the DMMA form takes 773 us with that pipe 97% busy and the FMA form 724 us
// at 94%, about 1.1 TFLOP/s of tile work either way; the FMA form is the
// default.  A complex product is four real products per panel.  The
// per-slice partial tiles go to a caller-owned scratch array and a second
// kernel sums them in a fixed order, so results are reproducible run to run.
// For k <= 2 (a matrix-vector product) a plain FP64 FMA kernel with one block
// per output element and slice is used instead.
#include "qs_common.cuh"

namespace {

constexpr int TM = 32, TN = 32, KC = 16;      // output tile and panel depth
constexpr int QS = KC + 4;                    // padded row of the Q panel (doubles)
constexpr int XS = TN + 4;                    // padded row of the X panel (doubles)

__device__ __forceinline__ void dmma(double &d0, double &d1, double a, double b)
{
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(b));
}

// Stage one KC-deep panel of Q (TM rows) and X (TN columns) into shared memory
// (zero outside [i0, m), [j0, k), [rb, r1)).
template <bool CPLX, bool CONJ, bool XR, class PQ, class PX, class PQI, class PXI>
__device__ __forceinline__ void stage_panels(int m, int k, const double *__restrict__ Q, int64_t ldq,
                                             const double *__restrict__ X, int64_t ldx, int i0, int j0, int64_t rb,
                                             int64_t r1, PQ sQr, PX sXr, PQI sQi, PXI sXi)
{
    for (int e = threadIdx.x; e < TM * KC; e += blockDim.x) {
        const int ii = e / KC, rr = e % KC;
        const int64_t r = rb + rr;
        double vr = 0.0, vi = 0.0;
        if (i0 + ii < m && r < r1) {
            if (CPLX) {
                const double *p = Q + 2 * ((int64_t)(i0 + ii) * ldq + r);
                vr = p[0];
                vi = CONJ ? -p[1] : p[1];
            } else {
                vr = Q[(int64_t)(i0 + ii) * ldq + r];
            }
        }
        sQr[ii][rr] = vr;
        if (CPLX) sQi[ii][rr] = vi;
    }
    for (int e = threadIdx.x; e < KC * TN; e += blockDim.x) {
        // consecutive threads read consecutive addresses in either layout
        const int rr = XR ? e % KC : e / TN, jj = XR ? e / KC : e % TN;
        const int64_t r = rb + rr;
        const int64_t off = XR ? (int64_t)(j0 + jj) * ldx + r : r * ldx + j0 + jj;
        double vr = 0.0, vi = 0.0;
        if (j0 + jj < k && r < r1) {
            if (CPLX) {
                vr = X[2 * off];
                vi = X[2 * off + 1];
            } else {
                vr = X[off];
            }
        }
        sXr[rr][jj] = vr;
        if (CPLX) sXi[rr][jj] = vi;
    }
}

// Partial W tile of one slice [r0, r1): part[slice][i][j] (complex: 2
// doubles).  FP64 FMAs: thread t owns rows 2 (t / 8) + {0, 1} and columns
// 4 (t % 8) + {0..3} of the 32 x 32 tile.
template <bool CPLX, bool CONJ, bool XR>
__global__ void __launch_bounds__(128) block_inner_simt(int64_t n, int m, int k, const double *__restrict__ Q,
                                                        int64_t ldq, const double *__restrict__ X, int64_t ldx,
                                                        int64_t slice, double *__restrict__ part)
{
    __shared__ double sQr[TM][QS], sXr[KC][XS];
    __shared__ double sQi[CPLX ? TM : 1][CPLX ? QS : 1], sXi[CPLX ? KC : 1][CPLX ? XS : 1];
    const int tiles_n = (k + TN - 1) / TN;
    const int ti = blockIdx.x / tiles_n, tj = blockIdx.x % tiles_n;
    const int i0 = ti * TM, j0 = tj * TN;
    const int64_t r0 = (int64_t)blockIdx.y * slice;
    int64_t r1 = r0 + slice;
    if (r1 > n) r1 = n;
    const int tr = (threadIdx.x >> 3) * 2, tc = (threadIdx.x & 7) * 4;
    double acc[2][4], acci[2][4];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[a][c] = acci[a][c] = 0.0;
    for (int64_t rb = r0; rb < r1; rb += KC) {
        stage_panels<CPLX, CONJ, XR>(m, k, Q, ldq, X, ldx, i0, j0, rb, r1, sQr, sXr, sQi, sXi);
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < KC; kk++) {
            double ar[2], ai[2], br[4], bi[4];
#pragma unroll
            for (int a = 0; a < 2; a++) {
                ar[a] = sQr[tr + a][kk];
                ai[a] = CPLX ? sQi[tr + a][kk] : 0.0;
            }
#pragma unroll
            for (int c = 0; c < 4; c++) {
                br[c] = sXr[kk][tc + c];
                bi[c] = CPLX ? sXi[kk][tc + c] : 0.0;
            }
#pragma unroll
            for (int a = 0; a < 2; a++)
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    acc[a][c] = fma(ar[a], br[c], acc[a][c]);
                    if (CPLX) {
                        // (ar + i ai)(br + i bi): re += ar br - ai bi, im += ar bi + ai br
                        acc[a][c] = fma(-ai[a], bi[c], acc[a][c]);
                        acci[a][c] = fma(ar[a], bi[c], acci[a][c]);
                        acci[a][c] = fma(ai[a], br[c], acci[a][c]);
                    }
                }
        }
        __syncthreads();
    }
    double *out = part + (int64_t)blockIdx.y * m * k * (CPLX ? 2 : 1);
#pragma unroll
    for (int a = 0; a < 2; a++) {
        const int i = i0 + tr + a;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int jj = j0 + tc + c;
            if (i < m && jj < k) {
                if (CPLX) {
                    out[2 * ((int64_t)i * k + jj)] = acc[a][c];
                    out[2 * ((int64_t)i * k + jj) + 1] = acci[a][c];
                } else {
                    out[(int64_t)i * k + jj] = acc[a][c];
                }
            }
        }
    }
}

// The same partial tile with FP64 tensor instructions (DMMA).
template <bool CPLX, bool CONJ, bool XR>
__global__ void __launch_bounds__(128) block_inner_dmma(int64_t n, int m, int k, const double *__restrict__ Q,
                                                        int64_t ldq, const double *__restrict__ X, int64_t ldx,
                                                        int64_t slice, double *__restrict__ part)
{
    __shared__ double sQr[TM][QS], sXr[KC][XS];
    __shared__ double sQi[CPLX ? TM : 1][CPLX ? QS : 1], sXi[CPLX ? KC : 1][CPLX ? XS : 1];
    const int tiles_n = (k + TN - 1) / TN;
    const int ti = blockIdx.x / tiles_n, tj = blockIdx.x % tiles_n;
    const int i0 = ti * TM, j0 = tj * TN;
    const int64_t r0 = (int64_t)blockIdx.y * slice;
    int64_t r1 = r0 + slice;
    if (r1 > n) r1 = n;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    double acc[4][2], acci[4][2];
#pragma unroll
    for (int c = 0; c < 4; c++) acc[c][0] = acc[c][1] = acci[c][0] = acci[c][1] = 0.0;
    for (int64_t rb = r0; rb < r1; rb += KC) {
        stage_panels<CPLX, CONJ, XR>(m, k, Q, ldq, X, ldx, i0, j0, rb, r1, sQr, sXr, sQi, sXi);
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < KC; kk += 4) {
            const double ar = sQr[w * 8 + g][kk + t];
            const double ai = CPLX ? sQi[w * 8 + g][kk + t] : 0.0;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const double br = sXr[kk + t][c * 8 + g];
                dmma(acc[c][0], acc[c][1], ar, br);
                if (CPLX) {
                    const double bi = sXi[kk + t][c * 8 + g];
                    // (ar + i ai)(br + i bi): re += ar br - ai bi, im += ar bi + ai br
                    dmma(acc[c][0], acc[c][1], -ai, bi);
                    dmma(acci[c][0], acci[c][1], ar, bi);
                    dmma(acci[c][0], acci[c][1], ai, br);
                }
            }
        }
        __syncthreads();
    }
    // accumulator c of warp w: rows w*8 + g, columns c*8 + 2t + {0, 1}
    double *out = part + (int64_t)blockIdx.y * m * k * (CPLX ? 2 : 1);
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int i = i0 + w * 8 + g;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int jj = j0 + c * 8 + 2 * t + h;
            if (i < m && jj < k) {
                if (CPLX) {
                    out[2 * ((int64_t)i * k + jj)] = acc[c][h];
                    out[2 * ((int64_t)i * k + jj) + 1] = acci[c][h];
                } else {
                    out[(int64_t)i * k + jj] = acc[c][h];
                }
            }
        }
    }
}

// W = sum over slices of part (fixed order)
__global__ void block_inner_sum(int64_t count, int nslice, const double *__restrict__ part, double *__restrict__ W)
{
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int sl = 0; sl < nslice; sl++) s += part[(int64_t)sl * count + e];
        W[e] = s;
    }
}

// Matrix-vector shape (k <= 2): one block per row group and slice, FP64 FMA.
template <bool CPLX, bool CONJ, bool XR>
__global__ void __launch_bounds__(256) block_inner_gemv(int64_t n, int m, int k, const double *__restrict__ Q,
                                                        int64_t ldq, const double *__restrict__ X, int64_t ldx,
                                                        int64_t slice, double *__restrict__ part)
{
    __shared__ double red[8][2];
    const int i = blockIdx.x / k, j = blockIdx.x % k;
    const int64_t r0 = (int64_t)blockIdx.y * slice;
    int64_t r1 = r0 + slice;
    if (r1 > n) r1 = n;
    double sr = 0.0, si = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const int64_t xo = XR ? (int64_t)j * ldx + r : r * ldx + j;
        if (CPLX) {
            const double qr = Q[2 * ((int64_t)i * ldq + r)];
            const double qi = CONJ ? -Q[2 * ((int64_t)i * ldq + r) + 1] : Q[2 * ((int64_t)i * ldq + r) + 1];
            const double xr = X[2 * xo], xi = X[2 * xo + 1];
            sr = fma(qr, xr, fma(-qi, xi, sr));
            si = fma(qr, xi, fma(qi, xr, si));
        } else {
            sr = fma(Q[(int64_t)i * ldq + r], X[xo], sr);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_down_sync(0xffffffffu, sr, o);
        si += __shfl_down_sync(0xffffffffu, si, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[threadIdx.x >> 5][0] = sr;
        red[threadIdx.x >> 5][1] = si;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) {
            a += red[ww][0];
            b += red[ww][1];
        }
        double *out = part + (int64_t)blockIdx.y * m * k * (CPLX ? 2 : 1);
        if (CPLX) {
            out[2 * ((int64_t)i * k + j)] = a;
            out[2 * ((int64_t)i * k + j) + 1] = b;
        } else {
            out[(int64_t)i * k + j] = a;
        }
    }
}

int64_t slices_for(int64_t n, int64_t blocks_per_slice, int64_t depth)
{
    const int64_t target = (int64_t)qs_num_sms() * 4;
    int64_t s = (target + blocks_per_slice - 1) / blocks_per_slice;
    const int64_t most = (n + depth - 1) / depth;      // at least `depth` contraction rows per slice
    if (s > most) s = most;
    if (s > 1024) s = 1024;
    return s < 1 ? 1 : s;
}

}  // namespace

// Scratch (doubles) qs_block_inner needs for these sizes.
extern "C" int64_t qs_block_inner_scratch_doubles(int64_t n, int m, int k, int cplx)
{
    if (n < 0 || m < 0 || k < 0) return -1;
    const int64_t per = (int64_t)m * k * (cplx ? 2 : 1);
    const int64_t bps = k <= 2 ? (int64_t)m * k : (int64_t)((m + TM - 1) / TM) * ((k + TN - 1) / TN);
    return per * slices_for(n, bps > 0 ? bps : 1, k <= 2 ? 2048 : 256) + 1;
}

static int block_inner_run(int64_t n, int m, int k, const double *Q, int64_t ldq, const double *X, int64_t ldx,
                           int xrows, int cplx, int conj, double *W, double *scratch, void *stream, bool dmma)
{
    if (n < 0 || m < 0 || k < 0 || ldq < n || ldx < (xrows ? n : k) || !W || !scratch) return QS_ERR_ARG;
    if (m == 0 || k == 0) return QS_OK;
    if (n > 0 && (!Q || !X)) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    const int64_t count = (int64_t)m * k * (cplx ? 2 : 1);
    if (n == 0) {
        QS_CHECK(cudaMemsetAsync(W, 0, sizeof(double) * count, st));
        return QS_OK;
    }
    int64_t nslice, slice;
    if (k <= 2) {
        nslice = slices_for(n, (int64_t)m * k, 2048);
        slice = (n + nslice - 1) / nslice;
        nslice = (n + slice - 1) / slice;
        dim3 grid((unsigned)(m * k), (unsigned)nslice);
#define QS_GEMV(C, J, XR) block_inner_gemv<C, J, XR><<<grid, 256, 0, st>>>(n, m, k, Q, ldq, X, ldx, slice, scratch)
        if (cplx) {
            if (conj) { if (xrows) QS_GEMV(true, true, true); else QS_GEMV(true, true, false); }
            else { if (xrows) QS_GEMV(true, false, true); else QS_GEMV(true, false, false); }
        } else {
            if (xrows) QS_GEMV(false, false, true); else QS_GEMV(false, false, false);
        }
#undef QS_GEMV
    } else {
        const int tiles = ((m + TM - 1) / TM) * ((k + TN - 1) / TN);
        nslice = slices_for(n, tiles, 256);
        slice = (n + nslice - 1) / nslice;
        slice = (slice + KC - 1) / KC * KC;
        nslice = (n + slice - 1) / slice;
        dim3 grid((unsigned)tiles, (unsigned)nslice);
#define QS_DMMA(C, J, XR)                                                                                    \
    do {                                                                                                     \
        if (dmma) block_inner_dmma<C, J, XR><<<grid, 128, 0, st>>>(n, m, k, Q, ldq, X, ldx, slice, scratch);  \
        else block_inner_simt<C, J, XR><<<grid, 128, 0, st>>>(n, m, k, Q, ldq, X, ldx, slice, scratch);      \
    } while (0)
        if (cplx) {
            if (conj) { if (xrows) QS_DMMA(true, true, true); else QS_DMMA(true, true, false); }
            else { if (xrows) QS_DMMA(true, false, true); else QS_DMMA(true, false, false); }
        } else {
            if (xrows) QS_DMMA(false, false, true); else QS_DMMA(false, false, false);
        }
#undef QS_DMMA
    }
    QS_CHECK(cudaGetLastError());
    int64_t b = (count + 255) / 256;
    if (b > 1024) b = 1024;
    block_inner_sum<<<(unsigned)b, 256, 0, st>>>(count, (int)nslice, scratch, W);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// W[i, j] = sum_r op(Q[i, r]) X[r, j] (see the file header).  Q: [m, >= n]
// rows with stride ldq elements; X: [n, >= k] with stride ldx elements, or
// with xrows [k, >= n] rows with stride ldx; cplx: complex128 (interleaved)
// else float64; conj: op = complex conjugate; W: [m, k] C order (complex
// interleaved); scratch: qs_block_inner_scratch_doubles.  FP64 FMAs.
extern "C" int qs_block_inner(int64_t n, int m, int k, const double *Q, int64_t ldq, const double *X, int64_t ldx,
                              int xrows, int cplx, int conj, double *W, double *scratch, void *stream)
{
    return block_inner_run(n, m, k, Q, ldq, X, ldx, xrows, cplx, conj, W, scratch, stream, false);
}

// The same with FP64 tensor instructions for k > 2 (DMMA; on GB300 no faster
// than the FMA form, kept for the comparison).
extern "C" int qs_block_inner_dmma(int64_t n, int m, int k, const double *Q, int64_t ldq, const double *X,
                                   int64_t ldx, int xrows, int cplx, int conj, double *W, double *scratch,
                                   void *stream)
{
    return block_inner_run(n, m, k, Q, ldq, X, ldx, xrows, cplx, conj, W, scratch, stream, true);
}
