// Symmetry-reduced basis and Hamiltonian construction on the GPU.
//
// Replaces, for the hot path, the native basis core QuSpin 1.0.1 calls in
// the un-vendored package quspin-extensions==0.1.8 (pyproject.toml:8):
//   make_basis          src/quspin/basis/basis_general/base_general.py:862-885
//   make_basis_blocks   base_general.py:901-950
//   _get_basis_index    base_general.py:281-285
//   representative      base_general.py:1085-1117
//   normalization       base_general.py:1158-1181
//   op                  base_general.py:324-336
//   inplace_op          base_general.py:395-408
// and the COO -> canonical CSR assembly of src/quspin/basis/base.py:265-304.
//
// Conventions: site i <-> bit N-1-i; a map moves the value on site i to site
// map[i] (negative entries invert); representatives are the largest orbit
// element; norms are integer character sums over the stabiliser; matrix
// elements are J * me * phase * sign * sqrt(n_j / n_i).  This file is built
// with --fmad=false so every multiply/add rounds separately: matrix elements
// are bit-identical to the CPU restatement.
#include "qs_common.cuh"
#include <cstring>
#include <cstdlib>
#include <vector>
#include <new>

#define QS_MAXMAPS 32
#define QS_MAXOPS 16

// ---------------------------------------------------------------------------
// symmetry context

struct QsSym {
    int N, nmaps, fermion, L, nbytes, sbytes;
    int pers[QS_MAXMAPS];
    int step[QS_MAXMAPS];
    void *d_tab;          // lut | flip | later_lower, contiguous
    size_t lut_elems, flip_off, ll_off, tab_bytes;
    double *d_phase;      // re[L] | im[L]
    double *d_cos;        // cos table [L]
};

template <typename S>
struct SymView {
    int N, nmaps, fermion, L, nbytes;
    int pers[QS_MAXMAPS];
    int step[QS_MAXMAPS];
    const S *lut;    // nmaps * nbytes * 256
    const S *flip;   // nmaps
    const S *ll;     // nmaps * N (fermion)
    const double *ph_re, *ph_im, *cost;
};

template <typename S>
static SymView<S> make_view(const QsSym *q)
{
    SymView<S> v;
    v.N = q->N; v.nmaps = q->nmaps; v.fermion = q->fermion; v.L = q->L; v.nbytes = q->nbytes;
    for (int k = 0; k < QS_MAXMAPS; k++) { v.pers[k] = q->pers[k]; v.step[k] = q->step[k]; }
    const S *base = reinterpret_cast<const S *>(q->d_tab);
    v.lut = base;
    v.flip = base + q->flip_off;
    v.ll = base + q->ll_off;
    v.ph_re = q->d_phase;
    v.ph_im = q->d_phase + q->L;
    v.cost = q->d_cos;
    return v;
}

// Copies the map tables into shared memory and repoints the view.
template <typename S>
__device__ __forceinline__ void stage_tables(SymView<S> &V, S *smem, size_t nelem)
{
    const S *src = V.lut;
    for (size_t i = threadIdx.x; i < nelem; i += blockDim.x) smem[i] = src[i];
    __syncthreads();
    size_t flip_off = V.flip - V.lut, ll_off = V.ll - V.lut;
    V.lut = smem;
    V.flip = smem + flip_off;
    V.ll = smem + ll_off;
}

template <typename S>
__device__ __forceinline__ S map_state(const SymView<S> &V, int k, S s, int &sign)
{
    const S *lk = V.lut + (size_t)k * V.nbytes * 256;
    S out = 0;
    for (int b = 0; b < V.nbytes; b++) out |= lk[b * 256 + (int)((s >> (8 * b)) & 0xff)];
    if (V.fermion) {
        const S *ll = V.ll + (size_t)k * V.N;
        int inv = 0;
        S m = s;
        while (m) {
            int pos;
            if (sizeof(S) == 8) pos = 63 - __clzll((long long)m);
            else pos = 31 - __clz((int)m);
            m &= ~((S)1 << pos);
            int site = V.N - 1 - pos;
            S x = s & ll[site];
            inv += (sizeof(S) == 8) ? __popcll((unsigned long long)x) : __popc((unsigned)x);
        }
        if (inv & 1) sign = -sign;
    }
    return out ^ V.flip[k];
}

// norm of s as a representative (0 if not a representative)
template <typename S>
__device__ double check_state(const SymView<S> &V, S s)
{
    const int K = V.nmaps;
    if (K == 0) return 1.0;
    S cur[QS_MAXMAPS + 1];
    int sg[QS_MAXMAPS + 1], ph[QS_MAXMAPS + 1], idx[QS_MAXMAPS];
    for (int d = 0; d <= K; d++) { cur[d] = s; sg[d] = 1; ph[d] = 0; }
    for (int d = 0; d < K; d++) idx[d] = 0;
    double norm = 0.0;
    for (;;) {
        S t = cur[K];
        if (t > s) return 0.0;
        if (t == s) norm += sg[K] * V.cost[ph[K]];
        int d = K - 1;
        while (d >= 0) {
            idx[d]++;
            if (idx[d] < V.pers[d]) {
                cur[d + 1] = map_state(V, d, cur[d + 1], sg[d + 1]);
                int p = ph[d + 1] + V.step[d];
                ph[d + 1] = p >= V.L ? p - V.L : p;
                for (int e = d + 1; e < K; e++) { cur[e + 1] = cur[d + 1]; sg[e + 1] = sg[d + 1]; ph[e + 1] = ph[d + 1]; }
                break;
            }
            idx[d] = 0;
            d--;
        }
        if (d < 0) break;
    }
    double r = floor(norm + 0.5);
    return r < 0.5 ? 0.0 : r;
}

template <typename S>
__device__ S ref_state(const SymView<S> &V, S s, int *g, int &sign_out, int &phase_out)
{
    const int K = V.nmaps;
    sign_out = 1; phase_out = 0;
    if (g) for (int d = 0; d < K; d++) g[d] = 0;
    if (K == 0) return s;
    S cur[QS_MAXMAPS + 1];
    int sg[QS_MAXMAPS + 1], ph[QS_MAXMAPS + 1], idx[QS_MAXMAPS];
    for (int d = 0; d <= K; d++) { cur[d] = s; sg[d] = 1; ph[d] = 0; }
    for (int d = 0; d < K; d++) idx[d] = 0;
    S best = s;
    for (;;) {
        S t = cur[K];
        if (t > best) {
            best = t; sign_out = sg[K]; phase_out = ph[K];
            if (g) for (int d = 0; d < K; d++) g[d] = idx[d];
        }
        int d = K - 1;
        while (d >= 0) {
            idx[d]++;
            if (idx[d] < V.pers[d]) {
                cur[d + 1] = map_state(V, d, cur[d + 1], sg[d + 1]);
                int p = ph[d + 1] + V.step[d];
                ph[d + 1] = p >= V.L ? p - V.L : p;
                for (int e = d + 1; e < K; e++) { cur[e + 1] = cur[d + 1]; sg[e + 1] = sg[d + 1]; ph[e + 1] = ph[d + 1]; }
                break;
            }
            idx[d] = 0;
            d--;
        }
        if (d < 0) break;
    }
    return best;
}

static int gcd_i(int a, int b) { while (b) { int t = a % b; a = b; b = t; } return a; }

template <typename S>
static void build_tables(QsSym *q, const int32_t *maps, std::vector<S> &tab)
{
    int N = q->N, K = q->nmaps, nb = q->nbytes;
    q->lut_elems = (size_t)K * nb * 256;
    q->flip_off = q->lut_elems;
    q->ll_off = q->flip_off + K;
    size_t total = q->ll_off + (size_t)K * N;
    tab.assign(total > 0 ? total : 1, 0);
    for (int k = 0; k < K; k++) {
        const int32_t *m = maps + (size_t)k * N;
        int dst_bit[64];
        for (int i = 0; i < N; i++) {
            int j = m[i];
            if (j < 0) { j = -(j + 1); tab[q->flip_off + k] |= (S)1 << (N - 1 - j); }
            dst_bit[N - 1 - i] = N - 1 - j;
        }
        for (int b = 0; b < nb; b++)
            for (int v = 0; v < 256; v++) {
                S img = 0;
                for (int t = 0; t < 8; t++) {
                    int src = b * 8 + t;
                    if (src >= N) break;
                    if ((v >> t) & 1) img |= (S)1 << dst_bit[src];
                }
                tab[(size_t)k * nb * 256 + b * 256 + v] = img;
            }
        if (q->fermion)
            for (int i = 0; i < N; i++) {
                S mask = 0;
                for (int j = i + 1; j < N; j++)
                    if (m[j] < m[i]) mask |= (S)1 << (N - 1 - j);
                tab[q->ll_off + (size_t)k * N + i] = mask;
            }
    }
    q->tab_bytes = tab.size() * sizeof(S);
}

extern "C" int qs_sym_create(int N, int fermion, int nmaps, const int32_t *maps, const int32_t *pers,
                             const int32_t *qs, const double *phase_re, const double *phase_im,
                             const double *costab, int L, void **out)
{
    if (!out || N < 1 || N > 64 || nmaps < 0 || nmaps > QS_MAXMAPS) return QS_ERR_ARG;
    *out = nullptr;
    QsSym *q = new (std::nothrow) QsSym();
    if (!q) return QS_ERR_ARG;
    memset(q, 0, sizeof(*q));
    q->N = N; q->nmaps = nmaps; q->fermion = fermion; q->nbytes = (N + 7) / 8;
    q->sbytes = N <= 32 ? 4 : 8;
    int Lc = 1;
    for (int k = 0; k < nmaps; k++) {
        if (pers[k] < 1) { delete q; return QS_ERR_ARG; }
        Lc = Lc / gcd_i(Lc, pers[k]) * pers[k];
        q->pers[k] = pers[k];
    }
    if (Lc != L) { delete q; return QS_ERR_ARG; }
    q->L = L;
    for (int k = 0; k < nmaps; k++) {
        long st = (long)qs[k] * (L / pers[k]);
        st %= L; if (st < 0) st += L;
        q->step[k] = (int)st;
        if (fermion)
            for (int i = 0; i < N; i++) if (maps[(size_t)k * N + i] < 0) { delete q; return QS_ERR_UNSUPPORTED; }
    }
    std::vector<uint32_t> t32;
    std::vector<uint64_t> t64;
    const void *hsrc;
    if (q->sbytes == 4) { build_tables<uint32_t>(q, maps, t32); hsrc = t32.data(); }
    else { build_tables<uint64_t>(q, maps, t64); hsrc = t64.data(); }
    if (cudaMalloc(&q->d_tab, q->tab_bytes) != cudaSuccess) { delete q; return QS_ERR_CUDA; }
    if (cudaMalloc((void **)&q->d_phase, sizeof(double) * 3 * L) != cudaSuccess) {
        cudaFree(q->d_tab); delete q; return QS_ERR_CUDA;
    }
    q->d_cos = q->d_phase + 2 * L;
    cudaMemcpy(q->d_tab, hsrc, q->tab_bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(q->d_phase, phase_re, sizeof(double) * L, cudaMemcpyHostToDevice);
    cudaMemcpy(q->d_phase + L, phase_im, sizeof(double) * L, cudaMemcpyHostToDevice);
    if (cudaMemcpy(q->d_cos, costab, sizeof(double) * L, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(q->d_tab); cudaFree(q->d_phase); delete q; return QS_ERR_CUDA;
    }
    *out = q;
    return QS_OK;
}

extern "C" int qs_sym_destroy(void *h)
{
    QsSym *q = reinterpret_cast<QsSym *>(h);
    if (!q) return QS_OK;
    cudaFree(q->d_tab);
    cudaFree(q->d_phase);
    delete q;
    return QS_OK;
}

static size_t sym_smem(const QsSym *q) { return q->tab_bytes; }

template <typename K>
static int set_smem(K kernel, size_t bytes)
{
    if (bytes > 48 * 1024) {
        if (bytes > 220 * 1024) return QS_ERR_UNSUPPORTED;
        QS_CHECK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    }
    return QS_OK;
}

// ---------------------------------------------------------------------------
// exclusive / inclusive scan of int64 (three-phase, tiles of 2048)

#define SCAN_TILE 2048
#define SCAN_THREADS 512

__device__ __forceinline__ int64_t block_scan_incl(int64_t v, int64_t *sh)
{
    // inclusive scan across a block of SCAN_THREADS threads
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        int64_t x = lane < (SCAN_THREADS / 32) ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t t = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += t;
        }
        if (lane < (SCAN_THREADS / 32)) sh[lane] = x;
    }
    __syncthreads();
    if (w > 0) v += sh[w - 1];
    __syncthreads();
    return v;
}

__global__ void scan_tile_sums(const int64_t *__restrict__ x, int64_t n, int64_t *__restrict__ sums)
{
    __shared__ int64_t sh[32];
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    int64_t acc = 0;
    for (int k = 0; k < SCAN_TILE / SCAN_THREADS; k++) {
        int64_t i = base + k * SCAN_THREADS + threadIdx.x;
        if (i < n) acc += x[i];
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t s = 0;
        for (int w = 0; w < SCAN_THREADS / 32; w++) s += sh[w];
        sums[blockIdx.x] = s;
    }
}

// in-place inclusive scan of each tile with the tile's exclusive prefix added
__global__ void scan_tiles(int64_t *__restrict__ x, int64_t n, const int64_t *__restrict__ prefix)
{
    __shared__ int64_t sh[32];
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    int64_t carry = prefix ? prefix[blockIdx.x] : 0;
    // each thread owns 4 consecutive elements
    const int PER = SCAN_TILE / SCAN_THREADS;
    int64_t v[PER];
    int64_t loc = 0;
    for (int k = 0; k < PER; k++) {
        int64_t i = base + threadIdx.x * PER + k;
        v[k] = i < n ? x[i] : 0;
        loc += v[k];
    }
    int64_t incl = block_scan_incl(loc, sh);
    int64_t run = carry + incl - loc;
    for (int k = 0; k < PER; k++) {
        run += v[k];
        int64_t i = base + threadIdx.x * PER + k;
        if (i < n) x[i] = run;
    }
}

static int64_t scan_scratch_elems(int64_t n)
{
    int64_t tot = 0;
    while (n > SCAN_TILE) {
        n = (n + SCAN_TILE - 1) / SCAN_TILE;
        tot += n + 1;
    }
    return tot + 1;
}

// In-place inclusive scan of x[0..n).  scratch: scan_scratch_elems(n) int64.
static int scan_inclusive(int64_t *x, int64_t n, int64_t *scratch, cudaStream_t st)
{
    if (n <= 0) return QS_OK;
    if (n <= SCAN_TILE) {
        scan_tiles<<<1, SCAN_THREADS, 0, st>>>(x, n, nullptr);
        return cudaGetLastError() == cudaSuccess ? QS_OK : QS_ERR_CUDA;
    }
    int64_t nt = (n + SCAN_TILE - 1) / SCAN_TILE;
    int64_t *sums = scratch;           // nt + 1: sums[0] = 0, sums[1..nt] tile sums
    scan_tile_sums<<<(unsigned)nt, SCAN_THREADS, 0, st>>>(x, n, sums + 1);
    cudaMemsetAsync(sums, 0, sizeof(int64_t), st);
    int rc = scan_inclusive(sums + 1, nt, scratch + nt + 1, st);
    if (rc) return rc;
    scan_tiles<<<(unsigned)nt, SCAN_THREADS, 0, st>>>(x, n, sums);
    return cudaGetLastError() == cudaSuccess ? QS_OK : QS_ERR_CUDA;
}

extern "C" int64_t qs_scan_scratch_elems(int64_t n) { return scan_scratch_elems(n); }

// In-place inclusive prefix sum of an int64 array on the device.
extern "C" int qs_scan_inclusive_i64(int64_t *x, int64_t n, int64_t *scratch, void *stream)
{
    if (n < 0 || (n > 0 && !x)) return QS_ERR_ARG;
    return scan_inclusive(x, n, scratch, qs_stream(stream));
}

// ---------------------------------------------------------------------------
// enumeration

#define ENUM_CH 128

__host__ __device__ static inline uint64_t binom_u64(int n, int k)
{
    if (k < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    uint64_t r = 1;
    for (int i = 1; i <= k; i++) {
        // r * m / i is an integer; split r = q*i + rem so nothing overflows
        uint64_t m = (uint64_t)(n - k + i);
        r = (r / i) * m + (r % i) * m / i;
    }
    return r;
}

extern "C" int64_t qs_enum_num_candidates(int N, int kind, int p0, int p1)
{
    if (kind == 0) return N >= 63 ? -1 : (int64_t)1 << N;
    if (kind == 1) return (int64_t)binom_u64(N, p0);
    if (kind == 2) return (int64_t)(binom_u64(N / 2, p0) * binom_u64(N / 2, p1));
    return -1;
}

template <typename S>
__device__ __forceinline__ S unrank_comb(int n, int k, uint64_t rank)
{
    S s = 0;
    for (int b = n - 1; b >= 0 && k > 0; b--) {
        uint64_t c = binom_u64(b, k);
        if (rank >= c) { s |= (S)1 << b; rank -= c; k--; }
    }
    return s;
}

template <typename S>
__device__ __forceinline__ S gosper_next(S s)
{
    S c = s & (~s + 1);
    S r = s + c;
    return (((r ^ s) >> 2) / c) | r;
}

struct EnumArgs {
    int kind, p0, p1, half;
    uint64_t total, n_lo;
    int64_t nchunks;
};

// PASS 0: count representatives per chunk into cnt[chunk + 1].
// PASS 1: write states/norms; chunk c fills [off[c], off[c+1]) from the back.
template <typename S, int PASS>
__global__ void enum_kernel(SymView<S> V, EnumArgs A, int64_t *__restrict__ off,
                            S *__restrict__ states, uint32_t *__restrict__ norms, size_t tab_elems)
{
    extern __shared__ unsigned char smem_raw[];
    stage_tables(V, reinterpret_cast<S *>(smem_raw), tab_elems);
    const S lo_full = A.kind == 2 ? (S)((uint64_t)1 << A.half) : (S)0;
    const S min_lo = (A.kind == 2 && A.p1 > 0) ? (S)(((uint64_t)1 << A.p1) - 1) : (S)0;
    for (int64_t ch = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ch < A.nchunks;
         ch += (int64_t)gridDim.x * blockDim.x) {
        uint64_t c0 = (uint64_t)ch * ENUM_CH, c1 = c0 + ENUM_CH;
        if (c1 > A.total) c1 = A.total;
        uint64_t rlo = A.total - c1, len = c1 - c0;
        S s, hi = 0, lo = 0;
        if (A.kind == 0) s = (S)rlo;
        else if (A.kind == 1) s = unrank_comb<S>(V.N, A.p0, rlo);
        else {
            hi = unrank_comb<S>(A.half, A.p0, rlo / A.n_lo);
            lo = unrank_comb<S>(A.half, A.p1, rlo % A.n_lo);
            s = (S)((hi << A.half) | lo);
        }
        int64_t wend = PASS ? off[ch + 1] : 0;
        int64_t local = 0;
        for (uint64_t t = 0; t < len; t++) {
            double nv = check_state(V, s);
            if (nv > 0.0) {
                if (PASS) {
                    int64_t w = wend - 1 - local;
                    states[w] = s;
                    norms[w] = (uint32_t)nv;
                }
                local++;
            }
            if (t + 1 == len) break;
            if (A.kind == 0) s++;
            else if (A.kind == 1) s = gosper_next(s);
            else {
                S nx = A.p1 > 0 ? gosper_next(lo) : lo_full;
                if (A.p1 > 0 && nx < lo_full) lo = nx;
                else { lo = min_lo; hi = gosper_next(hi); }
                s = (S)((hi << A.half) | lo);
            }
        }
        if (!PASS) off[ch + 1] = local;
    }
}

static int enum_setup(const QsSym *q, int kind, int p0, int p1, EnumArgs &A)
{
    int64_t tot = qs_enum_num_candidates(q->N, kind, p0, p1);
    if (tot < 0) return QS_ERR_ARG;
    A.kind = kind; A.p0 = p0; A.p1 = p1; A.half = q->N / 2;
    A.total = (uint64_t)tot;
    A.n_lo = kind == 2 ? binom_u64(q->N / 2, p1) : 1;
    A.nchunks = (int64_t)((A.total + ENUM_CH - 1) / ENUM_CH);
    if (kind == 1 && (p0 < 0 || p0 > q->N)) return QS_ERR_ARG;
    if (kind == 2 && (q->N % 2 || p0 < 0 || p1 < 0 || p0 > q->N / 2 || p1 > q->N / 2)) return QS_ERR_ARG;
    return QS_OK;
}

extern "C" int64_t qs_enum_num_chunks(int N, int kind, int p0, int p1)
{
    int64_t tot = qs_enum_num_candidates(N, kind, p0, p1);
    if (tot < 0) return -1;
    return (tot + ENUM_CH - 1) / ENUM_CH;
}

// Counts the representatives of one particle sector.  off: int64[nchunks+1]
// device buffer (becomes the chunk output offsets); scratch: int64 scan
// scratch of qs_scan_scratch_elems(nchunks) elements.  *total_out receives
// the number of states (the call synchronises the stream to read it).
extern "C" int qs_enum_count(void *sym, int kind, int p0, int p1, int64_t *off, int64_t nchunks,
                             int64_t *scratch, int64_t *total_out, void *stream)
{
    const QsSym *q = reinterpret_cast<const QsSym *>(sym);
    if (!q || !off || !total_out) return QS_ERR_ARG;
    EnumArgs A;
    int rc = enum_setup(q, kind, p0, p1, A);
    if (rc) return rc;
    if (nchunks != A.nchunks) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    QS_CHECK(cudaMemsetAsync(off, 0, sizeof(int64_t), st));
    size_t sm = sym_smem(q);
    int blocks = qs_num_sms() * 8, threads = 128;
    if (q->sbytes == 4) {
        auto k = enum_kernel<uint32_t, 0>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<blocks, threads, sm, st>>>(make_view<uint32_t>(q), A, off, nullptr, nullptr, q->tab_bytes / 4);
    } else {
        auto k = enum_kernel<uint64_t, 0>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<blocks, threads, sm, st>>>(make_view<uint64_t>(q), A, off, nullptr, nullptr, q->tab_bytes / 8);
    }
    QS_CHECK(cudaGetLastError());
    rc = scan_inclusive(off + 1, nchunks, scratch, st);
    if (rc) return rc;
    QS_CHECK(cudaMemcpyAsync(total_out, off + nchunks, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    QS_CHECK(cudaStreamSynchronize(st));
    return QS_OK;
}

// Writes the states (descending) and norms of one particle sector using the
// offsets produced by qs_enum_count.  states: uint32 (N <= 32) or uint64.
extern "C" int qs_enum_write(void *sym, int kind, int p0, int p1, const int64_t *off, int64_t nchunks,
                             void *states, uint32_t *norms, void *stream)
{
    const QsSym *q = reinterpret_cast<const QsSym *>(sym);
    if (!q || !off || !states || !norms) return QS_ERR_ARG;
    EnumArgs A;
    int rc = enum_setup(q, kind, p0, p1, A);
    if (rc) return rc;
    if (nchunks != A.nchunks) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    size_t sm = sym_smem(q);
    int blocks = qs_num_sms() * 8, threads = 128;
    if (q->sbytes == 4) {
        auto k = enum_kernel<uint32_t, 1>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<blocks, threads, sm, st>>>(make_view<uint32_t>(q), A, const_cast<int64_t *>(off),
                                       reinterpret_cast<uint32_t *>(states), norms, q->tab_bytes / 4);
    } else {
        auto k = enum_kernel<uint64_t, 1>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<blocks, threads, sm, st>>>(make_view<uint64_t>(q), A, const_cast<int64_t *>(off),
                                       reinterpret_cast<uint64_t *>(states), norms, q->tab_bytes / 8);
    }
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// ---------------------------------------------------------------------------
// prefix blocks and index search

template <typename S>
__global__ void blocks_kernel(const S *__restrict__ states, int64_t Ns, int sh, int64_t nb,
                              int64_t *__restrict__ begin, int64_t *__restrict__ end)
{
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nb; p += (int64_t)gridDim.x * blockDim.x) {
        // first index whose prefix <= p, first index whose prefix < p
        int64_t lo = 0, hi = Ns;
        while (lo < hi) {
            int64_t mid = (lo + hi) >> 1;
            if ((int64_t)(states[mid] >> sh) > p) lo = mid + 1; else hi = mid;
        }
        begin[p] = lo;
        hi = Ns;
        while (lo < hi) {
            int64_t mid = (lo + hi) >> 1;
            if ((int64_t)(states[mid] >> sh) >= p) lo = mid + 1; else hi = mid;
        }
        end[p] = lo;
    }
}

extern "C" int qs_make_blocks(int N, int state_bytes, int N_p, const void *states, int64_t Ns,
                              int64_t *begin, int64_t *end, void *stream)
{
    if (N_p < 1 || N_p > N || N_p > 40 || !begin || !end) return QS_ERR_ARG;
    int64_t nb = (int64_t)1 << N_p;
    int sh = N - N_p;
    cudaStream_t st = qs_stream(stream);
    int blocks = (int)((nb + 255) / 256); if (blocks > 65535) blocks = 65535;
    if (state_bytes == 4) blocks_kernel<uint32_t><<<blocks, 256, 0, st>>>((const uint32_t *)states, Ns, sh, nb, begin, end);
    else blocks_kernel<uint64_t><<<blocks, 256, 0, st>>>((const uint64_t *)states, Ns, sh, nb, begin, end);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

struct BasisView {
    const void *states;
    const uint32_t *norms;
    int64_t Ns;
    int N_p;
    const int64_t *begin, *end;
};

template <typename S>
__device__ __forceinline__ int64_t find_index(const BasisView &B, int N, S r)
{
    const S *basis = reinterpret_cast<const S *>(B.states);
    int64_t lo = 0, hi = B.Ns;
    if (B.N_p > 0) {
        int64_t p = (int64_t)(r >> (N - B.N_p));
        lo = B.begin[p]; hi = B.end[p];
    }
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        S v = basis[mid];
        if (v == r) return mid;
        if (v > r) lo = mid + 1; else hi = mid;
    }
    return -1;
}

template <typename S>
__global__ void index_kernel(BasisView B, int N, const S *__restrict__ q, int64_t nq, int64_t *__restrict__ out)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = find_index<S>(B, N, q[i]);
}

extern "C" int qs_index(int N, int state_bytes, const void *states, int64_t Ns, int N_p, const int64_t *begin,
                        const int64_t *end, const void *queries, int64_t nq, int64_t *out, void *stream)
{
    if (nq < 0 || (nq > 0 && (!queries || !out))) return QS_ERR_ARG;
    if (nq == 0) return QS_OK;
    BasisView B{states, nullptr, Ns, N_p, begin, end};
    cudaStream_t st = qs_stream(stream);
    int blocks = (int)((nq + 255) / 256); if (blocks > qs_num_sms() * 16) blocks = qs_num_sms() * 16;
    if (state_bytes == 4) index_kernel<uint32_t><<<blocks, 256, 0, st>>>(B, N, (const uint32_t *)queries, nq, out);
    else index_kernel<uint64_t><<<blocks, 256, 0, st>>>(B, N, (const uint64_t *)queries, nq, out);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// ---------------------------------------------------------------------------
// representative / normalization

template <typename S>
__global__ void rep_kernel(SymView<S> V, size_t tab_elems, const S *__restrict__ in, int64_t n, S *__restrict__ out,
                           int32_t *__restrict__ g_out, int8_t *__restrict__ sign_out)
{
    extern __shared__ unsigned char smem_raw[];
    stage_tables(V, reinterpret_cast<S *>(smem_raw), tab_elems);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int g[QS_MAXMAPS];
        int sg, ph;
        out[i] = ref_state(V, in[i], g_out ? g : nullptr, sg, ph);
        if (g_out) for (int d = 0; d < V.nmaps; d++) g_out[i * V.nmaps + d] = g[d];
        if (sign_out) sign_out[i] = (int8_t)sg;
    }
}

extern "C" int qs_representative(void *sym, const void *states, int64_t n, void *out, int32_t *g_out,
                                 int8_t *sign_out, void *stream)
{
    const QsSym *q = reinterpret_cast<const QsSym *>(sym);
    if (!q || n < 0 || (n > 0 && (!states || !out))) return QS_ERR_ARG;
    if (n == 0) return QS_OK;
    cudaStream_t st = qs_stream(stream);
    size_t sm = sym_smem(q);
    int blocks = (int)((n + 127) / 128); if (blocks > qs_num_sms() * 8) blocks = qs_num_sms() * 8;
    int rc;
    if (q->sbytes == 4) {
        auto k = rep_kernel<uint32_t>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<blocks, 128, sm, st>>>(make_view<uint32_t>(q), q->tab_bytes / 4, (const uint32_t *)states, n,
                                   (uint32_t *)out, g_out, sign_out);
    } else {
        auto k = rep_kernel<uint64_t>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<blocks, 128, sm, st>>>(make_view<uint64_t>(q), q->tab_bytes / 8, (const uint64_t *)states, n,
                                   (uint64_t *)out, g_out, sign_out);
    }
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

template <typename S>
__global__ void norm_kernel(SymView<S> V, size_t tab_elems, const S *__restrict__ in, int64_t n, uint32_t *__restrict__ out)
{
    extern __shared__ unsigned char smem_raw[];
    stage_tables(V, reinterpret_cast<S *>(smem_raw), tab_elems);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (uint32_t)check_state(V, in[i]);
}

extern "C" int qs_normalization(void *sym, const void *states, int64_t n, uint32_t *out, void *stream)
{
    const QsSym *q = reinterpret_cast<const QsSym *>(sym);
    if (!q || n < 0 || (n > 0 && (!states || !out))) return QS_ERR_ARG;
    if (n == 0) return QS_OK;
    cudaStream_t st = qs_stream(stream);
    size_t sm = sym_smem(q);
    int blocks = (int)((n + 127) / 128); if (blocks > qs_num_sms() * 8) blocks = qs_num_sms() * 8;
    int rc;
    if (q->sbytes == 4) {
        auto k = norm_kernel<uint32_t>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<blocks, 128, sm, st>>>(make_view<uint32_t>(q), q->tab_bytes / 4, (const uint32_t *)states, n, out);
    } else {
        auto k = norm_kernel<uint64_t>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<blocks, 128, sm, st>>>(make_view<uint64_t>(q), q->tab_bytes / 8, (const uint64_t *)states, n, out);
    }
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// ---------------------------------------------------------------------------
// operator strings

// Term table (device): for term t, ops op_chr[off[t] .. off[t]+nop[t]) acting
// on sites op_site[...], coupling (J[2t], J[2t+1]).
struct TermView {
    const int32_t *nop, *off;
    const int8_t *chr;
    const int32_t *site;
    const double *J;
    int T;
};

// Local action of one operator string on a spin-1/2 state (spin operators,
// pauli = 0), right to left.  Returns false for an unknown character.
template <typename S>
__device__ __forceinline__ bool op_hcb(int N, S &r, double &mr, double &mi, const TermView &TV, int t)
{
    int n = TV.nop[t], o = TV.off[t];
    for (int k = n - 1; k >= 0; k--) {
        int b = N - 1 - TV.site[o + k];
        int bit = (int)((r >> b) & 1);
        double tmp;
        switch ((char)TV.chr[o + k]) {
        case 'I': break;
        case 'z': { double f = bit ? 0.5 : -0.5; mr *= f; mi *= f; } break;
        case 'n': if (!bit) { mr = 0.0; mi = 0.0; } break;
        case 'x': r ^= (S)1 << b; mr *= 0.5; mi *= 0.5; break;
        case 'y':
            r ^= (S)1 << b;
            if (bit) { tmp = mr; mr = -mi * 0.5; mi = tmp * 0.5; }
            else { tmp = mr; mr = mi * 0.5; mi = -tmp * 0.5; }
            break;
        case '+': if (bit) { mr = 0.0; mi = 0.0; } else r ^= (S)1 << b; break;
        case '-': if (bit) r ^= (S)1 << b; else { mr = 0.0; mi = 0.0; } break;
        default: return false;
        }
        if (mr == 0.0 && mi == 0.0) return true;
    }
    return true;
}

// Fermion action: Jordan-Wigner sign counts occupied sites with a smaller
// site index (higher bits) than the acted-on site.
template <typename S>
__device__ __forceinline__ bool op_fermion(int N, S &r, double &mr, double &mi, const TermView &TV, int t)
{
    int n = TV.nop[t], o = TV.off[t];
    for (int k = n - 1; k >= 0; k--) {
        int b = N - 1 - TV.site[o + k];
        int bit = (int)((r >> b) & 1);
        S above = (b >= (int)(8 * sizeof(S)) - 1) ? (S)0 : (S)(r >> (b + 1));
        int pc = sizeof(S) == 8 ? __popcll((unsigned long long)above) : __popc((unsigned)above);
        double sg = (pc & 1) ? -1.0 : 1.0;
        double tmp;
        switch ((char)TV.chr[o + k]) {
        case 'I': break;
        case 'z': { double f = bit ? 0.5 : -0.5; mr *= f; mi *= f; } break;
        case 'n': if (!bit) { mr = 0.0; mi = 0.0; } break;
        case 'x': r ^= (S)1 << b; mr *= sg; mi *= sg; break;
        case 'y':
            r ^= (S)1 << b;
            if (bit) { tmp = mr; mr = mi * sg; mi = -tmp * sg; }
            else { tmp = mr; mr = -mi * sg; mi = tmp * sg; }
            break;
        case '+': if (bit) { mr = 0.0; mi = 0.0; } else { r ^= (S)1 << b; mr *= sg; mi *= sg; } break;
        case '-': if (bit) { r ^= (S)1 << b; mr *= sg; mi *= sg; } else { mr = 0.0; mi = 0.0; } break;
        default: return false;
        }
        if (mr == 0.0 && mi == 0.0) return true;
    }
    return true;
}

// Matrix element of term t on ket i: returns bra index (or -1 if the image
// vanishes or is outside the sector); err |= 1 for a bad character.
template <typename S>
__device__ __forceinline__ int64_t term_element(const SymView<S> &V, const BasisView &B, const TermView &TV, int t,
                                                int64_t i, double &outr, double &outi, int &err)
{
    const S s = reinterpret_cast<const S *>(B.states)[i];
    S r = s;
    double mr = TV.J[2 * t], mi = TV.J[2 * t + 1];
    bool ok = V.fermion ? op_fermion<S>(V.N, r, mr, mi, TV, t) : op_hcb<S>(V.N, r, mr, mi, TV, t);
    outr = 0.0; outi = 0.0;
    if (!ok) { err |= 1; return -1; }
    if (mr == 0.0 && mi == 0.0) return -1;
    int sg = 1, ph = 0;
    int64_t j = i;
    if (r != s) {
        S rep = ref_state<S>(V, r, nullptr, sg, ph);
        j = (rep == s) ? i : find_index<S>(B, V.N, rep);
    }
    if (j < 0) return -1;
    double pr = V.ph_re[ph], pi = V.ph_im[ph];
    double ar = mr * pr - mi * pi;
    double ai = mr * pi + mi * pr;
    double f = sqrt((double)B.norms[j] / (double)B.norms[i]);
    if (sg < 0) f = -f;
    outr = ar * f;
    outi = ai * f;
    return j;
}

// cast a complex double matrix element into the value type T
template <typename T> struct VCast;
template <> struct VCast<double> {
    __device__ static double get(double r, double i, int &err) {
        if (i != 0.0 && fabs(i) > 1.1e-15 * fmax(1.0, fabs(r))) err |= 2;
        return r;
    }
    __device__ static bool nz(double v) { return v != 0.0; }
    __device__ static double add(double a, double b) { return a + b; }
    __device__ static double zero() { return 0.0; }
};
template <> struct VCast<float> {
    __device__ static float get(double r, double i, int &err) {
        if (i != 0.0 && fabs(i) > 1.1e-15 * fmax(1.0, fabs(r))) err |= 2;
        return (float)r;
    }
    __device__ static bool nz(float v) { return v != 0.0f; }
    __device__ static float add(float a, float b) { return a + b; }
    __device__ static float zero() { return 0.0f; }
};
template <> struct VCast<cdbl> {
    __device__ static cdbl get(double r, double i, int &) { return cdbl{r, i}; }
    __device__ static bool nz(cdbl v) { return v.x != 0.0 || v.y != 0.0; }
    __device__ static cdbl add(cdbl a, cdbl b) { return cdbl{a.x + b.x, a.y + b.y}; }
    __device__ static cdbl zero() { return cdbl{0.0, 0.0}; }
};
template <> struct VCast<cflt> {
    __device__ static cflt get(double r, double i, int &) { return cflt{(float)r, (float)i}; }
    __device__ static bool nz(cflt v) { return v.x != 0.0f || v.y != 0.0f; }
    __device__ static cflt add(cflt a, cflt b) { return cflt{a.x + b.x, a.y + b.y}; }
    __device__ static cflt zero() { return cflt{0.0f, 0.0f}; }
};

// -- reference-shaped op: one term, ME/row/col per ket --------------------

template <typename S>
__global__ void op_kernel(SymView<S> V, size_t tab_elems, BasisView B, TermView TV, int64_t *__restrict__ row,
                          int64_t *__restrict__ col, double *__restrict__ ME, int *__restrict__ d_err)
{
    extern __shared__ unsigned char smem_raw[];
    stage_tables(V, reinterpret_cast<S *>(smem_raw), tab_elems);
    int err = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < B.Ns; i += (int64_t)gridDim.x * blockDim.x) {
        double r, im;
        int64_t j = term_element<S>(V, B, TV, 0, i, r, im, err);
        row[i] = j >= 0 ? j : i;
        col[i] = i;
        ME[2 * i] = j >= 0 ? r : 0.0;
        ME[2 * i + 1] = j >= 0 ? im : 0.0;
    }
    if (err) atomicOr(d_err, err);
}

static TermView make_terms(const int32_t *nop, const int32_t *off, const int8_t *chr, const int32_t *site,
                           const double *J, int T)
{
    TermView t;
    t.nop = nop; t.off = off; t.chr = chr; t.site = site; t.J = J; t.T = T;
    return t;
}

// The reference's _core.op for a single term held in a one-entry term table.
// row/col int64[Ns]; ME complex128[Ns] (interleaved).  d_err: device int
// (bit 0: unknown operator character).
extern "C" int qs_op(void *sym, const void *states, const uint32_t *norms, int64_t Ns, int N_p, const int64_t *begin,
                     const int64_t *end, const int32_t *t_nop, const int32_t *t_off, const int8_t *t_chr,
                     const int32_t *t_site, const double *t_J, int64_t *row, int64_t *col, double *ME, int *d_err,
                     void *stream)
{
    const QsSym *q = reinterpret_cast<const QsSym *>(sym);
    if (!q || Ns < 0 || !d_err) return QS_ERR_ARG;
    if (Ns == 0) return QS_OK;
    BasisView B{states, norms, Ns, N_p, begin, end};
    TermView TV = make_terms(t_nop, t_off, t_chr, t_site, t_J, 1);
    cudaStream_t st = qs_stream(stream);
    size_t sm = sym_smem(q);
    int blocks = (int)((Ns + 127) / 128); if (blocks > qs_num_sms() * 8) blocks = qs_num_sms() * 8;
    int rc;
    if (q->sbytes == 4) {
        auto k = op_kernel<uint32_t>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<blocks, 128, sm, st>>>(make_view<uint32_t>(q), q->tab_bytes / 4, B, TV, row, col, ME, d_err);
    } else {
        auto k = op_kernel<uint64_t>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<blocks, 128, sm, st>>>(make_view<uint64_t>(q), q->tab_bytes / 8, B, TV, row, col, ME, d_err);
    }
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// ---------------------------------------------------------------------------
// canonical CSR assembly
//
// Off-diagonal terms (T of them, in the consolidated order) produce one entry
// per (ket i, term t) with a nonzero element.  Entries are bucketed by bra
// row, sorted by (column, term), summed left to right in term order, the
// diagonal array added last, exact zeros dropped: the same arithmetic as the
// reference's chain of scipy CSR additions.

#define TERM_BITS 22
#define POS_BITS 9
#define ROW_SORT_MAX 512

template <typename S, typename T>
__global__ void csr_count_kernel(SymView<S> V, size_t tab_elems, BasisView B, TermView TV,
                                 int64_t *__restrict__ rowcnt, int *__restrict__ term_flags, int *__restrict__ d_err)
{
    extern __shared__ unsigned char smem_raw[];
    stage_tables(V, reinterpret_cast<S *>(smem_raw), tab_elems);
    int err = 0;
    const int64_t total = B.Ns * (int64_t)TV.T;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x) {
        int t = (int)(w / B.Ns);
        int64_t i = w - (int64_t)t * B.Ns;
        double r, im;
        int64_t j = term_element<S>(V, B, TV, t, i, r, im, err);
        if (j < 0) continue;
        T v = VCast<T>::get(r, im, err);
        if (!VCast<T>::nz(v)) continue;
        atomicAdd((unsigned long long *)&rowcnt[j], 1ull);
        int f = 1 | (j != i ? 2 : 0);
        if ((term_flags[t] & f) != f) atomicOr(&term_flags[t], f);
    }
    if (err) atomicOr(d_err, err);
}

template <typename S, typename T>
__global__ void csr_fill_kernel(SymView<S> V, size_t tab_elems, BasisView B, TermView TV,
                                const int64_t *__restrict__ rowptr, int64_t *__restrict__ cursor,
                                uint64_t *__restrict__ keys, T *__restrict__ vals, int *__restrict__ d_err)
{
    extern __shared__ unsigned char smem_raw[];
    stage_tables(V, reinterpret_cast<S *>(smem_raw), tab_elems);
    int err = 0;
    const int64_t total = B.Ns * (int64_t)TV.T;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x) {
        int t = (int)(w / B.Ns);
        int64_t i = w - (int64_t)t * B.Ns;
        double r, im;
        int64_t j = term_element<S>(V, B, TV, t, i, r, im, err);
        if (j < 0) continue;
        T v = VCast<T>::get(r, im, err);
        if (!VCast<T>::nz(v)) continue;
        int64_t slot = rowptr[j] + (int64_t)atomicAdd((unsigned long long *)&cursor[j], 1ull);
        keys[slot] = ((uint64_t)i << (TERM_BITS + POS_BITS)) | ((uint64_t)t << POS_BITS);
        vals[slot] = v;
    }
    if (err) atomicOr(d_err, err);
}

// diag[i] = sum over diagonal terms (in order) of their element on ket i
template <typename S, typename T>
__global__ void csr_diag_kernel(SymView<S> V, size_t tab_elems, BasisView B, TermView TV, T *__restrict__ diag,
                                int *__restrict__ term_flags, int *__restrict__ d_err)
{
    extern __shared__ unsigned char smem_raw[];
    stage_tables(V, reinterpret_cast<S *>(smem_raw), tab_elems);
    int err = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < B.Ns; i += (int64_t)gridDim.x * blockDim.x) {
        T acc = VCast<T>::zero();
        for (int t = 0; t < TV.T; t++) {
            double r, im;
            int64_t j = term_element<S>(V, B, TV, t, i, r, im, err);
            if (j < 0) continue;
            if (j != i) { err |= 4; continue; }
            T v = VCast<T>::get(r, im, err);
            if (VCast<T>::nz(v)) {
                acc = VCast<T>::add(acc, v);
                if (term_flags && !(term_flags[t] & 1)) atomicOr(&term_flags[t], 1);
            }
        }
        diag[i] = acc;
    }
    if (err) atomicOr(d_err, err);
}

// One warp per row: bitonic sort of the row's keys in shared memory, then a
// serial term-ordered merge by lane 0.  Merged (col, value) pairs overwrite
// the row's range; mcount[r] receives their number.  When a diagonal array is
// given, each row range must hold one slot more than its scattered entries.
template <typename T>
__global__ void __launch_bounds__(128) csr_merge_kernel(int64_t Ns, const int64_t *__restrict__ rowptr,
                                                        const int64_t *__restrict__ fillcnt,
                                                        uint64_t *__restrict__ keys, T *__restrict__ vals,
                                                        const T *__restrict__ diag, int64_t *__restrict__ mcount,
                                                        int *__restrict__ d_err)
{
    __shared__ uint64_t sk[4][ROW_SORT_MAX];
    __shared__ T sv[4][ROW_SORT_MAX];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t nwarps = (int64_t)gridDim.x * 4;
    for (int64_t r = (int64_t)blockIdx.x * 4 + wib; r < Ns; r += nwarps) {
        const int64_t p0 = rowptr[r], p1 = rowptr[r + 1];
        // fillcnt[r] entries were scattered into [p0, p1); with a diagonal
        // array the row range holds one spare slot for a new diagonal entry
        const int len = (int)(fillcnt ? fillcnt[r] : (p1 - p0));
        if (len > ROW_SORT_MAX || (diag && (int64_t)len + 1 > p1 - p0)) {
            if (lane == 0) atomicOr(d_err, 8);
            continue;
        }
        int npow = 1;
        while (npow < len) npow <<= 1;
        for (int k = lane; k < npow; k += 32) {
            if (k < len) { sk[wib][k] = keys[p0 + k] | (uint64_t)k; sv[wib][k] = vals[p0 + k]; }
            else sk[wib][k] = ~0ull;
        }
        __syncwarp();
        for (int size = 2; size <= npow; size <<= 1) {
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int k = lane; k < npow; k += 32) {
                    int l = k ^ stride;
                    if (l > k) {
                        uint64_t a = sk[wib][k], b = sk[wib][l];
                        bool up = (k & size) == 0;
                        if ((a > b) == up) { sk[wib][k] = b; sk[wib][l] = a; }
                    }
                }
                __syncwarp();
            }
        }
        if (lane == 0) {
            const bool hasd = diag != nullptr;
            const T dv = hasd ? diag[r] : VCast<T>::zero();
            bool diag_done = !hasd;
            int out = 0;
            int k = 0;
            while (k < len || !diag_done) {
                int64_t col = k < len ? (int64_t)(sk[wib][k] >> (TERM_BITS + POS_BITS)) : INT64_MAX;
                if (!diag_done && r < col) {
                    // diagonal present only in the diagonal array
                    if (VCast<T>::nz(dv)) {
                        keys[p0 + out] = (uint64_t)r;
                        vals[p0 + out] = dv;
                        out++;
                    }
                    diag_done = true;
                    continue;
                }
                T acc = sv[wib][sk[wib][k] & ((1u << POS_BITS) - 1)];
                int kk = k + 1;
                while (kk < len && (int64_t)(sk[wib][kk] >> (TERM_BITS + POS_BITS)) == col) {
                    acc = VCast<T>::add(acc, sv[wib][sk[wib][kk] & ((1u << POS_BITS) - 1)]);
                    kk++;
                }
                if (!diag_done && col == r) { acc = VCast<T>::add(acc, dv); diag_done = true; }
                if (VCast<T>::nz(acc)) {
                    keys[p0 + out] = (uint64_t)col;
                    vals[p0 + out] = acc;
                    out++;
                }
                k = kk;
            }
            mcount[r] = out;
        }
        __syncwarp();
    }
}

template <typename T, typename I>
__global__ void csr_compact_kernel(int64_t Ns, const int64_t *__restrict__ rowptr, const uint64_t *__restrict__ keys,
                                   const T *__restrict__ vals, const int64_t *__restrict__ incl,
                                   I *__restrict__ indptr, int32_t *__restrict__ indices, T *__restrict__ data)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < Ns; r += nw) {
        int64_t start = r == 0 ? 0 : incl[r - 1];
        int64_t n = incl[r] - start;
        int64_t p0 = rowptr[r];
        for (int64_t k = lane; k < n; k += 32) {
            indices[start + k] = (int32_t)keys[p0 + k];
            data[start + k] = vals[p0 + k];
        }
        if (lane == 0) {
            indptr[r + 1] = (I)incl[r];
            if (r == 0) indptr[0] = 0;
        }
    }
}

template <typename S>
static int launch_grid(const QsSym *q, int64_t work, int threads = 128)
{
    int64_t b = (work + threads - 1) / threads;
    int64_t cap = (int64_t)qs_num_sms() * 16;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

template <typename T>
static int csr_count_t(const QsSym *q, const BasisView &B, const TermView &TV, int64_t *rowcnt, int *flags,
                       int *d_err, cudaStream_t st)
{
    size_t sm = sym_smem(q);
    int rc;
    int64_t work = B.Ns * (int64_t)TV.T;
    if (q->sbytes == 4) {
        auto k = csr_count_kernel<uint32_t, T>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<launch_grid<uint32_t>(q, work), 128, sm, st>>>(make_view<uint32_t>(q), q->tab_bytes / 4, B, TV, rowcnt,
                                                          flags, d_err);
    } else {
        auto k = csr_count_kernel<uint64_t, T>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<launch_grid<uint64_t>(q, work), 128, sm, st>>>(make_view<uint64_t>(q), q->tab_bytes / 8, B, TV, rowcnt,
                                                          flags, d_err);
    }
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

template <typename T>
static int csr_fill_t(const QsSym *q, const BasisView &B, const TermView &TV, const int64_t *rowptr, int64_t *cursor,
                      uint64_t *keys, void *vals, int *d_err, cudaStream_t st)
{
    size_t sm = sym_smem(q);
    int rc;
    int64_t work = B.Ns * (int64_t)TV.T;
    if (q->sbytes == 4) {
        auto k = csr_fill_kernel<uint32_t, T>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<launch_grid<uint32_t>(q, work), 128, sm, st>>>(make_view<uint32_t>(q), q->tab_bytes / 4, B, TV, rowptr,
                                                          cursor, keys, (T *)vals, d_err);
    } else {
        auto k = csr_fill_kernel<uint64_t, T>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<launch_grid<uint64_t>(q, work), 128, sm, st>>>(make_view<uint64_t>(q), q->tab_bytes / 8, B, TV, rowptr,
                                                          cursor, keys, (T *)vals, d_err);
    }
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

template <typename T>
static int csr_diag_t(const QsSym *q, const BasisView &B, const TermView &TV, void *diag, int *flags, int *d_err,
                      cudaStream_t st)
{
    size_t sm = sym_smem(q);
    int rc;
    if (q->sbytes == 4) {
        auto k = csr_diag_kernel<uint32_t, T>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<launch_grid<uint32_t>(q, B.Ns), 128, sm, st>>>(make_view<uint32_t>(q), q->tab_bytes / 4, B, TV, (T *)diag,
                                                          flags, d_err);
    } else {
        auto k = csr_diag_kernel<uint64_t, T>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<launch_grid<uint64_t>(q, B.Ns), 128, sm, st>>>(make_view<uint64_t>(q), q->tab_bytes / 8, B, TV, (T *)diag,
                                                          flags, d_err);
    }
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

#define DISPATCH_VT(vt, FN, ...)                                   \
    switch (vt) {                                                  \
    case QS_F32: return FN<float>(__VA_ARGS__);                    \
    case QS_F64: return FN<double>(__VA_ARGS__);                   \
    case QS_C64: return FN<cflt>(__VA_ARGS__);                     \
    case QS_C128: return FN<cdbl>(__VA_ARGS__);                    \
    default: return QS_ERR_ARG;                                    \
    }

// Pass 1 of the CSR build: per-row entry counts of the off-diagonal terms.
// rowcnt: int64[Ns + 1], zeroed, counts land in rowcnt[1 + row];
// term_flags: int32[T], zeroed (bit 0: term has a nonzero element, bit 1:
// term has an element off the diagonal).  d_err bits: 1 unknown operator
// character, 2 complex element in a real value type.
extern "C" int qs_csr_count(void *sym, int vtype, const void *states, const uint32_t *norms, int64_t Ns, int N_p,
                            const int64_t *begin, const int64_t *end, const int32_t *t_nop, const int32_t *t_off,
                            const int8_t *t_chr, const int32_t *t_site, const double *t_J, int T, int64_t *rowcnt,
                            int *term_flags, int *d_err, void *stream)
{
    const QsSym *q = reinterpret_cast<const QsSym *>(sym);
    if (!q || Ns < 0 || T < 0 || T >= (1 << TERM_BITS) || !rowcnt || !term_flags || !d_err) return QS_ERR_ARG;
    if (Ns == 0 || T == 0) return QS_OK;
    BasisView B{states, norms, Ns, N_p, begin, end};
    TermView TV = make_terms(t_nop, t_off, t_chr, t_site, t_J, T);
    DISPATCH_VT(vtype, csr_count_t, q, B, TV, rowcnt + 1, term_flags, d_err, qs_stream(stream));
}

// Pass 2: scatter entries.  rowptr: int64[Ns+1] exclusive offsets (the
// inclusive scan of rowcnt); cursor: int64[Ns] zeroed; keys uint64[nnz_pre];
// vals of the value type [nnz_pre].
extern "C" int qs_csr_fill(void *sym, int vtype, const void *states, const uint32_t *norms, int64_t Ns, int N_p,
                           const int64_t *begin, const int64_t *end, const int32_t *t_nop, const int32_t *t_off,
                           const int8_t *t_chr, const int32_t *t_site, const double *t_J, int T,
                           const int64_t *rowptr, int64_t *cursor, uint64_t *keys, void *vals, int *d_err,
                           void *stream)
{
    const QsSym *q = reinterpret_cast<const QsSym *>(sym);
    if (!q || Ns < 0 || T < 0 || T >= (1 << TERM_BITS) || !rowptr || !cursor || !d_err) return QS_ERR_ARG;
    if (Ns == 0 || T == 0) return QS_OK;
    if (Ns >= ((int64_t)1 << (64 - TERM_BITS - POS_BITS))) return QS_ERR_UNSUPPORTED;
    BasisView B{states, norms, Ns, N_p, begin, end};
    TermView TV = make_terms(t_nop, t_off, t_chr, t_site, t_J, T);
    DISPATCH_VT(vtype, csr_fill_t, q, B, TV, rowptr, cursor, keys, vals, d_err, qs_stream(stream));
}

// Diagonal array: diag[i] = sum, in term order, of the diagonal terms'
// elements (bit 4 of d_err if a term given here leaves the diagonal).
// term_flags (nullable, int32[T]): bit 0 set for terms with a nonzero element.
extern "C" int qs_csr_diag(void *sym, int vtype, const void *states, const uint32_t *norms, int64_t Ns, int N_p,
                           const int64_t *begin, const int64_t *end, const int32_t *t_nop, const int32_t *t_off,
                           const int8_t *t_chr, const int32_t *t_site, const double *t_J, int T, void *diag,
                           int *term_flags, int *d_err, void *stream)
{
    const QsSym *q = reinterpret_cast<const QsSym *>(sym);
    if (!q || Ns < 0 || T < 0 || !diag || !d_err) return QS_ERR_ARG;
    if (Ns == 0) return QS_OK;
    BasisView B{states, norms, Ns, N_p, begin, end};
    TermView TV = make_terms(t_nop, t_off, t_chr, t_site, t_J, T);
    DISPATCH_VT(vtype, csr_diag_t, q, B, TV, diag, term_flags, d_err, qs_stream(stream));
}

template <typename T>
static int csr_merge_t(int64_t Ns, const int64_t *rowptr, const int64_t *fillcnt, uint64_t *keys, void *vals,
                       const void *diag, int64_t *mcount, int *d_err, cudaStream_t st)
{
    int64_t blocks = (Ns + 3) / 4;
    int64_t cap = (int64_t)qs_num_sms() * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    csr_merge_kernel<T><<<(unsigned)blocks, 128, 0, st>>>(Ns, rowptr, fillcnt, keys, (T *)vals, (const T *)diag,
                                                          mcount, d_err);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// Pass 3: per-row sort / term-ordered sum / diagonal add / zero drop.
// fillcnt: int64[Ns] entries scattered per row (the fill cursor); with a
// diagonal array (nullable) every row range [rowptr[r], rowptr[r+1]) must
// hold fillcnt[r] + 1 slots.  mcount: int64[Ns] merged counts.  d_err bit 8:
// a row longer than 512 entries or without its spare slot.
extern "C" int qs_csr_merge(int vtype, int64_t Ns, const int64_t *rowptr, const int64_t *fillcnt, uint64_t *keys,
                            void *vals, const void *diag, int64_t *mcount, int *d_err, void *stream)
{
    if (Ns < 0 || !rowptr || !fillcnt || !mcount || !d_err) return QS_ERR_ARG;
    if (Ns == 0) return QS_OK;
    DISPATCH_VT(vtype, csr_merge_t, Ns, rowptr, fillcnt, keys, vals, diag, mcount, d_err, qs_stream(stream));
}

template <typename T>
static int csr_compact_t(int64_t Ns, const int64_t *rowptr, const uint64_t *keys, const void *vals,
                         const int64_t *incl, void *indptr, int idx64, int32_t *indices, void *data, cudaStream_t st)
{
    int64_t blocks = (Ns * 32 + 255) / 256;
    int64_t cap = (int64_t)qs_num_sms() * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    if (idx64)
        csr_compact_kernel<T, int64_t><<<(unsigned)blocks, 256, 0, st>>>(Ns, rowptr, keys, (const T *)vals, incl,
                                                                        (int64_t *)indptr, indices, (T *)data);
    else
        csr_compact_kernel<T, int32_t><<<(unsigned)blocks, 256, 0, st>>>(Ns, rowptr, keys, (const T *)vals, incl,
                                                                        (int32_t *)indptr, indices, (T *)data);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// Pass 4: write the canonical CSR.  incl: inclusive scan of mcount;
// indptr int32 or int64 (idx64) [Ns+1]; indices int32[nnz]; data [nnz].
extern "C" int qs_csr_compact(int vtype, int64_t Ns, const int64_t *rowptr, const uint64_t *keys, const void *vals,
                              const int64_t *incl, void *indptr, int idx64, int32_t *indices, void *data,
                              void *stream)
{
    if (Ns < 0 || !rowptr || !incl || !indptr) return QS_ERR_ARG;
    if (Ns == 0) return QS_OK;
    DISPATCH_VT(vtype, csr_compact_t, Ns, rowptr, keys, vals, incl, indptr, idx64, indices, data, qs_stream(stream));
}

// ---------------------------------------------------------------------------
// matrix-free apply (the reference's inplace_op)
//
// v_out[j, c] += a * ME(i -> j) * v_in[i, c]  over every ket i and term t;
// transposed swaps the roles of i and j; conjugated conjugates ME.  Complex
// vectors (complex128, C order [Ns, nvec]); the scatter uses atomics.

template <typename S>
__global__ void inplace_kernel(SymView<S> V, size_t tab_elems, BasisView B, TermView TV, int transposed,
                               int conjugated, double ar, double ai, const cdbl *__restrict__ vin,
                               cdbl *__restrict__ vout, int64_t nvec, int *__restrict__ d_err)
{
    extern __shared__ unsigned char smem_raw[];
    stage_tables(V, reinterpret_cast<S *>(smem_raw), tab_elems);
    int err = 0;
    const int64_t total = B.Ns * (int64_t)TV.T;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x) {
        int t = (int)(w / B.Ns);
        int64_t i = w - (int64_t)t * B.Ns;
        double r, im;
        int64_t j = term_element<S>(V, B, TV, t, i, r, im, err);
        if (j < 0) continue;
        if (conjugated) im = -im;
        double mr = ar * r - ai * im, mi = ar * im + ai * r;
        int64_t dst = transposed ? i : j, src = transposed ? j : i;
        for (int64_t c = 0; c < nvec; c++) {
            cdbl x = vin[src * nvec + c];
            atomicAdd(&vout[dst * nvec + c].x, mr * x.x - mi * x.y);
            atomicAdd(&vout[dst * nvec + c].y, mr * x.y + mi * x.x);
        }
    }
    if (err) atomicOr(d_err, err);
}

extern "C" int qs_inplace_op(void *sym, const void *states, const uint32_t *norms, int64_t Ns, int N_p,
                             const int64_t *begin, const int64_t *end, const int32_t *t_nop, const int32_t *t_off,
                             const int8_t *t_chr, const int32_t *t_site, const double *t_J, int T, int transposed,
                             int conjugated, double a_re, double a_im, const void *v_in, void *v_out, int64_t nvec,
                             int *d_err, void *stream)
{
    const QsSym *q = reinterpret_cast<const QsSym *>(sym);
    if (!q || Ns < 0 || T < 0 || nvec < 1 || !v_in || !v_out || !d_err) return QS_ERR_ARG;
    if (Ns == 0 || T == 0) return QS_OK;
    BasisView B{states, norms, Ns, N_p, begin, end};
    TermView TV = make_terms(t_nop, t_off, t_chr, t_site, t_J, T);
    cudaStream_t st = qs_stream(stream);
    size_t sm = sym_smem(q);
    int64_t work = Ns * (int64_t)T;
    int rc;
    if (q->sbytes == 4) {
        auto k = inplace_kernel<uint32_t>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<launch_grid<uint32_t>(q, work), 128, sm, st>>>(make_view<uint32_t>(q), q->tab_bytes / 4, B, TV,
                                                          transposed, conjugated, a_re, a_im, (const cdbl *)v_in,
                                                          (cdbl *)v_out, nvec, d_err);
    } else {
        auto k = inplace_kernel<uint64_t>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<launch_grid<uint64_t>(q, work), 128, sm, st>>>(make_view<uint64_t>(q), q->tab_bytes / 8, B, TV,
                                                          transposed, conjugated, a_re, a_im, (const cdbl *)v_in,
                                                          (cdbl *)v_out, nvec, d_err);
    }
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// ---------------------------------------------------------------------------
// conjugate transpose of a CSR matrix (the rmatvec operand of the 1-norm
// estimator): entries are bucketed by column, then the row merge above puts
// each new row in ascending order.  Keys carry the original row in the
// column position of the merge's (column, term) key.

template <typename IT>
__global__ void csr_t_count_kernel(int64_t n, const IT *__restrict__ indptr, const int32_t *__restrict__ indices,
                                   int64_t *__restrict__ cnt)
{
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        for (IT k = indptr[r]; k < indptr[r + 1]; k++) atomicAdd((unsigned long long *)&cnt[indices[k]], 1ull);
}

template <typename T> __device__ __forceinline__ T conj_of(T v) { return v; }
template <> __device__ __forceinline__ cdbl conj_of<cdbl>(cdbl v) { return cdbl{v.x, -v.y}; }
template <> __device__ __forceinline__ cflt conj_of<cflt>(cflt v) { return cflt{v.x, -v.y}; }

template <typename T, typename IT>
__global__ void csr_t_fill_kernel(int64_t n, const IT *__restrict__ indptr, const int32_t *__restrict__ indices,
                                  const T *__restrict__ data, const int64_t *__restrict__ rowptr,
                                  int64_t *__restrict__ cursor, uint64_t *__restrict__ keys, T *__restrict__ vals)
{
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        for (IT k = indptr[r]; k < indptr[r + 1]; k++) {
            const int64_t c = indices[k];
            const int64_t slot = rowptr[c] + (int64_t)atomicAdd((unsigned long long *)&cursor[c], 1ull);
            keys[slot] = (uint64_t)r << (TERM_BITS + POS_BITS);
            vals[slot] = conj_of(data[k]);
        }
}

template <typename T>
static int csr_t_fill_t(int64_t n, const void *indptr, int idx64, const int32_t *indices, const void *data,
                        const int64_t *rowptr, int64_t *cursor, uint64_t *keys, void *vals, cudaStream_t st)
{
    int64_t b = (n + 255) / 256, cap = (int64_t)qs_num_sms() * 16;
    unsigned blocks = (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
    if (idx64)
        csr_t_fill_kernel<T, int64_t><<<blocks, 256, 0, st>>>(n, (const int64_t *)indptr, indices, (const T *)data,
                                                               rowptr, cursor, keys, (T *)vals);
    else
        csr_t_fill_kernel<T, int32_t><<<blocks, 256, 0, st>>>(n, (const int32_t *)indptr, indices, (const T *)data,
                                                               rowptr, cursor, keys, (T *)vals);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// Column counts of an n x n CSR into cnt[1 + col] (cnt zeroed, int64[n+1]).
extern "C" int qs_csr_t_count(int64_t n, const void *indptr, int idx64, const int32_t *indices, int64_t *cnt,
                              void *stream)
{
    if (n < 0 || !indptr || !cnt) return QS_ERR_ARG;
    if (n == 0) return QS_OK;
    cudaStream_t st = qs_stream(stream);
    int64_t b = (n + 255) / 256, cap = (int64_t)qs_num_sms() * 16;
    unsigned blocks = (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
    if (idx64) csr_t_count_kernel<int64_t><<<blocks, 256, 0, st>>>(n, (const int64_t *)indptr, indices, cnt + 1);
    else csr_t_count_kernel<int32_t><<<blocks, 256, 0, st>>>(n, (const int32_t *)indptr, indices, cnt + 1);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// Scatter the conjugated entries into column buckets (rowptr: inclusive scan
// of the counts; cursor zeroed); then qs_csr_merge (no diagonal array) and
// qs_csr_compact produce the canonical conjugate transpose.
extern "C" int qs_csr_t_fill(int vtype, int64_t n, const void *indptr, int idx64, const int32_t *indices,
                             const void *data, const int64_t *rowptr, int64_t *cursor, uint64_t *keys, void *vals,
                             void *stream)
{
    if (n < 0 || !indptr || !rowptr || !cursor) return QS_ERR_ARG;
    if (n == 0) return QS_OK;
    if (n >= ((int64_t)1 << (64 - TERM_BITS - POS_BITS))) return QS_ERR_UNSUPPORTED;
    DISPATCH_VT(vtype, csr_t_fill_t, n, indptr, idx64, indices, data, rowptr, cursor, keys, vals, qs_stream(stream));
}

// ---------------------------------------------------------------------------
// projector from the symmetry-reduced basis to the full (or the
// particle-conserving) basis: the reference's basis.get_proj / project_from /
// project_to (src/quspin/basis/basis_general/base_general.py:521-718).
//
// Column i is the symmetric state of representative s_i,
//     |psi_i> = c_i sum_{g in G} chi(g) sigma(g, s_i) |g s_i>,
//     c_i = 1 / sqrt(n_i prod_k per_k),
// summed over the odometer's group elements (maps applied map 0 first), with
// chi(g) the phase-table entry and sigma the fermion sign of g -- the pair
// term_element applies to a matrix element, so that P^dagger H_full P
// reproduces the sector matrix.  Elements reaching the same image are summed
// (for commuting maps the n_i elements of a coset carry the same chi sigma,
// so an image gets sqrt(n_i / |G|) chi sigma; for maps that do not commute
// the sums can differ or cancel).  Images whose summed unit phases fall
// below 1e-12 are dropped.  One warp per column: every group element is
// formed, the images are sorted descending in shared memory (bitonic), runs
// are summed and the entries written in ascending row order.  Two passes:
// mode 0 counts the entries of each column, mode 1 writes them.

#define PROJ_DROP 1e-12

template <typename S>
__global__ void proj_kernel(SymView<S> V, size_t tab_elems, const S *__restrict__ states,
                            const uint32_t *__restrict__ norms, int64_t Ns, int gsize, int gpow2, int pcon,
                            BasisView Pc, int mode, int64_t *__restrict__ colptr, int64_t *__restrict__ rows,
                            double *__restrict__ vals, int *__restrict__ d_err)
{
    extern __shared__ unsigned char smem_raw[];
    stage_tables(V, reinterpret_cast<S *>(smem_raw), tab_elems);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const size_t tab_bytes = (tab_elems * sizeof(S) + 15) & ~(size_t)15;
    S *key = reinterpret_cast<S *>(smem_raw + tab_bytes) + (size_t)warp * gpow2;
    int *aux = reinterpret_cast<int *>(smem_raw + tab_bytes + (size_t)wpb * gpow2 * sizeof(S)) + (size_t)warp * gpow2;
    const int K = V.nmaps;
    const S full_mask = (V.N >= (int)(8 * sizeof(S))) ? ~(S)0 : (((S)1 << V.N) - 1);
    int err = 0;
    for (int64_t i = (int64_t)blockIdx.x * wpb + warp; i < Ns; i += (int64_t)gridDim.x * wpb) {
        const S s = states[i];
        for (int e = lane; e < gpow2; e += 32) {
            S t = s;
            int sg = 1, ph = 0, pad = 0;
            if (e < gsize) {
                int rem = e;
                int dig[QS_MAXMAPS];
                for (int d = K - 1; d >= 0; d--) { dig[d] = rem % V.pers[d]; rem /= V.pers[d]; }
                for (int d = 0; d < K; d++) {
                    for (int r = 0; r < dig[d]; r++) t = map_state(V, d, t, sg);
                    ph = (int)((ph + (int64_t)dig[d] * V.step[d]) % V.L);
                }
            } else {
                pad = 1;   // padding: a copy of s that adds nothing to the sums
            }
            key[e] = t;
            aux[e] = ph | (sg < 0 ? (1 << 30) : 0) | (pad << 29);
        }
        __syncwarp();
        for (int k = 2; k <= gpow2; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int e = lane; e < gpow2; e += 32) {
                    const int x = e ^ j;
                    if (x > e) {
                        const S a = key[e], b = key[x];
                        const bool desc = (e & k) == 0;
                        if (desc ? (a < b) : (a > b)) {
                            key[e] = b; key[x] = a;
                            const int t = aux[e]; aux[e] = aux[x]; aux[x] = t;
                        }
                    }
                }
                __syncwarp();
            }
        const int64_t c0 = mode ? colptr[i] : 0, cnt = mode ? colptr[i + 1] - c0 : 0;
        const double c = 1.0 / sqrt((double)norms[i] * (double)gsize);
        int64_t base = 0;
        for (int e0 = 0; e0 < gpow2; e0 += 32) {
            const int e = e0 + lane;
            bool keep = false;
            double re = 0.0, im = 0.0;
            if (e < gpow2 && (e == 0 || key[e] != key[e - 1])) {
                const S t = key[e];
                for (int f = e; f < gpow2 && key[f] == t; f++) {
                    const int a = aux[f];
                    if ((a >> 29) & 1) continue;
                    const int ph = a & ((1 << 29) - 1);
                    const double sgn = ((a >> 30) & 1) ? -1.0 : 1.0;
                    re += sgn * V.ph_re[ph];
                    im += sgn * V.ph_im[ph];
                }
                keep = hypot(re, im) > PROJ_DROP;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            if (keep && mode) {
                const int64_t pos = base + __popc(bal & ((1u << lane) - 1u));
                if (pos < cnt) {
                    const S t = key[e];
                    int64_t row;
                    if (pcon) row = find_index<S>(Pc, V.N, t);
                    else row = (int64_t)(full_mask - t);
                    if (row < 0) err |= 4;
                    rows[c0 + pos] = row;
                    vals[2 * (c0 + pos)] = c * re;
                    vals[2 * (c0 + pos) + 1] = c * im;
                } else {
                    err |= 2;
                }
            }
            base += __popc(bal);
        }
        if (lane == 0) {
            if (!mode) colptr[i + 1] = base;
            else if (base != cnt) err |= 2;
        }
        __syncwarp();
    }
    if (err) atomicOr(d_err, err);
}

static int proj_layout(const QsSym *q, int gsize, int &gpow2, int &wpb, size_t &smem)
{
    if (gsize < 1 || gsize > 8192) return QS_ERR_UNSUPPORTED;
    gpow2 = 1;
    while (gpow2 < gsize) gpow2 <<= 1;
    wpb = 4;
    while (wpb > 1 && (size_t)wpb * gpow2 * (q->sbytes + 4) > 96 * 1024) wpb >>= 1;
    smem = ((q->tab_bytes + 15) & ~(size_t)15) + (size_t)wpb * gpow2 * (q->sbytes + 4);
    return smem > 200 * 1024 ? QS_ERR_UNSUPPORTED : QS_OK;
}

// Entries of the projector, column by column (CSC).  gsize = |G| (product
// of the map periods, <= 8192).  mode 0: colptr[i + 1] = number of entries
// of column i (colptr int64[Ns + 1]; the caller sets colptr[0] = 0 and turns
// the counts into offsets); mode 1: rows int64[colptr[Ns]] and vals
// complex128[colptr[Ns]] written from those offsets.
// pcon = 0: rows index the full space, row = 2^N - 1 - state (N <= 62);
// pcon = 1: rows index the particle-conserving basis given by p_states ...
// p_end (descending states with prefix blocks, as qs_index takes them).
// d_err bits: 2 count mismatch between the passes, 4 image outside the row
// basis.
extern "C" int qs_proj_fill(void *sym, const void *states, const uint32_t *norms, int64_t Ns, int gsize, int mode,
                            int64_t *colptr, int pcon, const void *p_states, int64_t p_Ns, int p_N_p,
                            const int64_t *p_begin, const int64_t *p_end, int64_t *rows, void *vals, int *d_err,
                            void *stream)
{
    const QsSym *q = reinterpret_cast<const QsSym *>(sym);
    if (!q || Ns < 0 || !d_err || (mode != 0 && mode != 1)) return QS_ERR_ARG;
    if (Ns > 0 && (!states || !norms || !colptr || (mode == 1 && (!rows || !vals)))) return QS_ERR_ARG;
    if (pcon && mode == 1 && (!p_states || p_Ns < 0)) return QS_ERR_ARG;
    if (!pcon && q->N > 62) return QS_ERR_UNSUPPORTED;
    int prod = 1;
    for (int d = 0; d < q->nmaps; d++) {
        prod *= q->pers[d];
        if (prod > 8192) return QS_ERR_UNSUPPORTED;
    }
    if (prod != gsize) return QS_ERR_ARG;
    if (Ns == 0) return QS_OK;
    int gpow2, wpb;
    size_t sm;
    int rc = proj_layout(q, gsize, gpow2, wpb, sm);
    if (rc) return rc;
    BasisView Pc{p_states, nullptr, p_Ns, p_N_p, p_begin, p_end};
    cudaStream_t st = qs_stream(stream);
    int64_t b = (Ns + wpb - 1) / wpb, cap = (int64_t)qs_num_sms() * 16;
    const unsigned blocks = (unsigned)(b > cap ? cap : b);
    if (q->sbytes == 4) {
        auto k = proj_kernel<uint32_t>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<blocks, 32 * wpb, sm, st>>>(make_view<uint32_t>(q), q->tab_bytes / 4, (const uint32_t *)states, norms,
                                        Ns, gsize, gpow2, pcon, Pc, mode, colptr, rows, (double *)vals, d_err);
    } else {
        auto k = proj_kernel<uint64_t>;
        if ((rc = set_smem(k, sm))) return rc;
        k<<<blocks, 32 * wpb, sm, st>>>(make_view<uint64_t>(q), q->tab_bytes / 8, (const uint64_t *)states, norms,
                                        Ns, gsize, gpow2, pcon, Pc, mode, colptr, rows, (double *)vals, d_err);
    }
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

namespace {

// y[rows[e], c] += P[e] x[i, c] for the entries e of column i (one warp per
// column; the columns of one projector own disjoint rows -- disjoint
// orbits -- so no atomics).
__global__ void proj_from_kernel(int64_t Ns, const int64_t *__restrict__ colptr, const int64_t *__restrict__ rows,
                                 const cdbl *__restrict__ P, const cdbl *__restrict__ x, int64_t k,
                                 cdbl *__restrict__ y)
{
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (int64_t i = (int64_t)blockIdx.x * wpb + (threadIdx.x >> 5); i < Ns; i += (int64_t)gridDim.x * wpb)
        for (int64_t e = colptr[i] + lane; e < colptr[i + 1]; e += 32) {
            const cdbl p = P[e];
            const int64_t r = rows[e];
            for (int64_t c = 0; c < k; c++) {
                const cdbl v = x[i * k + c];
                cdbl *o = y + r * k + c;
                o->x += p.x * v.x - p.y * v.y;
                o->y += p.x * v.y + p.y * v.x;
            }
        }
}

// y[i, c] = sum_e conj(P[e]) x[rows[e], c] (one warp per column, fixed-order
// lane partials and butterfly sum).
__global__ void proj_to_kernel(int64_t Ns, const int64_t *__restrict__ colptr, const int64_t *__restrict__ rows,
                               const cdbl *__restrict__ P, const cdbl *__restrict__ x, int64_t k,
                               cdbl *__restrict__ y)
{
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (int64_t i = (int64_t)blockIdx.x * wpb + (threadIdx.x >> 5); i < Ns; i += (int64_t)gridDim.x * wpb)
        for (int64_t c = 0; c < k; c++) {
            double re = 0.0, im = 0.0;
            for (int64_t e = colptr[i] + lane; e < colptr[i + 1]; e += 32) {
                const cdbl p = P[e];
                const cdbl v = x[rows[e] * k + c];
                re += p.x * v.x + p.y * v.y;
                im += p.x * v.y - p.y * v.x;
            }
            for (int o = 16; o > 0; o >>= 1) {
                re += __shfl_xor_sync(0xffffffffu, re, o);
                im += __shfl_xor_sync(0xffffffffu, im, o);
            }
            if (lane == 0) y[i * k + c] = cdbl{re, im};
        }
}

}  // namespace

// direction 0 (project_from): y[Nfull, k] += P x (zero y first for P x;
// several symmetry sectors accumulate into one full-space state);
// direction 1 (project_to): y[Ns, k] = P^dagger x.  Complex128, C order.
extern "C" int qs_proj_apply(int direction, int64_t Ns, const int64_t *colptr, const int64_t *rows, const void *P,
                             const void *x, int64_t k, void *y, void *stream)
{
    if (Ns < 0 || k < 1 || (direction != 0 && direction != 1)) return QS_ERR_ARG;
    if (Ns == 0) return QS_OK;
    if (!colptr || !rows || !P || !x || !y) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    int64_t b = (Ns + 7) / 8, cap = (int64_t)qs_num_sms() * 16;
    const unsigned blocks = (unsigned)(b > cap ? cap : b);
    if (direction == 0)
        proj_from_kernel<<<blocks, 256, 0, st>>>(Ns, colptr, rows, (const cdbl *)P, (const cdbl *)x, k, (cdbl *)y);
    else
        proj_to_kernel<<<blocks, 256, 0, st>>>(Ns, colptr, rows, (const cdbl *)P, (const cdbl *)x, k, (cdbl *)y);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}
