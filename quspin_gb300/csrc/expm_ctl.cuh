// Device control blocks of the Taylor loops and the helpers that fold the
// per-block norms into them (shared by csrc/expm.cu and csrc/expm_lp.cu).
#pragma once
#include "qs_common.cuh"

struct ExpmCtl {
    double c1;                 // ||B||_inf at the start of the current term
    unsigned long long c2;     // running max row-norm of the new term (bits of a double >= 0)
    unsigned long long fn;     // running max row-norm of F
    int done;                  // stopping test fired in this substep
    unsigned int arrive;       // blocks finished in the current launch
    long long terms;           // Taylor terms executed so far
    int nonconv;               // substeps that used all m* terms without the test firing
    int bexp;                  // B is stored scaled by 2^-bexp (paired / single-precision storage)
    int err;                   // nonzero: a bounded device wait gave up (staged term kernel)
    int pad_;
};

// block-wide max of two non-negative doubles, atomically folded into ctl
__device__ __forceinline__ void fold_max2(double a, double b, unsigned long long *ga, unsigned long long *gb)
{
    __shared__ double sa[32], sb[32];
    for (int o = 16; o > 0; o >>= 1) {
        a = fmax(a, __shfl_down_sync(0xffffffffu, a, o));
        b = fmax(b, __shfl_down_sync(0xffffffffu, b, o));
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sa[w] = a; sb[w] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ma = 0.0, mb = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) { ma = fmax(ma, sa[k]); mb = fmax(mb, sb[k]); }
        if (ga) atomicMax(ga, (unsigned long long)__double_as_longlong(ma));
        if (gb) atomicMax(gb, (unsigned long long)__double_as_longlong(mb));
    }
}

// returns true in thread 0 of the last block to arrive
__device__ __forceinline__ bool last_block(ExpmCtl *ctl)
{
    __shared__ bool is_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int t = atomicAdd(&ctl->arrive, 1u);
        is_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    return is_last;
}

#define QS_MAX_SECTORS 64

struct MultiCtl {
    unsigned int arrive;
    int nsec;
    long long terms;                       // sector-terms executed
    double c1[QS_MAX_SECTORS];
    unsigned long long c2[QS_MAX_SECTORS];
    unsigned long long fn[QS_MAX_SECTORS];
    int done[QS_MAX_SECTORS];
    int bexp[QS_MAX_SECTORS];              // B of sector b stored scaled by 2^-bexp[b]
};


__device__ __forceinline__ int sector_of(const int64_t *soff, int nsec, int64_t r)
{
    int lo = 0, hi = nsec;          // largest b with soff[b] <= r
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (soff[mid] <= r) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ bool last_block_multi(MultiCtl *ctl)
{
    __shared__ bool is_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int t = atomicAdd(&ctl->arrive, 1u);
        is_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    return is_last;
}


// Grid for the row-handout kernels: G lanes per row, 256 threads per block,
// at most 16 blocks per SM.
static inline int taylor_grid(int64_t n, int G)
{
    int64_t gpb = 256 / G;   // rows per block per iteration
    int64_t b = (n + gpb - 1) / gpb;
    int64_t cap = (int64_t)qs_num_sms() * 16;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

// Launch description shared by the single-matrix and stacked-sector forms of
// the paired-single / single-precision Taylor term (csrc/expm_lp.cu).
struct LpTerm {
    int64_t n;
    const void *indptr;
    int idx64;
    const int32_t *indices;
    const void *data;
    int dtype;
    const void *Bin;
    void *Bout;
    int btype;
    cdbl *F;
    int64_t nvec;
    cdbl mu0;                 // shift of the single-matrix form
    const cdbl *mus;          // per-sector shifts of the stacked form (device)
    const int64_t *sec_off;   // sector row offsets of the stacked form (device)
    const cdbl *coeff;
    int j;
    double tol;
    void *ctl;
    int G, U;
    int chunk_outer;          // sweep rows once per NB-wide vector chunk (needs rownorm)
    int narrow;               // chunk-outer with 4-vector chunks instead of 8
    void *rownorm;            // n double pairs of row-sum scratch for chunk_outer, or null
    cudaStream_t st;
    int occ = 0;              // single-vector float-pair shapes: 1 / 2 cap registers for 6 / 8 blocks per SM
    int64_t nnz = 0;          // stored entries (the staged kernel's copy bounds)
    int staged = 0;           // one vector: kernel of csrc/expm_st.cu (1..3 32-row, 4..7 row hand-out);
                              // several: 1..3 the vectors-across-lanes kernel of csrc/expm_vl.cu
};

// The single-vector terms of csrc/expm_st.cu.
int st_taylor_term(const LpTerm &a);
// The many-vector terms with the vectors across the lanes (csrc/expm_vl.cu).
int vl_taylor_term(const LpTerm &a, bool multi);

int lp_taylor_term(const LpTerm &a, bool multi);
// F = eta F, norms, scale exponent, then B0 = F 2^-bexp in btype storage.
int lp_taylor_rescale(int64_t n, int64_t nvec, cdbl *F, void *B0, int btype, const cdbl *eta, int use_eta,
                      const int64_t *sec_off, void *ctl, int substep_end, bool multi, cudaStream_t st);
static inline bool lp_btype(int btype) { return btype == QS_C64 || btype == QS_CPF; }
