/*
 * oracle/basis_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement (plain C + OpenMP) of the symmetry-reduced basis core that
 * QuSpin 1.0.1 calls through the un-vendored package quspin-extensions==0.1.8
 * (pinned at pyproject.toml:8).  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline / reference leg may load this library; the product
 * path (quspin_gb300/) never does.
 *
 * What is restated, and where the reference calls it:
 *   make_basis            src/quspin/basis/basis_general/base_general.py:862-885
 *   make_basis_blocks     base_general.py:901-950 (N_p rule at :935)
 *   _get_basis_index      base_general.py:281-285
 *   representative        base_general.py:1035-1117
 *   normalization         base_general.py:1119-1181
 *   op (ME,row,col)       base_general.py:292-352
 *   inplace_op            base_general.py:354-410
 *   orbit (get_proj)      base_general.py:521-582
 *
 * Conventions (documented in sphinx/source/tutorials/user_basis.rst:56-93 and
 * the class docstrings; see the header of oracle/oracle.py for the list):
 *   - site i <-> bit N-1-i of the state integer;
 *   - a map array m acts on a state by moving the value on site i to site
 *     m[i]; a negative entry m[i] = -(j+1) moves it to site j and inverts it;
 *   - group elements are M_{K-1}^{g_{K-1}} ... M_0^{g_0}, enumerated by an
 *     odometer whose innermost digit is the last map;
 *   - the representative of an orbit is its largest integer;
 *   - the norm of a representative is sum over stabilising elements of
 *     sign * Re chi(g), chi(g) = exp(-2 pi i sum_k q_k g_k / per_k);
 *   - matrix element for ket i -> bra j:
 *       ME = J * me_local * conj-phase(g) * sign * sqrt(n_j / n_i)
 *     where g brings the image state to its representative.
 *
 * All arithmetic that feeds matrix elements is written out in real
 * operations and this file is compiled with -ffp-contract=off, so the GPU
 * kernels (compiled with --fmad=false for the same code) reproduce it
 * bit for bit.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

typedef uint64_t u64;

#define ORC_MAX_MAPS 32

typedef struct {
    int N;          /* number of bits */
    int nmaps;
    int fermion;    /* 1: track fermion permutation signs */
    int L;          /* common phase denominator */
    int step[ORC_MAX_MAPS];   /* q_k * (L/per_k) mod L */
    int pers[ORC_MAX_MAPS];
    u64 *lut;       /* [nmaps][nbytes][256] permutation images */
    u64 *flip;      /* [nmaps] xor mask applied after the permutation */
    u64 *later_lower; /* [nmaps][N] fermion inversion masks (bit positions) */
    int nbytes;
} orc_sym;

static int gcd_i(int a, int b) { while (b) { int t = a % b; a = b; b = t; } return a; }

static inline int popc64(u64 x) { return __builtin_popcountll(x); }

/* Build the per-map lookup tables.  Returns 0 on success, -1 if a fermion
 * map contains an inversion (particle-hole maps are not restated). */
static int orc_sym_init(orc_sym *S, int N, int fermion, int nmaps,
                        const int32_t *maps, const int32_t *pers, const int32_t *qs)
{
    memset(S, 0, sizeof(*S));
    S->N = N; S->nmaps = nmaps; S->fermion = fermion;
    S->nbytes = (N + 7) / 8;
    int L = 1;
    for (int k = 0; k < nmaps; k++) { L = L / gcd_i(L, pers[k]) * pers[k]; S->pers[k] = pers[k]; }
    S->L = L;
    for (int k = 0; k < nmaps; k++) {
        long st = (long)qs[k] * (L / pers[k]);
        st %= L; if (st < 0) st += L;
        S->step[k] = (int)st;
    }
    if (nmaps == 0) return 0;
    S->lut = (u64 *)calloc((size_t)nmaps * S->nbytes * 256, sizeof(u64));
    S->flip = (u64 *)calloc((size_t)nmaps, sizeof(u64));
    S->later_lower = (u64 *)calloc((size_t)nmaps * 64, sizeof(u64));
    for (int k = 0; k < nmaps; k++) {
        const int32_t *m = maps + (size_t)k * N;
        int dst_bit[64];
        for (int i = 0; i < N; i++) {
            int j = m[i];
            if (j < 0) {
                if (fermion) return -1;
                j = -(j + 1);
                S->flip[k] |= (u64)1 << (N - 1 - j);
            }
            dst_bit[N - 1 - i] = N - 1 - j;   /* source bit -> destination bit */
        }
        u64 *lk = S->lut + (size_t)k * S->nbytes * 256;
        for (int byte = 0; byte < S->nbytes; byte++) {
            for (int v = 0; v < 256; v++) {
                u64 img = 0;
                for (int b = 0; b < 8; b++) {
                    int src = byte * 8 + b;
                    if (src >= N) break;
                    if ((v >> b) & 1) img |= (u64)1 << dst_bit[src];
                }
                lk[byte * 256 + v] = img;
            }
        }
        if (fermion) {
            /* site i (bit N-1-i) -> site pi(i).  For each site i, mask of
             * sites j > i with pi(j) < pi(i). */
            for (int i = 0; i < N; i++) {
                int pi_i = m[i];
                u64 mask = 0;
                for (int j = i + 1; j < N; j++)
                    if (m[j] < pi_i) mask |= (u64)1 << (N - 1 - j);
                S->later_lower[(size_t)k * 64 + i] = mask;
            }
        }
    }
    return 0;
}

static void orc_sym_free(orc_sym *S)
{
    free(S->lut); free(S->flip); free(S->later_lower);
    S->lut = NULL; S->flip = NULL; S->later_lower = NULL;
}

static inline u64 orc_map(const orc_sym *S, int k, u64 s, int *sign)
{
    const u64 *lk = S->lut + (size_t)k * S->nbytes * 256;
    u64 out = 0;
    for (int byte = 0; byte < S->nbytes; byte++)
        out |= lk[byte * 256 + ((s >> (8 * byte)) & 0xff)];
    if (S->fermion) {
        int inv = 0;
        const u64 *ll = S->later_lower + (size_t)k * 64;
        for (int i = 0; i < S->N; i++)
            if ((s >> (S->N - 1 - i)) & 1) inv += popc64(s & ll[i]);
        if (inv & 1) *sign = -*sign;
    }
    return out ^ S->flip[k];
}

/* Norm of s as a representative: 0 if some group image is larger.
 * Sum over stabilising elements of sign * cos(2 pi phi / L), rounded to the
 * nearest integer (the exact value is an integer for a one-dimensional
 * representation). */
static double orc_check_state(const orc_sym *S, u64 s, const double *costab)
{
    int K = S->nmaps;
    if (K == 0) return 1.0;
    u64 cur[ORC_MAX_MAPS + 1];
    int sg[ORC_MAX_MAPS + 1];
    int idx[ORC_MAX_MAPS];
    int ph[ORC_MAX_MAPS + 1];
    for (int d = 0; d <= K; d++) { cur[d] = s; sg[d] = 1; ph[d] = 0; }
    for (int d = 0; d < K; d++) idx[d] = 0;
    double norm = 0.0;
    for (;;) {
        u64 t = cur[K];
        if (t > s) return 0.0;
        if (t == s) norm += sg[K] * costab[ph[K]];
        int d = K - 1;
        while (d >= 0) {
            idx[d]++;
            if (idx[d] < S->pers[d]) {
                cur[d + 1] = orc_map(S, d, cur[d + 1], &sg[d + 1]);
                ph[d + 1] = (ph[d + 1] + S->step[d]) % S->L;
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

/* Representative (largest orbit element), the odometer digits g of the
 * first element reaching it, the fermion sign and the phase index. */
static u64 orc_ref_state(const orc_sym *S, u64 s, int *g, int *sign_out, int *phase_out)
{
    int K = S->nmaps;
    if (g) for (int d = 0; d < K; d++) g[d] = 0;
    *sign_out = 1; *phase_out = 0;
    if (K == 0) return s;
    u64 cur[ORC_MAX_MAPS + 1];
    int sg[ORC_MAX_MAPS + 1];
    int idx[ORC_MAX_MAPS];
    int ph[ORC_MAX_MAPS + 1];
    for (int d = 0; d <= K; d++) { cur[d] = s; sg[d] = 1; ph[d] = 0; }
    for (int d = 0; d < K; d++) idx[d] = 0;
    u64 best = s;
    for (;;) {
        u64 t = cur[K];
        if (t > best) {
            best = t; *sign_out = sg[K]; *phase_out = ph[K];
            if (g) for (int d = 0; d < K; d++) g[d] = idx[d];
        }
        int d = K - 1;
        while (d >= 0) {
            idx[d]++;
            if (idx[d] < S->pers[d]) {
                cur[d + 1] = orc_map(S, d, cur[d + 1], &sg[d + 1]);
                ph[d + 1] = (ph[d + 1] + S->step[d]) % S->L;
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

/* ---------------------------------------------------------------------- */
/* enumeration                                                            */

static double *orc_costab(const orc_sym *S)
{
    double *c = (double *)malloc(sizeof(double) * S->L);
    for (int p = 0; p < S->L; p++) {
        /* exact values on the quarter points */
        if (p == 0) c[p] = 1.0;
        else if (4 * p == S->L || 4 * p == 3 * S->L) c[p] = 0.0;
        else if (2 * p == S->L) c[p] = -1.0;
        else c[p] = cos(2.0 * M_PI * (double)p / (double)S->L);
    }
    return c;
}

static u64 binom_u64(int n, int k)
{
    if (k < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    unsigned __int128 r = 1;
    for (int i = 1; i <= k; i++) r = r * (unsigned)(n - k + i) / (unsigned)i;
    return (u64)r;
}

/* rank-th (0-based) n-bit word with popcount k, in increasing order */
static u64 unrank_comb(int n, int k, u64 rank)
{
    u64 s = 0;
    for (int b = n - 1; b >= 0 && k > 0; b--) {
        u64 c = binom_u64(b, k);   /* words with bit b clear */
        if (rank >= c) { s |= (u64)1 << b; rank -= c; k--; }
    }
    return s;
}

static inline u64 gosper_next(u64 s)
{
    u64 c = s & (~s + 1);
    u64 r = s + c;
    return (((r ^ s) >> 2) / c) | r;
}

/*
 * Enumerate the candidates of one particle sector in DESCENDING order and
 * keep the representatives with nonzero norm.
 *   kind 0: all 2^N words;  kind 1: popcount(word) == p0;
 *   kind 2: spinful -- p0 ones in the high N/2 bits, p1 in the low N/2 bits.
 * Writes at most cap states; returns the count, -2 on a bad symmetry
 * description, or -1-need when cap is too small (need = required size).
 */
int64_t orc_make_basis(int N, int fermion, int nmaps, const int32_t *maps,
                       const int32_t *pers, const int32_t *qs,
                       int kind, int p0, int p1,
                       uint64_t *states, uint32_t *norms, int64_t cap)
{
    orc_sym S;
    if (orc_sym_init(&S, N, fermion, nmaps, maps, pers, qs)) { orc_sym_free(&S); return -2; }
    double *costab = orc_costab(&S);
    int half = N / 2;
    u64 n_hi = 1, n_lo = 1;
    if (kind == 0) { n_hi = (N == 64) ? 0 : ((u64)1 << N); n_lo = 1; }
    else if (kind == 1) { n_hi = binom_u64(N, p0); n_lo = 1; }
    else { n_hi = binom_u64(half, p0); n_lo = binom_u64(half, p1); }
    u64 total = n_hi * n_lo;
    /* chunks of descending candidate positions; candidate position c
     * (0 = largest word) has ascending rank total-1-c.  Each chunk walks its
     * ascending ranks with Gosper's successor and fills its output slot range
     * from the back, so the global order stays descending. */
    const u64 CH = 1 << 16;
    u64 nch = (total + CH - 1) / CH;
    int64_t *cnt = (int64_t *)calloc(nch + 1, sizeof(int64_t));
    u64 min_lo = (kind == 2 && p1 > 0) ? (((u64)1 << p1) - 1) : 0;
    for (int pass = 0; pass < 2; pass++) {
        #pragma omp parallel for schedule(dynamic, 1)
        for (u64 ch = 0; ch < nch; ch++) {
            u64 c0 = ch * CH, c1 = c0 + CH; if (c1 > total) c1 = total;
            u64 rlo = total - c1;            /* smallest ascending rank */
            u64 len = c1 - c0;
            int64_t wend = pass ? cnt[ch + 1] : 0;
            int64_t local = 0;
            u64 s = 0, hi = 0, lo = 0;
            if (kind == 0) s = rlo;
            else if (kind == 1) s = unrank_comb(N, p0, rlo);
            else {
                hi = unrank_comb(half, p0, rlo / n_lo);
                lo = unrank_comb(half, p1, rlo % n_lo);
                s = (hi << half) | lo;
            }
            for (u64 t = 0; t < len; t++) {
                double nv = orc_check_state(&S, s, costab);
                if (nv > 0.0) {
                    if (pass) {
                        int64_t w = wend - 1 - local;
                        states[w] = s; norms[w] = (uint32_t)nv;
                    }
                    local++;
                }
                if (t + 1 == len) break;
                if (kind == 0) s++;
                else if (kind == 1) s = gosper_next(s);
                else {
                    u64 rl_next_ok = (p1 > 0) ? gosper_next(lo) : ((u64)1 << half);
                    if (p1 > 0 && rl_next_ok < ((u64)1 << half)) lo = rl_next_ok;
                    else { lo = min_lo; hi = gosper_next(hi); }
                    s = (hi << half) | lo;
                }
            }
            if (!pass) cnt[ch + 1] = local;
        }
        if (!pass) {
            for (u64 ch = 0; ch < nch; ch++) cnt[ch + 1] += cnt[ch];
            /* cnt[ch+1] is the inclusive end of chunk ch in the output */
            if (cnt[nch] > cap) { int64_t need = cnt[nch]; free(cnt); free(costab); orc_sym_free(&S); return -1 - need; }
        }
    }
    int64_t Ns = cnt[nch];
    free(cnt); free(costab); orc_sym_free(&S);
    return Ns;
}

/* QuSpin's prefix blocks: for each N_p-bit prefix p, [begin[p], end[p]) is
 * the range of the descending state array whose top N_p bits equal p.
 * Empty prefixes get begin == end (the insertion point). */
void orc_make_blocks(int N, int N_p, const uint64_t *states, int64_t Ns,
                     int64_t *begin, int64_t *end)
{
    int64_t nb = (int64_t)1 << N_p;
    int sh = N - N_p;
    /* states descending: prefix descending along the array */
    int64_t pos = 0;
    for (int64_t p = nb - 1; p >= 0; p--) {
        begin[p] = pos;
        while (pos < Ns && (int64_t)(states[pos] >> sh) == p) pos++;
        end[p] = pos;
    }
}

static inline int64_t orc_search(const uint64_t *basis, int64_t lo, int64_t hi, u64 r)
{
    /* descending array: find r in [lo, hi) */
    while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        u64 v = basis[mid];
        if (v == r) return mid;
        if (v > r) lo = mid + 1; else hi = mid;
    }
    return -1;
}

static inline int64_t orc_index(int N, int N_p, const uint64_t *basis, int64_t Ns,
                                const int64_t *begin, const int64_t *end, u64 r)
{
    if (N_p > 0) {
        u64 p = r >> (N - N_p);
        return orc_search(basis, begin[p], end[p], r);
    }
    return orc_search(basis, 0, Ns, r);
}

void orc_index_many(int N, int N_p, const uint64_t *basis, int64_t Ns,
                    const int64_t *begin, const int64_t *end,
                    const uint64_t *q, int64_t nq, int64_t *out)
{
    #pragma omp parallel for
    for (int64_t i = 0; i < nq; i++) out[i] = orc_index(N, N_p, basis, Ns, begin, end, q[i]);
}

int orc_representative(int N, int fermion, int nmaps, const int32_t *maps,
                       const int32_t *pers, const int32_t *qs,
                       const uint64_t *states, int64_t n, uint64_t *out,
                       int32_t *g_out, int8_t *sign_out)
{
    orc_sym S;
    if (orc_sym_init(&S, N, fermion, nmaps, maps, pers, qs)) { orc_sym_free(&S); return -2; }
    #pragma omp parallel for
    for (int64_t i = 0; i < n; i++) {
        int g[ORC_MAX_MAPS]; int sg, ph;
        out[i] = orc_ref_state(&S, states[i], g, &sg, &ph);
        if (g_out) for (int d = 0; d < nmaps; d++) g_out[i * nmaps + d] = g[d];
        if (sign_out) sign_out[i] = (int8_t)sg;
    }
    orc_sym_free(&S);
    return 0;
}

int orc_normalization(int N, int fermion, int nmaps, const int32_t *maps,
                      const int32_t *pers, const int32_t *qs,
                      const uint64_t *states, int64_t n, uint32_t *out)
{
    orc_sym S;
    if (orc_sym_init(&S, N, fermion, nmaps, maps, pers, qs)) { orc_sym_free(&S); return -2; }
    double *costab = orc_costab(&S);
    #pragma omp parallel for
    for (int64_t i = 0; i < n; i++) out[i] = (uint32_t)orc_check_state(&S, states[i], costab);
    free(costab);
    orc_sym_free(&S);
    return 0;
}

/* Every group element applied to each state, in the odometer order of
 * orc_ref_state: images[i*G + e], the fermion sign and the phase index of
 * the element (G = product of the periods).  The projector of get_proj
 * (base_general.py:521-582) is sum_g chi(g) sign(g) |g s> / sqrt(n |G|)
 * per representative s; the Python side sums the duplicate images. */
int orc_orbit(int N, int fermion, int nmaps, const int32_t *maps,
              const int32_t *pers, const int32_t *qs,
              const uint64_t *states, int64_t n, int64_t G,
              uint64_t *images, int8_t *signs, int32_t *phases)
{
    orc_sym S;
    if (orc_sym_init(&S, N, fermion, nmaps, maps, pers, qs)) { orc_sym_free(&S); return -2; }
    int K = S.nmaps;
    #pragma omp parallel for
    for (int64_t i = 0; i < n; i++) {
        u64 cur[ORC_MAX_MAPS + 1];
        int sg[ORC_MAX_MAPS + 1], ph[ORC_MAX_MAPS + 1], idx[ORC_MAX_MAPS];
        for (int d = 0; d <= K; d++) { cur[d] = states[i]; sg[d] = 1; ph[d] = 0; }
        for (int d = 0; d < K; d++) idx[d] = 0;
        int64_t e = 0;
        for (;;) {
            if (e < G) {
                images[i * G + e] = cur[K];
                signs[i * G + e] = (int8_t)sg[K];
                phases[i * G + e] = ph[K];
            }
            e++;
            int d = K - 1;
            while (d >= 0) {
                idx[d]++;
                if (idx[d] < S.pers[d]) {
                    cur[d + 1] = orc_map(&S, d, cur[d + 1], &sg[d + 1]);
                    ph[d + 1] = (ph[d + 1] + S.step[d]) % S.L;
                    for (int f = d + 1; f < K; f++) { cur[f + 1] = cur[d + 1]; sg[f + 1] = sg[d + 1]; ph[f + 1] = ph[d + 1]; }
                    break;
                }
                idx[d] = 0;
                d--;
            }
            if (d < 0) break;
        }
    }
    orc_sym_free(&S);
    return 0;
}

/* ---------------------------------------------------------------------- */
/* local operator action                                                  */

/* Spin-1/2 / hard-core boson action (spin-1/2 operators, pauli=0); applied
 * right to left.  Returns -1 for an unknown character. */
static inline int orc_op_hcb(int N, u64 *r, double *mr, double *mi,
                             int nop, const char *opstr, const int32_t *indx)
{
    for (int k = nop - 1; k >= 0; k--) {
        int b = N - 1 - indx[k];
        int bit = (int)((*r >> b) & 1);
        double t;
        switch (opstr[k]) {
        case 'I': break;
        case 'z': { double f = bit ? 0.5 : -0.5; *mr *= f; *mi *= f; } break;
        case 'n': if (!bit) { *mr = 0.0; *mi = 0.0; } break;
        case 'x': *r ^= (u64)1 << b; *mr *= 0.5; *mi *= 0.5; break;
        case 'y': /* S^y: up -> (i/2) down, down -> (-i/2) up */
            *r ^= (u64)1 << b;
            if (bit) { t = *mr; *mr = -*mi * 0.5; *mi = t * 0.5; }
            else     { t = *mr; *mr = *mi * 0.5;  *mi = -t * 0.5; }
            break;
        case '+': if (bit) { *mr = 0.0; *mi = 0.0; } else *r ^= (u64)1 << b; break;
        case '-': if (bit) *r ^= (u64)1 << b; else { *mr = 0.0; *mi = 0.0; } break;
        default: return -1;
        }
        if (*mr == 0.0 && *mi == 0.0) return 0;
    }
    return 0;
}

/* Fermion action; the Jordan-Wigner sign counts occupied sites with a
 * smaller site index (higher bits) than the acted-on site. */
static inline int orc_op_fermion(int N, u64 *r, double *mr, double *mi,
                                 int nop, const char *opstr, const int32_t *indx)
{
    for (int k = nop - 1; k >= 0; k--) {
        int b = N - 1 - indx[k];
        int bit = (int)((*r >> b) & 1);
        u64 above = (b == 63) ? 0 : (*r >> (b + 1));
        double sg = (popc64(above) & 1) ? -1.0 : 1.0;
        double t;
        switch (opstr[k]) {
        case 'I': break;
        case 'z': { double f = bit ? 0.5 : -0.5; *mr *= f; *mi *= f; } break;
        case 'n': if (!bit) { *mr = 0.0; *mi = 0.0; } break;
        case 'x': *r ^= (u64)1 << b; *mr *= sg; *mi *= sg; break;
        case 'y': /* -i (c - c^dagger) */
            *r ^= (u64)1 << b;
            if (bit) { t = *mr; *mr = *mi * sg; *mi = -t * sg; }   /* * (-i sg) */
            else     { t = *mr; *mr = -*mi * sg; *mi = t * sg; }   /* * (+i sg) */
            break;
        case '+': if (bit) { *mr = 0.0; *mi = 0.0; } else { *r ^= (u64)1 << b; *mr *= sg; *mi *= sg; } break;
        case '-': if (bit) { *r ^= (u64)1 << b; *mr *= sg; *mi *= sg; } else { *mr = 0.0; *mi = 0.0; } break;
        default: return -1;
        }
        if (*mr == 0.0 && *mi == 0.0) return 0;
    }
    return 0;
}

/*
 * One operator-string term over the whole basis (the reference's _core.op):
 * for every ket i, ME[i] (complex, interleaved) and row[i] = bra index,
 * col[i] = i.  ME = 0 where the image is annihilated or not in the sector.
 * phase_re/phase_im: table of exp(-2 pi i p / L), p = 0..L-1.
 * Returns 0, or -1 for an unknown operator character.
 */
int orc_op(int N, int fermion, int nmaps, const int32_t *maps,
           const int32_t *pers, const int32_t *qs,
           const double *phase_re, const double *phase_im,
           const char *opstr, const int32_t *indx, int nop,
           double J_re, double J_im,
           const uint64_t *basis, const uint32_t *norms, int64_t Ns,
           int N_p, const int64_t *begin, const int64_t *end,
           int64_t *row, int64_t *col, double *ME)
{
    orc_sym S;
    if (orc_sym_init(&S, N, fermion, nmaps, maps, pers, qs)) { orc_sym_free(&S); return -2; }
    int err = 0;
    #pragma omp parallel for reduction(|:err)
    for (int64_t i = 0; i < Ns; i++) {
        u64 s = basis[i];
        u64 r = s;
        double mr = J_re, mi = J_im;
        int e = fermion ? orc_op_fermion(N, &r, &mr, &mi, nop, opstr, indx)
                        : orc_op_hcb(N, &r, &mr, &mi, nop, opstr, indx);
        row[i] = i; col[i] = i;
        if (e) { err |= 1; ME[2 * i] = 0.0; ME[2 * i + 1] = 0.0; continue; }
        if (mr == 0.0 && mi == 0.0) { ME[2 * i] = 0.0; ME[2 * i + 1] = 0.0; continue; }
        int sg = 1, ph = 0;
        int64_t j = i;
        if (r != s) {
            u64 rep = orc_ref_state(&S, r, NULL, &sg, &ph);
            j = (rep == s) ? i : orc_index(N, N_p, basis, Ns, begin, end, rep);
        }
        if (j < 0) { ME[2 * i] = 0.0; ME[2 * i + 1] = 0.0; continue; }
        /* m *= phase */
        double pr = phase_re[ph], pi = phase_im[ph];
        double ar = mr * pr - mi * pi;
        double ai = mr * pi + mi * pr;
        /* m *= sign * sqrt(n_j / n_i) */
        double f = sqrt((double)norms[j] / (double)norms[i]);
        if (sg < 0) f = -f;
        ME[2 * i] = ar * f;
        ME[2 * i + 1] = ai * f;
        row[i] = j;
    }
    orc_sym_free(&S);
    return err ? -1 : 0;
}

/*
 * Matrix-free apply (the reference's _core.inplace_op):
 *   v_out[j, :] += a * ME(i->j) * v_in[i, :]     (complex, interleaved)
 * for every ket i; transposed: v_out[i] += a * ME * v_in[j]; conjugated
 * conjugates ME.  nvec columns, C order.  Serial (deterministic).
 */
int orc_inplace_op(int N, int fermion, int nmaps, const int32_t *maps,
                   const int32_t *pers, const int32_t *qs,
                   const double *phase_re, const double *phase_im,
                   const char *opstr, const int32_t *indx, int nop,
                   double J_re, double J_im,
                   const uint64_t *basis, const uint32_t *norms, int64_t Ns,
                   int N_p, const int64_t *begin, const int64_t *end,
                   int transposed, int conjugated,
                   const double *v_in, double *v_out, int64_t nvec)
{
    int64_t *row = (int64_t *)malloc(sizeof(int64_t) * (Ns ? Ns : 1));
    int64_t *col = (int64_t *)malloc(sizeof(int64_t) * (Ns ? Ns : 1));
    double *ME = (double *)malloc(sizeof(double) * 2 * (Ns ? Ns : 1));
    int rc = orc_op(N, fermion, nmaps, maps, pers, qs, phase_re, phase_im, opstr, indx, nop,
                    J_re, J_im, basis, norms, Ns, N_p, begin, end, row, col, ME);
    if (rc == 0) {
        for (int64_t i = 0; i < Ns; i++) {
            double mr = ME[2 * i], mi = ME[2 * i + 1];
            if (mr == 0.0 && mi == 0.0) continue;
            if (conjugated) mi = -mi;
            int64_t dst = transposed ? col[i] : row[i];
            int64_t src = transposed ? row[i] : col[i];
            for (int64_t c = 0; c < nvec; c++) {
                double xr = v_in[2 * (src * nvec + c)], xi = v_in[2 * (src * nvec + c) + 1];
                v_out[2 * (dst * nvec + c)] += mr * xr - mi * xi;
                v_out[2 * (dst * nvec + c) + 1] += mr * xi + mi * xr;
            }
        }
    }
    free(row); free(col); free(ME);
    return rc;
}

/* ---------------------------------------------------------------------- */
/* canonical CSR assembly on the CPU                                      */
/*
 * Restates basis._make_matrix (src/quspin/basis/base.py:265-304) for the
 * terms of one operator list without scipy: the off-diagonal terms' entries
 * are bucketed by row, ordered by (column, term), summed left to right in
 * term order, the diagonal array (sum of the diagonal terms, in order) added
 * last and exact zeros dropped -- the arithmetic of the reference's chain of
 * scipy CSR additions.  Used where scipy's pairwise additions are too slow
 * (the CPU leg of the benchmark at 4.7M states).
 *
 * Terms: nop[t], off[t] into chr/site, J[2t..2t+1]; is_diag[t] marks the
 * diagonal terms.  real_out: 1 -> values are the real parts (float64 CSR).
 * Outputs are malloc'ed and returned through the pointers; free with
 * orc_free.  Returns nnz, or -1 (bad operator character) / -2.
 */
typedef struct { u64 key; double re, im; } orc_ent;

static int orc_ent_cmp(const void *a, const void *b)
{
    u64 x = ((const orc_ent *)a)->key, y = ((const orc_ent *)b)->key;
    return x < y ? -1 : (x > y ? 1 : 0);
}

void orc_free(void *p) { free(p); }

static inline int64_t orc_term_elem(const orc_sym *S, const double *phase_re, const double *phase_im,
                                    const char *chr, const int32_t *site, int nop, double Jr, double Ji,
                                    const uint64_t *basis, const uint32_t *norms, int64_t Ns, int N_p,
                                    const int64_t *begin, const int64_t *end, int64_t i,
                                    double *outr, double *outi, int *err)
{
    u64 s = basis[i], r = s;
    double mr = Jr, mi = Ji;
    int e = S->fermion ? orc_op_fermion(S->N, &r, &mr, &mi, nop, chr, site)
                       : orc_op_hcb(S->N, &r, &mr, &mi, nop, chr, site);
    *outr = 0.0; *outi = 0.0;
    if (e) { *err = 1; return -1; }
    if (mr == 0.0 && mi == 0.0) return -1;
    int sg = 1, ph = 0;
    int64_t j = i;
    if (r != s) {
        u64 rep = orc_ref_state(S, r, NULL, &sg, &ph);
        j = (rep == s) ? i : orc_index(S->N, N_p, basis, Ns, begin, end, rep);
    }
    if (j < 0) return -1;
    double pr = phase_re[ph], pi = phase_im[ph];
    double ar = mr * pr - mi * pi;
    double ai = mr * pi + mi * pr;
    double f = sqrt((double)norms[j] / (double)norms[i]);
    if (sg < 0) f = -f;
    *outr = ar * f; *outi = ai * f;
    return j;
}

int64_t orc_build_csr(int N, int fermion, int nmaps, const int32_t *maps, const int32_t *pers, const int32_t *qs,
                      const double *phase_re, const double *phase_im,
                      int T, const int32_t *nop, const int32_t *off, const char *chr, const int32_t *site,
                      const double *J, const int32_t *is_diag,
                      const uint64_t *basis, const uint32_t *norms, int64_t Ns, int N_p,
                      const int64_t *begin, const int64_t *end, int real_out,
                      int64_t **indptr_out, int32_t **indices_out, double **data_out)
{
    orc_sym S;
    if (orc_sym_init(&S, N, fermion, nmaps, maps, pers, qs)) { orc_sym_free(&S); return -2; }
    int err = 0;
    int has_diag = 0;
    for (int t = 0; t < T; t++) if (is_diag[t]) has_diag = 1;
    double *dre = (double *)calloc(Ns > 0 ? Ns : 1, sizeof(double));
    double *dim = (double *)calloc(Ns > 0 ? Ns : 1, sizeof(double));
    int64_t *cnt = (int64_t *)calloc(Ns + 1, sizeof(int64_t));
    /* pass 1: diagonal array and per-row counts (+1 slot per row for the
     * diagonal entry when there is a diagonal array) */
    #pragma omp parallel for schedule(dynamic, 4096) reduction(|:err)
    for (int64_t i = 0; i < Ns; i++) {
        int e = 0;
        for (int t = 0; t < T; t++) {
            double r, im;
            int64_t j = orc_term_elem(&S, phase_re, phase_im, chr + off[t], site + off[t], nop[t], J[2 * t],
                                      J[2 * t + 1], basis, norms, Ns, N_p, begin, end, i, &r, &im, &e);
            if (j < 0) continue;
            if (real_out) im = 0.0;
            if (r == 0.0 && im == 0.0) continue;
            if (is_diag[t]) { dre[i] += r; dim[i] += im; }
            else {
                #pragma omp atomic
                cnt[j + 1]++;
            }
        }
        err |= e;
    }
    if (err) { free(dre); free(dim); free(cnt); orc_sym_free(&S); return -1; }
    if (has_diag) for (int64_t i = 0; i < Ns; i++) cnt[i + 1]++;
    for (int64_t i = 0; i < Ns; i++) cnt[i + 1] += cnt[i];
    int64_t tot = cnt[Ns];
    orc_ent *ent = (orc_ent *)malloc(sizeof(orc_ent) * (tot > 0 ? tot : 1));
    int64_t *cur = (int64_t *)calloc(Ns > 0 ? Ns : 1, sizeof(int64_t));
    /* pass 2: scatter (column, term) keyed entries into their rows */
    #pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t i = 0; i < Ns; i++) {
        int e = 0;
        for (int t = 0; t < T; t++) {
            if (is_diag[t]) continue;
            double r, im;
            int64_t j = orc_term_elem(&S, phase_re, phase_im, chr + off[t], site + off[t], nop[t], J[2 * t],
                                      J[2 * t + 1], basis, norms, Ns, N_p, begin, end, i, &r, &im, &e);
            if (j < 0) continue;
            if (real_out) im = 0.0;
            if (r == 0.0 && im == 0.0) continue;
            int64_t slot;
            #pragma omp atomic capture
            slot = cur[j]++;
            orc_ent *p = &ent[cnt[j] + slot];
            p->key = ((u64)i << 22) | (u64)t;
            p->re = r; p->im = im;
        }
    }
    /* pass 3: per row sort, term-ordered sums, diagonal last, zero drop */
    int64_t *mc = (int64_t *)calloc(Ns + 1, sizeof(int64_t));
    #pragma omp parallel
    {
        int64_t cap = 256;
        orc_ent *tmp = (orc_ent *)malloc(sizeof(orc_ent) * cap);
        #pragma omp for schedule(dynamic, 1024)
        for (int64_t rrow = 0; rrow < Ns; rrow++) {
            orc_ent *p = ent + cnt[rrow];
            int64_t len = cur[rrow];
            if (len + 1 > cap) { cap = 2 * (len + 1); tmp = (orc_ent *)realloc(tmp, sizeof(orc_ent) * cap); }
            qsort(p, len, sizeof(orc_ent), orc_ent_cmp);
            int64_t out = 0, k = 0;
            int diag_done = !has_diag;
            while (k < len || !diag_done) {
                int64_t col = k < len ? (int64_t)(p[k].key >> 22) : INT64_MAX;
                if (!diag_done && rrow < col) {
                    if (dre[rrow] != 0.0 || dim[rrow] != 0.0) {
                        tmp[out].key = (u64)rrow; tmp[out].re = dre[rrow]; tmp[out].im = dim[rrow]; out++;
                    }
                    diag_done = 1;
                    continue;
                }
                double sr = p[k].re, si = p[k].im;
                int64_t kk = k + 1;
                while (kk < len && (int64_t)(p[kk].key >> 22) == col) { sr += p[kk].re; si += p[kk].im; kk++; }
                if (!diag_done && col == rrow) { sr += dre[rrow]; si += dim[rrow]; diag_done = 1; }
                if (sr != 0.0 || si != 0.0) { tmp[out].key = (u64)col; tmp[out].re = sr; tmp[out].im = si; out++; }
                k = kk;
            }
            memcpy(p, tmp, sizeof(orc_ent) * out);
            mc[rrow + 1] = out;
        }
        free(tmp);
    }
    for (int64_t i = 0; i < Ns; i++) mc[i + 1] += mc[i];
    int64_t nnz = mc[Ns];
    int64_t *indptr = (int64_t *)malloc(sizeof(int64_t) * (Ns + 1));
    int32_t *indices = (int32_t *)malloc(sizeof(int32_t) * (nnz > 0 ? nnz : 1));
    double *data = (double *)malloc(sizeof(double) * (real_out ? 1 : 2) * (nnz > 0 ? nnz : 1));
    memcpy(indptr, mc, sizeof(int64_t) * (Ns + 1));
    #pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t rrow = 0; rrow < Ns; rrow++) {
        const orc_ent *p = ent + cnt[rrow];
        for (int64_t k = 0; k < mc[rrow + 1] - mc[rrow]; k++) {
            int64_t o = mc[rrow] + k;
            indices[o] = (int32_t)p[k].key;
            if (real_out) data[o] = p[k].re;
            else { data[2 * o] = p[k].re; data[2 * o + 1] = p[k].im; }
        }
    }
    free(mc); free(cur); free(ent); free(cnt); free(dre); free(dim); orc_sym_free(&S);
    *indptr_out = indptr; *indices_out = indices; *data_out = data;
    return nnz;
}
