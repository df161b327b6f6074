/*
 * qsgpu.h -- C ABI of libqsgpu.so, the GB300 (sm_103a) hot path of QuSpin's
 * symmetry-reduced Hamiltonian apply, expm_multiply_parallel and Lanczos.
 *
 * All pointers named d_* or documented as "device" are CUDA device pointers
 * owned by the caller; `stream` is a cudaStream_t (NULL = legacy stream).
 * Every function returns 0 on success or a negative status:
 *   -1 invalid argument, -2 CUDA error, -3 unknown operator character,
 *   -4 complex element in a real dtype, -5 buffer too small,
 *   -6 unsupported configuration, -7 iteration cap reached.
 * Element type codes: 0 float32, 1 float64, 2 complex64, 3 complex128,
 * 4 real value as a float pair hi + lo (8 bytes), 5 complex value as two
 * float pairs {re.hi, re.lo, im.hi, im.lo} (16 bytes); as matrix values
 * only: 6 / 7 the values of 4 / 5 coded -- a table of 256 such values
 * followed by one uint8 code per nonzero (int32 column indices only).
 *
 * Each declaration names the reference interface it replaces (QuSpin 1.0.1;
 * paths relative to the reference project root; "html" = the Sphinx
 * viewcode copy of the un-vendored parallel-sparse-tools 0.2.5 wrappers,
 * docs/modules/parallel_sparse_tools/...).
 */
#ifndef QSGPU_H
#define QSGPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- symmetry context ------------------------------------------------
 * Replaces the construction of the native basis core
 * (hcb_basis_core_wrap / spinless_fermion_basis_core_wrap at
 * src/quspin/basis/basis_general/base_hcb.py:74-76 and fermion.py:178-180):
 * per-bit site maps (negative = inversion), periods, quantum numbers and the
 * phase tables exp(-2 pi i p / L), cos(2 pi p / L), L = lcm(periods). */
int qs_sym_create(int N, int fermion, int nmaps, const int32_t *maps, const int32_t *pers, const int32_t *qs,
                  const double *phase_re, const double *phase_im, const double *costab, int L, void **out);
int qs_sym_destroy(void *sym);

/* ---- prefix sums (device int64, in place) ------------------------------ */
int64_t qs_scan_scratch_elems(int64_t n);
int qs_scan_inclusive_i64(int64_t *x, int64_t n, int64_t *scratch, void *stream);

/* ---- basis enumeration: _core.make_basis (base_general.py:862-867) ------
 * kind 0: all 2^N words; 1: popcount == p0; 2: spinful, p0 ones in the high
 * N/2 bits and p1 in the low N/2 bits.  States come out sorted descending,
 * as the reference keeps them (base_general.py:875-885). */
int64_t qs_enum_num_candidates(int N, int kind, int p0, int p1);
int64_t qs_enum_num_chunks(int N, int kind, int p0, int p1);
int qs_enum_count(void *sym, int kind, int p0, int p1, int64_t *d_off, int64_t nchunks, int64_t *d_scratch,
                  int64_t *h_total, void *stream);
int qs_enum_write(void *sym, int kind, int p0, int p1, const int64_t *d_off, int64_t nchunks, void *d_states,
                  uint32_t *d_norms, void *stream);

/* ---- _core.make_basis_blocks (base_general.py:944-947) ------------------ */
int qs_make_blocks(int N, int state_bytes, int N_p, const void *d_states, int64_t Ns, int64_t *d_begin,
                   int64_t *d_end, void *stream);

/* ---- _get_basis_index (base_general.py:281-285) ------------------------- */
int qs_index(int N, int state_bytes, const void *d_states, int64_t Ns, int N_p, const int64_t *d_begin,
             const int64_t *d_end, const void *d_queries, int64_t nq, int64_t *d_out, void *stream);

/* ---- _core.representative (base_general.py:1085-1117) ------------------- */
int qs_representative(void *sym, const void *d_states, int64_t n, void *d_out, int32_t *d_g_out, int8_t *d_sign_out,
                      void *stream);

/* ---- _core.normalization (base_general.py:1158-1181) -------------------- */
int qs_normalization(void *sym, const void *d_states, int64_t n, uint32_t *d_out, void *stream);

/* ---- _core.op (base_general.py:324-336): one operator-string term -------
 * Term table (device): nop[t], off[t] into chr/site, J[2t..2t+1]. */
int qs_op(void *sym, const void *d_states, const uint32_t *d_norms, int64_t Ns, int N_p, const int64_t *d_begin,
          const int64_t *d_end, const int32_t *t_nop, const int32_t *t_off, const int8_t *t_chr,
          const int32_t *t_site, const double *t_J, int64_t *d_row, int64_t *d_col, double *d_ME, int *d_err,
          void *stream);

/* ---- canonical CSR assembly: basis._make_matrix (src/quspin/basis/base.py:265-304)
 * count -> inclusive scan -> fill -> merge -> inclusive scan -> compact. */
int qs_csr_count(void *sym, int vtype, const void *d_states, const uint32_t *d_norms, int64_t Ns, int N_p,
                 const int64_t *d_begin, const int64_t *d_end, const int32_t *t_nop, const int32_t *t_off,
                 const int8_t *t_chr, const int32_t *t_site, const double *t_J, int T, int64_t *d_rowcnt,
                 int *d_term_flags, int *d_err, void *stream);
int qs_csr_fill(void *sym, int vtype, const void *d_states, const uint32_t *d_norms, int64_t Ns, int N_p,
                const int64_t *d_begin, const int64_t *d_end, const int32_t *t_nop, const int32_t *t_off,
                const int8_t *t_chr, const int32_t *t_site, const double *t_J, int T, const int64_t *d_rowptr,
                int64_t *d_cursor, uint64_t *d_keys, void *d_vals, int *d_err, void *stream);
int qs_csr_diag(void *sym, int vtype, const void *d_states, const uint32_t *d_norms, int64_t Ns, int N_p,
                const int64_t *d_begin, const int64_t *d_end, const int32_t *t_nop, const int32_t *t_off,
                const int8_t *t_chr, const int32_t *t_site, const double *t_J, int T, void *d_diag,
                int *d_term_flags, int *d_err, void *stream);
int qs_csr_merge(int vtype, int64_t Ns, const int64_t *d_rowptr, const int64_t *d_fillcnt, uint64_t *d_keys,
                 void *d_vals, const void *d_diag, int64_t *d_mcount, int *d_err, void *stream);
int qs_csr_compact(int vtype, int64_t Ns, const int64_t *d_rowptr, const uint64_t *d_keys, const void *d_vals,
                   const int64_t *d_incl, void *d_indptr, int idx64, int32_t *d_indices, void *d_data,
                   void *stream);

/* ---- conjugate transpose A^H on the device: the rmatvec operand of the
 * onenormest products in ExpmMultiplyParallel's norm information
 * (html expm_multiply_parallel_core.html:436-449).  count -> scan -> fill ->
 * qs_csr_merge (no diagonal) -> scan -> qs_csr_compact. --------------------- */
int qs_csr_t_count(int64_t n, const void *d_indptr, int idx64, const int32_t *d_indices, int64_t *d_cnt, void *stream);
int qs_csr_t_fill(int vtype, int64_t n, const void *d_indptr, int idx64, const int32_t *d_indices, const void *d_data,
                  const int64_t *d_rowptr, int64_t *d_cursor, uint64_t *d_keys, void *d_vals, void *stream);

/* ---- _core.inplace_op (base_general.py:395-408): matrix-free apply ------ */
int qs_inplace_op(void *sym, const void *d_states, const uint32_t *d_norms, int64_t Ns, int N_p,
                  const int64_t *d_begin, const int64_t *d_end, const int32_t *t_nop, const int32_t *t_off,
                  const int8_t *t_chr, const int32_t *t_site, const double *t_J, int T, int transposed,
                  int conjugated, double a_re, double a_im, const void *d_vin, void *d_vout, int64_t nvec,
                  int *d_err, void *stream);

/* ---- basis.get_proj / project_from / project_to (base_general.py:521-718)
 * Projector columns (CSC): column i sums c_i chi(g) sigma(g) over the group
 * elements g reaching each image of representative i, c_i = 1/sqrt(n_i |G|),
 * rows ascending; images whose unit-phase sum is below 1e-12 are dropped.
 * mode 0 writes the entry count of column i to d_colptr[i + 1]; mode 1
 * (d_colptr now offsets) writes rows and complex128 values.  pcon = 0:
 * row = 2^N - 1 - state (N <= 62); pcon = 1: row = index in the
 * particle-conserving basis p_states..p_end.  d_err bits: 2 count mismatch,
 * 4 image outside the row basis.  |G| <= 8192. */
int qs_proj_fill(void *sym, const void *d_states, const uint32_t *d_norms, int64_t Ns, int gsize, int mode,
                 int64_t *d_colptr, int pcon, const void *d_p_states, int64_t p_Ns, int p_N_p,
                 const int64_t *d_p_begin, const int64_t *d_p_end, int64_t *d_rows, void *d_vals, int *d_err,
                 void *stream);
/* direction 0: y[Nfull, k] += P x (zero y first; sectors accumulate);
 * direction 1: y[Ns, k] = P^dagger x.  Complex128, C order. */
int qs_proj_apply(int direction, int64_t Ns, const int64_t *d_colptr, const int64_t *d_rows, const void *d_P,
                  const void *d_x, int64_t k, void *d_y, void *stream);

/* ---- _matvec for csr / dia (html matvec/matvec_core.html:146-201) ------- */
int qs_csr_matvec(int64_t n, int64_t nnz, const void *d_indptr, int idx64, const int32_t *d_indices,
                  const void *d_data, int dtype, const void *d_x, int xtype, void *d_y, int64_t nvec, double a_re,
                  double a_im, int overwrite, int group, void *stream);
/* Paired-single form of qs_csr_matvec for float64 / complex128 x and y: the
 * values split by qs_split_pairs (pdtype 4 / 5), coded (6 / 7: a table of
 * 256 pairs, then one code byte per nonzero) or packed (8 / 9: d_indices
 * holds col << 8 | code with col < 2^23, d_pdata the table only), x scaled
 * by a power of two and split into d_xs (n*nvec*8 or 16 bytes of scratch;
 * d_norm: 8 bytes), products and row sums in FP32 instructions with 48-bit
 * significands. */
int qs_csr_matvec_pairs(int64_t n, int64_t nnz, const void *d_indptr, int idx64, const int32_t *d_indices,
                        const void *d_pdata, int pdtype, const void *d_x, int xtype, void *d_y, int64_t nvec,
                        double a_re, double a_im, int overwrite, int group, void *d_xs, void *d_norm, void *stream);
int qs_dia_matvec(int64_t n, int ndiag, const int64_t *d_offsets, int64_t ldd, const void *d_data, int dtype,
                  const void *d_x, int xtype, void *d_y, int64_t nvec, double a_re, double a_im, int overwrite,
                  void *stream);

/* ---- reductions: numpy vdot / norm of the Lanczos recurrence
 * (src/quspin/tools/lanczos/_lanczos_utils.py:180-204) ------------------ */
int qs_reduce_scratch_doubles(void);
int qs_vdot(int64_t n, const void *d_x, const void *d_y, int cplx, double *d_out, double *d_scratch, void *stream);
int qs_nrm2(int64_t n2, const void *d_x, double *d_out, double *d_scratch, void *stream);

/* ---- _wrapper_csr_trace / _wrapper_csr_1_norm
 * (html expm_multiply_parallel_core.html:196-202) ---------------------- */
int qs_csr_trace(int64_t n, const void *d_indptr, int idx64, const int32_t *d_indices, const void *d_data, int cplx,
                 double *d_out, double *d_scratch, void *stream);
int qs_csr_1_norm(int64_t n, const void *d_indptr, int idx64, const int32_t *d_indices, const void *d_data, int cplx,
                  double sh_re, double sh_im, double *d_out, double *d_colsum, double *d_scratch, void *stream);

/* ---- _wrapper_expm_multiply / _wrapper_expm_multiply_batch
 * (html expm_multiply_parallel_core.html:347-372) ----------------------- */
int qs_expm_ctl_bytes(void);
/* Taylor-term storage (btype): 3 = complex128 with IEEE double products;
 * 5 = float pairs with FP32-instruction products (values from qs_split_pairs,
 * dtype 4 / 5, or coded / packed, dtype 6..9); 2 = complex64 with float32 /
 * complex64 values.  F, the shift, the coefficients and the stopping test
 * are double in all three.  group (0: defaults) is a launch code: bits 0-7
 * lanes per row, 8-15 entries in flight, 18-19 a register cap, 20-22 the
 * single-vector kernel (1..3 32-row, 4..5 row hand-out, 6..7 row hand-out
 * reading packed column words four per 16-byte load: dtype 8 / 9 only, with
 * d_indices readable up to the next multiple of four words). */
int qs_split_pairs(int64_t count, const double *d_src, void *d_dst, void *stream);
/* The truncated pair of d_src[i] 2^-k (hi: top 24 significant bits, lo: the
 * rest truncated likewise; zero below the normal float range), the split
 * the many-vector stopping tests use for their moduli. */
int qs_split_pairs_trunc(int64_t count, const double *d_src, int k, void *d_dst, void *stream);
int qs_taylor_term(int64_t n, int64_t nnz, const void *d_indptr, int idx64, const int32_t *d_indices,
                   const void *d_data, int dtype, const void *d_Bin, void *d_Bout, int btype, void *d_F,
                   int64_t nvec, double mu_re, double mu_im, const void *d_coeff, int j, double tol, void *d_ctl,
                   int group, void *stream);
int qs_taylor_rescale(int64_t n, int64_t nvec, void *d_F, void *d_B0, int btype, const void *d_eta, void *d_ctl,
                      int substep_end, void *stream);
int qs_expm_multiply(int64_t n, int64_t nnz, const void *d_indptr, int idx64, const int32_t *d_indices,
                     const void *d_data, int dtype, void *d_F, int64_t nvec, int s, int m_star, double tol,
                     double mu_re, double mu_im, const void *d_coeff, const void *d_eta, const void *d_one,
                     void *d_work, int btype, void *d_ctl, int group, void *stream);
/* The same two calls with a row-sum scratch d_rownorm of n double pairs (16n bytes): with bit 16 of group set and
 * more than 8 right-hand sides, the float forms sweep the rows once per chunk of 8 vectors, so the gathered
 * slice of B stays in L2 (the many-state evolutions of hamiltonian_core.py:1472-1486 and block_tools.py:618-795
 * call the Taylor loop with such blocks). */
int qs_taylor_term_rows(int64_t n, int64_t nnz, const void *d_indptr, int idx64, const int32_t *d_indices,
                        const void *d_data, int dtype, const void *d_Bin, void *d_Bout, int btype, void *d_F,
                        int64_t nvec, double mu_re, double mu_im, const void *d_coeff, int j, double tol, void *d_ctl,
                        int group, void *d_rownorm, void *stream);
int qs_expm_multiply_rows(int64_t n, int64_t nnz, const void *d_indptr, int idx64, const int32_t *d_indices,
                          const void *d_data, int dtype, void *d_F, int64_t nvec, int s, int m_star, double tol,
                          double mu_re, double mu_im, const void *d_coeff, const void *d_eta, const void *d_one,
                          void *d_work, int btype, void *d_ctl, int group, void *d_rownorm, void *stream);

/* ---- Runge-Kutta stage arithmetic of hamiltonian.evolve: replaces the
 * state updates of scipy's DOP853 that the reference drives through
 * src/quspin/tools/evolution.py:300-345 (hamiltonian_core.py:1489-1630 builds
 * the right-hand side).  The state is viewed as n2 real components; K holds
 * nk stage derivatives of n2 doubles; coefficient arrays are host memory. --- */
int qs_rk_error_scratch_doubles(int64_t n2);
int qs_rk_combine(int64_t n2, const double *d_y, const double *d_K, int nk, const double *c_host, double h,
                  double *d_out, void *stream);
int qs_rk_error(int64_t n2, const double *d_y0, const double *d_y1, const double *d_K, int nk,
                const double *e5_host, const double *e3_host, double atol, double rtol, double *d_scratch,
                double *d_out, void *stream);
/* Liouville right-hand side helper (hamiltonian_core.py:1394-1420): out = alpha X^dagger or out += alpha
 * X^dagger for complex128 n x n matrices (C order; out must not alias X). */
int qs_adjoint_axpy(int64_t n, const void *d_X, void *d_out, double alpha_re, double alpha_im, int accumulate,
                    void *stream);

/* ---- many sectors in one launch: block-diagonal stack of sector matrices,
 * per-sector shift / factor / stopping test, common (s, m*) schedule.  The
 * reference fans sectors out to processes (src/quspin/tools/block_tools.py:
 * 135-220, 618-795); this replaces that fan-out for the expm path. ------ */
int qs_multi_ctl_bytes(void);
int qs_max_sectors(void);
int qs_taylor_multi_term(int64_t n, const void *d_indptr, const int32_t *d_indices, const void *d_data, int dtype,
                         const void *d_Bin, void *d_Bout, int btype, void *d_F, int64_t nvec, const int64_t *d_sec_off,
                         const void *d_mu, const void *d_coeff, int j, double tol, void *d_ctl, int group,
                         void *stream);
int qs_taylor_multi_term_rows(int64_t n, const void *d_indptr, const int32_t *d_indices, const void *d_data, int dtype,
                              const void *d_Bin, void *d_Bout, int btype, void *d_F, int64_t nvec,
                              const int64_t *d_sec_off, const void *d_mu, const void *d_coeff, int j, double tol,
                              void *d_ctl, int group, void *d_rownorm, void *stream);
int qs_taylor_multi_rescale(int64_t n, int64_t nvec, void *d_F, void *d_B0, int btype, const int64_t *d_sec_off,
                            const void *d_eta, int use_eta, void *d_ctl, void *stream);

/* ---- dense layers of the learned (m*, s) predictor (no counterpart in
 * the reference, whose selection is scipy's onenormest-based fragment 3.1,
 * html expm_multiply_parallel_core.html:377-463): y = act(x W^T + b) with
 * bfloat16 weights and FP32 accumulation, the matching backward products, a
 * weighted mean-squared-error gradient and an Adam update. ----------------- */
int qs_mlp_dense_fwd(int B, int din, int dout, const float *d_x, const void *d_w_bf16, const float *d_bias,
                     float *d_z, float *d_y, int relu, void *stream);
int qs_mlp_dense_bwd(int B, int din, int dout, const float *d_dy, const void *d_w_bf16, const float *d_x,
                     const float *d_zin, float *d_dx, float *d_gw, float *d_gb, void *stream);
int qs_mlp_mse(int64_t total, int dout, const float *d_y, const float *d_target, const float *d_colw, float scale,
               float *d_dy, float *d_partial, int nblocks, void *stream);
int qs_mlp_adam(int64_t n, float *d_w, const float *d_g, float *d_m, float *d_v, void *d_w_bf16, float lr, float b1,
                float b2, float eps, int step, void *stream);
int qs_mlp_to_bf16(int64_t n, const float *d_w, void *d_w_bf16, void *stream);

/* ---- e^{aA} v without any device allocation.  No counterpart in the
 * reference: this entry point exists for callers that cannot allocate GPU
 * memory (a host application or plugin framework that owns the device memory
 * budget, or a time-stepping loop that must not synchronise on cudaMalloc).
 * Same arithmetic as qs_expm_multiply with complex128 Taylor buffers; its
 * scratch is a static device array in the library (about 32 MiB per GPU, kept
 * until exit).  Limits: n * nvec <= qs_expm_noalloc_max_elems() (1,048,576)
 * and m_star <= 64, else -5.  The first call on a device looks up the array's
 * device address; make it before capturing work.  Calls that overlap on the
 * GPU share the scratch and race; serialise them. ------------------------- */
int64_t qs_expm_noalloc_max_elems(void);
int qs_expm_multiply_noalloc(int64_t n, int64_t nnz, const void *d_indptr, int idx64, const int32_t *d_indices,
                             const void *d_data, int dtype, void *d_F, int64_t nvec, int s, int m_star, double tol,
                             double mu_re, double mu_im, double a_re, double a_im, int group, void *stream);

/* ---- Lanczos recurrence steps: lanczos_full / lanczos_iter
 * (src/quspin/tools/lanczos/_lanczos_utils.py:158-204, :283-311), the
 * optional full reorthogonalisation, and lin_comb_Q_T (:366-425).  Vectors
 * are float64 or complex128 (cplx); n2 counts doubles (2n if complex). --- */
int qs_lanczos_ctl_bytes(void);
int qs_lanczos_scratch_doubles(void);
int64_t qs_lanczos_reorth_scratch_doubles(int nk);
int qs_lanczos_scale(int64_t n2, const double *d_r, const double *d_b, double *d_q, const void *d_ctl, void *stream);
int qs_lanczos_alpha(int64_t n, int cplx, double *d_r, const double *d_v, const double *d_b, const double *d_q,
                     double *d_a_out, double *d_scratch, void *d_ctl, void *stream);
int qs_lanczos_beta(int64_t n2, double *d_r, const double *d_a, const double *d_q, int do_axpy, double *d_b_out,
                    double eps, int i, double *d_scratch, void *d_ctl, void *stream);
/* Classical Gram-Schmidt against the rows Q[0..nk-1] (row stride ldq in
 * elements), `passes` times; the adaptive form runs a further pass only
 * while a pass removes more than 1 - 1/sqrt(2) of the norm of r (at most
 * max_passes), decided on the device.  d_scratch: at least
 * qs_lanczos_reorth_scratch_doubles(nk) doubles. */
int qs_lanczos_reorth(int64_t n, int cplx, int nk, const double *d_Q, int64_t ldq, double *d_r, int passes,
                      double *d_scratch, void *d_ctl, void *stream);
int qs_lanczos_reorth_adaptive(int64_t n, int cplx, int nk, const double *d_Q, int64_t ldq, double *d_r,
                               int max_passes, double *d_scratch, void *d_ctl, void *stream);
int qs_lanczos_lincomb(int64_t n_el, int nk, const double *d_c, int cplx_c, const double *d_Q, int64_t ldq,
                       int cplx_q, double *d_out, void *stream);

/* ---- dense FP64 panels of the Lanczos tools: W[i, j] = sum_r op(Q[i, r]) X[r, j]
 * (the Krylov matrix elements of _LTLM.py:110-126, the overlaps of _FTLM.py:95-105 and
 * full_ortho's re-projection, _lanczos_utils.py:206-222; the reference computes them with
 * numpy dot products).  Q [m, >= n] rows (stride ldq), X [n, >= k] C order (stride ldx) or,
 * with xrows, [k, >= n] rows; W [m, k]; cplx: complex128 interleaved; conj: op = complex
 * conjugate.  FP64 FMAs on 32 x 32 tiles staged through shared memory (k > 2) or per
 * output element (k <= 2); the _dmma form uses FP64 tensor instructions (mma.sync m8n8k4
 * .f64) for k > 2, which on GB300 run on the same FP64 pipe no faster.  The contraction is split over
 * n and the partial tiles summed in a fixed order (scratch from
 * qs_block_inner_scratch_doubles, the same for both forms). -------------------------- */
int64_t qs_block_inner_scratch_doubles(int64_t n, int m, int k, int cplx);
int qs_block_inner(int64_t n, int m, int k, const double *d_Q, int64_t ldq, const double *d_X, int64_t ldx,
                   int xrows, int cplx, int conj, double *d_W, double *d_scratch, void *stream);
int qs_block_inner_dmma(int64_t n, int m, int k, const double *d_Q, int64_t ldq, const double *d_X, int64_t ldx,
                        int xrows, int cplx, int conj, double *d_W, double *d_scratch, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* QSGPU_H */
