/*
 * bsg.h -- C ABI of libbsg.so, the GB300 (sm_103a) MPS-construction path for
 * lossy Gaussian boson sampling.  Drop-in for the per-cut truncation
 * (kron_cpu.py) and the per-site Gamma/Lambda build (MPS_cpu.py) of
 * sss441803/BosonSupremacy, plus the transfer contraction that consumes
 * Gamma/Lambda (sampling_cpu.py:75-90).
 *
 * Conventions
 *  - Every entry point returns 0 on success and a negative BSG_ERR_* code on
 *    failure; bsg_last_error() returns a message for the calling thread.
 *  - Pointers are DEVICE pointers unless the parameter name ends in _host.
 *    The caller owns every buffer it passes; the library never frees them.
 *  - Complex numbers are interleaved (re, im) pairs: "c128" = 2 doubles,
 *    "c64" = 2 floats.  Matrices are row-major (C order), as numpy saves them.
 *  - Work space (plans, partition programs, per-warp scratch) lives in the
 *    handle.  One handle per stream; a handle is not re-entrant.
 *  - Every kernel is launched on the given stream.  Entry points that must
 *    plan on the host (they read small arrays back) synchronise that stream;
 *    this is stated per function.
 *  - Spin-free: no kernel waits on a flag written by another block.
 */
#ifndef BSG_H_
#define BSG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bsg_handle_s* bsg_handle_t;
typedef struct CUstream_st* bsg_stream_t; /* == cudaStream_t */

/* status codes */
#define BSG_OK 0
#define BSG_ERR_INVALID (-1)     /* bad argument (shape, pointer, range)      */
#define BSG_ERR_CUDA (-2)        /* a CUDA runtime call failed                 */
#define BSG_ERR_NOT_PD (-3)      /* covariance not symmetric positive definite */
#define BSG_ERR_NO_CONVERGE (-4) /* an iterative factorisation hit its limit   */
#define BSG_ERR_LIMIT (-5)       /* a size exceeds a documented maximum        */
#define BSG_ERR_ALLOC (-6)       /* device or host allocation failed           */

/* arithmetic of the hafnian evaluation */
#define BSG_PREC_FP64 0  /* complex128 throughout (plain FP64 path)                      */
#define BSG_PREC_SPLIT 1 /* split: FP32 products with exact error terms, sums kept as    */
                         /* FP32 pairs (~48-bit significand) -- FP32 pipe, FP64-class     */
#define BSG_PREC_FP32 2  /* complex64 throughout (the reference's own working precision)  */
#define BSG_PREC_SLICED 3 /* contraction only: FP64 operands cut into fixed-point BF16     */
                          /* slices, tcgen05 products with exact FP32 accumulation per    */
                          /* slice level, FP64 results (complex128 Gamma in)              */

/* site kinds (MPS_cpu.py:402, 430, 461) */
#define BSG_SITE_FIRST 0
#define BSG_SITE_MIDDLE 1
#define BSG_SITE_LAST 2

/* output element type of Gamma */
#define BSG_OUT_C64 0  /* complex64, the reference's Gamma_i.npy dtype (MPS_cpu.py:397) */
#define BSG_OUT_C128 1 /* complex128 (FP64-promoted layout)                             */

/* documented limits */
#define BSG_MAX_CLASSES 24     /* distinct Sigma indices in one hafnian            */
#define BSG_MAX_ORDER 63       /* hafnian order n                                   */
#define BSG_MAX_STATES 65536   /* states of one partition program                   */
#define BSG_MAX_LABEL_NNZ 32   /* non-zero Fock entries in one Schmidt label row    */
#define BSG_MAX_DD 16          /* sampler Fock cutoff after displacement (dd)       */

/* ---- handle ------------------------------------------------------------ */
/* No reference counterpart (the reference keeps module-level CuPy state,
 * MPS_utils.py:13-19). */
int bsg_create(int device, bsg_handle_t* out);
int bsg_destroy(bsg_handle_t h);
const char* bsg_last_error(void);
int bsg_version(void);

/* ---- batched hafnian / A_elem seam -------------------------------------
 * Replaces A_elem + Sigma_select + hafnian (MPS_cpu.py:19-37, 117-187,
 * 334-355; GPU twin MPS_utils.py:21-47, 127-197, 273-297;
 * direct_mps_kernels.cu:3-39).
 *   out[b] = haf(Sigma[t_b][:, t_b]) / denominator[b]
 * Sigma: c128 [n_len, n_len] symmetric; targets: int32 [B, n] (indices may
 * repeat, as the reference's targets do); denominator: float64 [B] or NULL
 * (= 1); out: c128 [B].  Odd n gives 0, n = 0 gives 1/denominator.
 * Synchronises `stream` (plans the partition programs on the host). */
int bsg_hafnian_batched(bsg_handle_t h, const double* Sigma, int n_len, const int32_t* targets, int n,
                        int64_t B, const double* denominator, int precision, double* out,
                        bsg_stream_t stream);

/* Same, taking explicit matrices: A c128 [B, n, n] (the reference's
 * hafnian(A) input, MPS_cpu.py:117).  Synchronises `stream`. */
int bsg_hafnian_matrices(bsg_handle_t h, const double* A, int n, int64_t B, int precision, double* out,
                         bsg_stream_t stream);

/* ---- Sigma of a site ------------------------------------------------------
 * Replaces get_U2_sq_U1 + blochmessiah + get_Sigma (MPS_cpu.py:189-229,
 * 305-312, 357-372).  With S = (1 (+) S_l)^{-1} S_r (xxpp, 2M_r x 2M_r) and
 * its complex form [[A, B], [conj B, conj A]], Sigma = [[B X, X^T], [X, -X conj B]]
 * with X = conj(A)^{-1}, and Z = sqrt|det A| -- the same matrix the
 * reference reaches through Bloch-Messiah, without the SVDs.
 * S_l: float64 [2 m_l, 2 m_l] with m_l = M_r - 1 (ignored when m_l == 0, the
 * last site); S_r: float64 [2 M_r, 2 M_r]; Sigma: c128 [2 M_r, 2 M_r];
 * Z: float64 [1].  Asynchronous: a singular A (impossible for a symplectic
 * S, whose A satisfies A A^dag = I + B B^dag) is not reported by this call;
 * bsg_build_mps checks it on its own status words. */
int bsg_site_sigma(bsg_handle_t h, const double* S_l, int m_l, const double* S_r, int M_r, double* Sigma,
                   double* Z, bsg_stream_t stream);

/* Allocation-free variant of bsg_site_sigma (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc: code running while
 * another allocator has reserved the device's memory, latency-critical loops
 * that must not pay cudaMalloc/cudaFree's implicit device synchronisation,
 * and plug-in hosts that forbid raw device allocation.  It needs no handle
 * and allocates nothing: its scratch is a fixed ~2.75 MiB device array inside
 * libbsg.so (held on every GPU that loads the library until exit), so
 * M_r <= 160; larger M_r returns BSG_ERR_LIMIT.  The first call on a device
 * looks up that array's device address (make it before any stream capture).
 * Every call shares the array: calls that overlap on the GPU race, so issue
 * them on one stream or serialise them.  The array's address is kept per
 * device, so a cudaDeviceReset of that device ends its use in this process.
 * Same arguments and results as bsg_site_sigma.  Asynchronous. */
int bsg_site_sigma_noalloc(const double* S_l, int m_l, const double* S_r, int M_r, double* Sigma, double* Z,
                           bsg_stream_t stream);

/* Site 0 from the pure covariance itself (MPS_cpu.py:395, 409-414): the
 * output-output block of Sigma for V' = (1 (+) S_0^{-1}) sq_cov (1 (+) S_0^{-1})^T,
 * Sigma11 = Mc (conj(Nc) + I)^{-1} with [[Nc, Mc], ...] = R V' R^dag, and
 * Z = det((Nc + I)/2)^{1/4}.  Only Sigma[:M, :M] is written (the other blocks
 * are zero): site 0 has no input labels.  Asynchronous. */
int bsg_first_sigma(bsg_handle_t h, const double* S_0, int M, const double* sq_cov, double* Sigma, double* Z,
                    bsg_stream_t stream);

/* ---- Gamma of a site -------------------------------------------------------
 * Replaces the site loop body of MPS_cpu.py:402-520 (GPU twin
 * distributed_MPS.py:88-258):
 *   Gamma[a, b, j] = haf(Sigma[T(j, b, a)]) / (sqrt(j!) sqrt(prod num_l[b]!)
 *                     sqrt(prod num_r[a]!)) / Z / lambda_l[b]
 * with T = j copies of index 0, mode q of label num_l[b] at index 1 + q, mode
 * q of label num_r[a] at index M_r + q.  Every even-order (a, b, j) of the
 * bond grid is one work item of the site's DP launches; items are bucketed by
 * the multiplicity partition of T so that a warp runs one program.
 *   kind FIRST : num_r ignored (one empty right label), Gamma[0, b, j]
 *   kind MIDDLE: Gamma[a, b, j]
 *   kind LAST  : num_l ignored (one empty left label), lambda_l ignored, Gamma[a, 0, j]
 * num_l: int8 [k_l, m_l] (cut `site`, rows with res > err_tol only);
 * num_r: int8 [k_r, m_r] (cut `site-1`, all rows); lambda_l: float64 [k_l];
 * Z: float64 [1] (device); Gamma: [chi, chi, d] of out_dtype, fully written
 * (zeros outside the computed grid).  Synchronises `stream` once (reads the
 * label partition keys back to plan). */
int bsg_build_site(bsg_handle_t h, int kind, const double* Sigma, int M_r, const int8_t* num_l, int k_l, int m_l,
                   const double* lambda_l, const int8_t* num_r, int k_r, int m_r, const double* Z, int d, int chi,
                   int precision, int out_dtype, void* Gamma, bsg_stream_t stream);

/* ---- per-cut spectra (truncation to chi) ---------------------------------
 * Replaces williamson + get_cumsum_kron (kron_cpu.py:46-127; CuPy twin
 * distributed_kron.py:105-137) for cuts L = L0 .. L0+n_cuts-1 at once.
 * For each cut: symplectic eigenvalues nu and a Williamson symplectic S of
 * the sub-covariance of modes L..M-1 (FP64 Cholesky + Jacobi), thermal
 * occupations nbar = max(0, (nu-1)/2), then the chi largest products of
 * the per-mode geometric distributions truncated at d photons with weights
 * > err_tol, in descending order, with their Fock labels.
 * sq_cov: float64 [2M, 2M]; res: float64 [n_cuts, chi] (zero padded);
 * num: int8 [n_cuts, chi, M-1] (cut c uses the first M-1-L columns);
 * S: float64 [n_cuts, 2(M-1), 2(M-1)] (cut c uses the leading 2(M-L) block);
 * kept: int32 [n_cuts].  Asynchronous. */
int bsg_cut_spectra(bsg_handle_t h, const double* sq_cov, int M, int L0, int n_cuts, int d, int chi, double err_tol,
                    double* res, int8_t* num, double* S, int32_t* kept, bsg_stream_t stream);

/* One cut L, the per-cut form of kron_cpu.py's loop body (kron_cpu.py:147-153,
 * get_cumsum_kron(nbar, d, max_dim, err_tol) at kron_cpu.py:92-127): res
 * float64 [chi], num int8 [chi, M-1], S float64 [2(M-1), 2(M-1)] (leading
 * 2(M-L) block), *kept.  max_dim is the reference's per-step candidate cap
 * (1e5 there); keeping the top chi products per step selects the same final
 * set whenever max_dim >= chi, so a smaller max_dim is rejected.  Same as
 * bsg_cut_spectra with L0 = L, n_cuts = 1. */
int bsg_cut_spectrum(bsg_handle_t h, const double* sq_cov, int M, int L, int d, int chi, double err_tol,
                     int64_t max_dim, double* res, int8_t* num, double* S, int32_t* kept, bsg_stream_t stream);

/* ---- the whole MPS ---------------------------------------------------------
 * kron_cpu.py (all M-1 cuts, kron_cpu.py:147-153) followed by MPS_cpu.py
 * (all M sites, MPS_cpu.py:384-525) in one call, device-resident:
 * cut spectra with err_tol = cut_tol (the reference's 1e-12), Lambda_c =
 * sqrt(res_c) where res_c > site_tol (the reference's 1e-10) else 0.  The
 * cuts and sites run in three groups (right edge, left edge, middle) on
 * internal streams: per group Williamson, top-chi, label tables, Sigma, then
 * host planning of its items and its DP launches; the groups overlap (no
 * kernel waits on another).  gammas_host: host array of M device pointers to
 * [chi, chi, d] of out_dtype; Lambdas: float64 [M-1, chi]; res, num, S, kept
 * as bsg_cut_spectra with L0 = 1, n_cuts = M-1.  Waits on the host for each
 * group's label keys and synchronises `stream` at the end. */
int bsg_build_mps(bsg_handle_t h, const double* sq_cov, int M, int d, int chi, double cut_tol, double site_tol,
                  int precision, int out_dtype, void* const* gammas_host, double* Lambdas, double* res, int8_t* num,
                  double* S, int32_t* kept, bsg_stream_t stream);

/* The whole MPS of n independent instances, each with its own M[i], d[i] and
 * chi[i] (the reference builds one state per run; its MPI driver spreads
 * hafnian batches over idle ranks, distributed_MPS.py:214-240, and A_elem
 * chunks them, MPS_cpu.py:339-354).  One launch per phase for all instances:
 * the Williamson and top-chi kernels over every cut of every instance, the
 * Sigma construction over every site of every instance, one host wait for
 * the label keys, then one item scatter and one set of hafnian DP launches
 * over the items of every site of every instance (work items of all
 * instances bucketed together by partition program).  Results equal
 * bsg_build_mps of each instance bit for bit.  sq_covs, M, d, chi, Lambdas,
 * res, num, S, kept: host arrays of n (per-instance buffers as in
 * bsg_build_mps); gammas: host array of sum(M) device pointers, instance 0's
 * sites first.  Synchronises `stream`. */
int bsg_build_mps_batch(bsg_handle_t h, int n, const double* const* sq_covs, const int* M, const int* d,
                        const int* chi, double cut_tol, double site_tol, int precision, int out_dtype,
                        void* const* gammas, double* const* Lambdas, double* const* res, int8_t* const* num,
                        double* const* S, int32_t* const* kept, bsg_stream_t stream);

/* Sites [s0, s1) of one MPS from given cut data -- the kron step's res_i /
 * num_i / S_i files, as MPS_cpu.py reads them (MPS_cpu.py:384-525 restricted
 * to a site range, the per-rank range of distributed_MPS.py:72) -- in one
 * pipelined call: Lambda and label tables of the cuts the sites read
 * (cuts max(0, s0 - 1) .. min(s1, M - 1) - 1), the Sigma of every site in
 * one set of launches, one host wait, one item scatter and one set of DP
 * launches.  res [M-1, chi] float64, num [M-1, chi, M-1] int8, S
 * [M-1, 2(M-1), 2(M-1)] float64 and kept [M-1] int32 are device inputs laid
 * out as bsg_cut_spectra writes them (only the rows of the cuts read need to
 * be filled); gammas: host array of s1 - s0 device pointers; Lambdas
 * [M-1, chi] float64 (rows of the cuts read are written).  Synchronises
 * `stream`. */
int bsg_build_sites(bsg_handle_t h, const double* sq_cov, int M, int d, int chi, double site_tol, int precision,
                    int out_dtype, int s0, int s1, const double* res, const int8_t* num, const double* S,
                    const int32_t* kept, void* const* gammas, double* Lambdas, bsg_stream_t stream);

/* bsg_build_mps plus the download of its outputs: each group's DP runs in four
 * site parts and each part's Gammas are copied from gammas_dev[i] (device) to
 * gammas_pinned[i] (pinned host) as soon as that part is done, overlapping the
 * copies with the rest of the build, and the Lambdas to lambdas_pinned
 * [M-1, chi] float64.  Returns after every copy has landed. */
int bsg_build_mps_to_host(bsg_handle_t h, const double* sq_cov, int M, int d, int chi, double cut_tol,
                          double site_tol, int precision, int out_dtype, void* const* gammas_dev,
                          void* const* gammas_pinned, double* Lambdas, double* lambdas_pinned, double* res,
                          int8_t* num, double* S, int32_t* kept, bsg_stream_t stream);

/* ---- transfer contraction (pattern amplitudes) ---------------------------
 * The bond contraction that consumes Gamma/Lambda (sampling_cpu.py:75-90):
 * amp[p] = (... ((Gamma_0[0, :, n_0] * Lambda_0) @ Gamma_1[:, :, n_1]) * Lambda_1 ...) @ Gamma_{M-1}[:, 0, n_{M-1}]
 * for P photon patterns (int32 [P, M], device).  Gammas: HOST array of M
 * device pointers to [chi, chi, d] -- c128 for BSG_PREC_FP64, c64 otherwise;
 * Lambdas: float64 [M-1, chi]; amp: c128 [P].  Patterns are contracted
 * meet-in-the-middle: left environments of every distinct prefix up to site
 * (M-1)/2, right environments of every distinct suffix, one dot per pattern;
 * every (level, photon number) group is one batched complex GEMM.
 * precision: BSG_PREC_FP64 (FP64 CUDA cores), BSG_PREC_FP32 (FP32 CUDA cores),
 * BSG_PREC_SPLIT (3-way split TF32 products on the tcgen05 tensor cores,
 * FP32 accumulation; complex64 Gamma, ~1e-4 relative in the probabilities)
 * or BSG_PREC_SLICED (complex128 Gamma and FP64 environments, every level's
 * GEMM as fixed-point BF16 slice products on the tcgen05 tensor cores with
 * exact FP32 accumulation, see bsg_gemm_sliced; needs chi % 4 == 0).
 * Synchronises `stream`: the prefix tries are planned on the GPU, and the
 * host reads each level's row counts to size its GEMM launches. */
int bsg_pattern_amplitudes(bsg_handle_t h, const void* const* Gammas, const double* Lambdas, int M, int chi, int d,
                           const int32_t* patterns, int64_t P, int precision, double* amp, bsg_stream_t stream);

/* The same contraction under the name the reference-side bindings use for
 * the pattern-probability consumer (sampling_cpu.py:75-81): identical
 * arguments and results to bsg_pattern_amplitudes. */
int bsg_contract_patterns(bsg_handle_t h, const void* const* Gammas, const double* Lambdas, int M, int chi, int d,
                          const int32_t* patterns, int64_t P, int precision, double* amp, bsg_stream_t stream);

/* FP64 GEMM from BF16 tensor-core products (no counterpart in the reference;
 * the primitive of BSG_PREC_SLICED): C[M, N] = A[M, K] B[N, K]^T, all three
 * row-major float64 on the device.  Every row of A and of B is scaled by a
 * power of two and cut into S fixed-point slices of b bits (b such that
 * 3 K 2^(2b) < 2^23, S = ceil(42 / b)); the slice products of each level
 * s + t <= 2 sum exactly in FP32 in TMEM, the rest below 2^-40 of the
 * result, so C carries ~42 bits of each row's scale.  0 < K <= 32768,
 * K % 8 == 0.  Synchronises `stream`. */
int bsg_gemm_sliced(bsg_handle_t h, const double* A, const double* B, double* C, int M, int N, int K,
                    bsg_stream_t stream);

/* ---- sampling ------------------------------------------------------------
 * Photon-number samples of the lossy state from the MPS, replacing
 * sampling_cpu.py:30-117 (`sampling`; GPU twin distributed_sampling.py:62-155):
 * a random displacement per sample from the thermal part, then sequential
 * inverse-CDF sampling along the chain.  The random numbers are inputs, in
 * the reference's draw order, so a seeded numpy stream reproduces the
 * reference's samples:
 *   normals  float64 [2M, n] (np.random.normal(size=(2M, n)), sampling_cpu.py:37)
 *   uniforms float64 [M, n]  (row i = np.random.rand(n, 1) of site i, :52, :92)
 * sqrtW: float64 [2M, 2M] row-major, the Cholesky factor of the thermal
 * covariance (sampling_cpu.py:168-170).  Gammas: HOST array of M device
 * pointers to [chi, chi, d] (c128 for BSG_PREC_FP64, c64 otherwise);
 * Lambdas float64 [M-1, chi].  samples: int64 [n, M] (the reference's
 * `results`).  d <= dd <= BSG_MAX_DD.  precision: the chain GEMM
 * (pre * Lambda) @ Gamma_i.reshape(chi, chi d) in FP64 or FP32 on the CUDA
 * cores, or BSG_PREC_SPLIT: 3xTF32 on the tcgen05 tensor cores (even
 * chi >= 16); the per-sample displacement/probability/draw step runs in the
 * same precision (FP32 for split).  Synchronises `stream`. */
int bsg_sample(bsg_handle_t h, const void* const* Gammas, const double* Lambdas, int M, int chi, int d, int dd,
               const double* sqrtW, const double* normals, const double* uniforms, int64_t n, int precision,
               int64_t* samples, bsg_stream_t stream);

/* Batched displacement operators D(alpha) = expm(alpha a^dag - alpha^* a) in
 * the dd-dimensional truncation (sampling_cpu.py:133-148, `batch_displaces`;
 * distributed_sampling.py:169 uses torch.linalg.matrix_exp), from a closed
 * form of the truncated generator's eigen-decomposition.  alpha: c128
 * [count] (device); D: c128 [count, dd, dd] row-major.  1 <= dd <= BSG_MAX_DD. */
int bsg_displacements(bsg_handle_t h, const double* alpha, int64_t count, int dd, double* D, bsg_stream_t stream);

/* 3-way split TF32 GEMM on the tcgen05 tensor cores (no reference
 * counterpart; the building block of the split-precision contraction, exposed
 * for testing): C[M, N] = A[M, K] B[N, K]^T with A, B fp32 row-major (K
 * contiguous, K % 4 == 0), each split into TF32 hi + lo, products
 * hi*hi + hi*lo + lo*hi accumulated in FP32 in TMEM.  Synchronises `stream`. */
int bsg_gemm_tf32x3(bsg_handle_t h, const float* A, const float* B, float* C, int M, int N, int K,
                    bsg_stream_t stream);

/* Per-cut Williamson phase times of the last cut-spectra launch made while
 * profiling was enabled (bsg_cut_spectra or bsg_build_mps): ms[c * n_phases + i]
 * for phases 1 load + symmetry check, 2 Cholesky, 3 L^-1, 4 G, 5 H = G^T G
 * (full path) or F, QR and K (low-rank path), 6 Jacobi, 7 back-transform,
 * 8 ordering, 9 pairing, 10 S and nbar; columns 11 and 12 are the FP32 Jacobi
 * sweeps and the refinement steps (counts, not times), columns 13, 14 and 15
 * the ms of the FP32 sweeps, of the refinement's products and of the whole
 * refinement inside phase 6, columns 16-21 the ms of six parts of the
 * pairing (cluster setup, pivots and loads, projections, G products,
 * in-block Gram-Schmidt, residual tracking; the blocked vacuum pairing).
 * Pass ms = NULL to query the sizes. */
int bsg_profile_cut_phases(bsg_handle_t h, int* n_cuts, int* n_phases, double* ms);

/* Milestones of the last bsg_build_mps made while profiling was enabled, in
 * ms after the call's first launch: ms[4 g + k] for build group g (0 right
 * edge, 1 left edge, 2 middle; a small M runs one group) and k = 0 Williamson
 * done, 1 label keys queued to the host, 2 Sigma done, 3 DP done; -1 where
 * absent.  n: entries to fill (12 covers every group). */
int bsg_profile_build_timeline(bsg_handle_t h, double* ms, int n);

/* Host wall time (ms, summed since the last bsg_profile_reset while
 * profiling was enabled) of the site DP's planning phases: 0 row grouping
 * and partition keys of every (j, left group, right group) combination
 * (parallel), 1 new partition programs (serial), 2 per-site buckets
 * (parallel), 3 the global bucket list, 4 bucket layout and remap,
 * 5 program upload and the plan / scatter / DP launches, 6 plan staging
 * (the host tables copied into the pinned plan buffer), 7 the whole of it.
 * n: entries to fill (8 covers every phase). */
int bsg_profile_plan_phases(bsg_handle_t h, double* ms, int n);

/* Hafnian DP launches since the last bsg_profile_reset while profiling was
 * enabled.  *n_rows = buckets seen; rows[6 r + f] (r < max_rows) = launch
 * (0 large-table, 1 small-table programs), 32-item chunks, classes k, F ring
 * slots, DP states, transitions of the bucket's program.  state_hist[c]
 * (c < hist_len) = chunk-weighted count of states with c transitions (the
 * last entry collects larger counts).  rows / state_hist may be null. */
int bsg_profile_dp_buckets(bsg_handle_t h, double* rows, int max_rows, int* n_rows, double* state_hist,
                           int hist_len);

/* ---- covariance decomposition ---------------------------------------------
 * The pure quantum part of a Gaussian covariance, replacing
 * get_decomposition.py:16-29 (cvxpy/CVXOPT):
 *   sq_cov = argmin tr X  s.t.  [[X, Omega], [-Omega, X]] >= 0,  cov - X >= 0,
 * Omega = kron([[0, 1], [-1, 0]], I_M).  cov, sq_cov: device float64
 * [2M, 2M] row-major, xxpp order.  An infeasible-start primal-dual
 * interior-point method (HKM direction, Mehrotra predictor-corrector), all
 * in FP64 on the device; the Schur complement takes (M (2M + 1))^2 * 8
 * bytes (M <= 315; 0.2 GB at M = 50, 13.9 GB at M = 144).  Stops when the
 * relative duality gap, primal and dual residuals are all below tol, or
 * after max_iter (<= 1000) iterations (BSG_ERR_NO_CONVERGE; sq_cov then holds
 * the last iterate).  info (host, may be NULL): [iterations, relative gap,
 * primal residual, dual residual, primal objective tr X, dual objective].
 * Synchronises `stream`. */
int bsg_cov_decomposition(bsg_handle_t h, const double* cov, int M, double* sq_cov, double tol, int max_iter,
                          double* info, bsg_stream_t stream);

/* In-place lower Cholesky factor of a device float64 [n, n] row-major
 * symmetric matrix (the decomposition's blocked factorisation, exposed for
 * testing; the strict upper triangle is left as it was).  *info (host) = 0,
 * or the 1-based column of the first non-positive pivot.  Synchronises
 * `stream`. */
int bsg_potrf_f64(bsg_handle_t h, double* A, int n, int* info, bsg_stream_t stream);

/* ---- tuning knobs (no reference counterpart) ------------------------------
 * Launch parameters an autotuner may change per handle (bosonsupremacy_gb300
 * /autotune.py).  Values outside the documented range return BSG_ERR_INVALID. */
#define BSG_TUNE_DP_BLOCKS_PER_SM 0  /* resident 256-thread DP blocks per SM, 1..8 (default 8) */
#define BSG_TUNE_DP_L1_CARVEOUT 1    /* shared-memory carve-out percent for the DP kernel, 0..100 (default 0) */
#define BSG_TUNE_DP_SMALL_ENTRIES 2  /* programs with <= this many table entries per item run in a second DP
                                        launch with small per-warp slices, 0..4096 (default 64; 0 = one launch) */
#define BSG_TUNE_DP_SMALL_BLOCKS 3   /* resident DP blocks per SM in that second launch, 1..8 (default 8) */
#define BSG_TUNE_DP_SCRATCH_MIB 4    /* device memory for per-warp DP tables per launch, 64..65536 MiB (default 8192) */
#define BSG_TUNE_DP_FP64_BLOCKS 5    /* split precision: resident blocks per SM of a concurrent FP64 DP
                                        launch sharing the work queue (FP64 pipe), 0..8 (default 0 = off) */
#define BSG_TUNE_FACTOR_THREADS 6    /* threads per CTA of the Williamson and Sigma kernels, 256 / 512 / 1024
                                        (default 1024; fewer leave registers for DP blocks on the same SM) */
#define BSG_TUNE_GEMM_KERNEL 7       /* 3xTF32 tcgen05 GEMM: 0 one 128x128 tile per CTA, 1 persistent 128x256 tiles
                                        with a double TMEM accumulator (default 1) */
#define BSG_TUNE_DP_QUANTUM 8        /* hafnian DP: a warp leaves its launch after this many x 256 program
                                        transitions, so kernels on higher-priority streams get SMs; 0 keeps
                                        every DP block until the queue is empty (default 2) */
#define BSG_TUNE_DP_HOLD 9           /* pipelined build: 1 = the right group's DP waits until the left group's
                                        Williamson kernel is done (the left group's factorisations, the
                                        build's critical path, then run without the DP's memory traffic
                                        beside them), 0 = it starts with its Sigma (default 0) */
#define BSG_TUNE_RIGHT_PCT 10        /* pipelined build: percent of the cuts in the right group, 5..60,
                                        0 = built-in (33) */
#define BSG_TUNE_LEFT_PCT 11         /* pipelined build: percent of the cuts in the left group, 5..60,
                                        0 = built-in (33) */
#define BSG_TUNE_FACTOR_DUAL 12       /* Williamson launches: 1 = two CTAs of half the threads per SM when two fit
                                        in shared memory (the launches of small eigen-problems), 0 = one CTA of
                                        BSG_TUNE_FACTOR_THREADS (default 0) */
#define BSG_TUNE_DP_ORDER 13         /* pipelined build: priority order of the groups' DP streams, 0 = right >
                                        middle > left, 1 = left > right > middle, 2 = left > middle > right,
                                        3 = middle > left > right (default 0) */
#define BSG_TUNE_COUNT 14
int bsg_tune_set(bsg_handle_t h, int key, int value);
int bsg_tune_get(bsg_handle_t h, int key, int* value);

/* ---- measurement helpers (no reference counterpart) ---------------------
 * When enabled, every kernel launch of the handle is bracketed by CUDA
 * events on its stream; bsg_profile_read accumulates the elapsed times per
 * kernel class and the algorithmic work the launches were planned with.
 * Kernel classes: */
#define BSG_K_DP 0        /* hafnian DP (work: complex multiply-adds)           */
#define BSG_K_WILLIAMSON 1 /* per-cut Cholesky + Jacobi (work: FP64 FMAs)        */
#define BSG_K_THERMAL 2   /* per-cut top-chi selection (work: candidates ranked) */
#define BSG_K_SIGMA 3     /* per-site Sigma (work: FP64 FMAs)                    */
#define BSG_K_PREP 4      /* label rows, bucketing, conversions (work: items)    */
#define BSG_K_CONTRACT 5  /* transfer contraction (work: real flops)             */
#define BSG_K_HOST_PLAN 6 /* host wall time of bsg_build_mps between the label keys'
                             arrival and the DP launch: item planning, plan upload,
                             scatter launches (work: items planned)              */
#define BSG_K_HOST_WAIT 7 /* host wall time bsg_build_mps spends blocked on the
                             device (cut status, keys, final status)              */
#define BSG_K_SAMPLE 8    /* sampler: displacement, probability, draw, collapse
                             (work: complex multiply-adds); its chain GEMMs
                             count as BSG_K_CONTRACT                            */
#define BSG_K_COUNT 9
int bsg_profile_enable(bsg_handle_t h, int on);
/* Synchronises the recorded events; totals since the last reset. */
int bsg_profile_read(bsg_handle_t h, int kernel_class, double* total_ms, int64_t* launches, double* work);
int bsg_profile_reset(bsg_handle_t h);

/* Measured FMA throughput of this GPU's CUDA cores, in flop/s (2 per FMA),
 * for BSG_PREC_FP64 or BSG_PREC_FP32, from a register-resident FMA loop on
 * every SM.  Synchronises `stream`. */
int bsg_fma_peak(bsg_handle_t h, int precision, double* flops_per_s, bsg_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* BSG_H_ */
