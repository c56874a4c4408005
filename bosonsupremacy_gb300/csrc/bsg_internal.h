// Internal declarations shared by the libbsg translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <unordered_map>
#include <vector>

#include "bsg.h"

namespace bsg {

// ---- error state (per host thread) ---------------------------------------
void set_error(const char* fmt, ...);

#define BSG_CHECK_ARG(cond, ...)           \
  do {                                     \
    if (!(cond)) {                         \
      ::bsg::set_error(__VA_ARGS__);       \
      return BSG_ERR_INVALID;              \
    }                                      \
  } while (0)

#define BSG_CUDA(call)                                                                        \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) {                                                                  \
      ::bsg::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return BSG_ERR_CUDA;                                                                    \
    }                                                                                         \
  } while (0)

#define BSG_TRY(call)             \
  do {                            \
    int s_ = (call);              \
    if (s_ != BSG_OK) return s_;  \
  } while (0)

// ---- partition programs ------------------------------------------------------
// A hafnian of a matrix whose rows/columns repeat class c m_c times equals
// prod_c m_c! * [x^m] exp(x^T A x / 2), A the k x k matrix between classes.
// The power-series coefficients F_r (r <= m componentwise) satisfy
//   F_r = (1 / r_a) * sum_{b >= a, r_b > 0 (r_a >= 2 if b == a)} A_ab F_{r - e_a - e_b},
// a = the first class with r_a > 0 (classes in ascending multiplicity), F_0 = 1.
// A "program" lists the reachable states of one multiplicity partition in
// topological order with their transitions; every item whose target has that
// multiplicity partition runs the same program, which makes warps uniform.
// Site programs have several roots: the site mode is the last class, and the
// hafnians with site multiplicity j = jmax, jmax - 2, ..., (one parity, the
// Gamma entries (a, b, j) of one row pair) are all states of one program,
// read out as the program reaches them (F_r does not depend on the root).
struct ProgramSet {
  // host mirror
  std::vector<uint64_t> keys;          // partition key per program
  std::vector<int32_t> k;              // classes per program
  std::vector<int32_t> nstates;        // states per program (>= 1)
  std::vector<int32_t> state_off;      // first state (global index) per program
  std::vector<int32_t> mult;           // [prog * BSG_MAX_CLASSES + c] multiplicities in class order
  // host-only per-state tables (planning, statistics); the device reads st_pack
  std::vector<int32_t> st_trans_off;   // per global state: first transition
  std::vector<int32_t> st_trans_cnt;   // per global state: number of transitions
  std::vector<int32_t> st_ra;          // per global state: r_a (0 for the empty state)
  std::vector<uint32_t> trans;         // packed (src F slot << 9) | (b << 2), b >= the state's class a
  std::vector<int32_t> fslots;         // F table entries per program (two levels of states)
  std::vector<uint4> st_pack;          // per global state: {first transition, count | r_a << 8 | (root j + 1) << 16,
                                       //  F slot, a}; root j + 1 = 0 when the state is not a root
  std::unordered_map<uint64_t, int32_t> index;
  // device copies (valid when dev_valid)
  int32_t* d_k = nullptr;
  int32_t* d_nstates = nullptr;
  int32_t* d_state_off = nullptr;
  uint32_t* d_trans = nullptr;
  uint4* d_st_pack = nullptr;
  size_t dev_states_cap = 0, dev_trans_cap = 0, dev_prog_cap = 0;
  size_t dev_states_n = 0, dev_trans_n = 0, dev_prog_n = 0;  // entries already on the device
  bool dev_valid = false;
  int max_states = 1;
  int max_k = 0;
};

// Key of a multiplicity multiset: 6 bits per multiplicity value 1..10.
constexpr int kKeyBits = 6;
constexpr int kKeyMaxMult = 10;
inline uint64_t key_add_class(uint64_t key, int mult) {
  return mult <= 0 ? key : key + (uint64_t(1) << (kKeyBits * (mult - 1)));
}
// Site programs: the multiset X of the label classes plus a last class (the
// site mode) with roots at multiplicities jmax, jmax - 2, ..., >= 0; the key
// carries jmax + 1 in its top four bits.
constexpr int kKeyRootShift = kKeyBits * kKeyMaxMult;
static_assert(kKeyRootShift + 4 <= 64, "root field");
inline uint64_t key_site_roots(uint64_t x_key, int jmax) { return x_key | (uint64_t(jmax + 1) << kKeyRootShift); }
int key_order(uint64_t key);            // sum of multiplicities (hafnian order n)
int key_classes(uint64_t key);          // number of classes

// Returns the program index for `key` (generating it on first use), or a
// negative status.
int program_for_key(ProgramSet& ps, uint64_t key, int32_t* prog_out);
// A program built apart from the set (thread-safe) and its serial append.
struct ProgramBuild {
  int k = 0, nstates = 0, fslots = 1, err = 0;
  std::string msg;
  std::vector<int> mult, st_trans_off, st_trans_cnt, st_ra;
  std::vector<uint32_t> trans;
  std::vector<uint4> st_pack;
};
int build_program(uint64_t key, ProgramBuild& b);
int append_program(ProgramSet& ps, uint64_t key, const ProgramBuild& b);
int programs_upload(ProgramSet& ps, cudaStream_t stream);
void programs_free(ProgramSet& ps);

// ---- device buffer helper ---------------------------------------------------
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  int ensure(size_t need);  // grows (never shrinks); contents not preserved
  void release();
};

// Per-handle launch timing (enabled by bsg_profile_enable).
struct Profiler {
  bool on = false;
  struct Rec {
    int cls;
    cudaEvent_t a, b;
    double work;
  };
  std::vector<Rec> pending;
  std::vector<cudaEvent_t> pool;
  double total_ms[BSG_K_COUNT] = {0};
  int64_t launches[BSG_K_COUNT] = {0};
  double work[BSG_K_COUNT] = {0};
  std::vector<double> cut_phases;  // ms per (cut, Williamson phase) of the last profiled cut launch
  std::vector<double> timeline;    // last profiled whole-MPS build: ms per (group, milestone)
  double plan_ms[8] = {0};         // host planning of the site DP since the last reset, ms per phase
  // DP launches since the last reset: one row per bucket (launch, chunks, classes,
  // F ring slots, states, transitions) and chunk-weighted states by transition count
  std::vector<double> dp_rows;
  std::vector<double> dp_state_hist;
  cudaEvent_t get();
  // begin/end bracket one launch on `st`
  int begin(int cls, cudaStream_t st, cudaEvent_t* ev);
  int end(int cls, cudaStream_t st, cudaEvent_t ev, double work);
  int flush();
  void add_work(int cls, double w) {
    if (on) work[cls] += w;
  }
  // host-timed classes (BSG_K_HOST_*): wall milliseconds measured by the caller
  void add_host(int cls, double ms, double w) {
    if (!on) return;
    total_ms[cls] += ms;
    launches[cls] += 1;
    work[cls] += w;
  }
  void release();
};

struct HostBuf {  // pinned host staging
  void* ptr = nullptr;
  size_t bytes = 0;
  int ensure(size_t need);
  void release();
};

// Launch arguments of the cut-spectra kernels (bsg_cuts.cu).
struct CutArgs {
  const double* sq_cov;
  int M, L0, n_cuts, d, chi;
  double err_tol;
  double* ws;          // per cut: 8 * nmax^2 doubles
  size_t ws_stride;    // doubles per cut
  double* S;           // [n_cuts, 2(M-1), 2(M-1)]
  int ldS;
  double* nbar;        // [n_cuts, kmax]
  int kmax;
  double* res;         // [n_cuts, chi]
  int8_t* num;         // [n_cuts, chi, M-1]
  int32_t* kept;       // [n_cuts]
  uint32_t* rec;       // per cut: kmax * chi records (parent << 8 | digit)
  int* status;         // [n_cuts]
  int* sweeps;         // [n_cuts] Jacobi sweeps used
  double* mu;          // [n_cuts, 2 kmax] eigenvalues of G^T G, then 1/nu per pair
  int max_sweeps;
  int c0;              // first cut of this launch (block b handles cut c0 + b)
  int jac_smem_m;      // > 0: the FP32 Jacobi matrix (and, with jac_q_smem, its eigenvectors) of eigen-problems up to this size live in shared memory
  int jac_q_smem;      // 1: the FP32 eigenvector rows in shared memory too
  unsigned long long* phase_t;  // [n_cuts, kCutPhases] phase timestamps (profiling) or null
};
constexpr int kCutTimedPhases = 11;  // stamps 0..10
constexpr int kCutPhases = 22;       // + FP32 sweeps, refinement steps, FP32 sweep / refinement product / refinement times, six pairing parts (ns)

// A byte range to set to one byte value; many of them are cleared by one
// launch (fill_spans).
struct FillSpan {
  void* p;
  int64_t bytes;
  int value;
};
// Fills every span in one launch.  stage: pinned host room and dev: device
// room for n spans (the span list is copied up first).
int fill_spans(bsg_handle_t h, const FillSpan* spans, int n, void* dev, void* stage, cudaStream_t st);
// The same with the span list already on the device; max_bytes: the largest span.
int fill_spans_dev(bsg_handle_t h, const FillSpan* dev_spans, int n, int64_t max_bytes, cudaStream_t st);

int cut_prepare(bsg_handle_t h, const double* sq_cov, int M, int L0, int n_cuts, int d, int chi, double err_tol,
                double* res, int8_t* num, double* S, int32_t* kept, CutArgs* out, cudaStream_t st);
size_t cut_ws_bytes(int M, int L0, int n_cuts, int chi);
// With `defer` non-null the output and status clears are appended to it
// instead of being queued as memsets (the caller fills them, e.g. together
// with other instances' in one launch).
int cut_prepare_at(bsg_handle_t h, char* base, const double* sq_cov, int M, int L0, int n_cuts, int d, int chi,
                   double err_tol, double* res, int8_t* num, double* S, int32_t* kept, CutArgs* out, cudaStream_t st,
                   std::vector<FillSpan>* defer = nullptr);
size_t cut_batch_bytes(const CutArgs* args, int n);
int cut_launch_batch(bsg_handle_t h, CutArgs* args, int n, void* dev, void* stage, cudaStream_t st);
int cut_launch_williamson(bsg_handle_t h, const CutArgs& a, int c0, int c1, cudaStream_t st);
int cut_launch_thermal(bsg_handle_t h, const CutArgs& a, int c0, int c1, cudaStream_t st);
// status of cuts [c0, c1) into hst[c0..c1) and their sweep counts into hst[n_cuts + c0 ..)
int cut_queue_status(const CutArgs& a, int c0, int c1, int* hst, cudaStream_t st);
int cut_check_status(bsg_handle_t h, const CutArgs& a, int c0, int c1, const int* status);
int cut_read_phases(bsg_handle_t h, const CutArgs& a, cudaStream_t st);

// One Sigma construction (bsg_sigma.cu).
struct SigmaJob {
  const double* S_l;  // [2 m_l, 2 m_l] (leading dimension ld_l) or null
  const double* S_r;  // general: [2Mr, 2Mr] (leading dimension ld_r); first: sq_cov
  int ld_l, ld_r;
  int m_l;
  int Mr;
  int first;          // 1: site-0 formula
  double2* Sigma;     // [2Mr, 2Mr]
  double* Z;
  double* ws;         // workspace, sigma_ws_bytes(Mr)
  int* status;        // 0 ok, 1 singular
};
size_t sigma_ws_bytes(int Mr);

// tcgen05 3xTF32 GEMM (bsg_umma.cu): C[M, N] (ldc) = (Ahi+Alo)(Bhi+Blo)^T, K-major
// operands already split; *d_err set on a pipeline timeout.
// 3xTF32 tcgen05 GEMM C[M, N] = A[M, K] B[N, K]^T (TF32 hi/lo operands).
// Grouped mode (mtiles non-null): n_mtiles row tiles {first row, end row, B
// row offset, 0}; B then has b_rows rows (one N-row block per group).
int gemm_tf32x3(bsg_handle_t h, const float* Ahi, const float* Alo, const float* Bhi, const float* Blo, float* C,
                int M, int N, int K, int ldc, int* d_err, cudaStream_t st, bool profile,
                const int4* mtiles = nullptr, int n_mtiles = 0, int b_rows = 0);
int split_tf32(bsg_handle_t h, const float* x, float* hi, float* lo, int64_t n, cudaStream_t st);

// Sliced GEMM (bsg_sliced.cu): C[M, N] fp64 (ldc) = A[M, K] B[N, K]^T from
// S fixed-point BF16 slices of b bits per FP64 operand row, exact FP32
// accumulation per slice level on the tcgen05 tensor cores.  Operands are
// stacked [S, rows, K] bf16 with per-row exponents; grouped mode as for
// gemm_tf32x3 (B rows of a tile group from mtiles[].z on).
void sliced_params(int K, int* S, int* b);
size_t sliced_operand_bytes(int64_t rows, int K, int S);
int sliced_slice_env(const double2* E, const int32_t* pidx, const double* lam, int rows, int chi, int S, int b,
                     void* A, int* ea, cudaStream_t st);
size_t sliced_gamma_scratch_bytes(int chi, int d);
int sliced_slice_gamma(const double2* G, int chi, int d, bool left, int S, int b, void* B, int* eb, void* scratch,
                       cudaStream_t st);
int sliced_gemm(bsg_handle_t h, const void* A, int a_rows, const int* ea, const void* B, int b_rows, const int* eb,
                double* C, int M, int N, int K, int ldc, int S, int b, int* d_err, cudaStream_t st, bool profile,
                const int4* mtiles, int n_mtiles);
// df_products: the Sigma products in double-float on the FP32 pipe (the
// split-precision build), else FP64.
int launch_sigma_jobs(bsg_handle_t h, const SigmaJob* jobs_host, int n_jobs, void* jobs_dev, cudaStream_t st,
                      bool df_products);

}  // namespace bsg

struct bsg_handle_s {
  int device = 0;
  int num_sms = 0;
  bsg::ProgramSet programs;
  // scratch reused across calls
  bsg::DevBuf warp_scratch;   // per-warp F rings of the DP kernel
  bsg::DevBuf items;          // bucketed item ids
  bsg::DevBuf plan;           // per-call plan tables
  bsg::DevBuf keys;           // per-row / per-item partition keys
  bsg::DevBuf misc;           // small counters
  bsg::DevBuf sigma_ws;       // Sigma construction workspace
  bsg::DevBuf cut_ws;         // cut spectra workspace
  bsg::DevBuf contract_ws;    // contraction workspace
  bsg::DevBuf mps_ws;         // whole-MPS build: Sigma, row tables, plans
  bsg::DevBuf sample_ws;      // sampler: chain GEMM operands and outputs
  bsg::DevBuf disp_tab;       // displacement eigen-tables for disp_dd
  bsg::DevBuf decomp_ws;      // covariance decomposition: iterates, Schur complement, step tests
  bsg::HostBuf decomp_host;   // its pinned scalars and index list
  int disp_dd = 0;
  bsg::HostBuf host_stage;    // pinned staging for plans
  bsg::HostBuf host_stage2;
  bsg::Profiler prof;
  // side streams for concurrent launches (created on first use) and events:
  // aux_stream (FP64 helper), grp[3] high-priority streams of the build
  // groups, dp_lo[3] lower-priority streams of the groups' DP (ranked right >
  // middle > left among themselves)
  cudaStream_t aux_stream = nullptr, grp[3] = {}, dp_lo[3] = {}, copy[2] = {};
  cudaEvent_t aux_fork = nullptr, aux_join = nullptr;
  cudaEvent_t ev[25] = {};
  int ensure_aux();
  // per-group buffers of the site DP (plan tables, item slots, per-warp
  // scratch, pinned plan staging); slot 0 serves the single-site calls,
  // slots 3 + 3 g .. 5 + 3 g the later site parts of build group g when the
  // Gammas are downloaded part by part
  struct SiteSlot {
    bsg::DevBuf plan, items, scratch;
    bsg::HostBuf stage;
  } slot[12];
  int tune[BSG_TUNE_COUNT] = {8, 0, 64, 8, 8192, 0, 1024, 1, 2, 0, 0, 0, 0, 0};
};

// Brackets a kernel launch with profiler events when profiling is on.
#define BSG_PROFILED(h, cls, st, work, launch)                  \
  do {                                                          \
    cudaEvent_t ev_ = nullptr;                                  \
    if ((h)->prof.on) BSG_TRY((h)->prof.begin(cls, st, &ev_));  \
    launch;                                                     \
    BSG_CUDA(cudaGetLastError());                               \
    if ((h)->prof.on) BSG_TRY((h)->prof.end(cls, st, ev_, work)); \
  } while (0)
