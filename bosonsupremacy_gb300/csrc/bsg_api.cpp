// Handle lifetime, error reporting and buffer helpers of libbsg.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "bsg_internal.h"

namespace bsg {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int DevBuf::ensure(size_t need) {
  if (need <= bytes && ptr) return BSG_OK;
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
  size_t sz = need < 256 ? 256 : need;
  cudaError_t e = cudaMalloc(&ptr, sz);
  if (e != cudaSuccess) {
    ptr = nullptr;
    set_error("cudaMalloc(%zu) failed: %s", sz, cudaGetErrorString(e));
    return BSG_ERR_ALLOC;
  }
  bytes = sz;
  return BSG_OK;
}

void DevBuf::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

int HostBuf::ensure(size_t need) {
  if (need <= bytes && ptr) return BSG_OK;
  if (ptr) cudaFreeHost(ptr);
  ptr = nullptr;
  bytes = 0;
  size_t sz = need < 256 ? 256 : need;
  cudaError_t e = cudaMallocHost(&ptr, sz);
  if (e != cudaSuccess) {
    ptr = nullptr;
    set_error("cudaMallocHost(%zu) failed: %s", sz, cudaGetErrorString(e));
    return BSG_ERR_ALLOC;
  }
  bytes = sz;
  return BSG_OK;
}

void HostBuf::release() {
  if (ptr) cudaFreeHost(ptr);
  ptr = nullptr;
  bytes = 0;
}

cudaEvent_t Profiler::get() {
  if (!pool.empty()) {
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

int Profiler::begin(int cls, cudaStream_t st, cudaEvent_t* ev) {
  (void)cls;
  *ev = get();
  if (!*ev) {
    set_error("cudaEventCreate failed");
    return BSG_ERR_CUDA;
  }
  BSG_CUDA(cudaEventRecord(*ev, st));
  return BSG_OK;
}

int Profiler::end(int cls, cudaStream_t st, cudaEvent_t ev, double w) {
  cudaEvent_t e2 = get();
  if (!e2) {
    set_error("cudaEventCreate failed");
    return BSG_ERR_CUDA;
  }
  BSG_CUDA(cudaEventRecord(e2, st));
  pending.push_back(Rec{cls, ev, e2, w});
  return BSG_OK;
}

int Profiler::flush() {
  for (auto& r : pending) {
    BSG_CUDA(cudaEventSynchronize(r.b));
    float ms = 0.f;
    BSG_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
    total_ms[r.cls] += ms;
    launches[r.cls] += 1;
    work[r.cls] += r.work;
    pool.push_back(r.a);
    pool.push_back(r.b);
  }
  pending.clear();
  return BSG_OK;
}

void Profiler::release() {
  for (auto& r : pending) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  pending.clear();
  for (auto e : pool) cudaEventDestroy(e);
  pool.clear();
}

}  // namespace bsg

int bsg_handle_s::ensure_aux() {
  if (aux_stream) return BSG_OK;
  int least = 0, greatest = 0;
  BSG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  BSG_CUDA(cudaStreamCreateWithFlags(&aux_stream, cudaStreamNonBlocking));
  for (auto& s : grp) BSG_CUDA(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, greatest));
  // the DP streams of the whole-MPS build's groups (right, left, middle)
  // rank below the factorisation streams and among themselves in the order
  // the groups should finish (right, middle, left): with one shared level
  // the middle group's later launches queue behind the left group's blocks
  // and both groups finish at the end of the build, which bunches up their
  // host downloads
  const int dp_prio[3] = {std::min(least, std::max(greatest + 1, least - 2)), least,
                          std::min(least, std::max(greatest + 1, least - 1))};
  for (int g = 0; g < 3; ++g) BSG_CUDA(cudaStreamCreateWithPriority(&dp_lo[g], cudaStreamNonBlocking, dp_prio[g]));
  for (auto& s : copy) BSG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  BSG_CUDA(cudaEventCreateWithFlags(&aux_fork, cudaEventDisableTiming));
  BSG_CUDA(cudaEventCreateWithFlags(&aux_join, cudaEventDisableTiming));
  for (auto& e : ev) BSG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return BSG_OK;
}

extern "C" {

int bsg_profile_enable(bsg_handle_t h, int on) {
  BSG_CHECK_ARG(h, "bsg_profile_enable: null handle");
  h->prof.on = on != 0;
  return BSG_OK;
}

int bsg_profile_reset(bsg_handle_t h) {
  BSG_CHECK_ARG(h, "bsg_profile_reset: null handle");
  BSG_TRY(h->prof.flush());
  for (int i = 0; i < BSG_K_COUNT; ++i) {
    h->prof.total_ms[i] = 0;
    h->prof.launches[i] = 0;
    h->prof.work[i] = 0;
  }
  h->prof.dp_rows.clear();
  h->prof.dp_state_hist.clear();
  for (double& x : h->prof.plan_ms) x = 0.0;
  return BSG_OK;
}

int bsg_profile_plan_phases(bsg_handle_t h, double* ms, int n) {
  BSG_CHECK_ARG(h && ms, "bsg_profile_plan_phases: null pointer");
  for (int i = 0; i < n; ++i) ms[i] = i < 8 ? h->prof.plan_ms[i] : 0.0;
  return BSG_OK;
}

int bsg_profile_dp_buckets(bsg_handle_t h, double* rows, int max_rows, int* n_rows, double* state_hist,
                           int hist_len) {
  BSG_CHECK_ARG(h && n_rows, "bsg_profile_dp_buckets: null pointer");
  const int n = int(h->prof.dp_rows.size() / 6);
  *n_rows = n;
  if (rows)
    for (int i = 0; i < std::min(n, max_rows) * 6; ++i) rows[i] = h->prof.dp_rows[i];
  if (state_hist)
    for (int i = 0; i < hist_len; ++i)
      state_hist[i] = i < (int)h->prof.dp_state_hist.size() ? h->prof.dp_state_hist[i] : 0.0;
  return BSG_OK;
}

int bsg_profile_read(bsg_handle_t h, int cls, double* total_ms, int64_t* launches, double* work) {
  BSG_CHECK_ARG(h, "bsg_profile_read: null handle");
  BSG_CHECK_ARG(cls >= 0 && cls < BSG_K_COUNT, "bsg_profile_read: bad kernel class %d", cls);
  BSG_TRY(h->prof.flush());
  if (total_ms) *total_ms = h->prof.total_ms[cls];
  if (launches) *launches = h->prof.launches[cls];
  if (work) *work = h->prof.work[cls];
  return BSG_OK;
}

int bsg_profile_cut_phases(bsg_handle_t h, int* n_cuts, int* n_phases, double* ms) {
  BSG_CHECK_ARG(h, "bsg_profile_cut_phases: null handle");
  const int np = bsg::kCutPhases - 1;
  const int nc = int(h->prof.cut_phases.size() / bsg::kCutPhases);
  if (n_cuts) *n_cuts = nc;
  if (n_phases) *n_phases = np;
  if (ms)
    for (int c = 0; c < nc; ++c)
      for (int i = 0; i < np; ++i) ms[(size_t)c * np + i] = h->prof.cut_phases[(size_t)c * bsg::kCutPhases + i + 1];
  return BSG_OK;
}

int bsg_profile_build_timeline(bsg_handle_t h, double* ms, int n) {
  BSG_CHECK_ARG(h && ms, "bsg_profile_build_timeline: null pointer");
  for (int i = 0; i < n; ++i) ms[i] = i < (int)h->prof.timeline.size() ? h->prof.timeline[i] : -1.0;
  return BSG_OK;
}

int bsg_tune_set(bsg_handle_t h, int key, int value) {
  BSG_CHECK_ARG(h, "bsg_tune_set: null handle");
  BSG_CHECK_ARG(key >= 0 && key < BSG_TUNE_COUNT, "bsg_tune_set: unknown key %d", key);
  if (key == BSG_TUNE_DP_BLOCKS_PER_SM) BSG_CHECK_ARG(value >= 1 && value <= 8, "bsg_tune_set: blocks per SM %d", value);
  if (key == BSG_TUNE_DP_L1_CARVEOUT) BSG_CHECK_ARG(value >= 0 && value <= 100, "bsg_tune_set: carve-out %d", value);
  if (key == BSG_TUNE_DP_SMALL_ENTRIES)
    BSG_CHECK_ARG(value >= 0 && value <= 4096, "bsg_tune_set: small-program entries %d", value);
  if (key == BSG_TUNE_DP_SMALL_BLOCKS)
    BSG_CHECK_ARG(value >= 1 && value <= 8, "bsg_tune_set: small-launch blocks per SM %d", value);
  if (key == BSG_TUNE_DP_FP64_BLOCKS)
    BSG_CHECK_ARG(value >= 0 && value <= 8, "bsg_tune_set: FP64 helper blocks per SM %d", value);
  if (key == BSG_TUNE_GEMM_KERNEL) BSG_CHECK_ARG(value == 0 || value == 1, "bsg_tune_set: GEMM kernel %d", value);
  if (key == BSG_TUNE_FACTOR_THREADS)
    BSG_CHECK_ARG(value == 256 || value == 512 || value == 1024, "bsg_tune_set: factor threads %d", value);
  if (key == BSG_TUNE_DP_SCRATCH_MIB)
    BSG_CHECK_ARG(value >= 64 && value <= 65536, "bsg_tune_set: DP scratch %d MiB", value);
  if (key == BSG_TUNE_RIGHT_PCT || key == BSG_TUNE_LEFT_PCT)
    BSG_CHECK_ARG(value == 0 || (value >= 5 && value <= 60), "bsg_tune_set: group share %d %%", value);
  if (key == BSG_TUNE_DP_HOLD) BSG_CHECK_ARG(value == 0 || value == 1, "bsg_tune_set: DP hold %d", value);
  if (key == BSG_TUNE_FACTOR_DUAL) BSG_CHECK_ARG(value == 0 || value == 1, "bsg_tune_set: factor dual %d", value);
  if (key == BSG_TUNE_DP_ORDER) BSG_CHECK_ARG(value >= 0 && value <= 3, "bsg_tune_set: DP order %d", value);
  if (key == BSG_TUNE_DP_QUANTUM)
    BSG_CHECK_ARG(value >= 0 && value <= (1 << 20), "bsg_tune_set: DP quantum %d", value);
  h->tune[key] = value;
  return BSG_OK;
}

int bsg_tune_get(bsg_handle_t h, int key, int* value) {
  BSG_CHECK_ARG(h && value, "bsg_tune_get: null pointer");
  BSG_CHECK_ARG(key >= 0 && key < BSG_TUNE_COUNT, "bsg_tune_get: unknown key %d", key);
  *value = h->tune[key];
  return BSG_OK;
}

const char* bsg_last_error(void) { return bsg::g_err; }

int bsg_version(void) { return 10000; }

int bsg_create(int device, bsg_handle_t* out) {
  BSG_CHECK_ARG(out != nullptr, "bsg_create: out is NULL");
  *out = nullptr;
  int n = 0;
  BSG_CUDA(cudaGetDeviceCount(&n));
  BSG_CHECK_ARG(device >= 0 && device < n, "bsg_create: device %d out of range (%d devices)", device, n);
  BSG_CUDA(cudaSetDevice(device));
  auto* h = new bsg_handle_s();
  h->device = device;
  cudaError_t e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    delete h;
    bsg::set_error("cudaDeviceGetAttribute failed: %s", cudaGetErrorString(e));
    return BSG_ERR_CUDA;
  }
  *out = h;
  return BSG_OK;
}

int bsg_destroy(bsg_handle_t h) {
  if (!h) return BSG_OK;
  cudaSetDevice(h->device);
  if (h->aux_stream) {
    cudaStreamSynchronize(h->aux_stream);
    cudaStreamDestroy(h->aux_stream);
    for (auto s : h->grp) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
    for (auto s : h->dp_lo) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
    for (auto s : h->copy) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
    cudaEventDestroy(h->aux_fork);
    cudaEventDestroy(h->aux_join);
    for (auto e : h->ev) cudaEventDestroy(e);
  }
  bsg::programs_free(h->programs);
  h->warp_scratch.release();
  h->items.release();
  h->plan.release();
  h->keys.release();
  h->misc.release();
  h->sigma_ws.release();
  h->cut_ws.release();
  h->contract_ws.release();
  h->mps_ws.release();
  h->sample_ws.release();
  h->disp_tab.release();
  h->decomp_ws.release();
  h->decomp_host.release();
  for (auto& sl : h->slot) {
    sl.plan.release();
    sl.items.release();
    sl.scratch.release();
    sl.stage.release();
  }
  h->host_stage.release();
  h->host_stage2.release();
  h->prof.release();
  delete h;
  return BSG_OK;
}

}  // extern "C"
