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

}  // namespace bsg

extern "C" {

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
  bsg::programs_free(h->programs);
  h->warp_scratch.release();
  h->items.release();
  h->plan.release();
  h->keys.release();
  h->misc.release();
  h->sigma_ws.release();
  h->cut_ws.release();
  h->contract_ws.release();
  h->host_stage.release();
  h->host_stage2.release();
  delete h;
  return BSG_OK;
}

}  // extern "C"
