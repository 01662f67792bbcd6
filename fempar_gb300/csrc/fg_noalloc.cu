// fg_noalloc.cu -- fg_system_spmv_device_noalloc: y = A x without any device allocation.
//
// For callers that cannot call cudaMalloc: serving loops that reserve all of their HBM up
// front and may not grow it, and host frameworks whose caching allocator owns the device
// memory (a cudaMalloc behind its back can fail or fragment its pool).
// fg_system_spmv_device stages x and y in the solver's padded vector layout inside work
// buffers that the system allocates the first time they are needed; this variant stages
// them in the file-scope device array below instead, so a call allocates nothing.
//
// The array is FG_NOALLOC_SCRATCH_BYTES (32 MiB) on every GPU that loads the library,
// held until the process exits.  With lazy module loading (the CUDA default) the module,
// and with it the array, is loaded on a device at the first call there; that takes 32 MiB
// outside the context's HBM budget, so a caller that reserves its HBM up front makes the
// first call before reserving.  The array's host-side name is only a stand-in: host code
// must not pass `g_noalloc_scratch` to a kernel.  The first call on a device looks up the
// array's device address there with cudaGetSymbolAddress (once per device, with that
// device current) and caches it; make that first call before any stream capture.  All
// calls share the array and it keeps the last call's contents, so every call first clears
// the part of the staged x vector that must read zero (entries of nodes that are not free
// dofs).  Calls that overlap on the GPU race on the array.  The call is synchronous: it
// waits on the context's stream until y holds the result, and leaves the caller's current
// device as it found it.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "fg_internal.h"

static __device__ __align__(256) unsigned char g_noalloc_scratch[FG_NOALLOC_SCRATCH_BYTES];

namespace fg {

static constexpr int NB = 256;

template <typename T>
__global__ void k_na_zero(int64_t n, T* a) {
  for (int64_t i = blockIdx.x * (int64_t)NB + threadIdx.x; i < n; i += (int64_t)gridDim.x * NB) a[i] = (T)0;
}
template <typename T>
__global__ void k_na_rows_to_vec(int64_t n, const int32_t* __restrict__ row2vec, const T* __restrict__ src,
                                 T* __restrict__ dst) {
  int64_t r = blockIdx.x * (int64_t)NB + threadIdx.x;
  if (r < n) dst[row2vec[r]] = src[r];
}
template <typename T>
__global__ void k_na_vec_to_rows(int64_t n, const int32_t* __restrict__ row2vec, const T* __restrict__ src,
                                 T* __restrict__ dst) {
  int64_t r = blockIdx.x * (int64_t)NB + threadIdx.x;
  if (r < n) dst[r] = src[row2vec[r]];
}

// device address of the scratch array, per device (looked up once, then cached)
static fg_status scratch_address(int device, void** out) {
  static std::mutex mu;
  static void* addr[64] = {nullptr};
  if (device < 0 || device >= 64) { set_error("device id %d out of range", device); return FG_ERR_BADARG; }
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      set_error("cudaGetSymbolAddress(noalloc scratch) on device %d: %s", device, cudaGetErrorString(e));
      return FG_ERR_CUDA;
    }
    addr[device] = p;
  }
  *out = addr[device];
  return FG_OK;
}

template <typename T>
static fg_status spmv_noalloc(fg_system* sys, int precision, const T* x, T* y, unsigned char* scratch) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  cudaStream_t st = ctx->stream;
  const int64_t n = sp->nfree, nv = sp->nvec;
  T* xv = reinterpret_cast<T*>(scratch);
  // y's staging starts on a 256-byte boundary after x's
  const size_t xbytes = ((size_t)nv * sizeof(T) + 255) / 256 * 256;
  T* yv = reinterpret_cast<T*>(scratch + xbytes);
  const unsigned gz = (unsigned)std::min<int64_t>((nv + NB - 1) / NB, (int64_t)ctx->sm_count * 8);
  k_na_zero<T><<<gz > 0 ? gz : 1, NB, 0, st>>>(nv, xv);
  k_na_rows_to_vec<T><<<(unsigned)((n + NB - 1) / NB), NB, 0, st>>>(n, sp->d_row2vec, x, xv);
  FG_CUDA_TRY(cudaGetLastError());
  FG_TRY(system_spmv_layout_noalloc(sys, precision, xv, yv, st));
  k_na_vec_to_rows<T><<<(unsigned)((n + NB - 1) / NB), NB, 0, st>>>(n, sp->d_row2vec, yv, y);
  FG_CUDA_TRY(cudaGetLastError());
  ctx->launches += 3;
  FG_CUDA_TRY(cudaStreamSynchronize(st));
  return FG_OK;
}

}  // namespace fg

using namespace fg;

extern "C" fg_status fg_system_spmv_device_noalloc(fg_system* sys, int precision, const void* x, void* y) {
  if (!sys || !x || !y) {
    set_error("bad argument: system/x/y");
    return FG_ERR_BADARG;
  }
  if (precision != FG_FP64 && precision != FG_MIXED) {
    set_error("bad argument: precision");
    return FG_ERR_BADARG;
  }
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  const size_t elem = precision == FG_MIXED ? sizeof(float) : sizeof(double);
  const size_t need = (((size_t)sp->nvec * elem + 255) / 256 * 256) + (size_t)sp->nvec * elem;
  if (need > (size_t)FG_NOALLOC_SCRATCH_BYTES) {
    set_error("fg_system_spmv_device_noalloc: the system needs %zu bytes of staging (solver_vec_len %lld), more "
              "than the %u-byte no-allocation scratch; use fg_system_spmv_device",
              need, (long long)sp->nvec, (unsigned)FG_NOALLOC_SCRATCH_BYTES);
    return FG_ERR_BADARG;
  }
  if (sp->nfree == 0) return FG_OK;  // nothing to multiply (all dofs Dirichlet), as fg_system_spmv_device
  int prev = -1;
  cudaError_t e = cudaGetDevice(&prev);
  if (e != cudaSuccess) {
    set_error("cudaGetDevice: %s", cudaGetErrorString(e));
    return FG_ERR_CUDA;
  }
  e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) {
    set_error("cudaSetDevice: %s", cudaGetErrorString(e));
    return FG_ERR_CUDA;
  }
  void* scratch = nullptr;
  fg_status st = scratch_address(ctx->device, &scratch);
  if (st == FG_OK) {
    if (precision == FG_MIXED)
      st = spmv_noalloc<float>(sys, precision, (const float*)x, (float*)y, (unsigned char*)scratch);
    else
      st = spmv_noalloc<double>(sys, precision, (const double*)x, (double*)y, (unsigned char*)scratch);
  }
  // the caller's current device is left as it was
  if (prev != ctx->device) cudaSetDevice(prev);
  return st;
}
