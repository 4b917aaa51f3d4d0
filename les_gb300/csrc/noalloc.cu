// Tridiagonal solve that allocates no device memory.
//
// les_tridag_array_noalloc runs the same kernel as les_tridag_array, but
// takes device pointers and sizes directly (no les_ctx, whose creation
// allocates) and draws its scratch from a fixed array compiled into this
// library.  It exists for callers that must not allocate device memory
// themselves or have a library do it for them: code that owns all device
// memory through its own pool or arena (a host application that reserves
// the GPU up front, a framework allocator that accounts every byte), and
// code that runs where an allocation would fail or serialise the device.
//
// The scratch array below is held on every GPU that loads this library,
// until the process exits.  All calls share it and it keeps the last call's
// contents, so each call clears the part that must start at zero (the pivot
// flag); the Thomas coefficients are written before they are read.  Two
// calls whose kernels overlap on the GPU (different streams, or different
// host threads on one device) race on the array and give wrong results:
// serialise them on one stream.
#include <cstdint>
#include <mutex>

#include "common.cuh"
#include "les_internal.h"

namespace {

// 256 B for the pivot flag, then the Thomas coefficients gam(lh, ny, n).
constexpr size_t kFlagBytes = 256;
constexpr size_t kGamDoubles = LES_NOALLOC_TRIDAG_MAX_ELEMS;
static __device__ __align__(256) unsigned char g_tridag_scratch[kFlagBytes + kGamDoubles * sizeof(double)];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_tridag_scratch on the current device, looked up once
// per device (the first call on each device does it).
int scratch_address(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    les_set_error("tridag_array_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    return LES_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    les_set_error("tridag_array_noalloc: device %d beyond the %d supported", dev, kMaxDevices);
    return LES_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_tridag_scratch);
    if (e != cudaSuccess || !p) {
      les_set_error("tridag_array_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      return LES_ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return LES_OK;
}

// Device memory of the current device (or managed memory), 'align'-aligned.
int device_pointer(const void* p, size_t align, const char* name) {
  if (!p || (reinterpret_cast<uintptr_t>(p) & (align - 1))) {
    les_set_error("tridag_array_noalloc: %s is null or not %zu-byte aligned", name, align);
    return LES_ERR_ARG;
  }
  cudaPointerAttributes at;
  cudaError_t e = cudaPointerGetAttributes(&at, p);
  int dev = -1;
  cudaGetDevice(&dev);
  if (e != cudaSuccess || (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) ||
      at.device != dev) {
    cudaGetLastError();
    les_set_error("tridag_array_noalloc: %s is not device memory of the current device", name);
    return LES_ERR_ARG;
  }
  return LES_OK;
}

// Row-1 pivot check of tridag_array.f90:32-39 (every ky, kx < lh): bit 2.
__global__ void k_first_pivot(const double* __restrict__ b, int lh, int ny, int* flag) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= lh * ny) return;
  if (t % lh != lh - 1 && b[t] == 0.0) atomicOr(flag, 2);
}

}  // namespace

extern "C" int les_tridag_array_noalloc(const double* a, const double* b, const double* c, const double* r,
                                        double* u, int lh, int ny, int n, void* stream) {
  if (lh < 2 || ny < 2 || (ny & 1) || n < 1) {
    les_set_error("tridag_array_noalloc: bad sizes lh=%d ny=%d n=%d", lh, ny, n);
    return LES_ERR_ARG;
  }
  const size_t elems = (size_t)lh * ny * n;
  if (elems > kGamDoubles) {
    les_set_error("tridag_array_noalloc: lh*ny*n = %zu exceeds the fixed scratch of %zu elements", elems,
                  (size_t)kGamDoubles);
    return LES_ERR_ARG;
  }
  int st;
  if ((st = device_pointer(a, 8, "a")) || (st = device_pointer(b, 8, "b")) || (st = device_pointer(c, 8, "c")) ||
      (st = device_pointer(r, 16, "r")) || (st = device_pointer(u, 16, "u")))
    return st;
  void* base = nullptr;
  if ((st = scratch_address(&base))) return st;
  int* flag = static_cast<int*>(base);
  double* gam = reinterpret_cast<double*>(static_cast<unsigned char*>(base) + kFlagBytes);
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  // Row 1 is checked before the solve is launched, as tridag_array.f90:32-39
  // stops before writing u: on that error u is left as the caller passed it.
  LES_CUDA_CHECK(cudaMemsetAsync(flag, 0, sizeof(int), s));
  const int nk = lh * ny;
  k_first_pivot<<<(nk + 127) / 128, 128, 0, s>>>(b, lh, ny, flag); LES_COUNT_LAUNCH();
  int fl = 0;
  LES_CUDA_CHECK(cudaMemcpyAsync(&fl, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  LES_CUDA_CHECK(cudaStreamSynchronize(s));
  LES_CUDA_CHECK(cudaGetLastError());
  if (fl & 2) { les_set_error("tridag_array_noalloc: rewrite eqs, zero b in row 1"); return LES_ERR_PIVOT; }
  les::launch_tridag_generic(a, b, c, r, u, gam, lh, ny, n, flag, s);
  LES_CUDA_CHECK(cudaMemcpyAsync(&fl, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  LES_CUDA_CHECK(cudaStreamSynchronize(s));
  LES_CUDA_CHECK(cudaGetLastError());
  if (fl) { les_set_error("tridag_array_noalloc failed: zero pivot"); return LES_ERR_PIVOT; }
  return LES_OK;
}
