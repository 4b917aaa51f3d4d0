// Stand-alone throughput probe (not part of the library): FP64 and FP32 FMA
// issue rates with 8 independent chains per thread, and a device copy
// bandwidth.  Built and run by les_gb300/peaks.py; the FP64 figure is the
// denominator of the FP64 step's compute roofline.
#include <cstdio>
#include <cuda_runtime.h>
template <typename T>
__global__ void fma_kernel(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void copy_kernel(const double2* __restrict__ a, double2* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) b[i] = a[i];
}
int main() {
  cudaDeviceProp p; cudaGetDeviceProperties(&p, 0);
  printf("name=%s sms=%d cc=%d.%d smem_optin=%zu l2=%d\n", p.name, p.multiProcessorCount, p.major, p.minor, p.sharedMemPerBlockOptin, p.l2CacheSize);
  int blocks = p.multiProcessorCount * 8, threads = 256, iters = 4096;
  double* od; float* of; cudaMalloc(&od, blocks * threads * 8); cudaMalloc(&of, blocks * threads * 4);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  for (int rep = 0; rep < 3; ++rep) {
    fma_kernel<double><<<blocks, threads>>>(od, iters, 0.999999, 1e-7);
    cudaEventRecord(e0);
    fma_kernel<double><<<blocks, threads>>>(od, iters, 0.999999, 1e-7);
    cudaEventRecord(e1); cudaEventSynchronize(e1);
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    double flops = 2.0 * 8 * iters * (double)blocks * threads;
    printf("fp64 fma: %.3f ms  %.3f TFLOP/s\n", ms, flops / ms / 1e9);
    fma_kernel<float><<<blocks, threads>>>(of, iters * 4, 0.999999f, 1e-7f);
    cudaEventRecord(e0);
    fma_kernel<float><<<blocks, threads>>>(of, iters * 4, 0.999999f, 1e-7f);
    cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    flops = 2.0 * 8 * iters * 4 * (double)blocks * threads;
    printf("fp32 fma: %.3f ms  %.3f TFLOP/s\n", ms, flops / ms / 1e9);
  }
  size_t n = (size_t)1 << 27;  // 2 GiB per buffer
  double2 *a, *b; cudaMalloc(&a, n * 16); cudaMalloc(&b, n * 16); cudaMemset(a, 0, n * 16);
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    copy_kernel<<<p.multiProcessorCount * 16, 512>>>(a, b, n);
    cudaEventRecord(e1); cudaEventSynchronize(e1);
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    printf("copy: %.3f ms %.1f GB/s\n", ms, 2.0 * n * 16 / ms / 1e6);
  }
  printf("err=%s\n", cudaGetErrorString(cudaGetLastError()));
  return 0;
}
