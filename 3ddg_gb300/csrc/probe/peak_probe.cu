// Throughput probe for the roofline denominators of the FP64 path: FP64 and
// FP32 FMA chains (8 independent accumulators per thread) and a 2 GiB
// streaming copy.  Built and run by build.run_peak_probe().
#include <cstdio>
#include <cuda_runtime.h>
template <typename T>
__global__ void fma_kernel(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x * (T)1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < iters; i++) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void copy_kernel(const double2* __restrict__ a, double2* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) b[i] = a[i];
}
int main() {
  int dev = 0; cudaDeviceProp p; cudaGetDeviceProperties(&p, dev);
  printf("name %s sms %d smem/block optin %zu regs/sm %d l2 %d clock? cc %d.%d\n", p.name, p.multiProcessorCount, p.sharedMemPerBlockOptin, p.regsPerMultiprocessor, p.l2CacheSize, p.major, p.minor);
  int blocks = p.multiProcessorCount * 8, threads = 256, iters = 4096;
  double* od; float* of; cudaMalloc(&od, blocks * threads * 8); cudaMalloc(&of, blocks * threads * 4);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1); float ms;
  for (int rep = 0; rep < 2; rep++) {
    cudaEventRecord(e0); fma_kernel<double><<<blocks, threads>>>(od, iters, 0.999, 1e-3); cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    printf("fp64 fma: %.3f ms  %.3f TFLOP/s\n", ms, 2.0 * 8 * iters * (double)blocks * threads / ms / 1e9);
    cudaEventRecord(e0); fma_kernel<float><<<blocks, threads>>>(of, iters * 8, 0.999f, 1e-3f); cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    printf("fp32 fma: %.3f ms  %.3f TFLOP/s\n", ms, 2.0 * 8 * iters * 8 * (double)blocks * threads / ms / 1e9);
  }
  size_t n = (size_t)1 << 27; double2 *a, *b; cudaMalloc(&a, n * 16); cudaMalloc(&b, n * 16); cudaMemset(a, 0, n*16);
  for (int rep = 0; rep < 3; rep++) {
    cudaEventRecord(e0); copy_kernel<<<p.multiProcessorCount * 8, 512>>>(a, b, n); cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1); printf("copy %.3f ms  %.1f GB/s\n", ms, 2.0 * n * 16 / ms / 1e6);
  }
  printf("err %s\n", cudaGetErrorString(cudaGetLastError()));
  return 0;
}
