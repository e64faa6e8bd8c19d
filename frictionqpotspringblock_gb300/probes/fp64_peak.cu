// FP64 / FP32 / u64 throughput probe for the roofline denominator of the FP64-bound step kernel:
// independent register chains, one output per thread.  Build: nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o fp64_peak fp64_peak.cu
#include <cstdio>
#include <cuda_runtime.h>
template <int OP>
__global__ void kd(double* out, double x0, int iters) {
  double a0 = x0 + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  const double b = 1.0000001, c = 1e-9;
  for (int i = 0; i < iters; ++i) {
    if (OP == 0) { a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c); a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c); }
    if (OP == 1) { a0 = __dadd_rn(a0, c); a1 = __dadd_rn(a1, c); a2 = __dadd_rn(a2, c); a3 = __dadd_rn(a3, c); a4 = __dadd_rn(a4, c); a5 = __dadd_rn(a5, c); a6 = __dadd_rn(a6, c); a7 = __dadd_rn(a7, c); }
    if (OP == 2) { a0 = __dmul_rn(a0, b); a1 = __dmul_rn(a1, b); a2 = __dmul_rn(a2, b); a3 = __dmul_rn(a3, b); a4 = __dmul_rn(a4, b); a5 = __dmul_rn(a5, b); a6 = __dmul_rn(a6, b); a7 = __dmul_rn(a7, b); }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}
__global__ void kf(float* out, float x0, int iters) {
  float a0 = x0 + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  const float b = 1.0000001f, c = 1e-9f;
  for (int i = 0; i < iters; ++i) { a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c); a4 = fmaf(a4, b, c); a5 = fmaf(a5, b, c); a6 = fmaf(a6, b, c); a7 = fmaf(a7, b, c); }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}
__global__ void ki(unsigned long long* out, unsigned long long x0, int iters) {
  unsigned long long a0 = x0 + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
  const unsigned long long m = 0x5851f42d4c957f2dULL, inc = 1;
  for (int i = 0; i < iters; ++i) { a0 = a0 * m + inc; a1 = a1 * m + inc; a2 = a2 * m + inc; a3 = a3 * m + inc; }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 ^ a1 ^ a2 ^ a3;
}
int main() {
  int dev = 0; cudaDeviceProp p; cudaGetDeviceProperties(&p, dev);
  printf("device %s sms %d cc %d.%d\n", p.name, p.multiProcessorCount, p.major, p.minor);
  const int blocks = p.multiProcessorCount * 8, threads = 256, iters = 1 << 14;
  size_t n = (size_t)blocks * threads;
  double* od; float* of; unsigned long long* oi;
  cudaMalloc(&od, n * 8); cudaMalloc(&of, n * 4); cudaMalloc(&oi, n * 8);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  const char* names[3] = {"dfma", "dadd", "dmul"};
  for (int rep = 0; rep < 2; ++rep) {
    float ms;
    cudaEventRecord(e0); kd<0><<<blocks, threads>>>(od, 1.0, iters / 4); cudaEventRecord(e1); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    printf("%s: %.3f Gop/s\n", names[0], 8.0 * n * (iters / 4) / ms / 1e6);
    cudaEventRecord(e0); kd<1><<<blocks, threads>>>(od, 1.0, iters / 4); cudaEventRecord(e1); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    printf("%s: %.3f Gop/s\n", names[1], 8.0 * n * (iters / 4) / ms / 1e6);
    cudaEventRecord(e0); kd<2><<<blocks, threads>>>(od, 1.0, iters / 4); cudaEventRecord(e1); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    printf("%s: %.3f Gop/s\n", names[2], 8.0 * n * (iters / 4) / ms / 1e6);
    cudaEventRecord(e0); kf<<<blocks, threads>>>(of, 1.0f, iters); cudaEventRecord(e1); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    printf("ffma: %.3f Gop/s\n", 8.0 * n * iters / ms / 1e6);
    cudaEventRecord(e0); ki<<<blocks, threads>>>(oi, 1ull, iters); cudaEventRecord(e1); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    printf("u64 mul-add: %.3f Gop/s\n", 4.0 * n * iters / ms / 1e6);
  }
  cudaError_t err = cudaGetLastError(); printf("status %s\n", cudaGetErrorString(err));
  return err == cudaSuccess ? 0 : 1;
}
