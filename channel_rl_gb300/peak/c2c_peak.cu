// Host<->device bandwidth over NVLink-C2C: cudaMemcpyAsync of pinned host
// buffers (one stream, and split over two) against kernels that read or write
// pinned host memory directly.  118 MB per transfer, the U, V, W of a
// 256x96x192 channel.
#include <cstdio>
#include <cuda_runtime.h>
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("err %s line %d\n",cudaGetErrorString(e),__LINE__); return 1;}}while(0)
__global__ void rd(const double2* __restrict__ src, double2* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) dst[i] = src[i];
}
int main() {
  const size_t bytes = 118027784 / 16 * 16, n2 = bytes / 16;
  double *h_in, *h_out, *d;
  CK(cudaMallocHost(&h_in, bytes)); CK(cudaMallocHost(&h_out, bytes)); CK(cudaMalloc(&d, bytes));
  for (size_t i = 0; i < bytes / 8; ++i) h_in[i] = (double)i;
  cudaStream_t s, s2; CK(cudaStreamCreate(&s)); CK(cudaStreamCreate(&s2));
  cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
  int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  for (int rep = 0; rep < 3; ++rep) {
    float ms;
    cudaEventRecord(a, s); CK(cudaMemcpyAsync(d, h_in, bytes, cudaMemcpyHostToDevice, s)); cudaEventRecord(b, s);
    cudaEventSynchronize(b); cudaEventElapsedTime(&ms, a, b); if (rep == 2) printf("memcpy H2D %.1f GB/s\n", bytes / ms / 1e6);
    cudaEventRecord(a, s); CK(cudaMemcpyAsync(h_out, d, bytes, cudaMemcpyDeviceToHost, s)); cudaEventRecord(b, s);
    cudaEventSynchronize(b); cudaEventElapsedTime(&ms, a, b); if (rep == 2) printf("memcpy D2H %.1f GB/s\n", bytes / ms / 1e6);
    // 4 chunks on 2 streams each way
    cudaEventRecord(a, s);
    for (int c = 0; c < 4; ++c) CK(cudaMemcpyAsync((char*)d + c * (bytes / 4), (char*)h_in + c * (bytes / 4), bytes / 4, cudaMemcpyHostToDevice, (c & 1) ? s2 : s));
    cudaEvent_t j; cudaEventCreate(&j); cudaEventRecord(j, s2); cudaStreamWaitEvent(s, j, 0);
    cudaEventRecord(b, s); cudaEventSynchronize(b); cudaEventElapsedTime(&ms, a, b); if (rep == 2) printf("memcpy H2D 2 streams %.1f GB/s\n", bytes / ms / 1e6);
    for (int mult = 1; mult <= 8; mult *= 2) {
      cudaEventRecord(a, s); rd<<<sms * mult, 512, 0, s>>>((const double2*)h_in, (double2*)d, n2); cudaEventRecord(b, s);
      CK(cudaEventSynchronize(b)); cudaEventElapsedTime(&ms, a, b); if (rep == 2) printf("kernel read host x%d %.1f GB/s\n", mult, bytes / ms / 1e6);
      cudaEventRecord(a, s); rd<<<sms * mult, 512, 0, s>>>((const double2*)d, (double2*)h_out, n2); cudaEventRecord(b, s);
      CK(cudaEventSynchronize(b)); cudaEventElapsedTime(&ms, a, b); if (rep == 2) printf("kernel write host x%d %.1f GB/s\n", mult, bytes / ms / 1e6);
    }
  }
  CK(cudaGetLastError());
  printf("check %f %f\n", h_out[12345], h_in[12345]);
  return 0;
}
