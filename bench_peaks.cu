// Peak probes behind bench.py's rooflines (`python bench.py --measure-peaks`
// compiles and runs this file and writes profiles/fp64_peak.json and
// profiles/c2c_bandwidth.json).
//
//   bench_peaks fp64     FP64 / FP32 issue rates (the FP64 roofline's denominator)
//   bench_peaks c2c      host<->device bandwidth (the end-to-end line's transfer floor)
//   bench_peaks barrier  a grid-wide barrier inside one cooperative persistent
//                        kernel against a kernel boundary inside a CUDA graph
//                        (with and without programmatic dependent launch): the
//                        cost per phase of the two ways to order a step's phases
//
#include <cstdio>
#include <cstring>
#include <cuda_runtime.h>
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("err %s line %d\n",cudaGetErrorString(e),__LINE__); return 1;}}while(0)

// Throughput probe: DFMA / DADD / DMUL / DDIV / DSQRT / FFMA rates on this GPU.
// Each FP64 probe runs CH independent dependency chains per thread (8, 16
// and 32 are swept, the loop body unrolled four times) so that the issue
// rate, not the latency of one chain, is what is measured; the largest rate
// of the sweep is the peak.  A mixed stream (DFMA, DADD, DMUL in the 2:1:1
// ratio of the solver's kernels) is measured the same way.  The operands
// other than the chain's own value are kernel parameters (constant bank) in
// the first probes and registers loaded from memory in the "reg" probes,
// which is how the solver's kernels hold theirs.

template <int OP, int CH>
__global__ void kd(double* out, double a_, double b_, int iters, const double* ab) {
  // OP >= 10: the same stream with a and b in registers (loaded, so not constants)
  const double a = OP >= 10 ? ab[0] : a_, b = OP >= 10 ? ab[1] : b_;
  const double one = ab[2], mzero = ab[3];   // 1.0 and -0.0, unknown to the compiler
  // OP 18: every DFMA reads three different registers (no operand reuse
  // between consecutive instructions), as the stencil kernels' FMAs do
  double x[8], y[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) { x[q] = OP == 18 ? ab[0] + q * 1e-9 : 0.0; y[q] = OP == 18 ? ab[1] * (q + 1) : 0.0; }
  double r[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) r[c] = threadIdx.x * 1e-9 + 1.0 + c * 1e-3;
  for (int it = 0; it < iters; ++it) {
#pragma unroll 4
    for (int u = 0; u < 4; ++u) {
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        if (OP == 0 || OP == 10) r[c] = fma(r[c], a, b);
        if (OP == 1 || OP == 11) r[c] = r[c] + a;
        if (OP == 12) r[c] = r[c] * a;                 // DMUL, register operand
        if (OP == 13) r[c] = fma(r[c], one, b);        // an addition issued as DFMA (exact: r*1 is r)
        if (OP == 15) r[c] = fma(r[c], a, mzero);      // a product issued as DFMA (exact: adding -0)
        if (OP == 16) r[c] = fma(r[c], 0.5, b);        // DFMA with a literal power of two
        if (OP == 17) r[c] = fma(r[c], 0.999999, b);   // DFMA with a general literal
        if (OP == 18) r[c] = fma(x[c & 7], r[c], y[(c + 3) & 7]);   // three distinct registers
        if (OP == 2) r[c] = b / r[c];
        if (OP == 3) r[c] = sqrt(r[c] + a);
        if (OP == 4 || OP == 14) {   // mixed: per 4 ops, 2 DFMA, 1 DADD, 1 DMUL
          if ((c & 3) < 2) r[c] = fma(r[c], a, b);
          else if ((c & 3) == 2) r[c] = r[c] + b;
          else r[c] = r[c] * a;
        }
      }
    }
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += r[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void kf(float* out, float a, float b, int iters) {
  float r[8];
  for (int i = 0; i < 8; i++) r[i] = threadIdx.x * 1e-6f + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; i++) r[i] = fmaf(r[i], a, b);
  }
  float s = 0;
  for (int i = 0; i < 8; i++) s += r[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <int OP, int CH>
int run(const char* name, double* d, int nb, int nt, int iters, int sms, int clk, double a, double b, double* best,
        const double* ab) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  for (int rep = 0; rep < 3; rep++) {
    cudaEventRecord(e0);
    kd<OP, CH><<<nb, nt>>>(d, a, b, iters, ab);
    cudaEventRecord(e1);
    CK(cudaEventSynchronize(e1));
    float ms;
    cudaEventElapsedTime(&ms, e0, e1);
    const double nops = (double)nb * nt * iters * 4 * CH;
    const double g = nops / ms / 1e6;
    if (rep == 2) {
      printf("%s x%d chains: %.3f ms, %.3f Gop/s (thread-ops), %.2f ops/clk/SM at %d MHz\n", name, CH, ms, g,
             nops / (ms * 1e-3) / sms / (clk * 1e3), clk / 1000);
      if (g > *best) *best = g;
    }
  }
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  return 0;
}

static int fp64_main() {
  int dev = 0;
  cudaDeviceProp p;
  CK(cudaGetDeviceProperties(&p, dev));
  int clk = 0;
  cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, dev);
  printf("name %s SMs %d cc %d.%d smem/block optin %zu L2 %d clock %d kHz\n", p.name, p.multiProcessorCount, p.major,
         p.minor, p.sharedMemPerBlockOptin, p.l2CacheSize, clk);
  const int sms = p.multiProcessorCount, nb = sms * 8, nt = 256;
  double* d;
  float* f;
  double* ab;
  CK(cudaMalloc(&d, nb * nt * 8));
  CK(cudaMalloc(&f, nb * nt * 4));
  CK(cudaMalloc(&ab, 4 * 8));
  const double hab[4] = {0.999999, 1e-7, 1.0, -0.0};
  CK(cudaMemcpy(ab, hab, sizeof(hab), cudaMemcpyHostToDevice));
  double dfma = 0, dadd = 0, ddiv = 0, dsqrt = 0, mixed = 0, regs = 0;
  if (run<0, 8>("DFMA", d, nb, nt, 1024, sms, clk, 0.999999, 1e-7, &dfma, ab)) return 1;
  if (run<0, 16>("DFMA", d, nb, nt, 512, sms, clk, 0.999999, 1e-7, &dfma, ab)) return 1;
  if (run<0, 32>("DFMA", d, nb, nt, 256, sms, clk, 0.999999, 1e-7, &dfma, ab)) return 1;
  if (run<1, 8>("DADD", d, nb, nt, 1024, sms, clk, 1e-7, 1e-7, &dadd, ab)) return 1;
  if (run<1, 16>("DADD", d, nb, nt, 512, sms, clk, 1e-7, 1e-7, &dadd, ab)) return 1;
  if (run<1, 32>("DADD", d, nb, nt, 256, sms, clk, 1e-7, 1e-7, &dadd, ab)) return 1;
  if (run<4, 8>("MIXED", d, nb, nt, 1024, sms, clk, 0.999999, 1e-7, &mixed, ab)) return 1;
  if (run<4, 16>("MIXED", d, nb, nt, 512, sms, clk, 0.999999, 1e-7, &mixed, ab)) return 1;
  if (run<4, 32>("MIXED", d, nb, nt, 256, sms, clk, 0.999999, 1e-7, &mixed, ab)) return 1;
  if (run<10, 8>("DFMA reg", d, nb, nt, 1024, sms, clk, 0.0, 0.0, &regs, ab)) return 1;
  if (run<10, 16>("DFMA reg", d, nb, nt, 512, sms, clk, 0.0, 0.0, &regs, ab)) return 1;
  if (run<10, 32>("DFMA reg", d, nb, nt, 256, sms, clk, 0.0, 0.0, &regs, ab)) return 1;
  if (run<11, 8>("DADD reg", d, nb, nt, 1024, sms, clk, 0.0, 0.0, &regs, ab)) return 1;
  if (run<11, 16>("DADD reg", d, nb, nt, 512, sms, clk, 0.0, 0.0, &regs, ab)) return 1;
  if (run<14, 16>("MIXED reg", d, nb, nt, 512, sms, clk, 0.0, 0.0, &regs, ab)) return 1;
  double dmulr = 0, addf = 0, mulf = 0, lit2 = 0, litg = 0;
  if (run<12, 16>("DMUL reg", d, nb, nt, 512, sms, clk, 0.0, 0.0, &dmulr, ab)) return 1;
  if (run<13, 16>("ADD as DFMA", d, nb, nt, 512, sms, clk, 0.0, 0.0, &addf, ab)) return 1;
  if (run<15, 16>("MUL as DFMA", d, nb, nt, 512, sms, clk, 0.0, 0.0, &mulf, ab)) return 1;
  if (run<16, 16>("DFMA literal 0.5", d, nb, nt, 512, sms, clk, 0.0, 0.0, &lit2, ab)) return 1;
  if (run<17, 16>("DFMA literal 0.999999", d, nb, nt, 512, sms, clk, 0.0, 0.0, &litg, ab)) return 1;
  double distinct = 0;
  if (run<18, 16>("DFMA 3 distinct regs", d, nb, nt, 512, sms, clk, 0.0, 0.0, &distinct, ab)) return 1;
  if (run<18, 32>("DFMA 3 distinct regs", d, nb, nt, 256, sms, clk, 0.0, 0.0, &distinct, ab)) return 1;
  if (run<2, 8>("DDIV", d, nb, nt, 64, sms, clk, 1e-7, 1.0000001, &ddiv, ab)) return 1;
  if (run<3, 8>("DSQRT", d, nb, nt, 64, sms, clk, 1e-7, 1e-7, &dsqrt, ab)) return 1;
  double ffma = 0;
  for (int rep = 0; rep < 3; rep++) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    cudaEventRecord(e0);
    kf<<<nb, nt>>>(f, 0.999f, 1e-3f, 16384);
    cudaEventRecord(e1);
    CK(cudaEventSynchronize(e1));
    float ms;
    cudaEventElapsedTime(&ms, e0, e1);
    const double nops = (double)nb * nt * 16384 * 8;
    if (rep == 2) { ffma = nops / ms / 1e6; printf("FFMA: %.3f ms, %.1f Gop/s\n", ms, ffma); }
    cudaEventDestroy(e0); cudaEventDestroy(e1);
  }
  printf("BEST dfma %.3f dadd %.3f mixed %.3f ddiv %.3f dsqrt %.3f ffma %.1f reg %.3f\n", dfma, dadd, mixed, ddiv, dsqrt,
         ffma, regs);
  CK(cudaGetLastError());
  return 0;
}

// Host<->device bandwidth over NVLink-C2C: cudaMemcpyAsync of pinned host
// buffers (one stream, and split over two) against kernels that read or write
// pinned host memory directly.  118 MB per transfer, the U, V, W of a
// 256x96x192 channel.
__global__ void rd(const double2* __restrict__ src, double2* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) dst[i] = src[i];
}
static int c2c_main() {
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

// ---------------------------------------------------------------- barrier
// Phase ordering cost.  Each phase updates 49152 doubles (the points of a
// 32x48x32 channel) once.  Persistent: all phases in one cooperative kernel,
// separated by a grid barrier (arrival counter plus generation word, every
// wait bounded: a block that gives up sets the error word and returns).
// Graph: one kernel per phase captured into a CUDA graph.
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ bool grid_barrier(unsigned* count, unsigned* gen, unsigned nb, long max_iter) {
  __syncthreads();
  int ok = 1;
  if (threadIdx.x == 0) {
    const unsigned g = ld_acquire_gpu(gen);
    __threadfence();
    if (atomicAdd(count, 1u) + 1u == nb) {
      atomicExch(count, 0u);
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      long it = 0;
      while (ld_acquire_gpu(gen) == g) if (++it > max_iter) { ok = 0; break; }
    }
    __threadfence();
  }
  return __syncthreads_and(ok);
}
__global__ void k_persist(unsigned* count, unsigned* gen, int nphase, double* buf, int n, int* err) {
  for (int ph = 0; ph < nphase; ++ph) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) buf[t] = fma(buf[t], 0.999, 1e-3);
    if (!grid_barrier(count, gen, gridDim.x, 2000000L)) { if (threadIdx.x == 0) atomicExch(err, 1); return; }
  }
}
__global__ void k_phase(double* buf, int n) {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) buf[t] = fma(buf[t], 0.999, 1e-3);
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
static int barrier_main() {
  int sms;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  const int n = 49152, nphase = 2000, ngraph = 200;
  double* buf; unsigned* cnt; int* err;
  CK(cudaMalloc(&buf, n * 8)); CK(cudaMemset(buf, 0, n * 8));
  CK(cudaMalloc(&cnt, 64)); CK(cudaMemset(cnt, 0, 64));
  CK(cudaMalloc(&err, 4)); CK(cudaMemset(err, 0, 4));
  cudaStream_t st;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  cudaEvent_t a, b;
  cudaEventCreate(&a); cudaEventCreate(&b);
  for (int tpb : {256, 512}) {
    int per = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_persist, tpb, 0));
    for (int mult = 1; mult <= 2 && mult <= per; ++mult) {   // co-resident grids only
      int nb = sms * mult, np = nphase, nn = n;
      unsigned* gen = cnt + 1;
      void* args[] = {&cnt, &gen, &np, &buf, &nn, &err};
      for (int rep = 0; rep < 3; ++rep) {
        CK(cudaEventRecord(a, st));
        CK(cudaLaunchCooperativeKernel((void*)k_persist, nb, tpb, args, 0, st));
        CK(cudaEventRecord(b, st));
        CK(cudaEventSynchronize(b));
        float ms;
        cudaEventElapsedTime(&ms, a, b);
        if (rep == 2) printf("persistent %d blocks x %d: %.3f us per phase\n", nb, tpb, ms * 1e3 / nphase);
      }
    }
  }
  int herr = 0;
  CK(cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost));
  printf("barrier timeouts %d\n", herr);
  for (int nb : {192, 768}) {
    for (int pdl = 1; pdl >= 0; --pdl) {
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
      at[0].val.programmaticStreamSerializationAllowed = 1;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = nb; cfg.blockDim = 64; cfg.stream = st; cfg.attrs = at; cfg.numAttrs = pdl;
      cudaGraph_t g;
      cudaGraphExec_t ge;
      CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      for (int i = 0; i < ngraph; ++i) CK(cudaLaunchKernelEx(&cfg, k_phase, buf, n));
      CK(cudaStreamEndCapture(st, &g));
      CK(cudaGraphInstantiate(&ge, g, 0));
      for (int rep = 0; rep < 4; ++rep) {
        CK(cudaEventRecord(a, st));
        CK(cudaGraphLaunch(ge, st));
        CK(cudaEventRecord(b, st));
        CK(cudaEventSynchronize(b));
        float ms;
        cudaEventElapsedTime(&ms, a, b);
        if (rep == 3) printf("graph %s %d blocks x 64: %.3f us per phase\n", pdl ? "pdl" : "plain", nb, ms * 1e3 / ngraph);
      }
      cudaGraphExecDestroy(ge);
      cudaGraphDestroy(g);
    }
  }
  CK(cudaGetLastError());
  return 0;
}

int main(int argc, char** argv) {
  if (argc > 1 && !std::strcmp(argv[1], "fp64")) return fp64_main();
  if (argc > 1 && !std::strcmp(argv[1], "c2c")) return c2c_main();
  if (argc > 1 && !std::strcmp(argv[1], "barrier")) return barrier_main();
  std::printf("usage: bench_peaks fp64|c2c|barrier\n");
  return 2;
}
