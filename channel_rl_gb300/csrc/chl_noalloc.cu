// Allocation-free divergence check.
//
// chl_check_divergence_noalloc computes what chl_check_divergence reports
// (the signed maximum of div u of check_divergence, projection.f90:223-245,
// and max |div u|) directly from caller-owned device arrays, without a
// handle and without allocating anything.
//
// Who needs it: a caller that owns all device memory itself and must not
// let a library allocate.  Examples are a Fortran or C code whose device
// memory comes from its own pool or from a framework's allocator (a
// cudaMalloc outside that pool breaks its accounting and can fail when the
// pool holds the device), and a time loop that cannot afford the implicit
// device synchronisation that cudaMalloc/cudaFree may cause.  Such a caller
// cannot use chl_create, which allocates the channel state.
//
// Scratch: one partial (max, max|.|) pair per z plane plus the final pair,
// in the file-scope array below, so the largest grid has
// CHL_NOALLOC_MAX_PLANES interior z planes (nz - 1 <= 4096; 64 KiB on every
// GPU that loads the library, held until the process exits).  Every slot
// that a call reads is written earlier in the same call, so nothing needs
// clearing between calls.  All calls share the array: calls that overlap on
// the GPU (different streams, or different host threads on one device)
// race on it and must be serialised by the caller.
//
// Address lookup: host code cannot use the array's name as a device
// address (it is a host-side stand-in), so every call asks the CUDA runtime
// for the array's address with cudaGetSymbolAddress in the context current
// on the calling thread.  The array sits at a different address in each
// context the library's kernels are loaded into (a context the caller made
// with the driver API, or the primary context after a device reset), so an
// address kept from an earlier call could point outside the current one.
// The call is a host-side table lookup once the module is loaded.
//
// Stream capture: a call copies its two results to pageable host memory and
// synchronises `stream`, so it cannot be made while any stream is being
// captured.
#include "../../include/chl.h"

#include <cuda_runtime.h>
#include <cstring>

#define CHL_NOALLOC_MAX_PLANES 4096

static __device__ __align__(256) double chl_noalloc_scratch[2 * CHL_NOALLOC_MAX_PLANES + 2];

namespace {

thread_local char g_err[256] = "";

void set_err(const char* m) { std::strncpy(g_err, m, sizeof(g_err) - 1); g_err[sizeof(g_err) - 1] = 0; }

// One block per interior z plane k_f = 2..nzg-1; centres i_f = 2..nxg-1,
// j_f = 2..nyg-1 of Fortran arrays U(nx,nyg,nzg), V(nxg,ny,nzg), W(nxg,nyg,nz).
__global__ void __launch_bounds__(256)
k_div_planes(const double* __restrict__ U, const double* __restrict__ V, const double* __restrict__ W,
             const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
             int nx, int ny, int nz, double* scratch) {
  const int nxg = nx + 1, nyg = ny + 1, nzg = nz + 1;
  const int kf = 2 + blockIdx.x;                       // Fortran k
  const int ni = nxg - 2, nj = nyg - 2;
  const double rz = 1.0 / (z[kf - 1] - z[kf - 2]);     // z(k) - z(k-1)
  double mx = 0.0, ma = 0.0;
  for (int w = threadIdx.x; w < ni * nj; w += blockDim.x) {
    const int i = 2 + w % ni, j = 2 + w / ni;          // Fortran i, j
    const size_t u = (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)nyg * (kf - 1));
    const size_t v = (size_t)(i - 1) + (size_t)nxg * ((size_t)(j - 1) + (size_t)ny * (kf - 1));
    const size_t ww = (size_t)(i - 1) + (size_t)nxg * ((size_t)(j - 1) + (size_t)nyg * (kf - 1));
    const double d = (U[u] - U[u - 1]) / (x[i - 1] - x[i - 2])
                   + (V[v] - V[v - nxg]) / (y[j - 1] - y[j - 2])
                   + (W[ww] - W[ww - (size_t)nxg * nyg]) * rz;
    mx = fmax(mx, d);
    ma = fmax(ma, fabs(d));
  }
  __shared__ double r0[256], r1[256];
  r0[threadIdx.x] = mx; r1[threadIdx.x] = ma;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      r0[threadIdx.x] = fmax(r0[threadIdx.x], r0[threadIdx.x + h]);
      r1[threadIdx.x] = fmax(r1[threadIdx.x], r1[threadIdx.x + h]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) { scratch[2 * blockIdx.x] = r0[0]; scratch[2 * blockIdx.x + 1] = r1[0]; }
  (void)nzg;
}

__global__ void k_div_final(double* scratch, int nplanes) {
  double mx = 0.0, ma = 0.0;
  for (int p = threadIdx.x; p < nplanes; p += blockDim.x) {
    mx = fmax(mx, scratch[2 * p]);
    ma = fmax(ma, scratch[2 * p + 1]);
  }
  __shared__ double r0[256], r1[256];
  r0[threadIdx.x] = mx; r1[threadIdx.x] = ma;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      r0[threadIdx.x] = fmax(r0[threadIdx.x], r0[threadIdx.x + h]);
      r1[threadIdx.x] = fmax(r1[threadIdx.x], r1[threadIdx.x + h]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    scratch[2 * CHL_NOALLOC_MAX_PLANES] = r0[0];
    scratch[2 * CHL_NOALLOC_MAX_PLANES + 1] = r1[0];
  }
}

}  // namespace

extern "C" {

const char* chl_noalloc_last_error(void) { return g_err; }

int chl_check_divergence_noalloc(const double* U, const double* V, const double* W,
                                 const double* x, const double* y, const double* z,
                                 int nx, int ny, int nz, void* stream,
                                 double* max_div, double* max_abs_div) {
  if (!U || !V || !W || !x || !y || !z || !max_div || !max_abs_div) {
    set_err("chl_check_divergence_noalloc: null pointer");
    return CHL_E_ARG;
  }
  if (nx < 3 || ny < 3 || nz < 3) {
    set_err("chl_check_divergence_noalloc: nx, ny, nz must be >= 3");
    return CHL_E_ARG;
  }
  const int nplanes = nz - 1;                          // k_f = 2..nzg-1
  if (nplanes > CHL_NOALLOC_MAX_PLANES) {
    set_err("chl_check_divergence_noalloc: nz - 1 exceeds the 4096 z planes its fixed scratch holds");
    return CHL_E_ARG;
  }
  void* sym = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&sym, chl_noalloc_scratch);
  if (e != cudaSuccess || !sym) {
    set_err("chl_check_divergence_noalloc: cudaGetSymbolAddress of the scratch array failed (no usable CUDA context?)");
    return CHL_E_CUDA;
  }
  double* scratch = static_cast<double*>(sym);
  cudaStream_t st = (cudaStream_t)stream;
  // cudaLaunchKernel returns this launch's own status, so an error that an
  // unrelated earlier call left pending is neither reported here nor cleared
  {
    void* a[] = {(void*)&U, (void*)&V, (void*)&W, (void*)&x, (void*)&y, (void*)&z,
                 (void*)&nx, (void*)&ny, (void*)&nz, (void*)&scratch};
    e = cudaLaunchKernel((const void*)k_div_planes, dim3(nplanes), dim3(256), a, 0, st);
  }
  if (e == cudaSuccess) {
    int np = nplanes;
    void* a[] = {(void*)&scratch, (void*)&np};
    e = cudaLaunchKernel((const void*)k_div_final, dim3(1), dim3(256), a, 0, st);
  }
  if (e != cudaSuccess) {
    set_err(cudaGetErrorString(e));
    return CHL_E_CUDA;
  }
  double r[2];
  e = cudaMemcpyAsync(r, scratch + 2 * CHL_NOALLOC_MAX_PLANES, sizeof(r), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    set_err(cudaGetErrorString(e));
    return CHL_E_CUDA;
  }
  *max_div = r[0];
  *max_abs_div = r[1];
  return CHL_OK;
}

}  // extern "C"
