// Statistics of compute_statistics (statistics.f90:22-145): plane means of
// U, V, W, their squares and UV per row, the wall shear, u_tau, Re_tau and
// the bulk flows (mass_flow.f90:24-98).  The reference's summation ranges
// are kept, including their duplicated periodic columns and planes:
//   U   : x faces 1..nx-2 (each unique face once), z centres 1..nzg-2 (plane nzg-2 twice)
//   W   : x centres 1..nxg-2 (centre nxg-2 twice), z faces 1..nz-2 (once each)
//   V,UV: x centres 2..nxg-1 and z centres 2..nzg-1 (centre 2 / plane 2 twice)
// The wall shear uses the bottom wall for both walls, as statistics.f90:108-116 does.
#include "chl_common.cuh"

#define NST 7

// one block per (instance, Fortran row jj = r+1), r in [0, Ny]
__global__ void __launch_bounds__(256)
k_stats_rows(ChlMap map, int s, double* out, int pitch) {
  int lb;
  const int q = chl_find(map, blockIdx.x, lb);
  const ChlInst& I = map.inst[q];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const int r = lb;
  const double *U = I.U[s], *V = I.V[s], *W = I.W[s];
  const double w0 = 0.5 * I.w0x2[r], w1 = 0.5 * I.w1x2[r];   // exact halvings
  double acc[NST] = {0, 0, 0, 0, 0, 0, 0};
  for (int w = threadIdx.x; w < Nx * Nz; w += blockDim.x) {
    const int i = w % Nx, k = w / Nx;
    const double u = U[cidx(I, i, r, k)];
    const double wu = k == Nz - 1 ? 2.0 : 1.0;
    const double ww_ = W[cidx(I, i, r, k)];
    const double wwt = i == Nx - 1 ? 2.0 : 1.0;
    const double v = V[vidx(I, i, r, k)];
    const double wv = (i == 0 ? 2.0 : 1.0) * (k == 0 ? 2.0 : 1.0);
    const int im = wrap(i - 1, Nx);
    const double uyl = w0 * U[cidx(I, im, r, k)] + w1 * U[cidx(I, im, r + 1, k)];
    const double uyh = w0 * u + w1 * U[cidx(I, i, r + 1, k)];
    const double uc = 0.5 * (uyl + uyh);
    acc[0] += wu * u;  acc[1] += wv * v;  acc[2] += wwt * ww_;
    acc[3] += wu * u * u; acc[4] += wv * v * v; acc[5] += wwt * ww_ * ww_;
    acc[6] += wv * v * uc;
  }
  __shared__ double red[NST][256];
#pragma unroll
  for (int m = 0; m < NST; ++m) red[m][threadIdx.x] = acc[m];
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h)
#pragma unroll
      for (int m = 0; m < NST; ++m) red[m][threadIdx.x] += red[m][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double cu = (double)Nx * (Nz + 1), cv = (double)(Nx + 1) * (Nz + 1), cw = (double)(Nx + 1) * Nz;
    const double norm[NST] = {cu, cv, cw, cu, cv, cw, cv};
    for (int m = 0; m < NST; ++m) out[(size_t)q * pitch + (size_t)m * (Ny + 1) + r] = red[m][0] / norm[m];
  }
}

// one block per instance: tau (bottom wall), Qflow_x, Qflow_y
__global__ void __launch_bounds__(256)
k_stats_wall(ChlMap map, int s, double* out, int pitch) {
  const int q = blockIdx.x;
  const ChlInst& I = map.inst[q];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const double *U = I.U[s], *V = I.V[s], *nt = I.nut;
  double tau = 0.0, qx = 0.0, nx_ = 0.0, qy = 0.0, ny_ = 0.0;
  const double w0 = 0.5 * I.w0x2[0], w1 = 0.5 * I.w1x2[0];
  for (long w = threadIdx.x; w < (long)Nx * Nz; w += blockDim.x) {
    const int i = (int)(w % Nx), k = (int)(w / Nx), ip = wrap(i + 1, Nx);
    const double ntf0 = 0.5 * (nt[cidx(I, i, 0, k)] + nt[cidx(I, ip, 0, k)]);
    const double ntf1 = 0.5 * (nt[cidx(I, i, 1, k)] + nt[cidx(I, ip, 1, k)]);
    const double ntw = w0 * ntf0 + w1 * ntf1;      // nu + nu_t at the wall (weights sum to 1)
    tau += (U[cidx(I, i, 1, k)] - U[cidx(I, i, 0, k)]) / I.dyw * ntw;
  }
  for (long w = threadIdx.x; w < (long)Nx * (Ny - 1) * Nz; w += blockDim.x) {
    const int i = (int)(w % Nx), jc = 2 + (int)((w / Nx) % (Ny - 1)), k = (int)(w / ((long)Nx * (Ny - 1)));
    const double dyg = I.dyf[jc - 1];
    qx += (U[cidx(I, i, jc, k)] + U[cidx(I, i, jc - 1, k)]) * 0.5 * dyg;
    nx_ += (1.0 + 1.0) * 0.5 * dyg;
  }
  for (long w = threadIdx.x; w < (long)Nx * Ny * Nz; w += blockDim.x) {
    const int i = (int)(w % Nx), jv = 1 + (int)((w / Nx) % Ny), k = (int)(w / ((long)Nx * Ny));
    const double wv = (i == 0 ? 2.0 : 1.0) * (k == 0 ? 2.0 : 1.0);
    const double dy = 1.0 / I.rdyc[jv];      // y(j)-y(j-1), j_f = jv+1
    qy += wv * (V[vidx(I, i, jv, k)] + V[vidx(I, i, jv - 1, k)]) * 0.5 * dy;
    ny_ += wv * (1.0 + 1.0) * 0.5 * dy;
  }
  __shared__ double red[5][256];
  red[0][threadIdx.x] = tau; red[1][threadIdx.x] = qx; red[2][threadIdx.x] = nx_;
  red[3][threadIdx.x] = qy; red[4][threadIdx.x] = ny_;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h)
      for (int m = 0; m < 5; ++m) red[m][threadIdx.x] += red[m][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double* o = out + (size_t)q * pitch + (size_t)NST * (Ny + 1);
    o[0] = red[0][0] / ((double)Nx * Nz);
    o[1] = red[1][0] / red[2][0];
    o[2] = red[3][0] / red[4][0];
  }
}

extern "C" void chl_launch_stats(const ChlMap& rows, int nrows_blocks, double* out, int pitch, int s,
                                 cudaStream_t st) {
  k_stats_rows<<<nrows_blocks, 256, 0, st>>>(rows, s, out, pitch);
  k_stats_wall<<<rows.n, 256, 0, st>>>(rows, s, out, pitch);
}
