// Layout conversion, time step, constant mass flow, reductions.
#include "chl_common.cuh"

// ------------------------------------------------------------ Fortran <-> device layout
// Fortran array F(n1,n2,n3) (column-major, full ghosted extents of the
// reference) <-> device field: x/z unique points, all y rows.  Unpacking
// (k_unpack3): kind 0 U/W-like (ghost rows 0 and Ny+1 = minus the first
// interior row), kind 1 V-like (wall rows 0 and Ny set to zero).

// device field -> Fortran array with every ghost filled (periodic copies in
// x and z, stored ghost/wall rows in y)
__global__ void k_pack(double* __restrict__ F, const double* __restrict__ src, int Nx, int nrow, int Nz,
                       int n1, int n2, int n3, double sub) {
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)n1 * n2 * n3) return;
  const int i1 = (int)(t % n1), j1 = (int)((t / n1) % n2), k1 = (int)(t / ((long)n1 * n2));
  int i = (i1 - 1) % Nx; if (i < 0) i += Nx;
  int k = (k1 - 1) % Nz; if (k < 0) k += Nz;
  const int j = j1 < nrow ? j1 : nrow - 1;
  const double v = src[(size_t)i + (size_t)Nx * ((size_t)j + (size_t)nrow * k)];
  F[t] = sub == 0.0 ? v : v - sub;     // nu_t is stored as nu + nu_t
}

// The same two conversions for U, V and W in one launch (blockIdx.y picks
// the field), between the device fields and the three Fortran-layout
// arrays of the staging area, so that the three host copies of a transfer
// run back to back and one kernel converts them.  A block is 4 rows of 64
// lanes (threadIdx.y, threadIdx.x); a row is one (j, k) line of x, whose
// coordinates take one 32-bit division per row, and the lanes stride along
// it: these kernels only move memory, and a 64-bit division per element (a
// long integer sequence) had held them to a fifth of the HBM bandwidth.
#define CHL_CONV_ROWS 4
#define CHL_CONV_LANES 64
__global__ void __launch_bounds__(CHL_CONV_ROWS * CHL_CONV_LANES)
k_unpack3(ChlFields3 f3, int Nx, int Nz) {
  const ChlField1& q = f3.f[blockIdx.y];
  const int nrow = q.nrow;
  const int r = blockIdx.x * CHL_CONV_ROWS + threadIdx.y;      // row (j, k) of the device field
  if (r >= nrow * Nz) return;
  const int j = r % nrow, k = r / nrow;
  double* __restrict__ dst = q.dev + (size_t)Nx * r;
  const int last = nrow - 1;
  if (q.kind == 1 && (j == 0 || j == last)) {
    for (int i = threadIdx.x; i < Nx; i += CHL_CONV_LANES) dst[i] = 0.0;
    return;
  }
  int js = j;
  bool neg = false;
  if (q.kind == 0 && j == 0) { js = 1; neg = true; }
  if (q.kind == 0 && j == last) { js = last - 1; neg = true; }
  const double* __restrict__ src = q.fort + 1 + (size_t)q.n1 * ((size_t)js + (size_t)q.n2 * (size_t)(k + 1));
  if (neg) { for (int i = threadIdx.x; i < Nx; i += CHL_CONV_LANES) dst[i] = -src[i]; }
  else { for (int i = threadIdx.x; i < Nx; i += CHL_CONV_LANES) dst[i] = src[i]; }
}

__global__ void __launch_bounds__(CHL_CONV_ROWS * CHL_CONV_LANES)
k_pack3(ChlFields3 f3, int Nx, int Nz) {
  const ChlField1& q = f3.f[blockIdx.y];
  const int n1 = q.n1, n2 = q.n2, nrow = q.nrow;
  const int r = blockIdx.x * CHL_CONV_ROWS + threadIdx.y;      // row (j1, k1) of the Fortran array
  if (r >= n2 * q.n3) return;
  const int j1 = r % n2, k1 = r / n2;
  const int k = k1 == 0 ? Nz - 1 : (k1 - 1 >= Nz ? k1 - 1 - Nz : k1 - 1);
  const int j = j1 < nrow ? j1 : nrow - 1;
  const double* __restrict__ src = q.dev + (size_t)Nx * ((size_t)j + (size_t)nrow * k);
  double* __restrict__ dst = q.fort + (size_t)n1 * r;
  for (int i1 = threadIdx.x; i1 < n1; i1 += CHL_CONV_LANES) {
    const int i = i1 == 0 ? Nx - 1 : (i1 - 1 >= Nx ? i1 - 1 - Nx : i1 - 1);
    dst[i1] = src[i];
  }
}

// device field (rows jlo..jhi) -> dense unique-point array (Nx, jhi-jlo+1, Nz)
__global__ void k_pack_unique(double* __restrict__ F, const double* __restrict__ src, int Nx, int nrow,
                              int Nz, int jlo, int nj) {
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)Nx * nj * Nz) return;
  const int i = (int)(t % Nx), j = (int)((t / Nx) % nj), k = (int)(t / ((long)Nx * nj));
  F[t] = src[(size_t)i + (size_t)Nx * ((size_t)(j + jlo) + (size_t)nrow * k)];
}

extern "C" {
void chl_launch_pack(double* F, const double* src, int Nx, int nrow, int Nz, int n1, int n2, int n3, double sub,
                     cudaStream_t st) {
  long n = (long)n1 * n2 * n3;
  k_pack<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(F, src, Nx, nrow, Nz, n1, n2, n3, sub);
}
// one launch for the three fields; grid x covers the rows of the largest
void chl_launch_unpack3(const ChlFields3& f3, int Nx, int Nz, cudaStream_t st) {
  int rows = 0;
  for (auto& q : f3.f) rows = rows > q.nrow * Nz ? rows : q.nrow * Nz;
  k_unpack3<<<dim3((unsigned)((rows + CHL_CONV_ROWS - 1) / CHL_CONV_ROWS), 3), dim3(CHL_CONV_LANES, CHL_CONV_ROWS),
              0, st>>>(f3, Nx, Nz);
}
void chl_launch_pack3(const ChlFields3& f3, int Nx, int Nz, cudaStream_t st) {
  int rows = 0;
  for (auto& q : f3.f) rows = rows > q.n2 * q.n3 ? rows : q.n2 * q.n3;
  k_pack3<<<dim3((unsigned)((rows + CHL_CONV_ROWS - 1) / CHL_CONV_ROWS), 3), dim3(CHL_CONV_LANES, CHL_CONV_ROWS),
            0, st>>>(f3, Nx, Nz);
}
void chl_launch_pack_unique(double* F, const double* src, int Nx, int nrow, int Nz, int jlo, int nj, cudaStream_t st) {
  long n = (long)Nx * nj * Nz;
  k_pack_unique<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(F, src, Nx, nrow, Nz, jlo, nj);
}
}

// ------------------------------------------------------------ compute_dt (time_integration.f90:102-150)
// max(dx/|u|) over points = max over the index with its own spacing of
// dx/min|u|, so only min |u| per x face (U), per y face row (V) and per z
// face (W) is reduced; |u| is reduced on its bit pattern (integer pipe).
#define CHL_BIG_BITS 0x7FF0000000000000ULL
__device__ __forceinline__ unsigned long long absbits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFULL;
}

// dt of one instance from the minima of |U|, |V|, |W| (compute_dt,
// time_integration.f90:102-150), by one whole block of up to 1024 threads;
// thread 0 stores it.  With a fixed time step (CFL < 0) the step is -CFL
// whatever the velocities, so nothing is reduced.  The maxima are formed by
// warp shuffles and one pass over the warps' results.  The minima are read
// from L2 (other blocks formed them with atomics).
__device__ __forceinline__ double warp_fmax(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ void dt_from_minima(const ChlInst& I) {
  if (I.CFL < 0.0) {
    if (threadIdx.x == 0) chl_put_dt(I.scal, -I.CFL);
    return;
  }
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const unsigned long long* g = I.minabs;
  __shared__ double r[3][32];
  double lu = 0.0, lv = 0.0, lw = 0.0;
  // U: faces i_f = 2..nxg-1 (my 0..Nx, face Nx is the copy of face 0)
  for (int i = threadIdx.x; i <= Nx; i += blockDim.x)
    lu = fmax(lu, I.dxf[i] / __longlong_as_double((long long)__ldcg(g + (i == Nx ? 0 : i))));
  // V: face rows j_f = 2..nyg-1 (my 1..Ny; row Ny is the wall, |V| = 0)
  for (int j = 1 + threadIdx.x; j <= Ny; j += blockDim.x)
    lv = fmax(lv, I.dyf[j] / __longlong_as_double((long long)__ldcg(g + Nx + j)));
  // W: faces k_f = 2..nzg-1 (my 0..Nz)
  for (int k = threadIdx.x; k <= Nz; k += blockDim.x)
    lw = fmax(lw, I.dzf[k] / __longlong_as_double((long long)__ldcg(g + Nx + Ny + 1 + (k == Nz ? 0 : k))));
  lu = warp_fmax(lu); lv = warp_fmax(lv); lw = warp_fmax(lw);
  const int warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if ((threadIdx.x & 31) == 0) { r[0][warp] = lu; r[1][warp] = lv; r[2][warp] = lw; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < nw; ++w) {
      lu = fmax(lu, r[0][w]); lv = fmax(lv, r[1][w]); lw = fmax(lw, r[2][w]);
    }
    const double C = I.CFL;
    const double dt_conv = fmin(fmin(C * lu, C * lv), C * lw);
    double dt = fmin(dt_conv, I.dt_vis);
    dt = fmin(dt, 1e-3);
    chl_put_dt(I.scal, dt);
  }
}

// Blocks per instance: Nz planes x MINABS_CHUNKS(Ny) row chunks.  The
// block's threads run over (x, row) with x fastest in whole warps (x padded
// to a multiple of 32), so a warp covers 32 x-points of one row and every
// warp of the block has work even when Nx is 32.  Each thread keeps its
// minima of |U| at its x-face and of |W|; the per-row minimum of |V| is
// formed by warp shuffles.  Mins of non-negative doubles are mins of their
// bit patterns, so the reductions are exact and order-free.
#define MINABS_ROWS 16
__device__ __forceinline__ int minabs_chunks(int Ny) { return (Ny + MINABS_ROWS - 1) / MINABS_ROWS; }

__global__ void __launch_bounds__(256)
k_minabs(ChlMap map, int s) {
  chl_pdl_wait();
  __shared__ unsigned long long sv[MINABS_ROWS];
  __shared__ unsigned long long swm[8];
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny;
  const int nch = minabs_chunks(Ny);
  const int k = lb / nch, j0 = 1 + (lb % nch) * MINABS_ROWS;
  const int j1 = min(Ny, j0 + MINABS_ROWS - 1);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x < MINABS_ROWS) sv[threadIdx.x] = CHL_BIG_BITS;
  __syncthreads();
  const double* U = I.U[s]; const double* V = I.V[s]; const double* W = I.W[s];
  unsigned long long* g = I.minabs;      // [Nx] U, [Ny+1] V, [Nz] W
  unsigned long long mw = CHL_BIG_BITS;
  bool bad = false;                      // a non-finite velocity (|x| bits >= those of inf)
  const int nxr = (Nx + 31) & ~31;       // whole warps take part in the shuffles
  const int nw = nxr * (j1 - j0 + 1);    // a multiple of 32: loop exits are warp-uniform
  // a thread's x is the same in every iteration when the block size is a
  // multiple of the padded row: its U minimum then goes out once at the end
  const bool fixed_x = blockDim.x % nxr == 0;
  unsigned long long mu = CHL_BIG_BITS;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) {
    const int i = w % nxr, jc = j0 + w / nxr;
    const bool ok = i < Nx;
    unsigned long long bv = CHL_BIG_BITS;
    if (ok) {
      const unsigned long long bu = absbits(U[cidx(I, i, jc, k)]);
      const unsigned long long bw = absbits(W[cidx(I, i, jc, k)]);
      bv = absbits(V[vidx(I, i, jc, k)]);
      mu = bu < mu ? bu : mu;
      mw = bw < mw ? bw : mw;
      bad |= (bu >= CHL_BIG_BITS) | (bw >= CHL_BIG_BITS) | (bv >= CHL_BIG_BITS);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long x = __shfl_xor_sync(0xffffffffu, bv, o);
      bv = x < bv ? x : bv;
    }
    if (lane == 0) atomicMin(sv + (jc - j0), bv);
    if (!fixed_x && ok) { atomicMin(g + i, mu); mu = CHL_BIG_BITS; }
  }
  if (fixed_x && (int)(threadIdx.x % nxr) < Nx && (int)threadIdx.x < nw) atomicMin(g + threadIdx.x % nxr, mu);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, mw, o);
    mw = x < mw ? x : mw;
  }
  if (lane == 0) swm[warp] = mw;
  if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(I.status, CHL_STATUS_NONFINITE);
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = swm[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = swm[w] < m ? swm[w] : m;
    atomicMin(g + Nx + Ny + 1 + k, m);
  }
  if (threadIdx.x <= j1 - j0) atomicMin(g + Nx + j0 + threadIdx.x, sv[threadIdx.x]);
  // the instance's last block to finish forms dt from the minima and
  // resets them for the next step
  __shared__ int last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(I.status + CHL_CNT_DT, 1) == I.Nz * nch - 1;
  __syncthreads();
  if (last) {
    __threadfence();
    dt_from_minima(I);
    __syncthreads();
    const int n = Nx + Ny + 1 + I.Nz;
    for (int w = threadIdx.x; w < n; w += blockDim.x) g[w] = CHL_BIG_BITS;
    if (threadIdx.x == 0) I.status[CHL_CNT_DT] = 0;
  }
}

// With a fixed time step the minima are not needed (compute_dt reduces them
// and then replaces dt by -CFL, time_integration.f90:146-148); what the pass
// must still do is flag non-finite velocities.  One thread per centre
// (i, jc, k), jc = 1..Ny, reading the same U, V, W entries as k_minabs.
__global__ void __launch_bounds__(256)
k_nonfinite(ChlMap map, int s) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const long t = (long)lb * blockDim.x + threadIdx.x;
  if (t == 0) chl_put_dt(I.scal, -I.CFL);   // fixed step (compute_dt, time_integration.f90:146-148)
  bool bad = false;
  if (t < (long)Nx * Ny * Nz) {
    const int i = (int)(t % Nx);
    const int jc = 1 + (int)((t / Nx) % Ny);
    const int k = (int)(t / ((long)Nx * Ny));
    const unsigned long long bu = absbits(I.U[s][cidx(I, i, jc, k)]);
    const unsigned long long bv = absbits(I.V[s][vidx(I, i, jc, k)]);
    const unsigned long long bw = absbits(I.W[s][cidx(I, i, jc, k)]);
    bad = (bu >= CHL_BIG_BITS) | (bv >= CHL_BIG_BITS) | (bw >= CHL_BIG_BITS);
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(I.status, CHL_STATUS_NONFINITE);
}

__global__ void k_minabs_init(ChlMap map) {
  chl_pdl_wait();
  const ChlInst& I = map.inst[blockIdx.x];
  const int n = I.Nx + I.Ny + 1 + I.Nz;
  for (int w = threadIdx.x; w < n; w += blockDim.x) I.minabs[w] = CHL_BIG_BITS;
}

// ------------------------------------------------------------ constant mass flow
// compute_dPx_for_constant_mass_flow (mass_flow.f90:113-166) over the unique
// x-z points of rows j_f = 3 and nyg-2, then U += dPdx on the interior
// (time_integration.f90:89-94); one block per instance for the sum.
__global__ void k_massflow(ChlMap map, int s, int force) {
  chl_pdl_wait();
  const ChlInst& I = map.inst[blockIdx.x];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  if (!I.x_mass_cte && !force) {                 // pressure-gradient forcing: no shift
    if (threadIdx.x == 0) I.scal[CHL_S_SHIFT] = 0.0;
    return;
  }
  const double* U = I.U[s];
  double acc = 0.0;
  for (int w = threadIdx.x; w < Nx * Nz; w += blockDim.x) {
    const int i = w % Nx, k = w / Nx;
    acc += 0.5 * (U[cidx(I, i, 2, k)] + U[cidx(I, i, Ny - 1, k)]);
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double d = I.scal[CHL_S_Q0] - red[0] / (double)(Nx * Nz);
    I.scal[CHL_S_SHIFT] = d;
    if (!force) I.scal[CHL_S_DPDX] = 0.0;   // dPdx = 0 after the shift (time_integration.f90:92)
  }
}

__device__ __forceinline__ void time_advance(const ChlInst& I) {
  I.scal[CHL_S_T] = I.scal[CHL_S_T] + 1.0 * I.scal[CHL_S_DT];
}

// The shift of the constant-mass-flow instances, and the time advance of
// every instance (its first block; k_tadvance's work when no instance of
// the batch has a constant mass flow and the shift is not launched).
__global__ void __launch_bounds__(256)
k_shift(ChlMap map, int s) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const unsigned t = (unsigned)lb * blockDim.x + threadIdx.x;
  if (t == 0) {
    time_advance(I);
    // step counter of the wall-model exploration noise (shared by the batch)
    if (blockIdx.x == 0 && I.mlp_cfg) atomicAdd(I.mlp_cfg + 4, 1u);
  }
  if (t >= (unsigned)(Nx * Ny * Nz) || !I.x_mass_cte) return;
  const ChlIdx p = chl_split(t, Nx, Ny);
  const int i = p.i, jc = 1 + p.j, k = p.k;
  double* U = I.U[s];
  const double d = I.scal[CHL_S_SHIFT];
  const double un = U[cidx(I, i, jc, k)] + d;
  U[cidx(I, i, jc, k)] = un;
  if (jc == 1) U[cidx(I, i, 0, k)] = -un;
  if (jc == Ny) U[cidx(I, i, Ny + 1, k)] = -un;
}

// time advance t += dt (compute_time_step_RK3 leaves t = to + rk_t(3)*dt)
__global__ void k_tadvance(ChlMap map) {
  chl_pdl_wait();
  const ChlInst& I = map.inst[blockIdx.x];
  if (threadIdx.x == 0) time_advance(I);
  // step counter of the wall-model exploration noise (shared by the batch)
  if (blockIdx.x == 0 && threadIdx.x == 0 && I.mlp_cfg) atomicAdd(I.mlp_cfg + 4, 1u);
}

// ------------------------------------------------------------ divergence check
// check_divergence (projection.f90:223-245): signed max and max |div| over
// the unique centres.  One block per z plane of every instance writes the
// plane's pair into red[2k], red[2k+1] (the upload's bulk-flow partials,
// free outside chl_upload); k_divmax_final reduces an instance's planes.
__device__ __forceinline__ void block_max2(double& mx, double& ma) {
  __shared__ double r0[256], r1[256];
  r0[threadIdx.x] = mx; r1[threadIdx.x] = ma;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) { r0[threadIdx.x] = fmax(r0[threadIdx.x], r0[threadIdx.x + h]); r1[threadIdx.x] = fmax(r1[threadIdx.x], r1[threadIdx.x + h]); }
    __syncthreads();
  }
  mx = r0[0]; ma = r1[0];
}

__global__ void __launch_bounds__(256) k_divmax_plane(ChlMap map, int s) {
  int k;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, k)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const double *U = I.U[s], *V = I.V[s], *W = I.W[s];
  const double rz = I.rdzc[k];
  const int km = wrap(k - 1, Nz);
  double mx = 0.0, ma = 0.0;
  for (int w = threadIdx.x; w < Nx * Ny; w += blockDim.x) {
    const int i = w % Nx, jc = 1 + w / Nx;
    const double d = (U[cidx(I, i, jc, k)] - U[cidx(I, wrap(i - 1, Nx), jc, k)]) * I.rdxc[i]
                   + (V[vidx(I, i, jc, k)] - V[vidx(I, i, jc - 1, k)]) * I.rdyc[jc]
                   + (W[cidx(I, i, jc, k)] - W[cidx(I, i, jc, km)]) * rz;
    mx = fmax(mx, d); ma = fmax(ma, fabs(d));
  }
  block_max2(mx, ma);
  if (threadIdx.x == 0) { I.red[2 * k] = mx; I.red[2 * k + 1] = ma; }
}

__global__ void __launch_bounds__(256) k_divmax_final(ChlMap map, double* out) {
  const ChlInst& I = map.inst[blockIdx.x];
  double mx = 0.0, ma = 0.0;
  for (int k = threadIdx.x; k < I.Nz; k += blockDim.x) { mx = fmax(mx, I.red[2 * k]); ma = fmax(ma, I.red[2 * k + 1]); }
  block_max2(mx, ma);
  if (threadIdx.x == 0) { out[2 * blockIdx.x] = mx; out[2 * blockIdx.x + 1] = ma; }
}

// ------------------------------------------------------------ initial bulk flow Qflow_x_0
// compute_mean_mass_flow_U (mass_flow.f90:24-61), trapezoid over rows
// j_f = 3..nyg-1 of the unique x-z points; one block per instance.
// one block per z plane: compensated (Kahan) partial sums of the plane
// into red[2k], red[2k+1]; k_qflow_final adds them in plane order
__global__ void k_qflow_part(const ChlInst* inst, int s) {
  const ChlInst& I = *inst;
  const int Nx = I.Nx, Ny = I.Ny, k = blockIdx.x;
  const double* U = I.U[s];
  double q = 0.0, qc = 0.0, n = 0.0, nc = 0.0;
  for (int w = threadIdx.x; w < Nx * (Ny - 1); w += blockDim.x) {
    const int i = w % Nx, jc = 2 + w / Nx;
    const double dyg = I.dyf[jc - 1];          // yg(j)-yg(j-1), j_f = jc+1
    const double y1 = (U[cidx(I, i, jc, k)] + U[cidx(I, i, jc - 1, k)]) * 0.5 * dyg - qc;
    const double t1 = q + y1;
    qc = (t1 - q) - y1; q = t1;
    const double y2 = (1.0 + 1.0) * 0.5 * dyg - nc;
    const double t2 = n + y2;
    nc = (t2 - n) - y2; n = t2;
  }
  __shared__ double r0[256], r1[256];
  r0[threadIdx.x] = q; r1[threadIdx.x] = n;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) { r0[threadIdx.x] += r0[threadIdx.x + h]; r1[threadIdx.x] += r1[threadIdx.x + h]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { I.red[2 * k] = r0[0]; I.red[2 * k + 1] = r1[0]; }
}

__global__ void k_qflow_final(const ChlInst* inst, int slot) {
  const ChlInst& I = *inst;
  double q = 0.0, qc = 0.0, n = 0.0, nc = 0.0;
  for (int k = 0; k < I.Nz; ++k) {
    const double y1 = I.red[2 * k] - qc, t1 = q + y1;
    qc = (t1 - q) - y1; q = t1;
    const double y2 = I.red[2 * k + 1] - nc, t2 = n + y2;
    nc = (t2 - n) - y2; n = t2;
  }
  I.scal[slot] = q / n;
}

// chl_sqrt on given values, for its check against correctly rounded roots
__global__ void k_sqrt_selftest(const double* __restrict__ a, double* __restrict__ y, long n) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) y[t] = chl_sqrt(a[t]);
}

extern "C" {
void chl_launch_sqrt_selftest(const double* a, double* y, long n, cudaStream_t st) {
  if (n > 0) k_sqrt_selftest<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a, y, n);
}
// the minima hold CHL_BIG_BITS between steps: set once here when an
// instance is created, then by the block of k_minabs that forms dt
void chl_launch_minabs_init(const ChlMap& m, cudaStream_t st) {
  chl_launch_pdl(k_minabs_init, dim3(m.n), dim3(128), 0, st, m);
}
// compute_dt: the minima and, in the instance's last block, dt itself
void chl_launch_minabs(const ChlMap& m, int nb, int s, cudaStream_t st) {
  chl_launch_pdl(k_minabs, dim3(nb), dim3(256), 0, st, m, s);
}
// nb: blocks of 256 centres (the point map)
void chl_launch_nonfinite(const ChlMap& m, int nb, int s, cudaStream_t st) {
  chl_launch_pdl(k_nonfinite, dim3(nb), dim3(m.tb), 0, st, m, s);
}
void chl_launch_massflow(const ChlMap& m, cudaStream_t st, int s, int force) { chl_launch_pdl(k_massflow, dim3(m.n), dim3(256), 0, st, m, s, force); }
void chl_launch_shift(const ChlMap& m, int nb, int s, cudaStream_t st) { chl_launch_pdl(k_shift, dim3(nb), dim3(m.tb), 0, st, m, s); }
void chl_launch_tadvance(const ChlMap& m, cudaStream_t st) { chl_launch_pdl(k_tadvance, dim3(m.n), dim3(32), 0, st, m); }
void chl_launch_divmax(const ChlMap& planes, int nplanes, int s, double* out, cudaStream_t st) {
  k_divmax_plane<<<nplanes, 256, 0, st>>>(planes, s);
  k_divmax_final<<<planes.n, 256, 0, st>>>(planes, out);
}
void chl_launch_qflow(const ChlInst* inst, int Nz, int s, int slot, cudaStream_t st) {
  k_qflow_part<<<Nz, 256, 0, st>>>(inst, s);
  k_qflow_final<<<1, 1, 0, st>>>(inst, slot);
}
}
