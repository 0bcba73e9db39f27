// Shared definitions for the GB300 channel-LES kernels.
//
// Data layout (per channel instance, all FP64, x fastest):
//   * x and z are periodic and stored on their unique points only:
//     i in [0,Nx) is Fortran index i_f = i+2 (faces and centres alike),
//     k in [0,Nz) is k_f = k+2.  Face i is the right face of centre i.
//     Neighbours wrap: i-1 of 0 is Nx-1 (the reference's ghost copies,
//     boundary_conditions.f90:60-226).
//   * y is stored with the reference's full extent: centre rows
//     jc in [0,Ny+1] (Fortran j_f = jc+1, rows 0 and Ny+1 are the ghost
//     rows that apply_Dirichlet_bc_y keeps at minus the first interior row)
//     and face rows jv in [0,Ny] (Fortran j_f = jv+1, rows 0 and Ny are the
//     walls).  Centre row jc lies between face rows jc-1 and jc.
//   * a centre field has Ny+2 rows: index i + Nx*(jc + (Ny+2)*k);
//     U and W are stored the same way; V has Ny+1 rows.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define CHL_NQ 18   // filtered DSM components
#define CHL_WALL_THREADS 32   // block width of the equilibrium wall-stress solve (one warp)
// SMs of a GB300.  The small transforms are cut finer until their grid
// covers the SMs about four times: with about one block per SM a few SMs
// run two, and the launch takes twice one block's time.
#define CHL_SMS 152
#define CHL_MIN_BLOCKS (4 * CHL_SMS)
#define CHL_FFT_MIN_BLOCKS CHL_MIN_BLOCKS
// Lanes sharing one mode's tridiagonal column (k_tri_scan).  The split
// pays only where the whole solve is a few hundred serial chains; it costs
// about twice the FP64 work, which a batch that fills the GPU would feel.
// So: 1 for instances of CHL_TRI_SPLIT_MODES modes or more, else doubled
// up to 8 while the instance has fewer than CHL_MIN_BLOCKS x 32 mode-lanes
// and every lane keeps at least two rows.  A function of the instance's own
// extents only, like chl_dsm_ppt.
#define CHL_TRI_SPLIT_MODES 1024
__host__ __device__ inline int chl_tri_lanes(long modes, int Ny) {
  int P = 1;
  if (modes >= CHL_TRI_SPLIT_MODES) return 1;
  while (P < 8 && modes * P < (long)CHL_MIN_BLOCKS * 32 && Ny >= 4 * P) P *= 2;
  return P;
}
// x-z points per thread of the DSM plane sums (k_dsm_final, blocks of
// CHL_DSMF_THREADS): 4, halved while the instance's Ny x chunks grid would
// have fewer than CHL_MIN_BLOCKS blocks.  A large instance has chunks of 256
// points (192 per plane at 256x192); a 32x48x32 channel gets 768 blocks of
// one point per thread, 5 per SM, where 256-thread blocks left 2 blocks on
// some SMs and 1 on most.  A function of the instance's own extents only,
// so an instance sums its planes in the same order alone and in a batch.
// Stockham FFT passes (chl_fft.cu): radix 4 while the remaining length
// allows, then 3, then 2.  Each pass with twiddles (sub-transform size
// Ns > 1) has CHL_TW_F fields of Ns doubles in the length's pass table.
#define CHL_TW_F 7
__host__ __device__ inline int chl_fft_radix(int rem) { return rem % 4 == 0 ? 4 : (rem % 3 == 0 ? 3 : 2); }
__host__ __device__ inline int chl_tw_len(int N) {
  int Ns = 1, rem = N, len = 0;
  while (rem > 1) {
    const int R = chl_fft_radix(rem);
    if (Ns > 1) len += CHL_TW_F * Ns;
    Ns *= R; rem /= R;
  }
  return len;
}
// bytes of a pass table in shared memory, kept a multiple of 16
__host__ __device__ inline size_t chl_tw_bytes(int len) { return ((size_t)len * 8 + 15) & ~(size_t)15; }

#define CHL_DSMF_THREADS 64
// Points of one plane sum: the Nx x Nz plane, then the reference's
// duplicated periodic column (i = 0, every k) and plane (k = 0, every i) and
// one more (0, 0) - its weights 2 and 4 as extra points of weight 1.
__host__ __device__ inline int chl_dsm_points(int Nx, int Nz) { return Nx * Nz + Nx + Nz + 1; }
__host__ __device__ inline int chl_dsm_ppt(int Nx, int Ny, int Nz) {
  const int n = chl_dsm_points(Nx, Nz);
  int ppt = 4;
  while (ppt > 1 && (long)Ny * ((n + CHL_DSMF_THREADS * ppt - 1) / (CHL_DSMF_THREADS * ppt)) < CHL_MIN_BLOCKS)
    ppt >>= 1;
  return ppt;
}
// complex rows (pairs of real x lines) per x-transform block: up to
// 1024/Nx, halved while the instance's grid would have fewer than
// min_blocks blocks (CHL_FFT_MIN_BLOCKS unless the tuner chose another)
__host__ __device__ inline int chl_fftx_rows(int Nx, int nrow, int min_blocks) {
  int cr = 1024 / Nx;
  if (cr < 1) cr = 1;
  while (cr > 1 && (nrow + cr - 1) / cr < min_blocks) cr >>= 1;
  return cr;
}
// threads of a transform block staging `lines` lines of length n: one
// radix-4 butterfly each per pass, in whole warps, 64..256
__host__ __device__ inline int chl_fft_threads(int lines, int n) {
  int t = (lines * n / 4 + 31) & ~31;
  return t < 64 ? 64 : (t > 256 ? 256 : t);
}
#ifndef CHL_TRI_SMEM_MAX
#define CHL_TRI_SMEM_MAX (128 * 1024)   // largest staged tridiagonal column block
#endif

// Constants that the FP64 kernels take as register operands (F64 below);
// held in each instance's descriptor in device memory, set by the host.
enum { FK_ONE = 0, FK_MZERO, FK_FOUR, FK_NSLOT };

struct ChlInst {
  double fk[FK_NSLOT];          // 1, -0, 4 (FK_*)
  int Nx, Ny, Nz, Nxh;          // unique cells; Nxh = Nx/2+1
  int LES_model, Dirichlet_nu_t, wall_model, x_mass_cte;
  double nu, CFL, Cs;
  double dxmin, dymin, dzmin;   // initialization.f90:233-235
  double dt_vis;                // viscous limit of compute_dt, min(CFL d^2/nu) over x, y, z (host-formed)
  double dyw;                   // yg(2)-yg(1), used for both walls (wallmodel.f90:32-35)
  double hb, ht;                // matching heights of the log-law wall model
  double cbc1, cbc2;            // coef_bc_1*(yg(2)-yg(1)), coef_bc_2*(yg(nyg)-yg(nyg-1))
  double ybot, ytop;            // y(1), y(ny)
  double dy1;                   // y(2)-y(1) (nu_t ghost rule 2 of AMD and Vreman)
  double gb1, gb2, gt1, gt2;    // pressure-BC metric factors g, g2 (pressure.f90:282-316)
  double dygb, dygt;            // yg(2)-yg(1), yg(nyg)-yg(nyg-1)
  double mass_norm;             // 1/(Nx*Nz)
  // geometry (reciprocal spacings; see chl_host.cpp for the exact list)
  const double *rdxc, *rdxf, *rdyc, *rdyf, *rdzc, *rdzf;
  const double *dxf, *dyf, *dzf;  // raw spacings (dt)
  const double *hx2, *hy2, *hz2;  // squared centre widths (x(i)-x(i-1))^2 etc. (Vreman)
  const double *w0x2, *w1x2;      // 2 x weight_y_0/1 by face row jv
  const double *w0, *w1;          // weight_y_0/1 by face row jv (w1 = 1 - w0)
  const double *rdxc4, *rdyc4, *rdzc4;   // 4 x rdxc, rdyc, rdzc (centre fluxes, kept 4 x)
  const double *rdxc2, *rdyc2, *rdzc2;   // 2 x rdxc, rdyc, rdzc (xy and yz edge fluxes, kept 2 x)
  // sqrt(4/216) x rdxc, rdyc, rdzc and rdxf, rdyf, rdzf: the dynamic model's
  // filtered strain, whose M_ij term needs 4/216 x |S| S_ij
  const double *rdxcs, *rdycs, *rdzcs, *rdxfs, *rdyfs, *rdzfs;
  const double *ygc;              // yg(1..nyg), centre y coordinates with the ghost rows
  const double *smag_csdelta;     // Cs*Delta_j by centre row (static Smagorinsky)
  const double *smag_dwall;       // distance of centre row to the nearer wall (van Driest)
  // Fourier / tridiagonal
  const double *twx, *twz;        // pass tables of the x and z transforms (chl_tw_len doubles)
  const double *tri_inv, *tri_m, *tri_c;   // [Ny][Nz][Nxh] Thomas factors
  // state: three velocity sets (start-of-step / stage 1 / stage 2)
  double *U[3], *V[3], *W[3];
  double *F1[3];                  // stage-1 RHS (kept for stages 2 and 3)
  double *Fp[3];                  // RHS for the actual pressure
  double *nut, *S;                // nu + nu_t (Ny+2 rows), |S| (Ny+2 rows)
  double *G[9];                   // momentum face fluxes (chl_rhs.cu)
  double *q[CHL_NQ], *r[CHL_NQ];  // DSM filter ping-pong
  double *E[3];                   // edge fields (S12, S13, S23 numerators)
  double2 *spec;                  // [Ny+2][Nz][Nxh] spectra (rows 1..Ny used)
  double *p;                      // pseudo-pressure (centres)
  double *P;                      // actual pressure (centres)
  double *alpha;                  // wall stress [2][Nz][Nx]
  double *bc;                     // pressure BC planes [2][Nz][Nx]
  double *part;                   // DSM plane partial sums [2][Ny+2][npart][CHL_DSMF_THREADS]
  int npart, dsm_ppt;             // chunks per plane, points per thread (chl_dsm_ppt)
  double *coef;                   // nu_t coefficient per centre row [Ny+2]
  double *scal;                   // device scalars (CHL_S_*)
  unsigned long long *minabs;     // [Nx+1 | Nz] min |u| bit patterns (dt)
  double *red;                    // plane partials [2][Nz]: bulk flow (upload), divergence check
  int *status;                    // device status word (0 ok); [CHL_CNT_DT] block counter of k_minabs
  int *dsm_cnt;                   // [Ny+2] block counters of the DSM plane sums per centre row
  // learned wall model (chl_mlp.cu)
  double retau;                   // nominal Re_tau of the instance (feature ln(h Re_tau))
  float *mlp_trace;               // policy-gradient trace of this instance (4545)
  const float *mlp_theta;         // network parameters, shared by the batch (4545)
  unsigned int *mlp_cfg;          // shared: sigma bits, train, seed lo/hi, evaluation counter,
                                  //   record flag, withheld-commit poll limit (chl_mlp_debug),
                                  //   shared-exploration flag (chl_mlp_set_exploration)
  float *mlp_rec;                 // [3 stages][2 Nx Nz][8] per-point record (chl_mlp_debug), or null
};

// FP64 issue forms.  In a throughput loop on GB300 an FP64 FMA whose
// operands are all registers issues at 1.91 per clock per SM, while DADD,
// DMUL and any FP64 instruction with a literal operand issue at 1.61.  Sums,
// differences and products can be issued as register FMAs:
// a + b = fma(a, 1, b), a - b = fma(a, 1, -b), a b = fma(a, b, -0).  Each is
// exact (a times 1 is a, adding -0 leaves a product unchanged, signed zeros
// included), so the results are bit-identical to the plain operators.  The 1,
// the -0 and the 4 are read from the instance descriptor in device memory, so
// they reach the instructions as registers.  Used where it measured faster:
// the filter passes, the edge strains and the stage update; the flux, strain
// and L:M kernels and the transforms measured no faster (or slower) with it.
struct F64 {
  double one, mz;
  __device__ __forceinline__ double add(double a, double b) const { return fma(a, one, b); }
  __device__ __forceinline__ double sub(double a, double b) const { return fma(a, one, -b); }
  __device__ __forceinline__ double mul(double a, double b) const { return fma(a, b, mz); }
};
__device__ __forceinline__ F64 f64_of(const ChlInst& I) { return F64{I.fk[FK_ONE], I.fk[FK_MZERO]}; }

// fmax(x, 0.0) on the integer pipe: x where its bit pattern is that of a
// positive finite number or +inf, else +0 (negative numbers, zeros and NaN,
// for which fmax returns its other operand, 0).  The FP64 pipe, which bounds
// the per-point kernels, would otherwise spend an instruction on the clip.
__device__ __forceinline__ double chl_pos(double x) {
  long long r;
  asm("{\n\t.reg .pred p;\n\t"
      "setp.gt.s64 p, %1, 0;\n\t"
      "setp.le.and.s64 p, %1, 0x7FF0000000000000, p;\n\t"
      "selp.b64 %0, %1, 0, p;\n\t}"
      : "=l"(r) : "l"(__double_as_longlong(x)));
  return __longlong_as_double(r);
}

// max(x, lo) for lo > 0 on the integer pipe: x where its bit pattern lies in
// [bits(lo), bits(+inf)] (for non-negative numbers the order of the bit
// patterns is the order of the values), else lo - also for a NaN x.
__device__ __forceinline__ double chl_atleast(double x, double lo) {
  long long r;
  asm("{\n\t.reg .pred p;\n\t"
      "setp.ge.s64 p, %1, %2;\n\t"
      "setp.le.and.s64 p, %1, 0x7FF0000000000000, p;\n\t"
      "selp.b64 %0, %1, %2, p;\n\t}"
      : "=l"(r) : "l"(__double_as_longlong(x)), "l"(__double_as_longlong(lo)));
  return __longlong_as_double(r);
}

// Square root for the per-point strain magnitudes: Heron's iteration
// x <- x + (a - x^2) / (2x), in the coupled form with a reciprocal square
// root y ~ 1/sqrt(a) (Markstein, IBM J. Res. Dev. 34 (1990) 111), seeded by
// the GPU's approximate reciprocal square root (rsqrt.approx.f64, relative
// error below 2^-20): x = a y, then twice x += (a - x^2) y/2.  The error
// after the first step is about (2^-20)^2, after the second below an ulp.
// Five FP64-pipe instructions (one multiply, four FMAs) against eight for
// the correctly rounded sqrt(), and within one ulp of it
// (chl_sqrt_selftest).  y/2 is an exponent decrement on the integer pipe.
// Only positive normal a take this path (one unsigned compare); zero,
// subnormal, negative, infinite and NaN a go to sqrt(), so every special
// case is IEEE's (a negative argument gives NaN, as the reference's ** 0.5).
// The special arguments' sqrt() is a call, not inlined: inlined, the
// compiler may predicate its instructions into the common path, where every
// warp would issue them.
static __device__ __noinline__ double chl_sqrt_special(double a) { return sqrt(a); }
__device__ __forceinline__ double chl_sqrt(double a) {
  const unsigned long long ub = (unsigned long long)__double_as_longlong(a);
  if (ub - (1ULL << 52) >= 0x7FF0000000000000ULL - (1ULL << 52)) return chl_sqrt_special(a);
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(a));
  const double h = __longlong_as_double(__double_as_longlong(y) - (1LL << 52));
  double x = a * y;
  double r = fma(-x, x, a);
  x = fma(r, h, x);
  r = fma(-x, x, a);
  return fma(r, h, x);
}

// device scalar slots
enum {
  CHL_S_DT = 0, CHL_S_T, CHL_S_DPDX, CHL_S_Q0, CHL_S_SHIFT, CHL_S_DIVMAX,
  CHL_S_DC,            // 6 slots: dt c1 / 4, dt c2 / 4 of RK3 stages 0, 1, 2
  CHL_S_NSCAL = 16
};

// Stage coefficients of compute_time_step_RK3 (time_integration.f90:42-81):
// stage s writes U^n + dt (c1 F(U^n) + c2 F(stage input)).
__host__ __device__ inline double chl_rk_c1(int s) { return s == 0 ? 0.0 : 1.0 / 4.0; }
__host__ __device__ inline double chl_rk_c2(int s) { return s == 0 ? 8.0 / 15.0 : (s == 1 ? 5.0 / 12.0 : 3.0 / 4.0); }

// Writes dt and the stage products dt c / 4 that the stage update reads
// (its fluxes are 4 x), so that no grid point forms them.  Every writer of
// the step size goes through here.
__host__ __device__ inline void chl_put_dt(double* scal, double dt) {
  scal[CHL_S_DT] = dt;
  for (int s = 0; s < 3; ++s) {
    scal[CHL_S_DC + 2 * s] = dt * (0.25 * chl_rk_c1(s));
    scal[CHL_S_DC + 2 * s + 1] = dt * (0.25 * chl_rk_c2(s));
  }
}

// block -> instance map shared by all multi-instance kernels
// One field of a three-field layout conversion: the Fortran-layout array
// (in the staging area) with its extents n1 x n2 x n3, the device field with
// nrow stored y rows, and the unpack rule (0 U/W-like, 1 V-like).
struct ChlField1 {
  double* fort;
  double* dev;
  int n1, n2, n3, nrow, kind;
};
struct ChlFields3 { ChlField1 f[3]; };

struct ChlMap {
  const ChlInst* inst;   // device array of instances
  const int* off;        // prefix sum of blocks per instance, off[n] = total
  int n;
  int tb;                // threads per block of the one-thread-per-point maps (tuned)
};

__device__ __forceinline__ int chl_find(const ChlMap& m, int b, int& local) {
  int lo = 0, hi = m.n - 1;
  while (lo < hi) {                 // last instance with off[idx] <= b
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(m.off + mid) <= b) lo = mid; else hi = mid - 1;
  }
  local = b - __ldg(m.off + lo);
  return lo;
}

// (i, j, k) of point t of an Nx x rows x Nz block, x fastest, in 32-bit
// unsigned arithmetic (an instance has fewer than 2^31 points, checked at
// creation): the 64-bit divisions this replaces were long integer sequences
// ahead of every kernel's first load.
struct ChlIdx { int i, j, k; };
__device__ __forceinline__ ChlIdx chl_split(unsigned t, unsigned Nx, unsigned rows) {
  const unsigned q = t / Nx, k = q / rows;
  return ChlIdx{(int)(t - q * Nx), (int)(q - k * rows), (int)k};
}
__device__ __forceinline__ int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// Status word bits of an instance: 1 non-finite velocity (k_minabs),
// 4 an index outside the field (bounds-checked build only).
#define CHL_STATUS_NONFINITE 1
#define CHL_STATUS_BOUNDS 4
// slot of the status area that counts k_minabs's finished blocks (the last
// one forms dt); the counters return to 0 after each use
#define CHL_CNT_DT 4

// The bounds-checked build (-DCHL_BOUNDS_CHECK, build.build(variant="bounds"))
// records an out-of-range index in the status word and clamps it, so the
// access stays inside the field.
__device__ __forceinline__ void chl_clamp(const ChlInst& I, int& i, int& j, int& k, int jmax) {
#ifdef CHL_BOUNDS_CHECK
  if (i < 0 || i >= I.Nx || j < 0 || j > jmax || k < 0 || k >= I.Nz) {
    atomicOr(I.status, CHL_STATUS_BOUNDS);
    i = min(max(i, 0), I.Nx - 1); j = min(max(j, 0), jmax); k = min(max(k, 0), I.Nz - 1);
  }
#else
  (void)I; (void)i; (void)j; (void)k; (void)jmax;
#endif
}

__device__ __forceinline__ size_t cidx(const ChlInst& I, int i, int jc, int k) {
  chl_clamp(I, i, jc, k, I.Ny + 1);
  return (size_t)i + (size_t)I.Nx * ((size_t)jc + (size_t)(I.Ny + 2) * (size_t)k);
}
__device__ __forceinline__ size_t vidx(const ChlInst& I, int i, int jv, int k) {
  chl_clamp(I, i, jv, k, I.Ny);
  return (size_t)i + (size_t)I.Nx * ((size_t)jv + (size_t)(I.Ny + 1) * (size_t)k);
}

#define LDG(p) __ldg(p)

// wall-model eddy viscosity at the x face a of a wall: tau / (dU/dy) - nu
// with dU/dy = (U(wall row) - U(ghost row)) / dyw (one division)
// (compute_wall_model, wallmodel.f90:23-46)
__device__ __forceinline__ double wm_face(const ChlInst& I, const double* U, int a, int k, int wall) {
  const double al = I.alpha[(size_t)wall * I.Nx * I.Nz + (size_t)k * I.Nx + a];
  const double du = wall == 0 ? U[cidx(I, a, 1, k)] - U[cidx(I, a, 0, k)]
                              : U[cidx(I, a, I.Ny, k)] - U[cidx(I, a, I.Ny + 1, k)];
  return al * I.dyw / du - I.nu;
}

// The ghost-row value of nu_t next to a wall from the clipped value v of the
// first interior row: Neumann (copy), Dirichlet (mirror), or for AMD and
// Vreman the mirror plus 2*0.38*dPdx^0.5*(y(2)-y(1))/2 (subgrid.f90:858-871,
// 991-1002).
__device__ __forceinline__ double nut_ghost(const ChlInst& I, double v) {
  if (I.Dirichlet_nu_t == 1) return -v;
  if (I.Dirichlet_nu_t == 2 && I.LES_model >= 3) return -v + 2.0 * 0.38 * sqrt(I.scal[CHL_S_DPDX]) * I.dy1 / 2.0;
  return v;
}

// Programmatic dependent launch inside the step graph: each step kernel is
// launched with programmatic stream serialisation, so its blocks may be
// scheduled while the previous kernel drains, and waits here, first thing,
// until that kernel has finished and its writes are visible.  Without the
// launch attribute the wait returns at once.
__device__ __forceinline__ void chl_pdl_wait() {
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 900)
  cudaGridDependencySynchronize();
#endif
}

template <typename... KArgs, typename... Args>
inline cudaError_t chl_launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                  Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid; cfg.blockDim = block; cfg.dynamicSmemBytes = smem; cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at; cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
