// Fractional-step projection: divergence, 2-D Fourier transform in x and z,
// one tridiagonal solve in y per wavenumber pair, inverse transform and the
// velocity correction.  Restates compute_projection_step
// (projection.f90:20-214) and, for the actual pressure, the right-hand side
// and solver that compute_pressure (pressure.f90:21-29) calls
// (pressure.f90:42-172).
//
// The reference transforms each y-plane with FFTW-MPI and calls LAPACK
// zgtsv per mode.  Here:
//  * x: two real rows are packed as one complex row, transformed by a
//    shared-memory Stockham FFT (radix 4/3/2) and split into two
//    half-spectra (kx = 0..Nx/2) - fused with the divergence that produces
//    the rows;
//  * z: complex columns of the half-spectrum, staged 16 kx-columns at a time
//    in shared memory;
//  * y: one thread per mode runs the Thomas elimination with factors
//    precomputed once per grid (the matrix of a mode never changes between
//    steps), into which the 1/(Nx*Nz) of the inverse transform and the 2 of
//    the real-row packing are folded; the mode's column is staged in shared
//    memory by asynchronous copies when it fits;
//  * the inverse runs the same way back and the x pass writes the pressure.
#include "chl_common.cuh"

#include <cooperative_groups.h>

// ------------------------------------------------------------ Stockham passes
// Data of `nrows` transforms of length N; element e of row r is at
// r*rs + e*es.  One pass of radix R with sub-transform size Ns.
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

template <int R>
__device__ __forceinline__ void dft_small(double2* v, bool inv) {
  if (R == 2) {
    const double2 a = v[0], b = v[1];
    v[0] = cadd(a, b); v[1] = csub(a, b);
  } else if (R == 4) {
    const double2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    const double2 c = cadd(v[1], v[3]), e = csub(v[1], v[3]);
    // d = e * (-i) forward, e * (+i) inverse
    const double2 d = inv ? make_double2(-e.y, e.x) : make_double2(e.y, -e.x);
    v[0] = cadd(a, c); v[2] = csub(a, c);
    v[1] = cadd(b, d); v[3] = csub(b, d);
  } else if (R == 3) {
    const double s3 = 0.86602540378443864676;   // sin(2 pi/3)
    const double2 s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
    const double2 t = make_double2(fma(-0.5, s.x, v[0].x), fma(-0.5, s.y, v[0].y));
    // forward: out1 = t - i s3 d, out2 = t + i s3 d (inverse swaps)
    const double2 m = inv ? make_double2(-s3 * d.y, s3 * d.x) : make_double2(s3 * d.y, -s3 * d.x);
    v[0] = cadd(v[0], s);
    v[1] = cadd(t, m);
    v[2] = csub(t, m);
  }
}

// Twiddle multiplications in tangent form (E. Linzer and E. Feig, Modified
// FFTs for fused multiply-add architectures, Math. Comp. 60 (1993) 347): a
// twiddle w = C + iS
// is kept as a scale sigma and a multiplier m with |m| <= 1 - sigma = C,
// m = S/C where |C| >= |S|, else sigma = S, m = C/S - so v w = sigma y with
// y two FMAs away from v, and each sigma is folded into an FMA of the
// butterfly instead of costing a multiplication.  A radix-4 butterfly with
// twiddles then takes 22 FP64 instructions instead of 28, a radix-3 one 16
// instead of 22, a radix-2 one 6 instead of 8.  The choice of form and the
// sign flips of the inverse transform (conjugate twiddles) are integer
// operations on bit patterns, which the FP64-bound passes get for free.
//
// Pass table of a length N, per pass with twiddles (sub-transform size
// Ns > 1, radix R), CHL_TW_F fields of Ns entries, entry jm being the
// butterflies j with j mod Ns = jm (twiddles w_r = exp(-2 pi i jm r/(Ns R)),
// r = 1..R-1, in the forward direction):
//   0 m1, 1 m2, 2 m3 (radix 4) or sin(2 pi/3) sigma1 (radix 3), 3 sigma1,
//   4 sigma2 (radix 4) or sigma1 / 2 (radix 3), 5 sigma3/sigma1 (radix 4)
//   or sigma2/sigma1 (radix 3), 6 form bits (bit r set: w_r in the S form),
//   stored as the bit pattern of a double.
// The sign flips and operand selects are inline PTX: written as C++ the
// compiler folds "FMA of two selects on one condition" into two FMAs and a
// select, which doubles the FP64 work these forms exist to save.
__device__ __forceinline__ double flip(double x, unsigned f) {
  long long r;
  asm("{\n\t.reg .b64 t;\n\tcvt.u64.u32 t, %2;\n\tshl.b64 t, t, 63;\n\txor.b64 %0, %1, t;\n\t}"
      : "=l"(r) : "l"(__double_as_longlong(x)), "r"(f));
  return __longlong_as_double(r);
}
// v w / sigma: (a - b m, b + a m) in the C form, (a m - b, b m + a) =
// (-(b - a m), a + b m) in the S form.  With (p, q) = (b, a) in the C form
// and (a, b) in the S form both are (+/- fma(p, -m, q), fma(q, m, p)): two
// selects and, in the S form, a sign flip of the first component.  The flip
// XORs a mask chosen between 0 and sgn, the bit pattern of -0.0 read from
// device memory: were the mask visibly the sign bit, ptxas would turn the
// flip into a pair of predicated FMAs, one per form, and every warp would
// issue both.
__device__ __forceinline__ double2 tw_apply(double2 v, double m, unsigned sform, long long sgn) {
  long long p, q, t;
  asm("{\n\t.reg .pred s;\n\t"
      "setp.ne.u32 s, %5, 0;\n\t"
      "selp.b64 %0, %3, %4, s;\n\t"     // p = S form ? a : b
      "selp.b64 %1, %4, %3, s;\n\t"     // q = S form ? b : a
      "selp.b64 %2, %6, 0, s;\n\t}"     // t = S form ? sgn : 0
      : "=l"(p), "=l"(q), "=l"(t)
      : "l"(__double_as_longlong(v.x)), "l"(__double_as_longlong(v.y)), "r"(sform), "l"(sgn));
  const double P = __longlong_as_double(p), Q = __longlong_as_double(q);
  return make_double2(__longlong_as_double(__double_as_longlong(fma(P, -m, Q)) ^ t), fma(Q, m, P));
}
__device__ __forceinline__ double2 fma2(double s, double2 y, double2 v) {
  return make_double2(fma(s, y.x, v.x), fma(s, y.y, v.y));
}

// Work items (row, butterfly j) are numbered so that consecutive threads
// touch neighbouring shared-memory words: j fastest when a row is contiguous
// (es = 1, the x lines), the row fastest when rows are interleaved (rs = 1,
// the z columns), which keeps the 16-byte accesses free of bank conflicts.
// tab: this pass's table (Ns > 1), staged in shared memory by the caller.
// TW: the pass has twiddles (Ns > 1) - a template parameter, not a branch
// on Ns inside the loop: ptxas predicates both sides of such a branch, and
// a predicated-off FP64 instruction still takes its turn on the FP64 pipe
// (measured: 2 extra instructions per complex point over a 128-point
// transform).
// INV (the inverse transform) likewise: a runtime direction would put
// predicated sign flips into every butterfly.
template <int R, bool TW, bool INV>
__device__ void stockham_pass(const double2* __restrict__ x, double2* __restrict__ y, int nrows, int rs, int es,
                              int N, int Ns, const double* __restrict__ tab, long long sgn) {
  const int nb = N / R;
  const bool rowfast = rs < es;
  constexpr unsigned iv = INV ? 1u : 0u;
  for (int w = threadIdx.x; w < nrows * nb; w += blockDim.x) {
    int row, j;
    if (rowfast) { j = w / nrows; row = w - j * nrows; }
    else { row = w / nb; j = w - row * nb; }
    const double2* xr = x + (size_t)row * rs;
    double2* yr = y + (size_t)row * rs;
    const int jm = j % Ns;
    double2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = xr[(j + r * nb) * es];
    if (!TW) {
      dft_small<R>(v, INV);
    } else {
      const unsigned fb = (unsigned)__double_as_longlong(tab[6 * Ns + jm]);
      const unsigned f1 = (fb >> 1) & 1u, f2 = (fb >> 2) & 1u;
      const double s1 = flip(tab[3 * Ns + jm], iv & f1);
      const double2 y1 = tw_apply(v[1], flip(tab[jm], iv), f1, sgn);
      if (R == 2) {
        const double2 v0 = v[0];
        v[0] = fma2(s1, y1, v0);
        v[1] = fma2(-s1, y1, v0);
      } else if (R == 4) {
        const unsigned f3 = (fb >> 3) & 1u;
        const double2 y2 = tw_apply(v[2], flip(tab[Ns + jm], iv), f2, sgn);
        const double2 y3 = tw_apply(v[3], flip(tab[2 * Ns + jm], iv), f3, sgn);
        const double s2 = flip(tab[4 * Ns + jm], iv & f2);
        const double rho = flip(tab[5 * Ns + jm], iv & (f1 ^ f3));
        const double2 a = fma2(s2, y2, v[0]), b = fma2(-s2, y2, v[0]);
        const double2 c = fma2(rho, y3, y1), e = fma2(-rho, y3, y1);
        // (v1 w1 - v3 w3) times -i (forward) or +i (inverse) is s1 e times it
        const double si = flip(s1, iv);
        v[0] = fma2(s1, c, a);
        v[2] = fma2(-s1, c, a);
        v[1] = make_double2(fma(si, e.y, b.x), fma(-si, e.x, b.y));
        v[3] = make_double2(fma(-si, e.y, b.x), fma(si, e.x, b.y));
      } else {   // R == 3
        const double2 y2 = tw_apply(v[2], flip(tab[Ns + jm], iv), f2, sgn);
        const double h1 = flip(tab[4 * Ns + jm], iv & f1);
        const double rho = flip(tab[5 * Ns + jm], iv & (f1 ^ f2));
        // forward: out1,2 = t -/+ i sin(2pi/3) (v1 w1 - v2 w2); inverse +/-
        const double k1 = flip(tab[2 * Ns + jm], iv & (f1 ^ 1u));
        const double2 sp = fma2(rho, y2, y1), dp = fma2(-rho, y2, y1);
        const double2 v0 = v[0];
        const double2 t = fma2(-h1, sp, v0);
        v[0] = fma2(s1, sp, v0);
        v[1] = make_double2(fma(k1, dp.y, t.x), fma(-k1, dp.x, t.y));
        v[2] = make_double2(fma(-k1, dp.y, t.x), fma(k1, dp.x, t.y));
      }
    }
    const int idxD = (j / Ns) * Ns * R + jm;
#pragma unroll
    for (int r = 0; r < R; ++r) yr[(idxD + r * Ns) * es] = v[r];
  }
}

// Copies a length's pass table (len doubles) into shared memory; the first
// barrier of fft_smem orders it before any use.
__device__ __forceinline__ void stage_twiddles(double* tws, const double* __restrict__ tab, int len) {
  for (int w = threadIdx.x; w < len; w += blockDim.x) tws[w] = LDG(tab + w);
}

// Full transform; returns the buffer holding the result (a or b).  tab: the
// length's pass table in shared memory (stage_twiddles); sgn: the bit
// pattern of -0.0 from the instance's constants (see tw_apply).
template <bool INV>
__device__ double2* fft_smem_dir(double2* a, double2* b, int nrows, int rs, int es, int N,
                                 const double* tab, long long sgn) {
  int Ns = 1, rem = N, off = 0;
  double2 *src = a, *dst = b;
  while (rem > 1) {
    __syncthreads();
    const int R = chl_fft_radix(rem);
    const double* tp = tab + off;
    if (R == 4) {
      if (Ns == 1) stockham_pass<4, false, INV>(src, dst, nrows, rs, es, N, Ns, tp, sgn);
      else stockham_pass<4, true, INV>(src, dst, nrows, rs, es, N, Ns, tp, sgn);
    } else if (R == 3) {
      if (Ns == 1) stockham_pass<3, false, INV>(src, dst, nrows, rs, es, N, Ns, tp, sgn);
      else stockham_pass<3, true, INV>(src, dst, nrows, rs, es, N, Ns, tp, sgn);
    } else {
      if (Ns == 1) stockham_pass<2, false, INV>(src, dst, nrows, rs, es, N, Ns, tp, sgn);
      else stockham_pass<2, true, INV>(src, dst, nrows, rs, es, N, Ns, tp, sgn);
    }
    if (Ns > 1) off += CHL_TW_F * Ns;
    Ns *= R; rem /= R;
    double2* t = src; src = dst; dst = t;
  }
  __syncthreads();
  return src;
}
__device__ __forceinline__ double2* fft_smem(double2* a, double2* b, int nrows, int rs, int es, int N,
                                             const double* tab, bool inv, long long sgn) {
  return inv ? fft_smem_dir<true>(a, b, nrows, rs, es, N, tab, sgn)
             : fft_smem_dir<false>(a, b, nrows, rs, es, N, tab, sgn);
}


// ------------------------------------------------------------ divergence + forward x
// mode 0: div of velocity set s_in (compute_pseudo_pressure_rhs, projection.f90:40-55)
// mode 1: div of the actual-pressure RHS Fp with the wall rows of Fv set to
//         the pressure BC planes and the BC source terms of pressure.f90:138-139.
__global__ void __launch_bounds__(256)
k_div_fftx(ChlMap map, int s_in, int mode, int xmb) {
  chl_pdl_wait();
  extern __shared__ double2 sm[];
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz, Nxh = I.Nxh;
  const int nrow = Ny * (Nz / 2);
  const int CR = chl_fftx_rows(Nx, nrow, xmb);
  const int g0 = lb * CR;
  const int cr_n = min(CR, nrow - g0);
  double2* A = sm;
  double2* B = sm + CR * Nx;
  double* T = reinterpret_cast<double*>(sm + 2 * CR * Nx);   // pass table
  stage_twiddles(T, I.twx, chl_tw_len(Nx));
  const double *U, *V, *W;
  if (mode == 0) { U = I.U[s_in]; V = I.V[s_in]; W = I.W[s_in]; }
  else { U = I.Fp[0]; V = I.Fp[1]; W = I.Fp[2]; }
  for (int w = threadIdx.x; w < cr_n * Nx; w += blockDim.x) {
    const int cr = w / Nx, i = w - cr * Nx;
    const int g = g0 + cr;
    const int jc = 1 + g / (Nz / 2), k0 = 2 * (g % (Nz / 2));
    const int im = wrap(i - 1, Nx);
    double dv[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = k0 + h, km = wrap(k - 1, Nz);
      double vlo = LDG(V + vidx(I, i, jc - 1, k)), vhi = LDG(V + vidx(I, i, jc, k));
      if (mode == 1) {
        if (jc == 1) vlo = I.bc[(size_t)k * Nx + i];
        if (jc == Ny) vhi = I.bc[(size_t)Nx * Nz + (size_t)k * Nx + i];
      }
      double d = (LDG(U + cidx(I, i, jc, k)) - LDG(U + cidx(I, im, jc, k))) * LDG(I.rdxc + i)
               + (vhi - vlo) * LDG(I.rdyc + jc)
               + (LDG(W + cidx(I, i, jc, k)) - LDG(W + cidx(I, i, jc, km))) * LDG(I.rdzc + k);
      if (mode == 1) {
        if (jc == 1) d += I.cbc1 * I.bc[(size_t)k * Nx + i];
        if (jc == Ny) d -= I.cbc2 * I.bc[(size_t)Nx * Nz + (size_t)k * Nx + i];
      }
      dv[h] = d;
    }
    A[cr * Nx + i] = make_double2(dv[0], dv[1]);
  }
  double2* res = fft_smem(A, B, cr_n, Nx, 1, Nx, T, false, __double_as_longlong(I.fk[FK_MZERO]));
  // split the packed spectrum into the two half-spectra (each times 2)
  for (int w = threadIdx.x; w < cr_n * Nxh; w += blockDim.x) {
    const int cr = w / Nxh, kx = w - cr * Nxh;
    const int g = g0 + cr;
    const int jc = 1 + g / (Nz / 2), k0 = 2 * (g % (Nz / 2));
    const double2 z = res[cr * Nx + kx];
    const double2 zc = res[cr * Nx + (kx == 0 ? 0 : Nx - kx)];   // conj taken below
    const double2 Aa = make_double2(z.x + zc.x, z.y - zc.y);
    const double2 Bb = make_double2(z.y + zc.y, zc.x - z.x);
    I.spec[((size_t)jc * Nz + k0) * Nxh + kx] = Aa;
    I.spec[((size_t)jc * Nz + k0 + 1) * Nxh + kx] = Bb;
  }
}

// ------------------------------------------------------------ z transform of the half spectrum
__global__ void __launch_bounds__(256)
k_fftz(ChlMap map, int inv, int zcw) {
  chl_pdl_wait();
  // The Ny x Nxh columns (jc, kx) of an instance are numbered jc-major and
  // cut into runs of zcw (chl_fftz_cols); a run may cross into the next
  // jc row, so every column is a full one and only the instance's last
  // block is short.
  extern __shared__ double2 sm[];
  __shared__ size_t coff[16];
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nz = I.Nz, Nxh = I.Nxh;
  const int q0 = lb * zcw;
  const int cw = min(zcw, I.Ny * Nxh - q0);
  if (threadIdx.x < cw) {
    const int q = q0 + threadIdx.x;
    coff[threadIdx.x] = (size_t)(1 + q / Nxh) * Nz * Nxh + (q % Nxh);
  }
  __syncthreads();
  double2* A = sm;
  double2* B = sm + Nz * zcw;
  double* T = reinterpret_cast<double*>(sm + 2 * Nz * zcw);   // pass table
  stage_twiddles(T, I.twz, chl_tw_len(Nz));
  double2* spec = I.spec;
  for (int w = threadIdx.x; w < Nz * cw; w += blockDim.x) {
    const int k = w / cw, c = w - k * cw;
    A[k * zcw + c] = spec[coff[c] + (size_t)k * Nxh];
  }
  double2* res = fft_smem(A, B, cw, 1, zcw, Nz, T, inv != 0, __double_as_longlong(I.fk[FK_MZERO]));
  for (int w = threadIdx.x; w < Nz * cw; w += blockDim.x) {
    const int k = w / cw, c = w - k * cw;
    spec[coff[c] + (size_t)k * Nxh] = res[k * zcw + c];
  }
}

// ------------------------------------------------------------ tridiagonal per mode
__global__ void __launch_bounds__(128)
k_tri(ChlMap map) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Ny = I.Ny, Nz = I.Nz, Nxh = I.Nxh;
  const int mode = lb * blockDim.x + threadIdx.x;
  if (mode >= Nz * Nxh) return;
  const size_t ps = (size_t)Nz * Nxh;           // row pitch of spec and factors
  double2* __restrict__ s = I.spec + ps + mode;  // row jc = 1
  const double* __restrict__ fi = I.tri_inv + mode;
  const double* __restrict__ fm = I.tri_m + mode;
  const double* __restrict__ fc = I.tri_c + mode;
  // The recurrence is serial in j; the loads are not.  Rows are fetched
  // TB at a time ahead of the chain so their latency overlaps.
  constexpr int TB = 8;
  double2 prev = make_double2(0.0, 0.0);
  for (int j0 = 0; j0 < Ny; j0 += TB) {
    double2 d[TB]; double iv[TB], m[TB];
#pragma unroll
    for (int q = 0; q < TB; ++q) {
      const int j = j0 + q;
      if (j < Ny) { d[q] = s[(size_t)j * ps]; iv[q] = LDG(fi + (size_t)j * ps); m[q] = LDG(fm + (size_t)j * ps); }
    }
#pragma unroll
    for (int q = 0; q < TB; ++q) {
      const int j = j0 + q;
      if (j < Ny) {
        d[q].x = fma(d[q].x, iv[q], -m[q] * prev.x);   // m = 0 on the first row
        d[q].y = fma(d[q].y, iv[q], -m[q] * prev.y);
        prev = d[q];
        s[(size_t)j * ps] = d[q];
      }
    }
  }
  // back substitution from the last row (prev holds it)
  for (int j1 = Ny - 2; j1 >= 0; j1 -= TB) {
    double2 d[TB]; double c[TB];
#pragma unroll
    for (int q = 0; q < TB; ++q) {
      const int j = j1 - q;
      if (j >= 0) { d[q] = s[(size_t)j * ps]; c[q] = LDG(fc + (size_t)j * ps); }
    }
#pragma unroll
    for (int q = 0; q < TB; ++q) {
      const int j = j1 - q;
      if (j >= 0) {
        d[q].x = fma(-c[q], prev.x, d[q].x);
        d[q].y = fma(-c[q], prev.y, d[q].y);
        prev = d[q];
        s[(size_t)j * ps] = d[q];
      }
    }
  }
}

// Staged form, for columns that fit in shared memory.  One warp of TRI_W
// modes per block.  Each thread copies its own mode's Ny rows of right side
// and factors into shared memory with cp.async (all rows in flight at once,
// where the form above waits once per TB rows), runs both sweeps there and
// writes only the solution.  A thread reads back only what it copied
// itself, so the copies need a wait but no block barrier.  The arithmetic
// and its order are those of k_tri.
#define TRI_W 32
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" :: "r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async8(void* sdst, const void* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" :: "r"(s), "l"(gsrc) : "memory");
}

__global__ void __launch_bounds__(TRI_W)
k_tri_staged(ChlMap map) {
  chl_pdl_wait();
  extern __shared__ double2 smt[];
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Ny = I.Ny, Nz = I.Nz, Nxh = I.Nxh;
  const int t = threadIdx.x;
  const int mode = lb * TRI_W + t;
  if (mode >= Nz * Nxh) return;
  const size_t ps = (size_t)Nz * Nxh;
  double2* __restrict__ s = I.spec + ps + mode;  // row jc = 1
  // [Ny][TRI_W] right side, then [Ny][TRI_W] x (inv, m, c) as doubles
  double2* sd = smt;
  double* sf = reinterpret_cast<double*>(smt + (size_t)Ny * TRI_W);
  double* si = sf;
  double* sm = sf + (size_t)Ny * TRI_W;
  double* sc = sf + (size_t)2 * Ny * TRI_W;
  for (int j = 0; j < Ny; ++j) {
    const size_t g = (size_t)j * ps, l = (size_t)j * TRI_W + t;
    cp_async16(sd + l, s + g);
    cp_async8(si + l, I.tri_inv + mode + g);
    cp_async8(sm + l, I.tri_m + mode + g);
    cp_async8(sc + l, I.tri_c + mode + g);
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  double2 prev = make_double2(0.0, 0.0);
  for (int j = 0; j < Ny; ++j) {
    const size_t l = (size_t)j * TRI_W + t;
    double2 d = sd[l];
    const double iv = si[l], m = sm[l];
    d.x = fma(d.x, iv, -m * prev.x);   // m = 0 on the first row
    d.y = fma(d.y, iv, -m * prev.y);
    prev = d;
    sd[l] = d;
  }
  s[(size_t)(Ny - 1) * ps] = prev;
  for (int j = Ny - 2; j >= 0; --j) {
    const size_t l = (size_t)j * TRI_W + t;
    double2 d = sd[l];
    const double c = sc[l];
    d.x = fma(-c, prev.x, d.x);
    d.y = fma(-c, prev.y, d.y);
    prev = d;
    s[(size_t)j * ps] = d;
  }
}

// Lane-split form, for instances with few modes: chl_tri_lanes(modes, Ny) =
// P lanes per mode (P = 1 for the larger instances of the same launch).
// Lane p owns rows [p L, (p+1) L), L = ceil(Ny / P).  Forward, the
// elimination y_j = iv_j d_j - m_j y_{j-1} maps the value entering a lane's
// rows affinely to the value leaving them: A y_in + B, A the product of the
// -m_j.  Each lane forms (A, B) from y_in = 0, an inclusive scan of these
// maps over the P lanes (warp shuffles within the lane group) gives every
// lane its y_in, and the lane reruns its rows from it, storing them.  The
// back substitution x_j = y_j - c_j x_{j+1} (c = 0 on the last row) is split
// the same way from the top.  With P = 1 the arithmetic is k_tri's; with
// P > 1 the scan rounds differently from the serial sweep (the multipliers
// are below 1 in magnitude, so the maps are contractions).  Every lane of a
// warp reaches the shuffles: a lane group belongs to one mode, and lanes
// past the last mode carry no rows.
// Rows of a lane are streamed TB at a time, their loads issued ahead of the
// serial arithmetic as in k_tri.
#define TSB 8
__global__ void __launch_bounds__(128)
k_tri_scan(ChlMap map) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Ny = I.Ny;
  const long modes = (long)I.Nz * I.Nxh;
  const int P = chl_tri_lanes(modes, Ny);
  const long g = (long)lb * blockDim.x + threadIdx.x;
  const long mode = g / P;
  const int p = (int)(g % P);
  const bool valid = mode < modes;
  const int L = (Ny + P - 1) / P;
  const int lo = min(Ny, p * L);
  const int hi = valid ? min(Ny, lo + L) : lo;      // rows [lo, hi) of this lane
  const size_t ps = (size_t)modes;                  // row pitch of spec and factors
  const long mm = valid ? mode : 0;
  double2* __restrict__ s = I.spec + ps + mm;       // row jc = 1
  const double* __restrict__ fi = I.tri_inv + mm;
  const double* __restrict__ fm = I.tri_m + mm;
  const double* __restrict__ fc = I.tri_c + mm;
  const unsigned full = 0xffffffffu;
  // forward sweep over [lo, hi) from `prev`; store = false only forms the
  // lane's affine map (prev from 0, A the product of the -m_j)
  auto forward = [&](double2 prev, bool store, double& A) {
    for (int j0 = lo; j0 < hi; j0 += TSB) {
      double2 d[TSB]; double iv[TSB], m[TSB];
#pragma unroll
      for (int q = 0; q < TSB; ++q) {
        const int j = j0 + q;
        if (j < hi) { d[q] = s[(size_t)j * ps]; iv[q] = LDG(fi + (size_t)j * ps); m[q] = LDG(fm + (size_t)j * ps); }
      }
#pragma unroll
      for (int q = 0; q < TSB; ++q) {
        const int j = j0 + q;
        if (j < hi) {
          d[q].x = fma(d[q].x, iv[q], -m[q] * prev.x);   // m = 0 on the first row
          d[q].y = fma(d[q].y, iv[q], -m[q] * prev.y);
          prev = d[q];
          if (store) s[(size_t)j * ps] = d[q];
          else A = -m[q] * A;
        }
      }
    }
    return prev;
  };
  auto backward = [&](double2 prev, bool store, double& A) {
    for (int j1 = hi - 1; j1 >= lo; j1 -= TSB) {
      double2 d[TSB]; double c[TSB];
#pragma unroll
      for (int q = 0; q < TSB; ++q) {
        const int j = j1 - q;
        if (j >= lo) { d[q] = s[(size_t)j * ps]; c[q] = LDG(fc + (size_t)j * ps); }
      }
#pragma unroll
      for (int q = 0; q < TSB; ++q) {
        const int j = j1 - q;
        if (j >= lo) {
          d[q].x = fma(-c[q], prev.x, d[q].x);        // c = 0 on the last row
          d[q].y = fma(-c[q], prev.y, d[q].y);
          prev = d[q];
          if (store) s[(size_t)j * ps] = d[q];
          else A = -c[q] * A;
        }
      }
    }
    return prev;
  };
  // ---- forward elimination
  double2 yin = make_double2(0.0, 0.0);
  if (P > 1) {
    double A = 1.0;
    double2 z = forward(make_double2(0.0, 0.0), false, A);
    for (int off = 1; off < P; off <<= 1) {
      const double Ao = __shfl_up_sync(full, A, off, P);
      const double bx = __shfl_up_sync(full, z.x, off, P), by = __shfl_up_sync(full, z.y, off, P);
      if (p >= off) { z.x = fma(A, bx, z.x); z.y = fma(A, by, z.y); A *= Ao; }
    }
    yin.x = __shfl_up_sync(full, z.x, 1, P);
    yin.y = __shfl_up_sync(full, z.y, 1, P);
    if (p == 0) yin = make_double2(0.0, 0.0);
  }
  double unused = 1.0;
  forward(yin, true, unused);
  // ---- back substitution from the top
  double2 xin = make_double2(0.0, 0.0);   // x of the row above the lane's rows
  if (P > 1) {
    double A = 1.0;
    double2 w = backward(make_double2(0.0, 0.0), false, A);
    for (int off = 1; off < P; off <<= 1) {
      const double Ao = __shfl_down_sync(full, A, off, P);
      const double bx = __shfl_down_sync(full, w.x, off, P), by = __shfl_down_sync(full, w.y, off, P);
      if (p + off < P) { w.x = fma(A, bx, w.x); w.y = fma(A, by, w.y); A *= Ao; }
    }
    xin.x = __shfl_down_sync(full, w.x, 1, P);
    xin.y = __shfl_down_sync(full, w.y, 1, P);
    if (p == P - 1) xin = make_double2(0.0, 0.0);
  }
  backward(xin, true, unused);
}

// ------------------------------------------------------------ fused z transform + tridiagonal + inverse z
// For instances whose wavenumber column block fits in shared memory: one
// thread-block cluster of P CTAs per (instance, kx), P = chl_tri_lanes of
// the instance (the lane count of k_tri_scan).  CTA r holds the rows that
// lane r of k_tri_scan owns, [r L, min(Ny, (r+1) L)) with L = ceil(Ny/P),
// for all Nz wavenumbers kz, and runs on them
//   the forward z transform (the Stockham passes of k_fftz),
//   the Thomas sweeps of k_tri_scan, whose lane maps (A, z) it exchanges
//     with the other CTAs of its cluster through distributed shared memory
//     and scans with the same warp shuffles (one thread per (kz, lane)),
//   the inverse z transform,
// so the result is bit-identical to k_fftz, the tridiagonal kernel and
// k_fftz again, in one launch and without the two round trips of the
// spectrum.  The cluster barriers are hardware barriers that every thread
// of the cluster reaches (no early exit).
namespace cg = cooperative_groups;

__global__ void __launch_bounds__(256)
k_zsolve(ChlMap map) {
  chl_pdl_wait();
  extern __shared__ double2 sm[];
  cg::cluster_group cl = cg::this_cluster();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Ny = I.Ny, Nz = I.Nz, Nxh = I.Nxh;
  const long modes = (long)Nz * Nxh;
  const int P = chl_tri_lanes(modes, Ny);       // the cluster size (host-checked)
  const int r = lb % P, kx = lb / P;
  const int L = (Ny + P - 1) / P;
  const int lo = min(Ny, r * L), hi = min(Ny, lo + L), nr = hi - lo;
  const size_t ps = (size_t)modes;              // row pitch of spec and factors
  double2* A = sm;
  double2* B = sm + (size_t)L * Nz;
  double* T = reinterpret_cast<double*>(sm + (size_t)2 * L * Nz);   // pass table
  double2* fz = reinterpret_cast<double2*>(reinterpret_cast<char*>(T) + chl_tw_bytes(chl_tw_len(Nz)));
                                                // forward lane values
  double2* bw = fz + Nz;                        // backward lane values
  double2* yin = bw + Nz;
  double2* xin = yin + Nz;
  double* fA = reinterpret_cast<double*>(xin + Nz);
  double* bA = fA + Nz;
  const int t = threadIdx.x, bd = blockDim.x;
  stage_twiddles(T, I.twz, chl_tw_len(Nz));
  // rows [lo, hi) of column kx: element (row l, kz) at l + kz*nr
  double2* spec = I.spec + ps + kx;             // row jc = 1
  for (int w = t; w < nr * Nz; w += bd) {
    const int l = w % nr, kz = w / nr;
    A[l + (size_t)kz * nr] = spec[(size_t)(lo + l) * ps + (size_t)kz * Nxh];
  }
  double2* res = fft_smem(A, B, nr, 1, nr, Nz, T, false, __double_as_longlong(I.fk[FK_MZERO]));
  double2* other = res == A ? B : A;
  const double* __restrict__ fi = I.tri_inv + kx;
  const double* __restrict__ fm = I.tri_m + kx;
  const double* __restrict__ fc = I.tri_c + kx;
  const unsigned full = 0xffffffffu;
  // ---- forward elimination: this CTA's lane maps
  if (P > 1) {
    for (int kz = t; kz < Nz; kz += bd) {
      const size_t mo = (size_t)kz * Nxh;
      double Am = 1.0;
      double2 prev = make_double2(0.0, 0.0);
      for (int j = lo; j < hi; ++j) {
        double2 d = res[(j - lo) + (size_t)kz * nr];
        const double iv = LDG(fi + (size_t)j * ps + mo), m = LDG(fm + (size_t)j * ps + mo);
        d.x = fma(d.x, iv, -m * prev.x);
        d.y = fma(d.y, iv, -m * prev.y);
        prev = d;
        Am = -m * Am;
      }
      fA[kz] = Am;
      fz[kz] = prev;
    }
  }
  cl.sync();
  if (P > 1) {
    // one thread per (kz, lane p): the inclusive scan of k_tri_scan
    for (int base = 0; base < Nz * P; base += bd) {
      const int w = base + t, kz = w / P, p = w % P;
      const bool ok = kz < Nz;
      const double* rA = cl.map_shared_rank(fA, p);
      const double2* rz = cl.map_shared_rank(fz, p);
      double Av = ok ? rA[kz] : 1.0;
      double2 z = ok ? rz[kz] : make_double2(0.0, 0.0);
      for (int off = 1; off < P; off <<= 1) {
        const double Ao = __shfl_up_sync(full, Av, off, P);
        const double bx = __shfl_up_sync(full, z.x, off, P), by = __shfl_up_sync(full, z.y, off, P);
        if (p >= off) { z.x = fma(Av, bx, z.x); z.y = fma(Av, by, z.y); Av *= Ao; }
      }
      double2 y;
      y.x = __shfl_up_sync(full, z.x, 1, P);
      y.y = __shfl_up_sync(full, z.y, 1, P);
      if (p == 0) y = make_double2(0.0, 0.0);
      if (ok && p == r) yin[kz] = y;
    }
  }
  __syncthreads();
  for (int kz = t; kz < Nz; kz += bd) {
    const size_t mo = (size_t)kz * Nxh;
    double2 prev = P > 1 ? yin[kz] : make_double2(0.0, 0.0);
    for (int j = lo; j < hi; ++j) {
      double2 d = res[(j - lo) + (size_t)kz * nr];
      const double iv = LDG(fi + (size_t)j * ps + mo), m = LDG(fm + (size_t)j * ps + mo);
      d.x = fma(d.x, iv, -m * prev.x);   // m = 0 on the first row
      d.y = fma(d.y, iv, -m * prev.y);
      prev = d;
      res[(j - lo) + (size_t)kz * nr] = d;
    }
  }
  // ---- back substitution from the top
  if (P > 1) {
    for (int kz = t; kz < Nz; kz += bd) {
      const size_t mo = (size_t)kz * Nxh;
      double Am = 1.0;
      double2 prev = make_double2(0.0, 0.0);
      for (int j = hi - 1; j >= lo; --j) {
        double2 d = res[(j - lo) + (size_t)kz * nr];
        const double c = LDG(fc + (size_t)j * ps + mo);
        d.x = fma(-c, prev.x, d.x);
        d.y = fma(-c, prev.y, d.y);
        prev = d;
        Am = -c * Am;
      }
      bA[kz] = Am;
      bw[kz] = prev;
    }
  }
  cl.sync();
  if (P > 1) {
    for (int base = 0; base < Nz * P; base += bd) {
      const int w = base + t, kz = w / P, p = w % P;
      const bool ok = kz < Nz;
      const double* rA = cl.map_shared_rank(bA, p);
      const double2* rw = cl.map_shared_rank(bw, p);
      double Av = ok ? rA[kz] : 1.0;
      double2 v = ok ? rw[kz] : make_double2(0.0, 0.0);
      for (int off = 1; off < P; off <<= 1) {
        const double Ao = __shfl_down_sync(full, Av, off, P);
        const double bx = __shfl_down_sync(full, v.x, off, P), by = __shfl_down_sync(full, v.y, off, P);
        if (p + off < P) { v.x = fma(Av, bx, v.x); v.y = fma(Av, by, v.y); Av *= Ao; }
      }
      double2 x;
      x.x = __shfl_down_sync(full, v.x, 1, P);
      x.y = __shfl_down_sync(full, v.y, 1, P);
      if (p == P - 1) x = make_double2(0.0, 0.0);
      if (ok && p == r) xin[kz] = x;
    }
  }
  __syncthreads();
  for (int kz = t; kz < Nz; kz += bd) {
    const size_t mo = (size_t)kz * Nxh;
    double2 prev = P > 1 ? xin[kz] : make_double2(0.0, 0.0);
    for (int j = hi - 1; j >= lo; --j) {
      double2 d = res[(j - lo) + (size_t)kz * nr];
      const double c = LDG(fc + (size_t)j * ps + mo);
      d.x = fma(-c, prev.x, d.x);        // c = 0 on the last row
      d.y = fma(-c, prev.y, d.y);
      prev = d;
      res[(j - lo) + (size_t)kz * nr] = d;
    }
  }
  double2* out = fft_smem(res, other, nr, 1, nr, Nz, T, true, __double_as_longlong(I.fk[FK_MZERO]));
  for (int w = t; w < nr * Nz; w += bd) {
    const int l = w % nr, kz = w / nr;
    spec[(size_t)(lo + l) * ps + (size_t)kz * Nxh] = out[l + (size_t)kz * nr];
  }
  cl.sync();   // no CTA leaves while another may still read its lane values
}

// ------------------------------------------------------------ inverse x -> pressure field
__global__ void __launch_bounds__(256)
k_fftx_inv(ChlMap map, int dst, int xmb) {
  chl_pdl_wait();
  extern __shared__ double2 sm[];
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz, Nxh = I.Nxh;
  const int nrow = Ny * (Nz / 2);
  const int CR = chl_fftx_rows(Nx, nrow, xmb);
  const int g0 = lb * CR;
  const int cr_n = min(CR, nrow - g0);
  double2* A = sm;
  double2* B = sm + CR * Nx;
  double* T = reinterpret_cast<double*>(sm + 2 * CR * Nx);   // pass table
  stage_twiddles(T, I.twx, chl_tw_len(Nx));
  for (int w = threadIdx.x; w < cr_n * Nx; w += blockDim.x) {
    const int cr = w / Nx, kx = w - cr * Nx;
    const int g = g0 + cr;
    const int jc = 1 + g / (Nz / 2), k0 = 2 * (g % (Nz / 2));
    const bool lo = kx <= Nx / 2;
    const int kk = lo ? kx : Nx - kx;
    const double2 pa = I.spec[((size_t)jc * Nz + k0) * Nxh + kk];
    const double2 pb = I.spec[((size_t)jc * Nz + k0 + 1) * Nxh + kk];
    A[cr * Nx + kx] = lo ? make_double2(pa.x - pb.y, pa.y + pb.x)
                         : make_double2(pa.x + pb.y, pb.x - pa.y);
  }
  double2* res = fft_smem(A, B, cr_n, Nx, 1, Nx, T, true, __double_as_longlong(I.fk[FK_MZERO]));
  double* out = dst == 0 ? I.p : I.P;
  for (int w = threadIdx.x; w < cr_n * Nx; w += blockDim.x) {
    const int cr = w / Nx, i = w - cr * Nx;
    const int g = g0 + cr;
    const int jc = 1 + g / (Nz / 2), k0 = 2 * (g % (Nz / 2));
    const double2 z = res[cr * Nx + i];
    out[cidx(I, i, jc, k0)] = z.x;
    out[cidx(I, i, jc, k0 + 1)] = z.y;
  }
}

// ------------------------------------------------------------ velocity correction
// project_velocity (projection.f90:192-214) + Dirichlet ghost rows.
__global__ void __launch_bounds__(256)
k_project(ChlMap map, int s) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const unsigned t = (unsigned)lb * blockDim.x + threadIdx.x;
  if (t >= (unsigned)(Nx * Ny * Nz)) return;
  const ChlIdx ix = chl_split(t, Nx, Ny);
  const int i = ix.i, jc = 1 + ix.j, k = ix.k;
  const double* p = I.p;
  const size_t c = cidx(I, i, jc, k);
  const double p0 = LDG(p + c);
  double* U = I.U[s]; double* V = I.V[s]; double* W = I.W[s];
  const double un = U[c] - (LDG(p + cidx(I, wrap(i + 1, Nx), jc, k)) - p0) * LDG(I.rdxf + i);
  const double wn = W[c] - (LDG(p + cidx(I, i, jc, wrap(k + 1, Nz))) - p0) * LDG(I.rdzf + k);
  U[c] = un; W[c] = wn;
  if (jc <= Ny - 1) {
    const size_t v = vidx(I, i, jc, k);
    V[v] = V[v] - (LDG(p + cidx(I, i, jc + 1, k)) - p0) * LDG(I.rdyf + jc);
  }
  if (jc == 1) { U[cidx(I, i, 0, k)] = -un; W[cidx(I, i, 0, k)] = -wn; }
  if (jc == Ny) { U[cidx(I, i, Ny + 1, k)] = -un; W[cidx(I, i, Ny + 1, k)] = -wn; }
}

// ------------------------------------------------------------ actual pressure: wall BC planes
// compute_pressure_BC (pressure.f90:269-340): bc = d/dy(nu dV/dy) at both walls.
__global__ void k_pbc(ChlMap map, int s) {
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  long t = (long)lb * blockDim.x + threadIdx.x;
  if (t >= 2L * Nx * Nz) return;
  const int i = (int)(t % Nx), k = (int)((t / Nx) % Nz), wall = (int)(t / ((long)Nx * Nz));
  const double* V = I.V[s];
  const double* nt = I.nut;      // nu + nu_t
  double bcv;
  if (wall == 0) {
    const double g = I.gb1, g2 = I.gb2;
    const double nui = 0.5 * (nt[cidx(I, i, 0, k)] + nt[cidx(I, i, 1, k)]);
    const double dnu = (nt[cidx(I, i, 1, k)] - nt[cidx(I, i, 0, k)]) / I.dygb;
    const double v1 = V[vidx(I, i, 0, k)], v2 = V[vidx(I, i, 1, k)], v3 = V[vidx(I, i, 2, k)], v4 = V[vidx(I, i, 3, k)];
    const double dV = (-3.0 * v1 + 4.0 * v2 - v3) / 2.0 * (1.0 / g);
    double ddV = 2.0 * v1 - 5.0 * v2 + 4.0 * v3 - 1.0 * v4;
    ddV = (ddV - dV * g2) / (g * g);
    bcv = dnu * dV + nui * ddV;
  } else {
    const double g = I.gt1, g2 = I.gt2;
    const double nui = 0.5 * (nt[cidx(I, i, Ny + 1, k)] + nt[cidx(I, i, Ny, k)]);
    const double dnu = (nt[cidx(I, i, Ny + 1, k)] - nt[cidx(I, i, Ny, k)]) / I.dygt;
    const double v1 = V[vidx(I, i, Ny, k)], v2 = V[vidx(I, i, Ny - 1, k)], v3 = V[vidx(I, i, Ny - 2, k)], v4 = V[vidx(I, i, Ny - 3, k)];
    const double dV = (3.0 * v1 - 4.0 * v2 + v3) / 2.0 * (1.0 / g);
    double ddV = 2.0 * v1 - 5.0 * v2 + 4.0 * v3 - 1.0 * v4;
    ddV = (ddV - dV * g2) / (g * g);
    bcv = dnu * dV + nui * ddV;
  }
  I.bc[t] = bcv;
}

// P ghost rows (pressure.f90:158-159)
__global__ void k_pghost(ChlMap map) {
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  long t = (long)lb * blockDim.x + threadIdx.x;
  if (t >= (long)Nx * Nz) return;
  const int i = (int)(t % Nx), k = (int)(t / Nx);
  double* P = I.P;
  P[cidx(I, i, 0, k)] = P[cidx(I, i, 1, k)] - I.dygb * I.bc[t];
  P[cidx(I, i, Ny + 1, k)] = P[cidx(I, i, Ny, k)] + I.dygt * I.bc[(size_t)Nx * Nz + t];
}

extern "C" {
// two ping-pong tiles plus the pass table (twz: the longest z pass table
// of the launch's instances, in doubles)
size_t chl_smem_fftx(int Nx, int nrow, int xmb) {
  return (size_t)2 * chl_fftx_rows(Nx, nrow, xmb) * Nx * sizeof(double2) + chl_tw_bytes(chl_tw_len(Nx));
}
size_t chl_smem_fftz(int maxNz, int zcw, int twz) { return (size_t)2 * zcw * maxNz * sizeof(double2) + chl_tw_bytes(twz); }
// kx columns staged per z-transform block: 16, halved while two Nz x cols
// complex tiles would exceed the 227 KB a block may use, and halved (down
// to 2) while the grid over all `ncols` columns would have fewer than
// min_blocks blocks (CHL_FFT_MIN_BLOCKS, about four per SM, unless the
// tuner chose another)
int chl_fftz_cols(int maxNz, long ncols, int min_blocks, int twz) {
  int c = 16;
  while (c > 1 && chl_smem_fftz(maxNz, c, twz) > (size_t)227 * 1024) c /= 2;
  while (c > 2 && (ncols + c - 1) / c < min_blocks) c /= 2;
  return c;
}
int chl_fft_setup(size_t smx, size_t smz, size_t smt) {
  cudaError_t e1 = cudaFuncSetAttribute(k_div_fftx, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smx);
  cudaError_t e2 = cudaFuncSetAttribute(k_fftx_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smx);
  cudaError_t e3 = cudaFuncSetAttribute(k_fftz, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smz);
  cudaError_t e4 = smt ? cudaFuncSetAttribute(k_tri_staged, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smt)
                       : cudaSuccess;
  return (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess || e4 != cudaSuccess) ? 1 : 0;
}
void chl_launch_div_fftx(const ChlMap& m, int nb, int nt, size_t smem, int s_in, int mode, int xmb, cudaStream_t st) { chl_launch_pdl(k_div_fftx, dim3(nb), dim3(nt), smem, st, m, s_in, mode, xmb); }
void chl_launch_fftz(const ChlMap& m, int nb, int nt, size_t smem, int inv, int zcw, cudaStream_t st) { chl_launch_pdl(k_fftz, dim3(nb), dim3(nt), smem, st, m, inv, zcw); }
// smem > 0: the staged form with TRI_W-mode blocks (chl_tri_modes_per_block)
void chl_launch_tri(const ChlMap& m, int nb, size_t smem, cudaStream_t st) {
  if (smem) chl_launch_pdl(k_tri_staged, dim3(nb), dim3(TRI_W), smem, st, m);
  else chl_launch_pdl(k_tri, dim3(nb), dim3(128), 0, st, m);
}
// Shared memory of the staged form for the tallest column (40 bytes per
// row and mode), or 0 for the row-batched form.  mode 0: row-batched;
// 1: staged whenever it fits; 2 (default): staged only while all `modes`
// fit in one wave of resident blocks - the staged form has one warp per
// block, and beyond one wave the row-batched form keeps more warps per SM.
size_t chl_smem_tri(int maxNy, long modes, int mode) {
  const size_t b = (size_t)maxNy * TRI_W * (sizeof(double2) + 3 * sizeof(double));
  if (mode == 0 || b > (size_t)CHL_TRI_SMEM_MAX) return 0;
  if (mode == 1) return b;
  const long per_sm = (long)((228 * 1024) / (b + 1024));   // + the 1 KB the runtime reserves per block
  const long blocks = (modes + TRI_W - 1) / TRI_W;
  return blocks <= per_sm * CHL_SMS ? b : 0;
}
int chl_tri_modes_per_block(size_t smem) { return smem ? TRI_W : 128; }
// Fused z solve: shared memory of a CTA for an instance (0 if its block does
// not fit, or its lane count is not a cluster size of 1, 2, 4 or 8), and its
// launch: cluster (P, 1, 1), Nxh x P CTAs per instance.
size_t chl_smem_zsolve(int Nx, int Ny, int Nz) {
  const int Nxh = Nx / 2 + 1;
  const int P = chl_tri_lanes((long)Nz * Nxh, Ny);
  if (P != 1 && P != 2 && P != 4 && P != 8) return 0;
  const int L = (Ny + P - 1) / P;
  const size_t b = (size_t)2 * L * Nz * sizeof(double2) + chl_tw_bytes(chl_tw_len(Nz)) + (size_t)4 * Nz * sizeof(double2) +
                   (size_t)2 * Nz * sizeof(double);
  return b <= (size_t)227 * 1024 ? b : 0;
}
int chl_zsolve_setup(size_t smem) {
  return cudaFuncSetAttribute(k_zsolve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess ? 0 : 1;
}
void chl_launch_zsolve(const ChlMap& m, int nb, int P, size_t smem, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nb); cfg.blockDim = dim3(256); cfg.dynamicSmemBytes = smem; cfg.stream = st;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  at[1].id = cudaLaunchAttributeClusterDimension;
  at[1].val.clusterDim.x = P; at[1].val.clusterDim.y = 1; at[1].val.clusterDim.z = 1;
  cfg.attrs = at; cfg.numAttrs = 2;
  cudaLaunchKernelEx(&cfg, k_zsolve, m);
}
void chl_launch_tri_scan(const ChlMap& m, int nb, cudaStream_t st) { chl_launch_pdl(k_tri_scan, dim3(nb), dim3(128), 0, st, m); }
void chl_launch_fftx_inv(const ChlMap& m, int nb, int nt, size_t smem, int dst, int xmb, cudaStream_t st) { chl_launch_pdl(k_fftx_inv, dim3(nb), dim3(nt), smem, st, m, dst, xmb); }
void chl_launch_project(const ChlMap& m, int nb, int s, cudaStream_t st) { chl_launch_pdl(k_project, dim3(nb), dim3(m.tb), 0, st, m, s); }
void chl_launch_pbc(const ChlMap& m, int nb, int s, cudaStream_t st) { k_pbc<<<nb, 256, 0, st>>>(m, s); }
void chl_launch_pghost(const ChlMap& m, int nb, cudaStream_t st) { k_pghost<<<nb, 256, 0, st>>>(m); }
}
