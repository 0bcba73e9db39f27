// Subgrid-scale eddy viscosity and wall models.
//
// Dynamic Smagorinsky (Lilly) as sgs_dynamic_Smagorinsky does it
// (subgrid.f90:379-537): test filter filter_xzy (subgrid.f90:140-190, the
// 1/6-2/3-1/6 rule in x, z and y, one-sided 2/3-1/3 at the first and last
// row), strain rates of compute_Sij (subgrid.f90:1014-1072), plane sums of
// L:M and M:M over i=2..nxg-1, k=2..nzg-1 (the duplicated periodic column
// and plane counted twice, subgrid.f90:492-509), nu_t = max(0,-1/2 <LM>/<MM>|S|)
// and the ghost-row rule of Dirichlet_nu_t.
//
// The filter is applied as three separable passes with unnormalised weights
// (1,4,1) and (4,2); the 6^3 = 216 scale, the 1/2 of the centre averages
// and the 1/8 of the edge averages are folded into the final L:M and M:M
// dot products, which only enter as the ratio <LM>/<MM>.  This keeps the
// FP64 instruction count per point at its minimum (the GB300 FP64 pipe, not
// HBM, bounds this code).
//
// Static Smagorinsky with van Driest damping (subgrid.f90:563-612, which
// aborts in the reference) is written from its formula.  The stress wall
// model is compute_wall_model (wallmodel.f90:23-46); the equilibrium log-law
// wall stress that feeds it is new.
#include "chl_common.cuh"

// ---------------------------------------------------------------- edges
// E12 at (x-face a, y-face jv, z-centre k), E13 at (x-face a, centre row jc,
// z-face b), E23 at (x-centre i, y-face jv, z-face b): 2 x the edge strain
// rates of compute_Sij, stored V-like (E12, E23: Ny+1 rows) and centre-like
// (E13, rows 1..Ny).  Of the filtered faces (src 3) with the reciprocals
// scaled by sqrt(4/216) (rdxfs ...), for the filtered strain of k_dsm_final.
__global__ void __launch_bounds__(256)
k_edges(ChlMap map, int src) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const unsigned t = (unsigned)lb * blockDim.x + threadIdx.x;
  if (t >= (unsigned)(Nx * (Ny + 1) * Nz)) return;
  const ChlIdx p = chl_split(t, Nx, Ny + 1);
  const int a = p.i, j = p.j, k = p.k;
  const double *U, *V, *W;
  if (src < 3) { U = I.U[src]; V = I.V[src]; W = I.W[src]; }
  else { U = I.r[15]; V = I.r[16]; W = I.r[17]; }
  const int ap = wrap(a + 1, Nx), kp = wrap(k + 1, Nz);
  const bool filt = src == 3;
  const double rxf = LDG((filt ? I.rdxfs : I.rdxf) + a), rzf = LDG((filt ? I.rdzfs : I.rdzf) + k);
  const double ryf = LDG((filt ? I.rdyfs : I.rdyf) + j);
  const F64 f = f64_of(I);   // differences and products as register FMAs
  // E12 (jv = j): dU/dy + dV/dx
  const double e12 = fma(f.sub(LDG(U + cidx(I, a, j + 1, k)), LDG(U + cidx(I, a, j, k))), ryf,
                         f.mul(f.sub(LDG(V + vidx(I, ap, j, k)), LDG(V + vidx(I, a, j, k))), rxf));
  // E23 (jv = j, b = k): dV/dz + dW/dy
  const double e23 = fma(f.sub(LDG(V + vidx(I, a, j, kp)), LDG(V + vidx(I, a, j, k))), rzf,
                         f.mul(f.sub(LDG(W + cidx(I, a, j + 1, k)), LDG(W + cidx(I, a, j, k))), ryf));
  I.E[0][vidx(I, a, j, k)] = e12;
  I.E[2][vidx(I, a, j, k)] = e23;
  if (j >= 1 && j <= Ny) {
    // E13 (jc = j, b = k): dU/dz + dW/dx
    const double e13 = fma(f.sub(LDG(U + cidx(I, a, j, kp)), LDG(U + cidx(I, a, j, k))), rzf,
                           f.mul(f.sub(LDG(W + cidx(I, ap, j, k)), LDG(W + cidx(I, a, j, k))), rxf));
    I.E[1][cidx(I, a, j, k)] = e13;
  }
}

// The same edges, with the x-pair sums that every centre strain needs
// formed once per edge: P12(a) = E12(a-1) + E12(a) and P13(a) = E13(a-1) +
// E13(a) are stored in place of E12 and E13 (E23 as it is).  A block (64,
// 128 or 256 threads: the launch's largest Nx rounded up to a power of two,
// at least 64) holds blockDim / Nx whole x-rows (j, k) (Nx <= 256), so the
// left neighbour, periodic, comes from shared memory: one addition per edge
// instead of two per centre.  The centre strain's sums keep their order,
// (E(i-1) + E(i)) + (E'(i-1) + E'(i)), so the result is bit-identical.
__global__ void __launch_bounds__(256)
k_edges_pair(ChlMap map, int src) {
  chl_pdl_wait();
  __shared__ double s12[256], s13[256];
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const int RB = blockDim.x / Nx;
  const int r = threadIdx.x / Nx, a = threadIdx.x - r * Nx;
  const unsigned g = (unsigned)lb * RB + r;          // the row (j, k), j = 0..Ny
  const bool valid = r < RB && g < (unsigned)((Ny + 1) * Nz);
  const unsigned gk = valid ? g / (unsigned)(Ny + 1) : 0u;
  const int j = valid ? (int)(g - gk * (unsigned)(Ny + 1)) : 0, k = (int)gk;
  const double *U, *V, *W;
  if (src < 3) { U = I.U[src]; V = I.V[src]; W = I.W[src]; }
  else { U = I.r[15]; V = I.r[16]; W = I.r[17]; }
  const int ap = wrap(a + 1, Nx), kp = wrap(k + 1, Nz);
  const bool filt = src == 3;
  const double rxf = LDG((filt ? I.rdxfs : I.rdxf) + a), rzf = LDG((filt ? I.rdzfs : I.rdzf) + k);
  const double ryf = LDG((filt ? I.rdyfs : I.rdyf) + j);
  const F64 f = f64_of(I);   // differences and products as register FMAs
  const double e12 = fma(f.sub(LDG(U + cidx(I, a, j + 1, k)), LDG(U + cidx(I, a, j, k))), ryf,
                         f.mul(f.sub(LDG(V + vidx(I, ap, j, k)), LDG(V + vidx(I, a, j, k))), rxf));
  const double e23 = fma(f.sub(LDG(V + vidx(I, a, j, kp)), LDG(V + vidx(I, a, j, k))), rzf,
                         f.mul(f.sub(LDG(W + cidx(I, a, j + 1, k)), LDG(W + cidx(I, a, j, k))), ryf));
  // E13 on the centre rows 1..Ny (row 0 computes an unused value from the ghost row)
  const double e13 = fma(f.sub(LDG(U + cidx(I, a, j, kp)), LDG(U + cidx(I, a, j, k))), rzf,
                         f.mul(f.sub(LDG(W + cidx(I, ap, j, k)), LDG(W + cidx(I, a, j, k))), rxf));
  s12[threadIdx.x] = e12;
  s13[threadIdx.x] = e13;
  __syncthreads();
  if (!valid) return;
  const int left = r * Nx + (a == 0 ? Nx - 1 : a - 1);
  I.E[0][vidx(I, a, j, k)] = s12[left] + e12;
  I.E[2][vidx(I, a, j, k)] = e23;
  if (j >= 1) I.E[1][cidx(I, a, j, k)] = s13[left] + e13;
}

// Centre strain: diagonal D, 8*S_offdiag O (sum of four edges), and
// s = |S|/sqrt(2).  The sqrt(2) never needs forming: nu_t = c |S| where the
// dynamic model's c comes from L:M / M:M with M linear in |S| and |S^| (so
// keeping both /sqrt(2) scales c by sqrt(2) and c s = c_true |S|), and the
// static model's row coefficient carries the sqrt(2) itself (k_coef).
struct Strain { double d1, d2, d3, o12, o13, o23, s; };

// The six face velocities around centre (i, jc, k): u0 = U(i-1), u1 = U(i),
// v0 = V(jc-1), v1 = V(jc), w0 = W(k-1), w1 = W(k).
struct Faces { double u0, u1, v0, v1, w0, w1; };

__device__ __forceinline__ Faces centre_faces(const ChlInst& I, const double* U, const double* V,
                                              const double* W, int i, int jc, int k) {
  const int im = wrap(i - 1, I.Nx), km = wrap(k - 1, I.Nz);
  Faces f;
  f.u0 = LDG(U + cidx(I, im, jc, k)); f.u1 = LDG(U + cidx(I, i, jc, k));
  f.v0 = LDG(V + vidx(I, i, jc - 1, k)); f.v1 = LDG(V + vidx(I, i, jc, k));
  f.w0 = LDG(W + cidx(I, i, jc, km)); f.w1 = LDG(W + cidx(I, i, jc, k));
  return f;
}

// FILT: the filtered strain, with the sqrt(4/216)-scaled reciprocals and
// edges, so that it comes out times sqrt(4/216).  PAIR: E12 and E13 hold the
// x-pair sums of k_edges_pair.
template <bool FILT, bool PAIR>
__device__ __forceinline__ Strain centre_strain(const ChlInst& I, const Faces& f, int i, int jc, int k) {
  const int im = wrap(i - 1, I.Nx), km = wrap(k - 1, I.Nz);
  Strain s;
  s.d1 = (f.u1 - f.u0) * LDG((FILT ? I.rdxcs : I.rdxc) + i);
  s.d2 = (f.v1 - f.v0) * LDG((FILT ? I.rdycs : I.rdyc) + jc);
  s.d3 = (f.w1 - f.w0) * LDG((FILT ? I.rdzcs : I.rdzc) + k);
  const double* E12 = I.E[0]; const double* E13 = I.E[1]; const double* E23 = I.E[2];
  if (PAIR) {
    s.o12 = LDG(E12 + vidx(I, i, jc - 1, k)) + LDG(E12 + vidx(I, i, jc, k));
    s.o13 = LDG(E13 + cidx(I, i, jc, km)) + LDG(E13 + cidx(I, i, jc, k));
  } else {
    s.o12 = (LDG(E12 + vidx(I, im, jc - 1, k)) + LDG(E12 + vidx(I, i, jc - 1, k)))
          + (LDG(E12 + vidx(I, im, jc, k)) + LDG(E12 + vidx(I, i, jc, k)));
    s.o13 = (LDG(E13 + cidx(I, im, jc, km)) + LDG(E13 + cidx(I, i, jc, km)))
          + (LDG(E13 + cidx(I, im, jc, k)) + LDG(E13 + cidx(I, i, jc, k)));
  }
  s.o23 = (LDG(E23 + vidx(I, i, jc - 1, km)) + LDG(E23 + vidx(I, i, jc, km)))
        + (LDG(E23 + vidx(I, i, jc - 1, k)) + LDG(E23 + vidx(I, i, jc, k)));
  // |S|^2 = 2 (d.d) + 4 (S12^2+S13^2+S23^2) = 2 (d.d + (o.o)/32)
  double dd = s.d1 * s.d1; dd = fma(s.d2, s.d2, dd); dd = fma(s.d3, s.d3, dd);
  double oo = s.o12 * s.o12; oo = fma(s.o13, s.o13, oo); oo = fma(s.o23, s.o23, oo);
  s.s = chl_sqrt(fma(oo, 0.03125, dd));   // |S| / sqrt(2)
  return s;
}

// Raw strain and the DSM filter inputs at centres (rows 1..Ny):
// q0..2 = 2*(centre velocities), q3..8 = their products, q9..14 = |S|*(d, o).
// q0..2 are stored only in the two rows next to each wall: the filter is
// linear and shift-invariant, so away from the walls the filtered centre
// velocity is the centre average of the filtered face velocity (k_dsm_final
// forms it there); only rows 1 and Ny, where the centre filter takes its
// one-sided rule and the face filter does not, need the centre velocity
// filtered in its own right.
// DSM and PAIR are template parameters: a runtime switch would leave the
// FP64 work of the other side predicated in every warp.
template <bool DSM, bool PAIR>
__global__ void __launch_bounds__(256)
k_centre(ChlMap map, int s_in) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const unsigned t = (unsigned)lb * blockDim.x + threadIdx.x;
  if (t >= (unsigned)(Nx * Ny * Nz)) return;
  const ChlIdx p = chl_split(t, Nx, Ny);
  const int i = p.i, jc = 1 + p.j, k = p.k;
  const Faces f = centre_faces(I, I.U[s_in], I.V[s_in], I.W[s_in], i, jc, k);
  const Strain s = centre_strain<false, PAIR>(I, f, i, jc, k);
  const size_t c = cidx(I, i, jc, k);
  I.S[c] = s.s;
  if (!DSM) return;
  const double uc = f.u0 + f.u1, vc = f.v0 + f.v1, wc = f.w0 + f.w1;
  if (jc <= 2 || jc >= Ny - 1) { I.q[0][c] = uc; I.q[1][c] = vc; I.q[2][c] = wc; }
  I.q[3][c] = uc * uc; I.q[4][c] = vc * vc; I.q[5][c] = wc * wc;
  I.q[6][c] = uc * vc; I.q[7][c] = uc * wc; I.q[8][c] = vc * wc;
  I.q[9][c] = s.s * s.d1; I.q[10][c] = s.s * s.d2; I.q[11][c] = s.s * s.d3;
  I.q[12][c] = s.s * s.o12; I.q[13][c] = s.s * s.o13; I.q[14][c] = s.s * s.o23;
}

// ------------------------------------------------------------ filter passes
// y pass: q (and the velocity set s_in for the three face components) -> r.
// Centre components use rows 1..Ny, U and W rows 0..Ny+1, V rows 0..Ny, each
// with the one-sided rule at its first and last row.
// Branch-free: at the first (last) row the missing neighbour is replaced by
// the other one, so lo + 4q + hi becomes 4q + 2*hi (4q + 2*lo), the
// one-sided 2/3-1/3 rule times 6.  Only the addresses are selected.
__device__ __forceinline__ double fy(const double* f, size_t c, size_t pitch, int j, int j0, int j1, const F64& k,
                                     double four) {
  const size_t lo = (j == j0) ? c + pitch : c - pitch;
  const size_t hi = (j == j1) ? c - pitch : c + pitch;
  return fma(four, LDG(f + c), k.add(LDG(f + lo), LDG(f + hi)));
}

// N components from N0 on: out = in(lo) + 4 in(c) + in(hi).  All loads are
// issued before the stores: the stores may alias the loads as far as the
// compiler knows, so this is what keeps enough loads in flight.  The sum
// and the 4 go in as registers (F64): the filter passes are made of nothing
// else, and that form measured 12 % faster for the y pass.
template <int N0, int N>
__device__ __forceinline__ void filter_group(double* const* in, double* const* out, size_t c, size_t lo,
                                             size_t hi, const F64& k, double four) {
  double a[N], b[N], d[N];
#pragma unroll
  for (int q = 0; q < N; ++q) {
    const double* f = in[N0 + q];
    a[q] = LDG(f + c); b[q] = LDG(f + lo); d[q] = LDG(f + hi);
  }
#pragma unroll
  for (int q = 0; q < N; ++q) out[N0 + q][c] = fma(four, a[q], k.add(b[q], d[q]));
}

// The centre components: products and |S| S (3..14) on every row, the centre
// velocities (0..2) on the wall rows 1 and Ny only (see k_centre).
__device__ __forceinline__ void filter_centre(double* const* in, double* const* out, size_t c, size_t lo,
                                              size_t hi, bool wall_row, const F64& k, double four) {
  filter_group<3, 6>(in, out, c, lo, hi, k, four);
  filter_group<9, 6>(in, out, c, lo, hi, k, four);
  if (wall_row) filter_group<0, 3>(in, out, c, lo, hi, k, four);
}

__global__ void __launch_bounds__(256)
k_filter_y(ChlMap map, int s_in) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const unsigned t = (unsigned)lb * blockDim.x + threadIdx.x;
  if (t >= (unsigned)(Nx * (Ny + 2) * Nz)) return;
  const ChlIdx p = chl_split(t, Nx, Ny + 2);
  const int i = p.i, j = p.j, k = p.k;
  const size_t c = cidx(I, i, j, k);
  const size_t pc = (size_t)Nx;
  const F64 f = f64_of(I);
  const double four = I.fk[FK_FOUR];
  if (j >= 1 && j <= Ny) {
    const size_t lo = (j == 1) ? c + pc : c - pc, hi = (j == Ny) ? c - pc : c + pc;
    filter_centre(I.q, I.r, c, lo, hi, j == 1 || j == Ny, f, four);
  }
  I.r[15][c] = fy(I.U[s_in], c, pc, j, 0, Ny + 1, f, four);
  I.r[17][c] = fy(I.W[s_in], c, pc, j, 0, Ny + 1, f, four);
  if (j <= Ny) {
    const size_t v = vidx(I, i, j, k);
    I.r[16][v] = fy(I.V[s_in], v, pc, j, 0, Ny, f, four);
  }
}

// x pass over point pairs: thread (pair, j, k) forms x points i = 2 pair and
// i + 1 from the 16-byte pairs to its left, at itself and to its right
// (periodic; Nx is even and every row starts on a pair, so the pairs are
// 16-byte aligned) and stores its two results as one pair: three vector
// loads and one vector store per component for two points, instead of six
// loads and two stores.  Same arithmetic and operand order as the one-point
// pass, so bit-identical.  r -> q.
template <int N0, int N>
__device__ __forceinline__ void filter_x2_group(double* const* in, double* const* out, size_t cl, size_t cc,
                                                size_t cr, const F64& f, double four) {
  double2 l[N], c[N], r[N];
#pragma unroll
  for (int q = 0; q < N; ++q) {
    const double2* g = reinterpret_cast<const double2*>(in[N0 + q]);
    l[q] = __ldg(g + cl); c[q] = __ldg(g + cc); r[q] = __ldg(g + cr);
  }
#pragma unroll
  for (int q = 0; q < N; ++q)
    reinterpret_cast<double2*>(out[N0 + q])[cc] =
        make_double2(fma(four, c[q].x, f.add(l[q].y, c[q].y)), fma(four, c[q].y, f.add(c[q].x, r[q].x)));
}

__global__ void __launch_bounds__(256)
k_filter_x2(ChlMap map) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const int nxp = Nx / 2;
  const unsigned t = (unsigned)lb * blockDim.x + threadIdx.x;
  if (t >= (unsigned)(nxp * (Ny + 2) * Nz)) return;
  const ChlIdx p = chl_split(t, nxp, Ny + 2);
  const int pi = p.i, j = p.j, k = p.k;
  const int pl = pi == 0 ? nxp - 1 : pi - 1, pr = pi == nxp - 1 ? 0 : pi + 1;
  const F64 f = f64_of(I);
  const double four = I.fk[FK_FOUR];
  double* const* in = I.r;
  double* const* out = I.q;
  // pair indices: row (j, k) of the centre-like layout starts at pair nxp (j + (Ny+2) k)
  const size_t rc = (size_t)nxp * ((size_t)j + (size_t)(Ny + 2) * k);
  if (j >= 1 && j <= Ny) {
    filter_x2_group<3, 6>(in, out, rc + pl, rc + pi, rc + pr, f, four);
    filter_x2_group<9, 6>(in, out, rc + pl, rc + pi, rc + pr, f, four);
    if (j == 1 || j == Ny) filter_x2_group<0, 3>(in, out, rc + pl, rc + pi, rc + pr, f, four);
  }
  filter_x2_group<15, 1>(in, out, rc + pl, rc + pi, rc + pr, f, four);
  filter_x2_group<17, 1>(in, out, rc + pl, rc + pi, rc + pr, f, four);
  if (j <= Ny) {
    const size_t rv = (size_t)nxp * ((size_t)j + (size_t)(Ny + 1) * k);   // the V-like layout
    filter_x2_group<16, 1>(in, out, rv + pl, rv + pi, rv + pr, f, four);
  }
}

// z pass over plane pairs: thread (i, j, pair) forms planes k = 2 pair and
// k + 1 from planes k - 1 .. k + 2 (periodic), so each output takes two
// loads instead of three, all of them independent (the neighbours lie a
// plane apart, mostly in L2).  Same arithmetic and operand order as the
// one-plane pass, so bit-identical.  Nz is even (chl_create: nz even), so
// the planes pair up.  q -> r.
template <int N0, int N>
__device__ __forceinline__ void filter_z2_group(double* const* in, double* const* out, size_t km, size_t ka,
                                                size_t kb, size_t kc, const F64& f, double four) {
  double a[N], b[N], c[N], d[N];
#pragma unroll
  for (int q = 0; q < N; ++q) {
    const double* g = in[N0 + q];
    a[q] = LDG(g + km); b[q] = LDG(g + ka); c[q] = LDG(g + kb); d[q] = LDG(g + kc);
  }
#pragma unroll
  for (int q = 0; q < N; ++q) {
    out[N0 + q][ka] = fma(four, b[q], f.add(a[q], c[q]));
    out[N0 + q][kb] = fma(four, c[q], f.add(b[q], d[q]));
  }
}

__global__ void __launch_bounds__(256)
k_filter_z2(ChlMap map) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const int npair = Nz / 2;
  const unsigned t = (unsigned)lb * blockDim.x + threadIdx.x;
  if (t >= (unsigned)(Nx * (Ny + 2) * npair)) return;
  const ChlIdx p = chl_split(t, Nx, Ny + 2);
  const int i = p.i, j = p.j, k0 = 2 * p.k;
  const int km = k0 == 0 ? Nz - 1 : k0 - 1, kb = k0 + 1, kc = k0 + 2 == Nz ? 0 : k0 + 2;
  const F64 f = f64_of(I);
  const double four = I.fk[FK_FOUR];
  double* const* in = I.q;
  double* const* out = I.r;
  const size_t c0 = cidx(I, i, j, km), c1 = cidx(I, i, j, k0), c2 = cidx(I, i, j, kb), c3 = cidx(I, i, j, kc);
  if (j >= 1 && j <= Ny) {
    filter_z2_group<3, 6>(in, out, c0, c1, c2, c3, f, four);
    filter_z2_group<9, 6>(in, out, c0, c1, c2, c3, f, four);
    if (j == 1 || j == Ny) filter_z2_group<0, 3>(in, out, c0, c1, c2, c3, f, four);
  }
  filter_z2_group<15, 1>(in, out, c0, c1, c2, c3, f, four);
  filter_z2_group<17, 1>(in, out, c0, c1, c2, c3, f, four);
  if (j <= Ny)
    filter_z2_group<16, 1>(in, out, vidx(I, i, j, km), vidx(I, i, j, k0), vidx(I, i, j, kb), vidx(I, i, j, kc), f, four);
}

// ------------------------------------------------------------ L:M, M:M
// One block of CHL_DSMF_THREADS per (centre row jc, chunk of the row's
// chl_dsm_points points); each thread sums its points in a fixed order and
// writes its partials to part[0|1][jc][chunk][thread] (no reduction tree in
// every block: its mostly idle warps would issue an FP64 instruction per
// level for a handful of lanes).  Filtered fields live in r after the three
// passes.  The last block of a row to finish (a counter per row) adds the
// row's partials - thread t the entries t, t + CHL_DSMF_THREADS, ... in
// order, then a fixed-order block tree - and writes the row's coefficient
// -1/2 <LM>/<MM>, then returns the counter to 0.
__device__ __forceinline__ void block_sum2(double* sl, double* sm, double& a, double& b) {
  sl[threadIdx.x] = a; sm[threadIdx.x] = b;
  __syncthreads();
  for (int w = CHL_DSMF_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) { sl[threadIdx.x] += sl[threadIdx.x + w]; sm[threadIdx.x] += sm[threadIdx.x + w]; }
    __syncthreads();
  }
  a = sl[0]; b = sm[0];
}

// -1/2 <LM>/<MM>: the filter and average scales give 1/8 (see the scaling
// note above); L and M are both stored / 216, so <LM>/<MM> = lm/mm (times
// the sqrt(2) that the strain leaves out).  Whole block; every thread gets it.
// Thread t adds the partials of chunks t mod 4 = 0..3 into four chains
// (their loads in flight together: on a small instance this tail is
// latency, not throughput), then the chains in a fixed order.
__device__ __forceinline__ double dsm_row_coef(const ChlInst& I, int jc, double* sl, double* sm) {
  const int np = I.npart;
  const size_t n = (size_t)np * CHL_DSMF_THREADS;
  const double* pl = I.part + (size_t)jc * n + threadIdx.x;
  const double* pm = I.part + (size_t)(I.Ny + 2) * n + (size_t)jc * n + threadIdx.x;
  double l[4] = {0.0, 0.0, 0.0, 0.0}, m[4] = {0.0, 0.0, 0.0, 0.0};
  int c = 0;
  for (; c + 4 <= np; c += 4) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      l[u] += __ldcg(pl + (size_t)(c + u) * CHL_DSMF_THREADS);
      m[u] += __ldcg(pm + (size_t)(c + u) * CHL_DSMF_THREADS);
    }
  }
  for (int u = 0; c < np; ++c, ++u) {
    l[u] += __ldcg(pl + (size_t)c * CHL_DSMF_THREADS);
    m[u] += __ldcg(pm + (size_t)c * CHL_DSMF_THREADS);
  }
  double lm = (l[0] + l[1]) + (l[2] + l[3]), mm = (m[0] + m[1]) + (m[2] + m[3]);
  __syncthreads();
  block_sum2(sl, sm, lm, mm);
  return -0.125 * (lm / mm);
}

// One thread's points of row jc: the diagonal and off-diagonal parts of L:M
// and M:M, each a chain of FMAs straight into its accumulator (the
// off-diagonal scales 1/4 and 1/32 are applied once by the caller).  The
// point set is the plane followed by the reference's duplicated periodic
// column and plane (chl_dsm_points), so every point has weight 1.
// WALL: row 1 or Ny, whose filtered centre velocities were filtered in their
// own right; a template parameter rather than a per-point select, since the
// row is the same for the whole block.
template <bool WALL, bool PAIR>
__device__ __forceinline__ void dsm_sums(const ChlInst& I, int jc, int chunk, double& ald, double& alo,
                                         double& amd, double& amo) {
  const int Nx = I.Nx, Nz = I.Nz;
  const int plane = Nx * Nz, npts = chl_dsm_points(Nx, Nz);
  const double* const* R = I.r;
  const int ppt = I.dsm_ppt;
  for (int m = 0; m < ppt; ++m) {
    const int pidx = chunk * (CHL_DSMF_THREADS * ppt) + m * CHL_DSMF_THREADS + threadIdx.x;
    if (pidx >= npts) break;
    int i, k;
    if (pidx < plane) { i = pidx % Nx; k = pidx / Nx; }
    else {                                   // the duplicated column, plane and (0, 0)
      const int e = pidx - plane;
      i = e < Nz ? 0 : (e < Nz + Nx ? e - Nz : 0);
      k = e < Nz ? e : 0;
    }
    const size_t c = cidx(I, i, jc, k);
    const Faces f = centre_faces(I, R[15], R[16], R[17], i, jc, k);    // 216 x filtered faces
    const Strain h = centre_strain<true, PAIR>(I, f, i, jc, k);               // sqrt(4/216) x 216 x filtered strain
    // M_ij / 216: the 216 of the filtered |S| S_ij terms moves into the
    // strain factor (4/216, as sqrt(4/216) in each of |S| and S_ij, from the
    // scaled reciprocals); L_ij / 216: the filtered velocities are divided
    // once, each product is then one FMA; k_coef's constant carries both
    const double M1 = fma(h.s, h.d1, -LDG(R[9] + c));
    const double M2 = fma(h.s, h.d2, -LDG(R[10] + c));
    const double M3 = fma(h.s, h.d3, -LDG(R[11] + c));
    const double M4 = fma(h.s, h.o12, -LDG(R[12] + c));
    const double M5 = fma(h.s, h.o13, -LDG(R[13] + c));
    const double M6 = fma(h.s, h.o23, -LDG(R[14] + c));
    // 2 x 216 x filtered centre velocities: filtered in their own right on
    // the wall rows, the centre average of the filtered faces elsewhere
    const double fu = WALL ? LDG(R[0] + c) : f.u0 + f.u1;
    const double fv = WALL ? LDG(R[1] + c) : f.v0 + f.v1;
    const double fw = WALL ? LDG(R[2] + c) : f.w0 + f.w1;
    const double gu = fu * (1.0 / 216.0), gv = fv * (1.0 / 216.0);
    const double L1 = fma(-gu, fu, LDG(R[3] + c));
    const double L2 = fma(-gv, fv, LDG(R[4] + c));
    const double L3 = fma(-fw * (1.0 / 216.0), fw, LDG(R[5] + c));
    const double L4 = fma(-gu, fv, LDG(R[6] + c));
    const double L5 = fma(-gu, fw, LDG(R[7] + c));
    const double L6 = fma(-gv, fw, LDG(R[8] + c));
    ald = fma(L1, M1, ald); ald = fma(L2, M2, ald); ald = fma(L3, M3, ald);
    alo = fma(L4, M4, alo); alo = fma(L5, M5, alo); alo = fma(L6, M6, alo);
    amd = fma(M1, M1, amd); amd = fma(M2, M2, amd); amd = fma(M3, M3, amd);
    amo = fma(M4, M4, amo); amo = fma(M5, M5, amo); amo = fma(M6, M6, amo);
  }
}

template <bool PAIR>
__global__ void __launch_bounds__(CHL_DSMF_THREADS)
k_dsm_final(ChlMap map) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Ny = I.Ny;
  const int np = I.npart;
  const int jc = 1 + lb / np, chunk = lb % np;
  double ald = 0.0, alo = 0.0, amd = 0.0, amo = 0.0;
  if (jc == 1 || jc == Ny) dsm_sums<true, PAIR>(I, jc, chunk, ald, alo, amd, amo);
  else dsm_sums<false, PAIR>(I, jc, chunk, ald, alo, amd, amo);
  const size_t n = (size_t)np * CHL_DSMF_THREADS;
  const size_t q = (size_t)jc * n + (size_t)chunk * CHL_DSMF_THREADS + threadIdx.x;
  I.part[q] = fma(0.25, alo, ald);
  I.part[(size_t)(Ny + 2) * n + q] = fma(0.03125, amo, amd);
  __threadfence();
  __shared__ double sl[CHL_DSMF_THREADS], sm[CHL_DSMF_THREADS];
  __shared__ int last;
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(I.dsm_cnt + jc, 1) == np - 1;     // the row's last block
  __syncthreads();
  if (last) {
    __threadfence();
    const double c = dsm_row_coef(I, jc, sl, sm);
    if (threadIdx.x == 0) { I.coef[jc] = c; I.dsm_cnt[jc] = 0; }
  }
}

// ------------------------------------------------------------ nu_t coefficient per row
// The static model's row coefficient (the dynamic model's is written by
// k_dsm_final, and this kernel leaves it alone).
__global__ void k_coef(ChlMap map) {
  chl_pdl_wait();
  const ChlInst& I = map.inst[blockIdx.x];
  const int Ny = I.Ny;
  if (I.LES_model == 2) return;
  for (int jc = threadIdx.x; jc < Ny + 2; jc += blockDim.x) {
    double c = 0.0;
    if (jc >= 1 && jc <= Ny) {
      if (I.LES_model == 1) {
        // van Driest: f = 1 - exp(-d/25/(nu/utau)), utau = dPdx^0.5 (subgrid.f90:581-599)
        const double ut = sqrt(I.scal[CHL_S_DPDX]);
        double f = 1.0 - exp(-I.smag_dwall[jc] / 25.0 / (I.nu / ut));
        if (I.Dirichlet_nu_t == 0) f = 1.0;
        const double cd = I.smag_csdelta[jc] * f;   // Cs*Delta_j*f
        c = cd * cd * 1.41421356237309504880;      // (Cs Delta f)^2 |S| with S holding |S|/sqrt(2)
      } else if (I.LES_model >= 3) {
        c = 1.0;                           // AMD, Vreman: S holds nu_t itself (not launched for them)
      }
    }
    I.coef[jc] = c;
  }
}

// ------------------------------------------------------------ equilibrium log-law wall stress
#define EQWM_KAPPA 0.41
#define EQWM_B 5.2
#define EQWM_ITERS 12
// Newton on f(ut) = ut (ln(h ut/nu)/kappa + B) - |u|.  f is convex and
// increasing, so Newton converges from either side of the root (from the
// left the first step lands right of it, then the iterates decrease).  The
// start is `guess` (the previous stage's u_tau) when it lies above the
// laminar estimate, which the root always does.  Convergence is quadratic
// with relative constant 1/(2 kappa f') < 0.1 (f' = u+ + 1/kappa > 11 where
// the log law applies), so once a correction is below 3e-8 of ut the error
// left after it is below 0.09 * (3e-8)^2 < 1e-16, under half an ulp: the
// iteration stops there and the root agrees with a fixed-count solve to
// rounding.  The log of the
// branch test is reused as the first iterate's when the start is laminar.
// FP64 is the scarce pipe here: h/nu is formed once, 1/kappa is a constant
// multiplier, and each iteration holds one log and one division.
__device__ double eqlog_tau(double u, double h, double nu, double guess) {
  const double inv_k = 1.0 / EQWM_KAPPA;   // folded at compile time
  const double au = fabs(u);
  const double hn = h / nu;
  const double ut_lam = sqrt(au / hn);
  const double yp_lam = hn * ut_lam;
  const double l0 = log(yp_lam);
  const double f0 = ut_lam * fma(l0, inv_k, EQWM_B) - au;
  double ut = ut_lam;
  // log law only above its upper crossing with u+ = y+ (y+ ~ 11)
  if (f0 < 0.0 && yp_lam >= 1.0) {
    const bool warm = guess > ut_lam;
    if (warm) ut = guess;
    for (int it = 0; it < 2 * EQWM_ITERS; ++it) {
      const double lg = (it == 0 && !warm) ? l0 : log(hn * ut);
      const double g = fma(lg, inv_k, EQWM_B);          // u+ at ut
      const double d = fma(ut, g, -au) / (g + inv_k);   // f / f'
      ut = ut - d;
      if (fabs(d) <= 3e-8 * ut) break;
    }
  }
  const double tau = ut * ut;
  return u < 0.0 ? -tau : (u > 0.0 ? tau : 0.0);
}

// CHL_WALL_THREADS-wide blocks: the 2 Nx Nz wall points of a small channel
// are few, and the serial Newton chains are FP64-issue bound, so they are
// spread over as many SMs as there are blocks.
__global__ void __launch_bounds__(CHL_WALL_THREADS)
k_eqwm(ChlMap map, int s_in) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const unsigned t = (unsigned)lb * blockDim.x + threadIdx.x;
  if (t >= (unsigned)(2 * Nx * Nz)) return;
  const ChlIdx p = chl_split(t, Nx, Nz);
  const int a = p.i, k = p.j, wall = p.k;
  const double* U = I.U[s_in];
  const double u = wall == 0 ? U[cidx(I, a, 3, k)] : U[cidx(I, a, Ny - 2, k)];
  const double prev = I.alpha[t];
  I.alpha[t] = eqlog_tau(u, wall == 0 ? I.hb : I.ht, I.nu, sqrt(fabs(prev)));
}

// ------------------------------------------------------------ nu_t (+ wall model rows)
// One thread per centre (i, jc, k), jc = 0..Ny+1.  On the wall-model rows
// (jc = 0, 1 and Ny, Ny+1) nu_t is the mean of the face values at x faces
// i-1 and i: each thread forms face i and takes face i-1 from the lane to
// its left when that lane is on the same row (i > 0), so no thread returns
// before the shuffle.
__global__ void __launch_bounds__(256)
k_nut(ChlMap map, int s_in, int use_wm) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const unsigned t = (unsigned)lb * blockDim.x + threadIdx.x;
  const bool valid = t < (unsigned)(Nx * (Ny + 2) * Nz);
  const ChlIdx p = chl_split(valid ? t : 0u, Nx, Ny + 2);
  const int i = p.i, jc = p.j, k = p.k;
  const bool wmrow = valid && use_wm && I.wall_model != 0 && (jc <= 1 || jc >= Ny);
  const int wall = jc <= 1 ? 0 : 1;
  const double* U = I.U[s_in];
  const double f = wmrow ? wm_face(I, U, i, k, wall) : 0.0;
  const double f_left = __shfl_up_sync(0xffffffffu, f, 1);
  if (!valid) return;
  // stored as nu + nu_t: every consumer adds nu (equations.f90:139-155)
  double* out = I.nut + cidx(I, i, jc, k);
  if (wmrow) {
    const double fl = ((threadIdx.x & 31) > 0 && i > 0) ? f_left : wm_face(I, U, wrap(i - 1, Nx), k, wall);
    *out = I.nu + 0.5 * (fl + f);
  } else if (I.LES_model == 0) {
    *out = I.nu;
  } else if (jc == 0 || jc == Ny + 1) {         // ghost rows: the rule of Dirichlet_nu_t
    const int js = jc == 0 ? 1 : Ny;
    const double sv = I.S[cidx(I, i, js, k)];
    *out = I.nu + nut_ghost(I, chl_pos(I.LES_model >= 3 ? sv : I.coef[js] * sv));
  } else if (I.LES_model >= 3) {                // AMD and Vreman store nu_t itself in S
    *out = I.nu + chl_pos(I.S[cidx(I, i, jc, k)]);
  } else {
    // nu + max(0, c |S|) as one FMA, nu + c |S|, clipped below at nu by the
    // bit patterns (both positive; a NaN, for which max gives 0, gives nu)
    const double nu = I.nu;
    *out = chl_atleast(fma(I.coef[jc], I.S[cidx(I, i, jc, k)], nu), nu);
  }
}

// ------------------------------------------------------------ launchers
extern "C" {
// pair: the x-pair form (k_edges_pair on its row map, blocks of pair threads)
void chl_launch_edges(const ChlMap& m, int nb, int src, int pair, cudaStream_t st) {
  if (pair) chl_launch_pdl(k_edges_pair, dim3(nb), dim3(pair), 0, st, m, src);
  else chl_launch_pdl(k_edges, dim3(nb), dim3(m.tb), 0, st, m, src);
}
void chl_launch_centre(const ChlMap& m, int nb, int s_in, int dsm, int pair, cudaStream_t st) {
  if (dsm && pair) chl_launch_pdl(k_centre<true, true>, dim3(nb), dim3(m.tb), 0, st, m, s_in);
  else if (dsm) chl_launch_pdl(k_centre<true, false>, dim3(nb), dim3(m.tb), 0, st, m, s_in);
  else if (pair) chl_launch_pdl(k_centre<false, true>, dim3(nb), dim3(m.tb), 0, st, m, s_in);
  else chl_launch_pdl(k_centre<false, false>, dim3(nb), dim3(m.tb), 0, st, m, s_in);
}
void chl_launch_filter_y(const ChlMap& m, int nb, int s_in, cudaStream_t st) { chl_launch_pdl(k_filter_y, dim3(nb), dim3(m.tb), 0, st, m, s_in); }
void chl_launch_filter_x(const ChlMap& m, int nb, cudaStream_t st) { chl_launch_pdl(k_filter_x2, dim3(nb), dim3(m.tb), 0, st, m); }
void chl_launch_filter_z(const ChlMap& m, int nb, cudaStream_t st) { chl_launch_pdl(k_filter_z2, dim3(nb), dim3(m.tb), 0, st, m); }
void chl_launch_dsm_final(const ChlMap& m, int nb, int pair, cudaStream_t st) {
  if (pair) chl_launch_pdl(k_dsm_final<true>, dim3(nb), dim3(CHL_DSMF_THREADS), 0, st, m);
  else chl_launch_pdl(k_dsm_final<false>, dim3(nb), dim3(CHL_DSMF_THREADS), 0, st, m);
}
void chl_launch_coef(const ChlMap& m, cudaStream_t st) { chl_launch_pdl(k_coef, dim3(m.n), dim3(128), 0, st, m); }
void chl_launch_eqwm(const ChlMap& m, int nb, int s_in, cudaStream_t st) { chl_launch_pdl(k_eqwm, dim3(nb), dim3(CHL_WALL_THREADS), 0, st, m, s_in); }
void chl_launch_nut(const ChlMap& m, int nb, int s_in, int use_wm, cudaStream_t st) { chl_launch_pdl(k_nut, dim3(nb), dim3(m.tb), 0, st, m, s_in, use_wm); }
}
