// Anisotropic minimum-dissipation (AMD) and Vreman eddy viscosities, one
// fused kernel each, one thread per interior centre (rows 1..Ny).  Both write
// the unclipped nu_t into S; k_coef sets the row coefficient to 1 and k_nut
// applies max(.,0), the ghost-row rule of Dirichlet_nu_t and the wall model.
//
// AMD (subgrid.f90:632-874):
//   nu_t = max(0, -C N / D),  C = 0.3,
//   N = sum_k (d^_k u_i)(d^_k u_j) S_ij,   D = sum_kl (d_k u_l)^2,
// d^_k = grid-scaled difference, d_k = derivative; off-diagonal entries are
// interpolated to the centre from the four surrounding edges in the order the
// reference's interpolate_x/y/z calls use (interpolation.f90:24-105), and
// the three mixed products of each S_ij row are formed as written: two from
// centre values, one interpolated after the product.  S_ij is compute_Sij's
// (subgrid.f90:1014-1072) from the edge fields of k_edges.
//
// Vreman (subgrid.f90:897-1004):
//   nu_t = C sqrt(B_b / a_ij a_ij),  C = 2.5 * 0.1^2,
//   b_ij = sum_m dx_m^2 a_mi a_mj,  B_b = b11 b22 - b12^2 + b11 b33 - b13^2 + b22 b33 - b23^2,
// a_ij = du_j/dx_i at the centre, off-diagonals the mean of four edge
// derivatives.  Two U sections of the reference are written 2:ny, 1:ny-1
// where 2:nx, 1:nx-1 are meant (subgrid.f90:930-931,946-947); they start at
// the same index, so element-wise they read the intended values, which is
// what is computed here.
#include "chl_common.cuh"

namespace {

struct StrainRows { double s11, s22, s33, s12, s13, s23; };

__device__ __forceinline__ StrainRows strain_ij(const ChlInst& I, const double* U, const double* V,
                                                const double* W, int i, int jc, int k) {
  const int im = wrap(i - 1, I.Nx), km = wrap(k - 1, I.Nz);
  StrainRows s;
  s.s11 = (LDG(U + cidx(I, i, jc, k)) - LDG(U + cidx(I, im, jc, k))) * LDG(I.rdxc + i);
  s.s22 = (LDG(V + vidx(I, i, jc, k)) - LDG(V + vidx(I, i, jc - 1, k))) * LDG(I.rdyc + jc);
  s.s33 = (LDG(W + cidx(I, i, jc, k)) - LDG(W + cidx(I, i, jc, km))) * LDG(I.rdzc + k);
  const double* E12 = I.E[0]; const double* E13 = I.E[1]; const double* E23 = I.E[2];
  // E = 2 x edge strain; centre value = 1/4 sum of 4 edges = 1/8 sum of E
  s.s12 = 0.125 * ((LDG(E12 + vidx(I, im, jc - 1, k)) + LDG(E12 + vidx(I, i, jc - 1, k)))
                 + (LDG(E12 + vidx(I, im, jc, k)) + LDG(E12 + vidx(I, i, jc, k))));
  s.s13 = 0.125 * ((LDG(E13 + cidx(I, im, jc, km)) + LDG(E13 + cidx(I, i, jc, km)))
                 + (LDG(E13 + cidx(I, im, jc, k)) + LDG(E13 + cidx(I, i, jc, k))));
  s.s23 = 0.125 * ((LDG(E23 + vidx(I, i, jc - 1, km)) + LDG(E23 + vidx(I, i, jc, km)))
                 + (LDG(E23 + vidx(I, i, jc - 1, k)) + LDG(E23 + vidx(I, i, jc, k))));
  return s;
}

__device__ __forceinline__ double avg(double a, double b) { return 0.5 * (a + b); }

}  // namespace

__global__ void __launch_bounds__(256)
k_amd(ChlMap map, int s_in) {
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  long t = (long)lb * blockDim.x + threadIdx.x;
  if (t >= (long)Nx * Ny * Nz) return;
  const int i = (int)(t % Nx);
  const int jc = 1 + (int)((t / Nx) % Ny);
  const int k = (int)(t / ((long)Nx * Ny));
  const int im = wrap(i - 1, Nx), ip = wrap(i + 1, Nx), km = wrap(k - 1, Nz), kp = wrap(k + 1, Nz);
  const double *U = I.U[s_in], *V = I.V[s_in], *W = I.W[s_in];
  auto u = [&](int a, int j, int kk) { return LDG(U + cidx(I, a, j, kk)); };
  auto v = [&](int a, int j, int kk) { return LDG(V + vidx(I, a, j, kk)); };
  auto w = [&](int a, int j, int kk) { return LDG(W + cidx(I, a, j, kk)); };
  // reciprocal spacings: centre widths, and centre-to-centre distances of the
  // faces at i-1 | i (x), jc-1 | jc (y), k-1 | k (z)
  const double rxc = LDG(I.rdxc + i), ryc = LDG(I.rdyc + jc), rzc = LDG(I.rdzc + k);
  const double rxl = LDG(I.rdxf + i - 1), rxr = LDG(I.rdxf + i);
  const double ryl = LDG(I.rdyf + jc - 1), ryr = LDG(I.rdyf + jc);
  const double rzl = LDG(I.rdzf + k - 1), rzr = LDG(I.rdzf + k);

  // --- U row: x diagonal, y and z edge differences (x-interpolated first)
  const double dux = u(i, jc, k) - u(im, jc, k);
  double uy_lo_m = u(im, jc, k) - u(im, jc - 1, k), uy_lo_p = u(i, jc, k) - u(i, jc - 1, k);
  double uy_hi_m = u(im, jc + 1, k) - u(im, jc, k), uy_hi_p = u(i, jc + 1, k) - u(i, jc, k);
  const double Yu = avg(avg(uy_lo_m, uy_lo_p), avg(uy_hi_m, uy_hi_p));
  const double Yu_d = avg(avg(uy_lo_m * ryl, uy_lo_p * ryl), avg(uy_hi_m * ryr, uy_hi_p * ryr));
  const double uz_lo_m = u(im, jc, k) - u(im, jc, km), uz_lo_p = u(i, jc, k) - u(i, jc, km);
  const double uz_hi_m = u(im, jc, kp) - u(im, jc, k), uz_hi_p = u(i, jc, kp) - u(i, jc, k);
  const double Zu = avg(avg(uz_lo_m, uz_lo_p), avg(uz_hi_m, uz_hi_p));
  const double Zu_d = avg(avg(uz_lo_m * rzl, uz_lo_p * rzl), avg(uz_hi_m * rzr, uz_hi_p * rzr));

  // --- V row: y diagonal, x and z edge differences (y-interpolated first)
  const double dvy = v(i, jc, k) - v(i, jc - 1, k);
  const double vx_l_lo = v(i, jc - 1, k) - v(im, jc - 1, k), vx_l_hi = v(i, jc, k) - v(im, jc, k);
  const double vx_r_lo = v(ip, jc - 1, k) - v(i, jc - 1, k), vx_r_hi = v(ip, jc, k) - v(i, jc, k);
  const double Xv = avg(avg(vx_l_lo, vx_l_hi), avg(vx_r_lo, vx_r_hi));
  const double Xv_d = avg(avg(vx_l_lo * rxl, vx_l_hi * rxl), avg(vx_r_lo * rxr, vx_r_hi * rxr));
  const double vz_l_lo = v(i, jc - 1, k) - v(i, jc - 1, km), vz_l_hi = v(i, jc, k) - v(i, jc, km);
  const double vz_r_lo = v(i, jc - 1, kp) - v(i, jc - 1, k), vz_r_hi = v(i, jc, kp) - v(i, jc, k);
  const double Zv = avg(avg(vz_l_lo, vz_l_hi), avg(vz_r_lo, vz_r_hi));
  const double Zv_d = avg(avg(vz_l_lo * rzl, vz_l_hi * rzl), avg(vz_r_lo * rzr, vz_r_hi * rzr));

  // --- W row: z diagonal, x and y edge differences (z-interpolated first)
  const double dwz = w(i, jc, k) - w(i, jc, km);
  const double wx_l_lo = w(i, jc, km) - w(im, jc, km), wx_l_hi = w(i, jc, k) - w(im, jc, k);
  const double wx_r_lo = w(ip, jc, km) - w(i, jc, km), wx_r_hi = w(ip, jc, k) - w(i, jc, k);
  const double Xw = avg(avg(wx_l_lo, wx_l_hi), avg(wx_r_lo, wx_r_hi));
  const double Xw_d = avg(avg(wx_l_lo * rxl, wx_l_hi * rxl), avg(wx_r_lo * rxr, wx_r_hi * rxr));
  const double wy_l_lo = w(i, jc, km) - w(i, jc - 1, km), wy_l_hi = w(i, jc, k) - w(i, jc - 1, k);
  const double wy_r_lo = w(i, jc + 1, km) - w(i, jc, km), wy_r_hi = w(i, jc + 1, k) - w(i, jc, k);
  const double Yw = avg(avg(wy_l_lo, wy_l_hi), avg(wy_r_lo, wy_r_hi));
  const double Yw_d = avg(avg(wy_l_lo * ryl, wy_l_hi * ryl), avg(wy_r_lo * ryr, wy_r_hi * ryr));

  // --- denominator, in the reference's accumulation order
  double D = (dux * dux) * (rxc * rxc);
  D += Yu_d * Yu_d; D += Zu_d * Zu_d;
  D += (dvy * dvy) * (ryc * ryc);
  D += Xv_d * Xv_d; D += Zv_d * Zv_d;
  D += (dwz * dwz) * (rzc * rzc);
  D += Xw_d * Xw_d; D += Yw_d * Yw_d;

  // --- numerator
  const StrainRows s = strain_ij(I, U, V, W, i, jc, k);
  double N = (dux * dux) * s.s11;
  N += (Yu * Yu) * s.s11; N += (Zu * Zu) * s.s11;
  N += (dvy * dvy) * s.s22; N += (Xv * Xv) * s.s22; N += (Zv * Zv) * s.s22;
  N += (dwz * dwz) * s.s33; N += (Xw * Xw) * s.s33; N += (Yw * Yw) * s.s33;
  // S12: k = x (centre values), y (centre values), z (product on z edges, then averaged)
  N += 2.0 * (Xv * dux) * s.s12;
  N += 2.0 * (Yu * dvy) * s.s12;
  const double p12_lo = avg(uz_lo_m, uz_lo_p) * avg(vz_l_lo, vz_l_hi);
  const double p12_hi = avg(uz_hi_m, uz_hi_p) * avg(vz_r_lo, vz_r_hi);
  N += 2.0 * avg(p12_lo, p12_hi) * s.s12;
  // S13: k = x, z (centre values), y (product on y edges, then averaged)
  N += 2.0 * (Xw * dux) * s.s13;
  N += 2.0 * (Zu * dwz) * s.s13;
  const double p13_lo = avg(uy_lo_m, uy_lo_p) * avg(wy_l_lo, wy_l_hi);
  const double p13_hi = avg(uy_hi_m, uy_hi_p) * avg(wy_r_lo, wy_r_hi);
  N += 2.0 * avg(p13_lo, p13_hi) * s.s13;
  // S23: k = y, z (centre values), x (product on x edges, then averaged)
  N += 2.0 * (Yw * dvy) * s.s23;
  N += 2.0 * (Zv * dwz) * s.s23;
  const double p23_l = avg(vx_l_lo, vx_l_hi) * avg(wx_l_lo, wx_l_hi);
  const double p23_r = avg(vx_r_lo, vx_r_hi) * avg(wx_r_lo, wx_r_hi);
  N += 2.0 * avg(p23_l, p23_r) * s.s23;

  I.S[cidx(I, i, jc, k)] = (-0.3 * N) / D;
}

__global__ void __launch_bounds__(256)
k_vreman(ChlMap map, int s_in) {
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  long t = (long)lb * blockDim.x + threadIdx.x;
  if (t >= (long)Nx * Ny * Nz) return;
  const int i = (int)(t % Nx);
  const int jc = 1 + (int)((t / Nx) % Ny);
  const int k = (int)(t / ((long)Nx * Ny));
  const int im = wrap(i - 1, Nx), ip = wrap(i + 1, Nx), km = wrap(k - 1, Nz), kp = wrap(k + 1, Nz);
  const double *U = I.U[s_in], *V = I.V[s_in], *W = I.W[s_in];
  auto u = [&](int a, int j, int kk) { return LDG(U + cidx(I, a, j, kk)); };
  auto v = [&](int a, int j, int kk) { return LDG(V + vidx(I, a, j, kk)); };
  auto w = [&](int a, int j, int kk) { return LDG(W + cidx(I, a, j, kk)); };
  const double rxc = LDG(I.rdxc + i), ryc = LDG(I.rdyc + jc), rzc = LDG(I.rdzc + k);
  const double rxl = LDG(I.rdxf + i - 1), rxr = LDG(I.rdxf + i);
  const double ryl = LDG(I.rdyf + jc - 1), ryr = LDG(I.rdyf + jc);
  const double rzl = LDG(I.rdzf + k - 1), rzr = LDG(I.rdzf + k);
  // a_ij = du_j/dx_i, stored as in the reference: 1 4 5 / 7 2 6 / 8 9 3
  const double a1 = (u(i, jc, k) - u(im, jc, k)) * rxc;
  const double a4 = 0.25 * (v(i, jc, k) - v(im, jc, k)) * rxl + 0.25 * (v(i, jc - 1, k) - v(im, jc - 1, k)) * rxl
                  + 0.25 * (v(ip, jc, k) - v(i, jc, k)) * rxr + 0.25 * (v(ip, jc - 1, k) - v(i, jc - 1, k)) * rxr;
  const double a5 = 0.25 * (w(i, jc, k) - w(im, jc, k)) * rxl + 0.25 * (w(i, jc, km) - w(im, jc, km)) * rxl
                  + 0.25 * (w(ip, jc, k) - w(i, jc, k)) * rxr + 0.25 * (w(ip, jc, km) - w(i, jc, km)) * rxr;
  const double a2 = (v(i, jc, k) - v(i, jc - 1, k)) * ryc;
  const double a7 = 0.25 * (u(i, jc, k) - u(i, jc - 1, k)) * ryl + 0.25 * (u(im, jc, k) - u(im, jc - 1, k)) * ryl
                  + 0.25 * (u(i, jc + 1, k) - u(i, jc, k)) * ryr + 0.25 * (u(im, jc + 1, k) - u(im, jc, k)) * ryr;
  const double a6 = 0.25 * (w(i, jc, k) - w(i, jc - 1, k)) * ryl + 0.25 * (w(i, jc, km) - w(i, jc - 1, km)) * ryl
                  + 0.25 * (w(i, jc + 1, k) - w(i, jc, k)) * ryr + 0.25 * (w(i, jc + 1, km) - w(i, jc, km)) * ryr;
  const double a3 = (w(i, jc, k) - w(i, jc, km)) * rzc;
  const double a8 = 0.25 * (u(i, jc, k) - u(i, jc, km)) * rzl + 0.25 * (u(im, jc, k) - u(im, jc, km)) * rzl
                  + 0.25 * (u(i, jc, kp) - u(i, jc, k)) * rzr + 0.25 * (u(im, jc, kp) - u(im, jc, k)) * rzr;
  const double a9 = 0.25 * (v(i, jc, k) - v(i, jc, km)) * rzl + 0.25 * (v(i, jc - 1, k) - v(i, jc - 1, km)) * rzl
                  + 0.25 * (v(i, jc, kp) - v(i, jc, k)) * rzr + 0.25 * (v(i, jc - 1, kp) - v(i, jc - 1, k)) * rzr;
  // squared cell widths (x(i)-x(i-1))^2 etc.
  const double hx = 1.0 / rxc, hy = 1.0 / ryc, hz = 1.0 / rzc;
  const double dx2 = hx * hx, dy2 = hy * hy, dz2 = hz * hz;
  const double b11 = dx2 * a1 * a1 + dy2 * a7 * a7 + dz2 * a8 * a8;
  const double b22 = dx2 * a4 * a4 + dy2 * a2 * a2 + dz2 * a9 * a9;
  const double b33 = dx2 * a5 * a5 + dy2 * a6 * a6 + dz2 * a3 * a3;
  const double b12 = dx2 * a1 * a4 + dy2 * a7 * a2 + dz2 * a8 * a9;
  const double b13 = dx2 * a1 * a5 + dy2 * a7 * a6 + dz2 * a8 * a3;
  const double b23 = dx2 * a4 * a5 + dy2 * a2 * a6 + dz2 * a9 * a3;
  const double Bb = b11 * b22 - b12 * b12 + b11 * b33 - b13 * b13 + b22 * b33 - b23 * b23;
  double Ab = a1 * a1;
  Ab += a2 * a2; Ab += a3 * a3; Ab += a4 * a4; Ab += a5 * a5;
  Ab += a6 * a6; Ab += a7 * a7; Ab += a8 * a8; Ab += a9 * a9;
  I.S[cidx(I, i, jc, k)] = 2.5 * (0.1 * 0.1) * sqrt(Bb / Ab);
}

extern "C" {
void chl_launch_amd(const ChlMap& m, int nb, int s_in, cudaStream_t st) { k_amd<<<nb, 256, 0, st>>>(m, s_in); }
void chl_launch_vreman(const ChlMap& m, int nb, int s_in, cudaStream_t st) { k_vreman<<<nb, 256, 0, st>>>(m, s_in); }
}
