// Anisotropic minimum-dissipation (AMD) and Vreman eddy viscosities, one
// fused kernel each, one thread per interior centre (rows 1..Ny).  Both write
// the unclipped nu_t into S and, in the same pass, nu + nu_t with k_nut's
// rules for these models (write_nut_rows): max(., 0), the ghost-row rule of
// Dirichlet_nu_t and, when use_wm, the wall-model rows - so the step runs the
// wall-stress kernels first and no separate nu_t pass.
//
// AMD (subgrid.f90:632-874):
//   nu_t = max(0, -C N / D),  C = 0.3,
//   N = sum_k (d^_k u_i)(d^_k u_j) S_ij,   D = sum_kl (d_k u_l)^2,
// d^_k = grid-scaled difference, d_k = derivative; off-diagonal entries are
// interpolated to the centre from the four surrounding edges in the order the
// reference's interpolate_x/y/z calls use (interpolation.f90:24-105), and
// the three mixed products of each S_ij row are formed as written: two from
// centre values, one interpolated after the product.  S_ij is compute_Sij's
// (subgrid.f90:1014-1072), formed from the same edge sums.  The halves and
// quarters of the interpolations are folded into constants (0.0625,
// 0.03125): the FP64 pipe bounds these kernels.
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

// Edge differences around a centre (device indices i, jc, k).  For each
// off-diagonal velocity gradient the four edge differences are summed in
// two pairs: s?L/s?H are the two-point sums on the near/far edge in the
// derivative direction (2 x the reference's first interpolation), s = sL+sH
// (4 x the centre value) and d = rl sL + rr sH (4 x the centre derivative,
// the edge differences divided by their centre-to-centre spacings first;
// along the uniform x and z that is r (sL + sH)).
// The centre strain of compute_Sij (subgrid.f90:1014-1072) is the same sums:
// S12 = (dUy + dVx)/8 from the four edges, etc.
struct Grad {
  double dux, dvy, dwz;                  // diagonal differences
  double uyL, uyH, uzL, uzH;             // U: y and z edge pair sums
  double vxL, vxR, vzL, vzH;             // V: x and z
  double wxL, wxR, wyL, wyH;             // W: x and y
  double dUy, dUz, dVx, dVz, dWx, dWy;   // 4 x centre derivatives
  double rxc, ryc, rzc;
};

__device__ __forceinline__ Grad gradients(const ChlInst& I, const double* U, const double* V, const double* W,
                                          int i, int jc, int k) {
  const int im = wrap(i - 1, I.Nx), ip = wrap(i + 1, I.Nx), km = wrap(k - 1, I.Nz), kp = wrap(k + 1, I.Nz);
  auto u = [&](int a, int j, int kk) { return LDG(U + cidx(I, a, j, kk)); };
  auto v = [&](int a, int j, int kk) { return LDG(V + vidx(I, a, j, kk)); };
  auto w = [&](int a, int j, int kk) { return LDG(W + cidx(I, a, j, kk)); };
  const double rxl = LDG(I.rdxf + i - 1), rxr = LDG(I.rdxf + i);
  const double ryl = LDG(I.rdyf + jc - 1), ryr = LDG(I.rdyf + jc);
  const double rzl = LDG(I.rdzf + k - 1), rzr = LDG(I.rdzf + k);
  Grad g;
  g.rxc = LDG(I.rdxc + i); g.ryc = LDG(I.rdyc + jc); g.rzc = LDG(I.rdzc + k);
  const double u0 = u(i, jc, k), um = u(im, jc, k);
  const double v0 = v(i, jc, k), vm = v(i, jc - 1, k);
  const double w0 = w(i, jc, k), wm = w(i, jc, km);
  g.dux = u0 - um; g.dvy = v0 - vm; g.dwz = w0 - wm;
  // U at x-faces im, i
  g.uyL = (um - u(im, jc - 1, k)) + (u0 - u(i, jc - 1, k));
  g.uyH = (u(im, jc + 1, k) - um) + (u(i, jc + 1, k) - u0);
  g.uzL = (um - u(im, jc, km)) + (u0 - u(i, jc, km));
  g.uzH = (u(im, jc, kp) - um) + (u(i, jc, kp) - u0);
  // V at y-faces jc-1, jc
  const double vmm = v(im, jc - 1, k), vm0 = v(im, jc, k);
  g.vxL = (vm - vmm) + (v0 - vm0);
  g.vxR = (v(ip, jc - 1, k) - vm) + (v(ip, jc, k) - v0);
  g.vzL = (vm - v(i, jc - 1, km)) + (v0 - v(i, jc, km));
  g.vzH = (v(i, jc - 1, kp) - vm) + (v(i, jc, kp) - v0);
  // W at z-faces km, k
  g.wxL = (wm - w(im, jc, km)) + (w0 - w(im, jc, k));
  g.wxR = (w(ip, jc, km) - wm) + (w(ip, jc, k) - w0);
  g.wyL = (wm - w(i, jc - 1, km)) + (w0 - w(i, jc - 1, k));
  g.wyH = (w(i, jc + 1, km) - wm) + (w(i, jc + 1, k) - w0);
  // y is stretched: each edge pair by its own spacing; x and z are uniform
  // (checked at creation), so one spacing times the pair sum
  (void)rxr; (void)rzr;
  g.dUy = fma(ryl, g.uyL, ryr * g.uyH); g.dUz = rzl * (g.uzL + g.uzH);
  g.dVx = rxl * (g.vxL + g.vxR); g.dVz = rzl * (g.vzL + g.vzH);
  g.dWx = rxl * (g.wxL + g.wxR); g.dWy = fma(ryl, g.wyL, ryr * g.wyH);
  return g;
}

// nu + nu_t for the interior centre (i, jc, k) from its unclipped value v,
// plus the ghost row next to the first and last interior rows; with the
// wall model on, rows 0, 1 and Ny, Ny+1 take the mean of the wall-model face
// values at x faces i-1 and i (face i-1 from the lane to the left when that
// lane is on the same row, i > 0).  Every lane of the warp reaches the
// shuffle; lanes past the instance's last centre carry valid = false.
__device__ __forceinline__ void write_nut_rows(const ChlInst& I, const double* U, int i, int jc, int k, double v,
                                               int use_wm, bool valid) {
  const int Ny = I.Ny;
  const bool wmrow = valid && use_wm && I.wall_model != 0 && (jc == 1 || jc == Ny);
  const int wall = jc == 1 ? 0 : 1;
  const double f = wmrow ? wm_face(I, U, i, k, wall) : 0.0;
  const double f_left = __shfl_up_sync(0xffffffffu, f, 1);
  if (!valid) return;
  const double nu = I.nu;
  double* nt = I.nut;
  if (wmrow) {
    const double fl = ((threadIdx.x & 31) > 0 && i > 0) ? f_left : wm_face(I, U, wrap(i - 1, I.Nx), k, wall);
    const double w = 0.5 * (fl + f);
    nt[cidx(I, i, jc, k)] = nu + w;
    nt[cidx(I, i, jc == 1 ? 0 : Ny + 1, k)] = nu + w;
    return;
  }
  const double vc = chl_pos(v);
  nt[cidx(I, i, jc, k)] = nu + vc;
  if (jc == 1) nt[cidx(I, i, 0, k)] = nu + nut_ghost(I, vc);
  if (jc == Ny) nt[cidx(I, i, Ny + 1, k)] = nu + nut_ghost(I, vc);
}

}  // namespace

__global__ void __launch_bounds__(256)
k_amd(ChlMap map, int s_in, int use_wm) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const unsigned t = (unsigned)lb * blockDim.x + threadIdx.x;
  const bool valid = t < (unsigned)(Nx * Ny * Nz);
  const ChlIdx p = chl_split(valid ? t : 0u, Nx, Ny);   // lanes past the end compute point 0 and write nothing
  const int i = p.i, jc = 1 + p.j, k = p.k;
  const Grad g = gradients(I, I.U[s_in], I.V[s_in], I.W[s_in], i, jc, k);
  // centre strain: diagonal S_ii; 8 S_ij off the diagonal
  const double s11 = g.dux * g.rxc, s22 = g.dvy * g.ryc, s33 = g.dwz * g.rzc;
  const double t12 = g.dUy + g.dVx, t13 = g.dUz + g.dWx, t23 = g.dVz + g.dWy;
  // grid-scaled centre differences, 4 x: Yu, Zu, Xv, Zv, Xw, Yw
  const double Yu = g.uyL + g.uyH, Zu = g.uzL + g.uzH, Xv = g.vxL + g.vxR;
  const double Zv = g.vzL + g.vzH, Xw = g.wxL + g.wxR, Yw = g.wyL + g.wyH;
  // Numerator and denominator are both formed 16 x (their ratio is what
  // counts), which takes the 1/16 of the 4 x off-diagonal terms out.
  // denominator: sum of squared centre derivatives (the off-diagonal ones are 4 x)
  double q = g.dUy * g.dUy;
  q = fma(g.dUz, g.dUz, q); q = fma(g.dVx, g.dVx, q); q = fma(g.dVz, g.dVz, q);
  q = fma(g.dWx, g.dWx, q); q = fma(g.dWy, g.dWy, q);
  double D = s11 * s11; D = fma(s22, s22, D); D = fma(s33, s33, D);
  D = fma(16.0, D, q);                                   // 16 x
  // numerator: sum_k (d^_k u_i)(d^_k u_j) S_ij with the reference's product
  // forms; the third mixed term of each S_ij is the edge product averaged.
  const double u4 = 4.0 * g.dux, v4 = 4.0 * g.dvy, w4 = 4.0 * g.dwz;
  const double a11 = fma(u4, u4, fma(Yu, Yu, Zu * Zu));   // 16 x
  const double a22 = fma(v4, v4, fma(Xv, Xv, Zv * Zv));
  const double a33 = fma(w4, w4, fma(Xw, Xw, Yw * Yw));
  const double a12 = fma(0.5, fma(g.uzL, g.vzL, g.uzH * g.vzH), fma(Xv, g.dux, Yu * g.dvy));
  const double a13 = fma(0.5, fma(g.uyL, g.wyL, g.uyH * g.wyH), fma(Xw, g.dux, Zu * g.dwz));
  const double a23 = fma(0.5, fma(g.vxL, g.wxL, g.vxR * g.wxR), fma(Yw, g.dvy, Zv * g.dwz));
  double N = a11 * s11;
  N = fma(a22, s22, N); N = fma(a33, s33, N);
  N = fma(a12, t12, N); N = fma(a13, t13, N); N = fma(a23, t23, N);
  const double v = (-0.3 * N) / D;
  if (valid) I.S[cidx(I, i, jc, k)] = v;
  write_nut_rows(I, I.U[s_in], i, jc, k, v, use_wm, valid);
}

__global__ void __launch_bounds__(256)
k_vreman(ChlMap map, int s_in, int use_wm) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const unsigned t = (unsigned)lb * blockDim.x + threadIdx.x;
  const bool valid = t < (unsigned)(Nx * Ny * Nz);
  const ChlIdx p = chl_split(valid ? t : 0u, Nx, Ny);
  const int i = p.i, jc = 1 + p.j, k = p.k;
  const Grad g = gradients(I, I.U[s_in], I.V[s_in], I.W[s_in], i, jc, k);
  // a_ij = du_j/dx_i (reference layout 1 4 5 / 7 2 6 / 8 9 3); the
  // off-diagonal entries are kept 4 x (the 1/16 is folded below)
  const double a1 = g.dux * g.rxc, a2 = g.dvy * g.ryc, a3 = g.dwz * g.rzc;
  const double a4 = g.dVx, a5 = g.dWx, a7 = g.dUy, a6 = g.dWy, a8 = g.dUz, a9 = g.dVz;
  const double hx = LDG(I.hx2 + i), hy = LDG(I.hy2 + jc), hz = LDG(I.hz2 + k);
  const double qx = 0.0625 * hx, qy = 0.0625 * hy, qz = 0.0625 * hz;
  // b_ij = sum_m dx_m^2 a_mi a_mj
  const double b11 = fma(hx * a1, a1, fma(qy * a7, a7, qz * a8 * a8));
  const double b22 = fma(qx * a4, a4, fma(hy * a2, a2, qz * a9 * a9));
  const double b33 = fma(qx * a5, a5, fma(qy * a6, a6, hz * a3 * a3));
  const double hx4 = 0.25 * hx, hy4 = 0.25 * hy, hz4 = 0.25 * hz;
  const double b12 = fma(hx4 * a1, a4, fma(hy4 * a7, a2, qz * a8 * a9));
  const double b13 = fma(hx4 * a1, a5, fma(qy * a7, a6, hz4 * a8 * a3));
  const double b23 = fma(qx * a4, a5, fma(hy4 * a2, a6, hz4 * a9 * a3));
  const double Bb = b11 * b22 - b12 * b12 + b11 * b33 - b13 * b13 + b22 * b33 - b23 * b23;
  double Ab = a1 * a1;
  Ab = fma(a2, a2, Ab); Ab = fma(a3, a3, Ab);
  double Ao = a4 * a4;
  Ao = fma(a5, a5, Ao); Ao = fma(a6, a6, Ao); Ao = fma(a7, a7, Ao); Ao = fma(a8, a8, Ao); Ao = fma(a9, a9, Ao);
  Ab = fma(0.0625, Ao, Ab);
  const double v = 2.5 * (0.1 * 0.1) * chl_sqrt(Bb / Ab);
  if (valid) I.S[cidx(I, i, jc, k)] = v;
  write_nut_rows(I, I.U[s_in], i, jc, k, v, use_wm, valid);
}

extern "C" {
void chl_launch_amd(const ChlMap& m, int nb, int s_in, int use_wm, cudaStream_t st) { chl_launch_pdl(k_amd, dim3(nb), dim3(m.tb), 0, st, m, s_in, use_wm); }
void chl_launch_vreman(const ChlMap& m, int nb, int s_in, int use_wm, cudaStream_t st) { chl_launch_pdl(k_vreman, dim3(nb), dim3(m.tb), 0, st, m, s_in, use_wm); }
}
