// Momentum right-hand side and Runge-Kutta stage update.
//
// Restates compute_rhs_u/v/w (equations.f90:24-468) with the reference's
// interpolations (interpolation.f90:24-105: plain averages in x,z, weighted
// average weight_y_0/1 in y) and fuses the RK3 stage update of
// compute_time_step_RK3 (time_integration.f90:42-44, 59-61, 76-81) and the
// Dirichlet ghost rows of apply_Dirichlet_bc_y (boundary_conditions.f90:239-254).
// Divisions by grid spacings are multiplications by precomputed reciprocals.
#include "chl_common.cuh"

struct RhsArgs {
  int sin, sbase, sout;   // velocity sets: RHS input, stage base (U^n), output
  double c1, c2;          // out = base + dt*(c1*F1 + c2*F)
  int mode;               // 0: stage 1 (store F1), 1: stages 2/3, 2: pressure RHS only
};

__global__ void __launch_bounds__(256)
k_rhs(ChlMap map, RhsArgs a) {
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  long t = (long)lb * blockDim.x + threadIdx.x;
  if (t >= (long)Nx * Ny * Nz) return;
  const int i = (int)(t % Nx);
  const int jc = 1 + (int)((t / Nx) % Ny);
  const int k = (int)(t / ((long)Nx * Ny));
  const int im = wrap(i - 1, Nx), ip = wrap(i + 1, Nx);
  const int km = wrap(k - 1, Nz), kp = wrap(k + 1, Nz);

  const double* __restrict__ U = I.U[a.sin];
  const double* __restrict__ V = I.V[a.sin];
  const double* __restrict__ W = I.W[a.sin];
  const double* __restrict__ nt = I.nut;
  const double nu = I.nu;
  const double* rdxc = I.rdxc; const double* rdxf = I.rdxf;
  const double* rdzc = I.rdzc; const double* rdzf = I.rdzf;
  const double* rdyc = I.rdyc; const double* rdyf = I.rdyf;
  const double* w0 = I.w0; const double* w1 = I.w1;

#define Uc(ii, jj, kk) LDG(U + cidx(I, ii, jj, kk))
#define Wc(ii, jj, kk) LDG(W + cidx(I, ii, jj, kk))
#define Vv(ii, jj, kk) LDG(V + vidx(I, ii, jj, kk))
#define NT(ii, jj, kk) LDG(nt + cidx(I, ii, jj, kk))

  const double rxc = LDG(rdxc + i), rxcp = LDG(rdxc + i + 1);
  const double rxf = LDG(rdxf + i), rxfm = LDG(rdxf + i - 1);
  const double rzc = LDG(rdzc + k), rzcp = LDG(rdzc + k + 1);
  const double rzf = LDG(rdzf + k), rzfm = LDG(rdzf + k - 1);

  // ------------------------------------------------------------------ u
  double Fu, Fv = 0.0, Fw;
  {
    const double u0 = Uc(i, jc, k), uxm = Uc(im, jc, k), uxp = Uc(ip, jc, k);
    const double uym = Uc(i, jc - 1, k), uyp = Uc(i, jc + 1, k);
    const double uzm = Uc(i, jc, km), uzp = Uc(i, jc, kp);
    // -d(uu)/dx: centre values 0.5(U(c-1)+U(c)) at centres i and i+1
    const double ca = 0.5 * (uxm + u0), cb = 0.5 * (u0 + uxp);
    double f = -(cb * cb - ca * ca) * rxf;
    // -d(uv)/dy: u on faces jc-1, jc times v on x-face i
    const double w0a = LDG(w0 + jc - 1), w1a = LDG(w1 + jc - 1);
    const double w0b = LDG(w0 + jc), w1b = LDG(w1 + jc);
    const double uyl = w0a * uym + w1a * u0, uyh = w0b * u0 + w1b * uyp;
    const double vxl = 0.5 * (Vv(i, jc - 1, k) + Vv(ip, jc - 1, k));
    const double vxh = 0.5 * (Vv(i, jc, k) + Vv(ip, jc, k));
    f += -(uyh * vxh - uyl * vxl) * LDG(rdyc + jc);
    // -d(uw)/dz
    const double uzl = 0.5 * (uzm + u0), uzh = 0.5 * (u0 + uzp);
    const double wxl = 0.5 * (Wc(i, jc, km) + Wc(ip, jc, km));
    const double wxh = 0.5 * (Wc(i, jc, k) + Wc(ip, jc, k));
    f += -(uzh * wxh - uzl * wxl) * rzc;
    // viscous
    const double n00 = NT(i, jc, k), n10 = NT(ip, jc, k);
    const double nux1 = nu + n00, nux2 = nu + n10;
    double vis = rxf * (nux2 * rxcp * (uxp - u0) - nux1 * rxc * (u0 - uxm));
    const double nym0 = NT(i, jc - 1, k), nym1 = NT(ip, jc - 1, k);
    const double nyp0 = NT(i, jc + 1, k), nyp1 = NT(ip, jc + 1, k);
    const double nuy1 = nu + 0.5 * (w0a * nym0 + w1a * n00 + w0a * nym1 + w1a * n10);
    const double nuy2 = nu + 0.5 * (w0b * n00 + w1b * nyp0 + w0b * n10 + w1b * nyp1);
    const double t2l = (u0 - uym) * LDG(rdyf + jc - 1), t2h = (uyp - u0) * LDG(rdyf + jc);
    vis += LDG(rdyc + jc) * (nuy2 * t2h - nuy1 * t2l);
    const double nuz1 = nu + 0.25 * (n00 + NT(i, jc, km) + n10 + NT(ip, jc, km));
    const double nuz2 = nu + 0.25 * (n00 + NT(i, jc, kp) + n10 + NT(ip, jc, kp));
    vis += rzc * (nuz2 * rzf * (uzp - u0) - nuz1 * rzfm * (u0 - uzm));
    Fu = f + vis + I.scal[CHL_S_DPDX];
  }
  // ------------------------------------------------------------------ v (face row jv = jc)
  const int jv = jc;
  const bool hasv = jv <= Ny - 1;
  if (hasv) {
    const double v0 = Vv(i, jv, k), vxm = Vv(im, jv, k), vxp = Vv(ip, jv, k);
    const double vym = Vv(i, jv - 1, k), vyp = Vv(i, jv + 1, k);
    const double vzm = Vv(i, jv, km), vzp = Vv(i, jv, kp);
    // -d(vv)/dy: centre values at rows jv and jv+1
    const double ca = 0.5 * (vym + v0), cb = 0.5 * (v0 + vyp);
    double f = -(cb * cb - ca * ca) * LDG(rdyf + jv);
    // -d(uv)/dx: u on y-face jv at x-faces i-1, i; v on those x-faces
    const double w0j = LDG(w0 + jv), w1j = LDG(w1 + jv);
    const double uyl = w0j * Uc(im, jv, k) + w1j * Uc(im, jv + 1, k);
    const double uyh = w0j * Uc(i, jv, k) + w1j * Uc(i, jv + 1, k);
    const double vxl = 0.5 * (vxm + v0), vxh = 0.5 * (v0 + vxp);
    f += -(uyh * vxh - uyl * vxl) * rxc;
    // -d(vw)/dz
    const double vzl = 0.5 * (vzm + v0), vzh = 0.5 * (v0 + vzp);
    const double wyl = w0j * Wc(i, jv, km) + w1j * Wc(i, jv + 1, km);
    const double wyh = w0j * Wc(i, jv, k) + w1j * Wc(i, jv + 1, k);
    f += -(vzh * wyh - vzl * wyl) * rzc;
    // viscous
    const double a0 = NT(i, jv, k), a1 = NT(i, jv + 1, k);
    const double bm0 = NT(im, jv, k), bm1 = NT(im, jv + 1, k);
    const double bp0 = NT(ip, jv, k), bp1 = NT(ip, jv + 1, k);
    const double nux1 = nu + 0.5 * (w0j * bm0 + w1j * bm1 + w0j * a0 + w1j * a1);
    const double nux2 = nu + 0.5 * (w0j * a0 + w1j * a1 + w0j * bp0 + w1j * bp1);
    double vis = rxc * (nux2 * rxf * (vxp - v0) - nux1 * rxfm * (v0 - vxm));
    vis += LDG(rdyf + jv) * ((nu + a1) * LDG(rdyc + jv + 1) * (vyp - v0) - (nu + a0) * LDG(rdyc + jv) * (v0 - vym));
    const double cm0 = NT(i, jv, km), cm1 = NT(i, jv + 1, km);
    const double cp0 = NT(i, jv, kp), cp1 = NT(i, jv + 1, kp);
    const double nuz1 = nu + 0.5 * (w0j * cm0 + w1j * cm1 + w0j * a0 + w1j * a1);
    const double nuz2 = nu + 0.5 * (w0j * a0 + w1j * a1 + w0j * cp0 + w1j * cp1);
    vis += rzc * (nuz2 * rzf * (vzp - v0) - nuz1 * rzfm * (v0 - vzm));
    Fv = f + vis;
  }
  // ------------------------------------------------------------------ w (face k, row jc)
  {
    const double w_0 = Wc(i, jc, k), wxm = Wc(im, jc, k), wxp = Wc(ip, jc, k);
    const double wym = Wc(i, jc - 1, k), wyp = Wc(i, jc + 1, k);
    const double wzm = Wc(i, jc, km), wzp = Wc(i, jc, kp);
    // -d(ww)/dz: centre values at z-centres k and k+1
    const double ca = 0.5 * (wzm + w_0), cb = 0.5 * (w_0 + wzp);
    double f = -(cb * cb - ca * ca) * rzf;
    // -d(uw)/dx
    const double uzl = 0.5 * (Uc(im, jc, k) + Uc(im, jc, kp));
    const double uzh = 0.5 * (Uc(i, jc, k) + Uc(i, jc, kp));
    const double wxl = 0.5 * (wxm + w_0), wxh = 0.5 * (w_0 + wxp);
    f += -(uzh * wxh - uzl * wxl) * rxc;
    // -d(vw)/dy
    const double w0a = LDG(w0 + jc - 1), w1a = LDG(w1 + jc - 1);
    const double w0b = LDG(w0 + jc), w1b = LDG(w1 + jc);
    const double vzl = 0.5 * (Vv(i, jc - 1, k) + Vv(i, jc - 1, kp));
    const double vzh = 0.5 * (Vv(i, jc, k) + Vv(i, jc, kp));
    const double wyl = w0a * wym + w1a * w_0, wyh = w0b * w_0 + w1b * wyp;
    f += -(vzh * wyh - vzl * wyl) * LDG(rdyc + jc);
    // viscous
    const double n0 = NT(i, jc, k), n1 = NT(i, jc, kp);
    const double nm0 = NT(im, jc, k), nm1 = NT(im, jc, kp);
    const double np0 = NT(ip, jc, k), np1 = NT(ip, jc, kp);
    const double nux1 = nu + 0.25 * (n0 + n1 + nm0 + nm1);
    const double nux2 = nu + 0.25 * (n0 + n1 + np0 + np1);
    double vis = rxc * (nux2 * rxf * (wxp - w_0) - nux1 * rxfm * (w_0 - wxm));
    const double ym0 = NT(i, jc - 1, k), ym1 = NT(i, jc - 1, kp);
    const double yp0 = NT(i, jc + 1, k), yp1 = NT(i, jc + 1, kp);
    const double nuy1 = nu + 0.5 * (w0a * ym0 + w1a * n0 + w0a * ym1 + w1a * n1);
    const double nuy2 = nu + 0.5 * (w0b * n0 + w1b * yp0 + w0b * n1 + w1b * yp1);
    const double t2l = (w_0 - wym) * LDG(rdyf + jc - 1), t2h = (wyp - w_0) * LDG(rdyf + jc);
    vis += LDG(rdyc + jc) * (nuy2 * t2h - nuy1 * t2l);
    vis += rzf * ((nu + n1) * rzcp * (wzp - w_0) - (nu + n0) * rzc * (w_0 - wzm));
    Fw = f + vis;
  }
#undef Uc
#undef Wc
#undef Vv
#undef NT
  const size_t ci = cidx(I, i, jc, k);
  const size_t vi = vidx(I, i, jv, k);
  if (a.mode == 2) {           // actual-pressure RHS: keep F only
    I.Fp[0][ci] = Fu; I.Fp[2][ci] = Fw;
    if (hasv) I.Fp[1][vi] = Fv;
    return;
  }
  const double dt = I.scal[CHL_S_DT];
  double* Uo = I.U[a.sout]; double* Vo = I.V[a.sout]; double* Wo = I.W[a.sout];
  const double* Ub = I.U[a.sbase]; const double* Vb = I.V[a.sbase]; const double* Wb = I.W[a.sbase];
  double un, vn = 0.0, wn;
  if (a.mode == 0) {
    I.F1[0][ci] = Fu; I.F1[2][ci] = Fw;
    if (hasv) I.F1[1][vi] = Fv;
    un = Ub[ci] + dt * (a.c2 * Fu);
    wn = Wb[ci] + dt * (a.c2 * Fw);
    if (hasv) vn = Vb[vi] + dt * (a.c2 * Fv);
  } else {
    un = Ub[ci] + dt * (a.c1 * I.F1[0][ci] + a.c2 * Fu);
    wn = Wb[ci] + dt * (a.c1 * I.F1[2][ci] + a.c2 * Fw);
    if (hasv) vn = Vb[vi] + dt * (a.c1 * I.F1[1][vi] + a.c2 * Fv);
  }
  Uo[ci] = un; Wo[ci] = wn;
  if (hasv) Vo[vi] = vn;
  if (jc == 1) { Uo[cidx(I, i, 0, k)] = -un; Wo[cidx(I, i, 0, k)] = -wn; }
  if (jc == Ny) { Uo[cidx(I, i, Ny + 1, k)] = -un; Wo[cidx(I, i, Ny + 1, k)] = -wn; }
}

extern "C" void chl_launch_rhs(const ChlMap& map, int nblocks, int sin, int sbase, int sout,
                               double c1, double c2, int mode, cudaStream_t st) {
  RhsArgs a{sin, sbase, sout, c1, c2, mode};
  k_rhs<<<nblocks, 256, 0, st>>>(map, a);
}
