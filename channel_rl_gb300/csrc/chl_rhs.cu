// Momentum right-hand side and Runge-Kutta stage update.
//
// Restates compute_rhs_u/v/w (equations.f90:24-468) - advection by the
// reference's interpolations (interpolation.f90:24-105: plain averages in x
// and z, weight_y_0/1 averages in y) plus variable-viscosity diffusion - and
// the stage update of compute_time_step_RK3 (time_integration.f90:42-81)
// with the Dirichlet ghost rows of apply_Dirichlet_bc_y
// (boundary_conditions.f90:239-254).
//
// The reference sums each derivative's advective and viscous part per
// component; here the same terms are grouped by the face they live on
// (flux form), so every face value is computed once:
//   * cell centres     : the diagonal fluxes of u (x), v (y), w (z);
//   * xy edges (x-face, y-face, z-centre): uv and the edge viscosity, shared
//                        by the y flux of u and the x flux of v;
//   * xz edges (x-face, y-centre, z-face): uw, shared by u (z) and w (x);
//   * yz edges (x-centre, y-face, z-face): vw, shared by v (z) and w (y).
// The edge viscosities are exactly the reference's averages (nu_y1/nu_y2 of
// compute_rhs_u equal nu_x1/nu_x2 of compute_rhs_v at the same edge, etc.).
// I.nut holds nu + nu_t, so no per-use "nu +" is needed.  The first kernel
// writes the nine face fluxes, the second takes their divergence and
// updates the stage: the FP64 pipe, not HBM, bounds this code, and each
// flux is computed once instead of twice.
//
// The centre and xz-edge fluxes are kept 4 x their value, the xy and yz
// edge fluxes 2 x: the quarter of the x-z edge averages and of the centre
// products -(u+u)^2/4 is then never formed, nor the half of the y-face
// averages, and the centre reciprocals come quadrupled (rdxc4 ...).  The
// update takes the edge fluxes' differences with doubled reciprocals
// (rdxc2 ...), so F is 4 x, and the quarter in its RK coefficients.
// Scalings by powers of two are exact.  The y-face value of u (and w) is
// u_a + w1 (u_b - u_a), the weighted average with w0 = 1 - w1, whose
// difference u_b - u_a is also the face's y derivative: one FMA on top of a
// difference the viscous flux needs anyway.
#include "chl_common.cuh"

// flux fields: centre-like (rows 1..Ny): 0 GUx, 1 GVy, 2 GWz, 3 GUz, 4 GWx;
// V-like (rows 0..Ny): 5 GUy, 6 GVx, 7 GVz, 8 GWy
enum { G_UX = 0, G_VY, G_WZ, G_UZ, G_WX, G_UY, G_VX, G_VZ, G_WY };

__global__ void __launch_bounds__(256)
k_flux(ChlMap map, int sin) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const unsigned t = (unsigned)lb * blockDim.x + threadIdx.x;
  if (t >= (unsigned)(Nx * (Ny + 1) * Nz)) return;
  const ChlIdx p = chl_split(t, Nx, Ny + 1);
  const int i = p.i, j = p.j, k = p.k;
  const int im = wrap(i - 1, Nx), ip = wrap(i + 1, Nx);
  const int km = wrap(k - 1, Nz), kp = wrap(k + 1, Nz);
  const double* __restrict__ U = I.U[sin];
  const double* __restrict__ V = I.V[sin];
  const double* __restrict__ W = I.W[sin];
  const double* __restrict__ nt = I.nut;   // nu + nu_t
  double* const* G = I.G;
#define UC(ii, jj, kk) LDG(U + cidx(I, ii, jj, kk))
#define WC(ii, jj, kk) LDG(W + cidx(I, ii, jj, kk))
#define VV(ii, jj, kk) LDG(V + vidx(I, ii, jj, kk))
#define NT(ii, jj, kk) LDG(nt + cidx(I, ii, jj, kk))
  const double rxf = LDG(I.rdxf + i), rzf = LDG(I.rdzf + k), ryf = LDG(I.rdyf + j);
  const double w0 = LDG(I.w0 + j), w1 = LDG(I.w1 + j);
  // row j and j+1 values shared by the xy and yz edges (y-face jv = j)
  const double u_a = UC(i, j, k), u_b = UC(i, j + 1, k);
  const double w_a = WC(i, j, k), w_b = WC(i, j + 1, k);
  const double v_0 = VV(i, j, k);
  const double n_a = NT(i, j, k), n_b = NT(i, j + 1, k);
  const double nx_a = n_a + NT(ip, j, k);   // x pair of row j: the xy and xz edges share it
  {  // yz edge (x-centre i, y-face j, z-face k): vw, nu -> GVz, GWy (both 2 x)
    const double v_z = VV(i, j, kp);
    const double dw = w_b - w_a;
    const double wy = fma(w1, dw, w_a);
    const double vw = wy * (v_0 + v_z);
    const double nyz = fma(w0, n_a + NT(i, j, kp), w1 * (n_b + NT(i, j + 1, kp)));
    const size_t e = vidx(I, i, j, k);
    G[G_VZ][e] = fma(nyz, (v_z - v_0) * rzf, -vw);
    G[G_WY][e] = fma(nyz, dw * ryf, -vw);
  }
  if (j >= 1 && j <= Ny) {
    const int jc = j;
    const size_t c = cidx(I, i, jc, k);
    {  // cell centre: diagonal fluxes, 4 x (nu du/dx - ((u+u)/2)^2)
      const double um = UC(im, jc, k), vm = VV(i, jc - 1, k), wm = WC(i, jc, km);
      const double su = um + u_a, sv = vm + v_0, sw = wm + w_a;
      G[G_UX][c] = fma(-su, su, n_a * LDG(I.rdxc4 + i) * (u_a - um));
      G[G_VY][c] = fma(-sv, sv, n_a * LDG(I.rdyc4 + jc) * (v_0 - vm));
      G[G_WZ][c] = fma(-sw, sw, n_a * LDG(I.rdzc4 + k) * (w_a - wm));
    }
    {  // xz edge (x-face i, y-centre jc, z-face k): uw, nu -> GUz, GWx (all 4 x)
      const double u_z = UC(i, jc, kp), w_p = WC(ip, jc, k);
      const double uw = (u_a + u_z) * (w_a + w_p);
      const double nxz = nx_a + (NT(i, jc, kp) + NT(ip, jc, kp));
      G[G_UZ][c] = fma(nxz, (u_z - u_a) * rzf, -uw);
      G[G_WX][c] = fma(nxz, (w_p - w_a) * rxf, -uw);
    }
  }
  {  // xy edge (x-face i, y-face j, z-centre k): uv, nu -> GUy, GVx (both 2 x)
    const double v_p = VV(ip, j, k);
    const double du = u_b - u_a;
    const double uy = fma(w1, du, u_a);                  // u on the y-face
    const double uv = uy * (v_0 + v_p);                  // 2 u v (v = 0.5 (v0+vp))
    const double nxy = fma(w0, nx_a, w1 * (n_b + NT(ip, j + 1, k)));   // 2 nu
    const size_t e = vidx(I, i, j, k);
    G[G_UY][e] = fma(nxy, du * ryf, -uv);
    G[G_VX][e] = fma(nxy, (v_p - v_0) * rxf, -uv);
  }
#undef UC
#undef WC
#undef VV
#undef NT
  (void)km; (void)im;
}

struct RhsArgs {
  int sbase, sout;        // velocity sets: stage base (U^n), output
  int stage;              // RK3 stage 0..2: out = base + dt (c1 F1 + c2 F) (chl_put_dt's products)
  int mode;               // 0: stage 1 (store F1), 1: stages 2/3, 2: actual-pressure RHS only
};

__global__ void __launch_bounds__(256)
k_rhs_update(ChlMap map, RhsArgs a) {
  chl_pdl_wait();
  int lb;
  const ChlInst& I = map.inst[chl_find(map, blockIdx.x, lb)];
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const unsigned t = (unsigned)lb * blockDim.x + threadIdx.x;
  if (t >= (unsigned)(Nx * Ny * Nz)) return;
  const ChlIdx p = chl_split(t, Nx, Ny);
  const int i = p.i, jc = 1 + p.j, k = p.k;
  const int im = wrap(i - 1, Nx), ip = wrap(i + 1, Nx);
  const int km = wrap(k - 1, Nz), kp = wrap(k + 1, Nz);
  const double* const* G = I.G;
  const double rxc = LDG(I.rdxc + i), rxf = LDG(I.rdxf + i);
  const double rzc = LDG(I.rdzc + k), rzf = LDG(I.rdzf + k);
  const double ryc2 = LDG(I.rdyc2 + jc);   // the xy and yz edge fluxes are 2 x, the others 4 x
  const size_t c = cidx(I, i, jc, k);
  const size_t e = vidx(I, i, jc, k), em = vidx(I, i, jc - 1, k);
  const F64 f = f64_of(I);   // sums, differences, products as register FMAs (bit-identical)
  // u at (x-face i, row jc, z-centre k)
  double Fu = f.mul(f.sub(LDG(G[G_UX] + cidx(I, ip, jc, k)), LDG(G[G_UX] + c)), rxf);
  Fu = fma(f.sub(LDG(G[G_UY] + e), LDG(G[G_UY] + em)), ryc2, Fu);
  Fu = fma(f.sub(LDG(G[G_UZ] + c), LDG(G[G_UZ] + cidx(I, i, jc, km))), rzc, Fu);
  Fu = fma(I.fk[FK_FOUR], I.scal[CHL_S_DPDX], Fu);   // the fluxes, so F, are 4 x (4 dPdx is exact)
  // w at (x-centre i, row jc, z-face k)
  double Fw = f.mul(f.sub(LDG(G[G_WX] + c), LDG(G[G_WX] + cidx(I, im, jc, k))), rxc);
  Fw = fma(f.sub(LDG(G[G_WY] + e), LDG(G[G_WY] + em)), ryc2, Fw);
  Fw = fma(f.sub(LDG(G[G_WZ] + cidx(I, i, jc, kp)), LDG(G[G_WZ] + c)), rzf, Fw);
  // v at (x-centre i, y-face jv = jc, z-centre k)
  const bool hasv = jc <= Ny - 1;
  double Fv = 0.0;
  if (hasv) {
    Fv = f.mul(f.sub(LDG(G[G_VX] + e), LDG(G[G_VX] + vidx(I, im, jc, k))), LDG(I.rdxc2 + i));
    Fv = fma(f.sub(LDG(G[G_VY] + cidx(I, i, jc + 1, k)), LDG(G[G_VY] + c)), LDG(I.rdyf + jc), Fv);
    Fv = fma(f.sub(LDG(G[G_VZ] + e), LDG(G[G_VZ] + vidx(I, i, jc, km))), LDG(I.rdzc2 + k), Fv);
  }
  if (a.mode == 2) {           // actual-pressure RHS: keep F only, at its own scale
    I.Fp[0][c] = 0.25 * Fu; I.Fp[2][c] = 0.25 * Fw;
    if (hasv) I.Fp[1][e] = 0.25 * Fv;
    return;
  }
  // out = base + dt (c1 F1 + c2 F) as two FMAs per component; the products
  // dt c / 4 (F1, F are 4 x) are formed once per step where dt is set
  const double dc1 = I.scal[CHL_S_DC + 2 * a.stage], dc2 = I.scal[CHL_S_DC + 2 * a.stage + 1];
  double* Uo = I.U[a.sout]; double* Vo = I.V[a.sout]; double* Wo = I.W[a.sout];
  const double* Ub = I.U[a.sbase]; const double* Vb = I.V[a.sbase]; const double* Wb = I.W[a.sbase];
  double un, vn = 0.0, wn;
  if (a.mode == 0) {
    I.F1[0][c] = Fu; I.F1[2][c] = Fw;
    if (hasv) I.F1[1][e] = Fv;
    un = fma(dc2, Fu, Ub[c]);
    wn = fma(dc2, Fw, Wb[c]);
    if (hasv) vn = fma(dc2, Fv, Vb[e]);
  } else {
    un = fma(dc1, I.F1[0][c], fma(dc2, Fu, Ub[c]));
    wn = fma(dc1, I.F1[2][c], fma(dc2, Fw, Wb[c]));
    if (hasv) vn = fma(dc1, I.F1[1][e], fma(dc2, Fv, Vb[e]));
  }
  Uo[c] = un; Wo[c] = wn;
  if (hasv) Vo[e] = vn;
  if (jc == 1) { Uo[cidx(I, i, 0, k)] = -un; Wo[cidx(I, i, 0, k)] = -wn; }
  if (jc == Ny) { Uo[cidx(I, i, Ny + 1, k)] = -un; Wo[cidx(I, i, Ny + 1, k)] = -wn; }
}

extern "C" {
void chl_launch_flux(const ChlMap& map, int nb_edge, int sin, cudaStream_t st) {
  chl_launch_pdl(k_flux, dim3(nb_edge), dim3(map.tb), 0, st, map, sin);
}
void chl_launch_update(const ChlMap& map, int nb_pt, int sbase, int sout, int stage, int mode, cudaStream_t st) {
  RhsArgs a{sbase, sout, stage, mode};
  chl_launch_pdl(k_rhs_update, dim3(nb_pt), dim3(map.tb), 0, st, map, a);
}
}
