// Multi-core CPU restatement of the reference's LES step — TEST AND
// BASELINE INFRASTRUCTURE ONLY (the timed host-core baseline of bench.py and
// a cross-check of the NumPy oracle; never part of the product path).
//
// It follows the Fortran reference routine by routine, with the same
// array extents (Fortran 1-based indexing through small accessors) and
// the same pass structure:
//   compute_dt                     time_integration.f90:102-150
//   compute_time_step_RK3          time_integration.f90:24-96
//   sgs_dynamic_Smagorinsky        subgrid.f90:379-537 (filter_xzy :140-190, compute_Sij :1014-1072)
//   sgs_Smagorinsky                subgrid.f90:563-612 (from its formula, Cs from the caller)
//   AMD, Vreman                    subgrid.f90:632-874, 897-1004 (ghost rows :858-871, 991-1002)
//   compute_wall_model             wallmodel.f90:23-46 (+ the equilibrium log law of the build)
//   compute_rhs_u/v/w              equations.f90:24-468
//   apply_boundary_conditions      boundary_conditions.f90:20-254 (P>=2 semantics)
//   compute_projection_step        projection.f90:20-214 (own mixed-radix FFT, Thomas elimination)
//   compute_dPx_for_constant_mass_flow  mass_flow.f90:113-166
// OpenMP parallelises the outer (z or plane) loop of every pass, standing
// in for the reference's MPI z-slabs.  Parity unpinned, like the oracle it
// is checked against (tests/test_refcpu_cpu.py).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef std::complex<double> cplx;

struct A3 {                 // Fortran array a(1:n1, 1:n2, 1:n3)
  int n1 = 0, n2 = 0, n3 = 0;
  std::vector<double> v;
  void init(int a, int b, int c) { n1 = a; n2 = b; n3 = c; v.assign((size_t)a * b * c, 0.0); }
  inline double& operator()(int i, int j, int k) { return v[(size_t)(i - 1) + (size_t)n1 * ((size_t)(j - 1) + (size_t)n2 * (k - 1))]; }
  inline double operator()(int i, int j, int k) const { return v[(size_t)(i - 1) + (size_t)n1 * ((size_t)(j - 1) + (size_t)n2 * (k - 1))]; }
};

const double RKT[3] = {8.0 / 15.0, 2.0 / 3.0, 1.0};
const double RKC[3][3] = {{8.0 / 15.0, 0.0, 0.0}, {0.25, 5.0 / 12.0, 0.0}, {0.25, 0.0, 0.75}};

// ---------------------------------------------------------------- FFT (radix 2/3/4, Stockham)
struct FFT {
  int N = 0;
  std::vector<cplx> tw;
  void init(int n) {
    N = n;
    tw.resize(n);
    const double pi = 4.0 * std::atan(1.0);
    for (int m = 0; m < n; ++m) tw[m] = cplx(std::cos(2 * pi * m / n), -std::sin(2 * pi * m / n));
  }
  // in place on x (stride 1), work buffer y; sign: false forward, true inverse (unnormalised)
  void run(cplx* x, cplx* y, bool inv) const {
    int Ns = 1, rem = N;
    cplx *src = x, *dst = y;
    while (rem > 1) {
      const int R = rem % 4 == 0 ? 4 : (rem % 3 == 0 ? 3 : 2);
      const int nb = N / R, ts = N / (Ns * R);
      for (int j = 0; j < nb; ++j) {
        const int jm = j % Ns;
        cplx v[4];
        for (int r = 0; r < R; ++r) v[r] = src[j + r * nb];
        if (Ns > 1)
          for (int r = 1; r < R; ++r) { cplx t = tw[jm * r * ts]; if (inv) t = std::conj(t); v[r] *= t; }
        if (R == 2) { cplx a = v[0], b = v[1]; v[0] = a + b; v[1] = a - b; }
        else if (R == 4) {
          cplx a = v[0] + v[2], b = v[0] - v[2], c = v[1] + v[3], e = v[1] - v[3];
          cplx d = inv ? cplx(-e.imag(), e.real()) : cplx(e.imag(), -e.real());
          v[0] = a + c; v[2] = a - c; v[1] = b + d; v[3] = b - d;
        } else {
          const double s3 = 0.86602540378443864676;
          cplx s = v[1] + v[2], d = v[1] - v[2], t = v[0] - 0.5 * s;
          cplx m = inv ? cplx(-s3 * d.imag(), s3 * d.real()) : cplx(s3 * d.imag(), -s3 * d.real());
          v[0] = v[0] + s; v[1] = t + m; v[2] = t - m;
        }
        const int idx = (j / Ns) * Ns * R + jm;
        for (int r = 0; r < R; ++r) dst[idx + r * Ns] = v[r];
      }
      std::swap(src, dst);
      Ns *= R; rem /= R;
    }
    if (src != x) std::memcpy(x, src, sizeof(cplx) * N);
  }
};

struct Ref {
  int nx, ny, nz, nxg, nyg, nzg, Nx, Nz;
  double nu, CFL, dPdx, Cs, Q0 = 0, dt = 0, t = 0;
  int x_mass_cte, LES_model, Dirichlet_nu_t, wall_model;
  std::vector<double> x, y, z, xg, yg, zg, w0, w1, kxx, kzz, Dd, Du, Dl;
  double dxmin, dymin, dzmin;
  A3 U, V, W, nut, Uo, Vo, Wo, rp;
  A3 F[3][3];                          // [stage][component]
  A3 alpha;                            // alpha_x(nx, 2, nzg)
  FFT fx, fz;

  static void centres(const std::vector<double>& f, int n, std::vector<double>& g) {
    std::vector<double> m(n + 1);
    for (int i = 1; i <= n - 1; ++i) m[i] = 0.5 * (f[i] + f[i + 1]);
    g.assign(n + 2, 0.0);
    for (int i = 2; i <= n; ++i) g[i] = m[i - 1];
    g[1] = m[1] - 2.0 * (m[1] - f[1]);
    g[n + 1] = m[n - 1] + 2.0 * (f[n] - m[n - 1]);
  }

  void setup(int nx_, int ny_, int nz_, const double* xf, const double* yf, const double* zf) {
    nx = nx_; ny = ny_; nz = nz_; nxg = nx + 1; nyg = ny + 1; nzg = nz + 1; Nx = nx - 2; Nz = nz - 2;
    x.assign(nx + 1, 0); y.assign(ny + 1, 0); z.assign(nz + 1, 0);
    for (int i = 1; i <= nx; ++i) x[i] = xf[i - 1];
    for (int i = 1; i <= ny; ++i) y[i] = yf[i - 1];
    for (int i = 1; i <= nz; ++i) z[i] = zf[i - 1];
    centres(x, nx, xg); centres(y, ny, yg); centres(z, nz, zg);
    auto dmin = [](const std::vector<double>& g, int n) { double m = 1e300; for (int i = 2; i <= n; ++i) m = std::min(m, g[i] - g[i - 1]); return m; };
    dxmin = dmin(xg, nxg); dymin = dmin(yg, nyg); dzmin = dmin(zg, nzg);
    const double pi = 4.0 * std::atan(1.0);
    auto km = [&](int N, double d, std::vector<double>& k) {
      k.assign(N, 0.0);
      const int half = (int)std::ceil(N / 2.0);
      for (int i = 0; i <= half && i < N; ++i) k[i] = 2.0 * (std::cos(2.0 * pi * i / N) - 1.0) / std::pow(d, 2.0);
      for (int i = half + 1; i < N; ++i) k[i] = 2.0 * (std::cos(2.0 * pi * (double)(-N + i) / N) - 1.0) / std::pow(d, 2.0);
    };
    km(Nx, dxmin, kxx); km(Nz, dzmin, kzz);
    Dd.assign(nyg + 1, 0); Du.assign(nyg + 1, 0); Dl.assign(nyg + 1, 0);
    auto abc = [&](int j, double& a, double& b, double& c) {
      a = 1.0 / (y[j] - y[j - 1]) / (yg[j + 1] - yg[j]);
      b = 1.0 / (y[j] - y[j - 1]) * (-1.0 / (yg[j + 1] - yg[j]) - 1.0 / (yg[j] - yg[j - 1]));
      c = 1.0 / (y[j] - y[j - 1]) / (yg[j] - yg[j - 1]);
    };
    double a, b, c;
    for (int j = 3; j <= nyg - 2; ++j) { abc(j, a, b, c); Du[j] = a; Dl[j] = c; Dd[j] = b; }
    abc(2, a, b, c); Dd[2] = b + c; Du[2] = a;
    abc(nyg - 1, a, b, c); Dd[nyg - 1] = a + b; Dl[nyg - 1] = c;
    w0.assign(ny + 1, 0); w1.assign(ny + 1, 0);
    for (int j = 1; j <= ny; ++j) { w0[j] = (yg[j + 1] - y[j]) / (yg[j + 1] - yg[j]); w1[j] = 1.0 - w0[j]; }
    U.init(nx, nyg, nzg); V.init(nxg, ny, nzg); W.init(nxg, nyg, nz); nut.init(nxg, nyg, nzg);
    rp.init(nxg, nyg, nzg);
    for (int s = 0; s < 3; ++s) { F[s][0].init(nx, nyg, nzg); F[s][1].init(nxg, ny, nzg); F[s][2].init(nxg, nyg, nz); }
    alpha.init(nx, 2, nzg);
    fx.init(Nx); fz.init(Nz);
  }

  // ------------------------------------------------------------ boundary conditions
  void per_x(A3& F, int id) const {
    for (int k = 1; k <= F.n3; ++k) for (int j = 1; j <= F.n2; ++j) {
      if (id == 1) { F(1, j, k) = F(nx - 1, j, k); F(nx, j, k) = F(2, j, k); }
      else { F(1, j, k) = F(nxg - 2, j, k); F(nxg - 1, j, k) = F(2, j, k); F(nxg, j, k) = F(3, j, k); }
    }
  }
  void per_z(A3& F, int id) const {
    for (int j = 1; j <= F.n2; ++j) for (int i = 1; i <= F.n1; ++i) {
      if (id == 3) { double a = F(i, j, nz - 1), b = F(i, j, 2); F(i, j, 1) = a; F(i, j, nz) = b; }
      else { double a = F(i, j, nzg - 2), b = F(i, j, 2), c = F(i, j, 3); F(i, j, 1) = a; F(i, j, nzg - 1) = b; F(i, j, nzg) = c; }
    }
  }
  void dir_y(A3& F, int id) const {
    for (int k = 1; k <= F.n3; ++k) for (int i = 1; i <= F.n1; ++i) {
      if (id == 1) { F(i, 1, k) = 0.0; F(i, ny, k) = 0.0; }
      else { F(i, 1, k) = -F(i, 2, k); F(i, nyg, k) = -F(i, nyg - 1, k); }
    }
  }
  void bc() {
    per_x(U, 1); per_x(V, 2); per_x(W, 2);
    per_z(U, 1); per_z(V, 2); per_z(W, 3);
    dir_y(U, 2); dir_y(V, 1); dir_y(W, 2);
  }

  double mass_flow_U() const {
    double q = 0, n = 0;
    for (int k = 2; k <= nzg - 2; ++k) for (int j = 3; j <= nyg - 1; ++j) for (int i = 2; i <= nx - 1; ++i) {
      q += (U(i, j, k) + U(i, j - 1, k)) * 0.5 * (yg[j] - yg[j - 1]);
      n += (1.0 + 1.0) * 0.5 * (yg[j] - yg[j - 1]);
    }
    return q / n;
  }

  // ------------------------------------------------------------ dt
  void compute_dt() {
    double lu = 0, lv = 0, lw = 0;
#pragma omp parallel for reduction(max : lu, lv, lw)
    for (int k = 2; k <= nzg - 1; ++k)
      for (int j = 2; j <= nyg - 1; ++j)
        for (int i = 2; i <= nxg - 1; ++i) {
          lu = std::max(lu, (xg[i + 1] - xg[i]) / std::fabs(U(i, j, k)));
          lv = std::max(lv, (yg[j + 1] - yg[j]) / std::fabs(V(i, j, k)));
          lw = std::max(lw, (zg[k + 1] - zg[k]) / std::fabs(W(i, j, k)));
        }
    double dc = std::min(std::min(CFL * lu, CFL * lv), CFL * lw);
    double dv = std::min(std::min(CFL * std::pow(dxmin, 2.0) / nu, CFL * std::pow(dymin, 2.0) / nu), CFL * std::pow(dzmin, 2.0) / nu);
    dt = std::min(std::min(dc, dv), 1e-3);
    if (CFL < 0) dt = -CFL;
  }

  // ------------------------------------------------------------ SGS
  // filter_xzy of src over (1:n1, j0:j1, 1:n3) -> dst(ii, j, kk) for ii=2..n1-1, kk=2..n3-1
  void filter(const A3& s, A3& d, int n1, int j0, int j1, int n3) const {
    const double f[3][3] = {{1.0 / 36, 1.0 / 9, 1.0 / 36}, {1.0 / 9, 4.0 / 9, 1.0 / 9}, {1.0 / 36, 1.0 / 9, 1.0 / 36}};
#pragma omp parallel for
    for (int kk = 2; kk <= n3 - 1; ++kk)
      for (int j = j0; j <= j1; ++j)
        for (int ii = 2; ii <= n1 - 1; ++ii) {
          double acc = 0.0;
          for (int di = -1; di <= 1; ++di)
            for (int dk = -1; dk <= 1; ++dk) {
              double yv;
              if (j == j0) yv = 2.0 / 3.0 * s(ii + di, j, kk + dk) + 1.0 / 3.0 * s(ii + di, j + 1, kk + dk);
              else if (j == j1) yv = 1.0 / 3.0 * s(ii + di, j - 1, kk + dk) + 2.0 / 3.0 * s(ii + di, j, kk + dk);
              else yv = 1.0 / 6.0 * s(ii + di, j - 1, kk + dk) + 2.0 / 3.0 * s(ii + di, j, kk + dk) + 1.0 / 6.0 * s(ii + di, j + 1, kk + dk);
              acc += yv * f[di + 1][dk + 1];
            }
          d(ii, j, kk) = acc;
        }
  }

  // Persistent work arrays of the SGS routines (the reference allocates its
  // equivalents per call; keeping them avoids re-faulting ~1 GB per stage).
  A3 sc_c[3], sc_cf[3], sc_L[6], sc_M[6], sc_Uf, sc_Vf, sc_Wf, sc_Sh[6], sc_Shat, sc_Sr[6], sc_S, sc_e[3], sc_tmp, sc_fq;
  void ensure(A3& a, int n1, int n2, int n3) { if (a.n1 != n1 || a.n2 != n2 || a.n3 != n3) a.init(n1, n2, n3); }

  // compute_Sij: Sij (6 arrays over (nxg, nyg, nzg), valid at interior centres) and |S|
  void sij(const A3& Uu, const A3& Vv, const A3& Ww, A3* S6, A3& S) {
    for (int m = 0; m < 6; ++m) ensure(S6[m], nxg, nyg, nzg);
    for (int m = 0; m < 3; ++m) ensure(sc_e[m], nxg, nyg, nzg);
    ensure(S, nxg, nyg, nzg);
    A3 &e4 = sc_e[0], &e5 = sc_e[1], &e6 = sc_e[2];
#pragma omp parallel for
    for (int k = 2; k <= nzg; ++k)
      for (int j = 2; j <= nyg; ++j)
        for (int i = 2; i <= nxg; ++i) {
          if (k <= nzg - 1 && j <= nyg - 1 && i <= nxg - 1) {
            S6[0](i, j, k) = (Uu(i, j, k) - Uu(i - 1, j, k)) / (x[i] - x[i - 1]);
            S6[1](i, j, k) = (Vv(i, j, k) - Vv(i, j - 1, k)) / (y[j] - y[j - 1]);
            S6[2](i, j, k) = (Ww(i, j, k) - Ww(i, j, k - 1)) / (z[k] - z[k - 1]);
          }
          e4(i, j, k) = 0.5 * ((Uu(i - 1, j, k) - Uu(i - 1, j - 1, k)) / (yg[j] - yg[j - 1]) + (Vv(i, j - 1, k) - Vv(i - 1, j - 1, k)) / (xg[i] - xg[i - 1]));
          e5(i, j, k) = 0.5 * ((Uu(i - 1, j, k) - Uu(i - 1, j, k - 1)) / (zg[k] - zg[k - 1]) + (Ww(i, j, k - 1) - Ww(i - 1, j, k - 1)) / (xg[i] - xg[i - 1]));
          e6(i, j, k) = 0.5 * ((Vv(i, j - 1, k) - Vv(i, j - 1, k - 1)) / (zg[k] - zg[k - 1]) + (Ww(i, j, k - 1) - Ww(i, j - 1, k - 1)) / (yg[j] - yg[j - 1]));
        }
#pragma omp parallel for
    for (int k = 2; k <= nzg - 1; ++k)
      for (int j = 2; j <= nyg - 1; ++j)
        for (int i = 2; i <= nxg - 1; ++i) {
          S6[3](i, j, k) = 0.25 * (e4(i, j, k) + e4(i + 1, j, k) + e4(i, j + 1, k) + e4(i + 1, j + 1, k));
          S6[4](i, j, k) = 0.25 * (e5(i, j, k) + e5(i + 1, j, k) + e5(i, j, k + 1) + e5(i + 1, j, k + 1));
          S6[5](i, j, k) = 0.25 * (e6(i, j, k) + e6(i, j + 1, k) + e6(i, j, k + 1) + e6(i, j + 1, k + 1));
          double a = 0.0;
          for (int m = 0; m < 6; ++m) a += (m < 3 ? 2.0 : 4.0) * S6[m](i, j, k) * S6[m](i, j, k);
          S(i, j, k) = std::sqrt(a);
        }
  }

  void dsm() {
    A3* c = sc_c;              // centre velocities (term, term_1, term_2 of subgrid.f90:394-420)
    for (int m = 0; m < 3; ++m) { ensure(c[m], nxg, nyg, nzg); ensure(sc_cf[m], nxg, nyg, nzg); }
    for (int m = 0; m < 6; ++m) { ensure(sc_L[m], nxg, nyg, nzg); ensure(sc_M[m], nxg, nyg, nzg); }
    ensure(sc_tmp, nxg, nyg, nzg); ensure(sc_fq, nxg, nyg, nzg);
    ensure(sc_Uf, nx, nyg, nzg); ensure(sc_Vf, nxg, ny, nzg); ensure(sc_Wf, nxg, nyg, nz);
#pragma omp parallel for
    for (int k = 1; k <= nzg; ++k)
      for (int j = 1; j <= nyg; ++j)
        for (int i = 1; i <= nxg; ++i) {
          if (i >= 2 && i <= nxg - 1) c[0](i, j, k) = 0.5 * (U(i - 1, j, k) + U(i, j, k));
          if (j >= 2 && j <= nyg - 1) c[1](i, j, k) = 0.5 * (V(i, j - 1, k) + V(i, j, k));
          if (k >= 2 && k <= nz) c[2](i, j, k) = 0.5 * (W(i, j, k - 1) + W(i, j, k));
        }
    per_x(c[0], 2); per_z(c[2], 4);
    const int pr[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
    A3 *L = sc_L, *cf = sc_cf, *M = sc_M;
    A3 &tmp = sc_tmp, &fq = sc_fq;
    for (int m = 0; m < 3; ++m) filter(c[m], cf[m], nxg, 2, nyg - 1, nzg);
    for (int m = 0; m < 6; ++m) {
      const A3 &ca = c[pr[m][0]], &cb = c[pr[m][1]];
#pragma omp parallel for
      for (int k = 2; k <= nzg; ++k) for (int j = 2; j <= nyg - 1; ++j) for (int i = 2; i <= nxg; ++i)
        tmp(i, j, k) = ca(i, j, k) * cb(i, j, k);
      per_x(tmp, 2); per_z(tmp, 4);
      filter(tmp, L[m], nxg, 2, nyg - 1, nzg);
      const A3 &fa = cf[pr[m][0]], &fb = cf[pr[m][1]];
#pragma omp parallel for
      for (int k = 2; k <= nzg - 1; ++k) for (int j = 2; j <= nyg - 1; ++j) for (int i = 2; i <= nxg - 1; ++i)
        L[m](i, j, k) -= fa(i, j, k) * fb(i, j, k);
    }
    filter(U, sc_Uf, nx, 1, nyg, nzg); filter(V, sc_Vf, nxg, 1, ny, nzg); filter(W, sc_Wf, nxg, 1, nyg, nz);
    per_x(sc_Uf, 1); per_z(sc_Uf, 1); per_x(sc_Vf, 2); per_z(sc_Vf, 2); per_x(sc_Wf, 2); per_z(sc_Wf, 3);
    sij(sc_Uf, sc_Vf, sc_Wf, sc_Sh, sc_Shat);
    sij(U, V, W, sc_Sr, sc_S);
    const A3 &S = sc_S, &Shat = sc_Shat;
    for (int m = 0; m < 6; ++m) {
      const A3 &sh = sc_Sh[m], &sr = sc_Sr[m];
#pragma omp parallel for
      for (int k = 2; k <= nzg - 1; ++k) for (int j = 2; j <= nyg - 1; ++j) for (int i = 2; i <= nxg - 1; ++i) {
        M[m](i, j, k) = 4.0 * Shat(i, j, k) * sh(i, j, k);
        tmp(i, j, k) = S(i, j, k) * sr(i, j, k);
      }
      per_x(tmp, 2); per_z(tmp, 4);
      filter(tmp, fq, nxg, 2, nyg - 1, nzg);
#pragma omp parallel for
      for (int k = 2; k <= nzg - 1; ++k) for (int j = 2; j <= nyg - 1; ++j) for (int i = 2; i <= nxg - 1; ++i)
        M[m](i, j, k) -= fq(i, j, k);
    }
    std::vector<double> LM(nyg + 1, 0.0), MM(nyg + 1, 0.0);
#pragma omp parallel for
    for (int j = 2; j <= nyg - 1; ++j) {
      double lm = 0, mm = 0;
      for (int k = 2; k <= nzg - 1; ++k) for (int i = 2; i <= nxg - 1; ++i) {
        lm += L[0](i, j, k) * M[0](i, j, k) + L[1](i, j, k) * M[1](i, j, k) + L[2](i, j, k) * M[2](i, j, k)
            + 2.0 * (L[3](i, j, k) * M[3](i, j, k) + L[4](i, j, k) * M[4](i, j, k) + L[5](i, j, k) * M[5](i, j, k));
        mm += M[0](i, j, k) * M[0](i, j, k) + M[1](i, j, k) * M[1](i, j, k) + M[2](i, j, k) * M[2](i, j, k)
            + 2.0 * (M[3](i, j, k) * M[3](i, j, k) + M[4](i, j, k) * M[4](i, j, k) + M[5](i, j, k) * M[5](i, j, k));
      }
      LM[j] = lm; MM[j] = mm;
    }
    std::fill(nut.v.begin(), nut.v.end(), 0.0);
#pragma omp parallel for
    for (int k = 2; k <= nzg - 1; ++k) for (int j = 2; j <= nyg - 1; ++j) for (int i = 2; i <= nxg - 1; ++i)
      nut(i, j, k) = -0.5 * (LM[j] / MM[j]) * S(i, j, k);
    finish_nut();
  }

  void smag() {
    sij(U, V, W, sc_Sr, sc_S);
    const A3& S = sc_S;
    const double ut = std::pow(dPdx, 0.5);
    const double ls = ut != 0.0 ? nu / ut : INFINITY;
    for (int j = 2; j <= nyg - 1; ++j) {
      double f = j < nyg / 2 ? 1.0 - std::exp(-(yg[j] - y[1]) / 25.0 / ls) : 1.0 - std::exp(-(y[ny] - yg[j]) / 25.0 / ls);
      if (Dirichlet_nu_t == 0) f = 1.0;
      const double Delta = std::pow(dxmin * dzmin * (y[j] - y[j - 1]), 1.0 / 3.0);
      const double c = std::pow(Cs * Delta * f, 2.0);
      for (int k = 2; k <= nzg - 1; ++k) for (int i = 2; i <= nxg - 1; ++i) nut(i, j, k) = c * S(i, j, k);
    }
    finish_nut();
  }

  // Grid-scaled differences of one velocity component interpolated to a
  // centre the way the reference's interpolate_* pairs do it: a0/b0 at the
  // near and a1/b1 at the far face in the derivative direction (a, b the two
  // faces in the other direction), h0/h1 the derivative spacings there.
  // Returns the centre derivative (d), the centre difference (d^) and the
  // two face averages of the difference (s1[0], s1[1]).
  struct Cavg { double der, dif, s1[2]; };
  static Cavg cavg(double a0, double b0, double a1, double b1, double h0, double h1) {
    Cavg c;
    const double t20 = 0.5 * (a0 / h0 + b0 / h0), t21 = 0.5 * (a1 / h1 + b1 / h1);
    c.der = 0.5 * (t20 + t21);
    c.s1[0] = 0.5 * (a0 + b0); c.s1[1] = 0.5 * (a1 + b1);
    c.dif = 0.5 * (c.s1[0] + c.s1[1]);
    return c;
  }

  // sgs_AMD (subgrid.f90:632-874): nu_t = max(0, -C N / D), C = 0.3, with
  // N = sum (d^_k u_i)(d^_k u_j) S_ij and D = sum (d_k u_l)^2, the terms in
  // the reference's order (U, V, W blocks, then the S12, S13, S23 cross
  // terms), one fused pass over the interior centres.
  void amd() {
    sij(U, V, W, sc_Sr, sc_S);
    const A3* S6 = sc_Sr;
    std::fill(nut.v.begin(), nut.v.end(), 0.0);
    const double Cp = 0.3;
#pragma omp parallel for
    for (int k = 2; k <= nzg - 1; ++k)
      for (int j = 2; j <= nyg - 1; ++j)
        for (int i = 2; i <= nxg - 1; ++i) {
          const double S11 = S6[0](i, j, k), S22 = S6[1](i, j, k), S33 = S6[2](i, j, k);
          const double S12 = S6[3](i, j, k), S13 = S6[4](i, j, k), S23 = S6[5](i, j, k);
          const double dy0 = yg[j] - yg[j - 1], dy1 = yg[j + 1] - yg[j];
          const double dz0 = zg[k] - zg[k - 1], dz1 = zg[k + 1] - zg[k];
          const double dx0 = xg[i] - xg[i - 1], dx1 = xg[i + 1] - xg[i];
          // U: x, y (faces j, j+1; x faces i-1, i), z
          const double dUx = U(i, j, k) - U(i - 1, j, k);
          const double hx = x[i] - x[i - 1];
          double t4 = dUx * dUx / (hx * hx);
          double nv = dUx * dUx * S11;
          const Cavg Uy = cavg(U(i - 1, j, k) - U(i - 1, j - 1, k), U(i, j, k) - U(i, j - 1, k),
                               U(i - 1, j + 1, k) - U(i - 1, j, k), U(i, j + 1, k) - U(i, j, k), dy0, dy1);
          t4 = t4 + Uy.der * Uy.der; nv = nv + Uy.dif * Uy.dif * S11;
          const Cavg Uz = cavg(U(i - 1, j, k) - U(i - 1, j, k - 1), U(i, j, k) - U(i, j, k - 1),
                               U(i - 1, j, k + 1) - U(i - 1, j, k), U(i, j, k + 1) - U(i, j, k), dz0, dz1);
          t4 = t4 + Uz.der * Uz.der; nv = nv + Uz.dif * Uz.dif * S11;
          // V: y, x (faces i, i+1; y faces j-1, j), z
          const double dVy = V(i, j, k) - V(i, j - 1, k);
          const double hy = y[j] - y[j - 1];
          t4 = t4 + dVy * dVy / (hy * hy);
          nv = nv + dVy * dVy * S22;
          const Cavg Vx = cavg(V(i, j - 1, k) - V(i - 1, j - 1, k), V(i, j, k) - V(i - 1, j, k),
                               V(i + 1, j - 1, k) - V(i, j - 1, k), V(i + 1, j, k) - V(i, j, k), dx0, dx1);
          t4 = t4 + Vx.der * Vx.der; nv = nv + Vx.dif * Vx.dif * S22;
          const Cavg Vz = cavg(V(i, j - 1, k) - V(i, j - 1, k - 1), V(i, j, k) - V(i, j, k - 1),
                               V(i, j - 1, k + 1) - V(i, j - 1, k), V(i, j, k + 1) - V(i, j, k), dz0, dz1);
          t4 = t4 + Vz.der * Vz.der; nv = nv + Vz.dif * Vz.dif * S22;
          // W: z, x (faces i, i+1; z faces k-1, k), y (faces j, j+1; z faces k-1, k)
          const double dWz = W(i, j, k) - W(i, j, k - 1);
          const double hz = z[k] - z[k - 1];
          const double dWz2 = dWz * dWz;
          t4 = t4 + dWz2 / (hz * hz);
          nv = nv + dWz2 * S33;
          const Cavg Wx = cavg(W(i, j, k - 1) - W(i - 1, j, k - 1), W(i, j, k) - W(i - 1, j, k),
                               W(i + 1, j, k - 1) - W(i, j, k - 1), W(i + 1, j, k) - W(i, j, k), dx0, dx1);
          t4 = t4 + Wx.der * Wx.der; nv = nv + Wx.dif * Wx.dif * S33;
          const Cavg Wy = cavg(W(i, j, k - 1) - W(i, j - 1, k - 1), W(i, j, k) - W(i, j - 1, k),
                               W(i, j + 1, k - 1) - W(i, j, k - 1), W(i, j + 1, k) - W(i, j, k), dy0, dy1);
          t4 = t4 + Wy.der * Wy.der; nv = nv + Wy.dif * Wy.dif * S33;
          // cross terms 2 (d^_k u_i)(d^_k u_j) S_ij, i != j (subgrid.f90:751-851)
          nv = nv + 2.0 * (Vx.dif * dUx) * S12;
          nv = nv + 2.0 * (Uy.dif * dVy) * S12;
          nv = nv + 2.0 * (0.5 * (Uz.s1[0] * Vz.s1[0] + Uz.s1[1] * Vz.s1[1])) * S12;
          nv = nv + 2.0 * (Wx.dif * dUx) * S13;
          nv = nv + 2.0 * (Uz.dif * dWz) * S13;
          nv = nv + 2.0 * (0.5 * (Uy.s1[0] * Wy.s1[0] + Uy.s1[1] * Wy.s1[1])) * S13;
          nv = nv + 2.0 * (Wy.dif * dVy) * S23;
          nv = nv + 2.0 * (Vz.dif * dWz) * S23;
          nv = nv + 2.0 * (0.5 * (Vx.s1[0] * Wx.s1[0] + Vx.s1[1] * Wx.s1[1])) * S23;
          nut(i, j, k) = -Cp * nv / t4;
        }
    finish_nut_amd_vreman(true);
  }

  // sgs_Vreman (subgrid.f90:897-1004): nu_t = C sqrt(B_b / a_ij a_ij),
  // C = 2.5 (0.1)^2, b_ij = sum_m dx_m^2 a_mi a_mj, a_ij = du_j/dx_i at the
  // centre (reference layout 1 4 5 / 7 2 6 / 8 9 3; off-diagonals the mean of
  // the four surrounding edge derivatives).  Not clipped, as written.
  void vreman() {
    std::fill(nut.v.begin(), nut.v.end(), 0.0);
    const double C = 2.5 * std::pow(0.1, 2.0);
#pragma omp parallel for
    for (int k = 2; k <= nzg - 1; ++k)
      for (int j = 2; j <= nyg - 1; ++j)
        for (int i = 2; i <= nxg - 1; ++i) {
          const double dxl = xg[i] - xg[i - 1], dxr = xg[i + 1] - xg[i];
          const double dyl = yg[j] - yg[j - 1], dyr = yg[j + 1] - yg[j];
          const double dzl = zg[k] - zg[k - 1], dzr = zg[k + 1] - zg[k];
          double a[10];
          a[1] = (U(i, j, k) - U(i - 1, j, k)) / (x[i] - x[i - 1]);
          a[4] = 0.25 * (V(i, j, k) - V(i - 1, j, k)) / dxl + 0.25 * (V(i, j - 1, k) - V(i - 1, j - 1, k)) / dxl
               + 0.25 * (V(i + 1, j, k) - V(i, j, k)) / dxr + 0.25 * (V(i + 1, j - 1, k) - V(i, j - 1, k)) / dxr;
          a[5] = 0.25 * (W(i, j, k) - W(i - 1, j, k)) / dxl + 0.25 * (W(i, j, k - 1) - W(i - 1, j, k - 1)) / dxl
               + 0.25 * (W(i + 1, j, k) - W(i, j, k)) / dxr + 0.25 * (W(i + 1, j, k - 1) - W(i, j, k - 1)) / dxr;
          a[2] = (V(i, j, k) - V(i, j - 1, k)) / (y[j] - y[j - 1]);
          a[7] = 0.25 * (U(i, j, k) - U(i, j - 1, k)) / dyl + 0.25 * (U(i - 1, j, k) - U(i - 1, j - 1, k)) / dyl
               + 0.25 * (U(i, j + 1, k) - U(i, j, k)) / dyr + 0.25 * (U(i - 1, j + 1, k) - U(i - 1, j, k)) / dyr;
          a[6] = 0.25 * (W(i, j, k) - W(i, j - 1, k)) / dyl + 0.25 * (W(i, j, k - 1) - W(i, j - 1, k - 1)) / dyl
               + 0.25 * (W(i, j + 1, k) - W(i, j, k)) / dyr + 0.25 * (W(i, j + 1, k - 1) - W(i, j, k - 1)) / dyr;
          a[3] = (W(i, j, k) - W(i, j, k - 1)) / (z[k] - z[k - 1]);
          a[8] = 0.25 * (U(i, j, k) - U(i, j, k - 1)) / dzl + 0.25 * (U(i - 1, j, k) - U(i - 1, j, k - 1)) / dzl
               + 0.25 * (U(i, j, k + 1) - U(i, j, k)) / dzr + 0.25 * (U(i - 1, j, k + 1) - U(i - 1, j, k)) / dzr;
          a[9] = 0.25 * (V(i, j, k) - V(i, j, k - 1)) / dzl + 0.25 * (V(i, j - 1, k) - V(i, j - 1, k - 1)) / dzl
               + 0.25 * (V(i, j, k + 1) - V(i, j, k)) / dzr + 0.25 * (V(i, j - 1, k + 1) - V(i, j - 1, k)) / dzr;
          const double ddx = (x[i] - x[i - 1]) * (x[i] - x[i - 1]);
          const double ddy = (y[j] - y[j - 1]) * (y[j] - y[j - 1]);
          const double ddz = (z[k] - z[k - 1]) * (z[k] - z[k - 1]);
          // b_ij, (11, 22, 33, 12, 13, 23) = 1..6
          static const int px[7][2] = {{0, 0}, {1, 1}, {4, 4}, {5, 5}, {1, 4}, {1, 5}, {4, 5}};
          static const int py[7][2] = {{0, 0}, {7, 7}, {2, 2}, {6, 6}, {7, 2}, {7, 6}, {2, 6}};
          static const int pz[7][2] = {{0, 0}, {8, 8}, {9, 9}, {3, 3}, {8, 9}, {8, 3}, {9, 3}};
          double b[7];
          for (int m = 1; m <= 6; ++m) {
            b[m] = 0.0 + ddx * a[px[m][0]] * a[px[m][1]];
            b[m] = b[m] + ddy * a[py[m][0]] * a[py[m][1]];
            b[m] = b[m] + ddz * a[pz[m][0]] * a[pz[m][1]];
          }
          const double Bb = b[1] * b[2] - b[4] * b[4] + b[1] * b[3] - b[5] * b[5] + b[2] * b[3] - b[6] * b[6];
          double Ab = a[1] * a[1];
          for (int m = 2; m <= 9; ++m) Ab = Ab + a[m] * a[m];
          nut(i, j, k) = C * std::pow(Bb / Ab, 0.5);
        }
    finish_nut_amd_vreman(false);
  }

  // ghost rows of the AMD and Vreman models (subgrid.f90:858-871, 991-1002)
  void finish_nut_amd_vreman(bool clip) {
    per_x(nut, 2); per_z(nut, 4);
    if (clip) for (auto& v : nut.v) v = std::max(v, 0.0);
    if (Dirichlet_nu_t == 1) dir_y(nut, 2);
    else if (Dirichlet_nu_t == 0) {
      for (int k = 1; k <= nzg; ++k) for (int i = 1; i <= nxg; ++i) { nut(i, 1, k) = nut(i, 2, k); nut(i, nyg, k) = nut(i, nyg - 1, k); }
    } else {
      const double c = 2.0 * 0.38 * std::pow(dPdx, 0.5) * (y[2] - y[1]) / 2.0;
      for (int k = 1; k <= nzg; ++k) for (int i = 1; i <= nxg; ++i) { nut(i, 1, k) = -nut(i, 2, k) + c; nut(i, nyg, k) = -nut(i, nyg - 1, k) + c; }
    }
  }

  void finish_nut() {
    per_x(nut, 2); per_z(nut, 4);
    for (auto& v : nut.v) v = std::max(v, 0.0);
    if (Dirichlet_nu_t == 1) dir_y(nut, 2);
    else for (int k = 1; k <= nzg; ++k) for (int i = 1; i <= nxg; ++i) { nut(i, 1, k) = nut(i, 2, k); nut(i, nyg, k) = nut(i, nyg - 1, k); }
  }

  static double eqlog(double u, double h, double nuv) {
    const double kap = 0.41, B = 5.2, au = std::fabs(u);
    const double utl = std::sqrt(nuv * au / h), ypl = h * utl / nuv;
    const double f0 = utl * (std::log(ypl) / kap + B) - au;
    double ut = utl;
    if (f0 < 0.0 && ypl >= 1.0)
      for (int it = 0; it < 12; ++it) {
        const double lg = std::log(h * ut / nuv);
        ut -= (ut * (lg / kap + B) - au) / (lg / kap + B + 1.0 / kap);
      }
    const double sg = u > 0.0 ? 1.0 : (u < 0.0 ? -1.0 : 0.0);
    return sg * ut * ut;
  }

  void compute_wall_model() {
    if (wall_model == 2) {
      const double hb = yg[4] - y[1], ht = y[ny] - yg[nyg - 3];
      for (int k = 2; k <= nzg - 2; ++k) for (int i = 2; i <= nx - 1; ++i) {
        alpha(i, 1, k) = eqlog(U(i, 4, k), hb, nu);
        alpha(i, 2, k) = eqlog(U(i, nyg - 3, k), ht, nu);
      }
      per_x(alpha, 1);
      for (int w = 1; w <= 2; ++w) for (int i = 1; i <= nx; ++i) {
        double a = alpha(i, w, nzg - 2), b = alpha(i, w, 2), c = alpha(i, w, 3);
        alpha(i, w, 1) = a; alpha(i, w, nzg - 1) = b; alpha(i, w, nzg) = c;
      }
    }
    const double dyw = yg[2] - yg[1];
    std::vector<double> tb(nx + 1), tt(nx + 1);
    for (int k = 1; k <= nzg; ++k) {
      for (int i = 1; i <= nx; ++i) {
        tb[i] = alpha(i, 1, k) / ((U(i, 2, k) - U(i, 1, k)) / dyw) - nu;
        tt[i] = alpha(i, 2, k) / ((U(i, nyg - 1, k) - U(i, nyg, k)) / dyw) - nu;
      }
      for (int i = 2; i <= nx; ++i) {
        const double cb = 0.5 * (tb[i - 1] + tb[i]), ct = 0.5 * (tt[i - 1] + tt[i]);
        nut(i, 1, k) = cb; nut(i, 2, k) = cb; nut(i, nyg - 1, k) = ct; nut(i, nyg, k) = ct;
      }
    }
    per_x(nut, 2);
  }

  // ------------------------------------------------------------ RHS (equations.f90)
  void rhs_u(A3& R) const {
#pragma omp parallel for
    for (int k = 2; k <= nzg - 1; ++k)
      for (int j = 2; j <= nyg - 1; ++j)
        for (int i = 2; i <= nx - 1; ++i) {
          const double cb = 0.5 * (U(i, j, k) + U(i + 1, j, k)), ca = 0.5 * (U(i - 1, j, k) + U(i, j, k));
          double r = -(cb * cb - ca * ca) / (xg[i + 1] - xg[i]);
          const double uh = w0[j] * U(i, j, k) + w1[j] * U(i, j + 1, k), ul = w0[j - 1] * U(i, j - 1, k) + w1[j - 1] * U(i, j, k);
          const double vh = 0.5 * (V(i, j, k) + V(i + 1, j, k)), vl = 0.5 * (V(i, j - 1, k) + V(i + 1, j - 1, k));
          r += -(uh * vh - ul * vl) / (y[j] - y[j - 1]);
          const double uzh = 0.5 * (U(i, j, k) + U(i, j, k + 1)), uzl = 0.5 * (U(i, j, k - 1) + U(i, j, k));
          const double wh = 0.5 * (W(i, j, k) + W(i + 1, j, k)), wl = 0.5 * (W(i, j, k - 1) + W(i + 1, j, k - 1));
          r += -(uzh * wh - uzl * wl) / (z[k] - z[k - 1]);
          const double nx1 = nu + nut(i, j, k), nx2 = nu + nut(i + 1, j, k);
          const double ny1 = nu + 0.5 * (w0[j - 1] * nut(i, j - 1, k) + w1[j - 1] * nut(i, j, k) + w0[j - 1] * nut(i + 1, j - 1, k) + w1[j - 1] * nut(i + 1, j, k));
          const double ny2 = nu + 0.5 * (w0[j] * nut(i, j, k) + w1[j] * nut(i, j + 1, k) + w0[j] * nut(i + 1, j, k) + w1[j] * nut(i + 1, j + 1, k));
          const double nz1 = nu + 0.25 * (nut(i, j, k) + nut(i, j, k - 1) + nut(i + 1, j, k) + nut(i + 1, j, k - 1));
          const double nz2 = nu + 0.25 * (nut(i, j, k) + nut(i, j, k + 1) + nut(i + 1, j, k) + nut(i + 1, j, k + 1));
          const double t2h = (U(i, j + 1, k) - U(i, j, k)) / (yg[j + 1] - yg[j]), t2l = (U(i, j, k) - U(i, j - 1, k)) / (yg[j] - yg[j - 1]);
          r += 1.0 / (xg[i + 1] - xg[i]) * (nx2 / (x[i + 1] - x[i]) * (U(i + 1, j, k) - U(i, j, k)) - nx1 / (x[i] - x[i - 1]) * (U(i, j, k) - U(i - 1, j, k)))
             + 1.0 / (y[j] - y[j - 1]) * (ny2 * t2h - ny1 * t2l)
             + 1.0 / (z[k] - z[k - 1]) * (nz2 / (zg[k + 1] - zg[k]) * (U(i, j, k + 1) - U(i, j, k)) - nz1 / (zg[k] - zg[k - 1]) * (U(i, j, k) - U(i, j, k - 1)));
          R(i, j, k) = r + dPdx;
        }
  }
  void rhs_v(A3& R) const {
#pragma omp parallel for
    for (int k = 2; k <= nzg - 1; ++k)
      for (int j = 2; j <= ny - 1; ++j)
        for (int i = 2; i <= nxg - 1; ++i) {
          const double cb = 0.5 * (V(i, j, k) + V(i, j + 1, k)), ca = 0.5 * (V(i, j - 1, k) + V(i, j, k));
          double r = -(cb * cb - ca * ca) / (yg[j + 1] - yg[j]);
          const double uh = w0[j] * U(i, j, k) + w1[j] * U(i, j + 1, k), ul = w0[j] * U(i - 1, j, k) + w1[j] * U(i - 1, j + 1, k);
          const double vh = 0.5 * (V(i, j, k) + V(i + 1, j, k)), vl = 0.5 * (V(i - 1, j, k) + V(i, j, k));
          r += -(uh * vh - ul * vl) / (x[i] - x[i - 1]);
          const double vzh = 0.5 * (V(i, j, k) + V(i, j, k + 1)), vzl = 0.5 * (V(i, j, k - 1) + V(i, j, k));
          const double wh = w0[j] * W(i, j, k) + w1[j] * W(i, j + 1, k), wl = w0[j] * W(i, j, k - 1) + w1[j] * W(i, j + 1, k - 1);
          r += -(vzh * wh - vzl * wl) / (z[k] - z[k - 1]);
          const double nx1 = nu + 0.5 * (w0[j] * nut(i - 1, j, k) + w1[j] * nut(i - 1, j + 1, k) + w0[j] * nut(i, j, k) + w1[j] * nut(i, j + 1, k));
          const double nx2 = nu + 0.5 * (w0[j] * nut(i, j, k) + w1[j] * nut(i, j + 1, k) + w0[j] * nut(i + 1, j, k) + w1[j] * nut(i + 1, j + 1, k));
          const double ny1 = nu + nut(i, j, k), ny2 = nu + nut(i, j + 1, k);
          const double nz1 = nu + 0.5 * (w0[j] * nut(i, j, k - 1) + w1[j] * nut(i, j + 1, k - 1) + w0[j] * nut(i, j, k) + w1[j] * nut(i, j + 1, k));
          const double nz2 = nu + 0.5 * (w0[j] * nut(i, j, k) + w1[j] * nut(i, j + 1, k) + w0[j] * nut(i, j, k + 1) + w1[j] * nut(i, j + 1, k + 1));
          r += 1.0 / (x[i] - x[i - 1]) * (nx2 / (xg[i + 1] - xg[i]) * (V(i + 1, j, k) - V(i, j, k)) - nx1 / (xg[i] - xg[i - 1]) * (V(i, j, k) - V(i - 1, j, k)))
             + 1.0 / (yg[j + 1] - yg[j]) * (ny2 / (y[j + 1] - y[j]) * (V(i, j + 1, k) - V(i, j, k)) - ny1 / (y[j] - y[j - 1]) * (V(i, j, k) - V(i, j - 1, k)))
             + 1.0 / (z[k] - z[k - 1]) * (nz2 / (zg[k + 1] - zg[k]) * (V(i, j, k + 1) - V(i, j, k)) - nz1 / (zg[k] - zg[k - 1]) * (V(i, j, k) - V(i, j, k - 1)));
          R(i, j, k) = r;
        }
  }
  void rhs_w(A3& R) const {
#pragma omp parallel for
    for (int k = 2; k <= nz - 1; ++k)
      for (int j = 2; j <= nyg - 1; ++j)
        for (int i = 2; i <= nxg - 1; ++i) {
          const double cb = 0.5 * (W(i, j, k) + W(i, j, k + 1)), ca = 0.5 * (W(i, j, k - 1) + W(i, j, k));
          double r = -(cb * cb - ca * ca) / (zg[k + 1] - zg[k]);
          const double uh = 0.5 * (U(i, j, k) + U(i, j, k + 1)), ul = 0.5 * (U(i - 1, j, k) + U(i - 1, j, k + 1));
          const double wh = 0.5 * (W(i, j, k) + W(i + 1, j, k)), wl = 0.5 * (W(i - 1, j, k) + W(i, j, k));
          r += -(uh * wh - ul * wl) / (x[i] - x[i - 1]);
          const double vh = 0.5 * (V(i, j, k) + V(i, j, k + 1)), vl = 0.5 * (V(i, j - 1, k) + V(i, j - 1, k + 1));
          const double wyh = w0[j] * W(i, j, k) + w1[j] * W(i, j + 1, k), wyl = w0[j - 1] * W(i, j - 1, k) + w1[j - 1] * W(i, j, k);
          r += -(vh * wyh - vl * wyl) / (y[j] - y[j - 1]);
          const double nx1 = nu + 0.25 * (nut(i, j, k) + nut(i, j, k + 1) + nut(i - 1, j, k) + nut(i - 1, j, k + 1));
          const double nx2 = nu + 0.25 * (nut(i, j, k) + nut(i, j, k + 1) + nut(i + 1, j, k) + nut(i + 1, j, k + 1));
          const double ny1 = nu + 0.5 * (w0[j - 1] * nut(i, j - 1, k) + w1[j - 1] * nut(i, j, k) + w0[j - 1] * nut(i, j - 1, k + 1) + w1[j - 1] * nut(i, j, k + 1));
          const double ny2 = nu + 0.5 * (w0[j] * nut(i, j, k) + w1[j] * nut(i, j + 1, k) + w0[j] * nut(i, j, k + 1) + w1[j] * nut(i, j + 1, k + 1));
          const double nz1 = nu + nut(i, j, k), nz2 = nu + nut(i, j, k + 1);
          const double t2h = (W(i, j + 1, k) - W(i, j, k)) / (yg[j + 1] - yg[j]), t2l = (W(i, j, k) - W(i, j - 1, k)) / (yg[j] - yg[j - 1]);
          r += 1.0 / (x[i] - x[i - 1]) * (nx2 / (xg[i + 1] - xg[i]) * (W(i + 1, j, k) - W(i, j, k)) - nx1 / (xg[i] - xg[i - 1]) * (W(i, j, k) - W(i - 1, j, k)))
             + 1.0 / (y[j] - y[j - 1]) * (ny2 * t2h - ny1 * t2l)
             + 1.0 / (zg[k + 1] - zg[k]) * (nz2 / (z[k + 1] - z[k]) * (W(i, j, k + 1) - W(i, j, k)) - nz1 / (z[k] - z[k - 1]) * (W(i, j, k) - W(i, j, k - 1)));
          R(i, j, k) = r;
        }
  }

  // ------------------------------------------------------------ projection
  void projection() {
    const int Ny = nyg - 2;
    std::vector<cplx> hat((size_t)Nx * Nz * Ny);
#pragma omp parallel
    {
      std::vector<cplx> row(std::max(Nx, Nz)), wk(std::max(Nx, Nz)), pl((size_t)Nx * Nz);
#pragma omp for
      for (int j = 2; j <= nyg - 1; ++j) {
        for (int k = 2; k <= Nz + 1; ++k)
          for (int i = 2; i <= Nx + 1; ++i)
            pl[(size_t)(i - 2) + (size_t)Nx * (k - 2)] = (U(i, j, k) - U(i - 1, j, k)) / (x[i] - x[i - 1]) +
                                                          (V(i, j, k) - V(i, j - 1, k)) / (y[j] - y[j - 1]) +
                                                          (W(i, j, k) - W(i, j, k - 1)) / (z[k] - z[k - 1]);
        for (int k = 0; k < Nz; ++k) fx.run(&pl[(size_t)Nx * k], wk.data(), false);
        for (int i = 0; i < Nx; ++i) {
          for (int k = 0; k < Nz; ++k) row[k] = pl[(size_t)i + (size_t)Nx * k];
          fz.run(row.data(), wk.data(), false);
          for (int k = 0; k < Nz; ++k) hat[((size_t)k * Nx + i) * Ny + (j - 2)] = row[k];
        }
      }
      // Thomas elimination per mode (zgtsv without pivoting, projection.f90:90-113)
      std::vector<cplx> d(Ny), b(Ny);
#pragma omp for
      for (int m = 0; m < Nx * Nz; ++m) {
        const int i = m % Nx, k = m / Nx;
        cplx* col = &hat[(size_t)m * Ny];
        for (int r = 0; r < Ny; ++r) { d[r] = Dd[r + 2] + kxx[i] + kzz[k]; b[r] = col[r]; }
        if (i == 0 && k == 0) d[0] *= 1.5;
        for (int r = 1; r < Ny; ++r) {
          const cplx mult = Dl[r + 2] / d[r - 1];
          d[r] -= mult * Du[r + 1];
          b[r] -= mult * b[r - 1];
        }
        col[Ny - 1] = b[Ny - 1] / d[Ny - 1];
        for (int r = Ny - 2; r >= 0; --r) col[r] = (b[r] - Du[r + 2] * col[r + 1]) / d[r];
      }
#pragma omp for
      for (int j = 2; j <= nyg - 1; ++j) {
        for (int i = 0; i < Nx; ++i) {
          for (int k = 0; k < Nz; ++k) row[k] = hat[((size_t)k * Nx + i) * Ny + (j - 2)];
          fz.run(row.data(), wk.data(), true);
          for (int k = 0; k < Nz; ++k) pl[(size_t)i + (size_t)Nx * k] = row[k];
        }
        for (int k = 0; k < Nz; ++k) {
          fx.run(&pl[(size_t)Nx * k], wk.data(), true);
          for (int i = 0; i < Nx; ++i) rp(i + 2, j, k + 2) = pl[(size_t)i + (size_t)Nx * k].real() / ((double)Nx * Nz);
        }
      }
    }
    for (int k = 1; k <= nzg; ++k) for (int j = 1; j <= nyg; ++j) rp(nxg - 1, j, k) = rp(2, j, k);
    for (int j = 1; j <= nyg; ++j) for (int i = 2; i <= nxg - 1; ++i) rp(i, j, Nz + 2) = rp(i, j, 2);
#pragma omp parallel for
    for (int k = 2; k <= nzg - 1; ++k)
      for (int j = 2; j <= nyg - 1; ++j) {
        for (int i = 2; i <= nx - 1; ++i) U(i, j, k) -= (rp(i + 1, j, k) - rp(i, j, k)) / (xg[i + 1] - xg[i]);
        if (j <= ny - 1)
          for (int i = 2; i <= nxg - 1; ++i) V(i, j, k) -= (rp(i, j + 1, k) - rp(i, j, k)) / (yg[j + 1] - yg[j]);
        if (k <= nz - 1)
          for (int i = 2; i <= nxg - 1; ++i) W(i, j, k) -= (rp(i, j, k + 1) - rp(i, j, k)) / (zg[k + 1] - zg[k]);
      }
  }

  // ------------------------------------------------------------ RK3
  void rk3() {
    Uo = U; Vo = V; Wo = W;
    const double to = t;
    for (int s = 0; s < 3; ++s) {
      if (LES_model == 2) dsm();
      else if (LES_model == 1) smag();
      else if (LES_model == 3) amd();
      else if (LES_model == 4) vreman();
      else std::fill(nut.v.begin(), nut.v.end(), 0.0);
      if (wall_model != 0) compute_wall_model();
      rhs_u(F[s][0]); rhs_v(F[s][1]); rhs_w(F[s][2]);
#pragma omp parallel for
      for (int k = 2; k <= nzg - 1; ++k)
        for (int j = 2; j <= nyg - 1; ++j) {
          for (int i = 2; i <= nx - 1; ++i) {
            double a = 0.0; for (int q = 0; q <= s; ++q) a += RKC[s][q] * F[q][0](i, j, k);
            U(i, j, k) = Uo(i, j, k) + dt * a;
          }
          if (j <= ny - 1) for (int i = 2; i <= nxg - 1; ++i) {
            double a = 0.0; for (int q = 0; q <= s; ++q) a += RKC[s][q] * F[q][1](i, j, k);
            V(i, j, k) = Vo(i, j, k) + dt * a;
          }
          if (k <= nz - 1) for (int i = 2; i <= nxg - 1; ++i) {
            double a = 0.0; for (int q = 0; q <= s; ++q) a += RKC[s][q] * F[q][2](i, j, k);
            W(i, j, k) = Wo(i, j, k) + dt * a;
          }
        }
      t = to + RKT[s] * dt;
      bc();
      projection();
      bc();
    }
    if (x_mass_cte == 1) {
      double su = 0.0; long n = 0;
      for (int k = 2; k <= nzg - 2; ++k) for (int i = 2; i <= nx - 1; ++i) { su += 0.5 * (U(i, 3, k) + U(i, nyg - 2, k)); ++n; }
      const double d = Q0 - su / (double)n;
      for (int k = 2; k <= nzg - 1; ++k) for (int j = 2; j <= nyg - 1; ++j) for (int i = 2; i <= nx - 1; ++i) U(i, j, k) += d;
      dPdx = 0.0;
      bc();
    }
  }
};

}  // namespace

extern "C" {

void* refcpu_create(int nx, int ny, int nz, const double* x, const double* y, const double* z, double nu, double CFL,
                    double dPdx, int x_mass_cte, int LES_model, int Dirichlet_nu_t, int wall_model, double Cs) {
  Ref* r = new Ref();
  r->nu = nu; r->CFL = CFL; r->dPdx = dPdx; r->x_mass_cte = x_mass_cte; r->LES_model = LES_model;
  r->Dirichlet_nu_t = Dirichlet_nu_t; r->wall_model = wall_model; r->Cs = Cs;
  r->setup(nx, ny, nz, x, y, z);
  return r;
}

void refcpu_upload(void* h, const double* U, const double* V, const double* W) {
  Ref* r = (Ref*)h;
  std::memcpy(r->U.v.data(), U, 8 * r->U.v.size());
  std::memcpy(r->V.v.data(), V, 8 * r->V.v.size());
  std::memcpy(r->W.v.data(), W, 8 * r->W.v.size());
  r->bc();
  r->Q0 = r->mass_flow_U();
}

void refcpu_step(void* h, int n) {
  Ref* r = (Ref*)h;
  for (int s = 0; s < n; ++s) { r->compute_dt(); r->rk3(); }
}

void refcpu_download(void* h, double* U, double* V, double* W, double* dt) {
  Ref* r = (Ref*)h;
  if (U) std::memcpy(U, r->U.v.data(), 8 * r->U.v.size());
  if (V) std::memcpy(V, r->V.v.data(), 8 * r->V.v.size());
  if (W) std::memcpy(W, r->W.v.data(), 8 * r->W.v.size());
  if (dt) *dt = r->dt;
}

int refcpu_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void refcpu_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

void refcpu_destroy(void* h) { delete (Ref*)h; }

}  // extern "C"
