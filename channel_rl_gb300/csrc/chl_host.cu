// C ABI (include/chl.h): instance setup, device memory, the step schedule and
// its CUDA graph.  The grid constants follow initialize
// (initialization.f90:187-427); the step schedule follows
// compute_time_step_RK3 (time_integration.f90:24-96) and the app_main loop
// (app_main.f90:114-117).
#include "../../include/chl.h"
#include "chl_common.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

// ------------------------------------------------------------ launchers (other TUs)
extern "C" {
void chl_launch_flux(const ChlMap&, int, int, cudaStream_t);
void chl_launch_update(const ChlMap&, int, int, int, int, int, cudaStream_t);
void chl_launch_edges(const ChlMap&, int, int, int, cudaStream_t);
void chl_launch_centre(const ChlMap&, int, int, int, int, cudaStream_t);
void chl_launch_filter_y(const ChlMap&, int, int, cudaStream_t);
void chl_launch_filter_x(const ChlMap&, int, cudaStream_t);
void chl_launch_filter_z(const ChlMap&, int, cudaStream_t);
void chl_launch_dsm_final(const ChlMap&, int, int, cudaStream_t);
void chl_launch_coef(const ChlMap&, cudaStream_t);
void chl_launch_eqwm(const ChlMap&, int, int, cudaStream_t);
void chl_launch_nut(const ChlMap&, int, int, int, cudaStream_t);
void chl_launch_amd(const ChlMap&, int, int, int, cudaStream_t);
void chl_launch_vreman(const ChlMap&, int, int, int, cudaStream_t);
void chl_launch_agent_obs(const ChlInst*, int, int, double, const int*, const double*, double*, double*, cudaStream_t);
size_t chl_smem_fftx(int, int, int);
size_t chl_smem_fftz(int, int, int);
int chl_fftz_cols(int, long, int, int);
int chl_fft_setup(size_t, size_t, size_t);
size_t chl_smem_tri(int, long, int);
int chl_tri_modes_per_block(size_t);
void chl_launch_div_fftx(const ChlMap&, int, int, size_t, int, int, int, cudaStream_t);
void chl_launch_fftz(const ChlMap&, int, int, size_t, int, int, cudaStream_t);
void chl_launch_tri(const ChlMap&, int, size_t, cudaStream_t);
void chl_launch_tri_scan(const ChlMap&, int, cudaStream_t);
size_t chl_smem_zsolve(int, int, int);
int chl_zsolve_setup(size_t);
void chl_launch_zsolve(const ChlMap&, int, int, size_t, cudaStream_t);
void chl_launch_fftx_inv(const ChlMap&, int, int, size_t, int, int, cudaStream_t);
void chl_launch_project(const ChlMap&, int, int, cudaStream_t);
void chl_launch_pbc(const ChlMap&, int, int, cudaStream_t);
void chl_launch_pghost(const ChlMap&, int, cudaStream_t);
void chl_launch_pack(double*, const double*, int, int, int, int, int, int, double, cudaStream_t);
void chl_launch_unpack3(const ChlFields3&, int, int, cudaStream_t);
void chl_launch_pack3(const ChlFields3&, int, int, cudaStream_t);
void chl_launch_pack_unique(double*, const double*, int, int, int, int, int, cudaStream_t);
void chl_launch_minabs(const ChlMap&, int, int, cudaStream_t);
void chl_launch_minabs_init(const ChlMap&, cudaStream_t);
void chl_launch_nonfinite(const ChlMap&, int, int, cudaStream_t);
void chl_launch_massflow(const ChlMap&, cudaStream_t, int, int);
void chl_launch_shift(const ChlMap&, int, int, cudaStream_t);
void chl_launch_tadvance(const ChlMap&, cudaStream_t);
void chl_launch_divmax(const ChlMap&, int, int, double*, cudaStream_t);
void chl_launch_qflow(const ChlInst*, int, int, int, cudaStream_t);
void chl_launch_stats(const ChlMap&, int, double*, int, int, cudaStream_t);
int chl_mlp_setup();
void chl_launch_mlp(const ChlMap&, int, int, int, int*, cudaStream_t);
void chl_launch_mlp_test(const float*, const float*, const float*, int, float*, float*, int*, cudaStream_t);
int chl_tc_selftest_launch(const void*, const void*, float*, int, int*, cudaStream_t);
void chl_launch_sqrt_selftest(const double*, double*, long, cudaStream_t);
}

namespace {

constexpr double RK_T[3] = {8.0 / 15.0, 2.0 / 3.0, 1.0};

enum { M_PT, M_EDGE, M_FULL, M_DSMF, M_WALL, M_PLANE, M_FFTX, M_FFTZ, M_TRI, M_MINABS, M_ROWS, M_MLP, M_WALLN,
       M_ZPLANE, M_ZSOLVE, M_EPAIR, M_FULLZ2, M_FULLX2, NMAP };
constexpr int MLP_NPARAM = 4545;

// Grid constants of one instance (host, FP64), in the device index
// convention of chl_common.cuh.  Arrays along x and z carry one slot of
// offset so that index -1 is addressable; undefined entries are NaN.
struct Consts {
  int nx, ny, nz, nxg, nyg, nzg, Nx, Ny, Nz, Nxh;
  std::vector<double> xf, yf, zf, xg, yg, zg;   // 1-based Fortran copies (index 0 unused)
  std::vector<double> rdxc, rdxf, dxf, rdzc, rdzf, dzf;   // offset 1, length N+3
  std::vector<double> hx2, hz2, hy2;                       // squared centre widths (x, z offset 1)
  std::vector<double> rdyc, rdyf, dyf, w0, w1;            // length Ny+2
  std::vector<double> csdelta, dwall;                     // length Ny+2
  std::vector<double> kxx, kzz;
  std::vector<double> Dd, Du, Dl;                          // 1-based by j_f
  double dxmin, dymin, dzmin, coef_bc_1, coef_bc_2;
};

const double NaN = std::nan("");

void centres(const std::vector<double>& f, int n, std::vector<double>& g) {
  // initialization.f90:194-220: g(2:n) = midpoints, g(1), g(n+1) mirrored
  std::vector<double> m(n);   // m[i] i=1..n-1
  for (int i = 1; i <= n - 1; ++i) m[i] = 0.5 * (f[i] + f[i + 1]);
  g.assign(n + 2, 0.0);
  for (int i = 2; i <= n; ++i) g[i] = m[i - 1];
  g[1] = m[1] - 2.0 * (m[1] - f[1]);
  g[n + 1] = m[n - 1] + 2.0 * (f[n] - m[n - 1]);
}

std::vector<double> kmod(int N, double d) {
  // initialization.f90:296-308
  std::vector<double> k(N, 0.0);
  const double pi = 4.0 * std::atan(1.0);
  const int half = (int)std::ceil((double)N / 2.0);
  for (int i = 0; i <= half && i < N; ++i) k[i] = 2.0 * (std::cos(2.0 * pi * (double)i / (double)N) - 1.0) / std::pow(d, 2.0);
  for (int i = half + 1; i < N; ++i) k[i] = 2.0 * (std::cos(2.0 * pi * (double)(-N + i) / (double)N) - 1.0) / std::pow(d, 2.0);
  return k;
}

int make_consts(const chl_grid_desc& d, Consts& c, std::string& err) {
  if (d.nx < 6 || d.nz < 6 || d.ny < 6 || (d.nx % 2) || (d.nz % 2)) {
    err = "grid: nx, nz must be even and >= 6, ny >= 6";
    return CHL_E_ARG;
  }
  if (!d.x || !d.y || !d.z) { err = "grid: null coordinate array"; return CHL_E_ARG; }
  c.nx = d.nx; c.ny = d.ny; c.nz = d.nz;
  c.nxg = d.nx + 1; c.nyg = d.ny + 1; c.nzg = d.nz + 1;
  c.Nx = d.nx - 2; c.Ny = d.ny - 1; c.Nz = d.nz - 2; c.Nxh = c.Nx / 2 + 1;
  auto rem = [](int n) { while (n % 4 == 0) n /= 4; while (n % 3 == 0) n /= 3; while (n % 2 == 0) n /= 2; return n; };
  if (rem(c.Nx) != 1 || rem(c.Nz) != 1) { err = "grid: Nx = nx-2 and Nz = nz-2 must be of the form 2^a 3^b"; return CHL_E_ARG; }
  // the kernels index an instance's points in 32 bits (chl_split)
  if ((long)c.Nx * (c.Ny + 2) * c.Nz >= (1L << 31)) { err = "grid: Nx (Ny+2) Nz must be below 2^31"; return CHL_E_ARG; }
  c.xf.assign(c.nx + 1, 0.0); c.yf.assign(c.ny + 1, 0.0); c.zf.assign(c.nz + 1, 0.0);
  for (int i = 1; i <= c.nx; ++i) c.xf[i] = d.x[i - 1];
  for (int j = 1; j <= c.ny; ++j) c.yf[j] = d.y[j - 1];
  for (int k = 1; k <= c.nz; ++k) c.zf[k] = d.z[k - 1];
  for (int i = 2; i <= c.nx; ++i) if (!(c.xf[i] > c.xf[i - 1])) { err = "grid: x not increasing"; return CHL_E_ARG; }
  for (int i = 2; i <= c.ny; ++i) if (!(c.yf[i] > c.yf[i - 1])) { err = "grid: y not increasing"; return CHL_E_ARG; }
  for (int i = 2; i <= c.nz; ++i) if (!(c.zf[i] > c.zf[i - 1])) { err = "grid: z not increasing"; return CHL_E_ARG; }
  // The Fourier solve's modified wavenumbers (initialization.f90:296-308)
  // take one spacing per periodic direction, as the reference's do: x and z
  // must be uniform (to rounding).
  auto uniform = [](const std::vector<double>& f, int n) {
    const double d0 = (f[n] - f[1]) / (n - 1);
    for (int i = 2; i <= n; ++i) if (std::fabs((f[i] - f[i - 1]) - d0) > 1e-9 * d0) return false;
    return true;
  };
  if (!uniform(c.xf, c.nx) || !uniform(c.zf, c.nz)) { err = "grid: x and z must be uniformly spaced"; return CHL_E_ARG; }
  centres(c.xf, c.nx, c.xg); centres(c.yf, c.ny, c.yg); centres(c.zf, c.nz, c.zg);
  auto dmin = [](const std::vector<double>& g, int n) {
    double m = INFINITY; for (int i = 2; i <= n; ++i) m = std::min(m, g[i] - g[i - 1]); return m; };
  c.dxmin = dmin(c.xg, c.nxg); c.dymin = dmin(c.yg, c.nyg); c.dzmin = dmin(c.zg, c.nzg);
  // x/z spacings (device index i <-> Fortran i+2), stored with offset 1
  auto periodic = [&](const std::vector<double>& f, const std::vector<double>& g, int N,
                      std::vector<double>& rc, std::vector<double>& rf, std::vector<double>& df) {
    rc.assign(N + 3, NaN); rf.assign(N + 3, NaN); df.assign(N + 3, NaN);
    for (int i = 0; i <= N; ++i) rc[i + 1] = 1.0 / (f[i + 2] - f[i + 1]);
    for (int i = -1; i <= N; ++i) { df[i + 1] = g[i + 3] - g[i + 2]; rf[i + 1] = 1.0 / df[i + 1]; }
  };
  periodic(c.xf, c.xg, c.Nx, c.rdxc, c.rdxf, c.dxf);
  periodic(c.zf, c.zg, c.Nz, c.rdzc, c.rdzf, c.dzf);
  auto widths2 = [&](const std::vector<double>& f, int N, std::vector<double>& w) {
    w.assign(N + 3, NaN);
    for (int i = 0; i <= N; ++i) { const double d = f[i + 2] - f[i + 1]; w[i + 1] = d * d; }
  };
  widths2(c.xf, c.Nx, c.hx2);
  widths2(c.zf, c.Nz, c.hz2);
  c.hy2.assign(c.Ny + 2, NaN);
  for (int jc = 1; jc <= c.Ny; ++jc) { const double d = c.yf[jc + 1] - c.yf[jc]; c.hy2[jc] = d * d; }
  const int Ny = c.Ny;
  c.rdyc.assign(Ny + 2, NaN); c.rdyf.assign(Ny + 2, NaN); c.dyf.assign(Ny + 2, NaN);
  c.w0.assign(Ny + 2, NaN); c.w1.assign(Ny + 2, NaN);
  for (int jc = 1; jc <= Ny; ++jc) c.rdyc[jc] = 1.0 / (c.yf[jc + 1] - c.yf[jc]);
  for (int jv = 0; jv <= Ny; ++jv) {
    c.dyf[jv] = c.yg[jv + 2] - c.yg[jv + 1];
    c.rdyf[jv] = 1.0 / c.dyf[jv];
    // weight_y_0(j) = (yg(j+1)-y(j))/(yg(j+1)-yg(j)), j = jv+1 (initialization.f90:399-400)
    c.w0[jv] = (c.yg[jv + 2] - c.yf[jv + 1]) / (c.yg[jv + 2] - c.yg[jv + 1]);
    c.w1[jv] = 1.0 - c.w0[jv];
  }
  // static Smagorinsky: Cs*Delta_j and the van Driest wall distance (subgrid.f90:589-599)
  c.csdelta.assign(Ny + 2, 0.0); c.dwall.assign(Ny + 2, 0.0);
  for (int jc = 1; jc <= Ny; ++jc) {
    const int jf = jc + 1;
    const double Delta = std::pow(c.dxmin * c.dzmin * (c.yf[jf] - c.yf[jf - 1]), 1.0 / 3.0);
    c.csdelta[jc] = d.Cs * Delta;
    c.dwall[jc] = (jf < c.nyg / 2) ? (c.yg[jf] - c.yf[1]) : (c.yf[c.ny] - c.yg[jf]);
  }
  c.kxx = kmod(c.Nx, c.dxmin);
  c.kzz = kmod(c.Nz, c.dzmin);
  // Dyy (initialization.f90:355-385)
  c.Dd.assign(c.nyg + 1, 0.0); c.Du.assign(c.nyg + 1, 0.0); c.Dl.assign(c.nyg + 1, 0.0);
  auto abc = [&](int j, double& a, double& b, double& cc) {
    const std::vector<double>& y = c.yf; const std::vector<double>& yg = c.yg;
    a = 1.0 / (y[j] - y[j - 1]) / (yg[j + 1] - yg[j]);
    b = 1.0 / (y[j] - y[j - 1]) * (-1.0 / (yg[j + 1] - yg[j]) - 1.0 / (yg[j] - yg[j - 1]));
    cc = 1.0 / (y[j] - y[j - 1]) / (yg[j] - yg[j - 1]);
  };
  double a, b, cc;
  for (int j = 3; j <= c.nyg - 2; ++j) { abc(j, a, b, cc); c.Du[j] = a; c.Dl[j] = cc; c.Dd[j] = b; }
  abc(2, a, b, cc); c.Dd[2] = b + cc; c.Du[2] = a; c.coef_bc_1 = cc;
  abc(c.nyg - 1, a, b, cc); c.Dd[c.nyg - 1] = a + b; c.Dl[c.nyg - 1] = cc; c.coef_bc_2 = a;
  return CHL_OK;
}

struct Inst {
  Consts c;
  chl_grid_desc d;
  ChlInst dev{};
  void* arena = nullptr;
  bool uploaded = false;
  double* staging = nullptr;   // Fortran-layout staging: 3 fields in, then 3 fields out
  size_t nstage = 0;
  // ordering of the host-buffer round trip (chl_set_fields, chl_download_async)
  // between the compute stream and the two copy streams; created on first use
  cudaEvent_t ev_h2d = nullptr, ev_unpacked = nullptr, ev_packed = nullptr, ev_d2h = nullptr;
};

struct Arena {
  size_t off = 0;
  std::vector<std::pair<size_t, size_t>> plan;   // (offset, bytes)
  size_t take(size_t bytes) { size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; }
};

// Pass table of the length-N Stockham FFT (layout in chl_fft.cu): per pass
// with twiddles and butterfly class jm, the twiddles w_r = C + iS =
// exp(-2 pi i m/N), m = jm r N/(Ns R), each as sigma (C or S, the larger in
// magnitude) and m (S/C or C/S), and the butterfly's combined scales.
std::vector<double> fft_pass_table(int N) {
  std::vector<double> t((size_t)chl_tw_len(N));
  const double pi = 4.0 * std::atan(1.0);
  const double s3 = 0.86602540378443864676;   // sin(2 pi/3)
  int Ns = 1, rem = N;
  size_t off = 0;
  while (rem > 1) {
    const int R = chl_fft_radix(rem);
    if (Ns > 1) {
      const int tstep = N / (Ns * R);
      for (int jm = 0; jm < Ns; ++jm) {
        double sg[4] = {1.0, 1.0, 1.0, 1.0}, mu[4] = {0.0, 0.0, 0.0, 0.0};
        long long forms = 0;
        for (int r = 1; r < R; ++r) {
          const int m = jm * r * tstep;
          const double C = std::cos(2.0 * pi * m / N), S = -std::sin(2.0 * pi * m / N);
          const bool sform = std::fabs(S) > std::fabs(C);
          sg[r] = sform ? S : C;
          mu[r] = sform ? C / S : S / C;
          if (sform) forms |= 1LL << r;
        }
        auto put = [&](int f, double v) { t[off + (size_t)f * Ns + jm] = v; };
        put(0, mu[1]); put(1, mu[2]); put(3, sg[1]);
        if (R == 4) { put(2, mu[3]); put(4, sg[2]); put(5, sg[3] / sg[1]); }
        else if (R == 3) { put(2, s3 * sg[1]); put(4, 0.5 * sg[1]); put(5, sg[2] / sg[1]); }
        double fd;
        std::memcpy(&fd, &forms, 8);
        put(6, fd);
      }
      off += (size_t)CHL_TW_F * Ns;
    }
    Ns *= R; rem /= R;
  }
  return t;
}

int dsm_npart(int Nx, int Ny, int Nz) {
  const int p = chl_dsm_ppt(Nx, Ny, Nz);
  return (chl_dsm_points(Nx, Nz) + CHL_DSMF_THREADS * p - 1) / (CHL_DSMF_THREADS * p);
}

}  // namespace

struct ProfRec { const char* name; int ev; };

struct chl_handle {
  std::vector<Inst> in;
  // per-launch event profiling (chl_profile_step)
  bool prof = false;
  std::vector<cudaEvent_t> ev;
  std::vector<ProfRec> rec;
  ChlInst* d_inst = nullptr;
  cudaStream_t st = nullptr;
  // copy streams of the host-buffer round trip: the next step's upload and
  // the previous step's download run on the copy engines while a step
  // computes (created on the first chl_set_fields / chl_download_async)
  cudaStream_t st_h2d = nullptr, st_d2h = nullptr;
  std::string err;
  int* d_off[NMAP] = {};
  int nblk[NMAP] = {};
  size_t smem_x = 0, smem_z = 0, smem_t = 0;
  int zcw = 16;                       // kx columns per z-transform block
  int tx = 256, tz = 256;             // threads of the x and z transform blocks
  // projection tile shapes (chl_autotune): block-count targets of the x and
  // z transforms and the tridiagonal form: 0 row-batched, 1 staged, 2 the
  // default rule, 3 the fused z solve (z transform, tridiagonal and inverse
  // z transform in one cluster launch; bit-identical to the others)
  int x_min_blocks = CHL_FFT_MIN_BLOCKS, z_min_blocks = CHL_FFT_MIN_BLOCKS, tri_mode = 2;
  bool zsolve_ok = false;             // every instance has the same lane count and fits (chl_smem_zsolve)
  bool zsolve = false;                // the fused form is in use
  int zlanes = 1;                     // its cluster size
  size_t smem_zs = 0;
  int twz = 0;                        // longest z pass table of the instances (doubles)
  bool epair = false;                 // edges as x-pair sums (k_edges_pair): every Nx <= 256
  int tb_epair = 256;                 // its block: the largest Nx rounded up to a power of two, >= 64
  int tb_pt = 256;                    // threads per block of the point maps (stencils, updates)
  bool tri_scan = false;              // some instance splits its tridiagonal columns (chl_tri_lanes)
  int LES_model = 0, wall_model = 0, any_mass = 0;
  float* d_mlp_theta = nullptr;       // learned wall model parameters (shared)
  unsigned int* d_mlp_cfg = nullptr;  // sigma, train, seed lo/hi, evaluation counter, debug [5..6], shared draws [7]
  int* d_mlp_status = nullptr;
  double* d_divout = nullptr;
  double* d_stats = nullptr;
  double* d_agent = nullptr;          // wall-agent observations: inputs and outputs
  size_t agent_cap = 0;
  int stats_pitch = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  ChlMap map(int which) const {
    const bool pt = which == M_PT || which == M_EDGE || which == M_FULL || which == M_FULLZ2 || which == M_FULLX2;
    return ChlMap{d_inst, d_off[which], (int)in.size(), pt ? tb_pt : 256};
  }
};

#define CK(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) { \
  h->err = std::string("CUDA: ") + cudaGetErrorString(e_) + " at " #call; return CHL_E_CUDA; } } while (0)
// Wraps one kernel launch: with profiling on, brackets it by two events.
#define KL(name, call) do { \
  if (h->prof && h->rec.size() * 2 + 2 <= h->ev.size()) { \
    int e0_ = (int)h->rec.size() * 2; cudaEventRecord(h->ev[e0_], h->st); call; \
    cudaEventRecord(h->ev[e0_ + 1], h->st); h->rec.push_back(ProfRec{name, e0_}); \
  } else { call; } } while (0)
#define LAUNCHED() do { cudaError_t e_ = cudaGetLastError(); if (e_ != cudaSuccess) { \
  h->err = std::string("CUDA launch: ") + cudaGetErrorString(e_); return CHL_E_CUDA; } } while (0)

static int upload_consts(chl_handle* h, Inst& I) {
  Consts& c = I.c;
  const int Nx = c.Nx, Ny = c.Ny, Nz = c.Nz, Nxh = c.Nxh;
  const size_t nc = (size_t)Nx * (Ny + 2) * Nz, nv = (size_t)Nx * (Ny + 1) * Nz;
  const size_t nspec = (size_t)(Ny + 2) * Nz * Nxh, ntri = (size_t)Ny * Nz * Nxh;
  const bool dsm = I.d.LES_model == CHL_LES_DYNAMIC;
  const int npart = dsm_npart(Nx, Ny, Nz);
  Arena A;
  // constants
  size_t o_rdxc = A.take(8 * (Nx + 3)), o_rdxf = A.take(8 * (Nx + 3)), o_dxf = A.take(8 * (Nx + 3));
  size_t o_rdzc = A.take(8 * (Nz + 3)), o_rdzf = A.take(8 * (Nz + 3)), o_dzf = A.take(8 * (Nz + 3));
  size_t o_rdyc = A.take(8 * (Ny + 2)), o_rdyf = A.take(8 * (Ny + 2)), o_dyf = A.take(8 * (Ny + 2));
  size_t o_hx2 = A.take(8 * (Nx + 3)), o_hz2 = A.take(8 * (Nz + 3)), o_hy2 = A.take(8 * (Ny + 2));
  size_t o_w0 = A.take(8 * (Ny + 2)), o_w1 = A.take(8 * (Ny + 2)), o_ygc = A.take(8 * (Ny + 2));
  size_t o_rdxc4 = A.take(8 * (Nx + 3)), o_rdyc4 = A.take(8 * (Ny + 2)), o_rdzc4 = A.take(8 * (Nz + 3));
  size_t o_rdxc2 = A.take(8 * (Nx + 3)), o_rdyc2 = A.take(8 * (Ny + 2)), o_rdzc2 = A.take(8 * (Nz + 3));
  size_t o_rdxcs = A.take(8 * (Nx + 3)), o_rdycs = A.take(8 * (Ny + 2)), o_rdzcs = A.take(8 * (Nz + 3));
  size_t o_rdxfs = A.take(8 * (Nx + 3)), o_rdyfs = A.take(8 * (Ny + 2)), o_rdzfs = A.take(8 * (Nz + 3));
  size_t o_w0u = A.take(8 * (Ny + 2)), o_w1u = A.take(8 * (Ny + 2));
  size_t o_csd = A.take(8 * (Ny + 2)), o_dw = A.take(8 * (Ny + 2));
  size_t o_twx = A.take(8 * (size_t)chl_tw_len(Nx)), o_twz = A.take(8 * (size_t)chl_tw_len(Nz));
  size_t o_ti = A.take(8 * ntri), o_tm = A.take(8 * ntri), o_tc = A.take(8 * ntri);
  // state
  size_t o_U[3], o_V[3], o_W[3], o_F1[3], o_Fp[3];
  for (int s = 0; s < 3; ++s) { o_U[s] = A.take(8 * nc); o_V[s] = A.take(8 * nv); o_W[s] = A.take(8 * nc); }
  for (int s = 0; s < 3; ++s) o_F1[s] = A.take(8 * (s == 1 ? nv : nc));
  for (int s = 0; s < 3; ++s) o_Fp[s] = A.take(8 * (s == 1 ? nv : nc));
  size_t o_nut = A.take(8 * nc), o_S = A.take(8 * nc);
  size_t o_G[9];
  for (int m = 0; m < 9; ++m) o_G[m] = A.take(8 * nc);
  size_t o_q[CHL_NQ] = {}, o_r[CHL_NQ] = {};
  if (dsm) for (int m = 0; m < CHL_NQ; ++m) { o_q[m] = A.take(8 * nc); o_r[m] = A.take(8 * nc); }
  size_t o_E[3];
  for (int m = 0; m < 3; ++m) o_E[m] = A.take(8 * nc);
  size_t o_spec = A.take(16 * nspec), o_p = A.take(8 * nc), o_P = A.take(8 * nc);
  size_t o_alpha = A.take(8 * 2 * (size_t)Nx * Nz), o_bc = A.take(8 * 2 * (size_t)Nx * Nz);
  size_t o_part = A.take(8 * 2 * (size_t)(Ny + 2) * npart * CHL_DSMF_THREADS);   // one partial per DSM thread
  size_t o_coef = A.take(8 * (Ny + 2)), o_scal = A.take(8 * CHL_S_NSCAL);
  size_t o_min = A.take(8 * (size_t)(Nx + Ny + 1 + Nz)), o_status = A.take(64);
  size_t o_dcnt = A.take(4 * (size_t)(Ny + 2));
  size_t o_red = A.take(8 * 2 * (size_t)Nz);
  size_t o_trace = A.take(4 * (size_t)MLP_NPARAM);
  const bool mlp = I.d.wall_model == CHL_WM_MLP;
  size_t o_rec = mlp ? A.take(4 * (size_t)CHL_MLP_REC * 3 * 2 * Nx * Nz) : 0;
  I.nstage = (size_t)c.nxg * c.nyg * c.nzg;
  size_t o_stage = A.take(6 * 8 * I.nstage);   // Fortran-layout fields: 3 in, 3 out (chl_set_fields, chl_download_async)
  cudaError_t e = cudaMalloc(&I.arena, A.off);
  if (e != cudaSuccess) { h->err = "device allocation failed (" + std::to_string(A.off) + " bytes)"; return CHL_E_NOMEM; }
  CK(cudaMemsetAsync(I.arena, 0, A.off, h->st));
  char* base = (char*)I.arena;
  auto P = [&](size_t o) { return (double*)(base + o); };
  ChlInst& D = I.dev;
  D.Nx = Nx; D.Ny = Ny; D.Nz = Nz; D.Nxh = Nxh;
  D.LES_model = I.d.LES_model; D.Dirichlet_nu_t = I.d.Dirichlet_nu_t;
  D.wall_model = I.d.wall_model; D.x_mass_cte = I.d.x_mass_cte;
  D.fk[FK_ONE] = 1.0; D.fk[FK_MZERO] = -0.0; D.fk[FK_FOUR] = 4.0;
  D.nu = I.d.nu; D.CFL = I.d.CFL; D.Cs = I.d.Cs;
  D.dxmin = c.dxmin; D.dymin = c.dymin; D.dzmin = c.dzmin;
  {
    // the viscous limit of compute_dt, CFL*dxmin**2/nu (time_integration.f90:
    // 131-134), in the reference's order of operations, once per instance
    const double C = I.d.CFL, nu = I.d.nu;
    const double vx = C * (c.dxmin * c.dxmin) / nu, vy = C * (c.dymin * c.dymin) / nu, vz = C * (c.dzmin * c.dzmin) / nu;
    D.dt_vis = std::fmin(std::fmin(vx, vy), vz);
  }
  D.dyw = c.yg[2] - c.yg[1];
  D.hb = c.yg[4] - c.yf[1];
  D.ht = c.yf[c.ny] - c.yg[c.nyg - 3];
  D.cbc1 = c.coef_bc_1 * (c.yg[2] - c.yg[1]);
  D.cbc2 = c.coef_bc_2 * (c.yg[c.nyg] - c.yg[c.nyg - 1]);
  D.ybot = c.yf[1]; D.ytop = c.yf[c.ny];
  D.dy1 = c.yf[2] - c.yf[1];
  const std::vector<double>& y = c.yf;
  D.gb1 = (-3.0 * y[1] + 4.0 * y[2] - y[3]) / 2.0;
  D.gb2 = 2.0 * y[1] - 5.0 * y[2] + 4.0 * y[3] - 1.0 * y[4];
  D.gt1 = (3.0 * y[c.ny] - 4.0 * y[c.ny - 1] + y[c.ny - 2]) / 2.0;
  D.gt2 = 2.0 * y[c.ny] - 5.0 * y[c.ny - 1] + 4.0 * y[c.ny - 2] - 1.0 * y[c.ny - 3];
  D.dygb = c.yg[2] - c.yg[1]; D.dygt = c.yg[c.nyg] - c.yg[c.nyg - 1];
  D.mass_norm = 1.0 / ((double)Nx * Nz);
  D.rdxc = P(o_rdxc) + 1; D.rdxf = P(o_rdxf) + 1; D.dxf = P(o_dxf) + 1;
  D.rdzc = P(o_rdzc) + 1; D.rdzf = P(o_rdzf) + 1; D.dzf = P(o_dzf) + 1;
  D.hx2 = P(o_hx2) + 1; D.hz2 = P(o_hz2) + 1; D.hy2 = P(o_hy2);
  D.rdyc = P(o_rdyc); D.rdyf = P(o_rdyf); D.dyf = P(o_dyf); D.w0x2 = P(o_w0); D.w1x2 = P(o_w1); D.ygc = P(o_ygc);
  D.rdxc4 = P(o_rdxc4) + 1; D.rdyc4 = P(o_rdyc4); D.rdzc4 = P(o_rdzc4) + 1;
  D.rdxc2 = P(o_rdxc2) + 1; D.rdyc2 = P(o_rdyc2); D.rdzc2 = P(o_rdzc2) + 1;
  D.rdxcs = P(o_rdxcs) + 1; D.rdycs = P(o_rdycs); D.rdzcs = P(o_rdzcs) + 1;
  D.rdxfs = P(o_rdxfs) + 1; D.rdyfs = P(o_rdyfs); D.rdzfs = P(o_rdzfs) + 1;
  D.w0 = P(o_w0u); D.w1 = P(o_w1u);
  D.smag_csdelta = P(o_csd); D.smag_dwall = P(o_dw);
  D.twx = (const double*)(base + o_twx); D.twz = (const double*)(base + o_twz);
  D.tri_inv = P(o_ti); D.tri_m = P(o_tm); D.tri_c = P(o_tc);
  for (int s = 0; s < 3; ++s) { D.U[s] = P(o_U[s]); D.V[s] = P(o_V[s]); D.W[s] = P(o_W[s]); D.F1[s] = P(o_F1[s]); D.Fp[s] = P(o_Fp[s]); }
  D.nut = P(o_nut); D.S = P(o_S);
  for (int m = 0; m < 9; ++m) D.G[m] = P(o_G[m]);
  for (int m = 0; m < CHL_NQ; ++m) { D.q[m] = dsm ? P(o_q[m]) : nullptr; D.r[m] = dsm ? P(o_r[m]) : nullptr; }
  for (int m = 0; m < 3; ++m) D.E[m] = P(o_E[m]);
  D.spec = (double2*)(base + o_spec); D.p = P(o_p); D.P = P(o_P);
  D.alpha = P(o_alpha); D.bc = P(o_bc); D.part = P(o_part); D.npart = npart; D.dsm_ppt = chl_dsm_ppt(Nx, Ny, Nz);
  D.coef = P(o_coef); D.scal = P(o_scal);
  D.minabs = (unsigned long long*)(base + o_min); D.red = P(o_red); D.status = (int*)(base + o_status);
  D.dsm_cnt = (int*)(base + o_dcnt);
  D.retau = I.d.Re_tau;
  D.mlp_trace = (float*)(base + o_trace);
  D.mlp_theta = h->d_mlp_theta;
  D.mlp_cfg = h->d_mlp_cfg;
  D.mlp_rec = mlp ? (float*)(base + o_rec) : nullptr;
  I.staging = P(o_stage);
  // host constant arrays -> device
  auto put = [&](size_t o, const std::vector<double>& v) { return cudaMemcpyAsync(base + o, v.data(), 8 * v.size(), cudaMemcpyHostToDevice, h->st); };
  CK(put(o_rdxc, c.rdxc)); CK(put(o_rdxf, c.rdxf)); CK(put(o_dxf, c.dxf));
  CK(put(o_rdzc, c.rdzc)); CK(put(o_rdzf, c.rdzf)); CK(put(o_dzf, c.dzf));
  CK(put(o_rdyc, c.rdyc)); CK(put(o_rdyf, c.rdyf)); CK(put(o_dyf, c.dyf));
  CK(put(o_hx2, c.hx2)); CK(put(o_hz2, c.hz2)); CK(put(o_hy2, c.hy2));
  const std::vector<double> ygc(c.yg.begin() + 1, c.yg.begin() + 1 + c.nyg);
  CK(put(o_ygc, ygc));
  // the flux kernel keeps its centre and xz-edge fluxes 4 x and its xy and
  // yz edge fluxes 2 x (chl_rhs.cu): doubled y weights, quadrupled and
  // doubled centre reciprocals, exact power-of-two scalings (kept in
  // `scaled` for the rest of this function)
  std::vector<std::vector<double>> scaled;
  auto times = [&scaled](const std::vector<double>& v, double f) -> const std::vector<double>& {
    scaled.emplace_back(v);
    for (auto& x : scaled.back()) x *= f;
    return scaled.back();
  };
  scaled.reserve(16);
  CK(put(o_w0, times(c.w0, 2.0))); CK(put(o_w1, times(c.w1, 2.0)));
  CK(put(o_w0u, c.w0)); CK(put(o_w1u, c.w1));
  CK(put(o_rdxc4, times(c.rdxc, 4.0))); CK(put(o_rdyc4, times(c.rdyc, 4.0))); CK(put(o_rdzc4, times(c.rdzc, 4.0)));
  CK(put(o_rdxc2, times(c.rdxc, 2.0))); CK(put(o_rdyc2, times(c.rdyc, 2.0))); CK(put(o_rdzc2, times(c.rdzc, 2.0)));
  const double fs = std::sqrt(4.0 / 216.0);
  CK(put(o_rdxcs, times(c.rdxc, fs))); CK(put(o_rdycs, times(c.rdyc, fs))); CK(put(o_rdzcs, times(c.rdzc, fs)));
  CK(put(o_rdxfs, times(c.rdxf, fs))); CK(put(o_rdyfs, times(c.rdyf, fs))); CK(put(o_rdzfs, times(c.rdzf, fs)));
  CK(put(o_csd, c.csdelta)); CK(put(o_dw, c.dwall));
  {
    const std::vector<double> tx = fft_pass_table(Nx), tz = fft_pass_table(Nz);
    if (!tx.empty()) CK(cudaMemcpy(base + o_twx, tx.data(), 8 * tx.size(), cudaMemcpyHostToDevice));
    if (!tz.empty()) CK(cudaMemcpy(base + o_twz, tz.data(), 8 * tz.size(), cudaMemcpyHostToDevice));
  }
  // Thomas factors per mode: denominators of the elimination of
  // Dyy + kxx + kzz (the zgtsv system of projection.f90:97-110), with the
  // 1/(2 Nx Nz) of the packed inverse transform folded into inv.
  {
    std::vector<double> fi(ntri), fm(ntri), fc(ntri);
    const double scale = 1.0 / (2.0 * (double)Nx * (double)Nz);
    for (int kz = 0; kz < Nz; ++kz)
      for (int kx = 0; kx < Nxh; ++kx) {
        const double lam = c.kxx[kx] + c.kzz[kz];
        double cprev = 0.0;
        for (int r = 0; r < Ny; ++r) {
          const int jf = r + 2;
          double D_ = c.Dd[jf] + lam;
          if (kx == 0 && kz == 0 && r == 0) D_ = 3.0 / 2.0 * D_;
          const double L = r > 0 ? c.Dl[jf] : 0.0;
          const double Uu = r < Ny - 1 ? c.Du[jf] : 0.0;
          const double den = D_ - L * cprev;
          const size_t o = ((size_t)r * Nz + kz) * Nxh + kx;
          fi[o] = scale / den;
          fm[o] = L / den;
          fc[o] = Uu / den;
          cprev = Uu / den;
        }
      }
    CK(cudaMemcpy(base + o_ti, fi.data(), 8 * ntri, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(base + o_tm, fm.data(), 8 * ntri, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(base + o_tc, fc.data(), 8 * ntri, cudaMemcpyHostToDevice));
  }
  std::vector<double> scal(CHL_S_NSCAL, 0.0);
  scal[CHL_S_DPDX] = I.d.dPdx;
  CK(cudaMemcpy(base + o_scal, scal.data(), 8 * CHL_S_NSCAL, cudaMemcpyHostToDevice));
  return CHL_OK;
}

static int build_maps(chl_handle* h) {
  const int n = (int)h->in.size();
  auto cdiv = [](long a, long b) { return (int)((a + b - 1) / b); };
  int mz = 0, my = 0;
  long zcols = 0, modes = 0;
  for (auto& I : h->in) {
    mz = std::max(mz, I.c.Nz); my = std::max(my, I.c.Ny);
    zcols += (long)I.c.Ny * I.c.Nxh;
    modes += (long)I.c.Nz * I.c.Nxh;
  }
  h->twz = 0;
  for (auto& I : h->in) h->twz = std::max(h->twz, chl_tw_len(I.c.Nz));
  h->zcw = chl_fftz_cols(mz, zcols, h->z_min_blocks, h->twz);
  h->tz = chl_fft_threads(h->zcw, mz);
  h->tx = 64;
  for (auto& I : h->in) {
    const int nrow = I.c.Ny * (I.c.Nz / 2);
    h->tx = std::max(h->tx, chl_fft_threads(chl_fftx_rows(I.c.Nx, nrow, h->x_min_blocks), I.c.Nx));
  }
  h->tri_scan = false;
  for (auto& I : h->in) h->tri_scan = h->tri_scan || chl_tri_lanes((long)I.c.Nz * I.c.Nxh, I.c.Ny) > 1;
  // fused z solve: needs one lane count for the whole launch (the cluster
  // size) and every instance's row block in shared memory; by default it is
  // used where the tridiagonal solve splits its columns (few modes)
  h->zsolve_ok = true;
  h->smem_zs = 0;
  h->zlanes = chl_tri_lanes((long)h->in[0].c.Nz * h->in[0].c.Nxh, h->in[0].c.Ny);
  for (auto& I : h->in) {
    const size_t b = chl_smem_zsolve(I.c.Nx, I.c.Ny, I.c.Nz);
    h->zsolve_ok = h->zsolve_ok && b > 0 && chl_tri_lanes((long)I.c.Nz * I.c.Nxh, I.c.Ny) == h->zlanes;
    h->smem_zs = std::max(h->smem_zs, b);
  }
  h->zsolve = h->zsolve_ok && (h->tri_mode == 3 || (h->tri_mode == 2 && h->zlanes > 1));
  h->epair = true;
  int mx = 0;
  for (auto& I : h->in) { h->epair = h->epair && I.c.Nx <= 256; mx = std::max(mx, I.c.Nx); }
  h->tb_epair = 64;
  while (h->tb_epair < mx && h->tb_epair < 256) h->tb_epair *= 2;
  h->smem_t = h->tri_scan ? 0 : chl_smem_tri(my, modes, h->tri_mode);
  const int tri_w = chl_tri_modes_per_block(h->smem_t);
  for (int m = 0; m < NMAP; ++m) {
    std::vector<int> off(n + 1, 0);
    for (int q = 0; q < n; ++q) {
      const Consts& c = h->in[q].c;
      const int Nx = c.Nx, Ny = c.Ny, Nz = c.Nz, Nxh = c.Nxh;
      int b = 0;
      switch (m) {
        case M_PT: b = cdiv((long)Nx * Ny * Nz, h->tb_pt); break;
        case M_EDGE: b = cdiv((long)Nx * (Ny + 1) * Nz, h->tb_pt); break;
        case M_FULL: b = cdiv((long)Nx * (Ny + 2) * Nz, h->tb_pt); break;
        case M_FULLZ2: b = cdiv((long)Nx * (Ny + 2) * (Nz / 2), h->tb_pt); break;   // z planes in pairs (Nz even)
        case M_FULLX2: b = cdiv((long)(Nx / 2) * (Ny + 2) * Nz, h->tb_pt); break;   // x points in pairs (Nx even)
        case M_DSMF: b = Ny * dsm_npart(Nx, Ny, Nz); break;
        case M_WALL: b = cdiv(2L * Nx * Nz, 256); break;
        case M_PLANE: b = cdiv((long)Nx * Nz, 256); break;
        case M_FFTX: b = cdiv((long)Ny * (Nz / 2), chl_fftx_rows(Nx, Ny * (Nz / 2), h->x_min_blocks)); break;
        case M_FFTZ: b = cdiv((long)Ny * Nxh, h->zcw); break;
        case M_TRI: b = h->tri_scan ? cdiv((long)Nz * Nxh * chl_tri_lanes((long)Nz * Nxh, Ny), 128)
                                    : cdiv((long)Nz * Nxh, tri_w); break;
        case M_MINABS: b = Nz * ((Ny + 15) / 16); break;   // planes x 16-row chunks (chl_misc.cu)
        case M_ROWS: b = Ny + 1; break;
        case M_MLP: b = cdiv(2L * Nx * Nz, 128); break;
        case M_WALLN: b = cdiv(2L * Nx * Nz, CHL_WALL_THREADS); break;
        case M_ZPLANE: b = Nz; break;
        case M_ZSOLVE: b = Nxh * h->zlanes; break;
        case M_EPAIR: b = Nx <= h->tb_epair ? cdiv((long)(Ny + 1) * Nz, h->tb_epair / Nx) : 1; break;   // whole x-rows
      }
      off[q + 1] = off[q] + b;
    }
    h->nblk[m] = off[n];
    if (!h->d_off[m]) CK(cudaMalloc(&h->d_off[m], sizeof(int) * (n + 1)));   // rebuilt by chl_autotune
    CK(cudaMemcpy(h->d_off[m], off.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
  }
  // dynamic shared memory is per launch, so it must hold the largest
  // per-instance need: the x transform of an instance stages
  // chl_fftx_rows rows of Nx, which is not monotonic in Nx
  size_t sx = 0;
  for (auto& I : h->in) sx = std::max(sx, chl_smem_fftx(I.c.Nx, I.c.Ny * (I.c.Nz / 2), h->x_min_blocks));
  h->smem_x = sx;
  h->smem_z = chl_smem_fftz(mz, h->zcw, h->twz);
  if (chl_fft_setup(h->smem_x, h->smem_z, h->smem_t)) { h->err = "FFT shared-memory size not supported"; return CHL_E_ARG; }
  if (h->zsolve && chl_zsolve_setup(h->smem_zs)) { h->err = "fused z solve: shared-memory size not supported"; return CHL_E_ARG; }
  if (chl_mlp_setup()) { h->err = "wall-model network shared-memory size not supported"; return CHL_E_ARG; }
  return CHL_OK;
}

// ------------------------------------------------------------ schedules
static int enqueue_sgs(chl_handle* h, int s, bool with_wm, int stage = 0) {
  cudaStream_t st = h->st;
  // AMD and Vreman write nu + nu_t in their own kernel, whose wall-model
  // rows need the wall stress first; the other models leave it to k_nut
  const bool fused = h->LES_model == CHL_LES_AMD || h->LES_model == CHL_LES_VREMAN;
  auto wall_stress = [&]() {
    if (with_wm && (h->wall_model == CHL_WM_EQLOG || h->wall_model == CHL_WM_MLP))
      KL("eq_wallmodel", chl_launch_eqwm(h->map(M_WALLN), h->nblk[M_WALLN], s, st));
    if (with_wm && h->wall_model == CHL_WM_MLP)
      KL("mlp_wallmodel", chl_launch_mlp(h->map(M_MLP), h->nblk[M_MLP], s, stage, h->d_mlp_status, st));
  };
  if (fused) wall_stress();
  if (h->LES_model == CHL_LES_DYNAMIC) {
    KL("edges", chl_launch_edges(h->map(h->epair ? M_EPAIR : M_EDGE), h->nblk[h->epair ? M_EPAIR : M_EDGE], s,
                                 h->epair ? h->tb_epair : 0, st));
    KL("centre_strain", chl_launch_centre(h->map(M_PT), h->nblk[M_PT], s, 1, h->epair, st));
    KL("filter_y", chl_launch_filter_y(h->map(M_FULL), h->nblk[M_FULL], s, st));
    KL("filter_x", chl_launch_filter_x(h->map(M_FULLX2), h->nblk[M_FULLX2], st));
    KL("filter_z", chl_launch_filter_z(h->map(M_FULLZ2), h->nblk[M_FULLZ2], st));
    KL("edges", chl_launch_edges(h->map(h->epair ? M_EPAIR : M_EDGE), h->nblk[h->epair ? M_EPAIR : M_EDGE], 3,
                                 h->epair ? h->tb_epair : 0, st));
    KL("dsm_LM_MM", chl_launch_dsm_final(h->map(M_DSMF), h->nblk[M_DSMF], h->epair, st));
  } else if (h->LES_model == CHL_LES_SMAGORINSKY) {
    KL("edges", chl_launch_edges(h->map(h->epair ? M_EPAIR : M_EDGE), h->nblk[h->epair ? M_EPAIR : M_EDGE], s,
                                 h->epair ? h->tb_epair : 0, st));
    KL("centre_strain", chl_launch_centre(h->map(M_PT), h->nblk[M_PT], s, 0, h->epair, st));
  } else if (h->LES_model == CHL_LES_AMD) {
    KL("amd", chl_launch_amd(h->map(M_PT), h->nblk[M_PT], s, with_wm ? 1 : 0, st));
  } else if (h->LES_model == CHL_LES_VREMAN) {
    KL("vreman", chl_launch_vreman(h->map(M_PT), h->nblk[M_PT], s, with_wm ? 1 : 0, st));
  }
  // the static model's row coefficient (the dynamic model's is formed by
  // the last block of each row of its plane sums)
  if (h->LES_model == CHL_LES_SMAGORINSKY) KL("nut_coef", chl_launch_coef(h->map(M_PT), st));
  if (!fused) {
    wall_stress();
    KL("nut", chl_launch_nut(h->map(M_FULL), h->nblk[M_FULL], s, with_wm ? 1 : 0, st));
  }
  LAUNCHED();
  return CHL_OK;
}

// mode 0: pseudo-pressure and the velocity correction of set s; 1: the
// actual pressure; 2: mode 0's transforms and solve without the correction
// (writes only the spectrum and the pseudo-pressure scratch; chl_autotune)
static int enqueue_projection(chl_handle* h, int s, int mode) {
  cudaStream_t st = h->st;
  const bool correct = mode == 0;
  if (mode == 2) mode = 0;
  KL("div_fft_x", chl_launch_div_fftx(h->map(M_FFTX), h->nblk[M_FFTX], h->tx, h->smem_x, s, mode, h->x_min_blocks, st));
  if (h->zsolve) {
    KL("z_solve", chl_launch_zsolve(h->map(M_ZSOLVE), h->nblk[M_ZSOLVE], h->zlanes, h->smem_zs, st));
  } else {
    KL("fft_z", chl_launch_fftz(h->map(M_FFTZ), h->nblk[M_FFTZ], h->tz, h->smem_z, 0, h->zcw, st));
    if (h->tri_scan) KL("tridiag", chl_launch_tri_scan(h->map(M_TRI), h->nblk[M_TRI], st));
    else KL("tridiag", chl_launch_tri(h->map(M_TRI), h->nblk[M_TRI], h->smem_t, st));
    KL("fft_z", chl_launch_fftz(h->map(M_FFTZ), h->nblk[M_FFTZ], h->tz, h->smem_z, 1, h->zcw, st));
  }
  KL("ifft_x", chl_launch_fftx_inv(h->map(M_FFTX), h->nblk[M_FFTX], h->tx, h->smem_x, mode == 0 ? 0 : 1, h->x_min_blocks, st));
  if (correct) KL("project", chl_launch_project(h->map(M_PT), h->nblk[M_PT], s, st));
  LAUNCHED();
  return CHL_OK;
}

// compute_dt: one launch.  k_minabs's last block per instance forms dt
// (and resets the minima); with every instance on a fixed step only the
// non-finite check runs, and it stores dt = -CFL.
static int enqueue_dt(chl_handle* h) {
  bool fixed = true;   // every instance on a fixed step: only the non-finite check
  for (auto& I : h->in) fixed = fixed && I.d.CFL < 0.0;
  if (fixed) KL("dt_minabs", chl_launch_nonfinite(h->map(M_PT), h->nblk[M_PT], 0, h->st));
  else KL("dt_minabs", chl_launch_minabs(h->map(M_MINABS), h->nblk[M_MINABS], 0, h->st));
  LAUNCHED();
  return CHL_OK;
}

static int enqueue_rk3(chl_handle* h) {
  // set in -> out per stage: 0 -> 1, 1 -> 2, 2 -> 0 (base is always set 0)
  const int sin[3] = {0, 1, 2}, sout[3] = {1, 2, 0};
  for (int s = 0; s < 3; ++s) {
    int rc = enqueue_sgs(h, sin[s], h->wall_model != CHL_WM_NONE, s);
    if (rc) return rc;
    KL("rhs_flux", chl_launch_flux(h->map(M_EDGE), h->nblk[M_EDGE], sin[s], h->st));
    KL("rhs_update", chl_launch_update(h->map(M_PT), h->nblk[M_PT], 0, sout[s], s, s == 0 ? 0 : 1, h->st));
    LAUNCHED();
    rc = enqueue_projection(h, sout[s], 0);
    if (rc) return rc;
  }
  if (h->any_mass) {
    KL("massflow", chl_launch_massflow(h->map(M_PT), h->st, 0, 0));
    KL("massflow_shift", chl_launch_shift(h->map(M_PT), h->nblk[M_PT], 0, h->st));   // and t += dt
  } else {
    KL("t_advance", chl_launch_tadvance(h->map(M_PT), h->st));
  }
  LAUNCHED();
  (void)RK_T;
  return CHL_OK;
}

static int check_ready(chl_handle* h) {
  if (!h) return CHL_E_ARG;
  for (auto& I : h->in) if (!I.uploaded) { h->err = "fields not uploaded"; return CHL_E_STATE; }
  return CHL_OK;
}

static int finish(chl_handle* h) {
  cudaError_t e = cudaStreamSynchronize(h->st);
  if (e == cudaSuccess && h->st_h2d) e = cudaStreamSynchronize(h->st_h2d);
  if (e == cudaSuccess && h->st_d2h) e = cudaStreamSynchronize(h->st_d2h);
  if (e != cudaSuccess) { h->err = std::string("CUDA: ") + cudaGetErrorString(e); return CHL_E_CUDA; }
  return CHL_OK;
}

// Waits for the copy streams: the synchronous entry points use the staging
// area on the compute stream only after any round-trip copy into or out of
// it has finished.
static int drain_copies(chl_handle* h) {
  cudaError_t e = cudaSuccess;
  if (h->st_h2d) e = cudaStreamSynchronize(h->st_h2d);
  if (e == cudaSuccess && h->st_d2h) e = cudaStreamSynchronize(h->st_d2h);
  if (e != cudaSuccess) { h->err = std::string("CUDA: ") + cudaGetErrorString(e); return CHL_E_CUDA; }
  return CHL_OK;
}

// Non-finite velocities: the CFL pass of every step flags them in the
// instance's status word (chl_misc.cu: k_minabs).  Checked at the calls that
// synchronise; the flag stays set until the instance is uploaded again.
// inst < 0 checks every instance (chl_synchronize); reads of one instance
// check only that one, so the others of a batch stay usable.
static int check_finite(chl_handle* h, int inst = -1) {
  for (size_t q = 0; q < h->in.size(); ++q) {
    if (inst >= 0 && (int)q != inst) continue;
    int st = 0;
    cudaError_t e = cudaMemcpy(&st, h->in[q].dev.status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { h->err = std::string("CUDA: ") + cudaGetErrorString(e); return CHL_E_CUDA; }
    if (st & CHL_STATUS_NONFINITE) {
      h->err = "non-finite velocity in instance " + std::to_string(q) + " (found by compute_dt); re-upload the fields";
      return CHL_E_NAN;
    }
  }
  return CHL_OK;
}

// The learned wall model's bounded tensor-core waits (chl_mlp.cu) set the
// handle's status word when they run out; the CTA then keeps the
// equilibrium stress for its points.  Checked at the calls that
// synchronise, reported once and cleared.
static int check_mlp(chl_handle* h) {
  if (h->wall_model != CHL_WM_MLP || !h->d_mlp_status) return CHL_OK;
  int st = 0;
  cudaError_t e = cudaMemcpy(&st, h->d_mlp_status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && st) e = cudaMemset(h->d_mlp_status, 0, sizeof(int));
  if (e != cudaSuccess) { h->err = std::string("CUDA: ") + cudaGetErrorString(e); return CHL_E_CUDA; }
  if (st) {
    h->err = "learned wall model: a tensor-core completion wait ran out; those points kept the equilibrium stress";
    return CHL_E_TIMEOUT;
  }
  return CHL_OK;
}

// ------------------------------------------------------------ C ABI
extern "C" {

int chl_grid_constants_size(const chl_grid_desc* d) {
  if (!d) return -1;
  const int Nx = d->nx - 2, Nz = d->nz - 2, nyg = d->ny + 1;
  return Nx + Nz + 3 * (nyg - 2) + d->ny + 5;
}

int chl_grid_constants(const chl_grid_desc* d, double* out) {
  if (!d || !out) return CHL_E_ARG;
  Consts c; std::string err;
  int rc = make_consts(*d, c, err);
  if (rc) return rc;
  size_t o = 0;
  for (int i = 0; i < c.Nx; ++i) out[o++] = c.kxx[i];
  for (int i = 0; i < c.Nz; ++i) out[o++] = c.kzz[i];
  for (int j = 2; j <= c.nyg - 1; ++j) out[o++] = c.Dd[j];
  for (int j = 2; j <= c.nyg - 1; ++j) out[o++] = c.Du[j];
  for (int j = 2; j <= c.nyg - 1; ++j) out[o++] = c.Dl[j];
  for (int jv = 0; jv <= c.Ny; ++jv) out[o++] = c.w0[jv];
  out[o++] = c.dxmin; out[o++] = c.dymin; out[o++] = c.dzmin; out[o++] = c.coef_bc_1; out[o++] = c.coef_bc_2;
  return CHL_OK;
}

int chl_fft_pass_table(int N, double* out, int cap) {
  if (N < 1) return -1;
  int r = N;
  while (r % 4 == 0) r /= 4;
  while (r % 3 == 0) r /= 3;
  while (r % 2 == 0) r /= 2;
  if (r != 1) return -1;
  const std::vector<double> t = fft_pass_table(N);
  if (out) {
    if (cap < (int)t.size()) return -2;
    std::copy(t.begin(), t.end(), out);
  }
  return (int)t.size();
}

int chl_batch_create(int n, const chl_grid_desc* descs, chl_handle** out) {
  if (!out || n <= 0 || !descs) return CHL_E_ARG;
  *out = nullptr;
  chl_handle* h = new chl_handle();
  h->in.resize(n);
  for (int q = 0; q < n; ++q) {
    Inst& I = h->in[q];
    I.d = descs[q];
    int rc = make_consts(I.d, I.c, h->err);
    if (rc) { *out = h; return rc; }
    if (I.d.LES_model < 0 || I.d.LES_model > 4 || I.d.wall_model < 0 || I.d.wall_model > 3) {
      h->err = "unsupported LES_model / wall_model"; *out = h; return CHL_E_ARG;
    }
    if (I.d.Dirichlet_nu_t < 0 || I.d.Dirichlet_nu_t > 2) {
      h->err = "unsupported Dirichlet_nu_t (0, 1 or 2)"; *out = h; return CHL_E_ARG;
    }
    if (q > 0 && (I.d.LES_model != h->in[0].d.LES_model || I.d.wall_model != h->in[0].d.wall_model)) {
      h->err = "instances of one batch must share LES_model and wall_model"; *out = h; return CHL_E_ARG;
    }
    if (I.d.wall_model >= CHL_WM_EQLOG && I.c.Ny < 8) { h->err = "equilibrium wall model needs Ny >= 8"; *out = h; return CHL_E_ARG; }
    if (I.d.wall_model == CHL_WM_MLP && !(I.d.Re_tau > 0.0)) { h->err = "learned wall model needs Re_tau > 0"; *out = h; return CHL_E_ARG; }
    if (I.d.x_mass_cte) h->any_mass = 1;
  }
  h->LES_model = h->in[0].d.LES_model;
  h->wall_model = h->in[0].d.wall_model;
  cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) { h->err = std::string("CUDA: ") + cudaGetErrorString(e); *out = h; return CHL_E_CUDA; }
  // learned wall model: zero network (mu = 0: the equilibrium stress), no noise, no trace
  if (cudaMalloc(&h->d_mlp_theta, sizeof(float) * MLP_NPARAM) != cudaSuccess ||
      cudaMalloc(&h->d_mlp_cfg, sizeof(unsigned int) * 8) != cudaSuccess ||
      cudaMalloc(&h->d_mlp_status, sizeof(int) * 2) != cudaSuccess) {
    h->err = "device allocation failed"; *out = h; return CHL_E_NOMEM;
  }
  cudaMemset(h->d_mlp_theta, 0, sizeof(float) * MLP_NPARAM);
  cudaMemset(h->d_mlp_cfg, 0, sizeof(unsigned int) * 8);
  cudaMemset(h->d_mlp_status, 0, sizeof(int) * 2);
  for (auto& I : h->in) { int rc = upload_consts(h, I); if (rc) { *out = h; return rc; } }
  std::vector<ChlInst> hv(n);
  for (int q = 0; q < n; ++q) hv[q] = h->in[q].dev;
  e = cudaMalloc(&h->d_inst, sizeof(ChlInst) * n);
  if (e != cudaSuccess) { h->err = "device allocation failed"; *out = h; return CHL_E_NOMEM; }
  e = cudaMemcpy(h->d_inst, hv.data(), sizeof(ChlInst) * n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { h->err = std::string("CUDA: ") + cudaGetErrorString(e); *out = h; return CHL_E_CUDA; }
  e = cudaMalloc(&h->d_divout, sizeof(double) * 2 * n);
  if (e != cudaSuccess) { h->err = "device allocation failed"; *out = h; return CHL_E_NOMEM; }
  for (auto& I : h->in) h->stats_pitch = std::max(h->stats_pitch, 7 * (I.c.Ny + 1) + 4);
  e = cudaMalloc(&h->d_stats, sizeof(double) * (size_t)h->stats_pitch * n);
  if (e != cudaSuccess) { h->err = "device allocation failed"; *out = h; return CHL_E_NOMEM; }
  int rc = build_maps(h);
  if (rc) { *out = h; return rc; }
  chl_launch_minabs_init(h->map(M_PT), h->st);   // the minima start every step at their initial value
  cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) { h->err = std::string("CUDA launch: ") + cudaGetErrorString(le); *out = h; return CHL_E_CUDA; }
  *out = h;
  return finish(h);
}

int chl_create(const chl_grid_desc* desc, chl_handle** out) { return chl_batch_create(1, desc, out); }

int chl_destroy(chl_handle* h) {
  if (!h) return CHL_OK;
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->st_h2d) cudaStreamSynchronize(h->st_h2d);   // no copy may still target the arena
  if (h->st_d2h) cudaStreamSynchronize(h->st_d2h);
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  if (h->graph) cudaGraphDestroy(h->graph);
  for (auto& I : h->in) if (I.arena) cudaFree(I.arena);
  for (int m = 0; m < NMAP; ++m) if (h->d_off[m]) cudaFree(h->d_off[m]);
  if (h->d_inst) cudaFree(h->d_inst);
  if (h->d_divout) cudaFree(h->d_divout);
  if (h->d_stats) cudaFree(h->d_stats);
  if (h->d_agent) cudaFree(h->d_agent);
  if (h->d_mlp_theta) cudaFree(h->d_mlp_theta);
  if (h->d_mlp_cfg) cudaFree(h->d_mlp_cfg);
  if (h->d_mlp_status) cudaFree(h->d_mlp_status);
  for (auto& e : h->ev) cudaEventDestroy(e);
  for (auto& I : h->in)
    for (cudaEvent_t e : {I.ev_h2d, I.ev_unpacked, I.ev_packed, I.ev_d2h}) if (e) cudaEventDestroy(e);
  if (h->st_h2d) cudaStreamDestroy(h->st_h2d);
  if (h->st_d2h) cudaStreamDestroy(h->st_d2h);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return CHL_OK;
}

const char* chl_last_error(const chl_handle* h) { return h ? h->err.c_str() : "null handle"; }
int chl_num_instances(const chl_handle* h) { return h ? (int)h->in.size() : 0; }

static Inst* get_inst(chl_handle* h, int inst) {
  if (!h || inst < 0 || inst >= (int)h->in.size()) { if (h) h->err = "instance index out of range"; return nullptr; }
  return &h->in[inst];
}

// U, V, W of velocity set 0 and their Fortran-layout slots in the staging
// area (out = false: the input half, true: the output half)
static ChlFields3 fields3(Inst* I, bool out = false) {
  const Consts& c = I->c;
  double* s = I->staging + (out ? 3 * I->nstage : 0);
  const size_t n = I->nstage;
  ChlFields3 f;
  f.f[0] = ChlField1{s, I->dev.U[0], c.nx, c.nyg, c.nzg, c.Ny + 2, 0};
  f.f[1] = ChlField1{s + n, I->dev.V[0], c.nxg, c.ny, c.nzg, c.Ny + 1, 1};
  f.f[2] = ChlField1{s + 2 * n, I->dev.W[0], c.nxg, c.nyg, c.nz, c.Ny + 2, 0};
  return f;
}

int chl_upload(chl_handle* h, int inst, const double* U, const double* V, const double* W) {
  Inst* I = get_inst(h, inst);
  if (!I) return CHL_E_ARG;
  if (!U || !V || !W) { h->err = "null field"; return CHL_E_ARG; }
  if (int rc = drain_copies(h)) return rc;
  const ChlFields3 f3 = fields3(I);
  const double* src[3] = {U, V, W};
  for (int q = 0; q < 3; ++q) {
    const ChlField1& d = f3.f[q];
    CK(cudaMemcpyAsync(d.fort, src[q], 8 * (size_t)d.n1 * d.n2 * d.n3, cudaMemcpyHostToDevice, h->st));
  }
  chl_launch_unpack3(f3, I->c.Nx, I->c.Nz, h->st);
  LAUNCHED();
  const int Nz = I->c.Nz;
  // Qflow_x_0 of this instance (mass_flow.f90:24-61); the kernel runs per instance
  chl_launch_qflow(h->d_inst + inst, Nz, 0, CHL_S_Q0, h->st);
  LAUNCHED();
  CK(cudaMemsetAsync(I->dev.status, 0, sizeof(int), h->st));
  I->uploaded = true;
  return finish(h);
}

static int download_field(chl_handle* h, Inst* I, double* dst, const double* src, int n1, int n2, int n3, int nrow,
                          double sub = 0.0) {
  if (int rc = drain_copies(h)) return rc;
  chl_launch_pack(I->staging, src, I->c.Nx, nrow, I->c.Nz, n1, n2, n3, sub, h->st);
  LAUNCHED();
  CK(cudaMemcpyAsync(dst, I->staging, 8 * (size_t)n1 * n2 * n3, cudaMemcpyDeviceToHost, h->st));
  return finish(h);
}

int chl_download(chl_handle* h, int inst, double* U, double* V, double* W, double* P, double* nu_t) {
  Inst* I = get_inst(h, inst);
  if (!I) return CHL_E_ARG;
  int rc0 = finish(h);
  if (rc0 || (rc0 = check_finite(h, inst)) || (rc0 = check_mlp(h))) return rc0;
  const Consts& c = I->c;
  const int Ny = c.Ny;
  int rc = 0;
  if (U && (rc = download_field(h, I, U, I->dev.U[0], c.nx, c.nyg, c.nzg, Ny + 2))) return rc;
  if (V && (rc = download_field(h, I, V, I->dev.V[0], c.nxg, c.ny, c.nzg, Ny + 1))) return rc;
  if (W && (rc = download_field(h, I, W, I->dev.W[0], c.nxg, c.nyg, c.nz, Ny + 2))) return rc;
  if (P && (rc = download_field(h, I, P, I->dev.P, c.nxg, c.nyg, c.nzg, Ny + 2))) return rc;
  if (nu_t && (rc = download_field(h, I, nu_t, I->dev.nut, c.nxg, c.nyg, c.nzg, Ny + 2, I->d.nu))) return rc;
  return CHL_OK;
}

int chl_save_snapshot(chl_handle* h, int inst, const char* path, int with_pressure) {
  Inst* I = get_inst(h, inst);
  if (!I || !path) return CHL_E_ARG;
  const Consts& c = I->c;
  int rc;
  if (with_pressure && (rc = chl_compute_pressure(h))) return rc;
  std::vector<double> U((size_t)c.nx * c.nyg * c.nzg), V((size_t)c.nxg * c.ny * c.nzg), W((size_t)c.nxg * c.nyg * c.nz);
  std::vector<double> P, nt;
  if (with_pressure) { P.resize((size_t)c.nxg * c.nyg * c.nzg); nt.resize(P.size()); }
  if ((rc = chl_download(h, inst, U.data(), V.data(), W.data(), with_pressure ? P.data() : nullptr,
                         with_pressure ? nt.data() : nullptr))) return rc;
  rc = chl_snapshot_write(path, c.nx, c.ny, c.nz, c.xf.data() + 1, c.yf.data() + 1, c.zf.data() + 1,
                          U.data(), V.data(), W.data(), with_pressure ? P.data() : nullptr,
                          with_pressure ? nt.data() : nullptr);
  if (rc) h->err = chl_io_last_error();
  return rc;
}

int chl_load_snapshot(chl_handle* h, int inst, const char* path) {
  Inst* I = get_inst(h, inst);
  if (!I || !path) return CHL_E_ARG;
  const Consts& c = I->c;
  std::vector<double> x(c.nx), y(c.ny), z(c.nz);
  std::vector<double> U((size_t)c.nx * c.nyg * c.nzg), V((size_t)c.nxg * c.ny * c.nzg), W((size_t)c.nxg * c.nyg * c.nz);
  int rc = chl_snapshot_read(path, c.nx, c.ny, c.nz, x.data(), y.data(), z.data(), U.data(), V.data(), W.data());
  if (rc) { h->err = chl_io_last_error(); return rc; }
  for (int i = 0; i < c.nx; ++i) if (x[i] != c.xf[i + 1]) { h->err = "snapshot: x mesh differs from the instance"; return CHL_E_ARG; }
  for (int j = 0; j < c.ny; ++j) if (y[j] != c.yf[j + 1]) { h->err = "snapshot: y mesh differs from the instance"; return CHL_E_ARG; }
  for (int k = 0; k < c.nz; ++k) if (z[k] != c.zf[k + 1]) { h->err = "snapshot: z mesh differs from the instance"; return CHL_E_ARG; }
  return chl_upload(h, inst, U.data(), V.data(), W.data());
}

int chl_download_pseudo_pressure(chl_handle* h, int inst, double* p) {
  Inst* I = get_inst(h, inst);
  if (!I || !p) return CHL_E_ARG;
  const Consts& c = I->c;
  return download_field(h, I, p, I->dev.p, c.nxg, c.nyg, c.nzg, c.Ny + 2);
}

int chl_set_wall_stress(chl_handle* h, int inst, const double* a) {
  Inst* I = get_inst(h, inst);
  if (!I || !a) return CHL_E_ARG;
  const Consts& c = I->c;
  std::vector<double> al(2 * (size_t)c.Nx * c.Nz);
  for (int w = 0; w < 2; ++w)
    for (int k = 0; k < c.Nz; ++k)
      for (int i = 0; i < c.Nx; ++i)   // alpha_x(i+2, w+1, k+2)
        al[((size_t)w * c.Nz + k) * c.Nx + i] = a[(size_t)(i + 1) + (size_t)c.nx * ((size_t)w + 2 * (size_t)(k + 1))];
  CK(cudaMemcpyAsync(I->dev.alpha, al.data(), 8 * al.size(), cudaMemcpyHostToDevice, h->st));
  return finish(h);
}

int chl_get_wall_stress(chl_handle* h, int inst, double* a) {
  Inst* I = get_inst(h, inst);
  if (!I || !a) return CHL_E_ARG;
  const Consts& c = I->c;
  std::vector<double> al(2 * (size_t)c.Nx * c.Nz);
  CK(cudaMemcpyAsync(al.data(), I->dev.alpha, 8 * al.size(), cudaMemcpyDeviceToHost, h->st));
  int rc = finish(h);
  if (rc) return rc;
  for (int k1 = 0; k1 < c.nzg; ++k1)
    for (int w = 0; w < 2; ++w)
      for (int i1 = 0; i1 < c.nx; ++i1) {
        int i = (i1 - 1) % c.Nx; if (i < 0) i += c.Nx;
        int k = (k1 - 1) % c.Nz; if (k < 0) k += c.Nz;
        a[(size_t)i1 + (size_t)c.nx * ((size_t)w + 2 * (size_t)k1)] = al[((size_t)w * c.Nz + k) * c.Nx + i];
      }
  return CHL_OK;
}

// ------------------------------------------------------------ wall agents (smarties_stat.f90:24-260)
static int agent_check(chl_handle* h, Inst* I, int nagents) {
  if (nagents < 1 || I->c.Nx % nagents) { h->err = "agents: nagents must divide Nx = nx-2"; return CHL_E_ARG; }
  if (I->c.Ny < 8) { h->err = "agents: Ny >= 8 needed"; return CHL_E_ARG; }
  return CHL_OK;
}

int chl_agent_observe(chl_handle* h, int inst, int nagents, const int* y_ind, const double* y_rand,
                      double* states, double* rewards) {
  Inst* I = get_inst(h, inst);
  if (!I || !y_ind || !y_rand || !states || !rewards) return CHL_E_ARG;
  int rc = agent_check(h, I, nagents); if (rc) return rc;
  const int n = 2 * nagents;
  for (int t = 0; t < n; ++t)
    if ((y_ind[t] != 3 && y_ind[t] != 4) || !(y_rand[t] >= 0.0 && y_rand[t] <= 1.0)) {
      h->err = "agents: y_ind must be 3 or 4 and y_rand in [0, 1]"; return CHL_E_ARG;
    }
  // buffer: y_rand[n], states[6n], rewards[n], y_ind[n] (as int)
  const size_t need = (size_t)8 * n + 8 * (size_t)n * 6 + 8 * (size_t)n + 4 * (size_t)n;
  if (need > h->agent_cap) {
    if (h->d_agent) { cudaFree(h->d_agent); h->d_agent = nullptr; h->agent_cap = 0; }
    CK(cudaMalloc(&h->d_agent, need));
    h->agent_cap = need;
  }
  double* d_r = h->d_agent;
  double* d_s = d_r + n;
  double* d_w = d_s + 6 * (size_t)n;
  int* d_y = reinterpret_cast<int*>(d_w + n);
  CK(cudaMemcpyAsync(d_r, y_rand, 8 * (size_t)n, cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(d_y, y_ind, 4 * (size_t)n, cudaMemcpyHostToDevice, h->st));
  chl_launch_agent_obs(h->d_inst + inst, nagents, I->c.Nx / nagents, I->d.dPdx, d_y, d_r, d_s, d_w, h->st);
  LAUNCHED();
  CK(cudaMemcpyAsync(states, d_s, 8 * 6 * (size_t)n, cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(rewards, d_w, 8 * (size_t)n, cudaMemcpyDeviceToHost, h->st));
  return finish(h);
}

int chl_agent_act(chl_handle* h, int inst, int nagents, const double* action) {
  Inst* I = get_inst(h, inst);
  if (!I || !action) return CHL_E_ARG;
  int rc = agent_check(h, I, nagents); if (rc) return rc;
  const Consts& c = I->c;
  const int Nx = c.Nx, Nz = c.Nz, nxa = Nx / nagents;
  std::vector<double> al(2 * (size_t)Nx * Nz);
  CK(cudaMemcpyAsync(al.data(), I->dev.alpha, 8 * al.size(), cudaMemcpyDeviceToHost, h->st));
  if ((rc = finish(h))) return rc;
  // actions(iwall,na) = alpha_x((na-1)*nx_nagents+2, iwall, 2) * action
  std::vector<double> act(2 * (size_t)nagents);
  for (int w = 0; w < 2; ++w)
    for (int na = 0; na < nagents; ++na)
      act[(size_t)w * nagents + na] = al[(size_t)w * Nz * Nx + (size_t)na * nxa] * action[(size_t)w * nagents + na];
  // linear in x between neighbouring agents, the last one towards the first;
  // then the z "interpolation" between planes 2 and nzg, which hold the same value
  for (int w = 0; w < 2; ++w)
    for (int na = 0; na < nagents; ++na) {
      const double a0 = act[(size_t)w * nagents + na], a1 = act[(size_t)w * nagents + (na + 1) % nagents];
      for (int j = 1; j <= nxa; ++j) {
        const double ax = (a0 * (double)(nxa - j + 1)) / (double)nxa + (a1 * (double)(j - 1)) / (double)nxa;
        const int i = na * nxa + (j - 1);
        for (int k = 0; k < Nz; ++k)
          al[((size_t)w * Nz + k) * Nx + i] = (ax * (double)(Nz - k)) / (double)Nz + (ax * (double)k) / (double)Nz;
      }
    }
  CK(cudaMemcpyAsync(I->dev.alpha, al.data(), 8 * al.size(), cudaMemcpyHostToDevice, h->st));
  return finish(h);
}

int chl_status_flags(chl_handle* h, int inst, int* flags) {
  Inst* I = get_inst(h, inst);
  if (!I || !flags) return CHL_E_ARG;
  int rc = finish(h); if (rc) return rc;
  CK(cudaMemcpy(flags, I->dev.status, sizeof(int), cudaMemcpyDeviceToHost));
  return CHL_OK;
}

int chl_get_scalars(chl_handle* h, int inst, double* out4) {
  Inst* I = get_inst(h, inst);
  if (!I || !out4) return CHL_E_ARG;
  double s[CHL_S_NSCAL];
  CK(cudaMemcpyAsync(s, I->dev.scal, sizeof(s), cudaMemcpyDeviceToHost, h->st));
  int rc = finish(h);
  if (rc) return rc;
  out4[0] = s[CHL_S_DT]; out4[1] = s[CHL_S_T]; out4[2] = s[CHL_S_DPDX]; out4[3] = s[CHL_S_Q0];
  return CHL_OK;
}

int chl_set_scalars(chl_handle* h, int inst, const double* in4) {
  Inst* I = get_inst(h, inst);
  if (!I || !in4) return CHL_E_ARG;
  double s[CHL_S_NSCAL];
  CK(cudaMemcpyAsync(s, I->dev.scal, sizeof(s), cudaMemcpyDeviceToHost, h->st));
  int rc = finish(h);
  if (rc) return rc;
  chl_put_dt(s, in4[0]); s[CHL_S_T] = in4[1]; s[CHL_S_DPDX] = in4[2]; s[CHL_S_Q0] = in4[3];
  CK(cudaMemcpyAsync(I->dev.scal, s, sizeof(s), cudaMemcpyHostToDevice, h->st));
  return finish(h);
}

int chl_compute_dt(chl_handle* h) {
  int rc = check_ready(h); if (rc) return rc;
  rc = enqueue_dt(h); if (rc) return rc;
  return finish(h);
}

int chl_compute_time_step_RK3(chl_handle* h) {
  int rc = check_ready(h); if (rc) return rc;
  rc = enqueue_rk3(h); if (rc) return rc;
  return finish(h);
}

int chl_rk3_step(chl_handle* h, int nsteps) {
  int rc = check_ready(h); if (rc) return rc;
  if (nsteps < 0) { h->err = "nsteps < 0"; return CHL_E_ARG; }
  if (!h->gexec) {
    CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    rc = enqueue_dt(h);
    if (!rc) rc = enqueue_rk3(h);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(h->st, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) { h->err = std::string("graph capture: ") + cudaGetErrorString(e); return CHL_E_CUDA; }
    h->graph = g;
    CK(cudaGraphInstantiate(&h->gexec, g, 0));
  }
  for (int s = 0; s < nsteps; ++s) CK(cudaGraphLaunch(h->gexec, h->st));
  return CHL_OK;
}

// ------------------------------------------------------------ tile-shape tuner
// Candidate tile shapes are timed one group at a time, keeping the fastest:
//   the block size of the one-thread-per-point kernels, timed on the eddy
//     viscosity (without the wall-model rows), the face fluxes and the RHS
//     divergence in its actual-pressure mode;
//   the x-transform and z-transform block targets and the tridiagonal form,
//     timed on the projection's transforms and solve without the velocity
//     correction;
// all on velocity set 0.  Every candidate partitions the same independent
// points, rows, columns and modes differently and leaves each one's
// arithmetic unchanged, so tuning never changes a result.  The timed kernels
// write only scratch that every step recomputes; the two arrays a caller can
// read before stepping (nu + nu_t and the pseudo-pressure) are saved and
// restored.  The step graph is rebuilt on the next step.
static int enqueue_stencils(chl_handle* h) {
  int rc = enqueue_sgs(h, 0, false);
  if (rc) return rc;
  chl_launch_flux(h->map(M_EDGE), h->nblk[M_EDGE], 0, h->st);
  chl_launch_update(h->map(M_PT), h->nblk[M_PT], 0, 0, 0, 2, h->st);
  LAUNCHED();
  return CHL_OK;
}

// events a, b: created by the caller, which also destroys them
static int time_group(chl_handle* h, int group, int reps, cudaEvent_t a, cudaEvent_t b, double* ms) {
  int rc = build_maps(h);
  if (rc) return rc;
  auto run = [&]() { return group == 0 ? enqueue_stencils(h) : enqueue_projection(h, 0, 2); };
  double best = 1e30;
  for (int trial = 0; trial < 3; ++trial) {           // best of three trials
    if ((rc = run())) return rc;                      // warm (and first-touch) outside the timing
    CK(cudaEventRecord(a, h->st));
    for (int r = 0; r < reps && !rc; ++r) rc = run();
    if (rc) return rc;
    CK(cudaEventRecord(b, h->st));
    CK(cudaEventSynchronize(b));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, a, b));
    best = std::min(best, (double)f / reps);
  }
  *ms = best;
  return CHL_OK;
}

int chl_autotune(chl_handle* h, int reps, char* report, int report_len) {
  int rc = check_ready(h); if (rc) return rc;
  if (reps < 1) reps = 1;
  // nu + nu_t, the pseudo-pressure, S (the strain or model nu_t that
  // chl_compute_wall_model rebuilds nu_t from) and the row coefficients of
  // every instance, restored at the end
  std::vector<double*> saved;
  cudaEvent_t ea = nullptr, eb = nullptr;
  auto ncent = [](const Inst& I) { return (size_t)I.c.Nx * (I.c.Ny + 2) * I.c.Nz; };   // centre-field length
  auto ncoef = [](const Inst& I) { return (size_t)I.c.Ny + 2; };
  // puts back what was saved (every instance saved so far), frees the copies and events
  auto restore = [&]() {
    for (size_t q = 0; q < saved.size(); ++q) {
      const Inst& I = h->in[q];
      const size_t n = ncent(I);
      cudaMemcpyAsync(I.dev.nut, saved[q], 8 * n, cudaMemcpyDeviceToDevice, h->st);
      cudaMemcpyAsync(I.dev.p, saved[q] + n, 8 * n, cudaMemcpyDeviceToDevice, h->st);
      cudaMemcpyAsync(I.dev.S, saved[q] + 2 * n, 8 * n, cudaMemcpyDeviceToDevice, h->st);
      cudaMemcpyAsync(I.dev.coef, saved[q] + 3 * n, 8 * ncoef(I), cudaMemcpyDeviceToDevice, h->st);
    }
    cudaStreamSynchronize(h->st);
    for (double* s : saved) cudaFree(s);
    saved.clear();
    if (ea) cudaEventDestroy(ea);
    if (eb) cudaEventDestroy(eb);
  };
  for (auto& I : h->in) {
    const size_t n = ncent(I);
    double* s = nullptr;
    cudaError_t e = cudaMalloc(&s, 8 * (3 * n + ncoef(I)));
    if (e == cudaSuccess) {
      e = cudaMemcpyAsync(s, I.dev.nut, 8 * n, cudaMemcpyDeviceToDevice, h->st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(s + n, I.dev.p, 8 * n, cudaMemcpyDeviceToDevice, h->st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(s + 2 * n, I.dev.S, 8 * n, cudaMemcpyDeviceToDevice, h->st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(s + 3 * n, I.dev.coef, 8 * ncoef(I), cudaMemcpyDeviceToDevice, h->st);
      if (e != cudaSuccess) cudaFree(s);
      else saved.push_back(s);
    }
    if (e != cudaSuccess) {
      restore();
      h->err = std::string("CUDA: ") + cudaGetErrorString(e) + " saving state for the tuner";
      return CHL_E_CUDA;
    }
  }
  {
    cudaError_t e = cudaEventCreate(&ea);
    if (e == cudaSuccess) e = cudaEventCreate(&eb);
    if (e != cudaSuccess) {
      restore();
      h->err = std::string("CUDA: ") + cudaGetErrorString(e);
      return CHL_E_CUDA;
    }
  }
  rc = [&]() -> int {
  static const int targets[] = {1, CHL_SMS, 2 * CHL_SMS, 4 * CHL_SMS, 8 * CHL_SMS, 16 * CHL_SMS};
  std::string rep;
  char buf[160];
  double t = 0.0, t0 = 0.0;
  int rc2 = time_group(h, 0, reps, ea, eb, &t0);
  if (!rc2) rc2 = time_group(h, 1, reps, ea, eb, &t);
  if (rc2) return rc2;
  std::snprintf(buf, sizeof buf, "defaults: stencils %.4f ms, projection %.4f ms;", t0, t);
  rep += buf;
  // point-kernel block size
  {
    int best_v = h->tb_pt;
    double best_t = 1e30;
    for (int v : {64, 128, 256}) {
      h->tb_pt = v;
      if ((rc2 = time_group(h, 0, reps, ea, eb, &t))) return rc2;
      if (t < best_t) { best_t = t; best_v = v; }
    }
    h->tb_pt = best_v;
    std::snprintf(buf, sizeof buf, " point_threads %d (%.4f ms);", best_v, best_t);
    rep += buf;
  }
  // x transform, then z transform: block-count targets
  for (int g = 0; g < 2; ++g) {
    int& knob = g == 0 ? h->x_min_blocks : h->z_min_blocks;
    int best_v = knob;
    double best_t = 1e30;
    for (int v : targets) {
      knob = v;
      if ((rc2 = time_group(h, 1, reps, ea, eb, &t))) return rc2;
      if (t < best_t) { best_t = t; best_v = v; }
    }
    knob = best_v;
    std::snprintf(buf, sizeof buf, " %s_min_blocks %d (%.4f ms);", g == 0 ? "x" : "z", best_v, best_t);
    rep += buf;
  }
  // tridiagonal: row-batched, or staged in shared memory where it fits
  {
    int my = 0;
    long modes = 0;
    for (auto& I : h->in) { my = std::max(my, I.c.Ny); modes += (long)I.c.Nz * I.c.Nxh; }
    const bool fits = !h->tri_scan && chl_smem_tri(my, modes, 1) > 0;
    const bool fused = h->zsolve_ok;
    int best_v = 0;
    double best_t = 1e30;
    for (int v = 0; v <= 3; ++v) {
      if ((v == 1 && !fits) || v == 2 || (v == 3 && !fused)) continue;
      h->tri_mode = v;
      if ((rc2 = time_group(h, 1, reps, ea, eb, &t))) return rc2;
      if (t < best_t) { best_t = t; best_v = v; }
    }
    h->tri_mode = best_v;
    std::snprintf(buf, sizeof buf, " tridiag %s (%.4f ms)",
                  best_v == 3 ? "fused z solve" : (h->tri_scan ? "lane-split" : (best_v == 1 ? "staged" : "row-batched")),
                  best_t);
    rep += buf;
  }
  if ((rc2 = build_maps(h))) return rc2;
  if (report && report_len > 0) {
    std::strncpy(report, rep.c_str(), (size_t)report_len - 1);
    report[report_len - 1] = 0;
  }
  return CHL_OK;
  }();
  restore();
  if (h->gexec) { cudaGraphExecDestroy(h->gexec); h->gexec = nullptr; }
  if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
  return rc ? rc : finish(h);
}

int chl_get_tile_shapes(chl_handle* h, int* out7) {
  if (!h || !out7) return CHL_E_ARG;
  out7[0] = h->x_min_blocks; out7[1] = h->z_min_blocks; out7[2] = h->tri_mode; out7[3] = h->tb_pt;
  out7[4] = h->zcw; out7[5] = h->zsolve ? 3 : (h->tri_scan ? 2 : (h->smem_t ? 1 : 0)); out7[6] = h->tx;
  return CHL_OK;
}

int chl_set_tile_shapes(chl_handle* h, int x_min_blocks, int z_min_blocks, int tri_mode, int point_threads) {
  if (!h || x_min_blocks < 1 || z_min_blocks < 1 || tri_mode < 0 || tri_mode > 3) return CHL_E_ARG;
  if (point_threads != 64 && point_threads != 128 && point_threads != 256) return CHL_E_ARG;
  h->x_min_blocks = x_min_blocks; h->z_min_blocks = z_min_blocks; h->tri_mode = tri_mode;
  h->tb_pt = point_threads;
  int rc = build_maps(h);
  if (rc) return rc;
  if (h->gexec) { cudaGraphExecDestroy(h->gexec); h->gexec = nullptr; }
  if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
  return CHL_OK;
}

int chl_device_reset(void) {
  return cudaDeviceReset() == cudaSuccess ? CHL_OK : CHL_E_CUDA;
}

int chl_synchronize(chl_handle* h) {
  if (!h) return CHL_E_ARG;
  int rc = finish(h);
  if (!rc) rc = check_finite(h);
  return rc ? rc : check_mlp(h);
}

int chl_compute_eddy_viscosity(chl_handle* h) {
  int rc = check_ready(h); if (rc) return rc;
  rc = enqueue_sgs(h, 0, false); if (rc) return rc;
  return finish(h);
}

int chl_compute_wall_model(chl_handle* h) {
  int rc = check_ready(h); if (rc) return rc;
  if (h->wall_model >= CHL_WM_EQLOG) chl_launch_eqwm(h->map(M_WALLN), h->nblk[M_WALLN], 0, h->st);
  if (h->wall_model == CHL_WM_MLP) chl_launch_mlp(h->map(M_MLP), h->nblk[M_MLP], 0, 0, h->d_mlp_status, h->st);
  chl_launch_nut(h->map(M_FULL), h->nblk[M_FULL], 0, h->wall_model != CHL_WM_NONE ? 1 : 0, h->st);
  LAUNCHED();
  return finish(h);
}

int chl_compute_rhs(chl_handle* h, int inst, double* Fu, double* Fv, double* Fw) {
  int rc = check_ready(h); if (rc) return rc;
  Inst* I = get_inst(h, inst);
  if (!I) return CHL_E_ARG;
  if ((rc = drain_copies(h))) return rc;
  chl_launch_flux(h->map(M_EDGE), h->nblk[M_EDGE], 0, h->st);
  chl_launch_update(h->map(M_PT), h->nblk[M_PT], 0, 0, 0, 2, h->st);
  LAUNCHED();
  const Consts& c = I->c;
  const int Nx = c.Nx, Ny = c.Ny, Nz = c.Nz;
  struct { double* dst; const double* src; int nrow, jlo, nj; } f[3] = {
      {Fu, I->dev.Fp[0], Ny + 2, 1, Ny}, {Fv, I->dev.Fp[1], Ny + 1, 1, Ny - 1}, {Fw, I->dev.Fp[2], Ny + 2, 1, Ny}};
  for (auto& q : f) {
    if (!q.dst) continue;
    chl_launch_pack_unique(I->staging, q.src, Nx, q.nrow, Nz, q.jlo, q.nj, h->st);
    LAUNCHED();
    CK(cudaMemcpyAsync(q.dst, I->staging, 8 * (size_t)Nx * q.nj * Nz, cudaMemcpyDeviceToHost, h->st));
  }
  return finish(h);
}

int chl_compute_projection_step(chl_handle* h) {
  int rc = check_ready(h); if (rc) return rc;
  rc = enqueue_projection(h, 0, 0); if (rc) return rc;
  return finish(h);
}

int chl_compute_dPx_for_constant_mass_flow(chl_handle* h, int inst, double* dPdx) {
  int rc = check_ready(h); if (rc) return rc;
  Inst* I = get_inst(h, inst);
  if (!I || !dPdx) return CHL_E_ARG;
  double s[CHL_S_NSCAL];
  CK(cudaMemcpyAsync(s, I->dev.scal, sizeof(s), cudaMemcpyDeviceToHost, h->st));
  if ((rc = finish(h))) return rc;
  chl_launch_massflow(h->map(M_PT), h->st, 0, 1);
  LAUNCHED();
  double s2[CHL_S_NSCAL];
  CK(cudaMemcpyAsync(s2, I->dev.scal, sizeof(s2), cudaMemcpyDeviceToHost, h->st));
  if ((rc = finish(h))) return rc;
  *dPdx = s2[CHL_S_SHIFT];
  // this entry point only reports dPdx: restore the imposed gradient
  CK(cudaMemcpyAsync(I->dev.scal, s, sizeof(s), cudaMemcpyHostToDevice, h->st));
  return finish(h);
}

int chl_compute_pressure(chl_handle* h) {
  int rc = check_ready(h); if (rc) return rc;
  chl_launch_pbc(h->map(M_WALL), h->nblk[M_WALL], 0, h->st);
  chl_launch_flux(h->map(M_EDGE), h->nblk[M_EDGE], 0, h->st);
  chl_launch_update(h->map(M_PT), h->nblk[M_PT], 0, 0, 0, 2, h->st);
  LAUNCHED();
  rc = enqueue_projection(h, 0, 1); if (rc) return rc;
  chl_launch_pghost(h->map(M_PLANE), h->nblk[M_PLANE], h->st);
  LAUNCHED();
  return finish(h);
}

int chl_check_divergence(chl_handle* h, int inst, double* max_div, double* max_abs_div) {
  int rc = check_ready(h); if (rc) return rc;
  if (!get_inst(h, inst)) return CHL_E_ARG;
  chl_launch_divmax(h->map(M_ZPLANE), h->nblk[M_ZPLANE], 0, h->d_divout, h->st);
  LAUNCHED();
  double r[2];
  CK(cudaMemcpyAsync(r, h->d_divout + 2 * inst, sizeof(r), cudaMemcpyDeviceToHost, h->st));
  if ((rc = finish(h))) return rc;
  if (max_div) *max_div = r[0];
  if (max_abs_div) *max_abs_div = r[1];
  return CHL_OK;
}

// The copy streams and the instance's ordering events, on first use.
static int round_trip_setup(chl_handle* h, Inst* I) {
  if (!h->st_h2d) CK(cudaStreamCreateWithFlags(&h->st_h2d, cudaStreamNonBlocking));
  if (!h->st_d2h) CK(cudaStreamCreateWithFlags(&h->st_d2h, cudaStreamNonBlocking));
  cudaEvent_t* ev[4] = {&I->ev_h2d, &I->ev_unpacked, &I->ev_packed, &I->ev_d2h};
  for (cudaEvent_t* e : ev)
    if (!*e) CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  return CHL_OK;
}

// Host-buffer round trip.  The input half of the staging area receives the
// three copies on the H2D stream, once the previous conversion out of it on
// the compute stream is done; the compute stream converts them into
// velocity set 0 once they have arrived.  The output half is filled on the
// compute stream, once the previous download out of it is done, and copied
// to the host on the D2H stream.  So with calls in the order set_fields,
// step, download_async for step after step, step n+1's upload and step
// n-1's download run on the copy engines while step n computes; each step
// still copies its own inputs in and its own result out.
int chl_set_fields(chl_handle* h, int inst, const double* U, const double* V, const double* W) {
  Inst* I = get_inst(h, inst);
  if (!I) return CHL_E_ARG;
  if (!I->uploaded) { h->err = "chl_set_fields before chl_upload"; return CHL_E_STATE; }
  if (!U || !V || !W) { h->err = "null field"; return CHL_E_ARG; }
  if (int rc = round_trip_setup(h, I)) return rc;
  const ChlFields3 f3 = fields3(I, false);
  const double* src[3] = {U, V, W};
  CK(cudaStreamWaitEvent(h->st_h2d, I->ev_unpacked, 0));
  for (int q = 0; q < 3; ++q) {
    const ChlField1& d = f3.f[q];
    CK(cudaMemcpyAsync(d.fort, src[q], 8 * (size_t)d.n1 * d.n2 * d.n3, cudaMemcpyHostToDevice, h->st_h2d));
  }
  CK(cudaEventRecord(I->ev_h2d, h->st_h2d));
  CK(cudaStreamWaitEvent(h->st, I->ev_h2d, 0));
  chl_launch_unpack3(f3, I->c.Nx, I->c.Nz, h->st);
  LAUNCHED();
  CK(cudaEventRecord(I->ev_unpacked, h->st));
  CK(cudaMemsetAsync(I->dev.status, 0, sizeof(int), h->st));
  return CHL_OK;   // stream-ordered; no synchronisation
}

int chl_download_async(chl_handle* h, int inst, double* U, double* V, double* W) {
  Inst* I = get_inst(h, inst);
  if (!I) return CHL_E_ARG;
  if (int rc = round_trip_setup(h, I)) return rc;
  const ChlFields3 f3 = fields3(I, true);
  double* dst[3] = {U, V, W};
  CK(cudaStreamWaitEvent(h->st, I->ev_d2h, 0));
  chl_launch_pack3(f3, I->c.Nx, I->c.Nz, h->st);
  LAUNCHED();
  CK(cudaEventRecord(I->ev_packed, h->st));
  CK(cudaStreamWaitEvent(h->st_d2h, I->ev_packed, 0));
  for (int q = 0; q < 3; ++q) {
    if (!dst[q]) continue;
    const ChlField1& d = f3.f[q];
    CK(cudaMemcpyAsync(dst[q], d.fort, 8 * (size_t)d.n1 * d.n2 * d.n3, cudaMemcpyDeviceToHost, h->st_d2h));
  }
  CK(cudaEventRecord(I->ev_d2h, h->st_d2h));
  return CHL_OK;
}

int chl_time_steps(chl_handle* h, int nsteps, double* ms) {
  if (!ms) return CHL_E_ARG;
  int rc = check_ready(h); if (rc) return rc;
  if (!h->gexec) { if ((rc = chl_rk3_step(h, 0))) return rc; }
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a)); CK(cudaEventCreate(&b));
  CK(cudaStreamSynchronize(h->st));
  CK(cudaEventRecord(a, h->st));
  for (int s = 0; s < nsteps; ++s) CK(cudaGraphLaunch(h->gexec, h->st));
  CK(cudaEventRecord(b, h->st));
  CK(cudaEventSynchronize(b));
  float f = 0.f;
  CK(cudaEventElapsedTime(&f, a, b));
  cudaEventDestroy(a); cudaEventDestroy(b);
  *ms = f;
  return CHL_OK;
}

int chl_graph_kernel_count(chl_handle* h, int* count) {
  if (!h || !count) return CHL_E_ARG;
  int rc = check_ready(h); if (rc) return rc;
  if (!h->gexec) { if ((rc = chl_rk3_step(h, 0))) return rc; }
  size_t n = 0;
  CK(cudaGraphGetNodes(h->graph, nullptr, &n));
  std::vector<cudaGraphNode_t> nodes(n);
  CK(cudaGraphGetNodes(h->graph, nodes.data(), &n));
  int k = 0;
  for (auto& nd : nodes) { cudaGraphNodeType t; CK(cudaGraphNodeGetType(nd, &t)); if (t == cudaGraphNodeTypeKernel) ++k; }
  *count = k;
  return CHL_OK;
}

int chl_profile_step(chl_handle* h, int reps, int maxk, char* names, double* ms_per_step, int* launches_per_step) {
  if (!h || reps <= 0 || maxk <= 0 || !names || !ms_per_step || !launches_per_step) return CHL_E_ARG;
  int rc = check_ready(h); if (rc) return rc;
  if (h->ev.empty()) {
    h->ev.resize(512);
    for (auto& e : h->ev) CK(cudaEventCreate(&e));
  }
  std::vector<std::string> keys; std::vector<double> tot; std::vector<int> cnt;
  for (int r = 0; r < reps; ++r) {
    h->rec.clear();
    h->prof = true;
    rc = enqueue_dt(h);
    if (!rc) rc = enqueue_rk3(h);
    h->prof = false;
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->st));
    for (auto& q : h->rec) {
      float f = 0.f;
      CK(cudaEventElapsedTime(&f, h->ev[q.ev], h->ev[q.ev + 1]));
      size_t i = 0;
      for (; i < keys.size(); ++i) if (keys[i] == q.name) break;
      if (i == keys.size()) { keys.push_back(q.name); tot.push_back(0.0); cnt.push_back(0); }
      tot[i] += f; if (r == 0) cnt[i] += 1;
    }
  }
  const int nk = std::min((int)keys.size(), maxk);
  for (int i = 0; i < nk; ++i) {
    std::strncpy(names + 32 * i, keys[i].c_str(), 31); names[32 * i + 31] = 0;
    ms_per_step[i] = tot[i] / reps;
    launches_per_step[i] = cnt[i];
  }
  return nk;
}

// ------------------------------------------------------------ learned wall model
int chl_mlp_set_params(chl_handle* h, const float* theta) {
  if (!h || !theta) return CHL_E_ARG;
  CK(cudaMemcpyAsync(h->d_mlp_theta, theta, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice, h->st));
  return finish(h);
}

int chl_mlp_get_params(chl_handle* h, float* theta) {
  if (!h || !theta) return CHL_E_ARG;
  CK(cudaMemcpyAsync(theta, h->d_mlp_theta, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, h->st));
  return finish(h);
}

int chl_mlp_configure(chl_handle* h, float sigma, unsigned long long seed, int train) {
  if (!h || !(sigma >= 0.0f)) { if (h) h->err = "sigma must be >= 0"; return CHL_E_ARG; }
  unsigned int c[4];
  std::memcpy(&c[0], &sigma, 4);
  c[1] = train ? 1u : 0u;
  c[2] = (unsigned int)(seed & 0xFFFFFFFFu);
  c[3] = (unsigned int)(seed >> 32);
  CK(cudaMemcpyAsync(h->d_mlp_cfg, c, sizeof(c), cudaMemcpyHostToDevice, h->st));   // counter [4] kept
  return finish(h);
}

int chl_mlp_read_trace(chl_handle* h, int inst, float* trace, int zero_after) {
  Inst* I = get_inst(h, inst);
  if (!I || !trace) return CHL_E_ARG;
  CK(cudaMemcpyAsync(trace, I->dev.mlp_trace, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, h->st));
  if (zero_after) CK(cudaMemsetAsync(I->dev.mlp_trace, 0, sizeof(float) * MLP_NPARAM, h->st));
  int rc = finish(h);
  if (rc) return rc;
  return check_mlp(h);
}

int chl_mlp_set_exploration(chl_handle* h, int shared) {
  if (!h) return CHL_E_ARG;
  const unsigned int c = shared ? 1u : 0u;
  CK(cudaMemcpyAsync(h->d_mlp_cfg + 7, &c, sizeof(c), cudaMemcpyHostToDevice, h->st));
  return finish(h);
}

int chl_mlp_debug(chl_handle* h, int record, int withhold_polls) {
  if (!h) return CHL_E_ARG;
  if (withhold_polls < 0 || withhold_polls > 64) { h->err = "withhold_polls must be in [0, 64]"; return CHL_E_ARG; }
  if (record && h->wall_model != CHL_WM_MLP) { h->err = "record: the instances have no learned wall model"; return CHL_E_ARG; }
  const unsigned int c[2] = {record ? 1u : 0u, (unsigned int)withhold_polls};
  CK(cudaMemcpyAsync(h->d_mlp_cfg + 5, c, sizeof(c), cudaMemcpyHostToDevice, h->st));
  return finish(h);
}

int chl_mlp_read_record(chl_handle* h, int inst, float* rec) {
  Inst* I = get_inst(h, inst);
  if (!I || !rec) return CHL_E_ARG;
  if (!I->dev.mlp_rec) { h->err = "no learned wall model in this instance"; return CHL_E_ARG; }
  const size_t n = (size_t)CHL_MLP_REC * 3 * 2 * I->c.Nx * I->c.Nz;
  CK(cudaMemcpyAsync(rec, I->dev.mlp_rec, sizeof(float) * n, cudaMemcpyDeviceToHost, h->st));
  return finish(h);
}

int chl_mlp_eval(chl_handle* h, const float* x, const float* g, int P, float* mu, float* trace) {
  if (!h || !x || !g || !mu || !trace || P <= 0) return CHL_E_ARG;
  float *dx = nullptr, *dg = nullptr, *dmu = nullptr, *dtr = nullptr;
  int rc = CHL_OK;
  if (cudaMalloc(&dx, sizeof(float) * 4 * P) != cudaSuccess || cudaMalloc(&dg, sizeof(float) * P) != cudaSuccess ||
      cudaMalloc(&dmu, sizeof(float) * P) != cudaSuccess || cudaMalloc(&dtr, sizeof(float) * MLP_NPARAM) != cudaSuccess) {
    h->err = "device allocation failed"; rc = CHL_E_NOMEM;
  }
  int st = 0;
  if (!rc) {
    cudaMemcpyAsync(dx, x, sizeof(float) * 4 * P, cudaMemcpyHostToDevice, h->st);
    cudaMemcpyAsync(dg, g, sizeof(float) * P, cudaMemcpyHostToDevice, h->st);
    cudaMemsetAsync(dtr, 0, sizeof(float) * MLP_NPARAM, h->st);
    cudaMemsetAsync(h->d_mlp_status, 0, sizeof(int), h->st);
    chl_launch_mlp_test(h->d_mlp_theta, dx, dg, P, dmu, dtr, h->d_mlp_status, h->st);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(mu, dmu, sizeof(float) * P, cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(trace, dtr, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, h->d_mlp_status, sizeof(int), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess) { h->err = std::string("CUDA: ") + cudaGetErrorString(e); rc = CHL_E_CUDA; }
    else if (st) {
      h->err = "wall-model network: tensor-core wait timed out";
      rc = CHL_E_TIMEOUT;
      cudaMemset(h->d_mlp_status, 0, sizeof(int));   // reported here, not again by a later call
    }
  }
  cudaFree(dx); cudaFree(dg); cudaFree(dmu); cudaFree(dtr);
  return rc;
}

int chl_tc_selftest(const unsigned short* A, const unsigned short* B, float* D, int variant) {
  if (!A || !B || !D || variant < 0 || variant > 2) return CHL_E_ARG;
  void *dA = nullptr, *dB = nullptr; float* dD = nullptr; int* ds = nullptr;
  int rc = CHL_OK;
  if (cudaMalloc(&dA, 2 * 128 * 64) != cudaSuccess || cudaMalloc(&dB, 2 * 64 * 64) != cudaSuccess ||
      cudaMalloc(&dD, 4 * 128 * 64) != cudaSuccess || cudaMalloc(&ds, sizeof(int)) != cudaSuccess) rc = CHL_E_NOMEM;
  if (!rc) {
    cudaMemcpy(dA, A, 2 * 128 * 64, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, B, 2 * 64 * 64, cudaMemcpyHostToDevice);
    cudaMemset(dD, 0, 4 * 128 * 64);
    cudaMemset(ds, 0, sizeof(int));
    if (chl_tc_selftest_launch(dA, dB, dD, variant, ds, 0)) rc = CHL_E_CUDA;
    cudaError_t e = cudaDeviceSynchronize();
    int st = 0;
    if (e == cudaSuccess) e = cudaMemcpy(D, dD, 4 * 128 * 64, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&st, ds, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = CHL_E_CUDA;
    else if (st) rc = CHL_E_TIMEOUT;
  }
  cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(ds);
  return rc;
}

int chl_sqrt_selftest(const double* a, double* y, long n) {
  if (!a || !y || n < 0 || n > (1L << 26)) return CHL_E_ARG;
  if (n == 0) return CHL_OK;
  double *da = nullptr, *dy = nullptr;
  int rc = CHL_OK;
  if (cudaMalloc(&da, 8 * (size_t)n) != cudaSuccess || cudaMalloc(&dy, 8 * (size_t)n) != cudaSuccess) rc = CHL_E_NOMEM;
  if (!rc) {
    cudaError_t e = cudaMemcpy(da, a, 8 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) { chl_launch_sqrt_selftest(da, dy, n, 0); e = cudaGetLastError(); }
    if (e == cudaSuccess) e = cudaMemcpy(y, dy, 8 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = CHL_E_CUDA;
  }
  cudaFree(da); cudaFree(dy);
  return rc;
}

static int run_stats(chl_handle* h, int inst, std::vector<double>& buf) {
  int rc = check_ready(h); if (rc) return rc;
  if (!get_inst(h, inst)) return CHL_E_ARG;
  chl_launch_stats(h->map(M_ROWS), h->nblk[M_ROWS], h->d_stats, h->stats_pitch, 0, h->st);
  LAUNCHED();
  buf.resize(h->stats_pitch);
  CK(cudaMemcpyAsync(buf.data(), h->d_stats + (size_t)inst * h->stats_pitch, 8 * (size_t)h->stats_pitch,
                     cudaMemcpyDeviceToHost, h->st));
  return finish(h);
}

int chl_stats(chl_handle* h, int inst, chl_stats_out* out) {
  if (!out || !h) return CHL_E_ARG;
  int rc0 = finish(h);
  if (rc0 || (rc0 = check_finite(h, inst)) || (rc0 = check_mlp(h))) return rc0;
  std::vector<double> buf;
  int rc = run_stats(h, inst, buf); if (rc) return rc;
  const Inst& I = h->in[inst];
  const double* w = buf.data() + 7 * (I.c.Ny + 1);
  const double Ly = I.c.yf[I.c.ny] - I.c.yf[1];
  out->tau_wall = w[0];
  out->utau = std::pow((w[0] + w[0]) / Ly, 0.5);
  out->Retau = out->utau * (I.c.yf[I.c.ny] - I.c.yf[1]) / 2.0 / I.d.nu;
  out->Qflow_x = w[1];
  out->Qflow_y = w[2];
  double sc[4];
  if ((rc = chl_get_scalars(h, inst, sc))) return rc;
  out->dt = sc[0]; out->t = sc[1]; out->dPdx = sc[2];
  return chl_check_divergence(h, inst, &out->max_div, &out->max_abs_div);
}

int chl_stats_profiles(chl_handle* h, int inst, double* Um, double* Vm, double* Wm, double* U2, double* V2,
                       double* W2, double* UV) {
  std::vector<double> buf;
  int rc = run_stats(h, inst, buf); if (rc) return rc;
  const int ny = h->in[inst].c.ny;
  double* dst[7] = {Um, Vm, Wm, U2, V2, W2, UV};
  for (int m = 0; m < 7; ++m)
    if (dst[m]) std::memcpy(dst[m], buf.data() + (size_t)m * ny, 8 * (size_t)ny);
  return CHL_OK;
}

}  // extern "C"
