/*
 * chl.h - C ABI of the GB300 channel-LES time step.
 *
 * Drop-in for the hot path of wadaniel/channel_RL: the Fortran subroutines
 * that advance the resident channel state one RK3 step.  Each entry point
 * names the reference routine it replaces (file:line in the reference's
 * code/ directory).  Plain pointers and sizes only; arrays are Fortran
 * column-major with the reference's full ghosted extents unless stated.
 *
 * Grid convention: nx, ny, nz are the reference's global FACE counts
 * (nx_global, ny_global, nz_global, global.f90:46); Nx = nx-2 and Nz = nz-2
 * are the FFT lengths (initialization.f90:258-259), Ny = ny-1 wall-normal
 * cells; nxg = nx+1, nyg = ny+1, nzg = nz+1.  Field extents:
 *   U(nx,nyg,nzg)  V(nxg,ny,nzg)  W(nxg,nyg,nz)  P, nu_t(nxg,nyg,nzg)
 *
 * Return values: 0 on success, >0 an error code (CHL_E_*); chl_last_error()
 * gives the message.  No entry point aborts the process.
 *
 * Threading: a handle belongs to one host thread at a time.  All device work
 * is ordered on the handle's CUDA stream; calls that return host data
 * synchronise that stream.
 */
#ifndef CHL_H
#define CHL_H

#ifdef __cplusplus
extern "C" {
#endif

#define CHL_OK 0
#define CHL_E_ARG 1      /* invalid argument / size */
#define CHL_E_CUDA 2     /* CUDA runtime error */
#define CHL_E_NOMEM 3    /* device allocation failed */
#define CHL_E_STATE 4    /* call out of order (e.g. step before upload) */
#define CHL_E_NAN 5      /* non-finite velocity found by the step's CFL pass; reported by
                            chl_synchronize, chl_download and chl_stats until the next upload */
#define CHL_E_IO 6       /* file could not be opened, read or written */
#define CHL_E_TIMEOUT 7  /* a bounded device wait ran out: the learned wall model's tensor-core
                            completion barrier.  Points of the CTAs that gave up kept the
                            equilibrium stress for that stage.  Reported once (then cleared) by
                            chl_synchronize, chl_download, chl_stats and chl_mlp_read_trace. */

/* LES_model (subgrid.f90:30-45) */
#define CHL_LES_NONE 0
#define CHL_LES_SMAGORINSKY 1
#define CHL_LES_DYNAMIC 2
#define CHL_LES_AMD 3          /* anisotropic minimum dissipation (subgrid.f90:632-874) */
#define CHL_LES_VREMAN 4       /* Vreman (subgrid.f90:897-1004) */
/* wall_model */
#define CHL_WM_NONE 0     /* no-slip: compute_wall_model skipped */
#define CHL_WM_STRESS 1   /* compute_wall_model with a caller-set alpha_x (wallmodel.f90:23-46) */
#define CHL_WM_EQLOG 2    /* equilibrium log law at the third cell computes alpha_x each stage */
#define CHL_WM_MLP 3      /* equilibrium stress times exp(MLP correction), chl_mlp_* below */

typedef struct chl_handle chl_handle;

/* Grid and input parameters of one channel instance: the reference's
 * parameter file (input_output.f90:20-91) plus the face coordinates it reads
 * from the snapshot (global.f90:63-67). */
typedef struct {
  int nx, ny, nz;              /* face counts; nx, nz even; ny >= 5 */
  const double* x;             /* x(1:nx) */
  const double* y;             /* y(1:ny), y(1) and y(ny) are the walls */
  const double* z;             /* z(1:nz) */
  double nu;                   /* kinematic viscosity */
  double CFL;                  /* CFL number, or -dt for a fixed step */
  double dPdx;                 /* imposed pressure gradient (x_mass_cte = 0) */
  int x_mass_cte;              /* 1: constant mass flow (mass_flow.f90:113-166) */
  int LES_model;               /* CHL_LES_* */
  int Dirichlet_nu_t;          /* 1: nu_t ghost = -nu_t (Dirichlet), 0: Neumann; 2 (AMD, Vreman):
                                  -nu_t + 0.38 sqrt(dPdx) (y(2)-y(1)) (subgrid.f90:868-871); DSM and
                                  static Smagorinsky treat 2 as Neumann (subgrid.f90:529-533) */
  int wall_model;              /* CHL_WM_* */
  double Cs;                   /* static Smagorinsky constant */
  double Re_tau;               /* nominal friction Reynolds number (CHL_WM_MLP feature) */
} chl_grid_desc;

/* Statistics of compute_statistics (statistics.f90:22-145). */
typedef struct {
  double utau, Retau, tau_wall, Qflow_x, Qflow_y, dt, t, dPdx, max_div, max_abs_div;
} chl_stats_out;

/* initialize (initialization.f90:23-497) for one instance / n instances
 * advanced together.  Allocates every device buffer once.  Grid limits:
 * nx-2 and nz-2 of the form 2^a 3^b, x and z uniformly spaced, and fewer
 * than 2^31 points (nx-2)(ny+1)(nz-2) per instance (the kernels index an
 * instance's points in 32 bits); CHL_E_ARG otherwise. */
int chl_create(const chl_grid_desc* desc, chl_handle** out);
int chl_batch_create(int n, const chl_grid_desc* descs, chl_handle** out);
/* finalize (finalization.f90:19-121). */
int chl_destroy(chl_handle* h);
const char* chl_last_error(const chl_handle* h);
int chl_num_instances(const chl_handle* h);

/* Load U, V, W (full Fortran extents; ghosts are re-derived by the
 * boundary conditions, as the snapshot reader does, input_output.f90:514-540)
 * and set the initial bulk flow Qflow_x_0 (initialization.f90:442). */
int chl_upload(chl_handle* h, int inst, const double* U, const double* V, const double* W);
/* Fields with every ghost filled; any pointer may be NULL.  P is the actual
 * pressure of the last chl_compute_pressure call. */
int chl_download(chl_handle* h, int inst, double* U, double* V, double* W, double* P, double* nu_t);
/* Pseudo-pressure of the last projection (rhs_p, projection.f90:119-126), P layout. */
int chl_download_pseudo_pressure(chl_handle* h, int inst, double* p);

/* Wall stress alpha_x(nx,2,nzg) of the stress wall model (set by the RL
 * driver in the reference, smarties_stat.f90:180-258).  Only the unique
 * points i=2..nx-1, k=2..nzg-2 are read. */
int chl_set_wall_stress(chl_handle* h, int inst, const double* alpha_x);
int chl_get_wall_stress(chl_handle* h, int inst, double* alpha_x);

/* scalars: [0] dt, [1] t, [2] dPdx, [3] Qflow_x_0 */
int chl_get_scalars(chl_handle* h, int inst, double* out4);
/* Status word of an instance: bit 0 (1) non-finite velocity found by the
 * CFL pass, bit 2 (4) an out-of-range field index (only the bounds-checked
 * build checks; it clamps the index and records it here).  Cleared by upload. */
int chl_status_flags(chl_handle* h, int inst, int* flags);
/* Sets the four scalars of chl_get_scalars.  The dt given here is the one
 * chl_compute_time_step_RK3 uses until the next chl_compute_dt (the stage
 * coefficients times dt are formed here too). */
int chl_set_scalars(chl_handle* h, int inst, const double* in4);

/* compute_dt (time_integration.f90:102-150), all instances. */
int chl_compute_dt(chl_handle* h);
/* compute_time_step_RK3 (time_integration.f90:24-96) with the current dt. */
int chl_compute_time_step_RK3(chl_handle* h);
/* nsteps x { compute_dt; compute_time_step_RK3 } (app_main.f90:114-117),
 * replayed from one captured CUDA graph; asynchronous. */
int chl_rk3_step(chl_handle* h, int nsteps);

/* Per-subroutine entry points on the current fields (for parity bisection). */
int chl_compute_eddy_viscosity(chl_handle* h);       /* subgrid.f90:23-47 */
int chl_compute_wall_model(chl_handle* h);           /* wallmodel.f90:23-46 (eq. log law first if CHL_WM_EQLOG) */
/* compute_rhs_u/v/w (equations.f90:24-468) of the current fields and nu_t;
 * outputs on the unique points: Fu(Nx,Ny,Nz), Fv(Nx,Ny-1,Nz), Fw(Nx,Ny,Nz). */
int chl_compute_rhs(chl_handle* h, int inst, double* Fu, double* Fv, double* Fw);
int chl_compute_projection_step(chl_handle* h);      /* projection.f90:20-28 */
int chl_compute_dPx_for_constant_mass_flow(chl_handle* h, int inst, double* dPdx); /* mass_flow.f90:113-166 */
int chl_compute_pressure(chl_handle* h);             /* pressure.f90:21-29 */
int chl_check_divergence(chl_handle* h, int inst, double* max_div, double* max_abs_div); /* projection.f90:223-245 */
int chl_stats(chl_handle* h, int inst, chl_stats_out* out);  /* statistics.f90:22-145 */

/* Profiles of compute_statistics, each of length ny: Umean, Vmean, Wmean,
 * U2mean, V2mean, W2mean, UVmean (any may be NULL). */
int chl_stats_profiles(chl_handle* h, int inst, double* Umean, double* Vmean, double* Wmean,
                       double* U2mean, double* V2mean, double* W2mean, double* UVmean);

int chl_synchronize(chl_handle* h);

/* Resets the current device in the library's own CUDA runtime (it is linked
 * statically, so a caller's cudaDeviceReset does not reach it): everything
 * the library holds on that device is released, including every handle's
 * memory, so those handles must not be used again, not even destroyed.  For
 * callers that reset the device themselves, e.g. at the end of a run or
 * before handing the device to other work.  No counterpart in the
 * reference. */
int chl_device_reset(void);

/* Replace U, V, W of a running instance (no new Qflow_x_0, no sync): the
 * host-buffer round trip of a Fortran caller that keeps its own copy.  The
 * copies run on a copy stream of the handle, ordered against the steps by
 * events: with set_fields, chl_rk3_step, download_async called step after
 * step, one step's upload and the previous step's download overlap the
 * computation in between.  The host buffers must stay valid and unchanged
 * until the next chl_synchronize (or a later call that synchronises). */
int chl_set_fields(chl_handle* h, int inst, const double* U, const double* V, const double* W);
/* Download of U, V, W after the work queued so far, into (pinned) host
 * buffers, on the handle's other copy stream; completes at the next
 * chl_synchronize. */
int chl_download_async(chl_handle* h, int inst, double* U, double* V, double* W);

/* Measurement: device time (CUDA events on the handle's stream) of nsteps
 * replays of the step graph. */
int chl_time_steps(chl_handle* h, int nsteps, double* ms);
/* Number of kernel nodes in one step graph (compute_dt + RK3). */
int chl_graph_kernel_count(chl_handle* h, int* count);
/* Per-kernel device time of one step, averaged over reps un-graphed steps:
 * names[32*i] (NUL-terminated), ms_per_step[i], launches_per_step[i];
 * returns the number of kernel kinds (<= maxk) or <0 on error. */
int chl_profile_step(chl_handle* h, int reps, int maxk, char* names, double* ms_per_step, int* launches_per_step);

/* Tile-shape tuner.  It stands where the reference plans its FFTW
 * transforms (initialization.f90:287-290) for the Poisson solve of
 * projection.f90:74-128, and extends to the stencil kernels.  On the
 * uploaded fields it times, one group at a time, the block size of the
 * one-thread-per-point kernels (eddy viscosity, fluxes, RHS divergence),
 * the block-count targets of the x and z transforms and the tridiagonal
 * form (reps runs per candidate, best of three), keeps the fastest and
 * rebuilds the step graph.  Candidates only regroup independent points,
 * rows, columns and modes, so results are bit-identical whatever is chosen,
 * and the state a caller can read (fields, nu_t, pseudo-pressure, wall
 * stress) is left as it was.  report (may be NULL) receives a one-line
 * summary. */
int chl_autotune(chl_handle* h, int reps, char* report, int report_len);
/* The current tile shapes: out7 = {x_min_blocks, z_min_blocks, tri_mode,
 * point_threads, z columns per block, tridiagonal form in use (0
 * row-batched, 1 staged in shared memory, 2 lane-split for instances with
 * few modes - chosen from the instances' extents, not tuned, 3 the fused z
 * solve: forward z transform, tridiagonal solve and inverse z transform in
 * one launch of thread-block clusters, one cluster per (instance, kx)),
 * x-transform threads}. */
int chl_get_tile_shapes(chl_handle* h, int* out7);
/* Sets the tile shapes by hand: block-count targets >= 1; tri_mode 0
 * row-batched, 1 staged where it fits, 2 the default rule (the fused z
 * solve where the columns are split into lanes and every instance of the
 * handle has the same lane count and fits, else staged while one wave holds
 * all modes), 3 the fused z solve wherever it applies; point_threads 64,
 * 128 or 256.  Every choice gives bit-identical results. */
int chl_set_tile_shapes(chl_handle* h, int x_min_blocks, int z_min_blocks, int tri_mode, int point_threads);

/* Learned wall model (CHL_WM_MLP).  Counterpart of the smarties policy that
 * sets alpha_x from per-agent states (smarties_stat.f90:24-260): a
 * 4-64-64-1 tanh network per wall point, BF16 weights, FP32 accumulation,
 * tensor-core GEMMs.  theta: 4545 FP32 values, W1(64x4) b1 W2(64x64) b2
 * w3(64) b3, row major (one network shared by all instances of a batch). */
#define CHL_MLP_NPARAM 4545
int chl_mlp_set_params(chl_handle* h, const float* theta);
int chl_mlp_get_params(chl_handle* h, float* theta);
/* Gaussian exploration noise sigma on the log-stress action, its seed, and
 * whether steps accumulate the policy-gradient trace sum_t eps/sigma dmu/dtheta. */
int chl_mlp_configure(chl_handle* h, float sigma, unsigned long long seed, int train);
/* Exploration draws: shared = 0 (default) draws eps per wall point, stage
 * and step; shared != 0 draws one eps per instance, used by every wall point,
 * stage and step until chl_mlp_configure sets another seed - a perturbation
 * of the whole wall's log-stress per rollout, whose effect on the plane-
 * averaged profile a per-instance reward can resolve. */
int chl_mlp_set_exploration(chl_handle* h, int shared);
/* Trace of one instance (4545 floats); zero it afterwards if zero_after. */
int chl_mlp_read_trace(chl_handle* h, int inst, float* trace, int zero_after);
/* Network on given points (no channel): x[P][4] normalised features,
 * g[P] upstream weights -> mu[P] and trace = sum_p g_p dmu_p/dtheta. */
int chl_mlp_eval(chl_handle* h, const float* x, const float* g, int P, float* mu, float* trace);
/* Checking hooks of the learned wall model.
 * record != 0: every evaluation in the channel writes, per wall point, the
 *   CHL_MLP_REC floats [x0, x1, x2, x3 (normalised features), mu, action a,
 *   trusted (1 or 0), 0] into its instance's record, one slot per RK3 stage
 *   (the record holds the last evaluation of each stage).
 * withhold_polls > 0: the tensor-core MMAs are not issued and the completion
 *   wait gives up after withhold_polls polls (at most 64): every evaluation
 *   times out, keeps the equilibrium stress and reports CHL_E_TIMEOUT.  0
 *   restores normal operation. */
#define CHL_MLP_REC 8
int chl_mlp_debug(chl_handle* h, int record, int withhold_polls);
/* Record of one instance: 3 x 2*Nx*Nz x CHL_MLP_REC floats, stage-major,
 * then wall point p = (wall*Nz + k)*Nx + i (i, k unique cells, wall 0 bottom). */
int chl_mlp_read_record(chl_handle* h, int inst, float* rec);
/* Standalone tensor-core check: D[128x64] = A[128x64] B[64x64]^T, BF16
 * inputs (raw 16-bit patterns, row major), FP32 output.  variant 0 and 1
 * place the K-direction core-matrix stride in the descriptor's LBO or SBO
 * field; variant 2 issues no MMA and waits with a limit of 64 polls on the
 * completion barrier that nothing arrives at: it frees its TMEM and returns
 * CHL_E_TIMEOUT (the bounded-wait path of the wall-model kernel). */
int chl_tc_selftest(const unsigned short* A, const unsigned short* B, float* D, int variant);
/* Standalone check of the square root the strain magnitudes use (a Newton
 * iteration seeded by the GPU's approximate reciprocal square root; IEEE
 * results for zero, subnormal, negative, infinite and NaN arguments):
 * y[t] = that root of a[t] for n <= 2^26 values in host memory. */
int chl_sqrt_selftest(const double* a, double* y, long n);

/* Allocation-free divergence check, for callers that must not let a
 * library allocate device memory (their device memory comes from their own
 * pool or a framework's allocator, or their time loop cannot take the
 * implicit synchronisation of cudaMalloc/cudaFree); such callers cannot use
 * chl_create.  No counterpart in the reference: it reports what
 * chl_check_divergence reports (signed max of div u and max |div u| over
 * centres i=2..nxg-1, j=2..nyg-1, k=2..nzg-1) from caller-owned DEVICE
 * arrays U(nx,nyg,nzg), V(nxg,ny,nzg), W(nxg,nyg,nz) and face coordinates
 * x(nx), y(ny), z(nz) with consistent ghosts, on `stream` (a cudaStream_t,
 * NULL for the default stream); it synchronises that stream.
 * Limit: nz - 1 <= 4096 (its scratch is a fixed 64 KiB device array held by
 * every GPU that loads the library); larger grids return CHL_E_ARG.
 * It cannot be called while any stream is being captured (it copies its
 * results to pageable host memory and synchronises `stream`).  Each call
 * looks up the scratch address in the calling thread's current context.
 * Calls that overlap on the GPU race on the shared scratch and must be
 * serialised by the caller.
 * Errors: chl_noalloc_last_error() (per host thread). */
int chl_check_divergence_noalloc(const double* U, const double* V, const double* W,
                                 const double* x, const double* y, const double* z,
                                 int nx, int ny, int nz, void* stream,
                                 double* max_div, double* max_abs_div);
const char* chl_noalloc_last_error(void);

/* Host-only: the grid constants chl_create derives (initialization.f90:
 * 187-427), for checking without a GPU.  out must hold chl_grid_constants_size
 * doubles: [kxx(0:Nx-1), kzz(0:Nz-1), Dd(2:nyg-1), Du(2:nyg-1), Dl(2:nyg-1),
 * w0(1:ny), dxmin, dymin, dzmin, coef_bc_1, coef_bc_2]. */
int chl_grid_constants_size(const chl_grid_desc* desc);
int chl_grid_constants(const chl_grid_desc* desc, double* out);
/* Host-only: the pass table of the length-N transform that chl_create
 * stages for the x (N = nx-2) and z (N = nz-2) transforms.  Per pass with
 * twiddles (radix R = 4 while the remaining length allows, then 3, then 2;
 * sub-transform size Ns > 1) 7 fields of Ns doubles, entry jm for the
 * twiddles w_r = exp(-2 pi i jm r/(Ns R)), r = 1..R-1, each kept as a scale
 * sigma_r (C or S of w_r = C + iS, the larger in magnitude) and a
 * multiplier m_r (S/C or C/S): 0 m1, 1 m2, 2 m3 (radix 4) or
 * sin(2 pi/3) sigma1 (radix 3), 3 sigma1, 4 sigma2 (radix 4) or sigma1/2
 * (radix 3), 5 sigma3/sigma1 (radix 4) or sigma2/sigma1 (radix 3), 6 the
 * form bits (bit r set: w_r divided by S) as the bit pattern of a double.
 * Returns the table's length in doubles and fills out when out is not NULL
 * and cap holds it; -1 when N is not of the form 2^a 3^b, -2 when cap is
 * too small. */
int chl_fft_pass_table(int N, double* out, int cap);

/* ---- files in the reference's formats (host only, no GPU needed) ----------
 * Snapshot: the stream layout of output_data / read_input_data
 * (input_output.f90:390-730), as scripts/check_file.m reads it: int32 n and
 * float64[n] for x, y, z and the centres xm, ym, zm, then per field int32[3]
 * extents and the float64 array in Fortran order (U, V, W; P and nu_t when
 * written by a solver step), little-endian.  Arrays have the reference's
 * global ghosted extents (nx, nyg, nzg etc.).  The reference stops on a
 * size mismatch; these return CHL_E_ARG / CHL_E_IO with chl_io_last_error().
 * read_input_data also adds 0.1 (rand() - 0.5) noise to the fields it read
 * (input_output.f90:526-550); chl_snapshot_read returns the file's values. */
int chl_snapshot_dims(const char* path, int* nx, int* ny, int* nz);
int chl_snapshot_read(const char* path, int nx, int ny, int nz, double* x, double* y, double* z,
                      double* U, double* V, double* W);
/* P and nu_t: both NULL (an initial-field file) or both given. */
int chl_snapshot_write(const char* path, int nx, int ny, int nz, const double* x, const double* y,
                       const double* z, const double* U, const double* V, const double* W,
                       const double* P, const double* nu_t);
const char* chl_io_last_error(void);

/* Parameter file of read_input_parameters (input_output.f90:20-91):
 * comment lines alternating with list-directed value lines. */
typedef struct {
  int nx, ny, nz;              /* face counts (nx_global, ny_global, nz_global) */
  double CFL, nu, dPdx;
  int x_mass_cte, LES_model;
  int nsteps, nsave, nstats, nmonitor;
  char filein[256], fileout[256];
  int nstep_init, random_init, Dirichlet_nu_t;
} chl_parameters;
int chl_read_parameters(const char* path, chl_parameters* out);

/* Device state of instance inst to/from a snapshot file (output_data without
 * the step-number suffix, read_input_data without the noise).  Save computes
 * the actual pressure first when with_pressure is 1 (output_data calls
 * compute_pressure unless it is current, input_output.f90:604-606) and writes
 * P and nu_t; with 0 it writes U, V, W only.  Load checks the file's extents
 * against the instance and uploads with the boundary conditions applied. */
int chl_save_snapshot(chl_handle* h, int inst, const char* path, int with_pressure);
int chl_load_snapshot(chl_handle* h, int inst, const char* path);

/* ---- wall agents of the reference's RL environment ----------------------
 * send_recv_state_action (smarties_stat.f90:24-260) without the smarties
 * transport.  nagents agents per wall sit at x faces (na-1)*(nx-2)/nagents+2
 * of the first z plane; nagents must divide nx-2 (the reference uses
 * NUM_AGENTS/nprocs/2 = 128 for one rank).
 * chl_agent_observe: states[2][nagents][6] = (dU l/u_tau, U/u_tau - dU l/u_tau
 * ln(l u_tau/nu), U, l, u_tau, dPdx_ref) and rewards[2][nagents] = 100 - 5000
 * |sqrt(tau_w) - sqrt(dPdx_ref)|/sqrt(dPdx_ref) (smarties_stat.f90:84-176),
 * index [wall][agent]; the reference draws the sampling row y_ind (3 or 4)
 * and weight y_rand in [0,1] with RANDOM_NUMBER, here the caller passes them
 * ([2][nagents] each).  dPdx_ref is the descriptor's dPdx.
 * chl_agent_act: action[2][nagents] multiplies the current wall stress at
 * each agent (smarties_stat.f90:193-216), and alpha_x is rebuilt by linear
 * interpolation along x between agents and the z pass of :228-256. */
int chl_agent_observe(chl_handle* h, int inst, int nagents, const int* y_ind, const double* y_rand,
                      double* states, double* rewards);
int chl_agent_act(chl_handle* h, int inst, int nagents, const double* action);

#ifdef __cplusplus
}
#endif
#endif
