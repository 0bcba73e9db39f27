/* A plain C caller of libchl: the reference's solver loop without Python.
 *
 *   chl_run <snapshot-in> <snapshot-out> <nsteps> <nu> <CFL> <dPdx> <x_mass_cte>
 *           <LES_model> <Dirichlet_nu_t> <wall_model>
 *
 * Reads the mesh and U, V, W from a snapshot in the reference's stream
 * layout (read_input_data), creates one channel instance, advances nsteps
 * steps of compute_dt + compute_time_step_RK3 (app_main.f90:114-117),
 * prints the statistics and max|div u|, and writes the final state with the
 * actual pressure and nu_t (output_data).  Exit status 0 on success.
 *
 * Build: gcc -O2 chl_run.c -I<repo>/include -L<repo>/channel_rl_gb300/_build -lchl \
 *            -Wl,-rpath,<repo>/channel_rl_gb300/_build -o chl_run
 */
#include <stdio.h>
#include <stdlib.h>

#include "chl.h"

static int fail(const char* what, int rc, const char* msg) {
  fprintf(stderr, "%s failed (%d): %s\n", what, rc, msg ? msg : "");
  return 1;
}

int main(int argc, char** argv) {
  if (argc != 11) {
    fprintf(stderr, "usage: %s in out nsteps nu CFL dPdx x_mass_cte LES_model Dirichlet_nu_t wall_model\n", argv[0]);
    return 2;
  }
  int nx, ny, nz, rc;
  if ((rc = chl_snapshot_dims(argv[1], &nx, &ny, &nz))) return fail("chl_snapshot_dims", rc, chl_io_last_error());
  const size_t nu_ = (size_t)nx * (ny + 1) * (nz + 1), nv = (size_t)(nx + 1) * ny * (nz + 1);
  const size_t nw = (size_t)(nx + 1) * (ny + 1) * nz;
  double* x = malloc(sizeof(double) * nx);
  double* y = malloc(sizeof(double) * ny);
  double* z = malloc(sizeof(double) * nz);
  double* U = malloc(sizeof(double) * nu_);
  double* V = malloc(sizeof(double) * nv);
  double* W = malloc(sizeof(double) * nw);
  if (!x || !y || !z || !U || !V || !W) return fail("malloc", 0, "out of host memory");
  if ((rc = chl_snapshot_read(argv[1], nx, ny, nz, x, y, z, U, V, W)))
    return fail("chl_snapshot_read", rc, chl_io_last_error());

  chl_grid_desc d;
  d.nx = nx; d.ny = ny; d.nz = nz; d.x = x; d.y = y; d.z = z;
  d.nu = atof(argv[4]); d.CFL = atof(argv[5]); d.dPdx = atof(argv[6]);
  d.x_mass_cte = atoi(argv[7]); d.LES_model = atoi(argv[8]); d.Dirichlet_nu_t = atoi(argv[9]);
  d.wall_model = atoi(argv[10]); d.Cs = 0.1; d.Re_tau = 0.0;
  chl_handle* h = NULL;
  if ((rc = chl_create(&d, &h))) return fail("chl_create", rc, h ? chl_last_error(h) : "");
  if ((rc = chl_upload(h, 0, U, V, W))) return fail("chl_upload", rc, chl_last_error(h));
  if ((rc = chl_rk3_step(h, atoi(argv[3])))) return fail("chl_rk3_step", rc, chl_last_error(h));
  if ((rc = chl_synchronize(h))) return fail("chl_synchronize", rc, chl_last_error(h));

  chl_stats_out st;
  double dmax, dabs;
  if ((rc = chl_stats(h, 0, &st))) return fail("chl_stats", rc, chl_last_error(h));
  if ((rc = chl_check_divergence(h, 0, &dmax, &dabs))) return fail("chl_check_divergence", rc, chl_last_error(h));
  printf("steps %s  t %.6e  dt %.6e  u_tau %.6e  Re_tau %.4f  Qflow_x %.12e  max|div| %.3e\n",
         argv[3], st.t, st.dt, st.utau, st.Retau, st.Qflow_x, dabs);
  if ((rc = chl_save_snapshot(h, 0, argv[2], 1))) return fail("chl_save_snapshot", rc, chl_last_error(h));
  chl_destroy(h);
  free(x); free(y); free(z); free(U); free(V); free(W);
  return dabs <= 1e-12 ? 0 : 3;
}
