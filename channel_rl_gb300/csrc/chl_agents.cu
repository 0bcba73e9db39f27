// Wall agents of the reference's RL environment (send_recv_state_action,
// smarties_stat.f90:24-260): per agent (x position (na-1)*nx_nagents + 2 in
// the first z plane, both walls) the 6-D state and the reward, read straight
// from the device fields by one thread per (agent, wall).
//
//   u_tau(bottom) = sqrt((nu + 1/4 sum nu_t(2 centres x 2 rows 1,2)) dU/dy|wall),
//   l = r yg(y) + (1-r) yg(y+1),  y in {3, 4} and r in [0,1) drawn by the caller,
//   U_loc  = 1/5 sum over the agent face, its two x neighbours and the two
//            z neighbours of r U(y) + (1-r) U(y+1),
//   dU_loc = 1/5 sum of U(y+1) - U(y) over the same five, / (yg(y+1)-yg(y)),
//   state  = (dU_loc l/u_tau, U_loc/u_tau - dU_loc l/u_tau ln(l u_tau/nu),
//             U_loc, l, u_tau, dPdx_ref),
//   reward = 100 - 5000 |sqrt((nu + 1/4 sum nu_t) dU/dy|wall) - sqrt(dPdx_ref)| / sqrt(dPdx_ref),
// mirrored at the top wall (rows nyg-1, nyg; l = 2 - (...)), with the
// reference's spacings (its u_tau uses yg(2)-yg(1) at both walls, its reward
// yg(nyg)-yg(nyg-1) at the top).  The device stores nu + nu_t, so nu_t is
// recovered as the stored value minus nu.
#include "chl_common.cuh"

__global__ void k_agent_obs(const ChlInst* inst, int nagents, int nxa, double dpdx_ref,
                            const int* y_ind, const double* y_rand, double* states, double* rewards) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * nagents) return;
  const ChlInst& I = *inst;
  const int wall = t / nagents, na = t % nagents;      // wall 0 bottom, 1 top
  const int Nx = I.Nx, Ny = I.Ny, Nz = I.Nz;
  const double nu = I.nu;
  const double* U = I.U[0];
  const double* nut = I.nut;
  const int a = na * nxa;                               // device face of Fortran (na-1)*nxa+2
  const int am = wrap(a - 1, Nx), ap = wrap(a + 1, Nx);
  const int k0 = 0, km = Nz - 1, kp = 1 % Nz;           // Fortran planes 2, 1, 3
  // centre rows: Fortran j <-> device jc = j - 1
  auto yg = [&](int j) { return I.ygc[j - 1]; };       // yg(j), Fortran j = 1..nyg
  auto u = [&](int face, int j, int k) { return U[cidx(I, face, j - 1, k)]; };
  auto nt = [&](int c, int j, int k) { return nut[cidx(I, c, j - 1, k)] - nu; };
  const int yi = y_ind[t];
  const double r = y_rand[t];
  const int nyg = Ny + 2;
  double ut, l, Uloc, dUloc, rew;
  const double sref = sqrt(dpdx_ref);
  if (wall == 0) {
    ut = sqrt((nu + 0.25 * (nt(ap, 2, k0) + nt(a, 2, k0) +
                            nt(ap, 1, k0) + nt(a, 1, k0))) *
              (u(a, 2, k0) - u(a, 1, k0)) / (yg(2) - yg(1)));
    l = r * yg(yi) + (1.0 - r) * yg(yi + 1);
    auto w = [&](int f, int k) { return r * u(f, yi, k) + (1.0 - r) * u(f, yi + 1, k); };
    Uloc = 0.2 * w(a, k0) + 0.2 * w(am, k0) + 0.2 * w(ap, k0) + 0.2 * w(a, km) + 0.2 * w(a, kp);
    dUloc = 0.2 * (u(a, yi + 1, k0) - u(a, yi, k0) + u(am, yi + 1, k0) - u(am, yi, k0) +
                   u(ap, yi + 1, k0) - u(ap, yi, k0) + u(a, yi + 1, km) - u(a, yi, km) +
                   u(a, yi + 1, kp) - u(a, yi, kp)) / (yg(yi + 1) - yg(yi));
    rew = 100.0 - 5000.0 * fabs(sqrt((nu + 0.25 * (nt(a, 1, k0) + nt(ap, 1, k0) + nt(a, 2, k0) + nt(ap, 2, k0))) *
                                     (u(a, 2, k0) - u(a, 1, k0)) / (yg(2) - yg(1))) - sref) / sref;
  } else {
    ut = sqrt((nu + 0.25 * (nt(ap, nyg, k0) + nt(a, nyg, k0) + nt(ap, nyg - 1, k0) + nt(a, nyg - 1, k0))) *
              (u(a, nyg - 1, k0) - u(a, nyg, k0)) / (yg(2) - yg(1)));
    l = 2.0 - (r * yg(nyg - yi + 1) + (1.0 - r) * yg(nyg - yi));
    auto w = [&](int f, int k) { return r * u(f, nyg - yi + 1, k) + (1.0 - r) * u(f, nyg - yi, k); };
    Uloc = 0.2 * w(a, k0) + 0.2 * w(am, k0) + 0.2 * w(ap, k0) + 0.2 * w(a, km) + 0.2 * w(a, kp);
    dUloc = 0.2 * (u(a, nyg - yi, k0) - u(a, nyg - yi + 1, k0) + u(am, nyg - yi, k0) - u(am, nyg - yi + 1, k0) +
                   u(ap, nyg - yi, k0) - u(ap, nyg - yi + 1, k0) + u(a, nyg - yi, km) - u(a, nyg - yi + 1, km) +
                   u(a, nyg - yi, kp) - u(a, nyg - yi + 1, kp)) / (yg(nyg - yi + 1) - yg(nyg - yi));
    rew = 100.0 - 5000.0 * fabs(sqrt((nu + 0.25 * (nt(a, nyg - 1, k0) + nt(ap, nyg - 1, k0) + nt(a, nyg, k0) +
                                                   nt(ap, nyg, k0))) *
                                     (u(a, nyg - 1, k0) - u(a, nyg, k0)) / (yg(nyg) - yg(nyg - 1))) - sref) / sref;
  }
  double* s = states + (size_t)t * 6;
  s[0] = (dUloc * l) / ut;
  s[1] = Uloc / ut - (dUloc * l) / ut * log(l * ut / nu);
  s[2] = Uloc;
  s[3] = l;
  s[4] = ut;
  s[5] = dpdx_ref;
  rewards[t] = rew;
}

extern "C" void chl_launch_agent_obs(const ChlInst* inst, int nagents, int nxa, double dpdx_ref, const int* y_ind,
                                     const double* y_rand, double* states, double* rewards, cudaStream_t st) {
  const int n = 2 * nagents;
  k_agent_obs<<<(n + 127) / 128, 128, 0, st>>>(inst, nagents, nxa, dpdx_ref, y_ind, y_rand, states, rewards);
}
