// Learned wall model: a 4 -> 64 -> 64 -> 1 tanh MLP per wall point that
// corrects the equilibrium log-law wall stress, tau_w = tau_eq * exp(a),
// a in [-0.5, 0.5].  It is the counterpart of the reference's smarties
// policy, which receives per-agent states and returns wall-stress actions
// (smarties_stat.f90:24-260); the network itself is the build's own.
//
// Per wall point (x-face a, z-centre k, wall w) the features are
//   f0 = u / U_b at the matching height (third off-wall cell, U_b = 1),
//   f1 = ln(h Re_tau),
//   f2 = local dp/dx * h / tau_eq (pseudo-pressure gradient of the last
//        projection divided by dt), clipped to [-10, 10],
//   f3 = ln((nu + nu_t)/nu) at the matching height,
// normalised to x = (f0 - 1, (f1 - 6)/2, f2/5, f3/3 - 1).  Outside the trust
// range (f0 in [0.05, 3], f1 in [2, 11], f3 in [0, 8]) the equilibrium
// stress is used unchanged and the point contributes no gradient.
//
// One CTA of 128 threads handles 128 wall points.  The 64x64 layer runs on
// the tensor cores (tcgen05, BF16 operands from shared memory, FP32
// accumulators in TMEM); so do the two GEMMs of the policy-gradient trace
// (d_h1 = d_h2 W2 and dW2 = d_h2^T h1).  The 4-wide first layer and the
// 64-wide output layer are FP32 FMAs.  See oracle/mlp_ref.py for the
// formulas and roundings.
#include "chl_common.cuh"
#include "chl_tc.cuh"

#define MLP_H 64
#define MLP_NPARAM 4545
#define MLP_TILE 128
#define MLP_WAIT_ITERS (1L << 24)

// parameter offsets (oracle/mlp_ref.py unpack)
#define P_W1 0
#define P_B1 256
#define P_W2 320
#define P_B2 4416
#define P_W3 4480
#define P_B3 4544

// shared-memory map (bytes)
#define S_BW2 0          // W2 as B operand  [64 out x 64 in]   8 KB
#define S_BW2T 8192      // W2^T as B operand [64 in x 64 out]  8 KB
#define S_A1 16384       // H1 [128 x 64]                       16 KB
#define S_A2 32768       // dH2 [128 x 64]                      16 KB
#define S_A3 49152       // [dH2^T ; 0] [128 x 128]             32 KB
#define S_B3 81920       // H1^T [64 x 128]                     16 KB
#define S_PAR 98304      // float params: W1 (256) b1 b2 w3 b3   (449 floats)
// reduction area, per warp RW floats: [0,64) db2, [64,128) dw3, [128] db3,
// [129,385) dW1 (4 per hidden unit), [385,449) db1
#define RW 456
#define S_RED (S_PAR + 2048)
#define S_MISC (S_RED + 4 * RW * 4)
#define MLP_SMEM (S_MISC + 64)

constexpr uint32_t IDESC_128x64 = tc::idesc_bf16_f32(128, 64);

struct MlpArgs {
  const float* theta;     // FP32 master parameters (MLP_NPARAM)
  const float* x;         // test mode: features [P][4] (null: channel mode)
  const float* g;         // test mode: upstream weights [P]
  float* mu_out;          // test mode: mu [P]
  float* trace_out;       // test mode: trace (MLP_NPARAM)
  int P;
  int s_in, stage;          // channel mode: velocity set and RK stage (noise counter)
  int* status;
};

__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// standard normal from a counter (Box-Muller on two 53-bit uniforms)
__device__ __forceinline__ float gauss(unsigned long long seed, unsigned long long ctr) {
  const unsigned long long a = mix64(seed ^ mix64(ctr));
  const unsigned long long b = mix64(a + 0x632BE59BD9B4E019ULL);
  const double u1 = ((a >> 11) + 1.0) * (1.0 / 9007199254740993.0);
  const double u2 = (b >> 11) * (1.0 / 9007199254740992.0);
  return (float)(sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
}

__global__ void __launch_bounds__(MLP_TILE)
k_mlp(ChlMap map, MlpArgs A) {
  chl_pdl_wait();
  extern __shared__ __align__(1024) unsigned char sm[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + S_MISC);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + S_MISC + 16);
  float* par = reinterpret_cast<float*>(sm + S_PAR);
  float* red = reinterpret_cast<float*>(sm + S_RED);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool chan = A.x == nullptr;
  const ChlInst* I = nullptr;
  int P, p0;
  if (chan) {
    int lb;
    I = &map.inst[chl_find(map, blockIdx.x, lb)];
    P = 2 * I->Nx * I->Nz;
    p0 = lb * MLP_TILE;
  } else {
    P = A.P;
    p0 = blockIdx.x * MLP_TILE;
  }
  const unsigned int* cfg = chan ? I->mlp_cfg : nullptr;
  const bool train = chan ? (cfg[1] != 0) : true;
  float* trace = chan ? I->mlp_trace : A.trace_out;
  // checking hooks (chl_mlp_debug): the per-point record, and a withheld
  // MMA whose completion wait gives up after cfg[6] polls
  float* rec = (chan && cfg[5] != 0u && I->mlp_rec) ? I->mlp_rec + (size_t)A.stage * P * 8 : nullptr;
  const unsigned int withhold = chan ? cfg[6] : 0u;
  const long wait_iters = withhold ? (long)withhold : MLP_WAIT_ITERS;

  if (tid == 0) tc::mbar_init(mbar, 1);
  if (warp == 0) tc::tmem_alloc(tslot, 256);
  // parameters: W1, b1, b2, w3, b3 as floats (weights BF16-rounded); W2 into both B tiles
  const float* th = chan ? I->mlp_theta : A.theta;
  for (int q = tid; q < 256; q += MLP_TILE) par[q] = bf16r(th[P_W1 + q]);
  for (int q = tid; q < 64; q += MLP_TILE) {
    par[256 + q] = th[P_B1 + q];
    par[320 + q] = th[P_B2 + q];
    par[384 + q] = bf16r(th[P_W3 + q]);
  }
  if (tid == 0) par[448] = th[P_B3];
  for (int q = tid; q < 64 * 64; q += MLP_TILE) {
    const int o = q >> 6, i = q & 63;            // W2[o][i]
    const float w = th[P_W2 + q];
    tc::store_elem(sm + S_BW2, o, i, w, 128, 1024);
    tc::store_elem(sm + S_BW2T, i, o, w, 128, 1024);
  }
  // rows 64..127 of the [dH2^T ; 0] tile stay zero
  for (int q = tid; q < 64 * 128 / 8; q += MLP_TILE) {
    const int r = 64 + q / 16, kb = q % 16;
    *reinterpret_cast<uint4*>(sm + S_A3 + tc::canon_off(r, 8 * kb, 128, 2048)) = make_uint4(0, 0, 0, 0);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *tslot;

  // ---------------------------------------------------------------- features
  const int gp = p0 + tid;
  const bool valid = gp < P;
  float x[4] = {0.f, 0.f, 0.f, 0.f};
  float g = 0.f;
  double taueq = 0.0;               // equilibrium stress, kept in FP64 (alpha is an FP64 field)
  bool trusted = valid;
  if (valid && chan) {
    const ChlInst& In = *I;
    const int Nx = In.Nx, Nz = In.Nz;
    const int a = gp % Nx, k = (gp / Nx) % Nz, wall = gp / (Nx * Nz);
    const int jm = wall == 0 ? 3 : In.Ny - 2;
    const double h = wall == 0 ? In.hb : In.ht;
    const double* U = In.U[A.s_in];
    const double u = U[cidx(In, a, jm, k)];
    taueq = In.alpha[gp];
    const double ap = fabs(taueq);
    const double dt = In.scal[CHL_S_DT];
    double dpdx = 0.0;
    if (dt > 0.0) dpdx = (In.p[cidx(In, wrap(a + 1, Nx), jm, k)] - In.p[cidx(In, a, jm, k)]) * In.rdxf[a] / dt;
    double f2 = ap > 0.0 ? dpdx * h / ap : 0.0;
    f2 = fmin(10.0, fmax(-10.0, f2));
    const double ntf = 0.5 * (In.nut[cidx(In, a, jm, k)] + In.nut[cidx(In, wrap(a + 1, Nx), jm, k)]);
    const double f0 = u, f1 = log(h * In.retau), f3 = log(fmax(ntf / In.nu, 1e-300));
    trusted = f0 >= 0.05 && f0 <= 3.0 && f1 >= 2.0 && f1 <= 11.0 && f3 >= 0.0 && f3 <= 8.0 && ap > 0.0;
    x[0] = (float)(f0 - 1.0); x[1] = (float)((f1 - 6.0) / 2.0); x[2] = (float)(f2 / 5.0); x[3] = (float)(f3 / 3.0 - 1.0);
  } else if (valid) {
    x[0] = A.x[4 * gp]; x[1] = A.x[4 * gp + 1]; x[2] = A.x[4 * gp + 2]; x[3] = A.x[4 * gp + 3];
    g = A.g[gp];
  }
  if (rec && valid) {
    float* r = rec + (size_t)gp * 8;
    r[0] = x[0]; r[1] = x[1]; r[2] = x[2]; r[3] = x[3];
    r[4] = __int_as_float(0x7fc00000); r[5] = 0.f;     // mu, a: set below unless the wait runs out
    r[6] = trusted ? 1.f : 0.f; r[7] = 0.f;
  }
  // ---------------------------------------------------------------- layer 1 (FP32) -> H1 tiles
  float h1[MLP_H];
#pragma unroll
  for (int n = 0; n < MLP_H; ++n) {
    float z = par[256 + n];
    z = fmaf(par[4 * n + 0], x[0], z); z = fmaf(par[4 * n + 1], x[1], z);
    z = fmaf(par[4 * n + 2], x[2], z); z = fmaf(par[4 * n + 3], x[3], z);
    h1[n] = valid ? bf16r(tanhf(z)) : 0.f;
  }
  tc::store_row64(sm + S_A1, tid, h1, 128, 1024);
#pragma unroll
  for (int n = 0; n < MLP_H; ++n) tc::store_elem(sm + S_B3, n, tid, h1[n], 128, 2048);
  tc::fence_proxy_async();
  __syncthreads();
  tc::fence_after_sync();
  // ---------------------------------------------------------------- layer 2 on the tensor cores
  if (tid == 0 && !withhold) {
#pragma unroll
    for (int s = 0; s < 4; ++s)
      tc::mma_bf16(taddr, tc::make_desc(tc::smem_u32(sm + S_A1 + 256 * s), 128, 1024),
                   tc::make_desc(tc::smem_u32(sm + S_BW2 + 256 * s), 128, 1024), IDESC_128x64, s);
    tc::mma_commit(mbar);
  }
  bool ok = tc::mbar_wait(mbar, 0, wait_iters);
  ok = __syncthreads_and(ok);
  float mu = 0.f;
  if (ok) {
    tc::fence_after_sync();
    float h2[MLP_H];
    const uint32_t trow = taddr + ((uint32_t)(warp * 32) << 16);
#pragma unroll
    for (int q = 0; q < 4; ++q) tc::tmem_ld16(trow + 16 * q, h2 + 16 * q);
    float o = par[448];
#pragma unroll
    for (int n = 0; n < MLP_H; ++n) {
      h2[n] = tanhf(h2[n] + par[320 + n]);
      o = fmaf(par[384 + n], h2[n], o);
    }
    mu = 0.5f * tanhf(o);
    // ---------------------------------------------------------------- action
    if (chan) {
      const float sigma = __uint_as_float(cfg[0]);
      float a = 0.f;
      if (valid && trusted) {
        float eps = 0.f;
        if (sigma > 0.f) {
          const unsigned long long seed = ((unsigned long long)cfg[3] << 32) | cfg[2];
          // cfg[7] != 0: one draw per instance, the same for every wall
          // point, stage and step until the seed changes (chl_mlp_set_exploration)
          const unsigned long long inst = (unsigned long long)(I - map.inst);
          const unsigned long long ctr = cfg[7] != 0u ? inst * 0x1000000ULL
              : ((unsigned long long)cfg[4] * 4ULL + (unsigned long long)A.stage) * 0x100000000ULL
                + inst * 0x1000000ULL + (unsigned long long)gp;
          eps = gauss(seed, ctr);
        }
        a = fminf(0.5f, fmaxf(-0.5f, mu + sigma * eps));
        g = (train && sigma > 0.f) ? eps / sigma : 0.f;
        I->alpha[gp] = taueq * exp((double)a);
      }
      if (rec && valid) { rec[(size_t)gp * 8 + 4] = mu; rec[(size_t)gp * 8 + 5] = a; }
    } else if (valid) {
      A.mu_out[gp] = mu;
    }
    // ---------------------------------------------------------------- policy-gradient trace
    if (train) {
      const float d_o = g * 0.5f * (1.f - 4.f * mu * mu);     // g * d mu / d o
      float dh2[MLP_H];
#pragma unroll
      for (int n = 0; n < MLP_H; ++n) dh2[n] = bf16r(d_o * par[384 + n] * (1.f - h2[n] * h2[n]));
      tc::store_row64(sm + S_A2, tid, dh2, 128, 1024);
#pragma unroll
      for (int n = 0; n < MLP_H; ++n) tc::store_elem(sm + S_A3, n, tid, dh2[n], 128, 2048);
      // per-thread small sums: db2 (64), dw3 (64), db3 (1) -> warp partials in smem
      float* wr = red + warp * RW;
#pragma unroll
      for (int n = 0; n < MLP_H; ++n) {
        float v = dh2[n], w = d_o * h2[n];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) { v += __shfl_xor_sync(0xffffffffu, v, off); w += __shfl_xor_sync(0xffffffffu, w, off); }
        if (lane == 0) { wr[n] = v; wr[64 + n] = w; }
      }
      float vb = d_o;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) vb += __shfl_xor_sync(0xffffffffu, vb, off);
      if (lane == 0) wr[128] = vb;
      tc::fence_proxy_async();
      __syncthreads();
      tc::fence_after_sync();
      if (tid == 0) {
#pragma unroll
        for (int s = 0; s < 4; ++s)       // d_h1 (pre-activation) = d_h2 W2
          tc::mma_bf16(taddr + 64, tc::make_desc(tc::smem_u32(sm + S_A2 + 256 * s), 128, 1024),
                       tc::make_desc(tc::smem_u32(sm + S_BW2T + 256 * s), 128, 1024), IDESC_128x64, s);
#pragma unroll
        for (int s = 0; s < 8; ++s)       // dW2 = d_h2^T h1 over the 128 points
          tc::mma_bf16(taddr + 128, tc::make_desc(tc::smem_u32(sm + S_A3 + 256 * s), 128, 2048),
                       tc::make_desc(tc::smem_u32(sm + S_B3 + 256 * s), 128, 2048), IDESC_128x64, s);
        tc::mma_commit(mbar);
      }
      bool ok2 = tc::mbar_wait(mbar, 1, MLP_WAIT_ITERS);
      ok2 = __syncthreads_and(ok2);
      if (ok2) {
        tc::fence_after_sync();
        float dh1[MLP_H];
#pragma unroll
        for (int q = 0; q < 4; ++q) tc::tmem_ld16(trow + 64 + 16 * q, dh1 + 16 * q);
        // d_h1 through tanh; dW1 (64x4) and db1 (64): warp sums into smem
        float* wr2 = red + warp * RW + 129;
#pragma unroll
        for (int n = 0; n < MLP_H; ++n) {
          const float d = dh1[n] * (1.f - h1[n] * h1[n]);
          float v0 = d * x[0], v1 = d * x[1], v2 = d * x[2], v3 = d * x[3], vb1 = d;
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) {
            v0 += __shfl_xor_sync(0xffffffffu, v0, off); v1 += __shfl_xor_sync(0xffffffffu, v1, off);
            v2 += __shfl_xor_sync(0xffffffffu, v2, off); v3 += __shfl_xor_sync(0xffffffffu, v3, off);
            vb1 += __shfl_xor_sync(0xffffffffu, vb1, off);
          }
          if (lane == 0) {
            wr2[4 * n] = v0; wr2[4 * n + 1] = v1; wr2[4 * n + 2] = v2; wr2[4 * n + 3] = v3;
            wr2[256 + n] = vb1;
          }
        }
        // dW2 rows from TMEM lanes 0..63 (warps 0 and 1)
        if (warp < 2) {
          float r[MLP_H];
#pragma unroll
          for (int q = 0; q < 4; ++q) tc::tmem_ld16(trow + 128 + 16 * q, r + 16 * q);
#pragma unroll
          for (int n = 0; n < MLP_H; ++n) atomicAdd(trace + P_W2 + 64 * tid + n, r[n]);
        } else {
          float r[MLP_H];   // keep the collective load uniform per warp; lanes 64..127 hold zeros
#pragma unroll
          for (int q = 0; q < 4; ++q) tc::tmem_ld16(trow + 128 + 16 * q, r + 16 * q);
        }
        __syncthreads();
        // combine the 4 warp partials and add to the trace
        for (int q = tid; q < 129 + 320; q += MLP_TILE) {
          const float v = red[q] + red[RW + q] + red[2 * RW + q] + red[3 * RW + q];
          int dst;
          if (q < 64) dst = P_B2 + q;
          else if (q < 128) dst = P_W3 + (q - 64);
          else if (q == 128) dst = P_B3;
          else if (q < 129 + 256) dst = P_W1 + (q - 129);
          else dst = P_B1 + (q - 129 - 256);
          atomicAdd(trace + dst, v);
        }
      }
      ok = ok2;
    }
  }
  if (!ok && tid == 0 && A.status) atomicExch(A.status, 1);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, 256);
}

// ---------------------------------------------------------------- tcgen05 self-test
// D[128x64] = A[128x64] . B[64x64]^T for BF16 A, B (row-major, K contiguous),
// one CTA.  `variant` selects which descriptor field carries the K-direction
// core-matrix stride (0: LBO, 1: SBO); both stay inside the tiles.  Variant
// 2 issues no MMA and waits at most 64 polls on the completion barrier,
// which nothing arrives at: the bounded-wait path (status set, TMEM freed).
__global__ void __launch_bounds__(128)
k_tc_selftest(const __nv_bfloat16* Ag, const __nv_bfloat16* Bg, float* D, int variant, int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* Bs = sm;            // 8 KB
  unsigned char* As = sm + 8192;     // 16 KB (+4 KB pad)
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + 28672);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + 28672 + 16);
  const int tid = threadIdx.x, warp = tid >> 5;
  if (tid == 0) tc::mbar_init(mbar, 1);
  if (warp == 0) tc::tmem_alloc(tslot, 64);
  for (int q = tid; q < 128 * 64; q += 128) {
    const int r = q >> 6, k = q & 63;
    *reinterpret_cast<__nv_bfloat16*>(As + tc::canon_off(r, k, 128, 1024)) = Ag[q];
  }
  for (int q = tid; q < 64 * 64; q += 128) {
    const int r = q >> 6, k = q & 63;
    *reinterpret_cast<__nv_bfloat16*>(Bs + tc::canon_off(r, k, 128, 1024)) = Bg[q];
  }
  for (int q = tid; q < 4096 / 16; q += 128) reinterpret_cast<uint4*>(As + 16384)[q] = make_uint4(0, 0, 0, 0);
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *tslot;
  const uint32_t lbo = variant == 1 ? 1024u : 128u, sbo = variant == 1 ? 128u : 1024u;
  const bool withhold = variant == 2;
  if (tid == 0 && !withhold) {
    for (int s = 0; s < 4; ++s)
      tc::mma_bf16(taddr, tc::make_desc(tc::smem_u32(As + 256 * s), lbo, sbo),
                   tc::make_desc(tc::smem_u32(Bs + 256 * s), lbo, sbo), IDESC_128x64, s);
    tc::mma_commit(mbar);
  }
  bool ok = tc::mbar_wait(mbar, 0, withhold ? 64L : MLP_WAIT_ITERS);
  ok = __syncthreads_and(ok);
  if (ok) {
    tc::fence_after_sync();
    float v[64];
    for (int q = 0; q < 4; ++q) tc::tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + 16 * q, v + 16 * q);
    for (int n = 0; n < 64; ++n) D[tid * 64 + n] = v[n];
  } else if (tid == 0) {
    *status = 1;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, 64);
}

extern "C" {
int chl_mlp_setup() {
  cudaError_t e = cudaFuncSetAttribute(k_mlp, cudaFuncAttributeMaxDynamicSharedMemorySize, MLP_SMEM);
  return e == cudaSuccess ? 0 : 1;
}
void chl_launch_mlp(const ChlMap& m, int nb, int s_in, int stage, int* status, cudaStream_t st) {
  MlpArgs a{nullptr, nullptr, nullptr, nullptr, nullptr, 0, s_in, stage, status};
  chl_launch_pdl(k_mlp, dim3(nb), dim3(MLP_TILE), MLP_SMEM, st, m, a);
}
void chl_launch_mlp_test(const float* theta, const float* x, const float* g, int P, float* mu, float* trace,
                         int* status, cudaStream_t st) {
  ChlMap m{nullptr, nullptr, 0};
  MlpArgs a{theta, x, g, mu, trace, P, 0, 0, status};
  chl_launch_pdl(k_mlp, dim3((P + MLP_TILE - 1) / MLP_TILE), dim3(MLP_TILE), MLP_SMEM, st, m, a);
}
int chl_tc_selftest_launch(const void* A, const void* B, float* D, int variant, int* status, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, 28672 + 64);
  if (e != cudaSuccess) return 1;
  k_tc_selftest<<<1, 128, 28672 + 64, st>>>((const __nv_bfloat16*)A, (const __nv_bfloat16*)B, D, variant, status);
  return 0;
}
}
