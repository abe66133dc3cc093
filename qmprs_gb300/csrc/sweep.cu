// (d) one gate update of the environment sweep, for every state at once.
//
// Restates the body of Sequential._sweep_unitary_layers (reference
// qmprs/synthesis/mps_encoding/sequential.py:452-505) on dense vectors:
//   psi <- G^H psi                           (circuit_mps @ gate.conj(), :460)
//   E[a][b] = sum_rest conj(t[a,rest]) psi[b,rest]   (target @ circuit, :463)
//   W = u @ vh of E, new gate = conj(W)      (:473-478, :501-505)
// The t <- new^H t update (:496) is the following k_apply_gate launch.
// E is accumulated per thread in fp32 over a few quads, then in fp64 across
// the block and across tiles (deterministic tile order); the polar factor is
// an fp64 one-sided Jacobi SVD.  nuc[b] receives the nuclear norm of E, i.e.
// |<t|new|psi>| after the update.
// Singular values of E at most 1e-6 of the largest count as zero: on that
// null space (inputs the circuit never feeds the gate, such as fresh |0>
// qubits) every completion is optimal, and the kernel keeps the one nearest
// to the current gate so that structured gates stay structured under fp32
// rounding.
#include "device_common.cuh"

__global__ void __launch_bounds__(BLOCK_THREADS) k_sweep_env(BatchDev bd, int step, float2* psi,
                                                             const float2* t, double2* gates,
                                                             const signed char* arity,
                                                             const int* nlayers, const int* active,
                                                             double2* partials, double* nuc) {
  GateSel sel;
  sel.mode = SEL_SWEEP;
  sel.step = step;
  sel.layer = 0;
  sel.adjoint = 1;
  sel.gates = gates;
  sel.arity = arity;
  sel.nlayers = nlayers;
  sel.active = active;
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    const int n = bd.n[b];
    int64_t slot;
    int q, k;
    if (!select_gate(sel, bd, b, n, &slot, &q, &k)) continue;
    const int nt = bd.state_ntiles[b];
    const double2* gptr = gates + bd.gate_off[b] + slot * 16;
    float2 g[16];
    float2* v = psi + bd.vec_off[b];
    const float2* tv = t + bd.vec_off[b];
    int64_t lo, hi;
    tile_range(ipow2(n - k), bd.tile_idx[tile], nt, &lo, &hi);
    float2 e[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) e[i] = cf(0.f, 0.f);
    if (k == 2) {
      load_gate_m<4>(gptr, 1, g);
      const int slo = n - 2 - q;
      const int64_t dlo = (int64_t)1 << slo, dhi = dlo << 1;
      for (int64_t r = lo + threadIdx.x; r < hi; r += blockDim.x) {
        const int64_t i0 = quad_base(r, slo);
        const int64_t idx[4] = {i0, i0 + dlo, i0 + dhi, i0 + dhi + dlo};
        float2 x[4], y[4], z[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) { x[a] = v[idx[a]]; z[a] = tv[idx[a]]; }
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          float2 acc = cf(0.f, 0.f);
#pragma unroll
          for (int c = 0; c < 4; ++c) acc = fmac(acc, g[a * 4 + c], x[c]);
          y[a] = acc;
          v[idx[a]] = acc;
        }
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const float2 ca = cf(z[a].x, -z[a].y);
#pragma unroll
          for (int c = 0; c < 4; ++c) e[a * 4 + c] = fmac(e[a * 4 + c], ca, y[c]);
        }
      }
    } else {
      load_gate_m<2>(gptr, 1, g);
      const int bit = n - 1 - q;
      const int64_t d = (int64_t)1 << bit;
      for (int64_t r = lo + threadIdx.x; r < hi; r += blockDim.x) {
        const int64_t i0 = pair_base(r, bit);
        float2 x0 = v[i0], x1 = v[i0 + d];
        float2 z0 = tv[i0], z1 = tv[i0 + d];
        float2 y0 = fmac(fmac(cf(0.f, 0.f), g[0], x0), g[1], x1);
        float2 y1 = fmac(fmac(cf(0.f, 0.f), g[2], x0), g[3], x1);
        v[i0] = y0;
        v[i0 + d] = y1;
        const float2 c0 = cf(z0.x, -z0.y), c1 = cf(z1.x, -z1.y);
        e[0] = fmac(e[0], c0, y0);
        e[1] = fmac(e[1], c0, y1);
        e[2] = fmac(e[2], c1, y0);
        e[3] = fmac(e[3], c1, y1);
      }
    }
    warp_partial16(e, partials + ((int64_t)tile * WARPS + (threadIdx.x >> 5)) * 16);
  }
}

// One block per state: sum the tile partials of E in tile order (16 lanes
// per entry, fixed order, then a fixed shuffle tree), then thread 0 takes
// the fp64 polar factor and writes the new gate conj(W) and |E|_*.
__global__ void __launch_bounds__(BLOCK_THREADS) k_sweep_polar(BatchDev bd, int step, double2* gates,
                                                               const signed char* arity, const int* nlayers,
                                                               const int* active, const double2* partials,
                                                               double* nuc) {
  __shared__ double2 env_s[16];
  GateSel sel;
  sel.mode = SEL_SWEEP;
  sel.step = step;
  sel.layer = 0;
  sel.adjoint = 1;
  sel.gates = gates;
  sel.arity = arity;
  sel.nlayers = nlayers;
  sel.active = active;
  for (int b = blockIdx.x; b < bd.B; b += gridDim.x) {
    const int n = bd.n[b];
    int64_t slot;
    int q, k;
    if (!select_gate(sel, bd, b, n, &slot, &q, &k)) continue;
    const int m = 1 << k;
    const int np = bd.state_ntiles[b] * WARPS;
    const int64_t p0 = (int64_t)bd.state_tile0[b] * WARPS;
    const int entry = threadIdx.x >> 4, lane = threadIdx.x & 15;   // 16 entries x 16 lanes
    double2 s = czero();
    if (entry < m * m)
      for (int t = lane; t < np; t += 16) s = cadd(s, partials[(p0 + t) * 16 + entry]);
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) {
      s.x += __shfl_down_sync(0xffffffffu, s.x, o, 16);
      s.y += __shfl_down_sync(0xffffffffu, s.y, o, 16);
    }
    if (lane == 0) env_s[entry] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double2 env[16], w[16], wprev[16];
      double2* gptr = gates + bd.gate_off[b] + slot * 16;
      bool finite = true;
      for (int i = 0; i < m * m; ++i) {
        env[i] = env_s[i];
        finite = finite && isfinite(env[i].x) && isfinite(env[i].y);
      }
      if (!finite) {
        atomicOr(bd.err, KERR_NONFINITE);
      } else {
        for (int i = 0; i < m * m; ++i) wprev[i] = cconj(gptr[i]);
        const double nn = polar_sweep(env, m, w, wprev);
        for (int i = 0; i < m * m; ++i) gptr[i] = cconj(w[i]);
        nuc[b] = nn;
      }
    }
    __syncthreads();
  }
}

// After a sweep: record |<target|C|0>| / ||target|| and retire finished states.
__global__ void k_sweep_finish(int B, int sweep, int num_sweeps, const double* nuc, const double2* tnorm2,
                               double* sweep_fid, int* sweeps_done, int* active, double stop_fid,
                               int* num_active) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
    if (!active[b]) continue;
    const double f = nuc[b] / sqrt(tnorm2[b].x);
    sweep_fid[(int64_t)b * num_sweeps + sweep] = f;
    sweeps_done[b] = sweep + 1;
    if (stop_fid > 0.0 && f >= stop_fid) active[b] = 0;
    else atomicAdd(num_active, 1);
  }
}

static int grid_for(const BatchDev& bd) {
  int g = bd.ntiles;
  const int cap = 152 * 8;
  return g < cap ? g : cap;
}

void launch_sweep_env(const BatchDev& bd, int step, float2* psi, const float2* t, double2* gates,
                      const signed char* arity, const int* nlayers, const int* active,
                      double2* partials, double* nuc, cudaStream_t s) {
  qm_note_launch();
  k_sweep_env<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, step, psi, t, gates, arity, nlayers, active,
                                                     partials, nuc);
}

void launch_sweep_polar(const BatchDev& bd, int step, double2* gates, const signed char* arity,
                        const int* nlayers, const int* active, const double2* partials, double* nuc,
                        cudaStream_t s) {
  qm_note_launch();
  const int blocks = bd.B < 152 * 8 ? bd.B : 152 * 8;
  k_sweep_polar<<<blocks, BLOCK_THREADS, 0, s>>>(bd, step, gates, arity, nlayers, active, partials, nuc);
}

void launch_sweep_finish(int B, int sweep, int num_sweeps, const double* nuc, const double2* tnorm2,
                         double* sweep_fid, int* sweeps_done, int* active, double stop_fid,
                         int* num_active, cudaStream_t s) {
  qm_note_launch();
  k_sweep_finish<<<(B + 127) / 128, 128, 0, s>>>(B, sweep, num_sweeps, nuc, tnorm2, sweep_fid,
                                                 sweeps_done, active, stop_fid, num_active);
}
