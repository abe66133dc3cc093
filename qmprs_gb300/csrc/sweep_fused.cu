// Fast mode: every sweep of a batch of small states in one launch.
//
// For batches whose states all have at most SWEEP_FUSED_MAXN qubits, one
// block per state keeps psi and t (complex64) in shared memory and runs the
// reference's per-gate sweep (qmprs/synthesis/mps_encoding/sequential.py:
// 452-505) for every sweep:
//   C|0>               rebuilt gate by gate (forward circuit order);
//   t                  the target;
//   per gate (backward circuit order)
//     psi <- G^H psi   peel the gate from the circuit state,
//     E = sum_rest conj(t[a, rest]) psi[c, rest]   (FP32 per thread and
//                      across a warp's lanes, FP64 across the warps, in
//                      fixed order),
//     W = polar(E)     thread 0, polar_sweep (FP32 Jacobi, null directions
//                      towards the current gate), G <- conj(W),
//     t <- G^H t;
//   the sweep fidelity nuc / ||target||, the sweep count, the stop at
//   stop_fidelity.
// With env_out set, one pass computes every gate's environment at the fixed
// circuit instead: E is written to the gate's slot of env_out (the gate
// store's layout, <target|C|0> = sum_ac G[a, c] E[a, c] for every gate),
// the gates stay as they are and no fidelity is written.
// On a 1024-amplitude state the grouped sweep is bound by launches and its
// FP64 window algebra (about 130 launches per sweep); here a step is a few
// block-wide passes over shared memory and one FP32 polar factor.
#include "device_common.cuh"

// one state's gate, or its adjoint, as complex64 in shared memory
__device__ __forceinline__ void fused_load_gate(const double2* g, int m, int adjoint, float2* gs) {
  if (threadIdx.x < m * m) {
    const int r = threadIdx.x / m, c = threadIdx.x % m;
    const double2 v = adjoint ? cconj(g[c * m + r]) : g[r * m + c];
    gs[threadIdx.x] = cf((float)v.x, (float)v.y);
  }
}

__device__ __forceinline__ void fused_apply(float2* v, int n, int q, int k, const float2* gs) {
  if (k == 2) {
    const int slo = n - 2 - q;
    const int64_t dlo = (int64_t)1 << slo, dhi = dlo << 1;
    for (int64_t r = threadIdx.x; r < ipow2(n - 2); r += blockDim.x) {
      const int64_t i0 = quad_base(r, slo);
      const int64_t idx[4] = {i0, i0 + dlo, i0 + dhi, i0 + dhi + dlo};
      float2 x[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) x[a] = v[idx[a]];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        float2 acc = cf(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < 4; ++c) acc = fmac(acc, gs[a * 4 + c], x[c]);
        v[idx[a]] = acc;
      }
    }
  } else {
    const int bit = n - 1 - q;
    const int64_t d = (int64_t)1 << bit;
    for (int64_t r = threadIdx.x; r < ipow2(n - 1); r += blockDim.x) {
      const int64_t i0 = pair_base(r, bit);
      const float2 x0 = v[i0], x1 = v[i0 + d];
      v[i0] = fmac(fmac(cf(0.f, 0.f), gs[0], x0), gs[1], x1);
      v[i0 + d] = fmac(fmac(cf(0.f, 0.f), gs[2], x0), gs[3], x1);
    }
  }
}

// Per-warp sum of 16 complex FP32 accumulators by a fixed FP32 butterfly;
// lane i < 16 writes entry i in FP64.  A lane holds one to four quads of a
// state of at most 13 qubits, so the FP32 sum over 32 lanes rounds at
// about 3e-7 of the entry; the FP64 butterfly it replaces held GB300's two
// FP64 units for about 1300 warp instructions per gate step.
__device__ __forceinline__ void warp_partial16_f32(const float2 (&e)[16], double2* out) {
  const int lane = threadIdx.x & 31;
  double2 mine = czero();
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    float re = e[i].x, im = e[i].y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == i) mine = cd((double)re, (double)im);
  }
  if (lane < 16) out[lane] = mine;
}

__device__ __forceinline__ float2 conj_mul(float2 a, float2 b) {   // conj(a) b
  return cf(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

__global__ void __launch_bounds__(BLOCK_THREADS) k_sweep_fused(BatchDev bd, const float2* target, double2* gates,
                                                               const signed char* arity, const int* nlayers,
                                                               int* active, const double2* tnorm2, int num_sweeps,
                                                               double stop_fid, double* sweep_fid,
                                                               int* sweeps_done, double2* env_out) {
  extern __shared__ float2 fsm[];
  __shared__ float2 gs[16];
  __shared__ double2 wred[WARPS][16];
  __shared__ double2 env[16];
  __shared__ double s_nuc;
  const int b = blockIdx.x;
  if (b >= bd.B) return;
  const int n = bd.n[b];
  const int64_t N = ipow2(n);
  float2* psi = fsm;
  float2* tt = fsm + N;
  const int L = nlayers[b];
  const int G = L * n;
  const int warp = threadIdx.x >> 5;
  const signed char* ar = arity + bd.gate_off[b] / 16;
  double2* gb = gates + bd.gate_off[b];
  if (threadIdx.x == 0) s_nuc = 0.0;
  for (int sw = 0; sw < num_sweeps; ++sw) {
    __syncthreads();
    if (!active[b]) break;
    for (int64_t i = threadIdx.x; i < N; i += blockDim.x) psi[i] = cf(i == 0 ? 1.f : 0.f, 0.f);
    for (int j = 0; j < G; ++j) {
      const int l = L - 1 - j / n, sidx = j % n, k = ar[l * n + sidx];
      if (!((k == 1) || (k == 2 && sidx <= n - 2))) {
        if (threadIdx.x == 0) atomicOr(bd.err, KERR_BAD_GATE);
        continue;
      }
      __syncthreads();
      fused_load_gate(gb + ((int64_t)l * n + sidx) * 16, 1 << k, 0, gs);
      __syncthreads();
      fused_apply(psi, n, sidx, k, gs);
    }
    for (int64_t i = threadIdx.x; i < N; i += blockDim.x) tt[i] = target[bd.vec_off[b] + i];
    for (int j = 0; j < G; ++j) {
      const int l = j / n, sidx = n - 1 - j % n, k = ar[l * n + sidx];
      if (!((k == 1) || (k == 2 && sidx <= n - 2))) {
        if (threadIdx.x == 0) atomicOr(bd.err, KERR_BAD_GATE);
        continue;
      }
      const int m = 1 << k;
      double2* gptr = gb + ((int64_t)l * n + sidx) * 16;
      __syncthreads();
      fused_load_gate(gptr, m, 1, gs);
      __syncthreads();
      float2 e[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) e[i] = cf(0.f, 0.f);
      if (k == 2) {
        const int slo = n - 2 - sidx;
        const int64_t dlo = (int64_t)1 << slo, dhi = dlo << 1;
        for (int64_t r = threadIdx.x; r < ipow2(n - 2); r += blockDim.x) {
          const int64_t i0 = quad_base(r, slo);
          const int64_t idx[4] = {i0, i0 + dlo, i0 + dhi, i0 + dhi + dlo};
          float2 x[4], y[4], tv[4];
#pragma unroll
          for (int a = 0; a < 4; ++a) x[a] = psi[idx[a]];
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            float2 acc = cf(0.f, 0.f);
#pragma unroll
            for (int c = 0; c < 4; ++c) acc = fmac(acc, gs[a * 4 + c], x[c]);
            y[a] = acc;
            psi[idx[a]] = acc;
            tv[a] = tt[idx[a]];
          }
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              const float2 p = conj_mul(tv[a], y[c]);
              e[a * 4 + c].x += p.x;
              e[a * 4 + c].y += p.y;
            }
        }
      } else {
        const int bit = n - 1 - sidx;
        const int64_t d = (int64_t)1 << bit;
        for (int64_t r = threadIdx.x; r < ipow2(n - 1); r += blockDim.x) {
          const int64_t i0 = pair_base(r, bit);
          const float2 x0 = psi[i0], x1 = psi[i0 + d];
          const float2 y0 = fmac(fmac(cf(0.f, 0.f), gs[0], x0), gs[1], x1);
          const float2 y1 = fmac(fmac(cf(0.f, 0.f), gs[2], x0), gs[3], x1);
          psi[i0] = y0;
          psi[i0 + d] = y1;
          const float2 t0 = tt[i0], t1 = tt[i0 + d];
          const float2 p0 = conj_mul(t0, y0), p1 = conj_mul(t0, y1), p2 = conj_mul(t1, y0), p3 = conj_mul(t1, y1);
          e[0].x += p0.x;
          e[0].y += p0.y;
          e[1].x += p1.x;
          e[1].y += p1.y;
          e[2].x += p2.x;
          e[2].y += p2.y;
          e[3].x += p3.x;
          e[3].y += p3.y;
        }
      }
      warp_partial16_f32(e, &wred[warp][0]);
      __syncthreads();
      if (threadIdx.x < 16) {
        double2 sum = czero();
        for (int w = 0; w < WARPS; ++w) sum = cadd(sum, wred[w][threadIdx.x]);
        env[threadIdx.x] = sum;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        double2 ee[16], w[16], wprev[16];
        bool finite = true;
        for (int i = 0; i < m * m; ++i) {
          ee[i] = env[i];
          finite = finite && isfinite(ee[i].x) && isfinite(ee[i].y);
        }
        if (!finite) {
          atomicOr(bd.err, KERR_NONFINITE);
        } else if (env_out) {
          double2* eo = env_out + bd.gate_off[b] + ((int64_t)l * n + sidx) * 16;
          for (int i = 0; i < m * m; ++i) eo[i] = ee[i];
        } else {
          for (int i = 0; i < m * m; ++i) wprev[i] = cconj(gptr[i]);
          const double nn = polar_sweep(ee, m, w, wprev);
          for (int i = 0; i < m * m; ++i) gptr[i] = cconj(w[i]);
          s_nuc = nn;
        }
      }
      __syncthreads();
      fused_load_gate(gptr, m, 1, gs);   // t <- G_new^H t
      __syncthreads();
      fused_apply(tt, n, sidx, k, gs);
    }
    __syncthreads();
    if (threadIdx.x == 0 && !env_out) {
      const double f = s_nuc / sqrt(tnorm2[b].x);
      sweep_fid[(int64_t)b * num_sweeps + sw] = f;
      sweeps_done[b] = sw + 1;
      if (stop_fid > 0.0 && f >= stop_fid) active[b] = 0;
    }
  }
}

int launch_sweep_fused(const BatchDev& bd, int max_n, const float2* target, double2* gates, const signed char* arity,
                       const int* nlayers, int* active, const double2* tnorm2, int num_sweeps, double stop_fid,
                       double* sweep_fid, int* sweeps_done, cudaStream_t s, double2* env_out) {
  const size_t smem = 2 * sizeof(float2) * (size_t)ipow2(max_n);
  cudaError_t e = cudaFuncSetAttribute(k_sweep_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  qm_note_launch();
  k_sweep_fused<<<bd.B, BLOCK_THREADS, smem, s>>>(bd, target, gates, arity, nlayers, active, tnorm2, num_sweeps,
                                                  stop_fid, sweep_fid, sweeps_done, env_out);
  return (int)cudaGetLastError();
}
