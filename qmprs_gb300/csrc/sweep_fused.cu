// Circuit rebuild of the sweep (reference
// qmprs/synthesis/mps_encoding/sequential.py:443-447 densifies C|0> at the
// start of every sweep).
//
// k_rebuild_win  builds C|0> applying up to three consecutive gates of every
//                state per pass: three consecutive gates of the circuit order
//                touch at most four qubits, so a thread holds the 16
//                amplitudes of one 4-qubit window and applies them in
//                registers.  16 B of HBM traffic per amplitude per pass.
#include "window.cuh"

// Gate of state b at forward position j (circuit order): generated layer L-1-j/n, site j%n.
__device__ __forceinline__ bool fwd_gate(const BatchDev& bd, const signed char* arity, int L, int n, int b, int j,
                                         int64_t* slot, int* q, int* k) {
  if (j < 0 || j >= L * n) return false;
  const int l = L - 1 - j / n, s = j % n;
  *slot = (int64_t)l * n + s;
  *q = s;
  *k = arity[bd.gate_off[b] / 16 + *slot];
  return (*k == 1) || (*k == 2 && s <= n - 2);
}

__device__ __forceinline__ void stage_gate(float2* dst, const double2* src, int k, int adjoint) {
  const int m = 1 << k;
  for (int i = threadIdx.x; i < m * m; i += blockDim.x) {
    const int r = i / m, c = i % m;
    const double2 v = adjoint ? cconj(src[c * m + r]) : src[r * m + c];
    dst[i] = cf((float)v.x, (float)v.y);
  }
}

template <int U>
__device__ __forceinline__ void rebuild_groups(const BatchDev& bd, int b, int n, int tile, float2* v, const WinSpec& w,
                                               const float2 (*gs)[16], const int* gk, const int* ghi, const int* glo,
                                               int ng) {
  int off[1 << U];
  win_offsets<U>(w, off);
  int64_t lo, hi;
  tile_range(ipow2(n - U), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
  for (int64_t r = lo + threadIdx.x; r < hi; r += blockDim.x) {
    const int64_t base = win_base(w, r);
    float2 a[1 << U];
#pragma unroll
    for (int li = 0; li < (1 << U); ++li) a[li] = v[base + off[li]];
    for (int g = 0; g < ng; ++g) win_apply<U>(a, gs[g], gk[g], ghi[g], glo[g]);
#pragma unroll
    for (int li = 0; li < (1 << U); ++li) v[base + off[li]] = a[li];
  }
}

__global__ void __launch_bounds__(BLOCK_THREADS, 2) k_rebuild_win(BatchDev bd, float2* psi, const double2* gates,
                                                               const signed char* arity, const int* nlayers,
                                                               const int* active, int j0, int count) {
  __shared__ float2 gs[3][16];
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    if (active && !active[b]) continue;
    const int n = bd.n[b];
    const int L = nlayers[b];
    int qs[6], nq = 0, gk[3], ghi[3], glo[3], ng = 0;
    int64_t slots[3];
    for (int g = 0; g < count && g < 3; ++g) {
      int64_t slot;
      int q, k;
      if (!fwd_gate(bd, arity, L, n, b, j0 + g, &slot, &q, &k)) break;
      slots[ng] = slot;
      gk[ng] = k;
      qs[nq++] = q;
      if (k == 2) qs[nq++] = q + 1;
      ghi[ng] = q;   // qubits for now, local bits below
      ++ng;
    }
    if (ng == 0) continue;
    WinSpec w;
    if (!win_build(w, n, qs, nq, n < 4 ? n : 4)) {
      if (threadIdx.x == 0) atomicOr(bd.err, KERR_BAD_GATE);
      continue;
    }
    for (int g = 0; g < ng; ++g) {
      const int q = ghi[g];
      ghi[g] = win_local(w, q);
      glo[g] = gk[g] == 2 ? win_local(w, q + 1) : 0;
    }
    __syncthreads();
    for (int g = 0; g < ng; ++g) stage_gate(gs[g], gates + bd.gate_off[b] + slots[g] * 16, gk[g], 0);
    __syncthreads();
    float2* v = psi + bd.vec_off[b];
    if (w.u == 4) rebuild_groups<4>(bd, b, n, tile, v, w, gs, gk, ghi, glo, ng);
    else if (w.u == 3) rebuild_groups<3>(bd, b, n, tile, v, w, gs, gk, ghi, glo, ng);
    else rebuild_groups<2>(bd, b, n, tile, v, w, gs, gk, ghi, glo, ng);
  }
}

static int grid_for(const BatchDev& bd) {
  int g = bd.ntiles;
  const int cap = 152 * 8;
  return g < cap ? g : cap;
}

void launch_rebuild_win(const BatchDev& bd, float2* psi, const double2* gates, const signed char* arity,
                        const int* nlayers, const int* active, int j0, int count, cudaStream_t s) {
  qm_note_launch();
  k_rebuild_win<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, psi, gates, arity, nlayers, active, j0, count);
}
