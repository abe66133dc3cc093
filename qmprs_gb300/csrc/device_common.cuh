// Device helpers shared by the kernels: tile ranges, block reductions, the
// last-tile ticket, index arithmetic for one- and two-qubit gates, and the
// per-step gate selection.
#pragma once

#include "internal.h"
#include "small_linalg.h"

__device__ __forceinline__ void tile_range(int64_t total, int idx, int nt, int64_t* lo, int64_t* hi) {
  int64_t per = (total + nt - 1) / nt;
  int64_t a = per * idx;
  int64_t b = a + per;
  if (a > total) a = total;
  if (b > total) b = total;
  *lo = a;
  *hi = b;
}

// Sum K doubles over the block; result valid in thread 0 (vals of thread 0).
template <int K>
__device__ __forceinline__ void block_sum(double (&vals)[K]) {
  __shared__ double red[BLOCK_THREADS / 32][K];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double v = vals[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    vals[k] = v;
  }
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) red[warp][k] = vals[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double v = 0.0;
      for (int w = 0; w < BLOCK_THREADS / 32; ++w) v += red[w][k];
      vals[k] = v;
    }
  }
  __syncthreads();
}

#define WARPS WARPS_PER_BLOCK
static_assert(WARPS_PER_BLOCK * 32 == BLOCK_THREADS, "per-warp partials assume BLOCK_THREADS / 32 warps");

// Per-warp partial of 16 complex fp32 accumulators: promoted to fp64 and
// summed over the warp with a fixed butterfly; lane i < 16 writes entry i.
__device__ __forceinline__ void warp_partial16(const float2 (&e)[16], double2* out) {
  const int lane = threadIdx.x & 31;
  double2 mine = czero();
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    double re = (double)e[i].x, im = (double)e[i].y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == i) mine = cd(re, im);
  }
  if (lane < 16) out[lane] = mine;
}

// Same for 16 complex fp64 accumulators held as 32 doubles.
__device__ __forceinline__ void warp_partial16_f64(const double (&acc)[32], double2* out) {
  const int lane = threadIdx.x & 31;
  double2 mine = czero();
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    double re = acc[2 * i], im = acc[2 * i + 1];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == i) mine = cd(re, im);
  }
  if (lane < 16) out[lane] = mine;
}

// Thread 0 publishes its partial (already written) and takes a ticket.
// Returns true in every thread of the block that finishes state b last.
__device__ __forceinline__ bool last_tile_ticket(int* ticket, int b, int nt) {
  __shared__ int s_last;
  if (threadIdx.x == 0) {
    __threadfence();
    int t = atomicAdd(&ticket[b], 1);
    s_last = (t == nt - 1);
  }
  __syncthreads();
  bool last = s_last != 0;
  if (last) __threadfence();
  return last;
}

__device__ __forceinline__ double2 ld_cg(const double2* p) { return __ldcg(p); }

// Tiles of a state that take part in the layer stage's Gram of a 2^c-row
// remainder: at least 4096 rows (16 per thread) each, so a short remainder
// is not spread over every tile of the state, each paying a full fp64 warp
// reduction.  The eigen kernel sums the partials of exactly these tiles.
__device__ __forceinline__ int layer_gram_tiles(int c, int nt) {
  const int64_t want = ((((int64_t)1) << c) + 4095) >> 12;
  return want < nt ? (int)want : nt;
}

// Index of amplitude for quad r on bits (hi, lo = hi - 1), with values (bh, bl).
__device__ __forceinline__ int64_t quad_base(int64_t r, int lo) {
  return ((r >> lo) << (lo + 2)) | (r & ((((int64_t)1) << lo) - 1));
}
__device__ __forceinline__ int64_t pair_base(int64_t r, int bit) {
  return ((r >> bit) << (bit + 1)) | (r & ((((int64_t)1) << bit) - 1));
}

// Which gate state b applies at this step (all threads of a block agree).
__device__ __forceinline__ bool select_gate(const GateSel& sel, const BatchDev& bd, int b, int n,
                                            int64_t* slot, int* q, int* k) {
  if (sel.active && !sel.active[b]) return false;
  int l, s;
  if (sel.mode == SEL_INVERSE || sel.mode == SEL_LAYER_FWD) {
    if (sel.step >= n) return false;
    l = sel.layer;
    s = sel.mode == SEL_INVERSE ? n - 1 - sel.step : sel.step;
  } else {
    int L = sel.nlayers[b];
    if (sel.step >= L * n) return false;
    if (sel.mode == SEL_REBUILD) {
      l = L - 1 - sel.step / n;
      s = sel.step % n;
    } else {
      l = sel.step / n;
      s = n - 1 - sel.step % n;
    }
  }
  *slot = (int64_t)l * n + s;
  *q = s;
  *k = sel.arity[bd.gate_off[b] / 16 + *slot];
  if (!((*k == 1) || (*k == 2 && s <= n - 2))) {   // never index with a bad slot
    if (threadIdx.x == 0) atomicOr(bd.err, KERR_BAD_GATE);
    return false;
  }
  return true;
}

// Load an M x M gate into fp32 registers, optionally as its adjoint.  M is a
// compile-time constant so every index is static and `out` stays in
// registers.
template <int M>
__device__ __forceinline__ void load_gate_m(const double2* g, int adjoint, float2 (&out)[16]) {
#pragma unroll
  for (int r = 0; r < M; ++r)
#pragma unroll
    for (int c = 0; c < M; ++c) {
      const double2 v = adjoint ? cconj(g[c * M + r]) : g[r * M + c];
      out[r * M + c] = cf((float)v.x, (float)v.y);
    }
}

__device__ __forceinline__ void load_gate(const double2* g, int m, int adjoint, float2 (&out)[16]) {
  if (m == 4) load_gate_m<4>(g, adjoint, out);
  else load_gate_m<2>(g, adjoint, out);
}

__device__ __forceinline__ float2 fmac(float2 acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x));
  acc.y = fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y));
  return acc;
}

// Compensated accumulation of exact products (double-float): p = u v is
// split exactly into ph + pl (fma), ph enters (hi, lo) through a TwoSum and
// pl and the TwoSum error land in lo.  Flushed to fp64 every TT_FLUSH rows,
// the relative error of a Gram entry is about TT_FLUSH * 2^-48 of the sum of
// |products|, far below the 1e-10 truncation cutoff the eigenvalues decide.
struct DF {
  float hi, lo;
};

// Every operation is an explicitly rounded intrinsic, so the compiler never
// contracts the product into the sum (which would break the error terms).
__device__ __forceinline__ void df_add_prod(DF& s, float u, float v) {
  const float ph = __fmul_rn(u, v);
  const float pl = __fmaf_rn(u, v, -ph);
  const float t = __fadd_rn(s.hi, ph);
  const float bv = __fsub_rn(t, s.hi);
  const float err = __fadd_rn(__fsub_rn(s.hi, __fsub_rn(t, bv)), __fsub_rn(ph, bv));
  s.lo = __fadd_rn(s.lo, __fadd_rn(err, pl));
  s.hi = t;
}

// rows summed in double-float between fp64 flushes
#define TT_FLUSH 32
