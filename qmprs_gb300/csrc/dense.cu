// Dense state-vector kernels: |0...0> initialisation, one gate per state per
// launch, overlaps and normalised copies.  All HBM-bandwidth bound.
#include "device_common.cuh"

__global__ void k_set_zero_state(BatchDev bd, float2* vec, const int* active) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    if (active && !active[b]) continue;
    const int n = bd.n[b];
    int64_t lo, hi;
    tile_range(ipow2(n), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    float2* v = vec + bd.vec_off[b];
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) v[i] = cf(i == 0 ? 1.f : 0.f, 0.f);
  }
}

// Apply the selected gate of every state: y = G x on (q, q+1) or q.
__global__ void __launch_bounds__(BLOCK_THREADS) k_apply_gate(BatchDev bd, float2* vec, GateSel sel) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    const int n = bd.n[b];
    int64_t slot;
    int q, k;
    if (!select_gate(sel, bd, b, n, &slot, &q, &k)) continue;
    const double2* gsrc = sel.gates + bd.gate_off[b] + slot * 16;
    float2 g[16];
    float2* v = vec + bd.vec_off[b];
    int64_t lo, hi;
    tile_range(ipow2(n - k), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    if (k == 2) {
      load_gate_m<4>(gsrc, sel.adjoint, g);
      const int slo = n - 2 - q;
      const int64_t dlo = (int64_t)1 << slo, dhi = dlo << 1;
      for (int64_t r = lo + threadIdx.x; r < hi; r += blockDim.x) {
        const int64_t i0 = quad_base(r, slo);
        float2 x0 = v[i0], x1 = v[i0 + dlo], x2 = v[i0 + dhi], x3 = v[i0 + dhi + dlo];
        float2 y[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          float2 acc = cf(0.f, 0.f);
          acc = fmac(acc, g[a * 4 + 0], x0);
          acc = fmac(acc, g[a * 4 + 1], x1);
          acc = fmac(acc, g[a * 4 + 2], x2);
          acc = fmac(acc, g[a * 4 + 3], x3);
          y[a] = acc;
        }
        v[i0] = y[0];
        v[i0 + dlo] = y[1];
        v[i0 + dhi] = y[2];
        v[i0 + dhi + dlo] = y[3];
      }
    } else {
      load_gate_m<2>(gsrc, sel.adjoint, g);
      const int bit = n - 1 - q;
      const int64_t d = (int64_t)1 << bit;
      for (int64_t r = lo + threadIdx.x; r < hi; r += blockDim.x) {
        const int64_t i0 = pair_base(r, bit);
        float2 x0 = v[i0], x1 = v[i0 + d];
        float2 y0 = fmac(fmac(cf(0.f, 0.f), g[0], x0), g[1], x1);
        float2 y1 = fmac(fmac(cf(0.f, 0.f), g[2], x0), g[3], x1);
        v[i0] = y0;
        v[i0 + d] = y1;
      }
    }
  }
}

// <a|b> per state in fp64.
__global__ void __launch_bounds__(BLOCK_THREADS) k_overlap(BatchDev bd, const float2* a, const float2* bv,
                                                           double2* partials, double2* out) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    const int n = bd.n[b];
    const int nt = bd.state_ntiles[b];
    int64_t lo, hi;
    tile_range(ipow2(n), bd.tile_idx[tile], nt, &lo, &hi);
    const float2* pa = a + bd.vec_off[b];
    const float2* pb = bv + bd.vec_off[b];
    // exact fp32 products in compensated (double-float) sums, flushed to
    // fp64 every TT_FLUSH elements: fp64-accurate at fp32 throughput
    double acc[2] = {0.0, 0.0};
    int64_t i = lo + threadIdx.x;
    while (i < hi) {
      DF re = {0.f, 0.f}, im = {0.f, 0.f};
      for (int f = 0; f < TT_FLUSH && i < hi; ++f, i += blockDim.x) {
        const float2 x = pa[i], y = pb[i];
        df_add_prod(re, x.x, y.x);   // conj(x) y
        df_add_prod(re, x.y, y.y);
        df_add_prod(im, x.x, y.y);
        df_add_prod(im, -x.y, y.x);
      }
      acc[0] += (double)re.hi + (double)re.lo;
      acc[1] += (double)im.hi + (double)im.lo;
    }
    block_sum<2>(acc);
    if (threadIdx.x == 0) partials[tile] = cd(acc[0], acc[1]);
  }
}

// One warp per state: partials summed in a fixed order (lane-strided, then a
// fixed shuffle tree).
__global__ void k_reduce_tiles(BatchDev bd, const double2* partials, double2* out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int b = warp; b < bd.B; b += nwarps) {
    const int nt = bd.state_ntiles[b], t0 = bd.state_tile0[b];
    double2 s = czero();
    for (int t = lane; t < nt; t += 32) s = cadd(s, partials[t0 + t]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s.x += __shfl_down_sync(0xffffffffu, s.x, o);
      s.y += __shfl_down_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) out[b] = s;
  }
}

__global__ void k_scale_copy(BatchDev bd, const float2* src, float2* dst, const double2* sq) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    const int n = bd.n[b];
    int64_t lo, hi;
    tile_range(ipow2(n), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    const double nrm = sqrt(sq[b].x);
    const float s = nrm > 0.0 ? (float)(1.0 / nrm) : 0.f;
    const float2* ps = src + bd.vec_off[b];
    float2* pd = dst + bd.vec_off[b];
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      float2 x = ps[i];
      pd[i] = cf(x.x * s, x.y * s);
    }
  }
}

static int grid_for(const BatchDev& bd) {
  int g = bd.ntiles;
  const int cap = 152 * 8;
  return g < cap ? g : cap;
}

void launch_set_zero_state(const BatchDev& bd, float2* vec, const int* active, cudaStream_t s) {
  qm_note_launch();
  k_set_zero_state<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, vec, active);
}

void launch_apply_gate(const BatchDev& bd, float2* vec, const GateSel& sel, cudaStream_t s) {
  qm_note_launch();
  k_apply_gate<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, vec, sel);
}

void launch_reduce_tiles(const BatchDev& bd, const double2* partials, double2* out, cudaStream_t s) {
  qm_note_launch();
  k_reduce_tiles<<<(bd.B + 7) / 8, 256, 0, s>>>(bd, partials, out);
}

void launch_overlap(const BatchDev& bd, const float2* a, const float2* b, double2* partials,
                    double2* out, cudaStream_t s) {
  qm_note_launch();
  k_overlap<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, a, b, partials, out);
  launch_reduce_tiles(bd, partials, out, s);
}

// dst = src / ||src||; sq[b].x receives ||src||^2
void launch_copy_normalize(const BatchDev& bd, const float2* src, float2* dst, double2* partials,
                           double2* sq, cudaStream_t s) {
  launch_overlap(bd, src, src, partials, sq, s);
  qm_note_launch();
  k_scale_copy<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, src, dst, sq);
}

// ---- input upload ---------------------------------------------------------------

// Grid-stride copy of a pinned host buffer into device memory by the SMs
// themselves: on a coherently attached host (NVLink-C2C) the loads go
// straight to host memory, with the address translations of many SMs in
// flight at once instead of one copy engine's.  16-byte words.
__global__ void k_upload(float4* __restrict__ dst, const float4* __restrict__ src, int64_t n16) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

void launch_upload(void* dst, const void* src_dev, int64_t bytes, cudaStream_t s) {
  const int64_t n16 = bytes / 16;
  int64_t grid = (n16 + 255) / 256;
  if (grid > 152 * 8) grid = 152 * 8;
  if (grid < 1) grid = 1;
  qm_note_launch();
  k_upload<<<(int)grid, 256, 0, s>>>((float4*)dst, (const float4*)src_dev, n16);
}
