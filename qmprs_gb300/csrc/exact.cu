// Exact precision mode: the encoding path with double-float working states.
//
// The bond-2 truncations of the layer stage amplify a perturbation of the
// working state by about 3-5x per layer, so a complex64 working state
// (relative rounding 6e-8) drifts from an FP64 run by 1e-4..1e-3 after
// 10-15 layers (10 qubits, 15 layers; 14 qubits, 10 layers), and the
// sweeps inherit it.  GB300 issues FP64 at 1/64 of the FP32 rate with a
// 64-cycle dependent latency, so this mode keeps every large vector in
// double-float instead: each complex amplitude is a float4 (re hi, im hi,
// re lo, im lo) with value hi + lo, 16 bytes like complex128, and all
// arithmetic on the vectors is FP32 with error-free transformations:
//   products     a*b = ph + pl exactly (ph = fl(a*b), pl = fma(a, b, -ph));
//   sums         TwoSum of the high parts, low parts and the cross terms
//                a_hi*b_lo + a_lo*b_hi accumulated in FP32;
// which keeps about 2^-46 of relative precision on the FP32 pipes.  The
// small algebra is FP64: the eigensolvers of stage (a) and of the layer
// cuts (shared with the fast mode), the closed-form gate construction, and
// the sweep's polar factor (FP64 one-sided Jacobi, started from FP32
// sweeps; the fast mode's FP32 polar is accurate to ~1e-7, which
// rank-deficient environments carry into later steps at first order).
//
// Caller-facing statevector buffers of this mode are complex128; the plan
// converts them to double-float scratch on entry and back on exit.
//
// Kernels (all deterministic: fixed-order reductions):
//   k_x_from_d / k_x_to_d / k_x_copy / k_x_zero / k_x_scale   conversions
//   k_x_dot, k_d_dot          per-state <a|b> partials (double-float / FP64)
//   k_x_gram_tile / k_x_gram_reduce   stage (a): Gram M^H M of one state's
//                             remainder, upper-triangle tiles x row splits
//   k_x_gemm                  C = A B, A double-float, B complex128 (the
//                             projection M V and the target contraction)
//   k_x_site0                 site 0 from the last remainder
//   k_x_layer_gram / _project / _build / _fidelity   the layer stage's
//                             bond-2 cuts (the FP64 eigen kernel is shared
//                             with the fast mode)
//   k_x_apply_gate            one gate per state
//   k_x_sweep_step            a backward sweep step: peel the step's gate
//                             from the circuit state, reduce the gate's
//                             environment, and (last tile of the state)
//                             replace the gate by the conjugate of the
//                             environment's polar factor
#include "dfloat.cuh"

static int grid_for(const BatchDev& bd) {
  const int cap = 152 * 8;
  return bd.ntiles < cap ? bd.ntiles : cap;
}

// ---- conversions -------------------------------------------------------------------

__global__ void k_x_from_d(BatchDev bd, const double2* src, xc* dst) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    int64_t lo, hi;
    tile_range(ipow2(bd.n[b]), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    const double2* s = src + bd.vec_off[b];
    xc* d = dst + bd.vec_off[b];
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) d[i] = xc_from_d(s[i]);
  }
}

__global__ void k_x_to_d(BatchDev bd, const xc* src, double2* dst) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    int64_t lo, hi;
    tile_range(ipow2(bd.n[b]), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    const xc* s = src + bd.vec_off[b];
    double2* d = dst + bd.vec_off[b];
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) d[i] = xc_to_d(s[i]);
  }
}

__global__ void k_x_copy(BatchDev bd, const xc* src, xc* dst, const int* active) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    if (active && !active[b]) continue;
    int64_t lo, hi;
    tile_range(ipow2(bd.n[b]), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    const xc* s = src + bd.vec_off[b];
    xc* d = dst + bd.vec_off[b];
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) d[i] = s[i];
  }
}

__global__ void k_x_zero(BatchDev bd, xc* vec, const int* active) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    if (active && !active[b]) continue;
    int64_t lo, hi;
    tile_range(ipow2(bd.n[b]), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    xc* v = vec + bd.vec_off[b];
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) v[i] = make_float4(i == 0 ? 1.f : 0.f, 0.f, 0.f, 0.f);
  }
}

// dst = src / sqrt(sq[b].x) in double-float (the factor split once per tile).
__global__ void k_x_scale(BatchDev bd, const xc* src, xc* dst, const double2* sq) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    int64_t lo, hi;
    tile_range(ipow2(bd.n[b]), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    const double f = sq[b].x > 0.0 ? 1.0 / sqrt(sq[b].x) : 0.0;
    const float fh = __double2float_rn(f), fl = __double2float_rn(f - (double)fh);
    const xc* s = src + bd.vec_off[b];
    xc* d = dst + bd.vec_off[b];
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const xc x = s[i];
      DF re = {0.f, 0.f}, im = {0.f, 0.f};
      df_mac(re, x.x, x.z, fh, fl);
      df_mac(im, x.y, x.w, fh, fl);
      const float2 r = df_norm(re), m = df_norm(im);
      d[i] = make_float4(r.x, m.x, r.y, m.y);
    }
  }
}

// <a|b> per tile: double-float accumulation flushed to fp64, block sum in
// fixed order; k_reduce_tiles (dense.cu) sums the tiles of each state.
__global__ void __launch_bounds__(BLOCK_THREADS) k_x_dot(BatchDev bd, const xc* a, const xc* bv, double2* partials) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    int64_t lo, hi;
    tile_range(ipow2(bd.n[b]), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    const xc* pa = a + bd.vec_off[b];
    const xc* pb = bv + bd.vec_off[b];
    double acc[2] = {0.0, 0.0};
    int64_t i = lo + threadIdx.x;
    while (i < hi) {
      XA s = xa_zero();
      for (int f = 0; f < TT_FLUSH && i < hi; ++f, i += blockDim.x) xa_macc(s, pa[i], pb[i]);
      const double2 d = xa_to_d(s);
      acc[0] += d.x;
      acc[1] += d.y;
    }
    block_sum<2>(acc);
    if (threadIdx.x == 0) partials[tile] = cd(acc[0], acc[1]);
  }
}

// <a|b> per tile of two complex128 vectors, in FP64 (one pass; used for the
// caller-facing overlaps of this mode).
__global__ void __launch_bounds__(BLOCK_THREADS) k_d_dot(BatchDev bd, const double2* a, const double2* bv,
                                                         double2* partials) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    int64_t lo, hi;
    tile_range(ipow2(bd.n[b]), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    const double2* pa = a + bd.vec_off[b];
    const double2* pb = bv + bd.vec_off[b];
    double acc[2] = {0.0, 0.0};
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const double2 p = cmulc(pa[i], pb[i]);
      acc[0] += p.x;
      acc[1] += p.y;
    }
    block_sum<2>(acc);
    if (threadIdx.x == 0) partials[tile] = cd(acc[0], acc[1]);
  }
}

// ---- stage (a): Gram, projection, contraction -----------------------------------------

// Tile geometry of a w x w Gram: tiles of TI x TI entries (TI = min(w, 32),
// w even), each thread a 2 x 2 entry block; the tiles of the upper triangle
// are numbered column block by column block.
__host__ __device__ inline int x_gram_ti(int w) { return w < 32 ? w : 32; }
__host__ __device__ inline int x_gram_nt(int w) { const int ti = x_gram_ti(w); return (w + ti - 1) / ti; }

// Partial Gram sums of the rows of split blockIdx.y for tile blockIdx.x:
// part[split * WW + a * w + c] for the tile's entries with a <= c.
__global__ void __launch_bounds__(BLOCK_THREADS) k_x_gram_tile(const xc* m, int64_t rows, int w, int nsplit,
                                                               double2* part, int64_t WW) {
  __shared__ double2 red[BLOCK_THREADS * 4];
  const int TI = x_gram_ti(w), G = TI / 2, EG = G * G;
  const int RL = BLOCK_THREADS / EG;
  int ti = 0, tj = 0;
  {
    int t = blockIdx.x, j = 0;
    while (t > j) {
      t -= j + 1;
      ++j;
    }
    ti = t;
    tj = j;
  }
  const int e = threadIdx.x % EG, rl = threadIdx.x / EG;
  const int a0 = ti * TI + 2 * (e / G), c0 = tj * TI + 2 * (e % G);
  int64_t lo, hi;
  tile_range(rows, blockIdx.y, nsplit, &lo, &hi);
  double2 acc[4] = {czero(), czero(), czero(), czero()};
  if (rl < RL && a0 < w && c0 < w) {
    int64_t r = lo + rl;
    while (r < hi) {
      XA s[4] = {xa_zero(), xa_zero(), xa_zero(), xa_zero()};
      for (int f = 0; f < TT_FLUSH && r < hi; ++f, r += RL) {
        const xc* x = m + r * w;
        const xc u0 = x[a0], u1 = x[a0 + 1], v0 = x[c0], v1 = x[c0 + 1];
        xa_macc(s[0], u0, v0);
        xa_macc(s[1], u0, v1);
        xa_macc(s[2], u1, v0);
        xa_macc(s[3], u1, v1);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[k] = cadd(acc[k], xa_to_d(s[k]));
    }
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) red[threadIdx.x * 4 + k] = acc[k];
  __syncthreads();
  for (int o = threadIdx.x; o < EG * 4; o += blockDim.x) {
    const int eo = o / 4, k = o % 4;
    double2 s = czero();
    for (int l = 0; l < RL; ++l) s = cadd(s, red[(l * EG + eo) * 4 + k]);
    const int a = ti * TI + 2 * (eo / G) + k / 2, c = tj * TI + 2 * (eo % G) + k % 2;
    if (a < w && c < w && a <= c) part[(int64_t)blockIdx.y * WW + (int64_t)a * w + c] = s;
  }
}

// gram[a * w + c] = sum over splits (in order), mirrored to the lower triangle.
__global__ void k_x_gram_reduce(const double2* part, int nsplit, int w, int64_t WW, double2* gram) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)w * w; e += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(e / w), c = (int)(e % w);
    if (a > c) continue;
    double2 s = czero();
    for (int t = 0; t < nsplit; ++t) s = cadd(s, part[(int64_t)t * WW + e]);
    if (a == c) {
      gram[e] = cd(s.x, 0.0);
    } else {
      gram[e] = s;
      gram[(int64_t)c * w + a] = cconj(s);
    }
  }
}

#define XG_KC 32   // K chunk of k_x_gemm

// C (M x N, double-float, ldc) = A (M x K, double-float, lda) * B (K x N,
// complex128, ldb).  Block tile: TN = min(N, 32) columns (a power of two) x
// 256 / TN rows, one output per thread; B is split into double-float in
// shared memory one K chunk at a time; sums flushed to fp64 per chunk.
__global__ void __launch_bounds__(BLOCK_THREADS) k_x_gemm(const xc* A, int64_t lda, const double2* B, int64_t ldb,
                                                          xc* C, int64_t ldc, int64_t M, int N, int K, int TN) {
  __shared__ xc Bs[XG_KC][32];
  const int TM = BLOCK_THREADS / TN;
  const int64_t row = (int64_t)blockIdx.x * TM + threadIdx.x / TN;
  const int col = blockIdx.y * TN + threadIdx.x % TN;
  const bool act = row < M && col < N;
  double2 acc = czero();
  for (int k0 = 0; k0 < K; k0 += XG_KC) {
    __syncthreads();
    for (int e = threadIdx.x; e < XG_KC * TN; e += blockDim.x) {
      const int kk = e / TN, nn = e % TN;
      const int gk = k0 + kk, gn = blockIdx.y * TN + nn;
      Bs[kk][nn] = (gk < K && gn < N) ? xc_from_d(B[(int64_t)gk * ldb + gn]) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    if (act) {
      XA s = xa_zero();
      const int kn = K - k0 < XG_KC ? K - k0 : XG_KC;
      const xc* ar = A + row * lda + k0;
      for (int kk = 0; kk < kn; ++kk) xa_mac(s, Bs[kk][threadIdx.x % TN], ar[kk]);
      acc = cadd(acc, xa_to_d(s));
    }
  }
  if (act) C[row * ldc + col] = xc_from_d(acc);
}

// Site 0 of state b: the last remainder (2 x r1) rescaled to the input norm
// (quimb's rsum2 renormalisation), in FP64; the factor goes to *f_out.
// One block.
__global__ void k_x_site0(const xc* rem, int r1, double in_sq, double2* t0, double* f_out) {
  __shared__ double s_nrm;
  if (threadIdx.x == 0) {
    double nrm = 0.0;
    for (int i = 0; i < 2 * r1; ++i) nrm += cnorm2(xc_to_d(rem[i]));
    s_nrm = sqrt(nrm);
  }
  __syncthreads();
  const double f = s_nrm > 0.0 ? sqrt(in_sq) / s_nrm : 0.0;
  if (threadIdx.x == 0) *f_out = f;
  for (int i = threadIdx.x; i < 2 * r1; i += blockDim.x) t0[i] = cscale(xc_to_d(rem[i]), f);
}

// dst[i] = f * src[i] for count entries, f = *f_ptr (double-float product).
__global__ void k_x_scale_flat(const xc* src, xc* dst, int64_t count, const double* f_ptr) {
  const double f = *f_ptr;
  const float fh = __double2float_rn(f), fl = __double2float_rn(f - (double)fh);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const xc x = src[i];
    DF re = {0.f, 0.f}, im = {0.f, 0.f};
    df_mac(re, x.x, x.z, fh, fl);
    df_mac(im, x.y, x.w, fh, fl);
    const float2 r = df_norm(re), m = df_norm(im);
    dst[i] = make_float4(r.x, m.x, r.y, m.y);
  }
}

// Row-major complex128 -> double-float copy of count entries.
__global__ void k_x_from_d_flat(const double2* src, xc* dst, int64_t count) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = xc_from_d(src[i]);
}

// ---- (b) layer stage -----------------------------------------------------------------

// Gram rows of width W (2 or 4) of the remainder: upper triangle in
// double-float, flushed to fp64 every TT_FLUSH rows, mirrored into the
// 4 x 4 layout of the fast mode's partials (entry a * 4 + e).
template <int W>
__device__ __forceinline__ void x_gram_rows(const xc* m, int64_t lo, int64_t hi, double (&acc)[32]) {
  constexpr int NE = W * (W + 1) / 2;
  int64_t row = lo + threadIdx.x;
  while (row < hi) {
    XA s[NE];
#pragma unroll
    for (int k = 0; k < NE; ++k) s[k] = xa_zero();
    for (int f = 0; f < TT_FLUSH && row < hi; ++f, row += blockDim.x) {
      xc x[W];
#pragma unroll
      for (int a = 0; a < W; ++a) x[a] = m[row * W + a];
      int k = 0;
#pragma unroll
      for (int a = 0; a < W; ++a)
#pragma unroll
        for (int e = a; e < W; ++e, ++k) xa_macc(s[k], x[a], x[e]);
    }
    int k = 0;
#pragma unroll
    for (int a = 0; a < W; ++a)
#pragma unroll
      for (int e = a; e < W; ++e, ++k) {
        const double2 v = xa_to_d(s[k]);
        acc[2 * (a * 4 + e)] += v.x;
        acc[2 * (a * 4 + e) + 1] += v.y;
        if (e != a) {
          acc[2 * (e * 4 + a)] += v.x;
          acc[2 * (e * 4 + a) + 1] -= v.y;
        }
      }
  }
}

// Same tiles and partial layout as the fast mode's k_layer_gram, so the
// shared FP64 eigen kernel (k_layer_eig) reads them unchanged.
__global__ void __launch_bounds__(BLOCK_THREADS) k_x_layer_gram(BatchDev bd, int step, const xc* work, const xc* src,
                                                                const int* bonds, double2* partials,
                                                                const int* active) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    const int n = bd.n[b];
    const int c = n - 1 - step;
    if (c < 1 || (active && !active[b])) continue;
    const int* bond = bonds + (int64_t)b * (bd.max_n + 1);
    const int r = bond[c + 1];
    if (r != 1 && r != 2) continue;
    const xc* m = (step == 0 ? work : src) + bd.vec_off[b];
    const int vnt = layer_gram_tiles(c, bd.state_ntiles[b]);
    if (bd.tile_idx[tile] >= vnt) continue;
    int64_t lo, hi;
    tile_range(ipow2(c), bd.tile_idx[tile], vnt, &lo, &hi);
    double acc[32];
#pragma unroll
    for (int e = 0; e < 32; ++e) acc[e] = 0.0;
    if (r == 1) x_gram_rows<2>(m, lo, hi, acc);
    else x_gram_rows<4>(m, lo, hi, acc);
    warp_partial16_f64(acc, partials + ((int64_t)tile * WARPS + (threadIdx.x >> 5)) * 16);
  }
}

template <int W, int K>
__device__ __forceinline__ void x_project_rows(const xc* m, xc* o, const xc (&vm)[16], int64_t lo, int64_t hi) {
  for (int64_t row = lo + threadIdx.x; row < hi; row += blockDim.x) {
    xc x[W];
#pragma unroll
    for (int a = 0; a < W; ++a) x[a] = m[row * W + a];
#pragma unroll
    for (int col = 0; col < K; ++col) {
      XA s = xa_zero();
#pragma unroll
      for (int a = 0; a < W; ++a) xa_mac(s, vm[a * 4 + col], x[a]);
      o[row * K + col] = xa_round(s);
    }
  }
}

__global__ void __launch_bounds__(BLOCK_THREADS) k_x_layer_project(BatchDev bd, int step, const xc* work,
                                                                   const xc* src, xc* dst, const int* bonds,
                                                                   const double2* vsel, const int* active) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    const int n = bd.n[b];
    const int c = n - 1 - step;
    if (c < 1 || (active && !active[b])) continue;
    const int* bond = bonds + (int64_t)b * (bd.max_n + 1);
    const int r = bond[c + 1];
    const int keep = bond[c];
    if ((r != 1 && r != 2) || (keep != 1 && keep != 2)) continue;
    xc vm[16];
    const double2* vs = vsel + (int64_t)b * 16;
#pragma unroll
    for (int a = 0; a < 16; ++a) vm[a] = xc_from_d(vs[a]);
    const xc* m = (step == 0 ? work : src) + bd.vec_off[b];
    xc* o = dst + bd.vec_off[b];
    int64_t lo, hi;
    tile_range(ipow2(c), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    if (r == 1) {
      if (keep == 1) x_project_rows<2, 1>(m, o, vm, lo, hi);
      else x_project_rows<2, 2>(m, o, vm, lo, hi);
    } else {
      if (keep == 1) x_project_rows<4, 1>(m, o, vm, lo, hi);
      else x_project_rows<4, 2>(m, o, vm, lo, hi);
    }
  }
}

// One thread per state: site 0 from the last remainder, then the n gates
// (Ran's completion in closed form, as the fast mode's k_layer_build).
__global__ void k_x_layer_build(BatchDev bd, int layer, const xc* rem0, const xc* rem1, const int* bonds,
                                double2* site_t, double2* gates, signed char* arity, const int* active) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < bd.B; b += gridDim.x * blockDim.x) {
    if (active && !active[b]) continue;
    const int n = bd.n[b];
    const int* bond = bonds + (int64_t)b * (bd.max_n + 1);
    const xc* rem = (((n - 2) & 1) ? rem1 : rem0) + bd.vec_off[b];
    const int r1 = bond[1];
    double2* st = site_t + (int64_t)b * bd.max_n * 8;
    double nrm = 0.0;
    for (int i = 0; i < 2 * r1; ++i) nrm += cnorm2(xc_to_d(rem[i]));
    nrm = sqrt(nrm);
    for (int i = 0; i < 2 * r1; ++i) st[i] = cscale(xc_to_d(rem[i]), nrm > 0.0 ? 1.0 / nrm : 0.0);
    double worst = 0.0;
    for (int s = 0; s < n; ++s) {
      const double2* d = st + s * 8;
      const bool is_end = (s == n - 1) || bond[s + 1] == 1;
      const bool is_start = (s == 0) || bond[s] == 1;
      double2 g[16];
      for (int i = 0; i < 16; ++i) g[i] = czero();
      int k;
      if (is_end) {
        k = 1;
        if (is_start) ran_gate_single(d, g);
        else ran_gate_last(d, g);
      } else {
        k = 2;
        if (is_start) ran_gate_first(d, g);
        else ran_gate_middle(d, g);
      }
      const double err = unitarity_error(g, 1 << k);
      if (!(err <= worst)) worst = err;
      const int64_t slot = (int64_t)layer * n + s;
      double2* out = gates + bd.gate_off[b] + slot * 16;
      for (int i = 0; i < 16; ++i) out[i] = g[i];
      arity[bd.gate_off[b] / 16 + slot] = (signed char)k;
    }
    if (!(worst <= 1e-6)) atomicOr(bd.err, KERR_NONUNITARY);
  }
}

__global__ void k_x_layer_fidelity(BatchDev bd, int layer, const xc* work, int num_layers, double atol,
                                   double2* layer_fid, int* nlayers, int* active) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < bd.B; b += gridDim.x * blockDim.x) {
    if (!active[b]) continue;
    const double2 f = cconj(xc_to_d(work[bd.vec_off[b]]));
    layer_fid[(int64_t)b * num_layers + layer] = f;
    nlayers[b] = layer + 1;
    const double d = cabs_(csub(f, cd(1.0, 0.0)));
    if (d <= atol + 1e-5) active[b] = 0;
  }
}

// ---- gates and sweeps ------------------------------------------------------------------

// The selected gate (or its adjoint) of state b as double-float, in shared memory.
__device__ __forceinline__ void x_load_gate(const double2* g, int m, int adjoint, xc* gs) {
  if (threadIdx.x < m * m) {
    const int r = threadIdx.x / m, c = threadIdx.x % m;
    gs[threadIdx.x] = xc_from_d(adjoint ? cconj(g[c * m + r]) : g[r * m + c]);
  }
}

__global__ void __launch_bounds__(BLOCK_THREADS) k_x_apply_gate(BatchDev bd, xc* vec, GateSel sel) {
  __shared__ xc gs[16];
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    const int n = bd.n[b];
    int64_t slot;
    int q, k;
    if (!select_gate(sel, bd, b, n, &slot, &q, &k)) continue;
    __syncthreads();
    x_load_gate(sel.gates + bd.gate_off[b] + slot * 16, 1 << k, sel.adjoint, gs);
    __syncthreads();
    xc* v = vec + bd.vec_off[b];
    int64_t lo, hi;
    tile_range(ipow2(n - k), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    if (k == 2) {
      const int slo = n - 2 - q;
      const int64_t dlo = (int64_t)1 << slo, dhi = dlo << 1;
      for (int64_t r = lo + threadIdx.x; r < hi; r += blockDim.x) {
        const int64_t i0 = quad_base(r, slo);
        const int64_t idx[4] = {i0, i0 + dlo, i0 + dhi, i0 + dhi + dlo};
        xc x[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) x[a] = v[idx[a]];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          XA s = xa_zero();
#pragma unroll
          for (int c = 0; c < 4; ++c) xa_mac(s, gs[a * 4 + c], x[c]);
          v[idx[a]] = xa_round(s);
        }
      }
    } else {
      const int bit = n - 1 - q;
      const int64_t d = (int64_t)1 << bit;
      for (int64_t r = lo + threadIdx.x; r < hi; r += blockDim.x) {
        const int64_t i0 = pair_base(r, bit);
        const xc x0 = v[i0], x1 = v[i0 + d];
        XA s0 = xa_zero(), s1 = xa_zero();
        xa_mac(s0, gs[0], x0);
        xa_mac(s0, gs[1], x1);
        xa_mac(s1, gs[2], x0);
        xa_mac(s1, gs[3], x1);
        v[i0] = xa_round(s0);
        v[i0 + d] = xa_round(s1);
      }
    }
  }
}

// Backward sweep step `step` of every active state (the reference's
// per-gate update, qmprs/synthesis/mps_encoding/sequential.py:452-505):
//   psi <- G^H psi                      (peel the gate from the circuit state)
//   E[a][b] = sum_rest conj(t[a, rest]) psi[b, rest]
//   W = polar(E) (null directions towards conj(G)), G <- conj(W)
// The environment is reduced per tile in fixed order (warps, then tiles);
// the last tile of a state (ticket) computes the polar factor.  The target
// update t <- G_new^H t is the next launch (k_x_apply_gate).
__global__ void __launch_bounds__(BLOCK_THREADS) k_x_sweep_step(BatchDev bd, int step, xc* psi, const xc* t,
                                                                double2* gates, const signed char* arity,
                                                                const int* nlayers, const int* active,
                                                                double2* partials, double* nuc) {
  __shared__ xc gs[16];
  __shared__ double2 wred[WARPS][16];
  __shared__ double2 env[16];
  GateSel sel;
  sel.mode = SEL_SWEEP;
  sel.step = step;
  sel.layer = 0;
  sel.adjoint = 1;
  sel.gates = gates;
  sel.arity = arity;
  sel.nlayers = nlayers;
  sel.active = active;
  const int warp = threadIdx.x >> 5;
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    const int n = bd.n[b];
    int64_t slot;
    int q, k;
    if (!select_gate(sel, bd, b, n, &slot, &q, &k)) continue;
    const int m = 1 << k;
    double2* gptr = gates + bd.gate_off[b] + slot * 16;
    __syncthreads();
    x_load_gate(gptr, m, 1, gs);
    __syncthreads();
    xc* v = psi + bd.vec_off[b];
    const xc* tv = t + bd.vec_off[b];
    const int nt = bd.state_ntiles[b];
    int64_t lo, hi;
    tile_range(ipow2(n - k), bd.tile_idx[tile], nt, &lo, &hi);
    XA e[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) e[i] = xa_zero();
    if (k == 2) {
      const int slo = n - 2 - q;
      const int64_t dlo = (int64_t)1 << slo, dhi = dlo << 1;
      for (int64_t r = lo + threadIdx.x; r < hi; r += blockDim.x) {
        const int64_t i0 = quad_base(r, slo);
        const int64_t idx[4] = {i0, i0 + dlo, i0 + dhi, i0 + dhi + dlo};
        xc x[4], y[4], tt[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) x[a] = v[idx[a]];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          XA s = xa_zero();
#pragma unroll
          for (int c = 0; c < 4; ++c) xa_mac(s, gs[a * 4 + c], x[c]);
          y[a] = xa_round(s);
          v[idx[a]] = y[a];
          tt[a] = tv[idx[a]];
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int c = 0; c < 4; ++c) xa_macc(e[a * 4 + c], tt[a], y[c]);
      }
    } else {
      const int bit = n - 1 - q;
      const int64_t d = (int64_t)1 << bit;
      for (int64_t r = lo + threadIdx.x; r < hi; r += blockDim.x) {
        const int64_t i0 = pair_base(r, bit);
        const xc x0 = v[i0], x1 = v[i0 + d];
        XA s0 = xa_zero(), s1 = xa_zero();
        xa_mac(s0, gs[0], x0);
        xa_mac(s0, gs[1], x1);
        xa_mac(s1, gs[2], x0);
        xa_mac(s1, gs[3], x1);
        const xc y0 = xa_round(s0), y1 = xa_round(s1);
        v[i0] = y0;
        v[i0 + d] = y1;
        const xc t0 = tv[i0], t1 = tv[i0 + d];
        xa_macc(e[0], t0, y0);
        xa_macc(e[1], t0, y1);
        xa_macc(e[2], t1, y0);
        xa_macc(e[3], t1, y1);
      }
    }
    // per warp (fixed butterfly), then the block's warps in order
    double acc[32];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const double2 d = xa_to_d(e[i]);
      acc[2 * i] = d.x;
      acc[2 * i + 1] = d.y;
    }
    warp_partial16_f64(acc, &wred[warp][0]);
    __syncthreads();
    if (threadIdx.x < 16) {
      double2 s = czero();
      for (int w = 0; w < WARPS; ++w) s = cadd(s, wred[w][threadIdx.x]);
      partials[(int64_t)tile * 16 + threadIdx.x] = s;
    }
    __syncthreads();
    if (last_tile_ticket(bd.ticket, b, nt)) {
      const int entry = threadIdx.x >> 4, l16 = threadIdx.x & 15;
      const int t0 = bd.state_tile0[b];
      double2 s = czero();
      for (int tt = l16; tt < nt; tt += 16) s = cadd(s, ld_cg(&partials[(int64_t)(t0 + tt) * 16 + entry]));
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) {
        s.x += __shfl_down_sync(0xffffffffu, s.x, o, 16);
        s.y += __shfl_down_sync(0xffffffffu, s.y, o, 16);
      }
      if (l16 == 0) env[entry] = s;
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
        } else {
          // FP64 Hestenes polar: rank-deficient environments leave null
          // directions that follow the current gate, and an FP32 completion
          // of them would enter the later steps at first order
          for (int i = 0; i < m * m; ++i) wprev[i] = cconj(gptr[i]);
          const double nn = polar_jacobi_pre(ee, m, w, wprev);
          for (int i = 0; i < m * m; ++i) gptr[i] = cconj(w[i]);
          nuc[b] = nn;
        }
        bd.ticket[b] = 0;
      }
      __syncthreads();
    }
  }
}

// Every sweep of a state in one block (states of at most X_FUSED_MAXN
// qubits): psi and t as double-float in shared memory, the same steps as
// the launch-per-step path (k_x_apply_gate / k_x_sweep_step /
// k_sweep_finish): C|0> rebuilt gate by gate, t from the target, then per
// gate (backward order) psi <- G^H psi, E = sum conj(t) psi, the FP64
// polar factor by thread 0 (G <- conj(W)), t <- G^H t; after the sweep
// the fidelity nuc / ||target||, the sweep count and the stop at
// stop_fidelity.  The environment is reduced per warp (fixed butterfly)
// and over the warps in order.
__device__ __forceinline__ void x_fused_apply(xc* v, int n, int q, int k, const xc* gs) {
  if (k == 2) {
    const int slo = n - 2 - q;
    const int64_t dlo = (int64_t)1 << slo, dhi = dlo << 1;
    for (int64_t r = threadIdx.x; r < ipow2(n - 2); r += blockDim.x) {
      const int64_t i0 = quad_base(r, slo);
      const int64_t idx[4] = {i0, i0 + dlo, i0 + dhi, i0 + dhi + dlo};
      xc x[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) x[a] = v[idx[a]];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        XA acc = xa_zero();
#pragma unroll
        for (int c = 0; c < 4; ++c) xa_mac(acc, gs[a * 4 + c], x[c]);
        v[idx[a]] = xa_round(acc);
      }
    }
  } else {
    const int bit = n - 1 - q;
    const int64_t d = (int64_t)1 << bit;
    for (int64_t r = threadIdx.x; r < ipow2(n - 1); r += blockDim.x) {
      const int64_t i0 = pair_base(r, bit);
      const xc x0 = v[i0], x1 = v[i0 + d];
      XA s0 = xa_zero(), s1 = xa_zero();
      xa_mac(s0, gs[0], x0);
      xa_mac(s0, gs[1], x1);
      xa_mac(s1, gs[2], x0);
      xa_mac(s1, gs[3], x1);
      v[i0] = xa_round(s0);
      v[i0 + d] = xa_round(s1);
    }
  }
}

__global__ void __launch_bounds__(BLOCK_THREADS) k_x_sweep_fused(BatchDev bd, const xc* target, double2* gates,
                                                                 const signed char* arity, const int* nlayers,
                                                                 int* active, const double2* tnorm2, int num_sweeps,
                                                                 double stop_fid, double* sweep_fid,
                                                                 int* sweeps_done) {
  extern __shared__ xc xsm[];
  __shared__ xc gs[16];
  __shared__ double2 wred[WARPS][16];
  __shared__ double2 env[16];
  __shared__ double s_nuc;
  const int b = blockIdx.x;
  if (b >= bd.B) return;
  const int n = bd.n[b];
  const int64_t N = ipow2(n);
  xc* psi = xsm;
  xc* tt = xsm + N;
  const int L = nlayers[b];
  const int G = L * n;
  const int warp = threadIdx.x >> 5;
  const signed char* ar = arity + bd.gate_off[b] / 16;
  double2* gb = gates + bd.gate_off[b];
  if (threadIdx.x == 0) s_nuc = 0.0;
  for (int sw = 0; sw < num_sweeps; ++sw) {
    __syncthreads();
    if (!active[b]) break;
    // C|0>
    for (int64_t i = threadIdx.x; i < N; i += blockDim.x) psi[i] = make_float4(i == 0 ? 1.f : 0.f, 0.f, 0.f, 0.f);
    for (int j = 0; j < G; ++j) {
      const int l = L - 1 - j / n, sidx = j % n, k = ar[l * n + sidx];
      if (!((k == 1) || (k == 2 && sidx <= n - 2))) {
        if (threadIdx.x == 0) atomicOr(bd.err, KERR_BAD_GATE);
        continue;
      }
      __syncthreads();
      x_load_gate(gb + ((int64_t)l * n + sidx) * 16, 1 << k, 0, gs);
      __syncthreads();
      x_fused_apply(psi, n, sidx, k, gs);
    }
    for (int64_t i = threadIdx.x; i < N; i += blockDim.x) tt[i] = target[bd.vec_off[b] + i];
    // backward sweep
    for (int j = 0; j < G; ++j) {
      const int l = j / n, sidx = n - 1 - j % n, k = ar[l * n + sidx];
      if (!((k == 1) || (k == 2 && sidx <= n - 2))) {
        if (threadIdx.x == 0) atomicOr(bd.err, KERR_BAD_GATE);
        continue;
      }
      const int m = 1 << k;
      double2* gptr = gb + ((int64_t)l * n + sidx) * 16;
      __syncthreads();
      x_load_gate(gptr, m, 1, gs);
      __syncthreads();
      XA e[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) e[i] = xa_zero();
      if (k == 2) {
        const int slo = n - 2 - sidx;
        const int64_t dlo = (int64_t)1 << slo, dhi = dlo << 1;
        for (int64_t r = threadIdx.x; r < ipow2(n - 2); r += blockDim.x) {
          const int64_t i0 = quad_base(r, slo);
          const int64_t idx[4] = {i0, i0 + dlo, i0 + dhi, i0 + dhi + dlo};
          xc x[4], y[4], tv[4];
#pragma unroll
          for (int a = 0; a < 4; ++a) x[a] = psi[idx[a]];
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            XA acc = xa_zero();
#pragma unroll
            for (int c = 0; c < 4; ++c) xa_mac(acc, gs[a * 4 + c], x[c]);
            y[a] = xa_round(acc);
            psi[idx[a]] = y[a];
            tv[a] = tt[idx[a]];
          }
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int c = 0; c < 4; ++c) xa_macc(e[a * 4 + c], tv[a], y[c]);
        }
      } else {
        const int bit = n - 1 - sidx;
        const int64_t d = (int64_t)1 << bit;
        for (int64_t r = threadIdx.x; r < ipow2(n - 1); r += blockDim.x) {
          const int64_t i0 = pair_base(r, bit);
          const xc x0 = psi[i0], x1 = psi[i0 + d];
          XA s0 = xa_zero(), s1 = xa_zero();
          xa_mac(s0, gs[0], x0);
          xa_mac(s0, gs[1], x1);
          xa_mac(s1, gs[2], x0);
          xa_mac(s1, gs[3], x1);
          const xc y0 = xa_round(s0), y1 = xa_round(s1);
          psi[i0] = y0;
          psi[i0 + d] = y1;
          const xc t0 = tt[i0], t1 = tt[i0 + d];
          xa_macc(e[0], t0, y0);
          xa_macc(e[1], t0, y1);
          xa_macc(e[2], t1, y0);
          xa_macc(e[3], t1, y1);
        }
      }
      double acc[32];
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const double2 dv = xa_to_d(e[i]);
        acc[2 * i] = dv.x;
        acc[2 * i + 1] = dv.y;
      }
      warp_partial16_f64(acc, &wred[warp][0]);
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
        } else {
          for (int i = 0; i < m * m; ++i) wprev[i] = cconj(gptr[i]);
          const double nn = polar_jacobi_pre(ee, m, w, wprev);
          for (int i = 0; i < m * m; ++i) gptr[i] = cconj(w[i]);
          s_nuc = nn;
        }
      }
      __syncthreads();
      // t <- G_new^H t
      x_load_gate(gptr, m, 1, gs);
      __syncthreads();
      x_fused_apply(tt, n, sidx, k, gs);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const double f = s_nuc / sqrt(tnorm2[b].x);
      sweep_fid[(int64_t)b * num_sweeps + sw] = f;
      sweeps_done[b] = sw + 1;
      if (stop_fid > 0.0 && f >= stop_fid) active[b] = 0;
    }
  }
}

// ---- launches ---------------------------------------------------------------------------

void launch_x_from_d(const BatchDev& bd, const double2* src, xc* dst, cudaStream_t s) {
  qm_note_launch();
  k_x_from_d<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, src, dst);
}

void launch_x_to_d(const BatchDev& bd, const xc* src, double2* dst, cudaStream_t s) {
  qm_note_launch();
  k_x_to_d<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, src, dst);
}

void launch_x_copy(const BatchDev& bd, const xc* src, xc* dst, const int* active, cudaStream_t s) {
  qm_note_launch();
  k_x_copy<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, src, dst, active);
}

void launch_x_zero(const BatchDev& bd, xc* vec, const int* active, cudaStream_t s) {
  qm_note_launch();
  k_x_zero<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, vec, active);
}

void launch_x_dot(const BatchDev& bd, const xc* a, const xc* b, double2* partials, double2* out, cudaStream_t s) {
  qm_note_launch();
  k_x_dot<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, a, b, partials);
  launch_reduce_tiles(bd, partials, out, s);
}

void launch_d_dot(const BatchDev& bd, const double2* a, const double2* b, double2* partials, double2* out,
                  cudaStream_t s) {
  qm_note_launch();
  k_d_dot<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, a, b, partials);
  launch_reduce_tiles(bd, partials, out, s);
}

void launch_x_normalize(const BatchDev& bd, const xc* src, xc* dst, double2* partials, double2* sq, cudaStream_t s) {
  launch_x_dot(bd, src, src, partials, sq, s);
  qm_note_launch();
  k_x_scale<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, src, dst, sq);
}

void launch_x_gram(const xc* m, int64_t rows, int w, double2* part, int64_t WW, double2* gram, cudaStream_t s) {
  int nsplit = (int)std::min<int64_t>(TT_SPLIT, std::max<int64_t>(1, rows / 1024));
  const int nt = x_gram_nt(w);
  dim3 grid(nt * (nt + 1) / 2, nsplit);
  qm_note_launch();
  k_x_gram_tile<<<grid, BLOCK_THREADS, 0, s>>>(m, rows, w, nsplit, part, WW);
  const int64_t ww = (int64_t)w * w;
  const int blocks = (int)std::min<int64_t>((ww + 255) / 256, 1024);
  qm_note_launch();
  k_x_gram_reduce<<<blocks, 256, 0, s>>>(part, nsplit, w, WW, gram);
}

void launch_x_gemm(const xc* A, int64_t lda, const double2* B, int64_t ldb, xc* C, int64_t ldc, int64_t M, int N,
                   int K, cudaStream_t s) {
  int TN = 1;
  while (TN < N && TN < 32) TN <<= 1;
  const int TM = BLOCK_THREADS / TN;
  dim3 grid((unsigned)((M + TM - 1) / TM), (unsigned)((N + TN - 1) / TN));
  qm_note_launch();
  k_x_gemm<<<grid, BLOCK_THREADS, 0, s>>>(A, lda, B, ldb, C, ldc, M, N, K, TN);
}

void launch_x_site0(const xc* rem, int r1, double in_sq, double2* t0, double* f_out, cudaStream_t s) {
  qm_note_launch();
  k_x_site0<<<1, 64, 0, s>>>(rem, r1, in_sq, t0, f_out);
}

void launch_x_scale_flat(const xc* src, xc* dst, int64_t count, const double* f, cudaStream_t s) {
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((count + 255) / 256, 1024));
  qm_note_launch();
  k_x_scale_flat<<<blocks, 256, 0, s>>>(src, dst, count, f);
}

void launch_x_from_d_flat(const double2* src, xc* dst, int64_t count, cudaStream_t s) {
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((count + 255) / 256, 1024));
  qm_note_launch();
  k_x_from_d_flat<<<blocks, 256, 0, s>>>(src, dst, count);
}

void launch_x_layer_gram(const BatchDev& bd, int step, const xc* work, const xc* src, const int* bonds,
                         double2* partials, const int* active, cudaStream_t s) {
  qm_note_launch();
  k_x_layer_gram<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, step, work, src, bonds, partials, active);
}

void launch_x_layer_project(const BatchDev& bd, int step, const xc* work, const xc* src, xc* dst, const int* bonds,
                            const double2* vsel, const int* active, cudaStream_t s) {
  qm_note_launch();
  k_x_layer_project<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, step, work, src, dst, bonds, vsel, active);
}

void launch_x_layer_build(const BatchDev& bd, int layer, const xc* rem0, const xc* rem1, const int* bonds,
                          double2* site_t, double2* gates, signed char* arity, const int* active, cudaStream_t s) {
  qm_note_launch();
  k_x_layer_build<<<(bd.B + 127) / 128, 128, 0, s>>>(bd, layer, rem0, rem1, bonds, site_t, gates, arity, active);
}

void launch_x_layer_fidelity(const BatchDev& bd, int layer, const xc* work, int num_layers, double atol,
                             double2* layer_fid, int* nlayers, int* active, cudaStream_t s) {
  qm_note_launch();
  k_x_layer_fidelity<<<(bd.B + 127) / 128, 128, 0, s>>>(bd, layer, work, num_layers, atol, layer_fid, nlayers,
                                                         active);
}

void launch_x_apply_gate(const BatchDev& bd, xc* vec, const GateSel& sel, cudaStream_t s) {
  qm_note_launch();
  k_x_apply_gate<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, vec, sel);
}

void launch_x_sweep_step(const BatchDev& bd, int step, xc* psi, const xc* t, double2* gates, const signed char* arity,
                         const int* nlayers, const int* active, double2* partials, double* nuc, cudaStream_t s) {
  qm_note_launch();
  k_x_sweep_step<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, step, psi, t, gates, arity, nlayers, active, partials,
                                                        nuc);
}

int launch_x_sweep_fused(const BatchDev& bd, int max_n, const xc* target, double2* gates, const signed char* arity,
                         const int* nlayers, int* active, const double2* tnorm2, int num_sweeps, double stop_fid,
                         double* sweep_fid, int* sweeps_done, cudaStream_t s) {
  const size_t smem = 2 * sizeof(xc) * (size_t)ipow2(max_n);
  cudaError_t e = cudaFuncSetAttribute(k_x_sweep_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  qm_note_launch();
  k_x_sweep_fused<<<bd.B, BLOCK_THREADS, smem, s>>>(bd, target, gates, arity, nlayers, active, tnorm2, num_sweeps,
                                                    stop_fid, sweep_fid, sweeps_done);
  return (int)cudaGetLastError();
}
