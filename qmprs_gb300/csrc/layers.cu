// (b) per-layer bond-2 truncation + Ran completion, on the dense working state.
//
// Restates MPS.generate_bond_D_unitary_layer (reference
// qmprs/primitives/mps.py:849-891) without an MPS: the bond-2 right-canonical
// form of the working state is its right-to-left truncated SVD, computed one
// cut at a time.  Cut c of state b holds the remainder M (2^c x w, w = 2 r,
// r = bond c+1, row-major, complex64).  k_layer_gram reduces its Gram matrix
// to fp64 (exact fp32 products, compensated sums), the last tile diagonalises it (Jacobi, fp64), applies quimb's
// rsum2 cutoff with max_bond 2, fixes the singular-vector phases and stores
// the site tensor; k_layer_project forms the next remainder M V.  The Gram
// sums exact fp32 products in double-float and flushes to fp64.  After the
// last cut, k_layer_build normalises site 0 and turns the n site tensors
// into n gates (mps.py:565-847) in closed form.
#include "device_common.cuh"

// Gram rows of width W (2 or 4): the upper triangle in double-float (exact
// fp32 products, compensated sums), flushed to fp64 every TT_FLUSH rows and
// mirrored into the lower triangle.
template <int W>
__device__ __forceinline__ void gram_rows(const float2* m, int64_t lo, int64_t hi, double (&acc)[32]) {
  constexpr int NE = W * (W + 1) / 2;
  int64_t row = lo + threadIdx.x;
  while (row < hi) {
    DF re[NE], im[NE];
#pragma unroll
    for (int k = 0; k < NE; ++k) re[k] = im[k] = DF{0.f, 0.f};
    for (int f = 0; f < TT_FLUSH && row < hi; ++f, row += blockDim.x) {
      float2 x[W];
#pragma unroll
      for (int a = 0; a < W; ++a) x[a] = m[row * W + a];
      int k = 0;
#pragma unroll
      for (int a = 0; a < W; ++a)
#pragma unroll
        for (int e = a; e < W; ++e, ++k) {
          df_add_prod(re[k], x[a].x, x[e].x);   // conj(x_a) x_e
          df_add_prod(re[k], x[a].y, x[e].y);
          df_add_prod(im[k], x[a].x, x[e].y);
          df_add_prod(im[k], -x[a].y, x[e].x);
        }
    }
    int k = 0;
#pragma unroll
    for (int a = 0; a < W; ++a)
#pragma unroll
      for (int e = a; e < W; ++e, ++k) {
        const double sr = (double)re[k].hi + (double)re[k].lo, si = (double)im[k].hi + (double)im[k].lo;
        acc[2 * (a * 4 + e)] += sr;
        acc[2 * (a * 4 + e) + 1] += si;
        if (e != a) {
          acc[2 * (e * 4 + a)] += sr;
          acc[2 * (e * 4 + a) + 1] -= si;
        }
      }
  }
}

__global__ void __launch_bounds__(BLOCK_THREADS) k_layer_gram(BatchDev bd, int step, const float2* work,
                                                              const float2* src, const int* bonds,
                                                              double2* partials, const int* active) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    const int n = bd.n[b];
    const int c = n - 1 - step;
    if (c < 1 || (active && !active[b])) continue;
    const int nt = bd.state_ntiles[b];
    const int* bond = bonds + (int64_t)b * (bd.max_n + 1);
    const int r = bond[c + 1];
    if (r != 1 && r != 2) continue;
    const float2* m = (step == 0 ? work : src) + bd.vec_off[b];
    const int vnt = layer_gram_tiles(c, nt);
    if (bd.tile_idx[tile] >= vnt) continue;
    int64_t lo, hi;
    tile_range(ipow2(c), bd.tile_idx[tile], vnt, &lo, &hi);
    double acc[32];
#pragma unroll
    for (int e = 0; e < 32; ++e) acc[e] = 0.0;
    if (r == 1) gram_rows<2>(m, lo, hi, acc);
    else gram_rows<4>(m, lo, hi, acc);
    warp_partial16_f64(acc, partials + ((int64_t)tile * WARPS + (threadIdx.x >> 5)) * 16);
  }
}

// One block per state: Gram reduced over the tile partials in tile order
// (16 lanes per entry, fixed shuffle tree), then thread 0 diagonalises it
// (fp64 Jacobi), applies the rsum2 cutoff with max_bond 2, fixes the
// singular-vector phases and stores V, the bond and the site tensor.
__global__ void __launch_bounds__(BLOCK_THREADS) k_layer_eig(BatchDev bd, int step, const double2* partials,
                                                             double2* vsel, int* bonds, double2* site_t,
                                                             const int* active) {
  __shared__ double2 g_s[16];
  for (int b = blockIdx.x; b < bd.B; b += gridDim.x) {
    const int n = bd.n[b];
    const int c = n - 1 - step;
    if (c < 1 || (active && !active[b])) continue;
    int* bond = bonds + (int64_t)b * (bd.max_n + 1);
    const int r = bond[c + 1];
    if (r != 1 && r != 2) continue;
    const int w = 2 * r;
    const int np = layer_gram_tiles(c, bd.state_ntiles[b]) * WARPS;   // the state's first tiles
    const int64_t p0 = (int64_t)bd.state_tile0[b] * WARPS;
    const int entry = threadIdx.x >> 4, lane = threadIdx.x & 15;
    double2 s = czero();
    for (int t = lane; t < np; t += 16) s = cadd(s, partials[(p0 + t) * 16 + entry]);
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) {
      s.x += __shfl_down_sync(0xffffffffu, s.x, o, 16);
      s.y += __shfl_down_sync(0xffffffffu, s.y, o, 16);
    }
    if (lane == 0) g_s[entry] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double2 g[16], v[16];
      double lam[4];
      for (int a = 0; a < w; ++a)
        for (int e = 0; e < w; ++e) g[a * w + e] = g_s[a * 4 + e];
      herm_eig_jacobi(g, w, v, lam);
      const int keep = rank_by_cutoff(lam, w, QM_CUTOFF, 2);
      for (int col = 0; col < keep; ++col) phase_fix_column(v, w, w, col);
      double2* vs = vsel + (int64_t)b * 16;
      for (int a = 0; a < 4; ++a)
        for (int col = 0; col < 4; ++col) vs[a * 4 + col] = (a < w && col < keep) ? v[a * w + col] : czero();
      bond[c] = keep;
      double2* st = site_t + ((int64_t)b * bd.max_n + c) * 8;
      for (int l = 0; l < keep; ++l)
        for (int p = 0; p < 2; ++p)
          for (int rr = 0; rr < r; ++rr) st[(l * 2 + p) * r + rr] = cconj(v[(p * r + rr) * w + l]);
    }
    __syncthreads();
  }
}

// M' = M V for rows of width W with K kept columns (V row-major, stride 4).
template <int W, int K>
__device__ __forceinline__ void project_rows(const float2* m, float2* o, const float2 (&vm)[16], int64_t lo,
                                             int64_t hi) {
  for (int64_t row = lo + threadIdx.x; row < hi; row += blockDim.x) {
    float2 x[W];
#pragma unroll
    for (int a = 0; a < W; ++a) x[a] = m[row * W + a];
#pragma unroll
    for (int col = 0; col < K; ++col) {
      float2 acc = cf(0.f, 0.f);
#pragma unroll
      for (int a = 0; a < W; ++a) acc = fmac(acc, x[a], vm[a * 4 + col]);
      o[row * K + col] = acc;
    }
  }
}

__global__ void __launch_bounds__(BLOCK_THREADS) k_layer_project(BatchDev bd, int step, const float2* work,
                                                                 const float2* src, float2* dst,
                                                                 const int* bonds, const double2* vsel,
                                                                 const int* active) {
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    const int n = bd.n[b];
    const int c = n - 1 - step;
    if (c < 1 || (active && !active[b])) continue;
    const int* bond = bonds + (int64_t)b * (bd.max_n + 1);
    const int r = bond[c + 1];
    const int keep = bond[c];
    if ((r != 1 && r != 2) || (keep != 1 && keep != 2)) continue;
    float2 vm[16];
    const double2* vs = vsel + (int64_t)b * 16;
#pragma unroll
    for (int a = 0; a < 16; ++a) vm[a] = cf((float)vs[a].x, (float)vs[a].y);
    const float2* m = (step == 0 ? work : src) + bd.vec_off[b];
    float2* o = dst + bd.vec_off[b];
    int64_t lo, hi;
    tile_range(ipow2(c), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    if (r == 1) {
      if (keep == 1) project_rows<2, 1>(m, o, vm, lo, hi);
      else project_rows<2, 2>(m, o, vm, lo, hi);
    } else {
      if (keep == 1) project_rows<4, 1>(m, o, vm, lo, hi);
      else project_rows<4, 2>(m, o, vm, lo, hi);
    }
  }
}

// One thread per state: site 0 from the last remainder, then the n gates.
__global__ void k_layer_build(BatchDev bd, int layer, const float2* rem0, const float2* rem1,
                              const int* bonds, double2* site_t, double2* gates, signed char* arity,
                              const int* active) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < bd.B; b += gridDim.x * blockDim.x) {
    if (active && !active[b]) continue;
    const int n = bd.n[b];
    const int* bond = bonds + (int64_t)b * (bd.max_n + 1);
    const float2* rem = (((n - 2) & 1) ? rem1 : rem0) + bd.vec_off[b];
    const int r1 = bond[1];
    double2* st = site_t + (int64_t)b * bd.max_n * 8;
    double nrm = 0.0;
    for (int i = 0; i < 2 * r1; ++i) nrm += cnorm2(f2d(rem[i]));
    nrm = sqrt(nrm);
    for (int i = 0; i < 2 * r1; ++i) st[i] = cscale(f2d(rem[i]), nrm > 0.0 ? 1.0 / nrm : 0.0);
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

// fidelity_with_zero_state (mps.py:1020-1039) and the early exit of
// Sequential._get_unitary_layers (sequential.py:390): np.isclose(f, 1, atol).
__global__ void k_layer_fidelity(BatchDev bd, int layer, const float2* work, int num_layers,
                                 double atol, double2* layer_fid, int* nlayers, int* active) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < bd.B; b += gridDim.x * blockDim.x) {
    if (!active[b]) continue;
    const double2 f = cconj(f2d(work[bd.vec_off[b]]));
    layer_fid[(int64_t)b * num_layers + layer] = f;
    nlayers[b] = layer + 1;
    const double d = cabs_(csub(f, cd(1.0, 0.0)));
    if (d <= atol + 1e-5) active[b] = 0;
  }
}

static int grid_for(const BatchDev& bd) {
  int g = bd.ntiles;
  const int cap = 152 * 8;
  return g < cap ? g : cap;
}

void launch_layer_gram(const BatchDev& bd, int step, const float2* work, const float2* src,
                       const int* bonds, double2* partials, double2* vsel, int* bonds_out,
                       double2* site_t, const int* active, cudaStream_t s) {
  (void)bonds;
  qm_note_launch();
  k_layer_gram<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, step, work, src, bonds_out, partials, active);
  launch_layer_eig(bd, step, partials, vsel, bonds_out, site_t, active, s);
}

void launch_layer_eig(const BatchDev& bd, int step, const double2* partials, double2* vsel, int* bonds,
                      double2* site_t, const int* active, cudaStream_t s) {
  qm_note_launch();
  const int blocks = bd.B < 152 * 8 ? bd.B : 152 * 8;
  k_layer_eig<<<blocks, BLOCK_THREADS, 0, s>>>(bd, step, partials, vsel, bonds, site_t, active);
}

void launch_layer_project(const BatchDev& bd, int step, const float2* work, const float2* src,
                          float2* dst, const int* bonds, const double2* vsel, const int* active,
                          cudaStream_t s) {
  qm_note_launch();
  k_layer_project<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, step, work, src, dst, bonds, vsel, active);
}

void launch_layer_build(const BatchDev& bd, int layer, const float2* rem0, const float2* rem1,
                         const int* bonds, double2* site_t, double2* gates, signed char* arity,
                         const int* active, cudaStream_t s) {
  int blocks = (bd.B + 127) / 128;
  qm_note_launch();
  k_layer_build<<<blocks, 128, 0, s>>>(bd, layer, rem0, rem1, bonds, site_t, gates, arity, active);
}

void launch_layer_fidelity(const BatchDev& bd, int layer, const float2* work, int num_layers,
                           double atol, double2* layer_fid, int* nlayers, int* active,
                           cudaStream_t s) {
  int blocks = (bd.B + 127) / 128;
  qm_note_launch();
  k_layer_fidelity<<<blocks, 128, 0, s>>>(bd, layer, work, num_layers, atol, layer_fid, nlayers, active);
}
