// (a) statevector -> MPS: right-to-left sequential truncated SVD to bond chi.
//
// Restates MPS.from_statevector (reference qmprs/primitives/mps.py:219-249):
// quimb's from_dense followed by tensor_network_1d_compress(max_bond=chi),
// whose density-matrix method truncates from the right and leaves a
// right-canonical MPS.  Cut c (c = n-1 .. 1) of state b holds the remainder
// M (2^c x w, w = 2 r, r = bond c+1).  Per cut:
//   k_tt_gram     Gram matrix M^H M in fp64, split over at most TT_SPLIT
//                 row ranges per state, partials reduced in order;
//   k_tt_eig      one CTA per state: parallel cyclic Jacobi (round-robin
//                 pairs) on the w x w Gram, fp64, working set in global
//                 memory (L2 resident); sort, rsum2 cutoff + max_bond,
//                 canonical phases; site tensor c;
//   k_tt_project  next remainder M V (fp32).
// k_tt_site0 stores site 0 (the last remainder, rescaled to the input norm,
// as quimb's rsum2 renormalisation does) and k_mps_contract rebuilds the
// truncated dense target, left to right.
//
// Widths: the one-block kernels take Grams up to bd.eig_wmax (128, or 64 in
// batches of at most BJ_SMALL_BATCH states); wider ones are diagonalised by
// the blocked solver (ttsvd_wide.cu).  A state whose bond exceeds the plan's
// capacity raises KERR_EIG_WIDTH and has its bond poisoned (-1); every
// later kernel of the stage skips a state whose bonds are out of range, so
// no access ever depends on an unset bond.
#include "device_common.cuh"

#define TT_CH 32
#define TT_EIG_SMEM_W 64   // widest Gram diagonalised in shared memory (3 x 65 KB)

__host__ __device__ inline int chi_eff(int chi, int n) {
  const int cap = 1 << (n / 2);
  return chi < cap ? chi : cap;
}

__device__ __forceinline__ bool bond_ok(int r, int lim) { return r >= 1 && r <= lim; }

#define TT_EPB 8   // entries per thread: a 2 x 4 block (a in {2i, 2i+1}, cc in {4j .. 4j+3})

// Entry block e of the upper triangle of a w x w Gram, ordered by column
// block j (2j + 2 blocks in column block j, capped at w / 2 rows).
__device__ __forceinline__ void gram_block(int e, int w, int* i0, int* j0) {
  const int half = w >> 1;
  int j = 0, base = 0;
  for (;; ++j) {
    const int cnt = min(half, 2 * j + 2);
    if (e < base + cnt) break;
    base += cnt;
  }
  *i0 = e - base;
  *j0 = j;
}

__device__ __forceinline__ int gram_nblocks(int w) {
  const int half = w >> 1, nj = (w + 3) / 4;
  int t = 0;
  for (int j = 0; j < nj; ++j) t += min(half, 2 * j + 2);
  return t;
}

// Upper triangle of M^H M (M = the 2^c x w remainder) per state: up to
// TT_SPLIT blocks per state take row ranges; in a block, thread t takes the
// entry block (t mod nb) and every (256 / nb)-th row of the range, sums
// exact fp32 products with compensation and flushes to fp64; the rest
// groups are then summed in fixed order through shared memory.  The last
// block of a state (ticket) sums the splits in order and mirrors the lower
// triangle.
__global__ void __launch_bounds__(BLOCK_THREADS) k_tt_gram(BatchDev bd, int step, const float2* sv,
                                                           const float2* src, const int* bonds,
                                                           double2* partials, double2* gram) {
  __shared__ double2 red[BLOCK_THREADS * TT_EPB];   // 32 KB
  const int64_t WW = (int64_t)bd.tt_w * bd.tt_w;
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    const int n = bd.n[b];
    const int c = n - 1 - step;
    if (c < 1) continue;
    const int* bond = bonds + (int64_t)b * (bd.max_n + 1);
    const int r = bond[c + 1];
    const int idx = bd.tile_idx[tile];
    if (!bond_ok(r, bd.tt_b)) {
      if (r > bd.tt_b && idx == 0 && threadIdx.x == 0) atomicOr(bd.err, KERR_EIG_WIDTH);
      continue;
    }
    const int w = 2 * r;
    if (w > bd.eig_wmax && ipow2(c) < (int64_t)w) continue;   // the row Gram (ttsvd_wide.cu)
    const int nt = bd.state_ntiles[b];
    const int nsplit = nt < TT_SPLIT ? nt : TT_SPLIT;
    const float2* m = (step == 0 ? sv : src) + bd.vec_off[b];
    const int nb = gram_nblocks(w);
    // work units: (row split, chunk of BLOCK_THREADS entry blocks), taken by
    // the state's tiles in turn, so wide Grams spread over many blocks
    const int nech = (nb + BLOCK_THREADS - 1) / BLOCK_THREADS;
    const int units = nsplit * nech;
    for (int unit = idx; unit < units; unit += nt) {
    const int split = unit % nsplit;
    int64_t lo, hi;
    tile_range(ipow2(c), split, nsplit, &lo, &hi);
    double2* part = partials + ((int64_t)b * TT_SPLIT + split) * WW;
    {
      const int e0 = (unit / nsplit) * BLOCK_THREADS;
      const int nbp = nb - e0 < BLOCK_THREADS ? nb - e0 : BLOCK_THREADS;
      const int nsub = BLOCK_THREADS / nbp;
      const int eb = threadIdx.x % nbp, sub = threadIdx.x / nbp;
      const bool act = sub < nsub;
      int bi = 0, bj = 0;
      if (act) gram_block(e0 + eb, w, &bi, &bj);
      const int a0 = 2 * bi, c0 = 4 * bj;
      double2 acc[TT_EPB];
#pragma unroll
      for (int k = 0; k < TT_EPB; ++k) acc[k] = czero();
      if (act) {
        int64_t row = lo + sub;
        while (row < hi) {
          DF re[TT_EPB], im[TT_EPB];
#pragma unroll
          for (int k = 0; k < TT_EPB; ++k) re[k] = im[k] = DF{0.f, 0.f};
          for (int f = 0; f < TT_FLUSH && row < hi; ++f, row += nsub) {
            const float2* x = m + row * w;
            float2 xa[2], xc[4];
#pragma unroll
            for (int u = 0; u < 2; ++u) xa[u] = x[a0 + u];
#pragma unroll
            for (int v = 0; v < 4; ++v) xc[v] = c0 + v < w ? x[c0 + v] : cf(0.f, 0.f);
#pragma unroll
            for (int u = 0; u < 2; ++u)
#pragma unroll
              for (int v = 0; v < 4; ++v) {
                // conj(xa) * xc
                df_add_prod(re[u * 4 + v], xa[u].x, xc[v].x);
                df_add_prod(re[u * 4 + v], xa[u].y, xc[v].y);
                df_add_prod(im[u * 4 + v], xa[u].x, xc[v].y);
                df_add_prod(im[u * 4 + v], -xa[u].y, xc[v].x);
              }
          }
#pragma unroll
          for (int k = 0; k < TT_EPB; ++k) {
            acc[k].x += (double)re[k].hi + (double)re[k].lo;
            acc[k].y += (double)im[k].hi + (double)im[k].lo;
          }
        }
      }
      // sum the row groups of each entry block in fixed order
      __syncthreads();
#pragma unroll
      for (int k = 0; k < TT_EPB; ++k) red[threadIdx.x * TT_EPB + k] = acc[k];
      __syncthreads();
      for (int o = threadIdx.x; o < nbp * TT_EPB; o += BLOCK_THREADS) {
        const int ebo = o / TT_EPB, k = o % TT_EPB;
        double2 sacc = czero();
        for (int sb = 0; sb < nsub; ++sb) sacc = cadd(sacc, red[(sb * nbp + ebo) * TT_EPB + k]);
        int gi, gj;
        gram_block(e0 + ebo, w, &gi, &gj);
        const int a = 2 * gi + k / 4, cc = 4 * gj + k % 4;
        if (a <= cc && cc < w) part[(int64_t)a * w + cc] = sacc;
      }
    }
    __syncthreads();
    if (last_tile_ticket(bd.ticket, b, units)) {
      for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
        const int a = e / w, cc = e % w;
        if (a > cc) continue;
        double2 s = czero();
        for (int t = 0; t < nsplit; ++t) s = cadd(s, ld_cg(&partials[((int64_t)b * TT_SPLIT + t) * WW + a * w + cc]));
        gram[(int64_t)b * WW + (int64_t)a * w + cc] = s;
        if (a != cc) gram[(int64_t)b * WW + (int64_t)cc * w + a] = cconj(s);
        else gram[(int64_t)b * WW + (int64_t)a * w + a] = cd(s.x, 0.0);
      }
      __syncthreads();
      if (threadIdx.x == 0) bd.ticket[b] = 0;
    }
    }   // units
  }
}

// ---- Jacobi rounds in either precision -----------------------------------------

__device__ __forceinline__ float2 jmk(float re, float im) { return cf(re, im); }
__device__ __forceinline__ double2 jmk(double re, double im) { return cd(re, im); }
template <class C, class R>
__device__ __forceinline__ C jscale(C a, R t) { return jmk(a.x * t, a.y * t); }
template <class C>
__device__ __forceinline__ C jmul(C a, C b) { return jmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <class C>
__device__ __forceinline__ C jadd(C a, C b) { return jmk(a.x + b.x, a.y + b.y); }
template <class C>
__device__ __forceinline__ C jsub(C a, C b) { return jmk(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float jsqrt(float v) { return sqrtf(v); }
__device__ __forceinline__ double jsqrt(double v) { return sqrt(v); }
__device__ __forceinline__ float jabs(float2 a) { return hypotf(a.x, a.y); }
__device__ __forceinline__ double jabs(double2 a) { return hypot(a.x, a.y); }

template <class C, class R>
struct JacobiShared {
  R c[TT_MAXW / 2];
  C se[TT_MAXW / 2], sce[TT_MAXW / 2];
  int p[TT_MAXW / 2], q[TT_MAXW / 2], flag[TT_MAXW / 2];
  int rot;
};

// Parallel cyclic Jacobi (round-robin pairing, w / 2 disjoint rotations per
// round) on the Hermitian G (row-major, stride ld), accumulating V <- V R.
// A pair rotates unless |g_pq| <= rel sqrt(|g_pp g_qq|) or |g_pq| <=
// floor_abs.  Runs whole sweeps until one makes no rotation (at most
// max_sweeps).  The block must call it uniformly.
template <class C, class R>
__device__ void jacobi_run(C* G, C* V, int w, int ld, R rel, R floor_abs, int max_sweeps, JacobiShared<C, R>& js) {
  const int half = w / 2;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    if (threadIdx.x == 0) js.rot = 0;
    __syncthreads();
    for (int k = 0; k < w - 1; ++k) {
      if (threadIdx.x < half) {
        const int i = threadIdx.x;
        const int t1 = i, t2 = w - 1 - i;
        int p = t1 == 0 ? 0 : 1 + ((t1 - 1 + k) % (w - 1));
        int q = 1 + ((t2 - 1 + k) % (w - 1));
        if (p > q) {
          const int tmp = p;
          p = q;
          q = tmp;
        }
        const C g = G[p * ld + q];
        const R ag = jabs(g);
        const R app = G[p * ld + p].x, aqq = G[q * ld + q].x;
        const int rot = !(ag == R(0) || ag <= rel * jsqrt(fabs(app * aqq)) || ag <= floor_abs);
        js.p[i] = p;
        js.q[i] = q;
        js.flag[i] = rot;
        if (rot) {
          const R zeta = (aqq - app) / (R(2) * ag);
          const R t = (zeta >= R(0) ? R(1) : R(-1)) / (fabs(zeta) + jsqrt(R(1) + zeta * zeta));
          const R cc = R(1) / jsqrt(R(1) + t * t);
          const R ss = cc * t;
          const C e = jscale(g, R(1) / ag);
          js.c[i] = cc;
          js.se[i] = jscale(e, ss);
          js.sce[i] = jscale(jmk(e.x, -e.y), ss);
          js.rot = 1;
        }
      }
      __syncthreads();
      for (int idx = threadIdx.x; idx < half * w; idx += blockDim.x) {
        const int i = idx / w, row = idx % w;
        if (!js.flag[i]) continue;
        const int p = js.p[i], q = js.q[i];
        const R cc = js.c[i];
        const C se = js.se[i], sce = js.sce[i];
        const C xp = G[row * ld + p], xq = G[row * ld + q];
        G[row * ld + p] = jsub(jscale(xp, cc), jmul(sce, xq));
        G[row * ld + q] = jadd(jmul(se, xp), jscale(xq, cc));
        const C vp = V[row * ld + p], vq = V[row * ld + q];
        V[row * ld + p] = jsub(jscale(vp, cc), jmul(sce, vq));
        V[row * ld + q] = jadd(jmul(se, vp), jscale(vq, cc));
      }
      __syncthreads();
      for (int idx = threadIdx.x; idx < half * w; idx += blockDim.x) {
        const int i = idx / w, col = idx % w;
        if (!js.flag[i]) continue;
        const int p = js.p[i], q = js.q[i];
        const R cc = js.c[i];
        const C se = js.se[i], sce = js.sce[i];
        const C xp = G[p * ld + col], xq = G[q * ld + col];
        G[p * ld + col] = jsub(jscale(xp, cc), jmul(se, xq));
        G[q * ld + col] = jadd(jmul(sce, xp), jscale(xq, cc));
      }
      __syncthreads();
      if (threadIdx.x < half && js.flag[threadIdx.x]) {
        const int p = js.p[threadIdx.x], q = js.q[threadIdx.x];
        G[p * ld + q] = jmk(R(0), R(0));
        G[q * ld + p] = jmk(R(0), R(0));
        G[p * ld + p].y = R(0);
        G[q * ld + q].y = R(0);
      }
      __syncthreads();
    }
    if (!js.rot) break;
    __syncthreads();
  }
}

// C = A^H B (adj = true) or A B, w x w row-major matrices of stride ld in
// shared memory; C is neither A nor B.
__device__ void smem_matmul(const double2* A, const double2* B, double2* Cm, int w, int ld, bool adj) {
  for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
    const int i = e / w, j = e % w;
    double2 acc = czero();
    if (adj)
      for (int k = 0; k < w; ++k) acc = cadd(acc, cmulc(A[k * ld + i], B[k * ld + j]));
    else
      for (int k = 0; k < w; ++k) acc = cadd(acc, cmul(A[i * ld + k], B[k * ld + j]));
    Cm[i * ld + j] = acc;
  }
}

// One CTA per state; G and V are row-major w x w.  For w <= TT_EIG_SMEM_W
// they live in shared memory (copied from `gram`, written back to `gram`
// and `vwork` at the end), otherwise in place in global memory: each
// Jacobi round is four block-wide phases, and shared memory takes the
// memory latency out of them.
//
// The eigenvectors are found in two precisions.  FP32 Jacobi sweeps on a
// float copy of G converge V to FP32 accuracy at the FP32 rate; V is then
// made orthonormal in FP64 by one Newton-Schulz step V <- V (3I - V^H V) / 2
// (its FP32 error of about 1e-7 leaves about 1e-14), G is replaced by the
// similar, nearly diagonal V^H G V, and the FP64 Jacobi sweeps finish from
// there, accumulating into the same V, down to `fine` of the trace.  On the
// Grams of the benchmark family this cuts the FP64 rotations from about 8.4
// sweeps' worth to about 2.2 (w = 64).  For 64 < w <= 128 the same steps
// run in global memory (L2 resident): the float copies in `scratch32` (the
// Gram partials, already reduced) and the FP64 scratch in the state's slot
// of `vsel` (written only at the end).
__global__ void __launch_bounds__(BLOCK_THREADS) k_tt_eig(BatchDev bd, int step, int* bonds, double2* gram,
                                                          double2* vwork, int max_bond, double cutoff,
                                                          double2* vsel, double2* tensors, int chi,
                                                          float2* scratch32, double fine) {
  __shared__ JacobiShared<double2, double> js64;
  __shared__ JacobiShared<float2, float> js32;
  __shared__ double s_floor;
  __shared__ double s_lam[TT_MAXW];
  __shared__ int s_perm[TT_MAXW];
  __shared__ int s_keep;
  const int64_t WW = (int64_t)bd.tt_w * bd.tt_w;
  const int b = blockIdx.x;
  if (b >= bd.B) return;
  const int n = bd.n[b];
  const int c = n - 1 - step;
  if (c < 1) return;
  int* bond = bonds + (int64_t)b * (bd.max_n + 1);
  const int r = bond[c + 1];
  if (!bond_ok(r, bd.tt_b)) {
    if (threadIdx.x == 0) bond[c] = -1;   // poison: every later step skips this state
    return;
  }
  const int w = 2 * r;
  if (w > bd.eig_wmax) return;   // diagonalised by the blocked solver (ttsvd_wide.cu)
  extern __shared__ double2 eig_sm[];
  double2* Gg = gram + (int64_t)b * WW;
  double2* Vg = vwork + (int64_t)b * WW;
  const bool in_smem = w <= TT_EIG_SMEM_W;
  const int ld = in_smem ? w + 1 : w;   // padded rows: column walks hit distinct banks
  double2* G = in_smem ? eig_sm : Gg;
  double2* V = in_smem ? eig_sm + w * ld : Vg;
  double2* Sc = in_smem ? eig_sm + 2 * w * ld : vsel + (int64_t)b * WW;   // FP64 scratch
  float2* G32 = in_smem ? reinterpret_cast<float2*>(Sc) : scratch32 + (int64_t)b * 2 * TT_SPLIT * WW;
  float2* V32 = G32 + w * ld;
  if (in_smem)
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) G[(e / w) * ld + e % w] = Gg[e];
  __syncthreads();
  // Absolute rotation floor: off-diagonals at most 1e-15 of the trace move
  // no eigenvalue by more than that (five orders below the 1e-10
  // truncation cutoff).  Without it the rounding-level null-space block of
  // a rank-deficient Gram keeps rotating until the sweep limit.
  if (threadIdx.x == 0) {
    double tr = 0.0;
    for (int i = 0; i < w; ++i) tr += fabs(G[i * ld + i].x);
    s_floor = tr;
  }
  __syncthreads();
  const double tr = s_floor;
  {
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
      const int i = e / w, j = e % w;
      const double2 g = G[i * ld + j];
      G32[i * ld + j] = cf((float)g.x, (float)g.y);
      V32[i * ld + j] = cf(i == j ? 1.f : 0.f, 0.f);
    }
    __syncthreads();
    jacobi_run<float2, float>(G32, V32, w, ld, 1e-7f, (float)(1e-7 * tr), 40, js32);
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
      const int i = e / w, j = e % w;
      V[i * ld + j] = f2d(V32[i * ld + j]);
    }
    __syncthreads();
    // Newton-Schulz: Sc = (3I - V^H V) / 2, then V <- V Sc row by row (a
    // warp per row, each lane up to four columns, written after the warp's reads)
    smem_matmul(V, V, Sc, w, ld, true);
    __syncthreads();
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
      const int i = e / w, j = e % w;
      const double2 v = Sc[i * ld + j];
      Sc[i * ld + j] = cd((i == j ? 1.5 : 0.0) - 0.5 * v.x, -0.5 * v.y);
    }
    __syncthreads();
    {
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
      for (int row = warp; row < w; row += nwarps) {
        double2 o[TT_MAXW / 32];
#pragma unroll
        for (int q = 0; q < TT_MAXW / 32; ++q) o[q] = czero();
        for (int k = 0; k < w; ++k) {
          const double2 v = V[row * ld + k];
#pragma unroll
          for (int q = 0; q < TT_MAXW / 32; ++q)
            if (lane + 32 * q < w) o[q] = cadd(o[q], cmul(v, Sc[k * ld + lane + 32 * q]));
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < TT_MAXW / 32; ++q)
          if (lane + 32 * q < w) V[row * ld + lane + 32 * q] = o[q];
      }
    }
    __syncthreads();
    // G <- V^H (G V)
    smem_matmul(G, V, Sc, w, ld, false);
    __syncthreads();
    smem_matmul(V, Sc, G, w, ld, true);
    __syncthreads();
    for (int i = threadIdx.x; i < w; i += blockDim.x) G[i * ld + i].y = 0.0;
  }
  __syncthreads();
  // After the FP32 stage the FP64 sweeps stop at 1e-13 of the trace (three
  // orders below the 1e-10 cutoff; eigenvalues move by about 1e-15 of the
  // trace against 1e-15): the remaining rotations are the null-space
  // cluster's rounding noise.
  jacobi_run<double2, double>(G, V, w, ld, 1e-15, fine * tr, 40, js64);
  if (threadIdx.x == 0) {
    for (int i = 0; i < w; ++i) { s_perm[i] = i; s_lam[i] = G[i * ld + i].x; }
    for (int i = 1; i < w; ++i) {
      const int kk = s_perm[i];
      const double key = s_lam[i];
      int j = i - 1;
      while (j >= 0 && s_lam[j] < key) { s_lam[j + 1] = s_lam[j]; s_perm[j + 1] = s_perm[j]; --j; }
      s_lam[j + 1] = key;
      s_perm[j + 1] = kk;
    }
    int keep = rank_by_cutoff(s_lam, w, cutoff, max_bond);
    if (keep > bd.tt_b) keep = bd.tt_b;
    if (c < 30 && keep > (1 << c)) keep = 1 << c;   // M has 2^c rows: rank <= 2^c
    s_keep = keep;
    bond[c] = keep;
  }
  __syncthreads();
  const int keep = s_keep;
  if (threadIdx.x < keep) phase_fix_column(V, w, ld, s_perm[threadIdx.x]);
  __syncthreads();
  double2* vs = vsel + (int64_t)b * WW;
  for (int e = threadIdx.x; e < w * keep; e += blockDim.x) {
    const int a = e / keep, col = e % keep;
    vs[(int64_t)a * bd.tt_b + col] = V[a * ld + s_perm[col]];
  }
  const int ce = chi_eff(chi, n);
  double2* ts = tensors + bd.tensor_off[b] + (int64_t)c * 2 * ce * ce;
  for (int e = threadIdx.x; e < keep * 2 * r; e += blockDim.x) {
    const int l = e / (2 * r), pr = e % (2 * r);   // e = l * 2r + (p * r + rr)
    ts[e] = cconj(V[pr * ld + s_perm[l]]);
  }
}

// Dynamic shared memory: V (TT_MAXW x TT_MAXB float2) then TT_CH rows.
__global__ void __launch_bounds__(BLOCK_THREADS) k_tt_project(BatchDev bd, int step, const float2* sv,
                                                              const float2* src, float2* dst,
                                                              const int* bonds, const double2* vsel) {
  extern __shared__ float2 sh[];
  float2* vs = sh;
  float2* xs = sh + TT_MAXW * TT_MAXB;
  const int64_t WW = (int64_t)bd.tt_w * bd.tt_w;
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    const int n = bd.n[b];
    const int c = n - 1 - step;
    if (c < 1) continue;
    const int* bond = bonds + (int64_t)b * (bd.max_n + 1);
    const int r = bond[c + 1];
    const int keep = bond[c];
    if (!bond_ok(r, bd.tt_b) || !bond_ok(keep, bd.tt_b)) continue;
    const int w = 2 * r;
    if (w > bd.eig_wmax || keep > TT_MAXB) continue;   // projected by k_cgemm
    __syncthreads();
    for (int e = threadIdx.x; e < w * keep; e += blockDim.x) {
      const double2 v = vsel[(int64_t)b * WW + (int64_t)(e / keep) * bd.tt_b + (e % keep)];
      vs[e] = cf((float)v.x, (float)v.y);
    }
    const float2* m = (step == 0 ? sv : src) + bd.vec_off[b];
    float2* o = dst + bd.vec_off[b];
    int64_t lo, hi;
    tile_range(ipow2(c), bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    for (int64_t r0 = lo; r0 < hi; r0 += TT_CH) {
      const int nr = (int)((hi - r0) < TT_CH ? (hi - r0) : TT_CH);
      __syncthreads();
      for (int e = threadIdx.x; e < nr * w; e += blockDim.x) xs[(e / w) * TT_MAXW + e % w] = m[(r0 + e / w) * w + e % w];
      __syncthreads();
      for (int e = threadIdx.x; e < nr * keep; e += blockDim.x) {
        const int rr = e / keep, col = e % keep;
        float2 acc = cf(0.f, 0.f);
        for (int a = 0; a < w; ++a) acc = fmac(acc, xs[rr * TT_MAXW + a], vs[a * keep + col]);
        o[(r0 + rr) * keep + col] = acc;
      }
    }
    __syncthreads();
  }
}

__global__ void k_tt_site0(BatchDev bd, const float2* rem0, const float2* rem1, const int* bonds,
                           double2* tensors, int chi, const double2* in_sq) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < bd.B; b += gridDim.x * blockDim.x) {
    const int n = bd.n[b];
    const int* bond = bonds + (int64_t)b * (bd.max_n + 1);
    const int r1 = bond[1];
    if (!bond_ok(r1, bd.tt_b)) continue;
    const float2* rem = (((n - 2) & 1) ? rem1 : rem0) + bd.vec_off[b];
    double nrm = 0.0;
    for (int i = 0; i < 2 * r1; ++i) nrm += cnorm2(f2d(rem[i]));
    nrm = sqrt(nrm);
    const double f = nrm > 0.0 ? sqrt(in_sq[b].x) / nrm : 0.0;
    double2* ts = tensors + bd.tensor_off[b];
    for (int i = 0; i < 2 * r1; ++i) ts[i] = cscale(f2d(rem[i]), f);
  }
}

// v_{c+1}[(x, p), r'] = sum_r v_c[x, r] A_c[r, p, r'], c = step + 1.
// Dynamic shared memory: A_c as float2, at most TT_MAXB x 2 x TT_MAXB.
__global__ void __launch_bounds__(BLOCK_THREADS) k_mps_contract(BatchDev bd, int step, const double2* tensors,
                                                                const int* bonds, int chi,
                                                                const float2* src, float2* dst_buf,
                                                                float2* target) {
  extern __shared__ float2 as[];
  for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) {
    const int b = bd.tile_state[tile];
    const int n = bd.n[b];
    const int c = step + 1;
    if (c > n - 1) continue;
    const int* bond = bonds + (int64_t)b * (bd.max_n + 1);
    const int rc = bond[c], rn = bond[c + 1];
    if (!bond_ok(rc, bd.tt_b) || !bond_ok(rn, bd.tt_b)) continue;
    if (rc > TT_MAXB || rn > TT_MAXB) continue;   // contracted by k_cgemm
    const int ce = chi_eff(chi, n);
    const double2* a = tensors + bd.tensor_off[b] + (int64_t)c * 2 * ce * ce;
    __syncthreads();
    for (int e = threadIdx.x; e < rc * 2 * rn; e += blockDim.x) as[e] = cf((float)a[e].x, (float)a[e].y);
    __syncthreads();
    const double2* t0 = tensors + bd.tensor_off[b];
    const float2* s = src + bd.vec_off[b];
    float2* o = (c == n - 1 ? target : dst_buf) + bd.vec_off[b];
    const int64_t total = ipow2(c + 1) * rn;
    int64_t lo, hi;
    tile_range(total, bd.tile_idx[tile], bd.state_ntiles[b], &lo, &hi);
    for (int64_t e = lo + threadIdx.x; e < hi; e += blockDim.x) {
      const int64_t x = e / (2 * rn);
      const int pr = (int)(e % (2 * rn));
      float2 acc = cf(0.f, 0.f);
      for (int rr = 0; rr < rc; ++rr) {
        float2 sv;
        if (step == 0) { const double2 d = t0[x * rc + rr]; sv = cf((float)d.x, (float)d.y); }
        else sv = s[x * rc + rr];
        acc = fmac(acc, sv, as[rr * 2 * rn + pr]);
      }
      o[e] = acc;
    }
  }
}

#define TT_EIG_SMEM ((size_t)3 * TT_EIG_SMEM_W * (TT_EIG_SMEM_W + 1) * sizeof(double2))   // G, V, scratch

static int grid_for(const BatchDev& bd) {
  int g = bd.ntiles;
  const int cap = 152 * 8;
  return g < cap ? g : cap;
}

void launch_tt_gram(const BatchDev& bd, int step, const float2* sv, const float2* src, const int* bonds,
                    double2* partials, double2* gram, cudaStream_t s) {
  qm_note_launch();
  k_tt_gram<<<grid_for(bd), BLOCK_THREADS, 0, s>>>(bd, step, sv, src, bonds, partials, gram);
}

void launch_tt_eig(const BatchDev& bd, int step, int* bonds, double2* gram, double2* vwork, int max_bond,
                   double cutoff, double2* vsel, double2* tensors, int chi, double2* scratch, double fine,
                   cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_tt_eig, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TT_EIG_SMEM);
    attr = true;
  }
  qm_note_launch();
  k_tt_eig<<<bd.B, BLOCK_THREADS, TT_EIG_SMEM, s>>>(bd, step, bonds, gram, vwork, max_bond, cutoff, vsel, tensors,
                                                    chi, reinterpret_cast<float2*>(scratch), fine);
}

void launch_tt_project(const BatchDev& bd, int step, const float2* sv, const float2* src, float2* dst,
                       const int* bonds, const double2* vsel, cudaStream_t s) {
  const size_t smem = sizeof(float2) * (TT_MAXW * TT_MAXB + TT_CH * TT_MAXW);
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(k_tt_project, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    configured = true;
  }
  qm_note_launch();
  k_tt_project<<<grid_for(bd), BLOCK_THREADS, smem, s>>>(bd, step, sv, src, dst, bonds, vsel);
}

void launch_tt_site0(const BatchDev& bd, const float2* rem0, const float2* rem1, const int* bonds,
                     double2* tensors, int chi, const double2* in_sq, cudaStream_t s) {
  qm_note_launch();
  k_tt_site0<<<(bd.B + 127) / 128, 128, 0, s>>>(bd, rem0, rem1, bonds, tensors, chi, in_sq);
}

void launch_mps_contract(const BatchDev& bd, int step, const double2* tensors, const int* bonds, int chi,
                         const float2* src, float2* dst_buf, float2* target, cudaStream_t s) {
  const size_t smem = sizeof(float2) * TT_MAXB * 2 * TT_MAXB;
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(k_mps_contract, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    configured = true;
  }
  qm_note_launch();
  k_mps_contract<<<grid_for(bd), BLOCK_THREADS, smem, s>>>(bd, step, tensors, bonds, chi, src, dst_buf, target);
}
