// Grouped backward sweep: the production sweep of qmprs_optimize_layers.
//
// Restates the body of Sequential._sweep_unitary_layers (reference
// qmprs/synthesis/mps_encoding/sequential.py:452-505) on dense vectors.  Per
// gate of the backward order:
//   psi <- G^H psi                                    (:460)
//   E[a][b] = sum_rest conj(t[a, rest]) psi[b, rest]  (:463)
//   new gate = conj(W), W = u @ vh of E               (:473-478, :501-505)
//   t <- new^H t                                      (:496)
//
// Consecutive steps of the backward order touch neighbouring qubits.  A
// group is a run of consecutive steps whose qubits fit a window of
// u = min(GW, n) qubits.  With x the circuit-side vector and z the
// target-side vector, both read as 2^u x rest matrices over the window, the
// cross matrix
//   M[i][k] = sum_rest conj(z[i, rest]) x[k, rest]
// carries every environment of the group: x <- Q x maps M to M Q^T,
// z <- P z maps M to conj(P) M, and the environment of a gate on window
// bits (h, l) is the partial trace E[r][c] = sum_o M[(r, o)][(c, o)].
// A group therefore costs one pass over the vectors and one small kernel:
//   k_group_pass   shared-memory tiles of 2^GT amplitudes: apply the
//                  previous group's peels to x and its new gates to z,
//                  write both back, and reduce this group's M (both
//                  products on the tensor cores, fp32 per warp over a
//                  chunk of GCHUNK tiles, fp64 across the block, one
//                  partial per chunk)
//   k_group_polar  one block per state: sum the chunk partials in chunk
//                  order, then run the group's steps on M in fp64 (target
//                  update, peel, partial trace, polar factor), keeping the
//                  replaced gates for the next pass
// Group 0 only reads (x = C|0>, z = the target); group 1 reads the target
// and writes t, so the target is never copied.  After the last group the
// vectors are not needed: the sweep's fidelity is the last step's trace.
#include <cuda_fp16.h>

#include "tile_layout.h"
#include "window.cuh"

// Gate of state b at backward step j: generated layer j / n, site
// n - 1 - j % n.
__device__ __forceinline__ bool bwd_step(const BatchDev& bd, const signed char* arity, int L, int n, int b, int j,
                                         int64_t* slot, int* q, int* k) {
  if (j < 0 || j >= L * n) return false;
  const int l = j / n, s = n - 1 - j % n;
  *slot = (int64_t)l * n + s;
  *q = s;
  *k = arity[bd.gate_off[b] / 16 + *slot];
  return (*k == 1) || (*k == 2 && s <= n - 2);
}

// Gate of state b at forward (circuit-order) position j: generated layer
// L - 1 - j / n, site j % n.
__device__ __forceinline__ bool fwd_step(const BatchDev& bd, const signed char* arity, int L, int n, int b, int j,
                                         int64_t* slot, int* q, int* k) {
  if (j < 0 || j >= L * n) return false;
  const int l = L - 1 - j / n, s = j % n;
  *slot = (int64_t)l * n + s;
  *q = s;
  *k = arity[bd.gate_off[b] / 16 + *slot];
  return (*k == 1) || (*k == 2 && s <= n - 2);
}

// Gate at step j of a step order: backward sweep order, forward circuit
// order, the inverse of one generated layer (sites n-1 .. 0, applied as
// G^H) or one layer itself (sites 0 .. n-1).
__device__ __forceinline__ bool step_gate(int mode, int layer, const BatchDev& bd, const signed char* arity, int L,
                                          int n, int b, int j, int64_t* slot, int* q, int* k) {
  if (mode == ORDER_BWD) return bwd_step(bd, arity, L, n, b, j, slot, q, k);
  if (mode == ORDER_FWD) return fwd_step(bd, arity, L, n, b, j, slot, q, k);
  if (j < 0 || j >= n) return false;
  const int s = mode == ORDER_LAYER_INV ? n - 1 - j : j;
  *slot = (int64_t)layer * n + s;
  *q = s;
  *k = arity[bd.gate_off[b] / 16 + *slot];
  return (*k == 1) || (*k == 2 && s <= n - 2);
}

__device__ __forceinline__ int order_steps(int mode, int L, int n) { return mode <= ORDER_FWD ? L * n : n; }

// Place the low bits of v, in order, at the set bits of mask (ascending).
__device__ __forceinline__ int64_t deposit_bits(int64_t v, int64_t mask) {
  int64_t r = 0;
  while (mask) {
    const int64_t bit = mask & (-mask);
    if (v & 1) r |= bit;
    v >>= 1;
    mask ^= bit;
  }
  return r;
}

// ---- group plan --------------------------------------------------------------

// Groups of consecutive steps of a step order whose qubits fit a window of
// min(GW, n) qubits.  States outside `active` (when given) get no groups.
__global__ void k_group_plan(BatchDev bd, GroupDev gd, const signed char* arity, const int* nlayers, int mode,
                             int layer, const int* active, GroupEnt* grp, int* ngroups) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < bd.B; b += gridDim.x * blockDim.x) {
    if (active && !active[b]) {
      ngroups[b] = 0;
      continue;
    }
    const int n = bd.n[b], L = mode <= ORDER_FWD ? nlayers[b] : 0, total = order_steps(mode, L, n);
    const int u = n < GW ? n : GW;
    int ng = 0, j = 0;
    while (j < total) {
      int64_t slot;
      int q, k;
      if (!step_gate(mode, layer, bd, arity, L, n, b, j, &slot, &q, &k)) {
        atomicOr(bd.err, KERR_BAD_GATE);   // skipped, as the per-gate launches do
        ++j;
        continue;
      }
      int mask = (k == 2 ? 3 : 1) << q;
      const int j0 = j++;
      while (j < total && j - j0 < GMAXSTEPS) {
        if (!step_gate(mode, layer, bd, arity, L, n, b, j, &slot, &q, &k)) break;
        const int m2 = mask | ((k == 2 ? 3 : 1) << q);
        if (__popc(m2) > u) break;
        mask = m2;
        ++j;
      }
      for (int qq = n - 1; qq >= 0 && __popc(mask) < u; --qq) mask |= 1 << qq;
      if (ng < gd.gmax) {
        GroupEnt e;
        e.j0 = j0;
        e.cnt = j - j0;
        e.qmask = mask;
        e.u = u;
        grp[(int64_t)b * gd.gmax + ng] = e;
        ++ng;
      }
    }
    ngroups[b] = ng;
  }
}

// ---- pass kernel ---------------------------------------------------------------

struct PassShared {
  int pos_mask;             // global bit positions held in the tile
  int T;                    // tile bits
  int wml_c, wml_p;         // tile-local bit masks of the current / previous window
  int npk;                  // previous group's steps
  int pk[GMAXSTEPS], phi[GMAXSTEPS], plo[GMAXSTEPS];
  int wl[GM], wlp[GM];      // window index -> swizzled tile offset
  int rl[1 << (GT - GW)];   // rest index -> swizzled tile offset (current window)
  int plp[1 << (GT - GW)];  // rest index -> swizzled tile offset (previous window)
  int d0[64], d1[64];       // global offset of tile index li: d0[li & 63] | d1[li >> 6]
  float2 gm[2][GMAXSTEPS][16];   // [peel | new][step]: the applied matrix, row-major complex
  uint4 gf[2][6][32];       // [side][Gr hi, Gr lo, Gi hi, Gi lo, -Gi hi, -Gi lo][lane]: tensor-core A fragments
  float sx, sz;             // tensor-core scales of x and z (powers of two)
};

// Dynamic shared memory: the tile of x and of z (float2 each).  Four blocks
// of four warps share an SM, so some blocks' loads overlap the others'
// arithmetic.
#define PASS_DYN_SMEM ((size_t)(2 * sizeof(float2)) * (1 << GT))
#define PASS_THREADS 128
#define PASS_BLOCKS_PER_SM 4

// tile-local bit of global position p (p must be in pos_mask)
__device__ __forceinline__ int tile_bit(int pos_mask, int p) { return __popc(pos_mask & ((1 << p) - 1)); }

// Previous group's peels on x and new gates on z, over the previous
// window: a thread owns the 2^U amplitudes of one window position and
// applies the group's gates in registers.
template <int U>
__device__ __forceinline__ void pass_apply(const PassShared& sh, float2* xs, float2* zs) {
  const int npos = 1 << (sh.T - U);
  for (int p = threadIdx.x; p < npos; p += blockDim.x) {
    const int po = sh.plp[p];
    for (int side = 0; side < 2; ++side) {
      float2* v = side ? zs : xs;
      float2 a[1 << U];
#pragma unroll
      for (int w = 0; w < (1 << U); ++w) a[w] = v[po ^ sh.wlp[w]];
      for (int s = 0; s < sh.npk; ++s)
        if (sh.pk[s]) win_apply<U>(a, sh.gm[side][s], sh.pk[s], sh.phi[s], sh.plo[s]);
#pragma unroll
      for (int w = 0; w < (1 << U); ++w) v[po ^ sh.wlp[w]] = a[w];
    }
  }
}

// acc[i * 4 + k] += conj(z[4 bi + i, r]) x[4 bk + k, r] over this thread's
// rests (the 4 x 4 block (bi, bk) of M).
template <int U>
__device__ __forceinline__ void pass_cross(const PassShared& sh, const float2* xs, const float2* zs,
                                           float2 (&acc)[16]) {
  constexpr int D = 1 << U, NBK = D / 4, NB = NBK * NBK;
  const int blk = threadIdx.x % NB, rg = threadIdx.x / NB, nrg = blockDim.x / NB;
  const int bi = blk / NBK, bk = blk % NBK;
  const int nrest = 1 << (sh.T - U);
  int wz[4], wx[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    wz[i] = sh.wl[4 * bi + i];
    wx[i] = sh.wl[4 * bk + i];
  }
  for (int r = rg; r < nrest; r += nrg) {
    const int ro = sh.rl[r];
    float2 zz[4], xx[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float2 v = zs[wz[i] ^ ro];
      zz[i] = cf(v.x, -v.y);
      xx[i] = xs[wx[i] ^ ro];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[i * 4 + k] = fmac(acc[i * 4 + k], zz[i], xx[k]);
  }
}

// Sum the accumulators over the block's rest groups (fixed order) into the
// chunk's partial (row-major 16 x 16 entries of M).  `red` aliases the tile
// buffers.
template <int U>
__device__ __forceinline__ void pass_flush(const float2 (&acc)[16], double2* red, double2* out) {
  constexpr int D = 1 << U, NBK = D / 4, NB = NBK * NBK;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int blk = threadIdx.x % NB;
  __syncthreads();   // tile buffers free
#pragma unroll
  for (int e = 0; e < 16; ++e) {
    double re = (double)acc[e].x, im = (double)acc[e].y;
#pragma unroll
    for (int o = NB; o < 32; o <<= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane < NB) red[(warp * NB + blk) * 16 + e] = cd(re, im);
  }
  __syncthreads();
  for (int ent = threadIdx.x; ent < NB * 16; ent += blockDim.x) {
    double2 s = czero();
    for (int w = 0; w < nwarps; ++w) s = cadd(s, red[(w * NB) * 16 + ent]);
    const int b = ent / 16, e = ent % 16;
    const int i = 4 * (b / NBK) + e / 4, k = 4 * (b % NBK) + e % 4;
    out[i * GM + k] = s;
  }
  __syncthreads();
}

// ---- window products on the tensor cores (4-qubit windows) ---------------------
//
// The two products of a pass, the cross matrix M = conj(Z) X^T (rows: window
// entry of z, columns: window entry of x, reduction over rests) and the
// window gates V <- G V, run as real m16n8k16 FP16 products with FP32
// accumulation:
//   Re M = Zr Xr^T + Zi Xi^T,   Im M = Zr Xi^T - Zi Xr^T,
//   Re V' = Gr Vr + (-Gi) Vi,   Im V' = Gr Vi + Gi Vr.
// Each operand is scaled by an exact power of two and split v s = hi + lo,
// hi = fp16(v s) and lo = fp16(v s - hi), both rounded to nearest (v s - hi
// is exact in FP32); a product is lo_a hi_b + hi_a lo_b + hi_a hi_b.  With
// 11-bit hi and lo the dropped lo_a lo_b and the rounding of lo leave a
// relative error of at most about 2^-21 per product (median about 2^-24),
// the same as the 3xTF32 scheme, as long as lo is a normal FP16 number: the
// scale puts typical amplitudes near 16 and keeps every |v s| <= 2^15
// (below the FP16 maximum).  Fragments come straight from the
// swizzled tile (no staging).
__device__ __forceinline__ unsigned h2_bits(__half2 h) { return *reinterpret_cast<unsigned*>(&h); }

// (a, b) = (element 2t, element 2t + 1) of an f16x2 fragment register
__device__ __forceinline__ void f16_split2(float a, float b, float sc, unsigned& hi, unsigned& lo) {
  const float as = a * sc, bs = b * sc;
  const __half2 h = __floats2half2_rn(as, bs);
  const float2 hf = __half22float2(h);
  hi = h2_bits(h);
  lo = h2_bits(__floats2half2_rn(as - hf.x, bs - hf.y));
}

__device__ __forceinline__ void mma_f16(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// c += a b, the small products first
__device__ __forceinline__ void mma3(float (&c)[4], const unsigned (&ah)[4], const unsigned (&al)[4],
                                     const unsigned (&bh)[2], const unsigned (&bl)[2]) {
  mma_f16(c, al, bh[0], bh[1]);
  mma_f16(c, ah, bl[0], bl[1]);
  mma_f16(c, ah, bh[0], bh[1]);
}

#define GATE_SCALE 256.f   // G entries (|g| <= 1) scaled into FP16's normal range

// Cross matrix of one tile, accumulated into acc (scaled by sx sz).  A warp
// owns k-steps of 16 rests; lane (g, t) reads window entries g and g + 8 at
// rests 16 s + 2t, +1, +8, +9.  acc[nt][0..3] = Zr Xr^T, Zr Xi^T, Zi Xr^T,
// Zi Xi^T for the column tiles nt = 0 (entries 0..7) and 1 (8..15).  Needs
// 2^(T - 4) >= 16 rests.
__device__ __forceinline__ void pass_cross_tc(const PassShared& sh, const float2* xs, const float2* zs,
                                              float (&acc)[2][4][4]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int gq = lane >> 2, tq = lane & 3;
  const int w0 = sh.wl[gq], w1 = sh.wl[gq + 8];
  const float sx = sh.sx, sz = sh.sz;
  const int nks = 1 << (sh.T - 8);
  for (int ks = warp; ks < nks; ks += nwarps) {
    const int* rr = sh.rl + ks * 16 + 2 * tq;
    const int r0 = rr[0], r1 = rr[1], r2 = rr[8], r3 = rr[9];
    // A = Z: reg0 (g; 2t, 2t+1), reg1 (g+8; 2t, 2t+1), reg2 (g; 2t+8, 2t+9), reg3 (g+8; 2t+8, 2t+9)
    const float2 za = zs[w0 ^ r0], zb = zs[w0 ^ r1], zc = zs[w1 ^ r0], zd = zs[w1 ^ r1];
    const float2 ze = zs[w0 ^ r2], zf = zs[w0 ^ r3], zg = zs[w1 ^ r2], zh = zs[w1 ^ r3];
    // B = X^T, column tile nt (entry 8 nt + g): reg0 (rests 2t, 2t+1), reg1 (2t+8, 2t+9)
    const float2 xa = xs[w0 ^ r0], xb = xs[w0 ^ r1], xc = xs[w1 ^ r0], xd = xs[w1 ^ r1];
    const float2 xe = xs[w0 ^ r2], xf = xs[w0 ^ r3], xg = xs[w1 ^ r2], xh = xs[w1 ^ r3];
    unsigned zrh[4], zrl[4], zih[4], zil[4];
    f16_split2(za.x, zb.x, sz, zrh[0], zrl[0]);
    f16_split2(zc.x, zd.x, sz, zrh[1], zrl[1]);
    f16_split2(ze.x, zf.x, sz, zrh[2], zrl[2]);
    f16_split2(zg.x, zh.x, sz, zrh[3], zrl[3]);
    f16_split2(za.y, zb.y, sz, zih[0], zil[0]);
    f16_split2(zc.y, zd.y, sz, zih[1], zil[1]);
    f16_split2(ze.y, zf.y, sz, zih[2], zil[2]);
    f16_split2(zg.y, zh.y, sz, zih[3], zil[3]);
    unsigned xrh[2][2], xrl[2][2], xih[2][2], xil[2][2];
    f16_split2(xa.x, xb.x, sx, xrh[0][0], xrl[0][0]);
    f16_split2(xe.x, xf.x, sx, xrh[0][1], xrl[0][1]);
    f16_split2(xc.x, xd.x, sx, xrh[1][0], xrl[1][0]);
    f16_split2(xg.x, xh.x, sx, xrh[1][1], xrl[1][1]);
    f16_split2(xa.y, xb.y, sx, xih[0][0], xil[0][0]);
    f16_split2(xe.y, xf.y, sx, xih[0][1], xil[0][1]);
    f16_split2(xc.y, xd.y, sx, xih[1][0], xil[1][0]);
    f16_split2(xg.y, xh.y, sx, xih[1][1], xil[1][1]);
#pragma unroll
    for (int nt = 0; nt < 2; ++nt) {
      mma3(acc[nt][0], zrh, zrl, xrh[nt], xrl[nt]);
      mma3(acc[nt][1], zrh, zrl, xih[nt], xil[nt]);
      mma3(acc[nt][2], zih, zil, xrh[nt], xrl[nt]);
      mma3(acc[nt][3], zih, zil, xih[nt], xil[nt]);
    }
  }
}

// V <- G V on the tensor cores, with V the 16 x position matrix of a tile
// over a 4-qubit window (wlt: window entry -> tile offset, plt: position ->
// tile offset, sc: the vector's scale) and G given as the A fragments `gf`
// of compose_gates (scaled by GATE_SCALE).  One k-step covers the 16 window
// entries.  A warp owns column tiles of 8 positions; all of its loads come
// before its stores and no other warp touches its positions.  Needs
// 2^(T - 4) >= 8.
static_assert(PASS_THREADS / 32 * 4 >= (1 << (GT - 7)), "four column tiles per warp cover a tile");
__device__ __forceinline__ void tile_apply_tc(const int* wlt, const int* plt, const uint4 (*gf)[32], int T,
                                              float sc, float2* v) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int gq = lane >> 2, tq = lane & 3;
  const int nnt = 1 << (T - 7), npos = 1 << (T - 4);   // column tiles, positions of the tile
  const uint4 frh = gf[0][lane], frl = gf[1][lane], fih = gf[2][lane], fil = gf[3][lane];
  const uint4 fnh = gf[4][lane], fnl = gf[5][lane];
  const unsigned grh[4] = {frh.x, frh.y, frh.z, frh.w}, grl[4] = {frl.x, frl.y, frl.z, frl.w};
  const unsigned gih[4] = {fih.x, fih.y, fih.z, fih.w}, gil[4] = {fil.x, fil.y, fil.z, fil.w};
  const unsigned gnh[4] = {fnh.x, fnh.y, fnh.z, fnh.w}, gnl[4] = {fnl.x, fnl.y, fnl.z, fnl.w};
  // B rows (window entries) 2t, 2t+1, 2t+8, 2t+9
  const int wa = wlt[2 * tq], wb = wlt[2 * tq + 1], wc = wlt[2 * tq + 8], wd = wlt[2 * tq + 9];
  float c[4][2][4];   // [column tile of this warp][Re, Im][fragment]
#pragma unroll
  for (int e = 0; e < 32; ++e) (&c[0][0][0])[e] = 0.f;
  // column tiles past the tile's positions (T < GT) read wrapped positions
  // and are not stored
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int nt = warp + j * nwarps;
    const int po = plt[(8 * nt + gq) & (npos - 1)];
    const float2 va = v[wa ^ po], vb = v[wb ^ po], vc = v[wc ^ po], vd = v[wd ^ po];
    unsigned rh[2], rl[2], ih[2], il[2];
    f16_split2(va.x, vb.x, sc, rh[0], rl[0]);
    f16_split2(vc.x, vd.x, sc, rh[1], rl[1]);
    f16_split2(va.y, vb.y, sc, ih[0], il[0]);
    f16_split2(vc.y, vd.y, sc, ih[1], il[1]);
    mma3(c[j][0], grh, grl, rh, rl);
    mma3(c[j][1], grh, grl, ih, il);
    mma3(c[j][0], gnh, gnl, ih, il);
    mma3(c[j][1], gih, gil, rh, rl);
  }
  // c0 (g, 2t), c1 (g, 2t + 1), c2 (g + 8, 2t), c3 (g + 8, 2t + 1), scaled
  // by sc GATE_SCALE (a power of two: the unscaling is exact)
  const float us = 1.f / (sc * GATE_SCALE);
  const int w0 = wlt[gq], w1 = wlt[gq + 8];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int nt = warp + j * nwarps;
    if (nt >= nnt) continue;
    const int p0 = plt[8 * nt + 2 * tq], p1 = plt[8 * nt + 2 * tq + 1];
    v[w0 ^ p0] = cf(c[j][0][0] * us, c[j][1][0] * us);
    v[w0 ^ p1] = cf(c[j][0][1] * us, c[j][1][1] * us);
    v[w1 ^ p0] = cf(c[j][0][2] * us, c[j][1][2] * us);
    v[w1 ^ p1] = cf(c[j][0][3] * us, c[j][1][3] * us);
  }
}

// Previous group's peels on x and new gates on z (pass kernel).
__device__ __forceinline__ void pass_apply_tc(const PassShared& sh, float2* xs, float2* zs) {
  tile_apply_tc(sh.wlp, sh.plp, sh.gf[0], sh.T, sh.sx, xs);
  tile_apply_tc(sh.wlp, sh.plp, sh.gf[1], sh.T, sh.sz, zs);
}

// The gate steps of one window: step s applies the row-major matrix gm[s]
// (arity pk[s], 0 = skip) on window bits (phi[s], plo[s]).
struct GateList {
  const int *pk, *phi, *plo;
  const float2 (*gm)[16];
  int n;
};

// Compose up to two gate lists into 16 x 16 matrices G (threads 0-31:
// matrix t / 16, column t % 16, written to `scratch` as [matrix][row][col])
// and split GATE_SCALE G into the A fragments of tile_apply_tc (one thread
// per matrix and lane): Gr hi, Gr lo, Gi hi, Gi lo, -Gi hi, -Gi lo.
// `scratch` aliases the tile buffers; the block must call this uniformly.
__device__ __forceinline__ void compose_gates(const GateList (&gl)[2], int nmat, float2* scratch,
                                              uint4 (*gf)[6][32]) {
  const int t = threadIdx.x;
  if (t < 16 * nmat) {
    const int m = t >> 4, col = t & 15;
    const GateList g = m ? gl[1] : gl[0];
    float2 a[16];
#pragma unroll
    for (int w = 0; w < 16; ++w) a[w] = cf(w == col ? 1.f : 0.f, 0.f);
    for (int s = 0; s < g.n; ++s)
      if (g.pk[s]) win_apply<4>(a, g.gm[s], g.pk[s], g.phi[s], g.plo[s]);
#pragma unroll
    for (int w = 0; w < 16; ++w) scratch[m * 256 + w * 16 + col] = a[w];
  }
  __syncthreads();
  for (int e = t; e < nmat * 32; e += blockDim.x) {
    const int m = e >> 5, lane = e & 31, gq = lane >> 2, tq = lane & 3;
    // reg0 (g; 2t, 2t+1), reg1 (g+8; 2t, 2t+1), reg2 (g; 2t+8, 2t+9), reg3 (g+8; 2t+8, 2t+9)
    const float2* G = scratch + m * 256;
    const int rows[4] = {gq, gq + 8, gq, gq + 8}, cols[4] = {2 * tq, 2 * tq, 2 * tq + 8, 2 * tq + 8};
    unsigned rh[4], rl[4], ih[4], il[4], nh[4], nl[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const float2 a = G[rows[r] * 16 + cols[r]], b = G[rows[r] * 16 + cols[r] + 1];
      f16_split2(a.x, b.x, GATE_SCALE, rh[r], rl[r]);
      f16_split2(a.y, b.y, GATE_SCALE, ih[r], il[r]);
      f16_split2(-a.y, -b.y, GATE_SCALE, nh[r], nl[r]);
    }
    gf[m][0][lane] = make_uint4(rh[0], rh[1], rh[2], rh[3]);
    gf[m][1][lane] = make_uint4(rl[0], rl[1], rl[2], rl[3]);
    gf[m][2][lane] = make_uint4(ih[0], ih[1], ih[2], ih[3]);
    gf[m][3][lane] = make_uint4(il[0], il[1], il[2], il[3]);
    gf[m][4][lane] = make_uint4(nh[0], nh[1], nh[2], nh[3]);
    gf[m][5][lane] = make_uint4(nl[0], nl[1], nl[2], nl[3]);
  }
  __syncthreads();
}

// Sum the warps' M (fixed order) into the chunk's partial, unscaled by
// 1 / (sx sz) (exact).  `red` aliases the tile buffers (needs
// nwarps * 256 double2).
__device__ __forceinline__ void pass_flush_tc(const float (&acc)[2][4][4], double us, double2* red, double2* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int gq = lane >> 2, tq = lane & 3;
  __syncthreads();   // tile buffers free
#pragma unroll
  for (int nt = 0; nt < 2; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int i = gq + (e >> 1) * 8, k = nt * 8 + 2 * tq + (e & 1);
      red[warp * GMM + i * GM + k] =
          cd(((double)acc[nt][0][e] + (double)acc[nt][3][e]) * us, ((double)acc[nt][1][e] - (double)acc[nt][2][e]) * us);
    }
  __syncthreads();
  for (int ent = threadIdx.x; ent < GMM; ent += blockDim.x) {
    double2 s = czero();
    for (int w = 0; w < nwarps; ++w) s = cadd(s, red[w * GMM + ent]);
    out[ent] = s;
  }
  __syncthreads();
}

// Tile loads: 8-byte cp.async copies straight into swizzled shared memory,
// one commit group per tile.  The rebuild pass keeps two tiles in flight
// (the next streams in while the current one is processed); the group pass
// holds one (x, z) tile pair per block and overlaps one block's loads with
// the arithmetic of the other three blocks on its SM (double-buffered at
// three blocks per SM it was slower).
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Full tiles (2^GT amplitudes): thread t handles tile indices
// li = t + PASS_THREADS u, whose offset is d0[t & 63] | d1[(t >> 6) + u PASS_THREADS / 64].
#define PASS_PER ((1 << GT) / PASS_THREADS)
static_assert(PASS_THREADS % 64 == 0 && (1 << GT) % PASS_THREADS == 0, "full-tile index split");

// swz(t + PASS_THREADS u) = swz(t) ^ swz(PASS_THREADS u) for t < PASS_THREADS
// (disjoint bits), the second term a constant of the unrolled loop.
__device__ __forceinline__ void pass_issue(const PassShared& sh, const float2* xg, const float2* zg, float2* xs,
                                           float2* zs) {
  if (sh.T == GT) {
    const int t = threadIdx.x, lo = sh.d0[t & 63], st = swz(t);
#pragma unroll
    for (int u = 0; u < PASS_PER; ++u) {
      const int o = lo | sh.d1[(t >> 6) + u * (PASS_THREADS / 64)];
      const int sl = st ^ swz(u * PASS_THREADS);
      cp_async8(xs + sl, xg + o);
      cp_async8(zs + sl, zg + o);
    }
  } else {
    for (int li = threadIdx.x; li < (1 << sh.T); li += blockDim.x) {
      const int o = sh.d0[li & 63] | sh.d1[li >> 6];
      cp_async8(xs + swz(li), xg + o);
      cp_async8(zs + swz(li), zg + o);
    }
  }
}

__device__ __forceinline__ void pass_store(const PassShared& sh, float2* xg, float2* zg, const float2* xs,
                                           const float2* zs) {
  if (sh.T == GT) {
    const int t = threadIdx.x, lo = sh.d0[t & 63], st = swz(t);
#pragma unroll
    for (int u = 0; u < PASS_PER; ++u) {
      const int o = lo | sh.d1[(t >> 6) + u * (PASS_THREADS / 64)];
      const int sl = st ^ swz(u * PASS_THREADS);
      xg[o] = xs[sl];
      zg[o] = zs[sl];
    }
  } else {
    for (int li = threadIdx.x; li < (1 << sh.T); li += blockDim.x) {
      const int o = sh.d0[li & 63] | sh.d1[li >> 6];
      xg[o] = xs[swz(li)];
      zg[o] = zs[swz(li)];
    }
  }
}

// next value with the same bits outside `mask` clear: the bits of `mask`
// read as a counter
__device__ __forceinline__ int64_t next_in_mask(int64_t x, int64_t mask) { return ((x | ~mask) + 1) & mask; }

// TC: the window products on the tensor cores (U = 4, T >= 8).
template <int U, bool TC>
__device__ __forceinline__ void pass_chunk(const BatchDev& bd, const GroupDev& gd, const PassShared& sh, float2* xs,
                                           float2* zs, int g, int b, int chunk, float2* psi, const float2* z_in,
                                           float2* z_out) {
  static_assert(!TC || U == 4, "tensor-core cross needs 16-entry windows");
  const int n = bd.n[b];
  const int64_t ntiles = (int64_t)1 << (n - sh.T);
  const int64_t rest_mask = (((int64_t)1 << n) - 1) & ~(int64_t)sh.pos_mask;
  float2* xv = psi + bd.vec_off[b];
  const float2* zv_in = z_in + bd.vec_off[b];
  float2* zv_out = z_out + bd.vec_off[b];
  float2 acc[TC ? 1 : 16];
  float tacc[2][4][4];
#pragma unroll
  for (int e = 0; e < (TC ? 1 : 16); ++e) acc[e] = cf(0.f, 0.f);
#pragma unroll
  for (int e = 0; e < 32; ++e) (&tacc[0][0][0])[e] = 0.f;
  const int64_t t0 = (int64_t)gd.chunk_idx[chunk] * GCHUNK;
  const int64_t t1 = t0 + GCHUNK < ntiles ? t0 + GCHUNK : ntiles;
  int64_t base = deposit_bits(t0, rest_mask);
  for (int64_t tt = t0; tt < t1; ++tt) {
    pass_issue(sh, xv + base, zv_in + base, xs, zs);
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    if (g > 0) {
      if constexpr (TC) pass_apply_tc(sh, xs, zs);
      else pass_apply<U>(sh, xs, zs);
      __syncthreads();
      pass_store(sh, xv + base, zv_out + base, xs, zs);
    }
    if constexpr (TC) pass_cross_tc(sh, xs, zs, tacc);
    else pass_cross<U>(sh, xs, zs, acc);
    __syncthreads();
    base = next_in_mask(base, rest_mask);
  }
  if constexpr (TC)
    pass_flush_tc(tacc, 1.0 / ((double)sh.sx * (double)sh.sz), reinterpret_cast<double2*>(xs),
                  gd.partials + (int64_t)chunk * GMM);
  else pass_flush<U>(acc, reinterpret_cast<double2*>(xs), gd.partials + (int64_t)chunk * GMM);
}

__global__ void __launch_bounds__(PASS_THREADS, PASS_BLOCKS_PER_SM) k_group_pass(BatchDev bd, GroupDev gd, int g, float2* psi,
                                                              const float2* z_in, float2* z_out,
                                                              const double2* gates, const double2* old_gates,
                                                              const signed char* arity, const int* nlayers,
                                                              const int* active, const double2* znorm) {
  extern __shared__ __align__(16) unsigned char dyn[];
  float2* xs = reinterpret_cast<float2*>(dyn);
  float2* zs = xs + (1 << GT);
  __shared__ PassShared sh;
  for (int chunk = blockIdx.x; chunk < gd.nchunks; chunk += gridDim.x) {
    const int b = gd.chunk_state[chunk];
    if (active && !active[b]) continue;
    if (g >= gd.ngroups[b]) continue;
    const int n = bd.n[b];
    const int L = nlayers[b];
    const GroupEnt cur = gd.grp[(int64_t)b * gd.gmax + g];
    const GroupEnt prv = g > 0 ? gd.grp[(int64_t)b * gd.gmax + g - 1] : cur;
    const int T = n < GT ? n : GT;
    const int U = cur.u;
    __syncthreads();   // previous chunk done with the tables
    // step data of the previous group, one thread per step; the plan only
    // groups valid steps
    if (g > 0 && threadIdx.x < prv.cnt && threadIdx.x < GMAXSTEPS) {
      const int s = threadIdx.x;
      int64_t slot;
      int q, k;
      if (bwd_step(bd, arity, L, n, b, prv.j0 + s, &slot, &q, &k)) {
        sh.pk[s] = k;
        sh.phi[s] = __popc(prv.qmask >> (q + 1));   // window qubits above q
        sh.plo[s] = k == 2 ? __popc(prv.qmask >> (q + 2)) : 0;
      } else {
        sh.pk[s] = 0;   // never applied
      }
    }
    if (threadIdx.x == 0) {
      int pm = 0;
      const int qm = cur.qmask | prv.qmask;
      for (int q = 0; q < n; ++q)
        if ((qm >> q) & 1) pm |= 1 << (n - 1 - q);
      for (int p = 0; p < n && __popc(pm) < T; ++p) pm |= 1 << p;
      int wc = 0, wp = 0;
      for (int q = 0; q < n; ++q) {
        if ((cur.qmask >> q) & 1) wc |= 1 << tile_bit(pm, n - 1 - q);
        if ((prv.qmask >> q) & 1) wp |= 1 << tile_bit(pm, n - 1 - q);
      }
      sh.pos_mask = pm;
      sh.T = T;
      sh.wml_c = wc;
      sh.wml_p = wp;   // the current window when g = 0
      sh.npk = g > 0 ? (prv.cnt < GMAXSTEPS ? prv.cnt : GMAXSTEPS) : 0;
      sh.sx = vec_scale(n, 1.0);   // x = C|0> (or its peels) has unit norm
      sh.sz = vec_scale(n, znorm ? sqrt(fabs(znorm[b].x)) : 1.0);
    }
    __syncthreads();
    const int full = (1 << T) - 1;
    {
      // split of pos_mask into its lowest six bits and the rest
      int lo6 = 0, m = sh.pos_mask;
      for (int i = 0; i < 6 && m; ++i) {
        lo6 |= m & (-m);
        m &= m - 1;
      }
      for (int j = threadIdx.x; j < 64; j += blockDim.x) {
        sh.d0[j] = deposit32(j, lo6);
        sh.d1[j] = deposit32(j, m);
      }
    }
    for (int a = threadIdx.x; a < (1 << U); a += blockDim.x) {
      sh.wl[a] = swz(deposit32(a, sh.wml_c));
      sh.wlp[a] = swz(deposit32(a, sh.wml_p));
    }
    for (int r = threadIdx.x; r < (1 << (T - U)); r += blockDim.x) {
      sh.rl[r] = swz(U == 4 && T >= 8 ? rest_offset(r, sh.wml_c, full & ~sh.wml_c) : deposit32(r, full & ~sh.wml_c));
      sh.plp[r] = swz(U == 4 && T >= 8 ? apply_pos_offset(r, sh.wml_p, full & ~sh.wml_p)
                                        : deposit32(r, full & ~sh.wml_p));
    }
    if (g > 0) {
      // stage P = (new gate)^H and Q = (replaced gate)^H of each previous
      // step, one thread per (step, entry)
      const int ns = prv.cnt < GMAXSTEPS ? prv.cnt : GMAXSTEPS;
      for (int t = threadIdx.x; t < ns * 16; t += blockDim.x) {
        const int st = t / 16, e = t % 16;
        int64_t slot;
        int q, k;
        if (!bwd_step(bd, arity, L, n, b, prv.j0 + st, &slot, &q, &k)) continue;
        const int m = 1 << k;
        if (e >= m * m) continue;
        const int r = e / m, c = e % m;
        const double2 vn = cconj(gates[bd.gate_off[b] + slot * 16 + c * m + r]);
        const double2 vo = cconj(old_gates[((int64_t)b * GMAXSTEPS + st) * 16 + c * m + r]);
        sh.gm[1][st][e] = cf((float)vn.x, (float)vn.y);
        sh.gm[0][st][e] = cf((float)vo.x, (float)vo.y);
      }
    }
    __syncthreads();
    if (U == 4 && T >= 8 && g > 0) {
      const GateList gl[2] = {{sh.pk, sh.phi, sh.plo, sh.gm[0], sh.npk}, {sh.pk, sh.phi, sh.plo, sh.gm[1], sh.npk}};
      compose_gates(gl, 2, xs, sh.gf);
    }
    if (U == 4 && T >= 8) pass_chunk<4, true>(bd, gd, sh, xs, zs, g, b, chunk, psi, z_in, z_out);
    else if (U == 4) pass_chunk<4, false>(bd, gd, sh, xs, zs, g, b, chunk, psi, z_in, z_out);
    else if (U == 3) pass_chunk<3, false>(bd, gd, sh, xs, zs, g, b, chunk, psi, z_in, z_out);
    else pass_chunk<2, false>(bd, gd, sh, xs, zs, g, b, chunk, psi, z_in, z_out);
  }
}

// ---- circuit rebuild ---------------------------------------------------------------

// C|0> before each sweep (reference qmprs/synthesis/mps_encoding/sequential.py:
// 443-447 densifies the circuit): the forward gate order cut into groups
// that fit a 4-qubit window (three consecutive gates); pass p applies
// forward groups 2p and 2p + 1 to a shared-memory tile holding both windows,
// so one read and one write of the state serve up to six gates.
struct RebuildShared {
  int pos_mask, T, nw;
  int wm[2];                       // tile-local masks of the two windows
  int nst[2];
  int pk[2][GMAXSTEPS], phi[2][GMAXSTEPS], plo[2][GMAXSTEPS];
  int wl[2][GM];                   // window index -> swizzled tile offset
  int pl[2][1 << (GT - GW)];       // position -> swizzled tile offset
  int d0[64], d1[64];
  float2 gm[2][GMAXSTEPS][16];     // the gates, row-major complex
  uint4 gf[2][6][32];              // [window][Gr hi, Gr lo, Gi hi, Gi lo, -Gi hi, -Gi lo][lane]: A fragments
  float sc;                        // tensor-core scale of the vector (a power of two)
};

template <int U>
__device__ __forceinline__ void rebuild_apply(const RebuildShared& sh, int w, float2* xs) {
  const int npos = 1 << (sh.T - U);
  for (int p = threadIdx.x; p < npos; p += blockDim.x) {
    const int po = sh.pl[w][p];
    float2 a[1 << U];
#pragma unroll
    for (int i = 0; i < (1 << U); ++i) a[i] = xs[po ^ sh.wl[w][i]];
    for (int s = 0; s < sh.nst[w]; ++s)
      if (sh.pk[w][s]) win_apply<U>(a, sh.gm[w][s], sh.pk[w][s], sh.phi[w][s], sh.plo[w][s]);
#pragma unroll
    for (int i = 0; i < (1 << U); ++i) xs[po ^ sh.wl[w][i]] = a[i];
  }
}

// TC: the windows' gates on the tensor cores (U = 4, T >= 8).
template <int U, bool TC>
__device__ __forceinline__ void rebuild_chunk(const BatchDev& bd, const GroupDev& gd, const RebuildShared& sh,
                                              float2* xs, int b, int chunk, float2* psi) {
  static_assert(!TC || U == 4, "tensor-core windows need 16 entries");
  const int n = bd.n[b];
  const int64_t ntiles = (int64_t)1 << (n - sh.T);
  const int64_t rest_mask = (((int64_t)1 << n) - 1) & ~(int64_t)sh.pos_mask;
  float2* xv = psi + bd.vec_off[b];
  const int64_t t0 = (int64_t)gd.chunk_idx[chunk] * GCHUNK;
  const int64_t t1 = t0 + GCHUNK < ntiles ? t0 + GCHUNK : ntiles;
  const int t = threadIdx.x, lo = sh.d0[t & 63], st = swz(t);
  // double-buffered: tile tt + 1 streams into the other buffer while tile
  // tt is processed (one commit group per tile)
  auto issue = [&](int64_t gbase, float2* buf) {
    const float2* xg = xv + gbase;
    if (sh.T == GT) {
#pragma unroll
      for (int u = 0; u < PASS_PER; ++u)
        cp_async8(buf + (st ^ swz(u * PASS_THREADS)), xg + (lo | sh.d1[(t >> 6) + u * (PASS_THREADS / 64)]));
    } else {
      for (int li = t; li < (1 << sh.T); li += blockDim.x)
        cp_async8(buf + swz(li), xg + (sh.d0[li & 63] | sh.d1[li >> 6]));
    }
  };
  int64_t base = deposit_bits(t0, rest_mask);
  issue(base, xs);
  cp_async_commit();
  for (int64_t tt = t0; tt < t1; ++tt) {
    float2* cur = xs + (((tt - t0) & 1) << GT);
    const int64_t nbase = next_in_mask(base, rest_mask);
    if (tt + 1 < t1) issue(nbase, xs + ((((tt - t0) + 1) & 1) << GT));
    cp_async_commit();
    cp_async_wait<1>();   // all but the newest group: tile tt has landed
    __syncthreads();
    for (int w = 0; w < sh.nw; ++w) {
      if constexpr (TC) tile_apply_tc(sh.wl[w], sh.pl[w], sh.gf[w], sh.T, sh.sc, cur);
      else rebuild_apply<U>(sh, w, cur);
      __syncthreads();
    }
    float2* xw = xv + base;
    if (sh.T == GT) {
#pragma unroll
      for (int u = 0; u < PASS_PER; ++u)
        xw[lo | sh.d1[(t >> 6) + u * (PASS_THREADS / 64)]] = cur[st ^ swz(u * PASS_THREADS)];
    } else {
      for (int li = t; li < (1 << sh.T); li += blockDim.x) xw[sh.d0[li & 63] | sh.d1[li >> 6]] = cur[swz(li)];
    }
    __syncthreads();   // cur is read out before tile tt + 2 is issued into it
    base = nbase;
  }
  cp_async_wait<0>();
}

__global__ void __launch_bounds__(PASS_THREADS, PASS_BLOCKS_PER_SM) k_rebuild_pass(BatchDev bd, GroupDev gd,
                                                                                 int pass, float2* psi,
                                                                                 const double2* gates,
                                                                                 const signed char* arity,
                                                                                 const int* nlayers,
                                                                                 const int* active, int mode,
                                                                                 int layer, bool exact) {
  extern __shared__ __align__(16) unsigned char dyn[];
  float2* xs = reinterpret_cast<float2*>(dyn);
  __shared__ RebuildShared sh;
  for (int chunk = blockIdx.x; chunk < gd.nchunks; chunk += gridDim.x) {
    const int b = gd.chunk_state[chunk];
    if (active && !active[b]) continue;
    const int ng = gd.nrgroups[b];
    const int ga = 2 * pass;
    if (ga >= ng) continue;
    const int n = bd.n[b];
    const int L = mode <= ORDER_FWD ? nlayers[b] : 0;
    const int nw = ga + 1 < ng ? 2 : 1;
    GroupEnt ge[2];
    ge[0] = gd.rgrp[(int64_t)b * gd.gmax + ga];
    ge[1] = nw == 2 ? gd.rgrp[(int64_t)b * gd.gmax + ga + 1] : ge[0];
    const int T = n < GT ? n : GT;
    const int U = ge[0].u;
    __syncthreads();   // previous chunk done with the tables
    if (threadIdx.x < 2 * GMAXSTEPS) {
      const int w = threadIdx.x / GMAXSTEPS, st = threadIdx.x % GMAXSTEPS;
      int64_t slot;
      int q, k;
      if (w < nw && st < ge[w].cnt && step_gate(mode, layer, bd, arity, L, n, b, ge[w].j0 + st, &slot, &q, &k)) {
        sh.pk[w][st] = k;
        sh.phi[w][st] = __popc(ge[w].qmask >> (q + 1));
        sh.plo[w][st] = k == 2 ? __popc(ge[w].qmask >> (q + 2)) : 0;
      } else {
        sh.pk[w][st] = 0;
      }
    }
    if (threadIdx.x == 0) {
      int pm = 0;
      const int qm = ge[0].qmask | ge[1].qmask;
      for (int q = 0; q < n; ++q)
        if ((qm >> q) & 1) pm |= 1 << (n - 1 - q);
      for (int p = 0; p < n && __popc(pm) < T; ++p) pm |= 1 << p;
      for (int w = 0; w < 2; ++w) {
        int m = 0;
        for (int q = 0; q < n; ++q)
          if ((ge[w].qmask >> q) & 1) m |= 1 << tile_bit(pm, n - 1 - q);
        sh.wm[w] = m;
        sh.nst[w] = ge[w].cnt < GMAXSTEPS ? ge[w].cnt : GMAXSTEPS;
      }
      sh.pos_mask = pm;
      sh.T = T;
      sh.nw = nw;
      sh.sc = vec_scale(n, 1.0);   // C|0> and the normalised working vector of the layer stage
    }
    __syncthreads();
    const int full = (1 << T) - 1;
    {
      int lo6 = 0, m = sh.pos_mask;
      for (int i = 0; i < 6 && m; ++i) {
        lo6 |= m & (-m);
        m &= m - 1;
      }
      for (int j = threadIdx.x; j < 64; j += blockDim.x) {
        sh.d0[j] = deposit32(j, lo6);
        sh.d1[j] = deposit32(j, m);
      }
    }
    for (int t = threadIdx.x; t < 2 * (1 << U); t += blockDim.x) {
      const int w = t >> U, a = t & ((1 << U) - 1);
      sh.wl[w][a] = swz(deposit32(a, sh.wm[w]));
    }
    for (int t = threadIdx.x; t < 2 * (1 << (T - U)); t += blockDim.x) {
      const int w = t / (1 << (T - U)), r = t % (1 << (T - U));
      sh.pl[w][r] = swz(U == 4 && T >= 8 && !exact ? apply_pos_offset(r, sh.wm[w], full & ~sh.wm[w])
                                         : deposit32(r, full & ~sh.wm[w]));
    }
    for (int t = threadIdx.x; t < 2 * GMAXSTEPS * 16; t += blockDim.x) {
      const int w = t / (GMAXSTEPS * 16), st = (t / 16) % GMAXSTEPS, e = t % 16;
      int64_t slot;
      int q, k;
      if (w >= nw || st >= ge[w].cnt || !step_gate(mode, layer, bd, arity, L, n, b, ge[w].j0 + st, &slot, &q, &k))
        continue;
      const int m = 1 << k;
      if (e >= m * m) continue;
      const int r = e / m, c = e % m;
      const double2 v = mode == ORDER_LAYER_INV ? cconj(gates[bd.gate_off[b] + slot * 16 + c * m + r])
                                                : gates[bd.gate_off[b] + slot * 16 + e];
      sh.gm[w][st][e] = cf((float)v.x, (float)v.y);
    }
    __syncthreads();
    if (U == 4 && T >= 8 && !exact) {
      const GateList gl[2] = {{sh.pk[0], sh.phi[0], sh.plo[0], sh.gm[0], sh.nst[0]},
                              {sh.pk[1], sh.phi[1], sh.plo[1], sh.gm[1], sh.nst[1]}};
      compose_gates(gl, nw, xs, sh.gf);
      rebuild_chunk<4, true>(bd, gd, sh, xs, b, chunk, psi);
    } else if (U == 4) rebuild_chunk<4, false>(bd, gd, sh, xs, b, chunk, psi);
    else if (U == 3) rebuild_chunk<3, false>(bd, gd, sh, xs, b, chunk, psi);
    else rebuild_chunk<2, false>(bd, gd, sh, xs, b, chunk, psi);
  }
}

// ---- per-group polar kernel ------------------------------------------------------

// M <- G^T M on the rows of gate bits (h, l): the target-side update z <- P z
// with P = G^H maps M to conj(P) M = G^T M.
__device__ void m_rows(double2* M, int D, const double2* G, int k, int h, int l) {
  if (k == 2) {
    const int items = D * (D / 4);
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
      const int col = it % D, o = it / D;
      int ob = 0, kk = 0;
      for (int bit = 0; (1 << bit) < D; ++bit) {
        if (bit == h || bit == l) continue;
        ob |= ((o >> kk) & 1) << bit;
        ++kk;
      }
      const int idx[4] = {ob, ob | (1 << l), ob | (1 << h), ob | (1 << h) | (1 << l)};
      double2 x[4], y[4];
      for (int r = 0; r < 4; ++r) x[r] = M[idx[r] * GM + col];
      for (int r = 0; r < 4; ++r) {
        double2 s = czero();
        for (int rp = 0; rp < 4; ++rp) s = cadd(s, cmul(G[rp * 4 + r], x[rp]));
        y[r] = s;
      }
      for (int r = 0; r < 4; ++r) M[idx[r] * GM + col] = y[r];
    }
  } else {
    const int items = D * (D / 2);
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
      const int col = it % D, o = it / D;
      const int ob = ((o >> h) << (h + 1)) | (o & ((1 << h) - 1));
      const double2 x0 = M[ob * GM + col], x1 = M[(ob | (1 << h)) * GM + col];
      M[ob * GM + col] = cadd(cmul(G[0], x0), cmul(G[2], x1));
      M[(ob | (1 << h)) * GM + col] = cadd(cmul(G[1], x0), cmul(G[3], x1));
    }
  }
}

// M <- M Q^T on the columns of gate bits (h, l), Q = G^H: the circuit-side
// peel x <- Q x.  (M Q^T)[i][c] = sum_c' M[i][c'] conj(G[c'][c]).
__device__ void m_cols(double2* M, int D, const double2* G, int k, int h, int l) {
  if (k == 2) {
    const int items = D * (D / 4);
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
      const int row = it % D, o = it / D;
      int ob = 0, kk = 0;
      for (int bit = 0; (1 << bit) < D; ++bit) {
        if (bit == h || bit == l) continue;
        ob |= ((o >> kk) & 1) << bit;
        ++kk;
      }
      const int idx[4] = {ob, ob | (1 << l), ob | (1 << h), ob | (1 << h) | (1 << l)};
      double2 x[4], y[4];
      for (int c = 0; c < 4; ++c) x[c] = M[row * GM + idx[c]];
      for (int c = 0; c < 4; ++c) {
        double2 s = czero();
        for (int cp = 0; cp < 4; ++cp) s = cadd(s, cmul(cconj(G[cp * 4 + c]), x[cp]));
        y[c] = s;
      }
      for (int c = 0; c < 4; ++c) M[row * GM + idx[c]] = y[c];
    }
  } else {
    const int items = D * (D / 2);
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
      const int row = it % D, o = it / D;
      const int ob = ((o >> h) << (h + 1)) | (o & ((1 << h) - 1));
      const double2 x0 = M[row * GM + ob], x1 = M[row * GM + (ob | (1 << h))];
      M[row * GM + ob] = cadd(cmul(cconj(G[0]), x0), cmul(cconj(G[2]), x1));
      M[row * GM + (ob | (1 << h))] = cadd(cmul(cconj(G[1]), x0), cmul(cconj(G[3]), x1));
    }
  }
}

// One block per state and group.  The polar factor of each step is the
// sweep polar of small_linalg.h: singular values of E at most 1e-6 of the
// largest count as zero, and on that null space (inputs the circuit never
// feeds the gate, such as fresh |0> qubits) every completion is optimal, so
// the kernel keeps the one nearest to the current gate; structured gates
// stay structured under fp32 rounding.  nuc[b] receives Re Tr(W^H E) of the
// last step, |<t|new|psi>| after the update.
#define POLAR_THREADS 64

__global__ void __launch_bounds__(POLAR_THREADS) k_group_polar(BatchDev bd, GroupDev gd, int g, double2* gates,
                                                               const signed char* arity, const int* nlayers,
                                                               const int* active, double* nuc, double2* env_out) {
  __shared__ double2 M[GMM];
  __shared__ double2 env[16];
  for (int b = blockIdx.x; b < bd.B; b += gridDim.x) {
    if (active && !active[b]) continue;
    if (g >= gd.ngroups[b]) continue;
    const GroupEnt ge = gd.grp[(int64_t)b * gd.gmax + g];
    const int n = bd.n[b], L = nlayers[b], D = 1 << ge.u;
    const int c0 = gd.state_chunk0[b], nc = gd.state_nchunks[b];
    __syncthreads();
    // sum of the chunk partials in chunk order; eight chunks' loads are
    // issued together so the L2 latency overlaps
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
      const int i = e / D, k = e % D;
      const double2* src = gd.partials + (int64_t)c0 * GMM + i * GM + k;
      double2 s = czero();
      int c = 0;
      for (; c + 8 <= nc; c += 8) {
        double2 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = src[(int64_t)(c + u) * GMM];
#pragma unroll
        for (int u = 0; u < 8; ++u) s = cadd(s, v[u]);
      }
      for (; c < nc; ++c) s = cadd(s, src[(int64_t)c * GMM]);
      M[i * GM + k] = s;
    }
    __syncthreads();
    const double2* pend = nullptr;
    int pk = 0, ph = 0, pl = 0;
    for (int s = 0; s < ge.cnt && s < GMAXSTEPS; ++s) {
      int64_t slot;
      int q, k;
      if (!bwd_step(bd, arity, L, n, b, ge.j0 + s, &slot, &q, &k)) continue;
      double2* gptr = gates + bd.gate_off[b] + slot * 16;
      const int h = __popc(ge.qmask >> (q + 1)), l = k == 2 ? __popc(ge.qmask >> (q + 2)) : 0;
      if (pend) {
        m_rows(M, D, pend, pk, ph, pl);
        __syncthreads();
      }
      m_cols(M, D, gptr, k, h, l);
      __syncthreads();
      const int m = 1 << k;
      if (threadIdx.x < m * m) {
        const int r = threadIdx.x / m, c = threadIdx.x % m;
        double2 acc = czero();
        for (int o = 0; o < D / m; ++o) {
          int ob = 0, kk = 0;
          for (int bit = 0; (1 << bit) < D; ++bit) {
            if (bit == h || (k == 2 && bit == l)) continue;
            ob |= ((o >> kk) & 1) << bit;
            ++kk;
          }
          const int ir = ob | (k == 2 ? (((r >> 1) & 1) << h) | ((r & 1) << l) : (r << h));
          const int ic = ob | (k == 2 ? (((c >> 1) & 1) << h) | ((c & 1) << l) : (c << h));
          acc = cadd(acc, M[ir * GM + ic]);
        }
        env[threadIdx.x] = acc;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        double2 e[16], w[16], wprev[16];
        bool finite = true;
        for (int i = 0; i < m * m; ++i) {
          e[i] = env[i];
          finite = finite && isfinite(e[i].x) && isfinite(e[i].y);
        }
        double2* keep = gd.old_gates + ((int64_t)b * GMAXSTEPS + s) * 16;
        for (int i = 0; i < m * m; ++i) keep[i] = gptr[i];
        if (!finite) {
          atomicOr(bd.err, KERR_NONFINITE);
        } else if (env_out) {   // environment at the fixed circuit: the gate stays
          double2* eo = env_out + bd.gate_off[b] + slot * 16;
          for (int i = 0; i < m * m; ++i) eo[i] = e[i];
        } else {
          for (int i = 0; i < m * m; ++i) wprev[i] = cconj(gptr[i]);
          const double nn = polar_sweep(e, m, w, wprev);
          for (int i = 0; i < m * m; ++i) gptr[i] = cconj(w[i]);
          nuc[b] = nn;
        }
      }
      __syncthreads();
      pend = gptr;
      pk = k;
      ph = h;
      pl = l;
    }
  }
}

// ---- launches ----------------------------------------------------------------------

void launch_group_plan(const BatchDev& bd, const GroupDev& gd, const signed char* arity, const int* nlayers,
                       cudaStream_t s) {
  const int blocks = (bd.B + 127) / 128;
  qm_note_launch();
  k_group_plan<<<blocks, 128, 0, s>>>(bd, gd, arity, nlayers, ORDER_BWD, 0, nullptr, gd.grp, gd.ngroups);
  qm_note_launch();
  k_group_plan<<<blocks, 128, 0, s>>>(bd, gd, arity, nlayers, ORDER_FWD, 0, nullptr, gd.rgrp, gd.nrgroups);
}

void launch_layer_plan(const BatchDev& bd, const GroupDev& gd, const signed char* arity, int mode, int layer,
                       const int* active, cudaStream_t s) {
  const int blocks = (bd.B + 127) / 128;
  qm_note_launch();
  k_group_plan<<<blocks, 128, 0, s>>>(bd, gd, arity, nullptr, mode, layer, active, gd.rgrp, gd.nrgroups);
}

// Blocks of a tile-pass launch: the autotuned count, or at most the
// resident blocks (PASS_BLOCKS_PER_SM per SM); never more than the chunks.
static int pass_grid(const GroupDev& gd) {
  int grid = gd.grid > 0 ? gd.grid : PASS_BLOCKS_PER_SM * 152;
  if (grid > gd.nchunks) grid = gd.nchunks;
  return grid < 1 ? 1 : grid;
}

int layer_pass_bound(int max_n) {
  // a group covers at least three new sites of the layer, except the last
  const int groups = (max_n + 2) / 3 + 1;
  return (groups + 1) / 2;
}

void launch_rebuild_pass(const BatchDev& bd, const GroupDev& gd, int pass, float2* psi, const double2* gates,
                         const signed char* arity, const int* nlayers, const int* active, cudaStream_t s, int mode,
                         int layer, bool exact) {
  int grid = pass_grid(gd);
  qm_note_launch();
  k_rebuild_pass<<<grid, PASS_THREADS, (size_t)2 * sizeof(float2) << GT, s>>>(bd, gd, pass, psi, gates, arity,
                                                                          nlayers, active, mode, layer, exact);
}

int launch_group_pass(const BatchDev& bd, const GroupDev& gd, int g, float2* psi, const float2* z_in, float2* z_out,
                      const double2* gates, const signed char* arity, const int* nlayers, const int* active,
                      const double2* znorm, cudaStream_t s) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_group_pass, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)PASS_DYN_SMEM);
    if (e != cudaSuccess) return (int)e;
    attr_set = true;
  }
  int grid = pass_grid(gd);
  qm_note_launch();
  k_group_pass<<<grid, PASS_THREADS, PASS_DYN_SMEM, s>>>(bd, gd, g, psi, z_in, z_out, gates, gd.old_gates, arity,
                                                          nlayers, active, znorm);
  return 0;
}

void launch_group_polar(const BatchDev& bd, const GroupDev& gd, int g, double2* gates, const signed char* arity,
                        const int* nlayers, const int* active, double* nuc, cudaStream_t s, double2* env_out) {
  qm_note_launch();
  k_group_polar<<<bd.B, POLAR_THREADS, 0, s>>>(bd, gd, g, gates, arity, nlayers, active, nuc, env_out);
}
