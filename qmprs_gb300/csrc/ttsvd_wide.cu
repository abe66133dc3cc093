// (a) statevector -> MPS for Gram widths above 128 (bonds above 64): the
// same right-to-left truncated SVD as ttsvd.cu, for the configurations with
// bond dimension 256 (20 qubits) and 1024 (24 qubits).
//
// The w x w Hermitian Gram (w up to 2048) is diagonalised in two precisions:
//
// 1. Blocked two-sided Jacobi in FP32.  The padded width W (a multiple of
//    32) is cut into blocks of 16 indices; a round pairs the blocks
//    (round-robin tournament) and every pair is one 32 x 32 subproblem.
//      k_bj_solve   one block per pair: the subproblem in shared memory,
//                   one cyclic Jacobi sweep (31 rounds of 16 disjoint
//                   rotations, each applied to 2 x 2 entry groups), the
//                   accumulated 32 x 32 unitary J, and the rotated
//                   diagonal tile written back;
//      k_bj_update  A[P,Q] <- J_P^H A[P,Q] J_Q on every off-diagonal tile of
//                   the round (upper triangle, mirrored) and V[:,Q] <- V J_Q.
//    Sweeps run until one sweep makes no rotation larger than 1e-5 of
//    sqrt(a_pp a_qq) (at most BJ_MAX_SWEEPS); rotations below FP32
//    resolution (1e-7 relative, or 1e-7 of ||G||_F / sqrt(W) absolute) are
//    skipped.
// 2. FP64 refinement of the K columns that can be kept (K = min(w,
//    max_bond, bond capacity, 2^c)), and of the discarded ones whose FP32
//    eigenvalue lies within 1e-5 (of the largest) of the last kept one
//    (their order and mixing with it are below FP32 resolution), by the
//    iterative refinement of
//    Ogita & Aishima (Japan J. Indust. Appl. Math. 35, 2018): with X the
//    FP32 eigenvectors ordered by eigenvalue,
//      S = X^H G X_K,  R = I - X^H X_K,  l_j = S_jj / (1 - R_jj),
//      E_ij = s_ij e_ij,  E_jj = R_jj / 2 + sum_i (c_ij - 1),
//    where (c_ij, s_ij e_ij) is the rotation that diagonalises the 2 x 2
//    block [[l_j, conj(b)], [b, l_i]], b = S_ij + l_j R_ij (to first order
//    E_ij = b / (l_j - l_i), the published step; the full rotation is
//    taken up to |s| = 0.3, beyond which a pair counts as a cluster), and
//      X_K <- X_K + X E.
//    S and R are FP64 products (k_zgemm) in the exact mode and double-float
//    products on the FP32 pipes (k_zgemm_df, about 5x the FP64 rate) in the
//    fast mode; the correction X E is double-float in the exact mode (the
//    first corrections reach 0.1-0.5, and FP32 rounding of them would set a
//    floor near 1e-8) and FP32 in the fast mode.  A step squares the error, so
//    one or two steps take FP32 eigenvectors to FP64 accuracy; it repeats
//    until max |E| is below the mode's tolerance, or stops halving (at most
//    BJ_MAX_REFINE steps).
//    The columns that stay (beyond K) enter only through their pairs with
//    the refined ones, whose denominators take their FP64 Rayleigh quotients
//    (k_bj_rq): the FP32 diagonal is accurate to first order only, which
//    would slow the convergence to linear.
//    FP32 resolves eigenvalues down to about 1e-7 of the largest.  When the
//    columns that may be kept reach below BJ_RESOLVED of it (rank-deficient
//    Grams, fast-decaying spectra, where the 1e-10 cutoff decides the
//    bond), the resolved columns are refined first, the rest of the basis
//    is projected off them and re-orthonormalised (one FP64 Newton-Schulz
//    step), and the Gram of that subspace, X_N^H G X_N, whose scale is the
//    small eigenvalues', is solved by the same two steps.
// 3. k_bj_finalize: the refined eigenvalues in descending order, quimb's
//    rsum2 cutoff with the tail sums taken from the bottom (the refined
//    small eigenvalues, plus the weight outside the refined columns from the
//    trace of the deflated subproblem, so that no sum near the trace is
//    subtracted from the trace); k_bj_emit, one
//    block per kept column: canonical phase, the selected column and the
//    site tensor of cut c.
//
//   k_cgemm       C = A B for a tall complex64 A and a small complex128 B
//                 (the projection M V of the remainder and the left-to-right
//                 contraction that rebuilds the dense target): 64 x 64 output
//                 tiles, K staged in shared memory, 4 x 4 outputs per
//                 thread.
//
// Method references: block Jacobi for the Hermitian eigenproblem (Golub &
// Van Loan, Matrix Computations, 4th ed., sec. 8.5.5), round-robin
// ordering (ibid. 8.5.4), the Rutishauser-style stable rotation.
#include <cstring>
#include <vector>

#include "dfloat.cuh"

#define BJ_B 16             // block of indices; a pair of blocks is a subproblem
#define BJ_S 32             // subproblem size
#define BJ_THREADS 256
#define BJ_MAX_SWEEPS 24
#define BJ_MAX_REFINE 6
#define BJ_PARTS 256        // blocks of the norm reduction (fixed: deterministic sums)
#define BJ_NOISE 1e-6       // eigenvalues below this fraction of the largest are FP32 noise
#define BJ_MARGIN 1e-5      // discarded columns this close (of the largest) to the last kept one ...
#define BJ_EXTRA 32         // ... are refined too, at most this many
#define BJ_MAX_ROT 0.3       // largest rotation (sin) a refinement step takes per pair

// Pair i of round k of the round-robin tournament over n (even) indices
// (round_robin_pair, small_linalg.h).
__host__ __device__ inline void bj_pair(int n, int k, int i, int* p, int* q) { round_robin_pair(n, k, i, p, q); }

// Global index of local index l (0..31) of pair i in round k: the first 16
// are block p, the next 16 block q.
__device__ __forceinline__ int bj_index(int nb, int k, int i, int l) {
  int p, q;
  bj_pair(nb, k, i, &p, &q);
  return (l < BJ_B ? p : q) * BJ_B + (l & (BJ_B - 1));
}

__device__ __forceinline__ float2 fcfma(float2 acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
  return acc;
}
__device__ __forceinline__ float2 fcfmac(float2 acc, float2 a, float2 b) {   // acc + conj(a) b
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(-a.y, b.x, acc.y);
  return acc;
}

// ---- FP32 blocked Jacobi --------------------------------------------------------------

// A <- G (FP32, padded with zeros to W), V <- I; per-block partial sums of
// |G_ij|^2 in FP64.
__global__ void k_bj_load(const double2* G, int w, float2* A, float2* V, int W, double* part) {
  double acc = 0.0;
  const int64_t total = (int64_t)W * W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / W), c = (int)(e % W);
    float2 a = cf(0.f, 0.f);
    if (r < w && c < w) {
      const double2 g = G[(int64_t)r * w + c];
      acc += cnorm2(g);
      a = cf((float)g.x, r == c ? 0.f : (float)g.y);
    }
    A[e] = a;
    V[e] = cf(r == c ? 1.f : 0.f, 0.f);
  }
  double v[1] = {acc};
  block_sum<1>(v);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

// stats[0] = ||G||_F, stats[1] = trace (fixed-order sums).
__global__ void k_bj_stats(const double* part, int nparts, const double2* G, int w, double* stats) {
  double v[2] = {0.0, 0.0};
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) v[0] += part[i];
  for (int i = threadIdx.x; i < w; i += blockDim.x) v[1] += G[(int64_t)i * w + i].x;
  block_sum<2>(v);
  if (threadIdx.x == 0) {
    stats[0] = sqrt(v[0]);
    stats[1] = v[1];
  }
}

// Rotation of pair (p, q) of the 32 x 32 subproblem m: c, s e and s conj(e)
// (the Rutishauser-style stable rotation that zeroes m[p][q]); flag 0 when
// |m[p][q]| is below FP32 resolution (1e-7 relative, or floor_abs), big 1
// when it is above 1e-5 relative (the sweep has not converged).  Correctly
// rounded reciprocal and square-root intrinsics.
struct BJRot {
  float c;
  float2 se;
  int flag, big;
};
__device__ __forceinline__ BJRot bj_rot(const float2 (*m)[BJ_S + 1], int p, int q, float floor_abs, float big_abs) {
  BJRot r;
  const float2 g = m[p][q];
  const float ag = __fsqrt_rn(g.x * g.x + g.y * g.y);
  const float app = m[p][p].x, aqq = m[q][q].x;
  const float scale = __fsqrt_rn(fabsf(app * aqq));
  r.flag = ag > floor_abs && ag > 1e-7f * scale;
  r.big = r.flag && ag > 1e-5f * scale && ag > big_abs;
  r.c = 1.f;
  r.se = cf(0.f, 0.f);
  if (r.flag) {
    const float inv = __frcp_rn(ag);
    const float zeta = 0.5f * (aqq - app) * inv;
    const float t = copysignf(__frcp_rn(fabsf(zeta) + __fsqrt_rn(fmaf(zeta, zeta, 1.f))), zeta);
    const float c = __frsqrt_rn(fmaf(t, t, 1.f));
    const float sg = c * t * inv;
    r.c = c;
    r.se = cf(g.x * sg, g.y * sg);
  }
  return r;
}

// One block per pair of round k: one Jacobi sweep of the 32 x 32
// subproblem; J (32 x 32, row-major) to Jbuf[pair]; the rotated diagonal
// tile back into A.  count += 1 if a rotation was above 1e-5 relative.
// Thread (gr, gc) owns the 2 x 2 entry group of inner pairs (gr, gc); lane
// l of a warp computes the rotation of pair l % 16 (its gc) and takes gr's
// from lane gr.  The subproblem is double-buffered (read one copy, write
// the other), so an inner round takes one barrier; the inner rounds' pairs
// come from a table built once.
__global__ void __launch_bounds__(BJ_THREADS) k_bj_solve(float2* A, int W, int nb, int k, float2* Jbuf,
                                                         const double* stats, int* count) {
  __shared__ float2 a[2][BJ_S][BJ_S + 1];
  __shared__ float2 j[BJ_S][BJ_S + 1];
  __shared__ unsigned char tp[BJ_S - 1][BJ_S / 2], tq[BJ_S - 1][BJ_S / 2];
  __shared__ int s_big;
  const int pair = blockIdx.x, tid = threadIdx.x;
  if (tid == 0) s_big = 0;
  for (int e = tid; e < BJ_S * BJ_S; e += blockDim.x) {
    const int r = e / BJ_S, c = e % BJ_S;
    a[0][r][c] = A[(int64_t)bj_index(nb, k, pair, r) * W + bj_index(nb, k, pair, c)];
    j[r][c] = cf(r == c ? 1.f : 0.f, 0.f);
  }
  for (int e = tid; e < (BJ_S - 1) * (BJ_S / 2); e += blockDim.x) {
    int p, q;
    bj_pair(BJ_S, e / (BJ_S / 2), e % (BJ_S / 2), &p, &q);
    tp[e / (BJ_S / 2)][e % (BJ_S / 2)] = (unsigned char)p;
    tq[e / (BJ_S / 2)][e % (BJ_S / 2)] = (unsigned char)q;
  }
  // rotations below FP32 rounding of the entries are skipped: ||G||_F /
  // sqrt(W) is the entries' scale (||G||_F alone overstates it by up to
  // sqrt(W) on flat spectra, where a floor that high leaves couplings at a
  // third of the eigenvalue gaps)
  const float floor_abs = 1e-7f * (float)stats[0] * rsqrtf((float)W), big_abs = 1e-6f * (float)stats[0];
  __syncthreads();
  const int gr = tid / (BJ_S / 2), gc = tid % (BJ_S / 2);
  int big = 0;
  for (int ir = 0; ir < BJ_S - 1; ++ir) {
    const float2 (*cur)[BJ_S + 1] = a[ir & 1];
    float2 (*nxt)[BJ_S + 1] = a[(ir + 1) & 1];
    const int pr = tp[ir][gr], qr = tq[ir][gr], pc = tp[ir][gc], qc = tq[ir][gc];
    const BJRot rcl = bj_rot(cur, pc, qc, floor_abs, big_abs);
    BJRot rr;
    rr.c = __shfl_sync(0xffffffffu, rcl.c, gr);
    rr.se.x = __shfl_sync(0xffffffffu, rcl.se.x, gr);
    rr.se.y = __shfl_sync(0xffffffffu, rcl.se.y, gr);
    rr.flag = __shfl_sync(0xffffffffu, rcl.flag, gr);
    big |= rcl.big;
    float2 x00 = cur[pr][pc], x01 = cur[pr][qc], x10 = cur[qr][pc], x11 = cur[qr][qc];
    if (rcl.flag) {   // columns: col_p <- c col_p - s conj(e) col_q ; col_q <- s e col_p + c col_q
      const float c = rcl.c;
      const float2 se = rcl.se, sce = cf(se.x, -se.y);
      const float2 n00 = cf(c * x00.x - (sce.x * x01.x - sce.y * x01.y), c * x00.y - (sce.x * x01.y + sce.y * x01.x));
      const float2 n01 = cf(se.x * x00.x - se.y * x00.y + c * x01.x, se.x * x00.y + se.y * x00.x + c * x01.y);
      const float2 n10 = cf(c * x10.x - (sce.x * x11.x - sce.y * x11.y), c * x10.y - (sce.x * x11.y + sce.y * x11.x));
      const float2 n11 = cf(se.x * x10.x - se.y * x10.y + c * x11.x, se.x * x10.y + se.y * x10.x + c * x11.y);
      x00 = n00;
      x01 = n01;
      x10 = n10;
      x11 = n11;
    }
    if (rr.flag) {    // rows: row_p <- c row_p - s e row_q ; row_q <- s conj(e) row_p + c row_q
      const float c = rr.c;
      const float2 se = rr.se, sce = cf(se.x, -se.y);
      const float2 n00 = cf(c * x00.x - (se.x * x10.x - se.y * x10.y), c * x00.y - (se.x * x10.y + se.y * x10.x));
      const float2 n01 = cf(c * x01.x - (se.x * x11.x - se.y * x11.y), c * x01.y - (se.x * x11.y + se.y * x11.x));
      const float2 n10 = cf(sce.x * x00.x - sce.y * x00.y + c * x10.x, sce.x * x00.y + sce.y * x00.x + c * x10.y);
      const float2 n11 = cf(sce.x * x01.x - sce.y * x01.y + c * x11.x, sce.x * x01.y + sce.y * x01.x + c * x11.y);
      x00 = n00;
      x01 = n01;
      x10 = n10;
      x11 = n11;
    }
    if (gr == gc) {   // the rotated pair: real diagonal, eliminated off-diagonal
      x00.y = 0.f;
      x11.y = 0.f;
      if (rr.flag) x01 = x10 = cf(0.f, 0.f);
    }
    nxt[pr][pc] = x00;
    nxt[pr][qc] = x01;
    nxt[qr][pc] = x10;
    nxt[qr][qc] = x11;
    // J <- J R on the columns of pair gc, rows gr and gr + 16 (one owner each)
    if (rcl.flag) {
      const float c = rcl.c;
      const float2 se = rcl.se, sce = cf(se.x, -se.y);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int row = gr + h * (BJ_S / 2);
        const float2 vp = j[row][pc], vq = j[row][qc];
        j[row][pc] = cf(c * vp.x - (sce.x * vq.x - sce.y * vq.y), c * vp.y - (sce.x * vq.y + sce.y * vq.x));
        j[row][qc] = cf(se.x * vp.x - se.y * vp.y + c * vq.x, se.x * vp.y + se.y * vp.x + c * vq.y);
      }
    }
    __syncthreads();
  }
  if (big) s_big = 1;
  const float2 (*fin)[BJ_S + 1] = a[(BJ_S - 1) & 1];
  float2* jo = Jbuf + (int64_t)pair * BJ_S * BJ_S;
  for (int e = tid; e < BJ_S * BJ_S; e += blockDim.x) {
    const int r = e / BJ_S, c = e % BJ_S;
    jo[e] = j[r][c];
    // Hermitian diagonal tile: the upper triangle and its mirror
    const float2 v = r <= c ? fin[r][c] : cf(fin[c][r].x, -fin[c][r].y);
    A[(int64_t)bj_index(nb, k, pair, r) * W + bj_index(nb, k, pair, c)] = v;
  }
  __syncthreads();
  if (tid == 0 && s_big) atomicAdd(count, 1);
}

// 32 x 32 complex products of k_bj_update in shared memory (rows padded to
// 34 entries: 16-byte aligned pairs, distinct banks for the 4 rows a warp
// reads): 128 threads, a 4 x 2 block of outputs each (rows 4 (tid / 16) ..,
// columns 2 (tid % 16) ..); out = (CONJ ? x^H : x) y.
#define BJU_THREADS 128
#define BJU_LD (BJ_S + 2)
template <bool CONJ>
__device__ __forceinline__ void bj_mm32(const float2 (*x)[BJU_LD], const float2 (*y)[BJU_LD], float2 (&out)[4][2]) {
  const int r0 = (threadIdx.x / 16) * 4, c0 = (threadIdx.x % 16) * 2;
#pragma unroll
  for (int i = 0; i < 4; ++i) out[i][0] = out[i][1] = cf(0.f, 0.f);
#pragma unroll 4
  for (int m = 0; m < BJ_S; ++m) {
    float2 xv[4];
    if (CONJ) {
      const float4 a = *reinterpret_cast<const float4*>(&x[m][r0]);
      const float4 b = *reinterpret_cast<const float4*>(&x[m][r0 + 2]);
      xv[0] = cf(a.x, a.y);
      xv[1] = cf(a.z, a.w);
      xv[2] = cf(b.x, b.y);
      xv[3] = cf(b.z, b.w);
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) xv[i] = x[r0 + i][m];
    }
    const float4 yy = *reinterpret_cast<const float4*>(&y[m][c0]);
    const float2 y0 = cf(yy.x, yy.y), y1 = cf(yy.z, yy.w);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      out[i][0] = CONJ ? fcfmac(out[i][0], xv[i], y0) : fcfma(out[i][0], xv[i], y0);
      out[i][1] = CONJ ? fcfmac(out[i][1], xv[i], y1) : fcfma(out[i][1], xv[i], y1);
    }
  }
}

__device__ __forceinline__ void bj_store32(float2 (*t)[BJU_LD], const float2 (&out)[4][2]) {
  const int r0 = (threadIdx.x / 16) * 4, c0 = (threadIdx.x % 16) * 2;
#pragma unroll
  for (int i = 0; i < 4; ++i) *reinterpret_cast<float4*>(&t[r0 + i][c0]) = make_float4(out[i][0].x, out[i][0].y,
                                                                                        out[i][1].x, out[i][1].y);
}

// Blocks [0, nA): off-diagonal tiles P < Q of round k (upper triangle in
// row order), A[P,Q] <- J_P^H A[P,Q] J_Q and its mirror (both written row
// by row from shared memory); blocks [nA, nA + nV): V[R rows, Q] <-
// V[R rows, Q] J_Q for row tiles R of 32 rows.
__global__ void __launch_bounds__(BJU_THREADS) k_bj_update(float2* A, float2* V, int W, int nb, int k,
                                                           const float2* Jbuf, int nA) {
  __shared__ __align__(16) float2 t[BJ_S][BJU_LD];
  __shared__ __align__(16) float2 jq[BJ_S][BJU_LD];
  __shared__ __align__(16) float2 jp[BJ_S][BJU_LD];
  const int np = nb / 2, tid = threadIdx.x;
  float2 out[4][2];
  if ((int)blockIdx.x < nA) {
    // tile index -> (P, Q), P < Q: row P holds np - 1 - P tiles
    int rem = blockIdx.x, P = 0;
    while (rem >= np - 1 - P) {
      rem -= np - 1 - P;
      ++P;
    }
    const int Q = P + 1 + rem;
    for (int e = tid; e < BJ_S * BJ_S; e += blockDim.x) {
      const int rr = e / BJ_S, cc = e % BJ_S;
      t[rr][cc] = A[(int64_t)bj_index(nb, k, P, rr) * W + bj_index(nb, k, Q, cc)];
      jq[rr][cc] = Jbuf[(int64_t)Q * BJ_S * BJ_S + e];
      jp[rr][cc] = Jbuf[(int64_t)P * BJ_S * BJ_S + e];
    }
    __syncthreads();
    bj_mm32<false>(t, jq, out);   // U = T J_Q
    __syncthreads();
    bj_store32(t, out);
    __syncthreads();
    bj_mm32<true>(jp, t, out);    // J_P^H U
    __syncthreads();
    bj_store32(t, out);
    __syncthreads();
    for (int e = tid; e < BJ_S * BJ_S; e += blockDim.x) {
      const int rr = e / BJ_S, cc = e % BJ_S;
      A[(int64_t)bj_index(nb, k, P, rr) * W + bj_index(nb, k, Q, cc)] = t[rr][cc];
      const float2 v = t[cc][rr];
      A[(int64_t)bj_index(nb, k, Q, rr) * W + bj_index(nb, k, P, cc)] = cf(v.x, -v.y);
    }
  } else {
    const int tI = blockIdx.x - nA;
    const int R = tI / np, Q = tI % np;
    for (int e = tid; e < BJ_S * BJ_S; e += blockDim.x) {
      const int rr = e / BJ_S, cc = e % BJ_S;
      t[rr][cc] = V[(int64_t)(R * BJ_S + rr) * W + bj_index(nb, k, Q, cc)];
      jq[rr][cc] = Jbuf[(int64_t)Q * BJ_S * BJ_S + e];
    }
    __syncthreads();
    bj_mm32<false>(t, jq, out);
    __syncthreads();
    bj_store32(t, out);
    __syncthreads();
    for (int e = tid; e < BJ_S * BJ_S; e += blockDim.x) {
      const int rr = e / BJ_S, cc = e % BJ_S;
      V[(int64_t)(R * BJ_S + rr) * W + bj_index(nb, k, Q, cc)] = t[rr][cc];
    }
  }
}

// Descending order of the FP32 eigenvalues (diagonal of A, ties by index):
// perm[rank] = index, lamA[rank] = value.  One block.
__global__ void __launch_bounds__(1024) k_bj_sort(const float2* A, int W, int n, int* perm, double* lamA) {
  extern __shared__ float dg[];
  for (int i = threadIdx.x; i < n; i += blockDim.x) dg[i] = A[(int64_t)i * W + i].x;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float li = dg[i];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const float lj = dg[j];
      rank += (lj > li) || (lj == li && j < i);
    }
    perm[rank] = i;
    lamA[rank] = (double)li;
  }
}

// X[r][j] = V[r][perm[j]] (r, j < n) in FP64.
__global__ void k_bj_basis(const float2* V, int W, int n, const int* perm, double2* X) {
  const int64_t total = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / n), jc = (int)(e % n);
    X[e] = f2d(V[(int64_t)r * W + perm[jc]]);
  }
}

// ---- FP64 refinement ------------------------------------------------------------------

// C[m][n] = alpha sum_k op(A)[m][k] B[k][n] (+ D[m][n]) in FP64; op(A)[m][k]
// = A[m][k], or conj(A[k][m]) with CONJ.  64 x 64 tiles, K in chunks of 8,
// 4 x 4 outputs per thread.
#define ZG_T 64
#define ZG_K 8
template <bool CONJ>
__global__ void __launch_bounds__(256) k_zgemm(const double2* A, int64_t lda, const double2* B, int64_t ldb,
                                               const double2* D, int64_t ldd, double2* C, int64_t ldc, int M, int N,
                                               int K, double alpha) {
  __shared__ double2 As[ZG_K][ZG_T + 1];
  __shared__ double2 Bs[ZG_K][ZG_T];
  const int m0 = blockIdx.x * ZG_T, n0 = blockIdx.y * ZG_T;
  const int tr = threadIdx.x / 16, tc = threadIdx.x % 16;
  double2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j2 = 0; j2 < 4; ++j2) acc[i][j2] = czero();
  for (int k0 = 0; k0 < K; k0 += ZG_K) {
    __syncthreads();
    for (int e = threadIdx.x; e < ZG_T * ZG_K; e += blockDim.x) {
      int mm, kk;
      if (CONJ) {
        kk = e / ZG_T;
        mm = e % ZG_T;
      } else {
        mm = e / ZG_K;
        kk = e % ZG_K;
      }
      const int gm = m0 + mm, gk = k0 + kk;
      double2 v = czero();
      if (gm < M && gk < K) v = CONJ ? cconj(A[(int64_t)gk * lda + gm]) : A[(int64_t)gm * lda + gk];
      As[kk][mm] = v;
      const int kb = e / ZG_T, nn = e % ZG_T;
      const int gkb = k0 + kb, gn = n0 + nn;
      Bs[kb][nn] = (gkb < K && gn < N) ? B[(int64_t)gkb * ldb + gn] : czero();
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < ZG_K; ++kk) {
      double2 av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[kk][tr * 4 + i];
#pragma unroll
      for (int j2 = 0; j2 < 4; ++j2) bv[j2] = Bs[kk][tc * 4 + j2];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j2 = 0; j2 < 4; ++j2) {
          acc[i][j2].x = fma(av[i].x, bv[j2].x, acc[i][j2].x);
          acc[i][j2].x = fma(-av[i].y, bv[j2].y, acc[i][j2].x);
          acc[i][j2].y = fma(av[i].x, bv[j2].y, acc[i][j2].y);
          acc[i][j2].y = fma(av[i].y, bv[j2].x, acc[i][j2].y);
        }
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + tr * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j2 = 0; j2 < 4; ++j2) {
      const int gn = n0 + tc * 4 + j2;
      if (gn >= N) continue;
      double2 v = cscale(acc[i][j2], alpha);
      if (D) v = cadd(v, D[(int64_t)gm * ldd + gn]);
      C[(int64_t)gm * ldc + gn] = v;
    }
  }
}

// The same product in double-float on the FP32 pipes (dfloat.cuh): both
// factors split into FP32 hi + lo on load, exact high products, TwoSum
// accumulation; about 2^-46 per operation, 1e-13 of the summed magnitudes
// over K = 2048 terms, at about 5x the FP64 rate.
template <bool CONJ>
__global__ void __launch_bounds__(256) k_zgemm_df(const double2* A, int64_t lda, const double2* B, int64_t ldb,
                                                  const double2* D, int64_t ldd, double2* C, int64_t ldc, int M,
                                                  int N, int K, double alpha) {
  __shared__ xc As[ZG_K][ZG_T + 1];
  __shared__ xc Bs[ZG_K][ZG_T];
  const int m0 = blockIdx.x * ZG_T, n0 = blockIdx.y * ZG_T;
  const int tr = threadIdx.x / 16, tc = threadIdx.x % 16;
  XA acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j2 = 0; j2 < 4; ++j2) acc[i][j2] = xa_zero();
  for (int k0 = 0; k0 < K; k0 += ZG_K) {
    __syncthreads();
    for (int e = threadIdx.x; e < ZG_T * ZG_K; e += blockDim.x) {
      int mm, kk;
      if (CONJ) {
        kk = e / ZG_T;
        mm = e % ZG_T;
      } else {
        mm = e / ZG_K;
        kk = e % ZG_K;
      }
      const int gm = m0 + mm, gk = k0 + kk;
      double2 v = czero();
      if (gm < M && gk < K) v = CONJ ? A[(int64_t)gk * lda + gm] : A[(int64_t)gm * lda + gk];
      As[kk][mm] = xc_from_d(v);
      const int kb = e / ZG_T, nn = e % ZG_T;
      const int gkb = k0 + kb, gn = n0 + nn;
      Bs[kb][nn] = xc_from_d((gkb < K && gn < N) ? B[(int64_t)gkb * ldb + gn] : czero());
    }
    __syncthreads();
#pragma unroll 2
    for (int kk = 0; kk < ZG_K; ++kk) {
      xc av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[kk][tr * 4 + i];
#pragma unroll
      for (int j2 = 0; j2 < 4; ++j2) bv[j2] = Bs[kk][tc * 4 + j2];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j2 = 0; j2 < 4; ++j2) {
          if (CONJ)
            xa_macc(acc[i][j2], av[i], bv[j2]);
          else
            xa_mac(acc[i][j2], av[i], bv[j2]);
        }
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + tr * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j2 = 0; j2 < 4; ++j2) {
      const int gn = n0 + tc * 4 + j2;
      if (gn >= N) continue;
      double2 v = cscale(xa_to_d(acc[i][j2]), alpha);
      if (D) v = cadd(v, D[(int64_t)gm * ldd + gn]);
      C[(int64_t)gm * ldc + gn] = v;
    }
  }
}

// C += A B with a small B (the fast mode's correction X E): FP32 products
// and sums (|X E| is at most the mode's tolerance, so the rounding is below
// 1e-10).  Same tiling as k_zgemm.
__global__ void __launch_bounds__(256) k_zgemm_small(const double2* A, int64_t lda, const double2* B, int64_t ldb,
                                                     double2* C, int64_t ldc, int M, int N, int K) {
  __shared__ float2 As[ZG_K][ZG_T + 1];
  __shared__ float2 Bs[ZG_K][ZG_T];
  const int m0 = blockIdx.x * ZG_T, n0 = blockIdx.y * ZG_T;
  const int tr = threadIdx.x / 16, tc = threadIdx.x % 16;
  float2 part[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j2 = 0; j2 < 4; ++j2) part[i][j2] = cf(0.f, 0.f);
  for (int k0 = 0; k0 < K; k0 += ZG_K) {
    __syncthreads();
    for (int e = threadIdx.x; e < ZG_T * ZG_K; e += blockDim.x) {
      const int mm = e / ZG_K, kk = e % ZG_K;
      const int gm = m0 + mm, gk = k0 + kk;
      const double2 v = (gm < M && gk < K) ? A[(int64_t)gm * lda + gk] : czero();
      As[kk][mm] = cf((float)v.x, (float)v.y);
      const int kb = e / ZG_T, nn = e % ZG_T;
      const int gkb = k0 + kb, gn = n0 + nn;
      const double2 u = (gkb < K && gn < N) ? B[(int64_t)gkb * ldb + gn] : czero();
      Bs[kb][nn] = cf((float)u.x, (float)u.y);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < ZG_K; ++kk) {
      float2 av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[kk][tr * 4 + i];
#pragma unroll
      for (int j2 = 0; j2 < 4; ++j2) bv[j2] = Bs[kk][tc * 4 + j2];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j2 = 0; j2 < 4; ++j2) part[i][j2] = fcfma(part[i][j2], av[i], bv[j2]);
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + tr * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j2 = 0; j2 < 4; ++j2) {
      const int gn = n0 + tc * 4 + j2;
      if (gn < N) C[(int64_t)gm * ldc + gn] = cadd(C[(int64_t)gm * ldc + gn], f2d(part[i][j2]));
    }
  }
}

// dst[r][c] = src[r][c] for r < rows, c < cols (row strides lds, ldd).
__global__ void k_bj_copy(const double2* src, int64_t lds, double2* dst, int64_t ldd, int rows, int cols) {
  const int64_t total = (int64_t)rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / cols), c = (int)(e % cols);
    dst[(int64_t)r * ldd + c] = src[(int64_t)r * lds + c];
  }
}

// l_j = S_jj / (1 - R_jj) for the Kc refined columns; SR holds [S | X^H X_K]
// (row stride 2 Kc), so 1 - R_jj is the (j, Kc + j) entry.
__global__ void k_bj_lam(const double2* SR, int Kc, double* lamK) {
  const int jc = blockIdx.x * blockDim.x + threadIdx.x;
  if (jc >= Kc) return;
  const int64_t o = (int64_t)jc * 2 * Kc;
  lamK[jc] = SR[o + jc].x / SR[o + Kc + jc].x;
}

// One block per refined column j: E (n x Kc) into the S half of SR.  Every
// pair (i, j) takes the rotation that diagonalises its 2 x 2 block
// [[l_j, conj(b)], [b, l_i]], b = S_ij + l_j R_ij: E_ij = s e (e = b / |b|)
// and cos - 1 into E_jj, next to R_jj / 2.  For a small coupling s e is
// the first-order b / (l_j - l_i); near-degenerate pairs get the full
// rotation.  Pairs of eigenvalues both below BJ_NOISE of the largest
// (lamA[0], below the FP32 sweeps' resolution) and couplings at the
// rounding level of the products (tiny_rel of the largest) take no rotation: between two refined columns they only
// restore orthonormality (E_ij = R_ij / 2), against an unrefined column
// nothing (its overlap is that column's own FP32 error).  emax =
// max |s| (float bits, atomicMax: order-independent); the diagonal sum is
// a fixed-order block reduction.
__global__ void __launch_bounds__(BLOCK_THREADS) k_bj_correct(double2* SR, int n, int Kc, const double* lamK,
                                                              const double* lamA, double tiny_rel, unsigned* emax) {
  const int jc = blockIdx.x;
  const double top = fabs(lamA[0]);
  const double noise = BJ_NOISE * top, tiny = tiny_rel * top;
  const double lj = lamK[jc];
  double dsum = 0.0;
  float mx = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    if (i == jc) continue;
    const int64_t o = (int64_t)i * 2 * Kc;
    const double2 xx = SR[o + Kc + jc];
    const double2 rv = cd(-xx.x, -xx.y);   // R = I - X^H X_K off the diagonal
    const double li = i < Kc ? lamK[i] : lamA[i];
    const double2 num = cadd(SR[o + jc], cscale(rv, lj));
    const double an = cabs_(num);
    const double den = lj - li;
    double2 ev;
    if ((fabs(lj) <= noise && fabs(li) <= noise) || an <= tiny) {
      // no rotation: a small coupling to first order; otherwise only the
      // orthonormality between refined columns (an unrefined column's
      // overlap is its own FP32 error, not a direction to move in)
      if (an <= tiny && fabs(den) > 100.0 * tiny)
        ev = cscale(num, 1.0 / den);
      else
        ev = i < Kc ? cscale(rv, 0.5) : czero();
    } else {
      const double zeta = den / (2.0 * an);
      const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
      const double c = 1.0 / sqrt(1.0 + t * t);
      const double sn = c * t;
      if (fabs(sn) > BJ_MAX_ROT) {
        // a near-degenerate pair (at the FP32 sweeps' resolution): rotations
        // this large over overlapping pairs of a dense cluster do not add up
        // to a unitary and diverge; the pair keeps its FP32 mixing (between
        // two refined columns only the orthonormality is restored; against
        // an unrefined column nothing moves)
        ev = i < Kc ? cscale(rv, 0.5) : czero();
      } else {
        ev = cscale(num, sn / an);
        dsum -= t * t * c * c / (1.0 + c);   // c - 1
        mx = fmaxf(mx, (float)fabs(sn));
      }
    }
    SR[o + jc] = ev;
  }
  double v[1] = {dsum};
  block_sum<1>(v);
  if (threadIdx.x == 0) {
    const int64_t o = (int64_t)jc * 2 * Kc;
    SR[o + jc] = cd(0.5 * (1.0 - SR[o + Kc + jc].x) + v[0], 0.0);
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0 && mx > 0.f) atomicMax(emax, __float_as_uint(mx));
}

// Rayleigh quotients of the columns c0 .. n-1 of X (n x n, stride n) that
// the refinement does not move: lamA[i] = Re(x_i^H (H x_i)) / |x_i|^2 with
// H x_i in T (column i - c0, stride ldt).  They are the denominators of
// those columns' pairs, accurate to second order in the FP32 eigenvectors'
// error where the FP32 diagonal is accurate only to first order.  One block
// per column, fixed-order reduction.
__global__ void __launch_bounds__(BLOCK_THREADS) k_bj_rq(const double2* X, int n, const double2* T, int ldt, int c0,
                                                         double* lamA) {
  const int i = c0 + blockIdx.x;
  double v[2] = {0.0, 0.0};
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const double2 x = X[(int64_t)k * n + i], t = T[(int64_t)k * ldt + (i - c0)];
    v[0] += x.x * t.x + x.y * t.y;
    v[1] += x.x * x.x + x.y * x.y;
  }
  block_sum<2>(v);
  if (threadIdx.x == 0) lamA[i] = v[1] > 0.0 ? v[0] / v[1] : 0.0;
}

// T <- (3 I - T) / 2 (m x m): one Newton-Schulz step's factor.
__global__ void k_bj_ns(double2* T, int m) {
  const int64_t total = (int64_t)m * m;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / m), c = (int)(e % m);
    const double2 t = T[e];
    T[e] = cd(((r == c ? 3.0 : 0.0) - t.x) * 0.5, -t.y * 0.5);
  }
}

// Order of the refined eigenvalues and the rsum2 cutoff: bond c of state b
// and order[] (the columns of X by descending eigenvalue).  The first Kr
// columns of X are refined; at most K (<= Kr) are kept.  The tail sums of
// the rule are summed from the bottom: tail_from(i) = rest + sum_{i <= j <
// Kr} l_j, where `rest` is the weight outside the refined columns: 0 when
// all are refined; for a deflated cut (tr_sub non-null) the subproblem's
// trace minus its refined eigenvalues (lamK[r .. Kr)), all at the small
// eigenvalues' scale; otherwise trace - sum of the refined ones, which then
// hold at most K <= r columns and leave resolved eigenvalues (above 1e-5 of
// the largest, far above the cutoff) in the rest.  Subtracting ~1 - 1e-10
// of the trace from the trace would carry the refined columns' rounding
// into the decision.  One block.
__global__ void __launch_bounds__(1024) k_bj_finalize(BatchDev bd, int b, int c, int w, int Kr, int K, int r,
                                                      const double* lamK, const double* stats, const double* tr_sub,
                                                      int* bonds, int max_bond, double cutoff, int* order,
                                                      double* lsort) {
  for (int i = threadIdx.x; i < Kr; i += blockDim.x) {
    const double li = lamK[i];
    int rank = 0;
    for (int j2 = 0; j2 < Kr; ++j2) {
      const double lj = lamK[j2];
      rank += (lj > li) || (lj == li && j2 < i);
    }
    order[rank] = i;
    lsort[rank] = li;
  }
  __syncthreads();
  int* bond = bonds + (int64_t)b * (bd.max_n + 1);
  if (threadIdx.x == 0) {
    const double total = stats[1];
    double rest = 0.0;
    if (tr_sub) {
      rest = *tr_sub;
      for (int i = r; i < Kr; ++i) rest -= lamK[i];
    } else if (Kr < w) {
      rest = total;
      for (int i = 0; i < Kr; ++i) rest -= lamK[i];
    }
    int keep = rank_from_tails(lsort, Kr, K, rest, total, cutoff, max_bond);
    if (keep > bd.tt_b) keep = bd.tt_b;
    if (c < 30 && keep > (1 << c)) keep = 1 << c;
    bond[c] = keep;
  }
}

// One block per kept column l (column order[l] of X, or column l without
// order; w entries, row stride ldx): the canonical phase (the pivot rule of
// phase_fix_column: the lowest row whose magnitude is within QM_PIVOT_TOL of
// the column's largest, made real positive), the selected column into vsel
// (stride vstride) and row l of the site tensor of cut c.
__global__ void __launch_bounds__(BLOCK_THREADS) k_bj_emit(BatchDev bd, int b, int c, const double2* X, int ldx,
                                                           int w, const int* bonds, const int* order, double2* vsel,
                                                           int vstride, double2* tensors, int chi) {
  __shared__ double s_m[BLOCK_THREADS / 32];
  __shared__ int s_j[BLOCK_THREADS / 32];
  __shared__ double2 s_ph;
  const int l = blockIdx.x;
  const int keep = bonds[(int64_t)b * (bd.max_n + 1) + c];
  if (l >= keep) return;
  const int col = order ? order[l] : l;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double m = -1.0;
  for (int i = threadIdx.x; i < w; i += blockDim.x) m = fmax(m, cabs_(X[(int64_t)i * ldx + col]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) s_m[warp] = m;
  __syncthreads();
  m = s_m[0];
  for (int k = 1; k < BLOCK_THREADS / 32; ++k) m = fmax(m, s_m[k]);
  int jp = w;
  for (int i = threadIdx.x; i < w; i += blockDim.x)
    if (cabs_(X[(int64_t)i * ldx + col]) >= (1.0 - QM_PIVOT_TOL) * m) {
      jp = i;
      break;
    }
  for (int o = 16; o > 0; o >>= 1) jp = min(jp, __shfl_xor_sync(0xffffffffu, jp, o));
  if (lane == 0) s_j[warp] = jp;
  __syncthreads();
  if (threadIdx.x == 0) {
    int j = s_j[0];
    for (int k = 1; k < BLOCK_THREADS / 32; ++k) j = min(j, s_j[k]);
    if (j >= w) j = 0;
    const double2 z = X[(int64_t)j * ldx + col];
    const double az = cabs_(z);
    s_ph = az > 0.0 ? cscale(cconj(z), 1.0 / az) : cd(1.0, 0.0);
  }
  __syncthreads();
  const double2 ph = s_ph;
  double2* vs = vsel + (int64_t)b * bd.tt_w * bd.tt_w;
  const int n = bd.n[b];
  const int ce = chi < (1 << (n / 2)) ? chi : (1 << (n / 2));
  double2* ts = tensors + bd.tensor_off[b] + (int64_t)c * 2 * ce * ce + (int64_t)l * w;
  for (int i = threadIdx.x; i < w; i += blockDim.x) {
    const double2 v = cmul(X[(int64_t)i * ldx + col], ph);
    vs[(int64_t)i * vstride + l] = v;
    ts[i] = cconj(v);
  }
}

// Row-Gram path.  Mt = M^H (w x rows, FP64) of the complex64 remainder M
// (rows x w): 32 x 32 tiles transposed through shared memory.
__global__ void k_bj_mt(const float2* M, int rows, int w, double2* Mt) {
  __shared__ float2 t[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {
    const int rr = e / 32, cc = e % 32;
    t[rr][cc] = (r0 + rr < rows && c0 + cc < w) ? M[(int64_t)(r0 + rr) * w + c0 + cc] : cf(0.f, 0.f);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {
    const int cc = e / 32, rr = e % 32;
    if (c0 + cc < w && r0 + rr < rows) Mt[(int64_t)(c0 + cc) * rows + r0 + rr] = cd(t[rr][cc].x, -t[rr][cc].y);
  }
}

// dst = src in FP64 (count complex entries).
__global__ void k_bj_f2d(const float2* src, int64_t count, double2* dst) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
    dst[e] = f2d(src[e]);
}

// U (n x K, row stride K): column l = X[:, order[l]] / sigma_l, sigma_l the
// square root of the l-th eigenvalue (descending); then V = M^H U holds the
// right singular vectors of the kept values.
__global__ void k_bj_gather(const double2* X, int n, const int* order, const double* lsort, int K, double2* U) {
  const int64_t total = (int64_t)n * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / K), l = (int)(e % K);
    const double lam = lsort[l];
    U[e] = lam > 0.0 ? cscale(X[(int64_t)i * n + order[l]], 1.0 / sqrt(lam)) : czero();
  }
}

// C[m][n] = sum_k A[m][k] B[k][n]: A complex64 (lda), B complex128 (ldb),
// C complex64 (ldc).  Block: a 64 x 64 tile of C, 256 threads, 4 x 4 per
// thread; K in chunks of 16 through shared memory.
#define CG_T 64
#define CG_K 16
__global__ void __launch_bounds__(256) k_cgemm(const float2* A, int64_t lda, const double2* B, int64_t ldb,
                                               float2* C, int64_t ldc, int64_t M, int N, int K) {
  __shared__ float2 As[CG_K][CG_T + 1];
  __shared__ float2 Bs[CG_K][CG_T];
  const int64_t m0 = (int64_t)blockIdx.x * CG_T;
  const int n0 = blockIdx.y * CG_T;
  const int tr = threadIdx.x / 16, tc = threadIdx.x % 16;   // 16 x 16 threads, 4 x 4 outputs each
  float2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = cf(0.f, 0.f);
  for (int k0 = 0; k0 < K; k0 += CG_K) {
    __syncthreads();
    for (int e = threadIdx.x; e < CG_T * CG_K; e += blockDim.x) {
      const int mm = e / CG_K, kk = e % CG_K;
      const int64_t gm = m0 + mm;
      const int gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? A[gm * lda + gk] : cf(0.f, 0.f);
      const int kb = e / CG_T, nn = e % CG_T;
      const int gkb = k0 + kb, gn = n0 + nn;
      if (gkb < K && gn < N) {
        const double2 v = B[(int64_t)gkb * ldb + gn];
        Bs[kb][nn] = cf((float)v.x, (float)v.y);
      } else {
        Bs[kb][nn] = cf(0.f, 0.f);
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < CG_K; ++kk) {
      float2 a[4], bb[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tr * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bb[j] = Bs[kk][tc * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmac(acc[i][j], a[i], bb[j]);
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t gm = m0 + tr * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tc * 4 + j;
      if (gn < N) C[gm * ldc + gn] = acc[i][j];
    }
  }
}


// ---- host-side drivers -------------------------------------------------------------

static int bj_round32(int w) { return (w + BJ_S - 1) / BJ_S * BJ_S; }

int bj_alloc(BJScratch& sc, int tt_w, int tt_b) {
  const int W = bj_round32(tt_w);
  const int kmax = tt_b + BJ_EXTRA < W ? tt_b + BJ_EXTRA : W;
  sc.W = W;
  sc.kmax = kmax;
  const size_t WW = (size_t)W * W;
  cudaError_t e = cudaSuccess;
  auto get = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
  };
  get(reinterpret_cast<void**>(&sc.A), sizeof(float2) * WW);
  get(reinterpret_cast<void**>(&sc.V), sizeof(float2) * WW);
  get(reinterpret_cast<void**>(&sc.J), sizeof(float2) * (size_t)(W / BJ_S) * BJ_S * BJ_S);
  get(reinterpret_cast<void**>(&sc.X), sizeof(double2) * WW);
  get(reinterpret_cast<void**>(&sc.H), sizeof(double2) * WW);
  get(reinterpret_cast<void**>(&sc.T), sizeof(double2) * WW);
  get(reinterpret_cast<void**>(&sc.T2), sizeof(double2) * WW);
  get(reinterpret_cast<void**>(&sc.Mt), sizeof(double2) * WW);
  get(reinterpret_cast<void**>(&sc.YX), sizeof(double2) * (size_t)W * 2 * kmax);
  get(reinterpret_cast<void**>(&sc.SR), sizeof(double2) * (size_t)W * 2 * kmax);
  get(reinterpret_cast<void**>(&sc.perm), sizeof(int) * W);
  get(reinterpret_cast<void**>(&sc.order), sizeof(int) * kmax);
  get(reinterpret_cast<void**>(&sc.count), sizeof(int) * 2);
  get(reinterpret_cast<void**>(&sc.lamA), sizeof(double) * W);
  get(reinterpret_cast<void**>(&sc.lamK), sizeof(double) * kmax);
  get(reinterpret_cast<void**>(&sc.lsort), sizeof(double) * kmax);
  get(reinterpret_cast<void**>(&sc.stats), sizeof(double) * 4);
  get(reinterpret_cast<void**>(&sc.part), sizeof(double) * BJ_PARTS);
  get(reinterpret_cast<void**>(&sc.emax), sizeof(unsigned));
  return (int)e;
}

void bj_free(BJScratch& sc) {
  void* ptrs[] = {sc.A,     sc.V,     sc.J,     sc.X,    sc.H,     sc.T,     sc.T2,   sc.Mt,  sc.YX,  sc.SR,
                  sc.perm,  sc.order, sc.count, sc.lamA, sc.lamK, sc.lsort, sc.stats, sc.part, sc.emax};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  sc = BJScratch();
}

#define BJ_EB (152 * 8)   // grid of the elementwise kernels

// FP64 products (df = false) or double-float (df = true)
static void zgemm(bool conj, const double2* A, int64_t lda, const double2* B, int64_t ldb, const double2* D,
                  int64_t ldd, double2* C, int64_t ldc, int M, int N, int K, double alpha, cudaStream_t s,
                  bool df = false) {
  if (M <= 0 || N <= 0) return;
  const dim3 g((M + ZG_T - 1) / ZG_T, (N + ZG_T - 1) / ZG_T);
  qm_note_launch();
  if (df) {
    if (conj)
      k_zgemm_df<true><<<g, 256, 0, s>>>(A, lda, B, ldb, D, ldd, C, ldc, M, N, K, alpha);
    else
      k_zgemm_df<false><<<g, 256, 0, s>>>(A, lda, B, ldb, D, ldd, C, ldc, M, N, K, alpha);
  } else if (conj) {
    k_zgemm<true><<<g, 256, 0, s>>>(A, lda, B, ldb, D, ldd, C, ldc, M, N, K, alpha);
  } else {
    k_zgemm<false><<<g, 256, 0, s>>>(A, lda, B, ldb, D, ldd, C, ldc, M, N, K, alpha);
  }
}

// FP32 blocked Jacobi of the n x n Hermitian H (stride n): eigenvalue order
// in sc.perm / sc.lamA, the FP64 basis in sc.X (columns in that order),
// ||H||_F and trace in sc.stats.
static int bj_fp32(const double2* H, int n, BJScratch& sc, cudaStream_t s, int* sweeps_out) {
  const int W = bj_round32(n);
  if (W > sc.W) return (int)cudaErrorInvalidValue;
  const int nb = W / BJ_B, np = nb / 2;
  qm_note_launch();
  k_bj_load<<<BJ_PARTS, BLOCK_THREADS, 0, s>>>(H, n, sc.A, sc.V, W, sc.part);
  qm_note_launch();
  k_bj_stats<<<1, BLOCK_THREADS, 0, s>>>(sc.part, BJ_PARTS, H, n, sc.stats);
  const int nA = np * (np - 1) / 2, nV = (W / BJ_S) * np;
  int sweeps = 0;
  for (int sweep = 0; sweep < BJ_MAX_SWEEPS; ++sweep) {
    cudaError_t e = cudaMemsetAsync(sc.count, 0, sizeof(int), s);
    if (e != cudaSuccess) return (int)e;
    for (int k = 0; k < nb - 1; ++k) {
      qm_note_launch();
      k_bj_solve<<<np, BJ_THREADS, 0, s>>>(sc.A, W, nb, k, sc.J, sc.stats, sc.count);
      if (nA + nV > 0) {
        qm_note_launch();
        k_bj_update<<<nA + nV, BJU_THREADS, 0, s>>>(sc.A, sc.V, W, nb, k, sc.J, nA);
      }
    }
    ++sweeps;
    int cnt = 0;
    e = cudaMemcpyAsync(&cnt, sc.count, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return (int)e;
    if (cnt == 0) break;
  }
  qm_note_launch();
  k_bj_sort<<<1, 1024, sizeof(float) * W, s>>>(sc.A, W, n, sc.perm, sc.lamA);
  qm_note_launch();
  k_bj_basis<<<BJ_EB, BLOCK_THREADS, 0, s>>>(sc.V, W, n, sc.perm, sc.X);
  *sweeps_out += sweeps;
  return (int)cudaGetLastError();
}

// Ogita-Aishima refinement of the first Kc columns of sc.X (eigenvectors of
// H, n x n, stride n): on return they are refined in sc.X and their
// eigenvalues in sc.lamK.
static int bj_refine(const double2* H, int n, BJScratch& sc, int Kc, double tol, bool df, cudaStream_t s,
                     int* steps_out, float* emax_out) {
  if (Kc < 1) return 0;
  if (Kc > sc.kmax) return (int)cudaErrorInvalidValue;
  if (Kc < n) {   // eigenvalue estimates of the columns that stay
    zgemm(false, H, n, sc.X + Kc, n, nullptr, 0, sc.T2, n - Kc, n, n - Kc, n, 1.0, s, df);
    qm_note_launch();
    k_bj_rq<<<n - Kc, BLOCK_THREADS, 0, s>>>(sc.X, n, sc.T2, n - Kc, Kc, sc.lamA);
  }
  double2* Xk = sc.YX + Kc;   // row stride 2 Kc
  qm_note_launch();
  k_bj_copy<<<BJ_EB, BLOCK_THREADS, 0, s>>>(sc.X, n, Xk, 2 * Kc, n, Kc);
  float emax = 0.f;
  for (int it = 0; it < BJ_MAX_REFINE; ++it) {
    // Y = H X_K into YX[:, :Kc]; [S | X^H X_K] = X^H YX
    zgemm(false, H, n, Xk, 2 * Kc, nullptr, 0, sc.YX, 2 * Kc, n, Kc, n, 1.0, s, df);
    zgemm(true, sc.X, n, sc.YX, 2 * Kc, nullptr, 0, sc.SR, 2 * Kc, n, 2 * Kc, n, 1.0, s, df);
    qm_note_launch();
    k_bj_lam<<<(Kc + 255) / 256, 256, 0, s>>>(sc.SR, Kc, sc.lamK);
    cudaError_t e = cudaMemsetAsync(sc.emax, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return (int)e;
    qm_note_launch();
    k_bj_correct<<<Kc, BLOCK_THREADS, 0, s>>>(sc.SR, n, Kc, sc.lamK, sc.lamA, df ? 1e-12 : 1e-14, sc.emax);
    // X_K += X E
    const dim3 g1((n + ZG_T - 1) / ZG_T, (Kc + ZG_T - 1) / ZG_T);
    qm_note_launch();
    if (df) {
      k_zgemm_small<<<g1, 256, 0, s>>>(sc.X, n, sc.SR, 2 * Kc, Xk, 2 * Kc, n, Kc, n);
    } else {   // the exact mode: large first corrections need their own low-order bits
      k_zgemm_df<false><<<g1, 256, 0, s>>>(sc.X, n, sc.SR, 2 * Kc, Xk, 2 * Kc, Xk, 2 * Kc, n, Kc, n, 1.0);
    }
    qm_note_launch();
    k_bj_copy<<<BJ_EB, BLOCK_THREADS, 0, s>>>(Xk, 2 * Kc, sc.X, n, n, Kc);
    ++*steps_out;
    unsigned bits = 0;
    e = cudaMemcpyAsync(&bits, sc.emax, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return (int)e;
    const float prev = emax;
    std::memcpy(&emax, &bits, sizeof(float));
    if ((double)emax <= tol) break;
    if (it > 0 && emax > 0.5f * prev) break;   // no longer converging: the rest is a cluster
  }
  if (emax > *emax_out) *emax_out = emax;
  return (int)cudaGetLastError();
}

// Diagonalise the w x w Gram of state b (stride w, at b's slot of `gram`)
// and finalize cut c.  Eigenvalues above BJ_RESOLVED of the largest are
// resolved by the FP32 sweeps and refined directly.  When the columns that
// may be kept reach below that (rank-deficient or fast-decaying spectra),
// the unresolved subspace is projected off the refined columns,
// re-orthonormalised (one Newton-Schulz step in FP64), and its own Gram
// X_N^H G X_N, whose scale is that of the small eigenvalues, is solved the
// same way in `sub`.  Synchronises the stream once per sweep and per
// refinement step.  Returns a cudaError_t.
int tt_block_eig(const BatchDev& bd, int b, int c, int wv, double2* gram, const float2* rowsrc,
                 BJScratch& sc, BJScratch& sub, int* bonds, double2* vsel, double2* tensors, int chi, int max_bond,
                 double cutoff, double refine_tol, cudaStream_t s, BJStats* st) {
  double2* G = gram + (int64_t)b * bd.tt_w * bd.tt_w;
  // the fast mode's tolerance leaves about 1e-8 of error: double-float
  // refinement products suffice there; the exact mode takes FP64 products
  const bool df = refine_tol > BJ_TOL_EXACT;
  // the Gram's size: the column Gram (wv), or the row Gram M M^H of the
  // 2^c x wv remainder
  int w = rowsrc ? (int)ipow2(c) : wv;
  if (rowsrc) {
    if (w > sc.W || wv > sc.W) return (int)cudaErrorInvalidValue;
    qm_note_launch();
    k_bj_mt<<<dim3((wv + 31) / 32, (w + 31) / 32), BLOCK_THREADS, 0, s>>>(rowsrc, w, wv, sc.Mt);
    zgemm(true, sc.Mt, w, sc.Mt, w, nullptr, 0, G, w, w, w, wv, 1.0, s, true);
  }
  int sweeps = 0, steps = 0;
  float emax = 0.f;
  int e = 0, K = 0, Kr = 0, r = 0;
  std::vector<double> lam;
  cudaError_t ce = cudaSuccess;
  for (;;) {
    if ((e = bj_fp32(G, w, sc, s, &sweeps)) != 0) return e;
    K = w;
    if (max_bond > 0 && K > max_bond) K = max_bond;
    if (K > bd.tt_b) K = bd.tt_b;
    if (c < 30 && K > (1 << c)) K = 1 << c;
    if (K > sc.kmax) return (int)cudaErrorInvalidValue;
    lam.resize(w);
    ce = cudaMemcpyAsync(lam.data(), sc.lamA, sizeof(double) * w, cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return (int)ce;
    // refined columns: the K that may be kept and the discarded ones whose
    // FP32 eigenvalue is within BJ_MARGIN of the last kept one (their order
    // and their mixing with it are below FP32 resolution)
    Kr = K;
    while (Kr < w && Kr < sc.kmax && Kr < K + BJ_EXTRA && lam[Kr] >= lam[K - 1] - BJ_MARGIN * lam[0]) ++Kr;
    r = 0;
    while (r < w && lam[r] > BJ_RESOLVED * lam[0]) ++r;
    // the split between refined and deflated columns sits at a gap (5% of
    // the eigenvalue, and 1e-6 of the largest): the pairs across it are
    // refined from one side only, which cannot resolve near-degenerate ones
    while (r > 0 && r < w && lam[r - 1] - lam[r] < fmax(0.05 * lam[r - 1], 1e-6 * lam[0])) --r;
    // the row Gram's kept right vectors M^H u / sigma carry the eigenvector
    // error times sigma_1 / sigma: kept only while every refined column is
    // resolved (sigma_1 / sigma < 316); otherwise the column Gram of the
    // same remainder, M^H M, in double-float products
    if (rowsrc && Kr > r) {
      qm_note_launch();
      k_bj_f2d<<<BJ_EB, BLOCK_THREADS, 0, s>>>(rowsrc, (int64_t)w * wv, sc.T);
      zgemm(true, sc.T, wv, sc.T, wv, nullptr, 0, G, wv, wv, wv, w, 1.0, s, true);
      rowsrc = nullptr;
      w = wv;
      continue;
    }
    break;
  }
  const bool deflated = !(Kr <= r || r == 0);
  if (!deflated) {
    e = bj_refine(G, w, sc, Kr, refine_tol, df, s, &steps, &emax);
    if (e) return e;
  } else {
    const int m = w - r, K1 = Kr - r;
    e = bj_refine(G, w, sc, r, refine_tol, df, s, &steps, &emax);
    if (e) return e;
    if (sub.W == 0 && (e = bj_alloc(sub, sc.W, sc.kmax)) != 0) return e;
    double2* Xn = sc.X + r;   // row stride w
    // X_N <- X_N - X_R (X_R^H X_N), then Newton-Schulz steps (the refined
    // columns took small one-sided corrections towards X_N, so the
    // projection shortens some columns by up to a few percent)
    zgemm(true, sc.X, w, Xn, w, nullptr, 0, sc.T, m, r, m, w, 1.0, s, df);
    zgemm(false, sc.X, w, sc.T, m, Xn, w, sc.T2, m, w, m, r, -1.0, s, df);
    for (int ns = 0; ns < 4; ++ns) {
      zgemm(true, sc.T2, m, sc.T2, m, nullptr, 0, sc.T, m, m, m, w, 1.0, s, df);
      qm_note_launch();
      k_bj_ns<<<BJ_EB, BLOCK_THREADS, 0, s>>>(sc.T, m);
      zgemm(false, sc.T2, m, sc.T, m, nullptr, 0, ns == 3 ? Xn : sc.YX, ns == 3 ? w : m, w, m, m, 1.0, s, df);
      if (ns < 3) {
        qm_note_launch();
        k_bj_copy<<<BJ_EB, BLOCK_THREADS, 0, s>>>(sc.YX, m, sc.T2, m, w, m);
      }
    }
    // Gram of the unresolved subspace, solved in `sub`
    zgemm(false, G, w, Xn, w, nullptr, 0, sc.T2, m, w, m, w, 1.0, s, df);
    zgemm(true, Xn, w, sc.T2, m, nullptr, 0, sub.H, m, m, m, w, 1.0, s, df);
    if ((e = bj_fp32(sub.H, m, sub, s, &sweeps)) != 0) return e;
    if ((e = bj_refine(sub.H, m, sub, K1, refine_tol, df, s, &steps, &emax)) != 0) return e;
    // X_N <- X_N U, the refined eigenvalues after those of the resolved part
    zgemm(false, Xn, w, sub.X, m, nullptr, 0, sc.T2, m, w, m, m, 1.0, s, df);
    qm_note_launch();
    k_bj_copy<<<BJ_EB, BLOCK_THREADS, 0, s>>>(sc.T2, m, Xn, w, w, m);
    ce = cudaMemcpyAsync(sc.lamK + r, sub.lamK, sizeof(double) * K1, cudaMemcpyDeviceToDevice, s);
    if (ce != cudaSuccess) return (int)ce;
  }
  qm_note_launch();
  k_bj_finalize<<<1, 1024, 0, s>>>(bd, b, c, w, Kr, K, r, sc.lamK, sc.stats, deflated ? sub.stats + 1 : nullptr,
                                    bonds, max_bond, cutoff, sc.order, sc.lsort);
  if (rowsrc) {   // V = M^H U Sigma^-1 (wv x K), then emitted in order
    qm_note_launch();
    k_bj_gather<<<BJ_EB, BLOCK_THREADS, 0, s>>>(sc.X, w, sc.order, sc.lsort, K, sc.T);
    zgemm(false, sc.Mt, w, sc.T, K, nullptr, 0, sc.T2, K, wv, K, w, 1.0, s, true);
    // the division by sigma_l amplifies the eigenvector's error by
    // sigma_1 / sigma_l: two Newton-Schulz steps V <- V (3I - V^H V) / 2
    // restore the isometry (the kept subspace keeps an error of at most
    // that amplification, weighted by sigma_l in the truncated state)
    for (int ns = 0; ns < 2; ++ns) {
      zgemm(true, sc.T2, K, sc.T2, K, nullptr, 0, sc.H, K, K, K, wv, 1.0, s, true);
      qm_note_launch();
      k_bj_ns<<<BJ_EB, BLOCK_THREADS, 0, s>>>(sc.H, K);
      zgemm(false, sc.T2, K, sc.H, K, nullptr, 0, sc.T, K, wv, K, K, 1.0, s, true);
      qm_note_launch();
      k_bj_copy<<<BJ_EB, BLOCK_THREADS, 0, s>>>(sc.T, K, sc.T2, K, wv, K);
    }
    qm_note_launch();
    k_bj_emit<<<K, BLOCK_THREADS, 0, s>>>(bd, b, c, sc.T2, K, wv, bonds, nullptr, vsel, bd.tt_b, tensors, chi);
  } else {
    qm_note_launch();
    k_bj_emit<<<K, BLOCK_THREADS, 0, s>>>(bd, b, c, sc.X, w, w, bonds, sc.order, vsel, bd.tt_b, tensors, chi);
  }
  if (st) {
    st->sweeps += sweeps;
    st->refine_steps += steps;
    st->calls += 1;
    if (emax > st->last_emax) st->last_emax = emax;
  }
  return (int)cudaGetLastError();
}

void launch_cgemm(const float2* A, int64_t lda, const double2* B, int64_t ldb, float2* C, int64_t ldc, int64_t M,
                  int N, int K, cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0) return;
  dim3 grid((unsigned)((M + CG_T - 1) / CG_T), (unsigned)((N + CG_T - 1) / CG_T));
  qm_note_launch();
  k_cgemm<<<grid, 256, 0, s>>>(A, lda, B, ldb, C, ldc, M, N, K);
}
