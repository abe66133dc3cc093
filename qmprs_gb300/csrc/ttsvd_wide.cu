// (a) statevector -> MPS for Gram widths above 128 (bonds above 64): the
// same right-to-left truncated SVD as ttsvd.cu, for the configurations with
// bond dimension 256 (20 qubits) and 1024 (24 qubits).
//
// The w x w Gram (w up to 2048) no longer fits one block, so the parallel
// cyclic Jacobi runs over the whole GPU with one launch per phase of each
// round (host-driven rounds, no device-wide barrier):
//   k_wj_params   rotation of every pair of the round (w/2 threads) and a
//                 rotation count per sweep;
//   k_wj_cols     G <- G J and V <- V J on the two columns of every pair;
//   k_wj_rows     G <- J^H G on the two rows of every pair, zeroing the
//                 eliminated entries.
// The host reads the rotation count once per sweep and stops when a sweep
// rotates nothing (at most TTW_MAX_SWEEPS sweeps).  The thresholds are the
// ones of the one-block solver: relative 1e-15 and an absolute floor of
// 1e-15 of the trace.
//   k_wide_finalize  eigenvalue ranks (parallel), quimb's rsum2 cutoff with
//                 max_bond, canonical phases of the kept eigenvectors, the
//                 selected columns and the site tensor;
//   k_cgemm       C = A B for a tall complex64 A and a small complex128 B
//                 (the projection M V of the remainder and the left-to-right
//                 contraction that rebuilds the dense target): 64 x 64 output
//                 tiles, K staged in shared memory, 4 x 4 outputs per
//                 thread.
#include "device_common.cuh"

#define TTW_THREADS 256
#define TTW_MAX_SWEEPS 40

struct WJRot {
  int p, q, flag;
  double c;
  double2 se, sce;
};

__global__ void k_wj_params(const double2* G, int w, int k, double floor_abs, WJRot* rot, int* count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= w / 2) return;
  const int t1 = i, t2 = w - 1 - i;
  int p = t1 == 0 ? 0 : 1 + ((t1 - 1 + k) % (w - 1));
  int q = 1 + ((t2 - 1 + k) % (w - 1));
  if (p > q) {
    const int tmp = p;
    p = q;
    q = tmp;
  }
  const double2 g = G[(int64_t)p * w + q];
  const double ag = cabs_(g);
  const double app = G[(int64_t)p * w + p].x, aqq = G[(int64_t)q * w + q].x;
  WJRot r;
  r.p = p;
  r.q = q;
  r.flag = !(ag == 0.0 || ag <= 1e-15 * sqrt(fabs(app * aqq)) || ag <= floor_abs);
  r.c = 1.0;
  r.se = r.sce = czero();
  if (r.flag) {
    const double zeta = (aqq - app) / (2.0 * ag);
    const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
    const double cc = 1.0 / sqrt(1.0 + t * t);
    const double ss = cc * t;
    const double2 e = cscale(g, 1.0 / ag);
    r.c = cc;
    r.se = cscale(e, ss);
    r.sce = cscale(cconj(e), ss);
    atomicAdd(count, 1);
  }
  rot[i] = r;
}

__global__ void k_wj_cols(double2* G, double2* V, int w, const WJRot* rot) {
  const int64_t total = (int64_t)(w / 2) * w;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx / w), row = (int)(idx % w);
    const WJRot r = rot[i];
    if (!r.flag) continue;
    const int64_t o = (int64_t)row * w;
    const double2 xp = G[o + r.p], xq = G[o + r.q];
    G[o + r.p] = csub(cscale(xp, r.c), cmul(r.sce, xq));
    G[o + r.q] = cadd(cmul(r.se, xp), cscale(xq, r.c));
    const double2 vp = V[o + r.p], vq = V[o + r.q];
    V[o + r.p] = csub(cscale(vp, r.c), cmul(r.sce, vq));
    V[o + r.q] = cadd(cmul(r.se, vp), cscale(vq, r.c));
  }
}

__global__ void k_wj_rows(double2* G, int w, const WJRot* rot) {
  const int64_t total = (int64_t)(w / 2) * w;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx / w), col = (int)(idx % w);
    const WJRot r = rot[i];
    if (!r.flag) continue;
    const int64_t op = (int64_t)r.p * w, oq = (int64_t)r.q * w;
    const double2 xp = G[op + col], xq = G[oq + col];
    double2 np_ = csub(cscale(xp, r.c), cmul(r.se, xq));
    double2 nq = cadd(cmul(r.sce, xp), cscale(xq, r.c));
    if (col == r.q) np_ = czero();          // the eliminated pair
    if (col == r.p) {
      nq = czero();
      np_.y = 0.0;                           // real diagonal
    }
    if (col == r.q) nq.y = 0.0;
    G[op + col] = np_;
    G[oq + col] = nq;
  }
}

__global__ void k_wj_init(const double2* G, double2* V, int w, double* trace) {
  const int64_t total = (int64_t)w * w;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    V[e] = cd((e / w) == (e % w) ? 1.0 : 0.0, 0.0);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double tr = 0.0;
    for (int i = 0; i < w; ++i) tr += fabs(G[(int64_t)i * w + i].x);
    *trace = tr;
  }
}

// Descending order of the diagonal (ties by index), rsum2 cutoff, phases,
// selected columns (stride vstride) and the site tensor of cut c.  One block.
__global__ void __launch_bounds__(1024) k_wide_finalize(BatchDev bd, int b, int c, const double2* G, double2* V,
                                                         int w, int* bonds, double2* vsel, int vstride,
                                                         double2* tensors, int chi, int max_bond, double cutoff,
                                                         int* perm, double* lam) {
  __shared__ int s_keep;
  for (int i = threadIdx.x; i < w; i += blockDim.x) {
    const double li = G[(int64_t)i * w + i].x;
    int rank = 0;
    for (int j = 0; j < w; ++j) {
      const double lj = G[(int64_t)j * w + j].x;
      rank += (lj > li) || (lj == li && j < i);
    }
    perm[rank] = i;
    lam[rank] = li;
  }
  __syncthreads();
  int* bond = bonds + (int64_t)b * (bd.max_n + 1);
  if (threadIdx.x == 0) {
    int keep = rank_by_cutoff(lam, w, cutoff, max_bond);
    if (keep > bd.tt_b) keep = bd.tt_b;
    if (c < 30 && keep > (1 << c)) keep = 1 << c;
    s_keep = keep;
    bond[c] = keep;
  }
  __syncthreads();
  const int keep = s_keep;
  for (int col = threadIdx.x; col < keep; col += blockDim.x) phase_fix_column(V, w, w, perm[col]);
  __syncthreads();
  double2* vs = vsel + (int64_t)b * bd.tt_w * bd.tt_w;
  for (int64_t e = threadIdx.x; e < (int64_t)w * keep; e += blockDim.x) {
    const int a = (int)(e / keep), col = (int)(e % keep);
    vs[(int64_t)a * vstride + col] = V[(int64_t)a * w + perm[col]];
  }
  const int r = w / 2;
  const int n = bd.n[b];
  const int ce = chi < (1 << (n / 2)) ? chi : (1 << (n / 2));
  double2* ts = tensors + bd.tensor_off[b] + (int64_t)c * 2 * ce * ce;
  for (int64_t e = threadIdx.x; e < (int64_t)keep * 2 * r; e += blockDim.x) {
    const int l = (int)(e / (2 * r)), pr = (int)(e % (2 * r));
    ts[e] = cconj(V[(int64_t)pr * w + perm[l]]);
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

// Diagonalise the w x w Gram of state b (in place in `gram`, stride w) with
// eigenvectors in `vwork`, then finalize cut c.  Synchronises the stream
// once per sweep.  Returns a cudaError_t.
int tt_wide_eig(const BatchDev& bd, int b, int c, int w, double2* gram, double2* vwork, WJRot* rot, int* d_count,
                double* d_trace, int* perm, double* lam, int* bonds, double2* vsel, double2* tensors, int chi,
                int max_bond, double cutoff, cudaStream_t s) {
  const int64_t off = (int64_t)b * bd.tt_w * bd.tt_w;
  double2* G = gram + off;
  double2* V = vwork + off;
  const int64_t ww = (int64_t)w * w;
  int blocks = (int)((ww / 2 + TTW_THREADS - 1) / TTW_THREADS);
  if (blocks > 152 * 16) blocks = 152 * 16;
  qm_note_launch();
  k_wj_init<<<blocks, TTW_THREADS, 0, s>>>(G, V, w, d_trace);
  double tr = 0.0;
  cudaError_t e = cudaMemcpyAsync(&tr, d_trace, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return (int)e;
  const double floor_abs = 1e-15 * tr;
  const int pblocks = (w / 2 + 127) / 128;
  for (int sweep = 0; sweep < TTW_MAX_SWEEPS; ++sweep) {
    e = cudaMemsetAsync(d_count, 0, sizeof(int), s);
    if (e != cudaSuccess) return (int)e;
    for (int k = 0; k < w - 1; ++k) {
      qm_note_launch();
      k_wj_params<<<pblocks, 128, 0, s>>>(G, w, k, floor_abs, rot, d_count);
      qm_note_launch();
      k_wj_cols<<<blocks, TTW_THREADS, 0, s>>>(G, V, w, rot);
      qm_note_launch();
      k_wj_rows<<<blocks, TTW_THREADS, 0, s>>>(G, w, rot);
    }
    int cnt = 0;
    e = cudaMemcpyAsync(&cnt, d_count, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return (int)e;
    if (cnt == 0) break;
  }
  qm_note_launch();
  k_wide_finalize<<<1, 1024, 0, s>>>(bd, b, c, G, V, w, bonds, vsel, bd.tt_b, tensors, chi, max_bond, cutoff, perm,
                                     lam);
  return (int)cudaGetLastError();
}

void launch_cgemm(const float2* A, int64_t lda, const double2* B, int64_t ldb, float2* C, int64_t ldc, int64_t M,
                  int N, int K, cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0) return;
  dim3 grid((unsigned)((M + CG_T - 1) / CG_T), (unsigned)((N + CG_T - 1) / CG_T));
  qm_note_launch();
  k_cgemm<<<grid, 256, 0, s>>>(A, lda, B, ldb, C, ldc, M, N, K);
}

size_t wj_rot_bytes(int w) { return sizeof(WJRot) * (size_t)(w / 2 + 1); }
