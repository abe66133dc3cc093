// Small dense FP64 linear algebra used inside the kernels (one thread each).
//
// Everything here is __host__ __device__ so that the same code is compiled
// into the CUDA library and into a host-only check library; tests compare
// the host build against the FP64 oracle before any GPU run.
//
// Contents
//   herm_eig_jacobi      cyclic complex Jacobi eigensolver (Hermitian, n <= 8)
//   phase_fix_column     canonical singular-vector phase (pivot entry > 0)
//   rank_by_cutoff       quimb's "rsum2" truncation rule, then max_bond
//   householder_complement  canonical orthonormal completion (pivoted
//                        Householder product), n <= 4
//   polar_jacobi         unitary polar factor of a 2x2 / 4x4 matrix via
//                        one-sided (Hestenes) Jacobi SVD; also returns the
//                        nuclear norm
//   ran_gate_*           the reference's gate construction in closed form
//
// Method references: Jacobi eigenvalue method with the Rutishauser-style
// stable rotation (t = sgn(z) / (|z| + sqrt(1 + z^2))), Hestenes one-sided
// Jacobi SVD, Householder reflections (Golub & Van Loan, Matrix
// Computations, ch. 5 and 8).
#pragma once

#include "qm_complex.h"

#define QM_PIVOT_TOL 1e-6
#define QM_ZERO_TOL 1e-12
#define QM_CUTOFF 1e-10

// --------------------------------------------------------------------------
// Hermitian eigen-decomposition, matrices stored row-major a[i*n + j].
// On return lam[] is descending and column k of v holds its eigenvector.
// --------------------------------------------------------------------------
QM_HD void herm_eig_jacobi(double2* a, int n, double2* v, double* lam) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) v[i * n + j] = cd(i == j ? 1.0 : 0.0, 0.0);
  // absolute floor: off-diagonals at most 1e-15 of the trace move no
  // eigenvalue by more than that; without it the rounding-level null block
  // of a rank-deficient matrix keeps rotating until the sweep limit
  double tr = 0.0;
  for (int i = 0; i < n; ++i) tr += fabs(a[i * n + i].x);
  const double floor_abs = 1e-15 * tr;
  for (int sweep = 0; sweep < 60; ++sweep) {
    int rotated = 0;
    for (int p = 0; p < n - 1; ++p) {
      for (int q = p + 1; q < n; ++q) {
        double2 g = a[p * n + q];
        double ag = cabs_(g);
        double app = a[p * n + p].x, aqq = a[q * n + q].x;
        if (ag == 0.0 || ag <= 1e-17 * sqrt(fabs(app * aqq)) || ag <= floor_abs) continue;
        rotated = 1;
        double zeta = (aqq - app) / (2.0 * ag);
        double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        double c = 1.0 / sqrt(1.0 + t * t);
        double s = c * t;
        double2 e = cscale(g, 1.0 / ag);
        double2 se = cscale(e, s);          // s e
        double2 sce = cscale(cconj(e), s);  // s conj(e)
        // columns: col_p <- c col_p - s conj(e) col_q ; col_q <- s e col_p + c col_q
        for (int i = 0; i < n; ++i) {
          double2 xp = a[i * n + p], xq = a[i * n + q];
          a[i * n + p] = csub(cscale(xp, c), cmul(sce, xq));
          a[i * n + q] = cadd(cmul(se, xp), cscale(xq, c));
          double2 vp = v[i * n + p], vq = v[i * n + q];
          v[i * n + p] = csub(cscale(vp, c), cmul(sce, vq));
          v[i * n + q] = cadd(cmul(se, vp), cscale(vq, c));
        }
        // rows: row_p <- c row_p - s e row_q ; row_q <- s conj(e) row_p + c row_q
        for (int j = 0; j < n; ++j) {
          double2 xp = a[p * n + j], xq = a[q * n + j];
          a[p * n + j] = csub(cscale(xp, c), cmul(se, xq));
          a[q * n + j] = cadd(cmul(sce, xp), cscale(xq, c));
        }
        a[p * n + q] = czero();
        a[q * n + p] = czero();
        a[p * n + p].y = 0.0;
        a[q * n + q].y = 0.0;
      }
    }
    if (!rotated) break;
  }
  int idx[8];
  for (int i = 0; i < n; ++i) { idx[i] = i; lam[i] = a[i * n + i].x; }
  // stable insertion sort, descending
  for (int i = 1; i < n; ++i) {
    int k = idx[i];
    double key = lam[i];
    int j = i - 1;
    while (j >= 0 && lam[j] < key) { lam[j + 1] = lam[j]; idx[j + 1] = idx[j]; --j; }
    lam[j + 1] = key;
    idx[j + 1] = k;
  }
  double2 tmp[64];
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < n; ++c) tmp[i * n + c] = v[i * n + idx[c]];
  for (int i = 0; i < n * n; ++i) v[i] = tmp[i];
}

// Pivot: lowest index whose magnitude is >= (1 - QM_PIVOT_TOL) * max.
// `stride` walks a column of a row-major matrix; `used` (may be null) masks
// indices that are excluded.
QM_HD int pivot_index(const double2* x, int n, int stride, const int* used) {
  double m = -1.0;
  for (int i = 0; i < n; ++i) {
    if (used && used[i]) continue;
    double a = cabs_(x[i * stride]);
    if (a > m) m = a;
  }
  for (int i = 0; i < n; ++i) {
    if (used && used[i]) continue;
    if (cabs_(x[i * stride]) >= (1.0 - QM_PIVOT_TOL) * m) return i;
  }
  return 0;
}

// Make the pivot entry of column `col` (row-major n x ncols) real positive.
QM_HD void phase_fix_column(double2* v, int n, int ncols, int col) {
  int j = pivot_index(v + col, n, ncols, nullptr);
  double2 z = v[j * ncols + col];
  double az = cabs_(z);
  if (az <= 0.0) return;
  double2 ph = cscale(cconj(z), 1.0 / az);
  for (int i = 0; i < n; ++i) v[i * ncols + col] = cmul(v[i * ncols + col], ph);
}

// quimb rsum2 rule on squared singular values (descending, may hold tiny
// negatives from rounding), then capped by max_bond; at least 1.
QM_HD int rank_by_cutoff(const double* sq_in, int n, double cutoff, int max_bond) {
  double total = 0.0;
  for (int i = 0; i < n; ++i) total += sq_in[i] > 0.0 ? sq_in[i] : 0.0;
  int keep = 0;
  if (total <= 0.0) {
    keep = 1;
  } else {
    double tail = 0.0;
    for (int i = n - 1; i >= 0; --i) {
      tail += sq_in[i] > 0.0 ? sq_in[i] : 0.0;
      if (tail > cutoff * total) { keep = i + 1; break; }
    }
    if (keep < 1) keep = 1;
  }
  if (max_bond > 0 && keep > max_bond) keep = max_bond;
  return keep;
}

// The same rule when only the largest Kr eigenvalues are known (descending
// in lsort) and `rest` is the weight of all the others: tail sums are
// formed from the bottom, rest + sum_{i <= j < Kr} l_j, so that no sum near
// the total is subtracted from the total; the keep count is capped at K
// (<= Kr) and by max_bond; total is the trace.  With Kr = n and rest = 0
// it equals rank_by_cutoff up to the total's rounding.
QM_HD int rank_from_tails(const double* lsort, int Kr, int K, double rest, double total, double cutoff,
                          int max_bond) {
  double tail = rest > 0.0 ? rest : 0.0;
  for (int i = Kr - 1; i >= K; --i) tail += lsort[i] > 0.0 ? lsort[i] : 0.0;
  int keep = 0;
  if (tail > cutoff * total) keep = K;   // tail_from(K): more than K would be kept
  for (int i = K - 1; i >= 0 && keep == 0; --i) {
    tail += lsort[i] > 0.0 ? lsort[i] : 0.0;
    if (tail > cutoff * total) keep = i + 1;
  }
  if (keep < 1) keep = 1;
  if (max_bond > 0 && keep > max_bond) keep = max_bond;
  return keep;
}

// Pair i (0 <= i < n/2) of round k (0 <= k < n-1) of the round-robin
// tournament over n (even) indices, p < q: index 0 stays, 1..n-1 rotate.
// The rounds of a sweep are perfect matchings and meet every pair once
// (Golub & Van Loan, Matrix Computations, 4th ed., sec. 8.5.4).
QM_HD void round_robin_pair(int n, int k, int i, int* p, int* q) {
  const int t2 = n - 1 - i;
  int a = i == 0 ? 0 : 1 + ((i - 1 + k) % (n - 1));
  int b = 1 + ((t2 - 1 + k) % (n - 1));
  if (a > b) {
    const int t = a;
    a = b;
    b = t;
  }
  *p = a;
  *q = b;
}

// v <- v - w * (2 <w, v> / <w, w>)
QM_HD void householder_apply(const double2* w, double2* v, int n) {
  double2 dot = czero();
  double ww = 0.0;
  for (int i = 0; i < n; ++i) { dot = cadd(dot, cmulc(w[i], v[i])); ww += cnorm2(w[i]); }
  double2 f = cscale(dot, 2.0 / ww);
  for (int i = 0; i < n; ++i) v[i] = csub(v[i], cmul(w[i], f));
}

// Canonical orthonormal complement of k orthonormal kets (rows of x, k x n,
// row-major), n <= 4.  Writes the (n - k) columns into cols[c * n + i].
QM_HD void householder_complement(const double2* x, int k, int n, double2* cols) {
  double2 ws[4][4];
  int used[4] = {0, 0, 0, 0};
  for (int a = 0; a < k; ++a) {
    double2 v[4];
    for (int i = 0; i < n; ++i) v[i] = x[a * n + i];
    for (int b = 0; b < a; ++b) householder_apply(ws[b], v, n);
    for (int i = 0; i < n; ++i) if (used[i]) v[i] = czero();
    int j = pivot_index(v, n, 1, used);
    double av = cabs_(v[j]);
    double2 ph = av > 0.0 ? cscale(v[j], 1.0 / av) : cd(1.0, 0.0);
    for (int i = 0; i < n; ++i) ws[a][i] = cmulc(ph, v[i]);   // conj(phase) * v
    ws[a][j].x += 1.0;
    used[j] = 1;
  }
  int c = 0;
  for (int j = 0; j < n; ++j) {
    if (used[j]) continue;
    double2 v[4];
    for (int i = 0; i < n; ++i) v[i] = cd(i == j ? 1.0 : 0.0, 0.0);
    for (int b = k - 1; b >= 0; --b) householder_apply(ws[b], v, n);
    for (int i = 0; i < n; ++i) cols[c * n + i] = v[i];
    ++c;
  }
}

// One-sided (Hestenes) Jacobi on the `nc` columns (length m <= 4) of a
// (column-major a[col][row]): on return a = U S and vv (nc x nc,
// column-major) = V with A_in V = U S.
QM_HD void onesided_jacobi(double2 (&a)[4][4], int m, int nc, double2 (&vv)[4][4]) {
  for (int c = 0; c < nc; ++c)
    for (int r = 0; r < nc; ++r) vv[c][r] = cd(r == c ? 1.0 : 0.0, 0.0);
  for (int sweep = 0; sweep < 60; ++sweep) {
    int rotated = 0;
    for (int p = 0; p < nc - 1; ++p) {
      for (int q = p + 1; q < nc; ++q) {
        double alpha = 0.0, beta = 0.0;
        double2 gam = czero();
        for (int r = 0; r < m; ++r) {
          alpha += cnorm2(a[p][r]);
          beta += cnorm2(a[q][r]);
          gam = cadd(gam, cmulc(a[p][r], a[q][r]));
        }
        double ag = cabs_(gam);
        if (ag == 0.0 || ag <= 1e-15 * sqrt(alpha * beta)) continue;
        rotated = 1;
        double zeta = (beta - alpha) / (2.0 * ag);
        double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        double c = 1.0 / sqrt(1.0 + t * t);
        double s = c * t;
        double2 ph = cscale(gam, 1.0 / ag);
        double2 se = cscale(ph, s), sce = cscale(cconj(ph), s);
        for (int r = 0; r < m; ++r) {
          double2 xp = a[p][r], xq = a[q][r];
          a[p][r] = csub(cscale(xp, c), cmul(sce, xq));
          a[q][r] = cadd(cmul(se, xp), cscale(xq, c));
        }
        for (int r = 0; r < nc; ++r) {
          double2 vp = vv[p][r], vq = vv[q][r];
          vv[p][r] = csub(cscale(vp, c), cmul(sce, vq));
          vv[q][r] = cadd(cmul(se, vp), cscale(vq, c));
        }
      }
    }
    if (!rotated) break;
  }
}

// Orthonormal columns u[c] (length m) for the columns of a = U S; columns
// whose norm is not above `tiny` are completed by Gram-Schmidt on e_0, e_1,
// ... against `fixed` (first nfixed columns of fx) and the others.
QM_HD void normalise_or_complete(double2 (&a)[4][4], int m, int nc, double tiny, const double2 (*fx)[4],
                                 int nfixed, double2 (&u)[4][4]) {
  int ok[4] = {0, 0, 0, 0};
  for (int c = 0; c < nc; ++c) {
    double nrm = 0.0;
    for (int r = 0; r < m; ++r) nrm += cnorm2(a[c][r]);
    nrm = sqrt(nrm);
    if (nrm > tiny && isfinite(nrm)) {
      for (int r = 0; r < m; ++r) u[c][r] = cscale(a[c][r], 1.0 / nrm);
      ok[c] = 1;
    }
  }
  for (int c = 0; c < nc; ++c) {
    if (ok[c]) continue;
    for (int k = 0; k < m; ++k) {
      double2 v[4];
      for (int r = 0; r < m; ++r) v[r] = cd(r == k ? 1.0 : 0.0, 0.0);
      for (int pass = 0; pass < 2; ++pass) {
        for (int o = 0; o < nfixed + nc; ++o) {
          const double2* col;
          if (o < nfixed) col = fx[o];
          else if (ok[o - nfixed]) col = u[o - nfixed];
          else continue;
          double2 d = czero();
          for (int r = 0; r < m; ++r) d = cadd(d, cmulc(col[r], v[r]));
          for (int r = 0; r < m; ++r) v[r] = csub(v[r], cmul(col[r], d));
        }
      }
      double nv = 0.0;
      for (int r = 0; r < m; ++r) nv += cnorm2(v[r]);
      nv = sqrt(nv);
      if (nv > 0.5) {
        for (int r = 0; r < m; ++r) u[c][r] = cscale(v[r], 1.0 / nv);
        ok[c] = 1;
        break;
      }
    }
  }
}

#define QM_POLAR_NULL_TOL 1e-6

// One Hestenes rotation of columns p, q of a (length M) and of v (length M),
// restricted to pairs where both `use` flags are set.  Returns 1 if rotated.
template <int M>
QM_HD int jacobi_pair(double2 (&a)[M][M], double2 (&v)[M][M], int p, int q) {
  double alpha = 0.0, beta = 0.0;
  double2 gam = czero();
#pragma unroll
  for (int r = 0; r < M; ++r) {
    alpha += cnorm2(a[p][r]);
    beta += cnorm2(a[q][r]);
    gam = cadd(gam, cmulc(a[p][r], a[q][r]));
  }
  const double ag2 = cnorm2(gam);
  if (ag2 == 0.0 || ag2 <= 1e-30 * alpha * beta) return 0;
  const double ag = sqrt(ag2);
  const double zeta = (beta - alpha) / (2.0 * ag);
  const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
  const double c = 1.0 / sqrt(1.0 + t * t);
  const double s = c * t;
  const double2 ph = cscale(gam, 1.0 / ag);
  const double2 se = cscale(ph, s), sce = cscale(cconj(ph), s);
#pragma unroll
  for (int r = 0; r < M; ++r) {
    const double2 xp = a[p][r], xq = a[q][r];
    a[p][r] = csub(cscale(xp, c), cmul(sce, xq));
    a[q][r] = cadd(cmul(se, xp), cscale(xq, c));
    const double2 vp = v[p][r], vq = v[q][r];
    v[p][r] = csub(cscale(vp, c), cmul(sce, vq));
    v[q][r] = cadd(cmul(se, vp), cscale(vq, c));
  }
  return 1;
}

// Hestenes sweeps over the column pairs (p < q) whose mask bits are both set.
template <int M>
QM_HD void jacobi_sweeps(double2 (&a)[M][M], double2 (&v)[M][M], int mask) {
  for (int sweep = 0; sweep < 60; ++sweep) {
    int rotated = 0;
#pragma unroll
    for (int p = 0; p < M - 1; ++p)
#pragma unroll
      for (int q = p + 1; q < M; ++q)
        if (((mask >> p) & 1) && ((mask >> q) & 1)) rotated |= jacobi_pair<M>(a, v, p, q);
    if (!rotated) break;
  }
}

// Gram-Schmidt completion of column c of u (length M) on e_0, e_1, ...
// against the columns of u selected by `against`.
template <int M>
QM_HD void complete_column(double2 (&u)[M][M], int c, int against) {
#pragma unroll
  for (int k = 0; k < M; ++k) {
    double2 v[M];
#pragma unroll
    for (int r = 0; r < M; ++r) v[r] = cd(r == k ? 1.0 : 0.0, 0.0);
    for (int pass = 0; pass < 2; ++pass)
#pragma unroll
      for (int o = 0; o < M; ++o) {
        if (!((against >> o) & 1)) continue;
        double2 d = czero();
#pragma unroll
        for (int r = 0; r < M; ++r) d = cadd(d, cmulc(u[o][r], v[r]));
#pragma unroll
        for (int r = 0; r < M; ++r) v[r] = csub(v[r], cmul(u[o][r], d));
      }
    double nv = 0.0;
#pragma unroll
    for (int r = 0; r < M; ++r) nv += cnorm2(v[r]);
    nv = sqrt(nv);
    if (nv > 0.5) {
#pragma unroll
      for (int r = 0; r < M; ++r) u[c][r] = cscale(v[r], 1.0 / nv);
      return;
    }
  }
}

// Unitary polar factor W (row-major M x M, M in {2, 4}) of E: the maximiser
// of Re Tr(W^H E), via one-sided Jacobi SVD E V = U S, W = U V^H.  Singular
// values at most QM_POLAR_NULL_TOL * s_max are treated as zero: on that
// null space every completion maximises Re Tr(W^H E), and W takes the one
// nearest to `w_prev` (if not null), the orthogonal-Procrustes fit
// W_N = polar((I - U_s U_s^H) w_prev V_N).  Returns the nuclear norm of E.
// Every loop has a compile-time trip count so the arrays stay in registers;
// the null-space completion (rank-deficient E only) is a separate,
// non-inlined function so the common path keeps only E's U S and V live.
#if defined(__CUDACC__)
#define QM_NOINLINE __noinline__
#else
#define QM_NOINLINE
#endif

template <int M>
QM_HD QM_NOINLINE void polar_null_part(const double2 (&u)[M][M], const double2 (&vv)[M][M], int smask, int nmask,
                                       const double2* w_prev, double2* w_out);

template <int M>
QM_HD void jacobi_precondition(double2 (&a)[M][M], double2 (&vv)[M][M]);

// PRE: start the FP64 sweeps from FP32 ones (jacobi_precondition); the
// FP64 sweeps then converge in one or two rounds instead of six to eight,
// with the same stopping rule and the same result to FP64 rounding.
template <int M, bool PRE = false>
QM_HD double polar_jacobi_m(const double2* e, double2* w_out, const double2* w_prev) {
  double2 a[M][M], vv[M][M];
#pragma unroll
  for (int c = 0; c < M; ++c)
#pragma unroll
    for (int r = 0; r < M; ++r) {
      a[c][r] = e[r * M + c];
      vv[c][r] = cd(r == c ? 1.0 : 0.0, 0.0);
    }
  if constexpr (PRE) jacobi_precondition<M>(a, vv);
  jacobi_sweeps<M>(a, vv, (1 << M) - 1);
  double sig[M], smax = 0.0, nuc = 0.0;
#pragma unroll
  for (int c = 0; c < M; ++c) {
    double nrm = 0.0;
#pragma unroll
    for (int r = 0; r < M; ++r) nrm += cnorm2(a[c][r]);
    sig[c] = sqrt(nrm);
    nuc += sig[c];
    smax = sig[c] > smax ? sig[c] : smax;
  }
  const double thr = QM_POLAR_NULL_TOL * smax;
  int smask = 0;
#pragma unroll
  for (int c = 0; c < M; ++c)
    if (sig[c] > thr && sig[c] > 1e-300) smask |= 1 << c;
  const int nmask = ((1 << M) - 1) & ~smask;
  // a <- U (significant columns normalised in place)
#pragma unroll
  for (int c = 0; c < M; ++c)
#pragma unroll
    for (int r = 0; r < M; ++r) a[c][r] = ((smask >> c) & 1) ? cscale(a[c][r], 1.0 / sig[c]) : czero();
#pragma unroll
  for (int r = 0; r < M; ++r)
#pragma unroll
    for (int s = 0; s < M; ++s) {
      double2 acc = czero();
#pragma unroll
      for (int c = 0; c < M; ++c)
        if ((smask >> c) & 1) acc = cadd(acc, cmul(a[c][r], cconj(vv[c][s])));
      w_out[r * M + s] = acc;
    }
  if (nmask != 0) {
    // copies whose address escapes into the non-inlined call, so that a and
    // vv themselves never need a memory home
    double2 ua[M][M], uv[M][M];
#pragma unroll
    for (int c = 0; c < M; ++c)
#pragma unroll
      for (int r = 0; r < M; ++r) {
        ua[c][r] = a[c][r];
        uv[c][r] = vv[c][r];
      }
    polar_null_part<M>(ua, uv, smask, nmask, w_prev, w_out);
  }
  return nuc;
}

template <int M>
QM_HD QM_NOINLINE void polar_null_part(const double2 (&us)[M][M], const double2 (&vv)[M][M], int smask, int nmask,
                                       const double2* w_prev, double2* w_out) {
  double2 u[M][M];
#pragma unroll
  for (int c = 0; c < M; ++c)
#pragma unroll
    for (int r = 0; r < M; ++r) u[c][r] = us[c][r];
  // null part: X[:, c] = (I - U_s U_s^H) w_prev V[:, c] for null c
  double2 x[M][M], vx[M][M];
#pragma unroll
  for (int c = 0; c < M; ++c) {
#pragma unroll
    for (int r = 0; r < M; ++r) {
      double2 acc = czero();
      if (w_prev && ((nmask >> c) & 1)) {
#pragma unroll
        for (int k = 0; k < M; ++k) acc = cadd(acc, cmul(w_prev[r * M + k], vv[c][k]));
      }
      x[c][r] = acc;
      vx[c][r] = cd(r == c ? 1.0 : 0.0, 0.0);
    }
#pragma unroll
    for (int i = 0; i < M; ++i) {
      if (!((smask >> i) & 1)) continue;
      double2 d = czero();
#pragma unroll
      for (int r = 0; r < M; ++r) d = cadd(d, cmulc(u[i][r], x[c][r]));
#pragma unroll
      for (int r = 0; r < M; ++r) x[c][r] = csub(x[c][r], cmul(u[i][r], d));
    }
  }
  jacobi_sweeps<M>(x, vx, nmask);
  // orthonormal null columns: normalise, complete the tiny ones in order
  int okmask = smask;
#pragma unroll
  for (int c = 0; c < M; ++c) {
    if (!((nmask >> c) & 1)) continue;
    double nrm = 0.0;
#pragma unroll
    for (int r = 0; r < M; ++r) nrm += cnorm2(x[c][r]);
    nrm = sqrt(nrm);
    if (nrm > 1e-8 && isfinite(nrm)) {
#pragma unroll
      for (int r = 0; r < M; ++r) u[c][r] = cscale(x[c][r], 1.0 / nrm);
      okmask |= 1 << c;
    }
  }
#pragma unroll
  for (int c = 0; c < M; ++c) {
    if (!((nmask >> c) & 1) || ((okmask >> c) & 1)) continue;
    complete_column<M>(u, c, okmask);
    okmask |= 1 << c;
  }
  // W += Q V_N^H, Q[:, j] = sum_{i null} u_i conj(vx[i][j])
#pragma unroll
  for (int j = 0; j < M; ++j) {
    if (!((nmask >> j) & 1)) continue;
    double2 q[M];
#pragma unroll
    for (int r = 0; r < M; ++r) {
      double2 acc = czero();
#pragma unroll
      for (int i = 0; i < M; ++i)
        if ((nmask >> i) & 1) acc = cadd(acc, cmul(u[i][r], cconj(vx[i][j])));
      q[r] = acc;
    }
#pragma unroll
    for (int r = 0; r < M; ++r)
#pragma unroll
      for (int s = 0; s < M; ++s) w_out[r * M + s] = cadd(w_out[r * M + s], cmul(q[r], cconj(vv[j][s])));
  }
}

// ---------------------------------------------------------------------------
// Polar factor for the sweep kernel.  GB300 issues FP64 at a small fraction
// of the FP32 rate, and a single thread's FP64 chain costs a full warp
// instruction per operation, so the Hestenes sweeps run in FP32 and only the
// final step is FP64: W = U V^H is re-orthonormalised by modified
// Gram-Schmidt in FP64 (unitary to rounding) and the overlap after the
// update is Re Tr(W^H E) in FP64.  W maximises that trace, so the 1e-7
// difference from the exact polar factor changes it only at second order.
// Singular values below QM_POLAR_NULL_TOL * s_max are null as in
// polar_jacobi_m, completed towards w_prev.
// ---------------------------------------------------------------------------
QM_HD float2 fcmul(float2 a, float2 b) { return cf(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
QM_HD float2 fcmulc(float2 a, float2 b) { return cf(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x); }
QM_HD float fcnorm2(float2 a) { return a.x * a.x + a.y * a.y; }
QM_HD float2 fcscale(float2 a, float s) { return cf(a.x * s, a.y * s); }
QM_HD float2 fcadd(float2 a, float2 b) { return cf(a.x + b.x, a.y + b.y); }
QM_HD float2 fcsub(float2 a, float2 b) { return cf(a.x - b.x, a.y - b.y); }

template <int M>
QM_HD int jacobi_pair_f(float2 (&a)[M][M], float2 (&v)[M][M], int p, int q) {
  float alpha = 0.f, beta = 0.f;
  float2 gam = cf(0.f, 0.f);
#pragma unroll
  for (int r = 0; r < M; ++r) {
    alpha += fcnorm2(a[p][r]);
    beta += fcnorm2(a[q][r]);
    gam = fcadd(gam, fcmulc(a[p][r], a[q][r]));
  }
  const float ag2 = fcnorm2(gam);
  // converged at |gam| <= 1e-6 sqrt(alpha beta): FP32 rounding leaves
  // |gam| near 1e-7 of it, so a tighter test never ends the sweeps (30 of
  // them); the polar factor's fidelity moves at second order in what is
  // left, and the FP64 preconditioned solver finishes from it anyway
  if (ag2 == 0.f || ag2 <= 1e-12f * alpha * beta) return 0;
  const float ag = sqrtf(ag2);
  const float zeta = (beta - alpha) / (2.f * ag);
  const float t = (zeta >= 0.f ? 1.f : -1.f) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
  const float c = 1.f / sqrtf(1.f + t * t);
  const float s = c * t;
  const float2 ph = fcscale(gam, 1.f / ag);
  const float2 se = fcscale(ph, s), sce = fcscale(cf(ph.x, -ph.y), s);
#pragma unroll
  for (int r = 0; r < M; ++r) {
    const float2 xp = a[p][r], xq = a[q][r];
    a[p][r] = fcsub(fcscale(xp, c), fcmul(sce, xq));
    a[q][r] = fcadd(fcmul(se, xp), fcscale(xq, c));
    const float2 vp = v[p][r], vq = v[q][r];
    v[p][r] = fcsub(fcscale(vp, c), fcmul(sce, vq));
    v[q][r] = fcadd(fcmul(se, vp), fcscale(vq, c));
  }
  return 1;
}

template <int M>
QM_HD void jacobi_sweeps_f(float2 (&a)[M][M], float2 (&v)[M][M], int mask) {
  for (int sweep = 0; sweep < 30; ++sweep) {
    int rotated = 0;
#pragma unroll
    for (int p = 0; p < M - 1; ++p)
#pragma unroll
      for (int q = p + 1; q < M; ++q)
        if (((mask >> p) & 1) && ((mask >> q) & 1)) rotated |= jacobi_pair_f<M>(a, v, p, q);
    if (!rotated) break;
  }
}

// Preconditioner of the FP64 one-sided Jacobi: FP32 Hestenes sweeps on a
// float copy of the columns of a (scaled by a power of two) give V0 to
// FP32 accuracy; V0 is made unitary in FP64 (modified Gram-Schmidt, twice)
// and a <- a V0, vv <- V0, so the FP64 sweeps that follow start from
// nearly orthogonal columns.  GB300's FP64 units run a single thread's
// dependent chain at about 31 ns per operation, FP32 at about 2 ns.
template <int M>
QM_HD void jacobi_precondition(double2 (&a)[M][M], double2 (&vv)[M][M]) {
  double amax = 0.0;
#pragma unroll
  for (int c = 0; c < M; ++c)
#pragma unroll
    for (int r = 0; r < M; ++r) amax = fmax(amax, fmax(fabs(a[c][r].x), fabs(a[c][r].y)));
  if (!(amax > 0.0) || !isfinite(amax)) return;
  int ex = 0;
  frexp(amax, &ex);
  float2 a32[M][M], v32[M][M];
#pragma unroll
  for (int c = 0; c < M; ++c)
#pragma unroll
    for (int r = 0; r < M; ++r) {
      a32[c][r] = cf((float)ldexp(a[c][r].x, -ex), (float)ldexp(a[c][r].y, -ex));
      v32[c][r] = cf(r == c ? 1.f : 0.f, 0.f);
    }
  jacobi_sweeps_f<M>(a32, v32, (1 << M) - 1);
  double2 v[M][M];
#pragma unroll
  for (int c = 0; c < M; ++c) {
#pragma unroll
    for (int r = 0; r < M; ++r) v[c][r] = f2d(v32[c][r]);
    for (int pass = 0; pass < 2; ++pass) {
#pragma unroll
      for (int o = 0; o < c; ++o) {
        double2 d = czero();
#pragma unroll
        for (int r = 0; r < M; ++r) d = cadd(d, cmulc(v[o][r], v[c][r]));
#pragma unroll
        for (int r = 0; r < M; ++r) v[c][r] = csub(v[c][r], cmul(v[o][r], d));
      }
      double nrm = 0.0;
#pragma unroll
      for (int r = 0; r < M; ++r) nrm += cnorm2(v[c][r]);
      const double in = 1.0 / sqrt(nrm);
#pragma unroll
      for (int r = 0; r < M; ++r) v[c][r] = cscale(v[c][r], in);
    }
  }
  double2 av[M][M];   // (A V0) column c = sum_k a[k] V0[k][c]
#pragma unroll
  for (int c = 0; c < M; ++c)
#pragma unroll
    for (int r = 0; r < M; ++r) {
      double2 acc = czero();
#pragma unroll
      for (int k = 0; k < M; ++k) acc = cadd(acc, cmul(a[k][r], v[c][k]));
      av[c][r] = acc;
    }
#pragma unroll
  for (int c = 0; c < M; ++c)
#pragma unroll
    for (int r = 0; r < M; ++r) {
      a[c][r] = av[c][r];
      vv[c][r] = v[c][r];
    }
}

template <int M>
QM_HD double polar_fast(const double2* e, double2* w_out, const double2* w_prev) {
  float2 a[M][M], vv[M][M];
  double scale = 0.0;
#pragma unroll
  for (int i = 0; i < M * M; ++i) scale = fmax(scale, fmax(fabs(e[i].x), fabs(e[i].y)));
  const double inv = scale > 0.0 ? 1.0 / scale : 1.0;
#pragma unroll
  for (int c = 0; c < M; ++c)
#pragma unroll
    for (int r = 0; r < M; ++r) {
      a[c][r] = cf((float)(e[r * M + c].x * inv), (float)(e[r * M + c].y * inv));
      vv[c][r] = cf(r == c ? 1.f : 0.f, 0.f);
    }
  jacobi_sweeps_f<M>(a, vv, (1 << M) - 1);
  float sig[M], smax = 0.f;
#pragma unroll
  for (int c = 0; c < M; ++c) {
    float nrm = 0.f;
#pragma unroll
    for (int r = 0; r < M; ++r) nrm += fcnorm2(a[c][r]);
    sig[c] = sqrtf(nrm);
    smax = fmaxf(smax, sig[c]);
  }
  int smask = 0;
#pragma unroll
  for (int c = 0; c < M; ++c)
    if (sig[c] > (float)QM_POLAR_NULL_TOL * smax && sig[c] > 0.f) smask |= 1 << c;
  const int nmask = ((1 << M) - 1) & ~smask;
#pragma unroll
  for (int c = 0; c < M; ++c)
#pragma unroll
    for (int r = 0; r < M; ++r) a[c][r] = ((smask >> c) & 1) ? fcscale(a[c][r], 1.f / sig[c]) : cf(0.f, 0.f);
  if (nmask != 0) {
    // X[:, c] = (I - U_s U_s^H) w_prev V[:, c] on the null columns, then the
    // nearest isometry (Jacobi on those columns), tiny ones completed
    float2 x[M][M], vx[M][M];
#pragma unroll
    for (int c = 0; c < M; ++c) {
#pragma unroll
      for (int r = 0; r < M; ++r) {
        float2 acc = cf(0.f, 0.f);
        if (w_prev && ((nmask >> c) & 1)) {
#pragma unroll
          for (int k = 0; k < M; ++k)
            acc = fcadd(acc, fcmul(cf((float)w_prev[r * M + k].x, (float)w_prev[r * M + k].y), vv[c][k]));
        }
        x[c][r] = acc;
        vx[c][r] = cf(r == c ? 1.f : 0.f, 0.f);
      }
#pragma unroll
      for (int i = 0; i < M; ++i) {
        if (!((smask >> i) & 1)) continue;
        float2 d = cf(0.f, 0.f);
#pragma unroll
        for (int r = 0; r < M; ++r) d = fcadd(d, fcmulc(a[i][r], x[c][r]));
#pragma unroll
        for (int r = 0; r < M; ++r) x[c][r] = fcsub(x[c][r], fcmul(a[i][r], d));
      }
    }
    jacobi_sweeps_f<M>(x, vx, nmask);
    int okmask = smask;
    float2 u[M][M];
#pragma unroll
    for (int c = 0; c < M; ++c)
#pragma unroll
      for (int r = 0; r < M; ++r) u[c][r] = a[c][r];
#pragma unroll
    for (int c = 0; c < M; ++c) {
      if (!((nmask >> c) & 1)) continue;
      float nrm = 0.f;
#pragma unroll
      for (int r = 0; r < M; ++r) nrm += fcnorm2(x[c][r]);
      nrm = sqrtf(nrm);
      if (nrm > 1e-4f) {
#pragma unroll
        for (int r = 0; r < M; ++r) u[c][r] = fcscale(x[c][r], 1.f / nrm);
        okmask |= 1 << c;
      }
    }
#pragma unroll
    for (int c = 0; c < M; ++c) {
      if (!((nmask >> c) & 1) || ((okmask >> c) & 1)) continue;
#pragma unroll
      for (int k = 0; k < M; ++k) {
        float2 v[M];
#pragma unroll
        for (int r = 0; r < M; ++r) v[r] = cf(r == k ? 1.f : 0.f, 0.f);
        for (int pass = 0; pass < 2; ++pass)
#pragma unroll
          for (int o = 0; o < M; ++o) {
            if (!((okmask >> o) & 1)) continue;
            float2 d = cf(0.f, 0.f);
#pragma unroll
            for (int r = 0; r < M; ++r) d = fcadd(d, fcmulc(u[o][r], v[r]));
#pragma unroll
            for (int r = 0; r < M; ++r) v[r] = fcsub(v[r], fcmul(u[o][r], d));
          }
        float nv = 0.f;
#pragma unroll
        for (int r = 0; r < M; ++r) nv += fcnorm2(v[r]);
        nv = sqrtf(nv);
        if (nv > 0.5f) {
#pragma unroll
          for (int r = 0; r < M; ++r) u[c][r] = fcscale(v[r], 1.f / nv);
          okmask |= 1 << c;
          break;
        }
      }
    }
    // U on the null columns becomes Ux Vx^H: column j = sum_{i null} u_i conj(vx[i][j])
#pragma unroll
    for (int j = 0; j < M; ++j) {
      if (!((nmask >> j) & 1)) continue;
#pragma unroll
      for (int r = 0; r < M; ++r) {
        float2 acc = cf(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < M; ++i)
          if ((nmask >> i) & 1) acc = fcadd(acc, fcmul(u[i][r], cf(vx[i][j].x, -vx[i][j].y)));
        a[j][r] = acc;
      }
    }
  }
  // W = U V^H in FP64, then modified Gram-Schmidt on its columns
  double2 w[M][M];   // column-major w[col][row]
#pragma unroll
  for (int s = 0; s < M; ++s)
#pragma unroll
    for (int r = 0; r < M; ++r) {
      double2 acc = czero();
#pragma unroll
      for (int c = 0; c < M; ++c) acc = cadd(acc, cmul(f2d(a[c][r]), cconj(f2d(vv[c][s]))));
      w[s][r] = acc;
    }
#pragma unroll
  for (int s = 0; s < M; ++s) {
#pragma unroll
    for (int o = 0; o < s; ++o) {
      double2 d = czero();
#pragma unroll
      for (int r = 0; r < M; ++r) d = cadd(d, cmulc(w[o][r], w[s][r]));
#pragma unroll
      for (int r = 0; r < M; ++r) w[s][r] = csub(w[s][r], cmul(w[o][r], d));
    }
    double nrm = 0.0;
#pragma unroll
    for (int r = 0; r < M; ++r) nrm += cnorm2(w[s][r]);
    const double in = 1.0 / sqrt(nrm);
#pragma unroll
    for (int r = 0; r < M; ++r) w[s][r] = cscale(w[s][r], in);
  }
  double tr = 0.0;   // Re Tr(W^H E)
#pragma unroll
  for (int s = 0; s < M; ++s)
#pragma unroll
    for (int r = 0; r < M; ++r) {
      w_out[r * M + s] = w[s][r];
      const double2 p = cmulc(w[s][r], e[r * M + s]);
      tr += p.x;
    }
  return tr;
}

// Reference implementation with runtime sizes (kept for the host build's
// cross-check of polar_jacobi_m); the kernels call polar_jacobi_m.
QM_HD double polar_jacobi_ref(const double2* e, int m, double2* w_out, const double2* w_prev = nullptr) {
  double2 a[4][4], vv[4][4], u[4][4];
  for (int c = 0; c < m; ++c)
    for (int r = 0; r < m; ++r) a[c][r] = e[r * m + c];
  onesided_jacobi(a, m, m, vv);
  double sig[4], smax = 0.0, nuc = 0.0;
  for (int c = 0; c < m; ++c) {
    double nrm = 0.0;
    for (int r = 0; r < m; ++r) nrm += cnorm2(a[c][r]);
    sig[c] = sqrt(nrm);
    nuc += sig[c];
    if (sig[c] > smax) smax = sig[c];
  }
  const double thr = QM_POLAR_NULL_TOL * smax;
  int ns = 0, nn = 0, sidx[4], nidx[4];
  for (int c = 0; c < m; ++c) {
    if (sig[c] > thr && sig[c] > 1e-300) sidx[ns++] = c;
    else nidx[nn++] = c;
  }
  for (int r = 0; r < m * m; ++r) w_out[r] = czero();
  // significant part: U_s V_s^H
  double2 us[4][4];
  {
    double2 as[4][4];
    for (int i = 0; i < ns; ++i)
      for (int r = 0; r < m; ++r) as[i][r] = a[sidx[i]][r];
    normalise_or_complete(as, m, ns, 0.0, nullptr, 0, us);
    for (int i = 0; i < ns; ++i)
      for (int r = 0; r < m; ++r)
        for (int s = 0; s < m; ++s)
          w_out[r * m + s] = cadd(w_out[r * m + s], cmul(us[i][r], cconj(vv[sidx[i]][s])));
  }
  if (nn == 0) return nuc;
  // null part: X = (I - U_s U_s^H) w_prev V_N, then W_N = polar(X) V_N^H
  double2 x[4][4];
  for (int j = 0; j < nn; ++j) {
    const int c = nidx[j];
    for (int r = 0; r < m; ++r) {
      double2 acc = czero();
      if (w_prev)
        for (int k = 0; k < m; ++k) acc = cadd(acc, cmul(w_prev[r * m + k], vv[c][k]));
      x[j][r] = acc;
    }
    for (int i = 0; i < ns; ++i) {
      double2 d = czero();
      for (int r = 0; r < m; ++r) d = cadd(d, cmulc(us[i][r], x[j][r]));
      for (int r = 0; r < m; ++r) x[j][r] = csub(x[j][r], cmul(us[i][r], d));
    }
  }
  double2 vx[4][4];
  onesided_jacobi(x, m, nn, vx);
  normalise_or_complete(x, m, nn, 1e-8, us, ns, u);
  // Q = Ux Vx^H (m x nn); W += Q V_N^H
  for (int j = 0; j < nn; ++j) {
    double2 q[4];
    for (int r = 0; r < m; ++r) {
      double2 acc = czero();
      for (int i = 0; i < nn; ++i) acc = cadd(acc, cmul(u[i][r], cconj(vx[i][j])));
      q[r] = acc;
    }
    const int c = nidx[j];
    for (int r = 0; r < m; ++r)
      for (int s = 0; s < m; ++s) w_out[r * m + s] = cadd(w_out[r * m + s], cmul(q[r], cconj(vv[c][s])));
  }
  return nuc;
}

// max |G G^H - I| over entries, G row-major m x m
QM_HD double unitarity_error(const double2* g, int m) {
  double err = 0.0;
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) {
      double2 acc = czero();
      for (int k = 0; k < m; ++k) acc = cadd(acc, cmul(g[i * m + k], cconj(g[j * m + k])));
      if (i == j) acc.x -= 1.0;
      double a = cabs_(acc);
      if (a > err) err = a;
    }
  return err;
}

// --------------------------------------------------------------------------
// Ran's gate construction (reference qmprs/primitives/mps.py:565-744) in
// closed form.  Gates are row-major 4x4 (two-qubit) or 2x2 (one-qubit); the
// row index is the output (MSB qubit first), the column the input.
// --------------------------------------------------------------------------

// First site of a block: data = 4 amplitudes m[2p + r].  Column 0 of G is m
// (mps.py:602); the three completion columns are fixed by the Schmidt form
// G = (A (x) B) CX (Ry (x) I): with M[p][r] = m[2p + r] = sum_i s_i a_i b_i^T
// (a_i = M v_i / s_i, b_i = conj(v_i), v_i the canonical-phase eigenvectors
// of M^H M), Ry = [[s0, -s1], [s1, s0]] and CX controlled by the first qubit.
// G|00> = m, and G needs a single CX.
QM_HD void ran_gate_first(const double2* m4, double2* g) {
  double2 gm[4], v[4], a[4];
  double lam[2];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      double2 acc = czero();
      for (int p = 0; p < 2; ++p) acc = cadd(acc, cmulc(m4[2 * p + i], m4[2 * p + j]));
      gm[i * 2 + j] = acc;
    }
  herm_eig_jacobi(gm, 2, v, lam);
  phase_fix_column(v, 2, 2, 0);
  phase_fix_column(v, 2, 2, 1);
  double s0 = sqrt(lam[0] > 0.0 ? lam[0] : 0.0), s1 = sqrt(lam[1] > 0.0 ? lam[1] : 0.0);
  const double ns = sqrt(s0 * s0 + s1 * s1);
  s0 /= ns;
  s1 /= ns;
  // a_i = M v_i normalised (row-major a[p*2 + i])
  for (int i = 0; i < 2; ++i) {
    double2 col[2];
    double nrm = 0.0;
    for (int p = 0; p < 2; ++p) {
      col[p] = cadd(cmul(m4[2 * p + 0], v[0 * 2 + i]), cmul(m4[2 * p + 1], v[1 * 2 + i]));
      nrm += cnorm2(col[p]);
    }
    nrm = sqrt(nrm);
    if (i == 1 && !(s1 > 1e-8 * s0)) {
      double2 a0[2] = {a[0], a[2]}, c[2];
      householder_complement(a0, 1, 2, c);
      a[1] = c[0];
      a[3] = c[1];
    } else {
      for (int p = 0; p < 2; ++p) a[p * 2 + i] = cscale(col[p], 1.0 / nrm);
    }
  }
  // K = A (x) B, B[r][y] = conj(v[r][y]); then G[:, 2x'+y'] = sum_x R[x][x'] K[:, 2x + (y' ^ x)]
  const double rr[2][2] = {{s0, -s1}, {s1, s0}};
  for (int row = 0; row < 4; ++row) {
    const int p = row >> 1, r = row & 1;
    for (int xp = 0; xp < 2; ++xp)
      for (int yp = 0; yp < 2; ++yp) {
        double2 acc = czero();
        for (int x = 0; x < 2; ++x) {
          const int y = yp ^ x;
          const double2 k = cmul(a[p * 2 + x], cconj(v[r * 2 + y]));
          acc = cadd(acc, cscale(k, rr[x][xp]));
        }
        g[row * 4 + (xp * 2 + yp)] = acc;
      }
  }
}

// Middle site: data[l][2p + r] (2 x 4).  Columns [M0, B0, M1, B1] with B the
// canonical complement of the rows, each column divided by the phase of its
// row-0 entry (mps.py:661-662).
QM_HD void ran_gate_middle(const double2* m8, double2* g) {
  double2 b[8];
  householder_complement(m8, 2, 4, b);
  for (int c = 0; c < 2; ++c) {
    double2 z = b[c * 4 + 0];
    double az = cabs_(z);
    if (az > QM_ZERO_TOL) {
      double2 ph = cscale(cconj(z), 1.0 / az);
      for (int i = 0; i < 4; ++i) b[c * 4 + i] = cmul(b[c * 4 + i], ph);
    }
  }
  for (int i = 0; i < 4; ++i) {
    g[i * 4 + 0] = m8[0 * 4 + i];
    g[i * 4 + 1] = b[0 * 4 + i];
    g[i * 4 + 2] = m8[1 * 4 + i];
    g[i * 4 + 3] = b[1 * 4 + i];
  }
}

// Last site of a multi-site block: data[l][p] (2 x 2); G[p][l] = data[l][p].
QM_HD void ran_gate_last(const double2* d4, double2* g) {
  for (int p = 0; p < 2; ++p)
    for (int l = 0; l < 2; ++l) g[p * 2 + l] = d4[l * 2 + p];
}

// Single-site block: data = 2 amplitudes; columns [v, complement(v)].
QM_HD void ran_gate_single(const double2* v2, double2* g) {
  double2 b[2];
  householder_complement(v2, 1, 2, b);
  for (int p = 0; p < 2; ++p) {
    g[p * 2 + 0] = v2[p];
    g[p * 2 + 1] = b[p];
  }
}

// Polar factor dispatch (m in {2, 4}).
QM_HD double polar_jacobi(const double2* e, int m, double2* w_out, const double2* w_prev = nullptr) {
  return m == 4 ? polar_jacobi_m<4>(e, w_out, w_prev) : polar_jacobi_m<2>(e, w_out, w_prev);
}

// FP64 polar factor (polar_jacobi) started from FP32 sweeps: the exact
// mode's sweep update.
QM_HD double polar_jacobi_pre(const double2* e, int m, double2* w_out, const double2* w_prev = nullptr) {
  return m == 4 ? polar_jacobi_m<4, true>(e, w_out, w_prev) : polar_jacobi_m<2, true>(e, w_out, w_prev);
}

// Polar factor used by the sweep kernel (FP32 sweeps, FP64 finish).
QM_HD double polar_sweep(const double2* e, int m, double2* w_out, const double2* w_prev = nullptr) {
  return m == 4 ? polar_fast<4>(e, w_out, w_prev) : polar_fast<2>(e, w_out, w_prev);
}
