// Host-only build of the small FP64 linear algebra compiled into the CUDA
// kernels (small_linalg.h).  Exposes it through a C ABI so CPU tests can
// compare the exact routines the kernels run against the FP64 oracle.
#include "small_linalg.h"

#include "tile_layout.h"

extern "C" {

void hc_herm_eig(const double* g, int n, double* v_out, double* lam_out) {
  double2 a[64], v[64];
  for (int i = 0; i < n * n; ++i) a[i] = cd(g[2 * i], g[2 * i + 1]);
  herm_eig_jacobi(a, n, v, lam_out);
  for (int i = 0; i < n * n; ++i) { v_out[2 * i] = v[i].x; v_out[2 * i + 1] = v[i].y; }
}

double hc_polar(const double* e, int m, double* w_out, const double* w_prev) {
  double2 a[16], w[16], wp[16];
  for (int i = 0; i < m * m; ++i) a[i] = cd(e[2 * i], e[2 * i + 1]);
  if (w_prev)
    for (int i = 0; i < m * m; ++i) wp[i] = cd(w_prev[2 * i], w_prev[2 * i + 1]);
  double nuc = polar_jacobi(a, m, w, w_prev ? wp : nullptr);
  for (int i = 0; i < m * m; ++i) { w_out[2 * i] = w[i].x; w_out[2 * i + 1] = w[i].y; }
  return nuc;
}

double hc_polar_pre(const double* e, int m, double* w_out, const double* w_prev) {
  double2 a[16], w[16], wp[16];
  for (int i = 0; i < m * m; ++i) a[i] = cd(e[2 * i], e[2 * i + 1]);
  if (w_prev)
    for (int i = 0; i < m * m; ++i) wp[i] = cd(w_prev[2 * i], w_prev[2 * i + 1]);
  double nuc = polar_jacobi_pre(a, m, w, w_prev ? wp : nullptr);
  for (int i = 0; i < m * m; ++i) { w_out[2 * i] = w[i].x; w_out[2 * i + 1] = w[i].y; }
  return nuc;
}

double hc_polar_sweep(const double* e, int m, double* w_out, const double* w_prev) {
  double2 a[16], w[16], wp[16];
  for (int i = 0; i < m * m; ++i) a[i] = cd(e[2 * i], e[2 * i + 1]);
  if (w_prev)
    for (int i = 0; i < m * m; ++i) wp[i] = cd(w_prev[2 * i], w_prev[2 * i + 1]);
  double nuc = polar_sweep(a, m, w, w_prev ? wp : nullptr);
  for (int i = 0; i < m * m; ++i) { w_out[2 * i] = w[i].x; w_out[2 * i + 1] = w[i].y; }
  return nuc;
}

void hc_complement(const double* x, int k, int n, double* cols_out) {
  double2 a[16], c[16];
  for (int i = 0; i < k * n; ++i) a[i] = cd(x[2 * i], x[2 * i + 1]);
  householder_complement(a, k, n, c);
  for (int i = 0; i < (n - k) * n; ++i) { cols_out[2 * i] = c[i].x; cols_out[2 * i + 1] = c[i].y; }
}

int hc_rank_by_cutoff(const double* sq, int n, double cutoff, int max_bond) {
  return rank_by_cutoff(sq, n, cutoff, max_bond);
}

void hc_round_robin_pair(int n, int k, int i, int* p, int* q) { round_robin_pair(n, k, i, p, q); }

int hc_rank_from_tails(const double* lsort, int kr, int k, double rest, double total, double cutoff, int max_bond) {
  return rank_from_tails(lsort, kr, k, rest, total, cutoff, max_bond);
}

void hc_phase_fix_column(double* v, int n, int ncols, int col) {
  double2 a[64];
  for (int i = 0; i < n * ncols; ++i) a[i] = cd(v[2 * i], v[2 * i + 1]);
  phase_fix_column(a, n, ncols, col);
  for (int i = 0; i < n * ncols; ++i) { v[2 * i] = a[i].x; v[2 * i + 1] = a[i].y; }
}

// kind: 0 first (4 in), 1 middle (8 in), 2 last (4 in), 3 single (2 in)
void hc_ran_gate(int kind, const double* data, double* g_out) {
  double2 d[8], g[16];
  const int nin = kind == 1 ? 8 : (kind == 3 ? 2 : 4);
  for (int i = 0; i < nin; ++i) d[i] = cd(data[2 * i], data[2 * i + 1]);
  for (int i = 0; i < 16; ++i) g[i] = czero();
  if (kind == 0) ran_gate_first(d, g);
  else if (kind == 1) ran_gate_middle(d, g);
  else if (kind == 2) ran_gate_last(d, g);
  else ran_gate_single(d, g);
  const int m = kind <= 1 ? 4 : 2;
  for (int i = 0; i < m * m; ++i) { g_out[2 * i] = g[i].x; g_out[2 * i + 1] = g[i].y; }
}

int hc_swz(int li) { return swz(li); }
int hc_rest_offset(int r, int wmask, int rmask) { return rest_offset(r, wmask, rmask); }
int hc_apply_pos_offset(int p, int wmask, int rmask) { return apply_pos_offset(p, wmask, rmask); }
float hc_vec_scale(int n, double nrm) { return vec_scale(n, nrm); }

}  // extern "C"
