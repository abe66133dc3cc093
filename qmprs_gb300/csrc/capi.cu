// C ABI of the library: handles, batch plans and the stage entry points.
//
// The host side here is the native runtime of the encoder: it owns the
// per-plan device scratch and work tables, sequences the kernel launches of
// every stage on the caller's stream, and turns kernel error flags into
// status codes and messages.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "exact.h"
#include "internal.h"
#include "qmprs_gb300.h"

struct qmprs_ctx {
  int device = 0;
  std::string err;
  // autotuned tile-pass grids, by batch signature (see plan_signature)
  std::vector<std::pair<uint64_t, int>> tuned;
};

struct qmprs_plan {
  qmprs_ctx* h = nullptr;
  int B = 0, max_n = 0, max_layers = 0, max_bond = 0, ntiles = 0, tile_bits = 0;
  std::vector<int> n;
  std::vector<int64_t> vec_off, gate_off, tensor_off;
  int64_t vec_total = 0, gate_total = 0, tensor_total = 0;
  // device tables
  int *d_n = nullptr, *d_tile_state = nullptr, *d_tile_idx = nullptr, *d_state_tile0 = nullptr,
      *d_state_ntiles = nullptr, *d_ticket = nullptr, *d_err = nullptr;
  int64_t *d_vec_off = nullptr, *d_gate_off = nullptr, *d_tensor_off = nullptr;
  int* d_bond_init = nullptr;
  // scratch
  float2 *S0 = nullptr, *S1 = nullptr, *S2 = nullptr;
  double2* partials = nullptr;
  double2* tt_partials = nullptr;
  double2 *gram = nullptr, *vsel = nullptr, *vsel2 = nullptr, *vwork = nullptr;
  double2* site_t = nullptr;
  float2* d_input = nullptr;   // qmprs_plan_upload's statevector batch (allocated on first use)
  int *bonds = nullptr, *active = nullptr, *nlayers = nullptr, *num_active = nullptr;
  double* nuc = nullptr;
  double2 *sq = nullptr, *tnorm = nullptr;
  BatchDev bd;
  // grouped sweep: chunk tables, group plan, replaced gates, chunk partials
  int nchunks = 0;
  int *d_chunk_state = nullptr, *d_chunk_idx = nullptr, *d_state_chunk0 = nullptr, *d_state_nchunks = nullptr,
      *d_ngroups = nullptr, *d_nrgroups = nullptr;
  GroupEnt *d_grp = nullptr, *d_rgrp = nullptr;
  // stage (a) beyond bond 64: blocked eigensolver scratch
  int tt_w = TT_MAXW, tt_b = TT_MAXB;
  BJScratch bj, bj_sub;   // blocked eigensolver of Grams wider than TT_MAXW, its deflated subproblem
  BJStats bj_stats;
  double2 *d_old_gates = nullptr, *d_gpartials = nullptr;
  GroupDev gd;
  // profiling of the sweep kernels (kernel classes: 0 environment stream,
  // 1 target update, 2 circuit rebuild, 3 environment reduce + polar):
  // launches, event time, algorithmic bytes
  bool prof = false;
  int64_t prof_launches[4] = {0, 0, 0, 0};
  double prof_ms[4] = {0, 0, 0, 0};
  double prof_bytes[4] = {0, 0, 0, 0};
  std::vector<int> gates_per_state;
  // exact precision mode: double-float working states (allocated on first use)
  int precision = QMPRS_PRECISION_FAST;
  xc *X0 = nullptr, *X1 = nullptr, *X2 = nullptr, *XT = nullptr;
  // CUDA graphs of the layer and sweep stages, keyed by everything their
  // launches embed (see run_stage)
  bool graphs = true;
  cudaStream_t cap = nullptr;
  int64_t graph_replays = 0;
  bool autotune = true;
  bool tuned = false;
  struct Graph {
    std::vector<uint64_t> key;
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;
  };
  std::vector<Graph> graph_cache;
};

static std::atomic<long long> g_launches{0};

void qm_note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

namespace {

int set_err(qmprs_ctx* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

int cuda_fail(qmprs_ctx* h, cudaError_t e, const char* what) {
  return set_err(h, QMPRS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                         \
  do {                                                   \
    cudaError_t _e = (call);                             \
    if (_e != cudaSuccess) return cuda_fail(p->h, _e, #call); \
  } while (0)

template <typename T>
cudaError_t dalloc(T** ptr, int64_t count) {
  if (count <= 0) count = 1;
  return cudaMalloc(reinterpret_cast<void**>(ptr), sizeof(T) * (size_t)count);
}

int chi_eff_host(int chi, int n) {
  const int cap = 1 << (n / 2);
  return chi < cap ? chi : cap;
}

int check_kernel_errors(qmprs_plan* p, cudaStream_t s) {
  CK(cudaGetLastError());
  int flags = 0;
  CK(cudaMemcpyAsync(&flags, p->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (flags & KERR_BAD_INPUT)
    return set_err(p->h, QMPRS_ERR_INVALID, "The statevector must have a finite, non-zero norm.");
  if (flags & KERR_NONUNITARY)
    return set_err(p->h, QMPRS_ERR_NONUNITARY, "All the generated unitaries must be unitary.");
  if (flags & KERR_EIG_WIDTH)
    return set_err(p->h, QMPRS_ERR_UNSUPPORTED,
                   "a bond of the MPS exceeds the supported width (bond > 1024)");
  if (flags & KERR_NONFINITE) return set_err(p->h, QMPRS_ERR_NUMERIC, "non-finite environment in a sweep");
  if (flags & KERR_BAD_GATE)
    return set_err(p->h, QMPRS_ERR_INVALID, "a gate slot has an invalid arity or position (gates skipped)");
  return QMPRS_OK;
}

int read_max_gates(qmprs_plan* p, const int* nlayers_dev, cudaStream_t s, int* max_gates) {
  std::vector<int> L(p->B);
  CK(cudaMemcpyAsync(L.data(), nlayers_dev, sizeof(int) * p->B, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  int m = 0;
  p->gates_per_state.assign(p->B, 0);
  for (int b = 0; b < p->B; ++b) {
    if (L[b] < 0 || L[b] > p->max_layers) return set_err(p->h, QMPRS_ERR_INVALID, "num_layers entry out of range");
    p->gates_per_state[b] = L[b] * p->n[b];
    m = std::max(m, L[b] * p->n[b]);
  }
  *max_gates = m;
  return QMPRS_OK;
}

// Event pairs around launches of one kernel class; summed after a sync.
struct ProfLog {
  std::vector<cudaEvent_t> ev;
  std::vector<int> cls;
  void begin(bool on, cudaStream_t s) {
    if (!on) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, s);
    ev.push_back(e);
  }
  void end(bool on, int c, cudaStream_t s) {
    if (!on) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, s);
    ev.push_back(e);
    cls.push_back(c);
  }
  void flush(qmprs_plan* p) {
    if (ev.empty()) return;
    cudaEventSynchronize(ev.back());
    for (size_t i = 0; i < cls.size(); ++i) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
      p->prof_ms[cls[i]] += ms;
      p->prof_launches[cls[i]] += 1;
    }
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    ev.clear();
    cls.clear();
  }
};

__global__ void k_fill_int(int* p, int64_t count, int value) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = value;
}

__global__ void k_check_norms(int B, const double2* sq, int* err) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x)
    if (!(isfinite(sq[b].x) && sq[b].x > 0.0)) atomicOr(err, KERR_BAD_INPUT);
}

__global__ void k_count_active(int B, const int* active, int* num_active) {
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  for (int b = threadIdx.x; b < B; b += blockDim.x)
    if (active[b]) atomicAdd(&cnt, 1);
  __syncthreads();
  if (threadIdx.x == 0) *num_active = cnt;
}

}  // namespace

void launch_fill_int(int* p, int64_t count, int value, cudaStream_t s) {
  int blocks = (int)std::min<int64_t>((count + 255) / 256, 1024);
  if (blocks < 1) blocks = 1;
  qm_note_launch();
  k_fill_int<<<blocks, 256, 0, s>>>(p, count, value);
}

void launch_check_norms(int B, const double2* sq, int* err, cudaStream_t s) {
  qm_note_launch();
  k_check_norms<<<(B + 127) / 128, 128, 0, s>>>(B, sq, err);
}

void launch_count_active(int B, const int* active, int* num_active, cudaStream_t s) {
  qm_note_launch();
  k_count_active<<<1, 256, 0, s>>>(B, active, num_active);
}

// Left-to-right contraction steps of the dense target for states whose bond
// pair at this step exceeds the one-block kernel (bonds read on the host).
void launch_wide_contract(qmprs_plan* p, int step, const double2* tensors, const std::vector<int>& hb,
                          const float2* src, float2* dst_buf, float2* target, cudaStream_t s) {
  const int stride = p->max_n + 1;
  for (int b = 0; b < p->B; ++b) {
    const int n = p->n[b], c = step + 1;
    if (c > n - 1) continue;
    const int rc = hb[(size_t)b * stride + c], rn = hb[(size_t)b * stride + c + 1];
    if (rc < 1 || rn < 1 || rc > p->tt_b || rn > p->tt_b) continue;
    if (rc <= TT_MAXB && rn <= TT_MAXB) continue;
    const int ce = chi_eff_host(p->max_bond, n);
    const double2* a = tensors + p->tensor_off[b] + (int64_t)c * 2 * ce * ce;
    float2* o = (c == n - 1 ? target : dst_buf) + p->vec_off[b];
    launch_cgemm(src + p->vec_off[b], rc, a, 2 * rn, o, 2 * rn, ipow2(c), 2 * rn, rc, s);
  }
}

// ---- exact precision mode: orchestration ---------------------------------------------
//
// The same stages as the fast mode, on double-float working states (exact.cu).
// Caller-facing statevector buffers are complex128.  Stage (a) runs state by
// state with the bonds read on the host after every cut; the layer stage and
// the sweeps batch all states in every launch like the fast mode, with one
// gate per launch.

namespace {

// Enqueue a stage whose launch sequence is fixed by `key` (pointers, sizes,
// options) through body(stream, capturing).  Without graphs body runs on the
// caller's stream.  With graphs: the first call with a key runs body
// directly; the second captures body on the plan's own capture stream (a
// stream the caller never sees, so nothing of the caller's work is
// captured), instantiates the graph and launches it on the caller's
// stream; later calls launch the cached graph.  A capturing body must not
// synchronise: it enqueues every sweep or layer and leaves converged states
// to the kernels' device-side active flags.  Kernel launches replayed from
// a graph are added to the launch counter at every replay.
template <class F>
int run_stage(qmprs_plan* p, const std::vector<uint64_t>& key, cudaStream_t s, F&& body) {
  if (!p->graphs || p->prof) return body(s, false);
  qmprs_plan::Graph* e = nullptr;
  for (auto& g : p->graph_cache)
    if (g.key == key) e = &g;
  if (e && e->exec) {
    CK(cudaGraphLaunch(e->exec, s));
    g_launches.fetch_add(e->launches, std::memory_order_relaxed);
    ++p->graph_replays;
    return QMPRS_OK;
  }
  if (!e) {
    if (p->graph_cache.size() >= 16) {   // bound the cache: drop the oldest graph
      if (p->graph_cache.front().exec) cudaGraphExecDestroy(p->graph_cache.front().exec);
      p->graph_cache.erase(p->graph_cache.begin());
    }
    p->graph_cache.push_back(qmprs_plan::Graph{key, nullptr, 0});
    return body(s, false);
  }
  if (!p->cap) CK(cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking));
  const long long before = g_launches.load();
  CK(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal));
  const int rc = body(p->cap, true);
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(p->cap, &graph);
  const long long n = g_launches.load() - before;
  g_launches.fetch_sub(n, std::memory_order_relaxed);
  if (rc != QMPRS_OK || ce != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    if (rc != QMPRS_OK) return rc;
    return cuda_fail(p->h, ce, "stage graph capture");
  }
  const cudaError_t ie = cudaGraphInstantiate(&e->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) {
    e->exec = nullptr;
    return cuda_fail(p->h, ie, "cudaGraphInstantiate");
  }
  e->launches = n;
  CK(cudaGraphLaunch(e->exec, s));
  g_launches.fetch_add(n, std::memory_order_relaxed);
  ++p->graph_replays;
  return QMPRS_OK;
}

inline uint64_t ptr_key(const void* q) { return (uint64_t)(uintptr_t)q; }

// Signature of a batch for the autotuner: the qubit-count histogram, the
// bond dimension and the layer count (FNV-1a).
uint64_t plan_signature(const qmprs_plan* p) {
  int hist[MAX_QUBITS + 1] = {0};
  for (int n : p->n) ++hist[n];
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](uint64_t v) {
    for (int i = 0; i < 8; ++i) {
      h ^= (v >> (8 * i)) & 0xff;
      h *= 1099511628211ull;
    }
  };
  for (int n = 0; n <= MAX_QUBITS; ++n) mix((uint64_t)hist[n]);
  mix((uint64_t)p->max_bond);
  mix((uint64_t)p->max_layers);
  return h;
}
inline uint64_t dbl_key(double v) {
  uint64_t u;
  std::memcpy(&u, &v, sizeof(u));
  return u;
}

int ensure_tt_scratch(qmprs_plan* p) {
  if (p->tt_partials) return QMPRS_OK;
  const int64_t WW = (int64_t)p->tt_w * p->tt_w;
  CK(dalloc(&p->tt_partials, (int64_t)p->B * TT_SPLIT * WW));
  CK(dalloc(&p->gram, (int64_t)p->B * WW));
  CK(dalloc(&p->vsel2, (int64_t)p->B * WW));
  CK(dalloc(&p->vwork, (int64_t)p->B * WW));
  if (2 * p->tt_b > p->bd.eig_wmax) CK((cudaError_t)bj_alloc(p->bj, p->tt_w, p->tt_b));
  return QMPRS_OK;
}

int ensure_exact(qmprs_plan* p) {
  if (p->X0) return QMPRS_OK;
  CK(dalloc(&p->X0, p->vec_total));
  CK(dalloc(&p->X1, p->vec_total));
  CK(dalloc(&p->X2, p->vec_total));
  CK(dalloc(&p->XT, p->vec_total));
  return QMPRS_OK;
}

int read_ints(qmprs_plan* p, const int* dev, std::vector<int>& host, cudaStream_t s) {
  CK(cudaMemcpyAsync(host.data(), dev, sizeof(int) * host.size(), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return QMPRS_OK;
}

// Dense statevector of the MPS in `tensors` (bonds hb on the host), left to
// right in double-float: X_1 = A_0, X_{c+1} = X_c A_c, into `out`.  With
// `start` (stage (a)), state b starts instead from X_c = f_b Y_c at
// c = start[b], where Y_c = M_c V_c is the projected remainder saved in
// `saved` and f_b (device, `scale`) the norm factor of site 0: when no cut
// left of c truncates, every kept space there holds the remainder's whole
// row space, so A_0 ... A_{c-1} contract to exactly that, and the
// rank-deficient left cuts (2^c rows, more columns) add no rounding of
// their eigenvectors to the target.
void x_contract(qmprs_plan* p, const double2* tensors, const std::vector<int>& hb, xc* out, cudaStream_t s,
                const std::vector<int>* start = nullptr, const xc* saved = nullptr, const double* scale = nullptr) {
  const int stride = p->max_n + 1;
  for (int b = 0; b < p->B; ++b) {
    const int n = p->n[b];
    const int* bb = hb.data() + (size_t)b * stride;
    bool ok = true;
    for (int c = 0; c <= n; ++c) ok = ok && bb[c] >= 1 && bb[c] <= p->tt_b;
    if (!ok) continue;
    const int ce = chi_eff_host(p->max_bond, n);
    const double2* t0 = tensors + p->tensor_off[b];
    xc* cur = p->X0 + p->vec_off[b];
    xc* nxt = p->X1 + p->vec_off[b];
    int c_first = 1;
    if (start && (*start)[b] >= 1) {
      c_first = (*start)[b];
      launch_x_scale_flat(saved + p->vec_off[b], cur, ipow2(c_first) * bb[c_first], scale + b, s);
    } else {
      launch_x_from_d_flat(t0, cur, 2 * (int64_t)bb[1], s);
    }
    for (int c = c_first; c <= n - 1; ++c) {
      const int rc = bb[c], rn = bb[c + 1];
      const double2* a = t0 + (int64_t)c * 2 * ce * ce;
      xc* o = c == n - 1 ? out + p->vec_off[b] : nxt;
      launch_x_gemm(cur, rc, a, 2 * rn, o, 2 * rn, ipow2(c), 2 * rn, rc, s);
      std::swap(cur, nxt);
    }
  }
}

int exact_mps_from_statevector(qmprs_plan* p, const double2* sv, int max_bond, double cutoff, double2* tensors,
                               int* bonds, double2* target, cudaStream_t s) {
  int rc = ensure_tt_scratch(p);
  if (rc == QMPRS_OK) rc = ensure_exact(p);
  if (rc != QMPRS_OK) return rc;
  const int64_t WW = (int64_t)p->tt_w * p->tt_w;
  const int stride = p->max_n + 1;
  CK(cudaMemsetAsync(p->d_err, 0, sizeof(int), s));
  CK(cudaMemcpyAsync(bonds, p->d_bond_init, sizeof(int) * (size_t)p->B * stride, cudaMemcpyDeviceToDevice, s));
  launch_x_from_d(p->bd, sv, p->X0, s);
  launch_x_dot(p->bd, p->X0, p->X0, p->partials, p->sq, s);
  launch_check_norms(p->B, p->sq, p->d_err, s);
  std::vector<double2> sq(p->B);
  CK(cudaMemcpyAsync(sq.data(), p->sq, sizeof(double2) * p->B, cudaMemcpyDeviceToHost, s));
  std::vector<int> hb((size_t)p->B * stride), start(p->B, -1);
  xc* buf[2] = {p->X1, p->X2};
  for (int j = 0; j + 2 <= p->max_n; ++j) {
    if ((rc = read_ints(p, bonds, hb, s)) != QMPRS_OK) return rc;
    const xc* src = j == 0 ? p->X0 : buf[(j - 1) & 1];
    bool wide = false;
    for (int b = 0; b < p->B; ++b) {
      const int c = p->n[b] - 1 - j;
      if (c < 1) continue;
      const int r = hb[(size_t)b * stride + c + 1];
      if (r < 1 || r > p->tt_b) continue;
      launch_x_gram(src + p->vec_off[b], ipow2(c), 2 * r, p->tt_partials + (int64_t)b * TT_SPLIT * WW, WW,
                    p->gram + (int64_t)b * WW, s);
      wide = wide || 2 * r > p->bd.eig_wmax;
    }
    launch_tt_eig(p->bd, j, bonds, p->gram, p->vwork, max_bond, cutoff, p->vsel2, tensors, p->max_bond,
                  p->tt_partials, 1e-15, s);
    if (wide) {
      for (int b = 0; b < p->B; ++b) {
        const int c = p->n[b] - 1 - j;
        if (c < 1) continue;
        const int r = hb[(size_t)b * stride + c + 1];
        if (r < 1 || r > p->tt_b || 2 * r <= p->bd.eig_wmax) continue;
        const int e = tt_block_eig(p->bd, b, c, 2 * r, p->gram, nullptr, p->bj, p->bj_sub, bonds, p->vsel2, tensors,
                                   p->max_bond, max_bond, cutoff, BJ_TOL_EXACT, s, &p->bj_stats);
        if (e != 0) return cuda_fail(p->h, (cudaError_t)e, "stage (a) blocked eigensolver");
      }
    }
    if ((rc = read_ints(p, bonds, hb, s)) != QMPRS_OK) return rc;
    for (int b = 0; b < p->B; ++b) {
      const int c = p->n[b] - 1 - j;
      if (c < 1) continue;
      const int r = hb[(size_t)b * stride + c + 1], keep = hb[(size_t)b * stride + c];
      if (r < 1 || keep < 1 || r > p->tt_b || keep > p->tt_b) continue;
      launch_x_gemm(src + p->vec_off[b], 2 * r, p->vsel2 + (int64_t)b * WW, p->tt_b, buf[j & 1] + p->vec_off[b],
                    keep, ipow2(c), keep, 2 * r, s);
      // the last cut (so far, right to left) that truncates, or the first
      // cut: the target's contraction starts from its projected remainder
      if (c == p->n[b] - 1 || keep < std::min<int64_t>(ipow2(c), 2 * r)) {
        CK(cudaMemcpyAsync(p->XT + p->vec_off[b], buf[j & 1] + p->vec_off[b], sizeof(xc) * ipow2(c) * keep,
                           cudaMemcpyDeviceToDevice, s));
        start[b] = c;
      }
    }
  }
  for (int b = 0; b < p->B; ++b) {
    const int r1 = hb[(size_t)b * stride + 1];
    if (r1 < 1 || r1 > p->tt_b) continue;
    launch_x_site0(buf[(p->n[b] - 2) & 1] + p->vec_off[b], r1, sq[b].x, tensors + p->tensor_off[b], p->nuc + b, s);
  }
  x_contract(p, tensors, hb, p->XT, s, &start, p->XT, p->nuc);
  launch_x_to_d(p->bd, p->XT, target, s);
  return check_kernel_errors(p, s);
}

int exact_unitary_layers(qmprs_plan* p, const double2* target, int num_layers, double fidelity_threshold,
                         double2* gates, signed char* ar, int* layers_out, double2* layer_fid, cudaStream_t s) {
  int rc = ensure_exact(p);
  if (rc != QMPRS_OK) return rc;
  CK(cudaMemsetAsync(p->d_err, 0, sizeof(int), s));
  CK(cudaMemsetAsync(layers_out, 0, sizeof(int) * p->B, s));
  CK(cudaMemsetAsync(layer_fid, 0, sizeof(double2) * (size_t)p->B * num_layers, s));
  launch_fill_int(p->active, p->B, 1, s);
  xc* work = p->X0;
  launch_x_from_d(p->bd, target, work, s);
  launch_x_normalize(p->bd, work, work, p->partials, p->sq, s);
  xc* buf[2] = {p->X1, p->X2};
  const double atol = 1.0 - fidelity_threshold;
  const int64_t nb = (int64_t)p->B * (p->max_n + 1);
  auto body = [&](cudaStream_t s2, bool capturing) -> int {
    for (int l = 0; l < num_layers; ++l) {
      CK(cudaMemcpyAsync(p->bonds, p->d_bond_init, sizeof(int) * nb, cudaMemcpyDeviceToDevice, s2));
      for (int j = 0; j + 2 <= p->max_n; ++j) {
        const xc* src = j == 0 ? work : buf[(j - 1) & 1];
        launch_x_layer_gram(p->bd, j, work, src, p->bonds, p->partials, p->active, s2);
        launch_layer_eig(p->bd, j, p->partials, p->vsel, p->bonds, p->site_t, p->active, s2);
        launch_x_layer_project(p->bd, j, work, src, buf[j & 1], p->bonds, p->vsel, p->active, s2);
      }
      launch_x_layer_build(p->bd, l, buf[0], buf[1], p->bonds, p->site_t, gates, ar, p->active, s2);
      for (int st = 0; st < p->max_n; ++st) {
        GateSel sel{SEL_INVERSE, st, l, 1, gates, ar, nullptr, p->active};
        launch_x_apply_gate(p->bd, work, sel, s2);
      }
      launch_x_layer_fidelity(p->bd, l, work, num_layers, atol, layer_fid, layers_out, p->active, s2);
      if (!capturing) {
        launch_count_active(p->B, p->active, p->num_active, s2);
        int na = 0;
        CK(cudaMemcpyAsync(&na, p->num_active, sizeof(int), cudaMemcpyDeviceToHost, s2));
        CK(cudaStreamSynchronize(s2));
        if (na == 0) break;
      }
    }
    return QMPRS_OK;
  };
  const std::vector<uint64_t> key = {3, ptr_key(target), ptr_key(gates), ptr_key(ar), ptr_key(layers_out),
                                     ptr_key(layer_fid), (uint64_t)num_layers, dbl_key(fidelity_threshold)};
  rc = run_stage(p, key, s, body);
  if (rc != QMPRS_OK) return rc;
  return check_kernel_errors(p, s);
}

int exact_optimize_layers(qmprs_plan* p, const double2* target, double2* gates, const signed char* ar,
                          const int* num_layers, int num_sweeps, double stop_fidelity, double* sweep_fid,
                          int* sweeps_done, cudaStream_t s) {
  int rc = ensure_exact(p);
  if (rc != QMPRS_OK) return rc;
  int max_gates = 0;
  if ((rc = read_max_gates(p, num_layers, s, &max_gates)) != QMPRS_OK) return rc;
  launch_fill_int(p->active, p->B, 1, s);
  launch_x_from_d(p->bd, target, p->XT, s);
  launch_x_dot(p->bd, p->XT, p->XT, p->partials, p->tnorm, s);
  if (p->max_n <= X_FUSED_MAXN) {   // every state fits one block's shared memory
    const int e = launch_x_sweep_fused(p->bd, p->max_n, p->XT, gates, ar, num_layers, p->active, p->tnorm,
                                       num_sweeps, stop_fidelity, sweep_fid, sweeps_done, s);
    if (e != 0) return cuda_fail(p->h, (cudaError_t)e, "k_x_sweep_fused");
    return check_kernel_errors(p, s);
  }
  xc* psi = p->X0;
  xc* t = p->X1;
  auto body = [&](cudaStream_t s2, bool capturing) -> int {
    for (int sw = 0; sw < num_sweeps; ++sw) {
      launch_x_zero(p->bd, psi, p->active, s2);
      for (int j = 0; j < max_gates; ++j) {
        GateSel sel{SEL_REBUILD, j, 0, 0, gates, ar, num_layers, p->active};
        launch_x_apply_gate(p->bd, psi, sel, s2);
      }
      launch_x_copy(p->bd, p->XT, t, p->active, s2);
      for (int j = 0; j < max_gates; ++j) {
        launch_x_sweep_step(p->bd, j, psi, t, gates, ar, num_layers, p->active, p->partials, p->nuc, s2);
        GateSel sel{SEL_SWEEP, j, 0, 1, gates, ar, num_layers, p->active};
        launch_x_apply_gate(p->bd, t, sel, s2);
      }
      CK(cudaMemsetAsync(p->num_active, 0, sizeof(int), s2));
      launch_sweep_finish(p->B, sw, num_sweeps, p->nuc, p->tnorm, sweep_fid, sweeps_done, p->active,
                          stop_fidelity, p->num_active, s2);
      if (stop_fidelity > 0.0 && !capturing) {
        int na = 0;
        CK(cudaMemcpyAsync(&na, p->num_active, sizeof(int), cudaMemcpyDeviceToHost, s2));
        CK(cudaStreamSynchronize(s2));
        if (na == 0) break;
      }
    }
    return QMPRS_OK;
  };
  const std::vector<uint64_t> key = {4, ptr_key(target), ptr_key(gates), ptr_key(ar), ptr_key(num_layers),
                                     ptr_key(sweep_fid), ptr_key(sweeps_done), (uint64_t)num_sweeps,
                                     dbl_key(stop_fidelity), (uint64_t)max_gates};
  rc = run_stage(p, key, s, body);
  if (rc != QMPRS_OK) return rc;
  return check_kernel_errors(p, s);
}

int exact_circuit_state(qmprs_plan* p, const double2* gates, const signed char* ar, const int* num_layers,
                        double2* out, cudaStream_t s) {
  int rc = ensure_exact(p);
  if (rc != QMPRS_OK) return rc;
  int max_gates = 0;
  if ((rc = read_max_gates(p, num_layers, s, &max_gates)) != QMPRS_OK) return rc;
  launch_x_zero(p->bd, p->X0, nullptr, s);
  for (int j = 0; j < max_gates; ++j) {
    GateSel sel{SEL_REBUILD, j, 0, 0, gates, ar, num_layers, nullptr};
    launch_x_apply_gate(p->bd, p->X0, sel, s);
  }
  launch_x_to_d(p->bd, p->X0, out, s);
  return check_kernel_errors(p, s);
}

}  // namespace

extern "C" {

int qmprs_version(void) { return 100; }

int64_t qmprs_launch_count(void) { return (int64_t)g_launches.load(); }

int qmprs_plan_set_profiling(qmprs_plan_t p, int enable) {
  if (!p) return QMPRS_ERR_INVALID;
  p->prof = enable != 0;
  for (int k = 0; k < 4; ++k) {
    p->prof_launches[k] = 0;
    p->prof_ms[k] = 0.0;
    p->prof_bytes[k] = 0.0;
  }
  return QMPRS_OK;
}

int qmprs_plan_profile(qmprs_plan_t p, int kernel, int64_t* launches, double* milliseconds, double* bytes) {
  if (!p || kernel < 0 || kernel > 3) return QMPRS_ERR_INVALID;
  if (launches) *launches = p->prof_launches[kernel];
  if (milliseconds) *milliseconds = p->prof_ms[kernel];
  if (bytes) *bytes = p->prof_bytes[kernel];
  return QMPRS_OK;
}

int qmprs_create(qmprs_handle_t* out) {
  if (!out) return QMPRS_ERR_INVALID;
  qmprs_ctx* h = new qmprs_ctx();
  cudaError_t e = cudaGetDevice(&h->device);
  if (e != cudaSuccess) {
    delete h;
    *out = nullptr;
    return QMPRS_ERR_CUDA;
  }
  *out = h;
  return QMPRS_OK;
}

void qmprs_destroy(qmprs_handle_t h) { delete h; }

const char* qmprs_last_error(qmprs_handle_t h) { return h ? h->err.c_str() : "null handle"; }

void qmprs_plan_destroy(qmprs_plan_t p) {
  if (!p) return;
  for (auto& g : p->graph_cache)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  if (p->cap) cudaStreamDestroy(p->cap);
  void* ptrs[] = {p->d_n,      p->d_tile_state, p->d_tile_idx, p->d_state_tile0, p->d_state_ntiles,
                  p->d_ticket, p->d_err,        p->d_vec_off,  p->d_gate_off,    p->d_tensor_off,
                  p->d_bond_init, p->S0,        p->S1,         p->S2,            p->partials,
                  p->tt_partials, p->gram,      p->vsel,       p->vsel2,         p->site_t, p->vwork,
                  p->bonds,    p->active,       p->nlayers,    p->num_active,    p->nuc,
                  p->sq,       p->tnorm,        p->d_chunk_state, p->d_chunk_idx, p->d_state_chunk0,
                  p->d_state_nchunks, p->d_ngroups, p->d_grp,    p->d_old_gates,   p->d_gpartials,
                  p->d_rgrp,   p->d_nrgroups,   p->d_input, p->X0, p->X1, p->X2, p->XT};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  bj_free(p->bj);
  bj_free(p->bj_sub);
  delete p;
}

int qmprs_plan_create(qmprs_handle_t h, int num_states, const int* num_qubits, int max_layers, int max_bond,
                      qmprs_plan_t* out) {
  if (!h || !out) return QMPRS_ERR_INVALID;
  *out = nullptr;
  if (num_states < 1 || !num_qubits) return set_err(h, QMPRS_ERR_INVALID, "num_states must be >= 1");
  if (max_layers < 1) return set_err(h, QMPRS_ERR_INVALID, "The number of layers must be a positive integer.");
  if (max_bond < 1) return set_err(h, QMPRS_ERR_INVALID, "`bond_dimension` must be an integer greater than 0.");
  qmprs_plan* p = new qmprs_plan();
  p->h = h;
  p->B = num_states;
  p->max_layers = max_layers;
  p->max_bond = max_bond;
  p->n.assign(num_qubits, num_qubits + num_states);
  std::vector<int> tile_state, tile_idx, state_tile0(num_states), state_ntiles(num_states);
  // Tile size: aim at ~16 tiles per SM over the whole batch (152 SMs), so
  // that per-tile reduction overhead amortises over many amplitudes; never
  // below 2^TILE_BITS_MIN amplitudes nor above 2^TILE_BITS_MAX.
  int64_t total_amps = 0;
  for (int b = 0; b < num_states; ++b) {
    const int n = p->n[b];
    if (n < 2 || n > MAX_QUBITS) {
      delete p;
      return set_err(h, QMPRS_ERR_INVALID, "The statevector must have at least 2 qubits (and at most 30).");
    }
    total_amps += ipow2(n);
  }
  int tile_bits = TILE_BITS_MIN;
  while (tile_bits < TILE_BITS_MAX && (total_amps >> (tile_bits + 1)) >= 152 * 16) ++tile_bits;
  p->tile_bits = tile_bits;
  for (int b = 0; b < num_states; ++b) {
    const int n = p->n[b];
    p->max_n = std::max(p->max_n, n);
    p->vec_off.push_back(p->vec_total);
    p->vec_total += ipow2(n);
    p->gate_off.push_back(p->gate_total);
    p->gate_total += (int64_t)max_layers * n * 16;
    p->tensor_off.push_back(p->tensor_total);
    const int ce = chi_eff_host(max_bond, n);
    p->tensor_total += (int64_t)n * 2 * ce * ce;
    const int nt = n > tile_bits ? (1 << (n - tile_bits)) : 1;
    state_tile0[b] = (int)tile_state.size();
    state_ntiles[b] = nt;
    for (int t = 0; t < nt; ++t) {
      tile_state.push_back(b);
      tile_idx.push_back(t);
    }
  }
  p->ntiles = (int)tile_state.size();
  for (int b = 0; b < num_states; ++b) p->tt_b = std::max(p->tt_b, chi_eff_host(max_bond, p->n[b]));
  p->tt_w = std::max(TT_MAXW, 2 * p->tt_b);
  // grouped sweep: tiles of 2^min(n, GT) amplitudes, GCHUNK tiles per chunk
  std::vector<int> chunk_state, chunk_idx, state_chunk0(num_states), state_nchunks(num_states);
  for (int b = 0; b < num_states; ++b) {
    const int n = p->n[b];
    const int64_t tiles = n > GT ? ipow2(n - GT) : 1;
    const int nc = (int)((tiles + GCHUNK - 1) / GCHUNK);
    state_chunk0[b] = (int)chunk_state.size();
    state_nchunks[b] = nc;
    for (int c = 0; c < nc; ++c) {
      chunk_state.push_back(b);
      chunk_idx.push_back(c);
    }
  }
  p->nchunks = (int)chunk_state.size();
  std::vector<int> bond_init((size_t)num_states * (p->max_n + 1), 0);
  for (int b = 0; b < num_states; ++b) {
    bond_init[(size_t)b * (p->max_n + 1)] = 1;
    bond_init[(size_t)b * (p->max_n + 1) + p->n[b]] = 1;
  }
#define PC(call)                                  \
  do {                                            \
    cudaError_t _e = (call);                      \
    if (_e != cudaSuccess) {                      \
      int code = cuda_fail(h, _e, #call);         \
      qmprs_plan_destroy(p);                      \
      return code;                                \
    }                                             \
  } while (0)
  const int B = num_states;
  PC(dalloc(&p->d_n, B));
  PC(dalloc(&p->d_vec_off, B));
  PC(dalloc(&p->d_gate_off, B));
  PC(dalloc(&p->d_tensor_off, B));
  PC(dalloc(&p->d_tile_state, p->ntiles));
  PC(dalloc(&p->d_tile_idx, p->ntiles));
  PC(dalloc(&p->d_state_tile0, B));
  PC(dalloc(&p->d_state_ntiles, B));
  PC(dalloc(&p->d_ticket, B));
  PC(dalloc(&p->d_err, 1));
  PC(dalloc(&p->d_bond_init, (int64_t)bond_init.size()));
  PC(cudaMemcpy(p->d_n, p->n.data(), sizeof(int) * B, cudaMemcpyHostToDevice));
  PC(cudaMemcpy(p->d_vec_off, p->vec_off.data(), sizeof(int64_t) * B, cudaMemcpyHostToDevice));
  PC(cudaMemcpy(p->d_gate_off, p->gate_off.data(), sizeof(int64_t) * B, cudaMemcpyHostToDevice));
  PC(cudaMemcpy(p->d_tensor_off, p->tensor_off.data(), sizeof(int64_t) * B, cudaMemcpyHostToDevice));
  PC(cudaMemcpy(p->d_tile_state, tile_state.data(), sizeof(int) * p->ntiles, cudaMemcpyHostToDevice));
  PC(cudaMemcpy(p->d_tile_idx, tile_idx.data(), sizeof(int) * p->ntiles, cudaMemcpyHostToDevice));
  PC(cudaMemcpy(p->d_state_tile0, state_tile0.data(), sizeof(int) * B, cudaMemcpyHostToDevice));
  PC(cudaMemcpy(p->d_state_ntiles, state_ntiles.data(), sizeof(int) * B, cudaMemcpyHostToDevice));
  PC(cudaMemcpy(p->d_bond_init, bond_init.data(), sizeof(int) * bond_init.size(), cudaMemcpyHostToDevice));
  PC(cudaMemset(p->d_ticket, 0, sizeof(int) * B));
  PC(cudaMemset(p->d_err, 0, sizeof(int)));
  PC(dalloc(&p->S0, p->vec_total));
  PC(dalloc(&p->S1, p->vec_total));
  PC(dalloc(&p->S2, p->vec_total));
  PC(dalloc(&p->partials, (int64_t)p->ntiles * WARPS_PER_BLOCK * 16));
  PC(dalloc(&p->vsel, (int64_t)B * 16));
  PC(dalloc(&p->site_t, (int64_t)B * p->max_n * 8));
  PC(dalloc(&p->bonds, (int64_t)bond_init.size()));
  PC(dalloc(&p->active, B));
  PC(dalloc(&p->nlayers, B));
  PC(dalloc(&p->num_active, 1));
  PC(dalloc(&p->nuc, B));
  PC(dalloc(&p->sq, B));
  PC(dalloc(&p->tnorm, B));
  const int gmax = max_layers * p->max_n;
  PC(dalloc(&p->d_chunk_state, p->nchunks));
  PC(dalloc(&p->d_chunk_idx, p->nchunks));
  PC(dalloc(&p->d_state_chunk0, B));
  PC(dalloc(&p->d_state_nchunks, B));
  PC(dalloc(&p->d_ngroups, B));
  PC(dalloc(&p->d_grp, (int64_t)B * gmax));
  PC(dalloc(&p->d_rgrp, (int64_t)B * gmax));
  PC(dalloc(&p->d_nrgroups, B));
  PC(dalloc(&p->d_old_gates, (int64_t)B * GMAXSTEPS * 16));
  PC(dalloc(&p->d_gpartials, (int64_t)p->nchunks * GMM));
  PC(cudaMemcpy(p->d_chunk_state, chunk_state.data(), sizeof(int) * p->nchunks, cudaMemcpyHostToDevice));
  PC(cudaMemcpy(p->d_chunk_idx, chunk_idx.data(), sizeof(int) * p->nchunks, cudaMemcpyHostToDevice));
  PC(cudaMemcpy(p->d_state_chunk0, state_chunk0.data(), sizeof(int) * B, cudaMemcpyHostToDevice));
  PC(cudaMemcpy(p->d_state_nchunks, state_nchunks.data(), sizeof(int) * B, cudaMemcpyHostToDevice));
  PC(cudaMemset(p->d_gpartials, 0, sizeof(double2) * (size_t)p->nchunks * GMM));
#undef PC
  GroupDev& gd = p->gd;
  gd.nchunks = p->nchunks;
  gd.gmax = gmax;
  gd.chunk_state = p->d_chunk_state;
  gd.chunk_idx = p->d_chunk_idx;
  gd.state_chunk0 = p->d_state_chunk0;
  gd.state_nchunks = p->d_state_nchunks;
  gd.grp = p->d_grp;
  gd.ngroups = p->d_ngroups;
  gd.old_gates = p->d_old_gates;
  gd.partials = p->d_gpartials;
  gd.rgrp = p->d_rgrp;
  gd.grid = 0;
  gd.nrgroups = p->d_nrgroups;
  BatchDev& bd = p->bd;
  bd.B = B;
  bd.ntiles = p->ntiles;
  bd.max_n = p->max_n;
  bd.n = p->d_n;
  bd.vec_off = p->d_vec_off;
  bd.gate_off = p->d_gate_off;
  bd.tensor_off = p->d_tensor_off;
  bd.tile_state = p->d_tile_state;
  bd.tile_idx = p->d_tile_idx;
  bd.state_tile0 = p->d_state_tile0;
  bd.state_ntiles = p->d_state_ntiles;
  bd.ticket = p->d_ticket;
  bd.err = p->d_err;
  bd.tt_w = p->tt_w;
  bd.tt_b = p->tt_b;
  bd.eig_wmax = num_states <= BJ_SMALL_BATCH ? TT_MAXB : TT_MAXW;
  *out = p;
  return QMPRS_OK;
}

int qmprs_plan_layout(qmprs_plan_t p, int64_t* vec_elems, int64_t* gate_elems, int64_t* tensor_elems,
                      int64_t* vec_off, int64_t* gate_off, int64_t* tensor_off) {
  if (!p) return QMPRS_ERR_INVALID;
  if (vec_elems) *vec_elems = p->vec_total;
  if (gate_elems) *gate_elems = p->gate_total;
  if (tensor_elems) *tensor_elems = p->tensor_total;
  for (int b = 0; b < p->B; ++b) {
    if (vec_off) vec_off[b] = p->vec_off[b];
    if (gate_off) gate_off[b] = p->gate_off[b];
    if (tensor_off) tensor_off[b] = p->tensor_off[b];
  }
  return QMPRS_OK;
}

int qmprs_plan_max_qubits(qmprs_plan_t p) { return p ? p->max_n : -1; }

int qmprs_plan_set_precision(qmprs_plan_t p, int precision) {
  if (!p) return QMPRS_ERR_INVALID;
  if (precision != QMPRS_PRECISION_FAST && precision != QMPRS_PRECISION_EXACT)
    return set_err(p->h, QMPRS_ERR_INVALID, "precision must be QMPRS_PRECISION_FAST or QMPRS_PRECISION_EXACT");
  p->precision = precision;
  return QMPRS_OK;
}

int qmprs_plan_precision(qmprs_plan_t p) { return p ? p->precision : -1; }

int qmprs_plan_set_autotune(qmprs_plan_t p, int enable) {
  if (!p) return QMPRS_ERR_INVALID;
  p->autotune = enable != 0;
  if (!p->autotune) p->gd.grid = 0;
  return QMPRS_OK;
}

int qmprs_plan_tuning(qmprs_plan_t p, int* pass_grid, int* tuned) {
  if (!p) return QMPRS_ERR_INVALID;
  if (pass_grid) *pass_grid = p->gd.grid > 0 ? std::min(p->gd.grid, p->nchunks) : std::min(PASS_GRID_DEFAULT, p->nchunks);
  if (tuned) *tuned = p->tuned ? 1 : 0;
  return QMPRS_OK;
}

int qmprs_plan_set_graphs(qmprs_plan_t p, int enable) {
  if (!p) return QMPRS_ERR_INVALID;
  p->graphs = enable != 0;
  return QMPRS_OK;
}

int qmprs_plan_graph_stats(qmprs_plan_t p, int* cached, int64_t* replays) {
  if (!p) return QMPRS_ERR_INVALID;
  int c = 0;
  for (auto& g : p->graph_cache) c += g.exec != nullptr;
  if (cached) *cached = c;
  if (replays) *replays = p->graph_replays;
  return QMPRS_OK;
}

int qmprs_plan_wide_stats(qmprs_plan_t p, int* grams, int* sweeps, int* refine_steps, float* last_correction) {
  if (!p) return QMPRS_ERR_INVALID;
  if (grams) *grams = p->bj_stats.calls;
  if (sweeps) *sweeps = p->bj_stats.sweeps;
  if (refine_steps) *refine_steps = p->bj_stats.refine_steps;
  if (last_correction) *last_correction = p->bj_stats.last_emax;
  return QMPRS_OK;
}

int qmprs_plan_upload(qmprs_plan_t p, const void* host, int64_t bytes, void* stream, void** dev_out) {
  if (!p || !host || !dev_out) return QMPRS_ERR_INVALID;
  *dev_out = nullptr;
  const int64_t elem = p->precision == QMPRS_PRECISION_EXACT ? (int64_t)sizeof(double2) : (int64_t)sizeof(float2);
  if (bytes != p->vec_total * elem)
    return set_err(p->h, QMPRS_ERR_INVALID, "packed statevector buffer does not match the qubit counts");
  if (!p->d_input) CK(cudaMalloc(&p->d_input, (size_t)p->vec_total * sizeof(double2)));
  // Pinned, device-mapped host memory is read by a copy kernel (k_upload);
  // anything else goes through the copy engine.
  cudaPointerAttributes at{};
  const bool mapped = cudaPointerGetAttributes(&at, host) == cudaSuccess && at.type == cudaMemoryTypeHost &&
                      at.devicePointer != nullptr && ((uintptr_t)at.devicePointer % 16) == 0 && bytes % 16 == 0;
  cudaGetLastError();   // clear a failed query of pageable memory
  if (mapped) launch_upload(p->d_input, at.devicePointer, bytes, (cudaStream_t)stream);
  else CK(cudaMemcpyAsync(p->d_input, host, (size_t)bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  CK(cudaGetLastError());
  *dev_out = p->d_input;
  return QMPRS_OK;
}

int qmprs_mps_from_statevector(qmprs_plan_t p, const void* sv_, int max_bond, double cutoff, void* tensors_,
                               int* bonds, void* target_, void* stream) {
  if (!p || !sv_ || !tensors_ || !bonds || !target_) return QMPRS_ERR_INVALID;
  if (max_bond < 1 || max_bond > p->max_bond)
    return set_err(p->h, QMPRS_ERR_INVALID, "`bond_dimension` must be an integer in [1, plan max_bond].");
  if (!(cutoff >= 0.0)) return set_err(p->h, QMPRS_ERR_INVALID, "cutoff must be >= 0");
  cudaStream_t s = (cudaStream_t)stream;
  const float2* sv = (const float2*)sv_;
  float2* target = (float2*)target_;
  double2* tensors = (double2*)tensors_;
  for (int b = 0; b < p->B; ++b)
    if (chi_eff_host(max_bond, p->n[b]) > TT_WIDE_MAXB)
      return set_err(p->h, QMPRS_ERR_UNSUPPORTED,
                     "statevector -> MPS supports bond dimensions up to 1024 (min(bond_dimension, 2^(n/2)) > 1024)");
  if (p->precision == QMPRS_PRECISION_EXACT)
    return exact_mps_from_statevector(p, (const double2*)sv_, max_bond, cutoff, tensors, bonds, (double2*)target_, s);
  const int64_t WW = (int64_t)p->tt_w * p->tt_w;
  const bool wide = 2 * p->tt_b > p->bd.eig_wmax;
  // the first step at which a Gram can be wider than eig_wmax (bond 2^(j+1))
  const int jwide = p->bd.eig_wmax >= TT_MAXW ? 6 : 5;
  {
    const int rc = ensure_tt_scratch(p);
    if (rc != QMPRS_OK) return rc;
  }
  CK(cudaMemsetAsync(p->d_err, 0, sizeof(int), s));
  const int64_t nb = (int64_t)p->B * (p->max_n + 1);
  CK(cudaMemcpyAsync(bonds, p->d_bond_init, sizeof(int) * nb, cudaMemcpyDeviceToDevice, s));
  launch_overlap(p->bd, sv, sv, p->partials, p->sq, s);
  launch_check_norms(p->B, p->sq, p->d_err, s);
  float2* buf[2] = {p->S0, p->S1};
  const int stride = p->max_n + 1;
  std::vector<int> hb(wide ? (size_t)p->B * stride : 0);
  auto read_bonds = [&]() -> int {
    CK(cudaMemcpyAsync(hb.data(), bonds, sizeof(int) * hb.size(), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return QMPRS_OK;
  };
  for (int j = 0; j + 2 <= p->max_n; ++j) {
    const float2* src = j == 0 ? sv : buf[(j - 1) & 1];
    launch_tt_gram(p->bd, j, sv, src, bonds, p->tt_partials, p->gram, s);
    launch_tt_eig(p->bd, j, bonds, p->gram, p->vwork, max_bond, cutoff, p->vsel2, tensors, p->max_bond,
                  p->tt_partials, 1e-13, s);
    launch_tt_project(p->bd, j, sv, src, buf[j & 1], bonds, p->vsel2, s);
    // Grams wider than eig_wmax and projections to more than 64 columns:
    // the blocked eigensolver and tiled products, state by state (possible
    // only from step jwide on)
    if (wide && j >= jwide) {
      int rc = read_bonds();
      if (rc != QMPRS_OK) return rc;
      bool any = false;
      for (int b = 0; b < p->B; ++b) {
        const int c = p->n[b] - 1 - j;
        if (c < 1) continue;
        const int r = hb[(size_t)b * stride + c + 1];
        if (r < 1 || r > p->tt_b || 2 * r <= p->bd.eig_wmax) continue;
        // fewer remainder rows than Gram columns: the row Gram (rank <= 2^c)
        const float2* rowsrc = ipow2(c) < 2 * r ? src + p->vec_off[b] : nullptr;
        const int e = tt_block_eig(p->bd, b, c, 2 * r, p->gram, rowsrc, p->bj, p->bj_sub, bonds, p->vsel2, tensors,
                                   p->max_bond, max_bond, cutoff, BJ_TOL_FAST, s, &p->bj_stats);
        if (e != 0) return cuda_fail(p->h, (cudaError_t)e, "stage (a) blocked eigensolver");
        any = true;
      }
      if (any) {
        rc = read_bonds();
        if (rc != QMPRS_OK) return rc;
      }
      for (int b = 0; b < p->B; ++b) {
        const int c = p->n[b] - 1 - j;
        if (c < 1) continue;
        const int r = hb[(size_t)b * stride + c + 1], keep = hb[(size_t)b * stride + c];
        if (r < 1 || keep < 1 || r > p->tt_b || keep > p->tt_b) continue;
        if (2 * r <= p->bd.eig_wmax && keep <= TT_MAXB) continue;
        const int w = 2 * r;
        const float2* m = src + p->vec_off[b];
        launch_cgemm(m, w, p->vsel2 + (int64_t)b * WW, p->tt_b, buf[j & 1] + p->vec_off[b], keep, ipow2(c), keep, w,
                     s);
      }
    }
  }
  launch_tt_site0(p->bd, buf[0], buf[1], bonds, tensors, p->max_bond, p->sq, s);
  if (wide) {
    const int rc = read_bonds();
    if (rc != QMPRS_OK) return rc;
  }
  for (int j = 0; j + 2 <= p->max_n; ++j) {
    const float2* src = j == 0 ? buf[0] : buf[(j - 1) & 1];
    launch_mps_contract(p->bd, j, tensors, bonds, p->max_bond, src, buf[j & 1], target, s);
    if (wide) launch_wide_contract(p, j, tensors, hb, src, buf[j & 1], target, s);
  }
  return check_kernel_errors(p, s);
}

int qmprs_mps_to_statevector(qmprs_plan_t p, const void* tensors, const int* bonds, void* out, void* stream) {
  if (!p || !tensors || !bonds || !out) return QMPRS_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  CK(cudaMemsetAsync(p->d_err, 0, sizeof(int), s));
  if (p->precision == QMPRS_PRECISION_EXACT) {
    int rc = ensure_exact(p);
    if (rc != QMPRS_OK) return rc;
    std::vector<int> hbx((size_t)p->B * (p->max_n + 1));
    if ((rc = read_ints(p, bonds, hbx, s)) != QMPRS_OK) return rc;
    for (int b = 0; b < p->B; ++b)
      for (int c = 0; c <= p->n[b]; ++c) {
        const int r = hbx[(size_t)b * (p->max_n + 1) + c];
        if (r < 1 || r > chi_eff_host(p->max_bond, p->n[b]) || (c > 0 && c < p->n[b] && r > (1 << std::min(c, p->n[b] - c))))
          return set_err(p->h, QMPRS_ERR_INVALID, "a bond of the MPS is out of range for the plan");
      }
    x_contract(p, (const double2*)tensors, hbx, p->XT, s);
    launch_x_to_d(p->bd, p->XT, (double2*)out, s);
    return check_kernel_errors(p, s);
  }
  float2* buf[2] = {p->S0, p->S1};
  const bool wide = p->tt_b > TT_MAXB;
  std::vector<int> hb(wide ? (size_t)p->B * (p->max_n + 1) : 0);
  if (wide) {
    CK(cudaMemcpyAsync(hb.data(), bonds, sizeof(int) * hb.size(), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  for (int j = 0; j + 2 <= p->max_n; ++j) {
    const float2* src = j == 0 ? buf[0] : buf[(j - 1) & 1];
    launch_mps_contract(p->bd, j, (const double2*)tensors, bonds, p->max_bond, src, buf[j & 1], (float2*)out, s);
    if (wide) launch_wide_contract(p, j, (const double2*)tensors, hb, src, buf[j & 1], (float2*)out, s);
  }
  return check_kernel_errors(p, s);
}

int qmprs_unitary_layers(qmprs_plan_t p, const void* target_, int num_layers, double fidelity_threshold,
                         void* gates_, int8_t* arity, int* layers_out, void* layer_fid_, void* stream) {
  if (!p || !target_ || !gates_ || !arity || !layers_out || !layer_fid_) return QMPRS_ERR_INVALID;
  if (num_layers < 1 || num_layers > p->max_layers)
    return set_err(p->h, QMPRS_ERR_INVALID, "The number of layers must be a positive integer (<= plan max_layers).");
  if (!(fidelity_threshold >= 0.0 && fidelity_threshold <= 1.0))
    return set_err(p->h, QMPRS_ERR_INVALID, "The fidelity threshold must be a float between 0 and 1.");
  cudaStream_t s = (cudaStream_t)stream;
  if (p->precision == QMPRS_PRECISION_EXACT)
    return exact_unitary_layers(p, (const double2*)target_, num_layers, fidelity_threshold, (double2*)gates_,
                                (signed char*)arity, layers_out, (double2*)layer_fid_, s);
  const float2* target = (const float2*)target_;
  double2* gates = (double2*)gates_;
  signed char* ar = (signed char*)arity;
  double2* layer_fid = (double2*)layer_fid_;
  CK(cudaMemsetAsync(p->d_err, 0, sizeof(int), s));
  CK(cudaMemsetAsync(layers_out, 0, sizeof(int) * p->B, s));
  CK(cudaMemsetAsync(layer_fid, 0, sizeof(double2) * (size_t)p->B * num_layers, s));
  launch_fill_int(p->active, p->B, 1, s);
  float2* work = p->S0;
  launch_copy_normalize(p->bd, target, work, p->partials, p->sq, s);
  float2* buf[2] = {p->S1, p->S2};
  const double atol = 1.0 - fidelity_threshold;
  const int64_t nb = (int64_t)p->B * (p->max_n + 1);
  auto body = [&](cudaStream_t st, bool capturing) -> int {
    for (int l = 0; l < num_layers; ++l) {
      CK(cudaMemcpyAsync(p->bonds, p->d_bond_init, sizeof(int) * nb, cudaMemcpyDeviceToDevice, st));
      for (int j = 0; j + 2 <= p->max_n; ++j) {
        const float2* src = j == 0 ? work : buf[(j - 1) & 1];
        launch_layer_gram(p->bd, j, work, src, p->bonds, p->partials, p->vsel, p->bonds, p->site_t, p->active,
                          st);
        launch_layer_project(p->bd, j, work, src, buf[j & 1], p->bonds, p->vsel, p->active, st);
      }
      launch_layer_build(p->bd, l, buf[0], buf[1], p->bonds, p->site_t, gates, ar, p->active, st);
      // inverse of the new layer: tile passes of two 4-qubit windows (up to
      // six gates per read and write of the working state)
      launch_layer_plan(p->bd, p->gd, ar, ORDER_LAYER_INV, l, p->active, st);
      for (int r = 0; r < layer_pass_bound(p->max_n); ++r)
        // exact FP32 products: the next layer's bond-2 truncation decides at
        // singular values near the 1e-10 cutoff of this working state
        launch_rebuild_pass(p->bd, p->gd, r, work, gates, ar, nullptr, p->active, st, ORDER_LAYER_INV, l, true);
      launch_layer_fidelity(p->bd, l, work, num_layers, atol, layer_fid, layers_out, p->active, st);
      if (!capturing) {
        launch_count_active(p->B, p->active, p->num_active, st);
        int na = 0;
        CK(cudaMemcpyAsync(&na, p->num_active, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (na == 0) break;
      }
    }
    return QMPRS_OK;
  };
  const std::vector<uint64_t> key = {2, ptr_key(target), ptr_key(gates), ptr_key(ar), ptr_key(layers_out),
                                     ptr_key(layer_fid), (uint64_t)num_layers, dbl_key(fidelity_threshold)};
  const int rc = run_stage(p, key, s, body);
  if (rc != QMPRS_OK) return rc;
  return check_kernel_errors(p, s);
}

int qmprs_optimize_layers(qmprs_plan_t p, const void* target_, void* gates_, const int8_t* arity,
                          const int* num_layers, int num_sweeps, double stop_fidelity, double* sweep_fid,
                          int* sweeps_done, void* stream) {
  if (!p || !target_ || !gates_ || !arity || !num_layers || !sweep_fid || !sweeps_done) return QMPRS_ERR_INVALID;
  if (num_sweeps < 0) return set_err(p->h, QMPRS_ERR_INVALID, "num_sweeps must be >= 0");
  cudaStream_t s = (cudaStream_t)stream;
  const float2* target = (const float2*)target_;
  double2* gates = (double2*)gates_;
  const signed char* ar = (const signed char*)arity;
  CK(cudaMemsetAsync(p->d_err, 0, sizeof(int), s));
  CK(cudaMemsetAsync(sweeps_done, 0, sizeof(int) * p->B, s));
  if (num_sweeps == 0) return QMPRS_OK;
  CK(cudaMemsetAsync(sweep_fid, 0, sizeof(double) * (size_t)p->B * num_sweeps, s));
  if (p->precision == QMPRS_PRECISION_EXACT)
    return exact_optimize_layers(p, (const double2*)target_, (double2*)gates_, (const signed char*)arity, num_layers,
                                 num_sweeps, stop_fidelity, sweep_fid, sweeps_done, s);
  int max_gates = 0;
  int rc = read_max_gates(p, num_layers, s, &max_gates);
  if (rc != QMPRS_OK) return rc;
  launch_fill_int(p->active, p->B, 1, s);
  launch_overlap(p->bd, target, target, p->partials, p->tnorm, s);
  if (p->max_n <= SWEEP_FUSED_MAXN && !p->prof) {   // every state fits one block's shared memory
    const int e = launch_sweep_fused(p->bd, p->max_n, target, gates, ar, num_layers, p->active, p->tnorm, num_sweeps,
                                     stop_fidelity, sweep_fid, sweeps_done, s);
    if (e != 0) return cuda_fail(p->h, (cudaError_t)e, "k_sweep_fused");
    return check_kernel_errors(p, s);
  }
  // group plan of the backward order (the gates' arity does not change
  // between sweeps)
  launch_group_plan(p->bd, p->gd, ar, num_layers, s);
  std::vector<int> ngroups(p->B, 0), nrgroups(p->B, 0);
  CK(cudaMemcpyAsync(ngroups.data(), p->d_ngroups, sizeof(int) * p->B, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(nrgroups.data(), p->d_nrgroups, sizeof(int) * p->B, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  int max_groups = 0, max_rpasses = 0;
  for (int b = 0; b < p->B; ++b) {
    max_groups = std::max(max_groups, ngroups[b]);
    max_rpasses = std::max(max_rpasses, (nrgroups[b] + 1) / 2);
  }
  float2* psi = p->S0;
  float2* t = p->S1;
  const bool prof = p->prof;
  // Autotuner of the tile passes' grid: on a batch signature the handle has
  // not tuned yet, the first sweeps run one candidate each (the resident
  // blocks, 4 per SM; one block per chunk, scheduled by the hardware; 2 per
  // SM), timed with events over the sweep and divided by the states active
  // in it; the fastest is kept for the rest of the call and cached on the
  // handle.  The grid changes no result: every chunk is reduced in a fixed
  // order whichever block takes it.
  const uint64_t sig = plan_signature(p);
  bool tune = false;
  if (p->autotune && !prof) {
    bool found = false;
    for (auto& e : p->h->tuned)
      if (e.first == sig) {
        p->gd.grid = e.second;
        found = true;
      }
    tune = !found && num_sweeps >= 2;
    p->tuned = found;
  }
  const std::vector<int> cands = {PASS_GRID_DEFAULT, p->nchunks, 2 * 152};
  auto body = [&](cudaStream_t st, bool capturing) -> int {
    ProfLog log;
    std::vector<int> act(p->B, 1);
    std::vector<double> cost;
    cudaEvent_t te[2] = {nullptr, nullptr};
    if (tune) {
      CK(cudaEventCreate(&te[0]));
      CK(cudaEventCreate(&te[1]));
    }
    for (int sw = 0; sw < num_sweeps; ++sw) {
      const bool trial = tune && sw < (int)cands.size();
      int nact = 0;
      if (trial) {
        p->gd.grid = cands[sw];
        launch_count_active(p->B, p->active, p->num_active, st);
        CK(cudaMemcpyAsync(&nact, p->num_active, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        CK(cudaEventRecord(te[0], st));
      }
      // algorithmic bytes per rebuild pass / group pass, counted from the
      // states active in this sweep
      std::vector<double> amp_rb(prof ? max_rpasses : 0, 0.0), amp_grp(prof ? max_groups : 0, 0.0);
      if (prof) {
        CK(cudaMemcpyAsync(act.data(), p->active, sizeof(int) * p->B, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int b = 0; b < p->B; ++b)
          if (act[b]) {
            for (int r = 0; r < (nrgroups[b] + 1) / 2; ++r) amp_rb[r] += (double)ipow2(p->n[b]);
            for (int g = 0; g < ngroups[b]; ++g) amp_grp[g] += (double)ipow2(p->n[b]);
          }
      }
      // C|0>: two 4-qubit windows of consecutive gates per pass
      launch_set_zero_state(p->bd, psi, p->active, st);
      for (int r = 0; r < max_rpasses; ++r) {
        log.begin(prof, st);
        launch_rebuild_pass(p->bd, p->gd, r, psi, gates, ar, num_layers, p->active, st);
        log.end(prof, 2, st);
        if (prof) p->prof_bytes[2] += 16.0 * amp_rb[r];
      }
      // backward sweep by groups: the pass applies group g-1's peels to psi
      // and its new gates to t (the target itself for g = 1) and reduces the
      // cross matrix of group g; the polar kernel runs group g's steps on it
      for (int g = 0; g < max_groups; ++g) {
        log.begin(prof, st);
        const int e = launch_group_pass(p->bd, p->gd, g, psi, g <= 1 ? target : t, t, gates, ar, num_layers,
                                        p->active, p->tnorm, st);
        if (e != 0) return cuda_fail(p->h, (cudaError_t)e, "cudaFuncSetAttribute(k_group_pass)");
        log.end(prof, 0, st);
        log.begin(prof, st);
        launch_group_polar(p->bd, p->gd, g, gates, ar, num_layers, p->active, p->nuc, st);
        log.end(prof, 3, st);
        if (prof) p->prof_bytes[0] += (g == 0 ? 16.0 : 32.0) * amp_grp[g];
      }
      log.flush(p);
      if (trial) {
        CK(cudaEventRecord(te[1], st));
        CK(cudaEventSynchronize(te[1]));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, te[0], te[1]));
        cost.push_back(nact > 0 ? ms / nact : 1e30);
        if (sw + 1 == (int)cands.size() || sw + 1 == num_sweeps) {
          const int best = (int)(std::min_element(cost.begin(), cost.end()) - cost.begin());
          p->gd.grid = cands[best];
          p->h->tuned.push_back({sig, cands[best]});
          p->tuned = true;
        }
      }
      CK(cudaMemsetAsync(p->num_active, 0, sizeof(int), st));
      launch_sweep_finish(p->B, sw, num_sweeps, p->nuc, p->tnorm, sweep_fid, sweeps_done, p->active,
                          stop_fidelity, p->num_active, st);
      if (stop_fidelity > 0.0 && !capturing) {
        int na = 0;
        CK(cudaMemcpyAsync(&na, p->num_active, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (na == 0) break;
      }
    }
    if (tune && !p->tuned && !cost.empty()) {   // the call ended before every candidate ran
      const int best = (int)(std::min_element(cost.begin(), cost.end()) - cost.begin());
      p->gd.grid = cands[best];
      p->h->tuned.push_back({sig, cands[best]});
      p->tuned = true;
    }
    for (cudaEvent_t e : te)
      if (e) cudaEventDestroy(e);
    return QMPRS_OK;
  };
  const std::vector<uint64_t> key = {1, ptr_key(target), ptr_key(gates), ptr_key(ar), ptr_key(num_layers),
                                     ptr_key(sweep_fid), ptr_key(sweeps_done), (uint64_t)num_sweeps,
                                     dbl_key(stop_fidelity), (uint64_t)max_groups, (uint64_t)max_rpasses,
                                     (uint64_t)p->gd.grid};
  rc = tune ? body(s, false) : run_stage(p, key, s, body);
  if (rc != QMPRS_OK) return rc;
  return check_kernel_errors(p, s);
}

// One sweep's backward pass with the update left out: the same kernels
// (fused for small states, rebuild + group passes otherwise) write every
// gate's environment to env and keep the gates.
int qmprs_layer_environments(qmprs_plan_t p, const void* target_, const void* gates_, const int8_t* arity,
                             const int* num_layers, void* env_, void* stream) {
  if (!p || !target_ || !gates_ || !arity || !num_layers || !env_) return QMPRS_ERR_INVALID;
  if (p->precision == QMPRS_PRECISION_EXACT)
    return set_err(p->h, QMPRS_ERR_INVALID, "qmprs_layer_environments runs in the fast precision only");
  cudaStream_t s = (cudaStream_t)stream;
  const float2* target = (const float2*)target_;
  // the environment mode reads the gates and never writes them
  double2* gates = const_cast<double2*>((const double2*)gates_);
  double2* env = (double2*)env_;
  const signed char* ar = (const signed char*)arity;
  CK(cudaMemsetAsync(p->d_err, 0, sizeof(int), s));
  CK(cudaMemsetAsync(env, 0, sizeof(double2) * (size_t)p->gate_total, s));
  int max_gates = 0;
  int rc = read_max_gates(p, num_layers, s, &max_gates);
  if (rc != QMPRS_OK) return rc;
  launch_fill_int(p->active, p->B, 1, s);
  launch_overlap(p->bd, target, target, p->partials, p->tnorm, s);
  if (p->max_n <= SWEEP_FUSED_MAXN) {
    const int e = launch_sweep_fused(p->bd, p->max_n, target, gates, ar, num_layers, p->active, p->tnorm, 1, 0.0,
                                     nullptr, nullptr, s, env);
    if (e != 0) return cuda_fail(p->h, (cudaError_t)e, "k_sweep_fused");
    return check_kernel_errors(p, s);
  }
  launch_group_plan(p->bd, p->gd, ar, num_layers, s);
  std::vector<int> ngroups(p->B, 0), nrgroups(p->B, 0);
  CK(cudaMemcpyAsync(ngroups.data(), p->d_ngroups, sizeof(int) * p->B, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(nrgroups.data(), p->d_nrgroups, sizeof(int) * p->B, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  int max_groups = 0, max_rpasses = 0;
  for (int b = 0; b < p->B; ++b) {
    max_groups = std::max(max_groups, ngroups[b]);
    max_rpasses = std::max(max_rpasses, (nrgroups[b] + 1) / 2);
  }
  float2* psi = p->S0;
  float2* t = p->S1;
  launch_set_zero_state(p->bd, psi, p->active, s);
  for (int r = 0; r < max_rpasses; ++r)
    launch_rebuild_pass(p->bd, p->gd, r, psi, gates, ar, num_layers, p->active, s);
  for (int g = 0; g < max_groups; ++g) {
    const int e = launch_group_pass(p->bd, p->gd, g, psi, g <= 1 ? target : t, t, gates, ar, num_layers, p->active,
                                    p->tnorm, s);
    if (e != 0) return cuda_fail(p->h, (cudaError_t)e, "cudaFuncSetAttribute(k_group_pass)");
    launch_group_polar(p->bd, p->gd, g, gates, ar, num_layers, p->active, p->nuc, s, env);
  }
  return check_kernel_errors(p, s);
}

int qmprs_circuit_state(qmprs_plan_t p, const void* gates, const int8_t* arity, const int* num_layers, void* out,
                        void* stream) {
  if (!p || !gates || !arity || !num_layers || !out) return QMPRS_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  CK(cudaMemsetAsync(p->d_err, 0, sizeof(int), s));
  if (p->precision == QMPRS_PRECISION_EXACT)
    return exact_circuit_state(p, (const double2*)gates, (const signed char*)arity, num_layers, (double2*)out, s);
  int max_gates = 0;
  int rc = read_max_gates(p, num_layers, s, &max_gates);
  if (rc != QMPRS_OK) return rc;
  const signed char* ar = (const signed char*)arity;
  // C|0> with the rebuild passes of the sweep: two 4-qubit windows of
  // consecutive gates per pass, in fp32 FMAs (the reported state, so not
  // the split-precision tensor-core products of the sweep's rebuild)
  launch_group_plan(p->bd, p->gd, ar, num_layers, s);
  std::vector<int> nrgroups(p->B, 0);
  CK(cudaMemcpyAsync(nrgroups.data(), p->d_nrgroups, sizeof(int) * p->B, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  int passes = 0;
  for (int b = 0; b < p->B; ++b) passes = std::max(passes, (nrgroups[b] + 1) / 2);
  float2* psi = (float2*)out;
  launch_set_zero_state(p->bd, psi, nullptr, s);
  for (int r = 0; r < passes; ++r)
    launch_rebuild_pass(p->bd, p->gd, r, psi, (const double2*)gates, ar, num_layers, nullptr, s, ORDER_FWD, 0, true);
  CK(cudaGetLastError());
  return QMPRS_OK;
}

int qmprs_overlap(qmprs_plan_t p, const void* a, const void* b, void* out, void* stream) {
  if (!p || !a || !b || !out) return QMPRS_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (p->precision == QMPRS_PRECISION_EXACT)
    launch_d_dot(p->bd, (const double2*)a, (const double2*)b, p->partials, (double2*)out, s);
  else
    launch_overlap(p->bd, (const float2*)a, (const float2*)b, p->partials, (double2*)out, s);
  CK(cudaGetLastError());
  return QMPRS_OK;
}

int qmprs_apply_layer(qmprs_plan_t p, void* vec, const void* gates, const int8_t* arity, int layer, int inverse,
                      void* stream) {
  if (!p || !vec || !gates || !arity) return QMPRS_ERR_INVALID;
  if (layer < 0 || layer >= p->max_layers) return set_err(p->h, QMPRS_ERR_INVALID, "layer index out of range");
  cudaStream_t s = (cudaStream_t)stream;
  const signed char* ar = (const signed char*)arity;
  if (p->precision == QMPRS_PRECISION_EXACT) {
    const int rc = ensure_exact(p);
    if (rc != QMPRS_OK) return rc;
    CK(cudaMemsetAsync(p->d_err, 0, sizeof(int), s));
    launch_x_from_d(p->bd, (const double2*)vec, p->X0, s);
    for (int st = 0; st < p->max_n; ++st) {
      GateSel sel{inverse ? SEL_INVERSE : SEL_LAYER_FWD, st, layer, inverse ? 1 : 0, (const double2*)gates, ar, nullptr,
                  nullptr};
      launch_x_apply_gate(p->bd, p->X0, sel, s);
    }
    launch_x_to_d(p->bd, p->X0, (double2*)vec, s);
    return check_kernel_errors(p, s);
  }
  const int mode = inverse ? ORDER_LAYER_INV : ORDER_LAYER_FWD;
  launch_layer_plan(p->bd, p->gd, ar, mode, layer, nullptr, s);
  for (int r = 0; r < layer_pass_bound(p->max_n); ++r)
    launch_rebuild_pass(p->bd, p->gd, r, (float2*)vec, (const double2*)gates, ar, nullptr, nullptr, s, mode, layer,
                        true);
  CK(cudaGetLastError());
  return QMPRS_OK;
}

}  // extern "C"
