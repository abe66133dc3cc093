// Learned warm start: the BF16 multilayer perceptron that maps a two-site
// block's analytic initial gate (plus its neighbours and a position
// embedding) to the gate the sweeps converge to.  No reference counterpart
// (the reference initialises layers analytically only).
//
// k_gemm_tc      C = A B^T for row-major BF16 A [M x K] and B [N x K] on the
//                5th-generation tensor cores: operands staged into shared
//                memory in the canonical K-major no-swizzle layout (8-row x
//                16-byte core matrices), one elected thread issues
//                tcgen05.mma (kind::f16, M = 128, N <= 256, K = 16 per
//                instruction) into an FP32 accumulator in tensor memory,
//                tcgen05.commit arrives on an mbarrier, and all four warps
//                read their 32 accumulator lanes back with tcgen05.ld.
//                Epilogue: bias, GELU (tanh form), FP32 pre-activation, BF16
//                activation and its transpose; or FP32 split-K partials.
// k_mlp_loss     phase-invariant gate loss |M - e^{i phi} U|_F^2 minimised
//                over phi, and its gradient.
// k_mlp_overlap_grad  circuit-overlap loss: the gradient of a state's
//                fidelity |<t|C|0>|^2 / <t|t> with respect to each
//                projected gate, from the gate's environment.
// k_act_back     dZ = dH * GELU'(Z), BF16 and transposed BF16.
// k_col_sum      bias gradients (column sums in fixed order).
// k_splitk_sum   split-K reduction in fixed order.
// k_adam         Adam on FP32 master weights, BF16 copies W and W^T.
//
// Every wait on the tensor cores has an iteration limit; a timeout sets an
// error flag, waits once more (bounded) and frees the tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"
#include "qmprs_gb300.h"
#include "small_linalg.h"

#define MLP_BM 128
#define MLP_BK 64
#define MLP_MAXN 256
#define MLP_THREADS 128
#define MLP_TMEM_COLS 256
// A tile 128 x 64 BF16 (16 KB) + B tile 256 x 64 BF16 (32 KB); the request
// is padded to 96 KB so at most two blocks share an SM (2 x 256 TMEM columns).
#define MLP_SMEM_A 16384
#define MLP_SMEM_B 32768
#define MLP_SMEM_REQ (96 * 1024)
#define MLP_WAIT_LIMIT (1 << 22)
#define MLP_WAIT_NS 1000000000ull   // and at most one second of wall time

enum { MLP_ACT_NONE = 0, MLP_ACT_GELU = 1 };

struct GemmArgs {
  const __nv_bfloat16* A;
  int lda;
  const __nv_bfloat16* B;
  int ldb;
  int M, N, K;
  int ksplit;          // K range per blockIdx.z
  const float* bias;   // [N] or null
  int act;
  float* Cf;           // fp32 [M x ldc] (pre-activation) or null
  int ldc;
  __nv_bfloat16* Cb;   // bf16 activation [M x ldc] or null
  __nv_bfloat16* CbT;  // bf16 activation transposed [N x ldt] or null
  int ldt;
  float* part;         // split-K partials [gridDim.z][M][N] (used when gridDim.z > 1)
  const float* resid;  // fp32 [M x ldr] added to z before the activation, or null
  int ldr;
  int* err;
};

__device__ __forceinline__ float gelu_f(float z) {
  const float c = 0.7978845608028654f;   // sqrt(2 / pi)
  const float u = c * (z + 0.044715f * z * z * z);
  return 0.5f * z * (1.f + tanhf(u));
}

__device__ __forceinline__ float gelu_grad_f(float z) {
  const float c = 0.7978845608028654f;
  const float u = c * (z + 0.044715f * z * z * z);
  const float t = tanhf(u);
  return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * c * (1.f + 3.f * 0.044715f * z * z);
}

// ---- PTX wrappers -----------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

// Canonical K-major, no-swizzle shared-memory descriptor: core matrices of
// 8 rows x 16 bytes, LBO = byte step between core matrices along K, SBO =
// byte step between 8-row groups; version 1 (bits 46-47), layout 0.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// kind::f16 instruction descriptor: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
__host__ __device__ constexpr uint32_t make_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         int accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                   smem_u32(mbar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait for the phase with the given parity; false on timeout.
// try_wait may suspend the thread for a system-dependent time, so the
// bound is both an iteration count and a wall-clock limit.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity) {
  const uint64_t t0 = globaltimer_ns();
  for (int it = 0; it < MLP_WAIT_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
    if (done) return true;
    if (globaltimer_ns() - t0 > MLP_WAIT_NS) return false;
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// ---- GEMM ------------------------------------------------------------------------

// Stage rows [r0, r0 + rows) x K columns [k0, k0 + kc) of a row-major BF16
// matrix into the core-matrix layout: 16-byte chunk (r, kg) at
// (r / 8) * 1024 + kg * 128 + (r % 8) * 16.  kc is a multiple of 16;
// chunks past kc are zero-filled.
__device__ __forceinline__ void stage_tile(uint8_t* s, const __nv_bfloat16* g, int ld, int r0, int rows, int k0,
                                           int kc) {
  for (int c = threadIdx.x; c < rows * 8; c += blockDim.x) {
    const int r = c >> 3, kg = c & 7;
    uint8_t* dst = s + (r >> 3) * 1024 + kg * 128 + (r & 7) * 16;
    if (kg * 8 < kc) {
      cp_async16(dst, g + (int64_t)(r0 + r) * ld + k0 + kg * 8);
    } else {
      *reinterpret_cast<uint4*>(dst) = make_uint4(0, 0, 0, 0);
    }
  }
}

__global__ void __launch_bounds__(MLP_THREADS, 1) k_gemm_tc(GemmArgs g) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem;
  uint8_t* sB = smem + MLP_SMEM_A;
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_sh;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * MLP_BM;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_sh)),
                 "r"(MLP_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (threadIdx.x == 0) {
    mbar_init(&mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_sh;
  const uint32_t idesc = make_idesc_bf16(MLP_BM, g.N);
  const int kbeg = blockIdx.z * g.ksplit;
  const int kend = kbeg + g.ksplit < g.K ? kbeg + g.ksplit : g.K;
  uint32_t phase = 0;
  bool ok = true;
  for (int k0 = kbeg; k0 < kend; k0 += MLP_BK) {
    const int kc = kend - k0 < MLP_BK ? kend - k0 : MLP_BK;
    stage_tile(sA, g.A, g.lda, m0, MLP_BM, k0, kc);
    stage_tile(sB, g.B, g.ldb, 0, g.N, k0, kc);
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
      tc_fence_after();
      for (int kk = 0; kk < kc / 16; ++kk) {
        const uint64_t ad = make_desc(smem_u32(sA) + kk * 256, 128, 1024);
        const uint64_t bd = make_desc(smem_u32(sB) + kk * 256, 128, 1024);
        mma_bf16(tmem, ad, bd, idesc, (k0 > kbeg || kk > 0) ? 1 : 0);
      }
      mma_commit(&mbar);
    }
    ok = __syncthreads_and(mbar_wait(&mbar, phase) ? 1 : 0) != 0;   // uniform decision
    phase ^= 1u;
    if (!ok) break;
  }
  if (!ok) {
    if (threadIdx.x == 0) atomicOr(g.err, KERR_TC_TIMEOUT);
    (void)mbar_wait(&mbar, phase ^ 1u);   // the outstanding commit, bounded
  } else if (kend > kbeg) {
    tc_fence_after();
    const int row = m0 + warp * 32 + lane;
    const bool split = gridDim.z > 1;
    for (int c0 = 0; c0 < g.N; c0 += 16) {
      uint32_t v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int col = c0 + j;
        float z = __uint_as_float(v[j]);
        if (split) {
          g.part[((int64_t)blockIdx.z * g.M + row) * g.N + col] = z;
          continue;
        }
        if (g.bias) z += g.bias[col];
        if (g.resid) z += g.resid[(int64_t)row * g.ldr + col];
        if (g.Cf) g.Cf[(int64_t)row * g.ldc + col] = z;
        const float a = g.act == MLP_ACT_GELU ? gelu_f(z) : z;
        if (g.Cb) g.Cb[(int64_t)row * g.ldc + col] = __float2bfloat16_rn(a);
        if (g.CbT) g.CbT[(int64_t)col * g.ldt + row] = __float2bfloat16_rn(a);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(MLP_TMEM_COLS)
                 : "memory");
  }
}

// Test of the bounded completion wait: one block allocates tensor memory as
// k_gemm_tc does and waits on an mbarrier at which no tcgen05.commit will
// arrive (nothing is issued).  The wait gives up after its limit, the
// timeout bit is raised and the tensor memory is freed: the path k_gemm_tc
// takes after a timeout, without a fault and with the context usable.
__global__ void __launch_bounds__(MLP_THREADS, 1) k_tc_wait_selftest(int* err) {
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_sh;
  const int warp = threadIdx.x >> 5;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_sh)),
                 "r"(MLP_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (threadIdx.x == 0) {
    mbar_init(&mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_sh;
  const bool ok = __syncthreads_and(mbar_wait(&mbar, 0u) ? 1 : 0) != 0;
  if (!ok && threadIdx.x == 0) atomicOr(err, KERR_TC_TIMEOUT);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(MLP_TMEM_COLS)
                 : "memory");
  }
}

// part [S][M][N] -> C (+bias, act), fixed order over S
__global__ void k_splitk_sum(const float* part, int S, int M, int N, const float* bias, const float* resid, int ldr,
                             int act, float* Cf, int ldc, __nv_bfloat16* Cb, __nv_bfloat16* CbT, int ldt) {
  const int64_t total = (int64_t)M * N;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int row = (int)(i / N), col = (int)(i % N);
    float z = 0.f;
    for (int s = 0; s < S; ++s) z += part[(int64_t)s * total + i];
    if (bias) z += bias[col];
    if (resid) z += resid[(int64_t)row * ldr + col];
    if (Cf) Cf[(int64_t)row * ldc + col] = z;
    const float a = act == MLP_ACT_GELU ? gelu_f(z) : z;
    if (Cb) Cb[(int64_t)row * ldc + col] = __float2bfloat16_rn(a);
    if (CbT) CbT[(int64_t)col * ldt + row] = __float2bfloat16_rn(a);
  }
}

// ---- elementwise kernels -----------------------------------------------------------

// Per sample: Y = 4x4 complex M (row-major, interleaved re/im, 32 floats),
// U the target unitary in the same layout, w the sample weight (0 for
// padding).  loss = w (|M|^2 + |U|^2 - 2 |Tr(U^H M)|) = w min_phi |M - e^{i phi} U|^2;
// dY = w (2 M - 2 e^{i phi*} U) / sum(w), phi* = arg Tr(U^H M).
__global__ void k_mlp_loss(const float* Y, const float* U, const float* w, int B, float inv_wsum, float* loss,
                           float* dY, __nv_bfloat16* dYb, __nv_bfloat16* dYT, int ldt) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < B; s += gridDim.x * blockDim.x) {
    const float* y = Y + (int64_t)s * 32;
    const float* u = U + (int64_t)s * 32;
    float tr_re = 0.f, tr_im = 0.f, my = 0.f, uu = 0.f;
    for (int i = 0; i < 16; ++i) {
      const float mr = y[2 * i], mi = y[2 * i + 1], ur = u[2 * i], ui = u[2 * i + 1];
      tr_re += ur * mr + ui * mi;   // conj(u) m
      tr_im += ur * mi - ui * mr;
      my += mr * mr + mi * mi;
      uu += ur * ur + ui * ui;
    }
    const float at = sqrtf(tr_re * tr_re + tr_im * tr_im);
    const float ws = w[s];
    loss[s] = ws * (my + uu - 2.f * at);
    const float pr = at > 0.f ? tr_re / at : 1.f, pi = at > 0.f ? tr_im / at : 0.f;   // e^{i phi*}
    const float sc = 2.f * ws * inv_wsum;
    for (int i = 0; i < 16; ++i) {
      const float ur = u[2 * i], ui = u[2 * i + 1];
      const float gr = sc * (y[2 * i] - (pr * ur - pi * ui));
      const float gi = sc * (y[2 * i + 1] - (pr * ui + pi * ur));
      dY[(int64_t)s * 32 + 2 * i] = gr;
      dY[(int64_t)s * 32 + 2 * i + 1] = gi;
      dYb[(int64_t)s * 32 + 2 * i] = __float2bfloat16_rn(gr);
      dYb[(int64_t)s * 32 + 2 * i + 1] = __float2bfloat16_rn(gi);
      dYT[(int64_t)(2 * i) * ldt + s] = __float2bfloat16_rn(gr);
      dYT[(int64_t)(2 * i + 1) * ldt + s] = __float2bfloat16_rn(gi);
    }
  }
}

// Circuit-overlap loss.  Row r's gate U (the projected network output, in
// its slot of the gate store) and its environment E give the state's overlap
// f = sum_ac U[a,c] E[a,c] (the same for every gate of the state, up to
// rounding) and fidelity F = |f|^2 tinv[r], written to fid[r].  The gradient
// of -gscale F with respect to U (complex form d/dRe + i d/dIm) is
// G = -2 gscale tinv[r] f conj(E); it reaches the network output Y through
// the tangent map of the polar factor at U: dY = U skew(U^H G),
// skew(X) = (X - X^H) / 2 (the Hermitian part of U^H dY does not move the
// polar factor).  Rows rows..B-1 (padding) get zero gradient.
__global__ void k_mlp_overlap_grad(const double2* env, const double2* gates, const int64_t* slots,
                                   const signed char* kind, const float* tinv, int rows, int B, float gscale,
                                   float* fid, float* dY, __nv_bfloat16* dYb, __nv_bfloat16* dYT, int ldt) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < B; s += gridDim.x * blockDim.x) {
    float out[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) out[i] = 0.f;
    if (s < rows) {
      const int m = kind[s] == 1 ? 2 : 4;
      const double2* u = gates + slots[s] * 16;
      const double2* e = env + slots[s] * 16;
      double2 f = czero();
      for (int i = 0; i < m * m; ++i) f = cadd(f, cmul(u[i], e[i]));
      const double ti = (double)tinv[s];
      fid[s] = (float)((f.x * f.x + f.y * f.y) * ti);
      const double c = -2.0 * (double)gscale * ti;
      double2 G[16], X[16];
      for (int i = 0; i < m * m; ++i) {
        const double2 fe = cmul(f, cconj(e[i]));
        G[i] = cd(c * fe.x, c * fe.y);
      }
      for (int a = 0; a < m; ++a)   // X = U^H G
        for (int b2 = 0; b2 < m; ++b2) {
          double2 acc = czero();
          for (int k = 0; k < m; ++k) acc = cadd(acc, cmul(cconj(u[k * m + a]), G[k * m + b2]));
          X[a * m + b2] = acc;
        }
      for (int a = 0; a < m; ++a)   // dY = U skew(X)
        for (int b2 = 0; b2 < m; ++b2) {
          double2 acc = czero();
          for (int k = 0; k < m; ++k) {
            const double2 xk = X[k * m + b2], xt = cconj(X[b2 * m + k]);
            acc = cadd(acc, cmul(u[a * m + k], cd(0.5 * (xk.x - xt.x), 0.5 * (xk.y - xt.y))));
          }
          out[2 * (a * m + b2)] = (float)acc.x;
          out[2 * (a * m + b2) + 1] = (float)acc.y;
        }
    } else {
      fid[s] = 0.f;
    }
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      dY[(int64_t)s * 32 + i] = out[i];
      dYb[(int64_t)s * 32 + i] = __float2bfloat16_rn(out[i]);
      dYT[(int64_t)i * ldt + s] = __float2bfloat16_rn(out[i]);
    }
  }
}

// dZ = dH * GELU'(Z) for [B x N]; BF16 copy and transposed BF16 copy [N x ldt]
__global__ void k_act_back(const float* dH, const float* Z, int B, int N, float* dZ, __nv_bfloat16* dZb,
                           __nv_bfloat16* dZT, int ldt) {
  const int64_t total = (int64_t)B * N;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int row = (int)(i / N), col = (int)(i % N);
    const float d = dH[i] * gelu_grad_f(Z[i]);
    dZ[i] = d;
    dZb[i] = __float2bfloat16_rn(d);
    dZT[(int64_t)col * ldt + row] = __float2bfloat16_rn(d);
  }
}

// out[c] = sum_r X[r][c] over r < B, one thread per column, fixed order
__global__ void k_col_sum(const float* X, int B, int N, float* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  float s = 0.f;
  for (int r = 0; r < B; ++r) s += X[(int64_t)r * N + c];
  out[c] = s;
}

// Adam on master weights W [rows x cols]; gradient G in the same layout, or
// transposed ([cols x rows]) when gT != 0.  Writes BF16 W and W^T.
__global__ void k_adam(float* W, const float* G, int gT, float* m, float* v, int rows, int cols, float lr, float b1,
                       float b2, float eps, float bc1, float bc2, float wd, __nv_bfloat16* Wb, __nv_bfloat16* WTb) {
  const int64_t total = (int64_t)rows * cols;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i % cols);
    const float gr = gT ? G[(int64_t)c * rows + r] : G[i];
    const float mm = b1 * m[i] + (1.f - b1) * gr;
    const float vv = b2 * v[i] + (1.f - b2) * gr * gr;
    m[i] = mm;
    v[i] = vv;
    float w = W[i];
    w -= lr * ((mm / bc1) / (sqrtf(vv / bc2) + eps) + wd * w);
    W[i] = w;
    if (Wb) Wb[i] = __float2bfloat16_rn(w);
    if (WTb) WTb[(int64_t)c * rows + r] = __float2bfloat16_rn(w);
  }
}

__global__ void k_adam_vec(float* W, const float* G, float* m, float* v, int n, float lr, float b1, float b2,
                           float eps, float bc1, float bc2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gr = G[i];
    const float mm = b1 * m[i] + (1.f - b1) * gr;
    const float vv = b2 * v[i] + (1.f - b2) * gr * gr;
    m[i] = mm;
    v[i] = vv;
    W[i] -= lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
  }
}

// Row r of Y (4 x 4 complex, interleaved fp32) -> unitary polar factor
// written to gate slot slots[r]; singular directions below the null
// threshold are completed towards the gate already in the slot.
__global__ void k_mlp_project(const float* Y, int rows, const int64_t* slots, const signed char* kind,
                              double2* gates) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
    const int m = kind[r] == 1 ? 2 : 4;
    double2 e[16], w[16], prev[16];
    bool finite = true;
    for (int i = 0; i < m * m; ++i) {
      e[i] = cd((double)Y[(int64_t)r * 32 + 2 * i], (double)Y[(int64_t)r * 32 + 2 * i + 1]);
      finite = finite && isfinite(e[i].x) && isfinite(e[i].y);
    }
    double2* g = gates + slots[r] * 16;
    if (!finite) continue;   // keep the analytic gate
    for (int i = 0; i < m * m; ++i) prev[i] = g[i];
    polar_sweep(e, m, w, prev);
    for (int i = 0; i < m * m; ++i) g[i] = w[i];
  }
}

// ---- C ABI -----------------------------------------------------------------------

namespace {

int g_attr_done = 0;

int grid1(int64_t total, int threads) {
  int64_t b = (total + threads - 1) / threads;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace

extern "C" {

int qmprs_gemm_bf16(const void* A, int lda, const void* B, int ldb, int M, int N, int K, int ksplit,
                    const float* bias, const float* resid, int ldr, int act, float* Cf, int ldc, void* Cb, void* CbT,
                    int ldt, float* part, int* err, void* stream) {
  if (!A || !B || !err) return QMPRS_ERR_INVALID;
  if (M <= 0 || M % MLP_BM != 0 || N < 16 || N > MLP_MAXN || N % 16 != 0 || K <= 0 || K % 16 != 0)
    return QMPRS_ERR_INVALID;
  if (lda % 8 != 0 || ldb % 8 != 0) return QMPRS_ERR_INVALID;   // 16-byte rows for cp.async
  if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) return QMPRS_ERR_INVALID;
  if (ksplit <= 0 || ksplit >= K) ksplit = K;
  if (ksplit % 16 != 0) return QMPRS_ERR_INVALID;
  const int S = (K + ksplit - 1) / ksplit;
  if (S > 1 && !part) return QMPRS_ERR_INVALID;
  if (!g_attr_done) {
    cudaError_t e = cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, MLP_SMEM_REQ);
    if (e != cudaSuccess) return QMPRS_ERR_CUDA;
    g_attr_done = 1;
  }
  cudaStream_t s = (cudaStream_t)stream;
  GemmArgs g;
  g.A = (const __nv_bfloat16*)A;
  g.lda = lda;
  g.B = (const __nv_bfloat16*)B;
  g.ldb = ldb;
  g.M = M;
  g.N = N;
  g.K = K;
  g.ksplit = ksplit;
  g.bias = bias;
  g.act = act;
  g.Cf = Cf;
  g.ldc = ldc;
  g.Cb = (__nv_bfloat16*)Cb;
  g.CbT = (__nv_bfloat16*)CbT;
  g.ldt = ldt;
  g.part = part;
  g.resid = resid;
  g.ldr = ldr;
  g.err = err;
  dim3 grid(M / MLP_BM, 1, S);
  qm_note_launch();
  k_gemm_tc<<<grid, MLP_THREADS, MLP_SMEM_REQ, s>>>(g);
  if (S > 1) {
    qm_note_launch();
    k_splitk_sum<<<grid1((int64_t)M * N, 256), 256, 0, s>>>(part, S, M, N, bias, resid, ldr, act, Cf, ldc,
                                                             (__nv_bfloat16*)Cb, (__nv_bfloat16*)CbT, ldt);
  }
  return cudaGetLastError() == cudaSuccess ? QMPRS_OK : QMPRS_ERR_CUDA;
}

int qmprs_mlp_loss(const float* Y, const float* U, const float* w, int B, float inv_wsum, float* loss, float* dY,
                   void* dYb, void* dYT, int ldt, void* stream) {
  if (!Y || !U || !w || !loss || !dY || !dYb || !dYT || B <= 0) return QMPRS_ERR_INVALID;
  qm_note_launch();
  k_mlp_loss<<<grid1(B, 128), 128, 0, (cudaStream_t)stream>>>(Y, U, w, B, inv_wsum, loss, dY, (__nv_bfloat16*)dYb,
                                                               (__nv_bfloat16*)dYT, ldt);
  return cudaGetLastError() == cudaSuccess ? QMPRS_OK : QMPRS_ERR_CUDA;
}

int qmprs_mlp_act_back(const float* dH, const float* Z, int B, int N, float* dZ, void* dZb, void* dZT, int ldt,
                       void* stream) {
  if (!dH || !Z || !dZ || !dZb || !dZT || B <= 0 || N <= 0) return QMPRS_ERR_INVALID;
  qm_note_launch();
  k_act_back<<<grid1((int64_t)B * N, 256), 256, 0, (cudaStream_t)stream>>>(dH, Z, B, N, dZ, (__nv_bfloat16*)dZb,
                                                                          (__nv_bfloat16*)dZT, ldt);
  return cudaGetLastError() == cudaSuccess ? QMPRS_OK : QMPRS_ERR_CUDA;
}

int qmprs_mlp_col_sum(const float* X, int B, int N, float* out, void* stream) {
  if (!X || !out || B <= 0 || N <= 0) return QMPRS_ERR_INVALID;
  qm_note_launch();
  k_col_sum<<<(N + 127) / 128, 128, 0, (cudaStream_t)stream>>>(X, B, N, out);
  return cudaGetLastError() == cudaSuccess ? QMPRS_OK : QMPRS_ERR_CUDA;
}

int qmprs_mlp_adam(float* W, const float* G, int gT, float* m, float* v, int rows, int cols, float lr, float b1,
                   float b2, float eps, int step, float wd, void* Wb, void* WTb, void* stream) {
  if (!W || !G || !m || !v || rows <= 0 || cols <= 0 || step < 1) return QMPRS_ERR_INVALID;
  const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
  qm_note_launch();
  if (cols == 1 && !Wb && !WTb) {
    k_adam_vec<<<grid1(rows, 256), 256, 0, (cudaStream_t)stream>>>(W, G, m, v, rows, lr, b1, b2, eps, bc1, bc2);
  } else {
    k_adam<<<grid1((int64_t)rows * cols, 256), 256, 0, (cudaStream_t)stream>>>(
        W, G, gT, m, v, rows, cols, lr, b1, b2, eps, bc1, bc2, wd, (__nv_bfloat16*)Wb, (__nv_bfloat16*)WTb);
  }
  return cudaGetLastError() == cudaSuccess ? QMPRS_OK : QMPRS_ERR_CUDA;
}

int qmprs_tc_wait_selftest(int* err, void* stream) {
  if (!err) return QMPRS_ERR_INVALID;
  qm_note_launch();
  k_tc_wait_selftest<<<1, MLP_THREADS, 0, (cudaStream_t)stream>>>(err);
  return cudaGetLastError() == cudaSuccess ? QMPRS_OK : QMPRS_ERR_CUDA;
}

int qmprs_mlp_overlap_grad(const void* env, const void* gates, const int64_t* slots, const int8_t* kind,
                           const float* tinv, int rows, int B, float gscale, float* fid, float* dY, void* dYb,
                           void* dYT, int ldt, void* stream) {
  if (!env || !gates || !slots || !kind || !tinv || !fid || !dY || !dYb || !dYT || rows < 0 || B < rows ||
      B <= 0 || ldt < B)
    return QMPRS_ERR_INVALID;
  qm_note_launch();
  k_mlp_overlap_grad<<<grid1(B, 128), 128, 0, (cudaStream_t)stream>>>(
      (const double2*)env, (const double2*)gates, slots, (const signed char*)kind, tinv, rows, B, gscale, fid, dY,
      (__nv_bfloat16*)dYb, (__nv_bfloat16*)dYT, ldt);
  return cudaGetLastError() == cudaSuccess ? QMPRS_OK : QMPRS_ERR_CUDA;
}

int qmprs_mlp_project(const float* Y, int rows, const int64_t* slots, const int8_t* kind, void* gates,
                      void* stream) {
  if (!Y || !slots || !kind || !gates || rows < 0) return QMPRS_ERR_INVALID;
  if (rows == 0) return QMPRS_OK;
  qm_note_launch();
  k_mlp_project<<<grid1(rows, 64), 64, 0, (cudaStream_t)stream>>>(Y, rows, slots, (const signed char*)kind,
                                                                   (double2*)gates);
  return cudaGetLastError() == cudaSuccess ? QMPRS_OK : QMPRS_ERR_CUDA;
}

}  // extern "C"
