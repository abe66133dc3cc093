// Batched overlaps <a|b> that allocate nothing.
//
// Some callers of this library cannot call cudaMalloc: their device memory is
// owned by another allocator (a framework's caching allocator that has
// already reserved the GPU), or they run on a latency-critical stream where
// the implicit device synchronisation of cudaMalloc/cudaFree is not
// acceptable.  qmprs_overlap_noalloc serves them: it takes the caller's
// statevectors and output buffer, passes the per-state layout to the kernels
// by value, and keeps its reduction scratch in the file-scope device array
// below, which every GPU that loads this library holds until the process
// exits (1 MiB).
//
// The array is shared by every call and keeps the last call's contents.
// Every slot a call reads is written by the same call first, so nothing has
// to be cleared; calls that overlap on the GPU (concurrent streams) race on
// it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <mutex>

#include "device_common.cuh"
#include "qmprs_gb300.h"

#define NOALLOC_TILE_BITS 12
#define NOALLOC_PARTIALS (QMPRS_NOALLOC_MAX_TILES * WARPS_PER_BLOCK)

static __device__ __align__(256) double2 g_noalloc_partials[NOALLOC_PARTIALS];

struct NoallocLayout {
  int num_states;
  int ntiles;
  int n[QMPRS_NOALLOC_MAX_STATES];
  int tile0[QMPRS_NOALLOC_MAX_STATES];
  long long off[QMPRS_NOALLOC_MAX_STATES];
};

__device__ __forceinline__ int noalloc_state_of(const NoallocLayout& L, int tile) {
  int b = 0;
  while (b + 1 < L.num_states && L.tile0[b + 1] <= tile) ++b;
  return b;
}

__global__ void __launch_bounds__(BLOCK_THREADS) k_noalloc_overlap(NoallocLayout L, const float2* a,
                                                                   const float2* bv, double2* scratch) {
  for (int tile = blockIdx.x; tile < L.ntiles; tile += gridDim.x) {
    const int b = noalloc_state_of(L, tile);
    const int n = L.n[b];
    const int nt = n > NOALLOC_TILE_BITS ? (1 << (n - NOALLOC_TILE_BITS)) : 1;
    int64_t lo, hi;
    tile_range(ipow2(n), tile - L.tile0[b], nt, &lo, &hi);
    const float2* pa = a + L.off[b];
    const float2* pb = bv + L.off[b];
    double re = 0.0, im = 0.0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const double2 x = f2d(pa[i]), y = f2d(pb[i]);
      re += x.x * y.x + x.y * y.y;
      im += x.x * y.y - x.y * y.x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if ((threadIdx.x & 31) == 0) scratch[(int64_t)tile * WARPS_PER_BLOCK + (threadIdx.x >> 5)] = cd(re, im);
  }
}

// One warp per state: the state's warp partials in a fixed order.
__global__ void k_noalloc_reduce(NoallocLayout L, const double2* scratch, double2* out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int b = warp; b < L.num_states; b += nwarps) {
    const int n = L.n[b];
    const int nt = n > NOALLOC_TILE_BITS ? (1 << (n - NOALLOC_TILE_BITS)) : 1;
    const int64_t p0 = (int64_t)L.tile0[b] * WARPS_PER_BLOCK;
    const int np = nt * WARPS_PER_BLOCK;
    double2 s = czero();
    for (int t = lane; t < np; t += 32) s = cadd(s, scratch[p0 + t]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s.x += __shfl_down_sync(0xffffffffu, s.x, o);
      s.y += __shfl_down_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) out[b] = s;
  }
}

// Device address of the scratch array, looked up once per device with that
// device current (the array's host-side name is not a device address).
// Threads that call at the same time on a fresh device serialise on the
// lookup; the published address is read with acquire ordering.
static std::atomic<double2*> g_noalloc_ptr[64];
static std::mutex g_noalloc_mu;

extern "C" int qmprs_overlap_noalloc(const void* a, const void* b, int num_states, const int* num_qubits,
                                     void* out, void* stream) {
  if (!a || !b || !out || !num_qubits || num_states < 1) return QMPRS_ERR_INVALID;
  if (num_states > QMPRS_NOALLOC_MAX_STATES) return QMPRS_ERR_UNSUPPORTED;
  NoallocLayout L;
  std::memset(&L, 0, sizeof(L));
  L.num_states = num_states;
  long long off = 0;
  int tiles = 0;
  for (int i = 0; i < num_states; ++i) {
    const int n = num_qubits[i];
    if (n < 1 || n > 30) return QMPRS_ERR_INVALID;
    L.n[i] = n;
    L.off[i] = off;
    L.tile0[i] = tiles;
    off += 1LL << n;
    tiles += n > NOALLOC_TILE_BITS ? (1 << (n - NOALLOC_TILE_BITS)) : 1;
    if (tiles > QMPRS_NOALLOC_MAX_TILES) return QMPRS_ERR_UNSUPPORTED;
  }
  L.ntiles = tiles;
  // An error left pending by earlier work on this thread belongs to its
  // caller: refuse to launch and leave it in place rather than report it
  // as ours (or clear it).
  if (cudaPeekAtLastError() != cudaSuccess) return QMPRS_ERR_CUDA;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return QMPRS_ERR_CUDA;
  double2* scratch = g_noalloc_ptr[dev].load(std::memory_order_acquire);
  if (!scratch) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    scratch = g_noalloc_ptr[dev].load(std::memory_order_relaxed);
    if (!scratch) {
      if (cudaGetSymbolAddress((void**)&scratch, g_noalloc_partials) != cudaSuccess || scratch == nullptr)
        return QMPRS_ERR_CUDA;
      g_noalloc_ptr[dev].store(scratch, std::memory_order_release);
    }
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int grid = tiles < 152 * 8 ? tiles : 152 * 8;
  qm_note_launch();
  k_noalloc_overlap<<<grid, BLOCK_THREADS, 0, s>>>(L, (const float2*)a, (const float2*)b, scratch);
  if (cudaGetLastError() != cudaSuccess) return QMPRS_ERR_CUDA;   // the reduce is not queued
  qm_note_launch();
  k_noalloc_reduce<<<(num_states + 7) / 8, 256, 0, s>>>(L, scratch, (double2*)out);
  return cudaGetLastError() == cudaSuccess ? QMPRS_OK : QMPRS_ERR_CUDA;
}
