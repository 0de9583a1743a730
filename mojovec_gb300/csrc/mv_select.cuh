// Deterministic k-selection for the search kernels.
//
// A candidate is packed into one 64-bit key: the high word is the distance
// mapped to an order-preserving unsigned integer (with -0.0 folded onto
// +0.0, since the reference compares floats with `<`), the low word is the
// 32-bit id. The k smallest keys are the canonical result "distance
// ascending, ties broken by the smaller id". The selected set does not
// depend on the order in which candidates arrive, so the result is the same
// for any launch shape, batch composition or split of a list.
//
// The reference keeps its top-k in a binary max-heap with a strict `<`
// replace test (utils/heap.mojo:17-213); for distinct keys that heap returns
// the same set as this selection, and the canonical order fixes the order of
// equal distances, which the heap leaves to its pop sequence.
#pragma once

#include <cstdint>

namespace mv {

constexpr uint64_t KEY_NONE = ~0ull;

__device__ __forceinline__ uint32_t float_to_ordered(float f) {
  if (f == 0.0f) f = 0.0f;  // -0.0 == +0.0 under `<`
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float ordered_to_float(uint32_t o) {
  uint32_t u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
  return __uint_as_float(u);
}

__device__ __forceinline__ uint64_t make_key(float dist, uint32_t id) {
  return ((uint64_t)float_to_ordered(dist) << 32) | id;
}

__device__ __forceinline__ float key_dist(uint64_t key) { return ordered_to_float((uint32_t)(key >> 32)); }
__device__ __forceinline__ uint32_t key_id(uint64_t key) { return (uint32_t)key; }

// In-place ascending bitonic sort of n (a power of two) keys in shared
// memory by the whole block.
__device__ __forceinline__ void block_bitonic_sort(uint64_t* a, int n) {
  for (int size = 2; size <= n; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      __syncthreads();
      for (int t = threadIdx.x; t < (n >> 1); t += blockDim.x) {
        int lo = 2 * t - (t & (stride - 1));
        int hi = lo + stride;
        bool up = ((lo & size) == 0);
        uint64_t x = a[lo], y = a[hi];
        if ((x > y) == up) {
          a[lo] = y;
          a[hi] = x;
        }
      }
    }
  }
  __syncthreads();
}

__host__ __device__ __forceinline__ int next_pow2(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

// Block-wide top-k over a stream of candidate rounds. Shared memory layout:
// keys[0, P) where P = next_pow2(k + bufcap); keys[0, k) hold the current
// best (sorted after each flush), keys[k, k + count) the pending buffer.
//
// Protocol per round: every thread calls push() with at most one key, then
// the whole block calls end_round(). finish() leaves keys[0, k) sorted.
// The flush decision uses a per-thread copy of the pending count that is
// advanced by __syncthreads_count, so it is the same in every thread: a
// thread that has already started the next round cannot change another
// thread's decision through the shared counter.
struct BlockTopK {
  uint64_t* keys;
  int* count;          // shared slot allocator
  uint64_t* thresh;    // shared: k-th best so far (KEY_NONE until k found)
  int k, bufcap, P;
  int pending;         // keys in the buffer (uniform across the block)
  bool pushed;         // this thread pushed in the current round

  static __host__ __device__ int smem_keys(int k, int bufcap) { return next_pow2(k + bufcap); }

  __device__ void init(uint64_t* keys_, int* count_, uint64_t* thresh_, int k_, int bufcap_) {
    keys = keys_;
    count = count_;
    thresh = thresh_;
    k = k_;
    bufcap = bufcap_;
    P = next_pow2(k + bufcap);
    pending = 0;
    pushed = false;
    for (int i = threadIdx.x; i < P; i += blockDim.x) keys[i] = KEY_NONE;
    if (threadIdx.x == 0) {
      *count = 0;
      *thresh = KEY_NONE;
    }
    __syncthreads();
  }

  // Seeds the current best with a sorted list of k keys (KEY_NONE padded).
  __device__ void seed(const uint64_t* sorted_k) {
    for (int i = threadIdx.x; i < k; i += blockDim.x) keys[i] = sorted_k[i];
    __syncthreads();
    if (threadIdx.x == 0) *thresh = keys[k - 1];
    __syncthreads();
  }

  __device__ __forceinline__ void push(uint64_t key) {
    if (key < *thresh) {
      int pos = atomicAdd(count, 1);
      keys[k + pos] = key;
      pushed = true;
    }
  }

  __device__ void flush() {
    block_bitonic_sort(keys, P);
    for (int i = k + threadIdx.x; i < P; i += blockDim.x) keys[i] = KEY_NONE;
    if (threadIdx.x == 0) {
      *count = 0;
      *thresh = keys[k - 1];
    }
    pending = 0;
    __syncthreads();
  }

  // Call after every round; guarantees room for one key per thread next round.
  __device__ void end_round() {
    pending += __syncthreads_count(pushed ? 1 : 0);
    pushed = false;
    if (pending > bufcap - (int)blockDim.x) flush();
  }

  __device__ void finish() {
    pending += __syncthreads_count(pushed ? 1 : 0);
    pushed = false;
    if (pending > 0) flush();
  }
};

}  // namespace mv
