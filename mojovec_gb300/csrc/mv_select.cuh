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

// ---------------------------------------------------------------------------
// Block radix select: the R smallest of n distinct 64-bit keys held in
// shared memory, in O(passes * n) shared-memory accesses instead of the
// O(n log^2 n) of a sort.
//
// The keys between the block's min and max share their high bits; digits of
// 11 bits are taken from the first bit where min and max differ. Each pass
// histograms the digit of the keys still matching the chosen prefix, finds
// the bucket holding the R-th key and extends the prefix; it stops as soon as
// that bucket is taken whole. The result (all keys <= the final bound) is
// exactly the R smallest; it is written unsorted to out[0, R) and does not
// depend on the order of the input.
// ---------------------------------------------------------------------------
struct RadixScratch {
  uint32_t hist[2048];
  uint32_t wsum[32];
  unsigned long long lo, hi;
  uint32_t bucket, before;
  int out_n;
};

// Returns min(n, R). All threads of the block must call it with the same
// arguments. keys[0, n) are not modified; out must not alias keys. Keys are
// expected to be distinct; equal keys at the boundary are cut at R.
template <int NT>
__device__ int block_radix_select(const uint64_t* keys, int n, int R, uint64_t* out,
                                  RadixScratch& s) {
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  constexpr int NW = NT / 32;
  if (n <= R) {
    for (int i = tid; i < n; i += NT) out[i] = keys[i];
    __syncthreads();
    return n;
  }
  // min / max of the keys
  unsigned long long lo = ~0ull, hi = 0ull;
  for (int i = tid; i < n; i += NT) {
    const unsigned long long v = keys[i];
    lo = v < lo ? v : lo;
    hi = v > hi ? v : hi;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long a = __shfl_xor_sync(0xffffffffu, lo, o);
    const unsigned long long b = __shfl_xor_sync(0xffffffffu, hi, o);
    lo = a < lo ? a : lo;
    hi = b > hi ? b : hi;
  }
  if (tid == 0) {
    s.lo = ~0ull;
    s.hi = 0ull;
    s.out_n = 0;
  }
  __syncthreads();
  if (lane == 0) {
    atomicMin(&s.lo, lo);
    atomicMax(&s.hi, hi);
  }
  __syncthreads();
  lo = s.lo;
  hi = s.hi;
  // shift = number of low bits still undetermined
  int shift = 64 - __clzll((long long)(lo ^ hi));
  unsigned long long prefix = shift >= 64 ? 0ull : (lo >> shift) << shift;
  int need = R;
  while (shift > 0) {
    const int bits = shift < 11 ? shift : 11;
    const int nb = 1 << bits;
    shift -= bits;
    const int top = shift + bits;  // bits at or above `top` must match the prefix
    for (int b = tid; b < nb; b += NT) s.hist[b] = 0;
    __syncthreads();
    for (int i = tid; i < n; i += NT) {
      const unsigned long long v = keys[i];
      const bool match = top >= 64 || ((v >> top) == (prefix >> top));
      if (match) atomicAdd(&s.hist[(uint32_t)(v >> shift) & (uint32_t)(nb - 1)], 1u);
    }
    __syncthreads();
    // exclusive scan over nb bins: each thread owns a contiguous run
    const int per = (nb + NT - 1) / NT;
    const int b0 = tid * per;
    uint32_t local = 0;
    for (int b = b0; b < b0 + per && b < nb; ++b) local += s.hist[b];
    uint32_t incl = local;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) s.wsum[warp] = incl;
    __syncthreads();
    uint32_t wbase = 0;
    for (int w = 0; w < warp; ++w) wbase += s.wsum[w];
    uint32_t run = wbase + incl - local;  // bins before b0
    for (int b = b0; b < b0 + per && b < nb; ++b) {
      const uint32_t h = s.hist[b];
      if (run < (uint32_t)need && (uint32_t)need <= run + h) {
        s.bucket = (uint32_t)b;
        s.before = run;
      }
      run += h;
    }
    __syncthreads();
    const uint32_t b = s.bucket;
    need -= (int)s.before;
    prefix |= (unsigned long long)b << shift;
    const bool whole = s.hist[b] == (uint32_t)need;
    __syncthreads();
    if (whole) break;
  }
  // keys <= bound are exactly the R smallest
  const unsigned long long bound = shift >= 64 ? ~0ull : (prefix | ((1ull << shift) - 1ull));
  for (int i0 = 0; i0 < n; i0 += NT) {
    const int i = i0 + tid;
    const bool take = i < n && keys[i] <= bound;
    const unsigned mask = __ballot_sync(0xffffffffu, take);
    int base = 0;
    if (lane == 0 && mask) base = atomicAdd(&s.out_n, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, 0);
    const int slot = base + __popc(mask & ((1u << lane) - 1u));
    if (take && slot < R) out[slot] = keys[i];  // equal keys (duplicate ids) never overflow
  }
  __syncthreads();
  return R;
}

// Same selection over keys stored as two word arrays, key = (hi << 32) | lo
// (hi: ordered distance, lo: payload), with 8-bit digits: 256-bin passes are
// cheaper to clear and scan than 2048-bin ones, and measured faster for the
// fast IVF-PQ shortlist (256 of about 2 000 keys). Histogram passes whose digit lies in
// the high word read 4 bytes per key; the low word is read only when
// distances tie down to the last bit. Histogram updates are aggregated per
// warp (one atomic per distinct digit).
template <int NT>
__device__ int block_radix_select_soa(const uint32_t* khi, const uint32_t* klo, int n, int R,
                                      uint64_t* out, RadixScratch& s) {
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  auto key_at = [&](int i) -> unsigned long long {
    return ((unsigned long long)khi[i] << 32) | klo[i];
  };
  if (n <= R) {
    for (int i = tid; i < n; i += NT) out[i] = key_at(i);
    __syncthreads();
    return n;
  }
  unsigned long long lo = ~0ull, hi = 0ull;
  for (int i = tid; i < n; i += NT) {
    const unsigned long long v = key_at(i);
    lo = v < lo ? v : lo;
    hi = v > hi ? v : hi;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long a = __shfl_xor_sync(0xffffffffu, lo, o);
    const unsigned long long b = __shfl_xor_sync(0xffffffffu, hi, o);
    lo = a < lo ? a : lo;
    hi = b > hi ? b : hi;
  }
  if (tid == 0) {
    s.lo = ~0ull;
    s.hi = 0ull;
    s.out_n = 0;
  }
  __syncthreads();
  if (lane == 0) {
    atomicMin(&s.lo, lo);
    atomicMax(&s.hi, hi);
  }
  __syncthreads();
  lo = s.lo;
  hi = s.hi;
  int shift = 64 - __clzll((long long)(lo ^ hi));
  unsigned long long prefix = shift >= 64 ? 0ull : (lo >> shift) << shift;
  int need = R;
  while (shift > 0) {
    const int bits = shift < 8 ? shift : 8;
    const int nb = 1 << bits;
    shift -= bits;
    const int top = shift + bits;
    for (int b = tid; b < nb; b += NT) s.hist[b] = 0;
    __syncthreads();
    const bool hi_only = shift >= 32;
    for (int i0 = 0; i0 < n; i0 += NT) {
      const int i = i0 + tid;
      bool match = false;
      uint32_t digit = 0;
      if (i < n) {
        const unsigned long long v = hi_only ? ((unsigned long long)khi[i] << 32) : key_at(i);
        match = top >= 64 || ((v >> top) == (prefix >> top));
        digit = (uint32_t)(v >> shift) & (uint32_t)(nb - 1);
      }
      const unsigned act = __ballot_sync(0xffffffffu, match);
      if (match) {
        const unsigned peers = __match_any_sync(act, digit);
        if (lane == __ffs(peers) - 1) atomicAdd(&s.hist[digit], (uint32_t)__popc(peers));
      }
    }
    __syncthreads();
    const int per = (nb + NT - 1) / NT;
    const int b0 = tid * per;
    uint32_t local = 0;
    for (int b = b0; b < b0 + per && b < nb; ++b) local += s.hist[b];
    uint32_t incl = local;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) s.wsum[warp] = incl;
    __syncthreads();
    uint32_t wbase = 0;
    for (int w = 0; w < warp; ++w) wbase += s.wsum[w];
    uint32_t run = wbase + incl - local;
    for (int b = b0; b < b0 + per && b < nb; ++b) {
      const uint32_t h = s.hist[b];
      if (run < (uint32_t)need && (uint32_t)need <= run + h) {
        s.bucket = (uint32_t)b;
        s.before = run;
      }
      run += h;
    }
    __syncthreads();
    const uint32_t b = s.bucket;
    need -= (int)s.before;
    prefix |= (unsigned long long)b << shift;
    const bool whole = s.hist[b] == (uint32_t)need;
    __syncthreads();
    if (whole) break;
  }
  const unsigned long long bound = shift >= 64 ? ~0ull : (prefix | ((1ull << shift) - 1ull));
  for (int i0 = 0; i0 < n; i0 += NT) {
    const int i = i0 + tid;
    const unsigned long long v = i < n ? key_at(i) : ~0ull;
    const bool take = i < n && v <= bound;
    const unsigned mask = __ballot_sync(0xffffffffu, take);
    int base = 0;
    if (lane == 0 && mask) base = atomicAdd(&s.out_n, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, 0);
    const int slot = base + __popc(mask & ((1u << lane) - 1u));
    if (take && slot < R) out[slot] = v;
  }
  __syncthreads();
  return R;
}

// Ascending bitonic sort of the warp's 32 * RR keys held in registers,
// element r * 32 + lane in v[r] of that lane: cross-lane steps by xor
// shuffles, in-lane steps between registers (all indices static).
template <int RR>
__device__ __forceinline__ void warp_sort_regs(uint64_t (&v)[RR]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 2; k <= 32 * RR; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
        const int jr = j >> 5;
#pragma unroll
        for (int r = 0; r < RR; ++r) {
          if (r & jr) continue;
          const int r2 = r | jr;
          const bool up = (((r << 5) | lane) & k) == 0;
          const uint64_t a = v[r], b = v[r2];
          const bool sw = (a > b) == up;
          v[r] = sw ? b : a;
          v[r2] = sw ? a : b;
        }
      } else {
        const bool low = (lane & j) == 0;
#pragma unroll
        for (int r = 0; r < RR; ++r) {
          const bool up = (((r << 5) | lane) & k) == 0;
          const uint64_t a = v[r];
          const uint64_t b = __shfl_xor_sync(0xffffffffu, a, j);
          const bool keep_min = low == up;
          v[r] = keep_min ? (a < b ? a : b) : (a < b ? b : a);
        }
      }
    }
  }
}

// Sorts a bitonic sequence of 32 keys (one per lane) ascending.
__device__ __forceinline__ uint64_t warp_bitonic_merge32(uint64_t a) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 16; j > 0; j >>= 1) {
    const uint64_t b = __shfl_xor_sync(0xffffffffu, a, j);
    const bool low = (lane & j) == 0;
    a = low ? (a < b ? a : b) : (a < b ? b : a);
  }
  return a;
}

// The k-th smallest (1 <= k <= 64) of the warp's 64 values v0, v1 (value
// r * 32 + lane in v_r): bitonic sort of the 64, then position k - 1.
__device__ __forceinline__ uint32_t warp_kth_smallest64(uint32_t v0, uint32_t v1, int k) {
  const int lane = threadIdx.x & 31;
  uint32_t v[2] = {v0, v1};
#pragma unroll
  for (int size = 2; size <= 64; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      if (stride == 32) {  // size 64, ascending: the pair is (v0, v1) of one lane
        const uint32_t lo = min(v[0], v[1]), hi = max(v[0], v[1]);
        v[0] = lo;
        v[1] = hi;
      } else {
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          const int e = r * 32 + lane;
          const uint32_t o = __shfl_xor_sync(0xffffffffu, v[r], stride);
          const bool asc = (e & size) == 0, lower = (e & stride) == 0;
          v[r] = lower == asc ? min(v[r], o) : max(v[r], o);
        }
      }
    }
  }
  const int pos = k - 1;
  return __shfl_sync(0xffffffffu, pos < 32 ? v[0] : v[1], pos & 31);
}

// best (ascending across lanes) <- the 32 smallest of best and v (any order).
__device__ __forceinline__ uint64_t warp_merge_smallest32(uint64_t best, uint64_t v) {
  const int lane = threadIdx.x & 31;
  uint64_t t[1] = {v};
  warp_sort_regs<1>(t);
  const uint64_t r = __shfl_sync(0xffffffffu, t[0], 31 - lane);
  return warp_bitonic_merge32(best < r ? best : r);
}

// Ascending sort of the warp's 32 * RR keys, element r * 32 + lane in v[r].
template <int RR>
__device__ __forceinline__ void sort_side(const uint64_t* side, int h, int need, uint64_t* out,
                                          unsigned long long* kth) {
  const int lane = threadIdx.x & 31;
  uint64_t v[RR];
#pragma unroll
  for (int r = 0; r < RR; ++r) {
    const int e = r * 32 + lane;
    v[r] = e < h ? side[e] : ~0ull;
  }
  warp_sort_regs<RR>(v);
#pragma unroll
  for (int r = 0; r < RR; ++r) {
    const int e = r * 32 + lane;
    if (e < need) out[e] = v[r];
    if (e == need - 1) *kth = v[r];
  }
}

// The R smallest of the n keys (khi[i] << 32 | klo[i]) into out[0, r),
// unsorted, r = min(n, R); when n > R, *kth (shared memory) holds the R-th
// smallest. One histogram pass: the range of the keys' high words is cut
// into at most 2048 bins, the bin holding the R-th key is found by a prefix
// scan, every key of a lower bin is taken and the boundary bin's keys are
// sorted by one warp; the radix select takes over when that bin holds more
// than 256 keys (many equal distances). All threads call it; khi / klo are
// not modified; out must not alias them.
template <int NT>
__device__ int block_hist_select(const uint32_t* khi, const uint32_t* klo, int n, int R,
                                 uint64_t* out, RadixScratch& rs, unsigned long long* kth) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (n <= R) {
    for (int i = tid; i < n; i += NT) out[i] = ((uint64_t)khi[i] << 32) | klo[i];
    __syncthreads();
    return n;
  }
  uint32_t lo = 0xffffffffu, hi = 0u;
  for (int i = tid; i < n; i += NT) {
    const uint32_t v = khi[i];
    lo = min(lo, v);
    hi = max(hi, v);
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  if (tid == 0) {
    rs.lo = ~0ull;
    rs.hi = 0ull;
    rs.out_n = 0;
  }
  __syncthreads();
  if (lane == 0) {
    atomicMin(&rs.lo, (unsigned long long)lo);
    atomicMax(&rs.hi, (unsigned long long)hi);
  }
  __syncthreads();
  const uint32_t base = (uint32_t)rs.lo, span = (uint32_t)rs.hi - base;
  const int sh = span < 2048u ? 0 : (32 - __clz((int)span)) - 11;  // (span >> sh) < 2048
  const int nb = (int)(span >> sh) + 1;
  for (int b = tid; b < nb; b += NT) rs.hist[b] = 0;
  __syncthreads();
  for (int i = tid; i < n; i += NT) atomicAdd(&rs.hist[(khi[i] - base) >> sh], 1u);
  __syncthreads();
  // the bin holding the R-th key: per-thread runs of bins, block prefix sums
  const int per = (nb + NT - 1) / NT;
  const int b0 = tid * per;
  uint32_t local = 0;
  for (int b = b0; b < b0 + per && b < nb; ++b) local += rs.hist[b];
  uint32_t incl = local;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) rs.wsum[warp] = incl;
  __syncthreads();
  uint32_t wbase = 0;
  for (int w = 0; w < warp; ++w) wbase += rs.wsum[w];
  uint32_t run = wbase + incl - local;
  for (int b = b0; b < b0 + per && b < nb; ++b) {
    const uint32_t h = rs.hist[b];
    if (run < (uint32_t)R && (uint32_t)R <= run + h) {
      rs.bucket = (uint32_t)b;
      rs.before = run;
      rs.wsum[32 - 1] = h;  // read below, after the barrier (no warp reads wsum[31] again)
    }
    run += h;
  }
  __syncthreads();
  const uint32_t bk = rs.bucket, before = rs.before, h = rs.wsum[31];
  __syncthreads();  // every thread has the bin before the histogram is reused
  if (h > 256u) {
    // many keys share the boundary bin (equal distances): radix select
    const int r = block_radix_select_soa<NT>(khi, klo, n, R, out, rs);
    unsigned long long mx = 0ull;
    for (int i = tid; i < r; i += NT) mx = out[i] > mx ? out[i] : mx;
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_xor_sync(0xffffffffu, mx, o);
      mx = t > mx ? t : mx;
    }
    if (tid == 0) *kth = 0ull;
    __syncthreads();
    if (lane == 0) atomicMax(kth, mx);
    __syncthreads();
    return r;
  }
  uint64_t* side = reinterpret_cast<uint64_t*>(rs.hist);  // up to 256 keys of the boundary bin
  if (tid == 0) rs.wsum[0] = 0;
  __syncthreads();
  for (int i0 = 0; i0 < n; i0 += NT) {
    const int i = i0 + tid;
    uint64_t v = ~0ull;
    uint32_t bin = 0xffffffffu;
    if (i < n) {
      v = ((uint64_t)khi[i] << 32) | klo[i];
      bin = (khi[i] - base) >> sh;
    }
    const bool below = bin < bk, at = bin == bk;
    const unsigned mb = __ballot_sync(0xffffffffu, below);
    const unsigned ma = __ballot_sync(0xffffffffu, at);
    int ob = 0, oa = 0;
    if (lane == 0) {
      if (mb) ob = atomicAdd(&rs.out_n, __popc(mb));
      if (ma) oa = atomicAdd(&rs.wsum[0], (uint32_t)__popc(ma));
    }
    ob = __shfl_sync(0xffffffffu, ob, 0);
    oa = __shfl_sync(0xffffffffu, oa, 0);
    const unsigned lt = (1u << lane) - 1u;
    if (below) out[ob + __popc(mb & lt)] = v;
    if (at) side[oa + __popc(ma & lt)] = v;
  }
  __syncthreads();
  if (warp == 0) {
    const int need = R - (int)before;
    if (h <= 32u) sort_side<1>(side, (int)h, need, out + before, kth);
    else if (h <= 64u) sort_side<2>(side, (int)h, need, out + before, kth);
    else if (h <= 128u) sort_side<4>(side, (int)h, need, out + before, kth);
    else sort_side<8>(side, (int)h, need, out + before, kth);
  }
  __syncthreads();
  return R;
}

}  // namespace mv
