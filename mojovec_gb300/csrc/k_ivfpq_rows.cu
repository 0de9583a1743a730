// Fast-form IVF-PQ ADC scan in two kernels: per-candidate distance rows,
// then a per-query select (index/index_ivf_pq.mojo:295-347, the fast form's
// expansion of the distance; k_ivfpq_fast.cu states it).
//
// k_ivfpq_rows (one CTA per query) builds the query's FP32 table from the
// FP16 codebook exactly as the single-kernel scan does, walks the probed
// lists laid end to end and writes every candidate's distance as an
// order-preserving word into the query's row of a distance matrix (word i
// is candidate i; ROW_EXCLUDED marks a row the exclusion filter names,
// index_ivf_pq.mojo:328-334). There is no staging area or compaction; the
// row's last word gets a bound on the R-th smallest word (from each
// thread's two smallest), the select's starting bound.
// k_row_select_stream (one warp per query, shortlists up to 256) streams
// its row once from that bound, staging keys below a running bound and
// keeping the R smallest whenever its staging area could overflow; k_row_select_wide
// (longer shortlists) narrows the key range of the R-th key with 256-bin
// histogram passes. Keys are (distance word, CSR position), the same keys
// the single-kernel scan selects from, so both return the same shortlist.
#include <cuda_fp16.h>

#include <algorithm>

#include "mv_adc.cuh"
#include "mv_fast.h"
#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_select.cuh"

namespace mv {
namespace {

constexpr uint32_t ROW_EXCLUDED = 0xffffffffu;

template <int NT, int CPT>
__global__ void __launch_bounds__(NT, 1024 / NT)
    k_ivfpq_rows(FastScanArgs a, uint32_t* __restrict__ dist, int64_t smax) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int M = a.M, d = a.d, dsub = d / M;
  float* lut = reinterpret_cast<float*>(smraw);  // M x 256
  float* qv = lut + M * 256;                     // d
  int64_t* poff = reinterpret_cast<int64_t*>(smraw + (((size_t)(M * 256 + d) * 4 + 15) & ~size_t(15)));
  int* pbeg = reinterpret_cast<int*>(poff + a.nprobe);  // nprobe + 1 prefix sums
  float* pterm = reinterpret_cast<float*>(pbeg + a.nprobe + 1);
  const int tid = threadIdx.x, lane = tid & 31;
  const int64_t row = blockIdx.x;
  const int nprobe = a.nprobe_q ? min(max(a.nprobe_q[row], 1), a.nprobe) : a.nprobe;
  for (int j = tid; j < d; j += NT) qv[j] = a.q[row * d + j];
  if (tid < 32) {  // probe table: offsets, lengths -> prefix sums
    int carry = 0;
    for (int p0 = 0; p0 < nprobe; p0 += 32) {
      const int p = p0 + lane;
      int len = 0;
      if (p < nprobe) {
        int list = a.probes[row * a.nprobe + p];
        if (list >= a.nlist) {
          atomicExch(a.err, 108);
          list = -1;
        }
        int64_t off = 0;
        if (list >= 0) {
          off = a.list_off[list];
          len = (int)(a.list_off[list + 1] - off);
        }
        poff[p] = off;
        pterm[p] = a.term[row * a.nprobe + p];
      }
      int incl = len;
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      if (p < nprobe) pbeg[p] = carry + incl - len;
      carry += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) pbeg[nprobe] = carry;
  }
  __syncthreads();
  const float scale = a.metric == MV_METRIC_L2 ? -2.0f : -1.0f;
  if (a.pq16) build_lut16<NT>([&](int i, float v) { lut[i] = v; }, qv, a.pq16, M, dsub, scale * a.pq16_inv);
  else build_lut<NT>([&](int i, float v) { lut[i] = v; }, qv, a.pq, M, dsub, scale);
  __syncthreads();
  const int total = pbeg[nprobe];
  if (total > smax - 1) {  // never expected: smax - 1 bounds every query's candidates
    if (tid == 0) atomicExch(a.err, 106);
    return;
  }
  uint32_t* drow = dist + row * smax;
  uint32_t m1 = 0xffffffffu, m2 = 0xffffffffu;  // the thread's two smallest kept words
  // per-thread probe cursor (candidate indices only grow) with the probe's
  // end, CSR base (offset - first index) and term kept in registers, and
  // whether the probe's CSR range lies in the index (then so does every
  // candidate position of it)
  int p = 0, pend = pbeg[1];
  int64_t pbase = poff[0];  // pbeg[0] = 0
  float pt = pterm[0];
  bool pok = poff[0] >= 0 && poff[0] + pend <= a.ntotal;
  // CPT candidates per thread per step: every row's loads are issued before
  // any table walk.
  for (int j0 = 0; j0 < total; j0 += CPT * NT) {
    int64_t pos[CPT];
    float t[CPT];
    bool has[CPT], keep[CPT];
    bool bad = false;
#pragma unroll
    for (int u = 0; u < CPT; ++u) {
      const int c = j0 + tid + u * NT;
      has[u] = c < total;
      // Lanes without a candidate keep their cursor and use position 0 (a
      // valid entry: the index is not empty), so no load leaves the lists.
      if (has[u] && c >= pend) {  // c < pbeg[nprobe]: p stops below nprobe
        do {
          ++p;
        } while (pbeg[p + 1] <= c);
        pend = pbeg[p + 1];
        pbase = poff[p] - pbeg[p];
        pt = pterm[p];
        pok = poff[p] >= 0 && poff[p] + (pend - pbeg[p]) <= a.ntotal;
      }
      pos[u] = has[u] ? pbase + c : 0;
      t[u] = has[u] ? pt : 0.0f;
      keep[u] = has[u];
      bad = bad || (has[u] && !pok);
    }
    if (bad) {
      atomicExch(a.err, 109);  // never expected: skip the step, stay warp-uniform
#pragma unroll
      for (int u = 0; u < CPT; ++u) {
        pos[u] = 0;
        keep[u] = false;
      }
    }
    if (a.filter) {  // filtered ids never enter the shortlist
#pragma unroll
      for (int u = 0; u < CPT; ++u) {
        const uint32_t id = a.ids[pos[u]];
        if ((int64_t)id < a.filter_len && a.filter[id] != 0) keep[u] = false;
      }
    }
    float v[CPT];
#pragma unroll
    for (int u = 0; u < CPT; ++u) v[u] = a.vterm ? a.vterm[pos[u]] : 0.0f;
#pragma unroll
    for (int u = 0; u < CPT; ++u) {
      const float dd = adc_fast(lut, a.codes + pos[u] * M, M, t[u] + v[u]);
      // ROW_EXCLUDED marks no key: a NaN distance keeps the word below it
      const uint32_t wd = keep[u] ? min(float_to_ordered(dd), ROW_EXCLUDED - 1u) : ROW_EXCLUDED;
      if (has[u]) drow[j0 + tid + u * NT] = wd;
      const uint32_t x = has[u] ? wd : 0xffffffffu;
      m2 = min(m2, max(m1, x));
      m1 = min(m1, x);
    }
  }
  // Starting bound for the select, in the row's last word: each warp's kw-th
  // smallest of its threads' two smallest words, kw = ceil(R / warps), and
  // the largest of those. NW * kw >= R distinct candidates have words at or
  // below it, so the R-th smallest word is too; 0xffffffff (no bound) when
  // kw > 64 or a warp lacks kw kept candidates.
  constexpr int NW = NT / 32;
  __shared__ uint32_t wb[NW];
  const int kw = (a.R + NW - 1) / NW;
  const uint32_t b = kw >= 1 && kw <= 64 ? warp_kth_smallest64(m1, m2, kw) : 0xffffffffu;
  if (lane == 0) wb[tid >> 5] = b;
  __syncthreads();
  if (tid == 0) {
    uint32_t tmax = 0u;
#pragma unroll
    for (int w = 0; w < NW; ++w) tmax = max(tmax, wb[w]);
    drow[smax - 1] = tmax;
  }
}

// ---- selection -------------------------------------------------------------
constexpr int SEL_WARPS = 8;
constexpr int SEL_BINS = 256;
constexpr int SEL_SIDE = 256;

struct SelArgs {
  const uint32_t* dist;
  int64_t smax;
  const int32_t* probes;
  const int32_t* nprobe_q;
  const int64_t* list_off;
  int P, nlist, R;
  int64_t nq;
  uint64_t* out;
  int* err;
};

__host__ __device__ inline size_t sel_warp_bytes(int P) {
  return (size_t)SEL_BINS * 4 + (size_t)SEL_SIDE * 8 + (size_t)P * 8 + (((size_t)P + 1) * 4 + 7) / 8 * 8;
}

__device__ __forceinline__ unsigned long long shfl_min64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
    v = t < v ? t : v;
  }
  return v;
}
__device__ __forceinline__ unsigned long long shfl_max64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
    v = t > v ? t : v;
  }
  return v;
}

// Ascending sort of the h (<= 32 * RR) keys side[0, h) by the warp; the
// first `need` go to out.
template <int RR>
__device__ __forceinline__ void sel_sort_side(const uint64_t* side, int h, int need, uint64_t* out) {
  const int lane = threadIdx.x & 31;
  uint64_t v[RR];
#pragma unroll
  for (int i = 0; i < RR; ++i) {
    const int e = i * 32 + lane;
    v[i] = e < h ? side[e] : KEY_NONE;
  }
  warp_sort_regs<RR>(v);
#pragma unroll
  for (int i = 0; i < RR; ++i) {
    const int e = i * 32 + lane;
    if (e < need) out[e] = v[i];
  }
}

// Shortlists longer than SS_RMAX: one warp per query over its row in
// global memory. The query's candidates are its distance row's first
// n words, probe by probe; candidate i of probe p is CSR row
// off[p] + (i - beg[p]) and its key is (word << 32) | row. Pass 1 finds the
// valid keys' count, min and max; histogram passes over the keys still in
// play narrow [lo, hi] to the bin holding the R-th key (256 linear bins per
// pass) until that bin holds at most SEL_SIDE keys; the last pass writes
// every key below the bin and stages the bin's keys, which one warp sort
// orders to fill the shortlist. The shortlist is written unsorted in a
// fixed order (the row order of the passes).
__global__ void __launch_bounds__(SEL_WARPS * 32) k_row_select_wide(SelArgs a) {
  extern __shared__ __align__(16) uint8_t smraw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * SEL_WARPS + warp;
  if (row >= a.nq) return;
  uint8_t* base = smraw + (size_t)warp * sel_warp_bytes(a.P);
  uint32_t* hist = reinterpret_cast<uint32_t*>(base);
  uint64_t* side = reinterpret_cast<uint64_t*>(base + SEL_BINS * 4);
  int64_t* poff = reinterpret_cast<int64_t*>(base + SEL_BINS * 4 + SEL_SIDE * 8);
  int* pbeg = reinterpret_cast<int*>(poff + a.P);
  const int np = a.nprobe_q ? min(max(a.nprobe_q[row], 1), a.P) : a.P;
  int carry = 0;
  for (int p0 = 0; p0 < np; p0 += 32) {
    const int p = p0 + lane;
    int len = 0;
    if (p < np) {
      const int L = a.probes[row * a.P + p];
      int64_t off = 0;
      if (L >= 0 && L < a.nlist) {
        off = a.list_off[L];
        len = (int)(a.list_off[L + 1] - off);
      }
      poff[p] = off;
    }
    int incl = len;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (p < np) pbeg[p] = carry + incl - len;
    carry += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) pbeg[np] = carry;
  __syncwarp();
  // a row over smax was left unwritten (error site 106): no candidates
  const int n = carry <= a.smax ? carry : 0;
  const uint32_t* src = a.dist + row * a.smax;
  uint64_t* out = a.out + row * a.R;
  const int R = a.R;
  // Visits every key in a fixed order: f(valid, key) per element, per lane
  // elements lane, lane + 32, ... (four loads in flight). The loop bound is
  // the same for every lane (f may hold warp votes); lanes past n pass
  // valid = false.
  auto for_keys = [&](auto&& f) {
    int p = 0;
    for (int i0 = 0; i0 < n; i0 += 128) {
      uint32_t w[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = i0 + lane + 32 * u;
        w[u] = i < n ? __ldg(src + i) : ROW_EXCLUDED;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = i0 + lane + 32 * u;
        bool valid = false;
        uint64_t key = KEY_NONE;
        if (i < n) {
          while (pbeg[p + 1] <= i) ++p;
          valid = w[u] != ROW_EXCLUDED;
          key = ((uint64_t)w[u] << 32) | (uint32_t)(poff[p] + (i - pbeg[p]));
        }
        f(valid, key);
      }
    }
  };
  // pass 1: count, min, max
  unsigned long long kmin = ~0ull, kmax = 0ull;
  int nv = 0;
  for_keys([&](bool valid, uint64_t key) {
    if (valid) {
      ++nv;
      kmin = key < kmin ? key : kmin;
      kmax = key > kmax ? key : kmax;
    }
  });
  nv = __reduce_add_sync(0xffffffffu, nv);
  kmin = shfl_min64(kmin);
  kmax = shfl_max64(kmax);
  const unsigned lt = (1u << lane) - 1u;
  if (nv <= R) {
    int o = 0;
    for_keys([&](bool valid, uint64_t key) {
      const unsigned b = __ballot_sync(0xffffffffu, valid);
      if (valid) out[o + __popc(b & lt)] = key;
      o += __popc(b);
    });
    for (int j = nv + lane; j < R; j += 32) out[j] = KEY_NONE;
    return;
  }
  uint64_t lo = kmin, hi = kmax;
  int need = R;  // keys below lo taken: R - need
  int h = 0;
  for (int level = 0; level < 8; ++level) {
    const uint64_t span = hi - lo;
    const int sh = span < (uint64_t)SEL_BINS ? 0 : (64 - __clzll((long long)span)) - 8;
    for (int b = lane; b < SEL_BINS; b += 32) hist[b] = 0u;
    __syncwarp();
    for_keys([&](bool valid, uint64_t key) {
      if (valid && key >= lo && key <= hi) atomicAdd(&hist[(key - lo) >> sh], 1u);
    });
    __syncwarp();
    // the bin holding the need-th key: lane t sums bins [8t, 8t + 8)
    uint32_t c[8], local = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      c[j] = hist[lane * 8 + j];
      local += c[j];
    }
    uint32_t incl = local;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    uint32_t run = incl - local;
    int hit = -1;
    uint32_t hb = 0, before = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (hit < 0 && run < (uint32_t)need && (uint32_t)need <= run + c[j]) {
        hit = lane * 8 + j;
        hb = c[j];
        before = run;
      }
      run += c[j];
    }
    const unsigned who = __ballot_sync(0xffffffffu, hit >= 0);
    const int src_lane = __ffs(who) - 1;  // exactly one lane holds the bin
    const int b = __shfl_sync(0xffffffffu, hit, src_lane);
    h = (int)__shfl_sync(0xffffffffu, hb, src_lane);
    need -= (int)__shfl_sync(0xffffffffu, before, src_lane);
    const uint64_t nlo = lo + ((uint64_t)b << sh);
    const uint64_t wdt = (1ull << sh) - 1ull;  // sh <= 56
    const uint64_t nhi = hi - nlo <= wdt ? hi : nlo + wdt;
    lo = nlo;
    hi = nhi;
    __syncwarp();
    if (h <= SEL_SIDE) break;
  }
  if (h > SEL_SIDE) {  // never expected: each pass divides the range by 256
    if (lane == 0) atomicExch(a.err, 107);
    h = SEL_SIDE;
  }
  // keys below lo -> out; keys in [lo, hi] -> side
  int o = 0, so = 0;
  for_keys([&](bool valid, uint64_t key) {
    const bool below = valid && key < lo;
    const bool at = valid && key >= lo && key <= hi;
    const unsigned bb = __ballot_sync(0xffffffffu, below);
    const unsigned ba = __ballot_sync(0xffffffffu, at);
    if (below) out[o + __popc(bb & lt)] = key;
    if (at) {
      const int k = so + __popc(ba & lt);
      if (k < SEL_SIDE) side[k] = key;
    }
    o += __popc(bb);
    so += __popc(ba);
  });
  __syncwarp();
  if (h <= 32) sel_sort_side<1>(side, h, need, out + (R - need));
  else if (h <= 64) sel_sort_side<2>(side, h, need, out + (R - need));
  else if (h <= 128) sel_sort_side<4>(side, h, need, out + (R - need));
  else sel_sort_side<8>(side, h, need, out + (R - need));
}

// ---- shortlists of up to SS_RMAX keys: one streaming pass ----------------
constexpr int SS_WARPS = 4;
constexpr int SS_RMAX = 256;
constexpr int SS_CAP = 640;  // staged keys per warp: R kept + at least three rounds of 128

__host__ __device__ inline size_t ss_warp_bytes(int P) {
  return (size_t)SS_CAP * 8 + (size_t)SEL_SIDE * 8 + (size_t)SEL_BINS * 4 + (size_t)P * 8 +
         (((size_t)P + 1) * 4 + 7) / 8 * 8;
}

// Keeps the R smallest of the m (> R) distinct keys buf[0, m) in buf[0, R),
// unsorted, and returns the largest kept key. One warp: min and max, then
// 256-bin histogram passes over [lo, hi] until the bin holding the R-th key
// holds at most SEL_SIDE keys; the keys below that bin are compacted in
// place (in order) and the bin's keys sorted to fill the rest.
__device__ uint64_t warp_keep_smallest(uint64_t* buf, int m, int R, uint64_t* side, uint32_t* hist) {
  const int lane = threadIdx.x & 31;
  unsigned long long kmin = ~0ull, kmax = 0ull;
  for (int j = lane; j < m; j += 32) {
    const unsigned long long k = buf[j];
    kmin = k < kmin ? k : kmin;
    kmax = k > kmax ? k : kmax;
  }
  uint64_t lo = shfl_min64(kmin), hi = shfl_max64(kmax);
  int need = R, h = m;
  for (int level = 0; level < 8; ++level) {
    const uint64_t span = hi - lo;
    const int sh = span < (uint64_t)SEL_BINS ? 0 : (64 - __clzll((long long)span)) - 8;
    for (int b = lane; b < SEL_BINS; b += 32) hist[b] = 0u;
    __syncwarp();
    for (int j = lane; j < m; j += 32) {
      const uint64_t k = buf[j];
      if (k >= lo && k <= hi) atomicAdd(&hist[(k - lo) >> sh], 1u);
    }
    __syncwarp();
    uint32_t c[8], local = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      c[j] = hist[lane * 8 + j];
      local += c[j];
    }
    uint32_t incl = local;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    uint32_t run = incl - local;
    int hit = -1;
    uint32_t hb = 0, before = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (hit < 0 && run < (uint32_t)need && (uint32_t)need <= run + c[j]) {
        hit = lane * 8 + j;
        hb = c[j];
        before = run;
      }
      run += c[j];
    }
    const int src_lane = __ffs(__ballot_sync(0xffffffffu, hit >= 0)) - 1;
    const int b = __shfl_sync(0xffffffffu, hit, src_lane);
    h = (int)__shfl_sync(0xffffffffu, hb, src_lane);
    need -= (int)__shfl_sync(0xffffffffu, before, src_lane);
    const uint64_t nlo = lo + ((uint64_t)b << sh);
    const uint64_t wdt = (1ull << sh) - 1ull;  // sh <= 56
    hi = hi - nlo <= wdt ? hi : nlo + wdt;
    lo = nlo;
    __syncwarp();
    if (h <= SEL_SIDE) break;
  }
  // distinct keys: a one-key-wide bin holds one key, so h <= SEL_SIDE here
  const unsigned lt = (1u << lane) - 1u;
  int o = 0, so = 0;
  for (int j0 = 0; j0 < m; j0 += 32) {
    const int j = j0 + lane;
    const uint64_t k = j < m ? buf[j] : KEY_NONE;
    const bool below = j < m && k < lo;
    const bool at = j < m && k >= lo && k <= hi;
    const unsigned bb = __ballot_sync(0xffffffffu, below);  // every read of this round is done
    const unsigned ba = __ballot_sync(0xffffffffu, at);
    if (below) buf[o + __popc(bb & lt)] = k;  // o + rank <= j: never ahead of the reads
    if (at) {
      const int s = so + __popc(ba & lt);
      if (s < SEL_SIDE) side[s] = k;
    }
    o += __popc(bb);
    so += __popc(ba);
  }
  __syncwarp();
  h = min(h, SEL_SIDE);
  if (h <= 32) sel_sort_side<1>(side, h, need, buf + (R - need));
  else if (h <= 64) sel_sort_side<2>(side, h, need, buf + (R - need));
  else if (h <= 128) sel_sort_side<4>(side, h, need, buf + (R - need));
  else sel_sort_side<8>(side, h, need, buf + (R - need));
  __syncwarp();
  return buf[R - 1];
}

// One warp per query, one pass over its distance row (16-byte loads, three
// rounds ahead of the keys being built): keys below the running bound T
// (whose word starts at the rows kernel's bound on the R-th smallest word)
// are staged in shared memory; when the staging area could overflow, the R
// smallest are kept and T becomes the largest of them (a later key at or
// above T cannot be among the R smallest). The kept set is the R smallest
// keys whatever the order of arrival; it is written unsorted, in a fixed
// order.
__global__ void __launch_bounds__(SS_WARPS * 32) k_row_select_stream(SelArgs a) {
  extern __shared__ __align__(16) uint8_t smraw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * SS_WARPS + warp;
  if (row >= a.nq) return;
  uint8_t* base = smraw + (size_t)warp * ss_warp_bytes(a.P);
  uint64_t* buf = reinterpret_cast<uint64_t*>(base);
  uint64_t* side = buf + SS_CAP;
  uint32_t* hist = reinterpret_cast<uint32_t*>(side + SEL_SIDE);
  int64_t* poff = reinterpret_cast<int64_t*>(hist + SEL_BINS);
  int* pbeg = reinterpret_cast<int*>(poff + a.P);
  const int np = a.nprobe_q ? min(max(a.nprobe_q[row], 1), a.P) : a.P;
  int carry = 0;
  for (int p0 = 0; p0 < np; p0 += 32) {
    const int p = p0 + lane;
    int len = 0;
    if (p < np) {
      const int L = a.probes[row * a.P + p];
      int64_t off = 0;
      if (L >= 0 && L < a.nlist) {
        off = a.list_off[L];
        len = (int)(a.list_off[L + 1] - off);
      }
      poff[p] = off;
    }
    int incl = len;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (p < np) pbeg[p] = carry + incl - len;
    carry += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) pbeg[np] = carry;
  __syncwarp();
  const int n = carry <= a.smax - 1 ? carry : 0;  // a row over smax - 1 was left unwritten (106)
  const uint32_t* src = a.dist + row * a.smax;  // smax is a multiple of 4: 16-byte rows
  const int R = a.R;
  const unsigned lt = (1u << lane) - 1u;
  uint64_t T = KEY_NONE;
  // T's distance word; it starts at the rows kernel's bound on the R-th
  // smallest word (the row's last word)
  uint32_t Tw = n > 0 ? __ldg(src + a.smax - 1) : 0xffffffffu;
  int m = 0, p = 0;           // p: probe cursor, advanced only for words that may enter
  // words i0 + 4 lane .. + 3 of each 128-word round (the row holds smax
  // >= roundup(n, 4) words, so the vector load stays in the row)
  auto load4 = [&](int i0) {
    const int i = i0 + 4 * lane;
    return i < n ? __ldg(reinterpret_cast<const uint4*>(src + i))
                 : make_uint4(ROW_EXCLUDED, ROW_EXCLUDED, ROW_EXCLUDED, ROW_EXCLUDED);
  };
  // four rounds of the row in flight (the select is bound by the latency of
  // its row reads, not by their bytes)
  uint4 cur = load4(0), n1 = load4(128), n2 = load4(256);
  for (int i0 = 0; i0 < n; i0 += 128) {
    const uint4 n3 = load4(i0 + 384);
    if (m + 128 > SS_CAP) {
      T = warp_keep_smallest(buf, m, R, side, hist);
      Tw = (uint32_t)(T >> 32);
      m = R;
    }
    const uint32_t w[4] = {cur.x, cur.y, cur.z, cur.w};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + 4 * lane + u;
      uint64_t key = KEY_NONE;
      // a key below T has a word at or below T's; only those build the key
      bool in = i < n && w[u] != ROW_EXCLUDED && w[u] <= Tw;
      if (in) {
        while (pbeg[p + 1] <= i) ++p;
        key = ((uint64_t)w[u] << 32) | (uint32_t)(poff[p] + (i - pbeg[p]));
        in = key < T;
      }
      const unsigned b = __ballot_sync(0xffffffffu, in);
      if (in) buf[m + __popc(b & lt)] = key;
      m += __popc(b);
    }
    cur = n1;
    n1 = n2;
    n2 = n3;
  }
  __syncwarp();
  if (m > R) {
    warp_keep_smallest(buf, m, R, side, hist);
    m = R;
  }
  uint64_t* out = a.out + row * R;
  for (int j = lane; j < R; j += 32) out[j] = j < m ? buf[j] : KEY_NONE;
}

// Rows of R keys sorted ascending in place (KEY_NONE padded to Rp in
// shared memory).
__global__ void __launch_bounds__(256) k_row_sort(uint64_t* keys, int R, int Rp) {
  extern __shared__ __align__(16) uint64_t sk[];
  uint64_t* rowp = keys + (int64_t)blockIdx.x * R;
  for (int i = threadIdx.x; i < Rp; i += 256) sk[i] = i < R ? rowp[i] : KEY_NONE;
  block_bitonic_sort(sk, Rp);
  for (int i = threadIdx.x; i < R; i += 256) rowp[i] = sk[i];
}


}  // namespace

size_t ivfpq_rows_smem(int M, int d, int nprobe) {
  return (((size_t)(M * 256 + d) * 4 + 15) & ~size_t(15)) + (size_t)nprobe * 8 +
         (size_t)(nprobe + 1) * 4 + (size_t)nprobe * 4;
}

// A row holds smax candidate words and, in its last word, the select's
// starting bound (16-byte aligned rows).
int64_t ivfpq_rows_stride(int64_t smax) { return std::max<int64_t>(4, (smax + 4) & ~int64_t(3)); }

void launch_ivfpq_scan_rows(FastScanArgs f, uint32_t* dist, int64_t smax, cudaStream_t s, int nt,
                            mv_ctx* prof) {
  const int64_t nq = f.nq;
  if (nq == 0) return;
  const int64_t stride = ivfpq_rows_stride(smax);
  const size_t smem = ivfpq_rows_smem(f.M, f.d, f.nprobe);
  MV_REQUIRE(smem <= 200 * 1024, MV_ERR_UNSUPPORTED, "two-kernel ADC scan: M, d or nprobe too large");
  auto go = [&](auto kernel, int threads) {
    smem_limit(kernel, smem);
    StageTimer t(prof, MV_STAGE_ADC, s);
    kernel<<<(unsigned)nq, threads, smem, s>>>(f, dist, stride);
  };
  if (nt == 64) go(k_ivfpq_rows<64, 2>, 64);
  else if (nt == 128) go(k_ivfpq_rows<128, 2>, 128);
  else if (nt == 512) go(k_ivfpq_rows<512, 2>, 512);
  else go(k_ivfpq_rows<256, 2>, 256);
  count_launch();
  SelArgs sa;
  sa.dist = dist;
  sa.smax = stride;
  sa.probes = f.probes;
  sa.nprobe_q = f.nprobe_q;
  sa.list_off = f.list_off;
  sa.P = f.nprobe;
  sa.nlist = f.nlist;
  sa.R = f.R;
  sa.nq = nq;
  sa.out = f.out_keys;
  sa.err = f.err;
  if (f.R <= SS_RMAX) {
    const size_t ssm = ss_warp_bytes(f.nprobe) * SS_WARPS;
    MV_REQUIRE(ssm <= 200 * 1024, MV_ERR_UNSUPPORTED, "two-kernel ADC scan: nprobe too large");
    smem_limit(k_row_select_stream, ssm);
    k_row_select_stream<<<(unsigned)((nq + SS_WARPS - 1) / SS_WARPS), SS_WARPS * 32, ssm, s>>>(sa);
  } else {
    const size_t ssm = sel_warp_bytes(f.nprobe) * SEL_WARPS;
    MV_REQUIRE(ssm <= 200 * 1024, MV_ERR_UNSUPPORTED, "two-kernel ADC scan: nprobe too large");
    smem_limit(k_row_select_wide, ssm);
    k_row_select_wide<<<(unsigned)((nq + SEL_WARPS - 1) / SEL_WARPS), SEL_WARPS * 32, ssm, s>>>(sa);
  }
  count_launch();
  if (f.sorted) {
    const int Rp = next_pow2(f.R);
    MV_REQUIRE((size_t)Rp * 8 <= 200 * 1024, MV_ERR_UNSUPPORTED, "shortlist too long to sort");
    smem_limit(k_row_sort, (size_t)Rp * 8);
    k_row_sort<<<(unsigned)nq, 256, (size_t)Rp * 8, s>>>(f.out_keys, f.R, Rp);
    count_launch();
  }
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
