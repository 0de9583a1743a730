// Fast-form IVF-PQ ADC scan with bank-rotated fixed-point tables
// (index/index_ivf_pq.mojo:295-347, the fast form's expansion of the
// distance; k_ivfpq_fast.cu states it).
//
// One CTA per query (or a persistent grid taking queries from a counter).
// The per-query table -scale * <q_m, C[m][k]> is built in shared memory as
// 32-bit fixed-point entries (a per-query power of two from the
// Cauchy-Schwarz bound sum_m ||q_m|| max_k ||C[m][k]|| keeps every sum of M
// entries below 2^29) in a bank-rotated layout: the 128-byte row of code k
// holds the entries of S subspaces, 32 / S copies side by side, so word
// (k, m + S h) sits in bank m + S h. Lane l handles subspace (r + s) mod S
// at step s, r = l mod S, in copy h = l / S: the 32 lanes of a warp read 32
// different banks at every step whatever the codes, so every table lookup
// of a warp is one shared-memory wavefront (with the plain layout the
// random codes put several lanes on one bank). A candidate's code bytes are
// rotated by r in registers once so that step s reads a fixed byte.
// Integer sums do not depend on the order of the lookups.
//
// Candidates are the probed lists laid end to end; candidate i's distance
// is staged in slot i as an order-preserving word (no compaction), and the
// R smallest (distance, candidate index) keys are found by a range select:
// adaptive 2048-bin histograms over the keys narrow the key range holding
// the R-th key until it holds at most 256 keys, which one warp sorts. Lists
// longer than the staging area run in chunks, each chunk's keys selected
// together with the R kept from the chunks before (keys at or above the
// R-th kept key are not staged). The shortlist is written as
// (distance, CSR position) keys.
#include <cuda_fp16.h>

#include <algorithm>

#include "mv_fast.h"
#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_select.cuh"

namespace mv {
namespace {

constexpr int RT_NB_LOG = 10;     // histogram bins of one select level: 2^RT_NB_LOG
constexpr int RT_NB = 1 << RT_NB_LOG;
constexpr int RT_SIDE = 256;      // keys of the boundary range sorted by one warp
constexpr uint32_t RT_EXCL = 0xffffffffu;  // staged word of a candidate that takes no part

struct RtScratch {
  uint32_t wsum[32];
  unsigned int lo, hi;      // min / max high word of the valid keys
  int nvalid;
  int out_n, side_n;
  uint32_t bin, before, h;
  unsigned long long kth;   // the R-th smallest key of the last select (R kept)
  int q;                    // persistent grid: query being scanned
  int bad;                  // non-finite table bound
  int e;                    // table entries are in units of 2^-e
};

__device__ __forceinline__ void warp_sort_side(uint64_t* side, int h, int need, uint64_t* out,
                                               unsigned long long* kth) {
  if (h <= 32) sort_side<1>(side, h, need, out, kth);
  else if (h <= 64) sort_side<2>(side, h, need, out, kth);
  else if (h <= 128) sort_side<4>(side, h, need, out, kth);
  else sort_side<8>(side, h, need, out, kth);
}

// R smallest of the n keys key_at(e) (KEY_NONE: no key), unsorted into
// out[0, r), r = min(R, valid keys); when r == R, rs.kth is the R-th
// smallest. Keys are distinct. Every thread of the block calls it.
template <int NT, typename KeyAt>
__device__ int range_select(KeyAt key_at, int n, int R, uint64_t* out, uint32_t* hist,
                            uint64_t* side, RtScratch& rs) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // valid keys and the range of their high words
  uint32_t lo = 0xffffffffu, hi = 0u;
  int cnt = 0;
  for (int e = tid; e < n; e += NT) {
    const uint64_t k = key_at(e);
    if (k != KEY_NONE) {
      lo = min(lo, (uint32_t)(k >> 32));
      hi = max(hi, (uint32_t)(k >> 32));
      ++cnt;
    }
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  if (tid == 0) {
    rs.lo = 0xffffffffu;
    rs.hi = 0u;
    rs.nvalid = 0;
    rs.out_n = 0;
    rs.side_n = 0;
    rs.kth = KEY_NONE;  // set only when more than R keys compete
  }
  __syncthreads();
  if (lane == 0) {
    atomicMin(&rs.lo, lo);
    atomicMax(&rs.hi, hi);
    atomicAdd(&rs.nvalid, cnt);
  }
  __syncthreads();
  const int nvalid = rs.nvalid;
  if (nvalid <= R) {
    for (int e0 = 0; e0 < n; e0 += NT) {
      const int e = e0 + tid;
      const uint64_t k = e < n ? key_at(e) : KEY_NONE;
      const bool v = k != KEY_NONE;
      const unsigned b = __ballot_sync(0xffffffffu, v);
      int o = 0;
      if (lane == 0 && b) o = atomicAdd(&rs.out_n, __popc(b));
      o = __shfl_sync(0xffffffffu, o, 0);
      if (v) out[o + __popc(b & ((1u << lane) - 1u))] = k;
    }
    __syncthreads();
    return nvalid;
  }
  // narrow [L, H] (64-bit keys) to a range holding the R-th key
  uint64_t L = (uint64_t)rs.lo << 32, H = ((uint64_t)rs.hi << 32) | 0xffffffffull;
  uint32_t before = 0, h = 0;
  for (;;) {
    const bool high = (uint32_t)(L >> 32) != (uint32_t)(H >> 32);
    const uint32_t base = high ? (uint32_t)(L >> 32) : (uint32_t)L;
    const uint32_t span = high ? (uint32_t)(H >> 32) - base : (uint32_t)H - base;
    const int sh = span < (uint32_t)RT_NB ? 0 : (32 - __clz((int)(span >> RT_NB_LOG)));
    const int nb = (int)(span >> sh) + 1;
    for (int b = tid; b < nb; b += NT) hist[b] = 0u;
    __syncthreads();
    for (int e = tid; e < n; e += NT) {
      const uint64_t k = key_at(e);
      if (k != KEY_NONE && k >= L && k <= H) {
        const uint32_t w = high ? (uint32_t)(k >> 32) : (uint32_t)k;
        atomicAdd(&hist[(w - base) >> sh], 1u);
      }
    }
    __syncthreads();
    // the bin holding key number R - before of the range: per-thread runs
    // of bins, block prefix sums
    const int per = (nb + NT - 1) / NT;
    const int b0 = tid * per;
    uint32_t local = 0;
    for (int b = b0; b < b0 + per && b < nb; ++b) local += hist[b];
    uint32_t incl = local;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) rs.wsum[warp] = incl;
    __syncthreads();
    uint32_t wbase = 0;
    for (int w = 0; w < warp; ++w) wbase += rs.wsum[w];
    uint32_t run = before + wbase + incl - local;
    for (int b = b0; b < b0 + per && b < nb; ++b) {
      const uint32_t c = hist[b];
      if (run < (uint32_t)R && (uint32_t)R <= run + c) {
        rs.bin = (uint32_t)b;
        rs.before = run;
        rs.h = c;
      }
      run += c;
    }
    __syncthreads();
    const uint32_t bin = rs.bin;
    before = rs.before;
    h = rs.h;
    __syncthreads();  // rs and hist are reused below
    const uint64_t blo = (uint64_t)base + ((uint64_t)bin << sh);
    const uint64_t bhi = blo + ((1ull << sh) - 1ull);
    if (high) {
      L = blo << 32;
      const uint64_t hh = H >> 32;
      H = ((bhi < hh ? bhi : hh) << 32) | 0xffffffffull;
    } else {
      L = (L & 0xffffffff00000000ull) | blo;
      const uint64_t hl = H & 0xffffffffull;
      H = (H & 0xffffffff00000000ull) | (bhi < hl ? bhi : hl);
    }
    if (h <= (uint32_t)RT_SIDE) break;
  }
  // every key below L is taken; the range's keys are sorted by one warp
  for (int e0 = 0; e0 < n; e0 += NT) {
    const int e = e0 + tid;
    const uint64_t k = e < n ? key_at(e) : KEY_NONE;
    const bool below = k != KEY_NONE && k < L;
    const bool at = k != KEY_NONE && k >= L && k <= H;
    const unsigned mb = __ballot_sync(0xffffffffu, below);
    const unsigned ma = __ballot_sync(0xffffffffu, at);
    int ob = 0, oa = 0;
    if (lane == 0) {
      if (mb) ob = atomicAdd(&rs.out_n, __popc(mb));
      if (ma) oa = atomicAdd(&rs.side_n, __popc(ma));
    }
    ob = __shfl_sync(0xffffffffu, ob, 0);
    oa = __shfl_sync(0xffffffffu, oa, 0);
    const unsigned lt = (1u << lane) - 1u;
    if (below) out[ob + __popc(mb & lt)] = k;
    if (at) side[oa + __popc(ma & lt)] = k;
  }
  __syncthreads();
  if (warp == 0) warp_sort_side(side, (int)h, R - (int)before, out + before, &rs.kth);
  __syncthreads();
  return R;
}

// Lane state of the rotated lookups: rotation r = lane mod S, copy h =
// lane / S, byte offsets of step s's word within a code row (S <= 16; the
// 32-subspace layout computes them per step).
template <int S>
struct RtLane {
  static constexpr int WS = S / 4;
  int boff[S <= 16 ? S : 1];
  int r4, qw, rb8, h;
  __device__ __forceinline__ void init(int lane) {
    const int r = lane & (S - 1);
    h = lane / S;
    r4 = 4 * r;
    qw = r >> 2;
    rb8 = 8 * (r & 3);
    if constexpr (S <= 16) {
#pragma unroll
      for (int s = 0; s < S; ++s) boff[s] = 4 * (((r + s) & (S - 1)) + S * h);
    }
  }
  // Sum of a code's table entries; w holds the code's first WS words (zero
  // past M, whose table slots hold 0).
  __device__ __forceinline__ int sum(const char* tab, const uint32_t (&w)[WS]) const {
    uint32_t L[WS];
#pragma unroll
    for (int i = 0; i < WS; ++i) L[i] = w[i];
#pragma unroll
    for (int b = 1; b < WS; b <<= 1) {
      const bool f = (qw & b) != 0;
      uint32_t T[WS];
#pragma unroll
      for (int i = 0; i < WS; ++i) T[i] = f ? L[(i + b) % WS] : L[i];
#pragma unroll
      for (int i = 0; i < WS; ++i) L[i] = T[i];
    }
    uint32_t o[WS];
#pragma unroll
    for (int i = 0; i < WS; ++i) o[i] = __funnelshift_r(L[i], L[(i + 1) % WS], rb8);
    int a0 = 0, a1 = 0, a2 = 0;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const uint32_t c = __byte_perm(o[s >> 2], 0u, 0x4440u + (s & 3));
      int off;
      if constexpr (S <= 16) off = boff[s];
      else off = (r4 + 4 * s) & 127;
      const int v = *reinterpret_cast<const int*>(tab + (c << 7) + off);
      if (s % 3 == 0) a0 += v;
      else if (s % 3 == 1) a1 += v;
      else a2 += v;
    }
    return a0 + a1 + a2;
  }
};

template <int WS>
__device__ __forceinline__ void rt_load_code(const uint8_t* __restrict__ row, int M,
                                             uint32_t (&w)[WS]) {
  const int nw = M >> 2;
  if ((M & 15) == 0) {
#pragma unroll
    for (int i = 0; i < WS; i += 4) {
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (i < nw) v = __ldg(reinterpret_cast<const uint4*>(row + 4 * i));
      w[i] = v.x;
      if (i + 1 < WS) w[i + 1] = v.y;
      if (i + 2 < WS) w[i + 2] = v.z;
      if (i + 3 < WS) w[i + 3] = v.w;
    }
  } else if ((M & 7) == 0) {
#pragma unroll
    for (int i = 0; i < WS; i += 2) {
      uint2 v = make_uint2(0u, 0u);
      if (i < nw) v = __ldg(reinterpret_cast<const uint2*>(row + 4 * i));
      w[i] = v.x;
      if (i + 1 < WS) w[i + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < WS; ++i)
      w[i] = i < nw ? __ldg(reinterpret_cast<const uint32_t*>(row + 4 * i)) : 0u;
  }
}

// Dynamic shared memory of one CTA: table, staged words, kept and output
// keys, the boundary range, the histogram, the query, the probe table.
struct RtLayout {
  size_t tab, vals, kept, outk, side, hist, qv, poff, pbeg, pterm, total;
  __host__ __device__ RtLayout(int cap, int R, int Rp, int d, int nprobe) {
    size_t o = 0;
    tab = o;
    o += 256 * 128;
    vals = o;
    o += (size_t)cap * 4;
    o = (o + 15) & ~size_t(15);
    kept = o;
    o += (size_t)R * 8;
    outk = o;
    o += (size_t)Rp * 8;
    side = o;
    o += (size_t)RT_SIDE * 8;
    hist = o;
    o += (size_t)RT_NB * 4;
    qv = o;
    o += (size_t)((d + 3) & ~3) * 4;
    poff = o;
    o += (size_t)nprobe * 8;
    pbeg = o;
    o += (size_t)(nprobe + 1) * 4;
    pterm = o;
    o += (size_t)nprobe * 4;
    total = (o + 15) & ~size_t(15);
  }
};

template <int NT, int S>
__global__ void __launch_bounds__(NT, 1024 / NT) k_ivfpq_scan_rt(FastScanArgs a) {
  constexpr int C = 32 / S;        // copies of the table in a code row
  constexpr int NW = NT / 32;
  constexpr int WS = S / 4;
  extern __shared__ __align__(128) unsigned char smraw[];
  const int M = a.M, d = a.d, dsub = d / M;
  const RtLayout lay(a.cap, a.R, a.Rp, d, a.nprobe);
  int* tab = reinterpret_cast<int*>(smraw + lay.tab);
  uint32_t* vals = reinterpret_cast<uint32_t*>(smraw + lay.vals);
  uint64_t* kept = reinterpret_cast<uint64_t*>(smraw + lay.kept);
  uint64_t* outk = reinterpret_cast<uint64_t*>(smraw + lay.outk);
  uint64_t* side = reinterpret_cast<uint64_t*>(smraw + lay.side);
  uint32_t* hist = reinterpret_cast<uint32_t*>(smraw + lay.hist);
  float* qv = reinterpret_cast<float*>(smraw + lay.qv);
  int64_t* poff = reinterpret_cast<int64_t*>(smraw + lay.poff);
  int* pbeg = reinterpret_cast<int*>(smraw + lay.pbeg);
  float* pterm = reinterpret_cast<float*>(smraw + lay.pterm);
  __shared__ RtScratch rs;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const float scale = a.metric == MV_METRIC_L2 ? -2.0f : -1.0f;
  RtLane<S> rl;
  rl.init(lane);
  for (int iter = 0;; ++iter) {
    int qi;
    if (a.counter) {
      __syncthreads();  // the previous query is done with shared memory
      if (tid == 0) rs.q = atomicAdd(a.counter, 1);
      __syncthreads();
      qi = rs.q;
      if (qi >= a.nq) break;
    } else {
      if (iter > 0) break;
      qi = blockIdx.x;
    }
    const int64_t row = a.order ? a.order[qi] : qi;
    const int nprobe = a.nprobe_q ? min(max(a.nprobe_q[row], 1), a.nprobe) : a.nprobe;
    for (int j = tid; j < d; j += NT) qv[j] = a.q[row * d + j];
    // probe table: offsets, lengths -> prefix sums (warp 0)
    if (warp == 0) {
      int carry = 0;
      for (int p0 = 0; p0 < nprobe; p0 += 32) {
        const int p = p0 + lane;
        int len = 0;
        if (p < nprobe) {
          int list = a.probes[row * a.nprobe + p];
          if (list >= a.nlist) {
            atomicExch(a.err, 106);
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
    // fixed-point scale: |sum of M entries| <= B 2^e < 2^29
    if (warp == 0) {
      float b = 0.0f;
      for (int m = lane; m < M; m += 32) {
        float s2 = 0.0f;
        for (int t = 0; t < dsub; ++t) s2 = fmaf(qv[m * dsub + t], qv[m * dsub + t], s2);
        b += sqrtf(s2) * a.pq_cn[m];
      }
      for (int o = 16; o > 0; o >>= 1) b += __shfl_xor_sync(0xffffffffu, b, o);
      if (lane == 0) {
        b *= fabsf(scale) * 1.0625f;
        const bool bad = !(b <= 3.0e38f);  // NaN or infinite
        int e = 0;
        if (!bad && b > 0.0f) e = min(max(29 - (ilogbf(b) + 1), -120), 120);
        rs.e = e;
        rs.bad = bad ? 1 : 0;
      }
    }
    __syncthreads();
    const float mul = scale * a.pq16_inv * __int_as_float((rs.e + 127) << 23);
    const float lscale = __int_as_float((127 - rs.e) << 23);  // 2^-e
    const bool bad = rs.bad != 0;
    // table: lane (m = lane mod S, co = lane / S) builds entry (m, code c)
    // for C codes per warp step and writes its C copies, copy (co + t) mod C
    // at store t so that the warp's stores cover the 32 banks
    {
      const int m = lane & (S - 1), co = lane / S;
      float qm[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) qm[t] = (m < M && t < dsub) ? qv[m * dsub + t] : 0.0f;
      const __half* cm = a.pq16 + (int64_t)min(m, M - 1) * 256 * dsub;
      constexpr int U = NT >= 512 ? 4 : 8;
      for (int c0 = warp * C; c0 < 256; c0 += NW * C * U) {
        uint4 cw[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int c = c0 + u * NW * C + co;
          cw[u] = make_uint4(0u, 0u, 0u, 0u);
          if (c < 256 && m < M) {
            if (dsub == 8) {
              cw[u] = __ldg(reinterpret_cast<const uint4*>(cm + c * 8));
            } else {
              const uint2 v = __ldg(reinterpret_cast<const uint2*>(cm + c * 4));
              cw[u].x = v.x;
              cw[u].y = v.y;
            }
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int c = c0 + u * NW * C + co;
          if (c0 + u * NW * C >= 256) break;  // warp-uniform
          const float2 h0 = __half22float2(*reinterpret_cast<const __half2*>(&cw[u].x));
          const float2 h1 = __half22float2(*reinterpret_cast<const __half2*>(&cw[u].y));
          const float2 h2 = __half22float2(*reinterpret_cast<const __half2*>(&cw[u].z));
          const float2 h3 = __half22float2(*reinterpret_cast<const __half2*>(&cw[u].w));
          float dot = qm[0] * h0.x;
          dot = fmaf(qm[1], h0.y, dot);
          dot = fmaf(qm[2], h1.x, dot);
          dot = fmaf(qm[3], h1.y, dot);
          dot = fmaf(qm[4], h2.x, dot);
          dot = fmaf(qm[5], h2.y, dot);
          dot = fmaf(qm[6], h3.x, dot);
          dot = fmaf(qm[7], h3.y, dot);
          const int v = (m < M && !bad) ? __float2int_rn(dot * mul) : 0;
#pragma unroll
          for (int t = 0; t < C; ++t) tab[c * 32 + m + S * ((co + t) % C)] = v;
        }
      }
    }
    __syncthreads();
    const int total = pbeg[nprobe];
    const int cap = a.cap;
    const char* tabb = reinterpret_cast<const char*>(tab);
    int nk = 0;                        // kept keys from earlier chunks
    uint32_t bound_hi = 0xffffffffu;   // staged words at or above it take no part
    int p = 0;                         // per-thread probe cursor (indices only grow)
    for (int base = 0; base < total || (base == 0 && total == 0); base += cap) {
      const int len = min(cap, total - base);
      // stage the chunk's distance words, two candidates per thread per step
      for (int j0 = 0; j0 < len; j0 += 2 * NT) {
        const int j = j0 + tid;
        const bool has0 = j < len, has1 = j + NT < len;
        const int c0 = base + j, c1 = c0 + NT;
        if (has0)
          while (pbeg[p + 1] <= c0) ++p;
        int p1 = p;
        if (has1)
          while (pbeg[p1 + 1] <= c1) ++p1;
        int64_t pos0 = has0 ? poff[p] + (c0 - pbeg[p]) : 0;
        int64_t pos1 = has1 ? poff[p1] + (c1 - pbeg[p1]) : 0;
        bool keep0 = has0, keep1 = has1;
        if ((has0 && (pos0 < 0 || pos0 >= a.ntotal)) || (has1 && (pos1 < 0 || pos1 >= a.ntotal))) {
          atomicExch(a.err, 107);  // never expected: skip both
          pos0 = 0;
          pos1 = 0;
          keep0 = keep1 = false;
        }
        uint32_t w0[WS], w1[WS];
        rt_load_code<WS>(a.codes + pos0 * M, M, w0);
        rt_load_code<WS>(a.codes + pos1 * M, M, w1);
        const float v0 = a.vterm ? __ldg(a.vterm + pos0) : 0.0f;
        const float v1 = a.vterm ? __ldg(a.vterm + pos1) : 0.0f;
        if (a.filter) {  // filtered ids never enter the shortlist
          const uint32_t id0 = a.ids[pos0], id1 = a.ids[pos1];
          if ((int64_t)id0 < a.filter_len && a.filter[id0] != 0) keep0 = false;
          if ((int64_t)id1 < a.filter_len && a.filter[id1] != 0) keep1 = false;
        }
        const int s0 = rl.sum(tabb, w0);
        const int s1 = rl.sum(tabb, w1);
        float d0 = fmaf((float)s0, lscale, (has0 ? pterm[p] : 0.0f) + v0);
        float d1 = fmaf((float)s1, lscale, (has1 ? pterm[p1] : 0.0f) + v1);
        if (bad) d0 = d1 = __int_as_float(0x7fc00000);
        uint32_t o0 = min(float_to_ordered(d0), RT_EXCL - 1u);  // RT_EXCL marks no key
        uint32_t o1 = min(float_to_ordered(d1), RT_EXCL - 1u);
        if (!keep0 || o0 >= bound_hi) o0 = RT_EXCL;
        if (!keep1 || o1 >= bound_hi) o1 = RT_EXCL;
        if (has0) vals[j] = o0;
        if (has1) vals[j + NT] = o1;
        if (has0) p = p1;
      }
      __syncthreads();
      auto key_at = [&](int e) -> uint64_t {
        if (e < nk) return kept[e];
        const uint32_t v = vals[e - nk];
        return v == RT_EXCL ? KEY_NONE : ((uint64_t)v << 32) | (uint32_t)(base + e - nk);
      };
      const int r = range_select<NT>(key_at, nk + max(len, 0), a.R, outk, hist, side, rs);
      const bool more = base + cap < total;
      if (more) {
        for (int i = tid; i < r; i += NT) kept[i] = outk[i];
        // later candidates have larger indices: one whose word equals the
        // R-th kept key's cannot enter either
        if (rs.kth != KEY_NONE) bound_hi = (uint32_t)(rs.kth >> 32);
        nk = r;
        __syncthreads();
      } else {
        nk = r;
      }
    }
    // output: (distance, CSR position) keys; sorted by (distance, candidate)
    // first when the shortlist is the answer
    if (a.sorted) {
      for (int i = nk + tid; i < a.Rp; i += NT) outk[i] = KEY_NONE;
      __syncthreads();
      block_bitonic_sort(outk, a.Rp);
      __syncthreads();
    }
    for (int i = tid; i < a.R; i += NT) {
      uint64_t key = KEY_NONE;
      if (i < nk) {
        const uint64_t k = outk[i];
        const int idx = (int)(uint32_t)k;
        int lo = 0, hi = nprobe - 1;  // the probe holding candidate idx
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (pbeg[mid] <= idx) lo = mid;
          else hi = mid - 1;
        }
        const int64_t pos = poff[lo] + (idx - pbeg[lo]);
        key = (k & 0xffffffff00000000ull) | (uint32_t)pos;
      }
      a.out_keys[row * a.R + i] = key;
    }
  }  // queries
}

int rt_pass_width(int M) { return M <= 8 ? 8 : (M <= 16 ? 16 : 32); }

}  // namespace

bool ivfpq_rt_supported(const FastScanArgs& a) {
  const int dsub = a.M > 0 ? a.d / a.M : 0;
  return a.pq16 && a.pq_cn && (a.M & 3) == 0 && a.M >= 4 && a.M <= 32 && a.M * dsub == a.d &&
         (dsub == 4 || dsub == 8) && a.R >= 1 && a.R <= 2048 && a.nprobe >= 1;
}

size_t ivfpq_rt_smem(const FastScanArgs& a, int cap) {
  return RtLayout(cap, a.R, next_pow2(a.R), a.d, a.nprobe).total;
}

void launch_ivfpq_scan_rt(FastScanArgs a, cudaStream_t s, int nt, int persistent_ctas) {
  if (a.nq == 0) return;
  MV_REQUIRE(ivfpq_rt_supported(a), MV_ERR_INTERNAL, "rotated-table scan: unsupported shape");
  MV_REQUIRE(!a.counter || persistent_ctas > 0, MV_ERR_INTERNAL, "persistent scan without a grid");
  a.Rp = next_pow2(a.R);
  const int threads = nt >= 512 ? 512 : 256;
  // staging area: the most candidates per chunk (at most 8192, at least
  // 2 R) within the shared memory that lets 1024 / threads CTAs share an SM
  const size_t budget = threads == 512 ? 110 * 1024 : 54 * 1024;
  int cap = 8192;
  while (cap > 512 && ivfpq_rt_smem(a, cap) > budget) cap -= 256;
  cap = std::max(cap, 2 * a.R);
  a.cap = cap;
  const size_t smem = ivfpq_rt_smem(a, cap);
  MV_REQUIRE(smem <= 220 * 1024, MV_ERR_UNSUPPORTED, "rotated-table scan: nprobe or d too large");
  const unsigned grid =
      a.counter ? (unsigned)std::min<int64_t>(persistent_ctas, a.nq) : (unsigned)a.nq;
  auto go = [&](auto kernel) {
    smem_limit(kernel, smem);
    kernel<<<grid, threads, smem, s>>>(a);
  };
  const int S = rt_pass_width(a.M);
  if (threads == 512) {
    if (S == 8) go(k_ivfpq_scan_rt<512, 8>);
    else if (S == 16) go(k_ivfpq_scan_rt<512, 16>);
    else go(k_ivfpq_scan_rt<512, 32>);
  } else {
    if (S == 8) go(k_ivfpq_scan_rt<256, 8>);
    else if (S == 16) go(k_ivfpq_scan_rt<256, 16>);
    else go(k_ivfpq_scan_rt<256, 32>);
  }
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
