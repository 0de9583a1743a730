// List-major IVF-PQ ADC scan on the tensor cores (fast form).
//
// The fast form ranks a candidate y of list c for query q by
//   ||q - c||^2 + (||y||^2 + 2<c, y>) - 2<q, y>          (L2)
//   -<q, c> - <q, y>                                      (IP)
// (index/index_ivf_pq.mojo:306-347 expanded; y is the PQ reconstruction of
// the residual). The per-query-table scan evaluates <q, y> as M table
// lookups per (query, candidate). Here the probed (query, list) pairs are
// grouped by list on the device and, per tile of 128 list rows, the rows'
// codes are decoded once into FP16 reconstructions in shared memory and
// multiplied with every probing query on the tensor cores
// (tcgen05.mma kind::f16, FP16 x FP16 -> FP32 in TMEM). The table lookups
// per (query, candidate) become one decode per list row and batch.
//
// Pipeline (one stream, no host reads):
//   k_tc_q16      queries -> FP16 rows scaled by a power of two per query
//   k_tc_pairs    per (query, probe): its candidates' offset in the query's
//                 distance row (the probed lists laid end to end, as the
//                 per-query scan numbers them); counts pairs per list
//   k_tc_items    work items per list: chunks of at most qc queries x
//                 pieces of at most TC_RS rows (long lists are split)
//   k_tc_place    pairs grouped by list
//   k_tc_scan     persistent tensor-core kernel, one CTA per SM, items from
//                 an atomic counter: ordered FP32 distances into the
//                 per-query distance rows
//   k_tc_select   one warp per query: the R smallest (distance, position)
//                 keys of its row, by min/max, 256-bin histogram passes
//                 over the row and a sort of the boundary bin's keys
//   k_tc_sort     (shortlist is the answer) rows sorted ascending
//
// The distance rows hold the distance as an order-preserving word; a row
// whose id the exclusion filter names (index_ivf_pq.mojo:328-334) holds
// TC_EXCLUDED and never enters the shortlist. Results depend only on the
// data, not on the grouping order or launch shape: every (query, row)
// distance is computed by one MMA column with the same operands, and the
// selection returns the R smallest keys whatever the order it reads them in.
#include <cuda_fp16.h>

#include "mv_fast.h"
#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_select.cuh"
#include "mv_sm100.cuh"

namespace mv {
namespace {

using namespace sm100;

constexpr int TC_THREADS = 256;  // 8 warps: two per TMEM lane quarter
constexpr int TC_BM = 128;       // list rows per tile (UMMA M)
constexpr int TC_RS = 1024;      // list rows per work item
constexpr uint32_t TC_EXCLUDED = 0xffffffffu;

// Instruction descriptor of tcgen05.mma kind::f16 with FP16 A and B
// (format code 0), FP32 D, both K-major, tile m x n.
__host__ __device__ constexpr uint32_t idesc_f16_f32(int m, int n) {
  return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Byte offset of 16-byte chunk c (0..7) of row r in a K-major tile stored
// with the 128-byte swizzle (8-row atoms of 1024 bytes).
__device__ __forceinline__ uint32_t sw128(int r, int c) {
  return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
}

// ---- queries -> FP16 ------------------------------------------------------
// One warp per query: e with max|q| * 2^e in [2^14, 2^15) (no FP16
// overflow), rows zero padded to kp; qmul = mul * 2^-e undoes the scale and
// applies the table scale (-2 L2, -1 IP) and the codebook's 1 / scale. A
// non-finite query keeps e = 0 and yields non-finite distances.
__global__ void __launch_bounds__(256) k_tc_q16(const float* __restrict__ q, int64_t nq, int d,
                                                int kp, float mul, __half* __restrict__ q16,
                                                float* __restrict__ qmul) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  if (row >= nq) return;
  const float* x = q + row * d;
  float mx = 0.0f;
  bool bad = false;
  for (int j = lane; j < d; j += 32) {
    const float a = fabsf(x[j]);
    bad = bad || !(a <= 3.4028235e38f);
    mx = fmaxf(mx, a);
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  bad = __any_sync(0xffffffffu, bad);
  int e = 0;
  if (!bad && mx > 0.0f) e = min(max(14 - ilogbf(mx), -126), 126);
  const float sc = __int_as_float((127 + e) << 23);
  for (int j = lane; j < kp; j += 32) q16[row * kp + j] = __float2half_rn(j < d ? x[j] * sc : 0.0f);
  if (lane == 0) qmul[row] = mul * __int_as_float((127 - e) << 23);
}

// ---- (query, probe) pairs ----------------------------------------------
// One warp per query: seg[q * P + p] = q * smax + (candidates of the probes
// before p), cnt[list] += 1 per probe. Probes at or past the query's own
// nprobe take no part.
__global__ void __launch_bounds__(256)
    k_tc_pairs(const int32_t* __restrict__ probes, int64_t nq, int P,
               const int32_t* __restrict__ nprobe_q, const int64_t* __restrict__ list_off,
               int nlist, int64_t smax, int64_t* __restrict__ seg, int* __restrict__ cnt,
               int* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  if (row >= nq) return;
  const int np = nprobe_q ? min(max(nprobe_q[row], 1), P) : P;
  // smax bounds the candidates of np distinct lists; a query over it (never
  // expected) takes no part: seg -1 (the placement skips it), error site 106
  int64_t tot = 0;
  for (int p = lane; p < np; p += 32) {
    const int L = probes[row * P + p];
    if (L >= 0 && L < nlist) tot += list_off[L + 1] - list_off[L];
  }
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  if (tot > smax) {
    for (int p = lane; p < np; p += 32) seg[row * P + p] = -1;
    if (lane == 0) atomicExch(err, 106);
    return;
  }
  int64_t carry = 0;
  for (int p0 = 0; p0 < np; p0 += 32) {
    const int p = p0 + lane;
    int64_t len = 0;
    int L = -1;
    if (p < np) {
      L = probes[row * P + p];
      if (L >= nlist) {
        atomicExch(err, 103);
        L = -1;
      }
      if (L >= 0) len = list_off[L + 1] - list_off[L];
    }
    int64_t incl = len;
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (p < np) {
      seg[row * P + p] = row * smax + carry + incl - len;
      if (L >= 0) atomicAdd(&cnt[L], 1);
    }
    carry += __shfl_sync(0xffffffffu, incl, 31);
  }
}

// Exclusive scans over the lists of the pair counts (start) and of the
// work items (istart): cnt[L] > 0 pairs give ceil(cnt / qc) query chunks
// times ceil(len / TC_RS) row pieces. One block of 1024 threads.
__global__ void __launch_bounds__(1024)
    k_tc_items(const int* __restrict__ cnt, const int64_t* __restrict__ list_off, int nlist, int qc,
               int64_t* __restrict__ start, int* __restrict__ istart) {
  __shared__ long long ws1[32];
  __shared__ int ws2[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int per = (nlist + 1023) / 1024;
  const int b0 = min(nlist, t * per), b1 = min(nlist, b0 + per);
  auto items = [&](int L) {
    const int c = cnt[L];
    const int64_t len = list_off[L + 1] - list_off[L];
    if (c == 0 || len == 0) return 0;
    return ((c + qc - 1) / qc) * (int)((len + TC_RS - 1) / TC_RS);
  };
  long long s1 = 0;
  int s2 = 0;
  for (int L = b0; L < b1; ++L) {
    s1 += cnt[L];
    s2 += items(L);
  }
  long long i1 = s1;
  int i2 = s2;
  for (int o = 1; o < 32; o <<= 1) {
    const long long a = __shfl_up_sync(0xffffffffu, i1, o);
    const int b = __shfl_up_sync(0xffffffffu, i2, o);
    if (lane >= o) {
      i1 += a;
      i2 += b;
    }
  }
  if (lane == 31) {
    ws1[w] = i1;
    ws2[w] = i2;
  }
  __syncthreads();
  if (w == 0) {
    long long a = ws1[lane];
    int b = ws2[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const long long x = __shfl_up_sync(0xffffffffu, a, o);
      const int y = __shfl_up_sync(0xffffffffu, b, o);
      if (lane >= o) {
        a += x;
        b += y;
      }
    }
    ws1[lane] = a;
    ws2[lane] = b;
  }
  __syncthreads();
  long long base1 = (w ? ws1[w - 1] : 0) + i1 - s1;
  int base2 = (w ? ws2[w - 1] : 0) + i2 - s2;
  for (int L = b0; L < b1; ++L) {
    start[L] = base1;
    istart[L] = base2;
    base1 += cnt[L];
    base2 += items(L);
  }
  if (t == 1023) {
    start[nlist] = ws1[31];
    istart[nlist] = ws2[31];
  }
}

__global__ void k_tc_place(const int32_t* __restrict__ probes, int64_t nq, int P,
                           const int32_t* __restrict__ nprobe_q, int nlist,
                           const int64_t* __restrict__ seg, const int64_t* __restrict__ start,
                           int* __restrict__ cursor, int32_t* __restrict__ pairs) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq * P) return;
  const int64_t row = i / P;
  const int p = (int)(i - row * P);
  const int np = nprobe_q ? min(max(nprobe_q[row], 1), P) : P;
  if (p >= np || seg[i] < 0) return;
  const int L = probes[i];
  if (L >= 0 && L < nlist) pairs[start[L] + atomicAdd(&cursor[L], 1)] = (int32_t)i;
}

// ---- the tensor-core scan -------------------------------------------------
struct TcArgs {
  const __half* q16;
  const float* qmul;
  const float* term;      // nq x P coarse terms
  const int64_t* seg;     // nq x P distance-row offsets
  const int* cnt;
  const int64_t* start;
  const int* istart;
  const int32_t* pairs;
  const int64_t* list_off;
  const uint8_t* codes;
  const float* vterm;     // per CSR row (L2), null for IP
  const __half* pq16;     // M x 256 x dsub FP16 codebook (scaled)
  const uint8_t* filter;
  int64_t filter_len;
  const uint32_t* ids;
  uint32_t* dist;         // distance rows
  int* counter;
  int* err;
  int nlist, P, M, dsub, d, kp, qc;
  long long wait_limit;
};

struct TcSmem {
  int abytes, bbytes, cbbytes;
  __host__ __device__ TcSmem(int kp, int qc, int d)
      : abytes(TC_BM * kp * 2), bbytes(qc * kp * 2), cbbytes(d * 512) {}
  __host__ __device__ int a_off(int b) const { return b * abytes; }
  __host__ __device__ int b_off(int b) const { return 2 * abytes + b * bbytes; }
  __host__ __device__ int cb_off() const { return 2 * abytes + 2 * bbytes; }
  __host__ __device__ int meta_off() const { return cb_off() + cbbytes; }
  // per buffer and column: seg (8 bytes), term, qmul
  __host__ __device__ int bars_off(int qc) const { return meta_off() + 2 * qc * 16; }
  __host__ __device__ size_t total(int qc) const { return 1024 + (size_t)bars_off(qc) + 64; }
};

// Persistent: one CTA per SM takes work items (list, query chunk, row
// piece) from a counter. Per item the chunk's FP16 query rows go to B[item
// parity]; per 128-row tile of the piece all eight warps decode the rows'
// codes into A[tile parity] (thread r of a lane quarter owns row r, the two
// warps of a quarter split the subspaces), one thread issues the d / 16
// MMAs into accumulator (tile parity) and commits, and the warps then run
// the epilogue of the PREVIOUS tile (its MMA overlaps this tile's decode):
// distance = term + vterm + qmul * acc, one coalesced 128-byte store per
// warp and query column.
__global__ void __launch_bounds__(TC_THREADS, 1) k_tc_scan(TcArgs a) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                           ~uintptr_t(1023));
  const TcSmem L(a.kp, a.qc, a.d);
  uint8_t* cb = sm + L.cb_off();
  int64_t* mseg = reinterpret_cast<int64_t*>(sm + L.meta_off());  // [2][qc]
  float* mterm = reinterpret_cast<float*>(mseg + 2 * a.qc);        // [2][qc]
  float* mmul = mterm + 2 * a.qc;                                  // [2][qc]
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + L.bars_off(a.qc));
  uint32_t* holder = reinterpret_cast<uint32_t*>(bars + 2);
  __shared__ int s_item, s_L, s_nq, s_err;
  __shared__ long long s_rbeg, s_rend, s_pb;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int qc = a.qc, kp = a.kp, M = a.M, dsub = a.dsub;
  const uint32_t bar0 = smem_u32(bars);
  if (tid == 0) {
    s_err = 0;
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(smem_u32(holder), 2 * qc);
  // the codebook, once per CTA
  {
    const uint4* src = reinterpret_cast<const uint4*>(a.pq16);
    uint4* dst = reinterpret_cast<uint4*>(cb);
    for (int i = tid; i < L.cbbytes / 16; i += TC_THREADS) dst[i] = __ldg(src + i);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(holder);
  volatile int* verr = &s_err;
  const int total_items = a.istart[a.nlist];

  const int lq = warp & 3, half = warp >> 2;
  const int r = lq * 32 + lane;  // this thread's tile row (decode and epilogue)
  const int msplit = M >> 1;
  const int m0 = half * msplit;
  // the previous tile, waiting for its epilogue
  bool have_prev = false;
  int prev_g = 0, prev_ib = 0, prev_nq = 0, prev_nr = 0, prev_npad = 16;
  int64_t prev_row0 = 0;
  float prev_v = 0.0f;
  bool prev_ex = false;
  int g = 0, ic = 0;
  int last_commit = -1;  // thread 0: index of the last committed tile

  auto epilogue = [&]() {
    const int buf = prev_g & 1;
    bool ok = !*verr && mbar_wait(bar0 + 8u * buf, (uint32_t)(prev_g >> 1) & 1u, a.wait_limit);
    if (!__all_sync(0xffffffffu, ok)) {
      *verr = 1;
      return;
    }
    tc_fence_after();
    const int64_t* sg = mseg + prev_ib * qc;
    const float* tm = mterm + prev_ib * qc;
    const float* mu = mmul + prev_ib * qc;
    const bool row_ok = r < prev_nr;
    for (int cg = half; cg * 16 < prev_npad; cg += 2) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)(buf * qc + cg * 16), v);
      if (row_ok) {
#pragma unroll
        for (int jj = 0; jj < 16; ++jj) {
          const int j = cg * 16 + jj;
          if (j < prev_nq) {
            const float dd = fmaf(v[jj], mu[j], tm[j] + prev_v);
            uint32_t o = float_to_ordered(dd);
            o = o == TC_EXCLUDED ? TC_EXCLUDED - 1u : o;  // a NaN stays a candidate
            a.dist[sg[j] + prev_row0 + r] = prev_ex ? TC_EXCLUDED : o;
          }
        }
      }
    }
    tc_fence_before();
  };

  while (true) {
    if (tid == 0) {
      const int it = atomicAdd(a.counter, 1);
      s_item = it;
      if (it < total_items) {
        int lo = 0, hi = a.nlist - 1;  // the list with istart[lo] <= it < istart[lo + 1]
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (a.istart[mid] <= it) lo = mid;
          else hi = mid - 1;
        }
        const int64_t len = a.list_off[lo + 1] - a.list_off[lo];
        const int nseg = (int)((len + TC_RS - 1) / TC_RS);
        const int c = it - a.istart[lo];
        const int chunk = c / nseg, piece = c - chunk * nseg;
        s_L = lo;
        s_rbeg = (int64_t)piece * TC_RS;
        s_rend = min(len, (int64_t)(piece + 1) * TC_RS);
        s_pb = a.start[lo] + (int64_t)chunk * qc;
        s_nq = min(qc, a.cnt[lo] - chunk * qc);
      }
    }
    const bool stop = __syncthreads_or(*verr);  // one answer for every thread
    if (s_item >= total_items || stop) break;
    const int ib = ic & 1;
    const int Lst = s_L, nqi = s_nq;
    const int64_t rbeg = s_rbeg, rend = s_rend, pb = s_pb;
    const int64_t loff = a.list_off[Lst];
    const int npad = max(16, (nqi + 15) & ~15);
    // B[ib]: the chunk's query rows; meta[ib]: per column offset, term, scale
    {
      uint8_t* B = sm + L.b_off(ib);
      const int cpr = kp >> 3;  // 16-byte chunks per row
      for (int i = tid; i < nqi * cpr; i += TC_THREADS) {
        const int j = i / cpr, c = i - j * cpr;
        const int64_t pr = a.pairs[pb + j];
        const int64_t qrow = pr / a.P;
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(a.q16 + qrow * kp) + c);
        *reinterpret_cast<uint4*>(B + (c >> 3) * (qc * 128) + sw128(j, c & 7)) = v;
      }
      if (tid < nqi) {
        const int64_t pr = a.pairs[pb + tid];
        mseg[ib * qc + tid] = a.seg[pr];  // + row within the list = the row's slot
        mterm[ib * qc + tid] = a.term[pr];
        mmul[ib * qc + tid] = a.qmul[pr / a.P];
      }
    }
    for (int64_t row0 = rbeg; row0 < rend; row0 += TC_BM) {
      const int nr = (int)min((int64_t)TC_BM, rend - row0);
      const int buf = g & 1;
      uint8_t* A = sm + L.a_off(buf);
      float cur_v = 0.0f;
      bool cur_ex = false;
      if (r < nr) {
        const int64_t pos = loff + row0 + r;
        const uint8_t* crow = a.codes + pos * M + m0;
        for (int w0 = 0; w0 < msplit; w0 += 4) {
          const uint32_t word = __ldg(reinterpret_cast<const uint32_t*>(crow + w0));
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int m = m0 + w0 + b;
            const uint32_t code = (word >> (8 * b)) & 255u;
            if (dsub == 8) {
              const uint4 cw = *reinterpret_cast<const uint4*>(cb + ((m << 8) + code) * 16);
              *reinterpret_cast<uint4*>(A + (m >> 3) * (TC_BM * 128) + sw128(r, m & 7)) = cw;
            } else {  // dsub 4: half a chunk per subspace
              const uint2 cw = *reinterpret_cast<const uint2*>(cb + ((m << 8) + code) * 8);
              *reinterpret_cast<uint2*>(A + (m >> 4) * (TC_BM * 128) + sw128(r, (m >> 1) & 7) +
                                        (m & 1) * 8) = cw;
            }
          }
        }
        if (a.vterm) cur_v = __ldg(a.vterm + pos);
        if (a.filter) {
          const uint32_t id = a.ids[pos];
          cur_ex = (int64_t)id < a.filter_len && a.filter[id] != 0;
        }
      }
      fence_proxy_async();
      if (__syncthreads_or(*verr)) break;  // one answer for every thread
      if (tid == 0) {
        tc_fence_after();
        const uint32_t dt = tmem + (uint32_t)(buf * qc);
        const uint32_t idesc = idesc_f16_f32(TC_BM, npad);
        const uint32_t abase = smem_u32(A), bbase = smem_u32(sm + L.b_off(ib));
        const int ks = a.d >> 4;
        for (int s = 0; s < ks; ++s) {
          const int kb = s >> 2, kk = s & 3;
          const uint64_t ad = desc_k_sw128(abase + kb * (TC_BM * 128)) + 2u * kk;
          const uint64_t bd = desc_k_sw128(bbase + kb * (qc * 128)) + 2u * kk;
          umma_f16(dt, ad, bd, idesc, s > 0 ? 1u : 0u);
        }
        umma_commit(bar0 + 8u * buf);
        last_commit = g;
      }
      if (have_prev) epilogue();
      have_prev = true;
      prev_g = g;
      prev_ib = ib;
      prev_nq = nqi;
      prev_nr = nr;
      prev_npad = npad;
      prev_row0 = row0;
      prev_v = cur_v;
      prev_ex = cur_ex;
      ++g;
    }
    ++ic;
  }
  if (have_prev && !*verr) epilogue();
  __syncthreads();
  // Unwind: the last issued MMAs retire before TMEM is freed (full limit).
  if (tid == 0 && last_commit >= 0) {
    if (!mbar_wait(bar0 + 8u * (last_commit & 1), (uint32_t)(last_commit >> 1) & 1u)) *verr = 1;
  }
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 2 * qc);
  }
  if (tid == 0 && *verr) atomicExch(a.err, 1);
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

// One warp per query. The query's candidates are its distance row's first
// n words, probe by probe; candidate i of probe p is CSR row
// off[p] + (i - beg[p]) and its key is (word << 32) | row. Pass 1 finds the
// valid keys' count, min and max; histogram passes over the keys still in
// play narrow [lo, hi] to the bin holding the R-th key (256 linear bins per
// pass) until that bin holds at most SEL_SIDE keys; the last pass writes
// every key below the bin and stages the bin's keys, which one warp sort
// orders to fill the shortlist. The shortlist is written unsorted in a
// fixed order (the row order of the passes).
__global__ void __launch_bounds__(SEL_WARPS * 32) k_tc_select(SelArgs a) {
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
        w[u] = i < n ? __ldg(src + i) : TC_EXCLUDED;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = i0 + lane + 32 * u;
        bool valid = false;
        uint64_t key = KEY_NONE;
        if (i < n) {
          while (pbeg[p + 1] <= i) ++p;
          valid = w[u] != TC_EXCLUDED;
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

// Rows of R keys sorted ascending in place (KEY_NONE padded to Rp in
// shared memory).
__global__ void __launch_bounds__(256) k_tc_sort(uint64_t* keys, int R, int Rp) {
  extern __shared__ __align__(16) uint64_t sk[];
  uint64_t* rowp = keys + (int64_t)blockIdx.x * R;
  for (int i = threadIdx.x; i < Rp; i += 256) sk[i] = i < R ? rowp[i] : KEY_NONE;
  block_bitonic_sort(sk, Rp);
  for (int i = threadIdx.x; i < R; i += 256) rowp[i] = sk[i];
}

size_t al(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

bool ivfpq_tc_supported(int d, int M, bool has_pq16) {
  const int dsub = M > 0 ? d / M : 0;
  return has_pq16 && M % 8 == 0 && (dsub == 4 || dsub == 8) && d % 32 == 0 && d <= 128;
}

int ivfpq_tc_qc(int64_t nq, int nprobe, int nlist) {
  const double per_list = (double)nq * nprobe / (nlist > 0 ? nlist : 1);
  return per_list > 48.0 ? 128 : per_list > 20.0 ? 64 : 32;
}

size_t ivfpq_tc_scratch_bytes(int64_t nq, int nprobe, int nlist, int d, int64_t smax) {
  const int kp = (d + 63) / 64 * 64;
  return al((size_t)nq * kp * 2) + al((size_t)nq * 4) + al((size_t)nq * nprobe * 8) +
         3 * al((size_t)(nlist + 1) * 4) + al((size_t)(nlist + 1) * 8) +
         al((size_t)nq * nprobe * 4) + al(16) + al((size_t)nq * smax * 4);
}

void launch_ivfpq_scan_tc(const FastScanArgs& f, int64_t smax, int qc, void* scratch, int num_sms,
                          long long wait_limit, cudaStream_t s) {
  const int64_t nq = f.nq;
  if (nq == 0) return;
  const int d = f.d, M = f.M, P = f.nprobe, nlist = f.nlist;
  MV_REQUIRE(f.pq16 && ivfpq_tc_supported(d, M, true), MV_ERR_INTERNAL,
             "tensor-core ADC scan: unsupported shape");
  MV_REQUIRE(qc == 32 || qc == 64 || qc == 128, MV_ERR_INTERNAL, "tensor-core ADC scan: bad chunk");
  MV_REQUIRE(nq * P < (1ll << 31) && smax < (1ll << 31), MV_ERR_UNSUPPORTED,
             "tensor-core ADC scan: batch too large");
  const int kp = (d + 63) / 64 * 64;
  unsigned char* p = static_cast<unsigned char*>(scratch);
  auto take = [&](size_t bytes) {
    unsigned char* r = p;
    p += al(bytes);
    return r;
  };
  __half* q16 = reinterpret_cast<__half*>(take((size_t)nq * kp * 2));
  float* qmul = reinterpret_cast<float*>(take((size_t)nq * 4));
  int64_t* seg = reinterpret_cast<int64_t*>(take((size_t)nq * P * 8));
  int* cnt = reinterpret_cast<int*>(take((size_t)(nlist + 1) * 4));
  int* cursor = reinterpret_cast<int*>(take((size_t)(nlist + 1) * 4));
  int* istart = reinterpret_cast<int*>(take((size_t)(nlist + 1) * 4));
  int64_t* start = reinterpret_cast<int64_t*>(take((size_t)(nlist + 1) * 8));
  int32_t* pairs = reinterpret_cast<int32_t*>(take((size_t)nq * P * 4));
  int* counter = reinterpret_cast<int*>(take(16));
  uint32_t* dist = reinterpret_cast<uint32_t*>(take((size_t)nq * smax * 4));
  MV_CHECK_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * (nlist + 1), s));
  MV_CHECK_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int) * (nlist + 1), s));
  MV_CHECK_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), s));
  const float scale = f.metric == MV_METRIC_L2 ? -2.0f : -1.0f;
  const unsigned gw = (unsigned)((nq + 7) / 8);
  k_tc_q16<<<gw, 256, 0, s>>>(f.q, nq, d, kp, scale * f.pq16_inv, q16, qmul);
  k_tc_pairs<<<gw, 256, 0, s>>>(f.probes, nq, P, f.nprobe_q, f.list_off, nlist, smax, seg, cnt,
                                f.err);
  k_tc_items<<<1, 1024, 0, s>>>(cnt, f.list_off, nlist, qc, start, istart);
  k_tc_place<<<(unsigned)((nq * P + 255) / 256), 256, 0, s>>>(f.probes, nq, P, f.nprobe_q, nlist,
                                                               seg, start, cursor, pairs);
  for (int i = 0; i < 4; ++i) count_launch();
  TcArgs t;
  t.q16 = q16;
  t.qmul = qmul;
  t.term = f.term;
  t.seg = seg;
  t.cnt = cnt;
  t.start = start;
  t.istart = istart;
  t.pairs = pairs;
  t.list_off = f.list_off;
  t.codes = f.codes;
  t.vterm = f.vterm;
  t.pq16 = f.pq16;
  t.filter = f.filter;
  t.filter_len = f.filter_len;
  t.ids = f.ids;
  t.dist = dist;
  t.counter = counter;
  t.err = f.err;
  t.nlist = nlist;
  t.P = P;
  t.M = M;
  t.dsub = d / M;
  t.d = d;
  t.kp = kp;
  t.qc = qc;
  t.wait_limit = wait_limit;
  const size_t smem = TcSmem(kp, qc, d).total(qc);
  smem_limit(k_tc_scan, smem);
  k_tc_scan<<<(unsigned)num_sms, TC_THREADS, smem, s>>>(t);
  count_launch();
  SelArgs sa;
  sa.dist = dist;
  sa.smax = smax;
  sa.probes = f.probes;
  sa.nprobe_q = f.nprobe_q;
  sa.list_off = f.list_off;
  sa.P = P;
  sa.nlist = nlist;
  sa.R = f.R;
  sa.nq = nq;
  sa.out = f.out_keys;
  sa.err = f.err;
  const size_t ssm = sel_warp_bytes(P) * SEL_WARPS;
  MV_REQUIRE(ssm <= 200 * 1024, MV_ERR_UNSUPPORTED, "tensor-core ADC scan: nprobe too large");
  smem_limit(k_tc_select, ssm);
  k_tc_select<<<(unsigned)((nq + SEL_WARPS - 1) / SEL_WARPS), SEL_WARPS * 32, ssm, s>>>(sa);
  count_launch();
  if (f.sorted) {
    const int Rp = next_pow2(f.R);
    MV_REQUIRE((size_t)Rp * 8 <= 200 * 1024, MV_ERR_UNSUPPORTED, "shortlist too long to sort");
    smem_limit(k_tc_sort, (size_t)Rp * 8);
    k_tc_sort<<<(unsigned)nq, 256, (size_t)Rp * 8, s>>>(f.out_keys, f.R, Rp);
    count_launch();
  }
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
