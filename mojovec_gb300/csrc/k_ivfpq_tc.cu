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

// One work item: rows [rbeg, rend) of list L (at CSR offset loff) against
// query chunk `chunk` (nq queries, their FP16 rows and column data in the
// chunk's images).
struct TcItem {
  int L, nq, chunk, pad;
  long long loff, rbeg, rend;
};

// Per query column of a chunk: the distance-row offset of its probe of the
// list, the coarse term and the scale of its accumulators.
struct TcMeta {
  long long seg;
  float term, qmul;
};

// Exclusive scans over the lists of the pair counts (start), the query
// chunks (cstart: ceil(cnt / qc)) and the work items (istart: chunks times
// ceil(len / TC_RS) row pieces). One block of 1024 threads.
__global__ void __launch_bounds__(1024)
    k_tc_items(const int* __restrict__ cnt, const int64_t* __restrict__ list_off, int nlist, int qc,
               int64_t* __restrict__ start, int* __restrict__ cstart, int* __restrict__ istart) {
  __shared__ long long ws1[32];
  __shared__ int ws2[32], ws3[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int per = (nlist + 1023) / 1024;
  const int b0 = min(nlist, t * per), b1 = min(nlist, b0 + per);
  auto chunks = [&](int L) { return (cnt[L] + qc - 1) / qc; };
  auto pieces = [&](int L) {
    const int64_t len = list_off[L + 1] - list_off[L];
    return (int)((len + TC_RS - 1) / TC_RS);
  };
  long long s1 = 0;
  int s2 = 0, s3 = 0;
  for (int L = b0; L < b1; ++L) {
    s1 += cnt[L];
    s2 += chunks(L) * pieces(L);
    s3 += chunks(L);
  }
  long long i1 = s1;
  int i2 = s2, i3 = s3;
  for (int o = 1; o < 32; o <<= 1) {
    const long long a = __shfl_up_sync(0xffffffffu, i1, o);
    const int b = __shfl_up_sync(0xffffffffu, i2, o);
    const int c = __shfl_up_sync(0xffffffffu, i3, o);
    if (lane >= o) {
      i1 += a;
      i2 += b;
      i3 += c;
    }
  }
  if (lane == 31) {
    ws1[w] = i1;
    ws2[w] = i2;
    ws3[w] = i3;
  }
  __syncthreads();
  if (w == 0) {
    long long a = ws1[lane];
    int b = ws2[lane], c = ws3[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const long long x = __shfl_up_sync(0xffffffffu, a, o);
      const int y = __shfl_up_sync(0xffffffffu, b, o);
      const int z = __shfl_up_sync(0xffffffffu, c, o);
      if (lane >= o) {
        a += x;
        b += y;
        c += z;
      }
    }
    ws1[lane] = a;
    ws2[lane] = b;
    ws3[lane] = c;
  }
  __syncthreads();
  long long base1 = (w ? ws1[w - 1] : 0) + i1 - s1;
  int base2 = (w ? ws2[w - 1] : 0) + i2 - s2;
  int base3 = (w ? ws3[w - 1] : 0) + i3 - s3;
  for (int L = b0; L < b1; ++L) {
    start[L] = base1;
    istart[L] = base2;
    cstart[L] = base3;
    base1 += cnt[L];
    base2 += chunks(L) * pieces(L);
    base3 += chunks(L);
  }
  if (t == 1023) {
    start[nlist] = ws1[31];
    istart[nlist] = ws2[31];
    cstart[nlist] = ws3[31];
  }
}

// Every list's work-item records, one thread per list.
__global__ void k_tc_fill(const int* __restrict__ cnt, const int64_t* __restrict__ list_off, int nlist,
                          int qc, const int* __restrict__ cstart, const int* __restrict__ istart,
                          TcItem* __restrict__ items) {
  const int L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= nlist) return;
  const int c = cnt[L];
  const int64_t loff = list_off[L], len = list_off[L + 1] - loff;
  if (c == 0 || len == 0) return;
  const int nch = (c + qc - 1) / qc, npc = (int)((len + TC_RS - 1) / TC_RS);
  const int i0 = istart[L], c0 = cstart[L];
  for (int ch = 0; ch < nch; ++ch) {
    for (int pc = 0; pc < npc; ++pc) {
      TcItem it;
      it.L = L;
      it.nq = min(qc, c - ch * qc);
      it.chunk = c0 + ch;
      it.pad = 0;
      it.loff = loff;
      it.rbeg = (long long)pc * TC_RS;
      it.rend = min(len, (int64_t)(pc + 1) * TC_RS);
      items[i0 + ch * npc + pc] = it;
    }
  }
}

// Groups the pairs by list and writes each chunk's images: the FP16 query
// rows in the MMA's B layout (K-major, 128-byte swizzle, k-block major:
// image[kb][j][128 bytes]) and the column data. A pair's column j within
// its list is taken by an atomic, so the order of the columns varies; every
// column is computed the same way.
__global__ void k_tc_place(const int32_t* __restrict__ probes, int64_t nq, int P,
                           const int32_t* __restrict__ nprobe_q, int nlist,
                           const int64_t* __restrict__ seg, const float* __restrict__ term,
                           const __half* __restrict__ q16, const float* __restrict__ qmul, int kp,
                           int qc, const int* __restrict__ cstart, int* __restrict__ cursor,
                           uint8_t* __restrict__ bimg, TcMeta* __restrict__ meta) {
  // 16 threads per pair: the group's first thread takes the column, each
  // thread copies one 16-byte chunk of the query row (kp <= 128)
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i = gt >> 4;
  const int cc = (int)(gt & 15);
  const int lane = threadIdx.x & 31;
  const unsigned gmask = 0xffffu << (lane & 16);
  bool on = i < nq * P;
  int64_t row = 0;
  int L = -1;
  if (on) {
    row = i / P;
    const int p = (int)(i - row * P);
    const int np = nprobe_q ? min(max(nprobe_q[row], 1), P) : P;
    L = probes[i];
    on = p < np && seg[i] >= 0 && L >= 0 && L < nlist;
  }
  int c = 0;
  if (on && cc == 0) c = atomicAdd(&cursor[L], 1);
  c = __shfl_sync(gmask, c, lane & 16);
  if (!on) return;
  const int64_t chunk = cstart[L] + c / qc;
  const int j = c % qc;
  if (cc == 0) {
    TcMeta m;
    m.seg = seg[i];
    m.term = term[i];
    m.qmul = qmul[row];
    meta[chunk * qc + j] = m;
  }
  if (cc < (kp >> 3)) {
    uint8_t* img = bimg + chunk * ((int64_t)qc * kp * 2);
    *reinterpret_cast<uint4*>(img + (cc >> 3) * (qc * 128) + sw128(j, cc & 7)) =
        reinterpret_cast<const uint4*>(q16 + row * kp)[cc];
  }
}

// excl[pos] = 1 when the exclusion filter names the id of CSR row pos.
__global__ void k_tc_excl(const uint32_t* __restrict__ ids, int64_t ntotal,
                          const uint8_t* __restrict__ filter, int64_t filter_len,
                          uint8_t* __restrict__ excl) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ntotal) return;
  const uint32_t id = ids[i];
  excl[i] = ((int64_t)id < filter_len && filter[id] != 0) ? 1 : 0;
}

// ---- the tensor-core scan -------------------------------------------------
// Warp roles of one CTA: 0-7 decode, 8-15 epilogue, 16 MMA (and TMEM
// owner), 17 producer.
constexpr int TC_DEC_WARPS = 8;
constexpr int TC_EPI_WARPS = 8;
constexpr int TC_MMA_WARP = 16;
constexpr int TC_PROD_WARP = 17;
constexpr int TC_THREADS = 18 * 32;
constexpr int TC_STAGES = 5;  // tiles of codes in flight
constexpr int TC_NB = 4;      // items in flight (query images), at most

struct TcArgs {
  const TcItem* items;
  const int* total_items;  // device word: the item count
  const uint8_t* bimg;     // chunk images of the B operand
  const TcMeta* meta;      // chunk column data
  const uint8_t* codes;    // CSR codes (16 bytes of slack at the end)
  const float* vterm;      // per CSR row (L2; 16 bytes of slack), null for IP
  const uint8_t* excl;     // per CSR row (16 bytes of slack), null without a filter
  const __half* pq16;      // M x 256 x dsub FP16 codebook (scaled)
  uint32_t* dist;          // distance rows
  int* err;
  int M, dsub, d, kp, qc;
  int nb;  // query-image buffers (2 .. TC_NB)
  long long wait_limit;
};

struct TcSmem {
  int nb, abytes, bbytes, mbytes, cbbytes, code_bytes, slot_bytes;
  __host__ __device__ TcSmem(int kp, int qc, int d, int M, int nb_)
      : nb(nb_), abytes(TC_BM * kp * 2), bbytes(qc * kp * 2), mbytes(qc * 16), cbbytes(d * 512),
        code_bytes((TC_BM * M + 32 + 15) & ~15), slot_bytes(code_bytes + 544 + 160) {}
  __host__ __device__ int a_off(int b) const { return b * abytes; }
  __host__ __device__ int b_off(int b) const { return 2 * abytes + b * bbytes; }
  __host__ __device__ int m_off(int b) const { return 2 * abytes + nb * bbytes + b * mbytes; }
  __host__ __device__ int cb_off() const { return 2 * abytes + nb * bbytes + nb * mbytes; }
  __host__ __device__ int slot_off(int s) const { return cb_off() + cbbytes + s * slot_bytes; }
  __host__ __device__ int bars_off() const { return slot_off(TC_STAGES); }
  static constexpr int kBars = 2 * TC_NB + 8 + 2 * TC_STAGES;
  __host__ __device__ size_t total() const { return 1024 + (size_t)bars_off() + 8 * kBars + 16; }
};

// Persistent: one CTA per SM walks the work items blockIdx.x, + gridDim.x,
// ... and every role walks the same items and 128-row tiles in the same
// order, handing them on through mbarriers:
//   producer  cp.async.bulk of each item's query image and column data into
//             B[item % nb] and of each tile's codes, per-row terms and
//             exclusion flags (16-byte aligned supersets) into slot
//             (tile % S);
//   decode    (two threads per row, each half of the subspaces) the FP16
//             reconstructions of the tile's rows into A[tile & 1];
//   MMA       d / 16 tcgen05.mma into accumulator (tile & 1), committed to
//             the epilogue and back to the decoders;
//   epilogue  (a row per thread, half of the query columns per warp)
//             distance = term + vterm + qmul * acc, one 128-byte store per
//             warp and column.
// Decode, MMA and epilogue of consecutive tiles overlap. Every wait is
// bounded; on expiry the role stops, the others stop at their next wait,
// issued copies and MMAs retire before the CTA frees TMEM and exits.
template <int DSUB>
__global__ void __launch_bounds__(TC_THREADS, 1) k_tc_scan(TcArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // 1024-byte aligned, and kept a pointer into the shared array (not an
  // integer round trip) so that every access compiles to a shared-memory one
  uint8_t* sm = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const TcSmem L(a.kp, a.qc, a.d, a.M, a.nb);
  uint8_t* cb = sm + L.cb_off();
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + L.bars_off());
  uint32_t* holder = reinterpret_cast<uint32_t*>(bars + TcSmem::kBars);
  __shared__ int s_err;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int qc = a.qc, kp = a.kp, M = a.M, nb = a.nb;
  const uint32_t bar0 = smem_u32(bars);
  auto b_full = [&](int b) { return bar0 + 8u * b; };
  auto b_empty = [&](int b) { return bar0 + 8u * (TC_NB + b); };
  auto a_full = [&](int b) { return bar0 + 8u * (2 * TC_NB + b); };
  auto a_empty = [&](int b) { return bar0 + 8u * (2 * TC_NB + 2 + b); };
  auto acc_full = [&](int b) { return bar0 + 8u * (2 * TC_NB + 4 + b); };
  auto acc_empty = [&](int b) { return bar0 + 8u * (2 * TC_NB + 6 + b); };
  auto s_full = [&](int s) { return bar0 + 8u * (2 * TC_NB + 8 + s); };
  auto s_empty = [&](int s) { return bar0 + 8u * (2 * TC_NB + 8 + TC_STAGES + s); };
  if (tid == 0) {
    s_err = 0;
    for (int b = 0; b < TC_NB; ++b) {
      mbar_init(b_full(b), 1);
      mbar_init(b_empty(b), TC_EPI_WARPS);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(a_full(b), TC_DEC_WARPS);
      mbar_init(a_empty(b), 1);
      mbar_init(acc_full(b), 1);
      mbar_init(acc_empty(b), TC_EPI_WARPS);
    }
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(s_full(s), 1);
      mbar_init(s_empty(s), TC_DEC_WARPS + TC_EPI_WARPS);
    }
    fence_mbar_init();
  }
  if (warp == TC_MMA_WARP) tmem_alloc(smem_u32(holder), 2 * qc);
  {  // the codebook, once per CTA
    const uint4* src = reinterpret_cast<const uint4*>(a.pq16);
    uint4* dst = reinterpret_cast<uint4*>(cb);
    for (int i = tid; i < L.cbbytes / 16; i += TC_THREADS) dst[i] = __ldg(src + i);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(holder);
  volatile int* verr = &s_err;
  const int total = *a.total_items;
  const int nkb = kp >> 6;
  const long long lim = a.wait_limit;
  auto wait = [&](uint32_t bar, uint32_t parity) {
    if (*verr) return false;
    if (mbar_wait(bar, parity, lim)) return true;
    *verr = 1;
    return false;
  };
  // the record of item it, one item ahead
  TcItem nrec;
  if ((int)blockIdx.x < total) nrec = a.items[blockIdx.x];
  auto next_item = [&](int it) {
    const TcItem rec = nrec;
    if (it + (int)gridDim.x < total) nrec = a.items[it + gridDim.x];
    return rec;
  };

  if (warp == TC_PROD_WARP) {
    if (lane == 0) {
      int g = 0, i = 0;
      bool ok = true;
      for (int it = blockIdx.x; it < total && ok; it += gridDim.x, ++i) {
        const TcItem rec = next_item(it);
        const int ib = i % nb;
        if (!wait(b_empty(ib), ((uint32_t)(i / nb) & 1u) ^ 1u)) break;
        const int npad = max(16, (rec.nq + 15) & ~15);
        mbar_arrive_expect_tx(b_full(ib), (uint32_t)(nkb * npad * 128 + npad * 16));
        const uint8_t* img = a.bimg + (int64_t)rec.chunk * ((int64_t)qc * kp * 2);
        for (int kb = 0; kb < nkb; ++kb)
          bulk_load(smem_u32(sm + L.b_off(ib) + kb * qc * 128), img + kb * qc * 128,
                    (uint32_t)(npad * 128), b_full(ib));
        bulk_load(smem_u32(sm + L.m_off(ib)), a.meta + (int64_t)rec.chunk * qc, (uint32_t)(npad * 16),
                  b_full(ib));
        for (long long row0 = rec.rbeg; row0 < rec.rend; row0 += TC_BM, ++g) {
          const int s = g % TC_STAGES;
          if (!wait(s_empty(s), ((uint32_t)(g / TC_STAGES) & 1u) ^ 1u)) {
            ok = false;
            break;
          }
          const int nr = (int)min((long long)TC_BM, rec.rend - row0);
          const long long pos = rec.loff + row0;
          const long long c0 = (pos * M) & ~15ll, c1 = (pos * M + (long long)nr * M + 15) & ~15ll;
          uint32_t bytes = (uint32_t)(c1 - c0);
          long long v0 = 0, v1 = 0, e0 = 0, e1 = 0;
          if (a.vterm) {
            v0 = (pos * 4) & ~15ll;
            v1 = (pos * 4 + (long long)nr * 4 + 15) & ~15ll;
            bytes += (uint32_t)(v1 - v0);
          }
          if (a.excl) {
            e0 = pos & ~15ll;
            e1 = (pos + nr + 15) & ~15ll;
            bytes += (uint32_t)(e1 - e0);
          }
          uint8_t* slot = sm + L.slot_off(s);
          mbar_arrive_expect_tx(s_full(s), bytes);
          bulk_load(smem_u32(slot), a.codes + c0, (uint32_t)(c1 - c0), s_full(s));
          if (a.vterm)
            bulk_load(smem_u32(slot + L.code_bytes), reinterpret_cast<const uint8_t*>(a.vterm) + v0,
                      (uint32_t)(v1 - v0), s_full(s));
          if (a.excl)
            bulk_load(smem_u32(slot + L.code_bytes + 544), a.excl + e0, (uint32_t)(e1 - e0), s_full(s));
        }
      }
      // Unwind: every issued copy lands before the CTA may exit (full limit).
      for (int j = (g > TC_STAGES ? g - TC_STAGES : 0); j < g; ++j)
        if (!mbar_wait(s_full(j % TC_STAGES), (uint32_t)(j / TC_STAGES) & 1u)) *verr = 1;
      for (int j = (i > nb ? i - nb : 0); j < i; ++j)
        if (!mbar_wait(b_full(j % nb), (uint32_t)(j / nb) & 1u)) *verr = 1;
    }
  } else if (warp == TC_MMA_WARP) {
    if (lane == 0) {
      int g = 0, i = 0, last_commit = -1;
      bool ok = true;
      for (int it = blockIdx.x; it < total && ok; it += gridDim.x, ++i) {
        const TcItem rec = next_item(it);
        const int ib = i % nb;
        if (!wait(b_full(ib), (uint32_t)(i / nb) & 1u)) break;
        const int npad = max(16, (rec.nq + 15) & ~15);
        const uint32_t idesc = idesc_f16_f32(TC_BM, npad);
        const uint32_t bbase = smem_u32(sm + L.b_off(ib));
        for (long long row0 = rec.rbeg; row0 < rec.rend; row0 += TC_BM, ++g) {
          const int buf = g & 1;
          const uint32_t ph = (uint32_t)(g >> 1) & 1u;
          if (!wait(a_full(buf), ph) || !wait(acc_empty(buf), ph ^ 1u)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t dt = tmem + (uint32_t)(buf * qc);
          const uint32_t abase = smem_u32(sm + L.a_off(buf));
          const int ks = a.d >> 4;
          for (int k = 0; k < ks; ++k) {
            const int kb = k >> 2, kk = k & 3;
            const uint64_t ad = desc_k_sw128(abase + kb * (TC_BM * 128)) + 2u * kk;
            const uint64_t bd = desc_k_sw128(bbase + kb * (qc * 128)) + 2u * kk;
            umma_f16(dt, ad, bd, idesc, k > 0 ? 1u : 0u);
          }
          umma_commit(acc_full(buf));
          umma_commit(a_empty(buf));
          last_commit = g;
        }
      }
      // Unwind: the issued MMAs retire before TMEM is freed (full limit).
      if (last_commit >= 0 &&
          !mbar_wait(acc_full(last_commit & 1), (uint32_t)(last_commit >> 1) & 1u))
        *verr = 1;
    }
  } else if (warp < TC_DEC_WARPS) {
    // ---- decode: thread (quarter, lane) owns row r, half of the subspaces
    const int r = (warp & 3) * 32 + lane;
    const int msplit = M >> 1, m0 = (warp >> 2) * msplit;
    int g = 0;
    bool ok = true;
    for (int it = blockIdx.x; it < total && ok; it += gridDim.x) {
      const TcItem rec = next_item(it);
      for (long long row0 = rec.rbeg; row0 < rec.rend; row0 += TC_BM, ++g) {
        const int s = g % TC_STAGES, buf = g & 1;
        if (!wait(s_full(s), (uint32_t)(g / TC_STAGES) & 1u) ||
            !wait(a_empty(buf), ((uint32_t)(g >> 1) & 1u) ^ 1u)) {
          ok = false;
          break;
        }
        const int nr = (int)min((long long)TC_BM, rec.rend - row0);
        if (r < nr) {
          uint8_t* A = sm + L.a_off(buf);
          const long long pos = rec.loff + row0;
          const uint8_t* crow = sm + L.slot_off(s) + (int)((pos * M) & 15) + r * M + m0;
          for (int w0 = 0; w0 < msplit; w0 += 4) {
            const uint32_t word = *reinterpret_cast<const uint32_t*>(crow + w0);
#pragma unroll
            for (int b = 0; b < 4; ++b) {
              const int m = m0 + w0 + b;
              const uint32_t code = (word >> (8 * b)) & 255u;
              if (DSUB == 8) {
                const uint4 cw = *reinterpret_cast<const uint4*>(cb + ((m << 8) + code) * 16);
                *reinterpret_cast<uint4*>(A + (m >> 3) * (TC_BM * 128) + sw128(r, m & 7)) = cw;
              } else {  // dsub 4: half a chunk per subspace
                const uint2 cw = *reinterpret_cast<const uint2*>(cb + ((m << 8) + code) * 8);
                *reinterpret_cast<uint2*>(A + (m >> 4) * (TC_BM * 128) + sw128(r, (m >> 1) & 7) +
                                          (m & 1) * 8) = cw;
              }
            }
          }
        }
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(a_full(buf));
          mbar_arrive(s_empty(s));
        }
      }
    }
  } else {
    // ---- epilogue: thread (quarter, lane) owns row r, warp half h takes
    // the column groups h, h + 2, ...
    const int ew = warp - TC_DEC_WARPS;
    const int lq = ew & 3, half = ew >> 2;  // warp % 4 == lq: this warp's TMEM lanes
    const int r = lq * 32 + lane;
    int g = 0, i = 0;
    bool ok = true;
    for (int it = blockIdx.x; it < total && ok; it += gridDim.x, ++i) {
      const TcItem rec = next_item(it);
      const int ib = i % nb;
      if (!wait(b_full(ib), (uint32_t)(i / nb) & 1u)) break;
      const int nqi = rec.nq, npad = max(16, (nqi + 15) & ~15);
      const TcMeta* mt = reinterpret_cast<const TcMeta*>(sm + L.m_off(ib));
      for (long long row0 = rec.rbeg; row0 < rec.rend; row0 += TC_BM, ++g) {
        const int s = g % TC_STAGES, buf = g & 1;
        if (!wait(s_full(s), (uint32_t)(g / TC_STAGES) & 1u) ||
            !wait(acc_full(buf), (uint32_t)(g >> 1) & 1u)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const int nr = (int)min((long long)TC_BM, rec.rend - row0);
        const long long pos = rec.loff + row0;
        const uint8_t* slot = sm + L.slot_off(s);
        const bool row_ok = r < nr;
        float vr = 0.0f;
        bool ex = false;
        if (row_ok && a.vterm)
          vr = *reinterpret_cast<const float*>(slot + L.code_bytes + (int)((pos * 4) & 15) + r * 4);
        if (row_ok && a.excl) ex = slot[L.code_bytes + 544 + (int)(pos & 15) + r] != 0;
        for (int cg = half; cg * 16 < npad; cg += 2) {
          float v[16];
          tmem_ld16(tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)(buf * qc + cg * 16), v);
          // Straight-line over the 16 columns (the loads of padding columns
          // read the image's unused entries; only their stores are off), so
          // the columns' load-compute-store chains interleave.
          uint32_t* drow = a.dist + row0 + r;
          const int jmax = row_ok ? nqi - cg * 16 : 0;
#pragma unroll
          for (int jj = 0; jj < 16; ++jj) {
            const TcMeta m = mt[cg * 16 + jj];  // one broadcast shared load per column
            uint32_t o = float_to_ordered(fmaf(v[jj], m.qmul, m.term + vr));
            o = o == TC_EXCLUDED ? TC_EXCLUDED - 1u : o;  // a NaN stays a candidate
            if (jj < jmax) drow[m.seg] = ex ? TC_EXCLUDED : o;
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(acc_empty(buf));
          mbar_arrive(s_empty(s));
          if (row0 + TC_BM >= rec.rend) mbar_arrive(b_empty(ib));
        }
      }
    }
  }
  __syncthreads();
  if (warp == TC_MMA_WARP) {
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
__global__ void __launch_bounds__(SEL_WARPS * 32) k_tc_select_wide(SelArgs a) {
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

// One warp per query, one pass over its distance row (16-byte loads, the
// next round's load issued before this round's keys are built): keys below
// the running bound T are staged in shared memory; when the staging area
// could overflow, the R smallest are kept and T becomes the largest of
// them (a later key at or above T cannot be among the R smallest). The
// kept set is the R smallest keys whatever the order of arrival; it is
// written unsorted, in a fixed order.
__global__ void __launch_bounds__(SS_WARPS * 32) k_tc_select_stream(SelArgs a) {
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
  const int n = carry <= a.smax ? carry : 0;  // a row over smax was left unwritten (site 106)
  const uint32_t* src = a.dist + row * a.smax;  // smax is a multiple of 4: 16-byte rows
  const int R = a.R;
  const unsigned lt = (1u << lane) - 1u;
  uint64_t T = KEY_NONE;
  int m = 0, p = 0;
  // words i0 + 4 lane .. + 3 of each 128-word round (the row holds smax
  // >= roundup(n, 4) words, so the vector load stays in the row)
  auto load4 = [&](int i0) {
    const int i = i0 + 4 * lane;
    return i < n ? __ldg(reinterpret_cast<const uint4*>(src + i))
                 : make_uint4(TC_EXCLUDED, TC_EXCLUDED, TC_EXCLUDED, TC_EXCLUDED);
  };
  uint4 cur = load4(0);
  for (int i0 = 0; i0 < n; i0 += 128) {
    const uint4 nxt = load4(i0 + 128);
    if (m + 128 > SS_CAP) {
      T = warp_keep_smallest(buf, m, R, side, hist);
      m = R;
    }
    const uint32_t w[4] = {cur.x, cur.y, cur.z, cur.w};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + 4 * lane + u;
      uint64_t key = KEY_NONE;
      bool in = false;
      if (i < n) {
        while (pbeg[p + 1] <= i) ++p;
        key = ((uint64_t)w[u] << 32) | (uint32_t)(poff[p] + (i - pbeg[p]));
        in = w[u] != TC_EXCLUDED && key < T;
      }
      const unsigned b = __ballot_sync(0xffffffffu, in);
      if (in) buf[m + __popc(b & lt)] = key;
      m += __popc(b);
    }
    cur = nxt;
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
  return per_list > 48.0 ? 128 : 64;
}

namespace {

// Scratch layout of one launch (every part 256-byte aligned).
struct TcLayout {
  int64_t smax4, chunks, items;
  size_t q16, qmul, seg, ints, start, items_b, bimg, meta, excl, dist, total;
  TcLayout(int64_t nq, int P, int nlist, int d, int64_t smax, int qc, int64_t ntotal) {
    const int kp = (d + 63) / 64 * 64;
    const int64_t npairs = nq * P;
    smax4 = (smax + 3) & ~3ll;
    chunks = npairs / qc + nlist + 1;
    items = nq * smax4 / ((int64_t)qc * TC_RS) + npairs / qc + ntotal / TC_RS + 2 * (int64_t)nlist + 4;
    q16 = al((size_t)nq * kp * 2);
    qmul = al((size_t)nq * 4);
    seg = al((size_t)npairs * 8);
    ints = 4 * al((size_t)(nlist + 1) * 4);  // cnt, cursor, cstart, istart
    start = al((size_t)(nlist + 1) * 8);
    items_b = al((size_t)items * sizeof(TcItem));
    bimg = al((size_t)chunks * qc * kp * 2);
    meta = al((size_t)chunks * qc * sizeof(TcMeta));
    excl = al((size_t)ntotal + 16);
    dist = al((size_t)nq * smax4 * 4);
    total = q16 + qmul + seg + ints + start + items_b + bimg + meta + excl + dist;
  }
};

}  // namespace

size_t ivfpq_tc_scratch_bytes(int64_t nq, int nprobe, int nlist, int d, int64_t smax, int qc,
                              int64_t ntotal) {
  return TcLayout(nq, nprobe, nlist, d, smax, qc, ntotal).total;
}

void launch_ivfpq_scan_tc(const FastScanArgs& f, int64_t smax, int qc, void* scratch, int num_sms,
                          long long wait_limit, cudaStream_t s) {
  const int64_t nq = f.nq;
  if (nq == 0) return;
  const int d = f.d, M = f.M, P = f.nprobe, nlist = f.nlist;
  MV_REQUIRE(f.pq16 && ivfpq_tc_supported(d, M, true), MV_ERR_INTERNAL,
             "tensor-core ADC scan: unsupported shape");
  MV_REQUIRE(qc == 64 || qc == 128, MV_ERR_INTERNAL, "tensor-core ADC scan: bad chunk");
  MV_REQUIRE(nq * P < (1ll << 31) && smax < (1ll << 31), MV_ERR_UNSUPPORTED,
             "tensor-core ADC scan: batch too large");
  const int kp = (d + 63) / 64 * 64;
  const TcLayout lay(nq, P, nlist, d, smax, qc, f.ntotal);
  unsigned char* p = static_cast<unsigned char*>(scratch);
  auto take = [&](size_t bytes) {
    unsigned char* r = p;
    p += bytes;
    return r;
  };
  __half* q16 = reinterpret_cast<__half*>(take(lay.q16));
  float* qmul = reinterpret_cast<float*>(take(lay.qmul));
  int64_t* seg = reinterpret_cast<int64_t*>(take(lay.seg));
  int* ints = reinterpret_cast<int*>(take(lay.ints));
  const size_t ni = lay.ints / 16;  // ints per array (256-byte aligned parts)
  int* cnt = ints;
  int* cursor = ints + ni;
  int* cstart = ints + 2 * ni;
  int* istart = ints + 3 * ni;
  int64_t* start = reinterpret_cast<int64_t*>(take(lay.start));
  TcItem* items = reinterpret_cast<TcItem*>(take(lay.items_b));
  uint8_t* bimg = take(lay.bimg);
  TcMeta* meta = reinterpret_cast<TcMeta*>(take(lay.meta));
  uint8_t* excl = take(lay.excl);
  uint32_t* dist = reinterpret_cast<uint32_t*>(take(lay.dist));
  MV_CHECK_CUDA(cudaMemsetAsync(cnt, 0, 2 * lay.ints / 4, s));  // cnt and cursor
  const float scale = f.metric == MV_METRIC_L2 ? -2.0f : -1.0f;
  const unsigned gw = (unsigned)((nq + 7) / 8);
  k_tc_q16<<<gw, 256, 0, s>>>(f.q, nq, d, kp, scale * f.pq16_inv, q16, qmul);
  k_tc_pairs<<<gw, 256, 0, s>>>(f.probes, nq, P, f.nprobe_q, f.list_off, nlist, lay.smax4, seg,
                                cnt, f.err);
  k_tc_items<<<1, 1024, 0, s>>>(cnt, f.list_off, nlist, qc, start, cstart, istart);
  k_tc_fill<<<(unsigned)((nlist + 255) / 256), 256, 0, s>>>(cnt, f.list_off, nlist, qc, cstart,
                                                            istart, items);
  k_tc_place<<<(unsigned)((nq * P * 16 + 255) / 256), 256, 0, s>>>(
      f.probes, nq, P, f.nprobe_q, nlist, seg, f.term, q16, qmul, kp, qc, cstart, cursor, bimg, meta);
  for (int i = 0; i < 5; ++i) count_launch();
  if (f.filter) {
    k_tc_excl<<<(unsigned)((f.ntotal + 255) / 256), 256, 0, s>>>(f.ids, f.ntotal, f.filter,
                                                                  f.filter_len, excl);
    count_launch();
  }
  TcArgs t;
  t.items = items;
  t.total_items = istart + nlist;
  t.bimg = bimg;
  t.meta = meta;
  t.codes = f.codes;
  t.vterm = f.vterm;
  t.excl = f.filter ? excl : nullptr;
  t.pq16 = f.pq16;
  t.dist = dist;
  t.err = f.err;
  t.M = M;
  t.dsub = d / M;
  t.d = d;
  t.kp = kp;
  t.qc = qc;
  t.wait_limit = wait_limit;
  int nbuf = TC_NB;  // as many query images in flight as shared memory allows
  while (nbuf > 2 && TcSmem(kp, qc, d, M, nbuf).total() > 227 * 1024) nbuf /= 2;
  t.nb = nbuf;
  const size_t smem = TcSmem(kp, qc, d, M, nbuf).total();
  MV_REQUIRE(smem <= 227 * 1024, MV_ERR_INTERNAL, "tensor-core ADC scan: shared memory");
  if (t.dsub == 8) {
    smem_limit(k_tc_scan<8>, smem);
    k_tc_scan<8><<<(unsigned)num_sms, TC_THREADS, smem, s>>>(t);
  } else {
    smem_limit(k_tc_scan<4>, smem);
    k_tc_scan<4><<<(unsigned)num_sms, TC_THREADS, smem, s>>>(t);
  }
  count_launch();
  SelArgs sa;
  sa.dist = dist;
  sa.smax = lay.smax4;
  sa.probes = f.probes;
  sa.nprobe_q = f.nprobe_q;
  sa.list_off = f.list_off;
  sa.P = P;
  sa.nlist = nlist;
  sa.R = f.R;
  sa.nq = nq;
  sa.out = f.out_keys;
  sa.err = f.err;
  if (f.R <= SS_RMAX) {
    const size_t ssm = ss_warp_bytes(P) * SS_WARPS;
    MV_REQUIRE(ssm <= 200 * 1024, MV_ERR_UNSUPPORTED, "tensor-core ADC scan: nprobe too large");
    smem_limit(k_tc_select_stream, ssm);
    k_tc_select_stream<<<(unsigned)((nq + SS_WARPS - 1) / SS_WARPS), SS_WARPS * 32, ssm, s>>>(sa);
  } else {
    const size_t ssm = sel_warp_bytes(P) * SEL_WARPS;
    MV_REQUIRE(ssm <= 200 * 1024, MV_ERR_UNSUPPORTED, "tensor-core ADC scan: nprobe too large");
    smem_limit(k_tc_select_wide, ssm);
    k_tc_select_wide<<<(unsigned)((nq + SEL_WARPS - 1) / SEL_WARPS), SEL_WARPS * 32, ssm, s>>>(sa);
  }
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
