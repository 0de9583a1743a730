// Staged ADC scan of the fast IVF-PQ form (FP32 tables): the default scan.
//
// One CTA per query (or a persistent CTA taking queries from a counter).
// The probed lists are laid end to end in one candidate index space (prefix
// sums of their lengths, as index/index_ivf_pq.mojo:295-347 walks them list
// by list) and processed in rounds of at most E candidates. For each round
// one warp copies the codes and the per-vector terms of the round's list
// pieces into shared memory with cp.async.bulk (the TMA engine's 1-D copy;
// each piece a 16-byte aligned superset of its bytes) on the round's
// mbarrier, into one of two buffers: while the CTA computes round r from one
// buffer, round r + 1 is already in flight into the other, and rounds 0 and 1
// are copied while the query's table is built. The ADC loop then reads
// codes and terms from shared memory only.
//
// Each candidate's distance is adc_fast over the FP32 table (the same
// arithmetic as the unstaged kernel, so the same bits). Keys (ordered
// distance, CSR position) are staged and the R smallest kept by an exact
// select with one histogram pass: the range of the keys' high words is cut
// into at most 2048 bins, the bin holding the R-th key found by a prefix
// scan, every key of a lower bin taken and the boundary bin's keys sorted by
// one warp (the radix select takes over when that bin holds more than 256
// keys). Whenever staging would overflow, the R smallest are kept and later
// candidates must beat the R-th.
#include <cuda_fp16.h>

#include <algorithm>

#include "mv_adc.cuh"
#include "mv_fast.h"
#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_select.cuh"
#include "mv_sm100.cuh"

namespace mv {
namespace {

using namespace sm100;

constexpr int SEG_MAX = 32;  // list pieces per round: one per lane of the planning warp

struct Seg {
  int cbeg;       // first candidate of the piece, relative to the round's start
  int code_off;   // byte offset of its first code in the round's code buffer
  int vt_off;     // byte offset of its first term in the round's term buffer
  int probe;      // probe index (its coarse term)
  long long pos0; // CSR position of its first entry
};

struct StageState {
  Seg seg[2][SEG_MAX + 1];  // [buffer][piece]; piece SEG_MAX holds the round length
  int rlen[2];              // candidates of the round in each buffer (0: none)
  int next_c0;              // first candidate of the next round to plan
  int fill;                 // keys staged
  int bad;                  // a staged copy's wait gave up
  int q;                    // persistent grid: the query taken
  unsigned long long kth;   // the R-th smallest key of the last select
};

__host__ __device__ inline int round16(int v) { return (v + 15) & ~15; }

// Warp 0 plans the next round (at most E candidates and SEG_MAX list
// pieces) into buffer b and issues its bulk copies; lane j takes the j-th
// probe from the one holding the first unplanned candidate. Writes
// rlen[b] = 0 when every candidate is planned.
__device__ __forceinline__ void plan_round(const FastScanArgs& a, StageState& st, int b, int E,
                                           int total, int nprobe, const int* pbeg,
                                           const int64_t* poff, unsigned char* cbuf,
                                           unsigned char* vbuf, uint32_t bar) {
  const int lane = threadIdx.x & 31;
  const int c0 = st.next_c0;
  if (c0 >= total) {
    if (lane == 0) st.rlen[b] = 0;
    return;
  }
  // the probe holding candidate c0: the first p with pbeg[p + 1] > c0
  // (empty lists before it are skipped, however many)
  int lo = 0, hi = nprobe - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (pbeg[mid + 1] > c0) hi = mid;
    else lo = mid + 1;
  }
  const int p0 = lo;
  const int p = p0 + lane;
  const bool live = p < nprobe;
  const int pb = live ? pbeg[p] : total, pe = live ? pbeg[p + 1] : total;
  const int lastend = __shfl_sync(0xffffffffu, pe, 31);
  const int c1 = min(min(total, c0 + E), lastend);
  const int sb = min(max(pb, c0), c1), se = min(max(pe, c0), c1);
  const int len = se - sb;
  const long long pos0 = live ? (long long)poff[p] + (sb - pb) : 0;
  const int M = a.M;
  // 16-byte aligned supersets of the piece's codes and terms
  const uintptr_t gc = reinterpret_cast<uintptr_t>(a.codes) + (uintptr_t)pos0 * M;
  const uintptr_t gc_lo = gc & ~uintptr_t(15);
  const int csz = len > 0 ? (int)(((gc + (uintptr_t)len * M + 15) & ~uintptr_t(15)) - gc_lo) : 0;
  uintptr_t gv = 0, gv_lo = 0;
  int vsz = 0;
  if (a.vterm) {
    gv = reinterpret_cast<uintptr_t>(a.vterm) + (uintptr_t)pos0 * 4;
    gv_lo = gv & ~uintptr_t(15);
    vsz = len > 0 ? (int)(((gv + (uintptr_t)len * 4 + 15) & ~uintptr_t(15)) - gv_lo) : 0;
  }
  int cinc = csz, vinc = vsz;  // inclusive scans over the lanes
  for (int o = 1; o < 32; o <<= 1) {
    const int tc = __shfl_up_sync(0xffffffffu, cinc, o);
    const int tv = __shfl_up_sync(0xffffffffu, vinc, o);
    if (lane >= o) {
      cinc += tc;
      vinc += tv;
    }
  }
  const int cofs = cinc - csz, vofs = vinc - vsz;
  const int bytes = __shfl_sync(0xffffffffu, cinc + vinc, 31);
  if (lane == 0) mbar_arrive_expect_tx(bar, (uint32_t)bytes);
  __syncwarp();
  if (len > 0) {
    bulk_load(smem_u32(cbuf + cofs), reinterpret_cast<const void*>(gc_lo), (uint32_t)csz, bar);
    if (a.vterm)
      bulk_load(smem_u32(vbuf + vofs), reinterpret_cast<const void*>(gv_lo), (uint32_t)vsz, bar);
  }
  Seg& sg = st.seg[b][lane];
  sg.cbeg = sb - c0;
  sg.code_off = cofs + (int)(gc - gc_lo);
  sg.vt_off = vofs + (int)(gv - gv_lo);
  sg.probe = live ? p : 0;
  sg.pos0 = pos0;
  if (lane == 0) {
    st.seg[b][SEG_MAX].cbeg = c1 - c0;
    st.rlen[b] = c1 - c0;
    st.next_c0 = c1;
  }
}

// Two CTAs per SM fit the shared memory at the default round size.
template <int NT>
__global__ void __launch_bounds__(NT, 2)
    k_ivfpq_scan_staged(FastScanArgs a, int E, int cb_bytes, int vb_bytes) {
  extern __shared__ __align__(128) unsigned char smraw[];
  const int M = a.M, d = a.d, dsub = d / M;
  float* lut = reinterpret_cast<float*>(smraw);
  float* qv = lut + M * 256;
  size_t off = ((size_t)(M * 256 + d) * 4 + 127) & ~size_t(127);
  // two stage buffers, each codes (cb_bytes) then terms (vb_bytes)
  unsigned char* const stage = smraw + off;
  const int bstride = cb_bytes + vb_bytes;
  auto cbuf = [&](int b) { return stage + b * bstride; };
  auto vbuf = [&](int b) { return stage + b * bstride + cb_bytes; };
  off += 2 * (size_t)bstride;
  uint64_t* outb = reinterpret_cast<uint64_t*>(smraw + off);
  off += (size_t)a.Rp * 8;
  uint32_t* khi = reinterpret_cast<uint32_t*>(smraw + off);
  uint32_t* klo = khi + a.cap;
  off += (size_t)a.cap * 8;
  int64_t* poff = reinterpret_cast<int64_t*>(smraw + off);
  int* pbeg = reinterpret_cast<int*>(poff + a.nprobe);
  float* pterm = reinterpret_cast<float*>(pbeg + a.nprobe + 1);
  __shared__ RadixScratch rs;
  __shared__ StageState st;
  __shared__ __align__(8) uint64_t bars[2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t bar0 = smem_u32(&bars[0]), bar1 = smem_u32(&bars[1]);
  if (tid == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar1, 1);
    fence_mbar_init();
    st.bad = 0;
  }
  __syncthreads();
  uint32_t ph0 = 0u, ph1 = 0u;  // phase parity each buffer waits for next
  const float scale = a.metric == MV_METRIC_L2 ? -2.0f : -1.0f;
  for (int iter = 0;; ++iter) {
    int qi;
    if (a.counter) {
      __syncthreads();  // the previous query is done with shared memory
      if (tid == 0) st.q = atomicAdd(a.counter, 1);
      __syncthreads();
      qi = st.q;
      if (qi >= a.nq) break;
    } else {
      if (iter > 0) break;
      qi = blockIdx.x;
    }
    const int64_t row = a.order ? a.order[qi] : qi;
    const int nprobe = a.nprobe_q ? min(max(a.nprobe_q[row], 1), a.nprobe) : a.nprobe;
    if (tid == 0) st.fill = 0;
    for (int j = tid; j < d; j += NT) qv[j] = a.q[row * d + j];
    // probe table: offsets, lengths -> prefix sums, coarse terms (warp 0)
    if (warp == 0) {
      int carry = 0;
      for (int p0 = 0; p0 < nprobe; p0 += 32) {
        const int p = p0 + lane;
        int len = 0;
        if (p < nprobe) {
          int list = a.probes[row * a.nprobe + p];
          if (list >= a.nlist) {
            atomicExch(a.err, 103);
            list = -1;
          }
          int64_t o = 0;
          if (list >= 0) {
            o = a.list_off[list];
            len = (int)(a.list_off[list + 1] - o);
          }
          poff[p] = o;
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
      __syncwarp();
      // rounds 0 and 1 go out while the table is built
      const int total = pbeg[nprobe];
      if (lane == 0) st.next_c0 = 0;
      __syncwarp();
      plan_round(a, st, 0, E, total, nprobe, pbeg, poff, cbuf(0), vbuf(0), bar0);
      __syncwarp();
      plan_round(a, st, 1, E, total, nprobe, pbeg, poff, cbuf(1), vbuf(1), bar1);
    }
    __syncthreads();  // qv for the table build
    if (a.pq16) build_lut16<NT>([&](int i, float v) { lut[i] = v; }, qv, a.pq16, M, dsub, scale * a.pq16_inv);
    else build_lut<NT>([&](int i, float v) { lut[i] = v; }, qv, a.pq, M, dsub, scale);
    __syncthreads();
    const int total = pbeg[nprobe];
    int m = 0;
    unsigned long long bound = ~0ull;
    for (int r = 0;; ++r) {
      const int b = r & 1;
      const int len = st.rlen[b];
      if (len == 0) break;
      if (!mbar_wait(b ? bar1 : bar0, b ? ph1 : ph0)) {
        if (tid == 0) {
          st.bad = 1;
          atomicExch(a.err, 1);
        }
      }
      if (b) ph1 ^= 1u;
      else ph0 ^= 1u;
      if (m + len > a.cap) {  // keep the R smallest; later keys must beat the R-th
        const int kept = block_hist_select<NT>(khi, klo, m, a.R, outb, rs, &st.kth);
        for (int j = tid; j < kept; j += NT) {
          khi[j] = (uint32_t)(outb[j] >> 32);
          klo[j] = (uint32_t)outb[j];
        }
        if (kept == a.R) bound = st.kth;
        m = kept;
        if (tid == 0) st.fill = m;
        __syncthreads();
      }
      const unsigned char* cb = cbuf(b);
      const unsigned char* vb = vbuf(b);
      const Seg* sg = st.seg[b];
      int s = 0;
      for (int j0 = 0; j0 < len; j0 += 2 * NT) {
        const int r0 = j0 + tid, r1 = r0 + NT;
        const bool has0 = r0 < len, has1 = r1 < len;
        if (has0)
          while (sg[s + 1].cbeg <= r0) ++s;
        int s1 = s;
        if (has1)
          while (sg[s1 + 1].cbeg <= r1) ++s1;
        // lanes without a candidate use the first entry of the round
        const int e0 = has0 ? r0 - sg[s].cbeg : 0, e1 = has1 ? r1 - sg[s1].cbeg : 0;
        const Seg& g0 = sg[has0 ? s : 0];
        const Seg& g1 = sg[has1 ? s1 : 0];
        const int64_t pos0 = g0.pos0 + e0, pos1 = g1.pos0 + e1;
        bool keep0 = has0, keep1 = has1;
        if ((has0 && (pos0 < 0 || pos0 >= a.ntotal)) || (has1 && (pos1 < 0 || pos1 >= a.ntotal))) {
          atomicExch(a.err, 104);  // never expected
          keep0 = keep1 = false;
        }
        const unsigned char* c0p = keep0 ? cb + g0.code_off + e0 * M : cb + sg[0].code_off;
        const unsigned char* c1p = keep1 ? cb + g1.code_off + e1 * M : cb + sg[0].code_off;
        const float v0 = (a.vterm && keep0) ? *reinterpret_cast<const float*>(vb + g0.vt_off + 4 * e0) : 0.0f;
        const float v1 = (a.vterm && keep1) ? *reinterpret_cast<const float*>(vb + g1.vt_off + 4 * e1) : 0.0f;
        const float t0 = pterm[g0.probe], t1 = pterm[g1.probe];
        if (a.filter) {  // filtered ids never enter the shortlist
          if (keep0) {
            const uint32_t id0 = a.ids[pos0];
            if ((int64_t)id0 < a.filter_len && a.filter[id0] != 0) keep0 = false;
          }
          if (keep1) {
            const uint32_t id1 = a.ids[pos1];
            if ((int64_t)id1 < a.filter_len && a.filter[id1] != 0) keep1 = false;
          }
        }
        const float d0 = adc_fast(lut, c0p, M, t0 + v0);
        const float d1 = adc_fast(lut, c1p, M, t1 + v1);
        const unsigned long long k0 = ((unsigned long long)float_to_ordered(d0) << 32) | (uint32_t)pos0;
        const unsigned long long k1 = ((unsigned long long)float_to_ordered(d1) << 32) | (uint32_t)pos1;
        const bool in0 = keep0 && k0 < bound;
        const bool in1 = keep1 && k1 < bound;
        const unsigned b0m = __ballot_sync(0xffffffffu, in0);
        const unsigned b1m = __ballot_sync(0xffffffffu, in1);
        int wbase = 0;
        if (lane == 0 && (b0m | b1m)) wbase = atomicAdd(&st.fill, __popc(b0m) + __popc(b1m));
        wbase = __shfl_sync(0xffffffffu, wbase, 0);
        const unsigned below = (1u << lane) - 1u;
        if (in0) {
          const int slot = wbase + __popc(b0m & below);
          khi[slot] = (uint32_t)(k0 >> 32);
          klo[slot] = (uint32_t)k0;
        }
        if (in1) {
          const int slot = wbase + __popc(b0m) + __popc(b1m & below);
          khi[slot] = (uint32_t)(k1 >> 32);
          klo[slot] = (uint32_t)k1;
        }
        if (has0) s = s1;
      }
      __syncthreads();  // every thread is done with buffer b
      m = st.fill;
      if (warp == 0) plan_round(a, st, b, E, total, nprobe, pbeg, poff, cbuf(b), vbuf(b), b ? bar1 : bar0);
      __syncthreads();
    }
    const int r = block_hist_select<NT>(khi, klo, m, a.R, outb, rs, &st.kth);
    if (a.sorted) {
      for (int j = r + tid; j < a.Rp; j += NT) outb[j] = KEY_NONE;
      __syncthreads();
      block_bitonic_sort(outb, a.Rp);
    }
    for (int i = tid; i < a.R; i += NT) a.out_keys[row * a.R + i] = i < r ? outb[i] : KEY_NONE;
  }  // queries
  // A staged copy whose wait gave up may still be landing: wait once more
  // (bounded) so the CTA does not exit under it.
  if (tid == 0 && st.bad) {
    mbar_wait(bar0, ph0 ^ 1u);
    mbar_wait(bar1, ph1 ^ 1u);
  }
}

}  // namespace

// Round size (candidates staged per round) for the staged scan: the tuner's
// choice, else 1024 (512 for rows above 32 bytes).
static int staged_entries(int M, int E) {
  if (E > 0) return E;
  return M > 32 ? 512 : 1024;
}

size_t staged_scan_smem(const FastScanArgs& a, int E, int* cb_bytes, int* vb_bytes) {
  const int cb = round16(E * a.M + 32 * 32 + 16);
  const int vb = a.vterm ? round16(E * 4 + 32 * 32 + 16) : 0;
  if (cb_bytes) *cb_bytes = cb;
  if (vb_bytes) *vb_bytes = vb;
  const size_t head = ((size_t)(a.M * 256 + a.d) * 4 + 127) & ~size_t(127);
  return head + 2 * ((size_t)cb + vb) + (size_t)next_pow2(a.R) * 8 + (size_t)a.cap * 8 +
         (size_t)a.nprobe * 8 + (size_t)(a.nprobe + 1) * 4 + (size_t)a.nprobe * 4;
}

// Staged scan: cap = R + E (every round fits after at most one select).
bool launch_ivfpq_scan_staged(FastScanArgs a, cudaStream_t s, int nt, int persistent_ctas, int E) {
  if (a.nq == 0) return true;
  E = staged_entries(a.M, E);
  a.Rp = next_pow2(a.R);
  a.cap = std::max(a.R + E, 2 * a.R + 512);
  int cb = 0, vb = 0;
  const size_t smem = staged_scan_smem(a, E, &cb, &vb);
  if (smem > 200 * 1024) return false;  // the unstaged kernel takes it
  MV_REQUIRE(!a.counter || persistent_ctas > 0, MV_ERR_INTERNAL, "persistent scan without a grid");
  const unsigned grid = a.counter ? (unsigned)std::min<int64_t>(persistent_ctas, a.nq) : (unsigned)a.nq;
  auto go = [&](auto kernel, int threads) {
    smem_limit(kernel, smem);
    kernel<<<grid, threads, smem, s>>>(a, E, cb, vb);
  };
  if (nt == 128) go(k_ivfpq_scan_staged<128>, 128);
  else if (nt == 512) go(k_ivfpq_scan_staged<512>, 512);
  else go(k_ivfpq_scan_staged<256>, 256);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
  return true;
}

}  // namespace mv
