// BF16 tensor-core distance GEMM for sm_103a (tcgen05 + TMA + TMEM).
//
// Computes the dense query x base (or query x centroid) inner products that
// dominate the coarse quantizer (index/index_flat.mojo:260-325 used with
// k = nprobe), the flat scan and the k-means assign step
// (clustering/kmeans.mojo:114-161), and turns them into distances in the
// epilogue: L2 ||x||^2 + ||y||^2 - 2 x.y, IP -x.y.
//
// Layout: X (rows) and Y (cols) are BF16, row-major, rows padded with zeros
// to Kp = 64 * nkb elements. One work item is a 128 x BN output tile; CTAs
// are persistent (one per SM) and walk the items column-tile-major, so the
// CTAs running at the same time share the same Y tile through L2 while the
// small X row blocks stay L2-resident.
//
// Warp roles (192 threads):
//   warp 0      TMA producer: per item, the 128-row X tile and BN-row Y tile
//               (nkb k-blocks of 64 BF16 = one 128-byte swizzle row each)
//               into a 2-stage ring, completion on full[s].
//   warp 1      allocates 2*BN TMEM columns; lane 0 issues the UMMAs
//               (tcgen05.mma kind::f16, M = 128, N = BN, K = 16 per
//               instruction) into accumulator (item & 1) and commits
//               empty[s] / tfull[acc].
//   warps 2-5   epilogue: tcgen05.ld 32 columns at a time from their TMEM
//               lane quarter, apply the distance formula, then store the
//               distance matrix (EPI_MATRIX) or fold a per-row argmin into a
//               64-bit (distance, column) key with atomicMin (EPI_ARGMIN).
// Every mbarrier wait is bounded (2 s); on timeout the kernel records an
// error flag, drains what it issued and frees its TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <mutex>

#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_select.cuh"
#include "mv_sm100.cuh"
#include "mv_umma.h"

namespace mv {
namespace {

using namespace sm100;

constexpr int BM = 128;
constexpr int STAGES = 2;
// The fused top-k GEMM keeps the X block resident up to this many k-blocks
// (256 BF16 or E4M3 bytes of K ... 4 x 128-byte rows); longer rows stream
// X and Y k-blocks through KS_STAGES stages.
constexpr int KS_MAX_RESIDENT = 4, KS_STAGES = 4;
constexpr int NUM_THREADS = 192;

template <int BN>
struct Smem {
  static constexpr uint32_t a_bytes_kb = BM * 128;  // one k-block of the X tile
  static constexpr uint32_t b_bytes_kb = BN * 128;
  static __host__ __device__ uint32_t stage_bytes(int nkb) { return (uint32_t)nkb * (a_bytes_kb + b_bytes_kb); }
  static __host__ __device__ size_t total(int nkb) { return 1024 + (size_t)STAGES * stage_bytes(nkb) + 256; }
};

template <int BN, int EPI>
__global__ void __launch_bounds__(NUM_THREADS, 1)
    k_umma_dist(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap ty,
                UmmaArgs g) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const int nkb = g.nkb;
  const uint32_t stage_bytes = Smem<BN>::stage_bytes(nkb);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * stage_bytes);
  uint32_t* holder = reinterpret_cast<uint32_t*>(bars + 12);
  __shared__ int s_err;

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const uint32_t bar0 = smem_u32(bars);
  // bars[0..1] full, [2..3] empty, [4..5] tfull, [6..7] tempty, [8] done
  auto b_full = [&](int s) { return bar0 + 8u * s; };
  auto b_empty = [&](int s) { return bar0 + 8u * (2 + s); };
  auto b_tfull = [&](int a) { return bar0 + 8u * (4 + a); };
  auto b_tempty = [&](int a) { return bar0 + 8u * (6 + a); };
  const uint32_t b_done = bar0 + 8u * 8;

  if (threadIdx.x == 0) {
    s_err = 0;
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(b_full(s), 1);
      mbar_init(b_empty(s), 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(b_tfull(a), 1);
      mbar_init(b_tempty(a), 128);
    }
    mbar_init(b_done, 1);
    fence_mbar_init();
  }
  if (warp == 0 && lane == 0) {
    prefetch_tmap(&tx);
    prefetch_tmap(&ty);
  }
  if (warp == 1) tmem_alloc(smem_u32(holder), 2 * BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(holder);

  const int nrb = (g.nrows + BM - 1) / BM;
  const int nct = (g.ncols + BN - 1) / BN;
  const int64_t total = (int64_t)nrb * nct;
  const int64_t first = blockIdx.x;
  const int64_t step = gridDim.x;
  const int my_count = first < total ? (int)((total - 1 - first) / step + 1) : 0;
  volatile int* verr = &s_err;

  if (warp == 0) {
    if (lane == 0) {
      int i = 0;
      for (; i < my_count; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
        if (*verr || !mbar_wait(b_empty(s), ph ^ 1u, g.wait_limit)) {
          *verr = 1;
          break;
        }
        const int64_t w = first + (int64_t)i * step;
        const int ct = (int)(w / nrb);
        const int rb = (int)(w - (int64_t)ct * nrb);
        uint8_t* st = smem + (size_t)s * stage_bytes;
        mbar_arrive_expect_tx(b_full(s), stage_bytes);
        for (int kb = 0; kb < nkb; ++kb) {
          tma_load_2d(smem_u32(st + kb * Smem<BN>::a_bytes_kb), &tx, kb * 64, rb * BM, b_full(s));
          tma_load_2d(smem_u32(st + nkb * Smem<BN>::a_bytes_kb + kb * Smem<BN>::b_bytes_kb), &ty,
                      kb * 64, ct * BN, b_full(s));
        }
      }
      // Drain: every issued load must land before the CTA exits.
      for (int j = (i > STAGES ? i - STAGES : 0); j < i; ++j)
        if (!mbar_wait(b_full(j % STAGES), (uint32_t)(j / STAGES) & 1u)) *verr = 1;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(BM, BN);
      for (int i = 0; i < my_count; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
        const int acc = i & 1;
        const uint32_t aph = (uint32_t)(i >> 1) & 1u;
        if (*verr || !mbar_wait(b_tempty(acc), aph ^ 1u, g.wait_limit) || !mbar_wait(b_full(s), ph, g.wait_limit)) {
          *verr = 1;
          break;
        }
        tc_fence_after();
        const uint8_t* st = smem + (size_t)s * stage_bytes;
        const uint32_t d = tmem + (uint32_t)(acc * BN);
        for (int kb = 0; kb < nkb; ++kb) {
          const uint64_t ad = desc_k_sw128(smem_u32(st + kb * Smem<BN>::a_bytes_kb));
          const uint64_t bd =
              desc_k_sw128(smem_u32(st + nkb * Smem<BN>::a_bytes_kb + kb * Smem<BN>::b_bytes_kb));
#pragma unroll
          for (int kk = 0; kk < 4; ++kk)  // 4 x K16 per 64-element k-block (+32 B each)
            umma_bf16(d, ad + 2u * kk, bd + 2u * kk, idesc, (kb | kk) ? 1u : 0u);
        }
        umma_commit(b_empty(s));
        umma_commit(b_tfull(acc));
      }
      umma_commit(b_done);
    }
  } else {
    const int q = warp & 3;  // TMEM lane quarter of this warp
    const int rloc = q * 32 + lane;
    for (int i = 0; i < my_count; ++i) {
      const int acc = i & 1;
      const uint32_t aph = (uint32_t)(i >> 1) & 1u;
      bool ok = !*verr && mbar_wait(b_tfull(acc), aph, g.wait_limit);
      if (!__all_sync(0xffffffffu, ok)) {
        *verr = 1;
        break;
      }
      tc_fence_after();
      const int64_t w = first + (int64_t)i * step;
      const int ct = (int)(w / nrb);
      const int rb = (int)(w - (int64_t)ct * nrb);
      const int64_t row = (int64_t)rb * BM + rloc;
      const bool row_ok = row < g.nrows;
      const float rn = (row_ok && g.rnorm) ? g.rnorm[row] : 0.0f;
      uint64_t best = KEY_NONE;
      for (int c0 = 0; c0 < BN; c0 += 32) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN + c0), v);
        const int64_t col0 = (int64_t)ct * BN + c0;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int64_t col = col0 + j;
          float dist;
          if (g.metric == MV_METRIC_L2) {
            const float cn = (col < g.ncols) ? __ldg(g.cnorm + col) : 0.0f;
            dist = rn + cn - 2.0f * v[j];
          } else {
            dist = -v[j];
          }
          v[j] = dist;
        }
        if (EPI == EPI_MATRIX) {
          if (row_ok) {
            float* o = g.out + row * g.ldo + col0;
            if (col0 + 32 <= g.ncols && (g.ldo & 3) == 0) {
#pragma unroll
              for (int j = 0; j < 32; j += 4)
                *reinterpret_cast<float4*>(o + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
            } else {
              for (int j = 0; j < 32; ++j)
                if (col0 + j < g.ncols) o[j] = v[j];
            }
          }
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            if (col0 + j < g.ncols) {
              uint64_t key = make_key(v[j], (uint32_t)(col0 + j));
              best = key < best ? key : best;
            }
          }
        }
      }
      if (EPI == EPI_ARGMIN && row_ok && best != KEY_NONE)
        atomicMin(reinterpret_cast<unsigned long long*>(g.keys + row), (unsigned long long)best);
      tc_fence_before();
      mbar_arrive(b_tempty(acc));
    }
  }
  __syncthreads();
  if (warp == 1) {
    bool done = true;
    if (lane == 0) done = mbar_wait(b_done, 0);
    done = __shfl_sync(0xffffffffu, done, 0);
    if (!done && lane == 0) *verr = 1;
    tc_fence_after();
    tmem_dealloc(tmem, 2 * BN);
  }
  if (threadIdx.x == 0 && *verr && g.err) atomicExch(g.err, 1);
}

// GEMM with a per-row top-K epilogue. CTA (seg, rb) owns the 128-row X
// block rb (loaded once) and the column tiles [seg * tps, (seg + 1) * tps).
// Each epilogue thread owns one row and keeps the K smallest (distance,
// column) keys seen so far in a binary max-heap in shared memory,
// slot-major (heap[j * 128 + row]) so a warp's 32 rows sit in consecutive
// words. A distance is tested against the heap top (the current K-th key)
// with one compare; the few that pass go to a small pending buffer, and the
// whole warp drains all pending buffers into their heaps together when any
// of them is nearly full, so the heap updates run in step across the warp.
// The kept set is the K smallest keys of the segment whatever the order of
// arrival. The row-constant ||x||^2 is left out of the keys (rows rank the
// same without it). With gthr, the segments of a row share a threshold: a
// full heap publishes its K-th key (atomicMin) and every segment filters
// with the smallest published one, which can only drop keys that are not
// among the row's K smallest over all segments. At the end each thread writes its heap (unsorted,
// KEY_NONE padded to ncp) to out[(row * nseg + seg) * ncp + j].
// Pending slots per row: at least 16, up to 64 when shared memory allows.
// The warp drains when any row has more than pend - 4 (a check after every
// group of 4 columns), so a larger buffer means fewer, fuller drains.
constexpr int TOPK_PEND_MIN = 16, TOPK_PEND_MAX = 64;

__device__ __forceinline__ void heap_replace_top(uint64_t* h, int K, uint64_t key) {
  int i = 0;
  while (true) {
    const int l = 2 * i + 1;
    if (l >= K) break;
    int c = l;
    uint64_t hc = h[(size_t)l * BM];
    if (l + 1 < K) {
      const uint64_t hr = h[(size_t)(l + 1) * BM];
      if (hr > hc) {
        c = l + 1;
        hc = hr;
      }
    }
    if (hc <= key) break;
    h[(size_t)i * BM] = hc;
    i = c;
  }
  h[(size_t)i * BM] = key;
}

// KS (K streaming, rows longer than KS_MAX_RESIDENT k-blocks): the X block is
// not kept resident; every stage of a KS_STAGES ring holds one k-block of X
// and one of the Y tile, and the MMA warp walks (tile, k-block).
template <int BN, bool L2, int EG, bool F8 = false, bool KS = false>
__global__ void __launch_bounds__(64 + 128 * EG, 1)
    k_umma_topk(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap ty,
                UmmaTopkArgs g) {
  // A k-block is one 128-byte swizzled row: 64 BF16 or 128 E4M3 elements.
  constexpr int KB_ELEMS = F8 ? 128 : 64;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const int nkb = g.nkb;
  const uint32_t a_bytes = KS ? 0u : (uint32_t)nkb * BM * 128;
  const uint32_t b_stage = KS ? (uint32_t)(BM + BN) * 128 : (uint32_t)nkb * BN * 128;
  constexpr int NST = KS ? KS_STAGES : STAGES;
  uint8_t* sA = smem;
  uint8_t* sB = smem + a_bytes;
  // Per epilogue group: heaps (nc x BM), pending (g.pend x BM); per
  // epilogue warp: the tile's column biases (BN floats).
  uint64_t* heap = reinterpret_cast<uint64_t*>(sB + NST * b_stage);
  uint64_t* pend = heap + (size_t)EG * g.nc * BM;
  float* cnbuf = reinterpret_cast<float*>(pend + (size_t)EG * g.pend * BM);
  // E4M3: per epilogue warp also the tile's column scales (BN floats).
  float* csbuf = cnbuf + 4 * EG * BN;
  uint64_t* bars = reinterpret_cast<uint64_t*>(csbuf + (F8 ? 4 * EG * BN : 0));
  uint32_t* holder = reinterpret_cast<uint32_t*>(bars + 16);
  __shared__ int s_err;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t bar0 = smem_u32(bars);
  auto b_full = [&](int s) { return bar0 + 8u * s; };
  auto b_empty = [&](int s) { return bar0 + 8u * (4 + s); };
  auto b_tfull = [&](int a) { return bar0 + 8u * (8 + a); };
  auto b_tempty = [&](int a) { return bar0 + 8u * (10 + a); };
  const uint32_t b_done = bar0 + 8u * 12;
  const uint32_t b_fulla = bar0 + 8u * 13;
  if (threadIdx.x == 0) {
    s_err = 0;
    for (int s = 0; s < NST; ++s) {
      mbar_init(b_full(s), 1);
      mbar_init(b_empty(s), 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(b_tfull(a), 1);
      mbar_init(b_tempty(a), 128 * EG);
    }
    mbar_init(b_done, 1);
    mbar_init(b_fulla, 1);
    fence_mbar_init();
  }
  if (warp == 0 && lane == 0) {
    prefetch_tmap(&tx);
    prefetch_tmap(&ty);
  }
  if (warp == 1) tmem_alloc(smem_u32(holder), 2 * BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(holder);
  // Segments vary fastest across the grid, so the segments of a row block
  // run together and tighten the row's shared threshold from the start.
  const int seg = blockIdx.x;
  const int rb = blockIdx.y;
  const int nct = (int)((g.ncols + BN - 1) / BN);
  const int ct0 = seg * g.tps;
  const int ct1 = min(ct0 + g.tps, nct);
  const int my_count = ct1 > ct0 ? ct1 - ct0 : 0;
  volatile int* verr = &s_err;

  if constexpr (KS) {
    if (warp == 0) {
      if (lane == 0) {
        int it = 0;  // k-blocks issued
        bool stop = false;
        for (int i = 0; i < my_count && !stop; ++i) {
          for (int kb = 0; kb < nkb; ++kb, ++it) {
            const int s = it % NST;
            const uint32_t ph = (uint32_t)(it / NST) & 1u;
            if (*verr || !mbar_wait(b_empty(s), ph ^ 1u, g.wait_limit)) {
              *verr = 1;
              stop = true;
              break;
            }
            uint8_t* st = sB + (size_t)s * b_stage;
            mbar_arrive_expect_tx(b_full(s), b_stage);
            tma_load_2d(smem_u32(st), &tx, kb * KB_ELEMS, rb * BM, b_full(s));
            tma_load_2d(smem_u32(st + BM * 128), &ty, kb * KB_ELEMS, (ct0 + i) * BN, b_full(s));
          }
        }
        // Drain: every issued load must land before the CTA exits.
        for (int j = (it > NST ? it - NST : 0); j < it; ++j)
          if (!mbar_wait(b_full(j % NST), (uint32_t)(j / NST) & 1u)) *verr = 1;
      }
    } else if (warp == 1) {
      if (lane == 0) {
        const uint32_t idesc = F8 ? idesc_e4m3_f32(BM, BN) : idesc_bf16_f32(BM, BN);
        int it = 0;
        for (int i = 0; i < my_count; ++i) {
          const int acc = i & 1;
          const uint32_t aph = (uint32_t)(i >> 1) & 1u;
          if (*verr || !mbar_wait(b_tempty(acc), aph ^ 1u, g.wait_limit)) {
            *verr = 1;
            break;
          }
          tc_fence_after();
          const uint32_t d = tmem + (uint32_t)(acc * BN);
          bool bad = false;
          for (int kb = 0; kb < nkb; ++kb, ++it) {
            const int s = it % NST;
            const uint32_t ph = (uint32_t)(it / NST) & 1u;
            if (*verr || !mbar_wait(b_full(s), ph, g.wait_limit)) {
              *verr = 1;
              bad = true;
              break;
            }
            tc_fence_after();
            const uint8_t* st = sB + (size_t)s * b_stage;
            const uint64_t ad = desc_k_sw128(smem_u32(st));
            const uint64_t bd = desc_k_sw128(smem_u32(st + BM * 128));
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {  // 32 bytes of K per instruction
              if (F8) umma_e4m3(d, ad + 2u * kk, bd + 2u * kk, idesc, (kb | kk) ? 1u : 0u);
              else umma_bf16(d, ad + 2u * kk, bd + 2u * kk, idesc, (kb | kk) ? 1u : 0u);
            }
            umma_commit(b_empty(s));
          }
          if (bad) break;
          umma_commit(b_tfull(acc));
        }
        umma_commit(b_done);
      }
    }
  } else
  if (warp == 0) {
    if (lane == 0) {
      mbar_arrive_expect_tx(b_fulla, a_bytes);
      for (int kb = 0; kb < nkb; ++kb)
        tma_load_2d(smem_u32(sA + kb * (BM * 128)), &tx, kb * KB_ELEMS, rb * BM, b_fulla);
      int i = 0;
      for (; i < my_count; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
        if (*verr || !mbar_wait(b_empty(s), ph ^ 1u, g.wait_limit)) {
          *verr = 1;
          break;
        }
        uint8_t* st = sB + (size_t)s * b_stage;
        mbar_arrive_expect_tx(b_full(s), b_stage);
        for (int kb = 0; kb < nkb; ++kb)
          tma_load_2d(smem_u32(st + kb * (BN * 128)), &ty, kb * KB_ELEMS, (ct0 + i) * BN,
                      b_full(s));
      }
      // Drain: every issued load must land before the CTA exits.
      if (!mbar_wait(b_fulla, 0)) *verr = 1;
      for (int j = (i > STAGES ? i - STAGES : 0); j < i; ++j)
        if (!mbar_wait(b_full(j % STAGES), (uint32_t)(j / STAGES) & 1u)) *verr = 1;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = F8 ? idesc_e4m3_f32(BM, BN) : idesc_bf16_f32(BM, BN);
      bool ok = mbar_wait(b_fulla, 0, g.wait_limit);
      if (!ok) *verr = 1;
      for (int i = 0; ok && i < my_count; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
        const int acc = i & 1;
        const uint32_t aph = (uint32_t)(i >> 1) & 1u;
        if (*verr || !mbar_wait(b_tempty(acc), aph ^ 1u, g.wait_limit) || !mbar_wait(b_full(s), ph, g.wait_limit)) {
          *verr = 1;
          break;
        }
        tc_fence_after();
        const uint8_t* st = sB + (size_t)s * b_stage;
        const uint32_t d = tmem + (uint32_t)(acc * BN);
        for (int kb = 0; kb < nkb; ++kb) {
          const uint64_t ad = desc_k_sw128(smem_u32(sA + kb * (BM * 128)));
          const uint64_t bd = desc_k_sw128(smem_u32(st + kb * (BN * 128)));
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {  // 32 bytes of K per instruction
            if (F8) umma_e4m3(d, ad + 2u * kk, bd + 2u * kk, idesc, (kb | kk) ? 1u : 0u);
            else umma_bf16(d, ad + 2u * kk, bd + 2u * kk, idesc, (kb | kk) ? 1u : 0u);
          }
        }
        umma_commit(b_empty(s));
        umma_commit(b_tfull(acc));
      }
      umma_commit(b_done);
    }
  }
  if (warp >= 2) {
    // Epilogue warp (q, h): TMEM lane quarter q (= warp % 4, as tcgen05.ld
    // requires) and group h, which owns chunks [h * NCHG, (h + 1) * NCHG) of
    // every tile and keeps its own heaps (an output segment of its own).
    const int q = warp & 3;
    const int h = (warp - 2) >> 2;
    const int rloc = q * 32 + lane;
    const int64_t row = (int64_t)rb * BM + rloc;
    const bool row_ok = row < g.nrows;
    const int K = g.nc;
    const float INF = __int_as_float(0x7f800000);
    constexpr float SCALE = L2 ? 2.0f : 1.0f;
    uint64_t* H = heap + (size_t)h * K * BM + rloc;      // H[j * BM]
    uint64_t* P = pend + (size_t)h * g.pend * BM + rloc;  // P[j * BM]
    float* cs = cnbuf + (h * 4 + q) * BN;  // this warp's copy of the tile's column biases
    float* css = csbuf + (h * 4 + q) * BN;  // E4M3: its column scales
    // E4M3: acc = <x8, y8> with x = sx x8, y = sy y8, so x.y = sx sy acc; the
    // row's factor SCALE * sx stays in a register, the columns' sy are staged.
    const float rsc = F8 ? SCALE * ((row_ok && g.rscale) ? g.rscale[row] : 1.0f) : SCALE;
    for (int j = 0; j < K; ++j) H[(size_t)j * BM] = KEY_NONE;
    int pc = 0;
    // Work with e = -distance (2 x.y - ||y||^2 for L2, x.y for IP): a column
    // can enter the heap when e >= thr_e. Rows past the end never enter.
    float thr_e = row_ok ? -INF : INF;
    auto drain = [&]() {
      const int mx = __reduce_max_sync(0xffffffffu, pc);
      for (int t = 0; t < mx; ++t) {
        if (t < pc) {
          const uint64_t pe = P[(size_t)t * BM];
          const uint64_t key = make_key(-__uint_as_float((uint32_t)(pe >> 32)), (uint32_t)pe);
          if (key < H[0]) heap_replace_top(H, K, key);
        }
      }
      pc = 0;
      uint64_t thr = H[0];
      if (g.gthr && row_ok) {
        // Publish this segment's K-th key and filter with the row's best.
        if (thr != KEY_NONE) atomicMin(reinterpret_cast<unsigned long long*>(g.gthr + row), thr);
        const uint64_t gt = *reinterpret_cast<volatile uint64_t*>(g.gthr + row);
        thr = gt < thr ? gt : thr;
      }
      // e == thr_e may still lose the tie on the column; the drain decides.
      thr_e = !row_ok ? INF : (thr == KEY_NONE ? -INF : -key_dist(thr));
    };
    // e = SCALE * acc + bias: bias = -||y||^2 (L2) or 0 (IP), and -inf for
    // columns past the end, so the hot loop needs no masking. The next
    // tile's biases are prefetched into registers (lane t holds columns
    // t * CPL ...) while the current tile is processed.
    constexpr int CPL = BN / 32;
    float cpre[CPL];
    float spre[F8 ? CPL : 1];
    auto load_cn = [&](int i) {
      const int64_t base = (int64_t)(ct0 + i) * BN + lane * CPL;
#pragma unroll
      for (int u = 0; u < CPL; ++u)
        cpre[u] = base + u >= g.ncols ? -INF : (L2 ? -__ldg(g.cnorm + base + u) : 0.0f);
      if constexpr (F8) {
#pragma unroll
        for (int u = 0; u < CPL; ++u)
          spre[u] = base + u >= g.ncols ? 0.0f : __ldg(g.cscale + base + u);
      }
    };
    if (my_count > 0) load_cn(0);
    uint64_t gpre = KEY_NONE;  // the row's shared threshold, read one tile ahead
    if (g.gthr && row_ok) gpre = *reinterpret_cast<volatile uint64_t*>(g.gthr + row);
    for (int i = 0; i < my_count; ++i) {
      const int acc = i & 1;
      const uint32_t aph = (uint32_t)(i >> 1) & 1u;
      bool ok = !*verr && mbar_wait(b_tfull(acc), aph, g.wait_limit);
      if (!__all_sync(0xffffffffu, ok)) {
        *verr = 1;
        break;
      }
      tc_fence_after();
      __syncwarp();
#pragma unroll
      for (int u = 0; u < CPL; ++u) cs[lane * CPL + u] = cpre[u];
      if constexpr (F8) {
#pragma unroll
        for (int u = 0; u < CPL; ++u) css[lane * CPL + u] = spre[u];
      }
      __syncwarp();
      if (i + 1 < my_count) load_cn(i + 1);
      if (g.gthr && row_ok) {
        const float ge = gpre == KEY_NONE ? -INF : -key_dist(gpre);
        thr_e = ge > thr_e ? ge : thr_e;
        gpre = *reinterpret_cast<volatile uint64_t*>(g.gthr + row);
      }
      const int64_t tile0 = (int64_t)(ct0 + i) * BN;
      const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN);
      constexpr int NCH = BN / 32 / EG;  // chunks of this group
      const int chb = h * NCH;           // its first chunk
      // e = -distance of the 32 columns of chunk ch (-inf past the end).
      auto chunk_e = [&](const uint32_t* rv, int ch, float* e) {
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
          const float4 b4 = *reinterpret_cast<const float4*>(cs + ch * 32 + j);  // broadcast
          if constexpr (F8) {
            const float4 s4 = *reinterpret_cast<const float4*>(css + ch * 32 + j);
            e[j] = fmaf(rsc * s4.x, __uint_as_float(rv[j]), b4.x);
            e[j + 1] = fmaf(rsc * s4.y, __uint_as_float(rv[j + 1]), b4.y);
            e[j + 2] = fmaf(rsc * s4.z, __uint_as_float(rv[j + 2]), b4.z);
            e[j + 3] = fmaf(rsc * s4.w, __uint_as_float(rv[j + 3]), b4.w);
          } else {
            e[j] = fmaf(SCALE, __uint_as_float(rv[j]), b4.x);
            e[j + 1] = fmaf(SCALE, __uint_as_float(rv[j + 1]), b4.y);
            e[j + 2] = fmaf(SCALE, __uint_as_float(rv[j + 2]), b4.z);
            e[j + 3] = fmaf(SCALE, __uint_as_float(rv[j + 3]), b4.w);
          }
        }
      };
      // Phase 1, no branches: the largest e of each chunk. All of the
      // tile's TMEM loads are issued before the first wait.
      float cmax[NCH];
      {
        uint32_t r[NCH][32];
#pragma unroll
        for (int ch = 0; ch < NCH; ++ch) tmem_ld32_issue(tbase + (uint32_t)((chb + ch) * 32), r[ch]);
#pragma unroll
        for (int ch = 0; ch < NCH; ++ch) tmem_ld32_wait(r[ch]);
#pragma unroll
        for (int ch = 0; ch < NCH; ++ch) {
          float e[32];
          chunk_e(r[ch], chb + ch, e);
#pragma unroll
          for (int j = 0; j < 16; ++j) e[j] = fmaxf(e[j], e[j + 16]);
#pragma unroll
          for (int w = 8; w > 0; w >>= 1)
#pragma unroll
            for (int j = 0; j < w; ++j) e[j] = fmaxf(e[j], e[j + w]);
          cmax[ch] = e[0];
        }
      }
      float tmax = cmax[0];
#pragma unroll
      for (int ch = 1; ch < NCH; ++ch) tmax = fmaxf(tmax, cmax[ch]);
      // Phase 2 (rare once the thresholds settle): the chunks where some
      // row may gain a key are read again from TMEM and appended per group
      // of 4 columns (g, g + 8, g + 16, g + 24) with predicated stores.
      if (__any_sync(0xffffffffu, tmax >= thr_e)) {
#pragma unroll 1
        for (int ch = 0; ch < NCH; ++ch) {
          float cm = cmax[0];
#pragma unroll
          for (int c = 1; c < NCH; ++c)
            if (ch == c) cm = cmax[c];
          if (!__any_sync(0xffffffffu, cm >= thr_e)) continue;
          uint32_t rv[32];
          tmem_ld32_issue(tbase + (uint32_t)((chb + ch) * 32), rv);
          tmem_ld32_wait(rv);
          float e[32];
          chunk_e(rv, chb + ch, e);
          const int64_t col0 = tile0 + (chb + ch) * 32;
          const int64_t left = g.ncols - col0;
          float m[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) m[j] = fmaxf(fmaxf(e[j], e[j + 8]), fmaxf(e[j + 16], e[j + 24]));
#pragma unroll
          for (int gi = 0; gi < 8; ++gi) {
            if (__any_sync(0xffffffffu, m[gi] >= thr_e)) {
#pragma unroll
              for (int t = 0; t < 4; ++t) {
                const int j = gi + 8 * t;
                const bool pass = e[j] >= thr_e && j < left &&
                                  !(g.filter && g.filter[col0 + j]);
                if (pass)
                  P[(size_t)pc * BM] = ((uint64_t)__float_as_uint(e[j]) << 32) |
                                       (uint32_t)(col0 + j);
                pc += pass ? 1 : 0;
              }
              if (__any_sync(0xffffffffu, pc > g.pend - 4)) drain();
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(b_tempty(acc));
    }
    drain();
    if (row_ok) {
      uint64_t* o = g.out + ((size_t)row * g.nseg * EG + (size_t)seg * EG + h) * g.ncp;
      for (int j = 0; j < g.ncp; ++j) o[j] = j < K ? H[(size_t)j * BM] : KEY_NONE;
    }
  }
  __syncthreads();
  if (warp == 1) {
    bool done = true;
    if (lane == 0) done = mbar_wait(b_done, 0);
    done = __shfl_sync(0xffffffffu, done, 0);
    if (!done && lane == 0) *verr = 1;
    tc_fence_after();
    tmem_dealloc(tmem, 2 * BN);
  }
  if (threadIdx.x == 0 && *verr && g.err) atomicExch(g.err, 1);
}

// Descending bitonic network over N register values (static indices).
template <int N>
__device__ __forceinline__ void sort_desc_regs(float* v) {
#pragma unroll
  for (int k = 2; k <= N; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const int l = i ^ j;
        if (l > i) {
          const float a = v[i], b = v[l];
          const bool desc = (i & k) == 0;
          v[i] = desc ? fmaxf(a, b) : fminf(a, b);
          v[l] = desc ? fminf(a, b) : fmaxf(a, b);
        }
      }
    }
  }
}

// Keeps the K smallest of the n keys of a per-row list in lst[0..K)
// (selection in place; only reached when a row has more keys at or above
// its threshold than the list holds) and returns the largest of them.
__device__ __noinline__ uint64_t coarse_list_compact(uint64_t* lst, int n, int K) {
  for (int t = 0; t < K; ++t) {
    int best = t;
    uint64_t bv = lst[t];
    for (int i = t + 1; i < n; ++i) {
      const uint64_t v = lst[i];
      if (v < bv) {
        bv = v;
        best = i;
      }
    }
    lst[best] = lst[t];
    lst[t] = bv;
  }
  return lst[K - 1];
}

// Coarse top-nc in two passes over a segment of centroid tiles (few columns
// per row: the IVF coarse quantizer). Same pipeline as k_umma_topk with the
// query block resident; the producer streams the segment's tiles twice and
// the MMA warp computes them twice with the same instructions, so both
// passes see the same accumulators.
// Pass 1, branch-free: per row, the largest e = -distance of every column
// bucket (column mod NBK). The nc-th largest bucket maximum T has at least
// nc columns with e >= T, so each of the row's nc smallest keys has e >= T.
// Pass 2 appends the keys (distance, column) with e >= T to the row's list
// in global memory (the thread owns the row: no atomics), per 32-column
// chunk one store per set bit of the row's mask, in column order. A chunk
// that would overflow the list first
// compacts it to its nc smallest keys and raises T to the e of the largest
// of them (later columns have larger ids, so a key they tie with that one
// cannot be among the nc smallest); the list always contains the segment's
// nc smallest keys, whatever the data.
// With gthr, the segments of a row share their pass-1 thresholds (atomicMax
// on the ordered e): the segment holding the largest T has nc columns at or
// above it, so no column below it is among the row's nc smallest keys, and
// every segment may use it (read again at every pass-2 tile). Output: lists[(row * nseg + seg) * cap + j] for
// j < counts[row * nseg + seg], unsorted.
template <bool L2, int NBK>
__global__ void __launch_bounds__(192, 2)
    k_coarse_topk2(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap ty,
                   CoarseTopkArgs g) {
  constexpr int BN = 128;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  const int nkb = g.nkb;
  const uint32_t a_bytes = (uint32_t)nkb * BM * 128;
  const uint32_t b_stage = (uint32_t)nkb * BN * 128;
  uint8_t* sA = smem;
  uint8_t* sB = smem + a_bytes;
  float* cnbuf = reinterpret_cast<float*>(sB + STAGES * b_stage);  // 4 warps x BN biases
  uint64_t* bars = reinterpret_cast<uint64_t*>(cnbuf + 4 * BN);
  uint32_t* holder = reinterpret_cast<uint32_t*>(bars + 16);
  __shared__ int s_err;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t bar0 = smem_u32(bars);
  auto b_full = [&](int s) { return bar0 + 8u * s; };
  auto b_empty = [&](int s) { return bar0 + 8u * (4 + s); };
  auto b_tfull = [&](int a) { return bar0 + 8u * (8 + a); };
  auto b_tempty = [&](int a) { return bar0 + 8u * (10 + a); };
  const uint32_t b_done = bar0 + 8u * 12;
  const uint32_t b_fulla = bar0 + 8u * 13;
  if (threadIdx.x == 0) {
    s_err = 0;
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(b_full(s), 1);
      mbar_init(b_empty(s), 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(b_tfull(a), 1);
      mbar_init(b_tempty(a), 128);
    }
    mbar_init(b_done, 1);
    mbar_init(b_fulla, 1);
    fence_mbar_init();
  }
  if (warp == 0 && lane == 0) {
    prefetch_tmap(&tx);
    prefetch_tmap(&ty);
  }
  if (warp == 1) tmem_alloc(smem_u32(holder), 2 * BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(holder);
  const int seg = blockIdx.x;
  const int rb = blockIdx.y;
  const int nct = (int)((g.ncols + BN - 1) / BN);
  const int ct0 = seg * g.tps;
  const int ct1 = min(ct0 + g.tps, nct);
  const int my_count = ct1 > ct0 ? ct1 - ct0 : 0;
  const int total = 2 * my_count;  // both passes
  volatile int* verr = &s_err;

  if (warp == 0) {
    if (lane == 0) {
      mbar_arrive_expect_tx(b_fulla, a_bytes);
      for (int kb = 0; kb < nkb; ++kb)
        tma_load_2d(smem_u32(sA + kb * (BM * 128)), &tx, kb * 64, rb * BM, b_fulla);
      int it = 0;
      for (; it < total; ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
        if (*verr || !mbar_wait(b_empty(s), ph ^ 1u, g.wait_limit)) {
          *verr = 1;
          break;
        }
        const int tile = ct0 + (it < my_count ? it : it - my_count);
        uint8_t* st = sB + (size_t)s * b_stage;
        mbar_arrive_expect_tx(b_full(s), b_stage);
        for (int kb = 0; kb < nkb; ++kb)
          tma_load_2d(smem_u32(st + kb * (BN * 128)), &ty, kb * 64, tile * BN, b_full(s));
      }
      // Drain: every issued load must land before the CTA exits.
      if (!mbar_wait(b_fulla, 0)) *verr = 1;
      for (int j = (it > STAGES ? it - STAGES : 0); j < it; ++j)
        if (!mbar_wait(b_full(j % STAGES), (uint32_t)(j / STAGES) & 1u)) *verr = 1;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(BM, BN);
      bool ok = mbar_wait(b_fulla, 0, g.wait_limit);
      if (!ok) *verr = 1;
      for (int it = 0; ok && it < total; ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
        const int acc = it & 1;
        const uint32_t aph = (uint32_t)(it >> 1) & 1u;
        if (*verr || !mbar_wait(b_tempty(acc), aph ^ 1u, g.wait_limit) || !mbar_wait(b_full(s), ph, g.wait_limit)) {
          *verr = 1;
          break;
        }
        tc_fence_after();
        const uint8_t* st = sB + (size_t)s * b_stage;
        const uint32_t d = tmem + (uint32_t)(acc * BN);
        for (int kb = 0; kb < nkb; ++kb) {
          const uint64_t ad = desc_k_sw128(smem_u32(sA + kb * (BM * 128)));
          const uint64_t bd = desc_k_sw128(smem_u32(st + kb * (BN * 128)));
#pragma unroll
          for (int kk = 0; kk < 4; ++kk)
            umma_bf16(d, ad + 2u * kk, bd + 2u * kk, idesc, (kb | kk) ? 1u : 0u);
        }
        umma_commit(b_empty(s));
        umma_commit(b_tfull(acc));
      }
      umma_commit(b_done);
    }
  } else {
    const int q = warp & 3;  // TMEM lane quarter (warp % 4, as tcgen05.ld requires)
    const int rloc = q * 32 + lane;
    const int64_t row = (int64_t)rb * BM + rloc;
    const bool row_ok = row < g.nrows;
    const float INF = __int_as_float(0x7f800000);
    constexpr float SCALE = L2 ? 2.0f : 1.0f;
    constexpr int BO = NBK == 64 ? 32 : 0;  // bucket offset of the odd chunks
    constexpr int CL = 1;                   // chunks loaded from TMEM per wait
    float* cs = cnbuf + q * BN;
    float bm[NBK];
#pragma unroll
    for (int j = 0; j < NBK; ++j) bm[j] = -INF;
    float thr = INF;  // pass 2: e >= thr enters (never for rows past the end)
    int cnt = 0;
    uint32_t* grow = g.gthr && row_ok ? g.gthr + row : nullptr;
    uint64_t* lst = g.lists + ((size_t)(row_ok ? row : 0) * g.nseg + seg) * g.cap;
    float cpre[4];
    auto load_cn = [&](int ti) {
      const int64_t base = (int64_t)(ct0 + ti) * BN + lane * 4;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        cpre[u] = base + u >= g.ncols ? -INF : (L2 ? -__ldg(g.cnorm + base + u) : 0.0f);
    };
    if (my_count > 0) load_cn(0);
    for (int it = 0; it < total; ++it) {
      const bool pass2 = it >= my_count;
      const int ti = pass2 ? it - my_count : it;
      if (it == my_count && row_ok) {
        sort_desc_regs<NBK>(bm);
        // bm[nc - 1] without a dynamic register index: after the descending
        // sort it is the largest value at positions >= nc - 1.
        float t = -INF;
#pragma unroll
        for (int j = 0; j < NBK; ++j) t = fmaxf(t, j >= g.nc - 1 ? bm[j] : -INF);
        thr = t;
        if (grow) atomicMax(grow, float_to_ordered(t));
      }
      if (pass2 && grow) thr = fmaxf(thr, ordered_to_float(*reinterpret_cast<volatile uint32_t*>(grow)));
      const int acc = it & 1;
      const uint32_t aph = (uint32_t)(it >> 1) & 1u;
      bool ok = !*verr && mbar_wait(b_tfull(acc), aph, g.wait_limit);
      if (!__all_sync(0xffffffffu, ok)) {
        *verr = 1;
        break;
      }
      tc_fence_after();
      __syncwarp();
#pragma unroll
      for (int u = 0; u < 4; ++u) cs[lane * 4 + u] = cpre[u];
      __syncwarp();
      if (it + 1 < total) load_cn(it + 1 < my_count ? it + 1 : it + 1 - my_count);
      const int64_t tile0 = (int64_t)(ct0 + ti) * BN;
      const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN);
      // e = -distance of the 32 columns of chunk ch (-inf past the end), from
      // the chunk's raw accumulators (the TMEM loads of CL chunks are issued
      // before one wait).
      auto chunk_e = [&](const uint32_t* rv, int ch, float* e) {
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
          const float4 b4 = *reinterpret_cast<const float4*>(cs + ch * 32 + j);  // broadcast
          e[j] = fmaf(SCALE, __uint_as_float(rv[j]), b4.x);
          e[j + 1] = fmaf(SCALE, __uint_as_float(rv[j + 1]), b4.y);
          e[j + 2] = fmaf(SCALE, __uint_as_float(rv[j + 2]), b4.z);
          e[j + 3] = fmaf(SCALE, __uint_as_float(rv[j + 3]), b4.w);
        }
      };
      if (!pass2) {
#pragma unroll
        for (int c2 = 0; c2 < 4; c2 += CL) {
          uint32_t rr[CL][32];
#pragma unroll
          for (int h2 = 0; h2 < CL; ++h2) tmem_ld32_issue(tbase + (uint32_t)((c2 + h2) * 32), rr[h2]);
#pragma unroll
          for (int h2 = 0; h2 < CL; ++h2) tmem_ld32_wait(rr[h2]);
#pragma unroll
          for (int h2 = 0; h2 < CL; ++h2) {
            const int ch = c2 + h2;
            float e[32];
            chunk_e(rr[h2], ch, e);
#pragma unroll
            for (int j = 0; j < 32; ++j) bm[(ch & 1) * BO + j] = fmaxf(bm[(ch & 1) * BO + j], e[j]);
          }
        }
      } else {
#pragma unroll
        for (int c2 = 0; c2 < 4; c2 += CL) {
          uint32_t rr[CL][32];
#pragma unroll
          for (int h2 = 0; h2 < CL; ++h2) tmem_ld32_issue(tbase + (uint32_t)((c2 + h2) * 32), rr[h2]);
#pragma unroll
          for (int h2 = 0; h2 < CL; ++h2) tmem_ld32_wait(rr[h2]);
#pragma unroll
          for (int h2 = 0; h2 < CL; ++h2) {
            const int ch = c2 + h2;
            float e[32];
            chunk_e(rr[h2], ch, e);
            const int64_t col0 = tile0 + ch * 32;
            const int64_t left = g.ncols - col0;
            const uint32_t valid = left >= 32 ? 0xffffffffu : left <= 0 ? 0u : (1u << left) - 1u;
            uint32_t mk = 0;
#pragma unroll
            for (int j = 0; j < 32; ++j) mk |= e[j] >= thr ? (1u << j) : 0u;
            mk &= valid;
            if (!__any_sync(0xffffffffu, mk != 0u)) continue;
            if (cnt + __popc(mk) > g.cap) {  // rare
              const uint64_t km = coarse_list_compact(lst, cnt, g.nc);
              cnt = g.nc;
              thr = fmaxf(thr, -key_dist(km));
              mk = 0;
#pragma unroll
              for (int j = 0; j < 32; ++j) mk |= e[j] >= thr ? (1u << j) : 0u;
              mk &= valid;
            }
            // One store per set bit, in ascending column order; e[j] for the
            // lane's own j comes from a select tree (static register indices).
            while (mk) {
              const int j = __ffs(mk) - 1;
              mk &= mk - 1u;
              float t16[16], t8[8], t4[4], t2[2];
#pragma unroll
              for (int i = 0; i < 16; ++i) t16[i] = (j & 1) ? e[2 * i + 1] : e[2 * i];
#pragma unroll
              for (int i = 0; i < 8; ++i) t8[i] = (j & 2) ? t16[2 * i + 1] : t16[2 * i];
#pragma unroll
              for (int i = 0; i < 4; ++i) t4[i] = (j & 4) ? t8[2 * i + 1] : t8[2 * i];
#pragma unroll
              for (int i = 0; i < 2; ++i) t2[i] = (j & 8) ? t4[2 * i + 1] : t4[2 * i];
              const float ej = (j & 16) ? t2[1] : t2[0];
              lst[cnt++] = make_key(-ej, (uint32_t)(col0 + j));
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(b_tempty(acc));
    }
    if (row_ok) g.counts[(size_t)row * g.nseg + seg] = cnt;
  }
  __syncthreads();
  if (warp == 1) {
    bool done = true;
    if (lane == 0) done = mbar_wait(b_done, 0);
    done = __shfl_sync(0xffffffffu, done, 0);
    if (!done && lane == 0) *verr = 1;
    tc_fence_after();
    tmem_dealloc(tmem, 2 * BN);
  }
  if (threadIdx.x == 0 && *verr && g.err) atomicExch(g.err, 1);
}

__global__ void k_to_bf16(const float* __restrict__ x, int64_t n, int d, int kp,
                          __nv_bfloat16* __restrict__ out, float* __restrict__ norms) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= n) return;
  float acc = 0.0f;
  for (int j = lane; j < kp; j += 32) {
    float v = j < d ? x[row * d + j] : 0.0f;
    __nv_bfloat16 b = __float2bfloat16_rn(v);
    out[row * kp + j] = b;
    float r = __bfloat162float(b);
    acc = fmaf(r, r, acc);
  }
  for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
  if (norms && lane == 0) norms[row] = acc;
}

// One warp per row: scale = max|x| / 448 (the largest finite E4M3 is 448),
// E4M3 of x / scale (round to nearest, saturating), zero padding, and the
// norm of the dequantized row.
__global__ void k_to_e4m3(const float* __restrict__ x, int64_t n, int d, int kp,
                          uint8_t* __restrict__ out, float* __restrict__ scales,
                          float* __restrict__ norms) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= n) return;
  float amax = 0.0f;
  for (int j = lane; j < d; j += 32) amax = fmaxf(amax, fabsf(x[row * d + j]));
  for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  const float sc = amax > 0.0f ? amax / 448.0f : 1.0f;
  float acc = 0.0f;
  for (int j = lane; j < kp; j += 32) {
    const __nv_fp8_e4m3 v(j < d ? x[row * d + j] / sc : 0.0f);
    out[row * kp + j] = v.__x;
    const float r = (float)v * sc;
    acc = fmaf(r, r, acc);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    scales[row] = sc;
    if (norms) norms[row] = acc;
  }
}

__global__ void k_fill_keys(uint64_t* keys, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) keys[i] = KEY_NONE;
}

__global__ void k_keys_argmin(const uint64_t* __restrict__ keys, int64_t n, int32_t* __restrict__ out,
                              float* __restrict__ dist) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t k = keys[i];
  out[i] = k == KEY_NONE ? 0 : (int32_t)key_id(k);
  if (dist) dist[i] = k == KEY_NONE ? 0.0f : key_dist(k);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  MV_REQUIRE(fn != nullptr, MV_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
  return fn;
}

// E4M3 rows of kp bytes (a multiple of 128), 128-byte boxes.
CUtensorMap make_tmap8(const void* base, int64_t rows, int kp, int box_rows) {
  MV_REQUIRE((reinterpret_cast<uintptr_t>(base) & 15) == 0, MV_ERR_INTERNAL, "TMA base not 16-byte aligned");
  MV_REQUIRE(kp % 128 == 0, MV_ERR_INTERNAL, "TMA rows must be padded to 128 bytes");
  CUtensorMap tm;
  cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)kp};
  cuuint32_t box[2] = {128, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode_fn()(&tm, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims,
                           strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  MV_REQUIRE(r == CUDA_SUCCESS, MV_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return tm;
}

CUtensorMap make_tmap(const void* base, int64_t rows, int kp, int box_rows) {
  MV_REQUIRE((reinterpret_cast<uintptr_t>(base) & 15) == 0, MV_ERR_INTERNAL, "TMA base not 16-byte aligned");
  MV_REQUIRE(kp % 64 == 0, MV_ERR_INTERNAL, "TMA rows must be padded to 64 elements");
  CUtensorMap tm;
  cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)kp * 2};
  cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode_fn()(&tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims,
                           strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  MV_REQUIRE(r == CUDA_SUCCESS, MV_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return tm;
}

template <int BN, int EPI>
void launch_bn(const UmmaArgs& g, const CUtensorMap& tx, const CUtensorMap& ty, int num_sms,
               cudaStream_t s) {
  const size_t smem = Smem<BN>::total(g.nkb);
  MV_REQUIRE(smem <= 227 * 1024, MV_ERR_UNSUPPORTED, "BF16 GEMM: dimension too large");
  smem_limit(k_umma_dist<BN, EPI>, smem);
  const int64_t items = (int64_t)((g.nrows + BM - 1) / BM) * ((g.ncols + BN - 1) / BN);
  const int grid = (int)std::min<int64_t>(items, num_sms);
  k_umma_dist<BN, EPI><<<grid, NUM_THREADS, smem, s>>>(tx, ty, g);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace

int umma_kpad(int d) { return (d + 63) / 64 * 64; }
int umma_kpad8(int d) { return (d + 127) / 128 * 128; }

void launch_to_e4m3(const float* x, int64_t n, int d, uint8_t* out, float* scales, float* norms,
                    cudaStream_t s) {
  if (n == 0) return;
  k_to_e4m3<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(x, n, d, umma_kpad8(d), out, scales, norms);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_to_bf16(const float* x, int64_t n, int d, __nv_bfloat16* out, float* norms,
                    cudaStream_t s) {
  if (n == 0) return;
  k_to_bf16<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(x, n, d, umma_kpad(d), out, norms);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_umma_dist(int epi, const __nv_bfloat16* X, int64_t nx, const __nv_bfloat16* Y,
                      int64_t ny, int d, int metric, const float* xnorm, const float* ynorm,
                      float* out, int64_t ldo, uint64_t* keys, int* err, int num_sms,
                      cudaStream_t s) {
  if (nx == 0 || ny == 0) return;
  const int kp = umma_kpad(d);
  MV_REQUIRE(kp <= 256, MV_ERR_UNSUPPORTED, "BF16 GEMM supports d <= 256");
  MV_REQUIRE(nx < (1ll << 31) && ny < (1ll << 31), MV_ERR_UNSUPPORTED, "GEMM too large");
  UmmaArgs g;
  g.wait_limit = current_wait_limit();
  g.nrows = nx;
  g.ncols = ny;
  g.nkb = kp / 64;
  g.metric = metric;
  g.rnorm = xnorm;
  g.cnorm = ynorm;
  g.out = out;
  g.ldo = ldo;
  g.keys = keys;
  g.err = err;
  // Widest Y tile whose 2-stage ring fits in shared memory: BN = 256 up to
  // d = 128, 128 up to d = 192, 64 up to d = 256.
  const int bn = g.nkb <= 2 ? 256 : (g.nkb == 3 ? 128 : 64);
  const CUtensorMap tx = make_tmap(X, nx, kp, BM);
  const CUtensorMap ty = make_tmap(Y, ny, kp, bn);
  if (epi == EPI_ARGMIN) {
    k_fill_keys<<<(unsigned)((nx + 255) / 256), 256, 0, s>>>(keys, nx);
    count_launch();
  }
  if (bn == 256) {
    if (epi == EPI_MATRIX) launch_bn<256, EPI_MATRIX>(g, tx, ty, num_sms, s);
    else launch_bn<256, EPI_ARGMIN>(g, tx, ty, num_sms, s);
  } else if (bn == 128) {
    if (epi == EPI_MATRIX) launch_bn<128, EPI_MATRIX>(g, tx, ty, num_sms, s);
    else launch_bn<128, EPI_ARGMIN>(g, tx, ty, num_sms, s);
  } else {
    if (epi == EPI_MATRIX) launch_bn<64, EPI_MATRIX>(g, tx, ty, num_sms, s);
    else launch_bn<64, EPI_ARGMIN>(g, tx, ty, num_sms, s);
  }
}

namespace {
// Shape of the top-k GEMM: Y tile width, epilogue groups and pending slots.
// One epilogue group (4 warps) with the widest Y tile that fits: 128 up to
// d = 128, else 64. The kernel template also takes two groups (8 warps, two
// per TMEM lane quarter, each with its own heaps), which hides more of the
// epilogue's latency but needs 64-wide tiles to fit 227 KB; measured on
// 10k x 1M x 128 that halves the TMA/MMA pipeline's rate and leaves too few
// pending slots, so it is slower (14.7 ms against 10.9 ms) and not chosen.
struct TopkCfg {
  int bn, eg, pend;
};
size_t topk_smem_base(int nkb, int bn, int nc, int eg, bool f8 = false) {
  const size_t tiles = nkb > KS_MAX_RESIDENT
                           ? (size_t)KS_STAGES * (BM + bn) * 128
                           : (size_t)nkb * BM * 128 + (size_t)STAGES * nkb * bn * 128;
  return 1024 + tiles + (size_t)eg * nc * BM * 8 + (size_t)4 * eg * bn * 4 * (f8 ? 2 : 1) + 256;
}
int topk_pend_fit(int nkb, int bn, int nc, int eg, bool f8 = false) {
  const size_t base = topk_smem_base(nkb, bn, nc, eg, f8);
  const size_t room = base < 227 * 1024 ? (227 * 1024 - base) / ((size_t)eg * BM * 8) : 0;
  return (int)std::min<size_t>(TOPK_PEND_MAX, room / 8 * 8);
}
TopkCfg topk_cfg(int nkb, int nc, bool f8 = false) {
  if (nkb > KS_MAX_RESIDENT) {  // streamed K: 128-column tiles when the pending list fits
    const int p128 = topk_pend_fit(nkb, 128, nc, 1, f8);
    if (p128 >= TOPK_PEND_MIN) return {128, 1, p128};
    return {64, 1, topk_pend_fit(nkb, 64, nc, 1, f8)};
  }
  const int bn = nkb <= 2 ? 128 : 64;
  // Two epilogue groups (8 warps, each group half of every tile's columns
  // with heaps of its own) when they fit beside the tiles: the per-row heap
  // epilogue, not the MMAs, bounds this kernel.
  if (bn == 128 && !f8) {
    const int p2 = topk_pend_fit(nkb, bn, nc, 2, f8);
    if (p2 >= TOPK_PEND_MIN) return {bn, 2, p2};
  }
  return {bn, 1, topk_pend_fit(nkb, bn, nc, 1, f8)};
}
size_t topk_smem(int nkb, const TopkCfg& c, int nc, bool f8 = false) {
  return topk_smem_base(nkb, c.bn, nc, c.eg, f8) + (size_t)c.eg * c.pend * BM * 8;
}
}  // namespace

int umma_topk_groups(int d, int nc, bool e4m3) {
  return topk_cfg(e4m3 ? umma_kpad8(d) / 128 : umma_kpad(d) / 64, nc, e4m3).eg;
}

int umma_topk_nseg(int64_t nrows, int64_t ncols, int d, int nc, int num_sms, bool e4m3) {
  const int nkb = e4m3 ? umma_kpad8(d) / 128 : umma_kpad(d) / 64;
  const TopkCfg c = topk_cfg(nkb, nc, e4m3);
  const int64_t nrb = (nrows + BM - 1) / BM;
  const int64_t nct = (ncols + c.bn - 1) / c.bn;
  // CTAs resident per SM (228 KB of shared memory per SM, 1 KB reserved per
  // CTA), then the fewest column segments whose CTAs fill the last wave to
  // 90%; a segment is never shorter than 16 column tiles.
  const int64_t cps = std::max<int64_t>(1, std::min<int64_t>(4, (228 * 1024) / (topk_smem(nkb, c, nc, e4m3) + 1024)));
  const int64_t slots = (int64_t)std::max(num_sms, 1) * cps;
  const int64_t maxseg = std::max<int64_t>(1, std::min<int64_t>(nct / 16, 4096));
  int64_t best = 1;
  double best_eff = 0.0;
  for (int64_t ns = 1; ns <= maxseg; ++ns) {
    const int64_t ctas = nrb * ns;
    const int64_t waves = (ctas + slots - 1) / slots;
    const double eff = (double)ctas / (double)(waves * slots);
    if (eff > best_eff + 1e-9) {
      best_eff = eff;
      best = ns;
    }
    if (eff >= 0.9) break;
  }
  return (int)std::min<int64_t>(best, 65535);
}

void launch_umma_topk(const __nv_bfloat16* X, int64_t nx, const __nv_bfloat16* Y, int64_t ny,
                      int d, int metric, const float* xnorm, const float* ynorm, int nc, int nseg,
                      const uint8_t* filter, uint64_t* gthr, uint64_t* out, int* err,
                      cudaStream_t s) {
  if (nx == 0) return;
  const int kp = umma_kpad(d);
  MV_REQUIRE(kp <= UMMA_TOPK_MAX_K, MV_ERR_UNSUPPORTED, "fused top-k GEMM: d too large");
  MV_REQUIRE(nc >= 1 && nc <= UMMA_TOPK_MAX, MV_ERR_UNSUPPORTED, "fused top-k keeps at most 64 per row");
  MV_REQUIRE(nx < (1ll << 31) && ny < (1ll << 32) - 1, MV_ERR_UNSUPPORTED, "GEMM too large");
  MV_REQUIRE(nseg >= 1 && nseg <= 65535, MV_ERR_INTERNAL, "fused top-k: bad segment count");
  UmmaTopkArgs g;
  g.wait_limit = current_wait_limit();
  g.nrows = nx;
  g.ncols = ny;
  g.nkb = kp / 64;
  g.metric = metric;
  g.rnorm = xnorm;
  g.cnorm = ynorm;
  g.nc = nc;
  g.ncp = next_pow2(nc);
  g.nseg = nseg;
  g.filter = filter;
  g.gthr = gthr;
  if (gthr) MV_CHECK_CUDA(cudaMemsetAsync(gthr, 0xff, sizeof(uint64_t) * nx, s));
  g.out = out;
  g.err = err;
  const TopkCfg c = topk_cfg(g.nkb, nc);
  g.pend = c.pend;
  MV_REQUIRE(g.pend >= TOPK_PEND_MIN, MV_ERR_UNSUPPORTED, "fused top-k GEMM: nc or d too large");
  const int64_t nct = (ny + c.bn - 1) / c.bn;
  g.tps = (int)((nct + nseg - 1) / nseg);
  const CUtensorMap tx = make_tmap(X, nx, kp, BM);
  const CUtensorMap ty = make_tmap(Y, ny, kp, c.bn);
  MV_REQUIRE((nx + BM - 1) / BM <= 65535, MV_ERR_UNSUPPORTED, "fused top-k: too many rows per launch");
  dim3 grid((unsigned)nseg, (unsigned)((nx + BM - 1) / BM));
  const size_t smem = topk_smem(g.nkb, c, nc);
  MV_REQUIRE(smem <= 227 * 1024, MV_ERR_UNSUPPORTED, "fused top-k GEMM: nc or d too large");
  auto go = [&](auto kernel, int threads) {
    smem_limit(kernel, smem);
    kernel<<<grid, threads, smem, s>>>(tx, ty, g);
  };
  const bool l2m = metric == MV_METRIC_L2;
  if (g.nkb > KS_MAX_RESIDENT) {
    if (c.bn == 128) {
      l2m ? go(k_umma_topk<128, true, 1, false, true>, 192)
          : go(k_umma_topk<128, false, 1, false, true>, 192);
    } else {
      l2m ? go(k_umma_topk<64, true, 1, false, true>, 192)
          : go(k_umma_topk<64, false, 1, false, true>, 192);
    }
  } else if (c.bn == 128 && c.eg == 2) {
    l2m ? go(k_umma_topk<128, true, 2>, 320) : go(k_umma_topk<128, false, 2>, 320);
  } else if (c.bn == 128) {
    l2m ? go(k_umma_topk<128, true, 1>, 192) : go(k_umma_topk<128, false, 1>, 192);
  } else {
    l2m ? go(k_umma_topk<64, true, 1>, 192) : go(k_umma_topk<64, false, 1>, 192);
  }
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

namespace {
size_t coarse_topk2_smem(int nkb) {
  return 1024 + (size_t)nkb * BM * 128 + (size_t)STAGES * nkb * 128 * 128 + 4 * 128 * 4 + 256;
}
}  // namespace

// A list must take nc keys plus one chunk's 32 after a compaction.
int coarse_topk2_cap(int nc) { return nc <= 16 ? 48 : 128; }

int coarse_topk2_nseg(int64_t nrows, int64_t ncols, int d, int nc, int num_sms) {
  const int nkb = umma_kpad(d) / 64;
  const int64_t nrb = (nrows + BM - 1) / BM;
  const int64_t nct = (ncols + 127) / 128;
  // CTAs resident per SM (shared memory; 1 KB reserved per CTA), then the
  // fewest column segments (at least 4 tiles each) whose CTAs fill the last
  // wave to 90 %; the select kernel takes at most 256 keys per row.
  const int64_t cps = std::max<int64_t>(1, std::min<int64_t>(2, (228 * 1024) / (coarse_topk2_smem(nkb) + 1024)));
  const int64_t slots = (int64_t)std::max(num_sms, 1) * cps;
  const int64_t maxseg =
      std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(nct / 4, 256 / coarse_topk2_cap(nc)), 4));
  int64_t best = 1;
  double best_eff = 0.0;
  for (int64_t ns = 1; ns <= maxseg; ++ns) {
    const int64_t ctas = nrb * ns;
    const int64_t waves = (ctas + slots - 1) / slots;
    const double eff = (double)ctas / (double)(waves * slots);
    if (eff > best_eff + 1e-9) {
      best_eff = eff;
      best = ns;
    }
    if (eff >= 0.9) break;
  }
  return (int)best;
}

void launch_coarse_topk2(const __nv_bfloat16* X, int64_t nx, const __nv_bfloat16* Y, int64_t ny,
                         int d, int metric, const float* ynorm, int nc, int nseg, uint64_t* lists,
                         int* counts, uint32_t* gthr, int* err, cudaStream_t s) {
  if (nx == 0) return;
  const int kp = umma_kpad(d);
  MV_REQUIRE(kp <= 256, MV_ERR_UNSUPPORTED, "two-pass coarse GEMM: d must be at most 256");
  MV_REQUIRE(nc >= 1 && nc <= 32 && nc <= ny, MV_ERR_UNSUPPORTED, "two-pass coarse GEMM keeps 1..32 lists");
  MV_REQUIRE(nx < (1ll << 31) && ny < (1ll << 32) - 1, MV_ERR_UNSUPPORTED, "GEMM too large");
  MV_REQUIRE((nx + BM - 1) / BM <= 65535, MV_ERR_UNSUPPORTED, "two-pass coarse GEMM: too many rows");
  const int cap = coarse_topk2_cap(nc);
  MV_REQUIRE(nseg >= 1 && (int64_t)nseg * cap <= 256, MV_ERR_INTERNAL, "two-pass coarse GEMM: bad segment count");
  CoarseTopkArgs g;
  g.wait_limit = current_wait_limit();
  g.nrows = nx;
  g.ncols = ny;
  g.nkb = kp / 64;
  g.cnorm = ynorm;
  g.nc = nc;
  g.nseg = nseg;
  const int64_t nct = (ny + 127) / 128;
  g.tps = (int)((nct + nseg - 1) / nseg);
  g.cap = cap;
  g.lists = lists;
  g.counts = counts;
  g.gthr = nseg > 1 ? gthr : nullptr;
  if (g.gthr) MV_CHECK_CUDA(cudaMemsetAsync(g.gthr, 0, sizeof(uint32_t) * nx, s));
  g.err = err;
  const CUtensorMap tx = make_tmap(X, nx, kp, BM);
  const CUtensorMap ty = make_tmap(Y, ny, kp, 128);
  dim3 grid((unsigned)nseg, (unsigned)((nx + BM - 1) / BM));
  const size_t smem = coarse_topk2_smem(g.nkb);
  auto go = [&](auto kernel) {
    smem_limit(kernel, smem);
    kernel<<<grid, 192, smem, s>>>(tx, ty, g);
  };
  const bool l2m = metric == MV_METRIC_L2;
  if (nc <= 16) l2m ? go(k_coarse_topk2<true, 32>) : go(k_coarse_topk2<false, 32>);
  else l2m ? go(k_coarse_topk2<true, 64>) : go(k_coarse_topk2<false, 64>);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_umma_topk_e4m3(const uint8_t* X8, int64_t nx, const float* xscale, const uint8_t* Y8,
                           int64_t ny, const float* yscale, int d, int metric, const float* ynorm,
                           int nc, int nseg, const uint8_t* filter, uint64_t* gthr, uint64_t* out,
                           int* err, cudaStream_t s) {
  if (nx == 0) return;
  const int kp = umma_kpad8(d);
  MV_REQUIRE(kp <= UMMA_TOPK_MAX_K, MV_ERR_UNSUPPORTED, "E4M3 GEMM: d too large");
  MV_REQUIRE(nc >= 1 && nc <= UMMA_TOPK_MAX, MV_ERR_UNSUPPORTED, "fused top-k keeps at most 64 per row");
  MV_REQUIRE(nx < (1ll << 31) && ny < (1ll << 32) - 1, MV_ERR_UNSUPPORTED, "GEMM too large");
  MV_REQUIRE(nseg >= 1 && nseg <= 65535, MV_ERR_INTERNAL, "fused top-k: bad segment count");
  MV_REQUIRE(xscale && yscale, MV_ERR_INTERNAL, "E4M3 GEMM needs row and column scales");
  UmmaTopkArgs g;
  g.wait_limit = current_wait_limit();
  g.nrows = nx;
  g.ncols = ny;
  g.nkb = kp / 128;
  g.metric = metric;
  g.rnorm = nullptr;
  g.cnorm = ynorm;
  g.nc = nc;
  g.ncp = next_pow2(nc);
  g.nseg = nseg;
  g.filter = filter;
  g.gthr = gthr;
  if (gthr) MV_CHECK_CUDA(cudaMemsetAsync(gthr, 0xff, sizeof(uint64_t) * nx, s));
  g.out = out;
  g.err = err;
  g.rscale = xscale;
  g.cscale = yscale;
  const TopkCfg c = topk_cfg(g.nkb, nc, true);
  g.pend = c.pend;
  MV_REQUIRE(g.pend >= TOPK_PEND_MIN, MV_ERR_UNSUPPORTED, "fused top-k GEMM: nc or d too large");
  const int64_t nct = (ny + c.bn - 1) / c.bn;
  g.tps = (int)((nct + nseg - 1) / nseg);
  const CUtensorMap tx = make_tmap8(X8, nx, kp, BM);
  const CUtensorMap ty = make_tmap8(Y8, ny, kp, c.bn);
  MV_REQUIRE((nx + BM - 1) / BM <= 65535, MV_ERR_UNSUPPORTED, "fused top-k: too many rows per launch");
  dim3 grid((unsigned)nseg, (unsigned)((nx + BM - 1) / BM));
  const size_t smem = topk_smem(g.nkb, c, nc, true);
  MV_REQUIRE(smem <= 227 * 1024, MV_ERR_UNSUPPORTED, "fused top-k GEMM: nc or d too large");
  auto go = [&](auto kernel, int threads) {
    smem_limit(kernel, smem);
    kernel<<<grid, threads, smem, s>>>(tx, ty, g);
  };
  const bool l2m = metric == MV_METRIC_L2;
  if (g.nkb > KS_MAX_RESIDENT) {
    if (c.bn == 128) {
      l2m ? go(k_umma_topk<128, true, 1, true, true>, 192)
          : go(k_umma_topk<128, false, 1, true, true>, 192);
    } else {
      l2m ? go(k_umma_topk<64, true, 1, true, true>, 192)
          : go(k_umma_topk<64, false, 1, true, true>, 192);
    }
  } else if (c.bn == 128) {
    l2m ? go(k_umma_topk<128, true, 1, true>, 192) : go(k_umma_topk<128, false, 1, true>, 192);
  } else {
    l2m ? go(k_umma_topk<64, true, 1, true>, 192) : go(k_umma_topk<64, false, 1, true>, 192);
  }
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_keys_argmin(const uint64_t* keys, int64_t n, int32_t* out, float* dist, cudaStream_t s) {
  if (n == 0) return;
  k_keys_argmin<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(keys, n, out, dist);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
