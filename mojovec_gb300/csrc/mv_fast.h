// Host interface of the fast-form IVF-PQ kernels (k_ivfpq_fast.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cuda_runtime.h>

#include <cstdint>

struct mv_ctx;  // the C interface's context (stage profiler)

namespace mv {

struct FastScanArgs {
  const float* q;
  int64_t nq;
  int d, M, metric;
  const float* pq;
  // FP16 codebook scaled by a power of two (pq16 = pq / pq16_inv; dsub 4 or
  // 8), read instead of pq when set: the table values differ from FP32 ones
  // by the FP16 rounding of the codewords.
  const __half* pq16 = nullptr;
  float pq16_inv = 1.0f;
  // Per subspace, an upper bound on the largest codeword norm; when set the
  // scan uses the bank-rotated integer tables (M a multiple of 4, M >= 8).
  const float* pq_cn = nullptr;
  const int64_t* list_off;
  const uint8_t* codes;
  const float* vterm;     // per CSR entry, null for IP
  const int32_t* probes;  // nq x nprobe, ascending coarse distance
  const float* term;      // nq x nprobe coarse distances (exact FP32)
  int nprobe;
  int R;                  // shortlist length
  int sorted;             // 1: shortlist sorted ascending (it is the answer)
  uint64_t* out_keys;     // nq x R (distance, CSR position)
  int nlist;              // bounds of the data-dependent indices
  int64_t ntotal;
  int* err;               // set to a site code if an index is out of range
  const int32_t* nprobe_q = nullptr;  // per-query nprobe (<= nprobe), may be null
  const int32_t* order = nullptr;     // scan order of the queries, may be null
  int* counter = nullptr;             // persistent grid: next position in `order`
  // index_ivf_pq.mojo:328-334: an entry whose id is below filter_len and has
  // filter[id] != 0 is skipped (ids: the id of each CSR entry)
  const uint8_t* filter = nullptr;
  int64_t filter_len = 0;
  const uint32_t* ids = nullptr;
  int cap, Rp;            // set by the launcher
  int rot = 0;            // set by the launcher: rotated-table pass width (0: none)
  int stage_entries = 0;  // staged scan: candidates per staged round (0: automatic)
};

// Bank-rotated fixed-point table scan (k_ivfpq_rt.cu): M a multiple of 4
// up to 32, dsub 4 or 8 with the FP16 codebook and its subspace norm bounds.
bool ivfpq_rt_supported(const FastScanArgs& a);
// One CTA (nt threads: 256 or 512) per query, or with a.counter a
// persistent grid of persistent_ctas CTAs.
void launch_ivfpq_scan_rt(FastScanArgs a, cudaStream_t s, int nt, int persistent_ctas);

// Two-kernel scan (k_ivfpq_rows.cu): per-candidate distance rows, then a
// per-query select; the same shortlist as the single-kernel FP32-table scan.
// smax bounds every query's candidate count (the nprobe longest lists); the
// rows take nq * ivfpq_rows_stride(smax) words of scratch.
int64_t ivfpq_rows_stride(int64_t smax);
// prof: context whose stage profiler times the ADC kernel alone (MV_STAGE_ADC), or null.
void launch_ivfpq_scan_rows(FastScanArgs f, uint32_t* dist, int64_t smax, cudaStream_t s, int nt,
                            mv_ctx* prof = nullptr);

struct RerankArgs {
  const float* q;
  int64_t nq;
  int d, metric;
  const float* raw;       // FP32 rows in CSR order
  const uint32_t* ids;    // id per CSR entry (null: the position is the id)
  const uint64_t* cand;   // nq x R shortlist keys
  int R, k;
  float* out_d;
  int64_t* out_l;
  int64_t ntotal;         // CSR entries (bound of the shortlist positions)
  int* err;
  float fill_d = 1e38f;   // distance of an unfilled slot (label -1)
  const int32_t* k_q = nullptr;  // per-query k (<= k; the row keeps k slots), may be null
  int kp;                 // set by the launcher
  // Certified prescreen (k <= 32; all null: every candidate is computed in
  // FP32): 8-bit copies of the rows (d8 bytes each) with y8_j =
  // fmaf(S_j, 1 + u_j 2^-15, a''_j) from the per-dimension (a''_j, S_j) in
  // dim8 (S_j = 2^15 s_j, a''_j = a_j - S_j), and per row upper bounds on
  // ||y - y8|| and on ||y8|| in rmeta.
  const uint8_t* raw8 = nullptr;
  const float2* rmeta = nullptr;
  const float2* dim8 = nullptr;
  int d8 = 0;
};

// Row bytes of the 8-bit prescreen copy of d-element rows.
inline int rerank8_row_bytes(int d) { return (d + 15) & ~15; }

// 8-bit copies of FP32 rows (CSR order) for the certified rerank prescreen:
// per dimension j an offset a_j (the minimum over the rows) and a step s_j
// (the smallest power of two with 255 s_j >= max_j - min_j), codes
// u = round((y_j - a_j) / s_j), and per row upper bounds on ||y - y8|| and
// ||y8|| with y8_j = fmaf(S_j, 1 + u_j 2^-15, a_j - S_j), S_j = 2^15 s_j.
// dimord holds 2 d words of scratch.
void launch_rerank_rows8(const float* raw, int64_t n, int d, uint32_t* dimord, float2* dim8,
                         uint8_t* raw8, float2* rmeta, cudaStream_t s);

// Two-pass coarse GEMM lists (launch_coarse_topk2) -> the nprobe nearest
// lists, as launch_coarse_rows (one warp per query; nseg * cap <= 256).
// The same lists -> each row's nc (<= 32) smallest keys, sorted, padded with
// KEY_NONE to next_pow2(nc) per row.
void launch_lists_smallest(const uint64_t* lists, const int* counts, int nseg, int cap, int64_t nq,
                           int nc, uint64_t* out, cudaStream_t s);
void launch_coarse_lists(const uint64_t* lists, const int* counts, int nseg, int cap, int64_t nq,
                         int nlist, const float* q, int d, const float* cent, int metric, int nc,
                         int nprobe, int32_t* probes, float* term, int* err, cudaStream_t s);
void launch_vec_terms(const int64_t* off, int nlist, const uint8_t* codes, const float* pq,
                      const float* cent, int d, int M, float* out, cudaStream_t s);
// Top-nc of the approximate coarse distances, exact FP32 recheck, top-nprobe.
void launch_coarse_fast(const float* approx, int64_t nq, int nlist, const float* q, int d,
                        const float* cent, int metric, int nc, int nprobe, int32_t* probes,
                        float* term, int* err, cudaStream_t s);
// Same with one warp per query and a lane-minimum threshold (nc <= 64).
void launch_coarse_rows(const float* approx, int64_t nq, int nlist, const float* q, int d,
                        const float* cent, int metric, int nc, int nprobe, int32_t* probes,
                        float* term, int* err, cudaStream_t s);
// Same from per-row candidate keys (ncand per row, KEY_NONE padded).
void launch_coarse_from_keys(const uint64_t* cand, int64_t nq, int ncand, const float* q, int d,
                             const float* cent, int nlist, int metric, int nc, int nprobe,
                             int32_t* probes, float* term, int* err, cudaStream_t s);
size_t fast_scan_smem(const FastScanArgs& a);
// The staged scan (k_ivfpq_scan.cu); returns false, launching nothing, when
// its shared memory would not fit (the caller runs the unstaged kernel).
bool launch_ivfpq_scan_staged(FastScanArgs a, cudaStream_t s, int nt, int persistent_ctas, int E);
// lut: 0 or 2 = FP32 tables read with codes from global memory (with 0 the
// search itself may take the two-kernel scan instead, same results); 6 = the
// bank-rotated fixed-point table scan with per-candidate slots
// (k_ivfpq_rt.cu) or an error; 7 = the two-kernel scan (distance rows and a
// per-query select, launched by the search itself); 1 = FP16 tables with a per-query
// power-of-two scale (FP32 sums), 3 = bank-rotated fixed-point tables in
// the per-candidate layout where M allows (else FP32), 4 = FP32 tables with
// codes and terms staged in shared memory by bulk copies (the unstaged
// kernel when that does not fit).
void launch_ivfpq_scan_fast(FastScanArgs a, cudaStream_t s, int nt = 256, int persistent_ctas = 0,
                            int lut = 0);
// Flat fast form: merge nseg x ncp per-segment keys (kseg kept per segment)
// into the R-key shortlist per query. With out_keys the shortlist is
// written (unsorted) for the rerank; otherwise the k smallest become the
// results (L2 adds qnorm back). overflow[q] = 1 when a segment may have
// dropped a shortlist key (only possible when kseg < R); may be null.
// SQ8 tensor-core scan: per-segment (-e, row) keys -> the R smallest
// canonical (SQ8 distance, row) keys per query (unsorted, KEY_NONE padded);
// flag[q] = 1 when a dropped row could tie into the shortlist.
void launch_sq8_merge(const uint64_t* cand, int64_t nq, int nseg, int ncp, int kseg, int R,
                      const uint32_t* qnorm, bool ip, float scale_sq, uint64_t* out_keys, int* flag,
                      cudaStream_t s);
void launch_flat_merge(const uint64_t* cand, int64_t nq, int nseg, int ncp, int kseg, int R,
                       uint64_t* out_keys, int k, const float* qnorm, int metric, float fill_d,
                       float* out_d, int64_t* out_l, int* overflow, cudaStream_t s);
void launch_rerank_fast(RerankArgs a, cudaStream_t s);
void launch_short_to_results(const uint64_t* keys, int64_t nq, int R, int k, const uint32_t* ids,
                             int metric, float* out_d, int64_t* out_l, cudaStream_t s,
                             const int32_t* k_q = nullptr);

}  // namespace mv
