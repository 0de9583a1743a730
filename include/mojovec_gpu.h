/*
 * mojovec_gpu.h - C ABI of libmojovec_gpu.so, the GB300 (sm_103a) hot path
 * for MojoVec's vector-query and index-training path.
 *
 * Every entry point uses plain C types: float / int64_t / uint8_t pointers
 * and sizes. Host-pointer entry points take caller-owned host buffers (numpy
 * arrays, Mojo Lists) exactly as the reference passes Spans; "_device"
 * entry points take device pointers and a cudaStream_t passed as void*.
 *
 * Status convention: every function returns int32_t, MV_OK (0) on success or
 * a negative MV_ERR_* code; mv_last_error() returns the calling thread's last
 * message. The reference's index-level search/add cannot raise
 * (core/index.mojo:5-32); its collection layer raises. A Mojo shim therefore
 * raises on a non-zero status at the collection layer.
 *
 * Forms:
 *   MV_FORM_PLAIN - FP32 form that reproduces the reference CPU path: codes,
 *                   coarse assignments and ids bit-exact, ties broken by the
 *                   smaller id, distances equal to the FP32 reference order.
 *   MV_FORM_FAST  - tensor-core coarse/base GEMMs (BF16, FP32 accumulate),
 *                   per-query LUTs with per-vector precomputed terms and an
 *                   exact FP32 rerank of a shortlist; judged on recall.
 *
 * Ids: the GPU index stores ids in [0, 2^32 - 2]; add rejects others with
 * MV_ERR_ARG. The canonical result order is (distance asc, id asc).
 */
#ifndef MOJOVEC_GPU_H
#define MOJOVEC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MV_OK 0
#define MV_ERR_ARG (-1)
#define MV_ERR_OOM (-2)
#define MV_ERR_CUDA (-3)
#define MV_ERR_TIMEOUT (-4)
#define MV_ERR_STATE (-5)
#define MV_ERR_UNSUPPORTED (-6)
#define MV_ERR_INTERNAL (-7)

/* core/types.mojo:5-7 */
#define MV_METRIC_L2 0
#define MV_METRIC_IP 1

#define MV_FORM_PLAIN 0
#define MV_FORM_FAST 1

typedef struct mv_ctx mv_ctx;
typedef struct mv_ivfpq mv_ivfpq;
typedef struct mv_flat mv_flat;
typedef struct mv_sq8 mv_sq8;
typedef struct mv_ivfpq_plan mv_ivfpq_plan;
typedef struct mv_server mv_server;
typedef struct mv_ivfflat mv_ivfflat;

/* Search options for the IVF-PQ and Flat searches. Zero-initialised means
 * the plain form with the index's own nprobe. */
typedef struct mv_search_params {
  int32_t form;        /* MV_FORM_PLAIN or MV_FORM_FAST */
  int32_t nprobe;      /* 0 = the index's nprobe (index_ivf_pq.mojo:253) */
  int32_t rerank;      /* fast form: shortlist depth for the exact FP32 rerank
                          (0 = no rerank) */
  int32_t coarse_fp32; /* fast form: 1 = FP32 SIMT coarse instead of BF16 */
  int32_t lut_fp16;    /* fast form, table and scan variant: 0 or 2 = FP32 tables (0 may
                          run them as two kernels, per-candidate distance rows then a
                          per-query select, where that pays; 7 always does),
                          1 = FP16 tables, 3 = bank-rotated 32-bit fixed-point tables
                          (M a multiple of 4 and at least 8; else FP32), 4 = FP32
                          tables with the probed lists staged in shared memory by
                          bulk copies, 6 = bank-rotated fixed-point tables with one
                          staging slot per candidate and a range select (M a
                          multiple of 4 up to 32, d / M = 4 or 8; else an error).
                          0, 2, 4 and 7 return the same bits */
  int32_t coarse_path; /* fast form, BF16 coarse step: 0 = automatic, 1 = GEMM with a
                          per-row top-k epilogue, 2 = distance matrix then one warp
                          per query selecting its lists, 3 = two-pass GEMM (bucket
                          threshold, then per-row lists; nprobe + margin <= 32 and
                          d <= 256). All keep the same lists; automatic takes 3
                          where it applies, else 2 */
  int32_t plain_scan;  /* plain form, Flat and SQ8: 1 = the exact SIMT scan alone, without
                          the tensor-core shortlist that is proven (Flat) or exact by
                          construction (SQ8) to give the same results */
  int32_t flat_e4m3;   /* fast form, Flat: 1 = shortlist from an E4M3 (FP8) GEMM with
                          per-row scales instead of BF16 (exact FP32 rerank either way) */
  int32_t rerank_fp32; /* fast form, IVF-PQ: 1 = every shortlisted row reranked from its FP32
                          copy; 0 (default, k <= 32) = a certified prescreen from an
                          8-bit copy of the rows first, which provably leaves the
                          results unchanged */
} mv_search_params;

/* ---- library / context ---------------------------------------------- */

/* Copies the calling thread's last error message (NUL-terminated). */
int32_t mv_last_error(char* buf, size_t len);
/* Library version string, e.g. "mojovec-gb300 0.1 sm_103a". */
const char* mv_version(void);
/* Creates a context bound to one CUDA device. */
int32_t mv_ctx_create(int32_t device, mv_ctx** out);
int32_t mv_ctx_destroy(mv_ctx* ctx);
/* Waits for all work issued through ctx. */
int32_t mv_ctx_synchronize(mv_ctx* ctx);
/* Number of kernels this context launched since creation (for reports). */
int64_t mv_ctx_kernel_launches(mv_ctx* ctx);
/* Failure detection. Every wait inside a tensor-core kernel is bounded; when
 * one gives up, the kernel stops, lets its issued copies and MMAs finish,
 * frees its tensor memory, and the call returns MV_ERR_TIMEOUT with the
 * context still usable. `cycles` is how long a pipeline wait may take (SM
 * clock cycles; default 4e9, about 2 s at 2.07 GHz); 0 makes every wait that
 * is not already satisfied give up at once (a diagnostic setting that tests
 * the timeout path); negative restores the default. No reference
 * counterpart: the reference runs on the CPU and has no device waits. */
int32_t mv_ctx_set_wait_limit(mv_ctx* ctx, int64_t cycles);

/* Stage profiling: when enabled, each search stage is bracketed by CUDA
 * events on the stream it runs on. Stage ids (MV_STAGE_*) index the arrays
 * read by mv_ctx_stage_times (total milliseconds and launch counts since the
 * last enable). Enabling resets the totals. */
#define MV_STAGE_COARSE 0   /* query x centroid distances */
#define MV_STAGE_SELECT 1   /* top-nprobe / top-k selection passes */
#define MV_STAGE_SCAN 2     /* IVF-PQ LUT + ADC scan */
#define MV_STAGE_LUT 3      /* per-query lookup tables (fast form) */
#define MV_STAGE_RERANK 4   /* exact FP32 rerank */
#define MV_STAGE_FLAT 5     /* Flat / SQ8 distance tiles */
#define MV_STAGE_ENCODE 6   /* residuals + PQ codes of added rows */
#define MV_STAGE_APPEND 7   /* list append: CSR layout + scatter */
#define MV_STAGE_ADC 8      /* table + ADC kernel of the two-kernel fast scan (inside SCAN) */
#define MV_STAGE_COUNT 9
int32_t mv_ctx_profile(mv_ctx* ctx, int32_t enable);
/* Plain-form selections run on the tensor cores with an exact FP32 recheck
 * and an error bound that proves the result equals the exact scan's;
 * selections the bound cannot settle take the exact FP32 scan. out4: rows
 * assigned to their nearest centroid that way (index add, training, plain
 * k-means), how many of them took the exact scan, plain Flat queries
 * answered that way, how many of them took the exact scan (since context
 * creation). */
int32_t mv_ctx_certify_stats(mv_ctx* ctx, int64_t* out4);
int32_t mv_ctx_stage_times(mv_ctx* ctx, double* ms, int64_t* counts, int32_t nstages);

/* ---- IVF-PQ index: replaces IndexIVFPQ[IndexFlat]
 *      (index/index_ivf_pq.mojo:12-360) -------------------------------- */

/* IndexIVFPQ.__init__ (index_ivf_pq.mojo:35-71): M divides d, nlist in
 * [1, 1e6], metric L2 or IP. ksub is 256 (pq.mojo:93). nprobe starts at 1. */
int32_t mv_ivfpq_create(mv_ctx* ctx, int32_t d, int32_t nlist, int32_t M, int32_t metric,
                        mv_ivfpq** out);
int32_t mv_ivfpq_destroy(mv_ivfpq* index);
/* Field nprobe (index_ivf_pq.mojo:22). */
int32_t mv_ivfpq_set_nprobe(mv_ivfpq* index, int32_t nprobe);
/* Reads d, nlist, M, nprobe, ntotal, metric, is_trained (index_ivf_pq.mojo:19-33). */
int32_t mv_ivfpq_info(mv_ivfpq* index, int64_t* out7);
/* Loads trained codebooks (host): centroids nlist x d, pq M x 256 x (d/M).
 * Marks the index trained. The path that takes the reference's own trained
 * codebooks. */
int32_t mv_ivfpq_set_codebooks(mv_ivfpq* index, const float* centroids, const float* pq);
int32_t mv_ivfpq_get_codebooks(mv_ivfpq* index, float* centroids, float* pq);
/* IndexIVFPQ.train (index_ivf_pq.mojo:87-136): coarse k-means (niter_coarse,
 * the reference uses 15), index-metric assignment, residual PQ k-means
 * (niter_pq, reference 15) on the GPU in the plain exact form. */
int32_t mv_ivfpq_train(mv_ivfpq* index, const float* x, int64_t n, int32_t niter_coarse,
                       int32_t niter_pq);
/* Train with a form: MV_FORM_FAST runs the coarse k-means in its fast form
 * (tensor-core assignment with FP32 recheck, FP64 sums; d <= 256). */
int32_t mv_ivfpq_train_ex(mv_ivfpq* index, const float* x, int64_t n, int32_t niter_coarse,
                          int32_t niter_pq, const mv_search_params* params);
/* IndexIVFPQ.add (index_ivf_pq.mojo:138-148): sequential ids from ntotal. */
int32_t mv_ivfpq_add(mv_ivfpq* index, const float* x, int64_t n);
/* IndexIVFPQ.add_with_ids (index_ivf_pq.mojo:150-213). */
int32_t mv_ivfpq_add_with_ids(mv_ivfpq* index, const float* x, const int64_t* ids, int64_t n);
/* Exports the inverted lists as CSR: offsets[nlist+1], ids[ntotal],
 * codes[ntotal*M] (storage/inverted_lists.mojo:93-117 per list). */
int32_t mv_ivfpq_get_lists(mv_ivfpq* index, int64_t* offsets, int64_t* ids, uint8_t* codes);
/* Replaces the inverted lists with CSR data (offsets nlist + 1, ids and
 * M-byte codes per entry), e.g. lists built by the reference. Such an index
 * has no rows: the plain search and the fast form without rerank work. */
int32_t mv_ivfpq_set_lists(mv_ivfpq* index, const int64_t* offsets, const int64_t* ids,
                           const uint8_t* codes);
/* CollectionIVFPQ snapshots (api/collection_ivfpq.mojo:335-476): the
 * collection header (name, metric "l2" / "cosine" / "ip", user ids), the
 * IndexIVFPQ body (io/serialization.mojo:1024-1090) and the checksum trailer
 * (io/snapshot_file.mojo:64-108). load applies the reference's validation and
 * builds the device CSR directly; the loaded index carries no FP32 rows (the
 * snapshot has none), so the fast form runs without rerank. save writes the
 * same bytes the reference would for these lists (capacity written as size),
 * through a temporary file and a rename. */
int32_t mv_ivfpq_load_snapshot(mv_ctx* ctx, const char* path, mv_ivfpq** out);
int32_t mv_ivfpq_save_snapshot(mv_ivfpq* index, const char* path, const char* name,
                               const char* metric, const int64_t* user_ids, int64_t num_ids);
/* Collection metadata of a loaded snapshot: name and metric as
 * NUL-terminated strings (truncated to the buffer), user ids (num_ids of
 * them, indexed by internal id). Any output may be NULL. */
int32_t mv_ivfpq_snapshot_info(mv_ivfpq* index, char* name, size_t name_len, char* metric,
                               size_t metric_len, int64_t* user_ids, int64_t* num_ids);
/* The snapshot checksum of a payload (io/snapshot_file.mojo:19-61): seed
 * 0xD6E8FEB86659FD93, 8 MiB chunks. */
uint64_t mv_snapshot_checksum(const void* payload, size_t bytes);
/* IndexIVFPQ.search (index_ivf_pq.mojo:215-360), host buffers. filter may be
 * NULL; filter[id] != 0 excludes id (:328-334). Results distances[nq*k],
 * labels[nq*k]; unfilled slots are 1e38 / -1 (:284-286). params may be NULL
 * (plain form, index nprobe). */
int32_t mv_ivfpq_search(mv_ivfpq* index, const float* x, int64_t nq, int32_t k,
                        const uint8_t* filter, int64_t filter_len,
                        const mv_search_params* params, float* distances, int64_t* labels);
/* Same with device buffers on `stream` (cudaStream_t; NULL = the context's
 * own stream). Returns after enqueueing; results are ready when the stream
 * is. */
int32_t mv_ivfpq_search_device(mv_ivfpq* index, const float* d_x, int64_t nq, int32_t k,
                               const uint8_t* d_filter, int64_t filter_len,
                               const mv_search_params* params, float* d_distances,
                               int64_t* d_labels, void* stream);

/* Plain IVF-PQ search that allocates no device memory. No counterpart in
 * the reference: it exists for callers that cannot allocate while they
 * search, such as a serving process that gives all GPU memory to its own
 * pool at start-up, or a host loop that must not absorb cudaFree's implicit
 * device synchronisation. Inputs and outputs are device buffers owned by the
 * caller (d_x nq*d, d_distances / d_labels nq*k); nprobe 0 means the
 * index's nprobe; no filter. Its scratch is one fixed array of
 * MV_NOALLOC_SCRATCH_BYTES inside the library, held by every GPU that loads
 * it until the process exits; queries are processed in batches that fit,
 * and a configuration whose single query needs more scratch is rejected with
 * MV_ERR_ARG. The first call on a device resolves the array's address (make
 * it before any stream capture). All calls share the array: calls that
 * overlap on the GPU race and must be serialised by the caller. Returns
 * after enqueueing on `stream` (NULL = the legacy default stream). */
#define MV_NOALLOC_SCRATCH_BYTES (8u * 1024u * 1024u)
int32_t mv_ivfpq_search_noalloc(mv_ivfpq* index, const float* d_x, int64_t nq, int32_t k,
                                int32_t nprobe, float* d_distances, int64_t* d_labels,
                                void* stream);

/* ---- Batched IVF-PQ (fast form): per-query nprobe and k ---------------- */
/* One call over queries with their own nprobe (<= nprobe_max) and k
 * (<= kmax). Results: nq rows of kmax slots; slots past a query's k read
 * 1e38 / -1 (index_ivf_pq.mojo:284-286). */
int32_t mv_ivfpq_search_batch(mv_ivfpq* index, const float* x, int64_t nq, const int32_t* nprobe,
                              const int32_t* k, int32_t kmax, const mv_search_params* params,
                              float* distances, int64_t* labels);
/* A plan owns device buffers for up to max_nq queries of a batched search
 * and replays it as a CUDA graph (captured once per batch size). The scan
 * runs as a persistent grid that takes queries from a counter in order of
 * decreasing nprobe. */
int32_t mv_ivfpq_plan_create(mv_ivfpq* index, int64_t max_nq, int32_t nprobe_max, int32_t kmax,
                             const mv_search_params* params, mv_ivfpq_plan** out);
int32_t mv_ivfpq_plan_destroy(mv_ivfpq_plan* plan);
/* Device pointers of the plan's buffers (any may be NULL): queries
 * (max_nq x d), per-query nprobe, k and scan order, results (max_nq x kmax). */
int32_t mv_ivfpq_plan_buffers(mv_ivfpq_plan* plan, float** d_x, int32_t** d_nprobe, int32_t** d_k,
                              int32_t** d_order, float** d_distances, int64_t** d_labels);
/* Copies host per-query nprobe / k (and x when not NULL) into the plan and
 * sets the scan order. */
int32_t mv_ivfpq_plan_set_queries(mv_ivfpq_plan* plan, const float* x, int64_t nq,
                                  const int32_t* nprobe, const int32_t* k);
/* Tuner: times the plan's launch choices on its current batch and keeps the
 * fastest. config (may be NULL): [coarse by distance matrix (1) or fused
 * top-k GEMM (0), scan threads per CTA, scan CTAs per SM (0 = one per
 * query)]; best_ms: the chosen configuration's time. */
int32_t mv_ivfpq_plan_tune(mv_ivfpq_plan* plan, int64_t nq, int32_t* config, float* best_ms);
/* Runs the plan on its first nq queries; use_graph != 0 replays a CUDA graph.
 * stream NULL: the plan's own stream, and the call returns when done. */
int32_t mv_ivfpq_plan_run(mv_ivfpq_plan* plan, int64_t nq, int32_t use_graph, void* stream);
/* Copies the first nq result rows (nq x kmax) to host memory after all
 * pending work on the device. */
int32_t mv_ivfpq_plan_results(mv_ivfpq_plan* plan, int64_t nq, float* distances, int64_t* labels);

/* ---- Serving loop: continuous batching over resident collections ------- */
/* A server batches submitted requests per (collection, k) in arrival order
 * (up to max_batch_queries rows per batch) and runs them on `lanes` worker
 * streams; a batch is admitted when a lane is idle and its device-memory
 * estimate fits hbm_budget_bytes beside the batches in flight. Requests that
 * arrive while others run are admitted as lanes and memory free up. Each
 * request gets the same results alone and in any mix. */
int32_t mv_server_create(mv_ctx* ctx, int64_t hbm_budget_bytes, int32_t lanes,
                         int64_t max_batch_queries, mv_server** out);
/* Finishes queued and running requests, then stops the server. */
int32_t mv_server_destroy(mv_server* server);
/* Registers a collection searched with `params` (form, nprobe, rerank);
 * returns its id. The index must outlive the server. */
int32_t mv_server_add_ivfpq(mv_server* server, mv_ivfpq* index, const mv_search_params* params,
                            int32_t* id);
int32_t mv_server_add_flat(mv_server* server, mv_flat* index, const mv_search_params* params,
                           int32_t* id);
int32_t mv_server_add_sq8(mv_server* server, mv_sq8* index, int32_t rerank_factor,
                          const mv_search_params* params, int32_t* id);
/* Queues nq query rows (copied; x is free on return) for collection `id`;
 * distances / labels (nq x k) are written before mv_server_wait returns. A
 * request above the server's max_batch_queries is split into parts of at
 * most that many rows; it completes when its last part does. MV_ERR_ARG when
 * one part's memory estimate exceeds the HBM budget. */
int32_t mv_server_submit(mv_server* server, int32_t id, const float* x, int64_t nq, int32_t k,
                         float* distances, int64_t* labels, int64_t* request_id);
/* Blocks until the request is done; returns its status and the latency from
 * submit to completion in seconds (may be NULL). */
int32_t mv_server_wait(mv_server* server, int64_t request_id, double* latency_s);
/* [completed requests, batches, queries in batches, peak in-flight device
 * bytes (estimate)]. */
int32_t mv_server_stats(mv_server* server, int64_t* out4);
/* [peak number of batches that were on the device at the same instant, number
 * of batches recorded]: each batch's device interval runs from its input
 * copy to its result copy (CUDA events on its lane's stream); the most recent
 * few thousand batches are kept. Shows that lanes overlap on the device. No
 * reference counterpart (the reference has no serving loop). */
int32_t mv_server_device_overlap(mv_server* server, int64_t* out2);

/* ---- IVF-Flat (index/index_ivf_flat.mojo:10-243) ----------------------- */
int32_t mv_ivfflat_create(mv_ctx* ctx, int32_t d, int32_t nlist, int32_t metric, mv_ivfflat** out);
int32_t mv_ivfflat_destroy(mv_ivfflat* index);
int32_t mv_ivfflat_set_nprobe(mv_ivfflat* index, int32_t nprobe);
int64_t mv_ivfflat_ntotal(mv_ivfflat* index);
/* train (:65-77): k-means of nlist centroids, niter iterations (the
 * reference uses 15); params->form FAST runs the fast k-means. */
int32_t mv_ivfflat_train(mv_ivfflat* index, const float* x, int64_t n, int32_t niter,
                         const mv_search_params* params);
int32_t mv_ivfflat_get_centroids(mv_ivfflat* index, float* centroids);
/* add / add_with_ids (:79-135): rows kept exactly, in list order. */
int32_t mv_ivfflat_add(mv_ivfflat* index, const float* x, int64_t n);
int32_t mv_ivfflat_add_with_ids(mv_ivfflat* index, const float* x, const int64_t* ids, int64_t n);
/* search (:137-243): exact l2_distance_simd[8] / -inner_product_simd[4]
 * over the nprobe nearest lists, tail 1e38 / -1, IP un-negated. PLAIN is
 * bit-exact; FAST takes the probes from the BF16 coarse step. */
int32_t mv_ivfflat_search(mv_ivfflat* index, const float* x, int64_t nq, int32_t k,
                          const mv_search_params* params, float* distances, int64_t* labels);
/* Same with device buffers, enqueued on `stream` (null: the call's own
 * stream, synchronised). */
int32_t mv_ivfflat_search_device(mv_ivfflat* index, const float* d_x, int64_t nq, int32_t k,
                                 const mv_search_params* params, float* d_distances,
                                 int64_t* d_labels, void* stream);

/* ---- Flat index: replaces IndexFlat (index/index_flat.mojo:117-330) ---- */
int32_t mv_flat_create(mv_ctx* ctx, int32_t d, int32_t metric, mv_flat** out);
int32_t mv_flat_destroy(mv_flat* index);
/* IndexFlat.add (index_flat.mojo:185-210). */
int32_t mv_flat_add(mv_flat* index, const float* x, int64_t n);
int64_t mv_flat_ntotal(mv_flat* index);
/* IndexFlat.search (index_flat.mojo:229-325); filter[j] > 0 excludes row j
 * (:286-288). Unfilled slots (k > rows) are 0.0 / -1 (:232-238). */
int32_t mv_flat_search(mv_flat* index, const float* x, int64_t nq, int32_t k,
                       const uint8_t* filter, const mv_search_params* params,
                       float* distances, int64_t* labels);
/* Exact FP32 rerank of candidate lists against the index's rows, the HNSW
 * SQ8 shortlist rerank (index/index_hnsw.mojo:433-497): per query the k
 * smallest l2_distance_simd[64] / -inner_product_simd[64] over its ncand
 * candidate ids (-1 = empty slot), ascending, ties by the smaller id, tail
 * 0.0 / -1, IP un-negated. */
int32_t mv_flat_rerank(mv_flat* index, const float* x, int64_t nq, const int64_t* cand,
                       int32_t ncand, int32_t k, float* distances, int64_t* labels);
/* mv_flat_rerank with device buffers (index_hnsw.mojo:433-497 semantics),
 * enqueued on `stream` (null: synchronised). Candidate ids outside
 * [0, ntotal) count as empty slots (the host variant rejects them). */
int32_t mv_flat_rerank_device(mv_flat* index, const float* d_x, int64_t nq, const int64_t* d_cand,
                              int32_t ncand, int32_t k, float* d_distances, int64_t* d_labels,
                              void* stream);
int32_t mv_flat_search_device(mv_flat* index, const float* d_x, int64_t nq, int32_t k,
                              const uint8_t* d_filter, const mv_search_params* params,
                              float* d_distances, int64_t* d_labels, void* stream);

/* ---- Flat SQ8 index: replaces IndexFlatSQ8
 *      (index/index_flat_sq8.mojo:271-661) ------------------------------ */
int32_t mv_sq8_create(mv_ctx* ctx, int32_t d, int32_t metric, mv_sq8** out);
int32_t mv_sq8_destroy(mv_sq8* index);
/* IndexFlatSQ8.add (index_flat_sq8.mojo:365-476): global min/max, affine
 * UInt8 (L2) or symmetric Int8 (IP) codes, requantize on bound growth. */
int32_t mv_sq8_add(mv_sq8* index, const float* x, int64_t n);
/* out3 = {global_min, global_max, scale}. */
int32_t mv_sq8_params(mv_sq8* index, float* out3);
int64_t mv_sq8_ntotal(mv_sq8* index);
/* Codes (ntotal*d bytes) and norms (ntotal uint32). */
int32_t mv_sq8_get_codes(mv_sq8* index, uint8_t* codes, uint32_t* norms);
/* IndexFlatSQ8.search (index_flat_sq8.mojo:478-605): tail 0.0 / -1. */
int32_t mv_sq8_search(mv_sq8* index, const float* x, int64_t nq, int32_t k,
                      const uint8_t* filter, float* distances, int64_t* labels);
/* SQ8 shortlist of rerank_factor*k candidates reranked with exact FP32
 * distances on the retained rows (index/index_hnsw.mojo:433-497 semantics). */
int32_t mv_sq8_search_rerank(mv_sq8* index, const float* x, int64_t nq, int32_t k,
                             int32_t rerank_factor, float* distances, int64_t* labels);
/* SQ8 search with a form: MV_FORM_PLAIN is mv_sq8_search (rerank_factor 0)
 * or mv_sq8_search_rerank; MV_FORM_FAST takes the shortlist from the BF16
 * tensor cores over the codes (exact integer dot products) and returns the
 * same ids and distances as the plain form: used where exact (L2 for
 * d <= 129, IP for d <= 256), a query whose shortlist could differ through
 * a distance tie is rescanned with the integer kernel. */
int32_t mv_sq8_search_ex(mv_sq8* index, const float* x, int64_t nq, int32_t k,
                         const uint8_t* filter, int32_t rerank_factor,
                         const mv_search_params* params, float* distances, int64_t* labels);
/* Same on device buffers, enqueued on `stream` (NULL: a pool stream, and the
 * call returns when done). The SQ8 path synchronizes the stream before it
 * returns (it reads back the per-query tie flags). */
int32_t mv_sq8_search_device(mv_sq8* index, const float* d_x, int64_t nq, int32_t k,
                             const uint8_t* d_filter, int32_t rerank_factor,
                             const mv_search_params* params, float* d_distances,
                             int64_t* d_labels, void* stream);

/* ---- Training and encoding primitives --------------------------------- */

/* KMeans(d, k, niter).train (clustering/kmeans.mojo:60-220), plain exact
 * form: Philox init, 32-chunk FP32 accumulation in row order, ordered
 * chunk reduce, reciprocal-multiply update, deterministic reseed.
 * assignments (may be NULL) receive the last iteration's clusters. */
int32_t mv_kmeans_train(mv_ctx* ctx, const float* x, int64_t n, int32_t d, int32_t k,
                        int32_t niter, float* centroids, int64_t* assignments);
/* k-means with a form. MV_FORM_PLAIN is mv_kmeans_train. MV_FORM_FAST assigns
 * on the tensor cores (BF16 distances pick 4 candidate centroids per row, the
 * reference's FP32 distance picks among them) and accumulates the centroid
 * sums in FP64 in a fixed order (deterministic); same initial rows and empty-
 * cluster rule; d <= 256. objective (niter + 1 doubles, may be NULL): the sum
 * of squared distances at each assignment step and for the final centroids. */
int32_t mv_kmeans_train_ex(mv_ctx* ctx, const float* x, int64_t n, int32_t d, int32_t k,
                           int32_t niter, const mv_search_params* params, float* centroids,
                           int64_t* assignments, double* objective);
/* ProductQuantizer.train (quantization/pq.mojo:125-176): M subspace
 * k-means of 256 centroids each. out: M x 256 x (d/M). */
int32_t mv_pq_train(mv_ctx* ctx, const float* x, int64_t n, int32_t d, int32_t M,
                    int32_t niter, float* pq);
/* ProductQuantizer.compute_codes (pq.mojo:178-219). codes: n x M. */
int32_t mv_pq_encode(mv_ctx* ctx, const float* pq, int32_t d, int32_t M, const float* x,
                     int64_t n, uint8_t* codes);
/* ProductQuantizer.compute_distance_table (pq.mojo:252-292) for nq vectors:
 * tables nq x M x 256. */
int32_t mv_pq_distance_tables(mv_ctx* ctx, const float* pq, int32_t d, int32_t M,
                              const float* x, int64_t nq, int32_t metric, float* tables);
/* _encode_sq8_batch (quantization/sq8.mojo:41-59). */
int32_t mv_sq8_encode(mv_ctx* ctx, const float* x, int64_t n, int32_t d, float minimum,
                      float inverse_scale, int32_t symmetric, uint8_t* codes, uint32_t* norms);
/* Distance matrix out[nx*ny] between rows of x and y (host buffers).
 * precision 0: exact FP32 in the reference's l2_distance_simd[8] /
 * -inner_product_simd[8] order (distances.mojo:43-228);
 * precision 1: BF16 tensor cores (tcgen05) with FP32 accumulation,
 * ||x||^2 + ||y||^2 - 2 x.y over the BF16-rounded rows (d <= 256). */
int32_t mv_distance_matrix(mv_ctx* ctx, const float* x, int64_t nx, const float* y, int64_t ny,
                           int32_t d, int32_t metric, int32_t precision, float* out);
/* _normalize_vectors (api/collection_vector_query.mojo:24-46): FP64 sum of
 * squares, 1/sqrt in FP64. Returns MV_ERR_ARG for non-finite or zero rows. */
int32_t mv_normalize(mv_ctx* ctx, const float* x, int64_t n, int32_t d, float* out);

#ifdef __cplusplus
}
#endif

#endif /* MOJOVEC_GPU_H */
