// Inverted-list append on the device (storage/inverted_lists.mojo:162-186,
// index_ivf_pq.mojo:199-213, index_ivf_flat.mojo:118-133): n new entries with
// list numbers assign[i] join the CSR lists after each list's old entries,
// in input order; an entry whose list number is outside [0, nlist) is not
// stored (the reference skips it, index_ivf_pq.mojo:201) and is parked past
// the end.
//
// The new position of every old and new entry comes from a stable counting
// sort with one extra bucket (nlist) for the skipped rows: per-tile bucket
// counts, a column scan over tiles, one scan over buckets (giving the new
// offsets), and an in-order placement in which one warp walks its tile 32
// rows at a time, ranking equal buckets with __match_any_sync. Tiles grow
// with nlist so the tile x bucket table stays under LIST_HIST_MAX entries.
#include "mv_internal.h"
#include "mv_kernels.h"

namespace mv {
namespace {

constexpr int64_t LIST_HIST_MAX = 32ll << 20;  // int32 entries of the tile x bucket table
constexpr int LIST_TILE_MIN = 4096;

__device__ __forceinline__ int bucket_of(int32_t a, int nlist) {
  return (a >= 0 && a < nlist) ? a : nlist;
}

// hist[t][b] += rows of tile t in bucket b (hist zeroed beforehand).
template <bool SMEM>
__global__ void k_list_hist(const int32_t* __restrict__ assign, int64_t n, int nlist, int64_t tile,
                            int32_t* __restrict__ hist) {
  extern __shared__ int32_t cnt[];
  const int nb = nlist + 1;
  const int64_t t = blockIdx.x;
  int32_t* row = hist + t * nb;
  if (SMEM) {
    for (int b = threadIdx.x; b < nb; b += blockDim.x) cnt[b] = 0;
    __syncthreads();
  }
  const int64_t r0 = t * tile, r1 = r0 + tile < n ? r0 + tile : n;
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x)
    atomicAdd(SMEM ? &cnt[bucket_of(assign[r], nlist)] : &row[bucket_of(assign[r], nlist)], 1);
  if (SMEM) {
    __syncthreads();
    for (int b = threadIdx.x; b < nb; b += blockDim.x) row[b] = cnt[b];
  }
}

// hist[t][b] <- rows of bucket b in tiles before t; total[b].
__global__ void k_list_colscan(int32_t* __restrict__ hist, int64_t ntiles, int nb,
                               int64_t* __restrict__ total) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  int32_t run = 0;
  for (int64_t t = 0; t < ntiles; ++t) {
    const int32_t h = hist[t * nb + b];
    hist[t * nb + b] = run;
    run += h;
  }
  total[b] = run;
}

// One block: new_off[l] = sum over l' < l of (old size + added), l in
// [0, nlist]; start[l] = new_off[l] + old size of l (first new slot of l);
// start[nlist] = new_off[nlist] (the skipped rows follow the lists).
__global__ void k_list_offsets(const int64_t* __restrict__ old_off, const int64_t* __restrict__ total,
                               int nlist, int64_t* __restrict__ new_off, int64_t* __restrict__ start) {
  __shared__ int64_t part[1024];
  const int per = (nlist + blockDim.x - 1) / blockDim.x;
  const int l0 = threadIdx.x * per;
  const int l1 = min(l0 + per, nlist);
  int64_t s = 0;
  for (int l = l0; l < l1; ++l) s += (old_off[l + 1] - old_off[l]) + total[l];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t run = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      const int64_t v = part[i];
      part[i] = run;
      run += v;
    }
    new_off[nlist] = run;
    start[nlist] = run;
  }
  __syncthreads();
  int64_t run = part[threadIdx.x];
  for (int l = l0; l < l1; ++l) {
    new_off[l] = run;
    start[l] = run + (old_off[l + 1] - old_off[l]);
    run += (old_off[l + 1] - old_off[l]) + total[l];
  }
}

// One warp per tile: pos_new[r] = start[b] + (rows of b before r), in row
// order. hist row t (its own) is the running count.
__global__ void k_list_place(const int32_t* __restrict__ assign, int64_t n, int nlist, int64_t tile,
                             int32_t* __restrict__ hist, const int64_t* __restrict__ start,
                             int64_t* __restrict__ pos_new) {
  const int nb = nlist + 1;
  const int64_t t = blockIdx.x;
  const int lane = threadIdx.x;
  int32_t* cur = hist + t * nb;
  const int64_t r0 = t * tile, r1 = r0 + tile < n ? r0 + tile : n;
  for (int64_t g = r0; g < r1; g += 32) {
    const int64_t r = g + lane;
    const bool ok = r < r1;
    const int b = ok ? bucket_of(assign[r], nlist) : -1 - lane;  // distinct for idle lanes
    const unsigned peers = __match_any_sync(0xffffffffu, b);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    const int leader = __ffs(peers) - 1;
    int64_t pos = 0;
    if (ok) pos = start[b] + cur[b] + rank;
    __syncwarp();
    if (ok && lane == leader) cur[b] += __popc(peers);
    __syncwarp();
    if (ok) pos_new[r] = pos;
  }
}

// pos_old[p] = p - old_off[l] + new_off[l] for the list l holding entry p.
__global__ void k_list_pos_old(const int64_t* __restrict__ old_off, const int64_t* __restrict__ new_off,
                               int nlist, int64_t old_total, int64_t* __restrict__ pos_old) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= old_total) return;
  int lo = 0, hi = nlist;  // largest l with old_off[l] <= p (and a non-empty list)
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (old_off[mid] <= p) lo = mid;
    else hi = mid;
  }
  pos_old[p] = p - old_off[lo] + new_off[lo];
}

int64_t list_tile(int64_t n, int nlist) {
  const int64_t nb = (int64_t)nlist + 1;
  int64_t tile = LIST_TILE_MIN;
  while (((n + tile - 1) / tile) * nb > LIST_HIST_MAX) tile *= 2;
  return tile;
}

}  // namespace

size_t list_append_scratch_bytes(int64_t n, int nlist) {
  const int64_t nb = (int64_t)nlist + 1;
  const int64_t ntiles = (n + list_tile(n, nlist) - 1) / list_tile(n, nlist);
  return (size_t)(ntiles * nb) * 4 + (size_t)nb * 8 * 2 + 64;
}

void launch_list_append_layout(const int32_t* assign, int64_t n, int nlist, const int64_t* old_off,
                               int64_t old_total, int64_t* new_off, int64_t* pos, void* scratch,
                               cudaStream_t s) {
  MV_REQUIRE(n < (1ll << 31), MV_ERR_UNSUPPORTED, "at most 2^31 - 1 rows per append");
  const int nb = nlist + 1;
  const int64_t tile = list_tile(n, nlist);
  const int64_t ntiles = n ? (n + tile - 1) / tile : 0;
  int64_t* total = static_cast<int64_t*>(scratch);
  int64_t* start = total + nb;
  int32_t* hist = reinterpret_cast<int32_t*>(start + nb);
  if (ntiles) {
    MV_CHECK_CUDA(cudaMemsetAsync(hist, 0, (size_t)(ntiles * nb) * 4, s));
    const size_t smem = (size_t)nb * 4;
    if (smem <= 96 * 1024) {
      smem_limit(k_list_hist<true>, smem);
      k_list_hist<true><<<(unsigned)ntiles, 512, smem, s>>>(assign, n, nlist, tile, hist);
    } else {
      k_list_hist<false><<<(unsigned)ntiles, 512, 0, s>>>(assign, n, nlist, tile, hist);
    }
    count_launch();
    k_list_colscan<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(hist, ntiles, nb, total);
    count_launch();
  } else {
    MV_CHECK_CUDA(cudaMemsetAsync(total, 0, (size_t)nb * 8, s));
  }
  k_list_offsets<<<1, 1024, 0, s>>>(old_off, total, nlist, new_off, start);
  count_launch();
  if (old_total) {
    k_list_pos_old<<<(unsigned)((old_total + 255) / 256), 256, 0, s>>>(old_off, new_off, nlist,
                                                                      old_total, pos);
    count_launch();
  }
  if (ntiles) {
    k_list_place<<<(unsigned)ntiles, 32, 0, s>>>(assign, n, nlist, tile, hist, start, pos + old_total);
    count_launch();
  }
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
