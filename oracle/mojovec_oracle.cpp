// MojoVec hot-path oracle: a C++17 restatement of the reference's CPU path.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker for the CUDA product
// (libmojovec_gpu.so). Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg may load it. The product never links, imports or calls it.
//
// Parity status: the reference is Mojo (mojo==1.0.0b2) and cannot be built or
// run here, so this restatement is pinned only by the known-answer tests in
// the reference's own test suite (tests/test_pq.mojo:57-114,
// tests/test_index_flat.mojo:6-81, tests/test_distances_simd.mojo:87-129,
// tests/test_metrics.mojo:56-96, tests/test_ivf_pq.mojo:30-77,
// tests/test_ivf_flat.mojo:91-137, tests/test_kmeans.mojo:32-72) and by the
// published Philox4x32-10 known-answer vectors. Three Mojo stdlib semantics
// are fixed by documented choice (bit-level parity with real Mojo output is
// unpinned for them):
//   * SIMD.reduce_add: halving tree (lane i += lane i+W/2, repeated);
//   * no contraction of a*b+c outside explicit fma;
//   * math.round: round half away from zero (C roundf).
//
// Every function cites the reference file:line it restates (paths relative
// to the MojoVec project root).
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fno-fast-math -shared -fPIC
// (oracle/build_oracle.py). -ffp-contract=off keeps every product and sum
// separately rounded; explicit std::fma is used only where the reference
// calls fma.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <thread>
#include <vector>

namespace {

constexpr int METRIC_L2 = 0;
constexpr int METRIC_IP = 1;

// ---------------------------------------------------------------------------
// SIMD emulation helpers
// ---------------------------------------------------------------------------

// SIMD.reduce_add: recursive split into lower/upper halves added lane-wise.
template <int W>
inline float tree_sum(float* v) {
  for (int h = W / 2; h >= 1; h /= 2)
    for (int i = 0; i < h; ++i) v[i] = v[i] + v[i + h];
  return v[0];
}

// utils/distances.mojo:43-143  l2_distance_simd[W]
template <int W>
float l2_simd(const float* x, const float* y, int64_t d) {
  if (d < W) {  // :57-62 scalar path
    float r = 0.0f;
    for (int64_t i = 0; i < d; ++i) {
      float diff = x[i] - y[i];
      r = r + diff * diff;
    }
    return r;
  }
  float a0[W], a1[W], a2[W], a3[W];
  for (int l = 0; l < W; ++l) a0[l] = a1[l] = a2[l] = a3[l] = 0.0f;
  int64_t i = 0;
  while (i <= d - 4 * W) {  // :75-96
    for (int l = 0; l < W; ++l) {
      float d0 = x[i + l] - y[i + l];
      a0[l] = std::fma(d0, d0, a0[l]);
      float d1 = x[i + W + l] - y[i + W + l];
      a1[l] = std::fma(d1, d1, a1[l]);
      float d2 = x[i + 2 * W + l] - y[i + 2 * W + l];
      a2[l] = std::fma(d2, d2, a2[l]);
      float d3 = x[i + 3 * W + l] - y[i + 3 * W + l];
      a3[l] = std::fma(d3, d3, a3[l]);
    }
    i += 4 * W;
  }
  float s[W];
  for (int l = 0; l < W; ++l) s[l] = ((a0[l] + a1[l]) + a2[l]) + a3[l];  // :98
  while (i <= d - W) {  // :101-106
    for (int l = 0; l < W; ++l) {
      float df = x[i + l] - y[i + l];
      s[l] = std::fma(df, df, s[l]);
    }
    i += W;
  }
  float res = tree_sum<W>(s);  // :108
  if (W >= 32) {               // :110-117
    while (i <= d - 16) {
      float r[16];
      for (int l = 0; l < 16; ++l) {
        float df = x[i + l] - y[i + l];
        r[l] = df * df;
      }
      res = res + tree_sum<16>(r);
      i += 16;
    }
  }
  if (W >= 16) {  // :119-126
    while (i <= d - 8) {
      float r[8];
      for (int l = 0; l < 8; ++l) {
        float df = x[i + l] - y[i + l];
        r[l] = df * df;
      }
      res = res + tree_sum<8>(r);
      i += 8;
    }
  }
  if (W >= 8) {  // :128-135
    while (i <= d - 4) {
      float r[4];
      for (int l = 0; l < 4; ++l) {
        float df = x[i + l] - y[i + l];
        r[l] = df * df;
      }
      res = res + tree_sum<4>(r);
      i += 4;
    }
  }
  while (i < d) {  // :138-141
    float df = x[i] - y[i];
    res = res + df * df;
    ++i;
  }
  return res;
}

// utils/distances.mojo:146-228  inner_product_simd[W]
template <int W>
float ip_simd(const float* x, const float* y, int64_t d) {
  if (d < W) {  // :158-162
    float r = 0.0f;
    for (int64_t i = 0; i < d; ++i) r = r + x[i] * y[i];
    return r;
  }
  float p0[W], p1[W], p2[W], p3[W];
  for (int l = 0; l < W; ++l) p0[l] = p1[l] = p2[l] = p3[l] = 0.0f;
  int64_t i = 0;
  while (i <= d - 4 * W) {  // :170-187
    for (int l = 0; l < W; ++l) {
      p0[l] = std::fma(x[i + l], y[i + l], p0[l]);
      p1[l] = std::fma(x[i + W + l], y[i + W + l], p1[l]);
      p2[l] = std::fma(x[i + 2 * W + l], y[i + 2 * W + l], p2[l]);
      p3[l] = std::fma(x[i + 3 * W + l], y[i + 3 * W + l], p3[l]);
    }
    i += 4 * W;
  }
  float s[W];
  for (int l = 0; l < W; ++l) s[l] = ((p0[l] + p1[l]) + p2[l]) + p3[l];  // :189
  while (i <= d - W) {  // :191-195
    for (int l = 0; l < W; ++l) s[l] = std::fma(x[i + l], y[i + l], s[l]);
    i += W;
  }
  float res = tree_sum<W>(s);  // :197
  if (W >= 32) {
    while (i <= d - 16) {  // :199-205
      float r[16];
      for (int l = 0; l < 16; ++l) r[l] = std::fma(x[i + l], y[i + l], 0.0f);
      res = res + tree_sum<16>(r);
      i += 16;
    }
  }
  if (W >= 16) {
    while (i <= d - 8) {  // :207-213
      float r[8];
      for (int l = 0; l < 8; ++l) r[l] = std::fma(x[i + l], y[i + l], 0.0f);
      res = res + tree_sum<8>(r);
      i += 8;
    }
  }
  if (W >= 8) {
    while (i <= d - 4) {  // :215-221
      float r[4];
      for (int l = 0; l < 4; ++l) r[l] = std::fma(x[i + l], y[i + l], 0.0f);
      res = res + tree_sum<4>(r);
      i += 4;
    }
  }
  while (i < d) {  // :224-226
    res = res + x[i] * y[i];
    ++i;
  }
  return res;
}

// utils/distances.mojo:9-23  l2_distance_short4
float l2_short4(const float* x, const float* y, int64_t d) {
  if (d == 4) {
    float r[4];
    for (int l = 0; l < 4; ++l) {
      float df = x[l] - y[l];
      r[l] = df * df;
    }
    return tree_sum<4>(r);
  }
  float res = 0.0f;
  for (int64_t i = 0; i < d; ++i) {
    float df = x[i] - y[i];
    res = res + df * df;
  }
  return res;
}

// utils/distances.mojo:27-39  inner_product_short4
float ip_short4(const float* x, const float* y, int64_t d) {
  if (d == 4) {
    float r[4];
    for (int l = 0; l < 4; ++l) r[l] = x[l] * y[l];
    return tree_sum<4>(r);
  }
  float res = 0.0f;
  for (int64_t i = 0; i < d; ++i) res = res + x[i] * y[i];
  return res;
}

float l2_w(int W, const float* x, const float* y, int64_t d) {
  switch (W) {
    case 4: return l2_simd<4>(x, y, d);
    case 8: return l2_simd<8>(x, y, d);
    case 16: return l2_simd<16>(x, y, d);
    case 32: return l2_simd<32>(x, y, d);
    case 64: return l2_simd<64>(x, y, d);
    default: return l2_simd<8>(x, y, d);
  }
}

float ip_w(int W, const float* x, const float* y, int64_t d) {
  switch (W) {
    case 4: return ip_simd<4>(x, y, d);
    case 8: return ip_simd<8>(x, y, d);
    case 16: return ip_simd<16>(x, y, d);
    case 32: return ip_simd<32>(x, y, d);
    case 64: return ip_simd<64>(x, y, d);
    default: return ip_simd<8>(x, y, d);
  }
}

// ---------------------------------------------------------------------------
// Heaps (utils/heap.mojo:17-213), exact semantics
// ---------------------------------------------------------------------------

// utils/heap.mojo:17-54 max_heap_replace_top
void heap_replace_top(float* hd, int64_t* hl, int64_t k, float dist, int64_t label) {
  hd[0] = dist;
  hl[0] = label;
  int64_t i = 0;
  while (true) {
    int64_t left = 2 * i + 1, right = 2 * i + 2, largest = i;
    if (left < k && hd[left] > hd[largest]) largest = left;
    if (right < k && hd[right] > hd[largest]) largest = right;
    if (largest == i) break;
    std::swap(hd[i], hd[largest]);
    std::swap(hl[i], hl[largest]);
    i = largest;
  }
}

// utils/heap.mojo:56-84 max_heap_push
void heap_push(float* hd, int64_t* hl, int64_t size, float dist, int64_t label) {
  int64_t i = size;
  hd[i] = dist;
  hl[i] = label;
  while (i > 0) {
    int64_t parent = (i - 1) / 2;
    if (hd[parent] < hd[i]) {
      std::swap(hd[i], hd[parent]);
      std::swap(hl[i], hl[parent]);
      i = parent;
    } else {
      break;
    }
  }
}

// utils/heap.mojo:167-213 max_heap_pop
void heap_pop(float* hd, int64_t* hl, int64_t size, float* od, int64_t* ol) {
  *od = hd[0];
  *ol = hl[0];
  int64_t last = size - 1;
  if (last == 0) return;
  hd[0] = hd[last];
  hl[0] = hl[last];
  int64_t i = 0;
  while (true) {
    int64_t left = 2 * i + 1, right = 2 * i + 2, largest = i;
    if (left < last && hd[left] > hd[largest]) largest = left;
    if (right < last && hd[right] > hd[largest]) largest = right;
    if (largest == i) break;
    std::swap(hd[i], hd[largest]);
    std::swap(hl[i], hl[largest]);
    i = largest;
  }
}

// Canonical order: (distance ascending, id ascending). -0.0 equals +0.0.
inline bool key_less(float da, int64_t ia, float db, int64_t ib) {
  if (da < db) return true;
  if (db < da) return false;
  return ia < ib;
}

// Top-k collector. mode 0 = the reference heap (strict `<` against the top,
// pops to ascending order); mode 1 = canonical k smallest by (dist, id).
struct TopK {
  int mode;
  int64_t k;
  float* d;
  int64_t* l;
  int64_t size = 0;
  TopK(int mode_, int64_t k_, float* d_, int64_t* l_) : mode(mode_), k(k_), d(d_), l(l_) {}

  void push(float dist, int64_t label) {
    if (mode == 0) {
      if (size < k) {
        heap_push(d, l, size, dist, label);
        ++size;
      } else if (dist < d[0]) {
        heap_replace_top(d, l, k, dist, label);
      }
      return;
    }
    // canonical: max-heap ordered by (dist, id)
    if (size < k) {
      int64_t i = size++;
      d[i] = dist;
      l[i] = label;
      while (i > 0) {
        int64_t p = (i - 1) / 2;
        if (key_less(d[p], l[p], d[i], l[i])) {
          std::swap(d[p], d[i]);
          std::swap(l[p], l[i]);
          i = p;
        } else {
          break;
        }
      }
    } else if (key_less(dist, label, d[0], l[0])) {
      d[0] = dist;
      l[0] = label;
      int64_t i = 0;
      while (true) {
        int64_t a = 2 * i + 1, b = 2 * i + 2, g = i;
        if (a < k && key_less(d[g], l[g], d[a], l[a])) g = a;
        if (b < k && key_less(d[g], l[g], d[b], l[b])) g = b;
        if (g == i) break;
        std::swap(d[i], d[g]);
        std::swap(l[i], l[g]);
        i = g;
      }
    }
  }

  // Pops everything into ascending order at d[0..size). Returns the count.
  int64_t finish() {
    int64_t n = size;
    if (mode == 0) {
      std::vector<float> td(d, d + n);
      std::vector<int64_t> tl(l, l + n);
      int64_t hs = n;
      for (int64_t j = 0; j < n; ++j) {
        float pd;
        int64_t pl;
        heap_pop(td.data(), tl.data(), hs, &pd, &pl);
        --hs;
        d[n - 1 - j] = pd;
        l[n - 1 - j] = pl;
      }
    } else {
      std::vector<std::pair<float, int64_t>> v(n);
      for (int64_t j = 0; j < n; ++j) v[j] = {d[j], l[j]};
      std::sort(v.begin(), v.end(), [](const auto& a, const auto& b) {
        return key_less(a.first, a.second, b.first, b.second);
      });
      for (int64_t j = 0; j < n; ++j) {
        d[j] = v[j].first;
        l[j] = v[j].second;
      }
    }
    return n;
  }
};

template <typename F>
void parallel_for(int64_t n, int nthreads, F&& f) {
  if (nthreads <= 1 || n <= 1) {
    for (int64_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<int64_t> next{0};
  std::vector<std::thread> ts;
  int nt = (int)std::min<int64_t>(nthreads, n);
  for (int t = 0; t < nt; ++t) {
    ts.emplace_back([&]() {
      while (true) {
        int64_t i = next.fetch_add(1);
        if (i >= n) break;
        f(i);
      }
    });
  }
  for (auto& t : ts) t.join();
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), standing in for
// std.random.philox.Random(seed) used at clustering/kmeans.mojo:70-82.
// Key = (seed low 32, seed high 32); counter = (offset lo, offset hi,
// subsequence lo, subsequence hi) starting at zero, incremented by one per
// step() with carry.
// ---------------------------------------------------------------------------
struct Philox {
  uint32_t key[2];
  uint32_t ctr[4];
  explicit Philox(uint64_t seed) {
    key[0] = (uint32_t)seed;
    key[1] = (uint32_t)(seed >> 32);
    ctr[0] = ctr[1] = ctr[2] = ctr[3] = 0;
  }
  static void round(uint32_t* c, const uint32_t* k) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k[0];
    uint32_t n2 = hi0 ^ c[3] ^ k[1];
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
  }
  static void block(const uint32_t* in_ctr, const uint32_t* in_key, uint32_t* out) {
    uint32_t c[4] = {in_ctr[0], in_ctr[1], in_ctr[2], in_ctr[3]};
    uint32_t k[2] = {in_key[0], in_key[1]};
    for (int r = 0; r < 10; ++r) {
      if (r > 0) {
        k[0] += 0x9E3779B9u;
        k[1] += 0xBB67AE85u;
      }
      round(c, k);
    }
    for (int i = 0; i < 4; ++i) out[i] = c[i];
  }
  void step(uint32_t* out) {
    block(ctr, key, out);
    for (int i = 0; i < 4; ++i) {
      if (++ctr[i] != 0) break;
    }
  }
};

// ---------------------------------------------------------------------------
// K-means (clustering/kmeans.mojo:60-220)
// ---------------------------------------------------------------------------
constexpr uint64_t KMEANS_SEED = 0x4D4F4A4F564543ull;  // kmeans.mojo:70

// Distance used by the assign step: short4 for d <= 4, else l2_simd[8]
// (kmeans.mojo:131-139).
inline float kmeans_dist(const float* x, const float* c, int d) {
  return d <= 4 ? l2_short4(x, c, d) : l2_simd<8>(x, c, d);
}

void kmeans_train(const float* x, int64_t n, int d, int k, int niter, int nthreads,
                  float* centroids, int64_t* assignments) {
  if (n == 0) return;  // :62
  // :70-82 Philox-seeded initialisation
  Philox gen(KMEANS_SEED);
  uint32_t words[4];
  gen.step(words);
  int64_t sample_offset = (int64_t)(words[0] % (uint32_t)n);
  for (int i = 0; i < k; ++i) {
    if (i != 0 && i % 4 == 0) gen.step(words);
    int64_t src = (int64_t)(words[i % 4] % (uint32_t)n);
    std::memcpy(centroids + (int64_t)i * d, x + src * d, sizeof(float) * d);
  }
  const int num_chunks = 32;  // :84
  int64_t chunk_size = (n + num_chunks - 1) / num_chunks;
  std::vector<float> local_c((size_t)num_chunks * k * d);
  std::vector<int64_t> local_n((size_t)num_chunks * k);
  std::vector<int64_t> counts(k);
  std::vector<int64_t> assign_store(n);
  int64_t* assign = assignments ? assignments : assign_store.data();

  for (int it = 0; it < niter; ++it) {
    std::fill(local_c.begin(), local_c.end(), 0.0f);  // :101-106
    std::fill(local_n.begin(), local_n.end(), 0);
    // :114-161 fused assign + accumulate per chunk
    parallel_for(num_chunks, nthreads, [&](int64_t chunk) {
      int64_t start = chunk * chunk_size;
      int64_t end = std::min(start + chunk_size, n);
      float* my_c = local_c.data() + chunk * (int64_t)k * d;
      int64_t* my_n = local_n.data() + chunk * (int64_t)k;
      for (int64_t i = start; i < end; ++i) {
        float min_dist = 1e38f;
        int best = -1;
        const float* xp = x + i * d;
        for (int c = 0; c < k; ++c) {
          float dist = kmeans_dist(xp, centroids + (int64_t)c * d, d);
          if (dist < min_dist) {
            min_dist = dist;
            best = c;
          }
        }
        int c = std::max(best, 0);
        assign[i] = c;
        my_n[c] += 1;
        float* cp = my_c + (int64_t)c * d;
        for (int j = 0; j < d; ++j) cp[j] = cp[j] + xp[j];
      }
    });
    // :170-195 ordered reduce over chunks
    for (int c = 0; c < k; ++c) {
      counts[c] = 0;
      std::fill(centroids + (int64_t)c * d, centroids + (int64_t)(c + 1) * d, 0.0f);
    }
    for (int chunk = 0; chunk < num_chunks; ++chunk) {
      const float* my_c = local_c.data() + (int64_t)chunk * k * d;
      const int64_t* my_n = local_n.data() + (int64_t)chunk * k;
      for (int c = 0; c < k; ++c) {
        counts[c] += my_n[c];
        float* cp = centroids + (int64_t)c * d;
        const float* sp = my_c + (int64_t)c * d;
        for (int j = 0; j < d; ++j) cp[j] = cp[j] + sp[j];
      }
    }
    // :197-220 reciprocal-multiply update; deterministic empty reseed
    for (int c = 0; c < k; ++c) {
      float* cp = centroids + (int64_t)c * d;
      if (counts[c] > 0) {
        float inv = 1.0f / (float)counts[c];
        for (int j = 0; j < d; ++j) cp[j] = cp[j] * inv;
      } else {
        int64_t src = (sample_offset + (int64_t)(it + 1) * k + c) % n;
        std::memcpy(cp, x + src * d, sizeof(float) * d);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Product quantizer (quantization/pq.mojo)
// ---------------------------------------------------------------------------
struct PQ {
  int d, M, ksub, dsub;
  std::vector<float> centroids;  // [M][ksub][dsub]
};

// pq.mojo:45-69, :125-176 (one subspace per thread, serial k-means each)
void pq_train(PQ& pq, const float* x, int64_t n, int niter, int nthreads) {
  parallel_for(pq.M, nthreads, [&](int64_t m) {
    std::vector<float> sub((size_t)n * pq.dsub);
    for (int64_t i = 0; i < n; ++i)
      for (int j = 0; j < pq.dsub; ++j)
        sub[i * pq.dsub + j] = x[i * pq.d + m * pq.dsub + j];
    std::vector<float> cent((size_t)pq.ksub * pq.dsub);
    kmeans_train(sub.data(), n, pq.dsub, pq.ksub, niter, 1, cent.data(), nullptr);
    std::memcpy(pq.centroids.data() + m * (int64_t)pq.ksub * pq.dsub, cent.data(),
                sizeof(float) * pq.ksub * pq.dsub);
  });
}

// pq.mojo:178-219
// Rows are encoded independently (the reference loops over them serially);
// nthreads only splits the rows, so the codes do not depend on it.
void pq_compute_codes(const PQ& pq, const float* x, int64_t n, uint8_t* codes, int nthreads = 1) {
  parallel_for(n, nthreads, [&](int64_t i) {
    const float* xp = x + i * pq.d;
    for (int m = 0; m < pq.M; ++m) {
      float min_dist = 1e38f;
      int best = -1;
      const float* sub = xp + m * pq.dsub;
      const float* cm = pq.centroids.data() + (int64_t)m * pq.ksub * pq.dsub;
      for (int kk = 0; kk < pq.ksub; ++kk) {
        const float* cp = cm + (int64_t)kk * pq.dsub;
        float dist = pq.dsub <= 4 ? l2_short4(sub, cp, pq.dsub) : l2_simd<8>(sub, cp, pq.dsub);
        if (dist < min_dist) {
          min_dist = dist;
          best = kk;
        }
      }
      codes[i * pq.M + m] = (uint8_t)best;  // UInt8(-1) wraps to 255
    }
  });
}

// pq.mojo:221-250
void pq_decode(const PQ& pq, const uint8_t* codes, int64_t n, float* x) {
  for (int64_t i = 0; i < n; ++i)
    for (int m = 0; m < pq.M; ++m) {
      const float* cp = pq.centroids.data() + ((int64_t)m * pq.ksub + codes[i * pq.M + m]) * pq.dsub;
      std::memcpy(x + i * pq.d + m * pq.dsub, cp, sizeof(float) * pq.dsub);
    }
}

// pq.mojo:252-292
void pq_distance_table(const PQ& pq, const float* q, int metric, float* table) {
  for (int m = 0; m < pq.M; ++m) {
    const float* sq = q + m * pq.dsub;
    const float* cm = pq.centroids.data() + (int64_t)m * pq.ksub * pq.dsub;
    float* tm = table + (int64_t)m * pq.ksub;
    for (int kk = 0; kk < pq.ksub; ++kk) {
      const float* cp = cm + (int64_t)kk * pq.dsub;
      if (metric == METRIC_L2)
        tm[kk] = pq.dsub <= 4 ? l2_short4(sq, cp, pq.dsub) : l2_simd<8>(sq, cp, pq.dsub);
      else
        tm[kk] = -(pq.dsub <= 4 ? ip_short4(sq, cp, pq.dsub) : ip_simd<4>(sq, cp, pq.dsub));
    }
  }
}

// ---------------------------------------------------------------------------
// IndexFlat search (index/index_flat.mojo:229-325)
// ---------------------------------------------------------------------------
// Results for query i land at dist[i*k .. i*k+k). Entries past the number of
// candidates are left untouched (the reference leaves them unwritten).
void flat_search(const float* base, int64_t nb, int d, int metric, const float* q, int64_t nq,
                 int64_t k, const uint8_t* filter, int mode, float* dist, int64_t* labels,
                 int nthreads) {
  parallel_for(nq, nthreads, [&](int64_t i) {
    const float* qp = q + i * d;
    TopK top(mode, k, dist + i * k, labels + i * k);
    for (int64_t j = 0; j < nb; ++j) {
      if (filter && filter[j] > 0) continue;  // :286-288
      const float* bp = base + j * d;
      float dd = metric == METRIC_L2 ? l2_simd<8>(qp, bp, d) : -ip_simd<8>(qp, bp, d);
      top.push(dd, j);
    }
    int64_t cnt = top.finish();
    if (metric == METRIC_IP) {
      // :314-316 un-negates all k slots; only the written ones are defined.
      for (int64_t j = 0; j < cnt; ++j) dist[i * k + j] = -dist[i * k + j];
    }
  });
}

// ---------------------------------------------------------------------------
// IndexIVFPQ (index/index_ivf_pq.mojo) with ArrayInvertedLists storage
// (storage/inverted_lists.mojo:37-186).
// ---------------------------------------------------------------------------
struct IVFPQ {
  int d, nlist, M, metric;
  bool trained = false;
  int64_t ntotal = 0;
  std::vector<float> centroids;  // quantizer IndexFlat rows
  PQ pq;
  std::vector<std::vector<int64_t>> list_ids;
  std::vector<std::vector<uint8_t>> list_codes;
};

void ivfpq_assign(const IVFPQ& ix, const float* x, int64_t n, int64_t* labels, int nthreads) {
  // quantizer.search(x, 1): index metric, reference heap with k=1.
  std::vector<float> dd(n);
  flat_search(ix.centroids.data(), ix.nlist, ix.d, ix.metric, x, n, 1, nullptr, 0, dd.data(),
              labels, nthreads);
}

// index_ivf_pq.mojo:87-136
void ivfpq_train(IVFPQ& ix, const float* x, int64_t n, int niter_coarse, int niter_pq,
                 int nthreads) {
  if (ix.trained) return;
  ix.centroids.assign((size_t)ix.nlist * ix.d, 0.0f);
  kmeans_train(x, n, ix.d, ix.nlist, niter_coarse, nthreads, ix.centroids.data(), nullptr);
  std::vector<int64_t> lab(n);
  ivfpq_assign(ix, x, n, lab.data(), nthreads);
  std::vector<float> res((size_t)n * ix.d);
  for (int64_t i = 0; i < n; ++i) {
    int64_t l = lab[i];
    if (l < 0 || l >= ix.nlist) l = 0;
    for (int j = 0; j < ix.d; ++j) res[i * ix.d + j] = x[i * ix.d + j] - ix.centroids[l * ix.d + j];
  }
  pq_train(ix.pq, res.data(), n, niter_pq, nthreads);
  ix.trained = true;
}

// index_ivf_pq.mojo:150-213 (+ inverted_lists.mojo:162-186 append)
void ivfpq_add_with_ids(IVFPQ& ix, const float* x, int64_t n, const int64_t* ids, int nthreads) {
  if (!ix.trained) return;
  std::vector<int64_t> lab(n);
  ivfpq_assign(ix, x, n, lab.data(), nthreads);
  std::vector<float> res((size_t)n * ix.d);
  for (int64_t i = 0; i < n; ++i) {
    int64_t l = lab[i];
    if (l < 0 || l >= ix.nlist) l = 0;
    for (int j = 0; j < ix.d; ++j) res[i * ix.d + j] = x[i * ix.d + j] - ix.centroids[l * ix.d + j];
  }
  std::vector<uint8_t> codes((size_t)n * ix.M);
  pq_compute_codes(ix.pq, res.data(), n, codes.data(), nthreads);
  for (int64_t i = 0; i < n; ++i) {
    int64_t l = lab[i];
    if (l < 0 || l >= ix.nlist) continue;
    ix.list_ids[l].push_back(ids[i]);
    ix.list_codes[l].insert(ix.list_codes[l].end(), codes.begin() + i * ix.M,
                            codes.begin() + (i + 1) * ix.M);
  }
  ix.ntotal += n;
}

// index_ivf_pq.mojo:225-360. mode 0 = reference heaps everywhere; mode 1 =
// canonical (dist, id) selection for both the coarse top-nprobe and the
// top-k. nthreads parallelises the coarse step (as the reference does) and,
// when lut_threads > 1, the per-query LUT+ADC loop (the reference runs that
// loop serially; > 1 is the labelled all-cores variant).
void ivfpq_search(const IVFPQ& ix, const float* x, int64_t n, int64_t k, int64_t nprobe,
                  const uint8_t* filter, int64_t filter_len, int mode, float* distances,
                  int64_t* labels, int nthreads, int lut_threads) {
  if (!ix.trained || ix.ntotal == 0) {  // :247-251
    for (int64_t i = 0; i < n * k; ++i) {
      distances[i] = 1e38f;
      labels[i] = -1;
    }
    return;
  }
  if (nprobe > ix.nlist) nprobe = ix.nlist;  // :253-254
  std::vector<float> qd((size_t)n * nprobe);
  std::vector<int64_t> ql((size_t)n * nprobe);
  flat_search(ix.centroids.data(), ix.nlist, ix.d, ix.metric, x, n, nprobe, nullptr, mode,
              qd.data(), ql.data(), nthreads);  // :264
  const int ksub = ix.pq.ksub;
  parallel_for(n, lut_threads, [&](int64_t i) {  // :276
    std::vector<float> table((size_t)ix.M * ksub);
    std::vector<float> resid(ix.d);
    const float* qp = x + i * ix.d;
    float* rd = distances + i * k;
    int64_t* rl = labels + i * k;
    for (int64_t j = 0; j < k; ++j) {  // :284-286
      rd[j] = 1e38f;
      rl[j] = -1;
    }
    TopK top(mode, k, rd, rl);
    if (ix.metric == METRIC_IP) pq_distance_table(ix.pq, qp, ix.metric, table.data());  // :288-293
    for (int64_t p = 0; p < nprobe; ++p) {
      int64_t list_no = ql[i * nprobe + p];
      if (list_no < 0 || list_no >= ix.nlist) continue;
      const auto& ids = ix.list_ids[list_no];
      const auto& codes = ix.list_codes[list_no];
      int64_t ls = (int64_t)ids.size();
      if (ls == 0) continue;
      float coarse = 0.0f;
      const float* cp = ix.centroids.data() + list_no * ix.d;
      if (ix.metric == METRIC_L2) {  // :306-315
        for (int j = 0; j < ix.d; ++j) resid[j] = qp[j] - cp[j];
        pq_distance_table(ix.pq, resid.data(), ix.metric, table.data());
      } else {  // :316-324
        coarse = -ip_simd<8>(qp, cp, ix.d);
      }
      for (int64_t j = 0; j < ls; ++j) {  // :326-347
        int64_t cid = ids[j];
        if (filter && cid >= 0 && cid < filter_len && filter[cid] != 0) continue;
        const uint8_t* c = codes.data() + j * ix.M;
        float dist = coarse;
        for (int m = 0; m < ix.M; ++m) dist = dist + table[(int64_t)m * ksub + c[m]];
        top.push(dist, cid);
      }
    }
    int64_t cnt = top.finish();
    if (ix.metric == METRIC_IP)
      for (int64_t j = 0; j < cnt; ++j) rd[j] = -rd[j];  // :357-360
  });
}

// ---------------------------------------------------------------------------
// IndexIVFFlat (index/index_ivf_flat.mojo:10-243): coarse k-means of 15
// iterations (:65-77), rows appended to the list of their nearest centroid
// in input order (:91-135), search over the nprobe nearest lists with
// l2_distance_simd[8] or -inner_product_simd[4] (:176-243; the filter
// argument is not applied there), tail 1e38 / -1, IP un-negated.
// ---------------------------------------------------------------------------
struct IVFFlat {
  int d, nlist, metric;
  bool trained = false;
  int64_t ntotal = 0;
  std::vector<float> centroids;
  std::vector<std::vector<int64_t>> list_ids;
  std::vector<std::vector<float>> list_rows;
};

void ivfflat_train(IVFFlat& ix, const float* x, int64_t n, int niter, int nthreads) {
  if (ix.trained) return;  // :71
  ix.centroids.assign((size_t)ix.nlist * ix.d, 0.0f);
  kmeans_train(x, n, ix.d, ix.nlist, niter, nthreads, ix.centroids.data(), nullptr);
  ix.trained = true;
}

void ivfflat_add_with_ids(IVFFlat& ix, const float* x, int64_t n, const int64_t* ids, int nthreads) {
  if (!ix.trained) return;  // :103-105
  std::vector<float> dd(n);
  std::vector<int64_t> lab(n);
  flat_search(ix.centroids.data(), ix.nlist, ix.d, ix.metric, x, n, 1, nullptr, 0, dd.data(),
              lab.data(), nthreads);  // :117, quantizer.search(x, 1)
  for (int64_t i = 0; i < n; ++i) {
    const int64_t l = lab[i];
    if (l < 0 || l >= ix.nlist) continue;  // :126
    ix.list_ids[l].push_back(ids[i]);
    ix.list_rows[l].insert(ix.list_rows[l].end(), x + i * ix.d, x + (i + 1) * ix.d);
  }
  ix.ntotal += n;
}

void ivfflat_search(const IVFFlat& ix, const float* x, int64_t n, int64_t k, int64_t nprobe,
                    int mode, float* distances, int64_t* labels, int nthreads) {
  if (!ix.trained || ix.ntotal == 0) {  // :176-180
    for (int64_t i = 0; i < n * k; ++i) {
      distances[i] = 1e38f;
      labels[i] = -1;
    }
    return;
  }
  if (nprobe > ix.nlist) nprobe = ix.nlist;  // :182-183
  std::vector<float> qd((size_t)n * nprobe);
  std::vector<int64_t> ql((size_t)n * nprobe);
  flat_search(ix.centroids.data(), ix.nlist, ix.d, ix.metric, x, n, nprobe, nullptr, mode,
              qd.data(), ql.data(), nthreads);
  parallel_for(n, nthreads, [&](int64_t i) {
    const float* qp = x + i * ix.d;
    float* rd = distances + i * k;
    int64_t* rl = labels + i * k;
    for (int64_t j = 0; j < k; ++j) {  // :201-203
      rd[j] = 1e38f;
      rl[j] = -1;
    }
    TopK top(mode, k, rd, rl);
    for (int64_t p = 0; p < nprobe; ++p) {
      const int64_t list_no = ql[i * nprobe + p];
      if (list_no < 0 || list_no >= ix.nlist) continue;
      const auto& ids = ix.list_ids[list_no];
      const float* rows = ix.list_rows[list_no].data();
      for (size_t j = 0; j < ids.size(); ++j) {
        const float* bp = rows + j * ix.d;
        const float dist = ix.metric == METRIC_L2 ? l2_simd<8>(qp, bp, ix.d)
                                                  : -ip_simd<4>(qp, bp, ix.d);  // :222-226
        top.push(dist, ids[j]);
      }
    }
    const int64_t cnt = top.finish();
    if (ix.metric == METRIC_IP)
      for (int64_t j = 0; j < cnt; ++j) rd[j] = -rd[j];  // :241-243
  });
}

// ---------------------------------------------------------------------------
// SQ8 codec (quantization/sq8.mojo) and IndexFlatSQ8
// (index/index_flat_sq8.mojo:286-526)
// ---------------------------------------------------------------------------
inline float clampf(float v, float lo, float hi) { return std::min(std::max(v, lo), hi); }

// sq8.mojo:13-38
uint32_t sq8_encode_vector(bool symmetric, const float* src, uint8_t* dst, int d, float minimum,
                           float inv_scale) {
  uint32_t norm = 0;
  if (symmetric) {
    for (int c = 0; c < d; ++c) {
      float scaled = std::round(src[c] * inv_scale);
      int8_t code = (int8_t)clampf(scaled, -127.0f, 127.0f);
      dst[c] = (uint8_t)code;
      int32_t w = code;
      norm += (uint32_t)(w * w);
    }
  } else {
    for (int c = 0; c < d; ++c) {
      float scaled = std::round((src[c] - minimum) * inv_scale);
      uint8_t code = (uint8_t)clampf(scaled, 0.0f, 255.0f);
      dst[c] = code;
      norm += (uint32_t)code * (uint32_t)code;
    }
  }
  return norm;
}

struct SQ8 {
  int d, metric;
  int64_t ntotal = 0;
  std::vector<float> f32;
  std::vector<uint8_t> codes;
  std::vector<uint32_t> norms;
  float gmin = std::numeric_limits<float>::max();
  float gmax = -std::numeric_limits<float>::max();
  float scale = 1.0f;
};

// index_flat_sq8.mojo:365-476
void sq8_add(SQ8& s, const float* x, int64_t n) {
  if (n == 0) return;
  float bmin = std::numeric_limits<float>::max(), bmax = -std::numeric_limits<float>::max();
  for (int64_t i = 0; i < n * s.d; ++i) {
    float v = x[i];
    if (v < bmin) bmin = v;
    if (v > bmax) bmax = v;
  }
  bool requant = false;
  if (bmin < s.gmin) {
    s.gmin = bmin;
    requant = true;
  }
  if (bmax > s.gmax) {
    s.gmax = bmax;
    requant = true;
  }
  if (s.metric == METRIC_L2) {
    s.scale = (s.gmax == s.gmin) ? 1.0f : (s.gmax - s.gmin) / 255.0f;
  } else {
    float max_abs = std::max(std::fabs(s.gmin), std::fabs(s.gmax));
    s.scale = max_abs > 0.0f ? max_abs / 127.0f : 1.0f;
  }
  float inv = 1.0f / s.scale;
  bool sym = s.metric != METRIC_L2;
  float mn = sym ? 0.0f : s.gmin;
  if (requant && s.ntotal > 0)
    for (int64_t i = 0; i < s.ntotal; ++i)
      s.norms[i] = sq8_encode_vector(sym, s.f32.data() + i * s.d, s.codes.data() + i * s.d, s.d,
                                     mn, inv);
  s.f32.insert(s.f32.end(), x, x + n * s.d);
  s.codes.resize((size_t)(s.ntotal + n) * s.d);
  s.norms.resize(s.ntotal + n);
  for (int64_t i = 0; i < n; ++i)
    s.norms[s.ntotal + i] = sq8_encode_vector(sym, x + i * s.d,
                                              s.codes.data() + (s.ntotal + i) * s.d, s.d, mn, inv);
  s.ntotal += n;
}

// sq8.mojo:62-79 and distances.mojo:236-451 (integer dots; order-free)
inline float sq8_code_distance(bool ip, const uint8_t* q, const uint8_t* b, uint32_t qn,
                               uint32_t bn, int d, float scale_sq) {
  if (ip) {
    int32_t dot = 0;
    for (int c = 0; c < d; ++c) dot += (int32_t)(int8_t)q[c] * (int32_t)(int8_t)b[c];
    return -(float)dot * scale_sq;
  }
  uint32_t dot = 0;
  for (int c = 0; c < d; ++c) dot += (uint32_t)q[c] * (uint32_t)b[c];
  int64_t dd = (int64_t)qn + (int64_t)bn - 2 * (int64_t)dot;  // distances.mojo:450-451
  uint32_t dist = (uint32_t)std::max<int64_t>(dd, 0);
  return (float)dist * scale_sq;
}

// index_flat_sq8.mojo:507-605. Tail filled with 0.0 / -1.
void sq8_search(const SQ8& s, const float* x, int64_t n, int64_t k, const uint8_t* filter,
                int mode, float* distances, int64_t* labels, int nthreads) {
  bool ip = s.metric != METRIC_L2;
  parallel_for(n, nthreads, [&](int64_t i) {
    std::vector<uint8_t> qc(s.d);
    float inv = 1.0f / s.scale;
    uint32_t qn = sq8_encode_vector(ip, x + i * s.d, qc.data(), s.d, ip ? 0.0f : s.gmin, inv);
    float scale_sq = s.scale * s.scale;
    TopK top(mode, k, distances + i * k, labels + i * k);
    for (int64_t j = 0; j < s.ntotal; ++j) {
      if (filter && filter[j] > 0) continue;
      float dd = sq8_code_distance(ip, qc.data(), s.codes.data() + j * s.d, qn, s.norms[j], s.d,
                                   scale_sq);
      top.push(dd, j);
    }
    int64_t cnt = top.finish();
    for (int64_t j = cnt; j < k; ++j) {
      distances[i * k + j] = 0.0f;
      labels[i * k + j] = -1;
    }
    if (ip)
      for (int64_t j = 0; j < cnt; ++j)
        if (labels[i * k + j] >= 0) distances[i * k + j] = -distances[i * k + j];
  });
}

}  // namespace

// ===========================================================================
// extern "C" surface for ctypes (tests, smoke, CPU baseline)
// ===========================================================================
extern "C" {

float orc_l2_simd(int W, const float* x, const float* y, int64_t d) { return l2_w(W, x, y, d); }
float orc_ip_simd(int W, const float* x, const float* y, int64_t d) { return ip_w(W, x, y, d); }
float orc_l2_short4(const float* x, const float* y, int64_t d) { return l2_short4(x, y, d); }
float orc_ip_short4(const float* x, const float* y, int64_t d) { return ip_short4(x, y, d); }

uint32_t orc_sq8_dot_u8(const uint8_t* x, const uint8_t* y, int64_t d) {
  uint32_t r = 0;
  for (int64_t i = 0; i < d; ++i) r += (uint32_t)x[i] * (uint32_t)y[i];
  return r;
}
int32_t orc_sq8_dot_s8(const int8_t* x, const int8_t* y, int64_t d) {
  int32_t r = 0;
  for (int64_t i = 0; i < d; ++i) r += (int32_t)x[i] * (int32_t)y[i];
  return r;
}

void orc_philox_block(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  Philox::block(ctr, key, out);
}
void orc_philox_steps(uint64_t seed, int64_t nsteps, uint32_t* out) {
  Philox g(seed);
  for (int64_t s = 0; s < nsteps; ++s) g.step(out + 4 * s);
}

void orc_kmeans_train(const float* x, int64_t n, int d, int k, int niter, int nthreads,
                      float* centroids, int64_t* assignments) {
  kmeans_train(x, n, d, k, niter, nthreads, centroids, assignments);
}

void orc_pq_train(const float* x, int64_t n, int d, int M, int ksub, int niter, int nthreads,
                  float* out) {
  PQ pq{d, M, ksub, d / M, std::vector<float>((size_t)M * ksub * (d / M))};
  pq_train(pq, x, n, niter, nthreads);
  std::memcpy(out, pq.centroids.data(), sizeof(float) * pq.centroids.size());
}
void orc_pq_compute_codes(const float* cent, int d, int M, int ksub, const float* x, int64_t n,
                          uint8_t* codes) {
  PQ pq{d, M, ksub, d / M, std::vector<float>(cent, cent + (size_t)M * ksub * (d / M))};
  pq_compute_codes(pq, x, n, codes);
}
void orc_pq_decode(const float* cent, int d, int M, int ksub, const uint8_t* codes, int64_t n,
                   float* x) {
  PQ pq{d, M, ksub, d / M, std::vector<float>(cent, cent + (size_t)M * ksub * (d / M))};
  pq_decode(pq, codes, n, x);
}
void orc_pq_distance_table(const float* cent, int d, int M, int ksub, const float* q, int metric,
                           float* table) {
  PQ pq{d, M, ksub, d / M, std::vector<float>(cent, cent + (size_t)M * ksub * (d / M))};
  pq_distance_table(pq, q, metric, table);
}

void orc_flat_search(const float* base, int64_t nb, int d, int metric, const float* q, int64_t nq,
                     int64_t k, const uint8_t* filter, int mode, float* dist, int64_t* labels,
                     int nthreads) {
  flat_search(base, nb, d, metric, q, nq, k, filter, mode, dist, labels, nthreads);
}

// --- IVF-PQ handle ---
void* orc_ivfpq_create(int d, int nlist, int M, int metric) {
  auto* ix = new IVFPQ();
  ix->d = d;
  ix->nlist = nlist;
  ix->M = M;
  ix->metric = metric;
  ix->pq = PQ{d, M, 256, d / M, std::vector<float>((size_t)256 * d)};
  ix->list_ids.resize(nlist);
  ix->list_codes.resize(nlist);
  return ix;
}
void orc_ivfpq_destroy(void* h) { delete static_cast<IVFPQ*>(h); }
void orc_ivfpq_train(void* h, const float* x, int64_t n, int niter_coarse, int niter_pq,
                     int nthreads) {
  ivfpq_train(*static_cast<IVFPQ*>(h), x, n, niter_coarse, niter_pq, nthreads);
}
void orc_ivfpq_set_codebooks(void* h, const float* centroids, const float* pq) {
  auto& ix = *static_cast<IVFPQ*>(h);
  ix.centroids.assign(centroids, centroids + (size_t)ix.nlist * ix.d);
  ix.pq.centroids.assign(pq, pq + (size_t)256 * ix.d);
  ix.trained = true;
}
void orc_ivfpq_get_codebooks(void* h, float* centroids, float* pq) {
  auto& ix = *static_cast<IVFPQ*>(h);
  std::memcpy(centroids, ix.centroids.data(), sizeof(float) * ix.centroids.size());
  std::memcpy(pq, ix.pq.centroids.data(), sizeof(float) * ix.pq.centroids.size());
}
void orc_ivfpq_add_with_ids(void* h, const float* x, int64_t n, const int64_t* ids,
                            int nthreads) {
  ivfpq_add_with_ids(*static_cast<IVFPQ*>(h), x, n, ids, nthreads);
}
void orc_ivfpq_add(void* h, const float* x, int64_t n, int nthreads) {
  auto& ix = *static_cast<IVFPQ*>(h);
  std::vector<int64_t> ids(n);
  for (int64_t i = 0; i < n; ++i) ids[i] = ix.ntotal + i;
  ivfpq_add_with_ids(ix, x, n, ids.data(), nthreads);
}
int64_t orc_ivfpq_ntotal(void* h) { return static_cast<IVFPQ*>(h)->ntotal; }
// Loads CSR lists (offsets[nlist+1], ids, codes) in place of adds; ntotal
// becomes offsets[nlist]. Used to search an index built elsewhere.
void orc_ivfpq_set_lists(void* h, const int64_t* offsets, const int64_t* ids,
                         const uint8_t* codes) {
  auto& ix = *static_cast<IVFPQ*>(h);
  for (int l = 0; l < ix.nlist; ++l) {
    ix.list_ids[l].assign(ids + offsets[l], ids + offsets[l + 1]);
    ix.list_codes[l].assign(codes + offsets[l] * ix.M, codes + offsets[l + 1] * ix.M);
  }
  ix.ntotal = offsets[ix.nlist];
}
// Exports the lists as CSR: offsets[nlist+1], ids[ntotal], codes[ntotal*M].
void orc_ivfpq_get_lists(void* h, int64_t* offsets, int64_t* ids, uint8_t* codes) {
  auto& ix = *static_cast<IVFPQ*>(h);
  int64_t off = 0;
  for (int l = 0; l < ix.nlist; ++l) {
    offsets[l] = off;
    int64_t s = (int64_t)ix.list_ids[l].size();
    std::memcpy(ids + off, ix.list_ids[l].data(), sizeof(int64_t) * s);
    std::memcpy(codes + off * ix.M, ix.list_codes[l].data(), (size_t)s * ix.M);
    off += s;
  }
  offsets[ix.nlist] = off;
}
void orc_ivfpq_search(void* h, const float* x, int64_t n, int64_t k, int64_t nprobe,
                      const uint8_t* filter, int64_t filter_len, int mode, float* dist,
                      int64_t* labels, int nthreads, int lut_threads) {
  ivfpq_search(*static_cast<IVFPQ*>(h), x, n, k, nprobe, filter, filter_len, mode, dist, labels,
               nthreads, lut_threads);
}

// --- SQ8 handle ---
void* orc_ivfflat_create(int d, int nlist, int metric) {
  auto* ix = new IVFFlat();
  ix->d = d;
  ix->nlist = nlist;
  ix->metric = metric;
  ix->list_ids.resize(nlist);
  ix->list_rows.resize(nlist);
  return ix;
}
void orc_ivfflat_destroy(void* h) { delete static_cast<IVFFlat*>(h); }
void orc_ivfflat_train(void* h, const float* x, int64_t n, int niter, int nthreads) {
  ivfflat_train(*static_cast<IVFFlat*>(h), x, n, niter, nthreads);
}
void orc_ivfflat_add(void* h, const float* x, int64_t n, int nthreads) {
  auto* ix = static_cast<IVFFlat*>(h);
  std::vector<int64_t> ids(n);
  for (int64_t i = 0; i < n; ++i) ids[i] = ix->ntotal + i;  // :86-89
  ivfflat_add_with_ids(*ix, x, n, ids.data(), nthreads);
}
void orc_ivfflat_centroids(void* h, float* out) {
  auto* ix = static_cast<IVFFlat*>(h);
  std::copy(ix->centroids.begin(), ix->centroids.end(), out);
}
void orc_ivfflat_search(void* h, const float* x, int64_t n, int64_t k, int64_t nprobe, int mode,
                        float* distances, int64_t* labels, int nthreads) {
  ivfflat_search(*static_cast<IVFFlat*>(h), x, n, k, nprobe, mode, distances, labels, nthreads);
}

void* orc_sq8_create(int d, int metric) {
  auto* s = new SQ8();
  s->d = d;
  s->metric = metric;
  return s;
}
void orc_sq8_destroy(void* h) { delete static_cast<SQ8*>(h); }
void orc_sq8_add(void* h, const float* x, int64_t n) { sq8_add(*static_cast<SQ8*>(h), x, n); }
void orc_sq8_params(void* h, float* out3) {
  auto& s = *static_cast<SQ8*>(h);
  out3[0] = s.gmin;
  out3[1] = s.gmax;
  out3[2] = s.scale;
}
void orc_sq8_get_codes(void* h, uint8_t* codes, uint32_t* norms) {
  auto& s = *static_cast<SQ8*>(h);
  std::memcpy(codes, s.codes.data(), s.codes.size());
  std::memcpy(norms, s.norms.data(), sizeof(uint32_t) * s.norms.size());
}
void orc_sq8_search(void* h, const float* x, int64_t n, int64_t k, const uint8_t* filter,
                    int mode, float* dist, int64_t* labels, int nthreads) {
  sq8_search(*static_cast<SQ8*>(h), x, n, k, filter, mode, dist, labels, nthreads);
}
// One-shot SQ8 encode with given parameters (sq8.mojo:41-59).
void orc_sq8_encode(int symmetric, const float* x, int64_t n, int d, float minimum,
                    float inv_scale, uint8_t* codes, uint32_t* norms) {
  for (int64_t i = 0; i < n; ++i)
    norms[i] = sq8_encode_vector(symmetric != 0, x + i * d, codes + i * d, d, minimum, inv_scale);
}

// Exact FP32 rerank of a candidate shortlist (index/index_hnsw.mojo:433-497):
// l2_distance_simd[64] / -inner_product_simd[64] on the retained FP32 rows,
// top-k of the candidates; tail 0.0 / -1; IP un-negated.
void orc_rerank(const float* base, int d, int metric, const float* q, int64_t nq,
                const int64_t* cand, int64_t ncand, int64_t k, int mode, float* dist,
                int64_t* labels, int nthreads) {
  parallel_for(nq, nthreads, [&](int64_t i) {
    TopK top(mode, k, dist + i * k, labels + i * k);
    for (int64_t c = 0; c < ncand; ++c) {
      int64_t id = cand[i * ncand + c];
      if (id < 0) continue;
      const float* bp = base + id * d;
      float dd = metric == METRIC_L2 ? l2_simd<64>(q + i * d, bp, d) : -ip_simd<64>(q + i * d, bp, d);
      top.push(dd, id);
    }
    int64_t cnt = top.finish();
    for (int64_t j = cnt; j < k; ++j) {
      dist[i * k + j] = 0.0f;
      labels[i * k + j] = -1;
    }
    if (metric != METRIC_L2)
      for (int64_t j = 0; j < cnt; ++j) dist[i * k + j] = -dist[i * k + j];
  });
}

// api/collection_vector_query.mojo:24-46. Returns 0, or -1 on a non-finite
// component, -2 on a zero row.
int orc_normalize(const float* x, int64_t n, int d, float* out) {
  for (int64_t i = 0; i < n; ++i) {
    double sq = 0.0;
    for (int c = 0; c < d; ++c) {
      float v = x[i * d + c];
      if (!std::isfinite(v)) return -1;
      double w = (double)v;
      sq = sq + w * w;
    }
    if (!(sq > 0.0)) return -2;
    double inv = 1.0 / std::sqrt(sq);
    for (int c = 0; c < d; ++c) out[i * d + c] = (float)((double)x[i * d + c] * inv);
  }
  return 0;
}

// FP64 brute-force ground truth, canonical (dist, id) order. metric 0 = L2
// distance, 1 = inner product (similarity, returned as -ip so smaller is
// better).
void orc_ground_truth(const float* base, int64_t nb, int d, int metric, const float* q,
                      int64_t nq, int64_t k, double* dist, int64_t* labels, int nthreads) {
  parallel_for(nq, nthreads, [&](int64_t i) {
    std::vector<std::pair<double, int64_t>> heap;
    heap.reserve(k + 1);
    auto cmp = [](const std::pair<double, int64_t>& a, const std::pair<double, int64_t>& b) {
      return a.first < b.first || (a.first == b.first && a.second < b.second);
    };
    const float* qp = q + i * d;
    for (int64_t j = 0; j < nb; ++j) {
      const float* bp = base + j * d;
      double acc = 0.0;
      if (metric == METRIC_L2) {
        for (int c = 0; c < d; ++c) {
          double df = (double)qp[c] - (double)bp[c];
          acc += df * df;
        }
      } else {
        for (int c = 0; c < d; ++c) acc += (double)qp[c] * (double)bp[c];
        acc = -acc;
      }
      std::pair<double, int64_t> e{acc, j};
      if ((int64_t)heap.size() < k) {
        heap.push_back(e);
        std::push_heap(heap.begin(), heap.end(), cmp);
      } else if (cmp(e, heap.front())) {
        std::pop_heap(heap.begin(), heap.end(), cmp);
        heap.back() = e;
        std::push_heap(heap.begin(), heap.end(), cmp);
      }
    }
    std::sort(heap.begin(), heap.end(), cmp);
    for (int64_t j = 0; j < k; ++j) {
      if (j < (int64_t)heap.size()) {
        dist[i * k + j] = heap[j].first;
        labels[i * k + j] = heap[j].second;
      } else {
        dist[i * k + j] = 0.0;
        labels[i * k + j] = -1;
      }
    }
  });
}

}  // extern "C"
