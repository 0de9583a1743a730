// CollectionIVFPQ snapshots (api/collection_ivfpq.mojo:335-476) read into
// and written from GPU IVF-PQ indexes.
//
// Layout, all integers 64-bit little-endian, Bool one byte, strings a
// length then UTF-8 bytes (api/collection_codec.mojo:49-64):
//   collection header   magic 0x43495650, version 1, dimension, name,
//                       metric ("l2", "cosine", "ip"), user-id count, ids
//   IndexIVFPQ          (io/serialization.mojo:1024-1090) magic 0x4d4a4f50,
//                       d, nlist, M, nprobe, ntotal, is_trained, metric
//                       (0 L2, 1 IP), then
//     IndexFlat         (:229-262) magic 0x4d4a4f46, d, ntotal, capacity,
//                       metric, capacity * d FP32 rows (the centroids)
//     inverted lists    (:903-944) magic 0x4d4a4f4c, nlist, code_size, per
//                       list size, capacity, size ids, size * code_size codes
//     ProductQuantizer  (:946-972) magic 0x4d4a4f51, d, M, ksub, is_trained,
//                       M * ksub * dsub FP32
//   checksum trailer    (io/snapshot_file.mojo:19-108) magic
//                       0x4D4F4A4F534E4150 and a rolling checksum of the
//                       payload in 8 MiB chunks
// The reader applies the reference's validation; a loaded index has no FP32
// rows (snapshots do not carry them).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "mv_internal.h"

namespace {

constexpr int64_t COLL_MAGIC = 0x43495650, COLL_VERSION = 1;
constexpr int64_t MAGIC_FLAT = 0x4d4a4f46, MAGIC_IVF_PQ = 0x4d4a4f50;
constexpr int64_t MAGIC_INVLISTS = 0x4d4a4f4c, MAGIC_PQ = 0x4d4a4f51;
constexpr uint64_t CK_MAGIC = 0x4D4F4A4F534E4150ull, CK_SEED = 0xD6E8FEB86659FD93ull;
constexpr size_t CK_CHUNK = 8u << 20;

inline uint64_t rotl(uint64_t v, int a) { return (v << a) | (v >> (64 - a)); }

// One chunk of the snapshot checksum (io/snapshot_file.mojo:25-49).
uint64_t ck_update(uint64_t cs, const uint8_t* p, size_t n) {
  uint64_t r = cs;
  const size_t words = n / 8;
  for (size_t i = 0; i < words; ++i) {
    uint64_t w;
    std::memcpy(&w, p + 8 * i, 8);
    r ^= w;
    r = rotl(r, 27) ^ rotl(w, 17);
    r ^= r >> 23;
  }
  uint64_t tail = 0;
  for (size_t i = words * 8; i < n; ++i) tail |= (uint64_t)p[i] << ((i - words * 8) * 8);
  r ^= tail;
  r ^= (uint64_t)n << 32;
  return rotl(r, 11);
}

uint64_t ck_payload(const uint8_t* p, size_t n) {
  uint64_t cs = CK_SEED;
  for (size_t off = 0; off < n; off += CK_CHUNK) cs = ck_update(cs, p + off, std::min(CK_CHUNK, n - off));
  return cs;
}

struct Reader {
  const std::vector<uint8_t>& b;
  size_t pos = 0, end;
  Reader(const std::vector<uint8_t>& buf, size_t e) : b(buf), end(e) {}
  void need(size_t n) {
    MV_REQUIRE(n <= end - pos, MV_ERR_ARG, "unexpected end of snapshot data");
  }
  int64_t i64() {
    need(8);
    int64_t v;
    std::memcpy(&v, b.data() + pos, 8);
    pos += 8;
    return v;
  }
  bool boolean() {
    need(1);
    const uint8_t v = b[pos++];
    MV_REQUIRE(v <= 1, MV_ERR_ARG, "invalid serialized Bool value");
    return v == 1;
  }
  std::string str() {
    const int64_t n = i64();
    MV_REQUIRE(n >= 0 && n <= 1048576, MV_ERR_ARG, "snapshot string size out of range");
    need((size_t)n);
    std::string s(reinterpret_cast<const char*>(b.data() + pos), (size_t)n);
    pos += (size_t)n;
    return s;
  }
  template <typename T>
  void arr(T* out, int64_t count) {
    MV_REQUIRE(count >= 0 && (uint64_t)count <= (end - pos) / sizeof(T), MV_ERR_ARG,
               "unexpected end of snapshot data");
    if (count) std::memcpy(out, b.data() + pos, sizeof(T) * (size_t)count);
    pos += sizeof(T) * (size_t)count;
  }
};

void check_size(int64_t v, int64_t max) {
  MV_REQUIRE(v >= 0 && v <= max, MV_ERR_ARG,
             "Security Error: Deserialized size is out of valid range or exceeds safety limits");
}

struct Writer {
  std::vector<uint8_t> b;
  void i64(int64_t v) {
    const size_t o = b.size();
    b.resize(o + 8);
    std::memcpy(b.data() + o, &v, 8);
  }
  void boolean(bool v) { b.push_back(v ? 1 : 0); }
  void str(const std::string& s) {
    i64((int64_t)s.size());
    b.insert(b.end(), s.begin(), s.end());
  }
  template <typename T>
  void arr(const T* p, int64_t count) {
    const size_t o = b.size();
    b.resize(o + sizeof(T) * (size_t)count);
    if (count) std::memcpy(b.data() + o, p, sizeof(T) * (size_t)count);
  }
};

int32_t fail(int32_t code, const std::string& msg) {
  mv::set_last_error(msg);
  return code;
}

}  // namespace

extern "C" {

uint64_t mv_snapshot_checksum(const void* payload, size_t bytes) {
  return ck_payload(static_cast<const uint8_t*>(payload), bytes);
}

int32_t mv_ivfpq_load_snapshot(mv_ctx* ctx, const char* path, mv_ivfpq** out) {
  if (!ctx || !path || !out) return MV_ERR_ARG;
  *out = nullptr;
  mv_ivfpq* ix = nullptr;
  try {
    std::unique_ptr<FILE, int (*)(FILE*)> f(std::fopen(path, "rb"), std::fclose);
    MV_REQUIRE(f != nullptr, MV_ERR_ARG, std::string("cannot open snapshot ") + path);
    std::fseek(f.get(), 0, SEEK_END);
    const long total = std::ftell(f.get());
    std::fseek(f.get(), 0, SEEK_SET);
    MV_REQUIRE(total >= 16, MV_ERR_ARG, "IVF-PQ snapshot checksum trailer is missing.");
    std::vector<uint8_t> buf((size_t)total);
    MV_REQUIRE(std::fread(buf.data(), 1, buf.size(), f.get()) == buf.size(), MV_ERR_ARG,
               "cannot read snapshot");
    const size_t payload = buf.size() - 16;
    uint64_t magic, expected;
    std::memcpy(&magic, buf.data() + payload, 8);
    std::memcpy(&expected, buf.data() + payload + 8, 8);
    MV_REQUIRE(magic == CK_MAGIC, MV_ERR_ARG, "Invalid snapshot checksum trailer.");
    MV_REQUIRE(ck_payload(buf.data(), payload) == expected, MV_ERR_ARG, "Snapshot checksum mismatch.");
    Reader r(buf, payload);
    MV_REQUIRE(r.i64() == COLL_MAGIC, MV_ERR_ARG, "Invalid CollectionIVFPQ snapshot magic.");
    MV_REQUIRE(r.i64() == COLL_VERSION, MV_ERR_ARG, "Unsupported CollectionIVFPQ snapshot version.");
    const int64_t dim = r.i64();
    MV_REQUIRE(dim > 0 && dim <= 65536, MV_ERR_ARG, "dimension must be between 1 and 65536.");
    const std::string name = r.str();
    const std::string metric = r.str();
    MV_REQUIRE(metric == "l2" || metric == "cosine" || metric == "ip", MV_ERR_ARG,
               "metric must be \"l2\", \"cosine\", or \"ip\".");
    const int index_metric = metric == "l2" ? MV_METRIC_L2 : MV_METRIC_IP;
    const int64_t nids = r.i64();
    check_size(nids, 1000000000);
    std::vector<int64_t> user_ids((size_t)nids);
    r.arr(user_ids.data(), nids);
    // IndexIVFPQ (serialization.mojo:1041-1090)
    MV_REQUIRE(r.i64() == MAGIC_IVF_PQ, MV_ERR_ARG, "Invalid magic for IndexIVFPQ");
    const int64_t d = r.i64();
    MV_REQUIRE(d > 0 && d <= 65536, MV_ERR_ARG, "dimension must be between 1 and 65536.");
    const int64_t nlist = r.i64();
    check_size(nlist, 1000000);
    const int64_t M = r.i64();
    check_size(M, d);
    MV_REQUIRE(M > 0 && d % M == 0, MV_ERR_ARG, "Invalid IndexIVFPQ subvector count.");
    const int64_t nprobe = r.i64();
    check_size(nprobe, nlist);
    MV_REQUIRE(nprobe > 0, MV_ERR_ARG, "Invalid IndexIVFPQ nprobe.");
    const int64_t ntotal = r.i64();
    check_size(ntotal, 1000000000);
    const bool trained = r.boolean();
    const int64_t mi = r.i64();
    MV_REQUIRE(mi == 0 || mi == 1, MV_ERR_ARG, "Invalid IndexIVFPQ metric.");
    // quantizer IndexFlat (:240-262)
    MV_REQUIRE(r.i64() == MAGIC_FLAT, MV_ERR_ARG, "Invalid magic for IndexFlat");
    const int64_t qd = r.i64();
    const int64_t qn = r.i64();
    check_size(qn, 1000000000);
    const int64_t qcap = r.i64();
    check_size(qcap, 1000000000);
    MV_REQUIRE(qd > 0 && qd <= 65536, MV_ERR_ARG, "dimension must be between 1 and 65536.");
    const int64_t qm = r.i64() == 1 ? 1 : 0;  // any other value reads as L2 (:255-256)
    MV_REQUIRE(qd == d && ((trained && qn == nlist) || (!trained && qn == 0)) && qm == mi &&
                   qn <= qcap,
               MV_ERR_ARG, "IndexIVFPQ coarse quantizer header mismatch.");
    MV_REQUIRE((uint64_t)qcap <= (r.end - r.pos) / ((size_t)d * 4), MV_ERR_ARG,
               "unexpected end of snapshot data");
    std::vector<float> qrows((size_t)qcap * d);
    r.arr(qrows.data(), qcap * d);
    // inverted lists (:916-944)
    MV_REQUIRE(r.i64() == MAGIC_INVLISTS, MV_ERR_ARG, "Invalid magic for ArrayInvertedLists");
    const int64_t ln = r.i64();
    check_size(ln, 1000000);
    const int64_t code_size = r.i64();
    check_size(code_size, 65536);
    MV_REQUIRE(ln == nlist && code_size == M, MV_ERR_ARG,
               "Inverted-list shape does not match its index header.");
    std::vector<int64_t> off((size_t)nlist + 1, 0), ids;
    std::vector<uint8_t> codes;
    for (int64_t l = 0; l < nlist; ++l) {
      const int64_t size = r.i64();
      const int64_t cap = r.i64();
      check_size(cap, 1000000000);
      check_size(size, cap);
      const size_t o = ids.size();
      MV_REQUIRE((uint64_t)size <= (r.end - r.pos) / 8, MV_ERR_ARG, "unexpected end of snapshot data");
      ids.resize(o + (size_t)size);
      r.arr(ids.data() + o, size);
      MV_REQUIRE((uint64_t)size <= (r.end - r.pos) / (size_t)M, MV_ERR_ARG,
                 "unexpected end of snapshot data");
      codes.resize((o + (size_t)size) * (size_t)M);
      r.arr(codes.data() + o * (size_t)M, size * M);
      off[(size_t)l + 1] = off[(size_t)l] + size;
    }
    // ProductQuantizer (:954-972)
    MV_REQUIRE(r.i64() == MAGIC_PQ, MV_ERR_ARG, "Invalid magic for ProductQuantizer");
    const int64_t pd = r.i64(), pM = r.i64(), ksub = r.i64();
    MV_REQUIRE(pd == d && pM == M && ksub == 256, MV_ERR_ARG,
               "ProductQuantizer shape does not match its index header.");
    const bool pq_trained = r.boolean();
    std::vector<float> pq((size_t)256 * d);
    r.arr(pq.data(), 256 * d);
    MV_REQUIRE(pq_trained == trained, MV_ERR_ARG, "IndexIVFPQ training state mismatch.");
    MV_REQUIRE(r.pos == payload, MV_ERR_ARG, "IVF-PQ snapshot contains unexpected payload data.");
    // collection checks (api/collection_ivfpq.mojo:420-470)
    // (the index header's checks above already bound both; these restate the
    // collection's own range checks with its messages)
    MV_REQUIRE(nlist > 0 && nlist <= 1000000, MV_ERR_ARG, "nlist must be between 1 and 1000000.");
    MV_REQUIRE(nprobe > 0 && nprobe <= nlist && nprobe <= 65536, MV_ERR_ARG,
               "nprobe must be between 1 and nlist.");
    MV_REQUIRE(d == dim && ntotal == nids, MV_ERR_ARG,
               "IVF-PQ snapshot dimensions or record count mismatch.");
    MV_REQUIRE(mi == (index_metric == MV_METRIC_IP ? 1 : 0), MV_ERR_ARG, "IVF-PQ snapshot metric mismatch.");
    std::vector<uint8_t> seen((size_t)nids, 0);
    for (int64_t id : ids) {
      MV_REQUIRE(id >= 0 && id < nids, MV_ERR_ARG, "IVF-PQ snapshot contains an invalid internal ID.");
      MV_REQUIRE(!seen[(size_t)id], MV_ERR_ARG, "IVF-PQ snapshot contains a duplicate internal ID.");
      seen[(size_t)id] = 1;
    }
    MV_REQUIRE((int64_t)ids.size() == nids, MV_ERR_ARG,
               "IVF-PQ inverted-list count does not match its IDs.");
    {
      std::vector<int64_t> sorted_ids(user_ids);
      std::sort(sorted_ids.begin(), sorted_ids.end());
      MV_REQUIRE(std::adjacent_find(sorted_ids.begin(), sorted_ids.end()) == sorted_ids.end(),
                 MV_ERR_ARG, "IVF-PQ snapshot contains duplicate IDs.");
    }
    // the GPU index
    int32_t st = mv_ivfpq_create(ctx, (int32_t)d, (int32_t)nlist, (int32_t)M, index_metric, &ix);
    if (st != MV_OK) return st;
    if (trained) {
      if ((st = mv_ivfpq_set_codebooks(ix, qrows.data(), pq.data())) != MV_OK) throw mv::Error(st, "set_codebooks");
    }
    if ((st = mv_ivfpq_set_lists(ix, off.data(), ids.data(), codes.data())) != MV_OK)
      throw mv::Error(st, "set_lists");
    if ((st = mv_ivfpq_set_nprobe(ix, (int32_t)nprobe)) != MV_OK) throw mv::Error(st, "set_nprobe");
    ix->user_ids = std::move(user_ids);
    ix->coll_name = name;
    ix->coll_metric = metric;
    *out = ix;
    return MV_OK;
  } catch (const mv::Error& e) {
    if (ix) mv_ivfpq_destroy(ix);
    return fail(e.code, e.what());
  } catch (const std::bad_alloc&) {
    if (ix) mv_ivfpq_destroy(ix);
    return fail(MV_ERR_OOM, "host allocation failed");
  } catch (const std::exception& e) {
    if (ix) mv_ivfpq_destroy(ix);
    return fail(MV_ERR_INTERNAL, e.what());
  }
}

int32_t mv_ivfpq_snapshot_info(mv_ivfpq* ix, char* name, size_t name_len, char* metric,
                               size_t metric_len, int64_t* user_ids, int64_t* num_ids) {
  if (!ix) return MV_ERR_ARG;
  if (num_ids) *num_ids = (int64_t)ix->user_ids.size();
  if (user_ids && !ix->user_ids.empty())
    std::memcpy(user_ids, ix->user_ids.data(), sizeof(int64_t) * ix->user_ids.size());
  auto put = [](char* dst, size_t len, const std::string& s) {
    if (!dst || len == 0) return;
    const size_t n = std::min(len - 1, s.size());
    std::memcpy(dst, s.data(), n);
    dst[n] = 0;
  };
  put(name, name_len, ix->coll_name);
  put(metric, metric_len, ix->coll_metric);
  return MV_OK;
}

int32_t mv_ivfpq_save_snapshot(mv_ivfpq* ix, const char* path, const char* name,
                               const char* metric, const int64_t* user_ids, int64_t num_ids) {
  if (!ix || !path || !name || !metric || num_ids < 0 || (num_ids > 0 && !user_ids))
    return MV_ERR_ARG;
  try {
    const std::string m = metric;
    MV_REQUIRE(m == "l2" || m == "cosine" || m == "ip", MV_ERR_ARG,
               "metric must be \"l2\", \"cosine\", or \"ip\".");
    MV_REQUIRE((m == "l2") == (ix->metric == MV_METRIC_L2), MV_ERR_ARG,
               "the collection metric does not match the index metric");
    MV_REQUIRE(num_ids == ix->ntotal, MV_ERR_ARG, "one user id per indexed row is needed");
    std::lock_guard<std::mutex> lk(ix->mu);
    ix->ctx->set_device();
    MV_CHECK_CUDA(cudaDeviceSynchronize());
    const int64_t d = ix->d, nlist = ix->nlist, M = ix->M, total = ix->h_off[(size_t)nlist];
    MV_REQUIRE(total == ix->ntotal, MV_ERR_STATE, "rows outside the lists cannot be saved");
    std::vector<float> cent((size_t)nlist * d), pq((size_t)256 * d);
    std::vector<uint32_t> ids32((size_t)total);
    std::vector<uint8_t> codes((size_t)total * M);
    MV_CHECK_CUDA(cudaMemcpy(cent.data(), ix->centroids.p, cent.size() * 4, cudaMemcpyDeviceToHost));
    MV_CHECK_CUDA(cudaMemcpy(pq.data(), ix->pq.p, pq.size() * 4, cudaMemcpyDeviceToHost));
    if (total) {
      MV_CHECK_CUDA(cudaMemcpy(ids32.data(), ix->d_ids.p, ids32.size() * 4, cudaMemcpyDeviceToHost));
      MV_CHECK_CUDA(cudaMemcpy(codes.data(), ix->d_codes.p, codes.size(), cudaMemcpyDeviceToHost));
    }
    Writer w;
    w.i64(COLL_MAGIC);
    w.i64(COLL_VERSION);
    w.i64(d);
    w.str(name);
    w.str(m);
    w.i64(num_ids);
    w.arr(user_ids, num_ids);
    w.i64(MAGIC_IVF_PQ);
    w.i64(d);
    w.i64(nlist);
    w.i64(M);
    w.i64(std::min<int64_t>(std::max(ix->nprobe, 1), nlist));
    w.i64(ix->ntotal);
    w.boolean(ix->trained);
    const int64_t mi = ix->metric == MV_METRIC_IP ? 1 : 0;
    w.i64(mi);
    w.i64(MAGIC_FLAT);  // the quantizer: nlist rows when trained, none before
    w.i64(d);
    const int64_t qn = ix->trained ? nlist : 0;
    w.i64(qn);
    w.i64(qn);
    w.i64(mi);
    w.arr(cent.data(), qn * d);
    w.i64(MAGIC_INVLISTS);
    w.i64(nlist);
    w.i64(M);
    for (int64_t l = 0; l < nlist; ++l) {
      const int64_t o = ix->h_off[(size_t)l], size = ix->h_off[(size_t)l + 1] - o;
      w.i64(size);
      w.i64(size);  // capacity
      for (int64_t j = 0; j < size; ++j) w.i64((int64_t)ids32[(size_t)(o + j)]);
      w.arr(codes.data() + (size_t)o * M, size * M);
    }
    w.i64(MAGIC_PQ);
    w.i64(d);
    w.i64(M);
    w.i64(256);
    w.boolean(ix->trained);
    w.arr(pq.data(), 256 * d);
    const uint64_t cs = ck_payload(w.b.data(), w.b.size());
    w.arr(&CK_MAGIC, 1);
    w.arr(&cs, 1);
    const std::string tmp = std::string(path) + ".tmp";
    {
      std::unique_ptr<FILE, int (*)(FILE*)> f(std::fopen(tmp.c_str(), "wb"), std::fclose);
      MV_REQUIRE(f != nullptr, MV_ERR_ARG, "cannot create " + tmp);
      MV_REQUIRE(std::fwrite(w.b.data(), 1, w.b.size(), f.get()) == w.b.size(), MV_ERR_INTERNAL,
                 "short write");
      MV_REQUIRE(std::fflush(f.get()) == 0, MV_ERR_INTERNAL, "flush failed");
    }
    MV_REQUIRE(std::rename(tmp.c_str(), path) == 0, MV_ERR_INTERNAL, "cannot replace " + std::string(path));
    return MV_OK;
  } catch (const mv::Error& e) {
    return fail(e.code, e.what());
  } catch (const std::exception& e) {
    return fail(MV_ERR_INTERNAL, e.what());
  }
}

}  // extern "C"
