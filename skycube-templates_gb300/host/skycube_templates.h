// skycube_templates.h -- the suite's templated algorithm interface on top of
// the GB300 engine's C ABI (include/skycube_gb300.h).
//
// A program written against the suite's MDMC<D> / SDSC<D> class templates
// (src/mdmc/MDMC.h:21-213, src/sdsc/SDSC.h:15-81) and their result layouts
// (lattice_node, src/utilities/lattice_utilities.h:21-31; HashCube,
// src/skycube/Hashcube.h:36-178) compiles against this header instead and
// runs the skycube on one GB300 through libskycube_gb300.so:
//
//   Config cfg; cfg.devices = {0}; cfg.max_d = d; ...
//   MDMC<D>* cube = new MDMC<D>(&cfg, n);   // or SDSC<D>
//   cube->Init(data);                       // float** rows, as in the suite
//   cube->Execute();
//   getsubspace(c, cube->getHashCubeStructure());   // MDMC
//   cube->getLattice()[c].skyline;                  // SDSC
//
// Differences from the suite, all deliberate: errors raise skc::Error (the
// suite never checks CUDA status); there is no CPU worker (-p is the only
// mode, devices[0] is the GPU, device 0 when the list is empty); Config has
// one extra field, `mode` ("batched" or "plain"), selecting the execution
// form. Results are identical to the suite's STSC ground truth, ties
// included.
#pragma once

#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "skycube_gb300.h"

// --------------------------------------------------------------------------
// Config (src/utilities/config.h:13-27), plus the execution form.
typedef struct Config {
  bool verbose = false;
  bool check = false;
  bool cpu = false;
  bool cross_distribution = false;
  std::string input_fname;
  uint32_t alpha_size = 1024;
  uint32_t pq_size = 128;
  uint32_t partitioning_depth = 0;  // grid depth 1..7 (0 = engine default)
  std::string algo;
  uint32_t threads = 8;
  int max_d = -1;
  std::vector<int> devices;
  std::string papi;
  std::string mode = "batched";  // "batched" or "plain"
} Config;

namespace skc {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int code) {
  if (code != SKC_OK) throw Error(code, skc_last_error());
}

// One engine context per device, created on first use, kept for the
// process lifetime (the suite initialises each device once per run).
inline skc_context* context_for(int device) {
  static std::mutex mu;
  static std::map<int, skc_context*> ctx;
  std::lock_guard<std::mutex> lock(mu);
  auto it = ctx.find(device);
  if (it != ctx.end()) return it->second;
  skc_context* c = nullptr;
  check(skc_context_create(device, &c));
  ctx[device] = c;
  return c;
}

inline int device_of(const Config* cfg) {
  return (cfg && !cfg->devices.empty()) ? cfg->devices.front() : 0;
}

inline int mode_of(const Config* cfg) {
  if (!cfg || cfg->mode.empty() || cfg->mode == "batched") return SKC_MODE_BATCHED;
  if (cfg->mode == "plain") return SKC_MODE_PLAIN;
  throw Error(SKC_ERR_INVALID, "unknown execution form '" + cfg->mode + "' (batched|plain)");
}

// Copies the caller's rows and uploads them (the suite's Init + initializeGpu).
template <int DIMS>
inline skc_dataset* upload_rows(skc_context* ctx, float** data, uint32_t n) {
  std::vector<float> flat((size_t)n * DIMS);
  for (uint32_t i = 0; i < n; ++i) std::memcpy(&flat[(size_t)i * DIMS], data[i], sizeof(float) * DIMS);
  skc_dataset* ds = nullptr;
  check(skc_dataset_upload(ctx, flat.data(), n, DIMS, &ds));
  return ds;
}

}  // namespace skc

// --------------------------------------------------------------------------
// Lattice (src/utilities/lattice_utilities.{h,cpp}).
typedef struct lattice_node_struct {
  unsigned int index = 0;
  std::vector<int> dimensions;
  std::vector<unsigned int> parents;
  std::vector<unsigned int> children;
  std::vector<unsigned int> skyline;
  std::vector<unsigned int> extended_sky;
  std::map<int, std::vector<int> > prune_set;
} lattice_node;

// Attribute indices of a cuboid mask, ascending.
inline std::vector<int> getDimensions(unsigned int bitvector) {
  std::vector<int> res;
  for (int k = 0; bitvector; ++k, bitvector >>= 1)
    if (bitvector & 1u) res.push_back(k);
  return res;
}

// Cuboids 1 .. m-1 ordered by descending number of attributes (top-down).
inline std::vector<unsigned int> get_tds_list(int m) {
  std::vector<unsigned int> res;
  for (int i = 1; i < m; ++i) res.push_back((unsigned)i);
  std::stable_sort(res.begin(), res.end(), [](unsigned a, unsigned b) {
    return __builtin_popcount(a) > __builtin_popcount(b);
  });
  return res;
}

// m = 2^d nodes; the parents of a cuboid are the cuboids with one attribute
// more, listed by descending mask, its children those with one attribute
// less.
inline lattice_node* generate_lattice(int m) {
  lattice_node* lat = new lattice_node[m];
  for (int i = m - 1; i > 0; --i) {
    lat[i].index = (unsigned)i;
    lat[i].dimensions = getDimensions((unsigned)i);
    for (int k = 0; (1 << k) <= i; ++k) {
      if (!(i & (1 << k))) continue;
      const unsigned child = (unsigned)i ^ (1u << k);
      if (child) {
        lat[i].children.push_back(child);
        lat[child].parents.push_back((unsigned)i);
      }
    }
  }
  return lat;
}

// --------------------------------------------------------------------------
// HashCube (src/skycube/Hashcube.h:36-178): word j of every point's
// dominated-subspace bitmap keys map j; a point is listed under its word
// unless the word is all ones (dominated in all 32 of those cuboids).
template <int DIMS>
class HashCube {
 public:
  static const uint32_t bitvector_word_size_ = 32;
  static const uint32_t bitvector_num_words_ = ((1u << DIMS) / 32) + 1;

  std::map<uint32_t, std::vector<int> >* getMaps() { return maps_; }
  const std::map<uint32_t, std::vector<int> >* getMaps() const { return maps_; }

  void clear() {
    for (auto& mp : maps_) mp.clear();
  }

  // Adds n points: point pids[i]'s bitmap is bits[i*words .. (i+1)*words).
  void populateFromBitmaps(const uint32_t* bits, const uint32_t* pids, uint64_t n,
                           uint32_t words) {
    for (uint64_t i = 0; i < n; ++i)
      for (uint32_t j = 0; j < bitvector_num_words_; ++j) {
        const uint32_t v = j < words ? bits[i * words + j] : 0u;
        if (__builtin_popcount(v) != (int)bitvector_word_size_) maps_[j][v].push_back((int)pids[i]);
      }
  }

  // Skyline of one cuboid (the suite's getsubspace).
  std::vector<int> getSubspace(unsigned int subspace) const {
    std::vector<int> ret;
    const auto& mp = maps_[subspace / 32];
    const uint32_t bit = 1u << (subspace % 32);
    for (const auto& kv : mp)
      if (!(kv.first & bit)) ret.insert(ret.end(), kv.second.begin(), kv.second.end());
    return ret;
  }

  bool operator==(const HashCube<DIMS>& other) const {
    for (uint32_t j = 0; j < bitvector_num_words_; ++j) {
      if (maps_[j].size() != other.maps_[j].size()) return false;
      for (const auto& kv : maps_[j]) {
        auto it = other.maps_[j].find(kv.first);
        if (it == other.maps_[j].end()) return false;
        std::vector<int> a = kv.second, b = it->second;
        std::sort(a.begin(), a.end());
        std::sort(b.begin(), b.end());
        if (a != b) return false;
      }
    }
    return true;
  }

 private:
  std::map<uint32_t, std::vector<int> > maps_[bitvector_num_words_];
};

// Skyline of cuboid `subspace` from a HashCube's maps
// (src/utilities/utilities.h:253-267).
inline std::vector<int> getsubspace(unsigned int subspace,
                                    std::map<unsigned int, std::vector<int> >* hashcube) {
  std::vector<int> ret;
  const unsigned int index = subspace / 32;
  const unsigned int mask = 1u << (subspace % 32);
  for (auto it = hashcube[index].begin(); it != hashcube[index].end(); ++it)
    if (!(it->first & mask)) ret.insert(ret.end(), it->second.begin(), it->second.end());
  return ret;
}

// --------------------------------------------------------------------------
// MDMC (src/mdmc/MDMC.h:21-213): per-point dominated-subspace bitmaps of the
// extended skyline, collected into a HashCube.
template <int DIMS>
class MDMC {
 public:
  MDMC(Config* cfg, int n) : cfg_(cfg), n_((uint32_t)n) {}
  ~MDMC() {
    if (res_) skc_result_free(res_);
    if (ds_) skc_dataset_free(ds_);
  }
  MDMC(const MDMC&) = delete;
  MDMC& operator=(const MDMC&) = delete;

  void Init(float** data) {
    ctx_ = skc::context_for(skc::device_of(cfg_));
    if (ds_) skc_dataset_free(ds_);
    ds_ = skc::upload_rows<DIMS>(ctx_, data, n_);
  }

  void Execute() {
    if (!ds_) throw skc::Error(SKC_ERR_INVALID, "MDMC::Execute before Init");
    skc_options o;
    skc_options_init(&o);
    o.algo = SKC_ALGO_MDMC;
    o.mode = skc::mode_of(cfg_);
    o.max_d = cfg_ ? cfg_->max_d : 0;
    o.depth = cfg_ ? (int)cfg_->partitioning_depth : 0;
    // The suite's MDMC prefilters with pq_size pruners (src/mdmc/MDMC.cu:251).
    o.pq_size = cfg_ ? (int)std::min<uint32_t>(cfg_->pq_size, 1024) : 0;
    o.want_bitmaps = 1;
    if (res_) skc_result_free(res_);
    res_ = nullptr;
    skc::check(skc_skycube(ctx_, ds_, &o, &res_));
    const uint32_t *bits = nullptr, *pids = nullptr;
    uint64_t np = 0;
    uint32_t words = 0;
    skc::check(skc_result_bitmaps(res_, &bits, &pids, &np, &words));
    hashcube_.clear();
    hashcube_.populateFromBitmaps(bits, pids, np, words);
  }

  std::map<unsigned int, std::vector<int> >* getHashCubeStructure() { return hashcube_.getMaps(); }
  const HashCube<DIMS>& getHashCube() { return hashcube_; }

  // Not in the suite: one cuboid's skyline straight from the engine's
  // per-cuboid lists (ascending ids).
  std::vector<unsigned int> getSkyline(unsigned int cuboid) {
    const uint32_t* ids = nullptr;
    uint64_t cnt = 0;
    skc::check(skc_result_cuboid(res_, cuboid, &ids, &cnt));
    return std::vector<unsigned int>(ids, ids + cnt);
  }
  skc_result* result() { return res_; }

 private:
  Config* cfg_;
  uint32_t n_;
  skc_context* ctx_ = nullptr;
  skc_dataset* ds_ = nullptr;
  skc_result* res_ = nullptr;
  HashCube<DIMS> hashcube_;
};

// --------------------------------------------------------------------------
// SDSC (src/sdsc/SDSC.h:15-81): per-cuboid skyline and extended skyline in a
// lattice of 2^D nodes.
template <int DIMS>
class SDSC {
 public:
  SDSC(Config* cfg, int n) : cfg_(cfg), n_((uint32_t)n) {}
  virtual ~SDSC() {
    delete[] lattice_;
    if (res_) skc_result_free(res_);
    if (ds_) skc_dataset_free(ds_);
  }
  SDSC(const SDSC&) = delete;
  SDSC& operator=(const SDSC&) = delete;

  void Init(float** data) {
    ctx_ = skc::context_for(skc::device_of(cfg_));
    if (ds_) skc_dataset_free(ds_);
    ds_ = skc::upload_rows<DIMS>(ctx_, data, n_);
    delete[] lattice_;
    lattice_ = generate_lattice(1 << DIMS);
  }

  void Execute() {
    if (!ds_) throw skc::Error(SKC_ERR_INVALID, "SDSC::Execute before Init");
    skc_options o;
    skc_options_init(&o);
    o.algo = SKC_ALGO_SDSC;
    o.mode = skc::mode_of(cfg_);
    o.max_d = cfg_ ? cfg_->max_d : 0;
    o.depth = cfg_ ? (int)cfg_->partitioning_depth : 0;
    o.want_extended = 1;
    if (res_) skc_result_free(res_);
    res_ = nullptr;
    skc::check(skc_skycube(ctx_, ds_, &o, &res_));
    skc::check(skc_result_download(res_));
    const int max_d = (o.max_d <= 0 || o.max_d > DIMS) ? DIMS : o.max_d;
    const unsigned full = (1u << DIMS) - 1;
    for (unsigned c = 1; c <= full; ++c) {
      lattice_[c].skyline.clear();
      lattice_[c].extended_sky.clear();
      if (__builtin_popcount(c) > max_d && c != full) continue;
      const uint32_t* ids = nullptr;
      uint64_t cnt = 0;
      skc::check(skc_result_cuboid(res_, c, &ids, &cnt));
      lattice_[c].skyline.assign(ids, ids + cnt);
      skc::check(skc_result_extended(res_, c, &ids, &cnt));
      lattice_[c].extended_sky.assign(ids, ids + cnt);
    }
  }

  lattice_node* getLattice() { return lattice_; }
  // The suite's SDSC keeps an (unused) empty HashCube; so does this one.
  std::map<unsigned int, std::vector<int> >* getHashCubeStructure() { return hashcube_.getMaps(); }
  const HashCube<DIMS>& getHashCube() { return hashcube_; }
  skc_result* result() { return res_; }

 private:
  Config* cfg_;
  uint32_t n_;
  skc_context* ctx_ = nullptr;
  skc_dataset* ds_ = nullptr;
  skc_result* res_ = nullptr;
  lattice_node* lattice_ = nullptr;
  HashCube<DIMS> hashcube_;
};
