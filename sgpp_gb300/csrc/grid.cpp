// Host-side sparse-grid construction for Linear (no-boundary) grids: the inputs of the
// multi-evaluation path. C ABI in include/sgmev.h (sggrid_*).
//
// Regular grids follow the storage order of HashGenerator::regular_iter
// (base/src/sgpp/base/grid/generation/hashmap/HashGenerator.hpp:282-347), so the grids built
// here are index-for-index identical to the reference's. Surplus refinement follows
// HashRefinement::free_refine (base/.../HashRefinement.cpp:124-147) with
// SurplusRefinementFunctor (base/.../SurplusRefinementFunctor.cpp:23-28).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/sgmev.h"

namespace sgmev {
extern thread_local std::string g_last_error;
}

namespace {

int grid_fail(int code, const char* msg) {
  sgmev::g_last_error = msg;
  return code;
}

// A grid point is a row of `dim` (level, index) pairs; rows live in two flat int32 arrays.
struct PointKey {
  std::vector<uint64_t> packed;  // (level << 32) | index per dimension
  bool operator==(const PointKey& o) const { return packed == o.packed; }
};

struct PointKeyHash {
  size_t operator()(const PointKey& k) const {
    uint64_t h = 0xcbf29ce484222325ULL;
    for (uint64_t v : k.packed) {
      h ^= v + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2);
    }
    return static_cast<size_t>(h);
  }
};

class Storage {
 public:
  Storage(int dim, int64_t cap, int32_t* lev, int32_t* idx)
      : dim_(dim), cap_(cap), lev_(lev), idx_(idx) {}

  int64_t size() const { return n_; }

  void adopt(int64_t n) {
    for (int64_t q = 0; q < n; ++q) map_.emplace(key(&lev_[q * dim_], &idx_[q * dim_]), q);
    n_ = n;
  }

  bool contains(const int32_t* l, const int32_t* i) const {
    return map_.find(key(l, i)) != map_.end();
  }

  bool insert(const int32_t* l, const int32_t* i) {
    if (n_ >= cap_) return false;
    std::memcpy(&lev_[n_ * dim_], l, sizeof(int32_t) * dim_);
    std::memcpy(&idx_[n_ * dim_], i, sizeof(int32_t) * dim_);
    map_.emplace(key(l, i), n_);
    ++n_;
    return true;
  }

  // AbstractRefinement::createGridpoint1D / createGridpointSubroutine
  // (base/.../AbstractRefinement.cpp:36-52, AbstractRefinement.hpp:229-244): before a point is
  // appended, its hierarchical parent in every dimension must exist (created recursively).
  bool create_with_ancestors(std::vector<int32_t>& l, std::vector<int32_t>& i) {
    for (int t = 0; t < dim_; ++t) {
      if (l[t] > 1) {
        const int32_t sl = l[t], si = i[t];
        l[t] = sl - 1;
        i[t] = (((si + 1) / 2) % 2 == 1) ? (si + 1) / 2 : (si - 1) / 2;
        if (!contains(l.data(), i.data())) {
          if (!create_with_ancestors(l, i)) return false;
        }
        l[t] = sl;
        i[t] = si;
      }
    }
    return insert(l.data(), i.data());
  }

  // a point is refinable if some child (l+1, 2i-1) / (l+1, 2i+1) is missing
  // (HashRefinement::collectRefinablePoints, :42-91)
  bool refinable(int64_t q) const {
    std::vector<int32_t> l(&lev_[q * dim_], &lev_[q * dim_] + dim_);
    std::vector<int32_t> i(&idx_[q * dim_], &idx_[q * dim_] + dim_);
    for (int t = 0; t < dim_; ++t) {
      const int32_t sl = l[t], si = i[t];
      l[t] = sl + 1;
      i[t] = 2 * si - 1;
      if (!contains(l.data(), i.data())) return true;
      i[t] = 2 * si + 1;
      if (!contains(l.data(), i.data())) return true;
      l[t] = sl;
      i[t] = si;
    }
    return false;
  }

  const int32_t* level_row(int64_t q) const { return &lev_[q * dim_]; }
  const int32_t* index_row(int64_t q) const { return &idx_[q * dim_]; }

 private:
  PointKey key(const int32_t* l, const int32_t* i) const {
    PointKey k;
    k.packed.resize(dim_);
    for (int t = 0; t < dim_; ++t)
      k.packed[t] = (static_cast<uint64_t>(static_cast<uint32_t>(l[t])) << 32) |
                    static_cast<uint32_t>(i[t]);
    return k;
  }

  int dim_;
  int64_t cap_;
  int32_t* lev_;
  int32_t* idx_;
  int64_t n_ = 0;
  std::unordered_map<PointKey, int64_t, PointKeyHash> map_;
};

// Size of the regular grid: level vectors with |l|_1 <= level + dim - 1 and every l_t <= level,
// each holding 2^{|l|_1 - dim} points.
int64_t regular_size(int dim, int level) {
  const int smax = level + dim - 1;
  std::vector<double> cnt(smax + 1, 0.0), nxt(smax + 1, 0.0);
  cnt[0] = 1.0;
  for (int t = 0; t < dim; ++t) {
    std::fill(nxt.begin(), nxt.end(), 0.0);
    for (int s = 0; s <= smax; ++s) {
      if (cnt[s] == 0.0) continue;
      for (int l = 1; l <= level && s + l <= smax; ++l) nxt[s + l] += cnt[s] * std::ldexp(1.0, l - 1);
    }
    cnt.swap(nxt);
  }
  double total = 0.0;
  for (double c : cnt) total += c;
  return static_cast<int64_t>(total);
}

}  // namespace

extern "C" {

SGMEV_API int sggrid_regular(int dim, int level, int64_t* n_grid, int32_t* level_out,
                             int32_t* index_out) {
  if (!n_grid) return grid_fail(SGMEV_ERR_INVALID, "n_grid is NULL");
  if (dim < 1 || level < 1 || level > 30) return grid_fail(SGMEV_ERR_INVALID, "need dim >= 1, 1 <= level <= 30");
  const int64_t n = regular_size(dim, level);
  if (!level_out || !index_out) {
    *n_grid = n;
    return SGMEV_OK;
  }
  if (*n_grid < n) return grid_fail(SGMEV_ERR_INVALID, "output arrays too small");
  // dimension 0: the 1-D grid, levels ascending, odd indices ascending; every other dimension
  // starts at (1, 1)
  int64_t count = 0;
  auto row_l = [&](int64_t q) { return level_out + q * dim; };
  auto row_i = [&](int64_t q) { return index_out + q * dim; };
  for (int l = 1; l <= level; ++l) {
    for (int32_t i = 1; i < (int32_t(1) << l); i += 2) {
      std::fill(row_l(count), row_l(count) + dim, 1);
      std::fill(row_i(count), row_i(count) + dim, 1);
      row_l(count)[0] = l;
      row_i(count)[0] = i;
      ++count;
    }
  }
  // dimension t: each existing point keeps (1,1) and gets copies with every admissible (l, i)
  // appended behind the current end
  for (int t = 1; t < dim; ++t) {
    const int64_t before = count;
    for (int64_t g = 0; g < before; ++g) {
      int level_sum = -1, level_max = 0;
      for (int s = 0; s < dim; ++s) {
        level_sum += row_l(g)[s];
        level_max = std::max(level_max, static_cast<int>(row_l(g)[s]));
      }
      for (int l = 1; l + level_sum <= level + dim - 1 && std::max(l, level_max) <= level; ++l) {
        for (int32_t i = 1; i < (int32_t(1) << l); i += 2) {
          if (l == 1) continue;  // (1,1) is g itself
          std::copy(row_l(g), row_l(g) + dim, row_l(count));
          std::copy(row_i(g), row_i(g) + dim, row_i(count));
          row_l(count)[t] = l;
          row_i(count)[t] = i;
          ++count;
        }
      }
    }
  }
  *n_grid = count;
  return count == n ? SGMEV_OK : grid_fail(SGMEV_ERR_INVALID, "internal size mismatch");
}

SGMEV_API int sggrid_refine_surplus(int dim, int64_t n_grid, int64_t cap, int32_t* level,
                                    int32_t* index, const double* alpha, int64_t n_points,
                                    double threshold, int64_t* n_out) {
  if (dim < 1 || n_grid < 1 || cap < n_grid || !level || !index || !alpha || !n_out || n_points < 0)
    return grid_fail(SGMEV_ERR_INVALID, "bad arguments to sggrid_refine_surplus");
  Storage st(dim, cap, level, index);
  st.adopt(n_grid);
  struct Cand {
    double value;
    int64_t seq;
  };
  std::vector<Cand> cands;
  cands.reserve(static_cast<size_t>(n_grid));
  for (int64_t q = 0; q < n_grid; ++q)
    if (st.refinable(q)) cands.push_back({std::fabs(alpha[q]), q});
  // keep the n_points largest indicator values (addElementToCollection, HashRefinement.cpp:19-38);
  // walk them largest first, ties by sequence number
  std::sort(cands.begin(), cands.end(), [](const Cand& a, const Cand& b) {
    return a.value != b.value ? a.value > b.value : a.seq < b.seq;
  });
  if (static_cast<int64_t>(cands.size()) > n_points) cands.resize(static_cast<size_t>(n_points));
  std::vector<int32_t> l(dim), i(dim);
  for (const Cand& c : cands) {
    if (!(c.value >= threshold)) continue;  // refineGridpointsCollection, :112-122
    // refineGridpoint (:214-223): every dimension, left child then right child
    for (int t = 0; t < dim; ++t) {
      for (int side = 0; side < 2; ++side) {
        std::copy(st.level_row(c.seq), st.level_row(c.seq) + dim, l.begin());
        std::copy(st.index_row(c.seq), st.index_row(c.seq) + dim, i.begin());
        const int32_t si = i[t];
        l[t] += 1;
        i[t] = side == 0 ? 2 * si - 1 : 2 * si + 1;
        if (!st.contains(l.data(), i.data())) {
          if (!st.create_with_ancestors(l, i))
            return grid_fail(SGMEV_ERR_INVALID, "refinement exceeds the output capacity");
        }
      }
    }
  }
  *n_out = st.size();
  return SGMEV_OK;
}

SGMEV_API int sggrid_level_index_for_eval(int dim, int64_t n_grid, const int32_t* level,
                                          const int32_t* index, double* level_pow2,
                                          double* index_out) {
  if (dim < 1 || n_grid < 0 || (n_grid > 0 && (!level || !index || !level_pow2 || !index_out)))
    return grid_fail(SGMEV_ERR_INVALID, "bad arguments to sggrid_level_index_for_eval");
  for (int64_t k = 0; k < n_grid * dim; ++k) {
    level_pow2[k] = std::ldexp(1.0, level[k]);
    index_out[k] = static_cast<double>(index[k]);
  }
  return SGMEV_OK;
}

}  // extern "C"
