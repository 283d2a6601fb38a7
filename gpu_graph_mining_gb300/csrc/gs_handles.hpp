// Definitions behind the opaque handles of the C ABI (include/gspan_gb300.h)
// shared by the translation units that implement it.
#pragma once
#include <cstdint>
#include <vector>

#include "../../include/gspan_gb300.h"
#include "gs_engine.hpp"

struct gs_db {
  gsgb::Database d;
};

namespace gsgb {

// Host buffer behind gs_patterns: patterns appended in emission order.
struct PatternBuf {
  gs_patterns view;  // first member: gs_patterns_free casts back
  std::vector<int64_t> offset{ 0 };
  std::vector<int32_t> dfs;
  std::vector<int64_t> support;

  static void emit(const int32_t *d, int32_t n, int64_t sup, void *user)
  {
    PatternBuf *b = (PatternBuf *)user;
    b->dfs.insert(b->dfs.end(), d, d + 5 * n);
    b->offset.push_back(b->offset.back() + n);
    b->support.push_back(sup);
  }
  gs_patterns *publish()
  {
    view.count = (int64_t)support.size();
    view.n_tuples = offset.back();
    view.offset = offset.data();
    view.dfs = dfs.data();
    view.support = support.data();
    return &view;
  }
};

void capi_set_error(const char *msg);

}  // namespace gsgb
