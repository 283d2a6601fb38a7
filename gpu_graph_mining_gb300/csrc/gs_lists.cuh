// Lists strategy: which extension records go into the per-row lists of the
// frequent forward extensions (device code shared by the materialise pass,
// which counts the rows, and the list fill).
#pragma once
#include "gs_kernels.hpp"

namespace gsgb {

// the record's list row and its node's forward key, or false when the record
// does not go into a list (an unused slot, not a frequent forward key, or its
// node keeps no lists)
__device__ __forceinline__ bool list_entry(const int4 x, const ListBuild &lb, long long &row, int &lk,
                                           unsigned int *err)
{
  if(x.x < 0) return false;
  const int wkey = x.x & kRecKeyMask;
  const int n = __ldg(&lb.lnode[wkey]);
  if(n < 0) return false;
  const int rb = __ldg(&lb.rowbase[n]);
  if(rb < 0) return false;
  const NodeDesc &nd = lb.nodes[n];
  if((unsigned)x.z >= (unsigned)nd.nrows) {
    atomicOr(err, 2u);
    return false;
  }
  row = (long long)rb + x.z;
  lk = wkey - nd.key_base;
  return true;
}

}  // namespace gsgb
