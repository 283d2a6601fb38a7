// Mining kernels for one GB300 (sm_103a).
//
// The path is integer-only and memory-bound (no tensor-core work): each
// thread owns one embedding row, walks its back-links to recover the graph
// vertices of the pattern (one 8-byte load per column), then scans the
// adjacency of every right-most-path vertex (8-byte packed entries carrying
// neighbour, edge label and neighbour label, so no label gathers) and applies
// gSpan's extension rules:
//   backward  get_backward       src/globals/graph_types.cpp:389-413
//   forward   get_forward_pure   src/globals/graph_types.cpp:337-357
//             get_forward_rmpath src/globals/graph_types.cpp:305-322
// The reference materialises every extension as a 32-byte record
// (compute_extensions.cpp:243-390) and counts support per candidate with a
// records x candidates flag matrix (compute_support.cpp:805-960).  Here the
// count pass writes no records: each extension sets one bit in its key's
// bitmap over the node's graph ranks, so support = popcount; the
// materialise pass re-runs the enumeration for the selected children only.
#include "gs_kernels.hpp"

namespace gsgb {

namespace {

constexpr int kMaxV = 64;  // pattern vertices per embedding row
constexpr int kBlock = 256;

__device__ __forceinline__ int find_node_by_row(const NodeDesc *nodes, int n, long long r)
{
  int lo = 0, hi = n - 1;
  while(lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if(nodes[mid].row_begin <= r) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int find_node_by_key(const NodeDesc *nodes, int n, int key)
{
  int lo = 0, hi = n - 1;
  while(lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if(nodes[mid].key_base <= key) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Enumerates the valid one-edge extensions of embedding row i of a node and
// calls visit(key, neighbour, is_backward) for each.  phi receives the graph
// vertex of every pattern vertex.  Adds the algorithmic bytes read to bytes.
// Every data-dependent index is checked (back-link rows against column
// lengths, vertices against the database, pair indices against -1); a failed
// check skips the row and returns false so the caller can raise the error flag.
template <class Visit>
__device__ __forceinline__ bool enumerate_row(const NodeDesc &nd, const DevDB &db, const int2 *const *cols,
                                              const int32_t *collen, const SlotDesc *slots, const int32_t *vtab,
                                              int i, int *phi, int &last_prev, unsigned &bytes, Visit &visit)
{
  int idx = i;
  for(int c = nd.k - 1; c >= 0; --c) {
    if((unsigned)idx >= (unsigned)collen[c]) return false;
    const int2 e = __ldg(&cols[c][idx]);
    if((unsigned)e.x >= (unsigned)db.n_vertices) return false;
    phi[c] = e.x;
    if(c == nd.k - 1) last_prev = e.y;
    idx = e.y;
  }
  bytes += 8u * nd.k;
  const int rlab = slots[nd.nslot - 1].vlab;
  for(int s = 0; s < nd.nslot; ++s) {
    const SlotDesc sd = slots[s];
    const bool is_r = (s == nd.nslot - 1);
    const int v = phi[sd.vertex];
    const int a0 = __ldg(&db.adj_off[v]), a1 = __ldg(&db.adj_off[v + 1]);
    bytes += 8u + 8u * (unsigned)(a1 - a0);
    for(int e = a0; e < a1; ++e) {
      const unsigned long long a = __ldg(&db.adj[e]);
      const int w = (int)(unsigned)(a & 0xffffffffull);
      const unsigned hi = (unsigned)(a >> 32);
      const int el = (int)(hi >> 16), wl = (int)(hi & 0xffffu);
      if(!is_r) {
        // forward from a right-most-path vertex: label and order rules first
        if(wl < nd.minlabel) continue;
        if(!(sd.fel < el || (sd.fel == el && sd.ftl <= wl))) continue;
        bool in_emb = false;
        for(int t = 0; t < nd.k; ++t) in_emb |= (phi[t] == w);
        if(in_emb) continue;
        const int pk = __ldg(&db.pair_idx[((long long)sd.vlab * db.EL + el) * db.VL + wl]);
        if(pk < 0) return false;
        visit(sd.fkey_off + pk, w, false);
      } else {
        int j = -1;
        for(int t = 0; t < nd.k; ++t) if(phi[t] == w) j = t;
        if(j >= 0) {
          // backward edge from the right-most vertex to a right-most-path vertex
          const int bs = vtab[j];
          if(bs >= 0) {
            const SlotDesc &bd = slots[bs];
            if(bd.bel < el || (bd.bel == el && bd.blab <= rlab)) visit(bd.bkey_off + el, w, true);
          }
          continue;
        }
        if(wl < nd.minlabel) continue;
        const int pk = __ldg(&db.pair_idx[((long long)sd.vlab * db.EL + el) * db.VL + wl]);
        if(pk < 0) return false;
        visit(sd.fkey_off + pk, w, false);
      }
    }
  }
  return true;
}

struct CountVisit {
  uint32_t *bm;
  int32_t *cnt;
  long long base;
  int words, g, key_base;
  unsigned n;
  __device__ __forceinline__ void operator()(int key, int, bool)
  {
    atomicOr(&bm[base + (long long)key * words + (g >> 5)], 1u << (g & 31));
    atomicAdd(&cnt[key_base + key], 1);
    n++;
  }
};

struct MatVisit {
  const uint32_t *bm;
  const int32_t *bmx;
  const int32_t *childmap;
  int32_t *cursor;
  const ChildOut *outs;
  const int *phi;         // filled by the walk before the first visit
  const int *last_prev;   // back-link of the last column's row (backward children copy it)
  long long base;
  int words, g, key_base, row, k;
  unsigned n, nsel;
  bool overflow;
  __device__ __forceinline__ void operator()(int key, int w, bool bwd)
  {
    n++;
    const int c = childmap[key_base + key];
    if(c < 0) return;
    nsel++;
    const long long wi = base + (long long)key * words + (g >> 5);
    const int rank = bmx[wi] + __popc(bm[wi] & ((1u << (g & 31)) - 1u));
    const int pos = atomicAdd(&cursor[c], 1);
    const ChildOut o = outs[c];
    if(pos >= o.cap) {  // more rows than the count pass saw: never write past the slot
      overflow = true;
      return;
    }
    o.col[pos] = bwd ? make_int2(phi[k - 1], *last_prev) : make_int2(w, row);
    o.gord[pos] = rank;
  }
};

__device__ __forceinline__ void add_bytes(unsigned long long *bytes, unsigned long long mine)
{
  if(!bytes) return;
  // warp-reduce, one atomic per warp
  for(int o = 16; o > 0; o >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, o);
  if((threadIdx.x & 31) == 0 && mine) atomicAdd(bytes, mine);
}

__global__ void __launch_bounds__(kBlock) k_wave_count(const NodeDesc *__restrict__ nodes, int nnodes,
                                                        long long total_rows, const int2 *const *__restrict__ coltab,
                                                        const int32_t *__restrict__ collen,
                                                        const SlotDesc *__restrict__ slottab,
                                                        const int32_t *__restrict__ vtab,
                                                        const DevDB *__restrict__ dbs, uint32_t *bm, int32_t *cnt,
                                                        unsigned long long *bytes, unsigned int *err)
{
  int phi[kMaxV];
  unsigned long long mine = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for(long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < total_rows; r += stride) {
    const int n = find_node_by_row(nodes, nnodes, r);
    const NodeDesc nd = nodes[n];
    const DevDB db = dbs[nd.db];
    const int i = (int)(r - nd.row_begin);
    const int g = nd.gord[i];
    if((unsigned)g >= (unsigned)nd.words * 32u) {
      atomicOr(err, 1u);
      continue;
    }
    CountVisit v{ bm, cnt, nd.bm_base, nd.words, g, nd.key_base, 0u };
    int last_prev = 0;
    unsigned b = 0;
    if(!enumerate_row(nd, db, coltab + nd.col_off, collen + nd.col_off, slottab + nd.slot_off, vtab + nd.vtab_off,
                      i, phi, last_prev, b, v))
      atomicOr(err, 2u);
    mine += b + 4u + 8ull * v.n;  // gord read; one bitmap word and one counter update per extension
  }
  add_bytes(bytes, mine);
}

__global__ void __launch_bounds__(kBlock) k_wave_materialize(
    const NodeDesc *__restrict__ nodes, int nnodes, long long total_rows, const int2 *const *__restrict__ coltab,
    const int32_t *__restrict__ collen, const SlotDesc *__restrict__ slottab, const int32_t *__restrict__ vtab,
    const DevDB *__restrict__ dbs, const uint32_t *__restrict__ bm, const int32_t *__restrict__ bmx,
    const int32_t *__restrict__ childmap, int32_t *cursor, const ChildOut *__restrict__ outs,
    unsigned long long *bytes, unsigned int *err)
{
  int phi[kMaxV];
  unsigned long long mine = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for(long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < total_rows; r += stride) {
    const int n = find_node_by_row(nodes, nnodes, r);
    const NodeDesc nd = nodes[n];
    const DevDB db = dbs[nd.db];
    const int i = (int)(r - nd.row_begin);
    const int g = nd.gord[i];
    if((unsigned)g >= (unsigned)nd.words * 32u) {
      atomicOr(err, 1u);
      continue;
    }
    int last_prev = 0;
    MatVisit v{ bm, bmx, childmap, cursor, outs, phi, &last_prev, nd.bm_base, nd.words, g, nd.key_base, i, nd.k,
                0u, 0u, false };
    unsigned b = 0;
    if(!enumerate_row(nd, db, coltab + nd.col_off, collen + nd.col_off, slottab + nd.slot_off, vtab + nd.vtab_off,
                      i, phi, last_prev, b, v))
      atomicOr(err, 2u);
    if(v.overflow) atomicOr(err, 4u);
    mine += b + 4u + 4ull * v.n + 20ull * v.nsel;  // childmap per extension; bitmap, prefix, column, rank per selected
  }
  add_bytes(bytes, mine);
}

__global__ void __launch_bounds__(kBlock) k_root_count(DevDB db, const int32_t *__restrict__ root_off, uint32_t *bm,
                                                        int32_t *cnt, int32_t words, unsigned long long *bytes)
{
  unsigned long long mine = 0;
  const int stride = gridDim.x * blockDim.x;
  for(int v = blockIdx.x * blockDim.x + threadIdx.x; v < db.n_vertices; v += stride) {
    const int fl = db.vlabel[v];
    const int g = db.vgraph[v];
    const int a0 = db.adj_off[v], a1 = db.adj_off[v + 1];
    mine += 16u + 8u * (unsigned)(a1 - a0);
    for(int e = a0; e < a1; ++e) {
      const unsigned long long a = __ldg(&db.adj[e]);
      const unsigned hi = (unsigned)(a >> 32);
      const int el = (int)(hi >> 16), wl = (int)(hi & 0xffffu);
      if(fl > wl) continue;
      const int key = root_off[fl] + __ldg(&db.pair_idx[((long long)fl * db.EL + el) * db.VL + wl]);
      atomicOr(&bm[(long long)key * words + (g >> 5)], 1u << (g & 31));
      atomicAdd(&cnt[key], 1);
      mine += 8u;
    }
  }
  add_bytes(bytes, mine);
}

__global__ void __launch_bounds__(kBlock) k_root_materialize(DevDB db, const int32_t *__restrict__ root_off,
                                                              const uint32_t *__restrict__ bm,
                                                              const int32_t *__restrict__ bmx, int32_t words,
                                                              const int32_t *__restrict__ childmap, int32_t *cursor,
                                                              const ChildOut *__restrict__ outs, unsigned int *err)
{
  const int stride = gridDim.x * blockDim.x;
  for(int v = blockIdx.x * blockDim.x + threadIdx.x; v < db.n_vertices; v += stride) {
    const int fl = db.vlabel[v];
    const int g = db.vgraph[v];
    const int a0 = db.adj_off[v], a1 = db.adj_off[v + 1];
    for(int e = a0; e < a1; ++e) {
      const unsigned long long a = __ldg(&db.adj[e]);
      const int w = (int)(unsigned)(a & 0xffffffffull);
      const unsigned hi = (unsigned)(a >> 32);
      const int el = (int)(hi >> 16), wl = (int)(hi & 0xffffu);
      if(fl > wl) continue;
      const int key = root_off[fl] + __ldg(&db.pair_idx[((long long)fl * db.EL + el) * db.VL + wl]);
      const int c = childmap[key];
      if(c < 0) continue;
      const long long wi = (long long)key * words + (g >> 5);
      const int rank = bmx[wi] + __popc(bm[wi] & ((1u << (g & 31)) - 1u));
      const int pos = atomicAdd(&cursor[c], 1);
      const ChildOut o = outs[c];
      if(pos >= o.cap) {
        atomicOr(err, 4u);
        continue;
      }
      o.col0[pos] = make_int2(v, -1);
      o.col[pos] = make_int2(w, pos);
      o.gord[pos] = rank;
    }
  }
}

__global__ void __launch_bounds__(kBlock) k_support(const NodeDesc *__restrict__ nodes, int nnodes, int total_keys,
                                                     const uint32_t *__restrict__ bm, int32_t *bmx, int32_t *support)
{
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for(int key = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; key < total_keys; key += warps) {
    const int n = find_node_by_key(nodes, nnodes, key);
    const NodeDesc &nd = nodes[n];
    const long long base = nd.bm_base + (long long)(key - nd.key_base) * nd.words;
    int running = 0;
    for(int w0 = 0; w0 < nd.words; w0 += 32) {
      const int w = w0 + lane;
      const int c = (w < nd.words) ? __popc(bm[base + w]) : 0;
      int incl = c;
      for(int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if(lane >= o) incl += t;
      }
      if(w < nd.words) bmx[base + w] = running + incl - c;
      running += __shfl_sync(0xffffffffu, incl, 31);
    }
    if(lane == 0) support[key] = running;
  }
}

__global__ void __launch_bounds__(kBlock) k_records_bitmap(const int32_t *__restrict__ keys,
                                                            const int32_t *__restrict__ gids, long long n, int words,
                                                            uint32_t *bm)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int k = keys[i], g = gids[i];
    atomicOr(&bm[(long long)k * words + (g >> 5)], 1u << (g & 31));
  }
}

inline int grid_for(long long n)
{
  long long b = (n + kBlock - 1) / kBlock;
  if(b < 1) b = 1;
  const long long cap = 152LL * 16;  // 16 resident CTAs per SM worth of work, grid-stride beyond
  return (int)(b < cap ? b : cap);
}

}  // namespace

void launch_root_count(const DevDB &db, const int32_t *root_off, uint32_t *bm, int32_t *cnt, int32_t words,
                       unsigned long long *bytes, cudaStream_t s)
{
  k_root_count<<<grid_for(db.n_vertices), kBlock, 0, s>>>(db, root_off, bm, cnt, words, bytes);
}

void launch_root_materialize(const DevDB &db, const int32_t *root_off, const uint32_t *bm, const int32_t *bmx,
                             int32_t words, const int32_t *childmap, int32_t *cursor, const ChildOut *outs,
                             unsigned int *err, cudaStream_t s)
{
  k_root_materialize<<<grid_for(db.n_vertices), kBlock, 0, s>>>(db, root_off, bm, bmx, words, childmap, cursor, outs,
                                                                 err);
}

void launch_wave_count(const NodeDesc *nodes, int32_t nnodes, long long total_rows, const int2 *const *coltab,
                       const int32_t *collen, const SlotDesc *slots, const int32_t *vtab, const DevDB *dbs,
                       uint32_t *bm, int32_t *cnt, unsigned long long *bytes, unsigned int *err, cudaStream_t s)
{
  if(total_rows <= 0) return;
  k_wave_count<<<grid_for(total_rows), kBlock, 0, s>>>(nodes, nnodes, total_rows, coltab, collen, slots, vtab, dbs,
                                                        bm, cnt, bytes, err);
}

void launch_wave_materialize(const NodeDesc *nodes, int32_t nnodes, long long total_rows, const int2 *const *coltab,
                             const int32_t *collen, const SlotDesc *slots, const int32_t *vtab, const DevDB *dbs,
                             const uint32_t *bm, const int32_t *bmx, const int32_t *childmap, int32_t *cursor,
                             const ChildOut *outs, unsigned long long *bytes, unsigned int *err, cudaStream_t s)
{
  if(total_rows <= 0) return;
  k_wave_materialize<<<grid_for(total_rows), kBlock, 0, s>>>(nodes, nnodes, total_rows, coltab, collen, slots, vtab,
                                                              dbs, bm, bmx, childmap, cursor, outs, bytes, err);
}

void launch_records_bitmap(const int32_t *keys, const int32_t *gids, long long n, int32_t words, uint32_t *bm,
                           cudaStream_t s)
{
  if(n <= 0) return;
  k_records_bitmap<<<grid_for(n), kBlock, 0, s>>>(keys, gids, n, words, bm);
}

void launch_support(const NodeDesc *nodes, int32_t nnodes, int32_t total_keys, const uint32_t *bm, int32_t *bmx,
                    int32_t *support, cudaStream_t s)
{
  if(total_keys <= 0) return;
  k_support<<<grid_for((long long)total_keys * 32), kBlock, 0, s>>>(nodes, nnodes, total_keys, bm, bmx, support);
}

}  // namespace gsgb
