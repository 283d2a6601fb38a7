// Root-level and support kernels for one GB300 (sm_103a); the wave-level
// extension kernels are in gs_wave.cu.
//
// Support is counted without extension records: every embedding of a
// candidate sets one bit in the candidate's bitmap over the graph ranks of
// its parent node, so support = popcount.  The reference instead sorts or
// flags 32-byte extension records per candidate (compute_support.cpp:146-257,
// 805-960).
#include "gs_kernels.hpp"

namespace gsgb {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ int find_node_by_key(const NodeDesc *nodes, int n, int key)
{
  int lo = 0, hi = n - 1;
  while(lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if(nodes[mid].key_base <= key) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void add_bytes(unsigned long long *bytes, unsigned long long mine)
{
  if(!bytes) return;
  // warp-reduce, one atomic per warp
  for(int o = 16; o > 0; o >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, o);
  if((threadIdx.x & 31) == 0 && mine) atomicAdd(bytes, mine);
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
