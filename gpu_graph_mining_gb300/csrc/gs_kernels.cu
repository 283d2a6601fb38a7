// Root-level and support kernels for one GB300 (sm_103a); the wave-level
// extension kernels are in gs_wave.cu.
//
// Support is counted without extension records: every embedding of a
// candidate sets one bit in the candidate's bitmap over the graph ranks of
// its parent node, so support = popcount.  The reference instead sorts or
// flags 32-byte extension records per candidate (compute_support.cpp:146-257,
// 805-960).
#include "gs_kernels.hpp"
#include "gs_lists.cuh"

namespace gsgb {

int sm_count()
{
  static const int n = [] {
    int v = 0;
    if(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, 0) != cudaSuccess || v <= 0) {
      cudaGetLastError();
      v = 152;
    }
    return v;
  }();
  return n;
}

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

__device__ __forceinline__ unsigned lanemask_lt()
{
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Root level, warp-cooperative: a warp owns 32 consecutive vertices, whose
// adjacency entries form one contiguous range; lanes take consecutive entries
// (coalesced 8-byte loads) and find their source vertex by a 5-step shuffle
// search over the lanes' adjacency starts.  The warp stays converged, so the
// embedding counters and child cursors take one atomic per distinct key.
// The root level of a group of jobs in one launch: the jobs' vertex tiles
// laid end to end (a warp finds its tile's job in the table), each job's
// bitmaps, counter copies and keys at its own offsets.  The materialise pass
// runs the same grid over the same tiles, so a warp uses the same counter copy
// in both passes.
template <bool MAT>
__device__ __forceinline__ void root_tiles(const RootJob *__restrict__ jobs, int njobs, long long tiles,
                                           const DevDB *__restrict__ dbs, uint32_t *bm,
                                           const int32_t *__restrict__ bmx, int32_t *cnt,
                                           const int32_t *__restrict__ childmap, const ChildOut *__restrict__ outs,
                                           unsigned long long *bytes, unsigned int *err)
{
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  unsigned long long mine = 0;
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int jn = 0;  // a warp's tiles ascend, so its job index only moves forward
  for(long long tile = gw; tile < tiles; tile += nwarps) {
    while(jn + 1 < njobs && jobs[jn + 1].tile_begin <= tile) jn++;
    const RootJob J = jobs[jn];
    // the job's database: pointers into registers (the atomics below would
    // otherwise make the compiler re-read the table)
    const unsigned long long *__restrict__ adj = dbs[J.db].adj;
    const int32_t *__restrict__ adj_off = dbs[J.db].adj_off;
    const int32_t *__restrict__ vlabel = dbs[J.db].vlabel;
    const int32_t *__restrict__ vgraph = dbs[J.db].vgraph;
    const int32_t *__restrict__ adj_pair = dbs[J.db].adj_pair;
    const int32_t *__restrict__ root_off = dbs[J.db].root_off;
    const int n_vertices = dbs[J.db].n_vertices;
    // this warp's copy of the job's root counters (copies spread the hot
    // counters over L2 slices)
    const int cnt_copy_idx = (int)(gw % (J.copies > 0 ? J.copies : 1));
    int32_t *const cnt_copy = cnt + J.cnt_base + (long long)cnt_copy_idx * J.R;
    const long long vt = (tile - J.tile_begin) * 32;
    const long long v = vt + lane;
    const bool valid = v < n_vertices;
    const int a0 = valid ? __ldg(&adj_off[v]) : 0;
    const int a1 = valid ? __ldg(&adj_off[v + 1]) : 0;
    const int fl = valid ? __ldg(&vlabel[v]) : 0;
    const int g = valid ? __ldg(&vgraph[v]) : 0;
    const int W = a1 - a0;
    int incl = W;
    for(int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(full, incl, o);
      if(lane >= o) incl += t;
    }
    const int off = incl - W;
    const int T = __shfl_sync(full, incl, 31);
    if(valid) mine += 16;
    for(int base = 0; base < T; base += 32) {
      const int j = base + lane;
      const bool has = j < T;
      int o = 0;
#pragma unroll
      for(int step = 16; step >= 1; step >>= 1) {
        const int c = o + step;
        if(__shfl_sync(full, off, c) <= j) o = c;
      }
      const int e = __shfl_sync(full, a0, o) + (j - __shfl_sync(full, off, o));
      const int fl_o = __shfl_sync(full, fl, o);
      const int g_o = __shfl_sync(full, g, o);
      int key = -1, w = 0;
      if(has) {
        // entry, pair index and the label's first key: independent loads, in flight together
        const unsigned long long ent = __ldg(&adj[e]);
        const int pr = __ldg(&adj_pair[e]);
        const int ro = __ldg(&root_off[fl_o]);
        w = (int)(unsigned)(ent & 0xffffffffull);
        const unsigned hi = (unsigned)(ent >> 32);
        const int wl = (int)(hi & 0xffffu);
        mine += 8;
        if(fl_o <= wl) key = ro + pr;
      }
      if(!MAT) {
        if(key >= 0) {
          atomicOr(&bm[J.bm_base + (long long)key * J.words + (g_o >> 5)], 1u << (g_o & 31));
          mine += 8;
        }
        const unsigned peers = __match_any_sync(full, key);
        if(key >= 0 && lane == __ffs(peers) - 1) atomicAdd(&cnt_copy[key], __popc(peers));
      } else {
        const int c = key >= 0 ? childmap[J.key_base + key] : -1;
        const unsigned peers = __match_any_sync(full, c);
        const int leader = __ffs(peers) - 1;
        int pos = 0;
        // the cursor of this warp's counter copy of the key: the same warp
        // counted the same entries in the count pass (same grid, same tiles)
        if(c >= 0 && lane == leader) pos = atomicAdd(&cnt_copy[key], __popc(peers));
        pos = __shfl_sync(full, pos, leader) + __popc(peers & lanemask_lt());
        if(c >= 0) {
          const long long wi = J.bm_base + (long long)key * J.words + (g_o >> 5);
          const int rank = bmx[wi] + __popc(bm[wi] & ((1u << (g_o & 31)) - 1u));
          const ChildOut out = outs[c];
          if(pos < out.cap) {
            out.col0[pos] = make_int2((int)(vt + o), -1);
            out.col[pos] = make_int2(w, pos);
            out.gord[pos] = rank;
          } else {
            atomicOr(err, 4u);
          }
        }
      }
    }
  }
  if(!MAT) add_bytes(bytes, mine);
}

__global__ void __launch_bounds__(kBlock) k_root_count(const RootJob *__restrict__ jobs, int njobs, long long tiles,
                                                        const DevDB *__restrict__ dbs, uint32_t *bm, int32_t *cnt,
                                                        unsigned long long *bytes)
{
  root_tiles<false>(jobs, njobs, tiles, dbs, bm, nullptr, cnt, nullptr, nullptr, bytes, nullptr);
}

// Per key of the group, one warp: the job's counter copies turn into the
// offsets of each copy's share (copy q: the count of copies 0..q-1, a warp
// scan over the copies; copy 0 starts at 0 as the materialise pass's cursor)
// and the total goes to tot[key].
__global__ void __launch_bounds__(kBlock) k_sum_copies(const RootJob *__restrict__ jobs, int njobs, int total_keys,
                                                        int32_t *cnt, int32_t *tot)
{
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for(int kg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; kg < total_keys; kg += warps) {
    int lo = 0, hi = njobs - 1;
    while(lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if(jobs[mid].key_base <= kg) lo = mid; else hi = mid - 1;
    }
    const RootJob &J = jobs[lo];
    int32_t *c0 = cnt + J.cnt_base + (kg - J.key_base);
    int run = 0;
    for(int q0 = 0; q0 < J.copies; q0 += 32) {
      const int q = q0 + lane;
      const int x = q < J.copies ? c0[(long long)q * J.R] : 0;
      int incl = x;
      for(int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(full, incl, o);
        if(lane >= o) incl += t;
      }
      if(q < J.copies) c0[(long long)q * J.R] = run + incl - x;
      run += __shfl_sync(full, incl, 31);
    }
    if(lane == 0) tot[kg] = run;
  }
}

__global__ void __launch_bounds__(kBlock) k_root_materialize(const RootJob *__restrict__ jobs, int njobs,
                                                              long long tiles, const DevDB *__restrict__ dbs,
                                                              const uint32_t *__restrict__ bm,
                                                              const int32_t *__restrict__ bmx, int32_t *cursor,
                                                              const int32_t *__restrict__ childmap,
                                                              const ChildOut *__restrict__ outs, unsigned int *err)
{
  root_tiles<true>(jobs, njobs, tiles, dbs, const_cast<uint32_t *>(bm), bmx, cursor, childmap, outs, nullptr, err);
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

// Support of the candidates of one wave, and their selection, in two passes.
// Screening, one thread per key: a key with fewer embeddings than its node's
// minsup cannot be found in that many graphs, so only keys with cnt >= minsup
// are listed for counting; every key with embeddings gets childmap -1
// (overwritten afterwards for the children that are materialised).
// Counting, one warp per listed key: popcount of its bitmap with prefix
// counts for the materialise pass; the frequent keys are appended to sel as
// {key, support, embeddings, node << 2} (order unspecified; the low two bits
// take the canonicality verdict) and get keyword = their
// first bitmap word.  counters: [0] selected, [1] embeddings of all keys,
// [2] listed keys.
__global__ void __launch_bounds__(kBlock) k_screen_keys(const NodeDesc *__restrict__ nodes, int nnodes,
                                                         int total_keys, int32_t *cnt, int cnt_copies,
                                                         long long cnt_stride, int32_t *childmap, int2 *listed,
                                                         unsigned long long *counters,
                                                         unsigned int *err, unsigned long long *err_copy,
                                                         int32_t *lnode)
{
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  unsigned long long ext = 0, bytes = 0;
  // the consistency flags so far (the count pass has finished) travel back
  // with the wave's results
  if(blockIdx.x == 0 && threadIdx.x == 0) *err_copy = *err;
  // warp-uniform trip count: the list append below is warp-aggregated
  const long long n32 = ((long long)total_keys + 31) & ~31ll;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n32; i += stride) {
    const int key = (int)i;
    int c = 0;
    if(key < total_keys) {
      // the count pass spread its adds over copies: their total.  A copy that
      // wrapped (negative) or a total past 2^31 - 1 is clamped to 2^31 - 1
      // and flagged (bit 8): the host refuses such a key
      long long c64 = cnt[key];
      bool wrap = c64 < 0;
      for(int q = 1; q < cnt_copies; q++) {
        const int x = cnt[q * cnt_stride + key];
        wrap = wrap || x < 0;
        c64 += x;
      }
      if(wrap || c64 > (long long)INT32_MAX) {
        atomicOr(err, 8u);
        c = INT32_MAX;
      } else {
        c = (int)c64;
      }
      bytes += 4ull * (unsigned)cnt_copies;  // the counter copies read
    }
    int n = 0;
    bool cand = false;
    if(c > 0) {
      childmap[key] = -1;
      if(lnode) lnode[key] = -1;
      ext += (unsigned long long)c;
      n = find_node_by_key(nodes, nnodes, key);
      cand = c >= nodes[n].minsup;
      bytes += lnode ? 8 : 4;  // child map (and list node) reset
    }
    if(cand && cnt_copies > 1) {
      // a key that may be materialised: copy 0 keeps the total, copy q >= 1
      // becomes the count of copies 0..q-1 (the offset of its share)
      int run = cnt[key];
      for(int q = 1; q < cnt_copies; q++) {
        const int x = cnt[q * cnt_stride + key];
        cnt[q * cnt_stride + key] = run;
        run += x;
      }
      cnt[key] = c;
      bytes += 4ull * (unsigned)cnt_copies;  // the copies turned into offsets
    }
    if(cand) bytes += 8;  // the listed entry
    const unsigned m = __ballot_sync(full, cand);
    if(m) {
      unsigned long long at = 0;
      if(lane == 0) at = atomicAdd(&counters[2], (unsigned long long)__popc(m));
      at = __shfl_sync(full, at, 0);
      if(cand) listed[at + __popc(m & lanemask_lt())] = make_int2(key, n);
    }
  }
  for(int o = 16; o > 0; o >>= 1) {
    ext += __shfl_down_sync(full, ext, o);
    bytes += __shfl_down_sync(full, bytes, o);
  }
  if(lane == 0 && ext) atomicAdd(&counters[1], ext);
  if(lane == 0 && bytes) atomicAdd(&counters[3], bytes);
}

// A listed key's support: its bitmap words popcounted, their exclusive
// prefixes written (bmx), the total compared with minsup.  A key of at most
// kBigWords words is taken by one warp, 4 words per lane per step; a larger
// one (a key present in up to a million graphs has 31,250 words) by a whole
// block, 8 words per thread per step, so that its words are not read by one
// warp in a long chain of dependent steps.
constexpr int kBigWords = 1024;

__device__ __forceinline__ void listed_done(const int2 kn, const NodeDesc &nd, long long wbase, int running,
                                            int32_t *cnt, long long *keyword, int4 *sel, int sel_cap,
                                            unsigned long long *counters, int32_t *lnode)
{
  // algorithmic bytes: the listed entry, each bitmap word read and its
  // prefix written, and for a selected key its word offset, result and counter
  atomicAdd(&counters[3], 8ull + 8ull * (unsigned)nd.words + (running >= nd.minsup ? 32ull : 0ull));
  if(running >= nd.minsup) {
    keyword[kn.x] = wbase;
    const unsigned long long at = atomicAdd(&counters[0], 1ull);
    if(at < (unsigned long long)sel_cap) sel[at] = make_int4(kn.x, running, cnt[kn.x], kn.y << 2);
    // the total has been read: copy 0 turns into the cursor of copy 0's share
    cnt[kn.x] = 0;
    // lists strategy: a frequent forward key goes into its node's per-row lists
    if(lnode && kn.x - nd.key_base < nd.nfwd) lnode[kn.x] = kn.y;
  }
}

__global__ void __launch_bounds__(kBlock) k_count_listed(const NodeDesc *__restrict__ nodes,
                                                          const int2 *__restrict__ listed,
                                                          const uint32_t *__restrict__ bm,
                                                          int32_t *cnt, int32_t *bmx,
                                                          long long *keyword, int4 *sel, int sel_cap,
                                                          unsigned long long *counters, int32_t *lnode)
{
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long nlisted = (long long)counters[2];
  // small keys: one warp each
  const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
  for(long long li = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; li < nlisted; li += warps) {
    const int2 kn = listed[li];
    const NodeDesc &nd = nodes[kn.y];
    const int words = nd.words;
    if(words > kBigWords) continue;
    const long long wbase = nd.bm_base + (long long)(kn.x - nd.key_base) * words;
    int running = 0;
    for(int w0 = 0; w0 < words; w0 += 128) {
      const int w = w0 + 4 * lane;
      int c[4], t = 0;
#pragma unroll
      for(int q = 0; q < 4; q++) {
        c[q] = (w + q < words) ? __popc(bm[wbase + w + q]) : 0;
        t += c[q];
      }
      int incl = t;
      for(int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(full, incl, o);
        if(lane >= o) incl += u;
      }
      int at = running + incl - t;
#pragma unroll
      for(int q = 0; q < 4; q++) {
        if(w + q < words) bmx[wbase + w + q] = at;
        at += c[q];
      }
      running += __shfl_sync(full, incl, 31);
    }
    if(lane == 0) listed_done(kn, nd, wbase, running, cnt, keyword, sel, sel_cap, counters, lnode);
  }
  // large keys: one block each (the branch below is uniform over the block)
  __shared__ int wtot[kBlock / 32];
  constexpr int kPer = 8, kStep = kBlock * kPer;
  for(long long li = blockIdx.x; li < nlisted; li += gridDim.x) {
    const int2 kn = listed[li];
    const NodeDesc &nd = nodes[kn.y];
    const int words = nd.words;
    if(words <= kBigWords) continue;
    const long long wbase = nd.bm_base + (long long)(kn.x - nd.key_base) * words;
    int running = 0;
    for(int w0 = 0; w0 < words; w0 += kStep) {
      const int w = w0 + kPer * threadIdx.x;
      int c[kPer], t = 0;
#pragma unroll
      for(int q = 0; q < kPer; q++) {
        c[q] = (w + q < words) ? __popc(bm[wbase + w + q]) : 0;
        t += c[q];
      }
      int incl = t;
      for(int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(full, incl, o);
        if(lane >= o) incl += u;
      }
      if(lane == 31) wtot[warp] = incl;
      __syncthreads();
      int before = 0, total = 0;
#pragma unroll
      for(int x = 0; x < kBlock / 32; x++) {
        const int v = wtot[x];
        if(x < warp) before += v;
        total += v;
      }
      int at = running + before + incl - t;
#pragma unroll
      for(int q = 0; q < kPer; q++) {
        if(w + q < words) bmx[wbase + w + q] = at;
        at += c[q];
      }
      running += total;
      __syncthreads();  // wtot is rewritten by the next step
    }
    if(threadIdx.x == 0) listed_done(kn, nd, wbase, running, cnt, keyword, sel, sel_cap, counters, lnode);
  }
}

// ---- lists strategy: per-row lists of the frequent forward extensions

// cursor[r] starts at list row r's offset and ends at the next row's
__global__ void __launch_bounds__(kBlock) k_list_fill(const int4 *__restrict__ rec, long long n, const ListBuild lb,
                                                      int32_t *cursor, int2 *ent, long long ent_cap,
                                                      unsigned int *err)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int4 x = __ldg(&rec[i]);
    long long row;
    int lk;
    if(list_entry(x, lb, row, lk, err)) {
      const int pos = atomicAdd(&cursor[row], 1);
      if((unsigned)pos < (unsigned long long)ent_cap) ent[pos] = make_int2(x.y, lk);
      else atomicOr(err, 4u);
    }
  }
}

// ---- exclusive scan of int32 counts in place, 1024 per block
constexpr int kScanPer = 1024;

__global__ void __launch_bounds__(kBlock) k_xscan_blocks(int32_t *x, long long n, int32_t *sums)
{
  __shared__ int32_t wsum[kBlock / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long base = (long long)blockIdx.x * kScanPer + (long long)threadIdx.x * 4;
  int v[4], t = 0;
#pragma unroll
  for(int j = 0; j < 4; j++) {
    v[j] = base + j < n ? x[base + j] : 0;
    t += v[j];
  }
  int incl = t;
  for(int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, o);
    if(lane >= o) incl += u;
  }
  if(lane == 31) wsum[w] = incl;
  __syncthreads();
  if(w == 0) {
    int y = lane < kBlock / 32 ? wsum[lane] : 0;
    for(int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, y, o);
      if(lane >= o) y += u;
    }
    if(lane < kBlock / 32) wsum[lane] = y;
  }
  __syncthreads();
  int run = (w > 0 ? wsum[w - 1] : 0) + incl - t;
#pragma unroll
  for(int j = 0; j < 4; j++) {
    if(base + j < n) x[base + j] = run;
    run += v[j];
  }
  if(threadIdx.x == kBlock - 1) sums[blockIdx.x] = run;
}

__global__ void __launch_bounds__(kBlock) k_xscan_add(int32_t *x, long long n, const int32_t *offs)
{
  const long long base = (long long)blockIdx.x * kScanPer;
  const int add = offs[blockIdx.x];
  for(int j = threadIdx.x; j < kScanPer; j += kBlock)
    if(base + j < n) x[base + j] += add;
}

// x[0..n) -> exclusive prefix sums; scratch: xscan_scratch(n) ints
long long xscan_scratch(long long n)
{
  long long tot = 0;
  while(n > 1) {
    n = (n + kScanPer - 1) / kScanPer;
    tot += n;
  }
  return tot;
}

void xscan(int32_t *x, long long n, int32_t *scratch, cudaStream_t s)
{
  if(n <= 0) return;
  const long long nb = (n + kScanPer - 1) / kScanPer;
  k_xscan_blocks<<<(unsigned)nb, kBlock, 0, s>>>(x, n, scratch);
  if(nb > 1) {
    xscan(scratch, nb, scratch + nb, s);
    k_xscan_add<<<(unsigned)nb, kBlock, 0, s>>>(x, n, scratch);
  }
}

// childmap[pairs[i].x] = pairs[i].y for the children to materialise, and
// their output cursors reset
__global__ void __launch_bounds__(kBlock) k_scatter_childmap(const int2 *__restrict__ pairs, int n, int32_t *childmap,
                                                              int32_t *cursor, int ncursor)
{
  const int m = n > ncursor ? n : ncursor;
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    if(i < n) {
      const int2 p = pairs[i];
      childmap[p.x] = p.y;
    }
    if(i < ncursor) cursor[i] = 0;
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
  const long long cap = 16LL * sm_count();  // 16 resident CTAs per SM worth of work, grid-stride beyond
  return (int)(b < cap ? b : cap);
}

}  // namespace

void launch_root_count(const RootJob *jobs, int32_t njobs, long long tiles, const DevDB *dbs, uint32_t *bm,
                       int32_t *cnt, int32_t *tot, int32_t total_keys, unsigned long long *bytes, cudaStream_t s)
{
  if(tiles > 0) k_root_count<<<grid_for(tiles * 32), kBlock, 0, s>>>(jobs, njobs, tiles, dbs, bm, cnt, bytes);
  if(total_keys > 0)
    k_sum_copies<<<grid_for((long long)total_keys * 32), kBlock, 0, s>>>(jobs, njobs, total_keys, cnt, tot);
}

void launch_root_materialize(const RootJob *jobs, int32_t njobs, long long tiles, const DevDB *dbs,
                             const uint32_t *bm, const int32_t *bmx, int32_t *cursor, const int32_t *childmap,
                             const ChildOut *outs, unsigned int *err, cudaStream_t s)
{
  // the same grid as the count pass: warp w processes the same tiles and uses
  // the same counter copy
  if(tiles > 0)
    k_root_materialize<<<grid_for(tiles * 32), kBlock, 0, s>>>(jobs, njobs, tiles, dbs, bm, bmx, cursor, childmap,
                                                                outs, err);
}

void launch_records_bitmap(const int32_t *keys, const int32_t *gids, long long n, int32_t words, uint32_t *bm,
                           cudaStream_t s)
{
  if(n <= 0) return;
  k_records_bitmap<<<grid_for(n), kBlock, 0, s>>>(keys, gids, n, words, bm);
}

KernelCall screen_keys_call(const NodeDesc *nodes, int32_t nnodes, int32_t total_keys, int32_t *cnt,
                            int32_t cnt_copies, long long cnt_stride, int32_t *childmap, int2 *listed,
                            unsigned long long *counters, unsigned int *err, unsigned long long *err_copy,
                            int32_t *lnode)
{
  KernelCall c;
  c.func = (const void *)k_screen_keys;
  c.grid = dim3((unsigned)grid_for(((long long)total_keys + 31) / 32 * 32));
  c.block = dim3(kBlock);
  c.arg(nodes);
  c.arg(nnodes);
  c.arg(total_keys);
  c.arg(cnt);
  c.arg(cnt_copies);
  c.arg(cnt_stride);
  c.arg(childmap);
  c.arg(listed);
  c.arg(counters);
  c.arg(err);
  c.arg(err_copy);
  c.arg(lnode);
  return c;
}

KernelCall count_listed_call(const NodeDesc *nodes, const int2 *listed, const uint32_t *bm, int32_t *cnt,
                             int32_t *bmx, long long *keyword, int4 *sel, int32_t sel_cap,
                             unsigned long long *counters, int32_t *lnode)
{
  KernelCall c;
  c.func = (const void *)k_count_listed;
  c.grid = dim3((unsigned)(8 * sm_count()));
  c.block = dim3(kBlock);
  c.arg(nodes);
  c.arg(listed);
  c.arg(bm);
  c.arg(cnt);
  c.arg(bmx);
  c.arg(keyword);
  c.arg(sel);
  c.arg(sel_cap);
  c.arg(counters);
  c.arg(lnode);
  return c;
}

// ---- the reference's packed segmented scan and reduce as single operators
// (gs_segmented_scan / gs_segmented_reduce).  Element i holds a value in bits
// 0-30 and, in bit 31, a flag that starts a new segment (element 0 always
// starts one): the packed layout of src/reduction/segscanpacked.cu.  The
// segmented scan is two plain scans: one over the values (positions P) and
// one over the flags (segment numbers); a segment's result is P minus P at
// its first element.  Sums wrap modulo 2^32 like the reference's uint scans.

__global__ void __launch_bounds__(kBlock) k_seg_split(const uint32_t *__restrict__ x, long long n, int32_t *val,
                                                     int32_t *pos, int32_t *head, int32_t *seg)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint32_t v = x[i];
    const int32_t h = (i == 0 || (v >> 31)) ? 1 : 0;
    val[i] = (int32_t)(v & 0x7fffffffu);
    pos[i] = (int32_t)(v & 0x7fffffffu);
    head[i] = h;
    seg[i] = h;
  }
}

// pos, seg: exclusive scans of the values and of the flags
__global__ void __launch_bounds__(kBlock) k_seg_base(const int32_t *__restrict__ pos, const int32_t *__restrict__ head,
                                                    const int32_t *__restrict__ seg, long long n, int32_t *base)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    if(head[i]) base[seg[i]] = pos[i];
}

__global__ void __launch_bounds__(kBlock) k_seg_out(const int32_t *__restrict__ val, const int32_t *__restrict__ pos,
                                                   const int32_t *__restrict__ head, const int32_t *__restrict__ seg,
                                                   const int32_t *__restrict__ base, long long n, int exclusive,
                                                   uint32_t *out)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int32_t s = seg[i] + head[i] - 1;
    uint32_t r = (uint32_t)pos[i] - (uint32_t)base[s];
    if(!exclusive) r += (uint32_t)val[i];
    out[i] = r;
  }
}

__global__ void __launch_bounds__(kBlock) k_gather_ends(const uint32_t *__restrict__ scanned,
                                                       const long long *__restrict__ ends, long long m, long long n,
                                                       uint32_t *res, unsigned int *err)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  for(long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < m; j += stride) {
    const long long e = ends[j];
    if(e < 0 || e >= n) {
      atomicOr(err, 1u);
      res[j] = 0;
    } else {
      res[j] = scanned[e];
    }
  }
}

int64_t segmented_scan_scratch(int64_t n) { return 5 * n + xscan_scratch(n); }

void launch_segmented_scan(const uint32_t *x, int64_t n, int exclusive, int32_t *scratch, uint32_t *out,
                           cudaStream_t s)
{
  if(n <= 0) return;
  int32_t *val = scratch, *pos = val + n, *head = pos + n, *seg = head + n, *base = seg + n, *xs = base + n;
  const int g = grid_for(n);
  k_seg_split<<<g, kBlock, 0, s>>>(x, n, val, pos, head, seg);
  xscan(pos, n, xs, s);
  xscan(seg, n, xs, s);
  k_seg_base<<<g, kBlock, 0, s>>>(pos, head, seg, n, base);
  k_seg_out<<<g, kBlock, 0, s>>>(val, pos, head, seg, base, n, exclusive, out);
}

void launch_gather_ends(const uint32_t *scanned, int64_t n, const long long *ends, int64_t m, uint32_t *res,
                        unsigned int *err, cudaStream_t s)
{
  if(m <= 0) return;
  k_gather_ends<<<grid_for(m), kBlock, 0, s>>>(scanned, ends, m, n, res, err);
}

// ---- backward child column on its own (gs_filter_backward)
// flag[row] = 1 for every record {from, to, fromlabel, elabel, tolabel,
// from_grph, to_grph, row} equal to the edge e0..e4
__global__ void __launch_bounds__(kBlock) k_bwd_mark(const int32_t *__restrict__ rec, long long nrec, int e0, int e1,
                                                     int e2, int e3, int e4, int32_t *flag, long long nrows)
{
  for(long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < nrec; r += (long long)gridDim.x * blockDim.x) {
    const int32_t *x = rec + 8 * r;
    if(x[0] == e0 && x[1] == e1 && x[2] == e2 && x[3] == e3 && x[4] == e4 && (unsigned long long)x[7] < (unsigned long long)nrows)
      flag[x[7]] = 1;
  }
}

// the flagged rows' elements in row order: pos = the flags' exclusive scan
// (n + 1 entries), row r flagged iff pos[r + 1] > pos[r]
__global__ void __launch_bounds__(kBlock) k_bwd_gather(const int2 *__restrict__ col, const int32_t *__restrict__ pos,
                                                       long long n, int2 *out)
{
  for(long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
    const int p = pos[r];
    if(pos[r + 1] > p) out[p] = col[r];
  }
}

int64_t list_scan_scratch(int64_t n) { return xscan_scratch(n) + 1; }

int64_t filter_backward_scratch(int64_t nrows) { return xscan_scratch(nrows + 1); }

void launch_filter_backward(const int2 *col, int64_t nrows, const int32_t *rec, int64_t nrec, const int32_t *e,
                            int32_t *pos, int32_t *scratch, int2 *out, cudaStream_t s)
{
  if(nrows <= 0) return;
  if(nrec > 0) k_bwd_mark<<<grid_for(nrec), kBlock, 0, s>>>(rec, nrec, e[0], e[1], e[2], e[3], e[4], pos, nrows);
  xscan(pos, nrows + 1, scratch, s);
  k_bwd_gather<<<grid_for(nrows), kBlock, 0, s>>>(col, pos, nrows, out);
}

void launch_fill_lists(const int4 *rec, long long nrec, const ListBuild &lb, int32_t *off, int64_t nrows_total,
                       int2 *ent, int64_t ent_cap, int32_t *scratch, unsigned int *err, cudaStream_t s)
{
  if(nrec <= 0 || nrows_total <= 0) return;
  // the counts of row r are at off[r + 1]; their exclusive scan makes off[r + 1]
  // the start of row r, which the fill's cursor adds carry to the start of
  // row r + 1, with off[0] = 0
  int32_t *cnt = off + 1;
  xscan(cnt, nrows_total, scratch, s);
  k_list_fill<<<grid_for(nrec), kBlock, 0, s>>>(rec, nrec, lb, cnt, ent, ent_cap, err);
}

void launch_scatter_childmap(const int2 *pairs, int32_t n, int32_t *childmap, int32_t *cursor, int32_t ncursor,
                             cudaStream_t s)
{
  const int32_t m = n > ncursor ? n : ncursor;
  if(m <= 0) return;
  k_scatter_childmap<<<grid_for(m), kBlock, 0, s>>>(pairs, n, childmap, cursor, ncursor);
}

void launch_support(const NodeDesc *nodes, int32_t nnodes, int32_t total_keys, const uint32_t *bm, int32_t *bmx,
                    int32_t *support, cudaStream_t s)
{
  if(total_keys <= 0) return;
  k_support<<<grid_for((long long)total_keys * 32), kBlock, 0, s>>>(nodes, nnodes, total_keys, bm, bmx, support);
}

}  // namespace gsgb
