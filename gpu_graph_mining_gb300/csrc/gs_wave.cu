// Warp-cooperative extension kernels: count (support bitmaps + embedding
// counts) and materialise (children's columns), for one wave of DFS-tree nodes.
//
// gSpan's extension rules, from the sequential reference:
//   backward  get_backward       src/globals/graph_types.cpp:389-413
//   forward   get_forward_pure   src/globals/graph_types.cpp:337-357
//             get_forward_rmpath src/globals/graph_types.cpp:305-322
//
// Work layout.  A warp owns a tile of 32 consecutive embedding rows of one
// node (tiles never span nodes, so the node's descriptor, database and
// right-most-path slots are loaded once per tile).  Phase 1, per lane: walk
// the back-links column by column (one 8-byte load per
// column, into shared memory laid out [vertex][lane] so that a warp reads a
// column without bank conflicts), and record for every right-most-path vertex
// the start of its adjacency and the running degree sum.  Phase 2, per warp:
// the tile's (row, slot, neighbour) items are numbered 0..T-1 by a warp scan
// and processed 32 at a time, every lane busy: lane -> owner row by a 5-step
// shuffle search, -> slot by the degree prefix, -> one 8-byte packed adjacency
// entry (neighbour, edge label, neighbour label).  Neighbouring items read
// neighbouring entries, so the adjacency loads coalesce.  The warp stays
// converged, so counters and child cursors are updated with one atomic per
// distinct key per step (__match_any_sync).
//
// The reference enumerates with one thread per (row, rmpath column) into a
// dense max_degree x rows x columns flag array and writes 32-byte records for
// every extension (compute_extensions.cpp:110-390).  Here the count pass
// writes only bitmap bits and counters; the materialise pass writes only the
// selected children's 8-byte column elements and 4-byte graph ranks.
#include "gs_kernels.hpp"
#include "gs_lists.cuh"

namespace gsgb {

namespace {

// Launch shape (compile-time tunables): warps per block, the minimum blocks
// per SM the register allocation must allow (0 = no constraint), and the
// grid cap in blocks per SM (warps loop over tiles beyond it).
#ifndef GS_WAVE_WARPS
#define GS_WAVE_WARPS 4
#endif
#ifndef GS_WAVE_MINB
#define GS_WAVE_MINB 9
#endif
#ifndef GS_WAVE_GRID
#define GS_WAVE_GRID 64
#endif
constexpr int kWarps = GS_WAVE_WARPS;
constexpr unsigned kFull = 0xffffffffu;
#ifndef GS_REC_CHUNK
#define GS_REC_CHUNK 128
#endif
constexpr int kRecChunk = GS_REC_CHUNK;  // records a warp reserves at a time

struct WaveArgs {
  const NodeDesc *nodes;
  int nnodes;
  long long total_tiles;  // sum over nodes of ceil(rows / 32)
  const int2 *const *coltab;
  const int32_t *collen;
  const SlotDesc *slots;
  const int32_t *vtab;
  const DevDB *dbs;
  uint32_t *bm;          // count: bitmaps to set; materialise: read
  const int32_t *bmx;    // materialise: prefix popcounts
  int32_t *cnt;          // count: embeddings per key
  const int32_t *childmap;
  int32_t *cursor;
  const ChildOut *outs;
  unsigned long long *bytes;
  unsigned int *err;
  // count pass, optional: one record per extension {wave key, child column
  // element x, y, graph rank} for the record-driven materialise pass
  int4 *rec;
  long long rec_cap;
  unsigned long long *rec_n;  // records produced (may exceed rec_cap: then none past it are written)
  // count pass: cnt holds cnt_copies copies of the wave's counters, cnt_stride
  // apart; warp w adds into copy w % cnt_copies (summed by the screening pass)
  int cnt_copies;
  long long cnt_stride;
  int rule_skip;  // bisect past forward-rule prefixes of sorted adjacency lists
};

template <int KMAX> struct Smem {
  unsigned long long mask[32];  // small graphs: the row's graph-local vertex ids as a bit set
  int gb[32];                   // small graphs: first global vertex of the row's graph
  int lp[32];                   // the row's last column back-link (a backward child's element)
  unsigned long long bytes;     // the warp's algorithmic bytes (lane 0 adds, once per tile)
  int phi[KMAX][32];        // graph vertex of pattern vertex t for lane l
  int start[KMAX][32];      // scanned position p: adjacency (or parent list) start
  int pre[KMAX + 1][32];    // item prefix over the scanned positions
  SlotDesc slot[KMAX];      // the tile's node: right-most-path slots
  int join_lo, join_key, join_hi;  // the tile's node: join rule (lists strategy)
  int vtab[KMAX];           // the tile's node: pattern vertex -> backward slot
  const int2 *col[KMAX];    // the tile's node: its columns and their lengths,
  int clen[KMAX];           // loaded once so the walk's chain is one load per column
};

__device__ __forceinline__ unsigned lanemask_lt()
{
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// MASK: every graph of the wave's databases has at most 64 vertices, so
// "is w already in the embedding" is one bit test of the row's vertex set
// instead of a loop over its k vertices.  JOIN: some node of the wave joins
// its parent's per-row lists (lists strategy); without it the join code is
// compiled out.
template <int KMAX, bool MAT, bool MASK, bool JOIN>
__global__ void
#if GS_WAVE_MINB > 0
__launch_bounds__(kWarps * 32, GS_WAVE_MINB)
#else
__launch_bounds__(kWarps * 32)
#endif
k_wave(const WaveArgs a)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Smem<KMAX> &S = reinterpret_cast<Smem<KMAX> *>(smem_raw)[warp];
  const long long gwarp = (long long)blockIdx.x * kWarps + warp;
  const long long nwarps = (long long)gridDim.x * kWarps;
  if(lane == 0) S.bytes = 0;
  // count pass with records: the warp's current reserved chunk (warp-uniform);
  // starts "full" so the first batch reserves a chunk
  long long chunk_base = -1;
  int chunk_fill = kRecChunk;
  const int copy = (int)(gwarp % (a.cnt_copies > 0 ? a.cnt_copies : 1));
  int32_t *const cnt_copy = MAT ? nullptr : a.cnt + copy * a.cnt_stride;
  // records carry the copy their embedding was counted in (bits 27-30 of the
  // key field): the materialise pass places it in that copy's share of the
  // child column
  const int rec_tag = copy << kRecCopyShift;

  for(long long tile = gwarp; tile < a.total_tiles; tile += nwarps) {
    // ---- the tile's node (warp-uniform: tiles never span nodes): a 32-way
    // search, the lanes probing 32 nodes per round (3 rounds for 4096 nodes)
    int lo = 0, hi = a.nnodes;  // the node is the last in [lo, hi) with tile_begin <= tile
    while(hi - lo > 1) {
      const int step = (hi - lo + 31) >> 5;
      const int probe = lo + lane * step;
      const unsigned ok = __ballot_sync(kFull, probe < hi && a.nodes[probe].tile_begin <= tile);
      lo += (31 - __clz(ok | 1u)) * step;
      hi = min(hi, lo + step);
    }
    const int n = lo;
    const NodeDesc &nd = a.nodes[n];
    const int k = nd.k, nslot = nd.nslot, minlabel = nd.minlabel, words = nd.words, key_base = nd.key_base;
    const long long bm_base = nd.bm_base;
    const DevDB &dbr = a.dbs[nd.db];
    const unsigned long long *__restrict__ adj = dbr.adj;
    const int32_t *__restrict__ adj_off = dbr.adj_off;
    const int32_t *__restrict__ adj_pair = dbr.adj_pair;
    // The forward key needs the entry's pair index.  When the wave's
    // adjacency is larger than L2 (no rule skip), the per-entry pair array is
    // a second random DRAM access per entry (a 32-byte sector for 4 useful
    // bytes); a small label alphabet's pair table (VL * EL * VL entries) stays
    // in L1 instead, looked up from the entry's labels for the entries that
    // become forward extensions.  On configuration 5 this cut the kernel's
    // DRAM traffic from 1.62 to 1.17 times its algorithmic bytes.
    const int32_t *__restrict__ ptab =
        !JOIN && !a.rule_skip && (long long)dbr.VL * dbr.EL * dbr.VL <= 16384 ? dbr.pair_idx : nullptr;
    const int pEL = dbr.EL, pVL = dbr.VL;
    const int nv = dbr.n_vertices;
    if(k > KMAX || nslot > KMAX || k < 1 || nslot < 1) {
      if(lane == 0) atomicOr(a.err, 2u);
      continue;
    }
    // scanned positions: slots s0..nslot-1 (adjacency), then with a join the
    // parent's list of the row (lists strategy: s0 = the right-most vertex)
    const bool join = JOIN && nd.csr_off != nullptr;
    if(join && nslot < 2) {
      if(lane == 0) atomicOr(a.err, 2u);
      continue;
    }
    const int s0 = join ? nslot - 1 : 0;
    const int np = nslot - s0 + (join ? 1 : 0);
    // the node's tables, strided over the lanes (patterns of up to KMAX = 64
    // vertices have more columns and slots than a warp has lanes)
    for(int t = lane; t < nslot; t += 32) S.slot[t] = a.slots[nd.slot_off + t];
    if(join && lane == 0) {
      S.join_lo = nd.join_lo;
      S.join_key = nd.join_key;
      S.join_hi = nd.join_hi;
    }
    for(int t = lane; t < k; t += 32) {
      S.vtab[t] = a.vtab[nd.vtab_off + t];
      S.col[t] = a.coltab[nd.col_off + t];
      S.clen[t] = a.collen[nd.col_off + t];
    }
    // ---- phase 1: this lane's row
    // the tile's first row within the node (kept in a register: the emission
    // below stores to global memory, so a reload from the node would not be
    // hoisted out of the item loop)
    const int row0 = (int)((tile - nd.tile_begin) * 32);
    const int i = row0 + lane;
    bool valid = i < nd.nrows;
    int W = 0, g = 0, last_prev = 0;
    // the graph rank is loaded now and checked after the walk, so that the
    // walk's loads do not wait for it
    if(valid) g = __ldg(&nd.gord[i]);
    __syncwarp();
    if(valid) {
      int idx = i;
      for(int c = k - 1; c >= 0; --c) {
        if((unsigned)idx >= (unsigned)S.clen[c]) { valid = false; break; }
        const int2 e = __ldg(&S.col[c][idx]);
        if((unsigned)e.x >= (unsigned)nv) { valid = false; break; }
        S.phi[c][lane] = e.x;
        if(c == k - 1) {
          last_prev = e.y;
          S.lp[lane] = e.y;
        }
        idx = e.y;
      }
      if(!valid) atomicOr(a.err, 2u);
    }
    if(valid && (unsigned)g >= (unsigned)words * 32u) {
      atomicOr(a.err, 1u);
      valid = false;
    }
    if(MASK && valid) {
      const int gb = __ldg(&dbr.vgbase[S.phi[0][lane]]);
      unsigned long long m = 0;
      for(int c = 0; c < k; ++c) {
        const unsigned lv = (unsigned)(S.phi[c][lane] - gb);
        if(lv >= 64u) { valid = false; break; }
        m |= 1ull << lv;
      }
      if(!valid) atomicOr(a.err, 2u);
      S.mask[lane] = m;
      S.gb[lane] = gb;
    }
    if(valid && join && (unsigned)last_prev >= (unsigned)nd.csr_rows) {
      atomicOr(a.err, 2u);
      valid = false;
    }
    if(valid) {
      const bool sorted = a.rule_skip && dbr.adj_sorted != 0;
      for(int s = s0; s < nslot; ++s) {
        const int v = S.phi[S.slot[s].vertex][lane];
        int a0 = __ldg(&adj_off[v]);
        const int a1 = __ldg(&adj_off[v + 1]);
        const int fr = S.slot[s].frule;
        if(sorted && fr != INT32_MIN) {
          // a vertex of the right-most path below its end extends forward
          // only by entries at or above its rule; in an ascending list the
          // rest is a prefix, found by bisection and not scanned
          int lo = a0, hi = a1;
          while(lo < hi) {
            const int mid = (int)(((unsigned)lo + (unsigned)hi) >> 1);
            if((int)(__ldg(&adj[mid]) >> 32) < fr) lo = mid + 1;
            else hi = mid;
          }
          a0 = lo;
        }
        S.start[s - s0][lane] = a0;
        S.pre[s - s0][lane] = W;
        W += a1 - a0;
      }
      if(join) {
        // the parent row's list (the last column's back-link is the parent row)
        const int c0 = __ldg(&nd.csr_off[last_prev]), c1 = __ldg(&nd.csr_off[last_prev + 1]);
        S.start[np - 1][lane] = c0;
        S.pre[np - 1][lane] = W;
        W += c1 - c0;
      }
      S.pre[np][lane] = W;
    }
    __syncwarp();
    // ---- phase 2: the tile's (row, slot, neighbour) items, 32 at a time
    int incl = W;
    for(int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(kFull, incl, o);
      if(lane >= o) incl += t;
    }
    const int off = incl - W;
    const int T = __shfl_sync(kFull, incl, 31);
    // per valid row: its k column elements, graph rank, scanned offsets and bit
    // set; per item one packed adjacency entry (or list entry)
    {
      const unsigned nvalid = __popc(__ballot_sync(kFull, valid));
      if(lane == 0) S.bytes += (8ull * k + 4 + 8ull * np + (MASK ? 8 : 0)) * nvalid + 8ull * T;
    }
    // Items are located and their adjacency entries (and pair indices) loaded
    // one batch ahead: the next batch's loads are in flight while this batch
    // is decided and emitted.
    int o_n = 0, s_n = 0;
    bool has_n = false;
    unsigned long long ent_n = 0;
    int pr_n = 0;
    auto locate = [&](int j) {
      // owner lane: the largest o with off_o <= j (it has W_o > 0)
      int o = 0;
#pragma unroll
      for(int step = 16; step >= 1; step >>= 1) {
        const int c = o + step;
        const int oc = __shfl_sync(kFull, off, c);
        if(oc <= j) o = c;
      }
      const int q = j - __shfl_sync(kFull, off, o);
      o_n = o;
      s_n = 0;
      has_n = j < T;
      if(has_n) {
        int sl = 0;
        while(S.pre[sl + 1][o] <= q) sl++;
        const int e = S.start[sl][o] + (q - S.pre[sl][o]);
        if(join && sl == np - 1) {
          // a parent list entry {neighbour, parent's forward key}
          const int2 je = __ldg(&nd.csr_ent[e]);
          s_n = -1;
          ent_n = ((unsigned long long)(unsigned)je.y << 32) | (unsigned)je.x;
        } else {
          s_n = s0 + sl;
          ent_n = __ldg(&adj[e]);
          if(!ptab) pr_n = __ldg(&adj_pair[e]);
        }
      }
    };
    if(T > 0) locate(lane);
    for(int base = 0; base < T; base += 32) {
      const int o = o_n, s = s_n;
      const bool has = has_n;
      const unsigned long long ent = ent_n;
      const int pr = pr_n;
      if(base + 32 < T) locate(base + 32 + lane);  // warp-uniform condition
      const int g_o = __shfl_sync(kFull, g, o);
      int key = -1, w = 0;
      bool bwd = false;
      if(JOIN && has && s < 0) {
        // lists strategy: the parent's frequent forward extension, still one
        // of this node's if its source is on this node's right-most path
        // (key below join_hi), its (edge label, target label) is allowed from
        // there (from u: at or after the new edge's, keys follow that order),
        // and its target is not the node's new vertex
        w = (int)(unsigned)(ent & 0xffffffffull);
        const int lk = (int)(ent >> 32);
        if(lk < S.join_hi && (lk < S.join_lo || lk >= S.join_key) && w != S.phi[k - 1][o]) key = lk;
      } else if(has) {
        const int frule = S.slot[s].frule, fko = S.slot[s].fkey_off;
        w = (int)(unsigned)(ent & 0xffffffffull);
        const int hi = (int)(ent >> 32);  // (edge label << 16) | neighbour label
        const int wl = hi & 0xffff;
        const bool is_r = (s == nslot - 1);
        // forward: label >= minlabel and the right-most-path order rule (one
        // compare, INT32_MIN for the right-most vertex); needs a new vertex
        const bool fwd_rules = wl >= minlabel && hi >= frule;
        bool in_emb = false;
        if(MASK) {
          const unsigned lv = (unsigned)(w - S.gb[o]);
          in_emb = lv < 64u && ((S.mask[o] >> lv) & 1ull);
        } else if(fwd_rules || is_r) {
          for(int t = 0; t < k; ++t) in_emb |= (S.phi[t][o] == w);
        }
        if(fwd_rules && !in_emb) {
          key = fko + (ptab ? __ldg(&ptab[(S.slot[s].vlab * pEL + (hi >> 16)) * pVL + wl]) : pr);
        } else if(is_r && in_emb) {
          // backward edge from the right-most vertex to a right-most-path vertex
          int jv = -1;
          for(int t = 0; t < k; ++t) if(S.phi[t][o] == w) jv = t;
          const int bs = jv >= 0 ? S.vtab[jv] : -1;
          const int el = hi >> 16;
          if(bs >= 0 && el >= S.slot[bs].bmin) {
            key = S.slot[bs].bkey_off + el;
            bwd = true;
          }
        }
      }
      // ---- emission, warp converged
      if(!MAT) {
        // one counter add per distinct key of the step, into this warp's copy
        // of the counters (copies spread a node's hot counters over L2 slices);
        // one bitmap OR per distinct key unless a lane's graph differs from its
        // key group leader's (a tile's rows mostly share a graph).  The bytes of
        // the bitmap word, the counter and the record per extension are added
        // on the host from the wave's extension total.
        const unsigned peers = __match_any_sync(kFull, key);
        const int leader = __ffs(peers) - 1;
        const int g_lead = __shfl_sync(kFull, g_o, leader);
        if(key >= 0 && (lane == leader || g_o != g_lead))
          atomicOr(&a.bm[bm_base + (long long)key * words + (g_o >> 5)], 1u << (g_o & 31));
        if(key >= 0 && lane == leader) atomicAdd(&cnt_copy[key_base + key], __popc(peers));
        const unsigned ext = __ballot_sync(kFull, key >= 0);  // every lane takes part
        if(a.rec && ext) {
          // append this step's extensions to the warp's current chunk of
          // kRecChunk records; a batch that does not fit is split across a
          // freshly reserved chunk (one global atomic per chunk, not per step)
          const int cntx = __popc(ext);
          const int rank = __popc(ext & lanemask_lt());
          long long dst = -1;
          if(chunk_fill + cntx <= kRecChunk) {
            dst = chunk_base + chunk_fill + rank;
            chunk_fill += cntx;
          } else {
            const int room = kRecChunk - chunk_fill;
            long long nb = 0;
            if(lane == 0) nb = (long long)atomicAdd(a.rec_n, (unsigned long long)kRecChunk);
            nb = __shfl_sync(kFull, nb, 0);
            dst = rank < room ? chunk_base + chunk_fill + rank : nb + (rank - room);
            chunk_base = nb;
            chunk_fill = cntx - room;
          }
          if(key >= 0 && dst >= 0 && dst < a.rec_cap) {
            const int i_o = row0 + o;
            a.rec[dst] = bwd ? make_int4((key_base + key) | rec_tag, S.phi[k - 1][o], S.lp[o], g_o)
                             : make_int4((key_base + key) | rec_tag, w, i_o, g_o);
          }
        }
      } else {
        const int c = key >= 0 ? a.childmap[key_base + key] : -1;
        const unsigned ext = __ballot_sync(kFull, key >= 0), sel = __ballot_sync(kFull, c >= 0);
        if(lane == 0) S.bytes += 4ull * __popc(ext) + 20ull * __popc(sel);
        const unsigned peers = __match_any_sync(kFull, c);
        const int leader = __ffs(peers) - 1;
        int pos = 0;
        if(c >= 0 && lane == leader) pos = atomicAdd(&a.cursor[c], __popc(peers));
        pos = __shfl_sync(kFull, pos, leader) + __popc(peers & lanemask_lt());
        if(c >= 0) {
          const long long wi = bm_base + (long long)key * words + (g_o >> 5);
          const int rank = a.bmx[wi] + __popc(a.bm[wi] & ((1u << (g_o & 31)) - 1u));
          const ChildOut out = a.outs[c];
          if(pos < out.cap) {
            const int i_o = row0 + o;
            out.col[pos] = bwd ? make_int2(S.phi[k - 1][o], S.lp[o]) : make_int2(w, i_o);
            out.gord[pos] = rank;
          } else {
            atomicOr(a.err, 4u);
          }
        }
      }
    }
    __syncwarp();
  }
  if(!MAT && a.rec && chunk_base >= 0) {
    // mark the unused tail of the last chunk as holes (key -1)
    for(int f = chunk_fill + lane; f < kRecChunk; f += 32) {
      const long long dst = chunk_base + f;
      if(dst < a.rec_cap) a.rec[dst] = make_int4(-1, 0, 0, 0);
    }
  }
  __syncwarp();
  if(a.bytes && lane == 0 && S.bytes) atomicAdd(a.bytes, S.bytes);
}

template <int KMAX, bool MAT, bool MASK, bool JOIN> void launch_k(const WaveArgs &a, cudaStream_t s)
{
  const size_t smem = sizeof(Smem<KMAX>) * kWarps;
  // once per instance (a thread-safe static: schedulers may launch from several threads)
  static const bool configured = [smem] {
    cudaFuncSetAttribute(k_wave<KMAX, MAT, MASK, JOIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return true;
  }();
  (void)configured;
  long long blocks = (a.total_tiles + kWarps - 1) / kWarps;
  const long long cap = (long long)sm_count() * GS_WAVE_GRID;
  if(blocks > cap) blocks = cap;
  if(blocks < 1) blocks = 1;
  k_wave<KMAX, MAT, MASK, JOIN><<<(int)blocks, kWarps * 32, smem, s>>>(a);
}

template <bool MAT, bool MASK, bool JOIN> void dispatch_k(int kmax, const WaveArgs &a, cudaStream_t s)
{
  if(kmax <= 8) launch_k<8, MAT, MASK, JOIN>(a, s);
  else if(kmax <= 16) launch_k<16, MAT, MASK, JOIN>(a, s);
  else if(kmax <= 32) launch_k<32, MAT, MASK, JOIN>(a, s);
  else launch_k<64, MAT, MASK, JOIN>(a, s);
}

template <bool MAT> void dispatch(int kmax, bool small_graphs, bool join, const WaveArgs &a, cudaStream_t s)
{
  if(small_graphs) {
    if(join) dispatch_k<MAT, true, true>(kmax, a, s);
    else dispatch_k<MAT, true, false>(kmax, a, s);
  } else {
    if(join) dispatch_k<MAT, false, true>(kmax, a, s);
    else dispatch_k<MAT, false, false>(kmax, a, s);
  }
}

template <int KMAX, bool MASK, bool JOIN> KernelCall count_call_k(const WaveArgs &a, int grid_per_sm)
{
  const size_t smem = sizeof(Smem<KMAX>) * kWarps;
  static const bool configured = [smem] {
    cudaFuncSetAttribute(k_wave<KMAX, false, MASK, JOIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return true;
  }();
  (void)configured;
  long long blocks = (a.total_tiles + kWarps - 1) / kWarps;
  const long long cap = (long long)sm_count() * (grid_per_sm > 0 ? grid_per_sm : GS_WAVE_GRID);
  if(blocks > cap) blocks = cap;
  if(blocks < 1) blocks = 1;
  KernelCall c;
  c.func = (const void *)k_wave<KMAX, false, MASK, JOIN>;
  c.grid = dim3((unsigned)blocks);
  c.block = dim3(kWarps * 32);
  c.smem = (unsigned)smem;
  c.arg(a);
  return c;
}

template <bool MASK, bool JOIN> KernelCall count_call(int kmax, const WaveArgs &a, int grid_per_sm)
{
  if(kmax <= 8) return count_call_k<8, MASK, JOIN>(a, grid_per_sm);
  if(kmax <= 16) return count_call_k<16, MASK, JOIN>(a, grid_per_sm);
  if(kmax <= 32) return count_call_k<32, MASK, JOIN>(a, grid_per_sm);
  return count_call_k<64, MASK, JOIN>(a, grid_per_sm);
}

}  // namespace

KernelCall wave_count_call(const NodeDesc *nodes, int32_t nnodes, long long total_tiles, int32_t kmax,
                           bool small_graphs, const int2 *const *coltab, const int32_t *collen, const SlotDesc *slots,
                           const int32_t *vtab, const DevDB *dbs, uint32_t *bm, int32_t *cnt,
                           unsigned long long *bytes, unsigned int *err, int4 *rec, long long rec_cap,
                           unsigned long long *rec_n, int32_t grid_per_sm, int32_t cnt_copies,
                           long long cnt_stride, bool join, bool rule_skip)
{
  WaveArgs a{ nodes, nnodes, total_tiles, coltab, collen, slots, vtab, dbs, bm, nullptr, cnt,
              nullptr, nullptr, nullptr, bytes, err, rec, rec_cap, rec_n, cnt_copies, cnt_stride,
              rule_skip ? 1 : 0 };
  if(small_graphs)
    return join ? count_call<true, true>(kmax, a, grid_per_sm) : count_call<true, false>(kmax, a, grid_per_sm);
  return join ? count_call<false, true>(kmax, a, grid_per_sm) : count_call<false, false>(kmax, a, grid_per_sm);
}

void launch_wave_materialize(const NodeDesc *nodes, int32_t nnodes, long long total_tiles, int32_t kmax,
                             bool small_graphs,
                             const int2 *const *coltab, const int32_t *collen, const SlotDesc *slots,
                             const int32_t *vtab, const DevDB *dbs, const uint32_t *bm, const int32_t *bmx,
                             const int32_t *childmap, int32_t *cursor, const ChildOut *outs,
                             unsigned long long *bytes, unsigned int *err, bool join, bool rule_skip,
                             cudaStream_t s)
{
  if(total_tiles <= 0) return;
  WaveArgs a{ nodes, nnodes, total_tiles, coltab, collen, slots, vtab, dbs, const_cast<uint32_t *>(bm), bmx,
              nullptr, childmap, cursor, outs, bytes, err, nullptr, 0, nullptr, 0, 0, rule_skip ? 1 : 0 };
  dispatch<true>(kmax, small_graphs, join, a, s);
}

namespace {

// Materialise from the count pass's records: one thread per record, no graph
// access.  keyword[key] = the key's first bitmap word (node bm_base + key * words).
__global__ void __launch_bounds__(256) k_mat_records(const int4 *__restrict__ rec, long long n,
                                                     const int32_t *__restrict__ childmap,
                                                     const long long *__restrict__ keyword,
                                                     const uint32_t *__restrict__ bm, const int32_t *__restrict__ bmx,
                                                     int32_t *cursor, long long cursor_stride,
                                                     const ChildOut *__restrict__ outs, unsigned long long *bytes,
                                                     unsigned int *err, const ListBuild lb, int32_t *list_cnt)
{
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  unsigned long long mine = 0;
  // the loop runs a warp-uniform number of times: lanes past n carry no record
  const long long n32 = (n + 31) & ~31ll;
  for(long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n32; r += stride) {
    int c = -1, key = 0, cp = 0;
    int4 x = make_int4(0, 0, 0, 0);
    if(r < n) {
      x = __ldg(&rec[r]);
      if(x.x >= 0) {  // key -1: an unused slot of a reserved chunk
        key = x.x & kRecKeyMask;
        cp = x.x >> kRecCopyShift;
        c = childmap[key];
      }
      mine += 20;
      long long lrow;
      int lk;
      // lists strategy: count the record's list row
      if(list_cnt && list_entry(x, lb, lrow, lk, err)) atomicAdd(&list_cnt[lrow], 1);
    }
    // the graph rank's bitmap word and prefix, and the child's outputs, are
    // loaded before the cursor add so that their latencies overlap
    uint32_t bword = 0;
    int bpre = 0;
    ChildOut out{};
    if(c >= 0) {
      const long long wi = keyword[key] + (x.w >> 5);
      bword = bm[wi];
      bpre = bmx[wi];
      out = outs[c];
    }
    // one cursor per (key, counter copy): copy q of a key starts where the
    // counts of copies 0..q-1 end, so the adds spread over many addresses
    const unsigned peers = __match_any_sync(kFull, c >= 0 ? x.x : -1);
    const int leader = __ffs(peers) - 1;
    int pos = 0;
    if(c >= 0 && lane == leader) pos = atomicAdd(&cursor[cp * cursor_stride + key], __popc(peers));
    pos = __shfl_sync(kFull, pos, leader) + __popc(peers & lanemask_lt());
    if(c >= 0) {
      const int rank = bpre + __popc(bword & ((1u << (x.w & 31)) - 1u));
      if(pos < out.cap) {
        out.col[pos] = make_int2(x.y, x.z);
        out.gord[pos] = rank;
      } else {
        atomicOr(err, 4u);
      }
      mine += 28;
    }
  }
  if(bytes) {
    for(int o = 16; o > 0; o >>= 1) mine += __shfl_down_sync(kFull, mine, o);
    if(lane == 0 && mine) atomicAdd(bytes, mine);
  }
}

}  // namespace

void launch_materialize_records(const int4 *rec, long long n, const int32_t *childmap, const long long *keyword,
                                const uint32_t *bm, const int32_t *bmx, int32_t *cursor, long long cursor_stride,
                                const ChildOut *outs, unsigned long long *bytes, unsigned int *err,
                                const ListBuild *lists, int32_t *list_cnt, cudaStream_t s)
{
  if(n <= 0) return;
  long long blocks = ((n + 31) / 32 * 32 + 255) / 256;
  if(blocks > 16LL * sm_count()) blocks = 16LL * sm_count();
  const ListBuild lb = lists ? *lists : ListBuild{ nullptr, nullptr, nullptr };
  k_mat_records<<<(int)blocks, 256, 0, s>>>(rec, n, childmap, keyword, bm, bmx, cursor, cursor_stride, outs, bytes,
                                            err, lb, lists ? list_cnt : nullptr);
}

}  // namespace gsgb
