// Canonicality (minimum DFS code) check on the GPU: one warp per frequent
// candidate of a wave, run right after support selection so that only the
// verdicts travel back to the host with the candidate list.
//
// Semantics are those of the sequential reference's gSpan::is_min
// (src/gspan/ismin.cpp:36-143), the same as the host MinChecker
// (gs_dfs.cpp): rebuild the minimum DFS code of the candidate's pattern
// greedily, one edge per step, keeping every embedding of the partial
// minimum code in the pattern, and compare each new edge with the
// candidate's edge at the same position (from the second edge on).
//
// Warp-parallel form.  The pattern (at most 32 vertices and 64 edges here)
// lives in shared memory as an adjacency list in code order.  The lanes split
// the embeddings of the partial minimum code; each step takes the
// lexicographic minimum of the lanes' best extensions with one warp
// reduction (backward: by edge label; forward: by (edge label, to label)
// packed into one integer), and the embeddings of the chosen edge are
// appended to the other buffer with warp-aggregated positions.  An
// embedding records only its vertex map and used-vertex / used-edge bit
// sets: the labels of the minimum code's edges are the minimum code's own.
// A candidate whose pattern is larger, or whose embeddings outgrow the
// buffer, is left to the host checker (verdict 2).
#include "gs_kernels.hpp"

namespace gsgb {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kMinWarps = 4;
constexpr int kMinV = 32;     // pattern vertices checked on the GPU
constexpr int kMinE = 64;     // pattern edges checked on the GPU
constexpr int kMinCap = 128;  // embeddings per buffer

struct MEmb {
  uint8_t map[kMinV];  // minimum-code vertex -> pattern vertex
  uint32_t vmask;      // pattern vertices used
  uint32_t pad;
  uint64_t emask;      // pattern edges used
};

struct MinSmem {
  MEmb buf[2][kMinCap];
  uint32_t adj[2 * kMinE];  // (edge label << 16) | (edge id << 8) | neighbour
  int32_t aoff[kMinV + 1];
  int32_t vlab[kMinV];
  // the candidate code, sequential-reference style: to label -1 for backward edges
  int32_t cf[kMinE], ct[kMinE], cel[kMinE], ctl[kMinE];
  // the minimum code built so far
  int32_t mf[kMinE], mt[kMinE], mel[kMinE];
  int32_t rm[kMinE];
  int32_t nrm;
  int32_t ncur;
  int32_t nnext;
};

__device__ __forceinline__ unsigned lanemask_lt()
{
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ int node_of_key(const NodeDesc *nodes, int n, int key)
{
  int lo = 0, hi = n - 1;
  while(lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if(nodes[mid].key_base <= key) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// appends a copy of `src` (extended as given) to the next buffer; the warp
// calls it converged, `take` says which lanes append.  Returns false if the
// buffer overflowed.
__device__ __forceinline__ bool append(MinSmem &S, int nb, bool take, const MEmb &src, int newv, int pv, int eid,
                                       int lane)
{
  const unsigned m = __ballot_sync(kFull, take);
  const int base = S.nnext;
  const int pos = base + __popc(m & lanemask_lt());
  if(take && pos < kMinCap) {
    MEmb &d = S.buf[nb][pos];
    d = src;
    if(newv >= 0) {
      d.map[newv] = (uint8_t)pv;
      d.vmask |= 1u << pv;
    }
    d.emask |= 1ull << eid;
  }
  __syncwarp();
  if(lane == 0) S.nnext = base + __popc(m);
  __syncwarp();
  return base + __popc(m) <= kMinCap;
}

// 1 minimal, 0 not minimal, 2 left to the host
__device__ int warp_is_min(MinSmem &S, int n, int lane)
{
  // ---- pattern graph: labels and adjacency in code order
  int nv = 0;
  for(int i = 0; i < n; i++) nv = max(nv, max(S.cf[i], S.ct[i]) + 1);
  if(nv > kMinV) return 2;
  if(lane == 0) {
    for(int v = 0; v <= nv; v++) S.aoff[v] = 0;
    for(int i = 0; i < n; i++) {
      S.aoff[S.cf[i] + 1]++;
      S.aoff[S.ct[i] + 1]++;
    }
    for(int v = 0; v < nv; v++) S.aoff[v + 1] += S.aoff[v];
    int fill[kMinV];
    for(int v = 0; v < nv; v++) fill[v] = S.aoff[v];
    for(int i = 0; i < n; i++) {
      const uint32_t e = ((uint32_t)S.cel[i] << 16) | ((uint32_t)i << 8);
      S.adj[fill[S.cf[i]]++] = e | (uint32_t)S.ct[i];
      S.adj[fill[S.ct[i]]++] = e | (uint32_t)S.cf[i];
    }
  }
  __syncwarp();
  const int na = 2 * n;
  int maxdeg = 0;
  for(int v = 0; v < nv; v++) maxdeg = max(maxdeg, S.aoff[v + 1] - S.aoff[v]);

  // ---- first edge: minimum (from label, edge label, to label) with from label <= to label
  unsigned long long best = ~0ull;
  for(int t = lane; t < na; t += 32) {
    int v = 0;
    while(S.aoff[v + 1] <= t) v++;
    const uint32_t a = S.adj[t];
    const int to = a & 0xff, el = a >> 16;
    if(S.vlab[v] > S.vlab[to]) continue;
    const unsigned long long k = ((unsigned long long)S.vlab[v] << 32) | ((unsigned long long)el << 16) | S.vlab[to];
    best = min(best, k);
  }
  for(int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(kFull, best, o));
  if(best == ~0ull) return 2;
  const int b0 = (int)(best >> 32), b1 = (int)((best >> 16) & 0xffff), b2 = (int)(best & 0xffff);
  if(lane == 0) S.nnext = 0;
  __syncwarp();
  for(int t0 = 0; t0 < na; t0 += 32) {
    const int t = t0 + lane;
    bool take = false;
    int v = 0, to = 0, id = 0;
    if(t < na) {
      while(S.aoff[v + 1] <= t) v++;
      const uint32_t a = S.adj[t];
      to = a & 0xff;
      id = (a >> 8) & 0xff;
      take = S.vlab[v] <= S.vlab[to] && S.vlab[v] == b0 && (int)(a >> 16) == b1 && S.vlab[to] == b2;
    }
    MEmb e;
    e.map[0] = (uint8_t)v;
    e.vmask = 1u << v;
    e.pad = 0;
    e.emask = 0;
    if(!append(S, 0, take, e, 1, to, id, lane)) return 2;
  }
  if(lane == 0) {
    S.ncur = S.nnext;
    S.mf[0] = 0;
    S.mt[0] = 1;
    S.mel[0] = b1;
  }
  __syncwarp();
  const int minlabel = b0;
  int cb = 0;  // the buffer holding the current embeddings

  for(int m = 1;; m++) {
    // every pattern edge is in the minimum code
    if(m >= n) return 1;
    if(lane == 0) {
      // right-most path of the minimum code (forward edges, deepest first)
      int cnt = 0, old_from = -1;
      for(int i = m - 1; i >= 0; i--)
        if(S.mf[i] < S.mt[i] && (cnt == 0 || old_from == S.mt[i])) {
          S.rm[cnt++] = i;
          old_from = S.mf[i];
        }
      S.nrm = cnt;
      S.nnext = 0;
    }
    __syncwarp();
    const int nrm = S.nrm, ncur = S.ncur;
    const int maxtoc = S.mt[S.rm[0]];
    const MEmb *cur = S.buf[cb];

    // ---- backward edges from the right-most vertex: the right-most-path
    // index nearest the root with any wins; per embedding the first matching
    // adjacency entry counts (get_backward)
    int found = -1, bel = 0;
    for(int i = nrm - 1; i >= 1 && found < 0; --i) {
      const int v1f = S.mf[S.rm[i]], v1t = S.mt[S.rm[i]], e1el = S.mel[S.rm[i]];
      unsigned lb = 0xffffffffu;
      for(int j = lane; j < ncur; j += 32) {
        const MEmb &e = cur[j];
        const int r = e.map[maxtoc], e1from = e.map[v1f], e1to = e.map[v1t];
        for(int t = S.aoff[r]; t < S.aoff[r + 1]; t++) {
          const uint32_t a = S.adj[t];
          const int to = a & 0xff, id = (a >> 8) & 0xff, el = a >> 16;
          if((e.emask >> id) & 1ull) continue;
          if(to == e1from && (e1el < el || (e1el == el && S.vlab[e1to] <= S.vlab[r]))) {
            lb = min(lb, (unsigned)el);
            break;
          }
        }
      }
      lb = __reduce_min_sync(kFull, lb);
      if(lb != 0xffffffffu) {
        found = i;
        bel = (int)lb;
      }
    }
    if(found >= 0) {
      const int v1f = S.mf[S.rm[found]], v1t = S.mt[S.rm[found]], e1el = S.mel[S.rm[found]];
      for(int j0 = 0; j0 < ncur; j0 += 32) {
        const int j = j0 + lane;
        bool take = false;
        int id = 0;
        MEmb e;
        if(j < ncur) {
          e = cur[j];
          const int r = e.map[maxtoc], e1from = e.map[v1f], e1to = e.map[v1t];
          for(int t = S.aoff[r]; t < S.aoff[r + 1]; t++) {
            const uint32_t a = S.adj[t];
            const int to = a & 0xff, aid = (a >> 8) & 0xff, el = a >> 16;
            if((e.emask >> aid) & 1ull) continue;
            if(to == e1from && (e1el < el || (e1el == el && S.vlab[e1to] <= S.vlab[r]))) {
              take = el == bel;
              id = aid;
              break;
            }
          }
        }
        if(!append(S, cb ^ 1, take, e, -1, 0, id, lane)) return 2;
      }
      const int nf = maxtoc, nt = S.mf[S.rm[found]];
      if(S.cf[m] != nf || S.ct[m] != nt || S.cel[m] != bel || S.ctl[m] != -1) return 0;
      if(lane == 0) {
        S.mf[m] = nf;
        S.mt[m] = nt;
        S.mel[m] = bel;
        S.ncur = S.nnext;
      }
      cb ^= 1;
      __syncwarp();
      continue;
    }

    // ---- forward: pure from the right-most vertex, else from the right-most
    // path, deepest first; minimum (edge label, to label)
    if(maxtoc + 1 >= kMinV) return 2;
    int which = -2;
    unsigned fb = 0xffffffffu;
    {
      unsigned lb = 0xffffffffu;
      for(int j = lane; j < ncur; j += 32) {
        const MEmb &e = cur[j];
        const int r = e.map[maxtoc];
        for(int t = S.aoff[r]; t < S.aoff[r + 1]; t++) {
          const uint32_t a = S.adj[t];
          const int to = a & 0xff, el = a >> 16;
          if(minlabel > S.vlab[to] || ((e.vmask >> to) & 1u)) continue;
          lb = min(lb, ((unsigned)el << 16) | (unsigned)S.vlab[to]);
        }
      }
      lb = __reduce_min_sync(kFull, lb);
      if(lb != 0xffffffffu) {
        which = -1;
        fb = lb;
      }
    }
    for(int i = 0; which == -2 && i < nrm; ++i) {
      const int vf = S.mf[S.rm[i]], vt = S.mt[S.rm[i]], eel = S.mel[S.rm[i]];
      unsigned lb = 0xffffffffu;
      for(int j = lane; j < ncur; j += 32) {
        const MEmb &e = cur[j];
        const int efrom = e.map[vf], eto = e.map[vt], tolabel = S.vlab[eto];
        for(int t = S.aoff[efrom]; t < S.aoff[efrom + 1]; t++) {
          const uint32_t a = S.adj[t];
          const int to = a & 0xff, el = a >> 16, tl2 = S.vlab[to];
          if(eto == to || minlabel > tl2 || ((e.vmask >> to) & 1u)) continue;
          if(eel < el || (eel == el && tolabel <= tl2)) lb = min(lb, ((unsigned)el << 16) | (unsigned)tl2);
        }
      }
      lb = __reduce_min_sync(kFull, lb);
      if(lb != 0xffffffffu) {
        which = i;
        fb = lb;
      }
    }
    if(which == -2) return 1;
    const int fel = (int)(fb >> 16), ftl = (int)(fb & 0xffff);
    const int vf = which == -1 ? maxtoc : S.mf[S.rm[which]];
    const int vt = which == -1 ? -1 : S.mt[S.rm[which]];
    const int eel = which == -1 ? 0 : S.mel[S.rm[which]];
    for(int j0 = 0; j0 < ncur; j0 += 32) {
      const int j = j0 + lane;
      const bool live = j < ncur;
      MEmb e;
      int x = 0, deg = 0, eto = -1, tolabel = 0;
      if(live) {
        e = cur[j];
        x = e.map[vf];
        deg = S.aoff[x + 1] - S.aoff[x];
        if(which >= 0) {
          eto = e.map[vt];
          tolabel = S.vlab[eto];
        }
      }
      for(int t = 0; t < maxdeg; t++) {
        bool take = false;
        int to = 0, id = 0;
        if(live && t < deg) {
          const uint32_t a = S.adj[S.aoff[x] + t];
          to = a & 0xff;
          id = (a >> 8) & 0xff;
          const int el = a >> 16, tl2 = S.vlab[to];
          if(!(minlabel > tl2 || ((e.vmask >> to) & 1u)) && el == fel && tl2 == ftl) {
            if(which == -1) take = true;
            else take = eto != to && (eel < el || (eel == el && tolabel <= tl2));
          }
        }
        if(!append(S, cb ^ 1, take, e, maxtoc + 1, to, id, lane)) return 2;
      }
    }
    if(S.cf[m] != vf || S.ct[m] != maxtoc + 1 || S.cel[m] != fel || S.ctl[m] != ftl) return 0;
    if(lane == 0) {
      S.mf[m] = vf;
      S.mt[m] = maxtoc + 1;
      S.mel[m] = fel;
      S.ncur = S.nnext;
    }
    cb ^= 1;
    __syncwarp();
  }
}

__global__ void __launch_bounds__(kMinWarps * 32) k_is_min(const NodeDesc *__restrict__ nodes, int nnodes,
                                                           const SlotDesc *__restrict__ slots,
                                                           const DevDB *__restrict__ dbs,
                                                           const int32_t *__restrict__ codes, int4 *sel,
                                                           int sel_cap, const unsigned long long *counters)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  MinSmem &S = reinterpret_cast<MinSmem *>(smem_raw)[warp];
  const long long nsel = min((long long)counters[0], (long long)sel_cap);
  const long long nwarps = (long long)gridDim.x * kMinWarps;
  for(long long i = (long long)blockIdx.x * kMinWarps + warp; i < nsel; i += nwarps) {
    const int4 x = sel[i];
    // the node the selection recorded, or (out of range) the search by key
    int ni = x.w >> 2;
    if(ni < 0 || ni >= nnodes || x.x < nodes[ni].key_base || x.x >= nodes[ni].key_base + nodes[ni].nkeys)
      ni = node_of_key(nodes, nnodes, x.x);
    const NodeDesc &nd = nodes[ni];
    const int len = nd.code_len, n = len + 1;
    int verdict = 2;
    if(n <= kMinE) {
      // the parent's code, then the candidate edge decoded from its key
      for(int t = lane; t < len; t += 32) {
        const int32_t *c = codes + 5 * ((long long)nd.code_off + t);
        const bool fwd = c[0] < c[1];
        S.cf[t] = c[0];
        S.ct[t] = c[1];
        S.cel[t] = c[3];
        S.ctl[t] = fwd ? c[4] : -1;
        if(t == 0) S.vlab[c[0]] = c[2];
        if(fwd && c[1] < kMinV) S.vlab[c[1]] = c[4];
      }
      const DevDB &db = dbs[nd.db];
      const int kl = x.x - nd.key_base, maxtoc = nd.k - 1;
      const SlotDesc *sl = slots + nd.slot_off;
      int f, t, el, tl;
      if(kl < nd.nfwd) {
        int s = 0;
        for(int q = 1; q < nd.nslot; q++)
          if(sl[q].fkey_off <= kl) s = q;
        const int pc = db.pair_code[db.root_off[sl[s].vlab] + (kl - sl[s].fkey_off)];
        f = sl[s].vertex;
        t = maxtoc + 1;
        el = pc >> 16;
        tl = pc & 0xffff;
      } else {
        const int b = (kl - nd.nfwd) / db.EL;
        f = maxtoc;
        t = sl[b].vertex;
        el = (kl - nd.nfwd) % db.EL;
        tl = -1;
      }
      if(lane == 0) {
        S.cf[len] = f;
        S.ct[len] = t;
        S.cel[len] = el;
        S.ctl[len] = tl;
        if(tl >= 0 && t < kMinV) S.vlab[t] = tl;
      }
      __syncwarp();
      if(nd.k + 1 <= kMinV) verdict = warp_is_min(S, n, lane);
      __syncwarp();
    }
    if(lane == 0) sel[i].w = (x.w & ~3) | verdict;
  }
}

}  // namespace

KernelCall is_min_call(const NodeDesc *nodes, int32_t nnodes, const SlotDesc *slots, const DevDB *dbs,
                       const int32_t *codes, int4 *sel, int32_t sel_cap, const unsigned long long *counters)
{
  const size_t smem = sizeof(MinSmem) * kMinWarps;
  static const bool configured = [smem] {
    cudaFuncSetAttribute(k_is_min, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return true;
  }();
  (void)configured;
  KernelCall c;
  c.func = (const void *)k_is_min;
  c.grid = dim3((unsigned)(2 * sm_count()));
  c.block = dim3(kMinWarps * 32);
  c.smem = (unsigned)smem;
  c.arg(nodes);
  c.arg(nnodes);
  c.arg(slots);
  c.arg(dbs);
  c.arg(codes);
  c.arg(sel);
  c.arg(sel_cap);
  c.arg(counters);
  return c;
}

}  // namespace gsgb
