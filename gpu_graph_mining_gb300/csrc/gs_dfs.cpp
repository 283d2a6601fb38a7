#include "gs_dfs.hpp"

#include <cstdio>

namespace gsgb {

int build_rmpath(const DFS *code, int n, int *rm)
{
  int cnt = 0, old_from = -1;
  for(int i = n - 1; i >= 0; --i) {
    if(code[i].from < code[i].to && (cnt == 0 || old_from == code[i].to)) {
      rm[cnt++] = i;
      old_from = code[i].from;
    }
  }
  return cnt;
}

void to_style(const DFS *in, int n, LabelStyle style, DFS *out)
{
  for(int i = 0; i < n; i++) {
    out[i] = in[i];
    if(style == LABELS_SEQ && i > 0) {
      out[i].fromlabel = -1;
      if(!in[i].is_forward()) out[i].tolabel = -1;
    }
  }
}

std::string code_to_string(const DFS *code, int n)
{
  std::string s;
  char buf[96];
  for(int i = 0; i < n; i++) {
    std::snprintf(buf, sizeof(buf), "%s(%d %d %d %d %d)", i ? ";" : "", code[i].from, code[i].to, code[i].fromlabel,
                  code[i].elabel, code[i].tolabel);
    s += buf;
  }
  return s;
}

// The minimum code is rebuilt one edge at a time over all embeddings of its
// current prefix in the pattern graph (the sequential miner keeps them as
// PDFS chains and rebuilds a History per embedding; here each embedding
// carries its vertex map and used-vertex/used-edge masks directly).
bool MinChecker::is_min(const DFS *code, int n)
{
  if(n == 1) return true;
  if(n > kMaxPatternEdges) return false;
  to_style(code, n, LABELS_SEQ, seq_);

  // DFSCode::toGraph (dfs_code.cpp:245-266): labels from non -1 fields,
  // later fields overwrite earlier ones; adjacency in code order.
  nv_ = 0;
  for(int i = 0; i < n; i++) {
    int m = seq_[i].from > seq_[i].to ? seq_[i].from : seq_[i].to;
    if(m + 1 > nv_) nv_ = m + 1;
  }
  if(nv_ > kMaxPatternVertices) return false;
  for(int v = 0; v < nv_; v++) { vlab_[v] = 0; adj_[v].clear(); }
  for(int i = 0; i < n; i++) {
    if(seq_[i].fromlabel != -1) vlab_[seq_[i].from] = seq_[i].fromlabel;
    if(seq_[i].tolabel != -1) vlab_[seq_[i].to] = seq_[i].tolabel;
  }
  for(int i = 0; i < n; i++) {
    ef_[i] = seq_[i].from;
    et_[i] = seq_[i].to;
    adj_[seq_[i].from].push_back({ seq_[i].to, seq_[i].elabel, i });
    adj_[seq_[i].to].push_back({ seq_[i].from, seq_[i].elabel, i });
  }

  // root: minimum (fromlabel, elabel, tolabel) among edges with fl <= tl
  // (gSpan::is_min, ismin.cpp:45-60).  The first edge itself is not compared.
  bool have = false;
  int32_t b0 = 0, b1 = 0, b2 = 0;
  for(int v = 0; v < nv_; v++)
    for(const PAdj &a : adj_[v]) {
      if(vlab_[v] > vlab_[a.to]) continue;
      int32_t t0 = vlab_[v], t1 = a.elabel, t2 = vlab_[a.to];
      if(!have || t0 < b0 || (t0 == b0 && (t1 < b1 || (t1 == b1 && t2 < b2)))) { b0 = t0; b1 = t1; b2 = t2; have = true; }
    }
  cur_.clear();
  for(int v = 0; v < nv_; v++)
    for(const PAdj &a : adj_[v]) {
      if(vlab_[v] > vlab_[a.to]) continue;
      if(vlab_[v] == b0 && a.elabel == b1 && vlab_[a.to] == b2) {
        Emb e;
        e.map[0] = (uint8_t)v;
        e.map[1] = (uint8_t)a.to;
        e.hist[0] = (uint8_t)a.id;
        e.vmask = (1ull << v) | (1ull << a.to);
        e.emask[0] = e.emask[1] = 0;
        e.emask[a.id >> 6] |= 1ull << (a.id & 63);
        cur_.push_back(e);
      }
    }
  int m = 0;
  mc_[m++] = DFS{ 0, 1, b0, b1, b2 };

  int rm[kMaxPatternEdges];
  while(true) {
    // every pattern edge is in the minimum code: no extension remains, so the
    // reference's next project_is_min call returns true
    if(m >= n) return true;
    const int nrm = build_rmpath(mc_, m, rm);
    const int32_t minlabel = mc_[0].fromlabel;
    const int32_t maxtoc = mc_[rm[0]].to;
    auto has_e = [](const Emb &e, int id) { return (e.emask[id >> 6] >> (id & 63)) & 1ull; };

    // SUBBLOCK 1: backward edges from the right-most vertex; the rmpath
    // index nearest the root that has any wins (ismin.cpp:72-97).
    {
      int found_i = -1;
      int32_t bel = 0;
      for(int i = nrm - 1; found_i < 0 && i >= 1; --i) {
        for(const Emb &e : cur_) {
          // get_backward: e1 = history[rmpath[i]], e2 = history[rmpath[0]]
          const int e1 = e.hist[rm[i]], e2 = e.hist[rm[0]];
          const int32_t e1from = e.map[mc_[rm[i]].from], e1to = e.map[mc_[rm[i]].to];
          const int32_t e2to = e.map[mc_[rm[0]].to];
          (void)e2;
          for(const PAdj &a : adj_[e2to]) {
            if(has_e(e, a.id)) continue;
            const int32_t e1el = seq_[e1].elabel;
            if(a.to == e1from && (e1el < a.elabel || (e1el == a.elabel && vlab_[e1to] <= vlab_[e2to]))) {
              if(found_i < 0 || a.elabel < bel) bel = a.elabel;
              found_i = i;
              break;  // get_backward returns the first match
            }
          }
        }
      }
      if(found_i >= 0) {
        next_.clear();
        for(const Emb &e : cur_) {
          const int e1 = e.hist[rm[found_i]];
          const int32_t e1from = e.map[mc_[rm[found_i]].from], e1to = e.map[mc_[rm[found_i]].to];
          const int32_t e2to = e.map[mc_[rm[0]].to];
          for(const PAdj &a : adj_[e2to]) {
            if(has_e(e, a.id)) continue;
            const int32_t e1el = seq_[e1].elabel;
            if(a.to == e1from && (e1el < a.elabel || (e1el == a.elabel && vlab_[e1to] <= vlab_[e2to]))) {
              if(a.elabel == bel) {
                Emb x = e;
                x.hist[m] = (uint8_t)a.id;
                x.emask[a.id >> 6] |= 1ull << (a.id & 63);
                next_.push_back(x);
              }
              break;
            }
          }
        }
        mc_[m] = DFS{ maxtoc, mc_[rm[found_i]].from, -1, bel, -1 };
        if(seq_[m] != mc_[m]) return false;
        m++;
        cur_.swap(next_);
        continue;
      }
    }

    // SUBBLOCK 2: pure forward from the right-most vertex; otherwise forward
    // from the right-most path, deepest first (ismin.cpp:99-139).
    {
      int which = -2;  // -1 pure forward, >=0 rmpath index
      int32_t bel = 0, btl = 0;
      bool hv = false;
      for(const Emb &e : cur_) {
        const int32_t r = e.map[maxtoc];
        for(const PAdj &a : adj_[r]) {
          if(minlabel > vlab_[a.to] || ((e.vmask >> a.to) & 1ull)) continue;
          const int32_t tl = vlab_[a.to];
          if(!hv || a.elabel < bel || (a.elabel == bel && tl < btl)) { bel = a.elabel; btl = tl; hv = true; }
          which = -1;
        }
      }
      for(int i = 0; which == -2 && i < nrm; ++i) {
        for(const Emb &e : cur_) {
          const DFS &ce = mc_[rm[i]];
          const int32_t efrom = e.map[ce.from], eto = e.map[ce.to];
          const int32_t eel = seq_[e.hist[rm[i]]].elabel;
          const int32_t tolabel = vlab_[eto];
          for(const PAdj &a : adj_[efrom]) {
            const int32_t tl2 = vlab_[a.to];
            if(eto == a.to || minlabel > tl2 || ((e.vmask >> a.to) & 1ull)) continue;
            if(eel < a.elabel || (eel == a.elabel && tolabel <= tl2)) {
              if(!hv || a.elabel < bel || (a.elabel == bel && tl2 < btl)) { bel = a.elabel; btl = tl2; hv = true; }
              which = i;
            }
          }
        }
      }
      if(which == -2) return true;
      const int32_t newfrom = which == -1 ? maxtoc : mc_[rm[which]].from;
      next_.clear();
      for(const Emb &e : cur_) {
        if(which == -1) {
          const int32_t r = e.map[maxtoc];
          for(const PAdj &a : adj_[r]) {
            if(minlabel > vlab_[a.to] || ((e.vmask >> a.to) & 1ull)) continue;
            if(a.elabel == bel && vlab_[a.to] == btl) {
              Emb x = e;
              x.map[maxtoc + 1] = (uint8_t)a.to;
              x.hist[m] = (uint8_t)a.id;
              x.vmask |= 1ull << a.to;
              x.emask[a.id >> 6] |= 1ull << (a.id & 63);
              next_.push_back(x);
            }
          }
        } else {
          const DFS &ce = mc_[rm[which]];
          const int32_t efrom = e.map[ce.from], eto = e.map[ce.to];
          const int32_t eel = seq_[e.hist[rm[which]]].elabel;
          const int32_t tolabel = vlab_[eto];
          for(const PAdj &a : adj_[efrom]) {
            const int32_t tl2 = vlab_[a.to];
            if(eto == a.to || minlabel > tl2 || ((e.vmask >> a.to) & 1ull)) continue;
            if((eel < a.elabel || (eel == a.elabel && tolabel <= tl2)) && a.elabel == bel && tl2 == btl) {
              Emb x = e;
              x.map[maxtoc + 1] = (uint8_t)a.to;
              x.hist[m] = (uint8_t)a.id;
              x.vmask |= 1ull << a.to;
              x.emask[a.id >> 6] |= 1ull << (a.id & 63);
              next_.push_back(x);
            }
          }
        }
      }
      mc_[m] = DFS{ newfrom, maxtoc + 1, -1, bel, btl };
      if(seq_[m] != mc_[m]) return false;
      m++;
      cur_.swap(next_);
    }
  }
}

}  // namespace gsgb
