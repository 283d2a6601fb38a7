// Host-side graph database: readers/writers for the reference's four file
// formats, the simple-graph check, label compaction and the seeded
// synthetic generators.
#include "gs_db.hpp"

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>

namespace gsgb {

void parallel_ranges(int64_t n, const std::function<void(int64_t, int64_t, int)> &fn, int64_t min_chunk)
{
  int T = (int)std::min<unsigned>(32u, std::max(1u, std::thread::hardware_concurrency()));
  if(n < 2 * min_chunk) T = 1;
  else T = (int)std::min<int64_t>(T, n / min_chunk);
  if(T <= 1) {
    fn(0, n, 0);
    return;
  }
  std::vector<std::thread> th;
  for(int t = 0; t < T; t++) {
    const int64_t b = n * t / T, e = n * (t + 1) / T;
    th.emplace_back([&fn, b, e, t] { fn(b, e, t); });
  }
  for(auto &x : th) x.join();
}

int parse_filetype(const char *name)
{
  if(!name) return -1;
  std::string s(name);
  if(s == "-txt" || s == "txt") return FT_TXT;
  if(s == "-bin" || s == "bin") return FT_BIN;
  if(s == "-fsg" || s == "fsg") return FT_FSG;
  if(s == "-cudabin" || s == "cudabin") return FT_CUDABIN;
  return -1;
}

namespace {

constexpr int ST_ERR_IO = 2;
constexpr int ST_ERR_FORMAT = 3;

LoadResult fail(int code, const std::string &msg)
{
  LoadResult r;
  r.code = code;
  r.error = msg;
  return r;
}

bool read_file(const char *path, std::vector<char> &buf)
{
  FILE *f = std::fopen(path, "rb");
  if(!f) return false;
  std::fseek(f, 0, SEEK_END);
  long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if(n < 0) { std::fclose(f); return false; }
  buf.resize((size_t)n + 1);
  size_t got = n ? std::fread(buf.data(), 1, (size_t)n, f) : 0;
  std::fclose(f);
  if(got != (size_t)n) return false;
  buf[(size_t)n] = 0;
  buf.resize((size_t)n);
  return true;
}

// One graph under construction: vertex labels by local id plus the edge list
// in input order.  Appending to the database lays each vertex's adjacency out
// in push order: edge i contributes (f -> t) to f and (t -> f) to t
// (Graph::read, src/globals/graph_types.cpp:99-103).
struct GraphBuild {
  std::vector<int32_t> vl;
  std::vector<int32_t> ef, et, el;
  void clear() { vl.clear(); ef.clear(); et.clear(); el.clear(); }
  bool empty() const { return vl.empty(); }
};

void append_graph(HostDB &db, const GraphBuild &gb)
{
  if(db.vbase.empty()) db.vbase.push_back(0);
  if(db.aoff.empty()) db.aoff.push_back(0);
  const int64_t base = db.vbase.back();
  const int32_t nv = (int32_t)gb.vl.size();
  std::vector<int32_t> deg(nv, 0);
  for(size_t i = 0; i < gb.ef.size(); i++) { deg[gb.ef[i]]++; deg[gb.et[i]]++; }
  const int64_t a0 = (int64_t)db.adj_to.size();
  std::vector<int64_t> pos(nv);
  int64_t acc = a0;
  for(int32_t v = 0; v < nv; v++) {
    pos[v] = acc;
    acc += deg[v];
    db.vlabel.push_back(gb.vl[v]);
    db.aoff.push_back(acc);
  }
  db.adj_to.resize(acc);
  db.adj_el.resize(acc);
  for(size_t i = 0; i < gb.ef.size(); i++) {
    int32_t f = gb.ef[i], t = gb.et[i];
    db.adj_to[pos[f]] = (int32_t)(base + t);
    db.adj_el[pos[f]++] = gb.el[i];
    db.adj_to[pos[t]] = (int32_t)(base + f);
    db.adj_el[pos[t]++] = gb.el[i];
  }
  db.vbase.push_back(base + nv);
  db.n_graphs++;
}

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r'; }

// Line-oriented reader for the txt (t/v/e) and fsg (t/v/u, string labels
// renumbered per graph by first appearance) formats.
LoadResult read_text(const char *path, bool fsg, HostDB &db)
{
  std::vector<char> buf;
  if(!read_file(path, buf)) return fail(ST_ERR_IO, std::string("cannot read database file ") + path);
  GraphBuild gb;
  std::map<std::string, int32_t> vmap, emap;
  const char *p = buf.data();
  const char *end = p + buf.size();
  const char etag = fsg ? 'u' : 'e';
  int64_t lineno = 0;
  while(p < end) {
    const char *ls = p;
    while(p < end && *p != '\n') p++;
    const char *le = p;
    if(p < end) p++;
    lineno++;
    // tokenize
    const char *tok[6];
    int tl[6];
    int nt = 0;
    const char *q = ls;
    while(q < le && nt < 6) {
      while(q < le && is_space(*q)) q++;
      if(q >= le) break;
      tok[nt] = q;
      while(q < le && !is_space(*q)) q++;
      tl[nt] = (int)(q - tok[nt]);
      nt++;
    }
    if(nt == 0) continue;
    if(tl[0] == 1 && tok[0][0] == 't') {
      // a "t" line closes a non-empty graph (Graph::read treats it as a delimiter)
      if(!gb.empty()) append_graph(db, gb);
      gb.clear();
      vmap.clear();
      emap.clear();
    } else if(tl[0] == 1 && tok[0][0] == 'v' && nt >= 3) {
      int64_t id = std::strtoll(tok[1], nullptr, 10);
      if(id < 0 || id > (1 << 24)) return fail(ST_ERR_FORMAT, "vertex id out of range at line " + std::to_string(lineno));
      int32_t lab;
      if(fsg) {
        std::string s(tok[2], tl[2]);
        auto it = vmap.find(s);
        if(it == vmap.end()) it = vmap.emplace(s, (int32_t)vmap.size()).first;
        lab = it->second;
      } else {
        lab = (int32_t)std::strtol(tok[2], nullptr, 10);
      }
      if((int64_t)gb.vl.size() < id + 1) gb.vl.resize(id + 1, 0);
      gb.vl[id] = lab;
    } else if(tl[0] == 1 && tok[0][0] == etag && nt >= 4) {
      int64_t f = std::strtoll(tok[1], nullptr, 10);
      int64_t t = std::strtoll(tok[2], nullptr, 10);
      if(f < 0 || t < 0 || f >= (int64_t)gb.vl.size() || t >= (int64_t)gb.vl.size())
        return fail(ST_ERR_FORMAT, "Format Error: define vertex lists before edges (line " + std::to_string(lineno) + ")");
      int32_t lab;
      if(fsg) {
        std::string s(tok[3], tl[3]);
        auto it = emap.find(s);
        if(it == emap.end()) it = emap.emplace(s, (int32_t)emap.size()).first;
        lab = it->second;
      } else {
        lab = (int32_t)std::strtol(tok[3], nullptr, 10);
      }
      gb.ef.push_back((int32_t)f);
      gb.et.push_back((int32_t)t);
      gb.el.push_back(lab);
    }
  }
  if(!gb.empty()) append_graph(db, gb);
  return LoadResult();
}

template <class T> bool take(const std::vector<char> &b, size_t &pos, T &out)
{
  if(pos + sizeof(T) > b.size()) return false;
  std::memcpy(&out, b.data() + pos, sizeof(T));
  pos += sizeof(T);
  return true;
}

// BIN: size_t graph count, size_t offset per graph, then per graph a size_t
// byte count followed by Graph::serialize (src/globals/graph_types.cpp:
// 560-584: int size, int edge_size, bool directed, int nv, then per vertex
// int size, int label, int nedges, nedges x {from, to, elabel, id}),
// src/globals/dbio.cpp:132-191.
LoadResult read_bin(const char *path, HostDB &db)
{
  std::vector<char> b;
  if(!read_file(path, b)) return fail(ST_ERR_IO, std::string("cannot read database file ") + path);
  size_t pos = 0;
  uint64_t ng = 0;
  if(!take(b, pos, ng)) return fail(ST_ERR_FORMAT, "bin: truncated header");
  if(ng > (uint64_t)b.size()) return fail(ST_ERR_FORMAT, "bin: bad graph count");
  std::vector<uint64_t> index(ng);
  for(uint64_t i = 0; i < ng; i++)
    if(!take(b, pos, index[i])) return fail(ST_ERR_FORMAT, "bin: truncated index");
  GraphBuild gb;
  for(uint64_t i = 0; i < ng; i++) {
    if(index[i] != pos) return fail(ST_ERR_FORMAT, "bin: graph stored at an unexpected offset");
    uint64_t gsz = 0;
    if(!take(b, pos, gsz)) return fail(ST_ERR_FORMAT, "bin: truncated graph size");
    size_t gend = pos + gsz;
    if(gend > b.size()) return fail(ST_ERR_FORMAT, "bin: truncated graph");
    int32_t tot, esz, nv;
    uint8_t directed;
    if(!take(b, pos, tot) || !take(b, pos, esz) || !take(b, pos, directed) || !take(b, pos, nv))
      return fail(ST_ERR_FORMAT, "bin: truncated graph header");
    if(nv < 0) return fail(ST_ERR_FORMAT, "bin: negative vertex count");
    gb.clear();
    gb.vl.resize(nv);
    // the stored adjacency already holds both directions; keep each vertex's
    // list verbatim by pushing directed entries, then rebuild in order
    std::vector<std::vector<std::pair<int32_t, int32_t>>> lists(nv);
    for(int32_t v = 0; v < nv; v++) {
      int32_t vs, lab, ne;
      if(!take(b, pos, vs) || !take(b, pos, lab) || !take(b, pos, ne)) return fail(ST_ERR_FORMAT, "bin: truncated vertex");
      gb.vl[v] = lab;
      for(int32_t k = 0; k < ne; k++) {
        int32_t f, t, el, id;
        if(!take(b, pos, f) || !take(b, pos, t) || !take(b, pos, el) || !take(b, pos, id))
          return fail(ST_ERR_FORMAT, "bin: truncated edge");
        if(t < 0 || t >= nv) return fail(ST_ERR_FORMAT, "bin: edge target out of range");
        lists[v].push_back({t, el});
      }
    }
    if(pos != gend) return fail(ST_ERR_FORMAT, "bin: graph size mismatch");
    if(db.vbase.empty()) db.vbase.push_back(0);
    if(db.aoff.empty()) db.aoff.push_back(0);
    int64_t base = db.vbase.back();
    for(int32_t v = 0; v < nv; v++) {
      db.vlabel.push_back(gb.vl[v]);
      for(auto &e : lists[v]) { db.adj_to.push_back((int32_t)(base + e.first)); db.adj_el.push_back(e.second); }
      db.aoff.push_back((int64_t)db.adj_to.size());
    }
    db.vbase.push_back(base + nv);
    db.n_graphs++;
  }
  if(pos != b.size()) return fail(ST_ERR_FORMAT, "bin: trailing bytes");
  return LoadResult();
}

}  // namespace

// cudabin: int32 {db_size, edges_sizes, max_graph_vertex_count,
// vertex_count}, edges[], edges_labels[], vertex_labels[db*maxv],
// vertex_offsets[db*maxv+1] with -1 padding (src/globals/dbio.cpp:359-404).
// The end of vertex v's neighbourhood is the offset of the next valid slot
// (graph_database_cuda::get_next_valid_vertex_idx, cuda_graph_types.hpp:84-91).
LoadResult db_from_cudabin_arrays(int32_t db_size, int32_t edges_sizes, int32_t maxv,
                                  const int32_t *edges, const int32_t *elab,
                                  const int32_t *vlab, const int32_t *voff, HostDB &db)
{
  if(db_size < 0 || edges_sizes < 0 || maxv < 0) return fail(ST_ERR_FORMAT, "cudabin: negative sizes");
  db = HostDB();
  const int64_t slots = (int64_t)db_size * maxv;
  // pass 1 (parallel over graphs): vertices per graph (valid slots are a
  // prefix of the graph's slots) and adjacency entries per graph, which end
  // where the next graph's first slot (or the trailing sentinel) begins
  std::vector<int64_t> gnv((size_t)db_size + 1, 0), gadj((size_t)db_size + 1, 0);
  std::atomic<int> bad{ 0 };
  parallel_ranges(db_size, [&](int64_t g0, int64_t g1, int) {
    for(int64_t g = g0; g < g1; g++) {
      const int64_t base = g * maxv;
      int32_t nv = 0;
      while(nv < maxv && voff[base + nv] != -1) nv++;
      gnv[g] = nv;
      if(nv > 0) {
        const int64_t nxt = (g + 1) * maxv <= slots ? (g + 1) * maxv : slots;
        const int64_t b0 = voff[base], e1 = voff[nxt];
        if(b0 < 0 || e1 < b0 || e1 > edges_sizes) bad = 1;
        else gadj[g] = e1 - b0;
      }
    }
  });
  if(bad) return fail(ST_ERR_FORMAT, "cudabin: bad vertex offsets");
  db.vbase.resize((size_t)db_size + 1);
  std::vector<int64_t> gpos((size_t)db_size + 1);
  db.vbase[0] = 0;
  gpos[0] = 0;
  for(int64_t g = 0; g < db_size; g++) {
    db.vbase[g + 1] = db.vbase[g] + gnv[g];
    gpos[g + 1] = gpos[g] + gadj[g];
  }
  const int64_t V = db.vbase[db_size], nadj = gpos[db_size];
  db.vlabel.resize((size_t)V);
  db.aoff.resize((size_t)V + 1);
  db.adj_to.resize((size_t)nadj);
  db.adj_el.resize((size_t)nadj);
  db.aoff[0] = 0;
  // pass 2 (parallel over graphs): a vertex's neighbourhood ends at the next
  // valid slot's offset (graph_database_cuda::get_next_valid_vertex_idx)
  parallel_ranges(db_size, [&](int64_t g0, int64_t g1, int) {
    for(int64_t g = g0; g < g1; g++) {
      const int64_t base = g * maxv, gbase = db.vbase[g];
      const int32_t nv = (int32_t)(db.vbase[g + 1] - gbase);
      int64_t pos = gpos[g];
      for(int32_t v = 0; v < nv; v++) {
        int64_t nxt = (v + 1 < nv) ? base + v + 1 : (g + 1) * maxv;
        if(nxt > slots) nxt = slots;
        const int64_t b0 = voff[base + v], b1 = voff[nxt];
        if(b0 < 0 || b1 < b0 || b1 > edges_sizes || pos + (b1 - b0) > gpos[g + 1]) {
          bad = 1;
          return;
        }
        db.vlabel[gbase + v] = vlab[base + v];
        for(int64_t k = b0; k < b1; k++) {
          const int64_t t = (int64_t)edges[k] - base;
          if(t < 0 || t >= nv) {
            bad = 2;
            return;
          }
          db.adj_to[pos] = (int32_t)(gbase + t);
          db.adj_el[pos++] = elab[k];
        }
        db.aoff[gbase + v + 1] = pos;
      }
      if(pos != gpos[g + 1]) bad = 1;
    }
  });
  if(bad == 2) return fail(ST_ERR_FORMAT, "cudabin: edge leaves its graph");
  if(bad) return fail(ST_ERR_FORMAT, "cudabin: vertex offsets do not tile the edge array");
  db.n_graphs = db_size;
  return LoadResult();
}

namespace {

LoadResult read_cudabin(const char *path, HostDB &db)
{
  std::vector<char> b;
  if(!read_file(path, b)) return fail(ST_ERR_IO, std::string("cannot read database file ") + path);
  if(b.size() < 16) return fail(ST_ERR_FORMAT, "cudabin: truncated header");
  int32_t hdr[4];
  std::memcpy(hdr, b.data(), 16);
  int64_t dbsz = hdr[0], esz = hdr[1], maxv = hdr[2];
  if(dbsz < 0 || esz < 0 || maxv < 0) return fail(ST_ERR_FORMAT, "cudabin: negative sizes");
  int64_t slots = dbsz * maxv;
  uint64_t need = 16 + 4ull * (2 * esz + 2 * slots + 1);
  if(b.size() < need) return fail(ST_ERR_FORMAT, "cudabin: truncated arrays");
  const int32_t *p = reinterpret_cast<const int32_t *>(b.data() + 16);
  std::vector<int32_t> a(p, p + (2 * esz + 2 * slots + 1));
  const int32_t *edges = a.data();
  const int32_t *elab = edges + esz;
  const int32_t *vlab = elab + esz;
  const int32_t *voff = vlab + slots;
  return db_from_cudabin_arrays((int32_t)dbsz, (int32_t)esz, (int32_t)maxv, edges, elab, vlab, voff, db);
}

}  // namespace

LoadResult load_database(const char *path, int filetype, HostDB &db, bool validate)
{
  db = HostDB();
  LoadResult r;
  switch(filetype) {
  case FT_TXT: r = read_text(path, false, db); break;
  case FT_FSG: r = read_text(path, true, db); break;
  case FT_BIN: r = read_bin(path, db); break;
  case FT_CUDABIN: r = read_cudabin(path, db); break;
  default: return fail(1, "unknown filetype");
  }
  if(!r.error.empty()) return r;
  if(db.vbase.empty()) db.vbase.push_back(0);
  if(db.aoff.empty()) db.aoff.push_back(0);
  if(db.n_vertices() >= (int64_t)INT32_MAX || db.n_adj() >= (int64_t)INT32_MAX)
    return fail(ST_ERR_FORMAT, "database too large for 32-bit vertex/adjacency indices");
  return validate ? validate_simple(db) : LoadResult();
}

LoadResult fix_database(HostDB &db, int64_t *fixed, int64_t *renumbered)
{
  int64_t nfix = 0, nren = 0;
  HostDB out;
  out.vbase.push_back(0);
  out.aoff.push_back(0);
  std::vector<std::vector<std::pair<int32_t, int32_t>>> lists;
  for(int32_t g = 0; g < db.n_graphs; g++) {
    const int64_t base = db.vbase[g];
    const int32_t nv = db.graph_nv(g);
    lists.assign(nv, {});
    // check_graph: a self loop, or a neighbour listed twice at one vertex
    bool bad = false;
    for(int32_t v = 0; v < nv && !bad; v++) {
      std::set<int32_t> seen;
      for(int64_t k = db.aoff[base + v]; k < db.aoff[base + v + 1]; k++) {
        const int32_t t = (int32_t)(db.adj_to[k] - base);
        if(t == v || !seen.insert(t).second) {
          bad = true;
          break;
        }
      }
    }
    for(int32_t v = 0; v < nv; v++) {
      if(!bad) {
        for(int64_t k = db.aoff[base + v]; k < db.aoff[base + v + 1]; k++)
          lists[v].push_back({ (int32_t)(db.adj_to[k] - base), db.adj_el[k] });
        continue;
      }
      // fix_graph: one edge per neighbour, neighbours ascending, no self loops
      std::map<int32_t, int32_t> to_label;
      for(int64_t k = db.aoff[base + v]; k < db.aoff[base + v + 1]; k++) {
        const int32_t t = (int32_t)(db.adj_to[k] - base);
        if(t == v) continue;
        auto it = to_label.find(t);
        if(it == to_label.end()) to_label.emplace(t, db.adj_el[k]);
        else if(it->second != db.adj_el[k])
          return fail(ST_ERR_FORMAT, "error: unable to fix graph, parallel edge has different label (graph " +
                                         std::to_string(g) + ")");
      }
      for(const auto &e : to_label) lists[v].push_back(e);
    }
    if(bad) nfix++;
    // vertex 0 goes when no other vertex has it as a neighbour
    bool drop0 = nv > 0;
    for(int32_t v = 1; v < nv && drop0; v++)
      for(const auto &e : lists[v])
        if(e.first == 0) {
          drop0 = false;
          break;
        }
    const int32_t first = drop0 ? 1 : 0;
    if(drop0) nren++;
    const int64_t obase = out.vbase.back();
    for(int32_t v = first; v < nv; v++) {
      out.vlabel.push_back(db.vlabel[base + v]);
      for(const auto &e : lists[v]) {
        out.adj_to.push_back((int32_t)(obase + e.first - first));
        out.adj_el.push_back(e.second);
      }
      out.aoff.push_back((int64_t)out.adj_to.size());
    }
    out.vbase.push_back(obase + (nv - first));
    out.n_graphs++;
  }
  db = std::move(out);
  if(fixed) *fixed = nfix;
  if(renumbered) *renumbered = nren;
  return LoadResult();
}

LoadResult validate_simple(const HostDB &db)
{
  // one pass: stamp[w] = the last vertex that listed w as a neighbour, so a
  // repeat within one vertex's list is a parallel edge (no per-vertex sort)
  // (parallel over graphs: neighbours never leave their graph, so the stamp
  // entries a part touches belong to its own graphs)
  std::vector<int32_t> stamp((size_t)db.n_vertices(), -1);
  std::atomic<int64_t> first_bad{ INT64_MAX };
  std::atomic<int> kind{ 0 };
  parallel_ranges(db.n_graphs, [&](int64_t g0, int64_t g1, int) {
    for(int64_t v = db.vbase[g0]; v < db.vbase[g1]; v++) {
      for(int64_t k = db.aoff[v]; k < db.aoff[v + 1]; k++) {
        const int32_t w = db.adj_to[k];
        int why = 0;
        if(w == v) why = 1;
        else if(w < db.vbase[g0] || w >= db.vbase[g1]) why = 3;
        else if(stamp[w] == (int32_t)v) why = 2;
        if(why) {
          int64_t cur = first_bad.load();
          while(v < cur && !first_bad.compare_exchange_weak(cur, v)) {}
          if(first_bad.load() == v) kind = why;
          return;
        }
        stamp[w] = (int32_t)v;
      }
    }
  });
  if(kind) {
    const std::string v = std::to_string(first_bad.load());
    if(kind == 1) return fail(ST_ERR_FORMAT, "self loop at global vertex " + v + " (only simple graphs are supported)");
    if(kind == 2) return fail(ST_ERR_FORMAT, "parallel edges at global vertex " + v + " (only simple graphs are supported)");
    return fail(ST_ERR_FORMAT, "neighbour outside its graph at global vertex " + v);
  }
  return LoadResult();
}

namespace {

// Dense, order-preserving relabelling of one label array: a lookup table
// over [min, max] when that range is small, else sort + binary search.
void dense_labels(const std::vector<int32_t> &in, std::vector<int32_t> &out, std::vector<int32_t> &of)
{
  out.resize(in.size());
  of.clear();
  if(in.empty()) return;
  std::vector<int32_t> plo(32, INT32_MAX), phi_(32, INT32_MIN);
  parallel_ranges((int64_t)in.size(), [&](int64_t b, int64_t e, int t) {
    int32_t l = INT32_MAX, h = INT32_MIN;
    for(int64_t i = b; i < e; i++) { l = std::min(l, in[i]); h = std::max(h, in[i]); }
    plo[t] = l;
    phi_[t] = h;
  }, 1 << 16);
  const int32_t lo = *std::min_element(plo.begin(), plo.end()), hi = *std::max_element(phi_.begin(), phi_.end());
  const int64_t range = (int64_t)hi - lo + 1;
  if(range <= ((int64_t)1 << 24)) {
    std::vector<int32_t> map((size_t)range, -1);
    if(range <= 4096) {
      // small alphabets: per-part presence, merged
      std::vector<std::vector<uint8_t>> seen(32);
      parallel_ranges((int64_t)in.size(), [&](int64_t b, int64_t e, int t) {
        std::vector<uint8_t> s((size_t)range, 0);
        for(int64_t i = b; i < e; i++) s[(size_t)((int64_t)in[i] - lo)] = 1;
        seen[t].swap(s);
      }, 1 << 16);
      for(auto &s : seen)
        for(size_t r = 0; r < s.size(); r++)
          if(s[r]) map[r] = 0;
    } else {
      for(int32_t x : in) map[(size_t)((int64_t)x - lo)] = 0;
    }
    int32_t next = 0;
    for(int64_t r = 0; r < range; r++)
      if(map[r] == 0) { map[r] = next++; of.push_back((int32_t)(lo + r)); }
    parallel_ranges((int64_t)in.size(), [&](int64_t b, int64_t e, int) {
      for(int64_t i = b; i < e; i++) out[i] = map[(size_t)((int64_t)in[i] - lo)];
    }, 1 << 16);
  } else {
    of = in;
    std::sort(of.begin(), of.end());
    of.erase(std::unique(of.begin(), of.end()), of.end());
    for(size_t i = 0; i < in.size(); i++)
      out[i] = (int32_t)(std::lower_bound(of.begin(), of.end(), in[i]) - of.begin());
  }
}

}  // namespace

void compact_labels(const HostDB &db, std::vector<int32_t> &vl, std::vector<int32_t> &el, LabelMap &map)
{
  dense_labels(db.vlabel, vl, map.vlabel_of);
  dense_labels(db.adj_el, el, map.elabel_of);
}

// -------------------------------------------------------------- writers

LoadResult write_database(const HostDB &db, const char *path, int filetype)
{
  FILE *f = std::fopen(path, "wb");
  if(!f) return fail(ST_ERR_IO, std::string("cannot open for writing: ") + path);
  if(filetype == FT_TXT) {
    for(int32_t g = 0; g < db.n_graphs; g++) {
      std::fprintf(f, "t # %d\n", g);
      int64_t b = db.vbase[g];
      for(int64_t v = b; v < db.vbase[g + 1]; v++) std::fprintf(f, "v %lld %d\n", (long long)(v - b), db.vlabel[v]);
      for(int64_t v = b; v < db.vbase[g + 1]; v++)
        for(int64_t k = db.aoff[v]; k < db.aoff[v + 1]; k++)
          if(db.adj_to[k] > v) std::fprintf(f, "e %lld %lld %d\n", (long long)(v - b), (long long)(db.adj_to[k] - b), db.adj_el[k]);
    }
  } else if(filetype == FT_CUDABIN) {
    int32_t maxv = 0;
    for(int32_t g = 0; g < db.n_graphs; g++) maxv = std::max(maxv, db.graph_nv(g));
    int64_t slots = (int64_t)db.n_graphs * maxv;
    int32_t hdr[4] = { db.n_graphs, (int32_t)db.n_adj(), maxv, (int32_t)db.n_vertices() };
    std::vector<int32_t> edges(db.n_adj()), vl(slots, -1), vo(slots + 1, -1);
    for(int32_t g = 0; g < db.n_graphs; g++) {
      int64_t b = db.vbase[g];
      for(int64_t v = b; v < db.vbase[g + 1]; v++) {
        int64_t slot = (int64_t)g * maxv + (v - b);
        vl[slot] = db.vlabel[v];
        vo[slot] = (int32_t)db.aoff[v];
        for(int64_t k = db.aoff[v]; k < db.aoff[v + 1]; k++) edges[k] = (int32_t)((int64_t)g * maxv + (db.adj_to[k] - b));
      }
    }
    vo[slots] = (int32_t)db.n_adj();
    std::fwrite(hdr, 4, 4, f);
    std::fwrite(edges.data(), 4, edges.size(), f);
    std::fwrite(db.adj_el.data(), 4, db.adj_el.size(), f);
    std::fwrite(vl.data(), 4, vl.size(), f);
    std::fwrite(vo.data(), 4, vo.size(), f);
  } else if(filetype == FT_BIN) {
    // Graph::serialize per graph, with edge ids numbered as Graph::buildEdge
    // does (first appearance of each undirected edge in vertex order).
    std::vector<std::vector<char>> blobs(db.n_graphs);
    for(int32_t g = 0; g < db.n_graphs; g++) {
      int64_t b = db.vbase[g];
      int32_t nv = db.graph_nv(g);
      std::vector<int32_t> ids(db.aoff[b + nv] - db.aoff[b], -1);
      int32_t next = 0;
      for(int32_t v = 0; v < nv; v++) {
        for(int64_t k = db.aoff[b + v]; k < db.aoff[b + v + 1]; k++) {
          int32_t t = (int32_t)(db.adj_to[k] - b);
          int32_t found = -1;
          if(t < v) {
            for(int64_t j = db.aoff[b + t]; j < db.aoff[b + t + 1]; j++)
              if(db.adj_to[j] - b == v && db.adj_el[j] == db.adj_el[k]) { found = ids[j - db.aoff[b]]; break; }
          }
          ids[k - db.aoff[b]] = found >= 0 ? found : next++;
        }
      }
      std::vector<char> &o = blobs[g];
      auto put32 = [&o](int32_t x) { const char *c = (const char *)&x; o.insert(o.end(), c, c + 4); };
      put32(0);  // patched below
      put32(next);
      o.push_back(0);
      put32(nv);
      for(int32_t v = 0; v < nv; v++) {
        int32_t ne = (int32_t)(db.aoff[b + v + 1] - db.aoff[b + v]);
        put32(4 + 4 + 4 + 16 * ne);
        put32(db.vlabel[b + v]);
        put32(ne);
        for(int64_t k = db.aoff[b + v]; k < db.aoff[b + v + 1]; k++) {
          put32(v);
          put32((int32_t)(db.adj_to[k] - b));
          put32(db.adj_el[k]);
          put32(ids[k - db.aoff[b]]);
        }
      }
      int32_t tot = (int32_t)o.size();
      std::memcpy(o.data(), &tot, 4);
    }
    uint64_t ng = (uint64_t)db.n_graphs;
    std::fwrite(&ng, 8, 1, f);
    uint64_t off = (ng + 1) * 8;
    for(int32_t g = 0; g < db.n_graphs; g++) {
      std::fwrite(&off, 8, 1, f);
      off += 8 + blobs[g].size();
    }
    for(int32_t g = 0; g < db.n_graphs; g++) {
      uint64_t s = blobs[g].size();
      std::fwrite(&s, 8, 1, f);
      std::fwrite(blobs[g].data(), 1, s, f);
    }
  } else {
    std::fclose(f);
    return fail(1, "unsupported filetype for writing");
  }
  std::fclose(f);
  return LoadResult();
}

// ----------------------------------------------------------- generators

namespace {

// xoshiro256** seeded through splitmix64: identical streams on x86 and Arm.
struct Rng {
  uint64_t s[4];
  static uint64_t splitmix(uint64_t &x)
  {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  explicit Rng(uint64_t seed) { for(int i = 0; i < 4; i++) s[i] = splitmix(seed); }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next()
  {
    uint64_t r = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t; s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  int64_t range(int64_t lo, int64_t hi) { return lo + (int64_t)(next() % (uint64_t)(hi - lo + 1)); }  // inclusive
  int poisson(double mean)
  {
    // Knuth's product-of-uniforms method; means here are <= ~60
    double L = std::exp(-mean), p = 1.0;
    int k = 0;
    do { k++; p *= uniform(); } while(p > L);
    return k - 1;
  }
};

struct Categorical {
  std::vector<double> cdf;
  void set(const std::vector<double> &w)
  {
    cdf.resize(w.size());
    double s = 0;
    for(size_t i = 0; i < w.size(); i++) { s += w[i]; cdf[i] = s; }
    for(auto &c : cdf) c /= s;
  }
  int draw(Rng &r) const
  {
    double u = r.uniform();
    size_t i = std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin();
    return (int)std::min(i, cdf.size() - 1);
  }
};

struct SmallGraph {
  std::vector<int32_t> vl;
  std::vector<int32_t> ef, et, el;
  std::vector<std::vector<int32_t>> nb;
  int32_t add_vertex(int32_t lab) { vl.push_back(lab); nb.emplace_back(); return (int32_t)vl.size() - 1; }
  bool adjacent(int32_t a, int32_t b) const
  {
    for(int32_t x : nb[a]) if(x == b) return true;
    return false;
  }
  void add_edge(int32_t a, int32_t b, int32_t lab)
  {
    ef.push_back(a); et.push_back(b); el.push_back(lab);
    nb[a].push_back(b); nb[b].push_back(a);
  }
  // a random chord between two distinct non-adjacent vertices; false if none found
  bool add_chord(Rng &r, int32_t lab)
  {
    int32_t n = (int32_t)vl.size();
    if(n < 3) return false;
    for(int tries = 0; tries < 24; tries++) {
      int32_t a = (int32_t)r.range(0, n - 1), b = (int32_t)r.range(0, n - 1);
      if(a == b || adjacent(a, b)) continue;
      add_edge(a, b, lab);
      return true;
    }
    return false;
  }
};

}  // namespace

void generate_database(const GenParams &p, HostDB &db)
{
  db = HostDB();
  Rng rng(p.seed);
  Categorical vcat, ecat;
  {
    std::vector<double> w(p.n_vlabels);
    for(int i = 0; i < p.n_vlabels; i++) w[i] = p.vzipf > 0 ? 1.0 / std::pow((double)(i + 1), p.vzipf) : 1.0;
    vcat.set(w);
    std::vector<double> e(p.n_elabels, 1.0);
    if((int)p.eweights.size() == p.n_elabels) e = p.eweights;
    ecat.set(e);
  }
  GraphBuild gb;
  if(p.mode == 0) {
    for(int64_t g = 0; g < p.n_graphs; g++) {
      SmallGraph s;
      int32_t nv = (int32_t)rng.range(p.vmin, p.vmax);
      for(int32_t v = 0; v < nv; v++) s.add_vertex(vcat.draw(rng));
      for(int32_t v = 1; v < nv; v++) s.add_edge((int32_t)rng.range(0, v - 1), v, ecat.draw(rng));
      double x = nv * p.ring_per_vertex;
      int extra = (int)std::floor(x + rng.uniform());
      for(int i = 0; i < extra; i++) s.add_chord(rng, ecat.draw(rng));
      gb.clear();
      gb.vl = s.vl; gb.ef = s.ef; gb.et = s.et; gb.el = s.el;
      append_graph(db, gb);
    }
  } else {
    // seed patterns: connected, grown by attaching new vertices with an
    // occasional ring-closing chord
    std::vector<SmallGraph> seeds(p.n_seeds);
    for(int i = 0; i < p.n_seeds; i++) {
      int ne = std::max(p.seed_min_edges, rng.poisson(p.seed_mean_edges));
      if(p.seed_max_edges > 0) ne = std::min(ne, p.seed_max_edges);
      SmallGraph &s = seeds[i];
      s.add_vertex(vcat.draw(rng));
      for(int e = 0; e < ne; e++) {
        if(s.vl.size() >= 3 && rng.uniform() < 0.25 && s.add_chord(rng, ecat.draw(rng))) continue;
        int32_t a = (int32_t)rng.range(0, (int64_t)s.vl.size() - 1);
        int32_t b = s.add_vertex(vcat.draw(rng));
        s.add_edge(a, b, ecat.draw(rng));
      }
    }
    for(int64_t g = 0; g < p.n_graphs; g++) {
      int budget = std::max(1, rng.poisson(p.mean_edges));
      SmallGraph s;
      std::vector<int32_t> comp_first;  // first vertex of each embedded copy
      int covered = 0;
      while(p.n_seeds > 0 && covered < p.seed_cover * budget) {
        const SmallGraph &sp = seeds[rng.range(0, p.n_seeds - 1)];
        int32_t base = (int32_t)s.vl.size();
        comp_first.push_back(base);
        for(int32_t lab : sp.vl) s.add_vertex(lab);
        for(size_t e = 0; e < sp.ef.size(); e++) s.add_edge(base + sp.ef[e], base + sp.et[e], sp.el[e]);
        covered += (int)sp.ef.size();
      }
      if(s.vl.empty()) { s.add_vertex(vcat.draw(rng)); comp_first.push_back(0); }
      int used = covered;
      // link the copies into one connected graph
      for(size_t c = 1; c < comp_first.size(); c++) {
        int32_t lo = comp_first[c];
        int32_t hi = (c + 1 < comp_first.size()) ? comp_first[c + 1] - 1 : (int32_t)s.vl.size() - 1;
        int32_t a = (int32_t)rng.range(lo, hi);
        int32_t b = (int32_t)rng.range(0, lo - 1);
        s.add_edge(a, b, ecat.draw(rng));
        used++;
      }
      // fill the remaining edge budget with random growth and chords
      while(used < budget) {
        if(rng.uniform() < 0.5 || !s.add_chord(rng, ecat.draw(rng))) {
          int32_t a = (int32_t)rng.range(0, (int64_t)s.vl.size() - 1);
          int32_t b = s.add_vertex(vcat.draw(rng));
          s.add_edge(a, b, ecat.draw(rng));
        }
        used++;
      }
      gb.clear();
      gb.vl = s.vl; gb.ef = s.ef; gb.et = s.et; gb.el = s.el;
      append_graph(db, gb);
    }
  }
  if(db.vbase.empty()) db.vbase.push_back(0);
  if(db.aoff.empty()) db.aoff.push_back(0);
}

bool config_params(int config, uint64_t seed, double scale, GenParams &p)
{
  p = GenParams();
  auto scaled = [scale](int64_t n) { return std::max<int64_t>(1, (int64_t)std::llround((double)n * scale)); };
  switch(config) {
  case 1:  // stands in for testdata/Chemical_340
    p.mode = 0; p.n_graphs = scaled(340); p.vmin = 10; p.vmax = 60; p.ring_per_vertex = 0.05;
    p.n_vlabels = 66; p.vzipf = 1.5; p.n_elabels = 4; p.eweights = { 0.6, 0.3, 0.08, 0.02 };
    p.seed = seed ? seed : 1;
    return true;
  case 2:  // stands in for the PAFI T100000E5PL4P50TL30V5 database
    p.mode = 1; p.n_graphs = scaled(100000); p.mean_edges = 30; p.n_vlabels = 5; p.n_elabels = 5;
    p.n_seeds = 50; p.seed_mean_edges = 4; p.seed_min_edges = 1; p.seed_cover = 0.5;
    p.seed = seed ? seed : 2;
    return true;
  case 3: {  // one database of the 64-database batch: per-database parameters from the seed
    Rng r(seed ? seed : 1000);
    double lg = std::log(1000.0) + r.uniform() * (std::log(50000.0) - std::log(1000.0));
    p.mode = 1; p.n_graphs = scaled((int64_t)std::llround(std::exp(lg)));
    p.n_vlabels = (int)r.range(2, 20); p.n_elabels = (int)r.range(2, 20);
    p.mean_edges = 10.0 + 30.0 * r.uniform();
    p.n_seeds = 50; p.seed_mean_edges = 4; p.seed_min_edges = 1; p.seed_cover = 0.5;
    p.seed = seed ? seed : 1000;
    return true;
  }
  case 4: {  // one of the 8 resident serving databases
    Rng r(seed ? seed : 2000);
    double lg = std::log(10000.0) + r.uniform() * (std::log(200000.0) - std::log(10000.0));
    p.mode = 1; p.n_graphs = scaled((int64_t)std::llround(std::exp(lg)));
    p.mean_edges = 30; p.n_vlabels = 5; p.n_elabels = 5;
    p.n_seeds = 50; p.seed_mean_edges = 4; p.seed_min_edges = 1; p.seed_cover = 0.5;
    p.seed = seed ? seed : 2000;
    return true;
  }
  case 5:  // large single database
    p.mode = 1; p.n_graphs = scaled(1000000); p.mean_edges = 40; p.n_vlabels = 10; p.vzipf = 1.2;
    p.n_elabels = 3; p.n_seeds = 200; p.seed_mean_edges = 5.5; p.seed_min_edges = 3; p.seed_max_edges = 8;
    p.seed_cover = 0.5; p.seed = seed ? seed : 5;
    return true;
  default:
    return false;
  }
}

}  // namespace gsgb
