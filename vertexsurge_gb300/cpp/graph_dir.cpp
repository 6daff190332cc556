// Graph(dir).load(): the reference's on-disk graph directory into device CSR.
//
// Layout (the reference's Graph::load, storage/graph_store.cpp:48-73, and its
// names, meta/schema.cpp:36-66 and :160-205): schema.json describes the vertex
// types (with counts) and edge types (direction, edge count); every variable
// is a DiskArray file (storage/disk_array.hh:53, :330-352) — a 64-byte header
// whose first two int64 are the element count and element size, then the
// elements.  The CSR of a self edge type (src type == dst type) is
//   "{src}-{type}->{dst}_csr_src_dst" (+ "_index") and
//   "{dst}<-{type}-{src}_csr_dst_src" (+ "_index")   when directed,
//   "{src}-{type}-{dst}_csr_src_dst"  (+ "_index")   when undirected (both
// directions of every edge stored in it, meta/graph_loader.hh:64-66).
// The files are memory-mapped read-only, uploaded with vs_graph_upload and
// unmapped.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cctype>
#include <cstring>
#include <fstream>
#include <sstream>

#include "vs_operators.hh"

namespace vsgb {
namespace {

// ---- a small JSON reader (objects, arrays, strings, numbers, literals) ----
struct Json {
  enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
  bool b = false;
  double num = 0;
  std::string str;
  std::vector<Json> arr;
  std::vector<std::pair<std::string, Json>> obj;

  const Json &at(const std::string &k) const {
    if (kind == Obj)
      for (auto &kv : obj)
        if (kv.first == k) return kv.second;
    throw Error(VS_ERR_ARG, "schema.json: missing key \"" + k + "\"");
  }
  const Json *find(const std::string &k) const {
    if (kind == Obj)
      for (auto &kv : obj)
        if (kv.first == k) return &kv.second;
    return nullptr;
  }
};

class Parser {
  const std::string &s;
  size_t i = 0;
  [[noreturn]] void bad(const char *what) {
    throw Error(VS_ERR_ARG, std::string("schema.json: ") + what + " at offset " + std::to_string(i));
  }
  void ws() {
    while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
  }
  std::string string_lit() {
    if (s[i] != '"') bad("expected a string");
    i++;
    std::string out;
    while (i < s.size() && s[i] != '"') {
      char c = s[i++];
      if (c == '\\') {
        if (i >= s.size()) bad("bad escape");
        char e = s[i++];
        switch (e) {
          case 'n': out += '\n'; break;
          case 't': out += '\t'; break;
          case 'r': out += '\r'; break;
          case 'b': out += '\b'; break;
          case 'f': out += '\f'; break;
          case 'u': {  // names here are ASCII; keep BMP code points below 0x80, else '?'
            if (i + 4 > s.size()) bad("bad \\u escape");
            unsigned v = (unsigned)std::stoul(s.substr(i, 4), nullptr, 16);
            i += 4;
            out += v < 0x80 ? (char)v : '?';
            break;
          }
          default: out += e;
        }
      } else {
        out += c;
      }
    }
    if (i >= s.size()) bad("unterminated string");
    i++;
    return out;
  }

 public:
  explicit Parser(const std::string &src) : s(src) {}
  Json value() {
    ws();
    if (i >= s.size()) bad("unexpected end");
    Json j;
    char c = s[i];
    if (c == '{') {
      j.kind = Json::Obj;
      i++;
      ws();
      if (s[i] == '}') {
        i++;
        return j;
      }
      for (;;) {
        ws();
        std::string k = string_lit();
        ws();
        if (s[i] != ':') bad("expected ':'");
        i++;
        j.obj.emplace_back(k, value());
        ws();
        if (s[i] == ',') {
          i++;
          continue;
        }
        if (s[i] == '}') {
          i++;
          return j;
        }
        bad("expected ',' or '}'");
      }
    }
    if (c == '[') {
      j.kind = Json::Arr;
      i++;
      ws();
      if (s[i] == ']') {
        i++;
        return j;
      }
      for (;;) {
        j.arr.push_back(value());
        ws();
        if (s[i] == ',') {
          i++;
          continue;
        }
        if (s[i] == ']') {
          i++;
          return j;
        }
        bad("expected ',' or ']'");
      }
    }
    if (c == '"') {
      j.kind = Json::Str;
      j.str = string_lit();
      return j;
    }
    if (!s.compare(i, 4, "true")) {
      j.kind = Json::Bool;
      j.b = true;
      i += 4;
      return j;
    }
    if (!s.compare(i, 5, "false")) {
      j.kind = Json::Bool;
      i += 5;
      return j;
    }
    if (!s.compare(i, 4, "null")) {
      i += 4;
      return j;
    }
    size_t end = i;
    while (end < s.size() && (std::isdigit((unsigned char)s[end]) || std::strchr("+-.eE", s[end]))) end++;
    if (end == i) bad("unexpected character");
    j.kind = Json::Num;
    j.num = std::stod(s.substr(i, end - i));
    i = end;
    return j;
  }
};

// ---- DiskArray files ----
struct Mapped {
  void *base = nullptr;
  size_t bytes = 0;
  int64_t count = 0;
  const void *data() const { return static_cast<const char *>(base) + 64; }
  ~Mapped() {
    if (base) munmap(base, bytes);
  }
};

void map_disk_array(const std::filesystem::path &p, size_t elem, Mapped &m) {
  int fd = open(p.c_str(), O_RDONLY);
  if (fd < 0) throw Error(VS_ERR_ARG, "cannot open " + p.string());
  struct stat st {};
  if (fstat(fd, &st) != 0 || (size_t)st.st_size < 64) {
    close(fd);
    throw Error(VS_ERR_ARG, p.string() + ": shorter than the DiskArray header");
  }
  m.bytes = (size_t)st.st_size;
  m.base = mmap(nullptr, m.bytes, PROT_READ, MAP_SHARED, fd, 0);
  close(fd);
  if (m.base == MAP_FAILED) {
    m.base = nullptr;
    throw Error(VS_ERR_ARG, "cannot map " + p.string());
  }
  int64_t hdr[2];
  std::memcpy(hdr, m.base, sizeof(hdr));
  m.count = hdr[0];
  if (hdr[1] != (int64_t)elem)
    throw Error(VS_ERR_ARG, p.string() + ": element size " + std::to_string(hdr[1]) + ", expected " +
                                std::to_string(elem));
  if (m.count < 0 || 64 + (size_t)m.count * elem > m.bytes)
    throw Error(VS_ERR_ARG, p.string() + ": element count does not fit the file");
}

}  // namespace

std::string forward_edge_name(const TypeName &src, const TypeName &e, const TypeName &dst, bool directed) {
  return directed ? src + "-" + e + "->" + dst : src + "-" + e + "-" + dst;
}

std::string backward_edge_name(const TypeName &src, const TypeName &e, const TypeName &dst, bool directed) {
  return directed ? dst + "<-" + e + "-" + src : dst + "-" + e + "-" + src;
}

namespace {

// CSR (offsets, targets sorted per list) of the edges from[i] -> to[i].
void csr_of_pairs(size_t V, const std::vector<uint32_t> &from, const std::vector<uint32_t> &to,
                  std::vector<int64_t> &off, std::vector<uint32_t> &adj) {
  off.assign(V + 1, 0);
  for (uint32_t a : from) {
    if (a >= V) throw Error(VS_ERR_ARG, "flat edge list: vertex id out of range");
    off[a + 1]++;
  }
  for (size_t v = 0; v < V; v++) off[v + 1] += off[v];
  adj.assign(from.size(), 0);
  std::vector<int64_t> cur(off.begin(), off.end() - 1);
  for (size_t i = 0; i < from.size(); i++) adj[cur[from[i]]++] = to[i];
  for (size_t v = 0; v < V; v++) std::sort(adj.begin() + off[v], adj.begin() + off[v + 1]);
}

// The forward flat edge list of an edge type (its first unpartitioned order,
// else the blocks of its first partitioned order), as (src, dst) columns:
// the reference's flat files are VIDPair DiskArrays named
// "{edge name}_{order}[_{block}]" (meta/schema.cpp:69-97,
// meta/graph_loader.hh:202-276).
bool read_forward_flat(const std::filesystem::path &dir, const Json &e, const std::string &edge_name,
                       std::vector<uint32_t> &src, std::vector<uint32_t> &dst) {
  const Json *info = e.find("store_info");
  if (!info) return false;
  std::vector<std::string> files;
  const Json *flats = info->find("flats");
  const Json *parts = info->find("partitioned_flats");
  const Json *counts = info->find("partition_counts");
  if (flats && !flats->arr.empty()) {
    files.push_back(edge_name + "_" + flats->arr[0].str);
  } else if (parts && counts && !parts->arr.empty() && !counts->arr.empty()) {
    for (size_t i = 0; i < (size_t)counts->arr[0].num; i++)
      files.push_back(edge_name + "_" + parts->arr[0].str + "_" + std::to_string(i));
  } else {
    return false;
  }
  for (const std::string &name : files) {
    Mapped m;
    map_disk_array(dir / name, 2 * sizeof(uint32_t), m);
    const uint32_t *p = static_cast<const uint32_t *>(m.data());
    for (int64_t i = 0; i < m.count; i++) {
      src.push_back(p[2 * i]);
      dst.push_back(p[2 * i + 1]);
    }
  }
  return true;
}

}  // namespace

void Graph::load_dir() {
  std::ifstream f(dir / "schema.json");
  if (!f) throw Error(VS_ERR_ARG, "no schema.json in " + dir.string());
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string text = ss.str();
  Json schema = Parser(text).value();
  for (const Json &v : schema.at("vertex").arr) {
    const TypeName vt = v.at("type").str;
    const size_t n = (size_t)v.at("statistics").at("count").num;
    add_vertex_type(vt, n);
    // properties ("Type.name" DiskArray files, Graph::load's variable table, meta/schema.cpp:160-168)
    for (const auto &kv : v.at("properties").obj) {
      const std::string ty = kv.second.at("type").str;
      const size_t bytes = ty == "TagValue8" ? 1 : ty == "TagValue16" ? 2 : (ty == "VID" || ty == "Int32") ? 4
                         : ty == "Int64" ? 8 : 0;
      if (!bytes) continue;  // strings and pairs are not vertex filters of the path
      const std::filesystem::path f = dir / (vt + "." + kv.first);
      if (!std::filesystem::exists(f)) continue;
      Mapped m;
      map_disk_array(f, bytes, m);
      std::vector<uint64_t> vals((size_t)m.count);
      const unsigned char *p = static_cast<const unsigned char *>(m.data());
      for (size_t i = 0; i < vals.size(); i++) {
        if (bytes == 1) vals[i] = p[i];
        else if (bytes == 2) vals[i] = reinterpret_cast<const uint16_t *>(p)[i];
        else if (bytes == 4) vals[i] = reinterpret_cast<const uint32_t *>(p)[i];
        else vals[i] = (uint64_t)reinterpret_cast<const int64_t *>(p)[i];
      }
      add_vertex_property(vt + "." + kv.first, vals, bytes == 8 ? Type::Int64 : Type::VID);
    }
  }
  for (const Json &e : schema.at("edge").arr) {
    const TypeName src = e.at("src").str, dst = e.at("dst").str, type = e.at("type").str;
    const bool directed = e.at("directed").b;
    if (src != dst) continue;  // the expand runs over one vertex id space
    const uint64_t E = (uint64_t)e.at("statistics").at("count").num;
    const size_t V = vertex_count.at(src);
    const std::string fwd = forward_edge_name(src, type, dst, directed) + "_csr_src_dst";
    if (!std::filesystem::exists(dir / (fwd + "_index"))) {  // no CSR files: build them from a flat list
      std::vector<uint32_t> s, d;
      if (!read_forward_flat(dir, e, forward_edge_name(src, type, dst, directed), s, d))
        throw Error(VS_ERR_ARG, "edge type " + src + "_" + type + "_" + dst + ": neither CSR files nor flat edge lists");
      if (s.size() != E)
        throw Error(VS_ERR_ARG, "edge type " + src + "_" + type + "_" + dst + ": flat edge list length " +
                                    std::to_string(s.size()) + ", expected " + std::to_string(E));
      std::vector<int64_t> fo, ro;
      std::vector<uint32_t> fa, ra;
      csr_of_pairs(V, s, d, fo, fa);
      if (directed)
        csr_of_pairs(V, d, s, ro, ra);
      add_edge_type(src, type, dst, directed, (uint32_t)V, E, fo.data(), fa.data(),
                    directed ? ro.data() : fo.data(), directed ? ra.data() : fa.data());
      continue;
    }
    Mapped fi, fd, bi, bd;
    map_disk_array(dir / (fwd + "_index"), sizeof(int64_t), fi);
    map_disk_array(dir / fwd, sizeof(uint32_t), fd);
    const Mapped *ri = &fi, *rd = &fd;
    if (directed) {
      const std::string bwd = backward_edge_name(src, type, dst, directed) + "_csr_dst_src";
      map_disk_array(dir / (bwd + "_index"), sizeof(int64_t), bi);
      map_disk_array(dir / bwd, sizeof(uint32_t), bd);
      ri = &bi;
      rd = &bd;
    }
    for (const Mapped *idx : {(const Mapped *)&fi, ri})
      if ((size_t)idx->count != V + 1)
        throw Error(VS_ERR_ARG, "edge type " + src + "_" + type + "_" + dst + ": CSR index length " +
                                    std::to_string(idx->count) + ", expected " + std::to_string(V + 1));
    for (const Mapped *dat : {(const Mapped *)&fd, rd})
      if ((uint64_t)dat->count != E)
        throw Error(VS_ERR_ARG, "edge type " + src + "_" + type + "_" + dst + ": CSR data length " +
                                    std::to_string(dat->count) + ", expected " + std::to_string(E));
    add_edge_type(src, type, dst, directed, (uint32_t)V, E, static_cast<const int64_t *>(fi.data()),
                  static_cast<const uint32_t *>(fd.data()), static_cast<const int64_t *>(ri->data()),
                  static_cast<const uint32_t *>(rd->data()));
  }
}

}  // namespace vsgb
