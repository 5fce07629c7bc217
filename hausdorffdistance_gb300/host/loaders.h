// Point-set loaders and preprocessing for hd_exec, written for this engine
// without boost, rply or ITK.  Each follows the reference loader it stands in
// for (file:line given per function).  Points are returned as a flat
// row-major float array (n x dims), the layout the C ABI takes, and for
// -is_double also as doubles parsed from the same text (the reference's
// double instantiation of its loaders).
#pragma once
#include <dirent.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace hd {

struct PointSet {
  int dims = 0;
  std::vector<float> xyz;     // n * dims
  bool keep64 = false;        // also keep the coordinates as doubles
  std::vector<double> xyz64;  // n * dims when keep64
  size_t size() const { return dims ? xyz.size() / dims : 0; }
  void push(double v) {
    xyz.push_back((float) v);
    if (keep64) xyz64.push_back(v);
  }
};

inline void load_fail(const std::string& msg) { throw std::runtime_error(msg); }

// WKT (src/loaders/loader.h:26-147): one geometry per line; POINT,
// LINESTRING, MULTILINESTRING, POLYGON and MULTIPOLYGON contribute their
// vertices (polygons only their outer ring); GEOMETRYCOLLECTION lines are
// skipped; any other geometry is an error.  The first `dims` coordinates of
// each vertex are used.
inline PointSet LoadWKT(const std::string& path, int dims, size_t limit, bool keep64 = false) {
  std::ifstream ifs(path);
  if (!ifs) load_fail("cannot open " + path);
  PointSet ps;
  ps.dims = dims;
  ps.keep64 = keep64;
  std::string line;
  auto starts = [](const std::string& s, const char* p) { return s.rfind(p, 0) == 0; };
  while (std::getline(ifs, line) && ps.size() < limit) {
    size_t b = line.find_first_not_of(" \t\r");
    if (b == std::string::npos) continue;
    line = line.substr(b);
    // Depth (in parentheses) at which the vertex lists of the wanted rings
    // sit, and whether only the first ring of each enclosing group counts.
    int want_depth;
    bool outer_only = false;
    if (starts(line, "MULTIPOLYGON")) {
      want_depth = 3;
      outer_only = true;
    } else if (starts(line, "POLYGON")) {
      want_depth = 2;
      outer_only = true;
    } else if (starts(line, "MULTILINESTRING")) {
      want_depth = 2;
    } else if (starts(line, "LINESTRING") || starts(line, "POINT")) {
      want_depth = 1;
    } else if (starts(line, "GEOMETRYCOLLECTION")) {
      continue;
    } else {
      load_fail("unsupported WKT geometry in " + path + ": " + line.substr(0, 40));
    }
    int depth = 0;
    int ring_index = 0;  // index of the ring within its enclosing group
    std::vector<double> tuple;
    auto flush_tuple = [&]() {
      if (tuple.empty()) return;
      if ((int) tuple.size() < dims) load_fail("WKT vertex with too few coordinates in " + path);
      if (ps.size() < limit)
        for (int k = 0; k < dims; ++k) ps.push(tuple[k]);
      tuple.clear();
    };
    const char* p = line.c_str();
    while (*p) {
      const char ch = *p;
      if (ch == '(') {
        ++depth;
        if (depth == want_depth - 1) ring_index = 0;
        ++p;
      } else if (ch == ')') {
        if (depth == want_depth) {
          const bool take = !outer_only || ring_index == 0;
          if (take) flush_tuple();
          tuple.clear();
          ++ring_index;
        }
        --depth;
        ++p;
      } else if (ch == ',') {
        if (depth == want_depth && (!outer_only || ring_index == 0)) flush_tuple();
        tuple.clear();
        ++p;
      } else if (std::isdigit((unsigned char) ch) || ch == '-' || ch == '+' || ch == '.') {
        char* end = nullptr;
        const double v = std::strtod(p, &end);
        if (end == p) {
          ++p;
          continue;
        }
        if (depth == want_depth) tuple.push_back(v);
        p = end;
      } else {
        ++p;
      }
    }
  }
  return ps;
}

// OFF (src/loaders/loader.h:99-147): "OFF" header, counts on the same or the
// next line, then the vertices.  Like the reference, `dims` consecutive
// numbers are read per vertex.
inline PointSet LoadOFF(const std::string& path, int dims, size_t limit, bool keep64 = false) {
  std::ifstream ifs(path);
  if (!ifs) load_fail("cannot open " + path);
  std::string line;
  std::getline(ifs, line);
  if (line.substr(0, 3) != "OFF") load_fail("not an OFF file: " + path);
  line = line.substr(3);
  if (line.find_first_not_of(" \t\r") == std::string::npos) std::getline(ifs, line);
  std::istringstream hs(line);
  size_t nv = 0, nf = 0, ne = 0;
  hs >> nv >> nf >> ne;
  if (nv == 0) load_fail("OFF vertex count is zero or missing: " + path);
  PointSet ps;
  ps.dims = dims;
  ps.keep64 = keep64;
  for (size_t i = 0; i < nv && i < limit; ++i) {
    for (int k = 0; k < dims; ++k) {
      if (keep64) {
        // Each number parsed twice: directly to float (as the float
        // loader does) and to double.
        std::string tok;
        if (!(ifs >> tok)) load_fail("truncated OFF vertex list: " + path);
        char* end = nullptr;
        const float f = std::strtof(tok.c_str(), &end);
        if (end == tok.c_str()) load_fail("bad OFF coordinate in " + path);
        ps.xyz.push_back(f);
        ps.xyz64.push_back(std::strtod(tok.c_str(), nullptr));
      } else {
        float v;
        if (!(ifs >> v)) load_fail("truncated OFF vertex list: " + path);
        ps.xyz.push_back(v);
      }
    }
  }
  return ps;
}

// PLY (src/loaders/ply_loader.h:37-101): the x, y (, z) properties of the
// "vertex" element, ASCII or binary (either byte order), read as doubles,
// shifted so that the minimum of every axis is 0, then stored as float.
inline PointSet LoadPLY(const std::string& path, int dims, size_t limit, bool keep64 = false) {
  std::ifstream ifs(path, std::ios::binary);
  if (!ifs) load_fail("cannot open " + path);
  std::string line;
  std::getline(ifs, line);
  if (line.rfind("ply", 0) != 0) load_fail("not a PLY file: " + path);
  enum Fmt { kAscii, kLE, kBE } fmt = kAscii;
  struct Prop {
    std::string name, type;
    bool list = false;
    std::string count_type;
  };
  struct Elem {
    std::string name;
    size_t count = 0;
    std::vector<Prop> props;
  };
  std::vector<Elem> elems;
  while (std::getline(ifs, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    std::istringstream ls(line);
    std::string tok;
    ls >> tok;
    if (tok == "format") {
      std::string f;
      ls >> f;
      fmt = f == "ascii" ? kAscii : (f == "binary_little_endian" ? kLE : kBE);
    } else if (tok == "element") {
      Elem e;
      ls >> e.name >> e.count;
      elems.push_back(e);
    } else if (tok == "property") {
      if (elems.empty()) load_fail("PLY property before element: " + path);
      Prop pr;
      std::string t;
      ls >> t;
      if (t == "list") {
        pr.list = true;
        ls >> pr.count_type >> pr.type >> pr.name;
      } else {
        pr.type = t;
        ls >> pr.name;
      }
      elems.back().props.push_back(pr);
    } else if (tok == "end_header") {
      break;
    }
  }
  auto tsize = [](const std::string& t) -> int {
    if (t == "char" || t == "uchar" || t == "int8" || t == "uint8") return 1;
    if (t == "short" || t == "ushort" || t == "int16" || t == "uint16") return 2;
    if (t == "int" || t == "uint" || t == "float" || t == "int32" || t == "uint32" ||
        t == "float32")
      return 4;
    if (t == "double" || t == "float64") return 8;
    return 0;
  };
  auto read_bin = [&](const std::string& t) -> double {
    unsigned char buf[8];
    const int n = tsize(t);
    if (n == 0) load_fail("unsupported PLY type " + t);
    ifs.read((char*) buf, n);
    if (!ifs) load_fail("truncated PLY body: " + path);
    const bool host_le = [] {
      uint16_t x = 1;
      return *(unsigned char*) &x == 1;
    }();
    if ((fmt == kLE) != host_le) std::reverse(buf, buf + n);
    if (t == "char" || t == "int8") return (double) *(int8_t*) buf;
    if (t == "uchar" || t == "uint8") return (double) *(uint8_t*) buf;
    if (t == "short" || t == "int16") { int16_t v; std::memcpy(&v, buf, 2); return v; }
    if (t == "ushort" || t == "uint16") { uint16_t v; std::memcpy(&v, buf, 2); return v; }
    if (t == "int" || t == "int32") { int32_t v; std::memcpy(&v, buf, 4); return v; }
    if (t == "uint" || t == "uint32") { uint32_t v; std::memcpy(&v, buf, 4); return v; }
    if (t == "float" || t == "float32") { float v; std::memcpy(&v, buf, 4); return v; }
    double v;
    std::memcpy(&v, buf, 8);
    return v;
  };
  std::vector<double> verts;
  const char* names[3] = {"x", "y", "z"};
  for (const Elem& e : elems) {
    const bool is_vertex = e.name == "vertex";
    int col[3] = {-1, -1, -1};
    if (is_vertex)
      for (size_t i = 0; i < e.props.size(); ++i)
        for (int k = 0; k < dims; ++k)
          if (e.props[i].name == names[k]) col[k] = (int) i;
    if (is_vertex)
      for (int k = 0; k < dims; ++k)
        if (col[k] < 0) load_fail("PLY vertex lacks property " + std::string(names[k]));
    for (size_t r = 0; r < e.count; ++r) {
      double v[3] = {0, 0, 0};
      for (size_t i = 0; i < e.props.size(); ++i) {
        const Prop& pr = e.props[i];
        if (fmt == kAscii) {
          double x;
          if (pr.list) {
            size_t cnt;
            ifs >> cnt;
            for (size_t c = 0; c < cnt; ++c) ifs >> x;
            continue;
          }
          if (!(ifs >> x)) load_fail("truncated PLY body: " + path);
          for (int k = 0; k < dims; ++k)
            if ((int) i == col[k]) v[k] = x;
        } else {
          if (pr.list) {
            const size_t cnt = (size_t) read_bin(pr.count_type);
            for (size_t c = 0; c < cnt; ++c) read_bin(pr.type);
            continue;
          }
          const double x = read_bin(pr.type);
          for (int k = 0; k < dims; ++k)
            if ((int) i == col[k]) v[k] = x;
        }
      }
      if (is_vertex && verts.size() / dims < limit)
        for (int k = 0; k < dims; ++k) verts.push_back(v[k]);
    }
    if (is_vertex) break;  // later elements are not needed
  }
  PointSet ps;
  ps.dims = dims;
  ps.keep64 = keep64;
  const size_t n = verts.size() / dims;
  std::vector<double> lo(dims, std::numeric_limits<double>::max());
  for (size_t i = 0; i < n; ++i)
    for (int k = 0; k < dims; ++k) lo[k] = std::min(lo[k], verts[i * dims + k]);
  ps.xyz.resize(verts.size());
  if (keep64) ps.xyz64.resize(verts.size());
  for (size_t i = 0; i < n; ++i)
    for (int k = 0; k < dims; ++k) {
      const double v = verts[i * dims + k] - lo[k];
      ps.xyz[i * dims + k] = (float) v;
      if (keep64) ps.xyz64[i * dims + k] = v;
    }
  return ps;
}

// Point cache (src/loaders/loader.h:150-185): a 64-bit count followed by the
// packed points, floats, or doubles when keep64 (the reference's cache of
// its double instantiation).
inline PointSet LoadBin(const std::string& path, int dims, size_t limit, bool keep64 = false) {
  std::ifstream ifs(path, std::ios::binary);
  if (!ifs) load_fail("cannot open " + path);
  uint64_t n = 0;
  ifs.read((char*) &n, sizeof(n));
  n = std::min<uint64_t>(n, limit);
  PointSet ps;
  ps.dims = dims;
  ps.keep64 = keep64;
  ps.xyz.resize(n * dims);
  if (keep64) {
    ps.xyz64.resize(n * dims);
    ifs.read((char*) ps.xyz64.data(), (std::streamsize) (n * dims * sizeof(double)));
    for (size_t i = 0; i < ps.xyz64.size(); ++i) ps.xyz[i] = (float) ps.xyz64[i];
  } else {
    ifs.read((char*) ps.xyz.data(), (std::streamsize) (n * dims * sizeof(float)));
  }
  if (!ifs) load_fail("truncated point file: " + path);
  return ps;
}

inline void SaveBin(const std::string& path, const PointSet& ps) {
  std::ofstream ofs(path, std::ios::binary);
  if (!ofs) load_fail("cannot write " + path);
  const uint64_t n = ps.size();
  ofs.write((const char*) &n, sizeof(n));
  if (ps.keep64)
    ofs.write((const char*) ps.xyz64.data(), (std::streamsize) (ps.xyz64.size() * sizeof(double)));
  else
    ofs.write((const char*) ps.xyz.data(), (std::streamsize) (ps.xyz.size() * sizeof(float)));
}

// Loads with the reference's -serialize cache (loader.h:188-234): the cache
// file <folder>/points_<path with '/' as '_'>_limit_<limit>.bin is read when
// present, else written after loading (a separate "_f64" cache holds
// doubles).  type: wkt | off | ply | bin.
inline PointSet LoadPoints(const std::string& path, const std::string& type, int dims,
                           long long limit, const std::string& cache_folder,
                           bool keep64 = false) {
  const size_t lim = limit > 0 ? (size_t) limit : std::numeric_limits<size_t>::max();
  std::string cache;
  if (!cache_folder.empty() && type != "bin") {
    std::string esc = path;
    std::replace(esc.begin(), esc.end(), '/', '_');
    if (mkdir(cache_folder.c_str(), 0755) != 0 && errno != EEXIST)
      load_fail("cannot create " + cache_folder);
    cache = cache_folder + "/points_" + esc + "_limit_" + std::to_string(limit) +
            (keep64 ? "_f64" : "") + ".bin";
    if (access(cache.c_str(), R_OK) == 0) return LoadBin(cache, dims, lim, keep64);
  }
  PointSet ps;
  if (type == "wkt")
    ps = LoadWKT(path, dims, lim, keep64);
  else if (type == "off")
    ps = LoadOFF(path, dims, lim, keep64);
  else if (type == "ply")
    ps = LoadPLY(path, dims, lim, keep64);
  else if (type == "bin")
    ps = LoadBin(path, dims, lim, keep64);
  else
    load_fail("Unsupported input type: " + type);
  if (!cache.empty() && ps.size() > 0) SaveBin(cache, ps);
  return ps;
}

// The same preprocessing in double (keep64), the float copy re-rounded.
template <typename T>
inline void NormalizeRows(std::vector<T>& xyz, size_t n, int dims) {
  std::vector<T> lo(dims, std::numeric_limits<T>::max()), hi(dims, std::numeric_limits<T>::lowest());
  for (size_t i = 0; i < n; ++i)
    for (int k = 0; k < dims; ++k) {
      lo[k] = std::min(lo[k], xyz[i * dims + k]);
      hi[k] = std::max(hi[k], xyz[i * dims + k]);
    }
  T ext = 0;
  for (int k = 0; k < dims; ++k) ext = std::max(ext, hi[k] - lo[k]);
  if (ext == T(0)) ext = T(1);
  for (size_t i = 0; i < n; ++i)
    for (int k = 0; k < dims; ++k) xyz[i * dims + k] = (xyz[i * dims + k] - lo[k]) / ext;
}

// -normalize (translate_points.h:42-66): (x - min) / max extent per axis.
inline void NormalizePoints(PointSet& ps) {
  const size_t n = ps.size();
  if (n == 0) return;
  if (ps.keep64) {
    NormalizeRows(ps.xyz64, n, ps.dims);
    for (size_t i = 0; i < ps.xyz64.size(); ++i) ps.xyz[i] = (float) ps.xyz64[i];
    return;
  }
  NormalizeRows(ps.xyz, n, ps.dims);
}

// -translate (translate_points.h:68-79): shift axis `dim` by ratio x extent.
inline void TranslatePoints(PointSet& ps, int dim, double ratio) {
  const size_t n = ps.size();
  if (n == 0) return;
  if (ps.keep64) {
    double lo = std::numeric_limits<double>::max(), hi = std::numeric_limits<double>::lowest();
    for (size_t i = 0; i < n; ++i) {
      lo = std::min(lo, ps.xyz64[i * ps.dims + dim]);
      hi = std::max(hi, ps.xyz64[i * ps.dims + dim]);
    }
    const double shift = (hi - lo) * ratio;
    for (size_t i = 0; i < n; ++i) {
      ps.xyz64[i * ps.dims + dim] += shift;
      ps.xyz[i * ps.dims + dim] = (float) ps.xyz64[i * ps.dims + dim];
    }
    return;
  }
  float lo = std::numeric_limits<float>::max(), hi = std::numeric_limits<float>::lowest();
  for (size_t i = 0; i < n; ++i) {
    lo = std::min(lo, ps.xyz[i * ps.dims + dim]);
    hi = std::max(hi, ps.xyz[i * ps.dims + dim]);
  }
  const double shift = (double) (hi - lo) * ratio;
  for (size_t i = 0; i < n; ++i) ps.xyz[i * ps.dims + dim] += (float) shift;
}

}  // namespace hd
