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
  void push(double v) { push(v, (float) v); }
  // A coordinate parsed twice from text: f straight to float (correctly
  // rounded, as the reference's float loaders read it), v to double.
  void push(double v, float f) {
    xyz.push_back(f);
    if (keep64) xyz64.push_back(v);
  }
};

inline void load_fail(const std::string& msg) { throw std::runtime_error(msg); }

// WKT (src/loaders/loader.h:26-147): one geometry per line; POINT,
// LINESTRING, MULTILINESTRING, POLYGON and MULTIPOLYGON contribute their
// vertices (polygons only their outer ring); GEOMETRYCOLLECTION lines are
// skipped; any other geometry is an error.  The first `dims` coordinates of
// each vertex are used.  `limit` acts as in the reference, which tests it
// after each vertex it adds and then leaves only the innermost loop: a ring
// or linestring stops once the count reaches the limit, but every later one
// (the next polygon of a MULTIPOLYGON, the next line) still adds its first
// vertex; a POINT line that ends at or beyond the limit ends the file.
inline PointSet LoadWKT(const std::string& path, int dims, size_t limit, bool keep64 = false) {
  std::ifstream ifs(path);
  if (!ifs) load_fail("cannot open " + path);
  PointSet ps;
  ps.dims = dims;
  ps.keep64 = keep64;
  std::string line;
  auto starts = [](const std::string& s, const char* p) { return s.rfind(p, 0) == 0; };
  while (std::getline(ifs, line)) {
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
    int ring_index = 0;    // index of the ring within its enclosing group
    bool ring_full = false;  // this ring reached the limit: skip its rest
    std::vector<double> tuple;
    std::vector<float> tuple32;
    auto flush_tuple = [&]() {
      if (tuple.empty()) return;
      if ((int) tuple.size() < dims) load_fail("WKT vertex with too few coordinates in " + path);
      if (!ring_full) {
        for (int k = 0; k < dims; ++k) ps.push(tuple[k], tuple32[k]);
        ring_full = ps.size() >= limit;
      }
      tuple.clear();
      tuple32.clear();
    };
    const char* p = line.c_str();
    while (*p) {
      const char ch = *p;
      if (ch == '(') {
        ++depth;
        if (depth == want_depth - 1) ring_index = 0;
        if (depth == want_depth) ring_full = false;
        ++p;
      } else if (ch == ')') {
        if (depth == want_depth) {
          const bool take = !outer_only || ring_index == 0;
          if (take) flush_tuple();
          tuple.clear();
          tuple32.clear();
          ++ring_index;
        }
        --depth;
        ++p;
      } else if (ch == ',') {
        if (depth == want_depth && (!outer_only || ring_index == 0)) flush_tuple();
        tuple.clear();
        tuple32.clear();
        ++p;
      } else if (std::isdigit((unsigned char) ch) || ch == '-' || ch == '+' || ch == '.') {
        // boost.geometry's WKT reader (the reference's) converts each token
        // straight to the coordinate type: float directly, not via double.
        char* end = nullptr;
        const double v = std::strtod(p, &end);
        if (end == p) {
          ++p;
          continue;
        }
        if (depth == want_depth) {
          tuple.push_back(v);
          tuple32.push_back(std::strtof(p, nullptr));
        }
        p = end;
      } else {
        ++p;
      }
    }
    if (starts(line, "POINT") && ps.size() >= limit) break;
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
// `limit` keeps the first vertices.  (The reference's read callback returns
// 0 once its countdown reaches the limit, which aborts rply's read, so with a
// limit at or below the vertex count it loads no points at all and its driver
// stops on the empty set.)
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

// ---------------------------------------------------------------------------
// Images.  The reference reads them with ITK
// (src/loaders/img_loader.h:13-63: ImageFileReader<Image<unsigned char, N>>,
// then every voxel whose pixel is > 0 becomes the point of its index, index[0]
// fastest, until `limit` points).  ITK is not available here, so the header +
// raw formats are read directly: NIfTI-1 single files (.nii; the format of
// the reference's medical-image runs, expr/running_time.sh:132-160) and
// MetaImage (.mha with LOCAL data, .mhd with a raw file beside it).
namespace img {

enum class Elem { U8, I8, U16, I16, U32, I32, U64, I64, F32, F64 };

inline size_t elem_bytes(Elem e) {
  switch (e) {
    case Elem::U8: case Elem::I8: return 1;
    case Elem::U16: case Elem::I16: return 2;
    case Elem::U32: case Elem::I32: case Elem::F32: return 4;
    default: return 8;
  }
}

struct Volume {
  int ndim = 0;
  uint64_t size[8] = {1, 1, 1, 1, 1, 1, 1, 1};
  Elem elem = Elem::U8;
  bool swap = false;            // data in the other byte order than this host's
  std::string data_path;        // file holding the voxels
  uint64_t data_offset = 0;     // byte offset of the first voxel there
  bool rescale = false;         // NIfTI scl_slope / scl_inter in effect
  double slope = 1.0, inter = 0.0;
};

inline bool host_little_endian() {
  const uint16_t one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

// A real pixel value converted to unsigned char as a C++ static_cast does on
// the machines the reference ran on (truncation toward zero to a 32-bit
// integer, then its low byte); values outside the 32-bit range and NaN give 0.
inline uint8_t real_to_byte(double v) {
  if (!(v > -2147483649.0 && v < 2147483648.0)) return 0;
  return (uint8_t) (uint32_t) (int32_t) v;
}

// One voxel's value as ITK's reader hands it to the unsigned-char image: the
// stored value converted with a static_cast (integers keep their low byte).
// With a NIfTI rescale, ITK first scales into float (double for double data):
// value * slope + inter in double, rounded to the buffer type.
inline uint8_t voxel_byte(const unsigned char* p, const Volume& v) {
  unsigned char b[8];
  const size_t nb = elem_bytes(v.elem);
  for (size_t i = 0; i < nb; ++i) b[i] = v.swap ? p[nb - 1 - i] : p[i];
  double real = 0.0;
  uint64_t bits = 0;
  bool is_real = false;
  switch (v.elem) {
    case Elem::U8: bits = b[0]; real = b[0]; break;
    case Elem::I8: { int8_t x; std::memcpy(&x, b, 1); bits = (uint64_t) (int64_t) x; real = x; break; }
    case Elem::U16: { uint16_t x; std::memcpy(&x, b, 2); bits = x; real = x; break; }
    case Elem::I16: { int16_t x; std::memcpy(&x, b, 2); bits = (uint64_t) (int64_t) x; real = x; break; }
    case Elem::U32: { uint32_t x; std::memcpy(&x, b, 4); bits = x; real = x; break; }
    case Elem::I32: { int32_t x; std::memcpy(&x, b, 4); bits = (uint64_t) (int64_t) x; real = x; break; }
    case Elem::U64: { uint64_t x; std::memcpy(&x, b, 8); bits = x; real = (double) x; break; }
    case Elem::I64: { int64_t x; std::memcpy(&x, b, 8); bits = (uint64_t) x; real = (double) x; break; }
    case Elem::F32: { float x; std::memcpy(&x, b, 4); real = x; is_real = true; break; }
    case Elem::F64: { double x; std::memcpy(&x, b, 8); real = x; is_real = true; break; }
  }
  if (v.rescale) {
    // ITK rounds the product before adding the intercept; the volatile keeps
    // a compiler from fusing the two into one FMA.
    volatile double prod = (v.elem == Elem::F64 ? real : (double) (float) real) * v.slope;
    const double s = prod + v.inter;
    return real_to_byte(v.elem == Elem::F64 ? s : (double) (float) s);
  }
  return is_real ? real_to_byte(real) : (uint8_t) bits;
}

template <typename T>
inline T rd(const unsigned char* h, size_t off, bool swap) {
  unsigned char b[sizeof(T)];
  for (size_t i = 0; i < sizeof(T); ++i) b[i] = swap ? h[off + sizeof(T) - 1 - i] : h[off + i];
  T x;
  std::memcpy(&x, b, sizeof(T));
  return x;
}

// NIfTI-1 (the public nifti1.h layout): a 348-byte header, dim[] at byte 40,
// datatype at 70, vox_offset at 108, scl_slope/scl_inter at 112/116, magic
// "n+1" at 344 for a single file; either byte order (sizeof_hdr tells).
inline Volume ReadNifti(const std::string& path) {
  std::ifstream ifs(path, std::ios::binary);
  if (!ifs) load_fail("cannot open " + path);
  unsigned char h[348];
  ifs.read((char*) h, sizeof(h));
  if (!ifs) load_fail("truncated NIfTI header: " + path);
  if (h[0] == 0x1F && h[1] == 0x8B) load_fail("compressed images are not supported: " + path);
  Volume v;
  v.swap = rd<int32_t>(h, 0, false) != 348;
  if (v.swap && rd<int32_t>(h, 0, true) != 348)
    load_fail("not a NIfTI-1 file (sizeof_hdr != 348): " + path);
  if (std::memcmp(h + 344, "n+1", 4) != 0)
    load_fail("only single-file NIfTI-1 images (magic n+1) are supported: " + path);
  const int nd = rd<int16_t>(h, 40, v.swap);
  if (nd < 1 || nd > 7) load_fail("bad NIfTI dimension count: " + path);
  v.ndim = nd;
  for (int d = 0; d < nd; ++d) {
    const int s = rd<int16_t>(h, 42 + 2 * d, v.swap);
    if (s < 1) load_fail("bad NIfTI image size: " + path);
    v.size[d] = (uint64_t) s;
  }
  switch (rd<int16_t>(h, 70, v.swap)) {
    case 2: v.elem = Elem::U8; break;
    case 4: v.elem = Elem::I16; break;
    case 8: v.elem = Elem::I32; break;
    case 16: v.elem = Elem::F32; break;
    case 64: v.elem = Elem::F64; break;
    case 256: v.elem = Elem::I8; break;
    case 512: v.elem = Elem::U16; break;
    case 768: v.elem = Elem::U32; break;
    case 1024: v.elem = Elem::I64; break;
    case 1280: v.elem = Elem::U64; break;
    default: load_fail("unsupported NIfTI datatype (complex or RGB): " + path);
  }
  const float off = rd<float>(h, 108, v.swap);
  v.data_offset = off < 352.0f ? 352 : (uint64_t) off;
  const float slope = rd<float>(h, 112, v.swap), inter = rd<float>(h, 116, v.swap);
  // Rescaled when the slope is set (non-zero) and the pair is not the identity.
  v.rescale = std::isfinite(slope) && std::isfinite(inter) && slope != 0.0f &&
              (slope != 1.0f || inter != 0.0f);
  v.slope = slope;
  v.inter = inter;
  v.data_path = path;
  return v;
}

// MetaImage: "Key = Value" lines ending with ElementDataFile; LOCAL means the
// voxels follow that line (.mha), else they are in the named file beside the
// header (.mhd).  HeaderSize skips bytes at the start of the data.
inline Volume ReadMeta(const std::string& path) {
  std::ifstream ifs(path, std::ios::binary);
  if (!ifs) load_fail("cannot open " + path);
  Volume v;
  bool msb = false, have_type = false, have_file = false;
  std::string line, file;
  long long header_size = 0;
  int channels = 1;
  while (!have_file && std::getline(ifs, line)) {
    const size_t eq = line.find('=');
    if (eq == std::string::npos) continue;
    auto trim = [](std::string s) {
      const size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
      return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
    };
    const std::string key = trim(line.substr(0, eq)), val = trim(line.substr(eq + 1));
    std::string lval = val;
    for (char& ch : lval) ch = (char) std::tolower((unsigned char) ch);
    if (key == "NDims") {
      v.ndim = std::atoi(val.c_str());
      if (v.ndim < 1 || v.ndim > 8) load_fail("bad MetaImage NDims: " + path);
    } else if (key == "DimSize") {
      std::istringstream ss(val);
      for (int d = 0; d < 8; ++d) {
        long long s;
        if (!(ss >> s)) break;
        if (s < 1) load_fail("bad MetaImage DimSize: " + path);
        v.size[d] = (uint64_t) s;
      }
    } else if (key == "ElementType") {
      have_type = true;
      if (val == "MET_UCHAR") v.elem = Elem::U8;
      else if (val == "MET_CHAR") v.elem = Elem::I8;
      else if (val == "MET_USHORT") v.elem = Elem::U16;
      else if (val == "MET_SHORT") v.elem = Elem::I16;
      else if (val == "MET_UINT") v.elem = Elem::U32;
      else if (val == "MET_INT") v.elem = Elem::I32;
      else if (val == "MET_ULONG_LONG") v.elem = Elem::U64;
      else if (val == "MET_LONG_LONG") v.elem = Elem::I64;
      else if (val == "MET_FLOAT") v.elem = Elem::F32;
      else if (val == "MET_DOUBLE") v.elem = Elem::F64;
      else load_fail("unsupported MetaImage ElementType " + val + ": " + path);
    } else if (key == "BinaryDataByteOrderMSB" || key == "ElementByteOrderMSB") {
      msb = lval == "true";
    } else if (key == "CompressedData") {
      if (lval == "true") load_fail("compressed images are not supported: " + path);
    } else if (key == "BinaryData") {
      if (lval == "false") load_fail("ASCII MetaImage data is not supported: " + path);
    } else if (key == "ElementNumberOfChannels") {
      channels = std::atoi(val.c_str());
    } else if (key == "HeaderSize") {
      header_size = std::atoll(val.c_str());
    } else if (key == "ElementDataFile") {
      have_file = true;
      file = val;
    }
  }
  if (!have_file || !have_type || v.ndim == 0)
    load_fail("MetaImage header lacks NDims, ElementType or ElementDataFile: " + path);
  if (channels != 1) load_fail("multi-channel images are not supported: " + path);
  if (header_size < 0) load_fail("MetaImage HeaderSize -1 is not supported: " + path);
  v.swap = msb == host_little_endian() && elem_bytes(v.elem) > 1;
  if (file == "LOCAL") {
    v.data_path = path;
    v.data_offset = (uint64_t) ifs.tellg() + (uint64_t) header_size;
  } else {
    if (file == "LIST" || file.find('%') != std::string::npos)
      load_fail("MetaImage slice lists are not supported: " + path);
    const size_t slash = path.find_last_of('/');
    v.data_path = file[0] == '/' || slash == std::string::npos ? file
                                                                : path.substr(0, slash + 1) + file;
    v.data_offset = (uint64_t) header_size;
  }
  return v;
}

}  // namespace img

// Image inputs (src/loaders/img_loader.h:13-63): every voxel whose value,
// converted to unsigned char as ITK's reader converts pixel buffers (a
// static_cast; img::voxel_byte), is non-zero gives the point of its index,
// index 0 fastest, the first `limit` such voxels.  An image with fewer
// dimensions than `dims` has the missing indices 0 (ITK reads it as size 1
// there); extra dimensions must have size 1.
inline PointSet LoadImage(const std::string& path, int dims, size_t limit, bool keep64 = false) {
  std::string low = path;
  for (char& ch : low) ch = (char) std::tolower((unsigned char) ch);
  auto ends = [&](const char* s) {
    const size_t n = std::strlen(s);
    return low.size() >= n && low.compare(low.size() - n, n, s) == 0;
  };
  img::Volume v;
  if (ends(".nii"))
    v = img::ReadNifti(path);
  else if (ends(".mha") || ends(".mhd"))
    v = img::ReadMeta(path);
  else
    load_fail("unsupported image format (.nii, .mha or .mhd; compressed files are not read): " +
              path);
  for (int d = dims; d < v.ndim; ++d)
    if (v.size[d] != 1) load_fail("image has more than " + std::to_string(dims) + " dimensions: " + path);
  uint64_t count = 1;
  for (int d = 0; d < v.ndim; ++d) {
    if (v.size[d] > (uint64_t(1) << 40) / count) load_fail("image too large: " + path);
    count *= v.size[d];
  }
  const size_t eb = img::elem_bytes(v.elem);
  std::ifstream ifs(v.data_path, std::ios::binary);
  if (!ifs) load_fail("cannot open " + v.data_path);
  ifs.seekg((std::streamoff) v.data_offset);
  std::vector<unsigned char> raw(count * eb);
  ifs.read((char*) raw.data(), (std::streamsize) raw.size());
  if (!ifs) load_fail("truncated image data: " + v.data_path);
  PointSet ps;
  ps.dims = dims;
  ps.keep64 = keep64;
  const uint64_t sx = v.size[0], sy = v.ndim > 1 ? v.size[1] : 1;
  for (uint64_t i = 0; i < count && ps.size() < limit; ++i) {
    if (img::voxel_byte(&raw[i * eb], v) == 0) continue;
    const double idx[3] = {(double) (i % sx), (double) ((i / sx) % sy), (double) (i / (sx * sy))};
    for (int d = 0; d < dims; ++d) ps.push(d < 3 ? idx[d] : 0.0);
  }
  return ps;
}

// Loads with the reference's -serialize cache (loader.h:188-234): the cache
// file <folder>/points_<path with '/' as '_'>_limit_<limit>.bin is read when
// present, else written after loading (a separate "_f64" cache holds
// doubles).  type: wkt | off | ply | image | bin.  Like the reference
// (run_hausdorff_distance.cu:91-111), PLY and image inputs bypass the cache.
inline PointSet LoadPoints(const std::string& path, const std::string& type, int dims,
                           long long limit, const std::string& cache_folder,
                           bool keep64 = false) {
  const size_t lim = limit > 0 ? (size_t) limit : std::numeric_limits<size_t>::max();
  std::string cache;
  if (!cache_folder.empty() && (type == "wkt" || type == "off")) {
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
  else if (type == "image")
    ps = LoadImage(path, dims, lim, keep64);
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
    // Read through a volatile so the product is rounded before each add (no FMA).
    volatile double shift_v = (hi - lo) * ratio;
    const double shift = shift_v;
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
  // The reference adds the double product to the float coordinate
  // (`p += extent * ratio`): the sum is formed in double and rounded once.
  volatile double shift_v = (double) (hi - lo) * ratio;  // rounded before the adds (no FMA)
  const double shift = shift_v;
  for (size_t i = 0; i < n; ++i) {
    float& v = ps.xyz[i * ps.dims + dim];
    v = (float) ((double) v + shift);
  }
}

}  // namespace hd
