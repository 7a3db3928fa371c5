// rtg_vtk.cpp -- VTK XML files without VTK: the result writer and the surface
// readers of rti's io layer.
//
// Writer (rti io/vtp_writer.hpp:27-139, 392-413): ASCII PolyData, as rti's
// writer produces with SetDataModeToAscii.  Discs: the centres as points, one
// vertex cell per disc, cell arrays Normals (3 components), radius, value (S1),
// exposed-area, hitcnt, relative-error, variance-of-variance.  Triangles: the
// vertices as points, one polygon cell per triangle, the same result arrays
// without normals and radius.  Metadata: one string array per (key, value) in
// the field data.  Cell i is primitive i (discs first, then triangles).
//
// Readers (rti io/vtp_point_cloud_reader.hpp:23-95, io/vtp_triangle_reader.hpp:
// 19-68): PolyData or UnstructuredGrid pieces, DataArrays in ascii, inline
// binary (base64) or appended (raw or base64) form, uncompressed or zlib
// compressed (when built with zlib).  Point clouds: points, the cell "radius"
// array, else "sqrt-of-area" * sqrt(3)/2 * (1 + 1/32), and the cell normals
// (normalised when their length is off by more than 1e-6).  Triangles: points
// and every three-point polygon (PolyData) or triangle cell (UnstructuredGrid).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <new>
#include <stdexcept>
#include <sstream>
#include <string>
#include <vector>

#if defined(__has_include)
#if __has_include(<zlib.h>) && defined(RTG_WITH_ZLIB)
#include <zlib.h>
#define RTG_HAVE_ZLIB 1
#endif
#endif

#include "rtg.h"

namespace {

// ---------------------------------------------------------------- writing --

struct Out {
  FILE* f = nullptr;
  bool ok = true;
  void put(const char* s) {
    if (ok && std::fputs(s, f) < 0) ok = false;
  }
  void fmt(const char* format, ...) __attribute__((format(printf, 2, 3)));
};

void Out::fmt(const char* format, ...) {
  if (!ok) return;
  va_list ap;
  va_start(ap, format);
  if (std::vfprintf(f, format, ap) < 0) ok = false;
  va_end(ap);
}

std::string xml_escape(const char* s) {
  std::string o;
  for (; *s; ++s) {
    switch (*s) {
      case '&': o += "&amp;"; break;
      case '<': o += "&lt;"; break;
      case '>': o += "&gt;"; break;
      case '"': o += "&quot;"; break;
      default: o += *s;
    }
  }
  return o;
}

template <typename Get>
void data_array(Out& o, const char* type, const char* name, int ncomp, int64_t n, const char* numfmt, Get get) {
  o.fmt("        <DataArray type=\"%s\"", type);
  if (name) o.fmt(" Name=\"%s\"", name);
  if (ncomp != 1) o.fmt(" NumberOfComponents=\"%d\"", ncomp);
  o.put(" format=\"ascii\">\n");
  const int64_t total = n * ncomp;
  for (int64_t i = 0; i < total; ++i) {
    if (i % 6 == 0) o.put("          ");
    o.fmt(numfmt, get(i));
    o.put((i % 6 == 5 || i == total - 1) ? "\n" : " ");
  }
  o.put("        </DataArray>\n");
}

struct Results {
  const double* value;
  const uint64_t* hitcnt;
  const float* area;
  const double* relerr;
  const double* vov;
};

void result_arrays(Out& o, int64_t n, const Results& r) {
  if (r.value) data_array(o, "Float64", "value", 1, n, "%.17g", [&](int64_t i) { return r.value[i]; });
  if (r.area) data_array(o, "Float64", "exposed-area", 1, n, "%.9g", [&](int64_t i) { return (double)r.area[i]; });
  if (r.hitcnt)
    data_array(o, "UInt64", "hitcnt", 1, n, "%llu", [&](int64_t i) { return (unsigned long long)r.hitcnt[i]; });
  if (r.relerr) data_array(o, "Float64", "relative-error", 1, n, "%.17g", [&](int64_t i) { return r.relerr[i]; });
  if (r.vov) data_array(o, "Float64", "variance-of-variance", 1, n, "%.17g", [&](int64_t i) { return r.vov[i]; });
}

void field_data(Out& o, const char* const* keys, const char* const* values, int32_t n_meta) {
  if (n_meta <= 0) return;
  o.put("    <FieldData>\n");
  for (int32_t m = 0; m < n_meta; ++m) {
    const char* k = keys[m] ? keys[m] : "";
    const char* v = values[m] ? values[m] : "";
    o.fmt("      <Array type=\"String\" Name=\"%s\" NumberOfTuples=\"1\" format=\"ascii\">\n        ",
          xml_escape(k).c_str());
    for (const unsigned char* c = (const unsigned char*)v; *c; ++c) o.fmt("%u ", (unsigned)*c);
    o.put("0\n      </Array>\n");
  }
  o.put("    </FieldData>\n");
}

// One PolyData piece holding nd discs (vertex cells) and nt triangles
// (polygon cells); arrays indexed by primitive id.
int write_polydata(const char* path, int64_t nd, const float* pts, const float* nrm, const float* rad, int64_t nv,
                   const float* vtx, int64_t nt, const uint32_t* idx, const Results& r, const char* const* keys,
                   const char* const* values, int32_t n_meta) {
  if (!path || nd < 0 || nv < 0 || nt < 0 || (nd > 0 && (!pts || !nrm || !rad)) || (nt > 0 && (!vtx || !idx)) ||
      (n_meta > 0 && (!keys || !values)))
    return RTG_ERR_INVALID_ARGUMENT;
  for (int64_t t = 0; t < 3 * nt; ++t)
    if ((int64_t)idx[t] >= nv) return RTG_ERR_INVALID_ARGUMENT;
  Out o;
  o.f = std::fopen(path, "w");
  if (!o.f) return RTG_ERR_INVALID_ARGUMENT;
  const int64_t np = nd + nt;
  o.put("<?xml version=\"1.0\"?>\n");
  o.put("<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n");
  o.put("  <PolyData>\n");
  field_data(o, keys, values, n_meta);
  o.fmt("    <Piece NumberOfPoints=\"%lld\" NumberOfVerts=\"%lld\" NumberOfLines=\"0\" NumberOfStrips=\"0\" "
        "NumberOfPolys=\"%lld\">\n",
        (long long)(nd + nv), (long long)nd, (long long)nt);
  o.put("      <PointData>\n      </PointData>\n");
  o.put(nd > 0 ? "      <CellData Normals=\"Normals\">\n" : "      <CellData>\n");
  if (nd > 0) {
    // triangles (if any) carry their unit normals, from the cross product
    data_array(o, "Float64", "Normals", 3, np, "%.9g", [&](int64_t i) -> double {
      const int64_t c = i / 3, a = i % 3;
      if (c < nd) return nrm[3 * c + a];
      const uint32_t* t = idx + 3 * (c - nd);
      double e1[3], e2[3];
      for (int q = 0; q < 3; ++q) {
        e1[q] = (double)vtx[3 * t[1] + q] - vtx[3 * t[0] + q];
        e2[q] = (double)vtx[3 * t[2] + q] - vtx[3 * t[0] + q];
      }
      const double n3[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                            e1[0] * e2[1] - e1[1] * e2[0]};
      const double l = std::sqrt(n3[0] * n3[0] + n3[1] * n3[1] + n3[2] * n3[2]);
      return l > 0.0 ? n3[a] / l : 0.0;
    });
    data_array(o, "Float64", "radius", 1, np, "%.9g",
               [&](int64_t i) { return i < nd ? (double)rad[i] : 0.0; });
  }
  result_arrays(o, np, r);
  o.put("      </CellData>\n");
  o.put("      <Points>\n");
  data_array(o, "Float32", "Points", 3, nd + nv, "%.9g",
             [&](int64_t i) { return (double)(i < 3 * nd ? pts[i] : vtx[i - 3 * nd]); });
  o.put("      </Points>\n");
  o.put("      <Verts>\n");
  data_array(o, "Int64", "connectivity", 1, nd, "%lld", [&](int64_t i) { return (long long)i; });
  data_array(o, "Int64", "offsets", 1, nd, "%lld", [&](int64_t i) { return (long long)(i + 1); });
  o.put("      </Verts>\n");
  o.put("      <Lines>\n");
  data_array(o, "Int64", "connectivity", 1, 0, "%lld", [&](int64_t) { return 0LL; });
  data_array(o, "Int64", "offsets", 1, 0, "%lld", [&](int64_t) { return 0LL; });
  o.put("      </Lines>\n");
  o.put("      <Strips>\n");
  data_array(o, "Int64", "connectivity", 1, 0, "%lld", [&](int64_t) { return 0LL; });
  data_array(o, "Int64", "offsets", 1, 0, "%lld", [&](int64_t) { return 0LL; });
  o.put("      </Strips>\n");
  o.put("      <Polys>\n");
  data_array(o, "Int64", "connectivity", 1, 3 * nt, "%lld",
             [&](int64_t i) { return (long long)(nd + (int64_t)idx[i]); });
  data_array(o, "Int64", "offsets", 1, nt, "%lld", [&](int64_t i) { return (long long)(3 * (i + 1)); });
  o.put("      </Polys>\n");
  o.put("    </Piece>\n  </PolyData>\n</VTKFile>\n");
  const bool ok = o.ok;
  if (std::fclose(o.f) != 0 || !ok) return RTG_ERR_INTERNAL;
  return RTG_OK;
}

// ---------------------------------------------------------------- reading --

struct DataArray {
  std::string name, type, format;
  int ncomp = 1;
  int64_t offset = -1;
  std::string text;  // inline content
  std::vector<double> v;
};

struct Piece {
  bool unstructured = false;
  int64_t npoints = 0;
  std::vector<DataArray> arrays;  // in document order, with their section
  std::vector<std::string> section;
  std::string cell_normals;       // CellData Normals="..." attribute
};

struct Doc {
  std::string byte_order = "LittleEndian", header_type = "UInt32", compressor;
  std::string appended_encoding;
  size_t appended_start = std::string::npos;  // first byte after '_'
  Piece piece;
};

void attrs(const std::string& tag, std::vector<std::pair<std::string, std::string>>& out) {
  out.clear();
  size_t i = 0;
  while (i < tag.size() && !std::isspace((unsigned char)tag[i])) ++i;  // element name
  while (i < tag.size()) {
    while (i < tag.size() && (std::isspace((unsigned char)tag[i]) || tag[i] == '/')) ++i;
    size_t k0 = i;
    while (i < tag.size() && tag[i] != '=' && !std::isspace((unsigned char)tag[i])) ++i;
    std::string key = tag.substr(k0, i - k0);
    while (i < tag.size() && tag[i] != '=') ++i;
    if (i >= tag.size()) break;
    ++i;
    while (i < tag.size() && std::isspace((unsigned char)tag[i])) ++i;
    if (i >= tag.size() || (tag[i] != '"' && tag[i] != '\'')) break;
    const char q = tag[i++];
    size_t v0 = i;
    while (i < tag.size() && tag[i] != q) ++i;
    out.emplace_back(key, tag.substr(v0, i - v0));
    ++i;
  }
}

std::string get(const std::vector<std::pair<std::string, std::string>>& a, const char* key) {
  for (auto& kv : a)
    if (kv.first == key) return kv.second;
  return std::string();
}

bool parse_xml(const std::string& s, Doc& doc, std::string& err) {
  const size_t app = s.find("<AppendedData");
  const size_t xml_end = app == std::string::npos ? s.size() : app;
  if (app != std::string::npos) {
    const size_t gt = s.find('>', app);
    if (gt == std::string::npos) return err = "malformed AppendedData", false;
    std::vector<std::pair<std::string, std::string>> a;
    attrs(s.substr(app + 1, gt - app - 1), a);
    doc.appended_encoding = get(a, "encoding");
    const size_t us = s.find('_', gt);
    if (us == std::string::npos) return err = "AppendedData without '_'", false;
    doc.appended_start = us + 1;
  }
  std::vector<std::string> stack;
  std::vector<std::pair<std::string, std::string>> a;
  bool in_piece = false;
  size_t i = 0;
  while (i < xml_end) {
    const size_t lt = s.find('<', i);
    if (lt == std::string::npos || lt >= xml_end) break;
    if (s.compare(lt, 4, "<!--") == 0) {
      const size_t e = s.find("-->", lt);
      i = e == std::string::npos ? xml_end : e + 3;
      continue;
    }
    if (s.compare(lt, 2, "<?") == 0) {
      const size_t e = s.find("?>", lt);
      i = e == std::string::npos ? xml_end : e + 2;
      continue;
    }
    const size_t gt = s.find('>', lt);
    if (gt == std::string::npos) return err = "malformed XML", false;
    std::string tag = s.substr(lt + 1, gt - lt - 1);
    i = gt + 1;
    if (!tag.empty() && tag[0] == '/') {
      if (!stack.empty()) stack.pop_back();
      continue;
    }
    const bool self_close = !tag.empty() && tag.back() == '/';
    size_t ne = 0;
    while (ne < tag.size() && !std::isspace((unsigned char)tag[ne]) && tag[ne] != '/') ++ne;
    const std::string name = tag.substr(0, ne);
    attrs(tag, a);
    if (name == "VTKFile") {
      const std::string t = get(a, "type");
      if (t != "PolyData" && t != "UnstructuredGrid") return err = "unsupported VTKFile type " + t, false;
      doc.piece.unstructured = t == "UnstructuredGrid";
      if (!get(a, "byte_order").empty()) doc.byte_order = get(a, "byte_order");
      if (!get(a, "header_type").empty()) doc.header_type = get(a, "header_type");
      doc.compressor = get(a, "compressor");
    } else if (name == "Piece") {
      if (in_piece) return err = "files with more than one piece are not supported", false;
      in_piece = true;
      doc.piece.npoints = std::atoll(get(a, "NumberOfPoints").c_str());
    } else if (name == "CellData") {
      doc.piece.cell_normals = get(a, "Normals");
    } else if (name == "DataArray" || name == "Array") {
      DataArray d;
      d.name = get(a, "Name");
      d.type = get(a, "type");
      d.format = get(a, "format");
      if (!get(a, "NumberOfComponents").empty()) d.ncomp = std::atoi(get(a, "NumberOfComponents").c_str());
      if (!get(a, "offset").empty()) d.offset = std::atoll(get(a, "offset").c_str());
      if (!self_close) {
        const size_t close = s.find(name == "Array" ? "</Array>" : "</DataArray>", i);
        if (close == std::string::npos) return err = "unterminated DataArray", false;
        d.text = s.substr(i, close - i);
        i = close;
      }
      doc.piece.section.push_back(stack.empty() ? std::string() : stack.back());
      doc.piece.arrays.push_back(std::move(d));
    }
    if (!self_close) stack.push_back(name);
  }
  if (!in_piece) return err = "no Piece element", false;
  return true;
}

int b64val(char c) {
  if (c >= 'A' && c <= 'Z') return c - 'A';
  if (c >= 'a' && c <= 'z') return c - 'a' + 26;
  if (c >= '0' && c <= '9') return c - '0' + 52;
  if (c == '+') return 62;
  if (c == '/') return 63;
  return -1;
}

// Decodes base64 characters [p, p+n) (whitespace skipped); stops at padding.
std::vector<unsigned char> b64(const char* p, size_t n, size_t* used = nullptr) {
  std::vector<unsigned char> out;
  uint32_t acc = 0;
  int bits = 0;
  size_t i = 0;
  for (; i < n; ++i) {
    const char c = p[i];
    if (c == '=') {
      while (i < n && (p[i] == '=' || std::isspace((unsigned char)p[i]))) ++i;
      break;
    }
    const int v = b64val(c);
    if (v < 0) continue;
    acc = (acc << 6) | (uint32_t)v;
    bits += 6;
    if (bits >= 8) {
      bits -= 8;
      out.push_back((unsigned char)((acc >> bits) & 0xFF));
    }
  }
  if (used) *used = i;
  return out;
}

size_t type_size(const std::string& t) {
  if (t == "Int8" || t == "UInt8" || t == "Char" || t == "String") return 1;
  if (t == "Int16" || t == "UInt16") return 2;
  if (t == "Int32" || t == "UInt32" || t == "Float32") return 4;
  if (t == "Int64" || t == "UInt64" || t == "Float64") return 8;
  return 0;
}

double load_value(const unsigned char* p, const std::string& t, bool swap) {
  unsigned char b[8];
  const size_t n = type_size(t);
  for (size_t i = 0; i < n; ++i) b[i] = swap ? p[n - 1 - i] : p[i];
  if (t == "Float32") { float v; std::memcpy(&v, b, 4); return v; }
  if (t == "Float64") { double v; std::memcpy(&v, b, 8); return v; }
  if (t == "Int8") { int8_t v; std::memcpy(&v, b, 1); return v; }
  if (t == "UInt8" || t == "Char" || t == "String") { uint8_t v; std::memcpy(&v, b, 1); return v; }
  if (t == "Int16") { int16_t v; std::memcpy(&v, b, 2); return v; }
  if (t == "UInt16") { uint16_t v; std::memcpy(&v, b, 2); return v; }
  if (t == "Int32") { int32_t v; std::memcpy(&v, b, 4); return v; }
  if (t == "UInt32") { uint32_t v; std::memcpy(&v, b, 4); return v; }
  if (t == "Int64") { int64_t v; std::memcpy(&v, b, 8); return (double)v; }
  uint64_t v;
  std::memcpy(&v, b, 8);
  return (double)v;
}

bool host_little() {
  const uint16_t x = 1;
  unsigned char c;
  std::memcpy(&c, &x, 1);
  return c == 1;
}

// Reads header word k of a binary block header.
// Header word k (hs = 4 or 8 bytes), read as an integer straight from the
// bytes (through a double, sizes above 2^53 would round and some wrap).
uint64_t header_word(const std::vector<unsigned char>& h, size_t k, size_t hs, bool swap) {
  const unsigned char* p = h.data() + k * hs;
  const bool big = host_little() ? swap : !swap;  // the file's byte order
  uint64_t v = 0;
  for (size_t i = 0; i < hs; ++i) v |= (uint64_t)p[big ? hs - 1 - i : i] << (8 * i);
  return v;
}

bool inflate_blocks(const std::vector<unsigned char>& header, const unsigned char* data, size_t avail, size_t hs,
                    bool swap, std::vector<unsigned char>& out, std::string& err) {
#ifdef RTG_HAVE_ZLIB
  const uint64_t nb = header_word(header, 0, hs, swap), bs = header_word(header, 1, hs, swap);
  const uint64_t last = header_word(header, 2, hs, swap);
  if (nb > header.size() / hs || header.size() / hs - nb < 3) return err = "truncated compression header", false;
  out.clear();
  size_t pos = 0;
  for (uint64_t b = 0; b < nb; ++b) {
    const uint64_t cs = header_word(header, 3 + b, hs, swap);
    const uint64_t us = (b + 1 == nb && last != 0) ? last : bs;
    if (cs > avail - pos) return err = "truncated compressed block", false;
    // zlib expands at most about 1032:1, so a larger size is a damaged header
    if (us > 1100 * cs + 64) return err = "compressed block larger than zlib allows", false;
    const size_t o0 = out.size();
    out.resize(o0 + us);
    uLongf dl = (uLongf)us;
    if (uncompress(out.data() + o0, &dl, data + pos, (uLong)cs) != Z_OK || dl != us)
      return err = "zlib block does not inflate", false;
    pos += cs;
  }
  return true;
#else
  (void)header; (void)data; (void)avail; (void)hs; (void)swap; (void)out;
  return err = "compressed VTK data needs a build with zlib", false;
#endif
}

bool decode(const Doc& doc, const std::string& s, DataArray& d, std::string& err) {
  d.v.clear();
  if (d.type == "String") return true;  // field strings are not needed by the readers
  const size_t ts = type_size(d.type);
  if (ts == 0) return err = "unsupported data type " + d.type, false;
  const bool swap = (doc.byte_order == "BigEndian") == host_little();
  const size_t hs = doc.header_type == "UInt64" ? 8 : 4;
  const bool zl = !doc.compressor.empty();
  if (zl && doc.compressor != "vtkZLibDataCompressor") return err = "unsupported compressor " + doc.compressor, false;
  std::vector<unsigned char> bytes;
  if (d.format == "ascii") {
    const char* p = d.text.c_str();
    char* e = nullptr;
    for (;;) {
      const double v = std::strtod(p, &e);
      if (e == p) break;
      d.v.push_back(v);
      p = e;
    }
    return true;
  }
  if (d.format == "binary" || (d.format == "appended" && doc.appended_encoding == "base64")) {
    const char* p;
    size_t n;
    if (d.format == "binary") {
      p = d.text.c_str();
      n = d.text.size();
    } else {
      if (d.offset < 0 || doc.appended_start == std::string::npos) return err = "appended array without offset", false;
      if ((size_t)d.offset > s.size() - doc.appended_start) return err = "appended data out of range", false;
      p = s.c_str() + doc.appended_start + (size_t)d.offset;
      n = s.size() - doc.appended_start - (size_t)d.offset;
    }
    while (n > 0 && std::isspace((unsigned char)*p)) ++p, --n;
    if (!zl) {
      // header and data encoded together, or the header on its own first
      const size_t hc = (hs + 2) / 3 * 4;
      size_t used = 0;
      std::vector<unsigned char> all = b64(p, n, &used);
      if (all.size() < hs) return err = "truncated binary array", false;
      uint64_t nbytes = header_word(all, 0, hs, swap);
      if (all.size() == hs && used <= hc + 2) {
        bytes = b64(p + used, n - used);
      } else {
        bytes.assign(all.begin() + hs, all.end());
      }
      if (bytes.size() < nbytes) return err = "truncated binary array", false;
      bytes.resize(nbytes);
    } else {
      // compression header in its own base64 run, then the compressed blocks
      const size_t h3 = (3 * hs + 2) / 3 * 4;
      std::vector<unsigned char> h = b64(p, std::min(n, h3));
      if (h.size() < 3 * hs || n < h3) return err = "truncated compression header", false;
      const uint64_t nb = header_word(h, 0, hs, swap);
      if (nb > (n - h3) / hs) return err = "truncated compression header", false;
      const size_t hb = (nb * hs + 2) / 3 * 4;
      if (hb > n - h3) return err = "truncated compression header", false;
      std::vector<unsigned char> sizes = b64(p + h3, std::min(n - h3, hb));
      h.insert(h.end(), sizes.begin(), sizes.end());
      std::vector<unsigned char> data = b64(p + h3 + hb, n - h3 - hb);
      if (!inflate_blocks(h, data.data(), data.size(), hs, swap, bytes, err)) return false;
    }
  } else if (d.format == "appended") {  // raw
    if (d.offset < 0 || doc.appended_start == std::string::npos) return err = "appended array without offset", false;
    const size_t at = doc.appended_start + (size_t)d.offset;
    if (at + hs > s.size()) return err = "appended data out of range", false;
    const unsigned char* p = (const unsigned char*)s.data() + at;
    const size_t avail = s.size() - at;
    if (!zl) {
      std::vector<unsigned char> h(p, p + hs);
      const uint64_t nbytes = header_word(h, 0, hs, swap);
      if (nbytes > avail - hs) return err = "appended data out of range", false;
      bytes.assign(p + hs, p + hs + nbytes);
    } else {
      std::vector<unsigned char> h(p, p + std::min(avail, 3 * hs));
      if (h.size() < 3 * hs) return err = "truncated compression header", false;
      const uint64_t nb = header_word(h, 0, hs, swap);
      if (nb > avail / hs - 3) return err = "truncated compression header", false;
      h.assign(p, p + (3 + nb) * hs);
      if (!inflate_blocks(h, p + (3 + nb) * hs, avail - (3 + nb) * hs, hs, swap, bytes, err)) return false;
    }
  } else {
    return err = "unsupported DataArray format " + d.format, false;
  }
  const size_t count = bytes.size() / ts;
  d.v.resize(count);
  for (size_t i = 0; i < count; ++i) d.v[i] = load_value(bytes.data() + i * ts, d.type, swap);
  return true;
}

bool load_doc(const char* path, std::string& s, Doc& doc, std::string& err) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return err = std::string("cannot open ") + path, false;
  std::ostringstream ss;
  ss << f.rdbuf();
  s = ss.str();
  return parse_xml(s, doc, err);
}

DataArray* find(Piece& p, const char* section, const char* name) {
  for (size_t i = 0; i < p.arrays.size(); ++i)
    if (p.section[i] == section && (!name || p.arrays[i].name == name)) return &p.arrays[i];
  return nullptr;
}

void set_err(char* buf, int32_t len, const std::string& m) {
  if (buf && len > 0) {
    std::snprintf(buf, (size_t)len, "%s", m.c_str());
  }
}

// The readers' vectors grow with the file; a host allocation that fails (or
// any other exception) becomes an error code instead of crossing the C ABI.
template <typename F>
int guarded(char* err, int32_t err_len, F&& f) noexcept {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    set_err(err, err_len, "out of host memory");
    return RTG_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return RTG_ERR_INVALID_ARGUMENT;
  } catch (...) {
    set_err(err, err_len, "unexpected error");
    return RTG_ERR_INVALID_ARGUMENT;
  }
}

}  // namespace

extern "C" {

int rtg_write_vtp_segments(const char* path, const rtg_segment* seg, int64_t n) {
  if (!path || n < 0 || (n > 0 && !seg)) return RTG_ERR_INVALID_ARGUMENT;
  Out o;
  o.f = std::fopen(path, "w");
  if (!o.f) return RTG_ERR_INVALID_ARGUMENT;
  o.put("<?xml version=\"1.0\"?>\n");
  o.put("<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n");
  o.put("  <PolyData>\n");
  o.fmt("    <Piece NumberOfPoints=\"%lld\" NumberOfVerts=\"0\" NumberOfLines=\"%lld\" NumberOfStrips=\"0\" "
        "NumberOfPolys=\"0\">\n",
        (long long)(2 * n), (long long)n);
  o.put("      <PointData>\n      </PointData>\n");
  o.put("      <CellData>\n");
  data_array(o, "UInt64", "ray", 1, n, "%llu", [&](int64_t i) { return (unsigned long long)seg[i].ray; });
  data_array(o, "UInt32", "segment", 1, n, "%u", [&](int64_t i) { return (unsigned)seg[i].segment; });
  data_array(o, "Int32", "kind", 1, n, "%d", [&](int64_t i) { return (int)seg[i].kind; });
  data_array(o, "Int32", "primitive", 1, n, "%d", [&](int64_t i) { return (int)seg[i].primitive; });
  data_array(o, "Float32", "weight", 1, n, "%.9g", [&](int64_t i) { return (double)seg[i].weight; });
  o.put("      </CellData>\n");
  o.put("      <Points>\n");
  data_array(o, "Float32", "Points", 3, 2 * n, "%.9g", [&](int64_t i) -> double {
    const int64_t pt = i / 3, a = i % 3;
    const rtg_segment& s = seg[pt / 2];
    return (double)((pt & 1) ? s.end[a] : s.org[a]);
  });
  o.put("      </Points>\n");
  for (const char* sec : {"Verts", "Lines", "Strips", "Polys"}) {
    const bool lines = sec[0] == 'L';
    o.fmt("      <%s>\n", sec);
    data_array(o, "Int64", "connectivity", 1, lines ? 2 * n : 0, "%lld", [&](int64_t i) { return (long long)i; });
    data_array(o, "Int64", "offsets", 1, lines ? n : 0, "%lld", [&](int64_t i) { return (long long)(2 * (i + 1)); });
    o.fmt("      </%s>\n", sec);
  }
  o.put("    </Piece>\n  </PolyData>\n</VTKFile>\n");
  const bool ok = o.ok;
  if (std::fclose(o.f) != 0 || !ok) return RTG_ERR_INTERNAL;
  return RTG_OK;
}

int rtg_write_vtp_discs(const char* path, int64_t n, const float* points, const float* normals, const float* radii,
                        const double* value, const uint64_t* hitcnt, const float* exposed_area,
                        const double* relative_error, const double* vov, const char* const* meta_keys,
                        const char* const* meta_values, int32_t n_meta) {
  const Results r{value, hitcnt, exposed_area, relative_error, vov};
  return write_polydata(path, n, points, normals, radii, 0, nullptr, 0, nullptr, r, meta_keys, meta_values, n_meta);
}

int rtg_write_vtp_triangles(const char* path, int64_t nv, const float* vertices, int64_t nt, const uint32_t* indices,
                            const double* value, const uint64_t* hitcnt, const float* exposed_area,
                            const double* relative_error, const double* vov, const char* const* meta_keys,
                            const char* const* meta_values, int32_t n_meta) {
  const Results r{value, hitcnt, exposed_area, relative_error, vov};
  return write_polydata(path, 0, nullptr, nullptr, nullptr, nv, vertices, nt, indices, r, meta_keys, meta_values,
                        n_meta);
}

int rtg_write_vtp_mixed(const char* path, int64_t nd, const float* points, const float* normals, const float* radii,
                        int64_t nv, const float* vertices, int64_t nt, const uint32_t* indices, const double* value,
                        const uint64_t* hitcnt, const float* exposed_area, const double* relative_error,
                        const double* vov, const char* const* meta_keys, const char* const* meta_values,
                        int32_t n_meta) {
  const Results r{value, hitcnt, exposed_area, relative_error, vov};
  return write_polydata(path, nd, points, normals, radii, nv, vertices, nt, indices, r, meta_keys, meta_values,
                        n_meta);
}

static int rtg_read_point_cloud_impl(const char* path, int64_t* n, float* points, float* normals, float* radii, char* err,
                         int32_t err_len) {
  if (!path || !n) return RTG_ERR_INVALID_ARGUMENT;
  std::string s, e;
  Doc doc;
  if (!load_doc(path, s, doc, e)) return set_err(err, err_len, e), RTG_ERR_INVALID_ARGUMENT;
  Piece& p = doc.piece;
  DataArray* pts = find(p, "Points", nullptr);
  if (!pts) return set_err(err, err_len, "no Points"), RTG_ERR_INVALID_ARGUMENT;
  DataArray* rad = find(p, "CellData", "radius");
  DataArray* soa = find(p, "CellData", "sqrt-of-area");
  DataArray* nrm = p.cell_normals.empty() ? nullptr : find(p, "CellData", p.cell_normals.c_str());
  if (!nrm) nrm = find(p, "CellData", "Normals");
  if (!rad && !soa) return set_err(err, err_len, "no cell data named \"radius\" or \"sqrt-of-area\""), RTG_ERR_INVALID_ARGUMENT;
  if (!nrm) return set_err(err, err_len, "no cell normals"), RTG_ERR_INVALID_ARGUMENT;
  for (DataArray* d : {pts, rad ? rad : soa, nrm})
    if (!decode(doc, s, *d, e)) return set_err(err, err_len, e), RTG_ERR_INVALID_ARGUMENT;
  const int64_t np = (int64_t)(pts->v.size() / 3);
  const DataArray* r = rad ? rad : soa;
  if ((int64_t)r->v.size() < np || (int64_t)nrm->v.size() < 3 * np)
    return set_err(err, err_len, "fewer cell values than points"), RTG_ERR_INVALID_ARGUMENT;
  if (!points && !normals && !radii) {
    *n = np;
    return RTG_OK;
  }
  if (*n < np) return set_err(err, err_len, "output arrays too small"), RTG_ERR_INVALID_ARGUMENT;
  for (int64_t i = 0; i < np; ++i) {
    double radius = r->v[i];
    if (!rad) radius *= std::sqrt(3.0) / 2 * (1 + 1.0 / 32);  // vtp_point_cloud_reader.hpp:75-81
    float q[3] = {(float)nrm->v[3 * i], (float)nrm->v[3 * i + 1], (float)nrm->v[3 * i + 2]};
    const float len = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    if (!(1 - 1e-6f <= len && len <= 1 + 1e-6f) && len > 0.0f)  // utils.hpp:77-93
      for (float& c : q) c /= len;
    if (points)
      for (int a = 0; a < 3; ++a) points[3 * i + a] = (float)pts->v[3 * i + a];
    if (normals)
      for (int a = 0; a < 3; ++a) normals[3 * i + a] = q[a];
    if (radii) radii[i] = (float)radius;
  }
  *n = np;
  return RTG_OK;
}

static int rtg_read_triangles_impl(const char* path, int64_t* nv, float* vertices, int64_t* nt, uint32_t* indices, char* err,
                       int32_t err_len) {
  if (!path || !nv || !nt) return RTG_ERR_INVALID_ARGUMENT;
  std::string s, e;
  Doc doc;
  if (!load_doc(path, s, doc, e)) return set_err(err, err_len, e), RTG_ERR_INVALID_ARGUMENT;
  Piece& p = doc.piece;
  DataArray* pts = find(p, "Points", nullptr);
  if (!pts) return set_err(err, err_len, "no Points"), RTG_ERR_INVALID_ARGUMENT;
  const char* sec = p.unstructured ? "Cells" : "Polys";
  DataArray* conn = find(p, sec, "connectivity");
  DataArray* offs = find(p, sec, "offsets");
  DataArray* types = p.unstructured ? find(p, sec, "types") : nullptr;
  if (!conn || !offs || (p.unstructured && !types))
    return set_err(err, err_len, std::string("no ") + sec + " connectivity/offsets"), RTG_ERR_INVALID_ARGUMENT;
  for (DataArray* d : {pts, conn, offs})
    if (!decode(doc, s, *d, e)) return set_err(err, err_len, e), RTG_ERR_INVALID_ARGUMENT;
  if (types && !decode(doc, s, *types, e)) return set_err(err, err_len, e), RTG_ERR_INVALID_ARGUMENT;
  const int64_t npts = (int64_t)(pts->v.size() / 3);
  std::vector<uint32_t> tri;
  double start = 0;
  for (size_t c = 0; c < offs->v.size(); ++c) {
    const double end = offs->v[c];
    if (!(end >= start && end <= (double)conn->v.size()))
      return set_err(err, err_len, "cell offsets out of range"), RTG_ERR_INVALID_ARGUMENT;
    const bool is_tri = end - start == 3 && (!types || (c < types->v.size() && types->v[c] == 5));
    if (is_tri) {  // vtp_triangle_reader.hpp:56-63: three-point cells only
      for (int k = 0; k < 3; ++k) {
        const double id = conn->v[(size_t)start + k];
        if (!(id >= 0 && id < npts)) return set_err(err, err_len, "point index out of range"), RTG_ERR_INVALID_ARGUMENT;
        tri.push_back((uint32_t)id);
      }
    }
    start = end;
  }
  const int64_t ntri = (int64_t)tri.size() / 3;
  if (!vertices && !indices) {
    *nv = npts;
    *nt = ntri;
    return RTG_OK;
  }
  if (*nv < npts || *nt < ntri) return set_err(err, err_len, "output arrays too small"), RTG_ERR_INVALID_ARGUMENT;
  if (vertices)
    for (int64_t i = 0; i < 3 * npts; ++i) vertices[i] = (float)pts->v[i];
  if (indices) std::memcpy(indices, tri.data(), tri.size() * sizeof(uint32_t));
  *nv = npts;
  *nt = ntri;
  return RTG_OK;
}

// rti's io/christoph and io/xaver readers: UnstructuredGrid point clouds
// whose radius comes from an area or a grid spacing.
static int rtg_read_point_cloud_vtu_impl(const char* path, int32_t flavor, int64_t* n, float* points, float* normals,
                             float* radii, char* err, int32_t err_len) {
  if (!path || !n || (flavor != RTG_VTU_AREA && flavor != RTG_VTU_SPACING)) return RTG_ERR_INVALID_ARGUMENT;
  std::string s, e;
  Doc doc;
  if (!load_doc(path, s, doc, e)) return set_err(err, err_len, e), RTG_ERR_INVALID_ARGUMENT;
  Piece& p = doc.piece;
  DataArray* pts = find(p, "Points", nullptr);
  if (!pts) return set_err(err, err_len, "no Points"), RTG_ERR_INVALID_ARGUMENT;
  // christoph: point data area_around_vertex, else cell data gridSpacing; xaver: gridSpacing
  DataArray* size = flavor == RTG_VTU_AREA ? find(p, "PointData", "area_around_vertex") : nullptr;
  if (!size) size = find(p, "CellData", "gridSpacing");
  DataArray* nrm = find(p, "CellData", "Normals");
  if (!nrm) nrm = find(p, "PointData", "normal_vector");
  if (!size)
    return set_err(err, err_len, flavor == RTG_VTU_AREA ? "no area_around_vertex or gridSpacing data" : "no gridSpacing data"),
           RTG_ERR_INVALID_ARGUMENT;
  if (!nrm) return set_err(err, err_len, "no Normals or normal_vector data"), RTG_ERR_INVALID_ARGUMENT;
  for (DataArray* d : {pts, size, nrm})
    if (!decode(doc, s, *d, e)) return set_err(err, err_len, e), RTG_ERR_INVALID_ARGUMENT;
  const int64_t np = (int64_t)(pts->v.size() / 3);
  if ((int64_t)size->v.size() < np || (int64_t)nrm->v.size() < 3 * np)
    return set_err(err, err_len, "fewer size or normal values than points"), RTG_ERR_INVALID_ARGUMENT;
  const double grow = std::sqrt(3.0) / 2 * (1 + 1.0 / 4);  // about 25 %
  int64_t kept = 0;
  const bool count_only = !points && !normals && !radii;
  for (int64_t i = 0; i < np; ++i) {
    const double a = size->v[i];
    const double radius = (flavor == RTG_VTU_AREA ? std::sqrt(a) : a) * grow;
    const double* q = &nrm->v[3 * i];
    // points of zero area (radius) or with the zero vector as normal are left out
    if ((flavor == RTG_VTU_AREA ? a == 0 : radius == 0) || (q[0] == 0 && q[1] == 0 && q[2] == 0)) continue;
    if (!count_only) {
      if (kept >= *n) return set_err(err, err_len, "output arrays too small"), RTG_ERR_INVALID_ARGUMENT;
      float c[3] = {(float)pts->v[3 * i], (float)pts->v[3 * i + 1], (float)pts->v[3 * i + 2]};
      float u[3] = {(float)q[0], (float)q[1], (float)q[2]};
      if (flavor == RTG_VTU_AREA) {  // the christoph reader inverts every z coordinate
        c[2] *= -1;
        u[2] *= -1;
      }
      const float len = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
      if (!(1 - 1e-6f <= len && len <= 1 + 1e-6f) && len > 0.0f)  // utils.hpp:77-93
        for (float& x : u) x /= len;
      if (points)
        for (int k = 0; k < 3; ++k) points[3 * kept + k] = c[k];
      if (normals)
        for (int k = 0; k < 3; ++k) normals[3 * kept + k] = u[k];
      if (radii) radii[kept] = (float)radius;
    }
    ++kept;
  }
  *n = kept;
  return RTG_OK;
}

// rti's io/christoph/vtu_triangle_reader.hpp: every three-point cell, its
// second and third vertex swapped, with the mean of its vertices' normals.
static int rtg_read_triangles_vtu_impl(const char* path, int64_t* nv, float* vertices, int64_t* nt, uint32_t* indices,
                           float* normals, char* err, int32_t err_len) {
  if (!path || !nv || !nt) return RTG_ERR_INVALID_ARGUMENT;
  std::string s, e;
  Doc doc;
  if (!load_doc(path, s, doc, e)) return set_err(err, err_len, e), RTG_ERR_INVALID_ARGUMENT;
  Piece& p = doc.piece;
  DataArray* pts = find(p, "Points", nullptr);
  DataArray* conn = find(p, "Cells", "connectivity");
  DataArray* offs = find(p, "Cells", "offsets");
  DataArray* pn = find(p, "PointData", "normal_vector");
  if (!pts || !conn || !offs) return set_err(err, err_len, "no Points or Cells"), RTG_ERR_INVALID_ARGUMENT;
  if (normals && !pn) return set_err(err, err_len, "no normal_vector point data"), RTG_ERR_INVALID_ARGUMENT;
  for (DataArray* d : {pts, conn, offs})
    if (!decode(doc, s, *d, e)) return set_err(err, err_len, e), RTG_ERR_INVALID_ARGUMENT;
  if (pn && !decode(doc, s, *pn, e)) return set_err(err, err_len, e), RTG_ERR_INVALID_ARGUMENT;
  const int64_t npts = (int64_t)(pts->v.size() / 3);
  if (pn && (int64_t)pn->v.size() < 3 * npts)
    return set_err(err, err_len, "fewer normal_vector values than points"), RTG_ERR_INVALID_ARGUMENT;
  std::vector<uint32_t> tri;
  double start = 0;
  for (size_t c = 0; c < offs->v.size(); ++c) {
    const double end = offs->v[c];
    if (!(end >= start && end <= (double)conn->v.size()))
      return set_err(err, err_len, "cell offsets out of range"), RTG_ERR_INVALID_ARGUMENT;
    if (end - start == 3) {
      uint32_t id[3];
      for (int k = 0; k < 3; ++k) {
        const double v = conn->v[(size_t)start + k];
        if (!(v >= 0 && v < npts)) return set_err(err, err_len, "point index out of range"), RTG_ERR_INVALID_ARGUMENT;
        id[k] = (uint32_t)v;
      }
      tri.push_back(id[0]);
      tri.push_back(id[2]);
      tri.push_back(id[1]);
    }
    start = end;
  }
  const int64_t ntri = (int64_t)tri.size() / 3;
  if (!vertices && !indices && !normals) {
    *nv = npts;
    *nt = ntri;
    return RTG_OK;
  }
  if (*nv < npts || *nt < ntri) return set_err(err, err_len, "output arrays too small"), RTG_ERR_INVALID_ARGUMENT;
  if (vertices)
    for (int64_t i = 0; i < 3 * npts; ++i) vertices[i] = (float)pts->v[i];
  if (indices) std::memcpy(indices, tri.data(), tri.size() * sizeof(uint32_t));
  if (normals)
    for (int64_t t = 0; t < ntri; ++t) {
      const uint32_t a = tri[3 * t], b = tri[3 * t + 2], c = tri[3 * t + 1];  // the cell's own order
      float m[3];
      for (int k = 0; k < 3; ++k) m[k] = (float)((pn->v[3 * a + k] + pn->v[3 * b + k] + pn->v[3 * c + k]) / 3);
      // as the reference: every component below 1e-5 (signed) counts as no normal
      if (m[0] < 1e-5f && m[1] < 1e-5f && m[2] < 1e-5f) m[0] = 0, m[1] = 0, m[2] = 1;
      const float len = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
      for (int k = 0; k < 3; ++k) normals[3 * t + k] = m[k] / len;
    }
  *nv = npts;
  *nt = ntri;
  return RTG_OK;
}

int rtg_read_point_cloud(const char* path, int64_t* n, float* points, float* normals, float* radii, char* err,
                         int32_t err_len) {
  return guarded(err, err_len, [&] { return rtg_read_point_cloud_impl(path, n, points, normals, radii, err, err_len); });
}

int rtg_read_triangles(const char* path, int64_t* nv, float* vertices, int64_t* nt, uint32_t* indices, char* err,
                       int32_t err_len) {
  return guarded(err, err_len, [&] { return rtg_read_triangles_impl(path, nv, vertices, nt, indices, err, err_len); });
}

int rtg_read_point_cloud_vtu(const char* path, int32_t flavor, int64_t* n, float* points, float* normals,
                             float* radii, char* err, int32_t err_len) {
  return guarded(err, err_len, [&] { return rtg_read_point_cloud_vtu_impl(path, flavor, n, points, normals, radii, err, err_len); });
}

int rtg_read_triangles_vtu(const char* path, int64_t* nv, float* vertices, int64_t* nt, uint32_t* indices,
                           float* normals, char* err, int32_t err_len) {
  return guarded(err, err_len, [&] { return rtg_read_triangles_vtu_impl(path, nv, vertices, nt, indices, normals, err, err_len); });
}

}  // extern "C"
