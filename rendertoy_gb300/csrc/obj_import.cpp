// obj_import.cpp — OBJ and MTL import straight into the flattened scene
// arrays rtx_scene_upload takes (RenderToy OBJModelImporter::Import and
// MTLImporter::Import, src/importer.cpp:29-229).
//
// The reference reads the file through an std::ifstream token by token and
// builds a Mesh / Triangle object graph; this parser reads the file once into
// memory and walks it with the same token rules, writing triangles directly
// in World::triangles order.  What it keeps from the reference, because the
// triangle ids and the emitter order depend on it:
//   * tokens are whitespace-separated (operator>> rules): a "v" reads three
//     numbers even across a line break, and whatever follows them on the line
//     is read as the next identifier;
//   * unknown identifiers skip the rest of their line (comments included);
//   * "f" takes the rest of its line, trims and collapses runs of spaces
//     (importer.cpp:101), splits on single spaces and each vertex on '/';
//     each field is parsed like std::stoi (leading whitespace, sign, digits,
//     trailing garbage ignored); an empty or unparsable field means "absent"
//     (the zero vector);
//   * a face of V vertices is fanned into (0, b, b + 1), b = 1 .. V - 2
//     (Polygon::ConvertToTriangle, object.cpp:333-342), appended to the
//     world's triangles, and PREPENDED as a block to its mesh's triangle list
//     (importer.cpp:136), which is the order emitters are sampled in;
//   * "s" extracts a bool the way operator>>(bool&) does: 0 or 1; anything
//     else ("off", "2") stores false / true and fails the stream, which ends
//     the import silently (RenderToy's while (fs >> identifier) loop) with
//     the meshes read so far;
//   * a number that operator>>(float&) cannot read ends the import the same way.
// Where the reference has undefined behaviour (a vertex index out of range
// or negative, more than three '/' fields, "s" / "f" before any "o", material
// keys before any "newmtl"), this parser reports an error instead.
#include <cerrno>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <limits>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "rtx.h"

struct rtx_obj {
  // triangles in World::triangles order
  std::vector<float> verts, norms, uvs;  // 9, 9, 6 floats per triangle
  std::vector<int32_t> tri_mesh;
  // meshes in World::meshes order
  std::vector<std::string> mesh_names;
  std::vector<uint8_t> mesh_smooth;
  std::vector<std::vector<int32_t>> mesh_tris;  // Mesh::tris order
  // materials of the MTL file in World::materials order
  std::vector<std::string> mat_names;
  std::vector<float> mats;  // 24 floats each
};

namespace {

struct Cursor {
  const char* p;
  const char* end;
  bool failed = false;  // the stream's failbit

  static bool ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }
  void skip_ws() {
    while (p < end && ws(*p)) ++p;
  }
  // operator>>(std::string&)
  bool token(std::string& out) {
    skip_ws();
    if (p >= end) return false;
    const char* b = p;
    while (p < end && !ws(*p)) ++p;
    out.assign(b, p);
    return true;
  }
  // istream::ignore(max, '\n')
  void ignore_line() {
    while (p < end && *p != '\n') ++p;
    if (p < end) ++p;
  }
  // operator>>(float&): skips whitespace, then takes the longest prefix of
  // the form [+-]digits[.digits][(e|E)[+-]digits] (num_get's accepted
  // characters), converted with correct rounding; no digits fails the stream
  bool number(float& out) {
    skip_ws();
    const char* b = p;
    const char* q = p;
    if (q < end && (*q == '+' || *q == '-')) ++q;
    const char* d0 = q;
    while (q < end && *q >= '0' && *q <= '9') ++q;
    bool digits = q > d0;
    if (q < end && *q == '.') {
      ++q;
      const char* f0 = q;
      while (q < end && *q >= '0' && *q <= '9') ++q;
      digits = digits || q > f0;
    }
    if (!digits) {
      failed = true;
      return false;
    }
    if (q < end && (*q == 'e' || *q == 'E')) {
      const char* e = q + 1;
      if (e < end && (*e == '+' || *e == '-')) ++e;
      const char* e0 = e;
      while (e < end && *e >= '0' && *e <= '9') ++e;
      if (e > e0) q = e;
    }
    // std::from_chars rounds as strtof does (correctly) without a copy or
    // the locale; it takes no '+' and leaves out-of-range values to strtof
    float v;
    std::from_chars_result r = std::from_chars(*b == '+' ? b + 1 : b, q, v);
    if (r.ec != std::errc() || r.ptr != q) {
      std::string s(b, q);
      errno = 0;
      v = std::strtof(s.c_str(), nullptr);
      if (errno == ERANGE && std::isinf(v)) {  // num_get: out of range fails the stream
        failed = true;
        return false;
      }
    }
    out = v;
    p = q;
    return true;
  }
  // operator>>(bool&) without boolalpha: a long that must be 0 or 1.  On
  // failure the stream still stores a value: false when no number could be
  // read, true for any other number (num_get, C++11 and later)
  bool boolean(uint8_t& out) {
    skip_ws();
    const char* q = p;
    if (q < end && (*q == '+' || *q == '-')) ++q;
    const char* d0 = q;
    while (q < end && *q >= '0' && *q <= '9') ++q;
    if (q == d0) {
      out = 0;
      failed = true;
      return false;
    }
    std::string s(p, q);
    p = q;
    errno = 0;
    long v = std::strtol(s.c_str(), nullptr, 10);
    if (errno == ERANGE || (v != 0 && v != 1)) {
      out = 1;
      failed = true;
      return false;
    }
    out = (uint8_t)v;
    return true;
  }
};

// std::stoi on the characters [b, e): leading whitespace, optional sign,
// decimal digits (anything after them ignored); false when there are no
// digits or the value does not fit an int
bool parse_stoi(const char* b, const char* e, int& out) {
  while (b < e && (*b == ' ' || *b == '\t' || *b == '\n' || *b == '\r' || *b == '\v' || *b == '\f')) ++b;
  const char* q = b;
  bool neg = false;
  if (q < e && (*q == '+' || *q == '-')) neg = *q++ == '-';
  const char* d0 = q;
  long long v = 0;
  while (q < e && *q >= '0' && *q <= '9') {
    if (v <= (1LL << 40)) v = v * 10 + (*q - '0');  // saturates far beyond int
    ++q;
  }
  if (q == d0) return false;
  if (neg) v = -v;
  if (v < std::numeric_limits<int>::min() || v > std::numeric_limits<int>::max()) return false;
  out = (int)v;
  return true;
}

bool read_file(const char* path, std::string& data) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  // a regular file is read in one piece into a string of its size (a
  // third of the time of streaming it through a string stream)
  std::error_code ec;
  if (std::filesystem::is_regular_file(path, ec)) {
    uintmax_t n = std::filesystem::file_size(path, ec);
    if (!ec && n < ((uintmax_t)1 << 40)) {
      data.resize((size_t)n);
      f.read(&data[0], (std::streamsize)n);
      data.resize((size_t)f.gcount());
      return true;
    }
  }
  std::ostringstream ss;
  ss << f.rdbuf();
  data = ss.str();
  return true;
}

void set_msg(char* msg, size_t len, const std::string& m) {
  if (msg && len) {
    size_t n = std::min(len - 1, m.size());
    std::memcpy(msg, m.data(), n);
    msg[n] = 0;
  }
}

struct V3 {
  float x, y, z;
};
struct V2 {
  float x, y;
};

int parse_obj(const std::string& text, rtx_obj& o, std::string& err) {
  Cursor c{text.data(), text.data() + text.size()};
  std::vector<V3> vert{{0, 0, 0}}, norm{{0, 0, 0}};
  std::vector<V2> uv{{0, 0}};
  std::vector<V3> pv, pn;  // one face's vertices
  std::vector<V2> pt;
  int mesh = -1;
  // Each mesh's triangles as the faces append them, and where each face's
  // block starts; Mesh::tris is the blocks in reverse (each face's block is
  // prepended), each block in its own order.  Built once at the end rather
  // than by inserting at the front, which costs quadratic time in a large mesh.
  std::vector<std::vector<int32_t>> appended, blocks;
  auto finish_mesh_tris = [&] {
    for (size_t m = 0; m < appended.size(); ++m) {
      std::vector<int32_t>& mt = o.mesh_tris[m];
      mt.clear();
      mt.reserve(appended[m].size());
      for (size_t b = blocks[m].size(); b-- > 0;) {
        size_t e = b + 1 < blocks[m].size() ? (size_t)blocks[m][b + 1] : appended[m].size();
        mt.insert(mt.end(), appended[m].begin() + blocks[m][b], appended[m].begin() + e);
      }
    }
  };
  std::string id;
  while (!c.failed && c.token(id)) {
    if (id == "o") {
      mesh = (int)o.mesh_names.size();
      o.mesh_names.emplace_back();
      o.mesh_smooth.push_back(0);
      o.mesh_tris.emplace_back();
      appended.emplace_back();
      blocks.emplace_back();
      c.token(o.mesh_names.back());
      continue;
    }
    if (id == "v" || id == "vn") {
      V3 v{0, 0, 0};
      if (!c.number(v.x) || !c.number(v.y) || !c.number(v.z)) break;
      (id == "v" ? vert : norm).push_back(v);
      continue;
    }
    if (id == "vt") {
      V2 v{0, 0};
      if (!c.number(v.x) || !c.number(v.y)) break;
      uv.push_back(v);
      continue;
    }
    if (id == "s") {
      if (mesh < 0) {
        err = "'s' before any 'o'";
        return RTX_ERR_INVALID;
      }
      if (!c.boolean(o.mesh_smooth[mesh])) break;
      continue;
    }
    if (id == "f") {
      if (mesh < 0) {
        err = "'f' before any 'o'";
        return RTX_ERR_INVALID;
      }
      // the rest of the line (std::getline), trimmed and split at runs of
      // spaces (importer.cpp:101 collapses them first); each vertex split at
      // '/' as getline does (a trailing empty field dropped)
      const char* lb = c.p;
      while (c.p < c.end && *c.p != '\n') ++c.p;
      const char* le = c.p;
      if (c.p < c.end) ++c.p;
      pv.clear();
      pn.clear();
      pt.clear();
      for (const char* q = lb; q < le;) {
        if (*q == ' ') {
          ++q;
          continue;
        }
        const char* fb = q;
        while (q < le && *q != ' ') ++q;
        const char* fe = q;
        const char* sb[4];
        const char* se[4];
        int nf = 0;
        for (const char* i = fb; i < fe;) {
          const char* j = i;
          while (j < fe && *j != '/') ++j;
          if (nf == 3) {
            err = "a face vertex with more than three fields";
            return RTX_ERR_INVALID;
          }
          sb[nf] = i;
          se[nf++] = j;
          i = j < fe ? j + 1 : fe;
        }
        int idx[3] = {0, 0, 0};
        bool has[3] = {false, false, false};
        for (int k = 0; k < nf; ++k) has[k] = se[k] > sb[k] && parse_stoi(sb[k], se[k], idx[k]);
        auto check = [&](int k, size_t n) {
          if (has[k] && (idx[k] < 0 || (size_t)idx[k] >= n)) {
            err = "face index " + std::to_string(idx[k]) + " out of range";
            return false;
          }
          return true;
        };
        if (!check(0, vert.size()) || !check(1, uv.size()) || !check(2, norm.size())) return RTX_ERR_INVALID;
        pv.push_back(has[0] ? vert[idx[0]] : V3{0, 0, 0});
        pt.push_back(has[1] ? uv[idx[1]] : V2{0, 0});
        pn.push_back(has[2] ? norm[idx[2]] : V3{0, 0, 0});
      }
      blocks[mesh].push_back((int32_t)appended[mesh].size());
      for (size_t b = 1; b + 1 < pv.size(); ++b) {
        size_t ids[3] = {0, b, b + 1};
        int32_t t = (int32_t)o.tri_mesh.size();
        for (size_t k : ids) {
          // Mesh's identity object-to-world turns -0.0 into +0.0 (object.cpp:42-48)
          o.verts.insert(o.verts.end(), {pv[k].x + 0.0f, pv[k].y + 0.0f, pv[k].z + 0.0f});
          o.norms.insert(o.norms.end(), {pn[k].x, pn[k].y, pn[k].z});
          o.uvs.insert(o.uvs.end(), {pt[k].x, pt[k].y});
        }
        o.tri_mesh.push_back(mesh);
        appended[mesh].push_back(t);
      }
      continue;
    }
    c.ignore_line();
  }
  finish_mesh_tris();
  return RTX_OK;
}

// PrincipledBSDF's member initialisers (include/RenderToy/material.h:16-30)
void default_material(float* m) {
  const float d[24] = {1, 1, 1, 0, 0, 0, 0.5f, 0, 0, 0, 0, 0, 0.5f, 0, 0.03f, 0, 1.45f, 1, 1, 1, 1, 0, 0, 0};
  std::memcpy(m, d, sizeof d);
}

int parse_mtl(const std::string& text, rtx_obj& o, std::string& err) {
  Cursor c{text.data(), text.data() + text.size()};
  std::string id;
  int cur = -1;
  // MTL key -> (first float of the record, count)
  struct Key {
    const char* name;
    int at, n;
  };
  static const Key keys[] = {{"Kd", 0, 3},  {"Ni", 16, 1}, {"Ke", 3, 3},  {"Pr", 6, 1},   {"Pm", 7, 1},
                             {"Ps", 11, 1}, {"Pc", 13, 1}, {"Pcr", 14, 1}, {"aniso", 8, 1}};
  while (!c.failed && c.token(id)) {
    if (id == "newmtl") {
      cur = (int)o.mat_names.size();
      o.mat_names.emplace_back();
      o.mats.resize(o.mats.size() + 24);
      default_material(&o.mats[24 * (size_t)cur]);
      c.token(o.mat_names.back());
    }
    for (const Key& k : keys)
      if (id == k.name) {
        if (cur < 0) {
          err = std::string("'") + k.name + "' before any 'newmtl'";
          return RTX_ERR_INVALID;
        }
        for (int i = 0; i < k.n && !c.failed; ++i) c.number(o.mats[24 * (size_t)cur + k.at + i]);
      }
    if (c.failed) break;
    c.ignore_line();
  }
  return RTX_OK;
}

}  // namespace

extern "C" {

int rtx_obj_import(const char* obj_path, const char* mtl_path, rtx_obj** out, char* msg, size_t msg_len) {
  if (!out || (!obj_path && !mtl_path)) {
    set_msg(msg, msg_len, "NULL argument");
    return RTX_ERR_INVALID;
  }
  *out = nullptr;
  rtx_obj* o = new (std::nothrow) rtx_obj();
  if (!o) return RTX_ERR_NOMEM;
  std::string text, err;
  int r = RTX_OK;
  if (obj_path) {
    if (!read_file(obj_path, text)) {
      set_msg(msg, msg_len, std::string("cannot read ") + obj_path);
      delete o;
      return RTX_ERR_INVALID;
    }
    r = parse_obj(text, *o, err);
  }
  if (r == RTX_OK && mtl_path) {
    if (!read_file(mtl_path, text)) {
      err = std::string("cannot read ") + mtl_path;
      r = RTX_ERR_INVALID;
    } else {
      r = parse_mtl(text, *o, err);
    }
  }
  if (r != RTX_OK) {
    set_msg(msg, msg_len, err);
    delete o;
    return r;
  }
  *out = o;
  return RTX_OK;
}

void rtx_obj_free(rtx_obj* o) { delete o; }

int rtx_obj_info(const rtx_obj* o, int* n_tris, int* n_meshes, int* n_materials) {
  if (!o) return RTX_ERR_INVALID;
  if (n_tris) *n_tris = (int)o->tri_mesh.size();
  if (n_meshes) *n_meshes = (int)o->mesh_names.size();
  if (n_materials) *n_materials = (int)o->mat_names.size();
  return RTX_OK;
}

int rtx_obj_triangles(const rtx_obj* o, float* verts, float* norms, float* uvs, int32_t* tri_mesh) {
  if (!o) return RTX_ERR_INVALID;
  if (o->tri_mesh.empty()) return RTX_OK;  // (an empty array's data() may be null)
  if (verts) std::memcpy(verts, o->verts.data(), o->verts.size() * sizeof(float));
  if (norms) std::memcpy(norms, o->norms.data(), o->norms.size() * sizeof(float));
  if (uvs) std::memcpy(uvs, o->uvs.data(), o->uvs.size() * sizeof(float));
  if (tri_mesh) std::memcpy(tri_mesh, o->tri_mesh.data(), o->tri_mesh.size() * sizeof(int32_t));
  return RTX_OK;
}

int rtx_obj_mesh(const rtx_obj* o, int mesh, const char** name, uint8_t* smooth, int32_t* tris, int* n_tris) {
  if (!o || mesh < 0 || mesh >= (int)o->mesh_names.size()) return RTX_ERR_INVALID;
  if (name) *name = o->mesh_names[mesh].c_str();
  if (smooth) *smooth = o->mesh_smooth[mesh];
  const std::vector<int32_t>& t = o->mesh_tris[mesh];
  if (n_tris) *n_tris = (int)t.size();
  if (tris && !t.empty()) std::memcpy(tris, t.data(), t.size() * sizeof(int32_t));
  return RTX_OK;
}

int rtx_obj_material(const rtx_obj* o, int mat, const char** name, float* record) {
  if (!o || mat < 0 || mat >= (int)o->mat_names.size()) return RTX_ERR_INVALID;
  if (name) *name = o->mat_names[mat].c_str();
  if (record) std::memcpy(record, &o->mats[24 * (size_t)mat], 24 * sizeof(float));
  return RTX_OK;
}

}  // extern "C"
