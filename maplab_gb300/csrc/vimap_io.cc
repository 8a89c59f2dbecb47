// VIMap map-folder reader, problem exporter and state write-back (host).
//
// Map format (read and written with this file's own protobuf wire-format
// codec; no protobuf library):
//   <folder>/vi_map/vi_map_metadata   text-format VIMapMetadata: the files
//                                     by VIMapFileType (vi-map-metadata.h:18-23)
//   <folder>/vi_map/missions, vertices<i>, edges<i>, landmark_index
//                                     binary vi_map.proto VIMap messages
//                                     (map-structure/vi-map/proto/vi-map/vi_map.proto)
//   <folder>/vi_map/sensors.yaml      SensorManager YAML: sensors (IMU sigmas,
//                                     NCAMERA cameras with intrinsics,
//                                     distortion, T_B_C) and extrinsics T_B_S
// Message semantics follow the deserializers: Vertex::deserialize
// (vertex.cc:441-535), Landmark::deserialize (landmark.cc:191-245),
// Edge::deserialize (edge.cc:52-76), TransformationEdge / LoopClosureEdge /
// ViwlsEdge::deserialize, VIMission::deserialize (vi-mission.cc:230-290),
// deserializeVisualFrame / deserializeVisualNFrame
// (aslam-serialization/src/visual-frame-serialization.cc:88-247) and
// common::eigen_proto (eigen-proto-inl.h: column-major matrices,
// transformations as Eigen quaternion x y z w | p).
#include <sys/stat.h>

#include <algorithm>
#include <array>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "maplab_vimap.h"

namespace {

// ------------------------------------------------------------------ ids
// aslam::HashId: 16 bytes; the proto carries them as two uint64 words (the
// bytes in memory order on little-endian hosts), YAML as 32 hex characters
// (byte i = characters 2i, 2i + 1; hash-id.h:61-92).  All-zero is invalid.
struct Id {
  uint64_t w[2] = {0, 0};
  bool valid() const { return w[0] != 0 || w[1] != 0; }
  bool operator==(const Id& o) const { return w[0] == o.w[0] && w[1] == o.w[1]; }
  bool operator!=(const Id& o) const { return !(*this == o); }
};
struct IdHash {
  size_t operator()(const Id& a) const { return std::hash<uint64_t>()(a.w[0] ^ (a.w[1] * 0x9E3779B97F4A7C15ull)); }
};
template <typename V>
using IdMap = std::unordered_map<Id, V, IdHash>;

int hexval(char c) {
  if (c >= '0' && c <= '9') return c - '0';
  if (c >= 'a' && c <= 'f') return c - 'a' + 10;
  if (c >= 'A' && c <= 'F') return c - 'A' + 10;
  return -1;
}

bool id_from_hex(const std::string& s, Id* id) {
  if (s.size() != 32) return false;
  uint8_t b[16];
  for (int i = 0; i < 16; ++i) {
    const int hi = hexval(s[2 * i]), lo = hexval(s[2 * i + 1]);
    if (hi < 0 || lo < 0) return false;
    b[i] = (uint8_t)(hi * 16 + lo);
  }
  for (int k = 0; k < 2; ++k) {
    uint64_t v = 0;
    for (int j = 7; j >= 0; --j) v = (v << 8) | b[8 * k + j];
    id->w[k] = v;
  }
  return true;
}

// ------------------------------------------------------------------ wire format
struct Bytes {
  const uint8_t* p = nullptr;
  const uint8_t* e = nullptr;
  size_t size() const { return (size_t)(e - p); }
};

double bits_to_double(uint64_t u) {
  double d;
  std::memcpy(&d, &u, 8);
  return d;
}
uint64_t double_to_bits(double d) {
  uint64_t u;
  std::memcpy(&u, &d, 8);
  return u;
}

// Decoder of one message: field headers, varints, fixed 64/32-bit values,
// length-delimited payloads; repeated scalars packed or not.  Groups (wire
// types 3/4) are malformed input here (vi_map.proto has none).
class Wire {
 public:
  explicit Wire(Bytes b) : p_(b.p), e_(b.e) {}
  bool ok() const { return ok_; }
  const uint8_t* pos() const { return p_; }
  bool next(uint32_t* field, int* wt) {
    if (!ok_ || p_ >= e_) return false;
    uint64_t k;
    if (!varint(&k)) return false;
    *field = (uint32_t)(k >> 3);
    *wt = (int)(k & 7);
    if (*field == 0) return fail();
    return true;
  }
  bool varint(uint64_t* v) {
    uint64_t r = 0;
    for (int s = 0; s < 64; s += 7) {
      if (p_ >= e_) return fail();
      const uint8_t b = *p_++;
      r |= (uint64_t)(b & 0x7f) << s;
      if (!(b & 0x80)) {
        *v = r;
        return true;
      }
    }
    return fail();
  }
  bool fixed64(uint64_t* v) {
    if (e_ - p_ < 8) return fail();
    uint64_t r = 0;
    for (int i = 7; i >= 0; --i) r = (r << 8) | p_[i];
    p_ += 8;
    *v = r;
    return true;
  }
  bool bytes(Bytes* b) {
    uint64_t n;
    if (!varint(&n)) return false;
    if ((uint64_t)(e_ - p_) < n) return fail();
    b->p = p_;
    b->e = p_ + n;
    p_ += n;
    return true;
  }
  bool skip(int wt) {
    switch (wt) {
      case 0: {
        uint64_t v;
        return varint(&v);
      }
      case 1:
        if (e_ - p_ < 8) return fail();
        p_ += 8;
        return true;
      case 2: {
        Bytes b;
        return bytes(&b);
      }
      case 5:
        if (e_ - p_ < 4) return fail();
        p_ += 4;
        return true;
      default:
        return fail();
    }
  }
  bool doubles(int wt, std::vector<double>* out) {
    if (wt == 1) {
      uint64_t u;
      if (!fixed64(&u)) return false;
      out->push_back(bits_to_double(u));
      return true;
    }
    if (wt != 2) return fail();
    Bytes b;
    if (!bytes(&b)) return false;
    if (b.size() % 8) return fail();
    Wire inner(b);
    while (inner.p_ < inner.e_) {
      uint64_t u = 0;
      inner.fixed64(&u);
      out->push_back(bits_to_double(u));
    }
    return true;
  }
  bool varints(int wt, std::vector<uint64_t>* out) {
    if (wt == 0) {
      uint64_t v;
      if (!varint(&v)) return false;
      out->push_back(v);
      return true;
    }
    if (wt != 2) return fail();
    Bytes b;
    if (!bytes(&b)) return false;
    Wire inner(b);
    while (inner.p_ < inner.e_) {
      uint64_t v;
      if (!inner.varint(&v)) return fail();
      out->push_back(v);
    }
    return true;
  }
  bool fixed_double(int wt, double* d) {
    uint64_t u;
    if (wt != 1 || !fixed64(&u)) return fail();
    *d = bits_to_double(u);
    return true;
  }

 private:
  bool fail() {
    ok_ = false;
    return false;
  }
  const uint8_t* p_;
  const uint8_t* e_;
  bool ok_ = true;
};

// Encoder (the save path re-encodes state fields; proto2 repeated doubles
// without [packed = true] are written one element per field).
struct Out {
  std::string s;
  void varint(uint64_t v) {
    while (v >= 0x80) {
      s.push_back((char)(uint8_t)(v | 0x80));
      v >>= 7;
    }
    s.push_back((char)(uint8_t)v);
  }
  void tag(uint32_t field, int wt) { varint(((uint64_t)field << 3) | (uint64_t)wt); }
  void fixed64(uint64_t v) {
    for (int i = 0; i < 8; ++i) s.push_back((char)(uint8_t)(v >> (8 * i)));
  }
  void doubles(uint32_t field, const double* d, int n) {
    for (int i = 0; i < n; ++i) {
      tag(field, 1);
      fixed64(double_to_bits(d[i]));
    }
  }
  void double1(uint32_t field, double d) { doubles(field, &d, 1); }
  void message(uint32_t field, const std::string& body) {
    tag(field, 2);
    varint(body.size());
    s += body;
  }
  void raw(const uint8_t* a, const uint8_t* b) { s.append((const char*)a, (size_t)(b - a)); }
};

bool read_id(Bytes b, Id* id) {
  Wire w(b);
  std::vector<uint64_t> u;
  uint32_t f;
  int wt;
  while (w.next(&f, &wt)) {
    if (f == 1) {
      if (!w.varints(wt, &u)) return false;
    } else if (!w.skip(wt)) {
      return false;
    }
  }
  if (!w.ok()) return false;
  if (u.empty()) {  // an absent or cleared id: invalid
    id->w[0] = id->w[1] = 0;
    return true;
  }
  if (u.size() != 2) return false;  // aslam::Id::deserialize: exactly two words
  id->w[0] = u[0];
  id->w[1] = u[1];
  return true;
}

// ------------------------------------------------------------------ YAML subset
// Block mappings and sequences by indentation, "- key: value" items, flow
// sequences [a, b, [c, d]], plain and quoted scalars, comments.  Enough for
// the SensorManager files (sensor-manager.cc, aslam ncamera.cc / camera.cc).
struct YNode {
  enum Kind { kNull, kScalar, kMap, kSeq } kind = kNull;
  std::string scalar;
  std::vector<std::pair<std::string, std::unique_ptr<YNode>>> map;
  std::vector<std::unique_ptr<YNode>> seq;
  const YNode* get(const char* key) const {
    if (kind != kMap) return nullptr;
    for (const auto& kv : map)
      if (kv.first == key) return kv.second.get();
    return nullptr;
  }
  bool number(double* v) const {
    if (kind != kScalar || scalar.empty()) return false;
    char* end = nullptr;
    errno = 0;
    *v = std::strtod(scalar.c_str(), &end);
    return end && *end == '\0' && errno == 0;
  }
  bool integer(int64_t* v) const {
    double d;
    if (!number(&d) || d != std::floor(d)) return false;
    *v = (int64_t)d;
    return true;
  }
};

struct YLine {
  int indent;
  std::string text;
};

std::string strip_comment(const std::string& s) {
  bool sq = false, dq = false;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (c == '\'' && !dq) sq = !sq;
    else if (c == '"' && !sq) dq = !dq;
    else if (c == '#' && !sq && !dq && (i == 0 || s[i - 1] == ' ' || s[i - 1] == '\t')) return s.substr(0, i);
  }
  return s;
}

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && (s[a] == ' ' || s[a] == '\t' || s[a] == '\r')) ++a;
  while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\t' || s[b - 1] == '\r')) --b;
  return s.substr(a, b - a);
}

std::string unquote(const std::string& s) {
  if (s.size() >= 2 && ((s.front() == '"' && s.back() == '"') || (s.front() == '\'' && s.back() == '\'')))
    return s.substr(1, s.size() - 2);
  return s;
}

// Position of the ':' that ends a mapping key (followed by a space or the
// end), outside quotes and brackets; npos if the text is not "key: ...".
size_t key_colon(const std::string& s) {
  bool sq = false, dq = false;
  int depth = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (c == '\'' && !dq) sq = !sq;
    else if (c == '"' && !sq) dq = !dq;
    else if (!sq && !dq) {
      if (c == '[' || c == '{') ++depth;
      else if (c == ']' || c == '}') --depth;
      else if (c == ':' && depth == 0 && (i + 1 == s.size() || s[i + 1] == ' ')) return i;
    }
  }
  return std::string::npos;
}

class YParser {
 public:
  explicit YParser(const std::string& text) {
    std::istringstream in(text);
    std::string raw;
    while (std::getline(in, raw)) {
      std::string s = strip_comment(raw);
      if (trim(s).empty() || trim(s) == "---") continue;
      int ind = 0;
      while (ind < (int)s.size() && s[ind] == ' ') ++ind;
      if (ind < (int)s.size() && s[ind] == '\t') {
        ok_ = false;  // tabs are not YAML indentation
        return;
      }
      lines_.push_back({ind, trim(s)});
    }
  }
  bool parse(YNode* root) {
    if (!ok_) return false;
    size_t i = 0;
    if (lines_.empty()) {
      root->kind = YNode::kMap;
      return true;
    }
    if (!block(&i, lines_[0].indent, root)) return false;
    return ok_ && i == lines_.size();
  }

 private:
  // Flow value: scalar or [ ... ] (nested allowed).
  bool flow(const std::string& s, size_t* pos, YNode* n) {
    while (*pos < s.size() && s[*pos] == ' ') ++*pos;
    if (*pos < s.size() && s[*pos] == '[') {
      ++*pos;
      n->kind = YNode::kSeq;
      while (true) {
        while (*pos < s.size() && s[*pos] == ' ') ++*pos;
        if (*pos >= s.size()) return false;
        if (s[*pos] == ']') {
          ++*pos;
          return true;
        }
        auto child = std::make_unique<YNode>();
        if (!flow(s, pos, child.get())) return false;
        n->seq.push_back(std::move(child));
        while (*pos < s.size() && s[*pos] == ' ') ++*pos;
        if (*pos < s.size() && s[*pos] == ',') ++*pos;
      }
    }
    if (*pos < s.size() && s[*pos] == '{') return false;  // flow mappings: not used by the sensor files
    size_t a = *pos;
    bool sq = false, dq = false;
    while (*pos < s.size()) {
      const char c = s[*pos];
      if (c == '\'' && !dq) sq = !sq;
      else if (c == '"' && !sq) dq = !dq;
      else if (!sq && !dq && (c == ',' || c == ']')) break;
      ++*pos;
    }
    n->kind = YNode::kScalar;
    n->scalar = unquote(trim(s.substr(a, *pos - a)));
    return true;
  }
  bool value(const std::string& s, YNode* n) {
    if (s.empty()) {
      n->kind = YNode::kNull;
      return true;
    }
    size_t pos = 0;
    if (!flow(s, &pos, n)) return false;
    while (pos < s.size() && s[pos] == ' ') ++pos;
    return pos == s.size();
  }
  // Children of a "key:" or "-" line with nothing after it: the next lines,
  // if indented deeper (or a sequence at the same indent for a key).
  bool nested(size_t* i, int parent_indent, bool allow_same_indent_seq, YNode* n) {
    if (*i < lines_.size()) {
      const YLine& L = lines_[*i];
      const bool seq_line = L.text == "-" || L.text.compare(0, 2, "- ") == 0;
      if (L.indent > parent_indent || (allow_same_indent_seq && L.indent == parent_indent && seq_line))
        return block(i, L.indent, n);
    }
    n->kind = YNode::kNull;
    return true;
  }
  bool block(size_t* i, int indent, YNode* n) {
    if (++depth_ > 64) return fail();  // the sensor files nest a handful of levels
    struct Leave {
      int& d;
      ~Leave() { --d; }
    } leave{depth_};
    const YLine& first = lines_[*i];
    const bool is_seq = first.text == "-" || first.text.compare(0, 2, "- ") == 0;
    n->kind = is_seq ? YNode::kSeq : YNode::kMap;
    while (*i < lines_.size() && lines_[*i].indent == indent) {
      YLine& L = lines_[*i];
      const bool seq_line = L.text == "-" || L.text.compare(0, 2, "- ") == 0;
      if (seq_line != is_seq) break;
      if (is_seq) {
        auto item = std::make_unique<YNode>();
        const std::string rest = L.text.size() > 1 ? trim(L.text.substr(2)) : std::string();
        if (rest.empty()) {
          ++*i;
          if (!nested(i, indent, false, item.get())) return false;
        } else if (key_colon(rest) != std::string::npos) {
          // "- key: value": a mapping whose entries sit at the column of `key`.
          const int col = indent + (int)(L.text.size() - rest.size());
          L.indent = col;
          L.text = rest;
          if (!block(i, col, item.get())) return false;
        } else {
          if (!value(rest, item.get())) return fail();
          ++*i;
        }
        n->seq.push_back(std::move(item));
      } else {
        const size_t c = key_colon(L.text);
        if (c == std::string::npos) return fail();
        const std::string key = unquote(trim(L.text.substr(0, c)));
        const std::string rest = trim(L.text.substr(c + 1));
        auto child = std::make_unique<YNode>();
        ++*i;
        if (rest.empty()) {
          if (!nested(i, indent, true, child.get())) return false;
        } else if (!value(rest, child.get())) {
          return fail();
        }
        n->map.emplace_back(key, std::move(child));
      }
    }
    if (*i < lines_.size() && lines_[*i].indent > indent) return fail();
    return true;
  }
  bool fail() {
    ok_ = false;
    return false;
  }
  std::vector<YLine> lines_;
  bool ok_ = true;
  int depth_ = 0;
};

// YAML matrix: {rows, cols, data} with data flat or a list of rows (values
// row by row, as yaml-cpp's Eigen conversion reads them), or a bare list.
bool yaml_matrix(const YNode* n, int rows, int cols, double* out) {
  if (!n) return false;
  const YNode* data = n;
  if (n->kind == YNode::kMap) {
    int64_t r = 0, c = 0;
    const YNode* rn = n->get("rows");
    const YNode* cn = n->get("cols");
    if (!rn || !cn || !rn->integer(&r) || !cn->integer(&c) || r != rows || c != cols) return false;
    data = n->get("data");
    if (!data) return false;
  }
  if (data->kind != YNode::kSeq) return false;
  std::vector<double> v;
  for (const auto& e : data->seq) {
    if (e->kind == YNode::kSeq) {
      for (const auto& x : e->seq) {
        double d;
        if (!x->number(&d)) return false;
        v.push_back(d);
      }
    } else {
      double d;
      if (!e->number(&d)) return false;
      v.push_back(d);
    }
  }
  if ((int)v.size() != rows * cols) return false;
  std::copy(v.begin(), v.end(), out);
  return true;
}

// ------------------------------------------------------------------ rotations
// Hamilton quaternions x y z w (Eigen storage order), R(q) active.
void quat_to_R(const double* q, double* R) {
  const double x = q[0], y = q[1], z = q[2], w = q[3];
  R[0] = 1 - 2 * (y * y + z * z); R[1] = 2 * (x * y - z * w);     R[2] = 2 * (x * z + y * w);
  R[3] = 2 * (x * y + z * w);     R[4] = 1 - 2 * (x * x + z * z); R[5] = 2 * (y * z - x * w);
  R[6] = 2 * (x * z - y * w);     R[7] = 2 * (y * z + x * w);     R[8] = 1 - 2 * (x * x + y * y);
}

// Eigen's Quaternion(rotation matrix): Shoemake's trace / largest-diagonal
// method (the published algorithm Eigen implements).
void R_to_quat(const double* m, double* q) {
  const double t = m[0] + m[4] + m[8];
  if (t > 0) {
    double s = std::sqrt(t + 1.0);
    q[3] = 0.5 * s;
    s = 0.5 / s;
    q[0] = (m[7] - m[5]) * s;
    q[1] = (m[2] - m[6]) * s;
    q[2] = (m[3] - m[1]) * s;
  } else {
    int i = 0;
    if (m[4] > m[0]) i = 1;
    if (m[8] > m[3 * i + i]) i = 2;
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    double s = std::sqrt(m[3 * i + i] - m[3 * j + j] - m[3 * k + k] + 1.0);
    q[i] = 0.5 * s;
    s = 0.5 / s;
    q[3] = (m[3 * k + j] - m[3 * j + k]) * s;
    q[j] = (m[3 * j + i] + m[3 * i + j]) * s;
    q[k] = (m[3 * k + i] + m[3 * i + k]) * s;
  }
}

// Eigen's Quaternion::inverse (conjugate over the squared norm).
void quat_inverse(const double* q, double* o) {
  const double n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  o[0] = -q[0] / n2;
  o[1] = -q[1] / n2;
  o[2] = -q[2] / n2;
  o[3] = q[3] / n2;
}

// ensurePositiveQuaternion (optimization-state-buffer.cc): w >= 0.
void ensure_positive(double* q) {
  if (q[3] < 0)
    for (int a = 0; a < 4; ++a) q[a] = -q[a];
}

// 4x4 homogeneous matrix (row-major) -> Hamilton q | p.
void matrix_to_T(const double* M, double* T) {
  const double R[9] = {M[0], M[1], M[2], M[4], M[5], M[6], M[8], M[9], M[10]};
  R_to_quat(R, T);
  T[4] = M[3];
  T[5] = M[7];
  T[6] = M[11];
}

// Inverse of a transformation q | p (Hamilton): q^-1 | -(R^T p).
void T_inverse(const double* T, double* o) {
  double R[9];
  quat_to_R(T, R);
  quat_inverse(T, o);
  for (int i = 0; i < 3; ++i) o[4 + i] = -(R[i] * T[4] + R[3 + i] * T[5] + R[6 + i] * T[6]);
}

// The JPL block q | p of an extrinsic transformation T_X_B (camera T_C_I or
// other sensor T_S_B): q = inverse of the Hamilton rotation, positive w.
void jpl_block(const double* T_X_B, double* out) {
  quat_inverse(T_X_B, out);
  ensure_positive(out);
  for (int i = 0; i < 3; ++i) out[4 + i] = T_X_B[4 + i];
}

// ------------------------------------------------------------------ map model
struct Frame {
  bool set = false;    // frame id valid (an unset frame carries the invalid id)
  bool valid = true;   // is_valid absent or true
  int64_t timestamp_ns = 0;
  std::vector<double> uv;     // 2 per keypoint
  std::vector<double> sigma;  // 1 per keypoint
  std::vector<Id> lm;         // observed landmark per keypoint (may be invalid)
};

struct Backlink {
  Id vertex;
  int32_t frame;
  int32_t keypoint;
};

struct Landmark {
  Id id;
  double p_B[3] = {0, 0, 0};
  int32_t quality = 0;       // kUnknown 0, kBad 1, kGood 2
  int32_t feature_type = 0;  // sensors/external-features.h: kBinary 0, lidar >= 21
  std::vector<Backlink> obs;
};

struct AbsMeas {
  Id sensor;
  int64_t timestamp_ns = 0;
  double T_G_S[7];
  double cov[36];  // column-major as stored
};

struct Vertex {
  Id id, mission;
  double T_M_I[7];
  double v_M[3] = {0, 0, 0}, b_a[3] = {0, 0, 0}, b_g[3] = {0, 0, 0};
  std::vector<Frame> frames;
  std::vector<Landmark> landmarks;
  std::vector<AbsMeas> abs;
  std::vector<Id> outgoing, incoming;
  int file = -1;          // index into the loaded file buffers
  Bytes raw;              // ViwlsVertex message bytes
};

enum EdgeKind { kViwls = 0, kOdometry = 1, kLoopClosure = 2, kWheelOdometry = 3 };

struct Edge {
  Id id, from, to, mission, sensor;
  int kind = kViwls;
  std::vector<int64_t> ts;
  std::vector<double> imu;  // 6 per sample: acc xyz, gyro xyz
  double T_A_B[7] = {0, 0, 0, 1, 0, 0, 0};
  double cov[36];           // column-major as stored
  double switch_variable = 1.0, switch_variance = 0.0;
  int file = -1;
  Bytes raw;                // Edge message bytes
};

struct Mission {
  Id id, baseframe, root;
  int backbone = 0;  // kViwls 0, kOdometry 1
  Id ncamera, imu, odometry, wheel_odometry, absolute, loop_closure;
};

struct Camera {
  Id id;
  mba_camera c;  // intrinsics, distortion, size; q_CI_p_CI filled per export (JPL of T_C_B)
  double T_C_B[7];
};

struct Sensor {
  Id id;
  std::string type;
  // IMU
  double gyro_noise = 0, gyro_bias = 0, acc_noise = 0, acc_bias = 0, gravity = 0;
  bool has_sigmas = false, has_gravity = false;
  // NCAMERA
  std::vector<Camera> cameras;
};

}  // namespace

struct mba_vimap {
  std::vector<std::string> files;          // raw file contents, kept for the save path
  std::vector<std::string> file_names;     // relative names of the vi_map folder
  std::vector<int> file_types;             // VIMapFileType per file
  std::string metadata_text, sensors_text;
  std::vector<Mission> missions;
  IdMap<int> mission_of;
  IdMap<std::array<double, 7>> baseframes;  // T_G_M by baseframe id
  std::vector<Id> baseframe_order;
  std::vector<Vertex> vertices;
  IdMap<int> vertex_of;
  std::vector<Edge> edges;
  IdMap<int> edge_of;
  IdMap<Id> landmark_store;                 // landmark id -> store vertex id (landmark_index)
  IdMap<std::pair<int, int>> landmark_at;   // landmark id -> (vertex, index in its store)
  std::vector<Sensor> sensors;
  IdMap<int> sensor_of;
  IdMap<std::array<double, 7>> T_B_S;        // extrinsics by sensor id
  int64_t legacy_index_ids = 0, index_entries = 0;

  // Last export.
  struct Export {
    std::vector<int> kf_vertex;              // keyframe -> vertex index
    std::vector<std::pair<int, int>> lm;     // landmark -> (vertex, store index)
    std::vector<int> mission;                // problem mission -> map mission
    std::vector<int> pe_kind;                // 0 edge (relative / loop closure), 1 absolute
    std::vector<int> pe_edge;                // edge index or vertex index
    std::vector<int> pe_abs;                 // absolute measurement index within the vertex
    std::vector<double> obs_uv, obs_sigma, lm_p_B, kf_x, kf_v, kf_bg, kf_ba, mis, imu, pe_T, pe_cov, pe_ext, pe_sw,
        pe_swvar;
    std::vector<int32_t> obs_lm, obs_kf, obs_cam, lm_store, kf_mis, e_from, e_to, pe_from, pe_to, pe_type;
    std::vector<int64_t> e_off, ts;
    std::vector<uint32_t> kf_flags;
    std::vector<uint8_t> lm_const;
    std::vector<mba_camera> cams;
    bool valid = false;
  } ex;
};

namespace {

// ------------------------------------------------------------------ message parsers
// Each returns false on malformed input or on a condition the reference's
// deserializer CHECKs.

bool parse_frame(Bytes b, Frame* f) {
  Wire w(b);
  uint32_t fld;
  int wt;
  Id id;
  bool has_valid = false;
  uint64_t valid = 1;
  while (w.next(&fld, &wt)) {
    Bytes sub;
    switch (fld) {
      case 1:
        if (!w.bytes(&sub) || !read_id(sub, &id)) return false;
        break;
      case 2: {
        uint64_t t;
        if (wt != 0 || !w.varint(&t)) return false;
        f->timestamp_ns = (int64_t)t;
        break;
      }
      case 3:
        if (!w.doubles(wt, &f->uv)) return false;
        break;
      case 4:
        if (!w.doubles(wt, &f->sigma)) return false;
        break;
      case 7: {
        Id l;
        if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &l)) return false;
        f->lm.push_back(l);
        break;
      }
      case 9:
        if (wt != 0 || !w.varint(&valid)) return false;
        has_valid = true;
        break;
      default:
        if (!w.skip(wt)) return false;
    }
  }
  if (!w.ok()) return false;
  f->set = id.valid();
  f->valid = !(has_valid && valid == 0);
  if (!f->set) return true;
  if (f->uv.size() != 2 * f->sigma.size()) return false;  // visual-frame-serialization.cc:128-130
  if (f->lm.size() != f->sigma.size()) return false;      // one observed-landmark id per keypoint
  return true;
}

bool parse_nframe(Bytes b, std::vector<Frame>* frames) {
  Wire w(b);
  uint32_t fld;
  int wt;
  while (w.next(&fld, &wt)) {
    if (fld == 2) {
      Bytes sub;
      if (wt != 2 || !w.bytes(&sub)) return false;
      frames->emplace_back();
      if (!parse_frame(sub, &frames->back())) return false;
    } else if (!w.skip(wt)) {
      return false;
    }
  }
  return w.ok() && !frames->empty();  // deserializeVisualNFrame: CHECK_GT(frames_size, 0)
}

bool parse_landmark(Bytes b, Landmark* l) {
  Wire w(b);
  uint32_t fld;
  int wt;
  std::vector<double> pos;
  std::vector<Id> vids;
  std::vector<uint64_t> kps, frs, q;
  bool has_id = false;
  while (w.next(&fld, &wt)) {
    Bytes sub;
    switch (fld) {
      case 1:
        if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &l->id)) return false;
        has_id = true;
        break;
      case 2:
        if (!w.doubles(wt, &pos)) return false;
        break;
      case 4: {
        Id v;
        if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &v)) return false;
        vids.push_back(v);
        break;
      }
      case 5:
        if (!w.varints(wt, &kps)) return false;
        break;
      case 6:
        if (!w.varints(wt, &frs)) return false;
        break;
      case 7:
        if (!w.varints(wt, &q)) return false;
        break;
      case 9: {
        std::vector<uint64_t> t;
        if (!w.varints(wt, &t) || t.empty()) return false;
        l->feature_type = (int32_t)(int64_t)t.back();
        break;
      }
      default:
        if (!w.skip(wt)) return false;
    }
  }
  if (!w.ok() || !has_id || !l->id.valid() || pos.size() != 3) return false;
  if (vids.size() != kps.size()) return false;                // landmark.cc:194
  if (!kps.empty() && frs.size() != kps.size()) return false;  // landmark.cc:201-203
  std::copy(pos.begin(), pos.end(), l->p_B);
  if (!q.empty()) {
    if (q.back() > 2) return false;  // unknown quality value
    l->quality = (int32_t)q.back();
  }
  l->obs.resize(kps.size());
  for (size_t i = 0; i < kps.size(); ++i) l->obs[i] = {vids[i], (int32_t)frs[i], (int32_t)kps[i]};
  return true;
}

bool parse_abs(Bytes b, AbsMeas* a) {
  Wire w(b);
  uint32_t fld;
  int wt;
  std::vector<double> T, C;
  while (w.next(&fld, &wt)) {
    Bytes sub;
    uint64_t v;
    switch (fld) {
      case 1:
        if (wt != 0 || !w.varint(&v)) return false;
        a->timestamp_ns = (int64_t)v;
        break;
      case 2:
        if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &a->sensor)) return false;
        break;
      case 3:
        if (!w.doubles(wt, &T)) return false;
        break;
      case 4:
        if (!w.doubles(wt, &C)) return false;
        break;
      default:
        if (!w.skip(wt)) return false;
    }
  }
  if (!w.ok() || T.size() != 7 || C.size() != 36 || !a->sensor.valid()) return false;
  std::copy(T.begin(), T.end(), a->T_G_S);
  std::copy(C.begin(), C.end(), a->cov);
  for (double c : C)
    if (!std::isfinite(c)) return false;  // optimization-terms-addition.cc: covariance.allFinite()
  return true;
}

bool unit_quaternion(const double* q) {
  const double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  return std::fabs(n - 1.0) <= 1e-4;  // eigen-proto-inl.h: CHECK_NEAR(1, |q|, 1e-4)
}

bool fixed_vector(const std::vector<double>& v, size_t n, double* out) {
  if (v.size() != n) return false;
  std::copy(v.begin(), v.end(), out);
  return true;
}

bool parse_vertex(Bytes b, Vertex* v) {
  Wire w(b);
  uint32_t fld;
  int wt;
  std::vector<double> T, vel, ba, bg;
  bool has_mission = false, has_frames = false, has_store = false;
  while (w.next(&fld, &wt)) {
    Bytes sub;
    Id id;
    switch (fld) {
      case 1:
      case 2:
        if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &id)) return false;
        (fld == 1 ? v->incoming : v->outgoing).push_back(id);
        break;
      case 3:
        if (!w.doubles(wt, &T)) return false;
        break;
      case 4:
        if (!w.doubles(wt, &vel)) return false;
        break;
      case 5:
        if (!w.doubles(wt, &ba)) return false;
        break;
      case 6:
        if (!w.doubles(wt, &bg)) return false;
        break;
      case 7:
        if (wt != 2 || !w.bytes(&sub) || !parse_nframe(sub, &v->frames)) return false;
        has_frames = true;
        break;
      case 8: {
        if (wt != 2 || !w.bytes(&sub)) return false;
        Wire s(sub);
        uint32_t f2;
        int w2;
        while (s.next(&f2, &w2)) {
          Bytes lb;
          if (f2 == 1) {
            if (w2 != 2 || !s.bytes(&lb)) return false;
            v->landmarks.emplace_back();
            if (!parse_landmark(lb, &v->landmarks.back())) return false;
          } else if (!s.skip(w2)) {
            return false;
          }
        }
        if (!s.ok()) return false;
        has_store = true;
        break;
      }
      case 14:
        if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &v->mission)) return false;
        has_mission = true;
        break;
      case 15:
        if (wt != 2 || !w.bytes(&sub)) return false;
        v->abs.emplace_back();
        if (!parse_abs(sub, &v->abs.back())) return false;
        break;
      default:
        if (!w.skip(wt)) return false;
    }
  }
  if (!w.ok() || !has_mission || !has_frames || !has_store) return false;  // vertex.cc:448-469
  if (!fixed_vector(T, 7, v->T_M_I) || !unit_quaternion(v->T_M_I)) return false;
  if (!fixed_vector(vel, 3, v->v_M) || !fixed_vector(ba, 3, v->b_a) || !fixed_vector(bg, 3, v->b_g)) return false;
  for (double x : T) if (!std::isfinite(x)) return false;
  return true;
}

bool parse_pose_edge(Bytes b, Edge* e, bool loop_closure) {
  Wire w(b);
  uint32_t fld;
  int wt;
  std::vector<double> T, C;
  while (w.next(&fld, &wt)) {
    Bytes sub;
    switch (fld) {
      case 1:
        if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &e->from)) return false;
        break;
      case 2:
        if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &e->to)) return false;
        break;
      case 3:
        if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &e->mission)) return false;
        break;
      case 4:
        if (!w.doubles(wt, &T)) return false;
        break;
      case 5:
        if (!w.doubles(wt, &C)) return false;
        break;
      case 6:
        if (loop_closure) {
          if (!w.fixed_double(wt, &e->switch_variable)) return false;
        } else if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &e->sensor)) {
          return false;
        }
        break;
      case 7:
        if (!loop_closure) {
          if (!w.skip(wt)) return false;
        } else if (!w.fixed_double(wt, &e->switch_variance)) {
          return false;
        }
        break;
      default:
        if (!w.skip(wt)) return false;
    }
  }
  if (!w.ok() || !fixed_vector(T, 7, e->T_A_B) || !unit_quaternion(e->T_A_B)) return false;
  return fixed_vector(C, 36, e->cov);
}

bool parse_viwls(Bytes b, Edge* e) {
  Wire w(b);
  uint32_t fld;
  int wt;
  std::vector<uint64_t> ts;
  while (w.next(&fld, &wt)) {
    Bytes sub;
    switch (fld) {
      case 1:
        if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &e->from)) return false;
        break;
      case 2:
        if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &e->to)) return false;
        break;
      case 3:
        if (!w.varints(wt, &ts)) return false;
        break;
      case 4:
        if (!w.doubles(wt, &e->imu)) return false;
        break;
      case 5:
        if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &e->mission)) return false;
        break;
      default:
        if (!w.skip(wt)) return false;
    }
  }
  if (!w.ok() || e->imu.size() != 6 * ts.size()) return false;  // imu_data: 6 x N (viwls-edge.cc:57-58)
  e->ts.assign(ts.begin(), ts.end());
  return true;
}

bool parse_edge(Bytes b, Edge* e) {
  Wire w(b);
  uint32_t fld;
  int wt;
  int kinds = 0;
  while (w.next(&fld, &wt)) {
    Bytes sub;
    if (fld == 1 || fld == 2 || fld == 3 || fld == 7) {
      if (wt != 2 || !w.bytes(&sub)) return false;
      ++kinds;
      if (fld == 1) {
        e->kind = kViwls;
        if (!parse_viwls(sub, e)) return false;
      } else if (fld == 3) {
        e->kind = kLoopClosure;
        if (!parse_pose_edge(sub, e, true)) return false;
      } else {
        e->kind = fld == 2 ? kOdometry : kWheelOdometry;
        if (!parse_pose_edge(sub, e, false)) return false;
      }
    } else if (!w.skip(wt)) {
      return false;
    }
  }
  return w.ok() && kinds == 1;  // edge.cc:72-75: any other edge message is fatal
}

bool parse_mission(Bytes b, Mission* m) {
  Wire w(b);
  uint32_t fld;
  int wt;
  while (w.next(&fld, &wt)) {
    Bytes sub;
    Id* target = nullptr;
    switch (fld) {
      case 1: target = &m->baseframe; break;
      case 2: target = &m->root; break;
      case 8: target = &m->ncamera; break;
      case 9: target = &m->imu; break;
      case 11: target = &m->odometry; break;
      case 12: target = &m->loop_closure; break;
      case 13: target = &m->absolute; break;
      case 15: target = &m->wheel_odometry; break;
      case 3: {
        uint64_t v;
        if (wt != 0 || !w.varint(&v) || v > 1) return false;  // vi-mission.cc:238-252
        m->backbone = (int)v;
        continue;
      }
      default:
        if (!w.skip(wt)) return false;
        continue;
    }
    if (wt != 2 || !w.bytes(&sub) || !read_id(sub, target)) return false;
  }
  return w.ok();
}

bool parse_baseframe(Bytes b, double* T) {
  Wire w(b);
  uint32_t fld;
  int wt;
  std::vector<double> v;
  while (w.next(&fld, &wt)) {
    if (fld == 1) {
      if (!w.doubles(wt, &v)) return false;
    } else if (!w.skip(wt)) {
      return false;
    }
  }
  return w.ok() && fixed_vector(v, 7, T) && unit_quaternion(T);
}

// One VIMap message of a file: entities appended to the map.
bool parse_vimap_file(int file, mba_vimap* M) {
  const std::string& s = M->files[file];
  Bytes all{(const uint8_t*)s.data(), (const uint8_t*)s.data() + s.size()};
  Wire w(all);
  uint32_t fld;
  int wt;
  std::vector<Id> vids, eids, mids, bids;
  std::vector<Bytes> vmsg, emsg, mmsg, bmsg;
  while (w.next(&fld, &wt)) {
    Bytes sub;
    if (fld == 1 || fld == 3 || fld == 5 || fld == 7) {
      Id id;
      if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &id)) return false;
      (fld == 1 ? vids : fld == 3 ? eids : fld == 5 ? mids : bids).push_back(id);
    } else if (fld == 2 || fld == 4 || fld == 6 || fld == 8) {
      if (wt != 2 || !w.bytes(&sub)) return false;
      (fld == 2 ? vmsg : fld == 4 ? emsg : fld == 6 ? mmsg : bmsg).push_back(sub);
    } else if (fld == 9) {
      // Legacy store/global landmark ids: the frames name landmarks by these;
      // after loading, their ids are rewritten from the landmarks' back-links
      // (vi-map-serialization.cc:194-212).
      Id id;
      if (wt != 2 || !w.bytes(&sub) || !read_id(sub, &id)) return false;
      ++M->legacy_index_ids;
    } else if (fld == 10) {
      if (wt != 2 || !w.bytes(&sub)) return false;
      Wire r(sub);
      uint32_t f2;
      int w2;
      Id vtx, lm;
      while (r.next(&f2, &w2)) {
        Bytes x;
        if (f2 == 1 || f2 == 2) {
          if (w2 != 2 || !r.bytes(&x) || !read_id(x, f2 == 1 ? &vtx : &lm)) return false;
        } else if (!r.skip(w2)) {
          return false;
        }
      }
      if (!r.ok() || !vtx.valid() || !lm.valid()) return false;
      M->landmark_store[lm] = vtx;
      ++M->index_entries;
    } else if (!w.skip(wt)) {
      return false;
    }
  }
  if (!w.ok()) return false;
  if (vids.size() != vmsg.size() || eids.size() != emsg.size() || mids.size() != mmsg.size() ||
      bids.size() != bmsg.size())
    return false;  // vi-map-serialization.cc:111, 131, 143-144
  for (size_t i = 0; i < bids.size(); ++i) {
    std::array<double, 7> T;
    if (!bids[i].valid() || !parse_baseframe(bmsg[i], T.data())) return false;
    if (!M->baseframes.emplace(bids[i], T).second) return false;
    M->baseframe_order.push_back(bids[i]);
  }
  for (size_t i = 0; i < mids.size(); ++i) {
    Mission m;
    m.id = mids[i];
    if (!m.id.valid() || !parse_mission(mmsg[i], &m)) return false;
    if (!M->mission_of.emplace(m.id, (int)M->missions.size()).second) return false;
    M->missions.push_back(m);
  }
  for (size_t i = 0; i < vids.size(); ++i) {
    Vertex v;
    v.id = vids[i];
    v.file = file;
    v.raw = vmsg[i];
    if (!v.id.valid() || !parse_vertex(vmsg[i], &v)) return false;
    if (!M->vertex_of.emplace(v.id, (int)M->vertices.size()).second) return false;
    M->vertices.push_back(std::move(v));
  }
  for (size_t i = 0; i < eids.size(); ++i) {
    Edge e;
    e.id = eids[i];
    e.file = file;
    e.raw = emsg[i];
    if (!e.id.valid() || !parse_edge(emsg[i], &e)) return false;
    if (!M->edge_of.emplace(e.id, (int)M->edges.size()).second) return false;
    M->edges.push_back(std::move(e));
  }
  return true;
}

// Text-format VIMapMetadata: files { file_type: N path: "name" } ...
bool parse_metadata(const std::string& text, std::vector<std::pair<int, std::string>>* files) {
  std::vector<std::string> tok;
  for (size_t i = 0; i < text.size();) {
    const char c = text[i];
    if (std::isspace((unsigned char)c)) {
      ++i;
    } else if (c == '#') {
      while (i < text.size() && text[i] != '\n') ++i;
    } else if (c == '{' || c == '}' || c == ':' || c == '<' || c == '>') {
      tok.emplace_back(1, c);
      ++i;
    } else if (c == '"' || c == '\'') {
      size_t j = i + 1;
      std::string s;
      while (j < text.size() && text[j] != c) {
        if (text[j] == '\\' && j + 1 < text.size()) ++j;
        s.push_back(text[j++]);
      }
      if (j >= text.size()) return false;
      tok.push_back("\"" + s);
      i = j + 1;
    } else {
      size_t j = i;
      while (j < text.size() && !std::isspace((unsigned char)text[j]) && std::strchr("{}:<>#\"'", text[j]) == nullptr)
        ++j;
      tok.push_back(text.substr(i, j - i));
      i = j;
    }
  }
  size_t k = 0;
  auto take = [&](const char* s) { return k < tok.size() && tok[k] == s ? (++k, true) : false; };
  while (k < tok.size()) {
    if (!take("files")) return false;
    take(":");
    const bool angle = k < tok.size() && tok[k] == "<";
    if (!take(angle ? "<" : "{")) return false;
    int type = -1;
    std::string path;
    bool has_path = false;
    while (k < tok.size() && tok[k] != (angle ? ">" : "}")) {
      const std::string key = tok[k++];
      if (!take(":") || k >= tok.size()) return false;
      const std::string val = tok[k++];
      if (key == "file_type") {
        char* end = nullptr;
        type = (int)std::strtol(val.c_str(), &end, 10);
        if (!end || *end) return false;
      } else if (key == "path") {
        if (val.empty() || val[0] != '"') return false;
        path = val.substr(1);
        has_path = true;
      }
    }
    if (!take(angle ? ">" : "}") || type < 0 || type > 3 || !has_path) return false;
    files->emplace_back(type, path);
  }
  return true;
}

bool read_file(const std::string& path, std::string* out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  *out = ss.str();
  return (bool)f || f.eof();
}

// sensors.yaml -> sensors and extrinsics (sensor-manager.cc, aslam
// ncamera.cc:120-170, camera.cc:105-230, imu sigmas).
bool parse_sensors(const std::string& text, mba_vimap* M) {
  YNode root;
  YParser p(text);
  if (!p.parse(&root) || root.kind != YNode::kMap) return false;
  const YNode* sensors = root.get("sensors");
  if (sensors && sensors->kind == YNode::kSeq) {
    for (const auto& sn : sensors->seq) {
      if (sn->kind != YNode::kMap) return false;
      Sensor s;
      const YNode* id = sn->get("id");
      const YNode* type = sn->get("sensor_type");
      if (!id || !type || id->kind != YNode::kScalar || !id_from_hex(id->scalar, &s.id)) return false;
      s.type = type->scalar;
      if (s.type == "IMU") {
        const YNode* sig = sn->get("sigmas");
        if (sig) {
          const YNode *gn = sig->get("gyro_noise_density"), *gb = sig->get("gyro_bias_random_walk_noise_density"),
                      *an = sig->get("acc_noise_density"), *ab = sig->get("acc_bias_random_walk_noise_density");
          if (!gn || !gb || !an || !ab || !gn->number(&s.gyro_noise) || !gb->number(&s.gyro_bias) ||
              !an->number(&s.acc_noise) || !ab->number(&s.acc_bias))
            return false;
          s.has_sigmas = true;
        }
        const YNode* g = sn->get("gravity_magnitude_mps2");
        if (g) {
          if (!g->number(&s.gravity)) return false;
          s.has_gravity = true;
        }
      } else if (s.type == "NCAMERA") {
        const YNode* cams = sn->get("cameras");
        if (!cams || cams->kind != YNode::kSeq) return false;
        for (const auto& cn : cams->seq) {
          const YNode* c = cn->get("camera");
          if (!c) return false;
          Camera cam;
          std::memset(&cam.c, 0, sizeof(cam.c));
          const YNode* cid = c->get("id");
          if (cid && (cid->kind != YNode::kScalar || !id_from_hex(cid->scalar, &cam.id))) return false;
          const YNode* ctype = c->get("type");
          if (!ctype || ctype->scalar != "pinhole") return false;  // only the pinhole model is in the BA path
          int64_t wpx = 0, hpx = 0;
          const YNode *wn = c->get("image_width"), *hn = c->get("image_height");
          if (!wn || !hn || !wn->integer(&wpx) || !hn->integer(&hpx)) return false;
          cam.c.width = (int32_t)wpx;
          cam.c.height = (int32_t)hpx;
          if (!yaml_matrix(c->get("intrinsics"), 4, 1, cam.c.intrinsics)) return false;
          const YNode* dist = c->get("distortion");
          cam.c.distortion_type = MBA_DISTORTION_NONE;
          if (dist) {
            const YNode* dt = dist->get("type");
            if (!dt) return false;
            if (dt->scalar == "none") {
              cam.c.distortion_type = MBA_DISTORTION_NONE;
            } else if (dt->scalar == "radial-tangential") {
              cam.c.distortion_type = MBA_DISTORTION_RADTAN;
              if (!yaml_matrix(dist->get("parameters"), 4, 1, cam.c.distortion)) return false;
            } else if (dt->scalar == "equidistant") {
              cam.c.distortion_type = MBA_DISTORTION_EQUIDISTANT;
              if (!yaml_matrix(dist->get("parameters"), 4, 1, cam.c.distortion)) return false;
            } else {
              return false;  // fisheye: not in the BA path
            }
          }
          double Mx[16], T[7];
          if (cn->get("T_B_C")) {
            if (!yaml_matrix(cn->get("T_B_C"), 4, 4, Mx)) return false;
            matrix_to_T(Mx, T);
            T_inverse(T, cam.T_C_B);
          } else if (cn->get("T_C_B")) {
            if (!yaml_matrix(cn->get("T_C_B"), 4, 4, Mx)) return false;
            matrix_to_T(Mx, cam.T_C_B);
          } else {
            return false;
          }
          s.cameras.push_back(cam);
        }
      }
      if (!M->sensor_of.emplace(s.id, (int)M->sensors.size()).second) return false;
      M->sensors.push_back(std::move(s));
    }
  }
  const YNode* ext = root.get("extrinsics");
  if (ext && ext->kind == YNode::kSeq) {
    for (const auto& en : ext->seq) {
      Id sid;
      const YNode* id = en->get("sensor_id");
      double Mx[16];
      std::array<double, 7> T;
      if (!id || !id_from_hex(id->scalar, &sid) || !yaml_matrix(en->get("T_B_S"), 4, 4, Mx)) return false;
      matrix_to_T(Mx, T.data());
      M->T_B_S[sid] = T;
    }
  }
  return true;
}

std::string join(const std::string& a, const std::string& b) { return a.empty() || a.back() == '/' ? a + b : a + "/" + b; }

mba_status load(const char* folder, mba_vimap* M) {
  const std::string dir = join(folder, "vi_map");
  if (!read_file(join(dir, "vi_map_metadata"), &M->metadata_text)) return MBA_ERR_INVALID_ARG;
  if (!read_file(join(dir, "sensors.yaml"), &M->sensors_text)) return MBA_ERR_INVALID_ARG;
  std::vector<std::pair<int, std::string>> files;
  if (!parse_metadata(M->metadata_text, &files) || files.empty()) return MBA_ERR_INVALID_ARG;
  if (!parse_sensors(M->sensors_text, M)) return MBA_ERR_INVALID_ARG;
  // Missions first, then vertices, edges and the landmark index (the order of
  // deserializeFromProtoFromFunction).
  for (int type = 0; type <= 3; ++type) {
    for (const auto& f : files) {
      if (f.first != type) continue;
      if (f.second.find('/') != std::string::npos || f.second == ".." || f.second.empty()) return MBA_ERR_INVALID_ARG;
      std::string data;
      if (!read_file(join(dir, f.second), &data)) return MBA_ERR_INVALID_ARG;
      M->files.push_back(std::move(data));
      M->file_names.push_back(f.second);
      M->file_types.push_back(type);
      if (!parse_vimap_file((int)M->files.size() - 1, M)) return MBA_ERR_INVALID_ARG;
    }
  }
  // Referential integrity (the CHECKs of the deserializers and of VIMap::addVertex / addEdge).
  if (M->missions.size() != M->baseframes.size()) return MBA_ERR_INVALID_ARG;  // one baseframe per mission
  for (const Mission& m : M->missions) {
    if (!M->baseframes.count(m.baseframe)) return MBA_ERR_OUT_OF_RANGE_INDEX;
    if (m.root.valid() && !M->vertex_of.count(m.root)) return MBA_ERR_OUT_OF_RANGE_INDEX;
    if (m.ncamera.valid() && !M->sensor_of.count(m.ncamera)) return MBA_ERR_OUT_OF_RANGE_INDEX;
    if (m.imu.valid() && !M->sensor_of.count(m.imu)) return MBA_ERR_OUT_OF_RANGE_INDEX;
  }
  for (size_t vi = 0; vi < M->vertices.size(); ++vi) {
    Vertex& v = M->vertices[vi];
    auto mi = M->mission_of.find(v.mission);
    if (mi == M->mission_of.end()) return MBA_ERR_OUT_OF_RANGE_INDEX;
    const Mission& mis = M->missions[mi->second];
    if (mis.ncamera.valid()) {
      const Sensor& nc = M->sensors[M->sensor_of[mis.ncamera]];
      if (nc.type != "NCAMERA" || nc.cameras.size() != v.frames.size()) return MBA_ERR_INVALID_ARG;
    }
    for (size_t j = 0; j < v.landmarks.size(); ++j)
      if (!M->landmark_at.emplace(v.landmarks[j].id, std::make_pair((int)vi, (int)j)).second)
        return MBA_ERR_INVALID_ARG;  // a landmark stored twice
  }
  for (const auto& kv : M->landmark_store) {
    auto at = M->landmark_at.find(kv.first);
    if (at != M->landmark_at.end() && M->vertices[at->second.first].id != kv.second)
      return MBA_ERR_INVALID_ARG;  // vi-map-serialization.cc:187: index disagrees with the store
    if (!M->vertex_of.count(kv.second)) return MBA_ERR_OUT_OF_RANGE_INDEX;
  }
  for (const auto& kv : M->landmark_at) M->landmark_store[kv.first] = M->vertices[kv.second.first].id;
  if (M->legacy_index_ids > 0) {
    if (M->legacy_index_ids != M->index_entries) return MBA_ERR_INVALID_ARG;  // vi-map-serialization.cc:198
    // Every observation names its landmark by the landmark's own id again.
    for (const Vertex& sv : M->vertices)
      for (const Landmark& L : sv.landmarks)
        for (const Backlink& b : L.obs) {
          auto vi = M->vertex_of.find(b.vertex);
          if (vi == M->vertex_of.end()) return MBA_ERR_OUT_OF_RANGE_INDEX;
          Vertex& ov = M->vertices[vi->second];
          if (b.frame < 0 || b.frame >= (int32_t)ov.frames.size()) return MBA_ERR_OUT_OF_RANGE_INDEX;
          Frame& f = ov.frames[b.frame];
          if (b.keypoint < 0 || b.keypoint >= (int32_t)f.lm.size()) return MBA_ERR_OUT_OF_RANGE_INDEX;
          f.lm[b.keypoint] = L.id;
        }
  }
  for (const Vertex& v : M->vertices) {  // Vertex::incoming / outgoing name existing edges
    for (const Id& id : v.outgoing)
      if (!M->edge_of.count(id)) return MBA_ERR_OUT_OF_RANGE_INDEX;
    for (const Id& id : v.incoming)
      if (!M->edge_of.count(id)) return MBA_ERR_OUT_OF_RANGE_INDEX;
  }
  for (const Edge& e : M->edges) {
    if (!M->vertex_of.count(e.from) || !M->vertex_of.count(e.to)) return MBA_ERR_OUT_OF_RANGE_INDEX;
    if (e.kind == kViwls)
      for (size_t j = 1; j < e.ts.size(); ++j)
        if (e.ts[j] < e.ts[j - 1]) return MBA_ERR_UNORDERED_IMU;
  }
  return MBA_OK;
}

}  // namespace

namespace {

// ------------------------------------------------------------------ export helpers
void rot(const double* R, const double* x, double* y) {
  for (int i = 0; i < 3; ++i) y[i] = R[3 * i] * x[0] + R[3 * i + 1] * x[1] + R[3 * i + 2] * x[2];
}
void rotT(const double* R, const double* x, double* y) {
  for (int i = 0; i < 3; ++i) y[i] = R[i] * x[0] + R[3 + i] * x[1] + R[6 + i] * x[2];
}

const Camera* camera_of(const mba_vimap* M, const Vertex& v, int frame) {
  const Mission& m = M->missions[M->mission_of.at(v.mission)];
  if (!m.ncamera.valid()) return nullptr;
  const Sensor& nc = M->sensors[M->sensor_of.at(m.ncamera)];
  if (frame < 0 || frame >= (int)nc.cameras.size()) return nullptr;
  return &nc.cameras[frame];
}

// Squared pixel error of p_C against a keypoint (computeSquaredReprojectionError,
// landmark-quality-metrics.cc:57-73): pinhole projection with the camera's
// distortion (camera-pinhole.cc:65-164, distortion-radtan.cc:14-65,
// distortion-equidistant.cc:14-50); points not in front of the camera give
// the largest double.  Keypoints outside the image box still count.
double reprojection_sq(const mba_camera& c, const double* pC, double u, double v) {
  if (!(pC[2] > 1e-10)) return std::numeric_limits<double>::max();
  const double rz = 1.0 / pC[2];
  double x = pC[0] * rz, y = pC[1] * rz;
  const double* k = c.distortion;
  if (c.distortion_type == MBA_DISTORTION_RADTAN) {
    const double xx = x * x, yy = y * y, xy = x * y, r2 = xx + yy;
    const double rad = k[0] * r2 + k[1] * r2 * r2;
    const double nx = x + x * rad + 2.0 * k[2] * xy + k[3] * (r2 + 2.0 * xx);
    const double ny = y + y * rad + 2.0 * k[3] * xy + k[2] * (r2 + 2.0 * yy);
    x = nx;
    y = ny;
  } else if (c.distortion_type == MBA_DISTORTION_EQUIDISTANT) {
    const double r = std::sqrt(x * x + y * y);
    if (r >= 1e-10) {
      const double th = std::atan(r), t2 = th * th, t4 = t2 * t2, t6 = t2 * t4, t8 = t4 * t4;
      const double thd = th * (1 + k[0] * t2 + k[1] * t4 + k[2] * t6 + k[3] * t8);
      const double s = thd / r;
      x *= s;
      y *= s;
    }
  }
  const double du = c.intrinsics[0] * x + c.intrinsics[2] - u, dv = c.intrinsics[1] * y + c.intrinsics[3] - v;
  return du * du + dv * dv;
}

// isVisualLandmarkWellConstrained (landmark-quality-metrics.cc:105-172) on
// the map: observers from the landmark's back-links, camera centres and the
// landmark in G through the Hamilton T_G_M, T_M_I and T_B_C of the map.
// Returns -1 when a back-link names a vertex or camera that does not exist.
int well_constrained(const mba_vimap* M, const Landmark& L, const Vertex& store,
                     const mba_landmark_quality_options& q) {
  if ((int64_t)L.obs.size() < q.min_observers || L.obs.empty()) return 0;
  double R[9], pM[3], pG[3];
  const double* Tm = M->baseframes.at(M->missions[M->mission_of.at(store.mission)].baseframe).data();
  quat_to_R(store.T_M_I, R);
  rot(R, L.p_B, pM);
  for (int i = 0; i < 3; ++i) pM[i] += store.T_M_I[4 + i];
  quat_to_R(Tm, R);
  rot(R, pM, pG);
  for (int i = 0; i < 3; ++i) pG[i] += Tm[4 + i];
  std::vector<std::array<double, 3>> rays;
  double min_sd = std::numeric_limits<double>::max();
  for (const Backlink& b : L.obs) {
    auto vi = M->vertex_of.find(b.vertex);
    if (vi == M->vertex_of.end()) return -1;
    const Vertex& ov = M->vertices[vi->second];
    const Camera* cam = camera_of(M, ov, b.frame);
    if (!cam) return -1;
    const double* Tg = M->baseframes.at(M->missions[M->mission_of.at(ov.mission)].baseframe).data();
    double RCB[9], RMI[9], RGM[9], cI[3], cM[3], cG[3], a[3], b3[3], pI[3], pC[3];
    quat_to_R(cam->T_C_B, RCB);
    quat_to_R(ov.T_M_I, RMI);
    quat_to_R(Tg, RGM);
    rotT(RCB, cam->T_C_B + 4, cI);  // camera centre in I: -R_C_B^T p_C_B
    for (int i = 0; i < 3; ++i) cI[i] = -cI[i];
    rot(RMI, cI, cM);
    for (int i = 0; i < 3; ++i) cM[i] += ov.T_M_I[4 + i];
    rot(RGM, cM, cG);
    for (int i = 0; i < 3; ++i) cG[i] += Tg[4 + i];
    for (int i = 0; i < 3; ++i) a[i] = pG[i] - Tg[4 + i];
    rotT(RGM, a, b3);
    for (int i = 0; i < 3; ++i) b3[i] -= ov.T_M_I[4 + i];
    rotT(RMI, b3, pI);
    rot(RCB, pI, pC);
    for (int i = 0; i < 3; ++i) pC[i] += cam->T_C_B[4 + i];
    const double r[3] = {cG[0] - pG[0], cG[1] - pG[1], cG[2] - pG[2]};
    const double d = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    min_sd = std::min(min_sd, pC[2] < 0.0 ? -d : d);
    if (d > 0) rays.push_back({r[0] / d, r[1] / d, r[2] / d});
    if (q.max_reprojection_error_px > 0.0) {
      const Frame& fr = ov.frames[b.frame];
      if (!fr.set || b.keypoint < 0 || b.keypoint >= (int32_t)fr.sigma.size()) return -1;
      mba_camera cc = cam->c;
      const double e2 = reprojection_sq(cc, pC, fr.uv[2 * b.keypoint], fr.uv[2 * b.keypoint + 1]);
      if (e2 > q.max_reprojection_error_px * q.max_reprojection_error_px) return 0;
    }
  }
  if (min_sd > q.max_distance_from_closest_observer || min_sd < q.min_distance_from_closest_observer) return 0;
  double min_cos = 1.0;
  for (size_t x = 0; x < rays.size(); ++x)
    for (size_t y = x + 1; y < rays.size(); ++y)
      min_cos = std::min(min_cos, std::fabs(rays[x][0] * rays[y][0] + rays[x][1] * rays[y][1] + rays[x][2] * rays[y][2]));
  const double angle = rays.size() < 2 ? 0.0 : std::acos(min_cos) * (180.0 / M_PI);
  return angle < q.min_observation_angle_deg ? 0 : 1;
}

// Column-major 6x6 (as stored) -> row-major.
void cov_row_major(const double* cm, double* rm) {
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) rm[6 * r + c] = cm[6 * c + r];
}

template <typename T>
const T* ptr_or_null(const std::vector<T>& v) {
  return v.empty() ? nullptr : v.data();
}

mba_status do_export(mba_vimap* M, const mba_vimap_export_options& o, mba_problem_desc* d) {
  M->ex = mba_vimap::Export();
  mba_vimap::Export& X = M->ex;
  // ---- missions
  std::vector<int> sel;
  if (o.num_missions > 0) {
    if (!o.missions) return MBA_ERR_INVALID_ARG;
    std::vector<char> seen(M->missions.size(), 0);
    for (int i = 0; i < o.num_missions; ++i) {
      const int mi = o.missions[i];
      if (mi < 0 || mi >= (int)M->missions.size()) return MBA_ERR_OUT_OF_RANGE_INDEX;
      if (seen[mi]++) return MBA_ERR_INVALID_ARG;
      sel.push_back(mi);
    }
  } else {
    for (int i = 0; i < (int)M->missions.size(); ++i) sel.push_back(i);
  }
  if (sel.empty()) return MBA_ERR_INVALID_ARG;  // VIMapOptimizer::optimize: no missions
  std::vector<int> pm_of(M->missions.size(), -1);
  for (size_t p = 0; p < sel.size(); ++p) pm_of[sel[p]] = (int)p;
  X.mission = sel;
  if (o.landmark_selection < 0 || o.landmark_selection > 2) return MBA_ERR_INVALID_ARG;
  if (o.landmark_selection == MBA_VIMAP_LANDMARKS_MASK && !o.landmark_keep) return MBA_ERR_INVALID_ARG;

  // ---- keyframes along each mission's backbone
  IdMap<int> kf_of;
  std::vector<std::vector<int>> mission_kfs(sel.size());
  for (size_t p = 0; p < sel.size(); ++p) {
    const Mission& m = M->missions[sel[p]];
    if (!m.root.valid()) continue;
    const int backbone_kind = m.backbone == 0 ? kViwls : kOdometry;
    int cur = M->vertex_of.at(m.root);
    while (cur >= 0) {
      const Vertex& v = M->vertices[cur];
      if (v.mission != m.id) return MBA_ERR_INVALID_ARG;  // vi-map.cc:2304
      if (!kf_of.emplace(v.id, (int)X.kf_vertex.size()).second) return MBA_ERR_INVALID_ARG;  // backbone cycle
      mission_kfs[p].push_back((int)X.kf_vertex.size());
      X.kf_vertex.push_back(cur);
      int next = -1;
      for (const Id& eid : v.outgoing) {
        auto ei = M->edge_of.find(eid);
        if (ei == M->edge_of.end()) return MBA_ERR_OUT_OF_RANGE_INDEX;
        const Edge& e = M->edges[ei->second];
        if (e.kind == backbone_kind && e.from == v.id) {
          next = M->vertex_of.at(e.to);
          break;
        }
      }
      cur = next;
    }
  }
  const int64_t NK = (int64_t)X.kf_vertex.size();
  if (NK == 0) return MBA_ERR_INVALID_ARG;
  X.kf_x.resize(7 * NK);
  X.kf_v.resize(3 * NK);
  X.kf_bg.resize(3 * NK);
  X.kf_ba.resize(3 * NK);
  X.kf_mis.resize(NK);
  X.kf_flags.assign(NK, 0u);
  for (int64_t k = 0; k < NK; ++k) {
    const Vertex& v = M->vertices[X.kf_vertex[k]];
    // importKeyframePosesOfMissions: JPL q_IM = Hamilton q_M_I coefficient
    // for coefficient (positive w), then p_M_I.
    double q[4] = {v.T_M_I[0], v.T_M_I[1], v.T_M_I[2], v.T_M_I[3]};
    ensure_positive(q);
    for (int a = 0; a < 4; ++a) X.kf_x[7 * k + a] = q[a];
    for (int a = 0; a < 3; ++a) {
      X.kf_x[7 * k + 4 + a] = v.T_M_I[4 + a];
      X.kf_v[3 * k + a] = v.v_M[a];
      X.kf_bg[3 * k + a] = v.b_g[a];
      X.kf_ba[3 * k + a] = v.b_a[a];
    }
    X.kf_mis[k] = pm_of[M->mission_of.at(v.mission)];
    uint32_t f = 0;
    if (o.fix_vertices) f |= MBA_KF_POSE_CONSTANT;
    if (o.fix_velocity) f |= MBA_KF_VELOCITY_CONSTANT;
    if (o.fix_gyro_bias) f |= MBA_KF_GYRO_BIAS_CONSTANT;
    if (o.fix_accel_bias) f |= MBA_KF_ACCEL_BIAS_CONSTANT;
    X.kf_flags[k] = f;
  }

  // ---- baseframes (importBaseframePoseOfMissions: JPL q_GM = inverse of the
  // Hamilton q_G_M, positive w) and cameras (importCameraCalibrationsOfMissions).
  X.mis.resize(7 * sel.size());
  std::vector<int> cam_base(sel.size(), -1);
  IdMap<int> ncamera_base;
  for (size_t p = 0; p < sel.size(); ++p) {
    const Mission& m = M->missions[sel[p]];
    const double* T = M->baseframes.at(m.baseframe).data();
    jpl_block(T, &X.mis[7 * p]);
    if (!m.ncamera.valid()) continue;
    auto it = ncamera_base.find(m.ncamera);
    if (it != ncamera_base.end()) {
      cam_base[p] = it->second;
      continue;
    }
    const Sensor& nc = M->sensors[M->sensor_of.at(m.ncamera)];
    cam_base[p] = (int)X.cams.size();
    ncamera_base.emplace(m.ncamera, cam_base[p]);
    for (const Camera& c : nc.cameras) {
      mba_camera mc = c.c;
      jpl_block(c.T_C_B, mc.q_CI_p_CI);
      X.cams.push_back(mc);
    }
  }
  if (X.cams.size() > 255) return MBA_ERR_INVALID_ARG;

  // ---- landmarks and observations (addLandmarkTerms,
  // optimization-terms-addition.cc:242-350)
  std::vector<int64_t> lm_base(M->vertices.size() + 1, 0);
  for (size_t vi = 0; vi < M->vertices.size(); ++vi) lm_base[vi + 1] = lm_base[vi] + (int64_t)M->vertices[vi].landmarks.size();
  std::vector<int8_t> keep(lm_base.back(), -1);  // -1 undecided
  bool bad_backlink = false;
  auto kept = [&](int vi, int j) -> bool {
    int8_t& k = keep[lm_base[vi] + j];
    if (k < 0) {
      const Landmark& L = M->vertices[vi].landmarks[j];
      bool good;
      if (L.feature_type >= 21) good = false;  // LiDAR landmark: not a visual term
      else if (o.feature_type != -1 && L.feature_type != o.feature_type) good = false;
      else if (o.landmark_selection == MBA_VIMAP_LANDMARKS_ALL) good = true;
      else if (o.landmark_selection == MBA_VIMAP_LANDMARKS_MASK) good = o.landmark_keep[lm_base[vi] + j] != 0;
      else if (L.quality == 2) good = true;
      else if (L.quality == 1) good = false;
      else {
        const int w = well_constrained(M, L, M->vertices[vi], o.quality);
        if (w < 0) bad_backlink = true;
        good = w == 1;
      }
      k = good ? 1 : 0;
    }
    return k == 1;
  };
  struct ObsRec {
    int32_t kf, cam;
    int vi, j;
    double u, v, sigma;
  };
  std::vector<ObsRec> obs;
  if (o.add_visual_constraints) {
    for (size_t p = 0; p < sel.size(); ++p) {
      for (int k : mission_kfs[p]) {
        const Vertex& v = M->vertices[X.kf_vertex[k]];
        for (size_t f = 0; f < v.frames.size(); ++f) {
          const Frame& fr = v.frames[f];
          if (!fr.set || !fr.valid) continue;
          if (cam_base[p] < 0) return MBA_ERR_INVALID_ARG;  // visual frames without an ncamera
          auto resolve = [&](const Id& lid, int* vi, int* j) -> mba_status {
            auto st = M->landmark_store.find(lid);
            if (st == M->landmark_store.end()) return MBA_ERR_OUT_OF_RANGE_INDEX;
            auto at = M->landmark_at.find(lid);
            if (at == M->landmark_at.end()) return MBA_ERR_OUT_OF_RANGE_INDEX;
            *vi = at->second.first;
            *j = at->second.second;
            return MBA_OK;
          };
          if (o.min_landmarks_per_frame > 0) {
            int good = 0;
            for (const Id& lid : fr.lm) {
              int vi, j;
              if (!lid.valid() || resolve(lid, &vi, &j) != MBA_OK) continue;
              good += kept(vi, j) ? 1 : 0;
            }
            if (good < o.min_landmarks_per_frame) continue;
          }
          for (size_t i = 0; i < fr.lm.size(); ++i) {
            const Id& lid = fr.lm[i];
            if (!lid.valid()) continue;
            int vi, j;
            const mba_status s = resolve(lid, &vi, &j);
            if (s != MBA_OK) return s;
            const Vertex& sv = M->vertices[vi];
            if (pm_of[M->mission_of.at(sv.mission)] < 0) continue;  // store vertex outside the missions
            if (!kept(vi, j)) continue;
            if (!kf_of.count(sv.id)) return MBA_ERR_INVALID_ARG;  // store vertex not on its mission's backbone
            obs.push_back({(int32_t)k, (int32_t)(cam_base[p] + (int)f), vi, (int)j, fr.uv[2 * i], fr.uv[2 * i + 1],
                           fr.sigma[i]});
          }
        }
      }
    }
  }
  if (bad_backlink) return MBA_ERR_OUT_OF_RANGE_INDEX;
  // Landmarks that carry at least one term, in store-keyframe then store order.
  std::vector<int32_t> lm_index(lm_base.back(), -1);
  for (const ObsRec& r : obs) lm_index[lm_base[r.vi] + r.j] = 0;
  for (int64_t k = 0; k < NK; ++k) {
    const int vi = X.kf_vertex[k];
    for (size_t j = 0; j < M->vertices[vi].landmarks.size(); ++j) {
      int32_t& li = lm_index[lm_base[vi] + j];
      if (li < 0) continue;
      li = (int32_t)X.lm.size();
      X.lm.emplace_back(vi, (int)j);
      const double* pB = M->vertices[vi].landmarks[j].p_B;
      X.lm_p_B.insert(X.lm_p_B.end(), pB, pB + 3);
      X.lm_store.push_back((int32_t)k);
    }
  }
  X.lm_const.assign(X.lm.size(), o.fix_landmark_positions ? 1 : 0);
  for (const ObsRec& r : obs) {
    X.obs_uv.push_back(r.u);
    X.obs_uv.push_back(r.v);
    X.obs_sigma.push_back(r.sigma);
    X.obs_lm.push_back(lm_index[lm_base[r.vi] + r.j]);
    X.obs_kf.push_back(r.kf);
    X.obs_cam.push_back(r.cam);
  }

  // ---- inertial edges (addInertialTerms, :370-495): outgoing viwls edges of
  // the backbone vertices; IMU sigmas of the missions' IMU.
  bool have_imu = false;
  double sig[4] = {0, 0, 0, 0}, gimu = 0.0;
  X.e_off.push_back(0);
  auto outgoing_of_kind = [&](int kind, const std::function<mba_status(const Edge&, int)>& fn) -> mba_status {
    for (size_t p = 0; p < sel.size(); ++p)
      for (int k : mission_kfs[p])
        for (const Id& eid : M->vertices[X.kf_vertex[k]].outgoing) {
          const Edge& e = M->edges[M->edge_of.at(eid)];
          if (e.kind != kind || e.from != M->vertices[X.kf_vertex[k]].id) continue;
          const mba_status s = fn(e, (int)p);
          if (s != MBA_OK) return s;
        }
    return MBA_OK;
  };
  if (o.add_inertial_constraints) {
    const mba_status s = outgoing_of_kind(kViwls, [&](const Edge& e, int p) -> mba_status {
      auto ft = kf_of.find(e.to);
      if (ft == kf_of.end()) return MBA_ERR_INVALID_ARG;
      const Mission& m = M->missions[sel[p]];
      if (!m.imu.valid()) return MBA_ERR_INVALID_ARG;
      const Sensor& imu = M->sensors[M->sensor_of.at(m.imu)];
      if (imu.type != "IMU" || !imu.has_sigmas) return MBA_ERR_INVALID_ARG;
      const double s4[4] = {imu.gyro_noise, imu.gyro_bias, imu.acc_noise, imu.acc_bias};
      if (!have_imu) {
        std::copy(s4, s4 + 4, sig);
        gimu = imu.has_gravity ? imu.gravity : 0.0;
        have_imu = true;
      } else if (!std::equal(s4, s4 + 4, sig)) {
        return MBA_ERR_INVALID_ARG;  // one set of IMU sigmas per problem
      }
      X.e_from.push_back(kf_of.at(e.from));
      X.e_to.push_back(ft->second);
      X.ts.insert(X.ts.end(), e.ts.begin(), e.ts.end());
      X.imu.insert(X.imu.end(), e.imu.begin(), e.imu.end());
      X.e_off.push_back((int64_t)X.ts.size());
      return MBA_OK;
    });
    if (s != MBA_OK) return s;
  }

  // ---- pose edges in the builder's order: wheel odometry, 6-DoF odometry
  // (addRelativePoseTermsForEdges, :543-640), absolute (:650-738), loop
  // closures (augment-loopclosure.cc:165-194).
  auto sensor_block = [&](const Id& sid, double* out) -> mba_status {
    auto it = M->T_B_S.find(sid);
    if (!sid.valid() || it == M->T_B_S.end()) return MBA_ERR_OUT_OF_RANGE_INDEX;
    double T_S_B[7];
    T_inverse(it->second.data(), T_S_B);  // importOtherSensorExtrinsicsOfMissions
    jpl_block(T_S_B, out);
    return MBA_OK;
  };
  auto push_pe = [&](int type, int32_t from, int32_t to, const double* T, const double* cov_cm, const double* ext,
                     double sw, double swvar, int kind, int ref, int abs_i) {
    X.pe_type.push_back(type);
    X.pe_from.push_back(from);
    X.pe_to.push_back(to);
    X.pe_T.insert(X.pe_T.end(), T, T + 7);
    double rm[36];
    cov_row_major(cov_cm, rm);
    X.pe_cov.insert(X.pe_cov.end(), rm, rm + 36);
    X.pe_ext.insert(X.pe_ext.end(), ext, ext + 7);
    X.pe_sw.push_back(sw);
    X.pe_swvar.push_back(swvar);
    X.pe_kind.push_back(kind);
    X.pe_edge.push_back(ref);
    X.pe_abs.push_back(abs_i);
  };
  for (int pass = 0; pass < 2; ++pass) {
    const bool on = pass == 0 ? o.add_wheel_odometry_constraints : o.add_6dof_odometry_constraints;
    if (!on) continue;
    const mba_status s = outgoing_of_kind(pass == 0 ? kWheelOdometry : kOdometry, [&](const Edge& e, int) -> mba_status {
      auto ft = kf_of.find(e.to);
      if (ft == kf_of.end()) return MBA_ERR_INVALID_ARG;
      if (M->vertices[M->vertex_of.at(e.from)].mission != M->vertices[M->vertex_of.at(e.to)].mission)
        return MBA_ERR_INVALID_ARG;  // optimization-terms-addition.cc:581-583
      double ext[7];
      const mba_status st = sensor_block(e.sensor, ext);
      if (st != MBA_OK) return st;
      push_pe(MBA_POSE_EDGE_RELATIVE, kf_of.at(e.from), ft->second, e.T_A_B, e.cov, ext, 1.0, 0.0, 0,
              M->edge_of.at(e.id), -1);
      return MBA_OK;
    });
    if (s != MBA_OK) return s;
  }
  if (o.add_absolute_pose_constraints) {
    for (size_t p = 0; p < sel.size(); ++p) {
      const Mission& m = M->missions[sel[p]];
      if (!m.absolute.valid()) continue;
      double ext[7];
      const mba_status st = sensor_block(m.absolute, ext);
      if (st != MBA_OK) return st;
      for (int k : mission_kfs[p]) {
        const Vertex& v = M->vertices[X.kf_vertex[k]];
        // Vertex::getMinTimestampNanoseconds: the earliest set frame.
        int64_t min_ts = std::numeric_limits<int64_t>::max();
        for (const Frame& f : v.frames)
          if (f.set) min_ts = std::min(min_ts, f.timestamp_ns);
        for (size_t a = 0; a < v.abs.size(); ++a) {
          if (v.abs[a].sensor != m.absolute) return MBA_ERR_INVALID_ARG;  // :684-687
          if (v.abs[a].timestamp_ns != min_ts) return MBA_ERR_INVALID_ARG;  // :688-693
          push_pe(MBA_POSE_EDGE_ABSOLUTE, k, k, v.abs[a].T_G_S, v.abs[a].cov, ext, 1.0, 0.0, 1, X.kf_vertex[k],
                  (int)a);
        }
      }
    }
  }
  if (o.add_loop_closure_edges) {
    const double ident[7] = {0, 0, 0, 1, 0, 0, 0};
    for (size_t ei = 0; ei < M->edges.size(); ++ei) {
      const Edge& e = M->edges[ei];
      if (e.kind != kLoopClosure) continue;
      const Vertex& vf = M->vertices[M->vertex_of.at(e.from)];
      const Vertex& vt = M->vertices[M->vertex_of.at(e.to)];
      if (pm_of[M->mission_of.at(vf.mission)] < 0 || pm_of[M->mission_of.at(vt.mission)] < 0) continue;
      auto ff = kf_of.find(e.from), ft = kf_of.find(e.to);
      if (ff == kf_of.end() || ft == kf_of.end()) return MBA_ERR_INVALID_ARG;
      push_pe(MBA_POSE_EDGE_LOOP_CLOSURE, ff->second, ft->second, e.T_A_B, e.cov, ident, e.switch_variable,
              e.switch_variance, 0, (int)ei, -1);
    }
  }

  // ---- descriptor
  std::memset(d, 0, sizeof(*d));
  d->num_keyframes = NK;
  d->num_landmarks = (int64_t)X.lm.size();
  d->num_observations = (int64_t)X.obs_lm.size();
  d->num_cameras = (int64_t)X.cams.size();
  d->num_missions = (int64_t)sel.size();
  d->num_imu_edges = (int64_t)X.e_from.size();
  d->num_imu_samples = (int64_t)X.ts.size();
  d->obs_uv = ptr_or_null(X.obs_uv);
  d->obs_sigma = ptr_or_null(X.obs_sigma);
  d->obs_landmark = ptr_or_null(X.obs_lm);
  d->obs_keyframe = ptr_or_null(X.obs_kf);
  d->obs_camera = ptr_or_null(X.obs_cam);
  d->lm_p_B = ptr_or_null(X.lm_p_B);
  d->lm_store_keyframe = ptr_or_null(X.lm_store);
  d->lm_constant = ptr_or_null(X.lm_const);
  d->kf_q_IM_p_MI = X.kf_x.data();
  d->kf_v_M = X.kf_v.data();
  d->kf_b_g = X.kf_bg.data();
  d->kf_b_a = X.kf_ba.data();
  d->kf_mission = X.kf_mis.data();
  d->kf_flags = X.kf_flags.data();
  d->mission_q_GM_p_GM = X.mis.data();
  if (X.cams.empty()) {  // the descriptor needs one camera; a pose-graph-only problem gets a placeholder
    mba_camera c;
    std::memset(&c, 0, sizeof(c));
    c.intrinsics[0] = c.intrinsics[1] = 1.0;
    c.width = c.height = 1;
    c.q_CI_p_CI[3] = 1.0;
    X.cams.push_back(c);
    d->num_cameras = 1;
  }
  d->cameras = X.cams.data();
  d->edge_from = ptr_or_null(X.e_from);
  d->edge_to = ptr_or_null(X.e_to);
  d->edge_sample_offset = X.e_off.data();
  d->imu_timestamp_ns = ptr_or_null(X.ts);
  d->imu_acc_gyro = ptr_or_null(X.imu);
  d->gyro_noise_sigma = sig[0];
  d->gyro_bias_sigma = sig[1];
  d->acc_noise_sigma = sig[2];
  d->acc_bias_sigma = sig[3];
  d->gravity_magnitude = o.gravity_magnitude > 0.0 ? o.gravity_magnitude : gimu;
  d->use_huber = o.use_huber;
  d->huber_delta_local = 3.0;
  d->huber_delta_global = 10.0;
  d->num_pose_edges = (int64_t)X.pe_type.size();
  d->pose_edge_from = ptr_or_null(X.pe_from);
  d->pose_edge_to = ptr_or_null(X.pe_to);
  d->pose_edge_T_Bk_Bkp1 = ptr_or_null(X.pe_T);
  d->pose_edge_covariance = ptr_or_null(X.pe_cov);
  d->pose_edge_q_I_B_p_B_I = ptr_or_null(X.pe_ext);
  d->pose_edge_type = ptr_or_null(X.pe_type);
  d->pose_edge_switch = ptr_or_null(X.pe_sw);
  d->pose_edge_switch_variance = ptr_or_null(X.pe_swvar);
  if (o.apply_gauge_fixes) {
    std::vector<uint32_t> f(NK);
    std::vector<uint8_t> c(std::max<size_t>(1, X.lm.size()));
    int32_t nc = 0;
    const mba_status s = mba_gauge_fixes(d, f.data(), c.data(), &nc);
    if (s != MBA_OK) return s;
    X.kf_flags = f;
    X.lm_const.assign(c.begin(), c.begin() + X.lm.size());
    d->kf_flags = X.kf_flags.data();
    d->lm_constant = ptr_or_null(X.lm_const);
  }
  X.valid = true;
  return MBA_OK;
}

// ------------------------------------------------------------------ save
// Copies message `b` field by field; `repl(field, wire type, payload)`
// returns 1 to drop the field, 2 if it wrote a replacement, 0 to copy it.
template <typename F>
bool rewrite(Bytes b, Out* out, F repl) {
  Wire w(b);
  uint32_t f;
  int wt;
  while (true) {
    const uint8_t* start = w.pos();
    if (!w.next(&f, &wt)) break;
    const uint8_t* body = w.pos();
    if (!w.skip(wt)) return false;
    Bytes payload{body, w.pos()};
    if (wt == 2) {  // strip the length prefix
      Wire l(payload);
      Bytes inner;
      if (!l.bytes(&inner)) return false;
      payload = inner;
    }
    const int r = repl(f, wt, payload, out);
    if (r < 0) return false;
    if (r == 0) out->raw(start, w.pos());
  }
  return w.ok();
}

bool rewrite_landmark(Bytes b, const Landmark& L, std::string* o) {
  Out out;
  bool done = false;
  if (!rewrite(b, &out, [&](uint32_t f, int, Bytes, Out* ou) -> int {
        if (f != 2) return 0;
        if (done) return 1;
        ou->doubles(2, L.p_B, 3);
        done = true;
        return 2;
      }))
    return false;
  *o = out.s;
  return true;
}

bool rewrite_vertex(const Vertex& v, std::string* o) {
  Out out;
  bool done[7] = {false, false, false, false, false, false, false};
  const bool ok = rewrite(v.raw, &out, [&](uint32_t f, int, Bytes payload, Out* ou) -> int {
    if (f >= 3 && f <= 6) {
      if (done[f]) return 1;
      done[f] = true;
      if (f == 3) ou->doubles(3, v.T_M_I, 7);
      if (f == 4) ou->doubles(4, v.v_M, 3);
      if (f == 5) ou->doubles(5, v.b_a, 3);
      if (f == 6) ou->doubles(6, v.b_g, 3);
      return 2;
    }
    if (f != 8) return 0;
    Out store;
    size_t k = 0;
    const bool ok2 = rewrite(payload, &store, [&](uint32_t f2, int, Bytes lb, Out* so) -> int {
      if (f2 != 1) return 0;
      if (k >= v.landmarks.size()) return -1;
      std::string body;
      if (!rewrite_landmark(lb, v.landmarks[k++], &body)) return -1;
      so->message(1, body);
      return 2;
    });
    if (!ok2 || k != v.landmarks.size()) return -1;
    ou->message(8, store.s);
    return 2;
  });
  if (!ok) return false;
  *o = out.s;
  return true;
}

bool rewrite_edge(const Edge& e, std::string* o) {
  if (e.kind != kLoopClosure) {
    o->assign((const char*)e.raw.p, e.raw.size());
    return true;
  }
  Out out;
  const bool ok = rewrite(e.raw, &out, [&](uint32_t f, int, Bytes payload, Out* ou) -> int {
    if (f != 3) return 0;
    Out lc;
    bool done = false;
    if (!rewrite(payload, &lc, [&](uint32_t f2, int, Bytes, Out* lo) -> int {
          if (f2 != 6) return 0;
          if (done) return 1;
          lo->double1(6, e.switch_variable);
          done = true;
          return 2;
        }))
      return -1;
    if (!done) lc.double1(6, e.switch_variable);
    ou->message(3, lc.s);
    return 2;
  });
  if (!ok) return false;
  *o = out.s;
  return true;
}

bool rewrite_file(const mba_vimap* M, int file, std::string* o) {
  std::vector<int> vs, es;
  for (size_t i = 0; i < M->vertices.size(); ++i)
    if (M->vertices[i].file == file) vs.push_back((int)i);
  for (size_t i = 0; i < M->edges.size(); ++i)
    if (M->edges[i].file == file) es.push_back((int)i);
  const std::string& s = M->files[file];
  Bytes all{(const uint8_t*)s.data(), (const uint8_t*)s.data() + s.size()};
  Out out;
  size_t kv = 0, ke = 0;
  const bool ok = rewrite(all, &out, [&](uint32_t f, int, Bytes, Out* ou) -> int {
    std::string body;
    if (f == 2) {
      if (kv >= vs.size() || !rewrite_vertex(M->vertices[vs[kv++]], &body)) return -1;
      ou->message(2, body);
      return 2;
    }
    if (f == 4) {
      if (ke >= es.size() || !rewrite_edge(M->edges[es[ke++]], &body)) return -1;
      ou->message(4, body);
      return 2;
    }
    return 0;
  });
  if (!ok || kv != vs.size() || ke != es.size()) return false;
  *o = out.s;
  return true;
}

bool write_file(const std::string& path, const std::string& data) {
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) return false;
  f.write(data.data(), (std::streamsize)data.size());
  return (bool)f;
}

bool is_dir(const std::string& p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

void put_id(const Id& id, uint64_t* out) {
  out[0] = id.w[0];
  out[1] = id.w[1];
}

}  // namespace

extern "C" {

mba_status mba_vimap_load(const char* map_folder, mba_vimap** out) {
  if (!map_folder || !out) return MBA_ERR_INVALID_ARG;
  *out = nullptr;
  try {
    std::unique_ptr<mba_vimap> M(new mba_vimap());
    const mba_status s = load(map_folder, M.get());
    if (s != MBA_OK) return s;
    *out = M.release();
    return MBA_OK;
  } catch (...) {  // allocation failure or a lookup the validation missed: a status, never an abort
    return MBA_ERR_INVALID_ARG;
  }
}

void mba_vimap_destroy(mba_vimap* m) { delete m; }

mba_status mba_vimap_get_info(const mba_vimap* m, mba_vimap_info* info) {
  if (!m || !info) return MBA_ERR_INVALID_ARG;
  std::memset(info, 0, sizeof(*info));
  info->num_missions = (int64_t)m->missions.size();
  info->num_vertices = (int64_t)m->vertices.size();
  for (const Vertex& v : m->vertices) {
    info->num_landmarks += (int64_t)v.landmarks.size();
    info->num_absolute_measurements += (int64_t)v.abs.size();
    for (const Frame& f : v.frames)
      if (f.set) info->num_keypoints += (int64_t)f.sigma.size();
  }
  for (const Edge& e : m->edges) {
    if (e.kind == kViwls) ++info->num_viwls_edges;
    else if (e.kind == kOdometry) ++info->num_odometry_edges;
    else if (e.kind == kWheelOdometry) ++info->num_wheel_odometry_edges;
    else if (e.kind == kLoopClosure) ++info->num_loop_closure_edges;
    else ++info->num_other_edges;
  }
  info->num_sensors = (int64_t)m->sensors.size();
  for (const Sensor& s : m->sensors) info->num_cameras += (int64_t)s.cameras.size();
  return MBA_OK;
}

mba_status mba_vimap_mission_ids(const mba_vimap* m, uint64_t* ids) {
  if (!m || !ids) return MBA_ERR_INVALID_ARG;
  for (size_t i = 0; i < m->missions.size(); ++i) put_id(m->missions[i].id, ids + 2 * i);
  return MBA_OK;
}

void mba_vimap_default_export_options(mba_vimap_export_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->add_visual_constraints = 1;
  o->add_inertial_constraints = 1;
  o->apply_gauge_fixes = 1;
  o->landmark_selection = MBA_VIMAP_LANDMARKS_QUALITY;
  mba_default_landmark_quality_options(&o->quality);
  const double phi = 47.22 * M_PI / 180.0;
  const double s2 = std::sin(phi) * std::sin(phi), s22 = std::sin(2 * phi) * std::sin(2 * phi);
  o->gravity_magnitude = 9.780327 * (1 + 0.0053024 * s2 - 0.0000058 * s22) - 3.155 * 1e-7 * 392.0;
  o->use_huber = 1;
}

mba_status mba_vimap_export(mba_vimap* m, const mba_vimap_export_options* o, mba_problem_desc* desc) {
  if (!m || !o || !desc) return MBA_ERR_INVALID_ARG;
  mba_status s;
  try {
    s = do_export(m, *o, desc);
  } catch (...) {
    s = MBA_ERR_INVALID_ARG;
  }
  if (s != MBA_OK) m->ex = mba_vimap::Export();
  return s;
}

mba_status mba_vimap_export_ids(const mba_vimap* m, uint64_t* kf_vertex_ids, uint64_t* landmark_ids,
                                uint64_t* mission_ids, uint64_t* pose_edge_ids) {
  if (!m || !m->ex.valid) return MBA_ERR_INVALID_ARG;
  const auto& X = m->ex;
  if (kf_vertex_ids)
    for (size_t k = 0; k < X.kf_vertex.size(); ++k) put_id(m->vertices[X.kf_vertex[k]].id, kf_vertex_ids + 2 * k);
  if (landmark_ids)
    for (size_t l = 0; l < X.lm.size(); ++l)
      put_id(m->vertices[X.lm[l].first].landmarks[X.lm[l].second].id, landmark_ids + 2 * l);
  if (mission_ids)
    for (size_t p = 0; p < X.mission.size(); ++p) put_id(m->missions[X.mission[p]].id, mission_ids + 2 * p);
  if (pose_edge_ids)
    for (size_t j = 0; j < X.pe_kind.size(); ++j)
      put_id(X.pe_kind[j] == 0 ? m->edges[X.pe_edge[j]].id : m->vertices[X.pe_edge[j]].id, pose_edge_ids + 2 * j);
  return MBA_OK;
}

mba_status mba_vimap_landmark_ids(const mba_vimap* m, uint64_t* ids) {
  if (!m || !ids) return MBA_ERR_INVALID_ARG;
  size_t i = 0;
  for (const Vertex& v : m->vertices)
    for (const Landmark& l : v.landmarks) put_id(l.id, ids + 2 * i++);
  return MBA_OK;
}

mba_status mba_vimap_import_state(mba_vimap* m, const double* kx, const double* kv, const double* kbg,
                                  const double* kba, const double* lp, const double* sw) {
  if (!m || !m->ex.valid) return MBA_ERR_INVALID_ARG;
  const auto& X = m->ex;
  // Validate first so that a refused call leaves the map unchanged.
  for (size_t k = 0; kx && k < X.kf_vertex.size(); ++k) {
    for (int a = 0; a < 7; ++a)
      if (!std::isfinite(kx[7 * k + a])) return MBA_ERR_NON_FINITE;
    if (!unit_quaternion(kx + 7 * k)) return MBA_ERR_INVALID_ARG;  // assertValidQuaternion
  }
  for (size_t j = 0; sw && j < X.pe_type.size(); ++j)
    if (X.pe_type[j] == MBA_POSE_EDGE_LOOP_CLOSURE && !(sw[j] >= 0.0 && sw[j] <= 1.0)) return MBA_ERR_INVALID_ARG;
  for (size_t k = 0; k < X.kf_vertex.size(); ++k) {
    Vertex& v = m->vertices[X.kf_vertex[k]];
    for (int a = 0; kx && a < 7; ++a) v.T_M_I[a] = kx[7 * k + a];  // copyAllKeyframePosesBackToMap
    for (int a = 0; a < 3; ++a) {
      if (kv) v.v_M[a] = kv[3 * k + a];
      if (kbg) v.b_g[a] = kbg[3 * k + a];
      if (kba) v.b_a[a] = kba[3 * k + a];
    }
  }
  for (size_t l = 0; lp && l < X.lm.size(); ++l) {
    Landmark& L = m->vertices[X.lm[l].first].landmarks[X.lm[l].second];
    for (int a = 0; a < 3; ++a) L.p_B[a] = lp[3 * l + a];
  }
  for (size_t j = 0; sw && j < X.pe_type.size(); ++j)
    if (X.pe_type[j] == MBA_POSE_EDGE_LOOP_CLOSURE) m->edges[X.pe_edge[j]].switch_variable = sw[j];
  return MBA_OK;
}

mba_status mba_vimap_save(const mba_vimap* m, const char* map_folder) {
  if (!m || !map_folder) return MBA_ERR_INVALID_ARG;
  const std::string root(map_folder);
  const std::string dir = join(root, "vi_map");
  if (is_dir(dir)) return MBA_ERR_INVALID_ARG;  // no overwrite
  if (!is_dir(root) && mkdir(root.c_str(), 0755) != 0) return MBA_ERR_INVALID_ARG;
  if (mkdir(dir.c_str(), 0755) != 0) return MBA_ERR_INVALID_ARG;
  if (!write_file(join(dir, "vi_map_metadata"), m->metadata_text)) return MBA_ERR_INVALID_ARG;
  if (!write_file(join(dir, "sensors.yaml"), m->sensors_text)) return MBA_ERR_INVALID_ARG;
  try {
    for (size_t f = 0; f < m->files.size(); ++f) {
      std::string data;
      if (!rewrite_file(m, (int)f, &data)) return MBA_ERR_INVALID_ARG;
      if (!write_file(join(dir, m->file_names[f]), data)) return MBA_ERR_INVALID_ARG;
    }
  } catch (...) {
    return MBA_ERR_INVALID_ARG;
  }
  return MBA_OK;
}

}  // extern "C"
