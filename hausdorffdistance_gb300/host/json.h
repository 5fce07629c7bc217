// Minimal JSON value (objects keep insertion order) for run statistics and the
// hd_exec output file, whose keys follow the reference's RunningStats schema
// (src/running_stats.h:64-104, src/run_hausdorff_distance.cu:78-398).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <initializer_list>
#include <memory>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

namespace hd {

class Json {
 public:
  enum class Kind { kNull, kBool, kNumber, kString, kArray, kObject };

  Json() = default;
  Json(bool b) : kind_(Kind::kBool), b_(b) {}
  Json(int v) : kind_(Kind::kNumber), n_((double) v) {}
  Json(unsigned v) : kind_(Kind::kNumber), n_((double) v) {}
  Json(long v) : kind_(Kind::kNumber), n_((double) v) {}
  Json(unsigned long v) : kind_(Kind::kNumber), n_((double) v) {}
  Json(long long v) : kind_(Kind::kNumber), n_((double) v) {}
  Json(unsigned long long v) : kind_(Kind::kNumber), n_((double) v) {}
  Json(float v) : kind_(Kind::kNumber), n_((double) v) {}
  Json(double v) : kind_(Kind::kNumber), n_(v) {}
  Json(const char* s) : kind_(Kind::kString), s_(s) {}
  Json(const std::string& s) : kind_(Kind::kString), s_(s) {}

  static Json Array() {
    Json j;
    j.kind_ = Kind::kArray;
    return j;
  }
  static Json Object() {
    Json j;
    j.kind_ = Kind::kObject;
    return j;
  }

  Json& operator[](const std::string& key) {
    if (kind_ == Kind::kNull) kind_ = Kind::kObject;
    for (auto& kv : obj_)
      if (kv.first == key) return kv.second;
    obj_.emplace_back(key, Json());
    return obj_.back().second;
  }
  bool contains(const std::string& key) const {
    for (auto& kv : obj_)
      if (kv.first == key) return true;
    return false;
  }
  const Json& at(const std::string& key) const {
    for (auto& kv : obj_)
      if (kv.first == key) return kv.second;
    static const Json null_value;
    return null_value;
  }
  void push_back(const Json& v) {
    if (kind_ == Kind::kNull) kind_ = Kind::kArray;
    arr_.push_back(v);
  }
  Json& back() { return arr_.back(); }
  // Element i of an array (which must hold more than i elements).
  Json& element(size_t i) { return arr_.at(i); }
  void update(const Json& other) {
    for (auto& kv : other.obj_) (*this)[kv.first] = kv.second;
  }
  double number() const { return n_; }
  Kind kind() const { return kind_; }

  std::string dump(int indent = 2) const {
    std::ostringstream os;
    write(os, indent, 0);
    return os.str();
  }

 private:
  static void escape(std::ostringstream& os, const std::string& s) {
    os << '"';
    for (char ch : s) {
      switch (ch) {
      case '"': os << "\\\""; break;
      case '\\': os << "\\\\"; break;
      case '\n': os << "\\n"; break;
      case '\t': os << "\\t"; break;
      default:
        if ((unsigned char) ch < 0x20) {
          char buf[8];
          std::snprintf(buf, sizeof(buf), "\\u%04x", ch);
          os << buf;
        } else {
          os << ch;
        }
      }
    }
    os << '"';
  }
  void write(std::ostringstream& os, int indent, int depth) const {
    const std::string pad(indent > 0 ? (size_t) (indent * (depth + 1)) : 0, ' ');
    const std::string pad0(indent > 0 ? (size_t) (indent * depth) : 0, ' ');
    const char* nl = indent > 0 ? "\n" : "";
    switch (kind_) {
    case Kind::kNull: os << "null"; break;
    case Kind::kBool: os << (b_ ? "true" : "false"); break;
    case Kind::kNumber:
      if (std::isfinite(n_)) {
        char buf[40];
        std::snprintf(buf, sizeof(buf), "%.17g", n_);
        os << buf;
      } else {
        os << "null";
      }
      break;
    case Kind::kString: escape(os, s_); break;
    case Kind::kArray:
      os << '[' << nl;
      for (size_t i = 0; i < arr_.size(); ++i) {
        os << pad;
        arr_[i].write(os, indent, depth + 1);
        os << (i + 1 < arr_.size() ? "," : "") << nl;
      }
      os << pad0 << ']';
      break;
    case Kind::kObject:
      os << '{' << nl;
      for (size_t i = 0; i < obj_.size(); ++i) {
        os << pad;
        escape(os, obj_[i].first);
        os << (indent > 0 ? ": " : ":");
        obj_[i].second.write(os, indent, depth + 1);
        os << (i + 1 < obj_.size() ? "," : "") << nl;
      }
      os << pad0 << '}';
      break;
    }
  }

  Kind kind_ = Kind::kNull;
  bool b_ = false;
  double n_ = 0.0;
  std::string s_;
  std::vector<Json> arr_;
  std::vector<std::pair<std::string, Json>> obj_;
};

}  // namespace hd
