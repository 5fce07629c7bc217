// Minimal stand-in for nlohmann::json, covering only what the reference's
// early-break path and the headers it pulls in use (operator[], contains,
// at, get<T>, dump, array, push_back, update, clear).  Test infrastructure
// for oracle/build_ref.sh; not a general JSON library.
#pragma once
#include <cstdint>
#include <initializer_list>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace nlohmann {
class json {
 public:
  enum class kind { null_, boolean, number, string, array, object };

  json() = default;
  json(std::nullptr_t) {}
  json(bool b) : k_(kind::boolean), b_(b) {}
  template <typename T, typename std::enable_if<std::is_arithmetic<T>::value &&
                                                    !std::is_same<T, bool>::value,
                                                int>::type = 0>
  json(T v) : k_(kind::number), n_(static_cast<double>(v)) {}
  json(const char* s) : k_(kind::string), s_(s) {}
  json(const std::string& s) : k_(kind::string), s_(s) {}
  json(std::initializer_list<json> init) {
    bool is_object = init.size() > 0;
    for (const auto& e : init) {
      if (!(e.k_ == kind::array && e.a_.size() == 2 &&
            e.a_[0].k_ == kind::string)) {
        is_object = false;
        break;
      }
    }
    if (is_object) {
      k_ = kind::object;
      for (const auto& e : init) o_.emplace_back(e.a_[0].s_, e.a_[1]);
    } else {
      k_ = kind::array;
      a_.assign(init.begin(), init.end());
    }
  }

  static json array() {
    json j;
    j.k_ = kind::array;
    return j;
  }

  json& operator[](const std::string& key) {
    if (k_ == kind::null_) k_ = kind::object;
    if (k_ != kind::object) throw std::runtime_error("json: not an object");
    for (auto& kv : o_)
      if (kv.first == key) return kv.second;
    o_.emplace_back(key, json());
    return o_.back().second;
  }
  json& operator[](const char* key) { return (*this)[std::string(key)]; }

  bool contains(const std::string& key) const {
    if (k_ != kind::object) return false;
    for (const auto& kv : o_)
      if (kv.first == key) return true;
    return false;
  }
  const json& at(const std::string& key) const {
    for (const auto& kv : o_)
      if (kv.first == key) return kv.second;
    throw std::out_of_range("json: no key " + key);
  }
  json& at(const std::string& key) {
    for (auto& kv : o_)
      if (kv.first == key) return kv.second;
    throw std::out_of_range("json: no key " + key);
  }

  template <typename T>
  T get() const {
    return static_cast<T>(k_ == kind::boolean ? (b_ ? 1.0 : 0.0) : n_);
  }

  void push_back(const json& j) {
    if (k_ == kind::null_) k_ = kind::array;
    a_.push_back(j);
  }
  json& back() { return a_.back(); }
  void update(const json& other) {
    for (const auto& kv : other.o_) (*this)[kv.first] = kv.second;
  }
  void clear() {
    a_.clear();
    o_.clear();
  }

  std::string dump(int = -1) const {
    std::ostringstream os;
    write(os);
    return os.str();
  }

 private:
  void write(std::ostringstream& os) const {
    switch (k_) {
    case kind::null_: os << "null"; break;
    case kind::boolean: os << (b_ ? "true" : "false"); break;
    case kind::number: os.precision(17); os << n_; break;
    case kind::string: os << '"' << s_ << '"'; break;
    case kind::array:
      os << '[';
      for (size_t i = 0; i < a_.size(); ++i) {
        if (i) os << ',';
        a_[i].write(os);
      }
      os << ']';
      break;
    case kind::object:
      os << '{';
      for (size_t i = 0; i < o_.size(); ++i) {
        if (i) os << ',';
        os << '"' << o_[i].first << "\":";
        o_[i].second.write(os);
      }
      os << '}';
      break;
    }
  }

  kind k_ = kind::null_;
  bool b_ = false;
  double n_ = 0;
  std::string s_;
  std::vector<json> a_;
  std::vector<std::pair<std::string, json>> o_;
};
}  // namespace nlohmann
