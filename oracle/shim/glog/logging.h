// Minimal stand-in for the glog API surface that the reference's early-break
// header touches (LOG, VLOG, CHECK, CHECK_GT ...).  Test infrastructure only:
// it lets oracle/build_ref.sh compile the reference's own CPU path so that its
// outputs can pin the oracle.  Messages go to stderr; FATAL and failed CHECKs
// abort, matching glog's behaviour.
#pragma once
#include <cstdlib>
#include <iostream>
#include <sstream>

namespace shim_glog {
struct Line {
  std::ostringstream os;
  bool fatal;
  explicit Line(bool f) : fatal(f) {}
  ~Line() {
    std::cerr << os.str() << std::endl;
    if (fatal) std::abort();
  }
  template <typename T>
  Line& operator<<(const T& v) {
    os << v;
    return *this;
  }
};
struct Null {
  template <typename T>
  Null& operator<<(const T&) { return *this; }
};
}  // namespace shim_glog

#define SHIM_SEV_INFO false
#define SHIM_SEV_WARNING false
#define SHIM_SEV_ERROR false
#define SHIM_SEV_FATAL true
#define LOG(sev) shim_glog::Line(SHIM_SEV_##sev)
#define VLOG(n) shim_glog::Null()
#define CHECK(c) \
  if (!(c)) shim_glog::Line(true) << "Check failed: " #c " "
#define CHECK_OP_(a, b, op) \
  if (!((a)op(b))) shim_glog::Line(true) << "Check failed: " #a " " #op " " #b " "
#define CHECK_GT(a, b) CHECK_OP_(a, b, >)
#define CHECK_GE(a, b) CHECK_OP_(a, b, >=)
#define CHECK_LT(a, b) CHECK_OP_(a, b, <)
#define CHECK_LE(a, b) CHECK_OP_(a, b, <=)
#define CHECK_EQ(a, b) CHECK_OP_(a, b, ==)
#define CHECK_NE(a, b) CHECK_OP_(a, b, !=)
