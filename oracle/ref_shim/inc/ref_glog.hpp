// ref_glog.hpp - stand-in for glog's logging macros (TEST INFRASTRUCTURE: only the reference-pin
// recipe, oracle/ref_build.py, compiles against it).  Messages are discarded.
#pragma once

#include <ostream>

namespace ref_glog {
struct NullStream {
    template <class T>
    NullStream& operator<<(const T&) {
        return *this;
    }
    NullStream& operator<<(std::ostream& (*)(std::ostream&)) { return *this; }
};
}  // namespace ref_glog

#define LOG(severity) ::ref_glog::NullStream()
#define DLOG(severity) ::ref_glog::NullStream()
#define VLOG(level) ::ref_glog::NullStream()
