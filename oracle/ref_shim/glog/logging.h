// Minimal stand-in for glog's LOG(level) stream: discards everything.
// Test infrastructure only.
#pragma once
#include <ostream>
namespace ltpo_shim {
struct NullStream {
    template <typename T> NullStream &operator<<(const T &) { return *this; }
    NullStream &operator<<(std::ostream &(*)(std::ostream &)) { return *this; }
};
}
#define LOG(level) ::ltpo_shim::NullStream()
