// Minimal stand-in for the parts of glog the reference's host sources use:
// LOG(level) streams are discarded, initialisation and destinations are
// no-ops.  Test infrastructure only (lets the reference's host program be
// compiled and linked against this library for the drop-in check).
#pragma once
#include <ostream>
#include <string>
namespace ltpo_shim {
struct NullStream {
    template <typename T> NullStream &operator<<(const T &) { return *this; }
    NullStream &operator<<(std::ostream &(*)(std::ostream &)) { return *this; }
};
}
#define LOG(level) ::ltpo_shim::NullStream()
namespace google {
enum LogSeverity { GLOG_INFO = 0, GLOG_WARNING = 1, GLOG_ERROR = 2, GLOG_FATAL = 3 };
inline void InitGoogleLogging(const char *) {}
inline void ShutdownGoogleLogging() {}
inline void SetLogDestination(LogSeverity, const char *) {}
}  // namespace google
inline bool FLAGS_alsologtostderr = false;
inline bool FLAGS_colorlogtostderr = false;
inline std::string FLAGS_log_dir;
