// Minimal stand-in for the parts of glog the reference's host sources use:
// each LOG(level) statement becomes one line on stderr when the environment
// variable LTPMG_SHIM_LOG is set and is discarded otherwise; initialisation
// and destinations are no-ops.  Test infrastructure only (lets the
// reference's host program be compiled, linked against this library and
// run for the drop-in check).
#pragma once
#include <cstdio>
#include <cstdlib>
#include <ostream>
#include <sstream>
#include <string>
namespace ltpo_shim {
struct LogLine {
    bool on = std::getenv("LTPMG_SHIM_LOG") != nullptr;
    std::ostringstream os;
    ~LogLine() {
        if (on) std::fprintf(stderr, "%s\n", os.str().c_str());
    }
    template <typename T> LogLine &operator<<(const T &v) {
        if (on) os << v;
        return *this;
    }
    LogLine &operator<<(std::ostream &(*f)(std::ostream &)) {
        if (on) f(os);
        return *this;
    }
};
}  // namespace ltpo_shim
#define LOG(level) ::ltpo_shim::LogLine()
namespace google {
enum LogSeverity { GLOG_INFO = 0, GLOG_WARNING = 1, GLOG_ERROR = 2, GLOG_FATAL = 3 };
inline void InitGoogleLogging(const char *) {}
inline void ShutdownGoogleLogging() {}
inline void SetLogDestination(LogSeverity, const char *) {}
}  // namespace google
inline bool FLAGS_alsologtostderr = false;
inline bool FLAGS_colorlogtostderr = false;
inline std::string FLAGS_log_dir;
