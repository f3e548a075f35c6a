// Minimal stand-in for the gflags macros and calls the reference's host
// sources use: flags are plain globals with their defaults and the command
// line is not parsed.  Test infrastructure only.
#pragma once
#include <cstdint>
#include <string>
#define DECLARE_string(n) extern std::string FLAGS_##n
#define DECLARE_uint32(n) extern uint32_t FLAGS_##n
#define DECLARE_double(n) extern double FLAGS_##n
#define DEFINE_string(n, v, d) std::string FLAGS_##n = v
#define DEFINE_uint32(n, v, d) uint32_t FLAGS_##n = v
#define DEFINE_double(n, v, d) double FLAGS_##n = v
namespace gflags {
inline uint32_t ParseCommandLineFlags(int *, char ***, bool) { return 0; }
inline void ShutDownCommandLineFlags() {}
}  // namespace gflags
