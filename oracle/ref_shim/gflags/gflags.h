// Minimal stand-in for the gflags macros and calls the reference's host
// sources use: flags are plain globals with their defaults, registered by
// name so that ParseCommandLineFlags can set them from --name=value
// arguments (other arguments are left alone).  Test infrastructure only.
#pragma once
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
namespace ltpo_flags {
struct Flag {
    const char *name;
    void (*set)(const char *);
};
inline std::vector<Flag> &registry() {
    static std::vector<Flag> r;
    return r;
}
struct Add {
    Add(const char *n, void (*f)(const char *)) { registry().push_back({n, f}); }
};
}  // namespace ltpo_flags
#define DECLARE_string(n) extern std::string FLAGS_##n
#define DECLARE_uint32(n) extern uint32_t FLAGS_##n
#define DECLARE_double(n) extern double FLAGS_##n
#define DEFINE_string(n, v, d) \
    std::string FLAGS_##n = v; \
    static ::ltpo_flags::Add ltpo_flag_##n(#n, [](const char *s) { FLAGS_##n = s; })
#define DEFINE_uint32(n, v, d) \
    uint32_t FLAGS_##n = v;    \
    static ::ltpo_flags::Add ltpo_flag_##n(#n, [](const char *s) { FLAGS_##n = (uint32_t)std::strtoul(s, nullptr, 10); })
#define DEFINE_double(n, v, d) \
    double FLAGS_##n = v;      \
    static ::ltpo_flags::Add ltpo_flag_##n(#n, [](const char *s) { FLAGS_##n = std::strtod(s, nullptr); })
namespace gflags {
inline uint32_t ParseCommandLineFlags(int *argc, char ***argv, bool) {
    for (int i = 1; i < *argc; i++) {
        const char *a = (*argv)[i];
        if (std::strncmp(a, "--", 2) != 0) continue;
        const char *eq = std::strchr(a + 2, '=');
        if (!eq) continue;
        const std::string name(a + 2, eq - (a + 2));
        for (const auto &f : ::ltpo_flags::registry())
            if (name == f.name) f.set(eq + 1);
    }
    return 0;
}
inline void ShutDownCommandLineFlags() {}
}  // namespace gflags
