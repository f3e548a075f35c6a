// Minimal stand-in for the gflags macros the reference's host headers use,
// so that individual reference host sources compile for the oracle harness.
// Test infrastructure only.
#pragma once
#include <cstdint>
#include <string>
#define DECLARE_string(n) extern std::string FLAGS_##n
#define DECLARE_uint32(n) extern uint32_t FLAGS_##n
#define DECLARE_double(n) extern double FLAGS_##n
#define DEFINE_string(n, v, d) std::string FLAGS_##n = v
#define DEFINE_uint32(n, v, d) uint32_t FLAGS_##n = v
#define DEFINE_double(n, v, d) double FLAGS_##n = v
