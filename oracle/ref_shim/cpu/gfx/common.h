// Stand-in for the reference's gfx/common.h (which pulls in Vulkan, VMA and fmt): only the integer
// and float aliases, the includes that its CPU volume-map code takes from it, and fmt::println for
// its warning messages (printed without their arguments). Test infrastructure, with glm_shim.hpp
// in place of glm.
#pragma once

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstdint>
#include <functional>
#include <limits>
#include <string>
#include <tuple>
#include <vector>

#include "glm/glm_shim.hpp"

using u8 = uint8_t;
using u16 = uint16_t;
using u32 = uint32_t;
using u64 = uint64_t;
using i32 = int32_t;
using i64 = int64_t;
using f32 = float;
using f64 = double;

namespace fmt {
template <class... Args>
void println(const char* format, Args&&...) {
    std::fprintf(stderr, "%s\n", format);
}
}  // namespace fmt
