// Project-written stand-in for glm/gtx/string_cast.hpp (test infrastructure
// for the oracle's reference build): glm::to_string for the types the
// reference's debug printers format.
#pragma once
#include <cstdio>
#include <string>
#include "../glm.hpp"

namespace glm {
inline std::string to_string(const vec3& v) {
    char buf[128];
    std::snprintf(buf, sizeof(buf), "vec3(%f, %f, %f)", v.x, v.y, v.z);
    return std::string(buf);
}
inline std::string to_string(const vec4& v) {
    char buf[160];
    std::snprintf(buf, sizeof(buf), "vec4(%f, %f, %f, %f)", v.x, v.y, v.z, v.w);
    return std::string(buf);
}
}  // namespace glm
