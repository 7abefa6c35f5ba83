// Forward declarations standing in for glm's vector types; the reference's host
// headers only name them in type traits.
#pragma once
namespace glm {
struct vec2;
struct vec3;
struct vec4;
} // namespace glm
