// Part of the glm 0.9.7 API subset; every declaration lives in detail/subset_core.hpp.
#ifndef RAST_GLM_SUBSET_GTX_EXTENTED_MIN_MAX_HPP
#define RAST_GLM_SUBSET_GTX_EXTENTED_MIN_MAX_HPP
#include "../detail/subset_core.hpp"

namespace glm {
// Three-argument min and max, reduced left to right: min(min(a, b), c).
template <typename V> inline V min(const V& a, const V& b, const V& c) { return min(min(a, b), c); }
template <typename V> inline V max(const V& a, const V& b, const V& c) { return max(max(a, b), c); }
}  // namespace glm

#endif
