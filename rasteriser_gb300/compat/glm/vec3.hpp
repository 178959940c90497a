// Part of the glm 0.9.7 API subset; every declaration lives in detail/subset_core.hpp.
#ifndef RAST_GLM_SUBSET_VEC3_HPP
#define RAST_GLM_SUBSET_VEC3_HPP
#include "detail/subset_core.hpp"

#endif
