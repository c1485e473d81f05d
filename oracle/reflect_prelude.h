// reflect_prelude.h -- TEST INFRASTRUCTURE ONLY.
//
// Declarations that let the reference's Reflect.h be compiled on its own by
// oracle/build_ref.sh, which streams Reflect.h without its includes of Omega3D.h,
// Points.h and Surfaces.h (those pull in Eigen, Vc and the element classes).  Only the
// free function templates panel_point_distance, dot_product, cross_product and
// normalizeVec are instantiated; the element classes are never defined.  The values
// below are the ones Omega3D.h:26-48 defines.
#pragma once
#include <array>
#include <cassert>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <limits>
#include <tuple>
#include <variant>
#include <vector>

using Int = uint32_t;
const size_t Dimensions = 3;
enum move_t { lagrangian = 1, bodybound = 2, fixed = 3 };
template <class S> using Vector = std::vector<S>;
template <class S> class Points;
template <class S> class Surfaces;
using Collection = std::variant<std::monostate>;
