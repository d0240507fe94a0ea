// Forced into ray.cc alone when the reference is built with
// DIFFUSE_REFLECTIONS.  ray.cc:156 and :255 call max(int, int) unqualified
// inside namespace raptor_raytracer; at the reference's HEAD that finds the
// SIMD max(vfp_t, vfp_t) of common/simd.h (global namespace) and does not
// compile.  With std::max declared in the namespace first, the call means
// what it says; max on vfp_t arguments still resolves by argument-dependent
// lookup.
#pragma once
#include <algorithm>
namespace raptor_raytracer {
using std::max;
}
