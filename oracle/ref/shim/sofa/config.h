// Minimal stand-in for the generated sofa/config.h, written for the oracle's
// reference harness only: it defines the few macros the reference math
// headers (Type/Vec, Type/Mat, Helper/decompose) use. It is not generated from
// the reference's config.h.in.
#pragma once
#include <cstddef>
#include <cstdint>
#include <limits>
typedef double SReal;
#define SOFA_EXPORT_DYNAMIC_LIBRARY __attribute__((visibility("default")))
#define SOFA_IMPORT_DYNAMIC_LIBRARY
#define SOFA_ATTRIBUTE_DEPRECATED(a, b, c)
#define SOFA_ATTRIBUTE_DISABLED(a, b, c)
#define sofa_do_tostring(a) #a
#define sofa_tostring(a) sofa_do_tostring(a)
constexpr SReal operator""_sreal(long double r) { return static_cast<SReal>(r); }
constexpr SReal operator""_sreal(unsigned long long int i) { return static_cast<SReal>(i); }
#define SOFA_UNUSED(x) (void)(x)
namespace sofa {
using SignedIndex = int32_t;
using Index = uint32_t;
using Size = uint32_t;
constexpr Index InvalidID = (std::numeric_limits<Index>::max)();
}
