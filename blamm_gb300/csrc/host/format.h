// format.h -- the occurrence line fields as the reference prints them.
#pragma once
#include <cstddef>
#include <cstdint>

namespace blamm {

// `value` as printf("%g") / the default std::ostream prints it (6 significant
// digits, round half to even on the exact binary value, trailing zeros
// removed).  Writes at most 15 characters plus a terminating zero; returns the
// length.
int formatScore(float value, char *out);

// decimal digits of v (>= 0); returns the length (no terminating zero)
int formatUnsigned(uint64_t v, char *out);

}  // namespace blamm
