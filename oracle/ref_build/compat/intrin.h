/* Stand-in for MSVC <intrin.h>: maps the x64 intrinsics the reference's
 * bigfixed.h uses onto GCC builtins. Oracle build support only (x86-64). */
#ifndef MBX_COMPAT_INTRIN_H
#define MBX_COMPAT_INTRIN_H
#include <immintrin.h>
#include <x86intrin.h>
static inline unsigned long long _umul128(unsigned long long a, unsigned long long b, unsigned long long* hi) {
    unsigned __int128 p = (unsigned __int128)a * b;
    *hi = (unsigned long long)(p >> 64);
    return (unsigned long long)p;
}
#endif
