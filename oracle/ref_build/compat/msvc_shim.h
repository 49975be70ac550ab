/* Force-included when compiling the reference engine with GCC: neutralises
 * MSVC-only spellings (dllexport/stdcall, fopen_s, _putenv_s). */
#ifndef MBX_COMPAT_MSVC_SHIM_H
#define MBX_COMPAT_MSVC_SHIM_H
#include <stdio.h>
#include <stdlib.h>
#ifdef __cplusplus
#include <memory>
#endif
#define __declspec(x)
#define __stdcall
static inline int fopen_s(FILE** f, const char* name, const char* mode) {
    *f = fopen(name, mode);
    return *f ? 0 : 1;
}
static inline int _putenv_s(const char* k, const char* v) { return setenv(k, v, 1); }
#endif
