/* Linux stand-ins for the Windows CRT calls of the reference's rsq reader
 * (FBPG/rsq_load.cpp: _fseeki64, _ftelli64, fopen_s), force-included when
 * oracle/ref_build.py compiles that file where it lies into oracle/_ref/.
 * Test infrastructure only (the rsq golden fixtures). */
#pragma once
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#define _fseeki64 fseeko
#define _ftelli64 ftello
static inline int fopen_s(FILE **f, const char *name, const char *mode)
{
    *f = fopen(name, mode);
    return *f ? 0 : 1;
}
