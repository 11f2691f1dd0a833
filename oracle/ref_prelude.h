// ref_prelude.h -- TEST INFRASTRUCTURE ONLY.
//
// Force-included before the staged copy of the reference headers (see
// build_oracle.py).  It supplies what those headers assume from their original
// toolchain (icpc on x86):
//   * names they use unqualified inside namespace PADO (pair, ofstream,
//     make_pair) -- global using-declarations are visible there;
//   * on non-x86 hosts (the Arm GPU machine), the x86 prefetch hint and the two
//     AVX-512 type names that appear in signatures of helper members the
//     non-vectorised classes never call.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <utility>
#include <vector>

using std::make_pair;
using std::ofstream;
using std::pair;

#if defined(__x86_64__) || defined(__i386__)
#include <immintrin.h>
#include <xmmintrin.h>
#else
#ifndef _MM_HINT_T0
#define _MM_HINT_T0 0
#endif
#define _mm_prefetch(p, hint) __builtin_prefetch((const void *)(p))
typedef struct { int lanes[16]; } __m512i;
typedef uint16_t __mmask16;
#endif
