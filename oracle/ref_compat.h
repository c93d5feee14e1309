/*
 * ref_compat.h - force-included (g++ -include) when oracle/Makefile compiles the reference's
 * CPU sources on Linux/g++.  TEST INFRASTRUCTURE ONLY.
 *
 * The reference was written for MSVC.  Two things stop it compiling with g++ 13:
 *   - it calls the C99 float functions through std:: (std::powf, std::sinf, ...), which
 *     libstdc++ does not declare in namespace std;
 *   - a few files use std::memset without including <cstring>.
 * This header supplies those names and nothing else; it changes no behaviour.
 */
#pragma once
#include <cmath>
#include <cstring>
#include <cstdlib>
#include <math.h>

namespace std {
using ::acosf;
using ::atanf;
using ::cosf;
using ::expf;
using ::logf;
using ::powf;
using ::sinf;
using ::sqrtf;
using ::tanf;
}  // namespace std
