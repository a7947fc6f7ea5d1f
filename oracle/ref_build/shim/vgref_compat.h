/* Force-included compatibility header for building the reference's MSVC-era
 * C++ with GCC on LP64 Linux (x86-64 or aarch64).  TEST INFRASTRUCTURE ONLY:
 * used to build the CPU oracle / CPU baseline, never the product.
 *
 * - x87 control-word helpers become no-ops: on SSE/NEON, C's float->int
 *   conversion already truncates, which is what the reference requests by
 *   switching the x87 control word to "truncate" (Core/Math/math.h:347-590).
 * - StoreFloatAsInt(a) == (int)a, i.e. x87 fistp under a truncating control
 *   word.
 */
#pragma once
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <cstdio>
#include <cstdarg>
#include <cerrno>
#include <climits>
#include <limits>
#include <cfloat>
#include <cmath>
#include <algorithm>
#include <vector>
typedef unsigned short WORD;
#ifndef __declspec
#define __declspec(x)
#endif
inline WORD GetFloatingPointControlWord() { return 0; }
inline WORD SetFloatingPointControlWord(WORD w) { return w; }
inline WORD Changex87FloatingPointToTruncate() { return 0; }
inline unsigned GetMmxControlStatusRegister() { return 0; }
inline unsigned SetMmxControlStatusRegister(unsigned v) { return v; }
inline bool FpcwTruncates() { return true; }
inline int StoreFloatAsInt(float a) { return (int)a; }
template <class T> class NestedGrid;
template <class A, class B> inline A Max2(const A& a, const B& b) { return a > A(b) ? a : A(b); }
template <class A, class B> inline A Min2(const A& a, const B& b) { return a < A(b) ? a : A(b); }
