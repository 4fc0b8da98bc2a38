/*
 * Operation counter for the CPU oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * The Makefile builds a second copy of lw_oracle.cpp (liblworacle_count.so)
 * in which every `double` is this layout-compatible type, so that each
 * floating-point addition, subtraction, multiplication and division the
 * restatement of the reference executes increments g_flops.  Comparisons,
 * conversions and the library functions (exp, log, pow) are not counted.
 * The counts give the algorithmic floating-point work of rrtmg_lw per column
 * on the reference's own code path (the denominator of the FP32 roofline).
 */
#pragma once
#include <cmath>
#include <cstdint>
#include <type_traits>

extern "C" uint64_t g_flops;

struct cd_t {
  double v;
  cd_t() = default;
  constexpr cd_t(double x) : v(x) {}
  operator double() const { return v; }
  cd_t& operator+=(cd_t o) { ++g_flops; v += o.v; return *this; }
  cd_t& operator-=(cd_t o) { ++g_flops; v -= o.v; return *this; }
  cd_t& operator*=(cd_t o) { ++g_flops; v *= o.v; return *this; }
  cd_t& operator/=(cd_t o) { ++g_flops; v /= o.v; return *this; }
  cd_t operator-() const { return cd_t(-v); }
};
static_assert(sizeof(cd_t) == sizeof(double), "counted doubles keep the arrays' layout");

#define CD_BIN(op)                                                                                         \
  inline cd_t operator op(cd_t a, cd_t b) { ++g_flops; return cd_t(a.v op b.v); }                         \
  template <class T, class = std::enable_if_t<std::is_arithmetic<T>::value>>                               \
  inline cd_t operator op(cd_t a, T b) { ++g_flops; return cd_t(a.v op (double)b); }                       \
  template <class T, class = std::enable_if_t<std::is_arithmetic<T>::value>>                               \
  inline cd_t operator op(T a, cd_t b) { ++g_flops; return cd_t((double)a op b.v); }
CD_BIN(+) CD_BIN(-) CD_BIN(*) CD_BIN(/)
#undef CD_BIN
#define CD_CMP(op)                                                                                         \
  inline bool operator op(cd_t a, cd_t b) { return a.v op b.v; }                                          \
  template <class T, class = std::enable_if_t<std::is_arithmetic<T>::value>>                               \
  inline bool operator op(cd_t a, T b) { return a.v op (double)b; }                                        \
  template <class T, class = std::enable_if_t<std::is_arithmetic<T>::value>>                               \
  inline bool operator op(T a, cd_t b) { return (double)a op b.v; }
CD_CMP(<) CD_CMP(>) CD_CMP(<=) CD_CMP(>=) CD_CMP(==) CD_CMP(!=)
#undef CD_CMP

uint64_t g_flops = 0;
// operations per phase of a column: 0 inatm, 1 cldprmc, 2 setcoef, 3 taumol
// and the aerosol add, 4 rtrnmc (ORA_PHASE(k) closes phase k; -1 opens a column)
static uint64_t g_phase[5] = {0, 0, 0, 0, 0}, g_mark = 0;
#define ORA_PHASE(k)                    \
  do {                                  \
    if ((k) >= 0) g_phase[k] += g_flops - g_mark; \
    g_mark = g_flops;                   \
  } while (0)
extern "C" uint64_t ora_flops(int phase) { return phase < 0 ? g_flops : g_phase[phase]; }
extern "C" void ora_flops_reset(void) {
  g_flops = g_mark = 0;
  for (auto& p : g_phase) p = 0;
}
