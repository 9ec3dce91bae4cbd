// Host-side conversions between the reference's amplitude arrays and the
// engine's. The reference (and its Fortran caller) holds t1(o, v) and
// t2(o, o, v, v) column-major (mod_cc.f90:2727 allocates t1(Nocc, Nocc+1:N)
// and t2(Nocc, Nocc, Nocc+1:N, Nocc+1:N)); the engine keeps t1 row-major [i][a]
// and t2 in pair order [i][a][j][b]. For each (a, j) the t2 conversion is an
// o x v transpose between i (contiguous in the column-major array) and b
// (contiguous in the pair layout): reads and writes both run along cache
// lines, and the o + v lines one (a, j) touches stay in L1.
#pragma once
#include <cstddef>

namespace hx {

inline void t1_to_engine(const double *f, double *e, int o, int v)
{
    for (int i = 0; i < o; ++i)
        for (int a = 0; a < v; ++a) e[(size_t)i * v + a] = f[i + (size_t)o * a];
}

inline void t1_from_engine(const double *e, double *f, int o, int v)
{
    for (int a = 0; a < v; ++a)
        for (int i = 0; i < o; ++i) f[i + (size_t)o * a] = e[(size_t)i * v + a];
}

// column-major (i, j, a, b) <-> pair order [i][a][j][b]
template <bool TO_ENGINE>
inline void t2_convert(const double *src, double *dst, int o, int v)
{
    const size_t oo = (size_t)o * o, oov = oo * v, ov = (size_t)o * v, vov = ov * v;
    for (int a = 0; a < v; ++a)
        for (int j = 0; j < o; ++j) {
            const size_t f0 = (size_t)j * o + (size_t)a * oo;    // column-major (0, j, a, 0)
            const size_t p0 = (size_t)a * ov + (size_t)j * v;    // pair order [0][a][j][0]
            for (int b = 0; b < v; ++b)
                for (int i = 0; i < o; ++i) {
                    if (TO_ENGINE) dst[p0 + i * vov + b] = src[f0 + i + b * oov];
                    else dst[f0 + i + b * oov] = src[p0 + i * vov + b];
                }
        }
}

inline void t2_to_engine(const double *f, double *e, int o, int v) { t2_convert<true>(f, e, o, v); }
inline void t2_from_engine(const double *e, double *f, int o, int v) { t2_convert<false>(e, f, o, v); }

}  // namespace hx
