// Velocity sets as compile-time tables. The q ordering is lettuce's
// (lettuce/ext/_stencil/d1q3.py:6-10, d2q9.py:8-10, d3q15.py:6-12,
// d3q19.py:8-13, d3q27.py:8-12) because it defines the population index of
// the [Q, *resolution] field the plugin surface exchanges.
//
// Kernels work on an internal 3-D view (X, Y, Z) with Z contiguous: a
// lettuce grid of dimension D maps its dimensions onto the last D of (X, Y,
// Z); the velocities are remapped the same way (ix/iy/iz below).
#pragma once

#include <cstdint>

#include "lettuce_gb300.h"

namespace lgb {

template <int ID> struct Stencil;

#define LGB_HD __host__ __device__ __forceinline__

template <> struct Stencil<LGB_D1Q3> {
    static constexpr int D = 1, Q = 3;
    static LGB_HD constexpr int e(int q, int d) {
        constexpr int t[3] = {0, 1, -1};
        return d == 0 ? t[q] : 0;
    }
    static LGB_HD constexpr double w(int q) {
        constexpr double t[3] = {2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0};
        return t[q];
    }
    static LGB_HD constexpr int opp(int q) {
        constexpr int t[3] = {0, 2, 1};
        return t[q];
    }
};

template <> struct Stencil<LGB_D2Q9> {
    static constexpr int D = 2, Q = 9;
    static LGB_HD constexpr int e(int q, int d) {
        constexpr int t[9][2] = {{0, 0}, {1, 0}, {0, 1}, {-1, 0}, {0, -1},
                                 {1, 1}, {-1, 1}, {-1, -1}, {1, -1}};
        return t[q][d];
    }
    static LGB_HD constexpr double w(int q) {
        return q == 0 ? 4.0 / 9.0 : (q < 5 ? 1.0 / 9.0 : 1.0 / 36.0);
    }
    static LGB_HD constexpr int opp(int q) {
        constexpr int t[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
        return t[q];
    }
};

template <> struct Stencil<LGB_D3Q15> {
    static constexpr int D = 3, Q = 15;
    static LGB_HD constexpr int e(int q, int d) {
        constexpr int t[15][3] = {{0, 0, 0},   {1, 0, 0},   {-1, 0, 0},  {0, 1, 0},
                                  {0, -1, 0},  {0, 0, 1},   {0, 0, -1},  {1, 1, 1},
                                  {-1, -1, -1}, {1, 1, -1}, {-1, -1, 1}, {1, -1, 1},
                                  {-1, 1, -1}, {1, -1, -1}, {-1, 1, 1}};
        return t[q][d];
    }
    static LGB_HD constexpr double w(int q) {
        return q == 0 ? 2.0 / 9.0 : (q < 7 ? 1.0 / 9.0 : 1.0 / 72.0);
    }
    static LGB_HD constexpr int opp(int q) { return q == 0 ? 0 : (q % 2 ? q + 1 : q - 1); }
};

template <> struct Stencil<LGB_D3Q19> {
    static constexpr int D = 3, Q = 19;
    static LGB_HD constexpr int e(int q, int d) {
        constexpr int t[19][3] = {{0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                                  {0, 0, 1},  {0, 0, -1}, {0, 1, 1},  {0, -1, -1}, {0, 1, -1},
                                  {0, -1, 1}, {1, 0, 1},  {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1},
                                  {1, 1, 0},  {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}};
        return t[q][d];
    }
    static LGB_HD constexpr double w(int q) {
        return q == 0 ? 1.0 / 3.0 : (q < 7 ? 1.0 / 18.0 : 1.0 / 36.0);
    }
    static LGB_HD constexpr int opp(int q) { return q == 0 ? 0 : (q % 2 ? q + 1 : q - 1); }
};

template <> struct Stencil<LGB_D3Q27> {
    static constexpr int D = 3, Q = 27;
    static LGB_HD constexpr int e(int q, int d) {
        constexpr int t[27][3] = {
            {0, 0, 0},   {1, 0, 0},   {-1, 0, 0},  {0, 1, 0},   {0, -1, 0},  {0, 0, 1},
            {0, 0, -1},  {0, 1, 1},   {0, -1, -1}, {0, 1, -1},  {0, -1, 1},  {1, 0, 1},
            {-1, 0, -1}, {1, 0, -1},  {-1, 0, 1},  {1, 1, 0},   {-1, -1, 0}, {1, -1, 0},
            {-1, 1, 0},  {1, 1, 1},   {-1, -1, -1}, {1, 1, -1}, {-1, -1, 1}, {1, -1, 1},
            {-1, 1, -1}, {1, -1, -1}, {-1, 1, 1}};
        return t[q][d];
    }
    static LGB_HD constexpr double w(int q) {
        return q == 0 ? 8.0 / 27.0 : (q < 7 ? 2.0 / 27.0 : (q < 19 ? 1.0 / 54.0 : 1.0 / 216.0));
    }
    static LGB_HD constexpr int opp(int q) { return q == 0 ? 0 : (q % 2 ? q + 1 : q - 1); }
};

// velocity components in the internal (X, Y, Z) view
template <class S> LGB_HD constexpr int ix(int q) { return S::D == 3 ? S::e(q, 0) : 0; }
template <class S> LGB_HD constexpr int iy(int q) { return S::D >= 2 ? S::e(q, S::D - 2) : 0; }
template <class S> LGB_HD constexpr int iz(int q) { return S::e(q, S::D - 1); }
// velocity component along internal axis a (0 = X, 1 = Y, 2 = Z)
template <class S> LGB_HD constexpr int iaxis(int q, int a) {
    return a == 0 ? ix<S>(q) : (a == 1 ? iy<S>(q) : iz<S>(q));
}

}  // namespace lgb
