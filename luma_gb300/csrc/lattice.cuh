// Lattice velocity sets, weights and direction maps for D2Q9, D3Q19 and
// D3Q27, in the reference's direction order (LUMA src/stdafx.cpp:29-153,
// src/GridUtils.cpp:31-69).  Every accessor is constexpr so that, inside a
// fully unrolled direction loop, each lookup folds to an immediate.
#pragma once

#include <cstdint>

namespace luma {

template <int Q>
struct Lattice;

template <>
struct Lattice<9> {
    static constexpr int D = 2;
    __host__ __device__ static constexpr int c(int v, int d) {
        constexpr int t[9][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {1, 1, 0},
                                 {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {0, 0, 0}};
        return t[v][d];
    }
    __host__ __device__ static constexpr double w(int v) {
        return v < 4 ? 1.0 / 9.0 : (v < 8 ? 1.0 / 36.0 : 4.0 / 9.0);
    }
    __host__ __device__ static constexpr int opp(int v) {
        constexpr int t[9] = {1, 0, 3, 2, 5, 4, 7, 6, 8};
        return t[v];
    }
    __host__ __device__ static constexpr int reflect(int plane, int v) {
        constexpr int t[3][9] = {{1, 0, 2, 3, 7, 6, 5, 4, 8}, {0, 1, 3, 2, 6, 7, 4, 5, 8},
                                 {0, 1, 2, 3, 4, 5, 6, 7, 8}};
        return t[plane][v];
    }
};

template <>
struct Lattice<19> {
    static constexpr int D = 3;
    __host__ __device__ static constexpr int c(int v, int d) {
        constexpr int t[19][3] = {{1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {0, 0, 1},
                                  {0, 0, -1}, {1, 1, 0},  {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0},
                                  {0, 1, 1},  {0, -1, -1}, {0, 1, -1}, {0, -1, 1}, {1, 0, 1},
                                  {-1, 0, -1}, {-1, 0, 1}, {1, 0, -1}, {0, 0, 0}};
        return t[v][d];
    }
    __host__ __device__ static constexpr double w(int v) {
        return v < 6 ? 1.0 / 18.0 : (v < 18 ? 1.0 / 36.0 : 1.0 / 3.0);
    }
    __host__ __device__ static constexpr int opp(int v) {
        constexpr int t[19] = {1, 0, 3, 2, 5, 4, 7, 6, 9, 8, 11, 10, 13, 12, 15, 14, 17, 16, 18};
        return t[v];
    }
    __host__ __device__ static constexpr int reflect(int plane, int v) {
        constexpr int t[3][19] = {
            {1, 0, 2, 3, 4, 5, 9, 8, 7, 6, 10, 11, 12, 13, 16, 17, 14, 15, 18},
            {0, 1, 3, 2, 4, 5, 8, 9, 6, 7, 13, 12, 11, 10, 14, 15, 16, 17, 18},
            {0, 1, 2, 3, 5, 4, 6, 7, 8, 9, 12, 13, 10, 11, 17, 16, 15, 14, 18}};
        return t[plane][v];
    }
};

template <>
struct Lattice<27> {
    static constexpr int D = 3;
    __host__ __device__ static constexpr int c(int v, int d) {
        constexpr int t[27][3] = {
            {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},   {0, -1, 0}, {0, 0, 1},   {0, 0, -1}, {0, 1, 1},
            {0, -1, -1}, {0, 1, -1}, {0, -1, 1},  {1, 0, 1},  {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1},
            {1, 1, 0},   {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {1, 1, 1},   {-1, -1, -1},
            {-1, -1, 1}, {1, 1, -1}, {-1, 1, 1},  {1, -1, -1}, {1, -1, 1},  {-1, 1, -1}, {0, 0, 0}};
        return t[v][d];
    }
    __host__ __device__ static constexpr double w(int v) {
        return v < 6 ? 2.0 / 27.0 : (v < 18 ? 1.0 / 54.0 : (v < 26 ? 1.0 / 216.0 : 8.0 / 27.0));
    }
    __host__ __device__ static constexpr int opp(int v) {
        constexpr int t[27] = {1,  0,  3,  2,  5,  4,  7,  6,  9,  8,  11, 10, 13, 12,
                               15, 14, 17, 16, 19, 18, 21, 20, 23, 22, 25, 24, 26};
        return t[v];
    }
    __host__ __device__ static constexpr int reflect(int plane, int v) {
        constexpr int t[3][27] = {
            {1, 0, 2, 3, 4, 5, 6, 7, 8, 9, 13, 12, 11, 10, 17, 16, 15, 14, 22, 23, 24, 25, 18, 19, 20, 21, 26},
            {0, 1, 3, 2, 4, 5, 9, 8, 7, 6, 10, 11, 12, 13, 16, 17, 14, 15, 24, 25, 22, 23, 20, 21, 18, 19, 26},
            {0, 1, 2, 3, 5, 4, 8, 9, 6, 7, 12, 13, 10, 11, 14, 15, 16, 17, 21, 20, 19, 18, 25, 24, 23, 22, 26}};
        return t[plane][v];
    }
};

}  // namespace luma
