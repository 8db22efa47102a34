// Constant tables for the Q1 hex8 Laplacian element matrix.
#pragma once

#include "common.cuh"

namespace sfem_gb300 {

// A[c][e] = sum_m f_m * w[c*8+e][m] for the symmetric metric f = (00,01,02,11,12,22).
struct LapTable {
    double w[64][6];
    constexpr LapTable() : w() {
        for (int c = 0; c < 8; c++)
            for (int e = 0; e < 8; e++)
                for (int m = 0; m < 6; m++) w[c * 8 + e][m] = lap_weight(c, e, m);
    }
};

struct LapTableF {
    float w[64][6];
    constexpr LapTableF() : w() {
        for (int c = 0; c < 8; c++)
            for (int e = 0; e < 8; e++)
                for (int m = 0; m < 6; m++) w[c * 8 + e][m] = (float)lap_weight(c, e, m);
    }
};

// one copy per translation unit (whole-program compilation, no -rdc)
static __constant__ LapTable kLap = LapTable();
static __constant__ LapTableF kLapF = LapTableF();

template <typename T>
__device__ __forceinline__ T lap_w(int k, int m);
template <>
__device__ __forceinline__ double lap_w<double>(int k, int m) {
    return kLap.w[k][m];
}
template <>
__device__ __forceinline__ float lap_w<float>(int k, int m) {
    return kLapF.w[k][m];
}

}  // namespace sfem_gb300
