// Canonical (three-axis) plan of one convolution problem, built on the host
// by plan_problem() in abi.cu.
#pragma once
#include "common.cuh"
#include "direct.h"

namespace ndconv {

struct Plan3 {
    int rank;
    int dtype;
    int reverse;
    AxisGeom ax[3];
    double cval[3][2][2];  // per axis, side (front, back), (re, im)

    template <typename T> Geom3<T> geom() const {
        Geom3<T> g;
        for (int a = 0; a < 3; a++) {
            g.ax[a] = ax[a];
            g.cf[a] = Elem<T>::from(cval[a][0][0], cval[a][0][1]);
            g.cb[a] = Elem<T>::from(cval[a][1][0], cval[a][1][1]);
        }
        return g;
    }
    template <typename T> DirectParams<T> direct() const {
        DirectParams<T> d{};
        d.g = geom<T>();
        d.reverse = reverse;
        for (int a = 0; a < 3; a++) {
            d.t_lo[a] = 0;
            d.t_n[a] = ax[a].K;
        }
        d.ys_[2] = 1;
        d.ys_[1] = ax[2].out;
        d.ys_[0] = ax[1].out * ax[2].out;
        return d;
    }
};

int plan_problem(const ndconv_problem *p, int algo, Plan3 *out);

// Element types other than f32 / f64 / i32 / c32 / c64 (the 64-bit and
// narrow integers, u32): they run the single direct entry point only.
inline bool single_call_int(int dtype) { return dtype >= NDCONV_I64; }
inline bool integer_dtype(int dtype) { return dtype == NDCONV_I32 || dtype >= NDCONV_I64; }

// Whether the 3xBF16 tensor-core path takes the problem (bf16x3.cu).
bool bf16x3_applies(const Plan3 &P);

// ConvExt::conv for u8 / i8 / u16 / i16 (narrow_int.cu).
int conv_narrow_int(const Plan3 &P, const void *data, const void *kernel, void *out, cudaStream_t st);

}  // namespace ndconv
