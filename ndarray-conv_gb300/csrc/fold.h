// Axis folding for direct convolution (see fold.cu).
#pragma once
#include "common.cuh"
#include "direct.h"

namespace ndconv {

struct FoldParams {
    AxisGeom ax[3];         // canonical axes (live-tap restricted, not permuted)
    int m, f0, f1;          // main axis and the two folded axes (f0 < f1)
    int reverse;
    int64_t tlo_m, km;      // live taps of the main axis
    int64_t cin, cout;      // n_f0 n_f1 input channels, out_f0 out_f1 output channels
    int64_t ys_m, ys_f0, ys_f1;
};

// True (and F filled) when folding the two axes other than some main axis
// costs clearly less than the direct loops (all border constants zero).
template <typename T> bool plan_fold(const DirectParams<T> &P, FoldParams &F);
template <typename T> size_t fold_scratch_bytes(const FoldParams &F);
// full: the unrestricted parameters of the problem (the non-finite fallback).
// scratch may be null (stream-ordered allocation).
template <typename T>
cudaError_t fold_launch(const T *x, const T *k, T *y, const FoldParams &F, const DirectParams<T> &full,
                        cudaStream_t st, void *scratch, size_t scratch_bytes);

}  // namespace ndconv
