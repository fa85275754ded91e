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
    // per folded axis f (0: f0, 1: f1), the taps grouped by the input sample
    // they read: for output index o and sample i, taps tap[f][o K_f + e] for
    // e in [off[f][o (n_f + 1) + i], off[f][o (n_f + 1) + i + 1]), ascending
    const int32_t *off[2];
    const int32_t *tap[2];
};

// int32 entries of the tap tables of folded axis A (offsets, then taps)
__host__ __device__ inline int64_t fold_table_entries(const AxisGeom &A) { return A.out * (A.n + 1) + A.out * A.K; }

// The tap table row of output index o on axis A: off[0..n] and tap[0..K)
// (taps reading a padding zero are left out).
__host__ __device__ inline void fold_table_row(const AxisGeom &A, int64_t o, int32_t *off, int32_t *tap) {
    for (int64_t i = 0; i <= A.n; i++) off[i] = 0;
    for (int64_t t = 0; t < A.K; t++) {
        const int64_t i = axis_map(A, o * A.s + t * A.d);
        if (i >= 0) off[i + 1]++;
    }
    for (int64_t i = 0; i < A.n; i++) off[i + 1] += off[i];
    // scatter with off[i] as the cursor of bucket i, then shift back
    for (int64_t t = 0; t < A.K; t++) {
        const int64_t i = axis_map(A, o * A.s + t * A.d);
        if (i >= 0) tap[off[i]++] = (int32_t)t;
    }
    for (int64_t i = A.n; i > 0; i--) off[i] = off[i - 1];
    off[0] = 0;
}

// True (and F filled) when folding the two axes other than some main axis
// costs clearly less than the direct loops (all border constants zero).
template <typename T> bool plan_fold(const DirectParams<T> &P, FoldParams &F);
template <typename T> size_t fold_scratch_bytes(const FoldParams &F);
// point F's tap tables into `tables` (fold_table_entries of f0, then of f1)
void fold_set_tables(FoldParams &F, void *tables);
// full: the unrestricted parameters of the problem (the non-finite fallback).
// scratch may be null (stream-ordered allocation).
template <typename T>
cudaError_t fold_launch(const T *x, const T *k, T *y, const FoldParams &F, const DirectParams<T> &full,
                        cudaStream_t st, void *scratch, size_t scratch_bytes);

}  // namespace ndconv
