// Direct convolution launcher (ConvExt::conv on the GPU).
#pragma once
#include "common.cuh"

namespace ndconv {

template <typename T> struct DirectParams {
    Geom3<T> g;
    int reverse;
    // tiling, filled by the launcher
    int64_t cky, ckx;        // kernel rows / columns per staged chunk
    int64_t max_rows, max_cols;
    int64_t tile_elems, w_elems;
    int64_t maps_off;        // byte offset of the int64 border maps in shared memory
    int sw_ty, sw_nseg, sw_q;  // sliding-window tiling (rows, segments, swizzle pitch)
    int sw_ph, sw_res, sw_tr;  // x phases d/g, tap residues s/g (g = gcd(s, d)), tap slots per residue
    int sw_ry, sw_h;           // output rows per warp line; staged-row step (in d1) between them
    int tile_bx, tile_by;      // tiled kernel block shape
    // batch: device arrays of per-instance pointers (null for one instance)
    const T *const *xs;
    const T *const *ks;
    T *const *ys;
    int64_t inst_base;
    // one instance whose pointers travel in the parameters (persistent batch
    // kernel); null when the kernel arguments carry them
    const T *x1;
    const T *k1;
    T *y1;
    // live taps per axis: the kernels loop over [t_lo, t_lo + t_n)
    int64_t t_lo[3], t_n[3];
    // output element strides per (possibly permuted) axis
    int64_t ys_[3];
};

// x, k: device pointers (strided per g.ax[i].xs / ks); y: contiguous output.
// force_naive selects the unstaged kernel (tests use it as a second path).
// scratch (optional, direct_scratch_bytes(P) bytes) serves the axis-folding
// form; without it that form allocates stream-ordered.
template <typename T>
cudaError_t direct_conv_launch(const T *x, const T *k, T *y, DirectParams<T> P, cudaStream_t st,
                               int force_naive, void *scratch = nullptr, size_t scratch_bytes = 0);
// device scratch the launch would use (0 when no folding applies)
template <typename T> size_t direct_scratch_bytes(DirectParams<T> P);

// n instances sharing the geometry; xs / ks / ys: device arrays of n device pointers.
template <typename T>
cudaError_t direct_conv_batch_launch(int64_t n, const T *const *xs, const T *const *ks, T *const *ys,
                                     DirectParams<T> P, cudaStream_t st);

}  // namespace ndconv
