// Shared definitions for the ndconv CUDA library (sm_103a).
//
// Geometry is canonicalised to 3 axes: a rank-r problem occupies the last r
// axes, the leading ones have extent 1, no padding, stride 1, dilation 1.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ndconv.h"

// ------------------------------------------------------------------ types --
struct c32 {
    float re, im;
};
struct c64 {
    double re, im;
};

template <typename T> struct Elem;
template <> struct Elem<float> {
    using Acc = float;
    using Real = float;
    static constexpr bool kComplex = false;
    static constexpr bool kInteger = false;
    __host__ __device__ static float zero() { return 0.0f; }
    __host__ __device__ static float from(double re, double) { return (float)re; }
    __device__ static bool is_zero(float v) { return v == 0.0f; }
    __device__ static void mac(float &a, float x, float w) { a = fmaf(x, w, a); }
    __device__ static void add(float &a, float x) { a += x; }
    __device__ static float out(float a) { return a; }
};
template <> struct Elem<double> {
    using Acc = double;
    using Real = double;
    static constexpr bool kComplex = false;
    static constexpr bool kInteger = false;
    __host__ __device__ static double zero() { return 0.0; }
    __host__ __device__ static double from(double re, double) { return re; }
    __device__ static bool is_zero(double v) { return v == 0.0; }
    __device__ static void mac(double &a, double x, double w) { a = fma(x, w, a); }
    __device__ static void add(double &a, double x) { a += x; }
    __device__ static double out(double a) { return a; }
};
// i32: wrapping two's-complement arithmetic, as the reference's release build
template <> struct Elem<int32_t> {
    using Acc = uint32_t;
    using Real = int32_t;
    static constexpr bool kComplex = false;
    static constexpr bool kInteger = true;
    __host__ __device__ static int32_t zero() { return 0; }
    __host__ __device__ static int32_t from(double re, double) {
        return re >= 2147483648.0 ? (int32_t)(uint32_t)re : (int32_t)re;  // u32 constants above 2^31
    }
    __device__ static bool is_zero(int32_t v) { return v == 0; }
    __device__ static void mac(uint32_t &a, int32_t x, int32_t w) { a += (uint32_t)x * (uint32_t)w; }
    __device__ static void add(uint32_t &a, int32_t x) { a += (uint32_t)x; }
    __device__ static int32_t out(uint32_t a) { return (int32_t)a; }
};
// i64: wrapping two's-complement arithmetic (u64 runs as i64: the same bits)
template <> struct Elem<int64_t> {
    using Acc = uint64_t;
    using Real = int64_t;
    static constexpr bool kComplex = false;
    static constexpr bool kInteger = true;
    __host__ __device__ static int64_t zero() { return 0; }
    __host__ __device__ static int64_t from(double re, double) {
        return re >= 9223372036854775808.0 ? (int64_t)(uint64_t)re : (int64_t)re;
    }
    __device__ static bool is_zero(int64_t v) { return v == 0; }
    __device__ static void mac(uint64_t &a, int64_t x, int64_t w) { a += (uint64_t)x * (uint64_t)w; }
    __device__ static void add(uint64_t &a, int64_t x) { a += (uint64_t)x; }
    __device__ static int64_t out(uint64_t a) { return (int64_t)a; }
};
template <> struct Elem<c32> {
    using Acc = c32;
    using Real = float;
    static constexpr bool kComplex = true;
    static constexpr bool kInteger = false;
    __host__ __device__ static c32 zero() { return c32{0.0f, 0.0f}; }
    __host__ __device__ static c32 from(double re, double im) { return c32{(float)re, (float)im}; }
    __device__ static bool is_zero(c32 v) { return v.re == 0.0f && v.im == 0.0f; }
    __device__ static void mac(c32 &a, c32 x, c32 w) {
        a.re = fmaf(x.re, w.re, a.re);
        a.re = fmaf(-x.im, w.im, a.re);
        a.im = fmaf(x.re, w.im, a.im);
        a.im = fmaf(x.im, w.re, a.im);
    }
    __device__ static void add(c32 &a, c32 x) {
        a.re += x.re;
        a.im += x.im;
    }
    __device__ static c32 out(c32 a) { return a; }
};
template <> struct Elem<c64> {
    using Acc = c64;
    using Real = double;
    static constexpr bool kComplex = true;
    static constexpr bool kInteger = false;
    __host__ __device__ static c64 zero() { return c64{0.0, 0.0}; }
    __host__ __device__ static c64 from(double re, double im) { return c64{re, im}; }
    __device__ static bool is_zero(c64 v) { return v.re == 0.0 && v.im == 0.0; }
    __device__ static void mac(c64 &a, c64 x, c64 w) {
        a.re = fma(x.re, w.re, a.re);
        a.re = fma(-x.im, w.im, a.re);
        a.im = fma(x.re, w.im, a.im);
        a.im = fma(x.im, w.re, a.im);
    }
    __device__ static void add(c64 &a, c64 x) {
        a.re += x.re;
        a.im += x.im;
    }
    __device__ static c64 out(c64 a) { return a; }
};

// ------------------------------------------------------------- geometry --
// Border kinds after canonicalisation (ZEROS becomes CONST with value 0).
enum : int { BK_CONST = 1, BK_REFLECT = 2, BK_REPLICATE = 3, BK_CIRCULAR = 4 };

// Codes returned by axis_map for positions that are not input samples.
enum : int { MAP_PREFILL = -1, MAP_CONST_FRONT = -2, MAP_CONST_BACK = -3 };

struct AxisGeom {
    int64_t n;       // input extent
    int64_t p0, p1;  // pads
    int64_t L;       // padded extent n + p0 + p1 ("pds")
    int32_t kf, kb;  // border kinds, front / back
    int64_t K;       // kernel extent
    int64_t d;       // dilation
    int64_t keff;    // dilated kernel extent K*d - d + 1
    int64_t s;       // stride
    int64_t out;     // output extent (L - keff) / s + 1
    int64_t xs;      // data element stride
    int64_t ks;      // kernel element stride
};

template <typename T> struct Geom3 {
    AxisGeom ax[3];
    T cf[3], cb[3];  // BorderType::Const values, front / back, per axis
};

// Where a position j in [0, L) of the padded axis takes its value from.
//
// The reference pads axis by axis (axis 0 first), and within an axis fills
// the front pad (j ascending) and then the back pad (j ascending), each cell
// copying whole hyperplanes out of the buffer's CURRENT contents
// (src/padding/mod.rs:221-452, src/padding/half_dim.rs:30-343).  Following
// that chain for one axis gives a closed form: an input index in [0, n), or
// a constant of this axis' front/back side, or MAP_PREFILL when the chain
// ends on a cell that had not been filled yet (reflect-front reading the
// still-empty back pad, circular-front with p0 > n).  Because every fill
// copies whole hyperplanes, the N-d value is separable: scanning axes from
// the last to the first, the first constant wins; otherwise any PREFILL
// gives the pre-fill value (zero); otherwise the input sample at the mapped
// indices.  Positions that would make the reference panic are rejected on
// the host before launch.
__host__ __device__ __forceinline__ int64_t axis_map(const AxisGeom &a, int64_t j) {
    const int64_t p0 = a.p0, n = a.n;
    if (j >= p0) {
        const int64_t i = j - p0;
        if (i < n) return i;
        if (j >= a.L) return MAP_PREFILL;  // beyond the padded extent (FFT buffer zeros)
        switch (a.kb) {
        case BK_CONST: return MAP_CONST_BACK;
        case BK_REPLICATE: return n - 1;
        case BK_CIRCULAR: return i % n;
        default: {  // BK_REFLECT: copies buffer index 2(p0+n-1) - j
            const int64_t src = 2 * (p0 + n - 1) - j;
            if (src >= p0) return src - p0;
            j = src;  // lands in the (already filled) front pad
            break;
        }
        }
    }
    if (j < 0) return MAP_PREFILL;
    switch (a.kf) {
    case BK_CONST: return MAP_CONST_FRONT;
    case BK_REPLICATE: return 0;
    case BK_CIRCULAR: {  // copies buffer index n + j
        const int64_t r = n + j - p0;
        return r >= 0 ? r : MAP_PREFILL;
    }
    default: {  // BK_REFLECT: copies buffer index 2 p0 - j
        const int64_t r = p0 - j;
        return r < n ? r : MAP_PREFILL;
    }
    }
}

// Value of the padded array at mapped indices (m0, m1, m2).
template <typename T>
__device__ __forceinline__ T resolve_padded(const T *__restrict__ x, const Geom3<T> &g, int64_t m0,
                                            int64_t m1, int64_t m2) {
    if (m2 <= MAP_CONST_FRONT) return m2 == MAP_CONST_FRONT ? g.cf[2] : g.cb[2];
    if (m1 <= MAP_CONST_FRONT) return m1 == MAP_CONST_FRONT ? g.cf[1] : g.cb[1];
    if (m0 <= MAP_CONST_FRONT) return m0 == MAP_CONST_FRONT ? g.cf[0] : g.cb[0];
    if ((m0 | m1 | m2) < 0) return Elem<T>::zero();
    return x[m0 * g.ax[0].xs + m1 * g.ax[1].xs + m2 * g.ax[2].xs];
}

// Kernel element feeding tap t (0 <= t < K) of an axis: the reference
// iterates the kernel reversed when `reverse` (src/dilation/mod.rs:39-45).
__host__ __device__ __forceinline__ int64_t tap_source(int64_t t, int64_t K, int reverse) {
    return reverse ? (K - 1 - t) : t;
}

#define NDCONV_CUDA_OK(expr)                                                              \
    do {                                                                                  \
        cudaError_t e__ = (expr);                                                         \
        if (e__ != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e__)); \
    } while (0)

// Host helpers implemented in abi.cu
int ndconv_fail(int status, const char *msg);
// The calling thread's tuning knob (ndconv_set_tuning; 0: automatic).
int ndconv_tune(int knob);
void ndconv_count_launch(uint64_t n = 1);
// Opt a kernel into `bytes` of dynamic shared memory on the current device
// (once per device and kernel).
cudaError_t ndconv_allow_smem(const void *kernel, int bytes);
