// Per-cell update rules of the cells compiled into the library.  Each rule
// restates a Cell's update()/updateLineX() operation for operation; the
// FP64 rules use __dadd_rn/__dmul_rn so nothing is fused and the results
// are bit-identical to the reference's SerialSimulator build
// (-ffp-contract=off).  FP32 rules may fuse (their error is stated against
// the FP64 oracle instead).
#ifndef LGD_K_CELLS_CUH
#define LGD_K_CELLS_CUH

#include "k_common.cuh"

namespace lgd {

// Jacobi-7: temp' = (c + n + s + e + w + t + b) * (1/7), n = y-1, s = y+1,
// e = x+1, w = x-1, t = z+1, b = z-1, summed left to right (reference
// template: src/examples/jacobi3dupdateline/main.cpp:31-42, with the seventh
// centre term and 1/7).
struct Jacobi7F64 {
    typedef double T;
    static __device__ __forceinline__ T apply(T c, T n, T s, T e, T w, T t, T b)
    {
        T acc = __dadd_rn(c, n);
        acc = __dadd_rn(acc, s);
        acc = __dadd_rn(acc, e);
        acc = __dadd_rn(acc, w);
        acc = __dadd_rn(acc, t);
        acc = __dadd_rn(acc, b);
        return __dmul_rn(acc, 1.0 / 7.0);
    }
};

struct Jacobi7F32 {
    typedef float T;
    static __device__ __forceinline__ T apply(T c, T n, T s, T e, T w, T t, T b)
    {
        return (c + n + s + e + w + t + b) * (1.0f / 7.0f);
    }
};

// Jacobi-7 on the 64-bit fixed-point image of an FP64 grid (see
// fx_mul7_round): the neighbour sum is exact, the only rounding is the final
// multiplication by fl(1/7), at most half a unit of 2^(scale_exp - 56).
// NONNEG: every value and the edge cell are >= 0 (the sum is, too), which
// saves the sign handling; both forms give the same result there.
template<bool NONNEG>
struct Jacobi7FixT {
    typedef long long T;
    static __device__ __forceinline__ T apply(T c, T n, T s, T e, T w, T t, T b)
    {
        const T sum = c + n + s + e + w + t + b;
        return NONNEG ? fx_mul7_round_nonneg(sum) : fx_mul7_round(sum);
    }
};
typedef Jacobi7FixT<false> Jacobi7Fix;
typedef Jacobi7FixT<true> Jacobi7FixNonNeg;

// Two Jacobi-7 steps in one pass with one rounding (the temporally blocked
// fixed-point pass): the first level keeps the exact neighbour sum (7 times
// the average), the second sums those and multiplies by fl(1/7)^2.  The
// result is the rounded exact two-step product, within one unit of two
// rounded single steps.
template<bool NONNEG>
struct Jacobi7FixTwoStepT {
    typedef long long T;
    static __device__ __forceinline__ T inner(T c, T n, T s, T e, T w, T t, T b) { return c + n + s + e + w + t + b; }
    static __device__ __forceinline__ T last(T c, T n, T s, T e, T w, T t, T b)
    {
        const T sum = c + n + s + e + w + t + b;
        return NONNEG ? fx_mul49_round_nonneg(sum) : fx_mul49_round(sum);
    }
};
typedef Jacobi7FixTwoStepT<false> Jacobi7FixTwoStep;
typedef Jacobi7FixTwoStepT<true> Jacobi7FixTwoStepNonNeg;

// Variable-coefficient diffusion: u' = u + sum over faces (-x, +x, -y, +y,
// -z, +z) of 0.5 (k + k_nb)(u_nb - u).
template<typename R>
struct VarCoef;

template<>
struct VarCoef<double> {
    typedef double T;
    static __device__ __forceinline__ T face(T uc, T kc, T un, T kn)
    {
        return __dmul_rn(__dmul_rn(0.5, __dadd_rn(kc, kn)), __dadd_rn(un, -uc));
    }
    static __device__ __forceinline__ T apply(T uc, T kc, T uw, T kw, T ue, T ke, T un, T kn,
                                              T us, T ks, T ub, T kb, T ut, T kt)
    {
        T flux = face(uc, kc, uw, kw);
        flux = __dadd_rn(flux, face(uc, kc, ue, ke));
        flux = __dadd_rn(flux, face(uc, kc, un, kn));
        flux = __dadd_rn(flux, face(uc, kc, us, ks));
        flux = __dadd_rn(flux, face(uc, kc, ub, kb));
        flux = __dadd_rn(flux, face(uc, kc, ut, kt));
        return __dadd_rn(uc, flux);
    }
};

template<>
struct VarCoef<float> {
    typedef float T;
    static __device__ __forceinline__ T face(T uc, T kc, T un, T kn)
    {
        return 0.5f * (kc + kn) * (un - uc);
    }
    static __device__ __forceinline__ T apply(T uc, T kc, T uw, T kw, T ue, T ke, T un, T kn,
                                              T us, T ks, T ub, T kb, T ut, T kt)
    {
        T flux = face(uc, kc, uw, kw);
        flux += face(uc, kc, ue, ke);
        flux += face(uc, kc, un, kn);
        flux += face(uc, kc, us, ks);
        flux += face(uc, kc, ub, kb);
        flux += face(uc, kc, ut, kt);
        return uc + flux;
    }
};

// Two x-neighbouring FP32 cells (.x at x, .y at x + 1) in packed FP32
// arithmetic (one instruction updates both, sm_100 and later):
// u' = u + 0.5 * sum over faces (k + k_f)(u_f - u), each face's product
// fused into the sum, faces in VarCoef's order.  One rounding fewer per
// face than VarCoef<float>; both stay within the FP32 bound against the
// FP64 cell.
__device__ __forceinline__ float2 varcoef_pair_f32(float2 uc, float2 kc, float2 uw, float2 kw, float2 ue, float2 ke,
                                                   float2 un, float2 kn, float2 us, float2 ks, float2 ub, float2 kb,
                                                   float2 ut, float2 kt)
{
    const float2 m1 = make_float2(-1.0f, -1.0f);
    float2 acc = __fmul2_rn(__fadd2_rn(kc, kw), __ffma2_rn(uc, m1, uw));
    acc = __ffma2_rn(__fadd2_rn(kc, ke), __ffma2_rn(uc, m1, ue), acc);
    acc = __ffma2_rn(__fadd2_rn(kc, kn), __ffma2_rn(uc, m1, un), acc);
    acc = __ffma2_rn(__fadd2_rn(kc, ks), __ffma2_rn(uc, m1, us), acc);
    acc = __ffma2_rn(__fadd2_rn(kc, kb), __ffma2_rn(uc, m1, ub), acc);
    acc = __ffma2_rn(__fadd2_rn(kc, kt), __ffma2_rn(uc, m1, ut), acc);
    return __ffma2_rn(make_float2(0.5f, 0.5f), acc, uc);
}

// Conway's rule (src/examples/gameoflife/main.cpp:35-58).
__device__ __forceinline__ uint8_t gol_rule(uint8_t self, int living)
{
    return self ? (uint8_t)((living == 2) || (living == 3)) : (uint8_t)(living == 3);
}

}  // namespace lgd

#endif
