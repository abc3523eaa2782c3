// Shared device/host code of the ERI engine: record layouts, the Boys function, the
// per-shell-quartet driver (primitive loops -> generated VRR -> contraction -> HRR) and
// the class kernels.  Compiled by nvcc for sm_103a; the record layouts, Boys function and
// quartet driver also compile as plain C++ (GS_HOST_ONLY) for CPU checks of the generated
// recursions.
#pragma once
#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define GS_HD __host__ __device__
#define GS_INLINE __forceinline__
#define GS_UNROLL _Pragma("unroll")
#else
#define GS_HD
#define GS_INLINE inline
#define GS_UNROLL
#endif

#include "boys_table.h"

namespace gs {

// ------------------------------------------------------------------ records
// One primitive pair of a shell pair (a,b), la >= lb:
//   p = alpha+beta, i2p = 1/(2p), P = (alpha A + beta B)/p, PA = P - A,
//   Kp = sqrt(2 pi^(5/2)) * c_a c_b exp(-alpha beta/p |AB|^2) / p
// so that [00|00]^(m) = Kp_bra Kp_ket (p+q)^(-1/2) F_m(T).
template <typename T> struct PrimRec;
template <> struct alignas(16) PrimRec<double> {
    double p, i2p, Px, Py, Pz, PAx, PAy, PAz, Kp, pad;
};
template <> struct alignas(16) PrimRec<float> {
    float p, i2p, Px, Py, Pz, PAx, PAy, PAz, Kp, pad0, pad1, pad2;
};

// One shell pair: AB = A - B, its primitive pairs [prim_off, prim_off + nprim), and the
// two shells (sa has the larger angular momentum).
struct alignas(16) PairRec {
    double ABx, ABy, ABz;
    int prim_off, nprim, sa, sb;
    float qmax;   // Schwarz bound sqrt(max |(ab|ab)|) of the pair (0 until computed)
    int pad;
};

// Microbench / dense-block task: canonical bra and ket pair, 3-bit permutation code
// (bit0: bra shells swapped, bit1: ket shells swapped, bit2: bra<->ket swapped) and the
// offset of the block in the caller's original (a,b,c,d) order.
struct alignas(8) WriteTask {
    int bra, ket;
    int code, pad;
    long long off;
};

template <typename T> struct VrrCoef {
    T PAx, PAy, PAz, WPx, WPy, WPz, QCx, QCy, QCz, WQx, WQy, WQz, i2p, rp2, i2q, rq2, i2pq;
};

template <int LA, int LB, int LC, int LD> struct ClassGen;

// ------------------------------------------------------------------ math helpers
GS_HD GS_INLINE double gs_rsqrt(double x) {
#if defined(__CUDA_ARCH__)
    return rsqrt(x);
#else
    return 1.0 / std::sqrt(x);
#endif
}
GS_HD GS_INLINE float gs_rsqrt(float x) {
#if defined(__CUDA_ARCH__)
    return rsqrtf(x);
#else
    return 1.0f / std::sqrt(x);
#endif
}
GS_HD GS_INLINE double gs_exp(double x) { return exp(x); }
GS_HD GS_INLINE float gs_exp(float x) {
#if defined(__CUDA_ARCH__)
    return expf(x);
#else
    return std::exp(x);
#endif
}

// ------------------------------------------------------------------ Boys function
// F_m(T_k) and e^{-T_k} on the grid T_k = k / BOYS_INV_H (FP64; FP32 quartets evaluate
// the small-T branch in FP64 too)
#if defined(__CUDACC__)
__device__ const double g_boys_d[BOYS_ROWS * BOYS_NCOL] = {GS_BOYS_TABLE_VALUES};
#endif
static const double h_boys_d[BOYS_ROWS * BOYS_NCOL] = {GS_BOYS_TABLE_VALUES};

GS_HD GS_INLINE const double* boys_table() {
#if defined(__CUDA_ARCH__)
    return g_boys_d;
#else
    return h_boys_d;
#endif
}

// Taylor rows of the one Boys order the kernels of a translation unit evaluate most
// (GS_BOYS_ORDER, defined by the generated class and gradient units): row k holds
// F_{M+j}(T_k) / j!, j = 0..6, and the exponential's row exp(-T_k) / j!, so that an
// expansion about T_k is a Horner chain of FMAs in T_k - T.  Other orders use the grid.
#if defined(__CUDACC__) && defined(GS_BOYS_ORDER)
#define GS_BOYS_CAT2(a, b) a##b
#define GS_BOYS_CAT(a, b) GS_BOYS_CAT2(a, b)
__device__ __align__(16) const double g_boys_taylor[BOYS_ROWS * 8] = {
    GS_BOYS_CAT(GS_BOYS_TAYLOR_, GS_BOYS_ORDER)};
__device__ __align__(16) const double g_boys_expt[BOYS_ROWS * 8] = {GS_BOYS_EXPT};
constexpr int kBoysOrder = GS_BOYS_ORDER;
static_assert(kBoysOrder >= 0 && kBoysOrder <= BOYS_TAYLOR_MMAX, "Boys order without rows");
#else
constexpr int kBoysOrder = -1;
#endif

template <typename T> GS_HD GS_INLINE T ldg(const T* p) {
#if defined(__CUDA_ARCH__)
    return __ldg(p);
#else
    return *p;
#endif
}

// Boys function below BOYS_TMAX, always in FP64: 7-term Taylor expansion of F_M about the
// nearest grid point (grid step 1/BOYS_INV_H), then downward recursion
//   F_{m-1}(t) = (2t F_m(t) + e^{-t}) / (2m - 1),
// stable downwards; e^{-t} comes from the tabulated e^{-t_k} times the Taylor series of
// e^{-(t - t_k)}.  F[m] = pref * F_m(t).
template <int M>
GS_HD GS_INLINE void boys_small(double t, double pref, double* __restrict__ F) {
#if defined(__CUDA_ARCH__) && defined(GS_BOYS_ORDER)
    if constexpr (M == kBoysOrder) {
        // the same expansion and recursion from this order's Taylor rows
        const int k = __double2int_rn(t * BOYS_INV_H);
        const double d = fma((double)k, 1.0 / BOYS_INV_H, -t);     // t_k - t, exact
        const double2* g = reinterpret_cast<const double2*>(g_boys_taylor) + 4 * k;
        const double2 g01 = __ldg(g), g23 = __ldg(g + 1), g45 = __ldg(g + 2), g67 = __ldg(g + 3);
        double f = fma(g67.x, d, g45.y);
        f = fma(f, d, g45.x);
        f = fma(f, d, g23.y);
        f = fma(f, d, g23.x);
        f = fma(f, d, g01.y);
        F[M] = fma(f, d, g01.x) * pref;
        if (M > 0) {
            const double2* x = reinterpret_cast<const double2*>(g_boys_expt) + 4 * k;
            const double2 x01 = __ldg(x), x23 = __ldg(x + 1), x45 = __ldg(x + 2), x67 = __ldg(x + 3);
            double e = fma(x67.x, d, x45.y);
            e = fma(e, d, x45.x);
            e = fma(e, d, x23.y);
            e = fma(e, d, x23.x);
            e = fma(e, d, x01.y);
            const double et = fma(e, d, x01.x) * pref;
            const double t2 = t + t;
            GS_UNROLL for (int m = M; m >= 1; --m) F[m - 1] = (t2 * F[m] + et) * (1.0 / (2 * m - 1));
        }
        return;
    }
#endif
    const int k = (int)(t * BOYS_INV_H + 0.5);
    const double d = k * (1.0 / BOYS_INV_H) - t;
    const double* row = boys_table() + k * BOYS_NCOL;
    const double d2 = d * (1.0 / 2), d3 = d * (1.0 / 3), d4 = d * (1.0 / 4);
    const double d5 = d * (1.0 / 5), d6 = d * (1.0 / 6);
    double f = ldg(row + M + 6);
    f = f * d6 + ldg(row + M + 5);
    f = f * d5 + ldg(row + M + 4);
    f = f * d4 + ldg(row + M + 3);
    f = f * d3 + ldg(row + M + 2);
    f = f * d2 + ldg(row + M + 1);
    f = f * d + ldg(row + M);
    F[M] = f * pref;
    if (M > 0) {
        double e = d6 + 1.0;
        e = e * d5 + 1.0;
        e = e * d4 + 1.0;
        e = e * d3 + 1.0;
        e = e * d2 + 1.0;
        e = e * d + 1.0;
        const double et = e * ldg(row + BOYS_NCOL - 1) * pref;
        const double t2 = t + t;
        GS_UNROLL for (int m = M; m >= 1; --m) F[m - 1] = (t2 * F[m] + et) * (1.0 / (2 * m - 1));
    }
}

// Boys function below the asymptotic threshold for an FP32 quartet: the same grid, the
// Taylor expansion cut after the d^4 term (its remainder, at most d^5/5! < 3e-10 of F_M
// for |d| <= 1/32, is far below FP32 rounding) and the downward recursion, all in FP64;
// each F_m is rounded to float once and then scaled by pref in float.  t - t_k is exact in
// float (both are multiples of t's ulp and |t - t_k| <= 1/32).
template <int M>
GS_HD GS_INLINE void boys_small32(float t, float pref, float* __restrict__ F) {
    static_assert(M + 4 <= BOYS_NCOL - 2, "Taylor terms beyond the tabulated orders");
#if defined(__CUDA_ARCH__) && defined(GS_BOYS_ORDER)
    if constexpr (M == kBoysOrder) {
        // this order's Taylor rows, cut after the d^4 term as below
        const int k = __float2int_rn(t * float(BOYS_INV_H));
        const double d = (double)((float)k * (1.0f / BOYS_INV_H) - t);
        const double2* g = reinterpret_cast<const double2*>(g_boys_taylor) + 4 * k;
        const double2 g01 = __ldg(g), g23 = __ldg(g + 1), g45 = __ldg(g + 2);
        double Fd[M + 1];
        double f = fma(g45.x, d, g23.y);
        f = fma(f, d, g23.x);
        f = fma(f, d, g01.y);
        Fd[M] = fma(f, d, g01.x);
        if (M > 0) {
            const double2* x = reinterpret_cast<const double2*>(g_boys_expt) + 4 * k;
            const double2 x01 = __ldg(x), x23 = __ldg(x + 1), x45 = __ldg(x + 2);
            double e = fma(x45.x, d, x23.y);
            e = fma(e, d, x23.x);
            e = fma(e, d, x01.y);
            const double et = fma(e, d, x01.x);
            const double t2 = 2.0 * (double)t;
            GS_UNROLL for (int m = M; m >= 1; --m) Fd[m - 1] = (t2 * Fd[m] + et) * (1.0 / (2 * m - 1));
        }
        GS_UNROLL for (int m = 0; m <= M; ++m) F[m] = (float)Fd[m] * pref;
        return;
    }
#endif
    const int k = (int)(t * float(BOYS_INV_H) + 0.5f);
    const double d = (double)((float)k * (1.0f / BOYS_INV_H) - t);
    const double* row = boys_table() + k * BOYS_NCOL;
    const double d2 = d * (1.0 / 2), d3 = d * (1.0 / 3), d4 = d * (1.0 / 4);
    double Fd[M + 1];
    double f = ldg(row + M + 4);
    f = f * d4 + ldg(row + M + 3);
    f = f * d3 + ldg(row + M + 2);
    f = f * d2 + ldg(row + M + 1);
    Fd[M] = f * d + ldg(row + M);
    if (M > 0) {
        double e = d4 + 1.0;
        e = e * d3 + 1.0;
        e = e * d2 + 1.0;
        e = e * d + 1.0;
        const double et = e * ldg(row + BOYS_NCOL - 1);
        const double t2 = 2.0 * (double)t;
        GS_UNROLL for (int m = M; m >= 1; --m) Fd[m - 1] = (t2 * Fd[m] + et) * (1.0 / (2 * m - 1));
    }
    GS_UNROLL for (int m = 0; m <= M; ++m) F[m] = (float)Fd[m] * pref;
}

// Start of the asymptotic branch for orders 0..M: the smallest T (rounded up) at which
// F_m(T) ~ (2m-1)!! / (2T)^m * sqrt(pi/T) / 2 is within 2^-54 (FP64) or 2^-26 (FP32) of
// F_m for every m <= M.  Its relative error is the regularised upper incomplete gamma
// function Q(m + 1/2, T), which grows with m, so the threshold depends on M only.
constexpr double kBoysAsym64[17] = {36, 40, 43, 46, 49, 52, 54, 57, 59, 61, 64, 66, 68, 70, 72, 74, 76};
constexpr float kBoysAsym32[17] = {17, 20, 23, 25, 28, 30, 32, 34, 36, 38, 40, 42, 43, 45, 47, 48, 50};

// F[m] = pref * F_m(t), m = 0..M.  Below the threshold: the grid expansion and the
// downward recursion in FP64 (boys_small, or boys_small32 for an FP32 quartet, which
// rounds the FP64 values to float once).  Above it: F_0 = sqrt(pi/t)/2 and the upward
// recursion F_{m+1} = (2m+1) F_m / (2t) in the quartet's precision, exact to its rounding
// there.  Neither branch needs an exponential: lanes of one warp that take different
// branches cost the sum of both.
template <int M, typename T>
GS_HD GS_INLINE void boys(T t, T pref, T* __restrict__ F) {
    static_assert(M <= 16, "Boys orders beyond the table");
    constexpr bool dbl = sizeof(T) == 8;
    constexpr T thr = dbl ? T(kBoysAsym64[M]) : T(kBoysAsym32[M]);
    static_assert(thr <= T(BOYS_TMAX), "asymptotic threshold beyond the grid");
    if (t < thr) {
        if constexpr (dbl) boys_small<M>(t, pref, F);
        else boys_small32<M>(t, pref, F);
    } else {
        const T rs = gs_rsqrt(t);
        F[0] = pref * T(0.88622692545275801365) * rs;   // sqrt(pi)/2
        if (M > 0) {
            const T hit = T(0.5) * rs * rs;
            GS_UNROLL for (int m = 0; m < M; ++m) F[m + 1] = (T(2 * m + 1) * hit) * F[m];
        }
    }
}

// ------------------------------------------------------------------ one shell quartet
// Contracted Cartesian block of the canonical quartet (bra | ket), in the component
// order of ClassGen (blk[((ia*NB+ib)*NC+ic)*ND+id]), without per-component scaling.
template <int LA, int LB, int LC, int LD, typename T>
GS_HD GS_INLINE void eri_quartet(const PairRec& B, const PairRec& K,
                                 const PrimRec<T>* __restrict__ prims, T* __restrict__ blk) {
    using G = ClassGen<LA, LB, LC, LD>;
    T acc[G::NACC];
    GS_UNROLL for (int i = 0; i < G::NACC; ++i) acc[i] = T(0);
    for (int i = 0; i < B.nprim; ++i) {
        const PrimRec<T> P = prims[B.prim_off + i];
        for (int j = 0; j < K.nprim; ++j) {
            const PrimRec<T> Q = prims[K.prim_off + j];
            const T pq = P.p + Q.p;
            const T rs = gs_rsqrt(pq);
            const T ipq = rs * rs;
            const T PQx = Q.Px - P.Px, PQy = Q.Py - P.Py, PQz = Q.Pz - P.Pz;
            const T wq = Q.p * ipq, wp = P.p * ipq;
            const T t = P.p * wq * (PQx * PQx + PQy * PQy + PQz * PQz);
            T F[G::L + 1];
            boys<G::L, T>(t, P.Kp * Q.Kp * rs, F);
            VrrCoef<T> c;
            c.PAx = P.PAx; c.PAy = P.PAy; c.PAz = P.PAz;
            c.WPx = wq * PQx; c.WPy = wq * PQy; c.WPz = wq * PQz;
            c.QCx = Q.PAx; c.QCy = Q.PAy; c.QCz = Q.PAz;
            c.WQx = -wp * PQx; c.WQy = -wp * PQy; c.WQz = -wp * PQz;
            c.i2p = P.i2p; c.i2q = Q.i2p;
            c.rp2 = wq * P.i2p; c.rq2 = wp * Q.i2p;
            c.i2pq = T(0.5) * ipq;
            G::vrr(F, c, acc);
        }
    }
    G::hrr(acc, T(B.ABx), T(B.ABy), T(B.ABz), T(K.ABx), T(K.ABy), T(K.ABz), blk);
}

// Contraction accumulators of the quartet over primitive quartets start, start + stride,
// ... (flat index i * K.nprim + j): the lanes of a warp that shares one quartet's primitive
// quartets each call this with their own start and stride 32, then sum the accumulators.
template <int LA, int LB, int LC, int LD, typename T>
GS_HD GS_INLINE void eri_accumulate(const PairRec& B, const PairRec& K,
                                    const PrimRec<T>* __restrict__ prims, T* __restrict__ acc,
                                    int start, int stride) {
    using G = ClassGen<LA, LB, LC, LD>;
    const int nK = K.nprim, ntot = B.nprim * nK;
    for (int x = start; x < ntot; x += stride) {
        const PrimRec<T> P = prims[B.prim_off + x / nK];
        const PrimRec<T> Q = prims[K.prim_off + x % nK];
        const T pq = P.p + Q.p;
        const T rs = gs_rsqrt(pq);
        const T ipq = rs * rs;
        const T PQx = Q.Px - P.Px, PQy = Q.Py - P.Py, PQz = Q.Pz - P.Pz;
        const T wq = Q.p * ipq, wp = P.p * ipq;
        const T t = P.p * wq * (PQx * PQx + PQy * PQy + PQz * PQz);
        T F[G::L + 1];
        boys<G::L, T>(t, P.Kp * Q.Kp * rs, F);
        VrrCoef<T> c;
        c.PAx = P.PAx; c.PAy = P.PAy; c.PAz = P.PAz;
        c.WPx = wq * PQx; c.WPy = wq * PQy; c.WPz = wq * PQz;
        c.QCx = Q.PAx; c.QCy = Q.PAy; c.QCz = Q.PAz;
        c.WQx = -wp * PQx; c.WQy = -wp * PQy; c.WQz = -wp * PQz;
        c.i2p = P.i2p; c.i2q = Q.i2p;
        c.rp2 = wq * P.i2p; c.rq2 = wp * Q.i2p;
        c.i2pq = T(0.5) * ipq;
        G::vrr(F, c, acc);
    }
}

// ------------------------------------------------------------------ shell-pair records
// Shells as the engine stores them: centre (bohr), angular momentum l, primitives
// [prim_off[s], prim_off[s+1]) with exponent and effective coefficient (contraction times
// primitive and contracted normalisation of the shell's first Cartesian component), and
// comp_scale[s*6 + i], the ratio of component i's normalisation to the first one's.
struct ShellView {
    const double* centre;
    const int* l;
    const int* prim_off;
    const double* expo;
    const double* coef;
};

constexpr double kSqrt2Pi52 = 5.914967172795613;  // sqrt(2 pi^(5/2))

// Record of the primitive pair (a at A, b at B) with contraction coefficients ca, cb.
GS_HD GS_INLINE PrimRec<double> prim_pair(const double* A, const double* B, double a, double b,
                                          double ab2, double ca, double cb) {
    const double p = a + b, ip = 1.0 / p;
    PrimRec<double> r;
    r.p = p;
    r.i2p = 0.5 * ip;
    r.Px = (a * A[0] + b * B[0]) * ip;
    r.Py = (a * A[1] + b * B[1]) * ip;
    r.Pz = (a * A[2] + b * B[2]) * ip;
    r.PAx = r.Px - A[0]; r.PAy = r.Py - A[1]; r.PAz = r.Pz - A[2];
    r.Kp = kSqrt2Pi52 * ca * cb * exp(-a * b * ip * ab2) * ip;
    r.pad = a;          // exponent of the first shell (derivative weights)
    return r;
}

GS_HD GS_INLINE PrimRec<float> prim_pair32(const PrimRec<double>& r) {
    PrimRec<float> f;
    f.p = (float)r.p; f.i2p = (float)r.i2p;
    f.Px = (float)r.Px; f.Py = (float)r.Py; f.Pz = (float)r.Pz;
    f.PAx = (float)r.PAx; f.PAy = (float)r.PAy; f.PAz = (float)r.PAz;
    f.Kp = (float)r.Kp;
    f.pad0 = (float)r.pad;      // exponent of the first shell (FP32 derivative weights)
    f.pad1 = f.pad2 = 0.0f;
    return f;
}

// Primitive-pair screen: drop the pair when its Gaussian-product factor exp(-ab/p |AB|^2)
// is below exp(-max_exp) (max_exp > 0).  Written without the division (ab |AB|^2 >
// max_exp p), which on this part costs more FP64 issue slots than the rest of the test.
GS_HD GS_INLINE bool prim_pair_kept(double a, double b, double ab2, double max_exp) {
    return !(max_exp > 0.0 && a * b * ab2 > max_exp * (a + b));
}

// Fill the PairRec and the primitive-pair records of shell pair (sa, sb); la >= lb.
// Primitive pairs whose Gaussian-product factor exp(-ab/p |AB|^2) is below exp(-max_exp)
// are dropped when max_exp > 0 (their contributions are below that factor times the
// normalised block's scale); pr.nprim is the number kept.  Host form (tests); the device
// builds the same records one warp per pair (capi.cu, k_pairs_build).
GS_HD GS_INLINE void make_pair(const ShellView& S, int sa, int sb, int prim_off, PairRec& pr,
                               PrimRec<double>* pd, PrimRec<float>* pf, double max_exp = 0.0) {
    const double* A = S.centre + 3 * sa;
    const double* B = S.centre + 3 * sb;
    const double ABx = A[0] - B[0], ABy = A[1] - B[1], ABz = A[2] - B[2];
    const double ab2 = ABx * ABx + ABy * ABy + ABz * ABz;
    const int a0 = S.prim_off[sa], a1 = S.prim_off[sa + 1];
    const int b0 = S.prim_off[sb], b1 = S.prim_off[sb + 1];
    pr.ABx = ABx; pr.ABy = ABy; pr.ABz = ABz;
    pr.prim_off = prim_off;
    pr.sa = sa; pr.sb = sb;
    pr.qmax = 0.0f; pr.pad = 0;
    int n = prim_off;
    for (int i = a0; i < a1; ++i) {
        for (int j = b0; j < b1; ++j) {
            const double a = S.expo[i], b = S.expo[j];
            if (!prim_pair_kept(a, b, ab2, max_exp)) continue;
            const PrimRec<double> r = prim_pair(A, B, a, b, ab2, S.coef[i], S.coef[j]);
            pd[n] = r;
            if (pf) pf[n] = prim_pair32(r);
            ++n;
        }
    }
    pr.nprim = n - prim_off;
}

// Original-order strides of a canonical block (see WriteTask::code).
GS_HD GS_INLINE void block_strides(int code, int nA, int nB, int nC, int nD, long long s[4]) {
    const bool b0 = code & 1, b1 = code & 2, b2 = code & 4;
    int n[4];
    int posA, posB, posC, posD;
    if (!b2) {
        n[0] = b0 ? nB : nA; n[1] = b0 ? nA : nB;
        n[2] = b1 ? nD : nC; n[3] = b1 ? nC : nD;
        posA = b0 ? 1 : 0; posB = 1 - posA;
        posC = b1 ? 3 : 2; posD = 5 - posC;
    } else {
        n[2] = b0 ? nB : nA; n[3] = b0 ? nA : nB;
        n[0] = b1 ? nD : nC; n[1] = b1 ? nC : nD;
        posA = b0 ? 3 : 2; posB = 5 - posA;
        posC = b1 ? 1 : 0; posD = 1 - posC;
    }
    long long st[4] = {(long long)n[1] * n[2] * n[3], (long long)n[2] * n[3], n[3], 1};
    s[0] = st[posA]; s[1] = st[posB]; s[2] = st[posC]; s[3] = st[posD];
}

}  // namespace gs
