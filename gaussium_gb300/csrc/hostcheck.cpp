// CPU build of the generated ERI recursions, for tests only: it lets the generated
// VRR/HRR code and the Boys function be checked against the oracle without a GPU.  The
// product library never includes or links this file.
#include <cstring>
#include "eri_common.cuh"
#include "eri_classes.h"

using namespace gs;

extern "C" int hc_make_pairs(int npairs, const int* pair_shells, const int* pair_prim_off,
                             const double* centre, const int* l, const int* prim_off,
                             const double* expo, const double* coef, PairRec* pairs,
                             PrimRec<double>* pd, PrimRec<float>* pf) {
    ShellView S{centre, l, prim_off, expo, coef};
    for (int i = 0; i < npairs; ++i)
        make_pair(S, pair_shells[2 * i], pair_shells[2 * i + 1], pair_prim_off[i], pairs[i], pd, pf, 0.0);
    return 0;
}

extern "C" int hc_boys(int M, int prec, double t, double* F) {
    double pref = 1.0;
#define GS_B(MM) case MM: if (prec == 64) { double f[MM + 1]; boys<MM, double>(t, pref, f); \
        for (int i = 0; i <= MM; ++i) F[i] = f[i]; } else { float f[MM + 1]; \
        boys<MM, float>((float)t, 1.0f, f); for (int i = 0; i <= MM; ++i) F[i] = f[i]; } return 0;
    switch (M) { GS_B(0) GS_B(1) GS_B(2) GS_B(3) GS_B(4) GS_B(5) GS_B(6) GS_B(7) GS_B(8) GS_B(9) GS_B(10) }
#undef GS_B
    return -1;
}

// Canonical block of one quartet (bra, ket index into pairs); out gets NA*NB*NC*ND doubles.
extern "C" int hc_eri_block(int la, int lb, int lc, int ld, int prec, const PairRec* pairs,
                            const void* prims, int bra, int ket, double* out) {
#define GS_C(A, B, C, D)                                                                      \
    if (la == A && lb == B && lc == C && ld == D) {                                           \
        constexpr int n = ClassGen<A, B, C, D>::NBLK;                                        \
        if (prec == 64) {                                                                     \
            double blk[n];                                                                    \
            eri_quartet<A, B, C, D, double>(pairs[bra], pairs[ket],                           \
                                            (const PrimRec<double>*)prims, blk);              \
            for (int i = 0; i < n; ++i) out[i] = blk[i];                                      \
        } else {                                                                              \
            float blk[n];                                                                     \
            eri_quartet<A, B, C, D, float>(pairs[bra], pairs[ket],                            \
                                           (const PrimRec<float>*)prims, blk);                \
            for (int i = 0; i < n; ++i) out[i] = blk[i];                                      \
        }                                                                                     \
        return 0;                                                                             \
    }
    GS_FOR_EACH_CLASS(GS_C)
#undef GS_C
    return -1;
}

// ---------------------------------------------------------------------------------------
// FP32 error attribution (tests only).  The FP32 path of the library evaluates the Boys
// function below BOYS_TMAX in FP64 and everything else in FP32.  These variants change one
// stage at a time so a test can tell where FP32 error comes from:
//   mode 0  as the library: FP64 small-T Boys, FP32 VRR, FP32 HRR
//   mode 1  FP64 small-T Boys, FP32 VRR, HRR in FP64 on the FP32 contracted values
//   mode 2  all-FP32 Boys (4-term FP32 Taylor, FP32 downward recursion), FP32 VRR and HRR
//   mode 3  every stage in FP64 on the FP32 primitive-pair records (input rounding only)
namespace {
template <int M>
void boys_all_f32(float t, float pref, float* F) {
    if (t < float(BOYS_TMAX)) {
        const int k = (int)(t * float(BOYS_INV_H) + 0.5f);
        const float d = float(k) * float(1.0 / BOYS_INV_H) - t;
        const double* row = boys_table() + k * BOYS_NCOL;
        const float d2 = d * 0.5f, d3 = d * float(1.0 / 3);
        float f = (float)row[M + 3];
        f = f * d3 + (float)row[M + 2];
        f = f * d2 + (float)row[M + 1];
        f = f * d + (float)row[M];
        F[M] = f * pref;
        if (M > 0) {
            float e = d3 + 1.0f;
            e = e * d2 + 1.0f;
            e = e * d + 1.0f;
            const float et = e * (float)row[BOYS_NCOL - 1] * pref;
            const float t2 = t + t;
            for (int m = M; m >= 1; --m) F[m - 1] = (t2 * F[m] + et) * float(1.0 / (2 * m - 1));
        }
    } else {
        boys<M, float>(t, pref, F);
    }
}

template <int LA, int LB, int LC, int LD>
void quartet_f32_mode(const PairRec& B, const PairRec& K, const PrimRec<float>* prims, int mode,
                      double* out) {
    using G = ClassGen<LA, LB, LC, LD>;
    float acc[G::NACC];
    for (int i = 0; i < G::NACC; ++i) acc[i] = 0.0f;
    for (int i = 0; i < B.nprim; ++i) {
        const PrimRec<float> P = prims[B.prim_off + i];
        for (int j = 0; j < K.nprim; ++j) {
            const PrimRec<float> Q = prims[K.prim_off + j];
            const float pq = P.p + Q.p;
            const float rs = gs_rsqrt(pq);
            const float ipq = rs * rs;
            const float PQx = Q.Px - P.Px, PQy = Q.Py - P.Py, PQz = Q.Pz - P.Pz;
            const float wq = Q.p * ipq, wp = P.p * ipq;
            const float t = P.p * wq * (PQx * PQx + PQy * PQy + PQz * PQz);
            float F[G::L + 1];
            if (mode == 2) boys_all_f32<G::L>(t, P.Kp * Q.Kp * rs, F);
            else boys<G::L, float>(t, P.Kp * Q.Kp * rs, F);
            VrrCoef<float> c;
            c.PAx = P.PAx; c.PAy = P.PAy; c.PAz = P.PAz;
            c.WPx = wq * PQx; c.WPy = wq * PQy; c.WPz = wq * PQz;
            c.QCx = Q.PAx; c.QCy = Q.PAy; c.QCz = Q.PAz;
            c.WQx = -wp * PQx; c.WQy = -wp * PQy; c.WQz = -wp * PQz;
            c.i2p = P.i2p; c.i2q = Q.i2p;
            c.rp2 = wq * P.i2p; c.rq2 = wp * Q.i2p;
            c.i2pq = 0.5f * ipq;
            G::vrr(F, c, acc);
        }
    }
    if (mode == 1) {
        double accd[G::NACC], blk[G::NBLK];
        for (int i = 0; i < G::NACC; ++i) accd[i] = acc[i];
        G::hrr(accd, B.ABx, B.ABy, B.ABz, K.ABx, K.ABy, K.ABz, blk);
        for (int i = 0; i < G::NBLK; ++i) out[i] = blk[i];
    } else {
        float blk[G::NBLK];
        G::hrr(acc, float(B.ABx), float(B.ABy), float(B.ABz), float(K.ABx), float(K.ABy),
               float(K.ABz), blk);
        for (int i = 0; i < G::NBLK; ++i) out[i] = blk[i];
    }
}
}  // namespace

extern "C" int hc_eri_block_f32_mode(int la, int lb, int lc, int ld, int mode,
                                     const PairRec* pairs, const void* prims, int bra, int ket,
                                     double* out) {
    if (mode < 0 || mode > 3) return -1;
#define GS_C(A, B, C, D)                                                                    \
    if (la == A && lb == B && lc == C && ld == D) {                                         \
        if (mode == 3) {                                                                    \
            const PrimRec<float>* pf = (const PrimRec<float>*)prims;                        \
            const int n = pairs[bra].prim_off + pairs[bra].nprim > pairs[ket].prim_off +    \
                          pairs[ket].nprim ? pairs[bra].prim_off + pairs[bra].nprim :       \
                          pairs[ket].prim_off + pairs[ket].nprim;                           \
            PrimRec<double>* pd = new PrimRec<double>[n];                                   \
            for (int i = 0; i < n; ++i) {                                                   \
                pd[i].p = pf[i].p; pd[i].i2p = pf[i].i2p; pd[i].Px = pf[i].Px;               \
                pd[i].Py = pf[i].Py; pd[i].Pz = pf[i].Pz; pd[i].PAx = pf[i].PAx;             \
                pd[i].PAy = pf[i].PAy; pd[i].PAz = pf[i].PAz; pd[i].Kp = pf[i].Kp;           \
                pd[i].pad = 0.0;                                                            \
            }                                                                               \
            double blk[ClassGen<A, B, C, D>::NBLK];                                         \
            eri_quartet<A, B, C, D, double>(pairs[bra], pairs[ket], pd, blk);               \
            for (int i = 0; i < ClassGen<A, B, C, D>::NBLK; ++i) out[i] = blk[i];           \
            delete[] pd;                                                                    \
        } else {                                                                            \
            quartet_f32_mode<A, B, C, D>(pairs[bra], pairs[ket],                            \
                                         (const PrimRec<float>*)prims, mode, out);          \
        }                                                                                   \
        return 0;                                                                           \
    }
    GS_FOR_EACH_CLASS(GS_C)
#undef GS_C
    return -1;
}
