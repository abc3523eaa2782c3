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
