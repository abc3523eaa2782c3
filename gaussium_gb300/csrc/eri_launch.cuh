// Per-class launcher: the one-thread-per-quartet kernel or the warp-cooperative kernel.
// Which forms a class is built with depends on its total angular momentum L:
//   FP64 thread kernel for L <= GS_THREAD64_MAX, FP64 warp kernel for L >= GS_WIDE_FROM,
//   FP32 thread kernel for L <= GS_THREAD32_MAX, FP32 warp kernel for L >= GS_WIDE32_FROM.
// Where both exist the caller's choice (bits 8.. of the precision argument: 1 = thread,
// 2 = warp) wins, else the default: warp from L = GS_WIDE64_MIN (FP64) or GS_WIDE32_MIN
// (FP32) up.  On GB300 the FP64 pipe is the limit and the warp kernel keeps it busier for
// the larger classes; in FP32 the thread kernel is faster until its state no longer fits.
#pragma once
#include "eri_kernels.cuh"
#include "eri_wide.cuh"

#ifndef GS_WIDE64_MIN
#define GS_WIDE64_MIN 3
#endif
#ifndef GS_WIDE32_MIN
#define GS_WIDE32_MIN 8
#endif
#ifndef GS_THREAD64_MAX
#define GS_THREAD64_MAX 4
#endif
#ifndef GS_THREAD32_MAX
#define GS_THREAD32_MAX 7
#endif
#ifndef GS_WIDE_FROM
#define GS_WIDE_FROM 2
#endif
#ifndef GS_WIDE32_FROM
#define GS_WIDE32_FROM 5
#endif

namespace gs {

template <int L>
struct ClassForms {
    // a class always has at least one form in each precision
    static constexpr bool wide64 = L >= GS_WIDE_FROM;
    static constexpr bool thread64 = L <= GS_THREAD64_MAX || !wide64;
    static constexpr bool wide32 = L >= GS_WIDE32_FROM && L >= GS_WIDE_FROM;
    static constexpr bool thread32 = L <= GS_THREAD32_MAX || !wide32;
};

// bit 0: thread kernel built, bit 1: warp kernel built
template <int LA, int LB, int LC, int LD>
int variants(int prec) {
    using F = ClassForms<LA + LB + LC + LD>;
    if (prec == 64) return (F::thread64 ? 1 : 0) | (F::wide64 ? 2 : 0);
    return (F::thread32 ? 1 : 0) | (F::wide32 ? 2 : 0);
}

template <int LA, int LB, int LC, int LD>
int launch_any(int kind, int prec_variant, const void* args, cudaStream_t st) {
    constexpr int L = LA + LB + LC + LD;
    using F = ClassForms<L>;
    const int variant = prec_variant >> 8;
    int prec = prec_variant & 0xff;
    if (kind == GS_KIND_SCHWARZ) prec = 64;
    if (prec == 64) {
        if constexpr (F::wide64 && F::thread64) {
            const bool wide = variant ? variant == 2 : L >= GS_WIDE64_MIN;
            if (wide) return launch_wide<LA, LB, LC, LD, 64>(kind, args, st);
            return launch_class<LA, LB, LC, LD, 64>(kind, args, st);
        } else if constexpr (F::wide64) {
            return launch_wide<LA, LB, LC, LD, 64>(kind, args, st);
        } else {
            return launch_class<LA, LB, LC, LD, 64>(kind, args, st);
        }
    }
    if constexpr (F::wide32 && F::thread32) {
        const bool wide = variant ? variant == 2 : L >= GS_WIDE32_MIN;
        if (wide) return launch_wide<LA, LB, LC, LD, 32>(kind, args, st);
        return launch_class<LA, LB, LC, LD, 32>(kind, args, st);
    } else if constexpr (F::wide32) {
        return launch_wide<LA, LB, LC, LD, 32>(kind, args, st);
    } else {
        return launch_class<LA, LB, LC, LD, 32>(kind, args, st);
    }
}

}  // namespace gs
