// Per-class launcher: the one-thread-per-quartet kernel, the warp-cooperative kernel, or the
// warp kernel in its grouped form (WideProg::VGROUP primitive quartets per VRR pass).
// Which forms a class is built with depends on its total angular momentum L:
//   FP64 thread kernel for L <= GS_THREAD64_MAX, FP64 warp kernel for L >= GS_WIDE_FROM,
//   FP32 thread kernel for L <= GS_THREAD32_MAX, FP32 warp kernel for L >= GS_WIDE32_FROM,
//   grouped form wherever the warp kernel is built and the class's group is above 1.
// Where several exist the caller's choice (bits 8.. of the precision argument: 1 = thread,
// 2 = warp, 3 = grouped warp, 4 = split: thread code, one warp per quartet, 5 = cooperative:
// warp code, up to eight warps per quartet, 6 = stacked: warp code, several primitive
// quartets per lane) wins, else the default: the warp kernel from L = GS_WIDE64_MIN
// (FP64) or GS_WIDE32_MIN (FP32) up, grouped when its group is at least 4.  On GB300 a
// warp-wide FP64 instruction holds the pipe for the same time whatever its active lanes, so
// narrow recursion levels are filled with several primitive quartets.
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

template <int LA, int LB, int LC, int LD>
struct ClassForms {
    static constexpr int L = LA + LB + LC + LD;
    static constexpr int VG = WideProg<LA, LB, LC, LD>::VGROUP;
    // a class always has at least one form in each precision
    static constexpr bool wide64 = L >= GS_WIDE_FROM;
    static constexpr bool thread64 = L <= GS_THREAD64_MAX || !wide64;
    static constexpr bool wide32 = L >= GS_WIDE32_FROM && L >= GS_WIDE_FROM;
    static constexpr bool thread32 = L <= GS_THREAD32_MAX || !wide32;
    static constexpr bool grouped64 = wide64 && VG > 1;
    static constexpr bool grouped32 = wide32 && VG > 1;
    // stacked form: wherever the warp kernel is and its block fits the shared memory
    static constexpr bool stacked64 =
        wide64 && WideLayout<LA, LB, LC, LD, double, 1, kStack<double>>::BYTES_JK <= 227 * 1024;
    static constexpr bool stacked32 =
        wide32 && WideLayout<LA, LB, LC, LD, float, 1, kStack<float>>::BYTES_JK <= 227 * 1024;
};

// bit 0: thread kernel built, bit 1: warp kernel built, bit 2: grouped warp kernel built,
// bit 3: split form built (the thread kernel's code, one warp per quartet over its
// primitive quartets; wherever the thread kernel is), bit 4: cooperative form built (the
// warp kernel's code, several warps per quartet; wherever the warp kernel is), bit 5:
// stacked form built (the warp kernel with kStack primitive quartets per lane)
template <int LA, int LB, int LC, int LD>
int variants(int prec) {
    using F = ClassForms<LA, LB, LC, LD>;
    if (prec == 64)
        return (F::thread64 ? 9 : 0) | (F::wide64 ? 18 : 0) | (F::grouped64 ? 4 : 0) |
               (F::stacked64 ? 32 : 0);
    return (F::thread32 ? 9 : 0) | (F::wide32 ? 18 : 0) | (F::grouped32 ? 4 : 0) |
           (F::stacked32 ? 32 : 0);
}

template <int LA, int LB, int LC, int LD, int PREC>
int launch_prec(int kind, int variant, const void* args, cudaStream_t st) {
    using F = ClassForms<LA, LB, LC, LD>;
    constexpr bool thread = PREC == 64 ? F::thread64 : F::thread32;
    constexpr bool wide = PREC == 64 ? F::wide64 : F::wide32;
    constexpr bool grouped = PREC == 64 ? F::grouped64 : F::grouped32;
    constexpr bool stacked = PREC == 64 ? F::stacked64 : F::stacked32;
    constexpr int wide_min = PREC == 64 ? GS_WIDE64_MIN : GS_WIDE32_MIN;
    int v = variant;
    if (v == 0) v = (!thread || F::L >= wide_min) ? (grouped && F::VG >= 4 ? 3 : 2) : 1;
    if (kind == GS_KIND_SCHWARZ && v == 3) v = 2;
    if (kind == GS_KIND_FORM) {
        // the form a launch with this variant resolves to
        if (v == 4 && thread) return 4;
        if (v == 5 && wide) return 5;
        if (v == 6 && stacked) return 6;
        if (v == 3 && grouped) return 3;
        if (v >= 2 && v <= 3 && wide) return 2;
        return thread ? 1 : (wide ? 2 : 0);
    }
    if constexpr (thread) {
        if (v == 4 && kind != GS_KIND_SCHWARZ) {
            // task counts that live on the device run in the thread form
            if (kind == GS_KIND_JK && ((const JKArgs*)args)->ntask_dev)
                return launch_class<LA, LB, LC, LD, PREC>(kind, args, st);
            return launch_class_split<LA, LB, LC, LD, PREC>(kind, args, st);
        }
    }
    if (v == 4) v = 1;
    if constexpr (wide) {
        if (v == 5 && kind != GS_KIND_SCHWARZ) return launch_wide_coop<LA, LB, LC, LD, PREC>(kind, args, st);
    }
    if (v == 5) v = 2;
    if constexpr (stacked) {
        using T = typename std::conditional<PREC == 64, double, float>::type;
        if (v == 6 && kind != GS_KIND_SCHWARZ)
            return launch_wide<LA, LB, LC, LD, PREC, 1, kStack<T>>(kind, args, st);
    }
    if (v == 6) v = 2;
    if constexpr (grouped) {
        if (v == 3) return launch_wide<LA, LB, LC, LD, PREC, F::VG>(kind, args, st);
    }
    if constexpr (wide) {
        if (v >= 2 || !thread) return launch_wide<LA, LB, LC, LD, PREC>(kind, args, st);
    }
    if constexpr (thread) return launch_class<LA, LB, LC, LD, PREC>(kind, args, st);
    return GS_ERR_CLASS;
}

template <int LA, int LB, int LC, int LD>
int launch_any(int kind, int prec_variant, const void* args, cudaStream_t st) {
    const int variant = prec_variant >> 8;
    int prec = prec_variant & 0xff;
    if (kind == GS_KIND_SCHWARZ) prec = 64;
    if (prec == 64) return launch_prec<LA, LB, LC, LD, 64>(kind, variant, args, st);
    return launch_prec<LA, LB, LC, LD, 32>(kind, variant, args, st);
}

}  // namespace gs
