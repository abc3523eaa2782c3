// Per-class launcher: picks the one-thread-per-quartet kernel or the warp-cooperative
// kernel by total angular momentum and precision.  On GB300 the FP64 pipe is the limit and
// the warp kernel keeps it busier from L = GS_WIDE64_MIN up; in FP32 the thread kernel is
// faster until its state no longer fits (L >= GS_WIDE32_MIN).
#pragma once
#include "eri_kernels.cuh"
#include "eri_wide.cuh"

#ifndef GS_WIDE64_MIN
#define GS_WIDE64_MIN 5
#endif
#ifndef GS_WIDE32_MIN
#define GS_WIDE32_MIN 7
#endif

namespace gs {

template <int LA, int LB, int LC, int LD>
int launch_any(int kind, int prec, const void* args, cudaStream_t st) {
    constexpr int L = LA + LB + LC + LD;
    constexpr bool wide64 = L >= GS_WIDE64_MIN, wide32 = L >= GS_WIDE32_MIN;
    if (kind == GS_KIND_SCHWARZ) prec = 64;
    if (prec == 64) {
        if constexpr (wide64) return launch_wide<LA, LB, LC, LD, 64>(kind, args, st);
        else return launch_class<LA, LB, LC, LD, 64>(kind, args, st);
    }
    if constexpr (wide32) return launch_wide<LA, LB, LC, LD, 32>(kind, args, st);
    else return launch_class<LA, LB, LC, LD, 32>(kind, args, st);
}

}  // namespace gs
