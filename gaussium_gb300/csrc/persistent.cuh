// Persistent batched J/K: one launch per precision evaluates every angular-momentum class
// of every molecule of a batch.
//
// The batch's unique quartet tasks are ordered by class (segment c = [seg[c], seg[c+1])
// of the task array, c in canonical class order).  A partition pass (k_partition_all) puts
// each task that survives density-weighted screening into its class's FP64 or FP32 list,
// at the class's own offset of the list array, and counts them per class.  The persistent
// kernel then strides over the work items of all classes of its precision: a tile of 32
// tasks for a class run in the one-thread-per-quartet form, one task for a class run in
// the warp-per-quartet form.  Item i of warp w is w + k * (warps in the grid): the loop is
// bounded by the item count, nothing waits on another block, and no queue is polled.
//
// The reference distributes the same work over processes with multiprocessing.Pool.starmap
// (matrixelements/electron_repulsion_matrix.py:35-39).
#pragma once
#include "eri_kernels.cuh"
#include "eri_wide.cuh"

namespace gs {

constexpr int kNumClasses = 21;          // canonical classes up to (dd|dd)
constexpr int kPersistWarps = 2;         // warps per block

struct PersistArgs {
    JKArgs jk;                           // tasks = list base of this precision
    const int* counts;                   // [kNumClasses] surviving tasks per class
    int seg[kNumClasses + 1];            // class segment starts in the task / list arrays
};

// canonical class c -> (la lb | lc ld): bra pair class >= ket pair class
#define GS_PERSIST_CLASSES(X)                                                                 \
    X(0, 0, 0, 0, 0) X(1, 1, 0, 0, 0) X(2, 1, 0, 1, 0) X(3, 1, 1, 0, 0) X(4, 1, 1, 1, 0)      \
    X(5, 1, 1, 1, 1) X(6, 2, 0, 0, 0) X(7, 2, 0, 1, 0) X(8, 2, 0, 1, 1) X(9, 2, 0, 2, 0)      \
    X(10, 2, 1, 0, 0) X(11, 2, 1, 1, 0) X(12, 2, 1, 1, 1) X(13, 2, 1, 2, 0) X(14, 2, 1, 2, 1) \
    X(15, 2, 2, 0, 0) X(16, 2, 2, 1, 0) X(17, 2, 2, 1, 1) X(18, 2, 2, 2, 0) X(19, 2, 2, 2, 1) \
    X(20, 2, 2, 2, 2)

// Form of a class inside the persistent kernel: one thread per quartet for the small
// classes (total angular momentum up to 2 in FP64, 4 in FP32), one warp per quartet above,
// grouped (VGROUP primitive quartets per VRR pass) when the class's group is at least 4.
template <int LA, int LB, int LC, int LD, typename T> struct PersistForm {
    static constexpr int L = LA + LB + LC + LD;
    static constexpr bool THREAD = L <= (sizeof(T) == 8 ? 2 : 4);
    static constexpr int VG = WideProg<LA, LB, LC, LD>::VGROUP >= 4 ? WideProg<LA, LB, LC, LD>::VGROUP : 1;
    static constexpr int SMEM = THREAD ? 0 : WideLayout<LA, LB, LC, LD, T, VG>::WARP_JK;
};

template <typename T> struct PersistSmem {
#define GS_PS_MAX(I, A, B, C, D) \
    (PersistForm<A, B, C, D, T>::SMEM > m ? PersistForm<A, B, C, D, T>::SMEM : m);
    static constexpr int compute() {
        int m = 0;
#define GS_PS_STEP(I, A, B, C, D) m = GS_PS_MAX(I, A, B, C, D)
        GS_PERSIST_CLASSES(GS_PS_STEP)
#undef GS_PS_STEP
        return m;
    }
#undef GS_PS_MAX
    static constexpr int WARP = compute();            // elements of T per warp
    static constexpr size_t BYTES = (size_t)WARP * sizeof(T) * kPersistWarps;
};

template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ void persist_item(const PersistArgs& a, int c, int idx, T* sm,
                                             int lane) {
    using F = PersistForm<LA, LB, LC, LD, T>;
    const int begin = a.seg[c], n = a.counts[c];
    if constexpr (F::THREAD) {
        const int t = idx * 32 + lane;
        if (t < n) eri_jk_task<LA, LB, LC, LD, T>(a.jk, begin + t);
    } else {
        wide_jk_task<LA, LB, LC, LD, T, F::VG>(a.jk, begin + idx, sm, lane);
        __syncwarp();
    }
}

template <typename T>
__global__ void __launch_bounds__(32 * kPersistWarps) k_persistent_jk(const PersistArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T* sm = reinterpret_cast<T*>(smem_raw) + (size_t)warp * PersistSmem<T>::WARP;
    // item offsets of the classes: tiles of 32 tasks (thread form) or single tasks (warp)
    int first[kNumClasses + 1];
    first[0] = 0;
#define GS_PI_COUNT(I, A, B, C, D)                                                      \
    {                                                                                   \
        const int n = a.counts[I];                                                      \
        first[I + 1] = first[I] + (PersistForm<A, B, C, D, T>::THREAD ? (n + 31) / 32 : n); \
    }
    GS_PERSIST_CLASSES(GS_PI_COUNT)
#undef GS_PI_COUNT
    const int total = first[kNumClasses];
    const int nwarps = gridDim.x * kPersistWarps;
    int c = 0;
    for (int i = blockIdx.x * kPersistWarps + warp; i < total; i += nwarps) {
        while (i >= first[c + 1]) ++c;               // items ascend: the class only advances
        const int idx = i - first[c];
        switch (c) {
#define GS_PI_CASE(I, A, B, C, D) \
            case I: persist_item<A, B, C, D, T>(a, I, idx, sm, lane); break;
            GS_PERSIST_CLASSES(GS_PI_CASE)
#undef GS_PI_CASE
            default: break;
        }
    }
}

}  // namespace gs
