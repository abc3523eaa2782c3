// Class kernels of the ERI engine.  One thread evaluates one contracted shell quartet
// (primitive loops, VRR, contraction, HRR) and then either writes the block, digests it
// into Coulomb/exchange matrices, or reduces it to a Schwarz bound.  Each per-class
// translation unit includes this file and its generated ClassGen header and instantiates
// gs_launch_<class>.
#pragma once
#include <cuda_runtime.h>
#include <type_traits>
#include "eri_common.cuh"
#include "gs_args.h"

namespace gs {

constexpr int kBlock = 128;
#ifndef GS_THREAD_MINB
#define GS_THREAD_MINB 1
#endif

// Block write epilogue: the canonical block of `task`, scaled per component, at its
// original-order position.
template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ void write_block(const WriteArgs& a, const WriteTask& task,
                                            const PairRec& B, const PairRec& K, const T* blk) {
    using G = ClassGen<LA, LB, LC, LD>;
    long long s[4];
    block_strides(task.code, G::NA, G::NB, G::NC, G::ND, s);
    double sab[G::NA * G::NB], scd[G::NC * G::ND];
    GS_UNROLL for (int i = 0; i < G::NA; ++i)
        GS_UNROLL for (int j = 0; j < G::NB; ++j)
            sab[i * G::NB + j] = a.comp_scale[6 * B.sa + i] * a.comp_scale[6 * B.sb + j];
    GS_UNROLL for (int i = 0; i < G::NC; ++i)
        GS_UNROLL for (int j = 0; j < G::ND; ++j)
            scd[i * G::ND + j] = a.comp_scale[6 * K.sa + i] * a.comp_scale[6 * K.sb + j];
    double* out = a.out + task.off;
    GS_UNROLL for (int ia = 0; ia < G::NA; ++ia)
    GS_UNROLL for (int ib = 0; ib < G::NB; ++ib)
    GS_UNROLL for (int ic = 0; ic < G::NC; ++ic)
    GS_UNROLL for (int id = 0; id < G::ND; ++id) {
        const int e = ((ia * G::NB + ib) * G::NC + ic) * G::ND + id;
        out[ia * s[0] + ib * s[1] + ic * s[2] + id * s[3]] =
            (double)blk[e] * (sab[ia * G::NB + ib] * scd[ic * G::ND + id]);
    }
}

template <int LA, int LB, int LC, int LD, typename T>
__global__ void __launch_bounds__(kBlock, GS_THREAD_MINB) k_eri_write(const WriteArgs a) {
    using G = ClassGen<LA, LB, LC, LD>;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.ntask) return;
    const WriteTask task = a.tasks[t];
    const PairRec B = a.pairs[task.bra];
    const PairRec K = a.pairs[task.ket];
    T blk[G::NBLK];
    eri_quartet<LA, LB, LC, LD, T>(B, K, (const PrimRec<T>*)a.prims, blk);
    write_block<LA, LB, LC, LD, T>(a, task, B, K, blk);
}

// Split form of the thread kernel for quartets with many primitive quartets: one warp per
// quartet, lane l takes primitive quartets l, l + 32, ... with the thread form's
// straight-line recursion, the warp sums the contraction accumulators (butterfly), and
// lane 0 runs the horizontal recursion and the epilogue.
template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ bool split_accumulate(const PairRec& B, const PairRec& K,
                                                 const PrimRec<T>* prims, T* acc, int lane) {
    using G = ClassGen<LA, LB, LC, LD>;
    GS_UNROLL for (int i = 0; i < G::NACC; ++i) acc[i] = T(0);
    eri_accumulate<LA, LB, LC, LD, T>(B, K, prims, acc, lane, 32);
    GS_UNROLL for (int i = 0; i < G::NACC; ++i)
        GS_UNROLL for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
    return lane == 0;
}

constexpr int kSplitWarps = 4;          // warps (quartets) per block of the split form

template <int LA, int LB, int LC, int LD, typename T>
__global__ void __launch_bounds__(32 * kSplitWarps) k_eri_write_split(const WriteArgs a) {
    using G = ClassGen<LA, LB, LC, LD>;
    const int lane = threadIdx.x & 31;
    const int t = blockIdx.x * kSplitWarps + (threadIdx.x >> 5);
    if (t >= a.ntask) return;                      // warp-uniform
    const WriteTask task = a.tasks[t];
    const PairRec B = a.pairs[task.bra];
    const PairRec K = a.pairs[task.ket];
    T acc[G::NACC];
    if (split_accumulate<LA, LB, LC, LD, T>(B, K, (const PrimRec<T>*)a.prims, acc, lane)) {
        T blk[G::NBLK];
        G::hrr(acc, T(B.ABx), T(B.ABy), T(B.ABz), T(K.ABx), T(K.ABy), T(K.ABz), blk);
        write_block<LA, LB, LC, LD, T>(a, task, B, K, blk);
    }
}


// Density-weighted screening bound of a J/K task: true when the task is to be evaluated
// (always, without screening).
__device__ __forceinline__ bool jk_keep(const JKArgs& a, const PairRec& B, const PairRec& K) {
    if (a.screen_thr <= 0.0) return true;
    const double bound = (double)B.qmax * (double)K.qmax;
    double dm;
    if (a.shell_mol) {
        dm = a.mol_dmax[a.shell_mol[B.sa]];
    } else {
        const int ns = a.nshell;
        dm = a.shell_dmax[B.sa * ns + B.sb];
        dm = fmax(dm, a.shell_dmax[K.sa * ns + K.sb]);
        dm = fmax(dm, a.shell_dmax[B.sa * ns + K.sa]);
        dm = fmax(dm, a.shell_dmax[B.sa * ns + K.sb]);
        dm = fmax(dm, a.shell_dmax[B.sb * ns + K.sa]);
        dm = fmax(dm, a.shell_dmax[B.sb * ns + K.sb]);
    }
    const double est = bound * dm;
    return !(est < a.screen_thr || est < a.prec_lo || est >= a.prec_hi);
}

// The J/K digestion of one evaluated block (see eri_jk_task).
template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ void jk_digest(const JKArgs& a, const int2 task, const PairRec& B,
                                          const PairRec& K, const T* blk, int n,
                                          long long mbase) {
    using G = ClassGen<LA, LB, LC, LD>;
    constexpr int NA = G::NA, NB = G::NB, NC = G::NC, ND = G::ND;
    const double deg = (B.sa == B.sb ? 0.5 : 1.0) * (K.sa == K.sb ? 0.5 : 1.0) *
                       (task.x == task.y ? 0.5 : 1.0);
    const double* cs = a.comp_scale;
    T sc[NA * NB * NC * ND];
    {
        T sab[NA * NB], scd[NC * ND];
        GS_UNROLL for (int i = 0; i < NA; ++i)
            GS_UNROLL for (int j = 0; j < NB; ++j)
                sab[i * NB + j] = (T)(deg * cs[6 * B.sa + i] * cs[6 * B.sb + j]);
        GS_UNROLL for (int i = 0; i < NC; ++i)
            GS_UNROLL for (int j = 0; j < ND; ++j)
                scd[i * ND + j] = (T)(cs[6 * K.sa + i] * cs[6 * K.sb + j]);
        GS_UNROLL for (int ab = 0; ab < NA * NB; ++ab)
            GS_UNROLL for (int cd = 0; cd < NC * ND; ++cd)
                sc[ab * NC * ND + cd] = blk[ab * NC * ND + cd] * (sab[ab] * scd[cd]);
    }
    const int fa = a.func_off[B.sa], fb = a.func_off[B.sb];
    const int fc = a.func_off[K.sa], fd = a.func_off[K.sb];
    if (a.j) {
        const double* P = a.pj + mbase;
        double* Jo = a.j + mbase;
        T pab[NA * NB], pcd[NC * ND];
        GS_UNROLL for (int i = 0; i < NA; ++i)
            GS_UNROLL for (int j = 0; j < NB; ++j) pab[i * NB + j] = (T)P[(fa + i) * n + fb + j];
        GS_UNROLL for (int i = 0; i < NC; ++i)
            GS_UNROLL for (int j = 0; j < ND; ++j) pcd[i * ND + j] = (T)P[(fc + i) * n + fd + j];
        T jab[NA * NB], jcd[NC * ND];
        GS_UNROLL for (int i = 0; i < NA * NB; ++i) jab[i] = T(0);
        GS_UNROLL for (int i = 0; i < NC * ND; ++i) jcd[i] = T(0);
        GS_UNROLL for (int ab = 0; ab < NA * NB; ++ab)
            GS_UNROLL for (int cd = 0; cd < NC * ND; ++cd) {
                const T v = sc[ab * NC * ND + cd];
                jab[ab] += v * pcd[cd];
                jcd[cd] += v * pab[ab];
            }
        GS_UNROLL for (int i = 0; i < NA; ++i)
            GS_UNROLL for (int j = 0; j < NB; ++j)
                atomicAdd(Jo + (fa + i) * n + fb + j, 2.0 * (double)jab[i * NB + j]);
        GS_UNROLL for (int i = 0; i < NC; ++i)
            GS_UNROLL for (int j = 0; j < ND; ++j)
                atomicAdd(Jo + (fc + i) * n + fd + j, 2.0 * (double)jcd[i * ND + j]);
    }
    for (int s = 0; s < a.nk; ++s) {
        const double* P = a.pk + (size_t)s * a.mat_stride + mbase;
        double* Kout = a.k + (size_t)s * a.mat_stride + mbase;
        T pbd[NB * ND], pbc[NB * NC], pad[NA * ND], pac[NA * NC];
        GS_UNROLL for (int i = 0; i < NB; ++i)
            GS_UNROLL for (int j = 0; j < ND; ++j) pbd[i * ND + j] = (T)P[(fb + i) * n + fd + j];
        GS_UNROLL for (int i = 0; i < NB; ++i)
            GS_UNROLL for (int j = 0; j < NC; ++j) pbc[i * NC + j] = (T)P[(fb + i) * n + fc + j];
        GS_UNROLL for (int i = 0; i < NA; ++i)
            GS_UNROLL for (int j = 0; j < ND; ++j) pad[i * ND + j] = (T)P[(fa + i) * n + fd + j];
        GS_UNROLL for (int i = 0; i < NA; ++i)
            GS_UNROLL for (int j = 0; j < NC; ++j) pac[i * NC + j] = (T)P[(fa + i) * n + fc + j];
        T kac[NA * NC], kad[NA * ND], kbc[NB * NC], kbd[NB * ND];
        GS_UNROLL for (int i = 0; i < NA * NC; ++i) kac[i] = T(0);
        GS_UNROLL for (int i = 0; i < NA * ND; ++i) kad[i] = T(0);
        GS_UNROLL for (int i = 0; i < NB * NC; ++i) kbc[i] = T(0);
        GS_UNROLL for (int i = 0; i < NB * ND; ++i) kbd[i] = T(0);
        GS_UNROLL for (int ia = 0; ia < NA; ++ia)
        GS_UNROLL for (int ib = 0; ib < NB; ++ib)
        GS_UNROLL for (int ic = 0; ic < NC; ++ic)
        GS_UNROLL for (int id = 0; id < ND; ++id) {
            const T v = sc[((ia * NB + ib) * NC + ic) * ND + id];
            kac[ia * NC + ic] += v * pbd[ib * ND + id];
            kad[ia * ND + id] += v * pbc[ib * NC + ic];
            kbc[ib * NC + ic] += v * pad[ia * ND + id];
            kbd[ib * ND + id] += v * pac[ia * NC + ic];
        }
        GS_UNROLL for (int i = 0; i < NA; ++i)
            GS_UNROLL for (int j = 0; j < NC; ++j)
                atomicAdd(Kout + (fa + i) * n + fc + j, (double)kac[i * NC + j]);
        GS_UNROLL for (int i = 0; i < NA; ++i)
            GS_UNROLL for (int j = 0; j < ND; ++j)
                atomicAdd(Kout + (fa + i) * n + fd + j, (double)kad[i * ND + j]);
        GS_UNROLL for (int i = 0; i < NB; ++i)
            GS_UNROLL for (int j = 0; j < NC; ++j)
                atomicAdd(Kout + (fb + i) * n + fc + j, (double)kbc[i * NC + j]);
        GS_UNROLL for (int i = 0; i < NB; ++i)
            GS_UNROLL for (int j = 0; j < ND; ++j)
                atomicAdd(Kout + (fb + i) * n + fd + j, (double)kbd[i * ND + j]);
    }
}

// Digest the unique quartet (ab|cd) into the symmetric-accumulation matrices
//   J'_ab += 2 v P_cd,  J'_cd += 2 v P_ab,
//   K'_ac += v P_bd, K'_ad += v P_bc, K'_bc += v P_ad, K'_bd += v P_ac   (per density)
// with v = (ab|cd) / ((1+d_ab)(1+d_cd)(1+d_ab,cd)), so that J = J' + J'^T and
// K = K' + K'^T sum every permutation of every quartet once.
template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ void jk_target(const JKArgs& a, const PairRec& B, int& n,
                                          long long& mbase) {
    n = a.nbf;
    mbase = 0;
    if (a.shell_mol) {
        const int m = a.shell_mol[B.sa];
        n = a.mol_n[m];
        mbase = a.mol_base[m];
    }
}

template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ void eri_jk_task(const JKArgs& a, int t) {
    using G = ClassGen<LA, LB, LC, LD>;
    const int2 task = a.tasks[t];
    const PairRec B = a.pairs[task.x];
    const PairRec K = a.pairs[task.y];
    if (!jk_keep(a, B, K)) return;           // density-weighted screening, precision band
    int n;
    long long mbase;
    jk_target<LA, LB, LC, LD, T>(a, B, n, mbase);
    T blk[G::NBLK];
    eri_quartet<LA, LB, LC, LD, T>(B, K, (const PrimRec<T>*)a.prims, blk);
    jk_digest<LA, LB, LC, LD, T>(a, task, B, K, blk, n, mbase);
}

// Split form (see k_eri_write_split): one warp per task.
template <int LA, int LB, int LC, int LD, typename T>
__global__ void __launch_bounds__(32 * kSplitWarps) k_eri_jk_split(const JKArgs a) {
    using G = ClassGen<LA, LB, LC, LD>;
    const int lane = threadIdx.x & 31;
    const int t = blockIdx.x * kSplitWarps + (threadIdx.x >> 5);
    if (t >= a.ntask) return;                      // warp-uniform
    const int2 task = a.tasks[t];
    const PairRec B = a.pairs[task.x];
    const PairRec K = a.pairs[task.y];
    if (!jk_keep(a, B, K)) return;                 // warp-uniform: one task per warp
    T acc[G::NACC];
    if (split_accumulate<LA, LB, LC, LD, T>(B, K, (const PrimRec<T>*)a.prims, acc, lane)) {
        int n;
        long long mbase;
        jk_target<LA, LB, LC, LD, T>(a, B, n, mbase);
        T blk[G::NBLK];
        G::hrr(acc, T(B.ABx), T(B.ABy), T(B.ABz), T(K.ABx), T(K.ABy), T(K.ABz), blk);
        jk_digest<LA, LB, LC, LD, T>(a, task, B, K, blk, n, mbase);
    }
}

// One thread per task; with a task count on the device (after a partition) the grid is
// capped and each thread strides over the tasks.
template <int LA, int LB, int LC, int LD, typename T>
__global__ void __launch_bounds__(kBlock, GS_THREAD_MINB) k_eri_jk(const JKArgs a) {
    const int n = a.ntask_dev ? *a.ntask_dev : a.ntask;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
        eri_jk_task<LA, LB, LC, LD, T>(a, t);
}

// Blocks launched for a task count that lives on the device: 16 per SM fill the GPU.
constexpr int kDeviceCountBlocksPerSM = 16;

// Schwarz bound of shell pairs: q[p] = sqrt(max_ijkl |(ab|ab)|) over the scaled block.
template <int LA, int LB, typename T>
__global__ void __launch_bounds__(kBlock) k_schwarz(const SchwarzArgs a) {
    using G = ClassGen<LA, LB, LA, LB>;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.npair) return;
    const int p = a.pair_index[t];
    const PairRec B = a.pairs[p];
    T blk[G::NBLK];
    eri_quartet<LA, LB, LA, LB, T>(B, B, (const PrimRec<T>*)a.prims, blk);
    double m = 0.0;
    GS_UNROLL for (int ia = 0; ia < G::NA; ++ia)
    GS_UNROLL for (int ib = 0; ib < G::NB; ++ib) {
        // diagonal elements (ab|ab) carry the bound
        const int ab = ia * G::NB + ib;
        const double s = a.comp_scale[6 * B.sa + ia] * a.comp_scale[6 * B.sb + ib];
        m = fmax(m, fabs((double)blk[ab * G::NA * G::NB + ab]) * s * s);
    }
    a.q[p] = sqrt(m);
}

// The split form (one warp per quartet over its primitive quartets, thread-form code).
// Task counts on the device (partitioned lists) are not supported; those launches use the
// thread form.
template <int LA, int LB, int LC, int LD, int PREC>
int launch_class_split(int kind, const void* args, cudaStream_t st) {
    using T = typename std::conditional<PREC == 64, double, float>::type;
    constexpr int TPB = 32 * kSplitWarps;
    if (kind == GS_KIND_WRITE) {
        const WriteArgs& a = *(const WriteArgs*)args;
        if (a.ntask <= 0) return 0;
        k_eri_write_split<LA, LB, LC, LD, T><<<(a.ntask + kSplitWarps - 1) / kSplitWarps, TPB, 0, st>>>(a);
    } else if (kind == GS_KIND_JK) {
        const JKArgs& a = *(const JKArgs*)args;
        if (a.ntask <= 0) return 0;
        if (a.ntask_dev) return GS_ERR_ARG;
        k_eri_jk_split<LA, LB, LC, LD, T><<<(a.ntask + kSplitWarps - 1) / kSplitWarps, TPB, 0, st>>>(a);
    } else {
        return GS_ERR_ARG;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : GS_ERR_CUDA;
}

template <int LA, int LB, int LC, int LD, int PREC>
int launch_class(int kind, const void* args, cudaStream_t st) {
    using T = typename std::conditional<PREC == 64, double, float>::type;
    if (kind == GS_KIND_WRITE) {
        const WriteArgs& a = *(const WriteArgs*)args;
        if (a.ntask <= 0) return 0;
        k_eri_write<LA, LB, LC, LD, T><<<(a.ntask + kBlock - 1) / kBlock, kBlock, 0, st>>>(a);
    } else if (kind == GS_KIND_JK) {
        const JKArgs& a = *(const JKArgs*)args;
        if (a.ntask <= 0) return 0;
        int grid = (a.ntask + kBlock - 1) / kBlock;
        if (a.ntask_dev && grid > kDeviceCountBlocksPerSM * sm_count())
            grid = kDeviceCountBlocksPerSM * sm_count();
        k_eri_jk<LA, LB, LC, LD, T><<<grid, kBlock, 0, st>>>(a);
    } else if (kind == GS_KIND_SCHWARZ) {
        if constexpr (LA == LC && LB == LD && PREC == 64) {
            const SchwarzArgs& a = *(const SchwarzArgs*)args;
            if (a.npair <= 0) return 0;
            k_schwarz<LA, LB, double><<<(a.npair + kBlock - 1) / kBlock, kBlock, 0, st>>>(a);
        } else {
            return GS_ERR_CLASS;
        }
    } else {
        return GS_ERR_ARG;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : GS_ERR_CUDA;
}

}  // namespace gs
