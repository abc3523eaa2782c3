// Warp-cooperative class kernels for the high angular-momentum classes, whose per-quartet
// state (thousands of recursion intermediates) does not fit one thread.  One warp
// evaluates one contracted shell quartet:
//   1. setup, lane-parallel over primitive quartets: each lane prepares the recursion
//      coefficients and scaled Boys values of one primitive quartet in shared memory;
//   2. VRR, node-parallel: for each primitive quartet the warp walks the generated node
//      program level by level (nodes of a level are independent), reading operands and
//      coefficients from shared memory; each lane keeps a slice of the contracted
//      [e0|f0] accumulators in registers;
//   3. HRR, element-parallel on a liveness-planned shared buffer;
//   4. epilogue: block write, J/K digestion or Schwarz reduction.
// The node programs come from gen_eri.py (WideProg<...> tables).
#pragma once
#include <type_traits>
#include "eri_common.cuh"
#include "eri_kernels.cuh"
#include "gs_args.h"

namespace gs {

template <int LA, int LB, int LC, int LD> struct WideProg;

#ifndef GS_WIDE_WARPS
#define GS_WIDE_WARPS 2
#endif
#ifndef GS_SETUP_BATCH
#define GS_SETUP_BATCH 32
#endif
#ifndef GS_WIDE_MINB
#define GS_WIDE_MINB 1        // minimum resident blocks per SM asked of the compiler
#endif
constexpr int kWideWarps = GS_WIDE_WARPS;     // warps per block
constexpr int kNCoef = 32;                    // coefficient slots per primitive quartet
// coefficient slot set to zero after the set-up: the padding term of nodes whose wave holds
// nodes with more terms (gen_eri.py ZERO_COEF; the i2p_4 slot, unused up to (dd|dd))
constexpr int kZeroCoef = 15;
constexpr int kSetupBatch = GS_SETUP_BATCH;   // primitive quartets prepared per setup round
// primitive quartets per lane in the stacked form: FP32 nodes are cheap beside their record
// decode and operand loads, so four share one decode; FP64 stacks two, for the independent
// FMA chains
template <typename T> constexpr int kStack = sizeof(T) == 8 ? 2 : 4;
static_assert(kSetupBatch >= 1 && kSetupBatch <= 32, "one primitive quartet per lane at most");
static_assert(kWideWarps >= 1 && kWideWarps <= 32, "warps per block");
// VG: primitive quartets a warp pushes through the VRR node program at once (1, or the
// class's WideProg::VGROUP for the grouped form).  RQ: primitive quartets each lane runs its
// node record on (1, or kStack for the stacked form): the ungrouped program, one record
// decode for RQ quartets with RQ node buffers.
template <int LA, int LB, int LC, int LD, typename T, int VG = 1, int RQ = 1> struct WideLayout {
    using G = ClassGen<LA, LB, LC, LD>;
    using W = WideProg<LA, LB, LC, LD>;
    // primitive quartets set up per round: a grouped form with large node buffers prepares
    // half as many, so that its shared memory stays near the ungrouped form's
    // node slots of the program this form runs (the grouped form has its own schedule)
    static constexpr int NVS = VG == 1 ? W::NVSLOT : W::NVSLOT_G;
    // primitive quartets set up per round: 32, or 16 for a form whose node buffers are
    // large -- grouped with more than 1088 slots (above (pp|pp)'s 8 x 132, its slot count
    // padded for the banks), or an ungrouped class of total angular
    // momentum 7 or more whose VRR buffers would outgrow the HRR's (measured: (dd|dp)
    // 17.7 -> 16.0 ms at 2,000,000 quartets; the smaller classes lose setup parallelism)
    static constexpr int VRR32 = 32 * kNCoef + 32 * (G::L + 1) + VG * RQ * NVS;
    static constexpr int HRR_W = W::HSIZE + G::NA * G::NB + G::NC * G::ND;
    static constexpr int SB = kSetupBatch > 16 && ((VG * RQ > 1 && VG * RQ * NVS > 1088) ||
                                                   (VG * RQ == 1 && G::L >= 7 && VRR32 > HRR_W))
                                  ? 16 : kSetupBatch;
    static_assert(SB % RQ == 0, "setup rounds hold whole stacks");
    static constexpr int SC = SB * kNCoef;                       // coefficients
    static constexpr int SF = SB * (G::L + 1);                   // Boys values
    static constexpr int VRR = SC + SF + VG * RQ * NVS;
    // write/Schwarz epilogues need the HRR buffer and the scale vectors; the J/K epilogue
    // also a scaled copy of the block
    static constexpr int HR_W = W::HSIZE + G::NA * G::NB + G::NC * G::ND;
    static constexpr int HR_JK = W::HSIZE + G::NBLK + G::NA * G::NB + G::NC * G::ND;
    static constexpr int WARP_W = VRR > HR_W ? VRR : HR_W;       // elements of T per warp
    static constexpr int WARP_JK = VRR > HR_JK ? VRR : HR_JK;
    static constexpr size_t BYTES_W = (size_t)WARP_W * sizeof(T) * kWideWarps;
    static constexpr size_t BYTES_JK = (size_t)WARP_JK * sizeof(T) * kWideWarps;
};

template <typename T>
__device__ __forceinline__ void wide_setup(const PrimRec<T>& P, const PrimRec<T>& Q, int L,
                                           T* __restrict__ c, T* __restrict__ F);

template <int M, typename T>
__device__ __forceinline__ void wide_setup_m(const PrimRec<T>& P, const PrimRec<T>& Q,
                                             T* __restrict__ c, T* __restrict__ F) {
    const T pq = P.p + Q.p;
    const T rs = gs_rsqrt(pq);
    const T ipq = rs * rs;
    const T PQx = Q.Px - P.Px, PQy = Q.Py - P.Py, PQz = Q.Pz - P.Pz;
    const T wq = Q.p * ipq, wp = P.p * ipq;
    const T t = P.p * wq * (PQx * PQx + PQy * PQy + PQz * PQz);
    T f[M + 1];
    boys<M, T>(t, P.Kp * Q.Kp * rs, f);
#pragma unroll
    for (int m = 0; m <= M; ++m) F[m] = f[m];
    c[0] = P.PAx; c[1] = P.PAy; c[2] = P.PAz;
    c[3] = wq * PQx; c[4] = wq * PQy; c[5] = wq * PQz;
    c[6] = Q.PAx; c[7] = Q.PAy; c[8] = Q.PAz;
    c[9] = -wp * PQx; c[10] = -wp * PQy; c[11] = -wp * PQz;
    const T i2p = P.i2p, i2q = Q.i2p, rp2 = wq * P.i2p, rq2 = wp * Q.i2p, i2pq = T(0.5) * ipq;
#pragma unroll
    for (int k = 1; k <= 4; ++k) {
        c[12 + k - 1] = T(k) * i2p;
        c[16 + k - 1] = -T(k) * rp2;
        c[20 + k - 1] = T(k) * i2q;
        c[24 + k - 1] = -T(k) * rq2;
        c[28 + k - 1] = T(k) * i2pq;
    }
}

// One synchronisation step of the VRR node program: the step's records (noff .. noff+cnt)
// form waves of WAVE records, each carrying its wave's term count (padded terms multiply
// the zero coefficient).  A lane takes record j of every wave.  The loop is software
// pipelined: the operands of the next wave are read from shared memory, and the record of
// the wave after it from the read-only cache, before the current node is stored -- nodes of
// one step never read another node of the same step, and never overwrite a slot the step
// still reads (gen_eri.vrr_waves), so no ordering inside the step is needed.
template <int WAVE, typename T>
__device__ __forceinline__ void vrr_step(const uint4* __restrict__ vrec, int noff, int cnt,
                                         bool group_ok, const T* __restrict__ c, T* nd, int j) {
    const int nw = (cnt + WAVE - 1) / WAVE;
    uint4 a = make_uint4(0, 0, 0, 0), b = a, na = a, nb = a;
    T c0 = T(0), v0 = T(0), c1 = T(0), v1 = T(0), c2 = T(0), v2 = T(0), c3 = T(0), v3 = T(0);
    T c4 = T(0), v4 = T(0);
    int n = j;
    bool act = group_ok && n < cnt;
    if (act) {
        a = __ldg(vrec + 2 * (noff + n));
        b = __ldg(vrec + 2 * (noff + n) + 1);
        const int nt = a.x >> 16;
        c0 = c[a.y >> 16]; v0 = nd[a.y & 0xffff];
        c1 = c[a.z >> 16]; v1 = nd[a.z & 0xffff];
        if (nt > 2) { c2 = c[a.w >> 16]; v2 = nd[a.w & 0xffff]; }
        if (nt > 3) { c3 = c[b.x >> 16]; v3 = nd[b.x & 0xffff]; }
        if (nt > 4) { c4 = c[b.y >> 16]; v4 = nd[b.y & 0xffff]; }
    }
    bool nact = group_ok && n + WAVE < cnt;
    if (nact) {
        na = __ldg(vrec + 2 * (noff + n + WAVE));
        nb = __ldg(vrec + 2 * (noff + n + WAVE) + 1);
    }
    for (int w = 0; w < nw; ++w) {
        const int nt = a.x >> 16;
        T r = c0 * v0;
        r = fma(c1, v1, r);
        if (nt > 2) r = fma(c2, v2, r);
        if (nt > 3) r = fma(c3, v3, r);
        if (nt > 4) r = fma(c4, v4, r);
        const int out = a.x & 0xffff;
        const bool was = act;
        a = na; b = nb; act = nact;
        if (act) {                                   // operands of the next wave
            const int mt = a.x >> 16;
            c0 = c[a.y >> 16]; v0 = nd[a.y & 0xffff];
            c1 = c[a.z >> 16]; v1 = nd[a.z & 0xffff];
            if (mt > 2) { c2 = c[a.w >> 16]; v2 = nd[a.w & 0xffff]; }
            if (mt > 3) { c3 = c[b.x >> 16]; v3 = nd[b.x & 0xffff]; }
            if (mt > 4) { c4 = c[b.y >> 16]; v4 = nd[b.y & 0xffff]; }
        }
        nact = group_ok && n + 2 * WAVE < cnt;       // record of the wave after it
        if (nact) {
            na = __ldg(vrec + 2 * (noff + n + 2 * WAVE));
            nb = __ldg(vrec + 2 * (noff + n + 2 * WAVE) + 1);
        }
        if (was) nd[out] = r;
        n += WAVE;
    }
}

// One synchronisation step of the ungrouped node program for a stack of ng <= RQ primitive
// quartets: lane j takes record j of every wave of 32, decodes it once and runs it on each
// quartet of the stack (coefficients c + r kNCoef, node buffer nd + r NVS).  The quartets
// are independent FMA chains, so the record's operand loads overlap without prefetching.
// Nodes of one step never read one another, so each wave's results are stored before the
// next wave's operands are read.
template <int RQ, int NVS, typename T>
__device__ __forceinline__ void vrr_step_rq(const uint4* __restrict__ vrec, int noff, int cnt,
                                            int ng, const T* __restrict__ c, T* nd, int j) {
    uint4 a = make_uint4(0, 0, 0, 0), b = a, na = a, nb = a;
    int n = j;
    bool act = n < cnt;
    if (act) {
        a = __ldg(vrec + 2 * (noff + n));
        b = __ldg(vrec + 2 * (noff + n) + 1);
    }
    while (act) {
        const bool nact = n + 32 < cnt;
        if (nact) {                                  // record of the next wave
            na = __ldg(vrec + 2 * (noff + n + 32));
            nb = __ldg(vrec + 2 * (noff + n + 32) + 1);
        }
        const int nt = a.x >> 16, out = a.x & 0xffff;
        const int k0 = a.y >> 16, s0 = a.y & 0xffff, k1 = a.z >> 16, s1 = a.z & 0xffff;
        const int k2 = a.w >> 16, s2 = a.w & 0xffff, k3 = b.x >> 16, s3 = b.x & 0xffff;
        const int k4 = b.y >> 16, s4 = b.y & 0xffff;
        T r[RQ];
#pragma unroll
        for (int q = 0; q < RQ; ++q) {
            if (q < ng) {
                const T* __restrict__ cq = c + q * kNCoef;
                const T* vq = nd + q * NVS;
                T v = cq[k0] * vq[s0];
                v = fma(cq[k1], vq[s1], v);
                if (nt > 2) v = fma(cq[k2], vq[s2], v);
                if (nt > 3) v = fma(cq[k3], vq[s3], v);
                if (nt > 4) v = fma(cq[k4], vq[s4], v);
                r[q] = v;
            }
        }
#pragma unroll
        for (int q = 0; q < RQ; ++q)
            if (q < ng) nd[q * NVS + out] = r[q];
        a = na;
        b = nb;
        act = nact;
        n += 32;
    }
}

// Contracted [e0|f0] targets of primitive quartets first, first + stride, ... of the
// quartet (set up Lay::SB at a time): target lane + 32 k is added to acc[k].
template <int LA, int LB, int LC, int LD, typename T, int VG, int RQ = 1>
__device__ __forceinline__ void wide_contract(const PairRec& B, const PairRec& K,
                                              const PrimRec<T>* __restrict__ prims,
                                              T* __restrict__ sm, int lane, int first, int stride,
                                              T* __restrict__ acc) {
    static_assert(VG == 1 || RQ == 1, "grouped and stacked forms are separate");
    using G = ClassGen<LA, LB, LC, LD>;
    using W = WideProg<LA, LB, LC, LD>;
    using Lay = WideLayout<LA, LB, LC, LD, T, VG, RQ>;
    constexpr int L = G::L;
    constexpr int NACC = G::NACC;
    constexpr int NACCW = (NACC + 31) / 32;
    T* sC = sm;
    T* sF = sm + Lay::SC;
    T* node = sm + Lay::SC + Lay::SF;
    const int nK = K.nprim;
    const int nmine = first < B.nprim * nK ? (B.nprim * nK - first + stride - 1) / stride : 0;
    // the node program: waves of at most 32 nodes (one per lane), or of 32/VG nodes for the
    // grouped form (one per lane group of VG primitive quartets)
    constexpr int NVS = Lay::NVS;
    constexpr int NVSEG = VG == 1 ? W::NVSEG : W::NVSEG_G;
    const uint4* __restrict__ vrec = VG == 1 ? W::vrec() : W::vrec_g();
    const int* __restrict__ vseg = VG == 1 ? W::vseg() : W::vseg_g();
    const unsigned short* __restrict__ vtgt = VG == 1 ? W::vtgt() : W::vtgt_g();
    for (int base = 0; base < nmine; base += Lay::SB) {
        const int i = first + (base + lane) * stride;
        if (lane < Lay::SB && base + lane < nmine) {
            const PrimRec<T> P = prims[B.prim_off + i / nK];
            const PrimRec<T> Q = prims[K.prim_off + i % nK];
            wide_setup_m<L, T>(P, Q, sC + lane * kNCoef, sF + lane * (L + 1));
            sC[lane * kNCoef + kZeroCoef] = T(0);
        }
        __syncwarp();
        const int nb = min(Lay::SB, nmine - base);
        if constexpr (RQ > 1) {
        // RQ primitive quartets at a time, each with its own node buffer; lane j runs record
        // j of every wave on all of them.  The accumulators add the quartets in order, so
        // the sums match the one-at-a-time form.
        for (int j0 = 0; j0 < nb; j0 += RQ) {
            const int ng = min(RQ, nb - j0);
            for (int x = lane; x < ng * (L + 1); x += 32) {
                const int q = x / (L + 1), m = x - q * (L + 1);
                node[q * NVS + m] = sF[(j0 + q) * (L + 1) + m];
            }
            __syncwarp();
            int noff = __ldg(vseg), cnt = __ldg(vseg + 1);
            for (int s = 0; s < NVSEG; ++s) {
                int noff_n = 0, cnt_n = 0;
                if (s + 1 < NVSEG) {
                    noff_n = __ldg(vseg + 4 * (s + 1));
                    cnt_n = __ldg(vseg + 4 * (s + 1) + 1);
                }
                if (s > 0) __syncwarp();
                vrr_step_rq<RQ, NVS, T>(vrec, noff, cnt, ng, sC + j0 * kNCoef, node, lane);
                noff = noff_n;
                cnt = cnt_n;
            }
            __syncwarp();
#pragma unroll
            for (int k = 0; k < NACCW; ++k) {
                const int t = lane + 32 * k;
                if (t < NACC) {
                    const int v = __ldg(vtgt + t);
                    for (int q = 0; q < ng; ++q) acc[k] += node[q * NVS + v];
                }
            }
            __syncwarp();
        }
        } else if constexpr (VG == 1) {
        for (int j = 0; j < nb; ++j) {
            const T* __restrict__ c = sC + j * kNCoef;
            if (lane <= L) node[lane] = sF[j * (L + 1) + lane];
            __syncwarp();
            int noff = __ldg(vseg), cnt = __ldg(vseg + 1);
            for (int s = 0; s < NVSEG; ++s) {
                int noff_n = 0, cnt_n = 0;
                if (s + 1 < NVSEG) {                         // next step's header, early
                    noff_n = __ldg(vseg + 4 * (s + 1));
                    cnt_n = __ldg(vseg + 4 * (s + 1) + 1);
                }
                if (s > 0) __syncwarp();
                vrr_step<32, T>(vrec, noff, cnt, true, c, node, lane);
                noff = noff_n;
                cnt = cnt_n;
            }
            __syncwarp();
#pragma unroll
            for (int k = 0; k < NACCW; ++k) {
                const int t = lane + 32 * k;
                if (t < NACC) acc[k] += node[__ldg(vtgt + t)];
            }
            __syncwarp();
        }
        } else {
        // VG primitive quartets at a time: lane = (quartet g, record j of a wave of 32/VG);
        // quartet g has its own node buffer.  The accumulators add the quartets in order,
        // so the sums match the one-at-a-time form.
        constexpr int WAVE = 32 / VG;
        const int g = lane / WAVE, jw = lane - g * WAVE;
        for (int j0 = 0; j0 < nb; j0 += VG) {
            const int ng = min(VG, nb - j0);
            for (int x = lane; x < ng * (L + 1); x += 32) {
                const int gg = x / (L + 1), m = x - gg * (L + 1);
                node[gg * NVS + m] = sF[(j0 + gg) * (L + 1) + m];
            }
            __syncwarp();
            int noff = __ldg(vseg), cnt = __ldg(vseg + 1);
            for (int s = 0; s < NVSEG; ++s) {
                int noff_n = 0, cnt_n = 0;
                if (s + 1 < NVSEG) {
                    noff_n = __ldg(vseg + 4 * (s + 1));
                    cnt_n = __ldg(vseg + 4 * (s + 1) + 1);
                }
                if (s > 0) __syncwarp();
                vrr_step<WAVE, T>(vrec, noff, cnt, g < ng, sC + (j0 + g) * kNCoef,
                                  node + g * NVS, jw);
                noff = noff_n;
                cnt = cnt_n;
            }
            __syncwarp();
#pragma unroll
            for (int k = 0; k < NACCW; ++k) {
                const int t = lane + 32 * k;
                if (t < NACC) {
                    const int v = __ldg(vtgt + t);
                    for (int gg = 0; gg < ng; ++gg) acc[k] += node[gg * NVS + v];
                }
            }
            __syncwarp();
        }
        }
    }
}

// Horizontal recursion in shared memory from the contracted targets in sm[0 .. NACC); on
// return sm[0 .. HSIZE) holds the HRR buffer whose output slots are W::outslot().
template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ void wide_hrr(const PairRec& B, const PairRec& K, T* __restrict__ sm,
                                         int lane) {
    using W = WideProg<LA, LB, LC, LD>;
    T* H = sm;
    const unsigned int* __restrict__ hop = W::hop();
    const int* __restrict__ hlev = W::hlev();
    const T dv0 = T(B.ABx), dv1 = T(B.ABy), dv2 = T(B.ABz);
    const T dv3 = T(K.ABx), dv4 = T(K.ABy), dv5 = T(K.ABz);
    // Software pipelined per level like the VRR steps: an element of a level reads only
    // earlier levels' slots, and no level overwrites a slot it reads (gen_eri.py allocates
    // a level's outputs before releasing the arrays it reads last), so the operands of the
    // next element are loaded before the current one is stored.
    int e0 = __ldg(hlev), e1 = __ldg(hlev + 1);
    for (int lv = 0; lv < W::NHLEV; ++lv) {
        const int e2 = lv + 2 <= W::NHLEV ? __ldg(hlev + lv + 2) : 0;   // next level's end
        int e = e0 + lane;
        unsigned int a = 0, b = 0, na = 0, nb = 0;
        T x = T(0), y = T(0);
        if (e < e1) {
            a = __ldg(hop + 2 * e);
            b = __ldg(hop + 2 * e + 1);
            x = H[a >> 16];
            y = H[b & 0xffff];
        }
        if (e + 32 < e1) {
            na = __ldg(hop + 2 * (e + 32));
            nb = __ldg(hop + 2 * (e + 32) + 1);
        }
        for (; e < e1; e += 32) {
            const int d = b >> 16;
            const T dv = d == 0 ? dv0 : d == 1 ? dv1 : d == 2 ? dv2 : d == 3 ? dv3 : d == 4 ? dv4 : dv5;
            const T r = fma(dv, y, x);
            const int out = a & 0xffff;
            a = na;
            b = nb;
            if (e + 32 < e1) {                            // operands of the next element
                x = H[a >> 16];
                y = H[b & 0xffff];
            }
            if (e + 64 < e1) {                            // record of the one after it
                na = __ldg(hop + 2 * (e + 64));
                nb = __ldg(hop + 2 * (e + 64) + 1);
            }
            H[out] = r;
        }
        e0 = e1;
        e1 = e2;
        __syncwarp();
    }
}

// Evaluate one contracted quartet with one warp; on return sm[0 .. HSIZE) holds the HRR
// buffer whose output slots are W::outslot().
template <int LA, int LB, int LC, int LD, typename T, int VG, int RQ = 1>
__device__ __forceinline__ void wide_quartet(const PairRec& B, const PairRec& K,
                                             const PrimRec<T>* __restrict__ prims,
                                             T* __restrict__ sm, int lane) {
    constexpr int NACC = ClassGen<LA, LB, LC, LD>::NACC;
    constexpr int NACCW = (NACC + 31) / 32;
    T acc[NACCW];
#pragma unroll
    for (int k = 0; k < NACCW; ++k) acc[k] = T(0);
    wide_contract<LA, LB, LC, LD, T, VG, RQ>(B, K, prims, sm, lane, 0, 1, acc);
#pragma unroll
    for (int k = 0; k < NACCW; ++k) {
        const int t = lane + 32 * k;
        if (t < NACC) sm[t] = acc[k];
    }
    __syncwarp();
    wide_hrr<LA, LB, LC, LD, T>(B, K, sm, lane);
}

// Block write of an evaluated quartet (HRR buffer in sm).
template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ void wide_write_out(const WriteArgs& a, const WriteTask& task,
                                               const PairRec& B, const PairRec& K,
                                               T* __restrict__ sm, int lane) {
    using G = ClassGen<LA, LB, LC, LD>;
    using W = WideProg<LA, LB, LC, LD>;
    long long s[4];
    block_strides(task.code, G::NA, G::NB, G::NC, G::ND, s);
    T* sab = sm + W::HSIZE;
    T* scd = sab + G::NA * G::NB;
    for (int x = lane; x < G::NA * G::NB; x += 32)
        sab[x] = (T)(a.comp_scale[6 * B.sa + x / G::NB] * a.comp_scale[6 * B.sb + x % G::NB]);
    for (int x = lane; x < G::NC * G::ND; x += 32)
        scd[x] = (T)(a.comp_scale[6 * K.sa + x / G::ND] * a.comp_scale[6 * K.sb + x % G::ND]);
    __syncwarp();
    const T* H = sm;
    const unsigned short* __restrict__ os = W::outslot();
    double* out = a.out + task.off;
    for (int e = lane; e < G::NBLK; e += 32) {
        const int id = e % G::ND, ic = (e / G::ND) % G::NC;
        const int ib = (e / (G::ND * G::NC)) % G::NB, ia = e / (G::ND * G::NC * G::NB);
        out[ia * s[0] + ib * s[1] + ic * s[2] + id * s[3]] =
            (double)(H[__ldg(os + e)] * (sab[ia * G::NB + ib] * scd[ic * G::ND + id]));
    }
}

template <int LA, int LB, int LC, int LD, typename T, int VG, int RQ = 1>
__global__ void __launch_bounds__(32 * kWideWarps, GS_WIDE_MINB) k_wide_write(const WriteArgs a) {
    using Lay = WideLayout<LA, LB, LC, LD, T, VG, RQ>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T* sm = reinterpret_cast<T*>(smem_raw) + (size_t)warp * Lay::WARP_W;
    const int t = blockIdx.x * kWideWarps + warp;
    if (t >= a.ntask) return;
    const WriteTask task = a.tasks[t];
    const PairRec B = a.pairs[task.bra];
    const PairRec K = a.pairs[task.ket];
    wide_quartet<LA, LB, LC, LD, T, VG, RQ>(B, K, (const PrimRec<T>*)a.prims, sm, lane);
    wide_write_out<LA, LB, LC, LD, T>(a, task, B, K, sm, lane);
}

// J/K digestion of an evaluated quartet (HRR buffer in sm).
template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ void wide_jk_digest(const JKArgs& a, const int2& task,
                                               const PairRec& B, const PairRec& K,
                                               T* __restrict__ sm, int lane) {
    using G = ClassGen<LA, LB, LC, LD>;
    using W = WideProg<LA, LB, LC, LD>;
    constexpr int NA = G::NA, NB = G::NB, NC = G::NC, ND = G::ND;
    constexpr int NAB = NA * NB, NCD = NC * ND;
    int n = a.nbf;
    long long mbase = 0;
    if (a.shell_mol) {
        const int m = a.shell_mol[B.sa];
        n = a.mol_n[m];
        mbase = a.mol_base[m];
    }
    const double deg = (B.sa == B.sb ? 0.5 : 1.0) * (K.sa == K.sb ? 0.5 : 1.0) *
                       (task.x == task.y ? 0.5 : 1.0);
    T* V = sm + W::HSIZE;
    T* sab = V + G::NBLK;
    T* scd = sab + NAB;
    for (int x = lane; x < NAB; x += 32)
        sab[x] = (T)(deg * a.comp_scale[6 * B.sa + x / NB] * a.comp_scale[6 * B.sb + x % NB]);
    for (int x = lane; x < NCD; x += 32)
        scd[x] = (T)(a.comp_scale[6 * K.sa + x / ND] * a.comp_scale[6 * K.sb + x % ND]);
    __syncwarp();
    const unsigned short* __restrict__ os = W::outslot();
    for (int e = lane; e < G::NBLK; e += 32) V[e] = sm[__ldg(os + e)] * (sab[e / NCD] * scd[e % NCD]);
    __syncwarp();
    const int fa = a.func_off[B.sa], fb = a.func_off[B.sb];
    const int fc = a.func_off[K.sa], fd = a.func_off[K.sb];
    if (a.j) {
        const double* P = a.pj + mbase;
        double* Jo = a.j + mbase;
        for (int ab = lane; ab < NAB; ab += 32) {
            T r = T(0);
            for (int cd = 0; cd < NCD; ++cd)
                r = fma(V[ab * NCD + cd], (T)P[(fc + cd / ND) * n + fd + cd % ND], r);
            atomicAdd(Jo + (fa + ab / NB) * n + fb + ab % NB, 2.0 * (double)r);
        }
        for (int cd = lane; cd < NCD; cd += 32) {
            T r = T(0);
            for (int ab = 0; ab < NAB; ++ab)
                r = fma(V[ab * NCD + cd], (T)P[(fa + ab / NB) * n + fb + ab % NB], r);
            atomicAdd(Jo + (fc + cd / ND) * n + fd + cd % ND, 2.0 * (double)r);
        }
    }
    for (int s = 0; s < a.nk; ++s) {
        const double* P = a.pk + (size_t)s * a.mat_stride + mbase;
        double* Ko = a.k + (size_t)s * a.mat_stride + mbase;
        // K'_ac += sum_bd v P_bd ; K'_ad += sum_bc v P_bc ; K'_bc += sum_ad v P_ad ; K'_bd += sum_ac v P_ac
        for (int x = lane; x < NA * NC; x += 32) {
            const int ia = x / NC, ic = x % NC;
            T r = T(0);
            for (int ib = 0; ib < NB; ++ib)
                for (int id = 0; id < ND; ++id)
                    r = fma(V[((ia * NB + ib) * NC + ic) * ND + id], (T)P[(fb + ib) * n + fd + id], r);
            atomicAdd(Ko + (fa + ia) * n + fc + ic, (double)r);
        }
        for (int x = lane; x < NA * ND; x += 32) {
            const int ia = x / ND, id = x % ND;
            T r = T(0);
            for (int ib = 0; ib < NB; ++ib)
                for (int ic = 0; ic < NC; ++ic)
                    r = fma(V[((ia * NB + ib) * NC + ic) * ND + id], (T)P[(fb + ib) * n + fc + ic], r);
            atomicAdd(Ko + (fa + ia) * n + fd + id, (double)r);
        }
        for (int x = lane; x < NB * NC; x += 32) {
            const int ib = x / NC, ic = x % NC;
            T r = T(0);
            for (int ia = 0; ia < NA; ++ia)
                for (int id = 0; id < ND; ++id)
                    r = fma(V[((ia * NB + ib) * NC + ic) * ND + id], (T)P[(fa + ia) * n + fd + id], r);
            atomicAdd(Ko + (fb + ib) * n + fc + ic, (double)r);
        }
        for (int x = lane; x < NB * ND; x += 32) {
            const int ib = x / ND, id = x % ND;
            T r = T(0);
            for (int ia = 0; ia < NA; ++ia)
                for (int ic = 0; ic < NC; ++ic)
                    r = fma(V[((ia * NB + ib) * NC + ic) * ND + id], (T)P[(fa + ia) * n + fc + ic], r);
            atomicAdd(Ko + (fb + ib) * n + fd + id, (double)r);
        }
    }
}

template <int LA, int LB, int LC, int LD, typename T, int VG, int RQ = 1>
__device__ __forceinline__ void wide_jk_task(const JKArgs& a, int t, T* __restrict__ sm, int lane) {
    const int2 task = a.tasks[t];
    const PairRec B = a.pairs[task.x];
    const PairRec K = a.pairs[task.y];
    if (!jk_keep(a, B, K)) return;                 // warp-uniform
    wide_quartet<LA, LB, LC, LD, T, VG, RQ>(B, K, (const PrimRec<T>*)a.prims, sm, lane);
    wide_jk_digest<LA, LB, LC, LD, T>(a, task, B, K, sm, lane);
}

// One warp per task; with a task count on the device (after a partition) the grid is
// capped and each warp strides over the tasks.
template <int LA, int LB, int LC, int LD, typename T, int VG, int RQ = 1>
__global__ void __launch_bounds__(32 * kWideWarps, GS_WIDE_MINB) k_wide_jk(const JKArgs a) {
    using Lay = WideLayout<LA, LB, LC, LD, T, VG, RQ>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T* sm = reinterpret_cast<T*>(smem_raw) + (size_t)warp * Lay::WARP_JK;
    const int ntask = a.ntask_dev ? *a.ntask_dev : a.ntask;
    for (int t = blockIdx.x * kWideWarps + warp; t < ntask; t += gridDim.x * kWideWarps) {
        wide_jk_task<LA, LB, LC, LD, T, VG, RQ>(a, t, sm, lane);
        __syncwarp();
    }
}

// Blocks launched for a task count that lives on the device: 16 per SM fill the GPU.
constexpr int kWideDeviceCountBlocksPerSM = 16;

template <int LA, int LB, typename T>
__global__ void __launch_bounds__(32 * kWideWarps) k_wide_schwarz(const SchwarzArgs a) {
    using G = ClassGen<LA, LB, LA, LB>;
    using W = WideProg<LA, LB, LA, LB>;
    using Lay = WideLayout<LA, LB, LA, LB, T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T* sm = reinterpret_cast<T*>(smem_raw) + (size_t)warp * Lay::WARP_W;
    const int t = blockIdx.x * kWideWarps + warp;
    if (t >= a.npair) return;
    const int p = a.pair_index[t];
    const PairRec B = a.pairs[p];
    wide_quartet<LA, LB, LA, LB, T, 1>(B, B, (const PrimRec<T>*)a.prims, sm, lane);
    const unsigned short* __restrict__ os = W::outslot();
    double m = 0.0;
    constexpr int NAB = G::NA * G::NB;
    for (int ab = lane; ab < NAB; ab += 32) {
        const double s = a.comp_scale[6 * B.sa + ab / G::NB] * a.comp_scale[6 * B.sb + ab % G::NB];
        m = fmax(m, fabs((double)sm[__ldg(os + ab * NAB + ab)]) * s * s);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) a.q[p] = sqrt(m);
}

// Cooperative form for the heavy quartets of a warp-form class: one block of several warps
// per quartet.  Each warp contracts its share of the quartet's primitive quartets into its
// own accumulators; the partial sums meet in shared memory, added in
// warp order (the result does not depend on timing), and warp 0 runs the HRR and the
// epilogue.  A class's tasks are sorted by descending primitive work, so its heavy prefix
// is a contiguous range with a host count; this form takes that range and leaves the rest
// of the segment to the one-warp form.
//
// Warp w takes primitive quartets w, w + warps, ..., so the warps' shares differ by one at
// most and none waits long at the reduction.
//
// Shared memory: warp 0 has a full one-warp region (VRR buffers, then the HRR buffer and
// the epilogue's arrays), warps 1.. only the VRR buffers (which also take their partial
// sums).  Eight warps where that fits in 227 KB, else six, four or two.
template <int LA, int LB, int LC, int LD, typename T, bool JK> struct CoopLayout {
    using Lay = WideLayout<LA, LB, LC, LD, T, 1>;
    static constexpr int NACC = ClassGen<LA, LB, LC, LD>::NACC;
    static constexpr int FIRST = JK ? Lay::WARP_JK : Lay::WARP_W;
    static constexpr int REST = Lay::VRR > NACC ? Lay::VRR : NACC;
    static constexpr bool fits(int w) {
        return (size_t)(FIRST + (size_t)(w - 1) * REST) * sizeof(T) <= 227 * 1024;
    }
    static constexpr int WARPS = fits(8) ? 8 : fits(6) ? 6 : fits(4) ? 4 : 2;
    static_assert(fits(WARPS), "cooperative block beyond 227 KB");
    static constexpr size_t BYTES = (size_t)(FIRST + (size_t)(WARPS - 1) * REST) * sizeof(T);
    __device__ static T* region(T* base, int w) {
        return w == 0 ? base : base + FIRST + (size_t)(w - 1) * REST;
    }
};
constexpr int kCoopMaxWarps = 8;

// Contract the quartet over the block's warps; true in warp 0, whose region then holds
// the HRR buffer.
template <int LA, int LB, int LC, int LD, typename T, bool JK>
__device__ __forceinline__ bool coop_quartet(const PairRec& B, const PairRec& K,
                                             const PrimRec<T>* __restrict__ prims,
                                             T* __restrict__ base, int lane, int warp) {
    using CL = CoopLayout<LA, LB, LC, LD, T, JK>;
    constexpr int NACC = CL::NACC;
    constexpr int NACCW = (NACC + 31) / 32;
    T* sm = CL::region(base, warp);
    T acc[NACCW];
#pragma unroll
    for (int k = 0; k < NACCW; ++k) acc[k] = T(0);
    wide_contract<LA, LB, LC, LD, T, 1>(B, K, prims, sm, lane, warp, CL::WARPS, acc);
#pragma unroll
    for (int k = 0; k < NACCW; ++k) {
        const int t = lane + 32 * k;
        if (t < NACC) sm[t] = acc[k];
    }
    __syncthreads();
    if (warp != 0) return false;
    for (int t = lane; t < NACC; t += 32) {
        T v = base[t];
        for (int w = 1; w < CL::WARPS; ++w) v += CL::region(base, w)[t];
        base[t] = v;
    }
    __syncwarp();
    wide_hrr<LA, LB, LC, LD, T>(B, K, base, lane);
    return true;
}

template <int LA, int LB, int LC, int LD, typename T>
__global__ void __launch_bounds__(32 * kCoopMaxWarps) k_wide_write_coop(const WriteArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T* base = reinterpret_cast<T*>(smem_raw);
    const int t = blockIdx.x;
    if (t >= a.ntask) return;                      // block-uniform
    const WriteTask task = a.tasks[t];
    const PairRec B = a.pairs[task.bra];
    const PairRec K = a.pairs[task.ket];
    if (coop_quartet<LA, LB, LC, LD, T, false>(B, K, (const PrimRec<T>*)a.prims, base, lane, warp))
        wide_write_out<LA, LB, LC, LD, T>(a, task, B, K, base, lane);
}

template <int LA, int LB, int LC, int LD, typename T>
__global__ void __launch_bounds__(32 * kCoopMaxWarps) k_wide_jk_coop(const JKArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T* base = reinterpret_cast<T*>(smem_raw);
    const int t = blockIdx.x;
    if (t >= a.ntask) return;                      // block-uniform
    const int2 task = a.tasks[t];
    const PairRec B = a.pairs[task.x];
    const PairRec K = a.pairs[task.y];
    if (!jk_keep(a, B, K)) return;                 // block-uniform
    if (coop_quartet<LA, LB, LC, LD, T, true>(B, K, (const PrimRec<T>*)a.prims, base, lane, warp))
        wide_jk_digest<LA, LB, LC, LD, T>(a, task, B, K, base, lane);
}

// Raise a kernel's dynamic shared-memory limit once (the first launch happens before any
// stream capture, so later launches inside a captured graph make no attribute call).
template <auto Kernel>
int set_smem(size_t sh) {
    static bool done = false;     // one flag per kernel instantiation
    if (done) return 0;
    if (cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh))
        return GS_ERR_CUDA;
    done = true;
    return 0;
}

template <int LA, int LB, int LC, int LD, int PREC, int VG = 1, int RQ = 1>
int launch_wide(int kind, const void* args, cudaStream_t st) {
    using T = typename std::conditional<PREC == 64, double, float>::type;
    using Lay = WideLayout<LA, LB, LC, LD, T, VG, RQ>;
    constexpr int TPB = 32 * kWideWarps;
    if (kind == GS_KIND_WRITE) {
        const WriteArgs& a = *(const WriteArgs*)args;
        if (a.ntask <= 0) return 0;
        auto k = k_wide_write<LA, LB, LC, LD, T, VG, RQ>;
        if (set_smem<k_wide_write<LA, LB, LC, LD, T, VG, RQ>>(Lay::BYTES_W)) return GS_ERR_CUDA;
        k<<<(a.ntask + kWideWarps - 1) / kWideWarps, TPB, Lay::BYTES_W, st>>>(a);
    } else if (kind == GS_KIND_JK) {
        const JKArgs& a = *(const JKArgs*)args;
        if (a.ntask <= 0) return 0;
        auto k = k_wide_jk<LA, LB, LC, LD, T, VG, RQ>;
        if (set_smem<k_wide_jk<LA, LB, LC, LD, T, VG, RQ>>(Lay::BYTES_JK)) return GS_ERR_CUDA;
        int grid = (a.ntask + kWideWarps - 1) / kWideWarps;
        if (a.ntask_dev && grid > kWideDeviceCountBlocksPerSM * sm_count())
            grid = kWideDeviceCountBlocksPerSM * sm_count();
        k<<<grid, TPB, Lay::BYTES_JK, st>>>(a);
    } else if (kind == GS_KIND_SCHWARZ) {
        if constexpr (LA == LC && LB == LD && PREC == 64 && VG == 1 && RQ == 1) {
            const SchwarzArgs& a = *(const SchwarzArgs*)args;
            if (a.npair <= 0) return 0;
            auto k = k_wide_schwarz<LA, LB, double>;
            if (set_smem<k_wide_schwarz<LA, LB, double>>(Lay::BYTES_W)) return GS_ERR_CUDA;
            k<<<(a.npair + kWideWarps - 1) / kWideWarps, TPB, Lay::BYTES_W, st>>>(a);
        } else {
            return GS_ERR_CLASS;
        }
    } else {
        return GS_ERR_ARG;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : GS_ERR_CUDA;
}

// The cooperative form (host task counts only: the heavy prefix of a class segment).
template <int LA, int LB, int LC, int LD, int PREC>
int launch_wide_coop(int kind, const void* args, cudaStream_t st) {
    using T = typename std::conditional<PREC == 64, double, float>::type;
    if (kind == GS_KIND_WRITE) {
        using CL = CoopLayout<LA, LB, LC, LD, T, false>;
        const WriteArgs& a = *(const WriteArgs*)args;
        if (a.ntask <= 0) return 0;
        if (set_smem<k_wide_write_coop<LA, LB, LC, LD, T>>(CL::BYTES)) return GS_ERR_CUDA;
        k_wide_write_coop<LA, LB, LC, LD, T><<<a.ntask, 32 * CL::WARPS, CL::BYTES, st>>>(a);
    } else if (kind == GS_KIND_JK) {
        using CL = CoopLayout<LA, LB, LC, LD, T, true>;
        const JKArgs& a = *(const JKArgs*)args;
        if (a.ntask <= 0) return 0;
        if (a.ntask_dev) return GS_ERR_ARG;
        if (set_smem<k_wide_jk_coop<LA, LB, LC, LD, T>>(CL::BYTES)) return GS_ERR_CUDA;
        k_wide_jk_coop<LA, LB, LC, LD, T><<<a.ntask, 32 * CL::WARPS, CL::BYTES, st>>>(a);
    } else {
        return GS_ERR_ARG;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : GS_ERR_CUDA;
}

}  // namespace gs
