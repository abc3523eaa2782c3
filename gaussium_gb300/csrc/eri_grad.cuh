// K6 fused ERI adjoint: one warp per unique shell quartet evaluates the derivative
// integrals of all three independent centres from one VRR pass per primitive quartet
// (four weighted contraction sets: 1, 2 alpha, 2 beta, 2 gamma), forms the raised and
// lowered blocks by HRR in shared memory, contracts them with the RHF density weights
//   Gamma_abcd = w (1/2 P_ab P_cd - 1/8 (P_ac P_bd + P_ad P_bc))   (w = orbit size)
// and adds dE/dR of the four centres to the per-atom gradient (D by translational
// invariance).  Programs come from gen_grad.py (GradProg<...>).
#pragma once
#include "eri_wide.cuh"

namespace gs {

template <int LA, int LB, int LC, int LD> struct GradProg;
template <int LA, int LB, int LC, int LD> struct GradThread;

struct GradArgs {
    const PairRec* pairs;
    const PrimRec<double>* prims;   // pad holds the first shell's exponent
    const double* comp_scale;
    const int* func_off;
    const int* shell_atom;
    const int2* tasks;
    int ntask;
    int nbf;
    const double* P;
    double* grad;
    int natom;
    // FP32 evaluation (thread and split forms): recursion and accumulation in FP32 from the
    // FP32 records (pad0 holds the first shell's exponent), HRR and contraction in FP64
    const PrimRec<float>* prims32;
    bool fp32;
    // density-weighted screening: a quartet is evaluated when its Schwarz bound times the
    // largest |P| of its six shell blocks (shell_dmax, nshell x nshell) is at least
    // screen_thr and lies in [prec_lo, prec_hi); screen_thr <= 0 evaluates every quartet
    const double* shell_dmax;
    int nshell;
    double screen_thr, prec_lo, prec_hi;
};

__device__ __forceinline__ bool grad_keep(const GradArgs& a, const PairRec& B, const PairRec& K) {
    if (a.screen_thr <= 0.0) return true;
    const int ns = a.nshell;
    const double* d = a.shell_dmax;
    double dm = d[B.sa * ns + B.sb];
    dm = fmax(dm, d[K.sa * ns + K.sb]);
    dm = fmax(dm, d[B.sa * ns + K.sa]);
    dm = fmax(dm, d[B.sa * ns + K.sb]);
    dm = fmax(dm, d[B.sb * ns + K.sa]);
    dm = fmax(dm, d[B.sb * ns + K.sb]);
    const double est = (double)B.qmax * (double)K.qmax * dm;
    return !(est < a.screen_thr || est < a.prec_lo || est >= a.prec_hi);
}

__device__ __forceinline__ double prim_expo(const PrimRec<double>& r) { return r.pad; }
__device__ __forceinline__ float prim_expo(const PrimRec<float>& r) { return r.pad0; }

constexpr int kGradWarps = 2;        // warps per block, unless the class's buffer is too large
constexpr int kNCoefG = 36;
// classes with more contracted accumulators than this per warp (3 per lane... 24 per lane)
// keep them in shared memory at their HRR positions instead of in registers
constexpr int kGradRegAcc = 32 * 24;

// Per-warp shared memory of one class: the VRR buffers (coefficients, Boys values, node
// slots) and, in the shared-accumulator form, the accumulators [0, NACC) ahead of them;
// the HRR reuses the whole buffer afterwards.
template <int LA, int LB, int LC, int LD> struct GradLayout {
    using W = GradProg<LA, LB, LC, LD>;
    static constexpr bool SMEM_ACC = W::NACC > kGradRegAcc;
    static constexpr int ACC = SMEM_ACC ? W::NACC : 0;
    static constexpr int SC = kSetupBatch * kNCoefG;
    static constexpr int SF = kSetupBatch * (W::L + 1);
    static constexpr int VRR = ACC + SC + SF + W::NVSLOT;
    static constexpr int WARP = VRR > W::HSIZE ? VRR : W::HSIZE;
    // two warps per block while they fit the 227 KB a block may use, else one
    static constexpr int WARPS = (size_t)WARP * sizeof(double) * kGradWarps <= 227 * 1024 ? kGradWarps : 1;
    static constexpr size_t BYTES = (size_t)WARP * sizeof(double) * WARPS;
    static_assert((size_t)WARP * sizeof(double) <= 227 * 1024, "gradient class buffer exceeds shared memory");
};

__device__ __forceinline__ int g_ncart(int l) { return (l + 1) * (l + 2) / 2; }

__device__ __forceinline__ void g_comp(int l, int k, int& x, int& y, int& z) {
    if (l == 0) { x = y = z = 0; return; }
    if (l == 1) { x = k == 0; y = k == 1; z = k == 2; return; }
    if (l == 2) {
        const int t[6][3] = {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}};
        x = t[k][0]; y = t[k][1]; z = t[k][2]; return;
    }
    int c = 0;
    for (int lx = l; lx >= 0; --lx)
        for (int ly = l - lx; ly >= 0; --ly) {
            if (c == k) { x = lx; y = ly; z = l - lx - ly; return; }
            ++c;
        }
}

__device__ __forceinline__ int g_index(int x, int y, int z) {
    const int l = x + y + z;
    if (l == 0) return 0;
    if (l == 1) return x ? 0 : (y ? 1 : 2);
    if (l == 2) {
        if (x == 2) return 0;
        if (y == 2) return 1;
        if (z == 2) return 2;
        if (x && y) return 3;
        if (x && z) return 4;
        return 5;
    }
    int c = 0;
    for (int lx = l; lx >= 0; --lx)
        for (int ly = l - lx; ly >= 0; --ly) {
            if (lx == x && ly == y) return c;
            ++c;
        }
    return -1;
}

template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(32 * kGradWarps) k_eri_grad(const GradArgs a) {
    using W = GradProg<LA, LB, LC, LD>;
    using Lay = GradLayout<LA, LB, LC, LD>;
    constexpr int L = W::L;
    constexpr bool SMEM_ACC = Lay::SMEM_ACC;
    constexpr int NACCW = SMEM_ACC ? 1 : (W::NACC + 31) / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double* sm = reinterpret_cast<double*>(smem_raw) + (size_t)warp * Lay::WARP;
    const int t = blockIdx.x * Lay::WARPS + warp;
    if (t >= a.ntask) return;
    const int2 task = a.tasks[t];
    const PairRec B = a.pairs[task.x];
    const PairRec K = a.pairs[task.y];
    if (!grad_keep(a, B, K)) return;               // warp-uniform
    double acc[NACCW];
    int accs[NACCW], acck[NACCW];
#pragma unroll
    for (int k = 0; k < NACCW; ++k) {
        acc[k] = 0.0;
        const int q = lane + 32 * k;
        const unsigned e = q < W::NACC ? __ldg(W::acc() + q) : 0u;
        accs[k] = e & 0xffff;
        acck[k] = q < W::NACC ? (int)(e >> 16) : -1;
    }
    if constexpr (SMEM_ACC) {
        // accumulators at their HRR positions H[accpos[q]], which fill [0, NACC)
        for (int q = lane; q < W::NACC; q += 32) sm[q] = 0.0;
    }
    double* sC = sm + Lay::ACC;
    double* sF = sC + Lay::SC;
    double* node = sF + Lay::SF;
    const int nK = K.nprim;
    const int ntot = B.nprim * nK;
    const uint4* __restrict__ vrec = W::vrec();
    const int* __restrict__ vseg = W::vseg();
    for (int base = 0; base < ntot; base += kSetupBatch) {
        const int i = base + lane;
        if (lane < kSetupBatch && i < ntot) {
            const PrimRec<double> P = a.prims[B.prim_off + i / nK];
            const PrimRec<double> Q = a.prims[K.prim_off + i % nK];
            double* c = sC + lane * kNCoefG;
            wide_setup_m<L, double>(P, Q, c, sF + lane * (L + 1));
            c[32] = 2.0 * P.pad;               // 2 alpha (first bra shell)
            c[33] = 2.0 * (P.p - P.pad);       // 2 beta
            c[34] = 2.0 * Q.pad;               // 2 gamma (first ket shell)
            c[35] = 5.0 * c[28];               // 5/(2(p+q)), raised (dd|..) classes
        }
        __syncwarp();
        const int nb = min(kSetupBatch, ntot - base);
        for (int j = 0; j < nb; ++j) {
            const double* __restrict__ c = sC + j * kNCoefG;
            if (lane <= L) node[lane] = sF[j * (L + 1) + lane];
            __syncwarp();
            for (int s = 0; s < W::NVSEG; ++s) {
                const int noff = __ldg(vseg + 4 * s), cnt = __ldg(vseg + 4 * s + 1);
                const int nt = __ldg(vseg + 4 * s + 2), sync = __ldg(vseg + 4 * s + 3);
                if (sync && s > 0) __syncwarp();
                int n = lane;
                uint4 ra = make_uint4(0, 0, 0, 0), rb = ra;
                if (n < cnt) {
                    ra = __ldg(vrec + 2 * (noff + n));
                    rb = __ldg(vrec + 2 * (noff + n) + 1);
                }
                for (; n < cnt; n += 32) {
                    const uint4 x = ra, y = rb;
                    if (n + 32 < cnt) {
                        ra = __ldg(vrec + 2 * (noff + n + 32));
                        rb = __ldg(vrec + 2 * (noff + n + 32) + 1);
                    }
                    double r = c[x.y >> 16] * node[x.y & 0xffff];
                    r = fma(c[x.z >> 16], node[x.z & 0xffff], r);
                    if (nt > 2) r = fma(c[x.w >> 16], node[x.w & 0xffff], r);
                    if (nt > 3) r = fma(c[y.x >> 16], node[y.x & 0xffff], r);
                    if (nt > 4) r = fma(c[y.y >> 16], node[y.y & 0xffff], r);
                    node[x.x & 0xffff] = r;
                }
            }
            __syncwarp();
            if constexpr (SMEM_ACC) {
                for (int q = lane; q < W::NACC; q += 32) {
                    const unsigned e = __ldg(W::acc() + q);
                    const int kind = (int)(e >> 16);
                    const double w = kind == 0 ? 1.0 : c[31 + kind];
                    const int pos = __ldg(W::accpos() + q);
                    sm[pos] = fma(w, node[e & 0xffff], sm[pos]);
                }
            } else {
#pragma unroll
                for (int k = 0; k < NACCW; ++k) {
                    if (acck[k] >= 0) {
                        const double w = acck[k] == 0 ? 1.0 : c[31 + acck[k]];
                        acc[k] = fma(w, node[accs[k]], acc[k]);
                    }
                }
            }
            __syncwarp();
        }
    }
    double* H = sm;
    if constexpr (!SMEM_ACC) {
#pragma unroll
        for (int k = 0; k < NACCW; ++k) {
            const int q = lane + 32 * k;
            if (q < W::NACC) H[__ldg(W::accpos() + q)] = acc[k];
        }
    }
    __syncwarp();
    const unsigned int* __restrict__ hop = W::hop();
    const int* __restrict__ hlev = W::hlev();
    const double dv0 = B.ABx, dv1 = B.ABy, dv2 = B.ABz, dv3 = K.ABx, dv4 = K.ABy, dv5 = K.ABz;
    for (int lv = 0; lv < W::NHLEV; ++lv) {
        const int e1 = __ldg(hlev + lv + 1);
        for (int e = __ldg(hlev + lv) + lane; e < e1; e += 32) {
            const unsigned int u = __ldg(hop + 2 * e), v = __ldg(hop + 2 * e + 1);
            const int d = v >> 16;
            const double dv = d == 0 ? dv0 : d == 1 ? dv1 : d == 2 ? dv2 : d == 3 ? dv3 : d == 4 ? dv4 : dv5;
            H[u & 0xffff] = fma(dv, H[v & 0xffff], H[u >> 16]);
        }
        __syncwarp();
    }
    // contraction with the density weights
    const int sh[4] = {B.sa, B.sb, K.sa, K.sb};
    const int ls[4] = {LA, LB, LC, LD};
    const int n[4] = {g_ncart(LA), g_ncart(LB), g_ncart(LC), g_ncart(LD)};
    const int fo[4] = {a.func_off[B.sa], a.func_off[B.sb], a.func_off[K.sa], a.func_off[K.sb]};
    double w = 8.0;
    if (B.sa == B.sb) w *= 0.5;
    if (K.sa == K.sb) w *= 0.5;
    if (task.x == task.y) w *= 0.5;
    const int nbf = a.nbf;
    const double* Pm = a.P;
    const unsigned short* __restrict__ out = W::out();
    double g[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) g[k] = 0.0;
    const int nblk = n[0] * n[1] * n[2] * n[3];
    for (int e = lane; e < nblk; e += 32) {
        int idx[4] = {e / (n[1] * n[2] * n[3]), (e / (n[2] * n[3])) % n[1], (e / n[3]) % n[2], e % n[3]};
        const int pa = fo[0] + idx[0], pb = fo[1] + idx[1], pc = fo[2] + idx[2], pd = fo[3] + idx[3];
        const double gam = w * (0.5 * Pm[pa * nbf + pb] * Pm[pc * nbf + pd] -
                                0.125 * (Pm[pa * nbf + pc] * Pm[pb * nbf + pd] +
                                         Pm[pa * nbf + pd] * Pm[pb * nbf + pc]));
        // the HRR blocks are unscaled: the element carries the component scales of all four
        // functions (not 1 for the xy, xz, yz components of a d shell)
        const double s = gam * a.comp_scale[6 * sh[0] + idx[0]] * a.comp_scale[6 * sh[1] + idx[1]] *
                         a.comp_scale[6 * sh[2] + idx[2]] * a.comp_scale[6 * sh[3] + idx[3]];
        for (int cen = 0; cen < 3; ++cen) {
            int ex[3];
            g_comp(ls[cen], idx[cen], ex[0], ex[1], ex[2]);
            for (int x = 0; x < 3; ++x) {
                int up[3] = {ex[0], ex[1], ex[2]};
                up[x] += 1;
                int ii[4] = {idx[0], idx[1], idx[2], idx[3]};
                int nn[4] = {n[0], n[1], n[2], n[3]};
                ii[cen] = g_index(up[0], up[1], up[2]);
                nn[cen] = g_ncart(ls[cen] + 1);
                double v = H[out[__ldg(W::out_off() + cen) + ((ii[0] * nn[1] + ii[1]) * nn[2] + ii[2]) * nn[3] + ii[3]]];
                if (ex[x] > 0) {
                    int dn[3] = {ex[0], ex[1], ex[2]};
                    dn[x] -= 1;
                    ii[cen] = g_index(dn[0], dn[1], dn[2]);
                    nn[cen] = g_ncart(ls[cen] - 1);
                    v -= ex[x] * H[out[__ldg(W::out_off() + 3 + cen) + ((ii[0] * nn[1] + ii[1]) * nn[2] + ii[2]) * nn[3] + ii[3]]];
                }
                g[3 * cen + x] = fma(s, v, g[3 * cen + x]);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 9; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) g[k] += __shfl_xor_sync(0xffffffffu, g[k], o);
    if (lane == 0) {
        for (int cen = 0; cen < 3; ++cen)
            for (int x = 0; x < 3; ++x) {
                atomicAdd(a.grad + 3 * a.shell_atom[sh[cen]] + x, g[3 * cen + x]);
                atomicAdd(a.grad + 3 * a.shell_atom[sh[3]] + x, -g[3 * cen + x]);
            }
    }
}

// Thread-per-quartet form for the small classes (generated straight-line code, csrc
// gen_grad.py emit_grad_thread): each thread runs the same VRR, accumulation, HRR and
// density contraction as the warp form for its own quartet, with node values and
// accumulators in registers.  Gradient contributions are summed per block in shared
// memory (3 natom doubles) before one global atomic per atom coordinate.
constexpr int kGradThreads = 128;
constexpr int kGradSmemAtoms = 2048;

// HRR, contraction with the RHF weights and the atomic adds of one quartet whose weighted
// contraction sets are in H[0 .. NACC).  With warp_sum, lanes of a full warp whose quartets
// share an atom at a centre sum first and one lane adds (every lane of the warp must call
// it); without, each caller adds its own (a single lane may call it).
template <int LA, int LB, int LC, int LD>
__device__ __forceinline__ void grad_finish(const GradArgs& a, const int2 task, const PairRec& B,
                                            const PairRec& K, double* H, double* dst,
                                            bool warp_sum) {
    using W = GradThread<LA, LB, LC, LD>;
    constexpr int NA = (LA + 1) * (LA + 2) / 2, NB = (LB + 1) * (LB + 2) / 2;
    constexpr int NC = (LC + 1) * (LC + 2) / 2, ND = (LD + 1) * (LD + 2) / 2;
    const double dv[6] = {B.ABx, B.ABy, B.ABz, K.ABx, K.ABy, K.ABz};
    W::hrr(H, dv);
    const int fa = a.func_off[B.sa], fb = a.func_off[B.sb];
    const int fc = a.func_off[K.sa], fd = a.func_off[K.sb];
    const int nbf = a.nbf;
    const double* Pm = a.P;
    double pab[NA * NB], pcd[NC * ND], pac[NA * NC], pbd[NB * ND], pad[NA * ND], pbc[NB * NC];
#pragma unroll
    for (int i = 0; i < NA; ++i) {
#pragma unroll
        for (int j = 0; j < NB; ++j) pab[i * NB + j] = Pm[(fa + i) * nbf + fb + j];
#pragma unroll
        for (int j = 0; j < NC; ++j) pac[i * NC + j] = Pm[(fa + i) * nbf + fc + j];
#pragma unroll
        for (int j = 0; j < ND; ++j) pad[i * ND + j] = Pm[(fa + i) * nbf + fd + j];
    }
#pragma unroll
    for (int i = 0; i < NB; ++i) {
#pragma unroll
        for (int j = 0; j < ND; ++j) pbd[i * ND + j] = Pm[(fb + i) * nbf + fd + j];
#pragma unroll
        for (int j = 0; j < NC; ++j) pbc[i * NC + j] = Pm[(fb + i) * nbf + fc + j];
    }
#pragma unroll
    for (int i = 0; i < NC; ++i)
#pragma unroll
        for (int j = 0; j < ND; ++j) pcd[i * ND + j] = Pm[(fc + i) * nbf + fd + j];
    double cs0[NA], cs1[NB], cs2[NC], cs3[ND];
#pragma unroll
    for (int i = 0; i < NA; ++i) cs0[i] = a.comp_scale[6 * B.sa + i];
#pragma unroll
    for (int i = 0; i < NB; ++i) cs1[i] = a.comp_scale[6 * B.sb + i];
#pragma unroll
    for (int i = 0; i < NC; ++i) cs2[i] = a.comp_scale[6 * K.sa + i];
#pragma unroll
    for (int i = 0; i < ND; ++i) cs3[i] = a.comp_scale[6 * K.sb + i];
    double w = 8.0;
    if (B.sa == B.sb) w *= 0.5;
    if (K.sa == K.sb) w *= 0.5;
    if (task.x == task.y) w *= 0.5;
    double g[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) g[k] = 0.0;
    W::contract(H, w, pab, pcd, pac, pbd, pad, pbc, cs0, cs1, cs2, cs3, g);
    const int at[4] = {a.shell_atom[B.sa], a.shell_atom[B.sb], a.shell_atom[K.sa],
                       a.shell_atom[K.sb]};
    // per-centre contributions (D by translational invariance); when the whole warp is
    // active and every lane has the same atom at a centre (neighbouring tasks usually
    // share their bra pair), the warp sums first and one lane adds
    double gc[4][3];
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        gc[0][x] = g[x];
        gc[1][x] = g[3 + x];
        gc[2][x] = g[6 + x];
        gc[3][x] = -(g[x] + g[3 + x] + g[6 + x]);
    }
    const unsigned act = warp_sum ? __activemask() : 0u;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int cen = 0; cen < 4; ++cen) {
        const bool uniform = warp_sum && act == 0xffffffffu &&
                             __all_sync(act, at[cen] == __shfl_sync(act, at[cen], 0));
        if (uniform) {
#pragma unroll
            for (int x = 0; x < 3; ++x) {
                double v = gc[cen][x];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(act, v, o);
                if (lane == 0) atomicAdd(dst + 3 * at[cen] + x, v);
            }
        } else {
#pragma unroll
            for (int x = 0; x < 3; ++x) atomicAdd(dst + 3 * at[cen] + x, gc[cen][x]);
        }
    }
}

// Weighted contraction sets of primitive quartets start, start + stride, ... of the quartet
// into H[0 .. NACC), the recursion in T.
template <int LA, int LB, int LC, int LD, typename T>
__device__ __forceinline__ void grad_accumulate(const GradArgs& a, const PairRec& B,
                                                const PairRec& K, double* H, int start,
                                                int stride) {
    using W = GradThread<LA, LB, LC, LD>;
    constexpr int L = W::L;
    const PrimRec<T>* __restrict__ prims;
    if constexpr (sizeof(T) == 8) prims = a.prims;
    else prims = a.prims32;
    T acc[W::NACC];
#pragma unroll
    for (int k = 0; k < W::NACC; ++k) acc[k] = T(0);
    const int nK = K.nprim, ntot = B.nprim * nK;
    for (int i = start; i < ntot; i += stride) {
        const PrimRec<T> P = prims[B.prim_off + i / nK];
        const PrimRec<T> Q = prims[K.prim_off + i % nK];
        T c[kNCoefG], n[W::NVSLOT];
        wide_setup_m<L, T>(P, Q, c, n);
        const T ea = prim_expo(P);
        c[32] = T(2) * ea;                  // 2 alpha (first bra shell)
        c[33] = T(2) * (P.p - ea);          // 2 beta
        c[34] = T(2) * prim_expo(Q);        // 2 gamma (first ket shell)
        c[35] = T(5) * c[28];               // 5/(2(p+q)), raised (dd|..) classes
        W::template prim<T>(c, n, acc);
    }
#pragma unroll
    for (int k = 0; k < W::NACC; ++k) H[k] = (double)acc[k];
}

template <int LA, int LB, int LC, int LD, typename T>
__global__ void __launch_bounds__(kGradThreads) k_eri_grad_thread(const GradArgs a) {
    using W = GradThread<LA, LB, LC, LD>;
    extern __shared__ double sg[];
    const bool shared_sum = a.natom > 0 && a.natom <= kGradSmemAtoms;
    if (shared_sum) {
        for (int i = threadIdx.x; i < 3 * a.natom; i += blockDim.x) sg[i] = 0.0;
        __syncthreads();
    }
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < a.ntask) {
        const int2 task = a.tasks[t];
        const PairRec B = a.pairs[task.x];
        const PairRec K = a.pairs[task.y];
        if (grad_keep(a, B, K)) {
            double H[W::HSIZE];
            grad_accumulate<LA, LB, LC, LD, T>(a, B, K, H, 0, 1);
            grad_finish<LA, LB, LC, LD>(a, task, B, K, H, shared_sum ? sg : a.grad, true);
        }
    }
    if (shared_sum) {
        __syncthreads();
        for (int i = threadIdx.x; i < 3 * a.natom; i += blockDim.x)
            if (sg[i] != 0.0) atomicAdd(a.grad + i, sg[i]);
    }
}

template <int LA, int LB, int LC, int LD, typename T>
int launch_grad_thread_t(const GradArgs& a, cudaStream_t st) {
    const size_t sh = (a.natom > 0 && a.natom <= kGradSmemAtoms) ? 3 * sizeof(double) * a.natom : 0;
    if (set_smem<k_eri_grad_thread<LA, LB, LC, LD, T>>(3 * sizeof(double) * kGradSmemAtoms))
        return GS_ERR_CUDA;
    k_eri_grad_thread<LA, LB, LC, LD, T><<<(a.ntask + kGradThreads - 1) / kGradThreads,
                                           kGradThreads, sh, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : GS_ERR_CUDA;
}

template <int LA, int LB, int LC, int LD>
int launch_grad_thread(const GradArgs& a, cudaStream_t st) {
    if (a.ntask <= 0) return 0;
    return a.fp32 ? launch_grad_thread_t<LA, LB, LC, LD, float>(a, st)
                  : launch_grad_thread_t<LA, LB, LC, LD, double>(a, st);
}

// Split form of the thread kernel, for quartets with many primitive quartets (the heavy
// prefix of a class's task list, sorted by descending primitive work): one warp per
// quartet, its lanes taking the primitive quartets 32 apart with the same generated code,
// a butterfly sum of the weighted contraction sets, then lane 0 finishes the quartet.
constexpr int kGradSplitWarps = 4;

template <int LA, int LB, int LC, int LD, typename T>
__global__ void __launch_bounds__(32 * kGradSplitWarps) k_eri_grad_split(const GradArgs a) {
    using W = GradThread<LA, LB, LC, LD>;
    const int lane = threadIdx.x & 31;
    const int t = blockIdx.x * kGradSplitWarps + (threadIdx.x >> 5);
    if (t >= a.ntask) return;                      // warp-uniform
    const int2 task = a.tasks[t];
    const PairRec B = a.pairs[task.x];
    const PairRec K = a.pairs[task.y];
    if (!grad_keep(a, B, K)) return;               // warp-uniform
    double H[W::HSIZE];
    grad_accumulate<LA, LB, LC, LD, T>(a, B, K, H, lane, 32);
#pragma unroll
    for (int k = 0; k < W::NACC; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) H[k] += __shfl_xor_sync(0xffffffffu, H[k], o);
    if (lane == 0) grad_finish<LA, LB, LC, LD>(a, task, B, K, H, a.grad, false);
}

template <int LA, int LB, int LC, int LD>
int launch_grad_split(const GradArgs& a, cudaStream_t st) {
    if (a.ntask <= 0) return 0;
    const int grid = (a.ntask + kGradSplitWarps - 1) / kGradSplitWarps;
    if (a.fp32)
        k_eri_grad_split<LA, LB, LC, LD, float><<<grid, 32 * kGradSplitWarps, 0, st>>>(a);
    else
        k_eri_grad_split<LA, LB, LC, LD, double><<<grid, 32 * kGradSplitWarps, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : GS_ERR_CUDA;
}

template <int LA, int LB, int LC, int LD>
int launch_grad(const GradArgs& a, cudaStream_t st) {
    if (a.ntask <= 0) return 0;
    using Lay = GradLayout<LA, LB, LC, LD>;
    auto k = k_eri_grad<LA, LB, LC, LD>;
    if (set_smem<k_eri_grad<LA, LB, LC, LD>>(Lay::BYTES)) return GS_ERR_CUDA;
    k<<<(a.ntask + Lay::WARPS - 1) / Lay::WARPS, 32 * Lay::WARPS, Lay::BYTES, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : GS_ERR_CUDA;
}

}  // namespace gs
