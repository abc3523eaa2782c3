// C ABI of the GB300 ERI / Fock-build engine (declared in include/gaussium_gb300.h).
// Every entry point takes device pointers the caller owns, a cudaStream_t passed as
// void*, and returns a status code (0 = success); nothing here allocates device memory.
#include <cuda_runtime.h>
#include <cstdint>
#include "eri_common.cuh"
#include "gs_args.h"
#include "gs_built_classes.h"

#define GS_DECL(A, B, C, D)                                                \
    int gs_launch_##A##B##C##D(int, int, const void*, cudaStream_t); \
    int gs_variants_##A##B##C##D(int);
GS_FOR_EACH_BUILT(GS_DECL)
#undef GS_DECL

namespace {

typedef int (*launch_fn)(int, int, const void*, cudaStream_t);

launch_fn find_class(int la, int lb, int lc, int ld) {
#define GS_FIND(A, B, C, D) \
    if (la == A && lb == B && lc == C && ld == D) return gs_launch_##A##B##C##D;
    GS_FOR_EACH_BUILT(GS_FIND)
#undef GS_FIND
    return nullptr;
}

int find_variants(int la, int lb, int lc, int ld, int prec) {
#define GS_FIND(A, B, C, D) \
    if (la == A && lb == B && lc == C && ld == D) return gs_variants_##A##B##C##D(prec);
    GS_FOR_EACH_BUILT(GS_FIND)
#undef GS_FIND
    return 0;
}

// Kernel form per class and precision chosen at run time: 0 = the built-in default by
// total angular momentum, 1 = one thread per quartet, 2 = one warp per quartet, 3 = one warp
// per quartet with several primitive quartets per VRR pass.  It rides in bits 8.. of the
// precision argument of the class launchers; 4 = the thread form's code with one warp per
// quartet over its primitive quartets (split form); 5 = the warp form's code with several
// warps per quartet (cooperative form, per call only); 6 = the warp form with several
// primitive quartets per lane (stacked form).
int g_variant[3][3][3][3][2] = {};

inline int pv(int la, int lb, int lc, int ld, int prec) {
    return prec | (g_variant[la][lb][lc][ld][prec == 64 ? 0 : 1] << 8);
}

// The precision argument of the launch entry points: 64 or 32, optionally with an explicit
// kernel form in bits 8.. (1 thread, 2 warp, 3 grouped warp, 4 split, 5 cooperative, 6
// stacked; 0 = the class's configured form).  Returns the launcher's precision-and-form word, or -1 if invalid or not built.
int decode_precision(int la, int lb, int lc, int ld, int precision) {
    const int prec = precision & 0xff, form = precision >> 8;
    if ((prec != 64 && prec != 32) || form < 0 || form > 6) return -1;
    if (form == 0) return pv(la, lb, lc, ld, prec);
    if (!(find_variants(la, lb, lc, ld, prec) & (1 << (form - 1)))) return -1;
    return prec | (form << 8);
}

inline cudaStream_t S(void* s) { return (cudaStream_t)s; }

int check_launch() { return cudaGetLastError() == cudaSuccess ? GS_OK : GS_ERR_CUDA; }

// K0: one warp per shell pair.  Lane k takes primitive pair k (k = i nb + j, then k + 32),
// a ballot ranks the kept ones so that they are written contiguously in the same order as
// the host form (make_pair), and consecutive lanes write consecutive records.
__device__ __forceinline__ void build_pair(const gs::ShellView& sv, long long pi,
                                           const int* __restrict__ pair_shells,
                                           const int* __restrict__ pair_prim_off,
                                           gs::PairRec* pairs, gs::PrimRec<double>* p64,
                                           gs::PrimRec<float>* p32, double max_exp,
                                           int* __restrict__ kept, int lane) {
    const int sa = pair_shells[2 * pi], sb = pair_shells[2 * pi + 1];
    const double* A = sv.centre + 3 * sa;
    const double* B = sv.centre + 3 * sb;
    const double ABx = A[0] - B[0], ABy = A[1] - B[1], ABz = A[2] - B[2];
    const double ab2 = ABx * ABx + ABy * ABy + ABz * ABz;
    const int a0 = sv.prim_off[sa], b0 = sv.prim_off[sb];
    const int nb = sv.prim_off[sb + 1] - b0;
    const int ntot = (sv.prim_off[sa + 1] - a0) * nb;
    const int base = pair_prim_off[pi];
    int n = 0;
    for (int k0 = 0; k0 < ntot; k0 += 32) {
        const int k = k0 + lane;
        bool keep = false;
        double a = 0.0, b = 0.0;
        int i = 0, j = 0;
        if (k < ntot) {
            i = a0 + k / nb;
            j = b0 + k % nb;
            a = sv.expo[i];
            b = sv.expo[j];
            keep = gs::prim_pair_kept(a, b, ab2, max_exp);
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep) {
            const int r = base + n + __popc(m & ((1u << lane) - 1u));
            const gs::PrimRec<double> rec = gs::prim_pair(A, B, a, b, ab2, sv.coef[i], sv.coef[j]);
            p64[r] = rec;
            if (p32) p32[r] = gs::prim_pair32(rec);
        }
        n += __popc(m);
    }
    if (lane == 0) {
        gs::PairRec pr;
        pr.ABx = ABx; pr.ABy = ABy; pr.ABz = ABz;
        pr.prim_off = base;
        pr.nprim = n;
        pr.sa = sa; pr.sb = sb;
        pr.qmax = 0.0f; pr.pad = 0;
        pairs[pi] = pr;
        if (kept) kept[pi] = n;
    }
}

__global__ void __launch_bounds__(256) k_pairs_build(gs::ShellView sv, int npairs,
                                                     const int* __restrict__ pair_shells,
                                                     const int* __restrict__ pair_prim_off,
                                                     gs::PairRec* pairs, gs::PrimRec<double>* p64,
                                                     gs::PrimRec<float>* p32, double max_exp,
                                                     int* __restrict__ kept) {
    const int lane = threadIdx.x & 31;
    const long long pi = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (pi >= npairs) return;
    build_pair(sv, pi, pair_shells, pair_prim_off, pairs, p64, p32, max_exp, kept, lane);
}

// K0 for grouped pairs.  A group is a run of consecutive shell pairs whose primitive pairs
// fit one warp together (lane l takes primitive pair k of the pair whose lanes contain l),
// or a single larger pair taken 32 candidates at a time.  A warp walks kPairGroupsPerWarp
// groups but only tests the primitive-pair screen per lane there; the kept primitive
// pairs (about a third on a K = 1-6 basis with exponents over five decades) go to a
// per-warp queue in shared memory with their record positions, and are evaluated 32 at a
// time, so the FP64 division and exponential of prim_pair run on full warps.  Records
// and counts are those of k_pairs_build (each record goes to the position its ballot
// rank fixed).
struct PairCand {
    double ab2;
    int pi, i, j, r;
};
constexpr int kPairGroupsPerWarp = 8;
constexpr int kPairWarps = 8;                  // warps per block
constexpr int kPairQueue = 64;                 // a batch of 32 plus one chunk's kept pairs

__device__ __forceinline__ void pair_eval(const gs::ShellView& sv,
                                          const int* __restrict__ pair_shells,
                                          const PairCand& c, gs::PrimRec<double>* p64,
                                          gs::PrimRec<float>* p32) {
    const double* A = sv.centre + 3 * pair_shells[2 * c.pi];
    const double* B = sv.centre + 3 * pair_shells[2 * c.pi + 1];
    const gs::PrimRec<double> rec =
        gs::prim_pair(A, B, sv.expo[c.i], sv.expo[c.j], c.ab2, sv.coef[c.i], sv.coef[c.j]);
    p64[c.r] = rec;
    if (p32) p32[c.r] = gs::prim_pair32(rec);
}

// Append this lane's candidate if kept (m = the warp's ballot of keep); a full batch of 32
// is taken off the front and evaluated.  len is warp-uniform and stays below 32 on return.
__device__ __forceinline__ void pair_push(PairCand* q, int& len, bool keep, const PairCand& c,
                                          unsigned m, int lane, const gs::ShellView& sv,
                                          const int* __restrict__ pair_shells,
                                          gs::PrimRec<double>* p64, gs::PrimRec<float>* p32) {
    if (keep) q[len + __popc(m & ((1u << lane) - 1u))] = c;
    len += __popc(m);
    __syncwarp();
    if (len >= 32) {
        const PairCand e = q[lane];
        __syncwarp();
        if (lane < len - 32) q[lane] = q[lane + 32];
        __syncwarp();
        len -= 32;
        pair_eval(sv, pair_shells, e, p64, p32);
    }
}

__global__ void __launch_bounds__(32 * kPairWarps) k_pairs_build_compact(
    gs::ShellView sv, int ngroups, const int* __restrict__ group_start,
    const int* __restrict__ pair_shells, const int* __restrict__ pair_prim_off,
    gs::PairRec* pairs, gs::PrimRec<double>* p64, gs::PrimRec<float>* p32, double max_exp,
    int* __restrict__ kept) {
    __shared__ PairCand queue[kPairWarps][kPairQueue];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    PairCand* q = queue[warp];
    int len = 0;
    const long long g0 = ((long long)blockIdx.x * kPairWarps + warp) * kPairGroupsPerWarp;
    for (long long g = g0; g < g0 + kPairGroupsPerWarp && g < ngroups; ++g) {   // warp-uniform
        const int first = group_start[g], np = group_start[g + 1] - first;
        if (np == 1) {                                // one pair, chunks of 32 candidates
            const int pi = first;
            const int sa = pair_shells[2 * pi], sb = pair_shells[2 * pi + 1];
            const double* A = sv.centre + 3 * sa;
            const double* B = sv.centre + 3 * sb;
            const double ABx = A[0] - B[0], ABy = A[1] - B[1], ABz = A[2] - B[2];
            const double ab2 = ABx * ABx + ABy * ABy + ABz * ABz;
            const int a0 = sv.prim_off[sa], b0 = sv.prim_off[sb];
            const int nb = sv.prim_off[sb + 1] - b0;
            const int ntot = (sv.prim_off[sa + 1] - a0) * nb;
            const int base = pair_prim_off[pi];
            int n = 0;
            for (int k0 = 0; k0 < ntot; k0 += 32) {
                const int k = k0 + lane;
                bool keep = false;
                int i = 0, j = 0;
                if (k < ntot) {
                    i = a0 + k / nb;
                    j = b0 + k % nb;
                    keep = gs::prim_pair_kept(sv.expo[i], sv.expo[j], ab2, max_exp);
                }
                const unsigned m = __ballot_sync(0xffffffffu, keep);
                const PairCand c{ab2, pi, i, j, base + n + __popc(m & ((1u << lane) - 1u))};
                pair_push(q, len, keep, c, m, lane, sv, pair_shells, p64, p32);
                n += __popc(m);
            }
            if (lane == 0) {
                gs::PairRec pr;
                pr.ABx = ABx; pr.ABy = ABy; pr.ABz = ABz;
                pr.prim_off = base;
                pr.nprim = n;
                pr.sa = sa; pr.sb = sb;
                pr.qmax = 0.0f; pr.pad = 0;
                pairs[pi] = pr;
                if (kept) kept[pi] = n;
            }
            continue;
        }
        // several pairs in one warp: lanes [off_j, off_j + size_j) belong to pair j
        int size = 0;
        if (lane < np) {
            const int sa = pair_shells[2 * (first + lane)], sb = pair_shells[2 * (first + lane) + 1];
            size = (sv.prim_off[sa + 1] - sv.prim_off[sa]) * (sv.prim_off[sb + 1] - sv.prim_off[sb]);
        }
        int off = size;                               // inclusive scan of the pair sizes
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, off, o);
            if (lane >= o) off += y;
        }
        off -= size;
        const int total = __shfl_sync(0xffffffffu, off + size, 31);
        int jp = 0;
        for (int p = 1; p < np; ++p)
            if (__shfl_sync(0xffffffffu, off, p) <= lane) jp = p;
        const int my_off = __shfl_sync(0xffffffffu, off, jp);
        const int my_size = __shfl_sync(0xffffffffu, size, jp);
        const int pi = first + jp;
        const bool in = lane < total;
        const int sa = pair_shells[2 * pi], sb = pair_shells[2 * pi + 1];
        const double* A = sv.centre + 3 * sa;
        const double* B = sv.centre + 3 * sb;
        const double ABx = A[0] - B[0], ABy = A[1] - B[1], ABz = A[2] - B[2];
        const double ab2 = ABx * ABx + ABy * ABy + ABz * ABz;
        const int a0 = sv.prim_off[sa], b0 = sv.prim_off[sb];
        const int nb = sv.prim_off[sb + 1] - b0;
        const int k = lane - my_off;
        bool keep = false;
        int i = 0, jj = 0;
        if (in) {
            i = a0 + k / nb;
            jj = b0 + k % nb;
            keep = gs::prim_pair_kept(sv.expo[i], sv.expo[jj], ab2, max_exp);
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        const unsigned pair_mask = (my_size >= 32 ? 0xffffffffu : ((1u << my_size) - 1u)) << my_off;
        const unsigned mine = m & pair_mask;
        const int base = pair_prim_off[pi];
        const PairCand c{ab2, pi, i, jj, base + __popc(mine & ((1u << lane) - 1u))};
        pair_push(q, len, keep, c, m, lane, sv, pair_shells, p64, p32);
        if (in && lane == my_off) {
            gs::PairRec pr;
            pr.ABx = ABx; pr.ABy = ABy; pr.ABz = ABz;
            pr.prim_off = base;
            pr.nprim = __popc(mine);
            pr.sa = sa; pr.sb = sb;
            pr.qmax = 0.0f; pr.pad = 0;
            pairs[pi] = pr;
            if (kept) kept[pi] = pr.nprim;
        }
    }
    if (lane < len) pair_eval(sv, pair_shells, q[lane], p64, p32);    // the last partial batch
}

__global__ void k_set_qmax(gs::PairRec* pairs, const double* __restrict__ q, int npairs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < npairs) pairs[i].qmax = (float)q[i];
}

template <int M, typename T>
__global__ void k_boys(int n, const double* __restrict__ t, double* __restrict__ F) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T f[M + 1];
    gs::boys<M, T>((T)t[i], T(1), f);
    for (int m = 0; m <= M; ++m) F[(size_t)i * (M + 1) + m] = (double)f[m];
}

// Split a class's quartet tasks by their density-weighted Schwarz estimate
//   est = qmax_bra * qmax_ket * max |P| over the quartet's six shell blocks
// into an FP64 list (est >= cut), an FP32 list (thr <= est < cut) and dropped (est < thr).
// Warp-aggregated atomics keep each warp's survivors contiguous, so the primitive-count
// order of the input survives approximately.
// Largest |P| over the six shell blocks a quartet (ab|cd) touches, from an ns x ns table.
__device__ __forceinline__ double block_dmax(const double* __restrict__ d, int ns, int a, int b,
                                             int c, int e) {
    double dm = d[a * ns + b];
    dm = fmax(dm, d[c * ns + e]);
    dm = fmax(dm, d[a * ns + c]);
    dm = fmax(dm, d[a * ns + e]);
    dm = fmax(dm, d[b * ns + c]);
    dm = fmax(dm, d[b * ns + e]);
    return dm;
}

// dmax: per (shell, shell) block of one molecule (nshell x nshell); with shell_mol, per
// molecule: either one value per molecule (mol_sbase null) or molecule m's own block table
// at dmax + mol_sbase[m] over its mol_nshell[m] shells, numbered from mol_shell0[m].
__global__ void k_partition(int ntask, const int2* __restrict__ tasks,
                            const gs::PairRec* __restrict__ pairs,
                            const double* __restrict__ dmax, int nshell,
                            const int* __restrict__ shell_mol,
                            const int* __restrict__ mol_shell0, const int* __restrict__ mol_nshell,
                            const long long* __restrict__ mol_sbase, double thr, double cut,
                            int2* __restrict__ out64, int2* __restrict__ out32,
                            int* __restrict__ counts) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int kind = 0;
    int2 task = make_int2(0, 0);
    if (t < ntask) {
        task = tasks[t];
        const gs::PairRec B = pairs[task.x];
        const gs::PairRec K = pairs[task.y];
        double dm;
        if (shell_mol && mol_sbase) {
            const int m = shell_mol[B.sa], s0 = mol_shell0[m];
            dm = block_dmax(dmax + mol_sbase[m], mol_nshell[m], B.sa - s0, B.sb - s0, K.sa - s0,
                            K.sb - s0);
        } else if (shell_mol) {
            dm = dmax[shell_mol[B.sa]];
        } else {
            dm = block_dmax(dmax, nshell, B.sa, B.sb, K.sa, K.sb);
        }
        const double est = (double)B.qmax * (double)K.qmax * dm;
        kind = est < thr ? 0 : (est >= cut ? 1 : 2);
    }
    const unsigned lane = threadIdx.x & 31;
    for (int which = 1; which <= 2; ++which) {
        const unsigned m = __ballot_sync(0xffffffffu, kind == which);
        if (!m) continue;
        int base = 0;
        const int leader = __ffs(m) - 1;
        if ((int)lane == leader) base = atomicAdd(counts + which - 1, __popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (kind == which) {
            const int pos = base + __popc(m & ((1u << lane) - 1));
            (which == 1 ? out64 : out32)[pos] = task;
        }
    }
}

// Peak-rate probe: each thread runs `iters` rounds of 8 independent FMA chains.
template <typename T>
__global__ void k_fma(int iters, int lanes, T seed, T* __restrict__ sink) {
    // eight independent accumulator chains c_k <- a c_k + b per thread (a, b per thread);
    // only the first `lanes` lanes of each warp run them
    const T a = seed + T(1e-7) * threadIdx.x, b = seed * T(0.5);
    T c0 = T(1), c1 = T(2), c2 = T(3), c3 = T(4), c4 = T(5), c5 = T(6), c6 = T(7), c7 = T(8);
    if ((int)(threadIdx.x & 31) >= lanes) iters = 0;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            c0 = fma(a, c0, b); c1 = fma(a, c1, b); c2 = fma(a, c2, b); c3 = fma(a, c3, b);
            c4 = fma(a, c4, b); c5 = fma(a, c5, b); c6 = fma(a, c6, b); c7 = fma(a, c7, b);
        }
    }
    sink[blockIdx.x * blockDim.x + threadIdx.x] = c0 + c1 + c2 + c3 + c4 + c5 + c6 + c7;
}

}  // namespace

extern "C" {

int gs_version(void) { return 1; }

const char* gs_status_string(int status) {
    switch (status) {
        case GS_OK: return "ok";
        case GS_ERR_ARG: return "invalid argument";
        case GS_ERR_CUDA: return "CUDA launch or runtime error";
        case GS_ERR_CLASS: return "angular-momentum class not built into this library";
        case GS_ERR_DEVICE: return "device-side status error";
        case GS_ERR_NOMEM: return "workspace too small";
        case GS_ERR_LIMIT:
            return "task count exceeds the fixed workspace of the no-allocation entry point "
                   "(gs_fock_jk_mixed_noalloc_max_tasks), or orbital count exceeds "
                   "gs_spin_expand_max_orbitals";
        default: return "unknown status";
    }
}

int gs_record_sizes(int* sizes) {
    if (!sizes) return GS_ERR_ARG;
    sizes[0] = (int)sizeof(gs::PairRec);
    sizes[1] = (int)sizeof(gs::PrimRec<double>);
    sizes[2] = (int)sizeof(gs::PrimRec<float>);
    sizes[3] = (int)sizeof(gs::WriteTask);
    return GS_OK;
}

int gs_class_available(int la, int lb, int lc, int ld) {
    return find_class(la, lb, lc, ld) != nullptr;
}

int gs_class_variants(int la, int lb, int lc, int ld, int precision) {
    if (!find_class(la, lb, lc, ld)) return -GS_ERR_CLASS;
    if (precision != 64 && precision != 32) return -GS_ERR_ARG;
    return find_variants(la, lb, lc, ld, precision);
}

int gs_class_form(int la, int lb, int lc, int ld, int precision) {
    launch_fn f = find_class(la, lb, lc, ld);
    if (!f) return -GS_ERR_CLASS;
    if (precision != 64 && precision != 32) return -GS_ERR_ARG;
    return f(GS_KIND_FORM, pv(la, lb, lc, ld, precision), nullptr, nullptr);
}

int gs_set_class_variant(int la, int lb, int lc, int ld, int precision, int variant) {
    if (!find_class(la, lb, lc, ld)) return GS_ERR_CLASS;
    // the cooperative form (5) takes host task counts only, so it is per call, not per class
    if ((precision != 64 && precision != 32) || variant < 0 || variant > 6 || variant == 5)
        return GS_ERR_ARG;
    if (variant && !(find_variants(la, lb, lc, ld, precision) & (1 << (variant - 1))))
        return GS_ERR_ARG;
    g_variant[la][lb][lc][ld][precision == 64 ? 0 : 1] = variant;
    return GS_OK;
}

int gs_pairs_build(const double* centre, const int* l, const int* prim_off, const double* expo,
                   const double* coef, int npairs, const int* pair_shells,
                   const int* pair_prim_off, void* pair_rec, void* prim64, void* prim32,
                   double max_exp, int* kept, int ngroups, const int* group_start,
                   void* stream) {
    if (npairs < 0 || !centre || !l || !prim_off || !expo || !coef || !pair_rec || !prim64 ||
        ngroups < 0 || (ngroups > 0 && !group_start))
        return GS_ERR_ARG;
    if (npairs == 0) return GS_OK;
    gs::ShellView sv{centre, l, prim_off, expo, coef};
    if (ngroups > 0) {
        const long long warps = ((long long)ngroups + kPairGroupsPerWarp - 1) / kPairGroupsPerWarp;
        k_pairs_build_compact<<<(unsigned)((warps + kPairWarps - 1) / kPairWarps), 32 * kPairWarps,
                                0, S(stream)>>>(
            sv, ngroups, group_start, pair_shells, pair_prim_off, (gs::PairRec*)pair_rec,
            (gs::PrimRec<double>*)prim64, (gs::PrimRec<float>*)prim32, max_exp, kept);
        return check_launch();
    }
    k_pairs_build<<<(unsigned)(((long long)npairs * 32 + 255) / 256), 256, 0, S(stream)>>>(
        sv, npairs, pair_shells, pair_prim_off, (gs::PairRec*)pair_rec,
        (gs::PrimRec<double>*)prim64, (gs::PrimRec<float>*)prim32, max_exp, kept);
    return check_launch();
}

int gs_schwarz(int la, int lb, void* pair_rec, const void* prim64, const double* comp_scale,
               int npair, const int* pair_index, double* q, int npairs_total, void* stream) {
    launch_fn f = find_class(la, lb, la, lb);
    if (!f) return GS_ERR_CLASS;
    if (npair < 0 || !pair_rec || !prim64 || !comp_scale || !q) return GS_ERR_ARG;
    gs::SchwarzArgs a{(const gs::PairRec*)pair_rec, prim64, comp_scale, pair_index, npair, q};
    int rc = f(GS_KIND_SCHWARZ, pv(la, lb, la, lb, 64), &a, S(stream));
    if (rc) return rc;
    if (npairs_total > 0)
        k_set_qmax<<<(npairs_total + 127) / 128, 128, 0, S(stream)>>>((gs::PairRec*)pair_rec, q,
                                                                       npairs_total);
    return check_launch();
}

int gs_eri_blocks(int la, int lb, int lc, int ld, int precision, const void* pair_rec,
                  const void* prim, const double* comp_scale, int ntask, const void* tasks,
                  double* out, void* stream) {
    launch_fn f = find_class(la, lb, lc, ld);
    if (!f) return GS_ERR_CLASS;
    const int pf = decode_precision(la, lb, lc, ld, precision);
    if (pf < 0 || ntask < 0 || !pair_rec || !prim || !comp_scale || !out || (ntask > 0 && !tasks))
        return GS_ERR_ARG;
    gs::WriteArgs a{(const gs::PairRec*)pair_rec, prim, comp_scale, (const gs::WriteTask*)tasks,
                    ntask, out};
    return f(GS_KIND_WRITE, pf, &a, S(stream));
}

int gs_fock_jk(int la, int lb, int lc, int ld, int precision, const void* pair_rec,
               const void* prim, const double* comp_scale, const int* func_off, int nshell,
               int nbf, int ntask, const int* tasks, const double* pj, double* j, int nk,
               const double* pk, double* k, const double* shell_dmax, double screen_thr,
               double prec_lo, double prec_hi, void* stream) {
    launch_fn f = find_class(la, lb, lc, ld);
    if (!f) return GS_ERR_CLASS;
    const int pf = decode_precision(la, lb, lc, ld, precision);
    if (pf < 0 || ntask < 0 || nbf <= 0 || nk < 0 || !pair_rec || !prim || !comp_scale ||
        !func_off || (ntask > 0 && !tasks) || (!!pj != !!j) || (nk > 0 && (!pk || !k)) ||
        (screen_thr > 0 && !shell_dmax))
        return GS_ERR_ARG;
    gs::JKArgs a;
    a.pairs = (const gs::PairRec*)pair_rec;
    a.prims = prim;
    a.comp_scale = comp_scale;
    a.func_off = func_off;
    a.tasks = (const int2*)tasks;
    a.ntask = ntask;
    a.nbf = nbf;
    a.nshell = nshell;
    a.nk = nk;
    a.pj = pj;
    a.pk = pk;
    a.j = j;
    a.k = k;
    a.shell_dmax = shell_dmax;
    a.screen_thr = screen_thr;
    a.prec_lo = prec_lo;
    a.prec_hi = prec_hi;
    a.shell_mol = nullptr;
    a.mol_base = nullptr;
    a.mol_n = nullptr;
    a.mol_dmax = nullptr;
    a.mat_stride = (long long)nbf * nbf;
    a.ntask_dev = nullptr;
    return f(GS_KIND_JK, pf, &a, S(stream));
}

int gs_fock_jk_batched(int la, int lb, int lc, int ld, int precision, const void* pair_rec,
                       const void* prim, const double* comp_scale, const int* func_off,
                       const int* shell_mol, const long long* mol_base, const int* mol_n,
                       const double* mol_dmax, long long mat_stride, int ntask, const int* tasks,
                       const double* pj, double* j, int nk, const double* pk, double* k,
                       double screen_thr, double prec_lo, double prec_hi, void* stream) {
    launch_fn f = find_class(la, lb, lc, ld);
    if (!f) return GS_ERR_CLASS;
    const int pf = decode_precision(la, lb, lc, ld, precision);
    if (pf < 0 || ntask < 0 || nk < 0 || nk > 1 || !pair_rec || !prim || !comp_scale ||
        !func_off || !shell_mol || !mol_base || !mol_n || (ntask > 0 && !tasks) ||
        (!!pj != !!j) || (nk > 0 && (!pk || !k)) || (screen_thr > 0 && !mol_dmax) ||
        mat_stride <= 0)
        return GS_ERR_ARG;
    gs::JKArgs a;
    a.pairs = (const gs::PairRec*)pair_rec;
    a.prims = prim;
    a.comp_scale = comp_scale;
    a.func_off = func_off;
    a.tasks = (const int2*)tasks;
    a.ntask = ntask;
    a.nbf = 0;
    a.nshell = 0;
    a.nk = nk;
    a.pj = pj;
    a.pk = pk;
    a.j = j;
    a.k = k;
    a.shell_dmax = nullptr;
    a.screen_thr = screen_thr;
    a.prec_lo = prec_lo;
    a.prec_hi = prec_hi;
    a.shell_mol = shell_mol;
    a.mol_base = mol_base;
    a.mol_n = mol_n;
    a.mol_dmax = mol_dmax;
    a.mat_stride = mat_stride;
    a.ntask_dev = nullptr;
    return f(GS_KIND_JK, pf, &a, S(stream));
}

// Bytes of workspace gs_fock_jk_mixed needs for ntask tasks.
long long gs_fock_jk_mixed_workspace(int ntask) {
    return 256 + 2 * (long long)(ntask > 0 ? ntask : 0) * (long long)sizeof(int2);
}

namespace {
int fock_jk_mixed_impl(int la, int lb, int lc, int ld, const void* pair_rec, const void* prim64,
                       const void* prim32, const double* comp_scale, const int* func_off,
                       int nshell, int nbf, int ntask, const int* tasks, const double* pj,
                       double* j, int nk, const double* pk, double* k,
                       const double* shell_dmax, double screen_thr, double mixed_cut,
                       void* workspace, long long ws_bytes, void* stream) {
    launch_fn f = find_class(la, lb, lc, ld);
    if (!f) return GS_ERR_CLASS;
    if (ntask < 0 || nbf <= 0 || nk < 0 || !pair_rec || !prim64 || !prim32 || !comp_scale ||
        !func_off || (ntask > 0 && !tasks) || (!!pj != !!j) || (nk > 0 && (!pk || !k)) ||
        !shell_dmax || !workspace)
        return GS_ERR_ARG;
    if (ws_bytes < gs_fock_jk_mixed_workspace(ntask)) return GS_ERR_NOMEM;
    if (ntask == 0) return GS_OK;
    int* counts = (int*)workspace;
    int2* l64 = (int2*)((char*)workspace + 256);
    int2* l32 = l64 + ntask;
    if (cudaMemsetAsync(counts, 0, 2 * sizeof(int), S(stream)) != cudaSuccess) return GS_ERR_CUDA;
    k_partition<<<(ntask + 255) / 256, 256, 0, S(stream)>>>(
        ntask, (const int2*)tasks, (const gs::PairRec*)pair_rec, shell_dmax, nshell, nullptr,
        nullptr, nullptr, nullptr, screen_thr, mixed_cut, l64, l32, counts);
    if (check_launch()) return GS_ERR_CUDA;
    gs::JKArgs a;
    a.pairs = (const gs::PairRec*)pair_rec;
    a.comp_scale = comp_scale;
    a.func_off = func_off;
    a.ntask = ntask;
    a.nbf = nbf;
    a.nshell = nshell;
    a.nk = nk;
    a.pj = pj;
    a.pk = pk;
    a.j = j;
    a.k = k;
    a.shell_dmax = nullptr;
    a.screen_thr = 0.0;
    a.prec_lo = 0.0;
    a.prec_hi = 0.0;
    a.shell_mol = nullptr;
    a.mol_base = nullptr;
    a.mol_n = nullptr;
    a.mol_dmax = nullptr;
    a.mat_stride = (long long)nbf * nbf;
    a.prims = prim64;
    a.tasks = l64;
    a.ntask_dev = counts;
    int rc = f(GS_KIND_JK, pv(la, lb, lc, ld, 64), &a, S(stream));
    if (rc) return rc;
    a.prims = prim32;
    a.tasks = l32;
    a.ntask_dev = counts + 1;
    return f(GS_KIND_JK, pv(la, lb, lc, ld, 32), &a, S(stream));
}
}  // namespace

int gs_fock_jk_mixed(int la, int lb, int lc, int ld, const void* pair_rec, const void* prim64,
                     const void* prim32, const double* comp_scale, const int* func_off,
                     int nshell, int nbf, int ntask, const int* tasks, const double* pj, double* j,
                     int nk, const double* pk, double* k, const double* shell_dmax,
                     double screen_thr, double mixed_cut, void* workspace, long long ws_bytes,
                     void* stream) {
    return fock_jk_mixed_impl(la, lb, lc, ld, pair_rec, prim64, prim32, comp_scale, func_off,
                              nshell, nbf, ntask, tasks, pj, j, nk, pk, k, shell_dmax, screen_thr,
                              mixed_cut, workspace, ws_bytes, stream);
}

// ---------------------------------------------------------------------- no-allocation form
// Workspace of gs_fock_jk_mixed_noalloc: a fixed array in device memory that every GPU
// loading this library holds until the process exits.  Host code only ever sees the
// array's host-side stand-in symbol, so the device address is looked up per device with
// cudaGetSymbolAddress before use.
#define GS_NOALLOC_MAX_TASKS (1 << 20)
static __device__ __align__(256) unsigned char g_noalloc_ws[256 + 2 * (size_t)GS_NOALLOC_MAX_TASKS * 8];

namespace {
// looked up on every call: a cached address would go stale when a device reset reloads
// the module
int noalloc_workspace(void** ptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_ws) != cudaSuccess || !p) return GS_ERR_CUDA;
    *ptr = p;
    return GS_OK;
}
}  // namespace

int gs_fock_jk_mixed_noalloc_max_tasks(void) { return GS_NOALLOC_MAX_TASKS; }

int gs_fock_jk_mixed_noalloc(int la, int lb, int lc, int ld, const void* pair_rec,
                             const void* prim64, const void* prim32, const double* comp_scale,
                             const int* func_off, int nshell, int nbf, int ntask, const int* tasks,
                             const double* pj, double* j, int nk, const double* pk, double* k,
                             const double* shell_dmax, double screen_thr, double mixed_cut,
                             void* stream) {
    if (ntask > GS_NOALLOC_MAX_TASKS) return GS_ERR_LIMIT;
    void* ws = nullptr;
    const int rc = noalloc_workspace(&ws);
    if (rc) return rc;
    return fock_jk_mixed_impl(la, lb, lc, ld, pair_rec, prim64, prim32, comp_scale, func_off,
                              nshell, nbf, ntask, tasks, pj, j, nk, pk, k, shell_dmax, screen_thr,
                              mixed_cut, ws, (long long)sizeof(g_noalloc_ws), stream);
}

int gs_fock_jk_batched_mixed(int la, int lb, int lc, int ld, const void* pair_rec,
                             const void* prim64, const void* prim32, const double* comp_scale,
                             const int* func_off, const int* shell_mol, const long long* mol_base,
                             const int* mol_n, const double* mol_dmax, const int* mol_shell0,
                             const int* mol_nshell, const long long* mol_sbase,
                             long long mat_stride, int ntask, const int* tasks, const double* pj,
                             double* j, int nk, const double* pk, double* k, double screen_thr,
                             double mixed_cut, void* workspace, long long ws_bytes, void* stream) {
    launch_fn f = find_class(la, lb, lc, ld);
    if (!f) return GS_ERR_CLASS;
    if (ntask < 0 || nk < 0 || nk > 1 || !pair_rec || !prim64 || !prim32 || !comp_scale ||
        !func_off || !shell_mol || !mol_base || !mol_n || !mol_dmax || (ntask > 0 && !tasks) ||
        (!!pj != !!j) || (nk > 0 && (!pk || !k)) || mat_stride <= 0 || !workspace ||
        (!!mol_sbase != !!mol_shell0) || (!!mol_sbase != !!mol_nshell))
        return GS_ERR_ARG;
    if (ws_bytes < gs_fock_jk_mixed_workspace(ntask)) return GS_ERR_NOMEM;
    if (ntask == 0) return GS_OK;
    int* counts = (int*)workspace;
    int2* l64 = (int2*)((char*)workspace + 256);
    int2* l32 = l64 + ntask;
    if (cudaMemsetAsync(counts, 0, 2 * sizeof(int), S(stream)) != cudaSuccess) return GS_ERR_CUDA;
    k_partition<<<(ntask + 255) / 256, 256, 0, S(stream)>>>(
        ntask, (const int2*)tasks, (const gs::PairRec*)pair_rec, mol_dmax, 0, shell_mol,
        mol_shell0, mol_nshell, mol_sbase, screen_thr, mixed_cut, l64, l32, counts);
    if (check_launch()) return GS_ERR_CUDA;
    gs::JKArgs a;
    a.pairs = (const gs::PairRec*)pair_rec;
    a.comp_scale = comp_scale;
    a.func_off = func_off;
    a.ntask = ntask;
    a.nbf = 0;
    a.nshell = 0;
    a.nk = nk;
    a.pj = pj;
    a.pk = pk;
    a.j = j;
    a.k = k;
    a.shell_dmax = nullptr;
    a.screen_thr = 0.0;
    a.prec_lo = 0.0;
    a.prec_hi = 0.0;
    a.shell_mol = shell_mol;
    a.mol_base = mol_base;
    a.mol_n = mol_n;
    a.mol_dmax = mol_dmax;
    a.mat_stride = mat_stride;
    a.prims = prim64;
    a.tasks = l64;
    a.ntask_dev = counts;
    int rc = f(GS_KIND_JK, pv(la, lb, lc, ld, 64), &a, S(stream));
    if (rc) return rc;
    a.prims = prim32;
    a.tasks = l32;
    a.ntask_dev = counts + 1;
    return f(GS_KIND_JK, pv(la, lb, lc, ld, 32), &a, S(stream));
}

int gs_boys_eval(int m, int precision, int n, const double* t, double* F, void* stream) {
    if (n < 0 || !t || !F || (precision != 64 && precision != 32)) return GS_ERR_ARG;
    if (n == 0) return GS_OK;
    const int g = (n + 127) / 128;
#define GS_BM(MM)                                                                   \
    case MM:                                                                        \
        if (precision == 64) k_boys<MM, double><<<g, 128, 0, S(stream)>>>(n, t, F); \
        else k_boys<MM, float><<<g, 128, 0, S(stream)>>>(n, t, F);                  \
        break;
    switch (m) {
        GS_BM(0) GS_BM(1) GS_BM(2) GS_BM(3) GS_BM(4) GS_BM(5) GS_BM(6) GS_BM(7) GS_BM(8)
        GS_BM(9) GS_BM(10)
        default: return GS_ERR_ARG;
    }
#undef GS_BM
    return check_launch();
}

int gs_fma_probe_lanes(int precision, int blocks, int threads, int iters, int lanes, void* sink,
                       void* stream) {
    if (blocks <= 0 || threads <= 0 || threads > 1024 || iters < 0 || lanes < 1 || lanes > 32 ||
        !sink)
        return GS_ERR_ARG;
    if (precision == 64)
        k_fma<double><<<blocks, threads, 0, S(stream)>>>(iters, lanes, 1.0, (double*)sink);
    else if (precision == 32)
        k_fma<float><<<blocks, threads, 0, S(stream)>>>(iters, lanes, 1.0f, (float*)sink);
    else
        return GS_ERR_ARG;
    return check_launch();
}

int gs_fma_probe(int precision, int blocks, int threads, int iters, void* sink, void* stream) {
    return gs_fma_probe_lanes(precision, blocks, threads, iters, 32, sink, stream);
}

}  // extern "C"
