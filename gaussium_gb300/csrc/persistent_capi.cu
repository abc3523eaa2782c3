// C-ABI entry of the persistent batched J/K build (csrc/persistent.cuh): one partition
// pass over the tasks of every class, then one persistent launch per precision.
#include <cuda_runtime.h>
#include "persistent.cuh"

int gs_persist_launch_64(const gs::PersistArgs& a, cudaStream_t st);
int gs_persist_launch_32(const gs::PersistArgs& a, cudaStream_t st);

namespace {

struct SegTable {
    int seg[gs::kNumClasses + 1];
};

// Largest |P| over the six shell blocks of (ab|cd), molecule m's table (shells numbered
// from mol_shell0[m]).
__device__ __forceinline__ double quartet_dmax(const double* __restrict__ d, int ns, int a, int b,
                                               int c, int e) {
    double dm = d[a * ns + b];
    dm = fmax(dm, d[c * ns + e]);
    dm = fmax(dm, d[a * ns + c]);
    dm = fmax(dm, d[a * ns + e]);
    dm = fmax(dm, d[b * ns + c]);
    dm = fmax(dm, d[b * ns + e]);
    return dm;
}

// One thread per task of any class: the class comes from the segment table, the
// density-weighted bound q_bra q_ket max|P| decides dropped / FP32 / FP64, and survivors
// are appended to their class's list at the class's own offset.  Lanes that share class
// and kind append with one atomic.
__global__ void k_partition_all(int ntask, const int2* __restrict__ tasks,
                                const gs::PairRec* __restrict__ pairs, const SegTable seg,
                                const double* __restrict__ dmax, const int* __restrict__ shell_mol,
                                const int* __restrict__ mol_shell0,
                                const int* __restrict__ mol_nshell,
                                const long long* __restrict__ mol_sbase, double thr, double cut,
                                int2* __restrict__ out64, int2* __restrict__ out32,
                                int* __restrict__ counts) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int key = -1, c = 0;
    int2 task = make_int2(0, 0);
    if (t < ntask) {
        int lo = 0, hi = gs::kNumClasses;            // largest c with seg[c] <= t
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (seg.seg[mid] <= t) lo = mid; else hi = mid;
        }
        c = lo;
        task = tasks[t];
        const gs::PairRec B = pairs[task.x];
        const gs::PairRec K = pairs[task.y];
        const int m = shell_mol[B.sa], s0 = mol_shell0[m];
        const double dm = quartet_dmax(dmax + mol_sbase[m], mol_nshell[m], B.sa - s0, B.sb - s0,
                                       K.sa - s0, K.sb - s0);
        const double est = (double)B.qmax * (double)K.qmax * dm;
        if (est >= thr) key = est >= cut ? 2 * c : 2 * c + 1;
    }
    const unsigned lane = threadIdx.x & 31;
    const unsigned same = __match_any_sync(0xffffffffu, key);
    if (key >= 0) {
        const int leader = __ffs(same) - 1;
        const int which = key & 1;                    // 0: FP64, 1: FP32
        int base = 0;
        if ((int)lane == leader) base = atomicAdd(counts + which * gs::kNumClasses + c, __popc(same));
        base = __shfl_sync(same, base, leader);
        const int pos = base + __popc(same & ((1u << lane) - 1u));
        (which ? out32 : out64)[seg.seg[c] + pos] = task;
    }
}

}  // namespace

extern "C" {

long long gs_fock_jk_persistent_workspace(int ntask) {
    return 256 + 2 * (long long)(ntask > 0 ? ntask : 0) * (long long)sizeof(int2);
}

int gs_fock_jk_batched_persistent(const void* pair_rec, const void* prim64, const void* prim32,
                                  const double* comp_scale, const int* func_off,
                                  const int* shell_mol, const long long* mol_base,
                                  const int* mol_n, const double* mol_dmax,
                                  const int* mol_shell0, const int* mol_nshell,
                                  const long long* mol_sbase, long long mat_stride,
                                  const int* class_start, int ntask, const int* tasks,
                                  const double* pj, double* j, int nk, const double* pk,
                                  double* k, double screen_thr, double mixed_cut,
                                  void* workspace, long long ws_bytes, void* stream) {
    if (ntask < 0 || nk < 0 || nk > 1 || !pair_rec || !prim64 || !prim32 || !comp_scale ||
        !func_off || !shell_mol || !mol_base || !mol_n || !mol_dmax || !mol_shell0 ||
        !mol_nshell || !mol_sbase || !class_start || (ntask > 0 && !tasks) || (!!pj != !!j) ||
        (nk > 0 && (!pk || !k)) || mat_stride <= 0 || !workspace)
        return GS_ERR_ARG;
    SegTable seg;
    for (int c = 0; c <= gs::kNumClasses; ++c) {
        seg.seg[c] = class_start[c];
        if (seg.seg[c] < 0 || seg.seg[c] > ntask || (c > 0 && seg.seg[c] < seg.seg[c - 1]))
            return GS_ERR_ARG;
    }
    if (seg.seg[0] != 0 || seg.seg[gs::kNumClasses] != ntask) return GS_ERR_ARG;
    if (ws_bytes < gs_fock_jk_persistent_workspace(ntask)) return GS_ERR_NOMEM;
    if (ntask == 0) return GS_OK;
    cudaStream_t st = (cudaStream_t)stream;
    int* counts = (int*)workspace;
    int2* l64 = (int2*)((char*)workspace + 256);
    int2* l32 = l64 + ntask;
    if (cudaMemsetAsync(counts, 0, 2 * gs::kNumClasses * sizeof(int), st) != cudaSuccess)
        return GS_ERR_CUDA;
    k_partition_all<<<(ntask + 255) / 256, 256, 0, st>>>(
        ntask, (const int2*)tasks, (const gs::PairRec*)pair_rec, seg, mol_dmax, shell_mol,
        mol_shell0, mol_nshell, mol_sbase, screen_thr > 0 ? screen_thr : 1e-300,
        mixed_cut, l64, l32, counts);
    if (cudaGetLastError() != cudaSuccess) return GS_ERR_CUDA;
    gs::PersistArgs a;
    gs::JKArgs& jk = a.jk;
    jk.pairs = (const gs::PairRec*)pair_rec;
    jk.comp_scale = comp_scale;
    jk.func_off = func_off;
    jk.ntask = ntask;
    jk.nbf = 0;
    jk.nshell = 0;
    jk.nk = nk;
    jk.pj = pj;
    jk.pk = pk;
    jk.j = j;
    jk.k = k;
    jk.shell_dmax = nullptr;
    jk.screen_thr = 0.0;            // the partition applied the screening
    jk.prec_lo = 0.0;
    jk.prec_hi = 0.0;
    jk.shell_mol = shell_mol;
    jk.mol_base = mol_base;
    jk.mol_n = mol_n;
    jk.mol_dmax = mol_dmax;
    jk.mat_stride = mat_stride;
    jk.ntask_dev = nullptr;
    for (int c = 0; c <= gs::kNumClasses; ++c) a.seg[c] = seg.seg[c];
    jk.prims = prim64;
    jk.tasks = l64;
    a.counts = counts;
    int rc = gs_persist_launch_64(a, st);
    if (rc) return rc;
    jk.prims = prim32;
    jk.tasks = l32;
    a.counts = counts + gs::kNumClasses;
    return gs_persist_launch_32(a, st);
}

}  // extern "C"
