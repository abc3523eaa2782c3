// Spin-orbital expansions of an MO-basis two-electron tensor (h spatial orbitals, n = 2h
// spin orbitals, chemists' order in, row-major h^4 doubles), replacing the reference's
// Python element loops:
//   mode 0  spin_basis_set              matrixelements/transformations.py:73-92
//           (rs|tu) = [r%2 == s%2][t%2 == u%2] (r/2 s/2 | t/2 u/2)        (spins interleaved)
//   mode 1  blocked_spin_basis_set      matrixelements/transformations.py:29-70
//           (rs|tu) = [r<h == s<h][t<h == u<h] (r%h s%h | t%h u%h)        (alpha block first)
//   mode 2  spin_basis_anti_physicist   matrixelements/transformations.py:114-136
//           <rs||tu> = [r%2 == t%2][s%2 == u%2] (r/2 t/2 | s/2 u/2)
//                    - [r%2 == u%2][s%2 == t%2] (r/2 u/2 | s/2 t/2)
// Pure data movement, bound by the n^4 doubles written: one CTA per output tile (r, s)
// stages the h x h input slab that the n x n tile of (r, s) reads in shared memory (row
// pitch odd, so the transposed reads of mode 2 hit distinct banks), then writes the tile,
// which is one contiguous run of n^2 doubles, with coalesced stores (16-byte spin pairs
// for modes 0 and 2).  Neighbouring CTAs share their input slab (r and r+1, s and s+1
// differ only in spin), so DRAM reads stay near h^4 doubles against 16 h^4 written.
#include <cuda_runtime.h>
#include "gs_args.h"

namespace {

constexpr int kThreads = 256;

__host__ __device__ __forceinline__ int row_pitch(int h) { return h | 1; }

// Stages the h x h input slab of output tile (r, s) in shared memory; returns whether any
// element of the tile reads it.  Rows of the slab are copied by whole warps (no division)
// with cp.async, so a thread's copies overlap instead of each waiting on its load.  The
// caller's __syncthreads() makes every thread's copies visible to the block.
__device__ __forceinline__ bool stage_slab(const double* __restrict__ mo, int h, int mode, int r,
                                           int s, double* slab) {
    const int pitch = row_pitch(h);
    const long long h2 = (long long)h * h, h3 = h2 * h;
    bool live;                 // does any element of this (r, s) tile read the slab?
    const double* src;         // slab element (i, j) = src[i * si + j]
    long long si;
    if (mode == 0) {
        live = (r & 1) == (s & 1);
        src = mo + (r >> 1) * h3 + (s >> 1) * h2;
        si = h;
    } else if (mode == 1) {
        live = (r < h) == (s < h);
        src = mo + (r % h) * h3 + (s % h) * h2;
        si = h;
    } else {
        live = true;           // (r/2 i | s/2 j): i over the second index, j over the fourth
        src = mo + (r >> 1) * h3 + (s >> 1) * h;
        si = h2;
    }
    if (live) {
        // asynchronous 8-byte copies straight into shared memory, all in flight at once
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (int i = warp; i < h; i += kThreads / 32)
            for (int j = lane; j < h; j += 32) {
                const unsigned dst = (unsigned)__cvta_generic_to_shared(slab + i * pitch + j);
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst),
                             "l"(src + i * si + j));
            }
        asm volatile("cp.async.commit_group;\n" ::);
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    return live;
}

// Scalar form: any mode, any 8-byte-aligned output.  One warp per output row.
__global__ void __launch_bounds__(kThreads)
k_spin_expand(const double* __restrict__ mo, int h, int mode, double* __restrict__ out) {
    extern __shared__ double slab[];
    const int n = 2 * h;
    const int r = blockIdx.x / n, s = blockIdx.x % n;
    const int pitch = row_pitch(h);
    const bool live = stage_slab(mo, h, mode, r, s, slab);
    __syncthreads();
    double* tile = out + (long long)blockIdx.x * n * n;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int t = warp; t < n; t += kThreads / 32) {
        double* row = tile + (long long)t * n;
        if (mode == 0) {
            const int tp = t & 1;
            const double* sl = slab + (t >> 1) * pitch;
            for (int u = lane; u < n; u += 32)
                row[u] = (live && (u & 1) == tp) ? sl[u >> 1] : 0.0;
        } else if (mode == 1) {
            const bool tlo = t < h;
            const double* sl = slab + (tlo ? t : t - h) * pitch;
            for (int u = lane; u < n; u += 32)
                row[u] = (live && (u < h) == tlo) ? sl[u < h ? u : u - h] : 0.0;
        } else {
            const bool direct_rt = (r & 1) == (t & 1), swap_st = (s & 1) == (t & 1);
            const int sp = s & 1, rp = r & 1;
            const double* sl = slab + (t >> 1) * pitch;   // (r/2 t/2 | s/2 u/2) = sl[u/2]
            const double* sc = slab + (t >> 1);           // (r/2 u/2 | s/2 t/2) = sc[(u/2) pitch]
            for (int u = lane; u < n; u += 32) {
                const int up = u & 1, uh = u >> 1;
                const double a = (direct_rt && up == sp) ? sl[uh] : 0.0;
                const double b = (up == rp && swap_st) ? sc[uh * pitch] : 0.0;
                row[u] = a - b;
            }
        }
    }
}

// Paired form for the interleaved modes (0 and 2) and a 16-byte-aligned output: the n x n
// tile of (r, s) is one contiguous run of 2 h^2 spin pairs (u = 2k, 2k+1), which all
// threads stride over as 16-byte stores.  Within a pair only the element whose spin
// matches can be non-zero, so each pair needs one slab read per term, and a subtraction
// only where both terms of mode 2 meet (r, s of one spin, t of that spin: 1/8 of the
// elements).  Each thread carries its (row t, pair k) position forward by the stride
// instead of dividing.
__global__ void __launch_bounds__(kThreads)
k_spin_expand_pairs(const double* __restrict__ mo, int h, int mode, double* __restrict__ out) {
    extern __shared__ double slab[];
    const int n = 2 * h;
    const int r = blockIdx.x / n, s = blockIdx.x % n;
    const int pitch = row_pitch(h);
    const bool live = stage_slab(mo, h, mode, r, s, slab);
    __syncthreads();
    // elements move as 64-bit integers: selects, zeros and sign flips stay off the FP64 pipe
    longlong2* tile = reinterpret_cast<longlong2*>(out + (long long)blockIdx.x * n * n);
    const long long* bits = reinterpret_cast<const long long*>(slab);
    constexpr long long kSign = (long long)0x8000000000000000ULL;
    const int npairs = 2 * h * h;
    const int dt = kThreads / h, dk = kThreads - dt * h;
    int t = threadIdx.x / h, k = threadIdx.x - t * h;
    const int sp = s & 1, rp = r & 1;
    for (int e = threadIdx.x; e < npairs; e += kThreads) {
        const int tp = t & 1;
        long long x, y;
        if (mode == 0) {
            const long long a = live ? bits[(t >> 1) * pitch + k] : 0;
            x = tp ? 0 : a;
            y = tp ? a : 0;
        } else if (sp == rp) {
            // direct term (r/2 t/2 | s/2 u/2) at u parity s and exchange term
            // (r/2 u/2 | s/2 t/2) at u parity r land on one element, present together
            const long long d = (tp == sp) ? __double_as_longlong(slab[(t >> 1) * pitch + k] -
                                                                  slab[(t >> 1) + k * pitch])
                                           : 0;
            x = sp ? 0 : d;
            y = sp ? d : 0;
        } else {
            // one term per element: the direct term when t has r's spin, the negated
            // exchange term when t has s's spin
            const long long a = (tp == rp) ? bits[(t >> 1) * pitch + k] : 0;
            const long long b = (tp == sp) ? (bits[(t >> 1) + k * pitch] ^ kSign) : 0;
            x = sp ? b : a;
            y = sp ? a : b;
        }
        tile[e] = make_longlong2(x, y);
        k += dk;
        t += dt;
        if (k >= h) { k -= h; ++t; }
    }
}

}  // namespace

extern "C" {

int gs_spin_expand_max_orbitals(void) {
    int dev = 0, smem = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return 0;
    int h = 1;
    while ((long long)(h + 1) * row_pitch(h + 1) * (long long)sizeof(double) <= smem) ++h;
    return h;
}

int gs_spin_expand(const double* mo, int h, int mode, double* out, void* stream) {
    if (h < 0 || mode < 0 || mode > 2 || (h > 0 && (!mo || !out))) return GS_ERR_ARG;
    if (((unsigned long long)mo & 7) || ((unsigned long long)out & 7)) return GS_ERR_ARG;
    if (h == 0) return GS_OK;
    const int hmax = gs_spin_expand_max_orbitals();
    if (h > hmax) return GS_ERR_LIMIT;
    const size_t smem = (size_t)h * row_pitch(h) * sizeof(double);
    if (cudaFuncSetAttribute(k_spin_expand, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
        return GS_ERR_CUDA;
    const bool pairs = mode != 1 && ((unsigned long long)out & 15) == 0;
    if (cudaFuncSetAttribute(k_spin_expand_pairs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
        return GS_ERR_CUDA;
    const unsigned grid = (unsigned)(4LL * h * h);
    if (pairs)
        k_spin_expand_pairs<<<grid, kThreads, smem, (cudaStream_t)stream>>>(mo, h, mode, out);
    else
        k_spin_expand<<<grid, kThreads, smem, (cudaStream_t)stream>>>(mo, h, mode, out);
    return cudaGetLastError() == cudaSuccess ? GS_OK : GS_ERR_CUDA;
}

}  // extern "C"
