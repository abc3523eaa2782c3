// Dense N^4 ERI tensor from the unique shell-quartet blocks: the 8-fold expansion of the
// reference's create_repulsion_matrix (matrixelements/electron_repulsion_matrix.py:43-45,
// which fills repulsion[i,j,k,l] and its seven images for every canonical key).
//
// One warp per unique shell quartet (A B | C D): its lanes stride over the block's
// n_A n_B n_C n_D elements (row-major, as the class kernels write them at offset[q]) and
// store each value at its eight index images.  Where shells repeat (A = B, C = D, or
// AB = CD) a block holds an index orbit more than once, with values equal only to
// rounding (they come from different recursion paths); there only the element with
// a >= b, c >= d and (a, b) >= (c, d) writes, so every orbit has one writer and the tensor
// has the reference's exact 8-fold symmetry.  HBM-bound: every element written once or
// more, 8 bytes each.
#include <cuda_runtime.h>
#include "gs_args.h"

namespace {

constexpr int kWarps = 8;

__device__ __forceinline__ int ncart(int l) { return (l + 1) * (l + 2) / 2; }

__global__ void __launch_bounds__(32 * kWarps)
k_dense_expand(long long nq, const int4* __restrict__ quartets,
               const long long* __restrict__ offsets, const double* __restrict__ vals,
               const int* __restrict__ l, const int* __restrict__ func_off, long long n,
               double* __restrict__ out) {
    const long long q = (long long)blockIdx.x * kWarps + (threadIdx.x >> 5);
    if (q >= nq) return;
    const int lane = threadIdx.x & 31;
    const int4 s = quartets[q];
    const int nb = ncart(l[s.y]), nc = ncart(l[s.z]), nd = ncart(l[s.w]);
    const int size = ncart(l[s.x]) * nb * nc * nd;
    const long long fa = func_off[s.x], fb = func_off[s.y], fc = func_off[s.z], fd = func_off[s.w];
    const double* v = vals + offsets[q];
    for (int e = lane; e < size; e += 32) {
        const int id = e % nd, ic = (e / nd) % nc, ib = (e / (nd * nc)) % nb, ia = e / (nd * nc * nb);
        const long long a = fa + ia, b = fb + ib, c = fc + ic, d = fd + id;
        if ((s.x == s.y && a < b) || (s.z == s.w && c < d) ||
            (s.x == s.z && s.y == s.w && (a < c || (a == c && b < d))))
            continue;                              // another element of the orbit writes
        const double x = v[e];
        out[((a * n + b) * n + c) * n + d] = x;
        out[((b * n + a) * n + c) * n + d] = x;
        out[((a * n + b) * n + d) * n + c] = x;
        out[((b * n + a) * n + d) * n + c] = x;
        out[((c * n + d) * n + a) * n + b] = x;
        out[((d * n + c) * n + a) * n + b] = x;
        out[((c * n + d) * n + b) * n + a] = x;
        out[((d * n + c) * n + b) * n + a] = x;
    }
}

}  // namespace

extern "C" {

int gs_dense_expand(long long nq, const int* quartets, const long long* offsets,
                    const double* vals, const int* l, const int* func_off, int n, double* out,
                    void* stream) {
    if (nq < 0 || n < 0) return GS_ERR_ARG;
    if (nq == 0) return GS_OK;
    if (!quartets || !offsets || !vals || !l || !func_off || !out) return GS_ERR_ARG;
    const long long blocks = (nq + kWarps - 1) / kWarps;
    if (blocks > 0x7fffffffLL) return GS_ERR_ARG;
    k_dense_expand<<<(unsigned)blocks, 32 * kWarps, 0, (cudaStream_t)stream>>>(
        nq, (const int4*)quartets, offsets, vals, l, func_off, (long long)n, out);
    return cudaGetLastError() == cudaSuccess ? GS_OK : GS_ERR_CUDA;
}

}  // extern "C"
