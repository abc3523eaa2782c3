// Point-group zero screening of a dense two-electron tensor, replacing the reference's
// per-key Python test Symmetry.none_zero_integral (common/symmetry.py:18-47), which
// TwoElectronRepulsion.create_repulsion_matrix calls for every canonical key
// (matrixelements/electron_repulsion_matrix.py:30-33) before evaluating it.
//
// An element (ij|kl) vanishes when
//   * all four functions sit on one centre and the summed integral exponents are odd along
//     some axis, or
//   * some operation m maps the pair {i, j} onto itself and the pair {k, l} onto itself
//     (every function has an image) and flips the parity vector of the summed exponents.
// The test is symmetric under the 8 index permutations, so it is applied to every element
// of the dense tensor directly: one thread per element, grid-stride, zeroing in place.
#include <cuda_runtime.h>
#include "gs_args.h"

namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads)
k_symmetry_zero(int n, int nops, const int* __restrict__ table,
                const unsigned char* __restrict__ flip, const int* __restrict__ centre_id,
                const int* __restrict__ parity, double* __restrict__ tensor) {
    const long long n2 = (long long)n * n, total = n2 * n2;
    for (long long e = (long long)blockIdx.x * kThreads + threadIdx.x; e < total;
         e += (long long)gridDim.x * kThreads) {
        const long long ij = e / n2, kl = e - ij * n2;
        const int i = (int)(ij / n), j = (int)(ij - (long long)i * n);
        const int k = (int)(kl / n), l = (int)(kl - (long long)k * n);
        const int p = parity[i] ^ parity[j] ^ parity[k] ^ parity[l];
        bool zero = false;
        if (centre_id[i] == centre_id[j] && centre_id[j] == centre_id[k] &&
            centre_id[k] == centre_id[l]) {
            zero = p != 0;
        } else {
            for (int m = 0; m < nops && !zero; ++m) {
                const int a = table[i * nops + m], b = table[j * nops + m];
                const int c = table[k * nops + m], d = table[l * nops + m];
                if (a == 0 || b == 0 || c == 0 || d == 0) continue;
                const int w = abs(a) - 1, x = abs(b) - 1, y = abs(c) - 1, z = abs(d) - 1;
                const bool bra = (i == w && j == x) || (i == x && j == w);
                const bool ket = (k == y && l == z) || (k == z && l == y);
                zero = bra && ket && flip[m * 8 + p];
            }
        }
        if (zero) tensor[e] = 0.0;
    }
}

}  // namespace

extern "C" {

int gs_symmetry_zero(int n, int nops, const int* table, const unsigned char* flip,
                     const int* centre_id, const int* parity, double* tensor, void* stream) {
    if (n < 0 || nops < 0) return GS_ERR_ARG;
    if (n == 0) return GS_OK;
    if (!centre_id || !parity || !tensor || (nops > 0 && (!table || !flip))) return GS_ERR_ARG;
    const long long total = (long long)n * n * n * n;
    long long blocks = (total + kThreads - 1) / kThreads;
    const long long cap = 32LL * gs::sm_count();   // grid-stride beyond 32 blocks per SM
    if (blocks > cap) blocks = cap;
    k_symmetry_zero<<<(unsigned)blocks, kThreads, 0, (cudaStream_t)stream>>>(
        n, nops, table, flip, centre_id, parity, tensor);
    return cudaGetLastError() == cudaSuccess ? GS_OK : GS_ERR_CUDA;
}

}  // extern "C"
