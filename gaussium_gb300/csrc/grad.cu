// K6 ERI adjoint: contracts derivative integrals with density-weighted quartet weights into
// nuclear-coordinate gradients.  The reference has no gradients (geometry optimisation is
// Nelder-Mead over energies, geometryoptimization/nelder_mead.py:28-144); this is new.
//
// For a unique shell quartet (A B | C D) with integrals (ab|cd):
//   d(ab|cd)/dA_x = s_a [ (a+1x b|cd)_{2alpha} - a_x (a-1x b|cd) ]
// where (a+1x ..)_{2alpha} comes from the block of the "raised" shell A+ (l+1, primitive
// coefficients times 2 alpha, unit component scales) and (a-1x ..) from the "lowered"
// shell A- (l-1), both evaluated by the ERI class kernels in the caller's (A,B,C,D) order.
// The RHF weights are Gamma_abcd = 1/2 P_ab P_cd - 1/8 (P_ac P_bd + P_ad P_bc) times the
// quartet's orbit size; D follows from translational invariance.
#include <cuda_runtime.h>
#include "gs_args.h"

namespace {

__device__ __forceinline__ int ncart(int l) { return (l + 1) * (l + 2) / 2; }

// Cartesian component k of angular momentum l, in the engine's order (reference order up
// to l = 2, lexicographic beyond)
__device__ void comp(int l, int k, int& x, int& y, int& z) {
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

__device__ int comp_index(int x, int y, int z) {
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

__global__ void k_grad_contract(int nq, const int* __restrict__ quart,
                                const long long* __restrict__ boff,
                                const double* __restrict__ blocks, const int* __restrict__ l,
                                const int* __restrict__ func_off,
                                const double* __restrict__ comp_scale,
                                const int* __restrict__ shell_atom, int nbf,
                                const double* __restrict__ P, double* grad) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int sh[4] = {quart[4 * q], quart[4 * q + 1], quart[4 * q + 2], quart[4 * q + 3]};
    int ls[4], n[4], f[4];
    for (int k = 0; k < 4; ++k) {
        ls[k] = l[sh[k]];
        n[k] = ncart(ls[k]);
        f[k] = func_off[sh[k]];
    }
    double w = 8.0;
    if (sh[0] == sh[1]) w *= 0.5;
    if (sh[2] == sh[3]) w *= 0.5;
    if (sh[0] == sh[2] && sh[1] == sh[3]) w *= 0.5;
    double g[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};   // centres A, B, C
    for (int ia = 0; ia < n[0]; ++ia)
    for (int ib = 0; ib < n[1]; ++ib)
    for (int ic = 0; ic < n[2]; ++ic)
    for (int id = 0; id < n[3]; ++id) {
        const int a = f[0] + ia, b = f[1] + ib, c = f[2] + ic, d = f[3] + id;
        const double gam = w * (0.5 * P[a * nbf + b] * P[c * nbf + d] -
                                0.125 * (P[a * nbf + c] * P[b * nbf + d] + P[a * nbf + d] * P[b * nbf + c]));
        const int idx[4] = {ia, ib, ic, id};
        for (int cen = 0; cen < 3; ++cen) {
            int e[3];
            comp(ls[cen], idx[cen], e[0], e[1], e[2]);
            const double s = comp_scale[6 * sh[cen] + idx[cen]];
            for (int x = 0; x < 3; ++x) {
                // raised block of this centre: shape n with n[cen] -> ncart(l+1)
                int up[3] = {e[0], e[1], e[2]};
                up[x] += 1;
                int ii[4] = {ia, ib, ic, id};
                int nn[4] = {n[0], n[1], n[2], n[3]};
                ii[cen] = comp_index(up[0], up[1], up[2]);
                nn[cen] = ncart(ls[cen] + 1);
                const long long o1 = boff[6 * q + 2 * cen];
                double v = blocks[o1 + ((ii[0] * nn[1] + ii[1]) * nn[2] + ii[2]) * nn[3] + ii[3]];
                if (e[x] > 0) {
                    int dn[3] = {e[0], e[1], e[2]};
                    dn[x] -= 1;
                    int jj[4] = {ia, ib, ic, id};
                    int mm[4] = {n[0], n[1], n[2], n[3]};
                    jj[cen] = comp_index(dn[0], dn[1], dn[2]);
                    mm[cen] = ncart(ls[cen] - 1);
                    const long long o2 = boff[6 * q + 2 * cen + 1];
                    v -= e[x] * blocks[o2 + ((jj[0] * mm[1] + jj[1]) * mm[2] + jj[2]) * mm[3] + jj[3]];
                }
                g[cen][x] += gam * s * v;
            }
        }
    }
    for (int cen = 0; cen < 3; ++cen)
        for (int x = 0; x < 3; ++x) {
            atomicAdd(grad + 3 * shell_atom[sh[cen]] + x, g[cen][x]);
            atomicAdd(grad + 3 * shell_atom[sh[3]] + x, -g[cen][x]);
        }
}

}  // namespace

extern "C" int gs_eri_grad_contract(int nq, const int* quartets, const long long* block_off,
                                    const double* blocks, const int* l, const int* func_off,
                                    const double* comp_scale, const int* shell_atom, int nbf,
                                    const double* density, double* grad, void* stream) {
    if (nq < 0 || nbf <= 0 || (nq > 0 && (!quartets || !block_off || !blocks || !l || !func_off ||
                                          !comp_scale || !shell_atom || !density || !grad)))
        return GS_ERR_ARG;
    if (nq == 0) return GS_OK;
    k_grad_contract<<<(nq + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
        nq, quartets, block_off, blocks, l, func_off, comp_scale, shell_atom, nbf, density, grad);
    return cudaGetLastError() == cudaSuccess ? GS_OK : GS_ERR_CUDA;
}
