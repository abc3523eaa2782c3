// One-electron integrals S, T, V over shell pairs (support for the core Hamiltonian).
// Replaces the reference's Python element loops:
//   orbital_overlap      integrals/orbital_overlap_integral.py:16-36  (+ OrbitalOverlapMatrix)
//   kinetic energy       matrixelements/kinetic_energy_matrix.py:16-33 via del_operator
//                        (factory/primitive_basis_factory.py:89-122): -1/2 nabla^2 on the ket
//   nuclear_attraction   integrals/nuclear_attraction_integral.py:19-57 (+ NuclearAttractionMatrix)
// Method: Obara-Saika 1D overlap recursion for S and T; for V the Obara-Saika recursion
// (e|A(0)|0)^(m) from Boys values followed by horizontal transfer to (a|A|b).
// One thread per shell pair (any order of l), all in FP64.
#include <cuda_runtime.h>
#include <climits>
#include "eri_common.cuh"
#include "gs_args.h"

namespace {

constexpr int kMaxL = 2;
__device__ __forceinline__ int ncart(int L) { return (L + 1) * (L + 2) / 2; }

__device__ __forceinline__ void cart_of(int L, int k, int& x, int& y, int& z) {
    // component k of total L in the reference order for L <= 2, lexicographic beyond
    if (L == 0) { x = y = z = 0; return; }
    if (L == 1) { x = k == 0; y = k == 1; z = k == 2; return; }
    if (L == 2) {
        const int t[6][3] = {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}};
        x = t[k][0]; y = t[k][1]; z = t[k][2]; return;
    }
    int c = 0;
    for (int lx = L; lx >= 0; --lx)
        for (int ly = L - lx; ly >= 0; --ly) {
            if (c == k) { x = lx; y = ly; z = L - lx - ly; return; }
            ++c;
        }
}

// index of (x,y,z) among all components of total L = x+y+z in cart_of order
__device__ __forceinline__ int cart_index(int x, int y, int z) {
    const int L = x + y + z;
    if (L <= 2) {
        if (L == 0) return 0;
        if (L == 1) return x ? 0 : (y ? 1 : 2);
        if (x == 2) return 0;
        if (y == 2) return 1;
        if (z == 2) return 2;
        if (x && y) return 3;
        if (x && z) return 4;
        return 5;
    }
    int c = 0;
    for (int lx = L; lx >= 0; --lx)
        for (int ly = L - lx; ly >= 0; --ly) {
            if (lx == x && ly == y) return c;
            ++c;
        }
    return -1;
}

// offset of total angular momentum L in a table over all L' < L
__device__ __forceinline__ int lbase(int L) { return L * (L + 1) * (L + 2) / 6; }

__device__ __forceinline__ int binom(int n, int k) {
    int r = 1;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

__device__ __forceinline__ double ipow(double x, int n) {
    double r = 1.0;
    for (int i = 0; i < n; ++i) r *= x;
    return r;
}

// One thread per (shell pair, part): part == natom computes S and T of the pair (plain
// stores into both (a,b) and (b,a)); part < natom adds nucleus `part`'s attraction to V
// (V zeroed first; a diagonal pair adds only to (a,b) since its loop covers both orders).
// Neighbouring threads share a pair, so a warp runs uniform primitive loops.
__global__ void k_one_electron(gs::ShellView sv, const double* __restrict__ comp_scale,
                               const int* __restrict__ func_off, int npairs,
                               const int* __restrict__ pair_shells, int nbf, int natom,
                               const double* __restrict__ atom_xyz,
                               const double* __restrict__ atom_z, double* S, double* T,
                               double* V) {
    const int parts = natom + 1;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (long long)npairs * parts) return;
    const int t = (int)(tid / parts), part = (int)(tid % parts);
    const int sa = pair_shells[2 * t], sb = pair_shells[2 * t + 1];
    const int la = sv.l[sa], lb = sv.l[sb];
    const int na = ncart(la), nb = ncart(lb);
    const double* A = sv.centre + 3 * sa;
    const double* B = sv.centre + 3 * sb;
    const double AB[3] = {A[0] - B[0], A[1] - B[1], A[2] - B[2]};
    const double ab2 = AB[0] * AB[0] + AB[1] * AB[1] + AB[2] * AB[2];
    double s_acc[36], t_acc[36], v_acc[36];
    for (int i = 0; i < 36; ++i) s_acc[i] = t_acc[i] = v_acc[i] = 0.0;
    const int L = la + lb;
    for (int i = sv.prim_off[sa]; i < sv.prim_off[sa + 1]; ++i) {
        for (int j = sv.prim_off[sb]; j < sv.prim_off[sb + 1]; ++j) {
            const double al = sv.expo[i], be = sv.expo[j];
            const double p = al + be, ip = 1.0 / p, i2p = 0.5 * ip;
            const double Kab = sv.coef[i] * sv.coef[j] * exp(-al * be * ip * ab2);
            double P[3], PA[3], PB[3];
            for (int d = 0; d < 3; ++d) {
                P[d] = (al * A[d] + be * B[d]) * ip;
                PA[d] = P[d] - A[d];
                PB[d] = P[d] - B[d];
            }
            if (part == natom) {
                // 1D overlaps s[d][ia][ib], ia <= la, ib <= lb + 2 (kinetic shift)
                double s1[3][kMaxL + 1][kMaxL + 3];
                for (int d = 0; d < 3; ++d) {
                    s1[d][0][0] = 1.0;
                    for (int b = 1; b <= lb + 2; ++b)
                        s1[d][0][b] = PB[d] * s1[d][0][b - 1] + (b > 1 ? (b - 1) * i2p * s1[d][0][b - 2] : 0.0);
                    for (int a = 1; a <= la; ++a)
                        for (int b = 0; b <= lb + 2; ++b) {
                            double v = PA[d] * s1[d][a - 1][b];
                            if (a > 1) v += (a - 1) * i2p * s1[d][a - 2][b];
                            if (b > 0) v += b * i2p * s1[d][a - 1][b - 1];
                            s1[d][a][b] = v;
                        }
                }
                const double pref = Kab * ip * sqrt(ip) * 5.568327996831708;  // pi^{3/2}
                for (int ia = 0; ia < na; ++ia) {
                    int ax, ay, az;
                    cart_of(la, ia, ax, ay, az);
                    const int a3[3] = {ax, ay, az};
                    for (int ib = 0; ib < nb; ++ib) {
                        int bx, by, bz;
                        cart_of(lb, ib, bx, by, bz);
                        const int b3[3] = {bx, by, bz};
                        double sx[3], tx[3];
                        for (int d = 0; d < 3; ++d) {
                            const int a = a3[d], b = b3[d];
                            sx[d] = s1[d][a][b];
                            // -1/2 d^2/dx^2 on x^b exp(-be x^2)
                            tx[d] = be * (2 * b + 1) * s1[d][a][b] - 2.0 * be * be * s1[d][a][b + 2] -
                                    (b >= 2 ? 0.5 * b * (b - 1) * s1[d][a][b - 2] : 0.0);
                        }
                        s_acc[ia * nb + ib] += pref * sx[0] * sx[1] * sx[2];
                        t_acc[ia * nb + ib] += pref * (tx[0] * sx[1] * sx[2] + sx[0] * tx[1] * sx[2] +
                                                       sx[0] * sx[1] * tx[2]);
                    }
                }
                continue;
            }
            // nuclear attraction of nucleus `part`: (e|A|0)^(m), e up to L, then transfer
            const double vpref = Kab * ip * 6.283185307179586;   // 2 pi / p
            const double* C = atom_xyz + 3 * part;
            const double PC[3] = {P[0] - C[0], P[1] - C[1], P[2] - C[2]};
            const double u = p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]);
            double F[2 * kMaxL + 1];
            switch (L) {
                case 0: gs::boys<0, double>(u, 1.0, F); break;
                case 1: gs::boys<1, double>(u, 1.0, F); break;
                case 2: gs::boys<2, double>(u, 1.0, F); break;
                case 3: gs::boys<3, double>(u, 1.0, F); break;
                default: gs::boys<4, double>(u, 1.0, F); break;
            }
            // th[m][lbase(Le)+k]
            double th[2 * kMaxL + 1][35];
            for (int m = 0; m <= L; ++m) th[m][0] = F[m];
            for (int Le = 1; Le <= L; ++Le)
                for (int k = 0; k < ncart(Le); ++k) {
                    int e[3];
                    cart_of(Le, k, e[0], e[1], e[2]);
                    int d = e[0] ? 0 : (e[1] ? 1 : 2);
                    int e1[3] = {e[0], e[1], e[2]};
                    e1[d] -= 1;
                    const int i1 = lbase(Le - 1) + cart_index(e1[0], e1[1], e1[2]);
                    int i2 = -1;
                    if (e1[d] > 0) {
                        int e2[3] = {e1[0], e1[1], e1[2]};
                        e2[d] -= 1;
                        i2 = lbase(Le - 2) + cart_index(e2[0], e2[1], e2[2]);
                    }
                    for (int m = 0; m <= L - Le; ++m) {
                        double v = PA[d] * th[m][i1] - PC[d] * th[m + 1][i1];
                        if (i2 >= 0) v += e1[d] * i2p * (th[m][i2] - th[m + 1][i2]);
                        th[m][lbase(Le) + k] = v;
                    }
                }
            const double zc = atom_z[part];
            for (int ia = 0; ia < na; ++ia) {
                int ax, ay, az;
                cart_of(la, ia, ax, ay, az);
                for (int ib = 0; ib < nb; ++ib) {
                    int bx, by, bz;
                    cart_of(lb, ib, bx, by, bz);
                    // (x - B)^b = sum_k C(b,k) (x - A)^k AB^(b-k) per dimension
                    double val = 0.0;
                    for (int kx = 0; kx <= bx; ++kx)
                        for (int ky = 0; ky <= by; ++ky)
                            for (int kz = 0; kz <= bz; ++kz) {
                                const double cx = (bx == 2 && kx == 1 ? 2.0 : 1.0) * pow(AB[0], bx - kx);
                                const double cy = (by == 2 && ky == 1 ? 2.0 : 1.0) * pow(AB[1], by - ky);
                                const double cz = (bz == 2 && kz == 1 ? 2.0 : 1.0) * pow(AB[2], bz - kz);
                                const int ex = ax + kx, ey = ay + ky, ez = az + kz;
                                val += cx * cy * cz * th[0][lbase(ex + ey + ez) + cart_index(ex, ey, ez)];
                            }
                    v_acc[ia * nb + ib] -= zc * vpref * val;
                }
            }
        }
    }
    const int fa = func_off[sa], fb = func_off[sb];
    for (int ia = 0; ia < na; ++ia)
        for (int ib = 0; ib < nb; ++ib) {
            const double sc = comp_scale[6 * sa + ia] * comp_scale[6 * sb + ib];
            const int r = fa + ia, q = fb + ib;
            if (part == natom) {
                S[r * nbf + q] = S[q * nbf + r] = sc * s_acc[ia * nb + ib];
                T[r * nbf + q] = T[q * nbf + r] = sc * t_acc[ia * nb + ib];
            } else {
                atomicAdd(V + r * nbf + q, sc * v_acc[ia * nb + ib]);
                if (sa != sb) atomicAdd(V + q * nbf + r, sc * v_acc[ia * nb + ib]);
            }
        }
}


// (a|V_C|b) from the (e|A_C|0) table on the m = 0 row by the binomial transfer
// (x - B)^b = sum_k C(b,k) (x - A)^k AB^(b-k); components up to the table's L.
__device__ double v_transfer(const double* th0, int ax, int ay, int az, int bx, int by, int bz,
                             const double* AB) {
    double val = 0.0;
    for (int kx = 0; kx <= bx; ++kx) {
        const double cx = (double)binom(bx, kx) * ipow(AB[0], bx - kx);
        for (int ky = 0; ky <= by; ++ky) {
            const double cy = (double)binom(by, ky) * ipow(AB[1], by - ky);
            for (int kz = 0; kz <= bz; ++kz) {
                const double cz = (double)binom(bz, kz) * ipow(AB[2], bz - kz);
                const int ex = ax + kx, ey = ay + ky, ez = az + kz;
                val += cx * cy * cz * th0[lbase(ex + ey + ez) + cart_index(ex, ey, ez)];
            }
        }
    }
    return val;
}

// One-electron part of the RHF gradient for unique shell pairs (a >= b):
//   grad += f sum_ij [P_ij (dT_ij + dV_ij) - W_ij dS_ij],  f = 2 (a != b) or 1,
// S and T by translational invariance (d/dB = -d/dA), V per nucleus C with the operator
// term d/dC = -(d/dA + d/dB).  Derivatives from raised (2 alpha, l+1) and lowered (l-1)
// Cartesian components: d phi_a/dA_x = 2 alpha phi_{a+1x} - a_x phi_{a-1x}.
// One thread per (shell pair, part): part < natom is the nuclear-attraction term of
// nucleus `part`, part == natom the overlap and kinetic terms; neighbouring threads share
// a pair, so a warp runs uniform primitive loops.
__global__ void k_one_electron_grad(gs::ShellView sv, const double* __restrict__ comp_scale,
                                    const int* __restrict__ func_off,
                                    const int* __restrict__ shell_atom, int npairs,
                                    const int* __restrict__ pair_shells, int nbf, int natom,
                                    const double* __restrict__ atom_xyz,
                                    const double* __restrict__ atom_z,
                                    const double* __restrict__ P, const double* __restrict__ Wm,
                                    double* grad) {
    const int parts = natom + 1;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (long long)npairs * parts) return;
    const int t = (int)(tid / parts), part = (int)(tid % parts);
    const int sa = pair_shells[2 * t], sb = pair_shells[2 * t + 1];
    const int atom_a = shell_atom[sa], atom_b = shell_atom[sb];
    if ((unsigned)atom_a >= (unsigned)natom || (unsigned)atom_b >= (unsigned)natom) return;
    const int la = sv.l[sa], lb = sv.l[sb];
    const int na = ncart(la), nb = ncart(lb);
    const double* A = sv.centre + 3 * sa;
    const double* B = sv.centre + 3 * sb;
    const double AB[3] = {A[0] - B[0], A[1] - B[1], A[2] - B[2]};
    const double ab2 = AB[0] * AB[0] + AB[1] * AB[1] + AB[2] * AB[2];
    const double f = sa == sb ? 1.0 : 2.0;
    const int fa = func_off[sa], fb = func_off[sb];
    double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0}, gC[3] = {0, 0, 0};
    const int L = la + lb + 1;
    for (int i = sv.prim_off[sa]; i < sv.prim_off[sa + 1]; ++i) {
        for (int j = sv.prim_off[sb]; j < sv.prim_off[sb + 1]; ++j) {
            const double al = sv.expo[i], be = sv.expo[j];
            const double p = al + be, ip = 1.0 / p, i2p = 0.5 * ip;
            const double Kab = sv.coef[i] * sv.coef[j] * exp(-al * be * ip * ab2);
            double Pc[3], PA[3], PB[3];
            for (int d = 0; d < 3; ++d) {
                Pc[d] = (al * A[d] + be * B[d]) * ip;
                PA[d] = Pc[d] - A[d];
                PB[d] = Pc[d] - B[d];
            }
            if (part == natom) {
                // 1D overlaps, a <= la+1, b <= lb+2
                double s1[3][kMaxL + 2][kMaxL + 3];
                for (int d = 0; d < 3; ++d) {
                    s1[d][0][0] = 1.0;
                    for (int b = 1; b <= lb + 2; ++b)
                        s1[d][0][b] = PB[d] * s1[d][0][b - 1] + (b > 1 ? (b - 1) * i2p * s1[d][0][b - 2] : 0.0);
                    for (int a = 1; a <= la + 1; ++a)
                        for (int b = 0; b <= lb + 2; ++b) {
                            double v = PA[d] * s1[d][a - 1][b];
                            if (a > 1) v += (a - 1) * i2p * s1[d][a - 2][b];
                            if (b > 0) v += b * i2p * s1[d][a - 1][b - 1];
                            s1[d][a][b] = v;
                        }
                }
                const double pref = Kab * ip * sqrt(ip) * 5.568327996831708;
                for (int ia = 0; ia < na; ++ia) {
                    int ax, ay, az;
                    cart_of(la, ia, ax, ay, az);
                    const int a3[3] = {ax, ay, az};
                    for (int ib = 0; ib < nb; ++ib) {
                        int bx, by, bz;
                        cart_of(lb, ib, bx, by, bz);
                        const int b3[3] = {bx, by, bz};
                        const double sc = comp_scale[6 * sa + ia] * comp_scale[6 * sb + ib] * pref * f;
                        const double Pab = P[(fa + ia) * nbf + fb + ib], Wab = Wm[(fa + ia) * nbf + fb + ib];
                        // per-dimension overlap and kinetic factors for a shifted by -1, 0, +1
                        double sx[3][3], tx[3][3];
                        for (int d = 0; d < 3; ++d)
                            for (int sft = -1; sft <= 1; ++sft) {
                                const int a = a3[d] + sft, b = b3[d];
                                if (a < 0) { sx[d][sft + 1] = tx[d][sft + 1] = 0.0; continue; }
                                sx[d][sft + 1] = s1[d][a][b];
                                tx[d][sft + 1] = be * (2 * b + 1) * s1[d][a][b] - 2.0 * be * be * s1[d][a][b + 2] -
                                                 (b >= 2 ? 0.5 * b * (b - 1) * s1[d][a][b - 2] : 0.0);
                            }
                        for (int x = 0; x < 3; ++x) {
                            const int y = (x + 1) % 3, z = (x + 2) % 3;
                            // d/dA_x of S and T
                            const double dsx = 2.0 * al * sx[x][2] - a3[x] * sx[x][0];
                            const double dtx = 2.0 * al * tx[x][2] - a3[x] * tx[x][0];
                            const double dS = dsx * sx[y][1] * sx[z][1];
                            const double dT = dtx * sx[y][1] * sx[z][1] + dsx * (tx[y][1] * sx[z][1] + sx[y][1] * tx[z][1]);
                            const double gx = sc * (Pab * dT - Wab * dS);
                            gA[x] += gx;
                            gB[x] -= gx;
                        }
                    }
                }
                continue;
            }
            // nuclear attraction of nucleus `part`
            const double vpref = Kab * ip * 6.283185307179586;
            const double* C = atom_xyz + 3 * part;
            const double PC[3] = {Pc[0] - C[0], Pc[1] - C[1], Pc[2] - C[2]};
            const double u = p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]);
            double F[2 * kMaxL + 2];
            switch (L) {
                case 1: gs::boys<1, double>(u, 1.0, F); break;
                case 2: gs::boys<2, double>(u, 1.0, F); break;
                case 3: gs::boys<3, double>(u, 1.0, F); break;
                case 4: gs::boys<4, double>(u, 1.0, F); break;
                default: gs::boys<5, double>(u, 1.0, F); break;
            }
            double th[2 * kMaxL + 2][56];
            for (int m = 0; m <= L; ++m) th[m][0] = F[m];
            for (int Le = 1; Le <= L; ++Le)
                for (int k = 0; k < ncart(Le); ++k) {
                    int e[3];
                    cart_of(Le, k, e[0], e[1], e[2]);
                    const int d = e[0] ? 0 : (e[1] ? 1 : 2);
                    int e1[3] = {e[0], e[1], e[2]};
                    e1[d] -= 1;
                    const int i1 = lbase(Le - 1) + cart_index(e1[0], e1[1], e1[2]);
                    int i2 = -1;
                    if (e1[d] > 0) {
                        int e2[3] = {e1[0], e1[1], e1[2]};
                        e2[d] -= 1;
                        i2 = lbase(Le - 2) + cart_index(e2[0], e2[1], e2[2]);
                    }
                    for (int m = 0; m <= L - Le; ++m) {
                        double v = PA[d] * th[m][i1] - PC[d] * th[m + 1][i1];
                        if (i2 >= 0) v += e1[d] * i2p * (th[m][i2] - th[m + 1][i2]);
                        th[m][lbase(Le) + k] = v;
                    }
                }
            const double zc = atom_z[part];
            for (int ia = 0; ia < na; ++ia) {
                int ax, ay, az;
                cart_of(la, ia, ax, ay, az);
                const int a3[3] = {ax, ay, az};
                for (int ib = 0; ib < nb; ++ib) {
                    int bx, by, bz;
                    cart_of(lb, ib, bx, by, bz);
                    const int b3[3] = {bx, by, bz};
                    const double w = -zc * vpref * f * comp_scale[6 * sa + ia] *
                                     comp_scale[6 * sb + ib] * P[(fa + ia) * nbf + fb + ib];
                    for (int x = 0; x < 3; ++x) {
                        int ap[3] = {a3[0], a3[1], a3[2]}, am[3] = {a3[0], a3[1], a3[2]};
                        int bp[3] = {b3[0], b3[1], b3[2]}, bm[3] = {b3[0], b3[1], b3[2]};
                        ap[x] += 1; am[x] -= 1; bp[x] += 1; bm[x] -= 1;
                        double dA = 2.0 * al * v_transfer(th[0], ap[0], ap[1], ap[2], b3[0], b3[1], b3[2], AB);
                        if (a3[x] > 0) dA -= a3[x] * v_transfer(th[0], am[0], am[1], am[2], b3[0], b3[1], b3[2], AB);
                        double dB = 2.0 * be * v_transfer(th[0], a3[0], a3[1], a3[2], bp[0], bp[1], bp[2], AB);
                        if (b3[x] > 0) dB -= b3[x] * v_transfer(th[0], a3[0], a3[1], a3[2], bm[0], bm[1], bm[2], AB);
                        gA[x] += w * dA;
                        gB[x] += w * dB;
                        gC[x] -= w * (dA + dB);
                    }
                }
            }
        }
    }
    for (int x = 0; x < 3; ++x) {
        atomicAdd(grad + 3 * atom_a + x, gA[x]);
        atomicAdd(grad + 3 * atom_b + x, gB[x]);
        if (part < natom) atomicAdd(grad + 3 * part + x, gC[x]);
    }
}

}  // namespace

extern "C" int gs_one_electron(const double* centre, const int* l, const int* prim_off,
                               const double* expo, const double* coef, const double* comp_scale,
                               const int* func_off, int npairs, const int* pair_shells, int nbf,
                               int natom, const double* atom_xyz, const double* atom_z, double* S,
                               double* T, double* V, void* stream) {
    if (npairs < 0 || nbf <= 0 || natom < 0 || !centre || !l || !prim_off || !expo || !coef ||
        !comp_scale || !func_off || !S || !T || !V || (natom > 0 && (!atom_xyz || !atom_z)))
        return GS_ERR_ARG;
    if (npairs == 0) return GS_OK;
    gs::ShellView sv{centre, l, prim_off, expo, coef};
    const long long nthr = (long long)npairs * (natom + 1);
    if (nthr > (long long)INT_MAX * 64) return GS_ERR_ARG;
    if (cudaMemsetAsync(V, 0, sizeof(double) * (size_t)nbf * nbf, (cudaStream_t)stream) != cudaSuccess)
        return GS_ERR_CUDA;
    k_one_electron<<<(unsigned)((nthr + 63) / 64), 64, 0, (cudaStream_t)stream>>>(
        sv, comp_scale, func_off, npairs, pair_shells, nbf, natom, atom_xyz, atom_z, S, T, V);
    return cudaGetLastError() == cudaSuccess ? GS_OK : GS_ERR_CUDA;
}

extern "C" int gs_one_electron_grad(const double* centre, const int* l, const int* prim_off,
                                    const double* expo, const double* coef,
                                    const double* comp_scale, const int* func_off,
                                    const int* shell_atom, int npairs, const int* pair_shells,
                                    int nbf, int natom, const double* atom_xyz,
                                    const double* atom_z, const double* density,
                                    const double* energy_weighted, double* grad, void* stream) {
    if (npairs < 0 || nbf <= 0 || natom <= 0 || !centre || !l || !prim_off || !expo || !coef ||
        !comp_scale || !func_off || !shell_atom || !atom_xyz || !atom_z || !density ||
        !energy_weighted || !grad)
        return GS_ERR_ARG;
    if (npairs == 0) return GS_OK;
    gs::ShellView sv{centre, l, prim_off, expo, coef};
    const long long nthr = (long long)npairs * (natom + 1);
    if (nthr > (long long)INT_MAX * 64) return GS_ERR_ARG;
    k_one_electron_grad<<<(unsigned)((nthr + 63) / 64), 64, 0, (cudaStream_t)stream>>>(
        sv, comp_scale, func_off, shell_atom, npairs, pair_shells, nbf, natom, atom_xyz, atom_z,
        density, energy_weighted, grad);
    return cudaGetLastError() == cudaSuccess ? GS_OK : GS_ERR_CUDA;
}
