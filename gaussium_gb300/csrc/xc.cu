// LDA exchange-correlation on a quadrature grid, replacing the reference's per-element
// adaptive quadrature (kohnsham/integration.py:7-61):
//   k_basis_on_grid  Basis.value / PrimitiveBasis.value (objects/basis_function.py,
//                    objects/primitive_basis_function.py:44-60) of every function at every
//                    grid point, one thread per (point, shell): the contracted radial
//                    factor sum_k coef_k exp(-alpha_k r^2) once per shell, then one product
//                    per Cartesian component (s; x,y,z; xx,yy,zz,xy,xz,yz)
//   k_lda            per point: Slater exchange (kohnsham/exchange/slater_exchange.py) and
//                    Vosko-Wilk-Nusair correlation (kohnsham/correlation/local_density.py)
//                    energy density and potential, times the quadrature weight
// The contractions around them (rho = diag(Phi P Phi^T), V = Phi^T diag(w v) Phi) are
// plain GEMMs left to the caller.
#include <cuda_runtime.h>
#include "gs_args.h"

namespace {

constexpr int kThreads = 256;
constexpr double kRhoFloor = 1e-300;

__global__ void __launch_bounds__(kThreads)
k_basis_on_grid(const double* __restrict__ centre, const int* __restrict__ l,
                const int* __restrict__ prim_off, const double* __restrict__ expo,
                const double* __restrict__ coef, const double* __restrict__ comp_scale,
                const int* __restrict__ func_off, int nshell, int nbf, long long npts,
                const double* __restrict__ pts, double* __restrict__ phi) {
    const long long total = npts * nshell;
    for (long long q = (long long)blockIdx.x * kThreads + threadIdx.x; q < total;
         q += (long long)gridDim.x * kThreads) {
        const long long g = q / nshell;
        const int s = (int)(q - g * nshell);
        const double dx = pts[3 * g] - centre[3 * s];
        const double dy = pts[3 * g + 1] - centre[3 * s + 1];
        const double dz = pts[3 * g + 2] - centre[3 * s + 2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        double rad = 0.0;
        for (int k = prim_off[s]; k < prim_off[s + 1]; ++k) rad += coef[k] * exp(-expo[k] * r2);
        const double* cs = comp_scale + 6 * s;
        double* out = phi + g * nbf + func_off[s];
        const int L = l[s];
        if (L == 0) {
            out[0] = cs[0] * rad;
        } else if (L == 1) {
            out[0] = cs[0] * dx * rad;
            out[1] = cs[1] * dy * rad;
            out[2] = cs[2] * dz * rad;
        } else {
            out[0] = cs[0] * dx * dx * rad;
            out[1] = cs[1] * dy * dy * rad;
            out[2] = cs[2] * dz * dz * rad;
            out[3] = cs[3] * dx * dy * rad;
            out[4] = cs[4] * dx * dz * rad;
            out[5] = cs[5] * dy * dz * rad;
        }
    }
}

struct LdaParams {
    double slater_alpha;       // 0: no exchange
    int vwn;                   // 0: no correlation
    double a, x0, b, c;        // VWN fit (a in Rydberg)
};

// Energy per electron and potential of the selected functionals at density rho > 0.
__device__ __forceinline__ void lda_point(double rho, const LdaParams& p, double& eps, double& v) {
    eps = 0.0;
    v = 0.0;
    const double third = 1.0 / 3.0;
    if (p.slater_alpha != 0.0) {
        const double k = p.slater_alpha * cbrt(3.0 / 3.14159265358979323846) * cbrt(rho);
        eps += -(9.0 / 8.0) * k;
        v += -(3.0 / 2.0) * k;
    }
    if (p.vwn) {
        const double a = p.a / 2.0;   // Rydberg to Hartree
        const double x = sqrt(cbrt(3.0 / (4.0 * 3.14159265358979323846 * rho)));
        const double xx = x * x + p.b * x + p.c;
        const double xx0 = p.x0 * p.x0 + p.b * p.x0 + p.c;
        const double q = sqrt(4.0 * p.c - p.b * p.b);
        const double at = atan(q / (2.0 * x + p.b));
        const double dx0 = x - p.x0;
        const double e = a * (log(x * x / xx) + (2.0 * p.b / q) * at -
                              (p.b * p.x0 / xx0) *
                                  (log(dx0 * dx0 / xx) + (2.0 * (p.b + 2.0 * p.x0) / q) * at));
        eps += e;
        v += e - (a * third) * ((p.c * dx0 - p.b * p.x0 * x) / (dx0 * xx));
    }
}

__global__ void __launch_bounds__(kThreads)
k_lda(long long npts, const double* __restrict__ rho, const double* __restrict__ w, LdaParams p,
      double* __restrict__ wv, double* __restrict__ we) {
    for (long long g = (long long)blockIdx.x * kThreads + threadIdx.x; g < npts;
         g += (long long)gridDim.x * kThreads) {
        const double r = rho[g];
        double eps = 0.0, v = 0.0;
        // zero density contributes nothing (the reference returns 0 there); so do a
        // rounding-negative density of a positive semidefinite P and a subnormal one,
        // whose Wigner-Seitz radius 3 / (4 pi rho) would overflow
        if (r > kRhoFloor) lda_point(r, p, eps, v);
        wv[g] = w[g] * v;
        we[g] = w[g] * r * eps;
    }
}

unsigned grid_for(long long work) {
    long long b = (work + kThreads - 1) / kThreads;
    const long long cap = 16LL * gs::sm_count();   // grid-stride beyond 16 blocks per SM
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

extern "C" {

int gs_basis_on_grid(const double* centre, const int* l, const int* prim_off, const double* expo,
                     const double* coef, const double* comp_scale, const int* func_off,
                     int nshell, int nbf, long long npts, const double* points, double* phi,
                     void* stream) {
    if (nshell < 0 || nbf < 0 || npts < 0) return GS_ERR_ARG;
    if (nshell == 0 || npts == 0) return GS_OK;
    if (!centre || !l || !prim_off || !expo || !coef || !comp_scale || !func_off || !points ||
        !phi)
        return GS_ERR_ARG;
    k_basis_on_grid<<<grid_for(npts * nshell), kThreads, 0, (cudaStream_t)stream>>>(
        centre, l, prim_off, expo, coef, comp_scale, func_off, nshell, nbf, npts, points, phi);
    return cudaGetLastError() == cudaSuccess ? GS_OK : GS_ERR_CUDA;
}

int gs_lda_xc(long long npts, const double* rho, const double* weights, double slater_alpha,
              int vwn, double vwn_a, double vwn_x0, double vwn_b, double vwn_c,
              double* weighted_potential, double* weighted_energy, void* stream) {
    if (npts < 0) return GS_ERR_ARG;
    if (npts == 0) return GS_OK;
    if (!rho || !weights || !weighted_potential || !weighted_energy) return GS_ERR_ARG;
    if (vwn && !(4.0 * vwn_c - vwn_b * vwn_b > 0.0)) return GS_ERR_ARG;
    LdaParams p{slater_alpha, vwn, vwn_a, vwn_x0, vwn_b, vwn_c};
    k_lda<<<grid_for(npts), kThreads, 0, (cudaStream_t)stream>>>(npts, rho, weights, p,
                                                                 weighted_potential,
                                                                 weighted_energy);
    return cudaGetLastError() == cudaSuccess ? GS_OK : GS_ERR_CUDA;
}

}  // extern "C"
