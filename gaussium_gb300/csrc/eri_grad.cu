// C-ABI entry of the fused ERI adjoint (gradient) kernels, csrc/eri_grad.cuh.  Each
// gradient class is compiled in its own translation unit (written by build.py), which
// defines gs_grad_launch_<class>.
#include <cuda_runtime.h>
#include "eri_grad.cuh"
#include "eri_grad_list.h"

#define GS_GDECL(A, B, C, D) \
    int gs_grad_launch_##A##B##C##D(const gs::GradArgs&, int, cudaStream_t);
GS_FOR_EACH_GRAD(GS_GDECL)
#undef GS_GDECL

namespace {
// Kernel form per gradient class: 0 = default (thread per quartet up to total angular
// momentum 2, warp above), 1 = thread per quartet, 2 = warp per quartet.
int g_grad_variant[3][3][3][3] = {};

constexpr bool has_thread(int la, int lb, int lc, int ld) { return la + lb + lc + ld <= 3; }

bool valid_class(int la, int lb, int lc, int ld) {
#define GS_GV(A, B, C, D) \
    if (la == A && lb == B && lc == C && ld == D) return true;
    GS_FOR_EACH_GRAD(GS_GV)
#undef GS_GV
    return false;
}
}  // namespace

extern "C" int gs_eri_grad_variants(int la, int lb, int lc, int ld) {
    if (!valid_class(la, lb, lc, ld)) return -GS_ERR_CLASS;
    return (has_thread(la, lb, lc, ld) ? 1 : 0) | 2;
}

extern "C" int gs_set_eri_grad_variant(int la, int lb, int lc, int ld, int variant) {
    if (!valid_class(la, lb, lc, ld)) return GS_ERR_CLASS;
    if (variant < 0 || variant > 2 || (variant == 1 && !has_thread(la, lb, lc, ld)))
        return GS_ERR_ARG;
    g_grad_variant[la][lb][lc][ld] = variant;
    return GS_OK;
}

extern "C" int gs_eri_grad_band(int la, int lb, int lc, int ld, int form, int precision,
                                const void* pair_rec, const void* prim, const double* comp_scale,
                                const int* func_off, const int* shell_atom, int ntask,
                                const int* tasks, int nbf, int natom, const double* density,
                                int nshell, const double* shell_dmax, double screen_thr,
                                double prec_lo, double prec_hi, double* grad, void* stream) {
    if (ntask < 0 || nbf <= 0 || natom <= 0 || !pair_rec || !prim || !comp_scale || !func_off ||
        !shell_atom || (ntask > 0 && !tasks) || !density || !grad || form < 0 || form > 3 ||
        (precision != 64 && precision != 32) || (screen_thr > 0 && (!shell_dmax || nshell <= 0)))
        return GS_ERR_ARG;
    if (!valid_class(la, lb, lc, ld)) return GS_ERR_CLASS;
    if ((form == 1 || form == 3) && !has_thread(la, lb, lc, ld)) return GS_ERR_ARG;
    if (form == 0) {
        const int v = g_grad_variant[la][lb][lc][ld];
        form = has_thread(la, lb, lc, ld) && (v ? v == 1 : la + lb + lc + ld <= 2) ? 1 : 2;
    }
    if (precision == 32 && form == 2) return GS_ERR_ARG;     // the warp form is FP64 only
    gs::GradArgs a{};
    a.pairs = (const gs::PairRec*)pair_rec;
    a.prims = precision == 64 ? (const gs::PrimRec<double>*)prim : nullptr;
    a.prims32 = precision == 32 ? (const gs::PrimRec<float>*)prim : nullptr;
    a.fp32 = precision == 32;
    a.comp_scale = comp_scale;
    a.func_off = func_off;
    a.shell_atom = shell_atom;
    a.tasks = (const int2*)tasks;
    a.ntask = ntask;
    a.nbf = nbf;
    a.P = density;
    a.grad = grad;
    a.natom = natom;
    a.shell_dmax = shell_dmax;
    a.nshell = nshell;
    a.screen_thr = screen_thr;
    a.prec_lo = prec_lo;
    a.prec_hi = prec_hi;
    cudaStream_t st = (cudaStream_t)stream;
#define GS_GL(A, B, C, D) \
    if (la == A && lb == B && lc == C && ld == D) return gs_grad_launch_##A##B##C##D(a, form, st);
    GS_FOR_EACH_GRAD(GS_GL)
#undef GS_GL
    return GS_ERR_CLASS;
}

extern "C" int gs_eri_grad_form(int la, int lb, int lc, int ld, int form, const void* pair_rec,
                                const void* prim64, const double* comp_scale, const int* func_off,
                                const int* shell_atom, int ntask, const int* tasks, int nbf,
                                int natom, const double* density, double* grad, void* stream) {
    return gs_eri_grad_band(la, lb, lc, ld, form, 64, pair_rec, prim64, comp_scale, func_off,
                            shell_atom, ntask, tasks, nbf, natom, density, 0, nullptr, 0.0, 0.0,
                            0.0, grad, stream);
}

extern "C" int gs_eri_grad(int la, int lb, int lc, int ld, const void* pair_rec, const void* prim64,
                           const double* comp_scale, const int* func_off, const int* shell_atom,
                           int ntask, const int* tasks, int nbf, int natom, const double* density,
                           double* grad, void* stream) {
    return gs_eri_grad_form(la, lb, lc, ld, 0, pair_rec, prim64, comp_scale, func_off, shell_atom,
                            ntask, tasks, nbf, natom, density, grad, stream);
}

extern "C" int gs_eri_grad_class_form(int la, int lb, int lc, int ld) {
    if (!valid_class(la, lb, lc, ld)) return -GS_ERR_CLASS;
    const int v = g_grad_variant[la][lb][lc][ld];
    return has_thread(la, lb, lc, ld) && (v ? v == 1 : la + lb + lc + ld <= 2) ? 1 : 2;
}
