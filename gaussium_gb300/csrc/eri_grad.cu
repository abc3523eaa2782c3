// C-ABI entry of the fused ERI adjoint (gradient) kernels, csrc/eri_grad.cuh.
#include <cuda_runtime.h>
#include "eri_grad.cuh"
#include "eri_grad_list.h"

#include "eri_grad_0000.h"
#include "eri_grad_1000.h"
#include "eri_grad_1010.h"
#include "eri_grad_1100.h"
#include "eri_grad_1110.h"
#include "eri_grad_1111.h"

extern "C" int gs_eri_grad(int la, int lb, int lc, int ld, const void* pair_rec, const void* prim64,
                           const double* comp_scale, const int* func_off, const int* shell_atom,
                           int ntask, const int* tasks, int nbf, const double* density,
                           double* grad, void* stream) {
    if (ntask < 0 || nbf <= 0 || !pair_rec || !prim64 || !comp_scale || !func_off || !shell_atom ||
        (ntask > 0 && !tasks) || !density || !grad)
        return GS_ERR_ARG;
    gs::GradArgs a{(const gs::PairRec*)pair_rec, (const gs::PrimRec<double>*)prim64, comp_scale,
                   func_off, shell_atom, (const int2*)tasks, ntask, nbf, density, grad};
    cudaStream_t st = (cudaStream_t)stream;
#define GS_GL(A, B, C, D) \
    if (la == A && lb == B && lc == C && ld == D) return gs::launch_grad<A, B, C, D>(a, st);
    GS_FOR_EACH_GRAD(GS_GL)
#undef GS_GL
    return GS_ERR_CLASS;
}
