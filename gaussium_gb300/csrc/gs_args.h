// Argument blocks passed by value to the class kernels (device pointers only).
#pragma once
#include <cuda_runtime.h>

#define GS_KIND_WRITE 0
#define GS_KIND_JK 1
#define GS_KIND_SCHWARZ 2
#define GS_KIND_FORM 3      // launch nothing: return the form a launch would use

#define GS_OK 0
#define GS_ERR_ARG 1
#define GS_ERR_CUDA 2
#define GS_ERR_CLASS 3
#define GS_ERR_DEVICE 4
#define GS_ERR_NOMEM 5
#define GS_ERR_LIMIT 6

namespace gs {
// Streaming multiprocessors of the current device (queried once per device; grid caps for
// launches whose task count lives on the device are multiples of it).
inline int sm_count() {
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    if (!cache[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            return 1;
        cache[dev] = n;
    }
    return cache[dev];
}

struct PairRec;
struct WriteTask;

struct WriteArgs {
    const PairRec* pairs;
    const void* prims;          // PrimRec<double> or PrimRec<float>
    const double* comp_scale;   // [nshell][6]
    const WriteTask* tasks;
    int ntask;
    double* out;
};

struct JKArgs {
    const PairRec* pairs;
    const void* prims;
    const double* comp_scale;
    const int* func_off;        // [nshell]
    const int2* tasks;          // (bra pair, ket pair), canonical
    int ntask;
    int nbf;
    int nshell;
    int nk;                     // number of exchange densities
    const double* pj;           // density for J (nbf x nbf) or null
    const double* pk;           // nk densities for K
    double* j;                  // J' accumulator (nbf x nbf) or null
    double* k;                  // nk K' accumulators
    const double* shell_dmax;   // [nshell][nshell] max |P| per shell block (screening)
    double screen_thr;          // 0 disables screening and precision selection
    double prec_lo, prec_hi;    // evaluate only quartets with prec_lo <= bound < prec_hi
    // batched mode (several molecules in one launch): shell -> molecule, and per molecule
    // the offset of its nbf_m x nbf_m matrices, nbf_m, and max |P| (screening); func_off
    // is then local to the molecule.  Null shell_mol: one molecule of nbf functions.
    const int* shell_mol;
    const long long* mol_base;
    const int* mol_n;
    const double* mol_dmax;
    long long mat_stride;       // elements between the nk exchange densities / outputs
    const int* ntask_dev;       // if set, the task count is read here (ntask is the bound)
};

struct SchwarzArgs {
    const PairRec* pairs;
    const void* prims;          // PrimRec<double>
    const double* comp_scale;
    const int* pair_index;      // pairs of this class
    int npair;
    double* q;                  // [npairs total] output
};
}  // namespace gs
