// Persistent batched J/K kernel, FP64 instantiation (csrc/persistent.cuh).
#include "persistent.cuh"
#include "eri_all_classes.h"

int gs_persist_launch_64(const gs::PersistArgs& a, cudaStream_t st) {
    using T = double;
    constexpr size_t bytes = gs::PersistSmem<T>::BYTES;
    auto k = gs::k_persistent_jk<T>;
    if (gs::set_smem<gs::k_persistent_jk<T>>(bytes)) return GS_ERR_CUDA;
    // one resident wave: as many blocks per SM as the kernel's registers and shared memory
    // allow, on every SM
    static int per_sm[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return GS_ERR_CUDA;
    if (!per_sm[dev]) {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, 32 * gs::kPersistWarps, bytes) !=
                cudaSuccess || n <= 0)
            return GS_ERR_CUDA;
        per_sm[dev] = n;
    }
    k<<<per_sm[dev] * gs::sm_count(), 32 * gs::kPersistWarps, bytes, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? GS_OK : GS_ERR_CUDA;
}
