// tma_map.h -- TMA tensor maps for the library's kernels.  The encoder
// (cuTensorMapEncodeTiled) is reached through the runtime's driver entry
// point, so the library does not link against the driver library.
#pragma once
#include <cuda.h>  // CUtensorMap
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <mutex>

namespace fg {

inline cudaError_t tensor_map_encoder(PFN_cuTensorMapEncodeTiled_v12000* out) {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (q != cudaDriverEntryPointSuccess || !p) return cudaErrorNotSupported;
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    *out = fn;
    return cudaSuccess;
}

}  // namespace fg
