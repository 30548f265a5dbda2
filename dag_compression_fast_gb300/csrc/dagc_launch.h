// Host side of programmatic dependent launch: kernels whose first statement
// is pdl_prologue() can be launched with programmatic stream serialization, so
// that the next kernel is scheduled while the previous one runs. Off unless
// the context's DAGC_OPT_PDL asks for it: on GB300 plain stream order measured
// faster for this pipeline.
#pragma once

#include <cuda_runtime.h>

namespace dagc {

// Whether launch_pdl sets the attribute; set from the calling context's
// DAGC_OPT_PDL at the start of each call that launches kernels (the launches
// of a call happen on the calling thread).
inline thread_local bool t_pdl = false;

inline cudaLaunchConfig_t pdl_config(dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                     cudaLaunchAttribute* attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = t_pdl ? 1 : 0;
    return cfg;
}

template <typename... Params, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(Params...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg = pdl_config(grid, block, smem, s, attr);
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Params>(args)...);
}

// The same for a kernel known only by address, with its arguments as an array.
inline cudaError_t launch_pdl_c(const void* kernel, dim3 grid, dim3 block, void** args, size_t smem,
                                cudaStream_t s) {
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg = pdl_config(grid, block, smem, s, attr);
    return cudaLaunchKernelExC(&cfg, kernel, args);
}

}  // namespace dagc
