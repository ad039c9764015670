// launch.cuh -- kernel launches with an optional L2 access-policy window.
#pragma once

#include <cuda_runtime.h>

namespace vt {

// kernel<<<grid, block, smem, st>>>(args...), with `win` (when not null) as
// the launch's access-policy-window attribute: the window travels with this
// one launch (also into a graph being captured), nothing is set on the stream.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_kernel(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                 const cudaAccessPolicyWindow* win, Args... args) {
    if (!win) {
        kernel<<<grid, block, smem, st>>>(args...);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeAccessPolicyWindow;
    attr.val.accessPolicyWindow = *win;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace vt
