// launch_util.cpp -- host helpers shared by the kernel launchers.
#include <map>
#include <mutex>
#include <utility>

#include "gw_kernels.h"

namespace gwgpu {

// cudaFuncAttributeMaxDynamicSharedMemorySize is a property of the function,
// shared by every thread of the process.  Launchers on several streams and
// host threads (serving slots) must never lower it under one another, so the
// limit only ever rises, per device and function.
cudaError_t raise_smem_limit(const void* fn, size_t bytes)
{
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> current;
    int dev = 0;
    cudaError_t rc = cudaGetDevice(&dev);
    if (rc != cudaSuccess) return rc;
    std::lock_guard<std::mutex> lock(mu);
    size_t& cur = current[{dev, fn}];
    if (bytes <= cur) return cudaSuccess;
    rc = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (rc == cudaSuccess) cur = bytes;
    return rc;
}

}  // namespace gwgpu
