// gb_launch.cuh -- launching kernels as thread-block clusters.
#pragma once

#include <cuda_runtime.h>

namespace gb {

// Launch `clusters` clusters of `csize` CTAs each (sizes above the portable 8
// are enabled on the kernel first).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_clusters_dsm(void (*kernel)(KArgs...), int clusters, int csize, int threads, size_t dsm,
                                       cudaStream_t stream, Args... args) {
  if (csize > 8) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(clusters * csize));
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = dsm;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, (KArgs)args...);
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_clusters(void (*kernel)(KArgs...), int clusters, int csize, int threads,
                                   cudaStream_t stream, Args... args) {
  return launch_clusters_dsm(kernel, clusters, csize, threads, 0, stream, args...);
}

// Clusters of `csize` CTAs that can be resident at once (0 if none fit).
template <typename... KArgs>
inline int max_active_clusters(void (*kernel)(KArgs...), int csize, int threads, size_t dsm = 0) {
  if (csize > 8 && cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
    return 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)csize);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = dsm;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, kernel, &cfg) != cudaSuccess) return 0;
  return n;
}

}  // namespace gb
