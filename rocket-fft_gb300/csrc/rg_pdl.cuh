// Programmatic dependent launch (sm_90 and later) for the library's back-to-back kernels.
//
// A multi-axis transform is a chain of kernels on one stream, each reading what the previous
// one wrote. Launched plainly, every link costs the grid-completion and launch latency plus
// the tail of the last wave. Launched with programmatic stream serialization, the next grid is
// scheduled as soon as every CTA of the current one has started (each CTA signals
// griddepcontrol.launch_dependents first thing), so its CTAs take the SM slots the draining
// grid frees; each then waits in griddepcontrol.wait until the previous grid has completed and
// its memory is visible, before it touches global memory. A launch without the attribute
// makes both instructions no-ops, and a kernel launched with it always waits before any global
// access, so the chain keeps plain stream semantics.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <utility>

#include "rg_error.hpp"

namespace rg {

// First statement of every kernel launched through launch_pdl.
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// ROCKET_GPU_PDL=0 launches plainly (rg_launch.cpp).
bool pdl_enabled();
// CTAs of `fn` (with this block size and dynamic shared memory) resident on the device at once;
// cached (rg_launch.cpp).
int64_t resident_ctas(const void *fn, int threads, size_t smem);

// Only grids larger than one wave take the attribute. When a grid fits the device at once,
// every CTA triggers right after the launch and the next grid's CTAs wait on the same SMs
// beside running ones for the whole kernel: measured on GB300, a chain of single-wave
// complex128 kernels (256 CTAs of 256 threads, two per SM) ran 40 % slower that way, while
// the multi-wave passes of the 3-D transforms gain about 9 %.
template <typename... P, typename... A>
void launch_pdl(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A &&...args) {
  const int64_t ctas = int64_t(grid.x) * grid.y * grid.z;
  const bool pdl = pdl_enabled() &&
                   ctas > resident_ctas(reinterpret_cast<const void *>(kernel), int(block.x * block.y * block.z), smem);
  cudaLaunchConfig_t c{};
  c.gridDim = grid;
  c.blockDim = block;
  c.dynamicSmemBytes = smem;
  c.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  c.attrs = at;
  c.numAttrs = pdl ? 1 : 0;
  RG_CUDA(cudaLaunchKernelEx(&c, kernel, std::forward<A>(args)...));
}

}  // namespace rg
