// Status codes and error plumbing shared by the host code. Every C entry point converts an
// rg::Error (or a CUDA failure) into a status code plus a thread-local message; nothing
// throws across the C ABI and nothing aborts.
#pragma once
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "../../include/rocket_gpu.h"

namespace rg {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] inline void cuda_fail(cudaError_t e, const char *what) {
  cudaGetLastError();  // clear the sticky-free error state where possible
  throw Error(e == cudaErrorMemoryAllocation ? RG_ERR_NOMEM : RG_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace rg

#define RG_CUDA(call)                                  \
  do {                                                 \
    cudaError_t rg_e_ = (call);                        \
    if (rg_e_ != cudaSuccess) ::rg::cuda_fail(rg_e_, #call); \
  } while (0)

#define RG_CHECK(cond, code, msg)                 \
  do {                                            \
    if (!(cond)) throw ::rg::Error((code), (msg)); \
  } while (0)
