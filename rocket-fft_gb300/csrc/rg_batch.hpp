// Batched uneven-length complex FFTs in one persistent launch (rg_batch.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "rg_plan.hpp"

namespace rg {

struct BatchPlan;
BatchPlan *batch_create(const int64_t *lengths, int64_t count, DType dt, bool forward, double fct, bool autotune);
void batch_exec(BatchPlan &p, const void *in, void *out, cudaStream_t st);
void batch_destroy(BatchPlan *p);
std::string batch_info(const BatchPlan &p);

}  // namespace rg
