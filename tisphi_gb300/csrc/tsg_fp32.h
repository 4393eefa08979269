// FP32-mixed form: interface used by the C ABI layer (tsg_api.cu).
#pragma once
#include "tsg_internal.h"

namespace tsg {

struct Fp32State;

int fp32_create(const tsg_config& cfg, const Consts& c, const tsg_particles* p, bool from_device,
                Fp32State** out, cudaStream_t s);
void fp32_destroy(Fp32State* st);
void fp32_sort(Fp32State& st, cudaStream_t s);
// True when the neighbour lists must be rebuilt before the next step (always without a skin).
bool fp32_rebuild_due(Fp32State& st, cudaStream_t s);
void fp32_kernel_corr(Fp32State& st, cudaStream_t s);
void fp32_init_tmp(Fp32State& st, cudaStream_t s);
void fp32_one_step(Fp32State& st, cudaStream_t s);
void fp32_advect(Fp32State& st, int which, cudaStream_t s);
void fp32_rk_update(Fp32State& st, int m, cudaStream_t s);
int fp32_field(Fp32State& st, const char* name, tsg_view* out, cudaStream_t s);
const int* fp32_cell_start(const Fp32State& st);
void fp32_neighbors(Fp32State& st, int* counts, int* offsets, int* list, cudaStream_t s);
void fp32_diag(Fp32State& st, double* scratch, double* host_out8, cudaStream_t s);
int* fp32_err_ptr(Fp32State& st);
int fp32_write(Fp32State& st, const char* name, const void* src, bool from_device, cudaStream_t s);
int fp32_read(Fp32State& st, const char* name, void* dst, bool to_device, cudaStream_t s);

}  // namespace tsg
