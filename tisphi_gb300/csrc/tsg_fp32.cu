// FP32-mixed form (placeholder until the mixed-precision kernels land).
#include "tsg_fp32.h"

namespace tsg {

struct Fp32State { int err; };

int fp32_create(const tsg_config&, const Consts&, const tsg_particles*, bool, Fp32State** out, cudaStream_t) {
    *out = nullptr;
    return TSG_E_UNSUPPORTED;
}
void fp32_destroy(Fp32State* st) { delete st; }
void fp32_sort(Fp32State&, cudaStream_t) {}
void fp32_kernel_corr(Fp32State&, cudaStream_t) {}
void fp32_init_tmp(Fp32State&, cudaStream_t) {}
void fp32_one_step(Fp32State&, cudaStream_t) {}
void fp32_advect(Fp32State&, int, cudaStream_t) {}
void fp32_rk_update(Fp32State&, int, cudaStream_t) {}
int fp32_field(Fp32State&, const char*, tsg_view*, cudaStream_t) { return TSG_E_UNSUPPORTED; }
const int* fp32_cell_start(const Fp32State&) { return nullptr; }
void fp32_neighbors(Fp32State&, int*, int*, int*, cudaStream_t) {}
void fp32_diag(Fp32State&, double*, double*, cudaStream_t) {}
int* fp32_err_ptr(Fp32State& st) { return &st.err; }
int fp32_write(Fp32State&, const char*, const void*, bool, cudaStream_t) { return TSG_E_UNSUPPORTED; }
int fp32_read(Fp32State&, const char*, void*, bool, cudaStream_t) { return TSG_E_UNSUPPORTED; }

}  // namespace tsg
