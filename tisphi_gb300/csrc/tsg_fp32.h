// FP32-mixed form: interface used by the C ABI layer (tsg_api.cu).
#pragma once
#include <vector>
#include "tsg_internal.h"

namespace tsg {

struct Fp32State;

// Batched ensemble description (host arrays): scene number per particle and the per-scene
// Tait stiffness / viscosity factor 2 (d + 2) nu.
struct Fp32Scenes {
    const int* scene_of = nullptr;   // n entries
    const float* stiffness = nullptr;
    const float* visc_fac = nullptr;
    int nscenes = 0;
};

// Dynamic rigid objects of a scene: ids ascending, off[o] .. off[o + 1] their slice of a
// list of n_rigid_dyn particles.
struct RigidObjects {
    std::vector<int> ids, off;
};
int fp32_create(const tsg_config& cfg, const Consts& c, const tsg_particles* p, bool from_device,
                Fp32State** out, cudaStream_t s, const Fp32Scenes* scenes = nullptr,
                const RigidObjects* rigid = nullptr);
void fp32_solve_rigid(Fp32State& st, cudaStream_t s);
void fp32_destroy(Fp32State* st);
void fp32_sort(Fp32State& st, cudaStream_t s);
// True when the neighbour lists must be rebuilt before the next step (always without a skin).
bool fp32_rebuild_due(Fp32State& st, cudaStream_t s);
// One step of the FP32-mixed sequence the captured graphs replay (kernel correction through
// advect_something), launched eagerly; the caller re-sorts first when lists expire.
void fp32_step_body(Fp32State& st, bool collide, cudaStream_t s);
void fp32_kernel_corr(Fp32State& st, cudaStream_t s);
void fp32_init_tmp(Fp32State& st, cudaStream_t s);
void fp32_one_step(Fp32State& st, cudaStream_t s);
void fp32_advect(Fp32State& st, int which, cudaStream_t s);
void fp32_rk_update(Fp32State& st, int m, cudaStream_t s);
int fp32_field(Fp32State& st, const char* name, tsg_view* out, cudaStream_t s);
const int* fp32_cell_start(const Fp32State& st);
void fp32_neighbors(Fp32State& st, int* counts, int* offsets, int* list, cudaStream_t s);
void fp32_diag(Fp32State& st, double* scratch, double* host_out8, cudaStream_t s);
void fp32_density_sum(Fp32State& st, double* out, cudaStream_t s);
int* fp32_err_ptr(Fp32State& st);
// out[0] / out[1] list entries stored for the dynamic / static block, out[2] overflowed
// particles, out[3] list builds since creation.
int fp32_list_stats(Fp32State& st, int64_t* out5, cudaStream_t s);

// Graph mode: nsteps full steps replayed from captured graphs (the re-sort runs inside the
// graph when the device-side displacement check asks for it).  TSG_E_STATE while
// per-phase profiling is on.
int fp32_step_graph(Fp32State& st, int nsteps, bool collide, cudaStream_t s);
// Fold device-side rebuild counts of graph replays into the host counters (synchronises).
void fp32_flush_counters(Fp32State& st, cudaStream_t s);
void fp32_get_launch(const Fp32State& st, int* tpb, int* cells_per_cta, int* steps_per_graph);
int fp32_set_launch(Fp32State& st, int tpb, int cells_per_cta, int steps_per_graph);
// Time launch-parameter candidates from a saved state and keep the fastest; the particle
// state is restored (re-sorted) afterwards.  *ms_out = best milliseconds per step.
int fp32_autotune(Fp32State& st, int trial_steps, bool collide, cudaStream_t s, float* ms_out);
// Bitwise snapshot of the particle state in the current particle order (device buffer of
// fp32_snapshot_bytes bytes): load marks the lists stale, so the next step re-sorts first.
size_t fp32_snapshot_bytes(Fp32State& st);
int fp32_snapshot_copy(Fp32State& st, void* buf, bool load, cudaStream_t s);
// Replace the granular material constants (mu(I): tan(friction), cohesion; Drucker-Prager:
// the yield-surface constants) of a created state; captured graphs are dropped.
void fp32_set_soil(Fp32State& st, const Consts& c);
void fp32_set_fluid(Fp32State& st, const Consts& c);
// Adjoint of one mu(I) symplectic-Euler step from the loaded state (tsg_adjoint.cu).
int fp32_adjoint_step(Fp32State& st, double* ax, double* av, double* ar, double* avt, double* pbar,
                      cudaStream_t s);
void fp32_free_adjoint(Fp32State& st);
// Per-scene diagnostics of a batched ensemble (host out, 8 values per scene).
int fp32_batch_diag(Fp32State& st, double pitch, double* host_out, int nscenes, cudaStream_t s);
int fp32_write(Fp32State& st, const char* name, const void* src, bool from_device, cudaStream_t s);
// mode: 0 host destination (synchronises), 1 device destination, 2 host destination
// without synchronising (the caller synchronises the stream before using dst).
int fp32_read(Fp32State& st, const char* name, void* dst, int mode, cudaStream_t s);
int fp32_read_set(Fp32State& st, int count, const char* const* names, void* const* dsts, int mode,
                  cudaStream_t s);

}  // namespace tsg
