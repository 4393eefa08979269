// Internal declarations shared by the CUDA translation units of libtisphi_gb300.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "../../include/tisphi_gb300.h"

namespace tsg {

// Host-side count of kernel launches issued by this library (all handles).  Graph replays
// add their kernel-node counts through add_launches; launches recorded while a stream is
// being captured are taken back out (they are nodes, not launches).
void note_launch();
void add_launches(long long delta);
long long launch_total();
// True while tsg_profile is on (steps then run eagerly, with per-phase events).
bool profiling_on();
#define TSG_LAUNCH(kernel, grid, block, stream, ...)                   \
    do {                                                                \
        ::tsg::note_launch();                                           \
        kernel<<<(grid), (block), 0, (stream)>>>(__VA_ARGS__);          \
    } while (0)

// Phase profiling: when enabled, every launcher brackets its kernels with CUDA events
// recorded on the launching stream, and elapsed times are summed per phase.
enum Phase { PH_SORT = 0, PH_CORR, PH_INIT, PH_PRE, PH_BDY, PH_RATES, PH_INTEGRATE, PH_POS, PH_POST, PH_OTHER, PH_LISTS, PH_COUNT };
struct PhaseScope {
    PhaseScope(cudaStream_t s, int phase);
    ~PhaseScope();
    cudaStream_t s_;
    int phase_;
    void* stop_;
};

constexpr int MAT_REP = -2, MAT_DUMMY = -1, MAT_FLUID = 1, MAT_SOIL = 2, MAT_RIGID = 11;
constexpr double EPS = 1e-8;      // SPHBase.epsilon (eng/solver_sph_base.py:25)
constexpr double EPS_F = 1e-4;    // DPSPHSolver.eps_f (eng/solver_sph_dp.py:23)

// Scene constants derived on the host once, passed to every kernel by value.
struct Consts {
    int dim, solver, kernel, corr, xsph, boundary, exponent_is_int, ti;
    int n, n_flow, n_bdy, flow_type;
    int gnum[3];
    long long G;
    double vs[3], grid, R, h, h1, kk, visc_fac, eps_h2, h2;
    double rho0, B, gamma, dt, hdt, dt6, g[3];
    double mu, vsound2, coh;
    double alpha, k_c, kc_over_alpha, Gm, Km, sin_dila, lam_den, three_aK, nine_K_sin, twoG;
    double damp_E, damp_eps, K0;
    double rep_fac, diam, h075;
    double ds[3], de[3], r_eps;
    // f32 candidate prefilter: reject when |dx_f32|^2 > pf_r2; valid for centres with
    // every |x - vdomain_start| below pf_lim
    int pf_on;
    float pf_r2, pf_lim;
    int n_rigid_dyn;    // dynamic rigid particles (shape-matched bodies)
};

// Dynamic rigid bodies (eng/solver_sph_base.py:467-518): object ids, rest centres of mass
// (from the uploaded positions, in upload order) and, per object, the slice of `list`
// that the list builder (tsg_rigid_list.cuh) fills with the object's particles in
// ascending order before every shape matching.
// Largest cell segment the counting sort's last step gives to one thread (tsg_cellsort.cuh),
// and the size of its list of larger cells (at most n / (kSortSmall + 1) of them).
constexpr int kSortSmall = 256;
inline size_t cellsort_big_ints(long long n) { return (size_t)(n / kSortSmall + 2); }

// Block size of the rigid-object list builder (tsg_rigid_list.cuh) and its scratch size.
constexpr int kRListBlock = 256;
inline int rlist_blocks(int n) { return (n + kRListBlock - 1) / kRListBlock; }
inline size_t rlist_scratch_ints(int n, int nobj) { return (size_t)nobj * (size_t)rlist_blocks(n); }

struct Rigid64 {
    int nobj = 0;
    int* obj_id = nullptr;      // nobj (device)
    double* rest_cm = nullptr;  // 3 nobj (device)
    int* off = nullptr;         // nobj + 1 (device): slice starts in list
    int* list = nullptr;        // n_rigid_dyn (device)
    int* scratch = nullptr;     // nobj * ceil(n / 256) (device): the list builder's block offsets
};

// Persistent per-particle fields (permuted by the sort; double-buffered).
struct Persist64 {
    double* x;          // 3 planes of n
    double* v;          // 3 planes
    double* x0;         // 3 planes
    double* density;
    double* mass;
    double* m_V;
    double* pressure;
    double* stress;     // 9 planes (soil solvers) or nullptr
    double* strain_equ;
    double* strain_equ_p;
    int* flag_retmap;
    int* mat_type;
    int* mat_id;
    int* obj_id;
    int* is_dynamic;
    int* id0;
};

// Transient per-particle fields (recomputed every step, in sorted order).
struct Trans64 {
    double* v_tmp;      // 3 planes
    double* density_tmp;
    double* stress_tmp; // 9 planes or nullptr
    double* d_density;
    double* d_vel;      // 3 planes
    double* d_stress;   // 9 planes or nullptr (DP)
    double* v_grad;     // 9 planes or nullptr (soil)
    double* CSPM_f;
    double* CSPM_L;     // 9 planes or nullptr (kernel_corr)
    double* d_strain_equ;
    double* d_strain_equ_p;
    double* d_density_RK;
    double* d_vel_RK;   // 3 planes
    double* d_stress_RK;// 9 planes or nullptr
    double* aux3;       // 3 planes: XSPH sums
    double* aux9;       // 9 planes: regularised stress (mu(I))
    float4* pos32;      // (x - vdomain_start) as f32, candidate prefilter
};

// Sort scratch and cell table.
struct Grid {
    int* cell_of;       // per particle (old order)
    int* rank;          // per particle within-cell arrival rank
    int* count;         // G + 1
    int* cell_start;    // G + 2 exclusive starts; [G] = out-of-grid bin, [G+1] = n
    int* perm;          // new -> old
    int* tile_sum;      // scan partials
    int* list_flow;     // flow particles (sorted indices)
    int* list_bdy;      // boundary + rigid particles
    int* list_count;    // [0] flow, [1] bdy
    int* err;           // device error word
    int* big;           // cells above kSortSmall particles (cellsort_big_ints)
    int* nbig;          // their count
};

// ---- headless visual buffer (tsg_visual.cu) ----
// Planar f64 / int views of the fields a colour title may read (null when absent).
struct VisFields {
    const double *x, *x0, *v, *d_vel, *v_tmp, *density, *d_density, *pressure, *stress, *strain_equ,
        *strain_equ_p, *CSPM_L;
    const int *id0, *mat_type, *flag;
    int n;
};
int visual_launch(const VisFields& f, const tsg_visual_cfg& vc, double* scratch, float* pos, float* col,
                  double* range_out, cudaStream_t s);

// ---- launchers (tsg_sort.cu) ----
void sort_fp64(const Consts& c, Persist64& cur, Persist64& nxt, Trans64& t, Grid& g, cudaStream_t s);
void scan_exclusive(const int* in, int* out, int n, int* tile_sum, cudaStream_t s);

// ---- launchers (tsg_fp64.cu) ----
void fp64_kernel_corr(const Consts& c, const Persist64& p, Trans64& t, const Grid& g, cudaStream_t s);
void fp64_init_tmp(const Consts& c, const Persist64& p, Trans64& t, cudaStream_t s);
void fp64_one_step(const Consts& c, Persist64& p, Trans64& t, const Grid& g, cudaStream_t s);
void fp64_advect(const Consts& c, Persist64& p, Trans64& t, const Grid& g, int which, cudaStream_t s);
void fp64_rk_update(const Consts& c, Persist64& p, Trans64& t, int m, cudaStream_t s);
void fp64_neighbors(const Consts& c, const Persist64& p, const Trans64& t, const Grid& g,
                    int* counts, int* offsets, int* list, cudaStream_t s);
void fp64_diag(const Consts& c, const Persist64& p, double* out8, cudaStream_t s);
void fp64_solve_rigid(const Consts& c, Persist64& p, const Rigid64& r, cudaStream_t s);
void fp64_rest_cm(const Consts& c, const Persist64& p, const Rigid64& r, cudaStream_t s);
void fp64_density_sum(const Consts& c, const Persist64& p, const Trans64& t, const Grid& g, double* out,
                      cudaStream_t s);
void fp64_init_geostatic(const Consts& c, Persist64& p, double* scratch, cudaStream_t s);
void fp64_refresh_pos32(const Consts& c, const Persist64& p, Trans64& t, cudaStream_t s);

}  // namespace tsg
