// C ABI of libtisphi_gb300: handle life cycle, uploads, the step sequence and field views.
// The step sequence restates SPHBase.step / substep (eng/solver_sph_base.py:41-61,
// :89-91, :116-120, :172-180) as a fixed list of kernel launches on one stream.
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "tsg_internal.h"
#include "tsg_fp32.h"

using namespace tsg;

namespace tsg {
static std::atomic<long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void add_launches(long long delta) { g_launches.fetch_add(delta, std::memory_order_relaxed); }
long long launch_total() { return g_launches.load(std::memory_order_relaxed); }

struct ProfRec { int phase; cudaEvent_t a, b; };
struct Profiler {
    bool on = false;
    std::vector<ProfRec> recs;
    std::vector<cudaEvent_t> pool;
    cudaEvent_t get() {
        if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
        cudaEvent_t e; cudaEventCreate(&e); return e;
    }
};
static Profiler g_prof;
bool profiling_on() { return g_prof.on; }

PhaseScope::PhaseScope(cudaStream_t s, int phase) : s_(s), phase_(phase), stop_(nullptr) {
    if (!g_prof.on) return;
    cudaEvent_t a = g_prof.get(), b = g_prof.get();
    cudaEventRecord(a, s);
    g_prof.recs.push_back({phase, a, b});
    stop_ = reinterpret_cast<void*>(b);
}
PhaseScope::~PhaseScope() {
    if (stop_) cudaEventRecord(reinterpret_cast<cudaEvent_t>(stop_), s_);
}
}  // namespace tsg

struct tsg_handle {
    tsg_config cfg;
    Consts c;
    int n = 0;
    bool uploaded = false;
    bool sorted = false;
    bool pos32_dirty = true;
    Persist64 cur{}, nxt{};
    Trans64 t{};
    Grid g{};
    double* d_stage = nullptr;      // upload / download staging (9 n doubles)
    double* d_scratch = nullptr;    // small reductions
    std::vector<void*> allocs;
    Fp32State* f32 = nullptr;       // FP32-mixed form (nullptr for FP64)
    int nscenes = 0;                // batched ensemble (tsg_batch_create): scenes and x pitch
    double batch_pitch = 0.0;
    Rigid64 rigid{};                // dynamic rigid bodies (FP64 form)
};

namespace {

const char* kStatus[] = {"ok", "invalid argument", "invalid configuration", "CUDA error", "invalid state",
                         "unsupported scene feature", "unknown field name", "capacity too small"};

template <class T>
int dalloc(tsg_handle* h, T** p, size_t count) {
    *p = nullptr;
    if (count == 0) return 0;
    void* q = nullptr;
    if (cudaMalloc(&q, count * sizeof(T)) != cudaSuccess) return TSG_E_CUDA;
    cudaMemset(q, 0, count * sizeof(T));
    h->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return 0;
}

int check_cuda() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        std::fprintf(stderr, "tisphi_gb300: CUDA error: %s\n", cudaGetErrorString(e));
        return TSG_E_CUDA;
    }
    return 0;
}

int alloc_persist(tsg_handle* h, Persist64& p, bool soil) {
    const size_t n = h->n;
    int rc = 0;
    rc |= dalloc(h, &p.x, 3 * n); rc |= dalloc(h, &p.v, 3 * n); rc |= dalloc(h, &p.x0, 3 * n);
    rc |= dalloc(h, &p.density, n); rc |= dalloc(h, &p.mass, n); rc |= dalloc(h, &p.m_V, n);
    rc |= dalloc(h, &p.pressure, n);
    if (soil) {
        rc |= dalloc(h, &p.stress, 9 * n); rc |= dalloc(h, &p.strain_equ, n);
        rc |= dalloc(h, &p.strain_equ_p, n); rc |= dalloc(h, &p.flag_retmap, n);
    }
    rc |= dalloc(h, &p.mat_type, n); rc |= dalloc(h, &p.mat_id, n); rc |= dalloc(h, &p.obj_id, n);
    rc |= dalloc(h, &p.is_dynamic, n); rc |= dalloc(h, &p.id0, n);
    return rc ? TSG_E_CUDA : 0;
}

int alloc_all(tsg_handle* h) {
    const size_t n = h->n;
    const Consts& c = h->c;
    const bool soil = c.solver != 1;
    int rc = 0;
    rc |= alloc_persist(h, h->cur, soil);
    rc |= alloc_persist(h, h->nxt, soil);
    Trans64& t = h->t;
    rc |= dalloc(h, &t.v_tmp, 3 * n); rc |= dalloc(h, &t.density_tmp, n);
    if (soil) { rc |= dalloc(h, &t.stress_tmp, 9 * n); rc |= dalloc(h, &t.v_grad, 9 * n); rc |= dalloc(h, &t.aux9, 9 * n); }
    if (c.solver == 3) rc |= dalloc(h, &t.d_stress, 9 * n);
    rc |= dalloc(h, &t.d_density, n); rc |= dalloc(h, &t.d_vel, 3 * n);
    rc |= dalloc(h, &t.CSPM_f, n);
    if (c.corr == 1) rc |= dalloc(h, &t.CSPM_L, 9 * n);
    rc |= dalloc(h, &t.d_strain_equ, n); rc |= dalloc(h, &t.d_strain_equ_p, n);
    // RK4 accumulators for every integrator: substep_RK may be called on any handle
    rc |= dalloc(h, &t.d_density_RK, n); rc |= dalloc(h, &t.d_vel_RK, 3 * n);
    if (c.solver == 3) rc |= dalloc(h, &t.d_stress_RK, 9 * n);
    rc |= dalloc(h, &t.aux3, 3 * n);
    rc |= dalloc(h, &t.pos32, n);
    Grid& g = h->g;
    const size_t nb = (size_t)c.G + 1;
    rc |= dalloc(h, &g.cell_of, n); rc |= dalloc(h, &g.rank, n); rc |= dalloc(h, &g.count, nb);
    rc |= dalloc(h, &g.cell_start, nb + 1); rc |= dalloc(h, &g.perm, n);
    rc |= dalloc(h, &g.tile_sum, nb / 2048 + 2);
    rc |= dalloc(h, &g.big, cellsort_big_ints(n)); rc |= dalloc(h, &g.nbig, 1);
    rc |= dalloc(h, &g.list_flow, n + 1); rc |= dalloc(h, &g.list_bdy, n + 1);
    rc |= dalloc(h, &g.list_count, 2); rc |= dalloc(h, &g.err, 1);
    rc |= dalloc(h, &h->d_stage, 9 * n + 16);
    rc |= dalloc(h, &h->d_scratch, 64);
    return rc ? TSG_E_CUDA : 0;
}

__global__ void k_deinterleave(const double* __restrict__ src, double* __restrict__ dst, int n, int k) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int q = 0; q < k; ++q) dst[(size_t)q * n + i] = src[(size_t)i * k + q];
}

__global__ void k_iota(int* a, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = i;
}

inline int nb256(long long n) { return (int)((n + 255) / 256); }

cudaStream_t S(void* s) { return static_cast<cudaStream_t>(s); }

// Upload (n, k) row-major doubles into k planes.
int upload_planes(tsg_handle* h, const double* src, double* dst, int k, bool from_device, cudaStream_t s) {
    const size_t bytes = sizeof(double) * (size_t)h->n * k;
    if (!src) { cudaMemsetAsync(dst, 0, bytes, s); return 0; }
    cudaMemcpyAsync(h->d_stage, src, bytes, from_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s);
    if (k == 1) cudaMemcpyAsync(dst, h->d_stage, bytes, cudaMemcpyDeviceToDevice, s);
    else TSG_LAUNCH(k_deinterleave, nb256(h->n), 256, s, h->d_stage, dst, h->n, k);
    return 0;
}

int upload_ints(const int32_t* src, int* dst, size_t n, bool from_device, cudaStream_t s) {
    cudaMemcpyAsync(dst, src, sizeof(int) * n, from_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s);
    return 0;
}

bool use_fp32(const tsg_handle* h) { return h->f32 != nullptr; }

void refresh_pos32_if_dirty(tsg_handle* h, cudaStream_t s) {
    if (h->pos32_dirty && !use_fp32(h)) {
        fp64_refresh_pos32(h->c, h->cur, h->t, s);
        h->pos32_dirty = false;
    }
}

}  // namespace

extern "C" {

const char* tsg_status_string(int status) {
    if (status > 0) return "device error word set (see TSG_ERR_* bits)";
    int k = -status;
    if (k < 0 || k >= (int)(sizeof(kStatus) / sizeof(kStatus[0]))) return "unknown status";
    return kStatus[k];
}

int tsg_create(const tsg_config* cfg, tsg_handle** out) {
    if (!cfg || !out) return TSG_E_ARG;
    *out = nullptr;
    const tsg_config& f = *cfg;
    if (f.dim != 2 && f.dim != 3) return TSG_E_CONFIG;
    if (f.solver < 1 || f.solver > 3) return TSG_E_CONFIG;
    if (f.kernel != 0 && f.kernel != 1) return TSG_E_CONFIG;
    if (f.kernel_corr != 0 && f.kernel_corr != 1) return TSG_E_UNSUPPORTED;
    if (f.time_integration != 1 && f.time_integration != 2 && f.time_integration != 4) return TSG_E_UNSUPPORTED;
    if (f.boundary < 0 || f.boundary > 4) return TSG_E_CONFIG;
    if (f.precision != TSG_FP64 && f.precision != TSG_FP32_MIXED) return TSG_E_CONFIG;
    if (f.grid_num_total <= 0 || f.grid_num_total > (1ll << 30)) return TSG_E_CONFIG;
    if (!(f.grid_size > 0) || !(f.smoothing_len > 0) || !(f.dt > 0)) return TSG_E_CONFIG;
    tsg_handle* h = new tsg_handle();
    h->cfg = f;
    Consts& c = h->c;
    std::memset(&c, 0, sizeof c);
    c.dim = f.dim; c.solver = f.solver; c.kernel = f.kernel; c.corr = f.kernel_corr; c.xsph = f.xsph;
    c.boundary = f.boundary; c.exponent_is_int = f.exponent_is_int; c.ti = f.time_integration;
    c.flow_type = f.solver == 1 ? MAT_FLUID : MAT_SOIL;
    for (int d = 0; d < 3; ++d) {
        c.gnum[d] = f.grid_num[d];
        c.vs[d] = f.vdomain_start[d];
        c.g[d] = f.gravity[d];
        c.ds[d] = f.domain_start[d];
        c.de[d] = f.domain_end[d];
    }
    c.G = f.grid_num_total;
    c.grid = f.grid_size;
    c.R = f.support_radius;
    c.h = f.smoothing_len;
    c.h1 = 1.0 / c.h;
    const double pi = 3.141592653589793;
    double k;
    if (f.kernel == 1) k = f.dim == 2 ? 7.0 / (4.0 * pi) : 21.0 / (2.0 * pi);
    else k = f.dim == 2 ? 15.0 / 7.0 / pi : 3.0 / 2.0 / pi;
    c.kk = k * std::pow(c.h1, (double)f.dim);
    c.visc_fac = 2 * (f.dim + 2) * f.viscosity;
    c.h2 = std::pow(c.h, 2.0);
    c.eps_h2 = 0.01 * c.h2;
    c.rho0 = f.density0;
    c.B = f.stiffness;
    c.gamma = f.exponent;
    c.dt = f.dt;
    c.hdt = 0.5 * f.dt;
    c.dt6 = f.dt / 6.0;
    c.coh = f.cohesion;
    c.damp_E = f.E;
    c.damp_eps = f.damping_eps;
    double vsound = 60.0;
    if (f.solver == 2) {
        c.mu = std::tan(f.friction);
        vsound = 24.0;
        c.vsound2 = std::pow(24.0, 2.0);
    } else if (f.solver == 3) {
        double tf = std::tan(f.friction);
        double den = std::sqrt(9 + 12 * std::pow(tf, 2.0));
        c.alpha = tf / den;
        c.k_c = 3 * f.cohesion / den;
        c.Gm = f.E / (2 * (1 + f.poisson));
        c.Km = f.E / (3 * (1 - 2 * f.poisson));
        c.sin_dila = std::sin(f.dilatancy);
        c.kc_over_alpha = c.k_c / c.alpha;
        c.lam_den = 27.0 * c.alpha * c.Km * c.sin_dila + c.Gm;
        c.three_aK = 3.0 * c.alpha * c.Km;
        c.nine_K_sin = 9.0 * c.Km * c.sin_dila;
        c.twoG = 2.0 * c.Gm;
        c.K0 = 1.0 - std::sin(f.friction);
        vsound = std::sqrt(f.E / f.density0);
    }
    c.rep_fac = 0.01 * (vsound * vsound);
    c.diam = f.particle_diameter;
    c.h075 = 0.75 * f.smoothing_len;
    c.r_eps = f.particle_radius - EPS;
    // f32 prefilter: a relative margin of 2^-10 on R^2 covers the f32 rounding of
    // coordinates below 500 R (error ~ 6 R 2^-22 (|x| + R) << 2^-10 R^2).
    c.pf_on = 1;
    c.pf_r2 = std::nextafter((float)(c.R * c.R * (1.0 + 1.0 / 1024.0)), 1e30f);
    c.pf_lim = (float)(500.0 * c.R);
    *out = h;
    return 0;
}

}  // extern "C"

namespace {
int upload_impl(tsg_handle* h, const tsg_particles* p, int from_device, void* stream, const Fp32Scenes* scenes);
}

extern "C" {

int tsg_upload(tsg_handle* h, const tsg_particles* p, int from_device, void* stream) {
    return upload_impl(h, p, from_device, stream, nullptr);
}

}  // extern "C"

namespace {
int upload_impl(tsg_handle* h, const tsg_particles* p, int from_device, void* stream, const Fp32Scenes* scenes) {
    if (!h || !p || p->n <= 0 || p->n > (1ll << 30) || !p->x || !p->v || !p->density || !p->mass || !p->m_V ||
        !p->pressure || !p->mat_type || !p->mat_id || !p->obj_id || !p->is_dynamic)
        return TSG_E_ARG;
    if (h->uploaded) return TSG_E_STATE;
    cudaStream_t s = S(stream);
    h->n = (int)p->n;
    Consts& c = h->c;
    c.n = h->n;
    // particle classes (types never change)
    std::vector<int32_t> mt(h->n);
    std::vector<int32_t> dyn(h->n);
    if (from_device) {
        cudaMemcpy(mt.data(), p->mat_type, sizeof(int32_t) * h->n, cudaMemcpyDeviceToHost);
        cudaMemcpy(dyn.data(), p->is_dynamic, sizeof(int32_t) * h->n, cudaMemcpyDeviceToHost);
    } else {
        std::memcpy(mt.data(), p->mat_type, sizeof(int32_t) * h->n);
        std::memcpy(dyn.data(), p->is_dynamic, sizeof(int32_t) * h->n);
    }
    int nflow = 0, nbdy = 0, nfluid = 0, nsoil = 0, nrdyn = 0;
    std::vector<int32_t> oid(h->n);
    if (from_device) cudaMemcpy(oid.data(), p->obj_id, sizeof(int32_t) * h->n, cudaMemcpyDeviceToHost);
    else std::memcpy(oid.data(), p->obj_id, sizeof(int32_t) * h->n);
    std::vector<int> robj;          // dynamic rigid object ids and their particle counts
    std::vector<int> rcount;
    for (int i = 0; i < h->n; ++i) {
        const int t = mt[i];
        if (t == MAT_FLUID) ++nfluid;
        else if (t == MAT_SOIL) ++nsoil;
        else if (t == MAT_DUMMY || t == MAT_REP) ++nbdy;
        else if (t == MAT_RIGID) {
            ++nbdy;
            if (dyn[i]) {
                ++nrdyn;
                size_t q = 0;
                while (q < robj.size() && robj[q] != oid[i]) ++q;
                if (q == robj.size()) { robj.push_back(oid[i]); rcount.push_back(0); }
                ++rcount[q];
            }
        }
        else return TSG_E_ARG;
    }
    // dynamic rigid bodies: both forms for WCSPH, the FP64 form for the granular solvers; not
    // in batched ensembles
    if (nrdyn && (scenes || (h->cfg.precision == TSG_FP32_MIXED && c.solver != 1))) return TSG_E_UNSUPPORTED;
    c.n_rigid_dyn = nrdyn;
    RigidObjects robjs;  // ids ascending, slices of the per-object particle lists
    if (nrdyn) {
        std::vector<size_t> order(robj.size());
        for (size_t q = 0; q < order.size(); ++q) order[q] = q;
        std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return robj[a] < robj[b]; });
        robjs.off.push_back(0);
        for (size_t q : order) { robjs.ids.push_back(robj[q]); robjs.off.push_back(robjs.off.back() + rcount[q]); }
    }
    if ((c.solver == 1 && nsoil) || (c.solver != 1 && nfluid)) return TSG_E_UNSUPPORTED;
    nflow = c.solver == 1 ? nfluid : nsoil;
    c.n_flow = nflow;
    c.n_bdy = nbdy;
    if (c.dim == 2) {  // the 2D kernels assume every z coordinate and z velocity is zero
        std::vector<double> xz(3 * (size_t)h->n), vz(3 * (size_t)h->n);
        cudaMemcpyKind kind = from_device ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost;
        cudaMemcpy(xz.data(), p->x, sizeof(double) * 3 * h->n, kind);
        cudaMemcpy(vz.data(), p->v, sizeof(double) * 3 * h->n, kind);
        for (int i = 0; i < h->n; ++i)
            if (xz[3 * i + 2] != 0.0 || vz[3 * i + 2] != 0.0) return TSG_E_UNSUPPORTED;
    }
    if (h->cfg.precision == TSG_FP32_MIXED) {
        int rc = fp32_create(h->cfg, c, p, from_device != 0, &h->f32, s, scenes, nrdyn ? &robjs : nullptr);
        if (rc) return rc;
        h->uploaded = true;
        return check_cuda();
    }
    int rc = alloc_all(h);
    if (rc) return rc;
    const bool dev = from_device != 0;
    upload_planes(h, p->x, h->cur.x, 3, dev, s);
    upload_planes(h, p->x, h->cur.x0, 3, dev, s);
    upload_planes(h, p->v, h->cur.v, 3, dev, s);
    upload_planes(h, p->density, h->cur.density, 1, dev, s);
    upload_planes(h, p->mass, h->cur.mass, 1, dev, s);
    upload_planes(h, p->m_V, h->cur.m_V, 1, dev, s);
    upload_planes(h, p->pressure, h->cur.pressure, 1, dev, s);
    if (c.solver != 1) upload_planes(h, p->stress, h->cur.stress, 9, dev, s);
    upload_ints(p->mat_type, h->cur.mat_type, h->n, dev, s);
    upload_ints(p->mat_id, h->cur.mat_id, h->n, dev, s);
    if (nrdyn) {  // object table (ids ascending), list slices, rest centres of mass
        Rigid64& rb = h->rigid;
        rb.nobj = (int)robjs.ids.size();
        if ((rc = dalloc(h, &rb.obj_id, robjs.ids.size())) || (rc = dalloc(h, &rb.off, robjs.off.size())) ||
            (rc = dalloc(h, &rb.rest_cm, 3 * robjs.ids.size())) || (rc = dalloc(h, &rb.list, (size_t)nrdyn)) ||
            (rc = dalloc(h, &rb.scratch, rlist_scratch_ints(h->n, rb.nobj))))
            return rc;
        cudaMemcpy(rb.obj_id, robjs.ids.data(), sizeof(int) * robjs.ids.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(rb.off, robjs.off.data(), sizeof(int) * robjs.off.size(), cudaMemcpyHostToDevice);
    }
    upload_ints(p->obj_id, h->cur.obj_id, h->n, dev, s);
    upload_ints(p->is_dynamic, h->cur.is_dynamic, h->n, dev, s);
    TSG_LAUNCH(k_iota, nb256(h->n), 256, s, h->cur.id0, h->n);
    if (c.solver == 3 && h->cfg.init_geostatic) fp64_init_geostatic(c, h->cur, h->d_scratch, s);
    if (nrdyn) fp64_rest_cm(c, h->cur, h->rigid, s);
    h->uploaded = true;
    h->pos32_dirty = true;
    return check_cuda();
}
}  // namespace

extern "C" {

int64_t tsg_particle_num(const tsg_handle* h) { return h ? h->n : 0; }

int tsg_sort(tsg_handle* h, void* stream) {
    if (!h || !h->uploaded) return TSG_E_STATE;
    cudaStream_t s = S(stream);
    if (use_fp32(h)) fp32_sort(*h->f32, s);
    else sort_fp64(h->c, h->cur, h->nxt, h->t, h->g, s);
    h->sorted = true;
    h->pos32_dirty = false;
    return check_cuda();
}

int tsg_kernel_corr(tsg_handle* h, void* stream) {
    if (!h || !h->sorted) return TSG_E_STATE;
    cudaStream_t s = S(stream);
    if (use_fp32(h)) fp32_kernel_corr(*h->f32, s);
    else { refresh_pos32_if_dirty(h, s); fp64_kernel_corr(h->c, h->cur, h->t, h->g, s); }
    return check_cuda();
}

int tsg_init_tmp(tsg_handle* h, void* stream) {
    if (!h || !h->uploaded) return TSG_E_STATE;
    cudaStream_t s = S(stream);
    if (use_fp32(h)) fp32_init_tmp(*h->f32, s);
    else fp64_init_tmp(h->c, h->cur, h->t, s);
    return check_cuda();
}

int tsg_one_step(tsg_handle* h, void* stream) {
    if (!h || !h->sorted) return TSG_E_STATE;
    cudaStream_t s = S(stream);
    if (use_fp32(h)) fp32_one_step(*h->f32, s);
    else { refresh_pos32_if_dirty(h, s); fp64_one_step(h->c, h->cur, h->t, h->g, s); }
    return check_cuda();
}

int tsg_advect(tsg_handle* h, int which, void* stream) {
    if (!h || !h->uploaded) return TSG_E_STATE;
    if (which < TSG_ADVECT_FULL || which > TSG_RK_FINAL) return TSG_E_ARG;
    if ((which == TSG_ADVECT_POS || which == TSG_ADVECT_SOMETHING) && !h->sorted) return TSG_E_STATE;
    cudaStream_t s = S(stream);
    if (use_fp32(h)) {
        fp32_advect(*h->f32, which, s);
    } else {
        if (which == TSG_ADVECT_POS) refresh_pos32_if_dirty(h, s);
        fp64_advect(h->c, h->cur, h->t, h->g, which, s);
        if (which == TSG_ADVECT_POS || which == TSG_ENFORCE_BOUNDARY) h->pos32_dirty = true;
    }
    return check_cuda();
}

static void rk_update(tsg_handle* h, int m, cudaStream_t s) {
    if (use_fp32(h)) fp32_rk_update(*h->f32, m, s);
    else fp64_rk_update(h->c, h->cur, h->t, m, s);
}

int tsg_rk_update(tsg_handle* h, int32_t m, void* stream) {
    if (!h || !h->uploaded) return TSG_E_STATE;
    if (m < 1 || m > 2) return TSG_E_ARG;
    rk_update(h, m, S(stream));
    return check_cuda();
}

int tsg_substep(tsg_handle* h, void* stream) {
    if (!h || !h->sorted) return TSG_E_STATE;
    int rc = 0;
    switch (h->c.ti) {
    case 1:
        rc = tsg_one_step(h, stream); if (rc) return rc;
        return tsg_advect(h, TSG_ADVECT_FULL, stream);
    case 2:
        rc = tsg_one_step(h, stream); if (rc) return rc;
        rc = tsg_advect(h, TSG_ADVECT_LF_HALF, stream); if (rc) return rc;
        rc = tsg_one_step(h, stream); if (rc) return rc;
        return tsg_advect(h, TSG_ADVECT_FULL, stream);
    case 4: {
        rc = tsg_advect(h, TSG_RK_INIT, stream); if (rc) return rc;
        const int m[4] = {1, 2, 2, 1};
        for (int k = 0; k < 4; ++k) {
            rc = tsg_one_step(h, stream); if (rc) return rc;
            rk_update(h, m[k], S(stream));
            if (k < 3) { rc = tsg_advect(h, TSG_RK_STAGE, stream); if (rc) return rc; }
        }
        return tsg_advect(h, TSG_RK_FINAL, stream);
    }
    default: return TSG_E_CONFIG;
    }
}

int tsg_step(tsg_handle* h, int nsteps, void* stream) {
    if (!h || !h->uploaded) return TSG_E_STATE;
    if (nsteps < 0) return TSG_E_ARG;
    const bool collide = h->c.boundary == 1;
    // FP32-mixed: replay captured step graphs (no host round trip per step) unless per-phase
    // profiling wants its events, which the eager path below records
    if (use_fp32(h) && !profiling_on() && nsteps > 0) {
        int rc = fp32_step_graph(*h->f32, nsteps, collide, S(stream));
        if (rc) return rc;
        h->sorted = true;
        return check_cuda();
    }
    for (int k = 0; k < nsteps; ++k) {
        int rc;
        // FP32-mixed with a neighbour skin re-sorts only when its lists expire
        if (!use_fp32(h) || fp32_rebuild_due(*h->f32, S(stream)))
            if ((rc = tsg_sort(h, stream))) return rc;
        if (use_fp32(h)) {  // the kernel sequence the captured graphs replay, launched eagerly
            fp32_step_body(*h->f32, collide, S(stream));
            if ((rc = check_cuda())) return rc;
            continue;
        }
        if ((rc = tsg_kernel_corr(h, stream))) return rc;
        if ((rc = tsg_init_tmp(h, stream))) return rc;
        if ((rc = tsg_substep(h, stream))) return rc;
        if ((rc = tsg_advect(h, TSG_ADVECT_POS, stream))) return rc;
        if ((rc = tsg_advect(h, TSG_ADVECT_SOMETHING, stream))) return rc;
        if (h->c.n_rigid_dyn && (rc = tsg_solve_rigid_body(h, stream))) return rc;
        // enforce_boundary also clamps dynamic rigid particles in every boundary mode
        if ((collide || h->c.n_rigid_dyn) && (rc = tsg_advect(h, TSG_ENFORCE_BOUNDARY, stream))) return rc;
    }
    return 0;
}

int tsg_field(tsg_handle* h, const char* name, tsg_view* out, void* stream) {
    if (!h || !name || !out || !h->uploaded) return TSG_E_ARG;
    std::memset(out, 0, sizeof *out);
    if (use_fp32(h)) return fp32_field(*h->f32, name, out, S(stream));
    const int64_t n = h->n;
    const std::string f(name);
    const Persist64& p = h->cur;
    const Trans64& t = h->t;
    void* ptr = nullptr;
    int comps = 1, dtype = 0;
    if (f == "x") { ptr = p.x; comps = 3; }
    else if (f == "v") { ptr = p.v; comps = 3; }
    else if (f == "x0") { ptr = p.x0; comps = 3; }
    else if (f == "density") ptr = p.density;
    else if (f == "mass") ptr = p.mass;
    else if (f == "m_V") ptr = p.m_V;
    else if (f == "pressure") ptr = p.pressure;
    else if (f == "stress") { ptr = p.stress; comps = 9; }
    else if (f == "strain_equ") ptr = p.strain_equ;
    else if (f == "strain_equ_p") ptr = p.strain_equ_p;
    else if (f == "flag_retmap") { ptr = p.flag_retmap; dtype = 2; }
    else if (f == "mat_type") { ptr = p.mat_type; dtype = 2; }
    else if (f == "mat_id") { ptr = p.mat_id; dtype = 2; }
    else if (f == "obj_id") { ptr = p.obj_id; dtype = 2; }
    else if (f == "is_dynamic") { ptr = p.is_dynamic; dtype = 2; }
    else if (f == "id0") { ptr = p.id0; dtype = 2; }
    else if (f == "v_tmp") { ptr = t.v_tmp; comps = 3; }
    else if (f == "density_tmp") ptr = t.density_tmp;
    else if (f == "stress_tmp") { ptr = t.stress_tmp; comps = 9; }
    else if (f == "d_density") ptr = t.d_density;
    else if (f == "d_vel") { ptr = t.d_vel; comps = 3; }
    else if (f == "d_stress") { ptr = t.d_stress; comps = 9; }
    else if (f == "v_grad") { ptr = t.v_grad; comps = 9; }
    else if (f == "CSPM_f") ptr = t.CSPM_f;
    else if (f == "CSPM_L") { ptr = t.CSPM_L; comps = 9; }
    else if (f == "d_strain_equ") ptr = t.d_strain_equ;
    else if (f == "d_strain_equ_p") ptr = t.d_strain_equ_p;
    else return TSG_E_NAME;
    if (!ptr) return TSG_E_NAME;
    out->data = ptr;
    out->dtype = dtype;
    if (comps == 1) { out->ndim = 1; out->shape[0] = n; out->strides[0] = 1; }
    else if (comps == 3) { out->ndim = 2; out->shape[0] = n; out->shape[1] = 3; out->strides[0] = 1; out->strides[1] = n; }
    else {
        out->ndim = 3; out->shape[0] = n; out->shape[1] = 3; out->shape[2] = 3;
        out->strides[0] = 1; out->strides[1] = 3 * n; out->strides[2] = n;
    }
    return 0;
}

namespace {

__global__ void k_interleave(const double* __restrict__ src, double* __restrict__ dst, int n, int k) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int q = 0; q < k; ++q) dst[(size_t)i * k + q] = src[(size_t)q * n + i];
}

// Planar device field behind a name for tsg_write / tsg_read (FP64 form).
int planar_field(tsg_handle* h, const std::string& f, void** ptr, int* comps, int* is_int) {
    tsg_view v;
    int rc = tsg_field(h, f.c_str(), &v, nullptr);
    if (rc) return rc;
    *ptr = v.data;
    *comps = v.ndim == 1 ? 1 : (v.ndim == 2 ? 3 : 9);
    *is_int = v.dtype == 2;
    return 0;
}

}  // namespace

int tsg_write(tsg_handle* h, const char* name, const void* src, int from_device, void* stream) {
    if (!h || !name || !src || !h->uploaded) return TSG_E_ARG;
    cudaStream_t s = S(stream);
    if (use_fp32(h)) return fp32_write(*h->f32, name, src, from_device != 0, s);
    void* ptr;
    int comps, is_int;
    int rc = planar_field(h, name, &ptr, &comps, &is_int);
    if (rc) return rc;
    const size_t n = h->n;
    if (is_int) {
        cudaMemcpyAsync(ptr, src, sizeof(int) * n, from_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s);
    } else {
        upload_planes(h, static_cast<const double*>(src), static_cast<double*>(ptr), comps, from_device != 0, s);
    }
    if (std::string(name) == "x") h->pos32_dirty = true;
    return check_cuda();
}

int tsg_read_fields(tsg_handle* h, int count, const char* const* names, void* const* dsts, int to_device,
                    void* stream) {
    if (!h || !names || !dsts || count <= 0 || !h->uploaded) return TSG_E_ARG;
    if (to_device < 0 || to_device > 2) return TSG_E_ARG;
    cudaStream_t s = S(stream);
    if (use_fp32(h)) return fp32_read_set(*h->f32, count, names, dsts, to_device, s);
    for (int q = 0; q < count; ++q) {
        const int rc = tsg_read(h, names[q], dsts[q], to_device == 0 ? 2 : to_device, stream);
        if (rc) return rc;
    }
    if (to_device == 0) cudaStreamSynchronize(s);
    return check_cuda();
}

int tsg_read(tsg_handle* h, const char* name, void* dst, int to_device, void* stream) {
    if (!h || !name || !dst || !h->uploaded) return TSG_E_ARG;
    cudaStream_t s = S(stream);
    if (to_device < 0 || to_device > 2) return TSG_E_ARG;
    if (use_fp32(h)) return fp32_read(*h->f32, name, dst, to_device, s);
    void* ptr;
    int comps, is_int;
    int rc = planar_field(h, name, &ptr, &comps, &is_int);
    if (rc) return rc;
    const size_t n = h->n;
    const cudaMemcpyKind kind = to_device == 1 ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (is_int) {
        cudaMemcpyAsync(dst, ptr, sizeof(int) * n, kind, s);
    } else if (comps == 1) {
        cudaMemcpyAsync(dst, ptr, sizeof(double) * n, kind, s);
    } else {
        TSG_LAUNCH(k_interleave, nb256(n), 256, s, static_cast<const double*>(ptr), h->d_stage, (int)n, comps);
        cudaMemcpyAsync(dst, h->d_stage, sizeof(double) * n * comps, kind, s);
    }
    if (to_device == 0) cudaStreamSynchronize(s);
    return check_cuda();
}

int64_t tsg_launch_count(void) { return tsg::g_launches.load(); }

int tsg_profile(int enable) {
    tsg::g_prof.on = enable != 0;
    return 0;
}

int tsg_profile_read(double* ms, int64_t* counts, int nphase) {
    if (!ms || !counts || nphase <= 0) return TSG_E_ARG;
    for (int k = 0; k < nphase; ++k) { ms[k] = 0.0; counts[k] = 0; }
    cudaDeviceSynchronize();
    for (auto& r : tsg::g_prof.recs) {
        float t = 0.f;
        cudaEventElapsedTime(&t, r.a, r.b);
        if (r.phase < nphase) { ms[r.phase] += t; counts[r.phase] += 1; }
        tsg::g_prof.pool.push_back(r.a);
        tsg::g_prof.pool.push_back(r.b);
    }
    tsg::g_prof.recs.clear();
    return check_cuda();
}

int tsg_grid(tsg_handle* h, int32_t* out, void* stream) {
    if (!h || !out || !h->sorted) return TSG_E_STATE;
    if (use_fp32(h)) return TSG_E_UNSUPPORTED;  // the FP32-mixed form keeps its own cell tables
    cudaStream_t s = S(stream);
    const int* cs = h->g.cell_start;
    cudaMemcpyAsync(out, cs + 1, sizeof(int32_t) * (h->c.G + 1), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    return check_cuda();
}

int tsg_neighbors(tsg_handle* h, int32_t* counts, int32_t* list, int64_t cap, int64_t* total, void* stream) {
    if (!h || !counts || !total || !h->sorted) return TSG_E_STATE;
    cudaStream_t s = S(stream);
    const int n = h->n;
    int* d_counts = nullptr;
    int* d_off = nullptr;
    if (cudaMalloc(&d_counts, sizeof(int) * (n + 1)) != cudaSuccess) return TSG_E_CUDA;
    if (cudaMalloc(&d_off, sizeof(int) * (n + 2)) != cudaSuccess) { cudaFree(d_counts); return TSG_E_CUDA; }
    int* tiles = nullptr;
    cudaMalloc(&tiles, sizeof(int) * (n / 2048 + 4));
    if (use_fp32(h)) fp32_neighbors(*h->f32, d_counts, nullptr, nullptr, s);
    else { refresh_pos32_if_dirty(h, s); fp64_neighbors(h->c, h->cur, h->t, h->g, d_counts, nullptr, nullptr, s); }
    scan_exclusive(d_counts, d_off, n, tiles, s);
    int tot = 0;
    cudaMemcpyAsync(counts, d_counts, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&tot, d_off + n, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    *total = tot;
    int rc = 0;
    if (list) {
        if (cap < tot) rc = TSG_E_CAPACITY;
        else {
            int* d_list = nullptr;
            if (cudaMalloc(&d_list, sizeof(int) * ((size_t)tot + 1)) != cudaSuccess) rc = TSG_E_CUDA;
            else {
                if (use_fp32(h)) fp32_neighbors(*h->f32, d_counts, d_off, d_list, s);
                else fp64_neighbors(h->c, h->cur, h->t, h->g, d_counts, d_off, d_list, s);
                cudaMemcpyAsync(list, d_list, sizeof(int) * (size_t)tot, cudaMemcpyDeviceToHost, s);
                cudaStreamSynchronize(s);
                cudaFree(d_list);
            }
        }
    }
    cudaFree(d_counts);
    cudaFree(d_off);
    cudaFree(tiles);
    int e = check_cuda();
    return rc ? rc : e;
}

int tsg_solve_rigid_body(tsg_handle* h, void* stream) {
    if (!h || !h->uploaded) return TSG_E_STATE;
    if (!h->c.n_rigid_dyn) return 0;  // no dynamic rigid body: nothing to solve
    if (use_fp32(h)) {
        fp32_solve_rigid(*h->f32, S(stream));
    } else {
        fp64_solve_rigid(h->c, h->cur, h->rigid, S(stream));
        h->pos32_dirty = true;
    }
    return check_cuda();
}

int tsg_density_sum(tsg_handle* h, double* out, void* stream) {
    if (!h || !h->sorted) return TSG_E_STATE;
    if (!out) return TSG_E_ARG;
    cudaStream_t s = S(stream);
    if (use_fp32(h)) fp32_density_sum(*h->f32, out, s);
    else { refresh_pos32_if_dirty(h, s); fp64_density_sum(h->c, h->cur, h->t, h->g, out, s); }
    return check_cuda();
}

int tsg_reduce_diag(tsg_handle* h, double out[8], void* stream) {
    if (!h || !out || !h->uploaded) return TSG_E_STATE;
    cudaStream_t s = S(stream);
    if (use_fp32(h)) fp32_diag(*h->f32, h->d_scratch ? h->d_scratch : nullptr, out, s);
    else {
        fp64_diag(h->c, h->cur, h->d_scratch, s);
        cudaMemcpyAsync(out, h->d_scratch, sizeof(double) * 8, cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
    }
    return check_cuda();
}

int tsg_list_stats(tsg_handle* h, int64_t out[5], void* stream) {
    if (!h || !out || !h->uploaded) return TSG_E_STATE;
    if (!use_fp32(h)) return TSG_E_UNSUPPORTED;
    int rc = fp32_list_stats(*h->f32, out, S(stream));
    if (rc) return rc;
    return check_cuda();
}

int tsg_last_error(tsg_handle* h, void* stream) {
    if (!h || !h->uploaded) return TSG_E_STATE;
    cudaStream_t s = S(stream);
    int* err = use_fp32(h) ? fp32_err_ptr(*h->f32) : h->g.err;
    int v = 0;
    cudaMemcpyAsync(&v, err, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemsetAsync(err, 0, sizeof(int), s);
    cudaStreamSynchronize(s);
    int e = check_cuda();
    return e ? e : v;
}

int tsg_visual(tsg_handle* h, const tsg_visual_cfg* vc, float* pos, float* color, double* range_out, void* stream) {
    if (!h || !vc || !pos || !color || !h->uploaded) return TSG_E_ARG;
    static const int titles[] = {1, 2, 21, 3, 31, 32, 33, 34, 35, 36, 37, 4, 41, 42, 43, 44,
                                 51, 52, 53, 54, 55, 56, 57, 61, 62, 7, 8, 102, 103};
    bool known = false;
    for (int t : titles) known = known || t == vc->color_title;
    if (!known || vc->color_group < 0 || vc->color_group > 2) return TSG_E_ARG;
    cudaStream_t s = S(stream);
    auto view = [&](const char* name, bool needed, const void** out) -> int {
        *out = nullptr;
        if (!needed) return 0;
        tsg_view v;
        int rc = tsg_field(h, name, &v, stream);
        if (rc == TSG_E_NAME) return TSG_E_UNSUPPORTED;
        if (rc) return rc;
        *out = v.data;
        return 0;
    };
    const int t = vc->color_title;
    VisFields f{};
    f.n = h->n;
    int rc = 0;
    const void* q = nullptr;
    if ((rc = view("x", true, &q))) return rc; f.x = static_cast<const double*>(q);
    if ((rc = view("id0", true, &q))) return rc; f.id0 = static_cast<const int*>(q);
    if ((rc = view("mat_type", true, &q))) return rc; f.mat_type = static_cast<const int*>(q);
    if ((rc = view("x0", t == 44, &q))) return rc; f.x0 = static_cast<const double*>(q);
    if ((rc = view("v", t == 3 || (t >= 31 && t <= 33), &q))) return rc; f.v = static_cast<const double*>(q);
    if ((rc = view("d_vel", t >= 34 && t <= 37, &q))) return rc; f.d_vel = static_cast<const double*>(q);
    if ((rc = view("v_tmp", t == 103, &q))) return rc; f.v_tmp = static_cast<const double*>(q);
    if ((rc = view("density", t == 2, &q))) return rc; f.density = static_cast<const double*>(q);
    if ((rc = view("d_density", t == 21, &q))) return rc; f.d_density = static_cast<const double*>(q);
    if ((rc = view("pressure", t == 7, &q))) return rc; f.pressure = static_cast<const double*>(q);
    if ((rc = view("stress", t >= 51 && t <= 57, &q))) return rc; f.stress = static_cast<const double*>(q);
    if ((rc = view("strain_equ", t == 61, &q))) return rc; f.strain_equ = static_cast<const double*>(q);
    if ((rc = view("strain_equ_p", t == 62, &q))) return rc; f.strain_equ_p = static_cast<const double*>(q);
    if ((rc = view("flag_retmap", t == 8, &q))) return rc; f.flag = static_cast<const int*>(q);
    if ((rc = view("CSPM_L", t == 102, &q))) return rc; f.CSPM_L = static_cast<const double*>(q);
    double* scratch = nullptr;
    if (cudaMalloc(&scratch, sizeof(double) * ((size_t)h->n + 2)) != cudaSuccess) return TSG_E_CUDA;
    rc = visual_launch(f, *vc, scratch, pos, color, range_out, s);
    cudaStreamSynchronize(s);
    cudaFree(scratch);
    return rc ? rc : check_cuda();
}

int tsg_set_soil(tsg_handle* h, double friction, double cohesion) {
    if (!h) return TSG_E_ARG;
    Consts& c = h->c;
    if (c.solver != 2 && c.solver != 3) return TSG_E_UNSUPPORTED;
    h->cfg.friction = friction;
    h->cfg.cohesion = cohesion;
    c.coh = cohesion;
    if (c.solver == 2) {
        c.mu = std::tan(friction);
    } else {  // the DP constructor's constants (eng/solver_sph_dp.py:20-27)
        double tf = std::tan(friction);
        double den = std::sqrt(9 + 12 * std::pow(tf, 2.0));
        c.alpha = tf / den;
        c.k_c = 3 * cohesion / den;
        c.kc_over_alpha = c.k_c / c.alpha;
        c.lam_den = 27.0 * c.alpha * c.Km * c.sin_dila + c.Gm;
        c.three_aK = 3.0 * c.alpha * c.Km;
    }
    if (use_fp32(h)) fp32_set_soil(*h->f32, c);
    return 0;
}

int tsg_set_fluid(tsg_handle* h, double stiffness, double viscosity) {
    if (!h) return TSG_E_ARG;
    Consts& c = h->c;
    if (c.solver != 1 || h->nscenes > 0) return TSG_E_UNSUPPORTED;
    h->cfg.stiffness = stiffness;
    h->cfg.viscosity = viscosity;
    c.B = stiffness;
    c.visc_fac = 2 * (c.dim + 2) * viscosity;
    if (use_fp32(h)) fp32_set_fluid(*h->f32, c);
    return 0;
}

int64_t tsg_snapshot_bytes(tsg_handle* h) {
    if (!h || !h->uploaded || !use_fp32(h)) return 0;
    return (int64_t)fp32_snapshot_bytes(*h->f32);
}

int tsg_snapshot_save(tsg_handle* h, void* dst, void* stream) {
    if (!h || !h->uploaded) return TSG_E_STATE;
    if (!use_fp32(h)) return TSG_E_UNSUPPORTED;
    return fp32_snapshot_copy(*h->f32, dst, false, S(stream));
}

int tsg_snapshot_load(tsg_handle* h, const void* src, void* stream) {
    if (!h || !h->uploaded) return TSG_E_STATE;
    if (!use_fp32(h)) return TSG_E_UNSUPPORTED;
    return fp32_snapshot_copy(*h->f32, const_cast<void*>(src), true, S(stream));
}

int tsg_adjoint_step(tsg_handle* h, double* adj_x, double* adj_v, double* adj_density, double* adj_v_tmp,
                     double* adj_params, void* stream) {
    if (!h || !h->uploaded) return TSG_E_STATE;
    if (!adj_x || !adj_v || !adj_density || !adj_v_tmp || !adj_params) return TSG_E_ARG;
    if (!use_fp32(h)) return TSG_E_UNSUPPORTED;
    int rc = fp32_adjoint_step(*h->f32, adj_x, adj_v, adj_density, adj_v_tmp, adj_params, S(stream));
    if (rc) return rc;
    h->sorted = true;
    return check_cuda();
}

int tsg_set_launch(tsg_handle* h, const tsg_launch_cfg* cfg) {
    if (!h || !cfg) return TSG_E_ARG;
    if (!use_fp32(h)) return TSG_E_UNSUPPORTED;
    return fp32_set_launch(*h->f32, cfg->threads_per_block, cfg->cells_per_cta, cfg->steps_per_graph);
}

int tsg_get_launch(tsg_handle* h, tsg_launch_cfg* cfg) {
    if (!h || !cfg) return TSG_E_ARG;
    if (!use_fp32(h)) return TSG_E_UNSUPPORTED;
    fp32_get_launch(*h->f32, &cfg->threads_per_block, &cfg->cells_per_cta, &cfg->steps_per_graph);
    return 0;
}

int tsg_autotune(tsg_handle* h, int32_t trial_steps, tsg_launch_cfg* best, double* ms_per_step, void* stream) {
    if (!h || !h->uploaded) return TSG_E_STATE;
    if (!use_fp32(h)) return TSG_E_UNSUPPORTED;
    float ms = 0.f;
    int rc = fp32_autotune(*h->f32, trial_steps, h->c.boundary == 1, S(stream), &ms);
    if (rc) return rc;
    h->sorted = true;
    if (best) fp32_get_launch(*h->f32, &best->threads_per_block, &best->cells_per_cta, &best->steps_per_graph);
    if (ms_per_step) *ms_per_step = ms;
    return check_cuda();
}

int tsg_batch_create(const tsg_config* cfgs, const tsg_particles* parts, int32_t nscenes, void* stream,
                     tsg_handle** out) {
    if (!cfgs || !parts || !out || nscenes <= 0) return TSG_E_ARG;
    *out = nullptr;
    if (nscenes > 4096) return TSG_E_CAPACITY;
    const tsg_config& a = cfgs[0];
    if (a.precision != TSG_FP32_MIXED || a.solver != 1 || a.boundary != 2) return TSG_E_UNSUPPORTED;
    // every scene shares the geometry, the kernel and the integrator; stiffness and
    // viscosity may differ per scene
    for (int q = 1; q < nscenes; ++q) {
        const tsg_config& b = cfgs[q];
        bool same = b.dim == a.dim && b.solver == a.solver && b.kernel == a.kernel && b.kernel_corr == a.kernel_corr &&
                    b.time_integration == a.time_integration && b.xsph == a.xsph && b.boundary == a.boundary &&
                    b.precision == a.precision && b.exponent_is_int == a.exponent_is_int &&
                    b.grid_num_total == a.grid_num_total && b.grid_size == a.grid_size &&
                    b.support_radius == a.support_radius && b.smoothing_len == a.smoothing_len &&
                    b.particle_diameter == a.particle_diameter && b.particle_radius == a.particle_radius &&
                    b.dt == a.dt && b.density0 == a.density0 && b.exponent == a.exponent && b.list_skin == a.list_skin;
        for (int d = 0; d < 3; ++d)
            same = same && b.grid_num[d] == a.grid_num[d] && b.vdomain_start[d] == a.vdomain_start[d] &&
                   b.domain_start[d] == a.domain_start[d] && b.domain_end[d] == a.domain_end[d] &&
                   b.gravity[d] == a.gravity[d];
        if (!same) return TSG_E_CONFIG;
    }
    // scenes side by side along x, two reference cells apart beyond their virtual domains:
    // particles of different scenes are then farther apart than the support plus the skin
    const int pitch_cells = a.grid_num[0] + 2;
    const double pitch = pitch_cells * a.grid_size;
    tsg_config t = a;
    t.grid_num[0] = pitch_cells * nscenes;
    t.grid_num_total = (int64_t)t.grid_num[0] * t.grid_num[1] * t.grid_num[2];
    t.domain_end[0] = a.domain_end[0] + (nscenes - 1) * pitch;
    if (t.grid_num_total > (1ll << 30)) return TSG_E_CAPACITY;
    int64_t n = 0;
    for (int q = 0; q < nscenes; ++q) {
        const tsg_particles& p = parts[q];
        if (p.n <= 0 || !p.x || !p.v || !p.density || !p.mass || !p.m_V || !p.pressure || !p.mat_type || !p.mat_id ||
            !p.obj_id || !p.is_dynamic)
            return TSG_E_ARG;
        n += p.n;
    }
    if (n > (1ll << 30)) return TSG_E_CAPACITY;
    std::vector<double> x(3 * n), v(3 * n), rho(n), mass(n), mV(n), pr(n);
    std::vector<int32_t> mt(n), mid(n), oid(n), dyn(n), scene(n);
    std::vector<float> stiff(nscenes), vfac(nscenes);
    int64_t o = 0;
    for (int q = 0; q < nscenes; ++q) {
        const tsg_particles& p = parts[q];
        for (int64_t i = 0; i < p.n; ++i, ++o) {
            for (int d = 0; d < 3; ++d) {
                x[3 * o + d] = p.x[3 * i + d] + (d == 0 ? q * pitch : 0.0);
                v[3 * o + d] = p.v[3 * i + d];
            }
            rho[o] = p.density[i]; mass[o] = p.mass[i]; mV[o] = p.m_V[i]; pr[o] = p.pressure[i];
            mt[o] = p.mat_type[i]; mid[o] = p.mat_id[i]; oid[o] = p.obj_id[i]; dyn[o] = p.is_dynamic[i];
            scene[o] = q;
        }
        stiff[q] = (float)cfgs[q].stiffness;
        vfac[q] = (float)(2 * (a.dim + 2) * cfgs[q].viscosity);
    }
    tsg_handle* h = nullptr;
    int rc = tsg_create(&t, &h);
    if (rc) return rc;
    tsg_particles all{};
    all.n = n;
    all.x = x.data(); all.v = v.data(); all.density = rho.data(); all.mass = mass.data(); all.m_V = mV.data();
    all.pressure = pr.data(); all.stress = nullptr;
    all.mat_type = mt.data(); all.mat_id = mid.data(); all.obj_id = oid.data(); all.is_dynamic = dyn.data();
    Fp32Scenes sc;
    sc.scene_of = scene.data();
    sc.stiffness = stiff.data();
    sc.visc_fac = vfac.data();
    sc.nscenes = nscenes;
    rc = upload_impl(h, &all, 0, stream, &sc);
    if (rc) { tsg_destroy(h); return rc; }
    h->batch_pitch = pitch;
    h->nscenes = nscenes;
    *out = h;
    return 0;
}

int tsg_batch_diag(tsg_handle* h, double* out, int32_t nscenes, void* stream) {
    if (!h || !out || !h->uploaded) return TSG_E_STATE;
    if (!use_fp32(h) || h->nscenes <= 0) return TSG_E_UNSUPPORTED;
    int rc = fp32_batch_diag(*h->f32, h->batch_pitch, out, nscenes, S(stream));
    return rc ? rc : check_cuda();
}

double tsg_batch_pitch(const tsg_handle* h) { return h ? h->batch_pitch : 0.0; }

void tsg_destroy(tsg_handle* h) {
    if (!h) return;
    cudaDeviceSynchronize();
    if (h->f32) fp32_destroy(h->f32);
    for (void* p : h->allocs) cudaFree(p);
    delete h;
}

}  // extern "C"
