// FP64 form of the per-substep SPH path (the "plain FP64" GPU form).
//
// Every arithmetic expression follows the reference's evaluation order (Python/Taichi
// left-to-right; sums over neighbours in for_all_neighbors order, eng/particle_system.py:
// 259-269), and this file is compiled with -fmad=false, so with IEEE f64 division and
// square root the results are bit-identical to the f64 CPU oracle.  Constant powers are
// products: q1^4 = (q1*q1)*(q1*q1), q1^3 = (q1*q1)*q1, x**2 = x*x.
//
// Kernels (one thread per particle; boundary / flow particles through index lists):
//   k_corr        Shepard factor for all particles, CSPM matrix for flow particles
//                 (eng/solver_sph_base.py:386-423), one neighbour traversal.
//   k_init_tmp    init_real2tmp (eng/solver_sph_base.py:67-74).
//   k_pre         per-particle first phase of one_step: Tait EOS (WC,
//                 eng/solver_sph_wc.py:86-88) or stress adaptation (DP,
//                 eng/solver_sph_dp.py:215-217).
//   k_bdy         dummy-boundary extrapolation of v_tmp, density_tmp, pressure / stress
//                 (eng/solver_sph_wc.py:90-103, eng/solver_sph_muI.py:97-109,
//                 eng/solver_sph_dp.py:219-234), all sums in one traversal.
//   k_wc_rates    continuity + momentum (eng/solver_sph_wc.py:108-126), one traversal.
//   k_mui_stress  mu(I) velocity gradient, continuity, stress (eng/solver_sph_muI.py:67-92).
//   k_mui_mom     mu(I) stress divergence + damping (eng/solver_sph_muI.py:113-128).
//   k_dp_rates    DP velocity gradient, continuity, Bui-2008 stress rate, stress
//                 divergence, damping (eng/solver_sph_dp.py:236-270), one traversal.
//   advection / post-step kernels (eng/solver_sph_base.py:79-247, solver overrides).
#include <cfloat>

#include "tsg_internal.h"
#include "tsg_polar.cuh"
#include "tsg_rigid_list.cuh"

namespace tsg {

namespace {

constexpr int TPB = 128;

inline int nblk(long long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

// ---- kernel functions (eng/solver_sph_base.py:299-358) ----
// W and |grad W| factor from the precomputed norm rn; dW_c = s * r_c / rn (Wendland) or
// s * (r_c / rn * h1) (cubic), matching the reference's expression trees.
__device__ __forceinline__ double kernel_W(const Consts& c, double rn) {
    double res = 0.0;
    double q = rn * c.h1;
    if (rn > EPS && q <= 2.0) {
        if (c.kernel == 1) {
            double q1 = 1.0 - 0.5 * q;
            res = c.kk * ((q1 * q1) * (q1 * q1)) * (1.0 + 2.0 * q);
        } else if (q <= 1.0) {
            double q2 = q * q, q3 = q2 * q;
            res = c.kk * (0.5 * q3 - q2 + 2.0 / 3.0);
        } else {
            double t = 2.0 - q;
            res = c.kk / 6.0 * ((t * t) * t);
        }
    }
    return res;
}

template <int DIM>
__device__ __forceinline__ void kernel_dW(const Consts& c, const double* r, double rn, double* out) {
    out[0] = out[1] = out[2] = 0.0;
    double q = rn * c.h1;
    if (rn > EPS && q <= 2.0) {
        if (c.kernel == 1) {
            double q1 = 1.0 - 0.5 * q;
            double s = c.kk * ((q1 * q1) * q1) * (-5.0 * q) * c.h1;
            for (int d = 0; d < DIM; ++d) out[d] = s * r[d] / rn;
        } else {
            double s;
            if (q <= 1.0) s = c.kk * q * (1.5 * q - 2.0);
            else { double f = 2.0 - q; s = c.kk * (-0.5 * f * f); }
            for (int d = 0; d < DIM; ++d) out[d] = s * (r[d] / rn * c.h1);
        }
    }
}

template <int DIM>
__device__ __forceinline__ void matvec_corr(const double* L, const double* k, double* out) {
    for (int p = 0; p < DIM; ++p) {
        double s = L[3 * p] * k[0] + L[3 * p + 1] * k[1];
        if (DIM == 3) s = s + L[3 * p + 2] * k[2];
        out[p] = s;
    }
    if (DIM == 2) out[2] = 0.0;
}

template <int DIM>
__device__ __forceinline__ double dotv(const double* a, const double* b) {
    double s = a[0] * b[0] + a[1] * b[1];
    if (DIM == 3) s = s + a[2] * b[2];
    return s;
}

// ---- neighbour traversal (eng/particle_system.py:259-269) ----
// Visits the 3^dim cells around the centre's cell in ndrange order (z fastest); the three
// cells of one row have consecutive flattened indices, so each row is one contiguous index
// range (the reference's flattening, aliasing included).  Rows are clipped to [0, G).
// A candidate is a neighbour when j != i and sqrt(|x_i - x_j|^2) < support_radius in f64;
// the f32 prefilter only rejects candidates that are certainly farther away.
template <int DIM, class F>
__device__ __forceinline__ void for_neighbors(const Consts& c, const double* __restrict__ X,
                                              const float4* __restrict__ P32, const int* __restrict__ cs,
                                              int i, const double* xi, bool prefilter, F&& body) {
    const int n = c.n;
    long long cc[3];
    for (int d = 0; d < 3; ++d) {
        double t = (xi[d] - c.vs[d]) / c.grid;
        if (!(fabs(t) < 2147483647.0)) return;
        cc[d] = (int)t;
    }
    const long long ny = c.gnum[1], nz = c.gnum[2], G = c.G;
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    bool pf = prefilter && c.pf_on;
    if (pf) {
        pi = P32[i];
        pf = fabsf(pi.x) < c.pf_lim && fabsf(pi.y) < c.pf_lim && fabsf(pi.z) < c.pf_lim;
    }
#pragma unroll 1
    for (int ox = -1; ox <= 1; ++ox) {
#pragma unroll 1
        for (int oy = (DIM == 3 ? -1 : 0); oy <= (DIM == 3 ? 1 : 0); ++oy) {
            long long f0 = (cc[0] + ox) * ny * nz + (cc[1] + oy) * nz + cc[2];
            long long lo = f0 - 1 > 0 ? f0 - 1 : 0;
            long long hi = f0 + 1 < G - 1 ? f0 + 1 : G - 1;
            if (lo > hi) continue;
            const int jb = cs[lo], je = cs[hi + 1];
#pragma unroll 1
            for (int j = jb; j < je; ++j) {
                if (j == i) continue;
                if (pf) {
                    float4 pj = P32[j];
                    float fx = pi.x - pj.x, fy = pi.y - pj.y, fz = pi.z - pj.z;
                    float r2f = fx * fx + fy * fy;
                    if (DIM == 3) r2f += fz * fz;
                    if (r2f > c.pf_r2) continue;
                }
                double r[3];
                r[0] = xi[0] - X[j];
                r[1] = xi[1] - X[(size_t)n + j];
                r[2] = DIM == 3 ? xi[2] - X[2 * (size_t)n + j] : 0.0;
                double r2 = r[0] * r[0] + r[1] * r[1];
                if (DIM == 3) r2 = r2 + r[2] * r[2];
                double rn = sqrt(r2);
                if (!(rn < c.R)) continue;
                body(j, r, rn);
            }
        }
    }
}

template <int DIM>
__device__ __forceinline__ void load_x(const double* X, int i, int n, double* xi) {
    xi[0] = X[i];
    xi[1] = X[(size_t)n + i];
    xi[2] = DIM == 3 ? X[2 * (size_t)n + i] : X[2 * (size_t)n + i];
}

__device__ __forceinline__ bool is_flow(int t) { return t == MAT_FLUID || t == MAT_SOIL; }

// ---- CSPM (eng/solver_sph_base.py:386-423) ----
__device__ __forceinline__ double det2(const double* a) { return a[0] * a[4] - a[1] * a[3]; }
__device__ __forceinline__ double det3(const double* a) {
    return a[0] * (a[4] * a[8] - a[7] * a[5]) - a[3] * (a[1] * a[8] - a[7] * a[2]) + a[6] * (a[1] * a[5] - a[4] * a[2]);
}

template <int DIM>
__global__ void k_corr(Consts c, Persist64 p, Trans64 t, const int* __restrict__ cs) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int n = c.n;
    double xi[3];
    load_x<DIM>(p.x, i, n, xi);
    const int ti = p.mat_type[i];
    const bool want_L = c.corr == 1 && is_flow(ti);
    double s = 0.0;
    double L[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for_neighbors<DIM>(c, p.x, t.pos32, cs, i, xi, true, [&](int j, const double* r, double rn) {
        const int tj = p.mat_type[j];
        const double mVj = p.m_V[j];
        if (is_flow(tj)) s += mVj * kernel_W(c, rn);
        if (want_L && tj == ti) {
            double k[3];
            kernel_dW<DIM>(c, r, rn, k);
            for (int a = 0; a < DIM; ++a) {
                double av = mVj * (-r[a]);
                for (int b = 0; b < DIM; ++b) L[3 * a + b] = L[3 * a + b] + av * k[b];
            }
        }
    });
    t.CSPM_f[i] = s != 0.0 ? 1.0 / s : 1.0;
    if (c.corr == 1) {
        double inv[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        if (want_L) {
            if (DIM == 2) {
                double dt = det2(L);
                if (fabs(dt) > EPS) {
                    double id = 1.0 / dt;
                    inv[0] = id * L[4]; inv[1] = id * (-L[1]); inv[2] = 0.0;
                    inv[3] = id * (-L[3]); inv[4] = id * L[0]; inv[5] = 0.0;
                    inv[6] = 0.0; inv[7] = 0.0; inv[8] = 0.0;
                }
            } else {
                double dt = det3(L);
                if (fabs(dt) > EPS) {
                    double id = 1.0 / dt;
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b)
                            inv[3 * b + a] = id * (L[3 * ((a + 1) % 3) + (b + 1) % 3] * L[3 * ((a + 2) % 3) + (b + 2) % 3]
                                                 - L[3 * ((a + 2) % 3) + (b + 1) % 3] * L[3 * ((a + 1) % 3) + (b + 2) % 3]);
                }
            }
        }
        for (int q = 0; q < 9; ++q) t.CSPM_L[(size_t)q * n + i] = inv[q];
    }
}

// Density summation: calc_density_task summed over for_all_neighbors
// (eng/solver_sph_wc.py:30-31, eng/particle_system.py:259-269), sum_j mass_j W(x_i - x_j)
// over the neighbours j != i of every particle, in traversal order.
template <int DIM>
__global__ void k_density_sum(Consts c, Persist64 p, Trans64 t, const int* __restrict__ cs, double* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    double xi[3];
    load_x<DIM>(p.x, i, c.n, xi);
    double ret = 0.0;
    for_neighbors<DIM>(c, p.x, t.pos32, cs, i, xi, true, [&](int j, const double*, double rn) {
        ret += p.mass[j] * kernel_W(c, rn);
    });
    out[i] = ret;
}

__global__ void k_init_tmp(Consts c, Persist64 p, Trans64 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int n = c.n;
    const int ti = p.mat_type[i];
    if (ti > 0) {
        t.density_tmp[i] = p.density[i];
        for (int d = 0; d < 3; ++d) t.v_tmp[(size_t)d * n + i] = p.v[(size_t)d * n + i];
    }
    if (ti == MAT_SOIL)
        for (int q = 0; q < 9; ++q) t.stress_tmp[(size_t)q * n + i] = p.stress[(size_t)q * n + i];
}

// ---- Drucker-Prager invariants and return mapping (eng/solver_sph_dp.py:42-109) ----
__device__ __forceinline__ double mtrace(const double* a) { return (a[0] + a[4]) + a[8]; }
__device__ __forceinline__ double msum_sq(const double* a) {
    double s = a[0] * a[0];
    for (int k = 1; k < 9; ++k) s = s + a[k] * a[k];
    return s;
}
__device__ __forceinline__ double msum_prod(const double* a, const double* b) {
    double s = a[0] * b[0];
    for (int k = 1; k < 9; ++k) s = s + a[k] * b[k];
    return s;
}
__device__ __forceinline__ void dp_inv(const Consts& c, const double* st, double* s, double& I1, double& sJ2, double& f) {
    double t3 = mtrace(st) / 3.0;
    for (int k = 0; k < 9; ++k) s[k] = st[k] - t3 * ((k % 4 == 0) ? 1.0 : 0.0);
    I1 = mtrace(st);
    sJ2 = sqrt(0.5 * msum_sq(s));
    f = sJ2 + c.alpha * I1 - c.k_c;
}
__device__ __forceinline__ void dp_adapt(const Consts& c, double* st) {
    double s[9], I1, sJ2, f;
    dp_inv(c, st, s, I1, sJ2, f);
    if (f > EPS_F) {
        if (f > sJ2) {
            double tt = (I1 - c.kc_over_alpha) / 3.0;
            for (int k = 0; k < 9; ++k) st[k] = st[k] - tt * ((k % 4 == 0) ? 1.0 : 0.0);
        }
        dp_inv(c, st, s, I1, sJ2, f);
        double r = (-I1 * c.alpha + c.k_c) / sJ2;
        for (int k = 0; k < 9; ++k) st[k] = r * s[k] + (((k % 4 == 0) ? 1.0 : 0.0) * I1) / 3.0;
    }
}
__device__ __forceinline__ int dp_flag(const Consts& c, const double* st) {
    double s[9], I1, sJ2, f;
    dp_inv(c, st, s, I1, sJ2, f);
    int flag = 1;
    if (f < -EPS_F) flag = 0;
    else if (f > EPS_F) flag = (f >= sJ2) ? 3 : 2;
    return flag;
}

__device__ __forceinline__ double powi(double x, long n) {
    double r = 1.0;
    bool first = true;
    while (n > 0) {
        if (n & 1) { r = first ? x : r * x; first = false; }
        n >>= 1;
        if (n) x = x * x;
    }
    return r;
}

// First, per-particle phase of one_step.
__global__ void k_pre(Consts c, Persist64 p, Trans64 t, const int* __restrict__ list, int count) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int i = list[k];
    const int n = c.n;
    if (c.solver == 1) {
        double ratio = t.density_tmp[i] / c.rho0;
        double pw = c.exponent_is_int ? powi(ratio, (long)c.gamma) : pow(ratio, c.gamma);
        p.pressure[i] = fmax(c.B * (pw - 1.0), 0.0);
    } else if (c.solver == 3) {
        double st[9];
        for (int q = 0; q < 9; ++q) st[q] = t.stress_tmp[(size_t)q * n + i];
        dp_adapt(c, st);
        for (int q = 0; q < 9; ++q) t.stress_tmp[(size_t)q * n + i] = st[q];
    }
}

// Dummy-boundary extrapolation (Adami 2012 style), one traversal for every sum.
template <int DIM>
__global__ void k_bdy(Consts c, Persist64 p, Trans64 t, const int* __restrict__ cs,
                      const int* __restrict__ list, int count) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int i = list[k];
    const int n = c.n;
    const int ti = p.mat_type[i];
    double xi[3];
    load_x<DIM>(p.x, i, n, xi);
    double bv[3] = {0, 0, 0};
    double bp = 0.0, bd = 0.0;
    double bs[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const bool soil = c.solver != 1;
    for_neighbors<DIM>(c, p.x, t.pos32, cs, i, xi, true, [&](int j, const double* r, double rn) {
        if (!is_flow(p.mat_type[j])) return;
        const double w = kernel_W(c, rn);
        const double mVj = p.m_V[j];
        for (int d = 0; d < DIM; ++d) bv[d] += mVj * t.v_tmp[(size_t)d * n + j] * w;
        const double rtj = t.density_tmp[j];
        if (!soil) {
            bp += mVj * (p.pressure[j] + rtj * c.g[1] * (xi[1] - p.x[(size_t)n + j])) * w;
        } else {
            if (c.solver == 2) bd += mVj * rtj * w;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    double m = t.stress_tmp[(size_t)(3 * a + b) * n + j];
                    if (a == b) m = m + (rtj * c.g[a]) * r[a];
                    else m = m + (rtj * 0.0) * 0.0;
                    bs[3 * a + b] += mVj * m * w;
                }
        }
    });
    const double f = t.CSPM_f[i];
    for (int d = 0; d < DIM; ++d) t.v_tmp[(size_t)d * n + i] = 2 * p.v[(size_t)d * n + i] - bv[d] * f;
    if (DIM == 2) t.v_tmp[2 * (size_t)n + i] = 2 * p.v[2 * (size_t)n + i] - 0.0 * f;
    if (!soil) {
        t.density_tmp[i] = c.rho0;
        p.pressure[i] = fmax(bp * f, 0.0);
    } else {
        t.density_tmp[i] = c.solver == 2 ? fmax(bd * f, c.rho0) : c.rho0;
        for (int q = 0; q < 9; ++q) t.stress_tmp[(size_t)q * n + i] = bs[q] * f;
    }
    if (ti == MAT_RIGID) {  // static rigid: rates stay zero; dynamic rigid: gravity, then the reaction
        t.d_density[i] = 0.0;
        const bool dyn = p.is_dynamic[i] != 0;
        for (int d = 0; d < 3; ++d) t.d_vel[(size_t)d * n + i] = dyn ? c.g[d] : 0.0;
    } else {
        // dummy / repulsive particles have no rates: zero, as in the reference, where each
        // particle's never-written rates travel with it through the sort (the rate arrays
        // here are not reordered, so a slot may hold another particle's)
        t.d_density[i] = 0.0;
        for (int d = 0; d < 3; ++d) t.d_vel[(size_t)d * n + i] = 0.0;
    }
}

// ---- repulsive particles (eng/solver_sph_base.py:675-689) ----
template <int DIM>
__device__ __forceinline__ void rep_force(const Consts& c, const double* r, double rn, double* acc) {
    double chi = (rn > 0.0 && rn < c.diam) ? 1.0 - rn / c.diam : 0.0;
    double gm = rn / c.h075;
    double f = 0.0;
    if (gm > 0 && gm <= 2.0 / 3.0) f = 2.0 / 3.0;
    else if (gm > 2.0 / 3.0 && gm <= 1) f = 2 * gm - 1.5 * (gm * gm);
    else if (gm > 1 && gm < 2) f = 0.5 * ((2 - gm) * (2 - gm));
    double s = c.rep_fac * chi * f / (rn * rn);
    for (int d = 0; d < DIM; ++d) acc[d] = acc[d] + s * r[d];
}

// One neighbour's term of calc_d_vel_task (eng/solver_sph_wc.py:34-71): viscosity
// (fluid, or boundary / rigid neighbours with the rho0 / rho~_i factor) plus pressure, for
// centre i and neighbour j of type tj; dvv = v~_i - v~_j, r = x_i - x_j, kd = grad W(r).
template <int DIM>
__device__ __forceinline__ void wc_force_pair(const Consts& c, int tj, double mVj, const double* dvv, double rti,
                                              double pri, double ptj, double rtj, const double* r, double rn,
                                              const double* kd, double* out) {
    const double mn = fmin(dotv<DIM>(dvv, r), 0.0);
    const double den = rn * rn + c.eps_h2;
    double cv = 0.0;
    bool visc = false;
    if (tj == MAT_FLUID) { cv = c.visc_fac * mVj * mn / den; visc = true; }
    else if (tj == MAT_DUMMY || tj == MAT_REP || tj == MAT_RIGID) {
        cv = c.visc_fac * mVj * c.rho0 / rti * mn / den; visc = true;
    }
    const double cp = -c.rho0 * mVj * (pri + ptj / (rtj * rtj));
    for (int d = 0; d < DIM; ++d) {
        double pv = cp * kd[d];
        out[d] = visc ? cv * kd[d] + pv : 0.0 + pv;
    }
}

// ---- WCSPH rates (eng/solver_sph_wc.py:108-126) ----
template <int DIM>
__global__ void k_wc_rates(Consts c, Persist64 p, Trans64 t, const int* __restrict__ cs,
                           const int* __restrict__ list, int count) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int i = list[k];
    const int n = c.n;
    double xi[3], vti[3];
    load_x<DIM>(p.x, i, n, xi);
    for (int d = 0; d < 3; ++d) vti[d] = t.v_tmp[(size_t)d * n + i];
    const double rti = t.density_tmp[i];
    const double pti = p.pressure[i];
    const double pri = pti / (rti * rti);
    double L[9];
    if (c.corr == 1)
        for (int q = 0; q < 9; ++q) L[q] = t.CSPM_L[(size_t)q * n + i];
    double dd = 0.0;
    double dv[3] = {0, 0, 0};
    const bool rep = c.boundary == 3 || c.boundary == 4;
    for_neighbors<DIM>(c, p.x, t.pos32, cs, i, xi, true, [&](int j, const double* r, double rn) {
        const int tj = p.mat_type[j];
        const double mVj = p.m_V[j];
        double vtj[3], dvv[3];
        for (int d = 0; d < DIM; ++d) { vtj[d] = t.v_tmp[(size_t)d * n + j]; dvv[d] = vti[d] - vtj[d]; }
        double kd[3];
        kernel_dW<DIM>(c, r, rn, kd);
        // continuity: m_Vj (v_i - v_j) . grad~W
        double a[3];
        for (int d = 0; d < DIM; ++d) a[d] = mVj * dvv[d];
        if (c.corr == 1) {
            double kc[3];
            matvec_corr<DIM>(L, kd, kc);
            dd += dotv<DIM>(a, kc);
        } else {
            dd += dotv<DIM>(a, kd);
        }
        double f[3];
        wc_force_pair<DIM>(c, tj, mVj, dvv, rti, pri, p.pressure[j], t.density_tmp[j], r, rn, kd, f);
        for (int d = 0; d < DIM; ++d) dv[d] += f[d];
    });
    if (rep) {  // separate traversal: the reference adds these after the whole dv sum
        for_neighbors<DIM>(c, p.x, t.pos32, cs, i, xi, true, [&](int j, const double* r, double rn) {
            if (p.mat_type[j] == MAT_REP) rep_force<DIM>(c, r, rn, dv);
        });
    }
    t.d_density[i] = dd * rti;
    for (int d = 0; d < DIM; ++d) t.d_vel[(size_t)d * n + i] = dv[d] + c.g[d];
    if (DIM == 2) t.d_vel[2 * (size_t)n + i] = 0.0 + c.g[2];
}

// ---- soil helpers ----
__device__ __forceinline__ void damping_acc(const Consts& c, double rti, const double* vti, double* out, int dim) {
    double s = -c.damp_eps * sqrt(c.damp_E / (rti * c.h2));
    for (int d = 0; d < dim; ++d) out[d] = s * vti[d];
}

// mu(I) loop 1 (eng/solver_sph_muI.py:67-92): velocity gradient, continuity, pressure from
// density (not density_tmp), mu(I) stress, equivalent strain rate.
template <int DIM>
__global__ void k_mui_stress(Consts c, Persist64 p, Trans64 t, const int* __restrict__ cs,
                             const int* __restrict__ list, int count) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int i = list[k];
    const int n = c.n;
    double xi[3], vti[3];
    load_x<DIM>(p.x, i, n, xi);
    for (int d = 0; d < 3; ++d) vti[d] = t.v_tmp[(size_t)d * n + i];
    double L[9];
    if (c.corr == 1)
        for (int q = 0; q < 9; ++q) L[q] = t.CSPM_L[(size_t)q * n + i];
    double vg[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double dd = 0.0;
    for_neighbors<DIM>(c, p.x, t.pos32, cs, i, xi, true, [&](int j, const double* r, double rn) {
        const double mVj = p.m_V[j];
        double kd[3], kc[3];
        kernel_dW<DIM>(c, r, rn, kd);
        if (c.corr == 1) matvec_corr<DIM>(L, kd, kc);
        else { kc[0] = kd[0]; kc[1] = kd[1]; kc[2] = kd[2]; }
        double vtj[3];
        for (int d = 0; d < DIM; ++d) vtj[d] = t.v_tmp[(size_t)d * n + j];
        for (int a = 0; a < DIM; ++a) {
            double av = mVj * (vtj[a] - vti[a]);
            for (int b = 0; b < DIM; ++b) vg[3 * a + b] += av * kc[b];
        }
        double aa[3];
        for (int d = 0; d < DIM; ++d) aa[d] = mVj * (vti[d] - vtj[d]);
        dd += dotv<DIM>(aa, kc);
    });
    const double rti = t.density_tmp[i];
    for (int q = 0; q < 9; ++q) t.v_grad[(size_t)q * n + i] = vg[q];
    t.d_density[i] = dd * rti;
    const double pr = fmax(c.vsound2 * (p.density[i] - c.rho0), 0.0);
    p.pressure[i] = pr;
    double er[9];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) er[3 * a + b] = 0.5 * (vg[3 * a + b] + vg[3 * b + a]);
    const double dbdot = sqrt(0.5 * msum_sq(er)) + EPS;
    const double sc = 0.0 + (c.coh + pr * c.mu) / dbdot;
    for (int q = 0; q < 9; ++q) t.stress_tmp[(size_t)q * n + i] = sc * er[q] - pr * ((q % 4 == 0) ? 1.0 : 0.0);
    const double t3 = mtrace(er) / 3.0;
    double ed[9];
    for (int q = 0; q < 9; ++q) ed[q] = er[q] - t3 * ((q % 4 == 0) ? 1.0 : 0.0);
    t.d_strain_equ[i] = sqrt(msum_sq(ed) * 2 / 3);
}

// Stress-divergence sum (eng/solver_sph_muI.py:39-46), shared by mu(I) and DP.
template <int DIM>
__device__ __forceinline__ void stress_div_val(const double* sti, double ri2, const double* stj, double rtj,
                                               double mVj, const double* kc, double* out) {
    const double rj2 = rtj * rtj;
    const double sc = mVj * rtj;
    for (int a = 0; a < DIM; ++a) {
        double s = 0.0;
        for (int b = 0; b < DIM; ++b) {
            double m = stj[3 * a + b] / rj2 + sti[3 * a + b] / ri2;
            double v = (sc * m) * kc[b];
            s = b == 0 ? v : s + v;
        }
        out[a] = s;
    }
}
template <int DIM>
__device__ __forceinline__ void stress_div_term(const double* sti, double ri2, const double* stj, double rtj,
                                                double mVj, const double* kc, double* acc) {
    double v[3];
    stress_div_val<DIM>(sti, ri2, stj, rtj, mVj, kc, v);
    for (int a = 0; a < DIM; ++a) acc[a] += v[a];
}

template <int DIM>
__global__ void k_mui_mom(Consts c, Persist64 p, Trans64 t, const int* __restrict__ cs,
                          const int* __restrict__ list, int count) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int i = list[k];
    const int n = c.n;
    double xi[3];
    load_x<DIM>(p.x, i, n, xi);
    double L[9], sti[9];
    if (c.corr == 1)
        for (int q = 0; q < 9; ++q) L[q] = t.CSPM_L[(size_t)q * n + i];
    for (int q = 0; q < 9; ++q) sti[q] = t.stress_tmp[(size_t)q * n + i];
    const double rti = t.density_tmp[i];
    const double ri2 = rti * rti;
    double dv[3] = {0, 0, 0};
    const bool rep = c.boundary == 3 || c.boundary == 4;
    for_neighbors<DIM>(c, p.x, t.pos32, cs, i, xi, true, [&](int j, const double* r, double rn) {
        double kd[3], kc[3];
        kernel_dW<DIM>(c, r, rn, kd);
        if (c.corr == 1) matvec_corr<DIM>(L, kd, kc);
        else { kc[0] = kd[0]; kc[1] = kd[1]; kc[2] = kd[2]; }
        double stj[9];
        for (int q = 0; q < 9; ++q) stj[q] = t.stress_tmp[(size_t)q * n + j];
        stress_div_term<DIM>(sti, ri2, stj, t.density_tmp[j], p.m_V[j], kc, dv);
    });
    if (rep) {
        for_neighbors<DIM>(c, p.x, t.pos32, cs, i, xi, true, [&](int j, const double* r, double rn) {
            if (p.mat_type[j] == MAT_REP) rep_force<DIM>(c, r, rn, dv);
        });
    }
    double vti[3], fd[3] = {0, 0, 0};
    for (int d = 0; d < 3; ++d) vti[d] = t.v_tmp[(size_t)d * n + i];
    damping_acc(c, rti, vti, fd, 3);
    for (int d = 0; d < 3; ++d) t.d_vel[(size_t)d * n + i] = (dv[d] + c.g[d]) + fd[d];
}

// ---- DP rates (eng/solver_sph_dp.py:236-270, Bui 2008 :172-208) ----
template <int DIM>
__global__ void k_dp_rates(Consts c, Persist64 p, Trans64 t, const int* __restrict__ cs,
                           const int* __restrict__ list, int count) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int i = list[k];
    const int n = c.n;
    double xi[3], vti[3];
    load_x<DIM>(p.x, i, n, xi);
    for (int d = 0; d < 3; ++d) vti[d] = t.v_tmp[(size_t)d * n + i];
    double L[9], sti[9];
    if (c.corr == 1)
        for (int q = 0; q < 9; ++q) L[q] = t.CSPM_L[(size_t)q * n + i];
    for (int q = 0; q < 9; ++q) sti[q] = t.stress_tmp[(size_t)q * n + i];
    const double rti = t.density_tmp[i];
    const double ri2 = rti * rti;
    double vg[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double dd = 0.0;
    double dv[3] = {0, 0, 0};
    for_neighbors<DIM>(c, p.x, t.pos32, cs, i, xi, true, [&](int j, const double* r, double rn) {
        const double mVj = p.m_V[j];
        double kd[3], kc[3];
        kernel_dW<DIM>(c, r, rn, kd);
        if (c.corr == 1) matvec_corr<DIM>(L, kd, kc);
        else { kc[0] = kd[0]; kc[1] = kd[1]; kc[2] = kd[2]; }
        double vtj[3];
        for (int d = 0; d < DIM; ++d) vtj[d] = t.v_tmp[(size_t)d * n + j];
        for (int a = 0; a < DIM; ++a) {
            double av = mVj * (vtj[a] - vti[a]);
            for (int b = 0; b < DIM; ++b) vg[3 * a + b] += av * kc[b];
        }
        double aa[3];
        for (int d = 0; d < DIM; ++d) aa[d] = mVj * (vti[d] - vtj[d]);
        dd += dotv<DIM>(aa, kc);
        double stj[9];
        for (int q = 0; q < 9; ++q) stj[q] = t.stress_tmp[(size_t)q * n + j];
        stress_div_term<DIM>(sti, ri2, stj, t.density_tmp[j], mVj, kc, dv);
    });
    for (int q = 0; q < 9; ++q) t.v_grad[(size_t)q * n + i] = vg[q];
    t.d_density[i] = dd * rti;
    // Bui 2008 stress rate
    double s[9], I1, sJ2, f_old;
    dp_inv(c, sti, s, I1, sJ2, f_old);
    double er[9], wr[9];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            er[3 * a + b] = 0.5 * (vg[3 * a + b] + vg[3 * b + a]);
            wr[3 * a + b] = 0.5 * (vg[3 * a + b] - vg[3 * b + a]);
        }
    double J[9];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            J[3 * a + b] = sti[3 * a] * wr[3 * b] + sti[3 * a + 1] * wr[3 * b + 1] + sti[3 * a + 2] * wr[3 * b + 2]
                         + sti[b] * wr[3 * a] + sti[3 + b] * wr[3 * a + 1] + sti[6 + b] * wr[3 * a + 2];
    const double tr = mtrace(er);
    double ed[9], te[9];
    for (int q = 0; q < 9; ++q) {
        ed[q] = er[q] - (tr / 3.0) * ((q % 4 == 0) ? 1.0 : 0.0);
        te[q] = c.twoG * ed[q] + (c.Km * tr) * ((q % 4 == 0) ? 1.0 : 0.0);
    }
    const bool plastic = f_old >= -EPS_F && sJ2 > EPS;
    double lam = 0.0;
    double ds[9];
    for (int q = 0; q < 9; ++q) {
        double tg = 0.0;
        if (plastic && q == 0) lam = (c.three_aK * tr + (c.Gm / sJ2) * msum_prod(s, er)) / c.lam_den;
        if (plastic) tg = lam * (c.nine_K_sin * ((q % 4 == 0) ? 1.0 : 0.0) + c.Gm / sJ2 * s[q]);
        ds[q] = (J[q] + te[q]) - tg;
    }
    for (int q = 0; q < 9; ++q) t.d_stress[(size_t)q * n + i] = ds[q];
    t.d_strain_equ[i] = sqrt(msum_sq(ed) * 2 / 3);
    double dep = 0.0;
    if (plastic) {
        const double gp = sJ2 + 3 * I1 * c.sin_dila;
        const double gd = gp - 0.0;  // g_p is never written by the reference (eng/particle_func.py:52)
        double ep[9];
        for (int q = 0; q < 9; ++q) {
            double v = fabs(ds[q]) > EPS ? gd / ds[q] : 0.0;
            ep[q] = lam * v;
        }
        const double t3 = mtrace(ep) / 3.0;
        double epd[9];
        for (int q = 0; q < 9; ++q) epd[q] = ep[q] - t3 * ((q % 4 == 0) ? 1.0 : 0.0);
        dep = sqrt(msum_sq(epd) * 2 / 3);
    }
    t.d_strain_equ_p[i] = dep;
    double fd[3] = {0, 0, 0};
    damping_acc(c, rti, vti, fd, 3);
    for (int d = 0; d < 3; ++d) t.d_vel[(size_t)d * n + i] = (dv[d] + c.g[d]) + fd[d];
}

// ---- integrators (eng/solver_sph_base.py:79-170) ----
__global__ void k_advect_full(Consts c, Persist64 p, Trans64 t, int* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int n = c.n;
    const int ti = p.mat_type[i];
    if (ti > 0) {
        double rho = p.density[i] + c.dt * t.d_density[i];
        p.density[i] = rho;
        p.m_V[i] = p.mass[i] / rho;
        for (int d = 0; d < 3; ++d) p.v[(size_t)d * n + i] += c.dt * t.d_vel[(size_t)d * n + i];
        if (!isfinite(rho)) atomicOr(err, TSG_ERR_NONFINITE);
    }
    if (ti == MAT_SOIL && c.solver == 3)
        for (int q = 0; q < 9; ++q) p.stress[(size_t)q * n + i] += c.dt * t.d_stress[(size_t)q * n + i];
}

__global__ void k_advect_half(Consts c, Persist64 p, Trans64 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int n = c.n;
    const int ti = p.mat_type[i];
    if (ti > 0) {
        double rt = t.density_tmp[i] + c.hdt * t.d_density[i];
        t.density_tmp[i] = rt;
        p.m_V[i] = p.mass[i] / rt;
        for (int d = 0; d < 3; ++d) t.v_tmp[(size_t)d * n + i] += c.hdt * t.d_vel[(size_t)d * n + i];
    }
    if (ti == MAT_SOIL && c.solver == 3)
        for (int q = 0; q < 9; ++q) t.stress_tmp[(size_t)q * n + i] += c.hdt * t.d_stress[(size_t)q * n + i];
}

__global__ void k_rk_init(Consts c, Persist64 p, Trans64 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int n = c.n;
    const int ti = p.mat_type[i];
    if (ti > 0) {
        t.d_density_RK[i] = 0.0;
        for (int d = 0; d < 3; ++d) t.d_vel_RK[(size_t)d * n + i] = 0.0;
    }
    if (ti == MAT_SOIL && t.d_stress_RK)
        for (int q = 0; q < 9; ++q) t.d_stress_RK[(size_t)q * n + i] = 0.0;
}

__global__ void k_rk_update(Consts c, Persist64 p, Trans64 t, int m) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int n = c.n;
    const int ti = p.mat_type[i];
    if (ti > 0) {
        t.d_density_RK[i] += t.d_density[i] * m;
        for (int d = 0; d < 3; ++d) t.d_vel_RK[(size_t)d * n + i] += t.d_vel[(size_t)d * n + i] * m;
    }
    if (ti == MAT_SOIL && t.d_stress_RK)
        for (int q = 0; q < 9; ++q) t.d_stress_RK[(size_t)q * n + i] += (double)m * t.d_stress[(size_t)q * n + i];
}

__global__ void k_rk_stage(Consts c, Persist64 p, Trans64 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int n = c.n;
    const int ti = p.mat_type[i];
    if (ti > 0) {
        double rt = c.hdt * t.d_density[i] + p.density[i];
        t.density_tmp[i] = rt;
        p.m_V[i] = p.mass[i] / rt;
        for (int d = 0; d < 3; ++d)
            t.v_tmp[(size_t)d * n + i] = c.hdt * t.d_vel[(size_t)d * n + i] + p.v[(size_t)d * n + i];
    }
    if (ti == MAT_SOIL && c.solver == 3)
        for (int q = 0; q < 9; ++q)
            t.stress_tmp[(size_t)q * n + i] = c.hdt * t.d_stress[(size_t)q * n + i] + p.stress[(size_t)q * n + i];
}

__global__ void k_rk_final(Consts c, Persist64 p, Trans64 t, int* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int n = c.n;
    const int ti = p.mat_type[i];
    if (ti > 0) {
        double rho = p.density[i] + c.dt6 * t.d_density_RK[i];
        p.density[i] = rho;
        p.m_V[i] = p.mass[i] / rho;
        for (int d = 0; d < 3; ++d) p.v[(size_t)d * n + i] += c.dt6 * t.d_vel_RK[(size_t)d * n + i];
        if (!isfinite(rho)) atomicOr(err, TSG_ERR_NONFINITE);
    }
    if (ti == MAT_SOIL && c.solver == 3)
        for (int q = 0; q < 9; ++q) p.stress[(size_t)q * n + i] += c.dt6 * t.d_stress_RK[(size_t)q * n + i];
}

// ---- advect_pos with XSPH (eng/solver_sph_base.py:224-238), two phases ----
template <int DIM>
__global__ void k_xsph(Consts c, Persist64 p, Trans64 t, const int* __restrict__ cs) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int n = c.n;
    const int ti = p.mat_type[i];
    if (!(ti > 0 && p.is_dynamic[i])) return;
    double xi[3], vi[3];
    load_x<DIM>(p.x, i, n, xi);
    for (int d = 0; d < 3; ++d) vi[d] = p.v[(size_t)d * n + i];
    double s[3] = {0, 0, 0};
    for_neighbors<DIM>(c, p.x, t.pos32, cs, i, xi, true, [&](int j, const double* r, double rn) {
        if (p.mat_type[j] != ti) return;
        const double w = kernel_W(c, rn);
        const double mVj = p.m_V[j];
        for (int d = 0; d < DIM; ++d) s[d] += mVj * (p.v[(size_t)d * n + j] - vi[d]) * w;
    });
    for (int d = 0; d < 3; ++d) t.aux3[(size_t)d * n + i] = s[d];
}

__global__ void k_advect_pos(Consts c, Persist64 p, Trans64 t, int* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int n = c.n;
    const int ti = p.mat_type[i];
    if (!(ti > 0)) return;
    const bool xs = c.xsph && p.is_dynamic[i];
    bool ok = true;
    for (int d = 0; d < 3; ++d) {
        double v = p.v[(size_t)d * n + i];
        double nx = xs ? p.x[(size_t)d * n + i] + c.dt * (v + 0.5 * t.aux3[(size_t)d * n + i])
                       : p.x[(size_t)d * n + i] + c.dt * v;
        p.x[(size_t)d * n + i] = nx;
        ok = ok && isfinite(nx);
    }
    if (!ok) atomicOr(err, TSG_ERR_NONFINITE);
}

// ---- advect_something (solver post-steps) ----
__global__ void k_post_wc(Consts c, Persist64 p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    if (p.mat_type[i] != MAT_FLUID) return;
    double rho = fmax(c.rho0, p.density[i]);
    p.density[i] = rho;
    p.m_V[i] = p.mass[i] / rho;
}

__global__ void k_post_mui_a(Consts c, Persist64 p, Trans64 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    if (p.mat_type[i] != MAT_SOIL) return;
    const int n = c.n;
    double rho = fmax(c.rho0, p.density[i]);
    p.density[i] = rho;
    p.m_V[i] = p.mass[i] / rho;
    p.strain_equ[i] += c.dt * t.d_strain_equ[i];
    for (int q = 0; q < 9; ++q) p.stress[(size_t)q * n + i] = t.stress_tmp[(size_t)q * n + i];
}

// Stress regularisation after advect_pos: centres use their moved positions, candidate
// cells come from this step's sort (eng/solver_sph_muI.py:151-156); exact f64 tests only.
template <int DIM>
__global__ void k_post_mui_b(Consts c, Persist64 p, Trans64 t, const int* __restrict__ cs) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    if (p.mat_type[i] != MAT_SOIL) return;
    const int n = c.n;
    double xi[3];
    load_x<DIM>(p.x, i, n, xi);
    double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for_neighbors<DIM>(c, p.x, t.pos32, cs, i, xi, false, [&](int j, const double* r, double rn) {
        if (p.mat_type[j] != MAT_SOIL) return;
        const double w = kernel_W(c, rn);
        const double mVj = p.m_V[j];
        for (int q = 0; q < 9; ++q) s[q] += mVj * p.stress[(size_t)q * n + j] * w;
    });
    const double f = t.CSPM_f[i];
    for (int q = 0; q < 9; ++q) t.aux9[(size_t)q * n + i] = s[q] * f;
}

__global__ void k_post_mui_c(Consts c, Persist64 p, Trans64 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    if (p.mat_type[i] != MAT_SOIL) return;
    const int n = c.n;
    for (int q = 0; q < 9; ++q) p.stress[(size_t)q * n + i] = t.aux9[(size_t)q * n + i];
}

__global__ void k_post_dp(Consts c, Persist64 p, Trans64 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    if (p.mat_type[i] != MAT_SOIL) return;
    const int n = c.n;
    double rho = fmax(c.rho0, p.density[i]);
    p.density[i] = rho;
    p.m_V[i] = p.mass[i] / rho;
    double st[9];
    for (int q = 0; q < 9; ++q) st[q] = p.stress[(size_t)q * n + i];
    p.flag_retmap[i] = dp_flag(c, st);
    dp_adapt(c, st);
    for (int q = 0; q < 9; ++q) p.stress[(size_t)q * n + i] = st[q];
    p.strain_equ[i] += c.dt * t.d_strain_equ[i];
    p.strain_equ_p[i] += c.dt * t.d_strain_equ_p[i];
}

// ---- enforce_boundary (eng/solver_sph_base.py:525-601) ----
__global__ void k_enforce(Consts c, Persist64 p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int n = c.n;
    const int ti = p.mat_type[i];
    const bool rigid_dyn = ti == MAT_RIGID && p.is_dynamic[i];
    const bool on = c.boundary == 1 ? (is_flow(ti) || rigid_dyn) : rigid_dyn;
    if (!on) return;
    double pos[3], nrm[3] = {0, 0, 0};
    for (int d = 0; d < 3; ++d) pos[d] = p.x[(size_t)d * n + i];
    const double r = c.r_eps;
    if (pos[0] > c.de[0] - r) { nrm[0] += 1.0; p.x[i] = c.de[0] - r; }
    if (pos[0] <= c.ds[0] + r) { nrm[0] += -1.0; p.x[i] = c.ds[0] + r; }
    if (pos[1] <= c.ds[1] + r) { nrm[1] += -1.0; p.x[(size_t)n + i] = c.ds[1] + r; }
    if (c.dim == 3) {
        if (pos[2] > c.de[2] - r) { nrm[2] += 1.0; p.x[2 * (size_t)n + i] = c.de[2] - r; }
        if (pos[2] <= c.ds[2] + r) { nrm[2] += -1.0; p.x[2 * (size_t)n + i] = c.ds[2] + r; }
    }
    double ln = sqrt((nrm[0] * nrm[0] + nrm[1] * nrm[1]) + nrm[2] * nrm[2]);
    if (ln > EPS) {
        double u[3] = {nrm[0] / ln, nrm[1] / ln, nrm[2] / ln};
        double v[3];
        for (int d = 0; d < 3; ++d) v[d] = p.v[(size_t)d * n + i];
        double vd = (v[0] * u[0] + v[1] * u[1]) + v[2] * u[2];
        for (int d = 0; d < 3; ++d) p.v[(size_t)d * n + i] = v[d] - (1.0 + 0.3) * vd * u[d];
    }
}

// ---- inspection: neighbour lists in traversal order ----
template <int DIM>
__global__ void k_nbr_count(Consts c, Persist64 p, Trans64 t, const int* __restrict__ cs, int* counts) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    double xi[3];
    load_x<DIM>(p.x, i, c.n, xi);
    int m = 0;
    for_neighbors<DIM>(c, p.x, t.pos32, cs, i, xi, true, [&](int, const double*, double) { ++m; });
    counts[i] = m;
}

template <int DIM>
__global__ void k_nbr_fill(Consts c, Persist64 p, Trans64 t, const int* __restrict__ cs,
                           const int* __restrict__ offsets, int* list) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    double xi[3];
    load_x<DIM>(p.x, i, c.n, xi);
    int m = offsets[i];
    for_neighbors<DIM>(c, p.x, t.pos32, cs, i, xi, true, [&](int j, const double*, double) { list[m++] = j; });
}

// ---- FP64 diagnostics over flow particles ----
__device__ __forceinline__ void atomic_max_double(double* addr, double v) {
    unsigned long long* a = reinterpret_cast<unsigned long long*>(addr);
    unsigned long long old = *a;
    while (__longlong_as_double(old) < v) {
        unsigned long long prev = atomicCAS(a, old, __double_as_longlong(v));
        if (prev == old) break;
        old = prev;
    }
}

__global__ void k_diag(Consts c, Persist64 p, double* out) {
    __shared__ double sh[8][TPB / 32];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = c.n;
    double v[8] = {0, 0, 0, 0, 0, 0, 0, -DBL_MAX};
    if (i < n && is_flow(p.mat_type[i])) {
        double m = p.mass[i];
        double vx = p.v[i], vy = p.v[(size_t)n + i], vz = p.v[2 * (size_t)n + i];
        double v2 = (vx * vx + vy * vy) + vz * vz;
        v[0] = m;
        v[1] = m * vx; v[2] = m * vy; v[3] = m * vz;
        v[4] = 0.5 * m * v2;
        v[5] = -m * ((c.g[0] * p.x[i] + c.g[1] * p.x[(size_t)n + i]) + c.g[2] * p.x[2 * (size_t)n + i]);
        v[6] = sqrt(v2);
        v[7] = p.x[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        for (int q = 0; q < 6; ++q) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
        v[6] = fmax(v[6], __shfl_down_sync(0xffffffffu, v[6], o));
        v[7] = fmax(v[7], __shfl_down_sync(0xffffffffu, v[7], o));
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) for (int q = 0; q < 8; ++q) sh[q][wid] = v[q];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < TPB / 32; ++w) {
            for (int q = 0; q < 6; ++q) v[q] += sh[q][w];
            v[6] = fmax(v[6], sh[6][w]);
            v[7] = fmax(v[7], sh[7][w]);
        }
        for (int q = 0; q < 6; ++q) atomicAdd(&out[q], v[q]);
        atomic_max_double(&out[6], v[6]);
        atomic_max_double(&out[7], v[7]);
    }
}

__global__ void k_geostatic(Consts c, Persist64 p, const double* ymax_in, double K0) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    if (p.mat_type[i] != MAT_SOIL) return;
    const int n = c.n;
    double vs = c.rho0 * c.g[1] * (ymax_in[0] - p.x[(size_t)n + i]);
    p.stress[i] = K0 * vs;
    p.stress[4 * (size_t)n + i] = vs;
    p.stress[8 * (size_t)n + i] = K0 * vs;
}

__global__ void k_ymax_soil(Consts c, Persist64 p, double* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double y = -DBL_MAX;
    if (i < c.n && p.mat_type[i] == MAT_SOIL) y = p.x[(size_t)c.n + i];
    for (int o = 16; o > 0; o >>= 1) y = fmax(y, __shfl_down_sync(0xffffffffu, y, o));
    if ((threadIdx.x & 31) == 0) atomic_max_double(out, y);
}

}  // namespace

// ---------------------------------------------------------------- launchers
// ---- dynamic rigid bodies (eng/solver_sph_base.py:467-518) ----
// The reaction on dynamic rigid particles.  The reference subtracts every flow particle's
// pair term from its dynamic rigid neighbour inside the flow particle's loop
// (`pt[j].d_vel -= tmp`, eng/solver_sph_wc.py:70-71, eng/solver_sph_muI.py:45-46,
// eng/solver_sph_dp.py:164-165), an unsynchronised scatter.  Here every rigid particle
// gathers the terms of its flow neighbours in its own traversal order, which is ascending
// particle index (the serial order of the scatter), evaluating each term exactly as the flow
// particle's loop does (r = x_flow - x_rigid is the exact negation of the traversal's
// offset), starting from the gravity the boundary pass set.
template <int DIM>
__global__ void k_rigid_reaction(Consts c, Persist64 p, Trans64 t, const int* __restrict__ cs,
                                 const int* __restrict__ list, int count) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int j = list[k];
    if (!(p.mat_type[j] == MAT_RIGID && p.is_dynamic[j])) return;
    const int n = c.n;
    double xj[3];
    load_x<DIM>(p.x, j, n, xj);
    double dvj[3];
    for (int d = 0; d < 3; ++d) dvj[d] = t.d_vel[(size_t)d * n + j];
    const double mVj = p.m_V[j], rtj = t.density_tmp[j], ptj = p.pressure[j];
    double stj[9], vtj[3];
    if (c.solver != 1)
        for (int q = 0; q < 9; ++q) stj[q] = t.stress_tmp[(size_t)q * n + j];
    for (int d = 0; d < 3; ++d) vtj[d] = t.v_tmp[(size_t)d * n + j];
    for_neighbors<DIM>(c, p.x, t.pos32, cs, j, xj, true, [&](int i, const double* rji, double rn) {
        if (p.mat_type[i] != c.flow_type) return;
        double r[3] = {-rji[0], -rji[1], -rji[2]};
        if (DIM == 2) r[2] = 0.0;
        double kd[3], f[3] = {0.0, 0.0, 0.0};
        kernel_dW<DIM>(c, r, rn, kd);
        const double rti = t.density_tmp[i];
        if (c.solver == 1) {
            double dvv[3];
            for (int d = 0; d < DIM; ++d) dvv[d] = t.v_tmp[(size_t)d * n + i] - vtj[d];
            const double pri = p.pressure[i] / (rti * rti);
            wc_force_pair<DIM>(c, MAT_RIGID, mVj, dvv, rti, pri, ptj, rtj, r, rn, kd, f);
        } else {
            double kc[3], sti[9];
            if (c.corr == 1) {
                double L[9];
                for (int q = 0; q < 9; ++q) L[q] = t.CSPM_L[(size_t)q * n + i];
                matvec_corr<DIM>(L, kd, kc);
            } else {
                kc[0] = kd[0]; kc[1] = kd[1]; kc[2] = kd[2];
            }
            for (int q = 0; q < 9; ++q) sti[q] = t.stress_tmp[(size_t)q * n + i];
            stress_div_val<DIM>(sti, rti * rti, stj, rtj, mVj, kc, f);
        }
        for (int d = 0; d < DIM; ++d) dvj[d] = dvj[d] - f[d];
    });
    for (int d = 0; d < 3; ++d) t.d_vel[(size_t)d * n + j] = dvj[d];
}

// Object slot of a dynamic rigid particle (-1 for any other), for the list builder.
struct RigidSlot64 {
    const int* mt;
    const int* dyn;
    const int* oid;
    const int* ids;
    int nobj;
    __device__ int operator()(int i) const {
        if (mt[i] != MAT_RIGID || !dyn[i]) return -1;
        const int id = oid[i];
        for (int o = 0; o < nobj; ++o)
            if (ids[o] == id) return o;
        return -1;
    }
};

// The object sums of the shape matching are serial sums in ascending particle order (the
// oracle's order, so that the results are bit-identical).  The block stages each chunk of
// kSMChunk particles' terms (products rounded as in the serial expression: this unit is
// compiled without contracted multiply-adds) in shared memory with all its threads, and
// one thread adds them in order: the dependent additions run from shared memory instead of
// behind one gather per particle.
constexpr int kSMChunk = 512;

// init_rigid_body / calc_rigid_rest_m (eng/solver_sph_base.py:467-470, :517-518): the rest
// centre of mass of every dynamic rigid object from the uploaded positions, summed in upload
// order (the object's list, built before the first sort), one block per object.
__global__ void __launch_bounds__(kSMChunk) k_rest_cm(Consts c, Persist64 p, Rigid64 rb) {
    __shared__ double buf[4][kSMChunk];
    const int o = blockIdx.x;
    const int* list = rb.list + rb.off[o];
    const int m = rb.off[o + 1] - rb.off[o];
    const int n = c.n;
    double cm[3] = {0.0, 0.0, 0.0}, sum_m = 0.0;
    for (int k0 = 0; k0 < m; k0 += kSMChunk) {
        const int k = k0 + threadIdx.x;
        if (k < m) {
            const int i = list[k];
            const double mi = p.mass[i];
            for (int d = 0; d < 3; ++d) buf[d][threadIdx.x] = mi * p.x[(size_t)d * n + i];
            buf[3][threadIdx.x] = mi;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const int cnt = min(kSMChunk, m - k0);
            for (int q = 0; q < cnt; ++q) {
                for (int d = 0; d < 3; ++d) cm[d] = cm[d] + buf[d][q];
                sum_m += buf[3][q];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int d = 0; d < 3; ++d) rb.rest_cm[3 * o + d] = cm[d] / sum_m;
}

// solve_constraints (eng/solver_sph_base.py:478-500), one block per dynamic rigid object,
// over its list (ascending particle order, rebuilt after every sort): the centre of mass
// (calc_cm, :502-511) and A = sum (m_V rho p) q^T (p = x - cm, q = x0 - rest cm), both
// summed in list order, R = polar(A) (identity when every entry is below 1e-8), and finally
// every particle x += (cm + R q) - x.
__global__ void __launch_bounds__(kSMChunk) k_shape_match(Consts c, Persist64 p, Rigid64 rb) {
    __shared__ double buf[9][kSMChunk];
    __shared__ double cm_s[3], R_s[9];
    const int o = blockIdx.x;
    const int* list = rb.list + rb.off[o];
    const int m = rb.off[o + 1] - rb.off[o];
    const int n = c.n;
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double sum_m = 0.0;
    for (int k0 = 0; k0 < m; k0 += kSMChunk) {
        const int k = k0 + threadIdx.x;
        if (k < m) {
            const int i = list[k];
            const double mi = p.mass[i];
            for (int d = 0; d < 3; ++d) buf[d][threadIdx.x] = mi * p.x[(size_t)d * n + i];
            buf[3][threadIdx.x] = mi;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const int cnt = min(kSMChunk, m - k0);
            for (int q = 0; q < cnt; ++q) {
                for (int d = 0; d < 3; ++d) acc[d] = acc[d] + buf[d][q];
                sum_m += buf[3][q];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int d = 0; d < 3; ++d) cm_s[d] = acc[d] / sum_m;
    __syncthreads();
    for (int q = 0; q < 9; ++q) acc[q] = 0.0;
    for (int k0 = 0; k0 < m; k0 += kSMChunk) {
        const int k = k0 + threadIdx.x;
        if (k < m) {
            const int i = list[k];
            const double sc = p.m_V[i] * p.density[i];
            double sp[3], q[3];
            for (int d = 0; d < 3; ++d) {
                q[d] = p.x0[(size_t)d * n + i] - rb.rest_cm[3 * o + d];
                sp[d] = sc * (p.x[(size_t)d * n + i] - cm_s[d]);
            }
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) buf[3 * a + b][threadIdx.x] = sp[a] * q[b];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const int cnt = min(kSMChunk, m - k0);
            for (int q = 0; q < cnt; ++q)
                for (int e = 0; e < 9; ++e) acc[e] = acc[e] + buf[e][q];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double R[9];
        polar3(acc, R);
        bool small = true;
        for (int q = 0; q < 9; ++q) small = small && fabs(R[q]) < EPS;
        if (small)
            for (int q = 0; q < 9; ++q) R[q] = (q % 4 == 0) ? 1.0 : 0.0;
        for (int q = 0; q < 9; ++q) R_s[q] = R[q];
    }
    __syncthreads();
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        const int i = list[k];
        double q[3];
        for (int d = 0; d < 3; ++d) q[d] = p.x0[(size_t)d * n + i] - rb.rest_cm[3 * o + d];
        for (int a = 0; a < 3; ++a) {
            const double rq = (R_s[3 * a] * q[0] + R_s[3 * a + 1] * q[1]) + R_s[3 * a + 2] * q[2];
            const double goal = cm_s[a] + rq;
            const double xa = p.x[(size_t)a * n + i];
            const double corr = (goal - xa) * 1.0;
            p.x[(size_t)a * n + i] = xa + corr;
        }
    }
}

static void rigid_lists64(const Consts& c, const Persist64& p, const Rigid64& r, cudaStream_t s) {
    build_rigid_lists(c.n, r.nobj, RigidSlot64{p.mat_type, p.is_dynamic, p.obj_id, r.obj_id, r.nobj}, r.scratch,
                      r.off, r.list, s);
}

#define DISPATCH_DIM(c, KERNEL, GRID, ...)                                   \
    do {                                                                     \
        if ((c).dim == 2) TSG_LAUNCH(KERNEL<2>, GRID, TPB, s, __VA_ARGS__);       \
        else TSG_LAUNCH(KERNEL<3>, GRID, TPB, s, __VA_ARGS__);                    \
    } while (0)

void fp64_kernel_corr(const Consts& c, const Persist64& p, Trans64& t, const Grid& g, cudaStream_t s) {
    PhaseScope ph(s, PH_CORR);
    DISPATCH_DIM(c, k_corr, nblk(c.n), c, p, t, g.cell_start);
}

void fp64_rest_cm(const Consts& c, const Persist64& p, const Rigid64& r, cudaStream_t s) {
    if (r.nobj <= 0) return;
    rigid_lists64(c, p, r, s);
    TSG_LAUNCH(k_rest_cm, r.nobj, kSMChunk, s, c, p, r);
}

void fp64_solve_rigid(const Consts& c, Persist64& p, const Rigid64& r, cudaStream_t s) {
    if (r.nobj <= 0) return;
    PhaseScope ph(s, PH_POS);
    rigid_lists64(c, p, r, s);
    TSG_LAUNCH(k_shape_match, r.nobj, kSMChunk, s, c, p, r);
}

void fp64_density_sum(const Consts& c, const Persist64& p, const Trans64& t, const Grid& g, double* out,
                      cudaStream_t s) {
    PhaseScope ph(s, PH_OTHER);
    DISPATCH_DIM(c, k_density_sum, nblk(c.n), c, p, t, g.cell_start, out);
}

void fp64_init_tmp(const Consts& c, const Persist64& p, Trans64& t, cudaStream_t s) {
    PhaseScope ph(s, PH_INIT);
    TSG_LAUNCH(k_init_tmp, nblk(c.n), TPB, s, c, p, t);
}

void fp64_one_step(const Consts& c, Persist64& p, Trans64& t, const Grid& g, cudaStream_t s) {
    if (c.n_flow > 0 && (c.solver == 1 || c.solver == 3)) {
        PhaseScope ph(s, PH_PRE);
        TSG_LAUNCH(k_pre, nblk(c.n_flow), TPB, s, c, p, t, g.list_flow, c.n_flow);
    }
    if (c.solver == 2 && c.n_flow > 0) {
        PhaseScope ph(s, PH_PRE);
        DISPATCH_DIM(c, k_mui_stress, nblk(c.n_flow), c, p, t, g.cell_start, g.list_flow, c.n_flow);
    }
    if (c.n_bdy > 0) {
        PhaseScope ph(s, PH_BDY);
        DISPATCH_DIM(c, k_bdy, nblk(c.n_bdy), c, p, t, g.cell_start, g.list_bdy, c.n_bdy);
    }
    if (c.n_flow > 0) {
        PhaseScope ph(s, PH_RATES);
        if (c.solver == 1) DISPATCH_DIM(c, k_wc_rates, nblk(c.n_flow), c, p, t, g.cell_start, g.list_flow, c.n_flow);
        else if (c.solver == 2) DISPATCH_DIM(c, k_mui_mom, nblk(c.n_flow), c, p, t, g.cell_start, g.list_flow, c.n_flow);
        else DISPATCH_DIM(c, k_dp_rates, nblk(c.n_flow), c, p, t, g.cell_start, g.list_flow, c.n_flow);
    }
    if (c.n_rigid_dyn > 0 && c.n_bdy > 0) {  // the flow's reaction on dynamic rigid particles
        PhaseScope ph(s, PH_RATES);
        DISPATCH_DIM(c, k_rigid_reaction, nblk(c.n_bdy), c, p, t, g.cell_start, g.list_bdy, c.n_bdy);
    }
}

void fp64_advect(const Consts& c, Persist64& p, Trans64& t, const Grid& g, int which, cudaStream_t s) {
    const int nb = nblk(c.n);
    PhaseScope ph(s, which == TSG_ADVECT_POS ? PH_POS : which == TSG_ADVECT_SOMETHING ? PH_POST
                     : which == TSG_ENFORCE_BOUNDARY ? PH_OTHER : PH_INTEGRATE);
    switch (which) {
    case TSG_ADVECT_FULL: TSG_LAUNCH(k_advect_full, nb, TPB, s, c, p, t, g.err); break;
    case TSG_ADVECT_LF_HALF: TSG_LAUNCH(k_advect_half, nb, TPB, s, c, p, t); break;
    case TSG_ADVECT_POS:
        if (c.xsph) DISPATCH_DIM(c, k_xsph, nb, c, p, t, g.cell_start);
        TSG_LAUNCH(k_advect_pos, nb, TPB, s, c, p, t, g.err);
        break;
    case TSG_ADVECT_SOMETHING:
        if (c.solver == 1) TSG_LAUNCH(k_post_wc, nb, TPB, s, c, p);
        else if (c.solver == 2) {
            TSG_LAUNCH(k_post_mui_a, nb, TPB, s, c, p, t);
            DISPATCH_DIM(c, k_post_mui_b, nb, c, p, t, g.cell_start);
            TSG_LAUNCH(k_post_mui_c, nb, TPB, s, c, p, t);
        } else TSG_LAUNCH(k_post_dp, nb, TPB, s, c, p, t);
        break;
    case TSG_ENFORCE_BOUNDARY: TSG_LAUNCH(k_enforce, nb, TPB, s, c, p); break;
    case TSG_RK_INIT: TSG_LAUNCH(k_rk_init, nb, TPB, s, c, p, t); break;
    case TSG_RK_STAGE: TSG_LAUNCH(k_rk_stage, nb, TPB, s, c, p, t); break;
    case TSG_RK_FINAL: TSG_LAUNCH(k_rk_final, nb, TPB, s, c, p, t, g.err); break;
    default: break;
    }
}

void fp64_rk_update(const Consts& c, Persist64& p, Trans64& t, int m, cudaStream_t s) {
    PhaseScope ph(s, PH_INTEGRATE);
    TSG_LAUNCH(k_rk_update, nblk(c.n), TPB, s, c, p, t, m);
}

void fp64_neighbors(const Consts& c, const Persist64& p, const Trans64& t, const Grid& g,
                    int* counts, int* offsets, int* list, cudaStream_t s) {
    if (!list) {
        DISPATCH_DIM(c, k_nbr_count, nblk(c.n), c, p, t, g.cell_start, counts);
    } else {
        DISPATCH_DIM(c, k_nbr_fill, nblk(c.n), c, p, t, g.cell_start, offsets, list);
    }
}

void fp64_diag(const Consts& c, const Persist64& p, double* out8, cudaStream_t s) {
    double init[8] = {0, 0, 0, 0, 0, 0, 0, -DBL_MAX};
    cudaMemcpyAsync(out8, init, sizeof init, cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
    TSG_LAUNCH(k_diag, nblk(c.n), TPB, s, c, p, out8);
}

void fp64_init_geostatic(const Consts& c, Persist64& p, double* scratch, cudaStream_t s) {
    double init = -DBL_MAX;
    cudaMemcpyAsync(scratch, &init, sizeof init, cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
    TSG_LAUNCH(k_ymax_soil, nblk(c.n), TPB, s, c, p, scratch);
    TSG_LAUNCH(k_geostatic, nblk(c.n), TPB, s, c, p, scratch, c.K0);
}

__global__ void k_refresh_pos32_impl(Consts c, const double* __restrict__ x, float4* __restrict__ pos32) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const size_t n = c.n;
    pos32[i] = make_float4((float)(x[i] - c.vs[0]), (float)(x[n + i] - c.vs[1]), (float)(x[2 * n + i] - c.vs[2]), 0.f);
}

void fp64_refresh_pos32(const Consts& c, const Persist64& p, Trans64& t, cudaStream_t s) {
    TSG_LAUNCH(k_refresh_pos32_impl, nblk(c.n), TPB, s, c, p.x, t.pos32);
}

}  // namespace tsg
