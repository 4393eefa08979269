// ORACLE - test infrastructure only.  Never linked into, loaded by or called from the
// product path (tisphi_gb300/).  Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg use it, to check results or to time the CPU restatement.
//
// f64 CPU restatement of the reference's per-substep SPH path (Rabmelon/tiSPHi, Taichi).
// The reference keeps one array of structs (eng/particle_func.py:10-88) and runs every
// @ti.kernel as a parallel loop over particles; this file keeps the same array of structs
// and runs each loop with OpenMP.  Every sum over neighbours is accumulated by one thread
// in the reference's traversal order, so results do not depend on the thread count.
//
// Semantics fixed where the reference is racy or undefined:
//  * counting sort is stable (the serial order of eng/particle_system.py:240-245);
//  * a neighbour cell whose flattened index is outside [0, G) is skipped; a particle whose
//    own flattened index is outside [0, G) is binned after every cell and flagged;
//  * WC one_step loop 1 runs as two phases (fluid EOS first, then boundary extrapolation,
//    eng/solver_sph_wc.py:86-106);
//  * advect_pos computes every XSPH sum before any position moves
//    (eng/solver_sph_base.py:228-238);
//  * mu(I) post-step copies stress_tmp -> stress for all soil first, then regularises into
//    a fresh buffer (eng/solver_sph_muI.py:134-156).
// Powers with a constant exponent are written as products: q1^4 = (q1*q1)*(q1*q1),
// q1^3 = (q1*q1)*q1, x**2 = x*x; the integer Tait exponent uses binary exponentiation.
//
// Parity pin: this restatement is checked against golden vectors produced by running the
// reference's own Python/Taichi source under a serial Taichi-API emulator
// (tests/golden/make_golden.py).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <string>

#include "sph_oracle.h"

namespace {

constexpr int MAT_REP = -2, MAT_DUMMY = -1, MAT_FLUID = 1, MAT_SOIL = 2, MAT_RIGID = 11;
constexpr double EPS = 1e-8;       // SPHBase.epsilon (eng/solver_sph_base.py:25)
constexpr double EPS_F = 1e-4;     // DPSPHSolver.eps_f (eng/solver_sph_dp.py:23)

struct V3 { double c[3]; };
struct M3 { double m[3][3]; };

inline V3 v3(double a, double b, double c) { V3 r; r.c[0] = a; r.c[1] = b; r.c[2] = c; return r; }
inline V3 vzero() { return v3(0, 0, 0); }
inline M3 mzero() { M3 r; std::memset(&r, 0, sizeof r); return r; }
inline M3 meye() { M3 r = mzero(); r.m[0][0] = r.m[1][1] = r.m[2][2] = 1.0; return r; }
inline V3 vsub(const V3& a, const V3& b) { return v3(a.c[0] - b.c[0], a.c[1] - b.c[1], a.c[2] - b.c[2]); }
inline V3 vadd(const V3& a, const V3& b) { return v3(a.c[0] + b.c[0], a.c[1] + b.c[1], a.c[2] + b.c[2]); }
inline V3 vscale(double s, const V3& a) { return v3(s * a.c[0], s * a.c[1], s * a.c[2]); }
inline double vdot(const V3& a, const V3& b) { return (a.c[0] * b.c[0] + a.c[1] * b.c[1]) + a.c[2] * b.c[2]; }
inline double vnorm(const V3& a) { return std::sqrt((a.c[0] * a.c[0] + a.c[1] * a.c[1]) + a.c[2] * a.c[2]); }
inline M3 outer(const V3& a, const V3& b) {
    M3 r; for (int p = 0; p < 3; ++p) for (int q = 0; q < 3; ++q) r.m[p][q] = a.c[p] * b.c[q]; return r;
}
inline V3 matvec(const M3& a, const V3& v) {
    V3 r; for (int p = 0; p < 3; ++p) r.c[p] = (a.m[p][0] * v.c[0] + a.m[p][1] * v.c[1]) + a.m[p][2] * v.c[2]; return r;
}
inline M3 madd(const M3& a, const M3& b) { M3 r; for (int p = 0; p < 3; ++p) for (int q = 0; q < 3; ++q) r.m[p][q] = a.m[p][q] + b.m[p][q]; return r; }
inline M3 msub(const M3& a, const M3& b) { M3 r; for (int p = 0; p < 3; ++p) for (int q = 0; q < 3; ++q) r.m[p][q] = a.m[p][q] - b.m[p][q]; return r; }
inline M3 mscale(double s, const M3& a) { M3 r; for (int p = 0; p < 3; ++p) for (int q = 0; q < 3; ++q) r.m[p][q] = s * a.m[p][q]; return r; }
inline M3 mmul_elem(const M3& a, const M3& b) { M3 r; for (int p = 0; p < 3; ++p) for (int q = 0; q < 3; ++q) r.m[p][q] = a.m[p][q] * b.m[p][q]; return r; }
inline M3 mT(const M3& a) { M3 r; for (int p = 0; p < 3; ++p) for (int q = 0; q < 3; ++q) r.m[p][q] = a.m[q][p]; return r; }
inline double msum(const M3& a) {  // row-major sequential
    double s = a.m[0][0];
    for (int k = 1; k < 9; ++k) s = s + a.m[k / 3][k % 3];
    return s;
}
inline double mtrace(const M3& a) { return (a.m[0][0] + a.m[1][1]) + a.m[2][2]; }
inline M3 mdiag(const V3& v) { M3 r = mzero(); for (int p = 0; p < 3; ++p) r.m[p][p] = v.c[p]; return r; }

// 2x2 / 3x3 determinant and inverse by cofactors.
inline double det2(const M3& a) { return a.m[0][0] * a.m[1][1] - a.m[0][1] * a.m[1][0]; }
inline double det3(const M3& a) {
    return a.m[0][0] * (a.m[1][1] * a.m[2][2] - a.m[2][1] * a.m[1][2])
         - a.m[1][0] * (a.m[0][1] * a.m[2][2] - a.m[2][1] * a.m[0][2])
         + a.m[2][0] * (a.m[0][1] * a.m[1][2] - a.m[1][1] * a.m[0][2]);
}
inline M3 inv2_fill0(const M3& a) {
    double id = 1.0 / det2(a);
    M3 r = mzero();
    r.m[0][0] = id * a.m[1][1]; r.m[0][1] = id * (-a.m[0][1]);
    r.m[1][0] = id * (-a.m[1][0]); r.m[1][1] = id * a.m[0][0];
    return r;
}
inline M3 inv3(const M3& a) {
    double id = 1.0 / det3(a);
    M3 r;
    for (int p = 0; p < 3; ++p)
        for (int q = 0; q < 3; ++q)
            r.m[q][p] = id * (a.m[(p + 1) % 3][(q + 1) % 3] * a.m[(p + 2) % 3][(q + 2) % 3]
                            - a.m[(p + 2) % 3][(q + 1) % 3] * a.m[(p + 1) % 3][(q + 2) % 3]);
    return r;
}

inline double powi(double x, long n) {  // binary exponentiation, low bit first
    double r = 1.0;
    bool first = true;
    while (n > 0) {
        if (n & 1) { r = first ? x : r * x; first = false; }
        n >>= 1;
        if (n) x = x * x;
    }
    return r;
}

// Orthogonal polar factor of a 3x3 matrix: Higham's scaled Newton iteration
// X <- (g X + X^-T / g) / 2 with g = (|X^-1|_F / |X|_F)^(1/2) (N. J. Higham, "Computing the
// polar decomposition - with applications", SIAM J. Sci. Stat. Comput. 7, 1986), X^-T from
// the cofactors, until an update changes X by at most 1e-14 (Frobenius) or after 60 steps.
// A matrix whose third row and column are zero (a 2D body: every z offset is zero) gets
// A[2][2] = 1 first, so the z axis maps to itself; a singular matrix gives the identity.
inline M3 polar3(const M3& A) {
    M3 X = A;
    if (X.m[0][2] == 0.0 && X.m[1][2] == 0.0 && X.m[2][0] == 0.0 && X.m[2][1] == 0.0 && X.m[2][2] == 0.0)
        X.m[2][2] = 1.0;
    for (int it = 0; it < 60; ++it) {
        const double (*x)[3] = X.m;
        double c[3][3];
        c[0][0] = x[1][1] * x[2][2] - x[1][2] * x[2][1];
        c[0][1] = x[1][2] * x[2][0] - x[1][0] * x[2][2];
        c[0][2] = x[1][0] * x[2][1] - x[1][1] * x[2][0];
        c[1][0] = x[0][2] * x[2][1] - x[0][1] * x[2][2];
        c[1][1] = x[0][0] * x[2][2] - x[0][2] * x[2][0];
        c[1][2] = x[0][1] * x[2][0] - x[0][0] * x[2][1];
        c[2][0] = x[0][1] * x[1][2] - x[0][2] * x[1][1];
        c[2][1] = x[0][2] * x[1][0] - x[0][0] * x[1][2];
        c[2][2] = x[0][0] * x[1][1] - x[0][1] * x[1][0];
        const double det = (x[0][0] * c[0][0] + x[0][1] * c[0][1]) + x[0][2] * c[0][2];
        if (det == 0.0 || !std::isfinite(det)) return meye();
        double fx = 0.0, fy = 0.0;
        double y[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                y[a][b] = c[a][b] / det;
                fx += x[a][b] * x[a][b];
                fy += y[a][b] * y[a][b];
            }
        const double gm = std::sqrt(std::sqrt(fy) / std::sqrt(fx));
        double ch = 0.0;
        M3 Xn;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                Xn.m[a][b] = 0.5 * (gm * x[a][b] + y[a][b] / gm);
                const double d = Xn.m[a][b] - x[a][b];
                ch += d * d;
            }
        X = Xn;
        if (ch <= 1e-28) break;
    }
    return X;
}

// Particle record: the fields of eng/particle_func.py:10-88 that the path reads or writes.
struct P {
    int obj_id, mat_id, mat_type, is_dynamic;
    V3 x, x0, v;
    double m_V, density, mass, pressure;
    M3 stress;
    int grid_ids, id_new, id0;
    double CSPM_f;
    M3 CSPM_L;
    double d_density;
    V3 d_vel;
    M3 d_stress, v_grad;
    int flag_retmap;
    double g_p, strain_equ, d_strain_equ, strain_equ_p, d_strain_equ_p;
    double density_tmp;
    V3 v_tmp;
    M3 stress_tmp;
    double d_density_RK;
    V3 d_vel_RK;
    M3 d_stress_RK;
};

struct Sys {
    orc_params prm;
    int dim = 3;
    int n = 0;
    std::vector<P> pt, pt_buf;
    std::vector<int> grid_end;   // inclusive prefix sums of cell counts (G + 1: last = OOB bin)
    std::vector<int> grid_tmp;
    int err = 0;
    // derived constants
    double h1 = 0, kk = 0, visc_fac = 0, eps_h2 = 0, h2 = 0;
    double mu = 0, vsound2 = 0;           // mu(I)
    double alpha = 0, k_c = 0, G = 0, K = 0, sin_dila = 0, kc_over_alpha = 0;
    double lam_den = 0, three_aK = 0, nine_K_sin = 0, twoG = 0; // DP folded constants
    double damp_E = 0;
    double g[3];
    double vsound = 0;
    // dynamic rigid bodies (eng/solver_sph_base.py:467-518): object ids and rest centres of
    // mass, computed at creation from the input positions in input order
    int n_rigid_dyn = 0;
    std::vector<int> rigid_ids;
    std::vector<V3> rigid_rest_cm;

    bool is_fluid(int p) const { return pt[p].mat_type == MAT_FLUID; }
    bool is_soil(int p) const { return pt[p].mat_type == MAT_SOIL; }
    bool is_flow(int p) const { return pt[p].mat_type == MAT_FLUID || pt[p].mat_type == MAT_SOIL; }
    bool is_real(int p) const { return pt[p].mat_type > 0; }
    bool is_bdy(int p) const { return pt[p].mat_type == MAT_DUMMY || pt[p].mat_type == MAT_REP; }
    bool is_rep(int p) const { return pt[p].mat_type == MAT_REP; }
    bool is_rigid(int p) const { return pt[p].mat_type == MAT_RIGID; }
    bool is_rigid_static(int p) const { return pt[p].mat_type == MAT_RIGID && !pt[p].is_dynamic; }
    bool is_rigid_dynamic(int p) const { return pt[p].mat_type == MAT_RIGID && pt[p].is_dynamic; }
    bool same_type(int p, int q) const { return pt[p].mat_type == pt[q].mat_type; }

    // ---- neighbour search (eng/particle_system.py:216-269) ----
    // Truncating cast (eng/particle_system.py:216-218); false when a coordinate does not fit
    // an int (non-finite or huge), where the reference's cast is undefined.
    bool pos_to_index(const V3& x, int idx[3]) const {
        bool ok = true;
        for (int d = 0; d < 3; ++d) {
            double t = (x.c[d] - prm.vdomain_start[d]) / prm.grid_size;
            if (!(std::fabs(t) < 2147483647.0)) { ok = false; idx[d] = 0; }
            else idx[d] = (int)t;
        }
        return ok;
    }
    long flatten(const int idx[3]) const {
        return (long)idx[0] * prm.grid_num[1] * prm.grid_num[2] + (long)idx[1] * prm.grid_num[2] + idx[2];
    }
    template <class F>
    void for_all_neighbors(int i, F&& task) const {
        int c[3];
        if (!pos_to_index(pt[i].x, c)) return;
        const long G = prm.grid_num_total;
        for (int ox = -1; ox <= 1; ++ox)
            for (int oy = -1; oy <= 1; ++oy)
                for (int oz = -1; oz <= 1; ++oz) {
                    if (dim == 2 && oz != 0) continue;
                    int cc[3] = {c[0] + ox, c[1] + oy, c[2] + oz};
                    long f = flatten(cc);
                    if (f < 0 || f >= G) continue;
                    int b = f > 0 ? grid_end[f - 1] : 0;
                    int e = grid_end[f];
                    for (int j = b; j < e; ++j) {
                        if (i != j && vnorm(vsub(pt[i].x, pt[j].x)) < prm.support_radius) task(j);
                    }
                }
    }

    // ---- kernels (eng/solver_sph_base.py:279-358) ----
    double W(const V3& r) const {
        double res = 0.0;
        double rn = vnorm(r);
        double q = rn * h1;
        if (rn > EPS && q <= 2.0) {
            if (prm.kernel == 1) {
                double q1 = 1.0 - 0.5 * q;
                res = kk * ((q1 * q1) * (q1 * q1)) * (1.0 + 2.0 * q);
            } else {
                if (q <= 1.0) {
                    double q2 = q * q, q3 = q2 * q;
                    res = kk * (0.5 * q3 - q2 + 2.0 / 3.0);
                } else {
                    double t = 2.0 - q;
                    res = kk / 6.0 * ((t * t) * t);
                }
            }
        }
        return res;
    }
    V3 dW(const V3& r) const {
        V3 res = vzero();
        double rn = vnorm(r);
        double q = rn * h1;
        if (rn > EPS && q <= 2.0) {
            if (prm.kernel == 1) {
                double q1 = 1.0 - 0.5 * q;
                double s = kk * ((q1 * q1) * q1) * (-5.0 * q) * h1;
                for (int d = 0; d < 3; ++d) res.c[d] = s * r.c[d] / rn;
            } else {
                double s;
                if (q <= 1.0) s = kk * q * (1.5 * q - 2.0);
                else { double f = 2.0 - q; s = kk * (-0.5 * f * f); }
                for (int d = 0; d < 3; ++d) res.c[d] = s * (r.c[d] / rn * h1);
            }
        }
        return res;
    }
    V3 dW_corr(int i, int j) const {  // kernel_deriv_corr (eng/solver_sph_base.py:375-383)
        V3 t = dW(vsub(pt[i].x, pt[j].x));
        if (prm.kernel_corr == 1) t = matvec(pt[i].CSPM_L, t);
        return t;
    }

    // ---- counting sort (eng/particle_system.py:228-257) ----
    void sort() {
        const long G = prm.grid_num_total;
        std::vector<int> cnt(G + 1, 0);
        for (int i = 0; i < n; ++i) {
            int c[3];
            bool ok = pos_to_index(pt[i].x, c);
            long f = flatten(c);
            if (!ok || f < 0 || f >= G) { f = G; err |= ORC_ERR_CELL_OOB; }
            pt[i].grid_ids = (int)f;
            cnt[f] += 1;
        }
        grid_end.assign(G + 1, 0);
        int acc = 0;
        for (long c = 0; c <= G; ++c) { acc += cnt[c]; grid_end[c] = acc; }
        grid_tmp = cnt;
        for (int k = 0; k < n; ++k) {  // descending index, post-decrement from the cell end
            int I = n - 1 - k;
            int g = pt[I].grid_ids;
            int base = g - 1 >= 0 ? grid_end[g - 1] : 0;
            grid_tmp[g] -= 1;
            pt[I].id_new = grid_tmp[g] + base;
        }
        pt_buf.resize(n);
        for (int i = 0; i < n; ++i) pt_buf[pt[i].id_new] = pt[i];
        pt.swap(pt_buf);
    }

    // ---- CSPM (eng/solver_sph_base.py:386-423) ----
    void kernel_corr() {
        #pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < n; ++i) {
            double s = 0.0;
            for_all_neighbors(i, [&](int j) {
                if (is_flow(j)) s += pt[j].m_V * W(vsub(pt[i].x, pt[j].x));
            });
            pt[i].CSPM_f = s != 0.0 ? 1.0 / s : 1.0;
        }
        if (prm.kernel_corr != 1) return;
        #pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < n; ++i) {
            M3 inv = meye();
            if (is_flow(i)) {
                M3 L = mzero();
                for_all_neighbors(i, [&](int j) {
                    if (same_type(j, i)) {
                        V3 t = dW(vsub(pt[i].x, pt[j].x));
                        L = madd(L, outer(vscale(pt[j].m_V, vsub(pt[j].x, pt[i].x)), t));
                    }
                });
                if (dim == 2) {
                    if (std::fabs(det2(L)) > EPS) inv = inv2_fill0(L);
                } else {
                    if (std::fabs(det3(L)) > EPS) inv = inv3(L);
                }
            }
            pt[i].CSPM_L = inv;
        }
    }

    void init_real2tmp() {  // eng/solver_sph_base.py:67-74
        #pragma omp parallel for
        for (int i = 0; i < n; ++i) {
            if (is_real(i)) { pt[i].density_tmp = pt[i].density; pt[i].v_tmp = pt[i].v; }
            if (is_soil(i)) pt[i].stress_tmp = pt[i].stress;
        }
    }

    // ---- shared boundary extrapolation pieces (eng/solver_sph_base.py:648-669) ----
    V3 bdy_vel_sum(int i) const {
        V3 r = vzero();
        for_all_neighbors(i, [&](int j) {
            if (is_flow(j)) {
                double w = W(vsub(pt[i].x, pt[j].x));
                for (int d = 0; d < 3; ++d) r.c[d] += pt[j].m_V * pt[j].v_tmp.c[d] * w;
            }
        });
        return r;
    }
    void set_bdy_vel(int i, const V3& s) {
        for (int d = 0; d < 3; ++d) pt[i].v_tmp.c[d] = 2 * pt[i].v.c[d] - s.c[d] * pt[i].CSPM_f;
    }
    M3 bdy_stress_sum(int i) const {
        M3 r = mzero();
        M3 Gd = mdiag(v3(g[0], g[1], g[2]));
        for_all_neighbors(i, [&](int j) {
            if (is_flow(j)) {
                V3 dx = vsub(pt[i].x, pt[j].x);
                double w = W(dx);
                M3 t = madd(pt[j].stress_tmp, mmul_elem(mscale(pt[j].density_tmp, Gd), mdiag(dx)));
                r = madd(r, mscale(w, mscale(pt[j].m_V, t)));
            }
        });
        return r;
    }
    V3 rep_force(const V3& r) const {  // eng/solver_sph_base.py:675-689
        double rn = vnorm(r);
        double rj = prm.particle_diameter;
        double chi = (rn > 0.0 && rn < rj) ? 1.0 - rn / rj : 0.0;
        double gamma = rn / (0.75 * prm.smoothing_len);
        double f = 0.0;
        if (gamma > 0 && gamma <= 2.0 / 3.0) f = 2.0 / 3.0;
        else if (gamma > 2.0 / 3.0 && gamma <= 1) f = 2 * gamma - 1.5 * (gamma * gamma);
        else if (gamma > 1 && gamma < 2) f = 0.5 * ((2 - gamma) * (2 - gamma));
        double s = 0.01 * (vsound * vsound) * chi * f / (rn * rn);
        return vscale(s, r);
    }
    bool rep_on() const { return prm.boundary == 3 || prm.boundary == 4; }

    // ---- WCSPH one_step (eng/solver_sph_wc.py:82-127) ----
    void one_step_wc() {
        const double rho0 = prm.density0;
        #pragma omp parallel for
        for (int i = 0; i < n; ++i) {
            if (is_fluid(i)) {
                double ratio = pt[i].density_tmp / rho0;
                double pw = prm.exponent_is_int ? powi(ratio, (long)prm.exponent) : std::pow(ratio, prm.exponent);
                pt[i].pressure = std::max(prm.stiffness * (pw - 1.0), 0.0);
            }
        }
        #pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < n; ++i) {
            if (is_bdy(i) || is_rigid(i)) {
                set_bdy_vel(i, bdy_vel_sum(i));
                pt[i].density_tmp = rho0;
                double s = 0.0;
                for_all_neighbors(i, [&](int j) {
                    if (is_flow(j)) {
                        V3 dx = vsub(pt[i].x, pt[j].x);
                        s += pt[j].m_V * (pt[j].pressure + pt[j].density_tmp * g[1] * (pt[i].x.c[1] - pt[j].x.c[1])) * W(dx);
                    }
                });
                pt[i].pressure = std::max(s * pt[i].CSPM_f, 0.0);
            }
            if (is_rigid_dynamic(i)) pt[i].d_vel = v3(g[0], g[1], g[2]);
        }
        #pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < n; ++i) {
            if (is_fluid(i)) {
                double dd = 0.0;
                for_all_neighbors(i, [&](int j) {
                    V3 k = dW_corr(i, j);
                    V3 a = vscale(pt[j].m_V, vsub(pt[i].v_tmp, pt[j].v_tmp));
                    dd += vdot(a, k);
                });
                pt[i].d_density = dd * pt[i].density_tmp;
                V3 dv = vzero();
                for_all_neighbors(i, [&](int j) { dv = vadd(dv, wc_force_pair(i, j)); });
                if (rep_on()) {
                    for_all_neighbors(i, [&](int j) {
                        if (is_rep(j)) dv = vadd(dv, rep_force(vsub(pt[i].x, pt[j].x)));
                    });
                }
                pt[i].d_vel = vadd(dv, v3(g[0], g[1], g[2]));
            }
            if (is_rigid_static(i)) pt[i].d_vel = vzero();
        }
        if (n_rigid_dyn) rigid_reaction();
    }

    // One neighbour's term of calc_d_vel_task (eng/solver_sph_wc.py:34-71):
    // tmp = viscosity_force(i, j) + pressure_force(i, j).
    V3 wc_force_pair(int i, int j) const {
        const double rho0 = prm.density0;
        V3 xij = vsub(pt[i].x, pt[j].x);
        V3 visc = vzero();
        double xn = vnorm(xij);
        if (is_fluid(j)) {
            double c = visc_fac * pt[j].m_V * std::min(vdot(vsub(pt[i].v_tmp, pt[j].v_tmp), xij), 0.0) / (xn * xn + eps_h2);
            visc = vscale(c, dW(xij));
        } else if (is_bdy(j) || is_rigid(j)) {
            double c = visc_fac * pt[j].m_V * rho0 / pt[i].density_tmp * std::min(vdot(vsub(pt[i].v_tmp, pt[j].v_tmp), xij), 0.0) / (xn * xn + eps_h2);
            visc = vscale(c, dW(xij));
        }
        double cp = -rho0 * pt[j].m_V * (pt[i].pressure / (pt[i].density_tmp * pt[i].density_tmp) + pt[j].pressure / (pt[j].density_tmp * pt[j].density_tmp));
        V3 press = vscale(cp, dW(xij));
        return vadd(visc, press);
    }

    // The reaction on dynamic rigid particles: the reference subtracts each flow particle's
    // pair term from its dynamic rigid neighbour inside the flow particle's loop
    // (`pt[j].d_vel -= tmp`, eng/solver_sph_wc.py:70-71, eng/solver_sph_muI.py:45-46,
    // eng/solver_sph_dp.py:164-165), an unsynchronised scatter.  Serially, rigid particle j
    // receives the terms of its flow neighbours i in ascending i, which is the order of j's
    // own neighbour traversal (cells in increasing flattened index, particles ascending):
    // here each j gathers them in that order, starting from the g its first loop set.
    void rigid_reaction() {
        #pragma omp parallel for schedule(dynamic, 64)
        for (int j = 0; j < n; ++j) {
            if (!is_rigid_dynamic(j)) continue;
            V3 d = pt[j].d_vel;
            for_all_neighbors(j, [&](int i) {
                if (prm.solver == 1 ? is_fluid(i) : is_soil(i))
                    d = vsub(d, prm.solver == 1 ? wc_force_pair(i, j) : stress_div_pair(i, j));
            });
            pt[j].d_vel = d;
        }
    }

    // ---- shared soil pieces ----
    M3 v_grad_sum(int i) const {  // calc_v_grad_task (eng/solver_sph_base.py:187-193)
        M3 r = mzero();
        for_all_neighbors(i, [&](int j) {
            V3 t = dW_corr(i, j);
            r = madd(r, outer(vscale(pt[j].m_V, vsub(pt[j].v_tmp, pt[i].v_tmp)), t));
        });
        return r;
    }
    double d_density_sum(int i) const {  // calc_d_density_task (eng/solver_sph_base.py:196-203)
        double r = 0.0;
        for_all_neighbors(i, [&](int j) {
            V3 k = dW_corr(i, j);
            r += vdot(vscale(pt[j].m_V, vsub(pt[i].v_tmp, pt[j].v_tmp)), k);
        });
        return r;
    }
    // One neighbour's term of calc_d_vel_from_stress_task (eng/solver_sph_muI.py:39-46,
    // eng/solver_sph_dp.py:157-165): tmp = m_Vj rho~_j (s~_j / rho~_j^2 + s~_i / rho~_i^2) grad~W_ij.
    V3 stress_div_pair(int i, int j) const {
        double rj2 = pt[j].density_tmp * pt[j].density_tmp;
        double ri2 = pt[i].density_tmp * pt[i].density_tmp;
        M3 M;
        for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q)
                M.m[p][q] = (pt[j].stress_tmp.m[p][q] / rj2 + pt[i].stress_tmp.m[p][q] / ri2) + 0.0 * (p == q ? 1.0 : 0.0);
        M3 S = mscale(pt[j].m_V * pt[j].density_tmp, M);
        return matvec(S, dW_corr(i, j));
    }
    V3 stress_div_sum(int i) const {  // calc_d_vel_from_stress_task summed over the neighbours
        V3 r = vzero();
        for_all_neighbors(i, [&](int j) { r = vadd(r, stress_div_pair(i, j)); });
        return r;
    }
    V3 damping(int i) const {  // calc_viscous_damping (eng/solver_sph_base.py:714-715)
        double s = -prm.damping_eps * std::sqrt(damp_E / (pt[i].density_tmp * h2));
        return vscale(s, pt[i].v_tmp);
    }
    void soil_bdy(bool density_from_sum) {  // boundary loops of mu(I) / DP
        const double rho0 = prm.density0;
        #pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < n; ++i) {
            if (is_bdy(i) || is_rigid(i)) {
                set_bdy_vel(i, bdy_vel_sum(i));
                if (density_from_sum) {
                    double s = 0.0;
                    for_all_neighbors(i, [&](int j) {
                        if (is_flow(j)) s += pt[j].m_V * pt[j].density_tmp * W(vsub(pt[i].x, pt[j].x));
                    });
                    pt[i].density_tmp = std::max(s * pt[i].CSPM_f, rho0);
                } else {
                    pt[i].density_tmp = rho0;
                }
                M3 s = bdy_stress_sum(i);
                for (int p = 0; p < 3; ++p) for (int q = 0; q < 3; ++q) pt[i].stress_tmp.m[p][q] = s.m[p][q] * pt[i].CSPM_f;
            }
            if (is_rigid_dynamic(i)) pt[i].d_vel = v3(g[0], g[1], g[2]);
        }
    }

    // ---- mu(I) one_step (eng/solver_sph_muI.py:62-131) ----
    void one_step_mui() {
        const double rho0 = prm.density0;
        #pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < n; ++i) {
            if (!is_soil(i)) continue;
            P& a = pt[i];
            a.v_grad = v_grad_sum(i);
            a.d_density = d_density_sum(i) * a.density_tmp;
            a.pressure = std::max(vsound2 * (a.density - rho0), 0.0);
            M3 er = mscale(0.5, madd(a.v_grad, mT(a.v_grad)));
            double dbdot = std::sqrt(0.5 * msum(mmul_elem(er, er))) + EPS;
            double s = 0.0 + (prm.coh + a.pressure * mu) / dbdot;
            M3 tau = mscale(s, er);
            a.stress_tmp = msub(tau, mscale(a.pressure, meye()));
            M3 edev = msub(er, mscale(mtrace(er) / 3.0, meye()));
            a.d_strain_equ = std::sqrt(msum(mmul_elem(edev, edev)) * 2 / 3);
        }
        soil_bdy(true);
        #pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < n; ++i) {
            if (!is_soil(i)) continue;
            V3 dv = stress_div_sum(i);
            if (rep_on()) {
                for_all_neighbors(i, [&](int j) {
                    if (is_rep(j)) dv = vadd(dv, rep_force(vsub(pt[i].x, pt[j].x)));
                });
            }
            V3 fd = damping(i);
            pt[i].d_vel = vadd(vadd(dv, v3(g[0], g[1], g[2])), fd);
        }
        #pragma omp parallel for
        for (int i = 0; i < n; ++i)
            if (is_rigid_static(i)) pt[i].d_vel = vzero();
        if (n_rigid_dyn) rigid_reaction();
    }

    // ---- Drucker-Prager pieces (eng/solver_sph_dp.py:42-208) ----
    void dp_invariants(const M3& st, M3& s, double& I1, double& sJ2, double& f) const {
        s = msub(st, mscale(mtrace(st) / 3.0, meye()));
        I1 = mtrace(st);
        sJ2 = std::sqrt(0.5 * msum(mmul_elem(s, s)));
        f = sJ2 + alpha * I1 - k_c;
    }
    M3 adapt_stress(const M3& st) const {
        M3 res = st, s;
        double I1, sJ2, f;
        dp_invariants(res, s, I1, sJ2, f);
        if (f > EPS_F) {
            if (f > sJ2) {
                double t = (I1 - kc_over_alpha) / 3.0;
                res = msub(res, mscale(t, meye()));
            }
            dp_invariants(res, s, I1, sJ2, f);
            double r = (-I1 * alpha + k_c) / sJ2;
            M3 out;
            for (int p = 0; p < 3; ++p)
                for (int q = 0; q < 3; ++q)
                    out.m[p][q] = r * s.m[p][q] + ((p == q ? 1.0 : 0.0) * I1) / 3.0;
            res = out;
        }
        return res;
    }
    int flag_dp(const M3& st) const {
        M3 s; double I1, sJ2, f;
        dp_invariants(st, s, I1, sJ2, f);
        int flag = 1;
        if (f < -EPS_F) flag = 0;
        else if (f > EPS_F) flag = (f >= sJ2) ? 3 : 2;
        return flag;
    }
    static double dev_component(const M3& t) { return std::sqrt(msum(mmul_elem(t, t)) * 2 / 3); }
    void d_stress_bui(P& a) const {  // calc_d_stress_Bui2008
        M3 s; double I1, sJ2, f_old;
        dp_invariants(a.stress_tmp, s, I1, sJ2, f_old);
        M3 er = mscale(0.5, madd(a.v_grad, mT(a.v_grad)));
        M3 wr = mscale(0.5, msub(a.v_grad, mT(a.v_grad)));
        M3 J;
        for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q)
                J.m[p][q] = a.stress_tmp.m[p][0] * wr.m[q][0] + a.stress_tmp.m[p][1] * wr.m[q][1]
                          + a.stress_tmp.m[p][2] * wr.m[q][2] + a.stress_tmp.m[0][q] * wr.m[p][0]
                          + a.stress_tmp.m[1][q] * wr.m[p][1] + a.stress_tmp.m[2][q] * wr.m[p][2];
        double tr = mtrace(er);
        M3 edev = msub(er, mscale(tr / 3.0, meye()));
        M3 te;
        for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q)
                te.m[p][q] = twoG * edev.m[p][q] + (K * tr) * (p == q ? 1.0 : 0.0);
        double lam = 0.0;
        M3 tg = mzero();
        bool plastic = f_old >= -EPS_F && sJ2 > EPS;
        if (plastic) {
            lam = (three_aK * tr + (G / sJ2) * msum(mmul_elem(s, er))) / lam_den;
            for (int p = 0; p < 3; ++p)
                for (int q = 0; q < 3; ++q)
                    tg.m[p][q] = lam * (nine_K_sin * (p == q ? 1.0 : 0.0) + G / sJ2 * s.m[p][q]);
        }
        a.d_stress = msub(madd(J, te), tg);
        a.d_strain_equ = dev_component(edev);
        a.d_strain_equ_p = 0.0;
        if (plastic) {
            double gp = sJ2 + 3 * I1 * sin_dila;
            double gd = gp - a.g_p;
            M3 ep = mzero();
            for (int p = 0; p < 3; ++p)
                for (int q = 0; q < 3; ++q)
                    if (std::fabs(a.d_stress.m[p][q]) > EPS) ep.m[p][q] = gd / a.d_stress.m[p][q];
            ep = mscale(lam, ep);
            M3 epd = msub(ep, mscale(mtrace(ep) / 3.0, meye()));
            a.d_strain_equ_p = dev_component(epd);
        }
    }

    // ---- DP one_step (eng/solver_sph_dp.py:210-274) ----
    void one_step_dp() {
        #pragma omp parallel for
        for (int i = 0; i < n; ++i)
            if (is_soil(i)) pt[i].stress_tmp = adapt_stress(pt[i].stress_tmp);
        soil_bdy(false);
        #pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < n; ++i) {
            if (!is_soil(i)) continue;
            P& a = pt[i];
            a.v_grad = v_grad_sum(i);
            a.d_density = d_density_sum(i) * a.density_tmp;
            d_stress_bui(a);
            V3 dv = stress_div_sum(i);
            V3 fd = damping(i);
            a.d_vel = vadd(vadd(dv, v3(g[0], g[1], g[2])), fd);
        }
        #pragma omp parallel for
        for (int i = 0; i < n; ++i)
            if (is_rigid_static(i)) pt[i].d_vel = vzero();
        if (n_rigid_dyn) rigid_reaction();
    }

    void one_step() {
        if (prm.solver == 1) one_step_wc();
        else if (prm.solver == 2) one_step_mui();
        else one_step_dp();
    }

    // ---- integrators (eng/solver_sph_base.py:79-180) ----
    void set_volume(P& a) { a.m_V = a.mass / a.density; }
    void advect_full() {  // advect_SE == advect_LF
        const double dt = prm.dt;
        #pragma omp parallel for
        for (int i = 0; i < n; ++i) {
            P& a = pt[i];
            if (is_real(i)) {
                a.density += dt * a.d_density;
                set_volume(a);
                for (int d = 0; d < 3; ++d) a.v.c[d] += dt * a.d_vel.c[d];
            }
            if (is_soil(i)) a.stress = madd(a.stress, mscale(dt, a.d_stress));
        }
    }
    void advect_lf_half() {
        const double hdt = 0.5 * prm.dt;
        #pragma omp parallel for
        for (int i = 0; i < n; ++i) {
            P& a = pt[i];
            if (is_real(i)) {
                a.density_tmp += hdt * a.d_density;
                a.m_V = a.mass / a.density_tmp;
                for (int d = 0; d < 3; ++d) a.v_tmp.c[d] += hdt * a.d_vel.c[d];
            }
            if (is_soil(i)) a.stress_tmp = madd(a.stress_tmp, mscale(hdt, a.d_stress));
        }
    }
    void rk_init() {
        #pragma omp parallel for
        for (int i = 0; i < n; ++i) {
            if (is_real(i)) { pt[i].d_density_RK = 0.0; pt[i].d_vel_RK = vzero(); }
            if (is_soil(i)) pt[i].d_stress_RK = mzero();
        }
    }
    void rk_update(int m) {
        #pragma omp parallel for
        for (int i = 0; i < n; ++i) {
            P& a = pt[i];
            if (is_real(i)) {
                a.d_density_RK += a.d_density * m;
                for (int d = 0; d < 3; ++d) a.d_vel_RK.c[d] += a.d_vel.c[d] * m;
            }
            if (is_soil(i)) a.d_stress_RK = madd(a.d_stress_RK, mscale((double)m, a.d_stress));
        }
    }
    void rk_stage() {
        const double hdt = 0.5 * prm.dt;
        #pragma omp parallel for
        for (int i = 0; i < n; ++i) {
            P& a = pt[i];
            if (is_real(i)) {
                a.density_tmp = hdt * a.d_density + a.density;
                a.m_V = a.mass / a.density_tmp;
                for (int d = 0; d < 3; ++d) a.v_tmp.c[d] = hdt * a.d_vel.c[d] + a.v.c[d];
            }
            if (is_soil(i))
                for (int p = 0; p < 3; ++p) for (int q = 0; q < 3; ++q)
                    a.stress_tmp.m[p][q] = hdt * a.d_stress.m[p][q] + a.stress.m[p][q];
        }
    }
    void rk_final() {
        const double dt6 = prm.dt / 6.0;
        #pragma omp parallel for
        for (int i = 0; i < n; ++i) {
            P& a = pt[i];
            if (is_real(i)) {
                a.density += dt6 * a.d_density_RK;
                set_volume(a);
                for (int d = 0; d < 3; ++d) a.v.c[d] += dt6 * a.d_vel_RK.c[d];
            }
            if (is_soil(i)) a.stress = madd(a.stress, mscale(dt6, a.d_stress_RK));
        }
    }
    void substep() {
        switch (prm.time_integration) {
        case 1: one_step(); advect_full(); break;
        case 2: one_step(); advect_lf_half(); one_step(); advect_full(); break;
        case 4: {
            rk_init();
            const int m[4] = {1, 2, 2, 1};
            for (int s = 0; s < 4; ++s) { one_step(); rk_update(m[s]); if (s < 3) rk_stage(); }
            rk_final();
            break;
        }
        default: err |= ORC_ERR_BAD_CONFIG;
        }
    }

    void advect_pos() {  // eng/solver_sph_base.py:224-238 (two-phase)
        const double dt = prm.dt;
        std::vector<V3> xs(n, vzero());
        std::vector<char> use(n, 0);
        #pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < n; ++i) {
            if (is_real(i) && prm.xsph && pt[i].is_dynamic) {
                V3 s = vzero();
                for_all_neighbors(i, [&](int j) {
                    if (same_type(i, j)) {
                        double w = W(vsub(pt[i].x, pt[j].x));
                        for (int d = 0; d < 3; ++d) s.c[d] += pt[j].m_V * (pt[j].v.c[d] - pt[i].v.c[d]) * w;
                    }
                });
                xs[i] = s;
                use[i] = 1;
            }
        }
        #pragma omp parallel for
        for (int i = 0; i < n; ++i) {
            if (!is_real(i)) continue;
            P& a = pt[i];
            if (use[i]) for (int d = 0; d < 3; ++d) a.x.c[d] += dt * (a.v.c[d] + 0.5 * xs[i].c[d]);
            else for (int d = 0; d < 3; ++d) a.x.c[d] += dt * a.v.c[d];
        }
    }

    void chk_density(P& a) { a.density = std::max(prm.density0, a.density); set_volume(a); }
    void advect_something() {
        if (prm.solver == 1) {
            #pragma omp parallel for
            for (int i = 0; i < n; ++i) if (is_fluid(i)) chk_density(pt[i]);
        } else if (prm.solver == 2) {  // two-phase (see header)
            #pragma omp parallel for
            for (int i = 0; i < n; ++i) {
                if (!is_soil(i)) continue;
                chk_density(pt[i]);
                pt[i].strain_equ += prm.dt * pt[i].d_strain_equ;
                pt[i].stress = pt[i].stress_tmp;
            }
            std::vector<M3> reg(n);
            #pragma omp parallel for schedule(dynamic, 256)
            for (int i = 0; i < n; ++i) {
                if (!is_soil(i)) continue;
                M3 s = mzero();
                for_all_neighbors(i, [&](int j) {
                    if (pt[j].mat_type == pt[i].mat_type) {
                        double w = W(vsub(pt[i].x, pt[j].x));
                        s = madd(s, mscale(w, mscale(pt[j].m_V, pt[j].stress)));
                    }
                });
                for (int p = 0; p < 3; ++p) for (int q = 0; q < 3; ++q) reg[i].m[p][q] = s.m[p][q] * pt[i].CSPM_f;
            }
            #pragma omp parallel for
            for (int i = 0; i < n; ++i) if (is_soil(i)) pt[i].stress = reg[i];
        } else {
            #pragma omp parallel for
            for (int i = 0; i < n; ++i) {
                if (!is_soil(i)) continue;
                P& a = pt[i];
                chk_density(a);
                a.flag_retmap = flag_dp(a.stress);
                a.stress = adapt_stress(a.stress);
                a.strain_equ += prm.dt * a.d_strain_equ;
                a.strain_equ_p += prm.dt * a.d_strain_equ_p;
            }
        }
    }

    void enforce_boundary() {  // eng/solver_sph_base.py:525-601
        const double r = prm.particle_radius - EPS;
        #pragma omp parallel for
        for (int i = 0; i < n; ++i) {
            bool on = prm.boundary == 1 ? (is_flow(i) || is_rigid_dynamic(i)) : is_rigid_dynamic(i);
            if (!on) continue;
            P& a = pt[i];
            V3 pos = a.x;
            V3 nrm = vzero();
            if (pos.c[0] > prm.domain_end[0] - r) { nrm.c[0] += 1.0; a.x.c[0] = prm.domain_end[0] - r; }
            if (pos.c[0] <= prm.domain_start[0] + r) { nrm.c[0] += -1.0; a.x.c[0] = prm.domain_start[0] + r; }
            if (pos.c[1] <= prm.domain_start[1] + r) { nrm.c[1] += -1.0; a.x.c[1] = prm.domain_start[1] + r; }
            if (dim == 3) {
                if (pos.c[2] > prm.domain_end[2] - r) { nrm.c[2] += 1.0; a.x.c[2] = prm.domain_end[2] - r; }
                if (pos.c[2] <= prm.domain_start[2] + r) { nrm.c[2] += -1.0; a.x.c[2] = prm.domain_start[2] + r; }
            }
            double ln = vnorm(nrm);
            if (ln > EPS) {
                V3 u = v3(nrm.c[0] / ln, nrm.c[1] / ln, nrm.c[2] / ln);
                double vd = vdot(a.v, u);
                for (int d = 0; d < 3; ++d) a.v.c[d] -= (1.0 + 0.3) * vd * u.c[d];
            }
        }
    }

    void step() {  // SPHBase.step (eng/solver_sph_base.py:41-51)
        sort();
        kernel_corr();
        init_real2tmp();
        substep();
        advect_pos();
        advect_something();
        if (n_rigid_dyn) solve_rigid_body();
        enforce_boundary();
    }

    // calc_cm (eng/solver_sph_base.py:502-511): mass-weighted mean position of object o's
    // dynamic rigid particles, summed in particle order.
    V3 rigid_cm(int o) const {
        double sum_m = 0.0;
        V3 cm = vzero();
        for (int i = 0; i < n; ++i) {
            if (!(is_rigid_dynamic(i) && pt[i].obj_id == o)) continue;
            cm = vadd(cm, vscale(pt[i].mass, pt[i].x));
            sum_m += pt[i].mass;
        }
        return v3(cm.c[0] / sum_m, cm.c[1] / sum_m, cm.c[2] / sum_m);
    }

    // solve_rigid_body / solve_constraints (eng/solver_sph_base.py:472-500): shape matching
    // of every dynamic rigid object.  A = sum m_V rho ((p) (x) q) with p = x - cm,
    // q = x0 - rest cm (the reference's m_V * density * p @ q.T, scalar products first),
    // R the orthogonal polar factor of A (polar3: the reference calls ti.polar_decompose,
    // whose algorithm lives in Taichi; this is Higham's scaled Newton iteration), identity when
    // every entry of R is below 1e-8; then x += (cm + R q) - x.
    void solve_rigid_body() {
        for (size_t k = 0; k < rigid_ids.size(); ++k) {
            const int o = rigid_ids[k];
            const V3 cm = rigid_cm(o);
            M3 A = mzero();
            for (int i = 0; i < n; ++i) {
                if (!(is_rigid_dynamic(i) && pt[i].obj_id == o)) continue;
                const V3 q = vsub(pt[i].x0, rigid_rest_cm[k]);
                const V3 pp = vsub(pt[i].x, cm);
                const double s = pt[i].m_V * pt[i].density;
                const V3 sp = vscale(s, pp);
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) A.m[a][b] = A.m[a][b] + sp.c[a] * q.c[b];
            }
            M3 R = polar3(A);
            bool small = true;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) small = small && std::fabs(R.m[a][b]) < EPS;
            if (small) R = meye();
            #pragma omp parallel for
            for (int i = 0; i < n; ++i) {
                if (!(is_rigid_dynamic(i) && pt[i].obj_id == o)) continue;
                const V3 goal = vadd(cm, matvec(R, vsub(pt[i].x0, rigid_rest_cm[k])));
                const V3 corr = vscale(1.0, vsub(goal, pt[i].x));
                pt[i].x = vadd(pt[i].x, corr);
            }
        }
    }

    void init_stress_geostatic() {  // eng/solver_sph_base.py:249-260
        double ymax = -INFINITY;
        for (int i = 0; i < n; ++i) if (is_soil(i)) ymax = std::max(ymax, pt[i].x.c[1]);
        double K0 = 1.0 - std::sin(prm.fric);
        for (int i = 0; i < n; ++i) {
            if (!is_soil(i)) continue;
            double vs = prm.density0 * g[1] * (ymax - pt[i].x.c[1]);
            pt[i].stress.m[0][0] = K0 * vs;
            pt[i].stress.m[1][1] = vs;
            pt[i].stress.m[2][2] = K0 * vs;
        }
    }
};

}  // namespace

extern "C" {

void* orc_create(const orc_params* prm, int n, const double* x, const double* v, const double* density,
                 const double* mass, const double* m_V, const double* pressure, const double* stress,
                 const int* mat_type, const int* mat_id, const int* obj_id, const int* is_dynamic) {
    Sys* s = new Sys();
    s->prm = *prm;
    s->dim = prm->dim;
    s->n = n;
    s->pt.assign(n, P());
    for (int i = 0; i < n; ++i) {
        P& a = s->pt[i];
        std::memset(&a, 0, sizeof a);
        for (int d = 0; d < 3; ++d) { a.x.c[d] = x[3 * i + d]; a.x0.c[d] = x[3 * i + d]; a.v.c[d] = v[3 * i + d]; }
        a.density = density[i];
        a.mass = mass[i];
        a.m_V = m_V[i];
        a.pressure = pressure[i];
        if (stress) for (int p = 0; p < 3; ++p) for (int q = 0; q < 3; ++q) a.stress.m[p][q] = stress[9 * i + 3 * p + q];
        a.mat_type = mat_type[i];
        a.mat_id = mat_id[i];
        a.obj_id = obj_id[i];
        a.is_dynamic = is_dynamic[i];
        a.id0 = i;
    }
    const double h = prm->smoothing_len;
    s->h1 = 1.0 / h;
    const double pi = 3.141592653589793;
    double k;
    if (prm->kernel == 1) k = prm->dim == 2 ? 7.0 / (4.0 * pi) : 21.0 / (2.0 * pi);
    else k = prm->dim == 2 ? 15.0 / 7.0 / pi : 3.0 / 2.0 / pi;
    s->kk = k * std::pow(s->h1, (double)prm->dim);
    s->visc_fac = 2 * (prm->dim + 2) * prm->viscosity;
    s->h2 = std::pow(h, 2.0);
    s->eps_h2 = 0.01 * s->h2;
    for (int d = 0; d < 3; ++d) s->g[d] = prm->gravity[d];
    if (prm->solver == 1) {
        s->vsound = 60.0;
    } else if (prm->solver == 2) {
        s->mu = std::tan(prm->fric);
        s->vsound = 24.0;
        s->vsound2 = std::pow(24.0, 2.0);
    } else {
        double t = std::tan(prm->fric);
        double den = std::sqrt(9 + 12 * std::pow(t, 2.0));
        s->alpha = t / den;
        s->k_c = 3 * prm->coh / den;
        s->G = prm->E / (2 * (1 + prm->poi));
        s->K = prm->E / (3 * (1 - 2 * prm->poi));
        s->sin_dila = std::sin(prm->dila);
        s->kc_over_alpha = s->k_c / s->alpha;
        s->lam_den = 27.0 * s->alpha * s->K * s->sin_dila + s->G;
        s->three_aK = 3.0 * s->alpha * s->K;
        s->nine_K_sin = 9.0 * s->K * s->sin_dila;
        s->twoG = 2.0 * s->G;
        s->vsound = std::sqrt(prm->E / prm->density0);
    }
    s->damp_E = prm->E;
    if (prm->solver == 3 && prm->init_geostatic) s->init_stress_geostatic();
    // init_rigid_body (eng/solver_sph_base.py:467-470): rest centre of mass of every dynamic
    // rigid object, from the input positions
    for (int i = 0; i < n; ++i) {
        if (!s->is_rigid_dynamic(i)) continue;
        ++s->n_rigid_dyn;
        if (std::find(s->rigid_ids.begin(), s->rigid_ids.end(), s->pt[i].obj_id) == s->rigid_ids.end())
            s->rigid_ids.push_back(s->pt[i].obj_id);
    }
    std::sort(s->rigid_ids.begin(), s->rigid_ids.end());
    for (int o : s->rigid_ids) s->rigid_rest_cm.push_back(s->rigid_cm(o));
    return s;
}

void orc_destroy(void* h) { delete static_cast<Sys*>(h); }

int orc_n(void* h) { return static_cast<Sys*>(h)->n; }

int orc_call(void* h, int what) {
    Sys* s = static_cast<Sys*>(h);
    switch (what) {
    case ORC_SORT: s->sort(); break;
    case ORC_KERNEL_CORR: s->kernel_corr(); break;
    case ORC_INIT_TMP: s->init_real2tmp(); break;
    case ORC_ONE_STEP: s->one_step(); break;
    case ORC_ADVECT_FULL: s->advect_full(); break;
    case ORC_ADVECT_LF_HALF: s->advect_lf_half(); break;
    case ORC_SUBSTEP: s->substep(); break;
    case ORC_ADVECT_POS: s->advect_pos(); break;
    case ORC_ADVECT_SOMETHING: s->advect_something(); break;
    case ORC_ENFORCE_BOUNDARY: s->enforce_boundary(); break;
    case ORC_STEP: s->step(); break;
    default: return -1;
    }
    return s->err;
}

int orc_steps(void* h, int nsteps) {
    Sys* s = static_cast<Sys*>(h);
    for (int k = 0; k < nsteps; ++k) s->step();
    return s->err;
}

// Field read-back by name.  Vectors are (n, 3), matrices (n, 3, 3), scalars (n,);
// integers are returned as doubles.
int orc_get(void* h, const char* name, double* out) {
    Sys* s = static_cast<Sys*>(h);
    std::string f(name);
    const int n = s->n;
    auto vec = [&](V3 P::*m) { for (int i = 0; i < n; ++i) for (int d = 0; d < 3; ++d) out[3 * i + d] = (s->pt[i].*m).c[d]; };
    auto mat = [&](M3 P::*m) { for (int i = 0; i < n; ++i) for (int p = 0; p < 3; ++p) for (int q = 0; q < 3; ++q) out[9 * i + 3 * p + q] = (s->pt[i].*m).m[p][q]; };
    auto sca = [&](double P::*m) { for (int i = 0; i < n; ++i) out[i] = s->pt[i].*m; };
    auto itg = [&](int P::*m) { for (int i = 0; i < n; ++i) out[i] = (double)(s->pt[i].*m); };
    if (f == "x") vec(&P::x); else if (f == "x0") vec(&P::x0); else if (f == "v") vec(&P::v);
    else if (f == "v_tmp") vec(&P::v_tmp); else if (f == "d_vel") vec(&P::d_vel);
    else if (f == "stress") mat(&P::stress); else if (f == "stress_tmp") mat(&P::stress_tmp);
    else if (f == "d_stress") mat(&P::d_stress); else if (f == "v_grad") mat(&P::v_grad);
    else if (f == "CSPM_L") mat(&P::CSPM_L);
    else if (f == "m_V") sca(&P::m_V); else if (f == "density") sca(&P::density);
    else if (f == "mass") sca(&P::mass); else if (f == "pressure") sca(&P::pressure);
    else if (f == "CSPM_f") sca(&P::CSPM_f); else if (f == "d_density") sca(&P::d_density);
    else if (f == "density_tmp") sca(&P::density_tmp); else if (f == "strain_equ") sca(&P::strain_equ);
    else if (f == "d_strain_equ") sca(&P::d_strain_equ); else if (f == "strain_equ_p") sca(&P::strain_equ_p);
    else if (f == "d_strain_equ_p") sca(&P::d_strain_equ_p);
    else if (f == "id0") itg(&P::id0); else if (f == "mat_type") itg(&P::mat_type);
    else if (f == "obj_id") itg(&P::obj_id); else if (f == "mat_id") itg(&P::mat_id);
    else if (f == "is_dynamic") itg(&P::is_dynamic); else if (f == "grid_ids") itg(&P::grid_ids);
    else if (f == "id_new") itg(&P::id_new); else if (f == "flag_retmap") itg(&P::flag_retmap);
    else return -1;
    return 0;
}

// Inclusive end offsets per cell (G + 1 entries; the last bin holds out-of-grid particles).
int orc_grid(void* h, int* out) {
    Sys* s = static_cast<Sys*>(h);
    for (size_t c = 0; c < s->grid_end.size(); ++c) out[c] = s->grid_end[c];
    return (int)s->grid_end.size();
}

// Neighbour lists in traversal order: counts[i] for every particle, then the indices
// concatenated.  Returns the total number of pairs, or -1 when cap is too small.
long orc_neighbors(void* h, int* counts, int* list, long cap) {
    Sys* s = static_cast<Sys*>(h);
    long total = 0;
    for (int i = 0; i < s->n; ++i) {
        int c = 0;
        s->for_all_neighbors(i, [&](int j) {
            if (list && total < cap) list[total] = j;
            ++total; ++c;
        });
        counts[i] = c;
    }
    return (list && total > cap) ? -1 : total;
}

// Density summation: calc_density_task summed by for_all_neighbors
// (eng/solver_sph_wc.py:30-31, eng/particle_system.py:259-269), ret += mass_j W(x_i - x_j)
// in traversal order, for every particle.
int orc_density_sum(void* h, double* out) {
    Sys* s = static_cast<Sys*>(h);
#pragma omp parallel for
    for (int i = 0; i < s->n; ++i) {
        double ret = 0.0;
        s->for_all_neighbors(i, [&](int j) { ret += s->pt[j].mass * s->W(vsub(s->pt[i].x, s->pt[j].x)); });
        out[i] = ret;
    }
    return 0;
}

int orc_error(void* h) { return static_cast<Sys*>(h)->err; }

}  // extern "C"
