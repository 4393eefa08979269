// Hand-written adjoint (reverse mode) of one FP32-mixed mu(I) step, and bitwise state
// snapshots for checkpointed recomputation.
//
// Scope: 2D, mu(I) rheology (solver 2), symplectic Euler, no kernel-gradient correction,
// dummy-particle boundary, no XSPH - the configuration of the differentiable column
// collapse.  One step of that form (eng/solver_sph_base.py:41-91, :224-247;
// eng/solver_sph_muI.py:62-156) maps the state (x, v, rho of the soil particles, v_tmp of
// the dummy particles) to the next state through
//   S_b   = sum_{soil j} m_Vj W_bj,  cf_b = 1 / S_b                            (Shepard)
//   vg_i  = sum_j m_Vj (v~_j - v_i) (x) G_ij d_ij,  dd_i = -sum_j m_Vj (v~_j - v_i) . G_ij d_ij
//   p_i   = max(c^2 (rho_i - rho0), 0),  er = sym(vg),  |e| = sqrt(er:er / 2) + 1e-8
//   s~_i  = (coh + p_i mu) / |e| er - p_i I                                      (mu(I))
//   v~_b  = 2 v_b - cf_b sum m_Vj v_j W_bj,  rho~_b = max(cf_b sum m_Vj rho_j W_bj, rho0)
//   s~_b  = cf_b sum m_Vj (s~_j + diag(rho_j g_a d_bj,a)) W_bj                   (boundary)
//   dv_i  = sum_j m_Vj rho~_j (s~_j / rho~_j^2 + s~_i / rho~_i^2) G_ij d_ij + g
//           - eps sqrt(E / (rho_i h^2)) v_i
//   rho'  = rho + dt rho dd,  v' = v + dt dv,  x' = x + dt v',  rho'' = max(rho', rho0)
// with d_ij = x_i - x_j, grad W_ij = G(|d_ij|) d_ij, v~_j the dummy velocities of the
// previous step.  The stress regularisation of the post-step only rewrites the output
// stress (the next step recomputes s~ from velocities), so it has no adjoint.
//
// tsg_adjoint_step re-runs the step's forward (same kernels, same order, so it repeats the
// forward bit for bit from a loaded snapshot) keeping the step-start state, then runs the
// reverse sweep below on the step's neighbour lists.  Sums over j of a pair term that
// belong to the neighbour's adjoint ("scatter" terms) are evaluated as gathers over the
// neighbour's own list: the pair relation is symmetric, and every soil particle lists all
// its neighbours while every dummy lists its soil neighbours.  Adjoint arithmetic is f32;
// the parameter adjoints accumulate in f64.
#include "tsg_fp32_dev.cuh"

namespace tsg {

using namespace f32;

namespace {

// Step-start copies (sorted order) and the adjoint work arrays.
struct Start {
    float4 *hi, *lo, *vel, *vlo, *vt;
    float* drho;
};
struct A32 {
    float2 *x, *v, *dv, *vn, *b1;
    float *r, *mv, *rt, *dr, *b2, *bs, *dds;
    float4 *s, *b3, *vg;  // full 2 x 2 matrices: (xx, xy, yx, yy)
    double2* gp;          // per-particle (d/d mu, d/d cohesion), reduced in a fixed order
};

// dG/dr of the gradient factor G (grad W = G d).
__device__ __forceinline__ float w_grad_dr(const K32& k, float r) {
    const float q = r * k.h1;
    if (!(r > 1e-8f && q <= 2.f)) return 0.f;
    if (k.kernel == 1) {
        const float q1 = 1.f - 0.5f * q;
        return -1.5f * k.wgrad * k.h1 * q1 * q1;
    }
    if (q <= 1.f) return 1.5f * k.cub1 * k.h1 * k.h1;
    const float f = 2.f - q;
    return k.cub2 * (-2.f * f * k.h1 / r - f * f / (r * r));
}

__device__ __forceinline__ bool soil(float w) { return tf_type(w) == MAT_SOIL; }
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// Pair geometry at the step start: d = x_a - x_b, r, G, dG/dr (r < R only).
struct Pair {
    float dx, dy, r, G, Gp;
};
__device__ __forceinline__ bool pair(const K32& k, const Start& S, int a, int b, Pair& P) {
    float d[3];
    delta<2>(S.hi[a], S.lo[a], S.hi[b], S.lo[b], d);
    const float r2 = dist2<2>(d);
    if (!(r2 < k.R2)) return false;
    P.dx = d[0];
    P.dy = d[1];
    P.r = fast_sqrt(r2);
    P.G = w_grad(k, P.r);
    P.Gp = w_grad_dr(k, P.r);
    return true;
}

// Iterate the step's neighbour list of i (every list fits: the caller checks for overflow).
template <class F>
__device__ __forceinline__ void for_list(const K32& k, const T32& t, int i, F&& body) {
    const int m = t.cnt[i];
    for (int s = 0; s < m; ++s) body(entry_index(k, t.nbr[(size_t)s * k.n + i]));
}

__device__ __forceinline__ void sym2(const T32& t, size_t n, int i, float& xx, float& yy, float& xy) {
    xx = t.sigt[i];
    yy = t.sigt[n + i];
    xy = t.sigt[3 * n + i];
}

// ---- K0: end-of-step adjoint in, post-step / advection / damping reversed ----
__global__ void k_adj_init(K32 k, P32 p, T32 t, Start S, A32 A, const double* __restrict__ ax,
                           const double* __restrict__ av, const double* __restrict__ ar,
                           const double* __restrict__ avt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const int c = p.ids[i].x;
    A.x[i] = A.v[i] = A.dv[i] = A.vn[i] = A.b1[i] = f2(0.f, 0.f);
    A.r[i] = A.mv[i] = A.rt[i] = A.dr[i] = A.b2[i] = A.bs[i] = A.dds[i] = 0.f;
    A.s[i] = A.b3[i] = A.vg[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (soil(S.hi[i].w)) {
        const float2 xb = f2((float)ax[3 * (size_t)c], (float)ax[3 * (size_t)c + 1]);
        const float2 vb = f2((float)av[3 * (size_t)c], (float)av[3 * (size_t)c + 1]);
        const float rb = (float)ar[c];
        const float drho1 = S.drho[i] + k.dt * t.dd[i];  // before the density clamp
        const float rb1 = drho1 > 0.f ? rb : 0.f;
        const float2 vb1 = f2(vb.x + k.dt * xb.x, vb.y + k.dt * xb.y);  // x' = x + dt v'
        const float2 dvb = f2(k.dt * vb1.x, k.dt * vb1.y);               // v' = v + dt dv
        const float rho = k.rho0 + S.drho[i];
        const float damp = -k.damp_eps * sqrtf(k.damp_E / (rho * k.h2));
        const float4 v0 = S.vel[i];
        A.x[i] = xb;
        A.v[i] = f2(vb1.x + dvb.x * damp, vb1.y + dvb.y * damp);
        A.r[i] = rb1 + (dvb.x * v0.x + dvb.y * v0.y) * (-0.5f * damp / rho);
        A.dr[i] = k.dt * rb1;  // rho' = rho + dt d_density
        A.dv[i] = dvb;
    } else {
        A.vn[i] = f2((float)avt[3 * (size_t)c], (float)avt[3 * (size_t)c + 1]);
    }
}

// ---- K2: stress-divergence pair terms (both sides of every soil centre's sum) ----
__global__ void k_adj_mom(K32 k, P32 p, T32 t, Start S, A32 A) {
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    if (kk >= k.n) return;
    const size_t n = k.n;
    const bool ks = soil(S.hi[kk].w);
    float sxx, syy, sxy;
    sym2(t, n, kk, sxx, syy, sxy);
    const float rtk = k.rho0 + t.drt[kk];
    const float irk = 1.f / (rtk * rtk);
    const float mvk = S.lo[kk].w;
    const float2 ak = A.dv[kk];
    float2 ax = f2(0.f, 0.f);
    float4 as = make_float4(0.f, 0.f, 0.f, 0.f);
    float ar = 0.f, amv = 0.f;
    for_list(k, t, kk, [&](int j) {
        Pair P;
        if (!pair(k, S, kk, j, P)) return;
        const bool js = soil(S.hi[j].w);
        if (!ks && !js) return;
        float jxx, jyy, jxy;
        sym2(t, n, j, jxx, jyy, jxy);
        const float rtj = k.rho0 + t.drt[j];
        const float irj = 1.f / (rtj * rtj);
        const float mvj = S.lo[j].w;
        // M = s~_j / rho~_j^2 + s~_k / rho~_k^2 (symmetric in the pair)
        const float Mxx = jxx * irj + sxx * irk, Myy = jyy * irj + syy * irk, Mxy = jxy * irj + sxy * irk;
        if (ks) {  // k is the centre, j the neighbour: g = G d, d = x_k - x_j
            const float gx = P.G * P.dx, gy = P.G * P.dy;
            const float c1 = mvj * rtj * irk;
            as.x += c1 * ak.x * gx; as.y += c1 * ak.x * gy; as.z += c1 * ak.y * gx; as.w += c1 * ak.y * gy;
            const float asg = ak.x * (sxx * gx + sxy * gy) + ak.y * (sxy * gx + syy * gy);
            ar += -2.f * mvj * rtj * asg * irk / rtk;
            const float wx = Mxx * ak.x + Mxy * ak.y, wy = Mxy * ak.x + Myy * ak.y;
            const float sd = wx * P.dx + wy * P.dy;
            const float cm = mvj * rtj, cr = P.Gp / P.r;
            ax.x += cm * (P.G * wx + cr * sd * P.dx);
            ax.y += cm * (P.G * wy + cr * sd * P.dy);
        }
        if (js) {  // j is the centre, k the neighbour: d_jk = -d
            const float2 aj = A.dv[j];
            const float gx = -P.G * P.dx, gy = -P.G * P.dy;
            const float q = aj.x * (Mxx * gx + Mxy * gy) + aj.y * (Mxy * gx + Myy * gy);
            const float ajs = aj.x * (jxx * gx + jxy * gy) + aj.y * (jxy * gx + jyy * gy);
            const float aks = aj.x * (sxx * gx + sxy * gy) + aj.y * (sxy * gx + syy * gy);
            const float drt = mvk * (ajs * irj - aks * irk);  // d(a . T) / d rho~_k
            const float c1 = mvk / rtk;
            as.x += c1 * aj.x * gx; as.y += c1 * aj.x * gy; as.z += c1 * aj.y * gx; as.w += c1 * aj.y * gy;
            if (ks) {
                amv += rtk * q;
                ar += drt;
                const float wx = Mxx * aj.x + Mxy * aj.y, wy = Mxy * aj.x + Myy * aj.y;
                const float sd = -(wx * P.dx + wy * P.dy);
                const float cm = mvk * rtk, cr = P.Gp / P.r;
                ax.x -= cm * (P.G * wx - cr * sd * P.dx);
                ax.y -= cm * (P.G * wy - cr * sd * P.dy);
            } else {
                A.rt[kk] += drt;
            }
        }
    });
    A.s[kk] = make_float4(A.s[kk].x + as.x, A.s[kk].y + as.y, A.s[kk].z + as.z, A.s[kk].w + as.w);
    if (ks) {
        A.x[kk] = f2(A.x[kk].x + ax.x, A.x[kk].y + ax.y);
        A.r[kk] += ar;
        A.mv[kk] += amv;
    }
}

// ---- K3: boundary extrapolation reversed at each dummy (sums recomputed) ----
__global__ void k_adj_bdy(K32 k, P32 p, T32 t, Start S, A32 A) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= k.n || soil(S.hi[b].w) || tf_type(S.hi[b].w) > 0) return;
    const size_t n = k.n;
    float2 B1 = f2(0.f, 0.f);
    float B2 = 0.f, b1 = 0.f, b2 = 0.f;
    float4 B3 = make_float4(0.f, 0.f, 0.f, 0.f);
    for_list(k, t, b, [&](int j) {
        float d[3];
        delta<2>(S.hi[b], S.lo[b], S.hi[j], S.lo[j], d);
        const float r2 = dist2<2>(d);
        if (!(r2 < k.R2) || !soil(S.hi[j].w)) return;
        const float mw = S.lo[j].w * w_val(k, fast_sqrt(r2));
        const float4 v = S.vel[j];
        const float rho = k.rho0 + S.drho[j];
        float jxx, jyy, jxy;
        sym2(t, n, j, jxx, jyy, jxy);
        B1.x += mw * v.x; B1.y += mw * v.y;
        B2 += mw * rho;
        b1 += mw;
        b2 += mw * S.drho[j];
        B3.x += mw * (jxx + rho * k.g[0] * d[0]);
        B3.y += mw * jxy;
        B3.z += mw * jxy;
        B3.w += mw * (jyy + rho * k.g[1] * d[1]);
    });
    const float cf = t.cf[b];
    const float2 avn = A.vn[b];
    const float4 as = A.s[b];
    const bool open = k.rho0 * (cf * b1 - 1.f) + cf * b2 > 0.f;  // rho~_b above rho0
    const float cfb = -(avn.x * B1.x + avn.y * B1.y) + (open ? A.rt[b] * B2 : 0.f) +
                      (as.x * B3.x + as.y * B3.y + as.z * B3.z + as.w * B3.w);
    A.b1[b] = f2(-cf * avn.x, -cf * avn.y);
    A.b2[b] = open ? A.rt[b] * cf : 0.f;
    A.b3[b] = make_float4(cf * as.x, cf * as.y, cf * as.z, cf * as.w);
    A.bs[b] = b1 != 0.f ? -cfb * cf * cf : 0.f;
}

// ---- K4: boundary sums' terms gathered at each soil particle ----
__global__ void k_adj_bdy_soil(K32 k, P32 p, T32 t, Start S, A32 A) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k.n || !soil(S.hi[j].w)) return;
    const size_t n = k.n;
    float jxx, jyy, jxy;
    sym2(t, n, j, jxx, jyy, jxy);
    const float mvj = S.lo[j].w;
    const float4 v = S.vel[j];
    const float rho = k.rho0 + S.drho[j];
    float2 ax = f2(0.f, 0.f), av = f2(0.f, 0.f);
    float4 as = make_float4(0.f, 0.f, 0.f, 0.f);
    float amv = 0.f, ar = 0.f;
    for_list(k, t, j, [&](int b) {
        if (tf_type(S.hi[b].w) > 0) return;
        float d[3];
        delta<2>(S.hi[b], S.lo[b], S.hi[j], S.lo[j], d);  // d_bj = x_b - x_j
        const float r2 = dist2<2>(d);
        if (!(r2 < k.R2)) return;
        const float r = fast_sqrt(r2);
        const float W = w_val(k, r), G = w_grad(k, r);
        const float2 B1 = A.b1[b];
        const float B2 = A.b2[b], BS = A.bs[b];
        const float4 B3 = A.b3[b];
        const float Dxx = rho * k.g[0] * d[0], Dyy = rho * k.g[1] * d[1];
        const float T1 = B1.x * v.x + B1.y * v.y;
        const float T3 = B3.x * (jxx + Dxx) + B3.y * jxy + B3.z * jxy + B3.w * (jyy + Dyy);
        const float coef = T1 + B2 * rho + T3 + BS;
        const float wbar = mvj * coef;
        amv += W * coef;
        av.x += mvj * W * B1.x; av.y += mvj * W * B1.y;
        ar += mvj * W * (B2 + B3.x * k.g[0] * d[0] + B3.w * k.g[1] * d[1]);
        const float mw = mvj * W;
        as.x += mw * B3.x; as.y += mw * B3.y; as.z += mw * B3.z; as.w += mw * B3.w;
        ax.x += -wbar * G * d[0] - mw * rho * B3.x * k.g[0];
        ax.y += -wbar * G * d[1] - mw * rho * B3.w * k.g[1];
    });
    A.x[j] = f2(A.x[j].x + ax.x, A.x[j].y + ax.y);
    A.v[j] = f2(A.v[j].x + av.x, A.v[j].y + av.y);
    A.s[j] = make_float4(A.s[j].x + as.x, A.s[j].y + as.y, A.s[j].z + as.z, A.s[j].w + as.w);
    A.mv[j] += amv;
    A.r[j] += ar;
}

// v~ at the step start as hi + lo: the soil velocity (compensated), the dummies' previous
// extrapolated velocity (single f32).
struct Vc {
    float hx, hy, lx, ly;
};
__device__ __forceinline__ Vc vt_start(const Start& S, int j) {
    if (soil(S.hi[j].w)) return {S.vel[j].x, S.vel[j].y, S.vlo[j].x, S.vlo[j].y};
    return {S.vt[j].x, S.vt[j].y, 0.f, 0.f};
}
__device__ __forceinline__ float2 vdiff(const Vc& a, const Vc& b) {  // a - b
    return f2(dv_comp(a.hx, a.lx, b.hx, b.lx), dv_comp(a.hy, a.ly, b.hy, b.ly));
}

// ---- K5: mu(I) stress and continuity reversed at each soil particle, its own side of
// the velocity-gradient sums; parameter adjoints ----
__global__ void k_adj_stress(K32 k, P32 p, T32 t, Start S, A32 A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    double gmu = 0.0, gcoh = 0.0;
    if (soil(S.hi[i].w)) {
        const Vc vi = vt_start(S, i);
        float vxx = 0.f, vxy = 0.f, vyx = 0.f, vyy = 0.f;
        for_list(k, t, i, [&](int j) {
            Pair P;
            if (!pair(k, S, i, j, P)) return;
            const float mvj = S.lo[j].w;
            const float2 u = vdiff(vt_start(S, j), vi);
            const float ux = mvj * u.x, uy = mvj * u.y;
            const float gx = P.G * P.dx, gy = P.G * P.dy;
            vxx += ux * gx; vxy += ux * gy; vyx += uy * gx; vyy += uy * gy;
        });
        const float exx = vxx, eyy = vyy, exy = 0.5f * (vxy + vyx);
        const float sJ = sqrtf(0.5f * (exx * exx + eyy * eyy + 2.f * exy * exy));
        const float dbdot = sJ + (float)EPS;
        const float drho0 = S.drho[i];
        const float pr = fmaxf(k.c2 * drho0, 0.f);
        const float sc = (k.coh + pr * k.mu) / dbdot;
        const float4 a = A.s[i];
        const float scb = a.x * exx + a.y * exy + a.z * exy + a.w * eyy;
        float exxb = sc * a.x, exyb = sc * a.y, eyxb = sc * a.z, eyyb = sc * a.w;
        const float pb = -(a.x + a.w) + scb * k.mu / dbdot;
        const float dbb = -scb * sc / dbdot;
        gmu = (double)scb * pr / dbdot;
        gcoh = (double)scb / dbdot;
        if (sJ > 0.f) {
            const float c = dbb / (2.f * sJ);
            exxb += c * exx; eyyb += c * eyy; exyb += c * exy; eyxb += c * exy;
        }
        const float rtl = k.rho0 + drho0;
        const float ddb = A.dr[i] * rtl;                  // d_density = rho~ dd
        float ar = (drho0 > 0.f ? pb * k.c2 : 0.f) + A.dr[i] * (t.dd[i] / rtl);
        const float gxx = exxb, gyy = eyyb, gxy = 0.5f * (exyb + eyxb);  // er = sym(vg)
        A.vg[i] = make_float4(gxx, gxy, gxy, gyy);
        A.dds[i] = ddb;
        float2 av = f2(0.f, 0.f), ax = f2(0.f, 0.f);
        for_list(k, t, i, [&](int j) {
            Pair P;
            if (!pair(k, S, i, j, P)) return;
            const float mvj = S.lo[j].w;
            const float2 u = vdiff(vt_start(S, j), vi);
            const float ux = u.x, uy = u.y;
            const float gx = P.G * P.dx, gy = P.G * P.dy;
            av.x -= mvj * (gxx * gx + gxy * gy - ddb * gx);
            av.y -= mvj * (gxy * gx + gyy * gy - ddb * gy);
            const float hx = mvj * (gxx * ux + gxy * uy - ddb * ux);
            const float hy = mvj * (gxy * ux + gyy * uy - ddb * uy);
            const float cr = P.Gp / P.r * (hx * P.dx + hy * P.dy);
            ax.x += P.G * hx + cr * P.dx;
            ax.y += P.G * hy + cr * P.dy;
        });
        A.v[i] = f2(A.v[i].x + av.x, A.v[i].y + av.y);
        A.x[i] = f2(A.x[i].x + ax.x, A.x[i].y + ax.y);
        A.r[i] += ar;
    }
    A.gp[i] = make_double2(gmu, gcoh);
}

// Parameter adjoints summed in a fixed order (one block, strided partials, tree), so that
// repeated reversals of the same step give the same bits.
__global__ void k_adj_params(int n, const double2* __restrict__ gp, double* __restrict__ pbar) {
    __shared__ double smu[256], sco[256];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        a += gp[i].x;
        b += gp[i].y;
    }
    smu[threadIdx.x] = a;
    sco[threadIdx.x] = b;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            smu[threadIdx.x] += smu[threadIdx.x + w];
            sco[threadIdx.x] += sco[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        pbar[0] += smu[0];
        pbar[1] += sco[0];
    }
}

// ---- K6: the neighbour side of the velocity-gradient / continuity sums ----
__global__ void k_adj_vgrad(K32 k, P32 p, T32 t, Start S, A32 A) {
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    if (kk >= k.n) return;
    const bool ks = soil(S.hi[kk].w);
    const float mvk = S.lo[kk].w;
    const Vc vk = vt_start(S, kk);
    float2 av = f2(0.f, 0.f), ax = f2(0.f, 0.f);
    float amv = 0.f;
    for_list(k, t, kk, [&](int i) {
        if (!soil(S.hi[i].w)) return;
        Pair P;
        if (!pair(k, S, kk, i, P)) return;
        const float4 g4 = A.vg[i];
        const float ddb = A.dds[i];
        const float2 u = vdiff(vk, vt_start(S, i));           // u_ik = v~_k - v~_i
        const float ux = u.x, uy = u.y;
        const float dx = -P.dx, dy = -P.dy;                    // d_ik = x_i - x_k
        const float gx = P.G * dx, gy = P.G * dy;
        const float wgx = g4.x * gx + g4.y * gy - ddb * gx, wgy = g4.z * gx + g4.w * gy - ddb * gy;
        av.x += mvk * wgx;
        av.y += mvk * wgy;
        if (ks) {
            amv += ux * wgx + uy * wgy;
            const float hx = mvk * (g4.x * ux + g4.z * uy - ddb * ux);
            const float hy = mvk * (g4.y * ux + g4.w * uy - ddb * uy);
            const float cr = P.Gp / P.r * (hx * dx + hy * dy);
            ax.x -= P.G * hx + cr * dx;
            ax.y -= P.G * hy + cr * dy;
        }
    });
    A.v[kk] = f2(A.v[kk].x + av.x, A.v[kk].y + av.y);
    if (ks) {
        A.x[kk] = f2(A.x[kk].x + ax.x, A.x[kk].y + ax.y);
        A.mv[kk] += amv;
    }
}

// ---- K7: m_V = m / rho reversed; step-start adjoint out (canonical order) ----
__global__ void k_adj_out(K32 k, P32 p, Start S, A32 A, double* __restrict__ ax, double* __restrict__ av,
                          double* __restrict__ ar, double* __restrict__ avt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const size_t c = (size_t)p.ids[i].x;
    if (soil(S.hi[i].w)) {
        const float rho = k.rho0 + S.drho[i];
        const float r = A.r[i] - A.mv[i] * p.mass[i] / (rho * rho);
        ax[3 * c] = A.x[i].x; ax[3 * c + 1] = A.x[i].y; ax[3 * c + 2] = 0.0;
        av[3 * c] = A.v[i].x; av[3 * c + 1] = A.v[i].y; av[3 * c + 2] = 0.0;
        ar[c] = r;
        avt[3 * c] = avt[3 * c + 1] = avt[3 * c + 2] = 0.0;
    } else {
        ax[3 * c] = ax[3 * c + 1] = ax[3 * c + 2] = 0.0;
        av[3 * c] = av[3 * c + 1] = av[3 * c + 2] = 0.0;
        ar[c] = 0.0;
        avt[3 * c] = A.v[i].x; avt[3 * c + 1] = A.v[i].y; avt[3 * c + 2] = 0.0;
    }
}

__global__ void k_copy_start(int n, P32 p, RecView vt, Start S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    S.hi[i] = p.hi[i];
    S.lo[i] = p.lo[i];
    S.vel[i] = p.vel[i];
    S.vlo[i] = p.vlo ? p.vlo[i] : make_float4(0.f, 0.f, 0.f, 0.f);  // WCSPH keeps no compensated velocity
    S.drho[i] = p.drho[i];
    S.vt[i] = vt[i];
}

// ================================================================ WCSPH
// Adjoint of one FP32-mixed WCSPH step: 2D, symplectic Euler, no kernel-gradient
// correction, dummy-particle boundary, no XSPH.  The step (eng/solver_sph_base.py:41-91,
// :224-247, :386-398, :653-663; eng/solver_sph_wc.py:30-132) maps the fluid state (x, v, rho;
// m_V = m / rho) to the next one through
//   p_i   = max(B ((rho_i / rho0)^g - 1), 0),  P_i = p_i / rho_i^2                  (EOS)
//   S_b   = sum_{fluid j} m_Vj W_bj,  cf_b = 1 / S_b                                (Shepard)
//   U_b   = sum m_Vj v_j W_bj,  v~_b = 2 v_b - cf_b U_b
//   Q_b   = sum m_Vj (p_j + rho_j g_y (y_b - y_j)) W_bj,  p_b = max(cf_b Q_b, 0),  P_b = p_b / rho0^2
//   drho_i = rho_i sum_j m_Vj (v~_i - v~_j) . G_ij d_ij
//   dv_i  = g + sum_j m_Vj [c_ij nu' min(u_ij . d_ij, 0) / (|d_ij|^2 + eps_h) - rho0 (P_i + P_j)] G_ij d_ij
//           (u_ij = v~_i - v~_j, c_ij = 1 for fluid j and rho0 / rho_i for dummy j)
//   rho'  = rho + dt drho,  v' = v + dt dv,  x' = x + dt v',  rho'' = max(rho', rho0)
// The parameter adjoints are those of the Tait stiffness B and of nu' = 2 (d + 2) nu.
// Kernel roles: WK0 end-of-step adjoint in and the update reversed; WK1 the pair terms of
// continuity and momentum (both sides, gathered at each particle); WK2 the boundary
// extrapolation reversed at each dummy; WK3 its terms gathered at each fluid particle; WK4
// the EOS and m_V = m / rho reversed, adjoint out.

__device__ __forceinline__ bool fluid(float w) { return tf_type(w) == MAT_FLUID; }

// dp / d rho of the Tait EOS at density deviation drt (0 where the pressure is clamped).
__device__ __forceinline__ float tait_drho(const K32& k, float drt, float p) {
    if (!(p > 0.f)) return 0.f;
    const float a = 1.f + drt / k.rho0;
    float pw = 1.f;
    if (k.exponent_is_int && k.gamma_i >= 1)
        for (int q = 1; q < k.gamma_i; ++q) pw *= a;
    else
        pw = powf(a, k.gamma - 1.f);
    return k.B * k.gamma * pw / k.rho0;
}

__global__ void k_wadj_init(K32 k, P32 p, T32 t, Start S, A32 A, const double* __restrict__ ax,
                            const double* __restrict__ av, const double* __restrict__ ar) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const int c = p.ids[i].x;
    A.x[i] = A.v[i] = A.dv[i] = A.vn[i] = A.b1[i] = f2(0.f, 0.f);
    A.r[i] = A.mv[i] = A.rt[i] = A.dr[i] = A.b2[i] = A.bs[i] = A.dds[i] = 0.f;
    A.gp[i] = make_double2(0.0, 0.0);
    if (!fluid(S.hi[i].w)) return;
    const float2 xb = f2((float)ax[3 * (size_t)c], (float)ax[3 * (size_t)c + 1]);
    const float2 vb = f2((float)av[3 * (size_t)c], (float)av[3 * (size_t)c + 1]);
    const float drho1 = S.drho[i] + k.dt * t.dd[i];    // before the density clamp
    const float rb1 = drho1 > 0.f ? (float)ar[c] : 0.f;
    const float2 vt = f2(vb.x + k.dt * xb.x, vb.y + k.dt * xb.y);  // x' = x + dt v'
    A.x[i] = xb;
    A.v[i] = vt;                                       // v' = v + dt dv
    A.dv[i] = f2(k.dt * vt.x, k.dt * vt.y);
    A.r[i] = rb1;                                      // rho' = rho + dt drho
    A.dr[i] = k.dt * rb1;
}

// One pair's forward terms seen from the centre i (fluid) with neighbour j:
// d = x_i - x_j, u = v~_i - v~_j, s = m_Vj [c nu' min(u.d, 0) / (r^2 + eps_h) - rho0 (P_i + P_j)].
struct WPair {
    float dx, dy, r, G, Gp, ux, uy, w, Vn, V, dVdw, s;  // Vn = V / nu'
};
__device__ __forceinline__ bool wpair(const K32& k, const Start& S, const T32& t, int i, int j, float mvj,
                                      float rho_i, WPair& P) {
    Pair q;
    if (!pair(k, S, i, j, q)) return false;
    P.dx = q.dx; P.dy = q.dy; P.r = q.r; P.G = q.G; P.Gp = q.Gp;
    const float4 vi = t.vt[i], vj = t.vt[j];
    P.ux = vi.x - vj.x;
    P.uy = vi.y - vj.y;
    P.w = P.ux * P.dx + P.uy * P.dy;
    const float cij = fluid(S.hi[j].w) ? 1.f : k.rho0 / rho_i;
    const float den = 1.f / (q.r * q.r + k.eps_h2);
    const float cw = P.w < 0.f ? cij * mvj * den : 0.f;
    P.Vn = cw * P.w;                 // c m_Vj min(w, 0) / (r^2 + eps_h)
    P.dVdw = k.visc_fac * cw;
    P.V = k.visc_fac * P.Vn;
    P.s = P.V - k.rho0 * mvj * (vi.w + vj.w);
    return true;
}

__global__ void k_wadj_pairs(K32 k, P32 p, T32 t, Start S, A32 A) {
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    if (kk >= k.n) return;
    const bool kf = fluid(S.hi[kk].w);
    const float mvk = S.lo[kk].w;
    const float rho_k = k.rho0 + t.drt[kk];
    float2 ax = f2(0.f, 0.f), av = f2(0.f, 0.f);
    float ar = 0.f, amv = 0.f, aP = 0.f;
    double gnu = 0.0;
    const float2 ak = A.dv[kk];
    const float ck = A.dr[kk];
    for_list(k, t, kk, [&](int j) {
        const bool jf = fluid(S.hi[j].w);
        if (kf) {  // kk the centre i, j the neighbour
            WPair P;
            if (wpair(k, S, t, kk, j, S.lo[j].w, rho_k, P)) {
                const float mvj = S.lo[j].w;
                const float gx = P.G * P.dx, gy = P.G * P.dy;
                // continuity: rho_i m_Vj u . g
                const float cm = ck * rho_k * mvj;
                av.x += cm * gx; av.y += cm * gy;
                const float cr = P.Gp / P.r * (P.ux * P.dx + P.uy * P.dy);
                ax.x += cm * (P.G * P.ux + cr * P.dx);
                ax.y += cm * (P.G * P.uy + cr * P.dy);
                ar += ck * mvj * (P.ux * gx + P.uy * gy);
                // momentum: s (a . g)
                const float sb = ak.x * gx + ak.y * gy;
                const float ca = P.Gp / P.r * (ak.x * P.dx + ak.y * P.dy);
                ax.x += P.s * (P.G * ak.x + ca * P.dx);
                ax.y += P.s * (P.G * ak.y + ca * P.dy);
                if (P.w < 0.f) {
                    av.x += sb * P.dVdw * P.dx; av.y += sb * P.dVdw * P.dy;
                    const float e2 = 2.f * P.V / (P.r * P.r + k.eps_h2);
                    ax.x += sb * (P.dVdw * P.ux - e2 * P.dx);
                    ax.y += sb * (P.dVdw * P.uy - e2 * P.dy);
                    gnu += (double)sb * P.Vn;
                    if (!jf) ar += -sb * P.V / rho_k;
                }
                aP += -sb * k.rho0 * mvj;
            }
        }
        if (jf) {  // j the centre i, kk the neighbour
            const float rho_j = k.rho0 + t.drt[j];
            WPair P;
            if (wpair(k, S, t, j, kk, mvk, rho_j, P)) {  // d = x_j - x_kk, u = v~_j - v~_kk
                const float2 aj = A.dv[j];
                const float cj = A.dr[j];
                const float gx = P.G * P.dx, gy = P.G * P.dy;
                const float cm = cj * rho_j * mvk;
                av.x -= cm * gx; av.y -= cm * gy;
                const float cr = P.Gp / P.r * (P.ux * P.dx + P.uy * P.dy);
                ax.x -= cm * (P.G * P.ux + cr * P.dx);
                ax.y -= cm * (P.G * P.uy + cr * P.dy);
                if (kf) amv += cj * rho_j * (P.ux * gx + P.uy * gy);
                const float sb = aj.x * gx + aj.y * gy;
                const float ca = P.Gp / P.r * (aj.x * P.dx + aj.y * P.dy);
                ax.x -= P.s * (P.G * aj.x + ca * P.dx);
                ax.y -= P.s * (P.G * aj.y + ca * P.dy);
                if (P.w < 0.f) {
                    av.x -= sb * P.dVdw * P.dx; av.y -= sb * P.dVdw * P.dy;
                    const float e2 = 2.f * P.V / (P.r * P.r + k.eps_h2);
                    ax.x -= sb * (P.dVdw * P.ux - e2 * P.dx);
                    ax.y -= sb * (P.dVdw * P.uy - e2 * P.dy);
                    if (kf) amv += sb * P.V / mvk;
                }
                aP += -sb * k.rho0 * mvk;
                if (kf) amv += -sb * k.rho0 * (t.vt[j].w + t.vt[kk].w);
            }
        }
    });
    A.x[kk] = f2(A.x[kk].x + ax.x, A.x[kk].y + ax.y);
    A.v[kk] = f2(A.v[kk].x + av.x, A.v[kk].y + av.y);  // fluid: v; dummy: its v~
    A.rt[kk] += aP;                                      // P = p / rho^2
    if (kf) {
        A.r[kk] += ar;
        A.mv[kk] += amv;
        A.gp[kk].y += gnu;
    }
}

// Boundary extrapolation reversed at each dummy: coefficients of its sums.
__global__ void k_wadj_bdy(K32 k, P32 p, T32 t, Start S, A32 A) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= k.n || tf_type(S.hi[b].w) > 0 || t.cnt[b] == 0) return;
    float2 U = f2(0.f, 0.f);
    float Q = 0.f, Sb = 0.f;
    for_list(k, t, b, [&](int j) {
        if (!fluid(S.hi[j].w)) return;
        float d[3];
        delta<2>(S.hi[b], S.lo[b], S.hi[j], S.lo[j], d);
        const float r2 = dist2<2>(d);
        if (!(r2 < k.R2)) return;
        const float mw = S.lo[j].w * w_val(k, fast_sqrt(r2));
        const float4 v = t.vt[j];
        const float2 pr = t.pr[j];
        U.x += mw * v.x; U.y += mw * v.y;
        Q += mw * (pr.x + pr.y * k.g[1] * d[1]);
        Sb += mw;
    });
    const float cf = t.cf[b];
    const float2 avt = A.v[b];                          // adjoint of v~_b
    const float pb = A.rt[b] / (k.rho0 * k.rho0);       // P_b = p_b / rho0^2
    const bool open = cf * Q > 0.f;
    float cfb = -(avt.x * U.x + avt.y * U.y);
    if (open) cfb += pb * Q;
    A.b1[b] = f2(-cf * avt.x, -cf * avt.y);            // adjoint of U_b
    A.b2[b] = open ? pb * cf : 0.f;                     // adjoint of Q_b
    A.bs[b] = Sb != 0.f ? -cfb * cf * cf : 0.f;         // adjoint of S_b
}

// The boundary sums' terms gathered at each fluid particle.
__global__ void k_wadj_bdy_fluid(K32 k, P32 p, T32 t, Start S, A32 A) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k.n || !fluid(S.hi[j].w)) return;
    const float mvj = S.lo[j].w;
    const float4 v = t.vt[j];
    const float2 pr = t.pr[j];
    float2 ax = f2(0.f, 0.f), av = f2(0.f, 0.f);
    float amv = 0.f, ap = 0.f, ar = 0.f;
    for_list(k, t, j, [&](int b) {
        if (tf_type(S.hi[b].w) > 0) return;
        float d[3];
        delta<2>(S.hi[b], S.lo[b], S.hi[j], S.lo[j], d);  // d = x_b - x_j
        const float r2 = dist2<2>(d);
        if (!(r2 < k.R2)) return;
        const float r = fast_sqrt(r2);
        const float W = w_val(k, r), G = w_grad(k, r);
        const float2 B1 = A.b1[b];
        const float B2 = A.b2[b], BS = A.bs[b];
        const float qj = pr.x + pr.y * k.g[1] * d[1];
        const float coef = (B1.x * v.x + B1.y * v.y) + B2 * qj + BS;
        amv += coef * W;
        av.x += B1.x * mvj * W; av.y += B1.y * mvj * W;
        ap += B2 * mvj * W;
        ar += B2 * mvj * k.g[1] * d[1] * W;
        const float wb = mvj * coef;
        ax.x += -wb * G * d[0];
        ax.y += -wb * G * d[1] - B2 * mvj * pr.y * k.g[1] * W;
    });
    A.x[j] = f2(A.x[j].x + ax.x, A.x[j].y + ax.y);
    A.v[j] = f2(A.v[j].x + av.x, A.v[j].y + av.y);
    A.mv[j] += amv;
    A.dds[j] += ap;  // adjoint of p_j (the dummies' pressure sums)
    A.r[j] += ar;
}

// EOS and m_V = m / rho reversed; adjoint out in canonical order.
__global__ void k_wadj_out(K32 k, P32 p, T32 t, Start S, A32 A, double* __restrict__ ax, double* __restrict__ av,
                           double* __restrict__ ar, double* __restrict__ avt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const size_t c = (size_t)p.ids[i].x;
    avt[3 * c] = avt[3 * c + 1] = avt[3 * c + 2] = 0.0;
    if (!fluid(S.hi[i].w)) {
        ax[3 * c] = ax[3 * c + 1] = ax[3 * c + 2] = 0.0;
        av[3 * c] = av[3 * c + 1] = av[3 * c + 2] = 0.0;
        ar[c] = 0.0;
        return;
    }
    const float drt = t.drt[i];
    const float rho = k.rho0 + drt;
    const float pi = t.pr[i].x;
    const float pbar = A.dds[i] + A.rt[i] / (rho * rho);  // p enters the dummies' sums and P
    float r = A.r[i] + pbar * tait_drho(k, drt, pi) - A.rt[i] * 2.f * pi / (rho * rho * rho);
    r -= A.mv[i] * p.mass[i] / (rho * rho);
    if (pi > 0.f) A.gp[i].x += (double)pbar * pi / k.B;  // p is proportional to B
    ax[3 * c] = A.x[i].x; ax[3 * c + 1] = A.x[i].y; ax[3 * c + 2] = 0.0;
    av[3 * c] = A.v[i].x; av[3 * c + 1] = A.v[i].y; av[3 * c + 2] = 0.0;
    ar[c] = r;
}

template <class T>
T* grab(Fp32State& st, size_t count) {
    void* q = nullptr;
    if (cudaMalloc(&q, (count ? count : 1) * sizeof(T)) != cudaSuccess) return nullptr;
    st.allocs.push_back(q);
    return static_cast<T*>(q);
}

struct AdjBuffers {
    Start S{};
    A32 A{};
};

AdjBuffers* adj_buffers(Fp32State& st) {
    if (st.adj) return static_cast<AdjBuffers*>(st.adj);
    const size_t n = st.n;
    AdjBuffers* b = new AdjBuffers();
    Start& S = b->S;
    A32& A = b->A;
    S.hi = grab<float4>(st, n); S.lo = grab<float4>(st, n); S.vel = grab<float4>(st, n); S.vt = grab<float4>(st, n);
    S.vlo = grab<float4>(st, n);
    A.gp = grab<double2>(st, n);
    S.drho = grab<float>(st, n);
    A.x = grab<float2>(st, n); A.v = grab<float2>(st, n); A.dv = grab<float2>(st, n); A.vn = grab<float2>(st, n);
    A.b1 = grab<float2>(st, n);
    A.r = grab<float>(st, n); A.mv = grab<float>(st, n); A.rt = grab<float>(st, n); A.dr = grab<float>(st, n);
    A.b2 = grab<float>(st, n); A.bs = grab<float>(st, n); A.dds = grab<float>(st, n);
    A.s = grab<float4>(st, n); A.b3 = grab<float4>(st, n); A.vg = grab<float4>(st, n);
    if (!S.hi || !S.lo || !S.vel || !S.vt || !S.vlo || !A.gp || !S.drho || !A.x || !A.v || !A.dv || !A.vn || !A.b1 || !A.r || !A.mv ||
        !A.rt || !A.dr || !A.b2 || !A.bs || !A.dds || !A.s || !A.b3 || !A.vg) {
        delete b;
        return nullptr;
    }
    st.adj = b;
    return b;
}

}  // namespace

void fp32_free_adjoint(Fp32State& st) {
    delete static_cast<AdjBuffers*>(st.adj);
    st.adj = nullptr;
}

int fp32_adjoint_step(Fp32State& st, double* ax, double* av, double* ar, double* avt, double* pbar,
                      cudaStream_t s) {
    const K32& k = st.k;
    if ((k.solver != 1 && k.solver != 2) || k.dim != 2 || st.c.ti != 1 || k.corr != 0 || k.boundary != 2 ||
        k.xsph || k.scene_par)
        return TSG_E_UNSUPPORTED;
    if (st.c.n_bdy > st.n - st.nd) return TSG_E_UNSUPPORTED;  // rigid particles
    AdjBuffers* B = adj_buffers(st);
    if (!B) return TSG_E_CUDA;
    // forward of the step from the loaded state, keeping its start
    f32::rebuild(st, s, true);  // in place: v_tmp lives in the current buffer's records
    st.built = true;
    st.lists_valid = true;
    ++st.rebuilds;
    int novf = 0;
    cudaMemcpyAsync(&novf, st.novf, sizeof novf, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    if (novf) return TSG_E_CAPACITY;  // every list must hold all neighbours
    P32& p = st.P[st.cur];
    const int nb = nblk(st.n);
    TSG_LAUNCH(k_copy_start, nb, TPB, s, st.n, p, st.T.vt, B->S);
    f32::step_body(st, s, false);
    // reverse sweep
    if (k.solver == 1) {
        TSG_LAUNCH(k_wadj_init, nb, TPB, s, k, p, st.T, B->S, B->A, ax, av, ar);
        TSG_LAUNCH(k_wadj_pairs, nb, TPB, s, k, p, st.T, B->S, B->A);
        TSG_LAUNCH(k_wadj_bdy, nb, TPB, s, k, p, st.T, B->S, B->A);
        TSG_LAUNCH(k_wadj_bdy_fluid, nb, TPB, s, k, p, st.T, B->S, B->A);
        TSG_LAUNCH(k_wadj_out, nb, TPB, s, k, p, st.T, B->S, B->A, ax, av, ar, avt);
        TSG_LAUNCH(k_adj_params, 1, 256, s, st.n, B->A.gp, pbar);
        return cudaGetLastError() == cudaSuccess ? 0 : TSG_E_CUDA;
    }
    TSG_LAUNCH(k_adj_init, nb, TPB, s, k, p, st.T, B->S, B->A, ax, av, ar, avt);
    TSG_LAUNCH(k_adj_mom, nb, TPB, s, k, p, st.T, B->S, B->A);
    TSG_LAUNCH(k_adj_bdy, nb, TPB, s, k, p, st.T, B->S, B->A);
    TSG_LAUNCH(k_adj_bdy_soil, nb, TPB, s, k, p, st.T, B->S, B->A);
    TSG_LAUNCH(k_adj_stress, nb, TPB, s, k, p, st.T, B->S, B->A);
    TSG_LAUNCH(k_adj_params, 1, 256, s, st.n, B->A.gp, pbar);
    TSG_LAUNCH(k_adj_vgrad, nb, TPB, s, k, p, st.T, B->S, B->A);
    TSG_LAUNCH(k_adj_out, nb, TPB, s, k, p, B->S, B->A, ax, av, ar, avt);
    return cudaGetLastError() == cudaSuccess ? 0 : TSG_E_CUDA;
}

}  // namespace tsg
