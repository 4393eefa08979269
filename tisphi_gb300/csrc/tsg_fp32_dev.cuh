// Device-side definitions shared by the FP32-mixed translation units (tsg_fp32.cu: the
// forward step; tsg_adjoint.cu: the hand-written adjoint of the mu(I) step): launch sizes,
// the constant block K32, particle layouts P32 / T32, the compensated accumulator, kernel
// functions, neighbour enumeration and list traversal, and the host-side state.
#pragma once
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "tsg_fp32.h"

namespace tsg {
namespace f32 {

constexpr int TPB = 128;
inline int nblk(long long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

struct K32 {
    int n, nd, dim, kernel, corr, xsph, boundary, solver, maxn, exponent_is_int, gamma_i;
    int gnum[3];
    long long G;
    double vs[3], grid;
    float Q, inv_grid, h1, kk, kk6, wgrad, cub1, cub2, cub1h, R2, R2lo, R2hi, pf_lim;
    float R2L, R2Lhi, disp2_limit;  // list radius (support + skin) and rebuild threshold
    float visc_fac, eps_h2, rho0, B, gamma, dt, hdt, dt6, g[3], rep_fac, diam, h075, r_eps;
    float ds[3], de[3];
    // granular solvers (mu(I): mu, c2, coh; Drucker-Prager: alpha ... twoG; both: damping)
    float mu, c2, coh, alpha, k_c, kc_over_alpha, Gm, Km, sin_dila, lam_den, three_aK, nine_K_sin, twoG;
    float damp_eps, damp_E, h2;
    // batched ensembles: per-scene (stiffness B, viscosity factor), indexed by the scene
    // number in the type word; nullptr for a single scene (B and visc_fac above)
    const float2* scene_par;
    float inv_Q;    // 1 / Q (a power of two)
};

// The lo record (lx, ly, lz, m_V) and the v_tmp record (v_tmp, p / rho_tmp^2) of a particle
// sit side by side in one 32-byte record, so the rates pass gathers both of a neighbour with
// one 256-bit load.  RecView is one half of the interleaved array: element i at p[2 i].
struct RecView {
    float4* p;
    __host__ __device__ __forceinline__ float4& operator[](size_t i) const { return p[2 * i]; }
};
// Both halves of neighbour j's record in one read-only 256-bit load (base = the lo view's
// array; the array is 32-byte aligned and not written by the kernel that calls this).
__device__ __forceinline__ void ldg_rec(const float4* base, int j, float4& lo, float4& vt) {
    const float4* a = base + 2 * (size_t)j;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(lo.x), "=f"(lo.y), "=f"(lo.z), "=f"(lo.w), "=f"(vt.x), "=f"(vt.y), "=f"(vt.z), "=f"(vt.w)
        : "l"(a));
}

// Type word (the w lane of hi): bits 0-15 material type (signed), bit 16 is_dynamic, bits
// 17-28 scene number of a batched ensemble, bit 30 set (the word stays a normal float).
__device__ __forceinline__ int tf_type(float w) { return (int)(short)(__float_as_int(w) & 0xffff); }
__device__ __forceinline__ int tf_dyn(float w) { return (__float_as_int(w) >> 16) & 1; }
__device__ __forceinline__ int tf_scene(float w) { return (__float_as_int(w) >> 17) & 0xfff; }
constexpr int kMaxScenes = 4096;
__device__ __forceinline__ bool is_flow(int t) { return t == MAT_FLUID || t == MAT_SOIL; }

// Neighbour-list entries pack the neighbour index (bits 0-22, so this form holds at most
// 2^23 particles), its material code (bits 23-25) and the offset (hi_i - hi_j) / Q + 1 of
// the two particles' quantised positions per axis (bits 26-27, 28-29, 30-31; Q is at least
// one cell of the list grid, so two listed particles are never more than one quantum
// apart, and hi only changes when the lists are rebuilt).  A traversal therefore reads the
// neighbour's lo record and nothing of its hi record, and decodes the entry with shifts,
// masks and one float add per axis.
// Material codes: repulsive 0, dummy 1, rigid 2, fluid 4, soil 5 (bit 2 = flow particle),
// so the hot kernels test a neighbour's kind on the code itself.
constexpr int kEntryBits = 23;
constexpr int kEntryMask = (1 << kEntryBits) - 1;
constexpr int kCodeRep = 0, kCodeFluid = 4;
__device__ __forceinline__ int type_class(int t) {
    return t == MAT_FLUID ? 4 : t == MAT_SOIL ? 5 : t == MAT_DUMMY ? 1 : t == MAT_REP ? 0 : 2;
}
__device__ __forceinline__ int class_type(int c) {
    return c == 4 ? MAT_FLUID : c == 5 ? MAT_SOIL : c == 1 ? MAT_DUMMY : c == 0 ? MAT_REP : MAT_RIGID;
}
__device__ __forceinline__ bool code_flow(int c) { return (c & 4) != 0; }
__device__ __forceinline__ int make_entry(int j, int tj, int ox, int oy, int oz) {
    return (int)((unsigned)j | ((unsigned)type_class(tj) << kEntryBits) | ((unsigned)(ox + 1) << 26) |
                 ((unsigned)(oy + 1) << 28) | ((unsigned)(oz + 1) << 30));
}
// Offset field v of an axis as the float v - 1: v in the low mantissa bits of 2^23 gives
// the float 2^23 + v exactly, and subtracting 2^23 + 1 is exact.
__device__ __forceinline__ float entry_offset(int e, int axis) {
    return __fadd_rn(__int_as_float((int)(0x4B000000u | (((unsigned)e >> (26 + 2 * axis)) & 3u))), -8388609.f);
}
// Entry for neighbour j of i from their hi records (list builders without staged offsets).
__device__ __forceinline__ int entry_of(const K32& k, int j, const float4& hi_i, const float4& hi_j) {
    return make_entry(j, tf_type(hi_j.w), (int)rintf((hi_i.x - hi_j.x) * k.inv_Q),
                      (int)rintf((hi_i.y - hi_j.y) * k.inv_Q), (int)rintf((hi_i.z - hi_j.z) * k.inv_Q));
}
__device__ __forceinline__ int entry_index(const K32&, int e) { return e & kEntryMask; }

// Block-compensated accumulator: plain partial sums, Kahan-folded every flush (the list
// kernels flush after every kFlushEvery-th slot).
constexpr int kFlushEvery = 16;
// Block-compensated accumulator: plain partial sums, Kahan-folded every flush.
struct CSum {
    float s = 0.f, c = 0.f, p = 0.f;
    __device__ __forceinline__ void add(float x) { p += x; }
    __device__ __forceinline__ void flush() {
        float y = p - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
        p = 0.f;
    }
    __device__ __forceinline__ float get() { flush(); return s; }
};

// A plain f32 sum with CSum's interface (flush does nothing).
struct PSum {
    float p = 0.f;
    __device__ __forceinline__ void add(float x) { p += x; }
    __device__ __forceinline__ void flush() {}
    __device__ __forceinline__ float get() { return p; }
};

__device__ __forceinline__ void atomic_max_d(double* addr, double v) {
    unsigned long long* a = reinterpret_cast<unsigned long long*>(addr);
    unsigned long long old = *a;
    while (__longlong_as_double(old) < v) {
        unsigned long long prev = atomicCAS(a, old, __double_as_longlong(v));
        if (prev == old) break;
        old = prev;
    }
}

// Cell coordinate trunc((hi + lo) / grid) with the f64 semantics of the reference's cast:
// an f32 estimate decides unless it lies within its error bound (1e-3 + |t| 2^-20, well
// above the three roundings of the f32 estimate) of an integer, where f64 decides.
__device__ __forceinline__ long long cell_coord(const K32& k, float hi, float lo, bool& ok) {
    const float tf = (hi + lo) * k.inv_grid;
    const float fr = fabsf(tf - truncf(tf));
    const float margin = 1e-3f + fabsf(tf) * 9.5367431640625e-7f;
    if (fabsf(tf) < 1.0e6f && fr > margin && fr < 1.f - margin) return (long long)(int)tf;
    const double t = ((double)hi + (double)lo) / k.grid;
    if (!(fabs(t) < 2147483647.0)) { ok = false; return 0; }
    return (long long)(int)t;
}

// |x| from |x|^2 through the hardware reciprocal square root (~2 ulp; 0 -> NaN, which the
// kernel functions' support test rejects).
__device__ __forceinline__ float fast_sqrt(float r2) { return r2 * rsqrtf(r2); }

// Kernel value and gradient factor: W(r) and G with grad W = G * dx.
__device__ __forceinline__ float w_val(const K32& k, float r) {
    float q = r * k.h1;
    if (!(r > 1e-8f && q <= 2.f)) return 0.f;
    if (k.kernel == 1) {
        float q1 = 1.f - 0.5f * q;
        float q2 = q1 * q1;
        return k.kk * (q2 * q2) * (1.f + 2.f * q);
    }
    if (q <= 1.f) return k.kk * ((0.5f * q - 1.f) * q * q + 2.f / 3.f);
    float t = 2.f - q;
    return k.kk6 * t * t * t;
}
__device__ __forceinline__ float w_grad(const K32& k, float r) {
    float q = r * k.h1;
    if (!(r > 1e-8f && q <= 2.f)) return 0.f;
    if (k.kernel == 1) {
        float q1 = 1.f - 0.5f * q;
        return k.wgrad * (q1 * q1 * q1);                // -5 k h1^2 q1^3
    }
    const float inv = __fdividef(1.f, r);
    if (q <= 1.f) return k.cub1 * q * (1.5f * q - 2.f) * inv;   // k h1 q (1.5 q - 2) / r
    float f = 2.f - q;
    return k.cub2 * f * f * inv;                       // -0.5 k h1 f^2 / r
}

// Kernel value and gradient factor of a neighbour at squared distance r2 < R^2, from one
// reciprocal square root rs = 1 / r: the cubic spline's inner piece k h^-1 q (1.5 q - 2) / r
// is k h^-2 (1.5 q - 2) (q / r = 1 / h), the outer piece takes 1 / r from rs.  r2 < R^2
// bounds q = r / h by 2 up to the roundings of r and q, and both kernels vanish at q = 2, so
// the support test is not repeated here.  r = 0 gives r = NaN and both factors 0.
// KT selects the kernel function at compile time (1 Wendland C2, 0 cubic spline) or, for
// -1, at run time from k.kernel.
struct WG { float r, w, g; };
template <bool VAL, bool GRAD, int KT = -1>
__device__ __forceinline__ WG w_pair(const K32& k, float r2) {
    const float rs = rsqrtf(r2);
    WG o;
    o.r = __fmul_rn(r2, rs);
    o.w = 0.f;
    o.g = 0.f;
    if (!(o.r > 1e-8f)) return o;
    const float q = __fmul_rn(o.r, k.h1);
    if (KT == 1 || (KT < 0 && k.kernel == 1)) {
        // rounding spelled out, so every kernel that inlines this gets the same bits
        const float q1 = __fmaf_rn(-0.5f, q, 1.f), q2 = __fmul_rn(q1, q1);
        if (VAL) o.w = __fmul_rn(__fmul_rn(k.kk, __fmul_rn(q2, q2)), __fmaf_rn(2.f, q, 1.f));
        if (GRAD) o.g = __fmul_rn(k.wgrad, __fmul_rn(q2, q1));
        return o;
    }
    const float t = 2.f - q;
    if (q <= 1.f) {
        if (VAL) o.w = k.kk * ((0.5f * q - 1.f) * q * q + 2.f / 3.f);
        if (GRAD) o.g = k.cub1h * (1.5f * q - 2.f);
    } else {
        if (VAL) o.w = k.kk6 * t * t * t;
        if (GRAD) o.g = k.cub2 * t * t * rs;
    }
    return o;
}
// |d|^2 with its rounding spelled out, so that every kernel takes the support test and
// evaluates the kernel function on the same bits for the same pair.
template <int DIM>
__device__ __forceinline__ float dist2(const float* d) {
    float r2 = __fmaf_rn(d[1], d[1], __fmul_rn(d[0], d[0]));
    if (DIM == 3) r2 = __fmaf_rn(d[2], d[2], r2);
    return r2;
}
template <int DIM>
__device__ __forceinline__ void delta(const float4& hi_i, const float4& lo_i, const float4& hi_j, const float4& lo_j,
                                      float* d) {
    d[0] = (hi_i.x - hi_j.x) + (lo_i.x - lo_j.x);
    d[1] = (hi_i.y - hi_j.y) + (lo_i.y - lo_j.y);
    d[2] = DIM == 3 ? (hi_i.z - hi_j.z) + (lo_i.z - lo_j.z) : 0.f;
}

// Candidate enumeration over the stencil of i (reference traversal order of cells, dynamic
// block first, then the static block for flow centres).  body(j, d, r2) gets the exact
// f32 displacement x_i - x_j.  The cheap prefilter compares the positions of the last list
// build (PF): with a skin, particles have moved at most 0.45 skin since then while the
// lists are in use, so a build-time distance above (R + skin)(1 + 2^-11) rules a pair out
// for the current positions as well.  Callers after advect_pos (positions moved past the
// last check) pass use_pf = false.
template <int DIM, class F>
__device__ __forceinline__ void enum_neighbors(const K32& k, int i, const float4* __restrict__ HI,
                                               RecView LO, const float4* __restrict__ PF,
                                               const int* __restrict__ dstart, const int* __restrict__ sstart,
                                               bool flow_i, F&& body, bool list_radius = false,
                                               bool use_pf = true) {
    const float cut2 = list_radius ? k.R2L : k.R2;
    const float cut2hi = k.R2Lhi;
    const float4 hi_i = HI[i], lo_i = LO[i], pf_i = PF[i];
    bool ok = true;
    const long long cc0 = cell_coord(k, hi_i.x, lo_i.x, ok);
    const long long cc1 = cell_coord(k, hi_i.y, lo_i.y, ok);
    const long long cc2 = cell_coord(k, hi_i.z, lo_i.z, ok);
    if (!ok) return;
    const bool pf = use_pf && fabsf(pf_i.x) < k.pf_lim && fabsf(pf_i.y) < k.pf_lim && fabsf(pf_i.z) < k.pf_lim;
    const long long ny = k.gnum[1], nz = k.gnum[2], G = k.G;
    for (int blk = 0; blk < (flow_i ? 2 : 1); ++blk) {
        const int* cs = blk == 0 ? dstart : sstart;
#pragma unroll 1
        for (int ox = -1; ox <= 1; ++ox) {
#pragma unroll 1
            for (int oy = (DIM == 3 ? -1 : 0); oy <= (DIM == 3 ? 1 : 0); ++oy) {
                long long f0 = (cc0 + ox) * ny * nz + (cc1 + oy) * nz + cc2;
                long long lo = f0 - 1 > 0 ? f0 - 1 : 0;
                long long hi = f0 + 1 < G - 1 ? f0 + 1 : G - 1;
                if (lo > hi) continue;
                const int jb = cs[lo], je = cs[hi + 1];
#pragma unroll 2
                for (int j = jb; j < je; ++j) {
                    if (j == i) continue;
                    const float4 pj = PF[j];
                    if (!flow_i && !is_flow(tf_type(pj.w))) continue;
                    float r2f;
                    if (pf) {
                        float fx = pf_i.x - pj.x, fy = pf_i.y - pj.y, fz = pf_i.z - pj.z;
                        r2f = fx * fx + fy * fy;
                        if (DIM == 3) r2f += fz * fz;
                        if (r2f > cut2hi) continue;
                    }
                    float d[3];
                    delta<DIM>(hi_i, lo_i, HI[j], LO[j], d);
                    const float r2 = dist2<DIM>(d);
                    if (!(r2 < cut2)) continue;
                    body(j, d, r2);
                }
            }
        }
    }
}

// x_i - x_j of list entry e (neighbour lo record l) and its square, rounding spelled out
// once for every traversal.
template <int DIM>
__device__ __forceinline__ float list_delta(const K32& k, int e, const float4& lo_i, const float4& l, float* d) {
    d[0] = __fmaf_rn(entry_offset(e, 0), k.Q, __fadd_rn(lo_i.x, -l.x));
    d[1] = __fmaf_rn(entry_offset(e, 1), k.Q, __fadd_rn(lo_i.y, -l.y));
    d[2] = DIM == 3 ? __fmaf_rn(entry_offset(e, 2), k.Q, __fadd_rn(lo_i.z, -l.z)) : 0.f;
    return dist2<DIM>(d);
}

// Iterate i's neighbour list (FB = false) or traverse its stencil directly (FB = true: the
// particle's list overflowed).  body(j, d, r2, slot, type_j, m_V_j, g_j) (with CODE: the
// neighbour's material code in place of its type) gets the exact f32
// displacement x_i - x_j of every neighbour within the support and g_j = gather(j), the
// neighbour's payload, loaded together with its lo record (before the support test, so the
// two gathers overlap; the list's skin pairs load it for nothing).  Two neighbours per trip;
// the next trip's two list entries are loaded before this trip's gathers, so the entry
// stream (from DRAM) overlaps the gathers and the maths.  Entries are read once, with the
// evict-first streaming hint (ld.global.cs), so that they do not push the neighbours'
// records out of L1 and L2.
// REC: the payload is the neighbour's v_tmp record, loaded together with its lo record in
// one 256-bit read (ldg_rec) instead of through gather(j) (the overflow traversal still
// calls gather).
template <int DIM, bool FB, bool CODE = false, bool REC = false, class G, class F>
__device__ __forceinline__ void for_nbrs_g(const K32& k, int i, const int* __restrict__ cnt, const int* __restrict__ nbr,
                                           const float4* __restrict__ HI, RecView LO,
                                           const float4* __restrict__ PF, const int* __restrict__ dstart,
                                           const int* __restrict__ sstart, bool flow_i, G&& gather, F&& body) {
    if (!FB) {
        const int m = cnt[i];
        const float4 lo_i = LO[i];
        const size_t stride = (size_t)k.n;
        const int* lp = nbr + i;
        // neighbour record: position difference, type, m_V (lists hold support + skin)
        auto visit = [&](int e, const float4& l, const auto& g, int s) {
            float d[3];
            const float r2 = list_delta<DIM>(k, e, lo_i, l, d);
            const int c = (e >> kEntryBits) & 7;
            if (r2 < k.R2) body(e & kEntryMask, d, r2, s, CODE ? c : class_type(c), l.w, g);
        };
        int s = 0;
        int e0 = 0, e1 = 0;
        if (m > 1) { e0 = __ldcs(lp); e1 = __ldcs(lp + stride); lp += 2 * stride; }
        for (; s + 1 < m; s += 2) {
            int n0 = 0, n1 = 0;
            if (s + 3 < m) { n0 = __ldcs(lp); n1 = __ldcs(lp + stride); lp += 2 * stride; }
            const int j0 = e0 & kEntryMask, j1 = e1 & kEntryMask;
            float4 l0, l1;
            decltype(gather(0)) g0, g1;
            if constexpr (REC) {
                ldg_rec(LO.p, j0, l0, g0);
                ldg_rec(LO.p, j1, l1, g1);
            } else {
                l0 = LO[j0];
                l1 = LO[j1];
                g0 = gather(j0);
                g1 = gather(j1);
            }
            // s is even: the slot numbers' low bit is known, so a body's test of the slot
            // (a flush every eight) is decided at compile time for the first of the pair
            visit(e0, l0, g0, s & ~1);
            visit(e1, l1, g1, s | 1);
            e0 = n0;
            e1 = n1;
        }
        if (s < m) {
            const int e = nbr[(size_t)s * stride + i];
            const int j = e & kEntryMask;
            if constexpr (REC) {
                float4 l, g;
                ldg_rec(LO.p, j, l, g);
                visit(e, l, g, s);
            } else {
                visit(e, LO[j], gather(j), s);
            }
        }
    } else {
        int s = 0;
        enum_neighbors<DIM>(k, i, HI, LO, PF, dstart, sstart, flow_i, [&](int j, const float* d, float r2) {
            const int tj = tf_type(HI[j].w);
            body(j, d, r2, s++, CODE ? type_class(tj) : tj, LO[j].w, gather(j));
        });
    }
}

struct NoPayload {};

// i's list (not overflowed) four entries per trip, for the short, latency-bound lists of the
// boundary pass: each entry's lo + v_tmp record (one 256-bit read) and its extra payload
// X[j] are loaded for all four entries before the first is used, and the next trip's
// entries before this trip's gathers.  body(j, d, r2, slot, m_V_j, v_tmp_j, X_j) runs for
// the entries within the support, in slot order (so sums come out as with one entry per
// trip).
template <int DIM, class X, class F>
__device__ __forceinline__ void for_list4(const K32& k, int i, const int* __restrict__ cnt,
                                          const int* __restrict__ nbr, RecView LO, const X* __restrict__ XS,
                                          F&& body) {
    const int m = cnt[i];
    const float4 lo_i = LO[i];
    const size_t stride = (size_t)k.n;
    const int* lp = nbr + i;
    int e[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) e[u] = u < m ? __ldcs(lp + (size_t)u * stride) : 0;
    for (int s = 0; s < m; s += 4) {
        int nx[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) nx[u] = s + 4 + u < m ? __ldcs(lp + (size_t)(s + 4 + u) * stride) : 0;
        float4 l[4], g[4];
        X x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (s + u < m) {
                const int j = e[u] & kEntryMask;
                ldg_rec(LO.p, j, l[u], g[u]);
                x[u] = XS[j];
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (s + u < m) {
                float d[3];
                const float r2 = list_delta<DIM>(k, e[u], lo_i, l[u], d);
                if (r2 < k.R2) body(e[u] & kEntryMask, d, r2, s + u, l[u].w, g[u], x[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) e[u] = nx[u];
    }
}

// for_nbrs_g without a payload: body(j, d, r2, slot, type_j, m_V_j).
template <int DIM, bool FB, class F>
__device__ __forceinline__ void for_nbrs(const K32& k, int i, const int* __restrict__ cnt, const int* __restrict__ nbr,
                                         const float4* __restrict__ HI, RecView LO,
                                         const float4* __restrict__ PF, const int* __restrict__ dstart,
                                         const int* __restrict__ sstart, bool flow_i, F&& body) {
    for_nbrs_g<DIM, FB>(k, i, cnt, nbr, HI, LO, PF, dstart, sstart, flow_i, [](int) { return NoPayload{}; },
                        [&](int j, const float* d, float r2, int s, int tj, float mV, NoPayload) {
                            body(j, d, r2, s, tj, mV);
                        });
}

// Particle loop shared by the list kernels (FB = false: one particle per thread, skipping
// overflowed lists) and their overflow passes (FB = true: grid-stride over the overflow list).
struct Ovf {
    const int* list;
    const int* count;
};
#define FOR_PARTICLES(FB, BASE, N, OVF, CNT, MAXN, ...)                                         \
    do {                                                                                        \
        if (!(FB)) {                                                                            \
            const int i = (BASE) + blockIdx.x * blockDim.x + threadIdx.x;                       \
            if (i < (N) && (CNT)[i] <= (MAXN)) { __VA_ARGS__ }                                  \
        } else {                                                                                \
            const int no = *(OVF).count;                                                        \
            for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < no; q += gridDim.x * blockDim.x) { \
                const int i = (OVF).list[q];                                                    \
                if (i >= (BASE) && i < (N)) { __VA_ARGS__ }                                     \
            }                                                                                   \
        }                                                                                       \
    } while (0)

// FOR_PARTICLES over the direct range [BASE, LIM) followed by the listed particles
// ACT[0 .. *NACT) (ACT may be null) in the main pass; the overflow pass (FB) takes the
// overflowed particles in [BASE, N), as FOR_PARTICLES does.
#define FOR_PARTICLES_ACT(FB, BASE, LIM, ACT, NACT, N, OVF, CNT, MAXN, ...)                     \
    do {                                                                                        \
        if (!(FB)) {                                                                            \
            const int q_ = blockIdx.x * blockDim.x + threadIdx.x;                               \
            const int nlim_ = (LIM) - (BASE);                                                   \
            int i_ = -1;                                                                        \
            if (q_ < nlim_) i_ = (BASE) + q_;                                                   \
            else if ((ACT) && q_ - nlim_ < *(NACT)) i_ = (ACT)[q_ - nlim_];                     \
            const int i = i_;                                                                   \
            if (i >= 0 && (CNT)[i] <= (MAXN)) { __VA_ARGS__ }                                   \
        } else {                                                                                \
            const int no = *(OVF).count;                                                        \
            for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < no; q += gridDim.x * blockDim.x) { \
                const int i = (OVF).list[q];                                                    \
                if (i >= (BASE) && i < (N)) { __VA_ARGS__ }                                     \
            }                                                                                   \
        }                                                                                       \
    } while (0)

// Persistent per-particle state of the FP32-mixed form.
struct P32 {
    float4* hi;     // (hx, hy, hz, type word)
    RecView lo;     // (lx, ly, lz, m_V), first half of the interleaved records
    float4* vel;    // (vx, vy, vz, pressure)
    float* drho;    // density - rho0
    float* mass;
    int4* ids;      // (id0, mat_id, obj_id, is_dynamic)
    // granular solvers only (nullptr for WCSPH)
    float* sig;     // stress, 6 planes of n (symmetric: xx, yy, zz, xy, xz, yz)
    float* eeq;     // equivalent strain
    float* eeqp;    // equivalent plastic strain (Drucker-Prager)
    int* flag;      // return-mapping case (Drucker-Prager)
    float4* vlo;    // velocity low part: v = vel.xyz + vlo.xyz (compensated time integration)
};

// Symmetric 3x3 tensors are stored as six planes: xx, yy, zz, xy, xz, yz.
__device__ __forceinline__ int sym_idx(int a, int b) { return a == b ? a : 2 + a + b; }

// ---------------------------------------------------------------- transient state
struct T32 {
    RecView vt;     // (v_tmp, p / rho_tmp^2), second half of the current buffer's records
    float2* pr;     // (pressure, rho_tmp)
    float* drt;     // rho_tmp - rho0
    float* dd;      // d_density
    float4* dv;     // d_vel
    float* cf;      // CSPM_f
    float* L;       // inverse CSPM matrix, 6 symmetric planes (xx, yy, zz, xy, xz, yz)
    float4* xs;     // XSPH sums
    int* cnt;
    int* nbr;
    // granular solvers only
    float* sigt;    // stress_tmp, 6 planes
    float* dsig;    // d_stress, 6 planes (Drucker-Prager)
    float* dee;     // d_strain_equ
    float* deep;    // d_strain_equ_p (Drucker-Prager)
    float4* vtlo;   // v_tmp low part (zero for dummies)
    float4* srec;   // stress_tmp and rho_tmp - rho0 packed per particle (k_pack_stress32)
    // RK4 accumulators (time_integration 4 only)
    float* ddrk;
    float4* dvrk;
    float* dsigrk;  // 6 planes (Drucker-Prager)
};

// Compensated velocities of the granular solvers.  The strain rate of mu(I) is regularised
// only by 1e-8 1/s, so in regions of near-rigid motion (a free-falling surface layer) the
// f32 rounding noise of stored velocities (~1e-6 1/s of spurious strain rate) would set the
// stress direction and its sensitivity to cohesion; keeping v as an unevaluated sum
// hi + lo (two f32) makes velocity differences exact to ~1e-14 relative.
// (hi, lo) += a with an error-free two-sum.  The additions are explicit round-to-nearest
// operations: a contracted a = x * y into fma(x, y, hi) would break the error term.
__device__ __forceinline__ void two_sum_add(float& hi, float& lo, float a) {
    const float s = __fadd_rn(hi, a);
    const float bb = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(a, bb));
    const float l = __fadd_rn(lo, e);
    hi = __fadd_rn(s, l);
    lo = __fsub_rn(l, __fsub_rn(hi, s));
}
// (vj - vi) of two compensated velocities, component-wise.
__device__ __forceinline__ float dv_comp(float hj, float lj, float hi_, float li) { return (hj - hi_) + (lj - li); }

// ---------------------------------------------------------------- granular solvers
// Drucker-Prager invariants and stress adaptation (eng/solver_sph_dp.py:42-109) on the
// six stored components; s:s counts each off-diagonal entry twice.
__device__ __forceinline__ void dp_inv32(const K32& k, const float* st, float* s, float& I1, float& sJ2, float& f) {
    const float tr = (st[0] + st[1]) + st[2];
    const float t3 = tr / 3.f;
    s[0] = st[0] - t3; s[1] = st[1] - t3; s[2] = st[2] - t3;
    s[3] = st[3]; s[4] = st[4]; s[5] = st[5];
    I1 = tr;
    const float ss = s[0] * s[0] + s[1] * s[1] + s[2] * s[2] + 2.f * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]);
    sJ2 = sqrtf(0.5f * ss);
    f = sJ2 + k.alpha * I1 - k.k_c;
}
__device__ __forceinline__ void dp_adapt32(const K32& k, float* st) {
    float s[6], I1, sJ2, f;
    dp_inv32(k, st, s, I1, sJ2, f);
    if (f > (float)EPS_F) {
        if (f > sJ2) {
            const float tt = (I1 - k.kc_over_alpha) / 3.f;
            st[0] -= tt; st[1] -= tt; st[2] -= tt;
        }
        dp_inv32(k, st, s, I1, sJ2, f);
        const float r = (-I1 * k.alpha + k.k_c) / sJ2;
        for (int q = 0; q < 6; ++q) st[q] = r * s[q] + (q < 3 ? I1 / 3.f : 0.f);
    }
}
__device__ __forceinline__ int dp_flag32(const K32& k, const float* st) {
    float s[6], I1, sJ2, f;
    dp_inv32(k, st, s, I1, sJ2, f);
    if (f < -(float)EPS_F) return 0;
    if (f > (float)EPS_F) return f >= sJ2 ? 3 : 2;
    return 1;
}

__device__ __forceinline__ void load_sym(const float* __restrict__ a, size_t n, int i, float* out) {
    for (int q = 0; q < 6; ++q) out[q] = a[q * n + i];
}
__device__ __forceinline__ void store_sym(float* __restrict__ a, size_t n, int i, const float* v) {
    for (int q = 0; q < 6; ++q) a[q * n + i] = v[q];
}

// Corrected kernel gradient L (G d) (or G d when CORR is off).
template <int DIM, bool CORR>
__device__ __forceinline__ void grad_c(const float* L, float gf, const float* d, float* kc) {
    const float gx = gf * d[0], gy = gf * d[1], gz = DIM == 3 ? gf * d[2] : 0.f;
    if (CORR) {
        kc[0] = L[0] * gx + L[1] * gy + (DIM == 3 ? L[2] * gz : 0.f);
        kc[1] = L[3] * gx + L[4] * gy + (DIM == 3 ? L[5] * gz : 0.f);
        kc[2] = DIM == 3 ? L[6] * gx + L[7] * gy + L[8] * gz : 0.f;
    } else {
        kc[0] = gx; kc[1] = gy; kc[2] = gz;
    }
}

// Velocity gradient sum_j m_Vj (v_j - v_i) (x) kc and continuity sum_j m_Vj (v_i - v_j) . kc.
template <int DIM>
__device__ __forceinline__ void vgrad_add(float mVj, const float4& vti, const float4& vli, const float4& vtj,
                                          const float4& vlj, const float* kc, float* vg, CSum& dd) {
    const float u[3] = {mVj * dv_comp(vtj.x, vlj.x, vti.x, vli.x), mVj * dv_comp(vtj.y, vlj.y, vti.y, vli.y),
                        DIM == 3 ? mVj * dv_comp(vtj.z, vlj.z, vti.z, vli.z) : 0.f};
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
        for (int b = 0; b < DIM; ++b) vg[3 * a + b] += u[a] * kc[b];
    dd.add(-(u[0] * kc[0] + u[1] * kc[1] + (DIM == 3 ? u[2] * kc[2] : 0.f)));
}

// Symmetric / antisymmetric parts of a full velocity gradient.
__device__ __forceinline__ void strain_rate(const float* vg, float* er) {
    er[0] = vg[0]; er[1] = vg[4]; er[2] = vg[8];
    er[3] = 0.5f * (vg[1] + vg[3]); er[4] = 0.5f * (vg[2] + vg[6]); er[5] = 0.5f * (vg[5] + vg[7]);
}
__device__ __forceinline__ float sym_dd(const float* a, const float* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + 2.f * (a[3] * b[3] + a[4] * b[4] + a[5] * b[5]);
}
__device__ __forceinline__ float equiv_rate(const float* er) {  // sqrt(2/3 dev(e):dev(e))
    const float t3 = ((er[0] + er[1]) + er[2]) / 3.f;
    float ed[6] = {er[0] - t3, er[1] - t3, er[2] - t3, er[3], er[4], er[5]};
    return sqrtf(sym_dd(ed, ed) * 2.f / 3.f);
}

}  // namespace f32

// ---------------------------------------------------------------- host-side state
using f32::K32;
using f32::P32;
using f32::T32;

struct Fp32State {
    K32 k{};
    Consts c{};
    int n = 0, nd = 0;
    P32 P[2]{};
    int cur = 0;
    T32 T{};
    float4* pf = nullptr;
    int *dcount = nullptr, *dstart = nullptr, *scount = nullptr, *sstart = nullptr;
    int *cell_of = nullptr, *rank = nullptr, *perm = nullptr, *tiles = nullptr, *err = nullptr;
    int *cells_d = nullptr, *cells_s = nullptr, *ncells = nullptr;  // non-empty cells (dynamic, static)
    int *ovf_list = nullptr, *novf = nullptr;  // particles whose neighbours exceed the list capacity
    int *sact = nullptr, *nsact = nullptr;     // static-block particles with a non-empty list
    // dynamic rigid bodies (WCSPH): objects, per-object list slices, and each rigid
    // particle's rest offset x0 - rest centre of mass in f64, indexed by id0; the shape
    // matching's per-chunk partial sums (rnobj x r_chunks x 9), centres of mass (3 rnobj)
    // and rotations (9 rnobj)
    int rnobj = 0, r_chunks = 0;
    int *r_ids = nullptr, *r_off = nullptr, *r_list = nullptr, *r_scratch = nullptr;
    double *r_q = nullptr, *r_part = nullptr, *r_cm = nullptr, *r_rot = nullptr;
    unsigned* maxdisp = nullptr;               // squared displacement since the last list build
    int *sort_big = nullptr, *sort_nbig = nullptr;  // the cell sort's cells above kSortSmall particles
    bool built = false;
    double* stage = nullptr;       // f64 export staging (9 n)
    double* scratch = nullptr;
    std::vector<void*> allocs;
    std::vector<std::pair<std::string, double*>> views;
    bool lists_valid = false;
    long long rebuilds = 0;        // list builds since creation
    int nscenes = 0;               // > 0 for a batched ensemble
    // launch configuration (tsg_set_launch / tsg_autotune): threads per block of the
    // neighbour kernels, cells per CTA of the warp-per-cell list build (0: one thread per
    // particle), steps per captured graph
    int tpb = 128, cells_per_cta = 4, steps_per_graph = 1;
    // captured step graphs: [0] one step, [1] steps_per_graph steps
    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        int steps = 0, cur = -1, tpb = 0, cpc = 0;
        bool collide = false;
        long long kernels = 0;    // kernel nodes outside the conditional rebuild bodies
    } graphs[2];
    long long body_kernels = 0;   // kernel nodes of one rebuild body
    int* d_rebuilds = nullptr;    // rebuilds taken by graph replays (device counter)
    int rebuilds_seen = 0;        // part of d_rebuilds already folded into the counters
    // field export to host memory: conversion of one chunk overlaps the copy of the one before
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_ev[5] = {};
    void* snap = nullptr;         // autotuner snapshot of the particle state
    void* adj = nullptr;          // adjoint work buffers (tsg_adjoint.cu)
};


namespace f32 {
// Host helpers shared with the adjoint unit (defined in tsg_fp32.cu).
// Re-sort the dynamic block and rebuild every list (in_place keeps the current buffer).
void rebuild(Fp32State& st, cudaStream_t s, bool in_place);
// One step after the re-sort: correction, init_real2tmp, integrator, advect_pos, post-step.
void step_body(Fp32State& st, cudaStream_t s, bool collide, bool fold_disp = false);
}  // namespace f32

}  // namespace tsg
