// FP32-mixed form of the per-substep SPH path.
//
// Layout (unified particle index space, every array in the current sorted order):
//   [0, nd)  dynamic block: real particles (fluid / soil / kinematic rigid), re-sorted by
//            cell every step;
//   [nd, n)  static block: dummy and repulsive particles, which never move, sorted by cell
//            once at upload.  Each block has its own cell table (exclusive starts, G + 2).
// Positions are x - vdomain_start = hi + lo with hi an exact multiple of a power-of-two
// quantum Q (about one cell) and lo an f32 remainder, so x_i - x_j = (hi_i - hi_j) +
// (lo_i - lo_j) keeps ~1e-9 m resolution anywhere in the domain.  Density is stored as the
// deviation from the rest density (rho - rho0), which keeps the Tait pressure accurate.
// Arithmetic is f32 except the cell index (f64, truncating cast as the reference,
// eng/particle_system.py:216-218) and the FP64 conservation reductions.
//
// Neighbour lists: after the sort one kernel tests every candidate of the 3^dim stencil
// (f32 prefilter on absolute positions, exact test on hi/lo inside a thin band) and writes
// an ELL list per particle (slot-major, so a warp's reads coalesce).  Flow particles list
// every neighbour; boundary and rigid particles list flow neighbours only (all their sums
// run over flow particles).  Positions stay fixed until advect_pos, so the kernel
// correction, both boundary passes and both rate passes of a leap-frog step reuse one list.
// A particle whose count exceeds the capacity is handled by direct traversal.
//
// Sums over neighbours are block-compensated: plain f32 sums over 8 neighbours, then a
// Kahan update of the running total.
//
// Reference: eng/particle_system.py:228-269 (cell list), eng/solver_sph_base.py:41-238,
// :363-423, :648-669 (step, CSPM, boundary), eng/solver_sph_wc.py:82-132 (WCSPH).
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "tsg_fp32.h"

namespace tsg {

namespace {

constexpr int TPB = 128;
inline int nblk(long long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

struct K32 {
    int n, nd, dim, kernel, corr, xsph, boundary, solver, maxn, exponent_is_int, gamma_i;
    int gnum[3];
    long long G;
    double vs[3], grid;
    float Q, inv_grid, h1, kk, kk6, wgrad, cub1, cub2, R2, R2lo, R2hi, pf_lim;
    float R2L, R2Lhi, disp2_limit;  // list radius (support + skin) and rebuild threshold
    float visc_fac, eps_h2, rho0, B, gamma, dt, hdt, g[3], rep_fac, diam, h075, r_eps;
    float ds[3], de[3];
};

__device__ __forceinline__ int tf_type(float w) { return (int)(short)(__float_as_int(w) & 0xffff); }
__device__ __forceinline__ int tf_dyn(float w) { return (__float_as_int(w) >> 16) & 1; }
__device__ __forceinline__ bool is_flow(int t) { return t == MAT_FLUID || t == MAT_SOIL; }

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

// Cell coordinate trunc((hi + lo) / grid) with the f64 semantics of the reference's cast:
// an f32 estimate decides unless it lies within 1e-3 of an integer, where f64 decides.
__device__ __forceinline__ long long cell_coord(const K32& k, float hi, float lo, bool& ok) {
    const float tf = (hi + lo) * k.inv_grid;
    const float fr = tf - truncf(tf);
    if (fabsf(tf) < 1.0e6f && fabsf(fr) > 1e-3f && fabsf(fr) < 0.999f) return (long long)(int)tf;
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

template <int DIM>
__device__ __forceinline__ void delta(const float4& hi_i, const float4& lo_i, const float4& hi_j, const float4& lo_j,
                                      float* d) {
    d[0] = (hi_i.x - hi_j.x) + (lo_i.x - lo_j.x);
    d[1] = (hi_i.y - hi_j.y) + (lo_i.y - lo_j.y);
    d[2] = DIM == 3 ? (hi_i.z - hi_j.z) + (lo_i.z - lo_j.z) : 0.f;
}

// Candidate enumeration over the stencil of i (reference traversal order of cells, dynamic
// block first, then the static block for flow centres).  body(j, d, r2) gets the exact
// f32 displacement x_i - x_j.
template <int DIM, class F>
__device__ __forceinline__ void enum_neighbors(const K32& k, int i, const float4* __restrict__ HI,
                                               const float4* __restrict__ LO, const float4* __restrict__ PF,
                                               const int* __restrict__ dstart, const int* __restrict__ sstart,
                                               bool flow_i, F&& body, bool list_radius = false) {
    const float cut2 = list_radius ? k.R2L : k.R2;
    const float cut2hi = list_radius ? k.R2Lhi : k.R2hi;
    const float4 hi_i = HI[i], lo_i = LO[i], pf_i = PF[i];
    bool ok = true;
    const long long cc0 = cell_coord(k, hi_i.x, lo_i.x, ok);
    const long long cc1 = cell_coord(k, hi_i.y, lo_i.y, ok);
    const long long cc2 = cell_coord(k, hi_i.z, lo_i.z, ok);
    if (!ok) return;
    const bool pf = fabsf(pf_i.x) < k.pf_lim && fabsf(pf_i.y) < k.pf_lim && fabsf(pf_i.z) < k.pf_lim;
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
                    float r2 = d[0] * d[0] + d[1] * d[1];
                    if (DIM == 3) r2 += d[2] * d[2];
                    if (!(r2 < cut2)) continue;
                    body(j, d, r2);
                }
            }
        }
    }
}

// Iterate i's neighbour list (FB = false) or traverse its stencil directly (FB = true: the
// particle's list overflowed).  The next list index is fetched one iteration ahead.
template <int DIM, bool FB, class F>
__device__ __forceinline__ void for_nbrs(const K32& k, int i, const int* __restrict__ cnt, const int* __restrict__ nbr,
                                         const float4* __restrict__ HI, const float4* __restrict__ LO,
                                         const float4* __restrict__ PF, const int* __restrict__ dstart,
                                         const int* __restrict__ sstart, bool flow_i, F&& body) {
    if (!FB) {
        const int m = cnt[i];
        const float4 hi_i = HI[i], lo_i = LO[i];
        const size_t stride = (size_t)k.n;
        const int* lp = nbr + i;
        // two neighbours per trip: both index loads, then both position loads, then compute
        int s = 0;
        for (; s + 1 < m; s += 2) {
            const int j0 = lp[0], j1 = lp[stride];
            lp += 2 * stride;
            const float4 h0 = HI[j0], l0 = LO[j0], h1 = HI[j1], l1 = LO[j1];
            float d0[3], d1[3];
            delta<DIM>(hi_i, lo_i, h0, l0, d0);
            delta<DIM>(hi_i, lo_i, h1, l1, d1);
            float r20 = d0[0] * d0[0] + d0[1] * d0[1];
            float r21 = d1[0] * d1[0] + d1[1] * d1[1];
            if (DIM == 3) { r20 += d0[2] * d0[2]; r21 += d1[2] * d1[2]; }
            if (r20 < k.R2) body(j0, d0, r20, s);        // lists hold support + skin
            if (r21 < k.R2) body(j1, d1, r21, s + 1);
        }
        if (s < m) {
            const int j = lp[0];
            float d[3];
            delta<DIM>(hi_i, lo_i, HI[j], LO[j], d);
            float r2 = d[0] * d[0] + d[1] * d[1];
            if (DIM == 3) r2 += d[2] * d[2];
            if (r2 < k.R2) body(j, d, r2, s);
        }
    } else {
        int s = 0;
        enum_neighbors<DIM>(k, i, HI, LO, PF, dstart, sstart, flow_i,
                            [&](int j, const float* d, float r2) { body(j, d, r2, s++); });
    }
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

// ---------------------------------------------------------------- sort (dynamic block)
__global__ void k_hash32(K32 k, int count_n, int base, const float4* __restrict__ HI, const float4* __restrict__ LO,
                         int* __restrict__ cell_of, int* __restrict__ rank, int* __restrict__ count, int* __restrict__ err) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count_n) return;
    const int i = base + t;
    const float4 h = HI[i], l = LO[i];
    long long idx[3];
    bool ok = true;
    const float hv[3] = {h.x, h.y, h.z}, lv[3] = {l.x, l.y, l.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) idx[d] = cell_coord(k, hv[d], lv[d], ok);
    long long f = idx[0] * k.gnum[1] * k.gnum[2] + idx[1] * k.gnum[2] + idx[2];
    if (!ok || f < 0 || f >= k.G) {
        f = k.G;
        atomicOr(err, ok ? TSG_ERR_CELL_OOB : (TSG_ERR_CELL_OOB | TSG_ERR_NONFINITE));
    }
    cell_of[t] = (int)f;
    rank[t] = atomicAdd(&count[f], 1);
}

__global__ void k_scatter32(int count_n, const int* __restrict__ cell_of, const int* __restrict__ rank,
                            const int* __restrict__ cell_start, int* __restrict__ perm) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count_n) return;
    perm[cell_start[cell_of[t]] + rank[t]] = t;
}

__global__ void k_cell_sort32(long long ncell, const int* __restrict__ cell_start, int* __restrict__ perm) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    int b = cell_start[c], e = cell_start[c + 1];
    for (int q = b + 1; q < e; ++q) {
        int v = perm[q];
        int m = q - 1;
        while (m >= b && perm[m] > v) { perm[m + 1] = perm[m]; --m; }
        perm[m + 1] = v;
    }
}

// Persistent per-particle state of the FP32-mixed form.
struct P32 {
    float4* hi;     // (hx, hy, hz, m_V)
    float4* lo;     // (lx, ly, lz, type word)
    float4* vel;    // (vx, vy, vz, pressure)
    float* drho;    // density - rho0
    float* mass;
    int4* ids;      // (id0, mat_id, obj_id, is_dynamic)
};

// Gather block [base, base + count_n) from a into b (new order), renormalise hi/lo and
// refresh the prefilter position.
__global__ void k_reorder32(K32 k, int count_n, int base, const int* __restrict__ perm, P32 a, P32 b,
                            float4* __restrict__ PF) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count_n) return;
    const int dst = base + t, src = base + perm[t];
    float4 h = a.hi[src], l = a.lo[src];
    float hv[3] = {h.x, h.y, h.z}, lv[3] = {l.x, l.y, l.z};
    float pfv[3];
    for (int d = 0; d < 3; ++d) {
        double x = (double)hv[d] + (double)lv[d];
        double hq = (double)k.Q * rint(x / (double)k.Q);
        hv[d] = (float)hq;
        lv[d] = (float)(x - hq);
        pfv[d] = (float)x;
    }
    b.hi[dst] = make_float4(hv[0], hv[1], hv[2], h.w);
    b.lo[dst] = make_float4(lv[0], lv[1], lv[2], l.w);
    b.vel[dst] = a.vel[src];
    b.drho[dst] = a.drho[src];
    b.mass[dst] = a.mass[src];
    b.ids[dst] = a.ids[src];
    PF[dst] = make_float4(pfv[0], pfv[1], pfv[2], l.w);
}

// Record a particle whose neighbours exceed the list capacity (processed by FB passes).
__device__ __forceinline__ void note_overflow(int* ovf_list, int* novf, int i) {
    ovf_list[atomicAdd(novf, 1)] = i;
}

// ---------------------------------------------------------------- neighbour lists
template <int DIM>
__global__ void k_lists(K32 k, const float4* __restrict__ HI, const float4* __restrict__ LO,
                        const float4* __restrict__ PF, const int* __restrict__ dstart, const int* __restrict__ sstart,
                        int* __restrict__ cnt, int* __restrict__ nbr, int* __restrict__ ovf_list, int* __restrict__ novf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const bool flow_i = is_flow(tf_type(PF[i].w));
    int m = 0;
    enum_neighbors<DIM>(k, i, HI, LO, PF, dstart, sstart, flow_i, [&](int j, const float*, float) {
        if (m < k.maxn) nbr[(size_t)m * k.n + i] = j;
        ++m;
    }, true);
    cnt[i] = m;
    if (m > k.maxn) note_overflow(ovf_list, novf, i);
}

// Warp-per-cell list build (3D): the lanes of a warp are the particles of one cell, so
// they share one stencil; each candidate row is staged through shared memory with
// coalesced loads and tested by every lane from a broadcast read.  Lanes whose particle
// sits in an aliased cell (true cell coordinates outside the grid) and particles in the
// out-of-grid bin take the per-particle path.
template <int DIM>
__global__ void k_lists_cell(K32 k, int self_blk, const int* __restrict__ cells, const int* __restrict__ cell_count,
                             const float4* __restrict__ HI, const float4* __restrict__ LO,
                             const float4* __restrict__ PF, const int* __restrict__ dstart,
                             const int* __restrict__ sstart, int* __restrict__ cnt, int* __restrict__ nbr,
                             int* __restrict__ ovf_list, int* __restrict__ novf) {
    __shared__ float4 sh_rel[4][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int* own = self_blk == 0 ? dstart : sstart;
    const int ncell = *cell_count;
    const long long ny = k.gnum[1], nz = k.gnum[2], G = k.G;
    for (int w = blockIdx.x * 4 + wib; w < ncell; w += gridDim.x * 4) {
    const long long c = cells[w];
    const int cb = own[c], ce = own[c + 1];
    const long long cx = c / (ny * nz), cy = (c / nz) % ny, cz = c % nz;
    // reference quantum of this cell: positions are staged as (hi - ref) + lo, exact in hi - ref
    const float4 ref = HI[cb];
    for (int p0 = cb; p0 < ce; p0 += 32) {
        const int i = p0 + lane;
        const bool active = i < ce;
        float rx = 0.f, ry = 0.f, rz = 0.f;
        bool flow_i = false, alias = false;
        if (active) {
            const float4 hi_i = HI[i], lo_i = LO[i];
            flow_i = is_flow(tf_type(lo_i.w));
            bool ok = true;
            alias = cell_coord(k, hi_i.x, lo_i.x, ok) != cx || cell_coord(k, hi_i.y, lo_i.y, ok) != cy ||
                    cell_coord(k, hi_i.z, lo_i.z, ok) != cz || !ok;
            rx = (hi_i.x - ref.x) + lo_i.x;
            ry = (hi_i.y - ref.y) + lo_i.y;
            rz = (hi_i.z - ref.z) + lo_i.z;
        }
        int m = 0;
        int* wp = nbr + (active ? i : 0);
        const size_t stride = (size_t)k.n;
        const bool any_flow = __any_sync(0xffffffffu, active && flow_i && !alias);
        for (int blk = 0; blk < (any_flow ? 2 : 1); ++blk) {
            const int* cs = blk == 0 ? dstart : sstart;
#pragma unroll 1
            for (int ox = -1; ox <= 1; ++ox) {
#pragma unroll 1
                for (int oy = (DIM == 3 ? -1 : 0); oy <= (DIM == 3 ? 1 : 0); ++oy) {
                    const long long f0 = (cx + ox) * ny * nz + (cy + oy) * nz + cz;
                    const long long lo = f0 - 1 > 0 ? f0 - 1 : 0;
                    const long long hi = f0 + 1 < G - 1 ? f0 + 1 : G - 1;
                    if (lo > hi) continue;
                    const int rb = cs[lo], re = cs[hi + 1];
                    for (int base = rb; base < re; base += 32) {
                        const int jj = base + lane;
                        if (jj < re) {
                            const float4 hj = HI[jj], lj = LO[jj];
                            sh_rel[wib][lane] = make_float4((hj.x - ref.x) + lj.x, (hj.y - ref.y) + lj.y,
                                                            (hj.z - ref.z) + lj.z, lj.w);
                        }
                        __syncwarp();
                        const int mm = re - base < 32 ? re - base : 32;
                        if (active && !alias && (blk == 0 || flow_i)) {
                            // test all staged candidates first (no stores in this loop, so the
                            // shared loads pipeline), then write the accepted ones
                            unsigned acc = 0u;
#pragma unroll 8
                            for (int t = 0; t < 32; ++t) {
                                const float4 q = sh_rel[wib][t];
                                const float dx = rx - q.x, dy = ry - q.y;
                                float r2 = dx * dx + dy * dy;
                                if (DIM == 3) {
                                    const float dz = rz - q.z;
                                    r2 += dz * dz;
                                }
                                const bool ok_type = flow_i || is_flow(tf_type(q.w));
                                acc |= (t < mm && r2 < k.R2L && ok_type) ? (1u << t) : 0u;
                            }
                            if (i >= base && i < base + 32) acc &= ~(1u << (i - base));
                            while (acc) {
                                const int t = __ffs(acc) - 1;
                                acc &= acc - 1u;
                                if (m < k.maxn) { *wp = base + t; wp += stride; }
                                ++m;
                            }
                        }
                        __syncwarp();
                    }
                }
            }
        }
        if (active) {
            cnt[i] = alias ? -1 : m;  // -1: rebuilt by k_lists_fixup
            if (!alias && m > k.maxn) note_overflow(ovf_list, novf, i);
        }
    }
    }
}

// Non-empty cells of one block's cell table (order irrelevant: each cell is independent).
__global__ void k_nonempty_cells(long long G, const int* __restrict__ start, int* __restrict__ cells,
                                 int* __restrict__ count) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool pred = c < G && start[c + 1] > start[c];
    const unsigned mask = __ballot_sync(0xffffffffu, pred);
    if (!mask) return;
    const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (pred) cells[base + __popc(mask & ((1u << lane) - 1u))] = (int)c;
}

// Per-particle list build for particles the warp-per-cell pass could not serve (their true
// cell differs from the storage cell); flagged with count -1.
template <int DIM>
__global__ void k_lists_fixup(K32 k, const float4* __restrict__ HI, const float4* __restrict__ LO,
                              const float4* __restrict__ PF, const int* __restrict__ dstart,
                              const int* __restrict__ sstart, int* __restrict__ cnt, int* __restrict__ nbr,
                              int* __restrict__ ovf_list, int* __restrict__ novf) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k.n; i += gridDim.x * blockDim.x) {
        if (cnt[i] >= 0) continue;
        const bool flow_i = is_flow(tf_type(PF[i].w));
        int m = 0;
        enum_neighbors<DIM>(k, i, HI, LO, PF, dstart, sstart, flow_i, [&](int j, const float*, float) {
            if (m < k.maxn) nbr[(size_t)m * k.n + i] = j;
            ++m;
        }, true);
        cnt[i] = m;
        if (m > k.maxn) note_overflow(ovf_list, novf, i);
    }
}

// Per-particle list build for an index range (out-of-grid bin).
template <int DIM>
__global__ void k_lists_range(K32 k, const int* __restrict__ bounds, const float4* __restrict__ HI,
                              const float4* __restrict__ LO, const float4* __restrict__ PF,
                              const int* __restrict__ dstart, const int* __restrict__ sstart,
                              int* __restrict__ cnt, int* __restrict__ nbr, int* __restrict__ ovf_list,
                              int* __restrict__ novf) {
    const int b0 = bounds[0], b1 = bounds[1];
    for (int i = b0 + blockIdx.x * blockDim.x + threadIdx.x; i < b1; i += gridDim.x * blockDim.x) {
        const bool flow_i = is_flow(tf_type(PF[i].w));
        int m = 0;
        enum_neighbors<DIM>(k, i, HI, LO, PF, dstart, sstart, flow_i, [&](int j, const float*, float) {
            if (m < k.maxn) nbr[(size_t)m * k.n + i] = j;
            ++m;
        }, true);
        cnt[i] = m;
        if (m > k.maxn) note_overflow(ovf_list, novf, i);
    }
}

// ---------------------------------------------------------------- transient state
struct T32 {
    float4* vt;     // (v_tmp, p / rho_tmp^2)
    float2* pr;     // (pressure, rho_tmp)
    float* drt;     // rho_tmp - rho0
    float* dd;      // d_density
    float4* dv;     // d_vel
    float* cf;      // CSPM_f
    float* L;       // CSPM_L, 9 planes
    float4* xs;     // XSPH sums
    int* cnt;
    int* nbr;
};

template <int DIM>
__device__ __forceinline__ void inv_store(const K32& k, float* L, int i, const double* m, bool flow_i) {
    double inv[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (flow_i) {
        if (DIM == 2) {
            double dt = m[0] * m[4] - m[1] * m[3];
            if (fabs(dt) > EPS) {
                double id = 1.0 / dt;
                inv[0] = id * m[4]; inv[1] = -id * m[1]; inv[3] = -id * m[3]; inv[4] = id * m[0]; inv[8] = 0.0;
            }
        } else {
            double dt = m[0] * (m[4] * m[8] - m[7] * m[5]) - m[3] * (m[1] * m[8] - m[7] * m[2]) + m[6] * (m[1] * m[5] - m[4] * m[2]);
            if (fabs(dt) > EPS) {
                double id = 1.0 / dt;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        inv[3 * b + a] = id * (m[3 * ((a + 1) % 3) + (b + 1) % 3] * m[3 * ((a + 2) % 3) + (b + 2) % 3]
                                             - m[3 * ((a + 2) % 3) + (b + 1) % 3] * m[3 * ((a + 1) % 3) + (b + 2) % 3]);
            }
        }
    }
    for (int q = 0; q < 9; ++q) L[(size_t)q * k.n + i] = (float)inv[q];
}

// CSPM (eng/solver_sph_base.py:386-423).
template <int DIM, bool FB>
__global__ void k_corr32(K32 k, P32 p, T32 t, const float4* __restrict__ PF, const int* __restrict__ dstart,
                         const int* __restrict__ sstart, Ovf ovf) {
    FOR_PARTICLES(FB, 0, k.n, ovf, t.cnt, k.maxn, {
        const int ti = tf_type(p.lo[i].w);
        const bool flow_i = is_flow(ti);
        const bool want_L = k.corr == 1 && flow_i;
        CSum s;
        float L[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for_nbrs<DIM, FB>(k, i, t.cnt, t.nbr, p.hi, p.lo, PF, dstart, sstart, flow_i,
                          [&](int j, const float* d, float r2, int sidx) {
            const float4 hj = p.hi[j];
            const int tj = tf_type(p.lo[j].w);
            const float r = fast_sqrt(r2);
            if (is_flow(tj)) s.add(hj.w * w_val(k, r));
            if ((sidx & 7) == 7) s.flush();
            if (want_L && tj == ti) {
                const float gf = w_grad(k, r) * hj.w;
                for (int a = 0; a < DIM; ++a)
                    for (int b = 0; b < DIM; ++b) L[3 * a + b] += (-d[a]) * (gf * d[b]);
            }
        });
        const float sum = s.get();
        t.cf[i] = sum != 0.f ? 1.f / sum : 1.f;
        if (k.corr == 1) {
            double m[9];
            for (int q = 0; q < 9; ++q) m[q] = L[q];
            inv_store<DIM>(k, t.L, i, m, want_L);
        }
    });
}

__global__ void k_init_tmp32(K32 k, P32 p, T32 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    if (tf_type(p.lo[i].w) > 0) {
        const float4 v = p.vel[i];
        t.vt[i] = make_float4(v.x, v.y, v.z, t.vt[i].w);
        t.drt[i] = p.drho[i];
    }
}

// Tait EOS from the density deviation e = (rho_tmp - rho0) / rho0:
// (1 + e)^g - 1 = e * sum_{k<g} (1 + e)^k for an integer exponent (no cancellation).
__device__ __forceinline__ float tait(const K32& k, float drt) {
    const float e = drt / k.rho0;
    float r;
    if (k.exponent_is_int && k.gamma_i >= 1) {
        const float a = 1.f + e;
        float sum = 1.f;
        for (int q = 1; q < k.gamma_i; ++q) sum = 1.f + a * sum;
        r = e * sum;
    } else {
        r = expm1f(k.gamma * log1pf(e));
    }
    return fmaxf(k.B * r, 0.f);
}

__global__ void k_pre32(K32 k, P32 p, T32 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    if (tf_type(p.lo[i].w) != MAT_FLUID) return;
    const float drt = t.drt[i];
    const float pr = tait(k, drt);
    const float rt = k.rho0 + drt;
    p.vel[i].w = pr;
    t.vt[i].w = pr / (rt * rt);
    t.pr[i] = make_float2(pr, rt);
}

// Boundary extrapolation for dummy / repulsive / rigid particles in [base, base + count_n) (WC).
template <int DIM, bool FB>
__global__ void k_bdy32(K32 k, P32 p, T32 t, const float4* __restrict__ PF, const int* __restrict__ dstart,
                        const int* __restrict__ sstart, int base, int count_n, Ovf ovf) {
    const int lim = base + count_n;
    FOR_PARTICLES(FB, base, lim, ovf, t.cnt, k.maxn, {
        const int ti = tf_type(p.lo[i].w);
        if (ti == MAT_DUMMY || ti == MAT_REP || ti == MAT_RIGID) {
            CSum bv[3], bp;
            const float4 hi_i = p.hi[i], lo_i = p.lo[i];
            for_nbrs<DIM, FB>(k, i, t.cnt, t.nbr, p.hi, p.lo, PF, dstart, sstart, false,
                              [&](int j, const float* d, float r2, int sidx) {
                const float w = w_val(k, fast_sqrt(r2));
                const float mV = p.hi[j].w;
                const float4 vt = t.vt[j];
                const float2 pr = t.pr[j];
                const float mw = mV * w;
                bv[0].add(mw * vt.x);
                bv[1].add(mw * vt.y);
                if (DIM == 3) bv[2].add(mw * vt.z);
                bp.add(mw * (pr.x + pr.y * k.g[1] * d[1]));
                if ((sidx & 7) == 7) { bv[0].flush(); bv[1].flush(); bv[2].flush(); bp.flush(); }
            });
            (void)hi_i; (void)lo_i;
            const float f = t.cf[i];
            const float4 v = p.vel[i];
            const float pv = fmaxf(bp.get() * f, 0.f);
            const float b0 = bv[0].get(), b1 = bv[1].get(), b2 = DIM == 3 ? bv[2].get() : 0.f;
            t.vt[i] = make_float4(2.f * v.x - b0 * f, 2.f * v.y - b1 * f, 2.f * v.z - b2 * f, pv / (k.rho0 * k.rho0));
            t.pr[i] = make_float2(pv, k.rho0);
            t.drt[i] = 0.f;
            p.vel[i].w = pv;
            if (ti == MAT_RIGID) { t.dd[i] = 0.f; t.dv[i] = make_float4(0.f, 0.f, 0.f, 0.f); }
        }
    });
}

// WCSPH continuity + momentum (eng/solver_sph_wc.py:108-126).
template <int DIM, bool FB, bool CORR>
__global__ void k_rates32(K32 k, P32 p, T32 t, const float4* __restrict__ PF, const int* __restrict__ dstart,
                          const int* __restrict__ sstart, Ovf ovf) {
    FOR_PARTICLES(FB, 0, k.nd, ovf, t.cnt, k.maxn, {
      if (tf_type(p.lo[i].w) == MAT_FLUID) {
        const float4 vti = t.vt[i];
        const float rti = k.rho0 + t.drt[i];
        const float visc_b = k.rho0 / rti;
        float L[9];
        if (CORR)
            for (int q = 0; q < 9; ++q) L[q] = t.L[(size_t)q * k.n + i];
        CSum dd, dv[3];
        const bool rep_on = k.boundary == 3 || k.boundary == 4;
        for_nbrs<DIM, FB>(k, i, t.cnt, t.nbr, p.hi, p.lo, PF, dstart, sstart, true,
                          [&](int j, const float* d, float r2, int sidx) {
            const float4 hj = p.hi[j];
            const int tj = tf_type(p.lo[j].w);
            const float4 vtj = t.vt[j];
            const float r = fast_sqrt(r2);
            const float gf = w_grad(k, r);
            const float dvx = vti.x - vtj.x, dvy = vti.y - vtj.y, dvz = vti.z - vtj.z;
            // continuity: m_Vj (v_i - v_j) . (L_i grad W)
            const float gx = gf * d[0], gy = gf * d[1], gz = DIM == 3 ? gf * d[2] : 0.f;
            if (CORR) {
                const float cx = L[0] * gx + L[1] * gy + (DIM == 3 ? L[2] * gz : 0.f);
                const float cy = L[3] * gx + L[4] * gy + (DIM == 3 ? L[5] * gz : 0.f);
                const float cz = DIM == 3 ? L[6] * gx + L[7] * gy + L[8] * gz : 0.f;
                dd.add(hj.w * (dvx * cx + dvy * cy + (DIM == 3 ? dvz * cz : 0.f)));
            } else {
                dd.add(hj.w * (dvx * gx + dvy * gy + (DIM == 3 ? dvz * gz : 0.f)));
            }
            // viscosity (fluid or boundary neighbours) and pressure, on the uncorrected gradient
            const float vdx = dvx * d[0] + dvy * d[1] + (DIM == 3 ? dvz * d[2] : 0.f);
            // WCSPH scenes hold fluid, dummy, repulsive and rigid particles only (soil is rejected
            // at upload), so every non-fluid neighbour takes the boundary form
            const float cv = __fdividef(k.visc_fac * hj.w * fminf(vdx, 0.f), r2 + k.eps_h2) *
                             (tj == MAT_FLUID ? 1.f : visc_b);
            const float cp = -k.rho0 * hj.w * (vti.w + vtj.w);
            float sc = (cv + cp) * gf;
            float rs = 0.f;
            if (rep_on && tj == MAT_REP) {  // repulsive force (eng/solver_sph_base.py:675-689)
                const float chi = (r > 0.f && r < k.diam) ? 1.f - r / k.diam : 0.f;
                const float gm = r / k.h075;
                float f = 0.f;
                if (gm > 0.f && gm <= 2.f / 3.f) f = 2.f / 3.f;
                else if (gm > 2.f / 3.f && gm <= 1.f) f = 2.f * gm - 1.5f * gm * gm;
                else if (gm > 1.f && gm < 2.f) f = 0.5f * (2.f - gm) * (2.f - gm);
                rs = k.rep_fac * chi * f / r2;
            }
            sc += rs;
            dv[0].add(sc * d[0]);
            dv[1].add(sc * d[1]);
            if (DIM == 3) dv[2].add(sc * d[2]);
            if ((sidx & 7) == 7) { dd.flush(); dv[0].flush(); dv[1].flush(); dv[2].flush(); }
        });
        t.dd[i] = dd.get() * rti;
        t.dv[i] = make_float4(dv[0].get() + k.g[0], dv[1].get() + k.g[1],
                              (DIM == 3 ? dv[2].get() : 0.f) + k.g[2], 0.f);
      }
    });
}

// ---------------------------------------------------------------- integrators
__global__ void k_advect_half32(K32 k, P32 p, T32 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    if (tf_type(p.lo[i].w) <= 0) return;
    const float drt = t.drt[i] + k.hdt * t.dd[i];
    t.drt[i] = drt;
    p.hi[i].w = p.mass[i] / (k.rho0 + drt);
    const float4 dv = t.dv[i];
    float4 vt = t.vt[i];
    vt.x += k.hdt * dv.x; vt.y += k.hdt * dv.y; vt.z += k.hdt * dv.z;
    t.vt[i] = vt;
}

__global__ void k_advect_full32(K32 k, P32 p, T32 t, int* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    if (tf_type(p.lo[i].w) <= 0) return;
    const float dr = p.drho[i] + k.dt * t.dd[i];
    p.drho[i] = dr;
    p.hi[i].w = p.mass[i] / (k.rho0 + dr);
    const float4 dv = t.dv[i];
    float4 v = p.vel[i];
    v.x += k.dt * dv.x; v.y += k.dt * dv.y; v.z += k.dt * dv.z;
    p.vel[i] = v;
    if (!isfinite(dr)) atomicOr(err, TSG_ERR_NONFINITE);
}

template <int DIM, bool FB>
__global__ void k_xsph32(K32 k, P32 p, T32 t, const float4* __restrict__ PF, const int* __restrict__ dstart,
                         const int* __restrict__ sstart, Ovf ovf) {
    FOR_PARTICLES(FB, 0, k.nd, ovf, t.cnt, k.maxn, {
        const int ti = tf_type(p.lo[i].w);
        if (ti > 0 && tf_dyn(p.lo[i].w)) {
            const float4 vi = p.vel[i];
            CSum s[3];
            for_nbrs<DIM, FB>(k, i, t.cnt, t.nbr, p.hi, p.lo, PF, dstart, sstart, is_flow(ti),
                              [&](int j, const float*, float r2, int sidx) {
                if (tf_type(p.lo[j].w) != ti) return;
                const float w = w_val(k, fast_sqrt(r2)) * p.hi[j].w;
                const float4 vj = p.vel[j];
                s[0].add(w * (vj.x - vi.x));
                s[1].add(w * (vj.y - vi.y));
                if (DIM == 3) s[2].add(w * (vj.z - vi.z));
                if ((sidx & 7) == 7) { s[0].flush(); s[1].flush(); s[2].flush(); }
            });
            t.xs[i] = make_float4(s[0].get(), s[1].get(), DIM == 3 ? s[2].get() : 0.f, 0.f);
        }
    });
}

__global__ void k_advect_pos32(K32 k, P32 p, T32 t, int* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    const float w = p.lo[i].w;
    if (tf_type(w) <= 0) return;
    const float4 v = p.vel[i];
    float4 l = p.lo[i];
    if (k.xsph && tf_dyn(w)) {
        const float4 s = t.xs[i];
        l.x += k.dt * (v.x + 0.5f * s.x);
        l.y += k.dt * (v.y + 0.5f * s.y);
        l.z += k.dt * (v.z + 0.5f * s.z);
    } else {
        l.x += k.dt * v.x;
        l.y += k.dt * v.y;
        l.z += k.dt * v.z;
    }
    p.lo[i] = l;
    if (!(isfinite(l.x) && isfinite(l.y) && isfinite(l.z))) atomicOr(err, TSG_ERR_NONFINITE);
}

__global__ void k_post_wc32(K32 k, P32 p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    if (tf_type(p.lo[i].w) != MAT_FLUID) return;
    const float dr = fmaxf(p.drho[i], 0.f);
    p.drho[i] = dr;
    p.hi[i].w = p.mass[i] / (k.rho0 + dr);
}

// Collision boundary (eng/solver_sph_base.py:525-601), flow particles when boundary == 1.
__global__ void k_enforce32(K32 k, P32 p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    const int ti = tf_type(p.lo[i].w);
    const bool rigid_dyn = ti == MAT_RIGID && tf_dyn(p.lo[i].w);
    const bool on = k.boundary == 1 ? (is_flow(ti) || rigid_dyn) : rigid_dyn;
    if (!on) return;
    float4 h = p.hi[i], l = p.lo[i];
    float pos[3] = {h.x + l.x + (float)k.vs[0], h.y + l.y + (float)k.vs[1], h.z + l.z + (float)k.vs[2]};
    float nrm[3] = {0.f, 0.f, 0.f};
    float newp[3] = {pos[0], pos[1], pos[2]};
    const float r = k.r_eps;
    if (pos[0] > k.de[0] - r) { nrm[0] += 1.f; newp[0] = k.de[0] - r; }
    if (pos[0] <= k.ds[0] + r) { nrm[0] -= 1.f; newp[0] = k.ds[0] + r; }
    if (pos[1] <= k.ds[1] + r) { nrm[1] -= 1.f; newp[1] = k.ds[1] + r; }
    if (k.dim == 3) {
        if (pos[2] > k.de[2] - r) { nrm[2] += 1.f; newp[2] = k.de[2] - r; }
        if (pos[2] <= k.ds[2] + r) { nrm[2] -= 1.f; newp[2] = k.ds[2] + r; }
    }
    l.x = (newp[0] - (float)k.vs[0]) - h.x;
    l.y = (newp[1] - (float)k.vs[1]) - h.y;
    l.z = (newp[2] - (float)k.vs[2]) - h.z;
    if (nrm[0] != 0.f || nrm[1] != 0.f || nrm[2] != 0.f) p.lo[i] = l;
    const float ln = sqrtf(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    if (ln > 1e-8f) {
        float4 v = p.vel[i];
        const float u0 = nrm[0] / ln, u1 = nrm[1] / ln, u2 = nrm[2] / ln;
        const float vd = v.x * u0 + v.y * u1 + v.z * u2;
        v.x -= 1.3f * vd * u0; v.y -= 1.3f * vd * u1; v.z -= 1.3f * vd * u2;
        p.vel[i] = v;
    }
}

// ---------------------------------------------------------------- export / diagnostics
__global__ void k_export(K32 k, P32 p, T32 t, int what, double* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const size_t n = k.n;
    switch (what) {
    case 0: {  // x
        float4 h = p.hi[i], l = p.lo[i];
        out[i] = k.vs[0] + ((double)h.x + (double)l.x);
        out[n + i] = k.vs[1] + ((double)h.y + (double)l.y);
        out[2 * n + i] = k.vs[2] + ((double)h.z + (double)l.z);
        break;
    }
    case 1: { float4 v = p.vel[i]; out[i] = v.x; out[n + i] = v.y; out[2 * n + i] = v.z; break; }
    case 2: out[i] = tf_type(p.lo[i].w) > 0 ? (double)k.rho0 + (double)p.drho[i] : 0.0; break;  // density
    case 3: out[i] = p.vel[i].w; break;                       // pressure
    case 4: out[i] = p.hi[i].w; break;                        // m_V
    case 5: out[i] = p.mass[i]; break;                        // mass
    case 6: { float4 v = t.vt[i]; out[i] = v.x; out[n + i] = v.y; out[2 * n + i] = v.z; break; }  // v_tmp
    case 7: out[i] = (double)k.rho0 + (double)t.drt[i]; break;  // density_tmp
    case 8: out[i] = t.dd[i]; break;
    case 9: { float4 v = t.dv[i]; out[i] = v.x; out[n + i] = v.y; out[2 * n + i] = v.z; break; }
    case 10: out[i] = t.cf[i]; break;
    case 11: for (int q = 0; q < 9; ++q) out[(size_t)q * n + i] = t.L ? t.L[(size_t)q * n + i] : 0.0; break;
    default: break;
    }
}

__global__ void k_export_int(K32 k, P32 p, int what, int* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const int4 id = p.ids[i];
    switch (what) {
    case 0: out[i] = id.x; break;
    case 1: out[i] = tf_type(p.lo[i].w); break;
    case 2: out[i] = id.y; break;
    case 3: out[i] = id.z; break;
    case 4: out[i] = id.w; break;
    default: break;
    }
}

// Write a field from planar f64 staging (tsg_write).
__global__ void k_import(K32 k, P32 p, int what, const double* in) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const size_t n = k.n;
    switch (what) {
    case 0: {
        float4 h = p.hi[i], l = p.lo[i];
        double x[3] = {in[i] - k.vs[0], in[n + i] - k.vs[1], in[2 * n + i] - k.vs[2]};
        l.x = (float)(x[0] - (double)h.x); l.y = (float)(x[1] - (double)h.y); l.z = (float)(x[2] - (double)h.z);
        p.lo[i] = l;
        break;
    }
    case 1: { float4 v = p.vel[i]; v.x = (float)in[i]; v.y = (float)in[n + i]; v.z = (float)in[2 * n + i]; p.vel[i] = v; break; }
    case 2: if (tf_type(p.lo[i].w) > 0) p.drho[i] = (float)(in[i] - (double)k.rho0); break;
    case 3: p.vel[i].w = (float)in[i]; break;
    default: break;
    }
}

__device__ __forceinline__ void atomic_max_d(double* addr, double v) {
    unsigned long long* a = reinterpret_cast<unsigned long long*>(addr);
    unsigned long long old = *a;
    while (__longlong_as_double(old) < v) {
        unsigned long long prev = atomicCAS(a, old, __double_as_longlong(v));
        if (prev == old) break;
        old = prev;
    }
}

// FP64 conservation diagnostics over flow particles.
__global__ void k_diag32(K32 k, P32 p, double* out) {
    __shared__ double sh[8][TPB / 32];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[8] = {0, 0, 0, 0, 0, 0, 0, -DBL_MAX};
    if (i < k.nd && is_flow(tf_type(p.lo[i].w))) {
        const double m = p.mass[i];
        const float4 vv = p.vel[i];
        const float4 h = p.hi[i], l = p.lo[i];
        const double x = k.vs[0] + ((double)h.x + (double)l.x), y = k.vs[1] + ((double)h.y + (double)l.y),
                     z = k.vs[2] + ((double)h.z + (double)l.z);
        const double v2 = (double)vv.x * vv.x + (double)vv.y * vv.y + (double)vv.z * vv.z;
        v[0] = m; v[1] = m * vv.x; v[2] = m * vv.y; v[3] = m * vv.z; v[4] = 0.5 * m * v2;
        v[5] = -m * ((double)k.g[0] * x + (double)k.g[1] * y + (double)k.g[2] * z);
        v[6] = sqrt(v2); v[7] = x;
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
        atomic_max_d(&out[6], v[6]);
        atomic_max_d(&out[7], v[7]);
    }
}

// Upload: split f64 positions into hi / lo, pack the type word.
__global__ void k_load32(K32 k, const double* __restrict__ x, const double* __restrict__ v,
                         const double* __restrict__ dens, const double* __restrict__ mass,
                         const double* __restrict__ mV, const double* __restrict__ pres,
                         const int* __restrict__ mt, const int* __restrict__ mid, const int* __restrict__ oid,
                         const int* __restrict__ dyn, const int* __restrict__ slot, P32 p) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= k.n) return;
    const int i = slot[s];  // destination index for source particle s
    float hv[3], lv[3];
    for (int d = 0; d < 3; ++d) {
        double xr = x[3 * (size_t)s + d] - k.vs[d];
        double hq = (double)k.Q * rint(xr / (double)k.Q);
        hv[d] = (float)hq;
        lv[d] = (float)(xr - hq);
    }
    // bit 30 keeps the word a normal float, so no denormal flush can touch it in transit
    const int word = 0x40000000 | (mt[s] & 0xffff) | ((dyn[s] & 1) << 16);
    p.hi[i] = make_float4(hv[0], hv[1], hv[2], (float)mV[s]);
    p.lo[i] = make_float4(lv[0], lv[1], lv[2], __int_as_float(word));
    p.vel[i] = make_float4((float)v[3 * (size_t)s], (float)v[3 * (size_t)s + 1], (float)v[3 * (size_t)s + 2], (float)pres[s]);
    p.drho[i] = mt[s] > 0 ? (float)(dens[s] - (double)k.rho0) : 0.f;
    p.mass[i] = (float)mass[s];
    p.ids[i] = make_int4(s, mid[s], oid[s], dyn[s]);
}

__global__ void k_deinterleave32(const double* src, double* dst, int n, int k) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int q = 0; q < k; ++q) dst[(size_t)q * n + i] = src[(size_t)i * k + q];
}

__global__ void k_interleave32(const double* src, double* dst, int n, int k) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int q = 0; q < k; ++q) dst[(size_t)i * k + q] = src[(size_t)q * n + i];
}

// Inspection: enumerate every neighbour directly (independent of the ELL capacity).
template <int DIM>
__global__ void k_nbr_count32(K32 k, const float4* HI, const float4* LO, const float4* PF, const int* ds,
                              const int* ss, int* counts) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    int m = 0;
    enum_neighbors<DIM>(k, i, HI, LO, PF, ds, ss, is_flow(tf_type(PF[i].w)), [&](int, const float*, float) { ++m; });
    counts[i] = m;
}

template <int DIM>
__global__ void k_nbr_fill32(K32 k, const float4* HI, const float4* LO, const float4* PF, const int* ds,
                             const int* ss, const int* off, int* list) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    int m = off[i];
    enum_neighbors<DIM>(k, i, HI, LO, PF, ds, ss, is_flow(tf_type(PF[i].w)),
                        [&](int j, const float*, float) { list[m++] = j; });
}

template <int DIM>
__global__ void k_nbr_count_ell(K32 k, const float4* HI, const float4* LO, const int* cnt, const int* nbr, int* counts) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const int m = cnt[i] < k.maxn ? cnt[i] : k.maxn;
    int c = 0;
    for (int q = 0; q < m; ++q) {
        const int j = nbr[(size_t)q * k.n + i];
        float d[3];
        delta<DIM>(HI[i], LO[i], HI[j], LO[j], d);
        const float r2 = d[0] * d[0] + d[1] * d[1] + (DIM == 3 ? d[2] * d[2] : 0.f);
        if (r2 < k.R2) ++c;
    }
    counts[i] = c;
}

template <int DIM>
__global__ void k_nbr_fill_ell(K32 k, const float4* HI, const float4* LO, const float4* PF, const int* ds,
                               const int* ss, const int* cnt, const int* nbr, const int* off, int* list) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const int m = cnt[i];
    int w = off[i];
    if (m <= k.maxn) {
        for (int q = 0; q < m; ++q) {
            const int j = nbr[(size_t)q * k.n + i];
            float d[3];
            delta<DIM>(HI[i], LO[i], HI[j], LO[j], d);
            const float r2 = d[0] * d[0] + d[1] * d[1] + (DIM == 3 ? d[2] * d[2] : 0.f);
            if (r2 < k.R2) list[w++] = j;
        }
    } else {
        enum_neighbors<DIM>(k, i, HI, LO, PF, ds, ss, is_flow(tf_type(PF[i].w)),
                            [&](int j, const float*, float) { list[w++] = j; });
    }
}

// Largest squared displacement of a real particle since the last list build (pf holds the
// build-time positions); float bits of non-negative values order like unsigned integers.
__global__ void k_disp32(K32 k, const float4* __restrict__ HI, const float4* __restrict__ LO,
                         const float4* __restrict__ PF, unsigned* __restrict__ maxd) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float d2 = 0.f;
    if (i < k.nd) {
        const float4 h = HI[i], l = LO[i], f = PF[i];
        const float dx = (h.x + l.x) - f.x, dy = (h.y + l.y) - f.y, dz = (h.z + l.z) - f.z;
        d2 = dx * dx + dy * dy + dz * dz;
        if (!(d2 == d2)) d2 = 3.0e38f;  // non-finite: force a rebuild (the hash flags it)
    }
    for (int o = 16; o > 0; o >>= 1) d2 = fmaxf(d2, __shfl_down_sync(0xffffffffu, d2, o));
    if ((threadIdx.x & 31) == 0 && d2 > 0.f) atomicMax(maxd, __float_as_uint(d2));
}

}  // namespace

// ====================================================================== host side
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
    unsigned* maxdisp = nullptr;               // squared displacement since the last list build
    bool built = false;
    double* stage = nullptr;       // f64 export staging (9 n)
    double* scratch = nullptr;
    std::vector<void*> allocs;
    std::vector<std::pair<std::string, double*>> views;
    bool lists_valid = false;
};

namespace {

template <class T>
T* dal(Fp32State& st, size_t count) {
    void* q = nullptr;
    if (count == 0) count = 1;
    if (cudaMalloc(&q, count * sizeof(T)) != cudaSuccess) return nullptr;
    cudaMemset(q, 0, count * sizeof(T));
    st.allocs.push_back(q);
    return static_cast<T*>(q);
}

float pow2_quantum(double grid) {
    double q = 1.0;
    while (q > grid) q *= 0.5;
    while (q * 2.0 <= grid) q *= 2.0;
    return (float)q;
}

int ell_capacity(int dim, double R, double spacing) {
    // lattice points inside 1.1 R (plus slack for compression and boundary layers)
    const double rr = 1.1 * R / spacing;
    const int m = (int)std::ceil(rr);
    int count = 0;
    for (int a = -m; a <= m; ++a)
        for (int b = -m; b <= m; ++b)
            for (int c = (dim == 3 ? -m : 0); c <= (dim == 3 ? m : 0); ++c)
                if (a * a + b * b + c * c < rr * rr) ++count;
    return count + 8;
}

void build_cells(Fp32State& st, int base, int count_n, int* count, int* start, cudaStream_t s, bool reorder_into_next) {
    const K32& k = st.k;
    const long long nbins = k.G + 1;
    cudaMemsetAsync(count, 0, sizeof(int) * nbins, s);
    P32& a = st.P[st.cur];
    TSG_LAUNCH(k_hash32, nblk(count_n), TPB, s, k, count_n, base, a.hi, a.lo, st.cell_of, st.rank, count, st.err);
    scan_exclusive(count, start, (int)nbins, st.tiles, s);
    TSG_LAUNCH(k_scatter32, nblk(count_n), TPB, s, count_n, st.cell_of, st.rank, start, st.perm);
    TSG_LAUNCH(k_cell_sort32, nblk(nbins), TPB, s, nbins, start, st.perm);
    P32& b = st.P[1 - st.cur];
    TSG_LAUNCH(k_reorder32, nblk(count_n), TPB, s, k, count_n, base, st.perm, a, b, st.pf);
    (void)reorder_into_next;
}

__global__ void k_offset(int* a, long long m, int off) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) a[i] += off;
}

#define DISPATCH32(k, KERNEL, GRID, ...)                                  \
    do {                                                                  \
        if ((k).dim == 2) TSG_LAUNCH(KERNEL<2>, GRID, TPB, s, __VA_ARGS__); \
        else TSG_LAUNCH(KERNEL<3>, GRID, TPB, s, __VA_ARGS__);            \
    } while (0)

}  // namespace

int fp32_create(const tsg_config& cfg, const Consts& c, const tsg_particles* pp, bool from_device,
                Fp32State** out, cudaStream_t s) {
    *out = nullptr;
    if (c.solver != 1 || c.ti == 4) return TSG_E_UNSUPPORTED;  // WCSPH with SE / LF in this form
    Fp32State* st = new Fp32State();
    st->c = c;
    const int n = c.n;
    st->n = n;
    K32& k = st->k;
    k.n = n;
    k.dim = c.dim; k.kernel = c.kernel; k.corr = c.corr; k.xsph = c.xsph; k.boundary = c.boundary;
    k.solver = c.solver; k.exponent_is_int = c.exponent_is_int; k.gamma_i = (int)c.gamma;
    for (int d = 0; d < 3; ++d) {
        k.gnum[d] = c.gnum[d]; k.vs[d] = c.vs[d]; k.g[d] = (float)c.g[d];
        k.ds[d] = (float)c.ds[d]; k.de[d] = (float)c.de[d];
    }
    k.G = c.G; k.grid = c.grid;
    k.h1 = (float)c.h1;
    k.kk = (float)c.kk;
    k.kk6 = (float)(c.kk / 6.0);
    k.wgrad = (float)(-5.0 * c.kk * c.h1 * c.h1);
    k.cub1 = (float)(c.kk * c.h1);
    k.cub2 = (float)(-0.5 * c.kk * c.h1);
    k.R2 = (float)(c.R * c.R);
    k.R2hi = std::nextafter((float)(c.R * c.R * (1.0 + 1.0 / 1024.0)), 1e30f);
    k.R2lo = (float)(c.R * c.R * (1.0 - 1.0 / 1024.0));
    k.pf_lim = (float)(500.0 * c.R);
    k.visc_fac = (float)c.visc_fac; k.eps_h2 = (float)c.eps_h2; k.rho0 = (float)c.rho0; k.B = (float)c.B;
    k.gamma = (float)c.gamma; k.dt = (float)c.dt; k.hdt = (float)c.hdt;
    k.rep_fac = (float)c.rep_fac; k.diam = (float)c.diam; k.h075 = (float)c.h075; k.r_eps = (float)c.r_eps;
    // Verlet skin: lists hold pairs within R + skin and stay valid while no particle has moved
    // more than skin / 2 since they were built (0.45 skin for margin on f32 positions)
    const double skin = cfg.list_skin > 0 ? cfg.list_skin * c.R : 0.0;
    const double RL = c.R + skin;
    k.R2L = skin > 0 ? (float)(RL * RL) : k.R2;
    k.R2Lhi = skin > 0 ? std::nextafter((float)(RL * RL * (1.0 + 1.0 / 1024.0)), 1e30f) : k.R2hi;
    k.disp2_limit = skin > 0 ? (float)((0.45 * skin) * (0.45 * skin)) : 0.f;
    k.maxn = ell_capacity(c.dim, RL, cfg.particle_diameter);
    // internal cell grid: cells at least R + skin wide so that the 3^dim stencil covers the
    // list radius; it spans the reference's virtual domain (neighbour sets do not depend on it)
    if (RL > c.grid) {
        k.grid = RL;
        long long G = 1;
        for (int d = 0; d < 3; ++d) {
            if (d < c.dim) k.gnum[d] = (int)std::ceil((double)c.gnum[d] * c.grid / RL);
            else k.gnum[d] = c.gnum[d];
            if (d < c.dim) G *= k.gnum[d];
        }
        k.G = G;
    }
    k.Q = pow2_quantum(k.grid);
    k.inv_grid = (float)(1.0 / k.grid);
    // host copies of the classification to place particles: dynamic block first
    std::vector<int32_t> mt(n);
    cudaMemcpy(mt.data(), pp->mat_type, sizeof(int32_t) * n, from_device ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost);
    std::vector<int> slot(n);
    int nd = 0;
    for (int i = 0; i < n; ++i) if (mt[i] > 0) ++nd;
    int a = 0, b = nd;
    for (int i = 0; i < n; ++i) slot[i] = mt[i] > 0 ? a++ : b++;
    st->nd = nd;
    k.nd = nd;
    // allocations
    for (int q = 0; q < 2; ++q) {
        st->P[q].hi = dal<float4>(*st, n); st->P[q].lo = dal<float4>(*st, n); st->P[q].vel = dal<float4>(*st, n);
        st->P[q].drho = dal<float>(*st, n); st->P[q].mass = dal<float>(*st, n); st->P[q].ids = dal<int4>(*st, n);
    }
    T32& t = st->T;
    t.vt = dal<float4>(*st, n); t.pr = dal<float2>(*st, n); t.drt = dal<float>(*st, n); t.dd = dal<float>(*st, n);
    t.dv = dal<float4>(*st, n); t.cf = dal<float>(*st, n); t.xs = dal<float4>(*st, n);
    t.L = c.corr == 1 ? dal<float>(*st, 9 * (size_t)n) : nullptr;
    t.cnt = dal<int>(*st, n);
    t.nbr = dal<int>(*st, (size_t)k.maxn * n);
    st->pf = dal<float4>(*st, n);
    const size_t nb = (size_t)k.G + 1;
    st->dcount = dal<int>(*st, nb); st->dstart = dal<int>(*st, nb + 1);
    st->scount = dal<int>(*st, nb); st->sstart = dal<int>(*st, nb + 1);
    st->cell_of = dal<int>(*st, n); st->rank = dal<int>(*st, n); st->perm = dal<int>(*st, n);
    st->tiles = dal<int>(*st, nb / 2048 + 4); st->err = dal<int>(*st, 1);
    st->cells_d = dal<int>(*st, nb); st->cells_s = dal<int>(*st, nb); st->ncells = dal<int>(*st, 2);
    st->ovf_list = dal<int>(*st, n); st->novf = dal<int>(*st, 1);
    st->maxdisp = dal<unsigned>(*st, 1);
    st->stage = dal<double>(*st, 9 * (size_t)n + 16);
    st->scratch = dal<double>(*st, 64);
    if (!t.nbr || !st->stage) { fp32_destroy(st); return TSG_E_CUDA; }
    // upload raw arrays through the staging buffer, then split on the device
    double* dx = st->stage;                 // 3n
    double* dv = dx + 3 * (size_t)n;        // 3n
    double* d1 = dv + 3 * (size_t)n;        // density
    double* d2 = d1 + n;                    // mass
    double* d3 = d2 + n;                    // m_V
    // pressure reuses P[1].hi as scratch f64 storage (n doubles fit in n float4s)
    double* d4 = reinterpret_cast<double*>(st->P[1].hi);
    cudaMemcpyKind kind = from_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    cudaMemcpyAsync(dx, pp->x, sizeof(double) * 3 * n, kind, s);
    cudaMemcpyAsync(dv, pp->v, sizeof(double) * 3 * n, kind, s);
    cudaMemcpyAsync(d1, pp->density, sizeof(double) * n, kind, s);
    cudaMemcpyAsync(d2, pp->mass, sizeof(double) * n, kind, s);
    cudaMemcpyAsync(d3, pp->m_V, sizeof(double) * n, kind, s);
    cudaMemcpyAsync(d4, pp->pressure, sizeof(double) * n, kind, s);
    int* imt = reinterpret_cast<int*>(st->P[1].lo);
    int* imid = imt + n;
    int* ioid = imid + n;
    int* idyn = reinterpret_cast<int*>(st->P[1].vel);
    int* islot = st->perm;
    cudaMemcpyAsync(imt, pp->mat_type, sizeof(int) * n, kind, s);
    cudaMemcpyAsync(imid, pp->mat_id, sizeof(int) * n, kind, s);
    cudaMemcpyAsync(ioid, pp->obj_id, sizeof(int) * n, kind, s);
    cudaMemcpyAsync(idyn, pp->is_dynamic, sizeof(int) * n, kind, s);
    cudaMemcpyAsync(islot, slot.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
    TSG_LAUNCH(k_load32, nblk(n), TPB, s, k, dx, dv, d1, d2, d3, d4, imt, imid, ioid, idyn, islot, st->P[0]);
    cudaStreamSynchronize(s);
    cudaMemsetAsync(st->P[1].hi, 0, sizeof(float4) * n, s);
    cudaMemsetAsync(st->P[1].lo, 0, sizeof(float4) * n, s);
    cudaMemsetAsync(st->P[1].vel, 0, sizeof(float4) * n, s);
    // static block: sort once into P[1], copy the whole static block into both buffers
    if (n - nd > 0) {
        build_cells(*st, nd, n - nd, st->scount, st->sstart, s, true);
        const long long m = k.G + 2;
        TSG_LAUNCH(k_offset, nblk(m, 256), 256, s, st->sstart, m, nd);
        P32& src = st->P[1];
        P32& dst = st->P[0];
        const size_t off = nd;
        const size_t ns = n - nd;
        cudaMemcpyAsync(dst.hi + off, src.hi + off, sizeof(float4) * ns, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(dst.lo + off, src.lo + off, sizeof(float4) * ns, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(dst.vel + off, src.vel + off, sizeof(float4) * ns, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(dst.drho + off, src.drho + off, sizeof(float) * ns, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(dst.mass + off, src.mass + off, sizeof(float) * ns, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(dst.ids + off, src.ids + off, sizeof(int4) * ns, cudaMemcpyDeviceToDevice, s);
    } else {
        cudaMemsetAsync(st->sstart, 0, sizeof(int) * (k.G + 2), s);
    }
    cudaMemsetAsync(st->ncells + 1, 0, sizeof(int), s);
    TSG_LAUNCH(k_nonempty_cells, nblk(k.G, 256), 256, s, (long long)k.G, st->sstart, st->cells_s, st->ncells + 1);
    // the dynamic block of both buffers must agree before the first sort
    cudaStreamSynchronize(s);
    if (cudaGetLastError() != cudaSuccess) { fp32_destroy(st); return TSG_E_CUDA; }
    *out = st;
    return 0;
}

void fp32_destroy(Fp32State* st) {
    if (!st) return;
    for (void* p : st->allocs) cudaFree(p);
    delete st;
}

void fp32_sort(Fp32State& st, cudaStream_t s) {
    {
        PhaseScope ph(s, PH_SORT);
        if (st.nd > 0) {
            build_cells(st, 0, st.nd, st.dcount, st.dstart, s, true);
            st.cur = 1 - st.cur;
        } else {
            cudaMemsetAsync(st.dstart, 0, sizeof(int) * (st.k.G + 2), s);
        }
    }
    const K32& k = st.k;
    P32& p = st.P[st.cur];
    {
        PhaseScope ph2(s, PH_LISTS);
        cudaMemsetAsync(st.novf, 0, sizeof(int), s);
        if (k.dim == 3) {
            cudaMemsetAsync(st.ncells, 0, sizeof(int), s);
            TSG_LAUNCH(k_nonempty_cells, nblk(k.G, 256), 256, s, (long long)k.G, st.dstart, st.cells_d, st.ncells);
            const int nb = 152 * 16;
            TSG_LAUNCH(k_lists_cell<3>, nb, 128, s, k, 0, st.cells_d, st.ncells, p.hi, p.lo, st.pf, st.dstart,
                       st.sstart, st.T.cnt, st.T.nbr, st.ovf_list, st.novf);
            TSG_LAUNCH(k_lists_cell<3>, nb, 128, s, k, 1, st.cells_s, st.ncells + 1, p.hi, p.lo, st.pf, st.dstart,
                       st.sstart, st.T.cnt, st.T.nbr, st.ovf_list, st.novf);
            // particles in the out-of-grid bins (bounds read on the device)
            TSG_LAUNCH(k_lists_range<3>, 64, TPB, s, k, st.dstart + k.G, p.hi, p.lo, st.pf, st.dstart,
                       st.sstart, st.T.cnt, st.T.nbr, st.ovf_list, st.novf);
            TSG_LAUNCH(k_lists_range<3>, 64, TPB, s, k, st.sstart + k.G, p.hi, p.lo, st.pf, st.dstart,
                       st.sstart, st.T.cnt, st.T.nbr, st.ovf_list, st.novf);
            TSG_LAUNCH(k_lists_fixup<3>, 2 * 152, TPB, s, k, p.hi, p.lo, st.pf, st.dstart, st.sstart, st.T.cnt,
                       st.T.nbr, st.ovf_list, st.novf);
        } else {
            TSG_LAUNCH(k_lists<2>, nblk(k.n), TPB, s, k, p.hi, p.lo, st.pf, st.dstart, st.sstart, st.T.cnt, st.T.nbr,
                       st.ovf_list, st.novf);
        }
    }
    cudaMemsetAsync(st.maxdisp, 0, sizeof(unsigned), s);
    st.lists_valid = true;
    st.built = true;
}

bool fp32_rebuild_due(Fp32State& st, cudaStream_t s) {
    if (!st.built || st.k.disp2_limit <= 0.f) return true;
    const K32& k = st.k;
    P32& p = st.P[st.cur];
    TSG_LAUNCH(k_disp32, nblk(k.nd), TPB, s, k, p.hi, p.lo, st.pf, st.maxdisp);
    unsigned bits = 0;
    cudaMemcpyAsync(&bits, st.maxdisp, sizeof bits, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    float d2;
    std::memcpy(&d2, &bits, sizeof d2);
    return !(d2 <= k.disp2_limit);
}

void fp32_kernel_corr(Fp32State& st, cudaStream_t s) {
    PhaseScope ph(s, PH_CORR);
    const K32& k = st.k;
    const Ovf ovf{st.ovf_list, st.novf};
    if (k.dim == 2) {
        TSG_LAUNCH((k_corr32<2, false>), nblk(k.n), TPB, s, k, st.P[st.cur], st.T, st.pf, st.dstart, st.sstart, ovf);
        TSG_LAUNCH((k_corr32<2, true>), 64, TPB, s, k, st.P[st.cur], st.T, st.pf, st.dstart, st.sstart, ovf);
    } else {
        TSG_LAUNCH((k_corr32<3, false>), nblk(k.n), TPB, s, k, st.P[st.cur], st.T, st.pf, st.dstart, st.sstart, ovf);
        TSG_LAUNCH((k_corr32<3, true>), 64, TPB, s, k, st.P[st.cur], st.T, st.pf, st.dstart, st.sstart, ovf);
    }
}

void fp32_init_tmp(Fp32State& st, cudaStream_t s) {
    PhaseScope ph(s, PH_INIT);
    TSG_LAUNCH(k_init_tmp32, nblk(st.k.n), TPB, s, st.k, st.P[st.cur], st.T);
}

void fp32_one_step(Fp32State& st, cudaStream_t s) {
    const K32& k = st.k;
    P32& p = st.P[st.cur];
    {
        PhaseScope ph(s, PH_PRE);
        TSG_LAUNCH(k_pre32, nblk(k.nd), TPB, s, k, p, st.T);
    }
    {
        PhaseScope ph(s, PH_BDY);
        const Ovf ovf{st.ovf_list, st.novf};
        auto bdy = [&](int base, int count_n) {
            if (count_n <= 0) return;
            if (k.dim == 2) {
                TSG_LAUNCH((k_bdy32<2, false>), nblk(count_n), TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, base, count_n, ovf);
                TSG_LAUNCH((k_bdy32<2, true>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, base, count_n, ovf);
            } else {
                TSG_LAUNCH((k_bdy32<3, false>), nblk(count_n), TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, base, count_n, ovf);
                TSG_LAUNCH((k_bdy32<3, true>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, base, count_n, ovf);
            }
        };
        bdy(k.nd, k.n - k.nd);
        if (st.c.n_bdy > k.n - k.nd) bdy(0, k.nd);  // kinematic rigid particles live in the dynamic block
    }
    {
        PhaseScope ph(s, PH_RATES);
        const Ovf ovf{st.ovf_list, st.novf};
        const int nb = nblk(k.nd);
        if (k.dim == 2) {
            if (k.corr) { TSG_LAUNCH((k_rates32<2, false, true>), nb, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
                          TSG_LAUNCH((k_rates32<2, true, true>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf); }
            else { TSG_LAUNCH((k_rates32<2, false, false>), nb, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
                   TSG_LAUNCH((k_rates32<2, true, false>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf); }
        } else {
            if (k.corr) { TSG_LAUNCH((k_rates32<3, false, true>), nb, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
                          TSG_LAUNCH((k_rates32<3, true, true>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf); }
            else { TSG_LAUNCH((k_rates32<3, false, false>), nb, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
                   TSG_LAUNCH((k_rates32<3, true, false>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf); }
        }
    }
}

void fp32_advect(Fp32State& st, int which, cudaStream_t s) {
    const K32& k = st.k;
    P32& p = st.P[st.cur];
    switch (which) {
    case TSG_ADVECT_FULL: { PhaseScope ph(s, PH_INTEGRATE); TSG_LAUNCH(k_advect_full32, nblk(k.nd), TPB, s, k, p, st.T, st.err); break; }
    case TSG_ADVECT_LF_HALF: { PhaseScope ph(s, PH_INTEGRATE); TSG_LAUNCH(k_advect_half32, nblk(k.nd), TPB, s, k, p, st.T); break; }
    case TSG_ADVECT_POS: {
        PhaseScope ph(s, PH_POS);
        if (k.xsph) {
            const Ovf ovf{st.ovf_list, st.novf};
            if (k.dim == 2) {
                TSG_LAUNCH((k_xsph32<2, false>), nblk(k.nd), TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
                TSG_LAUNCH((k_xsph32<2, true>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
            } else {
                TSG_LAUNCH((k_xsph32<3, false>), nblk(k.nd), TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
                TSG_LAUNCH((k_xsph32<3, true>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
            }
        }
        TSG_LAUNCH(k_advect_pos32, nblk(k.nd), TPB, s, k, p, st.T, st.err);
        if (k.disp2_limit <= 0.f) st.lists_valid = false;
        break;
    }
    case TSG_ADVECT_SOMETHING: { PhaseScope ph(s, PH_POST); TSG_LAUNCH(k_post_wc32, nblk(k.nd), TPB, s, k, p); break; }
    case TSG_ENFORCE_BOUNDARY: { PhaseScope ph(s, PH_OTHER); TSG_LAUNCH(k_enforce32, nblk(k.nd), TPB, s, k, p); break; }
    default: break;
    }
}

void fp32_rk_update(Fp32State&, int, cudaStream_t) {}

int fp32_field(Fp32State& st, const char* name, tsg_view* out, cudaStream_t s) {
    const std::string f(name);
    struct Spec { const char* nm; int what; int comps; int is_int; };
    static const Spec specs[] = {
        {"x", 0, 3, 0}, {"v", 1, 3, 0}, {"density", 2, 1, 0}, {"pressure", 3, 1, 0}, {"m_V", 4, 1, 0},
        {"mass", 5, 1, 0}, {"v_tmp", 6, 3, 0}, {"density_tmp", 7, 1, 0}, {"d_density", 8, 1, 0},
        {"d_vel", 9, 3, 0}, {"CSPM_f", 10, 1, 0}, {"CSPM_L", 11, 9, 0},
        {"id0", 0, 1, 1}, {"mat_type", 1, 1, 1}, {"mat_id", 2, 1, 1}, {"obj_id", 3, 1, 1}, {"is_dynamic", 4, 1, 1}};
    const Spec* sp = nullptr;
    for (const Spec& x : specs) if (f == x.nm) sp = &x;
    if (!sp) return TSG_E_NAME;
    if (sp->what == 11 && !st.T.L) return TSG_E_NAME;
    double* buf = nullptr;
    for (auto& v : st.views) if (v.first == f) buf = v.second;
    if (!buf) {
        buf = dal<double>(st, (size_t)sp->comps * st.n);
        if (!buf) return TSG_E_CUDA;
        st.views.push_back({f, buf});
    }
    if (sp->is_int) TSG_LAUNCH(k_export_int, nblk(st.n), TPB, s, st.k, st.P[st.cur], sp->what, reinterpret_cast<int*>(buf));
    else TSG_LAUNCH(k_export, nblk(st.n), TPB, s, st.k, st.P[st.cur], st.T, sp->what, buf);
    const int64_t n = st.n;
    out->data = buf;
    out->dtype = sp->is_int ? 2 : 0;
    if (sp->comps == 1) { out->ndim = 1; out->shape[0] = n; out->strides[0] = 1; }
    else if (sp->comps == 3) { out->ndim = 2; out->shape[0] = n; out->shape[1] = 3; out->strides[0] = 1; out->strides[1] = n; }
    else { out->ndim = 3; out->shape[0] = n; out->shape[1] = 3; out->shape[2] = 3; out->strides[0] = 1; out->strides[1] = 3 * n; out->strides[2] = n; }
    return cudaGetLastError() == cudaSuccess ? 0 : TSG_E_CUDA;
}

const int* fp32_cell_start(const Fp32State& st) { return st.dstart; }

void fp32_neighbors(Fp32State& st, int* counts, int* offsets, int* list, cudaStream_t s) {
    const K32& k = st.k;
    P32& p = st.P[st.cur];
    if (st.lists_valid) {  // report the lists the physics kernels use
        if (!list) DISPATCH32(k, k_nbr_count_ell, nblk(k.n), k, p.hi, p.lo, st.T.cnt, st.T.nbr, counts);
        else DISPATCH32(k, k_nbr_fill_ell, nblk(k.n), k, p.hi, p.lo, st.pf, st.dstart, st.sstart, st.T.cnt,
                        st.T.nbr, offsets, list);
        return;
    }
    if (!list) DISPATCH32(k, k_nbr_count32, nblk(k.n), k, p.hi, p.lo, st.pf, st.dstart, st.sstart, counts);
    else DISPATCH32(k, k_nbr_fill32, nblk(k.n), k, p.hi, p.lo, st.pf, st.dstart, st.sstart, offsets, list);
}

void fp32_diag(Fp32State& st, double* /*scratch*/, double* host_out8, cudaStream_t s) {
    double init[8] = {0, 0, 0, 0, 0, 0, 0, -DBL_MAX};
    cudaMemcpyAsync(st.scratch, init, sizeof init, cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
    TSG_LAUNCH(k_diag32, nblk(st.n), TPB, s, st.k, st.P[st.cur], st.scratch);
    cudaMemcpyAsync(host_out8, st.scratch, sizeof(double) * 8, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
}

int* fp32_err_ptr(Fp32State& st) { return st.err; }

int fp32_write(Fp32State& st, const char* name, const void* src, bool from_device, cudaStream_t s) {
    const std::string f(name);
    int what = -1, comps = 1;
    if (f == "x") { what = 0; comps = 3; }
    else if (f == "v") { what = 1; comps = 3; }
    else if (f == "density") what = 2;
    else if (f == "pressure") what = 3;
    else return TSG_E_NAME;
    const size_t n = st.n;
    double* buf = st.stage;
    cudaMemcpyAsync(buf + 3 * n, src, sizeof(double) * comps * n, from_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s);
    TSG_LAUNCH(k_deinterleave32, nblk(n), TPB, s, buf + 3 * n, buf, (int)n, comps);
    TSG_LAUNCH(k_import, nblk(n), TPB, s, st.k, st.P[st.cur], what, buf);
    if (what == 0) st.lists_valid = false;
    return cudaGetLastError() == cudaSuccess ? 0 : TSG_E_CUDA;
}

int fp32_read(Fp32State& st, const char* name, void* dst, bool to_device, cudaStream_t s) {
    tsg_view v;
    int rc = fp32_field(st, name, &v, s);
    if (rc) return rc;
    const size_t n = st.n;
    const int comps = v.ndim == 1 ? 1 : (v.ndim == 2 ? 3 : 9);
    const cudaMemcpyKind kind = to_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (comps == 1) {
        cudaMemcpyAsync(dst, v.data, (v.dtype == 2 ? sizeof(int) : sizeof(double)) * n, kind, s);
    } else {
        TSG_LAUNCH(k_interleave32, nblk(n), TPB, s, static_cast<const double*>(v.data), st.stage, (int)n, comps);
        cudaMemcpyAsync(dst, st.stage, sizeof(double) * n * comps, kind, s);
    }
    if (!to_device) cudaStreamSynchronize(s);
    return cudaGetLastError() == cudaSuccess ? 0 : TSG_E_CUDA;
}

}  // namespace tsg
