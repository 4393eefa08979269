// FP32-mixed form of the per-substep SPH path.
//
// Layout (unified particle index space, every array in the current sorted order):
//   [0, nd)  dynamic block: real particles (fluid / soil / kinematic rigid), re-sorted by
//            cell whenever its neighbour lists expire;
//   [nd, n)  static block: dummy and repulsive particles, which never move, sorted by cell
//            once at upload.  Each block has its own cell table (exclusive starts, G + 2).
// Positions are x - vdomain_start = hi + lo with hi an exact multiple of a power-of-two
// quantum Q (about one cell) and lo an f32 remainder, so x_i - x_j = (hi_i - hi_j) +
// (lo_i - lo_j) keeps ~1e-9 m resolution anywhere in the domain.  Density is stored as the
// deviation from the rest density (rho - rho0), which keeps the Tait pressure accurate.
// Arithmetic is f32 except the cell index (f64, truncating cast as the reference,
// eng/particle_system.py:216-218) and the FP64 conservation reductions.
//
// Neighbour lists (Verlet lists of every pair within support + skin): after the sort one
// kernel tests every candidate of the 3^dim stencil and writes an ELL list per particle
// (slot-major, so a warp's reads coalesce) of 4-byte entries that carry the neighbour's
// index, material code and quantised-position offset.  Flow particles list every
// neighbour; boundary and rigid particles list flow neighbours only (all their sums run
// over flow particles).  The lists are rebuilt (with the sort) once a particle has moved
// 0.45 skin since the build; positions stay fixed until advect_pos, so every pass of a
// step reuses one list.  A particle whose count exceeds the capacity is handled by direct
// traversal.  Boundary particles with an empty list are written at the build and skipped
// by the per-step kernels.
//
// Sums over neighbours are block-compensated: plain f32 sums over 16 neighbours, then a
// Kahan update of the running total.  One exception: in a leap-frog WCSPH step with CSPM
// the first rates pass also builds the fluid's CSPM factors, so its continuity sum runs
// as a plain f32 tensor contracted with the inverse matrix after the loop; it sets only
// the half-step density, while the step's density update takes the second pass's
// compensated sum.
//
// Reference: eng/particle_system.py:228-269 (cell list), eng/solver_sph_base.py:41-238,
// :363-423, :648-669 (step, CSPM, boundary), eng/solver_sph_wc.py:82-132 (WCSPH).
#include <type_traits>

#include "tsg_fp32_dev.cuh"
#include "tsg_polar.cuh"
#include "tsg_rigid_list.cuh"
#include "tsg_cellsort.cuh"

namespace tsg {

using namespace f32;

namespace {

// ---------------------------------------------------------------- sort (dynamic block)
__global__ void k_hash32(K32 k, int count_n, int base, const float4* __restrict__ HI, RecView LO,
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
    if (a.sig) {
        const size_t n = k.n;
        for (int q = 0; q < 6; ++q) b.sig[q * n + dst] = a.sig[q * n + src];
        b.eeq[dst] = a.eeq[src];
        b.eeqp[dst] = a.eeqp[src];
        b.flag[dst] = a.flag[src];
    }
    if (a.vlo) b.vlo[dst] = a.vlo[src];
    PF[dst] = make_float4(pfv[0], pfv[1], pfv[2], h.w);
}

// Record a particle whose neighbours exceed the list capacity (processed by FB passes).
__device__ __forceinline__ void note_overflow(int* ovf_list, int* novf, int i) {
    ovf_list[atomicAdd(novf, 1)] = i;
}

// ---------------------------------------------------------------- neighbour lists
template <int DIM>
__global__ void k_lists(K32 k, const float4* __restrict__ HI, RecView LO,
                        const float4* __restrict__ PF, const int* __restrict__ dstart, const int* __restrict__ sstart,
                        int* __restrict__ cnt, int* __restrict__ nbr, int* __restrict__ ovf_list, int* __restrict__ novf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const bool flow_i = is_flow(tf_type(PF[i].w));
    const float4 hi_i = HI[i];
    int m = 0;
    enum_neighbors<DIM>(k, i, HI, LO, PF, dstart, sstart, flow_i, [&](int j, const float*, float) {
        if (m < k.maxn) nbr[(size_t)m * k.n + i] = entry_of(k, j, hi_i, HI[j]);
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
template <int DIM, int WPB>
__global__ void k_lists_cell(K32 k, int self_blk, const int* __restrict__ cells, const int* __restrict__ cell_count,
                             const float4* __restrict__ HI, RecView LO,
                             const float4* __restrict__ PF, const int* __restrict__ dstart,
                             const int* __restrict__ sstart, int* __restrict__ cnt, int* __restrict__ nbr,
                             int* __restrict__ ovf_list, int* __restrict__ novf) {
    __shared__ float4 sh_rel[WPB][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int* own = self_blk == 0 ? dstart : sstart;
    const int ncell = *cell_count;
    const long long ny = k.gnum[1], nz = k.gnum[2], G = k.G;
    for (int w = blockIdx.x * WPB + wib; w < ncell; w += gridDim.x * WPB) {
    const long long c = cells[w];
    const int cb = own[c], ce = own[c + 1];
    const long long cx = c / (ny * nz), cy = (c / nz) % ny, cz = c % nz;
    // reference quantum of this cell: positions are staged as (hi - ref) + lo, exact in hi - ref
    const float4 ref = HI[cb];
    for (int p0 = cb; p0 < ce; p0 += 32) {
        const int i = p0 + lane;
        const bool active = i < ce;
        float rx = 0.f, ry = 0.f, rz = 0.f;
        int qi[3] = {0, 0, 0};  // (hi_i - ref) / Q
        bool flow_i = false, alias = false;
        if (active) {
            const float4 hi_i = HI[i], lo_i = LO[i];
            flow_i = is_flow(tf_type(hi_i.w));
            qi[0] = (int)rintf((hi_i.x - ref.x) * k.inv_Q);
            qi[1] = (int)rintf((hi_i.y - ref.y) * k.inv_Q);
            qi[2] = (int)rintf((hi_i.z - ref.z) * k.inv_Q);
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
                            // w: material class (bits 0-2) and (hj - ref) / Q + 8 per axis (4 bits each)
                            const int qx = (int)rintf((hj.x - ref.x) * k.inv_Q) + 8;
                            const int qy = (int)rintf((hj.y - ref.y) * k.inv_Q) + 8;
                            const int qz = (int)rintf((hj.z - ref.z) * k.inv_Q) + 8;
                            const int tag = type_class(tf_type(hj.w)) | (qx << 3) | (qy << 7) | (qz << 11);
                            sh_rel[wib][lane] = make_float4((hj.x - ref.x) + lj.x, (hj.y - ref.y) + lj.y,
                                                            (hj.z - ref.z) + lj.z, __int_as_float(tag));
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
                                const bool ok_type = flow_i || is_flow(class_type(__float_as_int(q.w) & 7));
                                acc |= (t < mm && r2 < k.R2L && ok_type) ? (1u << t) : 0u;
                            }
                            if (i >= base && i < base + 32) acc &= ~(1u << (i - base));
                            while (acc) {
                                const int t = __ffs(acc) - 1;
                                acc &= acc - 1u;
                                if (m < k.maxn) {
                                    const int tag = __float_as_int(sh_rel[wib][t].w);
                                    *wp = make_entry(base + t, class_type(tag & 7), qi[0] - (((tag >> 3) & 15) - 8),
                                                     qi[1] - (((tag >> 7) & 15) - 8), qi[2] - (((tag >> 11) & 15) - 8));
                                    wp += stride;
                                }
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
__global__ void k_lists_fixup(K32 k, const float4* __restrict__ HI, RecView LO,
                              const float4* __restrict__ PF, const int* __restrict__ dstart,
                              const int* __restrict__ sstart, int* __restrict__ cnt, int* __restrict__ nbr,
                              int* __restrict__ ovf_list, int* __restrict__ novf) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k.n; i += gridDim.x * blockDim.x) {
        if (cnt[i] >= 0) continue;
        const bool flow_i = is_flow(tf_type(PF[i].w));
        const float4 hi_i = HI[i];
        int m = 0;
        enum_neighbors<DIM>(k, i, HI, LO, PF, dstart, sstart, flow_i, [&](int j, const float*, float) {
            if (m < k.maxn) nbr[(size_t)m * k.n + i] = entry_of(k, j, hi_i, HI[j]);
            ++m;
        }, true);
        cnt[i] = m;
        if (m > k.maxn) note_overflow(ovf_list, novf, i);
    }
}

// Per-particle list build for an index range (out-of-grid bin).
template <int DIM>
__global__ void k_lists_range(K32 k, const int* __restrict__ bounds, const float4* __restrict__ HI,
                              RecView LO, const float4* __restrict__ PF,
                              const int* __restrict__ dstart, const int* __restrict__ sstart,
                              int* __restrict__ cnt, int* __restrict__ nbr, int* __restrict__ ovf_list,
                              int* __restrict__ novf) {
    const int b0 = bounds[0], b1 = bounds[1];
    for (int i = b0 + blockIdx.x * blockDim.x + threadIdx.x; i < b1; i += gridDim.x * blockDim.x) {
        const bool flow_i = is_flow(tf_type(PF[i].w));
        const float4 hi_i = HI[i];
        int m = 0;
        enum_neighbors<DIM>(k, i, HI, LO, PF, dstart, sstart, flow_i, [&](int j, const float*, float) {
            if (m < k.maxn) nbr[(size_t)m * k.n + i] = entry_of(k, j, hi_i, HI[j]);
            ++m;
        }, true);
        cnt[i] = m;
        if (m > k.maxn) note_overflow(ovf_list, novf, i);
    }
}

// Inverse of the CSPM matrix (2D: the 2 x 2 block, zero (2, 2) entry; identity when
// |det| <= 1e-8, eng/solver_sph_base.py:400-423), in f32 like the rest of this form.  The
// matrix sum_j m_Vj (-dx_j) (grad W_j)^T is symmetric (grad W is parallel to dx), so it
// and its inverse are held as six planes (xx, yy, zz, xy, xz, yz); m holds them too.
template <int DIM>
__device__ __forceinline__ void inv6(const float* m, bool flow_i, float* inv) {
    inv[0] = inv[1] = inv[2] = 1.f;
    inv[3] = inv[4] = inv[5] = 0.f;
    if (flow_i) {
        const float xx = m[0], yy = m[1], zz = m[2], xy = m[3], xz = m[4], yz = m[5];
        if (DIM == 2) {
            const float dt = xx * yy - xy * xy;
            if (fabsf(dt) > (float)EPS) {
                const float id = 1.f / dt;
                inv[0] = id * yy; inv[1] = id * xx; inv[2] = 0.f; inv[3] = -id * xy;
            }
        } else {
            const float c00 = yy * zz - yz * yz, c11 = xx * zz - xz * xz, c22 = xx * yy - xy * xy;
            const float c01 = xz * yz - xy * zz, c02 = xy * yz - yy * xz, c12 = xy * xz - xx * yz;
            const float dt = xx * c00 + xy * c01 + xz * c02;
            if (fabsf(dt) > (float)EPS) {
                const float id = 1.f / dt;
                inv[0] = id * c00; inv[1] = id * c11; inv[2] = id * c22;
                inv[3] = id * c01; inv[4] = id * c02; inv[5] = id * c12;
            }
        }
    }
}
template <int DIM>
__device__ __forceinline__ void inv_store(const K32& k, float* L, int i, const float* m, bool flow_i) {
    float inv[6];
    inv6<DIM>(m, flow_i, inv);
    for (int q = 0; q < 6; ++q) L[(size_t)q * k.n + i] = inv[q];
}

// The inverse CSPM matrix of particle i as a full 3 x 3 (row-major) from its six planes.
__device__ __forceinline__ void load_L(const float* __restrict__ L6, size_t n, int i, float* L) {
    float l[6];
    for (int q = 0; q < 6; ++q) l[q] = L6[(size_t)q * n + i];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) L[3 * a + b] = l[sym_idx(a, b)];
}

// One neighbour's terms of the CSPM sums, shared by the correction kernel and the fused
// first rates pass so that both give the same bits: the Shepard sum over flow neighbours
// and the six planes of sum_j m_Vj (-dx_j) (G_j m_Vj dx_j)^T over same-type neighbours.
// e = G_j m_Vj dx_j (the corrected kernel gradient's input, e_b = __fmul_rn(G m_V, dx_b)).
template <int DIM>
__device__ __forceinline__ void cspm_terms(CSum& s, float* L, const float* d, const float* e, float w, float mVj,
                                           bool flow_j, bool want_L) {
    if (flow_j) s.p = __fmaf_rn(mVj, w, s.p);
    if (want_L)
        for (int a = 0; a < DIM; ++a)
            for (int b = a; b < DIM; ++b) L[sym_idx(a, b)] = __fmaf_rn(-d[a], e[b], L[sym_idx(a, b)]);
}

// CSPM (eng/solver_sph_base.py:386-423).
template <int DIM, bool FB, int KT>
// Main pass: the dynamic block up to lim, then the static-block particles with a non-empty
// list (act[0 .. *nact), act may be null); the others keep the values written at the list
// build.  The overflow pass takes the overflowed particles below nmax.  skip_fluid: the
// fluid's factors are computed by the first rates pass of the step, so fluid particles are
// passed over.
__global__ void __launch_bounds__(256, 6) k_corr32(K32 k, P32 p, T32 t, const float4* __restrict__ PF, const int* __restrict__ dstart,
                         const int* __restrict__ sstart, const int* __restrict__ act, const int* __restrict__ nact,
                         int lim, int nmax, int skip_fluid, Ovf ovf) {
    FOR_PARTICLES_ACT(FB, 0, lim, act, nact, nmax, ovf, t.cnt, k.maxn, {
        const int ti = tf_type(p.hi[i].w);
        if (!(skip_fluid && ti == MAT_FLUID)) {
            const bool flow_i = is_flow(ti);
            const bool want_L = k.corr == 1 && flow_i;
            CSum s;
            float L[6] = {0, 0, 0, 0, 0, 0};
            const int ci = type_class(ti);
            for_nbrs_g<DIM, FB, true>(k, i, t.cnt, t.nbr, p.hi, p.lo, PF, dstart, sstart, flow_i,
                                      [](int) { return NoPayload{}; },
                                      [&](int, const float* d, float r2, int sidx, int cj, float mVj, NoPayload) {
                const WG wg = w_pair<true, true, KT>(k, r2);
                const float gf = __fmul_rn(wg.g, mVj);
                const float e[3] = {__fmul_rn(gf, d[0]), __fmul_rn(gf, d[1]), __fmul_rn(gf, d[2])};
                cspm_terms<DIM>(s, L, d, e, wg.w, mVj, code_flow(cj), want_L && cj == ci);
                if (sidx % kFlushEvery == kFlushEvery - 1) s.flush();
            });
            const float sum = s.get();
            t.cf[i] = sum != 0.f ? 1.f / sum : 1.f;
            if (k.corr == 1) inv_store<DIM>(k, t.L, i, L, want_L);
        }
    });
}

// Density summation (eng/solver_sph_wc.py:30-31): sum_j mass_j W_ij over every neighbour
// j != i, by direct traversal of the stencil (every centre sees both blocks; a utility pass,
// not part of a step), compensated f32 sums folded every 16 neighbours, written as f64.
template <int DIM>
__global__ void k_density_sum32(K32 k, P32 p, const float4* __restrict__ PF, const int* __restrict__ dstart,
                                const int* __restrict__ sstart, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    CSum sum;
    int m = 0;
    enum_neighbors<DIM>(k, i, p.hi, p.lo, PF, dstart, sstart, true, [&](int j, const float*, float r2) {
        sum.add(p.mass[j] * w_pair<true, false>(k, r2).w);
        if (++m % kFlushEvery == 0) sum.flush();
    }, false, false);
    out[i] = (double)sum.get();
}

__device__ __forceinline__ float tait(const K32& k, float drt, float B);
__device__ __forceinline__ void eos_store(const K32& k, P32& p, T32& t, int i, float w, float drt, float4 v3);

// Real particles all live in the dynamic block (the static block holds fixed boundary
// particles only), so the dynamic block is covered.  EOS: also the fluid's Tait pressure
// from the new density_tmp (the first phase of the WCSPH one_step, fused here by the step
// sequence; the same arithmetic as k_pre32).
template <bool EOS>
__global__ void k_init_tmp32(K32 k, P32 p, T32 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    const float w = p.hi[i].w;
    const int ti = tf_type(w);
    if (ti > 0) {
        const float4 v = p.vel[i];
        const float drt = p.drho[i];
        t.drt[i] = drt;
        if (EOS && ti == MAT_FLUID) eos_store(k, p, t, i, w, drt, v);
        else t.vt[i] = make_float4(v.x, v.y, v.z, t.vt[i].w);
    }
    if (ti == MAT_SOIL && t.sigt) {
        const size_t n = k.n;
        for (int q = 0; q < 6; ++q) t.sigt[q * n + i] = p.sig[q * n + i];
    }
    if (ti > 0 && t.vtlo) t.vtlo[i] = p.vlo[i];
}

// Tait EOS from the density deviation e = (rho_tmp - rho0) / rho0:
// (1 + e)^g - 1 = e * sum_{k<g} (1 + e)^k for an integer exponent (no cancellation).
__device__ __forceinline__ float tait(const K32& k, float drt, float B) {
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
    return fmaxf(B * r, 0.f);
}

// Fluid pressure from density_tmp (WCSPH loop 1, eng/solver_sph_wc.py:86-90): p, p / rho^2
// and (p, rho_tmp); v3 gives the v_tmp components stored beside p / rho^2.
__device__ __forceinline__ void eos_store(const K32& k, P32& p, T32& t, int i, float w, float drt, float4 v3) {
    const float pr = tait(k, drt, k.scene_par ? k.scene_par[tf_scene(w)].x : k.B);
    const float rt = k.rho0 + drt;
    p.vel[i].w = pr;
    t.vt[i] = make_float4(v3.x, v3.y, v3.z, pr / (rt * rt));
    t.pr[i] = make_float2(pr, rt);
}

__global__ void k_pre32(K32 k, P32 p, T32 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    const float w = p.hi[i].w;
    if (tf_type(w) != MAT_FLUID) return;
    eos_store(k, p, t, i, w, t.drt[i], t.vt[i]);
}

// Boundary extrapolation for dummy / repulsive / rigid particles in [base, base + count_n) (WC).
// SH: the particle's Shepard factor is summed in the same loop (its list holds flow
// neighbours only, in the correction kernel's order, so the factor has the same bits) and
// stored, instead of read (the first one_step of a WCSPH step, whose correction kernel
// then skips the static block).
template <int DIM, bool FB, int KT, bool SH = false>
__global__ void k_bdy32(K32 k, P32 p, T32 t, const float4* __restrict__ PF, const int* __restrict__ dstart,
                        const int* __restrict__ sstart, int base, int count_n, const int* __restrict__ act,
                        const int* __restrict__ nact, Ovf ovf) {
    const int lim = base + count_n;
    // with act: the listed particles of [base, lim) (the main pass's direct range is empty)
    FOR_PARTICLES_ACT(FB, base, act ? base : lim, act, nact, lim, ovf, t.cnt, k.maxn, {
        const int ti = tf_type(p.hi[i].w);
        if (ti == MAT_DUMMY || ti == MAT_REP || ti == MAT_RIGID) {
            // plain sums for the extrapolated velocity and pressure (read by this pass only);
            // the Shepard sum keeps the correction kernel's compensated form
            PSum bv[3], bp;
            CSum sh;
            auto term = [&](const float* d, float r2, int sidx, float mV, const float4& vt, const float2& pr) {
                const float w = w_pair<true, false, KT>(k, r2).w;
                const float mw = mV * w;
                if (SH) sh.p = __fmaf_rn(mV, w, sh.p);
                bv[0].add(mw * vt.x);
                bv[1].add(mw * vt.y);
                if (DIM == 3) bv[2].add(mw * vt.z);
                bp.add(mw * (pr.x + pr.y * k.g[1] * d[1]));
                if (sidx % kFlushEvery == kFlushEvery - 1) {
                    bv[0].flush(); bv[1].flush(); bv[2].flush(); bp.flush();
                    if (SH) sh.flush();
                }
            };
            if (!FB) {  // the neighbour's v_tmp comes with its lo record, (p, rho~) beside it
                for_list4<DIM>(k, i, t.cnt, t.nbr, p.lo, t.pr,
                               [&](int, const float* d, float r2, int sidx, float mV, const float4& vt,
                                   const float2& pr) { term(d, r2, sidx, mV, vt, pr); });
            } else {
                for_nbrs<DIM, FB>(k, i, t.cnt, t.nbr, p.hi, p.lo, PF, dstart, sstart, false,
                                  [&](int j, const float* d, float r2, int sidx, int, float mV) {
                    term(d, r2, sidx, mV, t.vt[j], t.pr[j]);
                });
            }
            float f;
            if (SH) {
                const float sum = sh.get();
                f = sum != 0.f ? 1.f / sum : 1.f;
                t.cf[i] = f;
            } else {
                f = t.cf[i];
            }
            const float4 v = p.vel[i];
            const float pv = fmaxf(bp.get() * f, 0.f);
            const float b0 = bv[0].get(), b1 = bv[1].get(), b2 = DIM == 3 ? bv[2].get() : 0.f;
            t.vt[i] = make_float4(2.f * v.x - b0 * f, 2.f * v.y - b1 * f, 2.f * v.z - b2 * f, pv / (k.rho0 * k.rho0));
            t.pr[i] = make_float2(pv, k.rho0);
            t.drt[i] = 0.f;
            p.vel[i].w = pv;
            if (ti == MAT_RIGID) {  // static: rates stay zero; dynamic: gravity, then the reaction
                t.dd[i] = 0.f;
                t.dv[i] = tf_dyn(p.hi[i].w) ? make_float4(k.g[0], k.g[1], k.g[2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
    });
}

// The reaction of the fluid on dynamic rigid particles (eng/solver_sph_wc.py:70-71, where
// every fluid particle subtracts its pair term from its dynamic rigid neighbours without
// synchronisation): each rigid particle gathers, over its list, the momentum pair term its
// fluid neighbours' rates pass evaluates for it (viscosity in the boundary form with the
// fluid particle's rho0 / rho~ factor, plus pressure, on the uncorrected gradient), and
// subtracts it from the gravity its boundary pass set.  Compensated sums.
template <int DIM>
__global__ void k_rigid_reaction32(K32 k, P32 p, T32 t, const float4* __restrict__ PF, const int* __restrict__ dstart,
                                   const int* __restrict__ sstart) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd || t.cnt[i] > k.maxn) return;
    const float wi = p.hi[i].w;
    if (!(tf_type(wi) == MAT_RIGID && tf_dyn(wi))) return;
    const float4 vti = t.vt[i];
    const float mVi = p.lo[i].w;
    CSum acc[3];
    int m = 0;
    for_nbrs_g<DIM, false, true>(k, i, t.cnt, t.nbr, p.hi, p.lo, PF, dstart, sstart, false,
                                 [&](int j) { return t.vt[j]; },
                                 [&](int j, const float* dij, float r2, int, int cj, float, const float4& vtj) {
        if (cj != kCodeFluid) return;
        const float d[3] = {-dij[0], -dij[1], -dij[2]};  // x_fluid - x_rigid
        const WG wg = w_pair<false, true>(k, r2);
        const float mg = __fmul_rn(wg.g, mVi);
        const float dvx = vtj.x - vti.x, dvy = vtj.y - vti.y, dvz = DIM == 3 ? vtj.z - vti.z : 0.f;
        const float vdx = dvx * d[0] + dvy * d[1] + (DIM == 3 ? dvz * d[2] : 0.f);
        const float rtj = k.rho0 + t.drt[j];
        const float vf_b = k.visc_fac * (k.rho0 / rtj);
        const float cv = vf_b * __fdividef(fminf(vdx, 0.f), r2 + k.eps_h2);
        const float sc = mg * (cv + fmaf(-k.rho0, vti.w, -k.rho0 * vtj.w));
        acc[0].add(-sc * d[0]);
        acc[1].add(-sc * d[1]);
        if (DIM == 3) acc[2].add(-sc * d[2]);
        if (++m % kFlushEvery == 0) { acc[0].flush(); acc[1].flush(); acc[2].flush(); }
    });
    float4 dv = t.dv[i];
    dv.x += acc[0].get();
    dv.y += acc[1].get();
    if (DIM == 3) dv.z += acc[2].get();
    t.dv[i] = dv;
}

// Object slot of a dynamic rigid particle (-1 for any other), for the list builder: from
// the type word and object id of the current (sorted) arrays ...
struct RigidSlot32 {
    const float4* hi;
    const int4* ids;
    const int* tab;
    int nobj;
    __device__ int operator()(int i) const {
        const float w = hi[i].w;
        if (tf_type(w) != MAT_RIGID || !tf_dyn(w)) return -1;
        const int id = ids[i].z;
        for (int o = 0; o < nobj; ++o)
            if (tab[o] == id) return o;
        return -1;
    }
};
// ... and from the uploaded arrays (upload order, before the first sort).
struct RigidSlotUpload {
    const int* mt;
    const int* dyn;
    const int* oid;
    const int* tab;
    int nobj;
    __device__ int operator()(int i) const {
        if (mt[i] != MAT_RIGID || !dyn[i]) return -1;
        const int id = oid[i];
        for (int o = 0; o < nobj; ++o)
            if (tab[o] == id) return o;
        return -1;
    }
};

// The rigid-object sums of this form run in f64 over the object's list, spread over the
// GPU: the list is cut into chunks of kRigidChunk entries, one block per (chunk, object);
// each thread sums a fixed strided share of its chunk in list order, a pairwise tree over
// the block's threads (stride halving) gives the chunk's partial sums, and one block per
// object adds the partials in the same way.  The result depends only on the inputs and
// these fixed shapes (deterministic, not the serial order of the FP64 form).
constexpr int kRigidBlock = 256;
constexpr int kRigidChunk = 4 * kRigidBlock;
template <int NV>
__device__ __forceinline__ void block_sum_fixed(const double* v, double (*red)[kRigidBlock]) {
    for (int e = 0; e < NV; ++e) red[e][threadIdx.x] = v[e];
    __syncthreads();
    for (int w = kRigidBlock / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int e = 0; e < NV; ++e) red[e][threadIdx.x] += red[e][threadIdx.x + w];
        __syncthreads();
    }
}

// Shape matching of the dynamic rigid objects (eng/solver_sph_base.py:478-511), over each
// object's list (rebuilt before every shape matching), in three passes:
//   PASS 0: per chunk, sum m x and m (the centre of mass, calc_cm :502-511);
//   PASS 1: per chunk, sum A = sum (m_V rho p) q^T with p = x - cm, q = x0 - rest cm (q kept
//           per id0);
// each followed by k_rigid_reduce32, and then k_rigid_move32 moves every particle to
// cm + R q with R the orthogonal polar factor of A (identity when every entry is below
// 1e-8); its lo record takes the change, hi (a multiple of the list quantum) stays until
// the next list build.
template <int PASS>
__global__ void __launch_bounds__(kRigidBlock) k_rigid_part32(K32 k, P32 p, const int* __restrict__ off,
                                                             const int* __restrict__ lists,
                                                             const double* __restrict__ qtab,
                                                             const double* __restrict__ cm, double* __restrict__ part) {
    __shared__ double red[PASS == 0 ? 4 : 9][kRigidBlock];
    const int o = blockIdx.y, c = blockIdx.x;
    const int m = off[o + 1] - off[o];
    const int q0 = c * kRigidChunk;
    if (q0 >= m) return;  // the whole block: no barrier is left half-reached
    const int* list = lists + off[o];
    const int q1 = min(m, q0 + kRigidChunk);
    double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int q = q0 + threadIdx.x; q < q1; q += kRigidBlock) {
        const int i = list[q];
        const float4 h = p.hi[i], l = p.lo[i];
        const double x[3] = {k.vs[0] + ((double)h.x + (double)l.x), k.vs[1] + ((double)h.y + (double)l.y),
                             k.vs[2] + ((double)h.z + (double)l.z)};
        if (PASS == 0) {
            const double mi = p.mass[i];
            for (int d = 0; d < 3; ++d) v[d] += mi * x[d];
            v[3] += mi;
        } else {
            const double sc = (double)l.w * ((double)k.rho0 + (double)p.drho[i]);
            const double* qq = qtab + 3 * (size_t)p.ids[i].x;
            const double sp[3] = {sc * (x[0] - cm[3 * o]), sc * (x[1] - cm[3 * o + 1]), sc * (x[2] - cm[3 * o + 2])};
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) v[3 * a + b] += sp[a] * qq[b];
        }
    }
    block_sum_fixed<PASS == 0 ? 4 : 9>(v, red);
    if (threadIdx.x == 0)
        for (int e = 0; e < 9; ++e) part[((size_t)o * gridDim.x + c) * 9 + e] = e < (PASS == 0 ? 4 : 9) ? red[e][0] : 0.0;
}

// Orthogonal polar factor for this form's shape matching.  A 2D body (zero third row and
// column) in closed form: for A2 = [[a, b], [c, d]] = U P with det A2 > 0, U is the rotation
// by atan2(c - b, a + d), since tr(U P) = cos(t) tr P and (c - b) = sin(t) tr P for a
// symmetric P; so U = [[a + d, b - c], [c - b, a + d]] / |(a + d, c - b)|, with 1 as the
// third diagonal entry.  Otherwise polar3's scaled Newton iteration with each step's
// divisions taken through one reciprocal (this part's f64 divisions are slow); both agree
// with polar3 to rounding, and this form's sums are not in the oracle's order anyway.
__device__ void polar3_fp32form(const double* A, double* X) {
    const bool flat = A[2] == 0.0 && A[5] == 0.0 && A[6] == 0.0 && A[7] == 0.0 && A[8] == 0.0;
    if (flat) {
        const double det2 = A[0] * A[4] - A[1] * A[3];
        const double u = A[0] + A[4], v = A[3] - A[1];
        const double nrm = sqrt(u * u + v * v);
        if (det2 > 0.0 && nrm > 0.0 && isfinite(nrm)) {
            const double r = 1.0 / nrm;
            X[0] = u * r; X[1] = -v * r; X[2] = 0.0;
            X[3] = v * r; X[4] = u * r;  X[5] = 0.0;
            X[6] = 0.0;   X[7] = 0.0;    X[8] = 1.0;
            return;
        }
    }
    for (int q = 0; q < 9; ++q) X[q] = A[q];
    if (flat) X[8] = 1.0;
    for (int it = 0; it < 60; ++it) {
        double cf[9];
        cf[0] = X[4] * X[8] - X[5] * X[7];
        cf[1] = X[5] * X[6] - X[3] * X[8];
        cf[2] = X[3] * X[7] - X[4] * X[6];
        cf[3] = X[2] * X[7] - X[1] * X[8];
        cf[4] = X[0] * X[8] - X[2] * X[6];
        cf[5] = X[1] * X[6] - X[0] * X[7];
        cf[6] = X[1] * X[5] - X[2] * X[4];
        cf[7] = X[2] * X[3] - X[0] * X[5];
        cf[8] = X[0] * X[4] - X[1] * X[3];
        const double det = (X[0] * cf[0] + X[1] * cf[1]) + X[2] * cf[2];
        if (det == 0.0 || !isfinite(det)) {
            for (int q = 0; q < 9; ++q) X[q] = (q % 4 == 0) ? 1.0 : 0.0;
            return;
        }
        const double rdet = 1.0 / det;
        double fx = 0.0, fy = 0.0, y[9];
        for (int q = 0; q < 9; ++q) {
            y[q] = cf[q] * rdet;
            fx += X[q] * X[q];
            fy += y[q] * y[q];
        }
        const double gm = sqrt(sqrt(fy / fx));
        const double rgm = 1.0 / gm;
        double ch = 0.0;
        for (int q = 0; q < 9; ++q) {
            const double xn = 0.5 * (gm * X[q] + y[q] * rgm);
            const double d = xn - X[q];
            ch += d * d;
            X[q] = xn;
        }
        if (ch <= 1e-28) break;
    }
}

// One block per object: the chunk partials added (strided shares, then the tree); PASS 0
// writes the centre of mass, PASS 1 the rotation.
template <int PASS>
__global__ void __launch_bounds__(kRigidBlock) k_rigid_reduce32(const int* __restrict__ off, int chunks,
                                                               const double* __restrict__ part,
                                                               double* __restrict__ cm, double* __restrict__ rot) {
    __shared__ double red[9][kRigidBlock];
    const int o = blockIdx.x;
    const int nc = (off[o + 1] - off[o] + kRigidChunk - 1) / kRigidChunk;
    double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int c = threadIdx.x; c < nc; c += kRigidBlock)
        for (int e = 0; e < 9; ++e) v[e] += part[((size_t)o * chunks + c) * 9 + e];
    block_sum_fixed<9>(v, red);
    if (threadIdx.x != 0) return;
    if (PASS == 0) {
        for (int d = 0; d < 3; ++d) cm[3 * o + d] = red[d][0] / red[3][0];
    } else {
        double A[9], R[9];
        for (int e = 0; e < 9; ++e) A[e] = red[e][0];
        polar3_fp32form(A, R);
        bool small = true;
        for (int q = 0; q < 9; ++q) small = small && fabs(R[q]) < EPS;
        if (small)
            for (int q = 0; q < 9; ++q) R[q] = (q % 4 == 0) ? 1.0 : 0.0;
        for (int q = 0; q < 9; ++q) rot[9 * o + q] = R[q];
    }
}

__global__ void __launch_bounds__(kRigidBlock) k_rigid_move32(K32 k, P32 p, const int* __restrict__ off,
                                                             const int* __restrict__ lists,
                                                             const double* __restrict__ qtab,
                                                             const double* __restrict__ cm,
                                                             const double* __restrict__ rot) {
    const int o = blockIdx.y;
    const int m = off[o + 1] - off[o];
    const int q0 = blockIdx.x * kRigidChunk;
    const int q1 = min(m, q0 + kRigidChunk);
    const double* R = rot + 9 * o;
    const double* c = cm + 3 * o;
    for (int q = q0 + threadIdx.x; q < q1; q += kRigidBlock) {
        const int i = lists[off[o] + q];
        const double* qq = qtab + 3 * (size_t)p.ids[i].x;
        const float4 h = p.hi[i];
        float4 l = p.lo[i];
        const double g0 = c[0] + ((R[0] * qq[0] + R[1] * qq[1]) + R[2] * qq[2]);
        const double g1 = c[1] + ((R[3] * qq[0] + R[4] * qq[1]) + R[5] * qq[2]);
        const double g2 = c[2] + ((R[6] * qq[0] + R[7] * qq[1]) + R[8] * qq[2]);
        l.x = (float)((g0 - k.vs[0]) - (double)h.x);
        l.y = (float)((g1 - k.vs[1]) - (double)h.y);
        if (k.dim == 3) l.z = (float)((g2 - k.vs[2]) - (double)h.z);
        p.lo[i] = l;
    }
}

// init_rigid_body (eng/solver_sph_base.py:467-470) from the uploaded f64 positions, over the
// object's list in upload order, one block per object (once, at upload): the rest centre of
// mass (strided shares and the tree of block_sum_fixed), then every dynamic rigid particle's
// rest offset x0 - rest cm stored at its upload index (its id0).
__global__ void __launch_bounds__(kRigidBlock) k_rigid_rest32(const int* __restrict__ off,
                                                             const int* __restrict__ lists,
                                                             const double* __restrict__ x,
                                                             const double* __restrict__ mass, double* __restrict__ q) {
    __shared__ double red[4][kRigidBlock];
    __shared__ double cm_s[3];
    const int o = blockIdx.x;
    const int* list = lists + off[o];
    const int m = off[o + 1] - off[o];
    double v[4] = {0, 0, 0, 0};
    for (int k = threadIdx.x; k < m; k += kRigidBlock) {
        const int i = list[k];
        for (int d = 0; d < 3; ++d) v[d] += mass[i] * x[3 * (size_t)i + d];
        v[3] += mass[i];
    }
    block_sum_fixed<4>(v, red);
    if (threadIdx.x == 0)
        for (int d = 0; d < 3; ++d) cm_s[d] = red[d][0] / red[3][0];
    __syncthreads();
    for (int k = threadIdx.x; k < m; k += kRigidBlock) {
        const int i = list[k];
        for (int d = 0; d < 3; ++d) q[3 * (size_t)i + d] = x[3 * (size_t)i + d] - cm_s[d];
    }
}

// WCSPH continuity + momentum (eng/solver_sph_wc.py:108-126).
// KT: kernel function (w_pair); REP: repulsive boundary forces on (1), off (0) or chosen at
// run time from k.boundary (-1).
// FL: the fluid's CSPM factors (the Shepard factor; with CORR the CSPM matrix too) are
// computed here, in the same neighbour loop, instead of by the correction kernel (the
// first rates pass of the step: the particles do not move between the correction and the
// second pass, which reads them back).  With CORR the continuity sum of both passes runs
// on the symmetric part of sum_j m_Vj G_j (v_i - v_j) dx_j^T, contracted after the loop
// with the inverse CSPM matrix (built by the same loop in the first pass, read back in the
// second): (L (v_i - v_j)) . dx = sum_ab L_ab dv_b dx_a and L is symmetric, so a neighbour
// costs six multiply-adds into the tensor instead of L applied to its velocity difference.
template <int DIM, bool FB, bool CORR, int KT, int REP, bool FL = false>
__global__ void __launch_bounds__(256, 4) k_rates32(K32 k, P32 p, T32 t, const float4* __restrict__ PF, const int* __restrict__ dstart,
                          const int* __restrict__ sstart, Ovf ovf) {
    constexpr bool FLC = FL && CORR;  // the CSPM matrix is built in this pass
    // with CORR both passes sum the continuity tensor and contract it with L after the loop
    constexpr bool TEN = CORR;
    FOR_PARTICLES(FB, 0, k.nd, ovf, t.cnt, k.maxn, {
      const float wi = p.hi[i].w;
      if (tf_type(wi) == MAT_FLUID) {
        const float visc_fac = k.scene_par ? k.scene_par[tf_scene(wi)].y : k.visc_fac;
        const float4 vti = t.vt[i];
        const float rti = k.rho0 + t.drt[i];
        const float visc_b = k.rho0 / rti;
        float L[9];
        if (CORR && !TEN)
            load_L(t.L, k.n, i, L);
        // the first pass of a leap-frog step with CSPM sets only the half step's velocity
        // from its accelerations: plain sums there (the step's update takes the second's)
        CSum dd;
        typename std::conditional<FLC, PSum, CSum>::type dv[3];
        CSum sh;                                 // FL: Shepard sum
        float A[6] = {0, 0, 0, 0, 0, 0};         // TEN: continuity tensor (symmetric part)
        float M[6] = {0, 0, 0, 0, 0, 0};         // FLC: CSPM matrix
        const bool rep_on = REP < 0 ? (k.boundary == 3 || k.boundary == 4) : REP == 1;
        // viscosity factor for fluid and for boundary neighbours; -rho0 p_i / rho_i^2
        const float vf_f = visc_fac, vf_b = visc_fac * visc_b;
        const float pi_n = -k.rho0 * vti.w;
        for_nbrs_g<DIM, FB, true, true>(k, i, t.cnt, t.nbr, p.hi, p.lo, PF, dstart, sstart, true,
                                        [&](int j) { return t.vt[j]; },
                                  [&](int, const float* d, float r2, int sidx, int cj, float mVj, const float4& vtj) {
            const WG wg = w_pair<FL, true, KT>(k, r2);
            const float r = wg.r;
            const float mg = __fmul_rn(wg.g, mVj);   // m_Vj G, grad W = G d
            const float dvx = vti.x - vtj.x, dvy = vti.y - vtj.y, dvz = DIM == 3 ? vti.z - vtj.z : 0.f;
            const float vdx = dvx * d[0] + dvy * d[1] + (DIM == 3 ? dvz * d[2] : 0.f);
            const float e[3] = {__fmul_rn(mg, d[0]), __fmul_rn(mg, d[1]), __fmul_rn(mg, d[2])};
            // WCSPH scenes hold no soil: the flow neighbours are the fluid ones
            if (FL) cspm_terms<DIM>(sh, M, d, e, wg.w, mVj, cj == kCodeFluid, CORR && cj == kCodeFluid);
            if (TEN) {
                const float dvv[3] = {dvx, dvy, dvz};
                for (int a = 0; a < DIM; ++a) {
                    A[a] = fmaf(dvv[a], e[a], A[a]);
                    for (int b = a + 1; b < DIM; ++b) A[sym_idx(a, b)] = fmaf(dvv[a], e[b], fmaf(dvv[b], e[a], A[sym_idx(a, b)]));
                }
            } else {
                // continuity: m_Vj (v_i - v_j) . (L_i grad W) = m_Vj G (L_i (v_i - v_j)) . d (L_i symmetric)
                float cdx = vdx;
                if (CORR) {
                    const float ux = L[0] * dvx + L[1] * dvy + (DIM == 3 ? L[2] * dvz : 0.f);
                    const float uy = L[3] * dvx + L[4] * dvy + (DIM == 3 ? L[5] * dvz : 0.f);
                    const float uz = DIM == 3 ? L[6] * dvx + L[7] * dvy + L[8] * dvz : 0.f;
                    cdx = ux * d[0] + uy * d[1] + (DIM == 3 ? uz * d[2] : 0.f);
                }
                dd.add(mg * cdx);
            }
            // viscosity (fluid or boundary neighbours) and pressure, on the uncorrected gradient.
            // WCSPH scenes hold fluid, dummy, repulsive and rigid particles only (soil is rejected
            // at upload), so every non-fluid neighbour takes the boundary form
            const float cv = (cj == kCodeFluid ? vf_f : vf_b) * __fdividef(fminf(vdx, 0.f), r2 + k.eps_h2);
            float sc = mg * (cv + fmaf(-k.rho0, vtj.w, pi_n));
            float rs = 0.f;
            if (rep_on && cj == kCodeRep) {  // repulsive force (eng/solver_sph_base.py:675-689)
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
            if (sidx % kFlushEvery == kFlushEvery - 1) {
                if (FL) sh.flush();
                if (!TEN) dd.flush();
                dv[0].flush(); dv[1].flush(); dv[2].flush();
            }
        });
        if (FL) {
            const float sum = sh.get();
            t.cf[i] = sum != 0.f ? 1.f / sum : 1.f;
        }
        float ddi;
        if (FLC) {
            float inv[6];
            inv6<DIM>(M, true, inv);
            for (int q = 0; q < 6; ++q) t.L[(size_t)q * k.n + i] = inv[q];
            ddi = 0.f;
            for (int a = 0; a < DIM; ++a)
                for (int b = a; b < DIM; ++b) ddi = fmaf(inv[sym_idx(a, b)], A[sym_idx(a, b)], ddi);
        } else if (TEN) {
            ddi = 0.f;
            for (int a = 0; a < DIM; ++a)
                for (int b = a; b < DIM; ++b)
                    ddi = fmaf(t.L[(size_t)sym_idx(a, b) * k.n + i], A[sym_idx(a, b)], ddi);
        } else {
            ddi = dd.get();
        }
        t.dd[i] = ddi * rti;
        t.dv[i] = make_float4(dv[0].get() + k.g[0], dv[1].get() + k.g[1],
                              (DIM == 3 ? dv[2].get() : 0.f) + k.g[2], 0.f);
      }
    });
}

// Drucker-Prager first phase of one_step: adapt stress_tmp (eng/solver_sph_dp.py:215-217).
__global__ void k_pre_dp32(K32 k, P32 p, T32 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    if (tf_type(p.hi[i].w) != MAT_SOIL) return;
    float st[6];
    load_sym(t.sigt, k.n, i, st);
    dp_adapt32(k, st);
    store_sym(t.sigt, k.n, i, st);
}

// mu(I) loop 1 (eng/solver_sph_muI.py:67-92): velocity gradient, continuity, pressure from
// density (not density_tmp), mu(I) stress, equivalent strain rate.
template <int DIM, bool FB, bool CORR>
__global__ void k_mui_stress32(K32 k, P32 p, T32 t, const float4* __restrict__ PF, const int* __restrict__ dstart,
                               const int* __restrict__ sstart, Ovf ovf) {
    FOR_PARTICLES(FB, 0, k.nd, ovf, t.cnt, k.maxn, {
      if (tf_type(p.hi[i].w) == MAT_SOIL) {
        const float4 vti = t.vt[i], vli = t.vtlo[i];
        float L[9];
        if (CORR)
            load_L(t.L, k.n, i, L);
        float vg[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        CSum dd;
        for_nbrs<DIM, FB>(k, i, t.cnt, t.nbr, p.hi, p.lo, PF, dstart, sstart, true,
                          [&](int j, const float* d, float r2, int sidx, int, float mVj) {
            float kc[3];
            grad_c<DIM, CORR>(L, w_grad(k, fast_sqrt(r2)), d, kc);
            vgrad_add<DIM>(mVj, vti, vli, t.vt[j], t.vtlo[j], kc, vg, dd);
            if (sidx % kFlushEvery == kFlushEvery - 1) dd.flush();
        });
        const size_t n = k.n;
        t.dd[i] = dd.get() * (k.rho0 + t.drt[i]);
        const float pr = fmaxf(k.c2 * p.drho[i], 0.f);
        p.vel[i].w = pr;
        float er[6];
        strain_rate(vg, er);
        const float dbdot = sqrtf(0.5f * sym_dd(er, er)) + (float)EPS;
        const float sc = (k.coh + pr * k.mu) / dbdot;
        for (int q = 0; q < 6; ++q) t.sigt[q * n + i] = sc * er[q] - (q < 3 ? pr : 0.f);
        t.dee[i] = equiv_rate(er);
      }
    });
}

// Boundary extrapolation for the granular solvers (eng/solver_sph_muI.py:97-109,
// eng/solver_sph_dp.py:219-234): velocity, density (mu(I)) and stress with the
// hydrostatic correction rho_j g_a (x_i - x_j)_a on the diagonal.
template <int DIM, bool FB>
__global__ void k_bdy_soil32(K32 k, P32 p, T32 t, const float4* __restrict__ PF, const int* __restrict__ dstart,
                             const int* __restrict__ sstart, int base, int count_n, Ovf ovf) {
    const int lim = base + count_n;
    FOR_PARTICLES(FB, base, lim, ovf, t.cnt, k.maxn, {
        const int ti = tf_type(p.hi[i].w);
        if (ti == MAT_DUMMY || ti == MAT_REP || ti == MAT_RIGID) {
            const size_t n = k.n;
            CSum bv[3], b1, b2;
            float bs[6] = {0, 0, 0, 0, 0, 0};
            for_nbrs<DIM, FB>(k, i, t.cnt, t.nbr, p.hi, p.lo, PF, dstart, sstart, false,
                              [&](int j, const float* d, float r2, int sidx, int, float mVj) {
                const float mw = mVj * w_val(k, fast_sqrt(r2));
                const float4 vt = t.vt[j];
                const float drt = t.drt[j];
                const float rtj = k.rho0 + drt;
                bv[0].add(mw * vt.x);
                bv[1].add(mw * vt.y);
                if (DIM == 3) bv[2].add(mw * vt.z);
                if (k.solver == 2) { b1.add(mw); b2.add(mw * drt); }
                bs[0] += mw * (t.sigt[j] + rtj * k.g[0] * d[0]);
                bs[1] += mw * (t.sigt[n + j] + rtj * k.g[1] * d[1]);
                bs[2] += mw * (t.sigt[2 * n + j] + (DIM == 3 ? rtj * k.g[2] * d[2] : 0.f));
                bs[3] += mw * t.sigt[3 * n + j];
                if (DIM == 3) { bs[4] += mw * t.sigt[4 * n + j]; bs[5] += mw * t.sigt[5 * n + j]; }
                if (sidx % kFlushEvery == kFlushEvery - 1) { bv[0].flush(); bv[1].flush(); bv[2].flush(); b1.flush(); b2.flush(); }
            });
            const float f = t.cf[i];
            const float4 v = p.vel[i];
            const float b0 = bv[0].get(), b1v = bv[1].get(), b2v = DIM == 3 ? bv[2].get() : 0.f;
            t.vt[i] = make_float4(2.f * v.x - b0 * f, 2.f * v.y - b1v * f, 2.f * v.z - b2v * f, 0.f);
            // max(f sum m_V rho_tmp W, rho0) - rho0, with rho_tmp = rho0 + drt split off exactly
            t.drt[i] = k.solver == 2 ? fmaxf(k.rho0 * (f * b1.get() - 1.f) + f * b2.get(), 0.f) : 0.f;
            for (int q = 0; q < 6; ++q) t.sigt[q * n + i] = bs[q] * f;
            if (ti == MAT_RIGID) { t.dd[i] = 0.f; t.dv[i] = make_float4(0.f, 0.f, 0.f, 0.f); }
        }
    });
}

// The stress and rho_tmp - rho0 of every particle packed for the stress-divergence pass's
// neighbour reads: one 128-bit read per neighbour in 2D, (s_xx, s_yy, s_xy, rho~ - rho0), and
// one 256-bit read in 3D, (s_xx, s_yy, s_zz, rho~ - rho0), (s_xy, s_xz, s_yz, 0), in place
// of four / seven 32-bit reads from the planes.  Run right before that pass (after the
// boundary extrapolation has written the dummies' values).
template <int DIM>
__global__ void k_pack_stress32(K32 k, T32 t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const size_t n = k.n;
    if (DIM == 2) {
        t.srec[i] = make_float4(t.sigt[i], t.sigt[n + i], t.sigt[3 * n + i], t.drt[i]);
    } else {
        t.srec[2 * (size_t)i] = make_float4(t.sigt[i], t.sigt[n + i], t.sigt[2 * n + i], t.drt[i]);
        t.srec[2 * (size_t)i + 1] = make_float4(t.sigt[3 * n + i], t.sigt[4 * n + i], t.sigt[5 * n + i], 0.f);
    }
}

// Stress divergence + damping (mu(I), eng/solver_sph_muI.py:113-128), and for DP also the
// velocity gradient, continuity and Bui-2008 stress rate (eng/solver_sph_dp.py:172-208,
// :236-270), all in one traversal.
template <int DIM, bool FB, bool CORR, bool DP>
__global__ void k_soil_mom32(K32 k, P32 p, T32 t, const float4* __restrict__ PF, const int* __restrict__ dstart,
                             const int* __restrict__ sstart, Ovf ovf) {
    FOR_PARTICLES(FB, 0, k.nd, ovf, t.cnt, k.maxn, {
      if (tf_type(p.hi[i].w) == MAT_SOIL) {
        const size_t n = k.n;
        const float4 vti = t.vt[i], vli = t.vtlo[i];
        float L[9];
        if (CORR)
            load_L(t.L, n, i, L);
        float sti[6];
        load_sym(t.sigt, n, i, sti);
        const float rti = k.rho0 + t.drt[i];
        const float ir2 = 1.f / (rti * rti);
        float ai[6];
        for (int q = 0; q < 6; ++q) ai[q] = sti[q] * ir2;
        CSum dv[3], dd;
        float vg[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        const bool rep_on = k.boundary == 3 || k.boundary == 4;
        for_nbrs<DIM, FB>(k, i, t.cnt, t.nbr, p.hi, p.lo, PF, dstart, sstart, true,
                          [&](int j, const float* d, float r2, int sidx, int tj, float mVj) {
            // the neighbour's stress and rho_tmp - rho0 in one packed read
            float4 sa, sb = make_float4(0.f, 0.f, 0.f, 0.f);
            if (DIM == 2) sa = t.srec[j];
            else ldg_rec(t.srec, j, sa, sb);
            const float rtj = k.rho0 + sa.w;
            const float r = fast_sqrt(r2);
            float kc[3];
            grad_c<DIM, CORR>(L, w_grad(k, r), d, kc);
            const float irj = __fdividef(1.f, rtj * rtj);
            const float coef = mVj * rtj;
            // m_ab = sigma_j / rho_j^2 + sigma_i / rho_i^2
            const float mxx = sa.x * irj + ai[0];
            const float myy = sa.y * irj + ai[1];
            const float mxy = (DIM == 2 ? sa.z : sb.x) * irj + ai[3];
            if (DIM == 3) {
                const float mzz = sa.z * irj + ai[2];
                const float mxz = sb.y * irj + ai[4];
                const float myz = sb.z * irj + ai[5];
                dv[0].add(coef * (mxx * kc[0] + mxy * kc[1] + mxz * kc[2]));
                dv[1].add(coef * (mxy * kc[0] + myy * kc[1] + myz * kc[2]));
                dv[2].add(coef * (mxz * kc[0] + myz * kc[1] + mzz * kc[2]));
            } else {
                dv[0].add(coef * (mxx * kc[0] + mxy * kc[1]));
                dv[1].add(coef * (mxy * kc[0] + myy * kc[1]));
            }
            if (DP) vgrad_add<DIM>(mVj, vti, vli, t.vt[j], t.vtlo[j], kc, vg, dd);
            if (rep_on && tj == MAT_REP) {  // eng/solver_sph_base.py:675-689
                const float chi = (r > 0.f && r < k.diam) ? 1.f - r / k.diam : 0.f;
                const float gm = r / k.h075;
                float fr = 0.f;
                if (gm > 0.f && gm <= 2.f / 3.f) fr = 2.f / 3.f;
                else if (gm > 2.f / 3.f && gm <= 1.f) fr = 2.f * gm - 1.5f * gm * gm;
                else if (gm > 1.f && gm < 2.f) fr = 0.5f * (2.f - gm) * (2.f - gm);
                const float rs = k.rep_fac * chi * fr / r2;
                dv[0].add(rs * d[0]);
                dv[1].add(rs * d[1]);
                if (DIM == 3) dv[2].add(rs * d[2]);
            }
            if (sidx % kFlushEvery == kFlushEvery - 1) { dv[0].flush(); dv[1].flush(); dv[2].flush(); dd.flush(); }
        });
        const float damp = -k.damp_eps * sqrtf(k.damp_E / (rti * k.h2));
        t.dv[i] = make_float4(dv[0].get() + k.g[0] + damp * vti.x, dv[1].get() + k.g[1] + damp * vti.y,
                              (DIM == 3 ? dv[2].get() : 0.f) + k.g[2] + damp * vti.z, 0.f);
        if (DP) {
            t.dd[i] = dd.get() * rti;
            float s[6], I1, sJ2, f_old;
            dp_inv32(k, sti, s, I1, sJ2, f_old);
            float er[6];
            strain_rate(vg, er);
            const float w01 = 0.5f * (vg[1] - vg[3]), w02 = 0.5f * (vg[2] - vg[6]), w12 = 0.5f * (vg[5] - vg[7]);
            const float W[9] = {0.f, w01, w02, -w01, 0.f, w12, -w02, -w12, 0.f};
            float S[9];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) S[3 * a + b] = sti[sym_idx(a, b)];
            const float tr = (er[0] + er[1]) + er[2];
            const bool plastic = f_old >= -(float)EPS_F && sJ2 > (float)EPS;
            const float lam = plastic ? (k.three_aK * tr + (k.Gm / sJ2) * sym_dd(s, er)) / k.lam_den : 0.f;
            float ds[6];
            for (int q = 0; q < 6; ++q) {
                const int a = q < 3 ? q : (q == 5 ? 1 : 0);
                const int b = q < 3 ? q : (q == 3 ? 1 : 2);
                // Jaumann term J_ab = sum_k sigma_ak w_bk + sigma_kb w_ak
                const float J = S[3 * a] * W[3 * b] + S[3 * a + 1] * W[3 * b + 1] + S[3 * a + 2] * W[3 * b + 2] +
                                S[b] * W[3 * a] + S[3 + b] * W[3 * a + 1] + S[6 + b] * W[3 * a + 2];
                const float ed = er[q] - (q < 3 ? tr / 3.f : 0.f);
                const float te = k.twoG * ed + (q < 3 ? k.Km * tr : 0.f);
                const float tg = plastic ? lam * ((q < 3 ? k.nine_K_sin : 0.f) + k.Gm / sJ2 * s[q]) : 0.f;
                ds[q] = (J + te) - tg;
            }
            store_sym(t.dsig, n, i, ds);
            t.dee[i] = equiv_rate(er);
            float dep = 0.f;
            if (plastic) {
                // g_p is never written by the reference (eng/particle_func.py:52), so g_p - 0
                const float gd = sJ2 + 3.f * I1 * k.sin_dila;
                float ep[6];
                for (int q = 0; q < 6; ++q) ep[q] = lam * (fabsf(ds[q]) > (float)EPS ? gd / ds[q] : 0.f);
                dep = equiv_rate(ep);
            }
            t.deep[i] = dep;
        }
      }
    });
}

// mu(I) post-step, part 1 (eng/solver_sph_muI.py:134-149): density clamp, volume, equivalent
// strain.  stress <- stress_tmp is folded into the regularisation below.
__global__ void k_post_mui32(K32 k, P32 p, T32 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    if (tf_type(p.hi[i].w) != MAT_SOIL) return;
    const float dr = fmaxf(p.drho[i], 0.f);
    p.drho[i] = dr;
    p.lo[i].w = p.mass[i] / (k.rho0 + dr);
    p.eeq[i] += k.dt * t.dee[i];
}

// mu(I) stress regularisation (eng/solver_sph_muI.py:151-156): stress_i = CSPM_f_i
// sum_{soil j} m_Vj stress_tmp_j W_ij at the moved positions.  Both phases of the reference's
// racy in-place update are separated: every read is of stress_tmp.  The neighbours come
// from i's list while the lists still hold every pair within the support at the moved
// positions - no particle has moved more than 0.49 skin since the build (*maxd, measured
// from the moved positions just before this pass, against list_d2 > 0; a pair within R now
// was then within R + 0.98 skin at the build) and i's list did not overflow - and
// otherwise by direct enumeration over the cell table of the last sort (prefilter off: its
// positions predate the move).  The list builder enumerates the same stencil in the same
// order and the list offsets give the same displacement bits, so both visit the soil
// neighbours within the support in the same order and give the same sums (for particles
// that have not changed cell since the sort; otherwise the order, not the set, differs).
template <int DIM>
__global__ void k_reg_mui32(K32 k, P32 p, T32 t, const float4* __restrict__ PF, const int* __restrict__ dstart,
                            const int* __restrict__ sstart, const unsigned* __restrict__ maxd, float list_d2) {
    const bool lists_ok = list_d2 > 0.f && __uint_as_float(*maxd) <= list_d2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k.nd; i += gridDim.x * blockDim.x) {
        if (tf_type(p.hi[i].w) != MAT_SOIL) continue;
        const size_t n = k.n;
        float s[6] = {0, 0, 0, 0, 0, 0};
        const int m = t.cnt[i];
        if (lists_ok && m <= k.maxn) {
            const float4 lo_i = p.lo[i];
            for (int q = 0; q < m; ++q) {
                const int e = t.nbr[(size_t)q * n + i];
                if (class_type((e >> kEntryBits) & 7) != MAT_SOIL) continue;
                const int j = e & kEntryMask;
                const float4 l = p.lo[j];
                float d[3];
                const float r2 = list_delta<DIM>(k, e, lo_i, l, d);
                if (!(r2 < k.R2)) continue;
                const float mw = l.w * w_val(k, fast_sqrt(r2));
                for (int c = 0; c < 6; ++c) s[c] += mw * t.sigt[c * n + j];
            }
        } else {
            enum_neighbors<DIM>(k, i, p.hi, p.lo, PF, dstart, sstart, false, [&](int j, const float*, float r2) {
                if (tf_type(p.hi[j].w) != MAT_SOIL) return;
                const float mw = p.lo[j].w * w_val(k, fast_sqrt(r2));
                for (int c = 0; c < 6; ++c) s[c] += mw * t.sigt[c * n + j];
            }, false, false);
        }
        const float f = t.cf[i];
        for (int c = 0; c < 6; ++c) p.sig[c * n + i] = s[c] * f;
    }
}

// Drucker-Prager post-step (eng/solver_sph_dp.py:277-296).
__global__ void k_post_dp32(K32 k, P32 p, T32 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    if (tf_type(p.hi[i].w) != MAT_SOIL) return;
    const float dr = fmaxf(p.drho[i], 0.f);
    p.drho[i] = dr;
    p.lo[i].w = p.mass[i] / (k.rho0 + dr);
    float st[6];
    load_sym(p.sig, k.n, i, st);
    p.flag[i] = dp_flag32(k, st);
    dp_adapt32(k, st);
    store_sym(p.sig, k.n, i, st);
    p.eeq[i] += k.dt * t.dee[i];
    p.eeqp[i] += k.dt * t.deep[i];
}

// Geostatic initial stress (eng/solver_sph_base.py:249-260): sigma_yy = rho0 g_y (y_max - y),
// sigma_xx = sigma_zz = K0 sigma_yy, from the highest soil particle.
__global__ void k_ymax32(K32 k, P32 p, double* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double y = -DBL_MAX;
    if (i < k.nd && tf_type(p.hi[i].w) == MAT_SOIL) y = k.vs[1] + ((double)p.hi[i].y + (double)p.lo[i].y);
    for (int o = 16; o > 0; o >>= 1) y = fmax(y, __shfl_down_sync(0xffffffffu, y, o));
    if ((threadIdx.x & 31) == 0) atomic_max_d(out, y);
}
__global__ void k_geostatic32(K32 k, P32 p, const double* ymax, double K0) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    if (tf_type(p.hi[i].w) != MAT_SOIL) return;
    const double y = k.vs[1] + ((double)p.hi[i].y + (double)p.lo[i].y);
    const double vs = (double)k.rho0 * (double)k.g[1] * (ymax[0] - y);
    const size_t n = k.n;
    p.sig[i] = (float)(K0 * vs);
    p.sig[n + i] = (float)vs;
    p.sig[2 * n + i] = (float)(K0 * vs);
    p.sig[3 * n + i] = p.sig[4 * n + i] = p.sig[5 * n + i] = 0.f;
}

// ---------------------------------------------------------------- integrators
template <bool EOS>
__global__ void k_advect_half32(K32 k, P32 p, T32 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    const float wi = p.hi[i].w;
    const int ti = tf_type(wi);
    if (ti <= 0) return;
    if (ti == MAT_SOIL && k.solver == 3) {
        const size_t n = k.n;
        for (int q = 0; q < 6; ++q) t.sigt[q * n + i] += k.hdt * t.dsig[q * n + i];
    }
    const float drt = t.drt[i] + k.hdt * t.dd[i];
    t.drt[i] = drt;
    p.lo[i].w = p.mass[i] / (k.rho0 + drt);
    const float4 dv = t.dv[i];
    float4 vt = t.vt[i];
    if (t.vtlo) {
        float4 vl = t.vtlo[i];
        two_sum_add(vt.x, vl.x, k.hdt * dv.x);
        two_sum_add(vt.y, vl.y, k.hdt * dv.y);
        two_sum_add(vt.z, vl.z, k.hdt * dv.z);
        t.vtlo[i] = vl;
    } else {
        vt.x += k.hdt * dv.x; vt.y += k.hdt * dv.y; vt.z += k.hdt * dv.z;
    }
    if (EOS && ti == MAT_FLUID) eos_store(k, p, t, i, wi, drt, vt);  // the next one_step's first phase
    else t.vt[i] = vt;
}

// ---- RK4 (eng/solver_sph_base.py:134-180): accumulate m * rates over the four one_steps;
// the intermediate states use dt / 2 from the step-start values (the reference's stages)
__global__ void k_rk_init32(K32 k, P32 p, T32 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    const int ti = tf_type(p.hi[i].w);
    if (ti <= 0) return;
    t.ddrk[i] = 0.f;
    t.dvrk[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (ti == MAT_SOIL && t.dsigrk)
        for (int q = 0; q < 6; ++q) t.dsigrk[(size_t)q * k.n + i] = 0.f;
}

__global__ void k_rk_update32(K32 k, P32 p, T32 t, float m) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    const int ti = tf_type(p.hi[i].w);
    if (ti <= 0) return;
    t.ddrk[i] += t.dd[i] * m;
    const float4 dv = t.dv[i];
    float4 a = t.dvrk[i];
    a.x += dv.x * m; a.y += dv.y * m; a.z += dv.z * m;
    t.dvrk[i] = a;
    if (ti == MAT_SOIL && t.dsigrk)
        for (int q = 0; q < 6; ++q) t.dsigrk[(size_t)q * k.n + i] += m * t.dsig[(size_t)q * k.n + i];
}

__global__ void k_rk_stage32(K32 k, P32 p, T32 t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    const int ti = tf_type(p.hi[i].w);
    if (ti <= 0) return;
    const float drt = k.hdt * t.dd[i] + p.drho[i];
    t.drt[i] = drt;
    p.lo[i].w = p.mass[i] / (k.rho0 + drt);
    const float4 dv = t.dv[i];
    float4 vt = p.vel[i];
    if (t.vtlo) {
        float4 vl = p.vlo[i];
        two_sum_add(vt.x, vl.x, k.hdt * dv.x);
        two_sum_add(vt.y, vl.y, k.hdt * dv.y);
        two_sum_add(vt.z, vl.z, k.hdt * dv.z);
        t.vtlo[i] = vl;
    } else {
        vt.x = k.hdt * dv.x + vt.x; vt.y = k.hdt * dv.y + vt.y; vt.z = k.hdt * dv.z + vt.z;
    }
    t.vt[i] = make_float4(vt.x, vt.y, vt.z, t.vt[i].w);
    if (ti == MAT_SOIL && k.solver == 3)
        for (int q = 0; q < 6; ++q)
            t.sigt[(size_t)q * k.n + i] = k.hdt * t.dsig[(size_t)q * k.n + i] + p.sig[(size_t)q * k.n + i];
}

__global__ void k_rk_final32(K32 k, P32 p, T32 t, int* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    const int ti = tf_type(p.hi[i].w);
    if (ti <= 0) return;
    const float dr = p.drho[i] + k.dt6 * t.ddrk[i];
    p.drho[i] = dr;
    p.lo[i].w = p.mass[i] / (k.rho0 + dr);
    const float4 a = t.dvrk[i];
    float4 v = p.vel[i];
    if (p.vlo) {
        float4 vl = p.vlo[i];
        two_sum_add(v.x, vl.x, k.dt6 * a.x);
        two_sum_add(v.y, vl.y, k.dt6 * a.y);
        two_sum_add(v.z, vl.z, k.dt6 * a.z);
        p.vlo[i] = vl;
    } else {
        v.x += k.dt6 * a.x; v.y += k.dt6 * a.y; v.z += k.dt6 * a.z;
    }
    p.vel[i] = v;
    if (ti == MAT_SOIL && k.solver == 3)
        for (int q = 0; q < 6; ++q) p.sig[(size_t)q * k.n + i] += k.dt6 * t.dsigrk[(size_t)q * k.n + i];
    if (!isfinite(dr)) atomicOr(err, TSG_ERR_NONFINITE);
}

__global__ void k_advect_full32(K32 k, P32 p, T32 t, int* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    const int ti = tf_type(p.hi[i].w);
    if (ti <= 0) return;
    if (ti == MAT_SOIL && k.solver == 3) {
        const size_t n = k.n;
        for (int q = 0; q < 6; ++q) p.sig[q * n + i] += k.dt * t.dsig[q * n + i];
    }
    const float dr = p.drho[i] + k.dt * t.dd[i];
    p.drho[i] = dr;
    p.lo[i].w = p.mass[i] / (k.rho0 + dr);
    const float4 dv = t.dv[i];
    float4 v = p.vel[i];
    if (p.vlo) {
        float4 vl = p.vlo[i];
        two_sum_add(v.x, vl.x, k.dt * dv.x);
        two_sum_add(v.y, vl.y, k.dt * dv.y);
        two_sum_add(v.z, vl.z, k.dt * dv.z);
        p.vlo[i] = vl;
    } else {
        v.x = __fmaf_rn(k.dt, dv.x, v.x); v.y = __fmaf_rn(k.dt, dv.y, v.y); v.z = __fmaf_rn(k.dt, dv.z, v.z);
    }
    p.vel[i] = v;
    if (!isfinite(dr)) atomicOr(err, TSG_ERR_NONFINITE);
}

// Largest squared displacement of a real particle since the last list build (pf holds the
// build-time positions); float bits of non-negative values order like unsigned integers.
// block_max_disp is called by every thread of the block (one atomic per block: a warp's
// atomics on the one word serialise); the rounding of disp2 is spelled out so that the
// kernels computing it give the same bits.
__device__ __forceinline__ float disp2(const float4& h, const float4& l, const float4& f) {
    const float dx = __fsub_rn(__fadd_rn(h.x, l.x), f.x), dy = __fsub_rn(__fadd_rn(h.y, l.y), f.y),
                dz = __fsub_rn(__fadd_rn(h.z, l.z), f.z);
    const float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
    return d2 == d2 ? d2 : 3.0e38f;  // non-finite: force a rebuild (the hash flags it)
}
__device__ __forceinline__ void block_max_disp(float d2, unsigned* maxd) {
    __shared__ float wmax[32];
    for (int o = 16; o > 0; o >>= 1) d2 = fmaxf(d2, __shfl_down_sync(0xffffffffu, d2, o));
    const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0) wmax[w] = d2;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = 0.f;
        for (int q = 0; q < nw; ++q) m = fmaxf(m, wmax[q]);
        if (m > 0.f) atomicMax(maxd, __float_as_uint(m));
    }
}

// One real particle's advect_SE / advect_LF, advect_pos and density clamp; returns the new
// (lo, m_V) record.
__device__ __forceinline__ float4 advect_final_one(const K32& k, P32& p, T32& t, int i, int ti, int* err) {
    float dr = p.drho[i] + k.dt * t.dd[i];
    const bool dr_ok = isfinite(dr);
    const float4 dv = t.dv[i];
    float4 v = p.vel[i];
    float4 vs = v;  // velocity the positions move with (v + vlo)
    if (p.vlo) {
        float4 vl = p.vlo[i];
        two_sum_add(v.x, vl.x, k.dt * dv.x);
        two_sum_add(v.y, vl.y, k.dt * dv.y);
        two_sum_add(v.z, vl.z, k.dt * dv.z);
        p.vlo[i] = vl;
        vs = make_float4(v.x + vl.x, v.y + vl.y, v.z + vl.z, 0.f);
    } else {
        v.x = __fmaf_rn(k.dt, dv.x, v.x); v.y = __fmaf_rn(k.dt, dv.y, v.y); v.z = __fmaf_rn(k.dt, dv.z, v.z);
        vs = v;
    }
    p.vel[i] = v;
    float4 l = p.lo[i];
    l.x = __fmaf_rn(k.dt, vs.x, l.x);
    l.y = __fmaf_rn(k.dt, vs.y, l.y);
    l.z = __fmaf_rn(k.dt, vs.z, l.z);
    if (ti == MAT_FLUID) dr = fmaxf(dr, 0.f);
    p.drho[i] = dr;
    l.w = p.mass[i] / (k.rho0 + dr);
    p.lo[i] = l;
    if (!dr_ok || !(isfinite(l.x) && isfinite(l.y) && isfinite(l.z))) atomicOr(err, TSG_ERR_NONFINITE);
    return l;
}

// WCSPH without XSPH, symplectic Euler or leap-frog: advect_SE / advect_LF, advect_pos and
// the density clamp of advect_something in one pass over each particle's own state, in
// the order of the separate kernels.  The velocity and position updates are explicit fused
// multiply-adds here and there, so the compiler's contraction choices cannot make the two
// paths round differently.  maxd (may be null): the largest squared displacement since the
// list build is folded in from the new positions, as the next step's list-expiry check
// would compute it (a captured multi-step graph drops that check after its first step
// and has the steps before the last fold their positions in).
__global__ void k_advect_final_wc32(K32 k, P32 p, T32 t, int* err, const float4* __restrict__ PF,
                                    unsigned* __restrict__ maxd) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float d2 = 0.f;
    if (i < k.nd) {
        const float4 h = p.hi[i];
        if (tf_type(h.w) > 0) {
            const float4 l = advect_final_one(k, p, t, i, tf_type(h.w), err);
            if (maxd) d2 = disp2(h, l, PF[i]);
        }
    }
    if (maxd) block_max_disp(d2, maxd);
}

template <int DIM, bool FB>
__global__ void k_xsph32(K32 k, P32 p, T32 t, const float4* __restrict__ PF, const int* __restrict__ dstart,
                         const int* __restrict__ sstart, Ovf ovf) {
    FOR_PARTICLES(FB, 0, k.nd, ovf, t.cnt, k.maxn, {
        const int ti = tf_type(p.hi[i].w);
        if (ti > 0 && tf_dyn(p.hi[i].w)) {
            const float4 vi = p.vel[i];
            CSum s[3];
            for_nbrs<DIM, FB>(k, i, t.cnt, t.nbr, p.hi, p.lo, PF, dstart, sstart, is_flow(ti),
                              [&](int j, const float*, float r2, int sidx, int tj, float mVj) {
                if (tj != ti) return;
                const float w = w_val(k, fast_sqrt(r2)) * mVj;
                const float4 vj = p.vel[j];
                s[0].add(w * (vj.x - vi.x));
                s[1].add(w * (vj.y - vi.y));
                if (DIM == 3) s[2].add(w * (vj.z - vi.z));
                if (sidx % kFlushEvery == kFlushEvery - 1) { s[0].flush(); s[1].flush(); s[2].flush(); }
            });
            t.xs[i] = make_float4(s[0].get(), s[1].get(), DIM == 3 ? s[2].get() : 0.f, 0.f);
        }
    });
}

// POST: also the WCSPH density clamp of advect_something (k_post_wc32, which touches density
// and m_V only, so its order against the position update does not matter).
template <bool POST>
__global__ void k_advect_pos32(K32 k, P32 p, T32 t, int* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    const float w = p.hi[i].w;
    if (tf_type(w) <= 0) return;
    float4 v = p.vel[i];
    if (p.vlo) {
        const float4 vl = p.vlo[i];
        v.x += vl.x; v.y += vl.y; v.z += vl.z;
    }
    float4 l = p.lo[i];
    if (k.xsph && tf_dyn(w)) {
        const float4 s = t.xs[i];
        l.x += k.dt * (v.x + 0.5f * s.x);
        l.y += k.dt * (v.y + 0.5f * s.y);
        l.z += k.dt * (v.z + 0.5f * s.z);
    } else {
        l.x = __fmaf_rn(k.dt, v.x, l.x);
        l.y = __fmaf_rn(k.dt, v.y, l.y);
        l.z = __fmaf_rn(k.dt, v.z, l.z);
    }
    if (POST && tf_type(w) == MAT_FLUID) {
        const float dr = fmaxf(p.drho[i], 0.f);
        p.drho[i] = dr;
        l.w = p.mass[i] / (k.rho0 + dr);
    }
    p.lo[i] = l;
    if (!(isfinite(l.x) && isfinite(l.y) && isfinite(l.z))) atomicOr(err, TSG_ERR_NONFINITE);
}

__global__ void k_post_wc32(K32 k, P32 p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    if (tf_type(p.hi[i].w) != MAT_FLUID) return;
    const float dr = fmaxf(p.drho[i], 0.f);
    p.drho[i] = dr;
    p.lo[i].w = p.mass[i] / (k.rho0 + dr);
}

// Collision boundary (eng/solver_sph_base.py:525-601), flow particles when boundary == 1.
__global__ void k_enforce32(K32 k, P32 p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.nd) return;
    const int ti = tf_type(p.hi[i].w);
    const bool rigid_dyn = ti == MAT_RIGID && tf_dyn(p.hi[i].w);
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
// Export of one field in f64: component q of particle i goes to out[q * sq + i * si]
// (planar views: sq = n, si = 1; row-major host buffers: sq = 1, si = components).
__device__ __forceinline__ void export_one(const K32& k, const P32& p, const T32& t, int what, int i, double* o,
                                           size_t sq) {
    const size_t n = k.n;
    switch (what) {
    case 0: {  // x
        float4 h = p.hi[i], l = p.lo[i];
        o[0] = k.vs[0] + ((double)h.x + (double)l.x);
        o[sq] = k.vs[1] + ((double)h.y + (double)l.y);
        o[2 * sq] = k.vs[2] + ((double)h.z + (double)l.z);
        break;
    }
    case 1: {
        const float4 v = p.vel[i];
        const float4 vl = p.vlo ? p.vlo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        o[0] = (double)v.x + vl.x; o[sq] = (double)v.y + vl.y; o[2 * sq] = (double)v.z + vl.z;
        break;
    }
    case 2: o[0] = tf_type(p.hi[i].w) > 0 ? (double)k.rho0 + (double)p.drho[i] : 0.0; break;  // density
    case 3: o[0] = p.vel[i].w; break;                       // pressure
    case 4: o[0] = p.lo[i].w; break;                        // m_V
    case 5: o[0] = p.mass[i]; break;                        // mass
    case 6: {  // v_tmp
        const float4 v = t.vt[i];
        const float4 vl = t.vtlo ? t.vtlo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        o[0] = (double)v.x + vl.x; o[sq] = (double)v.y + vl.y; o[2 * sq] = (double)v.z + vl.z;
        break;
    }
    case 7: o[0] = (double)k.rho0 + (double)t.drt[i]; break;  // density_tmp
    case 8: o[0] = t.dd[i]; break;
    case 9: { float4 v = t.dv[i]; o[0] = v.x; o[sq] = v.y; o[2 * sq] = v.z; break; }
    case 10: o[0] = t.cf[i]; break;
    case 11: {  // CSPM_L: full 3 x 3 from the six stored planes
        float L[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (t.L) load_L(t.L, n, i, L);
        for (int q = 0; q < 9; ++q) o[q * sq] = L[q];
        break;
    }
    case 12: case 13: case 14: {  // stress, stress_tmp, d_stress: full 3 x 3 from the six stored
        const float* a = what == 12 ? p.sig : what == 13 ? t.sigt : t.dsig;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) o[(size_t)(3 * r + c) * sq] = a[(size_t)sym_idx(r, c) * n + i];
        break;
    }
    case 15: o[0] = p.eeq[i]; break;
    case 16: o[0] = p.eeqp[i]; break;
    case 17: o[0] = t.dee[i]; break;
    case 18: o[0] = t.deep[i]; break;
    default: break;
    }
}

__global__ void k_export(K32 k, P32 p, T32 t, int what, double* out, size_t sq, size_t si) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    export_one(k, p, t, what, i, out + (size_t)i * si, sq);
}

// Several float fields in one pass, field q row-major at out + off[q].
struct ExportSet {
    int count;
    int what[8];
    int comps[8];
    size_t off[8];
};
// Particles [i0, i1) of the fields in es, row-major per field into out + es.off[q].
__global__ void k_export_set(K32 k, P32 p, T32 t, ExportSet es, double* out, int i0, int i1) {
    int i = i0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= i1) return;
    for (int q = 0; q < es.count; ++q)
        export_one(k, p, t, es.what[q], i, out + es.off[q] + (size_t)i * es.comps[q], 1);
}

__global__ void k_export_int(K32 k, P32 p, int what, int* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const int4 id = p.ids[i];
    switch (what) {
    case 0: out[i] = id.x; break;
    case 1: out[i] = tf_type(p.hi[i].w); break;
    case 2: out[i] = id.y; break;
    case 3: out[i] = id.z; break;
    case 4: out[i] = id.w; break;
    case 5: out[i] = p.flag ? p.flag[i] : 0; break;
    default: break;
    }
}

// Write a field from planar f64 staging (tsg_write).
// Import of one field from a row-major f64 buffer (component q of particle i at
// in[i * comps + q]).
// Row-major input (device memory, or page-locked host memory read over the host link).
__global__ void k_import(K32 k, P32 p, int what, const double* in) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const double* r = in + (size_t)(what <= 1 ? 3 : 1) * i;
    switch (what) {
    case 0: {
        float4 h = p.hi[i], l = p.lo[i];
        double x[3] = {r[0] - k.vs[0], r[1] - k.vs[1], r[2] - k.vs[2]};
        l.x = (float)(x[0] - (double)h.x); l.y = (float)(x[1] - (double)h.y); l.z = (float)(x[2] - (double)h.z);
        p.lo[i] = l;
        break;
    }
    case 1: {
        float4 v = p.vel[i];
        const double a = r[0], b = r[1], c = r[2];
        v.x = (float)a; v.y = (float)b; v.z = (float)c;
        p.vel[i] = v;
        if (p.vlo) p.vlo[i] = make_float4((float)(a - v.x), (float)(b - v.y), (float)(c - v.z), 0.f);
        break;
    }
    case 2: if (tf_type(p.hi[i].w) > 0) p.drho[i] = (float)(r[0] - (double)k.rho0); break;
    case 3: p.vel[i].w = (float)r[0]; break;
    default: break;
    }
}

// FP64 conservation diagnostics over flow particles.
__global__ void k_diag32(K32 k, P32 p, double* out) {
    __shared__ double sh[8][TPB / 32];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[8] = {0, 0, 0, 0, 0, 0, 0, -DBL_MAX};
    if (i < k.nd && is_flow(tf_type(p.hi[i].w))) {
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
                         const int* __restrict__ dyn, const int* __restrict__ slot,
                         const int* __restrict__ scene_of, P32 p) {
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
    const int sc = scene_of ? (scene_of[s] & 0xfff) : 0;
    const int word = 0x40000000 | (mt[s] & 0xffff) | ((dyn[s] & 1) << 16) | (sc << 17);
    p.hi[i] = make_float4(hv[0], hv[1], hv[2], __int_as_float(word));
    p.lo[i] = make_float4(lv[0], lv[1], lv[2], (float)mV[s]);
    const double v0 = v[3 * (size_t)s], v1 = v[3 * (size_t)s + 1], v2 = v[3 * (size_t)s + 2];
    p.vel[i] = make_float4((float)v0, (float)v1, (float)v2, (float)pres[s]);
    if (p.vlo) p.vlo[i] = make_float4((float)(v0 - (float)v0), (float)(v1 - (float)v1), (float)(v2 - (float)v2), 0.f);
    p.drho[i] = mt[s] > 0 ? (float)(dens[s] - (double)k.rho0) : 0.f;
    p.mass[i] = (float)mass[s];
    p.ids[i] = make_int4(s, mid[s], oid[s], dyn[s]);
}

// Upload of the initial stress: (n, 3, 3) row-major -> six planes (upper triangle).
__global__ void k_load_stress32(K32 k, const double* __restrict__ st, const int* __restrict__ slot, P32 p) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= k.n) return;
    const int i = slot[s];
    const size_t n = k.n;
    const double* a = st + 9 * (size_t)s;
    p.sig[i] = (float)a[0];
    p.sig[n + i] = (float)a[4];
    p.sig[2 * n + i] = (float)a[8];
    p.sig[3 * n + i] = (float)a[1];
    p.sig[4 * n + i] = (float)a[2];
    p.sig[5 * n + i] = (float)a[5];
}

// Inspection: enumerate every neighbour directly (independent of the ELL capacity).
template <int DIM>
__global__ void k_nbr_count32(K32 k, const float4* HI, RecView LO, const float4* PF, const int* ds,
                              const int* ss, int* counts) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    int m = 0;
    enum_neighbors<DIM>(k, i, HI, LO, PF, ds, ss, is_flow(tf_type(PF[i].w)), [&](int, const float*, float) { ++m; },
                        false, false);
    counts[i] = m;
}

template <int DIM>
__global__ void k_nbr_fill32(K32 k, const float4* HI, RecView LO, const float4* PF, const int* ds,
                             const int* ss, const int* off, int* list) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    int m = off[i];
    enum_neighbors<DIM>(k, i, HI, LO, PF, ds, ss, is_flow(tf_type(PF[i].w)),
                        [&](int j, const float*, float) { list[m++] = j; }, false, false);
}

template <int DIM>
__global__ void k_nbr_count_ell(K32 k, const float4* HI, RecView LO, const int* cnt, const int* nbr, int* counts) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const int m = cnt[i] < k.maxn ? cnt[i] : k.maxn;
    int c = 0;
    for (int q = 0; q < m; ++q) {
        const int j = entry_index(k, nbr[(size_t)q * k.n + i]);
        float d[3];
        delta<DIM>(HI[i], LO[i], HI[j], LO[j], d);
        const float r2 = dist2<DIM>(d);
        if (r2 < k.R2) ++c;
    }
    counts[i] = c;
}

template <int DIM>
__global__ void k_nbr_fill_ell(K32 k, const float4* HI, RecView LO, const float4* PF, const int* ds,
                               const int* ss, const int* cnt, const int* nbr, const int* off, int* list) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const int m = cnt[i];
    int w = off[i];
    if (m <= k.maxn) {
        for (int q = 0; q < m; ++q) {
            const int j = entry_index(k, nbr[(size_t)q * k.n + i]);
            float d[3];
            delta<DIM>(HI[i], LO[i], HI[j], LO[j], d);
            const float r2 = dist2<DIM>(d);
            if (r2 < k.R2) list[w++] = j;
        }
    } else {
        enum_neighbors<DIM>(k, i, HI, LO, PF, ds, ss, is_flow(tf_type(PF[i].w)),
                            [&](int j, const float*, float) { list[w++] = j; });
    }
}

// Largest squared displacement of a real particle since the last list build.
__global__ void k_disp32(K32 k, const float4* __restrict__ HI, RecView LO,
                         const float4* __restrict__ PF, unsigned* __restrict__ maxd) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float d2 = 0.f;
    if (i < k.nd) d2 = disp2(HI[i], LO[i], PF[i]);
    block_max_disp(d2, maxd);
}

// List occupancy: out[0] / out[1] += stored entries (min(count, capacity)) of the dynamic /
// static block, out[2] += overflowed particles (each thread classifies its own particle).
__global__ void k_list_stats(K32 k, const int* __restrict__ cnt, unsigned long long* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long ed = 0, es = 0, o = 0;
    if (i < k.n) {
        const int m = cnt[i];
        const unsigned long long e = (unsigned long long)(m < k.maxn ? m : k.maxn);
        if (i < k.nd) ed = e; else es = e;
        o = m > k.maxn ? 1ull : 0ull;
    }
    for (int d = 16; d > 0; d >>= 1) {
        ed += __shfl_down_sync(0xffffffffu, ed, d);
        es += __shfl_down_sync(0xffffffffu, es, d);
        o += __shfl_down_sync(0xffffffffu, o, d);
    }
    if ((threadIdx.x & 31) == 0) {
        if (ed) atomicAdd(&out[0], ed);
        if (es) atomicAdd(&out[1], es);
        if (o) atomicAdd(&out[2], o);
    }
}

// Per-scene FP64 diagnostics of a batched ensemble (out[8 * scene + q], q as k_diag32;
// positions relative to the scene's own origin, x - scene * pitch).  Warps whose flow
// particles all belong to one scene reduce before their atomics.
__global__ void k_diag_batch32(K32 k, P32 p, double pitch, double* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[8] = {0, 0, 0, 0, 0, 0, 0, -DBL_MAX};
    int sc = -1;
    if (i < k.nd) {
        const float w = p.hi[i].w;
        if (is_flow(tf_type(w))) {
            sc = tf_scene(w);
            const double m = p.mass[i];
            const float4 vv = p.vel[i];
            const float4 h = p.hi[i], l = p.lo[i];
            const double x = k.vs[0] + ((double)h.x + (double)l.x) - sc * pitch;
            const double y = k.vs[1] + ((double)h.y + (double)l.y);
            const double z = k.vs[2] + ((double)h.z + (double)l.z);
            const double v2 = (double)vv.x * vv.x + (double)vv.y * vv.y + (double)vv.z * vv.z;
            v[0] = m; v[1] = m * vv.x; v[2] = m * vv.y; v[3] = m * vv.z; v[4] = 0.5 * m * v2;
            v[5] = -m * ((double)k.g[0] * x + (double)k.g[1] * y + (double)k.g[2] * z);
            v[6] = sqrt(v2); v[7] = x;
        }
    }
    const unsigned peers = __match_any_sync(0xffffffffu, sc);
    if (peers == 0xffffffffu) {
        if (sc < 0) return;
        for (int o = 16; o > 0; o >>= 1) {
            for (int q = 0; q < 6; ++q) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
            v[6] = fmax(v[6], __shfl_down_sync(0xffffffffu, v[6], o));
            v[7] = fmax(v[7], __shfl_down_sync(0xffffffffu, v[7], o));
        }
        if ((threadIdx.x & 31) != 0) return;
    } else if (sc < 0) {
        return;
    }
    double* o8 = out + 8 * (size_t)sc;
    for (int q = 0; q < 6; ++q) atomicAdd(&o8[q], v[q]);
    atomic_max_d(&o8[6], v[6]);
    atomic_max_d(&o8[7], v[7]);
}

// Graph mode: decide on the device whether this step re-sorts and rebuilds the lists
// (largest displacement since the last build above 0.45 skin), by setting the condition
// of the graph's IF node; count the rebuilds.
__global__ void k_set_rebuild32(cudaGraphConditionalHandle hnd, const unsigned* __restrict__ maxd, float limit,
                                int* __restrict__ counter) {
    const float d2 = __uint_as_float(*maxd);
    const unsigned r = !(d2 <= limit) ? 1u : 0u;
    cudaGraphSetConditional(hnd, r);
    if (r) atomicAdd(counter, 1);
}

}  // namespace

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

// Smallest power of two not below the cell size (list entries assume |hi_i - hi_j| <= Q).
float pow2_quantum(double grid) {
    double q = 1.0;
    while (q < grid) q *= 2.0;
    while (q * 0.5 >= grid) q *= 0.5;
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
    sort_within_cells(nbins, start, st.cell_of, count_n, st.perm, st.sort_big, st.sort_nbig, s);
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
                Fp32State** out, cudaStream_t s, const Fp32Scenes* scenes, const RigidObjects* rigid) {
    *out = nullptr;
    if (c.n > (1 << kEntryBits)) return TSG_E_CAPACITY;  // neighbour-list entries index 2^23 particles

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
    k.cub1h = (float)(c.kk * c.h1 * c.h1);
    k.R2 = (float)(c.R * c.R);
    k.R2hi = std::nextafter((float)(c.R * c.R * (1.0 + 1.0 / 1024.0)), 1e30f);
    k.R2lo = (float)(c.R * c.R * (1.0 - 1.0 / 1024.0));
    k.pf_lim = (float)(500.0 * c.R);
    k.visc_fac = (float)c.visc_fac; k.eps_h2 = (float)c.eps_h2; k.rho0 = (float)c.rho0; k.B = (float)c.B;
    k.gamma = (float)c.gamma; k.dt = (float)c.dt; k.hdt = (float)c.hdt; k.dt6 = (float)c.dt6;
    k.rep_fac = (float)c.rep_fac; k.diam = (float)c.diam; k.h075 = (float)c.h075; k.r_eps = (float)c.r_eps;
    k.mu = (float)c.mu; k.c2 = (float)c.vsound2; k.coh = (float)c.coh; k.alpha = (float)c.alpha;
    k.k_c = (float)c.k_c; k.kc_over_alpha = (float)c.kc_over_alpha; k.Gm = (float)c.Gm; k.Km = (float)c.Km;
    k.sin_dila = (float)c.sin_dila; k.lam_den = (float)c.lam_den; k.three_aK = (float)c.three_aK;
    k.nine_K_sin = (float)c.nine_K_sin; k.twoG = (float)c.twoG;
    k.damp_eps = (float)c.damp_eps; k.damp_E = (float)c.damp_E; k.h2 = (float)c.h2;
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
    k.inv_Q = 1.f / k.Q;
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
    const bool soil = c.solver != 1;
    for (int q = 0; q < 2; ++q) {
        st->P[q].hi = dal<float4>(*st, n); st->P[q].lo = RecView{dal<float4>(*st, 2 * (size_t)n)};
        st->P[q].vel = dal<float4>(*st, n);
        st->P[q].drho = dal<float>(*st, n); st->P[q].mass = dal<float>(*st, n); st->P[q].ids = dal<int4>(*st, n);
        if (soil) {
            st->P[q].sig = dal<float>(*st, 6 * (size_t)n); st->P[q].eeq = dal<float>(*st, n);
            st->P[q].eeqp = dal<float>(*st, n); st->P[q].flag = dal<int>(*st, n);
            st->P[q].vlo = dal<float4>(*st, n);
        }
    }
    T32& t = st->T;
    // v_tmp lives in the second half of the current buffer's records (sorts copy back in place,
    // so the current buffer is always P[0])
    t.vt = RecView{st->P[0].lo.p ? st->P[0].lo.p + 1 : nullptr}; t.pr = dal<float2>(*st, n); t.drt = dal<float>(*st, n); t.dd = dal<float>(*st, n);
    t.dv = dal<float4>(*st, n); t.cf = dal<float>(*st, n); t.xs = dal<float4>(*st, n);
    t.L = c.corr == 1 ? dal<float>(*st, 6 * (size_t)n) : nullptr;
    t.cnt = dal<int>(*st, n);
    t.nbr = dal<int>(*st, (size_t)k.maxn * n);
    // RK4 accumulators for every integrator (substep_RK may be called on any handle)
    t.ddrk = dal<float>(*st, n);
    t.dvrk = dal<float4>(*st, n);
    if (c.solver == 3) t.dsigrk = dal<float>(*st, 6 * (size_t)n);
    if (soil) {
        t.vtlo = dal<float4>(*st, n);
        t.sigt = dal<float>(*st, 6 * (size_t)n); t.dee = dal<float>(*st, n);
        t.srec = dal<float4>(*st, 2 * (size_t)n);
        if (c.solver == 3) { t.dsig = dal<float>(*st, 6 * (size_t)n); t.deep = dal<float>(*st, n); }
    }
    st->pf = dal<float4>(*st, n);
    const size_t nb = (size_t)k.G + 1;
    st->dcount = dal<int>(*st, nb); st->dstart = dal<int>(*st, nb + 1);
    st->scount = dal<int>(*st, nb); st->sstart = dal<int>(*st, nb + 1);
    st->cell_of = dal<int>(*st, n); st->rank = dal<int>(*st, n); st->perm = dal<int>(*st, n);
    st->tiles = dal<int>(*st, nb / 2048 + 4); st->err = dal<int>(*st, 1);
    st->cells_d = dal<int>(*st, nb); st->cells_s = dal<int>(*st, nb); st->ncells = dal<int>(*st, 2);
    st->ovf_list = dal<int>(*st, n); st->novf = dal<int>(*st, 1);
    st->sact = dal<int>(*st, n - nd > 0 ? n - nd : 1); st->nsact = dal<int>(*st, 1);
    st->maxdisp = dal<unsigned>(*st, 1);
    st->sort_big = dal<int>(*st, cellsort_big_ints(n));
    st->sort_nbig = dal<int>(*st, 1);
    st->d_rebuilds = dal<int>(*st, 1);
    st->cells_per_cta = c.dim == 3 ? 4 : 0;
    st->stage = dal<double>(*st, 9 * (size_t)n + 16);
    st->scratch = dal<double>(*st, 64);
    if (!t.nbr || !st->stage || !st->sort_big || !st->sort_nbig || (soil && !t.srec)) { fp32_destroy(st); return TSG_E_CUDA; }
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
    int* imt = reinterpret_cast<int*>(st->P[1].lo.p);
    int* imid = imt + n;
    int* ioid = imid + n;
    int* idyn = reinterpret_cast<int*>(st->P[1].vel);
    int* islot = st->perm;
    cudaMemcpyAsync(imt, pp->mat_type, sizeof(int) * n, kind, s);
    cudaMemcpyAsync(imid, pp->mat_id, sizeof(int) * n, kind, s);
    cudaMemcpyAsync(ioid, pp->obj_id, sizeof(int) * n, kind, s);
    cudaMemcpyAsync(idyn, pp->is_dynamic, sizeof(int) * n, kind, s);
    cudaMemcpyAsync(islot, slot.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
    int* iscene = nullptr;
    if (scenes && scenes->nscenes > 0) {
        if (scenes->nscenes > kMaxScenes) { fp32_destroy(st); return TSG_E_CAPACITY; }
        iscene = st->cell_of;  // scratch until the first sort
        cudaMemcpyAsync(iscene, scenes->scene_of, sizeof(int) * n, cudaMemcpyHostToDevice, s);
        std::vector<float2> par(scenes->nscenes);
        for (int q = 0; q < scenes->nscenes; ++q) par[q] = make_float2(scenes->stiffness[q], scenes->visc_fac[q]);
        float2* dpar = dal<float2>(*st, scenes->nscenes);
        if (!dpar) { fp32_destroy(st); return TSG_E_CUDA; }
        cudaMemcpyAsync(dpar, par.data(), sizeof(float2) * scenes->nscenes, cudaMemcpyHostToDevice, s);
        cudaStreamSynchronize(s);
        k.scene_par = dpar;
        st->nscenes = scenes->nscenes;
    }
    if (rigid && !rigid->ids.empty()) {  // dynamic rigid bodies: object table and rest offsets
        st->rnobj = (int)rigid->ids.size();
        st->r_ids = dal<int>(*st, rigid->ids.size());
        st->r_off = dal<int>(*st, rigid->off.size());
        st->r_list = dal<int>(*st, (size_t)rigid->off.back() + 1);
        st->r_q = dal<double>(*st, 3 * (size_t)n);
        if (!st->r_q) { fp32_destroy(st); return TSG_E_CUDA; }
        cudaMemcpyAsync(st->r_ids, rigid->ids.data(), sizeof(int) * rigid->ids.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(st->r_off, rigid->off.data(), sizeof(int) * rigid->off.size(), cudaMemcpyHostToDevice, s);
        int maxm = 0;
        for (size_t o = 0; o + 1 < rigid->off.size(); ++o) maxm = std::max(maxm, rigid->off[o + 1] - rigid->off[o]);
        st->r_chunks = std::max(1, (maxm + kRigidChunk - 1) / kRigidChunk);
        st->r_scratch = dal<int>(*st, rlist_scratch_ints(n, st->rnobj));
        st->r_part = dal<double>(*st, 9 * (size_t)st->rnobj * st->r_chunks);
        st->r_cm = dal<double>(*st, 3 * (size_t)st->rnobj);
        st->r_rot = dal<double>(*st, 9 * (size_t)st->rnobj);
        if (!st->r_scratch || !st->r_part || !st->r_cm || !st->r_rot) { fp32_destroy(st); return TSG_E_CUDA; }
        build_rigid_lists(n, st->rnobj, RigidSlotUpload{imt, idyn, ioid, st->r_ids, st->rnobj}, st->r_scratch,
                          st->r_off, st->r_list, s);
        TSG_LAUNCH(k_rigid_rest32, st->rnobj, kRigidBlock, s, st->r_off, st->r_list, dx, d2, st->r_q);
    }
    TSG_LAUNCH(k_load32, nblk(n), TPB, s, k, dx, dv, d1, d2, d3, d4, imt, imid, ioid, idyn, islot, iscene, st->P[0]);
    if (soil && pp->stress) {  // (n, 3, 3) row-major -> six planes (upper triangle)
        double* sst = nullptr;
        if (cudaMalloc(&sst, sizeof(double) * 9 * (size_t)n) != cudaSuccess) { fp32_destroy(st); return TSG_E_CUDA; }
        cudaMemcpyAsync(sst, pp->stress, sizeof(double) * 9 * n, kind, s);
        TSG_LAUNCH(k_load_stress32, nblk(n), TPB, s, k, sst, islot, st->P[0]);
        cudaStreamSynchronize(s);
        cudaFree(sst);
    }
    cudaStreamSynchronize(s);
    cudaMemsetAsync(st->P[1].hi, 0, sizeof(float4) * n, s);
    cudaMemsetAsync(st->P[1].lo.p, 0, sizeof(float4) * 2 * (size_t)n, s);
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
        cudaMemcpyAsync(dst.lo.p + 2 * off, src.lo.p + 2 * off, sizeof(float4) * 2 * ns, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(dst.vel + off, src.vel + off, sizeof(float4) * ns, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(dst.drho + off, src.drho + off, sizeof(float) * ns, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(dst.mass + off, src.mass + off, sizeof(float) * ns, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(dst.ids + off, src.ids + off, sizeof(int4) * ns, cudaMemcpyDeviceToDevice, s);
        if (soil) {
            for (int q = 0; q < 6; ++q)
                cudaMemcpyAsync(dst.sig + q * (size_t)n + off, src.sig + q * (size_t)n + off, sizeof(float) * ns,
                                cudaMemcpyDeviceToDevice, s);
            cudaMemcpyAsync(dst.eeq + off, src.eeq + off, sizeof(float) * ns, cudaMemcpyDeviceToDevice, s);
            cudaMemcpyAsync(dst.eeqp + off, src.eeqp + off, sizeof(float) * ns, cudaMemcpyDeviceToDevice, s);
            cudaMemcpyAsync(dst.flag + off, src.flag + off, sizeof(int) * ns, cudaMemcpyDeviceToDevice, s);
            cudaMemcpyAsync(dst.vlo + off, src.vlo + off, sizeof(float4) * ns, cudaMemcpyDeviceToDevice, s);
        }
    } else {
        cudaMemsetAsync(st->sstart, 0, sizeof(int) * (k.G + 2), s);
    }
    cudaMemsetAsync(st->ncells + 1, 0, sizeof(int), s);
    TSG_LAUNCH(k_nonempty_cells, nblk(k.G, 256), 256, s, (long long)k.G, st->sstart, st->cells_s, st->ncells + 1);
    if (c.solver == 3 && cfg.init_geostatic && nd > 0) {  // eng/solver_sph_dp.py:35 -> init_stress
        double lo = -DBL_MAX;
        cudaMemcpyAsync(st->scratch, &lo, sizeof lo, cudaMemcpyHostToDevice, s);
        TSG_LAUNCH(k_ymax32, nblk(nd), TPB, s, k, st->P[0], st->scratch);
        TSG_LAUNCH(k_geostatic32, nblk(nd), TPB, s, k, st->P[0], st->scratch, c.K0);
        cudaStreamSynchronize(s);
    }
    // the dynamic block of both buffers must agree before the first sort
    cudaStreamSynchronize(s);
    if (cudaGetLastError() != cudaSuccess) { fp32_destroy(st); return TSG_E_CUDA; }
    *out = st;
    return 0;
}

void fp32_destroy(Fp32State* st) {
    if (!st) return;
    for (auto& e : st->copy_ev)
        if (e) cudaEventDestroy(e);
    if (st->copy_stream) cudaStreamDestroy(st->copy_stream);
    for (auto& g : st->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    if (st->snap) cudaFree(st->snap);
    fp32_free_adjoint(*st);
    for (void* p : st->allocs) cudaFree(p);
    delete st;
}

namespace {

template <int DIM, int WPB>
void lists_by_cell(Fp32State& st, const P32& p, cudaStream_t s) {
    const K32& k = st.k;
    const int nb = 152 * 64 / WPB;
    TSG_LAUNCH((k_lists_cell<DIM, WPB>), nb, 32 * WPB, s, k, 0, st.cells_d, st.ncells, p.hi, p.lo, st.pf, st.dstart,
               st.sstart, st.T.cnt, st.T.nbr, st.ovf_list, st.novf);
    TSG_LAUNCH((k_lists_cell<DIM, WPB>), nb, 32 * WPB, s, k, 1, st.cells_s, st.ncells + 1, p.hi, p.lo, st.pf,
               st.dstart, st.sstart, st.T.cnt, st.T.nbr, st.ovf_list, st.novf);
}

template <int DIM>
void build_lists(Fp32State& st, const P32& p, cudaStream_t s) {
    const K32& k = st.k;
    cudaMemsetAsync(st.novf, 0, sizeof(int), s);
    if (st.cells_per_cta <= 0) {  // one thread per particle
        TSG_LAUNCH(k_lists<DIM>, nblk(k.n), TPB, s, k, p.hi, p.lo, st.pf, st.dstart, st.sstart, st.T.cnt, st.T.nbr,
                   st.ovf_list, st.novf);
        return;
    }
    cudaMemsetAsync(st.ncells, 0, sizeof(int), s);
    TSG_LAUNCH(k_nonempty_cells, nblk(k.G, 256), 256, s, (long long)k.G, st.dstart, st.cells_d, st.ncells);
    switch (st.cells_per_cta) {
    case 2: lists_by_cell<DIM, 2>(st, p, s); break;
    case 8: lists_by_cell<DIM, 8>(st, p, s); break;
    default: lists_by_cell<DIM, 4>(st, p, s); break;
    }
    // particles in the out-of-grid bins (bounds read on the device), then particles whose
    // true cell differs from their storage cell
    TSG_LAUNCH(k_lists_range<DIM>, 64, TPB, s, k, st.dstart + k.G, p.hi, p.lo, st.pf, st.dstart, st.sstart, st.T.cnt,
               st.T.nbr, st.ovf_list, st.novf);
    TSG_LAUNCH(k_lists_range<DIM>, 64, TPB, s, k, st.sstart + k.G, p.hi, p.lo, st.pf, st.dstart, st.sstart, st.T.cnt,
               st.T.nbr, st.ovf_list, st.novf);
    TSG_LAUNCH(k_lists_fixup<DIM>, 2 * 152, TPB, s, k, p.hi, p.lo, st.pf, st.dstart, st.sstart, st.T.cnt, st.T.nbr,
               st.ovf_list, st.novf);
}

// Static-block particles (fixed boundary) with a non-empty neighbour list, in warp-sized
// runs of the block's order (a run's place in the list depends on scheduling; every consumer
// treats its particles independently, so results do not).  A boundary particle with an
// empty list has no flow particle within support + skin: no flow particle reads its
// extrapolated state, and the values of the list kernels for it (Shepard factor 1, identity
// CSPM matrix, WCSPH extrapolation 2 v with zero pressure) depend on nothing but its own
// constant velocity; they are written here, once per list build, and the per-step kernels
// visit the listed particles only.
__global__ void k_static_active(K32 k, P32 p, T32 t, int wc, int* __restrict__ act, int* __restrict__ nact) {
    const int i = k.nd + blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = i < k.n;
    const bool on = in && t.cnt[i] != 0;
    const unsigned ball = __ballot_sync(0xffffffffu, on);
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0 && ball) base = atomicAdd(nact, __popc(ball));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (on) act[base + __popc(ball & ((1u << lane) - 1u))] = i;
    if (!in) return;
    if (t.L) {  // no static particle is a flow particle: its CSPM matrix is the identity
        const size_t n = k.n;
        for (int q = 0; q < 6; ++q) t.L[q * n + i] = q < 3 ? 1.f : 0.f;
    }
    if (on) return;
    t.cf[i] = 1.f;
    if (!wc) return;
    const int ti = tf_type(p.hi[i].w);
    if (ti == MAT_DUMMY || ti == MAT_REP || ti == MAT_RIGID) {
        const float4 v = p.vel[i];
        t.vt[i] = make_float4(2.f * v.x, 2.f * v.y, 2.f * v.z, 0.f);
        t.pr[i] = make_float2(0.f, k.rho0);
        t.drt[i] = 0.f;
        p.vel[i].w = 0.f;
        if (ti == MAT_RIGID) { t.dd[i] = 0.f; t.dv[i] = make_float4(0.f, 0.f, 0.f, 0.f); }
    }
}

// Copy the dynamic block of b back into a (graph mode keeps one current buffer).
__global__ void k_copy_back32(int nd, P32 b, P32 a, size_t n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nd) return;
    a.hi[i] = b.hi[i];
    a.lo[i] = b.lo[i];
    a.vel[i] = b.vel[i];
    a.drho[i] = b.drho[i];
    a.mass[i] = b.mass[i];
    a.ids[i] = b.ids[i];
    if (a.sig) {
        for (int q = 0; q < 6; ++q) a.sig[q * n + i] = b.sig[q * n + i];
        a.eeq[i] = b.eeq[i];
        a.eeqp[i] = b.eeqp[i];
        a.flag[i] = b.flag[i];
    }
    if (a.vlo) a.vlo[i] = b.vlo[i];
}

}  // namespace

// List the static-block particles with a non-empty list and write the state of the others.
static void static_active(Fp32State& st, cudaStream_t s) {
    cudaMemsetAsync(st.nsact, 0, sizeof(int), s);
    if (st.n > st.nd)
        TSG_LAUNCH(k_static_active, nblk(st.n - st.nd), TPB, s, st.k, st.P[st.cur], st.T, st.k.solver == 1 ? 1 : 0,
                   st.sact, st.nsact);
}

// Re-sort the dynamic block and rebuild every list.  in_place keeps the current buffer
// (the sorted block is copied back), as a captured graph needs fixed pointers.
void f32::rebuild(Fp32State& st, cudaStream_t s, bool in_place) {
    {
        PhaseScope ph(s, PH_SORT);
        if (st.nd > 0) {
            build_cells(st, 0, st.nd, st.dcount, st.dstart, s, true);
            if (in_place) TSG_LAUNCH(k_copy_back32, nblk(st.nd), TPB, s, st.nd, st.P[1 - st.cur], st.P[st.cur], (size_t)st.n);
            else st.cur = 1 - st.cur;
        } else {
            cudaMemsetAsync(st.dstart, 0, sizeof(int) * (st.k.G + 2), s);
        }
    }
    {
        PhaseScope ph2(s, PH_LISTS);
        if (st.k.dim == 3) build_lists<3>(st, st.P[st.cur], s);
        else build_lists<2>(st, st.P[st.cur], s);
        static_active(st, s);
    }
    cudaMemsetAsync(st.maxdisp, 0, sizeof(unsigned), s);
}

void fp32_sort(Fp32State& st, cudaStream_t s) {
    rebuild(st, s, true);  // in place: v_tmp lives in the current buffer's records
    st.lists_valid = true;
    st.built = true;
    ++st.rebuilds;
}

int fp32_list_stats(Fp32State& st, int64_t* out5, cudaStream_t s) {
    if (!st.built) return TSG_E_STATE;
    fp32_flush_counters(st, s);
    unsigned long long* acc = reinterpret_cast<unsigned long long*>(st.scratch);
    cudaMemsetAsync(acc, 0, 3 * sizeof(unsigned long long), s);
    TSG_LAUNCH(k_list_stats, nblk(st.k.n), TPB, s, st.k, st.T.cnt, acc);
    unsigned long long h[3] = {0, 0, 0};
    int nact = 0;
    cudaMemcpyAsync(h, acc, sizeof h, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&nact, st.nsact, sizeof nact, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    out5[0] = (int64_t)h[0];
    out5[1] = (int64_t)h[1];
    out5[2] = (int64_t)h[2];
    out5[3] = st.rebuilds;
    out5[4] = nact;
    return 0;
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

// The list kernels' main pass is compiled per kernel function (and, for the rates, per
// repulsive-boundary mode); their overflow pass (a few particles) decides both at run time.
// Grids of the main passes cover the largest possible count of listed static particles;
// the threads past the device count return at once.
// skip_fluid: the first rates pass computes the fluid's factors; when the dynamic block holds
// fluid only, the main pass then visits the listed static particles alone.  skip_static:
// the first boundary pass computes the static block's Shepard factors.
template <int DIM>
void corr_launch(Fp32State& st, cudaStream_t s, const Ovf& ovf, bool skip_fluid, bool skip_static) {
    const K32& k = st.k;
    const P32& p = st.P[st.cur];
    const int lim = skip_fluid && st.c.n_bdy <= k.n - k.nd ? 0 : k.nd;
    const int* act = skip_static ? nullptr : st.sact;
    const int nmax = skip_static ? k.nd : k.n;
    const int nb = nblk(lim + (skip_static ? 0 : k.n - k.nd), st.tpb);
    const int sf = skip_fluid ? 1 : 0;
    if (nb > 0) {
        if (k.kernel == 1)
            TSG_LAUNCH((k_corr32<DIM, false, 1>), nb, st.tpb, s, k, p, st.T, st.pf, st.dstart, st.sstart, act, st.nsact,
                       lim, nmax, sf, ovf);
        else
            TSG_LAUNCH((k_corr32<DIM, false, 0>), nb, st.tpb, s, k, p, st.T, st.pf, st.dstart, st.sstart, act, st.nsact,
                       lim, nmax, sf, ovf);
    }
    TSG_LAUNCH((k_corr32<DIM, true, -1>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, act, st.nsact, lim, nmax,
               sf, ovf);
}

// WCSPH boundary extrapolation over [base, base + count_n); the static block (base = nd)
// visits its listed particles only.
template <int DIM, bool SH>
void bdy_launch(Fp32State& st, const P32& p, int base, int count_n, cudaStream_t s, const Ovf& ovf) {
    const K32& k = st.k;
    const int nb = nblk(count_n, st.tpb);
    const int* act = base == k.nd ? st.sact : nullptr;
    if (k.kernel == 1)
        TSG_LAUNCH((k_bdy32<DIM, false, 1, SH>), nb, st.tpb, s, k, p, st.T, st.pf, st.dstart, st.sstart, base, count_n,
                   act, st.nsact, ovf);
    else
        TSG_LAUNCH((k_bdy32<DIM, false, 0, SH>), nb, st.tpb, s, k, p, st.T, st.pf, st.dstart, st.sstart, base, count_n,
                   act, st.nsact, ovf);
    TSG_LAUNCH((k_bdy32<DIM, true, -1, SH>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, base, count_n, act,
               st.nsact, ovf);
}

template <int DIM, bool CORR, int KT, bool FL>
void rates_main(Fp32State& st, const P32& p, cudaStream_t s, const Ovf& ovf) {
    const K32& k = st.k;
    const int nb = nblk(k.nd, st.tpb);
    if (k.boundary == 3 || k.boundary == 4)
        TSG_LAUNCH((k_rates32<DIM, false, CORR, KT, 1, FL>), nb, st.tpb, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
    else
        TSG_LAUNCH((k_rates32<DIM, false, CORR, KT, 0, FL>), nb, st.tpb, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
}

template <int DIM, bool CORR, bool FL = false>
void rates_launch(Fp32State& st, const P32& p, cudaStream_t s, const Ovf& ovf) {
    const K32& k = st.k;
    if (k.kernel == 1) rates_main<DIM, CORR, 1, FL>(st, p, s, ovf);
    else rates_main<DIM, CORR, 0, FL>(st, p, s, ovf);
    TSG_LAUNCH((k_rates32<DIM, true, CORR, -1, -1, FL>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
}

static void kernel_corr(Fp32State& st, cudaStream_t s, bool skip_fluid, bool skip_static) {
    PhaseScope ph(s, PH_CORR);
    const K32& k = st.k;
    const Ovf ovf{st.ovf_list, st.novf};
    if (k.dim == 2) corr_launch<2>(st, s, ovf, skip_fluid, skip_static);
    else corr_launch<3>(st, s, ovf, skip_fluid, skip_static);
}

void fp32_kernel_corr(Fp32State& st, cudaStream_t s) { kernel_corr(st, s, false, false); }

void fp32_init_tmp(Fp32State& st, cudaStream_t s) {
    PhaseScope ph(s, PH_INIT);
    TSG_LAUNCH(k_init_tmp32<false>, nblk(st.k.nd), TPB, s, st.k, st.P[st.cur], st.T);
}

// mu(I) / Drucker-Prager one_step (eng/solver_sph_muI.py:62-131, eng/solver_sph_dp.py:210-274).
template <int DIM>
void soil_one_step(Fp32State& st, cudaStream_t s) {
    const K32& k = st.k;
    P32& p = st.P[st.cur];
    const Ovf ovf{st.ovf_list, st.novf};
    const int nb = nblk(k.nd, st.tpb);
    {
        PhaseScope ph(s, PH_PRE);
        if (k.solver == 2) {
            if (k.corr) { TSG_LAUNCH((k_mui_stress32<DIM, false, true>), nb, st.tpb, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
                          TSG_LAUNCH((k_mui_stress32<DIM, true, true>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf); }
            else { TSG_LAUNCH((k_mui_stress32<DIM, false, false>), nb, st.tpb, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
                   TSG_LAUNCH((k_mui_stress32<DIM, true, false>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf); }
        } else {
            TSG_LAUNCH(k_pre_dp32, nblk(k.nd), TPB, s, k, p, st.T);
        }
    }
    {
        PhaseScope ph(s, PH_BDY);
        auto bdy = [&](int base, int count_n) {
            if (count_n <= 0) return;
            TSG_LAUNCH((k_bdy_soil32<DIM, false>), nblk(count_n, st.tpb), st.tpb, s, k, p, st.T, st.pf, st.dstart, st.sstart, base, count_n, ovf);
            TSG_LAUNCH((k_bdy_soil32<DIM, true>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, base, count_n, ovf);
        };
        bdy(k.nd, k.n - k.nd);
        if (st.c.n_bdy > k.n - k.nd) bdy(0, k.nd);
    }
    {
        PhaseScope ph(s, PH_RATES);
        TSG_LAUNCH(k_pack_stress32<DIM>, nblk(k.n), TPB, s, k, st.T);
#define SOIL_MOM(CORR, DP)                                                                                       \
        do {                                                                                                     \
            TSG_LAUNCH((k_soil_mom32<DIM, false, CORR, DP>), nb, st.tpb, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf); \
            TSG_LAUNCH((k_soil_mom32<DIM, true, CORR, DP>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);  \
        } while (0)
        if (k.solver == 2) { if (k.corr) SOIL_MOM(true, false); else SOIL_MOM(false, false); }
        else { if (k.corr) SOIL_MOM(true, true); else SOIL_MOM(false, true); }
#undef SOIL_MOM
    }
}

// eos = false: the fluid pressures were computed by the kernel before (the step sequence
// fuses them into init_real2tmp and the leap-frog half step).  fl: the rates pass computes
// the fluid's CSPM factors (the correction kernel of the step skipped them); sh: the
// boundary pass computes the static block's Shepard factors (no correction kernel ran).
static void one_step(Fp32State& st, cudaStream_t s, bool eos, bool fl = false, bool sh = false) {
    const K32& k = st.k;
    P32& p = st.P[st.cur];
    if (k.solver != 1) {
        if (k.dim == 2) soil_one_step<2>(st, s);
        else soil_one_step<3>(st, s);
        return;
    }
    if (eos) {
        PhaseScope ph(s, PH_PRE);
        TSG_LAUNCH(k_pre32, nblk(k.nd), TPB, s, k, p, st.T);
    }
    {
        PhaseScope ph(s, PH_BDY);
        const Ovf ovf{st.ovf_list, st.novf};
        auto bdy = [&](int base, int count_n, bool shep) {
            if (count_n <= 0) return;
            if (shep) {
                if (k.dim == 2) bdy_launch<2, true>(st, p, base, count_n, s, ovf);
                else bdy_launch<3, true>(st, p, base, count_n, s, ovf);
            } else {
                if (k.dim == 2) bdy_launch<2, false>(st, p, base, count_n, s, ovf);
                else bdy_launch<3, false>(st, p, base, count_n, s, ovf);
            }
        };
        bdy(k.nd, k.n - k.nd, sh);
        if (st.c.n_bdy > k.n - k.nd) bdy(0, k.nd, false);  // kinematic rigid particles live in the dynamic block
    }
    {
        PhaseScope ph(s, PH_RATES);
        const Ovf ovf{st.ovf_list, st.novf};
        if (fl) {
            if (k.dim == 2) { if (k.corr) rates_launch<2, true, true>(st, p, s, ovf); else rates_launch<2, false, true>(st, p, s, ovf); }
            else { if (k.corr) rates_launch<3, true, true>(st, p, s, ovf); else rates_launch<3, false, true>(st, p, s, ovf); }
        } else if (k.dim == 2) { if (k.corr) rates_launch<2, true>(st, p, s, ovf); else rates_launch<2, false>(st, p, s, ovf); }
        else { if (k.corr) rates_launch<3, true>(st, p, s, ovf); else rates_launch<3, false>(st, p, s, ovf); }
        if (st.rnobj) {  // the fluid's reaction on dynamic rigid particles, after the rates pass
            if (k.dim == 2) TSG_LAUNCH(k_rigid_reaction32<2>, nblk(k.nd), TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart);
            else TSG_LAUNCH(k_rigid_reaction32<3>, nblk(k.nd), TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart);
        }
    }
}

void fp32_one_step(Fp32State& st, cudaStream_t s) { one_step(st, s, true); }

// advect_pos with XSPH (eng/solver_sph_base.py:224-238); post: with the WCSPH density clamp
// of advect_something fused in (the step sequence).
static void advect_pos(Fp32State& st, cudaStream_t s, bool post) {
    const K32& k = st.k;
    P32& p = st.P[st.cur];
    PhaseScope ph(s, PH_POS);
    if (k.xsph) {
        const Ovf ovf{st.ovf_list, st.novf};
        if (k.dim == 2) {
            TSG_LAUNCH((k_xsph32<2, false>), nblk(k.nd, st.tpb), st.tpb, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
            TSG_LAUNCH((k_xsph32<2, true>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
        } else {
            TSG_LAUNCH((k_xsph32<3, false>), nblk(k.nd, st.tpb), st.tpb, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
            TSG_LAUNCH((k_xsph32<3, true>), 64, TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, ovf);
        }
    }
    if (post) TSG_LAUNCH(k_advect_pos32<true>, nblk(k.nd), TPB, s, k, p, st.T, st.err);
    else TSG_LAUNCH(k_advect_pos32<false>, nblk(k.nd), TPB, s, k, p, st.T, st.err);
    if (k.disp2_limit <= 0.f) st.lists_valid = false;
}

void fp32_advect(Fp32State& st, int which, cudaStream_t s) {
    const K32& k = st.k;
    P32& p = st.P[st.cur];
    switch (which) {
    case TSG_ADVECT_FULL: { PhaseScope ph(s, PH_INTEGRATE); TSG_LAUNCH(k_advect_full32, nblk(k.nd), TPB, s, k, p, st.T, st.err); break; }
    case TSG_ADVECT_LF_HALF: { PhaseScope ph(s, PH_INTEGRATE); TSG_LAUNCH(k_advect_half32<false>, nblk(k.nd), TPB, s, k, p, st.T); break; }
    case TSG_ADVECT_POS: advect_pos(st, s, false); break;
    case TSG_ADVECT_SOMETHING: {
        PhaseScope ph(s, PH_POST);
        if (k.solver == 1) TSG_LAUNCH(k_post_wc32, nblk(k.nd), TPB, s, k, p);
        else if (k.solver == 2) {
            TSG_LAUNCH(k_post_mui32, nblk(k.nd), TPB, s, k, p, st.T);
            // the regularisation reads the lists while no particle has moved more than 0.49
            // skin since their build ((0.49 / 0.45)^2 = 1.1857 times the rebuild threshold),
            // measured here from the moved positions (the next step's check finds the same)
            float list_d2 = -1.f;
            if (st.lists_valid && k.disp2_limit > 0.f) {
                TSG_LAUNCH(k_disp32, nblk(k.nd), TPB, s, k, p.hi, p.lo, st.pf, st.maxdisp);
                list_d2 = k.disp2_limit * 1.185f;
            }
            if (k.dim == 2)
                TSG_LAUNCH(k_reg_mui32<2>, nblk(k.nd), TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, st.maxdisp,
                           list_d2);
            else
                TSG_LAUNCH(k_reg_mui32<3>, nblk(k.nd), TPB, s, k, p, st.T, st.pf, st.dstart, st.sstart, st.maxdisp,
                           list_d2);
        } else TSG_LAUNCH(k_post_dp32, nblk(k.nd), TPB, s, k, p, st.T);
        break;
    }
    case TSG_ENFORCE_BOUNDARY: { PhaseScope ph(s, PH_OTHER); TSG_LAUNCH(k_enforce32, nblk(k.nd), TPB, s, k, p); break; }
    case TSG_RK_INIT: { PhaseScope ph(s, PH_INTEGRATE); TSG_LAUNCH(k_rk_init32, nblk(k.nd), TPB, s, k, p, st.T); break; }
    case TSG_RK_STAGE: { PhaseScope ph(s, PH_INTEGRATE); TSG_LAUNCH(k_rk_stage32, nblk(k.nd), TPB, s, k, p, st.T); break; }
    case TSG_RK_FINAL: { PhaseScope ph(s, PH_INTEGRATE); TSG_LAUNCH(k_rk_final32, nblk(k.nd), TPB, s, k, p, st.T, st.err); break; }
    default: break;
    }
}

void fp32_rk_update(Fp32State& st, int m, cudaStream_t s) {
    PhaseScope ph(s, PH_INTEGRATE);
    TSG_LAUNCH(k_rk_update32, nblk(st.k.nd), TPB, s, st.k, st.P[st.cur], st.T, (float)m);
}

// ---------------------------------------------------------------- captured steps
// One SPHBase.step() after the (conditional) re-sort: kernel correction, init_real2tmp,
// the integrator's one_step / advect sequence, advect_pos, advect_something and, in
// collision mode, enforce_boundary (eng/solver_sph_base.py:41-61, :79-120).
// fold_disp: the fused final update folds the new positions into the displacement maximum
// (the next step, captured in the same graph, skips its list-expiry check).
void f32::step_body(Fp32State& st, cudaStream_t s, bool collide, bool fold_disp) {
    // WCSPH with symplectic Euler or leap-frog: the fluid EOS (first phase of each one_step)
    // runs inside init_real2tmp and the half step, which produce its input density_tmp
    const bool fuse = st.k.solver == 1 && st.c.ti != 4;
    // The fluid's CSPM factors come from the first rates pass (positions stay fixed through
    // the step, so a second pass reads them back), except with symplectic Euler and CSPM,
    // whose single pass updates the density from the continuity sum and so keeps the
    // compensated per-neighbour form; and when the dynamic block holds fluid only, the
    // static block's Shepard factors come from the first boundary pass.  With both, the
    // correction kernel has nothing left to do.
    const bool fuse_corr = fuse && (st.c.ti == 2 || st.k.corr == 0);
    const bool fuse_shep = fuse && st.c.n_bdy <= st.k.n - st.k.nd;
    if (!(fuse_corr && fuse_shep)) kernel_corr(st, s, fuse_corr, fuse_shep);
    if (fuse) {
        PhaseScope ph(s, PH_INIT);
        TSG_LAUNCH(k_init_tmp32<true>, nblk(st.k.nd), TPB, s, st.k, st.P[st.cur], st.T);
    } else {
        fp32_init_tmp(st, s);
    }
    if (st.c.ti == 4) {
        fp32_advect(st, TSG_RK_INIT, s);
        const int m[4] = {1, 2, 2, 1};
        for (int q = 0; q < 4; ++q) {
            fp32_one_step(st, s);
            fp32_rk_update(st, m[q], s);
            if (q < 3) fp32_advect(st, TSG_RK_STAGE, s);
        }
        fp32_advect(st, TSG_RK_FINAL, s);
    } else {
        one_step(st, s, !fuse, fuse_corr, fuse_shep);
        if (st.c.ti == 2) {
            if (fuse) {
                PhaseScope ph(s, PH_INTEGRATE);
                TSG_LAUNCH(k_advect_half32<true>, nblk(st.k.nd), TPB, s, st.k, st.P[st.cur], st.T);
            } else {
                fp32_advect(st, TSG_ADVECT_LF_HALF, s);
            }
            one_step(st, s, !fuse);
        }
        if (fuse && !st.k.xsph) {  // advect_SE / _LF, advect_pos and the WCSPH clamp at once
            PhaseScope ph(s, PH_INTEGRATE);
            TSG_LAUNCH(k_advect_final_wc32, nblk(st.k.nd), TPB, s, st.k, st.P[st.cur], st.T, st.err, st.pf,
                       fold_disp ? st.maxdisp : nullptr);
            if (st.k.disp2_limit <= 0.f) st.lists_valid = false;
            fp32_solve_rigid(st, s);
            if (collide || st.rnobj) fp32_advect(st, TSG_ENFORCE_BOUNDARY, s);
            return;
        }
        fp32_advect(st, TSG_ADVECT_FULL, s);
    }
    if (st.k.solver == 1) {
        advect_pos(st, s, true);  // advect_something of WCSPH is the density clamp, fused
    } else {
        advect_pos(st, s, false);
        fp32_advect(st, TSG_ADVECT_SOMETHING, s);
    }
    fp32_solve_rigid(st, s);
    if (collide || st.rnobj) fp32_advect(st, TSG_ENFORCE_BOUNDARY, s);
}

void fp32_solve_rigid(Fp32State& st, cudaStream_t s) {
    if (st.rnobj == 0) return;
    PhaseScope ph(s, PH_POS);
    const auto& p = st.P[st.cur];
    build_rigid_lists(st.k.nd, st.rnobj, RigidSlot32{p.hi, p.ids, st.r_ids, st.rnobj}, st.r_scratch, st.r_off,
                      st.r_list, s);
    const dim3 g(st.r_chunks, st.rnobj);
    TSG_LAUNCH(k_rigid_part32<0>, g, kRigidBlock, s, st.k, p, st.r_off, st.r_list, st.r_q, st.r_cm, st.r_part);
    TSG_LAUNCH(k_rigid_reduce32<0>, st.rnobj, kRigidBlock, s, st.r_off, st.r_chunks, st.r_part, st.r_cm, st.r_rot);
    TSG_LAUNCH(k_rigid_part32<1>, g, kRigidBlock, s, st.k, p, st.r_off, st.r_list, st.r_q, st.r_cm, st.r_part);
    TSG_LAUNCH(k_rigid_reduce32<1>, st.rnobj, kRigidBlock, s, st.r_off, st.r_chunks, st.r_part, st.r_cm, st.r_rot);
    TSG_LAUNCH(k_rigid_move32, g, kRigidBlock, s, st.k, p, st.r_off, st.r_list, st.r_q, st.r_cm, st.r_rot);
}

void fp32_step_body(Fp32State& st, bool collide, cudaStream_t s) { f32::step_body(st, s, collide); }

namespace {

// Fold the device rebuild counter into the host counters (synchronises s).
void fold_rebuilds(Fp32State& st, cudaStream_t s) {
    int n = 0;
    cudaMemcpyAsync(&n, st.d_rebuilds, sizeof n, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    const int delta = n - st.rebuilds_seen;
    if (delta > 0) {
        st.rebuilds += delta;
        add_launches((long long)delta * st.body_kernels);
        st.rebuilds_seen = n;
    }
}

// Capture `steps` steps into one executable graph.  Each step: displacement check, then an
// Whether step_body ends with the fused final update (which folds the new positions into
// the displacement maximum) and moves no particle after it.
bool folds_disp(const Fp32State& st, bool collide) {
    // (shape matching and the boundary clamp move particles after the fused update)
    return st.k.solver == 1 && st.c.ti != 4 && !st.k.xsph && !collide && st.rnobj == 0 && st.k.disp2_limit > 0.f;
}

// IF node whose body re-sorts in place and rebuilds the lists, then the step body.
int capture_steps(Fp32State& st, int steps, bool collide, Fp32State::StepGraph& g) {
    cudaStream_t cs = nullptr, bs = nullptr;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return TSG_E_CUDA;
    if (cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking) != cudaSuccess) { cudaStreamDestroy(cs); return TSG_E_CUDA; }
    const K32& k = st.k;
    const long long c0 = launch_total();
    long long body = 0;
    int rc = 0;
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed) != cudaSuccess) rc = TSG_E_CUDA;
    for (int q = 0; q < steps && !rc; ++q) {
        cudaStreamCaptureStatus status;
        cudaGraph_t cg = nullptr;
        if (cudaStreamGetCaptureInfo(cs, &status, nullptr, &cg) != cudaSuccess || !cg) { rc = TSG_E_CUDA; break; }
        cudaGraphConditionalHandle hnd;
        if (cudaGraphConditionalHandleCreate(&hnd, cg, 0, cudaGraphCondAssignDefault) != cudaSuccess) { rc = TSG_E_CUDA; break; }
        P32& p = st.P[st.cur];
        // after the first step of the graph, the previous step's fused final update has folded
        // its new positions into the displacement maximum already
        if (q == 0 || !folds_disp(st, collide))
            TSG_LAUNCH(k_disp32, nblk(k.nd), TPB, cs, k, p.hi, p.lo, st.pf, st.maxdisp);
        TSG_LAUNCH(k_set_rebuild32, 1, 1, cs, hnd, st.maxdisp, k.disp2_limit, st.d_rebuilds);
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        if (cudaStreamGetCaptureInfo(cs, &status, nullptr, &cg, &deps, nullptr, &ndeps) != cudaSuccess) { rc = TSG_E_CUDA; break; }
        // (the union inside has no default constructor: zeroed storage, then fields)
        alignas(cudaGraphNodeParams) unsigned char cp_buf[sizeof(cudaGraphNodeParams)];
        std::memset(cp_buf, 0, sizeof cp_buf);
        cudaGraphNodeParams& cp = *reinterpret_cast<cudaGraphNodeParams*>(cp_buf);
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = hnd;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        if (cudaGraphAddNode(&node, cg, deps, nullptr, ndeps, &cp) != cudaSuccess) { rc = TSG_E_CUDA; break; }
        cudaGraph_t bodyg = cp.conditional.phGraph_out[0];
        if (cudaStreamUpdateCaptureDependencies(cs, &node, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess) {
            rc = TSG_E_CUDA;
            break;
        }
        const long long b0 = launch_total();
        if (cudaStreamBeginCaptureToGraph(bs, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
            rc = TSG_E_CUDA;
            break;
        }
        rebuild(st, bs, true);
        cudaGraph_t done = nullptr;
        if (cudaStreamEndCapture(bs, &done) != cudaSuccess) { rc = TSG_E_CUDA; break; }
        body = launch_total() - b0;
        step_body(st, cs, collide, q + 1 < steps && folds_disp(st, collide));
    }
    cudaError_t e = cudaStreamEndCapture(cs, &graph);
    if (!rc && (e != cudaSuccess || !graph)) rc = TSG_E_CUDA;
    const long long captured = launch_total() - c0;
    add_launches(-captured);  // nodes, not launches
    if (!rc) {
        if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
        if (cudaGraphInstantiate(&g.exec, graph, 0) != cudaSuccess) { rc = TSG_E_CUDA; g.exec = nullptr; }
    }
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(bs);
    cudaStreamDestroy(cs);
    cudaGetLastError();
    if (rc) return rc;
    g.steps = steps;
    g.cur = st.cur;
    g.tpb = st.tpb;
    g.cpc = st.cells_per_cta;
    g.collide = collide;
    g.kernels = captured - body * steps;
    st.body_kernels = body;
    return 0;
}

Fp32State::StepGraph* graph_for(Fp32State& st, int steps, bool collide, int* rc) {
    Fp32State::StepGraph& g = st.graphs[steps == 1 ? 0 : 1];
    *rc = 0;
    if (g.exec && g.steps == steps && g.cur == st.cur && g.tpb == st.tpb && g.cpc == st.cells_per_cta &&
        g.collide == collide)
        return &g;
    *rc = capture_steps(st, steps, collide, g);
    return *rc ? nullptr : &g;
}

}  // namespace

int fp32_step_graph(Fp32State& st, int nsteps, bool collide, cudaStream_t s) {
    if (profiling_on()) return TSG_E_STATE;  // per-phase events need the eager path
    if (!st.built) fp32_sort(st, s);
    const int K = st.steps_per_graph > 1 ? st.steps_per_graph : 1;
    int rc = 0;
    while (nsteps > 0) {
        const int take = (K > 1 && nsteps >= K) ? K : 1;
        Fp32State::StepGraph* g = graph_for(st, take, collide, &rc);
        if (!g) return rc;
        if (cudaGraphLaunch(g->exec, s) != cudaSuccess) return TSG_E_CUDA;
        add_launches(g->kernels);
        nsteps -= take;
    }
    st.lists_valid = st.k.disp2_limit > 0.f;
    return 0;
}

void fp32_flush_counters(Fp32State& st, cudaStream_t s) { fold_rebuilds(st, s); }

void fp32_get_launch(const Fp32State& st, int* tpb, int* cpc, int* spg) {
    *tpb = st.tpb;
    *cpc = st.cells_per_cta;
    *spg = st.steps_per_graph;
}

int fp32_set_launch(Fp32State& st, int tpb, int cpc, int spg) {
    if (tpb != 64 && tpb != 128 && tpb != 256) return TSG_E_ARG;  // kernels are bounded for 256
    if (cpc != 0 && cpc != 2 && cpc != 4 && cpc != 8) return TSG_E_ARG;
    if (spg < 1 || spg > 64) return TSG_E_ARG;
    st.tpb = tpb;
    st.cells_per_cta = cpc;
    st.steps_per_graph = spg;
    return 0;
}

// ---------------------------------------------------------------- autotuner
namespace {

// Particle state that carries from one step to the next: the current buffer of every
// persistent array and the boundary particles' v_tmp (the mu(I) first loop reads the
// previous step's extrapolated boundary velocity).
std::vector<std::pair<void*, size_t>> snap_items(Fp32State& st) {
    const size_t n = st.n;
    P32& p = st.P[st.cur];
    std::vector<std::pair<void*, size_t>> v = {
        {p.hi, sizeof(float4) * n}, {p.lo.p, sizeof(float4) * 2 * n}, {p.vel, sizeof(float4) * n},
        {p.drho, sizeof(float) * n}, {p.mass, sizeof(float) * n}, {p.ids, sizeof(int4) * n}};
    // (v_tmp, which the mu(I) first loop reads from the previous step for boundary particles,
    // travels in the second half of the lo records)
    if (p.sig) {
        v.push_back({p.sig, sizeof(float) * 6 * n});
        v.push_back({p.eeq, sizeof(float) * n});
        v.push_back({p.eeqp, sizeof(float) * n});
        v.push_back({p.flag, sizeof(int) * n});
    }
    if (p.vlo) v.push_back({p.vlo, sizeof(float4) * n});
    return v;
}

size_t snap_bytes(Fp32State& st) {
    size_t total = 0;
    for (auto& it : snap_items(st)) total += (it.second + 255) & ~size_t(255);
    return total;
}

void snap_copy(Fp32State& st, void* buf, bool restore, cudaStream_t s) {
    char* q = static_cast<char*>(buf);
    for (auto& it : snap_items(st)) {
        if (restore) cudaMemcpyAsync(it.first, q, it.second, cudaMemcpyDeviceToDevice, s);
        else cudaMemcpyAsync(q, it.first, it.second, cudaMemcpyDeviceToDevice, s);
        q += (it.second + 255) & ~size_t(255);
    }
}

int snapshot(Fp32State& st, cudaStream_t s, bool restore) {
    if (!restore && !st.snap && cudaMalloc(&st.snap, snap_bytes(st)) != cudaSuccess) {
        st.snap = nullptr;
        return TSG_E_CUDA;
    }
    snap_copy(st, st.snap, restore, s);
    return 0;
}

// Milliseconds per step of `steps` steps from the snapshot state (graph mode).
float time_steps(Fp32State& st, int steps, bool collide, cudaStream_t s, int* rc) {
    snapshot(st, s, true);
    rebuild(st, s, true);
    *rc = fp32_step_graph(st, 1, collide, s);  // captures the graphs outside the timed region
    if (st.steps_per_graph > 1 && !*rc) *rc = fp32_step_graph(st, st.steps_per_graph, collide, s);
    if (*rc) return 1e30f;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
    *rc = fp32_step_graph(st, steps, collide, s);
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return *rc ? 1e30f : ms / steps;
}

// Milliseconds of one re-sort + list build from the snapshot state.
float time_rebuild(Fp32State& st, cudaStream_t s) {
    snapshot(st, s, true);
    rebuild(st, s, true);  // warm
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
    for (int q = 0; q < 3; ++q) rebuild(st, s, true);
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms / 3.f;
}

}  // namespace

size_t fp32_snapshot_bytes(Fp32State& st) { return snap_bytes(st); }

int fp32_snapshot_copy(Fp32State& st, void* buf, bool load, cudaStream_t s) {
    if (!buf) return TSG_E_ARG;
    snap_copy(st, buf, load, s);
    if (load) {
        st.built = false;  // the next step re-sorts the loaded particles before anything else
        st.lists_valid = false;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : TSG_E_CUDA;
}

void fp32_set_soil(Fp32State& st, const Consts& c) {
    K32& k = st.k;
    k.mu = (float)c.mu; k.coh = (float)c.coh; k.alpha = (float)c.alpha; k.k_c = (float)c.k_c;
    k.kc_over_alpha = (float)c.kc_over_alpha; k.lam_den = (float)c.lam_den; k.three_aK = (float)c.three_aK;
    for (auto& g : st.graphs)
        if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
}

void fp32_set_fluid(Fp32State& st, const Consts& c) {
    st.k.B = (float)c.B;
    st.k.visc_fac = (float)c.visc_fac;
    for (auto& g : st.graphs)  // the captured launches hold the constants by value
        if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
}

// Coordinate search over the launch parameters, each candidate timed from the same saved
// state: threads per block of the neighbour kernels (full steps), cells per CTA of the
// list build (re-sort + build), steps per graph launch (full steps).  The state is put
// back afterwards, so tuning does not advance the simulation.
int fp32_autotune(Fp32State& st, int trial_steps, bool collide, cudaStream_t s, float* ms_out) {
    if (trial_steps < 1) return TSG_E_ARG;
    if (profiling_on()) return TSG_E_STATE;
    if (!st.built) fp32_sort(st, s);
    fold_rebuilds(st, s);
    const long long launches0 = launch_total();
    const long long rebuilds0 = st.rebuilds;
    int rc = snapshot(st, s, false);
    if (rc) return rc;
    const int tpbs[] = {64, 128, 256};
    const int cpcs3[] = {2, 4, 8}, cpcs2[] = {0, 2, 4, 8};
    const int spgs[] = {1, 4, 16};
    float best = 1e30f;
    int bt = st.tpb;
    for (int t : tpbs) {
        st.tpb = t;
        const float ms = time_steps(st, trial_steps, collide, s, &rc);
        if (rc) break;
        if (ms < best) { best = ms; bt = t; }
    }
    st.tpb = bt;
    if (!rc) {
        float bestr = 1e30f;
        int bc = st.cells_per_cta;
        const int* cp = st.k.dim == 3 ? cpcs3 : cpcs2;
        const int ncp = st.k.dim == 3 ? 3 : 4;
        for (int q = 0; q < ncp; ++q) {
            st.cells_per_cta = cp[q];
            const float ms = time_rebuild(st, s);
            if (ms < bestr) { bestr = ms; bc = cp[q]; }
        }
        st.cells_per_cta = bc;
    }
    if (!rc) {
        int bs = st.steps_per_graph;
        best = 1e30f;
        for (int k : spgs) {
            st.steps_per_graph = k;
            const float ms = time_steps(st, trial_steps < k ? k : trial_steps, collide, s, &rc);
            if (rc) break;
            if (ms < best) { best = ms; bs = k; }
        }
        st.steps_per_graph = bs;
    }
    snapshot(st, s, true);
    rebuild(st, s, true);
    cudaStreamSynchronize(s);
    cudaFree(st.snap);
    st.snap = nullptr;
    // tuning steps are not simulation steps: take their launches and rebuilds back out
    fold_rebuilds(st, s);
    add_launches(launches0 - launch_total());
    st.rebuilds = rebuilds0;
    if (ms_out) *ms_out = best;
    return rc ? rc : (cudaGetLastError() == cudaSuccess ? 0 : TSG_E_CUDA);
}

namespace {
// Float field code of k_export for a name this state keeps (-1: integer field or unknown).
int fp32_float_field(Fp32State& st, const char* name) {
    static const char* names[] = {"x", "v", "density", "pressure", "m_V", "mass", "v_tmp", "density_tmp",
                                  "d_density", "d_vel", "CSPM_f", "CSPM_L", "stress", "stress_tmp", "d_stress",
                                  "strain_equ", "strain_equ_p", "d_strain_equ", "d_strain_equ_p"};
    for (int q = 0; q < (int)(sizeof(names) / sizeof(names[0])); ++q) {
        if (std::strcmp(name, names[q]) != 0) continue;
        if (q == 11 && !st.T.L) return -1;
        if (q >= 12 && !st.P[0].sig) return -1;
        if ((q == 14 || q == 16 || q == 18) && !st.T.dsig) return -1;
        return q;
    }
    return -1;
}
int fp32_field_comps(int what) { return (what == 0 || what == 1 || what == 6 || what == 9) ? 3 : (what == 11 || (what >= 12 && what <= 14)) ? 9 : 1; }
}  // namespace

int fp32_field(Fp32State& st, const char* name, tsg_view* out, cudaStream_t s) {
    const std::string f(name);
    struct Spec { const char* nm; int what; int comps; int is_int; };
    static const Spec specs[] = {
        {"x", 0, 3, 0}, {"v", 1, 3, 0}, {"density", 2, 1, 0}, {"pressure", 3, 1, 0}, {"m_V", 4, 1, 0},
        {"mass", 5, 1, 0}, {"v_tmp", 6, 3, 0}, {"density_tmp", 7, 1, 0}, {"d_density", 8, 1, 0},
        {"d_vel", 9, 3, 0}, {"CSPM_f", 10, 1, 0}, {"CSPM_L", 11, 9, 0},
        {"stress", 12, 9, 0}, {"stress_tmp", 13, 9, 0}, {"d_stress", 14, 9, 0}, {"strain_equ", 15, 1, 0},
        {"strain_equ_p", 16, 1, 0}, {"d_strain_equ", 17, 1, 0}, {"d_strain_equ_p", 18, 1, 0},
        {"id0", 0, 1, 1}, {"mat_type", 1, 1, 1}, {"mat_id", 2, 1, 1}, {"obj_id", 3, 1, 1}, {"is_dynamic", 4, 1, 1},
        {"flag_retmap", 5, 1, 1}};
    const Spec* sp = nullptr;
    for (const Spec& x : specs) if (f == x.nm) sp = &x;
    if (!sp) return TSG_E_NAME;
    if (sp->what == 11 && !st.T.L) return TSG_E_NAME;
    const bool soil = st.P[0].sig != nullptr, dp = st.T.dsig != nullptr;
    if (!sp->is_int && sp->what >= 12 && !soil) return TSG_E_NAME;
    if (!sp->is_int && (sp->what == 14 || sp->what == 16 || sp->what == 18) && !dp) return TSG_E_NAME;
    if (sp->is_int && sp->what == 5 && !dp) return TSG_E_NAME;
    double* buf = nullptr;
    for (auto& v : st.views) if (v.first == f) buf = v.second;
    if (!buf) {
        buf = dal<double>(st, (size_t)sp->comps * st.n);
        if (!buf) return TSG_E_CUDA;
        st.views.push_back({f, buf});
    }
    if (sp->is_int) TSG_LAUNCH(k_export_int, nblk(st.n), TPB, s, st.k, st.P[st.cur], sp->what, reinterpret_cast<int*>(buf));
    else TSG_LAUNCH(k_export, nblk(st.n), TPB, s, st.k, st.P[st.cur], st.T, sp->what, buf, (size_t)st.n, (size_t)1);
    const int64_t n = st.n;
    out->data = buf;
    out->dtype = sp->is_int ? 2 : 0;
    if (sp->comps == 1) { out->ndim = 1; out->shape[0] = n; out->strides[0] = 1; }
    else if (sp->comps == 3) { out->ndim = 2; out->shape[0] = n; out->shape[1] = 3; out->strides[0] = 1; out->strides[1] = n; }
    else { out->ndim = 3; out->shape[0] = n; out->shape[1] = 3; out->shape[2] = 3; out->strides[0] = 1; out->strides[1] = 3 * n; out->strides[2] = n; }
    return cudaGetLastError() == cudaSuccess ? 0 : TSG_E_CUDA;
}

const int* fp32_cell_start(const Fp32State& st) { return st.dstart; }

void fp32_density_sum(Fp32State& st, double* out, cudaStream_t s) {
    PhaseScope ph(s, PH_OTHER);
    if (!st.built) fp32_sort(st, s);
    if (st.k.dim == 2)
        TSG_LAUNCH(k_density_sum32<2>, nblk(st.n), TPB, s, st.k, st.P[st.cur], st.pf, st.dstart, st.sstart, out);
    else
        TSG_LAUNCH(k_density_sum32<3>, nblk(st.n), TPB, s, st.k, st.P[st.cur], st.pf, st.dstart, st.sstart, out);
}

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

// Device address of a host buffer the GPU can read and write in place (page-locked host
// memory: under unified addressing every page-locked allocation is mapped), else null.
// Field transfers through such a buffer convert on the fly in one kernel pass over the
// host link, with no staging copy.
static void* mapped_host(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int fp32_write(Fp32State& st, const char* name, const void* src, bool from_device, cudaStream_t s) {
    const std::string f(name);
    int what = -1, comps = 1;
    if (f == "x") { what = 0; comps = 3; }
    else if (f == "v") { what = 1; comps = 3; }
    else if (f == "density") what = 2;
    else if (f == "pressure") what = 3;
    else return TSG_E_NAME;
    const size_t n = st.n;
    const double* in = from_device ? nullptr : static_cast<const double*>(mapped_host(src));
    if (!in) {
        cudaMemcpyAsync(st.stage, src, sizeof(double) * comps * n,
                        from_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s);
        in = st.stage;
    }
    TSG_LAUNCH(k_import, nblk(n), TPB, s, st.k, st.P[st.cur], what, in);
    if (what == 0) st.lists_valid = false;
    // boundary particles without flow neighbours: their extrapolated state follows an
    // imported velocity / pressure at once (it is otherwise written at list builds only)
    if (st.built && (what == 1 || what == 3)) static_active(st, s);
    return cudaGetLastError() == cudaSuccess ? 0 : TSG_E_CUDA;
}

// The copy stream and events of the chunked export, created on first use.
static bool export_pipe(Fp32State& st) {
    if (st.copy_stream) return true;
    if (cudaStreamCreateWithFlags(&st.copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
        st.copy_stream = nullptr;
        return false;
    }
    for (auto& e : st.copy_ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return false;
    return true;
}

int fp32_read_set(Fp32State& st, int count, const char* const* names, void* const* dsts, int mode,
                  cudaStream_t s) {
    if (count <= 0 || count > 8) return TSG_E_ARG;
    const size_t n = st.n;
    ExportSet es{};
    es.count = count;
    size_t total = 0;
    for (int q = 0; q < count; ++q) {
        const int what = fp32_float_field(st, names[q]);
        if (what < 0) return TSG_E_NAME;
        es.what[q] = what;
        es.comps[q] = fp32_field_comps(what);
        es.off[q] = total;
        total += (size_t)es.comps[q] * n;
    }
    if (total > 9 * n) {  // more than the staging holds: one field at a time
        for (int q = 0; q < count; ++q) {
            const int rc = fp32_read(st, names[q], dsts[q], mode == 0 ? 2 : mode, s);
            if (rc) return rc;
        }
    } else if (mode == 1 || !export_pipe(st)) {
        const cudaMemcpyKind kind = mode == 1 ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        TSG_LAUNCH(k_export_set, nblk(n), TPB, s, st.k, st.P[st.cur], st.T, es, st.stage, 0, (int)n);
        for (int q = 0; q < count; ++q)
            cudaMemcpyAsync(dsts[q], st.stage + es.off[q], sizeof(double) * es.comps[q] * n, kind, s);
    } else {
        // host destinations: the conversion runs chunk by chunk on s and each chunk's copies
        // on the copy stream, so the host link (the bound) starts after the first chunk
        constexpr int C = 4;
        for (int c = 0; c < C; ++c) {
            const size_t i0 = n * c / C, i1 = n * (c + 1) / C;
            if (i1 > i0)
                TSG_LAUNCH(k_export_set, nblk(i1 - i0), TPB, s, st.k, st.P[st.cur], st.T, es, st.stage, (int)i0,
                           (int)i1);
            cudaEventRecord(st.copy_ev[c], s);
            cudaStreamWaitEvent(st.copy_stream, st.copy_ev[c], 0);
            for (int q = 0; q < count; ++q) {
                const size_t a = (size_t)es.comps[q] * i0, b = (size_t)es.comps[q] * i1;
                if (b > a)
                    cudaMemcpyAsync(static_cast<double*>(dsts[q]) + a, st.stage + es.off[q] + a,
                                    sizeof(double) * (b - a), cudaMemcpyDeviceToHost, st.copy_stream);
            }
        }
        cudaEventRecord(st.copy_ev[C], st.copy_stream);
        cudaStreamWaitEvent(s, st.copy_ev[C], 0);
    }
    if (mode == 0) cudaStreamSynchronize(s);
    return cudaGetLastError() == cudaSuccess ? 0 : TSG_E_CUDA;
}

int fp32_read(Fp32State& st, const char* name, void* dst, int mode, cudaStream_t s) {
    const size_t n = st.n;
    const cudaMemcpyKind kind = mode == 1 ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const int what = fp32_float_field(st, name);
    if (what >= 0) {  // float fields: export row-major into the destination or staging + one copy
        const int comps = fp32_field_comps(what);
        // (host destinations go through staging and a copy: stores to host memory from the
        // SMs run no faster than the copy engine over the host link)
        double* out = mode == 1 ? static_cast<double*>(dst) : nullptr;
        TSG_LAUNCH(k_export, nblk(n), TPB, s, st.k, st.P[st.cur], st.T, what, out ? out : st.stage, (size_t)1,
                   (size_t)comps);
        if (!out) cudaMemcpyAsync(dst, st.stage, sizeof(double) * n * comps, kind, s);
    } else {
        tsg_view v;
        int rc = fp32_field(st, name, &v, s);
        if (rc) return rc;
        cudaMemcpyAsync(dst, v.data, sizeof(int) * n, kind, s);
    }
    if (mode == 0) cudaStreamSynchronize(s);
    return cudaGetLastError() == cudaSuccess ? 0 : TSG_E_CUDA;
}

}  // namespace tsg

namespace tsg {

int fp32_batch_diag(Fp32State& st, double pitch, double* host_out, int nscenes, cudaStream_t s) {
    if (st.nscenes <= 0 || nscenes != st.nscenes) return TSG_E_ARG;
    double* d = nullptr;
    if (cudaMalloc(&d, sizeof(double) * 8 * (size_t)nscenes) != cudaSuccess) return TSG_E_CUDA;
    std::vector<double> init(8 * (size_t)nscenes, 0.0);
    for (int q = 0; q < nscenes; ++q) init[8 * (size_t)q + 7] = -DBL_MAX;
    cudaMemcpyAsync(d, init.data(), sizeof(double) * init.size(), cudaMemcpyHostToDevice, s);
    TSG_LAUNCH(k_diag_batch32, nblk(st.nd), TPB, s, st.k, st.P[st.cur], pitch, d);
    cudaMemcpyAsync(host_out, d, sizeof(double) * init.size(), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    cudaFree(d);
    return cudaGetLastError() == cudaSuccess ? 0 : TSG_E_CUDA;
}

}  // namespace tsg
