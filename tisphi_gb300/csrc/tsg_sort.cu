// Cell-list build: cell hash, exclusive prefix sum, stable counting sort, SoA reorder.
//
// Reference: ParticleSystem.update_grid_id / PrefixSumExecutor.run / counting_sort
// (eng/particle_system.py:228-257).  The reference sorts an 800-byte struct with an
// atomic_sub in a parallel loop, so its within-cell order is nondeterministic; the serial
// order of that loop is a stable counting sort by cell (ascending old index inside a
// cell).  This file produces exactly that order:
//   k_hash      cell index per particle (truncating cast, eng/particle_system.py:216-226),
//               atomic arrival rank inside the cell;
//   scan        exclusive prefix sum of the G + 1 counts (the extra bin collects
//               particles whose flattened index falls outside [0, G));
//   k_scatter   perm[cell_start + rank] = old index (unstable inside a cell);
//   sort_within_cells (tsg_cellsort.cuh) orders each cell by old index (stable result);
//   k_reorder   gathers every persistent field into the other buffer set, writes the f32
//               prefilter positions and the flow / boundary index lists.
// Compiled with -fmad=false: the f64 cell arithmetic must round exactly like the oracle's.
#include <cstdio>

#include "tsg_cellsort.cuh"
#include "tsg_internal.h"

namespace tsg {

namespace {

constexpr int TPB = 256;

__global__ void k_hash(Consts c, const double* __restrict__ x, int* __restrict__ cell_of,
                       int* __restrict__ rank, int* __restrict__ count, int* __restrict__ err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    long long idx[3];
    bool ok = true;
    for (int d = 0; d < 3; ++d) {
        double t = (x[(size_t)d * c.n + i] - c.vs[d]) / c.grid;
        if (!(fabs(t) < 2147483647.0)) { ok = false; idx[d] = 0; }
        else idx[d] = (long long)(int)t;
    }
    long long f = idx[0] * c.gnum[1] * c.gnum[2] + idx[1] * c.gnum[2] + idx[2];
    if (!ok || f < 0 || f >= c.G) {
        f = c.G;
        atomicOr(err, ok ? TSG_ERR_CELL_OOB : (TSG_ERR_CELL_OOB | TSG_ERR_NONFINITE));
    }
    cell_of[i] = (int)f;
    rank[i] = atomicAdd(&count[f], 1);
}

// ---- three-phase exclusive scan (tile sums, scan of sums, tile rescan) ----
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = TPB * SCAN_ITEMS;

__device__ __forceinline__ int warp_incl_scan(int v) {
    const unsigned lane = threadIdx.x & 31u;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= (unsigned)o) v += y;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; every thread receives the total.
__device__ __forceinline__ int block_excl_scan(int v, int& total) {
    __shared__ int warp_sums[TPB / 32];
    __shared__ int s_total;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = warp_incl_scan(v);
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int w = lane < TPB / 32 ? warp_sums[lane] : 0;
        int wi = warp_incl_scan(w);
        if (lane < TPB / 32) warp_sums[lane] = wi - w;
        if (lane == TPB / 32 - 1) s_total = wi;
    }
    __syncthreads();
    int r = incl - v + warp_sums[wid];
    total = s_total;
    __syncthreads();
    return r;
}

__global__ void k_tile_sums(const int* __restrict__ in, int n, int* __restrict__ tile_sum) {
    __shared__ int red[TPB / 32];
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int s = 0;
    for (int k = 0; k < SCAN_ITEMS; ++k) if (base + k < n) s += in[base + k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        int w = threadIdx.x < TPB / 32 ? red[threadIdx.x] : 0;
        for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
        if (threadIdx.x == 0) tile_sum[blockIdx.x] = w;
    }
}

// One block scans all tile sums in place (exclusive), looping over chunks of TPB.
__global__ void k_scan_tiles(int* __restrict__ tile_sum, int ntiles) {
    int total = 0;
    int carry = 0;
    for (int b = 0; b < ntiles; b += TPB) {
        int i = b + threadIdx.x;
        int v = i < ntiles ? tile_sum[i] : 0;
        int e = block_excl_scan(v, total);
        if (i < ntiles) tile_sum[i] = e + carry;
        carry += total;
    }
}

__global__ void k_tile_rescan(const int* __restrict__ in, int n, const int* __restrict__ tile_sum,
                              int* __restrict__ out) {
    int total = 0;
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int s = 0;
    for (int k = 0; k < SCAN_ITEMS; ++k) { v[k] = base + k < n ? in[base + k] : 0; s += v[k]; }
    int e = block_excl_scan(s, total) + tile_sum[blockIdx.x];
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) out[base + k] = e;
        e += v[k];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = e;  // grand total
}

__global__ void k_scatter(int n, const int* __restrict__ cell_of, const int* __restrict__ rank,
                          const int* __restrict__ cell_start, int* __restrict__ perm) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    perm[cell_start[cell_of[i]] + rank[i]] = i;
}

__device__ __forceinline__ void append(int* list, int* counter, bool pred, int value) {
    unsigned mask = __ballot_sync(0xffffffffu, pred);
    if (!mask) return;
    const int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (pred) list[base + __popc(mask & ((1u << lane) - 1u))] = value;
}

// vt_src / vt_dst (3 planes each, may be null): v_tmp carried with its particle.  The
// mu(I) first loop reads the dummy particles' v_tmp of the previous step before the
// boundary loop rewrites it (eng/solver_sph_muI.py:67-109), and the reference's
// array-of-structs sort moves it with the particle.
template <bool SOIL>
__global__ void k_reorder64(Consts c, const int* __restrict__ perm, Persist64 a, Persist64 b,
                            float4* __restrict__ pos32, int* __restrict__ list_flow,
                            int* __restrict__ list_bdy, int* __restrict__ list_count,
                            const double* __restrict__ vt_src, double* __restrict__ vt_dst) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = k < c.n;
    int mt = 0;
    if (live) {
        const size_t n = c.n;
        const int s = perm[k];
        double xv[3];
        for (int d = 0; d < 3; ++d) {
            xv[d] = a.x[d * n + s];
            b.x[d * n + k] = xv[d];
            b.v[d * n + k] = a.v[d * n + s];
            b.x0[d * n + k] = a.x0[d * n + s];
        }
        b.density[k] = a.density[s];
        b.mass[k] = a.mass[s];
        b.m_V[k] = a.m_V[s];
        b.pressure[k] = a.pressure[s];
        if (SOIL) {
            for (int q = 0; q < 9; ++q) b.stress[q * n + k] = a.stress[q * n + s];
            b.strain_equ[k] = a.strain_equ[s];
            b.strain_equ_p[k] = a.strain_equ_p[s];
            b.flag_retmap[k] = a.flag_retmap[s];
        }
        mt = a.mat_type[s];
        b.mat_type[k] = mt;
        b.mat_id[k] = a.mat_id[s];
        b.obj_id[k] = a.obj_id[s];
        b.is_dynamic[k] = a.is_dynamic[s];
        b.id0[k] = a.id0[s];
        if (vt_src)
            for (int d = 0; d < 3; ++d) vt_dst[d * n + k] = vt_src[d * n + s];
        pos32[k] = make_float4((float)(xv[0] - c.vs[0]), (float)(xv[1] - c.vs[1]), (float)(xv[2] - c.vs[2]), 0.f);
    }
    append(list_flow, list_count + 0, live && mt == c.flow_type, k);
    append(list_bdy, list_count + 1, live && (mt == MAT_DUMMY || mt == MAT_REP || mt == MAT_RIGID), k);
}

inline int nblk(long long n) { return (int)((n + TPB - 1) / TPB); }

}  // namespace

void scan_exclusive(const int* in, int* out, int n, int* tile_sum, cudaStream_t s) {
    int ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    TSG_LAUNCH(k_tile_sums, ntiles, TPB, s, in, n, tile_sum);
    TSG_LAUNCH(k_scan_tiles, 1, TPB, s, tile_sum, ntiles);
    TSG_LAUNCH(k_tile_rescan, ntiles, TPB, s, in, n, tile_sum, out);
}

void sort_fp64(const Consts& c, Persist64& cur, Persist64& nxt, Trans64& t, Grid& g, cudaStream_t s) {
    PhaseScope ph(s, PH_SORT);
    const long long nbins = c.G + 1;
    cudaMemsetAsync(g.count, 0, sizeof(int) * nbins, s);
    cudaMemsetAsync(g.list_count, 0, sizeof(int) * 2, s);
    TSG_LAUNCH(k_hash, nblk(c.n), TPB, s, c, cur.x, g.cell_of, g.rank, g.count, g.err);
    scan_exclusive(g.count, g.cell_start, (int)nbins, g.tile_sum, s);
    TSG_LAUNCH(k_scatter, nblk(c.n), TPB, s, c.n, g.cell_of, g.rank, g.cell_start, g.perm);
    sort_within_cells(nbins, g.cell_start, g.cell_of, c.n, g.perm, g.big, g.nbig, s);
    if (c.solver == 1) {
        TSG_LAUNCH(k_reorder64<false>, nblk(c.n), TPB, s, c, g.perm, cur, nxt, t.pos32, g.list_flow, g.list_bdy,
                   g.list_count, nullptr, nullptr);
    } else {
        // mu(I) keeps v_tmp across steps: stage it in aux3 (free until advect_pos) and gather
        const double* src = nullptr;
        if (c.solver == 2) {
            cudaMemcpyAsync(t.aux3, t.v_tmp, sizeof(double) * 3 * (size_t)c.n, cudaMemcpyDeviceToDevice, s);
            src = t.aux3;
        }
        TSG_LAUNCH(k_reorder64<true>, nblk(c.n), TPB, s, c, g.perm, cur, nxt, t.pos32, g.list_flow, g.list_bdy,
                   g.list_count, src, src ? t.v_tmp : nullptr);
    }
    Persist64 tmp = cur;
    cur = nxt;
    nxt = tmp;
}

}  // namespace tsg
