// Allocation-free variant of the cell-list sort (tsg_sort_noalloc).
//
// Some callers cannot call cudaMalloc: code whose device memory is planned up front by a
// fixed-budget pool or by another framework's allocator, and stepping loops that must not
// risk the device-wide synchronisation cudaMalloc / cudaFree can cause.  For them this
// entry point runs the same stable counting sort as tsg_sort (cell hash with the
// truncating cast, exclusive prefix sum, per-cell ordering by old index) on caller-owned
// inputs and outputs, and keeps its own scratch (per-cell counts, per-particle cell index
// and arrival rank) in file-scope __device__ arrays of fixed size.
//
// Limits: at most TSG_NOALLOC_MAX_PARTICLES particles and TSG_NOALLOC_MAX_CELLS cells
// (grid_num_total + 1, counting the trailing bin for particles outside the grid).  Larger
// calls return TSG_E_CAPACITY.  The arrays occupy about 3 MB on every GPU that loads the
// library, for as long as the process lives.
//
// The scratch is shared by every call in the process: counts are cleared at the start of
// each call, and calls that overlap on the GPU (different streams, no ordering between
// them) race on it.  The first call on a device looks up the arrays' device address with
// cudaGetSymbolAddress (once per device, with that device current); make that first call
// before any stream capture begins.  The address is kept for the life of the process: a
// caller that resets the device (cudaDeviceReset) must not call this entry point again in
// that process, since the module may load at another address in the new context.
//
// Unlike tsg_sort, this entry point raises no status for particles outside the grid or
// with non-finite positions: they go to the trailing bin (ascending old index), and a
// caller counts them as cell_start[G + 1] - cell_start[G].
#include <cstdio>

#include "tsg_internal.h"

namespace {

constexpr int kMaxParticles = TSG_NOALLOC_MAX_PARTICLES;
constexpr int kMaxCells = TSG_NOALLOC_MAX_CELLS;
constexpr int kMaxDevices = 64;
constexpr int TPB = 256;

static __device__ __align__(256) int g_noalloc_scratch[kMaxCells + 2 * kMaxParticles];

struct Scratch {
    int* counts;   // kMaxCells
    int* cell_of;  // kMaxParticles
    int* rank;     // kMaxParticles
};

int* g_base[kMaxDevices] = {nullptr};

// Host-side address of the scratch on the current device (looked up once per device).
int scratch_for_current_device(Scratch* out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return TSG_E_CUDA;
    if (!g_base[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            std::fprintf(stderr, "tisphi_gb300: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            return TSG_E_CUDA;
        }
        g_base[dev] = static_cast<int*>(p);
    }
    out->counts = g_base[dev];
    out->cell_of = g_base[dev] + kMaxCells;
    out->rank = g_base[dev] + kMaxCells + kMaxParticles;
    return 0;
}

struct GridSpec {
    double vs[3], grid;
    long long gnum1, gnum2, G;
};

__global__ void k_na_clear(int* counts, int m) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m; c += gridDim.x * blockDim.x) counts[c] = 0;
}

// Cell index per particle (truncating cast of (x - vdomain_start) / grid_size, flattened
// x-major; out-of-range indices go to the trailing bin G) and arrival rank in the cell.
__global__ void k_na_hash(GridSpec g, const double* __restrict__ x, int n, Scratch s) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    long long idx[3];
    bool ok = true;
    for (int d = 0; d < 3; ++d) {
        double t = (x[3 * (size_t)i + d] - g.vs[d]) / g.grid;
        if (!(fabs(t) < 2147483647.0)) { ok = false; idx[d] = 0; }
        else idx[d] = (long long)(int)t;
    }
    long long f = idx[0] * g.gnum1 * g.gnum2 + idx[1] * g.gnum2 + idx[2];
    if (!ok || f < 0 || f >= g.G) f = g.G;
    s.cell_of[i] = (int)f;
    s.rank[i] = atomicAdd(&s.counts[f], 1);
}

// Exclusive prefix sum of m counts into out[0..m] by one block (m <= kMaxCells).
__global__ void k_na_scan(const int* __restrict__ counts, int m, int* __restrict__ out) {
    __shared__ int warp_tot[TPB / 32];
    __shared__ int carry_s;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int base = 0; base < m; base += TPB) {
        const int c = base + threadIdx.x;
        const int v = c < m ? counts[c] : 0;
        int incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_tot[wid] = incl;
        __syncthreads();
        int before = 0, total = 0;
        for (int w = 0; w < TPB / 32; ++w) {
            if (w < wid) before += warp_tot[w];
            total += warp_tot[w];
        }
        const int carry = carry_s;
        if (c < m) out[c] = carry + before + incl - v;
        __syncthreads();
        if (threadIdx.x == 0) carry_s = carry + total;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[m] = carry_s;
}

__global__ void k_na_scatter(int n, Scratch s, const int* __restrict__ cell_start, int* __restrict__ perm) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    perm[cell_start[s.cell_of[i]] + s.rank[i]] = i;
}

// Ascending old index inside every cell (the stable order of the reference's serial sort).
// Cells of at most kSmallCell particles (every cell of an ordinary scene: a cell holds a
// few dozen) are insertion-sorted by one thread; larger ones are left to k_na_sort_large.
constexpr int kSmallCell = 32;
constexpr int kMidCell = 4096;   // sorted in shared memory by one block
__global__ void k_na_cell_sort(long long ncell, const int* __restrict__ cell_start, int* __restrict__ perm) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    int b = cell_start[c], e = cell_start[c + 1];
    if (e - b > kSmallCell) return;
    for (int k = b + 1; k < e; ++k) {
        int v = perm[k];
        int j = k - 1;
        while (j >= b && perm[j] > v) { perm[j + 1] = perm[j]; --j; }
        perm[j + 1] = v;
    }
}

// Cells above kSmallCell particles (a coarse grid, or the trailing bin after particles left
// the grid), one block per cell, grid-stride over the cells.  Up to kMidCell particles: a
// bitonic sort of the cell's entries in shared memory.  Above: the cell's entries are
// rebuilt in ascending order from a block-wide scan over every particle of the flag
// "cell_of[i] == c" (n / TPB trips; at most n / kMidCell cells are that large).
__global__ void __launch_bounds__(TPB) k_na_sort_large(long long ncell, const int* __restrict__ cell_start,
                                                       const int* __restrict__ cell_of, int n,
                                                       int* __restrict__ perm) {
    __shared__ int buf[kMidCell];
    __shared__ int warp_tot[TPB / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (long long c = blockIdx.x; c < ncell; c += gridDim.x) {
        const int b = cell_start[c], e = cell_start[c + 1], m = e - b;
        if (m <= kSmallCell) continue;  // uniform across the block
        if (m <= kMidCell) {
            int p2 = 1;
            while (p2 < m) p2 <<= 1;
            for (int k = threadIdx.x; k < p2; k += TPB) buf[k] = k < m ? perm[b + k] : 0x7fffffff;
            __syncthreads();
            for (int size = 2; size <= p2; size <<= 1) {
                for (int stride = size >> 1; stride > 0; stride >>= 1) {
                    for (int k = threadIdx.x; k < p2; k += TPB) {
                        const int o = k ^ stride;
                        if (o > k) {
                            const bool up = (k & size) == 0;
                            const int a = buf[k], z = buf[o];
                            if ((a > z) == up) { buf[k] = z; buf[o] = a; }
                        }
                    }
                    __syncthreads();
                }
            }
            for (int k = threadIdx.x; k < m; k += TPB) perm[b + k] = buf[k];
            __syncthreads();
        } else {
            int base = 0;
            for (int i0 = 0; i0 < n; i0 += TPB) {
                const int i = i0 + threadIdx.x;
                const int f = (i < n && cell_of[i] == (int)c) ? 1 : 0;
                const unsigned bal = __ballot_sync(0xffffffffu, f);
                const int before_lane = __popc(bal & ((1u << lane) - 1u));
                if (lane == 0) warp_tot[wid] = __popc(bal);
                __syncthreads();
                int before = 0, total = 0;
                for (int w = 0; w < TPB / 32; ++w) {
                    if (w < wid) before += warp_tot[w];
                    total += warp_tot[w];
                }
                if (f) perm[b + base + before + before_lane] = i;
                base += total;
                __syncthreads();
            }
        }
    }
}

}  // namespace

extern "C" int tsg_sort_noalloc(const tsg_config* cfg, const double* x, int64_t n, int32_t* cell_start,
                                int32_t* perm, void* stream) {
    if (!cfg || !x || !cell_start || !perm || n <= 0) return TSG_E_ARG;
    if (cfg->grid_num_total <= 0 || !(cfg->grid_size > 0)) return TSG_E_CONFIG;
    if (n > kMaxParticles || cfg->grid_num_total + 1 > kMaxCells) return TSG_E_CAPACITY;
    Scratch s;
    int rc = scratch_for_current_device(&s);
    if (rc) return rc;
    GridSpec g;
    for (int d = 0; d < 3; ++d) g.vs[d] = cfg->vdomain_start[d];
    g.grid = cfg->grid_size;
    g.gnum1 = cfg->grid_num[1];
    g.gnum2 = cfg->grid_num[2];
    g.G = cfg->grid_num_total;
    const int m = (int)(g.G + 1);
    const int nn = (int)n;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    TSG_LAUNCH(k_na_clear, 256, TPB, st, s.counts, m);
    TSG_LAUNCH(k_na_hash, (nn + TPB - 1) / TPB, TPB, st, g, x, nn, s);
    TSG_LAUNCH(k_na_scan, 1, TPB, st, s.counts, m, cell_start);
    TSG_LAUNCH(k_na_scatter, (nn + TPB - 1) / TPB, TPB, st, nn, s, cell_start, perm);
    TSG_LAUNCH(k_na_cell_sort, (m + TPB - 1) / TPB, TPB, st, (long long)m, cell_start, perm);
    TSG_LAUNCH(k_na_sort_large, 152, TPB, st, (long long)m, cell_start, s.cell_of, nn, perm);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        std::fprintf(stderr, "tisphi_gb300: CUDA error: %s\n", cudaGetErrorString(e));
        return TSG_E_CUDA;
    }
    return 0;
}
