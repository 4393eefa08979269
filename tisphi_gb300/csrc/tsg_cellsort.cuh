// The last step of the counting sort, shared by the FP64 and FP32-mixed forms: inside every
// cell, ascending old index (the stable order of the reference's serial sort; the scatter
// before it places a cell's particles in atomic arrival order).
//
// Ordinary cells hold a few dozen particles and are insertion-sorted by one thread each
// (k_cell_sort_small).  A segment above kSortSmall - the out-of-grid bin after particles
// left the grid, or a very coarse grid - would make that quadratic in one thread (a
// blown-up run with every particle out of the grid would keep the GPU busy for hours), so
// such cells are listed instead and sorted by k_cell_sort_big, one block per cell: up to
// kSortMid particles by a bitonic sort in shared memory, above that rebuilt in ascending
// order from a block-wide scan over every particle of the flag "cell_of[i] == c" (n / 256
// trips; at most n / kSortMid cells are that large).  Both paths give the same order.
// Scratch: big (cellsort_big_ints, tsg_internal.h) and its counter nbig, zeroed before each
// sort.
#pragma once

#include <cuda_runtime.h>

#include "tsg_internal.h"

namespace tsg {
namespace {

constexpr int kSortMid = 4096;
constexpr int kSortBlock = 256;

__global__ void k_cell_sort_small(long long ncell, const int* __restrict__ cell_start, int* __restrict__ perm,
                                  int* __restrict__ big, int* __restrict__ nbig) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int b = cell_start[c], e = cell_start[c + 1];
    if (e - b > kSortSmall) {
        big[atomicAdd(nbig, 1)] = (int)c;
        return;
    }
    for (int q = b + 1; q < e; ++q) {
        const int v = perm[q];
        int m = q - 1;
        while (m >= b && perm[m] > v) { perm[m + 1] = perm[m]; --m; }
        perm[m + 1] = v;
    }
}

__global__ void __launch_bounds__(kSortBlock) k_cell_sort_big(const int* __restrict__ big, const int* __restrict__ nbig,
                                                              const int* __restrict__ cell_start,
                                                              const int* __restrict__ cell_of, int n,
                                                              int* __restrict__ perm) {
    __shared__ int buf[kSortMid];
    __shared__ int warp_tot[kSortBlock / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nb = *nbig;
    for (int q = blockIdx.x; q < nb; q += gridDim.x) {
        const int c = big[q];
        const int b = cell_start[c], m = cell_start[c + 1] - b;
        if (m <= kSortMid) {
            int p2 = 1;
            while (p2 < m) p2 <<= 1;
            for (int k = threadIdx.x; k < p2; k += kSortBlock) buf[k] = k < m ? perm[b + k] : 0x7fffffff;
            __syncthreads();
            for (int size = 2; size <= p2; size <<= 1) {
                for (int stride = size >> 1; stride > 0; stride >>= 1) {
                    for (int k = threadIdx.x; k < p2; k += kSortBlock) {
                        const int o = k ^ stride;
                        if (o > k) {
                            const bool up = (k & size) == 0;
                            const int x = buf[k], z = buf[o];
                            if ((x > z) == up) { buf[k] = z; buf[o] = x; }
                        }
                    }
                    __syncthreads();
                }
            }
            for (int k = threadIdx.x; k < m; k += kSortBlock) perm[b + k] = buf[k];
            __syncthreads();
        } else {
            int base = 0;  // the same in every thread: updated from warp_tot after each trip
            for (int i0 = 0; i0 < n; i0 += kSortBlock) {
                const int i = i0 + threadIdx.x;
                const bool f = i < n && cell_of[i] == c;
                const unsigned bal = __ballot_sync(0xffffffffu, f);
                if (lane == 0) warp_tot[wid] = __popc(bal);
                __syncthreads();
                int before = 0, total = 0;
                for (int w = 0; w < kSortBlock / 32; ++w) {
                    if (w < wid) before += warp_tot[w];
                    total += warp_tot[w];
                }
                if (f && base + before + __popc(bal & ((1u << lane) - 1u)) < m)
                    perm[b + base + before + __popc(bal & ((1u << lane) - 1u))] = i;
                __syncthreads();
                base += total;
            }
        }
    }
}

// Ascending old index inside every cell: ncell cells (bins) starting at cell_start, the
// particles' cells in cell_of (n entries, the same index base as perm's values).
inline void sort_within_cells(long long ncell, const int* cell_start, const int* cell_of, int n, int* perm, int* big,
                              int* nbig, cudaStream_t s) {
    cudaMemsetAsync(nbig, 0, sizeof(int), s);
    TSG_LAUNCH(k_cell_sort_small, (int)((ncell + kSortBlock - 1) / kSortBlock), kSortBlock, s, ncell, cell_start,
               perm, big, nbig);
    TSG_LAUNCH(k_cell_sort_big, 152, kSortBlock, s, big, nbig, cell_start, cell_of, n, perm);
}

}  // namespace
}  // namespace tsg
