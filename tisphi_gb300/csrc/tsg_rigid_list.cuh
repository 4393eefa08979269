// Per-object lists of the dynamic rigid particles, in ascending particle index, built by the
// whole grid instead of one block scanning every particle; shared by the FP64 and
// FP32-mixed forms (the shape matching of eng/solver_sph_base.py:478-511 sums each object's
// particles in that order).
//
// Slot is a device functor: slot(i) = the object slot (0 .. nobj - 1) of particle i, or -1
// for a particle that is not a dynamic rigid one.  Three launches:
//   k_rlist_count  per block of kRListBlock particles and per object, how many it holds;
//   k_rlist_scan   per object, the exclusive scan of those counts over the blocks (in place);
//   k_rlist_fill   every block writes its particles of each object at the object's slice
//                  start off[o] + its block offset + its rank inside the block (warps in
//                  order, lanes in order), so each slice comes out in ascending index.
// Scratch: nobj * nblocks ints (rlist_scratch_ints, tsg_internal.h).  The slices
// off[o] .. off[o + 1] are sized at upload from the same predicate, which no step changes.
// The count and fill passes take one ballot round (two barriers) per object in every
// block, so their cost grows with the number of dynamic bodies (scenes hold a few).
#pragma once

#include <cuda_runtime.h>

#include "tsg_internal.h"

namespace tsg {
namespace {

// Count of block b's particles in object o, for every o: counts[o * nblocks + b].
template <class Slot>
__global__ void __launch_bounds__(kRListBlock) k_rlist_count(int n, int nobj, Slot slot, int* __restrict__ counts) {
    __shared__ int wc[kRListBlock / 32];
    const int i = blockIdx.x * kRListBlock + threadIdx.x;
    const int oi = i < n ? slot(i) : -1;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 0; o < nobj; ++o) {
        const unsigned bal = __ballot_sync(0xffffffffu, oi == o);
        if (lane == 0) wc[wid] = __popc(bal);
        __syncthreads();
        if (threadIdx.x == 0) {
            int c = 0;
            for (int w = 0; w < kRListBlock / 32; ++w) c += wc[w];
            counts[(size_t)o * gridDim.x + blockIdx.x] = c;
        }
        __syncthreads();
    }
}

// Exclusive scan of counts[o * nblocks .. + nblocks) in place, one block of 1024 per object.
__global__ void __launch_bounds__(1024) k_rlist_scan(int nblocks, int* __restrict__ counts) {
    __shared__ int wsum[32];
    __shared__ int carry_s;
    int* c = counts + (size_t)blockIdx.x * nblocks;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (int b0 = 0; b0 < nblocks; b0 += 1024) {
        const int b = b0 + threadIdx.x;
        const int v = b < nblocks ? c[b] : 0;
        int x = v;  // inclusive scan within the warp
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) wsum[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int w = wsum[lane];
            for (int d = 1; d < 32; d <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, d);
                if (lane >= d) w += y;
            }
            wsum[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const int excl = carry_s + (wid ? wsum[wid - 1] : 0) + (x - v);
        if (b < nblocks) c[b] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry_s = excl + v;
        __syncthreads();
    }
}

// Writes each block's particles of object o at list[off[o] + counts[o * nblocks + b] + rank].
template <class Slot>
__global__ void __launch_bounds__(kRListBlock) k_rlist_fill(int n, int nobj, Slot slot, const int* __restrict__ counts,
                                                            const int* __restrict__ off, int* __restrict__ list) {
    __shared__ int wc[kRListBlock / 32];
    const int i = blockIdx.x * kRListBlock + threadIdx.x;
    const int oi = i < n ? slot(i) : -1;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 0; o < nobj; ++o) {
        const unsigned bal = __ballot_sync(0xffffffffu, oi == o);
        if (lane == 0) wc[wid] = __popc(bal);
        __syncthreads();
        if (oi == o) {
            int before = 0;
            for (int w = 0; w < wid; ++w) before += wc[w];
            const int at = off[o] + counts[(size_t)o * gridDim.x + blockIdx.x] + before +
                           __popc(bal & ((1u << lane) - 1u));
            if (at < off[o + 1]) list[at] = i;
        }
        __syncthreads();
    }
}

template <class Slot>
inline void build_rigid_lists(int n, int nobj, const Slot& slot, int* scratch, const int* off, int* list,
                              cudaStream_t s) {
    if (n <= 0 || nobj <= 0) return;
    const int nb = rlist_blocks(n);
    TSG_LAUNCH(k_rlist_count<Slot>, nb, kRListBlock, s, n, nobj, slot, scratch);
    TSG_LAUNCH(k_rlist_scan, nobj, 1024, s, nb, scratch);
    TSG_LAUNCH(k_rlist_fill<Slot>, nb, kRListBlock, s, n, nobj, slot, scratch, off, list);
}

}  // namespace
}  // namespace tsg
