// Headless visual buffer: the inputs the reference's GUI draws, computed on the device
// into caller buffers (no window, no graphics API).
//
// For every particle the reference picks a scalar by the scene's colour title
// (assign_value_color, eng/solver_sph_base.py:721-785), takes its range over the flow
// particles with optional given / fixed bounds (v_maxmin, eng/particle_system.py:389-398),
// maps (value - min) / (max - min) through the jet colour map (set_color,
// eng/particle_system.py:400-407; ColorMap / color_map, eng/colormap.py:8-50) and scales
// positions by the world-to-screen ratio (copy2vis, eng/particle_system.py:380-386).
// Outputs are indexed by particle id (id0), so they stay put while the particles re-sort;
// entries of particles the selection leaves out are not written (the reference keeps their
// previous values).
#include <cfloat>

#include "tsg_internal.h"

namespace tsg {

namespace {

constexpr int TPB = 256;

__device__ __forceinline__ double norm3(const double* a, size_t n, int i) {
    const double x = a[i], y = a[n + i], z = a[2 * n + i];
    return sqrt((x * x + y * y) + z * z);
}

__device__ __forceinline__ bool real_p(int t) { return t > 0; }
__device__ __forceinline__ bool flow_p(int t) { return t == MAT_FLUID || t == MAT_SOIL; }

__device__ double value_of(const VisFields& f, int title, int i) {
    const size_t n = f.n;
    switch (title) {
    case 1: return f.id0[i];
    case 2: return f.density[i];
    case 21: return f.d_density[i];
    case 3: return norm3(f.v, n, i);
    case 31: return f.v[i];
    case 32: return -f.v[n + i];
    case 33: return f.v[2 * n + i];
    case 34: return norm3(f.d_vel, n, i);
    case 35: return f.d_vel[i];
    case 36: return f.d_vel[n + i];
    case 37: return f.d_vel[2 * n + i];
    case 4: return norm3(f.x, n, i);
    case 41: return f.x[i];
    case 42: return f.x[n + i];
    case 43: return f.x[2 * n + i];
    case 44: {
        const double a = f.x[i] - f.x0[i], b = f.x[n + i] - f.x0[n + i], c = f.x[2 * n + i] - f.x0[2 * n + i];
        return sqrt((a * a + b * b) + c * c);
    }
    case 51: return f.stress[i];                       // (0, 0)
    case 52: return -f.stress[4 * n + i];              // (1, 1)
    case 53: return -f.stress[8 * n + i];              // (2, 2)
    case 54: return f.stress[1 * n + i];               // (0, 1)
    case 55: return f.stress[5 * n + i];               // (1, 2)
    case 56: return f.stress[6 * n + i];               // (2, 0)
    case 57: return -((f.stress[i] + f.stress[4 * n + i]) + f.stress[8 * n + i]) / 3.0;
    case 61: return f.strain_equ[i];
    case 62: return f.strain_equ_p[i];
    case 7: return f.pressure[i];
    case 8: return f.flag[i];
    case 102: return f.CSPM_L[i];                      // (0, 0)
    case 103: return norm3(f.v_tmp, n, i);
    default: return 0.0;
    }
}

// mm[0] = max(mm[0], vmax), mm[1] = min(mm[1], vmin) (a value that compares false, NaN, is
// never stored).
__device__ __forceinline__ void atomic_minmax(double* mm, double vmax, double vmin) {
    unsigned long long* amax = reinterpret_cast<unsigned long long*>(mm);
    unsigned long long* amin = reinterpret_cast<unsigned long long*>(mm + 1);
    unsigned long long old = *amax;
    while (__longlong_as_double(old) < vmax) {
        unsigned long long prev = atomicCAS(amax, old, __double_as_longlong(vmax));
        if (prev == old) break;
        old = prev;
    }
    old = *amin;
    while (__longlong_as_double(old) > vmin) {
        unsigned long long prev = atomicCAS(amin, old, __double_as_longlong(vmin));
        if (prev == old) break;
        old = prev;
    }
}

// Values of the selected particles (real ones, and dummies when shown); range over flow:
// reduced over the warp first (max and min are exact in any order), then one update of the
// range per warp.
__global__ void k_vis_value(VisFields f, int title, int show_bdy, double* __restrict__ val, double* mm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double hi = -INFINITY, lo = INFINITY;
    if (i < f.n) {
        const int t = f.mat_type[i];
        if (real_p(t) || (show_bdy && t == MAT_DUMMY)) {
            const double v = value_of(f, title, i);
            val[i] = v;
            if (flow_p(t)) hi = lo = v;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        hi = fmax(hi, __shfl_down_sync(0xffffffffu, hi, o));
        lo = fmin(lo, __shfl_down_sync(0xffffffffu, lo, o));
    }
    if ((threadIdx.x & 31) == 0 && lo <= hi) atomic_minmax(mm, hi, lo);
}

// The given / fixed bounds of v_maxmin (one thread).
__global__ void k_vis_range(double* mm, double given_max, double given_min, int fix_max, int fix_min) {
    const double vmax = mm[0], vmin = mm[1];
    mm[0] = (given_max == -1 || (vmax < given_max && !fix_max)) ? vmax : given_max;
    mm[1] = (given_min == -1 || (vmin > given_min && !fix_min)) ? vmin : given_min;
}

// ColorMap.map: clamp((w - |clamp(x) - c|) / w * h), w = wl left of the centre, wr right.
__device__ __forceinline__ double cmap(double x, double h, double wl, double wr, double c) {
    const double w = x < c ? wl : wr;
    const double cx = fmax(0.0, fmin(1.0, x));
    return fmax(0.0, fmin(1.0, (w - fabs(cx - c)) / w * h));
}

__global__ void k_vis_out(VisFields f, const double* __restrict__ val, const double* __restrict__ mm, int group,
                          int show_bdy, double w2s, float* __restrict__ pos, float* __restrict__ col) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.n) return;
    const int t = f.mat_type[i];
    const size_t o = 3 * (size_t)f.id0[i];
    const size_t n = f.n;
    if (real_p(t) || (show_bdy && (t == MAT_DUMMY || t == MAT_REP)))
        for (int d = 0; d < 3; ++d) pos[o + d] = (float)(f.x[d * n + i] * w2s);
    const bool pick = (group == 0 && flow_p(t)) || (group == 1 && real_p(t)) ||
                      (group == 2 && (real_p(t) || (show_bdy && t == MAT_DUMMY)));
    if (!pick) return;
    const double vrange1 = 1.0 / (mm[0] - mm[1]);
    const double tmp = (val[i] - mm[1]) * vrange1;
    col[o] = (float)cmap(tmp, 1.5, .37, .37, .75);
    col[o + 1] = (float)cmap(tmp, 1.5, .37, .37, .5);
    col[o + 2] = (float)cmap(tmp, 1.5, .37, .37, .25);
}

}  // namespace

int visual_launch(const VisFields& f, const tsg_visual_cfg& vc, double* scratch, float* pos, float* col,
                  double* range_out, cudaStream_t s) {
    double* val = scratch;         // n
    double* mm = scratch + f.n;    // max, min
    const double init[2] = {-DBL_MAX, DBL_MAX};
    cudaMemcpyAsync(mm, init, sizeof init, cudaMemcpyHostToDevice, s);
    const int nb = (int)((f.n + TPB - 1) / TPB);
    TSG_LAUNCH(k_vis_value, nb, TPB, s, f, vc.color_title, vc.show_bdy, val, mm);
    TSG_LAUNCH(k_vis_range, 1, 1, s, mm, vc.given_max, vc.given_min, vc.fix_max, vc.fix_min);
    TSG_LAUNCH(k_vis_out, nb, TPB, s, f, val, mm, vc.color_group, vc.show_bdy, vc.w2s_ratio, pos, col);
    if (range_out) {
        cudaMemcpyAsync(range_out, mm, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : TSG_E_CUDA;
}

}  // namespace tsg
