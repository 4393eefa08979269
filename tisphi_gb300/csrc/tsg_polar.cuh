// Orthogonal polar factor of a 3x3 matrix in f64, shared by the FP64 and FP32-mixed forms:
// the shape matching of dynamic rigid bodies (eng/solver_sph_base.py:478-500).
#pragma once

namespace tsg {

// Orthogonal polar factor of a 3x3 matrix (row-major), Higham's scaled Newton iteration
// X <- (g X + X^-T / g) / 2 with g = (|X^-1|_F / |X|_F)^(1/2) (N. J. Higham, "Computing the
// polar decomposition - with applications", SIAM J. Sci. Stat. Comput. 7, 1986), X^-T from
// the cofactors, until an update changes X by at most 1e-14 (Frobenius) or after 60 steps.
// A zero third row and column (a 2D body) get X[2][2] = 1 first; a singular matrix gives
// the identity.  The reference calls ti.polar_decompose, whose algorithm lives in Taichi.
__device__ inline void polar3(const double* A, double* X) {
    for (int q = 0; q < 9; ++q) X[q] = A[q];
    if (X[2] == 0.0 && X[5] == 0.0 && X[6] == 0.0 && X[7] == 0.0 && X[8] == 0.0) X[8] = 1.0;
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
        double fx = 0.0, fy = 0.0, y[9];
        for (int q = 0; q < 9; ++q) {
            y[q] = cf[q] / det;
            fx += X[q] * X[q];
            fy += y[q] * y[q];
        }
        const double gm = sqrt(sqrt(fy) / sqrt(fx));
        double ch = 0.0;
        for (int q = 0; q < 9; ++q) {
            const double xn = 0.5 * (gm * X[q] + y[q] / gm);
            const double d = xn - X[q];
            ch += d * d;
            X[q] = xn;
        }
        if (ch <= 1e-28) break;
    }
}

}  // namespace tsg
