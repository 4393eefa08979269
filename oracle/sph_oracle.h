// ORACLE - test infrastructure only (see sph_oracle.cpp).  C interface used through ctypes
// by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.
#pragma once
#ifdef __cplusplus
extern "C" {
#endif

enum {
    ORC_SORT = 1, ORC_KERNEL_CORR, ORC_INIT_TMP, ORC_ONE_STEP, ORC_ADVECT_FULL, ORC_ADVECT_LF_HALF,
    ORC_SUBSTEP, ORC_ADVECT_POS, ORC_ADVECT_SOMETHING, ORC_ENFORCE_BOUNDARY, ORC_STEP
};
enum { ORC_ERR_CELL_OOB = 1, ORC_ERR_BAD_CONFIG = 2 };

// Raw scene constants, as the reference's Python scope holds them.
typedef struct orc_params {
    int dim;                 // 2 or 3
    int solver;              // 1 WCSPH, 2 mu(I), 3 Drucker-Prager
    int kernel;              // 0 cubic spline, 1 Wendland C2
    int kernel_corr;         // 0 none, 1 CSPM
    int time_integration;    // 1 SE, 2 LF, 4 RK4
    int xsph;                // 0/1
    int boundary;            // 0..4
    int exponent_is_int;     // Tait exponent is an integer
    int init_geostatic;      // DP: apply init_stress at creation
    int grid_num[3];
    long grid_num_total;
    double vdomain_start[3];
    double domain_start[3];
    double domain_end[3];
    double grid_size;
    double support_radius;
    double smoothing_len;
    double particle_diameter;
    double particle_radius;
    double gravity[3];
    double dt;
    double density0;
    double viscosity;
    double stiffness;
    double exponent;
    double coh;              // cohesion (Pa)
    double fric;             // friction angle (rad)
    double E;                // Young's modulus
    double poi;              // Poisson ratio
    double dila;             // dilatancy angle (rad)
    double damping_eps;      // 5e-5 (eng/solver_sph_base.py:714)
} orc_params;

void* orc_create(const orc_params* prm, int n, const double* x, const double* v, const double* density,
                 const double* mass, const double* m_V, const double* pressure, const double* stress,
                 const int* mat_type, const int* mat_id, const int* obj_id, const int* is_dynamic);
void orc_destroy(void* h);
int orc_n(void* h);
int orc_call(void* h, int what);
int orc_steps(void* h, int nsteps);
int orc_get(void* h, const char* name, double* out);
int orc_grid(void* h, int* out);
long orc_neighbors(void* h, int* counts, int* list, long cap);
int orc_density_sum(void* h, double* out);
int orc_error(void* h);

#ifdef __cplusplus
}
#endif
