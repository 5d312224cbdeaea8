/*
 * Oracle for the Magritte formal-solve hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, FP64 restatement of the reference CPU algorithm (Magritte 0.9.3,
 * src/solver/solver.tpp, src/model/geometry/geometry.tpp, src/model/model.cpp,
 * src/model/lines/...).  It exists to check the CUDA product path and to time
 * the reference algorithm on host cores.  Only the test-suite, the smoke check
 * and the CPU-baseline leg of bench.py may load it; the product library never
 * links or calls it.
 *
 * Arithmetic follows the reference statement by statement: FP64 storage with
 * the single-precision libm calls the reference makes (expf, expm1f, erff,
 * logf, powf), no FMA contraction (built with -ffp-contract=off), vector dot
 * products summed x, y, z left to right.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Approximation used for summing lines (src/solver/solver.hpp:9). */
enum { ORC_NONE = 0, ORC_ONELINE = 1, ORC_CLOSELINES = 2 };

/* Boundary conditions (src/model/geometry/boundary/boundary.hpp:7). */
enum { ORC_BC_ZERO = 0, ORC_BC_THERMAL = 1, ORC_BC_CMB = 2 };

/* Flat view of the Model fields the formal solve reads.  All arrays are
 * row-major with the reference's index conventions:
 *   position/velocity [P][3] (velocity as v/c), emissivity/opacity/
 *   inverse_width/interp_criterion [P][L] (index l + p*L, lines.tpp:8-10),
 *   nu [P][F] (index f + p*F, radiation.tpp:3-5), ray_direction [nrays][3]. */
typedef struct {
    uint32_t npoints, nrays, hnrays, nlines, nquads, nfreqs, nlspecs, nboundary;
    const double*   position;
    const double*   velocity;
    const uint32_t* n_neighbors;
    const uint32_t* cum_n_neighbors;
    const uint32_t* neighbors;
    const uint32_t* point2boundary;       /* npoints for interior points */
    const int32_t*  boundary_condition;   /* [nboundary] */
    const double*   boundary_temperature; /* [nboundary] */
    const double*   ray_direction;
    const double*   ray_weight;           /* [nrays] */
    const uint32_t* antipod;              /* [nrays] */
    const double*   line;                 /* [L] line centre frequencies */
    const double*   sorted_line;          /* [L] ascending */
    const uint32_t* sorted_line_map;      /* [L] sorted -> original index */
    double          max_inverse_mass;
    const double*   emissivity;
    const double*   opacity;
    const double*   inverse_width;
    const double*   interp_criterion;     /* opacity / population_tot */
    const double*   temperature;          /* [P] */
    const double*   vturb2;               /* [P] */
    const double*   dshift_max;           /* [P] */
    const double*   nu;                   /* [P][F] */
    const uint32_t* corr_line;            /* [F] */
    const uint32_t* corr_lspec;           /* [F] */
    const uint32_t* corr_k;               /* [F] */
    const uint32_t* corr_z;               /* [F] */
    const uint8_t*  in_line_integral;     /* [F] */
    const uint32_t* nrad;                 /* [nlspecs] */
    const uint32_t* nrad_cum;             /* [nlspecs] */
    const double*   line_A;               /* [L] Einstein A per global line */
    const double*   lspec_inverse_mass;   /* [nlspecs] */
    const double*   quad_weights;         /* [nlspecs][Q] */
    const double*   quad_roots;           /* [nlspecs][Q] */
    double min_opacity;
    double min_dtau;
    double max_interpolation_diff;
    double max_distance_opacity_contribution;
    int    approx;
    int    spherical_symmetry;            /* 1D spherical symmetry: points on the x axis by radius */
    int    use_adaptive_directions;       /* ray_direction [P][nrays][3], ray_weight [P][nrays] */
} OrcModel;

/* One ray pair as the reference lays it out in its per-thread buffers
 * (solver.tpp:484-496): elements first..last, centre = origin. */
typedef struct {
    uint32_t  capacity;   /* length of each array */
    uint32_t  centre, first, last;
    uint32_t* nr;
    uint32_t* nr_interp;
    double*   interp_factor;
    double*   shift;
    double*   dZ;
} OrcRay;

/* Single-precision functions whose last ulp the results depend on: 0 = libm, as the
 * reference (default); 1 = rounded once from double, as the GPU FP64 mode: erff of the
 * line-integrated optical depth, (float)erf((double)x), and expf / expm1f of the
 * short-characteristics update, (float)exp((double)x) / (float)expm1((double)x). */
void orc_set_erf_mode(int mode);

/* Smooth arithmetic for gradient checks (0 = off, the default): interpolate_log,
 * the Gaussian profile, the Planck function and the line-integrated erf difference
 * use pow / exp / expm1 / erf in double precision instead of the reference's
 * single-precision calls (the erf difference as a difference of erfc where both
 * arguments have the same sign). */
void orc_set_smooth(int on);

/* Maximum ray-pair length over all (rr, o), reference Solver::get_ray_lengths_max
 * (solver.tpp:105-126) with get_n_interp over all lines. */
uint32_t orc_ray_lengths_max(const OrcModel* m, int nthreads);

/* Trace ray pair (o, rr) for global line l (trace_ray_for_line, solver.tpp:773-800). */
int orc_trace_ray_pair_for_line(const OrcModel* m, uint32_t o, uint32_t rr, uint32_t l, OrcRay* ray);

/* Model::compute_radiation_field_feautrier_order_2 -> Solver::solve_feautrier_order_2
 * (model.cpp:353-390, solver.tpp:458-540).  n_off_diag = 0.
 *   J          [P][F]      (required)
 *   u          [hnrays][P][F] or NULL
 *   lambda_diag [P][L]      summed diagonal ALO element per (point, global line), or NULL
 *   lambda_has  [P][L]      1 where the reference would hold an ALO element, or NULL */
int orc_formal_solve_fo2(const OrcModel* m, double* J, double* u, double* lambda_diag,
                         uint8_t* lambda_has, int nthreads);

/* Model::compute_radiation_field_feautrier_order_2_uv (model.cpp:395-433 ->
 * Solver::solve_feautrier_order_2_uv, solver.tpp:238-295, :2767-2921): u and v
 * [hnrays][P][F] per ray pair (v = 0 where the ray pair has one point). */
int orc_formal_solve_fo2_uv(const OrcModel* m, double* u, double* v, int nthreads);

/* Same driver restricted to the ray pairs [rr_begin, rr_end) and origins [o_begin, o_end);
 * used to time a bounded sample.  Accumulates into J (not cleared). */
int orc_formal_solve_fo2_range(const OrcModel* m, uint32_t rr_begin, uint32_t rr_end,
                               uint32_t o_begin, uint32_t o_end, double* J, int nthreads);
/* Every ray pair at the listed origins only (J [P][F], ALO diagonal [P][L] rows of
 * those origins accumulated; lambda_diag / lambda_has may be NULL). */
int orc_formal_solve_fo2_origins(const OrcModel* m, const uint32_t* origins, uint32_t n, double* J,
                                 double* lambda_diag, uint8_t* lambda_has, int nthreads);

/* Model::compute_radiation_field_shortchar_order_0 -> Solver::solve_shortchar_order_0
 * (model.cpp:313-349, solver.tpp:150-235, :1564-1757).
 *   I [nrays][P][F], u, v [hnrays][P][F] (each may be NULL), J [P][F]. */
int orc_formal_solve_sc0(const OrcModel* m, double* J, double* I, double* u, double* v,
                         double* lambda_diag, uint8_t* lambda_has, int nthreads);

/* Old imager, Solver::image_feautrier_order_2(model, rr) (solver.tpp:542-574) with
 * Rest-frame shifts.  I [P][F]. */
int orc_image_fo2(const OrcModel* m, uint32_t rr, double* I, int nthreads);

/* New imager, Model::compute_image_new(raydir, nx, ny) (model.cpp:989-1013 ->
 * Solver::image_feautrier_order_2_new_imager, solver.tpp:576-627): pixel rays from a
 * projection plane outside the model.  I [nx*ny][F] (pixel index y + ny*x), ImX, ImY
 * [nx*ny].  Returns 0, < 0 on failure. */
int orc_image_new(const OrcModel* m, const double* raydir, uint32_t nx, uint32_t ny, double* I, double* ImX,
                  double* ImY, int nthreads);

/* Solver::image_optical_depth(model, rr) (solver.tpp:655-684) and
 * image_optical_depth_new_imager (solver.tpp:686-736): the same rays as orc_image_fo2 /
 * orc_image_new, I = the summed optical depth from first to last
 * (image_optical_depth(model, o, f), solver.tpp:2718-2760), 0 for a ray of one point. */
int orc_image_optical_depth(const OrcModel* m, uint32_t rr, double* I, int nthreads);
/* Solver::image_feautrier_order_2_for_point (solver.tpp:629-653, :2582-2715): the rows
 * S_ray / dtau_ray / u_ray [n_tot][F] of point p's ray rr (capacity rows given; -3 when
 * n_tot exceeds it, *n_tot always set). */
int orc_image_for_point(const OrcModel* m, uint32_t rr, uint32_t p, uint32_t* n_tot, double* S, double* dtau,
                        double* u, uint32_t capacity);
/* Solver::set_column (solver.tpp:2953-2991): column [nrays][P] from density [P]. */
int orc_set_column(const OrcModel* m, const double* density, double* column, int nthreads);
/* Solver::solve_feautrier_order_2 with n_off_diag > 0 (solver.tpp:2319-2355): L_diag and
 * the off-diagonal bands of one ray pair at one frequency (see mgr_oracle.c). */
int orc_feautrier_bands(const OrcModel* m, uint32_t o, uint32_t rr, uint32_t f, uint32_t n_off_diag,
                        uint32_t* n_tot, double* A, double* C, double* L_diag, double* L_upper, double* L_lower,
                        uint32_t capacity);
int orc_image_optical_depth_new(const OrcModel* m, const double* raydir, uint32_t nx, uint32_t ny, double* I,
                                double* ImX, double* ImY, int nthreads);

/* ------------------------------------------------------------------ */
/* ALI level populations (mgr_oracle_ali.c)                             */
/* ------------------------------------------------------------------ */

/* One collision partner (collisionPartner.hpp): rates [ntmp][ncol] in m^3/s. */
typedef struct {
    uint32_t num_col_partner;   /* abundance column of the partner */
    int32_t  ortho_para;        /* 0: 'n', 1: 'o', 2: 'p' (orth_or_para_H2) */
    uint32_t ncol, ntmp;
    const uint32_t* icol;
    const uint32_t* jcol;
    const double*   tmp;
    const double*   Cd;
    const double*   Ce;
} OrcColPar;

/* One line-producing species (linedata.hpp); irad = upper, jrad = lower level. */
typedef struct {
    uint32_t num, nlev, nrad, ncolpar, line_offset;
    const double*   energy;
    const double*   weight;
    const uint32_t* irad;
    const uint32_t* jrad;
    const double*   A;
    const double*   Bs;
    const double*   Ba;
    const double*   frequency;
    const OrcColPar* colpar;
} OrcSpecies;

/* The formal solve with n_off_diag > 0 (solver.tpp:2319-2355) and the non-local ALO it
 * builds (update_Lambda, solver.tpp:1760-1850; Lambda::add_element, lambda.tpp:74-86):
 * J [P][F] and, per (point, line), alo_n[p][lid] elements (alo_nr, alo_ls)[p][lid][cap]
 * in the reference's insertion order (the first is the point itself).  Returns -4 when
 * a list would exceed cap (2 n_off_diag hnrays + 1 always suffices). */
int orc_formal_solve_fo2_alo(const OrcModel* m, uint32_t n_off_diag, double* J, uint32_t cap, uint32_t* alo_n,
                             uint32_t* alo_nr, double* alo_ls, int nthreads);

/* Parameters of compute_level_populations (parameters.hpp:76-104). */
typedef struct {
    double   pop_prec, min_rel_pop_for_convergence, convergence_fraction, population_inversion_fraction;
    double   min_line_opacity, min_line_emissivity;
    uint32_t Ng_acceleration_mem_limit, adaptive_Ng_acceleration_min_order, Ng_acceleration_remove_N_its;
    int32_t  use_adaptive_Ng_acceleration, adaptive_Ng_acceleration_use_max_criterion;
    uint32_t n_off_diag;      /* parameters.hpp:66; > 0: non-local ALO, global rate system */
    int32_t  global_stateq;   /* solve the global rate system also when n_off_diag = 0 */
} OrcAliParams;

/* Model::compute_Jeff (model.cpp:514-545) from J [P][F], the ALO diagonal lam [P][L]
 * and populations (per species [P][nlev]); outputs per species [P][nrad]. */
int orc_compute_jeff(const OrcModel* m, uint32_t nlspecs, const OrcSpecies* sp, const double* J, const double* lam,
                     double* const* pops, double* const* Jlin, double* const* Jeff, double* const* Jdif);

/* update_using_statistical_equilibrium of one species from Jeff and the ALO diagonal
 * Ls (both [P][nrad]) and the current populations; abundance [P][nspecs]. */
int orc_stateq(const OrcSpecies* s, uint32_t P, const double* abundance, uint32_t nspecs, const double* temperature,
               const double* Jeff, const double* Ls, const double* pop_in, double min_line_opacity, double* pop_out);

/* Model::compute_level_populations(use_ng, max_it) (model.cpp:654-747).  `em`, `op`,
 * `crit` are the (writable) arrays m->emissivity/opacity/interp_criterion point to;
 * pops (per species [P][nlev]) hold the initial populations and receive the result.
 * err_mean / err_max receive relative_change_mean / _max per normal iteration and
 * species (may be NULL).  Returns the number of normal iterations, < 0 on failure. */
int orc_ali_run(OrcModel* m, double* em, double* op, double* crit, uint32_t nlspecs, const OrcSpecies* sp,
                uint32_t nspecs, const double* abundance, const OrcAliParams* prm, int use_ng, long max_it,
                double* const* pops, double* err_mean, double* err_max, double* const* Jeff_out, int nthreads);

#ifdef __cplusplus
}
#endif
