/*
 * Oracle for the Magritte formal-solve hot path -- TEST INFRASTRUCTURE ONLY.
 * See mgr_oracle.h.  Every function cites the reference statement it restates
 * (paths relative to the Magritte 0.9.3 source tree).
 *
 * Build: -O2 -ffp-contract=off -fopenmp (oracle/Makefile).  The -ffp-contract=off
 * matters: the reference is compiled for x86-64 without FMA, so a*b+c rounds twice.
 */
#include "mgr_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/tools/constants.hpp:15-40 */
#define ORC_PI 3.14159265358979323846
static const double INVERSE_SQRT_PI            = 0.5 * 1.12837916709551257390; /* 0.5*M_2_SQRTPI */
static const double CC                         = 2.99792458E+8;
static const double HH                         = 6.62607004E-34;
static const double KB                         = 1.38064852E-23;
static const double AMU                        = 1.66053904E-27;
static const double T_CMB                      = 2.7254800;
static const double CC_SQUARED                 = 8.98755179E+16;
#define TWO_KB_OVER_AMU_CC_SQUARED (2.0 * KB / (AMU * CC_SQUARED))
#define TWO_HH_OVER_CC_SQUARED     (2.0 * HH / CC_SQUARED)
#define HH_OVER_KB                 (HH / KB)

/* ------------------------------------------------------------------ */
/* Per-thread solver buffers, Solver::setup (solver.tpp:32-77).        */
/* ------------------------------------------------------------------ */
typedef struct {
    uint32_t length, centre;
    uint32_t *nr, *nr_interp;
    double *interp_factor, *shift, *dZ;
    double *Su, *A, *C, *inverse_A, *inverse_C, *FF, *FI, *GG, *GP, *L_diag;
    uint32_t first, last, n_tot;
} Buf;

static int buf_init(Buf* b, uint32_t length) {
    memset(b, 0, sizeof(*b));
    b->length        = length;
    b->centre        = length / 2;
    b->nr            = (uint32_t*)calloc(length, sizeof(uint32_t));
    b->nr_interp     = (uint32_t*)calloc(length, sizeof(uint32_t));
    b->interp_factor = (double*)calloc(length, sizeof(double));
    b->shift         = (double*)calloc(length, sizeof(double));
    b->dZ            = (double*)calloc(length, sizeof(double));
    b->Su            = (double*)calloc(length, sizeof(double));
    b->A             = (double*)calloc(length, sizeof(double));
    b->C             = (double*)calloc(length, sizeof(double));
    b->inverse_A     = (double*)calloc(length, sizeof(double));
    b->inverse_C     = (double*)calloc(length, sizeof(double));
    b->FF            = (double*)calloc(length, sizeof(double));
    b->FI            = (double*)calloc(length, sizeof(double));
    b->GG            = (double*)calloc(length, sizeof(double));
    b->GP            = (double*)calloc(length, sizeof(double));
    b->L_diag        = (double*)calloc(length, sizeof(double));
    return (b->nr && b->nr_interp && b->interp_factor && b->shift && b->dZ && b->Su && b->A
               && b->C && b->inverse_A && b->inverse_C && b->FF && b->FI && b->GG && b->GP
               && b->L_diag)
             ? 0
             : -1;
}

static void buf_free(Buf* b) {
    free(b->nr); free(b->nr_interp); free(b->interp_factor); free(b->shift); free(b->dZ);
    free(b->Su); free(b->A); free(b->C); free(b->inverse_A); free(b->inverse_C);
    free(b->FF); free(b->FI); free(b->GG); free(b->GP); free(b->L_diag);
}

/* ------------------------------------------------------------------ */
/* Geometry                                                            */
/* ------------------------------------------------------------------ */

/* Vector3D::dot, summed x, y, z left to right. */
static inline double dot3(double ax, double ay, double az, const double* b) {
    return ax * b[0] + ay * b[1] + az * b[2];
}

/* Vector3D::squaredNorm, summed x, y, z left to right. */
static inline double sqnorm(const double* a) { return a[0] * a[0] + a[1] * a[1] + a[2] * a[2]; }

/* Geometry::get_next_spherical_symmetry (geometry.tpp:118-159): points are shells on the
 * x axis in ascending radius; inward (before the tangent point) to the next smaller shell
 * the ray meets, or across the tangent point back to the same shell; then outward. */
static uint32_t get_next_spherical(const OrcModel* m, const double* origin, const double* raydir, uint32_t c,
                                   double* Z, double* dZ) {
    uint32_t next;
    const double Rcos        = dot3(origin[0], origin[1], origin[2], raydir);
    const double R2          = sqnorm(origin);
    const double Rsin2       = R2 - Rcos * Rcos;
    const double Rcos_plus_Z = Rcos + *Z;
    if (*Z < -Rcos) {
        if (c == 0) return m->npoints;
        if (sqnorm(m->position + 3 * (c - 1)) >= Rsin2) {
            next = c - 1;
            *dZ  = -sqrt(sqnorm(m->position + 3 * next) - Rsin2) - Rcos_plus_Z;
        } else {
            next = c;
            *dZ  = -2.0 * Rcos_plus_Z;
        }
    } else {
        if (c >= m->npoints - 1) return m->npoints;
        next = c + 1;
        *dZ  = +sqrt(sqnorm(m->position + 3 * next) - Rsin2) - Rcos_plus_Z;
    }
    *Z += *dZ;
    return next;
}

static uint32_t get_next_general(const OrcModel* m, const double* origin, const double* raydir, uint32_t c,
                                 double* Z, double* dZ);

/* Geometry::get_next (geometry.tpp:246-258): spherical symmetry or general geometry. */
static uint32_t get_next(const OrcModel* m, const double* origin, const double* raydir, uint32_t c, double* Z,
                         double* dZ) {
    return m->spherical_symmetry ? get_next_spherical(m, origin, raydir, c, Z, dZ)
                                 : get_next_general(m, origin, raydir, c, Z, dZ);
}

/* Geometry::get_next_general_geometry<Defaulttracer> (geometry.tpp:13-44). */
static uint32_t get_next_general(const OrcModel* m, const double* origin, const double* raydir,
                                 uint32_t c, double* Z, double* dZ) {
    const uint32_t n_nbs     = m->n_neighbors[c];
    const uint32_t cum_n_nbs = m->cum_n_neighbors[c];
    double dmin              = DBL_MAX;
    uint32_t next            = m->npoints;
    for (uint32_t i = 0; i < n_nbs; i++) {
        const uint32_t n   = m->neighbors[cum_n_nbs + i];
        const double Rx    = m->position[3 * n + 0] - origin[0];
        const double Ry    = m->position[3 * n + 1] - origin[1];
        const double Rz    = m->position[3 * n + 2] - origin[2];
        const double Z_new = dot3(Rx, Ry, Rz, raydir);
        if (Z_new > *Z) {
            const double RR                 = Rx * Rx + Ry * Ry + Rz * Rz;
            const double distance_from_ray2 = RR - Z_new * Z_new;
            if (distance_from_ray2 < dmin) {
                dmin  = distance_from_ray2;
                next  = n;
                *dZ   = Z_new - *Z;
            }
        }
    }
    *Z += *dZ;
    return next;
}

/* Rays::get_direction / get_weight (rays.cpp:94-146): per point, [P][nrays], with
 * adaptive ray directions, else [nrays].  The formal solves and set_column use the
 * adaptive layout; the imagers always index [nrays] (their traces are
 * trace_ray<Rest, false>, solver.tpp:550-552). */
static inline const double* ray_dir(const OrcModel* m, int adaptive, uint32_t o, uint32_t r) {
    return m->ray_direction + 3 * (adaptive ? (size_t)o * m->nrays + r : (size_t)r);
}
static inline double ray_wt(const OrcModel* m, uint32_t o, uint32_t r) {
    return m->ray_weight[m->use_adaptive_directions ? (size_t)o * m->nrays + r : (size_t)r];
}

/* Geometry::get_shift_general_geometry<CoMoving|Rest> (geometry.tpp:203-221), the
 * spherical-symmetry shifts at distance Z along the ray (geometry.tpp:378-417) and the
 * reversal for the old imager (geometry.tpp:428-465).  frame: 0 CoMoving, 1 Rest. */
static inline double get_shift(const OrcModel* m, int frame, uint32_t o, uint32_t r, uint32_t c, double Z) {
    const double* d = ray_dir(m, frame == 0 && m->use_adaptive_directions, o, r);
    double shift;
    if (m->spherical_symmetry) {
        const double* org = m->position + 3 * o;
        const double* vo  = m->velocity + 3 * o;
        const double xc   = m->position[3 * c];
        if (frame == 0) {
            if (sqnorm(org) == 0.0) shift = 1.0;
            else if (xc == 0.0) shift = 1.0 - dot3(vo[0], vo[1], vo[2], d);
            else {
                const double Rcos_plus_Z = dot3(org[0], org[1], org[2], d) + Z;
                shift = 1.0 + (m->velocity[3 * c] * Rcos_plus_Z / xc - dot3(vo[0], vo[1], vo[2], d));
            }
        } else {
            if (xc == 0.0) shift = 1.0;
            else {
                const double Rcos_plus_Z = dot3(org[0], org[1], org[2], d) + Z;
                shift = 1.0 + m->velocity[3 * c] * Rcos_plus_Z / xc;
            }
            if (r >= m->hnrays) shift = 2.0 - shift;
        }
        return shift;
    }
    if (frame == 0) {
        const double vx = m->velocity[3 * c + 0] - m->velocity[3 * o + 0];
        const double vy = m->velocity[3 * c + 1] - m->velocity[3 * o + 1];
        const double vz = m->velocity[3 * c + 2] - m->velocity[3 * o + 2];
        shift           = 1.0 + dot3(vx, vy, vz, d);
    } else {
        shift = 1.0 + dot3(m->velocity[3 * c + 0], m->velocity[3 * c + 1], m->velocity[3 * c + 2], d);
        if (r >= m->hnrays) shift = 2.0 - shift;
    }
    return shift;
}

static inline int valid_point(const OrcModel* m, uint32_t p) { return p < m->npoints; }
static inline int not_on_boundary(const OrcModel* m, uint32_t p) {
    return m->point2boundary[p] == m->npoints;
}

/* ------------------------------------------------------------------ */
/* InterpHelper (solver_interp_helper.tpp)                             */
/* ------------------------------------------------------------------ */

/* get_n_interp_for_line (solver_interp_helper.tpp:55-75). */
static inline uint32_t get_n_interp_for_line(const OrcModel* m, uint32_t l, uint32_t crt, uint32_t nxt) {
    const double curr_source = m->interp_criterion[(size_t)crt * m->nlines + l];
    const double next_source = m->interp_criterion[(size_t)nxt * m->nlines + l];
    const double source_diff = fabsf(logf((float)(next_source / curr_source)));
    const double q           = source_diff / (double)logf((float)m->max_interpolation_diff);
    const uint32_t n         = (uint32_t)ceil(q);
    return n > 1 ? n : 1;
}

/* get_n_interp, over all lines (solver_interp_helper.tpp:10-46). */
static inline uint32_t get_n_interp(const OrcModel* m, uint32_t crt, uint32_t nxt) {
    double mx = -DBL_MAX;
    for (uint32_t l = 0; l < m->nlines; l++) {
        const double x = m->interp_criterion[(size_t)nxt * m->nlines + l];
        const double y = m->interp_criterion[(size_t)crt * m->nlines + l];
        const double d = fabsf(logf((float)(x / y)));
        if (d > mx) mx = d;
    }
    const uint32_t n = (uint32_t)ceil(mx / (double)logf((float)m->max_interpolation_diff));
    return n > 1 ? n : 1;
}

/* Smooth mode (test support for gradient checks, off by default): the reference's
 * single-precision powf / expf / expm1f / erff become their double-precision
 * counterparts, so that finite differences of the image see a smooth function. */
static int g_smooth = 0;
void orc_set_smooth(int on) { g_smooth = on; }

/* interpolate_linear / interpolate_log (solver_interp_helper.tpp:78-99). */
static inline double interpolate_linear(double f_start, double f_end, double factor) {
    if (factor == 0.0) return f_start;
    if (factor == 1.0) return f_end;
    return (f_end - f_start) * factor + f_start;
}
static inline double interpolate_log(double f_start, double f_end, double factor) {
    if (factor == 0.0) return f_start;
    if (factor == 1.0) return f_end;
    if (g_smooth) return f_start * pow(f_end / f_start, factor);
    return f_start * (double)powf((float)(f_end / f_start), (float)factor);
}

/* ------------------------------------------------------------------ */
/* Ray tracing (solver.tpp:741-800, :1003-1097)                         */
/* ------------------------------------------------------------------ */

/* Solver::set_data / set_data_for_line; line = UINT32_MAX selects get_n_interp. */
static void set_data(const OrcModel* m, Buf* b, uint32_t line, uint32_t crt, uint32_t nxt,
                     double shift_crt, double shift_nxt, double dZ_loc, int increment,
                     int64_t* id1, int64_t* id2, int* overflow) {
    const double dshift = shift_nxt - shift_crt;
    const uint32_t n_interp_points =
        (line == UINT32_MAX) ? get_n_interp(m, crt, nxt) : get_n_interp_for_line(m, line, crt, nxt);
    if (n_interp_points > 1) {
        const double dZ_interpl     = dZ_loc / n_interp_points;
        const double dshift_interpl = dshift / n_interp_points;
        for (uint32_t i = 1; i <= n_interp_points; i++) {
            if (*id1 < 0 || *id1 >= (int64_t)b->length || *id2 < 0 || *id2 >= (int64_t)b->length) {
                *overflow = 1;
                return;
            }
            b->nr[*id1]            = nxt;
            b->shift[*id1]         = shift_crt + i * dshift_interpl;
            b->nr_interp[*id1]     = crt;
            b->interp_factor[*id1] = 1.0 - ((double)i) / n_interp_points;
            b->dZ[*id2]            = dZ_interpl;
            *id1 += increment;
            *id2 += increment;
        }
    } else {
        if (*id1 < 0 || *id1 >= (int64_t)b->length || *id2 < 0 || *id2 >= (int64_t)b->length) {
            *overflow = 1;
            return;
        }
        b->nr[*id1]            = nxt;
        b->shift[*id1]         = shift_nxt;
        b->nr_interp[*id1]     = crt;
        b->interp_factor[*id1] = 0.0;
        b->dZ[*id2]            = dZ_loc;
        *id1 += increment;
        *id2 += increment;
    }
}

/* Solver::trace_ray_for_line (solver.tpp:773-800) / trace_ray (:741-768).
 * frame 0 CoMoving, 1 Rest.  Returns the final id1. */
static int64_t trace(const OrcModel* m, Buf* b, int frame, uint32_t line, uint32_t o, uint32_t r,
                     int increment, int64_t id1, int64_t id2, int* err) {
    double Z               = 0.0;
    double dZ              = 0.0;
    const double* origin   = m->position + 3 * o;
    const double* raydir   = ray_dir(m, frame == 0 && m->use_adaptive_directions, o, r);
    uint32_t nxt           = get_next(m, origin, raydir, o, &Z, &dZ);
    if (valid_point(m, nxt)) {
        uint32_t crt     = o;
        double shift_crt = get_shift(m, frame, o, r, crt, 0.0);
        double shift_nxt = get_shift(m, frame, o, r, nxt, Z);
        set_data(m, b, line, crt, nxt, shift_crt, shift_nxt, dZ, increment, &id1, &id2, err);
        while (!*err && not_on_boundary(m, nxt)) {
            crt       = nxt;
            shift_crt = shift_nxt;
            nxt       = get_next(m, origin, raydir, nxt, &Z, &dZ);
            if (!valid_point(m, nxt)) { /* reference would read past point2boundary */
                *err = 2;
                break;
            }
            shift_nxt = get_shift(m, frame, o, r, nxt, Z);
            set_data(m, b, line, crt, nxt, shift_crt, shift_nxt, dZ, increment, &id1, &id2, err);
        }
    }
    return id1;
}

/* Solver::get_ray_length (solver.tpp:79-103). */
static uint32_t get_ray_length(const OrcModel* m, uint32_t o, uint32_t r, int adaptive) {
    uint32_t l           = 0;
    double Z             = 0.0;
    double dZ            = 0.0;
    const double* origin = m->position + 3 * o;
    const double* raydir = ray_dir(m, adaptive, o, r);
    uint32_t nxt         = get_next(m, origin, raydir, o, &Z, &dZ);
    if (valid_point(m, nxt)) {
        uint32_t crt = o;
        l += get_n_interp(m, crt, nxt);
        while (not_on_boundary(m, nxt)) {
            crt = nxt;
            nxt = get_next(m, origin, raydir, nxt, &Z, &dZ);
            if (!valid_point(m, nxt)) break;
            l += get_n_interp(m, crt, nxt);
        }
    }
    return l;
}

static uint32_t ray_lengths_max_impl(const OrcModel* m, int nthreads, int adaptive);

/* Solver::get_ray_lengths_max<CoMoving, adaptive> (solver.tpp:105-126): the formal solves'
 * buffer length. */
uint32_t orc_ray_lengths_max(const OrcModel* m, int nthreads) {
    return ray_lengths_max_impl(m, nthreads, m->use_adaptive_directions);
}

/* The imagers' traces use the model-wide directions also in an adaptive model. */
static uint32_t image_ray_lengths_max(const OrcModel* m, int nthreads) {
    const uint32_t a = ray_lengths_max_impl(m, nthreads, 0);
    const uint32_t b = m->use_adaptive_directions ? ray_lengths_max_impl(m, nthreads, 1) : 0;
    return a > b ? a : b;
}

/* olist != NULL: over the origins olist[0 .. n-1] only (the sizing pass's share of a
 * sample of origins), else over every point. */
static uint32_t ray_lengths_max_of(const OrcModel* m, int nthreads, int adaptive, const uint32_t* olist,
                                   uint32_t n) {
    uint32_t mx = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    const int64_t no = olist ? (int64_t)n : (int64_t)m->npoints;
    for (uint32_t rr = 0; rr < m->hnrays; rr++) {
        const uint32_t ar = m->antipod[rr];
#pragma omp parallel for reduction(max : mx) schedule(dynamic, 64)
        for (int64_t i = 0; i < no; i++) {
            const uint32_t o = olist ? olist[i] : (uint32_t)i;
            const uint32_t len = get_ray_length(m, o, rr, adaptive) + get_ray_length(m, o, ar, adaptive);
            if (len > mx) mx = len;
        }
    }
    return mx;
}

static uint32_t ray_lengths_max_impl(const OrcModel* m, int nthreads, int adaptive) {
    return ray_lengths_max_of(m, nthreads, adaptive, NULL, 0);
}

/* ------------------------------------------------------------------ */
/* Line data, profiles, boundary (solver.tpp:1106-1351)                */
/* ------------------------------------------------------------------ */

/* Solver::gaussian (solver.tpp:1106-1110). */
static inline double gaussian(double inverse_width, double diff) {
    const double sqrt_exp = inverse_width * diff;
    if (g_smooth) return inverse_width * INVERSE_SQRT_PI * exp(-sqrt_exp * sqrt_exp);
    return inverse_width * INVERSE_SQRT_PI * (double)expf((float)(-sqrt_exp * sqrt_exp));
}

/* Solver::planck (solver.tpp:1119-1121). */
static inline double planck(double temp, double freq) {
    if (g_smooth) return TWO_HH_OVER_CC_SQUARED * (freq * freq * freq) / expm1(HH_OVER_KB / temp * freq);
    return TWO_HH_OVER_CC_SQUARED * (freq * freq * freq) / (double)expm1f((float)(HH_OVER_KB * freq / temp));
}

/* Solver::boundary_intensity (solver.tpp:1130-1142). */
static inline double boundary_intensity(const OrcModel* m, uint32_t p, double freq) {
    const uint32_t bdy_id = m->point2boundary[p];
    if (bdy_id >= m->nboundary) return 0.0; /* interior point: no boundary condition */
    switch (m->boundary_condition[bdy_id]) {
    case ORC_BC_ZERO: return 0.0;
    case ORC_BC_THERMAL: return planck(m->boundary_temperature[bdy_id], freq);
    default: return planck(T_CMB, freq);
    }
}

/* Thermodynamics::profile_width_upper_bound_with_linefreq (thermodynamics.tpp:42-53). */
static inline double upper_bound_width(const OrcModel* m, uint32_t p, double freq_line) {
    return freq_line * sqrt(TWO_KB_OVER_AMU_CC_SQUARED * m->max_inverse_mass * m->temperature[p] + m->vturb2[p]);
}

/* Thermodynamics::profile (thermodynamics.tpp:8-35). */
static inline double thermo_profile(const OrcModel* m, double inverse_mass, uint32_t p,
                                    double freq_line, double freq) {
    const double width = freq_line * sqrt(TWO_KB_OVER_AMU_CC_SQUARED * inverse_mass * m->temperature[p] + m->vturb2[p]);
    const double inverse_width = 1.0 / width;
    const double sqrtExponent  = inverse_width * (freq - freq_line);
    const double exponent      = sqrtExponent * sqrtExponent;
    return inverse_width * INVERSE_SQRT_PI * (double)expf((float)(-exponent));
}

/* std::lower_bound / std::upper_bound over sorted_line. */
static inline uint32_t lower_bound(const double* a, uint32_t n, double v) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) / 2;
        if (a[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}
static inline uint32_t upper_bound(const double* a, uint32_t n, double v) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) / 2;
        if (!(v < a[mid])) lo = mid + 1; else hi = mid;
    }
    return lo;
}

#define EM(p, l) m->emissivity[(size_t)(p) * m->nlines + (l)]
#define OP(p, l) m->opacity[(size_t)(p) * m->nlines + (l)]
#define IW(p, l) m->inverse_width[(size_t)(p) * m->nlines + (l)]

/* Solver::get_eta_and_chi<None|CloseLines|OneLine> (solver.tpp:1151-1165, :1197-1239, :1286-1294). */
static void get_eta_and_chi(const OrcModel* m, uint32_t p, uint32_t ll, double freq, double* eta, double* chi) {
    if (m->approx == ORC_ONELINE) {
        const double diff = freq - m->line[ll];
        const double prof = gaussian(IW(p, ll), diff);
        *eta              = prof * EM(p, ll);
        *chi              = prof * OP(p, ll) + m->min_opacity;
        return;
    }
    *eta = 0.0;
    *chi = m->min_opacity;
    if (m->approx == ORC_NONE) {
        for (uint32_t l = 0; l < m->nlines; l++) {
            const double diff = freq - m->line[l];
            const double prof = gaussian(IW(p, l), diff);
            *eta += prof * EM(p, l);
            *chi += prof * OP(p, l);
        }
        return;
    }
    const double ub = m->max_distance_opacity_contribution * upper_bound_width(m, p, freq);
    const uint32_t lo = lower_bound(m->sorted_line, m->nlines, freq - ub);
    const uint32_t hi = upper_bound(m->sorted_line, m->nlines, freq + ub);
    for (uint32_t s = lo; s < hi; s++) {
        const uint32_t l  = m->sorted_line_map[s];
        const double diff = freq - m->sorted_line[s];
        const double prof = gaussian(IW(p, l), diff);
        *eta += prof * EM(p, l);
        *chi += prof * OP(p, l);
    }
}

/* Solver::get_eta_and_chi_interpolated<None|CloseLines|OneLine> (solver.tpp:1176-1194, :1252-1283, :1306-1320). */
static void get_eta_and_chi_interpolated(const OrcModel* m, uint32_t p1, uint32_t p2, double factor,
                                         uint32_t ll, double freq, double* eta, double* chi) {
    if (m->approx == ORC_ONELINE) {
        const double diff = freq - m->line[ll];
        const double iw   = interpolate_linear(IW(p1, ll), IW(p2, ll), factor);
        const double prof = gaussian(iw, diff);
        const double ie   = interpolate_log(EM(p1, ll), EM(p2, ll), factor);
        const double io   = interpolate_log(OP(p1, ll), OP(p2, ll), factor);
        *eta              = prof * ie;
        *chi              = prof * io + m->min_opacity;
        return;
    }
    *eta = 0.0;
    *chi = m->min_opacity;
    uint32_t lo = 0, hi = m->nlines;
    if (m->approx == ORC_CLOSELINES) {
        const double ub = m->max_distance_opacity_contribution * upper_bound_width(m, p1, freq);
        lo              = lower_bound(m->sorted_line, m->nlines, freq - ub);
        hi              = upper_bound(m->sorted_line, m->nlines, freq + ub);
    }
    for (uint32_t s = lo; s < hi; s++) {
        uint32_t l;
        double diff;
        if (m->approx == ORC_CLOSELINES) {
            l    = m->sorted_line_map[s];
            diff = freq - m->sorted_line[s];
        } else {
            l    = s;
            diff = freq - m->line[l];
        }
        const double iw   = interpolate_linear(IW(p1, l), IW(p2, l), factor);
        const double prof = gaussian(iw, diff);
        const double ie   = interpolate_log(EM(p1, l), EM(p2, l), factor);
        const double io   = interpolate_log(OP(p1, l), OP(p2, l), factor);
        *eta += prof * ie;
        *chi += prof * io;
    }
}

/* erff used for the line-integrated optical depth.  Mode 0 (default): the libm
 * erff, as the reference calls it.  Mode 1: the correctly rounded erff,
 * (float)erf((double)x), which is platform independent; the GPU's FP64 mode uses
 * it, so parity between the two is not at the mercy of libm ulps (the reference's
 * erff(a) - erff(b) cancels for |a|, |b| >~ 2 and amplifies those ulps). */
static int g_erf_mode = 0;
void orc_set_erf_mode(int mode) { g_erf_mode = mode; }
static inline float orc_erff(float x) { return g_erf_mode ? (float)erf((double)x) : erff(x); }
/* Mode 1 also rounds the short-characteristics update's expf / expm1f once from double. */
static inline float orc_expf_sc(float x) { return g_erf_mode ? (float)exp((double)x) : expf(x); }
static inline float orc_expm1f_sc(float x) { return g_erf_mode ? (float)expm1((double)x) : expm1f(x); }

/* Smooth mode: erf(a) - erf(b) in double precision, as a difference of erfc when a
 * and b have the same sign (no cancellation in the line wings). */
static inline double orc_erf_diff(double a, double b) {
    if (a > 0.0 && b > 0.0) return erfc(b) - erfc(a);
    if (a < 0.0 && b < 0.0) return erfc(-a) - erfc(-b);
    return erf(a) - erf(b);
}

/* Solver::compute_dtau_single_line (solver.tpp:2374-2455). */
static double compute_dtau_single_line(const OrcModel* m, uint32_t curridx, uint32_t nextidx,
                                       uint32_t ci, uint32_t ni, uint32_t l, double curr_freq,
                                       double next_freq, double curr_interp, double next_interp, double dz) {
    const double linefreq = m->line[l];
    const double iwc      = interpolate_linear(IW(curridx, l), IW(ci, l), curr_interp);
    const double iwn      = interpolate_linear(IW(nextidx, l), IW(ni, l), next_interp);
    const double avg_iw   = (iwc + iwn) / 2.0;
    const double cop      = interpolate_log(OP(curridx, l), OP(ci, l), curr_interp);
    const double nop      = interpolate_log(OP(nextidx, l), OP(ni, l), next_interp);
    if (curr_freq == next_freq) {
        const double diff            = curr_freq - m->line[l];
        const double prof            = gaussian(avg_iw, diff);
        const double average_opacity = (cop + nop) / 2.0;
        return dz * (prof * average_opacity + m->min_opacity);
    }
    const double next_pos        = (linefreq - next_freq) * avg_iw;
    const double curr_pos        = (linefreq - curr_freq) * avg_iw;
    const double diff_pos        = next_pos - curr_pos;
    const double average_opacity = (nop + cop) / 2.0;
    const double erfdiff         = g_smooth ? orc_erf_diff(next_pos, curr_pos)
                                            : (double)(orc_erff((float)next_pos) - orc_erff((float)curr_pos));
    const double erfterm         = average_opacity / diff_pos / 2.0 * erfdiff;
    return dz * (avg_iw * erfterm + m->min_opacity);
}

/* Solver::compute_S_dtau_line_integrated<OneLine|None|CloseLines> (solver.tpp:1878-2111). */
static void compute_S_dtau_line_integrated(const OrcModel* m, uint32_t cp, uint32_t np, uint32_t ci,
                                           uint32_t ni, uint32_t lineidx, double currfreq,
                                           double nextfreq, double curr_interp, double next_interp,
                                           double dZ, double* dtau, double* Scurr, double* Snext) {
    if (m->approx == ORC_ONELINE) {
        const uint32_t l = lineidx;
        *dtau = compute_dtau_single_line(m, cp, np, ci, ni, l, currfreq, nextfreq, curr_interp, next_interp, dZ);
        const double Scp  = EM(cp, l) / OP(cp, l);
        const double Snp  = EM(np, l) / OP(np, l);
        const double Scip = EM(ci, l) / OP(ci, l);
        const double Snip = EM(ni, l) / OP(ni, l);
        *Scurr            = interpolate_log(Scp, Scip, curr_interp);
        *Snext            = interpolate_log(Snp, Snip, next_interp);
        return;
    }
    double sum_dtau = 0.0, sum_c = 0.0, sum_n = 0.0;
    uint32_t lo = 0, hi = m->nlines;
    if (m->approx == ORC_CLOSELINES) {
        double left_freq, right_freq;
        if (currfreq < nextfreq) { left_freq = currfreq; right_freq = nextfreq; }
        else { right_freq = currfreq; left_freq = nextfreq; }
        const double cb = m->max_distance_opacity_contribution * upper_bound_width(m, cp, right_freq);
        const double nb = m->max_distance_opacity_contribution * upper_bound_width(m, np, right_freq);
        const double ub = cb > nb ? cb : nb;
        lo              = lower_bound(m->sorted_line, m->nlines, left_freq - ub);
        hi              = upper_bound(m->sorted_line, m->nlines, right_freq + ub);
    }
    for (uint32_t s = lo; s < hi; s++) {
        const uint32_t l = (m->approx == ORC_CLOSELINES) ? m->sorted_line_map[s] : s;
        const double line_dtau =
            compute_dtau_single_line(m, cp, np, ci, ni, l, currfreq, nextfreq, curr_interp, next_interp, dZ);
        const double Scp  = EM(cp, l) / OP(cp, l);
        const double Snp  = EM(np, l) / OP(np, l);
        const double Scip = EM(ci, l) / OP(ci, l);
        const double Snip = EM(ni, l) / OP(ni, l);
        const double lsc  = interpolate_log(Scp, Scip, curr_interp);
        const double lsn  = interpolate_log(Snp, Snip, next_interp);
        sum_dtau += line_dtau;
        sum_c += line_dtau * lsc;
        sum_n += line_dtau * lsn;
    }
    if (m->approx == ORC_NONE) {
        *dtau  = sum_dtau;
        *Scurr = sum_c / sum_dtau;
        *Snext = sum_n / sum_dtau;
        return;
    }
    double d                    = sum_dtau;
    const double bound_min_dtau = m->min_opacity * dZ;
    if (-bound_min_dtau < d) d = (bound_min_dtau > d) ? bound_min_dtau : d;
    *dtau  = d;
    *Scurr = sum_c / d;
    *Snext = sum_n / d;
}

/* Solver::compute_source_dtau (solver.tpp:2139-2186). */
static void compute_source_dtau(const OrcModel* m, uint32_t cp, uint32_t np, uint32_t ci, uint32_t ni,
                                uint32_t line, double curr_freq, double next_freq, double curr_shift,
                                double next_shift, double dZ, double curr_interp, double next_interp,
                                int* compute_curr_opacity, double* dtaunext, double* chicurr,
                                double* chinext, double* Scurr, double* Snext) {
    const double dshift     = next_shift - curr_shift;
    const double dshift_abs = fabs(dshift);
    const double dmc        = m->dshift_max[cp];
    const double dmn        = m->dshift_max[np];
    const double dshift_max = dmc < dmn ? dmc : dmn;
    if (dshift_abs > dshift_max) {
        *compute_curr_opacity = 1;
        compute_S_dtau_line_integrated(m, cp, np, ci, ni, line, curr_freq, next_freq, curr_interp,
                                       next_interp, dZ, dtaunext, Scurr, Snext);
    } else {
        if (*compute_curr_opacity) {
            *compute_curr_opacity = 0;
            double eta_c          = 0.0;
            get_eta_and_chi_interpolated(m, cp, ci, curr_interp, line, curr_freq, &eta_c, chicurr);
            *Scurr = eta_c / *chicurr;
        }
        double eta_n = 0.0;
        get_eta_and_chi_interpolated(m, np, ni, next_interp, line, next_freq, &eta_n, chinext);
        *Snext    = eta_n / *chinext;
        *dtaunext = 0.5 * (*chicurr + *chinext) * dZ;
    }
}

/* ------------------------------------------------------------------ */
/* Feautrier (solver.tpp:2193-2318, n_off_diag == 0)                    */
/* ------------------------------------------------------------------ */
static void solve_feautrier_order_2(const OrcModel* m, Buf* b, uint32_t o, uint32_t f, int full_back) {
    const double freq  = m->nu[(size_t)o * m->nfreqs + f];
    const uint32_t l   = m->corr_line[f];
    const uint32_t first = b->first, last = b->last, centre = b->centre;
    double chi_c = 0.0, chi_n = 0.0, dtau_c, dtau_n = 0.0, term_c = 0.0, term_n = 0.0;
    int cco = 1;
    double* Su = b->Su; double* A = b->A; double* C = b->C; double* iA = b->inverse_A;
    double* iC = b->inverse_C; double* FF = b->FF; double* FI = b->FI; double* GG = b->GG;
    double* GP = b->GP;

    compute_source_dtau(m, b->nr[first], b->nr[first + 1], b->nr_interp[first], b->nr_interp[first + 1], l,
                        freq * b->shift[first], freq * b->shift[first + 1], b->shift[first],
                        b->shift[first + 1], b->dZ[first], b->interp_factor[first],
                        b->interp_factor[first + 1], &cco, &dtau_n, &chi_c, &chi_n, &term_c, &term_n);

    const double inverse_dtau_f = 1.0 / dtau_n;
    C[first]                    = 2.0 * inverse_dtau_f * inverse_dtau_f;
    iC[first]                   = 1.0 / C[first];
    const double Bf_min_Cf      = 1.0 + 2.0 * inverse_dtau_f;
    const double Bf             = Bf_min_Cf + C[first];
    const double I_bdy_f        = boundary_intensity(m, b->nr[first], freq * b->shift[first]);
    Su[first]                   = term_c + 2.0 * I_bdy_f * inverse_dtau_f;
    Su[first] /= Bf;
    FF[first] = 0.5 * Bf_min_Cf * dtau_n * dtau_n;
    FI[first] = 1.0 / (1.0 + FF[first]);

    for (uint32_t n = first + 1; n < last; n++) {
        term_c = term_n;
        dtau_c = dtau_n;
        chi_c  = chi_n;
        compute_source_dtau(m, b->nr[n], b->nr[n + 1], b->nr_interp[n], b->nr_interp[n + 1], l,
                            freq * b->shift[n], freq * b->shift[n + 1], b->shift[n], b->shift[n + 1],
                            b->dZ[n], b->interp_factor[n], b->interp_factor[n + 1], &cco, &dtau_n,
                            &chi_c, &chi_n, &term_c, &term_n);
        const double dtau_avg = 0.5 * (dtau_c + dtau_n);
        iA[n]                 = dtau_avg * dtau_c;
        iC[n]                 = dtau_avg * dtau_n;
        A[n]                  = 1.0 / iA[n];
        C[n]                  = 1.0 / iC[n];
        Su[n]                 = term_c;
        FF[n]                 = (A[n] * FF[n - 1] * FI[n - 1] + 1.0) * iC[n];
        FI[n]                 = 1.0 / (1.0 + FF[n]);
        Su[n]                 = (A[n] * Su[n - 1] + Su[n]) * FI[n] * iC[n];
    }

    const double inverse_dtau_l = 1.0 / dtau_n;
    A[last]                     = 2.0 * inverse_dtau_l * inverse_dtau_l;
    const double Bl_min_Al      = 1.0 + 2.0 * inverse_dtau_l;
    const double Bl             = Bl_min_Al + A[last];
    const double denominator    = 1.0 / (Bl * FF[last - 1] + Bl_min_Al);
    const double I_bdy_l        = boundary_intensity(m, b->nr[last], freq * b->shift[last]);
    Su[last]                    = term_n + 2.0 * I_bdy_l * inverse_dtau_l;
    Su[last]                    = (A[last] * Su[last - 1] + Su[last]) * (1.0 + FF[last - 1]) * denominator;

    if (!full_back) return; /* imager: forward elimination only (solver.tpp:2462-2574) */

    if (centre < last) {
        GG[last] = 0.5 * Bl_min_Al * dtau_n * dtau_n;
        GP[last] = GG[last] / (1.0 + GG[last]);
        for (int64_t n = (int64_t)last - 1; n > (int64_t)centre; n--) {
            Su[n] += Su[n + 1] * FI[n];
            GG[n] = (C[n] * GP[n + 1] + 1.0) * iA[n];
            GP[n] = GG[n] / (1.0 + GG[n]);
        }
        Su[centre] += Su[centre + 1] * FI[centre];
        b->L_diag[centre] = iC[centre] / (FF[centre] + GP[centre + 1]);
    } else {
        b->L_diag[centre] = (1.0 + FF[centre - 1]) / (Bl_min_Al + Bl * FF[centre - 1]);
    }
}

/* Solver::update_Lambda, n_off_diag == 0 (solver.tpp:1760-1800). */
static void update_lambda(const OrcModel* m, Buf* b, uint32_t rr, uint32_t f, double* lambda_diag,
                          uint8_t* lambda_has) {
    if (!m->in_line_integral[f]) return;
    const uint32_t c        = b->centre;
    const uint32_t p        = b->nr[c];
    const double w_ang      = 2.0 * ray_wt(m, p, rr);
    const uint32_t ls       = m->corr_lspec[f];
    const uint32_t k        = m->corr_k[f];
    const uint32_t z        = m->corr_z[f];
    const uint32_t lid      = m->nrad_cum[ls] + k;
    const double freq_line  = m->line[lid];
    const double invr_mass  = m->lspec_inverse_mass[ls];
    const double constante  = m->line_A[lid] * m->quad_weights[(size_t)ls * m->nquads + z] * w_ang;
    double eta, chi;
    get_eta_and_chi(m, p, k, freq_line, &eta, &chi);
    const double inverse_chi = 1.0 / chi;
    const double frq         = m->nu[(size_t)p * m->nfreqs + f] * b->shift[c];
    const double phi         = thermo_profile(m, invr_mass, p, freq_line, frq);
    const double L           = constante * frq * phi * b->L_diag[c] * inverse_chi;
    if (lambda_diag) lambda_diag[(size_t)p * m->nlines + lid] += L;
    if (lambda_has) lambda_has[(size_t)p * m->nlines + lid] = 1;
}

/* Solver::solve_feautrier_order_2 with n_off_diag > 0 (solver.tpp:2193-2298 and the
 * banded branch :2319-2355) for one (o, rr, f): the elimination of the whole ray, then
 * L_diag on every element and the off-diagonal bands L_upper(m, n) / L_lower(m, n) of
 * the inverse Feautrier matrix.  Rows are elements first .. last (index n - first);
 * A and C are the reference's per-row coefficients (A[first], C[last] unused), the
 * bands [n_off_diag][n_tot] row-major (entries the reference does not set stay 0). */
static void feautrier_bands(const OrcModel* m, Buf* b, uint32_t o, uint32_t f, uint32_t n_off_diag, double* Aout,
                            double* Cout, double* Ld, double* Lu, double* Ll) {
    const double freq  = m->nu[(size_t)o * m->nfreqs + f];
    const uint32_t l   = m->corr_line[f];
    const uint32_t first = b->first, last = b->last;
    const uint32_t N     = last + 1 - first;
    double chi_c = 0.0, chi_n = 0.0, dtau_c, dtau_n = 0.0, term_c = 0.0, term_n = 0.0;
    int cco = 1;
    double* Su = b->Su; double* A = b->A; double* C = b->C; double* iA = b->inverse_A;
    double* iC = b->inverse_C; double* FF = b->FF; double* FI = b->FI; double* GG = b->GG;
    double* GP = b->GP;
    double* GI = (double*)calloc(b->length, sizeof(double));
    double* LD = (double*)calloc(b->length, sizeof(double));

    compute_source_dtau(m, b->nr[first], b->nr[first + 1], b->nr_interp[first], b->nr_interp[first + 1], l,
                        freq * b->shift[first], freq * b->shift[first + 1], b->shift[first],
                        b->shift[first + 1], b->dZ[first], b->interp_factor[first],
                        b->interp_factor[first + 1], &cco, &dtau_n, &chi_c, &chi_n, &term_c, &term_n);
    const double inverse_dtau_f = 1.0 / dtau_n;
    C[first]                    = 2.0 * inverse_dtau_f * inverse_dtau_f;
    const double Bf_min_Cf      = 1.0 + 2.0 * inverse_dtau_f;
    const double Bf             = Bf_min_Cf + C[first];
    FF[first] = 0.5 * Bf_min_Cf * dtau_n * dtau_n;
    FI[first] = 1.0 / (1.0 + FF[first]);
    for (uint32_t n = first + 1; n < last; n++) {
        term_c = term_n;
        dtau_c = dtau_n;
        chi_c  = chi_n;
        compute_source_dtau(m, b->nr[n], b->nr[n + 1], b->nr_interp[n], b->nr_interp[n + 1], l,
                            freq * b->shift[n], freq * b->shift[n + 1], b->shift[n], b->shift[n + 1],
                            b->dZ[n], b->interp_factor[n], b->interp_factor[n + 1], &cco, &dtau_n,
                            &chi_c, &chi_n, &term_c, &term_n);
        const double dtau_avg = 0.5 * (dtau_c + dtau_n);
        iA[n] = dtau_avg * dtau_c;
        iC[n] = dtau_avg * dtau_n;
        A[n]  = 1.0 / iA[n];
        C[n]  = 1.0 / iC[n];
        FF[n] = (A[n] * FF[n - 1] * FI[n - 1] + 1.0) * iC[n];
        FI[n] = 1.0 / (1.0 + FF[n]);
    }
    const double inverse_dtau_l = 1.0 / dtau_n;
    A[last]                     = 2.0 * inverse_dtau_l * inverse_dtau_l;
    const double Bl_min_Al      = 1.0 + 2.0 * inverse_dtau_l;
    const double Bl             = Bl_min_Al + A[last];

    GG[last] = 0.5 * Bl_min_Al * dtau_n * dtau_n;
    GI[last] = 1.0 / (1.0 + GG[last]);
    GP[last] = GG[last] * GI[last];
    LD[last] = (1.0 + FF[last - 1]) / (Bl_min_Al + Bl * FF[last - 1]);
    for (int64_t n = (int64_t)last - 1; n > (int64_t)first; n--) {
        GG[n] = (C[n] * GP[n + 1] + 1.0) * iA[n];
        GI[n] = 1.0 / (1.0 + GG[n]);
        GP[n] = GG[n] * GI[n];
        LD[n] = iC[n] / (FF[n] + GP[n + 1]);
    }
    LD[first] = (1.0 + GG[first + 1]) / (Bf_min_Cf + Bf * GG[first + 1]);
    for (int64_t n = (int64_t)last - 1; n >= (int64_t)first; n--) {
        if (n_off_diag > 0) {
            Lu[0 * (size_t)N + (n + 1 - first)] = LD[n + 1] * FI[n];
            Ll[0 * (size_t)N + (n - first)]     = LD[n] * GI[n + 1];
        }
    }
    for (uint32_t mm = 1; mm < n_off_diag && mm < N - 1; mm++)
        for (int64_t n = (int64_t)last - 1 - mm; n >= (int64_t)first; n--) {
            Lu[(size_t)mm * N + (n + mm + 1 - first)] = Lu[(size_t)(mm - 1) * N + (n + mm + 1 - first)] * FI[n];
            Ll[(size_t)mm * N + (n - first)]          = Ll[(size_t)(mm - 1) * N + (n - first)] * GI[n + mm + 1];
        }
    for (uint32_t n = 0; n < N; n++) {
        Ld[n]   = LD[first + n];
        Aout[n] = A[first + n];
        Cout[n] = C[first + n];
    }
    free(GI);
    free(LD);
}

/* The banded ALO of one ray pair (o, rr) at frequency f, traced for f's line as the
 * formal solve traces it.  *n_tot receives the element count; A, C, L_diag [capacity],
 * L_upper, L_lower [n_off_diag][capacity] are written (zeroed first) when n_tot fits
 * capacity and exceeds 2.  Returns -3 when it does not fit. */
int orc_feautrier_bands(const OrcModel* m, uint32_t o, uint32_t rr, uint32_t f, uint32_t n_off_diag,
                        uint32_t* n_tot, double* A, double* C, double* L_diag, double* L_upper, double* L_lower,
                        uint32_t capacity) {
    const uint32_t length = 2 * orc_ray_lengths_max(m, 1) + 1;
    Buf b;
    if (buf_init(&b, length) != 0) return -1;
    const uint32_t c = b.centre;
    int err          = 0;
    b.nr[c]          = o;
    b.shift[c]       = 1.0;
    const uint32_t l = m->corr_line[f];
    const int64_t first = trace(m, &b, 0, l, o, rr, -1, (int64_t)c - 1, (int64_t)c - 1, &err) + 1;
    const int64_t last  = trace(m, &b, 0, l, o, m->antipod[rr], +1, (int64_t)c + 1, (int64_t)c, &err) - 1;
    if (err) {
        buf_free(&b);
        return -2;
    }
    b.first = (uint32_t)first;
    b.last  = (uint32_t)last;
    b.n_tot = (uint32_t)(last + 1 - first);
    *n_tot  = b.n_tot;
    int rc  = 0;
    if (b.n_tot > capacity) rc = -3;
    else if (b.n_tot > 2) {
        memset(L_upper, 0, sizeof(double) * (size_t)n_off_diag * capacity);
        memset(L_lower, 0, sizeof(double) * (size_t)n_off_diag * capacity);
        feautrier_bands(m, &b, o, f, n_off_diag, A, C, L_diag, L_upper, L_lower);
    }
    buf_free(&b);
    return rc;
}

/* ------------------------------------------------------------------ */
/* Non-local ALO (n_off_diag > 0)                                      */
/* ------------------------------------------------------------------ */
/* Lambda::add_element (lambda.tpp:74-86) on lists per (p, line): an element whose
 * emitting point nr is already listed accumulates, else it is appended. */
typedef struct {
    uint32_t cap;
    uint32_t* n;  /* [P][L] */
    uint32_t* nr; /* [P][L][cap] */
    double* ls;   /* [P][L][cap] */
    int overflow;
} AloLists;

static void alo_add(AloLists* a, uint32_t L, uint32_t p, uint32_t lid, uint32_t nr, double v) {
    const size_t key = (size_t)p * L + lid;
    uint32_t* nrs    = a->nr + key * a->cap;
    double* ls       = a->ls + key * a->cap;
    for (uint32_t i = 0; i < a->n[key]; i++)
        if (nrs[i] == nr) {
            ls[i] += v;
            return;
        }
    if (a->n[key] == a->cap) {
        a->overflow = 1;
        return;
    }
    nrs[a->n[key]] = nr;
    ls[a->n[key]]  = v;
    a->n[key]++;
}

/* The update_Lambda term of element n (solver.tpp:1787-1799, :1811-1846):
 * A_k w_z 2 w_rr nu(nr[n], f) shift[n] phi(nr[n]) L / chi(nr[n], line k). */
static double lambda_term(const OrcModel* m, const Buf* b, uint32_t rr, uint32_t f, uint32_t n, double L) {
    const uint32_t c        = b->centre;
    const double w_ang      = 2.0 * ray_wt(m, b->nr[c], rr);
    const uint32_t ls       = m->corr_lspec[f];
    const uint32_t k        = m->corr_k[f];
    const uint32_t z        = m->corr_z[f];
    const uint32_t lid      = m->nrad_cum[ls] + k;
    const double freq_line  = m->line[lid];
    const double invr_mass  = m->lspec_inverse_mass[ls];
    const double constante  = m->line_A[lid] * m->quad_weights[(size_t)ls * m->nquads + z] * w_ang;
    const uint32_t p        = b->nr[n];
    double eta, chi;
    get_eta_and_chi(m, p, k, freq_line, &eta, &chi);
    const double inverse_chi = 1.0 / chi;
    const double frq         = m->nu[(size_t)p * m->nfreqs + f] * b->shift[n];
    const double phi         = thermo_profile(m, invr_mass, p, freq_line, frq);
    return constante * frq * phi * L * inverse_chi;
}

/* Solver::update_Lambda with n_off_diag > 0 (solver.tpp:1760-1850): the diagonal
 * element, then for m < n_off_diag the lower (centre - m - 1) and upper (centre + m + 1)
 * elements that lie on the ray.  Ld [n_tot], Lu / Ll [n_off_diag][n_tot] as
 * feautrier_bands writes them (index n - first). */
static void update_lambda_bands(const OrcModel* m, const Buf* b, uint32_t rr, uint32_t f, uint32_t K,
                                const double* Ld, const double* Lu, const double* Ll, AloLists* a) {
    if (!m->in_line_integral[f]) return;
    const uint32_t c = b->centre, first = b->first, last = b->last, N = b->n_tot;
    const uint32_t p   = b->nr[c];
    const uint32_t lid = m->nrad_cum[m->corr_lspec[f]] + m->corr_k[f];
    alo_add(a, m->nlines, p, lid, p, lambda_term(m, b, rr, f, c, Ld[c - first]));
    for (uint32_t mm = 0; mm < K && mm + 1 < N; mm++) {
        if (c >= first + mm + 1) {
            const uint32_t n = c - mm - 1;
            alo_add(a, m->nlines, p, lid, b->nr[n], lambda_term(m, b, rr, f, n, Ll[(size_t)mm * N + (n - first)]));
        }
        if (c + mm + 1 <= last) {
            const uint32_t n = c + mm + 1;
            alo_add(a, m->nlines, p, lid, b->nr[n], lambda_term(m, b, rr, f, n, Lu[(size_t)mm * N + (n - first)]));
        }
    }
}

int orc_formal_solve_fo2_alo(const OrcModel* m, uint32_t n_off_diag, double* J, uint32_t cap, uint32_t* alo_n,
                             uint32_t* alo_nr, double* alo_ls, int nthreads) {
    const uint32_t length = 2 * orc_ray_lengths_max(m, nthreads) + 1;
    const uint32_t P = m->npoints, F = m->nfreqs, Q = m->nquads, L = m->nlines;
    const uint32_t K = n_off_diag;
    AloLists a = {cap, alo_n, alo_nr, alo_ls, 0};
    memset(J, 0, sizeof(double) * (size_t)P * F);
    memset(alo_n, 0, sizeof(uint32_t) * (size_t)P * L);
    int err_any = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        Buf b;
        int bad = buf_init(&b, length);
        double* Aw = (double*)calloc(length, sizeof(double));
        double* Cw = (double*)calloc(length, sizeof(double));
        double* Ld = (double*)calloc(length, sizeof(double));
        double* Lu = (double*)calloc((size_t)(K ? K : 1) * length, sizeof(double));
        double* Ll = (double*)calloc((size_t)(K ? K : 1) * length, sizeof(double));
        if (!Aw || !Cw || !Ld || !Lu || !Ll) bad = 1;
        for (uint32_t rr = 0; rr < m->hnrays; rr++) {
            const uint32_t ar = m->antipod[rr];
            for (uint32_t ls = 0; ls < m->nlspecs; ls++) {
#pragma omp for schedule(dynamic, 16)
                for (int64_t oo = 0; oo < (int64_t)P; oo++) {
                    if (bad) continue;
                    const uint32_t o = (uint32_t)oo;
                    const uint32_t c = b.centre;
                    b.nr[c]          = o;
                    b.shift[c]       = 1.0;
                    for (uint32_t k = 0; k < m->nrad[ls]; k++) {
                        const uint32_t l = m->nrad_cum[ls] + k;
                        int err          = 0;
                        const int64_t first = trace(m, &b, 0, l, o, rr, -1, (int64_t)c - 1, (int64_t)c - 1, &err) + 1;
                        const int64_t last  = trace(m, &b, 0, l, o, ar, +1, (int64_t)c + 1, (int64_t)c, &err) - 1;
                        if (err) {
#pragma omp atomic write
                            err_any = 1;
                            continue;
                        }
                        b.first = (uint32_t)first;
                        b.last  = (uint32_t)last;
                        b.n_tot = (uint32_t)(last + 1 - first);
                        for (uint32_t q = 0; q < Q; q++) {
                            const uint32_t f = l * Q + q;
                            if (b.n_tot > 1) {
                                solve_feautrier_order_2(m, &b, o, f, 1);
                                J[(size_t)o * F + f] += b.Su[c] * 2.0 * ray_wt(m, o, rr);
                                if (m->in_line_integral[f]) {
                                    memset(Lu, 0, sizeof(double) * (size_t)(K ? K : 1) * b.n_tot);
                                    memset(Ll, 0, sizeof(double) * (size_t)(K ? K : 1) * b.n_tot);
                                    feautrier_bands(m, &b, o, f, K, Aw, Cw, Ld, Lu, Ll);
                                    update_lambda_bands(m, &b, rr, f, K, Ld, Lu, Ll, &a);
                                }
                            } else {
                                J[(size_t)o * F + f] +=
                                    2.0 * ray_wt(m, o, rr) * boundary_intensity(m, o, m->nu[(size_t)o * F + f]);
                            }
                        }
                    }
                }
            }
        }
        buf_free(&b);
        free(Aw);
        free(Cw);
        free(Ld);
        free(Lu);
        free(Ll);
    }
    if (err_any) return -2;
    return a.overflow ? -4 : 0;
}

/* ------------------------------------------------------------------ */
/* Public traces                                                       */
/* ------------------------------------------------------------------ */
int orc_trace_ray_pair_for_line(const OrcModel* m, uint32_t o, uint32_t rr, uint32_t l, OrcRay* ray) {
    Buf b;
    if (buf_init(&b, ray->capacity) != 0) return -1;
    const uint32_t centre = b.centre;
    const uint32_t ar     = m->antipod[rr];
    int err               = 0;
    b.nr[centre]          = o;
    b.shift[centre]       = 1.0;
    const int64_t first   = trace(m, &b, 0, l, o, rr, -1, (int64_t)centre - 1, (int64_t)centre - 1, &err) + 1;
    const int64_t last    = trace(m, &b, 0, l, o, ar, +1, (int64_t)centre + 1, (int64_t)centre, &err) - 1;
    ray->centre           = centre;
    ray->first            = (uint32_t)first;
    ray->last             = (uint32_t)last;
    memcpy(ray->nr, b.nr, sizeof(uint32_t) * b.length);
    memcpy(ray->nr_interp, b.nr_interp, sizeof(uint32_t) * b.length);
    memcpy(ray->interp_factor, b.interp_factor, sizeof(double) * b.length);
    memcpy(ray->shift, b.shift, sizeof(double) * b.length);
    memcpy(ray->dZ, b.dZ, sizeof(double) * b.length);
    buf_free(&b);
    return err ? -2 : 0;
}

/* ------------------------------------------------------------------ */
/* Formal solve driver (solver.tpp:458-540)                             */
/* ------------------------------------------------------------------ */
static int fo2_range_v(const OrcModel* m, uint32_t rr0, uint32_t rr1, uint32_t o0, uint32_t o1,
                       const uint32_t* olist, double* J, double* u, double* v, double* lambda_diag,
                       uint8_t* lambda_has, int nthreads);

/* The v part of Solver::solve_feautrier_order_2_uv(model, o, f) (solver.tpp:2767-2921)
 * after solve_feautrier_order_2 with full back substitution (Su[centre .. last] hold u):
 * a boundary difference when the origin ends the ray, else the finite-difference
 * derivative of u at the origin from u[centre - 1], u[centre] and u[centre + 1]. */
static double feautrier_v(const OrcModel* m, Buf* b, uint32_t o, uint32_t f) {
    const double freq = m->nu[(size_t)o * m->nfreqs + f];
    const uint32_t l  = m->corr_line[f];
    const uint32_t first = b->first, last = b->last, centre = b->centre;
    double* Su = b->Su;
    if (centre == last) {
        const double I_bdy_l = boundary_intensity(m, b->nr[last], freq * b->shift[last]);
        return Su[last] - I_bdy_l;
    }
    if (centre > first) {
        Su[centre - 1] += Su[centre] * b->FI[centre - 1];
        double chi_c = 0.0, chi_n = 0.0, dtau_n = 0.0, term_c = 0.0, term_n = 0.0;
        int cco = 1;
        compute_source_dtau(m, b->nr[centre - 1], b->nr[centre], b->nr_interp[centre - 1], b->nr_interp[centre], l,
                            freq * b->shift[centre - 1], freq * b->shift[centre], b->shift[centre - 1],
                            b->shift[centre], b->dZ[centre - 1], b->interp_factor[centre - 1],
                            b->interp_factor[centre], &cco, &dtau_n, &chi_c, &chi_n, &term_c, &term_n);
        const double dtaumin = dtau_n;
        compute_source_dtau(m, b->nr[centre], b->nr[centre + 1], b->nr_interp[centre], b->nr_interp[centre + 1], l,
                            freq * b->shift[centre], freq * b->shift[centre + 1], b->shift[centre],
                            b->shift[centre + 1], b->dZ[centre], b->interp_factor[centre],
                            b->interp_factor[centre + 1], &cco, &dtau_n, &chi_c, &chi_n, &term_c, &term_n);
        const double dtauplus  = dtau_n;
        const double coeffmin  = -dtauplus / (dtaumin * dtaumin + dtaumin * dtauplus);
        const double coeffplus = dtaumin / (dtaumin * dtauplus + dtauplus * dtauplus);
        const double coeffzero = -coeffmin - coeffplus;
        return -(coeffmin * Su[centre - 1] + coeffplus * Su[centre + 1] + coeffzero * Su[centre]);
    }
    const double I_bdy_f = boundary_intensity(m, b->nr[first], freq * b->shift[first]);
    return I_bdy_f - Su[first];
}

static int fo2_range(const OrcModel* m, uint32_t rr0, uint32_t rr1, uint32_t o0, uint32_t o1,
                     double* J, double* u, double* lambda_diag, uint8_t* lambda_has, int nthreads) {
    return fo2_range_v(m, rr0, rr1, o0, o1, NULL, J, u, NULL, lambda_diag, lambda_has, nthreads);
}

/* Model::compute_radiation_field_feautrier_order_2_uv (model.cpp:395-433 ->
 * Solver::solve_feautrier_order_2_uv, solver.tpp:238-295): u and v per ray pair. */
int orc_formal_solve_fo2_uv(const OrcModel* m, double* u, double* v, int nthreads) {
    const size_t PF = (size_t)m->npoints * m->nfreqs;
    double* J = (double*)calloc(PF ? PF : 1, sizeof(double));
    if (!J) return -3;
    const int rc = fo2_range_v(m, 0, m->hnrays, 0, m->npoints, NULL, J, u, v, NULL, NULL, nthreads);
    free(J);
    return rc;
}

/* olist != NULL: the origins olist[o0 .. o1-1] instead of o0 .. o1-1. */
static int fo2_range_v(const OrcModel* m, uint32_t rr0, uint32_t rr1, uint32_t o0, uint32_t o1,
                       const uint32_t* olist, double* J, double* u, double* v, double* lambda_diag,
                       uint8_t* lambda_has, int nthreads) {
    const uint32_t length =
        2 * (olist ? ray_lengths_max_of(m, nthreads, m->use_adaptive_directions, olist + o0, o1 - o0)
                   : orc_ray_lengths_max(m, nthreads)) + 1;
    const uint32_t P = m->npoints, F = m->nfreqs, Q = m->nquads;
    int err_any = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        Buf b;
        int bad = buf_init(&b, length);
        for (uint32_t rr = rr0; rr < rr1; rr++) {
            const uint32_t ar = m->antipod[rr];
            for (uint32_t ls = 0; ls < m->nlspecs; ls++) {
#pragma omp for schedule(dynamic, 16)
                for (int64_t oo = o0; oo < (int64_t)o1; oo++) {
                    if (bad) continue;
                    const uint32_t o = olist ? olist[oo] : (uint32_t)oo;
                    const uint32_t c = b.centre;
                    b.nr[c]          = o;
                    b.shift[c]       = 1.0;
                    for (uint32_t k = 0; k < m->nrad[ls]; k++) {
                        const uint32_t l = m->nrad_cum[ls] + k;
                        int err          = 0;
                        const int64_t first = trace(m, &b, 0, l, o, rr, -1, (int64_t)c - 1, (int64_t)c - 1, &err) + 1;
                        const int64_t last  = trace(m, &b, 0, l, o, ar, +1, (int64_t)c + 1, (int64_t)c, &err) - 1;
                        if (err) {
#pragma omp atomic write
                            err_any = 1;
                            continue;
                        }
                        b.first = (uint32_t)first;
                        b.last  = (uint32_t)last;
                        b.n_tot = (uint32_t)(last + 1 - first);
                        for (uint32_t q = 0; q < Q; q++) {
                            const uint32_t f = l * Q + q;
                            double val;
                            if (b.n_tot > 1) {
                                solve_feautrier_order_2(m, &b, o, f, 1);
                                val = b.Su[c];
                                if (u) u[((size_t)rr * P + o) * F + f] = val;
                                if (v) v[((size_t)rr * P + o) * F + f] = feautrier_v(m, &b, o, f);
                                J[(size_t)o * F + f] += b.Su[c] * 2.0 * ray_wt(m, o, rr);
                                update_lambda(m, &b, rr, f, lambda_diag, lambda_has);
                            } else {
                                val = boundary_intensity(m, o, m->nu[(size_t)o * F + f]);
                                if (u) u[((size_t)rr * P + o) * F + f] = val;
                                if (v) v[((size_t)rr * P + o) * F + f] = 0.0;
                                J[(size_t)o * F + f] += 2.0 * ray_wt(m, o, rr) * val;
                            }
                        }
                    }
                }
            }
        }
        buf_free(&b);
    }
    return err_any ? -2 : 0;
}

int orc_formal_solve_fo2(const OrcModel* m, double* J, double* u, double* lambda_diag,
                         uint8_t* lambda_has, int nthreads) {
    const size_t PF = (size_t)m->npoints * m->nfreqs;
    memset(J, 0, sizeof(double) * PF);
    if (lambda_diag) memset(lambda_diag, 0, sizeof(double) * (size_t)m->npoints * m->nlines);
    if (lambda_has) memset(lambda_has, 0, (size_t)m->npoints * m->nlines);
    return fo2_range(m, 0, m->hnrays, 0, m->npoints, J, u, lambda_diag, lambda_has, nthreads);
}

int orc_formal_solve_fo2_range(const OrcModel* m, uint32_t rr_begin, uint32_t rr_end, uint32_t o_begin,
                               uint32_t o_end, double* J, int nthreads) {
    return fo2_range(m, rr_begin, rr_end, o_begin, o_end, J, NULL, NULL, NULL, nthreads);
}

/* The whole formal solve (every ray pair) at the listed origins only: their rows of
 * J [P][F] and of the ALO diagonal [P][L] (may be NULL) are accumulated, the others are
 * left alone.  Used to check a sample of origins of models too large to solve whole on
 * the host. */
int orc_formal_solve_fo2_origins(const OrcModel* m, const uint32_t* origins, uint32_t n, double* J,
                                 double* lambda_diag, uint8_t* lambda_has, int nthreads) {
    for (uint32_t i = 0; i < n; i++)
        if (origins[i] >= m->npoints) return -1;
    return fo2_range_v(m, 0, m->hnrays, 0, n, origins, J, NULL, NULL, lambda_diag, lambda_has, nthreads);
}

/* ------------------------------------------------------------------ */
/* Short characteristics, order 0 (solver.tpp:150-235, :1564-1757)      */
/* ------------------------------------------------------------------ */
static double sc0_lambda(const OrcModel* m, uint32_t o, uint32_t r, uint32_t f, double dtau, int have_dtau) {
    if (!have_dtau) return 0.0; /* reference reads an unset dtau here; contribution taken as 0 */
    const double factor     = (double)orc_expm1f_sc((float)(-dtau)) / dtau;
    const uint32_t ls       = m->corr_lspec[f];
    const uint32_t k        = m->corr_k[f];
    const uint32_t z        = m->corr_z[f];
    const uint32_t lid      = m->nrad_cum[ls] + k;
    const double freq_line  = m->line[lid];
    const double invr_mass  = m->lspec_inverse_mass[ls];
    const double constante  = m->line_A[lid] * m->quad_weights[(size_t)ls * m->nquads + z] * ray_wt(m, o, r);
    const double freq       = m->nu[(size_t)o * m->nfreqs + f];
    double eta, chi;
    get_eta_and_chi(m, o, k, freq_line, &eta, &chi);
    const double inverse_chi = 1.0 / chi;
    const double phi         = thermo_profile(m, invr_mass, o, freq_line, freq);
    return constante * freq * phi * (factor + 1.0) * inverse_chi;
}

/* solve_shortchar_order_0_ray_forward (solver.tpp:1564-1640). */
static double sc0_forward(const OrcModel* m, Buf* b, uint32_t o, uint32_t r, uint32_t f, double* L) {
    const double freq = m->nu[(size_t)o * m->nfreqs + f];
    const uint32_t l  = m->corr_line[f];
    double chi_c = 0.0, chi_n = 0.0, source_c = 0.0, source_n = 0.0, dtau = 0.0;
    int cco = 1, have = 0;
    double I = boundary_intensity(m, b->nr[b->first], freq * b->shift[b->first]);
    for (uint32_t idx = b->first + 1; idx <= b->centre; idx++) {
        chi_c    = chi_n;
        source_c = source_n;
        compute_source_dtau(m, b->nr[idx - 1], b->nr[idx], b->nr_interp[idx - 1], b->nr_interp[idx], l,
                            freq * b->shift[idx - 1], freq * b->shift[idx], b->shift[idx - 1], b->shift[idx],
                            b->dZ[idx - 1], b->interp_factor[idx - 1], b->interp_factor[idx], &cco, &dtau,
                            &chi_c, &chi_n, &source_c, &source_n);
        dtau = (m->min_dtau > dtau) ? m->min_dtau : dtau;
        I    = (double)orc_expf_sc((float)(-dtau)) * I
            + (double)orc_expm1f_sc((float)(-dtau)) / dtau * (source_c - source_n * (1.0 + dtau)) + source_c - source_n;
        have = 1;
    }
    *L = sc0_lambda(m, o, r, f, dtau, have);
    return I;
}

/* solve_shortchar_order_0_ray_backward (solver.tpp:1664-1757). */
static double sc0_backward(const OrcModel* m, Buf* b, uint32_t o, uint32_t r, uint32_t f, double* L) {
    const double freq = m->nu[(size_t)o * m->nfreqs + f];
    const uint32_t l  = m->corr_line[f];
    double chi_c = 0.0, chi_n = 0.0, source_c = 0.0, source_n = 0.0, dtau = 0.0;
    int cco = 1, have = 0;
    double I = boundary_intensity(m, b->nr[b->last], freq * b->shift[b->last]);
    for (uint32_t ip1 = b->last; ip1 >= b->centre + 1; ip1--) {
        chi_c    = chi_n;
        source_c = source_n;
        compute_source_dtau(m, b->nr[ip1], b->nr[ip1 - 1], b->nr_interp[ip1], b->nr_interp[ip1 - 1], l,
                            freq * b->shift[ip1], freq * b->shift[ip1 - 1], b->shift[ip1], b->shift[ip1 - 1],
                            b->dZ[ip1 - 1], b->interp_factor[ip1], b->interp_factor[ip1 - 1], &cco, &dtau,
                            &chi_c, &chi_n, &source_c, &source_n);
        dtau = (m->min_dtau > dtau) ? m->min_dtau : dtau;
        I    = (double)orc_expf_sc((float)(-dtau)) * I
            + (double)orc_expm1f_sc((float)(-dtau)) / dtau * (source_c - source_n * (1.0 + dtau)) + source_c - source_n;
        have = 1;
    }
    *L = sc0_lambda(m, o, r, f, dtau, have);
    return I;
}

int orc_formal_solve_sc0(const OrcModel* m, double* J, double* I, double* u, double* v,
                         double* lambda_diag, uint8_t* lambda_has, int nthreads) {
    const uint32_t P = m->npoints, F = m->nfreqs, Q = m->nquads;
    const size_t PF  = (size_t)P * F;
    memset(J, 0, sizeof(double) * PF);
    if (lambda_diag) memset(lambda_diag, 0, sizeof(double) * (size_t)P * m->nlines);
    if (lambda_has) memset(lambda_has, 0, (size_t)P * m->nlines);
    const uint32_t length = 2 * orc_ray_lengths_max(m, nthreads) + 1;
    int err_any           = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        Buf b;
        int bad = buf_init(&b, length);
        for (uint32_t rr = 0; rr < m->hnrays; rr++) {
            const uint32_t ar = m->antipod[rr];
            for (uint32_t ls = 0; ls < m->nlspecs; ls++) {
#pragma omp for schedule(dynamic, 16)
                for (int64_t oo = 0; oo < (int64_t)P; oo++) {
                    if (bad) continue;
                    const uint32_t o  = (uint32_t)oo;
                    const uint32_t c  = b.centre;
                    const double wt   = ray_wt(m, o, rr) * 2.0;
                    b.nr[c]           = o;
                    b.shift[c]        = 1.0;
                    for (uint32_t k = 0; k < m->nrad[ls]; k++) {
                        const uint32_t l = m->nrad_cum[ls] + k;
                        int err          = 0;
                        const int64_t first = trace(m, &b, 0, l, o, rr, -1, (int64_t)c - 1, (int64_t)c - 1, &err) + 1;
                        const int64_t last  = trace(m, &b, 0, l, o, ar, +1, (int64_t)c + 1, (int64_t)c, &err) - 1;
                        if (err) {
#pragma omp atomic write
                            err_any = 1;
                            continue;
                        }
                        b.first = (uint32_t)first;
                        b.last  = (uint32_t)last;
                        b.n_tot = (uint32_t)(last + 1 - first);
                        for (uint32_t z = 0; z < Q; z++) {
                            const uint32_t f = l * Q + z;
                            double If, Ib;
                            if (b.n_tot > 1) {
                                double Lf = 0.0, Lb = 0.0;
                                If = sc0_forward(m, &b, o, rr, f, &Lf);
                                Ib = sc0_backward(m, &b, o, rr, f, &Lb);
                                if (m->in_line_integral[f]) {
                                    if (lambda_diag) {
                                        lambda_diag[(size_t)o * m->nlines + l] += Lf;
                                        lambda_diag[(size_t)o * m->nlines + l] += Lb;
                                    }
                                    if (lambda_has) lambda_has[(size_t)o * m->nlines + l] = 1;
                                }
                                const double uu = 0.5 * (If + Ib);
                                if (u) u[((size_t)rr * P + o) * F + f] = uu;
                                if (v) v[((size_t)rr * P + o) * F + f] = 0.5 * (If - Ib);
                                J[(size_t)o * F + f] += wt * uu;
                            } else {
                                const double bdy_I = boundary_intensity(m, o, m->nu[(size_t)o * F + f]);
                                If = Ib = bdy_I;
                                if (u) u[((size_t)rr * P + o) * F + f] = bdy_I;
                                if (v) v[((size_t)rr * P + o) * F + f] = 0.0;
                                J[(size_t)o * F + f] += wt * bdy_I;
                            }
                            if (I) {
                                I[((size_t)rr * P + o) * F + f] = If;
                                I[((size_t)ar * P + o) * F + f] = Ib;
                            }
                        }
                    }
                }
            }
        }
        buf_free(&b);
    }
    return err_any ? -2 : 0;
}

/* ------------------------------------------------------------------ */
/* Old imager (solver.tpp:542-574, :2462-2574)                          */
/* ------------------------------------------------------------------ */
/* Solver::image_optical_depth(model, o, f) (solver.tpp:2718-2760): the sum of the pair
 * optical depths from first to last. */
static double optical_depth(const OrcModel* m, Buf* b, uint32_t o, uint32_t f) {
    const double freq = m->nu[(size_t)o * m->nfreqs + f];
    const uint32_t l  = m->corr_line[f];
    const uint32_t first = b->first, last = b->last;
    double chi_c = 0.0, chi_n = 0.0, dtau_n = 0.0, term_c = 0.0, term_n = 0.0;
    int cco = 1;
    double tau = 0.0;
    compute_source_dtau(m, b->nr[first], b->nr[first + 1], b->nr_interp[first], b->nr_interp[first + 1], l,
                        freq * b->shift[first], freq * b->shift[first + 1], b->shift[first],
                        b->shift[first + 1], b->dZ[first], b->interp_factor[first],
                        b->interp_factor[first + 1], &cco, &dtau_n, &chi_c, &chi_n, &term_c, &term_n);
    tau += dtau_n;
    for (uint32_t n = first + 1; n < last; n++) {
        term_c = term_n;
        chi_c  = chi_n;
        compute_source_dtau(m, b->nr[n], b->nr[n + 1], b->nr_interp[n], b->nr_interp[n + 1], l,
                            freq * b->shift[n], freq * b->shift[n + 1], b->shift[n], b->shift[n + 1],
                            b->dZ[n], b->interp_factor[n], b->interp_factor[n + 1], &cco, &dtau_n,
                            &chi_c, &chi_n, &term_c, &term_n);
        tau += dtau_n;
    }
    return tau;
}

static int image_fo2_impl(const OrcModel* m, uint32_t rr, double* I, int nthreads, int tau);

int orc_image_fo2(const OrcModel* m, uint32_t rr, double* I, int nthreads) {
    return image_fo2_impl(m, rr, I, nthreads, 0);
}

/* Solver::image_optical_depth(model, rr) (solver.tpp:655-684). */
int orc_image_optical_depth(const OrcModel* m, uint32_t rr, double* I, int nthreads) {
    return image_fo2_impl(m, rr, I, nthreads, 1);
}

static int image_fo2_impl(const OrcModel* m, uint32_t rr, double* I, int nthreads, int tau) {
    const uint32_t P = m->npoints, F = m->nfreqs;
    const uint32_t length = 2 * image_ray_lengths_max(m, nthreads) + 1;
    const uint32_t ar     = m->antipod[rr];
    int err_any           = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        Buf b;
        int bad = buf_init(&b, length);
#pragma omp for schedule(dynamic, 16)
        for (int64_t oo = 0; oo < (int64_t)P; oo++) {
            if (bad) continue;
            const uint32_t o = (uint32_t)oo;
            const uint32_t c = b.centre;
            int err          = 0;
            b.nr[c]          = o;
            b.shift[c]       = get_shift(m, 1, o, rr, o, 0.0);
            const int64_t first = trace(m, &b, 1, UINT32_MAX, o, rr, -1, (int64_t)c - 1, (int64_t)c - 1, &err) + 1;
            const int64_t last  = trace(m, &b, 1, UINT32_MAX, o, ar, +1, (int64_t)c + 1, (int64_t)c, &err) - 1;
            if (err) {
#pragma omp atomic write
                err_any = 1;
                continue;
            }
            b.first = (uint32_t)first;
            b.last  = (uint32_t)last;
            b.n_tot = (uint32_t)(last + 1 - first);
            for (uint32_t f = 0; f < F; f++) {
                if (tau) {
                    I[(size_t)o * F + f] = b.n_tot > 1 ? optical_depth(m, &b, o, f) : 0.0;
                } else if (b.n_tot > 1) {
                    solve_feautrier_order_2(m, &b, o, f, 0);
                    I[(size_t)o * F + f] = 2.0 * b.Su[b.last]
                                         - boundary_intensity(m, b.nr[b.last], m->nu[(size_t)o * F + f]);
                } else {
                    I[(size_t)o * F + f] = boundary_intensity(m, o, m->nu[(size_t)o * F + f]);
                }
            }
        }
        buf_free(&b);
    }
    return err_any ? -2 : 0;
}

/* Solver::image_feautrier_order_2_for_point_loc (solver.tpp:2582-2715): the old imager's
 * ray through o, eliminated forward and then back-substituted along the whole ray.
 * Row k of S / dtau / u (stride F) is element first + k: S holds each pair's source at
 * its far end (the first pair's near end in row 0), dtau the pair's optical depth
 * ending at that element (0 in row 0), u the Feautrier mean intensity. */
static void solve_for_point(const OrcModel* m, Buf* b, uint32_t o, uint32_t f, double* S, double* dtau,
                            double* u) {
    const uint32_t F     = m->nfreqs;
    const double freq    = m->nu[(size_t)o * F + f];
    const uint32_t l     = m->corr_line[f];
    const uint32_t first = b->first, last = b->last;
    double chi_c = 0.0, chi_n = 0.0, dtau_c, dtau_n = 0.0, term_c = 0.0, term_n = 0.0;
    int cco = 1;
    double* Su = b->Su; double* A = b->A; double* C = b->C; double* iA = b->inverse_A;
    double* iC = b->inverse_C; double* FF = b->FF; double* FI = b->FI;

    compute_source_dtau(m, b->nr[first], b->nr[first + 1], b->nr_interp[first], b->nr_interp[first + 1], l,
                        freq * b->shift[first], freq * b->shift[first + 1], b->shift[first],
                        b->shift[first + 1], b->dZ[first], b->interp_factor[first],
                        b->interp_factor[first + 1], &cco, &dtau_n, &chi_c, &chi_n, &term_c, &term_n);
    S[f]        = term_c;
    S[F + f]    = term_n;
    dtau[f]     = 0.0;
    dtau[F + f] = dtau_n;

    const double inverse_dtau_f = 1.0 / dtau_n;
    C[first]                    = 2.0 * inverse_dtau_f * inverse_dtau_f;
    const double Bf_min_Cf      = 1.0 + 2.0 * inverse_dtau_f;
    const double Bf             = Bf_min_Cf + C[first];
    const double I_bdy_f        = boundary_intensity(m, b->nr[first], freq * b->shift[first]);
    Su[first]                   = term_c + 2.0 * I_bdy_f * inverse_dtau_f;
    Su[first] /= Bf;
    FF[first] = 0.5 * Bf_min_Cf * dtau_n * dtau_n;
    FI[first] = 1.0 / (1.0 + FF[first]);

    for (uint32_t n = first + 1; n < last; n++) {
        term_c = term_n;
        dtau_c = dtau_n;
        chi_c  = chi_n;
        compute_source_dtau(m, b->nr[n], b->nr[n + 1], b->nr_interp[n], b->nr_interp[n + 1], l,
                            freq * b->shift[n], freq * b->shift[n + 1], b->shift[n], b->shift[n + 1],
                            b->dZ[n], b->interp_factor[n], b->interp_factor[n + 1], &cco, &dtau_n,
                            &chi_c, &chi_n, &term_c, &term_n);
        const double dtau_avg = 0.5 * (dtau_c + dtau_n);
        iA[n]                 = dtau_avg * dtau_c;
        iC[n]                 = dtau_avg * dtau_n;
        S[(size_t)(n + 1 - first) * F + f]    = term_n;
        dtau[(size_t)(n + 1 - first) * F + f] = dtau_n;
        A[n]  = 1.0 / iA[n];
        C[n]  = 1.0 / iC[n];
        Su[n] = term_c;
        FF[n] = (A[n] * FF[n - 1] * FI[n - 1] + 1.0) * iC[n];
        FI[n] = 1.0 / (1.0 + FF[n]);
        Su[n] = (A[n] * Su[n - 1] + Su[n]) * FI[n] * iC[n];
    }

    const double inverse_dtau_l = 1.0 / dtau_n;
    A[last]                     = 2.0 * inverse_dtau_l * inverse_dtau_l;
    const double Bl_min_Al      = 1.0 + 2.0 * inverse_dtau_l;
    const double Bl             = Bl_min_Al + A[last];
    const double denominator    = 1.0 / (Bl * FF[last - 1] + Bl_min_Al);
    const double I_bdy_l        = boundary_intensity(m, b->nr[last], freq * b->shift[last]);
    Su[last]                    = term_n + 2.0 * I_bdy_l * inverse_dtau_l;
    Su[last]                    = (A[last] * Su[last - 1] + Su[last]) * (1.0 + FF[last - 1]) * denominator;
    u[(size_t)(last - first) * F + f] = Su[last];
    for (int64_t n = (int64_t)last - 1; n >= (int64_t)first; n--) {
        Su[n] += Su[n + 1] * FI[n];
        u[(size_t)(n - first) * F + f] = Su[n];
    }
}

/* Solver::image_feautrier_order_2_for_point (solver.tpp:629-653) for point p along ray
 * rr.  *n_tot receives the ray's element count; the rows are written when it is at most
 * capacity (S / dtau / u are [capacity][F], rows past n_tot untouched; a ray of one
 * element writes nothing).  Returns -3 when the ray does not fit. */
int orc_image_for_point(const OrcModel* m, uint32_t rr, uint32_t p, uint32_t* n_tot, double* S, double* dtau,
                        double* u, uint32_t capacity) {
    const uint32_t length = 2 * image_ray_lengths_max(m, 1) + 1;
    Buf b;
    if (buf_init(&b, length) != 0) return -1;
    const uint32_t c  = b.centre;
    const uint32_t ar = m->antipod[rr];
    int err           = 0;
    b.nr[c]           = p;
    b.shift[c]        = get_shift(m, 1, p, rr, p, 0.0);
    const int64_t first = trace(m, &b, 1, UINT32_MAX, p, rr, -1, (int64_t)c - 1, (int64_t)c - 1, &err) + 1;
    const int64_t last  = trace(m, &b, 1, UINT32_MAX, p, ar, +1, (int64_t)c + 1, (int64_t)c, &err) - 1;
    if (err) {
        buf_free(&b);
        return -2;
    }
    b.first = (uint32_t)first;
    b.last  = (uint32_t)last;
    b.n_tot = (uint32_t)(last + 1 - first);
    *n_tot  = b.n_tot;
    int rc  = 0;
    if (b.n_tot > capacity) rc = -3;
    else if (b.n_tot > 1)
        for (uint32_t f = 0; f < m->nfreqs; f++) solve_for_point(m, &b, p, f, S, dtau, u);
    buf_free(&b);
    return rc;
}

/* Solver::set_column / get_column (solver.tpp:2953-2991): column[r][o] is the trapezoid
 * integral of density from o along ray r to the boundary, for every ray pair (rr and its
 * antipode).  Rays that no pair names stay as given. */
int orc_set_column(const OrcModel* m, const double* density, double* column, int nthreads) {
    const uint32_t P = m->npoints;
    int err_any      = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    for (uint32_t rr = 0; rr < m->hnrays; rr++) {
        const uint32_t ar = m->antipod[rr];
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t oo = 0; oo < (int64_t)P; oo++) {
            const uint32_t o = (uint32_t)oo;
            for (int side = 0; side < 2; side++) {
                const uint32_t r     = side ? ar : rr;
                const double* origin = m->position + 3 * o;
                const double* raydir = ray_dir(m, m->use_adaptive_directions, o, r);
                double col = 0.0, Z = 0.0, dZ = 0.0;
                uint32_t nxt = get_next(m, origin, raydir, o, &Z, &dZ);
                if (valid_point(m, nxt)) {
                    uint32_t crt = o;
                    col += 0.5 * (density[crt] + density[nxt]) * dZ;
                    while (not_on_boundary(m, nxt)) {
                        crt = nxt;
                        nxt = get_next(m, origin, raydir, nxt, &Z, &dZ);
                        if (!valid_point(m, nxt)) { /* the reference would read past point2boundary */
#pragma omp atomic write
                            err_any = 1;
                            break;
                        }
                        col += 0.5 * (density[crt] + density[nxt]) * dZ;
                    }
                }
                column[(size_t)r * P + o] = col;
            }
        }
    }
    return err_any ? -2 : 0;
}

/* ------------------------------------------------------------------ */
/* New imager (solver.tpp:576-627, :808-897; image.cpp:221-398;          */
/* geometry.tpp:55-106, :167-193, :310-367)                              */
/* ------------------------------------------------------------------ */

/* Geometry::get_closest_bdy_point_in_custom_raydir (geometry.tpp:346-367).  The reference
 * starts from point2boundary[0] read as a point index; where that is not a point index
 * (point 0 interior), the first boundary point is used instead. */
static uint32_t closest_bdy_point_in_raydir(const OrcModel* m, const uint32_t* b2p, const double* d) {
    uint32_t best = m->point2boundary[0];
    if (best >= m->npoints) best = b2p[0];
    double pmin = dot3(m->position[3 * best], m->position[3 * best + 1], m->position[3 * best + 2], d);
    for (uint32_t b = 1; b < m->nboundary; b++) {
        const uint32_t p = b2p[b];
        const double pd  = dot3(m->position[3 * p], m->position[3 * p + 1], m->position[3 * p + 2], d);
        if (pd < pmin) {
            best = p;
            pmin = pd;
        }
    }
    return best;
}

/* Geometry::get_boundary_point_closer_to_custom_ray (geometry.tpp:310-341). */
static uint32_t bdy_point_closer(const OrcModel* m, const double* origin, const double* d, uint32_t crt) {
    const double Rx = m->position[3 * crt] - origin[0], Ry = m->position[3 * crt + 1] - origin[1],
                 Rz = m->position[3 * crt + 2] - origin[2];
    const double Zc = dot3(Rx, Ry, Rz, d);
    double dmin2    = (Rx * Rx + Ry * Ry + Rz * Rz) - Zc * Zc;
    uint32_t next   = crt;
    const uint32_t n_nbs = m->n_neighbors[crt], cum = m->cum_n_neighbors[crt];
    for (uint32_t i = 0; i < n_nbs; i++) {
        const uint32_t n = m->neighbors[cum + i];
        if (!not_on_boundary(m, n)) {
            const double Nx = m->position[3 * n] - origin[0], Ny = m->position[3 * n + 1] - origin[1],
                         Nz = m->position[3 * n + 2] - origin[2];
            const double Zn  = dot3(Nx, Ny, Nz, d);
            const double d2  = (Nx * Nx + Ny * Ny + Nz * Nz) - Zn * Zn;
            if (d2 < dmin2) {
                dmin2 = d2;
                next  = n;
            }
        }
    }
    return next;
}

/* Geometry::get_shift<Rest>(origin, 0, raydir, c, Z, false) of a pixel ray (motionless
 * origin): 1 + v[c] . raydir, or in spherical symmetry 1 + v_x[c] (origin . raydir + Z)
 * / x[c] (geometry.tpp:407-417, 1 at x[c] = 0). */
static inline double image_shift(const OrcModel* m, const double* origin, const double* d, uint32_t c, double Z) {
    if (m->spherical_symmetry) {
        const double xc = m->position[3 * c];
        if (xc == 0.0) return 1.0;
        return 1.0 + m->velocity[3 * c] * (dot3(origin[0], origin[1], origin[2], d) + Z) / xc;
    }
    return 1.0 + dot3(m->velocity[3 * c], m->velocity[3 * c + 1], m->velocity[3 * c + 2], d);
}

/* Solver::trace_ray_imaging (solver.tpp:841-897), increment -1, Rest frame with a
 * motionless origin. */
static int64_t trace_imaging(const OrcModel* m, Buf* b, const double* origin, uint32_t start, const double* d,
                             double* Z, int64_t id1, int64_t id2, const double* center, int* err) {
    double dZ = 0.0;
    uint32_t crt = start;
    uint32_t nxt = get_next(m, origin, d, start, Z, &dZ);
    int accessed = 0;
    const int64_t original_id1 = id1;
#define SHIFT_REST(c) image_shift(m, origin, d, (c), *Z)
    if (valid_point(m, nxt)) {
        double shift_crt = image_shift(m, origin, d, crt, *Z - dZ);
        double shift_nxt = SHIFT_REST(nxt);
        set_data(m, b, UINT32_MAX, crt, nxt, shift_crt, shift_nxt, dZ, -1, &id1, &id2, err);
        while (!*err && (not_on_boundary(m, nxt) ||
                         dot3(m->position[3 * nxt] - center[0], m->position[3 * nxt + 1] - center[1],
                              m->position[3 * nxt + 2] - center[2], d) < 0)) {
            crt       = nxt;
            shift_crt = shift_nxt;
            if (not_on_boundary(m, nxt)) accessed = 1;
            nxt = get_next(m, origin, d, nxt, Z, &dZ);
            if (!valid_point(m, nxt)) break;
            shift_nxt = SHIFT_REST(nxt);
            set_data(m, b, UINT32_MAX, crt, nxt, shift_crt, shift_nxt, dZ, -1, &id1, &id2, err);
        }
    }
#undef SHIFT_REST
    /* spherically symmetric models keep boundary-only rays (solver.tpp:891-896) */
    if (!accessed && !m->spherical_symmetry) return original_id1;
    return id1;
}

static int image_new_impl(const OrcModel* m, const double* raydir_in, uint32_t nx, uint32_t ny, double* I,
                          double* ImX, double* ImY, int nthreads, int tau);

int orc_image_new(const OrcModel* m, const double* raydir_in, uint32_t nx, uint32_t ny, double* I, double* ImX,
                  double* ImY, int nthreads) {
    return image_new_impl(m, raydir_in, nx, ny, I, ImX, ImY, nthreads, 0);
}

/* Solver::image_optical_depth_new_imager (solver.tpp:686-736). */
int orc_image_optical_depth_new(const OrcModel* m, const double* raydir_in, uint32_t nx, uint32_t ny, double* I,
                                double* ImX, double* ImY, int nthreads) {
    return image_new_impl(m, raydir_in, nx, ny, I, ImX, ImY, nthreads, 1);
}

static int image_new_impl(const OrcModel* m, const double* raydir_in, uint32_t nx, uint32_t ny, double* I,
                          double* ImX, double* ImY, int nthreads, int tau) {
    const uint32_t P = m->npoints, F = m->nfreqs;
    const double n2 = raydir_in[0] * raydir_in[0] + raydir_in[1] * raydir_in[1] + raydir_in[2] * raydir_in[2];
    if (n2 == 0.0) return -1;
    const double inv = 1 / sqrt(n2);
    const double d[3] = {raydir_in[0] * inv, raydir_in[1] * inv, raydir_in[2] * inv};
    /* Image::set_coordinates_projection_surface (image.cpp:221-366), 3D */
    const double rx = d[0], ry = d[1], rz = d[2];
    const double den = sqrt(rx * rx + ry * ry), iden = 1.0 / den;
    const double ix = ry * iden, iy = -rx * iden, jx = rx * rz * iden, jy = ry * rz * iden, jz = -den;
    /* boundary2point from point2boundary */
    uint32_t* b2p = (uint32_t*)malloc(sizeof(uint32_t) * (m->nboundary ? m->nboundary : 1));
    if (!b2p) return -3;
    for (uint32_t p = 0; p < P; p++)
        if (m->point2boundary[p] < m->nboundary) b2p[m->point2boundary[p]] = p;
    double max_x = -DBL_MAX, max_y = -DBL_MAX, min_x = DBL_MAX, min_y = DBL_MAX;
    for (uint32_t bi = 0; bi < m->nboundary; bi++) {
        const uint32_t p = b2p[bi];
        const double* x = m->position + 3 * p;
        double X, Y;
        if (m->spherical_symmetry) {
            /* 1D (image.cpp:257-269): the boundary shells' x, mirrored below */
            if (x[0] > max_x) max_x = x[0];
            if (x[0] < min_x) min_x = x[0];
            continue;
        }
        if (den >= 1.0e-9) {
            X = ix * x[0] + iy * x[1];
            Y = jx * x[0] + jy * x[1] + jz * x[2];
        } else {
            X = x[0];
            Y = x[1];
        }
        if (X < min_x) min_x = X;
        if (X > max_x) max_x = X;
        if (Y < min_y) min_y = Y;
        if (Y > max_y) max_y = Y;
    }
    if (m->spherical_symmetry) {
        max_x = fabs(min_x) > max_x ? fabs(min_x) : max_x;
        min_x = -max_x;
        min_y = min_x;
        max_y = max_x;
    }
    /* get_closest_bdy_point_in_custom_raydir: the last point in spherical symmetry
     * (geometry.tpp:346-350); the plane at -x of it there (image.cpp:341-346) */
    const uint32_t cbp = m->spherical_symmetry ? P - 1 : closest_bdy_point_in_raydir(m, b2p, d);
    free(b2p);
    const double dist  = m->spherical_symmetry
                             ? -m->position[3 * cbp]
                             : dot3(m->position[3 * cbp], m->position[3 * cbp + 1], m->position[3 * cbp + 2], d);
    const double scp[3] = {d[0] * dist, d[1] * dist, d[2] * dist};
    const double deltax = (max_x - min_x) / nx, deltay = (max_y - min_y) / ny;
    for (uint32_t xi = 0; xi < nx; xi++)
        for (uint32_t yi = 0; yi < ny; yi++) {
            ImX[yi + (size_t)ny * xi] = min_x + deltax / 2.0 + xi * deltax;
            ImY[yi + (size_t)ny * xi] = min_y + deltay / 2.0 + yi * deltay;
        }
    /* Points::center: middle of the bounding box (points.cpp:30-42) */
    double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (uint32_t p = 0; p < P; p++)
        for (int k = 0; k < 3; k++) {
            const double v = m->position[3 * p + k];
            if (v < lo[k]) lo[k] = v;
            if (v > hi[k]) hi[k] = v;
        }
    const double center[3] = {(lo[0] + hi[0]) / 2, (lo[1] + hi[1]) / 2, (lo[2] + hi[2]) / 2};
    const uint32_t npix = nx * ny;
    int err_any = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        uint32_t length = 2 * 4096 + 1;
        Buf b;
        int bad = buf_init(&b, length);
#pragma omp for schedule(dynamic, 8)
        for (int64_t pp = 0; pp < (int64_t)npix; pp++) {
            if (bad) continue;
            const double X = ImX[pp], Y = ImY[pp];
            double origin[3];
            if (den >= 1.0e-9) {
                origin[0] = X * ix + Y * jx + scp[0];
                origin[1] = X * iy + Y * jy + scp[1];
                origin[2] = Y * jz + scp[2];
            } else {
                origin[0] = X + scp[0];
                origin[1] = Y + scp[1];
                origin[2] = 0.0 + scp[2];
            }
            /* trace_ray_imaging_get_start (solver.tpp:808-830) */
            uint32_t start = cbp;
            while (1) {
                const uint32_t nxt = bdy_point_closer(m, origin, d, start);
                if (nxt == start) break;
                start = nxt;
            }
            int err = 0;
            int64_t first = 0;
            while (1) {
                /* Geometry::get_distance_origin_to_boundary (geometry.tpp:167-193) */
                double Z = dot3(m->position[3 * start] - origin[0], m->position[3 * start + 1] - origin[1],
                                m->position[3 * start + 2] - origin[2], d);
                if (m->spherical_symmetry) {
                    const double Rcos  = dot3(origin[0], origin[1], origin[2], d);
                    const double R2    = origin[0] * origin[0] + origin[1] * origin[1] + origin[2] * origin[2];
                    const double Rsin2 = R2 - Rcos * Rcos;
                    const double horz2 = sqnorm(m->position + 3 * start) - Rsin2;
                    Z = horz2 > 0 ? -sqrt(horz2) - Rcos : -Rcos;
                }
                const uint32_t c = b.centre;
                b.nr[c]    = start;
                b.shift[c] = image_shift(m, origin, d, start, Z);
                err   = 0;
                first = trace_imaging(m, &b, origin, start, d, &Z, (int64_t)c - 1, (int64_t)c - 1, center, &err) + 1;
                if (err != 1) break;
                /* buffer too short: grow it and trace again */
                buf_free(&b);
                length = 2 * length + 1;
                if (buf_init(&b, length) != 0) {
                    bad = 1;
                    break;
                }
            }
            if (bad || err) {
#pragma omp atomic write
                err_any = 1;
                continue;
            }
            b.first = (uint32_t)first;
            b.last  = b.centre;
            b.n_tot = b.last + 1 - b.first;
            for (uint32_t f = 0; f < F; f++) {
                const double nu_f = m->nu[(size_t)start * F + f];
                if (tau) {
                    I[(size_t)pp * F + f] = b.n_tot > 1 ? optical_depth(m, &b, start, f) : 0.0;
                } else if (b.n_tot > 1) {
                    solve_feautrier_order_2(m, &b, start, f, 0);
                    I[(size_t)pp * F + f] = 2.0 * b.Su[b.last] - boundary_intensity(m, b.nr[b.last], nu_f);
                } else {
                    I[(size_t)pp * F + f] = boundary_intensity(m, start, nu_f);
                }
            }
        }
        buf_free(&b);
    }
    return err_any ? -2 : 0;
}
