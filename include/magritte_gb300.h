/*
 * magritte_gb300 -- C ABI of the GB300 (sm_103a) formal-solve library libmgr_gpu.so.
 *
 * The entry points replace the bodies of Magritte's Model::compute_* methods on the
 * formal-solve hot path (Magritte 0.9.3, src/model/model.hpp:58-80,
 * src/model/model.cpp).  Everything is plain C: pointers, sizes, int status codes.
 * Host arrays follow the reference's row-major layouts (index conventions noted per
 * field).  All functions return MGR_OK (0) or a negative MgrStatus; the message of
 * the last failure on the calling thread is available from mgr_last_error().
 *
 * Threading: one MgrModel is used by one host thread at a time.  Each MgrModel owns
 * its CUDA stream and its device copies; host buffers stay with the caller.
 */
#ifndef MAGRITTE_GB300_H
#define MAGRITTE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MGR_OK              = 0,
    MGR_ERR_ARGUMENT    = -1, /* invalid argument or size                                 */
    MGR_ERR_CUDA        = -2, /* CUDA runtime error (message has the CUDA error string)    */
    MGR_ERR_NO_DEVICE   = -3, /* no CUDA device visible                                    */
    MGR_ERR_TRACE       = -4, /* ray left the grid without meeting a boundary point        */
    MGR_ERR_CAPACITY    = -5, /* ray longer than the configured capacity                   */
    MGR_ERR_NONFINITE   = -6, /* non-finite optical depth or pivot detected in a solve     */
    MGR_ERR_UNSUPPORTED = -7  /* option not implemented on this path                       */
} MgrStatus;

/* Line-sum approximation, Solver ApproximationType (src/solver/solver.hpp:9). */
typedef enum { MGR_APPROX_NONE = 0, MGR_APPROX_ONELINE = 1, MGR_APPROX_CLOSELINES = 2 } MgrApprox;

/* Arithmetic of the formal solve.
 *  MGR_PRECISION_FP64  : the reference's arithmetic: FP64 storage with its
 *                        single-precision libm calls (expf, erff, logf, powf).
 *  MGR_PRECISION_SPLIT : profile, opacity, source and optical-depth arithmetic in
 *                        FP32; the Feautrier elimination and back substitution in
 *                        FP64.  Ray traces are identical in both modes.            */
typedef enum { MGR_PRECISION_FP64 = 0, MGR_PRECISION_SPLIT = 1 } MgrPrecision;

/* Boundary conditions (src/model/geometry/boundary/boundary.hpp:7). */
typedef enum { MGR_BC_ZERO = 0, MGR_BC_THERMAL = 1, MGR_BC_CMB = 2 } MgrBoundaryCondition;

/* Flat description of a Magritte Model after its set-up calls
 * (compute_spectral_discretisation, compute_inverse_line_widths, level populations,
 * set_dshift_max).  P = npoints, L = nlines, F = nfreqs, Q = nquads.
 * Layouts: position/velocity [P][3] (velocity as v/c, points.hpp); CSR neighbour
 * lists (points.hpp:15-17); emissivity/opacity/inverse_width/interp_criterion [P][L]
 * (index l + p*L, lines.tpp:8-10); nu [P][F] (index f + p*F, radiation.tpp:3-5);
 * ray_direction [nrays][3]; quad_* [nlspecs][Q]. */
typedef struct {
    uint32_t npoints, nrays, hnrays, nlines, nquads, nfreqs, nlspecs, nboundary;
    const double*   position;
    const double*   velocity;
    const uint32_t* n_neighbors;
    const uint32_t* cum_n_neighbors;
    const uint32_t* neighbors;
    const uint32_t* point2boundary;       /* npoints marks an interior point */
    const int32_t*  boundary_condition;   /* [nboundary] MgrBoundaryCondition */
    const double*   boundary_temperature; /* [nboundary] */
    const double*   ray_direction;
    const double*   ray_weight;           /* [nrays] */
    const uint32_t* antipod;              /* [nrays] */
    const double*   line;                 /* [L] line centre frequencies */
    const double*   sorted_line;          /* [L] ascending */
    const uint32_t* sorted_line_map;      /* [L] */
    double          max_inverse_mass;
    const double*   emissivity;
    const double*   opacity;
    const double*   inverse_width;
    const double*   interp_criterion;     /* opacity / population_tot */
    const double*   temperature;          /* [P] */
    const double*   vturb2;               /* [P] */
    const double*   dshift_max;           /* [P] */
    const double*   nu;                   /* [P][F] */
    const uint32_t* corr_line;            /* [F] global line of each frequency */
    const uint32_t* corr_lspec;           /* [F] */
    const uint32_t* corr_k;               /* [F] */
    const uint32_t* corr_z;               /* [F] */
    const uint8_t*  in_line_integral;     /* [F] */
    const uint32_t* nrad;                 /* [nlspecs] */
    const uint32_t* nrad_cum;             /* [nlspecs] */
    const double*   line_A;               /* [L] */
    const double*   lspec_inverse_mass;   /* [nlspecs] */
    const double*   quad_weights;         /* [nlspecs][Q] */
    const double*   quad_roots;           /* [nlspecs][Q] */
    double min_opacity;
    double min_dtau;
    double max_interpolation_diff;
    double max_distance_opacity_contribution;
    int32_t approx;                       /* MgrApprox */
    /* Parameters::spherical_symmetry (src/model/parameters/parameters.hpp:50): 1D model
     * of shells on the x axis in ascending radius (position [P][3] = (r, 0, 0)), rays in
     * the x-y plane; traced by Geometry::get_next_spherical_symmetry
     * (src/model/geometry/geometry.tpp:118-159) with the Z-dependent shifts of
     * get_shift_spherical_symmetry (:378-417).  The neighbour lists are not used. */
    int32_t spherical_symmetry;
    /* Rays::use_adaptive_directions (src/model/geometry/rays/rays.cpp:5-66): ray_direction
     * is [npoints][nrays][3] and ray_weight [npoints][nrays], ray r of origin o at
     * o * nrays + r (Rays::get_direction<true>, rays.cpp:94-146); antipod stays [nrays].
     * The formal solves, their ALO and set_column use the origin's rays; the imagers use
     * index r alone, as the reference's get_direction<false> does. */
    int32_t use_adaptive_directions;
} MgrModelDesc;

typedef struct MgrModel MgrModel;

/* Library / device state. */
const char* mgr_last_error(void);
int mgr_version(void);
int mgr_device_count(int* count);

/* Upload a model to the current CUDA device (host -> device copies, derived
 * per-edge and per-point tables).  Replaces the Paracabs host->device mirroring
 * (copy_vec_to_ptr) the reference's accelerated_for loops rely on. */
int mgr_model_create(const MgrModelDesc* desc, MgrModel** out);
void mgr_model_free(MgrModel* model);

/* Replace the per-(point, line) line data after new level populations
 * (Lines::set_emissivity_and_opacity, lines.tpp:29-40) or line widths
 * (Lines::set_inverse_width, lines.tpp:45-59).  Any pointer may be NULL to keep
 * the resident copy. */
int mgr_model_set_line_data(MgrModel* model, const double* emissivity, const double* opacity,
                            const double* inverse_width, const double* interp_criterion);

/* Longest ray pair in elements, including interpolation points
 * (Solver::get_ray_lengths_max, src/solver/solver.tpp:105-126). */
int mgr_ray_lengths_max(MgrModel* model, uint32_t* length);

/* Trace one ray pair (o, rr) for global line l, exactly as Solver::trace_ray_for_line
 * lays it out (solver.tpp:773-800): elements first..last with the origin at index
 * `centre` of the returned arrays (so centre = number of backward elements).
 * Arrays have room for `capacity` elements; *n_tot receives the element count.
 * dZ[i] is the distance between elements i and i+1. */
int mgr_trace_ray_pair(MgrModel* model, uint32_t o, uint32_t rr, uint32_t l, uint32_t capacity,
                       uint32_t* n_tot, uint32_t* centre, uint32_t* nr, uint32_t* nr_interp,
                       double* interp_factor, double* shift, double* dZ);

/* Model::compute_radiation_field_feautrier_order_2 (src/model/model.cpp:353-390 ->
 * Solver::solve_feautrier_order_2, src/solver/solver.tpp:458-540), n_off_diag = 0.
 * Host buffers (any may be NULL except J):
 *   J            [P][F]           mean intensity  (radiation.J)
 *   u            [hnrays][P][F]   Feautrier mean intensity per ray pair (radiation.u)
 *   lambda_diag  [P][L]           summed diagonal ALO element (Lambda::Ls, lambda.tpp:79-89)
 * The call blocks until the results are in host memory. */
int mgr_formal_solve_fo2(MgrModel* model, int precision, double* J, double* u, double* lambda_diag);

/* Device-resident variant: output pointers are device pointers; enqueued on the
 * model's stream and not synchronised.  Any of u / lambda_diag may be NULL. */
int mgr_formal_solve_fo2_device(MgrModel* model, int precision, double* J_dev, double* u_dev,
                                double* lambda_diag_dev);

/* Model::compute_radiation_field_feautrier_order_2_sparse (model.cpp:474-510 ->
 * Solver::solve_feautrier_order_2_sparse, solver.tpp:297-363), the memory-lean solve:
 * instead of J per frequency it returns the line-integrated mean intensity
 *   Jlin [P][L]  J(o, l) = sum_rr sum_z w_z (2 w_rr) u   (LineProducingSpecies::J, in
 *                the reference's order: ray pair outer, quadrature point inner)
 * and the ALO diagonal [P][L] (may be NULL).  Host buffers; blocks. */
int mgr_formal_solve_fo2_sparse(MgrModel* model, int precision, double* Jlin, double* lambda_diag);

/* Device-pointer variant; enqueued on the model's stream. */
int mgr_formal_solve_fo2_sparse_device(MgrModel* model, int precision, double* Jlin_dev, double* lambda_diag_dev);

/* Model::compute_radiation_field_feautrier_order_2_uv (model.cpp:395-433 ->
 * Solver::solve_feautrier_order_2_uv, solver.tpp:238-295, :2767-2921): u and v
 * [hnrays][P][F] per ray pair (radiation.u, radiation.v), v at the origin from the
 * u of its two neighbours (a boundary difference when the origin ends the ray; 0 for
 * a ray pair of one point).  Host buffers; blocks. */
int mgr_formal_solve_fo2_uv(MgrModel* model, int precision, double* u, double* v);

/* Model::compute_radiation_field_feautrier_order_2_anis (model.cpp:435-472 ->
 * Solver::solve_feautrier_order_2_anis, solver.tpp:366-456): per line, with
 * du = w_z w_rr u summed over ray pairs and quadrature points (ray pair outer):
 *   J [P][L]        sum 2 du                                 (LineProducingSpecies::J)
 *   J2_0            sum (3 n_z^2 - 1)/sqrt(2) du
 *   J2_1_Re, _Im    sum -sqrt(3) n_x n_z du, -sqrt(3) n_y n_z du
 *   J2_2_Re, _Im    sum sqrt(3)/2 (n_x^2 - n_y^2) du, sqrt(3) n_x n_y du
 * n the ray pair's direction.  Host buffers (all but J may be NULL); blocks. */
int mgr_formal_solve_fo2_anis(MgrModel* model, int precision, double* J, double* J2_0, double* J2_1_Re,
                              double* J2_1_Im, double* J2_2_Re, double* J2_2_Im);

/* Parameters::n_off_diag (src/model/parameters/parameters.hpp:66): the number of band
 * elements on each side of the origin that the formal solve adds to the ALO
 * (0, the default: the diagonal only; at most 4).  With n_off_diag > 0 the formal
 * solves of mgr_compute_level_populations run the banded FP64 solve and the global
 * rate system (below).  Replaces the reference's parameters->n_off_diag, read by
 * Solver::setup (src/solver/solver.tpp:6-36). */
int mgr_model_set_n_off_diag(MgrModel* model, uint32_t n_off_diag);

/* The formal solve with the non-local ALO (n_off_diag > 0, FP64): J_dev [P][F], u_dev
 * [hnrays][P][F] (may be NULL), the ALO diagonal lambda_diag_dev [P][L] as
 * mgr_formal_solve_fo2_device writes them, and the
 * band elements alo_off_dev / alo_nr_dev [P][L][hnrays][2 n_off_diag]: for origin p,
 * line l and ray pair rr, slot m < n_off_diag the update_Lambda term (summed over the
 * line's quadrature points) of the element centre - m - 1 of the ray and slot
 * n_off_diag + m that of centre + m + 1, with the element's point (a slot whose element
 * lies beyond the ray's end holds 0 and point 0).  The reference keeps these in
 * Lambda lists per (p, k) merged by point (Lambda::add_element,
 * src/model/lines/lineProducingSpecies/lambda/lambda.tpp:74-86), filled by
 * Solver::update_Lambda (src/solver/solver.tpp:1760-1850) from the banded inverse of
 * solve_feautrier_order_2 (solver.tpp:2319-2355).  Device pointers, model's stream. */
int mgr_formal_solve_fo2_alo_device(MgrModel* model, double* J_dev, double* u_dev, double* lambda_diag_dev,
                                    double* alo_off_dev, uint32_t* alo_nr_dev);

/* Host-buffer form of mgr_formal_solve_fo2_alo_device: J [P][F]; u [hnrays][P][F],
 * lambda_diag [P][L], alo_off and alo_nr (same layouts) may be NULL.  The band elements stay on the device
 * (model scratch) for a following mgr_compute_jeff, as the reference's Lambda lists
 * do for compute_Jeff.  Replaces Model::compute_radiation_field_feautrier_order_2
 * (src/model/model.cpp:353-390) with parameters->n_off_diag > 0. */
int mgr_formal_solve_fo2_alo(MgrModel* model, double* J, double* u, double* lambda_diag, double* alo_off,
                             uint32_t* alo_nr);

/* Partial formal solve over the ray pairs [rr_begin, rr_end) only: J_dev [P][F] and
 * lambda_diag_dev [P][L] (may be NULL) receive the sums over those ray pairs, so that
 * the sum over disjoint ranges covering [0, hnrays) is the full solve's J and ALO
 * diagonal up to the order of the additions.  This is the per-rank half of the
 * reference's multi-process formal solve: Solver::solve_feautrier_order_2 loops over
 * ray pairs (src/solver/solver.tpp:476), then combines the processes with
 * Radiation::MPI_reduce_J (solver.tpp:531 -> src/model/radiation/radiation.cpp:76-86)
 * and Lambda::MPI_gather (solver.tpp:537 ->
 * src/model/lines/lineProducingSpecies/lambda/lambda.tpp:121-206); here each shard
 * solves a block of ray pairs and the caller sums (e.g. an NCCL sum-allreduce).
 * Device pointers, enqueued on the model's stream. */
int mgr_formal_solve_fo2_rays_device(MgrModel* model, int precision, uint32_t rr_begin, uint32_t rr_end,
                                     double* J_dev, double* lambda_diag_dev);

/* Host-buffer variant of mgr_formal_solve_fo2_rays_device; blocks. */
int mgr_formal_solve_fo2_rays(MgrModel* model, int precision, uint32_t rr_begin, uint32_t rr_end, double* J,
                              double* lambda_diag);

/* Sum of the shards' partial J [nJ] and ALO diagonal [nlam] (device pointers, in
 * place), enqueued in order on `stream` (the model's cudaStream_t) or completed
 * before returning.  Returns 0 on success. */
typedef int (*mgr_reduce_fn)(void* user, double* J_dev, uint64_t nJ, double* lambda_diag_dev, uint64_t nlam,
                             void* stream);

/* Restricts the formal solves of mgr_compute_level_populations to the ray pairs
 * [rr_begin, rr_end) and sums the shards with `reduce` after each of them, before
 * Jeff and the rate equations, which every shard then runs on the same totals
 * (replicated statistical equilibrium).  reduce may not be NULL for a partial range.
 * capturable != 0 declares that reduce only enqueues stream work that a CUDA graph
 * capture can record (e.g. ncclAllReduce); otherwise the iterations run uncaptured.
 * rr_begin = 0, rr_end = hnrays and reduce = NULL restore the unsharded loop. */
int mgr_set_ray_shard(MgrModel* model, uint32_t rr_begin, uint32_t rr_end, mgr_reduce_fn reduce, void* user,
                      int capturable);

/* Model::compute_radiation_field_shortchar_order_0 (src/model/model.cpp:313-349 ->
 * Solver::solve_shortchar_order_0, src/solver/solver.tpp:150-235, :1564-1757).
 * Host buffers (any may be NULL except J):
 *   J            [P][F]
 *   I            [nrays][P][F]    intensity along each ray (radiation.I)
 *   u, v         [hnrays][P][F]   (I(rr) + I(ar))/2, (I(rr) - I(ar))/2
 *   lambda_diag  [P][L]           summed diagonal ALO element
 * Blocks until the results are in host memory. */
int mgr_formal_solve_sc0(MgrModel* model, int precision, double* J, double* I, double* u, double* v,
                         double* lambda_diag);

/* Device-pointer variant of mgr_formal_solve_sc0; enqueued on the model's stream. */
int mgr_formal_solve_sc0_device(MgrModel* model, int precision, double* J_dev, double* I_dev, double* u_dev,
                                double* v_dev, double* lambda_diag_dev);

/* Model::compute_image(ray_nr) (src/model/model.cpp:957-975 ->
 * Solver::image_feautrier_order_2(model, rr), src/solver/solver.tpp:542-574): the
 * rest-frame image along ray ray_nr with one ray per model point.
 *   I [P][F], ImX / ImY [P] image-plane coordinates (Image, image.cpp:154-219; may be
 *   NULL): the 3D plane of the ray, or (x, 0) for a spherically symmetric model (the
 *   reference's 1D rule, which a caller with other 1D models applies itself).
 *   CloseLines or None approximation (OneLine is rejected, as the reference does).
 *   Blocks. */
int mgr_image(MgrModel* model, int precision, uint32_t ray_nr, double* I, double* ImX, double* ImY);

/* Model::compute_image_new(raydir, nx, ny) (model.cpp:989-1013 ->
 * Solver::image_feautrier_order_2_new_imager, solver.tpp:576-627): nx * ny pixel rays
 * from a projection plane outside the model along the (normalised) direction raydir.
 *   I [nx*ny][F], ImX / ImY [nx*ny], pixel index y + ny*x (image.cpp:221-366).  Blocks. */
int mgr_image_new(MgrModel* model, int precision, const double* raydir, uint32_t nx, uint32_t ny, double* I,
                  double* ImX, double* ImY);

/* Model::compute_image_optical_depth(ray_nr) (model.cpp:1061-1079 ->
 * Solver::image_optical_depth, solver.tpp:655-684) and compute_image_optical_depth_new
 * (model.cpp:1081-1127 -> image_optical_depth_new_imager, solver.tpp:686-736): the
 * rays of mgr_image / mgr_image_new, I = the optical depth summed over the ray's pairs
 * (Solver::image_optical_depth(model, o, f), solver.tpp:2718-2760), 0 for a ray
 * without pairs.  Same arguments and outputs as mgr_image / mgr_image_new. */
int mgr_image_optical_depth(MgrModel* model, int precision, uint32_t ray_nr, double* I, double* ImX, double* ImY);
int mgr_image_optical_depth_new(MgrModel* model, int precision, const double* raydir, uint32_t nx, uint32_t ny,
                                double* I, double* ImX, double* ImY);

/* Model::compute_image_for_point(ray_nr, p) (src/model/model.cpp:1039-1058 ->
 * Solver::image_feautrier_order_2_for_point, src/solver/solver.tpp:629-653, :2582-2715):
 * the old imager's ray through point p along ray_nr (rest-frame shifts, all-line
 * interpolation points), eliminated and back-substituted along the whole ray.
 *  - *n_tot: the ray's element count (Model::S_ray / dtau_ray / u_ray rows).  With
 *    S_ray, dtau_ray, u_ray NULL and capacity 0 the call only returns it.
 *  - S_ray, dtau_ray, u_ray [capacity][nfreqs] host arrays: rows 0 .. n_tot-1 are
 *    written (row k = element first + k: the source at the far end of the pair ending
 *    there (row 0: the first pair's near end), that pair's optical depth (row 0: 0),
 *    and the Feautrier mean intensity u).  A ray of one element is written as zeros
 *    (the reference solves nothing there).  MGR_ERR_CAPACITY when n_tot > capacity.
 *  - OneLine is not supported for imaging (MGR_ERR_UNSUPPORTED), as in the reference. */
int mgr_image_for_point(MgrModel* model, int precision, uint32_t ray_nr, uint32_t p, uint32_t* n_tot, double* S_ray,
                        double* dtau_ray, double* u_ray, uint32_t capacity);

/* Model::set_column() (src/model/model.cpp:1143-1153 -> Solver::set_column / get_column,
 * src/solver/solver.tpp:2953-2991), general geometry with the model's own rays:
 * column [nrays][npoints] (host) = for each ray pair rr < hnrays and its antipode, the
 * trapezoid integral sum (density[crt] + density[nxt]) / 2 * dZ from each point to the
 * boundary (0 where the point has no next point); rows of rays no pair names are 0.
 * density [npoints] host (Model::density). */
int mgr_set_column(MgrModel* model, const double* density, double* column);

/* Same as mgr_formal_solve_fo2_device, but the call allocates no device memory.
 * No reference counterpart: an addition of this library for callers that cannot
 * allocate at solve time.
 * Per-ray results are staged in a fixed 64 MiB device array of the library (one
 * per device, shared by all models), processed in chunks of origins that fit.
 *  - Fails with MGR_ERR_CAPACITY if a single origin needs more than 64 MiB of
 *    staging, i.e. if hnrays * nfreqs * 8 * k > 64 MiB, where k = (u_dev == NULL) +
 *    (lambda_diag_dev != NULL).
 *  - The first call on a device looks up the array's address (a one-time set-up
 *    step); make it before any stream capture that includes this call.
 *  - Nothing in the staging array needs to start at zero.
 *  - Calls that run concurrently on one device (other threads, other models'
 *    streams) race on the shared array: serialise them. */
int mgr_formal_solve_fo2_device_noalloc(MgrModel* model, int precision, double* J_dev, double* u_dev,
                                        double* lambda_diag_dev);

/* ---- Differentiable new imager ---------------------------------------------------
 * No reference counterpart (the reference has no derivatives): a smooth FP64 form of
 * Model::compute_image_new (model.cpp:977-1013 -> Solver::image_feautrier_order_2_new_imager,
 * solver.tpp:576-627) and its adjoint.  The smooth form replaces the reference's
 * single-precision powf / expf / expm1f / erff by double-precision pow / exp / expm1 /
 * erf; the ray traces, interpolation points, CloseLines brackets, the large-shift
 * branch and the dtau clamp are held fixed (they are piecewise constant).  Device
 * pointers throughout; the calls block until done. */

/* Replaces the model's velocities (v/c, [P][3], device pointer). */
int mgr_model_set_velocity_device(MgrModel* model, const double* velocity_dev);

/* mgr_model_set_line_data with device pointers (any may be NULL to keep the resident
 * copy); the interpolation criterion is kept. */
int mgr_model_set_line_data_device(MgrModel* model, const double* emissivity_dev, const double* opacity_dev,
                                   const double* inverse_width_dev);

/* Smooth image: I_dev [nx*ny][F]; ImX / ImY host [nx*ny] (may be NULL). */
int mgr_image_new_smooth_device(MgrModel* model, const double* raydir, uint32_t nx, uint32_t ny, double* I_dev,
                                double* ImX, double* ImY);

/* Adjoint of mgr_image_new_smooth_device for d(loss)/d(I) = gI_dev [nx*ny][F]: adds
 * d(loss)/d(emissivity, opacity, inverse width, source emissivity/opacity) [P][L]
 * and d(loss)/d(velocity) [P][3] into the given device arrays (not zeroed). */
int mgr_image_new_adjoint_device(MgrModel* model, const double* raydir, uint32_t nx, uint32_t ny,
                                 const double* gI_dev, double* g_em_dev, double* g_op_dev, double* g_iw_dev,
                                 double* g_Sp_dev, double* g_vel_dev);

/* ---- Differentiable formal solve ---------------------------------------------------
 * No reference counterpart (the reference has no derivatives): a smooth FP64 form of
 * Model::compute_radiation_field_feautrier_order_2 (model.cpp:353-390 ->
 * Solver::solve_feautrier_order_2, solver.tpp:458-540, :2193-2318) and its adjoint, for
 * gradients of J.  As for the imager, the reference's single-precision powf / expf /
 * expm1f / erff become pow / exp / expm1 / erf, and the ray traces, interpolation
 * points, CloseLines brackets, the large-shift branch and the dtau clamp are held at
 * the model's state.  None and CloseLines approximations, general geometry (shared or
 * adaptive rays).  Device pointers; the calls block until done.
 * origins_dev: NULL for every origin, else n_origins origin indices (device array);
 * only those rows of J are written / only those rows of gJ are read. */

/* Replaces the model's frequencies nu [P][F] (device pointer), e.g. after the line
 * widths changed (Model::compute_spectral_discretisation, model.cpp:70-161). */
int mgr_model_set_frequencies_device(MgrModel* model, const double* nu_dev);

/* Puts the host's velocities (v/c, [P][3]) and frequencies nu [P][F] back on the
 * device if mgr_model_set_velocity_device or mgr_model_set_frequencies_device replaced
 * them since the model was created or last restored; otherwise does nothing.  A host
 * model that keeps its device copy between calls (the reference's Model methods run on
 * the model's own fields, model.cpp:353-390) calls it before a solve, so that a
 * differentiable solve run on the same device copy in between leaves no trace. */
int mgr_model_restore_inputs(MgrModel* model, const double* velocity, const double* nu);

/* Smooth J_dev [P][F]: J(o, f) = sum_rr 2 w_rr u(rr, o, f) in ray-pair order. */
int mgr_formal_solve_fo2_smooth_device(MgrModel* model, const uint32_t* origins_dev, uint32_t n_origins,
                                       double* J_dev);

/* Adjoint of mgr_formal_solve_fo2_smooth_device for d(loss)/d(J) = gJ_dev [P][F]: adds
 * d(loss)/d(emissivity, opacity, inverse width, source emissivity/opacity) [P][L],
 * d(loss)/d(velocity) [P][3] and d(loss)/d(nu) [P][F] into the given device arrays
 * (not zeroed). */
int mgr_formal_solve_fo2_adjoint_device(MgrModel* model, const uint32_t* origins_dev, uint32_t n_origins,
                                        const double* gJ_dev, double* g_em_dev, double* g_op_dev, double* g_iw_dev,
                                        double* g_Sp_dev, double* g_vel_dev, double* g_nu_dev);

/* ---- Many-model batch ------------------------------------------------------------
 * No single reference counterpart: the reference solves one Model per call
 * (Model::compute_radiation_field_feautrier_order_2, src/model/model.cpp:353-390);
 * a batch runs that call for many independent models with one persistent solve launch
 * and one reduction launch per wave of models (consecutive models whose staged per-ray
 * results fit the batch's staging area of up to 2 x 4 GiB; one wave for most batches).
 * Each model's J and ALO diagonal equal those of its own mgr_formal_solve_fo2 (same
 * lane code, same order of the sums; in FP64 mode up to a differently contracted
 * multiply-add). */
typedef struct MgrBatch MgrBatch;

/* Collects n_models models (same device, same line approximation, line spectral
 * discretisations, general geometry with shared rays: spherically symmetric models and
 * adaptive rays give MGR_ERR_UNSUPPORTED) into a batch.  The models stay owned by the
 * caller and must outlive the batch; their line data may change between solves. */
int mgr_batch_create(MgrModel* const* models, uint32_t n_models, MgrBatch** out);
void mgr_batch_free(MgrBatch* batch);

/* Launch shape of the batch kernel: CTAs of 256 threads per SM the register budget
 * is sized for (2, 3 or 4; 0 keeps) and warps per CTA (1..8; 0 keeps). */
int mgr_batch_set_tuning(MgrBatch* batch, int min_blocks_per_sm, int warps_per_block);

/* One formal solve of every model: J_dev[i] [P_i][F_i] and lambda_diag_dev[i]
 * [P_i][L_i] (device pointers; lambda_diag_dev or any of its entries may be NULL).
 * Enqueued on the batch's stream (mgr_batch_stream) after the models' own streams
 * are idle; returns once the launch is enqueued. */
int mgr_batch_formal_solve_fo2_device(MgrBatch* batch, int precision, double* const* J_dev,
                                      double* const* lambda_diag_dev);

/* Host-buffer variant (J[i] / lambda_diag[i] may be NULL to skip a result); blocks. */
int mgr_batch_formal_solve_fo2(MgrBatch* batch, int precision, double* const* J, double* const* lambda_diag);

/* Per-model timing of the last batch solve from the GPU's global timer, in ms since
 * the first CTA of the solve started: when the model's first ray pair started and
 * when its last origin was reduced.  Blocks until the solve is done. */
int mgr_batch_timings(MgrBatch* batch, double* start_ms, double* finish_ms);

/* The batch's CUDA stream (cudaStream_t). */
void* mgr_batch_stream(MgrBatch* batch);

/* Work counted over one formal solve (all origins, all ray pairs): trace steps,
 * neighbour records scanned by the trace (Geometry::get_next, geometry.tpp:22-38),
 * and ray-pair elements including interpolation points summed over lines
 * (the n_tot of solver.tpp:492-496 per line).  Used for algorithmic-byte counts. */
int mgr_ray_statistics(MgrModel* model, uint64_t* steps, uint64_t* neighbor_reads, uint64_t* elements);

/* Self-check of the ray trace (no reference counterpart; the reference's trace is
 * Geometry::get_next_general_geometry, src/model/geometry/geometry.tpp:13-44).  The
 * kernels pick each next point with an FP32 filter whose error bounds decide the
 * reference's FP64 argmin, falling back to the FP64 argmin on near ties.  This walks
 * every half ray (every origin, every ray) both ways and counts the rays, the steps and
 * the rays whose point sequence, edges or distance increments differ in any bit
 * (*mismatches, 0 when the filter is exact on this model).  Blocks until done.
 * Spherically symmetric models, and models whose ray directions are not unit vectors,
 * trace with the FP64 argmin alone: MGR_ERR_UNSUPPORTED. */
int mgr_trace_self_check(MgrModel* model, uint64_t* rays, uint64_t* steps, uint64_t* mismatches);

/* Launch shape of the formal-solve kernel for one precision mode: the register budget
 * (min_blocks_per_sm = 2, 3 or 4 CTAs of 256 threads per SM; 0 keeps the current value)
 * and warps per CTA for that precision (1..8; 0 keeps it).  Results do not depend on either; they are
 * picked by magritte_gb300.autotune for a given model. */
int mgr_set_tuning(MgrModel* model, int precision, int min_blocks_per_sm, int warps_per_block);

/* Time every launch shape of the formal-solve kernel for `precision` on a sample of
 * `sample_points` origins of this model (0 = 16384) and keep the fastest.  The shape
 * is also remembered for the model's device and that precision: models created later
 * in the process start from it (a fresh upload of the same model reuses the tuning).
 * Without a tuning a model starts from the shapes measured fastest on GB300 for the
 * 64^3 benchmark model (split: 4 CTAs x 8 warps, FP64: 2 CTAs x 4 warps).  Outputs may
 * be NULL.  Blocks until done. */
int mgr_autotune_fo2(MgrModel* model, int precision, uint32_t sample_points, int* best_min_blocks,
                     int* best_warps, float* best_ms);

/* ------------------------------------------------------------------------------
 * Level populations: compute_Jeff and the ALI loop (compute_level_populations).
 * ------------------------------------------------------------------------------ */

/* One collision partner of a species (CollisionPartner, collisionPartner.hpp).
 * Rates in m^3/s, [ntmp][ncol] row-major; icol = upper, jcol = lower level. */
typedef struct {
    uint32_t        num_col_partner;  /* abundance column of the partner        */
    int32_t         ortho_para;       /* orth_or_para_H2: 0 'n', 1 'o', 2 'p'   */
    uint32_t        ncol, ntmp;
    const uint32_t* icol;
    const uint32_t* jcol;
    const double*   tmp;              /* [ntmp] ascending                       */
    const double*   Cd;               /* de-excitation                          */
    const double*   Ce;               /* excitation                             */
} MgrCollisionPartnerDesc;

/* One line-producing species (Linedata, linedata.hpp).  Its lines are the global
 * lines nrad_cum .. nrad_cum + nrad - 1 of the model, in order; irad = upper,
 * jrad = lower level of each radiative transition.  nlev <= 64. */
typedef struct {
    uint32_t        num;              /* abundance column of the species        */
    uint32_t        nlev, nrad, ncolpar;
    const double*   energy;           /* [nlev] J                               */
    const double*   weight;           /* [nlev]                                 */
    const uint32_t* irad;             /* [nrad]                                 */
    const uint32_t* jrad;
    const double*   A;
    const double*   Bs;
    const double*   Ba;
    const double*   frequency;
    const MgrCollisionPartnerDesc* colpar;  /* [ncolpar] */
} MgrSpeciesDesc;

/* Parameters of Model::compute_level_populations (parameters.hpp:76-104). */
typedef struct {
    double   pop_prec;                          /* 1e-6  */
    double   min_rel_pop_for_convergence;       /* 1e-10 */
    double   convergence_fraction;              /* 0.995 */
    double   population_inversion_fraction;     /* -1    */
    double   min_line_opacity;                  /* 1e-13 */
    double   min_line_emissivity;               /* 1e-50 */
    uint32_t Ng_acceleration_mem_limit;         /* 9, at most 16 */
    uint32_t adaptive_Ng_acceleration_min_order;/* 2     */
    uint32_t Ng_acceleration_remove_N_its;      /* 0     */
    int32_t  use_adaptive_Ng_acceleration;      /* 1     */
    int32_t  adaptive_Ng_acceleration_use_max_criterion; /* 1 */
} MgrAliParams;

/* Attach the line-producing species, abundances [P][nspecs] (number densities, the
 * reference's chemistry.species.abundance) and current level populations (one
 * [P][nlev] array per species) to a model.  Replaces earlier species data and
 * starts a fresh population history (LineProducingSpecies::populations). */
int mgr_model_set_species(MgrModel* model, uint32_t nlspecs, const MgrSpeciesDesc* species, uint32_t nspecs,
                          const double* abundance, const double* const* populations);

/* Model::compute_Jeff (model.cpp:514-545) from the J and ALO of the last formal solve
 * on this model (its buffers must still be valid for the device entry points), with
 * the band elements when that solve was a banded one (mgr_formal_solve_fo2_alo*).
 * Outputs of species l, [P][nrad] each; any may be NULL.  Blocks. */
int mgr_compute_jeff(MgrModel* model, uint32_t l, double* Jlin, double* Jeff, double* Jdif);

/* Model::compute_level_populations(use_ng, max_it) (model.cpp:654-747): formal
 * solves in `precision`, Jeff, statistical equilibrium, corrections and Ng
 * acceleration until convergence, all on the device.  *iterations receives the
 * number of normal iterations; error_mean / error_max (may be NULL, room for
 * err_capacity values) receive relative_change_mean / _max per normal iteration and
 * species, as Model::error_mean / error_max.  Populations stay on the device
 * (mgr_get_populations); the line emissivities and opacities are updated.
 * With n_off_diag > 0 (mgr_model_set_n_off_diag) every iteration runs the banded FP64
 * formal solve (precision must be MGR_PRECISION_FP64; no ray-pair shard), Jeff with the
 * band elements, and the global rate system of each species
 * (lineProducingSpecies.tpp:377-581, the reference's Eigen SparseLU): here
 * BiCGSTAB preconditioned by the per-point blocks' LU factors, on unknowns scaled by
 * each point's population_tot, to a max-norm residual of 1e-13 of the right-hand
 * side (MGR_ERR_NONFINITE above 1e-9 after 200 iterations). */
int mgr_compute_level_populations(MgrModel* model, int precision, int use_ng, long max_iterations,
                                  const MgrAliParams* params, int* iterations, double* error_mean,
                                  double* error_max, uint32_t err_capacity);

/* Model::compute_level_populations_sparse (model.cpp:756-850): the same ALI loop with
 * the memory-lean formal solve and compute_Jeff_sparse (model.cpp:549-570; Jlin taken
 * from the solve, Jdif left unchanged) and the per-point rate solve of
 * update_using_statistical_equilibrium_sparse (lineProducingSpecies.tpp:589-705).
 * MGR_ERR_UNSUPPORTED with n_off_diag > 0, as the reference throws
 * (lineProducingSpecies.tpp:592-593). */
int mgr_compute_level_populations_sparse(MgrModel* model, int precision, int use_ng, long max_iterations,
                                         const MgrAliParams* params, int* iterations, double* error_mean,
                                         double* error_max, uint32_t err_capacity);

/* Model::compute_Jeff_sparse (model.cpp:549-570) for species l after
 * mgr_formal_solve_fo2_sparse: Jlin, Jeff [P][nrad] (host, may be NULL). */
int mgr_compute_jeff_sparse(MgrModel* model, uint32_t l, double* Jlin, double* Jeff);

/* Device time of the phases of the last mgr_compute_level_populations(_sparse) call on
 * this model (no reference counterpart), ms[4] summed over its iterations: the formal
 * solves (with the ray-shard reduce), compute_Jeff, the statistical equilibrium with the
 * population corrections, convergence statistics and line-data refresh, and the Ng
 * acceleration steps.  The iterations' events are recorded inside the captured graph.
 * MGR_ERR_UNSUPPORTED when the timing was not available. */
int mgr_ali_phase_times(MgrModel* model, double* ms);

/* Copy species l's level populations [P][nlev] to the host. */
int mgr_get_populations(MgrModel* model, uint32_t l, double* populations);

/* Copy the current line emissivity and opacity [P][L] to the host (either may be NULL). */
int mgr_get_line_data(MgrModel* model, double* emissivity, double* opacity);

/* Block until all work on the model's stream has finished; returns the first
 * kernel-side status recorded since the last call (trace / capacity / non-finite). */
int mgr_sync(MgrModel* model);

/* The model's CUDA stream (a cudaStream_t), for callers that time or order work. */
void* mgr_model_stream(MgrModel* model);

/* Number of this library's kernel launches so far (all models, all streams). */
uint64_t mgr_launch_count(void);

/* Measured issue rate of one instruction kind on the current device, for the
 * benchmark's FP64-pipe roofline (no reference counterpart: the reference has no GPU
 * path).  kind: 0 DFMA, 1 DADD, 2 DMUL, 3 DSETP (FP64 compare), 4 F2F (FP64 <-> FP32
 * conversion), 5 MUFU.RCP64H (rcp.approx.ftz.f64).  Eight independent chains per
 * thread, `iterations` steps each, over SMs x 8 CTAs of 256 threads; the best of three
 * timed launches.  Outputs (any may be NULL): thread operations per second for the
 * whole device, thread operations per SM clock cycle per SM (each SM's span from its
 * first CTA's start to its last CTA's end on its own clock64), and the launch time in
 * ms.  Blocks. */
int mgr_measure_pipe_rate(int kind, uint32_t iterations, double* thread_ops_per_s,
                          double* thread_ops_per_clk_per_sm, float* ms);

#ifdef __cplusplus
}
#endif

#endif /* MAGRITTE_GB300_H */
