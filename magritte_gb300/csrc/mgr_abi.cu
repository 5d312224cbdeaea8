// C ABI of libmgr_gpu.so: model upload, formal-solve entry points, status handling.
#include <atomic>
#include <mutex>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "mgr_ali.h"
#include "mgr_internal.h"

namespace mgr {

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches{0};

void set_error(const std::string& msg) { g_last_error = msg; }

int cuda_fail(cudaError_t e, const char* what) {
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return MGR_ERR_CUDA;
}

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

template <typename T>
static cudaError_t dalloc(MgrModel* m, T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T));
    if (e != cudaSuccess) return e;
    m->allocations.push_back(q);
    *p = static_cast<T*>(q);
    return cudaSuccess;
}

template <typename T>
static cudaError_t upload(MgrModel* m, const T** dst, const T* src, size_t count) {
    T* p = nullptr;
    cudaError_t e = dalloc(m, &p, count);
    if (e != cudaSuccess) return e;
    if (count) e = cudaMemcpyAsync(p, src, count * sizeof(T), cudaMemcpyHostToDevice, m->stream);
    *dst = p;
    return e;
}

int decode_status(int st) {
    if (st & ST_TRACE) {
        set_error("ray left the point cloud on an interior point (neighbour lists or boundary incomplete)");
        return MGR_ERR_TRACE;
    }
    if (st & ST_CAPACITY) {
        set_error("capacity exceeded: a ray longer than the sized ray buffer, or an interpolation count above "
                  "the per-edge table's 65535 (an interpolation-criterion jump too large for FP32)");
        return MGR_ERR_CAPACITY;
    }
    if (st & ST_NONFINITE) {
        set_error("non-finite intensity in a ray-pair solve");
        return MGR_ERR_NONFINITE;
    }
    return MGR_OK;
}

static int read_status(MgrModel* model) {
    int st = 0;
    cudaError_t e = cudaMemcpyAsync(&st, model->status, sizeof(int), cudaMemcpyDeviceToHost, model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "status read");
    e = cudaStreamSynchronize(model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "stream synchronize");
    e = cudaMemsetAsync(model->status, 0, sizeof(int), model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "status reset");
    return decode_status(st);
}

static int ensure_scratch(MgrModel* m, double** p, size_t* have, size_t bytes) {
    if (*have >= bytes) return MGR_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *have = 0;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "scratch allocation");
    *p = static_cast<double*>(q);
    *have = bytes;
    return MGR_OK;
}

// FP32 table scales of split precision (see mgr_scale.h); NULL keeps a scale.
static void apply_scales(MgrModel* m, const double* em, const double* op) {
    const size_t n = (size_t)m->dm.P * m->dm.L;
    set_line_scales(m, em ? pow2_scale_for_max(em, n) : m->scales.Ke, op ? pow2_scale_for_max(op, n) : m->scales.Ko);
}

void set_line_scales(MgrModel* m, double Ke, double Ko) {
    m->scales.Ke = Ke;
    m->scales.Ko = Ko;
    m->dm.min_op_s = (float)(m->dm.min_opacity * m->scales.Ko);
    m->dm.dz_scale = (float)(1.0 / m->scales.Ko);
    m->dm.s_scale = (float)(m->scales.Ko / m->scales.Ke);
}

// One correctly rounded erff table per device (51 MB), shared by every model on it.
static std::mutex g_erf_mutex;
static const float* g_erf_band[64] = {};

cudaError_t erf_band_table(const float** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_erf_mutex);
    if (!g_erf_band[dev]) {
        int nsm = 1;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        void* p = nullptr;
        e = cudaMalloc(&p, (size_t)kErfBandCount * sizeof(float));
        if (e != cudaSuccess) return e;
        cudaStream_t s = nullptr;
        e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = fill_erf_band(static_cast<float*>(p), s, nsm);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (s) cudaStreamDestroy(s);
        if (e != cudaSuccess) {
            cudaFree(p);
            return e;
        }
        g_erf_band[dev] = static_cast<const float*>(p);
    }
    *out = g_erf_band[dev];
    return cudaSuccess;
}

// Formal-solve launch shapes last picked by mgr_autotune_fo2, per device and precision
// (0: none yet): models created later in the process start from them.
static std::mutex g_tuned_mutex;
static int g_tuned[64][2][2] = {};

static void remember_tuned_shape(int dev, int precision, int minb, int warps) {
    if (dev < 0 || dev >= 64) return;
    std::lock_guard<std::mutex> lock(g_tuned_mutex);
    const int k = precision == MGR_PRECISION_SPLIT ? 1 : 0;
    g_tuned[dev][k][0] = minb;
    g_tuned[dev][k][1] = warps;
}

static void apply_tuned_shapes(MgrModel* m) {
    if (m->device < 0 || m->device >= 64) return;
    std::lock_guard<std::mutex> lock(g_tuned_mutex);
    const int(*t)[2] = g_tuned[m->device];
    if (t[0][0]) {
        m->fo2_minb_fp64 = t[0][0];
        m->fo2_warps_fp64 = t[0][1];
    }
    if (t[1][0]) {
        m->fo2_minb_split = t[1][0];
        m->fo2_warps_split = t[1][1];
    }
}

static int size_model(MgrModel* model) {
    uint32_t* d_max = nullptr;
    constexpr size_t nmax = 1 + kLenClasses;
    cudaError_t e = cudaMalloc(&d_max, nmax * sizeof(uint32_t));
    if (e != cudaSuccess) return cuda_fail(e, "sizing allocation");
    cudaMemsetAsync(d_max, 0, nmax * sizeof(uint32_t), model->stream);
    e = launch_size_rays(model, d_max);
    uint32_t mx[nmax] = {};
    if (e == cudaSuccess) e = cudaMemcpyAsync(mx, d_max, sizeof(mx), cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    cudaFree(d_max);
    if (e != cudaSuccess) return cuda_fail(e, "ray sizing");
    int st = read_status(model);
    if (st != MGR_OK) return st;
    model->half_cap = mx[0] > 0 ? mx[0] : 1;
    for (int c = 0; c < kLenClasses; c++) model->class_cap[c] = mx[1 + c];
    return MGR_OK;
}

}  // namespace mgr

using namespace mgr;

extern "C" {

const char* mgr_last_error(void) { return g_last_error.c_str(); }

int mgr_version(void) { return 1; }

uint64_t mgr_launch_count(void) { return g_launches.load(); }

int mgr_device_count(int* count) {
    if (!count) return MGR_ERR_ARGUMENT;
    cudaError_t e = cudaGetDeviceCount(count);
    if (e != cudaSuccess) {
        *count = 0;
        set_error(std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e));
        return MGR_ERR_NO_DEVICE;
    }
    return MGR_OK;
}

void mgr_model_free(MgrModel* model) {
    if (!model) return;
    DeviceScope on_device(model->device);
    if (model->stream) cudaStreamSynchronize(model->stream);
    for (void* p : model->allocations) cudaFree(p);
    if (model->J_scratch) cudaFree(model->J_scratch);
    if (model->u_scratch) cudaFree(model->u_scratch);
    if (model->lam_scratch) cudaFree(model->lam_scratch);
    if (model->work) cudaFree(model->work);
    if (model->adj_scratch) cudaFree(model->adj_scratch);
    if (model->v_scratch) cudaFree(model->v_scratch);
    if (model->alo_scratch) cudaFree(model->alo_scratch);
    if (model->alo_nr_scratch) cudaFree(model->alo_nr_scratch);
    ali_free(model);
    if (model->stream) cudaStreamDestroy(model->stream);
    delete model;
}

int mgr_model_create(const MgrModelDesc* d, MgrModel** out) {
    if (!d || !out) {
        set_error("mgr_model_create: null argument");
        return MGR_ERR_ARGUMENT;
    }
    *out = nullptr;
    if (d->npoints == 0 || d->nrays < 2 || d->hnrays * 2 != d->nrays || d->nlines == 0 || d->nquads == 0 ||
        d->nfreqs == 0 || d->nlspecs == 0) {
        set_error("mgr_model_create: inconsistent sizes (npoints, nrays = 2*hnrays, nlines, nquads, nfreqs, nlspecs)");
        return MGR_ERR_ARGUMENT;
    }
    if (!d->position || !d->velocity || !d->n_neighbors || !d->cum_n_neighbors || !d->neighbors ||
        !d->point2boundary || !d->ray_direction || !d->ray_weight || !d->antipod || !d->line || !d->sorted_line ||
        !d->sorted_line_map || !d->emissivity || !d->opacity || !d->inverse_width || !d->interp_criterion ||
        !d->temperature || !d->vturb2 || !d->dshift_max || !d->nu || !d->corr_line || !d->corr_lspec || !d->corr_k ||
        !d->corr_z || !d->in_line_integral || !d->nrad_cum || !d->line_A || !d->lspec_inverse_mass ||
        !d->quad_weights) {
        set_error("mgr_model_create: a required array is null");
        return MGR_ERR_ARGUMENT;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        set_error("mgr_model_create: no CUDA device");
        return MGR_ERR_NO_DEVICE;
    }
    const uint32_t P = d->npoints, L = d->nlines, F = d->nfreqs;
    // neighbour count and index checks (host side, before anything reaches the GPU)
    size_t E = 0;
    for (uint32_t p = 0; p < P; p++) {
        if ((size_t)d->cum_n_neighbors[p] != E) {
            set_error("mgr_model_create: cum_n_neighbors is not the prefix sum of n_neighbors");
            return MGR_ERR_ARGUMENT;
        }
        E += d->n_neighbors[p];
    }
    for (size_t i = 0; i < E; i++) {
        if (d->neighbors[i] >= P) {
            set_error("mgr_model_create: neighbour index out of range");
            return MGR_ERR_ARGUMENT;
        }
    }
    for (uint32_t p = 0; p < P; p++) {
        if (d->point2boundary[p] != P && d->point2boundary[p] >= d->nboundary) {
            set_error("mgr_model_create: point2boundary out of range");
            return MGR_ERR_ARGUMENT;
        }
    }
    for (uint32_t r = 0; r < d->nrays; r++) {
        if (d->antipod[r] >= d->nrays) {
            set_error("mgr_model_create: antipod index out of range");
            return MGR_ERR_ARGUMENT;
        }
    }
    // A line spectral discretisation (compute_spectral_discretisation(), model.cpp:70-161)
    // has every frequency mapped to (species, transition, quadrature point); the imaging
    // ones (model.cpp:165-275) leave the maps unset and serve only the imagers.
    bool line_disc = (F == L * d->nquads);
    for (uint32_t f = 0; f < F && line_disc; f++)
        if (d->corr_line[f] >= L || d->corr_lspec[f] >= d->nlspecs || d->corr_z[f] >= d->nquads) line_disc = false;
    // the line each frequency is measured from in split precision: its own line, or
    // for an imaging discretisation the nearest line
    std::vector<uint32_t> corr_line(F);
    for (uint32_t f = 0; f < F; f++) {
        if (line_disc) {
            corr_line[f] = d->corr_line[f];
        } else {
            uint32_t best = 0;
            for (uint32_t l = 1; l < L; l++)
                if (std::fabs(d->nu[f] - d->line[l]) < std::fabs(d->nu[f] - d->line[best])) best = l;
            corr_line[f] = best;
        }
    }

    MgrModel* m = new MgrModel();
    m->line_disc = line_disc;
    m->host_pos.assign(d->position, d->position + 3 * (size_t)P);
    m->host_p2b.assign(d->point2boundary, d->point2boundary + P);
    m->host_raydir.assign(d->ray_direction, d->ray_direction + 3 * (size_t)d->nrays);
    cudaGetDevice(&m->device);
    cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, m->device);
    if (m->sm_count < 1) m->sm_count = 1;
    apply_tuned_shapes(m);
    cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete m;
        return cuda_fail(e, "stream creation");
    }
    DevModel& dm = m->dm;
    dm.P = P;
    dm.nrays = d->nrays;
    dm.hnrays = d->hnrays;
    dm.L = L;
    dm.Q = d->nquads;
    dm.F = F;
    dm.nlspecs = d->nlspecs;
    dm.B = d->nboundary;
    dm.max_inv_mass = d->max_inverse_mass;
    dm.min_opacity = d->min_opacity;
    dm.min_dtau = d->min_dtau;
    dm.max_interp_diff = d->max_interpolation_diff;
    dm.max_dist = d->max_distance_opacity_contribution;
    dm.max_dist_f = (float)dm.max_dist;
    dm.log_max_interp_diff = logf((float)d->max_interpolation_diff);
    dm.approx = d->approx;
    dm.sph = d->spherical_symmetry ? 1u : 0u;
    dm.adaptive = d->use_adaptive_directions ? 1u : 0u;
    // ray directions / weights: per point with adaptive directions (Rays::read, rays.cpp:33-45)
    const size_t NR = (size_t)d->nrays * (dm.adaptive ? P : 1);
    m->n_edges = E;
    // interpolation-table slots: one per CSR edge, or three per point in spherical symmetry
    const size_t ET = dm.sph ? 3 * (size_t)P : E;

    // host-side derived tables
    std::vector<double4_32a> pos4(P), vel4(P);
    double maxabs = 0.0;
    for (uint32_t p = 0; p < P; p++) {
        pos4[p] = make_double4_32a(d->position[3 * p], d->position[3 * p + 1], d->position[3 * p + 2], 0.0);
        vel4[p] = make_double4_32a(d->velocity[3 * p], d->velocity[3 * p + 1], d->velocity[3 * p + 2], 0.0);
        for (int k = 0; k < 3; k++) maxabs = std::max(maxabs, std::fabs(d->position[3 * p + k]));
    }
    // power of two that brings every coordinate into [-1, 1] (trace filter tables)
    int pexp = 0;
    if (maxabs > 0.0 && std::isfinite(maxabs)) std::frexp(maxabs, &pexp);
    dm.pos_scale = std::ldexp(1.0, -pexp);
    // the trace filter's bounds take unit ray directions (|d|^2 = 1 within 2e-15, as
    // HEALPix and rotated directions are); other models trace with the exact argmin only
    bool unit_rays = true;
    for (size_t i = 0; i < NR && unit_rays; i++) {
        const double* v = d->ray_direction + 3 * i;
        unit_rays = std::fabs(v[0] * v[0] + v[1] * v[1] + v[2] * v[2] - 1.0) <= 2.0e-15;
    }
    // the neighbour records (position + index) are packed on the device from the points
    // and the CSR lists: check the indices here
    for (size_t i = 0; i < E; i++)
        if (d->neighbors[i] >= P) {
            mgr_model_free(m);
            set_error("mgr_model_create: neighbour index out of range");
            return MGR_ERR_ARGUMENT;
        }
    std::vector<double> ub(P);
    for (uint32_t p = 0; p < P; p++)
        ub[p] = std::sqrt(TWO_KB_OVER_AMU_CC_SQUARED * d->max_inverse_mass * d->temperature[p] + d->vturb2[p]);
    std::vector<float> dsm_f(P), ub_f(P);
    for (uint32_t p = 0; p < P; p++) {
        dsm_f[p] = (float)d->dshift_max[p];
        ub_f[p] = (float)ub[p];
    }
    std::vector<float> dls, dll;
    line_offset_tables(d->line, d->sorted_line, L, dls, dll);
    std::vector<float> bkt(2 * (size_t)d->nboundary);  // h / (k T) per boundary, double-float
    for (uint32_t b = 0; b < d->nboundary; b++) {
        const double k = HH_OVER_KB / (d->boundary_condition[b] == BC_THERMAL ? d->boundary_temperature[b] : T_CMB);
        bkt[2 * b] = (float)k;
        bkt[2 * b + 1] = (float)(k - (double)bkt[2 * b]);
    }
    std::vector<float> line_df(2 * (size_t)L);  // double-float line centres (hi, lo)
    for (uint32_t l = 0; l < L; l++) {
        line_df[2 * l] = (float)d->line[l];
        line_df[2 * l + 1] = (float)(d->line[l] - (double)line_df[2 * l]);
    }
    std::vector<uint32_t> lq2f((size_t)L * d->nquads, 0xffffffffu);
    for (uint32_t f = 0; f < F; f++) {
        const size_t i = (size_t)d->corr_line[f] * d->nquads + d->corr_z[f];
        if (d->corr_line[f] < L && d->corr_z[f] < d->nquads) lq2f[i] = f;
    }

    const size_t PL = (size_t)P * L;
    do {
        if ((e = upload(m, &dm.pos, pos4.data(), P)) != cudaSuccess) break;
        if ((e = upload(m, &dm.vel, vel4.data(), P)) != cudaSuccess) break;
        if ((e = upload(m, &dm.n_nb, d->n_neighbors, P)) != cudaSuccess) break;
        if ((e = upload(m, &dm.cum_nb, d->cum_n_neighbors, P)) != cudaSuccess) break;
        {
            const uint32_t* nbr = nullptr;
            double4_32a* edge = nullptr;
            if ((e = upload(m, &nbr, d->neighbors, E)) != cudaSuccess) break;
            if ((e = dalloc(m, &edge, E ? E : 1)) != cudaSuccess) break;
            if ((e = launch_edge_pack(m, dm.pos, nbr, E, edge)) != cudaSuccess) break;
            dm.edge = edge;
        }
        if ((e = upload(m, &dm.p2b, d->point2boundary, P)) != cudaSuccess) break;
        if ((e = upload(m, &dm.bc, d->boundary_condition, d->nboundary)) != cudaSuccess) break;
        if ((e = upload(m, &dm.bt, d->boundary_temperature, d->nboundary)) != cudaSuccess) break;
        if ((e = upload(m, &dm.bkt, bkt.data(), 2 * (size_t)d->nboundary)) != cudaSuccess) break;
        if ((e = upload(m, &dm.raydir, d->ray_direction, 3 * NR)) != cudaSuccess) break;
        if ((e = upload(m, &dm.rayw, d->ray_weight, NR)) != cudaSuccess) break;
        if ((e = upload(m, &dm.antipod, d->antipod, d->nrays)) != cudaSuccess) break;
        if ((e = upload(m, &dm.line, d->line, L)) != cudaSuccess) break;
        if ((e = upload(m, &dm.sorted_line, d->sorted_line, L)) != cudaSuccess) break;
        if ((e = upload(m, &dm.sorted_map, d->sorted_line_map, L)) != cudaSuccess) break;
        if ((e = upload(m, &dm.dls, dls.data(), (size_t)L * L)) != cudaSuccess) break;
        if ((e = upload(m, &dm.lq2f, lq2f.data(), lq2f.size())) != cudaSuccess) break;
        if ((e = upload(m, &dm.dll, dll.data(), (size_t)L * L)) != cudaSuccess) break;
        if ((e = upload(m, &dm.line_df, line_df.data(), line_df.size())) != cudaSuccess) break;
        if ((e = dalloc(m, &m->em, PL)) != cudaSuccess) break;
        if ((e = dalloc(m, &m->op, PL)) != cudaSuccess) break;
        if ((e = dalloc(m, &m->iw, PL)) != cudaSuccess) break;
        if ((e = dalloc(m, &m->Sp, PL)) != cudaSuccess) break;
        if ((e = dalloc(m, &m->crit, PL)) != cudaSuccess) break;
        if ((e = dalloc(m, &m->em_f, PL)) != cudaSuccess) break;
        if ((e = dalloc(m, &m->op_f, PL)) != cudaSuccess) break;
        if ((e = dalloc(m, &m->iw_f, PL)) != cudaSuccess) break;
        if ((e = dalloc(m, &m->Sp_f, PL)) != cudaSuccess) break;
        if ((e = dalloc(m, &m->iw_lo, PL)) != cudaSuccess) break;
        if ((e = dalloc(m, &m->nint, (ET ? ET : 1) * (size_t)L)) != cudaSuccess) break;
        if ((e = dalloc(m, &m->nint_all, ET ? ET : 1)) != cudaSuccess) break;
        if ((e = dalloc(m, &m->pair_class, (size_t)P * d->hnrays)) != cudaSuccess) break;
        {
            float4* ehl = nullptr;
            float4* phl = nullptr;
            if ((e = dalloc(m, &ehl, 2 * (E ? E : 1))) != cudaSuccess) break;
            if ((e = dalloc(m, &phl, 2 * (size_t)P)) != cudaSuccess) break;
            dm.edge_hl = unit_rays ? ehl : nullptr;
            dm.pos_hl = phl;
        }
        if ((e = cudaMemcpyAsync(m->em, d->emissivity, PL * 8, cudaMemcpyHostToDevice, m->stream)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(m->op, d->opacity, PL * 8, cudaMemcpyHostToDevice, m->stream)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(m->iw, d->inverse_width, PL * 8, cudaMemcpyHostToDevice, m->stream)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(m->crit, d->interp_criterion, PL * 8, cudaMemcpyHostToDevice, m->stream)) != cudaSuccess) break;
        if ((e = upload(m, &dm.ub, ub.data(), P)) != cudaSuccess) break;
        if ((e = upload(m, &dm.ub_f, ub_f.data(), P)) != cudaSuccess) break;
        if ((e = upload(m, &dm.T, d->temperature, P)) != cudaSuccess) break;
        if ((e = upload(m, &dm.vt2, d->vturb2, P)) != cudaSuccess) break;
        if ((e = upload(m, &dm.dshift_max, d->dshift_max, P)) != cudaSuccess) break;
        if ((e = upload(m, &dm.dshift_max_f, dsm_f.data(), P)) != cudaSuccess) break;
        if ((e = upload(m, &dm.nu, d->nu, (size_t)P * F)) != cudaSuccess) break;
        if ((e = upload(m, &dm.corr_line, corr_line.data(), F)) != cudaSuccess) break;
        if ((e = upload(m, &dm.corr_lspec, d->corr_lspec, F)) != cudaSuccess) break;
        if ((e = upload(m, &dm.corr_k, d->corr_k, F)) != cudaSuccess) break;
        if ((e = upload(m, &dm.corr_z, d->corr_z, F)) != cudaSuccess) break;
        if ((e = upload(m, &dm.in_line, d->in_line_integral, F)) != cudaSuccess) break;
        if ((e = upload(m, &dm.nrad_cum, d->nrad_cum, d->nlspecs)) != cudaSuccess) break;
        if ((e = upload(m, &dm.line_A, d->line_A, L)) != cudaSuccess) break;
        if ((e = upload(m, &dm.lspec_inv_mass, d->lspec_inverse_mass, d->nlspecs)) != cudaSuccess) break;
        if ((e = upload(m, &dm.quad_w, d->quad_weights, (size_t)d->nlspecs * d->nquads)) != cudaSuccess) break;
        if ((e = dalloc(m, &m->status, 1)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(m->status, 0, sizeof(int), m->stream)) != cudaSuccess) break;
    } while (false);
    if (e != cudaSuccess) {
        int rc = cuda_fail(e, "model upload");
        mgr_model_free(m);
        return rc;
    }
    dm.em = m->em;
    dm.op = m->op;
    dm.iw = m->iw;
    dm.Sp = m->Sp;
    dm.crit = m->crit;
    dm.em_f = m->em_f;
    dm.op_f = m->op_f;
    dm.iw_f = m->iw_f;
    dm.Sp_f = m->Sp_f;
    dm.iw_lo = m->iw_lo;
    if ((e = erf_band_table(&dm.erf_band)) != cudaSuccess) {
        int rc = cuda_fail(e, "erff table");
        mgr_model_free(m);
        return rc;
    }
    dm.nint = m->nint;
    dm.nint_all = m->nint_all;
    apply_scales(m, d->emissivity, d->opacity);
    if ((e = launch_line_tables(m)) != cudaSuccess || (e = launch_nint_table(m)) != cudaSuccess ||
        (e = launch_hl_tables(m)) != cudaSuccess) {
        int rc = cuda_fail(e, "line tables");
        mgr_model_free(m);
        return rc;
    }
    int rc = size_model(m);
    if (rc != MGR_OK) {
        mgr_model_free(m);
        return rc;
    }
    *out = m;
    return MGR_OK;
}

int mgr_model_set_line_data(MgrModel* model, const double* emissivity, const double* opacity,
                            const double* inverse_width, const double* interp_criterion) {
    MGR_MODEL_DEVICE(model);
    if (!model) {
        set_error("mgr_model_set_line_data: null model");
        return MGR_ERR_ARGUMENT;
    }
    const size_t bytes = (size_t)model->dm.P * model->dm.L * 8;
    cudaError_t e = cudaSuccess;
    if (emissivity && e == cudaSuccess) e = cudaMemcpyAsync(model->em, emissivity, bytes, cudaMemcpyHostToDevice, model->stream);
    if (opacity && e == cudaSuccess) e = cudaMemcpyAsync(model->op, opacity, bytes, cudaMemcpyHostToDevice, model->stream);
    if (inverse_width && e == cudaSuccess) e = cudaMemcpyAsync(model->iw, inverse_width, bytes, cudaMemcpyHostToDevice, model->stream);
    if (interp_criterion && e == cudaSuccess) e = cudaMemcpyAsync(model->crit, interp_criterion, bytes, cudaMemcpyHostToDevice, model->stream);
    apply_scales(model, emissivity, opacity);
    if (e == cudaSuccess) e = launch_line_tables(model);
    if (e == cudaSuccess && interp_criterion) e = launch_nint_table(model);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "line data update");
    return MGR_OK;
}

int mgr_model_restore_inputs(MgrModel* model, const double* velocity, const double* nu) {
    MGR_MODEL_DEVICE(model);
    if (!model || !velocity || !nu) {
        set_error("mgr_model_restore_inputs: null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (!model->inputs_replaced) return MGR_OK;
    const uint32_t P = model->dm.P;
    std::vector<double4_32a> vel4(P);
    for (uint32_t p = 0; p < P; p++)
        vel4[p] = make_double4_32a(velocity[3 * p], velocity[3 * p + 1], velocity[3 * p + 2], 0.0);
    cudaError_t e = cudaMemcpyAsync(const_cast<double4_32a*>(model->dm.vel), vel4.data(), P * sizeof(double4_32a),
                                    cudaMemcpyHostToDevice, model->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(const_cast<double*>(model->dm.nu), nu, (size_t)P * model->dm.F * 8, cudaMemcpyHostToDevice,
                            model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);  // vel4 is read by the copy
    if (e != cudaSuccess) return cuda_fail(e, "input restore");
    model->inputs_replaced = false;
    return MGR_OK;
}

int mgr_ray_lengths_max(MgrModel* model, uint32_t* length) {
    MGR_MODEL_DEVICE(model);
    if (!model || !length) {
        set_error("mgr_ray_lengths_max: null argument");
        return MGR_ERR_ARGUMENT;
    }
    uint32_t* d_max = nullptr;
    cudaError_t e = cudaMalloc(&d_max, sizeof(uint32_t));
    if (e != cudaSuccess) return cuda_fail(e, "allocation");
    cudaMemsetAsync(d_max, 0, sizeof(uint32_t), model->stream);
    e = launch_ray_lengths(model, d_max);
    uint32_t mx = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&mx, d_max, sizeof(uint32_t), cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    cudaFree(d_max);
    if (e != cudaSuccess) return cuda_fail(e, "ray lengths");
    int st = read_status(model);
    if (st != MGR_OK) return st;
    *length = mx;
    return MGR_OK;
}

int mgr_trace_ray_pair(MgrModel* model, uint32_t o, uint32_t rr, uint32_t l, uint32_t capacity, uint32_t* n_tot,
                       uint32_t* centre, uint32_t* nr, uint32_t* nr_interp, double* interp_factor, double* shift,
                       double* dZ) {
    MGR_MODEL_DEVICE(model);
    if (!model || !n_tot || !centre || !nr || !nr_interp || !interp_factor || !shift || !dZ || capacity == 0) {
        set_error("mgr_trace_ray_pair: null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (o >= model->dm.P || rr >= model->dm.hnrays || l >= model->dm.L) {
        set_error("mgr_trace_ray_pair: index out of range");
        return MGR_ERR_ARGUMENT;
    }
    uint32_t* d_meta = nullptr;
    uint32_t *d_nr = nullptr, *d_ni = nullptr;
    double *d_fac = nullptr, *d_shift = nullptr, *d_dZ = nullptr;
    cudaError_t e = cudaMalloc(&d_meta, 3 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&d_nr, capacity * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&d_ni, capacity * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&d_fac, capacity * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_shift, capacity * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_dZ, capacity * sizeof(double));
    if (e == cudaSuccess) e = cudaMemsetAsync(d_dZ, 0, capacity * sizeof(double), model->stream);
    if (e == cudaSuccess) e = launch_trace_export(model, o, rr, l, capacity, d_meta, d_nr, d_ni, d_fac, d_shift, d_dZ);
    uint32_t meta[3] = {0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(meta, d_meta, sizeof(meta), cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    int rc = MGR_OK;
    if (e != cudaSuccess) rc = cuda_fail(e, "trace export");
    if (rc == MGR_OK && meta[2] == 2) {
        set_error("mgr_trace_ray_pair: capacity too small");
        rc = MGR_ERR_CAPACITY;
    }
    if (rc == MGR_OK) {
        int st = read_status(model);
        if (st != MGR_OK) rc = st;
    }
    if (rc == MGR_OK) {
        const size_t n = meta[0];
        *n_tot = meta[0];
        *centre = meta[1];
        e = cudaMemcpy(nr, d_nr, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(nr_interp, d_ni, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(interp_factor, d_fac, n * sizeof(double), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(shift, d_shift, n * sizeof(double), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(dZ, d_dZ, n * sizeof(double), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cuda_fail(e, "trace export copy");
    }
    cudaFree(d_meta);
    cudaFree(d_nr);
    cudaFree(d_ni);
    cudaFree(d_fac);
    cudaFree(d_shift);
    cudaFree(d_dZ);
    return rc;
}

int mgr_formal_solve_fo2_device(MgrModel* model, int precision, double* J_dev, double* u_dev,
                                double* lambda_diag_dev) {
    MGR_MODEL_DEVICE(model);
    if (!model || !J_dev) {
        set_error("mgr_formal_solve_fo2_device: null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) {
        set_error("mgr_formal_solve_fo2_device: unknown precision mode");
        return MGR_ERR_ARGUMENT;
    }
    if (!model->line_disc) {
        set_error("mgr_formal_solve_fo2_device: the formal solve needs a line spectral discretisation "
                  "(nfreqs = nlines*nquads with every frequency mapped to its line)");
        return MGR_ERR_UNSUPPORTED;
    }
    const size_t wb = fo2_work_bytes(model, model->dm.P, u_dev == nullptr, lambda_diag_dev != nullptr);
    int rc = ensure_scratch(model, &model->work, &model->work_bytes, wb);
    if (rc != MGR_OK) return rc;
    cudaError_t e = launch_fo2_range(model, precision, 0, model->dm.P, J_dev, u_dev, lambda_diag_dev, model->work,
                                     model->work_bytes);
    if (e != cudaSuccess) return cuda_fail(e, "formal solve launch");
    model->last_J = J_dev;
    model->last_lam = lambda_diag_dev;
    model->last_alo_off = nullptr;
    model->last_alo_nr = nullptr;
    return MGR_OK;
}

int mgr_model_set_n_off_diag(MgrModel* model, uint32_t n_off_diag) {
    MGR_MODEL_DEVICE(model);
    if (!model) {
        set_error("mgr_model_set_n_off_diag: null model");
        return MGR_ERR_ARGUMENT;
    }
    if (n_off_diag > kMaxOffDiag) {
        set_error("mgr_model_set_n_off_diag: n_off_diag = " + std::to_string(n_off_diag) + " above the supported " +
                  std::to_string(kMaxOffDiag));
        return MGR_ERR_UNSUPPORTED;
    }
    model->dm.n_off_diag = n_off_diag;
    if (model->ali) ali_shard_changed(model);  // drop a captured ALI iteration
    return MGR_OK;
}

int mgr_formal_solve_fo2_alo_device(MgrModel* model, double* J_dev, double* u_dev, double* lambda_diag_dev,
                                    double* alo_off_dev, uint32_t* alo_nr_dev) {
    MGR_MODEL_DEVICE(model);
    if (!model || !J_dev || !lambda_diag_dev || !alo_off_dev || !alo_nr_dev) {
        set_error("mgr_formal_solve_fo2_alo_device: null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (model->dm.n_off_diag == 0) {
        set_error("mgr_formal_solve_fo2_alo_device: n_off_diag is 0 (mgr_model_set_n_off_diag)");
        return MGR_ERR_ARGUMENT;
    }
    if (!model->line_disc) {
        set_error("mgr_formal_solve_fo2_alo_device: the formal solve needs a line spectral discretisation");
        return MGR_ERR_UNSUPPORTED;
    }
    const size_t wb = fo2_work_bytes(model, model->dm.P, true, true);
    int rc = ensure_scratch(model, &model->work, &model->work_bytes, wb);
    if (rc != MGR_OK) return rc;
    cudaError_t e = launch_fo2_range(model, MGR_PRECISION_FP64, 0, model->dm.P, J_dev, u_dev, lambda_diag_dev,
                                     model->work, model->work_bytes, 0, 0xffffffffu, nullptr, nullptr, nullptr,
                                     alo_off_dev, alo_nr_dev);
    if (e != cudaSuccess) return cuda_fail(e, "banded formal solve launch");
    model->last_J = J_dev;
    model->last_lam = lambda_diag_dev;
    model->last_alo_off = alo_off_dev;
    model->last_alo_nr = alo_nr_dev;
    return MGR_OK;
}

int mgr_formal_solve_fo2_alo(MgrModel* model, double* J, double* u, double* lambda_diag, double* alo_off,
                             uint32_t* alo_nr) {
    MGR_MODEL_DEVICE(model);
    if (!model || !J) {
        set_error("mgr_formal_solve_fo2_alo: null argument");
        return MGR_ERR_ARGUMENT;
    }
    const DevModel& dm = model->dm;
    const size_t PF = (size_t)dm.P * dm.F, PL = (size_t)dm.P * dm.L;
    const size_t nalo = PL * dm.hnrays * 2 * (dm.n_off_diag ? dm.n_off_diag : 1);
    int rc = ensure_scratch(model, &model->J_scratch, &model->J_scratch_bytes, PF * 8);
    if (rc == MGR_OK) rc = ensure_scratch(model, &model->lam_scratch, &model->lam_scratch_bytes, PL * 8);
    if (rc == MGR_OK) rc = ensure_scratch(model, &model->alo_scratch, &model->alo_scratch_bytes, nalo * 8);
    if (rc == MGR_OK) rc = ensure_scratch(model, &model->alo_nr_scratch, &model->alo_nr_scratch_bytes, nalo * 4);
    if (rc == MGR_OK && u) rc = ensure_scratch(model, &model->u_scratch, &model->u_scratch_bytes, PF * dm.hnrays * 8);
    if (rc != MGR_OK) return rc;
    uint32_t* nr_dev = reinterpret_cast<uint32_t*>(model->alo_nr_scratch);
    rc = mgr_formal_solve_fo2_alo_device(model, model->J_scratch, u ? model->u_scratch : nullptr, model->lam_scratch,
                                         model->alo_scratch, nr_dev);
    if (rc != MGR_OK) return rc;
    cudaError_t e = cudaMemcpyAsync(J, model->J_scratch, PF * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && u)
        e = cudaMemcpyAsync(u, model->u_scratch, PF * dm.hnrays * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && lambda_diag)
        e = cudaMemcpyAsync(lambda_diag, model->lam_scratch, PL * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && alo_off)
        e = cudaMemcpyAsync(alo_off, model->alo_scratch, nalo * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && alo_nr)
        e = cudaMemcpyAsync(alo_nr, nr_dev, nalo * 4, cudaMemcpyDeviceToHost, model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "result copy");
    return read_status(model);
}

int mgr_formal_solve_fo2_rays_device(MgrModel* model, int precision, uint32_t rr_begin, uint32_t rr_end,
                                     double* J_dev, double* lambda_diag_dev) {
    MGR_MODEL_DEVICE(model);
    if (!model || !J_dev) {
        set_error("mgr_formal_solve_fo2_rays_device: null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) {
        set_error("mgr_formal_solve_fo2_rays_device: unknown precision mode");
        return MGR_ERR_ARGUMENT;
    }
    if (rr_begin >= rr_end || rr_end > model->dm.hnrays) {
        set_error("mgr_formal_solve_fo2_rays_device: ray-pair range [" + std::to_string(rr_begin) + ", " +
                  std::to_string(rr_end) + ") is empty or beyond hnrays = " + std::to_string(model->dm.hnrays));
        return MGR_ERR_ARGUMENT;
    }
    if (!model->line_disc) {
        set_error("mgr_formal_solve_fo2_rays_device: the formal solve needs a line spectral discretisation");
        return MGR_ERR_UNSUPPORTED;
    }
    const size_t wb = fo2_work_bytes(model, model->dm.P, true, lambda_diag_dev != nullptr);
    int rc = ensure_scratch(model, &model->work, &model->work_bytes, wb);
    if (rc != MGR_OK) return rc;
    cudaError_t e = launch_fo2_range(model, precision, 0, model->dm.P, J_dev, nullptr, lambda_diag_dev, model->work,
                                     model->work_bytes, rr_begin, rr_end);
    if (e != cudaSuccess) return cuda_fail(e, "partial formal solve launch");
    return MGR_OK;
}

int mgr_formal_solve_fo2_rays(MgrModel* model, int precision, uint32_t rr_begin, uint32_t rr_end, double* J,
                              double* lambda_diag) {
    MGR_MODEL_DEVICE(model);
    if (!model || !J) {
        set_error("mgr_formal_solve_fo2_rays: null argument");
        return MGR_ERR_ARGUMENT;
    }
    const DevModel& dm = model->dm;
    const size_t PF = (size_t)dm.P * dm.F;
    int rc = ensure_scratch(model, &model->J_scratch, &model->J_scratch_bytes, PF * 8);
    if (rc != MGR_OK) return rc;
    if (lambda_diag &&
        (rc = ensure_scratch(model, &model->lam_scratch, &model->lam_scratch_bytes, (size_t)dm.P * dm.L * 8)) != MGR_OK)
        return rc;
    rc = mgr_formal_solve_fo2_rays_device(model, precision, rr_begin, rr_end, model->J_scratch,
                                          lambda_diag ? model->lam_scratch : nullptr);
    if (rc != MGR_OK) return rc;
    cudaError_t e = cudaMemcpyAsync(J, model->J_scratch, PF * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && lambda_diag)
        e = cudaMemcpyAsync(lambda_diag, model->lam_scratch, (size_t)dm.P * dm.L * 8, cudaMemcpyDeviceToHost,
                            model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "result copy");
    return read_status(model);
}

int mgr_set_ray_shard(MgrModel* model, uint32_t rr_begin, uint32_t rr_end, mgr_reduce_fn reduce, void* user,
                      int capturable) {
    MGR_MODEL_DEVICE(model);
    if (!model) {
        set_error("mgr_set_ray_shard: null model");
        return MGR_ERR_ARGUMENT;
    }
    if (rr_begin >= rr_end || rr_end > model->dm.hnrays) {
        set_error("mgr_set_ray_shard: ray-pair range is empty or beyond hnrays");
        return MGR_ERR_ARGUMENT;
    }
    const bool full = rr_begin == 0 && rr_end == model->dm.hnrays;
    if (!full && !reduce) {
        set_error("mgr_set_ray_shard: a partial ray-pair range needs a reduce function");
        return MGR_ERR_ARGUMENT;
    }
    model->shard_begin = rr_begin;
    model->shard_end = rr_end;
    model->shard_reduce = reduce;
    model->shard_user = user;
    model->shard_capturable = capturable != 0;
    ali_shard_changed(model);
    return MGR_OK;
}

int mgr_formal_solve_fo2_sparse_device(MgrModel* model, int precision, double* Jlin_dev, double* lambda_diag_dev) {
    MGR_MODEL_DEVICE(model);
    if (!model || !Jlin_dev) {
        set_error("mgr_formal_solve_fo2_sparse_device: null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) {
        set_error("mgr_formal_solve_fo2_sparse_device: unknown precision mode");
        return MGR_ERR_ARGUMENT;
    }
    if (!model->line_disc) {
        set_error("mgr_formal_solve_fo2_sparse_device: the formal solve needs a line spectral discretisation");
        return MGR_ERR_UNSUPPORTED;
    }
    const size_t wb = fo2_work_bytes(model, model->dm.P, true, lambda_diag_dev != nullptr);
    int rc = ensure_scratch(model, &model->work, &model->work_bytes, wb);
    if (rc != MGR_OK) return rc;
    cudaError_t e = launch_fo2_range(model, precision, 0, model->dm.P, nullptr, nullptr, lambda_diag_dev, model->work,
                                     model->work_bytes, 0, model->dm.hnrays, Jlin_dev);
    if (e != cudaSuccess) return cuda_fail(e, "memory-lean formal solve launch");
    model->last_J = nullptr;
    model->last_Jlin = Jlin_dev;
    model->last_lam = lambda_diag_dev;
    model->last_alo_off = nullptr;
    model->last_alo_nr = nullptr;
    return MGR_OK;
}

int mgr_formal_solve_fo2_sparse(MgrModel* model, int precision, double* Jlin, double* lambda_diag) {
    MGR_MODEL_DEVICE(model);
    if (!model || !Jlin) {
        set_error("mgr_formal_solve_fo2_sparse: null argument");
        return MGR_ERR_ARGUMENT;
    }
    const DevModel& dm = model->dm;
    const size_t PL = (size_t)dm.P * dm.L;
    // the line-integrated J lives in the J scratch (>= P*L doubles), the ALO in the lambda scratch
    int rc = ensure_scratch(model, &model->J_scratch, &model->J_scratch_bytes,
                            std::max(PL, (size_t)dm.P * dm.F) * 8);
    if (rc != MGR_OK) return rc;
    if ((rc = ensure_scratch(model, &model->lam_scratch, &model->lam_scratch_bytes, PL * 8)) != MGR_OK) return rc;
    rc = mgr_formal_solve_fo2_sparse_device(model, precision, model->J_scratch, model->lam_scratch);
    if (rc != MGR_OK) return rc;
    cudaError_t e = cudaMemcpyAsync(Jlin, model->J_scratch, PL * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && lambda_diag)
        e = cudaMemcpyAsync(lambda_diag, model->lam_scratch, PL * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "result copy");
    return read_status(model);
}

int mgr_formal_solve_fo2_anis(MgrModel* model, int precision, double* J, double* J2_0, double* J2_1_Re,
                              double* J2_1_Im, double* J2_2_Re, double* J2_2_Im) {
    MGR_MODEL_DEVICE(model);
    if (!model || !J) {
        set_error("mgr_formal_solve_fo2_anis: null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) {
        set_error("mgr_formal_solve_fo2_anis: unknown precision mode");
        return MGR_ERR_ARGUMENT;
    }
    if (!model->line_disc) {
        set_error("mgr_formal_solve_fo2_anis: the formal solve needs a line spectral discretisation");
        return MGR_ERR_UNSUPPORTED;
    }
    const DevModel& dm = model->dm;
    const size_t PL = (size_t)dm.P * dm.L;
    int rc = ensure_scratch(model, &model->work, &model->work_bytes, fo2_work_bytes(model, dm.P, true, false));
    if (rc != MGR_OK) return rc;
    // the six [P][L] results live in the u scratch
    if ((rc = ensure_scratch(model, &model->u_scratch, &model->u_scratch_bytes, 6 * PL * 8)) != MGR_OK) return rc;
    cudaError_t e = launch_fo2_range(model, precision, 0, dm.P, nullptr, nullptr, nullptr, model->work,
                                     model->work_bytes, 0, dm.hnrays, nullptr, model->u_scratch);
    double* outs[6] = {J, J2_0, J2_1_Re, J2_1_Im, J2_2_Re, J2_2_Im};
    for (int k = 0; k < 6 && e == cudaSuccess; k++)
        if (outs[k]) e = cudaMemcpyAsync(outs[k], model->u_scratch + k * PL, PL * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "anisotropic formal solve");
    return read_status(model);
}

int mgr_formal_solve_fo2_uv(MgrModel* model, int precision, double* u, double* v) {
    MGR_MODEL_DEVICE(model);
    if (!model || !u || !v) {
        set_error("mgr_formal_solve_fo2_uv: null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) {
        set_error("mgr_formal_solve_fo2_uv: unknown precision mode");
        return MGR_ERR_ARGUMENT;
    }
    if (!model->line_disc) {
        set_error("mgr_formal_solve_fo2_uv: the formal solve needs a line spectral discretisation");
        return MGR_ERR_UNSUPPORTED;
    }
    const DevModel& dm = model->dm;
    const size_t RPF = (size_t)dm.hnrays * dm.P * dm.F;
    int rc = ensure_scratch(model, &model->u_scratch, &model->u_scratch_bytes, RPF * 8);
    if (rc != MGR_OK) return rc;
    if ((rc = ensure_scratch(model, &model->v_scratch, &model->v_scratch_bytes, RPF * 8)) != MGR_OK) return rc;
    // the solve writes u and v directly; J and the ALO are not part of this call
    cudaError_t e = launch_fo2_range(model, precision, 0, dm.P, nullptr, model->u_scratch, nullptr, nullptr, 0, 0,
                                     dm.hnrays, nullptr, nullptr, model->v_scratch);
    if (e == cudaSuccess) e = cudaMemcpyAsync(u, model->u_scratch, RPF * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(v, model->v_scratch, RPF * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "uv formal solve");
    return read_status(model);
}

int mgr_formal_solve_fo2(MgrModel* model, int precision, double* J, double* u, double* lambda_diag) {
    MGR_MODEL_DEVICE(model);
    if (!model || !J) {
        set_error("mgr_formal_solve_fo2: null argument");
        return MGR_ERR_ARGUMENT;
    }
    const DevModel& dm = model->dm;
    const size_t PF = (size_t)dm.P * dm.F;
    int rc = ensure_scratch(model, &model->J_scratch, &model->J_scratch_bytes, PF * 8);
    if (rc != MGR_OK) return rc;
    if (u && (rc = ensure_scratch(model, &model->u_scratch, &model->u_scratch_bytes, PF * dm.hnrays * 8)) != MGR_OK)
        return rc;
    if (lambda_diag &&
        (rc = ensure_scratch(model, &model->lam_scratch, &model->lam_scratch_bytes, (size_t)dm.P * dm.L * 8)) != MGR_OK)
        return rc;
    rc = mgr_formal_solve_fo2_device(model, precision, model->J_scratch, u ? model->u_scratch : nullptr,
                                     lambda_diag ? model->lam_scratch : nullptr);
    if (rc != MGR_OK) return rc;
    cudaError_t e = cudaMemcpyAsync(J, model->J_scratch, PF * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && u)
        e = cudaMemcpyAsync(u, model->u_scratch, PF * dm.hnrays * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && lambda_diag)
        e = cudaMemcpyAsync(lambda_diag, model->lam_scratch, (size_t)dm.P * dm.L * 8, cudaMemcpyDeviceToHost,
                            model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "result copy");
    return read_status(model);
}

int mgr_ray_statistics(MgrModel* model, uint64_t* steps, uint64_t* neighbor_reads, uint64_t* elements) {
    MGR_MODEL_DEVICE(model);
    if (!model || !steps || !neighbor_reads || !elements) {
        set_error("mgr_ray_statistics: null argument");
        return MGR_ERR_ARGUMENT;
    }
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMalloc(&d, 3 * sizeof(unsigned long long));
    if (e != cudaSuccess) return cuda_fail(e, "allocation");
    unsigned long long h[3] = {0, 0, 0};
    e = cudaMemsetAsync(d, 0, sizeof(h), model->stream);
    if (e == cudaSuccess) e = launch_ray_stats(model, d);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "ray statistics");
    int st = read_status(model);
    if (st != MGR_OK) return st;
    *steps = h[0];
    *neighbor_reads = h[1];
    *elements = h[2];
    return MGR_OK;
}

int mgr_trace_self_check(MgrModel* model, uint64_t* rays, uint64_t* steps, uint64_t* mismatches) {
    MGR_MODEL_DEVICE(model);
    if (!model || !rays || !steps || !mismatches) {
        set_error("mgr_trace_self_check: null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (model->dm.sph || !model->dm.edge_hl) {
        set_error("mgr_trace_self_check: this model traces with the exact argmin only (spherical symmetry, or ray "
                  "directions that are not unit vectors)");
        return MGR_ERR_UNSUPPORTED;
    }
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMalloc(&d, 3 * sizeof(unsigned long long));
    if (e != cudaSuccess) return cuda_fail(e, "allocation");
    unsigned long long h[3] = {0, 0, 0};
    e = cudaMemsetAsync(d, 0, sizeof(h), model->stream);
    if (e == cudaSuccess) e = launch_trace_check(model, d);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "trace self-check");
    int st = read_status(model);
    if (st != MGR_OK) return st;
    *rays = h[0];
    *steps = h[1];
    *mismatches = h[2];
    return MGR_OK;
}

int mgr_set_tuning(MgrModel* model, int precision, int min_blocks_per_sm, int warps_per_block) {
    MGR_MODEL_DEVICE(model);
    if (!model || (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) ||
        (min_blocks_per_sm != 0 && (min_blocks_per_sm < 2 || min_blocks_per_sm > 4)) || warps_per_block < 0 ||
        warps_per_block > 8) {
        set_error("mgr_set_tuning: min_blocks_per_sm must be 2..4 (0 keeps it), warps_per_block 1..8 (0 keeps it)");
        return MGR_ERR_ARGUMENT;
    }
    const bool split = precision == MGR_PRECISION_SPLIT;
    if (min_blocks_per_sm) (split ? model->fo2_minb_split : model->fo2_minb_fp64) = min_blocks_per_sm;
    if (warps_per_block) (split ? model->fo2_warps_split : model->fo2_warps_fp64) = warps_per_block;
    return MGR_OK;
}

int mgr_autotune_fo2(MgrModel* model, int precision, uint32_t sample_points, int* best_min_blocks, int* best_warps,
                     float* best_ms) {
    MGR_MODEL_DEVICE(model);
    if (!model || (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT)) {
        set_error("mgr_autotune_fo2: invalid argument");
        return MGR_ERR_ARGUMENT;
    }
    const DevModel& dm = model->dm;
    uint32_t n = sample_points ? sample_points : 16384;
    if (n > dm.P) n = dm.P;
    // an evenly spread sample of origins: a contiguous block from the middle of the index range
    const uint32_t o0 = (dm.P - n) / 2, o1 = o0 + n;
    int rc = ensure_scratch(model, &model->J_scratch, &model->J_scratch_bytes, (size_t)dm.P * dm.F * 8);
    if (rc != MGR_OK) return rc;
    rc = ensure_scratch(model, &model->work, &model->work_bytes, fo2_work_bytes(model, n, true, false));
    if (rc != MGR_OK) return rc;
    int& minb = precision == MGR_PRECISION_SPLIT ? model->fo2_minb_split : model->fo2_minb_fp64;
    int& nwarps = precision == MGR_PRECISION_SPLIT ? model->fo2_warps_split : model->fo2_warps_fp64;
    const int keep_minb = minb, keep_warps = nwarps;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int bm = keep_minb, bw = keep_warps;
    const int minbs[3] = {2, 3, 4};
    const int warps[2] = {4, 8};
    cudaError_t e = cudaSuccess;
    for (int mi = 0; mi < 3 && e == cudaSuccess; mi++) {
        for (int wi = 0; wi < 2 && e == cudaSuccess; wi++) {
            minb = minbs[mi];
            nwarps = warps[wi];
            e = launch_fo2_range(model, precision, o0, o1, model->J_scratch, nullptr, nullptr, model->work,
                                 model->work_bytes);  // warm
            if (e == cudaSuccess) e = cudaEventRecord(e0, model->stream);
            if (e == cudaSuccess)
                e = launch_fo2_range(model, precision, o0, o1, model->J_scratch, nullptr, nullptr, model->work,
                                     model->work_bytes);
            if (e == cudaSuccess) e = cudaEventRecord(e1, model->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (e == cudaSuccess && ms < best) {
                best = ms;
                bm = minbs[mi];
                bw = warps[wi];
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) {
        minb = keep_minb;
        nwarps = keep_warps;
        return cuda_fail(e, "autotune");
    }
    minb = bm;
    nwarps = bw;
    remember_tuned_shape(model->device, precision, bm, bw);
    if (best_min_blocks) *best_min_blocks = bm;
    if (best_warps) *best_warps = bw;
    if (best_ms) *best_ms = best;
    return read_status(model);
}

int mgr_sync(MgrModel* model) {
    MGR_MODEL_DEVICE(model);
    if (!model) {
        set_error("mgr_sync: null model");
        return MGR_ERR_ARGUMENT;
    }
    return read_status(model);
}

void* mgr_model_stream(MgrModel* model) { return model ? (void*)model->stream : nullptr; }

}  // extern "C"
