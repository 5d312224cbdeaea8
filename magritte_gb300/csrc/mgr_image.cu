// Imagers: Model::compute_image (src/model/model.cpp:957-975, the old imager: one ray
// per model point, Solver::image_feautrier_order_2(model, rr), solver.tpp:542-574) and
// Model::compute_image_new (model.cpp:977-1013, pixel rays from a projection plane,
// Solver::image_feautrier_order_2_new_imager, solver.tpp:576-627).
//
// Both run one warp per ray (model point or pixel), lanes over frequencies: the warp
// traces the ray into shared memory and every lane eliminates over the whole ray
// (image_lane).  The image-plane geometry (axes, pixel coordinates, the projection
// surface) is set up on the host from the model's positions, as Image does
// (src/model/image/image.cpp:154-398).
#include <cmath>
#include <cstring>
#include <algorithm>
#include <vector>

#include "mgr_image.cuh"

namespace mgr {

// ---------------------------------------------------------------------------------
// Old imager: warp per model point o, ray rr / antipode, rest-frame shifts.
// ---------------------------------------------------------------------------------
template <int MODE, int AP, bool TAU>
__global__ void __launch_bounds__(256) image_kernel(DevModel m, uint32_t cap, uint32_t rr, double* __restrict__ I,
                                                    int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nw = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* sl = reinterpret_cast<double*>(smem);
    const uint32_t Lpad = (m.L + 1) & ~1u;
    HalfSmem bk, fw;
    carve_halves(smem + (size_t)Lpad * 8 + (size_t)w * half_bytes_per_warp(cap), cap, bk, fw);
    for (uint32_t i = threadIdx.x; i < m.L; i += blockDim.x) sl[i] = m.sorted_line[i];
    __syncthreads();
    const uint32_t ar = m.antipod[rr];
    for (uint32_t o = blockIdx.x * nw + w; o < m.P; o += gridDim.x * nw) {
        // Geometry::get_shift<Rest, false>(o, r, o, 0): the origin's shift along each
        // half's own ray (the antipode's is reversed), the element's that of rr
        const double shb = origin_shift(m, 1, o, rr);
        const double shf = origin_shift(m, 1, o, ar);
        bk.shift0 = shb;
        fw.shift0 = shf;
        set_dsh0(bk, shb);
        set_dsh0(fw, shf);
        bk.cshift = fw.cshift = shb;
        int nb = 0, nf = 0;
        trace_pair<true, 1>(m, o, rr, ar, cap, bk, fw, lane, status, nb, nf);
        if (nb < 0 || nf < 0) continue;
        for (uint32_t f0 = 0; f0 < m.F; f0 += 32) {
            const uint32_t f = f0 + lane;
            if (f < m.F) {
                const LaneCtx c = lane_ctx(m, o, f);
                const double v = image_lane<MODE, AP, TAU>(m, sl, c, bk, nb, fw, nf);
                I[(size_t)o * m.F + f] = v;
                if (!isfinite(v)) atomicOr(status, ST_NONFINITE);
            }
        }
        __syncwarp();
    }
}

template <int MODE, int AP, bool TAU>
__global__ void __launch_bounds__(256) image_new_kernel(DevModel m, ImagePlane ip, uint32_t cap,
                                                        double* __restrict__ I, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nw = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* sl = reinterpret_cast<double*>(smem);
    const uint32_t Lpad = (m.L + 1) & ~1u;
    HalfSmem bk, fw;
    carve_halves(smem + (size_t)Lpad * 8 + (size_t)w * half_bytes_per_warp(cap), cap, bk, fw);
    for (uint32_t i = threadIdx.x; i < m.L; i += blockDim.x) sl[i] = m.sorted_line[i];
    __syncthreads();
    const uint32_t npix = ip.nx * ip.ny;
    for (uint32_t px = blockIdx.x * nw + w; px < npix; px += gridDim.x * nw) {
        double org[3];
        pixel_origin(ip, ip.ImX[px], ip.ImY[px], org);
        double Z;
        const uint32_t start = pixel_start(m, org, ip, lane, Z);
        const double sh0 = image_shift(m, org, ip, start, Z);
        bk.shift0 = fw.shift0 = bk.cshift = fw.cshift = sh0;
        set_dsh0(bk, sh0);
        set_dsh0(fw, sh0);
        const int nb = trace_image<true>(m, org, ip, start, Z, cap, bk, lane, status);
        if (nb < 0) continue;
        for (uint32_t f0 = 0; f0 < m.F; f0 += 32) {
            const uint32_t f = f0 + lane;
            if (f < m.F) {
                const LaneCtx c = lane_ctx(m, start, f);
                const double v = image_lane<MODE, AP, TAU>(m, sl, c, bk, nb, fw, 0);
                I[(size_t)px * m.F + f] = v;
                if (!isfinite(v)) atomicOr(status, ST_NONFINITE);
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------------
template <typename K>
static cudaError_t launch_warp_kernel(MgrModel* model, K kern, uint32_t cap, uint64_t items, size_t* smem_out,
                                      unsigned* grid_out) {
    const uint32_t Lpad = (model->dm.L + 1) & ~1u;
    int nw = 8;
    size_t smem = (size_t)Lpad * 8 + (size_t)nw * half_bytes_per_warp(cap);
    while (nw > 1 && smem > 200 * 1024) {
        nw /= 2;
        smem = (size_t)Lpad * 8 + (size_t)nw * half_bytes_per_warp(cap);
    }
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nw * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    uint64_t grid = (uint64_t)model->sm_count * per_sm;
    const uint64_t need = (items + nw - 1) / nw;
    if (grid > need) grid = need;
    *smem_out = smem;
    *grid_out = (unsigned)(grid ? grid : 1);
    return cudaSuccess;
}

template <int MODE, int AP, bool TAU>
static cudaError_t launch_image_t(MgrModel* model, uint32_t rr, double* I) {
    size_t smem;
    unsigned grid;
    auto kern = image_kernel<MODE, AP, TAU>;
    cudaError_t e = launch_warp_kernel(model, kern, model->half_cap, model->dm.P, &smem, &grid);
    if (e != cudaSuccess) return e;
    const int nw = (int)((smem - (size_t)((model->dm.L + 1) & ~1u) * 8) / half_bytes_per_warp(model->half_cap));
    count_launch();
    kern<<<grid, nw * 32, smem, model->stream>>>(model->dm, model->half_cap, rr, I, model->status);
    return cudaGetLastError();
}

template <int MODE, int AP, bool TAU>
static cudaError_t launch_image_new_t(MgrModel* model, const ImagePlane& ip, uint32_t cap, double* I) {
    size_t smem;
    unsigned grid;
    auto kern = image_new_kernel<MODE, AP, TAU>;
    cudaError_t e = launch_warp_kernel(model, kern, cap, (uint64_t)ip.nx * ip.ny, &smem, &grid);
    if (e != cudaSuccess) return e;
    const int nw = (int)((smem - (size_t)((model->dm.L + 1) & ~1u) * 8) / half_bytes_per_warp(cap));
    count_launch();
    kern<<<grid, nw * 32, smem, model->stream>>>(model->dm, ip, cap, I, model->status);
    return cudaGetLastError();
}

template <int MODE, bool TAU = false>
static cudaError_t dispatch_image(MgrModel* model, uint32_t rr, double* I) {
    if (model->dm.approx == APPROX_NONE) return launch_image_t<MODE, APPROX_NONE, TAU>(model, rr, I);
    return launch_image_t<MODE, APPROX_CLOSELINES, TAU>(model, rr, I);
}

template <int MODE, bool TAU = false>
static cudaError_t dispatch_image_new(MgrModel* model, const ImagePlane& ip, uint32_t cap, double* I) {
    if (model->dm.approx == APPROX_NONE) return launch_image_new_t<MODE, APPROX_NONE, TAU>(model, ip, cap, I);
    return launch_image_new_t<MODE, APPROX_CLOSELINES, TAU>(model, ip, cap, I);
}

// Image::set_coordinates_all_model_points, 3D (image.cpp:154-219).
int image_plane_setup(MgrModel* model, const char* who, const double* raydir, uint32_t nx, uint32_t ny,
                      ImagePlane& ip, std::vector<double>& hx, std::vector<double>& hy) {
    if (model->dm.approx == APPROX_ONELINE) {
        set_error(std::string(who) + ": One line approximation is not supported for imaging.");
        return MGR_ERR_UNSUPPORTED;
    }
    std::string err;
    const int rc = image_plane_compute(model->host_pos.data(), model->host_p2b.data(), model->dm.P, model->dm.B,
                                       raydir, nx, ny, ip, hx, hy, err, model->dm.sph != 0);
    if (rc != MGR_OK) set_error(std::string(who) + ": " + err);
    return rc;
}

cudaError_t image_plane_upload(MgrModel* model, ImagePlane& ip, const std::vector<double>& hx,
                               const std::vector<double>& hy, double* d_xy, uint32_t* d_max, uint32_t* cap) {
    const size_t npix = hx.size();
    cudaError_t e = cudaMemcpyAsync(d_xy, hx.data(), npix * 8, cudaMemcpyHostToDevice, model->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_xy + npix, hy.data(), npix * 8, cudaMemcpyHostToDevice, model->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_max, 0, sizeof(uint32_t), model->stream);
    ip.ImX = d_xy;
    ip.ImY = d_xy + npix;
    *cap = 0;
    if (e == cudaSuccess) {
        count_launch();
        const unsigned blocks = (unsigned)std::min<size_t>((npix * 32 + 255) / 256, (size_t)model->sm_count * 16);
        image_size_kernel<<<blocks ? blocks : 1, 256, 0, model->stream>>>(model->dm, ip, d_max, model->status);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(cap, d_max, sizeof(uint32_t), cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    if (*cap < 1) *cap = 1;
    return e;
}

static int image_old_impl(MgrModel* model, int precision, uint32_t ray_nr, double* I, double* ImX, double* ImY,
                          bool tau, const std::string& who) {
    if (!model || !I) {
        set_error(who + ": null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) {
        set_error(who + ": unknown precision mode");
        return MGR_ERR_ARGUMENT;
    }
    if (model->dm.approx == APPROX_ONELINE) {
        set_error(who + ": One line approximation is currently not supported for imaging.");
        return MGR_ERR_UNSUPPORTED;
    }
    const DevModel& dm = model->dm;
    if (ray_nr >= dm.nrays) {
        set_error(who + ": ray number out of range");
        return MGR_ERR_ARGUMENT;
    }
    const size_t PF = (size_t)dm.P * dm.F;
    double* dI = nullptr;
    cudaError_t e = cudaMalloc(&dI, PF * 8);
    if (e == cudaSuccess) {
        if (tau)
            e = (precision == MGR_PRECISION_SPLIT) ? dispatch_image<MODE_SPLIT, true>(model, ray_nr, dI)
                                                   : dispatch_image<MODE_FP64, true>(model, ray_nr, dI);
        else
            e = (precision == MGR_PRECISION_SPLIT) ? dispatch_image<MODE_SPLIT>(model, ray_nr, dI)
                                                   : dispatch_image<MODE_FP64>(model, ray_nr, dI);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(I, dI, PF * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    cudaFree(dI);
    if (e != cudaSuccess) return cuda_fail(e, who.c_str());
    if (ImX && ImY && model->dm.sph) {
        // Image::set_coordinates_all_model_points, 1D (image.cpp:160-171)
        for (uint32_t p = 0; p < dm.P; p++) {
            ImX[p] = model->host_pos[3 * (size_t)p];
            ImY[p] = 0.0;
        }
    } else if (ImX && ImY) {
        const double* d = model->host_raydir.data() + 3 * (size_t)ray_nr;
        double ix, iy, jx, jy, jz;
        bool tilted;
        plane_axes(d, ix, iy, jx, jy, jz, tilted);
        for (uint32_t p = 0; p < dm.P; p++) {
            const double* x = model->host_pos.data() + 3 * (size_t)p;
            if (tilted) {
                ImX[p] = ix * x[0] + iy * x[1];
                ImY[p] = jx * x[0] + jy * x[1] + jz * x[2];
            } else {
                ImX[p] = x[0];
                ImY[p] = x[1];
            }
        }
    }
    return mgr_sync(model);
}

static int image_new_impl(MgrModel* model, int precision, const double* raydir, uint32_t nx, uint32_t ny,
                          double* I, double* ImX, double* ImY, bool tau, const std::string& who) {
    if (!model || !I) {
        set_error(who + ": null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) {
        set_error(who + ": unknown precision mode");
        return MGR_ERR_ARGUMENT;
    }
    ImagePlane ip{};
    std::vector<double> hx, hy;
    int rc = image_plane_setup(model, who.c_str(), raydir, nx, ny, ip, hx, hy);
    if (rc != MGR_OK) return rc;
    const DevModel& dm = model->dm;
    const size_t npix = (size_t)nx * ny;
    double *dxy = nullptr, *dI = nullptr;
    uint32_t* dmax = nullptr;
    uint32_t cap = 0;
    cudaError_t e = cudaMalloc(&dxy, 2 * npix * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dI, npix * dm.F * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dmax, sizeof(uint32_t));
    if (e == cudaSuccess) e = image_plane_upload(model, ip, hx, hy, dxy, dmax, &cap);
    if (e == cudaSuccess) {
        if (tau)
            e = (precision == MGR_PRECISION_SPLIT) ? dispatch_image_new<MODE_SPLIT, true>(model, ip, cap, dI)
                                                   : dispatch_image_new<MODE_FP64, true>(model, ip, cap, dI);
        else
            e = (precision == MGR_PRECISION_SPLIT) ? dispatch_image_new<MODE_SPLIT>(model, ip, cap, dI)
                                                   : dispatch_image_new<MODE_FP64>(model, ip, cap, dI);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(I, dI, npix * dm.F * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    cudaFree(dxy);
    cudaFree(dI);
    cudaFree(dmax);
    if (e != cudaSuccess) return cuda_fail(e, who.c_str());
    if (ImX) std::copy(hx.begin(), hx.end(), ImX);
    if (ImY) std::copy(hy.begin(), hy.end(), ImY);
    return mgr_sync(model);
}

// ---------------------------------------------------------------------------------
// Model::compute_image_for_point (model.cpp:1039-1058 ->
// Solver::image_feautrier_order_2_for_point, solver.tpp:629-653): the old imager's ray
// through one point, every element's S, dtau and u.  A counting launch gives the ray's
// element count (traced steps plus interpolation points, both halves, the origin);
// the solve launch runs one warp per 32 frequencies, each retracing the ray.
// ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(32) image_point_count_kernel(DevModel m, uint32_t cap, uint32_t rr, uint32_t p,
                                                               int* out, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    HalfSmem bk, fw;
    carve_halves(smem, cap, bk, fw);
    const uint32_t ar = m.antipod[rr];
    int nb = 0, nf = 0;
    trace_pair<true, 1>(m, p, rr, ar, cap, bk, fw, lane, status, nb, nf);
    uint32_t n = 0;
    if (nb >= 0 && nf >= 0) {
        for (int s = lane; s < nb; s += 32) n += m.nint_all[bk.eid[s]];
        for (int s = lane; s < nf; s += 32) n += m.nint_all[fw.eid[s]];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) n += __shfl_xor_sync(FULL_MASK, n, off);
    if (lane == 0) {
        out[0] = (nb < 0 || nf < 0) ? -1 : (int)(n + 1);
        out[1] = nb;
        out[2] = nf;
    }
}

template <int MODE, int AP>
__global__ void __launch_bounds__(32) image_point_kernel(DevModel m, uint32_t cap, uint32_t rr, uint32_t p, RowOut ro,
                                                         int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    double* sl = reinterpret_cast<double*>(smem);
    const uint32_t Lpad = (m.L + 1) & ~1u;
    HalfSmem bk, fw;
    carve_halves(smem + (size_t)Lpad * 8, cap, bk, fw);
    for (uint32_t i = lane; i < m.L; i += 32) sl[i] = m.sorted_line[i];
    __syncwarp();
    const uint32_t ar = m.antipod[rr];
    const double shb = origin_shift(m, 1, p, rr);
    const double shf = origin_shift(m, 1, p, ar);
    bk.shift0 = shb;
    fw.shift0 = shf;
    set_dsh0(bk, shb);
    set_dsh0(fw, shf);
    bk.cshift = fw.cshift = shb;
    int nb = 0, nf = 0;
    trace_pair<true, 1>(m, p, rr, ar, cap, bk, fw, lane, status, nb, nf);
    if (nb < 0 || nf < 0) return;
    const uint32_t f = blockIdx.x * 32 + lane;
    if (f >= m.F) return;
    const LaneCtx c = lane_ctx(m, p, f);
    image_lane<MODE, AP, false, true>(m, sl, c, bk, nb, fw, nf, &ro);
    if (!isfinite(ro.u[f])) atomicOr(status, ST_NONFINITE);
}

template <int MODE>
static cudaError_t launch_image_point(MgrModel* model, uint32_t rr, uint32_t p, const RowOut& ro) {
    const uint32_t Lpad = (model->dm.L + 1) & ~1u;
    const size_t smem = (size_t)Lpad * 8 + half_bytes_per_warp(model->half_cap);
    auto kern = (model->dm.approx == APPROX_NONE) ? image_point_kernel<MODE, APPROX_NONE>
                                                  : image_point_kernel<MODE, APPROX_CLOSELINES>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    count_launch();
    kern<<<(model->dm.F + 31) / 32, 32, smem, model->stream>>>(model->dm, model->half_cap, rr, p, ro, model->status);
    return cudaGetLastError();
}

static int image_for_point_impl(MgrModel* model, int precision, uint32_t ray_nr, uint32_t p, uint32_t* n_tot,
                                double* S_ray, double* dtau_ray, double* u_ray, uint32_t capacity) {
    const char* who = "mgr_image_for_point";
    if (!model || !n_tot) {
        set_error(std::string(who) + ": null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) {
        set_error(std::string(who) + ": unknown precision mode");
        return MGR_ERR_ARGUMENT;
    }
    if (model->dm.approx == APPROX_ONELINE) {
        set_error(std::string(who) + ": One line approximation is currently not supported for imaging.");
        return MGR_ERR_UNSUPPORTED;
    }
    const DevModel& dm = model->dm;
    if (ray_nr >= dm.nrays || p >= dm.P) {
        set_error(std::string(who) + ": ray or point number out of range");
        return MGR_ERR_ARGUMENT;
    }
    int* d_cnt = nullptr;
    int cnt[3] = {0, 0, 0};
    cudaError_t e = cudaMalloc(&d_cnt, 3 * sizeof(int));
    if (e == cudaSuccess) {
        const size_t smem = half_bytes_per_warp(model->half_cap);
        e = cudaFuncSetAttribute(image_point_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) {
            count_launch();
            image_point_count_kernel<<<1, 32, smem, model->stream>>>(dm, model->half_cap, ray_nr, p, d_cnt,
                                                                     model->status);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(cnt, d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    cudaFree(d_cnt);
    if (e != cudaSuccess) return cuda_fail(e, who);
    if (cnt[0] < 0) return mgr_sync(model);  // the trace's status bits say why
    *n_tot = (uint32_t)cnt[0];
    if (!S_ray && !dtau_ray && !u_ray && capacity == 0) return MGR_OK;  // size query
    if (!S_ray || !dtau_ray || !u_ray) {
        set_error(std::string(who) + ": null output array");
        return MGR_ERR_ARGUMENT;
    }
    if (*n_tot > capacity) {
        set_error(std::string(who) + ": the ray has more elements than the output arrays' rows");
        return MGR_ERR_CAPACITY;
    }
    const size_t NF = (size_t)*n_tot * dm.F;
    std::memset(S_ray, 0, NF * 8);
    std::memset(dtau_ray, 0, NF * 8);
    std::memset(u_ray, 0, NF * 8);
    if (*n_tot <= 1) return MGR_OK;  // solver.tpp:646: nothing is solved on a one-element ray
    double* buf = nullptr;
    e = cudaMalloc(&buf, 4 * NF * 8);
    if (e == cudaSuccess) {
        const RowOut ro{buf, buf + NF, buf + 2 * NF, buf + 3 * NF, dm.F};
        e = (precision == MGR_PRECISION_SPLIT) ? launch_image_point<MODE_SPLIT>(model, ray_nr, p, ro)
                                               : launch_image_point<MODE_FP64>(model, ray_nr, p, ro);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(S_ray, buf, NF * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dtau_ray, buf + NF, NF * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(u_ray, buf + 2 * NF, NF * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(e, who);
    return mgr_sync(model);
}

// ---------------------------------------------------------------------------------
// Model::set_column (model.cpp:1143-1153 -> Solver::set_column / get_column,
// solver.tpp:2953-2991): column[r][o] = sum over the ray's steps of
// (density[crt] + density[nxt]) / 2 * dZ, from o along r to the boundary, for every ray
// pair rr < hnrays and its antipode.  Warp per (ray, point) walk with the solves'
// next-point argmin (shell steps in spherical symmetry); the sum in FP64 with the
// reference's roundings.
// ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) column_kernel(DevModel m, const double* __restrict__ density,
                                                     double* __restrict__ column, int* status) {
    const int nw = blockDim.x >> 5, lane = threadIdx.x & 31;
    const uint64_t items = (uint64_t)m.hnrays * 2 * m.P;
    for (uint64_t it = (uint64_t)blockIdx.x * nw + (threadIdx.x >> 5); it < items; it += (uint64_t)gridDim.x * nw) {
        const uint32_t o = (uint32_t)(it % m.P);
        const uint32_t side = (uint32_t)((it / m.P) & 1);
        const uint32_t rr = (uint32_t)(it / (2ull * m.P));
        const uint32_t r = side ? m.antipod[rr] : rr;
        const double* d = ray_dir(m, o, r);  // set_column<use_adaptive_directions>
        const double dx = d[0], dy = d[1], dz = d[2];
        const double4_32a po = m.pos[o];
        const double Rcos = dot3_rn(po.x, po.y, po.z, dx, dy, dz);
        const double Rsin2 = dsub_rn(sqnorm_rn(po), dmul_rn(Rcos, Rcos));
        double Z = 0.0, col = 0.0;
        uint32_t crt = o;
        int steps = 0;
        while (true) {
            uint32_t nxt, eid;
            double dZl;
            bool ok;
            if (m.sph) {
                ok = next_point_sph(m, Rcos, Rsin2, crt, Z, nxt, dZl);
            } else {
                double bestZ;
                ok = warp_next_point(m, po, dx, dy, dz, crt, Z, lane, nxt, bestZ, eid);
                dZl = dsub_rn(bestZ, Z);
            }
            if (!ok) {
                if (steps > 0 && lane == 0) atomicOr(status, ST_TRACE);
                break;
            }
            Z = dadd_rn(Z, dZl);
            col = dadd_rn(col, dmul_rn(dmul_rn(0.5, dadd_rn(density[crt], density[nxt])), dZl));
            steps++;
            if (m.p2b[nxt] != m.P) break;
            crt = nxt;
        }
        if (lane == 0) column[(size_t)r * m.P + o] = col;
    }
}

static int set_column_impl(MgrModel* model, const double* density, double* column) {
    const char* who = "mgr_set_column";
    if (!model || !density || !column) {
        set_error(std::string(who) + ": null argument");
        return MGR_ERR_ARGUMENT;
    }
    const DevModel& dm = model->dm;
    const size_t RP = (size_t)dm.nrays * dm.P;
    double* buf = nullptr;
    cudaError_t e = cudaMalloc(&buf, (RP + dm.P) * 8);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf + RP, density, (size_t)dm.P * 8, cudaMemcpyHostToDevice, model->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(buf, 0, RP * 8, model->stream);
    if (e == cudaSuccess) {
        const uint64_t warps = (uint64_t)dm.hnrays * 2 * dm.P;
        const unsigned blocks = (unsigned)std::min<uint64_t>((warps + 7) / 8, (uint64_t)model->sm_count * 8);
        count_launch();
        column_kernel<<<blocks ? blocks : 1, 256, 0, model->stream>>>(dm, buf + RP, buf, model->status);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(column, buf, RP * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(e, who);
    return mgr_sync(model);
}

}  // namespace mgr

using namespace mgr;

extern "C" {

int mgr_image(MgrModel* model, int precision, uint32_t ray_nr, double* I, double* ImX, double* ImY) {
    MGR_MODEL_DEVICE(model);
    return image_old_impl(model, precision, ray_nr, I, ImX, ImY, false, "mgr_image");
}

int mgr_image_new(MgrModel* model, int precision, const double* raydir, uint32_t nx, uint32_t ny, double* I,
                  double* ImX, double* ImY) {
    MGR_MODEL_DEVICE(model);
    return image_new_impl(model, precision, raydir, nx, ny, I, ImX, ImY, false, "mgr_image_new");
}

int mgr_image_optical_depth(MgrModel* model, int precision, uint32_t ray_nr, double* I, double* ImX, double* ImY) {
    MGR_MODEL_DEVICE(model);
    return image_old_impl(model, precision, ray_nr, I, ImX, ImY, true, "mgr_image_optical_depth");
}

int mgr_image_optical_depth_new(MgrModel* model, int precision, const double* raydir, uint32_t nx, uint32_t ny,
                                double* I, double* ImX, double* ImY) {
    MGR_MODEL_DEVICE(model);
    return image_new_impl(model, precision, raydir, nx, ny, I, ImX, ImY, true, "mgr_image_optical_depth_new");
}

int mgr_image_for_point(MgrModel* model, int precision, uint32_t ray_nr, uint32_t p, uint32_t* n_tot, double* S_ray,
                        double* dtau_ray, double* u_ray, uint32_t capacity) {
    MGR_MODEL_DEVICE(model);
    return image_for_point_impl(model, precision, ray_nr, p, n_tot, S_ray, dtau_ray, u_ray, capacity);
}

int mgr_set_column(MgrModel* model, const double* density, double* column) {
    MGR_MODEL_DEVICE(model);
    return set_column_impl(model, density, column);
}



}  // extern "C"
