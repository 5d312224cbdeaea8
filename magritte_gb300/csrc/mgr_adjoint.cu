// Differentiable new imager on the GPU: the smooth FP64 image (forward) and its
// adjoint (backward) for Model::compute_image_new (model.cpp:977-1013 ->
// Solver::image_feautrier_order_2_new_imager, solver.tpp:576-627), plus the
// device-pointer updates of the model's velocities and line data that an autograd
// wrapper needs between calls.
//
// Both kernels run one warp per pixel with lanes over frequencies, like the imager:
// the warp traces the pixel ray into shared memory, then every lane runs
// image_lane_s (forward) or image_lane_adj (backward).  The backward keeps, per
// lane, the elimination state of each pair in a scratch array of the warp's slot
// (recomputed from the inputs, not saved by the forward), and adds its derivatives
// into the per-point gradient arrays with one atomic per warp and entry.
#include <algorithm>
#include <cstring>
#include <vector>

#include "mgr_adjoint.cuh"
#include "mgr_image.cuh"

namespace mgr {

// Elements (pairs + 1) of the longest pixel ray: trace, then the interpolation
// points of every step (nint_all), as image_lane_s walks them.
__global__ void adj_size_kernel(DevModel m, ImagePlane ip, uint32_t cap, uint32_t* d_max_pairs, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nw = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    HalfSmem bk, fw;
    carve_halves(smem + (size_t)w * half_bytes_per_warp(cap), cap, bk, fw);
    const uint32_t npix = ip.nx * ip.ny;
    for (uint32_t px = blockIdx.x * nw + w; px < npix; px += gridDim.x * nw) {
        double org[3];
        pixel_origin(ip, ip.ImX[px], ip.ImY[px], org);
        double Z;
        const uint32_t start = pixel_start(m, org, ip, lane, Z);
        const int nb = trace_image<true>(m, org, ip, start, Z, cap, bk, lane, status);
        if (nb <= 0) continue;
        uint32_t n = 0;
        for (int s = lane; s < nb; s += 32) n += m.nint_all[bk.eid[s]];
        for (int off = 16; off > 0; off >>= 1) n += __shfl_xor_sync(FULL_MASK, n, off);
        if (lane == 0) atomicMax(d_max_pairs, n);
        __syncwarp();
    }
}

template <int AP>
__global__ void __launch_bounds__(256) image_s_kernel(DevModel m, ImagePlane ip, uint32_t cap,
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
        const double4_32a vs = m.vel[start];
        const double sh0 = dadd_rn(1.0, dot3_rn(vs.x, vs.y, vs.z, ip.d[0], ip.d[1], ip.d[2]));
        bk.shift0 = fw.shift0 = bk.cshift = fw.cshift = sh0;
        const int nb = trace_image<true>(m, org, ip, start, Z, cap, bk, lane, status);
        if (nb < 0) continue;
        for (uint32_t f = lane; f < m.F; f += 32) {
            uint32_t np;
            const double v = image_lane_s<AP>(m, sl, start, m.nu[(size_t)start * m.F + f], bk, nb, nullptr, &np);
            I[(size_t)px * m.F + f] = v;
            if (!isfinite(v)) atomicOr(status, ST_NONFINITE);
        }
        __syncwarp();
    }
}

template <int AP>
__global__ void __launch_bounds__(256) image_adj_kernel(DevModel m, ImagePlane ip, uint32_t cap,
                                                        const double* __restrict__ gI, AdjGrads g,
                                                        double* __restrict__ scratch, uint32_t scratch_pairs,
                                                        int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nw = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* sl = reinterpret_cast<double*>(smem);
    const uint32_t Lpad = (m.L + 1) & ~1u;
    HalfSmem bk, fw;
    carve_halves(smem + (size_t)Lpad * 8 + (size_t)w * half_bytes_per_warp(cap), cap, bk, fw);
    for (uint32_t i = threadIdx.x; i < m.L; i += blockDim.x) sl[i] = m.sorted_line[i];
    __syncthreads();
    const size_t slot = (size_t)blockIdx.x * nw + w;
    LaneScratch scr{scratch + slot * (size_t)scratch_pairs * 3 * 32 + lane, 32, scratch_pairs};
    const AdjAcc acc{g, m.L};
    const uint32_t npix = ip.nx * ip.ny;
    for (uint32_t px = blockIdx.x * nw + w; px < npix; px += gridDim.x * nw) {
        double org[3];
        pixel_origin(ip, ip.ImX[px], ip.ImY[px], org);
        double Z;
        const uint32_t start = pixel_start(m, org, ip, lane, Z);
        const double4_32a vs = m.vel[start];
        const double sh0 = dadd_rn(1.0, dot3_rn(vs.x, vs.y, vs.z, ip.d[0], ip.d[1], ip.d[2]));
        bk.shift0 = fw.shift0 = bk.cshift = fw.cshift = sh0;
        const int nb = trace_image<true>(m, org, ip, start, Z, cap, bk, lane, status);
        if (nb < 0) continue;
        // every lane runs each chunk (the warp sums its derivatives); lanes beyond the
        // frequencies carry gI = 0
        for (uint32_t f0 = 0; f0 < m.F; f0 += 32) {
            const uint32_t f = f0 + lane;
            const uint32_t fc = f < m.F ? f : m.F - 1;
            const double g = f < m.F ? gI[(size_t)px * m.F + f] : 0.0;
            if (!image_lane_adj<AP>(m, sl, start, m.nu[(size_t)start * m.F + fc], bk, nb, g, scr, acc)) {
                if (lane == 0) atomicOr(status, ST_CAPACITY);
            }
        }
        __syncwarp();
    }
}

__global__ void pack_velocity_kernel(const double* __restrict__ v, double4_32a* __restrict__ out, uint32_t P) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x)
        out[p] = make_double4_32a(v[3 * (size_t)p], v[3 * (size_t)p + 1], v[3 * (size_t)p + 2], 0.0);
}

// Largest value of a non-negative array (bit pattern order of non-negative doubles).
__global__ void max_nonneg_kernel(const double* __restrict__ a, size_t n, unsigned long long* out) {
    unsigned long long mx = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double x = a[i];
        if (x > 0.0 && isfinite(x)) mx = max(mx, (unsigned long long)__double_as_longlong(x));
    }
    for (int off = 16; off > 0; off >>= 1) mx = max(mx, __shfl_xor_sync(FULL_MASK, mx, off));
    if ((threadIdx.x & 31) == 0) atomicMax(out, mx);
}

// Shared-memory launch shape of the pixel kernels (as the imager's).
template <typename K>
static cudaError_t pixel_launch_shape(MgrModel* model, K kern, uint32_t cap, uint64_t items, int* nw_out,
                                      size_t* smem_out, unsigned* grid_out) {
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
    if (grid < 1) grid = 1;
    *nw_out = nw;
    *smem_out = smem;
    *grid_out = (unsigned)grid;
    return cudaSuccess;
}

// Image-plane set-up shared by the forward and the backward: plane, pixel
// coordinates on the device (d_xy, caller frees) and the trace capacity.
static int adj_plane(MgrModel* model, const char* who, const double* raydir, uint32_t nx, uint32_t ny,
                     ImagePlane& ip, double** d_xy, uint32_t* cap, std::vector<double>* hx_out,
                     std::vector<double>* hy_out) {
    if (model->dm.approx == APPROX_ONELINE) {
        set_error(std::string(who) + ": One line approximation is not supported for imaging.");
        return MGR_ERR_UNSUPPORTED;
    }
    if (model->dm.sph) {
        set_error(std::string(who) + ": the differentiable imager does not support spherically symmetric models.");
        return MGR_ERR_UNSUPPORTED;
    }
    std::vector<double> hx, hy;
    int rc = image_plane_setup(model, who, raydir, nx, ny, ip, hx, hy);
    if (rc != MGR_OK) return rc;
    uint32_t* dmax = nullptr;
    cudaError_t e = cudaMalloc(d_xy, 2 * hx.size() * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dmax, sizeof(uint32_t));
    if (e == cudaSuccess) e = image_plane_upload(model, ip, hx, hy, *d_xy, dmax, cap);
    cudaFree(dmax);
    if (e != cudaSuccess) {
        cudaFree(*d_xy);
        *d_xy = nullptr;
        return cuda_fail(e, who);
    }
    if (hx_out) *hx_out = std::move(hx);
    if (hy_out) *hy_out = std::move(hy);
    return MGR_OK;
}

static int finish(MgrModel* model, cudaError_t e, const char* who) {
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    if (e != cudaSuccess) return cuda_fail(e, who);
    int st = 0;
    e = cudaMemcpy(&st, model->status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemset(model->status, 0, sizeof(int));
    if (e != cudaSuccess) return cuda_fail(e, who);
    return decode_status(st);
}

}  // namespace mgr

using namespace mgr;

extern "C" {

int mgr_model_set_velocity_device(MgrModel* model, const double* velocity_dev) {
    MGR_MODEL_DEVICE(model);
    if (!model || !velocity_dev) {
        set_error("mgr_model_set_velocity_device: null argument");
        return MGR_ERR_ARGUMENT;
    }
    count_launch();
    const uint32_t P = model->dm.P;
    pack_velocity_kernel<<<(P + 255) / 256 < 2432 ? (P + 255) / 256 : 2432, 256, 0, model->stream>>>(
        velocity_dev, const_cast<double4_32a*>(model->dm.vel), P);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "velocity update");
    model->inputs_replaced = true;
    return MGR_OK;
}

int mgr_model_set_line_data_device(MgrModel* model, const double* emissivity_dev, const double* opacity_dev,
                                   const double* inverse_width_dev) {
    MGR_MODEL_DEVICE(model);
    if (!model) {
        set_error("mgr_model_set_line_data_device: null model");
        return MGR_ERR_ARGUMENT;
    }
    const size_t n = (size_t)model->dm.P * model->dm.L;
    cudaError_t e = cudaSuccess;
    if (emissivity_dev)
        e = cudaMemcpyAsync(model->em, emissivity_dev, n * 8, cudaMemcpyDeviceToDevice, model->stream);
    if (e == cudaSuccess && opacity_dev)
        e = cudaMemcpyAsync(model->op, opacity_dev, n * 8, cudaMemcpyDeviceToDevice, model->stream);
    if (e == cudaSuccess && inverse_width_dev)
        e = cudaMemcpyAsync(model->iw, inverse_width_dev, n * 8, cudaMemcpyDeviceToDevice, model->stream);
    unsigned long long* dmx = nullptr;
    unsigned long long hmx[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMalloc(&dmx, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemsetAsync(dmx, 0, 2 * sizeof(unsigned long long), model->stream);
    if (e == cudaSuccess) {
        const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 2432);
        count_launch();
        max_nonneg_kernel<<<blocks ? blocks : 1, 256, 0, model->stream>>>(model->em, n, dmx);
        count_launch();
        max_nonneg_kernel<<<blocks ? blocks : 1, 256, 0, model->stream>>>(model->op, n, dmx + 1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hmx, dmx, sizeof(hmx), cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    cudaFree(dmx);
    if (e != cudaSuccess) return cuda_fail(e, "line data update");
    double mx[2];
    for (int k = 0; k < 2; k++) {
        long long b = (long long)hmx[k];
        std::memcpy(&mx[k], &b, 8);
    }
    set_line_scales(model, pow2_scale_of(mx[0]), pow2_scale_of(mx[1]));
    e = launch_line_tables(model);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "line data update");
    return MGR_OK;
}

int mgr_image_new_smooth_device(MgrModel* model, const double* raydir, uint32_t nx, uint32_t ny, double* I_dev,
                                double* ImX, double* ImY) {
    MGR_MODEL_DEVICE(model);
    if (!model || !I_dev) {
        set_error("mgr_image_new_smooth_device: null argument");
        return MGR_ERR_ARGUMENT;
    }
    ImagePlane ip{};
    double* dxy = nullptr;
    uint32_t cap = 0;
    std::vector<double> hx, hy;
    int rc = adj_plane(model, "mgr_image_new_smooth_device", raydir, nx, ny, ip, &dxy, &cap, &hx, &hy);
    if (rc != MGR_OK) return rc;
    const uint64_t npix = (uint64_t)nx * ny;
    int nw;
    size_t smem;
    unsigned grid;
    cudaError_t e;
    if (model->dm.approx == APPROX_CLOSELINES) {
        e = pixel_launch_shape(model, image_s_kernel<APPROX_CLOSELINES>, cap, npix, &nw, &smem, &grid);
        if (e == cudaSuccess) {
            count_launch();
            image_s_kernel<APPROX_CLOSELINES><<<grid, nw * 32, smem, model->stream>>>(model->dm, ip, cap, I_dev,
                                                                                     model->status);
            e = cudaGetLastError();
        }
    } else {
        e = pixel_launch_shape(model, image_s_kernel<APPROX_NONE>, cap, npix, &nw, &smem, &grid);
        if (e == cudaSuccess) {
            count_launch();
            image_s_kernel<APPROX_NONE><<<grid, nw * 32, smem, model->stream>>>(model->dm, ip, cap, I_dev,
                                                                               model->status);
            e = cudaGetLastError();
        }
    }
    rc = finish(model, e, "mgr_image_new_smooth_device");
    cudaFree(dxy);
    if (rc == MGR_OK) {
        if (ImX) std::copy(hx.begin(), hx.end(), ImX);
        if (ImY) std::copy(hy.begin(), hy.end(), ImY);
    }
    return rc;
}

int mgr_image_new_adjoint_device(MgrModel* model, const double* raydir, uint32_t nx, uint32_t ny,
                                 const double* gI_dev, double* g_em_dev, double* g_op_dev, double* g_iw_dev,
                                 double* g_Sp_dev, double* g_vel_dev) {
    MGR_MODEL_DEVICE(model);
    if (!model || !gI_dev || !g_em_dev || !g_op_dev || !g_iw_dev || !g_Sp_dev || !g_vel_dev) {
        set_error("mgr_image_new_adjoint_device: null argument");
        return MGR_ERR_ARGUMENT;
    }
    ImagePlane ip{};
    double* dxy = nullptr;
    uint32_t cap = 0;
    int rc = adj_plane(model, "mgr_image_new_adjoint_device", raydir, nx, ny, ip, &dxy, &cap, nullptr, nullptr);
    if (rc != MGR_OK) return rc;
    const uint64_t npix = (uint64_t)nx * ny;
    // longest ray in pairs (elements including interpolation points)
    uint32_t* dmax = nullptr;
    uint32_t pairs = 0;
    cudaError_t e = cudaMalloc(&dmax, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(dmax, 0, sizeof(uint32_t), model->stream);
    int nw;
    size_t smem;
    unsigned grid;
    if (e == cudaSuccess) e = pixel_launch_shape(model, adj_size_kernel, cap, npix, &nw, &smem, &grid);
    if (e == cudaSuccess) {
        // adj_size_kernel carries no line table: its buffer is the trace halves only
        smem = (size_t)nw * half_bytes_per_warp(cap);
        count_launch();
        adj_size_kernel<<<grid, nw * 32, smem, model->stream>>>(model->dm, ip, cap, dmax, model->status);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&pairs, dmax, sizeof(uint32_t), cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    cudaFree(dmax);
    if (pairs < 1) pairs = 1;
    AdjGrads g{g_em_dev, g_op_dev, g_iw_dev, g_Sp_dev, g_vel_dev, {ip.d[0], ip.d[1], ip.d[2]}};
    auto run = [&](auto kern) -> cudaError_t {
        cudaError_t r = pixel_launch_shape(model, kern, cap, npix, &nw, &smem, &grid);
        if (r != cudaSuccess) return r;
        const size_t need = (size_t)grid * nw * pairs * 3 * 32 * sizeof(double);
        if (model->adj_scratch_bytes < need) {  // grown on demand, kept for the next call
            cudaFree(model->adj_scratch);
            model->adj_scratch = nullptr;
            model->adj_scratch_bytes = 0;
            r = cudaMalloc(&model->adj_scratch, need);
            if (r != cudaSuccess) return r;
            model->adj_scratch_bytes = need;
        }
        count_launch();
        kern<<<grid, nw * 32, smem, model->stream>>>(model->dm, ip, cap, gI_dev, g, model->adj_scratch, pairs,
                                                     model->status);
        return cudaGetLastError();
    };
    if (e == cudaSuccess)
        e = (model->dm.approx == APPROX_CLOSELINES) ? run(image_adj_kernel<APPROX_CLOSELINES>)
                                                     : run(image_adj_kernel<APPROX_NONE>);
    rc = finish(model, e, "mgr_image_new_adjoint_device");
    cudaFree(dxy);
    return rc;
}

}  // extern "C"
