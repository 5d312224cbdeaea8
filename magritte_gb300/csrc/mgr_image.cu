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
#include <vector>

#include "mgr_internal.h"
#include "mgr_solve.cuh"

namespace mgr {

// ---------------------------------------------------------------------------------
// Old imager: warp per model point o, ray rr / antipode, rest-frame shifts.
// ---------------------------------------------------------------------------------
template <int MODE, int AP>
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
    const double* d = m.raydir + 3 * rr;
    for (uint32_t o = blockIdx.x * nw + w; o < m.P; o += gridDim.x * nw) {
        // Geometry::get_shift<Rest, false>(o, r, o, 0): the origin's shift along each
        // half's own ray (the antipode's is reversed), the element's that of rr
        const double shb = shift_rest(m, rr, o, d);
        const double shf = shift_rest(m, ar, o, m.raydir + 3 * ar);
        bk.shift0 = shb;
        fw.shift0 = shf;
        bk.dsh0 = (float)dsub_rn(shb, 1.0);
        fw.dsh0 = (float)dsub_rn(shf, 1.0);
        bk.cshift = fw.cshift = shb;
        const int nb = trace_half<true, 1>(m, o, rr, cap, bk, lane, status);
        const int nf = trace_half<true, 1>(m, o, ar, cap, fw, lane, status);
        if (nb < 0 || nf < 0) continue;
        for (uint32_t f0 = 0; f0 < m.F; f0 += 32) {
            const uint32_t f = f0 + lane;
            if (f < m.F) {
                LaneCtx c;
                c.o = o;
                c.f = f;
                c.l0 = m.corr_line[f];
                c.freq = m.nu[(size_t)o * m.F + f];
                c.fq = (float)c.freq;
                c.a0 = (float)(c.freq - m.line[c.l0]);
                const double v = image_lane<MODE, AP>(m, sl, c, bk, nb, fw, nf);
                I[(size_t)o * m.F + f] = v;
                if (!isfinite(v)) atomicOr(status, ST_NONFINITE);
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------
// New imager
// ---------------------------------------------------------------------------------
struct ImagePlane {
    double ix, iy, jx, jy, jz;  // image axes (image.cpp:169-180)
    bool tilted;                // denominator >= 1e-9
    double scp[3];              // surface_center_point
    double d[3];                // normalised ray direction
    double center[3];           // Points::center (points.cpp:30-42)
    uint32_t start;             // get_closest_bdy_point_in_custom_raydir
    uint32_t nx, ny;
    const double* ImX;          // [nx*ny] device
    const double* ImY;
};

__device__ __forceinline__ void pixel_origin(const ImagePlane& ip, double x, double y, double* o) {
    // Image::surface_coords_to_3D_coordinates (image.cpp:370-398)
    // (uncontracted, as the reference evaluates it)
    if (ip.tilted) {
        o[0] = dadd_rn(dadd_rn(dmul_rn(x, ip.ix), dmul_rn(y, ip.jx)), ip.scp[0]);
        o[1] = dadd_rn(dadd_rn(dmul_rn(x, ip.iy), dmul_rn(y, ip.jy)), ip.scp[1]);
        o[2] = dadd_rn(dmul_rn(y, ip.jz), ip.scp[2]);
    } else {
        o[0] = dadd_rn(x, ip.scp[0]);
        o[1] = dadd_rn(y, ip.scp[1]);
        o[2] = dadd_rn(0.0, ip.scp[2]);
    }
}

// Warp argmin of the squared distance from the ray over the boundary neighbours of crt
// (Geometry::get_boundary_point_closer_to_custom_ray, geometry.tpp:310-341): strict <,
// starting from crt's own distance; ties keep the lowest neighbour order.
__device__ uint32_t bdy_point_closer(const DevModel& m, const double* org, const ImagePlane& ip, uint32_t crt,
                                     int lane) {
    const double4_32a pc = m.pos[crt];
    const double Rx = dsub_rn(pc.x, org[0]), Ry = dsub_rn(pc.y, org[1]), Rz = dsub_rn(pc.z, org[2]);
    const double Zc = dot3_rn(Rx, Ry, Rz, ip.d[0], ip.d[1], ip.d[2]);
    const unsigned long long k0 = dkey(dsub_rn(dot3_rn(Rx, Ry, Rz, Rx, Ry, Rz), dmul_rn(Zc, Zc)));
    unsigned long long best = k0;
    uint32_t besti = 0xffffffffu;
    const uint32_t nnb = m.n_nb[crt], cum = m.cum_nb[crt];
    for (uint32_t i = lane; i < nnb; i += 32) {
        const double4_32a e = m.edge[cum + i];
        const uint32_t n = (uint32_t)__double_as_longlong(e.w);
        if (m.p2b[n] == m.P) continue;  // boundary points only
        const double Nx = dsub_rn(e.x, org[0]), Ny = dsub_rn(e.y, org[1]), Nz = dsub_rn(e.z, org[2]);
        const double Zn = dot3_rn(Nx, Ny, Nz, ip.d[0], ip.d[1], ip.d[2]);
        const unsigned long long k = dkey(dsub_rn(dot3_rn(Nx, Ny, Nz, Nx, Ny, Nz), dmul_rn(Zn, Zn)));
        if (k < best) {
            best = k;
            besti = i;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long ob = __shfl_xor_sync(FULL_MASK, best, off);
        const uint32_t oi = __shfl_xor_sync(FULL_MASK, besti, off);
        if (ob < best || (ob == best && oi < besti)) {
            best = ob;
            besti = oi;
        }
    }
    if (besti == 0xffffffffu) return crt;
    return (uint32_t)__double_as_longlong(m.edge[cum + besti].w);
}

// Solver::trace_ray_imaging (solver.tpp:841-897), increment -1: walks from the start
// boundary point through the model until it leaves on the far side; rest-frame
// shifts 1 + v . d of a motionless observer.  Returns the steps stored, 0 if the ray
// met no interior point (the reference then keeps only the start point), -1 on
// capacity overflow.
template <bool STORE>
__device__ int trace_image(const DevModel& m, const double* org, const ImagePlane& ip, uint32_t start, double Z,
                           uint32_t cap, HalfSmem h, int lane, int* status) {
    const double dx = ip.d[0], dy = ip.d[1], dz = ip.d[2];
    uint32_t crt = start;
    int count = 0;
    bool accessed = false;
    while (true) {
        const uint32_t nnb = m.n_nb[crt];
        const uint32_t cum = m.cum_nb[crt];
        const unsigned long long zkey = dkey(Z);
        unsigned long long best = ~0ull;
        uint32_t besti = 0xffffffffu;
        double bestZ = 0.0;
        for (uint32_t i = lane; i < nnb; i += 32) {
            const double4_32a e = m.edge[cum + i];
            const double Rx = dsub_rn(e.x, org[0]);
            const double Ry = dsub_rn(e.y, org[1]);
            const double Rz = dsub_rn(e.z, org[2]);
            const double Zn = dot3_rn(Rx, Ry, Rz, dx, dy, dz);
            if (dkey(Zn) > zkey) {
                const unsigned long long k = dkey(dsub_rn(dot3_rn(Rx, Ry, Rz, Rx, Ry, Rz), dmul_rn(Zn, Zn)));
                if (k < best) {
                    best = k;
                    besti = i;
                    bestZ = Zn;
                }
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const unsigned long long ob = __shfl_xor_sync(FULL_MASK, best, off);
            const uint32_t oi = __shfl_xor_sync(FULL_MASK, besti, off);
            const double oz = __shfl_xor_sync(FULL_MASK, bestZ, off);
            if (ob < best || (ob == best && oi < besti)) {
                best = ob;
                besti = oi;
                bestZ = oz;
            }
        }
        if (besti == 0xffffffffu) break;  // no next point: the walk ends here
        if (STORE && (uint32_t)count >= cap) {
            if (lane == 0) atomicOr(status, ST_CAPACITY);
            count = -1;
            break;
        }
        const uint32_t nxt = (uint32_t)__double_as_longlong(m.edge[cum + besti].w);
        const double dZl = dsub_rn(bestZ, Z);
        Z = dadd_rn(Z, dZl);
        if (STORE && lane == 0) {
            h.ids[count] = nxt;
            h.eid[count] = cum + besti;
            h.dZ[count] = dZl;
        }
        count++;
        const bool interior = m.p2b[nxt] == m.P;
        if (!interior) {
            const double4_32a pn = m.pos[nxt];
            const double side = dot3_rn(dsub_rn(pn.x, ip.center[0]), dsub_rn(pn.y, ip.center[1]),
                                        dsub_rn(pn.z, ip.center[2]), dx, dy, dz);
            if (!(side < 0.0)) break;  // a boundary point on the far side ends the ray
        } else {
            accessed = true;
        }
        crt = nxt;
    }
    __syncwarp();
    if (count > 0 && !accessed) count = 0;
    if (STORE && count > 0) {
        for (int s = lane; s < count; s += 32) {
            const double4_32a v = m.vel[h.ids[s]];
            const double sh = dadd_rn(1.0, dot3_rn(v.x, v.y, v.z, dx, dy, dz));
            h.shift[s] = sh;
            h.dsh[s] = (float)dsub_rn(sh, 1.0);
            h.dzs[s] = (float)h.dZ[s] * m.dz_scale;
        }
        __syncwarp();
    }
    return count;
}

// trace_ray_imaging_get_start (solver.tpp:808-830): the boundary point closest to the
// pixel's ray, found by a greedy walk over boundary neighbours.
__device__ uint32_t pixel_start(const DevModel& m, const double* org, const ImagePlane& ip, int lane, double& Z) {
    uint32_t p = ip.start;
    for (uint32_t it = 0; it < m.P; it++) {  // a walk visits each point at most once
        const uint32_t q = bdy_point_closer(m, org, ip, p, lane);
        if (q == p) break;
        p = q;
    }
    const double4_32a ps = m.pos[p];
    Z = dot3_rn(dsub_rn(ps.x, org[0]), dsub_rn(ps.y, org[1]), dsub_rn(ps.z, org[2]), ip.d[0], ip.d[1], ip.d[2]);
    return p;
}

__global__ void image_size_kernel(DevModel m, ImagePlane ip, uint32_t* d_max, int* status) {
    const int lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwt = (gridDim.x * blockDim.x) >> 5;
    HalfSmem h{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    for (uint32_t px = gw; px < ip.nx * ip.ny; px += nwt) {
        double org[3];
        pixel_origin(ip, ip.ImX[px], ip.ImY[px], org);
        double Z;
        const uint32_t start = pixel_start(m, org, ip, lane, Z);
        const int n = trace_image<false>(m, org, ip, start, Z, 0xffffffffu, h, lane, status);
        if (lane == 0 && n > 0) atomicMax(d_max, (uint32_t)n);
    }
}

template <int MODE, int AP>
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
        const double4_32a vs = m.vel[start];
        const double sh0 = dadd_rn(1.0, dot3_rn(vs.x, vs.y, vs.z, ip.d[0], ip.d[1], ip.d[2]));
        bk.shift0 = fw.shift0 = bk.cshift = fw.cshift = sh0;
        bk.dsh0 = fw.dsh0 = (float)dsub_rn(sh0, 1.0);
        const int nb = trace_image<true>(m, org, ip, start, Z, cap, bk, lane, status);
        if (nb < 0) continue;
        for (uint32_t f0 = 0; f0 < m.F; f0 += 32) {
            const uint32_t f = f0 + lane;
            if (f < m.F) {
                LaneCtx c;
                c.o = start;
                c.f = f;
                c.l0 = m.corr_line[f];
                c.freq = m.nu[(size_t)start * m.F + f];
                c.fq = (float)c.freq;
                c.a0 = (float)(c.freq - m.line[c.l0]);
                const double v = image_lane<MODE, AP>(m, sl, c, bk, nb, fw, 0);
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

template <int MODE, int AP>
static cudaError_t launch_image_t(MgrModel* model, uint32_t rr, double* I) {
    size_t smem;
    unsigned grid;
    auto kern = image_kernel<MODE, AP>;
    cudaError_t e = launch_warp_kernel(model, kern, model->half_cap, model->dm.P, &smem, &grid);
    if (e != cudaSuccess) return e;
    const int nw = (int)((smem - (size_t)((model->dm.L + 1) & ~1u) * 8) / half_bytes_per_warp(model->half_cap));
    count_launch();
    kern<<<grid, nw * 32, smem, model->stream>>>(model->dm, model->half_cap, rr, I, model->status);
    return cudaGetLastError();
}

template <int MODE, int AP>
static cudaError_t launch_image_new_t(MgrModel* model, const ImagePlane& ip, uint32_t cap, double* I) {
    size_t smem;
    unsigned grid;
    auto kern = image_new_kernel<MODE, AP>;
    cudaError_t e = launch_warp_kernel(model, kern, cap, (uint64_t)ip.nx * ip.ny, &smem, &grid);
    if (e != cudaSuccess) return e;
    const int nw = (int)((smem - (size_t)((model->dm.L + 1) & ~1u) * 8) / half_bytes_per_warp(cap));
    count_launch();
    kern<<<grid, nw * 32, smem, model->stream>>>(model->dm, ip, cap, I, model->status);
    return cudaGetLastError();
}

template <int MODE>
static cudaError_t dispatch_image(MgrModel* model, uint32_t rr, double* I) {
    if (model->dm.approx == APPROX_NONE) return launch_image_t<MODE, APPROX_NONE>(model, rr, I);
    return launch_image_t<MODE, APPROX_CLOSELINES>(model, rr, I);
}

template <int MODE>
static cudaError_t dispatch_image_new(MgrModel* model, const ImagePlane& ip, uint32_t cap, double* I) {
    if (model->dm.approx == APPROX_NONE) return launch_image_new_t<MODE, APPROX_NONE>(model, ip, cap, I);
    return launch_image_new_t<MODE, APPROX_CLOSELINES>(model, ip, cap, I);
}

// Image::set_coordinates_all_model_points, 3D (image.cpp:154-219).
static void plane_axes(const double* d, double& ix, double& iy, double& jx, double& jy, double& jz, bool& tilted) {
    const double rx = d[0], ry = d[1], rz = d[2];
    const double denominator = std::sqrt(rx * rx + ry * ry);
    const double inverse_denominator = 1.0 / denominator;
    ix = ry * inverse_denominator;
    iy = -rx * inverse_denominator;
    jx = rx * rz * inverse_denominator;
    jy = ry * rz * inverse_denominator;
    jz = -denominator;
    tilted = denominator >= 1.0e-9;
}

}  // namespace mgr

using namespace mgr;

extern "C" {

int mgr_image(MgrModel* model, int precision, uint32_t ray_nr, double* I, double* ImX, double* ImY) {
    if (!model || !I) {
        set_error("mgr_image: null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) {
        set_error("mgr_image: unknown precision mode");
        return MGR_ERR_ARGUMENT;
    }
    if (model->dm.approx == APPROX_ONELINE) {
        set_error("mgr_image: One line approximation is currently not supported for imaging.");
        return MGR_ERR_UNSUPPORTED;
    }
    const DevModel& dm = model->dm;
    if (ray_nr >= dm.nrays) {
        set_error("mgr_image: ray number out of range");
        return MGR_ERR_ARGUMENT;
    }
    const size_t PF = (size_t)dm.P * dm.F;
    double* dI = nullptr;
    cudaError_t e = cudaMalloc(&dI, PF * 8);
    if (e == cudaSuccess) e = (precision == MGR_PRECISION_SPLIT) ? dispatch_image<MODE_SPLIT>(model, ray_nr, dI)
                                                                : dispatch_image<MODE_FP64>(model, ray_nr, dI);
    if (e == cudaSuccess) e = cudaMemcpyAsync(I, dI, PF * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    cudaFree(dI);
    if (e != cudaSuccess) return cuda_fail(e, "image");
    if (ImX && ImY) {
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

int mgr_image_new(MgrModel* model, int precision, const double* raydir, uint32_t nx, uint32_t ny, double* I,
                  double* ImX, double* ImY) {
    if (!model || !raydir || !I || nx == 0 || ny == 0) {
        set_error("mgr_image_new: null argument or empty image");
        return MGR_ERR_ARGUMENT;
    }
    if (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) {
        set_error("mgr_image_new: unknown precision mode");
        return MGR_ERR_ARGUMENT;
    }
    if (model->dm.approx == APPROX_ONELINE) {
        set_error("mgr_image_new: One line approximation is not supported for imaging.");
        return MGR_ERR_UNSUPPORTED;
    }
    const double n2 = raydir[0] * raydir[0] + raydir[1] * raydir[1] + raydir[2] * raydir[2];
    if (n2 == 0.0) {
        set_error("mgr_image_new: The given ray direction vector does not point in a direction.");
        return MGR_ERR_ARGUMENT;
    }
    const DevModel& dm = model->dm;
    const uint32_t P = dm.P;
    const std::vector<double>& pos = model->host_pos;
    const std::vector<uint32_t>& p2b = model->host_p2b;
    ImagePlane ip{};
    const double inv = 1 / std::sqrt(n2);
    for (int k = 0; k < 3; k++) ip.d[k] = raydir[k] * inv;
    plane_axes(ip.d, ip.ix, ip.iy, ip.jx, ip.jy, ip.jz, ip.tilted);
    // boundary2point from point2boundary
    std::vector<uint32_t> b2p(dm.B);
    for (uint32_t p = 0; p < P; p++)
        if (p2b[p] < dm.B) b2p[p2b[p]] = p;
    // Image::set_coordinates_projection_surface (image.cpp:221-366)
    double max_x = -1.7976931348623157e308, max_y = -1.7976931348623157e308;
    double min_x = 1.7976931348623157e308, min_y = 1.7976931348623157e308;
    for (uint32_t b = 0; b < dm.B; b++) {
        const double* x = pos.data() + 3 * (size_t)b2p[b];
        double X, Y;
        if (ip.tilted) {
            X = ip.ix * x[0] + ip.iy * x[1];
            Y = ip.jx * x[0] + ip.jy * x[1] + ip.jz * x[2];
        } else {
            X = x[0];
            Y = x[1];
        }
        min_x = std::fmin(min_x, X);
        max_x = std::fmax(max_x, X);
        min_y = std::fmin(min_y, Y);
        max_y = std::fmax(max_y, Y);
    }
    // get_closest_bdy_point_in_custom_raydir (geometry.tpp:346-367); the reference
    // starts from point2boundary[0] read as a point index (the first boundary point
    // where that is no point index)
    auto proj = [&](uint32_t p) {
        const double* x = pos.data() + 3 * (size_t)p;
        return (ip.d[0] * x[0] + ip.d[1] * x[1]) + ip.d[2] * x[2];
    };
    uint32_t cbp = p2b[0] < P ? p2b[0] : (dm.B ? b2p[0] : 0);
    double pmin = proj(cbp);
    for (uint32_t b = 1; b < dm.B; b++) {
        const double pd = proj(b2p[b]);
        if (pd < pmin) {
            cbp = b2p[b];
            pmin = pd;
        }
    }
    ip.start = cbp;
    const double dist = proj(cbp);
    for (int k = 0; k < 3; k++) ip.scp[k] = ip.d[k] * dist;
    double lo[3] = {1.7976931348623157e308, 1.7976931348623157e308, 1.7976931348623157e308};
    double hi[3] = {-1.7976931348623157e308, -1.7976931348623157e308, -1.7976931348623157e308};
    for (uint32_t p = 0; p < P; p++)
        for (int k = 0; k < 3; k++) {
            lo[k] = std::fmin(lo[k], pos[3 * (size_t)p + k]);
            hi[k] = std::fmax(hi[k], pos[3 * (size_t)p + k]);
        }
    for (int k = 0; k < 3; k++) ip.center[k] = (lo[k] + hi[k]) / 2;
    const double deltax = (max_x - min_x) / nx, deltay = (max_y - min_y) / ny;
    const size_t npix = (size_t)nx * ny;
    std::vector<double> hx(npix), hy(npix);
    for (uint32_t xi = 0; xi < nx; xi++)
        for (uint32_t yi = 0; yi < ny; yi++) {
            hx[yi + (size_t)ny * xi] = min_x + deltax / 2.0 + xi * deltax;
            hy[yi + (size_t)ny * xi] = min_y + deltay / 2.0 + yi * deltay;
        }
    ip.nx = nx;
    ip.ny = ny;
    double *dx = nullptr, *dy = nullptr, *dI = nullptr;
    uint32_t* dmax = nullptr;
    cudaError_t e = cudaMalloc(&dx, npix * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dy, npix * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dI, npix * dm.F * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dmax, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, hx.data(), npix * 8, cudaMemcpyHostToDevice, model->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dy, hy.data(), npix * 8, cudaMemcpyHostToDevice, model->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(dmax, 0, sizeof(uint32_t), model->stream);
    ip.ImX = dx;
    ip.ImY = dy;
    uint32_t cap = 0;
    if (e == cudaSuccess) {
        count_launch();
        const unsigned blocks = (unsigned)std::min<size_t>((npix * 32 + 255) / 256, (size_t)model->sm_count * 16);
        image_size_kernel<<<blocks ? blocks : 1, 256, 0, model->stream>>>(dm, ip, dmax, model->status);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&cap, dmax, sizeof(uint32_t), cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    if (cap < 1) cap = 1;
    if (e == cudaSuccess)
        e = (precision == MGR_PRECISION_SPLIT) ? dispatch_image_new<MODE_SPLIT>(model, ip, cap, dI)
                                               : dispatch_image_new<MODE_FP64>(model, ip, cap, dI);
    if (e == cudaSuccess) e = cudaMemcpyAsync(I, dI, npix * dm.F * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    cudaFree(dx);
    cudaFree(dy);
    cudaFree(dI);
    cudaFree(dmax);
    if (e != cudaSuccess) return cuda_fail(e, "image_new");
    if (ImX) std::copy(hx.begin(), hx.end(), ImX);
    if (ImY) std::copy(hy.begin(), hy.end(), ImY);
    return mgr_sync(model);
}

}  // extern "C"
