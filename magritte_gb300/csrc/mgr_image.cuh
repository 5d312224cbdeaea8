// Image-plane geometry and pixel-ray tracing of the new imager (shared by the
// imager and its adjoint).
#pragma once
#include <cmath>
#include <string>
#include <vector>

#include "mgr_internal.h"
#include "mgr_solve.cuh"

namespace mgr {

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
    bool sph;                   // 1D spherical symmetry (shell walk from the pixel origin)
    uint32_t nx, ny;
    const double* ImX;          // [nx*ny] device
    const double* ImY;
};

static __device__ __forceinline__ void pixel_origin(const ImagePlane& ip, double x, double y, double* o) {
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
static __device__ uint32_t bdy_point_closer(const DevModel& m, const double* org, const ImagePlane& ip, uint32_t crt,
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

// Geometry::get_shift<Rest>(origin, 0, raydir, c, Z, false) of a pixel ray (motionless
// origin): 1 + v[c] . d, or in spherical symmetry 1 + v_x[c] (origin . d + Z) / x[c]
// (geometry.tpp:407-417; 1 at x[c] = 0).
static __host__ __device__ __forceinline__ double image_shift(const DevModel& m, const double* org,
                                                              const ImagePlane& ip, uint32_t c, double Z) {
    if (ip.sph) {
        const double xc = m.pos[c].x;
        if (xc == 0.0) return 1.0;
        const double RcZ = dadd_rn(dot3_rn(org[0], org[1], org[2], ip.d[0], ip.d[1], ip.d[2]), Z);
        return dadd_rn(1.0, ddiv_rn(dmul_rn(m.vel[c].x, RcZ), xc));
    }
    const double4_32a v = m.vel[c];
    return dadd_rn(1.0, dot3_rn(v.x, v.y, v.z, ip.d[0], ip.d[1], ip.d[2]));
}

// Solver::trace_ray_imaging (solver.tpp:841-897), increment -1: walks from the start
// boundary point through the model until it leaves on the far side; rest-frame
// shifts 1 + v . d of a motionless observer.  Returns the steps stored, 0 if the ray
// met no interior point (the reference then keeps only the start point), -1 on
// capacity overflow.
template <bool STORE>
static __device__ int trace_image(const DevModel& m, const double* org, const ImagePlane& ip, uint32_t start, double Z,
                           uint32_t cap, HalfSmem h, int lane, int* status) {
    const double dx = ip.d[0], dy = ip.d[1], dz = ip.d[2];
    uint32_t crt = start;
    int count = 0;
    bool accessed = false;
    if (ip.sph) {
        // Geometry::get_next_spherical_symmetry from the pixel origin (every lane steps the
        // same shells; lane 0 stores each step with its shift at its distance Z)
        const double Rcos = dot3_rn(org[0], org[1], org[2], dx, dy, dz);
        const double Rsin2 = dsub_rn(dot3_rn(org[0], org[1], org[2], org[0], org[1], org[2]), dmul_rn(Rcos, Rcos));
        while (true) {
            uint32_t nxt;
            double dZl;
            if (!next_point_sph(m, Rcos, Rsin2, crt, Z, nxt, dZl)) break;
            if (STORE && (uint32_t)count >= cap) {
                if (lane == 0) atomicOr(status, ST_CAPACITY);
                count = -1;
                break;
            }
            Z = dadd_rn(Z, dZl);
            if (STORE && lane == 0) {
                h.ids[count] = nxt;
                h.eid[count] = sph_eid(crt, nxt);
                h.dZ[count] = dZl;
                const double sh = image_shift(m, org, ip, nxt, Z);
                h.shift[count] = sh;
                store_dsh(h, count, sh);
                h.dzs[count] = (float)dZl * m.dz_scale;
            }
            count++;
            if (m.p2b[nxt] != m.P) {
                const double4_32a pn = m.pos[nxt];
                const double side = dot3_rn(dsub_rn(pn.x, ip.center[0]), dsub_rn(pn.y, ip.center[1]),
                                            dsub_rn(pn.z, ip.center[2]), dx, dy, dz);
                if (!(side < 0.0)) break;
            }
            crt = nxt;
        }
        __syncwarp();
        return count;  // spherically symmetric models keep boundary-only rays (solver.tpp:891-896)
    }
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
            store_dsh(h, s, sh);
            h.dzs[s] = (float)h.dZ[s] * m.dz_scale;
        }
        __syncwarp();
    }
    return count;
}

// trace_ray_imaging_get_start (solver.tpp:808-830): the boundary point closest to the
// pixel's ray, found by a greedy walk over boundary neighbours.
static __device__ uint32_t pixel_start(const DevModel& m, const double* org, const ImagePlane& ip, int lane, double& Z) {
    uint32_t p = ip.start;
    for (uint32_t it = 0; it < m.P; it++) {  // a walk visits each point at most once
        const uint32_t q = bdy_point_closer(m, org, ip, p, lane);
        if (q == p) break;
        p = q;
    }
    const double4_32a ps = m.pos[p];
    Z = dot3_rn(dsub_rn(ps.x, org[0]), dsub_rn(ps.y, org[1]), dsub_rn(ps.z, org[2]), ip.d[0], ip.d[1], ip.d[2]);
    if (ip.sph) {
        // Geometry::get_distance_origin_to_boundary in spherical symmetry (geometry.tpp:172-190)
        const double Rcos = dot3_rn(org[0], org[1], org[2], ip.d[0], ip.d[1], ip.d[2]);
        const double Rsin2 = dsub_rn(dot3_rn(org[0], org[1], org[2], org[0], org[1], org[2]), dmul_rn(Rcos, Rcos));
        const double horz2 = dsub_rn(sqnorm_rn(ps), Rsin2);
        Z = horz2 > 0 ? dsub_rn(-dsqrt_rn(horz2), Rcos) : -Rcos;
    }
    return p;
}

static __global__ void image_size_kernel(DevModel m, ImagePlane ip, uint32_t* d_max, int* status) {
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


// Image axes of a ray direction (Image::Image, image.cpp:154-219).
inline void plane_axes(const double* d, double& ix, double& iy, double& jx, double& jy, double& jz, bool& tilted) {
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

// The projection plane of Model::compute_image_new from the model's positions
// [P][3] and point2boundary map (host computation; err receives the message).
inline int image_plane_compute(const double* pos, const uint32_t* p2b, uint32_t P, uint32_t B, const double* raydir,
                               uint32_t nx, uint32_t ny, ImagePlane& ip, std::vector<double>& hx,
                               std::vector<double>& hy, std::string& err, bool sph = false) {
    if (!raydir || nx == 0 || ny == 0) {
        err = "null direction or empty image";
        return MGR_ERR_ARGUMENT;
    }
    const double n2 = raydir[0] * raydir[0] + raydir[1] * raydir[1] + raydir[2] * raydir[2];
    if (n2 == 0.0) {
        err = "The given ray direction vector does not point in a direction.";
        return MGR_ERR_ARGUMENT;
    }
    ip = ImagePlane{};
    const double inv = 1 / std::sqrt(n2);
    for (int k = 0; k < 3; k++) ip.d[k] = raydir[k] * inv;
    plane_axes(ip.d, ip.ix, ip.iy, ip.jx, ip.jy, ip.jz, ip.tilted);
    // boundary2point from point2boundary
    std::vector<uint32_t> b2p(B);
    for (uint32_t p = 0; p < P; p++)
        if (p2b[p] < B) b2p[p2b[p]] = p;
    // Image::set_coordinates_projection_surface (image.cpp:221-366)
    double max_x = -1.7976931348623157e308, max_y = -1.7976931348623157e308;
    double min_x = 1.7976931348623157e308, min_y = 1.7976931348623157e308;
    for (uint32_t b = 0; b < B; b++) {
        const double* x = pos + 3 * (size_t)b2p[b];
        double X, Y;
        if (sph) {
            // 1D (image.cpp:257-269): the boundary shells' x, mirrored below
            min_x = std::fmin(min_x, x[0]);
            max_x = std::fmax(max_x, x[0]);
            continue;
        }
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
        const double* x = pos + 3 * (size_t)p;
        return (ip.d[0] * x[0] + ip.d[1] * x[1]) + ip.d[2] * x[2];
    };
    if (sph) {
        max_x = std::fmax(std::fabs(min_x), max_x);
        min_x = -max_x;
        min_y = min_x;
        max_y = max_x;
    }
    uint32_t cbp = p2b[0] < P ? p2b[0] : (B ? b2p[0] : 0);
    double pmin = proj(cbp);
    for (uint32_t b = 1; b < B; b++) {
        const double pd = proj(b2p[b]);
        if (pd < pmin) {
            cbp = b2p[b];
            pmin = pd;
        }
    }
    // spherical symmetry: the last point, and the plane at -x of it (geometry.tpp:348-350,
    // image.cpp:341-346)
    if (sph) cbp = P - 1;
    ip.start = cbp;
    ip.sph = sph;
    const double dist = sph ? -pos[3 * (size_t)cbp] : proj(cbp);
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
    hx.assign(npix, 0.0);
    hy.assign(npix, 0.0);
    for (uint32_t xi = 0; xi < nx; xi++)
        for (uint32_t yi = 0; yi < ny; yi++) {
            hx[yi + (size_t)ny * xi] = min_x + deltax / 2.0 + xi * deltax;
            hy[yi + (size_t)ny * xi] = min_y + deltay / 2.0 + yi * deltay;
        }
    ip.nx = nx;
    ip.ny = ny;
    return MGR_OK;
}

// Host set-up of the projection plane of Model::compute_image_new (image.cpp:154-398,
// geometry.tpp:346-367): validates the direction, fills the plane (axes, projection
// surface, start point) and the pixel coordinates hx / hy [nx*ny] (pixel y + ny*x).
// Returns MGR_OK or an error code with the message set (`who` prefixes it).
int image_plane_setup(MgrModel* model, const char* who, const double* raydir, uint32_t nx, uint32_t ny,
                      ImagePlane& ip, std::vector<double>& hx, std::vector<double>& hy);

// Uploads the pixel coordinates into d_xy [2*nx*ny] (device, owned by the caller), points
// ip.ImX / ip.ImY at them and sizes the longest pixel ray (trace steps) into *cap.
cudaError_t image_plane_upload(MgrModel* model, ImagePlane& ip, const std::vector<double>& hx,
                               const std::vector<double>& hy, double* d_xy, uint32_t* d_max, uint32_t* cap);

}  // namespace mgr
