// Short characteristics, order 0: Model::compute_radiation_field_shortchar_order_0
// (src/model/model.cpp:313-349) -> Solver::solve_shortchar_order_0
// (src/solver/solver.tpp:150-235, :1564-1757).
//
// Same two-stage structure as the Feautrier solve: stage 1 has one warp per
// (origin, ray pair) item and one lane per frequency; each lane integrates both
// halves of its ray pair toward the origin (solve_lane_sc0) and writes I(rr), I(ar),
// u, v and the per-direction ALO factors; stage 2 sums J and the ALO diagonal per
// origin in the reference's order (ray pair outer, quadrature point inner, forward
// then backward direction).
#include "mgr_internal.h"
#include "mgr_solve.cuh"

namespace mgr {

template <int MODE, int AP, int MINB>
__global__ void __launch_bounds__(256, MINB)
    sc0_kernel(DevModel m, uint32_t cap, uint32_t o_begin, uint32_t o_end, double* __restrict__ U, size_t u_stride,
               uint32_t u_o0, double* __restrict__ XF, double* __restrict__ XB, size_t x_stride, uint32_t x_o0,
               double* __restrict__ I, double* __restrict__ V, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nw = blockDim.x >> 5;
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    double* sl = reinterpret_cast<double*>(smem);
    const uint32_t Lpad = (m.L + 1) & ~1u;
    HalfSmem bk, fw;
    carve_halves(smem + (size_t)Lpad * 8 + (size_t)w * half_bytes_per_warp(cap), cap, bk, fw);
    for (uint32_t i = threadIdx.x; i < m.L; i += blockDim.x) sl[i] = m.sorted_line[i];
    __syncthreads();
    const uint32_t R = m.hnrays;
    const uint64_t n_items = (uint64_t)(o_end - o_begin) * R;
    const uint64_t stride = (uint64_t)gridDim.x * nw;
    for (uint64_t item = (uint64_t)blockIdx.x * nw + w; item < n_items; item += stride) {
        const uint32_t o = o_begin + (uint32_t)(item / R);
        const uint32_t rr = (uint32_t)(item % R);
        const uint32_t ar = m.antipod[rr];
        int nb = 0, nf = 0;
        trace_pair<true>(m, o, rr, ar, cap, bk, fw, lane, status, nb, nf);
        if (nb < 0 || nf < 0) continue;
        double* Ui = U + (size_t)rr * u_stride + (size_t)(o - u_o0) * m.F;
        const size_t xo = (size_t)rr * x_stride + (size_t)(o - x_o0) * m.F;
        for (uint32_t f0 = 0; f0 < m.F; f0 += 32) {
            const uint32_t f = f0 + lane;
            if (f < m.F) {
                const LaneCtx c = lane_ctx(m, o, f);
                const LaneResultSC r = solve_lane_sc0<MODE, AP>(m, sl, c, bk, nb, fw, nf);
                const double u = r.solved ? 0.5 * (r.If + r.Ib) : r.If;
                Ui[f] = u;
                if (XF) {
                    XF[xo + f] = r.Xf;
                    XB[xo + f] = r.Xb;
                }
                if (I) {
                    I[((size_t)rr * m.P + o) * m.F + f] = r.If;
                    I[((size_t)ar * m.P + o) * m.F + f] = r.Ib;
                }
                if (V) V[((size_t)rr * m.P + o) * m.F + f] = r.solved ? 0.5 * (r.If - r.Ib) : 0.0;
                if (!isfinite(u)) atomicOr(status, ST_NONFINITE);
            }
        }
        __syncwarp();
    }
}

// J(o, f) = sum_rr (2 w_rr) u(rr, o, f) (solver.tpp:205-223);
// Lambda(o, l) = sum_rr sum_q [element(forward) + element(backward)].
__global__ void __launch_bounds__(128) sc0_reduce_kernel(DevModel m, uint32_t o_begin, uint32_t o_end,
                                                         const double* __restrict__ U, size_t u_stride,
                                                         uint32_t u_o0, const double* __restrict__ XF,
                                                         const double* __restrict__ XB, size_t x_stride,
                                                         uint32_t x_o0, double* __restrict__ J,
                                                         double* __restrict__ lam) {
    const int nw = blockDim.x >> 5;
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t R = m.hnrays;
    for (uint32_t o = o_begin + blockIdx.x; o < o_end; o += gridDim.x) {
        for (uint32_t f = threadIdx.x; f < m.F; f += blockDim.x) {
            const double* Uo = U + (size_t)(o - u_o0) * m.F + f;
            double s = 0.0;
            for (uint32_t rr = 0; rr < R; rr++) s += (ray_w(m, o, rr) * 2.0) * Uo[(size_t)rr * u_stride];
            J[(size_t)o * m.F + f] = s;
        }
        if (!lam) continue;
        for (uint32_t l = w; l < m.L; l += nw) {
            const uint32_t* l2f = m.lq2f + (size_t)l * m.Q;
            double s = 0.0;
            for (uint32_t rr = 0; rr < R; rr++) {
                const size_t xo = (size_t)rr * x_stride + (size_t)(o - x_o0) * m.F;
                for (uint32_t q0 = 0; q0 < m.Q; q0 += 32) {
                    const uint32_t q = q0 + lane;
                    const uint32_t f = q < m.Q ? l2f[q] : 0xffffffffu;
                    double ef = 0.0, eb = 0.0;
                    bool add = false;
                    if (f != 0xffffffffu && m.in_line[f]) {
                        const double xf = XF[xo + f], xb = XB[xo + f];
                        add = (xf != 0.0) || (xb != 0.0);  // solved pairs only (update_Lambda per direction)
                        if (add) {
                            const LambdaFactors k = lambda_factors(m, m.sorted_line, o, f);
                            ef = lambda_element_sc0(k, ray_w(m, o, rr), xf);
                            eb = lambda_element_sc0(k, ray_w(m, o, rr), xb);
                        }
                    }
                    const uint32_t nq = min(32u, m.Q - q0);
                    for (uint32_t j = 0; j < nq; j++) {
                        s += __shfl_sync(FULL_MASK, ef, j);
                        s += __shfl_sync(FULL_MASK, eb, j);
                    }
                }
            }
            if (lane == 0) lam[(size_t)o * m.L + l] = s;
        }
    }
}

static size_t sc0_bytes_per_origin(const MgrModel* model) { return (size_t)model->dm.hnrays * model->dm.F * 8; }

size_t sc0_work_bytes(const MgrModel* model, uint32_t n_origins, bool stage_u, bool stage_x) {
    const int k = (stage_u ? 1 : 0) + (stage_x ? 2 : 0);
    if (k == 0 || n_origins == 0) return 0;
    const size_t per = sc0_bytes_per_origin(model) * k;
    size_t chunk = kFo2WorkBudget / per;
    if (chunk < 1) chunk = 1;
    if (chunk > n_origins) chunk = n_origins;
    return chunk * per;
}

template <int MODE, int AP, int MINB>
static cudaError_t launch_sc0_variant(MgrModel* model, uint32_t c0, uint32_t c1, double* U, size_t us, uint32_t uo,
                                      double* XF, double* XB, size_t xs, uint32_t xo, double* I, double* V) {
    const DevModel& m = model->dm;
    const uint32_t cap = model->half_cap;
    int nw = (MODE == MODE_SPLIT) ? model->fo2_warps_split : model->fo2_warps_fp64;
    if (nw < 1 || nw > 8) nw = 8;
    const uint32_t Lpad = (m.L + 1) & ~1u;
    const size_t smem = (size_t)Lpad * 8 + (size_t)nw * half_bytes_per_warp(cap);
    auto kern = sc0_kernel<MODE, AP, MINB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nw * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const uint64_t items = (uint64_t)(c1 - c0) * m.hnrays;
    uint64_t grid = (uint64_t)model->sm_count * per_sm;
    const uint64_t need = (items + nw - 1) / nw;
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    count_launch();
    kern<<<(unsigned)grid, nw * 32, smem, model->stream>>>(m, cap, c0, c1, U, us, uo, XF, XB, xs, xo, I, V,
                                                           model->status);
    return cudaGetLastError();
}

template <int MODE, int AP>
static cudaError_t launch_sc0_minb(MgrModel* model, uint32_t c0, uint32_t c1, double* U, size_t us, uint32_t uo,
                                   double* XF, double* XB, size_t xs, uint32_t xo, double* I, double* V) {
    const int minb = (MODE == MODE_SPLIT) ? model->fo2_minb_split : model->fo2_minb_fp64;
    if (minb == 2) return launch_sc0_variant<MODE, AP, 2>(model, c0, c1, U, us, uo, XF, XB, xs, xo, I, V);
    if (minb == 4) return launch_sc0_variant<MODE, AP, 4>(model, c0, c1, U, us, uo, XF, XB, xs, xo, I, V);
    return launch_sc0_variant<MODE, AP, 3>(model, c0, c1, U, us, uo, XF, XB, xs, xo, I, V);
}

template <int MODE>
static cudaError_t launch_sc0_approx(MgrModel* model, uint32_t c0, uint32_t c1, double* U, size_t us, uint32_t uo,
                                     double* XF, double* XB, size_t xs, uint32_t xo, double* I, double* V) {
    switch (model->dm.approx) {
        case APPROX_ONELINE:
            return launch_sc0_minb<MODE, APPROX_ONELINE>(model, c0, c1, U, us, uo, XF, XB, xs, xo, I, V);
        case APPROX_CLOSELINES:
            return launch_sc0_minb<MODE, APPROX_CLOSELINES>(model, c0, c1, U, us, uo, XF, XB, xs, xo, I, V);
        default: return launch_sc0_minb<MODE, APPROX_NONE>(model, c0, c1, U, us, uo, XF, XB, xs, xo, I, V);
    }
}

cudaError_t launch_sc0_range(MgrModel* model, int precision, uint32_t o_begin, uint32_t o_end, double* J, double* I,
                             double* u, double* v, double* lam, double* work, size_t work_bytes) {
    const DevModel& m = model->dm;
    if (o_end <= o_begin) return cudaSuccess;
    const int k = (u ? 0 : 1) + (lam ? 2 : 0);
    const size_t per = sc0_bytes_per_origin(model);
    uint32_t chunk = o_end - o_begin;
    if (k) {
        const size_t fit = work ? work_bytes / (per * k) : 0;
        if (fit < 1) return cudaErrorInvalidValue;
        if (fit < chunk) chunk = (uint32_t)fit;
    }
    for (uint32_t c0 = o_begin; c0 < o_end; c0 += chunk) {
        const uint32_t c1 = (o_end - c0 > chunk) ? c0 + chunk : o_end;
        const uint32_t n = c1 - c0;
        const size_t slab = (size_t)m.hnrays * n * m.F;
        double *U, *next = work;
        size_t us;
        uint32_t uo;
        if (u) {
            U = u;
            us = (size_t)m.P * m.F;
            uo = 0;
        } else {
            U = work;
            us = (size_t)n * m.F;
            uo = c0;
            next = work + slab;
        }
        double* XF = lam ? next : nullptr;
        double* XB = lam ? next + slab : nullptr;
        const size_t xs = (size_t)n * m.F;
        cudaError_t e = (precision == MGR_PRECISION_SPLIT)
                            ? launch_sc0_approx<MODE_SPLIT>(model, c0, c1, U, us, uo, XF, XB, xs, c0, I, v)
                            : launch_sc0_approx<MODE_FP64>(model, c0, c1, U, us, uo, XF, XB, xs, c0, I, v);
        if (e != cudaSuccess) return e;
        const unsigned grid = n < (uint32_t)model->sm_count * 16 ? n : (unsigned)model->sm_count * 16;
        count_launch();
        sc0_reduce_kernel<<<grid, 128, 0, model->stream>>>(m, c0, c1, U, us, uo, XF, XB, xs, c0, J, lam);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace mgr

using namespace mgr;

extern "C" {

int mgr_formal_solve_sc0_device(MgrModel* model, int precision, double* J_dev, double* I_dev, double* u_dev,
                                double* v_dev, double* lambda_diag_dev) {
    MGR_MODEL_DEVICE(model);
    if (!model || !J_dev) {
        set_error("mgr_formal_solve_sc0_device: null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) {
        set_error("mgr_formal_solve_sc0_device: unknown precision mode");
        return MGR_ERR_ARGUMENT;
    }
    if (!model->line_disc) {
        set_error("mgr_formal_solve_sc0_device: needs a line spectral discretisation");
        return MGR_ERR_UNSUPPORTED;
    }
    const size_t wb = sc0_work_bytes(model, model->dm.P, u_dev == nullptr, lambda_diag_dev != nullptr);
    if (model->work_bytes < wb) {
        if (model->work) cudaFree(model->work);
        model->work = nullptr;
        model->work_bytes = 0;
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, wb);
        if (e != cudaSuccess) return cuda_fail(e, "scratch allocation");
        model->work = static_cast<double*>(q);
        model->work_bytes = wb;
    }
    cudaError_t e = launch_sc0_range(model, precision, 0, model->dm.P, J_dev, I_dev, u_dev, v_dev, lambda_diag_dev,
                                     model->work, model->work_bytes);
    if (e != cudaSuccess) return cuda_fail(e, "short-characteristics launch");
    model->last_J = J_dev;
    model->last_lam = lambda_diag_dev;
    model->last_alo_off = nullptr;
    model->last_alo_nr = nullptr;
    return MGR_OK;
}

int mgr_formal_solve_sc0(MgrModel* model, int precision, double* J, double* I, double* u, double* v,
                         double* lambda_diag) {
    MGR_MODEL_DEVICE(model);
    if (!model || !J) {
        set_error("mgr_formal_solve_sc0: null argument");
        return MGR_ERR_ARGUMENT;
    }
    const DevModel& dm = model->dm;
    const size_t PF = (size_t)dm.P * dm.F, PL = (size_t)dm.P * dm.L, RPF = PF * dm.hnrays;
    struct Buf {
        double* p = nullptr;
        ~Buf() {
            if (p) cudaFree(p);
        }
    } dI, du, dv;
    auto dev = [&](double** p, size_t* have, size_t bytes) -> cudaError_t {
        if (*have >= bytes) return cudaSuccess;
        if (*p) cudaFree(*p);
        *p = nullptr;
        *have = 0;
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, bytes);
        if (e == cudaSuccess) {
            *p = static_cast<double*>(q);
            *have = bytes;
        }
        return e;
    };
    cudaError_t e = dev(&model->J_scratch, &model->J_scratch_bytes, PF * 8);
    if (e == cudaSuccess && lambda_diag) e = dev(&model->lam_scratch, &model->lam_scratch_bytes, PL * 8);
    if (e == cudaSuccess && I) e = cudaMalloc(&dI.p, 2 * RPF * 8);
    if (e == cudaSuccess && u) e = cudaMalloc(&du.p, RPF * 8);
    if (e == cudaSuccess && v) e = cudaMalloc(&dv.p, RPF * 8);
    if (e != cudaSuccess) return cuda_fail(e, "output allocation");
    int rc = mgr_formal_solve_sc0_device(model, precision, model->J_scratch, dI.p, du.p, dv.p,
                                         lambda_diag ? model->lam_scratch : nullptr);
    if (rc != MGR_OK) return rc;
    e = cudaMemcpyAsync(J, model->J_scratch, PF * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && I) e = cudaMemcpyAsync(I, dI.p, 2 * RPF * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && u) e = cudaMemcpyAsync(u, du.p, RPF * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && v) e = cudaMemcpyAsync(v, dv.p, RPF * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && lambda_diag)
        e = cudaMemcpyAsync(lambda_diag, model->lam_scratch, PL * 8, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "result copy");
    return mgr_sync(model);
}

}  // extern "C"
