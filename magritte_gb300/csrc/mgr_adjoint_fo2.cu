// Differentiable formal solve on the GPU: the smooth FP64 J (forward) and its adjoint
// (backward) of Model::compute_radiation_field_feautrier_order_2 (model.cpp:353-390 ->
// Solver::solve_feautrier_order_2, solver.tpp:458-540), plus the device-pointer update
// of the model's frequencies that an autograd wrapper needs between calls.
//
// Both kernels run one warp per origin (grid-stride over the origins, or over a list
// of them).  The warp walks the ray pairs in order, tracing both halves into shared
// memory; for each line it runs the lanes over that line's quadrature points (so all
// lanes share the ray's elements, which the adjoint's warp sums need), and J(o, f) is
// accumulated in shared memory in the reference's ray-pair order.  The backward keeps
// each lane's per-pair elimination state in a scratch array of the warp's slot
// (recomputed, not saved by the forward) and adds its derivatives with one atomic per
// warp and entry.
#include <algorithm>
#include <vector>

#include "mgr_adjoint_fo2.cuh"
#include "mgr_internal.h"

namespace mgr {

template <int AP>
__global__ void __launch_bounds__(256) fo2_s_kernel(DevModel m, uint32_t cap, const uint32_t* __restrict__ olist,
                                                    uint32_t n_o, double* __restrict__ J, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nw = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t Lpad = (m.L + 1) & ~1u, Fpad = (m.F + 1) & ~1u;
    double* sl = reinterpret_cast<double*>(smem);
    double* Jacc = sl + Lpad + (size_t)w * Fpad;
    HalfSmem bk, fw;
    carve_halves(smem + ((size_t)Lpad + (size_t)nw * Fpad) * 8 + (size_t)w * half_bytes_per_warp(cap), cap, bk, fw);
    for (uint32_t i = threadIdx.x; i < m.L; i += blockDim.x) sl[i] = m.sorted_line[i];
    __syncthreads();
    for (uint32_t item = blockIdx.x * nw + w; item < n_o; item += gridDim.x * nw) {
        const uint32_t o = olist ? olist[item] : item;
        for (uint32_t f = lane; f < m.F; f += 32) Jacc[f] = 0.0;
        __syncwarp();
        bool ok = true;
        for (uint32_t rr = 0; rr < m.hnrays; rr++) {
            int nb = 0, nf = 0;
            trace_pair<true, 0, 1>(m, o, rr, m.antipod[rr], cap, bk, fw, lane, status, nb, nf);
            if (nb < 0 || nf < 0) {
                ok = false;  // status recorded by the trace
                break;
            }
            const double wt = 2.0 * ray_w(m, o, rr);
            for (uint32_t l = 0; l < m.L; l++)
                for (uint32_t q0 = 0; q0 < m.Q; q0 += 32) {
                    const uint32_t q = q0 + lane;
                    if (q < m.Q) {
                        const uint32_t f = m.lq2f[(size_t)l * m.Q + q];
                        const LaneS r = solve_lane_s<AP>(m, sl, o, m.nu[(size_t)o * m.F + f], l, bk, nb, fw, nf,
                                                         nullptr);
                        Jacc[f] += r.u * wt;
                    }
                }
            __syncwarp();
        }
        if (ok)
            for (uint32_t f = lane; f < m.F; f += 32) {
                const double v = Jacc[f];
                J[(size_t)o * m.F + f] = v;
                if (!isfinite(v)) atomicOr(status, ST_NONFINITE);
            }
        __syncwarp();
    }
}

template <int AP>
__global__ void __launch_bounds__(256) fo2_adj_kernel(DevModel m, uint32_t cap, const uint32_t* __restrict__ olist,
                                                      uint32_t n_o, const double* __restrict__ gJ, AdjGrads g,
                                                      double* __restrict__ g_nu, double* __restrict__ scratch,
                                                      uint32_t scratch_pairs, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nw = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t Lpad = (m.L + 1) & ~1u, Fpad = (m.F + 1) & ~1u;
    double* sl = reinterpret_cast<double*>(smem);
    double* gnu_acc = sl + Lpad + (size_t)w * Fpad;
    HalfSmem bk, fw;
    carve_halves(smem + ((size_t)Lpad + (size_t)nw * Fpad) * 8 + (size_t)w * half_bytes_per_warp(cap), cap, bk, fw);
    for (uint32_t i = threadIdx.x; i < m.L; i += blockDim.x) sl[i] = m.sorted_line[i];
    __syncthreads();
    const size_t slot = (size_t)blockIdx.x * nw + w;
    const Fo2Scratch scr{scratch + slot * (size_t)scratch_pairs * 4 * 32 + lane, 32, scratch_pairs};
    for (uint32_t item = blockIdx.x * nw + w; item < n_o; item += gridDim.x * nw) {
        const uint32_t o = olist ? olist[item] : item;
        // origins without a derivative of the loss contribute nothing
        bool any = false;
        for (uint32_t f = lane; f < m.F; f += 32) any |= gJ[(size_t)o * m.F + f] != 0.0;
        if (!__any_sync(FULL_MASK, any)) continue;
        for (uint32_t f = lane; f < m.F; f += 32) gnu_acc[f] = 0.0;
        __syncwarp();
        double vo[3] = {0.0, 0.0, 0.0};
        for (uint32_t rr = 0; rr < m.hnrays; rr++) {
            const uint32_t ar = m.antipod[rr];
            int nb = 0, nf = 0;
            trace_pair<true, 0, 1>(m, o, rr, ar, cap, bk, fw, lane, status, nb, nf);
            if (nb < 0 || nf < 0) break;
            const double* db = ray_dir(m, o, rr);
            const double* df = ray_dir(m, o, ar);
            AdjGrads gb = g, gf = g;
            for (int k = 0; k < 3; k++) {
                gb.d[k] = db[k];
                gf.d[k] = df[k];
            }
            const AdjAcc acc_b{gb, m.L}, acc_f{gf, m.L};
            const double wt = 2.0 * ray_w(m, o, rr);
            for (uint32_t l = 0; l < m.L; l++)
                for (uint32_t q0 = 0; q0 < m.Q; q0 += 32) {
                    const uint32_t q = q0 + lane;
                    const uint32_t f = m.lq2f[(size_t)l * m.Q + (q < m.Q ? q : m.Q - 1)];
                    const double gu = q < m.Q ? gJ[(size_t)o * m.F + f] * wt : 0.0;
                    if (!__any_sync(FULL_MASK, gu != 0.0)) continue;
                    double gvb = 0.0, gvf = 0.0, gn = 0.0;
                    if (!solve_lane_s_adj<AP>(m, sl, o, m.nu[(size_t)o * m.F + f], l, bk, nb, fw, nf, gu, scr,
                                              acc_b, acc_f, gvb, gvf, gn)) {
                        if (lane == 0) atomicOr(status, ST_CAPACITY);
                        continue;
                    }
                    for (int k = 0; k < 3; k++) vo[k] += gvb * db[k] + gvf * df[k];
                    if (q < m.Q) gnu_acc[f] += gn;
                    __syncwarp();
                }
        }
        for (int k = 0; k < 3; k++) {
            double v = vo[k];
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(FULL_MASK, v, off);
            if (lane == 0 && v != 0.0) atomicAdd(g.vel + 3 * (size_t)o + k, v);
        }
        __syncwarp();
        for (uint32_t f = lane; f < m.F; f += 32) g_nu[(size_t)o * m.F + f] += gnu_acc[f];
        __syncwarp();
    }
}

// Launch shape of the per-origin kernels: CTAs of up to 8 warps whose ray buffers and
// per-warp frequency accumulators fit in shared memory.
template <typename K>
static cudaError_t origin_launch_shape(MgrModel* model, K kern, uint32_t cap, uint64_t items, int* nw_out,
                                       size_t* smem_out, unsigned* grid_out) {
    const uint32_t Lpad = (model->dm.L + 1) & ~1u, Fpad = (model->dm.F + 1) & ~1u;
    int nw = 8;
    auto bytes = [&](int n) { return ((size_t)Lpad + (size_t)n * Fpad) * 8 + (size_t)n * half_bytes_per_warp(cap); };
    while (nw > 1 && bytes(nw) > 200 * 1024) nw /= 2;
    const size_t smem = bytes(nw);
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

static int check_smooth_model(MgrModel* model, const char* who) {
    if (!model->line_disc) {
        set_error(std::string(who) + ": the formal solve needs a line spectral discretisation");
        return MGR_ERR_UNSUPPORTED;
    }
    if (model->dm.sph) {
        set_error(std::string(who) + ": the differentiable formal solve does not support spherically symmetric models");
        return MGR_ERR_UNSUPPORTED;
    }
    if (model->dm.approx == APPROX_ONELINE) {
        set_error(std::string(who) + ": the differentiable formal solve supports the None and CloseLines "
                                     "approximations");
        return MGR_ERR_UNSUPPORTED;
    }
    return MGR_OK;
}

static int finish_stream(MgrModel* model, cudaError_t e, const char* who) {
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

int mgr_model_set_frequencies_device(MgrModel* model, const double* nu_dev) {
    MGR_MODEL_DEVICE(model);
    if (!model || !nu_dev) {
        set_error("mgr_model_set_frequencies_device: null argument");
        return MGR_ERR_ARGUMENT;
    }
    cudaError_t e = cudaMemcpyAsync(const_cast<double*>(model->dm.nu), nu_dev, (size_t)model->dm.P * model->dm.F * 8,
                                    cudaMemcpyDeviceToDevice, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "frequency update");
    model->inputs_replaced = true;
    return MGR_OK;
}

int mgr_formal_solve_fo2_smooth_device(MgrModel* model, const uint32_t* origins_dev, uint32_t n_origins,
                                       double* J_dev) {
    MGR_MODEL_DEVICE(model);
    if (!model || !J_dev) {
        set_error("mgr_formal_solve_fo2_smooth_device: null argument");
        return MGR_ERR_ARGUMENT;
    }
    int rc = check_smooth_model(model, "mgr_formal_solve_fo2_smooth_device");
    if (rc != MGR_OK) return rc;
    const uint32_t n_o = origins_dev ? n_origins : model->dm.P;
    if (n_o == 0) return MGR_OK;
    const uint32_t cap = model->half_cap;
    int nw;
    size_t smem;
    unsigned grid;
    auto run = [&](auto kern) -> cudaError_t {
        cudaError_t r = origin_launch_shape(model, kern, cap, n_o, &nw, &smem, &grid);
        if (r != cudaSuccess) return r;
        count_launch();
        kern<<<grid, nw * 32, smem, model->stream>>>(model->dm, cap, origins_dev, n_o, J_dev, model->status);
        return cudaGetLastError();
    };
    cudaError_t e = (model->dm.approx == APPROX_CLOSELINES) ? run(fo2_s_kernel<APPROX_CLOSELINES>)
                                                             : run(fo2_s_kernel<APPROX_NONE>);
    return finish_stream(model, e, "mgr_formal_solve_fo2_smooth_device");
}

int mgr_formal_solve_fo2_adjoint_device(MgrModel* model, const uint32_t* origins_dev, uint32_t n_origins,
                                        const double* gJ_dev, double* g_em_dev, double* g_op_dev, double* g_iw_dev,
                                        double* g_Sp_dev, double* g_vel_dev, double* g_nu_dev) {
    MGR_MODEL_DEVICE(model);
    if (!model || !gJ_dev || !g_em_dev || !g_op_dev || !g_iw_dev || !g_Sp_dev || !g_vel_dev || !g_nu_dev) {
        set_error("mgr_formal_solve_fo2_adjoint_device: null argument");
        return MGR_ERR_ARGUMENT;
    }
    int rc = check_smooth_model(model, "mgr_formal_solve_fo2_adjoint_device");
    if (rc != MGR_OK) return rc;
    const uint32_t n_o = origins_dev ? n_origins : model->dm.P;
    if (n_o == 0) return MGR_OK;
    const uint32_t cap = model->half_cap;
    // pairs of the longest ray pair: elements with the interpolation points of all
    // lines (Solver::get_ray_lengths_max), an upper bound of every line's count
    uint32_t* dmax = nullptr;
    uint32_t pairs = 0;
    cudaError_t e = cudaMalloc(&dmax, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(dmax, 0, sizeof(uint32_t), model->stream);
    if (e == cudaSuccess) e = launch_ray_lengths(model, dmax);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&pairs, dmax, sizeof(uint32_t), cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    cudaFree(dmax);
    if (e != cudaSuccess) return cuda_fail(e, "mgr_formal_solve_fo2_adjoint_device: ray lengths");
    if (pairs < 1) pairs = 1;
    AdjGrads g{g_em_dev, g_op_dev, g_iw_dev, g_Sp_dev, g_vel_dev, {0.0, 0.0, 0.0}};
    int nw;
    size_t smem;
    unsigned grid;
    auto run = [&](auto kern) -> cudaError_t {
        cudaError_t r = origin_launch_shape(model, kern, cap, n_o, &nw, &smem, &grid);
        if (r != cudaSuccess) return r;
        const size_t need = (size_t)grid * nw * pairs * 4 * 32 * sizeof(double);
        if (model->adj_scratch_bytes < need) {  // grown on demand, kept for the next call
            cudaFree(model->adj_scratch);
            model->adj_scratch = nullptr;
            model->adj_scratch_bytes = 0;
            r = cudaMalloc(&model->adj_scratch, need);
            if (r != cudaSuccess) return r;
            model->adj_scratch_bytes = need;
        }
        count_launch();
        kern<<<grid, nw * 32, smem, model->stream>>>(model->dm, cap, origins_dev, n_o, gJ_dev, g, g_nu_dev,
                                                     model->adj_scratch, pairs, model->status);
        return cudaGetLastError();
    };
    e = (model->dm.approx == APPROX_CLOSELINES) ? run(fo2_adj_kernel<APPROX_CLOSELINES>)
                                                : run(fo2_adj_kernel<APPROX_NONE>);
    return finish_stream(model, e, "mgr_formal_solve_fo2_adjoint_device");
}

}  // extern "C"
