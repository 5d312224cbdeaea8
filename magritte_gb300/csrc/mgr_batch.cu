// Many-model batch of second-order Feautrier formal solves in one persistent launch.
//
// Each model is an ordinary MgrModel (mgr_model_create); a batch collects their device
// descriptions into one device array and solves all of them with one kernel launch.
// The unit of work is one (model, origin) item handled by one warp: the warp traces
// and solves every ray pair of its origin in turn (lanes over frequencies, the same
// solve_lane code as the single-model kernel) and keeps J and the ALO elements of the
// origin in shared memory per frequency, summed over the ray pairs in order
// (Solver::solve_feautrier_order_2, solver.tpp:476-540, and update_Lambda,
// solver.tpp:1760-1850); each line's ALO diagonal is then the sum of its quadrature
// points' sums across the lanes, the association fo2_reduce_kernel uses.  Every
// model's J and ALO diagonal are therefore the values its own mgr_formal_solve_fo2
// returns, bit for bit, with no staging of per-ray results in HBM.
//
// Items are ordered model by model; warps take them in a grid-stride loop over a
// persistent grid, so models finish roughly in submission order.  Per model the
// kernel records, from the GPU's global timer, when its origin 0 started (origins
// start in order) and when its last origin finished (the per-model latency).
#include <algorithm>
#include <vector>

#include "mgr_internal.h"
#include "mgr_solve.cuh"

struct MgrBatch {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<MgrModel*> models;
    int approx = 0;
    uint32_t cap = 1;       // longest half ray over the batch (trace buffer, base steps)
    uint32_t F_max = 1, L_max = 1;
    uint64_t n_items = 0;   // total origins
    mgr::DevModel* d_models = nullptr;     // [n]
    uint64_t* d_offsets = nullptr;         // [n + 1] first item of each model
    double** d_J = nullptr;                // [n] output pointers
    double** d_lam = nullptr;              // [n]
    unsigned long long* d_t = nullptr;     // [n][2] first-start / last-finish ns, [2n] batch start
    uint32_t* d_done = nullptr;            // [n] finished items per model
    int* status = nullptr;
    mgr::DevModel* h_models = nullptr;     // pinned staging of the device descriptions
    int warps = 8;
    int minb = 2;
};

namespace mgr {

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Per-warp shared memory: the current model's DevModel, sorted line centres [L_max],
// J accumulators [F_max], ALO accumulators per frequency [F_max], the origin's
// ray-independent ALO factors [F_max] (LambdaFactors), then the two trace halves.
// The single-model kernels take their DevModel as a kernel parameter, whose fields the
// instructions read from the constant bank; a batch kernel indexes its models at run
// time, and reading each field from the descriptor array in global memory put a
// dependent global load in front of every table access and kept the loaded pointers
// live in registers (spills).  The warp copies its model's descriptor into shared
// memory when the model changes.
constexpr size_t kDescBytes = (sizeof(DevModel) + 15) & ~size_t(15);
__host__ __device__ inline size_t batch_head_bytes(uint32_t F_max, uint32_t L_max) {
    const size_t head =
        kDescBytes + ((size_t)L_max + 2 * (size_t)F_max) * 8 + (size_t)F_max * sizeof(LambdaFactors);
    return (head + 15) & ~size_t(15);
}
__host__ __device__ inline size_t batch_warp_bytes(uint32_t cap, uint32_t F_max, uint32_t L_max) {
    return batch_head_bytes(F_max, L_max) + half_bytes_per_warp(cap);
}

template <int MODE, int AP, int MINB>
__global__ void __launch_bounds__(256, MINB)
    fo2_batch_kernel(const DevModel* __restrict__ models, const uint64_t* __restrict__ offsets, uint32_t n_models,
                     uint32_t cap, uint32_t F_max, uint32_t L_max, double* const* __restrict__ Jout,
                     double* const* __restrict__ Lout, unsigned long long* __restrict__ tstamp,
                     uint32_t* __restrict__ done, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nw = blockDim.x >> 5;
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    unsigned char* base = smem + (size_t)w * batch_warp_bytes(cap, F_max, L_max);
    DevModel* desc = reinterpret_cast<DevModel*>(base);
    double* sl = reinterpret_cast<double*>(base + kDescBytes);
    double* Jacc = sl + L_max;
    double* Lacc = Jacc + F_max;
    LambdaFactors* LF = reinterpret_cast<LambdaFactors*>(Lacc + F_max);
    HalfSmem bk, fw;
    carve_halves(base + batch_head_bytes(F_max, L_max), cap, bk, fw);
    if (threadIdx.x == 0) atomicMin(&tstamp[2 * n_models], global_ns());

    const uint64_t n_items = offsets[n_models];
    const uint64_t stride = (uint64_t)gridDim.x * nw;
    uint32_t mi = 0, desc_mi = 0xffffffffu;
    for (uint64_t item = (uint64_t)blockIdx.x * nw + w; item < n_items; item += stride) {
        // model of this item: offsets is ascending and items only grow within a warp
        while (offsets[mi + 1] <= item) mi++;
        if (mi != desc_mi) {
            static_assert(sizeof(DevModel) % 8 == 0, "DevModel copied in 8-byte words");
            const unsigned long long* src = reinterpret_cast<const unsigned long long*>(models + mi);
            unsigned long long* dst = reinterpret_cast<unsigned long long*>(desc);
            for (uint32_t i = lane; i < sizeof(DevModel) / 8; i += 32) dst[i] = src[i];
            desc_mi = mi;
            __syncwarp();
        }
        const DevModel& m = *desc;
        const uint32_t o = (uint32_t)(item - offsets[mi]);
        if (lane == 0 && o == 0) tstamp[2 * mi] = global_ns();  // origins start in order
        for (uint32_t i = lane; i < m.L; i += 32) sl[i] = m.sorted_line[i];
        for (uint32_t f = lane; f < m.F; f += 32) {
            Jacc[f] = 0.0;
            Lacc[f] = 0.0;
        }
        bool ok = true;
        const bool want_lam = Lout[mi] != nullptr;
        __syncwarp();
        if (want_lam)  // ray-independent factors of the origin's ALO elements, once per origin
            for (uint32_t f = lane; f < m.F; f += 32)
                if (m.in_line[f]) LF[f] = lambda_factors(m, sl, o, f);
        __syncwarp();
        for (uint32_t rr = 0; rr < m.hnrays && ok; rr++) {
            // general geometry with shared rays (mgr_batch_create refuses the other kinds)
            int nb = 0, nf = 0;
            trace_pair<true, 0, 0>(m, o, rr, m.antipod[rr], cap, bk, fw, lane, status, nb, nf);
            if (nb < 0 || nf < 0) {  // status recorded by the trace
                ok = false;
                break;
            }
            const double w2 = ray_w(m, o, rr);
            for (uint32_t f0 = 0; f0 < m.F; f0 += 32) {
                const uint32_t f = f0 + lane;
                if (f < m.F) {
                    const LaneCtx c = lane_ctx(m, o, f);
                    const LaneResult r = solve_lane<MODE, AP>(m, sl, c, bk, nb, fw, nf);
                    Jacc[f] += r.u * 2.0 * w2;
                    // the frequency's ALO elements over the ray pairs in order
                    if (want_lam && r.solved && m.in_line[f]) Lacc[f] += lambda_element(LF[f], w2, r.Ldiag);
                    if (!isfinite(r.u)) atomicOr(status, ST_NONFINITE);
                }
            }
            __syncwarp();
        }
        if (ok) {
            double* J = Jout[mi] + (size_t)o * m.F;
            for (uint32_t f = lane; f < m.F; f += 32) J[f] = Jacc[f];
            if (want_lam)
                // line l: its quadrature points' sums, lane by lane, then across the lanes
                // (fo2_reduce_kernel's association)
                for (uint32_t l = 0; l < m.L; l++) {
                    const uint32_t* l2f = m.lq2f + (size_t)l * m.Q;
                    double s = 0.0;
                    for (uint32_t q0 = 0; q0 < m.Q; q0 += 32) {
                        const uint32_t q = q0 + lane;
                        const uint32_t f = q < m.Q ? l2f[q] : 0xffffffffu;
                        if (f == 0xffffffffu || !m.in_line[f]) continue;
                        s += Lacc[f];
                    }
#pragma unroll
                    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(FULL_MASK, s, off);
                    if (lane == 0) Lout[mi][(size_t)o * m.L + l] = s;
                }
        }
        __syncwarp();
        if (lane == 0) {
            __threadfence();
            const uint32_t P = m.P;
            if (atomicAdd(&done[mi], 1u) + 1 == P) tstamp[2 * mi + 1] = global_ns();
        }
    }
}

template <int MODE, int AP, int MINB>
static cudaError_t launch_batch_variant(MgrBatch* b) {
    const int nw = b->warps;
    const size_t smem = (size_t)nw * batch_warp_bytes(b->cap, b->F_max, b->L_max);
    auto kern = fo2_batch_kernel<MODE, AP, MINB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nw * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;  // the per-warp buffers do not fit
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    uint64_t grid = (uint64_t)sms * per_sm;
    const uint64_t need = (b->n_items + nw - 1) / nw;
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    count_launch();
    kern<<<(unsigned)grid, nw * 32, smem, b->stream>>>(b->d_models, b->d_offsets, (uint32_t)b->models.size(), b->cap,
                                                       b->F_max, b->L_max, b->d_J, b->d_lam, b->d_t, b->d_done,
                                                       b->status);
    return cudaGetLastError();
}

template <int MODE, int AP>
static cudaError_t launch_batch_minb(MgrBatch* b) {
    if (b->minb == 3) return launch_batch_variant<MODE, AP, 3>(b);
    if (b->minb == 4) return launch_batch_variant<MODE, AP, 4>(b);
    return launch_batch_variant<MODE, AP, 2>(b);
}

template <int MODE>
static cudaError_t launch_batch_approx(MgrBatch* b) {
    switch (b->approx) {
        case APPROX_ONELINE: return launch_batch_minb<MODE, APPROX_ONELINE>(b);
        case APPROX_CLOSELINES: return launch_batch_minb<MODE, APPROX_CLOSELINES>(b);
        default: return launch_batch_minb<MODE, APPROX_NONE>(b);
    }
}

static void batch_release(MgrBatch* b) {
    if (!b) return;
    DeviceScope on_device(b->device);
    cudaFree(b->d_models);
    cudaFree(b->d_offsets);
    cudaFree(b->d_J);
    cudaFree(b->d_lam);
    cudaFree(b->d_t);
    cudaFree(b->d_done);
    cudaFree(b->status);
    if (b->h_models) cudaFreeHost(b->h_models);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// Uploads the current device descriptions of the batch's models (line data and FP32
// scales change with mgr_model_set_line_data and the ALI loop).
static cudaError_t batch_sync_models(MgrBatch* b) {
    const size_t n = b->models.size();
    for (size_t i = 0; i < n; i++) {
        cudaError_t e = cudaStreamSynchronize(b->models[i]->stream);  // pending work on the model's own stream
        if (e != cudaSuccess) return e;
        b->h_models[i] = b->models[i]->dm;
    }
    return cudaMemcpyAsync(b->d_models, b->h_models, n * sizeof(DevModel), cudaMemcpyHostToDevice, b->stream);
}

static int batch_status(MgrBatch* b) {
    int st = 0;
    cudaError_t e = cudaMemcpyAsync(&st, b->status, sizeof(int), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->status, 0, sizeof(int), b->stream);
    if (e != cudaSuccess) return cuda_fail(e, "batch status");
    return decode_status(st);
}

}  // namespace mgr

using namespace mgr;

extern "C" {

int mgr_batch_create(MgrModel* const* models, uint32_t n_models, MgrBatch** out) {
    if (!models || !out || n_models == 0) {
        set_error("mgr_batch_create: null argument or empty batch");
        return MGR_ERR_ARGUMENT;
    }
    *out = nullptr;
    auto* b = new MgrBatch();
    b->models.assign(models, models + n_models);
    std::vector<uint64_t> offsets(n_models + 1, 0);
    for (uint32_t i = 0; i < n_models; i++) {
        MgrModel* m = models[i];
        if (!m) {
            delete b;
            set_error("mgr_batch_create: null model in the batch");
            return MGR_ERR_ARGUMENT;
        }
        if (i == 0) {
            b->device = m->device;
            b->approx = m->dm.approx;
        }
        if (m->device != b->device || m->dm.approx != b->approx) {
            delete b;
            set_error("mgr_batch_create: the models of a batch share the device and the line approximation");
            return MGR_ERR_ARGUMENT;
        }
        if (!m->line_disc) {
            delete b;
            set_error("mgr_batch_create: model " + std::to_string(i) + " has no line spectral discretisation");
            return MGR_ERR_UNSUPPORTED;
        }
        if (m->dm.sph || m->dm.adaptive) {
            delete b;
            set_error("mgr_batch_create: model " + std::to_string(i) +
                      " is spherically symmetric or has adaptive rays; batches take general-geometry models with "
                      "shared rays (solve such models with mgr_formal_solve_fo2)");
            return MGR_ERR_UNSUPPORTED;
        }
        b->cap = std::max(b->cap, m->half_cap);
        b->F_max = std::max(b->F_max, m->dm.F);
        b->L_max = std::max(b->L_max, m->dm.L);
        offsets[i + 1] = offsets[i] + m->dm.P;
    }
    b->n_items = offsets[n_models];
    DeviceScope on_device(b->device);
    cudaError_t e = on_device.error();
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_models, n_models * sizeof(DevModel));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_offsets, (n_models + 1) * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_J, n_models * sizeof(double*));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_lam, n_models * sizeof(double*));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_t, (2 * n_models + 1) * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_done, n_models * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->status, sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_models, n_models * sizeof(DevModel));
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_offsets, offsets.data(), (n_models + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(b->status, 0, sizeof(int));
    if (e != cudaSuccess) {
        batch_release(b);
        return cuda_fail(e, "batch set-up");
    }
    const size_t per_warp = batch_warp_bytes(b->cap, b->F_max, b->L_max);
    int max_smem = 0;
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device);
    while (b->warps > 1 && (size_t)b->warps * per_warp > (size_t)max_smem) b->warps /= 2;
    if ((size_t)b->warps * per_warp > (size_t)max_smem) {
        batch_release(b);
        set_error("mgr_batch_create: the longest ray of the batch does not fit one warp's shared memory");
        return MGR_ERR_CAPACITY;
    }
    *out = b;
    return MGR_OK;
}

void mgr_batch_free(MgrBatch* batch) { batch_release(batch); }

int mgr_batch_set_tuning(MgrBatch* batch, int min_blocks_per_sm, int warps_per_block) {
    MGR_MODEL_DEVICE(batch);
    if (!batch) {
        set_error("mgr_batch_set_tuning: null batch");
        return MGR_ERR_ARGUMENT;
    }
    if (min_blocks_per_sm != 0 && (min_blocks_per_sm < 2 || min_blocks_per_sm > 4)) {
        set_error("mgr_batch_set_tuning: min_blocks_per_sm must be 2, 3 or 4");
        return MGR_ERR_ARGUMENT;
    }
    if (warps_per_block < 0 || warps_per_block > 8) {
        set_error("mgr_batch_set_tuning: warps_per_block must be 1..8");
        return MGR_ERR_ARGUMENT;
    }
    if (warps_per_block) {
        int max_smem = 0;
        cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, batch->device);
        if ((size_t)warps_per_block * batch_warp_bytes(batch->cap, batch->F_max, batch->L_max) > (size_t)max_smem) {
            set_error("mgr_batch_set_tuning: that many warps do not fit in shared memory");
            return MGR_ERR_CAPACITY;
        }
        batch->warps = warps_per_block;
    }
    if (min_blocks_per_sm) batch->minb = min_blocks_per_sm;
    return MGR_OK;
}

int mgr_batch_formal_solve_fo2_device(MgrBatch* batch, int precision, double* const* J_dev,
                                      double* const* lambda_diag_dev) {
    MGR_MODEL_DEVICE(batch);
    if (!batch || !J_dev) {
        set_error("mgr_batch_formal_solve_fo2_device: null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) {
        set_error("mgr_batch_formal_solve_fo2_device: unknown precision mode");
        return MGR_ERR_ARGUMENT;
    }
    const size_t n = batch->models.size();
    std::vector<double*> lam(n, nullptr);
    for (size_t i = 0; i < n; i++) {
        if (!J_dev[i]) {
            set_error("mgr_batch_formal_solve_fo2_device: null J pointer for model " + std::to_string(i));
            return MGR_ERR_ARGUMENT;
        }
        if (lambda_diag_dev) lam[i] = lambda_diag_dev[i];
    }
    cudaError_t e = batch_sync_models(batch);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(batch->d_J, J_dev, n * sizeof(double*), cudaMemcpyHostToDevice, batch->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(batch->d_lam, lam.data(), n * sizeof(double*), cudaMemcpyHostToDevice, batch->stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(batch->d_t, 0xff, (2 * n + 1) * sizeof(unsigned long long), batch->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(batch->d_done, 0, n * sizeof(uint32_t), batch->stream);
    // the host vectors above are read by the copies: wait for them before returning
    if (e == cudaSuccess) e = cudaStreamSynchronize(batch->stream);
    if (e == cudaSuccess)
        e = (precision == MGR_PRECISION_SPLIT) ? launch_batch_approx<MODE_SPLIT>(batch)
                                               : launch_batch_approx<MODE_FP64>(batch);
    if (e != cudaSuccess) return cuda_fail(e, "batch formal solve launch");
    return MGR_OK;
}

int mgr_batch_formal_solve_fo2(MgrBatch* batch, int precision, double* const* J, double* const* lambda_diag) {
    MGR_MODEL_DEVICE(batch);
    if (!batch || !J) {
        set_error("mgr_batch_formal_solve_fo2: null argument");
        return MGR_ERR_ARGUMENT;
    }
    const size_t n = batch->models.size();
    std::vector<void*> bufs;
    std::vector<double*> Jd(n), Ld(n, nullptr);
    auto cleanup = [&]() {
        for (void* p : bufs) cudaFree(p);
    };
    for (size_t i = 0; i < n; i++) {
        const DevModel& m = batch->models[i]->dm;
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, (size_t)m.P * m.F * 8);
        if (e != cudaSuccess) {
            cleanup();
            return cuda_fail(e, "batch output allocation");
        }
        bufs.push_back(p);
        Jd[i] = static_cast<double*>(p);
        if (lambda_diag && lambda_diag[i]) {
            e = cudaMalloc(&p, (size_t)m.P * m.L * 8);
            if (e != cudaSuccess) {
                cleanup();
                return cuda_fail(e, "batch output allocation");
            }
            bufs.push_back(p);
            Ld[i] = static_cast<double*>(p);
        }
    }
    int rc = mgr_batch_formal_solve_fo2_device(batch, precision, Jd.data(), Ld.data());
    cudaError_t e = cudaSuccess;
    for (size_t i = 0; rc == MGR_OK && e == cudaSuccess && i < n; i++) {
        const DevModel& m = batch->models[i]->dm;
        if (J[i]) e = cudaMemcpyAsync(J[i], Jd[i], (size_t)m.P * m.F * 8, cudaMemcpyDeviceToHost, batch->stream);
        if (e == cudaSuccess && Ld[i])
            e = cudaMemcpyAsync(lambda_diag[i], Ld[i], (size_t)m.P * m.L * 8, cudaMemcpyDeviceToHost, batch->stream);
    }
    if (rc == MGR_OK && e != cudaSuccess) rc = cuda_fail(e, "batch result copy");
    if (rc == MGR_OK) rc = batch_status(batch);
    cudaStreamSynchronize(batch->stream);
    cleanup();
    return rc;
}

int mgr_batch_timings(MgrBatch* batch, double* start_ms, double* finish_ms) {
    MGR_MODEL_DEVICE(batch);
    if (!batch || !start_ms || !finish_ms) {
        set_error("mgr_batch_timings: null argument");
        return MGR_ERR_ARGUMENT;
    }
    const size_t n = batch->models.size();
    std::vector<unsigned long long> t(2 * n + 1);
    cudaError_t e = cudaMemcpyAsync(t.data(), batch->d_t, t.size() * sizeof(unsigned long long),
                                    cudaMemcpyDeviceToHost, batch->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(batch->stream);
    if (e != cudaSuccess) return cuda_fail(e, "batch timings");
    const unsigned long long t0 = t[2 * n];
    for (size_t i = 0; i < n; i++) {
        start_ms[i] = 1e-6 * (double)(long long)(t[2 * i] - t0);
        finish_ms[i] = 1e-6 * (double)(long long)(t[2 * i + 1] - t0);
    }
    return batch_status(batch);
}

void* mgr_batch_stream(MgrBatch* batch) { return batch ? (void*)batch->stream : nullptr; }

}  // extern "C"
