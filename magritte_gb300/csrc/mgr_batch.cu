// Many-model batch of second-order Feautrier formal solves.
//
// Each model is an ordinary MgrModel (mgr_model_create); a batch collects their device
// descriptions into one device array.  The models are solved in waves: consecutive
// models whose staged per-ray results fit the batch's staging area (a few GiB; one
// wave for most batches) are solved by one persistent launch of fo2_multi_kernel and
// one launch of fo2_multi_reduce_kernel.
//   * fo2_multi_kernel: one warp per (model, origin, ray pair) item, lanes over
//     frequencies, the same trace and solve_lane code as the single-model fo2_kernel;
//     u and L_diag go to the model's slice of the staging area.  Items are ordered
//     model by model, origin by origin, and taken in a grid-stride loop, so short and
//     long rays and small and large models mix on every SM.
//   * fo2_multi_reduce_kernel: one CTA per (model, origin), the single-model
//     reduction's per-origin code (mgr_reduce.cuh): J and the ALO diagonal in the same
//     order as the model's own mgr_formal_solve_fo2, so every model's results are its
//     own solve's (bit for bit in split precision).
// Per model the kernels record, from the GPU's global timer, when its first item
// started and when its last origin was reduced (the per-model latency).
#include <algorithm>
#include <vector>

#include "mgr_internal.h"
#include "mgr_reduce.cuh"
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
    uint64_t* d_offsets = nullptr;         // [n + 1] first origin of each model (cumulative P)
    uint64_t* d_item_off = nullptr;        // [n + 1] first (origin, ray pair) item of each model
    uint64_t* d_stage_off = nullptr;       // [n + 1] first staging entry of each model (cumulative P R F)
    std::vector<uint64_t> item_off, stage_off, origin_off;  // host copies
    double* stage_u = nullptr;             // staging of u for one wave
    double* stage_ld = nullptr;            // staging of L_diag for one wave
    uint64_t stage_entries = 0;            // entries of each staging area
    double** d_J = nullptr;                // [n] output pointers
    double** d_lam = nullptr;              // [n]
    unsigned long long* d_t = nullptr;     // [n][2] first-start / last-finish ns, [2n] batch start
    uint32_t* d_done = nullptr;            // [n] reduced origins per model
    int* status = nullptr;
    mgr::DevModel* h_models = nullptr;     // pinned staging of the device descriptions
    int warps = 8;
    int minb = 4;
};

namespace mgr {

// Staged u (and L_diag) entries of one wave at most: 512 Mi doubles (4 GiB each) or,
// when larger, the biggest single model.
constexpr uint64_t kBatchStageEntries = uint64_t(1) << 29;

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The model of index i (an item or an origin) among models [m0, m1): offsets ascending.
__device__ __forceinline__ uint32_t model_of(const uint64_t* __restrict__ off, uint32_t m0, uint32_t m1, uint64_t i) {
    uint32_t lo = m0, hi = m1;  // off[lo] <= i < off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (off[mid] <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Per-warp shared memory of fo2_multi_kernel: the current model's DevModel and sorted
// line centres, then the two trace halves.  The single-model kernels take their
// DevModel as a kernel parameter, whose fields the instructions read from the constant
// bank; a batch kernel indexes its models at run time.  Read from the descriptor array
// in global memory, every table access waited on a dependent global load and the loaded
// pointers stayed live in registers; the warp copies its model's descriptor into shared
// memory when the model changes (measured faster than passing the wave's descriptors
// as a kernel parameter indexed by the model: 160 against 153 M solves/s).
constexpr size_t kDescBytes = (sizeof(DevModel) + 15) & ~size_t(15);
__host__ __device__ inline size_t batch_head_bytes(uint32_t L_max) {
    return (kDescBytes + (size_t)L_max * 8 + 15) & ~size_t(15);
}
__host__ __device__ inline size_t batch_warp_bytes(uint32_t cap, uint32_t L_max) {
    return batch_head_bytes(L_max) + half_bytes_per_warp(cap);
}

__device__ __forceinline__ void copy_desc(const DevModel* __restrict__ src, DevModel* dst, int t, int nt) {
    static_assert(sizeof(DevModel) % 8 == 0, "DevModel copied in 8-byte words");
    const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(dst);
    for (uint32_t i = (uint32_t)t; i < sizeof(DevModel) / 8; i += (uint32_t)nt) d[i] = s[i];
}

// Stage 1 of models [m0, m1): u (and L_diag) of every (model, origin, ray pair) item.
template <int MODE, int AP, int MINB>
__global__ void __launch_bounds__(256, MINB)
    fo2_multi_kernel(const DevModel* __restrict__ models, uint32_t m0, uint32_t m1,
                     const uint64_t* __restrict__ item_off, const uint64_t* __restrict__ stage_off, uint32_t cap,
                     uint32_t L_max, double* __restrict__ U, double* __restrict__ LD,
                     unsigned long long* __restrict__ tstamp, uint32_t n_models, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nw = blockDim.x >> 5;
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    unsigned char* base = smem + (size_t)w * batch_warp_bytes(cap, L_max);
    DevModel* desc = reinterpret_cast<DevModel*>(base);
    double* sl = reinterpret_cast<double*>(base + kDescBytes);
    HalfSmem bk, fw;
    carve_halves(base + batch_head_bytes(L_max), cap, bk, fw);
    if (threadIdx.x == 0) atomicMin(&tstamp[2 * n_models], global_ns());

    const uint64_t i0 = item_off[m0], i1 = item_off[m1];
    const uint64_t s0 = stage_off[m0];
    const uint64_t stride = (uint64_t)gridDim.x * nw;
    uint32_t mi = m0, desc_mi = 0xffffffffu;
    for (uint64_t item = i0 + (uint64_t)blockIdx.x * nw + w; item < i1; item += stride) {
        // the item's model: items only grow within a warp
        while (item_off[mi + 1] <= item) mi++;
        if (mi != desc_mi) {
            copy_desc(models + mi, desc, lane, 32);
            __syncwarp();
            for (uint32_t i = lane; i < desc->L; i += 32) sl[i] = desc->sorted_line[i];
            desc_mi = mi;
            __syncwarp();
        }
        const DevModel& m = *desc;
        const uint64_t k = item - item_off[mi];
        const uint32_t o = (uint32_t)(k / m.hnrays);
        const uint32_t rr = (uint32_t)(k % m.hnrays);
        if (k == 0 && lane == 0) tstamp[2 * mi] = global_ns();
        // general geometry with shared rays (mgr_batch_create refuses the other kinds)
        int nb = 0, nf = 0;
        trace_pair<true, 0, 0>(m, o, rr, m.antipod[rr], cap, bk, fw, lane, status, nb, nf);
        if (nb < 0 || nf < 0) continue;  // status recorded by the trace
        const size_t at = (size_t)(stage_off[mi] - s0) + ((size_t)rr * m.P + o) * m.F;
        double* Ui = U + at;
        double* Li = LD ? LD + at : nullptr;
        for (uint32_t f0 = 0; f0 < m.F; f0 += 32) {
            const uint32_t f = f0 + lane;
            if (f < m.F) {
                const LaneCtx c = lane_ctx(m, o, f);
                const LaneResult r = solve_lane<MODE, AP>(m, sl, c, bk, nb, fw, nf);
                Ui[f] = r.u;
                if (Li) Li[f] = r.solved ? r.Ldiag : 0.0;
                if (!isfinite(r.u)) atomicOr(status, ST_NONFINITE);
            }
        }
        __syncwarp();
    }
}

// Stage 2 of models [m0, m1): J and the ALO diagonal of every (model, origin), one CTA
// per origin, in the single-model reduction's order.  The CTA copies its model's
// descriptor into shared memory when the model changes.
__global__ void __launch_bounds__(128)
    fo2_multi_reduce_kernel(const DevModel* __restrict__ models, uint32_t m0, uint32_t m1,
                            const uint64_t* __restrict__ origin_off, const uint64_t* __restrict__ stage_off,
                            const double* __restrict__ U, const double* __restrict__ LD,
                            double* const* __restrict__ Jout, double* const* __restrict__ Lout,
                            unsigned long long* __restrict__ tstamp, uint32_t* __restrict__ done) {
    __shared__ __align__(16) unsigned char dbuf[kDescBytes];
    DevModel* desc = reinterpret_cast<DevModel*>(dbuf);
    const int nw = blockDim.x >> 5;
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint64_t g0 = origin_off[m0], g1 = origin_off[m1];
    const uint64_t s0 = stage_off[m0];
    uint32_t desc_mi = 0xffffffffu;
    for (uint64_t g = g0 + blockIdx.x; g < g1; g += gridDim.x) {
        const uint32_t mi = model_of(origin_off, m0, m1, g);
        if (mi != desc_mi) {
            __syncthreads();  // every thread is done with the previous model's descriptor
            copy_desc(models + mi, desc, threadIdx.x, blockDim.x);
            desc_mi = mi;
            __syncthreads();
        }
        const DevModel& m = *desc;
        const uint32_t o = (uint32_t)(g - origin_off[mi]);
        const double* Um = U + (stage_off[mi] - s0);
        const size_t stride = (size_t)m.P * m.F;
        reduce_J_origin(m, o, 0, m.hnrays, Um, stride, 0, Jout[mi], threadIdx.x, blockDim.x);
        if (LD && Lout[mi])
            reduce_lam_origin(m, o, 0, m.hnrays, LD + (stage_off[mi] - s0), stride, 0, Lout[mi], w, nw, lane);
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(&done[mi], 1u) + 1 == m.P) tstamp[2 * mi + 1] = global_ns();
        }
    }
}

template <int MODE, int AP, int MINB>
static cudaError_t launch_multi_variant(MgrBatch* b, uint32_t m0, uint32_t m1, bool want_lam) {
    const int nw = b->warps;
    const size_t smem = (size_t)nw * batch_warp_bytes(b->cap, b->L_max);
    auto kern = fo2_multi_kernel<MODE, AP, MINB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nw * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;  // the per-warp buffers do not fit
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    const uint64_t items = b->item_off[m1] - b->item_off[m0];
    uint64_t grid = (uint64_t)sms * per_sm;
    const uint64_t need = (items + nw - 1) / nw;
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    const uint32_t n = (uint32_t)b->models.size();
    count_launch();
    kern<<<(unsigned)grid, nw * 32, smem, b->stream>>>(b->d_models, m0, m1, b->d_item_off, b->d_stage_off, b->cap,
                                                       b->L_max, b->stage_u, want_lam ? b->stage_ld : nullptr,
                                                       b->d_t, n, b->status);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const uint64_t origins = b->origin_off[m1] - b->origin_off[m0];
    uint64_t rgrid = (uint64_t)sms * 16;
    if (rgrid > origins) rgrid = origins;
    if (rgrid < 1) rgrid = 1;
    count_launch();
    fo2_multi_reduce_kernel<<<(unsigned)rgrid, 128, 0, b->stream>>>(b->d_models, m0, m1, b->d_offsets,
                                                                    b->d_stage_off, b->stage_u,
                                                                    want_lam ? b->stage_ld : nullptr, b->d_J,
                                                                    b->d_lam, b->d_t, b->d_done);
    return cudaGetLastError();
}

// Every wave of the batch: consecutive models whose staging fits the staging area.
template <int MODE, int AP, int MINB>
static cudaError_t launch_batch_variant(MgrBatch* b, bool want_lam) {
    const uint32_t n = (uint32_t)b->models.size();
    uint32_t m0 = 0;
    while (m0 < n) {
        uint32_t m1 = m0 + 1;
        while (m1 < n && b->stage_off[m1 + 1] - b->stage_off[m0] <= b->stage_entries) m1++;
        cudaError_t e = launch_multi_variant<MODE, AP, MINB>(b, m0, m1, want_lam);
        if (e != cudaSuccess) return e;
        m0 = m1;
    }
    return cudaSuccess;
}

template <int MODE, int AP>
static cudaError_t launch_batch_minb(MgrBatch* b, bool want_lam) {
    if (b->minb == 3) return launch_batch_variant<MODE, AP, 3>(b, want_lam);
    if (b->minb == 2) return launch_batch_variant<MODE, AP, 2>(b, want_lam);
    return launch_batch_variant<MODE, AP, 4>(b, want_lam);
}

template <int MODE>
static cudaError_t launch_batch_approx(MgrBatch* b, bool want_lam) {
    switch (b->approx) {
        case APPROX_ONELINE: return launch_batch_minb<MODE, APPROX_ONELINE>(b, want_lam);
        case APPROX_CLOSELINES: return launch_batch_minb<MODE, APPROX_CLOSELINES>(b, want_lam);
        default: return launch_batch_minb<MODE, APPROX_NONE>(b, want_lam);
    }
}

static void batch_release(MgrBatch* b) {
    if (!b) return;
    DeviceScope on_device(b->device);
    cudaFree(b->d_models);
    cudaFree(b->d_offsets);
    cudaFree(b->d_item_off);
    cudaFree(b->d_stage_off);
    cudaFree(b->stage_u);
    cudaFree(b->stage_ld);
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
    std::vector<uint64_t> offsets(n_models + 1, 0), item_off(n_models + 1, 0), stage_off(n_models + 1, 0);
    uint64_t largest = 1;
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
        item_off[i + 1] = item_off[i] + (uint64_t)m->dm.P * m->dm.hnrays;
        const uint64_t entries = (uint64_t)m->dm.P * m->dm.hnrays * m->dm.F;
        stage_off[i + 1] = stage_off[i] + entries;
        largest = std::max(largest, entries);
    }
    b->n_items = offsets[n_models];
    b->origin_off = offsets;
    b->item_off = item_off;
    b->stage_off = stage_off;
    b->stage_entries = std::min(stage_off[n_models], std::max(kBatchStageEntries, largest));
    DeviceScope on_device(b->device);
    cudaError_t e = on_device.error();
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_models, n_models * sizeof(DevModel));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_offsets, (n_models + 1) * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_item_off, (n_models + 1) * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_stage_off, (n_models + 1) * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->stage_u, b->stage_entries * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&b->stage_ld, b->stage_entries * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_J, n_models * sizeof(double*));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_lam, n_models * sizeof(double*));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_t, (2 * n_models + 1) * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_done, n_models * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->status, sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_models, n_models * sizeof(DevModel));
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_offsets, offsets.data(), (n_models + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_item_off, item_off.data(), (n_models + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_stage_off, stage_off.data(), (n_models + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(b->status, 0, sizeof(int));
    if (e != cudaSuccess) {
        batch_release(b);
        return cuda_fail(e, "batch set-up");
    }
    const size_t per_warp = batch_warp_bytes(b->cap, b->L_max);
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
        if ((size_t)warps_per_block * batch_warp_bytes(batch->cap, batch->L_max) > (size_t)max_smem) {
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
    bool want_lam = false;
    for (size_t i = 0; i < n; i++) {
        if (!J_dev[i]) {
            set_error("mgr_batch_formal_solve_fo2_device: null J pointer for model " + std::to_string(i));
            return MGR_ERR_ARGUMENT;
        }
        if (lambda_diag_dev) lam[i] = lambda_diag_dev[i];
        want_lam = want_lam || lam[i] != nullptr;
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
        e = (precision == MGR_PRECISION_SPLIT) ? launch_batch_approx<MODE_SPLIT>(batch, want_lam)
                                               : launch_batch_approx<MODE_FP64>(batch, want_lam);
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
