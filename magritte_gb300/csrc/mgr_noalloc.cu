// mgr_formal_solve_fo2_device_noalloc: the device-pointer formal solve with its
// per-ray staging in a fixed, file-scope device array instead of model-owned
// cudaMalloc'd scratch.  The call itself allocates nothing: no cudaMalloc, no
// cudaFree, no library call that allocates.
//
// Staging area.  g_fo2_stage holds u(rr, o, f) (when the caller passes no u buffer)
// and L_diag(rr, o, f) (when the ALO is wanted) for one chunk of origins at a time:
// kStageBytes / (hnrays * nfreqs * 8 * k) origins per chunk, k = number of staged
// arrays.  Every staged value is written by the first stage before the second stage
// reads it within the same chunk, so nothing in the area has to start at zero (a
// trace failure is reported through the model's status word and leaves the outputs
// of the failed origins undefined, as in mgr_formal_solve_fo2_device).
//
// Sharing.  There is one area per device, shared by every model on that device.
// Calls whose work overlaps in time (two host threads, or two models' streams that
// run concurrently) race on it; callers serialise them.
#include <mutex>

#include "mgr_internal.h"

namespace {

constexpr size_t kStageBytes = size_t(64) << 20;  // 64 MiB per device
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_fo2_stage[kStageBytes / sizeof(double)];

std::mutex g_stage_mutex;
double* g_stage_ptr[kMaxDevices] = {};

// Device address of g_fo2_stage on `device`, looked up once per device.
cudaError_t stage_address(int device, double** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_stage_mutex);
    if (!g_stage_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_fo2_stage);
        if (e != cudaSuccess) return e;
        g_stage_ptr[device] = static_cast<double*>(p);
    }
    *out = g_stage_ptr[device];
    return cudaSuccess;
}

}  // namespace

using namespace mgr;

extern "C" int mgr_formal_solve_fo2_device_noalloc(MgrModel* model, int precision, double* J_dev, double* u_dev,
                                                   double* lambda_diag_dev) {
    // The model's device is current from here on, so the staging array's address
    // looked up below is the one on that device.
    MGR_MODEL_DEVICE(model);
    if (!model || !J_dev) {
        set_error("mgr_formal_solve_fo2_device_noalloc: null argument");
        return MGR_ERR_ARGUMENT;
    }
    if (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) {
        set_error("mgr_formal_solve_fo2_device_noalloc: unknown precision mode");
        return MGR_ERR_ARGUMENT;
    }
    if (!model->line_disc) {
        // frequencies of an imaging discretisation have no (line, quadrature point)
        // map, which the ALO and the per-line tables of the solve index
        set_error("mgr_formal_solve_fo2_device_noalloc: the formal solve needs a line spectral discretisation "
                  "(nfreqs = nlines*nquads with every frequency mapped to its line)");
        return MGR_ERR_UNSUPPORTED;
    }
    const int k = (u_dev ? 0 : 1) + (lambda_diag_dev ? 1 : 0);
    const size_t per_origin = (size_t)model->dm.hnrays * model->dm.F * sizeof(double) * k;
    if (per_origin > kStageBytes) {
        set_error("mgr_formal_solve_fo2_device_noalloc: one origin needs " + std::to_string(per_origin) +
                  " bytes of staging (hnrays * nfreqs * 8 per staged array), above the fixed " +
                  std::to_string(kStageBytes) + "-byte area; use mgr_formal_solve_fo2_device");
        return MGR_ERR_CAPACITY;
    }
    double* stage = nullptr;
    cudaError_t e = stage_address(model->device, &stage);
    if (e != cudaSuccess) return cuda_fail(e, "staging area address");
    e = launch_fo2_range(model, precision, 0, model->dm.P, J_dev, u_dev, lambda_diag_dev, stage, kStageBytes);
    if (e != cudaSuccess) return cuda_fail(e, "formal solve launch");
    // the caller's J and ALO buffers are this model's latest formal-solve results,
    // which mgr_compute_jeff reads
    model->last_J = J_dev;
    model->last_lam = lambda_diag_dev;
    model->last_alo_off = nullptr;
    model->last_alo_nr = nullptr;
    return MGR_OK;
}
