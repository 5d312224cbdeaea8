// Host-side internals shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/magritte_gb300.h"
#include "mgr_device.cuh"
#include "mgr_scale.h"

namespace mgr {
struct AliState;
}

namespace mgr {
// Ray-length classes of the formal solve (half-ray steps at most; the last is open).
constexpr int kLenClasses = 5;
constexpr uint32_t kLenClassBound[kLenClasses] = {32, 64, 128, 256, 0xffffffffu};
MGR_HD int len_class(uint32_t steps) {
    return steps <= 32 ? 0 : steps <= 64 ? 1 : steps <= 128 ? 2 : steps <= 256 ? 3 : 4;
}
}  // namespace mgr

struct MgrModel {
    int device = 0;
    cudaStream_t stream = nullptr;
    mgr::DevModel dm{};
    std::vector<void*> allocations;  // every device allocation owned by the model
    double* em = nullptr;
    double* op = nullptr;
    double* iw = nullptr;
    double* Sp = nullptr;
    double* crit = nullptr;
    float* em_f = nullptr;
    float* op_f = nullptr;
    float* iw_f = nullptr;
    float* Sp_f = nullptr;
    float* iw_lo = nullptr;          // [P][L] low part of the double-float inverse widths
    uint16_t* nint = nullptr;        // [E][L] interpolation counts
    uint16_t* nint_all = nullptr;    // [E] interpolation counts over all lines (imagers)
    // launch shape of the formal solve per precision: register budget variant (CTAs per
    // SM: 2, 3 or 4) and warps (ray pairs in flight) per CTA; a new model starts from the
    // shape last tuned on its device in this process (tuned_shape), else these defaults
    int fo2_minb_split = 4;
    int fo2_warps_split = 8;
    int fo2_minb_fp64 = 2;
    int fo2_warps_fp64 = 4;
    int sm_count = 1;                // multiprocessors of the model's device
    bool line_disc = true;           // frequencies form a line spectral discretisation
    bool inputs_replaced = false;    // velocities or frequencies replaced through a *_device setter
    int* status = nullptr;           // device status word
    mgr::LineScales scales;          // FP32 line-table scales (split precision)
    uint32_t half_cap = 0;           // longest half ray in base steps (0 = not sized yet)
    // ray-length classes of the formal solve: pair_class[o * hnrays + rr] is the class of
    // ray pair (o, rr) by its longer half (kLenClassBound), class_cap[c] the longest half
    // ray in class c (0: empty); each class is solved by its own launch, whose shared
    // memory holds that class's rays only
    uint8_t* pair_class = nullptr;
    uint32_t class_cap[mgr::kLenClasses] = {};
    size_t n_edges = 0;
    // scratch outputs for the host-buffer entry points
    double* J_scratch = nullptr;
    size_t J_scratch_bytes = 0;
    double* u_scratch = nullptr;
    size_t u_scratch_bytes = 0;
    double* lam_scratch = nullptr;
    size_t lam_scratch_bytes = 0;
    double* v_scratch = nullptr;  // v of the uv solve
    size_t v_scratch_bytes = 0;
    double* alo_scratch = nullptr;     // band elements of the host-buffer banded solve [P][L][hnrays][2K]
    size_t alo_scratch_bytes = 0;
    double* alo_nr_scratch = nullptr;  // their points (uint32 data in a double-sized allocation)
    size_t alo_nr_scratch_bytes = 0;
    // staging of u(rr, o, f) / L_diag(rr, o, f) between the two formal-solve stages
    double* work = nullptr;
    size_t work_bytes = 0;
    // J [P][F] and ALO diagonal [P][L] of the last formal solve (device), for Jeff
    const double* last_J = nullptr;
    const double* last_lam = nullptr;
    const double* last_Jlin = nullptr;  // line-integrated J [P][L] of the last memory-lean solve
    // band elements of the non-local ALO of the last formal solve (null when it had none)
    const double* last_alo_off = nullptr;
    const uint32_t* last_alo_nr = nullptr;
    // line-producing species and the ALI loop (mgr_ali.cu)
    mgr::AliState* ali = nullptr;
    // ray-pair shard of the ALI loop's formal solves and the sum over shards
    uint32_t shard_begin = 0;
    uint32_t shard_end = 0xffffffffu;
    mgr_reduce_fn shard_reduce = nullptr;
    void* shard_user = nullptr;
    bool shard_capturable = false;
    // per-lane elimination scratch of the image adjoint (mgr_adjoint.cu), kept between calls
    double* adj_scratch = nullptr;
    size_t adj_scratch_bytes = 0;
    // host copies for the image-plane set-up (mgr_image.cu)
    std::vector<double> host_pos;     // [P][3]
    std::vector<uint32_t> host_p2b;   // [P]
    std::vector<double> host_raydir;  // [nrays][3]
};

namespace mgr {

void set_error(const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

// Makes `device` the calling thread's current CUDA device for the lifetime of the
// object and restores the caller's device afterwards.  Every entry point that works
// on a model enters its device first: a process may drive several GPUs, and the
// model's stream, allocations and the staging array's address all belong to the
// device the model was created on.  device < 0 leaves the current device alone.
class DeviceScope {
  public:
    explicit DeviceScope(int device) {
        if (device < 0) return;
        if (cudaGetDevice(&prev_) != cudaSuccess) prev_ = -1;
        if (prev_ != device) {
            err_ = cudaSetDevice(device);
            restore_ = (err_ == cudaSuccess && prev_ >= 0);
        }
    }
    ~DeviceScope() {
        if (restore_) cudaSetDevice(prev_);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
    cudaError_t error() const { return err_; }

  private:
    int prev_ = -1;
    bool restore_ = false;
    cudaError_t err_ = cudaSuccess;
};

}  // namespace mgr

// First statement of an int-returning entry point taking a model (which may be null:
// the entry point's own argument check follows).
#define MGR_MODEL_DEVICE(mdl)                                                       \
    ::mgr::DeviceScope mgr_device_scope_((mdl) ? (mdl)->device : -1);              \
    if (mgr_device_scope_.error() != cudaSuccess)                                   \
    return ::mgr::cuda_fail(mgr_device_scope_.error(), "entering the model's device")

namespace mgr {
// Device status word (ST_* bits) -> MGR_* code with the error message set.
int decode_status(int st);
// FP32 line-table scales of split precision (powers of two) and the derived DevModel fields.
void set_line_scales(MgrModel* m, double Ke, double Ko);
void count_launch();

// Kernel launchers (mgr_fo2.cu).  All enqueue on model->stream.
// d_max_steps[0]: longest half ray; d_max_steps[1 + c]: longest half ray of class c
cudaError_t launch_size_rays(MgrModel* model, uint32_t* d_max_steps);
// Formal solve of origins [o_begin, o_end): J [P][F] and lam [P][L] rows of those
// origins, u [hnrays][P][F] (may be NULL).  Per-ray results are staged in `work`
// (sized by fo2_work_bytes for the same u / lam choice), in chunks of origins that fit.
// 6.5 GiB: the 64^3 benchmark model (6.2 GB of u and L_diag) in one chunk.
constexpr size_t kFo2WorkBudget = size_t(13) << 29;
size_t fo2_work_bytes(const MgrModel* model, uint32_t n_origins, bool stage_u, bool stage_ld);
// Ray pairs [rr_begin, rr_end) only (partial J / ALO sums, u must then be NULL).
// J may be NULL; Jlin [P][L] (may be NULL) receives the line-integrated J in the order
// of the memory-lean solve; anis [6][P][L] (may be NULL) the line-integrated J and
// anisotropy tensor elements of the anisotropic solve; v [hnrays][P][F] (may be NULL,
// needs u) the uv solve's v.
cudaError_t launch_fo2_range(MgrModel* model, int precision, uint32_t o_begin, uint32_t o_end, double* J, double* u,
                             double* lam, double* work, size_t work_bytes, uint32_t rr_begin = 0,
                             uint32_t rr_end = 0xffffffffu, double* Jlin = nullptr, double* anis = nullptr,
                             double* v = nullptr, double* alo_off = nullptr, uint32_t* alo_nr = nullptr);
cudaError_t launch_trace_export(MgrModel* model, uint32_t o, uint32_t rr, uint32_t l, uint32_t capacity,
                                uint32_t* d_meta, uint32_t* d_nr, uint32_t* d_ni, double* d_fac, double* d_shift,
                                double* d_dZ);
cudaError_t launch_line_tables(MgrModel* model);
cudaError_t launch_ray_lengths(MgrModel* model, uint32_t* d_max_len);
cudaError_t launch_ray_stats(MgrModel* model, unsigned long long* d_stats);
cudaError_t launch_trace_check(MgrModel* model, unsigned long long* d_stats);
cudaError_t launch_nint_table(MgrModel* model);
cudaError_t launch_hl_tables(MgrModel* model);  // trace filter tables (edge_hl, pos_hl)
cudaError_t launch_edge_pack(MgrModel* model, const double4_32a* pos, const uint32_t* nbr, uint64_t E,
                             double4_32a* edge);
// Fills the correctly rounded erff table (kErfBandCount floats) on `stream`.
cudaError_t fill_erf_band(float* table, cudaStream_t stream, int sm_count);
// The current device's erff table, created (cudaMalloc, one fill launch, synchronised)
// by the first call on each device and kept until the process exits.
cudaError_t erf_band_table(const float** out);

}  // namespace mgr
