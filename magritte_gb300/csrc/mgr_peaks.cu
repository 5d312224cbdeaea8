// Pipe-rate probes of the current device for the benchmark's FP64 roofline.
//
// The formal-solve kernels are bound by the FP64 pipe, not by HBM: GB300 executes
// FP64 arithmetic at a small fraction of its FP32 rate, so the denominator of their
// roofline is the measured rate of the FP64 instructions they issue.  Each probe kernel
// runs eight independent dependency chains of one instruction kind per thread over a
// full-occupancy grid (SMs x 8 CTAs of 256 threads); the rate is counted in thread
// operations (one lane executing one instruction).
//
// Kinds: 0 DFMA, 1 DADD, 2 DMUL, 3 DSETP (FP64 compare), 4 F2F (FP64 <-> FP32
// conversions, two per step), 5 MUFU.RCP64H (rcp.approx.ftz.f64).
#include <algorithm>
#include <vector>

#include "mgr_internal.h"

namespace mgr {

constexpr int kProbeChains = 8;
constexpr int kProbeThreads = 256;

// cycles[3 * block] = {SM id, clock64 at the start, clock64 at the end} of each CTA.
template <int KIND>
__global__ void __launch_bounds__(kProbeThreads) pipe_probe_kernel(double* __restrict__ out,
                                                                   unsigned long long* __restrict__ cycles,
                                                                   uint32_t iters, double a, double b) {
    double x[kProbeChains];
#pragma unroll
    for (int i = 0; i < kProbeChains; i++) x[i] = b + (double)(threadIdx.x * kProbeChains + i);
    uint32_t cnt = 0;
    __syncthreads();
    const unsigned long long t0 = clock64();
    for (uint32_t it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < kProbeChains; i++) {
            if constexpr (KIND == 0) {
                x[i] = fma(x[i], a, b);
            } else if constexpr (KIND == 1) {
                x[i] = x[i] + b;
            } else if constexpr (KIND == 2) {
                x[i] = x[i] * a;
            } else if constexpr (KIND == 3) {
                cnt += (x[i] < b) ? 1u : 0u;
                x[i] = __longlong_as_double(__double_as_longlong(x[i]) + 1);  // integer pipe
            } else if constexpr (KIND == 4) {
                // FP64 -> FP32 -> FP64 through explicit conversion instructions (a C++
                // cast chain would be folded to FP32 arithmetic)
                float f;
                asm volatile("cvt.rn.f32.f64 %0, %1;" : "=f"(f) : "d"(x[i]));
                asm volatile("cvt.f64.f32 %0, %1;" : "=d"(x[i]) : "f"(f));
            } else {
                asm volatile("rcp.approx.ftz.f64 %0, %1;" : "=d"(x[i]) : "d"(x[i]));
            }
        }
    }
    __syncthreads();
    const unsigned long long t1 = clock64();
    double s = (double)cnt;
#pragma unroll
    for (int i = 0; i < kProbeChains; i++) s += x[i];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
    if (threadIdx.x == 0) {
        uint32_t smid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        cycles[3 * blockIdx.x] = smid;
        cycles[3 * blockIdx.x + 1] = t0;
        cycles[3 * blockIdx.x + 2] = t1;
    }
}

template <int KIND>
static cudaError_t launch_probe(cudaStream_t s, int grid, double* out, unsigned long long* cyc, uint32_t iters) {
    count_launch();
    pipe_probe_kernel<KIND><<<grid, kProbeThreads, 0, s>>>(out, cyc, iters, 1.0000000001, 1.0e-3);
    return cudaGetLastError();
}

static cudaError_t launch_probe_kind(int kind, cudaStream_t s, int grid, double* out, unsigned long long* cyc,
                                     uint32_t iters) {
    switch (kind) {
        case 0: return launch_probe<0>(s, grid, out, cyc, iters);
        case 1: return launch_probe<1>(s, grid, out, cyc, iters);
        case 2: return launch_probe<2>(s, grid, out, cyc, iters);
        case 3: return launch_probe<3>(s, grid, out, cyc, iters);
        case 4: return launch_probe<4>(s, grid, out, cyc, iters);
        default: return launch_probe<5>(s, grid, out, cyc, iters);
    }
}

}  // namespace mgr

using namespace mgr;

extern "C" int mgr_measure_pipe_rate(int kind, uint32_t iterations, double* thread_ops_per_s,
                                     double* thread_ops_per_clk_per_sm, float* ms) {
    if (kind < 0 || kind > 5 || iterations == 0) {
        set_error("mgr_measure_pipe_rate: kind must be 0..5 and iterations > 0");
        return MGR_ERR_ARGUMENT;
    }
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(e, "device query");
    const int grid = nsm * 8;  // 2048 threads per SM
    double* out = nullptr;
    unsigned long long* cyc = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    e = cudaMalloc(&out, (size_t)grid * kProbeThreads * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&cyc, (size_t)grid * 3 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float best = 0.0f;
    double best_cyc = 0.0;
    for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {  // rep 0 warms up
        e = cudaEventRecord(e0, s);
        if (e == cudaSuccess) e = launch_probe_kind(kind, s, grid, out, cyc, iterations);
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float t = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
        std::vector<unsigned long long> c((size_t)grid * 3);
        if (e == cudaSuccess)
            e = cudaMemcpy(c.data(), cyc, c.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && rep > 0 && (best == 0.0f || t < best)) {
            best = t;
            // per SM: first CTA start to last CTA end on that SM's own clock
            std::vector<unsigned long long> lo(nsm, ~0ull), hi(nsm, 0ull);
            for (int b = 0; b < grid; b++) {
                const unsigned long long sm = c[3 * b];
                if (sm >= (unsigned long long)nsm) continue;
                lo[sm] = std::min(lo[sm], c[3 * b + 1]);
                hi[sm] = std::max(hi[sm], c[3 * b + 2]);
            }
            double span = 0.0;
            int used = 0;
            for (int k = 0; k < nsm; k++)
                if (hi[k] > lo[k]) {
                    span += (double)(hi[k] - lo[k]);
                    used++;
                }
            best_cyc = used ? span / used : 0.0;
        }
    }
    if (out) cudaFree(out);
    if (cyc) cudaFree(cyc);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (e != cudaSuccess) return cuda_fail(e, "pipe probe");
    const double per_step = (kind == 4) ? 2.0 : 1.0;
    const double ops = (double)grid * kProbeThreads * kProbeChains * (double)iterations * per_step;
    if (thread_ops_per_s) *thread_ops_per_s = ops / (best * 1e-3);
    if (thread_ops_per_clk_per_sm) *thread_ops_per_clk_per_sm = best_cyc > 0.0 ? (ops / nsm) / best_cyc : 0.0;
    if (ms) *ms = best;
    return MGR_OK;
}
