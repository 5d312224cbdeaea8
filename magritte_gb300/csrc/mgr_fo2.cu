// Kernels of the formal-solve path and their launchers.
#include "mgr_internal.h"
#include "mgr_reduce.cuh"
#include "mgr_solve.cuh"

namespace mgr {

// ---------------------------------------------------------------------------------
// Per-(point, line) tables: the source quotient emissivity/opacity the reference
// recomputes per call (solver.tpp:1901-1908) and FP32 copies for split precision.
// FP32 copies of positive values below the smallest normal float are raised to it
// (the reference's 1e-50 emissivity floor is not representable in FP32).
// ---------------------------------------------------------------------------------
__device__ __forceinline__ float to_f32_floor(double x) {
    const float f = (float)x;
    return (x > 0.0 && f < FLT_MIN) ? FLT_MIN : f;
}

__global__ void line_tables_kernel(const double* __restrict__ em, const double* __restrict__ op,
                                   const double* __restrict__ iw, double* __restrict__ Sp, float* __restrict__ em_f,
                                   float* __restrict__ op_f, float* __restrict__ iw_f, float* __restrict__ Sp_f,
                                   float* __restrict__ iw_lo, size_t n, double Ke, double Ko) {
    const double KeKo = Ke / Ko;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double e = em[i], o = op[i];
        const double s = e / o;
        Sp[i] = s;
        em_f[i] = to_f32_floor(e * Ke);
        op_f[i] = to_f32_floor(o * Ko);
        const float w = (float)iw[i];
        iw_f[i] = w;
        iw_lo[i] = (float)(iw[i] - (double)w);
        Sp_f[i] = to_f32_floor(s * KeKo);
    }
}

// ---------------------------------------------------------------------------------
// Correctly rounded erff table of split precision's same-wing erf differences:
// (float)erf((double)x) for every float x in [kErfBandLo, 3.919206).
// ---------------------------------------------------------------------------------
__global__ void erf_band_kernel(float* __restrict__ t) {
    const uint32_t base = __float_as_uint(kErfBandLo);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < kErfBandCount; i += gridDim.x * blockDim.x)
        t[i] = (float)erf((double)__uint_as_float(base + i));
}

cudaError_t fill_erf_band(float* table, cudaStream_t stream, int sm_count) {
    count_launch();
    erf_band_kernel<<<sm_count * 8, 256, 0, stream>>>(table);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// Neighbour records: edge[i] = position of neighbour nbr[i] with its index in the bits
// of w (one 32-byte load per neighbour in the trace), packed from the uploaded points.
// ---------------------------------------------------------------------------------
__global__ void edge_pack_kernel(const double4_32a* __restrict__ pos, const uint32_t* __restrict__ nbr, uint64_t E,
                                 double4_32a* __restrict__ edge) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < E; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t n = nbr[i];
        double4_32a e = pos[n];
        e.w = __longlong_as_double((long long)n);
        edge[i] = e;
    }
}

cudaError_t launch_edge_pack(MgrModel* model, const double4_32a* pos, const uint32_t* nbr, uint64_t E,
                             double4_32a* edge) {
    if (E == 0) return cudaSuccess;
    uint64_t blocks = (E + 255) / 256;
    if (blocks > (uint64_t)model->sm_count * 16) blocks = (uint64_t)model->sm_count * 16;
    count_launch();
    edge_pack_kernel<<<(unsigned)blocks, 256, 0, model->stream>>>(pos, nbr, E, edge);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// Hi/lo float copies of the neighbour records and points for the trace's FP32
// next-point filter (DevModel::edge_hl, pos_hl), positions scaled by pos_scale.
// ---------------------------------------------------------------------------------
__global__ void hl_tables_kernel(const double4_32a* __restrict__ edge, uint64_t E, const double4_32a* __restrict__ pos,
                                 uint32_t P, double scale, float4* __restrict__ edge_hl, float4* __restrict__ pos_hl) {
    const uint64_t n = E + P;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const bool is_edge = i < E;
        const double4_32a q = is_edge ? edge[i] : pos[i - E];
        float4 hi, lo;
        split_hl(dmul_rn(q.x, scale), hi.x, lo.x);
        split_hl(dmul_rn(q.y, scale), hi.y, lo.y);
        split_hl(dmul_rn(q.z, scale), hi.z, lo.z);
        hi.w = is_edge ? bits_f32((uint32_t)__double_as_longlong(q.w)) : 0.0f;
        lo.w = 0.0f;
        if (is_edge && !edge_hl) continue;
        float4* out = is_edge ? edge_hl + 2 * i : pos_hl + 2 * (i - E);
        out[0] = hi;
        out[1] = lo;
    }
}

cudaError_t launch_hl_tables(MgrModel* model) {
    const uint64_t n = (uint64_t)model->n_edges + model->dm.P;
    uint64_t blocks = (n + 255) / 256;
    if (blocks > (uint64_t)model->sm_count * 16) blocks = (uint64_t)model->sm_count * 16;
    count_launch();
    hl_tables_kernel<<<(unsigned)(blocks ? blocks : 1), 256, 0, model->stream>>>(
        model->dm.edge, model->n_edges, model->dm.pos, model->dm.P, model->dm.pos_scale,
        const_cast<float4*>(model->dm.edge_hl), const_cast<float4*>(model->dm.pos_hl));
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// Ray sizing: one warp per (point, ray pair) walks both halves; the longer half's step
// count gives the pair's length class (pair_class) and feeds the maxima of the class
// and of all rays (d_max[1 + c], d_max[0]), which size the shared-memory ray buffers.
// ---------------------------------------------------------------------------------
__global__ void size_rays_kernel(DevModel m, uint8_t* __restrict__ pair_class, uint32_t* d_max, int* status) {
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const uint64_t total = (uint64_t)m.P * m.hnrays;
    if (gw >= total) return;
    const uint32_t o = (uint32_t)(gw / m.hnrays);
    const uint32_t rr = (uint32_t)(gw % m.hnrays);
    HalfSmem h{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    const int nb = trace_half<false>(m, o, rr, 0xffffffffu, h, lane, status);
    const int nf = trace_half<false>(m, o, m.antipod[rr], 0xffffffffu, h, lane, status);
    if (lane != 0 || nb < 0 || nf < 0) return;
    const uint32_t n = (uint32_t)(nb > nf ? nb : nf);
    const int c = len_class(n);
    pair_class[gw] = (uint8_t)c;
    if (n > 0) atomicMax(d_max, n);
    atomicMax(d_max + 1 + c, n > 0 ? n : 1u);  // a class with pairs is never empty
}

// ---------------------------------------------------------------------------------
// Interpolation count of every CSR edge (crt -> nxt) and line:
// InterpHelper::get_n_interp_for_line (solver_interp_helper.tpp:55-75), evaluated
// once per edge instead of once per step, lane and frequency.
// ---------------------------------------------------------------------------------
// Spherical models (trace_half_sph) index the tables by sph_eid instead: three slots per
// point for the steps p -> p, p -> p - 1 and p -> p + 1.
__global__ void nint_table_kernel(DevModel m, uint16_t* __restrict__ nint, int* status) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (uint64_t)m.P * m.L;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t p = (uint32_t)(i / m.L), l = (uint32_t)(i % m.L);
        if (m.sph) {
            for (uint32_t k = 0; k < 3; k++) {
                const uint32_t nxt = sph_slot_point(p, k);
                uint32_t v = (nxt < m.P) ? n_interp_for_line(m, l, p, nxt) : 1u;
                if (v > 0xffffu) {
                    atomicOr(status, ST_CAPACITY);
                    v = 0xffffu;
                }
                nint[(size_t)(3u * p + k) * m.L + l] = (uint16_t)v;
            }
            continue;
        }
        const uint32_t cum = m.cum_nb[p], n = m.n_nb[p];
        for (uint32_t k = 0; k < n; k++) {
            const uint32_t nxt = (uint32_t)__double_as_longlong(m.edge[cum + k].w);
            uint32_t v = n_interp_for_line(m, l, p, nxt);
            if (v > 0xffffu) {
                atomicOr(status, ST_CAPACITY);
                v = 0xffffu;
            }
            nint[(size_t)(cum + k) * m.L + l] = (uint16_t)v;
        }
    }
}

// The same over all lines (InterpHelper::get_n_interp, solver_interp_helper.tpp:10-46),
// for the imagers' Solver::set_data.
__global__ void nint_all_kernel(DevModel m, uint16_t* __restrict__ nint_all, int* status) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < m.P; p += gridDim.x * blockDim.x) {
        if (m.sph) {
            for (uint32_t k = 0; k < 3; k++) {
                const uint32_t nxt = sph_slot_point(p, k);
                uint32_t v = (nxt < m.P) ? n_interp_all_lines(m, p, nxt) : 1u;
                if (v > 0xffffu) {
                    atomicOr(status, ST_CAPACITY);
                    v = 0xffffu;
                }
                nint_all[3u * p + k] = (uint16_t)v;
            }
            continue;
        }
        const uint32_t cum = m.cum_nb[p], n = m.n_nb[p];
        for (uint32_t k = 0; k < n; k++) {
            const uint32_t nxt = (uint32_t)__double_as_longlong(m.edge[cum + k].w);
            uint32_t v = n_interp_all_lines(m, p, nxt);
            if (v > 0xffffu) {
                atomicOr(status, ST_CAPACITY);
                v = 0xffffu;
            }
            nint_all[cum + k] = (uint16_t)v;
        }
    }
}

cudaError_t launch_nint_table(MgrModel* model) {
    const uint64_t n = (uint64_t)model->dm.P * model->dm.L;
    const int threads = 256;
    uint64_t blocks = (n + threads - 1) / threads;
    if (blocks > 152 * 32) blocks = 152 * 32;
    count_launch();
    nint_table_kernel<<<(unsigned)(blocks ? blocks : 1), threads, 0, model->stream>>>(model->dm, model->nint,
                                                                                       model->status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    count_launch();
    const uint64_t pb = ((uint64_t)model->dm.P + threads - 1) / threads;
    nint_all_kernel<<<(unsigned)(pb < 152 * 32 ? (pb ? pb : 1) : 152 * 32), threads, 0, model->stream>>>(
        model->dm, model->nint_all, model->status);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// Reference ray-pair length (Solver::get_ray_lengths_max, solver.tpp:79-126):
// elements of both halves with get_n_interp over all lines.
// ---------------------------------------------------------------------------------
__global__ void ray_lengths_kernel(DevModel m, uint32_t cap, uint32_t* d_max, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t gw = (uint64_t)blockIdx.x * (blockDim.x >> 5) + w;
    if (gw >= (uint64_t)m.P * m.hnrays) return;
    HalfSmem bk, fw;
    carve_halves(smem + (size_t)w * half_bytes_per_warp(cap), cap, bk, fw);
    const uint32_t o = (uint32_t)(gw / m.hnrays);
    const uint32_t rr = (uint32_t)(gw % m.hnrays);
    int nb = 0, nf = 0;
    trace_pair<true>(m, o, rr, m.antipod[rr], cap, bk, fw, lane, status, nb, nf);
    if (nb < 0 || nf < 0) return;
    uint32_t len = 0;
    for (int s = lane; s < nb; s += 32) len += n_interp_all_lines(m, s ? bk.ids[s - 1] : o, bk.ids[s]);
    for (int s = lane; s < nf; s += 32) len += n_interp_all_lines(m, s ? fw.ids[s - 1] : o, fw.ids[s]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) len += __shfl_xor_sync(FULL_MASK, len, off);
    if (lane == 0) atomicMax(d_max, len);
}

// ---------------------------------------------------------------------------------
// Formal solve, stage 1: one warp per (origin, ray pair) item, one lane per frequency.
// Warps take items in a grid-stride loop over a persistent grid (no block-level
// synchronisation); items of one origin are adjacent, so the warps of a CTA share
// the origin's neighbourhood in L1.  Each item writes u(rr, o, f) and, when the ALO
// is wanted, L_diag(rr, o, f): U[rr * u_stride + (o - u_o0) * F + f].
// ---------------------------------------------------------------------------------
// MINB = CTAs of 256 threads resident per SM the register budget is sized for
// (2: 128, 3: 80, 4: 64 registers per thread); picked at run time by the tuner.
// UV: also v (solve_feautrier_order_2_uv), written to V with U's layout.
template <int MODE, int AP, int MINB, bool UV = false, int GEO = 0>
__global__ void __launch_bounds__(256, MINB)
    fo2_kernel(DevModel m, uint32_t cap, uint32_t o_begin, uint32_t o_end, uint32_t rr0, uint32_t nR,
               double* __restrict__ U, size_t u_stride, uint32_t u_o0, double* __restrict__ LD, size_t ld_stride,
               uint32_t ld_o0, double* __restrict__ V, const uint8_t* __restrict__ cls, uint32_t cls_id,
               int* status) {
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

    const uint64_t n_items = (uint64_t)(o_end - o_begin) * nR;
    const uint64_t stride = (uint64_t)gridDim.x * nw;
    for (uint64_t item = (uint64_t)blockIdx.x * nw + w; item < n_items; item += stride) {
        const uint32_t o = o_begin + (uint32_t)(item / nR);
        const uint32_t rr = rr0 + (uint32_t)(item % nR);
        if (cls && cls[(size_t)o * m.hnrays + rr] != cls_id) continue;  // another length class's launch
        int nb = 0, nf = 0;
        trace_pair<true, 0, GEO>(m, o, rr, m.antipod[rr], cap, bk, fw, lane, status, nb, nf);
        if (nb < 0 || nf < 0) continue;  // status recorded by the trace
        double* Ui = U + (size_t)(rr - rr0) * u_stride + (size_t)(o - u_o0) * m.F;
        double* Li = LD ? LD + (size_t)(rr - rr0) * ld_stride + (size_t)(o - ld_o0) * m.F : nullptr;
        for (uint32_t f0 = 0; f0 < m.F; f0 += 32) {
            const uint32_t f = f0 + lane;
            if (f < m.F) {
                const LaneCtx c = lane_ctx(m, o, f);
                const LaneResult r = solve_lane<MODE, AP, UV>(m, sl, c, bk, nb, fw, nf);
                Ui[f] = r.u;
                if constexpr (UV) V[(size_t)(rr - rr0) * u_stride + (size_t)(o - u_o0) * m.F + f] = r.v;
                if (Li) Li[f] = r.solved ? r.Ldiag : 0.0;
                if (!isfinite(r.u)) atomicOr(status, ST_NONFINITE);
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------
// Formal solve with the non-local ALO (n_off_diag > 0, FP64 mode): fo2_kernel's work
// plus, per lane of a frequency in a line integral, the update_Lambda terms of the
// K = m.n_off_diag band elements on each side of the origin (solve_lane<..., NB>).
// They are summed over the line's quadrature points by a segmented shuffle scan (the
// lanes of one line are adjacent) and added to
//   alo_off[((o * L + l) * hnrays + rr) * 2K + slot],  alo_nr[...] the element's point
// (slot m: centre - m - 1, slot K + m: centre + m + 1).  One warp owns an (o, rr) item
// and adds its frequency chunks in order, so the sums are deterministic.
// ---------------------------------------------------------------------------------
constexpr int kMaxBand = (int)kMaxOffDiag;

template <int AP>
__global__ void __launch_bounds__(256, 2)
    fo2_alo_kernel(DevModel m, uint32_t cap, uint32_t o_begin, uint32_t o_end, uint32_t rr0, uint32_t nR,
                   double* __restrict__ U, size_t u_stride, uint32_t u_o0, double* __restrict__ LD, size_t ld_stride,
                   uint32_t ld_o0, double* __restrict__ alo_off, uint32_t* __restrict__ alo_nr, int* status) {
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
    const uint32_t K = m.n_off_diag;
    const uint64_t n_items = (uint64_t)(o_end - o_begin) * nR;
    const uint64_t stride = (uint64_t)gridDim.x * nw;
    for (uint64_t item = (uint64_t)blockIdx.x * nw + w; item < n_items; item += stride) {
        const uint32_t o = o_begin + (uint32_t)(item / nR);
        const uint32_t rr = rr0 + (uint32_t)(item % nR);
        int nb = 0, nf = 0;
        trace_pair<true, 0, 1>(m, o, rr, m.antipod[rr], cap, bk, fw, lane, status, nb, nf);
        if (nb < 0 || nf < 0) continue;  // status recorded by the trace
        double* Ui = U + (size_t)(rr - rr0) * u_stride + (size_t)(o - u_o0) * m.F;
        double* Li = LD ? LD + (size_t)(rr - rr0) * ld_stride + (size_t)(o - ld_o0) * m.F : nullptr;
        for (uint32_t f0 = 0; f0 < m.F; f0 += 32) {
            const uint32_t f = f0 + lane;
            BandOut<kMaxBand> bo;
            bo.K = K;
            bo.w_rr = 0.0;
            uint32_t lid = 0xffffffffu;
            bool bands = false;
            if (f < m.F) {
                const LaneCtx c = lane_ctx(m, o, f);
                bo.w_rr = ray_w(m, o, rr);
                const LaneResult r = solve_lane<MODE_FP64, AP, false, kMaxBand>(m, sl, c, bk, nb, fw, nf, &bo);
                Ui[f] = r.u;
                if (Li) Li[f] = r.solved ? r.Ldiag : 0.0;
                if (!isfinite(r.u)) atomicOr(status, ST_NONFINITE);
                lid = m.corr_line[f];
                bands = r.solved && m.in_line[f];
            }
            // lanes of one line are adjacent: a segment starts where the line changes
            const uint32_t prev = __shfl_up_sync(FULL_MASK, lid, 1);
            const uint32_t heads = __ballot_sync(FULL_MASK, lane == 0 || prev != lid);
            const int seg0 = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
            const uint32_t next = __shfl_down_sync(FULL_MASK, lid, 1);
            const bool tail = (lane == 31) || next != lid;
            // the segment's first lane with band terms supplies the elements' points
            const uint32_t with = __ballot_sync(FULL_MASK, bands) & (0xffffffffu << seg0);
            const int src = with ? __ffs(with) - 1 : lane;
            const bool write = tail && with != 0 && src <= lane;
            for (uint32_t s = 0; s < 2 * K; s++) {
                double v = bands ? bo.val[s] : 0.0;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const double up = __shfl_up_sync(FULL_MASK, v, off);
                    if (lane - off >= seg0) v += up;
                }
                const uint32_t seg_nr = __shfl_sync(FULL_MASK, bands ? bo.nr[s] : o, src);
                if (write) {
                    const size_t a = (((size_t)o * m.L + lid) * m.hnrays + rr) * 2 * K + s;
                    alo_off[a] += v;
                    alo_nr[a] = seg_nr;
                }
            }
            __syncwarp();  // a line split over two chunks: the next chunk's tail lane adds to these sums
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------
// Formal solve, stage 2: J and the ALO diagonal per origin.
//   J(o, f)      = sum_rr u(rr, o, f) 2 w_rr, in ray-pair order       (solver.tpp:497-504)
//   Lambda(o, l) = sum_q sum_rr lambda_element(o, rr, f(l, q))         (update_Lambda)
// One CTA per origin (grid-stride); J by threads over f; the line integrals (ALO,
// memory-lean J, anisotropic sums) by warps over lines, lane q summing its quadrature
// point over the ray pairs in order and the warp then summing its lanes by a butterfly
// (so every FP64 instruction does the work of all lanes; the reference's own order
// is rr outer, q inner, a different association of the same terms).
// lq2f[l * Q + q] is the frequency of (l, q).
// ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) fo2_reduce_kernel(DevModel m, uint32_t o_begin, uint32_t o_end,
                                                         uint32_t rr0, uint32_t nR,
                                                         const double* __restrict__ U, size_t u_stride, uint32_t u_o0,
                                                         const double* __restrict__ LD, size_t ld_stride,
                                                         uint32_t ld_o0, double* __restrict__ J,
                                                         double* __restrict__ lam, double* __restrict__ Jlin,
                                                         double* __restrict__ anis) {
    const int nw = blockDim.x >> 5;
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    for (uint32_t o = o_begin + blockIdx.x; o < o_end; o += gridDim.x) {
        if (J) reduce_J_origin(m, o, rr0, nR, U, u_stride, u_o0, J, threadIdx.x, blockDim.x);
        if (Jlin) {
            // line-integrated J of the memory-lean solve (solve_feautrier_order_2_sparse,
            // solver.tpp:297-363): J(o, l) = sum of w_z (2 w_rr) u over (rr, z)
            for (uint32_t l = w; l < m.L; l += nw) {
                const uint32_t* l2f = m.lq2f + (size_t)l * m.Q;
                double s = 0.0;
                for (uint32_t q0 = 0; q0 < m.Q; q0 += 32) {
                    const uint32_t q = q0 + lane;
                    if (q >= m.Q) continue;
                    const uint32_t f = l2f[q];
                    const double wz = m.quad_w[(size_t)m.corr_lspec[f] * m.Q + q];
                    double part = 0.0;
                    for (uint32_t rr = rr0; rr < rr0 + nR; rr++)
                        part += (wz * (ray_w(m, o, rr) * 2.0)) *
                                U[(size_t)(rr - rr0) * u_stride + (size_t)(o - u_o0) * m.F + f];
                    s += part;
                }
                s = warp_sum(s);
                if (lane == 0) Jlin[(size_t)o * m.L + l] = s;
            }
        }
        if (anis) {
            // line-integrated J and anisotropy tensor elements (solve_feautrier_order_2_anis,
            // solver.tpp:366-456): du = w_z w_rr u, J += 2 du, J2_x += wt_x(n) du over (rr, z)
            const double sqrt3 = sqrt(3.0), inv_sqrt2 = 1.0 / sqrt(2.0);
            const size_t PL = (size_t)m.P * m.L;
            for (uint32_t l = w; l < m.L; l += nw) {
                const uint32_t* l2f = m.lq2f + (size_t)l * m.Q;
                double sJ = 0.0, s0 = 0.0, s1r = 0.0, s1i = 0.0, s2r = 0.0, s2i = 0.0;
                for (uint32_t q0 = 0; q0 < m.Q; q0 += 32) {
                    const uint32_t q = q0 + lane;
                    if (q >= m.Q) continue;
                    const uint32_t f = l2f[q];
                    const double wz = m.quad_w[(size_t)m.corr_lspec[f] * m.Q + q];
                    double pJ = 0.0, p0 = 0.0, p1r = 0.0, p1i = 0.0, p2r = 0.0, p2i = 0.0;
                    for (uint32_t rr = rr0; rr < rr0 + nR; rr++) {
                        const double* dn = ray_dir(m, o, rr);
                        const double nx = dn[0], ny = dn[1], nz = dn[2];
                        const double d =
                            (wz * ray_w(m, o, rr)) * U[(size_t)(rr - rr0) * u_stride + (size_t)(o - u_o0) * m.F + f];
                        pJ += 2.0 * d;
                        p0 += (inv_sqrt2 * (3.0 * nz * nz - 1.0)) * d;
                        p1r += (-sqrt3 * nx * nz) * d;
                        p1i += (-sqrt3 * ny * nz) * d;
                        p2r += (0.5 * sqrt3 * (nx * nx - ny * ny)) * d;
                        p2i += (sqrt3 * nx * ny) * d;
                    }
                    sJ += pJ;
                    s0 += p0;
                    s1r += p1r;
                    s1i += p1i;
                    s2r += p2r;
                    s2i += p2i;
                }
                sJ = warp_sum(sJ);
                s0 = warp_sum(s0);
                s1r = warp_sum(s1r);
                s1i = warp_sum(s1i);
                s2r = warp_sum(s2r);
                s2i = warp_sum(s2i);
                if (lane == 0) {
                    const size_t i = (size_t)o * m.L + l;
                    anis[i] = sJ;
                    anis[PL + i] = s0;
                    anis[2 * PL + i] = s1r;
                    anis[3 * PL + i] = s1i;
                    anis[4 * PL + i] = s2r;
                    anis[5 * PL + i] = s2i;
                }
            }
        }
        if (lam) reduce_lam_origin(m, o, rr0, nR, LD, ld_stride, ld_o0, lam, w, nw, lane);
    }
}

// ---------------------------------------------------------------------------------
// One ray pair for one line in the reference's buffer layout (for parity checks).
// meta = {n_tot, centre, status}.
// ---------------------------------------------------------------------------------
__global__ void trace_export_kernel(DevModel m, uint32_t o, uint32_t rr, uint32_t l, uint32_t cap, uint32_t capacity,
                                    uint32_t* meta, uint32_t* nr, uint32_t* ni, double* fac, double* shift, double* dZ,
                                    int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    HalfSmem bk, fw;
    carve_halves(smem, cap, bk, fw);
    int nb = 0, nf = 0;
    trace_pair<true>(m, o, rr, m.antipod[rr], cap, bk, fw, lane, status, nb, nf);
    if (lane != 0) return;
    if (nb < 0 || nf < 0) {
        meta[0] = 0;
        meta[1] = 0;
        meta[2] = 1;
        return;
    }
    // count elements of each half
    uint32_t cb = 0, cf = 0;
    for (int s = 0; s < nb; s++) cb += m.nint[(size_t)bk.eid[s] * m.L + l];
    for (int s = 0; s < nf; s++) cf += m.nint[(size_t)fw.eid[s] * m.L + l];
    const uint32_t n_tot = cb + 1 + cf;
    if (n_tot > capacity) {
        meta[0] = n_tot;
        meta[1] = cb;
        meta[2] = 2;
        return;
    }
    // backward half: outer end first = array index 0
    uint32_t idx = 0;
    ElemIter it;
    Elem e;
    if (nb > 0) {
        iter_begin<MODE_FP64>(m, bk, o, l, nb, it);
        while (iter_next<MODE_FP64>(m, bk, o, l, it, e)) {
            nr[idx] = e.nr;
            ni[idx] = e.ni;
            fac[idx] = e.fac;
            shift[idx] = e.shift;
            dZ[idx] = e.dzin;  // distance to the next (inner) element
            idx++;
        }
    }
    nr[idx] = o;
    ni[idx] = 0;
    fac[idx] = 0.0;
    shift[idx] = 1.0;
    const uint32_t centre = idx;
    // forward half: elements centre+1 .. last are produced outer end first
    if (nf > 0) {
        iter_begin<MODE_FP64>(m, fw, o, l, nf, it);
        uint32_t j = n_tot - 1;
        while (iter_next<MODE_FP64>(m, fw, o, l, it, e)) {
            nr[j] = e.nr;
            ni[j] = e.ni;
            fac[j] = e.fac;
            shift[j] = e.shift;
            dZ[j - 1] = e.dzin;  // distance to the previous (inner) element
            j--;
        }
    }
    meta[0] = n_tot;
    meta[1] = centre;
    meta[2] = 0;
}

// ---------------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------------
cudaError_t launch_line_tables(MgrModel* model) {
    const size_t n = (size_t)model->dm.P * model->dm.L;
    const int threads = 256;
    const int blocks = (int)((n + threads - 1) / threads < 152 * 16 ? (n + threads - 1) / threads : 152 * 16);
    count_launch();
    line_tables_kernel<<<blocks > 0 ? blocks : 1, threads, 0, model->stream>>>(
        model->em, model->op, model->iw, model->Sp, model->em_f, model->op_f, model->iw_f, model->Sp_f, model->iw_lo,
        n, model->scales.Ke, model->scales.Ko);
    return cudaGetLastError();
}

cudaError_t launch_size_rays(MgrModel* model, uint32_t* d_max_steps) {
    const uint64_t warps = (uint64_t)model->dm.P * model->dm.hnrays;
    const int threads = 256;
    const uint64_t blocks = (warps * 32 + threads - 1) / threads;
    count_launch();
    size_rays_kernel<<<(unsigned)blocks, threads, 0, model->stream>>>(model->dm, model->pair_class, d_max_steps,
                                                                     model->status);
    return cudaGetLastError();
}

cudaError_t launch_ray_lengths(MgrModel* model, uint32_t* d_max_len) {
    const uint32_t cap = model->half_cap;
    const int wpb = 4;
    const size_t smem = wpb * half_bytes_per_warp(cap);
    const uint64_t warps = (uint64_t)model->dm.P * model->dm.hnrays;
    const uint64_t blocks = (warps + wpb - 1) / wpb;
    cudaError_t e = cudaFuncSetAttribute(ray_lengths_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    count_launch();
    ray_lengths_kernel<<<(unsigned)blocks, wpb * 32, smem, model->stream>>>(model->dm, cap, d_max_len, model->status);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// Work statistics of one formal solve: trace steps, neighbour records read by the
// trace, and ray-pair elements summed over lines (for the algorithmic-bytes roofline).
// stats = {steps, neighbour_reads, elements}.
// ---------------------------------------------------------------------------------
__global__ void ray_stats_kernel(DevModel m, uint32_t cap, unsigned long long* stats, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t gw = (uint64_t)blockIdx.x * (blockDim.x >> 5) + w;
    if (gw >= (uint64_t)m.P * m.hnrays) return;
    HalfSmem bk, fw;
    carve_halves(smem + (size_t)w * half_bytes_per_warp(cap), cap, bk, fw);
    const uint32_t o = (uint32_t)(gw / m.hnrays);
    const uint32_t rr = (uint32_t)(gw % m.hnrays);
    int nb = 0, nf = 0;
    trace_pair<true>(m, o, rr, m.antipod[rr], cap, bk, fw, lane, status, nb, nf);
    if (nb < 0 || nf < 0) return;
    unsigned long long nbr = 0, elems = 0;
    for (int s = lane; s < nb; s += 32) {
        const uint32_t crt = s ? bk.ids[s - 1] : o;
        nbr += m.n_nb[crt];
        for (uint32_t l = 0; l < m.L; l++) elems += m.nint[(size_t)bk.eid[s] * m.L + l];
    }
    for (int s = lane; s < nf; s += 32) {
        const uint32_t crt = s ? fw.ids[s - 1] : o;
        nbr += m.n_nb[crt];
        for (uint32_t l = 0; l < m.L; l++) elems += m.nint[(size_t)fw.eid[s] * m.L + l];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        nbr += __shfl_xor_sync(FULL_MASK, nbr, off);
        elems += __shfl_xor_sync(FULL_MASK, elems, off);
    }
    if (lane == 0) {
        atomicAdd(&stats[0], (unsigned long long)(nb + nf));
        atomicAdd(&stats[1], nbr);
        atomicAdd(&stats[2], elems + m.L);  // + the origin element of each line
    }
}

cudaError_t launch_ray_stats(MgrModel* model, unsigned long long* d_stats) {
    const uint32_t cap = model->half_cap;
    const int wpb = 4;
    const size_t smem = wpb * half_bytes_per_warp(cap);
    const uint64_t warps = (uint64_t)model->dm.P * model->dm.hnrays;
    const uint64_t blocks = (warps + wpb - 1) / wpb;
    cudaError_t e = cudaFuncSetAttribute(ray_stats_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    count_launch();
    ray_stats_kernel<<<(unsigned)blocks, wpb * 32, smem, model->stream>>>(model->dm, cap, d_stats, model->status);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// Self-check of the trace's FP32 next-point filter: one warp per (origin, ray) walks
// the half ray with the exact FP64 argmin into one buffer and with the filter into the
// other; stats = {rays, steps, rays whose point sequence, edges or dZ bits differ}.
// ---------------------------------------------------------------------------------
__global__ void trace_check_kernel(DevModel m, uint32_t cap, unsigned long long* stats, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t gw = (uint64_t)blockIdx.x * (blockDim.x >> 5) + w;
    if (gw >= (uint64_t)m.P * m.nrays) return;
    HalfSmem ex, fl;
    carve_halves(smem + (size_t)w * half_bytes_per_warp(cap), cap, ex, fl);
    const uint32_t o = (uint32_t)(gw / m.nrays);
    const uint32_t r = (uint32_t)(gw % m.nrays);
    const int n0 = trace_half<true, 0, 1, false>(m, o, r, cap, ex, lane, status);
    const int n1 = trace_half<true, 0, 1, true>(m, o, r, cap, fl, lane, status);
    bool same = n0 == n1;
    for (int k = lane; same && k < n0; k += 32)
        same = ex.ids[k] == fl.ids[k] && ex.eid[k] == fl.eid[k] &&
               __double_as_longlong(ex.dZ[k]) == __double_as_longlong(fl.dZ[k]);
    same = __all_sync(FULL_MASK, same);
    if (lane == 0) {
        atomicAdd(&stats[0], 1ull);
        if (n0 > 0) atomicAdd(&stats[1], (unsigned long long)n0);
        if (!same) atomicAdd(&stats[2], 1ull);
    }
}

cudaError_t launch_trace_check(MgrModel* model, unsigned long long* d_stats) {
    const uint32_t cap = model->half_cap;
    const int wpb = 4;
    const size_t smem = wpb * half_bytes_per_warp(cap);
    const uint64_t warps = (uint64_t)model->dm.P * model->dm.nrays;
    const uint64_t blocks = (warps + wpb - 1) / wpb;
    cudaError_t e = cudaFuncSetAttribute(trace_check_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    count_launch();
    trace_check_kernel<<<(unsigned)blocks, wpb * 32, smem, model->stream>>>(model->dm, cap, d_stats, model->status);
    return cudaGetLastError();
}

// Bytes of U / L_diag staging per origin and the origins one chunk may hold.
static size_t fo2_bytes_per_origin(const MgrModel* model) {
    return (size_t)model->dm.hnrays * model->dm.F * sizeof(double);
}

size_t fo2_work_bytes(const MgrModel* model, uint32_t n_origins, bool stage_u, bool stage_ld) {
    const int k = (stage_u ? 1 : 0) + (stage_ld ? 1 : 0);
    if (k == 0 || n_origins == 0) return 0;
    const size_t per = fo2_bytes_per_origin(model) * k;
    size_t chunk = kFo2WorkBudget / per;
    if (chunk < 1) chunk = 1;
    if (chunk > n_origins) chunk = n_origins;
    return chunk * per;
}

// One launch of fo2_kernel over origins [o_begin, o_end) x ray pairs [rr0, rr0 + nR):
// every pair (cls null, buffers sized for the model's longest half ray) or the pairs of
// length class cls_id (buffers sized for that class's longest half ray).
template <int MODE, int AP, int MINB, bool UV = false, int GEO = 0>
static cudaError_t launch_fo2_variant(MgrModel* model, uint32_t o_begin, uint32_t o_end, uint32_t rr0, uint32_t nR,
                                      double* U, size_t u_stride, uint32_t u_o0, double* LD, size_t ld_stride,
                                      uint32_t ld_o0, double* V = nullptr, const uint8_t* cls = nullptr,
                                      uint32_t cls_id = 0) {
    const DevModel& m = model->dm;
    const uint32_t cap = cls ? model->class_cap[cls_id] : model->half_cap;
    int nw = (MODE == MODE_SPLIT) ? model->fo2_warps_split : model->fo2_warps_fp64;
    if (nw < 1 || nw > 8) nw = 8;
    const uint32_t Lpad = (m.L + 1) & ~1u;
    const size_t smem = (size_t)Lpad * 8 + (size_t)nw * half_bytes_per_warp(cap);
    auto kern = fo2_kernel<MODE, AP, MINB, UV, GEO>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nw * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;  // the ray buffers do not fit in shared memory
    const uint64_t items = (uint64_t)(o_end - o_begin) * nR;
    uint64_t grid = (uint64_t)model->sm_count * per_sm;
    const uint64_t need = (items + nw - 1) / nw;
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    count_launch();
    kern<<<(unsigned)grid, nw * 32, smem, model->stream>>>(m, cap, o_begin, o_end, rr0, nR, U, u_stride, u_o0, LD,
                                                          ld_stride, ld_o0, V, cls, cls_id, model->status);
    return cudaGetLastError();
}

// The formal solve's launches.  Models whose longest half ray is over 128 steps (9 KB
// of shared memory per warp, fewer than 24 warps per SM) get one launch per non-empty
// ray-length class, each with shared memory for its own rays, so that short rays are
// not solved at the occupancy the longest ray allows; shorter models get one launch
// (measured on the 64^3 sphere cutout, longest half ray ~110 steps, the split launches
// were 4 % slower).
template <int MODE, int AP>
static cudaError_t launch_fo2_minb(MgrModel* model, uint32_t o_begin, uint32_t o_end, uint32_t rr0, uint32_t nR,
                                   double* U, size_t us, uint32_t uo, double* LD, size_t ls, uint32_t lo) {
    const int minb = (MODE == MODE_SPLIT) ? model->fo2_minb_split : model->fo2_minb_fp64;
    const bool any_geo = model->dm.sph || model->dm.adaptive;
    const uint8_t* cls = model->half_cap > kLenClassBound[2] ? model->pair_class : nullptr;
    for (int c = 0; c < (cls ? kLenClasses : 1); c++) {
        if (cls && model->class_cap[c] == 0) continue;
        cudaError_t e;
        // spherical symmetry and adaptive rays: the run-time geometry variant, one tile
        if (any_geo) e = launch_fo2_variant<MODE, AP, 3, false, 1>(model, o_begin, o_end, rr0, nR, U, us, uo, LD, ls, lo,
                                                                  nullptr, cls, c);
        else if (minb == 2)
            e = launch_fo2_variant<MODE, AP, 2>(model, o_begin, o_end, rr0, nR, U, us, uo, LD, ls, lo, nullptr, cls, c);
        else if (minb == 4)
            e = launch_fo2_variant<MODE, AP, 4>(model, o_begin, o_end, rr0, nR, U, us, uo, LD, ls, lo, nullptr, cls, c);
        else
            e = launch_fo2_variant<MODE, AP, 3>(model, o_begin, o_end, rr0, nR, U, us, uo, LD, ls, lo, nullptr, cls, c);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// The uv solve: one register budget (MINB 3), no tuning.
template <int MODE>
static cudaError_t launch_fo2_uv(MgrModel* model, uint32_t o_begin, uint32_t o_end, uint32_t rr0, uint32_t nR,
                                 double* U, size_t us, uint32_t uo, double* LD, size_t ls, uint32_t lo, double* V) {
    switch (model->dm.approx) {
        case APPROX_ONELINE:
            return launch_fo2_variant<MODE, APPROX_ONELINE, 3, true, 1>(model, o_begin, o_end, rr0, nR, U, us, uo, LD, ls,
                                                                     lo, V);
        case APPROX_CLOSELINES:
            return launch_fo2_variant<MODE, APPROX_CLOSELINES, 3, true, 1>(model, o_begin, o_end, rr0, nR, U, us, uo, LD,
                                                                        ls, lo, V);
        default:
            return launch_fo2_variant<MODE, APPROX_NONE, 3, true, 1>(model, o_begin, o_end, rr0, nR, U, us, uo, LD, ls,
                                                                  lo, V);
    }
}

template <int MODE>
static cudaError_t launch_fo2_approx(MgrModel* model, uint32_t o_begin, uint32_t o_end, uint32_t rr0, uint32_t nR,
                                     double* U, size_t us, uint32_t uo, double* LD, size_t ls, uint32_t lo) {
    switch (model->dm.approx) {
        case APPROX_ONELINE:
            return launch_fo2_minb<MODE, APPROX_ONELINE>(model, o_begin, o_end, rr0, nR, U, us, uo, LD, ls, lo);
        case APPROX_CLOSELINES:
            return launch_fo2_minb<MODE, APPROX_CLOSELINES>(model, o_begin, o_end, rr0, nR, U, us, uo, LD, ls, lo);
        default: return launch_fo2_minb<MODE, APPROX_NONE>(model, o_begin, o_end, rr0, nR, U, us, uo, LD, ls, lo);
    }
}

// Band elements of origins [o_begin, o_end) cleared: value 0 and the origin's own
// point, which an element keeps where no frequency of its line has a band term (a
// ray of one point, or an element beyond the ray's end), so that every slot names a
// point whatever the values.
__global__ void alo_init_kernel(uint32_t o_begin, uint32_t o_end, size_t per_o, double* __restrict__ alo_off,
                                uint32_t* __restrict__ alo_nr) {
    const size_t n = (size_t)(o_end - o_begin) * per_o;
    const size_t base = (size_t)o_begin * per_o;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        alo_off[base + t] = 0.0;
        alo_nr[base + t] = o_begin + (uint32_t)(t / per_o);
    }
}

// The banded solve (non-local ALO): FP64 mode, the run-time geometry variant.
static cudaError_t launch_fo2_alo(MgrModel* model, uint32_t o_begin, uint32_t o_end, uint32_t rr0, uint32_t nR,
                                  double* U, size_t us, uint32_t uo, double* LD, size_t ls, uint32_t lo,
                                  double* alo_off, uint32_t* alo_nr) {
    const DevModel& m = model->dm;
    const uint32_t cap = model->half_cap;
    const int nw = 4;
    const uint32_t Lpad = (m.L + 1) & ~1u;
    const size_t smem = (size_t)Lpad * 8 + (size_t)nw * half_bytes_per_warp(cap);
    auto kern = (m.approx == APPROX_ONELINE)      ? fo2_alo_kernel<APPROX_ONELINE>
                : (m.approx == APPROX_CLOSELINES) ? fo2_alo_kernel<APPROX_CLOSELINES>
                                                  : fo2_alo_kernel<APPROX_NONE>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nw * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const uint64_t items = (uint64_t)(o_end - o_begin) * nR;
    uint64_t grid = (uint64_t)model->sm_count * per_sm;
    const uint64_t need = (items + nw - 1) / nw;
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    count_launch();
    kern<<<(unsigned)grid, nw * 32, smem, model->stream>>>(m, cap, o_begin, o_end, rr0, nR, U, us, uo, LD, ls, lo,
                                                          alo_off, alo_nr, model->status);
    return cudaGetLastError();
}

cudaError_t launch_fo2_range(MgrModel* model, int precision, uint32_t o_begin, uint32_t o_end, double* J, double* u,
                             double* lam, double* work, size_t work_bytes, uint32_t rr_begin, uint32_t rr_end,
                             double* Jlin, double* anis, double* v, double* alo_off, uint32_t* alo_nr) {
    const DevModel& m = model->dm;
    if (o_end <= o_begin) return cudaSuccess;
    if (rr_end > m.hnrays) rr_end = m.hnrays;
    if (rr_begin >= rr_end) return cudaErrorInvalidValue;
    const uint32_t nR = rr_end - rr_begin;
    if (u && nR != m.hnrays) return cudaErrorInvalidValue;  // u is written for full solves only
    if (alo_off) {
        // every ray pair of the origins' lists, cleared first
        if (m.n_off_diag == 0 || m.n_off_diag > (uint32_t)kMaxBand || nR != m.hnrays || v || !alo_nr)
            return cudaErrorInvalidValue;
        const size_t per_o = (size_t)m.L * m.hnrays * 2 * m.n_off_diag;
        const size_t n0 = (size_t)(o_end - o_begin) * per_o;
        size_t g0 = (n0 + 255) / 256;
        if (g0 > (size_t)model->sm_count * 16) g0 = (size_t)model->sm_count * 16;
        count_launch();
        alo_init_kernel<<<(unsigned)(g0 ? g0 : 1), 256, 0, model->stream>>>(o_begin, o_end, per_o, alo_off, alo_nr);
        const cudaError_t e0 = cudaGetLastError();
        if (e0 != cudaSuccess) return e0;
    }
    const int k = (u ? 0 : 1) + (lam ? 1 : 0);
    const size_t per = fo2_bytes_per_origin(model);
    uint32_t chunk = o_end - o_begin;
    if (k) {
        const size_t fit = work ? work_bytes / (per * k) : 0;
        if (fit < 1) return cudaErrorInvalidValue;  // caller sizes the work area with fo2_work_bytes
        if (fit < chunk) chunk = (uint32_t)fit;
    }
    int nsm = model->sm_count;
    for (uint32_t c0 = o_begin; c0 < o_end; c0 += chunk) {
        const uint32_t c1 = (o_end - c0 > chunk) ? c0 + chunk : o_end;
        const uint32_t n = c1 - c0;
        double* U;
        size_t us;
        uint32_t uo;
        double* next = work;
        if (u) {
            U = u;
            us = (size_t)m.P * m.F;
            uo = 0;
        } else {
            U = work;
            us = (size_t)n * m.F;
            uo = c0;
            next = work + (size_t)nR * n * m.F;
        }
        double* LD = lam ? next : nullptr;
        const size_t ls = (size_t)n * m.F;
        cudaError_t e;
        if (alo_off)
            e = launch_fo2_alo(model, c0, c1, rr_begin, nR, U, us, uo, LD, ls, c0, alo_off, alo_nr);
        else if (v)  // v has u's layout: u is given (no chunked staging of U)
            e = (precision == MGR_PRECISION_SPLIT)
                    ? launch_fo2_uv<MODE_SPLIT>(model, c0, c1, rr_begin, nR, U, us, uo, LD, ls, c0, v)
                    : launch_fo2_uv<MODE_FP64>(model, c0, c1, rr_begin, nR, U, us, uo, LD, ls, c0, v);
        else
            e = (precision == MGR_PRECISION_SPLIT)
                    ? launch_fo2_approx<MODE_SPLIT>(model, c0, c1, rr_begin, nR, U, us, uo, LD, ls, c0)
                    : launch_fo2_approx<MODE_FP64>(model, c0, c1, rr_begin, nR, U, us, uo, LD, ls, c0);
        if (e != cudaSuccess) return e;
        if (!J && !lam && !Jlin && !anis) continue;  // u (and v) only
        unsigned grid = n < (uint32_t)nsm * 16 ? n : (unsigned)nsm * 16;
        count_launch();
        fo2_reduce_kernel<<<grid, 128, 0, model->stream>>>(m, c0, c1, rr_begin, nR, U, us, uo, LD, ls, c0, J, lam,
                                                           Jlin, anis);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_trace_export(MgrModel* model, uint32_t o, uint32_t rr, uint32_t l, uint32_t capacity,
                                uint32_t* d_meta, uint32_t* d_nr, uint32_t* d_ni, double* d_fac, double* d_shift,
                                double* d_dZ) {
    const uint32_t cap = model->half_cap;
    const size_t smem = half_bytes_per_warp(cap);
    cudaError_t e = cudaFuncSetAttribute(trace_export_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    count_launch();
    trace_export_kernel<<<1, 32, smem, model->stream>>>(model->dm, o, rr, l, cap, capacity, d_meta, d_nr, d_ni, d_fac,
                                                        d_shift, d_dZ, model->status);
    return cudaGetLastError();
}

}  // namespace mgr
