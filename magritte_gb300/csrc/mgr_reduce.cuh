// Per-origin reductions of the staged ray-pair results (the formal solve's second
// stage), shared by the single-model reduction kernel and the many-model batch so that
// both sum in the same order.
//   J(o, f)      = sum_rr u(rr, o, f) 2 w_rr, in ray-pair order       (solver.tpp:497-504)
//   Lambda(o, l) = sum_q sum_rr lambda_element(o, rr, f(l, q))         (update_Lambda,
//                  solver.tpp:1760-1800): lane q sums its quadrature point over the ray
//                  pairs in order, the warp then sums its lanes by a butterfly.
// U / LD hold u and L_diag at [(rr - rr0) * stride + (o - o0) * F + f].
#pragma once
#include "mgr_solve.cuh"

namespace mgr {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(FULL_MASK, v, off);
    return v;
}

// Threads t = 0 .. nt-1 over the frequencies.
__device__ __forceinline__ void reduce_J_origin(const DevModel& m, uint32_t o, uint32_t rr0, uint32_t nR,
                                                const double* __restrict__ U, size_t u_stride, uint32_t u_o0,
                                                double* __restrict__ J, int t, int nt) {
    for (uint32_t f = (uint32_t)t; f < m.F; f += (uint32_t)nt) {
        const double* Uo = U + (size_t)(o - u_o0) * m.F + f;
        double s = 0.0;
        for (uint32_t k = 0; k < nR; k++) s += Uo[(size_t)k * u_stride] * 2.0 * ray_w(m, o, rr0 + k);
        J[(size_t)o * m.F + f] = s;
    }
}

// Warps w = 0 .. nw-1 over the lines, lanes over the quadrature points.
__device__ __forceinline__ void reduce_lam_origin(const DevModel& m, uint32_t o, uint32_t rr0, uint32_t nR,
                                                  const double* __restrict__ LD, size_t ld_stride, uint32_t ld_o0,
                                                  double* __restrict__ lam, int w, int nw, int lane) {
    for (uint32_t l = (uint32_t)w; l < m.L; l += (uint32_t)nw) {
        // lane q: the ray-independent factors of quadrature point q, then its elements
        // over the ray pairs in order
        const uint32_t* l2f = m.lq2f + (size_t)l * m.Q;
        double s = 0.0;
        for (uint32_t q0 = 0; q0 < m.Q; q0 += 32) {
            const uint32_t q = q0 + lane;
            const uint32_t f = q < m.Q ? l2f[q] : 0xffffffffu;
            if (f == 0xffffffffu || !m.in_line[f]) continue;
            const LambdaFactors k = lambda_factors(m, m.sorted_line, o, f);
            double part = 0.0;
            for (uint32_t rr = rr0; rr < rr0 + nR; rr++)
                part += lambda_element(k, ray_w(m, o, rr),
                                       LD[(size_t)(rr - rr0) * ld_stride + (size_t)(o - ld_o0) * m.F + f]);
            s += part;
        }
        s = warp_sum(s);
        if (lane == 0) lam[(size_t)o * m.L + l] = s;
    }
}

}  // namespace mgr
