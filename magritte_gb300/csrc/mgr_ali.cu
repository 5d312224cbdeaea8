// ALI level populations on the GPU: compute_Jeff, statistical equilibrium,
// negative-population correction, convergence statistics, emissivity / opacity
// refresh and general-order Ng acceleration, all device resident, driven by the host
// loop of Model::compute_level_populations (src/model/model.cpp:654-747).  The
// per-iteration work after the Ng decision (formal solve, Jeff, rate equations,
// corrections, convergence, line data) is captured once as a CUDA graph and
// replayed every normal iteration.
//
// Reference: src/model/lines/lineProducingSpecies/lineProducingSpecies.tpp (LTE
// :52-75, convergence :128-205, Ng :266-372, statistical equilibrium :377-581,
// negative populations :711-802), src/model/lines/lines.tpp:29-40 (emissivity /
// opacity), src/model/model.cpp:514-545 (Jeff), :584-645 (Ng criteria).
//
// With n_off_diag = 0 the reference's global sparse rate system (solved with
// Eigen's SparseLU in long double) is block diagonal: one nlev x nlev block per
// point.  Here one warp solves one block in shared memory by Gaussian elimination
// with partial pivoting in FP64.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "mgr_ali.h"

namespace mgr {

constexpr double HH_OVER_FOUR_PI = HH / (4.0 * 3.14159265358979323846);  // constants.hpp:17,40

// ---------------------------------------------------------------------------------
// compute_Jeff, n_off_diag = 0 (model.cpp:514-545): thread per (p, k).
// ---------------------------------------------------------------------------------
// With Jlin_in (the memory-lean solve's line-integrated J, [P][L]): compute_Jeff_sparse
// (model.cpp:549-570), Jlin taken as it is and Jdif left unchanged.
__global__ void jeff_kernel(DevModel m, SpeciesView s, const double* __restrict__ J, const double* __restrict__ lam,
                            const double* __restrict__ Jlin_in) {
    const size_t n = (size_t)m.P * s.nrad;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const uint32_t p = (uint32_t)(t / s.nrad), k = (uint32_t)(t % s.nrad);
        const uint32_t lid = s.line_offset + k;
        double jl = 0.0;
        if (Jlin_in) {
            jl = Jlin_in[(size_t)p * m.L + lid];
        } else {
            for (uint32_t z = 0; z < m.Q; z++) {
                const uint32_t f = m.lq2f[(size_t)lid * m.Q + z];  // nr_line[p][k][z]
                jl = __dadd_rn(jl, __dmul_rn(m.quad_w[(size_t)m.corr_lspec[f] * m.Q + z], J[(size_t)p * m.F + f]));
            }
        }
        const double diff = __dmul_rn(lam[(size_t)p * m.L + lid], s.pop[(size_t)p * s.nlev + s.irad[k]]);
        s.Jlin[t] = jl;
        s.Jeff[t] = __dsub_rn(jl, __dmul_rn(HH_OVER_FOUR_PI, diff));
        if (!Jlin_in) s.Jdif[t] = __dmul_rn(HH_OVER_FOUR_PI, diff);
    }
}

// ---------------------------------------------------------------------------------
// Statistical equilibrium (lineProducingSpecies.tpp:377-581): warp per point.
// ---------------------------------------------------------------------------------
__device__ uint32_t search_table(const double* x, uint32_t n, double value) {  // interpolation.hpp:10-33
    uint32_t start = 0, stop = n - 1;
    if (value >= x[stop]) return stop;
    if (value <= x[start]) return start;
    while (stop > start + 1) {
        const uint32_t middle = (stop + start) / 2;
        if (value > x[middle]) start = middle;
        else if (value < x[middle]) stop = middle;
        else return middle;
    }
    return stop;
}

__device__ __forceinline__ double opacity_of(const SpeciesView& s, const double* pp, uint32_t k,
                                             double min_line_opacity) {
    const double v = __dmul_rn(__dmul_rn(s.freq[k], HH_OVER_FOUR_PI),
                               __dsub_rn(__dmul_rn(pp[s.jrad[k]], s.Ba[k]), __dmul_rn(pp[s.irad[k]], s.Bs[k])));
    return v > min_line_opacity ? v : min_line_opacity;
}

__device__ __forceinline__ double emissivity_of(const SpeciesView& s, const double* pp, uint32_t k,
                                                double min_line_emissivity) {
    const double v = __dmul_rn(__dmul_rn(__dmul_rn(s.freq[k], HH_OVER_FOUR_PI), s.A[k]), pp[s.irad[k]]);
    return v > min_line_emissivity ? v : min_line_emissivity;
}

// The rate block of point p into M (row-major, rows = equations), warp-cooperative.
// Stage 1: the lanes compute the transitions' rates into R (per radiative line k:
// A + Bs Jeff, Ba Jeff and the ALO term -L opacity / nu; per collisional transition:
// Cd abn, Ce abn interpolated in temperature).  Stage 2: lane r owns row r and adds the
// rates that land in it while scanning the transitions in the order the reference
// emits its triplets (radiative, ALO, collisional; then the normalisation row), so
// every entry receives its additions in the reference's order.
// R holds 3 nrad + 2 ncol_total doubles.
__device__ void rate_block(const DevModel& m, const SpeciesView& s, uint32_t p, const double* lam,
                           const double* abundance, uint32_t nspecs, double min_line_opacity, double* M, double* R,
                           int lane) {
    const uint32_t n = s.nlev, last = n - 1, nr = s.nrad;
    const double* pp = s.pop + (size_t)p * n;  // populations before this solve
    const double* Jeff = s.Jeff + (size_t)p * nr;
    double* rIJ = R;            // [nr]
    double* rJI = R + nr;       // [nr]
    double* rA = R + 2 * nr;    // [nr]
    double* cIJ = R + 3 * nr;   // [ncol_total]
    double* cJI = cIJ + s.ncol_total;
    for (uint32_t k = lane; k < nr; k += 32) {
        rIJ[k] = __dadd_rn(s.A[k], __dmul_rn(s.Bs[k], Jeff[k]));
        rJI[k] = __dmul_rn(s.Ba[k], Jeff[k]);
        const double Ls = lam[(size_t)p * m.L + s.line_offset + k];
        rA[k] = -__ddiv_rn(__dmul_rn(Ls, opacity_of(s, pp, k, min_line_opacity)), s.freq[k]);
    }
    const double T = m.T[p];
    uint32_t off = 0;
    for (uint32_t c = 0; c < s.ncolpar; c++) {
        const ColParView& cp = s.cp[c];
        double abn = abundance[(size_t)p * nspecs + cp.num];
        if (cp.ortho_para != 0) {  // collisionPartner.tpp:32-42
            const double frac_H2_para = 1.0 / (1.0 + 9.0 * (double)expf((float)(-170.5 / T)));
            if (cp.ortho_para == 1) abn *= (1.0 - frac_H2_para);
            if (cp.ortho_para == 2) abn *= frac_H2_para;
        }
        const uint32_t t = search_table(cp.tmp, cp.ntmp, T);
        const bool edge = (t == 0 || t == cp.ntmp - 1);
        const double step = edge ? 0.0 : __ddiv_rn(T - cp.tmp[t - 1], cp.tmp[t] - cp.tmp[t - 1]);
        for (uint32_t k = lane; k < cp.ncol; k += 32) {
            double Cd, Ce;
            if (edge) {
                Cd = cp.Cd[(size_t)t * cp.ncol + k];
                Ce = cp.Ce[(size_t)t * cp.ncol + k];
            } else {
                const double ce0 = cp.Ce[(size_t)(t - 1) * cp.ncol + k], ce1 = cp.Ce[(size_t)t * cp.ncol + k];
                const double cd0 = cp.Cd[(size_t)(t - 1) * cp.ncol + k], cd1 = cp.Cd[(size_t)t * cp.ncol + k];
                Ce = __dadd_rn(ce0, __dmul_rn(__dsub_rn(ce1, ce0), step));
                Cd = __dadd_rn(cd0, __dmul_rn(__dsub_rn(cd1, cd0), step));
            }
            cIJ[off + k] = __dmul_rn(Cd, abn);
            cJI[off + k] = __dmul_rn(Ce, abn);
        }
        off += cp.ncol;
    }
    __syncwarp();
    for (uint32_t r = lane; r < n; r += 32) {
        double* row = M + (size_t)r * n;
#define ADD(c, v) row[c] = __dadd_rn(row[c], (v))
        if (r != last) {
            for (uint32_t k = 0; k < nr; k++) {
                const uint32_t I = s.irad[k], J = s.jrad[k];
                if (J == r) {
                    ADD(I, rIJ[k]);
                    ADD(J, -rJI[k]);
                }
                if (I == r) {
                    ADD(J, rJI[k]);
                    ADD(I, -rIJ[k]);
                }
            }
            for (uint32_t k = 0; k < nr; k++) {
                const uint32_t I = s.irad[k], J = s.jrad[k];
                if (J == r) ADD(I, rA[k]);
                if (I == r) ADD(I, -rA[k]);
            }
            uint32_t o = 0;
            for (uint32_t c = 0; c < s.ncolpar; c++) {
                const ColParView& cp = s.cp[c];
                for (uint32_t k = 0; k < cp.ncol; k++) {
                    const uint32_t I = cp.icol[k], J = cp.jcol[k];
                    if (J == r) {
                        ADD(I, cIJ[o + k]);
                        ADD(J, -cJI[o + k]);
                    }
                    if (I == r) {
                        ADD(J, cJI[o + k]);
                        ADD(I, -cIJ[o + k]);
                    }
                }
                o += cp.ncol;
            }
        } else {
            for (uint32_t i = 0; i < n; i++) ADD(i, 1.0);
        }
#undef ADD
    }
}

// Doubles of shared memory per warp of stateq_kernel: the block, the right-hand side and
// the transitions' rates.
__host__ __device__ inline size_t stateq_warp_doubles(const SpeciesView& s) {
    return (size_t)s.nlev * (s.nlev + 1) + 3 * (size_t)s.nrad + 2 * (size_t)s.ncol_total;
}

// Warp per point; the block's warps each own stateq_warp_doubles of shared memory.
__global__ void stateq_kernel(DevModel m, SpeciesView s, const double* __restrict__ lam,
                              const double* __restrict__ abundance, uint32_t nspecs, double min_line_opacity,
                              double* pop_out, int* status) {
    extern __shared__ __align__(16) double smem_ali[];
    const uint32_t n = s.nlev;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double* M = smem_ali + (size_t)w * stateq_warp_doubles(s);
    double* y = M + (size_t)n * n;
    double* R = y + n;
    for (uint32_t p = blockIdx.x * nw + w; p < m.P; p += gridDim.x * nw) {
        for (uint32_t i = lane; i < n * (n + 1); i += 32) M[i] = 0.0;
        __syncwarp();
        rate_block(m, s, p, lam, abundance, nspecs, min_line_opacity, M, R, lane);
        if (lane == 0) y[n - 1] = s.tot[p];
        __syncwarp();
        bool singular = false;
        for (uint32_t c = 0; c < n; c++) {
            // pivot: largest |M[r][c]| over r >= c, lowest row on ties
            double best = -1.0;
            uint32_t piv = c;
            for (uint32_t r = c + lane; r < n; r += 32) {
                const double v = fabs(M[(size_t)r * n + c]);
                if (v > best) {
                    best = v;
                    piv = r;
                }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, off);
                const uint32_t op = __shfl_xor_sync(0xffffffffu, piv, off);
                if (ob > best || (ob == best && op < piv)) {
                    best = ob;
                    piv = op;
                }
            }
            if (!(best > 0.0)) {
                singular = true;
                break;
            }
            if (piv != c) {
                for (uint32_t j = lane; j < n; j += 32) {
                    const double t = M[(size_t)c * n + j];
                    M[(size_t)c * n + j] = M[(size_t)piv * n + j];
                    M[(size_t)piv * n + j] = t;
                }
                if (lane == 0) {
                    const double t = y[c];
                    y[c] = y[piv];
                    y[piv] = t;
                }
                __syncwarp();
            }
            const double d = M[(size_t)c * n + c];
            for (uint32_t r = c + 1; r < n; r++) {
                // column c of row r is not read again, so it is left as is
                const double f = M[(size_t)r * n + c] / d;
                if (f != 0.0) {
                    for (uint32_t j = c + 1 + lane; j < n; j += 32) M[(size_t)r * n + j] -= f * M[(size_t)c * n + j];
                    if (lane == 0) y[r] -= f * y[c];
                }
            }
            __syncwarp();
        }
        if (singular) {
            if (lane == 0) atomicOr(status, ST_NONFINITE);
            continue;
        }
        if (lane == 0) {
            for (uint32_t c = n; c-- > 0;) {
                double acc = y[c];
                for (uint32_t j = c + 1; j < n; j++) acc -= M[(size_t)c * n + j] * y[j];
                y[c] = acc / M[(size_t)c * n + c];
            }
        }
        __syncwarp();
        for (uint32_t i = lane; i < n; i += 32) pop_out[(size_t)p * n + i] = y[i];
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------
// correct_negative_populations (lineProducingSpecies.tpp:711-802): thread per point.
// ---------------------------------------------------------------------------------
__device__ void set_lte_line(const SpeciesView& s, double* pp, double T, uint32_t k) {
    const uint32_t i = s.irad[k], j = s.jrad[k];
    const double tot_line = pp[i] + pp[j];
    pp[i] = s.weight[i] * exp(-s.energy[i] / (KB * T));
    pp[j] = s.weight[j] * exp(-s.energy[j] / (KB * T));
    const double pf = pp[i] + pp[j];
    pp[i] *= tot_line / pf;
    pp[j] *= tot_line / pf;
}

__global__ void negcorr_kernel(DevModel m, SpeciesView s, double inversion_fraction) {
    const uint32_t n = s.nlev;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < m.P; p += gridDim.x * blockDim.x) {
        double* pp = s.pop + (size_t)p * n;
        const double tot = s.tot[p];
        if (tot > 0.0) {
            double tp = 0.0;
            for (uint32_t i = 0; i < n; i++) {
                if (pp[i] < 0.0) pp[i] = 0.0;
                else tp += pp[i];
            }
            for (uint32_t i = 0; i < n; i++) pp[i] = pp[i] * tot / tp;
        }
        if (!(inversion_fraction > 0.0)) continue;  // pop(j) < ratio * pop(i) * f never holds for pops >= 0
        uint64_t mod = 0;  // levels set to LTE (nlev <= 64)
        uint32_t next_n = 0, curr_n = 0;
        const double T = m.T[p];
        do {
            curr_n = next_n;
            bool inv = false;
            for (uint32_t k = s.nrad; k-- > 0;) {
                const uint32_t i = s.irad[k], j = s.jrad[k];
                if (pp[j] < s.Bs[k] / s.Ba[k] * pp[i] * inversion_fraction) {
                    set_lte_line(s, pp, T, k);
                    mod |= (1ull << i) | (1ull << j);
                    inv = true;
                }
            }
            for (uint32_t k = 0; k < s.nrad; k++) {
                const uint32_t i = s.irad[k], j = s.jrad[k];
                if (pp[j] < s.Bs[k] / s.Ba[k] * pp[i] * inversion_fraction) {
                    set_lte_line(s, pp, T, k);
                    mod |= (1ull << i) | (1ull << j);
                    inv = true;
                }
            }
            if (inv) {  // set_LTE_specific_levels (:106-125)
                double tl = 0.0, pf = 0.0;
                for (uint32_t i = 0; i < n; i++)
                    if (mod >> i & 1) {
                        tl += pp[i];
                        pp[i] = s.weight[i] * exp(-s.energy[i] / (KB * T));
                        pf += pp[i];
                    }
                for (uint32_t i = 0; i < n; i++)
                    if (mod >> i & 1) pp[i] *= tl / pf;
            }
            next_n = __popcll(mod);
        } while (next_n != curr_n);
    }
}

// ---------------------------------------------------------------------------------
// check_for_convergence (:128-165) / _trial (:169-205): block partials, then one
// block sums them in a fixed order.  out = {fraction_not_converged, mean, max}.
// ---------------------------------------------------------------------------------
__global__ void convergence_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                   const double* __restrict__ tot, uint32_t P, uint32_t nlev, double pop_prec,
                                   double min_rel, int use_min_rel, double* __restrict__ partial) {
    __shared__ double s_fnc[256], s_rcm[256], s_max[256];
    const double weight = 1.0 / (double)(P * nlev);
    double fnc = 0.0, rcm = 0.0, rmax = 0.0;
    const size_t n = (size_t)P * nlev;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const double x = a[t], y = b[t];
        if (use_min_rel && !(x > min_rel * tot[t / nlev])) continue;
        const double rc = 2.0 * fabs((x - y) / (x + y));
        if (rc > pop_prec) fnc += weight;
        rcm += weight * rc;
        rmax = fmax(rmax, rc);
    }
    s_fnc[threadIdx.x] = fnc;
    s_rcm[threadIdx.x] = rcm;
    s_max[threadIdx.x] = rmax;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            s_fnc[threadIdx.x] += s_fnc[threadIdx.x + h];
            s_rcm[threadIdx.x] += s_rcm[threadIdx.x + h];
            s_max[threadIdx.x] = fmax(s_max[threadIdx.x], s_max[threadIdx.x + h]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[3 * blockIdx.x + 0] = s_fnc[0];
        partial[3 * blockIdx.x + 1] = s_rcm[0];
        partial[3 * blockIdx.x + 2] = s_max[0];
    }
}

__global__ void convergence_finalize(const double* __restrict__ partial, int nblocks, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double fnc = 0.0, rcm = 0.0, rmax = 0.0;
    for (int b = 0; b < nblocks; b++) {
        fnc += partial[3 * b];
        rcm += partial[3 * b + 1];
        rmax = fmax(rmax, partial[3 * b + 2]);
    }
    out[0] = fnc;
    out[1] = rcm;
    out[2] = rmax;
}

// ---------------------------------------------------------------------------------
// set_emissivity_and_opacity (lines.tpp:29-40) and the interpolation criterion
// opacity / population_tot (solver_interp_helper.hpp:15-24): thread per (p, k).
// ---------------------------------------------------------------------------------
__global__ void line_data_kernel(DevModel m, SpeciesView s, double* __restrict__ em, double* __restrict__ op,
                                 double* __restrict__ crit, double min_line_emissivity, double min_line_opacity) {
    const size_t n = (size_t)m.P * s.nrad;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const uint32_t p = (uint32_t)(t / s.nrad), k = (uint32_t)(t % s.nrad);
        const double* pp = s.pop + (size_t)p * s.nlev;
        const size_t i = (size_t)p * m.L + s.line_offset + k;
        em[i] = emissivity_of(s, pp, k, min_line_emissivity);
        const double o = opacity_of(s, pp, k, min_line_opacity);
        op[i] = o;
        crit[i] = o / s.tot[p];
    }
}

// ---------------------------------------------------------------------------------
// Ng acceleration (update_using_acceleration(_trial), :266-372).
// ---------------------------------------------------------------------------------
__global__ void sub_kernel(double* __restrict__ out, const double* __restrict__ a, const double* __restrict__ b,
                           size_t n) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        out[t] = a[t] - b[t];
}

// Partial Gram matrix of `order` residual vectors: partial[block][i*order+j] (i <= j).
__global__ void gram_kernel(VecList r, int order, size_t n, double* __restrict__ partial) {
    __shared__ double s_acc[256];
    const int npairs = order * order;
    for (int ij = 0; ij < npairs; ij++) {
        const int i = ij / order, j = ij % order;
        if (j < i) continue;
        double acc = 0.0;
        for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
            acc += r.v[i][t] * r.v[j][t];
        s_acc[threadIdx.x] = acc;
        __syncthreads();
        for (int h = blockDim.x / 2; h > 0; h >>= 1) {
            if ((int)threadIdx.x < h) s_acc[threadIdx.x] += s_acc[threadIdx.x + h];
            __syncthreads();
        }
        if (threadIdx.x == 0) partial[(size_t)blockIdx.x * npairs + ij] = s_acc[0];
        __syncthreads();
    }
}

// Sums the partial Gram matrices, solves RTR c = 1 by Householder QR with column
// pivoting (the reference's colPivHouseholderQr) and normalises c to unit sum.
__global__ void ng_solve_kernel(const double* __restrict__ partial, int nblocks, int order, double* __restrict__ coef) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int n = order;
    double A[kMaxNgOrder * kMaxNgOrder], b[kMaxNgOrder], x[kMaxNgOrder];
    int perm[kMaxNgOrder];
    for (int i = 0; i < n; i++)
        for (int j = i; j < n; j++) {
            double acc = 0.0;
            for (int blk = 0; blk < nblocks; blk++) acc += partial[(size_t)blk * n * n + i * n + j];
            A[i * n + j] = acc;
            A[j * n + i] = acc;
        }
    for (int i = 0; i < n; i++) {
        b[i] = 1.0;
        perm[i] = i;
    }
    int rank = n;
    for (int k = 0; k < n; k++) {
        int best = k;
        double bn = -1.0;
        for (int j = k; j < n; j++) {
            double acc = 0.0;
            for (int i = k; i < n; i++) acc += A[i * n + j] * A[i * n + j];
            if (acc > bn) {
                bn = acc;
                best = j;
            }
        }
        if (best != k) {
            for (int i = 0; i < n; i++) {
                const double t = A[i * n + k];
                A[i * n + k] = A[i * n + best];
                A[i * n + best] = t;
            }
            const int t = perm[k];
            perm[k] = perm[best];
            perm[best] = t;
        }
        const double an = sqrt(bn);
        if (an == 0.0) {
            rank = k;
            break;
        }
        const double alpha = A[k * n + k] > 0 ? -an : an;
        double v[kMaxNgOrder];
        for (int i = 0; i < n; i++) v[i] = (i < k) ? 0.0 : A[i * n + k];
        v[k] -= alpha;
        double vn = 0.0;
        for (int i = k; i < n; i++) vn += v[i] * v[i];
        if (vn == 0.0) continue;
        for (int j = k; j < n; j++) {
            double acc = 0.0;
            for (int i = k; i < n; i++) acc += v[i] * A[i * n + j];
            acc = 2.0 * acc / vn;
            for (int i = k; i < n; i++) A[i * n + j] -= acc * v[i];
        }
        double acc = 0.0;
        for (int i = k; i < n; i++) acc += v[i] * b[i];
        acc = 2.0 * acc / vn;
        for (int i = k; i < n; i++) b[i] -= acc * v[i];
    }
    for (int i = 0; i < n; i++) x[i] = 0.0;
    for (int i = rank - 1; i >= 0; i--) {
        double acc = b[i];
        for (int j = i + 1; j < rank; j++) acc -= A[i * n + j] * x[j];
        x[i] = acc / A[i * n + i];
    }
    double c[kMaxNgOrder], sum = 0.0;
    for (int j = 0; j < n; j++) c[perm[j]] = x[j];
    for (int j = 0; j < n; j++) sum += c[j];
    for (int j = 0; j < n; j++) coef[j] = c[j] / sum;
}

// out = sum_i hist[i] * coef[order - 1 - i], hist[0] = most recent population.
__global__ void ng_combine_kernel(double* __restrict__ out, VecList hist, const double* __restrict__ coef, int order,
                                  size_t n) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int i = 0; i < order; i++) acc = __dadd_rn(acc, __dmul_rn(hist.v[i][t], coef[order - 1 - i]));
        out[t] = acc;
    }
}

// ---------------------------------------------------------------------------------
// Launch helpers
// ---------------------------------------------------------------------------------
static unsigned grid_for(size_t n, int threads, int cap) {
    size_t b = (n + threads - 1) / threads;
    if (b > (size_t)cap) b = cap;
    return (unsigned)(b ? b : 1);
}

cudaError_t ali_launch_jeff(MgrModel* model, const double* J, const double* lam, const double* Jlin) {
    for (auto& sp : model->ali->species) {
        const size_t n = (size_t)model->dm.P * sp.view.nrad;
        count_launch();
        jeff_kernel<<<grid_for(n, 256, model->sm_count * 16), 256, 0, model->stream>>>(model->dm, sp.view, J, lam,
                                                                                      Jlin);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

static cudaError_t launch_convergence(MgrModel* model, const double* a, const double* b, const double* tot,
                                      uint32_t nlev, bool use_min_rel, double* out) {
    AliState& st = *model->ali;
    const size_t n = (size_t)model->dm.P * nlev;
    const int blocks = (int)grid_for(n, 256, kConvBlocks);
    count_launch();
    convergence_kernel<<<blocks, 256, 0, model->stream>>>(a, b, tot, model->dm.P, nlev, st.prm.pop_prec,
                                                          st.prm.min_rel_pop_for_convergence, use_min_rel ? 1 : 0,
                                                          st.partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    count_launch();
    convergence_finalize<<<1, 32, 0, model->stream>>>(st.partial, blocks, out);
    return cudaGetLastError();
}

// Statistical equilibrium + corrections + convergence for every species, then the
// line data of all lines (Lines::iteration_using_statistical_equilibrium).
cudaError_t ali_launch_stateq_and_refresh(MgrModel* model, const double* lam) {
    AliState& st = *model->ali;
    for (size_t l = 0; l < st.species.size(); l++) {
        AliSpecies& sp = st.species[l];
        const uint32_t n = sp.view.nlev;
        const int wpb = 4;
        const size_t smem = (size_t)wpb * stateq_warp_doubles(sp.view) * sizeof(double);
        (void)n;
        cudaError_t e = cudaFuncSetAttribute(stateq_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        count_launch();
        stateq_kernel<<<grid_for(model->dm.P, wpb, model->sm_count * 8), wpb * 32, smem, model->stream>>>(
            model->dm, sp.view, lam, st.abundance, st.nspecs, st.prm.min_line_opacity, sp.view.pop, model->status);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        count_launch();
        negcorr_kernel<<<grid_for(model->dm.P, 128, model->sm_count * 8), 128, 0, model->stream>>>(
            model->dm, sp.view, st.prm.population_inversion_fraction);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        e = launch_convergence(model, sp.view.pop, sp.prev1, sp.view.tot, n, true, st.stats_dev + 3 * l);
        if (e != cudaSuccess) return e;
    }
    return ali_launch_line_refresh(model);
}

cudaError_t ali_launch_line_refresh(MgrModel* model) {
    AliState& st = *model->ali;
    for (auto& sp : st.species) {
        const size_t n = (size_t)model->dm.P * sp.view.nrad;
        count_launch();
        line_data_kernel<<<grid_for(n, 256, model->sm_count * 16), 256, 0, model->stream>>>(
            model->dm, sp.view, model->em, model->op, model->crit, st.prm.min_line_emissivity,
            st.prm.min_line_opacity);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = launch_line_tables(model);
    if (e == cudaSuccess) e = launch_nint_table(model);
    return e;
}

// History pushes of update_using_statistical_equilibrium / _acceleration:
// prev1 = pop; residuals.push_back(pop - populations.back()); populations.push_back(pop).
static cudaError_t history_push(MgrModel* model, AliSpecies& sp, bool set_prev1) {
    const size_t n = (size_t)model->dm.P * sp.view.nlev;
    cudaError_t e = cudaSuccess;
    if (set_prev1) e = cudaMemcpyAsync(sp.prev1, sp.view.pop, n * 8, cudaMemcpyDeviceToDevice, model->stream);
    if (e != cudaSuccess || !model->ali->keep_history) return e;
    double* r = sp.take_buffer();
    double* h = sp.take_buffer();
    if (!r || !h) {  // history longer than the pool (Ng never triggered): report instead of overwriting
        if (r) sp.free_bufs.push_back(r);
        if (h) sp.free_bufs.push_back(h);
        return cudaErrorMemoryAllocation;
    }
    count_launch();
    sub_kernel<<<grid_for(n, 256, model->sm_count * 16), 256, 0, model->stream>>>(r, sp.view.pop, sp.hist.back(), n);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    e = cudaMemcpyAsync(h, sp.view.pop, n * 8, cudaMemcpyDeviceToDevice, model->stream);
    sp.res.push_back(r);
    sp.hist.push_back(h);
    return e;
}

// Ng coefficients from the last `order` residuals, combined from the last `order`
// populations into `out`.
static cudaError_t ng_apply(MgrModel* model, AliSpecies& sp, int order, double* out) {
    AliState& st = *model->ali;
    const size_t n = (size_t)model->dm.P * sp.view.nlev;
    if (order < 1 || order > kMaxNgOrder || (size_t)order > sp.res.size() || (size_t)order > sp.hist.size())
        return cudaErrorInvalidValue;  // the history holds fewer iterations than the order asks for
    VecList r{}, h{};
    for (int i = 0; i < order; i++) {
        r.v[i] = sp.res[sp.res.size() - order + i];
        h.v[i] = sp.hist[sp.hist.size() - 1 - i];
    }
    const int blocks = (int)grid_for(n, 256, kGramBlocks);
    count_launch();
    gram_kernel<<<blocks, 256, 0, model->stream>>>(r, order, n, st.gram_partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    count_launch();
    ng_solve_kernel<<<1, 32, 0, model->stream>>>(st.gram_partial, blocks, order, st.coef);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    count_launch();
    ng_combine_kernel<<<grid_for(n, 256, model->sm_count * 16), 256, 0, model->stream>>>(out, h, st.coef, order, n);
    return cudaGetLastError();
}

cudaError_t ali_ng_step(MgrModel* model, int order) {
    AliState& st = *model->ali;
    for (size_t l = 0; l < st.species.size(); l++) {
        AliSpecies& sp = st.species[l];
        cudaError_t e = history_push(model, sp, true);
        if (e == cudaSuccess) e = ng_apply(model, sp, order, sp.view.pop);
        if (e != cudaSuccess) return e;
        sp.clear_residuals();
        sp.keep_last_population();
        count_launch();
        negcorr_kernel<<<grid_for(model->dm.P, 128, model->sm_count * 8), 128, 0, model->stream>>>(
            model->dm, sp.view, st.prm.population_inversion_fraction);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        e = launch_convergence(model, sp.view.pop, sp.prev1, sp.view.tot, sp.view.nlev, true, st.stats_dev + 3 * l);
        if (e != cudaSuccess) return e;
    }
    return ali_launch_line_refresh(model);
}

cudaError_t ali_ng_trial(MgrModel* model, int order) {
    AliState& st = *model->ali;
    for (size_t l = 0; l < st.species.size(); l++) {
        AliSpecies& sp = st.species[l];
        const size_t n = (size_t)model->dm.P * sp.view.nlev;
        cudaError_t e = history_push(model, sp, false);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(sp.trial_prev, sp.trial, n * 8, cudaMemcpyDeviceToDevice, model->stream);
        if (e == cudaSuccess) e = ng_apply(model, sp, order, sp.trial);
        if (e != cudaSuccess) return e;
        sp.pop_back_history();
        e = launch_convergence(model, sp.trial, sp.trial_prev, sp.view.tot, sp.view.nlev, false,
                               st.stats_dev + 3 * l);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t ali_history_push_all(MgrModel* model) {
    for (auto& sp : model->ali->species) {
        cudaError_t e = history_push(model, sp, true);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// ---------------------------------------------------------------------------------
// AliSpecies buffer pool
// ---------------------------------------------------------------------------------
double* AliSpecies::take_buffer() {
    if (free_bufs.empty()) return nullptr;  // the pool is sized for the longest history the loop keeps
    double* b = free_bufs.back();
    free_bufs.pop_back();
    return b;
}

void AliSpecies::clear_residuals() {
    for (double* b : res) free_bufs.push_back(b);
    res.clear();
}

void AliSpecies::keep_last_population() {
    while (hist.size() > 1) {
        free_bufs.push_back(hist.front());
        hist.erase(hist.begin());
    }
}

void AliSpecies::pop_back_history() {
    if (!res.empty()) {
        free_bufs.push_back(res.back());
        res.pop_back();
    }
    if (!hist.empty()) {
        free_bufs.push_back(hist.back());
        hist.pop_back();
    }
}

}  // namespace mgr

// ---------------------------------------------------------------------------------
// Host side: state management and the ALI loop
// ---------------------------------------------------------------------------------
namespace mgr {

void ali_free(MgrModel* model) {
    if (!model || !model->ali) return;
    AliState* st = model->ali;
    if (st->graph) cudaGraphExecDestroy(st->graph);
    for (cudaEvent_t& ev : st->ev)
        if (ev) cudaEventDestroy(ev);
    for (void* p : st->pool_allocs) cudaFree(p);
    for (void* p : st->allocs) cudaFree(p);
    if (st->stats_host) cudaFreeHost(st->stats_host);
    if (st->Jlin_buf) cudaFree(st->Jlin_buf);
    delete st;
    model->ali = nullptr;
}

template <typename T>
static cudaError_t ali_upload(AliState* st, cudaStream_t s, T** dst, const T* src, size_t n) {
    *dst = nullptr;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, (n ? n : 1) * sizeof(T));
    if (e != cudaSuccess) return e;
    st->allocs.push_back(p);
    *dst = static_cast<T*>(p);
    if (n && src) e = cudaMemcpyAsync(p, src, n * sizeof(T), cudaMemcpyHostToDevice, s);
    return e;
}

template <typename T>
static cudaError_t ali_alloc(AliState* st, T** dst, size_t n) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, (n ? n : 1) * sizeof(T));
    if (e == cudaSuccess) {
        st->allocs.push_back(p);
        *dst = static_cast<T*>(p);
    }
    return e;
}

// History buffers for Ng acceleration: enough for mem_limit + remove_N_its residuals
// and populations plus the trial step.
static cudaError_t ensure_pool(MgrModel* model, size_t per_species) {
    AliState& st = *model->ali;
    if (st.pool_per_species >= per_species) return cudaSuccess;
    for (auto& sp : st.species) {
        const size_t n = (size_t)model->dm.P * sp.view.nlev;
        for (size_t i = st.pool_per_species; i < per_species; i++) {
            void* p = nullptr;
            cudaError_t e = cudaMalloc(&p, n * sizeof(double));
            if (e != cudaSuccess) return e;
            st.pool_allocs.push_back(p);
            sp.free_bufs.push_back(static_cast<double*>(p));
        }
    }
    st.pool_per_species = per_species;
    return cudaSuccess;
}

static int read_stats(MgrModel* model) {
    AliState& st = *model->ali;
    cudaError_t e = cudaMemcpyAsync(st.stats_host, st.stats_dev, sizeof(double) * 3 * st.species.size(),
                                    cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "convergence statistics");
    return MGR_OK;
}

// One normal iteration after the history push: formal solve, Jeff, rate equations,
// corrections, convergence, line data.
// With a ray-pair shard, the formal solve covers the shard's ray pairs and the reduce
// function sums J and the ALO diagonal over the shards before Jeff.
// The memory-lean variant (compute_level_populations_sparse) sums the line-integrated
// J in the formal solve instead of J per frequency.
// Phase events (AliState::ev): recorded on the model's stream, i.e. as event nodes of
// the captured iteration.
static void mark(MgrModel* model, int i) {
    AliState& st = *model->ali;
    if (st.timing && cudaEventRecord(st.ev[i], model->stream) != cudaSuccess) {
        (void)cudaGetLastError();
        st.timing = false;
    }
}

// Adds the elapsed time between events a and b to phase_ms[k] (after the stream has
// been synchronised).
static void accumulate(AliState& st, int a, int b, int k) {
    if (!st.timing) return;
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, st.ev[a], st.ev[b]) != cudaSuccess) {
        (void)cudaGetLastError();
        st.timing = false;
        return;
    }
    st.phase_ms[k] += ms;
}

static cudaError_t normal_iteration_launches(MgrModel* model, int precision) {
    AliState& st = *model->ali;
    const DevModel& m = model->dm;
    double* J = st.sparse ? nullptr : model->J_scratch;
    double* Jlin = st.sparse ? st.Jlin_buf : nullptr;
    mark(model, 0);
    cudaError_t e = launch_fo2_range(model, precision, 0, m.P, J, nullptr, model->lam_scratch, model->work,
                                     model->work_bytes, model->shard_begin, model->shard_end, Jlin);
    if (e == cudaSuccess && model->shard_reduce) {
        double* Jr = st.sparse ? Jlin : J;
        const uint64_t nJ = st.sparse ? (uint64_t)m.P * m.L : (uint64_t)m.P * m.F;
        if (model->shard_reduce(model->shard_user, Jr, nJ, model->lam_scratch, (uint64_t)m.P * m.L,
                                (void*)model->stream) != 0) {
            st.reduce_failed = true;
            e = cudaErrorUnknown;
        }
    }
    mark(model, 1);
    if (e == cudaSuccess) e = ali_launch_jeff(model, J, model->lam_scratch, Jlin);
    mark(model, 2);
    if (e == cudaSuccess) e = ali_launch_stateq_and_refresh(model, model->lam_scratch);
    mark(model, 3);
    return e;
}

// Replays the captured iteration (capturing it on first use); falls back to direct
// launches if the capture is refused.
static cudaError_t normal_iteration(MgrModel* model, int precision) {
    AliState& st = *model->ali;
    if (st.graph && (st.graph_precision != precision || st.graph_sparse != (int)st.sparse)) {
        cudaGraphExecDestroy(st.graph);
        st.graph = nullptr;
    }
    const bool capture = !model->shard_reduce || model->shard_capturable;
    if (!st.graph && !st.graph_failed && capture) {
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(model->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const cudaError_t el = normal_iteration_launches(model, precision);
            e = cudaStreamEndCapture(model->stream, &g);
            if (el != cudaSuccess) e = el;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&st.graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            st.graph = nullptr;
            st.graph_failed = true;
        } else {
            st.graph_precision = precision;
            st.graph_sparse = (int)st.sparse;
        }
    }
    if (st.graph && capture) {
        count_launch();  // the graph's kernels were counted when captured; one more per replay is not kept exact
        return cudaGraphLaunch(st.graph, model->stream);
    }
    return normal_iteration_launches(model, precision);
}

void ali_shard_changed(MgrModel* model) {
    if (!model->ali) return;
    AliState& st = *model->ali;
    if (st.graph) cudaGraphExecDestroy(st.graph);
    st.graph = nullptr;
    st.graph_failed = false;
}

}  // namespace mgr

using namespace mgr;

extern "C" {

int mgr_model_set_species(MgrModel* model, uint32_t nlspecs, const MgrSpeciesDesc* species, uint32_t nspecs,
                          const double* abundance, const double* const* populations) {
    MGR_MODEL_DEVICE(model);
    if (!model || !species || nlspecs == 0 || !abundance || !populations || nspecs == 0) {
        set_error("mgr_model_set_species: null argument");
        return MGR_ERR_ARGUMENT;
    }
    const DevModel& dm = model->dm;
    uint32_t lines = 0;
    for (uint32_t l = 0; l < nlspecs; l++) {
        const MgrSpeciesDesc& d = species[l];
        if (d.nlev < 2 || d.nlev > (uint32_t)kMaxLevels || d.num >= nspecs || !d.energy || !d.weight || !d.irad ||
            !d.jrad || !d.A || !d.Bs || !d.Ba || !d.frequency || (d.ncolpar && !d.colpar) || !populations[l]) {
            set_error("mgr_model_set_species: species " + std::to_string(l) +
                      ": invalid sizes or null arrays (2 <= nlev <= 64, num < nspecs)");
            return MGR_ERR_ARGUMENT;
        }
        for (uint32_t k = 0; k < d.nrad; k++)
            if (d.irad[k] >= d.nlev || d.jrad[k] >= d.nlev) {
                set_error("mgr_model_set_species: radiative transition level out of range");
                return MGR_ERR_ARGUMENT;
            }
        for (uint32_t c = 0; c < d.ncolpar; c++) {
            const MgrCollisionPartnerDesc& cp = d.colpar[c];
            if (cp.ntmp == 0 || cp.num_col_partner >= nspecs || !cp.tmp || (cp.ncol && (!cp.icol || !cp.jcol || !cp.Cd || !cp.Ce))) {
                set_error("mgr_model_set_species: invalid collision partner");
                return MGR_ERR_ARGUMENT;
            }
            for (uint32_t k = 0; k < cp.ncol; k++)
                if (cp.icol[k] >= d.nlev || cp.jcol[k] >= d.nlev) {
                    set_error("mgr_model_set_species: collisional transition level out of range");
                    return MGR_ERR_ARGUMENT;
                }
        }
        lines += d.nrad;
    }
    if (lines != dm.L) {
        set_error("mgr_model_set_species: the species' radiative transitions must be the model's lines");
        return MGR_ERR_ARGUMENT;
    }
    ali_free(model);
    AliState* st = new AliState();
    model->ali = st;
    st->nspecs = nspecs;
    const uint32_t P = dm.P;
    cudaStream_t s = model->stream;
    double* dab = nullptr;
    cudaError_t e = ali_upload(st, s, &dab, abundance, (size_t)P * nspecs);
    st->abundance = dab;
    std::vector<double> tot(P);
    uint32_t offset = 0;
    for (uint32_t l = 0; l < nlspecs && e == cudaSuccess; l++) {
        const MgrSpeciesDesc& d = species[l];
        AliSpecies sp;
        SpeciesView& v = sp.view;
        v.num = d.num;
        v.nlev = d.nlev;
        v.nrad = d.nrad;
        v.line_offset = offset;
        v.ncolpar = d.ncolpar;
        v.ncol_total = 0;
        for (uint32_t c = 0; c < d.ncolpar; c++) v.ncol_total += d.colpar[c].ncol;
        offset += d.nrad;
        const double *en, *wt, *A, *Bs, *Ba, *fr;
        const uint32_t *ir, *jr;
        if ((e = ali_upload(st, s, (double**)&en, d.energy, d.nlev)) != cudaSuccess) break;
        if ((e = ali_upload(st, s, (double**)&wt, d.weight, d.nlev)) != cudaSuccess) break;
        if ((e = ali_upload(st, s, (uint32_t**)&ir, d.irad, d.nrad)) != cudaSuccess) break;
        if ((e = ali_upload(st, s, (uint32_t**)&jr, d.jrad, d.nrad)) != cudaSuccess) break;
        if ((e = ali_upload(st, s, (double**)&A, d.A, d.nrad)) != cudaSuccess) break;
        if ((e = ali_upload(st, s, (double**)&Bs, d.Bs, d.nrad)) != cudaSuccess) break;
        if ((e = ali_upload(st, s, (double**)&Ba, d.Ba, d.nrad)) != cudaSuccess) break;
        if ((e = ali_upload(st, s, (double**)&fr, d.frequency, d.nrad)) != cudaSuccess) break;
        v.energy = en; v.weight = wt; v.irad = ir; v.jrad = jr; v.A = A; v.Bs = Bs; v.Ba = Ba; v.freq = fr;
        std::vector<ColParView> cps(d.ncolpar);
        for (uint32_t c = 0; c < d.ncolpar && e == cudaSuccess; c++) {
            const MgrCollisionPartnerDesc& cd = d.colpar[c];
            ColParView& cv = cps[c];
            cv.num = cd.num_col_partner;
            cv.ortho_para = cd.ortho_para;
            cv.ncol = cd.ncol;
            cv.ntmp = cd.ntmp;
            const uint32_t *ic, *jc;
            const double *tm, *Cd, *Ce;
            if ((e = ali_upload(st, s, (uint32_t**)&ic, cd.icol, cd.ncol)) != cudaSuccess) break;
            if ((e = ali_upload(st, s, (uint32_t**)&jc, cd.jcol, cd.ncol)) != cudaSuccess) break;
            if ((e = ali_upload(st, s, (double**)&tm, cd.tmp, cd.ntmp)) != cudaSuccess) break;
            if ((e = ali_upload(st, s, (double**)&Cd, cd.Cd, (size_t)cd.ntmp * cd.ncol)) != cudaSuccess) break;
            if ((e = ali_upload(st, s, (double**)&Ce, cd.Ce, (size_t)cd.ntmp * cd.ncol)) != cudaSuccess) break;
            cv.icol = ic; cv.jcol = jc; cv.tmp = tm; cv.Cd = Cd; cv.Ce = Ce;
        }
        if (e != cudaSuccess) break;
        ColParView* dcp = nullptr;
        if ((e = ali_upload(st, s, &dcp, cps.data(), cps.size())) != cudaSuccess) break;
        v.cp = dcp;
        for (uint32_t p = 0; p < P; p++) tot[p] = abundance[(size_t)p * nspecs + d.num];
        const double* dtot = nullptr;
        if ((e = ali_upload(st, s, (double**)&dtot, tot.data(), P)) != cudaSuccess) break;
        v.tot = dtot;
        const size_t n = (size_t)P * d.nlev;
        if ((e = ali_upload(st, s, &v.pop, populations[l], n)) != cudaSuccess) break;
        if ((e = ali_alloc(st, &sp.prev1, n)) != cudaSuccess) break;
        if ((e = ali_alloc(st, &sp.trial, n)) != cudaSuccess) break;
        if ((e = ali_alloc(st, &sp.trial_prev, n)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(sp.trial, 0, n * 8, s)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(sp.trial_prev, 0, n * 8, s)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(sp.prev1, v.pop, n * 8, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) break;
        const size_t nk = (size_t)P * d.nrad;
        if ((e = ali_alloc(st, &v.Jlin, nk)) != cudaSuccess) break;
        if ((e = ali_alloc(st, &v.Jeff, nk)) != cudaSuccess) break;
        if ((e = ali_alloc(st, &v.Jdif, nk)) != cudaSuccess) break;
        st->species.push_back(sp);
    }
    if (e == cudaSuccess) e = ali_alloc(st, &st->partial, 3 * (size_t)kConvBlocks);
    if (e == cudaSuccess) e = ali_alloc(st, &st->stats_dev, 3 * (size_t)nlspecs);
    if (e == cudaSuccess) e = ali_alloc(st, &st->gram_partial, (size_t)kGramBlocks * kMaxNgOrder * kMaxNgOrder);
    if (e == cudaSuccess) e = ali_alloc(st, &st->coef, (size_t)kMaxNgOrder);
    if (e == cudaSuccess) e = cudaMallocHost(&st->stats_host, sizeof(double) * 3 * nlspecs);
    if (e == cudaSuccess) e = cudaMemsetAsync(st->stats_dev, 0, sizeof(double) * 3 * nlspecs, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        ali_free(model);
        return cuda_fail(e, "species upload");
    }
    return MGR_OK;
}

int mgr_compute_jeff(MgrModel* model, uint32_t l, double* Jlin, double* Jeff, double* Jdif) {
    MGR_MODEL_DEVICE(model);
    if (!model || !model->ali || l >= model->ali->species.size()) {
        set_error("mgr_compute_jeff: no species attached (mgr_model_set_species) or species index out of range");
        return MGR_ERR_ARGUMENT;
    }
    if (!model->last_J || !model->last_lam) {
        set_error("mgr_compute_jeff: needs a formal solve with the ALO diagonal first");
        return MGR_ERR_ARGUMENT;
    }
    cudaError_t e = ali_launch_jeff(model, model->last_J, model->last_lam, nullptr);
    const SpeciesView& v = model->ali->species[l].view;
    const size_t bytes = (size_t)model->dm.P * v.nrad * sizeof(double);
    if (e == cudaSuccess && Jlin) e = cudaMemcpyAsync(Jlin, v.Jlin, bytes, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && Jeff) e = cudaMemcpyAsync(Jeff, v.Jeff, bytes, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && Jdif) e = cudaMemcpyAsync(Jdif, v.Jdif, bytes, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "compute_Jeff");
    return MGR_OK;
}

int mgr_compute_level_populations(MgrModel* model, int precision, int use_ng, long max_iterations,
                                  const MgrAliParams* params, int* iterations, double* error_mean,
                                  double* error_max, uint32_t err_capacity) {
    MGR_MODEL_DEVICE(model);
    if (!model || !params || !model->ali) {
        set_error("mgr_compute_level_populations: null argument or no species attached (mgr_model_set_species)");
        return MGR_ERR_ARGUMENT;
    }
    if (precision != MGR_PRECISION_FP64 && precision != MGR_PRECISION_SPLIT) {
        set_error("mgr_compute_level_populations: unknown precision mode");
        return MGR_ERR_ARGUMENT;
    }
    if (!model->line_disc) {
        set_error("mgr_compute_level_populations: needs a line spectral discretisation");
        return MGR_ERR_UNSUPPORTED;
    }
    const MgrAliParams& prm = *params;
    if (prm.Ng_acceleration_mem_limit < 1 || prm.Ng_acceleration_mem_limit > (uint32_t)kMaxNgOrder ||
        prm.adaptive_Ng_acceleration_min_order < 1) {
        set_error("mgr_compute_level_populations: Ng_acceleration_mem_limit must be 1..16");
        return MGR_ERR_UNSUPPORTED;
    }
    AliState& st = *model->ali;
    st.prm = prm;
    st.keep_history = use_ng != 0;
    const DevModel& dm = model->dm;
    const size_t PF = (size_t)dm.P * dm.F, PL = (size_t)dm.P * dm.L;
    int rc = MGR_OK;
    auto scratch = [&](double** p, size_t* have, size_t bytes) -> int {
        if (*have >= bytes) return MGR_OK;
        if (*p) cudaFree(*p);
        *p = nullptr;
        *have = 0;
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, bytes);
        if (e != cudaSuccess) return cuda_fail(e, "scratch allocation");
        *p = static_cast<double*>(q);
        *have = bytes;
        if (st.graph) {  // captured pointers changed
            cudaGraphExecDestroy(st.graph);
            st.graph = nullptr;
        }
        return MGR_OK;
    };
    if ((rc = scratch(&model->J_scratch, &model->J_scratch_bytes, PF * 8)) != MGR_OK) return rc;
    if ((rc = scratch(&model->lam_scratch, &model->lam_scratch_bytes, PL * 8)) != MGR_OK) return rc;
    if (st.sparse && (rc = scratch(&st.Jlin_buf, &st.Jlin_bytes, PL * 8)) != MGR_OK) return rc;
    if ((rc = scratch(&model->work, &model->work_bytes, fo2_work_bytes(model, dm.P, true, true))) != MGR_OK) return rc;
    // Between two Ng steps the history grows by one residual and one population per
    // normal iteration (at most mem_limit + remove_N_its of them), plus the initial
    // population and one trial residual/population pair.
    cudaError_t e = ensure_pool(model, 2 * ((size_t)prm.Ng_acceleration_mem_limit + prm.Ng_acceleration_remove_N_its) + 6);
    if (e != cudaSuccess) return cuda_fail(e, "Ng history allocation");
    // populations.push_back(population) of update_using_LTE: the history starts at the current populations
    for (auto& sp : st.species) {
        sp.clear_residuals();
        while (!sp.hist.empty()) {
            sp.free_bufs.push_back(sp.hist.back());
            sp.hist.pop_back();
        }
        if (st.keep_history) {
            double* h = sp.take_buffer();
            if (!h) return cuda_fail(cudaErrorMemoryAllocation, "history");
            e = cudaMemcpyAsync(h, sp.view.pop, (size_t)dm.P * sp.view.nlev * 8, cudaMemcpyDeviceToDevice,
                                model->stream);
            if (e != cudaSuccess) return cuda_fail(e, "history");
            sp.hist.push_back(h);
        }
    }
    if ((e = ali_launch_line_refresh(model)) != cudaSuccess) return cuda_fail(e, "line data");
    for (double& t : st.phase_ms) t = 0.0;
    st.timing = true;
    for (cudaEvent_t& ev : st.ev)
        if (!ev && cudaEventCreate(&ev) != cudaSuccess) {
            (void)cudaGetLastError();
            st.timing = false;
        }

    const uint32_t nls = (uint32_t)st.species.size();
    const uint32_t skip = prm.Ng_acceleration_remove_N_its;
    int iteration = 0, iteration_normal = 0;
    bool some_not_converged = true;
    uint32_t nerr = 0;
    std::vector<double> fnc(nls, 0.0), rcm(nls, 0.0), rcmax(nls, 0.0);
    auto take_stats = [&]() {
        for (uint32_t l = 0; l < nls; l++) {
            fnc[l] = st.stats_host[3 * l];
            rcm[l] = st.stats_host[3 * l + 1];
            rcmax[l] = st.stats_host[3 * l + 2];
        }
    };
    while (some_not_converged && iteration < max_iterations) {
        bool use_step = false;
        int order = 0;
        if (!prm.use_adaptive_Ng_acceleration) {  // ng_acceleration_criterion<Default>
            if (use_ng && (uint32_t)iteration_normal == prm.Ng_acceleration_mem_limit + skip) {
                use_step = true;
                order = (int)prm.Ng_acceleration_mem_limit;
            }
        } else if (use_ng && (uint32_t)iteration_normal >= prm.adaptive_Ng_acceleration_min_order + skip) {
            double curr = 0.0, trial = 0.0;
            for (uint32_t l = 0; l < nls; l++) curr += prm.adaptive_Ng_acceleration_use_max_criterion ? rcmax[l] : rcm[l];
            const int trial_order = iteration_normal - (int)skip;
            if (trial_order > kMaxNgOrder) {
                set_error("mgr_compute_level_populations: adaptive Ng order above 16");
                return MGR_ERR_UNSUPPORTED;
            }
            if ((e = ali_ng_trial(model, trial_order)) != cudaSuccess) return cuda_fail(e, "Ng trial");
            if ((rc = read_stats(model)) != MGR_OK) return rc;
            take_stats();
            for (uint32_t l = 0; l < nls; l++) trial += prm.adaptive_Ng_acceleration_use_max_criterion ? rcmax[l] : rcm[l];
            if (trial < curr || (uint32_t)iteration_normal == prm.Ng_acceleration_mem_limit + skip) {
                use_step = true;
                order = trial_order;
            }
        }
        if (use_step) {
            mark(model, 4);
            if ((e = ali_ng_step(model, order)) != cudaSuccess) return cuda_fail(e, "Ng acceleration");
            mark(model, 5);
            if ((rc = read_stats(model)) != MGR_OK) return rc;
            accumulate(st, 4, 5, 3);
            take_stats();
            iteration_normal = 0;
            continue;
        }
        iteration++;
        some_not_converged = false;
        if ((e = ali_history_push_all(model)) != cudaSuccess) return cuda_fail(e, "population history");
        if ((e = normal_iteration(model, precision)) != cudaSuccess) {
            if (st.reduce_failed) {
                st.reduce_failed = false;
                set_error("mgr_compute_level_populations: the ray-shard reduce function failed");
                return MGR_ERR_CUDA;
            }
            return cuda_fail(e, "ALI iteration");
        }
        if ((rc = read_stats(model)) != MGR_OK) return rc;
        accumulate(st, 0, 1, 0);
        accumulate(st, 1, 2, 1);
        accumulate(st, 2, 3, 2);
        take_stats();
        iteration_normal++;
        for (uint32_t l = 0; l < nls; l++) {
            if (nerr < err_capacity) {
                if (error_mean) error_mean[nerr] = rcm[l];
                if (error_max) error_max[nerr] = rcmax[l];
            }
            nerr++;
            if (fnc[l] > 1.0 - prm.convergence_fraction) some_not_converged = true;
        }
    }
    model->last_J = st.sparse ? nullptr : model->J_scratch;
    model->last_Jlin = st.sparse ? st.Jlin_buf : nullptr;
    model->last_lam = model->lam_scratch;
    if (iterations) *iterations = iteration;
    int st_rc = MGR_OK;
    {
        int stw = 0;
        e = cudaMemcpyAsync(&stw, model->status, sizeof(int), cudaMemcpyDeviceToHost, model->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(model->status, 0, sizeof(int), model->stream);
        if (e != cudaSuccess) return cuda_fail(e, "status");
        if (stw) {
            set_error("mgr_compute_level_populations: a kernel reported a trace, capacity or non-finite/singular failure");
            st_rc = (stw & ST_TRACE) ? MGR_ERR_TRACE : (stw & ST_CAPACITY) ? MGR_ERR_CAPACITY : MGR_ERR_NONFINITE;
        }
    }
    return st_rc;
}

int mgr_ali_phase_times(MgrModel* model, double* ms) {
    MGR_MODEL_DEVICE(model);
    if (!model || !ms || !model->ali) {
        set_error("mgr_ali_phase_times: null argument or no species attached");
        return MGR_ERR_ARGUMENT;
    }
    const AliState& st = *model->ali;
    if (!st.timing) {
        set_error("mgr_ali_phase_times: no timed ALI loop on this model");
        return MGR_ERR_UNSUPPORTED;
    }
    for (int k = 0; k < 4; k++) ms[k] = st.phase_ms[k];
    return MGR_OK;
}

int mgr_compute_level_populations_sparse(MgrModel* model, int precision, int use_ng, long max_iterations,
                                         const MgrAliParams* params, int* iterations, double* error_mean,
                                         double* error_max, uint32_t err_capacity) {
    MGR_MODEL_DEVICE(model);
    if (!model || !model->ali) {
        set_error("mgr_compute_level_populations_sparse: null argument or no species attached (mgr_model_set_species)");
        return MGR_ERR_ARGUMENT;
    }
    model->ali->sparse = true;
    const int rc = mgr_compute_level_populations(model, precision, use_ng, max_iterations, params, iterations,
                                                 error_mean, error_max, err_capacity);
    model->ali->sparse = false;
    return rc;
}

int mgr_compute_jeff_sparse(MgrModel* model, uint32_t l, double* Jlin, double* Jeff) {
    MGR_MODEL_DEVICE(model);
    if (!model || !model->ali || l >= model->ali->species.size()) {
        set_error("mgr_compute_jeff_sparse: no species attached (mgr_model_set_species) or species index out of range");
        return MGR_ERR_ARGUMENT;
    }
    if (!model->last_Jlin || !model->last_lam) {
        set_error("mgr_compute_jeff_sparse: needs a memory-lean formal solve (mgr_formal_solve_fo2_sparse) first");
        return MGR_ERR_ARGUMENT;
    }
    cudaError_t e = ali_launch_jeff(model, nullptr, model->last_lam, model->last_Jlin);
    const SpeciesView& v = model->ali->species[l].view;
    const size_t bytes = (size_t)model->dm.P * v.nrad * sizeof(double);
    if (e == cudaSuccess && Jlin) e = cudaMemcpyAsync(Jlin, v.Jlin, bytes, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && Jeff) e = cudaMemcpyAsync(Jeff, v.Jeff, bytes, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "compute_Jeff_sparse");
    return MGR_OK;
}

int mgr_get_populations(MgrModel* model, uint32_t l, double* populations) {
    MGR_MODEL_DEVICE(model);
    if (!model || !model->ali || l >= model->ali->species.size() || !populations) {
        set_error("mgr_get_populations: invalid argument");
        return MGR_ERR_ARGUMENT;
    }
    const SpeciesView& v = model->ali->species[l].view;
    cudaError_t e = cudaMemcpyAsync(populations, v.pop, (size_t)model->dm.P * v.nlev * 8, cudaMemcpyDeviceToHost,
                                    model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "population read-back");
    return MGR_OK;
}

int mgr_get_line_data(MgrModel* model, double* emissivity, double* opacity) {
    MGR_MODEL_DEVICE(model);
    if (!model) {
        set_error("mgr_get_line_data: null model");
        return MGR_ERR_ARGUMENT;
    }
    const size_t bytes = (size_t)model->dm.P * model->dm.L * 8;
    cudaError_t e = cudaSuccess;
    if (emissivity) e = cudaMemcpyAsync(emissivity, model->em, bytes, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess && opacity) e = cudaMemcpyAsync(opacity, model->op, bytes, cudaMemcpyDeviceToHost, model->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(model->stream);
    if (e != cudaSuccess) return cuda_fail(e, "line data read-back");
    return MGR_OK;
}

}  // extern "C"
