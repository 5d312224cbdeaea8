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
// alo_off / alo_nr (n_off_diag > 0): the band elements of the non-local ALO, whose
// terms Ls * population(nr, upper) join the diagonal's in diff.
__global__ void jeff_kernel(DevModel m, SpeciesView s, const double* __restrict__ J, const double* __restrict__ lam,
                            const double* __restrict__ Jlin_in, const double* __restrict__ alo_off,
                            const uint32_t* __restrict__ alo_nr) {
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
        double diff = __dmul_rn(lam[(size_t)p * m.L + lid], s.pop[(size_t)p * s.nlev + s.irad[k]]);
        if (alo_off) {
            const size_t nb = (size_t)m.hnrays * 2 * m.n_off_diag;
            const size_t b0 = ((size_t)p * m.L + lid) * nb;
            for (size_t e = 0; e < nb; e++) {
                const double v = alo_off[b0 + e];
                if (v != 0.0) diff = __dadd_rn(diff, __dmul_rn(v, s.pop[(size_t)alo_nr[b0 + e] * s.nlev + s.irad[k]]));
            }
        }
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
// The global rate system with the non-local ALO (n_off_diag > 0;
// lineProducingSpecies.tpp:377-581 with the band elements of Lambda, :440-462): the
// element (nr, Ls) of point p's list for line k adds
//     v = -Ls opacity(p, k) / frequency(k)
// at row (p, lower k), column (nr, upper k) and -v at row (nr, upper k), column
// (nr, upper k) (rows of the last level are the normalisation).  Elements with nr = p
// stay inside p's block; the others couple blocks.  Unknowns are scaled by
// population_tot (xi = population / tot), and with B the block diagonal and E the
// coupling, the preconditioned system
//     xi + S^-1 B^-1 E S xi = S^-1 B^-1 b
// is solved by BiCGSTAB.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ double tot_scale(const SpeciesView& s, uint32_t p) {
    const double t = s.tot[p];
    return t > 0.0 ? t : 1.0;
}

// v of every band element of the species (thread per element): coef[(p nrad + k) nb + e].
__global__ void band_coef_kernel(DevModel m, SpeciesView s, const double* __restrict__ alo_off,
                                 double min_line_opacity, double* __restrict__ coef) {
    const size_t nb = (size_t)m.hnrays * 2 * m.n_off_diag;
    const size_t n = (size_t)m.P * s.nrad * nb;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const size_t pk = t / nb, e = t % nb;
        const uint32_t p = (uint32_t)(pk / s.nrad), k = (uint32_t)(pk % s.nrad);
        const double Ls = alo_off[((size_t)p * m.L + s.line_offset + k) * nb + e];
        coef[t] = (Ls == 0.0) ? 0.0
                              : -__ddiv_rn(__dmul_rn(Ls, opacity_of(s, s.pop + (size_t)p * s.nlev, k, min_line_opacity)),
                                           s.freq[k]);
    }
}

// Warp per point: the block (rate_block, the point's own band elements, the -v of
// other points' elements emitted by this point, gathered through the CSR), its LU
// factorisation with partial pivoting, and S^-1 B^-1 b as the right-hand side and the
// first iterate.  Shared memory per warp: stateq_warp_doubles.
__global__ void global_block_kernel(DevModel m, SpeciesView s, const double* __restrict__ lam,
                                    const double* __restrict__ abundance, uint32_t nspecs, double min_line_opacity,
                                    const double* __restrict__ coef, const uint32_t* __restrict__ alo_nr,
                                    const uint32_t* __restrict__ csr_off, const uint32_t* __restrict__ csr_ent,
                                    double* __restrict__ lu, uint32_t* __restrict__ piv, double* __restrict__ rhs,
                                    double* __restrict__ x, int* status) {
    extern __shared__ __align__(16) double smem_ali[];
    const uint32_t n = s.nlev, last = n - 1;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double* M = smem_ali + (size_t)w * stateq_warp_doubles(s);
    double* y = M + (size_t)n * n;
    double* R = y + n;
    const size_t nb = (size_t)m.hnrays * 2 * m.n_off_diag;
    for (uint32_t p = blockIdx.x * nw + w; p < m.P; p += gridDim.x * nw) {
        for (uint32_t i = lane; i < n * (n + 1); i += 32) M[i] = 0.0;
        __syncwarp();
        rate_block(m, s, p, lam, abundance, nspecs, min_line_opacity, M, R, lane);
        __syncwarp();
        if (lane == 0) {
            // the point's own elements with nr = p (an interpolated element of its own rays)
            for (uint32_t k = 0; k < s.nrad; k++) {
                const uint32_t I = s.irad[k], J = s.jrad[k];
                const size_t b0 = ((size_t)p * m.L + s.line_offset + k) * nb;
                for (size_t e = 0; e < nb; e++) {
                    const double v = coef[((size_t)p * s.nrad + k) * nb + e];
                    if (v == 0.0 || alo_nr[b0 + e] != p) continue;
                    if (J != last) M[(size_t)J * n + I] += v;
                    if (I != last) M[(size_t)I * n + I] -= v;
                }
            }
            // other points' elements emitted by p: -v on (p, upper)
            for (uint32_t lv = 0; lv < last; lv++) {
                const uint32_t row = p * n + lv;
                for (uint32_t j = csr_off[row]; j < csr_off[row + 1]; j++) M[(size_t)lv * n + lv] -= coef[csr_ent[j]];
            }
            for (uint32_t i = 0; i < n; i++) y[i] = 0.0;
            y[last] = s.tot[p];
        }
        __syncwarp();
        bool singular = false;
        uint32_t* pv = piv + (size_t)p * n;
        for (uint32_t c = 0; c < n; c++) {
            double best = -1.0;
            uint32_t pr = c;
            for (uint32_t r = c + lane; r < n; r += 32) {
                const double v = fabs(M[(size_t)r * n + c]);
                if (v > best) {
                    best = v;
                    pr = r;
                }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, off);
                const uint32_t op = __shfl_xor_sync(0xffffffffu, pr, off);
                if (ob > best || (ob == best && op < pr)) {
                    best = ob;
                    pr = op;
                }
            }
            if (!(best > 0.0)) {
                singular = true;
                break;
            }
            if (lane == 0) pv[c] = pr;
            if (pr != c) {
                for (uint32_t j = lane; j < n; j += 32) {
                    const double t = M[(size_t)c * n + j];
                    M[(size_t)c * n + j] = M[(size_t)pr * n + j];
                    M[(size_t)pr * n + j] = t;
                }
                __syncwarp();
            }
            const double d = M[(size_t)c * n + c];
            for (uint32_t r = c + 1; r < n; r++) {
                const double f = M[(size_t)r * n + c] / d;
                for (uint32_t j = c + 1 + lane; j < n; j += 32) M[(size_t)r * n + j] -= f * M[(size_t)c * n + j];
                __syncwarp();
                if (lane == 0) M[(size_t)r * n + c] = f;  // the multiplier, kept for the solves
                __syncwarp();
            }
        }
        if (singular) {
            if (lane == 0) atomicOr(status, ST_NONFINITE);
            continue;
        }
        for (uint32_t i = lane; i < n * n; i += 32) lu[(size_t)p * n * n + i] = M[i];
        if (lane == 0) {
            // B^-1 b with the factors just stored (b = tot e_last): the row interchanges in
            // order (they moved whole rows, multipliers included), then L and U
            for (uint32_t c = 0; c < n; c++) {
                const uint32_t pr = pv[c];
                if (pr != c) {
                    const double t = y[c];
                    y[c] = y[pr];
                    y[pr] = t;
                }
            }
            for (uint32_t c = 0; c < n; c++)
                for (uint32_t r = c + 1; r < n; r++) y[r] -= M[(size_t)r * n + c] * y[c];
            for (uint32_t c = n; c-- > 0;) {
                double acc = y[c];
                for (uint32_t j = c + 1; j < n; j++) acc -= M[(size_t)c * n + j] * y[j];
                y[c] = acc / M[(size_t)c * n + c];
            }
            const double sc = tot_scale(s, p);
            for (uint32_t i = 0; i < n; i++) {
                rhs[(size_t)p * n + i] = y[i] / sc;
                x[(size_t)p * n + i] = y[i] / sc;
            }
        }
        __syncwarp();
    }
}

// out = xi + S^-1 B^-1 E S xi, warp per point: lanes gather the coupling of the
// point's elements with nr != p (rows of the lower levels) into per-lane partial rows,
// summed in lane order; lane 0 applies the stored LU factors.  Shared memory per warp:
// 33 nlev doubles.
__global__ void global_op_kernel(DevModel m, SpeciesView s, const double* __restrict__ coef,
                                 const uint32_t* __restrict__ alo_nr, const double* __restrict__ lu,
                                 const uint32_t* __restrict__ piv, const double* __restrict__ xi,
                                 double* __restrict__ out) {
    extern __shared__ __align__(16) double smem_ali[];
    const uint32_t n = s.nlev, last = n - 1;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double* part = smem_ali + (size_t)w * 33 * n;  // [32][n] partial rows, then [n] the sum
    double* c = part + (size_t)32 * n;
    const size_t nb = (size_t)m.hnrays * 2 * m.n_off_diag;
    const size_t ne = (size_t)s.nrad * nb;
    for (uint32_t p = blockIdx.x * nw + w; p < m.P; p += gridDim.x * nw) {
        for (uint32_t i = 0; i < n; i++) part[(size_t)lane * n + i] = 0.0;
        for (size_t t = lane; t < ne; t += 32) {
            const uint32_t k = (uint32_t)(t / nb);
            const size_t e = t % nb;
            const double v = coef[(size_t)p * ne + t];
            const uint32_t nr = alo_nr[((size_t)p * m.L + s.line_offset + k) * nb + e];
            if (v == 0.0 || nr == p || s.jrad[k] == last) continue;
            part[(size_t)lane * n + s.jrad[k]] += v * (tot_scale(s, nr) * xi[(size_t)nr * n + s.irad[k]]);
        }
        __syncwarp();
        if (lane == 0) {
            for (uint32_t i = 0; i < n; i++) {
                double acc = 0.0;
                for (int l = 0; l < 32; l++) acc += part[(size_t)l * n + i];
                c[i] = acc;
            }
            const double* M = lu + (size_t)p * n * n;
            const uint32_t* pv = piv + (size_t)p * n;
            for (uint32_t cc = 0; cc < n; cc++) {
                const uint32_t pr = pv[cc];
                if (pr != cc) {
                    const double t = c[cc];
                    c[cc] = c[pr];
                    c[pr] = t;
                }
            }
            for (uint32_t cc = 0; cc < n; cc++)
                for (uint32_t r = cc + 1; r < n; r++) c[r] -= M[(size_t)r * n + cc] * c[cc];
            for (uint32_t cc = n; cc-- > 0;) {
                double acc = c[cc];
                for (uint32_t j = cc + 1; j < n; j++) acc -= M[(size_t)cc * n + j] * c[j];
                c[cc] = acc / M[(size_t)cc * n + cc];
            }
            const double sc = tot_scale(s, p);
            for (uint32_t i = 0; i < n; i++) out[(size_t)p * n + i] = xi[(size_t)p * n + i] + c[i] / sc;
        }
        __syncwarp();
    }
}

// Partial sums of a.b (mode 0) or partial maxima of |a| (mode 1) over blocks; then
// reduce_finalize sums / maximises them in block order.
__global__ void dot_kernel(const double* __restrict__ a, const double* __restrict__ b, size_t n, int mode,
                           double* __restrict__ partial) {
    __shared__ double acc[256];
    double v = 0.0;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        v = mode ? fmax(v, fabs(a[t])) : v + a[t] * b[t];
    acc[threadIdx.x] = v;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            acc[threadIdx.x] = mode ? fmax(acc[threadIdx.x], acc[threadIdx.x + h]) : acc[threadIdx.x] + acc[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = acc[0];
}

__global__ void reduce_finalize(const double* __restrict__ partial, int nblocks, int mode, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double v = 0.0;
    for (int b = 0; b < nblocks; b++) v = mode ? fmax(v, partial[b]) : v + partial[b];
    *out = v;
}

// out = a + alpha b + beta c (any of b, c may be null).
__global__ void axpby_kernel(double* __restrict__ out, const double* __restrict__ a, double alpha,
                             const double* __restrict__ b, double beta, const double* __restrict__ c, size_t n) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        double v = a[t];
        if (b) v += alpha * b[t];
        if (c) v += beta * c[t];
        out[t] = v;
    }
}

// population = tot xi
__global__ void unscale_kernel(SpeciesView s, uint32_t P, const double* __restrict__ xi) {
    const size_t n = (size_t)P * s.nlev;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        s.pop[t] = xi[t] * tot_scale(s, (uint32_t)(t / s.nlev));
}

// CSR of the band elements by the row whose diagonal their -v reaches: (element point
// nr, upper level), for nr != p and upper levels below the last.  Element index t is
// the coef index ((p nrad + k) hnrays 2K + e).
__device__ __forceinline__ bool csr_row_of(const DevModel& m, const SpeciesView& s, const uint32_t* alo_nr, size_t t,
                                           size_t nb, size_t* row) {
    const size_t pk = t / nb, e = t % nb;
    const uint32_t p = (uint32_t)(pk / s.nrad), k = (uint32_t)(pk % s.nrad);
    const uint32_t nr = alo_nr[((size_t)p * m.L + s.line_offset + k) * nb + e];
    if (nr == p || s.irad[k] == s.nlev - 1) return false;
    *row = (size_t)nr * s.nlev + s.irad[k];
    return true;
}

__global__ void csr_count_kernel(DevModel m, SpeciesView s, const uint32_t* __restrict__ alo_nr,
                                 uint32_t* __restrict__ cnt) {
    const size_t nb = (size_t)m.hnrays * 2 * m.n_off_diag;
    const size_t n = (size_t)m.P * s.nrad * nb;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        size_t row;
        if (csr_row_of(m, s, alo_nr, t, nb, &row)) atomicAdd(&cnt[row], 1u);
    }
}

// Exclusive scan of cnt [rows] into off [rows + 1], one block of 1024 threads (each a
// contiguous range); off[rows] is the total.
__global__ void csr_scan_kernel(const uint32_t* __restrict__ cnt, size_t rows, uint32_t* __restrict__ off) {
    __shared__ unsigned long long part[1024];
    const size_t per = (rows + blockDim.x - 1) / blockDim.x;
    const size_t b = (size_t)threadIdx.x * per;
    const size_t e = b + per < rows ? b + per : rows;
    unsigned long long sum = 0;
    for (size_t i = b; i < e; i++) sum += cnt[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long acc = 0;
        for (unsigned i = 0; i < blockDim.x; i++) {
            const unsigned long long v = part[i];
            part[i] = acc;
            acc += v;
        }
        off[rows] = (uint32_t)acc;
    }
    __syncthreads();
    unsigned long long acc = part[threadIdx.x];
    for (size_t i = b; i < e; i++) {
        off[i] = (uint32_t)acc;
        acc += cnt[i];
    }
}

__global__ void csr_fill_kernel(DevModel m, SpeciesView s, const uint32_t* __restrict__ alo_nr,
                                uint32_t* __restrict__ cursor, uint32_t* __restrict__ ent) {
    const size_t nb = (size_t)m.hnrays * 2 * m.n_off_diag;
    const size_t n = (size_t)m.P * s.nrad * nb;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        size_t row;
        if (csr_row_of(m, s, alo_nr, t, nb, &row)) ent[atomicAdd(&cursor[row], 1u)] = (uint32_t)t;
    }
}

// Thread per row: the row's entries in ascending element order, so that the sums over
// them do not depend on the order of the atomic fill.
__global__ void csr_sort_kernel(const uint32_t* __restrict__ off, size_t rows, uint32_t* __restrict__ ent) {
    for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (size_t)gridDim.x * blockDim.x) {
        const uint32_t b = off[r], e = off[r + 1];
        for (uint32_t i = b + 1; i < e; i++) {
            const uint32_t v = ent[i];
            uint32_t j = i;
            while (j > b && ent[j - 1] > v) {
                ent[j] = ent[j - 1];
                j--;
            }
            ent[j] = v;
        }
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

cudaError_t ali_launch_jeff(MgrModel* model, const double* J, const double* lam, const double* Jlin,
                            const double* alo_off, const uint32_t* alo_nr) {
    const bool bands = alo_off && alo_nr && !Jlin && model->dm.n_off_diag > 0;
    for (auto& sp : model->ali->species) {
        const size_t n = (size_t)model->dm.P * sp.view.nrad;
        count_launch();
        jeff_kernel<<<grid_for(n, 256, model->sm_count * 16), 256, 0, model->stream>>>(
            model->dm, sp.view, J, lam, Jlin, bands ? alo_off : nullptr, bands ? alo_nr : nullptr);
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

static void grs_free(GlobalRate& g);

void ali_free(MgrModel* model) {
    if (!model || !model->ali) return;
    AliState* st = model->ali;
    if (st->graph) cudaGraphExecDestroy(st->graph);
    for (cudaEvent_t& ev : st->ev)
        if (ev) cudaEventDestroy(ev);
    for (void* p : st->pool_allocs) cudaFree(p);
    for (void* p : st->allocs) cudaFree(p);
    grs_free(st->grs);
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
    // External: inside a stream capture a plain record only orders the graph's nodes;
    // an external record node takes the timestamp on every replay
    if (!st.timing) return;
    // the external flag is for captures only: outside one the record is a plain one
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(model->stream, &cs);
    if (e == cudaSuccess)
        e = cudaEventRecordWithFlags(st.ev[i], model->stream,
                                     cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        st.timing = false;
        st.timing_error = std::string("event record ") + std::to_string(i) + ": " + cudaGetErrorString(e);
    }
}

// Adds the elapsed time between events a and b to phase_ms[k] (after the stream has
// been synchronised).
static void accumulate(AliState& st, int a, int b, int k) {
    if (!st.timing) return;
    float ms = 0.0f;
    const cudaError_t e = cudaEventElapsedTime(&ms, st.ev[a], st.ev[b]);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        st.timing = false;
        st.timing_error = std::string("elapsed time ") + std::to_string(a) + "-" + std::to_string(b) + ": " +
                          cudaGetErrorString(e);
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

// ---------------------------------------------------------------------------------
// The global rate system with the non-local ALO (n_off_diag > 0)
// ---------------------------------------------------------------------------------
template <typename T>
static cudaError_t grs_alloc(GlobalRate& g, T** dst, size_t n) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, (n ? n : 1) * sizeof(T));
    if (e == cudaSuccess) {
        g.allocs.push_back(p);
        *dst = static_cast<T*>(p);
    }
    return e;
}

static void grs_free(GlobalRate& g) {
    for (void* p : g.allocs) cudaFree(p);
    if (g.red_host) cudaFreeHost(g.red_host);
    g = GlobalRate();
}

static size_t band_slots(const DevModel& m) { return (size_t)m.hnrays * 2 * m.n_off_diag; }

// Device state of the global solve and of the band elements, sized for the model.
static cudaError_t ensure_global(MgrModel* model) {
    AliState& st = *model->ali;
    GlobalRate& g = st.grs;
    const DevModel& m = model->dm;
    const size_t nb = band_slots(m);
    const size_t alo = (size_t)m.P * m.L * nb;
    cudaError_t e = cudaSuccess;
    auto grow = [](double** p, size_t* have, size_t bytes) -> cudaError_t {
        if (*have >= bytes) return cudaSuccess;
        if (*p) cudaFree(*p);
        *p = nullptr;
        *have = 0;
        const cudaError_t r = cudaMalloc(p, bytes);
        if (r == cudaSuccess) *have = bytes;
        return r;
    };
    if ((e = grow(&model->alo_scratch, &model->alo_scratch_bytes, alo * 8)) != cudaSuccess) return e;
    if ((e = grow(&model->alo_nr_scratch, &model->alo_nr_scratch_bytes, alo * 4)) != cudaSuccess) return e;
    st.alo_off = model->alo_scratch;
    st.alo_nr = reinterpret_cast<uint32_t*>(model->alo_nr_scratch);
    uint32_t nmax = 0, rmax = 0;
    for (auto& sp : st.species) {
        nmax = std::max(nmax, sp.view.nlev);
        rmax = std::max(rmax, sp.view.nrad);
    }
    const size_t n = (size_t)m.P * nmax, ncoef = (size_t)m.P * rmax * nb;
    if (g.cap_n >= n && g.cap_coef >= ncoef && g.csr_off.size() == st.species.size()) return cudaSuccess;
    grs_free(g);
    if ((e = grs_alloc(g, &g.lu, (size_t)m.P * nmax * nmax)) != cudaSuccess) return e;
    if ((e = grs_alloc(g, &g.piv, n)) != cudaSuccess) return e;
    if ((e = grs_alloc(g, &g.coef, ncoef)) != cudaSuccess) return e;
    if ((e = grs_alloc(g, &g.vec, 9 * n)) != cudaSuccess) return e;
    if ((e = grs_alloc(g, &g.red, (size_t)kConvBlocks + 8)) != cudaSuccess) return e;
    if ((e = grs_alloc(g, &g.cursor, n + 1)) != cudaSuccess) return e;
    if ((e = cudaMallocHost(&g.red_host, 8 * sizeof(double))) != cudaSuccess) return e;
    g.csr_off.assign(st.species.size(), nullptr);
    g.csr_ent.assign(st.species.size(), nullptr);
    g.csr_cap.assign(st.species.size(), 0);
    for (size_t l = 0; l < st.species.size(); l++)
        if ((e = grs_alloc(g, &g.csr_off[l], (size_t)m.P * st.species[l].view.nlev + 1)) != cudaSuccess) return e;
    g.cap_n = n;
    g.cap_coef = ncoef;
    g.built = false;
    return cudaSuccess;
}

// The CSR of every species from the band elements' points of the latest banded solve.
static cudaError_t build_csr(MgrModel* model) {
    AliState& st = *model->ali;
    GlobalRate& g = st.grs;
    const DevModel& m = model->dm;
    cudaStream_t s = model->stream;
    for (size_t l = 0; l < st.species.size(); l++) {
        const SpeciesView& v = st.species[l].view;
        const size_t rows = (size_t)m.P * v.nlev;
        const size_t n = (size_t)m.P * v.nrad * band_slots(m);
        cudaError_t e = cudaMemsetAsync(g.cursor, 0, (rows + 1) * 4, s);
        if (e != cudaSuccess) return e;
        count_launch();
        csr_count_kernel<<<grid_for(n, 256, model->sm_count * 16), 256, 0, s>>>(m, v, st.alo_nr, g.cursor);
        count_launch();
        csr_scan_kernel<<<1, 1024, 0, s>>>(g.cursor, rows, g.csr_off[l]);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        uint32_t total = 0;
        if ((e = cudaMemcpyAsync(&total, g.csr_off[l] + rows, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        if (g.csr_cap[l] < total) {
            if ((e = grs_alloc(g, &g.csr_ent[l], total)) != cudaSuccess) return e;
            g.csr_cap[l] = total;
        }
        if ((e = cudaMemcpyAsync(g.cursor, g.csr_off[l], rows * 4, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
            return e;
        count_launch();
        csr_fill_kernel<<<grid_for(n, 256, model->sm_count * 16), 256, 0, s>>>(m, v, st.alo_nr, g.cursor,
                                                                              g.csr_ent[l]);
        count_launch();
        csr_sort_kernel<<<grid_for(rows, 128, model->sm_count * 8), 128, 0, s>>>(g.csr_off[l], rows, g.csr_ent[l]);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    g.built = true;
    return cudaSuccess;
}

// Dot product (mode 0) or max-norm (mode 1, b unused) into result slot `slot`.
static cudaError_t grs_reduce(MgrModel* model, const double* a, const double* b, size_t n, int mode, int slot) {
    GlobalRate& g = model->ali->grs;
    const int blocks = (int)grid_for(n, 256, kConvBlocks);
    count_launch();
    dot_kernel<<<blocks, 256, 0, model->stream>>>(a, b ? b : a, n, mode, g.red);
    count_launch();
    reduce_finalize<<<1, 32, 0, model->stream>>>(g.red, blocks, mode, g.red + kConvBlocks + slot);
    return cudaGetLastError();
}

static cudaError_t grs_read(MgrModel* model, int nslots) {
    GlobalRate& g = model->ali->grs;
    cudaError_t e = cudaMemcpyAsync(g.red_host, g.red + kConvBlocks, nslots * sizeof(double),
                                    cudaMemcpyDeviceToHost, model->stream);
    return e == cudaSuccess ? cudaStreamSynchronize(model->stream) : e;
}

static cudaError_t grs_axpby(MgrModel* model, double* out, const double* a, double alpha, const double* b,
                             double beta, const double* c, size_t n) {
    count_launch();
    axpby_kernel<<<grid_for(n, 256, model->sm_count * 16), 256, 0, model->stream>>>(out, a, alpha, b, beta, c, n);
    return cudaGetLastError();
}

static cudaError_t grs_op(MgrModel* model, const SpeciesView& v, const double* xi, double* out) {
    GlobalRate& g = model->ali->grs;
    const int wpb = 4;
    const size_t smem = (size_t)wpb * 33 * v.nlev * sizeof(double);
    cudaError_t e = cudaFuncSetAttribute(global_op_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    count_launch();
    global_op_kernel<<<grid_for(model->dm.P, wpb, model->sm_count * 8), wpb * 32, smem, model->stream>>>(
        model->dm, v, g.coef, model->ali->alo_nr, g.lu, g.piv, xi, out);
    return cudaGetLastError();
}

constexpr double kRateTol = 1.0e-13;   // BiCGSTAB: max-norm residual relative to the right-hand side
constexpr double kRateAccept = 1.0e-9;  // larger final residuals fail the solve
constexpr int kRateMaxIt = 200;

// The rate system of species l with the band elements of the latest banded solve:
// populations(new) = tot xi, xi from BiCGSTAB on xi + S^-1 B^-1 E S xi = S^-1 B^-1 b
// started at the block-Jacobi solution.
static int global_stateq(MgrModel* model, size_t l) {
    AliState& st = *model->ali;
    GlobalRate& g = st.grs;
    AliSpecies& sp = st.species[l];
    const SpeciesView& v = sp.view;
    const DevModel& m = model->dm;
    cudaStream_t s = model->stream;
    const size_t n = (size_t)m.P * v.nlev;
    const size_t ncoef = (size_t)m.P * v.nrad * band_slots(m);
    double *x = g.vec, *r = x + n, *rh = r + n, *pp = rh + n, *vv = pp + n, *ss = vv + n, *tt = ss + n,
           *rhs = tt + n;
    count_launch();
    band_coef_kernel<<<grid_for(ncoef, 256, model->sm_count * 16), 256, 0, s>>>(m, v, st.alo_off,
                                                                               st.prm.min_line_opacity, g.coef);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "band coefficients");
    const int wpb = 4;
    const size_t smem = (size_t)wpb * stateq_warp_doubles(v) * sizeof(double);
    if ((e = cudaFuncSetAttribute(global_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
        cudaSuccess)
        return cuda_fail(e, "rate blocks");
    count_launch();
    global_block_kernel<<<grid_for(m.P, wpb, model->sm_count * 8), wpb * 32, smem, s>>>(
        m, v, model->lam_scratch, st.abundance, st.nspecs, st.prm.min_line_opacity, g.coef, st.alo_nr,
        g.csr_off[l], g.csr_ent[l], g.lu, g.piv, rhs, x, model->status);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "rate blocks");
    // r = rhs - A x, rhat = r
    if ((e = grs_op(model, v, x, tt)) != cudaSuccess) return cuda_fail(e, "rate operator");
    if ((e = grs_axpby(model, r, rhs, -1.0, tt, 0.0, nullptr, n)) != cudaSuccess) return cuda_fail(e, "BiCGSTAB");
    if ((e = cudaMemcpyAsync(rh, r, n * 8, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return cuda_fail(e, "BiCGSTAB");
    if ((e = grs_reduce(model, rhs, nullptr, n, 1, 0)) != cudaSuccess) return cuda_fail(e, "BiCGSTAB");
    if ((e = grs_read(model, 1)) != cudaSuccess) return cuda_fail(e, "BiCGSTAB");
    const double bn = g.red_host[0] > 0.0 ? g.red_host[0] : 1.0;
    double rho = 1.0, alpha = 1.0, omega = 1.0, rn = 0.0;
    bool first = true;
    int it = 0;
    for (;; it++) {
        if ((e = grs_reduce(model, r, nullptr, n, 1, 0)) != cudaSuccess) break;
        if ((e = grs_reduce(model, rh, r, n, 0, 1)) != cudaSuccess) break;
        if ((e = grs_read(model, 2)) != cudaSuccess) break;
        rn = g.red_host[0] / bn;
        const double rho_new = g.red_host[1];
        if (!(rn > kRateTol) || it >= kRateMaxIt || rho_new == 0.0) break;
        // p = r + beta (p - omega v)
        if (first) {
            if ((e = cudaMemcpyAsync(pp, r, n * 8, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) break;
            first = false;
        } else {
            const double beta = (rho_new / rho) * (alpha / omega);
            if ((e = grs_axpby(model, pp, r, beta, pp, -beta * omega, vv, n)) != cudaSuccess) break;
        }
        rho = rho_new;
        if ((e = grs_op(model, v, pp, vv)) != cudaSuccess) break;
        if ((e = grs_reduce(model, rh, vv, n, 0, 0)) != cudaSuccess) break;
        if ((e = grs_read(model, 1)) != cudaSuccess) break;
        if (g.red_host[0] == 0.0) break;
        alpha = rho / g.red_host[0];
        // s = r - alpha v; t = A s; omega = (t, s) / (t, t)
        if ((e = grs_axpby(model, ss, r, -alpha, vv, 0.0, nullptr, n)) != cudaSuccess) break;
        if ((e = grs_op(model, v, ss, tt)) != cudaSuccess) break;
        if ((e = grs_reduce(model, tt, ss, n, 0, 0)) != cudaSuccess) break;
        if ((e = grs_reduce(model, tt, tt, n, 0, 1)) != cudaSuccess) break;
        if ((e = grs_read(model, 2)) != cudaSuccess) break;
        omega = g.red_host[1] > 0.0 ? g.red_host[0] / g.red_host[1] : 0.0;
        // x += alpha p + omega s; r = s - omega t
        if ((e = grs_axpby(model, x, x, alpha, pp, omega, ss, n)) != cudaSuccess) break;
        if ((e = grs_axpby(model, r, ss, -omega, tt, 0.0, nullptr, n)) != cudaSuccess) break;
        if (omega == 0.0) {
            it++;
            if ((e = grs_reduce(model, r, nullptr, n, 1, 0)) != cudaSuccess) break;
            if ((e = grs_read(model, 1)) != cudaSuccess) break;
            rn = g.red_host[0] / bn;
            break;
        }
    }
    if (e != cudaSuccess) return cuda_fail(e, "BiCGSTAB");
    g.last_iterations = it;
    g.last_residual = rn;
    if (!(rn <= kRateAccept)) {
        set_error("mgr_compute_level_populations: the global rate system (n_off_diag > 0) did not converge: "
                  "relative residual " + std::to_string(rn) + " after " + std::to_string(it) + " iterations");
        return MGR_ERR_NONFINITE;
    }
    count_launch();
    unscale_kernel<<<grid_for(n, 256, model->sm_count * 16), 256, 0, s>>>(v, m.P, x);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "populations");
    return MGR_OK;
}

// One normal iteration with the non-local ALO: the banded FP64 formal solve, Jeff with
// the band elements, the global rate system per species, corrections, convergence and
// the line data.  Launched directly (the rate solve reads its scalars on the host).
static int banded_iteration(MgrModel* model) {
    AliState& st = *model->ali;
    const DevModel& m = model->dm;
    mark(model, 0);
    cudaError_t e = launch_fo2_range(model, MGR_PRECISION_FP64, 0, m.P, model->J_scratch, nullptr,
                                     model->lam_scratch, model->work, model->work_bytes, 0, 0xffffffffu, nullptr,
                                     nullptr, nullptr, st.alo_off, st.alo_nr);
    mark(model, 1);
    if (e == cudaSuccess)
        e = ali_launch_jeff(model, model->J_scratch, model->lam_scratch, nullptr, st.alo_off, st.alo_nr);
    mark(model, 2);
    if (e == cudaSuccess && !st.grs.built) e = build_csr(model);
    if (e != cudaSuccess) return cuda_fail(e, "banded ALI iteration");
    for (size_t l = 0; l < st.species.size(); l++) {
        AliSpecies& sp = st.species[l];
        const int rc = global_stateq(model, l);
        if (rc != MGR_OK) return rc;
        count_launch();
        negcorr_kernel<<<grid_for(m.P, 128, model->sm_count * 8), 128, 0, model->stream>>>(
            m, sp.view, st.prm.population_inversion_fraction);
        if ((e = cudaGetLastError()) == cudaSuccess)
            e = launch_convergence(model, sp.view.pop, sp.prev1, sp.view.tot, sp.view.nlev, true, st.stats_dev + 3 * l);
        if (e != cudaSuccess) return cuda_fail(e, "banded ALI iteration");
    }
    e = ali_launch_line_refresh(model);
    mark(model, 3);
    return e == cudaSuccess ? MGR_OK : cuda_fail(e, "line data");
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
    cudaError_t e = ali_launch_jeff(model, model->last_J, model->last_lam, nullptr, model->last_alo_off,
                                    model->last_alo_nr);
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
    const DevModel& dm = model->dm;
    const bool bands = dm.n_off_diag > 0;
    if (bands) {
        if (st.sparse) {  // lineProducingSpecies.tpp:592-593
            set_error("mgr_compute_level_populations_sparse: n_off_diag != 0, so the sparse update cannot be used");
            return MGR_ERR_UNSUPPORTED;
        }
        if (precision != MGR_PRECISION_FP64) {
            set_error("mgr_compute_level_populations: n_off_diag > 0 runs the banded FP64 formal solve "
                      "(precision must be FP64)");
            return MGR_ERR_UNSUPPORTED;
        }
        if (model->shard_reduce || model->shard_begin != 0 || model->shard_end < dm.hnrays) {
            set_error("mgr_compute_level_populations: n_off_diag > 0 needs every ray pair on this model "
                      "(no ray-pair shard)");
            return MGR_ERR_UNSUPPORTED;
        }
        if ((size_t)dm.P * dm.L * band_slots(dm) >= ((size_t)1 << 32)) {
            set_error("mgr_compute_level_populations: more than 2^32 band elements");
            return MGR_ERR_UNSUPPORTED;
        }
    }
    st.prm = prm;
    st.keep_history = use_ng != 0;
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
    if (bands) {
        cudaError_t eg = ensure_global(model);
        if (eg != cudaSuccess) return cuda_fail(eg, "global rate system allocation");
        st.grs.built = false;  // the CSR follows the first banded solve of this call
    }
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
    st.timing_error.clear();
    for (cudaEvent_t& ev : st.ev)
        if (!ev) {
            const cudaError_t ec = cudaEventCreate(&ev);
            if (ec != cudaSuccess) {
                (void)cudaGetLastError();
                st.timing = false;
                st.timing_error = std::string("event create: ") + cudaGetErrorString(ec);
            }
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
        if (bands) {
            if ((rc = banded_iteration(model)) != MGR_OK) return rc;
        } else if ((e = normal_iteration(model, precision)) != cudaSuccess) {
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
    model->last_alo_off = bands ? st.alo_off : nullptr;
    model->last_alo_nr = bands ? st.alo_nr : nullptr;
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
        set_error("mgr_ali_phase_times: no timed ALI loop on this model" +
                  (st.timing_error.empty() ? std::string() : " (" + st.timing_error + ")"));
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
