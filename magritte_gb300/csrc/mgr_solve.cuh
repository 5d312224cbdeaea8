// Ray-pair formal solve: warp-cooperative trace and the per-lane two-sided
// second-order Feautrier elimination.
//
// Reference: Solver::solve_feautrier_order_2 (src/solver/solver.tpp:458-540 driver,
// :2193-2318 per frequency), Solver::trace_ray_for_line (:773-800),
// Solver::set_data_for_line (:1057-1097), compute_source_dtau (:2139-2186),
// compute_S_dtau_line_integrated (:1878-2111), compute_dtau_single_line (:2374-2455),
// update_Lambda (:1760-1800).
//
// The reference eliminates forward over the whole ray pair and back-substitutes down
// to the origin, keeping FF/FI/Su/A/C/... arrays per element.  Here each lane
// eliminates from both ends toward the origin (the same economical (1+B)/C
// recurrences, Rybicki & Hummer 1991: F from the first element, G from the last)
// and combines them at the origin:
//     u[c]      = (Su_c (1 + F_c) + Sb_{c+1}) / (F_c + G_{c+1}/(1 + G_{c+1}))
//     L_diag[c] = (1/C_c)                    / (F_c + G_{c+1}/(1 + G_{c+1}))
// which is algebraically the reference's result (its back substitution ends with
// Su[c] += Su[c+1] FI[c] and L_diag[c] = inverse_C[c] / (FF[c] + GP[c+1])), needs
// O(1) registers per lane instead of O(ray length) scratch, and visits every element
// once.  Pair quantities (optical depth, row source) are pure functions of the two
// elements, so they can be evaluated in either sweep direction.
#pragma once
#include <cstring>

#include "mgr_device.cuh"

namespace mgr {

constexpr unsigned FULL_MASK = 0xffffffffu;

// One base step of a traced half ray, staged in shared memory by the warp.
struct HalfSmem {
    uint32_t* ids;   // next point of step s
    double* shift;   // Doppler shift of ids[s]
    double* dZ;      // distance increment of step s
    float* dsh;      // (float)(shift - 1)
    float* dzs;      // (float)dZ * dz_scale (split precision)
    uint32_t* eid;   // CSR edge of step s (index into the interpolation-count table)
    double shift0 = 1.0;  // shift of the origin as this half's trace starts from it (1 comoving)
    float dsh0 = 0.0f;    // shift0 - 1
    double cshift = 1.0;  // shift of the origin element itself (the backward half's shift0)
    float* dsl = nullptr;  // (shift - 1) - dsh, the low part of a double-float shift - 1
    float dsl0 = 0.0f;     // the same for shift0
};

// shift - 1 of step s as a float and its low part (exact: shift - 1 is an FP64 value
// near 0; hi + lo carries about 48 of its bits).
MGR_HD void store_dsh(const HalfSmem& h, int s, double shift) {
    const double d = dsub_rn(shift, 1.0);
    const float hi = (float)d;
    h.dsh[s] = hi;
    h.dsl[s] = (float)dsub_rn(d, (double)hi);
}
MGR_HD void set_dsh0(HalfSmem& h, double shift0) {
    const double d = dsub_rn(shift0, 1.0);
    h.dsh0 = (float)d;
    h.dsl0 = (float)dsub_rn(d, (double)h.dsh0);
}

// Interpolation over all lines (Solver::set_data, solver.tpp:1003-1043) instead of
// one line's criterion, as the imagers trace.
constexpr uint32_t kAllLines = 0xffffffffu;

// Shared-memory carve-up of one warp's two half-ray buffers.
__device__ __forceinline__ void carve_halves(unsigned char* base, uint32_t cap, HalfSmem& bk, HalfSmem& fw) {
    double* d = reinterpret_cast<double*>(base);
    bk.shift = d;
    bk.dZ = d + cap;
    fw.shift = d + 2 * cap;
    fw.dZ = d + 3 * cap;
    uint32_t* u = reinterpret_cast<uint32_t*>(d + 4 * cap);
    bk.ids = u;
    fw.ids = u + cap;
    bk.eid = u + 2 * cap;
    fw.eid = u + 3 * cap;
    float* f = reinterpret_cast<float*>(u + 4 * cap);
    bk.dsh = f;
    fw.dsh = f + cap;
    bk.dzs = f + 2 * cap;
    fw.dzs = f + 3 * cap;
    bk.dsl = f + 4 * cap;
    fw.dsl = f + 5 * cap;
}

__host__ __device__ constexpr size_t half_bytes_per_warp(uint32_t cap) { return (size_t)cap * (4 * 8 + 4 * 4 + 6 * 4); }

// Order-preserving 64-bit key of a finite double (total order, -0 below +0; the
// squared distances compared here are never -0).  Lets the warp's argmin run on the
// integer pipe.
__device__ __forceinline__ unsigned long long dkey(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// One step of Geometry::get_next_general_geometry<Defaulttracer> (geometry.tpp:13-44),
// warp-cooperative: among crt's neighbours with Zn > Z (Zn the distance along the ray
// from the origin po), the one closest to the ray; lanes scan the neighbour list and the
// argmin of (distance to ray, neighbour order) reproduces the reference's strict-< scan.
// Every lane returns the same result: false when no neighbour lies further along the
// ray, else the next point, its Zn and its neighbour-record index.
__device__ __forceinline__ bool warp_next_point(const DevModel& m, const double4_32a& po, double dx, double dy,
                                                double dz, uint32_t crt, double Z, int lane, uint32_t& nxt,
                                                double& Znext, uint32_t& eid) {
    const uint32_t nnb = m.n_nb[crt];
    const uint32_t cum = m.cum_nb[crt];
    const unsigned long long zkey = dkey(Z);
    unsigned long long best = ~0ull;
    uint32_t besti = 0xffffffffu;
    double bestZ = 0.0;
#pragma unroll 1
    for (uint32_t i = lane; i < nnb; i += 32) {
        const double4_32a e = m.edge[cum + i];
        const double Rx = dsub_rn(e.x, po.x);
        const double Ry = dsub_rn(e.y, po.y);
        const double Rz = dsub_rn(e.z, po.z);
        const double Zn = dot3_rn(Rx, Ry, Rz, dx, dy, dz);
        if (dkey(Zn) > zkey) {  // Zn > Z
            const double d2 = dsub_rn(dot3_rn(Rx, Ry, Rz, Rx, Ry, Rz), dmul_rn(Zn, Zn));
            const unsigned long long k = dkey(d2);
            if (k < best) {
                best = k;
                besti = i;
                bestZ = Zn;
            }
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long ob = __shfl_xor_sync(FULL_MASK, best, off);
        const uint32_t oi = __shfl_xor_sync(FULL_MASK, besti, off);
        const double oz = __shfl_xor_sync(FULL_MASK, bestZ, off);
        if (ob < best || (ob == best && oi < besti)) {
            best = ob;
            besti = oi;
            bestZ = oz;
        }
    }
    if (besti == 0xffffffffu) return false;
    eid = cum + besti;
    nxt = (uint32_t)__double_as_longlong(m.edge[eid].w);
    Znext = bestZ;
    return true;
}

// ---------------------------------------------------------------------------------
// FP32 filter of the next-point argmin.  On GB300 the FP64 pipe issues one warp
// instruction per 16 cycles whatever the number of active lanes, and the exact argmin
// above costs 15 FP64 instructions per step.  The filter evaluates every neighbour's
// distance along the ray and squared distance to the ray in FP32, from hi/lo float
// copies of the positions (the origin-relative vector is then accurate to about
// 3 u |R|, u = 2^-24, with no cancellation against the absolute coordinates), with
// rigorous bounds on how far each FP32 value can lie from the FP64 value the reference
// computes:
//   |Zf  - Zn_ref|  <= EZ  = 10 u s1 + 32 u^2,             s1 = sum |r_i d_i|
//   |d2f - d2_ref|  <= Ed2 = 2 ec |c|_1 + 3 ec^2 + 6 u d2f + 1e-14 |r|_1^2,
//                           ec = 8 u |r|_1 + 32 u^2,  c = r x d
// (positions scaled into [-1, 1] by a power of two; d2 through the cross product, which
// equals |R|^2 - (R.d)^2 up to |R|^2 (1 - |d|^2) and the FP64 roundings, both covered by
// the last term for unit directions: models whose directions are not unit to 2e-15 get
// no filter tables (edge_hl null) and trace with the exact argmin).  A neighbour is
// certainly ahead (Zn > Z) when Zf - Zc exceeds EZ plus the bound of the current Z's
// estimate Zc, certainly behind when it is below minus that, else undecided.  When
// exactly one neighbour that is certainly ahead or undecided has a lower bound of d2 at
// or below the smallest upper bound among the certainly-ahead ones, and it is certainly
// ahead, it is the reference's choice: every other candidate's d2 is strictly larger.
// Otherwise (near ties, undecided ahead/behind, more than 32 neighbours) the step is
// taken by the exact FP64 argmin.  The exact Z of the chosen points (and dZ) are
// computed afterwards, one step per lane, and chained in the reference's order
// (Z += Zn - Z).
// ---------------------------------------------------------------------------------
constexpr float kU32 = 5.9604644775390625e-8f;     // 2^-24
constexpr float kU32Sq = 3.552713678800501e-15f;   // 2^-48

// Float bits (host and device).
MGR_HD uint32_t f32_bits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    uint32_t b;
    std::memcpy(&b, &x, 4);
    return b;
#endif
}
MGR_HD float bits_f32(uint32_t b) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float x;
    std::memcpy(&x, &b, 4);
    return x;
#endif
}

// A double as the unevaluated sum hi + lo of two floats (round to nearest each).
MGR_HD void split_hl(double x, float& hi, float& lo) {
    hi = (float)x;
    lo = (float)dsub_rn(x, (double)hi);
}

// Per-trace state of the filter: the origin's hi/lo position, the direction as floats,
// and the estimate Zc of the current Z with its bound eZc (all in scaled units).
struct TraceF32 {
    float4 poh, pol;
    float dx, dy, dz;
    float Zc, eZc;
};

// One neighbour's filter values: Zf and its bound EZ, and the bounds lo <= d2 <= hi.
struct FiltCand {
    float Zf, EZ, lo, hi;
};

// Explicit fmaf everywhere, so that the host emulation and the device compute the same
// floats (nothing is left for the compiler to contract).
MGR_HD FiltCand filt_cand(const float4& a, const float4& b, const TraceF32& t) {
    const float rx = (a.x - t.poh.x) + (b.x - t.pol.x);
    const float ry = (a.y - t.poh.y) + (b.y - t.pol.y);
    const float rz = (a.z - t.poh.z) + (b.z - t.pol.z);
    FiltCand c;
    c.Zf = fmaf(rz, t.dz, fmaf(ry, t.dy, rx * t.dx));
    const float s1 = fabsf(rx * t.dx) + fabsf(ry * t.dy) + fabsf(rz * t.dz);
    const float rn1 = fabsf(rx) + fabsf(ry) + fabsf(rz);
    const float cx = fmaf(ry, t.dz, -(rz * t.dy));
    const float cy = fmaf(rz, t.dx, -(rx * t.dz));
    const float cz = fmaf(rx, t.dy, -(ry * t.dx));
    const float d2 = fmaf(cz, cz, fmaf(cy, cy, cx * cx));
    const float cn1 = fabsf(cx) + fabsf(cy) + fabsf(cz);
    const float ec = fmaf(8.0f * kU32, rn1, 32.0f * kU32Sq);
    const float rr = rn1 * rn1;
    const float e = fmaf(2.0f * ec, cn1, fmaf(3.0f * ec, ec, fmaf(6.0f * kU32, d2, 1.0e-14f * rr)));
    const float Ed2 = e * 1.001f;
    c.EZ = fmaf(10.0f * kU32, s1, 32.0f * kU32Sq);
    c.lo = d2 - Ed2;
    c.hi = d2 + Ed2;
    return c;
}

// Ahead / behind decision of a candidate against the current Z estimate: 1 certainly
// ahead (Zn > Z), -1 certainly not, 0 undecided.
MGR_HD int filt_ahead(const FiltCand& c, const TraceF32& t) {
    const float diff = c.Zf - t.Zc;
    const float tol = (c.EZ + t.eZc) * 1.0001f;
    return diff > tol ? 1 : (diff < -tol ? -1 : 0);
}

// The filter's step, warp-cooperative (lane i holds neighbour i).  Returns 1 with the
// next point, its neighbour-record index and its Zf / EZ when the filter decides; 0
// when no neighbour can lie further along the ray; -1 when the exact argmin must decide.
__device__ __forceinline__ int warp_next_point_f32(const DevModel& m, const TraceF32& t, uint32_t crt, int lane,
                                                   uint32_t& nxt, uint32_t& eid, float& Zw, float& EZw) {
    const uint32_t nnb = m.n_nb[crt];
    if (nnb > 32) return -1;
    const uint32_t cum = m.cum_nb[crt];
    int ah = -1;
    FiltCand c{0.0f, 0.0f, 0.0f, 0.0f};
    uint32_t idx = 0;
    if ((uint32_t)lane < nnb) {
        const float4 a = m.edge_hl[2 * (size_t)(cum + lane)];
        const float4 b = m.edge_hl[2 * (size_t)(cum + lane) + 1];
        c = filt_cand(a, b, t);
        ah = filt_ahead(c, t);
        idx = f32_bits(a.w);
    }
    float best = ah > 0 ? c.hi : INFINITY;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) best = fminf(best, __shfl_xor_sync(FULL_MASK, best, off));
    const unsigned cont = __ballot_sync(FULL_MASK, ah >= 0 && c.lo <= best);
    if (cont == 0) return 0;
    if (__popc(cont) != 1) return -1;
    const int w = __ffs(cont) - 1;
    if (__shfl_sync(FULL_MASK, ah, w) != 1) return -1;
    nxt = __shfl_sync(FULL_MASK, idx, w);
    eid = cum + (uint32_t)w;
    Zw = __shfl_sync(FULL_MASK, c.Zf, w);
    EZw = __shfl_sync(FULL_MASK, c.EZ, w);
    return 1;
}

// The walk of trace_half in 1D spherical symmetry (Geometry::get_next_spherical_symmetry,
// geometry.tpp:118-159): every lane steps the same shells; lane 0 stores the steps, with
// each step's shift at its distance along the ray (get_shift_spherical_symmetry) and the
// half's origin shift (shift0, not 1 in the comoving frame there).
template <bool STORE, int FRAME>
__device__ int trace_half_sph(const DevModel& m, uint32_t o, uint32_t r, uint32_t cap, HalfSmem& h, int lane,
                              int* status) {
    const double* d = FRAME ? m.raydir + 3 * r : ray_dir(m, o, r);
    const double4_32a po = m.pos[o];
    const double Rcos = dot3_rn(po.x, po.y, po.z, d[0], d[1], d[2]);
    const double Rsin2 = dsub_rn(sqnorm_rn(po), dmul_rn(Rcos, Rcos));
    if (STORE) {
        h.shift0 = origin_shift(m, FRAME, o, r);
        set_dsh0(h, h.shift0);
    }
    double Z = 0.0;
    uint32_t crt = o;
    int count = 0;
    while (true) {
        uint32_t nxt;
        double dZl;
        if (!next_point_sph(m, Rcos, Rsin2, crt, Z, nxt, dZl)) {
            if (count > 0 && lane == 0) atomicOr(status, ST_TRACE);
            if (count > 0) count = -1;
            break;
        }
        if (STORE && (uint32_t)count >= cap) {
            if (lane == 0) atomicOr(status, ST_CAPACITY);
            count = -1;
            break;
        }
        Z = dadd_rn(Z, dZl);
        if (STORE && lane == 0) {
            h.ids[count] = nxt;
            h.eid[count] = sph_eid(crt, nxt);
            h.dZ[count] = dZl;
            const double sh = shift_sph(m, FRAME, o, r, nxt, Z, d);
            h.shift[count] = sh;
            store_dsh(h, count, sh);
            h.dzs[count] = (float)dZl * m.dz_scale;
        }
        count++;
        if (m.p2b[nxt] != m.P) break;
        crt = nxt;
    }
    __syncwarp();
    return count;
}

// Warp-cooperative Geometry::get_next_general_geometry<Defaulttracer> walk
// (geometry.tpp:13-44) from origin o along ray r until a boundary point is met
// (warp_next_point per step).  Returns the number of steps, or -1 on capacity
// overflow / invalid geometry (status bits set).  Spherical models walk shells
// (trace_half_sph).
// FRAME 0: comoving shifts relative to the origin point (the formal solves);
// FRAME 1: rest-frame shifts of the old imager (Geometry::get_shift<Rest>, reversed for
// r >= hnrays, geometry.tpp:428-465).
// GEO 0 compiles the general geometry with shared rays only (the caller has checked the
// model); GEO 1 handles every geometry at run time.
template <bool STORE, int FRAME = 0, int GEO = 1, bool FILTER = true>
__device__ int trace_half(const DevModel& m, uint32_t o, uint32_t r, uint32_t cap, HalfSmem& h, int lane,
                          int* status) {
    if (GEO && m.sph) return trace_half_sph<STORE, FRAME>(m, o, r, cap, h, lane, status);
    // the formal solves trace along the origin's (adaptive) directions, the old imager
    // along the shared ones (trace_ray<Rest, false>, solver.tpp:550-552)
    const double* d = (FRAME || !GEO) ? m.raydir + 3 * r : ray_dir(m, o, r);
    const double dx = d[0], dy = d[1], dz = d[2];
    const double4_32a po = m.pos[o];
    TraceF32 t;
    if (FILTER) {
        t.poh = m.pos_hl[2 * (size_t)o];
        t.pol = m.pos_hl[2 * (size_t)o + 1];
        t.dx = (float)dx;
        t.dy = (float)dy;
        t.dz = (float)dz;
        t.Zc = 0.0f;
        t.eZc = 0.0f;
    }
    double Z = 0.0;  // exact Z after the last step whose Zn is known in FP64
    // Steps chosen by the filter whose exact Zn and dZ are not computed yet: the last
    // np steps; lane j holds the point of the j-th of them.
    uint32_t pend = 0;
    int np = 0;
    uint32_t crt = o;
    int count = 0;
    // Exact Zn of the pending steps, one step per lane, then Z += Zn - Z in step order.
    auto flush = [&]() {
        if (np == 0) return;
        double Zn = 0.0;
        if (lane < np) {
            const double4_32a q = m.pos[pend];
            Zn = dot3_rn(dsub_rn(q.x, po.x), dsub_rn(q.y, po.y), dsub_rn(q.z, po.z), dx, dy, dz);
        }
        const int base = count - np;
        for (int j = 0; j < np; j++) {
            const double dZl = dsub_rn(__shfl_sync(FULL_MASK, Zn, j), Z);
            Z = dadd_rn(Z, dZl);
            if (STORE && lane == 0) h.dZ[base + j] = dZl;
        }
        np = 0;
    };
    while (true) {
        uint32_t nxt = 0, eid = 0;
        float Zw = 0.0f, EZw = 0.0f;
        int found = (FILTER && m.edge_hl) ? warp_next_point_f32(m, t, crt, lane, nxt, eid, Zw, EZw) : -1;
        bool exact = false;
        double dZl = 0.0;
        if (found < 0) {
            flush();
            double bestZ;
            found = warp_next_point(m, po, dx, dy, dz, crt, Z, lane, nxt, bestZ, eid) ? 1 : 0;
            if (found) {
                exact = true;
                dZl = dsub_rn(bestZ, Z);
                Z = dadd_rn(Z, dZl);
                if (FILTER) {
                    Zw = (float)dmul_rn(Z, m.pos_scale);
                    EZw = fmaf(2.0f * kU32, fabsf(Zw), 32.0f * kU32Sq);
                }
            }
        }
        if (!found) {
            // No point further along the ray.  From the origin this is an empty half;
            // after a step it means the walk left the grid on an interior point, where
            // the reference would index point2boundary out of range.
            if (count > 0 && lane == 0) atomicOr(status, ST_TRACE);
            if (count > 0) count = -1;
            break;
        }
        if (STORE && (uint32_t)count >= cap) {
            if (lane == 0) atomicOr(status, ST_CAPACITY);
            count = -1;
            break;
        }
        if (STORE && lane == 0) {
            h.ids[count] = nxt;
            h.eid[count] = eid;
            if (exact) h.dZ[count] = dZl;
        }
        if (!exact) {
            if (lane == np) pend = nxt;
            np++;
        }
        count++;
        if (FILTER) {
            t.Zc = Zw;
            t.eZc = EZw;
        }
        if (np == 32) flush();
        if (m.p2b[nxt] != m.P) break;
        crt = nxt;
    }
    if (count > 0) flush();
    __syncwarp();
    if (STORE && count > 0) {
        // Per-step Doppler shifts and FP32 copies, one step per lane.
        for (int s = lane; s < count; s += 32) {
            const double sh = FRAME ? shift_rest(m, r, h.ids[s], d) : shift_comoving(m, o, h.ids[s], d);
            h.shift[s] = sh;
            store_dsh(h, s, sh);
            h.dzs[s] = (float)h.dZ[s] * m.dz_scale;
        }
        __syncwarp();
    }
    return count;
}

// Both halves of a ray pair: r into `bk`, its antipode ar into `fw`.  One loop over
// the two halves, so that a kernel holds a single copy of the trace's code.
template <bool STORE, int FRAME = 0, int GEO = 1, bool FILTER = true>
__device__ __forceinline__ void trace_pair(const DevModel& m, uint32_t o, uint32_t r, uint32_t ar, uint32_t cap,
                                           HalfSmem& bk, HalfSmem& fw, int lane, int* status, int& nb, int& nf) {
#pragma unroll 1
    for (int side = 0; side < 2; side++) {
        const int n = trace_half<STORE, FRAME, GEO, FILTER>(m, o, side ? ar : r, cap, side ? fw : bk, lane, status);
        if (side) nf = n;
        else nb = n;
    }
}

// An element of the ray pair as the reference's per-thread buffers hold it
// (nr, nr_interp, interp_factor, shift) plus its distance to the neighbouring
// element on the origin side.  FP64 mode fills the double fields; split precision
// fills the FP32 ones and keeps (s, i, n) so that the FP64 shift and factor can be
// recomputed exactly where a pair needs them (elem_shift_fac).
struct Elem {
    uint32_t nr, ni;
    double fac;
    double shift;
    double dzin;
    float dsh;   // shift - 1
    float dshm;  // |shift - 1| of the step's two ends, summed (bound for FP32 rounding)
    float facf;  // interpolation factor
    float dzf;   // distance * dz_scale
    int s;       // base step (split precision)
    uint32_t i;  // sub-element i of n; n == 0 marks the origin
    uint32_t n;
};

// Walks the elements of one half ray from its outer end toward the origin,
// expanding the interpolation points Solver::set_data_for_line inserts
// (solver.tpp:1057-1097).  Elements of one step are visited i = n .. 1.
struct ElemIter {
    int s;          // current base step
    int nsteps;     // steps of the half (upward iteration)
    uint32_t i;     // current sub-element (n .. 1), 0 = step exhausted
    uint32_t n;     // interpolation count of step s
    uint32_t crt, nxt;
    double shc, shn, dzs, dshi, dzi;  // FP64: step ends, distance, per-sub-element increments
    float dshc, ddsh, dshm, dzi_f, rn;
};

template <int MODE>
MGR_HD void iter_load_step(const DevModel& m, const HalfSmem& h, uint32_t o, uint32_t l, ElemIter& it) {
    const int s = it.s;
    it.crt = s ? h.ids[s - 1] : o;
    it.nxt = h.ids[s];
    it.n = (l == kAllLines) ? m.nint_all[h.eid[s]] : m.nint[(size_t)h.eid[s] * m.L + l];
    it.i = it.n;
    const uint32_t n = it.n;
    if constexpr (MODE == MODE_FP64) {
        it.shc = s ? h.shift[s - 1] : h.shift0;
        it.shn = h.shift[s];
        it.dzs = h.dZ[s];
        // per-step parts of the reference's per-element expressions (same roundings)
        it.dshi = dsub_rn(it.shn, it.shc) / (double)n;
        it.dzi = it.dzs / (double)n;
    } else {
        const float dshc = s ? h.dsh[s - 1] : h.dsh0;
        const float dshn = h.dsh[s];
        const float rn = fast_div(1.0f, (float)n);
        it.dshc = dshc;
        it.ddsh = (dshn - dshc) * rn;
        it.dshm = fabsf(dshc) + fabsf(dshn);
        it.dzi_f = h.dzs[s] * rn;
        it.rn = rn;
    }
}

// Element (step it.s, sub-element i of n) of the loaded step, with the reference's
// per-element expressions (set_data_for_line / set_data).
template <int MODE>
MGR_HD void step_elem(const ElemIter& it, uint32_t i, Elem& e) {
    const uint32_t n = it.n;
    e.nr = it.nxt;
    e.ni = it.crt;
    if constexpr (MODE == MODE_FP64) {
        if (n > 1) {
            e.shift = dadd_rn(it.shc, dmul_rn((double)i, it.dshi));
            e.fac = 1.0 - ((double)i) / (double)n;
            e.dzin = it.dzi;
        } else {
            e.shift = it.shn;
            e.fac = 0.0;
            e.dzin = it.dzs;
        }
    } else {
        e.dsh = fmaf((float)i, it.ddsh, it.dshc);
        e.facf = fmaf(-(float)i, it.rn, 1.0f);
        e.dzf = it.dzi_f;
        e.dshm = it.dshm;
        e.s = it.s;
        e.i = i;
        e.n = n;
    }
}

// Produces the next element (outer to inner).  Returns false when only the
// centre element remains.
template <int MODE>
MGR_HD bool iter_next(const DevModel& m, const HalfSmem& h, uint32_t o, uint32_t l, ElemIter& it, Elem& e) {
    if (it.i == 0) {
        if (it.s == 0) return false;
        it.s--;
        iter_load_step<MODE>(m, h, o, l, it);
    }
    step_elem<MODE>(it, it.i, e);
    it.i--;
    return true;
}

// The same half from the origin outward (inner to outer, the array order of a forward
// half): steps 0 .. nsteps-1, sub-elements 1 .. n.  it.s == nsteps when done.
template <int MODE>
MGR_HD void iter_up_begin(const DevModel& m, const HalfSmem& h, uint32_t o, uint32_t l, int nsteps, ElemIter& it) {
    it.s = 0;
    it.nsteps = nsteps;
    if (nsteps > 0) {
        iter_load_step<MODE>(m, h, o, l, it);
        it.i = 1;
    }
}

template <int MODE>
MGR_HD bool iter_up_next(const DevModel& m, const HalfSmem& h, uint32_t o, uint32_t l, ElemIter& it, Elem& e) {
    if (it.s >= it.nsteps) return false;
    step_elem<MODE>(it, it.i, e);
    if (++it.i > it.n) {
        it.s++;
        if (it.s < it.nsteps) {
            iter_load_step<MODE>(m, h, o, l, it);
            it.i = 1;
        }
    }
    return true;
}

template <int MODE>
MGR_HD void iter_begin(const DevModel& m, const HalfSmem& h, uint32_t o, uint32_t l, int nsteps, ElemIter& it) {
    if (nsteps <= 0) {
        it.s = 0;
        it.i = 0;
        return;
    }
    it.s = nsteps - 1;
    iter_load_step<MODE>(m, h, o, l, it);
}

MGR_HD Elem centre_elem(uint32_t o, double shift0 = 1.0, float dsh0 = 0.0f) {
    Elem e;
    e.nr = o;
    e.ni = o;  // never read: its interpolation factor is 0
    e.fac = 0.0;
    e.shift = shift0;
    e.dzin = 0.0;
    e.dsh = dsh0;
    e.dshm = fabsf(dsh0);
    e.facf = 0.0f;
    e.dzf = 0.0f;
    e.s = 0;
    e.i = 0;
    e.n = 0;
    return e;
}

// The FP64 shift and interpolation factor of a split-precision element, computed
// exactly as the FP64 iterator does.
MGR_HD void elem_shift_fac(const HalfSmem& h, const Elem& e, double& shift, double& fac) {
    if (e.n == 0) {
        shift = h.cshift;
        fac = 0.0;
        return;
    }
    const double shn = h.shift[e.s];
    if (e.n > 1) {
        const double shc = e.s ? h.shift[e.s - 1] : h.shift0;
        shift = dadd_rn(shc, dmul_rn((double)e.i, dsub_rn(shn, shc) / (double)e.n));
        fac = 1.0 - ((double)e.i) / (double)e.n;
    } else {
        shift = shn;
        fac = 0.0;
    }
}

// ---------------------------------------------------------------------------------
// Pair physics.  Lane context: origin o, frequency f, its line l0, nu(o, f).
// ---------------------------------------------------------------------------------
struct LaneCtx {
    uint32_t o, f, l0;
    double freq;   // nu(o, f)
    float fq;      // (float)freq
    float a0;      // (float)(freq - line[l0])
    float fql;     // freq - fq, the low part of a double-float freq
};

// The lane context of frequency f at origin o.
MGR_HD LaneCtx lane_ctx(const DevModel& m, uint32_t o, uint32_t f) {
    LaneCtx c;
    c.o = o;
    c.f = f;
    c.l0 = m.corr_line[f];
    c.freq = m.nu[(size_t)o * m.F + f];
    c.fq = (float)c.freq;
    c.a0 = (float)(c.freq - m.line[c.l0]);
    c.fql = (float)(c.freq - (double)c.fq);
    return c;
}

// FP64 (reference arithmetic) -------------------------------------------------------

// get_eta_and_chi_interpolated<approx> (solver.tpp:1176-1194, :1252-1283, :1306-1320).
template <int AP>
MGR_HD void eta_chi_fp64(const DevModel& m, const double* sl, const LaneCtx& c, const Elem& e,
                                             double& eta, double& chi) {
    // The FP64 mode's frequency products and differences are explicitly rounded: a
    // product contracted into the difference that follows it rounds once where the
    // reference rounds twice, and which ones the compiler contracts differs between
    // kernels; an ulp of a profile's or an erff's argument can flip its rounding to
    // float and move J by ~1e-8.
    const double freq = dmul_rn(c.freq, e.shift);
    const size_t b1 = (size_t)e.nr * m.L, b2 = (size_t)e.ni * m.L;
    if (AP == APPROX_ONELINE) {
        const uint32_t l = c.l0;
        const double iw = interpolate_linear(m.iw[b1 + l], m.iw[b2 + l], e.fac);
        const double prof = gaussian(iw, dsub_rn(freq, m.line[l]));
        eta = prof * interpolate_log(m.em[b1 + l], m.em[b2 + l], e.fac);
        chi = prof * interpolate_log(m.op[b1 + l], m.op[b2 + l], e.fac) + m.min_opacity;
        return;
    }
    eta = 0.0;
    chi = m.min_opacity;
    uint32_t lo = 0, hi = m.L;
    if (AP == APPROX_CLOSELINES) {
        // explicitly rounded: a contracted freq - max_dist * (...) moves the bracket's
        // edge by an ulp and can add or drop a far line (the reference rounds twice)
        const double ub = dmul_rn(m.max_dist, dmul_rn(freq, m.ub[e.nr]));
        lo = lower_bound(sl, m.L, dsub_rn(freq, ub));
        hi = upper_bound(sl, m.L, dadd_rn(freq, ub));
    }
    for (uint32_t s = lo; s < hi; s++) {
        uint32_t l;
        double diff;
        if (AP == APPROX_CLOSELINES) {
            l = m.sorted_map[s];
            diff = dsub_rn(freq, sl[s]);
        } else {
            l = s;
            diff = dsub_rn(freq, m.line[l]);
        }
        const double iw = interpolate_linear(m.iw[b1 + l], m.iw[b2 + l], e.fac);
        const double prof = gaussian(iw, diff);
        eta += prof * interpolate_log(m.em[b1 + l], m.em[b2 + l], e.fac);
        chi += prof * interpolate_log(m.op[b1 + l], m.op[b2 + l], e.fac);
    }
}

// compute_dtau_single_line (solver.tpp:2374-2455).
MGR_HD double dtau_single_line_fp64(const DevModel& m, const Elem& lo, const Elem& hi, uint32_t l,
                                                        double cf, double nf, double dz) {
    const size_t c1 = (size_t)lo.nr * m.L, c2 = (size_t)lo.ni * m.L;
    const size_t n1 = (size_t)hi.nr * m.L, n2 = (size_t)hi.ni * m.L;
    const double linefreq = m.line[l];
    const double iwc = interpolate_linear(m.iw[c1 + l], m.iw[c2 + l], lo.fac);
    const double iwn = interpolate_linear(m.iw[n1 + l], m.iw[n2 + l], hi.fac);
    const double avg_iw = (iwc + iwn) / 2.0;
    const double cop = interpolate_log(m.op[c1 + l], m.op[c2 + l], lo.fac);
    const double nop = interpolate_log(m.op[n1 + l], m.op[n2 + l], hi.fac);
    if (cf == nf) {
        const double prof = gaussian(avg_iw, dsub_rn(cf, m.line[l]));
        return dz * (prof * ((cop + nop) / 2.0) + m.min_opacity);
    }
    const double next_pos = dmul_rn(dsub_rn(linefreq, nf), avg_iw);
    const double curr_pos = dmul_rn(dsub_rn(linefreq, cf), avg_iw);
    const double diff_pos = next_pos - curr_pos;
    const double average_opacity = (nop + cop) / 2.0;
    // The reference subtracts two single-precision erff values (solver.tpp:2450).
    // For |pos| >~ 2 that difference cancels catastrophically, so a one-ulp change
    // of erff moves J by up to ~1e-4 on strongly Doppler-shifted models: FP64 mode
    // therefore uses the correctly rounded erff, (float)erf((double)x), which is the
    // same on every platform (and in the oracle's matching mode).
    const float erfdiff = erff_cr((float)next_pos) - erff_cr((float)curr_pos);
    const double erfterm = average_opacity / diff_pos / 2.0 * (double)erfdiff;
    return dz * (avg_iw * erfterm + m.min_opacity);
}

// compute_S_dtau_line_integrated<approx> (solver.tpp:1878-2111).
template <int AP>
MGR_HD void pair_li_fp64(const DevModel& m, const double* sl, const LaneCtx& c, const Elem& lo,
                                             const Elem& hi, double dz, double& out_dtau, double& out_Slo,
                                             double& out_Shi) {
    const double cf = dmul_rn(c.freq, lo.shift);
    const double nf = dmul_rn(c.freq, hi.shift);
    const size_t c1 = (size_t)lo.nr * m.L, c2 = (size_t)lo.ni * m.L;
    const size_t n1 = (size_t)hi.nr * m.L, n2 = (size_t)hi.ni * m.L;
    if (AP == APPROX_ONELINE) {
        const uint32_t l = c.l0;
        out_dtau = dtau_single_line_fp64(m, lo, hi, l, cf, nf, dz);
        out_Slo = interpolate_log(m.Sp[c1 + l], m.Sp[c2 + l], lo.fac);
        out_Shi = interpolate_log(m.Sp[n1 + l], m.Sp[n2 + l], hi.fac);
        return;
    }
    double sum_dtau = 0.0, sum_c = 0.0, sum_n = 0.0;
    uint32_t a = 0, b = m.L;
    if (AP == APPROX_CLOSELINES) {
        double left_freq, right_freq;
        if (cf < nf) { left_freq = cf; right_freq = nf; }
        else { right_freq = cf; left_freq = nf; }
        const double cb = dmul_rn(m.max_dist, dmul_rn(right_freq, m.ub[lo.nr]));
        const double nb = dmul_rn(m.max_dist, dmul_rn(right_freq, m.ub[hi.nr]));
        const double ubw = cb > nb ? cb : nb;
        a = lower_bound(sl, m.L, dsub_rn(left_freq, ubw));
        b = upper_bound(sl, m.L, dadd_rn(right_freq, ubw));
    }
    for (uint32_t s = a; s < b; s++) {
        const uint32_t l = (AP == APPROX_CLOSELINES) ? m.sorted_map[s] : s;
        const double ld = dtau_single_line_fp64(m, lo, hi, l, cf, nf, dz);
        const double lsc = interpolate_log(m.Sp[c1 + l], m.Sp[c2 + l], lo.fac);
        const double lsn = interpolate_log(m.Sp[n1 + l], m.Sp[n2 + l], hi.fac);
        sum_dtau += ld;
        sum_c += ld * lsc;
        sum_n += ld * lsn;
    }
    if (AP == APPROX_NONE) {
        out_dtau = sum_dtau;
        out_Slo = sum_c / sum_dtau;
        out_Shi = sum_n / sum_dtau;
        return;
    }
    double d = sum_dtau;
    const double bound_min_dtau = m.min_opacity * dz;
    if (-bound_min_dtau < d) d = (bound_min_dtau > d) ? bound_min_dtau : d;
    out_dtau = d;
    out_Slo = sum_c / d;
    out_Shi = sum_n / d;
}

// FP32 (split precision) ------------------------------------------------------------
// Frequencies are FP32 offsets from the lane's own line centre:
//   nu(o,f) shift - line[l] = (nu(o,f) - line[l0]) + nu(o,f) (shift - 1) - (line[l] - line[l0]),
// the last term from the [L][L] tables dll/dls.  Line data are the scaled FP32 tables
// (DevModel::em_f, ...); element factors and distances arrive precomputed in FP32.

MGR_HD float offset_f32(const DevModel& m, const LaneCtx& c, float dsh, uint32_t l) {
    const float off0 = fmaf(c.fq, dsh, c.a0);
    return (l == c.l0) ? off0 : off0 - m.dll[(size_t)c.l0 * m.L + l];
}

// CloseLines bracket in offsets: the sorted lines s with dls[l0][s] in [lo_off, hi_off].
MGR_HD void bracket_f32(const DevModel& m, const LaneCtx& c, float lo_off, float hi_off, uint32_t& a, uint32_t& b) {
    const float* d = m.dls + (size_t)c.l0 * m.L;
    a = m.L;
    b = 0;
    for (uint32_t s = 0; s < m.L; s++) {
        const float dl = d[s];
        if (dl >= lo_off && dl <= hi_off) {
            if (s < a) a = s;
            b = s + 1;
        }
    }
    if (b < a) b = a;
}

template <int AP>
MGR_HD void eta_chi_f32(const DevModel& m, const LaneCtx& c, const Elem& e, float& eta, float& chi) {
    const size_t b1 = (size_t)e.nr * m.L, b2 = (size_t)e.ni * m.L;
    const float fac = e.facf;
    const float min_op = m.min_op_s;
    if (AP == APPROX_ONELINE) {
        const uint32_t l = c.l0;
        const float iw = interpolate_linear(m.iw_f[b1 + l], m.iw_f[b2 + l], fac);
        const float prof = gaussian(iw, offset_f32(m, c, e.dsh, l));
        eta = prof * interpolate_log(m.em_f[b1 + l], m.em_f[b2 + l], fac);
        chi = prof * interpolate_log(m.op_f[b1 + l], m.op_f[b2 + l], fac) + min_op;
        return;
    }
    eta = 0.0f;
    chi = min_op;
    uint32_t lo = 0, hi = m.L;
    if (AP == APPROX_CLOSELINES) {
        // lines inside freq -+ max_dist * freq * ub[p] (solver.tpp:1216-1227)
        const float off0 = fmaf(c.fq, e.dsh, c.a0);
        const float ub = m.max_dist_f * ((c.fq + c.fq * e.dsh) * m.ub_f[e.nr]);
        bracket_f32(m, c, off0 - ub, off0 + ub, lo, hi);
    }
    for (uint32_t s = lo; s < hi; s++) {
        const uint32_t l = (AP == APPROX_CLOSELINES) ? m.sorted_map[s] : s;
        const float iw = interpolate_linear(m.iw_f[b1 + l], m.iw_f[b2 + l], fac);
        const float prof = gaussian(iw, offset_f32(m, c, e.dsh, l));
        eta += prof * interpolate_log(m.em_f[b1 + l], m.em_f[b2 + l], fac);
        chi += prof * interpolate_log(m.op_f[b1 + l], m.op_f[b2 + l], fac);
    }
}

// Out-of-line paths of split precision.  They run for a small fraction of pairs and
// are kept out of the hot loop so that its code stays small.

// ---- double-float arithmetic: a value carried as the unevaluated sum hi + lo of two
// floats (about 48 significant bits), with Knuth's TwoSum and an FMA-based exact
// product (Dekker 1971).  Split precision uses it for the same-wing erf arguments.
struct F2 {
    float hi, lo;
};
MGR_HD F2 f2_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return F2{s, (a - (s - bb)) + (b - bb)};
}
MGR_HD F2 f2_quick(float a, float b) {  // |a| >= |b| or a == 0
    const float s = a + b;
    return F2{s, b - (s - a)};
}
MGR_HD F2 f2_add(F2 a, F2 b) {
    F2 s = f2_two_sum(a.hi, b.hi);
    const F2 t = f2_two_sum(a.lo, b.lo);
    s = f2_quick(s.hi, s.lo + t.hi);
    return f2_quick(s.hi, s.lo + t.lo);
}
MGR_HD F2 f2_sub(F2 a, F2 b) { return f2_add(a, F2{-b.hi, -b.lo}); }
MGR_HD F2 f2_mul(F2 a, F2 b) {
    const float p = a.hi * b.hi;
    const float e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p)));
    return f2_quick(p, e);
}

// i / n as a double-float: q = fl(i / n) and the exact remainder i - q n over n.
MGR_HD F2 f2_ratio(uint32_t i, uint32_t n) {
    const float fi = (float)i, fn = (float)n;
#ifdef __CUDA_ARCH__
    const float q = __fdiv_rn(fi, fn);
#else
    const float q = fi / fn;
#endif
    return f2_quick(q, fmaf(-q, fn, fi) / fn);
}

// shift - 1 of a split-precision element as a double-float: the step's stored value
// (n = 1), the FP64 iterator's shc + i (shn - shc) / n (n > 1), or the origin's.
MGR_HD F2 elem_dsh_f2(const HalfSmem& h, const Elem& e) {
    if (e.n == 0) {
        const double d = h.cshift - 1.0;
        const float hi = (float)d;
        return F2{hi, (float)(d - (double)hi)};
    }
    const F2 dn{h.dsh[e.s], h.dsl[e.s]};
    if (e.n == 1) return dn;
    const F2 dc = e.s ? F2{h.dsh[e.s - 1], h.dsl[e.s - 1]} : F2{h.dsh0, h.dsl0};
    return f2_add(dc, f2_mul(f2_sub(dn, dc), f2_ratio(e.i, e.n)));
}

// The element's inverse width of line l as a double-float (interpolate_linear with the
// factor 1 - i / n between its two points).
MGR_HD F2 elem_iw_f2(const DevModel& m, const Elem& e, uint32_t l) {
    const size_t a = (size_t)e.nr * m.L + l;
    const F2 w1{m.iw_f[a], m.iw_lo[a]};
    if (e.n <= 1) return w1;
    const size_t b = (size_t)e.ni * m.L + l;
    const F2 w2{m.iw_f[b], m.iw_lo[b]};
    const F2 fac = f2_sub(F2{1.0f, 0.0f}, f2_ratio(e.i, e.n));
    return f2_add(w1, f2_mul(f2_sub(w2, w1), fac));
}

// Correctly rounded erff(x) (the FP64 mode's erff_cr) without FP64 arithmetic: +-1 for
// |x| >= 3.919206, the device's table of (float)erf((double)x) over every float in
// [kErfBandLo, 3.919206) (erf_band_table), and FP64 below (the same-wing arguments
// start at 1.5: the float positions that select them are within 1e-5 of the exact ones).
// erff_cr out of line, for the band's lower edge: the same-wing arguments start at
// 1.5, so the kernels reach it only through FP32 rounding, and their code stays small.
static __host__ __device__ __noinline__ float erff_cr_cold(float x) { return erff_cr(x); }

MGR_HD float erff_band(const DevModel& m, float x) {
#ifdef __CUDA_ARCH__
    const float ax = fabsf(x);
    if (ax >= 3.919206f) return copysignf(1.0f, x);
    if (ax < kErfBandLo) return erff_cr_cold(x);
    return copysignf(m.erf_band[__float_as_uint(ax) - __float_as_uint(kErfBandLo)], x);
#else
    (void)m;  // the host emulation evaluates the table's entries directly
    return erff_cr(x);
#endif
}

// Same-wing erf difference on the FP64 mode's arguments (linefreq - nu shift) * avg_iw,
// without FP64 arithmetic: the arguments are evaluated in double-float, written as
// (linefreq - nu) - nu (shift - 1), so that the float they round to is the one the FP64
// expressions of dtau_single_line_fp64 round to (except for values within about 1e-10
// relative of a rounding midpoint), and the correctly rounded erff of each comes from
// the table.  Returns {erff(next) - erff(curr), next - curr}; both arguments are in
// the table's range.
MGR_HD float2 band_erf(const DevModel& m, const LaneCtx& c, const HalfSmem& h, const Elem& lo, const Elem& hi,
                       uint32_t l) {
    const F2 freq{c.fq, c.fql};
    const F2 a = f2_sub(F2{m.line_df[2 * l], m.line_df[2 * l + 1]}, freq);
    F2 avg = f2_add(elem_iw_f2(m, lo, l), elem_iw_f2(m, hi, l));
    avg.hi *= 0.5f;
    avg.lo *= 0.5f;
    const F2 np = f2_mul(f2_sub(a, f2_mul(freq, elem_dsh_f2(h, hi))), avg);
    const F2 cp = f2_mul(f2_sub(a, f2_mul(freq, elem_dsh_f2(h, lo))), avg);
    float2 r;
    r.x = erff_band(m, np.hi) - erff_band(m, cp.hi);
    r.y = f2_sub(np, cp).hi;
    return r;
}

// The reference's branch test |shift_hi - shift_lo| > min(dshift_max) on the FP64 shifts.
static __host__ __device__ __noinline__ bool large_shift_fp64(const double* hshift, double shift0, double cshift,
                                                       const double* dshift_max, Elem lo, Elem hi) {
    double lsh, lfac, hsh, hfac;
    const HalfSmem h{nullptr, const_cast<double*>(hshift), nullptr, nullptr, nullptr, nullptr, shift0, 0.0f, cshift};
    elem_shift_fac(h, lo, lsh, lfac);
    elem_shift_fac(h, hi, hsh, hfac);
    const double dshift_abs = fabs(dsub_rn(hsh, lsh));
    const double a = dshift_max[lo.nr], b = dshift_max[hi.nr];
    return dshift_abs > (a < b ? a : b);
}

// Elimination coefficients {dt_in/dt_out, dtau_avg dt_in} in FP64 for optical depths
// whose ratio or product would leave the FP32 range.
static __host__ __device__ __noinline__ double2 elim_coeffs_fp64(float dt_out, float dt_in) {
    const double o = dt_out, i = dt_in;
    double2 r;
    r.x = i / o;
    r.y = 0.5 * (o + i) * i;
    return r;
}

MGR_HD float dtau_single_line_f32(const DevModel& m, const LaneCtx& c, const HalfSmem& h, const Elem& lo,
                                  const Elem& hi, uint32_t l, float dz) {
    const size_t c1 = (size_t)lo.nr * m.L, c2 = (size_t)lo.ni * m.L;
    const size_t n1 = (size_t)hi.nr * m.L, n2 = (size_t)hi.ni * m.L;
    const float iwc = interpolate_linear(m.iw_f[c1 + l], m.iw_f[c2 + l], lo.facf);
    const float iwn = interpolate_linear(m.iw_f[n1 + l], m.iw_f[n2 + l], hi.facf);
    const float avg_iw = (iwc + iwn) * 0.5f;
    const float cop = interpolate_log(m.op_f[c1 + l], m.op_f[c2 + l], lo.facf);
    const float nop = interpolate_log(m.op_f[n1 + l], m.op_f[n2 + l], hi.facf);
    const float offc = offset_f32(m, c, lo.dsh, l);
    const float offn = offset_f32(m, c, hi.dsh, l);
    const float min_op = m.min_op_s;
    if (offc == offn) {
        const float prof = gaussian(avg_iw, offc);
        return dz * (prof * ((cop + nop) * 0.5f) + min_op);
    }
    const float next_pos = -offn * avg_iw;
    const float curr_pos = -offc * avg_iw;
    float erfdiff, diff_pos;
    const float amin = fminf(fabsf(next_pos), fabsf(curr_pos));
    if ((next_pos > 0.0f) == (curr_pos > 0.0f) && amin > 1.5f && amin < 3.919206f) {
        // Both positions in the same far wing: the reference's erff(next) - erff(curr)
        // cancels and its single-ulp roundings decide the result, so take it on the
        // FP64 mode's arguments with the correctly rounded erff (split precision then
        // stays within 1e-5 of the FP64 path in J).
        const float2 r = band_erf(m, c, h, lo, hi, l);
        erfdiff = r.x;
        diff_pos = r.y;
    } else {
        erfdiff = erff(next_pos) - erff(curr_pos);
        diff_pos = next_pos - curr_pos;
    }
    const float average_opacity = (nop + cop) * 0.5f;
    // Far from the line both FP32 positions can coincide while the FP64 ones differ;
    // both erf values saturate there and the reference's term is 0.
    const float erfterm = (erfdiff == 0.0f) ? 0.0f : average_opacity / diff_pos * 0.5f * erfdiff;
    return dz * (avg_iw * erfterm + min_op);
}

// compute_S_dtau_line_integrated<approx> in FP32; dz is the scaled FP32 distance.
template <int AP>
MGR_HD void pair_li_f32(const DevModel& m, const LaneCtx& c, const HalfSmem& h, const Elem& lo, const Elem& hi,
                        float dz, float& dtau, float& Slo, float& Shi) {
    const size_t c1 = (size_t)lo.nr * m.L, c2 = (size_t)lo.ni * m.L;
    const size_t n1 = (size_t)hi.nr * m.L, n2 = (size_t)hi.ni * m.L;
    const float fc = lo.facf, fn = hi.facf;
    if (AP == APPROX_ONELINE) {
        const uint32_t l = c.l0;
        dtau = dtau_single_line_f32(m, c, h, lo, hi, l, dz);
        Slo = interpolate_log(m.Sp_f[c1 + l], m.Sp_f[c2 + l], fc) * m.s_scale;
        Shi = interpolate_log(m.Sp_f[n1 + l], m.Sp_f[n2 + l], fn) * m.s_scale;
        return;
    }
    float sum_dtau = 0.0f, sum_c = 0.0f, sum_n = 0.0f;
    uint32_t a = 0, b = m.L;
    if (AP == APPROX_CLOSELINES) {
        const float oc = fmaf(c.fq, lo.dsh, c.a0);
        const float on = fmaf(c.fq, hi.dsh, c.a0);
        const float rf = c.fq + fmaxf(c.fq * lo.dsh, c.fq * hi.dsh);
        const float cb = m.max_dist_f * (rf * m.ub_f[lo.nr]);
        const float nb = m.max_dist_f * (rf * m.ub_f[hi.nr]);
        const float ubw = fmaxf(cb, nb);
        bracket_f32(m, c, fminf(oc, on) - ubw, fmaxf(oc, on) + ubw, a, b);
    }
    for (uint32_t s = a; s < b; s++) {
        const uint32_t l = (AP == APPROX_CLOSELINES) ? m.sorted_map[s] : s;
        const float ld = dtau_single_line_f32(m, c, h, lo, hi, l, dz);
        const float lsc = interpolate_log(m.Sp_f[c1 + l], m.Sp_f[c2 + l], fc);
        const float lsn = interpolate_log(m.Sp_f[n1 + l], m.Sp_f[n2 + l], fn);
        sum_dtau += ld;
        sum_c += ld * lsc;
        sum_n += ld * lsn;
    }
    if (AP == APPROX_NONE) {
        dtau = sum_dtau;
        Slo = sum_c / sum_dtau * m.s_scale;
        Shi = sum_n / sum_dtau * m.s_scale;
        return;
    }
    float d = sum_dtau;
    const float bound_min_dtau = m.min_op_s * dz;
    if (-bound_min_dtau < d) d = fmaxf(bound_min_dtau, d);
    dtau = d;
    Slo = sum_c / d * m.s_scale;
    Shi = sum_n / d * m.s_scale;
}

// Precision-dependent scalar of the pair quantities (optical depths, sources, opacities).
template <int MODE>
struct Real_ {
    using T = double;
};
template <>
struct Real_<MODE_SPLIT> {
    using T = float;
};

template <int MODE>
struct PairOut {
    typename Real_<MODE>::T dtau;  // optical depth increment between the two elements
    typename Real_<MODE>::T Slo;   // row source of the lower-index element if line-integrated
    typename Real_<MODE>::T Shi;   // source of the higher-index element if line-integrated
    bool large;
};

// Source/opacity cache of one element (trapezoid branch quantities; in split mode
// chi is in the scaled FP32 units).
template <int MODE>
struct EC {
    typename Real_<MODE>::T S, chi;
    bool ok;
};

template <int MODE, int AP>
MGR_HD void elem_fresh(const DevModel& m, const double* sl, const LaneCtx& c, const Elem& e, EC<MODE>& ec) {
    if (ec.ok) return;
    if constexpr (MODE == MODE_FP64) {
        double eta, chi;
        eta_chi_fp64<AP>(m, sl, c, e, eta, chi);
        ec.S = eta / chi;
        ec.chi = chi;
    } else {
        float eta, chi;
        eta_chi_f32<AP>(m, c, e, eta, chi);
        ec.S = fast_div(eta, chi) * m.s_scale;
        ec.chi = chi;
    }
    ec.ok = true;
}

// compute_source_dtau (solver.tpp:2139-2186) for the pair of `outer` (farther from
// the origin) and `inner`, both elements of the half `h` (or the origin); dz (FP64
// mode) or dzf (split, scaled FP32) is the pair's distance.  Every pair quantity is
// symmetric in its two elements (erf and position differences change sign together),
// so the reference's (lower index, higher index) order need not be kept: out.Slo is
// the source of `outer`, out.Shi that of `inner`, from the line integral or from the
// element caches (trapezoid rule).
template <int MODE, int AP>
MGR_HD void eval_pair(const DevModel& m, const double* sl, const LaneCtx& c, const HalfSmem& h, const Elem& outer,
                      const Elem& inner, double dz, float dzf, EC<MODE>& eco, EC<MODE>& eci, PairOut<MODE>& out) {
    if constexpr (MODE == MODE_FP64) {
        const double dshift_abs = fabs(dsub_rn(inner.shift, outer.shift));
        const double a = m.dshift_max[outer.nr], b = m.dshift_max[inner.nr];
        out.large = dshift_abs > (a < b ? a : b);
    } else {
        // the reference's branch test in FP32, and in FP64 within a margin of the
        // threshold that covers the FP32 roundings of the shifts
        const float dsf = fabsf(inner.dsh - outer.dsh);
        const float thr = fminf(m.dshift_max_f[outer.nr], m.dshift_max_f[inner.nr]);
        const float margin = 4.0e-3f * thr + 2.0e-6f * (outer.dshm + inner.dshm);
        if (fabsf(dsf - thr) > margin) out.large = dsf > thr;
        else out.large = large_shift_fp64(h.shift, h.shift0, h.cshift, m.dshift_max, outer, inner);
    }
    if (out.large) {
        if constexpr (MODE == MODE_FP64) {
            pair_li_fp64<AP>(m, sl, c, outer, inner, dz, out.dtau, out.Slo, out.Shi);
        } else {
            pair_li_f32<AP>(m, c, h, outer, inner, dzf, out.dtau, out.Slo, out.Shi);
        }
    } else {
        // one call site for both caches (the outer element's is usually the previous
        // pair's inner one): a second inlined copy of the line sum would only grow the
        // loop's code
#pragma unroll 1
        for (int k = 0; k < 2; k++) {
            if (k ? eci.ok : eco.ok) continue;
            EC<MODE> r{};
            elem_fresh<MODE, AP>(m, sl, c, k ? inner : outer, r);
            if (k) eci = r;
            else eco = r;
        }
        out.Slo = eco.S;
        out.Shi = eci.S;
        if constexpr (MODE == MODE_FP64) {
            out.dtau = 0.5 * (eco.chi + eci.chi) * dz;
        } else {
            out.dtau = 0.5f * (eco.chi + eci.chi) * dzf;
        }
    }
}

// Reciprocal of a positive finite value.  FP64 mode: IEEE division, as the reference.
// Split mode: the hardware's approximate FP64 reciprocal (relative error below 2^-22)
// refined by one Newton step (relative error ~1e-14).
template <int MODE>
MGR_HD double drcp(double x) {
    if (MODE == MODE_FP64) return 1.0 / x;
#ifdef __CUDA_ARCH__
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    return fma(r, fma(-x, r, 1.0), r);
#else
    return 1.0 / x;
#endif
}

// Exact conversion of a finite FP32 value to FP64 on the integer pipe (the FP64 pipe
// is the scarce unit of this kernel).  Subnormal inputs become 0.
MGR_HD double f2d(float x) {
#ifdef __CUDA_ARCH__
    const uint32_t b = __float_as_uint(x);
    const uint32_t mag = b & 0x7fffffffu;
    if (mag < 0x00800000u) return 0.0;
    const uint32_t hi = ((mag >> 3) + 0x38000000u) | (b & 0x80000000u);  // exponent bias 127 -> 1023
    return __hiloint2double((int)hi, (int)(b << 29));
#else
    return (std::fabs(x) < FLT_MIN) ? 0.0 : (double)x;
#endif
}

// The FP64 Planck function out of line (split precision's boundary intensities
// beyond h nu / k T = 40).
static __host__ __device__ __noinline__ double planck_cold(double temp, double freq) { return planck(temp, freq); }

// 2h/c^2 2^108 as a double-float: with nu scaled by 2^-36, nu^3 and the product stay
// normal floats for every nu between 1e8 and 1e16 Hz.
constexpr double kPlanckScaled = TWO_HH_OVER_CC_SQUARED * 0x1p108;
constexpr float kPlanckHi = (float)kPlanckScaled;
constexpr float kPlanckLo = (float)(kPlanckScaled - (double)kPlanckHi);

// Split precision's boundary intensity (Solver::boundary_intensity / planck,
// solver.tpp:1119-1142) without FP64 arithmetic, at the double-float frequency nu:
//   x = h nu / (k T)  as a double-float product, rounded once to the float the
//       reference passes to expm1f (the reference rounds its FP64 quotient; the two
//       agree except within ~1e-14 of a rounding boundary),
//   B = (2h/c^2 2^108) (nu 2^-36)^3 / expm1f(x)  as double-float products and a
//       double-float quotient (q = fl(N / e), then the exact remainder N - q e over e),
// so B carries ~1e-14 relative error against the FP64 expression instead of the FP32
// roundings of nu, T and nu^3.  Beyond x = 40 (B below 1e-17 of its peak), the FP64
// expression.
MGR_HD double boundary_intensity_f2(const DevModel& m, uint32_t p, F2 nu) {
    const uint32_t b = m.p2b[p];
    if (b >= m.B) return 0.0;
    if (m.bc[b] == BC_ZERO) return 0.0;
    const F2 x = f2_mul(nu, F2{m.bkt[2 * b], m.bkt[2 * b + 1]});
    if (!(x.hi < 40.0f)) return planck_cold(m.bc[b] == BC_THERMAL ? m.bt[b] : T_CMB, (double)nu.hi + (double)nu.lo);
    const F2 n{nu.hi * 0x1p-36f, nu.lo * 0x1p-36f};
    const F2 num = f2_mul(f2_mul(f2_mul(n, n), n), F2{kPlanckHi, kPlanckLo});
    const float e = expm1f(x.hi);
    const float q = num.hi / e;
    const float q2 = (fmaf(-q, e, num.hi) + num.lo) / e;
    return (double)q + (double)q2;
}

// Split-precision Planck function / boundary intensity: the reference's expressions
// with the two divisions as reciprocals.
template <int MODE>
MGR_HD double boundary_intensity_m(const DevModel& m, uint32_t p, double freq) {
    if constexpr (MODE == MODE_FP64) {
        return boundary_intensity(m, p, freq);
    } else {
        const uint32_t b = m.p2b[p];
        if (b >= m.B) return 0.0;
        const int c = m.bc[b];
        if (c == BC_ZERO) return 0.0;
        const double temp = (c == BC_THERMAL) ? m.bt[b] : T_CMB;
        const float x = (float)(HH_OVER_KB * freq * drcp<MODE>(temp));
        return TWO_HH_OVER_CC_SQUARED * (freq * freq * freq) * drcp<MODE>((double)expm1f(x));
    }
}

// One interior elimination row in the economical (1+B)/C form (solver.tpp:2266-2281
// forward, :2304-2309 backward): `dt_out` is the optical depth of the pair already
// eliminated, `dt_in` of the pair toward the origin.  F, FI = 1/(1+F) and the modified
// source Su are updated in place:
//     F' = (A F FI + 1) C^-1,  FI' = 1/(1 + F'),  Su' = (A Su + S) FI' C^-1
// with A = 1/(dtau_avg dt_out), C^-1 = dtau_avg dt_in.  Split mode forms the
// coefficients A C^-1 = dt_in/dt_out and C^-1 from the FP32 optical depths and keeps
// the recurrence in FP64.
template <int MODE>
MGR_HD void elim_row(typename Real_<MODE>::T dt_out, typename Real_<MODE>::T dt_in, typename Real_<MODE>::T S,
                     double& F, double& FI, double& Su) {
    if constexpr (MODE == MODE_FP64) {
        const double dtau_avg = 0.5 * (dt_out + dt_in);
        const double iA = dtau_avg * dt_out;
        const double iC = dtau_avg * dt_in;
        const double A = 1.0 / iA;
        F = (A * F * FI + 1.0) * iC;
        FI = 1.0 / (1.0 + F);
        Su = (A * Su + S) * FI * iC;
    } else {
        if (dt_out > 1.0e-18f && dt_out < 1.0e18f && dt_in > 1.0e-18f && dt_in < 1.0e18f) {
            // q, iC in [1e-36, 1e36]: F = q G + iC stays below 2e36, a safe pivot range
            const double q = f2d(fast_div(dt_in, dt_out));
            const double iC = f2d(0.5f * (dt_out + dt_in) * dt_in);
            F = fma(q, F * FI, iC);
            FI = drcp<MODE>(1.0 + F);
            Su = fma(q, Su, f2d(S) * iC) * FI;
        } else {
            const double2 k = elim_coeffs_fp64(dt_out, dt_in);
            F = fma(k.x, F * FI, k.y);
            FI = 1.0 / (1.0 + F);
            Su = fma(k.x, Su, (double)S * k.y) * FI;
        }
    }
}

// Split precision, the elimination in projective form.  A sweep keeps (NG, D, NS)
// with G = F / (1 + F) = NG / D and Su = NS / D, and D_prev = D - NG (so that
// 1 / (1 + F) = D_prev / D).  A row
//     F' = q G + iC,  Su' = (q Su + S iC) / (1 + F')
// becomes, multiplied through by D' = D (1 + F'),
//     NG' = q NG + iC D,   D' = NG' + D,   NS' = q NS + S iC D:
// five FP64 operations and no reciprocal per element, all of them sums of positive
// terms as in the (1+B)/C form.  D never decreases; the state is scaled by 2^-600
// (exact) once D passes 2^600, well before it could leave the FP64 range (one row
// multiplies D by 1 + F' < 2^122).
struct Proj {
    double NG, D, NS, Dp;
};

MGR_HD void proj_rescale(Proj& s) {
#ifdef __CUDA_ARCH__
    const bool big = __double2hiint(s.D) > 0x65700000;  // D > 2^600
#else
    const bool big = s.D > 0x1p600;
#endif
    if (big) {
        s.NG *= 0x1p-600;
        s.D *= 0x1p-600;
        s.NS *= 0x1p-600;
        s.Dp *= 0x1p-600;
    }
}

MGR_HD void elim_row_proj(float dt_out, float dt_in, float S, Proj& s) {
    double q, iC;
    if (dt_out > 1.0e-18f && dt_out < 1.0e18f && dt_in > 1.0e-18f && dt_in < 1.0e18f) {
        q = f2d(fast_div(dt_in, dt_out));
        iC = f2d(0.5f * (dt_out + dt_in) * dt_in);
    } else {
        const double2 k = elim_coeffs_fp64(dt_out, dt_in);
        q = k.x;
        iC = k.y;
    }
    const double iCD = iC * s.D;
    s.Dp = s.D;
    s.NG = fma(q, s.NG, iCD);
    s.NS = fma(q, s.NS, f2d(S) * iCD);
    s.D = s.NG + s.D;
    proj_rescale(s);
}

// Result of one lane's ray-pair solve.
struct LaneResult {
    double u;       // Su[centre]
    double Ldiag;   // L_diag[centre]
    bool solved;    // n_tot > 1
    double v;       // Sv[centre] of the uv solve (solve_lane<..., UV = true> only)
    double dtm, dtp;  // the uv solve's optical depths of the pairs before / after the origin
};

// State of one elimination sweep toward the origin.
struct Sweep {
    double F, FI, Su;  // F (top) / G (bottom), 1/(1+F), modified source
    double dt;         // optical depth of the last pair (next to the origin)
    double S_in;       // source of the origin from the last pair (its inner element)
    bool rows;         // at least one row eliminated
    // uv solve only: the last pair's branch, its outer element's opacity, its distance
    bool last_large;
    double chi_out, dz_last;
    float dtf = 0.0f, S_inf = 0.0f;  // dt and S_in as the split sweep's floats
};

// Non-local ALO (n_off_diag > 0, FP64 mode): the last NB + 1 rows of one sweep as it
// reaches the origin, so that the band entries of the inverse Feautrier matrix next
// to the origin can be formed once both sweeps are done (band_tail).
template <int NB>
struct BandRing {
    double F[NB + 1];    // FF (backward half) or GG (forward half) of the row
    double dt[NB + 1];   // optical depth of the row's pair toward the origin
    double sh[NB + 1];   // the row element's shift
    uint32_t nr[NB + 1]; // the row element's point
    int rows = 0;        // rows eliminated so far (the ring holds the last NB + 1)
};

// In: K (the model's n_off_diag, at most NB) and w_rr (the ray pair's weight).  Out:
// the update_Lambda terms of the elements centre - m - 1 (slot m) and centre + m + 1
// (slot K + m), m < K, and their points; 0 and the origin where the ray ends first.
template <int NB>
struct BandOut {
    uint32_t K;
    double w_rr;
    double val[2 * NB + 1];
    uint32_t nr[2 * NB + 1];
};

template <int NB>
MGR_HD void band_tail(const DevModel& m, const double* sl, const LaneCtx& c, const BandRing<NB>& tp,
                      const BandRing<NB>& bt, BandOut<NB>& out);

// Two-sided Feautrier solve of frequency c.f on the ray pair staged in `bk`
// (backward half, direction rr) and `fw` (forward half, antipode).  Both halves run
// through the same sweep code (outer end first):
//   backward half: elements first .. centre, rows first .. centre-1 with row source
//                  S[i] from pair (i, i+1) = this pair's outer element;
//   forward half:  elements last .. centre+1, row `last` with the source of its own
//                  pair, rows i < last with S[i] from pair (i, i+1) = the previous
//                  pair's inner element.
// NB > 0 (FP64 mode): also the non-local ALO terms of the K = bo->K band elements on
// each side of the origin (solver.tpp:2319-2355, :1800-1846).
template <int MODE, int AP, bool UV = false, int NB = 0>
__host__ __device__ LaneResult solve_lane(const DevModel& m, const double* sl, const LaneCtx& c, const HalfSmem& bk,
                                          int nb, const HalfSmem& fw, int nf, BandOut<NB>* bo = nullptr) {
    static_assert(NB == 0 || (MODE == MODE_FP64 && !UV), "band elements: FP64 mode, J / ALO solve");
    using T = typename Real_<MODE>::T;
    // split precision eliminates in projective form (the uv solve keeps the (F, FI, Su)
    // state its origin rows need)
    constexpr bool PROJ = (MODE == MODE_SPLIT) && !UV;
    LaneResult res;
    res.solved = (nb > 0) || (nf > 0);
    res.v = 0.0;
    res.dtm = res.dtp = 0.0;
    // the origin's own boundary intensity (no ray pair, or a one-sided one: boundary
    // origins only; 0 at once for interior points), evaluated at one site
    double Io;
    if constexpr (MODE == MODE_SPLIT) Io = boundary_intensity_f2(m, c.o, F2{c.fq, c.fql});
    else Io = boundary_intensity_m<MODE>(m, c.o, c.freq);
    if (!res.solved) {
        res.u = Io;
        res.Ldiag = 0.0;
        return res;
    }
    const Elem cen = centre_elem(c.o);
    const uint32_t l = c.l0;
    EC<MODE> ec_cen{T(0), T(0), false};
    Sweep top{0.0, 0.0, 0.0, 0.0, 0.0, false, false, 0.0, 0.0}, bot = top;
    Proj ptop{0.0, 1.0, 0.0, 1.0}, pbot = ptop;
    BandRing<NB> rtop{}, rbot{};

#pragma unroll 1
    for (int side = 0; side < 2; side++) {
        const HalfSmem& h = side ? fw : bk;
        const int n = side ? nf : nb;
        Sweep st{0.0, 0.0, 0.0, 0.0, 0.0, false, false, 0.0, 0.0};
        Proj ps{0.0, 1.0, 0.0, 1.0};
        if (n > 0) {
            ElemIter it;
            iter_begin<MODE>(m, h, c.o, l, n, it);
            Elem outer;
            EC<MODE> ec_out{T(0), T(0), false};
            double Ibdy = 0.0;
            T dt_prev = T(0), S_carry = T(0);
            bool first = true, have_outer = false;
            while (true) {
                // one iter_next site: the first element taken is the half's outer end
                Elem inner;
                const bool more = iter_next<MODE>(m, h, c.o, l, it, inner);
                if (!more) inner = cen;
                if (!have_outer) {
                    outer = inner;
                    have_outer = true;
                    if constexpr (MODE == MODE_SPLIT) {
                        // at the outer element's frequency nu shift = nu + nu (shift - 1), double-float
                        const F2 nu{c.fq, c.fql};
                        Ibdy = boundary_intensity_f2(m, outer.nr, f2_add(nu, f2_mul(nu, elem_dsh_f2(h, outer))));
                    } else {
                        Ibdy = boundary_intensity_m<MODE>(m, outer.nr, c.freq * outer.shift);
                    }
                    continue;
                }
                EC<MODE> ec_inn{T(0), T(0), false};
                EC<MODE>& eci = more ? ec_inn : ec_cen;
                PairOut<MODE> po;
                eval_pair<MODE, AP>(m, sl, c, h, outer, inner, outer.dzin, outer.dzf, ec_out, eci, po);
                if constexpr (UV) {
                    st.last_large = po.large;
                    st.chi_out = (double)ec_out.chi;
                    st.dz_last = (MODE == MODE_FP64) ? outer.dzin : (double)outer.dzf;
                }
                const T rowS = (side == 0 || first) ? po.Slo : S_carry;
                if (PROJ && first) {
                    // boundary row multiplied through by dtau^2/2: F = h = dtau (dtau/2 + 1),
                    // Su = (S dtau^2/2 + I_bdy dtau) / (1 + h); from the FP32 dtau, as the
                    // interior rows form their coefficients, but h with one FP64 FMA: in
                    // FP32 the factor 1 + dtau/2 rounds away dtau/2 below ~1e-7, and
                    // NS / NG, the boundary intensity the sweep carries, with it
                    const float dtf = (float)po.dtau;
                    const double dt = f2d(dtf);
                    const double hb = fma(f2d(0.5f * dtf), dt, dt);
                    ps.NG = hb;
                    ps.D = 1.0 + hb;
                    ps.NS = fma(f2d((float)rowS * 0.5f) * dt, dt, Ibdy * dt);
                    ps.Dp = 1.0;
                    first = false;
                } else if (PROJ) {
                    elim_row_proj((float)dt_prev, (float)po.dtau, (float)rowS, ps);
                } else if (first) {
                    // boundary row (solver.tpp:2239-2252 first, :2284-2293 last)
                    const double dt = po.dtau;
                    const double inverse_dtau = drcp<MODE>(dt);
                    const double Cb = 2.0 * inverse_dtau * inverse_dtau;
                    const double Bb_min_Cb = 1.0 + 2.0 * inverse_dtau;
                    const double Bb = Bb_min_Cb + Cb;
                    if constexpr (MODE == MODE_FP64) st.Su = ((double)rowS + 2.0 * Ibdy * inverse_dtau) / Bb;
                    else st.Su = ((double)rowS + 2.0 * Ibdy * inverse_dtau) * drcp<MODE>(Bb);
                    st.F = 0.5 * Bb_min_Cb * dt * dt;
                    st.FI = drcp<MODE>(1.0 + st.F);
                    first = false;
                } else {
                    elim_row<MODE>(dt_prev, po.dtau, rowS, st.F, st.FI, st.Su);
                }
                if constexpr (NB > 0) {
                    BandRing<NB>& rg = side ? rbot : rtop;
                    const int r = rg.rows % (NB + 1);
                    rg.F[r] = st.F;
                    rg.dt[r] = (double)po.dtau;
                    rg.nr[r] = outer.nr;
                    rg.sh[r] = outer.shift;
                    rg.rows++;
                }
                dt_prev = po.dtau;
                S_carry = po.Shi;
                if (!more) break;
                outer = inner;
                ec_out = ec_inn;
            }
            st.dt = dt_prev;
            st.S_in = S_carry;
            st.dtf = (float)dt_prev;
            st.S_inf = (float)S_carry;
            st.rows = true;
        }
        if (side) {
            bot = st;
            pbot = ps;
        } else {
            top = st;
            ptop = ps;
        }
    }

    if constexpr (NB > 0) band_tail<NB>(m, sl, c, rtop, rbot, *bo);

    if constexpr (PROJ) {
        if (top.rows && bot.rows) {
            // the origin's row in projective form with elim_row_proj's FP32 coefficients
            // q = dtau_b / dtau_t, iC = (dtau_t + dtau_b) dtau_b / 2:
            //   u = (q Su_t + S_in iC + Su_b) / (q G_t + iC + G_b),  L_diag = iC / (same)
            // (the reference's u[c] and L_diag[c], with G = NG / D, Su = NS / D per side)
            const float dto = top.dtf, dti = bot.dtf;
            double q, iC;
            if (dto > 1.0e-18f && dto < 1.0e18f && dti > 1.0e-18f && dti < 1.0e18f) {
                q = f2d(fast_div(dti, dto));
                iC = f2d(0.5f * (dto + dti) * dti);
            } else {
                const double2 k = elim_coeffs_fp64(dto, dti);
                q = k.x;
                iC = k.y;
            }
            const double qrt = q * drcp<MODE>(ptop.D);
            const double rb = drcp<MODE>(pbot.D);
            const double num = fma(qrt, ptop.NS, fma(rb, pbot.NS, f2d(bot.S_inf) * iC));
            const double rd = drcp<MODE>(fma(qrt, ptop.NG, fma(rb, pbot.NG, iC)));
            res.u = num * rd;
            res.Ldiag = iC * rd;
            return res;
        }
        // one-sided rays: back to (F / (1 + F), 1 / (1 + F), Su) at the origin
        if (top.rows) {
            const double r = drcp<MODE>(ptop.D);
            top.F = ptop.NG * r;  // G
            top.FI = ptop.Dp * r;
            top.Su = ptop.NS * r;
        }
        if (bot.rows) {
            const double r = drcp<MODE>(pbot.D);
            bot.F = pbot.NG * r;
            bot.FI = pbot.Dp * r;
            bot.Su = pbot.NS * r;
        }
    }

    // ---- combine at the origin ----
    if (top.rows && bot.rows) {
        const double dtau_avg = 0.5 * (top.dt + bot.dt);
        const double iA = dtau_avg * top.dt;
        const double iC = dtau_avg * bot.dt;
        const double A = drcp<MODE>(iA);
        const double FFc = (A * (PROJ ? top.F : top.F * top.FI) + 1.0) * iC;
        const double Su_pre = (A * top.Su + bot.S_in) * iC;
        const double GP = PROJ ? bot.F : bot.F * bot.FI;
        const double D = drcp<MODE>(FFc + GP);
        res.u = (Su_pre + bot.Su) * D;
        res.Ldiag = iC * D;
        if constexpr (UV) {
            // solve_feautrier_order_2_uv (solver.tpp:2896-2916): u at the neighbours of the
            // origin from each side's last row, v the finite-difference derivative
            const double u_min = top.Su + res.u * top.FI;
            const double u_plus = bot.Su + res.u * bot.FI;
            const double dtaumin = (double)top.dt;
            double dtauplus = (double)bot.dt;
            if (!top.last_large && !bot.last_large) {
                // The reference evaluates the pair (origin, next) with compute_curr_opacity
                // left false by the pair (previous, origin), so its "current" opacity is
                // that of the previous element (solver.tpp:2899-2907, :2161-2170).
                if constexpr (MODE == MODE_FP64) dtauplus = 0.5 * (top.chi_out + bot.chi_out) * bot.dz_last;
                else dtauplus = (double)(0.5f * ((float)top.chi_out + (float)bot.chi_out) * (float)bot.dz_last);
            }
            res.dtm = dtaumin;
            res.dtp = dtauplus;
            const double coeffmin = -dtauplus / (dtaumin * dtaumin + dtaumin * dtauplus);
            const double coeffplus = dtaumin / (dtaumin * dtauplus + dtauplus * dtauplus);
            const double coeffzero = -coeffmin - coeffplus;
            res.v = -(coeffmin * u_min + coeffplus * u_plus + coeffzero * res.u);
        }
    } else if (bot.rows) {  // origin is the first element
        const double Ibdy = Io;
        const double inverse_dtau_f = drcp<MODE>(bot.dt);
        const double Cf = 2.0 * inverse_dtau_f * inverse_dtau_f;
        const double Bf_min_Cf = 1.0 + 2.0 * inverse_dtau_f;
        const double Bf = Bf_min_Cf + Cf;
        double Suf;
        if constexpr (MODE == MODE_FP64) Suf = (bot.S_in + 2.0 * Ibdy * inverse_dtau_f) / Bf;
        else Suf = (bot.S_in + 2.0 * Ibdy * inverse_dtau_f) * drcp<MODE>(Bf);
        const double FFf = 0.5 * Bf_min_Cf * bot.dt * bot.dt;
        const double GP = PROJ ? bot.F : bot.F * bot.FI;
        const double D = drcp<MODE>(FFf + GP);
        res.u = (Suf * (1.0 + FFf) + bot.Su) * D;
        res.Ldiag = drcp<MODE>(Cf) * D;
        if constexpr (UV) res.v = Ibdy - res.u;  // Sv[first] = I_bdy_f - Su[first]
    } else {  // origin is the last element
        const double Ibdy = Io;
        const double inverse_dtau_l = drcp<MODE>(top.dt);
        const double Al = 2.0 * inverse_dtau_l * inverse_dtau_l;
        const double Bl_min_Al = 1.0 + 2.0 * inverse_dtau_l;
        const double Bl = Bl_min_Al + Al;
        const double Sl = top.S_in + 2.0 * Ibdy * inverse_dtau_l;
        if constexpr (PROJ) {
            // with G = F / (1 + F) and FI = 1 / (1 + F): (1 + F) / (Bl F + Bl - Al) = 1 / (Bl G + (Bl - Al) FI)
            const double den = drcp<MODE>(Bl * top.F + Bl_min_Al * top.FI);
            res.u = (Al * top.Su + Sl) * den;
            res.Ldiag = den;
        } else {
            const double denominator = drcp<MODE>(Bl * top.F + Bl_min_Al);
            res.u = (Al * top.Su + Sl) * (1.0 + top.F) * denominator;
            if constexpr (UV) res.v = res.u - Ibdy;  // Sv[last] = Su[last] - I_bdy_l
            if constexpr (MODE == MODE_FP64) res.Ldiag = (1.0 + top.F) / (Bl_min_Al + Bl * top.F);
            else res.Ldiag = (1.0 + top.F) * denominator;
        }
    }
    return res;
}

// Imagers (Solver::image_feautrier_order_2(model, o, f), solver.tpp:2462-2574): the
// forward elimination over the whole ray, elements first .. last = the backward half
// (outer to inner), the origin, and the forward half (inner to outer); the pixel is
// 2 Su[last] - I_bdy(nr[last], nu(o, f)), Su[last] being the last row's solution.  The
// ray's elements use all-line interpolation (kAllLines) and the halves' shift0.  With
// nf = 0 (new imager) the origin itself is the last element.
//
// ROWS (Solver::image_feautrier_order_2_for_point_loc, solver.tpp:2582-2715): the lane
// also writes, per element k of the ray (row k, stride ro->F, column c.f), the source at
// the far end of the pair ending there (row 0: the first pair's near end), that pair's
// optical depth (row 0: 0) and, after back substitution u[k] = Su[k] + FI[k] u[k+1], the
// Feautrier mean intensity; ro->FI holds the rows' FI meanwhile.
struct RowOut {
    double* S;
    double* dtau;
    double* u;
    double* FI;
    uint32_t F;
};

template <int MODE, int AP, bool TAU = false, bool ROWS = false>
__host__ __device__ double image_lane(const DevModel& m, const double* sl, const LaneCtx& c, const HalfSmem& bk,
                                      int nb, const HalfSmem& fw, int nf, const RowOut* ro = nullptr) {
    using T = typename Real_<MODE>::T;
    if (nb <= 0 && nf <= 0) return TAU ? 0.0 : boundary_intensity(m, c.o, c.freq);
    size_t row = 0;  // ROWS: index of the row the current pair ends on, times F
    const size_t rstep = ROWS ? ro->F : 0;
    const Elem cen = centre_elem(c.o, bk.cshift, (float)dsub_rn(bk.cshift, 1.0));
    ElemIter ib, iu;
    int phase;  // 0: backward half, 2: forward half, 3: done
    Elem prev;
    if (nb > 0) {
        iter_begin<MODE>(m, bk, c.o, kAllLines, nb, ib);
        iter_next<MODE>(m, bk, c.o, kAllLines, ib, prev);
        phase = 0;
    } else {
        prev = cen;
        iter_up_begin<MODE>(m, fw, c.o, kAllLines, nf, iu);
        phase = 2;
    }
    const HalfSmem& h_first = (nb > 0) ? bk : fw;
    double bshift = prev.shift;
    if constexpr (MODE == MODE_SPLIT) {
        double fac;
        elem_shift_fac(h_first, prev, bshift, fac);
    }
    const double Ibdy_f = boundary_intensity(m, prev.nr, c.freq * bshift);
    EC<MODE> ec_prev{T(0), T(0), false};
    double tau = 0.0;
    Sweep st{0.0, 0.0, 0.0, 0.0, 0.0, false};
    T dt_prev = T(0), S_last = T(0);
    Elem last = prev;
    bool first = true;
    while (true) {
        Elem cur;
        bool from_fw = false;
        if (phase == 0) {
            if (!iter_next<MODE>(m, bk, c.o, kAllLines, ib, cur)) {
                cur = cen;
                phase = 1;
            }
        } else {
            if (phase == 1) {
                iter_up_begin<MODE>(m, fw, c.o, kAllLines, nf, iu);
                phase = 2;
            }
            if (!iter_up_next<MODE>(m, fw, c.o, kAllLines, iu, cur)) break;
            from_fw = true;
        }
        const HalfSmem& h = from_fw ? fw : bk;
        const double dz = from_fw ? cur.dzin : prev.dzin;
        const float dzf = from_fw ? cur.dzf : prev.dzf;
        EC<MODE> ec_cur{T(0), T(0), false};
        PairOut<MODE> po;
        eval_pair<MODE, AP>(m, sl, c, h, prev, cur, dz, dzf, ec_prev, ec_cur, po);
        if constexpr (TAU) {
            // image_optical_depth (solver.tpp:2718-2760): the pairs' optical depths summed
            // from first to last
            tau += (double)po.dtau;
        } else if (first) {
            const double dt = po.dtau;
            const double inverse_dtau = drcp<MODE>(dt);
            const double Cb = 2.0 * inverse_dtau * inverse_dtau;
            const double Bb_min_Cb = 1.0 + 2.0 * inverse_dtau;
            const double Bb = Bb_min_Cb + Cb;
            if constexpr (MODE == MODE_FP64) st.Su = ((double)po.Slo + 2.0 * Ibdy_f * inverse_dtau) / Bb;
            else st.Su = ((double)po.Slo + 2.0 * Ibdy_f * inverse_dtau) * drcp<MODE>(Bb);
            st.F = 0.5 * Bb_min_Cb * dt * dt;
            st.FI = drcp<MODE>(1.0 + st.F);
            first = false;
            if constexpr (ROWS) {
                ro->S[c.f] = (double)po.Slo;
                ro->dtau[c.f] = 0.0;
            }
        } else {
            elim_row<MODE>(dt_prev, po.dtau, po.Slo, st.F, st.FI, st.Su);
        }
        if constexpr (ROWS) {
            ro->u[row + c.f] = st.Su;
            ro->FI[row + c.f] = st.FI;
            row += rstep;
            ro->S[row + c.f] = (double)po.Shi;
            ro->dtau[row + c.f] = (double)po.dtau;
        }
        dt_prev = po.dtau;
        S_last = po.Shi;
        last = cur;
        prev = cur;
        ec_prev = ec_cur;
        if (phase == 1 && nf <= 0) break;  // the origin is the last element
    }
    if constexpr (TAU) return tau;
    // last row (solver.tpp:2284-2297)
    double lshift = last.shift;
    if constexpr (MODE == MODE_SPLIT) {
        double fac;
        elem_shift_fac((nf > 0) ? fw : bk, last, lshift, fac);
    }
    const double Ibdy_l = boundary_intensity(m, last.nr, c.freq * lshift);
    const double dtl = dt_prev;
    const double inverse_dtau_l = drcp<MODE>(dtl);
    const double Al = 2.0 * inverse_dtau_l * inverse_dtau_l;
    const double Bl_min_Al = 1.0 + 2.0 * inverse_dtau_l;
    const double Bl = Bl_min_Al + Al;
    const double denominator = drcp<MODE>(Bl * st.F + Bl_min_Al);
    const double Sl = (double)S_last + 2.0 * Ibdy_l * inverse_dtau_l;
    const double u = (Al * st.Su + Sl) * (1.0 + st.F) * denominator;
    if constexpr (ROWS) {
        double un = u;
        ro->u[row + c.f] = un;
        while (row > 0) {
            row -= rstep;
            un = ro->u[row + c.f] + un * ro->FI[row + c.f];
            ro->u[row + c.f] = un;
        }
    }
    return 2.0 * u - boundary_intensity(m, last.nr, c.freq);
}

// Result of one lane's short-characteristics solve.
struct LaneResultSC {
    double If;   // intensity at the origin along rr (integrated over the backward half)
    double Ib;   // along the antipode (integrated over the forward half)
    double Xf;   // (expm1f(-dtau)/dtau + 1) of the last pair of each half, 0 if the half is empty
    double Xb;
    bool solved; // n_tot > 1
};

// Solver::solve_shortchar_order_0_ray_forward / _backward (solver.tpp:1564-1757):
// each half is integrated from its outer end to the origin,
//   I = e^{-dtau} I + expm1(-dtau)/dtau (S_c - S_n (1 + dtau)) + S_c - S_n,
// with S_c / S_n the sources of the pair's outer / inner element (the line-integrated
// ones for large Doppler jumps) and dtau >= min_dtau.  The reference evaluates the
// exponentials in single precision; FP64 mode uses correctly rounded single-precision
// values (expf_cr / expm1f_cr, as the oracle's matching mode) because the update's
// cancellation makes J depend on their last ulp.  The pair evaluation is the
// Feautrier path's.
template <int MODE, int AP>
__host__ __device__ LaneResultSC solve_lane_sc0(const DevModel& m, const double* sl, const LaneCtx& c,
                                                const HalfSmem& bk, int nb, const HalfSmem& fw, int nf) {
    using T = typename Real_<MODE>::T;
    LaneResultSC res;
    res.solved = (nb > 0) || (nf > 0);
    res.Xf = 0.0;
    res.Xb = 0.0;
    if (!res.solved) {
        res.If = res.Ib = boundary_intensity(m, c.o, m.nu[(size_t)c.o * m.F + c.f]);
        return res;
    }
    const Elem cen = centre_elem(c.o);
    const uint32_t l = c.l0;
    EC<MODE> ec_cen{T(0), T(0), false};
#pragma unroll 1
    for (int side = 0; side < 2; side++) {
        const HalfSmem& h = side ? fw : bk;
        const int n = side ? nf : nb;
        double I, X = 0.0;
        if (n == 0) {
            I = boundary_intensity(m, c.o, c.freq);  // nr[first] = o, shift 1
        } else {
            ElemIter it;
            iter_begin<MODE>(m, h, c.o, l, n, it);
            Elem outer;
            iter_next<MODE>(m, h, c.o, l, it, outer);
            EC<MODE> ec_out{T(0), T(0), false};
            double bshift = outer.shift;
            if constexpr (MODE == MODE_SPLIT) {
                double fac;
                elem_shift_fac(h, outer, bshift, fac);
            }
            I = boundary_intensity(m, outer.nr, c.freq * bshift);
            double dtau = 0.0;
            while (true) {
                Elem inner;
                const bool more = iter_next<MODE>(m, h, c.o, l, it, inner);
                if (!more) inner = cen;
                EC<MODE> ec_inn{T(0), T(0), false};
                EC<MODE>& eci = more ? ec_inn : ec_cen;
                PairOut<MODE> po;
                eval_pair<MODE, AP>(m, sl, c, h, outer, inner, outer.dzin, outer.dzf, ec_out, eci, po);
                dtau = (double)po.dtau;
                if (m.min_dtau > dtau) dtau = m.min_dtau;
                const double Sc = (double)po.Slo, Sn = (double)po.Shi;
                const float x = (float)(-dtau);
                const double ex = (MODE == MODE_FP64) ? (double)expf_cr(x) : (double)expf(x);
                const double em = (MODE == MODE_FP64) ? (double)expm1f_cr(x) : (double)expm1f(x);
                // evaluated as the reference's uncontracted expression: for tiny dtau the
                // terms cancel to rounding level, so a fused multiply-add would change J
                const double t = dsub_rn(Sc, dmul_rn(Sn, dadd_rn(1.0, dtau)));
                I = dsub_rn(dadd_rn(dadd_rn(dmul_rn(ex, I), dmul_rn(em / dtau, t)), Sc), Sn);
                if (!more) break;
                outer = inner;
                ec_out = ec_inn;
            }
            const float x = (float)(-dtau);
            X = (double)((MODE == MODE_FP64) ? expm1f_cr(x) : expm1f(x)) / dtau + 1.0;
        }
        if (side) {
            res.Ib = I;
            res.Xb = X;
        } else {
            res.If = I;
            res.Xf = X;
        }
    }
    return res;
}

// update_Lambda, n_off_diag = 0 (solver.tpp:1760-1800): the ALO element of this
// (origin, ray pair, frequency).
struct LambdaFactors {
    double Aqw;          // line_A * quadrature weight
    double frq;          // nu(o, f)
    double phi;          // line profile at nu(o, f)
    double inverse_chi;  // 1 / opacity at the origin
};

// The ray-independent factors of the ALO element of (origin o, frequency f).
MGR_HD LambdaFactors lambda_factors(const DevModel& m, const double* sl, uint32_t o, uint32_t f) {
    const uint32_t ls = m.corr_lspec[f];
    const uint32_t k = m.corr_k[f];
    const uint32_t z = m.corr_z[f];
    const uint32_t lid = m.nrad_cum[ls] + k;
    const double freq_line = m.line[lid];
    const double invr_mass = m.lspec_inv_mass[ls];
    LambdaFactors r;
    r.Aqw = m.line_A[lid] * m.quad_w[(size_t)ls * m.Q + z];
    double eta, chi;
    get_eta_and_chi(m, sl, o, k, freq_line, eta, chi);  // the reference passes k as the line index here
    r.inverse_chi = 1.0 / chi;
    r.frq = m.nu[(size_t)o * m.F + f] * 1.0;
    r.phi = thermo_profile(m, invr_mass, o, freq_line, r.frq);
    return r;
}

// The element itself, with the reference's order of operations:
// constante * frq * phi * L_diag * inverse_chi, constante = line_A * weight * 2 w_rr.
MGR_HD double lambda_element(const LambdaFactors& k, double w_rr, double Ldiag) {
    const double constante = k.Aqw * (2.0 * w_rr);
    return constante * k.frq * k.phi * Ldiag * k.inverse_chi;
}

// The update_Lambda factors of element n of the ray (point p, shift sh) for
// frequency f (solver.tpp:1811-1846): chi at p for line k, nu(p, f) sh and the profile
// of p there.
MGR_HD LambdaFactors lambda_factors_at(const DevModel& m, const double* sl, uint32_t p, uint32_t f, double sh) {
    const uint32_t ls = m.corr_lspec[f];
    const uint32_t k = m.corr_k[f];
    const uint32_t z = m.corr_z[f];
    const uint32_t lid = m.nrad_cum[ls] + k;
    const double freq_line = m.line[lid];
    const double invr_mass = m.lspec_inv_mass[ls];
    LambdaFactors r;
    r.Aqw = m.line_A[lid] * m.quad_w[(size_t)ls * m.Q + z];
    double eta, chi;
    get_eta_and_chi(m, sl, p, k, freq_line, eta, chi);
    r.inverse_chi = 1.0 / chi;
    r.frq = m.nu[(size_t)p * m.F + f] * sh;
    r.phi = thermo_profile(m, invr_mass, p, freq_line, r.frq);
    return r;
}

// The band entries next to the origin from the two sweeps' last rows, in the
// reference's banded form (solver.tpp:2319-2355) with elements indexed by i = n - centre:
//   FF(i), i >= 0: the forward recurrence continued over the forward half's pairs
//                  (FF(0) the boundary row when the origin is the first element);
//   GG(i), i <= 0: the backward recurrence continued over the backward half's pairs
//                  (GG(0) the boundary row when the origin is the last element);
//   L_diag(i) = iC(i) / (FF(i) + GP(i + 1)), with the boundary rows' own forms at the
//                  ray's two ends;
//   L_lower(m) = L_diag(-m-1) GI(-m) ... GI(0),  L_upper(m) = L_diag(m+1) FI(m) ... FI(0),
// then the update_Lambda term of each (solver.tpp:1800-1846).
template <int NB>
MGR_HD void band_tail(const DevModel& m, const double* sl, const LaneCtx& c, const BandRing<NB>& tp,
                      const BandRing<NB>& bt, BandOut<NB>& out) {
    constexpr int O = NB + 1;  // index offset of element i in the local arrays
    const int K = (int)out.K;
    const int Rt = tp.rows, Rb = bt.rows;  // rows of each sweep: centre - first, last - centre
    double dtv[2 * NB + 3], FF[2 * NB + 3], GG[2 * NB + 3], LD[2 * NB + 3];
    uint32_t nrv[2 * NB + 3];
    double shv[2 * NB + 3];
    for (int j = 1; j <= NB + 1 && j <= Rt; j++) {  // backward half: element -j, pair (-j, -j+1)
        const int r = (Rt - j) % (NB + 1);
        dtv[O - j] = tp.dt[r];
        FF[O - j] = tp.F[r];
        nrv[O - j] = tp.nr[r];
        shv[O - j] = tp.sh[r];
    }
    for (int j = 1; j <= NB + 1 && j <= Rb; j++) {  // forward half: element j, pair (j-1, j)
        const int r = (Rb - j) % (NB + 1);
        dtv[O + j - 1] = bt.dt[r];
        GG[O + j] = bt.F[r];
        nrv[O + j] = bt.nr[r];
        shv[O + j] = bt.sh[r];
    }
    // FF(i), 0 <= i <= K, element i not the last
    for (int i = 0; i <= K && i <= Rb - 1; i++) {
        if (i == 0 && Rt == 0) {
            const double dt = dtv[O];
            const double Bf_min_Cf = 1.0 + 2.0 * (1.0 / dt);
            FF[O] = 0.5 * Bf_min_Cf * dt * dt;
        } else {
            const double dc = dtv[O + i - 1], dn = dtv[O + i];
            const double dtau_avg = 0.5 * (dc + dn);
            const double A = 1.0 / (dtau_avg * dc);
            const double FIp = 1.0 / (1.0 + FF[O + i - 1]);
            FF[O + i] = (A * FF[O + i - 1] * FIp + 1.0) * (dtau_avg * dn);
        }
    }
    // GG(i), -K + 1 <= i <= 0, element i not the first
    for (int i = 0; i >= -K + 1 && i >= -Rt + 1; i--) {
        if (i == 0 && Rb == 0) {
            const double dt = dtv[O - 1];
            const double Bl_min_Al = 1.0 + 2.0 * (1.0 / dt);
            GG[O] = 0.5 * Bl_min_Al * dt * dt;
        } else {
            const double dc = dtv[O + i - 1], dn = dtv[O + i];
            const double dtau_avg = 0.5 * (dc + dn);
            const double C = 1.0 / (dtau_avg * dn);
            const double GP = GG[O + i + 1] * (1.0 / (1.0 + GG[O + i + 1]));
            GG[O + i] = (C * GP + 1.0) * (dtau_avg * dc);
        }
    }
    // L_diag(i), -K <= i <= K on the ray
    for (int i = -K; i <= K; i++) {
        if (i < -Rt || i > Rb || i == 0) continue;
        if (i == Rb) {  // the last element
            const double inverse_dtau_l = 1.0 / dtv[O + i - 1];
            const double Al = 2.0 * inverse_dtau_l * inverse_dtau_l;
            const double Bl_min_Al = 1.0 + 2.0 * inverse_dtau_l;
            const double Bl = Bl_min_Al + Al;
            LD[O + i] = (1.0 + FF[O + i - 1]) / (Bl_min_Al + Bl * FF[O + i - 1]);
        } else if (i == -Rt) {  // the first element
            const double inverse_dtau_f = 1.0 / dtv[O + i];
            const double Cf = 2.0 * inverse_dtau_f * inverse_dtau_f;
            const double Bf_min_Cf = 1.0 + 2.0 * inverse_dtau_f;
            const double Bf = Bf_min_Cf + Cf;
            LD[O + i] = (1.0 + GG[O + i + 1]) / (Bf_min_Cf + Bf * GG[O + i + 1]);
        } else {
            const double dc = dtv[O + i - 1], dn = dtv[O + i];
            const double dtau_avg = 0.5 * (dc + dn);
            const double GP = GG[O + i + 1] * (1.0 / (1.0 + GG[O + i + 1]));
            LD[O + i] = (dtau_avg * dn) / (FF[O + i] + GP);
        }
    }
    const double w2 = 2.0 * out.w_rr;
    for (int mm = 0; mm < K; mm++) {
        // lower: element -(mm + 1), L_diag GI(-mm) ... GI(0) in the reference's order
        out.val[mm] = 0.0;
        out.nr[mm] = c.o;
        if (mm + 1 <= Rt) {
            const int i = -(mm + 1);
            double L = LD[O + i];
            for (int j = i + 1; j <= 0; j++) L *= 1.0 / (1.0 + GG[O + j]);
            const LambdaFactors f = lambda_factors_at(m, sl, nrv[O + i], c.f, shv[O + i]);
            out.val[mm] = f.Aqw * w2 * f.frq * f.phi * L * f.inverse_chi;
            out.nr[mm] = nrv[O + i];
        }
        // upper: element mm + 1, L_diag FI(mm) ... FI(0)
        out.val[K + mm] = 0.0;
        out.nr[K + mm] = c.o;
        if (mm + 1 <= Rb) {
            const int i = mm + 1;
            double L = LD[O + i];
            for (int j = i - 1; j >= 0; j--) L *= 1.0 / (1.0 + FF[O + j]);
            const LambdaFactors f = lambda_factors_at(m, sl, nrv[O + i], c.f, shv[O + i]);
            out.val[K + mm] = f.Aqw * w2 * f.frq * f.phi * L * f.inverse_chi;
            out.nr[K + mm] = nrv[O + i];
        }
    }
}

// Short characteristics: one direction's element (solver.tpp:1624-1638),
// constante * freq * phi * (factor + 1) * inverse_chi with constante = line_A * weight * w_rr.
MGR_HD double lambda_element_sc0(const LambdaFactors& k, double w_rr, double X) {
    const double constante = k.Aqw * w_rr;
    return constante * k.frq * k.phi * X * k.inverse_chi;
}

}  // namespace mgr
