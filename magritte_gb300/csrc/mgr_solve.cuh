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
#include "mgr_device.cuh"

namespace mgr {

constexpr unsigned FULL_MASK = 0xffffffffu;

// One base step of a traced half ray, staged in shared memory by the warp.
struct HalfSmem {
    uint32_t* ids;   // next point of step s
    double* shift;   // Doppler shift of ids[s]
    double* dZ;      // distance increment of step s
    float* dsh;      // (float)(shift - 1)
    uint32_t* eid;   // CSR edge of step s (index into the interpolation-count table)
};

// Warp-cooperative Geometry::get_next_general_geometry<Defaulttracer> walk
// (geometry.tpp:13-44) from origin o along ray r until a boundary point is met.
// Lanes scan the neighbour list; the argmin of (distance to ray, neighbour order)
// reproduces the reference's strict-< scan.  Returns the number of steps, or -1 on
// capacity overflow / invalid geometry (status bits set).
template <bool STORE>
__device__ int trace_half(const DevModel& m, uint32_t o, uint32_t r, uint32_t cap, HalfSmem h, int lane,
                          int* status) {
    const double* d = m.raydir + 3 * r;
    const double dx = d[0], dy = d[1], dz = d[2];
    const double4_32a po = m.pos[o];
    double Z = 0.0;
    uint32_t crt = o;
    int count = 0;
    while (true) {
        const uint32_t nnb = m.n_nb[crt];
        const uint32_t cum = m.cum_nb[crt];
        double best = DBL_MAX;
        uint32_t besti = 0xffffffffu;
        double bestZ = 0.0;
        for (uint32_t i = lane; i < nnb; i += 32) {
            const double4_32a e = m.edge[cum + i];
            const double Rx = dsub_rn(e.x, po.x);
            const double Ry = dsub_rn(e.y, po.y);
            const double Rz = dsub_rn(e.z, po.z);
            const double Zn = dot3_rn(Rx, Ry, Rz, dx, dy, dz);
            if (Zn > Z) {
                const double d2 = dsub_rn(dot3_rn(Rx, Ry, Rz, Rx, Ry, Rz), dmul_rn(Zn, Zn));
                if (d2 < best) {
                    best = d2;
                    besti = i;
                    bestZ = Zn;
                }
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const double ob = __shfl_xor_sync(FULL_MASK, best, off);
            const uint32_t oi = __shfl_xor_sync(FULL_MASK, besti, off);
            const double oz = __shfl_xor_sync(FULL_MASK, bestZ, off);
            if (ob < best || (ob == best && oi < besti)) {
                best = ob;
                besti = oi;
                bestZ = oz;
            }
        }
        if (besti == 0xffffffffu) {
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
        const uint32_t nxt = (uint32_t)__double_as_longlong(m.edge[cum + besti].w);
        const double dZl = dsub_rn(bestZ, Z);
        Z = dadd_rn(Z, dZl);
        if (STORE && lane == 0) {
            h.ids[count] = nxt;
            h.eid[count] = cum + besti;
            h.dZ[count] = dZl;
            const double s = shift_comoving(m, o, nxt, d);
            h.shift[count] = s;
            h.dsh[count] = (float)dsub_rn(s, 1.0);
        }
        count++;
        if (m.p2b[nxt] != m.P) break;
        crt = nxt;
    }
    __syncwarp();
    return count;
}

// An element of the ray pair as the reference's per-thread buffers hold it
// (nr, nr_interp, interp_factor, shift) plus its distance to the neighbouring
// element on the origin side.
struct Elem {
    uint32_t nr, ni;
    double fac;
    double shift;
    double dzin;
    float dsh;  // shift - 1 (FP32), split precision only
};

// Walks the elements of one half ray from its outer end toward the origin,
// expanding the interpolation points Solver::set_data_for_line inserts
// (solver.tpp:1057-1097).  Elements of one step are visited i = n .. 1.
struct ElemIter {
    int s;          // current base step
    uint32_t i;     // current sub-element (n .. 1), 0 = step exhausted
    uint32_t n;     // interpolation count of step s
    uint32_t crt, nxt;
    double shc, shn, dzs;
    float dshc, dshn;
};

MGR_HD void iter_load_step(const DevModel& m, const HalfSmem& h, uint32_t o, uint32_t l,
                                               ElemIter& it) {
    const int s = it.s;
    it.crt = s ? h.ids[s - 1] : o;
    it.nxt = h.ids[s];
    it.shc = s ? h.shift[s - 1] : 1.0;
    it.shn = h.shift[s];
    it.dshc = s ? h.dsh[s - 1] : 0.0f;
    it.dshn = h.dsh[s];
    it.dzs = h.dZ[s];
    it.n = m.nint[(size_t)h.eid[s] * m.L + l];
    it.i = it.n;
}

// Produces the next element (outer to inner).  Returns false when only the
// centre element remains.
MGR_HD bool iter_next(const DevModel& m, const HalfSmem& h, uint32_t o, uint32_t l, ElemIter& it,
                                          Elem& e) {
    if (it.i == 0) {
        if (it.s == 0) return false;
        it.s--;
        iter_load_step(m, h, o, l, it);
    }
    const uint32_t n = it.n;
    const uint32_t i = it.i;
    e.nr = it.nxt;
    e.ni = it.crt;
    if (n > 1) {
        const double dshift = dsub_rn(it.shn, it.shc);
        const double dshift_interpl = dshift / (double)n;
        e.shift = dadd_rn(it.shc, dmul_rn((double)i, dshift_interpl));
        e.fac = 1.0 - ((double)i) / (double)n;
        e.dzin = it.dzs / (double)n;
        e.dsh = it.dshc + (float)i * ((it.dshn - it.dshc) / (float)n);
    } else {
        e.shift = it.shn;
        e.fac = 0.0;
        e.dzin = it.dzs;
        e.dsh = it.dshn;
    }
    it.i--;
    return true;
}

MGR_HD void iter_begin(const DevModel& m, const HalfSmem& h, uint32_t o, uint32_t l, int nsteps,
                                           ElemIter& it) {
    if (nsteps <= 0) {
        it.s = 0;
        it.i = 0;
        return;
    }
    it.s = nsteps - 1;
    iter_load_step(m, h, o, l, it);
}

MGR_HD Elem centre_elem(uint32_t o) {
    Elem e;
    e.nr = o;
    e.ni = o;  // never read: its interpolation factor is 0
    e.fac = 0.0;
    e.shift = 1.0;
    e.dzin = 0.0;
    e.dsh = 0.0f;
    return e;
}

// ---------------------------------------------------------------------------------
// Pair physics.  Lane context: origin o, frequency f, its line l0, nu(o, f).
// ---------------------------------------------------------------------------------
struct LaneCtx {
    uint32_t o, f, l0;
    double freq;   // nu(o, f)
    float fq;      // (float)freq
    float a0;      // (float)(freq - line[l0])
};

struct PairOut {
    double dtau;   // optical depth increment between the two elements
    double Slo;    // row source of the lower-index element if the pair is line-integrated
    double Shi;    // source of the higher-index element if line-integrated
    bool large;
};

// FP64 (reference arithmetic) -------------------------------------------------------

// get_eta_and_chi_interpolated<approx> (solver.tpp:1176-1194, :1252-1283, :1306-1320).
MGR_HD void eta_chi_fp64(const DevModel& m, const double* sl, const LaneCtx& c, const Elem& e,
                                             double& eta, double& chi) {
    const double freq = c.freq * e.shift;
    const size_t b1 = (size_t)e.nr * m.L, b2 = (size_t)e.ni * m.L;
    if (m.approx == APPROX_ONELINE) {
        const uint32_t l = c.l0;
        const double iw = interpolate_linear(m.iw[b1 + l], m.iw[b2 + l], e.fac);
        const double prof = gaussian(iw, freq - m.line[l]);
        eta = prof * interpolate_log(m.em[b1 + l], m.em[b2 + l], e.fac);
        chi = prof * interpolate_log(m.op[b1 + l], m.op[b2 + l], e.fac) + m.min_opacity;
        return;
    }
    eta = 0.0;
    chi = m.min_opacity;
    uint32_t lo = 0, hi = m.L;
    if (m.approx == APPROX_CLOSELINES) {
        const double ub = m.max_dist * (freq * m.ub[e.nr]);
        lo = lower_bound(sl, m.L, freq - ub);
        hi = upper_bound(sl, m.L, freq + ub);
    }
    for (uint32_t s = lo; s < hi; s++) {
        uint32_t l;
        double diff;
        if (m.approx == APPROX_CLOSELINES) {
            l = m.sorted_map[s];
            diff = freq - sl[s];
        } else {
            l = s;
            diff = freq - m.line[l];
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
        const double prof = gaussian(avg_iw, cf - m.line[l]);
        return dz * (prof * ((cop + nop) / 2.0) + m.min_opacity);
    }
    const double next_pos = (linefreq - nf) * avg_iw;
    const double curr_pos = (linefreq - cf) * avg_iw;
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
MGR_HD void pair_li_fp64(const DevModel& m, const double* sl, const LaneCtx& c, const Elem& lo,
                                             const Elem& hi, double dz, PairOut& out) {
    const double cf = c.freq * lo.shift;
    const double nf = c.freq * hi.shift;
    const size_t c1 = (size_t)lo.nr * m.L, c2 = (size_t)lo.ni * m.L;
    const size_t n1 = (size_t)hi.nr * m.L, n2 = (size_t)hi.ni * m.L;
    if (m.approx == APPROX_ONELINE) {
        const uint32_t l = c.l0;
        out.dtau = dtau_single_line_fp64(m, lo, hi, l, cf, nf, dz);
        out.Slo = interpolate_log(m.Sp[c1 + l], m.Sp[c2 + l], lo.fac);
        out.Shi = interpolate_log(m.Sp[n1 + l], m.Sp[n2 + l], hi.fac);
        return;
    }
    double sum_dtau = 0.0, sum_c = 0.0, sum_n = 0.0;
    uint32_t a = 0, b = m.L;
    if (m.approx == APPROX_CLOSELINES) {
        double left_freq, right_freq;
        if (cf < nf) { left_freq = cf; right_freq = nf; }
        else { right_freq = cf; left_freq = nf; }
        const double cb = m.max_dist * (right_freq * m.ub[lo.nr]);
        const double nb = m.max_dist * (right_freq * m.ub[hi.nr]);
        const double ubw = cb > nb ? cb : nb;
        a = lower_bound(sl, m.L, left_freq - ubw);
        b = upper_bound(sl, m.L, right_freq + ubw);
    }
    for (uint32_t s = a; s < b; s++) {
        const uint32_t l = (m.approx == APPROX_CLOSELINES) ? m.sorted_map[s] : s;
        const double ld = dtau_single_line_fp64(m, lo, hi, l, cf, nf, dz);
        const double lsc = interpolate_log(m.Sp[c1 + l], m.Sp[c2 + l], lo.fac);
        const double lsn = interpolate_log(m.Sp[n1 + l], m.Sp[n2 + l], hi.fac);
        sum_dtau += ld;
        sum_c += ld * lsc;
        sum_n += ld * lsn;
    }
    if (m.approx == APPROX_NONE) {
        out.dtau = sum_dtau;
        out.Slo = sum_c / sum_dtau;
        out.Shi = sum_n / sum_dtau;
        return;
    }
    double d = sum_dtau;
    const double bound_min_dtau = m.min_opacity * dz;
    if (-bound_min_dtau < d) d = (bound_min_dtau > d) ? bound_min_dtau : d;
    out.dtau = d;
    out.Slo = sum_c / d;
    out.Shi = sum_n / d;
}

// FP32 (split precision) ------------------------------------------------------------
// Frequencies are handled as FP32 offsets from the lane's own line centre:
//   nu(o,f) * shift - line[l] = (nu(o,f) - line[l0]) + nu(o,f) (shift - 1) - (line[l] - line[l0]).

MGR_HD float offset_f32(const DevModel& m, const LaneCtx& c, float dsh, uint32_t l) {
    const float off0 = fmaf(c.fq, dsh, c.a0);
    return (l == c.l0) ? off0 : off0 - (float)(m.line[l] - m.line[c.l0]);
}

MGR_HD void eta_chi_f32(const DevModel& m, const double* sl, const LaneCtx& c, const Elem& e,
                                            float& eta, float& chi) {
    const size_t b1 = (size_t)e.nr * m.L, b2 = (size_t)e.ni * m.L;
    const float fac = (float)e.fac;
    const float min_op = m.min_op_s;
    if (m.approx == APPROX_ONELINE) {
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
    if (m.approx == APPROX_CLOSELINES) {
        // lines with line[l] - line[l0] inside [off0 - ub, off0 + ub] (solver.tpp:1216-1227)
        const float off0 = fmaf(c.fq, e.dsh, c.a0);
        const float ub = (float)m.max_dist * ((c.fq + c.fq * e.dsh) * (float)m.ub[e.nr]);
        const double base = m.line[c.l0];
        lo = m.L;
        hi = 0;
        for (uint32_t s = 0; s < m.L; s++) {
            const float dl = (float)(sl[s] - base);
            if (dl >= off0 - ub && dl <= off0 + ub) {
                if (s < lo) lo = s;
                hi = s + 1;
            }
        }
        if (hi < lo) hi = lo;
    }
    for (uint32_t s = lo; s < hi; s++) {
        const uint32_t l = (m.approx == APPROX_CLOSELINES) ? m.sorted_map[s] : s;
        const float iw = interpolate_linear(m.iw_f[b1 + l], m.iw_f[b2 + l], fac);
        const float prof = gaussian(iw, offset_f32(m, c, e.dsh, l));
        eta += prof * interpolate_log(m.em_f[b1 + l], m.em_f[b2 + l], fac);
        chi += prof * interpolate_log(m.op_f[b1 + l], m.op_f[b2 + l], fac);
    }
}

MGR_HD float dtau_single_line_f32(const DevModel& m, const LaneCtx& c, const Elem& lo,
                                                      const Elem& hi, uint32_t l, float dz, double dzd) {
    const size_t c1 = (size_t)lo.nr * m.L, c2 = (size_t)lo.ni * m.L;
    const size_t n1 = (size_t)hi.nr * m.L, n2 = (size_t)hi.ni * m.L;
    const float fc = (float)lo.fac, fn = (float)hi.fac;
    const float iwc = interpolate_linear(m.iw_f[c1 + l], m.iw_f[c2 + l], fc);
    const float iwn = interpolate_linear(m.iw_f[n1 + l], m.iw_f[n2 + l], fn);
    const float avg_iw = (iwc + iwn) * 0.5f;
    const float cop = interpolate_log(m.op_f[c1 + l], m.op_f[c2 + l], fc);
    const float nop = interpolate_log(m.op_f[n1 + l], m.op_f[n2 + l], fn);
    const float offc = offset_f32(m, c, lo.dsh, l);
    const float offn = offset_f32(m, c, hi.dsh, l);
    const float min_op = m.min_op_s;
    if (offc == offn) {
        const float prof = gaussian(avg_iw, offc);
        return dz * (prof * ((cop + nop) * 0.5f) + min_op);
    }
    const float next_pos = -offn * avg_iw;
    const float curr_pos = -offc * avg_iw;
    // Both positions in the same far wing: the reference's erff(next) - erff(curr)
    // cancels, and its single-ulp roundings decide the result.  Take the FP64-mode
    // value there (same arguments, correctly rounded erff), so split precision stays
    // within 1e-5 of the FP64 path in J.
    if ((next_pos > 0.0f) == (curr_pos > 0.0f) && fminf(fabsf(next_pos), fabsf(curr_pos)) > 1.5f &&
        fminf(fabsf(next_pos), fabsf(curr_pos)) < 3.919206f) {
        return (float)dtau_single_line_fp64(m, lo, hi, l, c.freq * lo.shift, c.freq * hi.shift, dzd);
    }
    const float diff_pos = next_pos - curr_pos;
    const float average_opacity = (nop + cop) * 0.5f;
    // Far from the line both positions can round to the same FP32 value (diff_pos = 0)
    // where the FP64 positions still differ; both erf values saturate there and the
    // reference's term is 0.
    const float erfdiff = erff(next_pos) - erff(curr_pos);
    const float erfterm = (erfdiff == 0.0f) ? 0.0f : average_opacity / diff_pos * 0.5f * erfdiff;
    return dz * (avg_iw * erfterm + min_op);
}

MGR_HD void pair_li_f32(const DevModel& m, const double* sl, const LaneCtx& c, const Elem& lo,
                                            const Elem& hi, double dzd, float& dtau, float& Slo, float& Shi) {
    const size_t c1 = (size_t)lo.nr * m.L, c2 = (size_t)lo.ni * m.L;
    const size_t n1 = (size_t)hi.nr * m.L, n2 = (size_t)hi.ni * m.L;
    const float fc = (float)lo.fac, fn = (float)hi.fac;
    const float dz = (float)dzd * m.dz_scale;
    if (m.approx == APPROX_ONELINE) {
        const uint32_t l = c.l0;
        dtau = dtau_single_line_f32(m, c, lo, hi, l, dz, dzd);
        Slo = interpolate_log(m.Sp_f[c1 + l], m.Sp_f[c2 + l], fc) * m.s_scale;
        Shi = interpolate_log(m.Sp_f[n1 + l], m.Sp_f[n2 + l], fn) * m.s_scale;
        return;
    }
    float sum_dtau = 0.0f, sum_c = 0.0f, sum_n = 0.0f;
    uint32_t a = 0, b = m.L;
    if (m.approx == APPROX_CLOSELINES) {
        const float oc = fmaf(c.fq, lo.dsh, c.a0);
        const float on = fmaf(c.fq, hi.dsh, c.a0);
        const float left = fminf(oc, on), right = fmaxf(oc, on);
        const float rf = c.fq + fmaxf(c.fq * lo.dsh, c.fq * hi.dsh);
        const float cb = (float)m.max_dist * (rf * (float)m.ub[lo.nr]);
        const float nb = (float)m.max_dist * (rf * (float)m.ub[hi.nr]);
        const float ubw = fmaxf(cb, nb);
        const double base = m.line[c.l0];
        a = m.L;
        b = 0;
        for (uint32_t s = 0; s < m.L; s++) {
            const float dl = (float)(sl[s] - base);
            if (dl >= left - ubw && dl <= right + ubw) {
                if (s < a) a = s;
                b = s + 1;
            }
        }
        if (b < a) b = a;
    }
    for (uint32_t s = a; s < b; s++) {
        const uint32_t l = (m.approx == APPROX_CLOSELINES) ? m.sorted_map[s] : s;
        const float ld = dtau_single_line_f32(m, c, lo, hi, l, dz, dzd);
        const float lsc = interpolate_log(m.Sp_f[c1 + l], m.Sp_f[c2 + l], fc);
        const float lsn = interpolate_log(m.Sp_f[n1 + l], m.Sp_f[n2 + l], fn);
        sum_dtau += ld;
        sum_c += ld * lsc;
        sum_n += ld * lsn;
    }
    if (m.approx == APPROX_NONE) {
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

// Source/opacity cache of one element (trapezoid branch quantities).
struct EC {
    double S, chi;
    bool ok;
};

template <int MODE>
MGR_HD void elem_fresh(const DevModel& m, const double* sl, const LaneCtx& c, const Elem& e, EC& ec) {
    if (ec.ok) return;
    if (MODE == MODE_FP64) {
        double eta, chi;
        eta_chi_fp64(m, sl, c, e, eta, chi);
        ec.S = eta / chi;
        ec.chi = chi;
    } else {
        float eta, chi;
        eta_chi_f32(m, sl, c, e, eta, chi);
        ec.S = (double)(eta / chi) * (double)m.s_scale;
        ec.chi = (double)chi;
    }
    ec.ok = true;
}

// compute_source_dtau (solver.tpp:2139-2186) for the pair (lo, hi) with lo the lower
// array index.  Fills the caches of both elements when the trapezoid rule is used.
template <int MODE>
MGR_HD void eval_pair(const DevModel& m, const double* sl, const LaneCtx& c, const Elem& lo,
                                          const Elem& hi, double dz, EC& ecl, EC& ech, PairOut& out) {
    const double dshift_abs = fabs(dsub_rn(hi.shift, lo.shift));
    const double a = m.dshift_max[lo.nr], b = m.dshift_max[hi.nr];
    out.large = dshift_abs > (a < b ? a : b);
    if (out.large) {
        if (MODE == MODE_FP64) {
            pair_li_fp64(m, sl, c, lo, hi, dz, out);
        } else {
            float d, s1, s2;
            pair_li_f32(m, sl, c, lo, hi, dz, d, s1, s2);
            out.dtau = d;
            out.Slo = s1;
            out.Shi = s2;
        }
    } else {
        elem_fresh<MODE>(m, sl, c, lo, ecl);
        elem_fresh<MODE>(m, sl, c, hi, ech);
        if (MODE == MODE_FP64) {
            out.dtau = 0.5 * (ecl.chi + ech.chi) * dz;
        } else {
            out.dtau = (double)(0.5f * ((float)ecl.chi + (float)ech.chi) * ((float)dz * m.dz_scale));
        }
    }
}

// Reciprocal of an elimination pivot.  FP64 mode: IEEE division, as the reference.
// Split mode: an FP32 reciprocal refined by one Newton step in FP64 (relative error
// ~1e-14), which keeps the elimination in FP64 without the cost of FP64 division.
template <int MODE>
MGR_HD double rcp_pivot(double x) {
    if (MODE == MODE_FP64) return 1.0 / x;
    const float xf = (float)x;
    if (!(xf > 1.0e-30f && xf < 1.0e30f)) return 1.0 / x;
#ifdef __CUDA_ARCH__
    const double r = (double)__frcp_rn(xf);
#else
    const double r = (double)(1.0f / xf);
#endif
    return fma(r, fma(-x, r, 1.0), r);
}

// One interior elimination row in the economical (1+B)/C form (solver.tpp:2266-2281
// forward, :2304-2309 backward): `dt_out` is the optical depth of the pair already
// eliminated, `dt_in` of the pair toward the origin.  F, FI = 1/(1+F) and the modified
// source Su are updated in place.  Split mode computes the coefficients from the FP32
// optical depths in FP32 and keeps the recurrence itself in FP64.
template <int MODE>
MGR_HD void elim_row(double dt_out, double dt_in, double S, double& F, double& FI, double& Su) {
    double A, iC;
    if (MODE == MODE_FP64) {
        const double dtau_avg = 0.5 * (dt_out + dt_in);
        const double iA = dtau_avg * dt_out;
        iC = dtau_avg * dt_in;
        A = 1.0 / iA;
    } else {
        const float a = (float)dt_out, b = (float)dt_in;
        const float dtau_avg = 0.5f * (a + b);
        const float iAf = dtau_avg * a, iCf = dtau_avg * b;
        if (iAf > 1.0e-30f && iAf < 1.0e30f && iCf > 1.0e-30f && iCf < 1.0e30f) {
            A = (double)(1.0f / iAf);
            iC = (double)iCf;
        } else {  // optical depths so small (or large) that their product leaves FP32 range
            const double avg = 0.5 * (dt_out + dt_in);
            A = 1.0 / (avg * dt_out);
            iC = avg * dt_in;
        }
    }
    F = (A * F * FI + 1.0) * iC;
    FI = rcp_pivot<MODE>(1.0 + F);
    Su = (A * Su + S) * FI * iC;
}

// Result of one lane's ray-pair solve.
struct LaneResult {
    double u;       // Su[centre]
    double Ldiag;   // L_diag[centre]
    bool solved;    // n_tot > 1
};

// Two-sided Feautrier solve of frequency c.f on the ray pair staged in `bk`
// (backward half, direction rr) and `fw` (forward half, antipode).
template <int MODE>
__host__ __device__ LaneResult solve_lane(const DevModel& m, const double* sl, const LaneCtx& c, const HalfSmem& bk, int nb,
                                 const HalfSmem& fw, int nf) {
    LaneResult res;
    res.solved = (nb > 0) || (nf > 0);
    if (!res.solved) {
        res.u = boundary_intensity(m, c.o, m.nu[(size_t)c.o * m.F + c.f]);
        res.Ldiag = 0.0;
        return res;
    }
    const Elem cen = centre_elem(c.o);
    const uint32_t l = c.l0;

    // ---- top sweep: elements first .. centre (backward half, outer end first) ----
    double FF = 0.0, FI = 0.0, Su = 0.0, dt_top = 0.0;
    bool top_rows = false;     // at least one row eliminated
    bool top_large = false;    // last pair line-integrated
    double top_Shi = 0.0;      // its upper source
    EC ec_cen{0.0, 0.0, false};
    if (nb > 0) {
        ElemIter it;
        iter_begin(m, bk, c.o, l, nb, it);
        Elem prev;
        iter_next(m, bk, c.o, l, it, prev);
        EC ec_prev{0.0, 0.0, false};
        const double Ibdy = boundary_intensity(m, prev.nr, c.freq * prev.shift);
        bool first = true;
        while (true) {
            Elem cur;
            const bool more = iter_next(m, bk, c.o, l, it, cur);
            if (!more) cur = cen;
            EC ec_cur{0.0, 0.0, false};
            PairOut po;
            eval_pair<MODE>(m, sl, c, prev, cur, prev.dzin, ec_prev, more ? ec_cur : ec_cen, po);
            double S;
            if (po.large) S = po.Slo;
            else { elem_fresh<MODE>(m, sl, c, prev, ec_prev); S = ec_prev.S; }
            if (first) {
                const double inverse_dtau_f = 1.0 / po.dtau;
                const double Cf = 2.0 * inverse_dtau_f * inverse_dtau_f;
                const double Bf_min_Cf = 1.0 + 2.0 * inverse_dtau_f;
                const double Bf = Bf_min_Cf + Cf;
                Su = (S + 2.0 * Ibdy * inverse_dtau_f) / Bf;
                FF = 0.5 * Bf_min_Cf * po.dtau * po.dtau;
                FI = rcp_pivot<MODE>(1.0 + FF);
                first = false;
            } else {
                elim_row<MODE>(dt_top, po.dtau, S, FF, FI, Su);
            }
            top_rows = true;
            dt_top = po.dtau;
            top_large = po.large;
            top_Shi = po.Shi;
            if (!more) break;
            prev = cur;
            ec_prev = ec_cur;
        }
    }

    // ---- bottom sweep: elements last .. centre+1 (forward half, outer end first) ----
    double GG = 0.0, GI = 0.0, Sb = 0.0, dt_bot = 0.0, S_centre = 0.0;
    bool bot_rows = false;
    if (nf > 0) {
        ElemIter it;
        iter_begin(m, fw, c.o, l, nf, it);
        Elem prev;  // higher index element
        iter_next(m, fw, c.o, l, it, prev);
        EC ec_prev{0.0, 0.0, false};
        const double Ibdy = boundary_intensity(m, prev.nr, c.freq * prev.shift);
        bool first = true;
        double S_prev_row = 0.0;  // row source of `prev` (known once its upper pair was evaluated)
        while (true) {
            Elem cur;  // lower index element
            const bool more = iter_next(m, fw, c.o, l, it, cur);
            if (!more) cur = cen;
            EC ec_cur{0.0, 0.0, false};
            EC& ecc = more ? ec_cur : ec_cen;
            PairOut po;
            eval_pair<MODE>(m, sl, c, cur, prev, prev.dzin, ecc, ec_prev, po);
            // Row source of the lower element `cur` (index < last).
            double S_cur;
            if (po.large) S_cur = po.Slo;
            else { elem_fresh<MODE>(m, sl, c, cur, ecc); S_cur = ecc.S; }
            if (first) {
                double S_last;
                if (po.large) S_last = po.Shi;
                else { elem_fresh<MODE>(m, sl, c, prev, ec_prev); S_last = ec_prev.S; }
                const double inverse_dtau_l = 1.0 / po.dtau;
                const double Al = 2.0 * inverse_dtau_l * inverse_dtau_l;
                const double Bl_min_Al = 1.0 + 2.0 * inverse_dtau_l;
                const double Bl = Bl_min_Al + Al;
                Sb = (S_last + 2.0 * Ibdy * inverse_dtau_l) / Bl;
                GG = 0.5 * Bl_min_Al * po.dtau * po.dtau;
                GI = rcp_pivot<MODE>(1.0 + GG);
                first = false;
            } else {
                // row `prev`: upper pair dt_bot already eliminated, lower pair = this pair
                elim_row<MODE>(dt_bot, po.dtau, S_prev_row, GG, GI, Sb);
            }
            bot_rows = true;
            dt_bot = po.dtau;
            S_prev_row = S_cur;
            if (!more) {
                S_centre = S_cur;
                break;
            }
            prev = cur;
            ec_prev = ec_cur;
        }
    }

    // ---- combine at the origin ----
    if (top_rows && bot_rows) {
        const double dtau_avg = 0.5 * (dt_top + dt_bot);
        const double iA = dtau_avg * dt_top;
        const double iC = dtau_avg * dt_bot;
        const double A = 1.0 / iA;
        const double FFc = (A * FF * FI + 1.0) * iC;
        const double Su_pre = (A * Su + S_centre) * iC;
        const double GP = GG * GI;
        const double D = 1.0 / (FFc + GP);
        res.u = (Su_pre + Sb) * D;
        res.Ldiag = iC * D;
    } else if (bot_rows) {  // origin is the first element
        const double Ibdy = boundary_intensity(m, c.o, c.freq);
        const double inverse_dtau_f = 1.0 / dt_bot;
        const double Cf = 2.0 * inverse_dtau_f * inverse_dtau_f;
        const double Bf_min_Cf = 1.0 + 2.0 * inverse_dtau_f;
        const double Bf = Bf_min_Cf + Cf;
        const double Suf = (S_centre + 2.0 * Ibdy * inverse_dtau_f) / Bf;
        const double FFf = 0.5 * Bf_min_Cf * dt_bot * dt_bot;
        const double GP = GG * GI;
        const double D = 1.0 / (FFf + GP);
        res.u = (Suf * (1.0 + FFf) + Sb) * D;
        res.Ldiag = (1.0 / Cf) * D;
    } else {  // origin is the last element
        const double Ibdy = boundary_intensity(m, c.o, c.freq);
        double S_last;
        if (top_large) S_last = top_Shi;
        else { elem_fresh<MODE>(m, sl, c, cen, ec_cen); S_last = ec_cen.S; }
        const double inverse_dtau_l = 1.0 / dt_top;
        const double Al = 2.0 * inverse_dtau_l * inverse_dtau_l;
        const double Bl_min_Al = 1.0 + 2.0 * inverse_dtau_l;
        const double Bl = Bl_min_Al + Al;
        const double denominator = 1.0 / (Bl * FF + Bl_min_Al);
        const double Sl = S_last + 2.0 * Ibdy * inverse_dtau_l;
        res.u = (Al * Su + Sl) * (1.0 + FF) * denominator;
        res.Ldiag = (1.0 + FF) / (Bl_min_Al + Bl * FF);
    }
    return res;
}

// update_Lambda, n_off_diag = 0 (solver.tpp:1760-1800): the ALO element of this
// (origin, ray pair, frequency).
MGR_HD double lambda_element(const DevModel& m, const double* sl, uint32_t o, uint32_t rr,
                                                 uint32_t f, double Ldiag) {
    const double w_ang = 2.0 * m.rayw[rr];
    const uint32_t ls = m.corr_lspec[f];
    const uint32_t k = m.corr_k[f];
    const uint32_t z = m.corr_z[f];
    const uint32_t lid = m.nrad_cum[ls] + k;
    const double freq_line = m.line[lid];
    const double invr_mass = m.lspec_inv_mass[ls];
    const double constante = m.line_A[lid] * m.quad_w[(size_t)ls * m.Q + z] * w_ang;
    double eta, chi;
    get_eta_and_chi(m, sl, o, k, freq_line, eta, chi);  // the reference passes k as the line index here
    const double inverse_chi = 1.0 / chi;
    const double frq = m.nu[(size_t)o * m.F + f] * 1.0;
    const double phi = thermo_profile(m, invr_mass, o, freq_line, frq);
    return constante * frq * phi * Ldiag * inverse_chi;
}

}  // namespace mgr
