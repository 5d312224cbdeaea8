// Differentiable new imager: a smooth FP64 forward of the one-sided Feautrier image
// solve (Solver::image_feautrier_order_2_new_imager, solver.tpp:576-627, with the
// per-pixel solve of solver.tpp:2462-2574) and its hand-written adjoint.
//
// The forward follows image_lane's FP64 arithmetic with the reference's single-
// precision library calls replaced by their FP64 counterparts (exp in the Gaussian
// profile, pow in the logarithmic interpolation, erf in the line-integrated optical
// depth - as a difference of erfc where both arguments have the same sign, free of
// cancellation - and expm1 in the Planck function), so that the image is a smooth function of
// the per-point line data and velocities.  The ray trace, the interpolation points,
// the CloseLines brackets, the large-shift branch and the dtau clamp are held fixed
// (trace-fixed differentiation): they are piecewise constant in the inputs.
//
// Differentiated inputs, per point p and line l: emissivity em, opacity op, inverse
// width iw, source Sp = em / op (the library's own quotient, an input of its own
// here), and per point the rest-frame shift 1 + v . d, which the kernel turns into
// d(loss)/dv.  The adjoint recomputes each ray's elimination factors in a forward
// sweep (kept per lane in a scratch array), then walks the ray back from the
// observer: the reverse elimination gives d(loss)/d(dtau_k) and d(loss)/d(S_k) per
// pair, the pair and element adjoints give the per-point derivatives.
#pragma once
#include "mgr_solve.cuh"

namespace mgr {

// ---- smooth FP64 counterparts of the reference's profile, interpolation, Planck ----
MGR_HD double gauss_s(double iw, double diff) {
    const double x = iw * diff;
    return iw * INVERSE_SQRT_PI * exp(-x * x);
}

// a^(1-f) b^f as a (b / a)^f (interpolate_log)
MGR_HD double ilog_s(double a, double b, double f) {
    if (f == 0.0) return a;
    if (f == 1.0) return b;
    return a * pow(b / a, f);
}

// erf(a) - erf(b) without cancellation when a and b lie on the same side of 0
// (differences of erfc there, which keeps its relative precision in the wings).
MGR_HD double erf_diff_s(double a, double b) {
    if (a > 0.0 && b > 0.0) return erfc(b) - erfc(a);
    if (a < 0.0 && b < 0.0) return erfc(-a) - erfc(-b);
    return erf(a) - erf(b);
}

// Boundary intensity at `freq` (boundary_intensity) and its derivative in freq.
MGR_HD double bdy_s(const DevModel& m, uint32_t p, double freq, double& dfreq) {
    dfreq = 0.0;
    const uint32_t b = m.p2b[p];
    if (b >= m.B) return 0.0;
    const int c = m.bc[b];
    if (c == BC_ZERO) return 0.0;
    const double temp = (c == BC_THERMAL) ? m.bt[b] : T_CMB;
    const double a = HH_OVER_KB / temp;
    const double em1 = expm1(a * freq);
    const double B = TWO_HH_OVER_CC_SQUARED * (freq * freq * freq) / em1;
    dfreq = B * (3.0 / freq - a * (em1 + 1.0) / em1);
    return B;
}

// Gradient targets of one image (device pointers; [P][L] and [P][3]).
struct AdjGrads {
    double* em;
    double* op;
    double* iw;
    double* Sp;
    double* vel;
    double d[3];  // ray direction: d(shift)/dv
};

enum AdjKind : int { ADJ_EM = 0, ADJ_OP = 1, ADJ_IW = 2, ADJ_SP = 3 };

// Warp-uniform index range [lo, hi) over the lanes (the union of the lanes' brackets).
MGR_HD void warp_range(uint32_t& lo, uint32_t& hi) {
#ifdef __CUDA_ARCH__
    for (int off = 16; off > 0; off >>= 1) {
        lo = min(lo, __shfl_xor_sync(FULL_MASK, lo, off));
        hi = max(hi, __shfl_xor_sync(FULL_MASK, hi, off));
    }
#else
    (void)lo;
    (void)hi;
#endif
}

// Adds a lane's contribution to a gradient entry; on the device the warp's 32
// contributions are summed first (every lane must call with the same target).
struct AdjAcc {
    AdjGrads g;
    uint32_t L;
    MGR_HD void add(int kind, uint32_t p, uint32_t l, double v) const {
        double* base = kind == ADJ_EM ? g.em : kind == ADJ_OP ? g.op : kind == ADJ_IW ? g.iw : g.Sp;
#ifdef __CUDA_ARCH__
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(FULL_MASK, v, off);
        if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(base + (size_t)p * L + l, v);
#else
        base[(size_t)p * L + l] += v;
#endif
    }
    MGR_HD void add_shift(uint32_t p, double v) const {
#ifdef __CUDA_ARCH__
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(FULL_MASK, v, off);
        if ((threadIdx.x & 31) == 0 && v != 0.0)
            for (int k = 0; k < 3; k++) atomicAdd(g.vel + 3 * (size_t)p + k, v * g.d[k]);
#else
        for (int k = 0; k < 3; k++) g.vel[3 * (size_t)p + k] += v * g.d[k];
#endif
    }
};

// Lines that contribute at frequency `freq` of an element (eta_chi_fp64's range).
template <int AP>
MGR_HD void elem_bracket(const DevModel& m, const double* sl, double freq, uint32_t nr, uint32_t& lo, uint32_t& hi) {
    lo = 0;
    hi = m.L;
    if (AP == APPROX_CLOSELINES) {
        const double ub = dmul_rn(m.max_dist, dmul_rn(freq, m.ub[nr]));
        lo = lower_bound(sl, m.L, dsub_rn(freq, ub));
        hi = upper_bound(sl, m.L, dadd_rn(freq, ub));
    }
}

template <int AP>
MGR_HD uint32_t line_of(const DevModel& m, uint32_t s) {
    return (AP == APPROX_CLOSELINES) ? m.sorted_map[s] : s;
}

// Element emissivity and opacity (eta_chi_fp64, smooth).
template <int AP>
MGR_HD void elem_s(const DevModel& m, const double* sl, double nu, const Elem& e, double& eta, double& chi) {
    const double freq = nu * e.shift;
    uint32_t lo, hi;
    elem_bracket<AP>(m, sl, freq, e.nr, lo, hi);
    const size_t b1 = (size_t)e.nr * m.L, b2 = (size_t)e.ni * m.L;
    eta = 0.0;
    chi = m.min_opacity;
    for (uint32_t s = lo; s < hi; s++) {
        const uint32_t l = line_of<AP>(m, s);
        const double diff = freq - m.line[l];
        const double iw = interpolate_linear(m.iw[b1 + l], m.iw[b2 + l], e.fac);
        const double prof = gauss_s(iw, diff);
        eta += prof * ilog_s(m.em[b1 + l], m.em[b2 + l], e.fac);
        chi += prof * ilog_s(m.op[b1 + l], m.op[b2 + l], e.fac);
    }
}

// Adjoint of elem_s: d(loss)/d(eta), d(loss)/d(chi) of the element -> per-point
// line data and the element's shift (returned in g_shift, to be split over its two
// points by the caller).
template <int AP>
MGR_HD void elem_s_adj(const DevModel& m, const double* sl, double nu, const Elem& e, double g_eta, double g_chi,
                       const AdjAcc& acc, double& g_shift) {
    const double freq = nu * e.shift;
    uint32_t lo, hi;
    elem_bracket<AP>(m, sl, freq, e.nr, lo, hi);
    uint32_t wlo = lo, whi = hi;
    warp_range(wlo, whi);
    const size_t b1 = (size_t)e.nr * m.L, b2 = (size_t)e.ni * m.L;
    const double f = e.fac;
    for (uint32_t s = wlo; s < whi; s++) {
        const uint32_t l = line_of<AP>(m, s);
        double gem_nr = 0.0, gem_ni = 0.0, gop_nr = 0.0, gop_ni = 0.0, giw_nr = 0.0, giw_ni = 0.0;
        if (s >= lo && s < hi) {
            const double diff = freq - m.line[l];
            const double iw = interpolate_linear(m.iw[b1 + l], m.iw[b2 + l], f);
            const double prof = gauss_s(iw, diff);
            const double x = iw * diff;
            const double emE = ilog_s(m.em[b1 + l], m.em[b2 + l], f);
            const double opE = ilog_s(m.op[b1 + l], m.op[b2 + l], f);
            const double gprof = g_eta * emE + g_chi * opE;
            const double g_emE = g_eta * prof, g_opE = g_chi * prof;
            const double g_iwE = gprof * prof * (1.0 / iw - 2.0 * x * diff);
            g_shift += gprof * prof * (-2.0 * x * iw) * nu;
            gem_nr = g_emE * (1.0 - f) * emE / m.em[b1 + l];
            gop_nr = g_opE * (1.0 - f) * opE / m.op[b1 + l];
            giw_nr = g_iwE * (1.0 - f);
            if (f != 0.0) {
                gem_ni = g_emE * f * emE / m.em[b2 + l];
                gop_ni = g_opE * f * opE / m.op[b2 + l];
                giw_ni = g_iwE * f;
            }
        }
        acc.add(ADJ_EM, e.nr, l, gem_nr);
        acc.add(ADJ_OP, e.nr, l, gop_nr);
        acc.add(ADJ_IW, e.nr, l, giw_nr);
        if (f != 0.0) {
            acc.add(ADJ_EM, e.ni, l, gem_ni);
            acc.add(ADJ_OP, e.ni, l, gop_ni);
            acc.add(ADJ_IW, e.ni, l, giw_ni);
        }
    }
}

// Lines of a large-shift pair (pair_li_fp64's range).
template <int AP>
MGR_HD void pair_bracket(const DevModel& m, const double* sl, double cf, double nf, uint32_t lo_nr, uint32_t hi_nr,
                         uint32_t& a, uint32_t& b) {
    a = 0;
    b = m.L;
    if (AP == APPROX_CLOSELINES) {
        const double left = cf < nf ? cf : nf, right = cf < nf ? nf : cf;
        const double cb = dmul_rn(m.max_dist, dmul_rn(right, m.ub[lo_nr]));
        const double nb = dmul_rn(m.max_dist, dmul_rn(right, m.ub[hi_nr]));
        const double ubw = cb > nb ? cb : nb;
        a = lower_bound(sl, m.L, dsub_rn(left, ubw));
        b = upper_bound(sl, m.L, dadd_rn(right, ubw));
    }
}

// One line's optical depth over a large-shift pair (dtau_single_line_fp64, smooth).
MGR_HD double ld_s(const DevModel& m, const Elem& lo, const Elem& hi, uint32_t l, double cf, double nf, double dz) {
    const size_t c1 = (size_t)lo.nr * m.L, c2 = (size_t)lo.ni * m.L;
    const size_t n1 = (size_t)hi.nr * m.L, n2 = (size_t)hi.ni * m.L;
    const double linefreq = m.line[l];
    const double iwc = interpolate_linear(m.iw[c1 + l], m.iw[c2 + l], lo.fac);
    const double iwn = interpolate_linear(m.iw[n1 + l], m.iw[n2 + l], hi.fac);
    const double avg_iw = (iwc + iwn) / 2.0;
    const double cop = ilog_s(m.op[c1 + l], m.op[c2 + l], lo.fac);
    const double nop = ilog_s(m.op[n1 + l], m.op[n2 + l], hi.fac);
    if (cf == nf) return dz * (gauss_s(avg_iw, cf - linefreq) * ((cop + nop) / 2.0) + m.min_opacity);
    const double next_pos = (linefreq - nf) * avg_iw;
    const double curr_pos = (linefreq - cf) * avg_iw;
    const double diff_pos = next_pos - curr_pos;
    const double erfterm = (nop + cop) / 2.0 / diff_pos / 2.0 * erf_diff_s(next_pos, curr_pos);
    return dz * (avg_iw * erfterm + m.min_opacity);
}

// Adjoint of ld_s for d(loss)/d(ld) = gld: per-point opacity / inverse width of both
// elements and d(loss)/d(cf), d(loss)/d(nf).
struct LdAdj {
    double g_iwc, g_iwn, g_cop, g_nop, g_cf, g_nf;
};
MGR_HD LdAdj ld_s_adj(const DevModel& m, const Elem& lo, const Elem& hi, uint32_t l, double cf, double nf, double dz,
                      double gld) {
    const size_t c1 = (size_t)lo.nr * m.L, c2 = (size_t)lo.ni * m.L;
    const size_t n1 = (size_t)hi.nr * m.L, n2 = (size_t)hi.ni * m.L;
    const double linefreq = m.line[l];
    const double iwc = interpolate_linear(m.iw[c1 + l], m.iw[c2 + l], lo.fac);
    const double iwn = interpolate_linear(m.iw[n1 + l], m.iw[n2 + l], hi.fac);
    const double avg = (iwc + iwn) / 2.0;
    const double cop = ilog_s(m.op[c1 + l], m.op[c2 + l], lo.fac);
    const double nop = ilog_s(m.op[n1 + l], m.op[n2 + l], hi.fac);
    LdAdj r{0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (cf == nf) {
        const double diff = cf - linefreq;
        const double prof = gauss_s(avg, diff);
        const double x = avg * diff;
        const double gprof = gld * dz * ((cop + nop) / 2.0);
        r.g_cop = r.g_nop = gld * dz * prof / 2.0;
        const double gavg = gprof * prof * (1.0 / avg - 2.0 * x * diff);
        r.g_cf = gprof * prof * (-2.0 * x * avg);
        r.g_iwc = r.g_iwn = gavg / 2.0;
        return r;
    }
    const double np = (linefreq - nf) * avg;
    const double cp = (linefreq - cf) * avg;
    const double dp = np - cp;
    const double avg_op = (nop + cop) / 2.0;
    const double E = erf_diff_s(np, cp);
    const double erfterm = avg_op / dp / 2.0 * E;
    const double g_erfterm = gld * dz * avg;
    double gavg = gld * dz * erfterm;
    const double g_avg_op = g_erfterm * E / (2.0 * dp);
    const double gE = g_erfterm * avg_op / (2.0 * dp);
    const double gdp = -g_erfterm * erfterm / dp;
    const double two_rsqpi = 2.0 * INVERSE_SQRT_PI;
    double gnp = gE * two_rsqpi * exp(-np * np) + gdp;
    double gcp = -gE * two_rsqpi * exp(-cp * cp) - gdp;
    gavg += gnp * (linefreq - nf) + gcp * (linefreq - cf);
    r.g_nf = -gnp * avg;
    r.g_cf = -gcp * avg;
    r.g_iwc = r.g_iwn = gavg / 2.0;
    r.g_cop = r.g_nop = g_avg_op / 2.0;
    return r;
}

// Pair quantities (eval_pair, FP64, smooth).  For the trapezoid branch the element
// emissivity / opacity are returned too.
struct PairS {
    bool large;
    double dtau, Slo, Shi;
    double eta_o, chi_o, eta_i, chi_i;  // trapezoid branch
    double sum_dtau, sum_c, sum_n;       // large branch, before the clamp
};

template <int AP>
MGR_HD bool pair_large(const DevModel& m, const Elem& outer, const Elem& inner) {
    const double dshift_abs = fabs(dsub_rn(inner.shift, outer.shift));
    const double a = m.dshift_max[outer.nr], b = m.dshift_max[inner.nr];
    return dshift_abs > (a < b ? a : b);
}

template <int AP>
MGR_HD PairS pair_s(const DevModel& m, const double* sl, double nu, const Elem& outer, const Elem& inner, double dz) {
    PairS r{};
    r.large = pair_large<AP>(m, outer, inner);
    if (!r.large) {
        elem_s<AP>(m, sl, nu, outer, r.eta_o, r.chi_o);
        elem_s<AP>(m, sl, nu, inner, r.eta_i, r.chi_i);
        r.Slo = r.eta_o / r.chi_o;
        r.Shi = r.eta_i / r.chi_i;
        r.dtau = 0.5 * (r.chi_o + r.chi_i) * dz;
        return r;
    }
    const double cf = nu * outer.shift, nf = nu * inner.shift;
    uint32_t a, b;
    pair_bracket<AP>(m, sl, cf, nf, outer.nr, inner.nr, a, b);
    const size_t c1 = (size_t)outer.nr * m.L, c2 = (size_t)outer.ni * m.L;
    const size_t n1 = (size_t)inner.nr * m.L, n2 = (size_t)inner.ni * m.L;
    double sd = 0.0, sc = 0.0, sn = 0.0;
    for (uint32_t s = a; s < b; s++) {
        const uint32_t l = line_of<AP>(m, s);
        const double ld = ld_s(m, outer, inner, l, cf, nf, dz);
        sd += ld;
        sc += ld * ilog_s(m.Sp[c1 + l], m.Sp[c2 + l], outer.fac);
        sn += ld * ilog_s(m.Sp[n1 + l], m.Sp[n2 + l], inner.fac);
    }
    r.sum_dtau = sd;
    r.sum_c = sc;
    r.sum_n = sn;
    double d = sd;
    if (AP != APPROX_NONE) {
        const double bound_min_dtau = m.min_opacity * dz;
        if (-bound_min_dtau < d) d = (bound_min_dtau > d) ? bound_min_dtau : d;
    }
    r.dtau = d;
    r.Slo = sc / d;
    r.Shi = sn / d;
    return r;
}

// Adjoint of a large-shift pair: d(loss)/d(dtau, Slo, Shi) -> per-point line data and
// the two elements' shifts.
template <int AP>
MGR_HD void pair_large_adj(const DevModel& m, const double* sl, double nu, const Elem& outer, const Elem& inner,
                           double dz, const PairS& f, double g_dt, double g_Slo, double g_Shi, const AdjAcc& acc,
                           double& g_sh_o, double& g_sh_i) {
    const double d = f.dtau;
    const double gd = g_dt - g_Slo * f.Slo / d - g_Shi * f.Shi / d;
    const double gsc = g_Slo / d, gsn = g_Shi / d;
    const double gsd = (d == f.sum_dtau) ? gd : 0.0;  // a clamped dtau does not move
    const double cf = nu * outer.shift, nf = nu * inner.shift;
    uint32_t a, b;
    pair_bracket<AP>(m, sl, cf, nf, outer.nr, inner.nr, a, b);
    uint32_t wa = a, wb = b;
    warp_range(wa, wb);
    const size_t c1 = (size_t)outer.nr * m.L, c2 = (size_t)outer.ni * m.L;
    const size_t n1 = (size_t)inner.nr * m.L, n2 = (size_t)inner.ni * m.L;
    const double fo = outer.fac, fi = inner.fac;
    for (uint32_t s = wa; s < wb; s++) {
        const uint32_t l = line_of<AP>(m, s);
        // per point: [outer nr, outer ni, inner nr, inner ni]
        double gop[4] = {0.0, 0.0, 0.0, 0.0}, giw[4] = {0.0, 0.0, 0.0, 0.0}, gsp[4] = {0.0, 0.0, 0.0, 0.0};
        if (s >= a && s < b) {
            const double ld = ld_s(m, outer, inner, l, cf, nf, dz);
            const double lsc = ilog_s(m.Sp[c1 + l], m.Sp[c2 + l], fo);
            const double lsn = ilog_s(m.Sp[n1 + l], m.Sp[n2 + l], fi);
            const double gld = gsd + gsc * lsc + gsn * lsn;
            const double glsc = gsc * ld, glsn = gsn * ld;
            const LdAdj r = ld_s_adj(m, outer, inner, l, cf, nf, dz, gld);
            g_sh_o += r.g_cf * nu;
            g_sh_i += r.g_nf * nu;
            const double cop = ilog_s(m.op[c1 + l], m.op[c2 + l], fo);
            const double nop = ilog_s(m.op[n1 + l], m.op[n2 + l], fi);
            gop[0] = r.g_cop * (1.0 - fo) * cop / m.op[c1 + l];
            gop[2] = r.g_nop * (1.0 - fi) * nop / m.op[n1 + l];
            giw[0] = r.g_iwc * (1.0 - fo);
            giw[2] = r.g_iwn * (1.0 - fi);
            gsp[0] = glsc * (1.0 - fo) * lsc / m.Sp[c1 + l];
            gsp[2] = glsn * (1.0 - fi) * lsn / m.Sp[n1 + l];
            if (fo != 0.0) {
                gop[1] = r.g_cop * fo * cop / m.op[c2 + l];
                giw[1] = r.g_iwc * fo;
                gsp[1] = glsc * fo * lsc / m.Sp[c2 + l];
            }
            if (fi != 0.0) {
                gop[3] = r.g_nop * fi * nop / m.op[n2 + l];
                giw[3] = r.g_iwn * fi;
                gsp[3] = glsn * fi * lsn / m.Sp[n2 + l];
            }
        }
        const uint32_t pts[4] = {outer.nr, outer.ni, inner.nr, inner.ni};
        for (int j = 0; j < 4; j++) {
            if ((j == 1 && fo == 0.0) || (j == 3 && fi == 0.0)) continue;
            acc.add(ADJ_OP, pts[j], l, gop[j]);
            acc.add(ADJ_IW, pts[j], l, giw[j]);
            acc.add(ADJ_SP, pts[j], l, gsp[j]);
        }
    }
}

// An element's shift derivative onto its two points: shift = fac sh(ni) + (1 - fac) sh(nr).
MGR_HD void elem_shift_adj(const Elem& e, double g_shift, const AdjAcc& acc) {
    acc.add_shift(e.nr, g_shift * (1.0 - e.fac));
    if (e.fac != 0.0) acc.add_shift(e.ni, g_shift * e.fac);
}

// Scratch of one lane: elimination state after pair k, (F, Su, dtau) at
// scr[(3 k + j) * stride].
struct LaneScratch {
    double* p;
    int stride;
    uint32_t cap;  // pairs
    MGR_HD double& at(uint32_t k, int j) const { return p[(size_t)(3 * k + j) * stride]; }
};

// Smooth forward of one pixel ray for one frequency (image_lane with nb > 0, nf = 0):
// the elements of the traced half bk from its far end to the start point o.  With a
// scratch, stores the elimination state per pair.  Returns the intensity; *npairs is
// the number of pairs (0 for a ray without interior points), or ~0u on scratch
// overflow.
template <int AP>
MGR_HD double image_lane_s(const DevModel& m, const double* sl, uint32_t o, double nu, const HalfSmem& bk, int nb,
                           const LaneScratch* scr, uint32_t* npairs) {
    double dummy;
    *npairs = 0;
    if (nb <= 0) return bdy_s(m, o, nu, dummy);
    const Elem cen = centre_elem(o, bk.cshift);
    ElemIter it;
    Elem prev;
    iter_begin<MODE_FP64>(m, bk, o, kAllLines, nb, it);
    iter_next<MODE_FP64>(m, bk, o, kAllLines, it, prev);
    const double Ib = bdy_s(m, prev.nr, nu * prev.shift, dummy);
    double F = 0.0, Su = 0.0, dt_prev = 0.0, S_last = 0.0;
    uint32_t k = 0;
    bool done = false;
    while (!done) {
        Elem cur;
        if (!iter_next<MODE_FP64>(m, bk, o, kAllLines, it, cur)) {
            cur = cen;
            done = true;
        }
        const PairS ps = pair_s<AP>(m, sl, nu, prev, cur, prev.dzin);
        const double dt = ps.dtau;
        if (k == 0) {
            // first row, Su = (S + 2 Ib/dt) / (1 + 2/dt + 2/dt^2) and F = (1 + 2/dt) dt^2/2,
            // multiplied through by dt^2/2 (no 1/dt: well conditioned for thin pairs)
            const double h = dt * (0.5 * dt + 1.0);
            F = h;
            Su = (ps.Slo * (0.5 * dt * dt) + Ib * dt) / (1.0 + h);
        } else {
            // elimination row with q = A iC = dt / dt_prev
            const double q = dt / dt_prev;
            const double iC = 0.5 * (dt_prev + dt) * dt;
            F = q * (F / (1.0 + F)) + iC;
            Su = (q * Su + ps.Slo * iC) / (1.0 + F);
        }
        if (scr) {
            if (k >= scr->cap) {
                *npairs = ~0u;
                return 0.0;
            }
            scr->at(k, 0) = F;
            scr->at(k, 1) = Su;
            scr->at(k, 2) = dt;
        }
        dt_prev = dt;
        S_last = ps.Shi;
        prev = cur;
        k++;
    }
    *npairs = k;
    // last row, u = (Al Su + Sl)(1 + F) / (Bl F + Bl - Al) times dt^2/2 over dt^2/2
    const double Ibl = bdy_s(m, o, nu * cen.shift, dummy);
    const double e = dt_prev;
    const double h = e * (0.5 * e + 1.0);
    const double N = Su + S_last * (0.5 * e * e) + Ibl * e;
    const double u = N * (1.0 + F) / (F + (1.0 + F) * h);
    return 2.0 * u - bdy_s(m, o, nu, dummy);
}

// Adjoint of image_lane_s for d(loss)/d(I) = gI: runs the forward sweep into the
// scratch, then the reverse sweep from the start point outward, adding the per-point
// derivatives into acc.  Every lane of a warp calls it for the same ray (lanes beyond
// the frequencies with gI = 0).  Returns false on scratch overflow.
template <int AP>
MGR_HD bool image_lane_adj(const DevModel& m, const double* sl, uint32_t o, double nu, const HalfSmem& bk, int nb,
                           double gI, const LaneScratch& scr, const AdjAcc& acc) {
    uint32_t M = 0;
    image_lane_s<AP>(m, sl, o, nu, bk, nb, &scr, &M);
    bool ok = M != ~0u;
#ifdef __CUDA_ARCH__
    ok = __all_sync(FULL_MASK, ok);
#endif
    if (!ok) return false;
    if (nb <= 0) return true;  // I = B(nu) of the start point: no dependence
    const Elem cen = centre_elem(o, bk.cshift);
    double dummy, dB;
    // ---- end of the ray: u = N (1 + F) / (F + (1 + F) h), I = 2 u - B(nu) ----
    const double F_last = scr.at(M - 1, 0), Su_last = scr.at(M - 1, 1), dtl = scr.at(M - 1, 2);
    const double Ibl = bdy_s(m, o, nu * cen.shift, dB);
    const double hl = dtl * (0.5 * dtl + 1.0);
    const double Dn = F_last + (1.0 + F_last) * hl;
    const double gu = 2.0 * gI;
    // adjoints of the state (F, Su) after the current pair and of its dtau
    double gF = 0.0, gSu = 0.0, gdt = 0.0;
    // Pairs in reverse: pair k joins element k (outer) and k + 1 (inner, the start point
    // for the last pair).  The last pair comes first; its Shi is the S_last of the end.
    ElemIter it;
    iter_up_begin<MODE_FP64>(m, bk, o, kAllLines, nb, it);
    Elem inner = cen, outer;
    double carry_eta = 0.0, carry_chi = 0.0;  // adjoint of the inner element's eta/chi from the pair outside it
    bool have_carry = false;
    double g_sh_inner_carry = 0.0;  // shift adjoint of the inner element from the pair outside it
    for (uint32_t kk = M; kk-- > 0;) {
        iter_up_next<MODE_FP64>(m, bk, o, kAllLines, it, outer);
        const double dz = outer.dzin;
        const PairS ps = pair_s<AP>(m, sl, nu, outer, inner, dz);
        double gSlo = 0.0, gShi = 0.0;
        if (kk == M - 1) {
            const double N = Su_last + ps.Shi * (0.5 * dtl * dtl) + Ibl * dtl;
            const double u = N * (1.0 + F_last) / Dn;
            const double gN = gu * (1.0 + F_last) / Dn;
            gF += gu * (N - u * (1.0 + hl)) / Dn;
            const double gh = -gu * u * (1.0 + F_last) / Dn;
            gSu += gN;
            gShi = gN * (0.5 * dtl * dtl);
            const double gIbl = gN * dtl;
            gdt += gN * (ps.Shi * dtl + Ibl) + gh * (dtl + 1.0);
            acc.add_shift(o, gIbl * dB * nu);  // Ibl = B(nu shift(start))
        }
        const double dt = ps.dtau;
        double g_dt_k;
        double g_sh_o = 0.0, g_sh_i = g_sh_inner_carry;
        if (kk > 0) {
            // pair kk: F_k = q G' + iC, Su_k = Z / (1 + F_k), G' = F'/(1 + F'),
            // Z = q Su' + S iC, q = dt / dto, iC = (dto + dt) dt / 2
            const double Fp = scr.at(kk - 1, 0), Sup = scr.at(kk - 1, 1), dto = scr.at(kk - 1, 2);
            const double Fk = scr.at(kk, 0);
            const double q = dt / dto;
            const double iC = 0.5 * (dto + dt) * dt;
            const double FIp = 1.0 / (1.0 + Fp);
            const double G = Fp * FIp;
            const double FIk = 1.0 / (1.0 + Fk);
            const double Z = q * Sup + ps.Slo * iC;
            const double gZ = gSu * FIk;
            const double gFt = gF - gSu * Z * FIk * FIk;
            const double gq = gFt * G + gZ * Sup;
            const double giC = gFt + gZ * ps.Slo;
            gSlo = gZ * iC;
            g_dt_k = gdt + gq / dto + giC * (0.5 * dto + dt);
            // hand the state adjoint to pair kk - 1
            gF = gFt * q * FIp * FIp;
            gSu = gZ * q;
            gdt = -gq * q / dto + giC * 0.5 * dt;
        } else {
            // pair 0: F_0 = h, Su_0 = N0 / (1 + h), N0 = S0 dt^2/2 + Ib dt, h = dt (dt/2 + 1)
            double dBf;
            const double Ib = bdy_s(m, outer.nr, nu * outer.shift, dBf);
            const double h = dt * (0.5 * dt + 1.0);
            const double FI0 = 1.0 / (1.0 + h);
            const double N0 = ps.Slo * (0.5 * dt * dt) + Ib * dt;
            const double gN0 = gSu * FI0;
            const double gh = gF - gSu * N0 * FI0 * FI0;
            gSlo = gN0 * (0.5 * dt * dt);
            const double gIb = gN0 * dt;
            g_dt_k = gdt + gN0 * (ps.Slo * dt + Ib) + gh * (dt + 1.0);
            g_sh_o = gIb * dBf * nu;
        }
        // ---- pair adjoint ----
        if (ps.large) {
            pair_large_adj<AP>(m, sl, nu, outer, inner, dz, ps, g_dt_k, gSlo, gShi, acc, g_sh_o, g_sh_i);
            // the inner element's eta/chi adjoint from the pair outside it is complete
            if (have_carry) elem_s_adj<AP>(m, sl, nu, inner, carry_eta, carry_chi, acc, g_sh_i);
            carry_eta = carry_chi = 0.0;
            have_carry = false;
        } else {
            const double ce = carry_eta + gShi / ps.chi_i;
            const double cc = carry_chi + 0.5 * dz * g_dt_k - gShi * ps.Shi / ps.chi_i;
            elem_s_adj<AP>(m, sl, nu, inner, ce, cc, acc, g_sh_i);
            carry_eta = gSlo / ps.chi_o;
            carry_chi = 0.5 * dz * g_dt_k - gSlo * ps.Slo / ps.chi_o;
            have_carry = true;
        }
        elem_shift_adj(inner, g_sh_i, acc);
        if (kk == 0) {
            // element 0 (the far end) is complete
            if (have_carry) elem_s_adj<AP>(m, sl, nu, outer, carry_eta, carry_chi, acc, g_sh_o);
            elem_shift_adj(outer, g_sh_o, acc);
        }
        g_sh_inner_carry = g_sh_o;
        inner = outer;
    }
    (void)dummy;
    return true;
}

}  // namespace mgr
