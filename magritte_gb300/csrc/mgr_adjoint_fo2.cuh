// Differentiable formal solve: a smooth FP64 forward of the two-sided second-order
// Feautrier solve (Solver::solve_feautrier_order_2, src/solver/solver.tpp:458-540
// driver, :2193-2318 per frequency) and its hand-written adjoint, for gradients of J.
//
// Forward.  solve_lane's FP64 recurrences (both halves of the ray pair eliminated
// toward the origin, combined there) with the pair physics of the differentiable
// imager (mgr_adjoint.cuh: exp / pow / erf / expm1 in double precision instead of the
// reference's single-precision calls), so that u is a smooth function of the per-point
// line data, the velocities (through the comoving shifts 1 + (v[p] - v[o]) . n) and
// the origin's frequencies nu(o, f).  Boundary rows are multiplied through by dtau^2/2
// (no 1/dtau: well conditioned for thin pairs); an interior row is
//     F_k = q F_{k-1} / (1 + F_{k-1}) + iC,   Su_k = (q Su_{k-1} + S_k iC) / (1 + F_k)
// with q = dtau_k / dtau_{k-1} and iC = (dtau_{k-1} + dtau_k) dtau_k / 2, which is the
// reference's row A = 1/(dtau_avg dtau_{k-1}), C^-1 = dtau_avg dtau_k in product form.
// The ray traces, interpolation points, CloseLines brackets, the large-shift branch and
// the optical-depth clamp are held at the model's state (trace-fixed derivatives).
//
// Adjoint.  Per lane (origin o, ray pair rr, frequency f) the forward stores each
// pair's (F, Su, dtau, row source) in a scratch array of the warp's slot (recomputed,
// never saved by the forward pass), the combination at the origin is reversed, then
// each half is walked back from the origin outward: the reverse rows give the
// adjoints of each pair's optical depth and sources, and the pair / element adjoints of
// the imager turn those into per-point derivatives.  Lanes of a warp share the ray pair
// and the line, so every per-point entry is summed over the warp before one atomic.
#pragma once
#include "mgr_adjoint.cuh"

namespace mgr {

// Per-pair scratch of one lane: (F, Su, dtau, row source) of pair k at
// p[(4 k + j) * stride]; the backward half's pairs come first, then the forward half's.
struct Fo2Scratch {
    double* p;
    int stride;
    uint32_t cap;  // pairs
    MGR_HD double& at(uint32_t k, int j) const { return p[(size_t)(4 * k + j) * stride]; }
};

// End state of one half's elimination toward the origin.
struct HalfS {
    double F, Su, dt;  // after the last pair (the one ending on the origin)
    double S_in;       // source of the origin from the last pair
    uint32_t n;        // pairs (0: empty half)
    bool ovf;          // scratch too small
};

// Smooth elimination of one half (elements of h from the outer end to the origin,
// line l's interpolation points).  side 0 (the backward half, the first rows of the
// reference's ray) takes each pair's outer source as its row source; side 1 (the
// forward half, rows last .. centre+1) takes the outer source for its boundary row and
// the previous pair's inner source after it.  With a scratch, stores every pair's
// state at k0 + k.
template <int AP>
MGR_HD HalfS half_s(const DevModel& m, const double* sl, uint32_t o, double nu, const HalfSmem& h, int nsteps,
                    uint32_t l, int side, const Fo2Scratch* scr, uint32_t k0) {
    HalfS r{0.0, 0.0, 0.0, 0.0, 0u, false};
    if (nsteps <= 0) return r;
    const Elem cen = centre_elem(o);
    ElemIter it;
    Elem prev;
    iter_begin<MODE_FP64>(m, h, o, l, nsteps, it);
    iter_next<MODE_FP64>(m, h, o, l, it, prev);
    double dummy;
    const double Ib = bdy_s(m, prev.nr, nu * prev.shift, dummy);
    double F = 0.0, Su = 0.0, dt_prev = 0.0, S_carry = 0.0;
    uint32_t k = 0;
    bool done = false;
    while (!done) {
        Elem cur;
        if (!iter_next<MODE_FP64>(m, h, o, l, it, cur)) {
            cur = cen;
            done = true;
        }
        const PairS ps = pair_s<AP>(m, sl, nu, prev, cur, prev.dzin);
        const double dt = ps.dtau;
        const double S_row = (side == 0 || k == 0) ? ps.Slo : S_carry;
        if (k == 0) {
            const double h0 = dt * (0.5 * dt + 1.0);
            F = h0;
            Su = (S_row * (0.5 * dt * dt) + Ib * dt) / (1.0 + h0);
        } else {
            const double q = dt / dt_prev;
            const double iC = 0.5 * (dt_prev + dt) * dt;
            F = q * (F / (1.0 + F)) + iC;
            Su = (q * Su + S_row * iC) / (1.0 + F);
        }
        if (scr) {
            if (k0 + k >= scr->cap) {
                r.ovf = true;
                return r;
            }
            scr->at(k0 + k, 0) = F;
            scr->at(k0 + k, 1) = Su;
            scr->at(k0 + k, 2) = dt;
            scr->at(k0 + k, 3) = S_row;
        }
        dt_prev = dt;
        S_carry = ps.Shi;
        prev = cur;
        k++;
    }
    r.F = F;
    r.Su = Su;
    r.dt = dt_prev;
    r.S_in = S_carry;
    r.n = k;
    return r;
}

struct LaneS {
    double u;
    HalfS top, bot;
    bool ovf;
};

// Smooth u(o, rr, f) of the ray pair staged in bk (backward half) / fw (forward half)
// for frequency nu of line l, with solve_lane's three cases at the origin (both halves,
// origin first, origin last) and the boundary intensity for a ray pair of one point.
template <int AP>
MGR_HD LaneS solve_lane_s(const DevModel& m, const double* sl, uint32_t o, double nu, uint32_t l, const HalfSmem& bk,
                          int nb, const HalfSmem& fw, int nf, const Fo2Scratch* scr) {
    LaneS r;
    r.ovf = false;
    r.top = r.bot = HalfS{0.0, 0.0, 0.0, 0.0, 0u, false};
    double dummy;
    if (nb <= 0 && nf <= 0) {
        r.u = bdy_s(m, o, nu, dummy);
        return r;
    }
    r.top = half_s<AP>(m, sl, o, nu, bk, nb, l, 0, scr, 0);
    r.bot = half_s<AP>(m, sl, o, nu, fw, nf, l, 1, scr, r.top.n);
    r.ovf = r.top.ovf || r.bot.ovf;
    if (r.ovf) {
        r.u = 0.0;
        return r;
    }
    const HalfS& T = r.top;
    const HalfS& B = r.bot;
    if (T.n && B.n) {
        const double q = B.dt / T.dt;
        const double iC = 0.5 * (T.dt + B.dt) * B.dt;
        const double num = q * T.Su + B.S_in * iC + B.Su;
        const double den = q * (T.F / (1.0 + T.F)) + iC + B.F / (1.0 + B.F);
        r.u = num / den;
    } else if (B.n) {  // the origin is the first element: its own boundary row
        const double Ib = bdy_s(m, o, nu, dummy);
        const double e = B.dt;
        const double h = e * (0.5 * e + 1.0);
        r.u = (B.S_in * (0.5 * e * e) + Ib * e + B.Su) / (h + B.F / (1.0 + B.F));
    } else {  // the origin is the last element
        const double Ib = bdy_s(m, o, nu, dummy);
        const double e = T.dt;
        const double h = e * (0.5 * e + 1.0);
        const double N = T.Su + T.S_in * (0.5 * e * e) + Ib * e;
        r.u = N * (1.0 + T.F) / (T.F + (1.0 + T.F) * h);
    }
    return r;
}

// Shift adjoint of an element of a formal-solve ray onto the velocities (comoving
// shift 1 + (v[p] - v[o]) . n of the element's two points, interpolated with weights
// 1 - fac / fac; the origin's own shift is exactly 1) and onto the lane's frequency
// (the element's frequency is nu * shift).  gvo collects the origin's share along n.
MGR_HD void shift_adj_comoving(const Elem& e, double g, uint32_t o, double nu, const AdjAcc& acc, double& gvo,
                               double& g_nu) {
    g_nu += g * e.shift / nu;
    if (e.nr == o) return;  // the origin element
    const double w_nr = 1.0 - e.fac;
    acc.add_shift(e.nr, g * w_nr);
    double w = w_nr;
    if (e.fac != 0.0 && e.ni != o) {
        acc.add_shift(e.ni, g * e.fac);
        w += e.fac;
    }
    gvo -= g * w;
}

// Reverse of half_s for the adjoints (gF, gSu, gdt, gSin) of its end state: per-point
// line-data derivatives into acc (direction of this half for the velocities), the
// origin's velocity share into gvo, the frequency derivative into g_nu.  Every lane of
// the warp calls it for the same half and line.
template <int AP>
MGR_HD void half_s_adj(const DevModel& m, const double* sl, uint32_t o, double nu, const HalfSmem& h, int nsteps,
                       uint32_t l, int side, const Fo2Scratch& scr, uint32_t k0, uint32_t n, double gF, double gSu,
                       double gdt, double gSin, const AdjAcc& acc, double& gvo, double& g_nu) {
    if (n == 0) return;
    const Elem cen = centre_elem(o);
    ElemIter it;
    iter_up_begin<MODE_FP64>(m, h, o, l, nsteps, it);
    Elem inner = cen, outer;
    double carry_eta = 0.0, carry_chi = 0.0;  // inner element's eta / chi adjoint from the pair outside it
    bool have_carry = false;
    double g_sh_carry = 0.0;  // inner element's shift adjoint from the pair outside it
    double gShi_pend = gSin;  // adjoint of the current pair's inner source (next row's or the origin's)
    for (uint32_t kk = n; kk-- > 0;) {
        iter_up_next<MODE_FP64>(m, h, o, l, it, outer);
        const double dz = outer.dzin;
        const PairS ps = pair_s<AP>(m, sl, nu, outer, inner, dz);
        const double dt = scr.at(k0 + kk, 2);
        const double S_row = scr.at(k0 + kk, 3);
        double g_dt_k, gSrow, g_sh_o = 0.0;
        if (kk > 0) {
            const double Fp = scr.at(k0 + kk - 1, 0), Sup = scr.at(k0 + kk - 1, 1), dto = scr.at(k0 + kk - 1, 2);
            const double Fk = scr.at(k0 + kk, 0);
            const double q = dt / dto;
            const double iC = 0.5 * (dto + dt) * dt;
            const double FIp = 1.0 / (1.0 + Fp);
            const double G = Fp * FIp;
            const double FIk = 1.0 / (1.0 + Fk);
            const double Z = q * Sup + S_row * iC;
            const double gZ = gSu * FIk;
            const double gFt = gF - gSu * Z * FIk * FIk;
            const double gq = gFt * G + gZ * Sup;
            const double giC = gFt + gZ * S_row;
            gSrow = gZ * iC;
            g_dt_k = gdt + gq / dto + giC * (0.5 * dto + dt);
            gF = gFt * q * FIp * FIp;
            gSu = gZ * q;
            gdt = -gq * q / dto + giC * 0.5 * dt;
        } else {
            double dBf;
            const double Ib = bdy_s(m, outer.nr, nu * outer.shift, dBf);
            const double h0 = dt * (0.5 * dt + 1.0);
            const double FI0 = 1.0 / (1.0 + h0);
            const double N0 = S_row * (0.5 * dt * dt) + Ib * dt;
            const double gN0 = gSu * FI0;
            const double gh = gF - gSu * N0 * FI0 * FI0;
            gSrow = gN0 * (0.5 * dt * dt);
            g_dt_k = gdt + gN0 * (S_row * dt + Ib) + gh * (dt + 1.0);
            g_sh_o = gN0 * dt * dBf * nu;  // Ib = B(nu shift(outer))
        }
        const double gSlo = (side == 0 || kk == 0) ? gSrow : 0.0;
        const double gShi = gShi_pend;
        gShi_pend = (side == 1 && kk > 0) ? gSrow : 0.0;
        double g_sh_i = g_sh_carry;
        if (ps.large) {
            pair_large_adj<AP>(m, sl, nu, outer, inner, dz, ps, g_dt_k, gSlo, gShi, acc, g_sh_o, g_sh_i);
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
        shift_adj_comoving(inner, g_sh_i, o, nu, acc, gvo, g_nu);
        if (kk == 0) {
            if (have_carry) elem_s_adj<AP>(m, sl, nu, outer, carry_eta, carry_chi, acc, g_sh_o);
            shift_adj_comoving(outer, g_sh_o, o, nu, acc, gvo, g_nu);
        }
        g_sh_carry = g_sh_o;
        inner = outer;
    }
}

// Adjoint of solve_lane_s for d(loss)/d(u) = gu of one lane: the forward into the
// scratch, the reverse of the combination at the origin, then both halves in reverse.
// acc_b / acc_f carry the backward / forward half's direction for the velocity
// derivatives; gvo_b / gvo_f the origin's velocity shares along them; g_nu the lane's
// frequency derivative.  Every lane of a warp calls it for the same ray pair and line
// (lanes without a frequency with gu = 0).  Returns false on scratch overflow.
template <int AP>
MGR_HD bool solve_lane_s_adj(const DevModel& m, const double* sl, uint32_t o, double nu, uint32_t l,
                             const HalfSmem& bk, int nb, const HalfSmem& fw, int nf, double gu, const Fo2Scratch& scr,
                             const AdjAcc& acc_b, const AdjAcc& acc_f, double& gvo_b, double& gvo_f, double& g_nu) {
    double dB;
    if (nb <= 0 && nf <= 0) {
        bdy_s(m, o, nu, dB);
        g_nu += gu * dB;
        return true;
    }
    const LaneS fwd = solve_lane_s<AP>(m, sl, o, nu, l, bk, nb, fw, nf, &scr);
    bool ok = !fwd.ovf;
#ifdef __CUDA_ARCH__
    ok = __all_sync(FULL_MASK, ok);
#endif
    if (!ok) return false;
    const HalfS& T = fwd.top;
    const HalfS& B = fwd.bot;
    double gTF = 0.0, gTSu = 0.0, gTdt = 0.0, gTSin = 0.0;
    double gBF = 0.0, gBSu = 0.0, gBdt = 0.0, gBSin = 0.0;
    const double u = fwd.u;
    if (T.n && B.n) {
        const double GT = T.F / (1.0 + T.F), GB = B.F / (1.0 + B.F);
        const double q = B.dt / T.dt;
        const double iC = 0.5 * (T.dt + B.dt) * B.dt;
        const double den = q * GT + iC + GB;
        const double gNum = gu / den, gDen = -gu * u / den;
        gTSu = gNum * q;
        gBSu = gNum;
        gBSin = gNum * iC;
        const double gq = gNum * T.Su + gDen * GT;
        const double giC = gNum * B.S_in + gDen;
        gTF = gDen * q / ((1.0 + T.F) * (1.0 + T.F));
        gBF = gDen / ((1.0 + B.F) * (1.0 + B.F));
        gBdt = gq / T.dt + giC * (0.5 * T.dt + B.dt);
        gTdt = -gq * q / T.dt + giC * 0.5 * B.dt;
    } else if (B.n) {
        const double Ib = bdy_s(m, o, nu, dB);
        const double e = B.dt;
        const double den = e * (0.5 * e + 1.0) + B.F / (1.0 + B.F);
        const double gNum = gu / den, gDen = -gu * u / den;
        gBSu = gNum;
        gBSin = gNum * (0.5 * e * e);
        g_nu += gNum * e * dB;
        gBdt = gNum * (B.S_in * e + Ib) + gDen * (e + 1.0);
        gBF = gDen / ((1.0 + B.F) * (1.0 + B.F));
    } else {
        const double Ib = bdy_s(m, o, nu, dB);
        const double e = T.dt;
        const double h = e * (0.5 * e + 1.0);
        const double N = T.Su + T.S_in * (0.5 * e * e) + Ib * e;
        const double Dn = T.F + (1.0 + T.F) * h;
        const double gN = gu * (1.0 + T.F) / Dn;
        gTF = gu * (N - u * (1.0 + h)) / Dn;
        const double gh = -gu * u * (1.0 + T.F) / Dn;
        gTSu = gN;
        gTSin = gN * (0.5 * e * e);
        g_nu += gN * e * dB;
        gTdt = gN * (T.S_in * e + Ib) + gh * (e + 1.0);
    }
    half_s_adj<AP>(m, sl, o, nu, bk, nb, l, 0, scr, 0, T.n, gTF, gTSu, gTdt, gTSin, acc_b, gvo_b, g_nu);
    half_s_adj<AP>(m, sl, o, nu, fw, nf, l, 1, scr, T.n, B.n, gBF, gBSu, gBdt, gBSin, acc_f, gvo_f, g_nu);
    return true;
}

}  // namespace mgr
