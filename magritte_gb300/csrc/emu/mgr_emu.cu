#include <algorithm>
// CPU emulation of the formal-solve kernel for the test-suite.
//
// Runs the kernel's own per-lane code (solve_lane, lambda_element and everything
// they call, compiled for the host) over all origins, ray pairs and frequencies,
// with a sequential version of the warp trace.  It is never called by the product
// API (which fails without a GPU); it lets the CPU tests check the kernel's
// arithmetic against the oracle, and lets kernel logic be debugged without a GPU.
#include <cstring>
#include <vector>

#include "../../../include/magritte_gb300.h"
#include "../mgr_adjoint.cuh"
#include "../mgr_adjoint_fo2.cuh"
#include "../mgr_image.cuh"
#include "../mgr_scale.h"
#include "../mgr_solve.cuh"

using namespace mgr;

namespace {

// Failure returns of trace_half_host, as the kernel's status bits ST_TRACE / ST_CAPACITY.
constexpr int kTraceLeftGrid = -1;
constexpr int kTraceOverCapacity = -2;

// Sequential restatement of trace_half (same arithmetic, neighbour order, strict <).
int trace_half_host(const DevModel& m, uint32_t o, uint32_t r, uint32_t cap, HalfSmem& h, int frame = 0) {
    const double* d = frame ? m.raydir + 3 * r : ray_dir(m, o, r);
    const double4_32a po = m.pos[o];
    double Z = 0.0;
    uint32_t crt = o;
    int count = 0;
    if (m.sph) {
        // trace_half_sph
        const double Rcos = dot3_rn(po.x, po.y, po.z, d[0], d[1], d[2]);
        const double Rsin2 = dsub_rn(sqnorm_rn(po), dmul_rn(Rcos, Rcos));
        h.shift0 = origin_shift(m, frame, o, r);
        set_dsh0(h, h.shift0);
        while (true) {
            uint32_t nxt;
            double dZl;
            if (!next_point_sph(m, Rcos, Rsin2, crt, Z, nxt, dZl)) return count > 0 ? kTraceLeftGrid : 0;
            if ((uint32_t)count >= cap) return kTraceOverCapacity;
            Z = dadd_rn(Z, dZl);
            h.ids[count] = nxt;
            h.eid[count] = sph_eid(crt, nxt);
            h.dZ[count] = dZl;
            const double s = shift_sph(m, frame, o, r, nxt, Z, d);
            h.shift[count] = s;
            store_dsh(h, count, s);
            h.dzs[count] = (float)dZl * m.dz_scale;
            count++;
            if (m.p2b[nxt] != m.P) break;
            crt = nxt;
        }
        return count;
    }
    while (true) {
        const uint32_t nnb = m.n_nb[crt];
        const uint32_t cum = m.cum_nb[crt];
        double best = DBL_MAX;
        uint32_t besti = 0xffffffffu;
        double bestZ = 0.0;
        for (uint32_t i = 0; i < nnb; i++) {
            const double4_32a e = m.edge[cum + i];
            const double Rx = dsub_rn(e.x, po.x), Ry = dsub_rn(e.y, po.y), Rz = dsub_rn(e.z, po.z);
            const double Zn = dot3_rn(Rx, Ry, Rz, d[0], d[1], d[2]);
            if (Zn > Z) {
                const double d2 = dsub_rn(dot3_rn(Rx, Ry, Rz, Rx, Ry, Rz), dmul_rn(Zn, Zn));
                if (d2 < best) {
                    best = d2;
                    besti = i;
                    bestZ = Zn;
                }
            }
        }
        if (besti == 0xffffffffu) return count > 0 ? kTraceLeftGrid : 0;
        if ((uint32_t)count >= cap) return kTraceOverCapacity;
        long long bits;
        std::memcpy(&bits, &m.edge[cum + besti].w, 8);
        const uint32_t nxt = (uint32_t)bits;
        const double dZl = dsub_rn(bestZ, Z);
        Z = dadd_rn(Z, dZl);
        h.ids[count] = nxt;
        h.eid[count] = cum + besti;
        h.dZ[count] = dZl;
        const double s = frame ? shift_rest(m, r, nxt, d) : shift_comoving(m, o, nxt, d);
        h.shift[count] = s;
        store_dsh(h, count, s);
        h.dzs[count] = (float)dZl * m.dz_scale;
        count++;
        if (m.p2b[nxt] != m.P) break;
        crt = nxt;
    }
    return count;
}

// Sequential restatement of trace_half's FP32-filtered walk (the same float
// arithmetic as the device: filt_cand / filt_ahead, explicit fmaf): the filter's
// decision where the device's would decide, the exact argmin elsewhere, exact Zn and dZ
// of the filter's steps chained afterwards in step order.  Writes ids / eid / dZ and
// counts the steps the exact argmin took.
int trace_half_host_f32(const DevModel& m, uint32_t o, uint32_t r, uint32_t cap, uint32_t* ids, uint32_t* eids,
                        double* dZs, uint64_t& exact_steps) {
    const double* d = ray_dir(m, o, r);
    const double4_32a po = m.pos[o];
    TraceF32 t;
    t.poh = m.pos_hl[2 * (size_t)o];
    t.pol = m.pos_hl[2 * (size_t)o + 1];
    t.dx = (float)d[0];
    t.dy = (float)d[1];
    t.dz = (float)d[2];
    t.Zc = 0.0f;
    t.eZc = 0.0f;
    double Z = 0.0;
    int count = 0, np = 0;
    auto flush = [&]() {
        for (int j = count - np; j < count; j++) {
            const double4_32a q = m.pos[ids[j]];
            const double Zn = dot3_rn(dsub_rn(q.x, po.x), dsub_rn(q.y, po.y), dsub_rn(q.z, po.z), d[0], d[1], d[2]);
            const double dZl = dsub_rn(Zn, Z);
            Z = dadd_rn(Z, dZl);
            dZs[j] = dZl;
        }
        np = 0;
    };
    uint32_t crt = o;
    while (true) {
        const uint32_t nnb = m.n_nb[crt], cum = m.cum_nb[crt];
        int found = -1;
        uint32_t nxt = 0, eid = 0;
        float Zw = 0.0f, EZw = 0.0f;
        if (nnb <= 32) {
            FiltCand c[32];
            int ah[32];
            float best = INFINITY;
            for (uint32_t i = 0; i < nnb; i++) {
                c[i] = filt_cand(m.edge_hl[2 * (size_t)(cum + i)], m.edge_hl[2 * (size_t)(cum + i) + 1], t);
                ah[i] = filt_ahead(c[i], t);
                if (ah[i] > 0) best = std::fmin(best, c[i].hi);
            }
            int ncont = 0, w = -1;
            for (uint32_t i = 0; i < nnb; i++)
                if (ah[i] >= 0 && c[i].lo <= best) {
                    ncont++;
                    if (w < 0) w = (int)i;
                }
            if (ncont == 0) {
                found = 0;
            } else if (ncont == 1 && ah[w] == 1) {
                found = 1;
                nxt = f32_bits(m.edge_hl[2 * (size_t)(cum + w)].w);
                eid = cum + (uint32_t)w;
                Zw = c[w].Zf;
                EZw = c[w].EZ;
            }
        }
        bool exact = false;
        double dZl = 0.0;
        if (found < 0) {
            flush();
            exact_steps++;
            double best = DBL_MAX, bestZ = 0.0;
            uint32_t besti = 0xffffffffu;
            for (uint32_t i = 0; i < nnb; i++) {
                const double4_32a e = m.edge[cum + i];
                const double Rx = dsub_rn(e.x, po.x), Ry = dsub_rn(e.y, po.y), Rz = dsub_rn(e.z, po.z);
                const double Zn = dot3_rn(Rx, Ry, Rz, d[0], d[1], d[2]);
                if (Zn > Z) {
                    const double d2 = dsub_rn(dot3_rn(Rx, Ry, Rz, Rx, Ry, Rz), dmul_rn(Zn, Zn));
                    if (d2 < best) {
                        best = d2;
                        besti = i;
                        bestZ = Zn;
                    }
                }
            }
            found = besti != 0xffffffffu ? 1 : 0;
            if (found) {
                exact = true;
                long long bits;
                std::memcpy(&bits, &m.edge[cum + besti].w, 8);
                nxt = (uint32_t)bits;
                eid = cum + besti;
                dZl = dsub_rn(bestZ, Z);
                Z = dadd_rn(Z, dZl);
                Zw = (float)dmul_rn(Z, m.pos_scale);
                EZw = fmaf(2.0f * kU32, fabsf(Zw), 32.0f * kU32Sq);
            }
        }
        if (!found) return count > 0 ? kTraceLeftGrid : 0;
        if ((uint32_t)count >= cap) return kTraceOverCapacity;
        ids[count] = nxt;
        eids[count] = eid;
        if (exact) dZs[count] = dZl;
        else np++;
        count++;
        t.Zc = Zw;
        t.eZc = EZw;
        if (np == 32) flush();
        if (m.p2b[nxt] != m.P) break;
        crt = nxt;
    }
    flush();
    return count;
}

float to_f32_floor_host(double x) {
    const float f = (float)x;
    return (x > 0.0 && f < FLT_MIN) ? FLT_MIN : f;
}

// Host copies of the device-model tables mgr_model_create builds on the GPU.
struct EmuModel {
    std::vector<double4_32a> pos, vel, edge;
    std::vector<double> ub, Sp;
    std::vector<float> em_f, op_f, iw_f, Sp_f, dsm_f, dls, dll, ub_f, iw_lo, line_df, bkt;
    std::vector<uint16_t> nint, nint_all;
    std::vector<uint32_t> lq2f, corr_line;
    std::vector<float4> edge_hl, pos_hl;
    DevModel m{};
};

void build_emu_model(const MgrModelDesc* d, EmuModel& x) {
    const uint32_t P = d->npoints, L = d->nlines, F = d->nfreqs;
    size_t E = 0;
    for (uint32_t p = 0; p < P; p++) E += d->n_neighbors[p];
    x.pos.resize(P);
    x.vel.resize(P);
    x.edge.resize(E ? E : 1);
    for (uint32_t p = 0; p < P; p++) {
        x.pos[p] = make_double4_32a(d->position[3 * p], d->position[3 * p + 1], d->position[3 * p + 2], 0.0);
        x.vel[p] = make_double4_32a(d->velocity[3 * p], d->velocity[3 * p + 1], d->velocity[3 * p + 2], 0.0);
    }
    for (size_t i = 0; i < E; i++) {
        const uint32_t n = d->neighbors[i];
        long long bits = (long long)n;
        double w;
        std::memcpy(&w, &bits, 8);
        x.edge[i] = make_double4_32a(d->position[3 * n], d->position[3 * n + 1], d->position[3 * n + 2], w);
    }
    // trace filter tables, as hl_tables_kernel builds them
    double maxabs = 0.0;
    for (size_t i = 0; i < 3 * (size_t)P; i++) maxabs = std::max(maxabs, std::fabs(d->position[i]));
    int pexp = 0;
    if (maxabs > 0.0 && std::isfinite(maxabs)) std::frexp(maxabs, &pexp);
    const double pscale = std::ldexp(1.0, -pexp);
    x.edge_hl.resize(2 * (E ? E : 1));
    x.pos_hl.resize(2 * (size_t)P);
    auto hl = [&](const double4_32a& q, float w, float4* out) {
        split_hl(q.x * pscale, out[0].x, out[1].x);
        split_hl(q.y * pscale, out[0].y, out[1].y);
        split_hl(q.z * pscale, out[0].z, out[1].z);
        out[0].w = w;
        out[1].w = 0.0f;
    };
    for (size_t i = 0; i < E; i++) hl(x.edge[i], bits_f32(d->neighbors[i]), &x.edge_hl[2 * i]);
    for (uint32_t p = 0; p < P; p++) hl(x.pos[p], 0.0f, &x.pos_hl[2 * (size_t)p]);
    const size_t PL = (size_t)P * L;
    x.ub.resize(P);
    x.Sp.resize(PL);
    x.em_f.resize(PL);
    x.op_f.resize(PL);
    x.iw_f.resize(PL);
    x.iw_lo.resize(PL);
    x.Sp_f.resize(PL);
    x.dsm_f.resize(P);
    x.ub_f.resize(P);
    for (uint32_t p = 0; p < P; p++) {
        x.ub[p] = std::sqrt(TWO_KB_OVER_AMU_CC_SQUARED * d->max_inverse_mass * d->temperature[p] + d->vturb2[p]);
        x.dsm_f[p] = (float)d->dshift_max[p];
        x.ub_f[p] = (float)x.ub[p];
    }
    const double Ke = pow2_scale_for_max(d->emissivity, PL);
    const double Ko = pow2_scale_for_max(d->opacity, PL);
    for (size_t i = 0; i < PL; i++) {
        x.Sp[i] = d->emissivity[i] / d->opacity[i];
        x.em_f[i] = to_f32_floor_host(d->emissivity[i] * Ke);
        x.op_f[i] = to_f32_floor_host(d->opacity[i] * Ko);
        x.iw_f[i] = (float)d->inverse_width[i];
        x.iw_lo[i] = (float)(d->inverse_width[i] - (double)x.iw_f[i]);
        x.Sp_f[i] = to_f32_floor_host(x.Sp[i] * (Ke / Ko));
    }
    DevModel& m = x.m;
    m.P = P; m.nrays = d->nrays; m.hnrays = d->hnrays; m.L = L; m.Q = d->nquads; m.F = F;
    m.nlspecs = d->nlspecs; m.B = d->nboundary;
    m.pos = x.pos.data(); m.vel = x.vel.data(); m.n_nb = d->n_neighbors; m.cum_nb = d->cum_n_neighbors;
    m.edge = x.edge.data(); m.p2b = d->point2boundary; m.bc = d->boundary_condition;
    m.edge_hl = x.edge_hl.data(); m.pos_hl = x.pos_hl.data(); m.pos_scale = pscale;
    {
        const size_t NR = (size_t)d->nrays * (d->use_adaptive_directions ? P : 1);
        for (size_t i = 0; i < NR; i++) {
            const double* v = d->ray_direction + 3 * i;
            if (std::fabs(v[0] * v[0] + v[1] * v[1] + v[2] * v[2] - 1.0) > 2.0e-15) m.edge_hl = nullptr;
        }
    }
    m.bt = d->boundary_temperature; m.raydir = d->ray_direction; m.rayw = d->ray_weight; m.antipod = d->antipod;
    m.line = d->line; m.sorted_line = d->sorted_line; m.sorted_map = d->sorted_line_map;
    m.max_inv_mass = d->max_inverse_mass; m.em = d->emissivity; m.op = d->opacity; m.iw = d->inverse_width;
    m.Sp = x.Sp.data(); m.crit = d->interp_criterion; m.em_f = x.em_f.data(); m.op_f = x.op_f.data();
    m.iw_f = x.iw_f.data(); m.Sp_f = x.Sp_f.data(); m.ub = x.ub.data(); m.ub_f = x.ub_f.data(); m.T = d->temperature; m.vt2 = d->vturb2;
    m.dshift_max = d->dshift_max; m.dshift_max_f = x.dsm_f.data(); m.nu = d->nu; m.corr_line = d->corr_line;
    m.corr_lspec = d->corr_lspec; m.corr_k = d->corr_k; m.corr_z = d->corr_z; m.in_line = d->in_line_integral;
    m.nrad_cum = d->nrad_cum; m.line_A = d->line_A; m.lspec_inv_mass = d->lspec_inverse_mass;
    m.quad_w = d->quad_weights; m.min_opacity = d->min_opacity; m.min_dtau = d->min_dtau;
    m.max_interp_diff = d->max_interpolation_diff; m.max_dist = d->max_distance_opacity_contribution;
    m.max_dist_f = (float)m.max_dist;
    m.log_max_interp_diff = logf((float)d->max_interpolation_diff);
    m.approx = d->approx;
    m.sph = d->spherical_symmetry ? 1u : 0u;
    m.adaptive = d->use_adaptive_directions ? 1u : 0u;
    m.min_op_s = (float)(d->min_opacity * Ko);
    m.dz_scale = (float)(1.0 / Ko);
    m.s_scale = (float)(Ko / Ke);
    line_offset_tables(d->line, d->sorted_line, L, x.dls, x.dll);
    m.dls = x.dls.data();
    m.dll = x.dll.data();
    x.line_df.resize(2 * (size_t)L);
    for (uint32_t l = 0; l < L; l++) {
        x.line_df[2 * l] = (float)d->line[l];
        x.line_df[2 * l + 1] = (float)(d->line[l] - (double)x.line_df[2 * l]);
    }
    m.line_df = x.line_df.data();
    x.bkt.resize(d->nboundary ? 2 * (size_t)d->nboundary : 2);
    for (uint32_t b = 0; b < d->nboundary; b++) {
        const double k = HH_OVER_KB / (d->boundary_condition[b] == BC_THERMAL ? d->boundary_temperature[b] : T_CMB);
        x.bkt[2 * b] = (float)k;
        x.bkt[2 * b + 1] = (float)(k - (double)x.bkt[2 * b]);
    }
    m.bkt = x.bkt.data();
    m.iw_lo = x.iw_lo.data();
    // the maps of an imaging spectral discretisation are unset: keep only valid
    // (line, quadrature point) entries, and measure each frequency from its nearest
    // line, as mgr_model_create does
    x.lq2f.assign((size_t)L * d->nquads, 0xffffffffu);
    for (uint32_t f = 0; f < F; f++)
        if (d->corr_line[f] < L && d->corr_z[f] < d->nquads) x.lq2f[(size_t)d->corr_line[f] * d->nquads + d->corr_z[f]] = f;
    m.lq2f = x.lq2f.data();
    bool line_disc = (F == L * d->nquads);
    for (uint32_t f = 0; f < F && line_disc; f++)
        if (d->corr_line[f] >= L || d->corr_lspec[f] >= d->nlspecs || d->corr_z[f] >= d->nquads) line_disc = false;
    x.corr_line.resize(F);
    for (uint32_t f = 0; f < F; f++) {
        uint32_t best = 0;
        if (line_disc) {
            best = d->corr_line[f];
        } else {
            for (uint32_t l = 1; l < L; l++)
                if (std::fabs(d->nu[f] - d->line[l]) < std::fabs(d->nu[f] - d->line[best])) best = l;
        }
        x.corr_line[f] = best;
    }
    m.corr_line = x.corr_line.data();
    x.nint.resize((E ? E : 1) * (size_t)L);
    for (uint32_t p = 0; p < P; p++)
        for (uint32_t k = 0; k < d->n_neighbors[p]; k++)
            for (uint32_t l = 0; l < L; l++) {
                const size_t e = (size_t)d->cum_n_neighbors[p] + k;
                const uint32_t v = n_interp_for_line(m, l, p, d->neighbors[e]);
                x.nint[e * L + l] = (uint16_t)(v > 0xffffu ? 0xffffu : v);
            }
    m.nint = x.nint.data();
    x.nint_all.resize(E ? E : 1);
    for (uint32_t p = 0; p < P; p++)
        for (uint32_t k = 0; k < d->n_neighbors[p]; k++) {
            const size_t e = (size_t)d->cum_n_neighbors[p] + k;
            const uint32_t v = n_interp_all_lines(m, p, d->neighbors[e]);
            x.nint_all[e] = (uint16_t)(v > 0xffffu ? 0xffffu : v);
        }
    m.nint_all = x.nint_all.data();
    if (m.sph) {
        // three slots per point (sph_eid): p -> p, p -> p - 1, p -> p + 1
        x.nint.assign(3 * (size_t)P * L, 1);
        x.nint_all.assign(3 * (size_t)P, 1);
        for (uint32_t p = 0; p < P; p++)
            for (uint32_t k = 0; k < 3; k++) {
                const uint32_t nxt = sph_slot_point(p, k);
                if (nxt >= P) continue;
                for (uint32_t l = 0; l < L; l++) {
                    const uint32_t v = n_interp_for_line(m, l, p, nxt);
                    x.nint[(3 * (size_t)p + k) * L + l] = (uint16_t)(v > 0xffffu ? 0xffffu : v);
                }
                const uint32_t v = n_interp_all_lines(m, p, nxt);
                x.nint_all[3 * (size_t)p + k] = (uint16_t)(v > 0xffffu ? 0xffffu : v);
            }
        m.nint = x.nint.data();
        m.nint_all = x.nint_all.data();
    }
}

struct HalfBuf {
    std::vector<double> sh, dz;
    std::vector<uint32_t> id, ei;
    std::vector<float> ds, dzs, dl;
    explicit HalfBuf(uint32_t cap) : sh(cap), dz(cap), id(cap), ei(cap), ds(cap), dzs(cap), dl(cap) {}
    HalfSmem view() {
        HalfSmem h{id.data(), sh.data(), dz.data(), ds.data(), dzs.data(), ei.data()};
        h.dsl = dl.data();
        return h;
    }
};


constexpr uint32_t kCap = 1u << 16;

// Half-ray capacity the emulated formal solve traces with (the kernel's shared-memory
// ray buffers hold the longest half ray found by the sizing pass); tests lower it to
// reach the capacity-overflow status without a GPU.
uint32_t g_half_cap = kCap;

template <int MODE, bool UV = false>
LaneResult solve_any(const DevModel& m, const LaneCtx& c, const HalfSmem& bk, int nb, const HalfSmem& fw, int nf) {
    switch (m.approx) {
        case APPROX_ONELINE: return solve_lane<MODE, APPROX_ONELINE, UV>(m, m.sorted_line, c, bk, nb, fw, nf);
        case APPROX_CLOSELINES: return solve_lane<MODE, APPROX_CLOSELINES, UV>(m, m.sorted_line, c, bk, nb, fw, nf);
        default: return solve_lane<MODE, APPROX_NONE, UV>(m, m.sorted_line, c, bk, nb, fw, nf);
    }
}

template <int MODE>
LaneResultSC solve_any_sc0(const DevModel& m, const LaneCtx& c, const HalfSmem& bk, int nb, const HalfSmem& fw,
                           int nf) {
    switch (m.approx) {
        case APPROX_ONELINE: return solve_lane_sc0<MODE, APPROX_ONELINE>(m, m.sorted_line, c, bk, nb, fw, nf);
        case APPROX_CLOSELINES: return solve_lane_sc0<MODE, APPROX_CLOSELINES>(m, m.sorted_line, c, bk, nb, fw, nf);
        default: return solve_lane_sc0<MODE, APPROX_NONE>(m, m.sorted_line, c, bk, nb, fw, nf);
    }
}

LaneResult solve(const DevModel& m, int precision, const LaneCtx& c, const HalfSmem& bk, int nb, const HalfSmem& fw,
                 int nf) {
    return precision == MGR_PRECISION_SPLIT ? solve_any<MODE_SPLIT>(m, c, bk, nb, fw, nf)
                                            : solve_any<MODE_FP64>(m, c, bk, nb, fw, nf);
}

}  // namespace

// The kernel's two stages for every origin: per (rr, f) lane solves over the ray
// pairs [rr0, rr1), then J and the ALO summed in (rr, q) order as fo2_reduce_kernel does.
static int emu_fo2(const MgrModelDesc* d, int precision, uint32_t rr0, uint32_t rr1, double* J, double* lam) {
    EmuModel x;
    build_emu_model(d, x);
    const DevModel& m = x.m;
    const uint32_t P = m.P, L = m.L, F = m.F, R = m.hnrays, Q = m.Q;
    if (rr1 > R) rr1 = R;
    if (rr0 >= rr1) return MGR_ERR_ARGUMENT;
    int err = 0;  // status bits, as the kernel's status word
    const uint32_t cap = g_half_cap;
#pragma omp parallel
    {
        HalfBuf b(kCap), fbuf(kCap);
        HalfSmem bk = b.view(), fw = fbuf.view();
        std::vector<double> U((size_t)R * F), LD((size_t)R * F);
#pragma omp for schedule(dynamic, 16)
        for (long long oo = 0; oo < (long long)P; oo++) {
            const uint32_t o = (uint32_t)oo;
            bool ok = true;
            for (uint32_t rr = rr0; rr < rr1 && ok; rr++) {
                const int nb = trace_half_host(m, o, rr, cap, bk);
                const int nf = trace_half_host(m, o, m.antipod[rr], cap, fw);
                if (nb < 0 || nf < 0) {
                    const int bit = (nb == kTraceOverCapacity || nf == kTraceOverCapacity) ? ST_CAPACITY : ST_TRACE;
#pragma omp atomic
                    err |= bit;
                    ok = false;
                    break;
                }
                for (uint32_t f = 0; f < F; f++) {
                    const LaneResult r = solve(m, precision, lane_ctx(m, o, f), bk, nb, fw, nf);
                    U[(size_t)rr * F + f] = r.u;
                    LD[(size_t)rr * F + f] = r.solved ? r.Ldiag : 0.0;
                }
            }
            if (!ok) continue;
            for (uint32_t f = 0; f < F; f++) {
                double s = 0.0;
                for (uint32_t rr = rr0; rr < rr1; rr++) s += U[(size_t)rr * F + f] * 2.0 * ray_w(m, o, rr);
                J[(size_t)o * F + f] = s;
            }
            if (!lam) continue;
            for (uint32_t l = 0; l < L; l++) {
                std::vector<LambdaFactors> k(Q);
                for (uint32_t q = 0; q < Q; q++) {
                    const uint32_t f = m.lq2f[(size_t)l * Q + q];
                    if (f != 0xffffffffu && m.in_line[f]) k[q] = lambda_factors(m, m.sorted_line, o, f);
                }
                double s = 0.0;
                for (uint32_t rr = rr0; rr < rr1; rr++)
                    for (uint32_t q = 0; q < Q; q++) {
                        const uint32_t f = m.lq2f[(size_t)l * Q + q];
                        const double e = (f != 0xffffffffu && m.in_line[f])
                                             ? lambda_element(k[q], ray_w(m, o, rr), LD[(size_t)rr * F + f])
                                             : 0.0;
                        s += e;
                    }
                lam[(size_t)o * L + l] = s;
            }
        }
    }
    // the host's decoding of the kernel's status word: a trace failure first
    return (err & ST_TRACE) ? MGR_ERR_TRACE : (err & ST_CAPACITY) ? MGR_ERR_CAPACITY : MGR_OK;
}

// Half-ray capacity of the emulated formal solve; 0 restores the default.
extern "C" void mgr_emu_set_half_capacity(uint32_t cap) { g_half_cap = (cap == 0 || cap > kCap) ? kCap : cap; }

extern "C" int mgr_emu_formal_solve_fo2(const MgrModelDesc* d, int precision, double* J, double* lam) {
    return emu_fo2(d, precision, 0, 0xffffffffu, J, lam);
}

// Partial sums over the ray pairs [rr_begin, rr_end), as mgr_formal_solve_fo2_rays_device.
extern "C" int mgr_emu_formal_solve_fo2_rays(const MgrModelDesc* d, int precision, uint32_t rr_begin,
                                             uint32_t rr_end, double* J, double* lam) {
    return emu_fo2(d, precision, rr_begin, rr_end, J, lam);
}

// The uv solve (solve_lane<..., UV = true>): u and v [hnrays][P][F], and (may be NULL)
// the optical depths of the pairs on either side of the origin used by v.
extern "C" int mgr_emu_formal_solve_fo2_uv(const MgrModelDesc* d, int precision, double* u, double* v, double* dtm,
                                           double* dtp) {
    EmuModel x;
    build_emu_model(d, x);
    const DevModel& m = x.m;
    const uint32_t P = m.P, F = m.F, R = m.hnrays;
    int err = 0;
#pragma omp parallel
    {
        HalfBuf b(kCap), fbuf(kCap);
        HalfSmem bk = b.view(), fw = fbuf.view();
#pragma omp for schedule(dynamic, 16)
        for (long long oo = 0; oo < (long long)P; oo++) {
            const uint32_t o = (uint32_t)oo;
            for (uint32_t rr = 0; rr < R; rr++) {
                const int nb = trace_half_host(m, o, rr, kCap, bk);
                const int nf = trace_half_host(m, o, m.antipod[rr], kCap, fw);
                if (nb < 0 || nf < 0) {
#pragma omp atomic write
                    err = 1;
                    break;
                }
                for (uint32_t f = 0; f < F; f++) {
                    const LaneCtx c = lane_ctx(m, o, f);
                    const LaneResult r = precision == MGR_PRECISION_SPLIT
                                             ? solve_any<MODE_SPLIT, true>(m, c, bk, nb, fw, nf)
                                             : solve_any<MODE_FP64, true>(m, c, bk, nb, fw, nf);
                    const size_t i = ((size_t)rr * P + o) * F + f;
                    u[i] = r.u;
                    v[i] = r.v;
                    if (dtm) dtm[i] = r.dtm;
                    if (dtp) dtp[i] = r.dtp;
                }
            }
        }
    }
    return err ? MGR_ERR_TRACE : MGR_OK;
}

// Short characteristics: the kernel's per-lane code and the reduction order of
// sc0_reduce_kernel.  J [P][F], lam [P][L] (may be NULL).
extern "C" int mgr_emu_formal_solve_sc0(const MgrModelDesc* d, int precision, double* J, double* lam) {
    EmuModel x;
    build_emu_model(d, x);
    const DevModel& m = x.m;
    const uint32_t P = m.P, L = m.L, F = m.F, R = m.hnrays, Q = m.Q;
    int err = 0;
#pragma omp parallel
    {
        HalfBuf b(kCap), fbuf(kCap);
        HalfSmem bk = b.view(), fw = fbuf.view();
        std::vector<double> U((size_t)R * F), XF((size_t)R * F), XB((size_t)R * F);
#pragma omp for schedule(dynamic, 16)
        for (long long oo = 0; oo < (long long)P; oo++) {
            const uint32_t o = (uint32_t)oo;
            bool ok = true;
            for (uint32_t rr = 0; rr < R && ok; rr++) {
                const int nb = trace_half_host(m, o, rr, kCap, bk);
                const int nf = trace_half_host(m, o, m.antipod[rr], kCap, fw);
                if (nb < 0 || nf < 0) {
                    ok = false;
                    break;
                }
                for (uint32_t f = 0; f < F; f++) {
                    const LaneCtx c = lane_ctx(m, o, f);
                    const LaneResultSC r = precision == MGR_PRECISION_SPLIT ? solve_any_sc0<MODE_SPLIT>(m, c, bk, nb, fw, nf)
                                                                            : solve_any_sc0<MODE_FP64>(m, c, bk, nb, fw, nf);
                    U[(size_t)rr * F + f] = r.solved ? 0.5 * (r.If + r.Ib) : r.If;
                    XF[(size_t)rr * F + f] = r.Xf;
                    XB[(size_t)rr * F + f] = r.Xb;
                }
            }
            if (!ok) {
#pragma omp atomic write
                err = 1;
                continue;
            }
            for (uint32_t f = 0; f < F; f++) {
                double s = 0.0;
                for (uint32_t rr = 0; rr < R; rr++) s += (ray_w(m, o, rr) * 2.0) * U[(size_t)rr * F + f];
                J[(size_t)o * F + f] = s;
            }
            if (!lam) continue;
            for (uint32_t l = 0; l < L; l++) {
                double s = 0.0;
                for (uint32_t rr = 0; rr < R; rr++)
                    for (uint32_t q = 0; q < Q; q++) {
                        const uint32_t f = m.lq2f[(size_t)l * Q + q];
                        if (f == 0xffffffffu || !m.in_line[f]) continue;
                        const double xf = XF[(size_t)rr * F + f], xb = XB[(size_t)rr * F + f];
                        if (xf == 0.0 && xb == 0.0) continue;
                        const LambdaFactors k = lambda_factors(m, m.sorted_line, o, f);
                        s += lambda_element_sc0(k, ray_w(m, o, rr), xf);
                        s += lambda_element_sc0(k, ray_w(m, o, rr), xb);
                    }
                lam[(size_t)o * L + l] = s;
            }
        }
    }
    return err ? MGR_ERR_TRACE : MGR_OK;
}

// The old imager's per-ray code (image_lane with rest-frame traces), I [P][F].
extern "C" int mgr_emu_image(const MgrModelDesc* d, int precision, uint32_t rr, double* I) {
    EmuModel x;
    build_emu_model(d, x);
    const DevModel& m = x.m;
    const uint32_t P = m.P, F = m.F;
    int err = 0;
#pragma omp parallel
    {
        HalfBuf b(kCap), fbuf(kCap);
        HalfSmem bk = b.view(), fw = fbuf.view();
#pragma omp for schedule(dynamic, 16)
        for (long long oo = 0; oo < (long long)P; oo++) {
            const uint32_t o = (uint32_t)oo;
            const uint32_t ar = m.antipod[rr];
            const double shb = origin_shift(m, 1, o, rr);
            const double shf = origin_shift(m, 1, o, ar);
            bk.shift0 = shb;
            fw.shift0 = shf;
            set_dsh0(bk, shb);
            set_dsh0(fw, shf);
            bk.cshift = fw.cshift = shb;
            const int nb = trace_half_host(m, o, rr, kCap, bk, 1);
            const int nf = trace_half_host(m, o, m.antipod[rr], kCap, fw, 1);
            if (nb < 0 || nf < 0) {
#pragma omp atomic write
                err = 1;
                continue;
            }
            for (uint32_t f = 0; f < F; f++) {
                const LaneCtx c = lane_ctx(m, o, f);
                I[(size_t)o * F + f] =
                    precision == MGR_PRECISION_SPLIT
                        ? (m.approx == APPROX_NONE ? image_lane<MODE_SPLIT, APPROX_NONE>(m, m.sorted_line, c, bk, nb, fw, nf)
                                                   : image_lane<MODE_SPLIT, APPROX_CLOSELINES>(m, m.sorted_line, c, bk, nb, fw, nf))
                        : (m.approx == APPROX_NONE ? image_lane<MODE_FP64, APPROX_NONE>(m, m.sorted_line, c, bk, nb, fw, nf)
                                                   : image_lane<MODE_FP64, APPROX_CLOSELINES>(m, m.sorted_line, c, bk, nb, fw, nf));
            }
        }
    }
    return err ? MGR_ERR_TRACE : MGR_OK;
}

// The image_for_point rows (image_lane with ROWS) of point p's ray rr: n_tot and, when
// it fits capacity, S / dtau / u [n_tot][F] (zeros for a one-element ray).
extern "C" int mgr_emu_image_for_point(const MgrModelDesc* d, int precision, uint32_t rr, uint32_t p,
                                       uint32_t* n_tot, double* S, double* dtau, double* u, uint32_t capacity) {
    EmuModel x;
    build_emu_model(d, x);
    const DevModel& m = x.m;
    const uint32_t F = m.F;
    HalfBuf b(kCap), fbuf(kCap);
    HalfSmem bk = b.view(), fw = fbuf.view();
    const uint32_t ar = m.antipod[rr];
    const double shb = origin_shift(m, 1, p, rr);
    const double shf = origin_shift(m, 1, p, ar);
    bk.shift0 = shb;
    fw.shift0 = shf;
    set_dsh0(bk, shb);
    set_dsh0(fw, shf);
    bk.cshift = fw.cshift = shb;
    const int nb = trace_half_host(m, p, rr, kCap, bk, 1);
    const int nf = trace_half_host(m, p, ar, kCap, fw, 1);
    if (nb < 0 || nf < 0) return MGR_ERR_TRACE;
    uint32_t n = 1;
    for (int s = 0; s < nb; s++) n += m.nint_all[bk.eid[s]];
    for (int s = 0; s < nf; s++) n += m.nint_all[fw.eid[s]];
    *n_tot = n;
    if (n > capacity) return MGR_ERR_CAPACITY;
    const size_t NF = (size_t)n * F;
    std::fill(S, S + NF, 0.0);
    std::fill(dtau, dtau + NF, 0.0);
    std::fill(u, u + NF, 0.0);
    if (n <= 1) return MGR_OK;
    std::vector<double> FI(NF);
    const RowOut ro{S, dtau, u, FI.data(), F};
    for (uint32_t f = 0; f < F; f++) {
        const LaneCtx c = lane_ctx(m, p, f);
        if (precision == MGR_PRECISION_SPLIT) {
            if (m.approx == APPROX_NONE) image_lane<MODE_SPLIT, APPROX_NONE, false, true>(m, m.sorted_line, c, bk, nb, fw, nf, &ro);
            else image_lane<MODE_SPLIT, APPROX_CLOSELINES, false, true>(m, m.sorted_line, c, bk, nb, fw, nf, &ro);
        } else {
            if (m.approx == APPROX_NONE) image_lane<MODE_FP64, APPROX_NONE, false, true>(m, m.sorted_line, c, bk, nb, fw, nf, &ro);
            else image_lane<MODE_FP64, APPROX_CLOSELINES, false, true>(m, m.sorted_line, c, bk, nb, fw, nf, &ro);
        }
    }
    return MGR_OK;
}

// One lane's solve for (o, rr, f): out = {u, L_diag, solved}.
// The FP32-filtered walk against the exact one over every origin and every ray of a
// general-geometry model: counts rays, steps, steps the exact argmin took, and rays
// whose point sequence, edges or dZ bits differ.
extern "C" int mgr_emu_trace_filter_check(const MgrModelDesc* d, uint64_t* rays, uint64_t* steps,
                                          uint64_t* exact_steps, uint64_t* mismatches) {
    EmuModel x;
    build_emu_model(d, x);
    const DevModel& m = x.m;
    if (m.sph || !m.edge_hl) return MGR_ERR_UNSUPPORTED;
    HalfBuf b(kCap);
    std::vector<uint32_t> ids(kCap), eids(kCap);
    std::vector<double> dz(kCap);
    uint64_t nr = 0, ns = 0, ne = 0, bad = 0;
    for (uint32_t o = 0; o < m.P; o++)
        for (uint32_t r = 0; r < m.nrays; r++) {
            HalfSmem h = b.view();
            const int n0 = trace_half_host(m, o, r, kCap, h);
            const int n1 = trace_half_host_f32(m, o, r, kCap, ids.data(), eids.data(), dz.data(), ne);
            nr++;
            bool same = n0 == n1;
            for (int k = 0; same && k < n0; k++)
                same = ids[k] == b.id[k] && eids[k] == b.ei[k] && std::memcmp(&dz[k], &b.dz[k], 8) == 0;
            if (!same) bad++;
            if (n0 > 0) ns += (uint64_t)n0;
        }
    *rays = nr;
    *steps = ns;
    *exact_steps = ne;
    *mismatches = bad;
    return MGR_OK;
}

extern "C" int mgr_emu_lane(const MgrModelDesc* d, int precision, uint32_t o, uint32_t rr, uint32_t f,
                            double* out) {
    EmuModel x;
    build_emu_model(d, x);
    const DevModel& m = x.m;
    HalfBuf b(kCap), fbuf(kCap);
    HalfSmem bk = b.view(), fw = fbuf.view();
    const int nb = trace_half_host(m, o, rr, kCap, bk);
    const int nf = trace_half_host(m, o, m.antipod[rr], kCap, fw);
    if (nb < 0 || nf < 0) return MGR_ERR_TRACE;
    const LaneCtx c = lane_ctx(m, o, f);
    const LaneResult r = solve(m, precision, c, bk, nb, fw, nf);
    out[0] = r.u;
    out[1] = r.Ldiag;
    out[2] = r.solved ? 1.0 : 0.0;
    return MGR_OK;
}

// ---------------------------------------------------------------------------------
// Differentiable new imager: sequential pixel traces (bdy_point_closer, pixel_start,
// trace_image restated for one thread) and the lane code of image_s_kernel /
// image_adj_kernel.
// ---------------------------------------------------------------------------------
namespace {

unsigned long long host_dkey(double x) {
    unsigned long long b;
    std::memcpy(&b, &x, 8);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

uint32_t edge_target(const DevModel& m, size_t i) {
    long long bits;
    std::memcpy(&bits, &m.edge[i].w, 8);
    return (uint32_t)bits;
}

uint32_t bdy_point_closer_host(const DevModel& m, const double* org, const ImagePlane& ip, uint32_t crt) {
    const double4_32a pc = m.pos[crt];
    const double Rx = pc.x - org[0], Ry = pc.y - org[1], Rz = pc.z - org[2];
    const double Zc = dot3_rn(Rx, Ry, Rz, ip.d[0], ip.d[1], ip.d[2]);
    unsigned long long best = host_dkey(dot3_rn(Rx, Ry, Rz, Rx, Ry, Rz) - Zc * Zc);
    uint32_t besti = 0xffffffffu;
    const uint32_t nnb = m.n_nb[crt], cum = m.cum_nb[crt];
    for (uint32_t i = 0; i < nnb; i++) {
        const double4_32a e = m.edge[cum + i];
        const uint32_t n = edge_target(m, cum + i);
        if (m.p2b[n] == m.P) continue;
        const double Nx = e.x - org[0], Ny = e.y - org[1], Nz = e.z - org[2];
        const double Zn = dot3_rn(Nx, Ny, Nz, ip.d[0], ip.d[1], ip.d[2]);
        const unsigned long long k = host_dkey(dot3_rn(Nx, Ny, Nz, Nx, Ny, Nz) - Zn * Zn);
        if (k < best) {
            best = k;
            besti = i;
        }
    }
    return besti == 0xffffffffu ? crt : edge_target(m, cum + besti);
}

uint32_t pixel_start_host(const DevModel& m, const double* org, const ImagePlane& ip, double& Z) {
    uint32_t p = ip.start;
    for (uint32_t it = 0; it < m.P; it++) {
        const uint32_t q = bdy_point_closer_host(m, org, ip, p);
        if (q == p) break;
        p = q;
    }
    const double4_32a ps = m.pos[p];
    Z = dot3_rn(ps.x - org[0], ps.y - org[1], ps.z - org[2], ip.d[0], ip.d[1], ip.d[2]);
    return p;
}

int trace_image_host(const DevModel& m, const double* org, const ImagePlane& ip, uint32_t start, double Z,
                     uint32_t cap, HalfSmem h) {
    const double dx = ip.d[0], dy = ip.d[1], dz = ip.d[2];
    uint32_t crt = start;
    int count = 0;
    bool accessed = false;
    while (true) {
        const uint32_t nnb = m.n_nb[crt], cum = m.cum_nb[crt];
        const unsigned long long zkey = host_dkey(Z);
        unsigned long long best = ~0ull;
        uint32_t besti = 0xffffffffu;
        double bestZ = 0.0;
        for (uint32_t i = 0; i < nnb; i++) {
            const double4_32a e = m.edge[cum + i];
            const double Rx = e.x - org[0], Ry = e.y - org[1], Rz = e.z - org[2];
            const double Zn = dot3_rn(Rx, Ry, Rz, dx, dy, dz);
            if (host_dkey(Zn) > zkey) {
                const unsigned long long k = host_dkey(dot3_rn(Rx, Ry, Rz, Rx, Ry, Rz) - Zn * Zn);
                if (k < best) {
                    best = k;
                    besti = i;
                    bestZ = Zn;
                }
            }
        }
        if (besti == 0xffffffffu) break;
        if ((uint32_t)count >= cap) return -1;
        const uint32_t nxt = edge_target(m, cum + besti);
        const double dZl = bestZ - Z;
        Z = Z + dZl;
        h.ids[count] = nxt;
        h.eid[count] = cum + besti;
        h.dZ[count] = dZl;
        count++;
        if (m.p2b[nxt] != m.P) {
            const double4_32a pn = m.pos[nxt];
            const double side = dot3_rn(pn.x - ip.center[0], pn.y - ip.center[1], pn.z - ip.center[2], dx, dy, dz);
            if (!(side < 0.0)) break;
        } else {
            accessed = true;
        }
        crt = nxt;
    }
    if (count > 0 && !accessed) count = 0;
    for (int s = 0; s < count; s++) {
        const double4_32a v = m.vel[h.ids[s]];
        const double sh = 1.0 + dot3_rn(v.x, v.y, v.z, dx, dy, dz);
        h.shift[s] = sh;
        store_dsh(h, s, sh);
        h.dzs[s] = (float)h.dZ[s] * m.dz_scale;
    }
    return count;
}

// Pixel rays of the new imager: calls fn(px, start, bk, nb) for every pixel.
template <class Fn>
int for_each_pixel(const MgrModelDesc* d, const EmuModel& x, const double* raydir, uint32_t nx, uint32_t ny,
                   ImagePlane& ip, Fn fn) {
    const DevModel& m = x.m;
    std::vector<uint32_t> p2b(m.P);
    for (uint32_t p = 0; p < m.P; p++) p2b[p] = m.p2b[p];
    std::vector<double> hx, hy;
    std::string err;
    int rc = image_plane_compute(d->position, p2b.data(), m.P, m.B, raydir, nx, ny, ip, hx, hy, err);
    if (rc != MGR_OK) return rc;
    HalfBuf b(kCap);
    HalfSmem bk = b.view();
    for (uint32_t px = 0; px < nx * ny; px++) {
        double org[3];
        if (ip.tilted) {
            org[0] = hx[px] * ip.ix + hy[px] * ip.jx + ip.scp[0];
            org[1] = hx[px] * ip.iy + hy[px] * ip.jy + ip.scp[1];
            org[2] = hy[px] * ip.jz + ip.scp[2];
        } else {
            org[0] = hx[px] + ip.scp[0];
            org[1] = hy[px] + ip.scp[1];
            org[2] = 0.0 + ip.scp[2];
        }
        double Z;
        const uint32_t start = pixel_start_host(m, org, ip, Z);
        const double4_32a vs = m.vel[start];
        const double sh0 = 1.0 + dot3_rn(vs.x, vs.y, vs.z, ip.d[0], ip.d[1], ip.d[2]);
        bk.shift0 = bk.cshift = sh0;
        const int nb = trace_image_host(m, org, ip, start, Z, kCap, bk);
        if (nb < 0) return MGR_ERR_CAPACITY;
        fn(px, start, bk, nb);
    }
    return MGR_OK;
}

}  // namespace

// Smooth new image I [nx*ny][F] (image_s_kernel's lane code).
extern "C" int mgr_emu_image_new_smooth(const MgrModelDesc* d, const double* raydir, uint32_t nx, uint32_t ny,
                                        double* I) {
    EmuModel x;
    build_emu_model(d, x);
    const DevModel& m = x.m;
    ImagePlane ip{};
    return for_each_pixel(d, x, raydir, nx, ny, ip, [&](uint32_t px, uint32_t start, const HalfSmem& bk, int nb) {
        for (uint32_t f = 0; f < m.F; f++) {
            uint32_t np;
            const double nu = m.nu[(size_t)start * m.F + f];
            I[(size_t)px * m.F + f] = m.approx == APPROX_NONE
                                          ? image_lane_s<APPROX_NONE>(m, m.sorted_line, start, nu, bk, nb, nullptr, &np)
                                          : image_lane_s<APPROX_CLOSELINES>(m, m.sorted_line, start, nu, bk, nb, nullptr, &np);
        }
    });
}

// Adjoint of mgr_emu_image_new_smooth (image_adj_kernel's lane code): adds the
// derivatives of sum(gI * I) into g_em, g_op, g_iw, g_Sp [P][L] and g_vel [P][3].
extern "C" int mgr_emu_image_new_adjoint(const MgrModelDesc* d, const double* raydir, uint32_t nx, uint32_t ny,
                                         const double* gI, double* g_em, double* g_op, double* g_iw, double* g_Sp,
                                         double* g_vel) {
    EmuModel x;
    build_emu_model(d, x);
    const DevModel& m = x.m;
    ImagePlane ip{};
    std::vector<double> scratch;
    int fail = 0;
    int rc = for_each_pixel(d, x, raydir, nx, ny, ip, [&](uint32_t px, uint32_t start, const HalfSmem& bk, int nb) {
        size_t pairs = 1;
        for (int s = 0; s < nb; s++) pairs += m.nint_all[bk.eid[s]];
        if (scratch.size() < 3 * pairs) scratch.resize(3 * pairs);
        const LaneScratch scr{scratch.data(), 1, (uint32_t)pairs};
        const AdjAcc acc{AdjGrads{g_em, g_op, g_iw, g_Sp, g_vel, {ip.d[0], ip.d[1], ip.d[2]}}, m.L};
        for (uint32_t f = 0; f < m.F; f++) {
            const double nu = m.nu[(size_t)start * m.F + f];
            const double g = gI[(size_t)px * m.F + f];
            const bool ok = m.approx == APPROX_NONE
                                ? image_lane_adj<APPROX_NONE>(m, m.sorted_line, start, nu, bk, nb, g, scr, acc)
                                : image_lane_adj<APPROX_CLOSELINES>(m, m.sorted_line, start, nu, bk, nb, g, scr, acc);
            if (!ok) fail = 1;
        }
    });
    if (rc == MGR_OK && fail) rc = MGR_ERR_CAPACITY;
    return rc;
}

// ---- differentiable formal solve (fo2_s_kernel / fo2_adj_kernel lane code) ----

namespace {

// Runs fn(o, rr, bk, nb, fw, nf) for every origin and ray pair (host traces).
template <typename Fn>
int for_each_ray_pair(const DevModel& m, Fn fn) {
    HalfBuf b(kCap), fbuf(kCap);
    HalfSmem bk = b.view(), fw = fbuf.view();
    for (uint32_t o = 0; o < m.P; o++)
        for (uint32_t rr = 0; rr < m.hnrays; rr++) {
            const int nb = trace_half_host(m, o, rr, kCap, bk);
            const int nf = trace_half_host(m, o, m.antipod[rr], kCap, fw);
            if (nb < 0 || nf < 0) return (nb == kTraceOverCapacity || nf == kTraceOverCapacity) ? MGR_ERR_CAPACITY
                                                                                              : MGR_ERR_TRACE;
            fn(o, rr, bk, nb, fw, nf);
        }
    return MGR_OK;
}

}  // namespace

// Smooth J [P][F] (every origin), summed over ray pairs in order.
extern "C" int mgr_emu_fo2_smooth(const MgrModelDesc* d, double* J) {
    EmuModel x;
    build_emu_model(d, x);
    const DevModel& m = x.m;
    std::fill(J, J + (size_t)m.P * m.F, 0.0);
    return for_each_ray_pair(m, [&](uint32_t o, uint32_t rr, const HalfSmem& bk, int nb, const HalfSmem& fw, int nf) {
        const double wt = 2.0 * ray_w(m, o, rr);
        for (uint32_t l = 0; l < m.L; l++)
            for (uint32_t q = 0; q < m.Q; q++) {
                const uint32_t f = m.lq2f[(size_t)l * m.Q + q];
                const double nu = m.nu[(size_t)o * m.F + f];
                const LaneS r = m.approx == APPROX_NONE
                                    ? solve_lane_s<APPROX_NONE>(m, m.sorted_line, o, nu, l, bk, nb, fw, nf, nullptr)
                                    : solve_lane_s<APPROX_CLOSELINES>(m, m.sorted_line, o, nu, l, bk, nb, fw, nf,
                                                                      nullptr);
                J[(size_t)o * m.F + f] += r.u * wt;
            }
    });
}

// Adjoint of mgr_emu_fo2_smooth for d(loss)/d(J) = gJ: adds into g_em, g_op, g_iw, g_Sp
// [P][L], g_vel [P][3] and g_nu [P][F].
extern "C" int mgr_emu_fo2_adjoint(const MgrModelDesc* d, const double* gJ, double* g_em, double* g_op, double* g_iw,
                                   double* g_Sp, double* g_vel, double* g_nu) {
    EmuModel x;
    build_emu_model(d, x);
    const DevModel& m = x.m;
    std::vector<double> scratch;
    int fail = 0;
    int rc = for_each_ray_pair(m, [&](uint32_t o, uint32_t rr, const HalfSmem& bk, int nb, const HalfSmem& fw,
                                      int nf) {
        const uint32_t ar = m.antipod[rr];
        size_t pairs = 2;
        for (int s = 0; s < nb; s++) pairs += m.nint_all[bk.eid[s]];
        for (int s = 0; s < nf; s++) pairs += m.nint_all[fw.eid[s]];
        if (scratch.size() < 4 * pairs) scratch.resize(4 * pairs);
        const Fo2Scratch scr{scratch.data(), 1, (uint32_t)pairs};
        const double* db = ray_dir(m, o, rr);
        const double* df = ray_dir(m, o, ar);
        const AdjAcc acc_b{AdjGrads{g_em, g_op, g_iw, g_Sp, g_vel, {db[0], db[1], db[2]}}, m.L};
        const AdjAcc acc_f{AdjGrads{g_em, g_op, g_iw, g_Sp, g_vel, {df[0], df[1], df[2]}}, m.L};
        const double wt = 2.0 * ray_w(m, o, rr);
        for (uint32_t l = 0; l < m.L; l++)
            for (uint32_t q = 0; q < m.Q; q++) {
                const uint32_t f = m.lq2f[(size_t)l * m.Q + q];
                const double gu = gJ[(size_t)o * m.F + f] * wt;
                if (gu == 0.0) continue;
                const double nu = m.nu[(size_t)o * m.F + f];
                double gvb = 0.0, gvf = 0.0, gn = 0.0;
                const bool ok =
                    m.approx == APPROX_NONE
                        ? solve_lane_s_adj<APPROX_NONE>(m, m.sorted_line, o, nu, l, bk, nb, fw, nf, gu, scr, acc_b,
                                                        acc_f, gvb, gvf, gn)
                        : solve_lane_s_adj<APPROX_CLOSELINES>(m, m.sorted_line, o, nu, l, bk, nb, fw, nf, gu, scr,
                                                              acc_b, acc_f, gvb, gvf, gn);
                if (!ok) fail = 1;
                for (int k = 0; k < 3; k++) g_vel[3 * (size_t)o + k] += gvb * db[k] + gvf * df[k];
                g_nu[(size_t)o * m.F + f] += gn;
            }
    });
    if (rc == MGR_OK && fail) rc = MGR_ERR_CAPACITY;
    return rc;
}

// The band elements of the non-local ALO (fo2_alo_kernel's layout): alo_off / alo_nr
// [P][L][hnrays][2 n_off_diag], summed over each line's quadrature points in order.
extern "C" int mgr_emu_fo2_alo(const MgrModelDesc* d, uint32_t n_off_diag, double* alo_off, uint32_t* alo_nr) {
    if (n_off_diag == 0 || n_off_diag > kMaxOffDiag) return MGR_ERR_ARGUMENT;
    EmuModel x;
    build_emu_model(d, x);
    DevModel& m = x.m;
    m.n_off_diag = n_off_diag;
    const uint32_t K = n_off_diag;
    const size_t n = (size_t)m.P * m.L * m.hnrays * 2 * K;
    std::fill(alo_off, alo_off + n, 0.0);
    const size_t per_o = (size_t)m.L * m.hnrays * 2 * K;
    for (size_t t = 0; t < n; t++) alo_nr[t] = (uint32_t)(t / per_o);  // absent elements: the origin itself
    return for_each_ray_pair(m, [&](uint32_t o, uint32_t rr, const HalfSmem& bk, int nb, const HalfSmem& fw, int nf) {
        for (uint32_t f = 0; f < m.F; f++) {
            const LaneCtx c = lane_ctx(m, o, f);
            BandOut<kMaxOffDiag> bo;
            bo.K = K;
            bo.w_rr = ray_w(m, o, rr);
            LaneResult r;
            switch (m.approx) {
                case APPROX_ONELINE:
                    r = solve_lane<MODE_FP64, APPROX_ONELINE, false, kMaxOffDiag>(m, m.sorted_line, c, bk, nb, fw, nf,
                                                                                  &bo);
                    break;
                case APPROX_CLOSELINES:
                    r = solve_lane<MODE_FP64, APPROX_CLOSELINES, false, kMaxOffDiag>(m, m.sorted_line, c, bk, nb, fw,
                                                                                     nf, &bo);
                    break;
                default:
                    r = solve_lane<MODE_FP64, APPROX_NONE, false, kMaxOffDiag>(m, m.sorted_line, c, bk, nb, fw, nf,
                                                                               &bo);
            }
            if (!r.solved || !m.in_line[f]) continue;
            const uint32_t lid = m.corr_line[f];
            for (uint32_t s = 0; s < 2 * K; s++) {
                const size_t a = (((size_t)o * m.L + lid) * m.hnrays + rr) * 2 * K + s;
                alo_off[a] += bo.val[s];
                alo_nr[a] = bo.nr[s];
            }
        }
    });
}
