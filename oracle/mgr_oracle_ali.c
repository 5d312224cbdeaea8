/*
 * Oracle for the ALI level-population loop -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates Model::compute_level_populations (src/model/model.cpp:654-747) with the
 * Default and Adaptive Ng criteria (:584-645), Model::compute_Jeff (:514-545) and the
 * LineProducingSpecies steps it drives (src/model/lines/lineProducingSpecies/
 * lineProducingSpecies.tpp): statistical equilibrium (:377-581), negative-population
 * correction (:711-802), convergence checks (:128-205), general-order Ng acceleration
 * and its trial form (:266-372), emissivity / opacity (:23-44, lines.tpp:29-40).
 * Populations and the rate equations are long double as in the reference.
 *
 * Third-party boundary: the reference solves the global sparse rate system with
 * Eigen's SparseLU (COLAMD ordering) and the Ng coefficients with Eigen's
 * colPivHouseholderQr (Eigen is an absent submodule).  With n_off_diag = 0 the rate
 * system is block diagonal, one nlev x nlev block per point, so this oracle solves
 * each block by Gaussian elimination with partial pivoting and the Ng system by a
 * Householder QR with column pivoting, both in long double.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mgr_oracle.h"

static const double HH_ALI = 6.62607004E-34;
static const double KB_ALI = 1.38064852E-23;
#define HH_OVER_FOUR_PI_ALI (HH_ALI / (4.0 * 3.14159265358979323846)) /* constants.hpp:17,40 */

typedef long double ld;

/* ------------------------------------------------------------------ */
/* Jeff (model.cpp:514-545), n_off_diag = 0: one ALO element per (p, k) */
/* ------------------------------------------------------------------ */
static void jeff_species(const OrcModel* m, const OrcSpecies* s, const double* J, const double* lam, const ld* pop,
                         double* Jlin, double* Jeff, double* Jdif) {
    const uint32_t P = m->npoints, L = m->nlines, Q = m->nquads, F = m->nfreqs;
    /* nr_line[p][k][z]: the frequency of (line, quadrature point z); the same for every p */
    uint32_t* nr_line = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)s->nrad * Q);
    for (uint32_t g = 0; g < F; g++) {
        const uint32_t lid = m->corr_line[g];
        if (lid >= s->line_offset && lid < s->line_offset + s->nrad)
            nr_line[(size_t)(lid - s->line_offset) * Q + m->corr_z[g]] = g;
    }
    for (uint32_t p = 0; p < P; p++)
        for (uint32_t k = 0; k < s->nrad; k++) {
            const uint32_t lid = s->line_offset + k;
            double jl = 0.0;
            for (uint32_t z = 0; z < Q; z++) {
                const uint32_t f = nr_line[(size_t)k * Q + z];
                jl += m->quad_weights[(size_t)m->corr_lspec[f] * Q + z] * J[(size_t)p * F + f];
            }
            const ld popI = pop[(size_t)p * s->nlev + s->irad[k]];
            double diff = 0.0;
            diff += (double)((ld)lam[(size_t)p * L + lid] * popI);
            Jlin[(size_t)p * s->nrad + k] = jl;
            Jeff[(size_t)p * s->nrad + k] = jl - HH_OVER_FOUR_PI_ALI * diff;
            Jdif[(size_t)p * s->nrad + k] = HH_OVER_FOUR_PI_ALI * diff;
        }
    free(nr_line);
}

/* Jeff with the non-local ALO (model.cpp:514-545): diff sums Ls * population of the
 * emitting point's upper level over the (p, line) list, in list order. */
static void jeff_species_alo(const OrcModel* m, const OrcSpecies* s, const double* J, uint32_t cap,
                             const uint32_t* alo_n, const uint32_t* alo_nr, const double* alo_ls, const ld* pop,
                             double* Jlin, double* Jeff, double* Jdif) {
    const uint32_t P = m->npoints, L = m->nlines, Q = m->nquads, F = m->nfreqs;
    uint32_t* nr_line = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)s->nrad * Q);
    for (uint32_t g = 0; g < F; g++) {
        const uint32_t lid = m->corr_line[g];
        if (lid >= s->line_offset && lid < s->line_offset + s->nrad)
            nr_line[(size_t)(lid - s->line_offset) * Q + m->corr_z[g]] = g;
    }
    for (uint32_t p = 0; p < P; p++)
        for (uint32_t k = 0; k < s->nrad; k++) {
            const uint32_t lid = s->line_offset + k;
            const size_t key   = (size_t)p * L + lid;
            double jl          = 0.0;
            for (uint32_t z = 0; z < Q; z++) {
                const uint32_t f = nr_line[(size_t)k * Q + z];
                jl += m->quad_weights[(size_t)m->corr_lspec[f] * Q + z] * J[(size_t)p * F + f];
            }
            double diff = 0.0;
            for (uint32_t i = 0; i < alo_n[key]; i++)
                diff = (double)((ld)diff + (ld)alo_ls[key * cap + i] *
                                               pop[(size_t)alo_nr[key * cap + i] * s->nlev + s->irad[k]]);
            Jlin[(size_t)p * s->nrad + k] = jl;
            Jeff[(size_t)p * s->nrad + k] = jl - HH_OVER_FOUR_PI_ALI * diff;
            Jdif[(size_t)p * s->nrad + k] = HH_OVER_FOUR_PI_ALI * diff;
        }
    free(nr_line);
}

int orc_compute_jeff(const OrcModel* m, uint32_t nlspecs, const OrcSpecies* sp, const double* J, const double* lam,
                     double* const* pops, double* const* Jlin, double* const* Jeff, double* const* Jdif) {
    for (uint32_t l = 0; l < nlspecs; l++) {
        const OrcSpecies* s = &sp[l];
        const size_t n = (size_t)m->npoints * s->nlev;
        ld* pl = (ld*)malloc(sizeof(ld) * n);
        if (!pl) return -1;
        for (size_t i = 0; i < n; i++) pl[i] = pops[l][i];
        jeff_species(m, s, J, lam, pl, Jlin[l], Jeff[l], Jdif[l]);
        free(pl);
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Collision coefficients (collisionPartner.tpp:6-42, interpolation.hpp:10-33) */
/* ------------------------------------------------------------------ */
static uint32_t search_table(const double* x, uint32_t n, double value) {
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

static void collision_rates(const OrcColPar* c, double T, double* Cd, double* Ce) {
    const uint32_t t = search_table(c->tmp, c->ntmp, T);
    if (t == 0 || t == c->ntmp - 1) {
        for (uint32_t k = 0; k < c->ncol; k++) {
            Ce[k] = c->Ce[(size_t)t * c->ncol + k];
            Cd[k] = c->Cd[(size_t)t * c->ncol + k];
        }
        return;
    }
    const double step = (T - c->tmp[t - 1]) / (c->tmp[t] - c->tmp[t - 1]);
    for (uint32_t k = 0; k < c->ncol; k++) {
        const double ce0 = c->Ce[(size_t)(t - 1) * c->ncol + k], ce1 = c->Ce[(size_t)t * c->ncol + k];
        const double cd0 = c->Cd[(size_t)(t - 1) * c->ncol + k], cd1 = c->Cd[(size_t)t * c->ncol + k];
        Ce[k] = ce0 + (ce1 - ce0) * step;
        Cd[k] = cd0 + (cd1 - cd0) * step;
    }
}

static double partner_abundance(const OrcColPar* c, double T, double abn) {
    if (c->ortho_para != 0) {
        const double frac_H2_para = 1.0 / (1.0 + 9.0 * (double)expf((float)(-170.5 / T)));
        if (c->ortho_para == 1) abn *= (1.0 - frac_H2_para);
        if (c->ortho_para == 2) abn *= frac_H2_para;
    }
    return abn;
}

/* get_opacity (lineProducingSpecies.tpp:36-44) on long double populations. */
static double opacity_of(const OrcSpecies* s, const ld* pp, uint32_t k, double min_line_opacity) {
    const ld v = (ld)(s->frequency[k] * HH_OVER_FOUR_PI_ALI) *
                 (pp[s->jrad[k]] * (ld)s->Ba[k] - pp[s->irad[k]] * (ld)s->Bs[k]);
    return (double)(v > (ld)min_line_opacity ? v : (ld)min_line_opacity);
}

static double emissivity_of(const OrcSpecies* s, const ld* pp, uint32_t k, double min_line_emissivity) {
    const ld v = (ld)(s->frequency[k] * HH_OVER_FOUR_PI_ALI * s->A[k]) * pp[s->irad[k]];
    return (double)(v > (ld)min_line_emissivity ? v : (ld)min_line_emissivity);
}

/* ------------------------------------------------------------------ */
/* Statistical equilibrium of one point (lineProducingSpecies.tpp:377-581) */
/* ------------------------------------------------------------------ */
static int solve_dense(ld* M, ld* y, uint32_t n) {
    for (uint32_t c = 0; c < n; c++) {
        uint32_t piv = c;
        ld best = fabsl(M[(size_t)c * n + c]);
        for (uint32_t r = c + 1; r < n; r++) {
            const ld v = fabsl(M[(size_t)r * n + c]);
            if (v > best) {
                best = v;
                piv = r;
            }
        }
        if (best == 0.0L) return -1;
        if (piv != c) {
            for (uint32_t j = 0; j < n; j++) {
                const ld t = M[(size_t)c * n + j];
                M[(size_t)c * n + j] = M[(size_t)piv * n + j];
                M[(size_t)piv * n + j] = t;
            }
            const ld t = y[c];
            y[c] = y[piv];
            y[piv] = t;
        }
        for (uint32_t r = c + 1; r < n; r++) {
            const ld f = M[(size_t)r * n + c] / M[(size_t)c * n + c];
            if (f == 0.0L) continue;
            for (uint32_t j = c; j < n; j++) M[(size_t)r * n + j] -= f * M[(size_t)c * n + j];
            y[r] -= f * y[c];
        }
    }
    for (uint32_t c = n; c-- > 0;) {
        ld s = y[c];
        for (uint32_t j = c + 1; j < n; j++) s -= M[(size_t)c * n + j] * y[j];
        y[c] = s / M[(size_t)c * n + c];
    }
    return 0;
}

/* Row-major rate block M (rows = equations) for point p, as the reference's
 * triplets (row, column, value) with the last level's row replaced by the
 * normalisation.  Ls = ALO diagonal of (p, line), Jeff [nrad]. */
static void rate_block(const OrcSpecies* s, const ld* pp, const double* Jeff, const double* Ls, double T,
                       const double* abundance_p, double min_line_opacity, ld* M) {
    const uint32_t n = s->nlev, last = n - 1;
    memset(M, 0, sizeof(ld) * n * n);
#define ADD(r, c, v) M[(size_t)(r) * n + (c)] += (v)
    for (uint32_t k = 0; k < s->nrad; k++) {
        const ld v_IJ = (ld)s->A[k] + (ld)s->Bs[k] * (ld)Jeff[k];
        const ld v_JI = (ld)s->Ba[k] * (ld)Jeff[k];
        const uint32_t I = s->irad[k], J = s->jrad[k];
        if (J != last) {
            ADD(J, I, +v_IJ);
            ADD(J, J, -v_JI);
        }
        if (I != last) {
            ADD(I, J, +v_JI);
            ADD(I, I, -v_IJ);
        }
    }
    for (uint32_t k = 0; k < s->nrad; k++) {
        const double freq = s->frequency[k];
        const ld v_IJ = -(ld)Ls[k] * (ld)opacity_of(s, pp, k, min_line_opacity) / (ld)freq;
        const uint32_t I = s->irad[k], J = s->jrad[k];
        if (J != last) ADD(J, I, +v_IJ);
        if (I != last) ADD(I, I, -v_IJ);
    }
    for (uint32_t c = 0; c < s->ncolpar; c++) {
        const OrcColPar* cp = &s->colpar[c];
        const double abn = partner_abundance(cp, T, abundance_p[cp->num_col_partner]);
        double Cd[64], Ce[64];
        double* cd = cp->ncol <= 64 ? Cd : (double*)malloc(sizeof(double) * cp->ncol);
        double* ce = cp->ncol <= 64 ? Ce : (double*)malloc(sizeof(double) * cp->ncol);
        collision_rates(cp, T, cd, ce);
        for (uint32_t k = 0; k < cp->ncol; k++) {
            const ld v_IJ = (ld)cd[k] * (ld)abn;
            const ld v_JI = (ld)ce[k] * (ld)abn;
            const uint32_t I = cp->icol[k], J = cp->jcol[k];
            if (J != last) {
                ADD(J, I, +v_IJ);
                ADD(J, J, -v_JI);
            }
            if (I != last) {
                ADD(I, J, +v_JI);
                ADD(I, I, -v_IJ);
            }
        }
        if (cd != Cd) free(cd);
        if (ce != Ce) free(ce);
    }
    for (uint32_t i = 0; i < n; i++) ADD(last, i, 1.0L);
#undef ADD
}

/* The global rate system of update_using_statistical_equilibrium
 * (lineProducingSpecies.tpp:377-581) for every point at once: per point p its
 * radiative triplets, the ALO triplets of each element (nr, Ls) of its (p, line) lists
 * (row (p, lower) gains v at column (nr, upper); row (nr, upper) loses v on its
 * diagonal, v = -Ls opacity(p, k) / frequency), the collisional triplets and the
 * normalisation row, in that order, into a dense long-double matrix of order P nlev
 * solved by Gaussian elimination with partial pivoting (the reference: Eigen
 * SparseLU).  pp: populations before the solve; out: the solution. */
static int stateq_global(const OrcSpecies* s, uint32_t P, uint32_t L, const ld* pp, const double* Jeff, uint32_t cap,
                         const uint32_t* alo_n, const uint32_t* alo_nr, const double* alo_ls, const double* T,
                         const double* abundance, uint32_t nspecs, const ld* tot, double min_line_opacity, ld* out) {
    const uint32_t n = s->nlev, last = n - 1;
    const size_t N = (size_t)P * n;
    ld* M = (ld*)calloc(N * N, sizeof(ld));
    ld* y = (ld*)calloc(N, sizeof(ld));
    if (!M || !y) {
        free(M);
        free(y);
        return -1;
    }
#define GADD(r, c, v) M[(size_t)(r) * N + (c)] += (v)
    for (uint32_t p = 0; p < P; p++) {
        const size_t o = (size_t)p * n;
        for (uint32_t k = 0; k < s->nrad; k++) {
            const ld Je = (ld)Jeff[(size_t)p * s->nrad + k];
            const ld v_IJ = (ld)s->A[k] + (ld)s->Bs[k] * Je;
            const ld v_JI = (ld)s->Ba[k] * Je;
            const size_t I = o + s->irad[k], J = o + s->jrad[k];
            if (s->jrad[k] != last) {
                GADD(J, I, +v_IJ);
                GADD(J, J, -v_JI);
            }
            if (s->irad[k] != last) {
                GADD(I, J, +v_JI);
                GADD(I, I, -v_IJ);
            }
        }
        for (uint32_t k = 0; k < s->nrad; k++) {
            const size_t key = (size_t)p * L + s->line_offset + k;
            const double opac = opacity_of(s, pp + o, k, min_line_opacity);
            for (uint32_t i = 0; i < alo_n[key]; i++) {
                const ld v_IJ = -(ld)alo_ls[key * cap + i] * (ld)opac / (ld)s->frequency[k];
                const size_t I = (size_t)alo_nr[key * cap + i] * n + s->irad[k], J = o + s->jrad[k];
                if (s->jrad[k] != last) GADD(J, I, +v_IJ);
                if (s->irad[k] != last) GADD(I, I, -v_IJ);
            }
        }
        for (uint32_t c = 0; c < s->ncolpar; c++) {
            const OrcColPar* cp = &s->colpar[c];
            const double abn = partner_abundance(cp, T[p], abundance[(size_t)p * nspecs + cp->num_col_partner]);
            double* cd = (double*)malloc(sizeof(double) * cp->ncol);
            double* ce = (double*)malloc(sizeof(double) * cp->ncol);
            collision_rates(cp, T[p], cd, ce);
            for (uint32_t k = 0; k < cp->ncol; k++) {
                const ld v_IJ = (ld)cd[k] * (ld)abn;
                const ld v_JI = (ld)ce[k] * (ld)abn;
                const size_t I = o + cp->icol[k], J = o + cp->jcol[k];
                if (cp->jcol[k] != last) {
                    GADD(J, I, +v_IJ);
                    GADD(J, J, -v_JI);
                }
                if (cp->icol[k] != last) {
                    GADD(I, J, +v_JI);
                    GADD(I, I, -v_IJ);
                }
            }
            free(cd);
            free(ce);
        }
        for (uint32_t i = 0; i < n; i++) GADD(o + last, o + i, 1.0L);
        y[o + last] = tot[p];
    }
#undef GADD
    const int rc = solve_dense(M, y, (uint32_t)N);
    for (size_t i = 0; i < N; i++) out[i] = y[i];
    free(M);
    free(y);
    return rc;
}

int orc_stateq(const OrcSpecies* s, uint32_t P, const double* abundance, uint32_t nspecs, const double* temperature,
               const double* Jeff, const double* Ls, const double* pop_in, double min_line_opacity, double* pop_out) {
    const uint32_t n = s->nlev;
    ld* M = (ld*)malloc(sizeof(ld) * n * n);
    ld* y = (ld*)malloc(sizeof(ld) * n);
    ld* pp = (ld*)malloc(sizeof(ld) * n);
    int rc = 0;
    for (uint32_t p = 0; p < P && rc == 0; p++) {
        for (uint32_t i = 0; i < n; i++) pp[i] = pop_in[(size_t)p * n + i];
        rate_block(s, pp, Jeff + (size_t)p * s->nrad, Ls + (size_t)p * s->nrad, temperature[p],
                   abundance + (size_t)p * nspecs, min_line_opacity, M);
        for (uint32_t i = 0; i < n; i++) y[i] = 0.0L;
        y[n - 1] = abundance[(size_t)p * nspecs + s->num];
        if (solve_dense(M, y, n) != 0) rc = -1;
        for (uint32_t i = 0; i < n; i++) pop_out[(size_t)p * n + i] = (double)y[i];
    }
    free(M);
    free(y);
    free(pp);
    return rc;
}

/* ------------------------------------------------------------------ */
/* ALI state and steps                                                  */
/* ------------------------------------------------------------------ */
typedef struct {
    const OrcSpecies* s;
    size_t n;            /* P * nlev */
    ld* pop;             /* population */
    ld* prev1;           /* population_prev1 */
    ld* tot;             /* population_tot [P] */
    ld** hist;           /* populations list */
    uint32_t nhist, cap_hist;
    ld** res;            /* residuals list */
    uint32_t nres, cap_res;
    ld* trial;           /* trial_population */
    ld* trial_prev;      /* trial_population_prev */
    double fnc, rcm, rcmax;
    double* Jlin;
    double* Jeff;
    double* Jdif;
} Lsp;

static int push(ld*** list, uint32_t* n, uint32_t* cap, const ld* v, size_t len) {
    if (*n == *cap) {
        const uint32_t nc = *cap ? 2 * *cap : 8;
        ld** q = (ld**)realloc(*list, sizeof(ld*) * nc);
        if (!q) return -1;
        *list = q;
        *cap = nc;
    }
    ld* c = (ld*)malloc(sizeof(ld) * len);
    if (!c) return -1;
    memcpy(c, v, sizeof(ld) * len);
    (*list)[(*n)++] = c;
    return 0;
}

static void erase_front(ld** list, uint32_t* n, uint32_t keep) {
    /* keep the last `keep` entries */
    if (*n <= keep) return;
    const uint32_t drop = *n - keep;
    for (uint32_t i = 0; i < drop; i++) free(list[i]);
    memmove(list, list + drop, sizeof(ld*) * keep);
    *n = keep;
}

static void residual_push(Lsp* x) {
    /* residuals.push_back(population - populations.back()); populations.push_back(population) */
    ld* r = (ld*)malloc(sizeof(ld) * x->n);
    const ld* b = x->hist[x->nhist - 1];
    for (size_t i = 0; i < x->n; i++) r[i] = x->pop[i] - b[i];
    if (x->nres == x->cap_res) {
        x->cap_res = x->cap_res ? 2 * x->cap_res : 8;
        x->res = (ld**)realloc(x->res, sizeof(ld*) * x->cap_res);
    }
    x->res[x->nres++] = r;
    push(&x->hist, &x->nhist, &x->cap_hist, x->pop, x->n);
}

/* check_for_convergence (lineProducingSpecies.tpp:128-165) */
static void check_convergence(Lsp* x, uint32_t P, const OrcAliParams* prm) {
    const uint32_t nlev = x->s->nlev;
    const double weight = 1.0 / (P * nlev);
    double fnc = 0.0, rcm = 0.0, rcmax = 0.0;
    for (uint32_t p = 0; p < P; p++)
        for (uint32_t i = 0; i < nlev; i++) {
            const size_t ind = (size_t)p * nlev + i;
            if (x->pop[ind] > (ld)prm->min_rel_pop_for_convergence * x->tot[p]) {
                const double rc = (double)(2.0L * fabsl((x->pop[ind] - x->prev1[ind]) / (x->pop[ind] + x->prev1[ind])));
                if (rc > prm->pop_prec) fnc += weight;
                rcm += weight * rc;
                if (rc > rcmax) rcmax = rc;
            }
        }
    x->fnc = fnc;
    x->rcm = rcm;
    x->rcmax = rcmax;
}

static void check_convergence_trial(Lsp* x, uint32_t P, const OrcAliParams* prm) {
    const uint32_t nlev = x->s->nlev;
    const double weight = 1.0 / (P * nlev);
    double fnc = 0.0, rcm = 0.0, rcmax = 0.0;
    for (size_t ind = 0; ind < x->n; ind++) {
        const double rc =
            (double)(2.0L * fabsl((x->trial[ind] - x->trial_prev[ind]) / (x->trial[ind] + x->trial_prev[ind])));
        if (rc > prm->pop_prec) fnc += weight;
        rcm += weight * rc;
        if (rc > rcmax) rcmax = rc;
    }
    x->fnc = fnc;
    x->rcm = rcm;
    x->rcmax = rcmax;
}

/* set_LTE for line k at point p (lineProducingSpecies.tpp:84-99) */
static void set_lte_line(Lsp* x, const double* T, uint32_t p, uint32_t k) {
    const OrcSpecies* s = x->s;
    ld* pp = x->pop + (size_t)p * s->nlev;
    const uint32_t i = s->irad[k], j = s->jrad[k];
    const ld tot_line = pp[i] + pp[j];
    pp[i] = (ld)(s->weight[i] * exp(-s->energy[i] / (KB_ALI * T[p])));
    pp[j] = (ld)(s->weight[j] * exp(-s->energy[j] / (KB_ALI * T[p])));
    const ld pf = pp[i] + pp[j];
    pp[i] *= tot_line / pf;
    pp[j] *= tot_line / pf;
}

/* set_LTE_specific_levels (:106-125) */
static void set_lte_levels(Lsp* x, const double* T, uint32_t p, const char* mask) {
    const OrcSpecies* s = x->s;
    ld* pp = x->pop + (size_t)p * s->nlev;
    ld tot = 0.0L, pf = 0.0L;
    for (uint32_t i = 0; i < s->nlev; i++)
        if (mask[i]) {
            tot += pp[i];
            pp[i] = (ld)(s->weight[i] * exp(-s->energy[i] / (KB_ALI * T[p])));
            pf += pp[i];
        }
    for (uint32_t i = 0; i < s->nlev; i++)
        if (mask[i]) pp[i] *= tot / pf;
}

/* correct_negative_populations (:711-802) */
static void correct_negative(Lsp* x, uint32_t P, const double* T, const OrcAliParams* prm) {
    const OrcSpecies* s = x->s;
    const uint32_t nlev = s->nlev;
    for (uint32_t p = 0; p < P; p++) {
        if (x->tot[p] > 0.0L) {
            ld tp = 0.0L;
            ld* pp = x->pop + (size_t)p * nlev;
            for (uint32_t i = 0; i < nlev; i++) {
                if (pp[i] < 0.0L) pp[i] = 0.0L;
                else tp += pp[i];
            }
            for (uint32_t i = 0; i < nlev; i++) pp[i] = pp[i] * x->tot[p] / tp;
        }
    }
    char* mod = (char*)malloc(nlev);
    for (uint32_t p = 0; p < P; p++) {
        memset(mod, 0, nlev);
        uint32_t next_n = 0, curr_n = 0;
        do {
            curr_n = next_n;
            int inv = 0;
            ld* pp = x->pop + (size_t)p * nlev;
            for (uint32_t k = s->nrad; k-- > 0;) {
                const uint32_t i = s->irad[k], j = s->jrad[k];
                if (pp[j] < (ld)(s->Bs[k] / s->Ba[k]) * pp[i] * (ld)prm->population_inversion_fraction) {
                    set_lte_line(x, T, p, k);
                    mod[i] = mod[j] = 1;
                    inv = 1;
                }
            }
            for (uint32_t k = 0; k < s->nrad; k++) {
                const uint32_t i = s->irad[k], j = s->jrad[k];
                if (pp[j] < (ld)(s->Bs[k] / s->Ba[k]) * pp[i] * (ld)prm->population_inversion_fraction) {
                    set_lte_line(x, T, p, k);
                    mod[i] = mod[j] = 1;
                    inv = 1;
                }
            }
            if (inv) set_lte_levels(x, T, p, mod);
            next_n = 0;
            for (uint32_t i = 0; i < nlev; i++) next_n += mod[i] ? 1 : 0;
        } while (next_n != curr_n);
    }
    free(mod);
}

/* Householder QR with column pivoting, solve A c = b (A order x order), long double. */
static void qr_colpiv_solve(ld* A, ld* b, uint32_t n, ld* c) {
    uint32_t perm[64];
    for (uint32_t j = 0; j < n; j++) perm[j] = j;
    uint32_t rank = n;
    for (uint32_t k = 0; k < n; k++) {
        /* pivot: remaining column of largest norm */
        uint32_t best = k;
        ld bn = -1.0L;
        for (uint32_t j = k; j < n; j++) {
            ld s = 0.0L;
            for (uint32_t i = k; i < n; i++) s += A[(size_t)i * n + j] * A[(size_t)i * n + j];
            if (s > bn) {
                bn = s;
                best = j;
            }
        }
        if (best != k) {
            for (uint32_t i = 0; i < n; i++) {
                const ld t = A[(size_t)i * n + k];
                A[(size_t)i * n + k] = A[(size_t)i * n + best];
                A[(size_t)i * n + best] = t;
            }
            const uint32_t t = perm[k];
            perm[k] = perm[best];
            perm[best] = t;
        }
        const ld alpha_n = sqrtl(bn);
        if (alpha_n == 0.0L) {
            rank = k;
            break;
        }
        const ld alpha = A[(size_t)k * n + k] > 0 ? -alpha_n : alpha_n;
        ld v[64];
        for (uint32_t i = 0; i < n; i++) v[i] = (i < k) ? 0.0L : A[(size_t)i * n + k];
        v[k] -= alpha;
        ld vn = 0.0L;
        for (uint32_t i = k; i < n; i++) vn += v[i] * v[i];
        if (vn == 0.0L) continue;
        for (uint32_t j = k; j < n; j++) {
            ld s = 0.0L;
            for (uint32_t i = k; i < n; i++) s += v[i] * A[(size_t)i * n + j];
            s = 2.0L * s / vn;
            for (uint32_t i = k; i < n; i++) A[(size_t)i * n + j] -= s * v[i];
        }
        ld s = 0.0L;
        for (uint32_t i = k; i < n; i++) s += v[i] * b[i];
        s = 2.0L * s / vn;
        for (uint32_t i = k; i < n; i++) b[i] -= s * v[i];
    }
    ld x[64];
    for (uint32_t i = 0; i < n; i++) x[i] = 0.0L;
    for (uint32_t i = rank; i-- > 0;) {
        ld s = b[i];
        for (uint32_t j = i + 1; j < rank; j++) s -= A[(size_t)i * n + j] * x[j];
        x[i] = s / A[(size_t)i * n + i];
    }
    for (uint32_t j = 0; j < n; j++) c[perm[j]] = x[j];
}

/* Ng coefficients from the last `order` residuals (update_using_acceleration). */
static void ng_coefficients(Lsp* x, uint32_t order, ld* coef) {
    ld RTR[64 * 64], ones[64];
    for (uint32_t i = 0; i < order; i++)
        for (uint32_t j = 0; j < order; j++) {
            const ld* a = x->res[x->nres - order + i];
            const ld* b = x->res[x->nres - order + j];
            ld s = 0.0L;
            for (size_t t = 0; t < x->n; t++) s += a[t] * b[t];
            RTR[(size_t)i * order + j] = s;
        }
    for (uint32_t i = 0; i < order; i++) ones[i] = 1.0L;
    qr_colpiv_solve(RTR, ones, order, coef);
    ld sum = 0.0L;
    for (uint32_t i = 0; i < order; i++) sum += coef[i];
    for (uint32_t i = 0; i < order; i++) coef[i] /= sum;
}

static void update_using_acceleration(Lsp* x, uint32_t order) {
    memcpy(x->prev1, x->pop, sizeof(ld) * x->n);
    residual_push(x);
    ld coef[64];
    ng_coefficients(x, order, coef);
    for (size_t t = 0; t < x->n; t++) x->pop[t] = 0.0L;
    for (uint32_t i = 0; i < order; i++) {
        const ld* h = x->hist[x->nhist - 1 - i];
        const ld c = coef[order - 1 - i];
        for (size_t t = 0; t < x->n; t++) x->pop[t] += h[t] * c;
    }
    for (uint32_t i = 0; i < x->nres; i++) free(x->res[i]);
    x->nres = 0;
    erase_front(x->hist, &x->nhist, 1);
}

static void update_using_acceleration_trial(Lsp* x, uint32_t order) {
    residual_push(x);
    memcpy(x->trial_prev, x->trial, sizeof(ld) * x->n);
    ld coef[64];
    ng_coefficients(x, order, coef);
    for (size_t t = 0; t < x->n; t++) x->trial[t] = 0.0L;
    for (uint32_t i = 0; i < order; i++) {
        const ld* h = x->hist[x->nhist - 1 - i];
        const ld c = coef[order - 1 - i];
        for (size_t t = 0; t < x->n; t++) x->trial[t] += h[t] * c;
    }
    free(x->res[--x->nres]);
    free(x->hist[--x->nhist]);
}

static void set_line_data(OrcModel* m, double* em, double* op, double* crit, Lsp* xs, uint32_t nls,
                          const OrcAliParams* prm) {
    const uint32_t P = m->npoints, L = m->nlines;
    for (uint32_t l = 0; l < nls; l++) {
        const OrcSpecies* s = xs[l].s;
        for (uint32_t p = 0; p < P; p++) {
            const ld* pp = xs[l].pop + (size_t)p * s->nlev;
            for (uint32_t k = 0; k < s->nrad; k++) {
                const uint32_t lid = s->line_offset + k;
                em[(size_t)p * L + lid] = emissivity_of(s, pp, k, prm->min_line_emissivity);
                op[(size_t)p * L + lid] = opacity_of(s, pp, k, prm->min_line_opacity);
                crit[(size_t)p * L + lid] = op[(size_t)p * L + lid] / (double)xs[l].tot[p];
            }
        }
    }
}

int orc_ali_run(OrcModel* m, double* em, double* op, double* crit, uint32_t nlspecs, const OrcSpecies* sp,
                uint32_t nspecs, const double* abundance, const OrcAliParams* prm, int use_ng, long max_it,
                double* const* pops, double* err_mean, double* err_max, double* const* Jeff_out, int nthreads) {
    const uint32_t P = m->npoints, F = m->nfreqs, L = m->nlines;
    const double* T = m->temperature;
    Lsp* xs = (Lsp*)calloc(nlspecs, sizeof(Lsp));
    double* J = (double*)malloc(sizeof(double) * (size_t)P * F);
    double* lam = (double*)malloc(sizeof(double) * (size_t)P * L);
    double* Ls = NULL;
    size_t ls_cap = 0;
    int rc = 0;
    for (uint32_t l = 0; l < nlspecs; l++) {
        Lsp* x = &xs[l];
        x->s = &sp[l];
        x->n = (size_t)P * sp[l].nlev;
        x->pop = (ld*)malloc(sizeof(ld) * x->n);
        x->prev1 = (ld*)malloc(sizeof(ld) * x->n);
        x->trial = (ld*)calloc(x->n, sizeof(ld));
        x->trial_prev = (ld*)calloc(x->n, sizeof(ld));
        x->tot = (ld*)malloc(sizeof(ld) * P);
        for (size_t i = 0; i < x->n; i++) x->pop[i] = x->prev1[i] = pops[l][i];
        for (uint32_t p = 0; p < P; p++) x->tot[p] = abundance[(size_t)p * nspecs + sp[l].num];
        push(&x->hist, &x->nhist, &x->cap_hist, x->pop, x->n); /* update_using_LTE's push */
        x->Jlin = (double*)malloc(sizeof(double) * (size_t)P * sp[l].nrad);
        x->Jeff = (double*)malloc(sizeof(double) * (size_t)P * sp[l].nrad);
        x->Jdif = (double*)malloc(sizeof(double) * (size_t)P * sp[l].nrad);
        if ((size_t)P * sp[l].nrad > ls_cap) ls_cap = (size_t)P * sp[l].nrad;
    }
    Ls = (double*)malloc(sizeof(double) * (ls_cap ? ls_cap : 1));
    set_line_data(m, em, op, crit, xs, nlspecs, prm);
    /* n_off_diag > 0 (or global_stateq): ALO lists and the global rate system */
    const int global = prm->n_off_diag > 0 || prm->global_stateq;
    const uint32_t cap = 2 * prm->n_off_diag * m->hnrays + 1;
    uint32_t* alo_n = NULL;
    uint32_t* alo_nr = NULL;
    double* alo_ls = NULL;
    if (global) {
        alo_n = (uint32_t*)calloc((size_t)P * L, sizeof(uint32_t));
        alo_nr = (uint32_t*)calloc((size_t)P * L * cap, sizeof(uint32_t));
        alo_ls = (double*)calloc((size_t)P * L * cap, sizeof(double));
        if (!alo_n || !alo_nr || !alo_ls) rc = -1;
    }

    int iteration = 0, iteration_normal = 0, some_not_converged = 1;
    long nerr = 0;
    while (some_not_converged && iteration < max_it && rc == 0) {
        int use_step = 0;
        uint32_t order = 0;
        const uint32_t skip = prm->Ng_acceleration_remove_N_its;
        if (!prm->use_adaptive_Ng_acceleration) {
            if (use_ng && (uint32_t)iteration_normal == prm->Ng_acceleration_mem_limit + skip) {
                use_step = 1;
                order = prm->Ng_acceleration_mem_limit;
            }
        } else if (use_ng && (uint32_t)iteration_normal >= prm->adaptive_Ng_acceleration_min_order + skip) {
            double curr = 0.0, trial = 0.0;
            for (uint32_t l = 0; l < nlspecs; l++)
                curr += prm->adaptive_Ng_acceleration_use_max_criterion ? xs[l].rcmax : xs[l].rcm;
            for (uint32_t l = 0; l < nlspecs; l++) {
                update_using_acceleration_trial(&xs[l], (uint32_t)iteration_normal - skip);
                check_convergence_trial(&xs[l], P, prm);
            }
            for (uint32_t l = 0; l < nlspecs; l++)
                trial += prm->adaptive_Ng_acceleration_use_max_criterion ? xs[l].rcmax : xs[l].rcm;
            if (trial < curr || (uint32_t)iteration_normal == prm->Ng_acceleration_mem_limit + skip) {
                use_step = 1;
                order = (uint32_t)iteration_normal - skip;
            }
        }
        if (use_step) {
            for (uint32_t l = 0; l < nlspecs; l++) {
                update_using_acceleration(&xs[l], order);
                correct_negative(&xs[l], P, T, prm);
                check_convergence(&xs[l], P, prm);
            }
            set_line_data(m, em, op, crit, xs, nlspecs, prm);
            iteration_normal = 0;
            continue;
        }
        iteration++;
        some_not_converged = 0;
        if (global) {
            const int frc = orc_formal_solve_fo2_alo(m, prm->n_off_diag, J, cap, alo_n, alo_nr, alo_ls, nthreads);
            if (frc != 0) rc = frc;
            for (uint32_t l = 0; l < nlspecs; l++)
                jeff_species_alo(m, xs[l].s, J, cap, alo_n, alo_nr, alo_ls, xs[l].pop, xs[l].Jlin, xs[l].Jeff,
                                 xs[l].Jdif);
            for (uint32_t l = 0; l < nlspecs && rc == 0; l++) {
                Lsp* x = &xs[l];
                memcpy(x->prev1, x->pop, sizeof(ld) * x->n);
                residual_push(x);
                if (stateq_global(x->s, P, L, x->prev1, x->Jeff, cap, alo_n, alo_nr, alo_ls, T, abundance, nspecs,
                                  x->tot, prm->min_line_opacity, x->pop) != 0)
                    rc = -3;
                correct_negative(x, P, T, prm);
                check_convergence(x, P, prm);
            }
            set_line_data(m, em, op, crit, xs, nlspecs, prm);
            iteration_normal++;
            for (uint32_t l = 0; l < nlspecs; l++) {
                if (err_mean) err_mean[nerr] = xs[l].rcm;
                if (err_max) err_max[nerr] = xs[l].rcmax;
                nerr++;
                if (xs[l].fnc > 1.0 - prm->convergence_fraction) some_not_converged = 1;
            }
            continue;
        }
        if (orc_formal_solve_fo2(m, J, NULL, lam, NULL, nthreads) != 0) rc = -2;
        for (uint32_t l = 0; l < nlspecs; l++) jeff_species(m, xs[l].s, J, lam, xs[l].pop, xs[l].Jlin, xs[l].Jeff, xs[l].Jdif);
        for (uint32_t l = 0; l < nlspecs && rc == 0; l++) {
            Lsp* x = &xs[l];
            const OrcSpecies* s = x->s;
            /* update_using_statistical_equilibrium: history, then solve each block */
            memcpy(x->prev1, x->pop, sizeof(ld) * x->n);
            residual_push(x);
            for (uint32_t p = 0; p < P; p++)
                for (uint32_t k = 0; k < s->nrad; k++)
                    Ls[(size_t)p * s->nrad + k] = lam[(size_t)p * L + s->line_offset + k];
            const uint32_t n = s->nlev;
            ld* M = (ld*)malloc(sizeof(ld) * n * n);
            ld* y = (ld*)malloc(sizeof(ld) * n);
            for (uint32_t p = 0; p < P && rc == 0; p++) {
                rate_block(s, x->prev1 + (size_t)p * n, x->Jeff + (size_t)p * s->nrad, Ls + (size_t)p * s->nrad, T[p],
                           abundance + (size_t)p * nspecs, prm->min_line_opacity, M);
                for (uint32_t i = 0; i < n; i++) y[i] = 0.0L;
                y[n - 1] = x->tot[p];
                if (solve_dense(M, y, n) != 0) rc = -3;
                for (uint32_t i = 0; i < n; i++) x->pop[(size_t)p * n + i] = y[i];
            }
            free(M);
            free(y);
            correct_negative(x, P, T, prm);
            check_convergence(x, P, prm);
        }
        set_line_data(m, em, op, crit, xs, nlspecs, prm);
        iteration_normal++;
        for (uint32_t l = 0; l < nlspecs; l++) {
            if (err_mean) err_mean[nerr] = xs[l].rcm;
            if (err_max) err_max[nerr] = xs[l].rcmax;
            nerr++;
            if (xs[l].fnc > 1.0 - prm->convergence_fraction) some_not_converged = 1;
        }
    }
    for (uint32_t l = 0; l < nlspecs; l++) {
        Lsp* x = &xs[l];
        for (size_t i = 0; i < x->n; i++) pops[l][i] = (double)x->pop[i];
        if (Jeff_out && Jeff_out[l]) memcpy(Jeff_out[l], x->Jeff, sizeof(double) * (size_t)P * x->s->nrad);
        for (uint32_t i = 0; i < x->nhist; i++) free(x->hist[i]);
        for (uint32_t i = 0; i < x->nres; i++) free(x->res[i]);
        free(x->hist);
        free(x->res);
        free(x->pop);
        free(x->prev1);
        free(x->trial);
        free(x->trial_prev);
        free(x->tot);
        free(x->Jlin);
        free(x->Jeff);
        free(x->Jdif);
    }
    free(xs);
    free(J);
    free(lam);
    free(Ls);
    free(alo_n);
    free(alo_nr);
    free(alo_ls);
    return rc == 0 ? iteration : rc;
}
