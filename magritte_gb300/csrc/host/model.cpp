// Host-side Model: set-up arithmetic and the C-ABI calls of the formal solve.
// Compiled with -ffp-contract=off so every a*b+c rounds twice, as in the
// reference's x86-64 build.
#include "model.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>

namespace mgrhost {

static void check(int rc) {
    if (rc != MGR_OK) throw std::runtime_error(std::string("magritte_gb300: ") + mgr_last_error());
}

Model::~Model() { release_device(); }

void Model::release_device() {
    if (dev_) {
        mgr_model_free(dev_);
        dev_ = nullptr;
    }
}

uint64_t Model::launches() const { return mgr_launch_count(); }

std::vector<double> Model::ali_phase_times() const {
    double ms[4];
    if (!dev_ || mgr_ali_phase_times(dev_, ms) != MGR_OK) return {};
    return std::vector<double>(ms, ms + 4);
}

// ---------------------------------------------------------------------------------
// prepare(): derived data that the reference computes in its read() methods.
// ---------------------------------------------------------------------------------
void Model::prepare() {
    Parameters& prm = parameters;
    const Size P = (Size)(geometry.points.position.shape.empty() ? 0 : geometry.points.position.shape[0]);
    if (P == 0) throw std::runtime_error("Model::prepare: geometry.points.position is not set");
    prm.npoints_.set(P, "npoints");

    // Points::read (points.cpp:7-65): cumulative neighbour counts.
    Points& pts = geometry.points;
    if (pts.n_neighbors.size() != P) throw std::runtime_error("n_neighbors must have npoints entries");
    if (pts.velocity.size() != 3 * (size_t)P) throw std::runtime_error("velocity must be [npoints][3]");
    pts.cum_n_neighbors.resize({P});
    size_t E = 0;
    for (Size p = 0; p < P; p++) {
        pts.cum_n_neighbors[p] = (Size)E;
        E += pts.n_neighbors[p];
    }
    if (E != pts.neighbors.size()) throw std::runtime_error("neighbors length differs from sum(n_neighbors)");

    // Rays::read (rays.cpp:5-66): hnrays and antipodes (tolerance 1e-9, last match wins).
    Rays& rays = geometry.rays;
    // adaptive ray directions: [npoints * nrays] directions and weights (rays.cpp:5-45),
    // recognised from the flag or, with nrays set, from the array's length
    const Size ndir = (Size)(rays.direction.shape.empty() ? 0 : rays.direction.shape[0]);
    if (!rays.use_adaptive_directions && prm.nrays_.set_ && P > 1 && ndir == prm.nrays_.v * P)
        rays.use_adaptive_directions = true;
    if (rays.use_adaptive_directions && (P == 0 || ndir % P != 0))
        throw std::runtime_error("adaptive ray directions must hold npoints * nrays entries");
    const Size nrays = rays.use_adaptive_directions ? ndir / P : ndir;
    if (nrays == 0 || rays.weight.size() != ndir) throw std::runtime_error("ray directions/weights not set");
    prm.nrays_.set(nrays, "nrays");
    prm.hnrays_.set(nrays / 2, "hnrays");
    rays.antipod.resize({nrays});
    for (Size r1 = 0; r1 < nrays; r1++) {
        bool found = false;
        for (Size r2 = 0; r2 < nrays; r2++) {
            const double x = rays.direction[3 * r1] + rays.direction[3 * r2];
            const double y = rays.direction[3 * r1 + 1] + rays.direction[3 * r2 + 1];
            const double z = rays.direction[3 * r1 + 2] + rays.direction[3 * r2 + 2];
            if (x * x + y * y + z * z < 1.0e-9) {
                rays.antipod[r1] = r2;
                found = true;
            }
        }
        if (!found) throw std::runtime_error("ray without antipode: directions must come in opposite pairs");
    }

    // Boundary::read (boundary.cpp:5-48).
    Boundary& bd = geometry.boundary;
    const Size B = (Size)bd.boundary2point.size();
    prm.nboundary_.set(B, "nboundary");
    bd.point2boundary.resize({P});
    for (Size p = 0; p < P; p++) bd.point2boundary[p] = P;
    for (Size b = 0; b < B; b++) {
        if (bd.boundary2point[b] >= P) throw std::runtime_error("boundary2point index out of range");
        bd.point2boundary[bd.boundary2point[b]] = b;
    }
    if (bd.boundary_condition.size() != B) {
        std::vector<int32_t> cmb(B, CMB);
        bd.boundary_condition.assign({B}, cmb.data());
    }
    if (bd.boundary_temperature.size() != B) {
        std::vector<double> t(B, T_CMB);
        bd.boundary_temperature.assign({B}, t.data());
    }

    // Lines::read (lines.cpp:11-69) and the LAMDA-derived quantities
    // (magritte/setup.py:766-770) when the user did not set them.
    const Size nlspecs = (Size)lines.lineProducingSpecies.size();
    if (nlspecs == 0) throw std::runtime_error("no line producing species");
    prm.nlspecs_.set(nlspecs, "nlspecs");
    lines.nrad_cum.resize({nlspecs});
    Size L = 0;
    lines.max_inverse_mass = 0.0;
    for (Size l = 0; l < nlspecs; l++) {
        LineProducingSpecies& ls = lines.lineProducingSpecies[l];
        Linedata& ld = ls.linedata;
        ld.nlev = (Size)ld.energy.size();
        ld.nrad = (Size)ld.irad.size();
        if (ld.weight.size() != ld.nlev || ld.jrad.size() != ld.nrad || ld.A.size() != ld.nrad)
            throw std::runtime_error("inconsistent line data");
        if (ld.frequency.size() != ld.nrad) {
            ld.frequency.resize(ld.nrad);
            for (Size k = 0; k < ld.nrad; k++) ld.frequency[k] = (ld.energy[ld.irad[k]] - ld.energy[ld.jrad[k]]) / HH;
        }
        if (ld.Bs.size() != ld.nrad || ld.Ba.size() != ld.nrad) {
            ld.Bs.resize(ld.nrad);
            ld.Ba.resize(ld.nrad);
            for (Size k = 0; k < ld.nrad; k++) {
                ld.Bs[k] = ld.A[k] * CC * CC / (2.0 * HH * std::pow(ld.frequency[k], 3));
                ld.Ba[k] = ld.weight[ld.irad[k]] / ld.weight[ld.jrad[k]] * ld.Bs[k];
            }
        }
        lines.nrad_cum[l] = L;
        L += ld.nrad;
        lines.max_inverse_mass = std::max(ld.inverse_mass, lines.max_inverse_mass);
    }
    prm.nlines_.set(L, "nlines");
    if (lines.line.size() != L) {
        lines.line.resize({L});
        lines.sorted_line.resize({L});
        lines.sorted_line_map.resize({L});
    }
    Size idx = 0;
    for (auto& ls : lines.lineProducingSpecies)
        for (Size k = 0; k < ls.linedata.nrad; k++) lines.line[idx++] = ls.linedata.frequency[k];
    // heapsort in the reference (lines.cpp:59); a stable sort agrees for distinct lines
    std::vector<Size> order(L);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](Size a, Size b) { return lines.line[a] < lines.line[b]; });
    for (Size s = 0; s < L; s++) {
        lines.sorted_line_map[s] = order[s];
        lines.sorted_line[s] = lines.line[order[s]];
    }
    if (lines.emissivity.size() != (size_t)P * L) {
        lines.emissivity.resize({P, L});
        lines.opacity.resize({P, L});
        lines.inverse_width.resize({P, L});
    }

    // chemistry: population_tot = abundance[p][num] (lineProducingSpecies.tpp:55)
    const Array<double>& ab = chemistry.species.abundance;
    if (ab.shape.size() != 2 || ab.shape[0] != P) throw std::runtime_error("abundance must be [npoints][nspecs]");
    const Size nspecs = (Size)ab.shape[1];
    prm.nspecs_.set(nspecs, "nspecs");
    for (auto& ls : lines.lineProducingSpecies) {
        if (ls.linedata.num >= nspecs) throw std::runtime_error("line species index outside the abundance table");
        ls.population_tot.resize({P});
        for (Size p = 0; p < P; p++) ls.population_tot[p] = ab[(size_t)p * nspecs + ls.linedata.num];
        if (ls.population.size() != (size_t)P * ls.linedata.nlev) ls.population.resize({(size_t)P * ls.linedata.nlev});
        if (ls.quadrature.roots.size() == 0) throw std::runtime_error("quadrature roots/weights not set");
    }
    const Size Q = (Size)lines.lineProducingSpecies[0].quadrature.roots.size();
    prm.nquads_.set(Q, "nquads");
    for (auto& ls : lines.lineProducingSpecies)
        if (ls.quadrature.roots.size() != Q || ls.quadrature.weights.size() != Q)
            throw std::runtime_error("every species needs nquads roots and weights");
    if (thermodynamics.temperature.gas.size() != P || thermodynamics.turbulence.vturb2.size() != P)
        throw std::runtime_error("temperature and turbulence must have npoints entries");
}

// ---------------------------------------------------------------------------------
// Model::compute_inverse_line_widths -> Lines::set_inverse_width (lines.tpp:45-59)
// ---------------------------------------------------------------------------------
int Model::compute_inverse_line_widths() {
    prepare();
    const Size P = parameters.npoints_.v, L = parameters.nlines_.v;
    const auto& T = thermodynamics.temperature.gas;
    const auto& vt2 = thermodynamics.turbulence.vturb2;
    for (Size p = 0; p < P; p++) {
        for (Size l = 0; l < parameters.nlspecs_.v; l++) {
            const Linedata& ld = lines.lineProducingSpecies[l].linedata;
            for (Size k = 0; k < ld.nrad; k++) {
                const Size lid = lines.nrad_cum[l] + k;
                const double width =
                    ld.frequency[k] * std::sqrt(TWO_KB_OVER_AMU_CC_SQUARED * ld.inverse_mass * T[p] + vt2[p]);
                lines.inverse_width[(size_t)p * L + lid] = (Real)1.0 / width;
            }
        }
    }
    lines.inverse_width.touch();
    return 0;
}

// ---------------------------------------------------------------------------------
// Model::compute_spectral_discretisation (model.cpp:70-298)
// ---------------------------------------------------------------------------------
int Model::compute_spectral_discretisation() {
    prepare();
    const Size P = parameters.npoints_.v, L = parameters.nlines_.v, Q = parameters.nquads_.v;
    const Size F = L * Q;
    parameters.nfreqs_ = F;
    Frequencies& fr = radiation.frequencies;
    fr.nu.resize({P, F});
    fr.corresponding_line.resize({F});
    fr.corresponding_l_for_spec.resize({F});
    fr.corresponding_k_for_tran.resize({F});
    fr.corresponding_z_for_line.resize({F});
    fr.appears_in_line_integral.resize({F});
    const auto& T = thermodynamics.temperature.gas;
    const auto& vt2 = thermodynamics.turbulence.vturb2;
    for (Size p = 0; p < P; p++) {
        Size index0 = 0, index1 = 0;
        for (Size l = 0; l < parameters.nlspecs_.v; l++) {
            const LineProducingSpecies& ls = lines.lineProducingSpecies[l];
            const double inverse_mass = ls.linedata.inverse_mass;
            for (Size k = 0; k < ls.linedata.nrad; k++) {
                const double freqs_line = lines.line[index0];
                const double width =
                    freqs_line * std::sqrt(TWO_KB_OVER_AMU_CC_SQUARED * inverse_mass * T[p] + vt2[p]);
                for (Size z = 0; z < Q; z++) {
                    fr.nu[(size_t)p * F + index1] = freqs_line + width * ls.quadrature.roots[z];
                    index1++;
                }
                index0++;
            }
        }
    }
    Size index2 = 0;
    for (Size l = 0; l < parameters.nlspecs_.v; l++) {
        for (Size k = 0; k < lines.lineProducingSpecies[l].linedata.nrad; k++) {
            for (Size z = 0; z < Q; z++) {
                fr.appears_in_line_integral[index2] = 1;
                fr.corresponding_l_for_spec[index2] = l;
                fr.corresponding_k_for_tran[index2] = k;
                fr.corresponding_z_for_line[index2] = z;
                fr.corresponding_line[index2] = lines.nrad_cum[l] + k;
                index2++;
            }
        }
    }
    spectralDiscretisation = SD_Lines;
    return 0;
}

int Model::compute_spectral_discretisation(Real width) {
    prepare();
    const Size P = parameters.npoints_.v, L = parameters.nlines_.v, Q = parameters.nquads_.v;
    const Size F = L * Q;
    parameters.nfreqs_ = F;
    Frequencies& fr = radiation.frequencies;
    fr.nu.resize({P, F});
    fr.corresponding_line.resize({F});
    fr.corresponding_l_for_spec.resize({F});
    fr.corresponding_k_for_tran.resize({F});
    fr.corresponding_z_for_line.resize({F});
    fr.appears_in_line_integral.resize({F});
    for (Size p = 0; p < P; p++) {
        Size index0 = 0, index1 = 0;
        for (Size l = 0; l < parameters.nlspecs_.v; l++) {
            const LineProducingSpecies& ls = lines.lineProducingSpecies[l];
            for (Size k = 0; k < ls.linedata.nrad; k++) {
                const double freqs_line = lines.line[index0];
                for (Size z = 0; z < Q; z++) {
                    fr.nu[(size_t)p * F + index1] = freqs_line + freqs_line * width * ls.quadrature.roots[z];
                    index1++;
                }
                index0++;
            }
        }
    }
    Size index2 = 0;
    for (Size l = 0; l < parameters.nlspecs_.v; l++)
        for (Size k = 0; k < lines.lineProducingSpecies[l].linedata.nrad; k++)
            for (Size z = 0; z < Q; z++) {
                fr.appears_in_line_integral[index2] = 1;
                fr.corresponding_l_for_spec[index2] = l;
                fr.corresponding_k_for_tran[index2] = k;
                fr.corresponding_z_for_line[index2] = z;
                fr.corresponding_line[index2] = lines.nrad_cum[l] + k;
                index2++;
            }
    spectralDiscretisation = SD_Image;
    return 0;
}

int Model::compute_spectral_discretisation(Real nu_min, Real nu_max) {
    prepare();
    return compute_spectral_discretisation(nu_min, nu_max, parameters.nlines_.v * parameters.nquads_.v);
}

int Model::compute_spectral_discretisation(Real nu_min, Real nu_max, Size n_image_freqs) {
    if (n_image_freqs < 1)
        throw std::runtime_error("At least a single frequency is needed to compute a spectral discretization.");
    prepare();
    const Size P = parameters.npoints_.v;
    parameters.nfreqs_ = n_image_freqs;
    Frequencies& fr = radiation.frequencies;
    fr.nu.resize({P, n_image_freqs});
    fr.corresponding_line.resize({n_image_freqs});
    fr.corresponding_l_for_spec.resize({n_image_freqs});
    fr.corresponding_k_for_tran.resize({n_image_freqs});
    fr.corresponding_z_for_line.resize({n_image_freqs});
    fr.appears_in_line_integral.resize({n_image_freqs});
    for (Size f = 0; f < n_image_freqs; f++) {
        fr.appears_in_line_integral[f] = 0;
        fr.corresponding_l_for_spec[f] = n_image_freqs;
        fr.corresponding_k_for_tran[f] = n_image_freqs;
        fr.corresponding_z_for_line[f] = n_image_freqs;
        fr.corresponding_line[f] = 0;
    }
    if (n_image_freqs == 1) {
        for (Size p = 0; p < P; p++) fr.nu[p] = (Real)(nu_min + nu_max) / 2.0;
    } else {
        const long double dnu = (nu_max - nu_min) / (n_image_freqs - 1);
        for (Size p = 0; p < P; p++)
            for (Size f = 0; f < n_image_freqs; f++)
                fr.nu[(size_t)p * n_image_freqs + f] = (Real)(nu_min + f * dnu);
    }
    spectralDiscretisation = SD_Image;
    return 0;
}

// ---------------------------------------------------------------------------------
// LTE populations (lineProducingSpecies.tpp:52-75) and line emissivity/opacity
// (lineProducingSpecies.tpp:23-44, lines.tpp:29-40).  Populations are double here
// where the reference keeps long double.
// ---------------------------------------------------------------------------------
void Model::set_emissivity_and_opacity() {
    const Size P = parameters.npoints_.v, L = parameters.nlines_.v;
    for (Size p = 0; p < P; p++) {
        for (Size l = 0; l < parameters.nlspecs_.v; l++) {
            const LineProducingSpecies& ls = lines.lineProducingSpecies[l];
            const Linedata& ld = ls.linedata;
            for (Size k = 0; k < ld.nrad; k++) {
                const Size lid = lines.nrad_cum[l] + k;
                const Size i = ls.index(p, ld.irad[k]);
                const Size j = ls.index(p, ld.jrad[k]);
                const double freq = ld.frequency[k];
                const double em = freq * HH_OVER_FOUR_PI * ld.A[k] * ls.population[i];
                const double op = freq * HH_OVER_FOUR_PI * (ls.population[j] * ld.Ba[k] - ls.population[i] * ld.Bs[k]);
                lines.emissivity[(size_t)p * L + lid] = std::max(em, parameters.min_line_emissivity);
                lines.opacity[(size_t)p * L + lid] = std::max(op, parameters.min_line_opacity);
            }
        }
    }
    lines.emissivity.touch();
    lines.opacity.touch();
}

int Model::compute_LTE_level_populations() {
    prepare();
    const Size P = parameters.npoints_.v;
    const auto& T = thermodynamics.temperature.gas;
    for (auto& ls : lines.lineProducingSpecies) {
        const Linedata& ld = ls.linedata;
        for (Size p = 0; p < P; p++) {
            double partition_function = 0.0;
            for (Size i = 0; i < ld.nlev; i++) {
                const Size ind = ls.index(p, i);
                ls.population[ind] = ld.weight[i] * std::exp(-ld.energy[i] / (KB * T[p]));
                partition_function += ls.population[ind];
            }
            for (Size i = 0; i < ld.nlev; i++) ls.population[ls.index(p, i)] *= ls.population_tot[p] / partition_function;
        }
        ls.population.touch();
    }
    set_emissivity_and_opacity();
    return 0;
}

// Model::set_dshift_max (model.cpp:1158-1178)
int Model::set_dshift_max() {
    const Size P = parameters.npoints_.v;
    std::vector<double> d(P);
    const auto& T = thermodynamics.temperature.gas;
    const auto& vt2 = thermodynamics.turbulence.vturb2;
    for (Size o = 0; o < P; o++) {
        d[o] = std::numeric_limits<Real>::max();
        for (const auto& ls : lines.lineProducingSpecies) {
            const double nd = parameters.max_width_fraction *
                              std::sqrt(TWO_KB_OVER_AMU_CC_SQUARED * ls.linedata.inverse_mass * T[o] + vt2[o]);
            if (d[o] > nd) d[o] = nd;
        }
    }
    // unchanged values keep the array's version, so the resident device model is reused
    if (dshift_max.size() != P || std::memcmp(dshift_max.data(), d.data(), sizeof(double) * P) != 0)
        dshift_max.assign({P}, d.data());
    return 0;
}

// ---------------------------------------------------------------------------------
// Device model
// ---------------------------------------------------------------------------------
uint64_t Model::signature() const {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t x) {
        h ^= x;
        h *= 1099511628211ull;
    };
    mix(geometry.points.position.version);
    mix(geometry.points.velocity.version);
    mix(geometry.points.neighbors.version);
    mix(geometry.points.n_neighbors.version);
    mix(geometry.rays.direction.version);
    mix(geometry.rays.weight.version);
    mix((uint64_t)geometry.rays.use_adaptive_directions);
    mix(geometry.boundary.boundary2point.version);
    mix(geometry.boundary.boundary_condition.version);
    mix(geometry.boundary.boundary_temperature.version);
    mix(thermodynamics.temperature.gas.version);
    mix(thermodynamics.turbulence.vturb2.version);
    mix(radiation.frequencies.nu.version);
    mix(dshift_max.version);
    mix((uint64_t)parameters.approx());
    mix((uint64_t)parameters.spherical_symmetry_);
    double knobs[4] = {parameters.min_opacity, parameters.min_dtau, parameters.max_interpolation_diff,
                       parameters.max_distance_opacity_contribution};
    for (double k : knobs) {
        uint64_t b;
        std::memcpy(&b, &k, 8);
        mix(b);
    }
    return h;
}

namespace {
struct DescStorage {
    std::vector<Size> nrad;
    std::vector<double> line_A, inv_mass, quad_w, quad_r;
};
}  // namespace

void Model::fill_desc(MgrModelDesc& d) {
    std::memset(&d, 0, sizeof(d));
    d.npoints = parameters.npoints_.v;
    d.nrays = parameters.nrays_.v;
    d.hnrays = parameters.hnrays_.v;
    d.nlines = parameters.nlines_.v;
    d.nquads = parameters.nquads_.v;
    d.nfreqs = parameters.nfreqs_;
    d.nlspecs = parameters.nlspecs_.v;
    d.nboundary = parameters.nboundary_.v;
    d.position = geometry.points.position.data();
    d.velocity = geometry.points.velocity.data();
    d.n_neighbors = geometry.points.n_neighbors.data();
    d.cum_n_neighbors = geometry.points.cum_n_neighbors.data();
    d.neighbors = geometry.points.neighbors.data();
    d.point2boundary = geometry.boundary.point2boundary.data();
    d.boundary_condition = geometry.boundary.boundary_condition.data();
    d.boundary_temperature = geometry.boundary.boundary_temperature.data();
    d.ray_direction = geometry.rays.direction.data();
    d.ray_weight = geometry.rays.weight.data();
    d.antipod = geometry.rays.antipod.data();
    d.line = lines.line.data();
    d.sorted_line = lines.sorted_line.data();
    d.sorted_line_map = lines.sorted_line_map.data();
    d.max_inverse_mass = lines.max_inverse_mass;
    d.emissivity = lines.emissivity.data();
    d.opacity = lines.opacity.data();
    d.inverse_width = lines.inverse_width.data();
    d.interp_criterion = crit_.data();
    d.temperature = thermodynamics.temperature.gas.data();
    d.vturb2 = thermodynamics.turbulence.vturb2.data();
    d.dshift_max = dshift_max.data();
    d.nu = radiation.frequencies.nu.data();
    d.corr_line = radiation.frequencies.corresponding_line.data();
    d.corr_lspec = radiation.frequencies.corresponding_l_for_spec.data();
    d.corr_k = radiation.frequencies.corresponding_k_for_tran.data();
    d.corr_z = radiation.frequencies.corresponding_z_for_line.data();
    d.in_line_integral = radiation.frequencies.appears_in_line_integral.data();
    d.min_opacity = parameters.min_opacity;
    d.min_dtau = parameters.min_dtau;
    d.max_interpolation_diff = parameters.max_interpolation_diff;
    d.max_distance_opacity_contribution = parameters.max_distance_opacity_contribution;
    d.approx = parameters.approx();
    d.spherical_symmetry = parameters.spherical_symmetry_ ? 1 : 0;
    d.use_adaptive_directions = geometry.rays.use_adaptive_directions ? 1 : 0;
}

MgrModel* Model::device_model() {
    const Size P = parameters.npoints_.v, L = parameters.nlines_.v;
    // InterpHelper criterion: opacity / population_tot (solver_interp_helper.hpp:15-24)
    crit_.resize((size_t)P * L);
    for (Size l = 0; l < parameters.nlspecs_.v; l++) {
        const LineProducingSpecies& ls = lines.lineProducingSpecies[l];
        for (Size k = 0; k < ls.linedata.nrad; k++) {
            const Size lid = lines.nrad_cum[l] + k;
            for (Size p = 0; p < P; p++)
                crit_[(size_t)p * L + lid] = lines.opacity[(size_t)p * L + lid] / ls.population_tot[p];
        }
    }
    const uint64_t sig = signature();
    if (dev_ && sig == dev_signature_) {
        // a differentiable solve or imager (velocities, frequencies and line data set
        // from device tensors) may have run on this device copy since the last call
        check(mgr_model_restore_inputs(dev_, geometry.points.velocity.data(), radiation.frequencies.nu.data()));
        check(mgr_model_set_line_data(dev_, lines.emissivity.data(), lines.opacity.data(), lines.inverse_width.data(),
                                      crit_.data()));
        return dev_;
    }
    release_device();
    DescStorage st;
    const Size nls = parameters.nlspecs_.v, Q = parameters.nquads_.v;
    for (Size l = 0; l < nls; l++) {
        const LineProducingSpecies& ls = lines.lineProducingSpecies[l];
        st.nrad.push_back(ls.linedata.nrad);
        st.inv_mass.push_back(ls.linedata.inverse_mass);
        for (Size k = 0; k < ls.linedata.nrad; k++) st.line_A.push_back(ls.linedata.A[k]);
        for (Size z = 0; z < Q; z++) {
            st.quad_w.push_back(ls.quadrature.weights[z]);
            st.quad_r.push_back(ls.quadrature.roots[z]);
        }
    }
    MgrModelDesc d;
    fill_desc(d);
    d.nrad = st.nrad.data();
    d.nrad_cum = lines.nrad_cum.data();
    d.line_A = st.line_A.data();
    d.lspec_inverse_mass = st.inv_mass.data();
    d.quad_weights = st.quad_w.data();
    d.quad_roots = st.quad_r.data();
    check(mgr_model_create(&d, &dev_));
    dev_signature_ = sig;
    return dev_;
}

// ---------------------------------------------------------------------------------
// Model::compute_radiation_field_feautrier_order_2 (model.cpp:353-390)
// ---------------------------------------------------------------------------------
MgrModel* Model::upload() {
    prepare();
    if (radiation.frequencies.nu.size() == 0)
        throw std::runtime_error("compute_spectral_discretisation must be called before the formal solve");
    set_dshift_max();
    MgrModel* dev = device_model();
    check(mgr_model_set_n_off_diag(dev, (uint32_t)parameters.n_off_diag));
    return dev;
}

int Model::compute_radiation_field_feautrier_order_2() {
    MgrModel* dev = upload();
    const Size P = parameters.npoints_.v, F = parameters.nfreqs_, L = parameters.nlines_.v;
    const Size R = parameters.hnrays_.v;
    radiation.J.resize({P, F});
    if (parameters.store_u) radiation.u.resize({R, P, F});
    std::vector<double> lam((size_t)P * L);
    if (parameters.n_off_diag > 0) {
        // the banded solve (FP64): J, u, the diagonal, and the band elements kept on the
        // device for compute_Jeff (solver.tpp:2319-2355, :1760-1850)
        check(mgr_formal_solve_fo2_alo(dev, radiation.J.data(), parameters.store_u ? radiation.u.data() : nullptr,
                                       lam.data(), nullptr, nullptr));
    } else {
        check(mgr_formal_solve_fo2(dev, parameters.precision, radiation.J.data(),
                                   parameters.store_u ? radiation.u.data() : nullptr, lam.data()));
    }
    store_lambda(lam);
    return 0;
}

// Lambda::Ls diagonal per species (lambda.tpp:79-89) from the per-line ALO [P][L].
void Model::store_lambda(const std::vector<double>& lam) {
    const Size P = parameters.npoints_.v, L = parameters.nlines_.v;
    for (Size l = 0; l < parameters.nlspecs_.v; l++) {
        LineProducingSpecies& ls = lines.lineProducingSpecies[l];
        const Size nrad = ls.linedata.nrad;
        ls.lambda_diag.resize({P, nrad});
        ls.lambda_has.resize({P, nrad});
        for (Size p = 0; p < P; p++)
            for (Size k = 0; k < nrad; k++) {
                const double v = lam[(size_t)p * L + lines.nrad_cum[l] + k];
                ls.lambda_diag[(size_t)p * nrad + k] = v;
                ls.lambda_has[(size_t)p * nrad + k] = v != 0.0;
            }
    }
}

// Model::compute_radiation_field_shortchar_order_0 (model.cpp:313-349)
int Model::compute_radiation_field_shortchar_order_0() {
    MgrModel* dev = upload();
    const Size P = parameters.npoints_.v, F = parameters.nfreqs_, L = parameters.nlines_.v;
    const Size R = parameters.hnrays_.v, N = parameters.nrays_.v;
    radiation.J.resize({P, F});
    radiation.I.resize({N, P, F});
    radiation.u.resize({R, P, F});
    radiation.v.resize({R, P, F});
    std::vector<double> lam((size_t)P * L);
    check(mgr_formal_solve_sc0(dev, parameters.precision, radiation.J.data(), radiation.I.data(), radiation.u.data(),
                               radiation.v.data(), lam.data()));
    store_lambda(lam);
    return 0;
}

// ---------------------------------------------------------------------------------
// Level populations (model.cpp:514-545, :654-747) on the device
// ---------------------------------------------------------------------------------
void Model::attach_species() {
    const Size P = parameters.npoints_.v;
    const Size nls = parameters.nlspecs_.v;
    std::vector<MgrSpeciesDesc> sd(nls);
    std::vector<std::vector<MgrCollisionPartnerDesc>> cps(nls);
    std::vector<std::vector<double>> cd_flat, ce_flat;
    std::vector<const double*> pops(nls);
    for (Size l = 0; l < nls; l++) {
        const LineProducingSpecies& ls = lines.lineProducingSpecies[l];
        const Linedata& ld = ls.linedata;
        for (const CollisionPartner& c : ld.colpar) {
            MgrCollisionPartnerDesc d{};
            d.num_col_partner = c.num_col_partner;
            d.ortho_para = c.orth_or_para_H2 == "o" ? 1 : c.orth_or_para_H2 == "p" ? 2 : 0;
            d.ncol = c.ncol;
            d.ntmp = c.ntmp;
            d.icol = c.icol.data();
            d.jcol = c.jcol.data();
            d.tmp = c.tmp.data();
            std::vector<double> cdv, cev;
            for (Size t = 0; t < c.ntmp; t++)
                for (Size k = 0; k < c.ncol; k++) {
                    cdv.push_back(c.Cd[t][k]);
                    cev.push_back(c.Ce[t][k]);
                }
            cd_flat.push_back(std::move(cdv));
            ce_flat.push_back(std::move(cev));
            d.Cd = cd_flat.back().data();
            d.Ce = ce_flat.back().data();
            cps[l].push_back(d);
        }
        MgrSpeciesDesc& d = sd[l];
        d.num = ld.num;
        d.nlev = ld.nlev;
        d.nrad = ld.nrad;
        d.ncolpar = (uint32_t)cps[l].size();
        d.energy = ld.energy.data();
        d.weight = ld.weight.data();
        d.irad = ld.irad.data();
        d.jrad = ld.jrad.data();
        d.A = ld.A.data();
        d.Bs = ld.Bs.data();
        d.Ba = ld.Ba.data();
        d.frequency = ld.frequency.data();
        d.colpar = cps[l].data();
        pops[l] = ls.population.data();
    }
    // cd_flat / ce_flat may have reallocated while growing: refresh the pointers
    size_t c = 0;
    for (Size l = 0; l < nls; l++)
        for (auto& d : cps[l]) {
            d.Cd = cd_flat[c].data();
            d.Ce = ce_flat[c].data();
            c++;
        }
    const Size nspecs = (Size)(chemistry.species.abundance.size() / P);
    check(mgr_model_set_species(dev_, nls, sd.data(), nspecs, chemistry.species.abundance.data(), pops.data()));
}

int Model::compute_Jeff() {
    if (!dev_ || radiation.J.size() == 0)
        throw std::runtime_error("compute_Jeff needs a formal solve (compute_radiation_field_feautrier_order_2) first");
    attach_species();
    const Size P = parameters.npoints_.v;
    for (Size l = 0; l < parameters.nlspecs_.v; l++) {
        LineProducingSpecies& ls = lines.lineProducingSpecies[l];
        const Size nrad = ls.linedata.nrad;
        ls.Jlin.resize({P, nrad});
        ls.Jeff.resize({P, nrad});
        ls.Jdif.resize({P, nrad});
        check(mgr_compute_jeff(dev_, l, ls.Jlin.data(), ls.Jeff.data(), ls.Jdif.data()));
    }
    return 0;
}

// Model::compute_radiation_field_feautrier_order_2_sparse (model.cpp:474-510): the
// line-integrated J per species (LineProducingSpecies::J) and the ALO diagonal.
int Model::compute_radiation_field_feautrier_order_2_sparse() {
    MgrModel* dev = upload();
    const Size P = parameters.npoints_.v, L = parameters.nlines_.v;
    std::vector<double> Jl((size_t)P * L), lam((size_t)P * L);
    check(mgr_formal_solve_fo2_sparse(dev, parameters.precision, Jl.data(), lam.data()));
    for (Size l = 0; l < parameters.nlspecs_.v; l++) {
        LineProducingSpecies& ls = lines.lineProducingSpecies[l];
        const Size nrad = ls.linedata.nrad;
        ls.J.resize({P, nrad});
        for (Size p = 0; p < P; p++)
            for (Size k = 0; k < nrad; k++) ls.J[(size_t)p * nrad + k] = Jl[(size_t)p * L + lines.nrad_cum[l] + k];
    }
    store_lambda(lam);
    return 0;
}

// Model::compute_radiation_field_feautrier_order_2_anis (model.cpp:435-472): J and the
// anisotropy tensor elements per species.
int Model::compute_radiation_field_feautrier_order_2_anis() {
    MgrModel* dev = upload();
    const Size P = parameters.npoints_.v, L = parameters.nlines_.v;
    std::vector<double> buf(6 * (size_t)P * L);
    double* o[6];
    for (int k = 0; k < 6; k++) o[k] = buf.data() + k * (size_t)P * L;
    check(mgr_formal_solve_fo2_anis(dev, parameters.precision, o[0], o[1], o[2], o[3], o[4], o[5]));
    for (Size l = 0; l < parameters.nlspecs_.v; l++) {
        LineProducingSpecies& ls = lines.lineProducingSpecies[l];
        const Size nrad = ls.linedata.nrad;
        Array<double>* dst[6] = {&ls.J, &ls.J2_0, &ls.J2_1_Re, &ls.J2_1_Im, &ls.J2_2_Re, &ls.J2_2_Im};
        for (int k = 0; k < 6; k++) {
            dst[k]->resize({P, nrad});
            for (Size p = 0; p < P; p++)
                for (Size r = 0; r < nrad; r++)
                    (*dst[k])[(size_t)p * nrad + r] = o[k][(size_t)p * L + lines.nrad_cum[l] + r];
        }
    }
    return 0;
}

// Model::compute_radiation_field_feautrier_order_2_uv (model.cpp:395-433): radiation.u and .v
int Model::compute_radiation_field_feautrier_order_2_uv() {
    MgrModel* dev = upload();
    const Size P = parameters.npoints_.v, F = parameters.nfreqs_, R = parameters.hnrays_.v;
    radiation.u.resize({R, P, F});
    radiation.v.resize({R, P, F});
    check(mgr_formal_solve_fo2_uv(dev, parameters.precision, radiation.u.data(), radiation.v.data()));
    return 0;
}

// Model::compute_Jeff_sparse (model.cpp:549-570)
int Model::compute_Jeff_sparse() {
    if (!dev_ || lines.lineProducingSpecies.empty() || lines.lineProducingSpecies[0].J.size() == 0)
        throw std::runtime_error(
            "compute_Jeff_sparse needs a memory-lean formal solve (compute_radiation_field_feautrier_order_2_sparse) first");
    attach_species();
    const Size P = parameters.npoints_.v;
    for (Size l = 0; l < parameters.nlspecs_.v; l++) {
        LineProducingSpecies& ls = lines.lineProducingSpecies[l];
        const Size nrad = ls.linedata.nrad;
        ls.Jlin.resize({P, nrad});
        ls.Jeff.resize({P, nrad});
        check(mgr_compute_jeff_sparse(dev_, l, ls.Jlin.data(), ls.Jeff.data()));
    }
    return 0;
}

int Model::compute_level_populations(bool use_Ng_acceleration, long max_niterations) {
    return run_ali(use_Ng_acceleration, max_niterations, false);
}

// Model::compute_level_populations_sparse (model.cpp:756-850)
int Model::compute_level_populations_sparse(bool use_Ng_acceleration, long max_niterations) {
    return run_ali(use_Ng_acceleration, max_niterations, true);
}

int Model::run_ali(bool use_Ng_acceleration, long max_niterations, bool sparse) {
    if (spectralDiscretisation != SD_Lines) throw std::runtime_error("Spectral discretisation was not set for Lines!");
    MgrModel* dev = upload();
    attach_species();
    MgrAliParams prm{};
    prm.pop_prec = parameters.pop_prec;
    prm.min_rel_pop_for_convergence = parameters.min_rel_pop_for_convergence;
    prm.convergence_fraction = parameters.convergence_fraction;
    prm.population_inversion_fraction = parameters.population_inversion_fraction;
    prm.min_line_opacity = parameters.min_line_opacity;
    prm.min_line_emissivity = parameters.min_line_emissivity;
    prm.Ng_acceleration_mem_limit = parameters.Ng_acceleration_mem_limit;
    prm.adaptive_Ng_acceleration_min_order = parameters.adaptive_Ng_acceleration_min_order;
    prm.Ng_acceleration_remove_N_its = parameters.Ng_acceleration_remove_N_its;
    prm.use_adaptive_Ng_acceleration = parameters.use_adaptive_Ng_acceleration ? 1 : 0;
    prm.adaptive_Ng_acceleration_use_max_criterion = parameters.adaptive_Ng_acceleration_use_max_criterion ? 1 : 0;
    const Size nls = parameters.nlspecs_.v;
    const uint32_t cap = (uint32_t)(max_niterations > 0 ? max_niterations : 0) * nls;
    std::vector<double> emean(cap), emax(cap);
    int iterations = 0;
    auto ali = sparse ? mgr_compute_level_populations_sparse : mgr_compute_level_populations;
    check(ali(dev, parameters.precision, use_Ng_acceleration ? 1 : 0, max_niterations, &prm, &iterations,
              emean.data(), emax.data(), cap));
    error_mean.assign(emean.begin(), emean.begin() + (size_t)iterations * nls);
    error_max.assign(emax.begin(), emax.begin() + (size_t)iterations * nls);
    for (Size l = 0; l < nls; l++) {
        LineProducingSpecies& ls = lines.lineProducingSpecies[l];
        check(mgr_get_populations(dev, l, ls.population.data()));
        ls.population.touch();
    }
    check(mgr_get_line_data(dev, lines.emissivity.data(), lines.opacity.data()));
    lines.emissivity.touch();
    lines.opacity.touch();
    return iterations;
}

// ---------------------------------------------------------------------------------
// Imagers (model.cpp:957-1013)
// ---------------------------------------------------------------------------------
int Model::compute_image(Size ray_nr) { return image_old(ray_nr, false); }

// Model::compute_image_optical_depth (model.cpp:1061-1079 -> Solver::image_optical_depth,
// solver.tpp:655-684): the old imager's rays, the summed optical depth per frequency.
int Model::compute_image_optical_depth(Size ray_nr) { return image_old(ray_nr, true); }

int Model::image_old(Size ray_nr, bool tau) {
    if (parameters.one_line_approximation)
        throw std::runtime_error("One line approximation is currently not supported for imaging.");
    MgrModel* dev = upload();
    const Size P = parameters.npoints_.v, F = parameters.nfreqs_;
    Image im;
    im.imageType = tau ? 1 : 0;
    im.imagePointPosition = 0;
    im.ray_nr = (long)ray_nr;
    im.ray_direction.assign({3}, geometry.rays.direction.data() + 3 * (size_t)ray_nr);
    im.nfreqs = F;
    im.freqs.resize({F});
    for (Size f = 0; f < F; f++) im.freqs[f] = radiation.frequencies.nu[f];  // nu(0, f)
    im.I.resize({P, F});
    im.ImX.resize({P});
    im.ImY.resize({P});
    auto fn = tau ? mgr_image_optical_depth : mgr_image;
    check(fn(dev, parameters.precision, ray_nr, im.I.data(), im.ImX.data(), im.ImY.data()));
    if (parameters.dimension_.v == 1) {
        // Image::set_coordinates_all_model_points, 1D (image.cpp:160-171)
        for (Size p = 0; p < P; p++) {
            im.ImX[p] = geometry.points.position.data()[3 * (size_t)p];
            im.ImY[p] = 0.0;
        }
    }
    images.push_back(std::move(im));
    return 0;
}

// Model::compute_image_for_point (model.cpp:1039-1058 ->
// Solver::image_feautrier_order_2_for_point, solver.tpp:629-653): S_ray, dtau_ray and
// u_ray [n_tot][F] of point p's ray ray_nr.
int Model::compute_image_for_point(Size ray_nr, Size p) {
    if (parameters.one_line_approximation)
        throw std::runtime_error("One line approximation is currently not supported for imaging.");
    MgrModel* dev = upload();
    const Size F = parameters.nfreqs_;
    uint32_t n_tot = 0;
    check(mgr_image_for_point(dev, parameters.precision, ray_nr, p, &n_tot, nullptr, nullptr, nullptr, 0));
    S_ray.resize({n_tot, F});
    dtau_ray.resize({n_tot, F});
    u_ray.resize({n_tot, F});
    check(mgr_image_for_point(dev, parameters.precision, ray_nr, p, &n_tot, S_ray.data(), dtau_ray.data(),
                              u_ray.data(), n_tot));
    return 0;
}

// Model::set_column (model.cpp:1143-1153 -> Solver::set_column, solver.tpp:2953-2991):
// column [nrays][P] of the per-point density.
int Model::set_column() {
    const Size P = parameters.npoints_.v;
    if (density.size() != P) throw std::runtime_error("set_column: density must have npoints entries.");
    MgrModel* dev = upload();
    column.resize({(Size)parameters.nrays_.v, P});
    check(mgr_set_column(dev, density.data(), column.data()));
    return 0;
}

int Model::compute_image_new(Size ray_nr) { return compute_image_new(ray_nr, 256, 256); }

int Model::compute_image_new(Size ray_nr, Size Nxpix, Size Nypix) {
    const double* d = geometry.rays.direction.data() + 3 * (size_t)ray_nr;
    return compute_image_new(d[0], d[1], d[2], Nxpix, Nypix);
}

int Model::compute_image_new(double rx, double ry, double rz, Size Nxpix, Size Nypix) {
    return image_new(rx, ry, rz, Nxpix, Nypix, false);
}

// Model::compute_image_optical_depth_new (model.cpp:1081-1127 ->
// Solver::image_optical_depth_new_imager, solver.tpp:686-736)
int Model::compute_image_optical_depth_new(Size ray_nr) { return compute_image_optical_depth_new(ray_nr, 256, 256); }

int Model::compute_image_optical_depth_new(Size ray_nr, Size Nxpix, Size Nypix) {
    const double* d = geometry.rays.direction.data() + 3 * (size_t)ray_nr;
    return image_new(d[0], d[1], d[2], Nxpix, Nypix, true);
}

int Model::compute_image_optical_depth_new(double rx, double ry, double rz, Size Nxpix, Size Nypix) {
    return image_new(rx, ry, rz, Nxpix, Nypix, true);
}

int Model::image_new(double rx, double ry, double rz, Size Nxpix, Size Nypix, bool tau) {
    if (rx * rx + ry * ry + rz * rz == 0.0)
        throw std::runtime_error(
            "The given ray direction vector does not point in a direction. Please use a non-zero (normed) direction "
            "vector to generate an image.");
    if (parameters.one_line_approximation) throw std::runtime_error("One line approximation is not supported for imaging.");
    MgrModel* dev = upload();
    const Size F = parameters.nfreqs_;
    const size_t npix = (size_t)Nxpix * Nypix;
    const double inv = 1 / std::sqrt(rx * rx + ry * ry + rz * rz);
    const double d[3] = {rx * inv, ry * inv, rz * inv};
    Image im;
    im.imageType = tau ? 1 : 0;
    im.imagePointPosition = 1;
    im.ray_nr = -1;
    im.ray_direction.assign({3}, d);
    im.nfreqs = F;
    im.freqs.resize({F});
    for (Size f = 0; f < F; f++) im.freqs[f] = radiation.frequencies.nu[f];
    im.I.resize({npix, F});
    im.ImX.resize({npix});
    im.ImY.resize({npix});
    auto fn = tau ? mgr_image_optical_depth_new : mgr_image_new;
    check(fn(dev, parameters.precision, d, Nxpix, Nypix, im.I.data(), im.ImX.data(), im.ImY.data()));
    images.push_back(std::move(im));
    return 0;
}

}  // namespace mgrhost
