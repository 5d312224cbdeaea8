// Host-side Model of magritte_gb300: the data a Magritte user sets through the
// Python API (Magritte 0.9.3 src/model/*) and the compute_* entry points of the
// formal-solve path (src/model/model.hpp:58-80).  Set-up arithmetic (spectral
// discretisation, LTE, line widths, dshift_max) runs here on the host exactly as
// the reference states it; the formal solve runs on the GPU through the C ABI
// (include/magritte_gb300.h).
#pragma once
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/magritte_gb300.h"

namespace mgrhost {

using Size = uint32_t;
using Real = double;

// src/tools/constants.hpp:15-40
constexpr double PI = 3.14159265358979323846;
constexpr double CC = 2.99792458E+8;
constexpr double HH = 6.62607004E-34;
constexpr double KB = 1.38064852E-23;
constexpr double AMU = 1.66053904E-27;
constexpr double T_CMB = 2.7254800;
constexpr double CC_SQUARED = 8.98755179E+16;
constexpr double TWO_KB_OVER_AMU_CC_SQUARED = 2.0 * KB / (AMU * CC_SQUARED);
constexpr double HH_OVER_FOUR_PI = HH / (4.0 * PI);

// A contiguous row-major array with a shape; the Python side sees it through the
// buffer protocol (zero copy) and replaces it with set().
template <typename T>
struct Array {
    std::vector<T> vec;
    std::vector<size_t> shape;
    uint64_t version = 0;  // bumped on every set()/resize()

    void resize(std::vector<size_t> s) {
        size_t n = 1;
        for (size_t d : s) n *= d;
        shape = std::move(s);
        vec.assign(n, T());
        version++;
    }
    void assign(std::vector<size_t> s, const T* data) {
        size_t n = 1;
        for (size_t d : s) n *= d;
        shape = std::move(s);
        vec.assign(data, data + n);
        version++;
    }
    size_t size() const { return vec.size(); }
    T* data() { return vec.data(); }
    const T* data() const { return vec.data(); }
    T& operator[](size_t i) { return vec[i]; }
    const T& operator[](size_t i) const { return vec[i]; }
    void touch() { version++; }
};

// Parameters with the reference's set-once behaviour (src/model/parameters/parameters.hpp).
struct SetOnceSize {
    Size v = 0;
    bool set_ = false;
    void set(Size x, const char* name) {
        if (set_ && v != x) throw std::runtime_error(std::string("Parameter ") + name + " was already set to a different value");
        v = x;
        set_ = true;
    }
    Size get(const char* name) const {
        if (!set_) throw std::runtime_error(std::string("Parameter ") + name + " was not set");
        return v;
    }
};

struct Parameters {
    std::string model_name;
    SetOnceSize dimension_, npoints_, nrays_, nboundary_, nspecs_, nlspecs_, nquads_, hnrays_, nlines_;
    Size nfreqs_ = 0;
    bool spherical_symmetry_ = false;

    Size n_off_diag = 0;
    Real max_width_fraction = 0.35;
    Real convergence_fraction = 0.995;
    Real min_rel_pop_for_convergence = 1.0e-10;
    Real pop_prec = 1.0e-6;
    Real min_opacity = 1.0e-26;
    Real min_line_opacity = 1.0e-13;
    Real min_line_emissivity = 1.0e-50;
    Real min_dtau = 1.0e-15;
    Real max_interpolation_diff = 1.4;
    Real population_inversion_fraction = -1.0;
    bool store_intensities = false;
    bool use_adaptive_Ng_acceleration = true;
    Size Ng_acceleration_mem_limit = 9;
    Size adaptive_Ng_acceleration_min_order = 2;
    bool adaptive_Ng_acceleration_use_max_criterion = true;
    Size Ng_acceleration_remove_N_its = 0;
    bool one_line_approximation = false;
    bool sum_opacity_emissivity_over_all_lines = false;
    Real max_distance_opacity_contribution = 10.0;
    // GB300 options (no reference counterpart)
    int precision = MGR_PRECISION_FP64;  // MgrPrecision of the formal solve
    bool store_u = true;                 // copy radiation.u back to the host

    int approx() const {
        if (one_line_approximation) return MGR_APPROX_ONELINE;
        if (sum_opacity_emissivity_over_all_lines) return MGR_APPROX_NONE;
        return MGR_APPROX_CLOSELINES;
    }
};

struct Points {
    Array<double> position;  // [P][3]
    Array<double> velocity;  // [P][3] v/c
    Array<Size> neighbors;
    Array<Size> n_neighbors;
    Array<Size> cum_n_neighbors;
};

struct Rays {
    Array<double> direction;  // [nrays][3]
    Array<double> weight;     // [nrays]
    Array<Size> antipod;      // [nrays]
    bool use_adaptive_directions = false;
};

enum BoundaryCondition { Zero = 0, Thermal = 1, CMB = 2 };

struct Boundary {
    Array<Size> boundary2point;
    Array<Size> point2boundary;
    Array<int32_t> boundary_condition;
    Array<double> boundary_temperature;
};

struct Geometry {
    Points points;
    Rays rays;
    Boundary boundary;
};

struct Species {
    Array<double> abundance;  // [P][nspecs]
    std::vector<std::string> symbol;
};

struct Chemistry {
    Species species;
};

struct Temperature {
    Array<double> gas;  // [P]
};
struct Turbulence {
    Array<double> vturb2;  // [P] (v_turb/c)^2
};
struct Thermodynamics {
    Temperature temperature;
    Turbulence turbulence;
};

struct CollisionPartner {
    Size num_col_partner = 0;
    std::string orth_or_para_H2 = "n";
    Size ncol = 0, ntmp = 0;
    std::vector<Size> icol, jcol;
    std::vector<double> tmp;
    std::vector<std::vector<double>> Cd, Ce;  // [ntmp][ncol]
};

struct Linedata {
    Size num = 0;
    std::string sym;
    double inverse_mass = 1.0;
    Size nlev = 0, nrad = 0;
    std::vector<Size> irad, jrad;
    std::vector<double> energy, weight, frequency, A, Ba, Bs;
    std::vector<CollisionPartner> colpar;
};

struct Quadrature {
    Array<double> roots;
    Array<double> weights;
};

struct LineProducingSpecies {
    Linedata linedata;
    Quadrature quadrature;
    Array<double> population;      // [P*nlev]
    Array<double> population_tot;  // [P]
    Array<double> J;                 // [P][nrad] line-integrated J of the memory-lean / anisotropic solves
    Array<double> J2_0, J2_1_Re, J2_1_Im, J2_2_Re, J2_2_Im;  // [P][nrad] anisotropy tensor elements
    Array<double> Jlin, Jeff, Jdif;  // [P][nrad]
    Array<double> lambda_diag;     // [P][nrad] summed diagonal ALO
    Array<uint8_t> lambda_has;     // [P][nrad]
    double relative_change_mean = 0.0, relative_change_max = 0.0, fraction_not_converged = 0.0;
    Size index(Size p, Size i) const { return i + p * linedata.nlev; }
};

struct Lines {
    std::vector<LineProducingSpecies> lineProducingSpecies;
    void resize_LineProducingSpecies(size_t n) { lineProducingSpecies.resize(n); }
    Array<double> line;
    Array<Size> nrad_cum;
    Array<double> sorted_line;
    Array<Size> sorted_line_map;
    double max_inverse_mass = 0.0;
    Array<double> emissivity, opacity, inverse_width;  // [P][L]
};

struct Frequencies {
    Array<double> nu;  // [P][F]
    Array<Size> corresponding_line, corresponding_l_for_spec, corresponding_k_for_tran, corresponding_z_for_line;
    Array<uint8_t> appears_in_line_integral;
};

struct Radiation {
    Frequencies frequencies;
    Array<double> J;  // [P][F]
    Array<double> u;  // [hnrays][P][F]
    Array<double> v;  // [hnrays][P][F] (short characteristics)
    Array<double> I;  // [nrays][P][F]  (short characteristics)
};

// One image (src/model/image/image.hpp:30-60): intensities I [npix][nfreqs] and the
// image-plane coordinates of the pixels.
struct Image {
    int imageType = 0;           // 0 Intensity, 1 OpticalDepth
    int imagePointPosition = 0;  // 0 AllModelPoints (old imager), 1 ProjectionSurface
    long ray_nr = -1;
    Array<double> ray_direction;  // [3]
    Array<double> ImX, ImY;       // [npix]
    Array<double> I;              // [npix][nfreqs]
    Array<double> freqs;          // [nfreqs]
    Size nfreqs = 0;
};

class Model {
   public:
    Parameters parameters;
    Geometry geometry;
    Chemistry chemistry;
    Thermodynamics thermodynamics;
    Lines lines;
    Radiation radiation;
    Array<double> dshift_max;
    std::vector<double> error_max, error_mean;
    std::vector<Image> images;
    Array<double> S_ray, dtau_ray, u_ray;  // [n_tot][F] of compute_image_for_point (model.hpp:97-99)
    Array<double> density;                 // [P], set by the caller (model.hpp:118)
    Array<double> column;                  // [nrays][P] of set_column (model.hpp:119)

    enum SpectralDiscretisation { SD_None, SD_Lines, SD_Image } spectralDiscretisation = SD_None;

    Model() = default;
    ~Model();
    Model(const Model&) = delete;
    Model& operator=(const Model&) = delete;

    // Derived data the reference computes while reading a model (Points::read,
    // Rays::read, Boundary::read, Lines::read, LineProducingSpecies::read).
    void prepare();

    int compute_inverse_line_widths();
    int compute_spectral_discretisation();
    int compute_spectral_discretisation(Real width);
    int compute_spectral_discretisation(Real nu_min, Real nu_max);
    int compute_spectral_discretisation(Real nu_min, Real nu_max, Size n_image_freqs);
    int compute_LTE_level_populations();
    int set_dshift_max();
    int compute_radiation_field_feautrier_order_2();
    int compute_radiation_field_shortchar_order_0();
    int compute_image(Size ray_nr);
    int compute_image_new(Size ray_nr);
    int compute_image_new(Size ray_nr, Size Nxpix, Size Nypix);
    int compute_image_new(double rx, double ry, double rz, Size Nxpix, Size Nypix);
    int compute_image_optical_depth(Size ray_nr);
    int compute_image_optical_depth_new(Size ray_nr);
    int compute_image_optical_depth_new(Size ray_nr, Size Nxpix, Size Nypix);
    int compute_image_optical_depth_new(double rx, double ry, double rz, Size Nxpix, Size Nypix);
    int compute_image_for_point(Size ray_nr, Size p);
    int set_column();
    int compute_Jeff();
    int compute_level_populations(bool use_Ng_acceleration, long max_niterations);
    int compute_radiation_field_feautrier_order_2_sparse();
    int compute_radiation_field_feautrier_order_2_anis();
    int compute_radiation_field_feautrier_order_2_uv();
    int compute_Jeff_sparse();
    int compute_level_populations_sparse(bool use_Ng_acceleration, long max_niterations);

    // Device management (GB300): the MgrModel mirroring this Model.
    // upload(): prepare, dshift_max, and (re)create or refresh the device model.
    MgrModel* upload();
    void release_device();
    MgrModel* device_model();
    uint64_t launches() const;
    // Device time of each ALI phase in the latest compute_level_populations call
    // (formal solve, Jeff, rate equations + corrections + line refresh, Ng), in ms;
    // empty without a timed loop on the current device model.
    std::vector<double> ali_phase_times() const;

   private:
    MgrModel* dev_ = nullptr;
    uint64_t dev_signature_ = 0;
    std::vector<double> crit_;
    uint64_t signature() const;
    void fill_desc(MgrModelDesc& d);
    void attach_species();
    void store_lambda(const std::vector<double>& lam);
    int run_ali(bool use_Ng_acceleration, long max_niterations, bool sparse);
    int image_old(Size ray_nr, bool tau);
    int image_new(double rx, double ry, double rz, Size Nxpix, Size Nypix, bool tau);
    void set_emissivity_and_opacity();
};

}  // namespace mgrhost
