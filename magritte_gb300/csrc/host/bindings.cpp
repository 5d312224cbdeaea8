// pybind11 module magritte_gb300.core: the Python surface of the host Model,
// mirroring magritte.core (Magritte 0.9.3 src/bindings/pybindings.cpp:20-1113):
// nested data structs, buffer-protocol arrays with set(), and the compute_* calls.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>
#include <pybind11/stl_bind.h>

#include "model.hpp"

namespace py = pybind11;
using namespace mgrhost;

PYBIND11_MAKE_OPAQUE(std::vector<LineProducingSpecies>);
PYBIND11_MAKE_OPAQUE(std::vector<CollisionPartner>);

template <typename T>
static void bind_array(py::module_& m, const char* name) {
    py::class_<Array<T>>(m, name, py::buffer_protocol())
        .def(py::init<>())
        .def_buffer([](Array<T>& a) -> py::buffer_info {
            std::vector<py::ssize_t> shape(a.shape.begin(), a.shape.end());
            if (shape.empty()) shape.push_back(0);
            std::vector<py::ssize_t> strides(shape.size());
            py::ssize_t s = sizeof(T);
            for (int i = (int)shape.size() - 1; i >= 0; i--) {
                strides[i] = s;
                s *= shape[i];
            }
            return py::buffer_info(a.data(), sizeof(T), py::format_descriptor<T>::format(), (py::ssize_t)shape.size(),
                                   shape, strides);
        })
        .def("set",
             [](Array<T>& a, py::object obj) {
                 auto arr = py::array_t<T, py::array::c_style | py::array::forcecast>::ensure(obj);
                 if (!arr) throw std::runtime_error("set(): argument is not convertible to an array");
                 std::vector<size_t> shape(arr.shape(), arr.shape() + arr.ndim());
                 a.assign(shape, arr.data());
             })
        .def("size", [](const Array<T>& a) { return a.size(); })
        .def_property_readonly("shape", [](const Array<T>& a) { return a.shape; });
}

#define SETONCE(name) \
    .def("set_" #name, [](Parameters& p, Size v) { p.name##_.set(v, #name); }) \
    .def(#name, [](const Parameters& p) { return p.name##_.get(#name); })

PYBIND11_MODULE(core, m) {
    m.doc() = "GB300-native formal-solve path of Magritte: host Model over libmgr_gpu.so";
    m.attr("CC") = CC;
    m.attr("HH") = HH;
    m.attr("KB") = KB;
    m.attr("AMU") = AMU;
    m.attr("T_CMB") = T_CMB;

    bind_array<double>(m, "ArrayReal");
    bind_array<uint32_t>(m, "ArraySize");
    bind_array<int32_t>(m, "ArrayInt");
    bind_array<uint8_t>(m, "ArrayBool");

    py::enum_<BoundaryCondition>(m, "BoundaryCondition")
        .value("Zero", Zero)
        .value("Thermal", Thermal)
        .value("CMB", CMB)
        .export_values();

    py::class_<Parameters>(m, "Parameters")
        .def(py::init<>())
        SETONCE(dimension) SETONCE(npoints) SETONCE(nrays) SETONCE(nboundary) SETONCE(nspecs) SETONCE(nlspecs)
        SETONCE(nquads)
        .def("hnrays", [](const Parameters& p) { return p.hnrays_.get("hnrays"); })
        .def("nlines", [](const Parameters& p) { return p.nlines_.get("nlines"); })
        .def("nfreqs", [](const Parameters& p) { return p.nfreqs_; })
        .def("set_nfreqs", [](Parameters& p, Size v) { p.nfreqs_ = v; })
        .def("set_spherical_symmetry", [](Parameters& p, bool v) { p.spherical_symmetry_ = v; })
        .def("spherical_symmetry", [](const Parameters& p) { return p.spherical_symmetry_; })
        .def("set_model_name", [](Parameters& p, std::string s) { p.model_name = s; })
        .def("model_name", [](const Parameters& p) { return p.model_name; })
        .def_readwrite("n_off_diag", &Parameters::n_off_diag)
        .def_readwrite("max_width_fraction", &Parameters::max_width_fraction)
        .def_readwrite("convergence_fraction", &Parameters::convergence_fraction)
        .def_readwrite("min_rel_pop_for_convergence", &Parameters::min_rel_pop_for_convergence)
        .def_readwrite("pop_prec", &Parameters::pop_prec)
        .def_readwrite("min_opacity", &Parameters::min_opacity)
        .def_readwrite("min_line_opacity", &Parameters::min_line_opacity)
        .def_readwrite("min_line_emissivity", &Parameters::min_line_emissivity)
        .def_readwrite("min_dtau", &Parameters::min_dtau)
        .def_readwrite("max_interpolation_diff", &Parameters::max_interpolation_diff)
        .def_readwrite("population_inversion_fraction", &Parameters::population_inversion_fraction)
        .def_readwrite("store_intensities", &Parameters::store_intensities)
        .def_readwrite("use_adaptive_Ng_acceleration", &Parameters::use_adaptive_Ng_acceleration)
        .def_readwrite("Ng_acceleration_mem_limit", &Parameters::Ng_acceleration_mem_limit)
        .def_readwrite("adaptive_Ng_acceleration_min_order", &Parameters::adaptive_Ng_acceleration_min_order)
        .def_readwrite("adaptive_Ng_acceleration_use_max_criterion",
                       &Parameters::adaptive_Ng_acceleration_use_max_criterion)
        .def_readwrite("Ng_acceleration_remove_N_its", &Parameters::Ng_acceleration_remove_N_its)
        .def_readwrite("one_line_approximation", &Parameters::one_line_approximation)
        .def_readwrite("sum_opacity_emissivity_over_all_lines", &Parameters::sum_opacity_emissivity_over_all_lines)
        .def_readwrite("max_distance_opacity_contribution", &Parameters::max_distance_opacity_contribution)
        .def_property(
            "precision", [](const Parameters& p) { return p.precision == MGR_PRECISION_SPLIT ? "split" : "fp64"; },
            [](Parameters& p, std::string s) {
                if (s == "fp64") p.precision = MGR_PRECISION_FP64;
                else if (s == "split") p.precision = MGR_PRECISION_SPLIT;
                else throw std::runtime_error("precision must be 'fp64' or 'split'");
            })
        .def_readwrite("store_u", &Parameters::store_u);

    py::class_<Points>(m, "Points")
        .def_readwrite("position", &Points::position)
        .def_readwrite("velocity", &Points::velocity)
        .def_readwrite("neighbors", &Points::neighbors)
        .def_readwrite("n_neighbors", &Points::n_neighbors)
        .def_readwrite("cum_n_neighbors", &Points::cum_n_neighbors);

    py::class_<Rays>(m, "Rays")
        .def_readwrite("direction", &Rays::direction)
        .def_readwrite("weight", &Rays::weight)
        .def_readwrite("antipod", &Rays::antipod)
        .def_readwrite("use_adaptive_directions", &Rays::use_adaptive_directions);

    py::class_<Boundary>(m, "Boundary")
        .def_readwrite("boundary2point", &Boundary::boundary2point)
        .def_readwrite("point2boundary", &Boundary::point2boundary)
        .def_readwrite("boundary_temperature", &Boundary::boundary_temperature)
        .def_readwrite("boundary_condition", &Boundary::boundary_condition)
        .def("set_boundary_condition",
             [](Boundary& b, Size i, BoundaryCondition c) {
                 if (b.boundary_condition.size() != b.boundary2point.size()) {
                     std::vector<int32_t> v(b.boundary2point.size(), CMB);
                     b.boundary_condition.assign({v.size()}, v.data());
                 }
                 if (i >= b.boundary_condition.size()) throw std::runtime_error("boundary index out of range");
                 b.boundary_condition[i] = (int32_t)c;
                 b.boundary_condition.touch();
                 return c;
             })
        .def("get_boundary_condition", [](const Boundary& b, Size i) { return (BoundaryCondition)b.boundary_condition[i]; });

    py::class_<Geometry>(m, "Geometry")
        .def_readwrite("points", &Geometry::points)
        .def_readwrite("rays", &Geometry::rays)
        .def_readwrite("boundary", &Geometry::boundary);

    py::class_<Species>(m, "Species")
        .def_property(
            "abundance", [](Species& s) -> Array<double>& { return s.abundance; },
            [](Species& s, py::object obj) {
                auto arr = py::array_t<double, py::array::c_style | py::array::forcecast>::ensure(obj);
                if (!arr || arr.ndim() != 2) throw std::runtime_error("abundance must be [npoints][nspecs]");
                s.abundance.assign({(size_t)arr.shape(0), (size_t)arr.shape(1)}, arr.data());
            },
            py::return_value_policy::reference_internal)
        .def_readwrite("symbol", &Species::symbol);

    py::class_<Chemistry>(m, "Chemistry").def_readwrite("species", &Chemistry::species);
    py::class_<Temperature>(m, "Temperature").def_readwrite("gas", &Temperature::gas);
    py::class_<Turbulence>(m, "Turbulence").def_readwrite("vturb2", &Turbulence::vturb2);
    py::class_<Thermodynamics>(m, "Thermodynamics")
        .def_readwrite("temperature", &Thermodynamics::temperature)
        .def_readwrite("turbulence", &Thermodynamics::turbulence);

    py::class_<CollisionPartner>(m, "CollisionPartner")
        .def(py::init<>())
        .def_readwrite("num_col_partner", &CollisionPartner::num_col_partner)
        .def_readwrite("orth_or_para_H2", &CollisionPartner::orth_or_para_H2)
        .def_readwrite("ncol", &CollisionPartner::ncol)
        .def_readwrite("ntmp", &CollisionPartner::ntmp)
        .def_readwrite("icol", &CollisionPartner::icol)
        .def_readwrite("jcol", &CollisionPartner::jcol)
        .def_readwrite("tmp", &CollisionPartner::tmp)
        .def_readwrite("Cd", &CollisionPartner::Cd)
        .def_readwrite("Ce", &CollisionPartner::Ce);
    py::bind_vector<std::vector<CollisionPartner>>(m, "vCollisionPartner");

    py::class_<Linedata>(m, "Linedata")
        .def(py::init<>())
        .def_readwrite("num", &Linedata::num)
        .def_readwrite("sym", &Linedata::sym)
        .def_readwrite("inverse_mass", &Linedata::inverse_mass)
        .def_readwrite("nlev", &Linedata::nlev)
        .def_readwrite("nrad", &Linedata::nrad)
        .def_readwrite("irad", &Linedata::irad)
        .def_readwrite("jrad", &Linedata::jrad)
        .def_readwrite("energy", &Linedata::energy)
        .def_readwrite("weight", &Linedata::weight)
        .def_readwrite("frequency", &Linedata::frequency)
        .def_readwrite("A", &Linedata::A)
        .def_readwrite("Ba", &Linedata::Ba)
        .def_readwrite("Bs", &Linedata::Bs)
        .def_readwrite("colpar", &Linedata::colpar);

    py::class_<Quadrature>(m, "Quadrature")
        .def_readwrite("roots", &Quadrature::roots)
        .def_readwrite("weights", &Quadrature::weights);

    py::class_<LineProducingSpecies>(m, "LineProducingSpecies")
        .def(py::init<>())
        .def_readwrite("linedata", &LineProducingSpecies::linedata)
        .def_readwrite("quadrature", &LineProducingSpecies::quadrature)
        .def_readwrite("population", &LineProducingSpecies::population)
        .def_readwrite("population_tot", &LineProducingSpecies::population_tot)
        .def_readwrite("J", &LineProducingSpecies::J)
        .def_readwrite("J2_0", &LineProducingSpecies::J2_0)
        .def_readwrite("J2_1_Re", &LineProducingSpecies::J2_1_Re)
        .def_readwrite("J2_1_Im", &LineProducingSpecies::J2_1_Im)
        .def_readwrite("J2_2_Re", &LineProducingSpecies::J2_2_Re)
        .def_readwrite("J2_2_Im", &LineProducingSpecies::J2_2_Im)
        .def_readwrite("Jlin", &LineProducingSpecies::Jlin)
        .def_readwrite("Jeff", &LineProducingSpecies::Jeff)
        .def_readwrite("Jdif", &LineProducingSpecies::Jdif)
        .def_readwrite("lambda_diag", &LineProducingSpecies::lambda_diag)
        .def_readonly("relative_change_mean", &LineProducingSpecies::relative_change_mean)
        .def_readonly("relative_change_max", &LineProducingSpecies::relative_change_max)
        .def_readonly("fraction_not_converged", &LineProducingSpecies::fraction_not_converged);
    py::bind_vector<std::vector<LineProducingSpecies>>(m, "vLineProducingSpecies");

    py::class_<Lines>(m, "Lines")
        .def_readwrite("lineProducingSpecies", &Lines::lineProducingSpecies)
        .def("resize_LineProducingSpecies", &Lines::resize_LineProducingSpecies)
        .def_readwrite("line", &Lines::line)
        .def_readwrite("sorted_line", &Lines::sorted_line)
        .def_readwrite("sorted_line_map", &Lines::sorted_line_map)
        .def_readwrite("emissivity", &Lines::emissivity)
        .def_readwrite("opacity", &Lines::opacity)
        .def_readwrite("inverse_width", &Lines::inverse_width);

    py::class_<Frequencies>(m, "Frequencies")
        .def_readwrite("nu", &Frequencies::nu)
        .def_readwrite("corresponding_line", &Frequencies::corresponding_line)
        .def_readwrite("appears_in_line_integral", &Frequencies::appears_in_line_integral);

    py::class_<Radiation>(m, "Radiation")
        .def_readwrite("frequencies", &Radiation::frequencies)
        .def_readwrite("J", &Radiation::J)
        .def_readwrite("u", &Radiation::u)
        .def_readwrite("v", &Radiation::v)
        .def_readwrite("I", &Radiation::I);

    py::class_<Image>(m, "Image")
        .def_readonly("imageType", &Image::imageType)
        .def_readonly("imagePointPosition", &Image::imagePointPosition)
        .def_readonly("ray_nr", &Image::ray_nr)
        .def_readwrite("ray_direction", &Image::ray_direction)
        .def_readwrite("ImX", &Image::ImX)
        .def_readwrite("ImY", &Image::ImY)
        .def_readwrite("I", &Image::I)
        .def_readwrite("freqs", &Image::freqs)
        .def_readonly("nfreqs", &Image::nfreqs);

    py::class_<Model>(m, "Model")
        .def(py::init<>())
        .def_readwrite("parameters", &Model::parameters)
        .def_readwrite("geometry", &Model::geometry)
        .def_readwrite("chemistry", &Model::chemistry)
        .def_readwrite("thermodynamics", &Model::thermodynamics)
        .def_readwrite("lines", &Model::lines)
        .def_readwrite("radiation", &Model::radiation)
        .def_readwrite("dshift_max", &Model::dshift_max)
        .def_readonly("error_max", &Model::error_max)
        .def_readonly("error_mean", &Model::error_mean)
        .def("prepare", &Model::prepare)
        .def("compute_inverse_line_widths", &Model::compute_inverse_line_widths)
        .def("compute_spectral_discretisation", py::overload_cast<>(&Model::compute_spectral_discretisation))
        .def("compute_spectral_discretisation", py::overload_cast<Real>(&Model::compute_spectral_discretisation))
        .def("compute_spectral_discretisation",
             py::overload_cast<Real, Real>(&Model::compute_spectral_discretisation))
        .def("compute_spectral_discretisation",
             py::overload_cast<Real, Real, Size>(&Model::compute_spectral_discretisation))
        .def("compute_LTE_level_populations", &Model::compute_LTE_level_populations)
        .def("set_dshift_max", &Model::set_dshift_max)
        .def("compute_radiation_field_feautrier_order_2", &Model::compute_radiation_field_feautrier_order_2,
             py::call_guard<py::gil_scoped_release>())
        .def("compute_radiation_field_shortchar_order_0", &Model::compute_radiation_field_shortchar_order_0,
             py::call_guard<py::gil_scoped_release>())
        .def("compute_Jeff", &Model::compute_Jeff, py::call_guard<py::gil_scoped_release>())
        .def("compute_image", &Model::compute_image, py::call_guard<py::gil_scoped_release>())
        .def("compute_image_new", py::overload_cast<Size>(&Model::compute_image_new),
             py::call_guard<py::gil_scoped_release>())
        .def("compute_image_new", py::overload_cast<Size, Size, Size>(&Model::compute_image_new),
             py::call_guard<py::gil_scoped_release>())
        .def("compute_image_new", py::overload_cast<double, double, double, Size, Size>(&Model::compute_image_new),
             py::call_guard<py::gil_scoped_release>())
        .def("compute_image_optical_depth", &Model::compute_image_optical_depth,
             py::call_guard<py::gil_scoped_release>())
        .def("compute_image_optical_depth_new", py::overload_cast<Size>(&Model::compute_image_optical_depth_new),
             py::call_guard<py::gil_scoped_release>())
        .def("compute_image_optical_depth_new",
             py::overload_cast<Size, Size, Size>(&Model::compute_image_optical_depth_new),
             py::call_guard<py::gil_scoped_release>())
        .def("compute_image_optical_depth_new",
             py::overload_cast<double, double, double, Size, Size>(&Model::compute_image_optical_depth_new),
             py::call_guard<py::gil_scoped_release>())
        .def_readonly("images", &Model::images)
        .def_readonly("S_ray", &Model::S_ray)
        .def_readonly("dtau_ray", &Model::dtau_ray)
        .def_readonly("u_ray", &Model::u_ray)
        .def_readwrite("density", &Model::density)
        .def_readwrite("column", &Model::column)
        .def("compute_image_for_point", &Model::compute_image_for_point, py::call_guard<py::gil_scoped_release>())
        .def("set_column", &Model::set_column, "Set column (internally).", py::call_guard<py::gil_scoped_release>())
        .def("compute_level_populations", &Model::compute_level_populations, py::arg("use_Ng_acceleration"),
             py::arg("max_niterations"), py::call_guard<py::gil_scoped_release>())
        .def("compute_radiation_field_feautrier_order_2_sparse",
             &Model::compute_radiation_field_feautrier_order_2_sparse, py::call_guard<py::gil_scoped_release>())
        .def("compute_Jeff_sparse", &Model::compute_Jeff_sparse, py::call_guard<py::gil_scoped_release>())
        .def("compute_radiation_field_feautrier_order_2_anis", &Model::compute_radiation_field_feautrier_order_2_anis,
             py::call_guard<py::gil_scoped_release>())
        .def("compute_radiation_field_feautrier_order_2_uv", &Model::compute_radiation_field_feautrier_order_2_uv,
             py::call_guard<py::gil_scoped_release>())
        .def("compute_level_populations_sparse", &Model::compute_level_populations_sparse,
             py::arg("use_Ng_acceleration"), py::arg("max_niterations"), py::call_guard<py::gil_scoped_release>())
        .def_readonly("error_mean", &Model::error_mean)
        .def_readonly("error_max", &Model::error_max)
        .def("release_device", &Model::release_device)
        .def("upload", [](Model& m) { return (uintptr_t)m.upload(); },
             "Upload (or refresh) the device model; returns the MgrModel* handle as an integer")
        .def("gpu_launches", &Model::launches)
        .def("ali_phase_times", &Model::ali_phase_times,
             "Device ms of the latest ALI loop's phases: formal solve, Jeff, rate equations + corrections + "
             "line refresh, Ng steps (empty list without a timed loop)");
}
