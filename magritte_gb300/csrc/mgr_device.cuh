// Device-side model, physics and ray tracing for the Magritte formal-solve path.
//
// Every function restates one reference statement (Magritte 0.9.3 paths given per
// function).  Precision policy:
//   * Ray tracing (neighbour choice, Z, dZ, Doppler shift, interpolation split) uses
//     explicitly rounded FP64 operations (__dmul_rn/__dadd_rn) so that no multiply-add
//     is contracted: point sequences are bit-identical to the reference's FP64 CPU code.
//   * MGR_PRECISION_FP64 follows the reference's arithmetic: FP64 with the reference's
//     single-precision libm calls (expf, erff, logf, powf, expm1f).
//   * MGR_PRECISION_SPLIT evaluates profiles, opacities, sources and optical depths in
//     FP32 (frequencies as FP32 offsets from the line centre, so no catastrophic
//     cancellation), and keeps the Feautrier elimination in FP64.
#pragma once
#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

#include <cmath>
#include <math.h>

// Functions marked MGR_HD are compiled for the GPU and, for the CPU emulation used by
// the test-suite, for the host.
#define MGR_HD __host__ __device__ __forceinline__

namespace mgr {

// src/tools/constants.hpp:15-40
constexpr double INVERSE_SQRT_PI = 0.5 * 1.12837916709551257390;
constexpr double CC = 2.99792458E+8;
constexpr double HH = 6.62607004E-34;
constexpr double KB = 1.38064852E-23;
constexpr double AMU = 1.66053904E-27;
constexpr double T_CMB = 2.7254800;
constexpr double CC_SQUARED = 8.98755179E+16;
constexpr double TWO_KB_OVER_AMU_CC_SQUARED = 2.0 * KB / (AMU * CC_SQUARED);
constexpr double TWO_HH_OVER_CC_SQUARED = 2.0 * HH / CC_SQUARED;
constexpr double HH_OVER_KB = HH / KB;

enum { APPROX_NONE = 0, APPROX_ONELINE = 1, APPROX_CLOSELINES = 2 };
enum { BC_ZERO = 0, BC_THERMAL = 1, BC_CMB = 2 };
enum { MODE_FP64 = 0, MODE_SPLIT = 1 };

// Kernel-side status bits (combined with atomicOr; decoded by the host).
enum : int { ST_TRACE = 1, ST_CAPACITY = 2, ST_NONFINITE = 4 };

// Device-resident model.  Per-(point, line) tables are [P][L] (index l + p*L).
struct DevModel {
    uint32_t P, nrays, hnrays, L, Q, F, nlspecs, B;
    const double4_32a* pos;      // [P] x, y, z
    const double4_32a* vel;      // [P] vx, vy, vz (v/c)
    const uint32_t* n_nb;    // [P]
    const uint32_t* cum_nb;  // [P]
    const double4_32a* edge;     // [E] neighbour position x, y, z and its index (bits of w)
    // FP32 copies for the trace's next-point filter: edge_hl[2i] = neighbour position
    // times pos_scale as floats (hi) with its index in the bits of w, edge_hl[2i + 1] the
    // rounding remainders (lo); pos_hl the same per point.  pos_scale is the power of
    // two that brings every coordinate into [-1, 1].
    const float4* edge_hl;       // [E][2]
    const float4* pos_hl;        // [P][2]
    double pos_scale;
    const uint32_t* p2b;     // [P]
    const int32_t* bc;       // [B]
    const double* bt;        // [B]
    const float* bkt;        // [B][2] h / (k T) of each boundary (T_CMB for CMB) as a double-float (hi, lo)
    const double* raydir;    // [nrays][3]
    const double* rayw;      // [nrays]
    const uint32_t* antipod; // [nrays]
    const double* line;      // [L]
    const double* sorted_line;
    const uint32_t* sorted_map;
    double max_inv_mass;
    const double* em;        // emissivity
    const double* op;        // opacity
    const double* iw;        // inverse width
    const double* Sp;        // emissivity / opacity, the reference's per-call quotient
    const double* crit;      // interpolation criterion opacity / population_tot
    const uint16_t* nint;    // [E][L] interpolation count of each CSR edge (crt -> nxt) per line
    const uint16_t* nint_all;// [E] the same over all lines (imagers)
    const float* em_f;
    const float* op_f;
    const float* iw_f;
    const float* Sp_f;
    const double* ub;        // [P] sqrt(2 kB/(amu c^2) max_inv_mass T + vturb2)
    const float* ub_f;       // [P] (float)ub
    const double* T;         // [P]
    const double* vt2;       // [P]
    const double* dshift_max;// [P]
    const float* dshift_max_f;
    const double* nu;        // [P][F]
    const uint32_t* corr_line;
    const uint32_t* corr_lspec;
    const uint32_t* corr_k;
    const uint32_t* corr_z;
    const uint8_t* in_line;
    const uint32_t* nrad_cum;
    const double* line_A;        // [L]
    const double* lspec_inv_mass;// [nlspecs]
    const double* quad_w;        // [nlspecs][Q]
    double min_opacity;
    double min_dtau;
    double max_interp_diff;
    double max_dist;
    float log_max_interp_diff;   // logf((float)max_interp_diff)
    const uint32_t* lq2f;        // [L][Q] frequency of (line, quadrature point), ~0u if none
    // Split precision keeps FP32 line data in scaled units (exact powers of two):
    // em_f = em * Ke, op_f = op * Ko, Sp_f = Sp * Ke / Ko.
    // Low parts of double-float copies (value = hi + lo, about 48 significant bits) for
    // split precision's same-wing erf arguments: the line centres [L][2] (hi, lo) and
    // the inverse widths iw - (double)iw_f [P][L].
    const float* line_df;
    const float* iw_lo;
    // (float)erf((double)x) for every float x in [kErfBandLo, 3.919206), indexed by the
    // bit pattern of x minus that of kErfBandLo (one table per device, owned by the library)
    const float* erf_band;
    const float* dls;            // [L][L] (float)(sorted_line[s] - line[l0]) at l0*L + s
    const float* dll;            // [L][L] (float)(line[l] - line[l0]) at l0*L + l
    float max_dist_f;            // (float)max_dist
    float min_op_s;              // min_opacity * Ko
    float dz_scale;              // 1 / Ko  (true optical depth = chi_f * dz * dz_scale)
    float s_scale;               // Ko / Ke (true source = scaled source * s_scale)
    int approx;
    uint32_t n_off_diag;  // Parameters::n_off_diag: band elements of the non-local ALO (0: diagonal only)
    uint32_t sph;                // 1D spherical symmetry (Parameters::spherical_symmetry)
    uint32_t adaptive;           // Rays::use_adaptive_directions: raydir [P][nrays][3], rayw [P][nrays]
};

// Rays::get_direction / get_weight (rays.cpp:94-146) of ray r at origin o: per point
// with adaptive directions, else shared.  The formal solves and set_column use these;
// the imagers index raydir + 3 r as the reference's get_direction<false> does.
MGR_HD const double* ray_dir(const DevModel& m, uint32_t o, uint32_t r) {
    return m.raydir + 3 * (m.adaptive ? (size_t)o * m.nrays + r : (size_t)r);
}
MGR_HD double ray_w(const DevModel& m, uint32_t o, uint32_t r) {
    return m.rayw[m.adaptive ? (size_t)o * m.nrays + r : (size_t)r];
}

// ---------------------------------------------------------------------------------
// Exactly rounded FP64 helpers for the trace (no contraction into FMA).  The host
// build of these headers is compiled with -ffp-contract=off.
// ---------------------------------------------------------------------------------
MGR_HD double dadd_rn(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
MGR_HD double dsub_rn(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
MGR_HD double dmul_rn(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}

MGR_HD double ddiv_rn(double a, double b) {
#ifdef __CUDA_ARCH__
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}
MGR_HD double dsqrt_rn(double a) {
#ifdef __CUDA_ARCH__
    return __dsqrt_rn(a);
#else
    return std::sqrt(a);
#endif
}

// FP32 quotient without IEEE division: on the device the approximate __fdividef
// (2 ulp for |b| < 2^126; callers keep b in that range).
MGR_HD float fast_div(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fdividef(a, b);
#else
    return a / b;
#endif
}

MGR_HD double dot3_rn(double ax, double ay, double az, double bx, double by, double bz) {
    return dadd_rn(dadd_rn(dmul_rn(ax, bx), dmul_rn(ay, by)), dmul_rn(az, bz));
}

// Geometry::get_shift_general_geometry<CoMoving> (geometry.tpp:203-207):
// 1 + (v[c] - v[o]) . n
MGR_HD double shift_comoving(const DevModel& m, uint32_t o, uint32_t c, const double* d) {
    const double4_32a vc = m.vel[c];
    const double4_32a vo = m.vel[o];
    return dadd_rn(1.0, dot3_rn(dsub_rn(vc.x, vo.x), dsub_rn(vc.y, vo.y), dsub_rn(vc.z, vo.z), d[0], d[1], d[2]));
}

// Geometry::get_shift_general_geometry<Rest> and its reversal for r >= hnrays
// (geometry.tpp:209-221, :428-465).
MGR_HD double shift_rest(const DevModel& m, uint32_t r, uint32_t c, const double* d) {
    const double4_32a vc = m.vel[c];
    double s = dadd_rn(1.0, dot3_rn(vc.x, vc.y, vc.z, d[0], d[1], d[2]));
    if (r >= m.hnrays) s = dsub_rn(2.0, s);
    return s;
}

// ---------------------------------------------------------------------------------
// 1D spherical symmetry (Parameters::spherical_symmetry): points are shells on the x
// axis in ascending radius, rays lie in the x-y plane.
// ---------------------------------------------------------------------------------
MGR_HD double sqnorm_rn(const double4_32a& a) { return dot3_rn(a.x, a.y, a.z, a.x, a.y, a.z); }

// Geometry::get_shift_spherical_symmetry<CoMoving|Rest> (geometry.tpp:378-417) of point c
// at distance Z along ray r (direction d) from origin o, reversed for r >= hnrays in the
// rest frame (geometry.tpp:428-465).  frame: 0 CoMoving, 1 Rest.
MGR_HD double shift_sph(const DevModel& m, int frame, uint32_t o, uint32_t r, uint32_t c, double Z,
                        const double* d) {
    const double4_32a po = m.pos[o];
    const double xc = m.pos[c].x;
    double s;
    if (frame == 0) {
        if (sqnorm_rn(po) == 0.0) return 1.0;
        const double4_32a vo = m.vel[o];
        const double vd = dot3_rn(vo.x, vo.y, vo.z, d[0], d[1], d[2]);
        if (xc == 0.0) return dsub_rn(1.0, vd);
        const double RcZ = dadd_rn(dot3_rn(po.x, po.y, po.z, d[0], d[1], d[2]), Z);
        s = dadd_rn(1.0, dsub_rn(ddiv_rn(dmul_rn(m.vel[c].x, RcZ), xc), vd));
    } else {
        if (xc == 0.0) {
            s = 1.0;
        } else {
            const double RcZ = dadd_rn(dot3_rn(po.x, po.y, po.z, d[0], d[1], d[2]), Z);
            s = dadd_rn(1.0, ddiv_rn(dmul_rn(m.vel[c].x, RcZ), xc));
        }
        if (r >= m.hnrays) s = dsub_rn(2.0, s);
    }
    return s;
}

// Geometry::get_shift<frame>(o, r, o, 0.0): the origin's shift as a half's trace starts
// from it (solver.tpp:751; exactly 1 comoving in general geometry).
// The comoving frame uses the origin's own (adaptive) directions, the rest frame of the
// imagers the shared ones.
MGR_HD double origin_shift(const DevModel& m, int frame, uint32_t o, uint32_t r) {
    const double* d = frame ? m.raydir + 3 * r : ray_dir(m, o, r);
    if (m.sph) return shift_sph(m, frame, o, r, o, 0.0, d);
    return frame ? shift_rest(m, r, o, d) : 1.0;
}

// Interpolation-table slot of a spherical step crt -> nxt: three per point (the tangent
// crossing back to the same shell, the next shell inward, the next shell outward).
MGR_HD uint32_t sph_eid(uint32_t crt, uint32_t nxt) { return 3u * crt + (nxt == crt ? 0u : (nxt < crt ? 1u : 2u)); }
MGR_HD uint32_t sph_slot_point(uint32_t p, uint32_t k) { return k == 0 ? p : (k == 1 ? p - 1u : p + 1u); }

// Geometry::get_next_spherical_symmetry (geometry.tpp:118-159) for a ray with
// Rcos = origin . raydir and Rsin2 = |origin|^2 - Rcos^2: inward (Z < -Rcos) to the next
// smaller shell the ray meets, or across the tangent point back to the same shell; then
// outward.  Returns false when the ray leaves the grid (point 0 inward, the last point
// outward).
MGR_HD bool next_point_sph(const DevModel& m, double Rcos, double Rsin2, uint32_t c, double Z, uint32_t& nxt,
                           double& dZ) {
    const double Rcos_plus_Z = dadd_rn(Rcos, Z);
    if (Z < -Rcos) {
        if (c == 0) return false;
        if (sqnorm_rn(m.pos[c - 1]) >= Rsin2) {
            nxt = c - 1;
            dZ = dsub_rn(-dsqrt_rn(dsub_rn(sqnorm_rn(m.pos[nxt]), Rsin2)), Rcos_plus_Z);
        } else {
            nxt = c;
            dZ = dmul_rn(-2.0, Rcos_plus_Z);
        }
    } else {
        if (c >= m.P - 1) return false;
        nxt = c + 1;
        dZ = dsub_rn(dsqrt_rn(dsub_rn(sqnorm_rn(m.pos[nxt]), Rsin2)), Rcos_plus_Z);
    }
    return true;
}

// ---------------------------------------------------------------------------------
// InterpHelper (solver_interp_helper.tpp:55-99)
// ---------------------------------------------------------------------------------
MGR_HD uint32_t n_interp_for_line(const DevModel& m, uint32_t l, uint32_t crt, uint32_t nxt) {
    const double curr = m.crit[(size_t)crt * m.L + l];
    const double next = m.crit[(size_t)nxt * m.L + l];
    const double source_diff = fabsf(logf((float)(next / curr)));
    const double q = source_diff / (double)m.log_max_interp_diff;
    const double c = ceil(q);
    // (Size)NaN is 0 on the reference's targets; keep that outcome explicitly.
    const uint32_t n = (c == c && c > 0.0) ? (c < 4294967295.0 ? (uint32_t)c : 0xffffffffu) : 0u;
    return n > 1 ? n : 1;
}

MGR_HD uint32_t n_interp_all_lines(const DevModel& m, uint32_t crt, uint32_t nxt) {
    double mx = -DBL_MAX;
    for (uint32_t l = 0; l < m.L; l++) {
        const double x = m.crit[(size_t)nxt * m.L + l];
        const double y = m.crit[(size_t)crt * m.L + l];
        const double d = fabsf(logf((float)(x / y)));
        if (d > mx) mx = d;
    }
    const double c = ceil(mx / (double)m.log_max_interp_diff);
    const uint32_t n = (c == c && c > 0.0) ? (c < 4294967295.0 ? (uint32_t)c : 0xffffffffu) : 0u;
    return n > 1 ? n : 1;
}

// Range of the correctly rounded erff table of split precision: every float in
// [kErfBandLo, 3.919206) (12.8 M entries, 51 MB).
constexpr uint32_t kMaxOffDiag = 4;  // largest n_off_diag of the banded (non-local ALO) solve

constexpr float kErfBandLo = 1.4375f;
constexpr uint32_t kErfBandCount = 0x407ad445u - 0x3fb80000u;  // bits(3.919206f) - bits(1.4375f)

// Correctly rounded single-precision erf (double erf rounded once to float).
// For |x| >= 3.919206f (the smallest float whose erf rounds to 1.0f) the value is
// +-1 exactly, which saves the FP64 erf in the saturated wings.
MGR_HD float erff_cr(float x) {
    if (fabsf(x) >= 3.919206f) return copysignf(1.0f, x);
    return (float)erf((double)x);
}

// Single-precision exp and expm1 rounded once from double, for the short-
// characteristics update, whose (S_c - S_n) cancellation amplifies ulp differences
// between libm implementations to ~1e-4 in J.
MGR_HD float expf_cr(float x) { return (float)exp((double)x); }
MGR_HD float expm1f_cr(float x) { return (float)expm1((double)x); }

// The same correctly rounded erff without FP64 in most of [1.5, 3.92): there
// erf = 1 - erfc with erfc < 0.034, and an FP32 erfc (relative error of a few ulp of
// erfc, far below one ulp of erf) decides the rounding of 1 - erfc exactly unless the
// value lies within that error of a rounding midpoint; only then FP64 erf is used.
// t = fl(1 - e) and delta = e - (1 - t) are exact (1 - t is a multiple of 2^-24 and
// |delta| <= 2^-25).  The true erf rounds to t iff |delta + e*eps| < 2^-25; the test
// below allows |eps| up to 2^-19 (>= 16 ulp of e; CUDA documents 4 ulp for erfcf) and
// keeps a small margin for the rounding of the test itself.
MGR_HD float erff_cr_fast(float x) {
    const float ax = fabsf(x);
    if (ax >= 3.919206f) return copysignf(1.0f, x);
    if (ax >= 1.5f) {
        const float e = erfcf(ax);
        const float t = 1.0f - e;
        const float delta = e - (1.0f - t);
        if (fabsf(delta) + e * 0x1.0p-19f < 0x1.ffcp-26f) return copysignf(t, x);
    }
    return (float)erf((double)x);
}

template <typename R>
MGR_HD R interpolate_linear(R f_start, R f_end, R factor) {
    if (factor == R(0)) return f_start;
    if (factor == R(1)) return f_end;
    return (f_end - f_start) * factor + f_start;
}
// FP64: the product and the sum rounded separately, as the reference's build computes
// them.  A contracted multiply-add rounds once; which one the compiler contracts can
// differ between kernels that inline the same code, and the inverse widths interpolated
// here feed the single-precision erff arguments of the line-integrated optical depth,
// whose same-wing differences amplify an ulp of an argument to ~1e-8 of J.
template <>
MGR_HD double interpolate_linear<double>(double f_start, double f_end, double factor) {
    if (factor == 0.0) return f_start;
    if (factor == 1.0) return f_end;
    return dadd_rn(dmul_rn(dsub_rn(f_end, f_start), factor), f_start);
}

MGR_HD double interpolate_log(double f_start, double f_end, double factor) {
    if (factor == 0.0) return f_start;
    if (factor == 1.0) return f_end;
    return f_start * (double)powf((float)(f_end / f_start), (float)factor);
}
MGR_HD float interpolate_log(float f_start, float f_end, float factor) {
    if (factor == 0.0f) return f_start;
    if (factor == 1.0f) return f_end;
    return f_start * powf(f_end / f_start, factor);
}

// ---------------------------------------------------------------------------------
// Profiles and boundary (solver.tpp:1106-1142, thermodynamics.tpp:8-35)
// ---------------------------------------------------------------------------------
MGR_HD double gaussian(double inverse_width, double diff) {
    const double sqrt_exp = inverse_width * diff;
    return inverse_width * INVERSE_SQRT_PI * (double)expf((float)(-sqrt_exp * sqrt_exp));
}
MGR_HD float gaussian(float inverse_width, float diff) {
    const float sqrt_exp = inverse_width * diff;
    return inverse_width * (float)INVERSE_SQRT_PI * expf(-sqrt_exp * sqrt_exp);
}

MGR_HD double planck(double temp, double freq) {
    return TWO_HH_OVER_CC_SQUARED * (freq * freq * freq) / (double)expm1f((float)(HH_OVER_KB * freq / temp));
}

MGR_HD double boundary_intensity(const DevModel& m, uint32_t p, double freq) {
    const uint32_t b = m.p2b[p];
    if (b >= m.B) return 0.0;  // interior point: no boundary condition
    const int c = m.bc[b];
    if (c == BC_ZERO) return 0.0;
    if (c == BC_THERMAL) return planck(m.bt[b], freq);
    return planck(T_CMB, freq);
}

MGR_HD double thermo_profile(const DevModel& m, double inverse_mass, uint32_t p, double freq_line,
                                                 double freq) {
    const double width = freq_line * sqrt(TWO_KB_OVER_AMU_CC_SQUARED * inverse_mass * m.T[p] + m.vt2[p]);
    const double inverse_width = 1.0 / width;
    const double sqrtExponent = inverse_width * (freq - freq_line);
    const double exponent = sqrtExponent * sqrtExponent;
    return inverse_width * INVERSE_SQRT_PI * (double)expf((float)(-exponent));
}

template <typename T>
MGR_HD uint32_t lower_bound(const T* a, uint32_t n, T v) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}
template <typename T>
MGR_HD uint32_t upper_bound(const T* a, uint32_t n, T v) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (!(v < a[mid])) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Solver::get_eta_and_chi<approx> (solver.tpp:1151-1165, :1197-1239, :1286-1294), FP64.
// `sl` is the sorted line table staged in shared memory.
MGR_HD void get_eta_and_chi(const DevModel& m, const double* sl, uint32_t p, uint32_t ll,
                                                double freq, double& eta, double& chi) {
    const size_t base = (size_t)p * m.L;
    if (m.approx == APPROX_ONELINE) {
        const double prof = gaussian(m.iw[base + ll], freq - m.line[ll]);
        eta = prof * m.em[base + ll];
        chi = prof * m.op[base + ll] + m.min_opacity;
        return;
    }
    eta = 0.0;
    chi = m.min_opacity;
    if (m.approx == APPROX_NONE) {
        for (uint32_t l = 0; l < m.L; l++) {
            const double prof = gaussian(m.iw[base + l], freq - m.line[l]);
            eta += prof * m.em[base + l];
            chi += prof * m.op[base + l];
        }
        return;
    }
    const double ub = dmul_rn(m.max_dist, dmul_rn(freq, m.ub[p]));
    const uint32_t lo = lower_bound(sl, m.L, dsub_rn(freq, ub));
    const uint32_t hi = upper_bound(sl, m.L, dadd_rn(freq, ub));
    for (uint32_t s = lo; s < hi; s++) {
        const uint32_t l = m.sorted_map[s];
        const double prof = gaussian(m.iw[base + l], freq - sl[s]);
        eta += prof * m.em[base + l];
        chi += prof * m.op[base + l];
    }
}

}  // namespace mgr
