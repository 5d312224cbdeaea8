// Power-of-two scale factors of the FP32 line tables used by split precision.
// Scaling by 2^k is exact, so FP32 keeps its full 24-bit precision for emissivities
// and opacities far below FLT_MIN in SI units (line wings, population floors).
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace mgr {

struct LineScales {
    double Ke = 1.0;  // emissivity scale
    double Ko = 1.0;  // opacity scale
};

// 2^-e for the largest value mx = f 2^e (f in [0.5, 1)); 1 for no positive finite value.
inline double pow2_scale_of(double mx) {
    if (!(mx > 0.0) || !std::isfinite(mx)) return 1.0;
    int e = 0;
    std::frexp(mx, &e);
    return std::ldexp(1.0, -e);
}

inline double pow2_scale_for_max(const double* a, size_t n) {
    double mx = 0.0;
    for (size_t i = 0; i < n; i++)
        if (a[i] > mx) mx = a[i];
    return pow2_scale_of(mx);
}

// Line-offset tables of split precision, [L][L] row l0:
//   dls[l0 L + s] = (float)(sorted_line[s] - line[l0]),  dll[l0 L + l] = (float)(line[l] - line[l0]).
// A lane of line l0 forms its frequency offsets from these without FP64 arithmetic.
inline void line_offset_tables(const double* line, const double* sorted_line, uint32_t L, std::vector<float>& dls,
                               std::vector<float>& dll) {
    dls.resize((size_t)L * L);
    dll.resize((size_t)L * L);
    for (uint32_t a = 0; a < L; a++)
        for (uint32_t b = 0; b < L; b++) {
            dls[(size_t)a * L + b] = (float)(sorted_line[b] - line[a]);
            dll[(size_t)a * L + b] = (float)(line[b] - line[a]);
        }
}

}  // namespace mgr
