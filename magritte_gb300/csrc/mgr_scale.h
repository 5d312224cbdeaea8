// Power-of-two scale factors of the FP32 line tables used by split precision.
// Scaling by 2^k is exact, so FP32 keeps its full 24-bit precision for emissivities
// and opacities far below FLT_MIN in SI units (line wings, population floors).
#pragma once
#include <cmath>
#include <cstddef>

namespace mgr {

struct LineScales {
    double Ke = 1.0;  // emissivity scale
    double Ko = 1.0;  // opacity scale
};

inline double pow2_scale_for_max(const double* a, size_t n) {
    double mx = 0.0;
    for (size_t i = 0; i < n; i++)
        if (a[i] > mx) mx = a[i];
    if (!(mx > 0.0) || !std::isfinite(mx)) return 1.0;
    int e = 0;
    std::frexp(mx, &e);  // mx = f 2^e, f in [0.5, 1)
    return std::ldexp(1.0, -e);
}

}  // namespace mgr
