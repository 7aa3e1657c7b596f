// Host side of instancing: the world-to-local transform of an instance (its ray transform).
#include <cmath>

#include "sel_internal.h"

namespace sel {

bool affine_inverse(const float l2w[12], float w2l[12]) {
    const double a00 = l2w[0], a01 = l2w[1], a02 = l2w[2], t0 = l2w[3];
    const double a10 = l2w[4], a11 = l2w[5], a12 = l2w[6], t1 = l2w[7];
    const double a20 = l2w[8], a21 = l2w[9], a22 = l2w[10], t2 = l2w[11];
    // cofactors c_ij of the 3 x 3 part; inverse = transpose(cofactors) / det
    const double c00 = a11 * a22 - a12 * a21, c01 = a12 * a20 - a10 * a22, c02 = a10 * a21 - a11 * a20;
    const double c10 = a02 * a21 - a01 * a22, c11 = a00 * a22 - a02 * a20, c12 = a01 * a20 - a00 * a21;
    const double c20 = a01 * a12 - a02 * a11, c21 = a02 * a10 - a00 * a12, c22 = a00 * a11 - a01 * a10;
    const double det = a00 * c00 + a01 * c01 + a02 * c02;
    if (!(det != 0.0) || !std::isfinite(det)) return false;
    const double inv[3][3] = {{c00 / det, c10 / det, c20 / det},
                              {c01 / det, c11 / det, c21 / det},
                              {c02 / det, c12 / det, c22 / det}};
    for (int r = 0; r < 3; ++r) {
        const double tr = -(inv[r][0] * t0 + inv[r][1] * t1 + inv[r][2] * t2);
        for (int c = 0; c < 3; ++c) w2l[4 * r + c] = float(inv[r][c]);
        w2l[4 * r + 3] = float(tr);
    }
    for (int k = 0; k < 12; ++k)
        if (!std::isfinite(w2l[k])) return false;
    return true;
}

}  // namespace sel
