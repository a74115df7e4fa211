// host_math.cpp -- host-side geometry helpers of the C ABI.
// Compiled with -ffp-contract=off so only the explicit std::fma calls fuse.
#include "host_math.h"

#include <cmath>
#include <algorithm>

namespace mrg {

// Matrix3x4::Inverse arithmetic (Source/Core/Matrix.hpp:855-904): 2x2
// sub-determinants via fma, cofactors in plain float, one reciprocal.
void mat34_inverse(const float m[12], float inv[12], bool corrected)
{
    auto det2 = [](float m00, float m01, float m10, float m11)
    {
        return std::fma(m00, m11, -m01 * m10);
    };
    const float s0 = det2(m[0], m[1], m[4], m[5]);
    const float s1 = det2(m[0], m[2], m[4], m[6]);
    const float s2 = det2(m[0], m[3], m[4], m[7]);
    const float s3 = det2(m[1], m[2], m[5], m[6]);
    const float s4 = det2(m[1], m[3], m[5], m[7]);
    const float s5 = det2(m[2], m[3], m[6], m[7]);
    const float c5 = m[10], c4 = m[9], c2 = m[8];
    const float det = ((s0 * c5) - (s1 * c4) + (s3 * c2));
    const float detInv = 1.0f / det;
    const float r[12] =
    {
        (+m[5] * c5 - m[6] * c4),
        (-m[1] * c5 + m[2] * c4),
        s3,
        (-m[9] * s5 + m[10] * s4 - m[11] * s3),
        (-m[4] * c5 + m[6] * c2),
        (+m[0] * c5 - m[2] * c2),
        corrected ? -s1 : s1,   // MRay stores +s1 (Matrix.hpp:888); the cofactor is -s1
        (+m[8] * s5 - m[10] * s2 + m[11] * s1),
        (+m[4] * c4 - m[5] * c2),
        (-m[0] * c4 + m[1] * c2),
        s0,
        (-m[8] * s4 + m[9] * s2 - m[11] * s0)
    };
    for(int i = 0; i < 12; i++) inv[i] = r[i] * detInv;
}

// Conservative world box of a local box under m: the 8 transformed corners
// in double, rounded outward, then inflated by 1e-5 of the box's magnitude so
// the fp32 slab tests in the traversal can never cull a triangle hit.
void transform_box_conservative(const float m[12], const float box[6], float out[6])
{
    double mn[3] = { 1e300, 1e300, 1e300 }, mx[3] = { -1e300, -1e300, -1e300 };
    for(int c = 0; c < 8; c++)
    {
        double v[3] = { (c & 1) ? box[3] : box[0], (c & 2) ? box[4] : box[1], (c & 4) ? box[5] : box[2] };
        for(int r = 0; r < 3; r++)
        {
            double w = (double)m[4 * r] * v[0] + (double)m[4 * r + 1] * v[1] +
                       (double)m[4 * r + 2] * v[2] + (double)m[4 * r + 3];
            mn[r] = std::min(mn[r], w);
            mx[r] = std::max(mx[r], w);
        }
    }
    double mag = 0.0;
    for(int r = 0; r < 3; r++)
        mag = std::max(mag, std::max(std::fabs(mn[r]), std::fabs(mx[r])));
    const double pad = mag * 1e-5 + 1e-30;
    for(int r = 0; r < 3; r++)
    {
        out[r] = std::nextafter((float)(mn[r] - pad), -INFINITY);
        out[3 + r] = std::nextafter((float)(mx[r] + pad), INFINITY);
    }
}

// Matrix3x4::TransformAABB (Source/Core/Matrix.hpp:915-931): each corner
// (w = 1) through the 4-term fma Dot per row, std::min/std::max accumulation.
void transform_box_exact(const float m[12], const float box[6], float out[6])
{
    float rmin[3] = { INFINITY, INFINITY, INFINITY };
    float rmax[3] = { -INFINITY, -INFINITY, -INFINITY };
    for(unsigned c = 0; c < 8; c++)
    {
        const float v[4] = { (c & 1u) ? box[3] : box[0], (c & 2u) ? box[4] : box[1],
                             (c & 4u) ? box[5] : box[2], 1.0f };
        for(int r = 0; r < 3; r++)
        {
            float acc = 0.0f;
            for(int k = 0; k < 4; k++) acc = std::fma(m[4 * r + k], v[k], acc);
            rmax[r] = (rmax[r] < acc) ? acc : rmax[r];
            rmin[r] = (acc < rmin[r]) ? acc : rmin[r];
        }
    }
    for(int r = 0; r < 3; r++) { out[r] = rmin[r]; out[3 + r] = rmax[r]; }
}

} // namespace mrg
