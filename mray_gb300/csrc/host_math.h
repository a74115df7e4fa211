// host_math.h -- host-side geometry helpers of the C ABI.
#pragma once

namespace mrg {

// corrected = false: MRay's exact arithmetic, including its sign of the
// [1][2] cofactor; corrected = true: that element negated (true inverse).
void mat34_inverse(const float m[12], float inv[12], bool corrected);
void transform_box_conservative(const float m[12], const float box[6], float out[6]);
// MRay's world AABB of an instance, bit-exact (the box its TLAS leaf tests).
void transform_box_exact(const float m[12], const float box[6], float out[6]);

} // namespace mrg
