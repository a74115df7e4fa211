// spectra_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// extern "C" accessors over the MRay tree's own colour tables and matrices
// (Source/Core/ColorFunctions.{h,cpp}, compiled unmodified next to this
// file), used once to write the spectral fixture under tests/golden/:
// the CIE 1931 observer, the colour space's standard illuminant SPD and its
// normalisation, the RGB <-> XYZ matrices (Tracer/SpectrumContext.cu:400-420,
// 530-531).
#include "Core/ColorFunctions.h"

#include <cstdint>
#include <cstring>

extern "C" {

uint32_t ref_cie_count() { return Color::CIE_1931_N; }
uint32_t ref_cie_start() { return Color::CIE_1931_RANGE[0]; }

void ref_cie_xyz(float* out)
{
    for(uint32_t i = 0; i < Color::CIE_1931_N; i++)
        for(int k = 0; k < 3; k++) out[3 * i + k] = Color::CIE_1931_XYZ[i][k];
}

void ref_cie_integrals(float out[3])
{
    out[0] = Color::CIE_1931_X_INTEGRAL;
    out[1] = Color::CIE_1931_Y_INTEGRAL;
    out[2] = Color::CIE_1931_Z_INTEGRAL;
}

// Colour space 0 = Rec.709 (sRGB primaries, D65).
void ref_illuminant_spd(float* out, float* normFactor)
{
    const auto& spd = Color::SelectIlluminantSPD(MRayColorSpaceEnum::MR_REC_709);
    for(uint32_t i = 0; i < Color::CIE_1931_N; i++) out[i] = spd[i];
    *normFactor = Color::SelectIlluminantSPDNormFactor(MRayColorSpaceEnum::MR_REC_709);
}

void ref_rgb_xyz_matrices(float rgbToXyz[9], float xyzToRgb[9])
{
    const Matrix3x3 m = Color::SelectRGBToXYZMatrix(MRayColorSpaceEnum::MR_REC_709);
    const Matrix3x3 inv = m.Inverse();
    for(int i = 0; i < 9; i++) { rgbToXyz[i] = m[i]; xyzToRgb[i] = inv[i]; }
}

} // extern "C"
