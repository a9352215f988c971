// Device functions of the analytic MWA tile model and the parallactic-angle
// rotation (described in beam_model.cu), shared by the primary-beam kernel and
// the beam surrogate's training-data, validation and fallback paths.
#pragma once

#include <cstdint>

namespace vgb {

constexpr double kBmC = 299792458.0;
constexpr double kBmPitch = 1.1;          // m
constexpr double kBmDelayUnit = 435e-12;  // s
constexpr double kBmHeight = 0.278;       // m
constexpr double kBmPi = 3.14159265358979323846;

__device__ __forceinline__ void bm_jones(double az, double za, double f, const uint32_t *d, double2 (&J)[4])
{
    double saz, caz, sza, cza;
    sincos(az, &saz, &caz);
    sincos(za, &sza, &cza);
    const double k = 2.0 * kBmPi * f;
    double re = 0.0, im = 0.0;
    int live = 0;
    for (int i = 0; i < 16; i++) {
        if (d[i] == 32u) continue;
        live++;
        const double x = ((i & 3) - 1.5) * kBmPitch;
        const double y = (1.5 - (i >> 2)) * kBmPitch;
        const double tau = (x * sza * saz + y * sza * caz) / kBmC - (double)d[i] * kBmDelayUnit;
        double s, c;
        sincos(k * tau, &s, &c);
        re += c;
        im += s;
    }
    if (live == 0) {
        J[0] = J[1] = J[2] = J[3] = make_double2(0.0, 0.0);
        return;
    }
    const double g = sin(k * kBmHeight * cza / kBmC) / sin(k * kBmHeight / kBmC);
    const double ar = re / 16.0 * g, ai = im / 16.0 * g;
    const double p[4] = {cza * saz, cza * caz, caz, -saz};
    for (int e = 0; e < 4; e++) J[e] = make_double2(ar * p[e], ai * p[e]);
}

__device__ __forceinline__ void bm_pa(double lat, double az, double za, double (&P)[4])
{
    const double el = 0.5 * kBmPi - za;
    double saz, caz, sel, cel, slat, clat;
    sincos(az, &saz, &caz);
    sincos(el, &sel, &cel);
    sincos(lat, &slat, &clat);
    // horizon -> equatorial
    const double x = -caz * cel * slat + sel * clat;
    const double y = -saz * cel;
    const double z = caz * cel * clat + sel * slat;
    const double r = sqrt(x * x + y * y);
    const double ha = r == 0.0 ? 0.0 : atan2(y, x);
    const double dec = atan2(z, r);
    double sha, cha, sdec, cdec;
    sincos(ha, &sha, &cha);
    sincos(dec, &sdec, &cdec);
    const double num = clat * sha, den = slat * cdec - clat * sdec * cha;
    const double chi = (num != 0.0 || den != 0.0) ? atan2(num, den) : 0.0;
    double sc, cc;
    sincos(chi, &sc, &cc);
    P[0] = -cc;
    P[1] = -sc;
    P[2] = sc;
    P[3] = -cc;
}

} // namespace vgb
