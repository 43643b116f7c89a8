// gl_blade.h — authored iris blade silhouette (curvature, twist, tip notch).
//
// Restates ApertureProfile (ghostlight/src/aperture_profile.h:82-283) and
// make_aperture_profile (:285-358): in the normalised frame (1 = blade-tip
// radius) each half of a blade edge is a conic arc with its focus at the
// centre, linear in u = 1/r and stored in the cancellation-free form
//     u(phi) = u_w - (u_w - 1) sin^2((phi - phi_w)/2) / sin^2(span/2),
// and a notch trims each tip with a straight chord between two points on the
// edges either side of it.  Float arithmetic in the reference's operation
// order (the host translation units are built with -ffp-contract=off), so
// the stop mask and calibration built from it are the reference's bit for
// bit; the device evaluates the same expressions with CUDA's sinf/cosf.
#pragma once

#include <cmath>

#ifndef GLB
#ifdef __CUDACC__
#define GLB __host__ __device__ __forceinline__
#else
#define GLB inline
#endif
#endif

namespace gl {

constexpr float kBladeNegDepth = 0.55f;                                  // scoop depth, fraction of the apothem
constexpr float kBladeMinSpan = 4.0f * (float)(3.14159265358979323846 / 180.0);
constexpr float kBladeNotchFull = 45.0f * (float)(3.14159265358979323846 / 180.0);
constexpr float kBladeNotchMax = 0.45f;
constexpr float kBladeNotchSector = 0.90f;
constexpr float kBladeNotchLimit = (float)(3.14159265358979323846 / 4.0);
constexpr int kBladeAreaPanels = 512;                                    // Simpson panels over one sector

// Derived geometry of one bladed stop.  `deformed` = 0: the regular polygon
// test applies (and these fields are unused by the trace).
struct BladeProfile {
    int blades, deformed, facets, pad;
    float rotation, sigma, half, r_w;
    float phi_w, u_w, u_rise, qR;
    float qL, p, beta, eA;
    float eB, area_frac, pad1, pad2;
};

GLB float blade_clamp(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }

GLB float blade_u_edge(const BladeProfile& b, float phi)
{
    const float psi = phi - b.phi_w;
    const float sh = sinf(0.5f * psi);
    const float q = (psi >= 0.0f) ? b.qR : b.qL;
    return b.u_w - b.u_rise * (sh * sh) * q;
}

// fold an angle into [-sigma/2, +sigma/2)
GLB float blade_fold(const BladeProfile& b, float ang)
{
    float a = fmodf(ang + b.half, b.sigma);
    if (a < 0.0f) a += b.sigma;
    return a - b.half;
}

// u = 1/r at a sector-local angle: the conic edge, or the tip chord across
// its own angular span where that reaches further in
GLB float blade_u_raw(const BladeProfile& b, float phi)
{
    float u = blade_u_edge(b, phi);
    if (b.facets)
    {
        const float w = blade_fold(b, phi - b.half);
        if (w >= -b.eA && w <= b.eB)
        {
            const float uf = cosf(w + b.half - b.beta) / b.p;
            if (uf > u) u = uf;
        }
    }
    return u;
}

// boundary radius (normalised) at absolute angle theta
GLB float blade_radius_at(const BladeProfile& b, float theta)
{
    if (b.blades < 3) return 1.0f;
    float phi = fmodf(theta - b.rotation, b.sigma);
    if (phi < 0.0f) phi += b.sigma;
    phi -= b.half;
    return 1.0f / blade_u_raw(b, phi);
}

inline float blade_inv_sin2_half(float d)
{
    const float s = sinf(0.5f * d);
    return 1.0f / (s * s);
}

inline float blade_area_fraction(const BladeProfile& b)
{
    if (b.blades < 3) return 1.0f;
    const int n = kBladeAreaPanels;
    const double h = (double)b.sigma / n;
    double total = 0.0;
    for (int i = 0; i <= n; ++i)
    {
        const float phi = (float)(-(double)b.half + i * h);
        const double r = 1.0 / (double)blade_u_raw(b, phi);
        const double w = (i == 0 || i == n) ? 1.0 : ((i % 2) ? 4.0 : 2.0);
        total += w * r * r;
    }
    return (float)(b.blades * (total * h / 3.0) / (2.0 * 3.14159265358979323846));
}

// make_aperture_profile: blades < 3 gives an unused profile (area 1).
inline BladeProfile make_blade_profile(int blades, float rotation_rad, float curvature_in, float twist_in,
                                       float notch_in, float notch_angle_in)
{
    BladeProfile b{};
    b.r_w = 1.0f;
    b.u_w = 1.0f;
    b.area_frac = 1.0f;
    if (blades < 3) return b;
    const float curvature = blade_clamp(curvature_in, -1.0f, 1.0f);
    const float twist = blade_clamp(twist_in, -1.0f, 1.0f);
    const float notch = blade_clamp(notch_in, -kBladeNotchLimit, kBladeNotchLimit);
    const float rake = blade_clamp(notch_angle_in, 0.0f, kBladeNotchLimit);

    b.blades = blades;
    b.rotation = rotation_rad;
    b.sigma = 2.0f * (float)3.14159265358979323846 / (float)blades;
    b.half = 0.5f * b.sigma;
    b.deformed = (curvature == 0.0f && twist == 0.0f && notch == 0.0f) ? 0 : 1;

    const float a = cosf(b.half);
    b.r_w = (curvature >= 0.0f) ? (a + curvature * (1.0f - a)) : (a * (1.0f + curvature * kBladeNegDepth));
    const float lim = fmaxf(0.0f, b.half - kBladeMinSpan);
    b.phi_w = blade_clamp(twist * b.half, -lim, lim);
    const float dR = b.half - b.phi_w;
    const float dL = b.half + b.phi_w;
    b.u_w = 1.0f / b.r_w;
    b.u_rise = b.u_w - 1.0f;
    b.qR = blade_inv_sin2_half(dR);
    b.qL = blade_inv_sin2_half(dL);

    // tip chord between a point on this sector's edge and one on the
    // neighbour's, moved apart (skewed) by the notch angle
    const float e = (fabsf(notch) / kBladeNotchFull) * kBladeNotchMax * b.half;
    const float s = blade_clamp(rake / (float)(3.14159265358979323846 / 4.0), 0.0f, 1.0f);
    float eA = fminf(e * (1.0f + s), kBladeNotchSector * b.half);
    float eB = e * (1.0f - s);
    if (notch < 0.0f) { const float t = eA; eA = eB; eB = t; }
    if (e > 1e-9f && b.r_w < 1.0f && (eA + eB) > 1e-9f)
    {
        const float pa = b.half - eA;
        const float ra = 1.0f / blade_u_edge(b, pa);
        const float pb = b.half + eB;
        const float rb = 1.0f / blade_u_edge(b, -b.half + eB);
        const float ax = ra * cosf(pa), ay = ra * sinf(pa);
        const float bx = rb * cosf(pb), by = rb * sinf(pb);
        const float dx = bx - ax, dy = by - ay;
        const float dlen = sqrtf(dx * dx + dy * dy);
        if (dlen >= 1e-9f)
        {
            float nx = dy / dlen, ny = -dx / dlen;
            if (ax * nx + ay * ny < 0.0f) { nx = -nx; ny = -ny; }
            const float p = ax * nx + ay * ny;
            if (p > 1e-6f)
            {
                b.facets = 1;
                b.p = p;
                b.beta = atan2f(ny, nx);
                b.eA = eA;
                b.eB = eB;
            }
        }
    }
    b.area_frac = blade_area_fraction(b);
    return b;
}

}  // namespace gl
