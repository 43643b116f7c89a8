// gl_trace.cuh — sequential ghost/primary trace on a packed lens record.
//
// One __host__ __device__ implementation serves three callers:
//   * the device culler (compiled IEEE-exact, no FMA contraction) and its
//     host re-check (g++ -ffp-contract=off), which must reproduce the
//     reference host arithmetic (ghostlight/src/trace.cpp:171-237 over
//     trace_core.h / fresnel.h) so the surviving ghost set is bit-identical;
//   * the batched render kernel (compiled for speed), which only has to stay
//     within the image tolerance.
//
// Lens layout: a packed SurfRec per surface with the per-surface constants the
// reference recomputes at every hit (2*pi/blades, the polygon apothem, the
// rigid-transform flag) evaluated once on the host, plus per-wavelength IOR
// slices ior_at[s] / ior_before[s] (the reference kernel's
// d_ior_at / d_ior_before tables, ghost_render.cu:809-823).
#pragma once

#include <math.h>
#include <stdint.h>

#include "gl_blade.h"

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#ifndef __forceinline__
#define __forceinline__ inline
#endif
#endif

#define GLH __host__ __device__ __forceinline__

namespace gl {

constexpr int kMaxSurfaces = 64;
constexpr float kPi = 3.14159265358979323846f;
constexpr float kSpawnOffset = 20.0f;   // spawn plane ahead of the front vertex (mm)

enum SurfFlags : int32_t {
    SF_ACTIVE = 1, SF_TRANSFORMED = 2, SF_STOP = 4,
};

// Field meaning: struct Surface (optical_system.h:157-249).
struct SurfRec {
    float z, radius, semi_ap, aspect;
    float rot_rad, sector, apothem, conic;
    float dec_x, dec_y, inv_r;
    float rot[9];
    float asph[8];
    int32_t form, shape, flags, n_asph;
    int32_t coating, ar_layers, blades, cyl_axis;
    float tint_r, tint_g, tint_b, tint_s;
    float g_sigma, g_bg, g_peak, g_dx, g_dy;
    BladeProfile blade;         // authored blade silhouette of a polygon stop (blade.deformed)
    // table-backed coating (SPECTRAL / ANGULAR / SPECTRAL_ANGULAR): address
    // of the table in the memory space of the trace that reads the record
    // (split in two words so the record keeps 4-byte alignment), its
    // extents, the clamp/discard rule and the angle axis' medium index
    uint32_t tab_lo, tab_hi;
    int32_t tab_n0, tab_n1, tab_discard;
    float tab_ref_ior;
    // bitmap aperture (shape 2): address of its w x h luminance pixels (row
    // major, 0 = not loaded: passthrough), and the world radius of the
    // image boundary
    uint32_t img_lo, img_hi;
    int32_t img_w, img_h;
    float img_semi;
    int32_t img_pad;
};
// 77 words: an odd stride, so lanes reading the same field of different
// surfaces in shared memory hit different banks.
static_assert(sizeof(SurfRec) == 308, "SurfRec must stay 308 bytes");

struct V3 {
    float x, y, z;
};
GLH V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
GLH V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
GLH V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
GLH V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
GLH V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
GLH float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
GLH V3 normalized(V3 a)
{
    float l = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
    return (l > 1e-12f) ? a * (1.0f / l) : v3(0.0f, 0.0f, 0.0f);
}
GLH V3 m3mul(const float* m, V3 v)
{
    return v3(m[0] * v.x + m[1] * v.y + m[2] * v.z,
              m[3] * v.x + m[4] * v.y + m[5] * v.z,
              m[6] * v.x + m[7] * v.y + m[8] * v.z);
}
GLH V3 m3tmul(const float* m, V3 v)
{
    return v3(m[0] * v.x + m[3] * v.y + m[6] * v.z,
              m[1] * v.x + m[4] * v.y + m[7] * v.z,
              m[2] * v.x + m[5] * v.y + m[8] * v.z);
}

GLH V3 world_to_local(V3 p, const SurfRec& s)
{
    if (!(s.flags & SF_TRANSFORMED)) return p;
    V3 vtx = v3(s.dec_x, s.dec_y, s.z);
    return m3tmul(s.rot, p - vtx) + v3(0.0f, 0.0f, s.z);
}

// ---- fresnel / coatings (fresnel.h:69-178) -------------------------------
GLH float fresnel_reflectance(float cos_i, float n1, float n2)
{
    cos_i = fabsf(cos_i);
    float eta = n1 / n2;
    float sin2_t = eta * eta * (1.0f - cos_i * cos_i);
    if (sin2_t >= 1.0f) return 1.0f;
    float cos_t = sqrtf(1.0f - sin2_t);
    float rs = (n1 * cos_i - n2 * cos_t) / (n1 * cos_i + n2 * cos_t);
    float rp = (n2 * cos_i - n1 * cos_t) / (n2 * cos_i + n1 * cos_t);
    return 0.5f * (rs * rs + rp * rp);
}

GLH float coating_reflectance(float cos_i, float n1, float n2, float cn, float d_nm, float lam)
{
    float sin2_c = (n1 / cn) * (n1 / cn) * (1.0f - cos_i * cos_i);
    if (sin2_c >= 1.0f) return fresnel_reflectance(cos_i, n1, n2);
    float cos_c = sqrtf(1.0f - sin2_c);
    float delta = 2.0f * kPi * cn * d_nm * cos_c / lam;
    float r01 = (n1 * cos_i - cn * cos_c) / (n1 * cos_i + cn * cos_c);
    float sin2_2 = (cn / n2) * (cn / n2) * (1.0f - cos_c * cos_c);
    if (sin2_2 >= 1.0f) return fresnel_reflectance(cos_i, n1, n2);
    float cos_2 = sqrtf(1.0f - sin2_2);
    float r12 = (cn * cos_c - n2 * cos_2) / (cn * cos_c + n2 * cos_2);
    float c2d = cosf(2.0f * delta);
    float num = r01 * r01 + r12 * r12 + 2.0f * r01 * r12 * c2d;
    float den = 1.0f + r01 * r01 * r12 * r12 + 2.0f * r01 * r12 * c2d;
    float R = num / den;
    return fminf(fmaxf(R, 0.0f), 1.0f);
}

GLH float artist_reflectance(float tr, float tg, float tb, float strength, float lam)
{
    const float inv_2s2 = 1.0f / (2.0f * 65.0f * 65.0f);
    float dr = lam - 650.0f, dg = lam - 550.0f, db = lam - 450.0f;
    float br = expf(-dr * dr * inv_2s2), bg = expf(-dg * dg * inv_2s2), bb = expf(-db * db * inv_2s2);
    float sum = br + bg + bb;
    float R = strength * (tr * br + tg * bg + tb * bb) / sum;
    return fminf(fmaxf(R, 0.0f), 1.0f);
}

GLH float surface_reflectance(float cos_i, float n1, float n2, int layers, float lam)
{
    if (layers <= 0) return fresnel_reflectance(cos_i, n1, n2);
    const float mgf2 = 1.38f, design = 550.0f;
    float qw = design / (4.0f * mgf2);
    float R = coating_reflectance(cos_i, n1, n2, mgf2, qw, lam);
    for (int i = 1; i < layers; ++i) R *= 0.25f;
    return fminf(fmaxf(R, 0.0f), 1.0f);
}

// ---- table-backed coatings (trace_core.h:566-622, 655-760) ----------------
// Table layout: 1-D models [keys n0 | r n0] (keys ascending: nm or degrees);
// SPECTRAL_ANGULAR [wavelengths n0 | angles n1 | r n0*n1, wavelength-major].
GLH const float* coating_table(const SurfRec& s)
{
    return reinterpret_cast<const float*>(((uint64_t)s.tab_hi << 32) | (uint64_t)s.tab_lo);
}

// Bracket `key` on an ascending axis: the lower index and the fraction
// towards the next sample; keys outside the axis clamp to its ends and, in
// discard mode, flag the lookup as discarded.
GLH void coating_bracket(const float* ax, int n, float key, bool discard, int& i0, float& f, bool& dropped)
{
    i0 = 0;
    f = 0.0f;
    if (key <= ax[0])
    {
        if (discard && key < ax[0]) dropped = true;
        return;
    }
    if (key >= ax[n - 1])
    {
        if (discard && key > ax[n - 1]) dropped = true;
        i0 = (n > 1) ? n - 2 : 0;
        f = (n > 1) ? 1.0f : 0.0f;
        return;
    }
    for (int i = 1; i < n; ++i)
    {
        if (key <= ax[i])
        {
            i0 = i - 1;
            const float span = ax[i] - ax[i - 1];
            f = (span > 0.0f) ? (key - ax[i - 1]) / span : 0.0f;
            return;
        }
    }
}

// 1-D lookup: the end samples are returned as they are (no blend), the
// interior as r[i-1] + f (r[i] - r[i-1])
GLH float coating_lerp(const float* t, int n, float key, bool discard, bool& dropped)
{
    const float* r = t + n;
    if (key <= t[0])
    {
        if (discard && key < t[0]) dropped = true;
        return r[0];
    }
    if (key >= t[n - 1])
    {
        if (discard && key > t[n - 1]) dropped = true;
        return r[n - 1];
    }
    int i0;
    float f;
    coating_bracket(t, n, key, false, i0, f, dropped);
    return r[i0] + f * (r[i0 + 1] - r[i0]);
}

// The table's angle axis is measured in a medium of index ref_ior: carry the
// local incidence over by the Snell invariant n sin(theta); past grazing the
// lookup reads the 90-degree end.
GLH float coating_table_angle(float cos_i, float n1, float ref_ior)
{
    const float sin_i = sqrtf(fmaxf(0.0f, 1.0f - cos_i * cos_i));
    const float s_ref = (ref_ior > 0.0f) ? (n1 * sin_i / ref_ior) : sin_i;
    if (s_ref >= 1.0f) return 90.0f;
    return asinf(s_ref) * (180.0f / kPi);
}

// Reflectance of a table-backed coating; `dropped` is set when a discard-mode
// lookup falls outside the table (the interaction then carries no energy).
GLH float table_reflectance(const SurfRec& s, float cos_i, float n1, float n2, float lam, bool& dropped)
{
    const float* t = coating_table(s);
    if (t == nullptr || s.tab_n0 <= 0 || (s.coating == 3 && s.tab_n1 <= 0))
        return fresnel_reflectance(cos_i, n1, n2);
    const bool discard = s.tab_discard != 0;
    if (s.coating == 1) return coating_lerp(t, s.tab_n0, lam, discard, dropped);
    const float ang = coating_table_angle(cos_i, n1, s.tab_ref_ior);
    if (s.coating == 2) return coating_lerp(t, s.tab_n0, ang, discard, dropped);
    const int nw = s.tab_n0, na = s.tab_n1;
    int iw, ia;
    float fw, fa;
    coating_bracket(t, nw, lam, discard, iw, fw, dropped);
    coating_bracket(t + nw, na, ang, discard, ia, fa, dropped);
    if (dropped) return 0.0f;
    const float* r = t + nw + na;
    const int iw1 = (iw + 1 < nw) ? iw + 1 : iw;
    const int ia1 = (ia + 1 < na) ? ia + 1 : ia;
    const float r00 = r[iw * na + ia], r01 = r[iw * na + ia1];
    const float r10 = r[iw1 * na + ia], r11 = r[iw1 * na + ia1];
    return (1.0f - fw) * ((1.0f - fa) * r00 + fa * r01) + fw * ((1.0f - fa) * r10 + fa * r11);
}

// surface_weight (trace_core.h:635-783): SIMPLE, ARTIST, the three table
// models, and bare Fresnel for the attenuator (its positional factor is
// surface_attenuator's)
GLH float surface_weight(V3 dir, V3 nrm, float n1, float n2, const SurfRec& s, float lam, bool reflecting)
{
    float cos_i = fabsf(dot(nrm, dir));
    float R;
    if (s.coating == 0)      R = surface_reflectance(cos_i, n1, n2, s.ar_layers, lam);
    else if (s.coating == 5) R = artist_reflectance(s.tint_r, s.tint_g, s.tint_b, s.tint_s, lam);
    else if (s.coating >= 1 && s.coating <= 3)
    {
        bool dropped = false;
        R = table_reflectance(s, cos_i, n1, n2, lam, dropped);
        if (dropped) return 0.0f;
    }
    else                     R = fresnel_reflectance(cos_i, n1, n2);
    R = fminf(fmaxf(R, 0.0f), 1.0f);
    return reflecting ? R : (1.0f - R);
}

// surface_attenuator (trace_core.h:791-809)
GLH float surface_attenuator(V3 hit, const SurfRec& s)
{
    if (s.coating != 4) return 1.0f;
    if (!(s.g_sigma > 0.0f)) return s.g_bg;
    V3 l = world_to_local(hit, s);
    float dx = l.x - s.g_dx, dy = l.y - s.g_dy;
    float r2 = dx * dx + dy * dy;
    float s2 = s.g_sigma * s.g_sigma;
    return s.g_bg + s.g_peak * expf(-0.5f * r2 / s2);
}

// ---- geometry (trace_core.h:133-564) -------------------------------------
// Bitmap aperture (sample_aperture_image, trace.cpp:31-48): the surface
// point (x, y) in the image's frame, nearest pixel, open where > 0.5; outside
// the image closed; no pixels loaded: open.
GLH bool image_aperture_ok(float x, float y, const SurfRec& s)
{
    const float* px = reinterpret_cast<const float*>(((uint64_t)s.img_hi << 32) | (uint64_t)s.img_lo);
    if (px == nullptr) return true;
    if (s.img_w <= 0 || s.img_h <= 0 || !(s.aspect > 0.0f) || !(s.img_semi > 0.0f)) return false;
    const float hx = x / s.aspect;
    const float u = 0.5f + hx / (2.0f * s.img_semi);
    const float v = 0.5f + y / (2.0f * s.img_semi);
    if (u < 0.0f || u > 1.0f || v < 0.0f || v > 1.0f) return false;
    const int ix = (int)(u * (float)(s.img_w - 1) + 0.5f);
    const int iy = (int)(v * (float)(s.img_h - 1) + 0.5f);
    return px[(size_t)iy * s.img_w + ix] > 0.5f;
}

GLH bool check_aperture(V3 hit, const SurfRec& s)
{
    float hx = hit.x / s.aspect;
    float hy = hit.y;
    float h2 = hx * hx + hy * hy;
    if (!(h2 <= s.semi_ap * s.semi_ap)) return false;
    if (s.shape == 1)
    {
        float r = sqrtf(h2);
        if (r < 1e-9f) return true;
        // authored blade shape: the profile's boundary radius (trace_core.h:153-154)
        if (s.blade.deformed) return r <= s.semi_ap * blade_radius_at(s.blade, atan2f(hy, hx));
        const float angle = atan2f(hy, hx) - s.rot_rad;
        float off = fmodf(angle, s.sector);
        if (off < 0.0f) off += s.sector;
        off -= 0.5f * s.sector;
        return r <= s.apothem / cosf(off);
    }
    if (s.shape == 2) return image_aperture_ok(hit.x, hit.y, s);
    return true;
}

GLH float asag(float r, float inv_r, float K, const float* t, int nt)
{
    float r2 = r * r;
    float D = 1.0f - (1.0f + K) * inv_r * inv_r * r2;
    if (D <= 0.0f) return 1e30f;
    float z = inv_r * r2 / (1.0f + sqrtf(D));
    float rp = r2 * r2;
    for (int i = 0; i < nt; ++i) { z += t[i] * rp; rp *= r2; }
    return z;
}

GLH float adsag(float r, float inv_r, float K, const float* t, int nt)
{
    float r2 = r * r;
    float D = 1.0f - (1.0f + K) * inv_r * inv_r * r2;
    if (D <= 0.0f) return 0.0f;
    float dz = inv_r * r / sqrtf(D);
    float rp = r2 * r;
    for (int i = 0; i < nt; ++i) { dz += (4.0f + 2.0f * (float)i) * t[i] * rp; rp *= r2; }
    return dz;
}

GLH bool pick_root(float t1, float t2, float oz, float dz, float sz, float& t)
{
    if (t1 > 1e-6f && t2 > 1e-6f)
    {
        float z1 = oz + t1 * dz, z2 = oz + t2 * dz;
        t = (fabsf(z1 - sz) < fabsf(z2 - sz)) ? t1 : t2;
    }
    else if (t1 > 1e-6f) t = t1;
    else if (t2 > 1e-6f) t = t2;
    else return false;
    return true;
}

// intersect_surface (trace_core.h:299-525)
GLH bool intersect(V3 ro, V3 rd, const SurfRec& s, float& t_out, V3& n_out)
{
    const bool tr = (s.flags & SF_TRANSFORMED) != 0;
    V3 o = ro, d = rd;
    if (tr)
    {
        V3 vtx = v3(s.dec_x, s.dec_y, s.z);
        o = m3tmul(s.rot, ro - vtx) + v3(0.0f, 0.0f, s.z);
        d = m3tmul(s.rot, rd);
    }
    if (fabsf(s.radius) < 1e-6f)
    {
        if (fabsf(d.z) < 1e-12f) return false;
        float t = (s.z - o.z) / d.z;
        if (!(t > 1e-6f)) return false;
        V3 hit = o + d * t;
        if (!check_aperture(hit, s)) return false;
        t_out = t;
        V3 nn = v3(0.0f, 0.0f, (d.z > 0.0f) ? -1.0f : 1.0f);
        n_out = tr ? m3mul(s.rot, nn) : nn;
        return true;
    }
    if (s.form == 1)
    {
        const float R = s.radius, inv_r = s.inv_r, K = s.conic;
        V3 ctr = v3(0.0f, 0.0f, s.z + R);
        V3 oc = o - ctr;
        float qa = dot(d, d), qb = 2.0f * dot(oc, d), qc = dot(oc, oc) - R * R;
        float disc = qb * qb - 4.0f * qa * qc;
        float t;
        if (disc >= 0.0f)
        {
            float sd = sqrtf(disc), i2a = 0.5f / qa;
            if (!pick_root((-qb - sd) * i2a, (-qb + sd) * i2a, o.z, d.z, s.z, t)) return false;
        }
        else
        {
            if (fabsf(d.z) < 1e-12f) return false;
            t = (s.z - o.z) / d.z;
            if (!(t > 1e-6f)) return false;
        }
        for (int it = 0; it < 15; ++it)
        {
            V3 hi = o + d * t;
            float rx = hi.x, ry = hi.y, rad = sqrtf(rx * rx + ry * ry);
            float sag = asag(rad, inv_r, K, s.asph, s.n_asph);
            if (sag > 1e29f) return false;
            float f = hi.z - s.z - sag;
            if (fabsf(f) < 1e-5f) break;
            float ds = adsag(rad, inv_r, K, s.asph, s.n_asph);
            float rs = (rad > 1e-9f) ? rad : 1e-9f;
            float dfdt = d.z - ds * (rx * d.x + ry * d.y) / rs;
            if (fabsf(dfdt) < 1e-12f) break;
            t -= f / dfdt;
        }
        if (!(t > 1e-6f)) return false;
        V3 hit = o + d * t;
        float rad = sqrtf(hit.x * hit.x + hit.y * hit.y);
        if (!check_aperture(hit, s)) return false;
        float rs = (rad > 1e-9f) ? rad : 1e-9f;
        float ds = adsag(rad, inv_r, K, s.asph, s.n_asph);
        V3 nrm = v3(-ds * hit.x / rs, -ds * hit.y / rs, 1.0f);
        float nl = sqrtf(nrm.x * nrm.x + nrm.y * nrm.y + nrm.z * nrm.z);
        nrm = nrm * (1.0f / nl);
        if (dot(nrm, d) > 0.0f) nrm = -nrm;
        if (tr) nrm = m3mul(s.rot, nrm);
        t_out = t; n_out = nrm;
        return true;
    }
    if (s.form == 2)
    {
        float vx, vy;
        if (s.cyl_axis == 1) { vx = 1.0f; vy = 0.0f; } else { vx = 0.0f; vy = 1.0f; }
        const float R = s.radius;
        float oc_v = o.x * vx + o.y * vy;
        float oc_z = o.z - s.z - R;
        float dv = d.x * vx + d.y * vy;
        float qa = dv * dv + d.z * d.z;
        float qb = 2.0f * (oc_v * dv + oc_z * d.z);
        float qc = oc_v * oc_v + oc_z * oc_z - R * R;
        float disc = qb * qb - 4.0f * qa * qc;
        if (disc < 0.0f) return false;
        float sd = sqrtf(disc), i2a = 0.5f / qa, t;
        if (!pick_root((-qb - sd) * i2a, (-qb + sd) * i2a, o.z, d.z, s.z, t)) return false;
        V3 hit = o + d * t;
        if (!check_aperture(hit, s)) return false;
        float hv = hit.x * vx + hit.y * vy;
        V3 nrm = v3(hv * vx, hv * vy, hit.z - s.z - R);
        float nl = sqrtf(nrm.x * nrm.x + nrm.y * nrm.y + nrm.z * nrm.z);
        if (nl < 1e-12f) return false;
        nrm = nrm * (1.0f / nl);
        if (dot(nrm, d) > 0.0f) nrm = -nrm;
        if (tr) nrm = m3mul(s.rot, nrm);
        t_out = t; n_out = nrm;
        return true;
    }
    {
        const float R = s.radius;
        V3 ctr = v3(0.0f, 0.0f, s.z + R);
        V3 oc = o - ctr;
        float a = dot(d, d), b = 2.0f * dot(oc, d), c = dot(oc, oc) - R * R;
        float disc = b * b - 4.0f * a * c;
        if (disc < 0.0f) return false;
        float sd = sqrtf(disc), i2a = 0.5f / a, t;
        if (!pick_root((-b - sd) * i2a, (-b + sd) * i2a, o.z, d.z, s.z, t)) return false;
        V3 hit = o + d * t;
        if (!check_aperture(hit, s)) return false;
        V3 nrm = (hit - ctr) * (1.0f / fabsf(R));
        if (dot(nrm, d) > 0.0f) nrm = -nrm;
        if (tr) nrm = m3mul(s.rot, nrm);
        t_out = t; n_out = nrm;
        return true;
    }
}

GLH bool refract(V3 d, V3 nrm, float n1, float n2, V3& out)
{
    float nr = n1 / n2;
    float ci = -dot(nrm, d);
    float s2t = nr * nr * (1.0f - ci * ci);
    if (s2t >= 1.0f) return false;
    float ct = sqrtf(1.0f - s2t);
    V3 tmp = d * nr + nrm * (nr * ci - ct);
    float sq = tmp.x * tmp.x + tmp.y * tmp.y + tmp.z * tmp.z;
    if (sq < 1e-18f) return false;
    out = tmp * (1.0f / sqrtf(sq));
    return true;
}

GLH V3 reflect(V3 d, V3 nrm) { return normalized(d - nrm * (2.0f * dot(d, nrm))); }

struct TraceOut {
    float x, y, z, w;
    int status;   // GL_TRACE_*
};

// trace_surface_step (trace.cpp:84-135); returns false when the ray died.
GLH bool step(V3& o, V3& d, const SurfRec& s, float lam, float n2, bool reflecting,
              float reflect_ior, float& cur, TraceOut& res)
{
    float t = 0.0f; V3 nrm;
    if (!intersect(o, d, s, t, nrm)) return false;
    V3 hit = o + d * t;
    o = hit;
    const float n1 = cur;
    if (reflecting)
    {
        res.w *= surface_weight(d, nrm, n1, n2, s, lam, true);
        res.w *= surface_attenuator(hit, s);
        d = reflect(d, nrm);
        cur = reflect_ior;
    }
    else
    {
        V3 nd;
        if (!refract(d, nrm, n1, n2, nd)) { res.status = 2; return false; }
        res.w *= surface_weight(d, nrm, n1, n2, s, lam, false);
        res.w *= surface_attenuator(hit, s);
        d = nd;
        cur = n2;
    }
    return true;
}

GLH void to_sensor(V3 o, V3 d, TraceOut& res)
{
    if (fabsf(d.z) < 1e-12f) { res.status = 3; return; }
    float ts = -o.z / d.z;
    if (!(ts >= 0.0f)) { res.status = 3; return; }
    res.x = o.x + d.x * ts; res.y = o.y + d.y * ts; res.z = o.z + d.z * ts;
    res.status = 0;
}

// trace_ghost_ray (trace.cpp:171-237) with per-wavelength IOR slices.
GLH TraceOut trace_ghost(const SurfRec* S, int N, const float* ior_at, const float* ior_bf,
                         V3 o, V3 d, float lam, int a, int b)
{
    TraceOut res; res.x = res.y = res.z = 0.0f; res.w = 1.0f; res.status = 1;
    if (a < 0 || b < 0 || a >= b || b >= N) { res.status = 4; res.w = 0.0f; return res; }
    float cur = 1.0f;
    for (int s = 0; s <= b; ++s)
    {
        if (!(S[s].flags & SF_ACTIVE)) continue;
        if (!step(o, d, S[s], lam, ior_at[s], s == b, cur, cur, res)) return res;
    }
    for (int s = b - 1; s >= a; --s)
    {
        if (!(S[s].flags & SF_ACTIVE)) continue;
        const float rior = (s == a) ? ior_at[a] : cur;
        if (!step(o, d, S[s], lam, ior_bf[s], s == a, rior, cur, res)) return res;
    }
    for (int s = a + 1; s < N; ++s)
    {
        if (!(S[s].flags & SF_ACTIVE)) continue;
        if (!step(o, d, S[s], lam, ior_at[s], false, cur, cur, res)) return res;
    }
    to_sensor(o, d, res);
    return res;
}

// trace_primary_ray (trace.cpp:243-268)
GLH TraceOut trace_primary(const SurfRec* S, int N, const float* ior_at, V3 o, V3 d, float lam)
{
    TraceOut res; res.x = res.y = res.z = 0.0f; res.w = 1.0f; res.status = 1;
    float cur = 1.0f;
    for (int s = 0; s < N; ++s)
    {
        if (!(S[s].flags & SF_ACTIVE)) continue;
        if (!step(o, d, S[s], lam, ior_at[s], false, cur, cur, res)) return res;
    }
    to_sensor(o, d, res);
    return res;
}

}  // namespace gl
