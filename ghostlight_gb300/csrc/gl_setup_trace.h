// gl_setup_trace.h — primary-ray traces for the per-lens setup (calibration,
// source solve, PSF tile anchors), in float32 or FP64.
//
// A SetupLens<T> holds one lens at one wavelength and traces primary rays
// from the spawn plane to the sensor (trace_primary_ray, trace.cpp:243-268):
//
//  * T = float runs the renderer's own host trace (gl_trace.cuh
//    trace_primary over packed SurfRec records and per-wavelength IOR slices),
//    whose float arithmetic is the reference host build's, so setup results
//    equal the reference's bit for bit;
//  * T = double runs the same geometry in FP64 — the surface forms
//    (sphere, even asphere with Newton refinement, cylinder, plane), the
//    decentre / tilt frames, the clear-aperture tests and Snell refraction,
//    with the reference's thresholds (t > 1e-6, 15 Newton steps to 1e-5 mm,
//    1e-9 / 1e-12 guards) — so the setup solves in double precision as the
//    flare path's first-order optics asks.  The stop silhouette (regular
//    polygon, authored blade profile, bitmap) is the float definition the
//    pupil mask uses, evaluated at the FP64 hit point.
#pragma once

#include "gl_internal.h"

#include <cmath>
#include <vector>

namespace gl {
namespace setup {

template <class T> struct Math;
template <> struct Math<float> {
    static float tan(float x) { return tanf(x); }
    static float atan(float x) { return atanf(x); }
    static float sqrt(float x) { return sqrtf(x); }
    static float sin(float x) { return sinf(x); }
    static float cos(float x) { return cosf(x); }
    static float abs(float x) { return std::fabs(x); }
};
template <> struct Math<double> {
    static double tan(double x) { return std::tan(x); }
    static double atan(double x) { return std::atan(x); }
    static double sqrt(double x) { return std::sqrt(x); }
    static double sin(double x) { return std::sin(x); }
    static double cos(double x) { return std::cos(x); }
    static double abs(double x) { return std::fabs(x); }
};

template <class T> struct Vec { T x, y, z; };
template <class T> inline Vec<T> mk(T x, T y, T z) { return Vec<T>{x, y, z}; }
template <class T> inline Vec<T> add(Vec<T> a, Vec<T> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> inline Vec<T> sub(Vec<T> a, Vec<T> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> inline Vec<T> scl(Vec<T> a, T s) { return mk(a.x * s, a.y * s, a.z * s); }
template <class T> inline T dotp(Vec<T> a, Vec<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline Vec<T> unit(Vec<T> a)
{
    const T l = Math<T>::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return (l > T(1e-12)) ? scl(a, T(1) / l) : mk(T(0), T(0), T(0));
}

// One landing on the sensor plane.
template <class T> struct Hit { T x, y; bool ok; };

// FP64 surface: the trace-facing fields of gl_surface in double, plus the
// packed float record for the stop-silhouette tests.
struct SurfD {
    double z, radius, inv_r, conic, semi, aspect;
    double asph[8];
    int n_asph, form, cyl_axis;
    bool active, transformed;
    double dec_x, dec_y;
    double rot[9];
    const SurfRec* rec;
};

inline Vec<double> rot_t(const double* m, Vec<double> v)
{
    return mk(m[0] * v.x + m[3] * v.y + m[6] * v.z, m[1] * v.x + m[4] * v.y + m[7] * v.z,
              m[2] * v.x + m[5] * v.y + m[8] * v.z);
}
inline Vec<double> rot_n(const double* m, Vec<double> v)
{
    return mk(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
              m[6] * v.x + m[7] * v.y + m[8] * v.z);
}

// The clear aperture at a local hit point: bounding ellipse in FP64, then the
// stop's silhouette as the pupil mask defines it.
inline bool aperture_open(Vec<double> h, const SurfD& s)
{
    const double hx = h.x / s.aspect, hy = h.y;
    const double h2 = hx * hx + hy * hy;
    if (!(h2 <= s.semi * s.semi)) return false;
    const SurfRec& r = *s.rec;
    if (r.shape == 1)
    {
        const double rr = std::sqrt(h2);
        if (rr < 1e-9) return true;
        if (r.blade.deformed) return rr <= s.semi * (double)blade_radius_at(r.blade, (float)std::atan2(hy, hx));
        double off = std::fmod(std::atan2(hy, hx) - (double)r.rot_rad, (double)r.sector);
        if (off < 0.0) off += (double)r.sector;
        off -= 0.5 * (double)r.sector;
        return rr <= s.semi * std::cos(0.5 * (double)r.sector) / std::cos(off);
    }
    if (r.shape == 2) return image_aperture_ok((float)h.x, (float)h.y, r);
    return true;
}

inline double sag_d(double rad, const SurfD& s)
{
    const double r2 = rad * rad;
    const double D = 1.0 - (1.0 + s.conic) * s.inv_r * s.inv_r * r2;
    if (D <= 0.0) return 1e300;
    double z = s.inv_r * r2 / (1.0 + std::sqrt(D));
    double rp = r2 * r2;
    for (int i = 0; i < s.n_asph; ++i) { z += s.asph[i] * rp; rp *= r2; }
    return z;
}

inline double slope_d(double rad, const SurfD& s)
{
    const double r2 = rad * rad;
    const double D = 1.0 - (1.0 + s.conic) * s.inv_r * s.inv_r * r2;
    if (D <= 0.0) return 0.0;
    double dz = s.inv_r * rad / std::sqrt(D);
    double rp = r2 * rad;
    for (int i = 0; i < s.n_asph; ++i) { dz += (4.0 + 2.0 * i) * s.asph[i] * rp; rp *= r2; }
    return dz;
}

// The root of the two nearest the surface vertex among those ahead of the ray.
inline bool nearer_root(double t1, double t2, double oz, double dz, double sz, double& t)
{
    const bool a = t1 > 1e-6, b = t2 > 1e-6;
    if (a && b) t = (std::fabs(oz + t1 * dz - sz) < std::fabs(oz + t2 * dz - sz)) ? t1 : t2;
    else if (a) t = t1;
    else if (b) t = t2;
    else return false;
    return true;
}

// Hit distance and outward-against-the-ray unit normal (world frame).
inline bool meet(Vec<double> ro, Vec<double> rd, const SurfD& s, double& t_out, Vec<double>& n_out)
{
    Vec<double> o = ro, d = rd;
    const Vec<double> vtx = mk(s.dec_x, s.dec_y, s.z);
    if (s.transformed)
    {
        o = add(rot_t(s.rot, sub(ro, vtx)), mk(0.0, 0.0, s.z));
        d = rot_t(s.rot, rd);
    }
    Vec<double> nrm;
    double t = 0.0;
    if (std::fabs(s.radius) < 1e-6)
    {
        if (std::fabs(d.z) < 1e-12) return false;
        t = (s.z - o.z) / d.z;
        if (!(t > 1e-6)) return false;
        if (!aperture_open(add(o, scl(d, t)), s)) return false;
        nrm = mk(0.0, 0.0, d.z > 0.0 ? -1.0 : 1.0);
    }
    else if (s.form == GL_FORM_CYLINDRICAL)
    {
        const double vx = s.cyl_axis == 1 ? 1.0 : 0.0, vy = s.cyl_axis == 1 ? 0.0 : 1.0;
        const double ov = o.x * vx + o.y * vy, oz = o.z - s.z - s.radius, dv = d.x * vx + d.y * vy;
        const double qa = dv * dv + d.z * d.z, qb = 2.0 * (ov * dv + oz * d.z);
        const double qc = ov * ov + oz * oz - s.radius * s.radius;
        const double disc = qb * qb - 4.0 * qa * qc;
        if (disc < 0.0) return false;
        const double sd = std::sqrt(disc);
        if (!nearer_root((-qb - sd) / (2.0 * qa), (-qb + sd) / (2.0 * qa), o.z, d.z, s.z, t)) return false;
        const Vec<double> h = add(o, scl(d, t));
        if (!aperture_open(h, s)) return false;
        const double hv = h.x * vx + h.y * vy;
        nrm = mk(hv * vx, hv * vy, h.z - s.z - s.radius);
        const double nl = std::sqrt(dotp(nrm, nrm));
        if (nl < 1e-12) return false;
        nrm = scl(nrm, 1.0 / nl);
    }
    else
    {
        // sphere (exact quadratic), refined by Newton on the sag for an asphere
        const Vec<double> ctr = mk(0.0, 0.0, s.z + s.radius);
        const Vec<double> oc = sub(o, ctr);
        const double qa = dotp(d, d), qb = 2.0 * dotp(oc, d), qc = dotp(oc, oc) - s.radius * s.radius;
        const double disc = qb * qb - 4.0 * qa * qc;
        const bool asphere = s.form == GL_FORM_ASPHERE;
        if (disc >= 0.0)
        {
            const double sd = std::sqrt(disc);
            if (!nearer_root((-qb - sd) / (2.0 * qa), (-qb + sd) / (2.0 * qa), o.z, d.z, s.z, t)) return false;
        }
        else
        {
            if (!asphere || std::fabs(d.z) < 1e-12) return false;
            t = (s.z - o.z) / d.z;
            if (!(t > 1e-6)) return false;
        }
        if (asphere)
        {
            for (int it = 0; it < 15; ++it)
            {
                const Vec<double> h = add(o, scl(d, t));
                const double rad = std::sqrt(h.x * h.x + h.y * h.y);
                const double sg = sag_d(rad, s);
                if (sg > 1e299) return false;
                const double f = h.z - s.z - sg;
                if (std::fabs(f) < 1e-5) break;
                const double rs = rad > 1e-9 ? rad : 1e-9;
                const double dfdt = d.z - slope_d(rad, s) * (h.x * d.x + h.y * d.y) / rs;
                if (std::fabs(dfdt) < 1e-12) break;
                t -= f / dfdt;
            }
            if (!(t > 1e-6)) return false;
            const Vec<double> h = add(o, scl(d, t));
            if (!aperture_open(h, s)) return false;
            const double rad = std::sqrt(h.x * h.x + h.y * h.y), rs = rad > 1e-9 ? rad : 1e-9;
            const double ds = slope_d(rad, s);
            nrm = unit(mk(-ds * h.x / rs, -ds * h.y / rs, 1.0));
        }
        else
        {
            const Vec<double> h = add(o, scl(d, t));
            if (!aperture_open(h, s)) return false;
            nrm = scl(sub(h, ctr), 1.0 / std::fabs(s.radius));
        }
    }
    if (dotp(nrm, d) > 0.0) nrm = scl(nrm, -1.0);
    n_out = s.transformed ? rot_n(s.rot, nrm) : nrm;
    t_out = t;
    return true;
}

inline bool bend(Vec<double> d, Vec<double> n, double n1, double n2, Vec<double>& out)
{
    const double nr = n1 / n2, ci = -dotp(n, d);
    const double s2t = nr * nr * (1.0 - ci * ci);
    if (s2t >= 1.0) return false;                       // total internal reflection
    const Vec<double> v = add(scl(d, nr), scl(n, nr * ci - std::sqrt(1.0 - s2t)));
    const double q = dotp(v, v);
    if (q < 1e-18) return false;
    out = scl(v, 1.0 / std::sqrt(q));
    return true;
}

// Refractive index after a surface at a wavelength (nm), in double: the
// three-term Sellmeier form, or the d-line index and Abbe number as a Cauchy
// two-term fit through the F and C lines (fresnel.h:27-63).
inline double index_d(const gl_surface& s, double lam_nm)
{
    if (s.disp_model == GL_DISP_SELLMEIER)
    {
        const double l2 = (lam_nm * 1e-3) * (lam_nm * 1e-3);
        double n2 = 1.0;
        for (int k = 0; k < 3; ++k) n2 += (double)s.sellmeier_B[k] * l2 / (l2 - (double)s.sellmeier_C[k]);
        return n2 > 0.0 ? std::sqrt(n2) : 1.0;
    }
    const double nd = s.ior, vd = s.abbe_v;
    if (vd < 0.1 || nd <= 1.0001) return nd;
    const double iF = 1.0 / (486.13 * 486.13), iC = 1.0 / (656.27 * 656.27), id = 1.0 / (587.56 * 587.56);
    const double B = (nd - 1.0) / vd / (iF - iC);
    return nd - B * id + B / (lam_nm * lam_nm);
}

template <class T> class SetupLens;

// float32: the reference-formulation host trace
template <> class SetupLens<float> {
public:
    int open(const gl_surface* s, int n)
    {
        s_ = s; n_ = n;
        recs_.resize((size_t)n);
        const int rc = pack_lens(s, n, recs_.data(), kTablesHost);
        mask_ = resolve_pupil_mask(s, n, 0, 0.0f);
        return rc;
    }
    void set_lambda(float lam)
    {
        if (lam == lam_ && !at_.empty()) return;
        lam_ = lam;
        at_.assign((size_t)n_, 0.0f);
        bf_.assign((size_t)n_, 0.0f);
        build_ior_tables(s_, n_, &lam_, 1, at_.data(), bf_.data());
    }
    // launch at (hx, hy) on the spawn plane heading tan(ah), tan(av)
    Hit<float> trace(float hx, float hy, float ah, float av) const
    {
        const V3 o = v3(hx, hy, s_[0].z - kSpawnOffset);
        const V3 d = normalized(v3(tanf(ah), tanf(av), 1.0f));
        const TraceOut r = trace_primary(recs_.data(), n_, at_.data(), o, d, lam_);
        return Hit<float>{r.x, r.y, r.status == GL_TRACE_OK};
    }
    float front_R() const { return s_[0].semi_aperture; }
    bool pupil_has(float u, float v) const { return pupil_contains(mask_, u, v); }

private:
    const gl_surface* s_ = nullptr;
    int n_ = 0;
    float lam_ = 0.0f;
    std::vector<SurfRec> recs_;
    std::vector<float> at_, bf_;
    PupilMask mask_;
};

// FP64
template <> class SetupLens<double> {
public:
    int open(const gl_surface* s, int n)
    {
        s_ = s; n_ = n;
        recs_.resize((size_t)n);
        const int rc = pack_lens(s, n, recs_.data(), kTablesHost);
        mask_ = resolve_pupil_mask(s, n, 0, 0.0f);
        surf_.resize((size_t)n);
        for (int i = 0; i < n; ++i)
        {
            const gl_surface& g = s[i];
            SurfD& d = surf_[(size_t)i];
            d.z = g.z; d.radius = g.radius; d.inv_r = g.radius != 0.0f ? 1.0 / (double)g.radius : 0.0;
            d.conic = g.conic_k; d.semi = g.semi_aperture; d.aspect = g.aperture_aspect;
            d.n_asph = g.n_asphere_terms < 0 ? 0 : (g.n_asphere_terms > 8 ? 8 : g.n_asphere_terms);
            for (int k = 0; k < 8; ++k) d.asph[k] = g.asphere_terms[k];
            d.form = g.form; d.cyl_axis = g.cyl_axis;
            d.active = g.is_active != 0;
            d.dec_x = g.decenter_x; d.dec_y = g.decenter_y;
            for (int k = 0; k < 9; ++k) d.rot[k] = g.rot[k];
            d.transformed = (recs_[(size_t)i].flags & SF_TRANSFORMED) != 0;
            d.rec = &recs_[(size_t)i];
        }
        return rc;
    }
    void set_lambda(double lam)
    {
        if (lam == lam_ && !idx_.empty()) return;
        lam_ = lam;
        idx_.assign((size_t)n_, 1.0);
        for (int i = 0; i < n_; ++i) idx_[(size_t)i] = index_d(s_[i], lam);
    }
    Hit<double> trace(double hx, double hy, double ah, double av) const
    {
        Vec<double> o = mk(hx, hy, (double)s_[0].z - (double)kSpawnOffset);
        Vec<double> d = unit(mk(std::tan(ah), std::tan(av), 1.0));
        double cur = 1.0;
        for (int i = 0; i < n_; ++i)
        {
            const SurfD& s = surf_[(size_t)i];
            if (!s.active) continue;
            double t;
            Vec<double> nrm, nd;
            if (!meet(o, d, s, t, nrm)) return Hit<double>{0.0, 0.0, false};
            o = add(o, scl(d, t));
            if (!bend(d, nrm, cur, idx_[(size_t)i], nd)) return Hit<double>{0.0, 0.0, false};
            d = nd;
            cur = idx_[(size_t)i];
        }
        if (std::fabs(d.z) < 1e-12) return Hit<double>{0.0, 0.0, false};
        const double ts = -o.z / d.z;
        if (!(ts >= 0.0)) return Hit<double>{0.0, 0.0, false};
        return Hit<double>{o.x + d.x * ts, o.y + d.y * ts, true};
    }
    double front_R() const { return s_[0].semi_aperture; }
    bool pupil_has(double u, double v) const { return pupil_contains(mask_, (float)u, (float)v); }

private:
    const gl_surface* s_ = nullptr;
    int n_ = 0;
    double lam_ = 0.0;
    std::vector<SurfRec> recs_;
    std::vector<SurfD> surf_;
    std::vector<double> idx_;
    PupilMask mask_;
};

}  // namespace setup
}  // namespace gl
