// gl_ghost.cu — batched ghost trace + splat (the scatter of
// launch_ghost_render, ghostlight/src/ghost_render.cu:209-491 and :630-1442).
//
// GB300 layout
//   * A render plan keeps everything the trace reads resident in HBM: packed
//     lens records, per-wavelength IOR slices, the spectral table, the pupil
//     grids (one per pair; grids may differ in size), per-source beam data and
//     a list of work items = (pair, source, 256-sample tile).
//   * ONE persistent launch covers every pair x source: each CTA stages the
//     lens table and IOR slices in shared memory once, then pops work items
//     from a global counter until the list is empty.  Launch-bound
//     per-ghost loops and their tail effects disappear; the plan executes with
//     kernel launches only, so it can be captured in a CUDA graph.
//   * The reference's per-pair launch loop (ghost_render.cu:1544-1557) is kept
//     as `plain_per_pair` — the same kernel, one launch per pair, no queue.
//   * Splat: the reference issues 12 scalar float atomics per surviving
//     ray-wavelength.  Here the accumulator is RGBA float4 and each thread
//     carries its current 2x2 footprint in registers across the wavelength
//     loop (dispersion moves a ghost by a fraction of a pixel between
//     neighbouring wavelengths), flushing with one 16-byte vector atomic per
//     tap only when the footprint moves.
//   * The flush kernel reads the RGBA accumulator once, applies the 3x3
//     spectral correction (ghost_render.cu:610-622, same rounding order) and
//     writes the three planar float32 outputs with coalesced vector stores.
#include "gl_render.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

namespace gl {

#ifndef GL_RENDER_MIN_BLOCKS
#define GL_RENDER_MIN_BLOCKS 8
#endif
constexpr int kRenderMinBlocks = GL_RENDER_MIN_BLOCKS;
constexpr unsigned kFull = 0xffffffffu;

// Per-lane splat footprint kept in shared memory (12 floats, stride 13 so the
// lanes of a warp fall in distinct banks) together with its 2x2 origin.
constexpr int kAccStride = 13;

__device__ __forceinline__ void flush_taps(float4* accum, int W, int H, int cx, int cy, const float* acc)
{
    #pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        const int xi = cx + (k & 1), yi = cy + (k >> 1);
        if (xi < 0 || xi >= W || yi < 0 || yi >= H) continue;
        const float r = acc[3 * k], g = acc[3 * k + 1], b = acc[3 * k + 2];
        if (r == 0.0f && g == 0.0f && b == 0.0f) continue;
        atomicAdd(accum + ((size_t)yi * W + xi), make_float4(r, g, b, 0.0f));
    }
}

// ---- render-path surface interaction --------------------------------------
// Same physics as trace_surface_step (trace.cpp:84-135), arranged for the
// render kernel: the common case (untilted sphere or plane, round aperture,
// single-layer coating) is straight-line code; the general intersection
// (asphere Newton solve, cylinder, tilted/decentred frame) and the polygon
// stop are inlined behind warp-uniform branches (an out-of-line call saved
// and restored registers through local memory: measured 2% slower on the
// aspheric wide-angle frame, 8% on the decentred anamorphic sweep); other
// coating models stay out of line.

// Sphere or plane in the vertex-plane form c*|q|^2 - 2*q_z = 0 (q relative to
// the vertex, c = 1/R, c = 0 for a plane).  The ray is first moved to the
// vertex plane, then the root nearest to it is taken in the
// cancellation-free product form t = -C / (B + sign(B) sqrt(B^2 - A C)).
// Choosing the root with the smaller |t| is choosing the hit whose z lies
// nearer the vertex, which is the reference's root rule (trace_core.h:
// 505-515); unlike b^2 - 4ac about the centre of curvature, this form loses
// no precision for large radii or rays near the vertex.
//
// Every lane of the warp runs it (a lane whose ray is dead computes values
// nobody reads): it returns whether the ray hits instead of leaving early, so
// the lock-step walk pays for no divergent branches; the rare far-root case
// is a warp-uniform branch.
__device__ __forceinline__ bool sphere_hit(V3 o, V3 d, float z_s, float c, float& t_out, V3& q_out)
{
    const float t0 = (z_s - o.z) / d.z;
    const float px = o.x + d.x * t0, py = o.y + d.y * t0;
    const float A = c * (d.x * d.x + d.y * d.y + d.z * d.z);   // c |d|^2
    const float B = c * (px * d.x + py * d.y) - d.z;
    const float C = c * (px * px + py * py);
    const float disc = B * B - A * C;
    // den = B + sign(B) sqrt(disc) vanishes only when B = 0 and disc = 0,
    // i.e. A C = 0: A = 0 is a plane, whose B = -d_z, and C = 0 puts the
    // vertex-plane point on the axis, where B = -d_z too; with |d_z| >= 1e-12
    // neither can happen, so a live ray never divides by zero here
    const float den = B + copysignf(sqrtf(disc), B);
    const float ts = -C / den;
    float t = t0 + ts;
    bool ok = (fabsf(d.z) >= 1e-12f) & (disc >= 0.0f);
    const bool near = t > 1e-6f;
    if (__any_sync(kFull, ok & !near))
    {
        // the near root is behind the ray: the far root, if any, is the hit
        const float tb = t0 + (C / A) / ts;
        const bool far = (A != 0.0f) & (ts != 0.0f) & (tb > 1e-6f);
        ok = ok & (near | far);
        t = near ? t : tb;
    }
    t_out = t;
    q_out = v3(o.x + d.x * t, o.y + d.y * t, o.z + d.z * t - z_s);
    return ok;
}

__device__ __forceinline__ bool check_polygon(float hx, float hy, float h2, const SurfRec& s)
{
    float r = sqrtf(h2);
    if (r < 1e-9f) return true;
    if (s.blade.deformed) return r <= s.semi_ap * blade_radius_at(s.blade, atan2f(hy, hx));
    const float angle = atan2f(hy, hx) - s.rot_rad;
    float off = fmodf(angle, s.sector);
    if (off < 0.0f) off += s.sector;
    off -= 0.5f * s.sector;
    return r <= s.apothem / cosf(off);
}

__device__ __forceinline__ bool aperture_ok(float x, float y, const SurfRec& s)
{
    const float hx = x / s.aspect, hy = y;
    const float h2 = hx * hx + hy * hy;
    if (!(h2 <= s.semi_ap * s.semi_ap)) return false;
    if (s.shape == 1) return check_polygon(hx, hy, h2, s);
    if (s.shape == 2) return image_aperture_ok(x, y, s);
    return true;
}

// Everything but an untilted sphere/plane: the shared reference formulation.
__device__ __forceinline__ bool intersect_general(V3 o, V3 d, const SurfRec& s, float& t, V3& nrm)
{
    return intersect(o, d, s, t, nrm);
}

__device__ __noinline__ float weight_general(V3 d, V3 nrm, float n1, float n2, const SurfRec& s,
                                             float lam, bool reflecting)
{
    return surface_weight(d, nrm, n1, n2, s, lam, reflecting);
}

__device__ __noinline__ float attenuator_general(V3 hit, const SurfRec& s)
{
    return surface_attenuator(hit, s);
}

// The per-step fields of one surface packed into two 16-byte words (two
// vector shared-memory loads per step instead of a dozen scalar ones).
struct __align__(16) HotRec {
    float z, c, sa2, inv_aspect;
    int bits, ar_layers;
    float ar_scale;                 // 0.25^(ar_layers - 1): the extra AR layers of the SIMPLE model
    int pad;
};
// HB_FAST: the common surface — active, untilted sphere or plane, round or
// elliptical stop, single-layer coating with at least one layer, no
// attenuator — whose step is one straight-line path behind one test.
// HB_ROUND: an HB_FAST surface whose stop is round (aspect 1).
enum HotBits { HB_ACTIVE = 1, HB_GENERAL = 2, HB_POLYGON = 4, HB_SIMPLE = 8, HB_ATTEN = 16, HB_IMAGE = 32,
               HB_FAST = 64, HB_ROUND = 128 };

__device__ __forceinline__ HotRec make_hot(const SurfRec& s)
{
    HotRec h;
    h.z = s.z;
    h.c = (fabsf(s.radius) < 1e-6f) ? 0.0f : s.inv_r;
    h.sa2 = s.semi_ap * s.semi_ap;
    h.inv_aspect = 1.0f / s.aspect;
    h.bits = ((s.flags & SF_ACTIVE) ? HB_ACTIVE : 0) |
             ((s.form != 0 || (s.flags & SF_TRANSFORMED)) ? HB_GENERAL : 0) |
             ((s.shape == 1) ? HB_POLYGON : 0) | ((s.coating == 0) ? HB_SIMPLE : 0) |
             ((s.coating == 4) ? HB_ATTEN : 0) | ((s.shape == 2) ? HB_IMAGE : 0);
    if (h.bits == (HB_ACTIVE | HB_SIMPLE) && s.ar_layers >= 1) h.bits |= HB_FAST | (s.aspect == 1.0f ? HB_ROUND : 0);
    h.ar_layers = s.ar_layers;
    h.ar_scale = 1.0f;
    for (int i = 1; i < s.ar_layers; ++i) h.ar_scale *= 0.25f;
    h.pad = 0;
    return h;
}

// Single-layer MgF2 reflectance (coating_reflectance / surface_reflectance,
// fresnel.h:92-178) with the film phase factor 2*pi*n_c*d/lambda supplied per
// wavelength (kdelta) and cos(2 delta) formed as 2 cos^2(delta) - 1: delta is
// below pi here, where the SFU cosine is accurate.
//
// The Airy sum R = (r01^2 + r12^2 + 2 r01 r12 c) / (1 + r01^2 r12^2 + 2 r01 r12 c)
// with r01 = A/B, r12 = C/D is evaluated as one quotient of the numerators
// and denominators scaled by (B D)^2 — one division where the textbook form
// has three.  cos_2 >= 0 is the substrate-side cosine when the caller already
// has it (a refraction's transmitted cosine: the film keeps n sin(theta), so
// it is the same angle); cos_2 < 0 computes it here.
// HAVE_COS2: cos_2 is the substrate-side cosine (a refraction's transmitted
// cosine); otherwise it is computed here.  The film-TIR fallbacks to the bare
// Fresnel reflectance are rare: they are taken as warp-uniform branches and
// selected per lane (every lane of the warp calls this).
// LAYERED: the caller knows the surface has at least one layer.
// Returns R before the extra layers' scale, which it leaves in `scale` (1 for
// the bare Fresnel fallbacks), so a refraction's weight 1 - scale R is one FMA.
template <bool HAVE_COS2, bool LAYERED = false>
__device__ __forceinline__ float mgf2_reflectance(float cos_i, float n1, float n2, int layers, float ar_scale,
                                                  float kdelta, float cos_2, float& scale)
{
    scale = 1.0f;
    if (!LAYERED && layers <= 0) return fresnel_reflectance(cos_i, n1, n2);
    const float cn = 1.38f;
    const float a1 = n1 * (1.0f / cn);
    const float sin2_c = a1 * a1 * (1.0f - cos_i * cos_i);
    const float cos_c = sqrtf(1.0f - sin2_c);
    bool bare = sin2_c >= 1.0f;
    if (!HAVE_COS2)
    {
        const float a2 = cn / n2;
        const float sin2_2 = a2 * a2 * (1.0f - cos_c * cos_c);
        bare = bare | (sin2_2 >= 1.0f);
        cos_2 = sqrtf(1.0f - sin2_2);
    }
    const float p1 = n1 * cos_i, pc = cn * cos_c, p2 = n2 * cos_2;
    const float A = p1 - pc, B = p1 + pc, Cn = pc - p2, D = pc + p2;
    const float AD = A * D, CB = Cn * B, BD = B * D, AC = A * Cn;
    const float cd = __cosf(kdelta * cos_c);
    const float c2d = 2.0f * cd * cd - 1.0f;
    const float x = 2.0f * AC * BD * c2d;
    float R = (AD * AD + CB * CB + x) / (BD * BD + AC * AC + x);
    R = fminf(fmaxf(R, 0.0f), 1.0f);
    scale = ar_scale;
    if (__any_sync(kFull, bare))
    {
        const float Rb = fresnel_reflectance(cos_i, n1, n2);
        R = bare ? Rb : R;
        scale = bare ? 1.0f : ar_scale;
    }
    return R;
}

// Snell's law as refract_ray (trace_core.h:533-552), renormalised like it:
// the walk's directions then stay unit to rounding over every interaction
// (a drift in |d| would bias the next surface's root and the landing).
// ci = -dot(nrm, d) >= 0; returns the transmitted cosine (for the coating)
// and clears ok on total internal reflection.
__device__ __forceinline__ float refract_unit(V3& d, V3 nrm, float ci, float n1, float n2, bool& ok)
{
    const float nr = n1 / n2;
    const float s2t = nr * nr * (1.0f - ci * ci);
    ok = ok & (s2t < 1.0f);
    const float ct = sqrtf(1.0f - s2t);
    d = d * nr + nrm * (nr * ci - ct);
    d = d * rsqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
    return ct;
}

// The step of an HB_FAST surface: the common path of surface_step below with
// none of its per-kind tests (same arithmetic, same result).
// ROUND: the stop is round (no aspect scaling).  reflect_ior is read only
// on a reflecting step: through ior_a (the IOR after surface a) when the walk
// runs backward, else it is the current medium.
template <bool WEIGHT, bool ROUND>
__device__ __forceinline__ bool surface_step_fast(V3& o, V3& d, const HotRec& h, float kdelta, float n2,
                                                  bool reflecting, bool back, const float2* ior_a, float& cur,
                                                  float& w, bool alive)
{
    const float c = h.c;
    V3 q;
    float t;
    bool ok = alive & sphere_hit(o, d, h.z, c, t, q);
    const float hx = ROUND ? q.x : q.x * h.inv_aspect, hy = q.y;
    ok = ok & (hx * hx + hy * hy <= h.sa2);
    // The normal is not turned to oppose the ray: with cr = -nrm.d, ci = |cr|
    // and sg the sign of cr, reflection d + (sg nrm)(2 ci) = d + nrm (2 cr)
    // and Snell's nr d + (sg nrm)(nr ci - ct) = nr d + nrm (nr cr - sg ct),
    // the signs cancelling exactly.
    const V3 nrm = v3(c * q.x, c * q.y, c * q.z - 1.0f);
    const float cr = -dot(nrm, d);
    const float ci = fabsf(cr);
    o = v3(q.x, q.y, q.z + h.z);
    const float n1 = cur;
    if (reflecting)
    {
        if (WEIGHT)
        {
            float sc;
            const float R = mgf2_reflectance<false, true>(ci, n1, n2, h.ar_layers, h.ar_scale, kdelta, -1.0f, sc);
            w *= R * sc;
        }
        d = d + nrm * (2.0f * cr);
        d = d * rsqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
        cur = back ? ior_a->x : cur;
    }
    else
    {
        const float nr = n1 / n2;
        const float s2t = nr * nr * (1.0f - ci * ci);
        ok = ok & (s2t < 1.0f);
        const float ct = sqrtf(1.0f - s2t);
        d = d * nr + nrm * fmaf(nr, cr, cr < 0.0f ? ct : -ct);
        d = d * rsqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
        if (WEIGHT)
        {
            float sc;
            const float R = mgf2_reflectance<true, true>(ci, n1, n2, h.ar_layers, h.ar_scale, kdelta, ct, sc);
            w *= fmaf(-R, sc, 1.0f);
        }
        cur = n2;
    }
    return ok;
}

// One surface interaction on the lane's ray; returns whether the ray lives
// on.  Every lane of the warp runs it, whether or not its ray is still alive
// (the walk is lock-step, so a lane leaving early saves no issue slot, only
// adds branch and reconvergence instructions): the geometry of the common
// path (untilted sphere or plane, round stop, single-layer coating) is
// straight-line code whose tests fold into the result, and the caller
// ignores the state of a lane whose ray died.  Branches are on the
// surface's kind (the same for every lane) or warp-uniform votes; the
// out-of-line weight models and bitmap stops, which index memory with the
// ray's values, run only for lanes whose ray is alive.
// WEIGHT = false skips the energy weight: whether a ray dies (missed,
// clipped, TIR) is geometry only (trace_cuda.h sets the status from geometry
// alone), so the off-sensor probe needs none of it.
template <bool WEIGHT>
__device__ __forceinline__ bool surface_step(V3& o, V3& d, const HotRec& h, const SurfRec& s, float lam,
                                             float kdelta, float n2, bool reflecting, float reflect_ior,
                                             float& cur, float& w, bool alive)
{
    V3 nrm, hit;
    bool ok;
    if (!(h.bits & HB_GENERAL))
    {
        const float c = h.c;
        V3 q;
        float t;
        ok = alive & sphere_hit(o, d, h.z, c, t, q);
        const float hx = q.x * h.inv_aspect, hy = q.y;
        const float h2 = hx * hx + hy * hy;
        ok = ok & (h2 <= h.sa2);
        // one test on the common path: plain circular / elliptical stops
        if (h.bits & HB_POLYGON) ok = ok & check_polygon(hx, hy, h2, s);
        else if ((h.bits & HB_IMAGE) && ok) ok = image_aperture_ok(q.x, q.y, s);
        // outward normal (c q_x, c q_y, c q_z - 1), turned to oppose the ray
        // (for a plane, c = 0, it is (0, 0, -1) as it stands)
        nrm = v3(c * q.x, c * q.y, c * q.z - 1.0f);
        hit = v3(q.x, q.y, q.z + h.z);
    }
    else
    {
        float t = 0.0f;
        ok = alive && intersect_general(o, d, s, t, nrm);
        hit = o + d * t;
    }
    float ci = -dot(nrm, d);
    if (ci < 0.0f) { nrm = -nrm; ci = -ci; }
    o = hit;
    const float n1 = cur;
    const bool simple = (h.bits & HB_SIMPLE) != 0;
    if (reflecting)
    {
        if (WEIGHT)
        {
            if (simple)
            {
                float sc;
                const float R = mgf2_reflectance<false>(ci, n1, n2, h.ar_layers, h.ar_scale, kdelta, -1.0f, sc);
                w *= R * sc;
            }
            else if (ok) w *= weight_general(d, nrm, n1, n2, s, lam, true);
            if (h.bits & HB_ATTEN) w *= attenuator_general(hit, s);
        }
        d = d + nrm * (2.0f * ci);
        d = d * rsqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
        cur = reflect_ior;
    }
    else
    {
        const V3 d_in = d;
        const float ct = refract_unit(d, nrm, ci, n1, n2, ok);
        if (WEIGHT)
        {
            if (simple)
            {
                float sc;
                const float R = mgf2_reflectance<true>(ci, n1, n2, h.ar_layers, h.ar_scale, kdelta, ct, sc);
                w *= fmaf(-R, sc, 1.0f);
            }
            else if (ok) w *= weight_general(d_in, nrm, n1, n2, s, lam, false);
            if (h.bits & HB_ATTEN) w *= attenuator_general(hit, s);
        }
        cur = n2;
    }
    return ok;
}

// The three legs of trace_ghost_ray (trace.cpp:196-233) flattened into one
// step sequence k = 0 .. L-1 with a single step site.  The warp walks the
// sequence in lock step for one wavelength at a time: the surface, its form,
// its aperture shape, reflect-or-refract and the IOR pair are the same for
// every lane (uniform branches, broadcast shared-memory reads); only the ray
// state differs.  The walk stops as soon as every lane's ray has died.
__device__ __forceinline__ void splat_ray(const RenderArgs& A, const PairDev& P, const SourceDev& S,
                                          const float4& sp, V3 o, V3 d, float w,
                                          int& cx, int& cy, float* acc)
{
    // propagate_to_sensor (trace.cpp:147-162), then the splat (ghost_render.cu:423-463)
    if (!(fabsf(d.z) >= 1e-12f)) return;
    const float ts = -o.z / d.z;
    if (!(ts >= 0.0f)) return;
    const float rx = o.x + d.x * ts, ry = o.y + d.y * ts;
    if (!isfinite(rx) || !isfinite(ry)) return;
    const float base = w * P.w_ray * A.gain * P.boost;
    if (base < 1e-14f) return;
    float px = (rx / A.hw2 + 0.5f) * A.fmt_w + A.fmt_x0;
    float py = (ry / A.hh2 + 0.5f) * A.fmt_h + A.fmt_y0;
    if (!isfinite(px) || !isfinite(py)) return;
    px = fmaxf(-2.0e9f, fminf(2.0e9f, px));
    py = fmaxf(-2.0e9f, fminf(2.0e9f, py));
    const int x0 = (int)floorf(px - 0.5f), y0 = (int)floorf(py - 0.5f);
    const float fx = (px - 0.5f) - (float)x0, fy = (py - 0.5f) - (float)y0;
    const float power = (S.r * sp.y + S.g * sp.z + S.b * sp.w) * base;
    const float c0 = power * sp.y, c1 = power * sp.z, c2 = power * sp.w;
    if (x0 != cx || y0 != cy)
    {
        if (cx != INT_MIN) flush_taps(A.accum, A.width, A.height, cx, cy, acc);
        cx = x0; cy = y0;
        #pragma unroll
        for (int q = 0; q < 12; ++q) acc[q] = 0.0f;
    }
    const float wt[4] = {(1.0f - fx) * (1.0f - fy), fx * (1.0f - fy), (1.0f - fx) * fy, fx * fy};
    #pragma unroll
    for (int q = 0; q < 4; ++q)
    {
        acc[3 * q] += c0 * wt[q];
        acc[3 * q + 1] += c1 * wt[q];
        acc[3 * q + 2] += c2 * wt[q];
    }
}

template <bool PROBE>
__device__ __forceinline__ void trace_warp(const RenderArgs& A, const SurfRec* lens, const HotRec* hot,
                                           const float2* ab, const float4* spec,
                                           const float* kdel, const PairDev& P, const SourceDev& S,
                                           float2 uv, bool active, float* acc, int pair, int li0, int li1,
                                           int sidx)
{
    const int n = A.n_surf, a = P.a, b = P.b;
    const int L1 = b + 1, L2 = L1 + (b - a), L = L2 + (n - 1 - a);
    int cx = INT_MIN, cy = INT_MIN;

    const unsigned n_lanes = __popc(__ballot_sync(kFull, active));
    int n_lambda = 0;
    #pragma unroll 1
    for (int li = li0; li < li1; ++li)
    {
        // probe: stop once any warp has found the pair on the sensor (read
        // through L2, where the other warps' atomics land)
        if (PROBE && li > li0 && A.pair_hits != nullptr && __ldcg(A.pair_hits + pair) > 0) break;
        ++n_lambda;
        const float4 sp = spec[li];
        const float kdelta = kdel[li];
        const float2* abl = ab + li * n;
        V3 o = v3(uv.x * A.front_R + S.sdx, uv.y * A.front_R + S.sdy, A.start_z);
        V3 d = v3(S.dx, S.dy, S.dz);
        float w = 1.0f, cur = 1.0f;
        bool alive = active;
        int kdead = L;                          // the step the ray died at (L: it left the lens)
        #pragma unroll 1
        for (int k = 0; k < L; ++k)
        {
            if (!__any_sync(kFull, alive)) break;
            int s; float n2; bool refl; bool back = false;
            if (k < L1)      { s = k;                refl = (s == b); }
            else if (k < L2) { s = 2 * b - k;        refl = (s == a); back = true; }
            else             { s = a + 1 + (k - L2); refl = false; }
            const HotRec hr = hot[s];
            const float2 io = abl[s];
            n2 = back ? io.y : io.x;
            const float rior = (back && refl) ? abl[a].x : cur;
            // every lane steps (see surface_step); a dead lane's state is not
            // read; an inactive surface leaves the ray as it is
            bool ok;
            if (hr.bits & HB_ROUND)
                ok = surface_step_fast<!PROBE, true>(o, d, hr, kdelta, n2, refl, back, abl + a, cur, w, alive);
            else if (hr.bits & HB_FAST)
                ok = surface_step_fast<!PROBE, false>(o, d, hr, kdelta, n2, refl, back, abl + a, cur, w, alive);
            else if (hr.bits & HB_ACTIVE)
                ok = surface_step<!PROBE>(o, d, hr, lens[s], sp.x, kdelta, n2, refl, rior, cur, w, alive);
            else continue;
            if (PROBE && alive && !ok) kdead = k;
            alive = ok;
        }
        if (PROBE && A.death != nullptr && active)
            A.death[(size_t)pair * A.perm_stride + sidx] = (unsigned char)min(kdead, 255);
        if (PROBE)
        {
            // Off-sensor probe (the STATS pass of ghost_render.cu:402-415 with
            // the 1.25 margin of :148): did this ray land inside the inflated
            // frame?  One hit anywhere keeps the pair, so the warp stops at
            // the first wavelength that produced one.
            bool hit = false, surv = false;
            if (alive && fabsf(d.z) >= 1e-12f)
            {
                const float ts = -o.z / d.z;
                if (ts >= 0.0f)
                {
                    const float sx = o.x + d.x * ts, sy = o.y + d.y * ts;
                    surv = isfinite(sx) && isfinite(sy);
                    const float spx = (sx / A.hw2 + 0.5f) * A.fmt_w + A.fmt_x0;
                    const float spy = (sy / A.hh2 + 0.5f) * A.fmt_h + A.fmt_y0;
                    hit = isfinite(spx) && isfinite(spy) && spx >= 0.0f && spx < (float)A.width &&
                          spy >= 0.0f && spy < (float)A.height;
                }
            }
            if (A.stats != nullptr)
            {
                // diagnostic pass (the STATS instantiation, ghost_render.cu:402-415):
                // count, never stop early
                const unsigned sv = __ballot_sync(kFull, surv), hv = __ballot_sync(kFull, hit);
                if ((threadIdx.x & 31) == 0)
                {
                    if (sv) atomicAdd(A.stats + 3 * pair + 1, (unsigned long long)__popc(sv));
                    if (hv) atomicAdd(A.stats + 3 * pair + 2, (unsigned long long)__popc(hv));
                }
                continue;
            }
            if (__any_sync(kFull, hit))
            {
                if ((threadIdx.x & 31) == 0)
                {
                    atomicAdd(A.pair_hits + pair, 1);
                    if (A.traced) atomicAdd(A.traced, (unsigned long long)n_lanes * n_lambda);
                }
                return;
            }
        }
        else if (alive)
        {
            splat_ray(A, P, S, sp, o, d, w, cx, cy, acc);
        }
    }
    if (!PROBE && cx != INT_MIN) flush_taps(A.accum, A.width, A.height, cx, cy, acc);
    if (A.traced && (threadIdx.x & 31) == 0) atomicAdd(A.traced, (unsigned long long)n_lanes * n_lambda);
    if (PROBE && A.stats && (threadIdx.x & 31) == 0)
        atomicAdd(A.stats + 3 * pair, (unsigned long long)n_lanes * n_lambda);
}

template <bool PROBE>
__global__ void __launch_bounds__(kRenderThreads, kRenderMinBlocks) ghost_render_kernel(const RenderArgs A)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    HotRec* hot = reinterpret_cast<HotRec*>(smem_raw);
    float4* spec = reinterpret_cast<float4*>(hot + A.n_surf);
    // per (wavelength, surface): (IOR after the surface, IOR before it), one
    // 8-byte shared load for either direction of the walk
    float2* ab = reinterpret_cast<float2*>(spec + A.n_spec);
    float* kdel = reinterpret_cast<float*>(ab + A.n_spec * A.n_surf);
    SurfRec* lens = reinterpret_cast<SurfRec*>(kdel + A.n_spec);
    float* acc_base = reinterpret_cast<float*>(lens + A.n_surf);
    const int tid = threadIdx.x;
    float* acc = acc_base + tid * kAccStride;   // 13 floats per lane: conflict-free banks
    {
        const int words = A.n_surf * (int)(sizeof(SurfRec) / 4);
        const int* src = reinterpret_cast<const int*>(A.recs);
        int* dst = reinterpret_cast<int*>(lens);
        for (int i = tid; i < words; i += blockDim.x) dst[i] = src[i];
        for (int i = tid; i < A.n_spec; i += blockDim.x)
        {
            spec[i] = A.spec[i];
            // film phase factor of the MgF2 quarter-wave layer (fresnel.h:103, 168)
            kdel[i] = 2.0f * kPi * 1.38f * (550.0f / (4.0f * 1.38f)) / A.spec[i].x;
        }
        const int nt = A.n_spec * A.n_surf;
        for (int i = tid; i < nt; i += blockDim.x) ab[i] = make_float2(A.ior_at[i], A.ior_bf[i]);
    }
    __syncthreads();
    for (int i = tid; i < A.n_surf; i += blockDim.x) hot[i] = make_hot(lens[i]);
    __syncthreads();
    // Warp-granular work: each warp takes one task at a time — a (pair,
    // source, 32-sample) item and one of its l_chunks wavelength ranges — so
    // no CTA-wide barrier sits inside the loop, and splitting the wavelengths
    // shortens the tasks at the queue's tail.
    const int lane = tid & 31;
    const int gwarp = (int)((blockIdx.x * blockDim.x + tid) >> 5);
    const int nwarp = (int)((gridDim.x * blockDim.x) >> 5);
    const int chunks = A.l_chunks > 1 ? A.l_chunks : 1;
    const int l_size = (A.n_spec + chunks - 1) / chunks;
    const long long n_tasks = (long long)A.n_items * chunks;
    long long next_static = (long long)A.item_base * chunks + gwarp;
    for (;;)
    {
        long long task;
        if (A.counter != nullptr)
        {
            int v = 0;
            if (lane == 0) v = atomicAdd(A.counter, 1);
            task = __shfl_sync(kFull, v, 0);
        }
        else
        {
            task = next_static;
            next_static += nwarp;
        }
        if (task >= n_tasks) break;
        const int item = (int)(task / chunks);
        const int chunk = (int)(task - (long long)item * chunks);
        int li0 = chunk * l_size, li1 = min(A.n_spec, li0 + l_size);
        if (PROBE && A.lam_hi > 0)
        {
            li0 = max(li0, A.lam_lo);
            li1 = min(li1, A.lam_hi);
        }
        if (li0 >= li1) continue;
        int4 w;
        if (A.items != nullptr) w = A.items[item];
        else
        {
            int tiles = A.u_tiles, base = A.u_grid_base, gn = A.u_grid_n, local = item;
            if (A.u_npass > 0)
            {
                const int q = (item >= A.u_start[2]) ? 2 : (item >= A.u_start[1] ? 1 : 0);
                tiles = A.u_tl[q]; base = A.u_base[q]; gn = A.u_n[q]; local = item - A.u_start[q];
            }
            const int per_pair = tiles * A.u_n_src;
            const int pr = local / per_pair, rem = local - pr * per_pair;
            const int sr = rem / tiles, t = (rem - sr * tiles) * kTile;
            w = make_int4(pr, sr, base + t, min(kTile, gn - t));
        }
        if (A.pair_hits != nullptr)
        {
            // render: skip pairs the probe found off-sensor; probe passes
            // after the first: skip pairs already known to be on-sensor
            const int h = PROBE ? __ldcg(A.pair_hits + w.x) : A.pair_hits[w.x];
            if (PROBE ? (h > 0) : (h == 0)) continue;
        }
        PairDev P = A.pairs[w.x];
        if (A.items == nullptr) P.w_ray = A.w_uniform;
        const SourceDev S = A.sources[w.y];
        const bool active = lane < w.w;
        int sidx = w.z + lane;
        if (PROBE && A.perm != nullptr && active) sidx = A.perm[(size_t)w.x * A.perm_stride + sidx];
        const float2 uv = active ? A.samples[sidx] : make_float2(0.0f, 0.0f);
        trace_warp<PROBE>(A, lens, hot, ab, spec, kdel, P, S, uv, active, acc, w.x, li0, li1, sidx);
    }
}

// Between the probe's two stages: each (pair, pass) still without a hit gets
// its samples sorted by the death step of their first-wavelength ray (stable
// counting sort, one warp), so the second stage's warps hold rays that leave
// the lens together.  The set of samples is unchanged; only their order.
__global__ void __launch_bounds__(32) probe_sort_kernel(const unsigned char* __restrict__ death,
                                                        unsigned short* __restrict__ perm,
                                                        const int* __restrict__ pair_hits, int stride, int b0,
                                                        int b1, int b2, int b3)
{
    __shared__ int off[257];
    const int pair = blockIdx.x, pass = blockIdx.y, lane = threadIdx.x;
    if (pair_hits[pair] > 0) return;              // found on the sensor: stage 2 skips it
    const int lo = pass == 0 ? b0 : (pass == 1 ? b1 : b2);
    const int hi = pass == 0 ? b1 : (pass == 1 ? b2 : b3);
    const unsigned char* d = death + (size_t)pair * stride;
    unsigned short* out = perm + (size_t)pair * stride;
    for (int b = lane; b < 257; b += 32) off[b] = 0;
    __syncwarp();
    for (int i = lo + lane; i < hi; i += 32) atomicAdd(&off[d[i]], 1);
    __syncwarp();
    if (lane == 0)
    {
        int run = lo;
        for (int b = 0; b < 256; ++b)
        {
            const int c = off[b];
            off[b] = run;
            run += c;
        }
    }
    __syncwarp();
    for (int c0 = lo; c0 < hi; c0 += 32)
    {
        const int i = c0 + lane;
        const bool v = i < hi;
        const int key = v ? (int)d[i] : 256;
        const unsigned m = __match_any_sync(kFull, key);
        const int rank = __popc(m & ((1u << lane) - 1u));
        if (v) out[off[key] + rank] = (unsigned short)i;
        __syncwarp();
        if (v && rank == 0) off[key] += __popc(m);
        __syncwarp();
    }
}

// RGBA accumulator -> planar r/g/b with the optional 3x3 correction, four
// pixels per thread (one 64-byte read, three 16-byte writes).
__global__ void ghost_flush_kernel(const float4* __restrict__ accum, size_t n_px, float* __restrict__ out_r,
                                   float* __restrict__ out_g, float* __restrict__ out_b, int apply,
                                   float c00, float c01, float c02, float c10, float c11, float c12,
                                   float c20, float c21, float c22)
{
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t p0 = q * 4;
    if (p0 >= n_px) return;
    float r[4], g[4], b[4];
    #pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        float4 v = (p0 + k < n_px) ? accum[p0 + k] : make_float4(0, 0, 0, 0);
        if (apply)
        {
            r[k] = __fadd_rn(__fadd_rn(__fmul_rn(c00, v.x), __fmul_rn(c01, v.y)), __fmul_rn(c02, v.z));
            g[k] = __fadd_rn(__fadd_rn(__fmul_rn(c10, v.x), __fmul_rn(c11, v.y)), __fmul_rn(c12, v.z));
            b[k] = __fadd_rn(__fadd_rn(__fmul_rn(c20, v.x), __fmul_rn(c21, v.y)), __fmul_rn(c22, v.z));
        }
        else
        {
            r[k] = v.x; g[k] = v.y; b[k] = v.z;
        }
    }
    const bool vec = (p0 + 4 <= n_px) && ((((uintptr_t)(out_r + p0)) | ((uintptr_t)(out_g + p0)) |
                                          ((uintptr_t)(out_b + p0))) & 15) == 0;
    if (vec)
    {
        *reinterpret_cast<float4*>(out_r + p0) = make_float4(r[0], r[1], r[2], r[3]);
        *reinterpret_cast<float4*>(out_g + p0) = make_float4(g[0], g[1], g[2], g[3]);
        *reinterpret_cast<float4*>(out_b + p0) = make_float4(b[0], b[1], b[2], b[3]);
    }
    else
    {
        for (int k = 0; k < 4 && p0 + k < n_px; ++k) { out_r[p0 + k] = r[k]; out_g[p0 + k] = g[k]; out_b[p0 + k] = b[k]; }
    }
}

// ---------------------------------------------------------------------------
// Plan: resident device state of one ghost render request.
// ---------------------------------------------------------------------------
struct GhostPlan {
    int device = 0;
    int n_surf = 0, n_spec = 0, n_pairs = 0, n_items = 0;
    int width = 0, height = 0;
    gl_ghost_render_params prm{};
    std::vector<int> pair_item_begin;   // first item of each pair (+ sentinel)
    // device
    SurfRec* recs = nullptr;
    float* ior_at = nullptr;
    float* ior_bf = nullptr;
    float4* spec = nullptr;
    int4* items = nullptr;
    PairDev* pairs = nullptr;
    SourceDev* sources = nullptr;
    float2* samples = nullptr;
    int* counter = nullptr;
    float4* accum = nullptr;            // RGBA scratch, width x height
    size_t smem = 0;
    int grid_persistent = 0;
    int per_sm = 0, n_sm = 0;           // resident render CTAs per SM, SM count
    int launch_ipw = 0;                 // 0: persistent queue; > 0: static chunks of this many items per warp
    int l_chunks = 1;                   // wavelength ranges per item (tasks per item)
    long long rays = 0;                 // ray-wavelength traces per execute
    float front_R = 0.0f, start_z = 0.0f;
    // off-sensor cull (probe passes)
    bool cull = false;
    int4* probe_items = nullptr;
    float2* probe_samples = nullptr;
    unsigned char* probe_death = nullptr;     // two-stage probe (one source): death steps
    unsigned short* probe_perm = nullptr;     // and the sorted sample order, per pair
    int probe_samples_n = 0;
    int probe_sample_begin[4] = {0, 0, 0, 0}; // sample range of each pass
    int probe_begin[4] = {0, 0, 0, 0};   // item range of each pass
    int* pair_hits = nullptr;
    int* probe_counters = nullptr;
    int* pair_hits_init = nullptr;          // 1 = not probed (always rendered), 0 = probed
    long long probe_rays = 0;
    unsigned long long* traced = nullptr;   // [render, probe] traces executed by the last execute
    // optional timing events recorded around the probe and render launches
    cudaEvent_t ev_probe = nullptr, ev_render = nullptr, ev_end = nullptr;
    // Device memory comes from the device's stream-ordered pool: creating and
    // destroying a plan then costs no device-wide synchronisation (a
    // cudaFree waits for every stream).  `done` is recorded after each
    // execute; destroy waits for it (or, after a stream capture, for the
    // device) and releases the blocks in stream order.
    cudaMemPool_t pool = nullptr;
    cudaStream_t own = nullptr;         // the device's plan stream (uploads, releases)
    cudaEvent_t done = nullptr;
    bool executed = false, captured = false;
};

// One non-blocking stream per device for plan uploads and releases.
static cudaStream_t plan_stream(int dev)
{
    static std::mutex mu;
    static cudaStream_t st[64] = {};
    if (dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    if (!st[dev] && cudaStreamCreateWithFlags(&st[dev], cudaStreamNonBlocking) != cudaSuccess) st[dev] = nullptr;
    return st[dev];
}

static void plan_free(GhostPlan* p)
{
    if (!p) return;
    if (p->captured) cudaDeviceSynchronize();               // graph replays may still use the blocks
    else if (p->executed && p->done) cudaEventSynchronize(p->done);
    void* blocks[] = {p->recs, p->ior_at, p->ior_bf, p->spec, p->items, p->pairs, p->sources, p->samples,
                      p->counter, p->accum, p->probe_items, p->probe_samples, p->pair_hits, p->probe_counters,
                      p->traced, p->pair_hits_init, p->probe_death, p->probe_perm};
    for (void* b : blocks)
    {
        if (!b) continue;
        if (p->own) cudaFreeAsync(b, p->own);
        else cudaFree(b);
    }
    if (p->done) cudaEventDestroy(p->done);
    delete p;
}

template <class T>
static cudaError_t upload(T** dst, const T* src, size_t count, cudaMemPool_t pool, cudaStream_t st)
{
    cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(dst), std::max<size_t>(count, 1) * sizeof(T),
                                            pool, st);
    if (e != cudaSuccess) return e;
    if (count) e = cudaMemcpyAsync(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice, st);
    return e;
}

template <class T>
static cudaError_t alloc(T** dst, size_t bytes, cudaMemPool_t pool, cudaStream_t st)
{
    return cudaMallocFromPoolAsync(reinterpret_cast<void**>(dst), bytes, pool, st);
}

size_t render_smem(int n_surf, int n_spec)
{
    return (size_t)n_surf * 32 + (size_t)n_spec * 16 + (size_t)n_spec * 4 + 2 * (size_t)n_spec * n_surf * 4 +
           (size_t)n_surf * sizeof(SurfRec) + (size_t)kRenderThreads * kAccStride * 4;
}

// The opt-in only grows (per device and kernel), so a plan created earlier
// with a larger table keeps launching after a smaller one was prepared.
int raise_smem_limit(const void* kernel, size_t bytes)
{
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> limit;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    std::lock_guard<std::mutex> lk(mu);
    size_t& cur = limit[{dev, kernel}];
    if (bytes <= cur) return (int)cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return (int)e;
}

cudaError_t render_prepare(size_t smem, int* per_sm, int* n_sm)
{
    cudaError_t e = (cudaError_t)raise_smem_limit((const void*)ghost_render_kernel<false>, smem);
    if (e == cudaSuccess) e = (cudaError_t)raise_smem_limit((const void*)ghost_render_kernel<true>, smem);
    if (e == cudaSuccess && per_sm) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, ghost_render_kernel<false>, kRenderThreads, smem);
    int dev = 0;
    if (e == cudaSuccess && n_sm) e = cudaGetDevice(&dev);
    if (e == cudaSuccess && n_sm) e = cudaDeviceGetAttribute(n_sm, cudaDevAttrMultiProcessorCount, dev);
    return e;
}

cudaError_t render_launch(const RenderArgs& A, bool probe, int grid, size_t smem, cudaStream_t st)
{
    if (probe) ghost_render_kernel<true><<<grid, kRenderThreads, smem, st>>>(A);
    else ghost_render_kernel<false><<<grid, kRenderThreads, smem, st>>>(A);
    return cudaGetLastError();
}

cudaError_t flush_launch(const float4* accum, size_t n_px, float* r, float* g, float* b, int apply, const float* C,
                         cudaStream_t st)
{
    const size_t quads = (n_px + 3) / 4;
    const int fb = 256;
    ghost_flush_kernel<<<(unsigned)((quads + fb - 1) / fb), fb, 0, st>>>(accum, n_px, r, g, b, apply, C[0], C[1], C[2],
                                                                         C[3], C[4], C[5], C[6], C[7], C[8]);
    return cudaGetLastError();
}

SourceDev make_source(const gl_flare_source& s)
{
    const float bx = tanf(s.angle_x), by = tanf(s.angle_y);
    V3 dir = normalized(v3(bx, by, 1.0f));
    return {dir.x, dir.y, dir.z, -kSpawnOffset * bx, -kSpawnOffset * by, s.r, s.g, s.b};
}

// Pupil samples in Morton order over the unit square: 32 consecutive samples
// (one warp) then cover a compact patch of the pupil, whose rays tend to
// vignette together, instead of a strip across it.  The set of samples and
// each one's weight are unchanged.
static inline uint32_t morton_code(const gl_pupil_sample& p)
{
    auto spread = [](uint32_t x) {
        x &= 0x3ffu;
        x = (x | (x << 16)) & 0x030000ffu;
        x = (x | (x << 8)) & 0x0300f00fu;
        x = (x | (x << 4)) & 0x030c30c3u;
        x = (x | (x << 2)) & 0x09249249u;
        return x;
    };
    const float fu = std::min(std::max((p.u + 1.0f) * 512.0f, 0.0f), 1023.0f);
    const float fv = std::min(std::max((p.v + 1.0f) * 512.0f, 0.0f), 1023.0f);
    return (spread((uint32_t)fu) << 1) | spread((uint32_t)fv);
}

// A stable sort on the code: ordering an ordered grid again changes nothing,
// so a caller may hand in grids it has ordered (and cached) once, and the
// plan build then only checks them (one linear pass instead of a sort).
void morton_order(const gl_pupil_sample* in, int n, gl_pupil_sample* out)
{
    bool sorted = true;
    uint32_t prev = 0;
    for (int i = 0; i < n && sorted; ++i)
    {
        const uint32_t c = morton_code(in[i]);
        sorted = (i == 0) || c >= prev;
        prev = c;
    }
    if (sorted)
    {
        std::copy(in, in + n, out);
        return;
    }
    std::vector<std::pair<uint32_t, int>> key;
    key.reserve((size_t)n);
    for (int i = 0; i < n; ++i) key.push_back({morton_code(in[i]), i});
    std::stable_sort(key.begin(), key.end(),
                     [](const std::pair<uint32_t, int>& x, const std::pair<uint32_t, int>& y) { return x.first < y.first; });
    for (int i = 0; i < n; ++i) out[i] = in[key[i].second];
}

int probe_grids(const gl_surface* surfaces, int n_surf, int blades_override, float rotation_deg,
                std::vector<gl_pupil_sample>& out, int begin[4])
{
    out.clear();
    for (int pass = 0; pass < 3; ++pass)
    {
        gl_sampler_params sp;
        sp.ray_grid = 40;
        sp.pupil_jitter = 1;
        sp.jitter_seed = (int)(0x9E3779B9u * (unsigned)(pass + 1));
        sp.blades_override = blades_override;
        sp.rotation_deg = rotation_deg;
        std::vector<gl_pupil_sample> g;
        const int rc = build_aperture_samples(surfaces, n_surf, sp, g);
        if (rc) return rc;
        begin[pass] = (int)out.size();
        out.insert(out.end(), g.begin(), g.end());
    }
    begin[3] = (int)out.size();
    return GL_OK;
}

// Wavelength ranges per item by default: about eight wavelengths per task
// (31 -> 4, 16 -> 2, 8 -> 1), the split the autotuner picks on the
// 31-wavelength frames; set_lambda_split overrides it.
int default_lambda_split(int n_spec)
{
    return std::max(1, std::min(n_spec, (n_spec + 4) / 8));
}

int plan_create(const gl_surface* surfaces, int n_surf, const gl_ghost_pair* pairs, const float* boosts,
                const int32_t* pair_grid, int n_pairs, const gl_flare_source* sources, int n_src,
                const gl_pupil_sample* samples, const int32_t* grid_offsets, int n_grids,
                const gl_spectral_sample* spec, int n_spec, const gl_ghost_render_params* prm,
                GhostPlan** out)
{
    if (!surfaces || n_surf <= 0 || !prm || !out) return fail(GL_ERR_INVALID, "render_ghosts: bad arguments");
    if (n_pairs < 0 || n_src < 0 || n_grids < 0) return fail(GL_ERR_INVALID, "render_ghosts: negative count");
    if (n_pairs > 0 && (!pairs || !boosts)) return fail(GL_ERR_INVALID, "render_ghosts: missing pairs");
    if (n_src > 0 && !sources) return fail(GL_ERR_INVALID, "render_ghosts: missing sources");
    if (prm->width <= 0 || prm->height <= 0) return fail(GL_ERR_INVALID, "render_ghosts: width and height must be positive");
    if ((long long)prm->width * prm->height > (1LL << 31)) return fail(GL_ERR_INVALID, "render_ghosts: image has too many pixels");
    if (n_spec < 1 || n_spec > kMaxSpec || !spec) return fail(GL_ERR_INVALID, "render_ghosts: spectral table must hold 1..256 samples");
    if (!(prm->sensor_half_w > 0.0f) || !(prm->sensor_half_h > 0.0f))
        return fail(GL_ERR_INVALID, "render_ghosts: sensor half extents must be positive");
    if (n_grids > 0 && (!grid_offsets || !samples)) return fail(GL_ERR_INVALID, "render_ghosts: missing pupil grids");
    for (int i = 0; i < n_pairs; ++i)
    {
        const int a = pairs[i].surf_a, b = pairs[i].surf_b;
        if (a < 0 || b <= a || b >= n_surf) return fail(GL_ERR_INVALID, "render_ghosts: bounce indices must satisfy 0 <= a < b < n");
        const int g = pair_grid ? pair_grid[i] : 0;
        if (g < 0 || g >= n_grids) return fail(GL_ERR_INVALID, "render_ghosts: pair grid index out of range");
    }
    for (int g = 0; g < n_grids; ++g)
        if (grid_offsets[g + 1] < grid_offsets[g] || grid_offsets[g] < 0)
            return fail(GL_ERR_INVALID, "render_ghosts: grid offsets must be non-decreasing");

    int plan_dev = 0;
    GL_CUDA_TRY(cudaGetDevice(&plan_dev));
    std::vector<SurfRec> recs((size_t)n_surf);
    int rc = pack_lens(surfaces, n_surf, recs.data(), plan_dev);
    if (rc) return rc;

    GhostPlan* p = new GhostPlan();
    cudaGetDevice(&p->device);
    p->n_surf = n_surf; p->n_spec = n_spec; p->n_pairs = n_pairs;
    p->front_R = surfaces[0].semi_aperture;              // ghost_render.cu:738-739
    p->start_z = surfaces[0].z - kSpawnOffset;
    p->width = prm->width; p->height = prm->height; p->prm = *prm;
    // the per-pair form keeps the reference kernel's shape: every thread loops
    // over all wavelengths (ghost_render.cu:372)
    p->l_chunks = prm->plain_per_pair ? 1 : default_lambda_split(n_spec);

    std::vector<float> lams((size_t)n_spec), at((size_t)n_spec * n_surf), bf((size_t)n_spec * n_surf);
    std::vector<float4> sp((size_t)n_spec);
    for (int i = 0; i < n_spec; ++i)
    {
        lams[i] = spec[i].lambda;
        sp[i] = make_float4(spec[i].lambda, spec[i].cmf_r, spec[i].cmf_g, spec[i].cmf_b);
    }
    build_ior_tables(surfaces, n_surf, lams.data(), n_spec, at.data(), bf.data());

    // Per-source beam (ghost_render.cu:349-358): tanf slopes, the normalised
    // direction and the spawn-plane shift that follows the beam.
    std::vector<SourceDev> src((size_t)n_src);
    for (int i = 0; i < n_src; ++i) src[i] = make_source(sources[i]);

    const int n_samples_all = n_grids > 0 ? grid_offsets[n_grids] : 0;
    std::vector<gl_pupil_sample> ordered((size_t)n_samples_all);
    for (int g = 0; g < n_grids; ++g)
        morton_order(samples + grid_offsets[g], grid_offsets[g + 1] - grid_offsets[g], ordered.data() + grid_offsets[g]);

    std::vector<PairDev> pd((size_t)n_pairs);
    std::vector<int4> items;
    p->pair_item_begin.assign((size_t)n_pairs + 1, 0);
    for (int i = 0; i < n_pairs; ++i)
    {
        const int g = pair_grid ? pair_grid[i] : 0;
        const int g0 = grid_offsets[g], ng = grid_offsets[g + 1] - grid_offsets[g];
        pd[i] = {pairs[i].surf_a, pairs[i].surf_b, boosts[i], ng > 0 ? 1.0f / (float)ng : 0.0f};
        p->pair_item_begin[i] = (int)items.size();
        for (int s = 0; s < n_src; ++s)
            for (int t = 0; t < ng; t += kTile)
                items.push_back(make_int4(i, s, g0 + t, std::min(kTile, ng - t)));
        p->rays += (long long)ng * n_src * n_spec;
    }
    p->pair_item_begin[n_pairs] = (int)items.size();
    p->n_items = (int)items.size();

    // Off-sensor probe grids (ghost_render.cu:1022-1027): 40x40, wang-hash
    // jitter with a fixed seed per pass, the config's blade override.
    p->cull = prm->cull_dead_pairs && n_pairs > 1 && n_spec != 3 && !prm->plain_per_pair;
    std::vector<int4> pitems;
    std::vector<gl_pupil_sample> psamples;
    std::vector<int> hits_init((size_t)n_pairs, 1);
    if (p->cull)
    {
        // A pair is probed only when its own grid is larger than the three
        // probe passes: rendering a pair that lands nowhere costs less than
        // proving it, and never changes the image.
        int pbeg[4];
        {
            const int rcs = probe_grids(surfaces, n_surf, prm->blades_override, prm->rotation_deg, psamples, pbeg);
            if (rcs) { plan_free(p); return rcs; }
        }
        const int n_probe_samples = pbeg[3];
        p->probe_samples_n = n_probe_samples;
        for (int q = 0; q < 4; ++q) p->probe_sample_begin[q] = pbeg[q];
        for (int i = 0; i < n_pairs; ++i)
        {
            const int gi = pair_grid ? pair_grid[i] : 0;
            const int ng = grid_offsets[gi + 1] - grid_offsets[gi];
            hits_init[i] = (ng > n_probe_samples) ? 0 : 1;
        }
        for (int pass = 0; pass < 3; ++pass)
        {
            const int base = pbeg[pass], cnt = pbeg[pass + 1] - pbeg[pass];
            p->probe_begin[pass] = (int)pitems.size();
            for (int i = 0; i < n_pairs; ++i)
            {
                if (hits_init[i]) continue;
                for (int s = 0; s < n_src; ++s)
                    for (int t = 0; t < cnt; t += kTile)
                        pitems.push_back(make_int4(i, s, base + t, std::min(kTile, cnt - t)));
                p->probe_rays += (long long)cnt * n_src * n_spec;
            }
        }
        p->probe_begin[3] = (int)pitems.size();
    }
    const int n_samples = n_grids > 0 ? grid_offsets[n_grids] : 0;

    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    chk(shared_device_pool(p->device, &p->pool));
    p->own = plan_stream(p->device);
    if (e == cudaSuccess && !p->own) e = cudaErrorInvalidResourceHandle;
    if (e == cudaSuccess) chk(cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming));
    if (e != cudaSuccess)
    {
        p->own = nullptr;
        plan_free(p);
        return fail(GL_ERR_CUDA, std::string("render_ghosts: ") + cudaGetErrorString(e));
    }
    cudaMemPool_t pool = p->pool;
    cudaStream_t ost = p->own;
    chk(upload(&p->recs, recs.data(), recs.size(), pool, ost));
    chk(upload(&p->ior_at, at.data(), at.size(), pool, ost));
    chk(upload(&p->ior_bf, bf.data(), bf.size(), pool, ost));
    chk(upload(&p->spec, sp.data(), sp.size(), pool, ost));
    chk(upload(&p->items, items.data(), items.size(), pool, ost));
    chk(upload(&p->pairs, pd.data(), pd.size(), pool, ost));
    chk(upload(&p->sources, src.data(), src.size(), pool, ost));
    chk(upload(&p->samples, reinterpret_cast<const float2*>(ordered.data()), (size_t)n_samples, pool, ost));
    chk(alloc(&p->counter, sizeof(int), pool, ost));
    chk(alloc(&p->traced, 2 * sizeof(unsigned long long), pool, ost));
    if (p->cull)
    {
        chk(upload(&p->probe_items, pitems.data(), pitems.size(), pool, ost));
        chk(upload(&p->probe_samples, reinterpret_cast<const float2*>(psamples.data()), psamples.size(), pool, ost));
        chk(alloc(&p->pair_hits, sizeof(int) * std::max(1, n_pairs), pool, ost));
        chk(upload(&p->pair_hits_init, hits_init.data(), hits_init.size(), pool, ost));
        chk(alloc(&p->probe_counters, sizeof(int) * 4, pool, ost));
        if (n_src == 1 && n_spec > 1 && p->probe_samples_n > 0 && p->probe_samples_n < 65536)
        {
            const size_t cells = (size_t)std::max(1, n_pairs) * p->probe_samples_n;
            chk(alloc(&p->probe_death, cells, pool, ost));
            // the identity order to start from: every entry a valid sample of its own pass
            std::vector<unsigned short> ident(cells);
            for (size_t c = 0; c < cells; ++c) ident[c] = (unsigned short)(c % (size_t)p->probe_samples_n);
            chk(upload(&p->probe_perm, ident.data(), ident.size(), pool, ost));
        }
    }
    chk(alloc(&p->accum, (size_t)prm->width * prm->height * sizeof(float4), pool, ost));
    if (e == cudaSuccess) chk(cudaMemsetAsync(p->accum, 0, (size_t)prm->width * prm->height * sizeof(float4), ost));
    // the host vectors above go out of scope: the uploads must have landed
    chk(cudaStreamSynchronize(ost));
    p->smem = render_smem(n_surf, n_spec);
    int per_sm = 0, n_sm = 0;
    if (e == cudaSuccess) chk(render_prepare(p->smem, &per_sm, &n_sm));
    if (e != cudaSuccess)
    {
        plan_free(p);
        return fail(e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA,
                    std::string("render_ghosts: ") + cudaGetErrorString(e));
    }
    const int warps_per_block = kRenderThreads / 32;
    p->per_sm = std::max(1, per_sm);
    p->n_sm = n_sm;
    p->grid_persistent = std::max(1, std::min((p->n_items + warps_per_block - 1) / warps_per_block,
                                              p->per_sm * n_sm));
    *out = p;
    return GL_OK;
}

// Launch shape of the batched render (the autotuner's knob): items_per_warp
// 0 = persistent work queue over ctas_per_sm CTAs per SM (0 = every resident
// slot); > 0 = one-shot CTAs of that many 32-sample items per warp.
int plan_set_launch(GhostPlan* p, int items_per_warp, int ctas_per_sm)
{
    if (items_per_warp < 0 || ctas_per_sm < 0) return fail(GL_ERR_INVALID, "ghost_plan_set_launch: negative value");
    const int cps = ctas_per_sm == 0 ? p->per_sm : std::min(ctas_per_sm, p->per_sm);
    const int warps_per_block = kRenderThreads / 32;
    p->launch_ipw = items_per_warp;
    p->grid_persistent = std::max(1, std::min((p->n_items + warps_per_block - 1) / warps_per_block, cps * p->n_sm));
    return GL_OK;
}

// An event recorded inside a stream capture becomes an event-record node
// (external), so a replayed graph records it too.
static cudaError_t record_event(cudaEvent_t ev, cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return e;
    return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal)
                                               : cudaEventRecord(ev, st);
}

int plan_execute(GhostPlan* p, float* d_out_r, float* d_out_g, float* d_out_b, cudaStream_t st)
{
    if (!p || !d_out_r || !d_out_g || !d_out_b) return fail(GL_ERR_INVALID, "render_ghosts: null output");
    const size_t n_px = (size_t)p->width * p->height;
    int launches = 0;
    GL_CUDA_TRY(cudaMemsetAsync(p->accum, 0, n_px * sizeof(float4), st));
    RenderArgs A{};
    A.recs = p->recs; A.ior_at = p->ior_at; A.ior_bf = p->ior_bf; A.spec = p->spec;
    A.items = p->items; A.pairs = p->pairs; A.sources = p->sources; A.samples = p->samples;
    A.counter = nullptr; A.accum = p->accum;
    A.n_surf = p->n_surf; A.n_spec = p->n_spec; A.n_items = p->n_items; A.item_base = 0;
    A.l_chunks = p->l_chunks;
    A.width = p->width; A.height = p->height;
    A.fmt_w = (float)p->prm.fmt_w; A.fmt_h = (float)p->prm.fmt_h;
    A.fmt_x0 = (float)p->prm.fmt_x0; A.fmt_y0 = (float)p->prm.fmt_y0;
    A.hw2 = 2.0f * p->prm.sensor_half_w; A.hh2 = 2.0f * p->prm.sensor_half_h;
    A.gain = p->prm.flare_gain;
    A.front_R = p->front_R; A.start_z = p->start_z;
    A.pair_hits = nullptr;
    A.traced = p->traced;
    GL_CUDA_TRY(cudaMemsetAsync(p->traced, 0, 2 * sizeof(unsigned long long), st));
    if (p->ev_probe) GL_CUDA_TRY(record_event(p->ev_probe, st));
    if (p->cull && p->n_items > 0)
    {
        // Probe passes: the frame inflated by CULL_MARGIN = 1.25
        // (ghost_render.cu:148).  The three passes are one persistent launch
        // over their items in pass order: a pair is culled only when no item
        // of any pass hits, and an item whose pair already has a hit is
        // skipped, so a later pass re-probes only the pairs still without one
        // (the reference's candidate rule) without a launch boundary per pass.
        GL_CUDA_TRY(cudaMemcpyAsync(p->pair_hits, p->pair_hits_init, sizeof(int) * p->n_pairs,
                                    cudaMemcpyDeviceToDevice, st));
        GL_CUDA_TRY(cudaMemsetAsync(p->probe_counters, 0, sizeof(int) * 4, st));
        RenderArgs B = A;
        B.samples = p->probe_samples;
        B.items = p->probe_items;
        B.pair_hits = p->pair_hits;
        B.traced = p->traced + 1;
        B.hw2 = 2.0f * (p->prm.sensor_half_w * 1.25f);
        B.hh2 = 2.0f * (p->prm.sensor_half_h * 1.25f);
        const int warps_per_block = kRenderThreads / 32;
        const int n_it = p->probe_begin[3];
        if (n_it > 0)
        {
            B.items = p->probe_items;
            B.n_items = n_it;
            B.counter = p->probe_counters;
            const int grid = std::max(1, std::min((n_it + warps_per_block - 1) / warps_per_block, p->grid_persistent));
            if (p->probe_perm != nullptr)
            {
                // stage 1: every probe ray's first wavelength, recording where it died
                RenderArgs B1 = B;
                B1.lam_lo = 0; B1.lam_hi = 1; B1.l_chunks = 1;
                B1.death = p->probe_death; B1.perm_stride = p->probe_samples_n;
                ghost_render_kernel<true><<<grid, kRenderThreads, p->smem, st>>>(B1);
                const int* sb = p->probe_sample_begin;
                probe_sort_kernel<<<dim3((unsigned)p->n_pairs, 3), 32, 0, st>>>(
                    p->probe_death, p->probe_perm, p->pair_hits, p->probe_samples_n, sb[0], sb[1], sb[2], sb[3]);
                // stage 2: the other wavelengths of the pairs still without a hit, samples in sorted order
                RenderArgs B2 = B;
                B2.lam_lo = 1; B2.lam_hi = p->n_spec;
                B2.perm = p->probe_perm; B2.perm_stride = p->probe_samples_n;
                B2.counter = p->probe_counters + 1;
                ghost_render_kernel<true><<<grid, kRenderThreads, p->smem, st>>>(B2);
                launches += 3;
            }
            else
            {
                ghost_render_kernel<true><<<grid, kRenderThreads, p->smem, st>>>(B);
                ++launches;
            }
        }
        GL_CUDA_TRY(cudaGetLastError());
        A.pair_hits = p->pair_hits;
    }
    if (p->ev_render) GL_CUDA_TRY(record_event(p->ev_render, st));
    if (p->n_items > 0)
    {
        if (p->prm.plain_per_pair)
        {
            // The reference's per-ghost loop: one launch per pair, sized to it.
            for (int i = 0; i < p->n_pairs; ++i)
            {
                const int b0 = p->pair_item_begin[i], b1 = p->pair_item_begin[i + 1];
                if (b1 <= b0) continue;
                A.item_base = b0;
                A.n_items = b1;
                const int warps_per_block = kRenderThreads / 32;
                ghost_render_kernel<false><<<(b1 - b0 + warps_per_block - 1) / warps_per_block, kRenderThreads, p->smem, st>>>(A);
                ++launches;
            }
            GL_CUDA_TRY(cudaGetLastError());
        }
        else if (p->launch_ipw > 0)
        {
            const int per_cta = (kRenderThreads / 32) * p->launch_ipw;
            const int grid = std::max(1, (p->n_items + per_cta - 1) / per_cta);
            ghost_render_kernel<false><<<grid, kRenderThreads, p->smem, st>>>(A);
            GL_CUDA_TRY(cudaGetLastError());
            ++launches;
        }
        else
        {
            GL_CUDA_TRY(cudaMemsetAsync(p->counter, 0, sizeof(int), st));
            A.counter = p->counter;
            ghost_render_kernel<false><<<p->grid_persistent, kRenderThreads, p->smem, st>>>(A);
            GL_CUDA_TRY(cudaGetLastError());
            ++launches;
        }
    }
    if (p->ev_end) GL_CUDA_TRY(record_event(p->ev_end, st));
    const float* C = p->prm.correction;
    const size_t quads = (n_px + 3) / 4;
    const int fb = 256;
    ghost_flush_kernel<<<(unsigned)((quads + fb - 1) / fb), fb, 0, st>>>(
        p->accum, n_px, d_out_r, d_out_g, d_out_b, p->prm.apply_correction,
        C[0], C[1], C[2], C[3], C[4], C[5], C[6], C[7], C[8]);
    GL_CUDA_TRY(cudaGetLastError());
    ++launches;
    // completion marker for destroy (see GhostPlan::done)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    GL_CUDA_TRY(cudaStreamIsCapturing(st, &cs));
    if (cs == cudaStreamCaptureStatusActive)
        p->captured = true;
    else
    {
        GL_CUDA_TRY(cudaEventRecord(p->done, st));
        p->executed = true;
    }
    g_last_launches = launches;
    return GL_OK;
}

// ---------------------------------------------------------------------------
// Batched ray trace (trace_ghost_ray / trace_primary_ray, trace.cpp:171,243)
// with an arbitrary wavelength per ray: the IOR of every surface is
// evaluated per ray from the dispersion data.
// ---------------------------------------------------------------------------
struct DispRec {
    int model;
    float nd, vd, pad;
    float B[3], C[3];
};

__device__ __forceinline__ float disp_ior(const DispRec& d, float lam)
{
    if (d.model == GL_DISP_SELLMEIER)
    {
        float l = lam * 1e-3f;
        float l2 = l * l;
        float n2 = 1.0f;
        n2 += d.B[0] * l2 / (l2 - d.C[0]);
        n2 += d.B[1] * l2 / (l2 - d.C[1]);
        n2 += d.B[2] * l2 / (l2 - d.C[2]);
        return (n2 > 0.0f) ? sqrtf(n2) : 1.0f;
    }
    const float n_d = d.nd, V_d = d.vd;
    if (V_d < 0.1f || n_d <= 1.0001f) return n_d;
    const float lF = 486.13f, lC = 656.27f, ld = 587.56f;
    float dn = (n_d - 1.0f) / V_d;
    float iF = 1.0f / (lF * lF), iC = 1.0f / (lC * lC), id = 1.0f / (ld * ld);
    float B = dn / (iF - iC);
    float Aa = n_d - B * id;
    return Aa + B / (lam * lam);
}

__global__ void __launch_bounds__(128) trace_rays_kernel(const SurfRec* __restrict__ recs,
                                                         const DispRec* __restrict__ disp, int n,
                                                         int a, int b, const float* __restrict__ rays,
                                                         int n_rays, float* __restrict__ out)
{
    __shared__ SurfRec lens[kMaxSurfaces];
    __shared__ DispRec dr[kMaxSurfaces];
    {
        const int words = n * (int)(sizeof(SurfRec) / 4);
        for (int i = threadIdx.x; i < words; i += blockDim.x)
            reinterpret_cast<int*>(lens)[i] = reinterpret_cast<const int*>(recs)[i];
        const int dw = n * (int)(sizeof(DispRec) / 4);
        for (int i = threadIdx.x; i < dw; i += blockDim.x)
            reinterpret_cast<int*>(dr)[i] = reinterpret_cast<const int*>(disp)[i];
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_rays) return;
    const float* r = rays + 7 * (size_t)i;
    const float lam = r[6];
    float at[kMaxSurfaces], bf[kMaxSurfaces];
    float last = 1.0f;
    for (int k = 0; k < n; ++k)
    {
        at[k] = disp_ior(dr[k], lam);
        bf[k] = last;
        if (lens[k].flags & SF_ACTIVE) last = at[k];
    }
    const V3 o = v3(r[0], r[1], r[2]), d = v3(r[3], r[4], r[5]);
    TraceOut t = (b < 0) ? trace_primary(lens, n, at, o, d, lam) : trace_ghost(lens, n, at, bf, o, d, lam, a, b);
    float* q = out + 5 * (size_t)i;
    q[0] = t.x; q[1] = t.y; q[2] = t.z; q[3] = t.w; q[4] = (float)t.status;
}

}  // namespace gl

using namespace gl;

struct gl_ghost_plan { GhostPlan* p; };

extern "C" {

int gl_ghost_plan_create(const gl_surface* surfaces, int n_surfaces, const gl_ghost_pair* pairs,
                         const float* area_boosts, const int32_t* pair_grid, int n_pairs,
                         const gl_flare_source* sources, int n_sources, const gl_pupil_sample* samples,
                         const int32_t* grid_offsets, int n_grids, const gl_spectral_sample* spec,
                         int n_spec, const gl_ghost_render_params* params, gl_ghost_plan** out)
{
    if (!out) return fail(GL_ERR_INVALID, "ghost_plan_create: null out");
    GhostPlan* p = nullptr;
    int rc = plan_create(surfaces, n_surfaces, pairs, area_boosts, pair_grid, n_pairs, sources, n_sources,
                         samples, grid_offsets, n_grids, spec, n_spec, params, &p);
    if (rc) return rc;
    *out = new gl_ghost_plan{p};
    return GL_OK;
}

int gl_ghost_plan_execute(gl_ghost_plan* plan, float* d_out_r, float* d_out_g, float* d_out_b, void* stream)
{
    if (!plan) return fail(GL_ERR_INVALID, "ghost_plan_execute: null plan");
    return plan_execute(plan->p, d_out_r, d_out_g, d_out_b, (cudaStream_t)stream);
}

int gl_morton_order(const gl_pupil_sample* in, int n, gl_pupil_sample* out)
{
    if (n < 0 || (n > 0 && (!in || !out))) return fail(GL_ERR_INVALID, "morton_order: bad arguments");
    morton_order(in, n, out);
    return GL_OK;
}

int gl_ghost_plan_set_launch(gl_ghost_plan* plan, int items_per_warp, int ctas_per_sm)
{
    if (!plan) return fail(GL_ERR_INVALID, "ghost_plan_set_launch: null plan");
    return plan_set_launch(plan->p, items_per_warp, ctas_per_sm);
}

int gl_ghost_plan_set_lambda_split(gl_ghost_plan* plan, int chunks)
{
    if (!plan) return fail(GL_ERR_INVALID, "ghost_plan_set_lambda_split: null plan");
    if (chunks < 1) return fail(GL_ERR_INVALID, "ghost_plan_set_lambda_split: chunks must be >= 1");
    plan->p->l_chunks = std::min(chunks, plan->p->n_spec);
    return GL_OK;
}

int gl_ghost_plan_info(const gl_ghost_plan* plan, long long* rays, int* n_items, int* grid)
{
    if (!plan) return fail(GL_ERR_INVALID, "ghost_plan_info: null plan");
    if (rays) *rays = plan->p->rays + plan->p->probe_rays;
    if (n_items) *n_items = plan->p->n_items;
    if (grid) *grid = plan->p->grid_persistent;
    return GL_OK;
}

int gl_ghost_plan_traced(const gl_ghost_plan* plan, long long* out)
{
    if (!plan || !out) return fail(GL_ERR_INVALID, "ghost_plan_traced: bad arguments");
    unsigned long long v[2] = {0, 0};
    GL_CUDA_TRY(cudaMemcpy(v, plan->p->traced, sizeof(v), cudaMemcpyDeviceToHost));
    *out = (long long)(v[0] + v[1]);
    return GL_OK;
}

// The diagnostic stats pass (launch_ghost_render's collect_stats launch,
// ghost_render.cu:1357-1431): every render item of the plan traced again
// without weights or splat and without the off-sensor cull, counting per pair
// the ray-wavelength traces, the rays that left the lens and those landing
// inside the frame.  out: 3 x n_pairs host counters {traces, survived, on
// sensor}, pair-major.  Synchronises the stream.
int gl_ghost_plan_stats(gl_ghost_plan* plan, unsigned long long* out, void* stream)
{
    if (!plan || !out) return fail(GL_ERR_INVALID, "ghost_plan_stats: null argument");
    GhostPlan* p = plan->p;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t bytes = sizeof(unsigned long long) * 3 * (size_t)std::max(1, p->n_pairs);
    unsigned long long* d = nullptr;
    GL_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&d), bytes, st));
    cudaError_t e = cudaMemsetAsync(d, 0, bytes, st);
    if (e == cudaSuccess && p->n_items > 0)
    {
        RenderArgs A{};
        A.recs = p->recs; A.ior_at = p->ior_at; A.ior_bf = p->ior_bf; A.spec = p->spec;
        A.items = p->items; A.pairs = p->pairs; A.sources = p->sources; A.samples = p->samples;
        A.accum = p->accum;
        A.n_surf = p->n_surf; A.n_spec = p->n_spec; A.n_items = p->n_items; A.item_base = 0;
        A.l_chunks = 1;
        A.width = p->width; A.height = p->height;
        A.fmt_w = (float)p->prm.fmt_w; A.fmt_h = (float)p->prm.fmt_h;
        A.fmt_x0 = (float)p->prm.fmt_x0; A.fmt_y0 = (float)p->prm.fmt_y0;
        A.hw2 = 2.0f * p->prm.sensor_half_w; A.hh2 = 2.0f * p->prm.sensor_half_h;
        A.gain = p->prm.flare_gain;
        A.front_R = p->front_R; A.start_z = p->start_z;
        A.stats = d;
        const int warps_per_block = kRenderThreads / 32;
        ghost_render_kernel<true><<<(p->n_items + warps_per_block - 1) / warps_per_block, kRenderThreads, p->smem,
                                    st>>>(A);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, sizeof(unsigned long long) * 3 * p->n_pairs,
                                              cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(GL_ERR_CUDA, std::string("ghost_plan_stats: ") + cudaGetErrorString(e));
    g_last_launches = 1;
    return GL_OK;
}

int gl_ghost_plan_traced_split(const gl_ghost_plan* plan, long long* render, long long* probe)
{
    if (!plan) return fail(GL_ERR_INVALID, "ghost_plan_traced_split: null plan");
    unsigned long long v[2] = {0, 0};
    GL_CUDA_TRY(cudaMemcpy(v, plan->p->traced, sizeof(v), cudaMemcpyDeviceToHost));
    if (render) *render = (long long)v[0];
    if (probe) *probe = (long long)v[1];
    return GL_OK;
}

int gl_ghost_plan_set_timing(gl_ghost_plan* plan, void* ev_probe, void* ev_render, void* ev_end)
{
    if (!plan) return fail(GL_ERR_INVALID, "ghost_plan_set_timing: null plan");
    plan->p->ev_probe = (cudaEvent_t)ev_probe;
    plan->p->ev_render = (cudaEvent_t)ev_render;
    plan->p->ev_end = (cudaEvent_t)ev_end;
    return GL_OK;
}

int gl_ghost_plan_pair_hits(const gl_ghost_plan* plan, int32_t* out, int n)
{
    if (!plan || !out || n < plan->p->n_pairs) return fail(GL_ERR_INVALID, "ghost_plan_pair_hits: bad arguments");
    if (!plan->p->cull) { for (int i = 0; i < plan->p->n_pairs; ++i) out[i] = 1; return GL_OK; }
    GL_CUDA_TRY(cudaMemcpy(out, plan->p->pair_hits, sizeof(int) * plan->p->n_pairs, cudaMemcpyDeviceToHost));
    return GL_OK;
}

int gl_ghost_plan_destroy(gl_ghost_plan* plan)
{
    if (!plan) return GL_OK;
    plan_free(plan->p);
    delete plan;
    return GL_OK;
}

int gl_render_ghosts(const gl_surface* surfaces, int n_surfaces, const gl_ghost_pair* pairs,
                     const float* area_boosts, const int32_t* pair_grid, int n_pairs,
                     const gl_flare_source* sources, int n_sources, const gl_pupil_sample* samples,
                     const int32_t* grid_offsets, int n_grids, const gl_spectral_sample* spec, int n_spec,
                     const gl_ghost_render_params* params, float* d_out_r, float* d_out_g, float* d_out_b,
                     void* stream)
{
    GhostPlan* p = nullptr;
    int rc = plan_create(surfaces, n_surfaces, pairs, area_boosts, pair_grid, n_pairs, sources, n_sources,
                         samples, grid_offsets, n_grids, spec, n_spec, params, &p);
    if (rc) return rc;
    rc = plan_execute(p, d_out_r, d_out_g, d_out_b, (cudaStream_t)stream);
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    plan_free(p);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(GL_ERR_CUDA, std::string("render_ghosts: ") + cudaGetErrorString(e));
    return GL_OK;
}

int gl_trace_rays(const gl_surface* surfaces, int n, int bounce_a, int bounce_b, const float* d_rays,
                  int n_rays, float* d_out, void* stream)
{
    if (!surfaces || n <= 0) return fail(GL_ERR_INVALID, "trace_rays: lens has no surfaces");
    if (bounce_b >= 0 && (bounce_a < 0 || bounce_a >= bounce_b || bounce_b >= n))
        return fail(GL_ERR_INVALID, "bounce indices must satisfy 0 <= bounce_a < bounce_b < num_surfaces");
    if (n_rays < 0 || (n_rays > 0 && (!d_rays || !d_out))) return fail(GL_ERR_INVALID, "trace_rays: bad ray buffers");
    if (n_rays == 0) return GL_OK;
    int dev = 0;
    GL_CUDA_TRY(cudaGetDevice(&dev));
    std::vector<SurfRec> recs((size_t)n);
    int rc = pack_lens(surfaces, n, recs.data(), dev);
    if (rc) return rc;
    std::vector<DispRec> disp((size_t)n);
    for (int i = 0; i < n; ++i)
    {
        disp[i].model = surfaces[i].disp_model;
        disp[i].nd = surfaces[i].ior; disp[i].vd = surfaces[i].abbe_v; disp[i].pad = 0.0f;
        for (int k = 0; k < 3; ++k) { disp[i].B[k] = surfaces[i].sellmeier_B[k]; disp[i].C[k] = surfaces[i].sellmeier_C[k]; }
    }
    cudaStream_t st = (cudaStream_t)stream;
    SurfRec* d_recs = nullptr; DispRec* d_disp = nullptr;
    GL_CUDA_TRY(cudaMallocAsync(&d_recs, sizeof(SurfRec) * n, st));
    GL_CUDA_TRY(cudaMallocAsync(&d_disp, sizeof(DispRec) * n, st));
    GL_CUDA_TRY(cudaMemcpyAsync(d_recs, recs.data(), sizeof(SurfRec) * n, cudaMemcpyHostToDevice, st));
    GL_CUDA_TRY(cudaMemcpyAsync(d_disp, disp.data(), sizeof(DispRec) * n, cudaMemcpyHostToDevice, st));
    trace_rays_kernel<<<(n_rays + 127) / 128, 128, 0, st>>>(d_recs, d_disp, n, bounce_a, bounce_b, d_rays, n_rays, d_out);
    GL_CUDA_TRY(cudaGetLastError());
    GL_CUDA_TRY(cudaFreeAsync(d_recs, st));
    GL_CUDA_TRY(cudaFreeAsync(d_disp, st));
    // The host vectors above must outlive the async copies.
    GL_CUDA_TRY(cudaStreamSynchronize(st));
    g_last_launches = 1;
    return GL_OK;
}

}  // extern "C"

// ===========================================================================
// Allocation-free batched trace
//
// Some callers cannot allocate device memory while they run: a plug-in hosted
// by an application that owns the device heap through its own allocator, code
// on a real-time thread where an allocation's latency (and the device-wide
// synchronisation cudaMalloc may imply) is not allowed, or a host that has
// already reserved the whole device.  For them this entry point keeps the
// only scratch the trace needs — the packed lens records and dispersion
// terms — in one fixed array in device memory that is part of this library,
// sized for the largest lens the path accepts (64 surfaces).  The caller
// still passes the ray buffer and the result buffer.
//
// Every call looks up the array's device address with cudaGetSymbolAddress
// on the current device (the lookup allocates nothing), so the address is
// never stale, e.g. after a cudaDeviceReset.  A call ends with a
// cudaStreamSynchronize (the lens records are staged on its stack frame), so
// it must not be made while `stream` is being captured: it returns
// GL_ERR_INVALID there instead of breaking the caller's capture.  All calls
// share the array and it keeps whatever the last call wrote: each call
// overwrites the records it uses before launching, and calls that overlap on
// the GPU (other threads or streams) race on it.
// ===========================================================================
namespace gl {

constexpr int kNoAllocMaxSurfaces = 64;

struct NoAllocTables {
    SurfRec recs[kNoAllocMaxSurfaces];
    DispRec disp[kNoAllocMaxSurfaces];
};

static __device__ __align__(256) unsigned char g_trace_tables[sizeof(NoAllocTables)];

static int trace_tables_address(void** out)
{
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_trace_tables);
    if (e != cudaSuccess || ptr == nullptr)
        return fail(GL_ERR_CUDA, std::string("trace_rays_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    *out = ptr;
    return GL_OK;
}

}  // namespace gl

extern "C" int gl_trace_rays_noalloc(const gl_surface* surfaces, int n, int bounce_a, int bounce_b,
                                     const float* d_rays, int n_rays, float* d_out, void* stream)
{
    if (!surfaces || n <= 0) return fail(GL_ERR_INVALID, "trace_rays_noalloc: lens has no surfaces");
    if (n > kNoAllocMaxSurfaces)
        return fail(GL_ERR_INVALID, "trace_rays_noalloc: lens has more than 64 surfaces, the size of the fixed table");
    if (bounce_b >= 0 && (bounce_a < 0 || bounce_a >= bounce_b || bounce_b >= n))
        return fail(GL_ERR_INVALID, "bounce indices must satisfy 0 <= bounce_a < bounce_b < num_surfaces");
    if (n_rays < 0 || (n_rays > 0 && (!d_rays || !d_out))) return fail(GL_ERR_INVALID, "trace_rays_noalloc: bad ray buffers");
    if (n_rays == 0) return GL_OK;
    cudaStream_t st = (cudaStream_t)stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    GL_CUDA_TRY(cudaStreamIsCapturing(st, &cap));
    if (cap != cudaStreamCaptureStatusNone)
        return fail(GL_ERR_INVALID, "trace_rays_noalloc: the call synchronises its stream and cannot be captured");
    int device = 0;
    GL_CUDA_TRY(cudaGetDevice(&device));
    void* base = nullptr;
    int rc = trace_tables_address(&base);
    if (rc) return rc;
    NoAllocTables host;   // staged on the stack: no heap, no device allocation
    rc = pack_lens(surfaces, n, host.recs, device, false);
    if (rc) return rc;
    for (int i = 0; i < n; ++i)
    {
        host.disp[i].model = surfaces[i].disp_model;
        host.disp[i].nd = surfaces[i].ior; host.disp[i].vd = surfaces[i].abbe_v; host.disp[i].pad = 0.0f;
        for (int k = 0; k < 3; ++k) { host.disp[i].B[k] = surfaces[i].sellmeier_B[k]; host.disp[i].C[k] = surfaces[i].sellmeier_C[k]; }
    }
    NoAllocTables* dev_tables = static_cast<NoAllocTables*>(base);
    GL_CUDA_TRY(cudaMemcpyAsync(dev_tables->recs, host.recs, sizeof(SurfRec) * n, cudaMemcpyHostToDevice, st));
    GL_CUDA_TRY(cudaMemcpyAsync(dev_tables->disp, host.disp, sizeof(DispRec) * n, cudaMemcpyHostToDevice, st));
    trace_rays_kernel<<<(n_rays + 127) / 128, 128, 0, st>>>(dev_tables->recs, dev_tables->disp, n, bounce_a,
                                                            bounce_b, d_rays, n_rays, d_out);
    GL_CUDA_TRY(cudaGetLastError());
    // The staging copy lives on this stack frame until the copies are done.
    GL_CUDA_TRY(cudaStreamSynchronize(st));
    g_last_launches = 1;
    return GL_OK;
}
