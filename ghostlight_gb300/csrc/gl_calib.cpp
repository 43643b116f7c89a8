// gl_calib.cpp — first-order lens calibration and the source-position solve,
// by tracing the spawn disc (host, float32).
//
// Restates calibrate_lens (lens_calibration.cpp:24-443), the spawn-disc probe
// (spawn_probe.cpp:28-211), the 2x2 finite-difference Newton aim
// (newton_aim.h:20-63) and solve_source_angle / source_map_screen
// (source_map.cpp:61-483) in float32 with the same operation order, so the
// calibration a flare render is sized by equals the reference's bit for bit
// (this translation unit is compiled with -ffp-contract=off, like the
// reference host build).  The traces are the reference-formulation
// trace_primary of gl_trace.cuh with per-wavelength IOR slices.
//
// Bladed stops carry their authored shape (gl_blade.h): the traces test it and
// the pupil area fraction is its enclosed area (lens_calibration.cpp:363).
#include "gl_internal.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace gl {
namespace {

constexpr float kPiF = 3.14159265358979323846f;

struct Window {
    float cu = 0.0f, cv = 0.0f;
    float r = 1.0f;
};

struct DiscArea {
    float area = 0.0f, mean_x = 0.0f, mean_y = 0.0f;
    bool at_edge = false;
    Window fit;
};

// The lens as the probes see it: packed records and IOR slices per wavelength.
struct ProbeLens {
    const gl_surface* s = nullptr;
    int n = 0;
    std::vector<SurfRec> recs;
    float lam = 0.0f;
    std::vector<float> at, bf;
    PupilMask mask;
    float front_R = 0.0f;

    void set_lambda(float l)
    {
        if (l == lam && !at.empty()) return;
        lam = l;
        at.assign((size_t)n, 0.0f);
        bf.assign((size_t)n, 0.0f);
        build_ior_tables(s, n, &lam, 1, at.data(), bf.data());
    }
};

// A primary ray from the spawn plane (SPAWN_OFFSET ahead of the front vertex)
// at height (hx, hy) with slopes tan(angle); true when it reaches the sensor.
bool trace_from_ok(ProbeLens& L, float hx, float hy, float ah, float av, float lam, TraceOut* out = nullptr)
{
    L.set_lambda(lam);
    const V3 o = v3(hx, hy, L.s[0].z - kSpawnOffset);
    const V3 d = normalized(v3(tanf(ah), tanf(av), 1.0f));
    const TraceOut r = trace_primary(L.recs.data(), L.n, L.at.data(), o, d, lam);
    if (out) *out = r;
    return r.status == GL_TRACE_OK;
}

constexpr int kProbeGrid = 17;
constexpr int kProbeEdgeSS = 2;
constexpr float kDeepStopFill = 0.45f;
constexpr float kWindowDilation = 5.0f;

Window initial_window(float pupil_fill)
{
    Window w;
    if (pupil_fill > 0.0f && pupil_fill < kDeepStopFill) w.r = std::min(1.0f, pupil_fill * kWindowDilation);
    return w;
}

// Coverage-weighted surviving area of the sampled square and the survivors'
// mean landing: cell centres first, then every cell whose 4-neighbourhood
// disagrees about survival (or that survives on the rim) is resampled at
// edge_ss^2 sub-points.
DiscArea probe_window(ProbeLens& L, float ah, float av, float lam, const Window& win, int grid = 0,
                      int edge_ss = 0)
{
    const int n = grid > 0 ? grid : kProbeGrid;
    const int ess = edge_ss > 0 ? edge_ss : kProbeEdgeSS;
    const float step = 2.0f * win.r / (float)n;
    const float bx = tanf(ah), by = tanf(av);
    const float sdx = -kSpawnOffset * bx, sdy = -kSpawnOffset * by;   // the disc follows the beam
    const float front_R = L.front_R;

    std::vector<unsigned char> alive((size_t)n * n, 0);
    std::vector<float> lx((size_t)n * n, 0.0f), ly((size_t)n * n, 0.0f);
    auto sample = [&](float u, float v, float* x, float* y) -> bool {
        if (!pupil_contains(L.mask, u, v)) return false;
        TraceOut r;
        if (!trace_from_ok(L, u * front_R + sdx, v * front_R + sdy, ah, av, lam, &r)) return false;
        if (!std::isfinite(r.x) || !std::isfinite(r.y)) return false;
        *x = r.x;
        *y = r.y;
        return true;
    };
    const float u_org = win.cu - win.r, v_org = win.cv - win.r;
    for (int j = 0; j < n; ++j)
    {
        const float v = v_org + ((float)j + 0.5f) * step;
        for (int i = 0; i < n; ++i)
        {
            const float u = u_org + ((float)i + 0.5f) * step;
            const size_t k = (size_t)j * n + i;
            float x = 0.0f, y = 0.0f;
            if (sample(u, v, &x, &y)) { alive[k] = 1; lx[k] = x; ly[k] = y; }
        }
    }

    DiscArea out;
    const float cell_area = step * step;
    const float sub_w = 1.0f / (float)(ess * ess);
    float lo_u = 1e30f, hi_u = -1e30f, lo_v = 1e30f, hi_v = -1e30f;
    auto note = [&](float u, float v, float w, float x, float y) {
        out.area += w * cell_area;
        out.mean_x += w * cell_area * x;
        out.mean_y += w * cell_area * y;
        lo_u = std::min(lo_u, u); hi_u = std::max(hi_u, u);
        lo_v = std::min(lo_v, v); hi_v = std::max(hi_v, v);
    };
    static const int di[4] = {1, -1, 0, 0};
    static const int dj[4] = {0, 0, 1, -1};
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i)
        {
            const size_t k = (size_t)j * n + i;
            const bool here = alive[k] != 0;
            const float uc = u_org + ((float)i + 0.5f) * step;
            const float vc = v_org + ((float)j + 0.5f) * step;
            const bool rim = (i == 0 || i == n - 1 || j == 0 || j == n - 1);
            if (here && rim) out.at_edge = true;
            bool edge = here && rim;
            for (int q = 0; q < 4 && !edge; ++q)
            {
                const int ni = i + di[q], nj = j + dj[q];
                if (ni < 0 || ni >= n || nj < 0 || nj >= n) continue;
                if ((alive[(size_t)nj * n + ni] != 0) != here) edge = true;
            }
            if (!edge)
            {
                if (here) note(uc, vc, 1.0f, lx[k], ly[k]);
                continue;
            }
            const float u0 = u_org + (float)i * step, v0 = v_org + (float)j * step;
            const float sub = step / (float)ess;
            for (int sj = 0; sj < ess; ++sj)
            {
                const float v = v0 + ((float)sj + 0.5f) * sub;
                for (int si = 0; si < ess; ++si)
                {
                    const float u = u0 + ((float)si + 0.5f) * sub;
                    float x = 0.0f, y = 0.0f;
                    if (!sample(u, v, &x, &y)) continue;
                    note(u, v, sub_w, x, y);
                }
            }
        }
    if (out.area > 0.0f)
    {
        out.mean_x /= out.area;
        out.mean_y /= out.area;
        out.fit.cu = 0.5f * (lo_u + hi_u);
        out.fit.cv = 0.5f * (lo_v + hi_v);
        out.fit.r = std::max(std::max(hi_u - out.fit.cu, hi_v - out.fit.cv), step) + step;
    }
    return out;
}

// The window follows the beam: re-centre on the survivors while the beam
// touches the rim (three tries), then widen by 2.5x, up to the whole disc.
DiscArea probe_disc(ProbeLens& L, float ah, float av, float lam, Window* track, int grid = 0, int edge_ss = 0)
{
    Window win = *track;
    if (win.r >= 1.0f) { win.cu = 0.0f; win.cv = 0.0f; win.r = 1.0f; }
    DiscArea best;
    for (int attempt = 0; attempt < 6; ++attempt)
    {
        const DiscArea d = probe_window(L, ah, av, lam, win, grid, edge_ss);
        if (d.area > 0.0f) best = d;
        if (d.area > 0.0f && !d.at_edge)
        {
            *track = d.fit;
            track->r = win.r;
            return d;
        }
        if (win.r >= 1.0f) break;
        if (d.area > 0.0f && attempt < 3)
        {
            win.cu = d.fit.cu;
            win.cv = d.fit.cv;
            continue;
        }
        win.r = std::min(1.0f, win.r * 2.5f);
        if (win.r >= 1.0f) { win.cu = 0.0f; win.cv = 0.0f; }
    }
    track->cu = win.cu; track->cv = win.cv; track->r = win.r;
    return best;
}

// ---- first-order optics --------------------------------------------------------
float paraxial_efl(ProbeLens& L, float lam, bool horizontal)
{
    const float theta = (float)(1.0 * 3.14159265358979323846 / 180.0);
    TraceOut r;
    const bool ok = horizontal ? trace_from_ok(L, 0.0f, 0.0f, theta, 0.0f, lam, &r)
                               : trace_from_ok(L, 0.0f, 0.0f, 0.0f, theta, lam, &r);
    if (!ok) return 0.0f;
    const float h = horizontal ? r.x : r.y;
    if (!std::isfinite(h)) return 0.0f;
    return std::fabs(h) / tanf(theta);
}

float marginal_semi_along(ProbeLens& L, float lam, float ux, float uy)
{
    const float R = L.front_R;
    if (R <= 0.0f) return 0.0f;
    if (!trace_from_ok(L, 0.0f, 0.0f, 0.0f, 0.0f, lam)) return 0.0f;
    if (trace_from_ok(L, R * ux, R * uy, 0.0f, 0.0f, lam)) return R;
    float lo = 0.0f, hi = R;
    for (int it = 0; it < 40; ++it)
    {
        const float mid = 0.5f * (lo + hi);
        if (trace_from_ok(L, mid * ux, mid * uy, 0.0f, 0.0f, lam)) lo = mid;
        else hi = mid;
    }
    return lo;
}

void marginal_support(ProbeLens& L, const gl_surface& stop, float lam, float* sx, float* sy)
{
    const int n = stop.aperture_blades * 8;
    const float rot = stop.aperture_rotation_rad;
    float bx = 0.0f, by = 0.0f;
    auto consider = [&](float th) {
        const float c = cosf(th), s = sinf(th);
        const float h = marginal_semi_along(L, lam, c, s);
        bx = std::max(bx, h * std::fabs(c));
        by = std::max(by, h * std::fabs(s));
    };
    for (int i = 0; i < n; ++i) consider(rot + (float)(2.0 * 3.14159265358979323846) * (float)i / (float)n);
    consider(0.0f);
    consider((float)(3.14159265358979323846 / 2.0));
    *sx = bx;
    *sy = by;
}

// ---- covered field ----------------------------------------------------------------
const float kLadderDeg[8] = {0.0f, 4.0f, 8.0f, 14.0f, 22.0f, 32.0f, 45.0f, 60.0f};
constexpr int kLadder = 8;
constexpr float kRefineTolDeg = 0.15f;
constexpr int kMaxRefine = 7;
constexpr float kCircleTolDeg = 1.0f;
constexpr int kMaxRefineCircle = 2;
constexpr float kMapThreshold = 0.90f;
constexpr float kCircleThreshold = 0.05f;

struct FieldSolve {
    float angle = 0.0f, half_mm = 0.0f;
    bool crossed = false;
};

// Walk the field-angle ladder once and refine both threshold crossings of the
// surviving-area fraction with Illinois regula falsi (lens_calibration.cpp:
// 156-303): 90% gives the covered field and its landing, 5% the image circle.
void resolve_axis(ProbeLens& L, float pupil_fill, float lam, bool horizontal, FieldSolve* map_out,
                  FieldSolve* circle_out)
{
    Window track = initial_window(pupil_fill);
    const float DEG = (float)(3.14159265358979323846 / 180.0);
    *map_out = FieldSolve{};
    *circle_out = FieldSolve{};
    DiscArea axial;
    float axial_r = -1.0f;
    auto at = [&](float angle) {
        const DiscArea d = probe_disc(L, horizontal ? angle : 0.0f, horizontal ? 0.0f : angle, lam, &track);
        if (track.r != axial_r)
        {
            Window ax;
            ax.cu = 0.0f; ax.cv = 0.0f; ax.r = track.r;
            axial = probe_window(L, 0.0f, 0.0f, lam, ax);
            axial_r = track.r;
        }
        return d;
    };
    at(0.0f);
    if (axial.area <= 0.0f) return;
    int map_cross = -1, circle_cross = -1;
    float f_prev = 1.0f;
    float f_map[2] = {1.0f, 0.0f}, f_circle[2] = {1.0f, 0.0f};
    Window seed_map = track, seed_circle = track;
    for (int i = 1; i < kLadder; ++i)
    {
        const Window before = track;
        const float f = at(kLadderDeg[i] * DEG).area / axial.area;
        if (map_cross < 0 && f < kMapThreshold)
        {
            map_cross = i - 1;
            f_map[0] = f_prev; f_map[1] = f;
            seed_map = before;
        }
        if (circle_cross < 0 && f < kCircleThreshold)
        {
            circle_cross = i - 1;
            f_circle[0] = f_prev; f_circle[1] = f;
            seed_circle = before;
            break;
        }
        f_prev = f;
    }
    auto refine = [&](int cross, float thr, const float f_ends[2], const Window& seed, int max_steps,
                      float tol_deg) -> FieldSolve {
        FieldSolve r;
        auto probe_at = [&](float angle) {
            track.cu = seed.cu;
            track.cv = seed.cv;
            return at(angle);
        };
        if (cross < 0)
        {
            const DiscArea d = probe_at(kLadderDeg[kLadder - 1] * DEG);
            r.angle = kLadderDeg[kLadder - 1] * DEG;
            r.half_mm = std::fabs(horizontal ? d.mean_x : d.mean_y);
            r.crossed = false;
            return r;
        }
        float lo = kLadderDeg[cross] * DEG, hi = kLadderDeg[cross + 1] * DEG;
        float f_lo = f_ends[0] - thr, f_hi = f_ends[1] - thr;
        float t_lo = f_lo, t_hi = f_hi;
        const float tol = tol_deg * DEG;
        for (int it = 0; it < max_steps && (hi - lo) > tol; ++it)
        {
            const float denom = f_lo - f_hi;
            float mid = (std::fabs(denom) < 1e-12f) ? 0.5f * (lo + hi) : lo + (hi - lo) * f_lo / denom;
            const float edge = 0.01f * (hi - lo);
            mid = std::min(std::max(mid, lo + edge), hi - edge);
            const float f_mid = probe_at(mid).area / axial.area - thr;
            if (f_mid >= 0.0f) { lo = mid; f_lo = f_mid; t_lo = f_mid; f_hi *= 0.5f; }
            else { hi = mid; f_hi = f_mid; t_hi = f_mid; f_lo *= 0.5f; }
        }
        const float span = t_lo - t_hi;
        float root = (std::fabs(span) < 1e-12f) ? 0.5f * (lo + hi) : lo + (hi - lo) * t_lo / span;
        root = std::min(std::max(root, lo), hi);
        DiscArea d = probe_at(root);
        if (d.area <= 0.0f)
        {
            root = lo;
            d = probe_at(lo);
        }
        r.angle = root;
        r.half_mm = std::fabs(horizontal ? d.mean_x : d.mean_y);
        r.crossed = true;
        return r;
    };
    *map_out = refine(map_cross, kMapThreshold, f_map, seed_map, kMaxRefine, kRefineTolDeg);
    *circle_out = refine(circle_cross, kCircleThreshold, f_circle, seed_circle, kMaxRefineCircle, kCircleTolDeg);
    if (circle_out->angle < map_out->angle) *circle_out = *map_out;
    if (circle_out->half_mm < map_out->half_mm) circle_out->half_mm = map_out->half_mm;
}

bool axes_symmetric(const gl_surface* s, int n)
{
    static const float I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int i = 0; i < n; ++i)
    {
        if (s[i].form == GL_FORM_CYLINDRICAL) return false;
        if (s[i].aperture_aspect != 1.0f) return false;
        if (s[i].decenter_x != 0.0f || s[i].decenter_y != 0.0f) return false;
        for (int k = 0; k < 9; ++k)
            if (s[i].rot[k] != I[k]) return false;
        if (s[i].aperture_shape == GL_APERTURE_POLYGON)
        {
            if (s[i].aperture_blades % 4 != 0) return false;
            if (s[i].aperture_rotation_rad != 0.0f) return false;
        }
        else if (s[i].aperture_shape != GL_APERTURE_CIRCLE)
        {
            return false;
        }
    }
    return true;
}

int open_lens(const gl_surface* s, int n, ProbeLens& L)
{
    L.s = s;
    L.n = n;
    L.recs.resize((size_t)n);
    const int rc = pack_lens(s, n, L.recs.data(), kTablesHost);
    if (rc) return rc;
    L.mask = resolve_pupil_mask(s, n, 0, 0.0f);
    L.front_R = s[0].semi_aperture;
    return GL_OK;
}

// ---- source-position solve ---------------------------------------------------
constexpr float kSolveLambda = 587.56f;
constexpr int kSolveGrid = 17;
constexpr int kSolveEdgeSS = 2;
constexpr int kMaxIter = 8;
constexpr float kFdStep = 5e-3f;
constexpr float kTolMm = 1e-3f;
constexpr float kAcceptFrac = 0.01f;
constexpr int kBisectSteps = 6;
constexpr float kBisectTolMm = 0.02f;
constexpr float kMaxExtendRad = 1.55f;
constexpr float kWarmStepRad = 0.10f;

// Landing function whose sampling window advances after each successful probe.
struct SolveProbe {
    ProbeLens* L;
    Window win;
    int evals = 0;

    bool at(float ax, float ay, float& x, float& y)
    {
        ++evals;
        Window w = win;
        const DiscArea d = probe_disc(*L, ax, ay, kSolveLambda, &w, kSolveGrid, kSolveEdgeSS);
        const bool ok = (d.area > 0.0f) && std::isfinite(d.mean_x) && std::isfinite(d.mean_y);
        if (!ok) return false;
        win = w;
        x = d.mean_x;
        y = d.mean_y;
        return true;
    }
};

// 2x2 finite-difference Newton towards the target landing; keeps the best
// iterate (newton_aim.h:20-63).
template <class F>
bool newton_aim(F&& landing, float tx, float ty, float& ax, float& ay, float& out_res, int max_iter, float fd,
                float cap, float tol)
{
    float best_ax = ax, best_ay = ay, best_res = 1e30f;
    auto record = [&](float x, float y) {
        const float rx = x - tx, ry = y - ty;
        const float res = sqrtf(rx * rx + ry * ry);
        if (res < best_res) { best_res = res; best_ax = ax; best_ay = ay; }
        return res;
    };
    float cx, cy;
    if (!landing(ax, ay, cx, cy)) { out_res = 1e30f; return false; }
    for (int it = 0; it < max_iter; ++it)
    {
        const float rx = cx - tx, ry = cy - ty;
        if (record(cx, cy) < tol) break;
        float xx, xy, yx, yy;
        if (!landing(ax + fd, ay, xx, xy)) break;
        if (!landing(ax, ay + fd, yx, yy)) break;
        const float Jxx = (xx - cx) / fd, Jyx = (xy - cy) / fd;
        const float Jxy = (yx - cx) / fd, Jyy = (yy - cy) / fd;
        const float det = Jxx * Jyy - Jxy * Jyx;
        if (std::fabs(det) < 1e-12f) break;
        float dax = (-rx * Jyy + ry * Jxy) / det;
        float day = (rx * Jyx - ry * Jxx) / det;
        dax = std::max(-cap, std::min(cap, dax));
        day = std::max(-cap, std::min(cap, day));
        ax += dax;
        ay += day;
        if (!landing(ax, ay, cx, cy)) break;
    }
    if (landing(ax, ay, cx, cy)) record(cx, cy);
    ax = best_ax;
    ay = best_ay;
    out_res = best_res;
    return best_res < tol;
}

bool measure_jacobian(SolveProbe& P, float ax, float ay, float* land, float* J)
{
    float cx, cy;
    if (!P.at(ax, ay, cx, cy)) return false;
    auto slope = [&](float dax, float day, float* dx, float* dy) -> bool {
        float px, py;
        if (P.at(ax + dax, ay + day, px, py)) { *dx = (px - cx) / kFdStep; *dy = (py - cy) / kFdStep; return true; }
        if (P.at(ax - dax, ay - day, px, py)) { *dx = (cx - px) / kFdStep; *dy = (cy - py) / kFdStep; return true; }
        return false;
    };
    float dxdax, dydax, dxday, dyday;
    if (!slope(kFdStep, 0.0f, &dxdax, &dydax)) return false;
    if (!slope(0.0f, kFdStep, &dxday, &dyday)) return false;
    land[0] = cx; land[1] = cy;
    J[0] = dxdax; J[1] = dxday; J[2] = dydax; J[3] = dyday;
    return true;
}

// ---- PSF grid: chief-ray pre-pass (PSFRenderer.cpp:28-243) -------------------
constexpr float kChiefLambda = 587.56f;

// One pupil sample of the beam at (ax, ay), spawn-shifted, at the d line.
bool chief_candidate(ProbeLens& L, float start_z, float front_R, float ax, float ay, float u, float v, float& x,
                     float& y)
{
    const float bx = tanf(ax), by = tanf(ay);
    const float sdx = -kSpawnOffset * bx, sdy = -kSpawnOffset * by;
    L.set_lambda(kChiefLambda);
    const V3 o = v3(u * front_R + sdx, v * front_R + sdy, start_z);
    const V3 d = normalized(v3(bx, by, 1.0f));
    const TraceOut r = trace_primary(L.recs.data(), L.n, L.at.data(), o, d, kChiefLambda);
    if (r.status != GL_TRACE_OK || !std::isfinite(r.x) || !std::isfinite(r.y)) return false;
    x = r.x;
    y = r.y;
    return true;
}

struct PupilProbe {
    int hits = 0;
    float frac = 0.0f, mean_x = 0.0f, mean_y = 0.0f;
};

// N x N unit-disc pupil probe: transmitting fraction and survivor-mean landing.
PupilProbe pupil_probe(ProbeLens& L, float start_z, float front_R, float ax, float ay, int N)
{
    float sx = 0.0f, sy = 0.0f;
    int hits = 0, total = 0;
    for (int iy = 0; iy < N; ++iy)
    {
        const float v = -1.0f + ((float)iy + 0.5f) * (2.0f / (float)N);
        for (int ix = 0; ix < N; ++ix)
        {
            const float u = -1.0f + ((float)ix + 0.5f) * (2.0f / (float)N);
            if (u * u + v * v > 1.0f) continue;
            ++total;
            float x, y;
            if (chief_candidate(L, start_z, front_R, ax, ay, u, v, x, y)) { sx += x; sy += y; ++hits; }
        }
    }
    PupilProbe p;
    p.hits = hits;
    p.frac = total > 0 ? (float)hits / (float)total : 0.0f;
    p.mean_x = hits > 0 ? sx / (float)hits : 0.0f;
    p.mean_y = hits > 0 ? sy / (float)hits : 0.0f;
    return p;
}

struct AxialPupil {
    Window win;
    bool usable = false;
};

AxialPupil axial_pupil(ProbeLens& L)
{
    AxialPupil a;
    Window full;
    const DiscArea d = probe_window(L, 0.0f, 0.0f, kChiefLambda, full);
    if (d.area > 0.0f) { a.win = d.fit; a.usable = true; }
    return a;
}

// Aim the chief ray of one cell at its sensor target: the clean u = v = 0 ray
// first, then the survivor mean of a 9 x 9 probe, then the tracked window of a
// deep pupil; a cell with no light keeps its seed and is DARK.
void aim_chief(ProbeLens& L, float start_z, float front_R, const AxialPupil& axial, float seed_ax, float seed_ay,
               float tx, float ty, gl_psf_cell& c)
{
    constexpr int kIter = 8;
    constexpr float kFd = 1e-4f, kTol = 1e-4f, kTolSoft = 5e-3f;
    constexpr int kAimN = 9, kFracN = 17, kMinHits = 4;
    constexpr float kDeepFd = 1e-3f, kDeepWarm = 0.10f;
    const float seed_mag = sqrtf(seed_ax * seed_ax + seed_ay * seed_ay);
    const float cap = std::max(0.02f, 0.5f * seed_mag);
    {
        auto landing = [&](float ax, float ay, float& x, float& y) {
            return chief_candidate(L, start_z, front_R, ax, ay, 0.0f, 0.0f, x, y);
        };
        float ax = seed_ax, ay = seed_ay, tx0, ty0;
        if (landing(ax, ay, tx0, ty0))
        {
            float res = 0.0f;
            newton_aim(landing, tx, ty, ax, ay, res, kIter, kFd, cap, kTol);
            landing(ax, ay, c.chief_x_mm, c.chief_y_mm);
            c.beam_ax = ax; c.beam_ay = ay;
            c.status = GL_PSF_CELL_OK;
            c.aim_residual_mm = res;
            c.pupil_fraction = pupil_probe(L, start_z, front_R, ax, ay, kFracN).frac;
            return;
        }
    }
    {
        auto landing = [&](float ax, float ay, float& x, float& y) {
            const PupilProbe p = pupil_probe(L, start_z, front_R, ax, ay, kAimN);
            if (p.hits < kMinHits) return false;
            x = p.mean_x; y = p.mean_y;
            return true;
        };
        float ax = seed_ax, ay = seed_ay, tx0, ty0;
        if (landing(ax, ay, tx0, ty0))
        {
            float res = 0.0f;
            newton_aim(landing, tx, ty, ax, ay, res, kIter, kFd, cap, kTolSoft);
            landing(ax, ay, c.chief_x_mm, c.chief_y_mm);
            c.beam_ax = ax; c.beam_ay = ay;
            c.status = GL_PSF_CELL_CHIEF_VIGNETTED;
            c.aim_residual_mm = res;
            c.pupil_fraction = pupil_probe(L, start_z, front_R, ax, ay, kFracN).frac;
            return;
        }
    }
    if (axial.usable)
    {
        Window track = axial.win;
        auto landing = [&](float ax, float ay, float& x, float& y) {
            Window w = track;
            const DiscArea d = probe_disc(L, ax, ay, kChiefLambda, &w);
            if (!(d.area > 0.0f) || !std::isfinite(d.mean_x) || !std::isfinite(d.mean_y)) return false;
            track = w;
            x = d.mean_x; y = d.mean_y;
            return true;
        };
        if (track.r < 1.0f && seed_mag > 0.0f)
        {
            const int steps = std::max(3, std::min(16, (int)std::ceil(seed_mag / kDeepWarm)));
            float a, b;
            for (int k = 1; k <= steps; ++k)
            {
                const float f = (float)k / (float)steps;
                landing(seed_ax * f, seed_ay * f, a, b);
            }
        }
        float ax = seed_ax, ay = seed_ay, tx0, ty0;
        if (landing(ax, ay, tx0, ty0))
        {
            float res = 0.0f;
            newton_aim(landing, tx, ty, ax, ay, res, kIter, kDeepFd, cap, kTolSoft);
            if (landing(ax, ay, c.chief_x_mm, c.chief_y_mm))
            {
                c.beam_ax = ax; c.beam_ay = ay;
                c.status = GL_PSF_CELL_CHIEF_VIGNETTED;
                c.aim_residual_mm = res;
                c.pupil_fraction = pupil_probe(L, start_z, front_R, ax, ay, kFracN).frac;
                return;
            }
        }
    }
    c.beam_ax = seed_ax; c.beam_ay = seed_ay;
    c.chief_x_mm = tx; c.chief_y_mm = ty;
    c.status = GL_PSF_CELL_DARK;
    c.aim_residual_mm = 1e30f;
    c.pupil_fraction = 0.0f;
}

}  // namespace
}  // namespace gl

using namespace gl;

extern "C" int gl_psf_prepass(const gl_surface* surfaces, int n, const float* sources7, int n_src, int center_mode,
                              gl_psf_cell* out)
{
    if (!surfaces || n <= 0 || (n_src > 0 && (!sources7 || !out)) || n_src < 0)
        return fail(GL_ERR_INVALID, "psf_prepass: bad arguments");
    ProbeLens L;
    int rc = open_lens(surfaces, n, L);
    if (rc) return rc;
    const float start_z = surfaces[0].z - kSpawnOffset;
    const float front_R = L.front_R;
    const AxialPupil axial = axial_pupil(L);
    const bool target = center_mode == GL_PSF_CENTER_FIXED_TARGET;
    for (int i = 0; i < n_src; ++i)
    {
        const float* s = sources7 + 7 * (size_t)i;
        gl_psf_cell c{};
        c.beam_ax = s[0]; c.beam_ay = s[1];
        c.status = GL_PSF_CELL_OK;
        if (target)
        {
            aim_chief(L, start_z, front_R, axial, s[0], s[1], s[5], s[6], c);
        }
        else
        {
            // unweighted 7 x 7 pupil-mean landing; a deep pupil the full-disc
            // probe misses is found through the tracked axial window
            const PupilProbe p = pupil_probe(L, start_z, front_R, s[0], s[1], 7);
            c.chief_x_mm = p.mean_x; c.chief_y_mm = p.mean_y;
            c.status = p.hits > 0 ? GL_PSF_CELL_OK : GL_PSF_CELL_DARK;
            c.pupil_fraction = p.frac;
            if (p.hits == 0 && axial.usable)
            {
                Window w = axial.win;
                const float mag = sqrtf(s[0] * s[0] + s[1] * s[1]);
                if (w.r < 1.0f && mag > 0.0f)
                {
                    const int steps = std::max(3, std::min(16, (int)std::ceil(mag / 0.10f)));
                    for (int k = 1; k <= steps; ++k)
                    {
                        const float f = (float)k / (float)steps;
                        probe_disc(L, s[0] * f, s[1] * f, kChiefLambda, &w);
                    }
                }
                const DiscArea d = probe_disc(L, s[0], s[1], kChiefLambda, &w);
                if (d.area > 0.0f && std::isfinite(d.mean_x) && std::isfinite(d.mean_y))
                {
                    c.chief_x_mm = d.mean_x; c.chief_y_mm = d.mean_y;
                    c.status = GL_PSF_CELL_OK;
                }
            }
        }
        if (!std::isfinite(c.aim_residual_mm)) c.aim_residual_mm = 0.0f;
        out[i] = c;
    }
    return GL_OK;
}

extern "C" int gl_calibrate_lens(const gl_surface* surfaces, int n, float lens_focal_length, float d_line_nm,
                                 gl_lens_calibration* out)
{
    if (!surfaces || n <= 0 || !out) return fail(GL_ERR_INVALID, "calibrate_lens: bad arguments");
    *out = gl_lens_calibration{};
    out->pupil_area_frac = 1.0f;
    ProbeLens L;
    int rc = open_lens(surfaces, n, L);
    if (rc) return rc;
    const float lam = d_line_nm;
    out->focal_length_x = paraxial_efl(L, lam, true);
    out->focal_length_y = paraxial_efl(L, lam, false);
    const gl_surface* stop = nullptr;
    for (int i = 0; i < n; ++i)
        if (surfaces[i].is_stop) { stop = &surfaces[i]; break; }
    if (stop && stop->aperture_shape == GL_APERTURE_POLYGON && stop->aperture_blades >= 3)
    {
        marginal_support(L, *stop, lam, &out->entrance_pupil_semi_x, &out->entrance_pupil_semi_y);
        out->pupil_area_frac = make_blade_profile(stop->aperture_blades, stop->aperture_rotation_rad,
                                                  stop->aperture_curvature, stop->aperture_twist,
                                                  stop->aperture_notch_rad,
                                                  stop->aperture_notch_angle_rad).area_frac;
    }
    else
    {
        out->entrance_pupil_semi_x = marginal_semi_along(L, lam, 1.0f, 0.0f);
        out->entrance_pupil_semi_y = marginal_semi_along(L, lam, 0.0f, 1.0f);
    }
    const float R = L.front_R;
    const float fill_x = (R > 0.0f) ? out->entrance_pupil_semi_x / R : 1.0f;
    const float fill_y = (R > 0.0f) ? out->entrance_pupil_semi_y / R : 1.0f;
    FieldSolve mh, mv, ch, cv;
    resolve_axis(L, std::min(fill_x, fill_y), lam, true, &mh, &ch);
    if (axes_symmetric(surfaces, n)) { mv = mh; cv = ch; }
    else resolve_axis(L, std::min(fill_x, fill_y), lam, false, &mv, &cv);
    out->max_half_angle_h = mh.angle;
    out->max_half_angle_v = mv.angle;
    out->sensor_half_w = mh.half_mm;
    out->sensor_half_h = mv.half_mm;
    out->image_circle_semi_w = ch.half_mm;
    out->image_circle_semi_h = cv.half_mm;
    out->field_crossed = (mh.crossed && mv.crossed) ? 1 : 0;
    // a lens that resolves to nothing falls back to the lens file's focal length
    const float min_field = (float)(0.05 * 3.14159265358979323846 / 180.0);
    auto floor_axis = [&](float* angle, float* half) {
        if (*angle >= min_field && *half > 0.0f) return;
        *angle = min_field;
        *half = (lens_focal_length > 0.0f) ? lens_focal_length * tanf(min_field) : tanf(min_field);
    };
    floor_axis(&out->max_half_angle_h, &out->sensor_half_w);
    floor_axis(&out->max_half_angle_v, &out->sensor_half_h);
    if (out->image_circle_semi_w <= 0.0f) out->image_circle_semi_w = out->sensor_half_w;
    if (out->image_circle_semi_h <= 0.0f) out->image_circle_semi_h = out->sensor_half_h;
    if (out->entrance_pupil_semi_x > 0.0f) out->f_number_x = out->focal_length_x / (2.0f * out->entrance_pupil_semi_x);
    if (out->entrance_pupil_semi_y > 0.0f) out->f_number_y = out->focal_length_y / (2.0f * out->entrance_pupil_semi_y);
    return GL_OK;
}

extern "C" int gl_solve_source_angle(const gl_surface* surfaces, int n, const gl_lens_calibration* calib, float ndc_x,
                                     float ndc_y, float eff_half_w, float eff_half_h, gl_source_solve* out)
{
    if (!calib || !out) return fail(GL_ERR_INVALID, "solve_source_angle: bad arguments");
    gl_source_solve sm{};
    sm.eff_half_w = eff_half_w;
    sm.eff_half_h = eff_half_h;
    const gl_lens_calibration& c = *calib;
    const float scale_w = (c.sensor_half_w > 0.0f) ? eff_half_w / c.sensor_half_w : 1.0f;
    const float scale_h = (c.sensor_half_h > 0.0f) ? eff_half_h / c.sensor_half_h : 1.0f;
    const float seed_ax = atanf(ndc_x * scale_w * tanf(c.max_half_angle_h));
    const float seed_ay = atanf(ndc_y * scale_h * tanf(c.max_half_angle_v));
    sm.inv_tan_w = 1.0f / (scale_w * tanf(c.max_half_angle_h));
    sm.inv_tan_h = 1.0f / (scale_h * tanf(c.max_half_angle_v));
    sm.angle_x = seed_ax;
    sm.angle_y = seed_ay;
    sm.status = GL_SOURCE_FALLBACK;
    *out = sm;
    if (!surfaces || n <= 0) return GL_OK;                  // FALLBACK: nothing to trace

    ProbeLens L;
    int rc = open_lens(surfaces, n, L);
    if (rc) return rc;
    const float target_x = ndc_x * eff_half_w, target_y = ndc_y * eff_half_h;
    const float R = L.front_R;
    const float fill_x = (R > 0.0f) ? c.entrance_pupil_semi_x / R : 1.0f;
    const float fill_y = (R > 0.0f) ? c.entrance_pupil_semi_y / R : 1.0f;
    const Window win0 = initial_window(std::min(fill_x, fill_y));
    SolveProbe P{&L, win0};
    auto landing = [&](float ax, float ay, float& x, float& y) { return P.at(ax, ay, x, y); };
    auto reset_and_walk = [&](float ax, float ay) {
        P.win = win0;
        const float mag = sqrtf(ax * ax + ay * ay);
        if (!(P.win.r < 1.0f) || !(mag > 0.0f)) return;
        const int steps = std::max(3, std::min(16, (int)std::ceil(mag / kWarmStepRad)));
        float tx, ty;
        for (int k = 1; k <= steps; ++k)
        {
            const float f = (float)k / (float)steps;
            P.at(ax * f, ay * f, tx, ty);
        }
    };
    const float seed_mag = sqrtf(seed_ax * seed_ax + seed_ay * seed_ay);
    const float accept_mm = std::max(kTolMm, kAcceptFrac * std::min(std::fabs(eff_half_w), std::fabs(eff_half_h)));
    auto commit_solved = [&](float ax, float ay, float res) -> bool {
        float land[2], J[4];
        if (!measure_jacobian(P, ax, ay, land, J)) return false;
        sm.angle_x = ax; sm.angle_y = ay;
        sm.status = GL_SOURCE_SOLVED;
        sm.residual_mm = res;
        sm.anchor_ax = ax; sm.anchor_ay = ay;
        sm.anchor_x = land[0]; sm.anchor_y = land[1];
        for (int i = 0; i < 4; ++i) sm.J[i] = J[i];
        sm.probe_evals = P.evals;
        return true;
    };
    float best_ax = seed_ax, best_ay = seed_ay, best_res = 1e30f;
    auto attempt = [&](float fax, float fay, float cap) -> bool {
        reset_and_walk(fax, fay);
        float ax = fax, ay = fay, res = 1e30f;
        newton_aim(landing, target_x, target_y, ax, ay, res, kMaxIter, kFdStep, cap, kTolMm);
        if (res < best_res) { best_res = res; best_ax = ax; best_ay = ay; }
        if (!(res < accept_mm)) return false;
        return commit_solved(ax, ay, res);
    };
    auto done = [&]() { *out = sm; return GL_OK; };
    auto give_up = [&]() { sm.probe_evals = P.evals; *out = sm; return GL_OK; };

    if (attempt(seed_ax, seed_ay, std::max(0.02f, 0.5f * seed_mag))) return done();
    if (attempt(seed_ax, seed_ay, std::max(0.005f, 0.08f * seed_mag))) return done();

    // Past the last landing the lens delivers: find the furthest convergent
    // point along the ray to the target and join an arctangent to it.
    float ax_lo = 0.0f, ay_lo = 0.0f, anchor_radius = 0.0f;
    bool have_anchor = false;
    Window anchor_win;
    const float tmag = sqrtf(target_x * target_x + target_y * target_y);
    if (tmag > 0.0f)
    {
        const float ux = target_x / tmag, uy = target_y / tmag;
        const float rc = sqrtf(ux * ux * c.image_circle_semi_w * c.image_circle_semi_w +
                               uy * uy * c.image_circle_semi_h * c.image_circle_semi_h);
        float r_lo = 0.0f, r_hi = 1.05f * rc;
        const float aseed_ax = atanf(0.98f * rc * ux * tanf(c.max_half_angle_h) /
                                     (c.sensor_half_w > 0.0f ? c.sensor_half_w : 1.0f));
        const float aseed_ay = atanf(0.98f * rc * uy * tanf(c.max_half_angle_v) /
                                     (c.sensor_half_h > 0.0f ? c.sensor_half_h : 1.0f));
        const float amag = sqrtf(aseed_ax * aseed_ax + aseed_ay * aseed_ay);
        const float acap = std::max(0.02f, 0.5f * amag);
        reset_and_walk(aseed_ax, aseed_ay);
        auto try_target = [&](float tx, float ty, float& io_ax, float& io_ay) -> bool {
            float tax = io_ax, tay = io_ay, r = 1e30f;
            newton_aim(landing, tx, ty, tax, tay, r, kMaxIter, kFdStep, acap, kTolMm);
            if (!(r < accept_mm)) return false;
            io_ax = tax; io_ay = tay;
            return true;
        };
        {
            const float g = 0.98f * rc;
            float a = ax_lo, b = ay_lo;
            if (g > 0.0f && try_target(g * ux, g * uy, a, b))
            {
                r_lo = g; ax_lo = a; ay_lo = b; have_anchor = true;
                anchor_radius = g; anchor_win = P.win;
            }
            else
            {
                r_hi = g;
            }
        }
        for (int i = 0; i < kBisectSteps && (r_hi - r_lo) > kBisectTolMm; ++i)
        {
            const float mid = 0.5f * (r_lo + r_hi);
            float a = ax_lo, b = ay_lo;
            if (try_target(mid * ux, mid * uy, a, b))
            {
                r_lo = mid; ax_lo = a; ay_lo = b; have_anchor = true;
                anchor_radius = mid; anchor_win = P.win;
            }
            else
            {
                r_hi = mid;
            }
        }
    }
    if (!have_anchor && !(seed_mag > 0.0f)) return give_up();
    if (have_anchor && attempt(ax_lo, ay_lo, std::max(0.02f, 0.5f * seed_mag))) return done();
    if (have_anchor && anchor_radius >= tmag && best_res < 1e29f)
    {
        reset_and_walk(best_ax, best_ay);
        if (commit_solved(best_ax, best_ay, best_res)) return done();
    }
    if (have_anchor) P.win = anchor_win;
    float land[2], J[4];
    if (!measure_jacobian(P, ax_lo, ay_lo, land, J)) return give_up();
    const float det = J[0] * J[3] - J[1] * J[2];
    if (!(std::fabs(det) > 1e-12f)) return give_up();
    const float dx = target_x - land[0], dy = target_y - land[1];
    const float ux = (J[3] * dx - J[1] * dy) / det;
    const float uy = (-J[2] * dx + J[0] * dy) / det;
    const float um = sqrtf(ux * ux + uy * uy);
    if (um > 1e-12f)
    {
        const float th = atanf(um);
        sm.angle_x = ax_lo + (ux / um) * th;
        sm.angle_y = ay_lo + (uy / um) * th;
    }
    else
    {
        sm.angle_x = ax_lo;
        sm.angle_y = ay_lo;
    }
    sm.status = GL_SOURCE_CONTINUED;
    sm.residual_mm = sqrtf(dx * dx + dy * dy);
    sm.anchor_ax = ax_lo; sm.anchor_ay = ay_lo;
    sm.anchor_x = land[0]; sm.anchor_y = land[1];
    for (int i = 0; i < 4; ++i) sm.J[i] = J[i];
    sm.probe_evals = P.evals;
    return done();
}

extern "C" int gl_source_map_screen(const gl_source_solve* base, float angle_x, float angle_y, float* out_sx,
                                    float* out_sy)
{
    if (!base || !out_sx || !out_sy) return fail(GL_ERR_INVALID, "source_map_screen: bad arguments");
    if (base->status == GL_SOURCE_FALLBACK)
    {
        *out_sx = 0.5f + 0.5f * tanf(angle_x) * base->inv_tan_w;
        *out_sy = 0.5f + 0.5f * tanf(angle_y) * base->inv_tan_h;
        return GL_OK;
    }
    const float dax = angle_x - base->anchor_ax, day = angle_y - base->anchor_ay;
    const float d = sqrtf(dax * dax + day * day);
    float ux = dax, uy = day;
    if (d > 1e-12f)
    {
        const float t = tanf(std::min(d, kMaxExtendRad));
        ux = (dax / d) * t;
        uy = (day / d) * t;
    }
    const float x = base->anchor_x + base->J[0] * ux + base->J[1] * uy;
    const float y = base->anchor_y + base->J[2] * ux + base->J[3] * uy;
    *out_sx = (base->eff_half_w > 0.0f) ? 0.5f + 0.5f * x / base->eff_half_w : 0.5f;
    *out_sy = (base->eff_half_h > 0.0f) ? 0.5f + 0.5f * y / base->eff_half_h : 0.5f;
    return GL_OK;
}
