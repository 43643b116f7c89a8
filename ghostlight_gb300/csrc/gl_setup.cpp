// gl_setup.cpp — the per-lens first-order setup of the flare path: the lens
// calibration, the source-position solve and its forward map, and the PSF
// grid's tile anchors, in float32 or FP64 (gl_setup_trace.h).
//
// What is computed is the reference's (JaydenB/ghostlight): calibrate_lens
// (lens_calibration.cpp:24-443) measures the focal length from a 1 degree
// chief ray, the entrance pupil by bisecting the clear radius, and the
// covered field as the angle where the surviving area of the spawn disc falls
// to 90% (5% for the image circle) of its axial value (spawn_probe.cpp:
// 28-211); solve_source_angle (source_map.cpp:182-483) aims the disc's
// survivor-mean landing at the target with a finite-difference Newton
// (newton_aim.h:20-63), continuing past the last landing by the local
// Jacobian; the PSF pre-pass (PSFRenderer.cpp:28-243) anchors each tile on
// the pupil-mean landing or an aimed chief ray.  The grids, thresholds,
// iteration counts and step rules are the reference's, because its numbers
// size every render (sensor extents, field angles): in float32 this file
// reproduces them bit for bit (-ffp-contract=off host code, the same
// operation order).
//
// How it is organised here: a probe is gathered (every launch of the grid),
// traced as one batch and reduced in grid order; the window that follows the
// beam is a small state machine; the two root finders (Illinois regula falsi
// on the area fraction, 2 x 2 Newton on the landing) are generic over a
// callable; every routine is a template on the scalar type.
#include "gl_setup_trace.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace gl {
namespace setup {
namespace {

constexpr double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------------------
// Spawn-disc coverage
// ---------------------------------------------------------------------------
template <class T> struct Frame {        // square window over the unit spawn disc
    T cu = T(0), cv = T(0), r = T(1);
};

template <class T> struct Coverage {     // surviving area and its mean landing
    T area = T(0), mx = T(0), my = T(0);
    bool rim = false;                    // survivors on the window's border
    Frame<T> fit;                        // a window fitted around the survivors
};

struct Sampling { int grid, edge_ss; };
constexpr Sampling kDiscSampling{17, 2};
constexpr float kDeepStopFill = 0.45f;   // below this pupil fill the probe starts in a window
constexpr float kWindowDilation = 5.0f;

template <class T> Frame<T> seed_frame(T pupil_fill)
{
    Frame<T> f;
    if (pupil_fill > T(0) && pupil_fill < T(kDeepStopFill)) f.r = std::min(T(1), pupil_fill * T(kWindowDilation));
    return f;
}

// One launch of the probe: pupil point (u, v) of the beam (ah, av).
template <class T> struct Shot { T u, v; };

template <class T>
void shoot(const SetupLens<T>& L, T ah, T av, const std::vector<Shot<T>>& shots, std::vector<Hit<T>>& out)
{
    const T bx = Math<T>::tan(ah), by = Math<T>::tan(av);
    const T sdx = -T(kSpawnOffset) * bx, sdy = -T(kSpawnOffset) * by;   // the disc follows the beam
    const T R = L.front_R();
    out.resize(shots.size());
    for (size_t k = 0; k < shots.size(); ++k)
    {
        const Shot<T>& s = shots[k];
        Hit<T> h{T(0), T(0), false};
        if (L.pupil_has(s.u, s.v))
        {
            h = L.trace(s.u * R + sdx, s.v * R + sdy, ah, av);
            h.ok = h.ok && std::isfinite(h.x) && std::isfinite(h.y);
        }
        out[k] = h;
    }
}

// Coverage-weighted surviving area of the window: cell centres first; every
// cell that survives on the border, or disagrees with a 4-neighbour about
// survival, is replaced by its edge_ss^2 sub-samples.
template <class T>
Coverage<T> cover(const SetupLens<T>& L, T ah, T av, const Frame<T>& win, Sampling smp)
{
    const int n = smp.grid, ss = smp.edge_ss;
    const T step = T(2) * win.r / T(n);
    const T u0 = win.cu - win.r, v0 = win.cv - win.r;

    std::vector<Shot<T>> shots((size_t)n * n);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i)
            shots[(size_t)j * n + i] = Shot<T>{u0 + (T(i) + T(0.5)) * step, v0 + (T(j) + T(0.5)) * step};
    std::vector<Hit<T>> centre;
    shoot(L, ah, av, shots, centre);

    auto alive = [&](int i, int j) { return centre[(size_t)j * n + i].ok; };
    std::vector<char> refine((size_t)n * n, 0);
    bool rim_hit = false;
    std::vector<Shot<T>> sub_shots;
    const T sub = step / T(ss);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i)
        {
            const bool here = alive(i, j);
            const bool border = (i == 0 || i == n - 1 || j == 0 || j == n - 1);
            bool edge = here && border;
            rim_hit = rim_hit || edge;
            if (!edge && i + 1 < n) edge = alive(i + 1, j) != here;
            if (!edge && i > 0) edge = alive(i - 1, j) != here;
            if (!edge && j + 1 < n) edge = alive(i, j + 1) != here;
            if (!edge && j > 0) edge = alive(i, j - 1) != here;
            if (!edge) continue;
            refine[(size_t)j * n + i] = 1;
            const T cu = u0 + T(i) * step, cv = v0 + T(j) * step;
            for (int sj = 0; sj < ss; ++sj)
                for (int si = 0; si < ss; ++si)
                    sub_shots.push_back(Shot<T>{cu + (T(si) + T(0.5)) * sub, cv + (T(sj) + T(0.5)) * sub});
        }
    std::vector<Hit<T>> subs;
    shoot(L, ah, av, sub_shots, subs);

    // reduce in grid order (the summation order fixes the float result)
    Coverage<T> c;
    c.rim = rim_hit;
    const T cell = step * step, w_sub = T(1) / T(ss * ss);
    T lo_u = T(1e30), hi_u = T(-1e30), lo_v = T(1e30), hi_v = T(-1e30);
    auto add = [&](const Shot<T>& s, const Hit<T>& h, T w) {
        c.area += w * cell;
        c.mx += w * cell * h.x;
        c.my += w * cell * h.y;
        lo_u = std::min(lo_u, s.u); hi_u = std::max(hi_u, s.u);
        lo_v = std::min(lo_v, s.v); hi_v = std::max(hi_v, s.v);
    };
    size_t next_sub = 0;
    for (size_t k = 0; k < centre.size(); ++k)
    {
        if (!refine[k])
        {
            if (centre[k].ok) add(shots[k], centre[k], T(1));
            continue;
        }
        for (int q = 0; q < ss * ss; ++q, ++next_sub)
            if (subs[next_sub].ok) add(sub_shots[next_sub], subs[next_sub], w_sub);
    }
    if (c.area > T(0))
    {
        c.mx /= c.area;
        c.my /= c.area;
        c.fit.cu = T(0.5) * (lo_u + hi_u);
        c.fit.cv = T(0.5) * (lo_v + hi_v);
        c.fit.r = std::max(std::max(hi_u - c.fit.cu, hi_v - c.fit.cv), step) + step;
    }
    return c;
}

// The window that follows the beam across the disc: it settles on a probe
// whose survivors stay off its border; otherwise it recentres on them (three
// times at most) and then widens by 2.5x, to the whole disc at most, within
// six probes.  `track` carries the window from one field angle to the next.
template <class T>
Coverage<T> follow(const SetupLens<T>& L, T ah, T av, Frame<T>& track, Sampling smp = kDiscSampling)
{
    Frame<T> win = track;
    if (win.r >= T(1)) win = Frame<T>{};
    Coverage<T> best;
    for (int probe = 0; probe < 6; ++probe)
    {
        const Coverage<T> c = cover(L, ah, av, win, smp);
        const bool lit = c.area > T(0);
        if (lit) best = c;
        if (lit && !c.rim)
        {
            track = Frame<T>{c.fit.cu, c.fit.cv, win.r};
            return c;
        }
        if (win.r >= T(1)) break;
        if (lit && probe < 3)
        {
            win.cu = c.fit.cu;
            win.cv = c.fit.cv;
        }
        else
        {
            win.r = std::min(T(1), win.r * T(2.5));
            if (win.r >= T(1)) { win.cu = T(0); win.cv = T(0); }
        }
    }
    track = win;
    return best;
}

// ---------------------------------------------------------------------------
// Root finders
// ---------------------------------------------------------------------------
// A bracket [lo, hi] of a decreasing function crossing zero, refined by the
// Illinois variant of regula falsi: the end that stays put has its value
// halved.  `v_lo` / `v_hi` keep the measured values at the ends (the
// halved ones no longer interpolate the root).
template <class T> struct Illinois {
    T lo, hi, f_lo, f_hi, v_lo, v_hi;

    Illinois(T a, T b, T fa, T fb) : lo(a), hi(b), f_lo(fa), f_hi(fb), v_lo(fa), v_hi(fb) {}
    T width() const { return hi - lo; }
    T trial() const
    {
        const T den = f_lo - f_hi;
        T x = (Math<T>::abs(den) < T(1e-12)) ? T(0.5) * (lo + hi) : lo + (hi - lo) * f_lo / den;
        const T keep_in = T(0.01) * (hi - lo);
        return std::min(std::max(x, lo + keep_in), hi - keep_in);
    }
    void take(T x, T fx)
    {
        if (fx >= T(0)) { lo = x; f_lo = fx; v_lo = fx; f_hi *= T(0.5); }
        else { hi = x; f_hi = fx; v_hi = fx; f_lo *= T(0.5); }
    }
    // the crossing interpolated from the measured end values
    T root() const
    {
        const T span = v_lo - v_hi;
        const T x = (Math<T>::abs(span) < T(1e-12)) ? T(0.5) * (lo + hi) : lo + (hi - lo) * v_lo / span;
        return std::min(std::max(x, lo), hi);
    }
};

// Two-dimensional aim: finite-difference Newton steps (each clamped to
// +-cap) that drive landing(ax, ay) onto (tx, ty), keeping the best iterate.
// `landing(ax, ay, x, y)` returns false where nothing lands.  The call
// sequence (and so the state of a stateful landing function) is fixed: one
// evaluation at the start, two per Jacobian, one per step, one at the end.
template <class T, class Landing>
bool aim2d(Landing&& landing, T tx, T ty, T& ax, T& ay, T& residual, int max_steps, T fd, T cap, T tol)
{
    T keep_ax = ax, keep_ay = ay, keep = T(1e30);
    auto score = [&](T x, T y) {
        const T dx = x - tx, dy = y - ty;
        const T r = Math<T>::sqrt(dx * dx + dy * dy);
        if (r < keep) { keep = r; keep_ax = ax; keep_ay = ay; }
        return r;
    };
    T cx, cy;
    if (!landing(ax, ay, cx, cy)) { residual = T(1e30); return false; }
    for (int k = 0; k < max_steps; ++k)
    {
        const T ex = cx - tx, ey = cy - ty;
        if (score(cx, cy) < tol) break;
        T x1, y1, x2, y2;
        if (!landing(ax + fd, ay, x1, y1)) break;
        if (!landing(ax, ay + fd, x2, y2)) break;
        const T a = (x1 - cx) / fd, c = (y1 - cy) / fd;        // d(x, y) / d ax
        const T b = (x2 - cx) / fd, d = (y2 - cy) / fd;        // d(x, y) / d ay
        const T det = a * d - b * c;
        if (Math<T>::abs(det) < T(1e-12)) break;
        const T sx = std::max(-cap, std::min(cap, (-ex * d + ey * b) / det));
        const T sy = std::max(-cap, std::min(cap, (ex * c - ey * a) / det));
        ax += sx;
        ay += sy;
        if (!landing(ax, ay, cx, cy)) break;
    }
    if (landing(ax, ay, cx, cy)) score(cx, cy);
    ax = keep_ax;
    ay = keep_ay;
    residual = keep;
    return keep < tol;
}

// ---------------------------------------------------------------------------
// Calibration
// ---------------------------------------------------------------------------
// First-order focal length on one axis: image height of a 1 degree chief ray
// over tan(1 degree).
template <class T> T focal_length(SetupLens<T>& L, T lam, bool x_axis)
{
    const T one = T(1.0 * kPi / 180.0);
    L.set_lambda(lam);
    const Hit<T> h = x_axis ? L.trace(T(0), T(0), one, T(0)) : L.trace(T(0), T(0), T(0), one);
    if (!h.ok) return T(0);
    const T y = x_axis ? h.x : h.y;
    if (!std::isfinite(y)) return T(0);
    return Math<T>::abs(y) / Math<T>::tan(one);
}

// Clear radius of the axial beam along (ux, uy) on the front vertex plane:
// the largest launch height that still reaches the sensor, by 40 halvings.
template <class T> T clear_radius(SetupLens<T>& L, T lam, T ux, T uy)
{
    const T R = L.front_R();
    if (R <= T(0)) return T(0);
    L.set_lambda(lam);
    auto passes = [&](T h) { return L.trace(h * ux, h * uy, T(0), T(0)).ok; };
    if (!passes(T(0))) return T(0);
    if (passes(R)) return R;
    T in = T(0), out = R;
    for (int k = 0; k < 40; ++k)
    {
        const T mid = T(0.5) * (in + out);
        (passes(mid) ? in : out) = mid;
    }
    return in;
}

// Per-axis support of a bladed entrance pupil: the clear radius over eight
// azimuths per blade (tips, waists and between) and the two axes.
template <class T> void pupil_support(SetupLens<T>& L, const gl_surface& stop, T lam, T& sx, T& sy)
{
    const int n = stop.aperture_blades * 8;
    sx = T(0);
    sy = T(0);
    auto along = [&](T th) {
        const T c = Math<T>::cos(th), s = Math<T>::sin(th);
        const T h = clear_radius(L, lam, c, s);
        sx = std::max(sx, h * Math<T>::abs(c));
        sy = std::max(sy, h * Math<T>::abs(s));
    };
    for (int i = 0; i < n; ++i) along(T(stop.aperture_rotation_rad) + T(2.0 * kPi) * T(i) / T(n));
    along(T(0));
    along(T(kPi / 2.0));
}

// Where a threshold of the surviving-area fraction is crossed, and the
// survivors' mean landing there.
template <class T> struct Crossing {
    T angle = T(0), half_mm = T(0);
    bool crossed = false;
};

constexpr int kSteps = 8;
const float kFieldSteps[kSteps] = {0.0f, 4.0f, 8.0f, 14.0f, 22.0f, 32.0f, 45.0f, 60.0f};   // degrees
struct Threshold { float level, tol_deg; int max_refine; };
constexpr Threshold kCoveredField{0.90f, 0.15f, 7};
constexpr Threshold kImageCircle{0.05f, 1.0f, 2};

// The walk out along one axis of the field that both thresholds are found on.
template <class T> class FieldWalk {
public:
    FieldWalk(SetupLens<T>& L, T pupil_fill, T lam, bool x_axis)
        : L_(L), lam_(lam), x_axis_(x_axis), track_(seed_frame(pupil_fill)) {}

    // surviving-area fraction at a field angle; the axial reference is
    // re-measured whenever the tracked window has changed size
    Coverage<T> probe(T angle)
    {
        L_.set_lambda(lam_);
        const Coverage<T> c = follow(L_, x_axis_ ? angle : T(0), x_axis_ ? T(0) : angle, track_);
        if (track_.r != axial_size_)
        {
            Frame<T> f;
            f.r = track_.r;
            axial_ = cover(L_, T(0), T(0), f, kDiscSampling);
            axial_size_ = track_.r;
        }
        return c;
    }
    T fraction(const Coverage<T>& c) const { return c.area / axial_.area; }

    void run(Crossing<T>& field, Crossing<T>& circle)
    {
        field = Crossing<T>{};
        circle = Crossing<T>{};
        probe(T(0));
        if (axial_.area <= T(0)) return;
        const T DEG = T(kPi / 180.0);
        // one walk up the ladder brackets both crossings (the image circle
        // lies beyond the covered field); each bracket keeps the window the
        // beam had at its lower end
        struct Bracket { int at = -1; T f[2]; Frame<T> start; };
        Bracket bf, bc;
        T f_prev = T(1);
        for (int i = 1; i < kSteps; ++i)
        {
            const Frame<T> before = track_;
            const T f = fraction(probe(T(kFieldSteps[i]) * DEG));
            if (bf.at < 0 && f < T(kCoveredField.level)) bf = Bracket{i - 1, {f_prev, f}, before};
            if (bc.at < 0 && f < T(kImageCircle.level))
            {
                bc = Bracket{i - 1, {f_prev, f}, before};
                break;
            }
            f_prev = f;
        }
        field = settle(bf.at, kCoveredField, bf.f, bf.start);
        circle = settle(bc.at, kImageCircle, bc.f, bc.start);
        // the lower threshold cannot lie inside the covered field
        if (circle.angle < field.angle) circle = field;
        if (circle.half_mm < field.half_mm) circle.half_mm = field.half_mm;
    }

private:
    T landing_of(const Coverage<T>& c) const { return Math<T>::abs(x_axis_ ? c.mx : c.my); }

    // refine one bracket; every probe restarts from the bracket's window
    // centre (keeping the grown size)
    Crossing<T> settle(int at, const Threshold& th, const T f_ends[2], const Frame<T>& start)
    {
        const T DEG = T(kPi / 180.0);
        auto probe_from_start = [&](T angle) {
            track_.cu = start.cu;
            track_.cv = start.cv;
            return probe(angle);
        };
        Crossing<T> r;
        if (at < 0)
        {
            // never crossed inside the ladder: the ceiling, reported as such
            const Coverage<T> c = probe_from_start(T(kFieldSteps[kSteps - 1]) * DEG);
            r.angle = T(kFieldSteps[kSteps - 1]) * DEG;
            r.half_mm = landing_of(c);
            return r;
        }
        const T level = T(th.level);
        Illinois<T> b(T(kFieldSteps[at]) * DEG, T(kFieldSteps[at + 1]) * DEG, f_ends[0] - level, f_ends[1] - level);
        const T tol = T(th.tol_deg) * DEG;
        for (int k = 0; k < th.max_refine && b.width() > tol; ++k)
        {
            const T x = b.trial();
            b.take(x, fraction(probe_from_start(x)) - level);
        }
        T root = b.root();
        Coverage<T> c = probe_from_start(root);
        if (c.area <= T(0))
        {
            // interpolation overshot past the last light: the low end has survivors
            root = b.lo;
            c = probe_from_start(root);
        }
        r.angle = root;
        r.half_mm = landing_of(c);
        r.crossed = true;
        return r;
    }

    SetupLens<T>& L_;
    T lam_;
    bool x_axis_;
    Frame<T> track_;
    Coverage<T> axial_;
    T axial_size_ = T(-1);
};

// Rotational symmetry: one axis's answer serves both.
bool symmetric(const gl_surface* s, int n)
{
    for (int i = 0; i < n; ++i)
    {
        const gl_surface& g = s[i];
        if (g.form == GL_FORM_CYLINDRICAL || g.aperture_aspect != 1.0f) return false;
        if (g.decenter_x != 0.0f || g.decenter_y != 0.0f) return false;
        for (int k = 0; k < 9; ++k)
            if (g.rot[k] != ((k % 4 == 0) ? 1.0f : 0.0f)) return false;
        if (g.aperture_shape == GL_APERTURE_POLYGON)
        {
            if (g.aperture_blades % 4 != 0 || g.aperture_rotation_rad != 0.0f) return false;
        }
        else if (g.aperture_shape != GL_APERTURE_CIRCLE)
        {
            return false;
        }
    }
    return true;
}

template <class T>
int calibrate(const gl_surface* s, int n, float focal_length_mm, float d_line_nm, gl_lens_calibration* out)
{
    SetupLens<T> L;
    const int rc = L.open(s, n);
    if (rc) return rc;
    const T lam = T(d_line_nm);
    T efl_x = focal_length(L, lam, true), efl_y = focal_length(L, lam, false);
    T ep_x, ep_y;
    float area_frac = 1.0f;
    const gl_surface* stop = nullptr;
    for (int i = 0; i < n && !stop; ++i)
        if (s[i].is_stop) stop = &s[i];
    if (stop && stop->aperture_shape == GL_APERTURE_POLYGON && stop->aperture_blades >= 3)
    {
        pupil_support(L, *stop, lam, ep_x, ep_y);
        area_frac = make_blade_profile(stop->aperture_blades, stop->aperture_rotation_rad, stop->aperture_curvature,
                                       stop->aperture_twist, stop->aperture_notch_rad,
                                       stop->aperture_notch_angle_rad).area_frac;
    }
    else
    {
        ep_x = clear_radius(L, lam, T(1), T(0));
        ep_y = clear_radius(L, lam, T(0), T(1));
    }
    const T R = L.front_R();
    const T fill = std::min(R > T(0) ? ep_x / R : T(1), R > T(0) ? ep_y / R : T(1));
    Crossing<T> fh, ch, fv, cv;
    FieldWalk<T>(L, fill, lam, true).run(fh, ch);
    if (symmetric(s, n)) { fv = fh; cv = ch; }
    else FieldWalk<T>(L, fill, lam, false).run(fv, cv);

    gl_lens_calibration c{};
    c.focal_length_x = (float)efl_x;
    c.focal_length_y = (float)efl_y;
    c.entrance_pupil_semi_x = (float)ep_x;
    c.entrance_pupil_semi_y = (float)ep_y;
    c.pupil_area_frac = area_frac;
    c.field_crossed = (fh.crossed && fv.crossed) ? 1 : 0;
    // a lens that resolves to nothing falls back to the lens file's focal length
    const T min_field = T(0.05 * kPi / 180.0);
    auto field_or_floor = [&](const Crossing<T>& f, float& angle, float& half) {
        T a = f.angle, h = f.half_mm;
        if (!(a >= min_field && h > T(0)))
        {
            a = min_field;
            h = focal_length_mm > 0.0f ? T(focal_length_mm) * Math<T>::tan(min_field) : Math<T>::tan(min_field);
        }
        angle = (float)a;
        half = (float)h;
    };
    field_or_floor(fh, c.max_half_angle_h, c.sensor_half_w);
    field_or_floor(fv, c.max_half_angle_v, c.sensor_half_h);
    c.image_circle_semi_w = ch.half_mm > T(0) ? (float)ch.half_mm : c.sensor_half_w;
    c.image_circle_semi_h = cv.half_mm > T(0) ? (float)cv.half_mm : c.sensor_half_h;
    if (ep_x > T(0)) c.f_number_x = (float)(efl_x / (T(2) * ep_x));
    if (ep_y > T(0)) c.f_number_y = (float)(efl_y / (T(2) * ep_y));
    *out = c;
    return GL_OK;
}

// ---------------------------------------------------------------------------
// Source-position solve
// ---------------------------------------------------------------------------
struct SolveRule {
    float lambda_nm = 587.56f;
    int max_steps = 8;
    float fd_rad = 5e-3f;           // finite-difference step of the Jacobian
    float tol_mm = 1e-3f;
    float accept_frac = 0.01f;      // acceptable residual, fraction of the smaller frame half
    int anchor_halvings = 6;
    float anchor_tol_mm = 0.02f;
    float max_extend_rad = 1.55f;
    float walk_step_rad = 0.10f;
};
constexpr SolveRule kSolve{};

// The landing of a beam: the survivor-mean landing of the spawn disc, with
// the probe window carried from one evaluation to the next.
template <class T> struct Beam {
    SetupLens<T>& L;
    Frame<T> start, win;
    int evals = 0;

    bool land(T ax, T ay, T& x, T& y)
    {
        ++evals;
        Frame<T> w = win;
        L.set_lambda(T(kSolve.lambda_nm));
        const Coverage<T> c = follow(L, ax, ay, w);
        if (!(c.area > T(0)) || !std::isfinite(c.mx) || !std::isfinite(c.my)) return false;
        win = w;
        x = c.mx;
        y = c.my;
        return true;
    }
    // restart the window and walk it out to (ax, ay) in steps of 0.1 rad,
    // so a deep pupil's window finds the beam
    void walk_to(T ax, T ay)
    {
        win = start;
        const T mag = Math<T>::sqrt(ax * ax + ay * ay);
        if (!(win.r < T(1)) || !(mag > T(0))) return;
        const int steps = std::max(3, std::min(16, (int)std::ceil(mag / T(kSolve.walk_step_rad))));
        T x, y;
        for (int k = 1; k <= steps; ++k)
        {
            const T f = T(k) / T(steps);
            land(ax * f, ay * f, x, y);
        }
    }
    // landing and its Jacobian (one-sided differences, backward where the
    // forward point does not land); J = [dx/dax, dx/day, dy/dax, dy/day]
    bool linearise(T ax, T ay, T* at, T* J)
    {
        T cx, cy;
        if (!land(ax, ay, cx, cy)) return false;
        const T h = T(kSolve.fd_rad);
        auto column = [&](T dax, T day, T& dx, T& dy) {
            T px, py;
            if (land(ax + dax, ay + day, px, py)) { dx = (px - cx) / h; dy = (py - cy) / h; return true; }
            if (land(ax - dax, ay - day, px, py)) { dx = (cx - px) / h; dy = (cy - py) / h; return true; }
            return false;
        };
        T xa, ya, xb, yb;
        if (!column(h, T(0), xa, ya) || !column(T(0), h, xb, yb)) return false;
        at[0] = cx; at[1] = cy;
        J[0] = xa; J[1] = xb; J[2] = ya; J[3] = yb;
        return true;
    }
};

template <class T>
int solve(const gl_surface* s, int n, const gl_lens_calibration& c, float ndc_x, float ndc_y, float half_w,
          float half_h, gl_source_solve* out)
{
    gl_source_solve r{};
    r.eff_half_w = half_w;
    r.eff_half_h = half_h;
    const float kw = (c.sensor_half_w > 0.0f) ? half_w / c.sensor_half_w : 1.0f;
    const float kh = (c.sensor_half_h > 0.0f) ? half_h / c.sensor_half_h : 1.0f;
    const T tan_h = Math<T>::tan(T(c.max_half_angle_h)), tan_v = Math<T>::tan(T(c.max_half_angle_v));
    const T seed_ax = Math<T>::atan(T(ndc_x) * T(kw) * tan_h);
    const T seed_ay = Math<T>::atan(T(ndc_y) * T(kh) * tan_v);
    r.inv_tan_w = (float)(T(1) / (T(kw) * tan_h));
    r.inv_tan_h = (float)(T(1) / (T(kh) * tan_v));
    r.angle_x = (float)seed_ax;
    r.angle_y = (float)seed_ay;
    r.status = GL_SOURCE_FALLBACK;
    *out = r;
    if (!s || n <= 0) return GL_OK;              // nothing to trace: the paraxial map

    SetupLens<T> L;
    const int rc = L.open(s, n);
    if (rc) return rc;
    const T tx = T(ndc_x) * T(half_w), ty = T(ndc_y) * T(half_h);
    const T R = L.front_R();
    const T fill = std::min(R > T(0) ? T(c.entrance_pupil_semi_x) / R : T(1),
                            R > T(0) ? T(c.entrance_pupil_semi_y) / R : T(1));
    Beam<T> beam{L, seed_frame(fill), seed_frame(fill)};
    auto landing = [&](T ax, T ay, T& x, T& y) { return beam.land(ax, ay, x, y); };
    const T accept = std::max(T(kSolve.tol_mm),
                              T(kSolve.accept_frac) * std::min(Math<T>::abs(T(half_w)), Math<T>::abs(T(half_h))));
    const T seed_mag = Math<T>::sqrt(seed_ax * seed_ax + seed_ay * seed_ay);

    auto publish = [&](T ax, T ay, T res, T from_ax, T from_ay, const T* at, const T* J, int status) {
        r.angle_x = (float)ax; r.angle_y = (float)ay;
        r.status = status;
        r.residual_mm = (float)res;
        r.anchor_ax = (float)from_ax; r.anchor_ay = (float)from_ay;
        r.anchor_x = (float)at[0]; r.anchor_y = (float)at[1];
        for (int k = 0; k < 4; ++k) r.J[k] = (float)J[k];
        r.probe_evals = beam.evals;
        *out = r;
    };
    auto publish_solved = [&](T ax, T ay, T res) {
        T at[2], J[4];
        if (!beam.linearise(ax, ay, at, J)) return false;
        publish(ax, ay, res, ax, ay, at, J, GL_SOURCE_SOLVED);
        return true;
    };
    T best_ax = seed_ax, best_ay = seed_ay, best_res = T(1e30);
    auto newton_from = [&](T ax, T ay, T cap) {
        beam.walk_to(ax, ay);
        T res = T(1e30);
        aim2d<T>(landing, tx, ty, ax, ay, res, kSolve.max_steps, T(kSolve.fd_rad), cap, T(kSolve.tol_mm));
        if (res < best_res) { best_res = res; best_ax = ax; best_ay = ay; }
        return res < accept && publish_solved(ax, ay, res);
    };
    auto unsolved = [&]() { r.probe_evals = beam.evals; *out = r; return GL_OK; };

    // 1. Newton from the paraxial seed, with a wide and then a tight step cap
    if (newton_from(seed_ax, seed_ay, std::max(T(0.02), T(0.5) * seed_mag))) return GL_OK;
    if (newton_from(seed_ax, seed_ay, std::max(T(0.005), T(0.08) * seed_mag))) return GL_OK;

    // 2. The target may lie past the last landing the lens delivers: find the
    // outermost convergent landing on the line from the centre to the target
    // by halving the radius between 0 and 1.05 image-circle radii
    T anchor_ax = T(0), anchor_ay = T(0), anchor_r = T(0);
    bool anchored = false;
    Frame<T> anchor_win;
    const T tmag = Math<T>::sqrt(tx * tx + ty * ty);
    if (tmag > T(0))
    {
        const T ux = tx / tmag, uy = ty / tmag;
        const T rc_ = Math<T>::sqrt(ux * ux * T(c.image_circle_semi_w) * T(c.image_circle_semi_w) +
                                   uy * uy * T(c.image_circle_semi_h) * T(c.image_circle_semi_h));
        const T g = T(0.98) * rc_;
        const T wx = Math<T>::atan(g * ux * tan_h / (c.sensor_half_w > 0.0f ? T(c.sensor_half_w) : T(1)));
        const T wy = Math<T>::atan(g * uy * tan_v / (c.sensor_half_h > 0.0f ? T(c.sensor_half_h) : T(1)));
        const T cap = std::max(T(0.02), T(0.5) * Math<T>::sqrt(wx * wx + wy * wy));
        beam.walk_to(wx, wy);
        auto reaches = [&](T radius) {
            T ax = anchor_ax, ay = anchor_ay, res = T(1e30);
            aim2d<T>(landing, radius * ux, radius * uy, ax, ay, res, kSolve.max_steps, T(kSolve.fd_rad), cap,
                     T(kSolve.tol_mm));
            if (!(res < accept)) return false;
            anchor_ax = ax; anchor_ay = ay; anchor_r = radius;
            anchored = true;
            anchor_win = beam.win;
            return true;
        };
        T in = T(0), out_r = T(1.05) * rc_;
        if (!(g > T(0) && reaches(g))) out_r = g;
        else in = g;
        for (int k = 0; k < kSolve.anchor_halvings && (out_r - in) > T(kSolve.anchor_tol_mm); ++k)
        {
            const T mid = T(0.5) * (in + out_r);
            (reaches(mid) ? in : out_r) = mid;
        }
    }
    if (!anchored && !(seed_mag > T(0))) return unsolved();
    if (anchored && newton_from(anchor_ax, anchor_ay, std::max(T(0.02), T(0.5) * seed_mag))) return GL_OK;
    if (anchored && anchor_r >= tmag && best_res < T(1e29))
    {
        beam.walk_to(best_ax, best_ay);
        if (publish_solved(best_ax, best_ay, best_res)) return GL_OK;
    }
    // 3. continue from the anchor by the local Jacobian, bending the angle
    // offset through an arctangent so it never runs away
    if (anchored) beam.win = anchor_win;
    T at[2], J[4];
    if (!beam.linearise(anchor_ax, anchor_ay, at, J)) return unsolved();
    const T det = J[0] * J[3] - J[1] * J[2];
    if (!(Math<T>::abs(det) > T(1e-12))) return unsolved();
    const T dx = tx - at[0], dy = ty - at[1];
    const T px = (J[3] * dx - J[1] * dy) / det, py = (-J[2] * dx + J[0] * dy) / det;
    const T pm = Math<T>::sqrt(px * px + py * py);
    T ax = anchor_ax, ay = anchor_ay;
    if (pm > T(1e-12))
    {
        const T th = Math<T>::atan(pm);
        ax = anchor_ax + (px / pm) * th;
        ay = anchor_ay + (py / pm) * th;
    }
    publish(ax, ay, Math<T>::sqrt(dx * dx + dy * dy), anchor_ax, anchor_ay, at, J, GL_SOURCE_CONTINUED);
    return GL_OK;
}

// ---------------------------------------------------------------------------
// PSF tile anchors
// ---------------------------------------------------------------------------
constexpr float kChiefLambda = 587.56f;

// N x N probe of the unit pupil disc at the d line: transmitted fraction and
// the survivors' mean landing.
template <class T> struct PupilCloud { int hits = 0; T frac = T(0), mx = T(0), my = T(0); };

template <class T> PupilCloud<T> pupil_cloud(SetupLens<T>& L, T ax, T ay, int N)
{
    std::vector<Shot<T>> shots;
    for (int iy = 0; iy < N; ++iy)
    {
        const T v = T(-1) + (T(iy) + T(0.5)) * (T(2) / T(N));
        for (int ix = 0; ix < N; ++ix)
        {
            const T u = T(-1) + (T(ix) + T(0.5)) * (T(2) / T(N));
            if (u * u + v * v <= T(1)) shots.push_back(Shot<T>{u, v});
        }
    }
    L.set_lambda(T(kChiefLambda));
    const T bx = Math<T>::tan(ax), by = Math<T>::tan(ay);
    const T sdx = -T(kSpawnOffset) * bx, sdy = -T(kSpawnOffset) * by;
    const T R = L.front_R();
    PupilCloud<T> p;
    T sx = T(0), sy = T(0);
    for (const Shot<T>& s : shots)
    {
        const Hit<T> h = L.trace(s.u * R + sdx, s.v * R + sdy, ax, ay);
        if (!h.ok || !std::isfinite(h.x) || !std::isfinite(h.y)) continue;
        sx += h.x;
        sy += h.y;
        ++p.hits;
    }
    p.frac = shots.empty() ? T(0) : T(p.hits) / T(shots.size());
    p.mx = p.hits > 0 ? sx / T(p.hits) : T(0);
    p.my = p.hits > 0 ? sy / T(p.hits) : T(0);
    return p;
}

// The chief ray of a cell aimed at its target: the u = v = 0 ray first, then
// the mean of a 9 x 9 pupil cloud, then (deep pupils) the tracked disc probe;
// a cell with no light keeps its seed and is reported dark.
template <class T>
void aim_tile(SetupLens<T>& L, bool axial_ok, const Frame<T>& axial_win, T sx, T sy, T tx, T ty, gl_psf_cell& c)
{
    const int kSteps_ = 8, kCloudN = 9, kFracN = 17, kMinHits = 4;
    const T kFd = T(1e-4f), kTol = T(1e-4f), kTolSoft = T(5e-3f), kDeepFd = T(1e-3f);
    const T seed_mag = Math<T>::sqrt(sx * sx + sy * sy);
    const T cap = std::max(T(0.02f), T(0.5f) * seed_mag);
    // aim from the seed; the aimed landing is the tile anchor (where it
    // fails to land again, the deep search gives up on this cell and the
    // other two keep the anchor they had)
    auto try_aim = [&](auto&& landing, T fd, T tol, int status, bool must_land) {
        T ax = sx, ay = sy, x, y, res = T(0);
        if (!landing(ax, ay, x, y)) return false;
        aim2d<T>(landing, tx, ty, ax, ay, res, kSteps_, fd, cap, tol);
        if (landing(ax, ay, x, y)) { c.chief_x_mm = (float)x; c.chief_y_mm = (float)y; }
        else if (must_land) return false;
        c.beam_ax = (float)ax; c.beam_ay = (float)ay;
        c.status = status;
        c.aim_residual_mm = (float)res;
        c.pupil_fraction = (float)pupil_cloud(L, ax, ay, kFracN).frac;
        return true;
    };
    auto chief = [&](T ax, T ay, T& x, T& y) {
        L.set_lambda(T(kChiefLambda));
        const T bx = Math<T>::tan(ax), by = Math<T>::tan(ay);
        const Hit<T> h = L.trace(-T(kSpawnOffset) * bx, -T(kSpawnOffset) * by, ax, ay);
        if (!h.ok || !std::isfinite(h.x) || !std::isfinite(h.y)) return false;
        x = h.x; y = h.y;
        return true;
    };
    if (try_aim(chief, kFd, kTol, GL_PSF_CELL_OK, false)) return;
    auto cloud = [&](T ax, T ay, T& x, T& y) {
        const PupilCloud<T> p = pupil_cloud(L, ax, ay, kCloudN);
        if (p.hits < kMinHits) return false;
        x = p.mx; y = p.my;
        return true;
    };
    if (try_aim(cloud, kFd, kTolSoft, GL_PSF_CELL_CHIEF_VIGNETTED, false)) return;
    if (axial_ok)
    {
        Frame<T> track = axial_win;
        auto deep = [&](T ax, T ay, T& x, T& y) {
            Frame<T> w = track;
            L.set_lambda(T(kChiefLambda));
            const Coverage<T> d = follow(L, ax, ay, w);
            if (!(d.area > T(0)) || !std::isfinite(d.mx) || !std::isfinite(d.my)) return false;
            track = w;
            x = d.mx; y = d.my;
            return true;
        };
        if (track.r < T(1) && seed_mag > T(0))
        {
            const int steps = std::max(3, std::min(16, (int)std::ceil(seed_mag / T(0.10f))));
            T a, b;
            for (int k = 1; k <= steps; ++k)
            {
                const T f = T(k) / T(steps);
                deep(sx * f, sy * f, a, b);
            }
        }
        if (try_aim(deep, kDeepFd, kTolSoft, GL_PSF_CELL_CHIEF_VIGNETTED, true)) return;
    }
    c.beam_ax = (float)sx; c.beam_ay = (float)sy;
    c.chief_x_mm = (float)tx; c.chief_y_mm = (float)ty;
    c.status = GL_PSF_CELL_DARK;
    c.aim_residual_mm = 1e30f;
    c.pupil_fraction = 0.0f;
}

template <class T>
int psf_anchors(const gl_surface* s, int n, const float* src7, int n_src, int mode, gl_psf_cell* out)
{
    SetupLens<T> L;
    const int rc = L.open(s, n);
    if (rc) return rc;
    // where the pupil sits on axis: the deep-stop searches start there
    L.set_lambda(T(kChiefLambda));
    const Coverage<T> ax0 = cover(L, T(0), T(0), Frame<T>{}, kDiscSampling);
    const bool axial_ok = ax0.area > T(0);
    const Frame<T> axial_win = ax0.fit;
    for (int i = 0; i < n_src; ++i)
    {
        const float* q = src7 + 7 * (size_t)i;
        const T sx = T(q[0]), sy = T(q[1]);
        gl_psf_cell c{};
        c.beam_ax = q[0]; c.beam_ay = q[1];
        c.status = GL_PSF_CELL_OK;
        if (mode == GL_PSF_CENTER_FIXED_TARGET)
        {
            aim_tile(L, axial_ok, axial_win, sx, sy, T(q[5]), T(q[6]), c);
        }
        else
        {
            // the unweighted 7 x 7 pupil-mean landing; a deep pupil that the
            // full-disc cloud misses is found through the tracked axial window
            const PupilCloud<T> p = pupil_cloud(L, sx, sy, 7);
            c.chief_x_mm = (float)p.mx; c.chief_y_mm = (float)p.my;
            c.status = p.hits > 0 ? GL_PSF_CELL_OK : GL_PSF_CELL_DARK;
            c.pupil_fraction = (float)p.frac;
            if (p.hits == 0 && axial_ok)
            {
                Frame<T> w = axial_win;
                const T mag = Math<T>::sqrt(sx * sx + sy * sy);
                L.set_lambda(T(kChiefLambda));
                if (w.r < T(1) && mag > T(0))
                {
                    const int steps = std::max(3, std::min(16, (int)std::ceil(mag / T(0.10f))));
                    for (int k = 1; k <= steps; ++k) follow(L, sx * (T(k) / T(steps)), sy * (T(k) / T(steps)), w);
                }
                const Coverage<T> d = follow(L, sx, sy, w);
                if (d.area > T(0) && std::isfinite(d.mx) && std::isfinite(d.my))
                {
                    c.chief_x_mm = (float)d.mx; c.chief_y_mm = (float)d.my;
                    c.status = GL_PSF_CELL_OK;
                }
            }
        }
        if (!std::isfinite(c.aim_residual_mm)) c.aim_residual_mm = 0.0f;
        out[i] = c;
    }
    return GL_OK;
}

}  // namespace
}  // namespace setup
}  // namespace gl

using namespace gl;

extern "C" int gl_calibrate_lens2(const gl_surface* surfaces, int n, float lens_focal_length, float d_line_nm,
                                  int precision, gl_lens_calibration* out)
{
    if (!surfaces || n <= 0 || !out) return fail(GL_ERR_INVALID, "calibrate_lens: bad arguments");
    if (precision != GL_SETUP_FP32 && precision != GL_SETUP_FP64)
        return fail(GL_ERR_INVALID, "calibrate_lens: precision must be GL_SETUP_FP32 or GL_SETUP_FP64");
    return precision == GL_SETUP_FP64 ? setup::calibrate<double>(surfaces, n, lens_focal_length, d_line_nm, out)
                                      : setup::calibrate<float>(surfaces, n, lens_focal_length, d_line_nm, out);
}

extern "C" int gl_calibrate_lens(const gl_surface* surfaces, int n, float lens_focal_length, float d_line_nm,
                                 gl_lens_calibration* out)
{
    return gl_calibrate_lens2(surfaces, n, lens_focal_length, d_line_nm, GL_SETUP_FP32, out);
}

extern "C" int gl_solve_source_angle2(const gl_surface* surfaces, int n, const gl_lens_calibration* calib,
                                      float ndc_x, float ndc_y, float eff_half_w, float eff_half_h, int precision,
                                      gl_source_solve* out)
{
    if (!calib || !out) return fail(GL_ERR_INVALID, "solve_source_angle: bad arguments");
    if (precision != GL_SETUP_FP32 && precision != GL_SETUP_FP64)
        return fail(GL_ERR_INVALID, "solve_source_angle: precision must be GL_SETUP_FP32 or GL_SETUP_FP64");
    return precision == GL_SETUP_FP64
               ? setup::solve<double>(surfaces, n, *calib, ndc_x, ndc_y, eff_half_w, eff_half_h, out)
               : setup::solve<float>(surfaces, n, *calib, ndc_x, ndc_y, eff_half_w, eff_half_h, out);
}

extern "C" int gl_solve_source_angle(const gl_surface* surfaces, int n, const gl_lens_calibration* calib, float ndc_x,
                                     float ndc_y, float eff_half_w, float eff_half_h, gl_source_solve* out)
{
    return gl_solve_source_angle2(surfaces, n, calib, ndc_x, ndc_y, eff_half_w, eff_half_h, GL_SETUP_FP32, out);
}

extern "C" int gl_psf_prepass(const gl_surface* surfaces, int n, const float* sources7, int n_src, int center_mode,
                              gl_psf_cell* out)
{
    if (!surfaces || n <= 0 || (n_src > 0 && (!sources7 || !out)) || n_src < 0)
        return fail(GL_ERR_INVALID, "psf_prepass: bad arguments");
    return setup::psf_anchors<float>(surfaces, n, sources7, n_src, center_mode, out);
}

// The forward map of a solve (source_map_screen, source_map.cpp:456-483):
// the paraxial tangent map for a fallback, else the anchor's landing plus the
// Jacobian applied to tan of the angle offset (clamped at 1.55 rad).
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
    float px = dax, py = day;
    if (d > 1e-12f)
    {
        const float t = tanf(std::min(d, setup::kSolve.max_extend_rad));
        px = (dax / d) * t;
        py = (day / d) * t;
    }
    const float x = base->anchor_x + base->J[0] * px + base->J[1] * py;
    const float y = base->anchor_y + base->J[2] * px + base->J[3] * py;
    *out_sx = (base->eff_half_w > 0.0f) ? 0.5f + 0.5f * x / base->eff_half_w : 0.5f;
    *out_sy = (base->eff_half_h > 0.0f) ? 0.5f + 0.5f * y / base->eff_half_h : 0.5f;
    return GL_OK;
}
