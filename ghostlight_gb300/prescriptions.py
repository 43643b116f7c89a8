"""Seeded synthetic lens prescriptions for the flare-path workloads.

Each generator returns a list of ``gl_surface`` (sensor at z = 0, z laid out
by the thickness chain exactly like OpticalSystem::finalize,
ghostlight/src/optical_system.cpp:1425) built from
``numpy.random.default_rng(seed)``:

* ``double_gauss_12``  — 12 spherical glass surfaces + a 6-blade polygon stop
  between surfaces 6 and 7, R ~ +/-U(20,120) mm, t ~ U(1,12) mm, glasses with
  n_d ~ U(1.5,1.8) and V ~ U(30,60) fitted to 3-term Sellmeier, single-layer
  MgF2 on every glass surface, stop sized for f/2.
* ``wide_angle_24``    — 23 glass surfaces + stop (24 entries), two even
  aspheres with A4..A10 ~ N(0, 1e-6 * 10^(-2k)).
* ``anamorphic_18``    — 17 glass surfaces + stop (18 entries), 4 cylindrical
  surfaces forming a 1.5x squeeze front group, per-element decenter
  N(0, 0.05 mm) and tilt N(0, 0.1 deg).
* ``random_lens``      — 8..30 surfaces for the serving mix.

Focus, f-number and clear apertures come from a paraxial y-nu trace in FP64
(the per-lens paraxial setup the flare path keeps in double precision).
"""
from __future__ import annotations

import math

import numpy as np

from ._abi import default_surface, gl_surface

LAMBDA_D, LAMBDA_F, LAMBDA_C = 587.56, 486.13, 656.27
SELLMEIER_C = (0.006, 0.02, 100.0)
SELLMEIER_B3 = 1.0


# ---------------------------------------------------------------------------
# glass
# ---------------------------------------------------------------------------
def _sellmeier_terms(lam_nm: float):
    l2 = (lam_nm * 1e-3) ** 2
    return np.array([l2 / (l2 - c) for c in SELLMEIER_C])


def fit_sellmeier(n_d: float, v_d: float):
    """Three-term Sellmeier (B, C) with n(d) = n_d and n_F - n_C = (n_d-1)/V.

    C is fixed to a crown-like set; B3 (the IR term) is fixed and B1, B2 solve
    the two conditions (the F/C condition linearised through n_F+n_C with a
    partial dispersion P_dC = 0.3)."""
    dn = (n_d - 1.0) / v_d
    fd, ff, fc = _sellmeier_terms(LAMBDA_D), _sellmeier_terms(LAMBDA_F), _sellmeier_terms(LAMBDA_C)
    # n_F^2 - n_C^2 = (n_F - n_C)(n_F + n_C), n_F = n_d + 0.7 dn, n_C = n_d - 0.3 dn
    rhs1 = n_d * n_d - 1.0 - SELLMEIER_B3 * fd[2]
    rhs2 = dn * (2.0 * n_d + 0.4 * dn) - SELLMEIER_B3 * (ff[2] - fc[2])
    A = np.array([[fd[0], fd[1]], [ff[0] - fc[0], ff[1] - fc[1]]])
    b1, b2 = np.linalg.solve(A, np.array([rhs1, rhs2]))
    return (float(b1), float(b2), SELLMEIER_B3), SELLMEIER_C


def sellmeier_n_f32(B, Cc, lam_nm: float) -> np.float32:
    """sellmeier_n (ghostlight/src/fresnel.h:53-63) in float32 arithmetic."""
    f = np.float32
    l = f(lam_nm) * f(1e-3)
    l2 = l * l
    n2 = f(1.0)
    for i in range(3):
        n2 = n2 + f(B[i]) * l2 / (l2 - f(Cc[i]))
    return np.sqrt(n2) if n2 > 0 else f(1.0)


def sellmeier_to_abbe_f32(B, Cc):
    """n_d / V_d backfill of ghostlight/src/optical_system.cpp:69-77 (float32)."""
    f = np.float32
    n_d = sellmeier_n_f32(B, Cc, 587.56)
    n_f = sellmeier_n_f32(B, Cc, 486.13)
    n_c = sellmeier_n_f32(B, Cc, 656.27)
    v = (n_d - f(1.0)) / (n_f - n_c) if (n_f - n_c) > f(1e-9) else f(0.0)
    return float(n_d), float(v)


def set_glass(s: gl_surface, n_d: float, v_d: float) -> None:
    B, Cc = fit_sellmeier(n_d, v_d)
    s.disp_model = 2
    for k in range(3):
        s.sellmeier_B[k] = B[k]
        s.sellmeier_C[k] = Cc[k]
    nd32, v32 = sellmeier_to_abbe_f32([s.sellmeier_B[k] for k in range(3)],
                                      [s.sellmeier_C[k] for k in range(3)])
    s.ior = nd32
    s.abbe_v = v32


def set_air(s: gl_surface) -> None:
    s.disp_model = 0
    s.ior = 1.0
    s.abbe_v = 0.0


# ---------------------------------------------------------------------------
# paraxial layout (FP64)
# ---------------------------------------------------------------------------
def finalize_z(surfs) -> None:
    """OpticalSystem::finalize (optical_system.cpp:1425): float32 accumulation."""
    f = np.float32
    total = f(0.0)
    for s in surfs:
        total = f(total + f(s.thickness))
    z = f(-total)
    for s in surfs:
        s.z = float(z)
        z = f(z + f(s.thickness))


def _curv(s, plane: str) -> float:
    if abs(s.radius) < 1e-6:
        return 0.0
    if s.form == 2:  # cylinder: power only in its curving plane
        curving = "x" if s.cyl_axis == 1 else "y"   # CYL_AXIS_Y curves along X
        if plane != curving:
            return 0.0
    return 1.0 / s.radius


def paraxial_trace(surfs, y0: float, u0: float, plane: str = "y", lam: float = LAMBDA_D):
    """y-nu trace; returns per-surface heights and the final (y, u)."""
    ys = []
    y, nu, n = y0, u0, 1.0
    for i, s in enumerate(surfs):
        n2 = _index(s, lam)
        ys.append(y)
        nu = nu - y * (n2 - n) * _curv(s, plane)
        n = n2
        u = nu / n
        if i < len(surfs) - 1:
            y = y + u * s.thickness
    return ys, y, nu / n


def _index(s, lam):
    if s.disp_model == 2:
        l2 = (lam * 1e-3) ** 2
        n2 = 1.0 + sum(s.sellmeier_B[k] * l2 / (l2 - s.sellmeier_C[k]) for k in range(3))
        return math.sqrt(n2)
    return float(s.ior)


def paraxial_efl_bfd(surfs, plane="y"):
    """EFL and back focal distance (from the last vertex) for y0=1, u0=0."""
    ys, y_last, u_last = paraxial_trace(surfs, 1.0, 0.0, plane)
    if abs(u_last) < 1e-12:
        return math.inf, math.inf
    return -1.0 / u_last, -y_last / u_last


def _set_focus(surfs, plane="y"):
    surfs[-1].thickness = 0.0
    efl, bfd = paraxial_efl_bfd(surfs, plane)
    surfs[-1].thickness = float(bfd)
    return efl, bfd


def _stop_index(surfs):
    for i, s in enumerate(surfs):
        if s.is_stop:
            return i
    return None


def _set_apertures(surfs, f_number: float, field_deg: float, plane="y",
                   margin: float = 1.08, min_semi: float = 2.0):
    """Stop sized for f_number; other clear apertures from marginal+chief."""
    efl, _ = paraxial_efl_bfd(surfs, plane)
    epd_half = efl / (2.0 * f_number)
    st = _stop_index(surfs)
    ym, _, _ = paraxial_trace(surfs, epd_half, 0.0, plane)
    # chief ray: angle th, height h0 chosen so it crosses the stop centre
    th = math.tan(math.radians(field_deg))
    ya, _, _ = paraxial_trace(surfs, 0.0, th, plane)
    yb, _, _ = paraxial_trace(surfs, 1.0, th, plane)
    h0 = -ya[st] / (yb[st] - ya[st]) if abs(yb[st] - ya[st]) > 1e-12 else 0.0
    yc, _, _ = paraxial_trace(surfs, h0, th, plane)
    for i, s in enumerate(surfs):
        if i == st:
            s.semi_aperture = float(abs(ym[i]))
        else:
            s.semi_aperture = float(max(min_semi, margin * (abs(ym[i]) + abs(yc[i])) + 0.5))
    return efl


def _valid_geometry(surfs) -> bool:
    """Spheres must exceed their clear aperture; glass must not go negative at
    the rim (a real ray must be able to cross every element)."""
    for i, s in enumerate(surfs):
        if abs(s.radius) > 1e-6 and abs(s.radius) < 1.02 * s.semi_aperture:
            return False
    for i in range(len(surfs) - 1):
        a, b = surfs[i], surfs[i + 1]
        h = min(a.semi_aperture, b.semi_aperture)

        def sag(s):
            if abs(s.radius) < 1e-6:
                return 0.0
            R = s.radius
            return R - math.copysign(math.sqrt(max(R * R - h * h, 0.0)), R)
        edge = a.thickness + sag(b) - sag(a)
        if edge < 0.3:
            return False
    return True


def _new_surface(radius, thickness):
    s = default_surface()
    s.radius = float(radius)
    s.thickness = float(thickness)
    return s


def _stop(blades: int, rotation_deg: float = 0.0):
    s = default_surface()
    s.is_stop = 1
    set_air(s)
    if blades >= 3:
        s.aperture_shape = 1
        s.aperture_blades = blades
        s.aperture_rotation_rad = float(np.float32(math.radians(rotation_deg)))
    return s


def _coat_all(surfs):
    for s in surfs:
        if not s.is_stop:
            s.coating_model = 0
            s.ar_layers = 1


# ---------------------------------------------------------------------------
# generators
# ---------------------------------------------------------------------------
def double_gauss_12(seed: int = 1, f_number: float = 2.0, field_deg: float = 12.0):
    """Configuration 1: 12-surface double Gauss, stop between 6 and 7."""
    rng = np.random.default_rng(seed)
    for _attempt in range(4000):
        surfs = []
        for i in range(12):
            r = rng.uniform(20.0, 120.0)
            sign = 1.0 if i < 6 else -1.0          # classic DG bending
            s = _new_surface(sign * r, rng.uniform(1.0, 12.0))
            if i % 2 == 0:
                set_glass(s, rng.uniform(1.5, 1.8), rng.uniform(30.0, 60.0))
            else:
                set_air(s)
            surfs.append(s)
            if i == 5:
                gap = surfs[-1].thickness
                surfs[-1].thickness = gap * 0.5
                st = _stop(6)
                st.thickness = gap * 0.5
                surfs.append(st)
        efl, bfd = _set_focus(surfs)
        if not (30.0 < efl < 200.0 and 8.0 < bfd < 150.0):
            continue
        _set_apertures(surfs, f_number, field_deg)
        if not _valid_geometry(surfs):
            continue
        _coat_all(surfs)
        finalize_z(surfs)
        return surfs
    raise RuntimeError("double_gauss_12: no valid prescription for seed %d" % seed)


def wide_angle_24(seed: int = 2, f_number: float = 2.8, field_deg: float = 20.0):
    """Configuration 2: 24 entries (23 glass surfaces + stop), 2 aspheres."""
    rng = np.random.default_rng(seed)
    for _attempt in range(20000):
        surfs = []
        # front: 2 negative menisci, 3 singlets; stop; cemented doublet + 5 singlets
        elems = []
        elems.append(("neg", 2))
        elems.append(("neg", 2))
        elems += [("any", 2)] * 3
        elems.append(("stop", 0))
        elems.append(("cem", 3))
        elems += [("any", 2)] * 5
        for kind, nsurf in elems:
            if kind == "stop":
                st = _stop(7)
                st.thickness = rng.uniform(1.0, 6.0)
                surfs.append(st)
                continue
            if kind == "neg":
                r1 = rng.uniform(40.0, 120.0)
                r2 = rng.uniform(20.0, 0.7 * r1) if 0.7 * r1 > 20.0 else 20.0
                radii = [r1, r2]
            else:
                radii = [rng.choice([-1.0, 1.0]) * rng.uniform(20.0, 120.0) for _ in range(nsurf)]
            for k in range(nsurf):
                s = _new_surface(radii[k], rng.uniform(1.0, 12.0))
                if k < nsurf - 1:
                    set_glass(s, rng.uniform(1.5, 1.8), rng.uniform(30.0, 60.0))
                else:
                    set_air(s)
                surfs.append(s)
        efl, bfd = _set_focus(surfs)
        if not (15.0 < efl < 80.0 and 10.0 < bfd < 150.0):
            continue
        _set_apertures(surfs, f_number, field_deg, margin=1.1)
        if not _valid_geometry(surfs):
            continue
        # two even aspheres: front element's rear face and the last glass face
        glass_idx = [i for i, s in enumerate(surfs) if not s.is_stop]
        for i in (glass_idx[1], glass_idx[-2]):
            s = surfs[i]
            s.form = 1
            s.conic_k = 0.0
            s.n_asphere_terms = 4
            for k in range(4):
                s.asphere_terms[k] = float(rng.normal(0.0, 1e-6 * 10.0 ** (-2 * k)))
        _coat_all(surfs)
        finalize_z(surfs)
        return surfs
    raise RuntimeError("wide_angle_24: no valid prescription for seed %d" % seed)


def anamorphic_18(seed: int = 4, f_number: float = 2.8, field_deg: float = 20.0,
                  squeeze: float = 1.5):
    """Configuration 4: 18 entries, a 4-cylinder 1.5x squeeze group in front of
    a spherical prime, per-element decenter and tilt."""
    rng = np.random.default_rng(seed)
    for _attempt in range(20000):
        surfs = []
        # Cylinder group (curving along X, CYL_AXIS_Y): negative then positive
        # element; afocal in X with magnification ~1/squeeze.
        fa = -rng.uniform(60.0, 110.0)
        fb = -fa * squeeze
        for f_el in (fa, fb):
            n_d = rng.uniform(1.5, 1.8)
            v_d = rng.uniform(30.0, 60.0)
            # thin-lens bending: pick R2, solve R1 for the element power
            r2 = -np.sign(f_el) * rng.uniform(200.0, 400.0)
            r1 = 1.0 / (1.0 / ((n_d - 1.0) * f_el) + 1.0 / r2)
            s1 = _new_surface(r1, rng.uniform(2.0, 8.0))
            s1.form = 2
            s1.cyl_axis = 1
            set_glass(s1, n_d, v_d)
            s2 = _new_surface(r2, 0.0)
            s2.form = 2
            s2.cyl_axis = 1
            set_air(s2)
            surfs += [s1, s2]
        surfs[3].thickness = rng.uniform(3.0, 8.0)
        # adjust the air gap so the group is afocal in X (paraxial, FP64)
        best = None
        for gap in np.linspace(1.0, 200.0, 800):
            surfs[1].thickness = float(gap)
            _, y, u = paraxial_trace(surfs[:4], 1.0, 0.0, "x")
            if best is None or abs(u) < best[0]:
                best = (abs(u), gap)
        surfs[1].thickness = float(best[1])
        # spherical prime: 6 singlets + stop (13 entries) -> 17 + ... = 18 total
        prime = []
        for i in range(7):
            if i == 3:
                st = _stop(8)
                st.thickness = rng.uniform(1.0, 5.0)
                prime.append(st)
            r1 = rng.choice([-1.0, 1.0]) * rng.uniform(20.0, 120.0)
            r2 = rng.choice([-1.0, 1.0]) * rng.uniform(20.0, 120.0)
            if i == 6:
                s = _new_surface(r1, rng.uniform(1.0, 12.0))
                set_air(s)
                prime.append(s)
                break
            s1 = _new_surface(r1, rng.uniform(1.0, 12.0))
            set_glass(s1, rng.uniform(1.5, 1.8), rng.uniform(30.0, 60.0))
            s2 = _new_surface(r2, rng.uniform(1.0, 12.0))
            set_air(s2)
            prime += [s1, s2]
        surfs = surfs + prime
        if len(surfs) != 18:
            # trim or pad the tail to exactly 18 entries
            surfs = surfs[:18]
            if not surfs[-1].disp_model == 0:
                continue
        efl, bfd = _set_focus(surfs, "y")
        if not (20.0 < efl < 120.0 and 10.0 < bfd < 150.0):
            continue
        efl_x, _ = paraxial_efl_bfd(surfs, "x")
        _set_apertures(surfs, f_number, field_deg, "y", margin=1.1)
        # widen for the x plane (the anamorphic axis)
        save = [s.semi_aperture for s in surfs]
        _set_apertures(surfs, f_number, field_deg, "x", margin=1.1)
        st = _stop_index(surfs)
        for i, s in enumerate(surfs):
            s.semi_aperture = float(max(save[i], s.semi_aperture)) if i != st else save[i]
        if not _valid_geometry(surfs):
            continue
        # element decenters / tilts (both surfaces of an element share them)
        i = 0
        while i < len(surfs):
            s = surfs[i]
            if s.is_stop or s.disp_model == 0:
                i += 1
                continue
            dx, dy = rng.normal(0.0, 0.05, 2)
            tx, ty = np.radians(rng.normal(0.0, 0.1, 2))
            R = _rot_xy(tx, ty)
            j = i
            while j < len(surfs):
                surfs[j].decenter_x = float(dx)
                surfs[j].decenter_y = float(dy)
                for k in range(9):
                    surfs[j].rot[k] = float(R[k])
                if surfs[j].disp_model == 0:
                    break
                j += 1
            i = j + 1
        _coat_all(surfs)
        finalize_z(surfs)
        return surfs
    raise RuntimeError("anamorphic_18: no valid prescription for seed %d" % seed)


def _rot_xy(tx: float, ty: float):
    cx, sx, cy, sy = math.cos(tx), math.sin(tx), math.cos(ty), math.sin(ty)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    return (Ry @ Rx).astype(np.float32).reshape(-1)


def random_lens(seed: int, n_surfaces: int, f_number: float = 2.8, field_deg: float = 20.0):
    """Serving mix: n_surfaces entries (one of them the stop)."""
    rng = np.random.default_rng(seed)
    n_glass = n_surfaces - 1
    for _attempt in range(20000):
        surfs = []
        k = 0
        stop_at = n_glass // 2
        while k < n_glass:
            if len(surfs) == stop_at + (len(surfs) > stop_at) * 0 and not any(s.is_stop for s in surfs) and k >= stop_at:
                st = _stop(int(rng.integers(5, 10)))
                st.thickness = rng.uniform(1.0, 5.0)
                surfs.append(st)
            r = rng.choice([-1.0, 1.0]) * rng.uniform(20.0, 120.0)
            s = _new_surface(r, rng.uniform(1.0, 12.0))
            if (k % 2 == 0) and k < n_glass - 1:
                set_glass(s, rng.uniform(1.5, 1.8), rng.uniform(30.0, 60.0))
            else:
                set_air(s)
            surfs.append(s)
            k += 1
        if not any(s.is_stop for s in surfs):
            st = _stop(6)
            surfs.insert(len(surfs) // 2, st)
        if surfs[-1].disp_model != 0:
            set_air(surfs[-1])
        efl, bfd = _set_focus(surfs)
        if not (15.0 < efl < 200.0 and 8.0 < bfd < 150.0):
            continue
        _set_apertures(surfs, f_number, field_deg)
        if not _valid_geometry(surfs):
            continue
        _coat_all(surfs)
        finalize_z(surfs)
        return surfs
    raise RuntimeError("random_lens: no valid prescription for seed %d" % seed)


def stop_crossing(surfs, a: int, b: int) -> bool:
    """True when the pair (a, b) straddles the aperture stop."""
    st = _stop_index(surfs)
    if st is None:
        return False
    return (a < st) != (b < st)
