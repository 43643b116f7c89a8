/*
 * gl_oracle_impl.h — CPU restatement of the reference flare-path algorithm,
 * instantiated twice by gl_oracle.c: REAL = float (the reference host
 * arithmetic, used to pin decisions bit-exactly) and REAL = double (the FP64
 * oracle images are checked against).
 *
 * TEST INFRASTRUCTURE ONLY — imported by tests/, smoke() and bench.py's
 * cpu_baseline leg; never by the product.
 *
 * Each function cites the reference function (JaydenB/ghostlight, path within
 * that project) whose steps it restates.  Expected macros:
 *   R            scalar type            SFX(x)   name suffixing
 *   SQRT COS SIN ATAN2 FMOD FABS TAN EXP ASIN FLOOR FMIN FMAX
 */

typedef struct { R x, y, z; } SFX(v3);

static inline SFX(v3) SFX(mk)(R x, R y, R z) { SFX(v3) v; v.x = x; v.y = y; v.z = z; return v; }
static inline SFX(v3) SFX(add)(SFX(v3) a, SFX(v3) b) { return SFX(mk)(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline SFX(v3) SFX(sub)(SFX(v3) a, SFX(v3) b) { return SFX(mk)(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline SFX(v3) SFX(scl)(SFX(v3) a, R s) { return SFX(mk)(a.x * s, a.y * s, a.z * s); }
static inline SFX(v3) SFX(neg)(SFX(v3) a) { return SFX(mk)(-a.x, -a.y, -a.z); }
static inline R SFX(dot)(SFX(v3) a, SFX(v3) b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* Vec3f::normalized, ghostlight/src/vec3.h:48-52 */
static inline SFX(v3) SFX(normalized)(SFX(v3) a)
{
    R l = SQRT(a.x * a.x + a.y * a.y + a.z * a.z);
    return (l > (R)1e-12f) ? SFX(scl)(a, (R)1 / l) : SFX(mk)(0, 0, 0);
}

/* mat3_mul / mat3_T_mul / rot_is_identity, trace_core.h:33-57 */
static inline SFX(v3) SFX(m3mul)(const float* m, SFX(v3) v)
{
    return SFX(mk)((R)m[0] * v.x + (R)m[1] * v.y + (R)m[2] * v.z,
                   (R)m[3] * v.x + (R)m[4] * v.y + (R)m[5] * v.z,
                   (R)m[6] * v.x + (R)m[7] * v.y + (R)m[8] * v.z);
}
static inline SFX(v3) SFX(m3tmul)(const float* m, SFX(v3) v)
{
    return SFX(mk)((R)m[0] * v.x + (R)m[3] * v.y + (R)m[6] * v.z,
                   (R)m[1] * v.x + (R)m[4] * v.y + (R)m[7] * v.z,
                   (R)m[2] * v.x + (R)m[5] * v.y + (R)m[8] * v.z);
}

/* world_to_surface_point, trace_core.h:59-66 */
static inline SFX(v3) SFX(world_to_local)(SFX(v3) p, const gl_surface* s)
{
    if (s->decenter_x == 0.0f && s->decenter_y == 0.0f && orc_rot_identity(s->rot)) return p;
    SFX(v3) V = SFX(mk)((R)s->decenter_x, (R)s->decenter_y, (R)s->z);
    return SFX(add)(SFX(m3tmul)(s->rot, SFX(sub)(p, V)), SFX(mk)(0, 0, (R)s->z));
}

/* dispersion_ior, fresnel.h:27-48 (Cauchy from n_d and V_d) */
static inline R SFX(dispersion_ior)(R n_d, R V_d, R lam)
{
    if (V_d < (R)0.1f || n_d <= (R)1.0001f) return n_d;
    const R lF = (R)486.13f, lC = (R)656.27f, ld = (R)587.56f;
    R dn = (n_d - (R)1) / V_d;
    R iF = (R)1 / (lF * lF), iC = (R)1 / (lC * lC), id = (R)1 / (ld * ld);
    R B = dn / (iF - iC);
    R A = n_d - B * id;
    return A + B / (lam * lam);
}

/* sellmeier_n, fresnel.h:53-63 */
static inline R SFX(sellmeier_n)(const float* B, const float* Cc, R lam)
{
    R l = lam * (R)1e-3f;
    R l2 = l * l;
    R n2 = 1;
    n2 += (R)B[0] * l2 / (l2 - (R)Cc[0]);
    n2 += (R)B[1] * l2 / (l2 - (R)Cc[1]);
    n2 += (R)B[2] * l2 / (l2 - (R)Cc[2]);
    return (n2 > (R)0) ? SQRT(n2) : (R)1;
}

/* Surface::ior_at, optical_system.h:230-235 */
static inline R SFX(ior_at)(const gl_surface* s, R lam)
{
    if (s->disp_model == GL_DISP_SELLMEIER) return SFX(sellmeier_n)(s->sellmeier_B, s->sellmeier_C, lam);
    return SFX(dispersion_ior)((R)s->ior, (R)s->abbe_v, lam);
}

/* OpticalSystem::ior_before (wavelength form), optical_system.h:395-402 */
static inline R SFX(ior_before)(const gl_surface* s, int n, int idx, R lam)
{
    if (idx > n) idx = n;
    for (int k = idx - 1; k >= 0; --k)
        if (s[k].is_active) return SFX(ior_at)(&s[k], lam);
    return (R)1;
}

/* fresnel_reflectance, fresnel.h:69-84 */
static inline R SFX(fresnel)(R cos_i, R n1, R n2)
{
    cos_i = FABS(cos_i);
    R eta = n1 / n2;
    R sin2_t = eta * eta * ((R)1 - cos_i * cos_i);
    if (sin2_t >= (R)1) return (R)1;
    R cos_t = SQRT((R)1 - sin2_t);
    R rs = (n1 * cos_i - n2 * cos_t) / (n1 * cos_i + n2 * cos_t);
    R rp = (n2 * cos_i - n1 * cos_t) / (n2 * cos_i + n1 * cos_t);
    return (R)0.5f * (rs * rs + rp * rp);
}

/* coating_reflectance, fresnel.h:92-121 (single-layer Airy) */
static inline R SFX(coating_reflectance)(R cos_i, R n1, R n2, R cn, R d_nm, R lam)
{
    R sin2_c = (n1 / cn) * (n1 / cn) * ((R)1 - cos_i * cos_i);
    if (sin2_c >= (R)1) return SFX(fresnel)(cos_i, n1, n2);
    R cos_c = SQRT((R)1 - sin2_c);
    R delta = (R)2 * (R)(float)M_PI * cn * d_nm * cos_c / lam;
    R r01 = (n1 * cos_i - cn * cos_c) / (n1 * cos_i + cn * cos_c);
    R sin2_2 = (cn / n2) * (cn / n2) * ((R)1 - cos_c * cos_c);
    if (sin2_2 >= (R)1) return SFX(fresnel)(cos_i, n1, n2);
    R cos_2 = SQRT((R)1 - sin2_2);
    R r12 = (cn * cos_c - n2 * cos_2) / (cn * cos_c + n2 * cos_2);
    R c2d = COS((R)2 * delta);
    R num = r01 * r01 + r12 * r12 + (R)2 * r01 * r12 * c2d;
    R den = (R)1 + r01 * r01 * r12 * r12 + (R)2 * r01 * r12 * c2d;
    R Rr = num / den;
    return FMIN(FMAX(Rr, (R)0), (R)1);
}

/* artist_reflectance, fresnel.h:135-153 */
static inline R SFX(artist_reflectance)(R tr, R tg, R tb, R strength, R lam)
{
    const R inv_2s2 = (R)(1.0f / (2.0f * 65.0f * 65.0f));
    R dr = lam - (R)650, dg = lam - (R)550, db = lam - (R)450;
    R br = EXP(-dr * dr * inv_2s2), bg = EXP(-dg * dg * inv_2s2), bb = EXP(-db * db * inv_2s2);
    R sum = br + bg + bb;
    R Rr = strength * (tr * br + tg * bg + tb * bb) / sum;
    return FMIN(FMAX(Rr, (R)0), (R)1);
}

/* surface_reflectance, fresnel.h:159-178 (MgF2 quarter-wave at 550 nm) */
static inline R SFX(surface_reflectance)(R cos_i, R n1, R n2, int layers, R lam)
{
    if (layers <= 0) return SFX(fresnel)(cos_i, n1, n2);
    const R mgf2 = (R)1.38f, design = (R)550.0f;
    R qw = design / ((R)4 * mgf2);
    R Rr = SFX(coating_reflectance)(cos_i, n1, n2, mgf2, qw, lam);
    for (int i = 1; i < layers; ++i) Rr *= (R)0.25f;
    return FMIN(FMAX(Rr, (R)0), (R)1);
}

/* coating_lerp_1d, trace_core.h:575-602: the end rows are returned as they
 * are, the interior linearly; *dropped in discard mode outside the keys */
static inline R SFX(table_lerp)(const float* key, const float* r, int n, R x, int discard, int* dropped)
{
    if (x <= (R)key[0]) { if (discard && x < (R)key[0]) *dropped = 1; return (R)r[0]; }
    if (x >= (R)key[n - 1]) { if (discard && x > (R)key[n - 1]) *dropped = 1; return (R)r[n - 1]; }
    for (int i = 1; i < n; ++i)
        if (x <= (R)key[i])
        {
            R span = (R)key[i] - (R)key[i - 1];
            R f = (span > 0) ? (x - (R)key[i - 1]) / span : (R)0;
            return (R)r[i - 1] + f * ((R)r[i] - (R)r[i - 1]);
        }
    return (R)r[n - 1];
}

/* the bracketing of one SPECTRAL_ANGULAR axis, trace_core.h:699-752 */
static inline void SFX(table_axis)(const float* ax, int n, R x, int discard, int* i0, R* f, int* dropped)
{
    *i0 = 0; *f = 0;
    if (x <= (R)ax[0]) { if (discard && x < (R)ax[0]) *dropped = 1; return; }
    if (x >= (R)ax[n - 1])
    {
        *i0 = (n > 1) ? n - 2 : 0; *f = (n > 1) ? (R)1 : (R)0;
        if (discard && x > (R)ax[n - 1]) *dropped = 1;
        return;
    }
    for (int i = 1; i < n; ++i)
        if (x <= (R)ax[i])
        {
            R span = (R)ax[i] - (R)ax[i - 1];
            *i0 = i - 1;
            *f = (span > 0) ? (x - (R)ax[i - 1]) / span : (R)0;
            return;
        }
}

/* coating_ref_angle_deg, trace_core.h:614-621 */
static inline R SFX(table_angle)(R cos_i, R n1, R ref_ior)
{
    R sin_i = SQRT(FMAX((R)0, (R)1 - cos_i * cos_i));
    R s_ref = (ref_ior > 0) ? (n1 * sin_i / ref_ior) : sin_i;
    if (s_ref >= (R)1) return (R)90.0f;
    return ASIN(s_ref) * ((R)180.0f / (R)(float)M_PI);
}

/* surface_weight, trace_core.h:635-783 */
static inline R SFX(surface_weight)(SFX(v3) dir, SFX(v3) nrm, R n1, R n2,
                                     const gl_surface* s, R lam, int reflecting)
{
    R cos_i = FABS(SFX(dot)(nrm, dir));
    R Rr;
    const orc_table* t = (s->coating_model >= 1 && s->coating_model <= 3) ? orc_coating_find(s->ar_layers) : NULL;
    if (s->coating_model == GL_COATING_SIMPLE)
        Rr = SFX(surface_reflectance)(cos_i, n1, n2, s->ar_layers, lam);
    else if (s->coating_model == GL_COATING_ARTIST)
        Rr = SFX(artist_reflectance)((R)s->tint_r, (R)s->tint_g, (R)s->tint_b,
                                     (R)s->tint_strength, lam);
    else if (t && t->model == s->coating_model)
    {
        int dropped = 0;
        if (t->model == 1)
            Rr = SFX(table_lerp)(t->data, t->data + t->n0, t->n0, lam, t->discard, &dropped);
        else if (t->model == 2)
            Rr = SFX(table_lerp)(t->data, t->data + t->n0, t->n0, SFX(table_angle)(cos_i, n1, (R)t->ref_ior),
                                 t->discard, &dropped);
        else
        {
            const int nw = t->n0, na = t->n1;
            const float* rr = t->data + nw + na;
            const R ang = SFX(table_angle)(cos_i, n1, (R)t->ref_ior);
            int iw, ia;
            R fw, fa;
            SFX(table_axis)(t->data, nw, lam, t->discard, &iw, &fw, &dropped);
            SFX(table_axis)(t->data + nw, na, ang, t->discard, &ia, &fa, &dropped);
            if (dropped) return 0;
            const int iw1 = (iw + 1 < nw) ? iw + 1 : iw, ia1 = (ia + 1 < na) ? ia + 1 : ia;
            Rr = ((R)1 - fw) * (((R)1 - fa) * (R)rr[iw * na + ia] + fa * (R)rr[iw * na + ia1])
               + fw * (((R)1 - fa) * (R)rr[iw1 * na + ia] + fa * (R)rr[iw1 * na + ia1]);
        }
        if (dropped) return 0;
    }
    else
        Rr = SFX(fresnel)(cos_i, n1, n2);
    Rr = FMIN(FMAX(Rr, (R)0), (R)1);
    return reflecting ? Rr : ((R)1 - Rr);
}

/* surface_attenuator, trace_core.h:791-809 */
static inline R SFX(surface_attenuator)(SFX(v3) hit, const gl_surface* s)
{
    if (s->coating_model == GL_COATING_ATTENUATOR)
    {
        if (!(s->gauss_sigma > 0.0f)) return (R)s->gauss_background;
        SFX(v3) l = SFX(world_to_local)(hit, s);
        R dx = l.x - (R)s->gauss_decenter_x, dy = l.y - (R)s->gauss_decenter_y;
        R r2 = dx * dx + dy * dy;
        R s2 = (R)s->gauss_sigma * (R)s->gauss_sigma;
        return (R)s->gauss_background + (R)s->gauss_peak * EXP((R)-0.5f * r2 / s2);
    }
    return (R)1;
}

/* ApertureProfile::radius_at, aperture_profile.h:124-200 (u_edge, fold,
 * u_raw, sector_angle) on a float-built profile, in R */
static inline R SFX(blade_u_edge)(const orc_blade* b, R phi)
{
    const R psi = phi - (R)b->phi_w;
    const R sh = SIN((R)0.5f * psi);
    return (R)b->u_w - (R)b->u_rise * (sh * sh) * (R)((psi >= (R)0) ? b->qR : b->qL);
}
static inline R SFX(blade_radius)(const orc_blade* b, R theta)
{
    const R sigma = (R)b->sigma, half = (R)b->half;
    R phi = FMOD(theta - (R)b->rotation, sigma);
    if (phi < (R)0) phi += sigma;
    phi -= half;
    R u = SFX(blade_u_edge)(b, phi);
    if (b->facets)
    {
        R w = FMOD(phi - half + half, sigma);
        if (w < (R)0) w += sigma;
        w -= half;
        if (w >= -(R)b->eA && w <= (R)b->eB)
        {
            const R uf = COS(w + half - (R)b->beta) / (R)b->p;
            if (uf > u) u = uf;
        }
    }
    return (R)1 / u;
}

/* check_aperture, trace_core.h:133-170 (circle / ellipse / polygon, plain or
 * with its authored blade shape) */
static inline int SFX(check_aperture)(SFX(v3) hit, const gl_surface* s)
{
    R hx = hit.x / (R)s->aperture_aspect;
    R hy = hit.y;
    R h2 = hx * hx + hy * hy;
    if (!(h2 <= (R)s->semi_aperture * (R)s->semi_aperture)) return 0;
    if (s->aperture_shape == GL_APERTURE_POLYGON)
    {
        R r = SQRT(h2);
        if (r < (R)1e-9f) return 1;
        if (orc_blade_authored(s))
        {
            const orc_blade b = orc_make_blade(s);
            return r <= (R)s->semi_aperture * SFX(blade_radius)(&b, ATAN2(hy, hx));
        }
        const R sector = (R)2 * (R)(float)M_PI / (R)s->aperture_blades;
        const R angle = ATAN2(hy, hx) - (R)s->aperture_rotation_rad;
        R off = FMOD(angle, sector);
        if (off < (R)0) off += sector;
        off -= (R)0.5f * sector;
        const R apothem = (R)s->semi_aperture * COS((R)0.5f * sector);
        return r <= apothem / COS(off);
    }
    if (s->aperture_shape == GL_APERTURE_IMAGE)
    {
        /* sample_aperture_image, trace.cpp:31-48: nearest pixel > 0.5 */
        const orc_table* t = orc_coating_find(s->aperture_blades);
        if (!t || t->model != 100) return 1;          /* not loaded: passthrough */
        if (!(s->aperture_aspect > 0.0f) || !(t->ref_ior > 0.0f)) return 0;
        const R u = (R)0.5f + hit.x / (R)s->aperture_aspect / ((R)2.0f * (R)t->ref_ior);
        const R v = (R)0.5f + hit.y / ((R)2.0f * (R)t->ref_ior);
        if (u < 0 || u > 1 || v < 0 || v > 1) return 0;
        const int px = (int)(u * (R)(t->n0 - 1) + (R)0.5f);
        const int py = (int)(v * (R)(t->n1 - 1) + (R)0.5f);
        return t->data[(size_t)py * t->n0 + px] > 0.5f;
    }
    return 1;
}

/* asphere_sag / asphere_dsag_dr, trace_core.h:75-112 */
static inline R SFX(asag)(R r, R invR, R K, const float* t, int nt)
{
    if (nt < 0) nt = 0;
    if (nt > 8) nt = 8;
    R r2 = r * r;
    R D = (R)1 - ((R)1 + K) * invR * invR * r2;
    if (D <= (R)0) return (R)1e30f;
    R z = invR * r2 / ((R)1 + SQRT(D));
    R rp = r2 * r2;
    for (int i = 0; i < nt; ++i) { z += (R)t[i] * rp; rp *= r2; }
    return z;
}
static inline R SFX(adsag)(R r, R invR, R K, const float* t, int nt)
{
    if (nt < 0) nt = 0;
    if (nt > 8) nt = 8;
    R r2 = r * r;
    R D = (R)1 - ((R)1 + K) * invR * invR * r2;
    if (D <= (R)0) return (R)0;
    R dz = invR * r / SQRT(D);
    R rp = r2 * r;
    for (int i = 0; i < nt; ++i) { dz += ((R)4 + (R)2 * (R)i) * (R)t[i] * rp; rp *= r2; }
    return dz;
}

/* Pick the root closest to the vertex plane (trace_core.h:376-389 etc.) */
static inline int SFX(pick_root)(R t1, R t2, R oz, R dz, R sz, R* t)
{
    if (t1 > (R)1e-6f && t2 > (R)1e-6f)
    {
        R z1 = oz + t1 * dz, z2 = oz + t2 * dz;
        *t = (FABS(z1 - sz) < FABS(z2 - sz)) ? t1 : t2;
    }
    else if (t1 > (R)1e-6f) *t = t1;
    else if (t2 > (R)1e-6f) *t = t2;
    else return 0;
    return 1;
}

/* intersect_surface, trace_core.h:299-525 */
static int SFX(intersect)(SFX(v3) ro, SFX(v3) rd, const gl_surface* s, R* t_out, SFX(v3)* n_out)
{
    int transformed = (s->decenter_x != 0.0f || s->decenter_y != 0.0f || !orc_rot_identity(s->rot));
    SFX(v3) o = ro, d = rd;
    const R sz = (R)s->z;
    if (transformed)
    {
        SFX(v3) V = SFX(mk)((R)s->decenter_x, (R)s->decenter_y, sz);
        o = SFX(add)(SFX(m3tmul)(s->rot, SFX(sub)(ro, V)), SFX(mk)(0, 0, sz));
        d = SFX(m3tmul)(s->rot, rd);
    }
    if (FABS((R)s->radius) < (R)1e-6f)
    {
        if (FABS(d.z) < (R)1e-12f) return 0;
        R t = (sz - o.z) / d.z;
        if (!(t > (R)1e-6f)) return 0;
        SFX(v3) hit = SFX(add)(o, SFX(scl)(d, t));
        if (!SFX(check_aperture)(hit, s)) return 0;
        *t_out = t;
        SFX(v3) nn = SFX(mk)(0, 0, (d.z > (R)0) ? (R)-1 : (R)1);
        *n_out = transformed ? SFX(m3mul)(s->rot, nn) : nn;
        return 1;
    }
    if (s->form == GL_FORM_ASPHERE)
    {
        R Rr = (R)s->radius, invR = (R)1 / Rr, K = (R)s->conic_k;
        SFX(v3) ctr = SFX(mk)(0, 0, sz + Rr);
        SFX(v3) oc = SFX(sub)(o, ctr);
        R qa = SFX(dot)(d, d), qb = (R)2 * SFX(dot)(oc, d), qc = SFX(dot)(oc, oc) - Rr * Rr;
        R disc = qb * qb - (R)4 * qa * qc;
        R t;
        if (disc >= (R)0)
        {
            R sd = SQRT(disc), i2a = (R)0.5f / qa;
            R t1 = (-qb - sd) * i2a, t2 = (-qb + sd) * i2a;
            if (!SFX(pick_root)(t1, t2, o.z, d.z, sz, &t)) return 0;
        }
        else
        {
            if (FABS(d.z) < (R)1e-12f) return 0;
            t = (sz - o.z) / d.z;
            if (!(t > (R)1e-6f)) return 0;
        }
        for (int it = 0; it < 15; ++it)
        {
            SFX(v3) hi = SFX(add)(o, SFX(scl)(d, t));
            R rx = hi.x, ry = hi.y, rad = SQRT(rx * rx + ry * ry);
            R sag = SFX(asag)(rad, invR, K, s->asphere_terms, s->n_asphere_terms);
            if (sag > (R)1e29f) return 0;
            R f = hi.z - sz - sag;
            if (FABS(f) < (R)1e-5f) break;
            R ds = SFX(adsag)(rad, invR, K, s->asphere_terms, s->n_asphere_terms);
            R rs = (rad > (R)1e-9f) ? rad : (R)1e-9f;
            R dfdt = d.z - ds * (rx * d.x + ry * d.y) / rs;
            if (FABS(dfdt) < (R)1e-12f) break;
            t -= f / dfdt;
        }
        if (!(t > (R)1e-6f)) return 0;
        SFX(v3) hit = SFX(add)(o, SFX(scl)(d, t));
        R rad = SQRT(hit.x * hit.x + hit.y * hit.y);
        if (!SFX(check_aperture)(hit, s)) return 0;
        R rs = (rad > (R)1e-9f) ? rad : (R)1e-9f;
        R ds = SFX(adsag)(rad, invR, K, s->asphere_terms, s->n_asphere_terms);
        SFX(v3) nrm = SFX(mk)(-ds * hit.x / rs, -ds * hit.y / rs, (R)1);
        R nl = SQRT(nrm.x * nrm.x + nrm.y * nrm.y + nrm.z * nrm.z);
        nrm = SFX(scl)(nrm, (R)1 / nl);
        if (SFX(dot)(nrm, d) > (R)0) nrm = SFX(neg)(nrm);
        if (transformed) nrm = SFX(m3mul)(s->rot, nrm);
        *t_out = t; *n_out = nrm;
        return 1;
    }
    if (s->form == GL_FORM_CYLINDRICAL)
    {
        R vx, vy;
        if (s->cyl_axis == GL_CYL_AXIS_Y) { vx = 1; vy = 0; } else { vx = 0; vy = 1; }
        R Rr = (R)s->radius;
        R oc_v = o.x * vx + o.y * vy;
        R oc_z = o.z - sz - Rr;
        R dv = d.x * vx + d.y * vy;
        R qa = dv * dv + d.z * d.z;
        R qb = (R)2 * (oc_v * dv + oc_z * d.z);
        R qc = oc_v * oc_v + oc_z * oc_z - Rr * Rr;
        R disc = qb * qb - (R)4 * qa * qc;
        if (disc < (R)0) return 0;
        R sd = SQRT(disc), i2a = (R)0.5f / qa;
        R t1 = (-qb - sd) * i2a, t2 = (-qb + sd) * i2a, t;
        if (!SFX(pick_root)(t1, t2, o.z, d.z, sz, &t)) return 0;
        SFX(v3) hit = SFX(add)(o, SFX(scl)(d, t));
        if (!SFX(check_aperture)(hit, s)) return 0;
        R hv = hit.x * vx + hit.y * vy;
        SFX(v3) nrm = SFX(mk)(hv * vx, hv * vy, hit.z - sz - Rr);
        R nl = SQRT(nrm.x * nrm.x + nrm.y * nrm.y + nrm.z * nrm.z);
        if (nl < (R)1e-12f) return 0;
        nrm = SFX(scl)(nrm, (R)1 / nl);
        if (SFX(dot)(nrm, d) > (R)0) nrm = SFX(neg)(nrm);
        if (transformed) nrm = SFX(m3mul)(s->rot, nrm);
        *t_out = t; *n_out = nrm;
        return 1;
    }
    {
        R Rr = (R)s->radius;
        SFX(v3) ctr = SFX(mk)(0, 0, sz + Rr);
        SFX(v3) oc = SFX(sub)(o, ctr);
        R a = SFX(dot)(d, d), b = (R)2 * SFX(dot)(oc, d), c = SFX(dot)(oc, oc) - Rr * Rr;
        R disc = b * b - (R)4 * a * c;
        if (disc < (R)0) return 0;
        R sd = SQRT(disc), i2a = (R)0.5f / a;
        R t1 = (-b - sd) * i2a, t2 = (-b + sd) * i2a, t;
        if (!SFX(pick_root)(t1, t2, o.z, d.z, sz, &t)) return 0;
        SFX(v3) hit = SFX(add)(o, SFX(scl)(d, t));
        if (!SFX(check_aperture)(hit, s)) return 0;
        SFX(v3) nrm = SFX(scl)(SFX(sub)(hit, ctr), (R)1 / FABS(Rr));
        if (SFX(dot)(nrm, d) > (R)0) nrm = SFX(neg)(nrm);
        if (transformed) nrm = SFX(m3mul)(s->rot, nrm);
        *t_out = t; *n_out = nrm;
        return 1;
    }
}

/* refract_ray, trace_core.h:533-552 */
static inline int SFX(refract)(SFX(v3) d, SFX(v3) nrm, R n1, R n2, SFX(v3)* out)
{
    R nr = n1 / n2;
    R ci = -SFX(dot)(nrm, d);
    R s2t = nr * nr * ((R)1 - ci * ci);
    if (s2t >= (R)1) return 0;
    R ct = SQRT((R)1 - s2t);
    SFX(v3) tmp = SFX(add)(SFX(scl)(d, nr), SFX(scl)(nrm, nr * ci - ct));
    R sq = tmp.x * tmp.x + tmp.y * tmp.y + tmp.z * tmp.z;
    if (sq < (R)1e-18f) return 0;
    *out = SFX(scl)(tmp, (R)1 / SQRT(sq));
    return 1;
}

/* reflect_ray, trace_core.h:559-564 */
static inline SFX(v3) SFX(reflect)(SFX(v3) d, SFX(v3) nrm)
{
    return SFX(normalized)(SFX(sub)(d, SFX(scl)(nrm, (R)2 * SFX(dot)(d, nrm))));
}

typedef struct { R x, y, z, w; int status; } SFX(result);

/* trace_surface_step, trace.cpp:84-135: returns 1 to continue, 0 when dead */
static inline int SFX(step)(SFX(v3)* o, SFX(v3)* d, const gl_surface* s, R lam, R n2,
                            int reflecting, R reflect_ior, R* cur, SFX(result)* res)
{
    R t = 0; SFX(v3) nrm;
    if (!SFX(intersect)(*o, *d, s, &t, &nrm)) return 0;
    SFX(v3) hit = SFX(add)(*o, SFX(scl)(*d, t));
    *o = hit;
    const R n1 = *cur;
    if (reflecting)
    {
        R fw = SFX(surface_weight)(*d, nrm, n1, n2, s, lam, 1);
        res->w *= fw;
        res->w *= SFX(surface_attenuator)(hit, s);
        *d = SFX(reflect)(*d, nrm);
        *cur = reflect_ior;
    }
    else
    {
        SFX(v3) nd;
        if (!SFX(refract)(*d, nrm, n1, n2, &nd)) { res->status = GL_TRACE_TIR; return 0; }
        R fw = SFX(surface_weight)(*d, nrm, n1, n2, s, lam, 0);
        res->w *= fw;
        res->w *= SFX(surface_attenuator)(hit, s);
        *d = nd;
        *cur = n2;
    }
    return 1;
}

/* propagate_to_sensor, trace.cpp:147-162 */
static inline void SFX(to_sensor)(SFX(v3) o, SFX(v3) d, SFX(result)* res)
{
    if (FABS(d.z) < (R)1e-12f) { res->status = GL_TRACE_MISSED_SURFACE; return; }
    R ts = -o.z / d.z;
    if (!(ts >= (R)0)) { res->status = GL_TRACE_MISSED_SURFACE; return; }
    res->x = o.x + d.x * ts; res->y = o.y + d.y * ts; res->z = o.z + d.z * ts;
    res->status = GL_TRACE_OK;
}

/* trace_ghost_ray, trace.cpp:171-237 */
static SFX(result) SFX(trace_ghost)(const gl_surface* S, int N, SFX(v3) o, SFX(v3) d, R lam, int a, int b)
{
    SFX(result) res; res.x = res.y = res.z = 0; res.w = 1; res.status = GL_TRACE_VIGNETTED;
    if (a < 0 || b < 0 || a >= b || b >= N) { res.status = GL_TRACE_INVALID_INPUT; res.w = 0; return res; }
    R cur = 1;
    for (int s = 0; s <= b; ++s)
    {
        if (!S[s].is_active) continue;
        R n2 = SFX(ior_at)(&S[s], lam);
        if (!SFX(step)(&o, &d, &S[s], lam, n2, s == b, cur, &cur, &res)) return res;
    }
    for (int s = b - 1; s >= a; --s)
    {
        if (!S[s].is_active) continue;
        R n2 = SFX(ior_before)(S, N, s, lam);
        R rior = (s == a) ? SFX(ior_at)(&S[a], lam) : cur;
        if (!SFX(step)(&o, &d, &S[s], lam, n2, s == a, rior, &cur, &res)) return res;
    }
    for (int s = a + 1; s < N; ++s)
    {
        if (!S[s].is_active) continue;
        R n2 = SFX(ior_at)(&S[s], lam);
        if (!SFX(step)(&o, &d, &S[s], lam, n2, 0, cur, &cur, &res)) return res;
    }
    SFX(to_sensor)(o, d, &res);
    return res;
}

/* trace_primary_ray, trace.cpp:243-268 */
static SFX(result) SFX(trace_primary)(const gl_surface* S, int N, SFX(v3) o, SFX(v3) d, R lam)
{
    SFX(result) res; res.x = res.y = res.z = 0; res.w = 1; res.status = GL_TRACE_VIGNETTED;
    R cur = 1;
    for (int s = 0; s < N; ++s)
    {
        if (!S[s].is_active) continue;
        R n2 = SFX(ior_at)(&S[s], lam);
        if (!SFX(step)(&o, &d, &S[s], lam, n2, 0, cur, &cur, &res)) return res;
    }
    SFX(to_sensor)(o, d, &res);
    return res;
}

/* Bilinear point splat of one traced ray-wavelength, ghost_render.cu:423-463,
 * into three double planes. */
static inline void SFX(splat)(double* img, int W, int H, R px, R py, R cr, R cg, R cb)
{
    const size_t npx = (size_t)W * H;
    int x0 = (int)FLOOR(px - (R)0.5f), y0 = (int)FLOOR(py - (R)0.5f);
    R fx = (px - (R)0.5f) - (R)x0, fy = (py - (R)0.5f) - (R)y0;
    const R wt[4] = {((R)1 - fx) * ((R)1 - fy), fx * ((R)1 - fy), ((R)1 - fx) * fy, fx * fy};
    const int ox[4] = {0, 1, 0, 1}, oy[4] = {0, 0, 1, 1};
    const R c[3] = {cr, cg, cb};
    for (int k = 0; k < 4; ++k)
    {
        int xi = x0 + ox[k], yi = y0 + oy[k];
        if (xi < 0 || xi >= W || yi < 0 || yi >= H) continue;
        size_t pix = (size_t)yi * W + xi;
        for (int ch = 0; ch < 3; ++ch)
            if (FABS(c[ch]) > (R)1e-14f) img[ch * npx + pix] += (double)(c[ch] * wt[k]);
    }
}
