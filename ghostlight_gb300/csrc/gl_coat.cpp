// gl_coat.cpp — table-backed coatings: the table store, their residency on
// each device, and the thin-film (layers) bake.
//
// The reference keeps a surface's tables in OpticalSystem::coating_tables
// (optical_system.h:285-301) and patches raw pointers into the Surface POD
// (sync_coating_pointers, optical_system.cpp:1457-1481); its GPU renderers
// pack them into a per-render device blob (coating_upload.cu).  Here a table
// is an immutable, content-addressed entry of a process-wide store: the
// surface record carries the entry's id in `ar_layers`, creating the same
// table twice gives the same id, and an entry is copied to a device once, on
// first use there, and stays resident (tables are a few KB).  So a lens with
// table coatings packs into the trace records without a per-render upload,
// and the records of a captured graph keep pointing at live data.  The same
// store holds the bitmaps of IMAGE apertures (model kStoreImage: width x
// height luminance, the boundary semi-diameter in the angle-medium slot),
// named by the surface's aperture_blades.
//
// gl_coating_bake_layers restates OpticalSystem::bake_coating_layers
// (optical_system.cpp:1483-1575) over the thin-film transfer matrix of
// tmm.h: the characteristic matrix of each layer, multiplied front to back,
// gives the stack's amplitude reflectance r = (eta0 B - C) / (eta0 B + C)
// for s and p, and R = (|rs|^2 + |rp|^2) / 2, sampled on 400..700 nm (10 nm)
// x 0..85 degrees (5 degrees) of incidence in the medium before the surface.
// Complex float arithmetic in the same operation order (this unit is built
// with -ffp-contract=off, std::complex<float> as in the reference), so the
// baked table equals the reference's.
#include "gl_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

namespace gl {

namespace {

constexpr int kMaxDevices = 64;

struct TableEntry {
    int model = 0;                 // GL_COATING_SPECTRAL / ANGULAR / SPECTRAL_ANGULAR
    int n0 = 0, n1 = 0;
    int discard = 0;
    float ref_ior = 1.0f;
    std::vector<float> data;       // [axis0 | axis1 | r]
    void* dev[kMaxDevices] = {};
};

std::mutex g_mu;
std::vector<std::unique_ptr<TableEntry>> g_tables;       // id = index + 1
std::map<std::vector<uint32_t>, int> g_by_content;

std::vector<uint32_t> content_key(const TableEntry& e)
{
    std::vector<uint32_t> k(5 + e.data.size());
    uint32_t ref;
    std::memcpy(&ref, &e.ref_ior, 4);
    k[0] = (uint32_t)e.model; k[1] = (uint32_t)e.n0; k[2] = (uint32_t)e.n1;
    k[3] = (uint32_t)e.discard; k[4] = ref;
    if (!e.data.empty()) std::memcpy(k.data() + 5, e.data.data(), e.data.size() * 4);
    return k;
}

int intern(std::unique_ptr<TableEntry> e, int32_t* out_id)
{
    std::lock_guard<std::mutex> lock(g_mu);
    auto key = content_key(*e);
    auto it = g_by_content.find(key);
    if (it != g_by_content.end())
    {
        *out_id = it->second;
        return GL_OK;
    }
    g_tables.push_back(std::move(e));
    const int id = (int)g_tables.size();
    g_by_content.emplace(std::move(key), id);
    *out_id = id;
    return GL_OK;
}

TableEntry* lookup(int id)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (id < 1 || id > (int)g_tables.size()) return nullptr;
    return g_tables[(size_t)id - 1].get();
}

// ---- thin-film stack (tmm.h) ----------------------------------------------
using cplx = std::complex<float>;

struct FilmLayer {
    cplx n;
    float thickness_nm;
};

// cosine of the propagation angle in a medium of complex index n for the
// Snell invariant n0 sin(theta0), on the branch with Im(n cos) >= 0
cplx film_cos(const cplx& n, float invariant)
{
    const cplx s = cplx(invariant, 0.0f) / n;
    cplx c = std::sqrt(cplx(1.0f, 0.0f) - s * s);
    if ((n * c).imag() < 0.0f) c = -c;
    return c;
}

// amplitude reflectance of the stack for one polarisation: tilted
// admittances eta = n cos (s) or n / cos (p)
cplx film_amplitude(const std::vector<FilmLayer>& layers, const cplx& n_amb, const cplx& n_sub,
                    float lambda_nm, float invariant, bool s_pol)
{
    const cplx one(1.0f, 0.0f);
    auto admittance = [&](const cplx& n) {
        const cplx c = film_cos(n, invariant);
        return s_pol ? n * c : n / c;
    };
    const cplx eta0 = admittance(n_amb);
    const cplx eta_sub = admittance(n_sub);
    cplx m00 = one, m01(0.0f, 0.0f), m10(0.0f, 0.0f), m11 = one;
    for (const FilmLayer& L : layers)
    {
        const cplx c = film_cos(L.n, invariant);
        const cplx eta = s_pol ? L.n * c : L.n / c;
        const cplx phase = cplx(2.0f * 3.14159265358979323846f * L.thickness_nm / lambda_nm, 0.0f) * L.n * c;
        const cplx cd = std::cos(phase);
        const cplx sd = std::sin(phase);
        const cplx isd(-sd.imag(), sd.real());
        // characteristic matrix [[cos, i sin / eta], [i eta sin, cos]]
        const cplx a00 = cd, a01 = isd / eta, a10 = isd * eta, a11 = cd;
        const cplx p00 = m00 * a00 + m01 * a10;
        const cplx p01 = m00 * a01 + m01 * a11;
        const cplx p10 = m10 * a00 + m11 * a10;
        const cplx p11 = m10 * a01 + m11 * a11;
        m00 = p00; m01 = p01; m10 = p10; m11 = p11;
    }
    const cplx B = m00 + m01 * eta_sub;
    const cplx C = m10 + m11 * eta_sub;
    return (eta0 * B - C) / (eta0 * B + C);
}

float film_reflectance(const std::vector<FilmLayer>& layers, cplx n_amb, cplx n_sub, float lambda_nm,
                       float aoi_deg)
{
    const float theta0 = aoi_deg * (3.14159265358979323846f / 180.0f);
    const float invariant = n_amb.real() * std::sin(theta0);
    const cplx rs = film_amplitude(layers, n_amb, n_sub, lambda_nm, invariant, true);
    const cplx rp = film_amplitude(layers, n_amb, n_sub, lambda_nm, invariant, false);
    float R = 0.5f * (std::norm(rs) + std::norm(rp));
    if (R < 0.0f) R = 0.0f;
    if (R > 1.0f) R = 1.0f;
    return R;
}

// complex index of a layer at lambda (nm) from its n,k samples (um),
// linear between samples, clamped at the ends
cplx layer_index(const float* lam_um, const float* nn, const float* kk, int m, float lambda_nm)
{
    const float lu = lambda_nm * 1e-3f;
    if (lu <= lam_um[0]) return {nn[0], kk[0]};
    if (lu >= lam_um[m - 1]) return {nn[m - 1], kk[m - 1]};
    for (int k = 1; k < m; ++k)
    {
        if (lu <= lam_um[k])
        {
            const float span = lam_um[k] - lam_um[k - 1];
            const float f = (span > 0.0f) ? (lu - lam_um[k - 1]) / span : 0.0f;
            return {nn[k - 1] + f * (nn[k] - nn[k - 1]), kk[k - 1] + f * (kk[k] - kk[k - 1])};
        }
    }
    return {nn[m - 1], kk[m - 1]};
}

float ior_before_at(const gl_surface* s, int idx, float lam)
{
    for (int k = idx - 1; k >= 0; --k)
        if (s[k].is_active) return ior_at(s[k], lam);
    return 1.0f;
}

}  // namespace

// Table address of entry `id` for a trace on `device` (kTablesHost: the
// host copy).  The first request on a device copies the entry there, unless
// `may_upload` is false (an allocation-free caller), which then fails.
int coating_table_address(int id, int model, int device, bool may_upload, const float** out, int* n0, int* n1,
                          int* discard, float* ref_ior)
{
    TableEntry* e = lookup(id);
    if (!e) return fail(GL_ERR_INVALID, "unknown coating table id " + std::to_string(id));
    if (e->model != model)
        return fail(GL_ERR_INVALID, "coating table " + std::to_string(id) + " holds model " +
                                        std::to_string(e->model) + ", the surface asks for " + std::to_string(model));
    *n0 = e->n0;
    *n1 = e->n1;
    *discard = e->discard;
    *ref_ior = e->ref_ior;
    if (device == kTablesHost)
    {
        *out = e->data.data();
        return GL_OK;
    }
    if (device < 0 || device >= kMaxDevices) return fail(GL_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!e->dev[device])
    {
        if (!may_upload)
            return fail(GL_ERR_UNSUPPORTED, "coating table " + std::to_string(id) +
                                                " is not resident on this device (gl_coating_table_prepare)");
        void* p = nullptr;
        const size_t bytes = e->data.size() * sizeof(float);
        GL_CUDA_TRY(cudaMalloc(&p, bytes));
        cudaError_t ce = cudaMemcpy(p, e->data.data(), bytes, cudaMemcpyHostToDevice);
        if (ce != cudaSuccess)
        {
            cudaFree(p);
            return fail(GL_ERR_CUDA, std::string("coating table upload: ") + cudaGetErrorString(ce));
        }
        e->dev[device] = p;
    }
    *out = static_cast<const float*>(e->dev[device]);
    return GL_OK;
}

}  // namespace gl

using namespace gl;

extern "C" int gl_coating_table_create(int32_t model, const float* axis0, int32_t n0, const float* axis1,
                                       int32_t n1, const float* r, float angle_ref_ior,
                                       int32_t out_of_range_discard, int32_t* out_id)
{
    if (!out_id || !axis0 || !r || n0 < 1) return fail(GL_ERR_INVALID, "coating_table_create: bad arguments");
    auto e = std::make_unique<TableEntry>();
    e->model = model;
    e->discard = out_of_range_discard ? 1 : 0;
    e->ref_ior = angle_ref_ior;
    if (model == GL_COATING_SPECTRAL || model == GL_COATING_ANGULAR)
    {
        if (n1 != 0) return fail(GL_ERR_INVALID, "coating_table_create: a 1-D table has no second axis");
        e->n0 = n0;
        e->data.assign(axis0, axis0 + n0);
        e->data.insert(e->data.end(), r, r + n0);
        if (model == GL_COATING_SPECTRAL) e->ref_ior = 1.0f;   // no angle axis
    }
    else if (model == GL_COATING_SPECTRAL_ANGULAR)
    {
        if (!axis1 || n1 < 1) return fail(GL_ERR_INVALID, "coating_table_create: missing angle axis");
        e->n0 = n0;
        e->n1 = n1;
        e->data.assign(axis0, axis0 + n0);
        e->data.insert(e->data.end(), axis1, axis1 + n1);
        e->data.insert(e->data.end(), r, r + (size_t)n0 * n1);
        if (!std::is_sorted(axis1, axis1 + n1))
            return fail(GL_ERR_INVALID, "coating_table_create: angles must be sorted ascending");
    }
    else
    {
        return fail(GL_ERR_INVALID, "coating_table_create: model " + std::to_string(model) + " has no table");
    }
    if (!std::is_sorted(axis0, axis0 + n0))
        return fail(GL_ERR_INVALID, "coating_table_create: keys must be sorted ascending");
    return intern(std::move(e), out_id);
}

extern "C" int gl_aperture_image_create(int32_t width, int32_t height, const float* pixels, float semi_diameter,
                                        int32_t* out_id)
{
    if (!out_id || !pixels || width < 1 || height < 1 || (long long)width * height > (1LL << 28))
        return fail(GL_ERR_INVALID, "aperture_image_create: bad arguments");
    if (!std::isfinite(semi_diameter) || semi_diameter < 0.0f)
        return fail(GL_ERR_INVALID, "aperture_image_create: semi_diameter must be finite and non-negative");
    auto e = std::make_unique<TableEntry>();
    e->model = kStoreImage;
    e->n0 = width;
    e->n1 = height;
    e->ref_ior = semi_diameter;
    e->data.assign(pixels, pixels + (size_t)width * height);
    return intern(std::move(e), out_id);
}

extern "C" int gl_coating_table_info(int32_t id, int32_t* model, int32_t* n0, int32_t* n1, float* angle_ref_ior,
                                     int32_t* out_of_range_discard)
{
    TableEntry* e = lookup(id);
    if (!e) return fail(GL_ERR_INVALID, "unknown coating table id " + std::to_string(id));
    if (model) *model = e->model;
    if (n0) *n0 = e->n0;
    if (n1) *n1 = e->n1;
    if (angle_ref_ior) *angle_ref_ior = e->ref_ior;
    if (out_of_range_discard) *out_of_range_discard = e->discard;
    return GL_OK;
}

extern "C" int gl_coating_table_read(int32_t id, float* axis0, float* axis1, float* r)
{
    TableEntry* e = lookup(id);
    if (!e) return fail(GL_ERR_INVALID, "unknown coating table id " + std::to_string(id));
    const float* d = e->data.data();
    if (e->model == kStoreImage)
    {
        if (r) std::memcpy(r, d, (size_t)e->n0 * e->n1 * 4);
        return GL_OK;
    }
    if (axis0) std::memcpy(axis0, d, (size_t)e->n0 * 4);
    if (axis1 && e->n1) std::memcpy(axis1, d + e->n0, (size_t)e->n1 * 4);
    const size_t nr = (e->n1 ? (size_t)e->n0 * e->n1 : (size_t)e->n0);
    if (r) std::memcpy(r, d + e->n0 + e->n1, nr * 4);
    return GL_OK;
}

extern "C" int gl_coating_table_prepare(int32_t id)
{
    int dev = 0;
    GL_CUDA_TRY(cudaGetDevice(&dev));
    TableEntry* e = lookup(id);
    if (!e) return fail(GL_ERR_INVALID, "unknown coating table id " + std::to_string(id));
    const float* p;
    int a, b, c;
    float d;
    return coating_table_address(id, e->model, dev, true, &p, &a, &b, &c, &d);
}

extern "C" int gl_coating_bake_layers(const gl_surface* surfaces, int32_t n, int32_t index, int32_t n_layers,
                                      const float* thickness_nm, const int32_t* nk_count, const float* nk_lambda_um,
                                      const float* nk_n, const float* nk_k, int32_t* out_id)
{
    if (!surfaces || n < 1 || index < 0 || index >= n || n_layers < 1 || !thickness_nm || !nk_count ||
        !nk_lambda_um || !nk_n || !nk_k || !out_id)
        return fail(GL_ERR_INVALID, "coating_bake_layers: bad arguments");
    std::vector<int> first((size_t)n_layers);
    int total = 0;
    for (int l = 0; l < n_layers; ++l)
    {
        if (nk_count[l] < 1 || !(thickness_nm[l] > 0.0f))
            return fail(GL_ERR_INVALID, "coating layer stack has a layer with no nk data or non-positive thickness");
        first[(size_t)l] = total;
        total += nk_count[l];
    }
    constexpr float kLamMin = 400.0f, kLamStep = 10.0f, kAngStep = 5.0f;
    constexpr int kNw = 31, kNa = 18;
    std::vector<float> wl(kNw), ang(kNa), R((size_t)kNw * kNa);
    for (int a = 0; a < kNa; ++a) ang[(size_t)a] = 0.0f + a * kAngStep;
    std::vector<FilmLayer> film((size_t)n_layers);
    for (int w = 0; w < kNw; ++w)
    {
        const float lam = kLamMin + w * kLamStep;
        wl[(size_t)w] = lam;
        const float n_amb = ior_before_at(surfaces, index, lam);
        const float n_sub = ior_at(surfaces[index], lam);
        for (int l = 0; l < n_layers; ++l)
        {
            const int o = first[(size_t)l];
            film[(size_t)l].n = layer_index(nk_lambda_um + o, nk_n + o, nk_k + o, nk_count[l], lam);
            film[(size_t)l].thickness_nm = thickness_nm[l];
        }
        for (int a = 0; a < kNa; ++a)
            R[(size_t)w * kNa + a] = film_reflectance(film, {n_amb, 0.0f}, {n_sub, 0.0f}, lam, ang[(size_t)a]);
    }
    // the angle axis is measured in the medium before the surface
    const float ref = ior_before_at(surfaces, index, 587.56f);
    return gl_coating_table_create(GL_COATING_SPECTRAL_ANGULAR, wl.data(), kNw, ang.data(), kNa, R.data(), ref, 0,
                                   out_id);
}
