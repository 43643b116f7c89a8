// gl_serve.cu — serving path: resident lenses and stream-ordered flare
// requests.
//
// The reference renders one flare per blocking call, behind process-wide
// mutexes (ghost_render.cu:504-511), re-uploading the lens and rebuilding the
// pupil grid each time.  A server instead keeps per lens, in HBM: the packed
// surface table, the filtered ghost pairs, the off-sensor probe grids, and
// caches of IOR slices (per wavelength set) and Morton-ordered pupil grids
// (per grid side).  A request then only needs its accumulator, a few counters
// and its spectral table, all carved from one stream-ordered pool allocation,
// so creating, running and freeing it never synchronises the device: requests
// on different streams overlap on the GPU, and the CTA scheduler interleaves
// them (by stream priority) at CTA boundaries when a request runs as short
// CTAs (items_per_warp > 0).
//
// Work items are uniform: every pair traces the request's one pupil grid, so
// item i = (pair, source, 32-sample tile) is computed from the index and no
// item list is built or uploaded per request.
#include "gl_render.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

namespace gl {
namespace {

struct IorSet {
    float* at = nullptr;
    float* bf = nullptr;
};

struct GridSet {
    float2* samples = nullptr;
    int n = 0;
};

cudaMemPool_t g_pool[64] = {};
std::mutex g_pool_mutex;

// One pool per device; freed blocks stay reserved (release threshold at the
// maximum), so a steady request mix stops touching the driver's allocator.
cudaError_t device_pool(int dev, cudaMemPool_t* out)
{
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_pool_mutex);
    if (!g_pool[dev])
    {
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool;
        cudaError_t e = cudaMemPoolCreate(&pool, &props);
        if (e != cudaSuccess) return e;
        uint64_t thr = ~0ull;
        e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        if (e != cudaSuccess) { cudaMemPoolDestroy(pool); return e; }
        g_pool[dev] = pool;
    }
    *out = g_pool[dev];
    return cudaSuccess;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Pinned host words that receive each request's trace count at the end of
// its stream work, so reading it after completion needs no CUDA call.
constexpr int kTracedSlots = 8192;
unsigned long long* g_traced_host = nullptr;
unsigned g_traced_next = 0;
std::mutex g_traced_mutex;

unsigned long long* traced_slot()
{
    std::lock_guard<std::mutex> lk(g_traced_mutex);
    if (!g_traced_host)
    {
        void* p = nullptr;
        if (cudaHostAlloc(&p, sizeof(unsigned long long) * kTracedSlots, cudaHostAllocDefault) != cudaSuccess)
            return nullptr;
        g_traced_host = static_cast<unsigned long long*>(p);
    }
    return g_traced_host + (g_traced_next++ % kTracedSlots);
}

}  // namespace

// The device's stream-ordered pool (shared by requests and plans).
cudaError_t shared_device_pool(int dev, cudaMemPool_t* out) { return device_pool(dev, out); }


struct ResidentLens {
    int device = 0;
    int n_surf = 0, n_pairs = 0;
    std::vector<gl_surface> surfaces;
    SurfRec* recs = nullptr;
    PairDev* pairs = nullptr;
    float2* probe = nullptr;
    int probe_begin[4] = {0, 0, 0, 0};
    float front_R = 0.0f, start_z = 0.0f;
    int blades_override = 0;
    float rotation_deg = 0.0f;
    size_t smem_max = 0;
    std::mutex mu;
    std::map<std::vector<float>, IorSet> ior;
    std::map<int, GridSet> grids;
    long long device_bytes = 0;
};

struct Request {
    ResidentLens* lens = nullptr;
    int width = 0, height = 0, n_spec = 0, n_src = 0, grid_n = 0, tiles = 0, n_items = 0;
    int l_chunks = 1;                 // wavelength ranges per item (tasks per item), set at create
    gl_ghost_render_params prm{};
    IorSet ior;
    const float2* samples = nullptr;
    unsigned char* block = nullptr;   // one pool allocation, carved below
    float4* accum = nullptr;
    float* planes = nullptr;          // the request's own r | g | b output planes
    float4* spec = nullptr;
    SourceDev* sources = nullptr;
    int* counters = nullptr;          // 3 probe passes + render
    unsigned long long* traced = nullptr;
    unsigned long long* traced_host = nullptr;   // pinned slot, written at the end of the stream work
    int* pair_hits = nullptr;
    bool cull = false;
    size_t smem = 0;
    long long rays = 0, probe_rays = 0;
    size_t bytes = 0;
    std::vector<float4> h_spec;
    std::vector<SourceDev> h_src;
};

static int lens_ior(ResidentLens* L, const gl_spectral_sample* spec, int n_spec, IorSet* out)
{
    std::vector<float> key((size_t)n_spec);
    for (int i = 0; i < n_spec; ++i) key[i] = spec[i].lambda;
    std::lock_guard<std::mutex> lk(L->mu);
    auto it = L->ior.find(key);
    if (it != L->ior.end()) { *out = it->second; return GL_OK; }
    std::vector<float> at((size_t)n_spec * L->n_surf), bf((size_t)n_spec * L->n_surf);
    build_ior_tables(L->surfaces.data(), L->n_surf, key.data(), n_spec, at.data(), bf.data());
    IorSet s;
    cudaError_t e = cudaMalloc(&s.at, at.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&s.bf, bf.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(s.at, at.data(), at.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(s.bf, bf.data(), bf.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
    {
        cudaFree(s.at); cudaFree(s.bf);
        return fail(e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA, std::string("lens IOR tables: ") + cudaGetErrorString(e));
    }
    L->device_bytes += (long long)(at.size() + bf.size()) * 4;
    L->ior[key] = s;
    *out = s;
    return GL_OK;
}

static int lens_grid(ResidentLens* L, int ray_grid, GridSet* out)
{
    std::lock_guard<std::mutex> lk(L->mu);
    auto it = L->grids.find(ray_grid);
    if (it != L->grids.end()) { *out = it->second; return GL_OK; }
    gl_sampler_params sp{ray_grid, 0, 0, L->blades_override, L->rotation_deg};
    std::vector<gl_pupil_sample> g, o;
    int rc = build_aperture_samples(L->surfaces.data(), L->n_surf, sp, g);
    if (rc) return rc;
    o.resize(g.size());
    morton_order(g.data(), (int)g.size(), o.data());
    GridSet s;
    s.n = (int)o.size();
    cudaError_t e = cudaMalloc(&s.samples, std::max<size_t>(1, o.size()) * sizeof(float2));
    if (e == cudaSuccess && !o.empty())
        e = cudaMemcpy(s.samples, o.data(), o.size() * sizeof(float2), cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
    {
        cudaFree(s.samples);
        return fail(e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA, std::string("lens pupil grid: ") + cudaGetErrorString(e));
    }
    L->device_bytes += (long long)o.size() * 8;
    L->grids[ray_grid] = s;
    *out = s;
    return GL_OK;
}

static void lens_free(ResidentLens* L)
{
    if (!L) return;
    cudaFree(L->recs); cudaFree(L->pairs); cudaFree(L->probe);
    for (auto& kv : L->ior) { cudaFree(kv.second.at); cudaFree(kv.second.bf); }
    for (auto& kv : L->grids) cudaFree(kv.second.samples);
    delete L;
}

}  // namespace gl

using namespace gl;

struct gl_lens { ResidentLens* p; };
struct gl_request { Request* p; };

extern "C" {

int gl_lens_create(const gl_surface* surfaces, int n_surfaces, const gl_ghost_pair* pairs, const float* boosts,
                   int n_pairs, int blades_override, float rotation_deg, gl_lens** out)
{
    if (!out || !surfaces || n_surfaces <= 0) return fail(GL_ERR_INVALID, "lens_create: bad arguments");
    if (n_pairs < 0 || (n_pairs > 0 && (!pairs || !boosts))) return fail(GL_ERR_INVALID, "lens_create: missing pairs");
    for (int i = 0; i < n_pairs; ++i)
    {
        const int a = pairs[i].surf_a, b = pairs[i].surf_b;
        if (a < 0 || b <= a || b >= n_surfaces)
            return fail(GL_ERR_INVALID, "lens_create: bounce indices must satisfy 0 <= a < b < n");
    }
    int dev = 0;
    GL_CUDA_TRY(cudaGetDevice(&dev));
    std::vector<SurfRec> recs((size_t)n_surfaces);
    int rc = pack_lens(surfaces, n_surfaces, recs.data(), dev);
    if (rc) return rc;
    ResidentLens* L = new ResidentLens();
    cudaGetDevice(&L->device);
    L->n_surf = n_surfaces;
    L->n_pairs = n_pairs;
    L->surfaces.assign(surfaces, surfaces + n_surfaces);
    L->front_R = surfaces[0].semi_aperture;     // ghost_render.cu:738-739
    L->start_z = surfaces[0].z - kSpawnOffset;
    L->blades_override = blades_override;
    L->rotation_deg = rotation_deg;
    std::vector<PairDev> pd((size_t)std::max(1, n_pairs));
    for (int i = 0; i < n_pairs; ++i) pd[i] = {pairs[i].surf_a, pairs[i].surf_b, boosts[i], 0.0f};
    std::vector<gl_pupil_sample> probe;
    rc = probe_grids(surfaces, n_surfaces, blades_override, rotation_deg, probe, L->probe_begin);
    if (rc) { delete L; return rc; }
    cudaError_t e = cudaMalloc(&L->recs, recs.size() * sizeof(SurfRec));
    if (e == cudaSuccess) e = cudaMalloc(&L->pairs, pd.size() * sizeof(PairDev));
    if (e == cudaSuccess) e = cudaMalloc(&L->probe, std::max<size_t>(1, probe.size()) * sizeof(float2));
    if (e == cudaSuccess) e = cudaMemcpy(L->recs, recs.data(), recs.size() * sizeof(SurfRec), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(L->pairs, pd.data(), pd.size() * sizeof(PairDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !probe.empty())
        e = cudaMemcpy(L->probe, probe.data(), probe.size() * sizeof(float2), cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
    {
        lens_free(L);
        return fail(e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA, std::string("lens_create: ") + cudaGetErrorString(e));
    }
    L->device_bytes = (long long)(recs.size() * sizeof(SurfRec) + pd.size() * sizeof(PairDev) + probe.size() * 8);
    *out = new gl_lens{L};
    return GL_OK;
}

int gl_lens_prepare(gl_lens* lens, int ray_grid, const gl_spectral_sample* spec, int n_spec)
{
    if (!lens) return fail(GL_ERR_INVALID, "lens_prepare: null lens");
    if (ray_grid > 0)
    {
        if (ray_grid > 1024) return fail(GL_ERR_INVALID, "lens_prepare: ray_grid above 1024");
        GridSet g;
        int rc = lens_grid(lens->p, ray_grid, &g);
        if (rc) return rc;
    }
    if (spec && n_spec > 0)
    {
        if (n_spec > kMaxSpec) return fail(GL_ERR_INVALID, "lens_prepare: spectral table must hold 1..256 samples");
        IorSet s;
        int rc = lens_ior(lens->p, spec, n_spec, &s);
        if (rc) return rc;
    }
    return GL_OK;
}

int gl_lens_info(const gl_lens* lens, int* n_pairs, long long* device_bytes)
{
    if (!lens) return fail(GL_ERR_INVALID, "lens_info: null lens");
    if (n_pairs) *n_pairs = lens->p->n_pairs;
    if (device_bytes) *device_bytes = lens->p->device_bytes;
    return GL_OK;
}

int gl_lens_destroy(gl_lens* lens)
{
    if (!lens) return GL_OK;
    lens_free(lens->p);
    delete lens;
    return GL_OK;
}

int gl_request_create(gl_lens* lens, int ray_grid, const gl_spectral_sample* spec, int n_spec,
                      const gl_flare_source* sources, int n_sources, const gl_ghost_render_params* prm,
                      void* stream, gl_request** out)
{
    if (!lens || !out || !prm) return fail(GL_ERR_INVALID, "request_create: null argument");
    if (ray_grid < 1 || ray_grid > 1024) return fail(GL_ERR_INVALID, "request_create: ray_grid must be 1..1024");
    if (n_spec < 1 || n_spec > kMaxSpec || !spec) return fail(GL_ERR_INVALID, "request_create: spectral table must hold 1..256 samples");
    if (n_sources < 0 || (n_sources > 0 && !sources)) return fail(GL_ERR_INVALID, "request_create: bad sources");
    if (prm->width <= 0 || prm->height <= 0) return fail(GL_ERR_INVALID, "request_create: width and height must be positive");
    if ((long long)prm->width * prm->height > (1LL << 31)) return fail(GL_ERR_INVALID, "request_create: image has too many pixels");
    if (!(prm->sensor_half_w > 0.0f) || !(prm->sensor_half_h > 0.0f))
        return fail(GL_ERR_INVALID, "request_create: sensor half extents must be positive");
    ResidentLens* L = lens->p;
    Request* r = new Request();
    r->lens = L;
    r->prm = *prm;
    r->width = prm->width; r->height = prm->height; r->n_spec = n_spec; r->n_src = n_sources;
    r->l_chunks = default_lambda_split(n_spec);
    int rc = lens_ior(L, spec, n_spec, &r->ior);
    GridSet g;
    if (!rc) rc = lens_grid(L, ray_grid, &g);
    if (rc) { delete r; return rc; }
    r->samples = g.samples;
    r->grid_n = g.n;
    r->tiles = (g.n + kTile - 1) / kTile;
    const long long items = (long long)L->n_pairs * n_sources * r->tiles;
    if (items > (1LL << 31) - 1) { delete r; return fail(GL_ERR_INVALID, "request_create: too many work items"); }
    r->n_items = (int)items;
    r->rays = (long long)L->n_pairs * n_sources * g.n * n_spec;
    const int probe_total = L->probe_begin[3];
    r->cull = prm->cull_dead_pairs && L->n_pairs > 1 && n_spec != 3 && g.n > probe_total;
    if (r->cull) r->probe_rays = (long long)L->n_pairs * n_sources * probe_total * n_spec;
    r->h_spec.resize((size_t)n_spec);
    for (int i = 0; i < n_spec; ++i)
        r->h_spec[i] = make_float4(spec[i].lambda, spec[i].cmf_r, spec[i].cmf_g, spec[i].cmf_b);
    r->h_src.resize((size_t)std::max(1, n_sources));
    for (int i = 0; i < n_sources; ++i) r->h_src[i] = make_source(sources[i]);
    // one block: accumulator | r g b planes | spectral table | sources | counters + traced | pair hits
    const size_t n_px = (size_t)r->width * r->height;
    const size_t o_planes = align256(n_px * sizeof(float4));
    const size_t o_spec = o_planes + align256(3 * n_px * sizeof(float));
    const size_t o_src = o_spec + align256((size_t)n_spec * sizeof(float4));
    const size_t o_cnt = o_src + align256(r->h_src.size() * sizeof(SourceDev));
    const size_t o_hits = o_cnt + 256;
    r->bytes = o_hits + align256((size_t)std::max(1, L->n_pairs) * sizeof(int));
    r->smem = render_smem(L->n_surf, n_spec);
    cudaStream_t st = (cudaStream_t)stream;
    cudaMemPool_t pool;
    cudaError_t e = device_pool(L->device, &pool);
    if (e == cudaSuccess) e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&r->block), r->bytes, pool, st);
    if (e != cudaSuccess)
    {
        delete r;
        return fail(e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA, std::string("request_create: ") + cudaGetErrorString(e));
    }
    r->accum = reinterpret_cast<float4*>(r->block);
    r->planes = reinterpret_cast<float*>(r->block + o_planes);
    r->spec = reinterpret_cast<float4*>(r->block + o_spec);
    r->sources = reinterpret_cast<SourceDev*>(r->block + o_src);
    r->counters = reinterpret_cast<int*>(r->block + o_cnt);
    r->traced = reinterpret_cast<unsigned long long*>(r->block + o_cnt + 64);
    r->pair_hits = reinterpret_cast<int*>(r->block + o_hits);
    e = cudaMemcpyAsync(r->spec, r->h_spec.data(), r->h_spec.size() * sizeof(float4), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(r->sources, r->h_src.data(), r->h_src.size() * sizeof(SourceDev), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
    {
        int per_sm = 0, n_sm = 0;
        e = render_prepare(r->smem, &per_sm, &n_sm);
    }
    if (e != cudaSuccess)
    {
        cudaFreeAsync(r->block, st);
        delete r;
        return fail(GL_ERR_CUDA, std::string("request_create: ") + cudaGetErrorString(e));
    }
    *out = new gl_request{r};
    return GL_OK;
}

int gl_request_set_lambda_split(gl_request* req, int chunks)
{
    if (!req) return fail(GL_ERR_INVALID, "request_set_lambda_split: null request");
    if (chunks < 1) return fail(GL_ERR_INVALID, "request_set_lambda_split: chunks must be >= 1");
    req->p->l_chunks = std::min(chunks, std::max(1, req->p->n_spec));
    return GL_OK;
}

int gl_request_enqueue(gl_request* req, float* d_out_r, float* d_out_g, float* d_out_b, int items_per_warp,
                       void* stream)
{
    if (!req) return fail(GL_ERR_INVALID, "request_enqueue: null request");
    if ((d_out_r == nullptr) != (d_out_g == nullptr) || (d_out_r == nullptr) != (d_out_b == nullptr))
        return fail(GL_ERR_INVALID, "request_enqueue: give all three output planes or none");
    if (items_per_warp < 0) return fail(GL_ERR_INVALID, "request_enqueue: items_per_warp must be >= 0");
    Request* r = req->p;
    if (!d_out_r)
    {
        const size_t npx = (size_t)r->width * r->height;
        d_out_r = r->planes; d_out_g = r->planes + npx; d_out_b = r->planes + 2 * npx;
    }
    ResidentLens* L = r->lens;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n_px = (size_t)r->width * r->height;
    int launches = 0;
    GL_CUDA_TRY(cudaMemsetAsync(r->accum, 0, n_px * sizeof(float4), st));
    GL_CUDA_TRY(cudaMemsetAsync(r->counters, 0, 128, st));
    int per_sm = 0, n_sm = 0;
    GL_CUDA_TRY(render_prepare(r->smem, &per_sm, &n_sm));
    const int slots = std::max(1, per_sm) * n_sm;
    const int wpb = kRenderThreads / 32;
    // CTAs are sized by tasks (items x wavelength ranges): each CTA's warps
    // take items_per_warp tasks, so a split request runs more, shorter CTAs
    const long long chunks = std::max(1, r->l_chunks);
    auto grid_for = [&](int n_items) {
        const long long n_tasks = (long long)n_items * chunks;
        if (items_per_warp == 0) return (int)std::max(1LL, std::min((n_tasks + wpb - 1) / wpb, (long long)slots));
        const long long per_cta = (long long)wpb * items_per_warp;
        return (int)std::max(1LL, (n_tasks + per_cta - 1) / per_cta);
    };
    RenderArgs A{};
    A.recs = L->recs; A.ior_at = r->ior.at; A.ior_bf = r->ior.bf; A.spec = r->spec;
    A.items = nullptr; A.pairs = L->pairs; A.sources = r->sources; A.samples = r->samples;
    A.accum = r->accum; A.traced = r->traced; A.pair_hits = nullptr;
    A.n_surf = L->n_surf; A.n_spec = r->n_spec; A.n_items = r->n_items; A.item_base = 0;
    A.l_chunks = (int)chunks;
    A.width = r->width; A.height = r->height;
    A.fmt_w = (float)r->prm.fmt_w; A.fmt_h = (float)r->prm.fmt_h;
    A.fmt_x0 = (float)r->prm.fmt_x0; A.fmt_y0 = (float)r->prm.fmt_y0;
    A.hw2 = 2.0f * r->prm.sensor_half_w; A.hh2 = 2.0f * r->prm.sensor_half_h;
    A.gain = r->prm.flare_gain; A.front_R = L->front_R; A.start_z = L->start_z;
    A.u_tiles = r->tiles; A.u_n_src = r->n_src; A.u_grid_base = 0; A.u_grid_n = r->grid_n;
    A.w_uniform = r->grid_n > 0 ? 1.0f / (float)r->grid_n : 0.0f;
    if (r->n_items > 0 && r->cull)
    {
        // off-sensor probe passes over the frame inflated by 1.25 (ghost_render.cu:148)
        GL_CUDA_TRY(cudaMemsetAsync(r->pair_hits, 0, sizeof(int) * std::max(1, L->n_pairs), st));
        RenderArgs B = A;
        B.samples = L->probe;
        B.pair_hits = r->pair_hits;
        B.hw2 = 2.0f * (r->prm.sensor_half_w * 1.25f);
        B.hh2 = 2.0f * (r->prm.sensor_half_h * 1.25f);
        // the three passes as one launch over consecutive item ranges, in pass
        // order: an item whose pair already has a hit is skipped, so a later
        // pass re-probes only the pairs still without one
        int start = 0;
        B.u_npass = 3;
        for (int pass = 0; pass < 3; ++pass)
        {
            const int cnt = L->probe_begin[pass + 1] - L->probe_begin[pass];
            B.u_start[pass] = start;
            B.u_base[pass] = L->probe_begin[pass];
            B.u_n[pass] = cnt;
            B.u_tl[pass] = (cnt + kTile - 1) / kTile;
            start += L->n_pairs * r->n_src * B.u_tl[pass];
        }
        B.u_start[3] = start;
        B.n_items = start;
        B.counter = items_per_warp == 0 ? r->counters : nullptr;
        if (start > 0)
        {
            GL_CUDA_TRY(render_launch(B, true, grid_for(B.n_items), r->smem, st));
            ++launches;
        }
        A.pair_hits = r->pair_hits;
    }
    if (r->n_items > 0)
    {
        A.counter = items_per_warp == 0 ? r->counters + 3 : nullptr;
        GL_CUDA_TRY(render_launch(A, false, grid_for(r->n_items), r->smem, st));
        ++launches;
    }
    GL_CUDA_TRY(flush_launch(r->accum, n_px, d_out_r, d_out_g, d_out_b, r->prm.apply_correction, r->prm.correction, st));
    ++launches;
    if (!r->traced_host) r->traced_host = traced_slot();
    if (r->traced_host)
        GL_CUDA_TRY(cudaMemcpyAsync(r->traced_host, r->traced, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    g_last_launches = launches;
    return GL_OK;
}

int gl_request_planes(const gl_request* req, float** d_rgb)
{
    if (!req || !d_rgb) return fail(GL_ERR_INVALID, "request_planes: bad arguments");
    *d_rgb = req->p->planes;
    return GL_OK;
}

int gl_request_copy_out(const gl_request* req, void* host_rgb, void* stream)
{
    // host (pinned or pageable) or device destination: unified addressing picks the direction
    if (!req || !host_rgb) return fail(GL_ERR_INVALID, "request_copy_out: bad arguments");
    const size_t n = 3 * (size_t)req->p->width * req->p->height * sizeof(float);
    GL_CUDA_TRY(cudaMemcpyAsync(host_rgb, req->p->planes, n, cudaMemcpyDefault, (cudaStream_t)stream));
    return GL_OK;
}

int gl_request_info(const gl_request* req, long long* rays, long long* device_bytes, int* grid_samples)
{
    if (!req) return fail(GL_ERR_INVALID, "request_info: null request");
    if (rays) *rays = req->p->rays + req->p->probe_rays;
    if (device_bytes) *device_bytes = (long long)req->p->bytes;
    if (grid_samples) *grid_samples = req->p->grid_n;
    return GL_OK;
}

int gl_request_traced(const gl_request* req, long long* out, void* stream)
{
    if (!req || !out) return fail(GL_ERR_INVALID, "request_traced: bad arguments");
    if (req->p->traced_host && stream == nullptr)
    {
        // the caller has seen the request's work complete (event / stream sync)
        *out = (long long)*(volatile unsigned long long*)req->p->traced_host;
        return GL_OK;
    }
    unsigned long long v = 0;
    cudaStream_t st = (cudaStream_t)stream;
    GL_CUDA_TRY(cudaMemcpyAsync(&v, req->p->traced, sizeof(v), cudaMemcpyDeviceToHost, st));
    GL_CUDA_TRY(cudaStreamSynchronize(st));
    *out = (long long)v;
    return GL_OK;
}

int gl_request_destroy(gl_request* req, void* stream)
{
    if (!req) return GL_OK;
    if (req->p->block) cudaFreeAsync(req->p->block, (cudaStream_t)stream);
    delete req->p;
    delete req;
    return GL_OK;
}

int gl_pool_info(long long* reserved, long long* used)
{
    int dev = 0;
    GL_CUDA_TRY(cudaGetDevice(&dev));
    cudaMemPool_t pool;
    GL_CUDA_TRY(device_pool(dev, &pool));
    uint64_t a = 0, b = 0;
    GL_CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &a));
    GL_CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &b));
    if (reserved) *reserved = (long long)a;
    if (used) *used = (long long)b;
    return GL_OK;
}

int gl_pool_trim(long long keep_bytes)
{
    int dev = 0;
    GL_CUDA_TRY(cudaGetDevice(&dev));
    cudaMemPool_t pool;
    GL_CUDA_TRY(device_pool(dev, &pool));
    GL_CUDA_TRY(cudaMemPoolTrimTo(pool, (size_t)std::max(0LL, keep_bytes)));
    return GL_OK;
}

}  // extern "C"
