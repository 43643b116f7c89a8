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
#include "gl_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

namespace gl {

constexpr int kRenderThreads = 256;
constexpr int kTile = kRenderThreads;
constexpr int kMaxSpec = 256;

struct PairDev {
    int a, b;
    float boost, w_ray;
};

struct SourceDev {
    float dx, dy, dz, sdx;
    float sdy, r, g, b;
};

struct RenderArgs {
    const SurfRec* recs;
    const float* ior_at;
    const float* ior_bf;
    const float4* spec;
    const int4* items;        // (pair, source, sample_start, sample_count)
    const PairDev* pairs;
    const SourceDev* sources;
    const float2* samples;
    int* counter;             // persistent queue head; null = one item per CTA
    float4* accum;            // RGBA, width x height
    int n_surf, n_spec, n_items, item_base;
    int width, height;
    float fmt_w, fmt_h, fmt_x0, fmt_y0;
    float hw2, hh2, gain, front_R, start_z;
};

__device__ __forceinline__ void flush_taps(float4* accum, int W, int H, int cx, int cy,
                                           const float (&acc)[4][3])
{
    #pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        const int xi = cx + (k & 1), yi = cy + (k >> 1);
        if (xi < 0 || xi >= W || yi < 0 || yi >= H) continue;
        if (acc[k][0] == 0.0f && acc[k][1] == 0.0f && acc[k][2] == 0.0f) continue;
        atomicAdd(accum + ((size_t)yi * W + xi), make_float4(acc[k][0], acc[k][1], acc[k][2], 0.0f));
    }
}

__device__ __forceinline__ void trace_sample(const RenderArgs& A, const SurfRec* lens, const float* at,
                                             const float* bf, const float4* spec, const PairDev& P,
                                             const SourceDev& S, float2 uv)
{
    const V3 o = v3(uv.x * A.front_R + S.sdx, uv.y * A.front_R + S.sdy, A.start_z);
    const V3 d = v3(S.dx, S.dy, S.dz);
    int cx = INT_MIN, cy = INT_MIN;
    float acc[4][3];
    #pragma unroll
    for (int k = 0; k < 4; ++k) acc[k][0] = acc[k][1] = acc[k][2] = 0.0f;

    for (int li = 0; li < A.n_spec; ++li)
    {
        const float4 sp = spec[li];
        TraceOut r = trace_ghost(lens, A.n_surf, at + li * A.n_surf, bf + li * A.n_surf, o, d, sp.x, P.a, P.b);
        if (r.status != 0) continue;
        if (!isfinite(r.x) || !isfinite(r.y)) continue;
        const float base = r.w * P.w_ray * A.gain * P.boost;
        if (base < 1e-14f) continue;
        float px = (r.x / A.hw2 + 0.5f) * A.fmt_w + A.fmt_x0;
        float py = (r.y / A.hh2 + 0.5f) * A.fmt_h + A.fmt_y0;
        if (!isfinite(px) || !isfinite(py)) continue;
        px = fmaxf(-2.0e9f, fminf(2.0e9f, px));
        py = fmaxf(-2.0e9f, fminf(2.0e9f, py));
        const int x0 = (int)floorf(px - 0.5f), y0 = (int)floorf(py - 0.5f);
        const float fx = (px - 0.5f) - (float)x0, fy = (py - 0.5f) - (float)y0;
        const float P_l = S.r * sp.y + S.g * sp.z + S.b * sp.w;
        const float power = P_l * base;
        const float c0 = power * sp.y, c1 = power * sp.z, c2 = power * sp.w;
        if (x0 != cx || y0 != cy)
        {
            if (cx != INT_MIN) flush_taps(A.accum, A.width, A.height, cx, cy, acc);
            cx = x0; cy = y0;
            #pragma unroll
            for (int k = 0; k < 4; ++k) acc[k][0] = acc[k][1] = acc[k][2] = 0.0f;
        }
        const float w[4] = {(1.0f - fx) * (1.0f - fy), fx * (1.0f - fy), (1.0f - fx) * fy, fx * fy};
        #pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            acc[k][0] += c0 * w[k];
            acc[k][1] += c1 * w[k];
            acc[k][2] += c2 * w[k];
        }
    }
    if (cx != INT_MIN) flush_taps(A.accum, A.width, A.height, cx, cy, acc);
}

__global__ void __launch_bounds__(kRenderThreads, 2) ghost_render_kernel(const RenderArgs A)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    SurfRec* lens = reinterpret_cast<SurfRec*>(smem_raw);
    float4* spec = reinterpret_cast<float4*>(lens + A.n_surf);
    float* at = reinterpret_cast<float*>(spec + A.n_spec);
    float* bf = at + A.n_spec * A.n_surf;
    const int tid = threadIdx.x;
    {
        const int words = A.n_surf * (int)(sizeof(SurfRec) / 4);
        const int* src = reinterpret_cast<const int*>(A.recs);
        int* dst = reinterpret_cast<int*>(lens);
        for (int i = tid; i < words; i += blockDim.x) dst[i] = src[i];
        for (int i = tid; i < A.n_spec; i += blockDim.x) spec[i] = A.spec[i];
        const int nt = A.n_spec * A.n_surf;
        for (int i = tid; i < nt; i += blockDim.x) { at[i] = A.ior_at[i]; bf[i] = A.ior_bf[i]; }
    }
    __syncthreads();
    for (;;)
    {
        int item;
        if (A.counter != nullptr)
        {
            if (tid == 0) s_item = atomicAdd(A.counter, 1);
            __syncthreads();
            item = s_item;
            __syncthreads();
        }
        else
        {
            item = A.item_base + (int)blockIdx.x;
        }
        if (item >= A.n_items) break;
        const int4 w = A.items[item];
        if (tid < w.w)
        {
            const PairDev P = A.pairs[w.x];
            const SourceDev S = A.sources[w.y];
            trace_sample(A, lens, at, bf, spec, P, S, A.samples[w.z + tid]);
        }
        if (A.counter == nullptr) break;
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
    long long rays = 0;                 // ray-wavelength traces per execute
    float front_R = 0.0f, start_z = 0.0f;
};

static void plan_free(GhostPlan* p)
{
    if (!p) return;
    cudaFree(p->recs); cudaFree(p->ior_at); cudaFree(p->ior_bf); cudaFree(p->spec);
    cudaFree(p->items); cudaFree(p->pairs); cudaFree(p->sources); cudaFree(p->samples);
    cudaFree(p->counter); cudaFree(p->accum);
    delete p;
}

template <class T>
static cudaError_t upload(T** dst, const T* src, size_t count)
{
    cudaError_t e = cudaMalloc(dst, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return e;
    if (count) e = cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}

static size_t render_smem(int n_surf, int n_spec)
{
    return (size_t)n_surf * sizeof(SurfRec) + (size_t)n_spec * 16 + 2 * (size_t)n_spec * n_surf * 4;
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

    std::vector<SurfRec> recs((size_t)n_surf);
    int rc = pack_lens(surfaces, n_surf, recs.data());
    if (rc) return rc;

    GhostPlan* p = new GhostPlan();
    cudaGetDevice(&p->device);
    p->n_surf = n_surf; p->n_spec = n_spec; p->n_pairs = n_pairs;
    p->front_R = surfaces[0].semi_aperture;              // ghost_render.cu:738-739
    p->start_z = surfaces[0].z - kSpawnOffset;
    p->width = prm->width; p->height = prm->height; p->prm = *prm;

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
    for (int i = 0; i < n_src; ++i)
    {
        const float bx = tanf(sources[i].angle_x), by = tanf(sources[i].angle_y);
        V3 dir = normalized(v3(bx, by, 1.0f));
        src[i] = {dir.x, dir.y, dir.z, -kSpawnOffset * bx, -kSpawnOffset * by, sources[i].r, sources[i].g, sources[i].b};
    }

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
    const int n_samples = n_grids > 0 ? grid_offsets[n_grids] : 0;

    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    chk(upload(&p->recs, recs.data(), recs.size()));
    chk(upload(&p->ior_at, at.data(), at.size()));
    chk(upload(&p->ior_bf, bf.data(), bf.size()));
    chk(upload(&p->spec, sp.data(), sp.size()));
    chk(upload(&p->items, items.data(), items.size()));
    chk(upload(&p->pairs, pd.data(), pd.size()));
    chk(upload(&p->sources, src.data(), src.size()));
    chk(upload(&p->samples, reinterpret_cast<const float2*>(samples), (size_t)n_samples));
    chk(cudaMalloc(&p->counter, sizeof(int)));
    chk(cudaMalloc(&p->accum, (size_t)prm->width * prm->height * sizeof(float4)));
    if (e == cudaSuccess) chk(cudaMemset(p->accum, 0, (size_t)prm->width * prm->height * sizeof(float4)));
    p->smem = render_smem(n_surf, n_spec);
    if (e == cudaSuccess) chk(cudaFuncSetAttribute(ghost_render_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem));
    int per_sm = 0, n_sm = 0;
    if (e == cudaSuccess) chk(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ghost_render_kernel, kRenderThreads, p->smem));
    if (e == cudaSuccess) chk(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, p->device));
    if (e != cudaSuccess)
    {
        plan_free(p);
        return fail(e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA,
                    std::string("render_ghosts: ") + cudaGetErrorString(e));
    }
    p->grid_persistent = std::max(1, std::min(p->n_items, std::max(1, per_sm) * n_sm));
    *out = p;
    return GL_OK;
}

int plan_execute(GhostPlan* p, float* d_out_r, float* d_out_g, float* d_out_b, cudaStream_t st)
{
    if (!p || !d_out_r || !d_out_g || !d_out_b) return fail(GL_ERR_INVALID, "render_ghosts: null output");
    const size_t n_px = (size_t)p->width * p->height;
    int launches = 0;
    GL_CUDA_TRY(cudaMemsetAsync(p->accum, 0, n_px * sizeof(float4), st));
    RenderArgs A;
    A.recs = p->recs; A.ior_at = p->ior_at; A.ior_bf = p->ior_bf; A.spec = p->spec;
    A.items = p->items; A.pairs = p->pairs; A.sources = p->sources; A.samples = p->samples;
    A.counter = nullptr; A.accum = p->accum;
    A.n_surf = p->n_surf; A.n_spec = p->n_spec; A.n_items = p->n_items; A.item_base = 0;
    A.width = p->width; A.height = p->height;
    A.fmt_w = (float)p->prm.fmt_w; A.fmt_h = (float)p->prm.fmt_h;
    A.fmt_x0 = (float)p->prm.fmt_x0; A.fmt_y0 = (float)p->prm.fmt_y0;
    A.hw2 = 2.0f * p->prm.sensor_half_w; A.hh2 = 2.0f * p->prm.sensor_half_h;
    A.gain = p->prm.flare_gain;
    A.front_R = p->front_R; A.start_z = p->start_z;
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
                ghost_render_kernel<<<b1 - b0, kRenderThreads, p->smem, st>>>(A);
                ++launches;
            }
            GL_CUDA_TRY(cudaGetLastError());
        }
        else
        {
            GL_CUDA_TRY(cudaMemsetAsync(p->counter, 0, sizeof(int), st));
            A.counter = p->counter;
            ghost_render_kernel<<<p->grid_persistent, kRenderThreads, p->smem, st>>>(A);
            GL_CUDA_TRY(cudaGetLastError());
            ++launches;
        }
    }
    const float* C = p->prm.correction;
    const size_t quads = (n_px + 3) / 4;
    const int fb = 256;
    ghost_flush_kernel<<<(unsigned)((quads + fb - 1) / fb), fb, 0, st>>>(
        p->accum, n_px, d_out_r, d_out_g, d_out_b, p->prm.apply_correction,
        C[0], C[1], C[2], C[3], C[4], C[5], C[6], C[7], C[8]);
    GL_CUDA_TRY(cudaGetLastError());
    ++launches;
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

int gl_ghost_plan_info(const gl_ghost_plan* plan, long long* rays, int* n_items, int* grid)
{
    if (!plan) return fail(GL_ERR_INVALID, "ghost_plan_info: null plan");
    if (rays) *rays = plan->p->rays;
    if (n_items) *n_items = plan->p->n_items;
    if (grid) *grid = plan->p->grid_persistent;
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
    std::vector<SurfRec> recs((size_t)n);
    int rc = pack_lens(surfaces, n, recs.data());
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
