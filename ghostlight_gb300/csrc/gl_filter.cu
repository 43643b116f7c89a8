// gl_filter.cu — ghost-pair enumerator and energy culler on the device.
//
// Replaces filter_ghost_pairs (ghostlight/src/ghost.cpp:105-138).  One block
// per enumerated pair traces the reference's probes — three axial rays at
// 650/550/450 nm for the intensity estimate (ghost.cpp:34-50) and the 8x8
// green probe for the area boost (ghost.cpp:53-102) — in one launch instead of
// 67 host traces per pair.
//
// This translation unit is compiled IEEE-exact (-fmad=false, IEEE division
// and square root, no flush-to-zero), so its float arithmetic equals the
// reference host build's except inside cosf / atan2f / fmodf / sinf, which may
// differ in the last place.  Two guards make the results the reference's:
//  * a keep/drop decision whose estimate lies within a guard band of the
//    threshold is re-evaluated on the host with the identical code compiled
//    by the host compiler;
//  * the only libm-dependent tests of a probe ray are the silhouettes of
//    polygon and curved-blade apertures (atan2f, fmodf, cosf, sinf), so on a
//    lens that has one the probes also run with every such clear radius
//    scaled by 1 + 1e-6 and 1 - 1e-6; a pair whose probe outcome (which rays
//    land, their weights and landing box) changes between the two has a ray
//    grazing a silhouette and is traced again on the host.
// The surviving set, its order, the area boosts and the footprints are then
// the reference's bit for bit.
#include "gl_internal.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

namespace gl {

namespace {

constexpr int kProbeThreads = 96;   // 3 intensity rays + 64 spread probes, padded

using ProbeOut = FilterProbe;
constexpr float kGraze = 1e-6f;     // relative clear-radius perturbation of the graze test

bool has_silhouette(const gl_surface* s, int n)
{
    for (int i = 0; i < n; ++i)
        if (s[i].aperture_shape == GL_APERTURE_POLYGON && s[i].aperture_blades >= 3) return true;
    return false;
}

bool same_probe(const ProbeOut& x, const ProbeOut& y)
{
    return std::memcmp(&x, &y, sizeof(ProbeOut)) == 0;
}

// One out-of-line copy of the trace for both kinds of probe ray: the IEEE
// general step is large, and the launch is one wave whose time is one
// divergent trace, so a single copy keeps its code in the instruction cache.
__device__ __noinline__ TraceOut probe_trace(const SurfRec* lens, int n, const float* at, const float* bf, V3 o,
                                              float lam, int a, int b)
{
    return trace_ghost(lens, n, at, bf, o, v3(0.0f, 0.0f, 1.0f), lam, a, b);
}

__global__ void __launch_bounds__(kProbeThreads)
filter_probe_kernel(const SurfRec* __restrict__ recs, int n, const float* __restrict__ ior_at3,
                    const float* __restrict__ ior_bf3, const int2* __restrict__ pairs,
                    float front_R, float start_z, ProbeOut* __restrict__ out)
{
    // blockIdx.y: the record variant (exact, then the widened and narrowed
    // silhouettes of the graze test)
    recs += (size_t)blockIdx.y * n;
    out += (size_t)blockIdx.y * gridDim.x;
    __shared__ SurfRec lens[kMaxSurfaces];
    __shared__ float at[3 * kMaxSurfaces], bf[3 * kMaxSurfaces];
    __shared__ float px[64], py[64];
    __shared__ int ok[64];
    const int tid = threadIdx.x;
    {
        const int words = n * (int)(sizeof(SurfRec) / 4);
        const int* src = reinterpret_cast<const int*>(recs);
        int* dst = reinterpret_cast<int*>(lens);
        for (int i = tid; i < words; i += blockDim.x) dst[i] = src[i];
        for (int i = tid; i < 3 * n; i += blockDim.x) { at[i] = ior_at3[i]; bf[i] = ior_bf3[i]; }
    }
    __syncthreads();
    const int2 p = pairs[blockIdx.x];
    const float lams[3] = {650.0f, 550.0f, 450.0f};
    ProbeOut* o = out + blockIdx.x;
    if (tid < 3)
    {
        TraceOut r = probe_trace(lens, n, at + tid * n, bf + tid * n, v3(0.0f, 0.0f, start_z), lams[tid], p.x, p.y);
        o->w[tid] = r.w;
        o->wok[tid] = (r.status == 0);
    }
    else if (tid < 67)
    {
        const int k = tid - 3, gx = k % 8, gy = k / 8;
        const float u = ((gx + 0.5f) / 8) * 2.0f - 1.0f;
        const float v = ((gy + 0.5f) / 8) * 2.0f - 1.0f;
        int good = 0;
        if (!(u * u + v * v > 1.0f))
        {
            TraceOut r = probe_trace(lens, n, at + n, bf + n, v3(u * front_R, v * front_R, start_z), 550.0f, p.x, p.y);
            if (r.status == 0) { px[k] = r.x; py[k] = r.y; good = 1; }
        }
        ok[k] = good;
    }
    __syncthreads();
    if (tid == 0)
    {
        float mnx = 1e30f, mxx = -1e30f, mny = 1e30f, mxy = -1e30f;
        int valid = 0;
        for (int k = 0; k < 64; ++k)
        {
            if (!ok[k]) continue;
            mnx = fminf(mnx, px[k]); mxx = fmaxf(mxx, px[k]);
            mny = fminf(mny, py[k]); mxy = fmaxf(mxy, py[k]);
            ++valid;
        }
        o->mnx = mnx; o->mxx = mxx; o->mny = mny; o->mxy = mxy; o->valid = valid;
    }
}

}  // namespace
}  // namespace gl

using namespace gl;

// Device scratch of the filter, kept per device and grown on demand (never
// shrunk): a per-call cudaMalloc/cudaFree pair would cost a device-wide
// synchronisation each call, stalling whatever other streams have in flight
// (the reference keeps its ghost buffers in a leaked cache for the same
// reason, ghost_render.cu:505-510).  The mutex serialises callers; each call
// finishes its copies before it returns.
namespace {
std::mutex g_scratch_mu;
struct Scratch { void* ptr = nullptr; size_t bytes = 0; };
Scratch g_scratch[64];

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
}  // namespace

extern "C" int gl_filter_ghost_pairs(const gl_surface* surfaces, int n, float hw, float hh,
                                     const gl_filter_params* prm, gl_ghost_pair* out_pairs,
                                     float* out_boosts, float* out_fp, int cap, int* n_out,
                                     int* n_rechecked)
{
    if (!surfaces || n <= 0 || !prm || !n_out) return fail(GL_ERR_INVALID, "filter_ghost_pairs: bad arguments");
    std::vector<SurfRec> recs((size_t)n);
    int rc = pack_lens(surfaces, n, recs.data(), kTablesHost);     // the host re-check's records
    if (rc) return rc;

    // Enumerate (ghost.cpp:17-31) and apply the IOR-contrast test
    // (ghost.cpp:118-125) — exact float comparisons, done here.
    std::vector<int2> cand;
    for (int a = 0; a < n; ++a)
    {
        if (!surfaces[a].is_active) continue;
        for (int b = a + 1; b < n; ++b)
        {
            if (!surfaces[b].is_active) continue;
            float iba = ior_before_nd(surfaces, a), iaa = surfaces[a].ior;
            float ibb = ior_before_nd(surfaces, b), iab = surfaces[b].ior;
            if (std::abs(iba - iaa) < 0.001f || std::abs(ibb - iab) < 0.001f) continue;
            cand.push_back(make_int2(a, b));
        }
    }
    int rechecked = 0;
    int kept = 0;
    if (!cand.empty())
    {
        const float lams[3] = {650.0f, 550.0f, 450.0f};
        std::vector<float> at(3 * (size_t)n), bf(3 * (size_t)n);
        build_ior_tables(surfaces, n, lams, 3, at.data(), bf.data());
        const int np = (int)cand.size();
        const int nv = has_silhouette(surfaces, n) ? 3 : 1;         // record variants of the graze test
        std::vector<ProbeOut> res((size_t)np * nv);
        cudaError_t e = cudaSuccess;
        auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
        const size_t o_at = align256(sizeof(SurfRec) * n * nv), o_bf = o_at + align256(sizeof(float) * 3 * n);
        const size_t o_pairs = o_bf + align256(sizeof(float) * 3 * n);
        const size_t o_out = o_pairs + align256(sizeof(int2) * np);
        const size_t need = o_out + align256(sizeof(ProbeOut) * np * nv);
        int dev = 0;
        chk(cudaGetDevice(&dev));
        if (e == cudaSuccess && (dev < 0 || dev >= 64)) e = cudaErrorInvalidDevice;
        std::vector<SurfRec> drecs((size_t)n * nv);                 // the device probes' records
        if (e == cudaSuccess)
        {
            rc = pack_lens(surfaces, n, drecs.data(), dev);
            if (rc) return rc;
            for (int v = 1; v < nv; ++v)
            {
                std::vector<gl_surface> moved(surfaces, surfaces + n);
                const float f = v == 1 ? 1.0f + kGraze : 1.0f - kGraze;
                for (gl_surface& g : moved)
                    if (g.aperture_shape == GL_APERTURE_POLYGON && g.aperture_blades >= 3) g.semi_aperture *= f;
                rc = pack_lens(moved.data(), n, drecs.data() + (size_t)v * n, dev);
                if (rc) return rc;
            }
        }
        std::unique_lock<std::mutex> lock(g_scratch_mu);
        Scratch& sc = g_scratch[e == cudaSuccess ? dev : 0];
        if (e == cudaSuccess && sc.bytes < need)
        {
            if (sc.ptr) cudaFree(sc.ptr);
            sc.ptr = nullptr;
            sc.bytes = 0;
            chk(cudaMalloc(&sc.ptr, need));
            if (e == cudaSuccess) sc.bytes = need;
        }
        char* base = static_cast<char*>(sc.ptr);
        SurfRec* d_recs = reinterpret_cast<SurfRec*>(base);
        float* d_at = reinterpret_cast<float*>(base + o_at);
        float* d_bf = reinterpret_cast<float*>(base + o_bf);
        int2* d_pairs = reinterpret_cast<int2*>(base + o_pairs);
        ProbeOut* d_out = reinterpret_cast<ProbeOut*>(base + o_out);
        if (e == cudaSuccess)
        {
            chk(cudaMemcpy(d_recs, drecs.data(), sizeof(SurfRec) * n * nv, cudaMemcpyHostToDevice));
            chk(cudaMemcpy(d_at, at.data(), sizeof(float) * 3 * n, cudaMemcpyHostToDevice));
            chk(cudaMemcpy(d_bf, bf.data(), sizeof(float) * 3 * n, cudaMemcpyHostToDevice));
            chk(cudaMemcpy(d_pairs, cand.data(), sizeof(int2) * np, cudaMemcpyHostToDevice));
        }
        if (e == cudaSuccess)
        {
            const float front_R = surfaces[0].semi_aperture;
            const float start_z = surfaces[0].z - kSpawnOffset;
            filter_probe_kernel<<<dim3(np, nv), kProbeThreads>>>(d_recs, n, d_at, d_bf, d_pairs, front_R, start_z,
                                                                  d_out);
            chk(cudaGetLastError());
            chk(cudaMemcpy(res.data(), d_out, sizeof(ProbeOut) * np * nv, cudaMemcpyDeviceToHost));
        }
        lock.unlock();
        if (e != cudaSuccess)
            return fail(e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA,
                        std::string("filter_ghost_pairs: ") + cudaGetErrorString(e));
        g_last_launches = 1;

        const float thr = prm->min_ghost_intensity;
        for (int i = 0; i < np; ++i)
        {
            ProbeOut r = res[i];
            if (nv == 3 && !(same_probe(res[(size_t)np + i], res[(size_t)2 * np + i]) &&
                             same_probe(res[i], res[(size_t)np + i])))
            {
                // a probe ray grazes a polygon / blade silhouette: trace the
                // pair's probes again on the host
                host_filter_probe(surfaces, recs.data(), n, cand[i].x, cand[i].y, &r);
                ++rechecked;
            }
            // estimate_ghost_intensity's sum order: total += w650, w550, w450
            float total = 0.0f;
            for (int ch = 0; ch < 3; ++ch)
                if (r.wok[ch]) total += r.w[ch];
            float est = total / 3.0f;
            const float band = 1e-4f * std::fabs(thr);
            if (!(std::fabs(est - thr) > band))
            {
                est = host_intensity_estimate(surfaces, recs.data(), n, cand[i].x, cand[i].y);
                ++rechecked;
            }
            if (est < thr) continue;
            float boost = 1.0f;
            if (prm->ghost_normalize)
            {
                if (r.valid >= 2)
                {
                    float gw = std::max(r.mxx - r.mnx, 0.01f), gh = std::max(r.mxy - r.mny, 0.01f);
                    float area = (gw * gh) / ((2.0f * hw) * (2.0f * hh));
                    boost = (area < 1.0f) ? 1.0f : (prm->max_area_boost < area) ? prm->max_area_boost : area;
                }
            }
            if (out_pairs && kept < cap)
            {
                out_pairs[kept] = {cand[i].x, cand[i].y};
                if (out_boosts) out_boosts[kept] = boost;
                if (out_fp)
                {
                    out_fp[2 * kept] = (r.valid >= 2) ? r.mxx - r.mnx : 0.0f;
                    out_fp[2 * kept + 1] = (r.valid >= 2) ? r.mxy - r.mny : 0.0f;
                }
            }
            ++kept;
        }
    }
    *n_out = kept;
    if (n_rechecked) *n_rechecked = rechecked;
    if (out_pairs && kept > cap) return fail(GL_ERR_INVALID, "filter_ghost_pairs: capacity too small");
    return GL_OK;
}
