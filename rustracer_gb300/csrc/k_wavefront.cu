// The gather pass as a wavefront: rustracer-renderer/shaders/gather.wgsl:258-594 split into kernels that
// each run one uniform piece of code over a compacted queue of paths.
//
//   generate   camera ray of sample 0 for every pixel (gather.wgsl:262-297); fills queue 0
//   extend     closest hit of every queued path (gather.wgsl:300)
//   shade      one loop body of gather.wgsl:299-537 per queued path: hit shading, emission, debug
//              views, dielectric / metallic-roughness lobes, the light sample of NEE
//              (gather.wgsl:152-206, its shadow ray deferred to `shadow`), photon lookup, next
//              direction, Russian roulette; a finished sample starts the pixel's next sample in the
//              same slot; continuing paths are appended to the next queue (warp ballot + one atomic)
//   shadow     occlusion of each deferred NEE ray; a visible light adds its contribution
//   finalize   sigma clamp and the frame / moments / gbuffer writes (gather.wgsl:548-593)
//
// extend and shadow run as one persistent traversal launch (`wf_trace_kernel`): the occlusion rays of
// iteration i-1 ride with the closest-hit rays of iteration i, which need only shade(i-1) too.  The
// photon pass uses the closest-hit-only form (`wf_extend_kernel`).
//
// One path slot per pixel: a pixel's samples run one after the other in its slot, with one RNG
// stream, exactly as the reference's per-pixel loop.  Every pixel receives its contributions in the
// reference's order except that a bounce's NEE term lands after that bounce's other terms; floating
// point addition order is the only difference (an ulp).  The host launches spp * max_bounces
// iterations; a path extends at most once per iteration, so that bounds every pixel's segments.
#include <cstring>

#include "rt_kernels.h"

namespace rtd {

namespace {

__device__ __forceinline__ float luma(f3 c) { return dot(c, mk3(0.2126f, 0.7152f, 0.0722f)); }

struct Accum {
    f3 col;
    float lum_sum, lum2_sum;
    float sl[8];
};
// The words of a slot's accumulator one shade step can change: every term it adds belongs to the
// sample it started with, so only that sample's luminance sum is loaded and stored with the colour
// and the two luminance moments.
struct PathAcc {
    f3 col;
    float lum_sum, lum2_sum, sl;
};
__device__ __forceinline__ void add_radiance(uint32_t s, PathAcc &a, f3 c) {
    a.col = a.col + c;
    float l = luma(c);
    a.lum_sum += l;
    a.lum2_sum += l * l;
    if (s < 8u) a.sl += l;
}
// One radiance term (or only its luminance) added straight into a slot's accumulator in memory:
// colour, the two luminance moments and the sample's luminance sum, as every path step adds them.
__device__ __forceinline__ void acc_add_term(const WaveParams &p, uint32_t slot, uint32_t s, f3 c, bool luma_only) {
    float4 *a = p.acc + 4 * (size_t)slot;
    float4 a0 = a[0];
    float *lum2 = reinterpret_cast<float *>(a + 1);
    const float l = luma(c);
    if (!luma_only) {
        a0.x = a0.x + c.x;
        a0.y = a0.y + c.y;
        a0.z = a0.z + c.z;
    }
    a0.w += l;
    a[0] = a0;
    *lum2 += l * l;
    if (s < 8u) reinterpret_cast<float *>(a + 2)[s] += l;
}
__device__ __forceinline__ Accum load_acc(const WaveParams &p, uint32_t pix) {
    const float4 a = p.acc[4 * (size_t)pix], b = p.acc[4 * (size_t)pix + 1], c = p.acc[4 * (size_t)pix + 2],
                 d = p.acc[4 * (size_t)pix + 3];
    Accum A;
    A.col = mk3(a.x, a.y, a.z);
    A.lum_sum = a.w;
    A.lum2_sum = b.x;
    A.sl[0] = c.x; A.sl[1] = c.y; A.sl[2] = c.z; A.sl[3] = c.w;
    A.sl[4] = d.x; A.sl[5] = d.y; A.sl[6] = d.z; A.sl[7] = d.w;
    return A;
}

__device__ __forceinline__ f3 sky_color(f3 dir, f3 zenith, f3 horizon, float intensity) {
    float t = clampf(dir.y * 0.5f + 0.5f, 0.0f, 1.0f);
    return mix3(horizon, zenith, sqrtf(t)) * intensity;  // pow(t, 0.5) for t in [0, 1]
}
__device__ __forceinline__ float smith_g1(float nd, float a) {
    float k = a * 0.5f;
    return nd / (nd * (1.0f - k) + k);
}
__device__ __forceinline__ f3 spec_ggx(f3 wo, f3 n, f3 wi, float a, f3 f0) {
    float ndl = dot(n, wi);
    float ndv = dot(n, wo);
    if (ndl <= 0.0f || ndv <= 0.0f) return mk3(0.0f, 0.0f, 0.0f);
    f3 h = normalize(wo + wi);
    float ndh = fmaxf(dot(n, h), 0.0f);
    float a2 = a * a;
    float dd = ndh * ndh * (a2 - 1.0f) + 1.0f;
    float D = a2 / (kPi * dd * dd);
    f3 F = fresnel_schlick(fmaxf(dot(wo, h), 0.0f), f0);
    return F * (D * smith_g1(ndl, a) * smith_g1(ndv, a) / (4.0f * ndl * ndv));
}
__device__ __forceinline__ f3 sample_spec_dir(f3 rd, f3 n, float a, Rng &rng) {
    f3 up = fabsf(n.y) < 0.999f ? mk3(0.0f, 1.0f, 0.0f) : mk3(1.0f, 0.0f, 0.0f);
    f3 bt = normalize(cross(up, n));
    f3 bb = cross(n, bt);
    f3 mrd = -rd;
    f3 v = mk3(dot(bt, mrd), dot(bb, mrd), dot(n, mrd));
    f3 vh = normalize(mk3(a * v.x, a * v.y, fmaxf(v.z, 1e-4f)));
    float l2 = vh.x * vh.x + vh.y * vh.y;
    f3 t1 = l2 > 0.0f ? mk3(-vh.y, vh.x, 0.0f) * (1.0f / sqrtf(l2)) : mk3(1.0f, 0.0f, 0.0f);
    f3 t2 = cross(vh, t1);
    float r = sqrtf(rng_f32(rng));
    float phi = 2.0f * kPi * rng_f32(rng);
    float sp, cp;
    sincos_fixed(phi, sp, cp);
    float x = r * cp;
    float y = r * sp;
    float s = 0.5f * (1.0f + vh.z);
    float yy = (1.0f - s) * sqrtf(fmaxf(0.0f, 1.0f - x * x)) + s * y;
    f3 hh = x * t1 + yy * t2 + sqrtf(fmaxf(0.0f, 1.0f - x * x - yy * yy)) * vh;
    f3 hn = normalize(hh);
    f3 m = bt * hn.x + bb * hn.y + n * hn.z;
    f3 out = reflect(rd, m);
    return dot(out, n) > 0.0f ? out : reflect(rd, n);
}

// The light sample of direct_light (gather.wgsl:152-206) up to its shadow query.  `occlude` is set
// when the sample needs the shadow ray (origin o, direction ld, max_dist); e is the unoccluded value.
struct LightSample {
    f3 e, wi, o;
    float max_dist;
    bool occlude;
};
__device__ __forceinline__ LightSample light_sample(const DevJob &job, f3 hp, f3 sn, Rng &rng) {
    const DevScene &s = job.scene;
    const uint32_t n = s.light_count;
    const f3 zero = mk3(0.0f, 0.0f, 0.0f);
    LightSample ls{zero, sn, zero, 0.0f, false};
    if (n == 0u) return ls;
    uint32_t li = f2u_sat(rng_f32(rng) * (float)n);
    li = li < n ? li : n - 1u;
    const Light l = load_light(s, li);
    const float fn = (float)n;
    if (l.kind == 0u) {
        f3 to = l.data - hp;
        float r2 = dot(to, to);
        float r = sqrtf(r2);
        f3 ld = to / r;
        ls.wi = ld;
        if (dot(sn, ld) <= 0.0f) return ls;
        f3 pl = mk3(job.ip.point_light_emission[0], job.ip.point_light_emission[1], job.ip.point_light_emission[2]);
        ls.e = l.color * l.intensity * pl * fmaxf(dot(sn, ld), 0.0f) / (r2 + 0.01f) * fn;
        ls.o = hp + sn * 0.01f;
        ls.max_dist = r - 0.001f;
        ls.occlude = true;
    } else if (l.kind == 1u) {
        f3 ld = normalize(l.data);
        float ndl = dot(sn, ld);
        ls.wi = ld;
        if (ndl <= 0.0f) return ls;
        ls.e = l.color * l.intensity * ndl * fn;
        ls.o = hp + sn * 0.01f;
        ls.max_dist = 1e30f;
        ls.occlude = true;
    } else if (l.kind == 2u) {
        TriFull tri = load_tri(s, f2u_sat(l.data.x));
        Mat mat = load_mat(s, tri.material_id);
        float u1 = rng_f32(rng);
        float u2 = rng_f32(rng);
        float su = sqrtf(u1);
        float u = 1.0f - su;
        float v = u2 * su;
        float w = 1.0f - u - v;
        f3 lp = tri.v0 * w + tri.v1 * u + tri.v2 * v;
        float uvx = tri.uv0x * w + tri.uv1x * u + tri.uv2x * v;
        float uvy = tri.uv0y * w + tri.uv1y * u + tri.uv2y * v;
        f3 le = l.color;
        if (mat.tex_emissive != RT_TEX_NONE) {
            float4 t = tex_sample(s.tex[RT_TEX_EMISSIVE], uvx, uvy, (int32_t)mat.tex_emissive);
            le = le * mk3(t.x, t.y, t.z);
        }
        le = le * mk3(job.ip.light_emission[0], job.ip.light_emission[1], job.ip.light_emission[2]);
        f3 to = lp - hp;
        float r2 = dot(to, to);
        float r = sqrtf(r2);
        f3 ld = to / r;
        ls.wi = ld;
        float ndl = dot(sn, ld);
        if (ndl <= 0.0f) return ls;
        f3 ln = triangle_normal(tri.v0, tri.v1, tri.v2);
        float ndl_l = dot(ln, -ld);
        if (ndl_l <= 0.0f) return ls;
        float area = 0.5f * len3(cross(tri.v1 - tri.v0, tri.v2 - tri.v0));
        ls.e = le * l.intensity * ndl * ndl_l * area * fn / (r2 + 0.01f);
        ls.o = hp + sn * 0.01f;
        ls.max_dist = r - 0.001f;
        ls.occlude = true;
    }
    return ls;
}

__device__ __forceinline__ int32_t clampi(int32_t x, int32_t lo, int32_t hi) { return x < lo ? lo : (x > hi ? hi : x); }

// The camera ray of the pixel's next sample (gather.wgsl:292-297).
__device__ __forceinline__ void camera_ray(const DevJob &job, uint32_t px, uint32_t py, Rng &rng, f3 &ro, f3 &rd) {
    const rt_camera_uniform &cam = job.cam;
    float jx = rng_f32(rng) - 0.5f;
    float jy = rng_f32(rng) - 0.5f;
    float ux = ((float)px + jx) * cam.inv_half_res[0] - 1.0f;
    float uy = 1.0f - ((float)py + jy) * cam.inv_half_res[1];
    ro = mk3(cam.position[0], cam.position[1], cam.position[2]);
    rd = normalize(mk3(cam.forward[0], cam.forward[1], cam.forward[2]) +
                   mk3(cam.right[0], cam.right[1], cam.right[2]) * ux + mk3(cam.up[0], cam.up[1], cam.up[2]) * uy);
}

__device__ __forceinline__ uint32_t pack_sb(uint32_t s, uint32_t b) { return (s & 0xFFFFu) | (b << 16); }

}  // namespace

// The last job whose first index (`first` of DevJob: base slot or first tile) is at or below i; jobs
// are laid out in order, so their first indices ascend.
template <typename First>
__device__ __forceinline__ uint32_t job_of(const WaveParams &p, uint32_t i, First first) {
    uint32_t lo = 0u, hi = p.n_jobs;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (first(p.jobs[mid]) <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// ------------------------------------------------------------------------------------------------
// generate: 8 x 4 pixel tiles, one per warp, so the first queue is tile-coherent.  One launch over
// every job's tiles (job j's start at its tile0).
// ------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) wf_generate_kernel(const __grid_constant__ WaveParams p, uint32_t n_tiles) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t gtile = blockIdx.x * 4u + warp;
    if (gtile >= n_tiles) return;  // whole warps: warp_append below is warp-uniform
    const uint32_t jid = job_of(p, gtile, [](const DevJob &j) { return j.tile0; });
    const DevJob &job = p.jobs[jid];
    const uint32_t W = job.ip.width, H = job.ip.height;
    const uint32_t tiles_x = (W + 7u) / 8u;
    const uint32_t tile = gtile - job.tile0;
    const uint32_t tx = tile % tiles_x, ty = tile / tiles_x;
    const uint32_t px = tx * 8u + (lane & 7u), py = ty * 4u + (lane >> 3);
    const bool active = px < W && py < H;
    uint32_t slot = 0;
    if (active) {
        const uint32_t pix = py * W + px;
        slot = job.base + pix;
        uint32_t base_seed = pix + job.ip.frame * 2654435761u;
        Rng rng = rng_init(base_seed * 1664525u + 1013904223u);
        f3 ro, rd;
        camera_ray(job, px, py, rng, ro, rd);
        p.ro[slot] = make_float4(ro.x, ro.y, ro.z, __uint_as_float(rng.state));
        p.rd[slot] = make_float4(rd.x, rd.y, rd.z, __uint_as_float(pack_sb(0u, 0u)));
        p.thr[slot] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(jid));
        const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        p.acc[4 * (size_t)slot] = z;
        p.acc[4 * (size_t)slot + 1] = make_float4(0.0f, 1e30f, 0.0f, 0.0f);
        p.acc[4 * (size_t)slot + 2] = z;
        p.acc[4 * (size_t)slot + 3] = z;
        p.nrm[slot] = make_float4(0.0f, 1.0f, 0.0f, 0.0f);
    }
    warp_append(active, slot, p.queue[0], p.counts + 0);
}

// ------------------------------------------------------------------------------------------------
// Persistent traversal warps.  A warp takes chunks of `chunk` work items with one atomic and hands
// them to its idle lanes; every lane then advances its traversal by up to `steps` records before the
// warp refills again, so lanes whose ray finished early pick up new rays instead of idling.  The
// traversal stack lives in dynamic shared memory, kStack entries per lane, lane-interleaved.
// ------------------------------------------------------------------------------------------------

struct WarpFeed {
    uint32_t next = 0, end = 0;
    bool more = true;
};

// Gives each lane with need == true the next item index (or none when the items ran out).  Every lane
// of the warp calls it; returns the lane's index or 0xFFFFFFFF.
__device__ __forceinline__ uint32_t warp_take(WarpFeed &f, bool need, uint32_t n, uint32_t *fetch, uint32_t chunk) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t mine = 0xFFFFFFFFu;
    uint32_t mask = __ballot_sync(0xFFFFFFFFu, need);
    while (mask != 0u && f.more) {
        if (f.next >= f.end) {
            uint32_t base = 0;
            if (lane == 0u) base = atomicAdd(fetch, chunk);
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base >= n) {
                f.more = false;
                break;
            }
            f.next = base;
            f.end = min(base + chunk, n);
        }
        const uint32_t avail = f.end - f.next;
        const uint32_t rank = __popc(mask & lanemask_lt());
        if (need && rank < avail) {
            mine = f.next + rank;
            need = false;
        }
        f.next += min((uint32_t)__popc(mask), avail);
        mask = __ballot_sync(0xFFFFFFFFu, need);
    }
    return mine;
}

// extend: closest hit of each queued path (any job: each lane traces its own job's scene).
template <int kStack, int kBlock, bool kWide>
__global__ void __launch_bounds__(kBlock) wf_extend_kernel(const __grid_constant__ WaveParams p, uint32_t iter,
                                                           uint32_t chunk, uint32_t steps) {
    extern __shared__ uint32_t stack_smem[];
    uint32_t *stk = stack_smem + threadIdx.x;
    WarpLeaves &wl = reinterpret_cast<WarpLeaves *>(stack_smem + kStack * kBlock)[threadIdx.x >> 5];
    const uint32_t n = p.counts[4 * iter];
    const uint32_t *q = p.queue[iter & 1u];
    uint32_t *fetch = p.counts + 4 * iter + 2;
    WarpFeed feed;
    TravState st;
    bool has = false;
    uint32_t slot = 0;
    for (;;) {
        const uint32_t item = warp_take(feed, !has, n, fetch, chunk);
        if (item != 0xFFFFFFFFu) {
            slot = q[item];
            const float4 o = p.ro[slot], d = p.rd[slot];
            const DevScene &sc = p.jobs[__float_as_uint(p.thr[slot].w)].scene;
            st = trav_begin<kWide>(sc, xyz(o), xyz(d), kInf, (uint32_t)kStack);
            has = true;
            if (sc.cnode_count == 0u) {
                p.hit[slot] = make_float2(kInf, 0.0f);
                has = false;
            } else {
                warp_leaves_set_ray(wl, st);
            }
        }
        if (!__any_sync(0xFFFFFFFFu, has)) break;
        for (uint32_t k = 0; k < steps; ++k) {
            if (kWide ? trav_step_warp4(st, has, false, stk, (uint32_t)kBlock, wl)
                      : trav_step_warp(st, has, false, stk, (uint32_t)kBlock, wl)) {
                p.hit[slot] = make_float2(st.t, __uint_as_float(trav_hit_prim(st)));
                has = false;
            }
            if (!__any_sync(0xFFFFFFFFu, has)) break;
        }
    }
}

// ------------------------------------------------------------------------------------------------
// shade: one bounce of gather.wgsl's loop body per queued path.  kPhotons / kDebug compile the photon
// lookup and the debug views in; the host picks the variant that covers every job of the launch
// (a job without photons or debug view takes the same path through either variant), so frames
// without them run a smaller kernel.
//
// Each round a block takes 128 queue entries and orders them by what the hit needs -- a miss, a
// dielectric, a Lambertian or emissive surface, a metal -- before shading, so a warp runs mostly one
// of the loop body's branches (neighbouring paths hit triangles of unrelated materials).  Only the
// order in which paths are shaded changes: each path's operations are its own, so images are the
// same bit for bit.  Surviving paths, their shadow rays and photon-lookup requests are queued in the
// paths' original order (which keeps neighbouring pixels together for the traversal).
// ------------------------------------------------------------------------------------------------
constexpr uint32_t kShadeKeys = 5;  // miss, dielectric, Lambertian / emissive, metal, no entry

// The entry's order key; for a hit also its triangle and material word, read from the hit prim
// slot's record (the traversal stores the slot: `orig` = the triangle's index, `word` = key | material
// << 2, filled at scene upload).
__device__ __forceinline__ uint32_t shade_key(const WaveParams &p, const uint32_t *q, uint32_t i, uint32_t n,
                                              uint32_t &slot, uint32_t &orig, uint32_t &word) {
    slot = 0u;
    orig = 0u;
    word = 0u;
    if (i >= n) return 4u;
    slot = q[i];
    const float2 h = p.hit[slot];
    if (h.x >= kInf) return 0u;
    const float4 *rec = p.jobs[__float_as_uint(p.thr[slot].w)].scene.tri_ord + 3ull * __float_as_uint(h.y);
    orig = __float_as_uint(__ldg(rec).w);
    word = __float_as_uint(__ldg(rec + 1).w);
    return word & 3u;
}

// kBlocks: resident blocks per SM the register allocation aims at (4: ~123 registers; 5: 96
// registers with 62 bytes of spills; 6: 80 registers, ~200 bytes of spills, the default: the extra
// warps hide the kernel's dependent loads, config-2 shade 7.04 -> 6.56 -> 6.41 ms per frame), chosen
// per launch by the tuning's shade_blocks.
template <bool kPhotons, bool kDebug, int kBlocks>
__global__ void __launch_bounds__(128, kBlocks) wf_shade_kernel(const __grid_constant__ WaveParams p, uint32_t iter) {
    __shared__ uint32_t s_count[4][kShadeKeys];  // entries per warp and key
    __shared__ uint32_t s_order[128];
    __shared__ uint8_t s_emit[128];   // by original position: 1 survives, 2 shadow ray, 4 photon lookup
    __shared__ uint32_t s_spos[128];  // by original position: shadow record index
    __shared__ uint32_t s_ppos[128];  // by original position: photon-lookup record index
    __shared__ uint32_t s_orig[128], s_word[128];  // by shading position: the hit's triangle and material word
    const uint32_t n = p.counts[4 * iter];
    const uint32_t *q = p.queue[iter & 1u];
    uint32_t *q_next = p.queue[(iter + 1u) & 1u];
    uint32_t *n_next = p.counts + 4 * (iter + 1u);
    uint32_t *n_shadow = p.counts + 4 * iter + 1u;
    uint32_t *n_photon = p.counts + 4 * iter + 3u;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (n + stride - 1u) / stride;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;

    for (uint32_t r = 0; r < rounds; ++r) {
        // The block's entries ranked by key, stable (warp-major, then lane order within a key).
        const uint32_t round_base = r * stride + blockIdx.x * blockDim.x;
        const uint32_t i_own = round_base + threadIdx.x;
        uint32_t slot_own, orig_own, word_own;
        const uint32_t key = shade_key(p, q, i_own, n, slot_own, orig_own, word_own);
        uint32_t same = 0;
#pragma unroll
        for (uint32_t k = 0; k < kShadeKeys; ++k) {
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, key == k);
            if (lane == k) s_count[warp][k] = __popc(m);
            if (key == k) same = __popc(m & lanemask_lt());
        }
        __syncthreads();
        uint32_t pos = same;
#pragma unroll
        for (uint32_t k = 0; k < kShadeKeys; ++k)
#pragma unroll
            for (uint32_t w = 0; w < 4; ++w)
                if (k < key || (k == key && w < warp)) pos += s_count[w][k];
        s_order[pos] = i_own;
        s_orig[pos] = orig_own;
        s_word[pos] = word_own;
        __syncthreads();
        const uint32_t i = s_order[threadIdx.x];
        const bool valid = i < n;
        bool keep = false;
        bool emit_shadow = false, emit_photon = false;
        f3 ph_hp = mk3(0.0f, 0.0f, 0.0f), ph_n = ph_hp, ph_td = ph_hp;
        uint32_t ph_sidx = 0;
        uint32_t slot = 0;
        f3 sh_o = mk3(0.0f, 0.0f, 0.0f), sh_d = sh_o, sh_c = sh_o;
        float sh_max = 0.0f;
        uint32_t sh_tag = 0;
        if (valid) {
            slot = q[i];
            const float4 o4 = p.ro[slot], d4 = p.rd[slot], t4 = p.thr[slot];
            const uint32_t jid = __float_as_uint(t4.w);
            const DevJob &job = p.jobs[jid];
            const DevScene &s = job.scene;
            const rt_image_params &ip = job.ip;
            const uint32_t W = ip.width;
            const uint32_t spp = job.spp;
            const uint32_t debug_view = ip._pad[0];
            const float env_intensity = s.env_intensity;
            const f3 env_color = mk3(s.env_color[0], s.env_color[1], s.env_color[2]);
            const f3 env_horizon = mk3(s.env_horizon[0], s.env_horizon[1], s.env_horizon[2]);
            const uint32_t pix = slot - job.base;
            const uint32_t px = pix % W, py = pix / W;
            const float2 h2 = p.hit[slot];
            const uint32_t hmat = s_word[threadIdx.x] >> 2;  // the hit's material, known before its triangle
            f3 ro = xyz(o4), rd = xyz(d4), thr = xyz(t4);
            Rng rng{__float_as_uint(o4.w)};
            const uint32_t sb = __float_as_uint(d4.w);
            uint32_t sidx = sb & 0xFFFFu, b = sb >> 16;
            const float hit_t = h2.x;
            const uint32_t prim = s_orig[threadIdx.x];  // the hit triangle (h2.y holds its prim slot)
            float4 *acc = p.acc + 4 * (size_t)slot;
            const uint32_t sidx0 = sidx;
            const float4 acc0 = acc[0];
            float4 acc1 = acc[1];  // .x = lum2_sum, .y = first_depth
            PathAcc A{xyz(acc0), acc0.w, acc1.x, sidx0 < 8u ? reinterpret_cast<const float *>(acc + 2)[sidx0] : 0.0f};
            bool first_hit = false;  // this step found a nearer first hit (normal and depth change)
            float4 nrm = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            bool alive = true;  // the sample continues with another segment

            if (hit_t >= kInf) {
                if (b > 0u) add_radiance(sidx, A, thr * sky_color(rd, env_color, env_horizon, env_intensity));
                alive = false;
            } else {
                const TriFull tr = load_tri(s, prim);
                Mat mat;
                if (hmat != kNoMat) mat = load_mat(s, hmat);
                else mat = load_mat(s, tr.material_id);
                const f3 hp = ro + rd * hit_t;
                const Bary bb = barycentric(tr, ro, rd, hit_t);
                const float uvx = bb.uvx, uvy = bb.uvy;
                bool done_step = false;  // a `continue` of the reference loop

                if ((mat.flags & RT_MAT_FLAG_ALPHA_CUTOUT) != 0u && mat.tex_albedo != RT_TEX_NONE &&
                    tex_sample(s.tex[RT_TEX_ALBEDO], uvx, uvy, (int32_t)mat.tex_albedo).w < 0.5f) {
                    ro = hp + rd * 0.002f;
                    done_step = true;
                }
                if (!done_step) {
                    const f3 gn = triangle_normal(tr.v0, tr.v1, tr.v2);
                    const bool ff = dot(rd, gn) < 0.0f;
                    const f3 sn_geom = smooth_normal(tr, bb, gn);
                    const f3 sn = ff ? sn_geom : -sn_geom;
                    f3 shn = sn;
                    if (mat.tex_normal != RT_TEX_NONE) {
                        float4 t = tex_sample(s.tex[RT_TEX_NORMAL], uvx, uvy, (int32_t)mat.tex_normal);
                        f3 nm = mk3(t.x, t.y, t.z) * 2.0f - mk3(1.0f, 1.0f, 1.0f);
                        f3 ft, fb;
                        tangent_frame(tr, sn, ft, fb);
                        shn = normalize(ft * nm.x + fb * nm.y + sn * nm.z);
                    }
                    if (b == 0u && hit_t < acc1.y) {
                        nrm = make_float4(sn.x, sn.y, sn.z, 0.0f);
                        first_hit = true;
                        acc1.y = hit_t;
                    }
                    f3 albedo = mat.albedo;
                    float rough = mat.roughness, metal = mat.metallic;
                    if (mat.tex_albedo != RT_TEX_NONE) {
                        float4 t = tex_sample(s.tex[RT_TEX_ALBEDO], uvx, uvy, (int32_t)mat.tex_albedo);
                        albedo = mat.albedo * mk3(t.x, t.y, t.z);
                    }
                    if (mat.tex_mr != RT_TEX_NONE) {
                        float4 mr = tex_sample(s.tex[RT_TEX_MR], uvx, uvy, (int32_t)mat.tex_mr);
                        rough = clampf(mat.roughness * mr.y, 0.0f, 1.0f);
                        metal = clampf(mat.metallic * mr.z, 0.0f, 1.0f);
                    }
                    f3 emis = mat.emissive;
                    if (mat.tex_emissive != RT_TEX_NONE) {
                        float4 t = tex_sample(s.tex[RT_TEX_EMISSIVE], uvx, uvy, (int32_t)mat.tex_emissive);
                        emis = mat.emissive * mk3(t.x, t.y, t.z);
                    }
                    add_radiance(sidx, A, thr * emis);

                    bool stop = false;
                    if (kDebug && debug_view != 0u) {  // gather.wgsl:359-419
                        const f3 half = mk3(0.5f, 0.5f, 0.5f);
                        stop = true;
                        switch (debug_view) {
                            case 1: A.col = mk3(uvx, uvy, 0.0f); break;
                            case 2: A.col = sn * 0.5f + half; break;
                            case 3: A.col = shn * 0.5f + half; break;
                            case 4: A.col = gn * 0.5f + half; break;
                            case 5: A.col = emis; break;
                            case 8:
                            case 9: {
                                float pu = (float)px / (float)ip.width, pv = (float)py / (float)ip.height;
                                float4 t =
                                    tex_sample(s.tex[debug_view == 8 ? RT_TEX_EMISSIVE : RT_TEX_ALBEDO], pu, pv, 0);
                                A.col = mk3(t.x, t.y, t.z);
                                break;
                            }
                            case 11: {
                                float4 t = tex_sample(s.tex[RT_TEX_EMISSIVE], uvx, uvy, 0);
                                A.col = mk3(t.x, t.y, t.z);
                                break;
                            }
                            case 12: A.col = mat.emissive; break;
                            case 13: A.col = mk3((float)mat.tex_emissive / 65535.0f, 0.0f, 0.0f); break;
                            case 17: A.col = mk3(uvx - floorf(uvx), uvy - floorf(uvy), 0.0f); break;
                            case 18: {
                                float4 t = tex_sample(s.tex[RT_TEX_ALBEDO], uvx, uvy, (int32_t)mat.tex_albedo);
                                A.col = mk3(t.x, t.y, t.z);
                                break;
                            }
                            case 19:
                            case 20: {
                                f3 ft, fb;
                                tangent_frame(tr, sn, ft, fb);
                                A.col = (debug_view == 19 ? ft : fb) * 0.5f + half;
                                break;
                            }
                            case 21: A.col = hp; break;
                            default: stop = false; break;
                        }
                    }
                    if (stop) {
                        alive = false;
                    } else if (mat.kind == 2u) {  // dielectric (gather.wgsl:421-436)
                        float qd = (mat.ior - 1.0f) / (mat.ior + 1.0f);
                        float f0s = qd * qd;
                        float ct = fabsf(dot(rd, shn));
                        float fr = fresnel_schlick(ct, mk3(f0s, f0s, f0s)).x;
                        if (rng_f32(rng) < fr) {
                            rd = reflect(rd, shn);
                            ro = hp + shn * 0.001f;
                        } else {
                            float eta = ff ? 1.0f / mat.ior : mat.ior;
                            rd = refract(rd, shn, eta);
                            ro = hp - shn * 0.001f;
                            thr = thr * mat.albedo;
                        }
                    } else {  // metallic-roughness (gather.wgsl:439-537)
                        f3 f0 = mk3(0.04f * (1.0f - metal) + albedo.x * metal, 0.04f * (1.0f - metal) + albedo.y * metal,
                                    0.04f * (1.0f - metal) + albedo.z * metal);
                        f3 wo = -rd;
                        float a = fmaxf(rough * rough, 1e-3f);
                        f3 fr = fresnel_schlick(fabsf(dot(rd, shn)), f0);
                        f3 diffuse_weight = (1.0f - metal) * albedo;
                        float sp = max3(fr);
                        float dp = max3(diffuse_weight);
                        float ratio = sp / (sp + dp);
                        float spec_prob = clampf(sp + dp <= 0.0f ? 0.5f : ratio, 0.001f, 0.999f);
                        bool do_spec = rng_f32(rng) < spec_prob;
                        f3 dscale = diffuse_weight / (1.0f - spec_prob);

                        LightSample ls = light_sample(job, hp, shn, rng);
                        f3 c_nee;
                        if (!do_spec) {
                            if (env_intensity > 0.0f)
                                add_radiance(sidx, A, thr * dscale * sky_color(shn, env_color, env_horizon, env_intensity));
                            c_nee = thr * dscale * ls.e / kPi;
                            add_radiance(sidx, A, thr * albedo * ip.ambient);
                        } else {
                            c_nee = thr * spec_ggx(wo, shn, ls.wi, a, f0) * ls.e / spec_prob;
                        }
                        bool nee_luma_only = false;
                        if (kPhotons && ip.use_photons == 1u && !do_spec) {  // gather.wgsl:473-514
                            // The lookup runs in wf_photon_kernel right after this pass; its term
                            // lands before this bounce's NEE term, as here.  Photon debug mode
                            // overwrites the colour after the lookup and keeps only the luminance of
                            // the NEE term, whatever the lookup finds.
                            emit_photon = true;
                            ph_hp = hp;
                            ph_n = shn;
                            ph_td = thr * dscale;
                            ph_sidx = sidx;
                            if (ip.photon_debug == 1u) nee_luma_only = true;
                        }
                        if (ls.occlude && (c_nee.x != 0.0f || c_nee.y != 0.0f || c_nee.z != 0.0f)) {
                            emit_shadow = true;
                            sh_o = ls.o;
                            sh_d = ls.wi;
                            sh_c = c_nee;
                            sh_max = ls.max_dist;
                            sh_tag = (sidx & 0xFFFFu) | (nee_luma_only ? 0x10000u : 0u) | (jid << 17);
                        }
                        if (do_spec) {
                            rd = sample_spec_dir(rd, shn, a, rng);
                            ro = hp + shn * 0.001f;
                            f3 h = normalize(wo + rd);
                            float ndl = fmaxf(dot(shn, rd), 0.0f);
                            thr = thr * fresnel_schlick(fmaxf(dot(wo, h), 0.0f), f0) * smith_g1(ndl, a) / spec_prob;
                        } else {
                            f3 local = sample_cosine_hemisphere(rng);
                            rd = to_world(local, shn);
                            ro = hp + shn * 0.001f;
                            thr = thr * dscale;
                            if (kPhotons && ip.use_photons == 1u) alive = false;
                        }
                        if (alive) {
                            float pr = max3(thr);
                            if (pr <= 0.0f || rng_f32(rng) > pr) alive = false;
                            else thr = thr / pr;
                        }
                    }
                }
            }
            // for-loop step: the segment index advances; the sample ends after max_bounces segments.
            b += 1u;
            if (alive && b >= job.max_bounces) alive = false;
            if (!alive) {
                sidx += 1u;
                if (sidx < spp) {
                    camera_ray(job, px, py, rng, ro, rd);
                    thr = mk3(1.0f, 1.0f, 1.0f);
                    b = 0u;
                    keep = true;
                }
            } else {
                keep = true;
            }
            p.ro[slot] = make_float4(ro.x, ro.y, ro.z, __uint_as_float(rng.state));
            p.rd[slot] = make_float4(rd.x, rd.y, rd.z, __uint_as_float(pack_sb(sidx, b)));
            p.thr[slot] = make_float4(thr.x, thr.y, thr.z, __uint_as_float(jid));
            acc[0] = make_float4(A.col.x, A.col.y, A.col.z, A.lum_sum);
            acc[1] = make_float4(A.lum2_sum, acc1.y, acc1.z, acc1.w);
            if (sidx0 < 8u) reinterpret_cast<float *>(acc + 2)[sidx0] = A.sl;
            if (first_hit) p.nrm[slot] = nrm;
        }
        // Queue positions by original order: each thread appends for the entry it keyed, then the
        // thread that shaded it writes its records there.
        const uint32_t li = i - round_base;
        s_emit[li] = (keep ? 1u : 0u) | (emit_shadow ? 2u : 0u) | ((kPhotons && emit_photon) ? 4u : 0u);
        __syncthreads();
        {
            const uint32_t e = s_emit[threadIdx.x];
            warp_append((e & 1u) != 0u, slot_own, q_next, n_next);
            const uint32_t ms = __ballot_sync(0xFFFFFFFFu, (e & 2u) != 0u);
            if (ms) {
                const uint32_t leader = __ffs(ms) - 1u;
                uint32_t base = 0;
                if (lane == leader) base = atomicAdd(n_shadow, (uint32_t)__popc(ms));
                base = __shfl_sync(0xFFFFFFFFu, base, leader);
                if (e & 2u) s_spos[threadIdx.x] = base + __popc(ms & lanemask_lt());
            }
            if (kPhotons) {
                const uint32_t mp = __ballot_sync(0xFFFFFFFFu, (e & 4u) != 0u);
                if (mp) {
                    const uint32_t leader = __ffs(mp) - 1u;
                    uint32_t base = 0;
                    if (lane == leader) base = atomicAdd(n_photon, (uint32_t)__popc(mp));
                    base = __shfl_sync(0xFFFFFFFFu, base, leader);
                    if (e & 4u) s_ppos[threadIdx.x] = base + __popc(mp & lanemask_lt());
                }
            }
        }
        __syncthreads();
        // NEE shadow ray (deferred) and the photon-map lookup request.
        if (emit_shadow) {
            float4 *rec = p.shadow + 3ull * s_spos[li];
            rec[0] = make_float4(sh_o.x, sh_o.y, sh_o.z, sh_max);
            rec[1] = make_float4(sh_d.x, sh_d.y, sh_d.z, __uint_as_float(slot));
            rec[2] = make_float4(sh_c.x, sh_c.y, sh_c.z, __uint_as_float(sh_tag));
        }
        if (kPhotons && emit_photon) {
            float4 *rec = p.preq + 3ull * s_ppos[li];
            const uint32_t jid = __float_as_uint(p.thr[slot].w);
            rec[0] = make_float4(ph_hp.x, ph_hp.y, ph_hp.z, __uint_as_float(slot));
            rec[1] = make_float4(ph_n.x, ph_n.y, ph_n.z, __uint_as_float(ph_sidx));
            rec[2] = make_float4(ph_td.x, ph_td.y, ph_td.z, __uint_as_float(jid));
        }
    }
}

// ------------------------------------------------------------------------------------------------
// photon: the photon-map lookup of the diffuse bounces shade recorded (gather.wgsl:473-514), one
// request per thread.  A separate pass keeps the shade kernel's registers (and its occupancy) off the
// divergent cell loops.  Runs after shade(iter) and before the occlusion rays of iter, so a pixel's
// terms arrive in the order the inline lookup added them.
// ------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) wf_photon_kernel(const __grid_constant__ WaveParams p, uint32_t iter) {
    const uint32_t n = p.counts[4 * iter + 3];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 r0 = p.preq[3ull * i], r1 = p.preq[3ull * i + 1], r2 = p.preq[3ull * i + 2];
        const uint32_t slot = __float_as_uint(r0.w), sidx = __float_as_uint(r1.w);
        const DevJob &job = p.jobs[__float_as_uint(r2.w)];
        const rt_image_params &ip = job.ip;
        const rt_grid_params &gp = job.gp;
        const f3 hp = xyz(r0), shn = xyz(r1), td = xyz(r2);
        const float r2max = ip.photon_radius * ip.photon_radius;
        f3 ph_sum = mk3(0.0f, 0.0f, 0.0f);
        uint32_t ph_hits = 0u, budget = 384u;
        bool done = false;
        const int32_t bx = f2i_sat((hp.x - gp.room_min_x) / gp.cell_size);
        const int32_t by = f2i_sat((hp.y - gp.room_min_y) / gp.cell_size);
        const int32_t bz = f2i_sat((hp.z - gp.room_min_z) / gp.cell_size);
        const int32_t gxmax = (int32_t)gp.grid_x - 1, gymax = (int32_t)gp.grid_y - 1, gzmax = (int32_t)gp.grid_z - 1;
        // The 27 cells in the reference's order (dz, then dy, then dx), walked as one flat loop over
        // (cell, photon group) so each thread moves to its next cell on its own instead of the warp
        // waiting at every cell for its fullest one.
        auto cell_at = [&](uint32_t i) {
            const int32_t dz = (int32_t)(i / 9u) - 1, dy = (int32_t)((i / 3u) % 3u) - 1, dx = (int32_t)(i % 3u) - 1;
            const int32_t cx = clampi((int32_t)((uint32_t)bx + (uint32_t)dx), 0, gxmax);
            const int32_t cy = clampi((int32_t)((uint32_t)by + (uint32_t)dy), 0, gymax);
            const int32_t cz = clampi((int32_t)((uint32_t)bz + (uint32_t)dz), 0, gzmax);
            return (uint32_t)cx + (uint32_t)cy * gp.grid_x + (uint32_t)cz * gp.grid_x * gp.grid_y;
        };
        // Photon indices are u32 and clamped to the last sorted photon (the backend's rule for an
        // out-of-range index; the grid's ranges never leave the array).
        const uint32_t last = (uint32_t)job.sorted_count - 1u;
        const float4 *posv = job.sorted_pos ? job.sorted_pos : job.sorted_photons;
        const uint32_t pstride = job.sorted_pos ? 1u : 4u;
        uint32_t ci = 0u, k = 0u;
        uint2 m = __ldg(job.grid_meta + cell_at(0u));
        if (job.sorted_count == 0u) m.y = 0u, ci = 27u;
        while (!done) {
            if (k >= m.y) {
                if (++ci >= 27u) break;  // also ends at once for an empty photon map
                m = __ldg(job.grid_meta + cell_at(ci));
                k = 0u;
                continue;
            }
            // A group of four photons: positions loaded together (from the compact position array
            // when there is one), then tested in order with the budget and the hit cap.
            float4 pos[4];
#pragma unroll
            for (uint32_t j = 0; j < 4u; ++j) pos[j] = __ldg(posv + (size_t)min(m.x + k + j, last) * pstride);
#pragma unroll
            for (uint32_t j = 0; j < 4u; ++j) {
                if (done || k + j >= m.y) break;
                if (budget == 0u) {
                    done = true;
                    break;
                }
                budget -= 1u;
                const f3 dd = xyz(pos[j]) - hp;
                const float d2 = dot(dd, dd);
                if (d2 < r2max) {
                    const float4 *ph = job.sorted_photons + 4ull * min(m.x + k + j, last);
                    const f3 pw = xyz(__ldg(ph + 1));
                    const f3 inc = xyz(__ldg(ph + 2));
                    ph_sum = ph_sum + pw * fmaxf(dot(shn, -inc), 0.0f);
                    ph_hits += 1u;
                    if (ph_hits >= 64u) done = true;
                }
            }
            k += 4u;
        }
        if (ph_hits > 0u)
            acc_add_term(p, slot, sidx,
                         td * ph_sum * ip.photon_scale / (kPi * (float)ph_hits * ip.photon_radius * ip.photon_radius),
                         false);
        if (ip.photon_debug == 1u) {
            const float density = fminf((float)ph_hits / 64.0f, 1.0f);
            const f3 col = mk3(1.0f - density, density, 0.0f) * 2.0f;
            float4 *a = p.acc + 4 * (size_t)slot;
            a[0] = make_float4(col.x, col.y, col.z, a[0].w);
        }
    }
}

// ------------------------------------------------------------------------------------------------
// shadow: the deferred NEE occlusion test (gather.wgsl:91-103) and the contribution of visible lights.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ void shadow_resolve(const WaveParams &p, uint32_t rec_i, const TravState &st, float limit) {
    const float4 o = p.shadow[3ull * rec_i], d = p.shadow[3ull * rec_i + 1], c = p.shadow[3ull * rec_i + 2];
    const uint32_t tag = __float_as_uint(c.w);
    const DevScene &s = p.jobs[tag >> 17].scene;
    bool shadowed = !(st.t >= limit);
    if (shadowed && !s.any_hit_shadows) {
        TriFull bt = load_tri(s, trav_hit_prim(st));
        Mat bm = load_mat(s, bt.material_id);
        if ((bm.flags & RT_MAT_FLAG_ALPHA_CUTOUT) != 0u && bm.tex_albedo != RT_TEX_NONE) {
            Bary b = barycentric(bt, xyz(o), xyz(d), st.t);
            if (tex_sample(s.tex[RT_TEX_ALBEDO], b.uvx, b.uvy, (int32_t)bm.tex_albedo).w < 0.5f) shadowed = false;
        }
    }
    if (shadowed) return;
    acc_add_term(p, __float_as_uint(d.w), tag & 0xFFFFu, xyz(c), (tag & 0x10000u) != 0u);
}

// trace: the occlusion rays of iteration `shd_iter` and the closest-hit rays of iteration `ext_iter` in
// one persistent launch (either may be kNoIter).  Both depend only on the shade pass before them and
// touch disjoint state (shadow records and accumulators / path rays and hits), so one launch carries
// them with one tail instead of two.  Closest-hit rays come first in the work list: the longer rays
// start early and the shorter occlusion rays fill the end.
constexpr uint32_t kNoIter = 0xFFFFFFFFu;

// kCount: the profiling variant, which also counts the records each kind of ray visits and its leaf
// triangle tests into p.work (one atomic per warp at exit); the same rays and results otherwise.
// kTree (four-wide only): the block first stages the top kTree records of job 0's tree in shared
// memory (after the stacks and the WarpLeaves), and lanes on that scene read them from there.
template <int kStack, int kBlock, bool kWide, bool kCount, int kTree>
__global__ void __launch_bounds__(kBlock, 1024 / kBlock) wf_trace_kernel(const __grid_constant__ WaveParams p, uint32_t ext_iter,
                                                          uint32_t shd_iter, uint32_t chunk, uint32_t steps) {
    extern __shared__ uint32_t stack_smem[];
    uint32_t *stk = stack_smem + threadIdx.x;
    WarpLeaves &wl = reinterpret_cast<WarpLeaves *>(stack_smem + kStack * kBlock)[threadIdx.x >> 5];
    float4 *tree = nullptr;
    const float4 *tree_src = nullptr;
    uint32_t tree_n = 0u;
    if (kTree > 0) {
        tree = reinterpret_cast<float4 *>(reinterpret_cast<WarpLeaves *>(stack_smem + kStack * kBlock) + kBlock / 32);
        const DevScene &s0 = p.jobs[0].scene;
        tree_src = s0.wnodes;
        tree_n = s0.wnode_count < (uint32_t)kTree ? s0.wnode_count : (uint32_t)kTree;
        for (uint32_t i = threadIdx.x; i < 8u * tree_n; i += kBlock) tree[i] = __ldg(tree_src + i);
        __syncthreads();
    }
    const uint32_t n_ext = ext_iter != kNoIter ? p.counts[4 * ext_iter] : 0u;
    const uint32_t n_shd = shd_iter != kNoIter ? p.counts[4 * shd_iter + 1] : 0u;
    const uint32_t *q = p.queue[ext_iter & 1u];
    // Row ext_iter's cursor; the closing launch (no closest-hit rays) takes row shd_iter + 1's, which
    // no other launch uses.  Entry [3] of a row counts shade's photon-lookup requests.
    uint32_t *fetch = p.counts + 4 * (ext_iter != kNoIter ? ext_iter : shd_iter + 1u) + 2;
    WarpFeed feed;
    TravState st;
    bool has = false, occlusion = false, any_hit = false;
    uint32_t id = 0;  // path slot (closest hit) or shadow record (occlusion)
    float limit = 0.0f;
    uint32_t work[4] = {0u, 0u, 0u, 0u};  // kCount: records closest / occlusion, tests closest / occlusion
    // steps: records between refills (low 16 bits) and the idle-lane count that refills earlier (high)
    const uint32_t max_steps = steps & 0xFFFFu, refill_idle = steps >> 16;
    for (;;) {
        const uint32_t item = warp_take(feed, !has, n_ext + n_shd, fetch, chunk);
        if (item != 0xFFFFFFFFu) {
            occlusion = item >= n_ext;
            if (!occlusion) {
                id = q[item];
                const float4 o = p.ro[id], d = p.rd[id];
                const DevScene &sc = p.jobs[__float_as_uint(p.thr[id].w)].scene;
                any_hit = false;
                st = trav_begin<kWide>(sc, xyz(o), xyz(d), kInf, (uint32_t)kStack);
                has = sc.cnode_count != 0u;
                if (!has) p.hit[id] = make_float2(kInf, 0.0f);
            } else {
                id = item - n_ext;
                const float4 o = p.shadow[3ull * id], d = p.shadow[3ull * id + 1];
                const DevScene &sc = p.jobs[__float_as_uint(p.shadow[3ull * id + 2].w) >> 17].scene;
                limit = o.w - 0.001f;
                // Without cut-out materials the occlusion test may stop at the first triangle below
                // the limit; with them the reference's closest-hit-then-alpha rule is kept.
                any_hit = sc.any_hit_shadows != 0u;
                st = trav_begin<kWide>(sc, xyz(o), xyz(d), any_hit ? limit : kInf, (uint32_t)kStack);
                has = sc.cnode_count != 0u;
                if (!has) {
                    st.t = kInf;
                    shadow_resolve(p, id, st, limit);
                }
            }
            if (has) warp_leaves_set_ray(wl, st);
        }
        if (!__any_sync(0xFFFFFFFFu, has)) break;
        for (uint32_t k = 0; k < max_steps; ++k) {
            uint32_t tests = 0u;
            const bool visiting = has;
            if (kWide ? trav_step_warp4(st, has, any_hit, stk, (uint32_t)kBlock, wl, kCount ? &tests : nullptr,
                                        kTree > 0 ? tree : nullptr, tree_src, tree_n)
                      : trav_step_warp(st, has, any_hit, stk, (uint32_t)kBlock, wl, kCount ? &tests : nullptr)) {
                if (occlusion) shadow_resolve(p, id, st, limit);
                else p.hit[id] = make_float2(st.t, __uint_as_float(st.prim));  // the hit's prim slot
                has = false;
            }
            if (kCount && visiting) {
                work[occlusion ? 1 : 0] += 1u;
                work[occlusion ? 3 : 2] += tests;
            }
            const uint32_t busy = __ballot_sync(0xFFFFFFFFu, has);
            if (busy == 0u) break;
            // early refill once `refill_idle` lanes wait and the queue still has work
            if (refill_idle != 0u && 32u - (uint32_t)__popc(busy) >= refill_idle && feed.more) break;
        }
    }
    if (kCount && p.work) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            uint32_t v = work[i];
#pragma unroll
            for (uint32_t d = 16u; d > 0u; d >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, d);
            if ((threadIdx.x & 31u) == 0u) atomicAdd(p.work + i, (unsigned long long)v);
        }
    }
}

// ------------------------------------------------------------------------------------------------
// finalize: firefly sigma clamp and the frame outputs (gather.wgsl:548-593).  One launch over every
// job's slots.
// ------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) wf_finalize_kernel(const __grid_constant__ WaveParams p, uint32_t n_slots) {
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= n_slots) return;
    const DevJob &job = p.jobs[job_of(p, slot, [](const DevJob &j) { return j.base; })];
    const uint32_t pix = slot - job.base;
    if (pix >= job.npix) return;
    const uint32_t spp = job.spp;
    Accum A = load_acc(p, slot);
    const float first_depth = p.acc[4 * (size_t)slot + 1].y;
    const float4 nrm = p.nrm[slot];
    if (spp <= 8u) {
        float *sl = A.sl;
        for (uint32_t i = 1; i < spp; ++i) {
            float key = sl[i];
            uint32_t j = i;
            while (j > 0u && sl[j - 1u] > key) {
                sl[j] = sl[j - 1u];
                j -= 1u;
            }
            sl[j] = key;
        }
        float median = (sl[(spp - 1u) / 2u] + sl[spp / 2u]) * 0.5f;
        uint32_t half = spp / 2u > 1u ? spp / 2u : 1u;
        float spread = 0.0f;
        for (uint32_t i = 0; i < half; ++i) {
            float dd = sl[i] - median;
            spread += dd * dd;
        }
        float sigma = fmaxf(sqrtf(spread / (float)half), 0.25f * median + 1e-5f);
        float thresh = median + 3.0f * sigma;
        float cl = 0.0f, cl2 = 0.0f;
        for (uint32_t i = 0; i < spp; ++i) {
            float lc = fminf(sl[i], thresh);
            cl += lc;
            cl2 += lc * lc;
        }
        A.col = A.col * (cl / fmaxf(A.lum_sum, 1e-10f));
        A.lum_sum = cl;
        A.lum2_sum = cl2;
    }
    f3 col = vmin(A.col / (float)spp, mk3(10.0f, 10.0f, 10.0f));
    job.frame[pix] = make_float4(col.x, col.y, col.z, 1.0f);
    job.moments[pix] = make_float4(fminf(A.lum_sum / (float)spp, 10.0f), fminf(A.lum2_sum / (float)spp, 100.0f), 0.0f, 0.0f);
    job.gbuffer[pix] = make_float4(nrm.x, nrm.y, nrm.z, first_depth);
}

// Segments (paths queued per iteration) and shadow rays of the pass, added to the 64-bit counters.
__global__ void wf_count_kernel(const __grid_constant__ WaveParams p, uint32_t iters) {
    if (threadIdx.x != 0u || !p.counters) return;
    unsigned long long seg = 0, shd = 0;
    for (uint32_t i = 0; i < iters; ++i) {
        seg += p.counts[4 * i];
        shd += p.counts[4 * i + 1];
    }
    p.counters[0] += seg;
    p.counters[1] += shd;
}

// ------------------------------------------------------------------------------------------------
// Host launcher: the gather pass of one frame of every job.
// ------------------------------------------------------------------------------------------------
WaveTuning default_tuning() { return WaveTuning{128u, 8u, 32u, 3u, 32u, 0u, 6u, 0u}; }

bool normalize_tuning(WaveTuning &t, uint32_t stack_need) {
    const WaveTuning in = t;
    if (t.block_threads != 64u && t.block_threads != 128u && t.block_threads != 256u) t.block_threads = 128u;
    const uint32_t max_blocks = 2048u / t.block_threads;  // resident threads per SM
    t.blocks_per_sm = t.blocks_per_sm < 1u ? 1u : (t.blocks_per_sm > max_blocks ? max_blocks : t.blocks_per_sm);
    t.chunk = t.chunk < 32u ? 32u : (t.chunk > 1024u ? 1024u : (t.chunk + 31u) / 32u * 32u);
    t.steps = t.steps < 1u ? 1u : (t.steps > 64u ? 64u : t.steps);
    t.refill_idle = t.refill_idle > 31u ? 31u : t.refill_idle;
    const uint32_t need = stack_need > t.stack_entries ? stack_need : t.stack_entries;
    t.stack_entries = need <= 32u ? 32u : (need <= 48u ? 48u : 64u);
    t.treelet = t.treelet ? kTreeletRecords : 0u;
    t.shade_blocks = t.shade_blocks >= 4u && t.shade_blocks <= 6u ? t.shade_blocks : 6u;
    return std::memcmp(&in, &t, sizeof(t)) == 0;
}

namespace {

using ExtendKernel = void (*)(const WaveParams, uint32_t, uint32_t, uint32_t);
using TraceKernel = void (*)(const WaveParams, uint32_t, uint32_t, uint32_t, uint32_t);

template <int kStack, int kBlock>
void pick(const WaveTuning &t, bool wide, bool count, ExtendKernel &ext, TraceKernel &trc) {
    if ((int)t.stack_entries == kStack && (int)t.block_threads == kBlock) {
        ext = wide ? wf_extend_kernel<kStack, kBlock, true> : wf_extend_kernel<kStack, kBlock, false>;
        constexpr int kT = (int)kTreeletRecords;
        const bool tree = wide && t.treelet != 0u;
        if (!wide)
            trc = count ? wf_trace_kernel<kStack, kBlock, false, true, 0> : wf_trace_kernel<kStack, kBlock, false, false, 0>;
        else if (tree)
            trc = count ? wf_trace_kernel<kStack, kBlock, true, true, kT> : wf_trace_kernel<kStack, kBlock, true, false, kT>;
        else
            trc = count ? wf_trace_kernel<kStack, kBlock, true, true, 0> : wf_trace_kernel<kStack, kBlock, true, false, 0>;
    }
}

// Dynamic shared memory of a traversal block: the lane-interleaved stacks, then one WarpLeaves per warp,
// then the treelet (four-wide launches with t.treelet set).
size_t trav_smem_bytes(const WaveTuning &t, bool wide = false) {
    return (size_t)t.stack_entries * t.block_threads * sizeof(uint32_t) + (t.block_threads / 32u) * sizeof(WarpLeaves) +
           (wide && t.treelet ? (size_t)kTreeletRecords * 8u * sizeof(float4) : 0u);
}

void trav_kernels(const WaveTuning &t, bool wide, ExtendKernel &ext, TraceKernel &shd, bool count = false) {
    ext = nullptr;
    shd = nullptr;
    pick<32, 64>(t, wide, count, ext, shd);
    pick<32, 128>(t, wide, count, ext, shd);
    pick<32, 256>(t, wide, count, ext, shd);
    pick<48, 64>(t, wide, count, ext, shd);
    pick<48, 128>(t, wide, count, ext, shd);
    pick<48, 256>(t, wide, count, ext, shd);
    pick<64, 64>(t, wide, count, ext, shd);
    pick<64, 128>(t, wide, count, ext, shd);
    pick<64, 256>(t, wide, count, ext, shd);
}

}  // namespace

template <int kStack, int kBlock, bool kWide>
void opt_in_smem() {
    // Blocks above 48 KB of dynamic shared memory need the opt-in; set it for every shape.
    const int bytes = (int)trav_smem_bytes(WaveTuning{(uint32_t)kBlock, 1u, 64u, 8u, (uint32_t)kStack, 0u, 4u, 0u});
    const int tree_bytes =
        (int)trav_smem_bytes(WaveTuning{(uint32_t)kBlock, 1u, 64u, 8u, (uint32_t)kStack, 1u, 4u, 0u}, true);
    constexpr int kT = (int)kTreeletRecords;
    cudaFuncSetAttribute(wf_extend_kernel<kStack, kBlock, kWide>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(wf_trace_kernel<kStack, kBlock, kWide, false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         bytes);
    cudaFuncSetAttribute(wf_trace_kernel<kStack, kBlock, kWide, true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         bytes);
    if (kWide) {
        cudaFuncSetAttribute(wf_trace_kernel<kStack, kBlock, true, false, kT>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, tree_bytes);
        cudaFuncSetAttribute(wf_trace_kernel<kStack, kBlock, true, true, kT>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, tree_bytes);
    }
}

template <bool kWide>
void opt_in_all() {
    opt_in_smem<32, 64, kWide>();
    opt_in_smem<32, 128, kWide>();
    opt_in_smem<32, 256, kWide>();
    opt_in_smem<48, 64, kWide>();
    opt_in_smem<48, 128, kWide>();
    opt_in_smem<48, 256, kWide>();
    opt_in_smem<64, 64, kWide>();
    opt_in_smem<64, 128, kWide>();
    opt_in_smem<64, 256, kWide>();
}

void prepare_wavefront_kernels() {
    opt_in_all<false>();
    opt_in_all<true>();
}

cudaError_t launch_extend(const WaveParams &p, uint32_t iter, uint64_t max_items, const DevScene &scene, int num_sms,
                          const WaveTuning &tune, cudaStream_t st) {
    const bool wide = scene.wnodes != nullptr;
    WaveTuning t = tune;
    normalize_tuning(t, wide ? scene.wide_stack : scene.stack_cap);
    ExtendKernel ext;
    TraceKernel trc;
    trav_kernels(t, wide, ext, trc);
    const size_t smem = trav_smem_bytes(t);
    const uint64_t blocks_needed = (max_items + t.block_threads - 1u) / t.block_threads;
    const uint64_t persistent = (uint64_t)num_sms * t.blocks_per_sm;
    const uint32_t grid = (uint32_t)(blocks_needed < persistent ? (blocks_needed ? blocks_needed : 1u) : persistent);
    ext<<<grid, t.block_threads, smem, st>>>(p, iter, t.chunk, t.steps);
    return cudaGetLastError();
}

cudaError_t launch_wavefront(const WaveParams &p, const JobShape *jobs, uint32_t n_jobs, uint32_t iters, int num_sms,
                             const WaveTuning &tune, cudaStream_t st, WaveProfile *prof) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(p.counts, 0, sizeof(uint32_t) * 4 * (size_t)(iters + 1), st)) != cudaSuccess) return e;
    uint64_t slots = 0;
    uint32_t stack_need = 0, wide_need = 0;
    bool wide = n_jobs > 0;  // four-wide records when every job's scene has them
    uint64_t tiles = 0;
    for (uint32_t j = 0; j < n_jobs; ++j) {
        tiles += ((jobs[j].width + 7u) / 8u) * ((jobs[j].height + 3u) / 4u);
        slots += jobs[j].npix;
        stack_need = jobs[j].stack_cap > stack_need ? jobs[j].stack_cap : stack_need;
        wide_need = jobs[j].wide_stack > wide_need ? jobs[j].wide_stack : wide_need;
        wide = wide && jobs[j].wide != 0u;
    }
    if (tiles) wf_generate_kernel<<<(unsigned)((tiles + 3u) / 4u), 128, 0, st>>>(p, (uint32_t)tiles);
    WaveTuning t = tune;
    normalize_tuning(t, wide ? wide_need : stack_need);
    ExtendKernel ext;
    TraceKernel trc;
    trav_kernels(t, wide, ext, trc, p.work != nullptr);
    const size_t smem = trav_smem_bytes(t, wide);
    // A launch carries up to one path per slot plus one occlusion ray per slot.
    const uint64_t blocks_needed = (2u * slots + t.block_threads - 1u) / t.block_threads;
    const uint64_t persistent = (uint64_t)num_sms * t.blocks_per_sm;
    const uint32_t grid = (uint32_t)(blocks_needed < persistent ? blocks_needed : persistent);
    const uint64_t shade_needed = (slots + 127u) / 128u, shade_cap = (uint64_t)num_sms * 2u * t.shade_blocks;
    const uint32_t shade_grid = (uint32_t)(shade_needed < shade_cap ? shade_needed : shade_cap);
    const uint64_t photon_cap = (uint64_t)num_sms * 16u;
    const uint32_t photon_grid = (uint32_t)(shade_needed < photon_cap ? shade_needed : photon_cap);
    // extend(0), shade(0), then per iteration one trace launch with the occlusion rays of the
    // iteration before and the closest-hit rays of this one, then its shade; the last occlusion rays
    // close the pass.
    bool photons = false, debug = false;
    for (uint32_t j = 0; j < n_jobs; ++j) {
        photons = photons || jobs[j].photons != 0u;
        debug = debug || jobs[j].debug != 0u;
    }
    void (*shade)(const WaveParams, uint32_t);
    if (t.shade_blocks == 6u)
        shade = photons ? (debug ? wf_shade_kernel<true, true, 6> : wf_shade_kernel<true, false, 6>)
                        : (debug ? wf_shade_kernel<false, true, 6> : wf_shade_kernel<false, false, 6>);
    else if (t.shade_blocks == 5u)
        shade = photons ? (debug ? wf_shade_kernel<true, true, 5> : wf_shade_kernel<true, false, 5>)
                        : (debug ? wf_shade_kernel<false, true, 5> : wf_shade_kernel<false, false, 5>);
    else
        shade = photons ? (debug ? wf_shade_kernel<true, true, 4> : wf_shade_kernel<true, false, 4>)
                        : (debug ? wf_shade_kernel<false, true, 4> : wf_shade_kernel<false, false, 4>);
    uint32_t n_trc = 0, n_shd = 0, n_pho = 0;
    // Events of the profiled pass around one launch (never inside a captured graph: prof is null there).
    auto mark = [&](cudaEvent_t *ev, uint32_t i, int side) {
        if (prof && ev) cudaEventRecord(ev[2 * i + side], st);
    };
    for (uint32_t it = 0; it < iters; ++it) {
        mark(prof ? prof->trace_ev : nullptr, n_trc, 0);
        trc<<<grid, t.block_threads, smem, st>>>(p, it, it ? it - 1u : kNoIter, t.chunk, t.steps | (t.refill_idle << 16));
        mark(prof ? prof->trace_ev : nullptr, n_trc++, 1);
        mark(prof ? prof->shade_ev : nullptr, n_shd, 0);
        shade<<<shade_grid, 128, 0, st>>>(p, it);
        mark(prof ? prof->shade_ev : nullptr, n_shd++, 1);
        if (photons) {
            mark(prof ? prof->photon_ev : nullptr, n_pho, 0);
            wf_photon_kernel<<<photon_grid, 128, 0, st>>>(p, it);
            mark(prof ? prof->photon_ev : nullptr, n_pho++, 1);
        }
    }
    if (iters) {
        mark(prof ? prof->trace_ev : nullptr, n_trc, 0);
        trc<<<grid, t.block_threads, smem, st>>>(p, kNoIter, iters - 1u, t.chunk, t.steps | (t.refill_idle << 16));
        mark(prof ? prof->trace_ev : nullptr, n_trc++, 1);
    }
    if (prof) {
        prof->trace_launches = n_trc;
        prof->shade_launches = n_shd;
        prof->photon_launches = n_pho;
    }
    if (slots) wf_finalize_kernel<<<(unsigned)((slots + 255u) / 256u), 256, 0, st>>>(p, (uint32_t)slots);
    wf_count_kernel<<<1, 32, 0, st>>>(p, iters);
    return cudaGetLastError();
}

}  // namespace rtd
