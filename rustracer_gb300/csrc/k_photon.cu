// Photon pass and photon grid (config 3 of the photon map).
//
//   photon wavefront      photon_trace.wgsl:91-260 as generate (emission) + per bounce the shared
//                         closest-hit kernel and ph_shade (one bounce body per queued photon).  The
//                         bounce body also emits the u32 cell key of every slot it stores
//                         (photon_count.wgsl:18-23), so the grid build never re-reads positions.
//   photon_keys_kernel    keys of a photon buffer loaded from the host (same key function).
//   grid build            exact u32 counting sort of the slots by cell key; without per-slot ranks
//                         (the no-allocation entry, whose scratch holds no rank array):
//     count_kernel        histogram (photon_count.wgsl:25-34)
//     scan_*              device exclusive scan of the counts into (start, count) pairs; replaces the
//                         blocking read-back and host scan of lib.rs:956-1007
//     scatter_kernel      slot index to start + cursor (photon_scatter.wgsl:61-71)
//     multi_cells_kernel  the cells holding two or more photons
//     order_kernel        sorts each such cell's slot indices ascending: the result is the scatter in
//                         slot order, independent of atomic arrival order (the reference's order
//                         within a cell is unspecified)
//     gather_kernel       sorted[i] = photons[order[i]] (64-byte records)
//   grid build with ranks (the renderer's and the stage entry's path): count_rank (histogram + each
//   slot's rank in atomic order), scan_lookback_list (single-pass scan + list of occupied cells),
//   scatter_rank (start + rank, no atomics), then cell_gather: per occupied cell the slot order
//   restored and the records copied in one pass.  Same counts, offsets and slot order either way.
#include <algorithm>
#include <cstring>

#include "rt_kernels.h"

namespace rtd {

namespace {

__device__ __forceinline__ f3 surface_albedo(const DevScene &s, const Mat &m, float u, float v) {
    if (m.tex_albedo != RT_TEX_NONE) {
        float4 t = tex_sample(s.tex[RT_TEX_ALBEDO], u, v, (int32_t)m.tex_albedo);
        return mk3(t.x, t.y, t.z);
    }
    return m.albedo;
}

__device__ __forceinline__ f3 bounce_dir(f3 rd, f3 n, float rough, Rng &rng) {
    f3 mirror = reflect(rd, n);
    float blur = smoothstepf(0.0f, 1.0f, rough);
    if (blur <= 0.001f) return mirror;
    f3 diff = sample_cosine_hemisphere(rng);
    return normalize(mix3(mirror, to_world(diff, n), blur));
}

__device__ __forceinline__ uint32_t cell_key(const rt_grid_params &gp, f3 pos) {
    uint32_t gx = f2u_sat((pos.x - gp.room_min_x) / gp.cell_size);
    uint32_t gy = f2u_sat((pos.y - gp.room_min_y) / gp.cell_size);
    uint32_t gz = f2u_sat((pos.z - gp.room_min_z) / gp.cell_size);
    return gx + gy * gp.grid_x + gz * gp.grid_x * gp.grid_y;
}

__device__ __forceinline__ uint32_t slot_key(const rt_grid_params &gp, f3 pos, float power_r) {
    if (power_r <= 0.0f) return kInvalidKey;
    uint32_t k = cell_key(gp, pos);
    return k < gp.num_cells ? k : kInvalidKey;
}

}  // namespace

// The photon's origin, direction and power as emitted from a light picked uniformly
// (photon_trace.wgsl:91-190); false when no photon leaves (no lights, unknown kind).
__device__ bool photon_emit(const PhotonTraceParams &p, uint32_t photon_index, Rng &rng, f3 &origin, f3 &dir,
                            f3 &power) {
    const DevScene &s = p.scene;
    const uint32_t num_lights = s.light_count;
    if (num_lights == 0u) return false;
    rng = rng_init(photon_index * 1103515245u + 12345u);
    uint32_t li = f2u_sat(rng_f32(rng) * (float)num_lights);
    li = li < num_lights ? li : num_lights - 1u;
    const Light light = load_light(s, li);
    origin = light.data;
    dir = mk3(0.0f, 0.0f, 1.0f);
    power = mk3(0.0f, 0.0f, 0.0f);
    if (light.kind == 0u) {
        float u1 = 0.0f, u2 = 0.0f;
        for (uint32_t guard = 0;; ++guard) {
            u1 = rng_f32(rng) * 2.0f - 1.0f;
            u2 = rng_f32(rng) * 2.0f - 1.0f;
            if (u1 * u1 + u2 * u2 < 1.0f) break;
            if (guard >= (1u << 20)) return false;  // bounded; (1 - pi/4)^(2^20) is zero in practice
        }
        float z = 1.0f - 2.0f * (u1 * u1 + u2 * u2);
        float r = sqrtf(1.0f - z * z);
        dir = normalize(mk3(r * 2.0f * u1, r * 2.0f * u2, z));
        power = light.color * light.intensity;
    } else if (light.kind == 1u) {
        float du = (rng_f32(rng) - 0.5f) * 10.0f;
        float dv = (rng_f32(rng) - 0.5f) * 10.0f;
        f3 d = light.data;
        f3 up = fabsf(d.y) < 0.999f ? mk3(0.0f, 1.0f, 0.0f) : mk3(1.0f, 0.0f, 0.0f);
        f3 tangent = normalize(cross(up, d));
        f3 bitangent = cross(d, tangent);
        origin = du * tangent + dv * bitangent - d * 100.0f;
        dir = d;
        power = light.color * light.intensity;
    } else if (light.kind == 2u) {
        Tri tri = load_tri_verts(s, f2u_sat(light.data.x));
        float u1 = rng_f32(rng);
        float u2 = rng_f32(rng);
        float su = sqrtf(u1);
        float u = 1.0f - su;
        float v = u2 * su;
        float w = 1.0f - u - v;
        origin = tri.v0 * u + tri.v1 * v + tri.v2 * w;
        f3 n = triangle_normal(tri.v0, tri.v1, tri.v2);
        f3 local = sample_cosine_hemisphere(rng);
        dir = to_world(local, n);
        power = light.color * light.intensity;
    } else if (light.kind == 3u) {
        const rt_grid_params &gp = p.gp;
        f3 local = sample_cosine_hemisphere(rng);
        f3 d = to_world(local, mk3(0.0f, 1.0f, 0.0f));
        f3 span = mk3((float)gp.grid_x, (float)gp.grid_y, (float)gp.grid_z) * gp.cell_size;
        f3 center = mk3(gp.room_min_x, gp.room_min_y, gp.room_min_z) + span * 0.5f;
        float R = fmaxf(fmaxf(span.x, span.y), span.z) * 1.2f + 0.05f;
        origin = center + d * R;
        dir = -d;
        float t = clampf(d.y * 0.5f + 0.5f, 0.0f, 1.0f);
        power = mix3(light.color, light.data, sqrtf(t)) * light.intensity;  // pow(t, 0.5), t in [0, 1]
    } else {
        return false;
    }
    return true;

}

// One iteration of photon_trace.wgsl's bounce loop (:192-258) after the closest hit (t, prim) of
// (origin, dir): stores the photon at slot 6 i + bounce unless the surface passes it on, and updates
// the ray; false when the photon ends (emitter hit, Russian roulette).
__device__ bool photon_bounce(const PhotonTraceParams &p, uint32_t photon_index, uint32_t bounce, float hit_t,
                              uint32_t hit_prim, Rng &rng, f3 &origin, f3 &dir, f3 &power) {
    const DevScene &s = p.scene;
    struct {
        float t;
        uint32_t prim;
    } hit{hit_t, hit_prim};
    TriFull tri = load_tri(s, hit.prim);
    Mat mat = load_mat(s, tri.material_id);
    f3 hit_pos = origin + dir * hit.t;
    Bary bb = barycentric(tri, origin, dir, hit.t);
    f3 normal = triangle_normal(tri.v0, tri.v1, tri.v2);
    bool front = dot(dir, normal) < 0.0f;
    f3 sn_geom = smooth_normal(tri, bb, normal);
    f3 face_normal = front ? sn_geom : -sn_geom;
    f3 shn = face_normal;
    if (mat.tex_normal != RT_TEX_NONE) {
        float4 t = tex_sample(s.tex[RT_TEX_NORMAL], bb.uvx, bb.uvy, (int32_t)mat.tex_normal);
        f3 nm = mk3(t.x, t.y, t.z) * 2.0f - mk3(1.0f, 1.0f, 1.0f);
        f3 ft, fb;
        tangent_frame(tri, face_normal, ft, fb);
        shn = normalize(ft * nm.x + fb * nm.y + face_normal * nm.z);
    }
    if ((mat.flags & RT_MAT_FLAG_ALPHA_CUTOUT) != 0u && mat.tex_albedo != RT_TEX_NONE) {
        float alpha = tex_sample(s.tex[RT_TEX_ALBEDO], bb.uvx, bb.uvy, (int32_t)mat.tex_albedo).w;
        if (alpha < 0.5f) {
            origin = hit_pos + dir * 0.002f;
            return true;
        }
    }
    if (mat.tex_emissive != RT_TEX_NONE || len3(mat.emissive) > 1e-4f || mat.kind == 3u) return false;
    if (mat.kind == 2u) {
        float q = (mat.ior - 1.0f) / (mat.ior + 1.0f);
        float f0s = q * q;
        float ct = fabsf(dot(dir, face_normal));
        float fr = fresnel_schlick(ct, mk3(f0s, f0s, f0s)).x;
        if (rng_f32(rng) < fr) {
            dir = reflect(dir, face_normal);
            origin = hit_pos + face_normal * 0.001f;
        } else {
            float eta = front ? 1.0f / mat.ior : mat.ior;
            dir = refract(dir, face_normal, eta);
            origin = hit_pos - face_normal * 0.001f;
        }
        return true;
    }
    const uint64_t slot = (uint64_t)photon_index * 6u + bounce;
    if (slot < p.slot_count) {
        float4 *ph = p.photons + 4ull * slot;
        f3 inc = -dir;
        ph[0] = make_float4(hit_pos.x, hit_pos.y, hit_pos.z, 0.0f);
        ph[1] = make_float4(power.x, power.y, power.z, 0.0f);
        ph[2] = make_float4(inc.x, inc.y, inc.z, 0.0f);
        ph[3] = make_float4(shn.x, shn.y, shn.z, 0.0f);
        p.keys[slot] = slot_key(p.gp, hit_pos, power.x);
    }
    f3 albedo = surface_albedo(s, mat, bb.uvx, bb.uvy);
    const float mt = mat.metallic;
    f3 f0 = mk3(0.04f * (1.0f - mt) + albedo.x * mt, 0.04f * (1.0f - mt) + albedo.y * mt,
                0.04f * (1.0f - mt) + albedo.z * mt);
    float ct = fabsf(dot(dir, shn));
    f3 fr = fresnel_schlick(ct, f0);
    f3 diffuse_weight = (1.0f - mt) * albedo;
    float spec_prob = clampf(max3(fr), 0.0f, 0.98f);
    bool do_spec = rng_f32(rng) < spec_prob;
    if (do_spec) {
        dir = bounce_dir(dir, shn, mat.roughness, rng);
        power = power * f0;
    } else {
        f3 local = sample_cosine_hemisphere(rng);
        dir = to_world(local, shn);
        power = power * diffuse_weight;
    }
    origin = hit_pos + shn * 0.001f;
    float pr = max3(power);
    if (pr <= 0.0f || rng_f32(rng) > pr) return false;
    power = power / pr;
    return true;
}

// ------------------------------------------------------------------------------------------------
// Photon wavefront: generate (emission), then per bounce the shared closest-hit kernel (wf_extend,
// persistent traversal warps) and ph_shade (one bounce body per queued photon, survivors re-queued).
// Lanes stay busy when photons end at different bounces, and each kernel is small; the per-photon
// operations and their order are those of the loop, so every photon's path is unchanged.
// ------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) ph_generate_kernel(const __grid_constant__ PhotonTraceParams p,
                                                          const PhotonWave w) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t photon_index = p.photon_begin + i;
    bool live = false;
    if (photon_index < p.photon_end) {
        Rng rng;
        f3 origin, dir, power;
        live = photon_emit(p, photon_index, rng, origin, dir, power);
        if (live) {
            w.ro[i] = make_float4(origin.x, origin.y, origin.z, __uint_as_float(rng.state));
            w.rd[i] = make_float4(dir.x, dir.y, dir.z, __uint_as_float(photon_index));
            w.pw[i] = make_float4(power.x, power.y, power.z, __uint_as_float(0u));
        }
    }
    warp_append(live, i, w.queue[0], w.counts + 0);
}

__global__ void __launch_bounds__(128) ph_shade_kernel(const __grid_constant__ PhotonTraceParams p, const PhotonWave w,
                                                       uint32_t iter) {
    const uint32_t n = w.counts[4 * iter];
    const uint32_t *q = w.queue[iter & 1u];
    const bool last = iter + 1u >= RT_MAX_BOUNCES;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (n + stride - 1u) / stride;
    for (uint32_t r = 0; r < rounds; ++r) {
        const uint32_t item = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
        bool live = false;
        uint32_t slot = 0;
        if (item < n) {
            slot = q[item];
            const float2 h = w.hit[slot];
            const float4 d = w.rd[slot];
            const uint32_t photon_index = __float_as_uint(d.w);
            if (h.x < kInf) {
                const float4 o = w.ro[slot], pw = w.pw[slot];
                Rng rng;
                rng.state = __float_as_uint(o.w);
                f3 origin = xyz(o), dir = xyz(d), power = xyz(pw);
                live = photon_bounce(p, photon_index, iter, h.x, __float_as_uint(h.y), rng, origin, dir, power) && !last;
                if (live) {
                    w.ro[slot] = make_float4(origin.x, origin.y, origin.z, __uint_as_float(rng.state));
                    w.rd[slot] = make_float4(dir.x, dir.y, dir.z, d.w);
                    w.pw[slot] = make_float4(power.x, power.y, power.z, pw.w);
                }
            }
        }
        if (!last) warp_append(live, slot, w.queue[(iter + 1u) & 1u], w.counts + 4 * (iter + 1u));
    }
}

size_t photon_wave_bytes(uint32_t n) {
    return (size_t)n * (16 + 16 + 16 + 8 + 4 + 4) + sizeof(uint32_t) * 4 * (RT_MAX_BOUNCES + 1) + 64;
}

PhotonWave photon_wave_at(void *base, uint32_t n) {
    unsigned char *b = static_cast<unsigned char *>(base);
    PhotonWave w;
    w.ro = reinterpret_cast<float4 *>(b);
    w.rd = reinterpret_cast<float4 *>(b + 16ull * n);
    w.pw = reinterpret_cast<float4 *>(b + 32ull * n);
    w.hit = reinterpret_cast<float2 *>(b + 48ull * n);
    w.queue[0] = reinterpret_cast<uint32_t *>(b + 56ull * n);
    w.queue[1] = reinterpret_cast<uint32_t *>(b + 60ull * n);
    w.counts = reinterpret_cast<uint32_t *>(b + ((64ull * n + 15ull) & ~15ull));
    return w;
}

cudaError_t launch_photon_wave(const PhotonTraceParams &p, const PhotonWave &w, const DevJob *jobs_dev, int num_sms,
                               const WaveTuning &tune, cudaStream_t st) {
    if (p.photon_end <= p.photon_begin) return cudaSuccess;
    const uint32_t n = p.photon_end - p.photon_begin;
    cudaError_t e;
    if ((e = cudaMemsetAsync(w.counts, 0, sizeof(uint32_t) * 4 * (RT_MAX_BOUNCES + 1), st)) != cudaSuccess) return e;
    ph_generate_kernel<<<(n + 255u) / 256u, 256, 0, st>>>(p, w);
    WaveParams wp;
    std::memset(&wp, 0, sizeof(wp));
    wp.jobs = jobs_dev;
    wp.n_jobs = 1;
    wp.ro = w.ro;
    wp.rd = w.rd;
    wp.thr = w.pw;
    wp.hit = w.hit;
    wp.queue[0] = w.queue[0];
    wp.queue[1] = w.queue[1];
    wp.counts = w.counts;
    const uint64_t shade_needed = (n + 127u) / 128u, shade_cap = (uint64_t)num_sms * 8u;
    const uint32_t shade_grid = (uint32_t)(shade_needed < shade_cap ? shade_needed : shade_cap);
    for (uint32_t it = 0; it < RT_MAX_BOUNCES; ++it) {
        if ((e = launch_extend(wp, it, n, p.scene, num_sms, tune, st)) != cudaSuccess) return e;
        ph_shade_kernel<<<shade_grid, 128, 0, st>>>(p, w, it);
    }
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------------
// Keys of a host-provided photon buffer.
// ------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) photon_keys_kernel(const float4 *__restrict__ photons, uint64_t n,
                                                          const rt_grid_params gp, uint32_t *__restrict__ keys) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x) {
        float4 a = __ldg(photons + 4 * s), b = __ldg(photons + 4 * s + 1);
        keys[s] = slot_key(gp, xyz(a), b.x);
    }
}

int device_sm_count() {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
}
static int num_sms() { return device_sm_count(); }

cudaError_t launch_photon_keys(const float4 *photons, uint64_t slot_count, const rt_grid_params &gp, uint32_t *keys,
                               cudaStream_t st) {
    if (slot_count == 0) return cudaSuccess;
    uint64_t blocks = (slot_count + 255) / 256;
    uint64_t cap = (uint64_t)num_sms() * 8;
    photon_keys_kernel<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, st>>>(photons, slot_count, gp, keys);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------------
// Grid build
// ------------------------------------------------------------------------------------------------
// Four consecutive keys per thread (one 16-byte load when aligned and complete).
__device__ __forceinline__ uint4 load_keys4(const uint32_t *__restrict__ keys, uint64_t s, uint64_t n) {
    if (s + 3 < n) return __ldg(reinterpret_cast<const uint4 *>(keys + s));
    uint4 k = make_uint4(kInvalidKey, kInvalidKey, kInvalidKey, kInvalidKey);
    if (s < n) k.x = __ldg(keys + s);
    if (s + 1 < n) k.y = __ldg(keys + s + 1);
    if (s + 2 < n) k.z = __ldg(keys + s + 2);
    return k;
}

// Histogram: one reduction per valid key (no return value, so the adds do not hold the warp; keys of
// one warp rarely repeat, so merging lanes first costs more than it saves).
__global__ void __launch_bounds__(256) count_kernel(const uint32_t *__restrict__ keys, uint64_t n,
                                                    uint32_t *__restrict__ counts) {
    // eight keys per thread and pass, both 16-byte loads issued before the reductions
    const uint64_t stride = 8ull * gridDim.x * blockDim.x;
    const uint64_t start = 4ull * (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x);
    const uint64_t half = 4ull * gridDim.x * blockDim.x;
    const uint64_t rounds = (n + stride - 1) / stride;
    for (uint64_t r = 0; r < rounds; ++r) {
        const uint4 a = load_keys4(keys, start + r * stride, n);
        const uint4 b = load_keys4(keys, start + r * stride + half, n);
        const uint32_t kk[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (kk[j] != kInvalidKey) atomicAdd(counts + kk[j], 1u);
    }
}

// Slot indices to start[key] + cursor[key] (positions within a cell in atomic order; the order pass
// restores slot order).
__global__ void __launch_bounds__(256) scatter_kernel(const uint32_t *__restrict__ keys, uint64_t n,
                                                      const uint2 *__restrict__ meta, uint32_t *__restrict__ cursor,
                                                      uint32_t *__restrict__ order) {
    // eight keys per thread and pass: loads, then all atomics and meta reads, then the stores
    const uint64_t stride = 8ull * gridDim.x * blockDim.x;
    const uint64_t start = 4ull * (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x);
    const uint64_t half = 4ull * gridDim.x * blockDim.x;
    const uint64_t rounds = (n + stride - 1) / stride;
    for (uint64_t r = 0; r < rounds; ++r) {
        const uint64_t s0 = start + r * stride, s1 = s0 + half;
        const uint4 a = load_keys4(keys, s0, n);
        const uint4 b = load_keys4(keys, s1, n);
        const uint32_t kk[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        uint32_t pos[8];
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (kk[j] != kInvalidKey) pos[j] = atomicAdd(cursor + kk[j], 1u) + __ldg(&meta[kk[j]].x);
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (kk[j] != kInvalidKey) order[pos[j]] = (uint32_t)((j < 4 ? s0 : s1) + (j & 3));
    }
}

// Exclusive scan of counts into meta, three phases over tiles of kScanTile cells.
constexpr uint32_t kScanThreads = 256;
constexpr uint32_t kScanItems = 8;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;

uint32_t grid_scan_partials(uint32_t num_cells) { return (num_cells + kScanTile - 1) / kScanTile + 1; }

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *smem_warp, uint32_t *total) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31u) smem_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (kScanThreads / 32) ? smem_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= (uint32_t)o) w += y;
        }
        if (lane < (kScanThreads / 32)) smem_warp[lane] = w;
    }
    __syncthreads();
    uint32_t warp_prefix = warp ? smem_warp[warp - 1] : 0u;
    if (total) *total = smem_warp[kScanThreads / 32 - 1];
    return warp_prefix + x - v;
}

__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const uint32_t *__restrict__ counts, uint32_t n,
                                                                   uint32_t *__restrict__ partials) {
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const uint32_t base = blockIdx.x * kScanTile;
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t i = 0; i < kScanItems; ++i) {
        uint32_t c = base + i * kScanThreads + threadIdx.x;
        if (c < n) sum += __ldg(counts + c);
    }
    sum = __reduce_add_sync(0xFFFFFFFFu, sum);
    if ((threadIdx.x & 31u) == 0) warp_sums[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (uint32_t w = 0; w < kScanThreads / 32; ++w) t += warp_sums[w];
        partials[blockIdx.x] = t;
    }
}

// One block: exclusive scan of the tile sums in place; partials[ntiles] = grand total.
__global__ void __launch_bounds__(kScanThreads) scan_partials_kernel(uint32_t *partials, uint32_t ntiles,
                                                                     uint32_t *total_out) {
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    uint32_t carry = 0;
    for (uint32_t base = 0; base < ntiles; base += kScanThreads) {
        uint32_t i = base + threadIdx.x;
        uint32_t v = i < ntiles ? partials[i] : 0u;
        uint32_t tot = 0;
        uint32_t ex = block_exclusive_scan(v, warp_sums, &tot);
        if (i < ntiles) partials[i] = carry + ex;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[ntiles] = carry;
        if (total_out) *total_out = carry;
    }
}

// Rescan each tile with its offset; writes (start, count) per cell.  Items are blocked per thread
// (thread t owns cells t*8 .. t*8+7 of the tile, two 16-byte loads, four 16-byte stores) so the
// in-thread sums stay in cell order.
__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const uint32_t *__restrict__ counts, uint32_t n,
                                                                  const uint32_t *__restrict__ partials,
                                                                  uint2 *__restrict__ meta, bool vec) {
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    if (vec && base + kScanItems <= n) {
        const uint4 a = __ldg(reinterpret_cast<const uint4 *>(counts + base));
        const uint4 b = __ldg(reinterpret_cast<const uint4 *>(counts + base + 4));
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    } else {
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; ++i) v[i] = base + i < n ? __ldg(counts + base + i) : 0u;
    }
    uint32_t local = 0;
#pragma unroll
    for (uint32_t i = 0; i < kScanItems; ++i) local += v[i];
    uint32_t ex = block_exclusive_scan(local, warp_sums, nullptr) + __ldg(partials + blockIdx.x);
    uint32_t st[kScanItems];
#pragma unroll
    for (uint32_t i = 0; i < kScanItems; ++i) {
        st[i] = ex;
        ex += v[i];
    }
    if (vec && base + kScanItems <= n) {
        uint4 *m4 = reinterpret_cast<uint4 *>(meta + base);
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; i += 2) m4[i / 2] = make_uint4(st[i], v[i], st[i + 1], v[i + 1]);
    } else {
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; ++i)
            if (base + i < n) meta[base + i] = make_uint2(st[i], v[i]);
    }
}

// Ascending sort of one cell's slot indices.  Comparators always order (lower index, higher index)
// (the "flip" bitonic network), so positions past `count` act as +infinity and are never touched.
template <typename Seg>
__device__ __forceinline__ void warp_bitonic(Seg seg, uint32_t count, uint32_t lane) {
    uint32_t N = 1;
    while (N < count) N <<= 1;
    auto cas = [&](uint32_t a, uint32_t b) {
        if (b < count) {
            uint32_t x = seg[a], y = seg[b];
            if (x > y) {
                seg[a] = y;
                seg[b] = x;
            }
        }
    };
    for (uint32_t k = 2; k <= N; k <<= 1) {
        uint32_t hk = k >> 1;
        for (uint32_t i = lane; i < N / 2; i += 32) {
            uint32_t a = (i / hk) * k + (i % hk);
            uint32_t b = a ^ (k - 1);
            cas(a, b);
        }
        __syncwarp();
        for (uint32_t j = hk >> 1; j > 0; j >>= 1) {
            for (uint32_t i = lane; i < N / 2; i += 32) {
                uint32_t a = (i / j) * (2 * j) + (i % j);
                cas(a, a + j);
            }
            __syncwarp();
        }
    }
}

constexpr uint32_t kOrderWarps = 8;
constexpr uint32_t kOrderSmem = 1024;  // per-warp shared buffer (entries)

// Ascending bitonic sort of 32 * R values held R per lane (value e = lane * R + r).  Exchanges at
// distance j < R stay in the lane's registers; wider ones pair lanes lane ^ (j / R) by shuffle.
template <int R>
__device__ __forceinline__ void warp_sort_regs(uint32_t (&v)[R], uint32_t lane) {
#pragma unroll
    for (uint32_t k = 2; k <= 32u * R; k <<= 1) {
#pragma unroll
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            if (j >= (uint32_t)R) {
                const uint32_t lj = j / R;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const uint32_t e = lane * R + r;
                    const uint32_t o = __shfl_xor_sync(0xFFFFFFFFu, v[r], lj);
                    const bool up = (e & k) == 0u, lower = (e & j) == 0u;
                    v[r] = (lower == up) ? min(v[r], o) : max(v[r], o);
                }
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int q = r ^ (int)j;
                    if (q > r) {
                        const uint32_t e = lane * R + r;
                        const bool up = (e & k) == 0u;
                        const uint32_t a = v[r], b = v[q];
                        v[r] = up ? min(a, b) : max(a, b);
                        v[q] = up ? max(a, b) : min(a, b);
                    }
                }
            }
        }
    }
}

// Sorts the cell's `count` (<= 32 R) slot indices order[start ..], in place or (out != null) into out.
template <int R>
__device__ __forceinline__ void sort_cell_regs(uint32_t *__restrict__ order, uint32_t start, uint32_t count,
                                               uint32_t lane, uint32_t *out = nullptr) {
    uint32_t v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t e = lane * R + r;
        v[r] = e < count ? order[start + e] : 0xFFFFFFFFu;
    }
    warp_sort_regs<R>(v, lane);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t e = lane * R + r;
        if (e < count) {
            if (out) out[e] = v[r];
            else order[start + e] = v[r];
        }
    }
}

// Cells holding two or more photons, appended to `list` (two cells per 16-byte meta load).
__global__ void __launch_bounds__(256) multi_cells_kernel(const uint2 *__restrict__ meta, uint32_t n_cells,
                                                          uint32_t *__restrict__ list, uint32_t *__restrict__ n_list,
                                                          bool vec) {
    // four cells per thread and pass (two 16-byte meta loads in flight)
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t n_quads = (n_cells + 3u) / 4u;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (n_quads + stride - 1) / stride;
    for (uint32_t r = 0; r < rounds; ++r) {
        const uint32_t c0 = 4u * (r * stride + blockIdx.x * blockDim.x + threadIdx.x);
        uint32_t cnt[4] = {0u, 0u, 0u, 0u};
        if (vec && c0 + 3u < n_cells) {
            const uint4 m0 = __ldg(reinterpret_cast<const uint4 *>(meta + c0));
            const uint4 m1 = __ldg(reinterpret_cast<const uint4 *>(meta + c0 + 2u));
            cnt[0] = m0.y;
            cnt[1] = m0.w;
            cnt[2] = m1.y;
            cnt[3] = m1.w;
        } else {
#pragma unroll
            for (uint32_t j = 0; j < 4u; ++j)
                if (c0 + j < n_cells) cnt[j] = __ldg(&meta[c0 + j].y);
        }
        uint32_t masks[4], tot = 0;
#pragma unroll
        for (uint32_t j = 0; j < 4u; ++j) {
            masks[j] = __ballot_sync(0xFFFFFFFFu, cnt[j] > 1u);
            tot += __popc(masks[j]);
        }
        if (tot == 0u) continue;
        uint32_t base = 0;
        if (lane == 0u) base = atomicAdd(n_list, tot);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        const uint32_t lt = lanemask_lt();
#pragma unroll
        for (uint32_t j = 0; j < 4u; ++j) {
            if (cnt[j] > 1u) list[base + __popc(masks[j] & lt)] = c0 + j;
            base += __popc(masks[j]);
        }
    }
}

// One warp per listed cell: the cell's slot indices (in atomic order after the scatter) sorted
// ascending, so photons of a cell keep slot order, as a sequential scatter would leave them.
__global__ void __launch_bounds__(kOrderWarps * 32) order_kernel(const uint2 *__restrict__ meta,
                                                                  const uint32_t *__restrict__ list,
                                                                  const uint32_t *__restrict__ n_list,
                                                                  uint32_t *__restrict__ order) {
    __shared__ uint32_t buf[kOrderWarps][kOrderSmem];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const uint32_t warps_total = gridDim.x * kOrderWarps;
    const uint32_t n = *n_list;
    for (uint32_t li = blockIdx.x * kOrderWarps + w; li < n; li += warps_total) {
        const uint2 m = __ldg(meta + __ldg(list + li));
        const uint32_t start = m.x, count = m.y;
        if (count <= 1u) continue;
        if (count <= 32u) {
            sort_cell_regs<1>(order, start, count, lane);
        } else if (count <= 64u) {
            sort_cell_regs<2>(order, start, count, lane);
        } else if (count <= 128u) {
            sort_cell_regs<4>(order, start, count, lane);
        } else if (count <= 256u) {
            sort_cell_regs<8>(order, start, count, lane);
        } else if (count <= kOrderSmem) {
            uint32_t *sb = buf[w];
            for (uint32_t i = lane; i < count; i += 32) sb[i] = order[start + i];
            __syncwarp();
            warp_bitonic(sb, count, lane);
            for (uint32_t i = lane; i < count; i += 32) order[start + i] = sb[i];
            __syncwarp();
        } else {
            warp_bitonic(order + start, count, lane);
        }
    }
}

struct Photon8 {
    float v[16];
};

// 64 bytes as two 32-byte accesses (the records are 64-byte aligned when `wide`).  The L2 fetch size
// is held to 64 bytes: a record's neighbour in its 128-byte line belongs to another cell, and fetching
// whole lines made the per-cell copy read 1.7x the photon bytes it needs from DRAM.
__device__ __forceinline__ void load_photon_wide(const float4 *src, Photon8 &p) {
    const float *f = reinterpret_cast<const float *>(src);
    asm volatile("ld.global.nc.L2::64B.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(p.v[0]), "=f"(p.v[1]), "=f"(p.v[2]), "=f"(p.v[3]), "=f"(p.v[4]), "=f"(p.v[5]), "=f"(p.v[6]),
                   "=f"(p.v[7])
                 : "l"(f));
    asm volatile("ld.global.nc.L2::64B.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(p.v[8]), "=f"(p.v[9]), "=f"(p.v[10]), "=f"(p.v[11]), "=f"(p.v[12]), "=f"(p.v[13]),
                   "=f"(p.v[14]), "=f"(p.v[15])
                 : "l"(f + 8));
}

__device__ __forceinline__ void store_photon_wide(float4 *dst, const Photon8 &p) {
    float *f = reinterpret_cast<float *>(dst);
    asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(f), "f"(p.v[0]), "f"(p.v[1]), "f"(p.v[2]),
                 "f"(p.v[3]), "f"(p.v[4]), "f"(p.v[5]), "f"(p.v[6]), "f"(p.v[7])
                 : "memory");
    asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(f + 8), "f"(p.v[8]), "f"(p.v[9]),
                 "f"(p.v[10]), "f"(p.v[11]), "f"(p.v[12]), "f"(p.v[13]), "f"(p.v[14]), "f"(p.v[15])
                 : "memory");
}

// sorted[i] = photons[order[i]] for i < total, two photons per thread with both records loaded
// before the stores; 32-byte accesses when both buffers are 32-byte aligned (`wide`).  sorted_pos,
// when given, gets each photon's first float4.
__global__ void __launch_bounds__(256) photon_gather_kernel(const float4 *__restrict__ photons,
                                                            const uint32_t *__restrict__ order,
                                                            const uint32_t *__restrict__ total, uint64_t cap,
                                                            float4 *__restrict__ sorted,
                                                            float4 *__restrict__ sorted_pos, bool wide) {
    const uint64_t n = min((uint64_t)__ldg(total), cap);
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += 2 * step) {
        const uint64_t i2 = i + step;
        const bool two = i2 < n;
        const float4 *s0 = photons + 4ull * __ldg(order + i);
        const float4 *s1 = photons + 4ull * __ldg(order + (two ? i2 : i));
        if (wide) {
            Photon8 a, b;
            load_photon_wide(s0, a);
            load_photon_wide(s1, b);
            store_photon_wide(sorted + 4ull * i, a);
            if (sorted_pos) sorted_pos[i] = make_float4(a.v[0], a.v[1], a.v[2], a.v[3]);
            if (two) {
                store_photon_wide(sorted + 4ull * i2, b);
                if (sorted_pos) sorted_pos[i2] = make_float4(b.v[0], b.v[1], b.v[2], b.v[3]);
            }
        } else {
            const float4 a = __ldg(s0), b = __ldg(s0 + 1), c = __ldg(s0 + 2), d = __ldg(s0 + 3);
            const float4 e = __ldg(s1), f = __ldg(s1 + 1), g = __ldg(s1 + 2), h = __ldg(s1 + 3);
            float4 *d0 = sorted + 4ull * i;
            d0[0] = a;
            d0[1] = b;
            d0[2] = c;
            d0[3] = d;
            if (sorted_pos) sorted_pos[i] = a;
            if (two) {
                float4 *d1 = sorted + 4ull * i2;
                d1[0] = e;
                d1[1] = f;
                d1[2] = g;
                d1[3] = h;
                if (sorted_pos) sorted_pos[i2] = e;
            }
        }
    }
}

// ---- grid build with per-slot ranks ---------------------------------------------------------------
// The kernels after the count are launched as programmatic dependents of the one before (their blocks
// may be scheduled while it finishes and wait for it in grid_dependency_wait).

// Histogram with ranks: counts[key] += 1 and rank[slot] = the count found before the add (the slot's
// position within its cell, in atomic order).
__global__ void __launch_bounds__(256) count_rank_kernel(const uint32_t *__restrict__ keys, uint64_t n,
                                                         uint32_t *__restrict__ counts, uint32_t *__restrict__ rank,
                                                         uint32_t *__restrict__ clear, uint32_t n_clear,
                                                         uint32_t *__restrict__ n_list) {
    grid_launch_dependents();
    // the scan's chunk status words and ticket, and its count of listed cells, start at zero (this
    // launch precedes the scan)
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_clear; i += gridDim.x * blockDim.x) clear[i] = 0u;
    if (blockIdx.x == 0 && threadIdx.x == 0) *n_list = 0u;
    // eight keys per thread and pass (two 16-byte loads in flight), then the adds, then the ranks
    const uint64_t stride = 8ull * gridDim.x * blockDim.x;
    const uint64_t start = 4ull * (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x);
    const uint64_t half = 4ull * gridDim.x * blockDim.x;
    const uint64_t rounds = (n + stride - 1) / stride;
    for (uint64_t r = 0; r < rounds; ++r) {
        const uint64_t s0 = start + r * stride, s1 = s0 + half;
        const uint4 a = load_keys4(keys, s0, n);
        const uint4 b = load_keys4(keys, s1, n);
        const uint32_t kk[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        uint32_t rk[8];
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (kk[j] != kInvalidKey) rk[j] = atomicAdd(counts + kk[j], 1u);
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (kk[j] != kInvalidKey) rank[(j < 4 ? s0 : s1) + (j & 3)] = rk[j];
    }
}

// scan_apply plus the list of occupied cells (count >= 1), appended with one atomic per warp.
__global__ void __launch_bounds__(kScanThreads) scan_apply_list_kernel(const uint32_t *__restrict__ counts, uint32_t n,
                                                                       const uint32_t *__restrict__ partials,
                                                                       uint2 *__restrict__ meta, bool vec,
                                                                       uint32_t *__restrict__ list,
                                                                       uint32_t *__restrict__ n_list) {
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    if (vec && base + kScanItems <= n) {
        const uint4 a = __ldg(reinterpret_cast<const uint4 *>(counts + base));
        const uint4 b = __ldg(reinterpret_cast<const uint4 *>(counts + base + 4));
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    } else {
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; ++i) v[i] = base + i < n ? __ldg(counts + base + i) : 0u;
    }
    uint32_t local = 0, occ = 0;
#pragma unroll
    for (uint32_t i = 0; i < kScanItems; ++i) {
        local += v[i];
        occ += v[i] ? 1u : 0u;
    }
    uint32_t ex = block_exclusive_scan(local, warp_sums, nullptr) + __ldg(partials + blockIdx.x);
    uint32_t st[kScanItems];
#pragma unroll
    for (uint32_t i = 0; i < kScanItems; ++i) {
        st[i] = ex;
        ex += v[i];
    }
    if (vec && base + kScanItems <= n) {
        uint4 *m4 = reinterpret_cast<uint4 *>(meta + base);
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; i += 2) m4[i / 2] = make_uint4(st[i], v[i], st[i + 1], v[i + 1]);
    } else {
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; ++i)
            if (base + i < n) meta[base + i] = make_uint2(st[i], v[i]);
    }
    // warp-exclusive offsets of the occupied cells, one atomic per warp
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t x = occ;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    const uint32_t warp_total = __shfl_sync(0xFFFFFFFFu, x, 31);
    uint32_t wbase = 0;
    if (lane == 0u && warp_total) wbase = atomicAdd(n_list, warp_total);
    wbase = __shfl_sync(0xFFFFFFFFu, wbase, 0) + x - occ;
#pragma unroll
    for (uint32_t i = 0; i < kScanItems; ++i)
        if (v[i]) list[wbase++] = base + i;
}

// Single-pass exclusive scan of counts into (start, count) with decoupled look-back (Merrill and
// Garland, "Single-pass Parallel Prefix Scan with Decoupled Look-back", 2016), plus the list of
// occupied cells.  Each block owns a chunk of CT consecutive tiles of kScanTile cells: it loads and
// sums the chunk's counts (kept in registers), publishes one status word -- flag in bits 30-31 (1: the chunk's own sum,
// 2: the sum of all chunks up to and including it), value in bits 0-29 -- and warp 0 reads back 32
// predecessors at a time until it meets an inclusive sum; then the block scans its tiles with that
// prefix and writes (start, count).  Chunks are numbered by a ticket
// taken when the block starts, so every chunk a block waits on belongs to a block already running:
// the waits end.  They are bounded all the same (2^20 polls, then the block counts the timeout in
// g_scan_timeouts and uses the sums it has).  Values must stay below 2^30 (the host checks the slot
// count).
constexpr uint32_t kScanFlagAgg = 1u << 30, kScanFlagIncl = 2u << 30, kScanValMask = (1u << 30) - 1u;
__device__ unsigned int g_scan_timeouts = 0u;

__device__ __forceinline__ void load_counts8(const uint32_t *counts, uint32_t base, uint32_t n, bool vec,
                                             uint32_t (&v)[kScanItems]) {
    if (vec && base + kScanItems <= n) {
        const uint4 a = *reinterpret_cast<const uint4 *>(counts + base);
        const uint4 b = *reinterpret_cast<const uint4 *>(counts + base + 4);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    } else {
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; ++i) v[i] = base + i < n ? counts[base + i] : 0u;
    }
}

template <int CT>
__global__ void __launch_bounds__(kScanThreads) scan_lookback_list_kernel(uint32_t *__restrict__ counts,
                                                                          uint32_t n, uint32_t *status,
                                                                          uint32_t chunks, uint2 *__restrict__ meta,
                                                                          bool vec, uint32_t *__restrict__ list,
                                                                          uint32_t *__restrict__ n_list,
                                                                          uint32_t *__restrict__ total_out) {
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    __shared__ uint32_t s_chunk, s_prefix;
    grid_dependency_wait();
    grid_launch_dependents();
    if (threadIdx.x == 0) s_chunk = atomicAdd(status + chunks, 1u);
    __syncthreads();
    const uint32_t chunk = s_chunk;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t tile0 = chunk * CT;
    // the chunk's counts (all loads in flight at once, kept for the rescan) and their sum
    uint32_t v[CT][kScanItems];
#pragma unroll
    for (int t = 0; t < CT; ++t) load_counts8(counts, (tile0 + t) * kScanTile + threadIdx.x * kScanItems, n, vec, v[t]);
    uint32_t part = 0;
#pragma unroll
    for (int t = 0; t < CT; ++t)
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; ++i) part += v[t][i];
    part = __reduce_add_sync(0xFFFFFFFFu, part);
    if (lane == 0u) warp_sums[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x < 32u) {
        uint32_t chunk_total = lane < kScanThreads / 32 ? warp_sums[lane] : 0u;
        chunk_total = __reduce_add_sync(0xFFFFFFFFu, chunk_total);
        volatile uint32_t *vs = status;
        uint32_t prefix = 0;
        if (chunk == 0u) {
            if (lane == 0u) vs[0] = kScanFlagIncl | chunk_total;
        } else {
            if (lane == 0u) vs[chunk] = kScanFlagAgg | chunk_total;
            int64_t window = (int64_t)chunk - 1;  // predecessor read by lane 0
            uint32_t polls = 0;
            bool timed_out = false;
            for (;;) {
                const int64_t idx = window - (int64_t)lane;
                uint32_t sw = kScanFlagIncl;
                if (idx >= 0) sw = vs[idx];
                while (__any_sync(0xFFFFFFFFu, (sw >> 30) == 0u)) {
                    if (++polls >= (1u << 20)) {
                        timed_out = true;
                        break;
                    }
                    if ((sw >> 30) == 0u) sw = vs[idx];
                }
                if (timed_out) break;
                const uint32_t incl = __ballot_sync(0xFFFFFFFFu, (sw >> 30) == 2u);
                // lanes up to the nearest inclusive predecessor (lowest lane) contribute
                const uint32_t upto = incl ? (uint32_t)(__ffs(incl) - 1) : 31u;
                prefix += __reduce_add_sync(0xFFFFFFFFu, lane <= upto ? (sw & kScanValMask) : 0u);
                if (incl) break;
                window -= 32;
            }
            if (timed_out && lane == 0u) atomicAdd(&g_scan_timeouts, 1u);
            if (lane == 0u) vs[chunk] = kScanFlagIncl | ((prefix + chunk_total) & kScanValMask);
        }
        if (lane == 0u) {
            s_prefix = prefix;
            if (chunk == chunks - 1u && total_out) *total_out = prefix + chunk_total;
        }
    }
    __syncthreads();
    uint32_t carry = s_prefix;
#pragma unroll
    for (int t = 0; t < CT; ++t) {
        const uint32_t base = (tile0 + t) * kScanTile + threadIdx.x * kScanItems;
        uint32_t local = 0, occ = 0;
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; ++i) {
            local += v[t][i];
            occ += v[t][i] ? 1u : 0u;
        }
        uint32_t tile_total = 0;
        uint32_t ex = block_exclusive_scan(local, warp_sums, &tile_total) + carry;
        carry += tile_total;
        uint32_t st[kScanItems];
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; ++i) {
            st[i] = ex;
            ex += v[t][i];
        }
        // (start, count) written; the counts are cleared for the next build (meta keeps them)
        if (vec && base + kScanItems <= n) {
            uint4 *m4 = reinterpret_cast<uint4 *>(meta + base);
#pragma unroll
            for (uint32_t i = 0; i < kScanItems; i += 2)
                m4[i / 2] = make_uint4(st[i], v[t][i], st[i + 1], v[t][i + 1]);
            reinterpret_cast<uint4 *>(counts + base)[0] = make_uint4(0u, 0u, 0u, 0u);
            reinterpret_cast<uint4 *>(counts + base)[1] = make_uint4(0u, 0u, 0u, 0u);
        } else {
#pragma unroll
            for (uint32_t i = 0; i < kScanItems; ++i)
                if (base + i < n) {
                    meta[base + i] = make_uint2(st[i], v[t][i]);
                    counts[base + i] = 0u;
                }
        }
        // warp-exclusive offsets of the occupied cells, one atomic per warp
        uint32_t x = occ;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        const uint32_t warp_total = __shfl_sync(0xFFFFFFFFu, x, 31);
        uint32_t wbase = 0;
        if (lane == 0u && warp_total) wbase = atomicAdd(n_list, warp_total);
        wbase = __shfl_sync(0xFFFFFFFFu, wbase, 0) + x - occ;
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; ++i)
            if (v[t][i]) list[wbase++] = base + i;
        __syncthreads();  // warp_sums is reused by the next tile's scan
    }
}

uint32_t scan_timeouts() {
    unsigned int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_scan_timeouts, sizeof(v)) != cudaSuccess) return 0xFFFFFFFFu;
    return v;
}

// order[start[key] + rank[slot]] = slot: positions come from the ranks, no atomics.
__global__ void __launch_bounds__(256) scatter_rank_kernel(const uint32_t *__restrict__ keys,
                                                           const uint32_t *__restrict__ rank, uint64_t n,
                                                           const uint2 *__restrict__ meta,
                                                           uint32_t *__restrict__ order) {
    grid_dependency_wait();
    grid_launch_dependents();
    // eight keys per thread and pass (two 16-byte loads in flight), then the starts and ranks, then the
    // stores
    const uint64_t stride = 8ull * gridDim.x * blockDim.x;
    const uint64_t start = 4ull * (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x);
    const uint64_t half = 4ull * gridDim.x * blockDim.x;
    const uint64_t rounds = (n + stride - 1) / stride;
    for (uint64_t r = 0; r < rounds; ++r) {
        const uint64_t s0 = start + r * stride, s1 = s0 + half;
        const uint4 a = load_keys4(keys, s0, n);
        const uint4 b = load_keys4(keys, s1, n);
        const uint32_t kk[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        uint32_t pos[8];
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (kk[j] != kInvalidKey) pos[j] = __ldg(&meta[kk[j]].x) + __ldg(rank + (j < 4 ? s0 : s1) + (j & 3));
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (kk[j] != kInvalidKey) order[pos[j]] = (uint32_t)((j < 4 ? s0 : s1) + (j & 3));
    }
}

// Copies photon records order-sorted: sorted[dst] = photons[slot] (64 B) and sorted_pos[dst] = its first
// float4.  Two records per call with both loads issued before the stores.
__device__ __forceinline__ void copy_photon_pair(const float4 *__restrict__ photons, uint32_t s0, uint32_t s1, bool two,
                                                 float4 *__restrict__ sorted, float4 *__restrict__ sorted_pos,
                                                 uint64_t d0, uint64_t d1, bool wide) {
    if (wide) {
        Photon8 a, b;
        load_photon_wide(photons + 4ull * s0, a);
        if (two) load_photon_wide(photons + 4ull * s1, b);
        store_photon_wide(sorted + 4ull * d0, a);
        if (sorted_pos) sorted_pos[d0] = make_float4(a.v[0], a.v[1], a.v[2], a.v[3]);
        if (two) {
            store_photon_wide(sorted + 4ull * d1, b);
            if (sorted_pos) sorted_pos[d1] = make_float4(b.v[0], b.v[1], b.v[2], b.v[3]);
        }
    } else {
        const float4 *p0 = photons + 4ull * s0, *p1 = photons + 4ull * (two ? s1 : s0);
        const float4 a = __ldg(p0), b = __ldg(p0 + 1), c = __ldg(p0 + 2), d = __ldg(p0 + 3);
        const float4 e = __ldg(p1), f = __ldg(p1 + 1), g = __ldg(p1 + 2), h = __ldg(p1 + 3);
        float4 *q0 = sorted + 4ull * d0;
        q0[0] = a;
        q0[1] = b;
        q0[2] = c;
        q0[3] = d;
        if (sorted_pos) sorted_pos[d0] = a;
        if (two) {
            float4 *q1 = sorted + 4ull * d1;
            q1[0] = e;
            q1[1] = f;
            q1[2] = g;
            q1[3] = h;
            if (sorted_pos) sorted_pos[d1] = e;
        }
    }
}

// Copies a cell's records in slot order: sorted[start + i] = photons[src[i]], i < count, two records
// per lane and round (lanes i and i + 32).
__device__ __forceinline__ void copy_cell(const uint32_t *src, uint32_t start, uint32_t count, uint32_t lane,
                                          const float4 *__restrict__ photons, float4 *__restrict__ sorted,
                                          float4 *__restrict__ sorted_pos, bool wide) {
    for (uint32_t i = lane; i < count; i += 64) {
        const bool two = i + 32 < count;
        copy_photon_pair(photons, src[i], two ? src[i + 32] : 0u, two, sorted, sorted_pos, (uint64_t)start + i,
                         (uint64_t)start + i + 32, wide);
    }
}

// The slot indices of one cell of at most 32 R photons (atomic order, from the scatter) sorted
// ascending in registers into the warp's shared buffer.
template <int R>
__device__ __forceinline__ void sort_cell_to(const uint32_t *__restrict__ order, uint32_t start, uint32_t count,
                                             uint32_t lane, uint32_t *buf) {
    uint32_t v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t e = lane * R + r;
        v[r] = e < count ? __ldg(order + start + e) : 0xFFFFFFFFu;
    }
    if (count > 1u) warp_sort_regs<R>(v, lane);
#pragma unroll
    for (int r = 0; r < R; ++r) buf[lane * R + r] = v[r];
}

constexpr uint32_t kCellRegsMax = 256;  // cells up to this size are sorted in registers

// Per-cell slot order fused with the photon gather: one warp per listed (occupied) cell sorts the
// cell's slot indices ascending -- photons of a cell keep slot order, as a sequential scatter would
// leave them -- and copies the cell's records into sorted order.  Cells of more than 256 photons are
// sorted in place in `order`, then copied from there.
__global__ void __launch_bounds__(kOrderWarps * 32, 4) cell_gather_kernel(const uint2 *__restrict__ meta,
                                                                       const uint32_t *__restrict__ list,
                                                                       const uint32_t *__restrict__ n_list,
                                                                       uint32_t *__restrict__ order,
                                                                       const float4 *__restrict__ photons,
                                                                       float4 *__restrict__ sorted,
                                                                       float4 *__restrict__ sorted_pos, bool wide) {
    __shared__ uint32_t sbuf[kOrderWarps][kCellRegsMax];
    grid_dependency_wait();
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    uint32_t *buf = sbuf[w];
    const uint32_t warps_total = gridDim.x * kOrderWarps;
    const uint32_t n = *n_list;
    for (uint32_t li = blockIdx.x * kOrderWarps + w; li < n; li += warps_total) {
        const uint2 m = __ldg(meta + __ldg(list + li));
        const uint32_t start = m.x, count = m.y;
        if (count == 0u) continue;
        const uint32_t *src = buf;
        if (count <= 32u) {
            sort_cell_to<1>(order, start, count, lane, buf);
        } else if (count <= 64u) {
            sort_cell_to<2>(order, start, count, lane, buf);
        } else if (count <= 128u) {
            sort_cell_to<4>(order, start, count, lane, buf);
        } else if (count <= kCellRegsMax) {
            sort_cell_to<8>(order, start, count, lane, buf);
        } else {
            warp_bitonic(order + start, count, lane);
            src = order + start;
        }
        __syncwarp();
        copy_cell(src, start, count, lane, photons, sorted, sorted_pos, wide);
        __syncwarp();
    }
}

// Launches `kernel` as a programmatic dependent of the previous kernel in the stream: its blocks may
// be scheduled before that kernel has finished and wait for it in grid_dependency_wait().
template <typename... KArgs, typename... Args>
static cudaError_t launch_dependent(void (*kernel)(KArgs...), unsigned grid, unsigned block, cudaStream_t st,
                                    Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

cudaError_t launch_grid_build(const GridBuffers &g, cudaStream_t st) {
    cudaError_t e;
    const uint32_t C = g.num_cells;
    const uint64_t n = g.slot_count;
    const uint32_t sm = (uint32_t)num_sms();
    auto grid_for = [&](uint64_t items, uint32_t block, uint32_t per_sm) {
        uint64_t b = (items + block - 1) / block;
        uint64_t cap = (uint64_t)sm * per_sm;
        return (unsigned)(b < 1 ? 1 : (b < cap ? b : cap));
    };
    // 16-byte vector access to counts / meta, 32-byte photon copies, when the buffers allow it
    const bool vec = (reinterpret_cast<uintptr_t>(g.counts) % 16u) == 0u && (reinterpret_cast<uintptr_t>(g.meta) % 16u) == 0u;
    const bool wide = ((reinterpret_cast<uintptr_t>(g.photons) | reinterpret_cast<uintptr_t>(g.sorted)) % 32u) == 0u;
    const uint32_t tiles = (C + kScanTile - 1) / kScanTile;
    if (g.rank) {
        // One scan pass with decoupled look-back while every value fits its 30 bits, else the three
        // phases.  Chunks of up to four tiles, about two chunks per SM; the look-back's chunk status
        // words and ticket (scan_partials[0 .. chunks], chunks <= tiles) and the count of occupied cells
        // (total[1]; the cells are listed in the cursor array, which this path does not otherwise need)
        // are cleared by the count launch.  The counts are zero on entry: cleared when the renderer is
        // created and by the scan of every build once it has turned them into (start, count).
        const bool lookback = n && n < (uint64_t)kScanValMask;
        const uint32_t want = (tiles + 2 * sm - 1) / (2 * sm);
        const uint32_t ct = want <= 1u ? 1u : (want <= 2u ? 2u : 4u);
        const uint32_t chunks = (tiles + ct - 1) / ct;
        if (!lookback) {
            if ((e = cudaMemsetAsync(g.counts, 0, (size_t)C * 4, st)) != cudaSuccess) return e;
            if ((e = cudaMemsetAsync(g.total + 1, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
            if (n) count_rank_kernel<<<grid_for((n + 7) / 8, 256, 8), 256, 0, st>>>(g.keys, n, g.counts, g.rank, nullptr,
                                                                                    0u, g.total + 1);
            scan_reduce_kernel<<<tiles, kScanThreads, 0, st>>>(g.counts, C, g.scan_partials);
            scan_partials_kernel<<<1, kScanThreads, 0, st>>>(g.scan_partials, tiles, g.total);
            scan_apply_list_kernel<<<tiles, kScanThreads, 0, st>>>(g.counts, C, g.scan_partials, g.meta, vec, g.cursor,
                                                                   g.total + 1);
            if ((e = cudaMemsetAsync(g.counts, 0, (size_t)C * 4, st)) != cudaSuccess) return e;
            if (n) {
                scatter_rank_kernel<<<grid_for((n + 7) / 8, 256, 8), 256, 0, st>>>(g.keys, g.rank, n, g.meta, g.order);
                cell_gather_kernel<<<grid_for((uint64_t)C * 32, kOrderWarps * 32, 4), kOrderWarps * 32, 0, st>>>(
                    g.meta, g.cursor, g.total + 1, g.order, g.photons, g.sorted, g.sorted_pos, wide);
            }
            return cudaGetLastError();
        }
        count_rank_kernel<<<grid_for((n + 7) / 8, 256, 8), 256, 0, st>>>(g.keys, n, g.counts, g.rank, g.scan_partials,
                                                                         chunks + 1, g.total + 1);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if (ct == 1u)
            e = launch_dependent(scan_lookback_list_kernel<1>, chunks, kScanThreads, st, g.counts, C, g.scan_partials,
                                 chunks, g.meta, vec, g.cursor, g.total + 1, g.total);
        else if (ct == 2u)
            e = launch_dependent(scan_lookback_list_kernel<2>, chunks, kScanThreads, st, g.counts, C, g.scan_partials,
                                 chunks, g.meta, vec, g.cursor, g.total + 1, g.total);
        else
            e = launch_dependent(scan_lookback_list_kernel<4>, chunks, kScanThreads, st, g.counts, C, g.scan_partials,
                                 chunks, g.meta, vec, g.cursor, g.total + 1, g.total);
        if (e != cudaSuccess) return e;
        if ((e = launch_dependent(scatter_rank_kernel, grid_for((n + 7) / 8, 256, 8), 256, st, g.keys,
                                  (const uint32_t *)g.rank, n, (const uint2 *)g.meta, g.order)) != cudaSuccess)
            return e;
        return launch_dependent(cell_gather_kernel, grid_for((uint64_t)C * 32, kOrderWarps * 32, 4), kOrderWarps * 32, st,
                                (const uint2 *)g.meta, (const uint32_t *)g.cursor, (const uint32_t *)(g.total + 1),
                                g.order, g.photons, g.sorted, g.sorted_pos, wide);
    }
    if ((e = cudaMemsetAsync(g.counts, 0, (size_t)C * 4, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(g.cursor, 0, (size_t)C * 4, st)) != cudaSuccess) return e;
    if (n) {
        count_kernel<<<grid_for((n + 7) / 8, 256, 8), 256, 0, st>>>(g.keys, n, g.counts);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    scan_reduce_kernel<<<tiles, kScanThreads, 0, st>>>(g.counts, C, g.scan_partials);
    scan_partials_kernel<<<1, kScanThreads, 0, st>>>(g.scan_partials, tiles, g.total);
    scan_apply_kernel<<<tiles, kScanThreads, 0, st>>>(g.counts, C, g.scan_partials, g.meta, vec);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (n) {
        scatter_kernel<<<grid_for((n + 7) / 8, 256, 8), 256, 0, st>>>(g.keys, n, g.meta, g.cursor, g.order);
        // The cells to order are listed in the cursor array (the cursors are spent after the scatter);
        // the list length is total[1].
        if ((e = cudaMemsetAsync(g.total + 1, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
        multi_cells_kernel<<<grid_for((C + 3) / 4, 256, 8), 256, 0, st>>>(g.meta, C, g.cursor, g.total + 1, vec);
        order_kernel<<<grid_for((uint64_t)C * 32, kOrderWarps * 32, 8), kOrderWarps * 32, 0, st>>>(g.meta, g.cursor,
                                                                                                g.total + 1, g.order);
        photon_gather_kernel<<<grid_for((n + 1) / 2, 256, 8), 256, 0, st>>>(g.photons, g.order, g.total, n, g.sorted,
                                                                              g.sorted_pos, wide);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace rtd
