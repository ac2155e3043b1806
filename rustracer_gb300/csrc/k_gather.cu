// The gather pass: one thread per pixel, the spp loop and up to max_bounces segments per sample with
// next-event estimation, GGX / dielectric lobes, the photon-map lookup, Russian roulette and the
// firefly sigma clamp.  Restates rustracer-renderer/shaders/gather.wgsl:30-594 for sm_103a.
//
// Launch shape: 8 x 8 pixel blocks (two warps of 8 x 4 pixels, for ray coherence); traversal stacks
// in shared memory, one 4-byte column per thread (bank-conflict free); BVH nodes and triangle vertices
// fetched as 16-byte read-only vector loads.  Path segments (closest-hit traces on camera / bounce
// paths) and shadow rays are counted per warp and added once per warp to 64-bit counters.
#include "rt_device.cuh"
#include "rt_kernels.h"

namespace rtd {

namespace {

__device__ __forceinline__ float luma(f3 c) { return dot(c, mk3(0.2126f, 0.7152f, 0.0722f)); }

struct Accum {
    f3 col;
    float lum_sum, lum2_sum;
    float sample_lum[8];
};
__device__ __forceinline__ void add_radiance(uint32_t s, Accum &a, f3 c) {
    a.col = a.col + c;
    float l = luma(c);
    a.lum_sum += l;
    a.lum2_sum += l * l;
    if (s < 8u) a.sample_lum[s] += l;
}

__device__ __forceinline__ f3 sky_color(f3 dir, f3 zenith, f3 horizon, float intensity) {
    float t = clampf(dir.y * 0.5f + 0.5f, 0.0f, 1.0f);
    return mix3(horizon, zenith, powf(t, 0.5f)) * intensity;
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
    float x = r * cosf(phi);
    float y = r * sinf(phi);
    float s = 0.5f * (1.0f + vh.z);
    float yy = (1.0f - s) * sqrtf(fmaxf(0.0f, 1.0f - x * x)) + s * y;
    f3 hh = x * t1 + yy * t2 + sqrtf(fmaxf(0.0f, 1.0f - x * x - yy * yy)) * vh;
    f3 hn = normalize(hh);
    f3 m = bt * hn.x + bb * hn.y + n * hn.z;
    f3 out = reflect(rd, m);
    return dot(out, n) > 0.0f ? out : reflect(rd, n);
}

struct Ctx {
    const GatherParams &p;
    uint32_t *stk;
    uint32_t stride;
    uint32_t shadow_rays;
};

// gather.wgsl:91-103
__device__ __forceinline__ bool shadowed(Ctx &c, f3 origin, f3 dir, float max_dist) {
    c.shadow_rays += 1u;
    const DevScene &s = c.p.scene;
    Hit sh = trace_bvh<64>(s, origin, dir, c.stk, c.stride);
    if (sh.t >= max_dist - 0.001f) return false;
    TriFull bt = load_tri(s, sh.prim);
    Mat bm = load_mat(s, bt.material_id);
    if ((bm.flags & RT_MAT_FLAG_ALPHA_CUTOUT) != 0u && bm.tex_albedo != RT_TEX_NONE) {
        Bary b = barycentric(bt, origin, dir, sh.t);
        float alpha = tex_sample(s.tex[RT_TEX_ALBEDO], b.uvx, b.uvy, (int32_t)bm.tex_albedo).w;
        if (alpha < 0.5f) return false;
    }
    return true;
}

struct LightSample {
    f3 e, wi;
};
// gather.wgsl:152-206
__device__ __forceinline__ LightSample direct_light(Ctx &c, f3 hp, f3 sn, Rng &rng) {
    const DevScene &s = c.p.scene;
    const uint32_t n = s.light_count;
    const f3 zero = mk3(0.0f, 0.0f, 0.0f);
    if (n == 0u) return LightSample{zero, sn};
    uint32_t li = f2u_sat(rng_f32(rng) * (float)n);
    li = li < n ? li : n - 1u;
    Light l = load_light(s, li);
    const float fn = (float)n;
    if (l.kind == 0u) {
        f3 to = l.data - hp;
        float r2 = dot(to, to);
        float r = sqrtf(r2);
        f3 ld = to / r;
        if (dot(sn, ld) <= 0.0f) return LightSample{zero, ld};
        if (shadowed(c, hp + sn * 0.01f, ld, r - 0.001f)) return LightSample{zero, ld};
        f3 pl = mk3(c.p.ip.point_light_emission[0], c.p.ip.point_light_emission[1], c.p.ip.point_light_emission[2]);
        return LightSample{l.color * l.intensity * pl * fmaxf(dot(sn, ld), 0.0f) / (r2 + 0.01f) * fn, ld};
    } else if (l.kind == 1u) {
        f3 ld = normalize(l.data);
        float ndl = dot(sn, ld);
        if (ndl <= 0.0f) return LightSample{zero, ld};
        if (shadowed(c, hp + sn * 0.01f, ld, 1e30f)) return LightSample{zero, ld};
        return LightSample{l.color * l.intensity * ndl * fn, ld};
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
        le = le * mk3(c.p.ip.light_emission[0], c.p.ip.light_emission[1], c.p.ip.light_emission[2]);
        f3 to = lp - hp;
        float r2 = dot(to, to);
        float r = sqrtf(r2);
        f3 ld = to / r;
        float ndl = dot(sn, ld);
        if (ndl <= 0.0f) return LightSample{zero, ld};
        f3 ln = triangle_normal(tri.v0, tri.v1, tri.v2);
        float ndl_l = dot(ln, -ld);
        if (ndl_l <= 0.0f) return LightSample{zero, ld};
        if (shadowed(c, hp + sn * 0.01f, ld, r - 0.001f)) return LightSample{zero, ld};
        float area = 0.5f * len3(cross(tri.v1 - tri.v0, tri.v2 - tri.v0));
        return LightSample{le * l.intensity * ndl * ndl_l * area * fn / (r2 + 0.01f), ld};
    }
    return LightSample{zero, sn};
}

__device__ __forceinline__ int32_t clampi(int32_t x, int32_t lo, int32_t hi) { return x < lo ? lo : (x > hi ? hi : x); }

}  // namespace

__global__ void __launch_bounds__(64) gather_kernel(const __grid_constant__ GatherParams p) {
    __shared__ uint32_t stack_smem[64 * 64];
    const uint32_t tid = threadIdx.x + 8u * threadIdx.y;
    const uint32_t px = blockIdx.x * 8u + threadIdx.x;
    const uint32_t py = blockIdx.y * 8u + threadIdx.y;
    const rt_image_params &ip = p.ip;
    const bool active = px < ip.width && py < ip.height;
    Ctx c{p, stack_smem + tid, 64u, 0u};
    uint32_t segments = 0u;

    if (active) {
        const DevScene &s = p.scene;
        const rt_camera_uniform &cam = p.cam;
        const uint32_t debug_view = ip._pad[0];
        uint32_t base_seed = py * ip.width + px + ip.frame * 2654435761u;
        Rng rng = rng_init(base_seed * 1664525u + 1013904223u);
        Accum A;
        A.col = mk3(0.0f, 0.0f, 0.0f);
        A.lum_sum = 0.0f;
        A.lum2_sum = 0.0f;
#pragma unroll
        for (int i = 0; i < 8; ++i) A.sample_lum[i] = 0.0f;
        f3 first_normal = mk3(0.0f, 1.0f, 0.0f);
        float first_depth = 1e30f;
        const uint32_t spp = ip.spp > 1u ? ip.spp : 1u;
        const float env_intensity = s.env_intensity;
        const f3 env_color = mk3(s.env_color[0], s.env_color[1], s.env_color[2]);
        const f3 env_horizon = mk3(s.env_horizon[0], s.env_horizon[1], s.env_horizon[2]);
        const f3 cam_pos = mk3(cam.position[0], cam.position[1], cam.position[2]);
        const f3 cam_fwd = mk3(cam.forward[0], cam.forward[1], cam.forward[2]);
        const f3 cam_right = mk3(cam.right[0], cam.right[1], cam.right[2]);
        const f3 cam_up = mk3(cam.up[0], cam.up[1], cam.up[2]);

        for (uint32_t sidx = 0; sidx < spp; ++sidx) {
            float jx = rng_f32(rng) - 0.5f;
            float jy = rng_f32(rng) - 0.5f;
            float ux = ((float)px + jx) * cam.inv_half_res[0] - 1.0f;
            float uy = 1.0f - ((float)py + jy) * cam.inv_half_res[1];
            f3 ro = cam_pos;
            f3 rd = normalize(cam_fwd + cam_right * ux + cam_up * uy);
            f3 thr = mk3(1.0f, 1.0f, 1.0f);

            for (uint32_t b = 0; b < p.max_bounces; ++b) {
                segments += 1u;
                Hit hit = trace_bvh<64>(s, ro, rd, c.stk, c.stride);
                if (hit.t >= kInf) {
                    if (b > 0u) add_radiance(sidx, A, thr * sky_color(rd, env_color, env_horizon, env_intensity));
                    break;
                }
                TriFull tr = load_tri(s, hit.prim);
                Mat mat = load_mat(s, tr.material_id);
                f3 hp = ro + rd * hit.t;
                Bary bb = barycentric(tr, ro, rd, hit.t);
                const float uvx = bb.uvx, uvy = bb.uvy;

                if ((mat.flags & RT_MAT_FLAG_ALPHA_CUTOUT) != 0u && mat.tex_albedo != RT_TEX_NONE) {
                    if (tex_sample(s.tex[RT_TEX_ALBEDO], uvx, uvy, (int32_t)mat.tex_albedo).w < 0.5f) {
                        ro = hp + rd * 0.002f;
                        continue;
                    }
                }

                f3 gn = triangle_normal(tr.v0, tr.v1, tr.v2);
                bool ff = dot(rd, gn) < 0.0f;
                f3 sn_geom = smooth_normal(tr, bb, gn);
                f3 sn = ff ? sn_geom : -sn_geom;
                f3 shn = sn;
                if (mat.tex_normal != RT_TEX_NONE) {
                    float4 t = tex_sample(s.tex[RT_TEX_NORMAL], uvx, uvy, (int32_t)mat.tex_normal);
                    f3 nm = mk3(t.x, t.y, t.z) * 2.0f - mk3(1.0f, 1.0f, 1.0f);
                    f3 ft, fb;
                    tangent_frame(tr, sn, ft, fb);
                    shn = normalize(ft * nm.x + fb * nm.y + sn * nm.z);
                }

                if (b == 0u && hit.t < first_depth) {
                    first_normal = sn;
                    first_depth = hit.t;
                }

                // eval_material (gather.wgsl:120-134)
                f3 albedo = mat.albedo;
                float rough = mat.roughness;
                float metal = mat.metallic;
                if (mat.tex_albedo != RT_TEX_NONE) {
                    float4 t = tex_sample(s.tex[RT_TEX_ALBEDO], uvx, uvy, (int32_t)mat.tex_albedo);
                    albedo = mat.albedo * mk3(t.x, t.y, t.z);
                }
                if (mat.tex_mr != RT_TEX_NONE) {
                    float4 mr = tex_sample(s.tex[RT_TEX_MR], uvx, uvy, (int32_t)mat.tex_mr);
                    rough = clampf(mat.roughness * mr.y, 0.0f, 1.0f);
                    metal = clampf(mat.metallic * mr.z, 0.0f, 1.0f);
                }
                // emissive_at (gather.wgsl:136-141)
                f3 emis = mat.emissive;
                if (mat.tex_emissive != RT_TEX_NONE) {
                    float4 t = tex_sample(s.tex[RT_TEX_EMISSIVE], uvx, uvy, (int32_t)mat.tex_emissive);
                    emis = mat.emissive * mk3(t.x, t.y, t.z);
                }
                add_radiance(sidx, A, thr * emis);

                if (debug_view != 0u) {  // gather.wgsl:359-419
                    bool stop = true;
                    const f3 half = mk3(0.5f, 0.5f, 0.5f);
                    switch (debug_view) {
                        case 1: A.col = mk3(uvx, uvy, 0.0f); break;
                        case 2: A.col = sn * 0.5f + half; break;
                        case 3: A.col = shn * 0.5f + half; break;
                        case 4: A.col = gn * 0.5f + half; break;
                        case 5: A.col = emis; break;
                        case 8:
                        case 9: {
                            float pu = (float)px / (float)ip.width, pv = (float)py / (float)ip.height;
                            float4 t = tex_sample(s.tex[debug_view == 8 ? RT_TEX_EMISSIVE : RT_TEX_ALBEDO], pu, pv, 0);
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
                    if (stop) break;
                }

                if (mat.kind == 2u) {  // dielectric (gather.wgsl:421-436)
                    float q = (mat.ior - 1.0f) / (mat.ior + 1.0f);
                    float f0s = powf(q, 2.0f);
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
                    continue;
                }

                // metallic-roughness lobe choice (gather.wgsl:439-452)
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

                if (!do_spec) {
                    LightSample ls = direct_light(c, hp, shn, rng);
                    if (env_intensity > 0.0f)
                        add_radiance(sidx, A, thr * dscale * sky_color(shn, env_color, env_horizon, env_intensity));
                    add_radiance(sidx, A, thr * dscale * ls.e / kPi);
                    add_radiance(sidx, A, thr * albedo * ip.ambient);
                } else {
                    LightSample ls = direct_light(c, hp, shn, rng);
                    add_radiance(sidx, A, thr * spec_ggx(wo, shn, ls.wi, a, f0) * ls.e / spec_prob);
                }

                if (ip.use_photons == 1u && !do_spec) {  // gather.wgsl:473-514
                    const rt_grid_params &gp = p.gp;
                    float r2 = ip.photon_radius * ip.photon_radius;
                    f3 ph_sum = mk3(0.0f, 0.0f, 0.0f);
                    uint32_t ph_hits = 0u, budget = 384u;
                    bool done = false;
                    int32_t bx = f2i_sat((hp.x - gp.room_min_x) / gp.cell_size);
                    int32_t by = f2i_sat((hp.y - gp.room_min_y) / gp.cell_size);
                    int32_t bz = f2i_sat((hp.z - gp.room_min_z) / gp.cell_size);
                    int32_t gxmax = (int32_t)gp.grid_x - 1, gymax = (int32_t)gp.grid_y - 1,
                            gzmax = (int32_t)gp.grid_z - 1;
                    for (int32_t dz = -1; dz <= 1 && !done; ++dz)
                        for (int32_t dy = -1; dy <= 1 && !done; ++dy)
                            for (int32_t dx = -1; dx <= 1 && !done; ++dx) {
                                int32_t cx = clampi((int32_t)((uint32_t)bx + (uint32_t)dx), 0, gxmax);
                                int32_t cy = clampi((int32_t)((uint32_t)by + (uint32_t)dy), 0, gymax);
                                int32_t cz = clampi((int32_t)((uint32_t)bz + (uint32_t)dz), 0, gzmax);
                                uint32_t cell =
                                    (uint32_t)cx + (uint32_t)cy * gp.grid_x + (uint32_t)cz * gp.grid_x * gp.grid_y;
                                uint2 m = __ldg(p.grid_meta + cell);
                                for (uint32_t i = 0; i < m.y && !done; ++i) {
                                    if (budget == 0u) {
                                        done = true;
                                        break;
                                    }
                                    budget -= 1u;
                                    uint64_t k = (uint64_t)m.x + i;
                                    k = k < p.sorted_count ? k : p.sorted_count - 1;
                                    const float4 *ph = p.sorted_photons + 4ull * k;
                                    f3 pp = xyz(__ldg(ph));
                                    f3 dd = pp - hp;
                                    float d2 = dot(dd, dd);
                                    if (d2 < r2) {
                                        f3 pw = xyz(__ldg(ph + 1));
                                        f3 inc = xyz(__ldg(ph + 2));
                                        ph_sum = ph_sum + pw * fmaxf(dot(shn, -inc), 0.0f);
                                        ph_hits += 1u;
                                        if (ph_hits >= 64u) {
                                            done = true;
                                            break;
                                        }
                                    }
                                }
                            }
                    if (ph_hits > 0u) {
                        add_radiance(sidx, A,
                                     thr * dscale * ph_sum * ip.photon_scale /
                                         (kPi * (float)ph_hits * ip.photon_radius * ip.photon_radius));
                    }
                    if (ip.photon_debug == 1u) {
                        float density = fminf((float)ph_hits / 64.0f, 1.0f);
                        A.col = mk3(1.0f - density, density, 0.0f) * 2.0f;
                    }
                }

                if (do_spec) {  // gather.wgsl:517-532
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
                    if (ip.use_photons == 1u) break;
                }
                float pr = max3(thr);
                if (pr <= 0.0f || rng_f32(rng) > pr) break;
                thr = thr / pr;
            }
        }

        if (spp <= 8u) {  // gather.wgsl:548-579
            float *sl = A.sample_lum;
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
                float d = sl[i] - median;
                spread += d * d;
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
        const size_t idx = (size_t)py * ip.width + px;
        p.frame[idx] = make_float4(col.x, col.y, col.z, 1.0f);
        p.moments[idx] = make_float4(fminf(A.lum_sum / (float)spp, 10.0f), fminf(A.lum2_sum / (float)spp, 100.0f), 0.0f, 0.0f);
        p.gbuffer[idx] = make_float4(first_normal.x, first_normal.y, first_normal.z, first_depth);
    }

    // Counters: one 64-bit atomic per warp (every lane reaches this point).
    uint32_t seg_w = __reduce_add_sync(0xFFFFFFFFu, segments);
    uint32_t shd_w = __reduce_add_sync(0xFFFFFFFFu, c.shadow_rays);
    if ((tid & 31u) == 0u && p.counters) {
        if (seg_w) atomicAdd(p.counters + 0, (unsigned long long)seg_w);
        if (shd_w) atomicAdd(p.counters + 1, (unsigned long long)shd_w);
    }
}

}  // namespace rtd
