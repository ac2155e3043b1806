// Image-space kernels of the frame: the edge-aware a-trous denoise pass and the fused resolve
// (composite into the accumulation history, then exposure / Reinhard / gamma into rgba8).
//
//   denoise  rustracer-renderer/shaders/denoise.wgsl:122-195  (HBM-bound stencil: 64 B/px compulsory)
//   resolve  rustracer-renderer/shaders/composite.wgsl:211-221 + tonemap.wgsl:240-271
//            (streaming: frame 16 B + history 16 B read, history 16 B + rgba8 4 B written per pixel)
#include <cuda.h>
#include <cudaTypedefs.h>

#include "rt_kernels.h"

namespace rtd {

__device__ __forceinline__ float luminance(f3 c) { return dot(c, mk3(0.2126f, 0.7152f, 0.0722f)); }

// One a-trous pass, one thread per pixel.  The 3x3 moment window and the 5x5 tap window are served
// from L1/L2: each input pixel is fetched from HBM once per pass.
__global__ void __launch_bounds__(256) denoise_kernel(const float4 *__restrict__ in, float4 *__restrict__ out,
                                                      const float4 *__restrict__ gbuffer,
                                                      const float4 *__restrict__ moments,
                                                      const rt_denoise_params p, const float *alpha_dev) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
    const uint32_t W = p.width, H = p.height;
    if (x >= W || y >= H) return;
    const int32_t step = (int32_t)p.step_size;
    const size_t idx = (size_t)y * W + x;
    const f3 center = xyz(__ldg(in + idx));
    const float4 gc = __ldg(gbuffer + idx);
    const f3 n_center = xyz(gc);
    const float d_center = gc.w;
    const float lum_center = luminance(center);

    float var_acc = 0.0f, var_cnt = 0.0f;
    for (int32_t qy = -1; qy <= 1; ++qy)
        for (int32_t qx = -1; qx <= 1; ++qx) {
            int32_t nx = (int32_t)x + qx, ny = (int32_t)y + qy;
            if (nx < 0 || ny < 0 || nx >= (int32_t)W || ny >= (int32_t)H) continue;
            float2 m = __ldg(reinterpret_cast<const float2 *>(moments + (size_t)ny * W + nx));
            var_acc += fmaxf(m.y - m.x * m.x, 0.0f);
            var_cnt += 1.0f;
        }
    const float var_frame = var_acc / fmaxf(var_cnt, 1.0f);
    const float alpha = alpha_dev ? *alpha_dev : p.alpha;
    const float ema_scale = alpha / fmaxf(2.0f - alpha, 1e-4f);
    const float var_c = var_frame * ema_scale;
    const float denom_c = var_c * p.lambda + 1e-6f;
    const float denom_d = p.phi_depth * fmaxf(d_center, 1e-4f);
    const float k1d[3] = {0.375f, 0.25f, 0.0625f};

    f3 sum = mk3(0.0f, 0.0f, 0.0f);
    float total = 0.0f;
#pragma unroll
    for (int32_t dy = -2; dy <= 2; ++dy) {
#pragma unroll
        for (int32_t dx = -2; dx <= 2; ++dx) {
            int32_t nx = (int32_t)x + dx * step, ny = (int32_t)y + dy * step;
            if (nx < 0 || ny < 0 || nx >= (int32_t)W || ny >= (int32_t)H) continue;
            size_t q = (size_t)ny * W + nx;
            f3 nb = xyz(__ldg(in + q));
            float4 g = __ldg(gbuffer + q);
            float sw = k1d[dx < 0 ? -dx : dx] * k1d[dy < 0 ? -dy : dy];
            float nw = powf(fmaxf(dot(n_center, xyz(g)), 0.0f), p.phi_normal);
            float dw = expf(-fabsf(d_center - g.w) / denom_d);
            float dl = luminance(nb) - lum_center;
            float cw = expf(-(dl * dl) / denom_c);
            float w = sw * nw * dw * cw;
            sum = sum + nb * w;
            total += w;
        }
    }
    f3 o = total > 1e-6f ? sum / total : center;
    out[idx] = make_float4(o.x, o.y, o.z, 1.0f);
}

// The same pass for steps 1 and 2 (the reference's two passes) over a 32 x 32 pixel tile staged in
// shared memory with a 2*step halo: colour with its luminance, normal with depth, and the raw
// per-pixel variance of the moments with a 1-pixel halo.  Each thread computes four pixels of one
// column, (x, y + k*step) for k = 0..3, whose 5 x 5 tap windows share four of their five rows, so a
// tap row is read from shared memory once for up to four pixels (40 reads for 4 pixels instead of
// 100); a warp's lanes read consecutive x (no bank conflicts).  Tiles entirely inside the image skip
// the bounds tests.  A tap's weight is evaluated as
//   pow(max(n.n', 0), 12) * 2^(log2(B3(dx) B3(dy)) - log2(e) |dc - dn| / (phi_d max(dc, 1e-4))
//                                                  - log2(e) dl^2 / (lambda var + 1e-6)),
// the reference's product sw * nw * exp(depth term) * exp(luminance term) with the two exponentials
// and the spline weight merged into one base-2 exponential (ex2.approx), pow(x, 12) taken by
// squaring; this file is compiled with FMA contraction.  Results differ from the separate expf /
// powf form by a few ulps of the weights.
constexpr int kDnBX = 32, kDnRows = 32, kDnThreadsY = 8, kDnPix = 4;
constexpr float kLog2e = 1.4426950408889634f;
// log2 of the B3-spline taps 3/8, 1/4, 1/16 (index |offset|)
__device__ __forceinline__ constexpr float log_b3(int a) {
    return a == 0 ? -1.4150374992788438f : (a == 1 ? -2.0f : -4.0f);
}

__device__ __forceinline__ float ex2_approx(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float lg2_approx(float x) {
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Blocks whose tile copies did not arrive within the wait bound (none expected; read by
// rt_tma_timeouts).
__device__ unsigned int g_tma_timeouts = 0u;

// Bounded wait for an mbarrier phase: true once it completed, false after 2^20 polls.
__device__ __forceinline__ bool mbar_wait(uint32_t bar_s, uint32_t phase) {
    for (uint32_t i = 0; i < (1u << 20); ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(bar_s), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

template <int kStep, bool kInterior, bool kPow12>
__device__ __forceinline__ void denoise_column(const float4 (*s_cl)[kDnBX + 4 * kStep],
                                               const float4 (*s_nd)[kDnBX + 4 * kStep], const float *s_varc,
                                               int lx, int ly0, int x, int y0, int W, int Hh, const rt_denoise_params &p,
                                               float4 *__restrict__ out) {
    constexpr int H = 2 * kStep;
    float4 cn[kDnPix];
    float c_lum[kDnPix], a_l[kDnPix], a_d[kDnPix];
    float sr[kDnPix], sg[kDnPix], sb[kDnPix], tot[kDnPix];
#pragma unroll
    for (int k = 0; k < kDnPix; ++k) {
        c_lum[k] = s_cl[ly0 + H + k * kStep][lx + H].w;
        cn[k] = s_nd[ly0 + H + k * kStep][lx + H];
        a_l[k] = -kLog2e * rcp_approx(s_varc[k] * p.lambda + 1e-6f);
        a_d[k] = -kLog2e * rcp_approx(p.phi_depth * fmaxf(cn[k].w, 1e-4f));
        sr[k] = sg[k] = sb[k] = tot[k] = 0.0f;
    }
    // Tap rows j = 0 .. 7 (row offset (j - 2) * step from the first pixel); pixel k uses rows k .. k+4.
#pragma unroll
    for (int j = 0; j < kDnPix + 4; ++j) {
        const int ty = ly0 + j * kStep;  // tile row of this tap row
#pragma unroll
        for (int dx = -2; dx <= 2; ++dx) {
            const int nx = x + dx * kStep;
            if (!kInterior && (nx < 0 || nx >= W)) continue;
            const float4 nb = s_cl[ty][lx + H + dx * kStep];
            const float4 nd = s_nd[ty][lx + H + dx * kStep];
#pragma unroll
            for (int k = 0; k < kDnPix; ++k) {
                const int dy = j - k - 2;
                if (dy < -2 || dy > 2) continue;
                if (!kInterior) {
                    const int ny = y0 + (j - 2) * kStep;
                    if (ny < 0 || ny >= Hh || y0 + k * kStep >= Hh) continue;
                }
                const float d = fmaxf(cn[k].x * nd.x + cn[k].y * nd.y + cn[k].z * nd.z, 0.0f);
                const float dl = nb.w - c_lum[k];
                const float lsw = log_b3(dx < 0 ? -dx : dx) + log_b3(dy < 0 ? -dy : dy);
                float t = fmaf(fabsf(cn[k].w - nd.w), a_d[k], lsw);
                t = fmaf(dl * a_l[k], dl, t);
                float w;
                if (kPow12) {
                    // max(n.n', 0)^12 folded into the exponent: 2^(12 log2 d + t) (d = 0 gives 0)
                    w = ex2_approx(fmaf(12.0f, lg2_approx(d), t));
                } else {
                    w = powf(d, p.phi_normal) * ex2_approx(t);
                }
                sr[k] = fmaf(nb.x, w, sr[k]);
                sg[k] = fmaf(nb.y, w, sg[k]);
                sb[k] = fmaf(nb.z, w, sb[k]);
                tot[k] += w;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kDnPix; ++k) {
        const int y = y0 + k * kStep;
        if (!kInterior && (x >= W || y >= Hh)) continue;
        const size_t idx = (size_t)y * W + x;
        if (tot[k] > 1e-6f) {
            const float inv = rcp_approx(tot[k]);
            out[idx] = make_float4(sr[k] * inv, sg[k] * inv, sb[k] * inv, 1.0f);
        } else {
            const float4 c = s_cl[ly0 + H + k * kStep][lx + H];
            out[idx] = make_float4(c.x, c.y, c.z, 1.0f);
        }
    }
}

template <int kStep>
__global__ void __launch_bounds__(kDnBX * kDnThreadsY, 3) denoise_tiled_kernel(const __grid_constant__ CUtensorMap tm_in,
                                                                           const __grid_constant__ CUtensorMap tm_g,
                                                                           float4 *__restrict__ out,
                                                                           const float4 *__restrict__ moments,
                                                                           const rt_denoise_params p,
                                                                           const float *alpha_dev) {
    constexpr int H = 2 * kStep, TW = kDnBX + 2 * H, TH = kDnRows + 2 * H;
    constexpr uint32_t kBox = 16u * TW * TH;  // bytes of one staged tile
    extern __shared__ unsigned char dn_raw[];
    grid_launch_dependents();
    // TMA writes the tiles at a 128-byte aligned shared address; the mbarrier follows the tiles.
    float4 *dn_smem = reinterpret_cast<float4 *>(
        (reinterpret_cast<uintptr_t>(dn_raw) + 127u) & ~static_cast<uintptr_t>(127u));
    float4(*s_cl)[TW] = reinterpret_cast<float4(*)[TW]>(dn_smem);
    float4(*s_nd)[TW] = reinterpret_cast<float4(*)[TW]>(dn_smem + TW * TH);
    float(*s_var)[kDnBX + 2] = reinterpret_cast<float(*)[kDnBX + 2]>(dn_smem + 2 * TW * TH);
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(
        reinterpret_cast<float *>(s_var) + ((kDnBX + 2) * (kDnRows + 2) + 1) / 2 * 2);
    const int W = (int)p.width, Hh = (int)p.height;
    const int tid = threadIdx.y * kDnBX + threadIdx.x;
    const int x0 = (int)blockIdx.x * kDnBX, y0t = (int)blockIdx.y * kDnRows;
    constexpr int kThreads = kDnBX * kDnThreadsY;
    // Colour and G-buffer tiles (with the 2-step halo) staged by the tensor-memory accelerator: one
    // thread arms the barrier with both tiles' bytes and issues the two copies (positions outside the
    // image arrive as zeros and are never read: the taps check the image bounds) while the block
    // loads the variance window.
    const uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(bar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // A pass after another pass may start while that one finishes (programmatic dependent launch):
    // the G-buffer tile and the moments are the frame's, only the colour tile is the previous pass's
    // output, so its copy is issued after grid_dependency_wait().
    if (tid == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_s), "r"(2u * kBox) : "memory");
        const int cx = x0 - H, cy = y0t - H;
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
                (uint32_t)__cvta_generic_to_shared(&s_nd[0][0])),
            "l"(reinterpret_cast<uint64_t>(&tm_g)), "r"(0), "r"(cx), "r"(cy), "r"(bar_s)
            : "memory");
        grid_dependency_wait();
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
                (uint32_t)__cvta_generic_to_shared(&s_cl[0][0])),
            "l"(reinterpret_cast<uint64_t>(&tm_in)), "r"(0), "r"(cx), "r"(cy), "r"(bar_s)
            : "memory");
    }
    // Variance window ((32 + 2) x (32 + 2), -1 outside the image): columns 0..31 at rows
    // threadIdx.y + 8 k, and the last two columns one value each for threads 0..67.
    {
        constexpr int VW = kDnBX + 2, VH = kDnRows + 2, kRowsPer = (VH + kDnThreadsY - 1) / kDnThreadsY;
        const int tx = (int)threadIdx.x;
        auto inside = [&](int gx, int gy) { return gx >= 0 && gy >= 0 && gx < W && gy < Hh; };
        float2 m[kRowsPer], me = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int k = 0; k < kRowsPer; ++k) {
            const int vy = (int)threadIdx.y + k * kDnThreadsY, gx = x0 - 1 + tx, gy = y0t - 1 + vy;
            m[k] = make_float2(0.0f, 0.0f);
            if (vy < VH && inside(gx, gy)) m[k] = __ldg(reinterpret_cast<const float2 *>(moments + (size_t)gy * W + gx));
        }
        const int ey = tid >> 1, ex = kDnBX + (tid & 1), egx = x0 - 1 + ex, egy = y0t - 1 + ey;
        if (tid < 2 * VH && inside(egx, egy))
            me = __ldg(reinterpret_cast<const float2 *>(moments + (size_t)egy * W + egx));
#pragma unroll
        for (int k = 0; k < kRowsPer; ++k) {
            const int vy = (int)threadIdx.y + k * kDnThreadsY, gx = x0 - 1 + tx, gy = y0t - 1 + vy;
            if (vy < VH) s_var[vy][tx] = inside(gx, gy) ? fmaxf(m[k].y - m[k].x * m[k].x, 0.0f) : -1.0f;
        }
        if (tid < 2 * VH) s_var[ey][ex] = inside(egx, egy) ? fmaxf(me.y - me.x * me.x, 0.0f) : -1.0f;
    }
    grid_dependency_wait();  // nothing below reads or writes what the previous pass uses before it ends
    // Wait for the two tiles (phase 0 of the barrier), bounded: a block whose copies do not arrive
    // counts the fault, waits once more (bounded) for them and leaves without writing.
    if (__syncthreads_or(!mbar_wait(bar_s, 0u)) != 0) {
        if (tid == 0) {
            atomicAdd(&g_tma_timeouts, 1u);
            mbar_wait(bar_s, 0u);
        }
        return;
    }
    // The colour tile's fourth channel becomes the luminance the taps compare.
    for (int i = tid; i < TW * TH; i += kThreads) {
        float4 &c = (&s_cl[0][0])[i];
        c.w = luminance(mk3(c.x, c.y, c.z));
    }
    __syncthreads();
    // This thread's column: rows r0 + k*step of the tile, k = 0..3.
    const int ty = (int)threadIdx.y;
    const int r0 = (ty / kStep) * (kDnPix * kStep) + (ty % kStep);
    const int lx = (int)threadIdx.x, x = x0 + lx, y0 = y0t + r0;
    const float alpha = alpha_dev ? *alpha_dev : p.alpha;
    const float ema_scale = alpha / fmaxf(2.0f - alpha, 1e-4f);
    // Warps whose every tap and 3 x 3 window lies inside the image skip the bounds tests.
    const bool interior = __all_sync(0xFFFFFFFFu, x - H >= 0 && x + H < W && y0 - H >= 0 &&
                                                      y0 + (kDnPix - 1) * kStep + H < Hh);
    float varc[kDnPix];
    if (interior) {
        // every 3 x 3 window is inside the image: sums of three per tile row, shared by the
        // thread's four windows (rows r0 + t, t = 0 .. 3 step + 2)
        constexpr int kRows = 3 * kStep + 3;
        float rs[kRows];
#pragma unroll
        for (int t = 0; t < kRows; ++t)
            rs[t] = s_var[r0 + t][lx] + s_var[r0 + t][lx + 1] + s_var[r0 + t][lx + 2];
        const float scale = ema_scale * (1.0f / 9.0f);
#pragma unroll
        for (int k = 0; k < kDnPix; ++k) varc[k] = (rs[k * kStep] + rs[k * kStep + 1] + rs[k * kStep + 2]) * scale;
    } else {
#pragma unroll
        for (int k = 0; k < kDnPix; ++k) {
            float acc = 0.0f, cnt = 0.0f;
#pragma unroll
            for (int qy = 0; qy < 3; ++qy)
#pragma unroll
                for (int qx = 0; qx < 3; ++qx) {
                    const float v = s_var[r0 + k * kStep + qy][lx + qx];
                    if (v >= 0.0f) {
                        acc += v;
                        cnt += 1.0f;
                    }
                }
            varc[k] = (acc / fmaxf(cnt, 1.0f)) * ema_scale;
        }
    }
    if (p.phi_normal == 12.0f) {
        if (interior) denoise_column<kStep, true, true>(s_cl, s_nd, varc, lx, r0, x, y0, W, Hh, p, out);
        else denoise_column<kStep, false, true>(s_cl, s_nd, varc, lx, r0, x, y0, W, Hh, p, out);
    } else {
        if (interior) denoise_column<kStep, true, false>(s_cl, s_nd, varc, lx, r0, x, y0, W, Hh, p, out);
        else denoise_column<kStep, false, false>(s_cl, s_nd, varc, lx, r0, x, y0, W, Hh, p, out);
    }
}

template <int kStep>
constexpr size_t denoise_smem_bytes() {
    // 128 bytes of alignment slack, the two tiles, the variance window (rounded to 8 bytes), the barrier
    return 128 + sizeof(float4) * 2 * (kDnBX + 4 * kStep) * (kDnRows + 4 * kStep) +
           sizeof(float) * (((kDnBX + 2) * (kDnRows + 2) + 1) / 2 * 2) + 8;
}

void prepare_kernels() {
    static bool done = false;  // opt in to more than 48 KB of dynamic shared memory, once per process
    if (done) return;
    cudaFuncSetAttribute(denoise_tiled_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)denoise_smem_bytes<1>());
    cudaFuncSetAttribute(denoise_tiled_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)denoise_smem_bytes<2>());
    prepare_wavefront_kernels();
    done = true;
}

namespace {

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against libcuda).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }();
    return fn;
}

// A W x H image of float4 (16-byte rows of 4 floats, row pitch 16 W bytes) as a 3-D tensor
// (channel, x, y) copied in side x side pixel boxes; positions outside the image read as zeros.
cudaError_t encode_tile_map(CUtensorMap *tm, const float4 *base, uint32_t w, uint32_t h, uint32_t side) {
    const PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return cudaErrorNotSupported;
    const cuuint64_t dims[3] = {4u, w, h};
    const cuuint64_t strides[2] = {16u, 16ull * w};
    const cuuint32_t box[3] = {4u, side, side};
    const cuuint32_t elem[3] = {1u, 1u, 1u};
    const CUresult r = encode(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float4 *>(base), dims, strides, box,
                              elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace

uint32_t tma_timeouts() {
    unsigned int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_tma_timeouts, sizeof(v)) != cudaSuccess) return 0xFFFFFFFFu;
    return v;
}

cudaError_t launch_denoise(const float4 *in, float4 *out, const float4 *gbuffer, const float4 *moments,
                           const rt_denoise_params &p, const float *alpha_dev, cudaStream_t st, bool after_pass) {
    if (p.step_size == 1u || p.step_size == 2u) {
        prepare_kernels();
        dim3 block(kDnBX, kDnThreadsY);
        dim3 grid((p.width + kDnBX - 1) / kDnBX, (p.height + kDnRows - 1) / kDnRows);
        const uint32_t side = (uint32_t)(kDnBX + 4 * p.step_size);
        CUtensorMap tm_in, tm_g;
        cudaError_t e;
        if ((e = encode_tile_map(&tm_in, in, p.width, p.height, side)) != cudaSuccess) return e;
        if ((e = encode_tile_map(&tm_g, gbuffer, p.width, p.height, side)) != cudaSuccess) return e;
        // A pass right after another tiled pass is a programmatic dependent of it.
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = grid;
        cfg.blockDim = block;
        cfg.dynamicSmemBytes = p.step_size == 1u ? denoise_smem_bytes<1>() : denoise_smem_bytes<2>();
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = after_pass ? 1 : 0;
        if (p.step_size == 1u)
            return cudaLaunchKernelEx(&cfg, denoise_tiled_kernel<1>, tm_in, tm_g, out, moments, p, alpha_dev);
        return cudaLaunchKernelEx(&cfg, denoise_tiled_kernel<2>, tm_in, tm_g, out, moments, p, alpha_dev);
    }
    dim3 block(32, 8);
    dim3 grid((p.width + block.x - 1) / block.x, (p.height + block.y - 1) / block.y);
    denoise_kernel<<<grid, block, 0, st>>>(in, out, gbuffer, moments, p, alpha_dev);
    return cudaGetLastError();
}

// composite.wgsl mix() then tonemap.wgsl, one pixel per thread, 1-D over the image.
__global__ void __launch_bounds__(256) resolve_kernel(const float4 *__restrict__ frame, float4 *__restrict__ accum,
                                                      const float4 *__restrict__ gbuffer, uint32_t width,
                                                      uint32_t npix, float alpha_arg, const float *alpha_dev,
                                                      const rt_tonemap_params tp, uchar4 *__restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    const float alpha = alpha_dev ? *alpha_dev : alpha_arg;
    const float4 f = __ldg(frame + i);
    const float4 a = accum[i];
    // mix(prev, fresh, alpha) rounded as two products and a sum (no contraction: this file is
    // compiled with FMA, the composite stays bit-exact).
    const float om = 1.0f - alpha;
    auto mixr = [&](float x, float y) { return __fadd_rn(__fmul_rn(x, om), __fmul_rn(y, alpha)); };
    const float4 h = make_float4(mixr(a.x, f.x), mixr(a.y, f.y), mixr(a.z, f.z), mixr(a.w, f.w));
    accum[i] = h;
    const f3 exposed = mk3(h.x, h.y, h.z) * tp.exposure;
    const f3 mapped = exposed / (exposed + mk3(1.0f, 1.0f, 1.0f));
    const float ig = 1.0f / tp.gamma;
    // pow(mapped, 1/gamma) for mapped in [0, 1): the hardware exp2 / log2 form (the rgba8 result is
    // within one step of the correctly rounded pow, as the tonemap of the reference's backend is)
    f3 color = mk3(__powf(mapped.x, ig), __powf(mapped.y, ig), __powf(mapped.z, ig));
    if (tp.marker[3] > 0.0f) {
        const uint32_t x = i % width, y = i / width;
        float ddx = ((float)x + 0.5f) - tp.marker[0], ddy = ((float)y + 0.5f) - tp.marker[1];
        float d = sqrtf(ddx * ddx + ddy * ddy);
        float r = fmaxf(tp.marker[2], 1.5f);
        float hit_dist = gbuffer ? __ldg(gbuffer + i).w : 1e30f;
        if (hit_dist > tp.marker[3] - 0.2f) {
            float ball = 1.0f - smoothstepf(r * 0.75f, r, d);
            float halo = 1.0f - smoothstepf(r, r * 3.5f, d);
            f3 core = mk3(1.0f, 0.94f, 0.80f) * powf(ball, 1.4f) * 0.85f;
            f3 ring = mk3(1.0f, 0.46f, 0.14f) * halo * halo * 0.8f;
            color = color + (core + ring) * tp.glow * (mk3(1.0f, 1.0f, 1.0f) - 0.55f * color);
        }
    }
    auto q8 = [](float c) -> unsigned char {
        return (unsigned char)__float2uint_rz(clampf(c, 0.0f, 1.0f) * 255.0f + 0.5f);
    };
    out[i] = make_uchar4(q8(color.x), q8(color.y), q8(color.z), 255);
}

cudaError_t launch_resolve(const float4 *frame, float4 *accum, const float4 *gbuffer, uint32_t width,
                           uint32_t height, float alpha, const float *alpha_dev, const rt_tonemap_params &tp,
                           uchar4 *out, cudaStream_t st) {
    const uint32_t npix = width * height;
    const uint32_t block = 256;
    resolve_kernel<<<(npix + block - 1) / block, block, 0, st>>>(frame, accum, gbuffer, width, npix, alpha, alpha_dev,
                                                                 tp, out);
    return cudaGetLastError();
}

}  // namespace rtd
