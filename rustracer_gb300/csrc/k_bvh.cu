// BVH build on the GPU: a linear BVH (Karras, "Maximizing parallelism in the construction of BVHs,
// octrees, and k-d trees", HPG 2012) over the triangles' centroid Morton codes, written in the
// reference's BVHNode layout (rustracer-core/src/bvh.rs:79-88) so that every consumer of the host
// SAH build (BVHBuilder::build, bvh.rs:135-336) takes it unchanged.  It trades tree quality for build
// time: splits at Morton-code prefix changes instead of the SAH; subtrees of at most four primitives
// are collapsed into leaves afterwards, the reference's leaf policy.
//
//   keys      (morton30(centroid) << 32) | prim: unique, so the sorted order (and the tree) is
//             deterministic
//   sort      bitonic network: global passes for distances >= 2048, the rest in shared memory
//   hierarchy one thread per internal node finds its key range and split (longest common prefix)
//   boxes     one thread per leaf walks towards the root; at each node the second child to arrive
//             (atomic counter) writes the union of the two children's boxes and continues
//   leaves    on the host: subtrees of at most four primitives become leaves (the reference's
//             policy), and the tree is written root first with its depth measured
//
// Node numbering: internal nodes 0 .. n-2 (node 0 is the root), leaf of sorted position i is node
// n-1+i with prims[i] its primitive.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "rt_internal.h"
#include "rt_kernels.h"

namespace rtd {

namespace {

__device__ __forceinline__ uint32_t expand_bits10(uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void lbvh_keys_kernel(const float *__restrict__ centroids, uint32_t n, uint32_t n_pad, float3 lo,
                                 float3 scale, unsigned long long *__restrict__ keys) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_pad; i += gridDim.x * blockDim.x) {
        if (i >= n) {
            keys[i] = ~0ull;
            continue;
        }
        const float c[3] = {centroids[3 * i], centroids[3 * i + 1], centroids[3 * i + 2]};
        const float l[3] = {lo.x, lo.y, lo.z}, s[3] = {scale.x, scale.y, scale.z};
        uint32_t q[3];
        for (int a = 0; a < 3; ++a) {
            const float f = (c[a] - l[a]) * s[a];  // in [0, 1023] for finite input
            q[a] = f > 0.0f ? (f < 1023.0f ? (uint32_t)f : 1023u) : 0u;
        }
        const uint32_t m = (expand_bits10(q[0]) << 2) | (expand_bits10(q[1]) << 1) | expand_bits10(q[2]);
        keys[i] = ((unsigned long long)m << 32) | i;
    }
}

// One compare-exchange pass of the bitonic network (distance j >= 2048, sequence length k).
__global__ void bitonic_global_kernel(unsigned long long *keys, uint32_t n_pad, uint32_t j, uint32_t k) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n_pad / 2; t += gridDim.x * blockDim.x) {
        const uint32_t lo = (t / j) * 2u * j + (t % j), hi = lo + j;
        const bool up = (lo & k) == 0u;
        const unsigned long long a = keys[lo], b = keys[hi];
        if ((a > b) == up) {
            keys[lo] = b;
            keys[hi] = a;
        }
    }
}

// All passes with distance j <= j0 (j0 <= 1024) of sequence length k, on 2048-key segments held in
// shared memory.
__global__ void __launch_bounds__(1024) bitonic_local_kernel(unsigned long long *keys, uint32_t k, uint32_t j0) {
    __shared__ unsigned long long s[2048];
    const uint32_t base = blockIdx.x * 2048u, t = threadIdx.x;
    s[t] = keys[base + t];
    s[t + 1024] = keys[base + t + 1024];
    __syncthreads();
    for (uint32_t j = j0; j > 0; j >>= 1) {
        const uint32_t lo = (t / j) * 2u * j + (t % j), hi = lo + j;
        const bool up = ((base + lo) & k) == 0u;
        const unsigned long long a = s[lo], b = s[hi];
        if ((a > b) == up) {
            s[lo] = b;
            s[hi] = a;
        }
        __syncthreads();
    }
    keys[base + t] = s[t];
    keys[base + t + 1024] = s[t + 1024];
}

__device__ __forceinline__ int delta(const unsigned long long *keys, uint32_t n, int i, int j) {
    if (j < 0 || j >= (int)n) return -1;
    return __clzll(keys[i] ^ keys[j]);  // keys are unique: the xor is never 0
}

// Karras 2012, algorithm 3 (children of internal node i; leaves are n-1+position).
__global__ void lbvh_internal_kernel(const unsigned long long *__restrict__ keys, uint32_t n,
                                     uint2 *__restrict__ children, uint32_t *__restrict__ parent) {
    for (uint32_t ui = blockIdx.x * blockDim.x + threadIdx.x; ui + 1 < n; ui += gridDim.x * blockDim.x) {
        const int i = (int)ui;
        const int d = delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1) >= 0 ? 1 : -1;
        const int dmin = delta(keys, n, i, i - d);
        int lmax = 2;
        while (delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;  // at most log2(n) + 1 doublings
        int l = 0;
        for (int t = lmax / 2; t >= 1; t /= 2)
            if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
        const int j = i + l * d;
        const int dnode = delta(keys, n, i, j);
        int s = 0;
        for (int div = 2;; div *= 2) {
            const int t = (l + div - 1) / div;
            if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
            if (t <= 1) break;
        }
        const int g = i + s * d + min(d, 0);
        const uint32_t left = (min(i, j) == g) ? (n - 1u + (uint32_t)g) : (uint32_t)g;
        const uint32_t right = (max(i, j) == g + 1) ? (n - 1u + (uint32_t)g + 1u) : (uint32_t)g + 1u;
        children[i] = make_uint2(left, right);
        parent[left] = (uint32_t)i;
        parent[right] = (uint32_t)i;
    }
}

// Leaf boxes, then the internal boxes bottom-up: the second child to arrive at a node merges.
__global__ void lbvh_boxes_kernel(const unsigned long long *__restrict__ keys, uint32_t n,
                                  const float *__restrict__ bmin, const float *__restrict__ bmax,
                                  const uint2 *__restrict__ children, const uint32_t *__restrict__ parent,
                                  uint32_t *__restrict__ arrivals, float4 *lo, float4 *hi) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t prim = (uint32_t)(keys[i] & 0xFFFFFFFFull);
        uint32_t node = n - 1u + i;
        lo[node] = make_float4(bmin[3 * prim], bmin[3 * prim + 1], bmin[3 * prim + 2], 0.0f);
        hi[node] = make_float4(bmax[3 * prim], bmax[3 * prim + 1], bmax[3 * prim + 2], 0.0f);
        for (uint32_t guard = 0; node != 0u && guard < 64u; ++guard) {
            const uint32_t p = parent[node];
            if (p >= n - 1u) break;  // not an internal node: malformed input, stop
            __threadfence();
            if (atomicAdd(arrivals + p, 1u) == 0u) break;  // the sibling's thread finishes this node
            const uint2 c = children[p];
            const float4 al = __ldcg(lo + c.x), ah = __ldcg(hi + c.x), bl = __ldcg(lo + c.y), bh = __ldcg(hi + c.y);
            lo[p] = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.0f);
            hi[p] = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.0f);
            node = p;
        }
    }
}

struct Scratch {
    void *p = nullptr;
    ~Scratch() {
        if (p) cudaFree(p);
    }
};

}  // namespace

int build_lbvh(const float *centroids, const float *bmin, const float *bmax, uint32_t n, rt::BVH &out,
               uint32_t *max_depth) {
    out.nodes.clear();
    out.prims.clear();
    if (n < 2) return -1;  // the host build handles trivial trees
    uint32_t n_pad = 2048;
    while (n_pad < n) n_pad <<= 1;
    const size_t nodes = 2ull * n - 1ull;
    // one allocation: keys, centroids, boxes, children, parent, arrivals, node boxes
    const size_t off_keys = 0, off_c = off_keys + 8ull * n_pad, off_bmin = off_c + 12ull * n,
                 off_bmax = off_bmin + 12ull * n, off_child = (off_bmax + 12ull * n + 15) & ~15ull,
                 off_parent = off_child + 8ull * n, off_arr = off_parent + 4ull * nodes,
                 off_lo = (off_arr + 4ull * n + 15) & ~15ull, off_hi = off_lo + 16ull * nodes,
                 total = off_hi + 16ull * nodes;
    Scratch mem;
    if (cudaMalloc(&mem.p, total) != cudaSuccess) return -2;
    unsigned char *b = static_cast<unsigned char *>(mem.p);
    auto *keys = reinterpret_cast<unsigned long long *>(b + off_keys);
    auto *dc = reinterpret_cast<float *>(b + off_c);
    auto *dlo_t = reinterpret_cast<float *>(b + off_bmin);
    auto *dhi_t = reinterpret_cast<float *>(b + off_bmax);
    auto *children = reinterpret_cast<uint2 *>(b + off_child);
    auto *parent = reinterpret_cast<uint32_t *>(b + off_parent);
    auto *arrivals = reinterpret_cast<uint32_t *>(b + off_arr);
    auto *nlo = reinterpret_cast<float4 *>(b + off_lo);
    auto *nhi = reinterpret_cast<float4 *>(b + off_hi);
    // centroid bounds on the host (one pass) give the Morton grid
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (uint32_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], centroids[3 * i + a]);
            hi[a] = std::max(hi[a], centroids[3 * i + a]);
        }
    float sc[3];
    for (int a = 0; a < 3; ++a) sc[a] = hi[a] > lo[a] ? 1023.0f / (hi[a] - lo[a]) : 0.0f;
    if (cudaMemcpy(dc, centroids, 12ull * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dlo_t, bmin, 12ull * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dhi_t, bmax, 12ull * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(parent, 0xFF, 4ull * nodes) != cudaSuccess || cudaMemset(arrivals, 0, 4ull * n) != cudaSuccess)
        return -2;
    const int sms = device_sm_count();
    auto grid = [&](uint64_t items) {
        const uint64_t g = (items + 255) / 256, cap = (uint64_t)sms * 16;
        return (unsigned)std::max<uint64_t>(1, std::min(g, cap));
    };
    lbvh_keys_kernel<<<grid(n_pad), 256>>>(dc, n, n_pad, make_float3(lo[0], lo[1], lo[2]),
                                          make_float3(sc[0], sc[1], sc[2]), keys);
    for (uint32_t k = 2; k <= n_pad; k <<= 1) {
        uint32_t j = k >> 1;
        for (; j >= 2048u; j >>= 1) bitonic_global_kernel<<<grid(n_pad / 2), 256>>>(keys, n_pad, j, k);
        bitonic_local_kernel<<<n_pad / 2048u, 1024>>>(keys, k, j);
    }
    lbvh_internal_kernel<<<grid(n), 256>>>(keys, n, children, parent);
    lbvh_boxes_kernel<<<grid(n), 256>>>(keys, n, dlo_t, dhi_t, children, parent, arrivals, nlo, nhi);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return -2;
    std::vector<unsigned long long> hkeys(n);
    std::vector<uint2> hchild(n - 1);
    std::vector<float4> hlo(nodes), hhi(nodes);
    if (cudaMemcpy(hkeys.data(), keys, 8ull * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(hchild.data(), children, 8ull * (n - 1), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(hlo.data(), nlo, 16ull * nodes, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(hhi.data(), nhi, 16ull * nodes, cudaMemcpyDeviceToHost) != cudaSuccess)
        return -2;
    out.prims.resize(n);
    for (uint32_t i = 0; i < n; ++i) out.prims[i] = (uint32_t)(hkeys[i] & 0xFFFFFFFFull);
    // Leaf policy of BVHBuilder::build (bvh.rs:170-180): a subtree of at most max_prims_per_leaf (4)
    // primitives becomes one leaf.  A subtree's primitives are a contiguous run of the sorted order,
    // so its leaf covers prims[first, first + count).  Subtree sizes bottom-up (post-order walk).
    constexpr uint32_t kMaxLeaf = 4;
    std::vector<uint32_t> first(nodes), count(nodes);
    for (uint32_t i = 0; i < n; ++i) {
        first[n - 1 + i] = i;
        count[n - 1 + i] = 1;
    }
    {
        std::vector<std::pair<uint32_t, bool>> st;
        st.push_back({0u, false});
        while (!st.empty()) {
            auto [k, done] = st.back();
            st.pop_back();
            if (k + 1 >= n) continue;  // a leaf
            const uint32_t l = hchild[k].x, r = hchild[k].y;
            if (!done) {
                st.push_back({k, true});
                st.push_back({r, false});
                st.push_back({l, false});
            } else {
                first[k] = std::min(first[l], first[r]);
                count[k] = count[l] + count[r];
            }
        }
    }
    // Emit in the reference's layout, root first, children numbered as they are reached.
    out.nodes.clear();
    out.nodes.reserve(nodes);
    uint32_t deepest = 0;
    struct Item {
        uint32_t k, slot, depth;
    };
    std::vector<Item> st;
    out.nodes.emplace_back();
    st.push_back({0u, 0u, 0u});
    while (!st.empty()) {
        const Item it = st.back();
        st.pop_back();
        deepest = std::max(deepest, it.depth);
        rt_bvh_node nd;
        std::memset(&nd, 0, sizeof(nd));
        nd.bbox_min[0] = hlo[it.k].x;
        nd.bbox_min[1] = hlo[it.k].y;
        nd.bbox_min[2] = hlo[it.k].z;
        nd.bbox_max[0] = hhi[it.k].x;
        nd.bbox_max[1] = hhi[it.k].y;
        nd.bbox_max[2] = hhi[it.k].z;
        if (count[it.k] <= kMaxLeaf) {
            nd.left_first = first[it.k];
            nd.prim_count = count[it.k];
        } else {
            const uint32_t l = (uint32_t)out.nodes.size();
            out.nodes.emplace_back();
            out.nodes.emplace_back();
            nd.left_first = l;
            nd.right_child = l + 1u;
            nd.prim_count = 0;
            st.push_back({hchild[it.k].y, l + 1u, it.depth + 1u});
            st.push_back({hchild[it.k].x, l, it.depth + 1u});
        }
        out.nodes[it.slot] = nd;
    }
    if (max_depth) *max_depth = deepest;
    return 0;
}

}  // namespace rtd
