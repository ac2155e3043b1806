// JPEG decoding for the glTF ingest (rustracer-core/src/loader.rs:36-113, 266 decodes every image
// gltf::import supports; the reference gets JPEG from the `image` crate).  Written from the JPEG
// standard (ITU-T T.81 | ISO/IEC 10918-1) and JFIF 1.02:
//   * frames: baseline and extended sequential Huffman (SOF0, SOF1) and progressive Huffman (SOF2),
//     8-bit samples, 1 (grey) or 3 (YCbCr) components, sampling factors 1..2 per axis;
//   * Huffman tables (DHT) and quantisation tables (DQT, 8- and 16-bit), restart intervals (DRI /
//     RSTn), byte stuffing;
//   * progressive scans: spectral selection and successive approximation of DC and AC coefficients
//     (T.81 G.1.2), end-of-band runs;
//   * inverse DCT from its definition (T.81 A.3.3) in float, separable, with a table of cosines;
//     level shift and clamping; chroma upsampled by replication; YCbCr -> RGB by the JFIF equations.
// Arithmetic coding, lossless and hierarchical frames, 12-bit samples and CMYK / Adobe transforms are
// refused (the caller takes its solid-grey fallback, as the reference does for an undecodable image).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "rt_internal.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

struct Huff {
    // code lengths and values (T.81 C.2), then per length the first code, its index and the last code
    uint8_t vals[256] = {};
    int mincode[17] = {}, maxcode[18] = {}, valptr[17] = {};
    bool present = false;
    void build(const uint8_t counts[16], const uint8_t *v, int n) {
        std::memcpy(vals, v, (size_t)n);
        int code = 0, k = 0;
        for (int len = 1; len <= 16; ++len) {
            valptr[len] = k;
            mincode[len] = code;
            code += counts[len - 1];
            k += counts[len - 1];
            maxcode[len] = counts[len - 1] ? code - 1 : -1;
            code <<= 1;
        }
        maxcode[17] = 0x7FFFFFFF;
        present = true;
    }
};

struct Component {
    int id = 0, h = 1, v = 1, tq = 0;
    int td = 0, ta = 0;       // Huffman table selectors of the current scan
    int bw = 0, bh = 0;       // blocks per row / column (padded to whole MCUs)
    std::vector<int16_t> coef;  // bw * bh blocks of 64 coefficients (zig-zag order)
    int pred = 0;             // DC predictor
};

constexpr int kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                             12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                             35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                             58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

class Decoder {
  public:
    Decoder(const uint8_t *d, size_t n) : d_(d), n_(n) {}

    bool decode(std::vector<uint8_t> &rgba, uint32_t &w, uint32_t &h) {
        if (n_ < 4 || d_[0] != 0xFF || d_[1] != 0xD8) return false;
        pos_ = 2;
        bool frame = false;
        for (;;) {
            int m = next_marker();
            if (m < 0) return false;
            if (m == 0xD9) break;  // EOI
            if (m == 0xDA) {       // SOS: the scan's entropy-coded data follows its header
                if (!frame || !scan()) return false;
                continue;
            }
            if (pos_ + 2 > n_) return false;
            const size_t len = (size_t)(d_[pos_] << 8 | d_[pos_ + 1]);
            if (len < 2 || pos_ + len > n_) return false;
            const uint8_t *seg = d_ + pos_ + 2;
            const size_t sl = len - 2;
            pos_ += len;
            if (m == 0xC0 || m == 0xC1 || m == 0xC2) {
                if (frame || !sof(seg, sl, m == 0xC2)) return false;
                frame = true;
            } else if ((m >= 0xC3 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC)) {
                return false;  // lossless, hierarchical or arithmetic-coded frames
            } else if (m == 0xC4) {
                if (!dht(seg, sl)) return false;
            } else if (m == 0xDB) {
                if (!dqt(seg, sl)) return false;
            } else if (m == 0xDD) {
                if (sl < 2) return false;
                restart_ = seg[0] << 8 | seg[1];
            } else if (m == 0xEE) {
                adobe_ = sl >= 12 ? seg[11] : 0;
            }  // APPn, COM, DNL and the rest carry nothing the image needs
        }
        if (!frame || comps_.empty()) return false;
        if (comps_.size() == 3 && adobe_ == 2) return false;  // YCCK
        return output(rgba, w, h);
    }

  private:
    const uint8_t *d_;
    size_t n_, pos_ = 0;
    int qt_[4][64] = {};
    Huff dc_[4], ac_[4];
    std::vector<Component> comps_;
    int width_ = 0, height_ = 0, hmax_ = 1, vmax_ = 1, mcux_ = 0, mcuy_ = 0;
    bool progressive_ = false;
    int restart_ = 0, adobe_ = -1;
    // bit reader of the entropy-coded segment
    uint32_t bitbuf_ = 0;
    int bitcnt_ = 0;
    bool hit_marker_ = false;
    int eobrun_ = 0;

    int next_marker() {
        while (pos_ + 1 < n_) {
            if (d_[pos_] != 0xFF) {
                ++pos_;
                continue;
            }
            while (pos_ < n_ && d_[pos_] == 0xFF) ++pos_;
            if (pos_ >= n_) return -1;
            const int m = d_[pos_++];
            if (m != 0x00) return m;
        }
        return -1;
    }

    bool sof(const uint8_t *s, size_t n, bool prog) {
        if (n < 6 || s[0] != 8) return false;  // 8-bit samples only
        height_ = s[1] << 8 | s[2];
        width_ = s[3] << 8 | s[4];
        const int nc = s[5];
        if (width_ <= 0 || height_ <= 0 || width_ > 16384 || height_ > 16384) return false;
        if ((nc != 1 && nc != 3) || n < (size_t)(6 + 3 * nc)) return false;
        progressive_ = prog;
        comps_.resize(nc);
        for (int i = 0; i < nc; ++i) {
            Component &c = comps_[i];
            c.id = s[6 + 3 * i];
            c.h = s[7 + 3 * i] >> 4;
            c.v = s[7 + 3 * i] & 15;
            c.tq = s[8 + 3 * i];
            if (c.h < 1 || c.h > 2 || c.v < 1 || c.v > 2 || c.tq > 3) return false;
            hmax_ = std::max(hmax_, c.h);
            vmax_ = std::max(vmax_, c.v);
        }
        mcux_ = (width_ + 8 * hmax_ - 1) / (8 * hmax_);
        mcuy_ = (height_ + 8 * vmax_ - 1) / (8 * vmax_);
        for (Component &c : comps_) {
            c.bw = mcux_ * c.h;
            c.bh = mcuy_ * c.v;
            c.coef.assign((size_t)c.bw * c.bh * 64, 0);
        }
        return true;
    }

    bool dht(const uint8_t *s, size_t n) {
        size_t p = 0;
        while (p < n) {
            if (p + 17 > n) return false;
            const int tc = s[p] >> 4, th = s[p] & 15;
            if (tc > 1 || th > 3) return false;
            int total = 0;
            for (int i = 0; i < 16; ++i) total += s[p + 1 + i];
            if (total > 256 || p + 17 + (size_t)total > n) return false;
            (tc ? ac_ : dc_)[th].build(s + p + 1, s + p + 17, total);
            p += 17 + (size_t)total;
        }
        return true;
    }

    bool dqt(const uint8_t *s, size_t n) {
        size_t p = 0;
        while (p < n) {
            const int pq = s[p] >> 4, tq = s[p] & 15;
            if (tq > 3 || pq > 1 || p + 1 + (pq ? 128u : 64u) > n) return false;
            for (int i = 0; i < 64; ++i)
                qt_[tq][i] = pq ? (s[p + 1 + 2 * i] << 8 | s[p + 2 + 2 * i]) : s[p + 1 + i];
            p += 1 + (pq ? 128 : 64);
        }
        return true;
    }

    // ---- entropy-coded data ------------------------------------------------------------------
    void reset_bits() {
        bitbuf_ = 0;
        bitcnt_ = 0;
        hit_marker_ = false;
    }
    int bit() {
        if (bitcnt_ == 0) {
            uint32_t b = 0;
            if (!hit_marker_ && pos_ < n_) {
                b = d_[pos_];
                if (b == 0xFF) {
                    const uint32_t nx = pos_ + 1 < n_ ? d_[pos_ + 1] : 0;
                    if (nx == 0x00) {
                        pos_ += 2;  // stuffed byte
                    } else {
                        hit_marker_ = true;  // a marker ends the segment: feed zeros
                        b = 0;
                    }
                } else {
                    ++pos_;
                }
            }
            bitbuf_ = b;
            bitcnt_ = 8;
        }
        --bitcnt_;
        return (int)(bitbuf_ >> bitcnt_) & 1;
    }
    int bits(int n) {
        int v = 0;
        for (int i = 0; i < n; ++i) v = v << 1 | bit();
        return v;
    }
    // T.81 F.2.2.3 DECODE
    int decode_huff(const Huff &t) {
        int code = bit();
        for (int len = 1; len <= 16; ++len) {
            if (t.maxcode[len] >= 0 && code <= t.maxcode[len] && code >= t.mincode[len])
                return t.vals[t.valptr[len] + code - t.mincode[len]];
            code = code << 1 | bit();
        }
        return -1;
    }
    // T.81 F.2.2.1 EXTEND
    static int extend(int v, int t) { return t == 0 ? 0 : (v < (1 << (t - 1)) ? v - (1 << t) + 1 : v); }

    bool restart_marker() {
        // byte-align, then expect RSTn
        reset_bits();
        while (pos_ + 1 < n_ && !(d_[pos_] == 0xFF && d_[pos_ + 1] >= 0xD0 && d_[pos_ + 1] <= 0xD7)) {
            if (d_[pos_] == 0xFF && d_[pos_ + 1] != 0x00 && d_[pos_ + 1] != 0xFF) return false;
            ++pos_;
        }
        if (pos_ + 1 >= n_) return false;
        pos_ += 2;
        for (Component &c : comps_) c.pred = 0;
        eobrun_ = 0;
        return true;
    }

    bool block_baseline(Component &c, int16_t *blk) {
        const int t = decode_huff(dc_[c.td]);
        if (t < 0 || t > 11) return false;
        c.pred += extend(bits(t), t);
        blk[0] = (int16_t)c.pred;
        for (int k = 1; k < 64;) {
            const int rs = decode_huff(ac_[c.ta]);
            if (rs < 0) return false;
            const int r = rs >> 4, s = rs & 15;
            if (s == 0) {
                if (r != 15) break;  // EOB
                k += 16;
                continue;
            }
            k += r;
            if (k > 63) return false;
            blk[k++] = (int16_t)extend(bits(s), s);
        }
        return true;
    }

    bool dc_first(Component &c, int16_t *blk, int al) {
        const int t = decode_huff(dc_[c.td]);
        if (t < 0 || t > 11) return false;
        c.pred += extend(bits(t), t);
        blk[0] = (int16_t)(c.pred * (1 << al));
        return true;
    }
    void dc_refine(int16_t *blk, int al) {
        if (bit()) blk[0] = (int16_t)(blk[0] | (1 << al));
    }
    bool ac_first(const Component &c, int16_t *blk, int ss, int se, int al) {
        if (eobrun_ > 0) {
            --eobrun_;
            return true;
        }
        for (int k = ss; k <= se;) {
            const int rs = decode_huff(ac_[c.ta]);
            if (rs < 0) return false;
            const int r = rs >> 4, s = rs & 15;
            if (s == 0) {
                if (r < 15) {  // EOBn: this band and (2^r - 1 + bits) more end here
                    eobrun_ = (1 << r) - 1;
                    if (r) eobrun_ += bits(r);
                    break;
                }
                k += 16;
                continue;
            }
            k += r;
            if (k > 63) return false;
            blk[k++] = (int16_t)(extend(bits(s), s) * (1 << al));
        }
        return true;
    }
    // T.81 G.1.2.3: correction bits for coefficients already non-zero, new coefficients of +-1 << al.
    bool ac_refine(const Component &c, int16_t *blk, int ss, int se, int al) {
        const int p1 = 1 << al, m1 = -1 * (1 << al);
        int k = ss;
        if (eobrun_ <= 0) {
            for (; k <= se;) {
                const int rs = decode_huff(ac_[c.ta]);
                if (rs < 0) return false;
                int r = rs >> 4;
                const int s = rs & 15;
                int val = 0;
                if (s == 0) {
                    if (r < 15) {
                        eobrun_ = (1 << r);
                        if (r) eobrun_ += bits(r);
                        break;
                    }
                } else {
                    if (s != 1) return false;
                    val = bit() ? p1 : m1;
                }
                while (k <= se) {
                    int16_t &z = blk[k];
                    if (z != 0) {
                        if (bit() && (z & p1) == 0) z = (int16_t)(z >= 0 ? z + p1 : z + m1);
                    } else {
                        if (r == 0) {
                            if (val) z = (int16_t)val;
                            ++k;
                            break;
                        }
                        --r;
                    }
                    ++k;
                }
            }
        }
        if (eobrun_ > 0) {
            for (; k <= se; ++k) {
                int16_t &z = blk[k];
                if (z != 0 && bit() && (z & p1) == 0) z = (int16_t)(z >= 0 ? z + p1 : z + m1);
            }
            --eobrun_;
        }
        return true;
    }

    bool scan() {
        if (pos_ + 2 > n_) return false;
        const size_t len = (size_t)(d_[pos_] << 8 | d_[pos_ + 1]);
        if (len < 6 || pos_ + len > n_) return false;
        const uint8_t *s = d_ + pos_ + 2;
        const int ns = s[0];
        if (ns < 1 || ns > 4 || len != (size_t)(6 + 2 * ns)) return false;
        std::vector<Component *> sc;
        for (int i = 0; i < ns; ++i) {
            Component *c = nullptr;
            for (Component &x : comps_)
                if (x.id == s[1 + 2 * i]) c = &x;
            if (!c) return false;
            c->td = s[2 + 2 * i] >> 4;
            c->ta = s[2 + 2 * i] & 15;
            if (c->td > 3 || c->ta > 3) return false;
            sc.push_back(c);
        }
        const int ss = s[1 + 2 * ns], se = s[2 + 2 * ns], ah = s[3 + 2 * ns] >> 4, al = s[3 + 2 * ns] & 15;
        pos_ += len;
        if (!progressive_ && (ss != 0 || se != 63 || ah != 0 || al != 0)) return false;
        if (progressive_ && (se > 63 || ss > se || (ss == 0 && se != 0) || (ss > 0 && ns != 1) || al > 13)) return false;
        for (Component *c : sc) {
            c->pred = 0;
            if ((!progressive_ || ss == 0) && ah == 0 && !dc_[c->td].present) return false;
            if ((!progressive_ || ss > 0) && !ac_[c->ta].present) return false;
        }
        eobrun_ = 0;
        reset_bits();
        auto do_block = [&](Component &c, int bx, int by) {
            int16_t *blk = &c.coef[((size_t)by * c.bw + bx) * 64];
            if (!progressive_) return block_baseline(c, blk);
            if (ss == 0) {
                if (ah == 0) return dc_first(c, blk, al);
                dc_refine(blk, al);
                return true;
            }
            return ah == 0 ? ac_first(c, blk, ss, se, al) : ac_refine(c, blk, ss, se, al);
        };
        int todo = restart_;
        if (ns == 1) {
            // non-interleaved: the component's own blocks in raster order, clipped to the image
            Component &c = *sc[0];
            const int cw = (width_ * c.h + 8 * hmax_ - 1) / (8 * hmax_), ch = (height_ * c.v + 8 * vmax_ - 1) / (8 * vmax_);
            for (int by = 0; by < ch; ++by)
                for (int bx = 0; bx < cw; ++bx) {
                    if (restart_ && todo == 0) {
                        if (!restart_marker()) return false;
                        todo = restart_;
                    }
                    if (!do_block(c, bx, by)) return false;
                    if (restart_) --todo;
                }
        } else {
            for (int my = 0; my < mcuy_; ++my)
                for (int mx = 0; mx < mcux_; ++mx) {
                    if (restart_ && todo == 0) {
                        if (!restart_marker()) return false;
                        todo = restart_;
                    }
                    for (Component *c : sc)
                        for (int v = 0; v < c->v; ++v)
                            for (int h = 0; h < c->h; ++h)
                                if (!do_block(*c, mx * c->h + h, my * c->v + v)) return false;
                    if (restart_) --todo;
                }
        }
        // skip to the next marker (the rest of this segment, if the scan ended early)
        reset_bits();
        while (pos_ + 1 < n_ && !(d_[pos_] == 0xFF && d_[pos_ + 1] != 0x00 && !(d_[pos_ + 1] >= 0xD0 && d_[pos_ + 1] <= 0xD7)))
            ++pos_;
        return true;
    }

    // ---- reconstruction ------------------------------------------------------------------------
    bool output(std::vector<uint8_t> &rgba, uint32_t &w, uint32_t &h) {
        // cos((2x + 1) u pi / 16) * C(u) / 2, the 1-D factor of T.81 A.3.3's inverse DCT
        float basis[8][8];
        for (int x = 0; x < 8; ++x)
            for (int u = 0; u < 8; ++u)
                basis[x][u] = (float)((u == 0 ? std::sqrt(0.5) : 1.0) * std::cos((2 * x + 1) * u * kPi / 16.0) * 0.5);
        // every component's samples, dequantised and transformed block by block
        std::vector<std::vector<uint8_t>> planes(comps_.size());
        for (size_t ci = 0; ci < comps_.size(); ++ci) {
            Component &c = comps_[ci];
            const int pw = c.bw * 8;
            planes[ci].assign((size_t)pw * c.bh * 8, 0);
            const int *q = qt_[c.tq];
            for (int by = 0; by < c.bh; ++by)
                for (int bx = 0; bx < c.bw; ++bx) {
                    const int16_t *blk = &c.coef[((size_t)by * c.bw + bx) * 64];
                    float f[64], tmp[64];
                    for (int k = 0; k < 64; ++k) f[kZigzag[k]] = (float)blk[k] * (float)q[k];
                    for (int y = 0; y < 8; ++y)  // rows: tmp[v][x] = sum_u basis[x][u] f[v][u]
                        for (int x = 0; x < 8; ++x) {
                            float a = 0.0f;
                            for (int u = 0; u < 8; ++u) a += basis[x][u] * f[y * 8 + u];
                            tmp[y * 8 + x] = a;
                        }
                    for (int y = 0; y < 8; ++y)
                        for (int x = 0; x < 8; ++x) {
                            float a = 0.0f;
                            for (int v = 0; v < 8; ++v) a += basis[y][v] * tmp[v * 8 + x];
                            const float s = std::nearbyint(a + 128.0f);
                            planes[ci][(size_t)(by * 8 + y) * pw + bx * 8 + x] =
                                (uint8_t)(s < 0.0f ? 0.0f : (s > 255.0f ? 255.0f : s));
                        }
                }
        }
        w = (uint32_t)width_;
        h = (uint32_t)height_;
        rgba.assign((size_t)w * h * 4, 255);
        auto sample = [&](size_t ci, int x, int y) {
            const Component &c = comps_[ci];
            const int sx = x * c.h / hmax_, sy = y * c.v / vmax_;  // replication upsampling
            return (float)planes[ci][(size_t)sy * c.bw * 8 + sx];
        };
        for (int y = 0; y < height_; ++y)
            for (int x = 0; x < width_; ++x) {
                uint8_t *o = &rgba[((size_t)y * w + x) * 4];
                if (comps_.size() == 1) {
                    o[0] = o[1] = o[2] = (uint8_t)sample(0, x, y);
                    continue;
                }
                const float Y = sample(0, x, y), cb = sample(1, x, y) - 128.0f, cr = sample(2, x, y) - 128.0f;
                float rgb[3] = {Y + 1.402f * cr, Y - 0.344136f * cb - 0.714136f * cr, Y + 1.772f * cb};
                if (adobe_ == 0) {  // Adobe transform 0: the components are RGB already
                    rgb[0] = Y;
                    rgb[1] = cb + 128.0f;
                    rgb[2] = cr + 128.0f;
                }
                for (int k = 0; k < 3; ++k) {
                    const float v = std::nearbyint(rgb[k]);
                    o[k] = (uint8_t)(v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v));
                }
            }
        return true;
    }
};

}  // namespace

// Decodes a JPEG image to RGBA8 (alpha 255).  With out == NULL (or too small) only the size is
// returned: call once for the size, then again with w * h * 4 bytes.  RT_ERR_INVALID_ARGUMENT for a
// stream this decoder does not handle (see above).
extern "C" int rt_jpeg_decode(const uint8_t *data, uint64_t n, uint8_t *out_rgba, uint64_t out_bytes, uint32_t *w,
                              uint32_t *h) {
    rt::clear_error();
    if (!data || !w || !h) {
        rt::set_error("rt_jpeg_decode: null argument");
        return RT_ERR_INVALID_ARGUMENT;
    }
    std::vector<uint8_t> rgba;
    uint32_t ww = 0, hh = 0;
    bool ok = false;
    try {  // a huge declared frame can exhaust host memory; no exception crosses the C ABI
        Decoder dec(data, (size_t)n);
        ok = dec.decode(rgba, ww, hh);
    } catch (const std::bad_alloc &) {
        rt::set_error("rt_jpeg_decode: out of host memory for a %ux%u image", ww, hh);
        return RT_ERR_OUT_OF_MEMORY;
    }
    if (!ok) {
        rt::set_error("rt_jpeg_decode: not a JPEG stream this decoder handles (baseline / extended / progressive "
                      "Huffman, 8-bit, 1 or 3 components)");
        return RT_ERR_INVALID_ARGUMENT;
    }
    *w = ww;
    *h = hh;
    if (out_rgba && out_bytes >= rgba.size()) std::memcpy(out_rgba, rgba.data(), rgba.size());
    return RT_OK;
}
