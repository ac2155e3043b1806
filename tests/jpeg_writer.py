"""A small JPEG encoder for the decoder's tests (test infrastructure, written from ITU-T T.81).

Baseline sequential (interleaved, optional 4:2:0 chroma, optional restart interval) and progressive
(spectral selection, with or without successive approximation of DC and AC coefficients) frames
over the same quantised coefficients, so a progressive file must decode to exactly the baseline
file's image.  Huffman tables are built per file from the symbol counts (T.81 K.2, code lengths
limited to 16 bits as in K.3).
"""
from __future__ import annotations

import struct

import numpy as np

ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13,
                   6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52, 45,
                   38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])


def _dct_matrix():
    c = np.zeros((8, 8))
    for u in range(8):
        for x in range(8):
            c[u, x] = (np.sqrt(0.5) if u == 0 else 1.0) * np.cos((2 * x + 1) * u * np.pi / 16) * 0.5
    return c


DCT = _dct_matrix()


class BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def bits(self, v: int, n: int):
        for i in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((v >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc, self.n = 0, 0

    def flush(self):
        if self.n:
            self.bits((1 << (8 - self.n)) - 1, 8 - self.n)


def _category(v: int) -> int:
    return 0 if v == 0 else int(abs(v)).bit_length()


def _bits_of(v: int, s: int) -> int:
    return v if v >= 0 else v + (1 << s) - 1


def huffman_table(freq: dict[int, int]) -> tuple[list[int], list[int]]:
    """(BITS[1..16], HUFFVAL) for symbol frequencies: T.81 K.2 code sizes, K.3 length limiting."""
    f = dict(freq)
    f[256] = 1  # reserved so no code is all ones
    size = {s: 0 for s in f}
    others = {s: -1 for s in f}
    live = dict(f)
    while len(live) > 1:
        # the two least frequent trees merge; v1 (the head of the merged chain) stays live
        v1 = min(live, key=lambda s: (live[s], -s))
        c1 = live.pop(v1)
        v2 = min(live, key=lambda s: (live[s], -s))
        live[v1] = c1 + live.pop(v2)
        x = v1
        while True:
            size[x] += 1
            if others[x] == -1:
                break
            x = others[x]
        others[x] = v2
        x = v2
        while True:
            size[x] += 1
            if others[x] == -1:
                break
            x = others[x]
    bits = [0] * 33
    for s, n in size.items():
        if n:
            bits[n] += 1
    i = 32
    while i > 16:
        while bits[i] > 0:
            j = i - 2
            while bits[j] == 0:
                j -= 1
            bits[i] -= 2
            bits[i - 1] += 1
            bits[j + 1] += 2
            bits[j] -= 1
        i -= 1
    while bits[i] == 0:
        i -= 1
    bits[i] -= 1  # drop the reserved symbol's code
    order = sorted((s for s in size if s != 256), key=lambda s: (size[s], s))
    return bits[1:17], order


def _codes(bits, vals):
    codes, code, k = {}, 0, 0
    for length in range(1, 17):
        for _ in range(bits[length - 1]):
            codes[vals[k]] = (code, length)
            code += 1
            k += 1
        code <<= 1
    return codes


class _Sym:
    """Symbol stream of one scan, replayed once the table is built."""

    def __init__(self):
        self.items = []  # ("sym", table, value) or ("bits", value, n)

    def sym(self, table, v):
        self.items.append(("sym", table, v))

    def bits(self, v, n):
        if n:
            self.items.append(("bits", v, n))


def _emit_scan(stream: _Sym, tables: dict) -> bytes:
    w = BitWriter()
    for it in stream.items:
        if it[0] == "sym":
            code, n = tables[it[1]][it[2]]
            w.bits(code, n)
        elif it[0] == "bits":
            w.bits(it[1], it[2])
        else:  # restart marker
            w.flush()
            w.out += bytes([0xFF, 0xD0 + it[1]])
    w.flush()
    return bytes(w.out)


def _coefficients(img: np.ndarray, subsample: bool, q: np.ndarray):
    """Per component (h, v, quantised blocks [by, bx, 64] in zig-zag order)."""
    img = img.astype(np.float64)
    if img.ndim == 2:
        planes, factors = [img], [(1, 1)]
    else:
        r, g, b = img[..., 0], img[..., 1], img[..., 2]
        y = 0.299 * r + 0.587 * g + 0.114 * b
        cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128
        cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128
        planes = [y, cb, cr]
        factors = [(2, 2), (1, 1), (1, 1)] if subsample else [(1, 1)] * 3
    hmax = max(f[0] for f in factors)
    vmax = max(f[1] for f in factors)
    H, W = img.shape[:2]
    mcux, mcuy = -(-W // (8 * hmax)), -(-H // (8 * vmax))
    comps = []
    for plane, (h, v) in zip(planes, factors):
        if (h, v) != (hmax, vmax):  # box-filtered chroma at half resolution
            ph, pw = -(-H // 2) * 2, -(-W // 2) * 2
            pp = np.pad(plane, ((0, ph - H), (0, pw - W)), mode="edge")
            plane = pp.reshape(ph // 2, 2, pw // 2, 2).mean((1, 3))
        bw, bh = mcux * h, mcuy * v
        pp = np.pad(plane, ((0, bh * 8 - plane.shape[0]), (0, bw * 8 - plane.shape[1])), mode="edge") - 128.0
        blocks = pp.reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3)
        coef = np.einsum("ux,abxy,vy->abuv", DCT, blocks, DCT)
        qb = np.rint(coef / q.reshape(8, 8)).astype(np.int64).reshape(bh, bw, 64)[..., ZIGZAG]
        comps.append((h, v, qb))
    return comps, mcux, mcuy, W, H


def _headers(W, H, comps, q, progressive):
    out = bytearray(b"\xff\xd8")
    out += b"\xff\xe0" + struct.pack(">H", 16) + b"JFIF\x00\x01\x02\x00\x00\x01\x00\x01\x00\x00"
    out += b"\xff\xdb" + struct.pack(">HB", 67, 0) + bytes(int(x) for x in q[ZIGZAG])
    sof = b"\xff\xc2" if progressive else b"\xff\xc0"
    body = struct.pack(">BHHB", 8, H, W, len(comps))
    for i, (h, v, _) in enumerate(comps):
        body += struct.pack(">BBB", i + 1, (h << 4) | v, 0)
    out += sof + struct.pack(">H", 2 + len(body)) + body
    return out


def _dht(tc, th, bits, vals):
    body = bytes([(tc << 4) | th]) + bytes(bits) + bytes(vals)
    return b"\xff\xc4" + struct.pack(">H", 2 + len(body)) + body


def _sos(comp_ids, tables, ss, se, ah, al):
    body = bytes([len(comp_ids)])
    for cid, (td, ta) in zip(comp_ids, tables):
        body += bytes([cid, (td << 4) | ta])
    body += bytes([ss, se, (ah << 4) | al])
    return b"\xff\xda" + struct.pack(">H", 2 + len(body)) + body


def _finish_scan(out: bytearray, stream: _Sym, comp_ids, n_tables_dc, n_tables_ac, ss, se, ah, al, sel):
    """Builds the scan's tables from its symbols, writes DHT + SOS + data."""
    freqs = {}
    for it in stream.items:
        if it[0] == "sym":
            freqs.setdefault(it[1], {}).setdefault(it[2], 0)
            freqs[it[1]][it[2]] += 1
    codes = {}
    for key, f in sorted(freqs.items()):
        bits, vals = huffman_table(f)
        out += _dht(0 if key[0] == "dc" else 1, key[1], bits, vals)
        codes[key] = _codes(bits, vals)
    out += _sos(comp_ids, sel, ss, se, ah, al)
    out += _emit_scan(stream, codes)


def encode_baseline(img: np.ndarray, q: np.ndarray, subsample: bool = False, restart: int = 0) -> bytes:
    comps, mcux, mcuy, W, H = _coefficients(img, subsample, q)
    out = _headers(W, H, comps, q, False)
    if restart:
        out += b"\xff\xdd" + struct.pack(">HH", 4, restart)
    st = _Sym()
    pred = [0] * len(comps)
    mcu = 0
    tsel = [(0, 0)] + [(1, 1)] * (len(comps) - 1)
    for my in range(mcuy):
        for mx in range(mcux):
            if restart and mcu and mcu % restart == 0:
                st.items.append(("rst", (mcu // restart - 1) % 8))
                pred = [0] * len(comps)
            for ci, (h, v, qb) in enumerate(comps):
                dct, act = ("dc", tsel[ci][0]), ("ac", tsel[ci][1])
                for by in range(v):
                    for bx in range(h):
                        blk = qb[my * v + by, mx * h + bx]
                        d = int(blk[0]) - pred[ci]
                        pred[ci] = int(blk[0])
                        s = _category(d)
                        st.sym(dct, s)
                        st.bits(_bits_of(d, s), s)
                        run = 0
                        for k in range(1, 64):
                            c = int(blk[k])
                            if c == 0:
                                run += 1
                                continue
                            while run > 15:
                                st.sym(act, 0xF0)
                                run -= 16
                            s = _category(c)
                            st.sym(act, (run << 4) | s)
                            st.bits(_bits_of(c, s), s)
                            run = 0
                        if run:
                            st.sym(act, 0x00)
            mcu += 1
    _finish_scan(out, st, list(range(1, len(comps) + 1)), 2, 2, 0, 63, 0, 0, tsel)
    out += b"\xff\xd9"
    return bytes(out)


def _shift(c: int, al: int) -> int:
    """Point transform of an AC coefficient (toward zero)."""
    return -((-c) >> al) if c < 0 else c >> al


def encode_progressive(img: np.ndarray, q: np.ndarray, subsample: bool = False, approx: bool = False) -> bytes:
    """Scans: DC of all components (Al = 1 with approx), the AC bands 1-5 and 6-63 of luma and 1-63 of
    each chroma component (Al = 1 with approx), then with approx the DC and AC refinement scans."""
    comps, mcux, mcuy, W, H = _coefficients(img, subsample, q)
    out = _headers(W, H, comps, q, True)
    al0 = 1 if approx else 0
    nc = len(comps)

    def comp_blocks(ci):
        h, v, qb = comps[ci]
        cw, ch = -(-(W * h) // (8 * max(c[0] for c in comps))), -(-(H * v) // (8 * max(c[1] for c in comps)))
        for by in range(ch):
            for bx in range(cw):
                yield qb[by, bx]

    # DC first (interleaved)
    st = _Sym()
    pred = [0] * nc
    for my in range(mcuy):
        for mx in range(mcux):
            for ci, (h, v, qb) in enumerate(comps):
                for by in range(v):
                    for bx in range(h):
                        val = int(qb[my * v + by, mx * h + bx][0]) >> al0  # DC: arithmetic shift
                        d = val - pred[ci]
                        pred[ci] = val
                        s = _category(d)
                        st.sym(("dc", 0), s)
                        st.bits(_bits_of(d, s), s)
    _finish_scan(out, st, list(range(1, nc + 1)), 1, 0, 0, 0, 0, al0, [(0, 0)] * nc)

    bands = [(0, 1, 5), (0, 6, 63)] + [(ci, 1, 63) for ci in range(1, nc)]
    for ci, ss, se in bands:
        st = _Sym()
        eobrun = 0

        def flush_eob():
            nonlocal eobrun
            if eobrun:
                nb = eobrun.bit_length() - 1
                st.sym(("ac", 0), nb << 4)
                st.bits(eobrun & ((1 << nb) - 1), nb)
                eobrun = 0

        for blk in comp_blocks(ci):
            vals = [_shift(int(blk[k]), al0) for k in range(ss, se + 1)]
            if not any(vals):
                eobrun += 1
                if eobrun == 0x7FFF:
                    flush_eob()
                continue
            flush_eob()
            last = max(i for i, x in enumerate(vals) if x)
            run = 0
            for i, c in enumerate(vals[:last + 1]):
                if c == 0:
                    run += 1
                    continue
                while run > 15:
                    st.sym(("ac", 0), 0xF0)
                    run -= 16
                s = _category(c)
                st.sym(("ac", 0), (run << 4) | s)
                st.bits(_bits_of(c, s), s)
                run = 0
            if last < len(vals) - 1:
                eobrun += 1
                if eobrun == 0x7FFF:
                    flush_eob()
        flush_eob()
        _finish_scan(out, st, [ci + 1], 0, 1, ss, se, 0, al0, [(0, 0)])

    if approx:
        # DC refinement: the bit Al = 0 of every DC value, interleaved, no Huffman symbols
        st = _Sym()
        for my in range(mcuy):
            for mx in range(mcux):
                for ci, (h, v, qb) in enumerate(comps):
                    for by in range(v):
                        for bx in range(h):
                            st.bits(int(qb[my * v + by, mx * h + bx][0]) & 1, 1)
        out += _sos(list(range(1, nc + 1)), [(0, 0)] * nc, 0, 0, 1, 0)
        out += _emit_scan(st, {})
        for ci, ss, se in bands:
            st = _Sym()
            eobrun, be = 0, []

            def flush_eob():
                nonlocal eobrun, be
                if eobrun:
                    nb = eobrun.bit_length() - 1
                    st.sym(("ac", 0), nb << 4)
                    st.bits(eobrun & ((1 << nb) - 1), nb)
                    eobrun = 0
                    for b in be:
                        st.bits(b, 1)
                    be = []

            for blk in comp_blocks(ci):
                absval = [abs(int(blk[k])) for k in range(ss, se + 1)]  # Al = 0: the full magnitudes
                newly = [i for i, a in enumerate(absval) if a == 1]
                eob = newly[-1] if newly else -1
                run, br = 0, []
                for i, a in enumerate(absval):
                    if a == 0:
                        run += 1
                        continue
                    while run > 15 and i <= eob:
                        flush_eob()
                        st.sym(("ac", 0), 0xF0)
                        run -= 16
                        for b in br:
                            st.bits(b, 1)
                        br = []
                    if a > 1:
                        br.append(a & 1)
                        continue
                    flush_eob()
                    st.sym(("ac", 0), (run << 4) | 1)
                    st.bits(0 if int(blk[ss + i]) < 0 else 1, 1)
                    for b in br:
                        st.bits(b, 1)
                    br = []
                    run = 0
                if run > 0 or br:
                    eobrun += 1
                    be += br
                    if eobrun == 0x7FFF or len(be) > 900:
                        flush_eob()
            flush_eob()
            _finish_scan(out, st, [ci + 1], 0, 1, ss, se, 1, 0, [(0, 0)])
    out += b"\xff\xd9"
    return bytes(out)
