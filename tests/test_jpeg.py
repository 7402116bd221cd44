"""JPEG materials (main.rs:172-185 accepts jpg/jpeg; main.rs:492/548 image::open),
decoded by csrc/io_jpeg.cpp, on the CPU.

The files are written here by a small encoder of this test's own (ITU-T T.81:
JFIF YCbCr, FDCT in float64, quantisation, DC/AC Huffman codes built from the
symbol counts of the image, optional restart intervals, one interleaved scan
or one scan per component, 4:4:4 / 4:2:2 / 4:2:0 / grey; and the same
coefficients as progressive files by a scan script of spectral bands and
successive-approximation bit planes).
Because the encoder keeps the quantised coefficients, the decoder can be held
to a float32 restatement of its own output steps (T.81 A.3.3 inverse DCT in
the same order, replication upsampling, the JFIF colour equations) bit for
bit, and to the source pixels where the codec loses nothing (grey blocks of one
level at quantiser 1).  Parity with zune-jpeg (the reference's decoder) is not
pinned.  Defective files fail with MG_ERR_ARG and never crash.
"""
import heapq
import math
import struct

import numpy as np
import pytest

ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20,
                   13, 6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52,
                   45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])


@pytest.fixture(scope="module")
def capi(built):
    from mosaic_gpu import _capi

    return _capi


# ---- the test's encoder ----------------------------------------------------------------------
def _dct_matrix():
    m = np.zeros((8, 8))
    for u in range(8):
        for x in range(8):
            m[u, x] = (math.sqrt(0.5) if u == 0 else 1.0) * 0.5 * math.cos((2 * x + 1) * u * math.pi / 16)
    return m


def _blocks(plane, bw, bh):
    """(bh, bw, 8, 8) blocks of a plane padded by edge replication."""
    h, w = plane.shape
    p = np.pad(plane, ((0, bh * 8 - h), (0, bw * 8 - w)), mode="edge")
    return p.reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3)


def _category(v):
    return 0 if v == 0 else int(abs(v)).bit_length()


def _huffman_lengths(freq):
    """Code lengths (<= 16) for the symbols of `freq` (dict symbol -> count)."""
    syms = sorted(freq)
    if len(syms) == 1:
        return {syms[0]: 1}
    heap = [(freq[s], i, [s]) for i, s in enumerate(syms)]
    heapq.heapify(heap)
    depth = {s: 0 for s in syms}
    k = len(syms)
    while len(heap) > 1:
        a, b = heapq.heappop(heap), heapq.heappop(heap)
        for s in a[2] + b[2]:
            depth[s] += 1
        heapq.heappush(heap, (a[0] + b[0], k, a[2] + b[2]))
        k += 1
    if max(depth.values()) > 15 or len(syms) >= 2 ** max(depth.values()):
        L = max(1, math.ceil(math.log2(len(syms) + 1)))  # fixed length: never an all-ones code
        return {s: L for s in syms}
    # a canonical code must not use the all-ones word of its longest length: move one
    # longest symbol down a level when the lengths fill the code space exactly
    if sum(2.0 ** -d for d in depth.values()) == 1.0:
        worst = max(syms, key=lambda s: (depth[s], s))
        depth[worst] += 1
    return depth


def _canonical(lengths):
    """(counts per length 1..16, symbols in order, code of each symbol)."""
    order = sorted(lengths, key=lambda s: (lengths[s], s))
    counts = [0] * 16
    for s in order:
        counts[lengths[s] - 1] += 1
    codes, code, prev = {}, 0, lengths[order[0]]
    for s in order:
        code <<= lengths[s] - prev
        prev = lengths[s]
        codes[s] = (code, lengths[s])
        code += 1
    return counts, order, codes


class _BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, value, bits):
        for i in range(bits - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc, self.n = 0, 0

    def pad(self):
        while self.n:
            self.put(1, 1)


def _segment(marker, payload):
    return bytes([0xFF, marker]) + struct.pack(">H", len(payload) + 2) + payload


def _coefficients(img, sampling, quant, grey, rgb_ids=None):
    """The quantised DCT coefficients of each component: ({cid: (bh, bw, 64) natural
    order}, [(cid, h, v)], {cid: the component's own block grid (bx, by)}, mcux, mcuy).
    rgb_ids: the three component ids of an image stored as R, G, B (no YCbCr)."""
    if grey:
        planes = [img.astype(np.float64)]
        comps = [(1, 1, 1)]
    elif rgb_ids:
        planes = [img[..., i].astype(np.float64) for i in range(3)]
        comps = [(rgb_ids[0], sampling[0], sampling[1]), (rgb_ids[1], 1, 1), (rgb_ids[2], 1, 1)]
    else:
        r, g, b = (img[..., i].astype(np.float64) for i in range(3))
        y = np.clip(np.floor(0.299 * r + 0.587 * g + 0.114 * b + 0.5), 0, 255)
        cb = np.clip(np.floor(-0.168736 * r - 0.331264 * g + 0.5 * b + 128.5), 0, 255)
        cr = np.clip(np.floor(0.5 * r - 0.418688 * g - 0.081312 * b + 128.5), 0, 255)
        planes = [y, cb, cr]
        comps = [(1, sampling[0], sampling[1]), (2, 1, 1), (3, 1, 1)]
    H, W = img.shape[:2]
    hmax = max(c[1] for c in comps)
    vmax = max(c[2] for c in comps)
    mcux, mcuy = -(-W // (8 * hmax)), -(-H // (8 * vmax))
    D = _dct_matrix()
    coefs, scan_blocks = {}, {}
    for (cid, hs, vs), plane in zip(comps, planes):
        # chroma: the mean of each hmax/hs x vmax/vs box
        fx, fy = hmax // hs, vmax // vs
        cw, ch = -(-W * hs // hmax), -(-H * vs // vmax)
        pp = np.pad(plane, ((0, ch * fy - H), (0, cw * fx - W)), mode="edge")
        sub = np.floor(pp.reshape(ch, fy, cw, fx).mean(axis=(1, 3)) + 0.5)
        bw, bh = mcux * hs, mcuy * vs
        blk = _blocks(sub - 128.0, bw, bh)
        F = np.einsum("vy,bcyx,ux->bcvu", D, blk, D)  # natural order: [vertical v][horizontal u]
        q = np.floor(F / quant + 0.5).astype(np.int32)
        coefs[cid] = q.reshape(bh, bw, 64)
        scan_blocks[cid] = (-(-cw // 8), -(-ch // 8))  # the component's own grid (one-component scans)
    return coefs, comps, scan_blocks, mcux, mcuy


def _unit_order(cid_list, comps, scan_blocks, mcux, mcuy):
    """The scan's units, each a list of (cid, block row, block column): a
    one-component scan walks the component's own grid, an interleaved one the MCUs."""
    if len(cid_list) == 1:
        cid = cid_list[0]
        bx, by = scan_blocks[cid]
        return [[(cid, y, x)] for y in range(by) for x in range(bx)]
    units = []
    for uy in range(mcuy):
        for ux in range(mcux):
            units.append([(cid, uy * vs + y, ux * hs + x) for (cid, hs, vs) in comps if cid in cid_list
                          for y in range(vs) for x in range(hs)])
    return units


def _headers(comps, quant, grey, H, W, sof_marker, app="jfif"):
    """app: "jfif" (an APP0 JFIF segment), "adobe0" / "adobe1" (an APP14 Adobe
    segment, colour transform 0 or 1, no JFIF) or "none"."""
    out = b"\xff\xd8"
    if app == "jfif":
        out += _segment(0xE0, b"JFIF\x00\x01\x02\x00\x00\x01\x00\x01\x00\x00")
    elif app.startswith("adobe"):
        out += _segment(0xEE, b"Adobe" + struct.pack(">HHHB", 100, 0, 0, int(app[-1])))
    out += _segment(0xDB, bytes([0]) + bytes([quant] * 64) + (bytes([1]) + bytes([quant] * 64) if not grey else b""))
    sof = struct.pack(">BHHB", 8, H, W, len(comps))
    for cid, hs, vs in comps:
        sof += bytes([cid, (hs << 4) | vs, 0 if cid == comps[0][0] else 1])
    return out + _segment(sof_marker, sof)


def encode_jpeg(img, sampling=(1, 1), quant=1, restart=0, interleaved=True, grey=False, rgb_ids=None, app="jfif"):
    """img: (h, w, 3) uint8 (or (h, w) for grey).  sampling: the luma factors (h, v)
    with chroma at 1x1.  quant: one quantiser for every coefficient.  Returns
    (file bytes, {component: quantised coefficients (bh, bw, 64) natural order}, planes)."""
    H, W = img.shape[:2]
    coefs, comps, scan_blocks, mcux, mcuy = _coefficients(img, sampling, quant, grey, rgb_ids)

    # entropy-code the scans, collecting symbols first for the Huffman codes
    def mcu_order(cid_list):
        if len(cid_list) == 1:
            cid = cid_list[0]
            bx, by = scan_blocks[cid]
            return [(cid, y, x) for y in range(by) for x in range(bx)], bx * by
        units = []
        for uy in range(mcuy):
            for ux in range(mcux):
                u = []
                for (cid, hs, vs) in comps:
                    for y in range(vs):
                        for x in range(hs):
                            u.append((cid, uy * vs + y, ux * hs + x))
                units.append(u)
        return units, mcux * mcuy

    scans = [[c[0] for c in comps]] if interleaved or grey else [[c[0]] for c in comps]
    tables = {cid: (0 if cid == comps[0][0] else 1) for cid, _, _ in comps}
    symbols = {("dc", 0): {}, ("dc", 1): {}, ("ac", 0): {}, ("ac", 1): {}}
    streams = []
    for sc in scans:
        order, units = mcu_order(sc)
        if len(sc) == 1:
            order = [[o] for o in order]
        events = []  # per unit: list of (table kind, table id, symbol, extra value, extra bits)
        pred = {cid: 0 for cid in sc}
        for ui, unit in enumerate(order):
            if restart and ui and ui % restart == 0:
                events.append(("rst", (ui // restart - 1) % 8))
                pred = {cid: 0 for cid in sc}
            for cid, by, bx in unit:
                t = tables[cid]
                zz = coefs[cid][by, bx][ZIGZAG]
                diff = int(zz[0]) - pred[cid]
                pred[cid] = int(zz[0])
                s = _category(diff)
                events.append(("dc", t, s, diff if diff >= 0 else diff + (1 << s) - 1, s))
                run = 0
                last = max([i for i in range(1, 64) if zz[i] != 0], default=0)
                for k in range(1, last + 1):
                    v = int(zz[k])
                    if v == 0:
                        run += 1
                        continue
                    while run > 15:
                        events.append(("ac", t, 0xF0, 0, 0))
                        run -= 16
                    s = _category(v)
                    events.append(("ac", t, (run << 4) | s, v if v >= 0 else v + (1 << s) - 1, s))
                    run = 0
                if last < 63:
                    events.append(("ac", t, 0x00, 0, 0))
        for e in events:
            if e[0] != "rst":
                d = symbols[(e[0], e[1])]
                d[e[2]] = d.get(e[2], 0) + 1
        streams.append((sc, events))
    codes, dht = {}, b""
    for (kind, t), freq in symbols.items():
        if not freq:
            continue
        counts, order, code = _canonical(_huffman_lengths(freq))
        codes[(kind, t)] = code
        dht += bytes([(0 if kind == "dc" else 16) | t]) + bytes(counts) + bytes(order)
    out = _headers(comps, quant, grey, H, W, 0xC0, app) + _segment(0xC4, dht)
    if restart:
        out += _segment(0xDD, struct.pack(">H", restart))
    for sc, events in streams:
        sos = bytes([len(sc)])
        for cid in sc:
            t = tables[cid]
            sos += bytes([cid, (t << 4) | t])
        out += _segment(0xDA, sos + bytes([0, 63, 0]))
        bw = _BitWriter()
        for e in events:
            if e[0] == "rst":
                bw.pad()
                bw.out += bytes([0xFF, 0xD0 + e[1]])
                continue
            c, n = codes[(e[0], e[1])][e[2]]
            bw.put(c, n)
            if e[4]:
                bw.put(e[3], e[4])
        bw.pad()
        out += bytes(bw.out)
    return out + b"\xff\xd9", coefs, comps


PROGRESSIVE_COLOUR = [((1, 2, 3), 0, 0, 0, 1), ((1,), 1, 5, 0, 2), ((3,), 1, 63, 0, 1), ((2,), 1, 63, 0, 1),
                      ((1,), 6, 63, 0, 2), ((1,), 1, 63, 2, 1), ((1, 2, 3), 0, 0, 1, 0), ((3,), 1, 63, 1, 0),
                      ((2,), 1, 63, 1, 0), ((1,), 1, 63, 1, 0)]
PROGRESSIVE_SEPARATE_DC = [((1,), 0, 0, 0, 2), ((2,), 0, 0, 0, 0), ((3,), 0, 0, 0, 0), ((1,), 1, 63, 0, 3),
                           ((1,), 0, 0, 2, 1), ((1,), 1, 63, 3, 2), ((1,), 1, 63, 2, 1), ((1,), 0, 0, 1, 0),
                           ((1,), 1, 9, 1, 0), ((1,), 10, 63, 1, 0), ((2,), 1, 63, 0, 0), ((3,), 1, 63, 0, 0)]
PROGRESSIVE_GREY = [((1,), 0, 0, 0, 1), ((1,), 1, 5, 0, 2), ((1,), 6, 63, 0, 2), ((1,), 1, 63, 2, 1),
                    ((1,), 0, 0, 1, 0), ((1,), 1, 63, 1, 0)]


def encode_jpeg_progressive(img, sampling=(1, 1), quant=1, restart=0, grey=False, script=None):
    """The same quantised coefficients as encode_jpeg, written as a progressive
    file (SOF2) by the scan script [(components, Ss, Se, Ah, Al)]: DC first and
    refinement scans, AC first scans with end-of-band runs, AC refinement scans
    with correction bits (T.81 G.1.2), a Huffman table per scan from its own
    symbol counts.  Returns (file bytes, coefficients, components)."""
    H, W = img.shape[:2]
    coefs, comps, scan_blocks, mcux, mcuy = _coefficients(img, sampling, quant, grey)
    script = script or (PROGRESSIVE_GREY if grey else PROGRESSIVE_COLOUR)
    out = _headers(comps, quant, grey, H, W, 0xC2)
    if restart:
        out += _segment(0xDD, struct.pack(">H", restart))
    for cids, ss, se, ah, al in script:
        units = _unit_order(list(cids), comps, scan_blocks, mcux, mcuy)
        ev = []  # ("sym", symbol, value, bits) | ("bits", value, bits) | ("rst", n)
        st = {"eobrun": 0, "be": []}

        def flush_eobrun():
            n = st["eobrun"]
            if n:
                nb = n.bit_length() - 1
                ev.append(("sym", nb << 4, n - (1 << nb), nb))
                for bit in st["be"]:
                    ev.append(("bits", bit, 1))
            st["eobrun"], st["be"] = 0, []

        pred = {c: 0 for c in cids}
        for ui, unit in enumerate(units):
            if restart and ui and ui % restart == 0:
                flush_eobrun()
                ev.append(("rst", (ui // restart - 1) % 8))
                pred = {c: 0 for c in cids}
            for cid, by, bx in unit:
                zz = [int(v) for v in coefs[cid][by, bx][ZIGZAG]]
                if ss == 0 and ah == 0:  # DC first: arithmetic shift by al, then the difference
                    v = zz[0] >> al
                    diff, pred[cid] = v - pred[cid], v
                    t = _category(diff)
                    ev.append(("sym", t, diff if diff >= 0 else diff + (1 << t) - 1, t))
                elif ss == 0:  # DC refinement: bit al
                    ev.append(("bits", (zz[0] >> al) & 1, 1))
                elif ah == 0:  # AC first: magnitudes shifted by al, signs kept
                    vals = [(1 if c > 0 else -1) * (abs(c) >> al) for c in zz[ss:se + 1]]
                    nz = [i for i, v in enumerate(vals) if v]
                    if not nz:
                        st["eobrun"] += 1
                        if st["eobrun"] == 0x7FFF:
                            flush_eobrun()
                        continue
                    flush_eobrun()
                    run = 0
                    for v in vals[:nz[-1] + 1]:
                        if v == 0:
                            run += 1
                            continue
                        while run > 15:
                            ev.append(("sym", 0xF0, 0, 0))
                            run -= 16
                        t = _category(v)
                        ev.append(("sym", (run << 4) | t, v if v >= 0 else v + (1 << t) - 1, t))
                        run = 0
                    if nz[-1] < len(vals) - 1:
                        st["eobrun"] += 1
                        if st["eobrun"] == 0x7FFF:
                            flush_eobrun()
                else:  # AC refinement at bit al
                    absv = [abs(c) >> al for c in zz[ss:se + 1]]
                    eob = max([i for i, t in enumerate(absv) if t == 1], default=-1)
                    r, br = 0, []
                    for i, t in enumerate(absv):
                        if t == 0:
                            r += 1
                            continue
                        while r > 15 and i <= eob:
                            flush_eobrun()
                            ev.append(("sym", 0xF0, 0, 0))
                            r -= 16
                            ev.extend(("bits", bit, 1) for bit in br)
                            br = []
                        if t > 1:
                            br.append(t & 1)
                            continue
                        flush_eobrun()
                        ev.append(("sym", (r << 4) | 1, 1 if zz[ss + i] > 0 else 0, 1))
                        ev.extend(("bits", bit, 1) for bit in br)
                        br, r = [], 0
                    if r > 0 or br:
                        st["eobrun"] += 1
                        st["be"] += br
                        if st["eobrun"] == 0x7FFF or len(st["be"]) > 937:
                            flush_eobrun()
        flush_eobrun()
        freq = {}
        for e in ev:
            if e[0] == "sym":
                freq[e[1]] = freq.get(e[1], 0) + 1
        code = {}
        if freq:
            counts, order, code = _canonical(_huffman_lengths(freq))
            out += _segment(0xC4, bytes([(0 if ss == 0 else 16)]) + bytes(counts) + bytes(order))
        sos = bytes([len(cids)])
        for cid in cids:
            sos += bytes([cid, 0])
        out += _segment(0xDA, sos + bytes([ss, se, (ah << 4) | al]))
        bw = _BitWriter()
        for e in ev:
            if e[0] == "rst":
                bw.pad()
                bw.out += bytes([0xFF, 0xD0 + e[1]])
            elif e[0] == "bits":
                bw.put(e[1], e[2])
            else:
                c, n = code[e[1]]
                bw.put(c, n)
                if e[3]:
                    bw.put(e[2], e[3])
        bw.pad()
        out += bytes(bw.out)
    return out + b"\xff\xd9", coefs, comps


def decode_restated(coefs, comps, quant, W, H, rgb=False):
    """The decoder's output steps in float32, in its order: dequantise, rows then
    columns of the T.81 A.3.3 inverse DCT, + 128, round, clamp; replicate chroma;
    JFIF colour equations; round, clamp."""
    cs = np.zeros((8, 8), np.float32)
    for x in range(8):
        for u in range(8):
            cs[x, u] = np.float32((math.sqrt(0.5) if u == 0 else 1.0) * 0.5 * math.cos((2 * x + 1) * u * math.pi / 16))
    hmax = max(c[1] for c in comps)
    vmax = max(c[2] for c in comps)
    planes = {}
    for cid, hs, vs in comps:
        q = coefs[cid]
        bh, bw = q.shape[:2]
        t = q.reshape(bh, bw, 8, 8).astype(np.float32) * np.float32(quant)
        r = np.zeros_like(t)
        for x in range(8):
            s = np.zeros(t.shape[:3], np.float32)
            for u in range(8):
                s = s + cs[x, u] * t[..., u]
            r[..., x] = s
        o = np.zeros_like(t)
        for y in range(8):
            s = np.zeros((bh, bw, 8), np.float32)
            for v in range(8):
                s = s + cs[y, v] * r[:, :, v, :]
            o[:, :, y, :] = s
        o = np.clip(np.rint(o + np.float32(128.0)), 0, 255).astype(np.uint8)
        planes[cid] = o.transpose(0, 2, 1, 3).reshape(bh * 8, bw * 8)
    if len(comps) == 1:
        g = planes[comps[0][0]][:H, :W]
        return np.stack([g, g, g], -1)
    ys = np.arange(H)
    xs = np.arange(W)
    chan = []
    for cid, hs, vs in comps:
        p = planes[cid]
        chan.append(p[(ys * vs // vmax)[:, None], (xs // (hmax // hs))[None, :]].astype(np.float32))
    if rgb:  # stored as R, G, B: the samples themselves
        return np.stack(chan, -1).astype(np.uint8)
    Y, cb, cr = chan[0], chan[1] - np.float32(128), chan[2] - np.float32(128)
    rgb = [Y + np.float32(1.402) * cr, Y - np.float32(0.344136) * cb - np.float32(0.714136) * cr,
           Y + np.float32(1.772) * cb]
    return np.stack([np.clip(np.rint(c), 0, 255) for c in rgb], -1).astype(np.uint8)


def _image(rng, w, h, kind):
    if kind == "noise":
        return rng.integers(0, 256, (h, w, 3)).astype(np.uint8)
    y, x = np.mgrid[0:h, 0:w]
    base = np.stack([(x * 255 // max(w - 1, 1)), (y * 255 // max(h - 1, 1)), ((x + 2 * y) * 3) % 256], -1)
    return np.clip(base + rng.integers(-6, 7, (h, w, 3)), 0, 255).astype(np.uint8)


CASES = [((1, 1), 1, 0, True), ((2, 2), 1, 0, True), ((2, 1), 2, 0, True), ((2, 2), 4, 5, True),
         ((1, 1), 3, 7, False), ((2, 2), 1, 0, False), ((1, 2), 8, 3, True)]


@pytest.mark.parametrize("sampling,quant,restart,interleaved", CASES)
@pytest.mark.parametrize("size", [(64, 48), (37, 29), (8, 8), (1, 1), (250, 3)])
def test_decode_equals_restated_steps(capi, sampling, quant, restart, interleaved, size):
    rng = np.random.default_rng(size[0] * 7 + quant)
    for kind in ("smooth", "noise"):
        img = _image(rng, *size, kind)
        data, coefs, comps = encode_jpeg(img, sampling, quant, restart, interleaved)
        assert capi.image_info(data) == size
        got = capi.image_decode(data)
        assert np.array_equal(got, decode_restated(coefs, comps, quant, *size)), (kind, sampling, restart)
        if quant == 1 and sampling == (1, 1) and kind == "smooth":
            # quantiser 1, no subsampling: close to the source.  YCbCr is rounded to 8 bits
            # both ways and every coefficient by up to 1/2; 1.772 x a chroma error of 2
            # plus the luma's gives the bar (observed 4)
            assert np.abs(got.astype(np.int16) - img.astype(np.int16)).max() <= 5


PROG_CASES = [((1, 1), 1, 0, False, None), ((2, 2), 2, 0, False, None), ((2, 1), 1, 3, False, None),
              ((2, 2), 4, 2, False, PROGRESSIVE_SEPARATE_DC), ((1, 2), 3, 0, False, PROGRESSIVE_SEPARATE_DC),
              ((1, 1), 1, 0, True, None), ((1, 1), 2, 4, True, None)]


@pytest.mark.parametrize("sampling,quant,restart,grey,script", PROG_CASES)
@pytest.mark.parametrize("size", [(64, 48), (37, 29), (8, 8), (1, 1), (250, 3), (130, 70)])
def test_progressive_decodes_like_the_sequential_file(capi, sampling, quant, restart, grey, script, size):
    """A progressive file (SOF2: DC first and refinement scans, interleaved or
    not; AC first scans over spectral bands with end-of-band runs; AC
    refinement scans with correction bits; restart intervals) carries the same
    quantised coefficients as the sequential file of the same image, so both
    decode to the same pixels -- and to the restated output steps."""
    rng = np.random.default_rng(size[0] * 13 + quant + 7 * restart)
    for kind in ("smooth", "noise"):
        img = _image(rng, *size, kind)
        if grey:
            img = img[..., 0]
        data, coefs, comps = encode_jpeg_progressive(img, sampling, quant, restart, grey, script)
        seq = encode_jpeg(img, sampling, quant, 0, True, grey)[0]
        assert capi.image_info(data) == size
        got = capi.image_decode(data)
        assert np.array_equal(got, capi.image_decode(seq)), (kind, sampling, restart, script is None)
        assert np.array_equal(got, decode_restated(coefs, comps, quant, *size)), kind


@pytest.mark.parametrize("ids,app,is_rgb", [((82, 71, 66), "none", True), ((1, 2, 3), "adobe0", True),
                                             ((82, 71, 66), "adobe0", True), ((82, 71, 66), "jfif", False),
                                             ((1, 2, 3), "adobe1", False), ((1, 2, 3), "none", False)])
def test_rgb_coded_files(capi, ids, app, is_rgb):
    """Three components stored as R, G, B (no YCbCr): an Adobe segment with
    colour transform 0, or no JFIF / Adobe segment and components named 'R',
    'G', 'B'; a JFIF segment or an Adobe transform of 1 means YCbCr whatever the
    names."""
    rng = np.random.default_rng(sum(ids) + len(app))
    img = _image(rng, 45, 31, "smooth")
    for sampling in ((1, 1), (2, 2)):
        data, coefs, comps = encode_jpeg(img, sampling, 2, 0, True, rgb_ids=ids, app=app)
        got = capi.image_decode(data)
        assert np.array_equal(got, decode_restated(coefs, comps, 2, 45, 31, rgb=is_rgb)), sampling


def test_grey_blocks_decode_exactly(capi):
    """A grey image of 8x8 blocks of one level each, at quantiser 1: every block is
    its DC term alone, so the decoded pixels are the source's."""
    rng = np.random.default_rng(3)
    levels = rng.integers(0, 256, (6, 9))
    img = np.kron(levels, np.ones((8, 8), int)).astype(np.uint8)
    for restart in (0, 2):
        data, _, _ = encode_jpeg(img, quant=1, restart=restart, grey=True)
        got = capi.image_decode(data)
        assert np.array_equal(got, np.stack([img] * 3, -1))


def test_solid_colours_stay_close(capi):
    """main.rs:822-825 style: a solid red tile decodes to red (within the colour conversion's rounding)."""
    for rgb in ((255, 0, 0), (0, 255, 0), (0, 0, 255), (128, 128, 128), (12, 200, 77)):
        img = np.zeros((32, 24, 3), np.uint8) + np.array(rgb, np.uint8)
        data, _, _ = encode_jpeg(img, (2, 2), quant=2)
        got = capi.image_decode(data)
        assert np.abs(got.astype(np.int16) - img.astype(np.int16)).max() <= 3, rgb


def test_defects_fail_cleanly(capi):
    from mosaic_gpu import _capi

    rng = np.random.default_rng(9)
    img = _image(rng, 40, 24, "smooth")
    data, _, _ = encode_jpeg(img, (2, 2), 2, restart=3)
    lib = _capi.load()
    out = np.zeros((64, 64, 3), np.uint8)

    def code(d):
        return lib.mg_image_decode(d, len(d), _capi.ptr(out, np.ctypeslib.ctypes.c_uint8), 64 * 3)

    assert code(data) == _capi.MG_OK
    prog = data.replace(b"\xff\xc0", b"\xff\xc2", 1)  # a sequential scan in a progressive frame
    assert code(prog) == _capi.MG_ERR_ARG and b"progressive" in lib.mg_last_error()
    assert code(data.replace(b"\xff\xc0", b"\xff\xc3", 1)) == _capi.MG_ERR_ARG  # lossless
    assert code(data[:2] + b"\xff\xcc\x00\x04\x00\x00" + data[2:]) == _capi.MG_ERR_ARG  # arithmetic coding
    for cut in range(0, len(data), 3):  # truncation anywhere: an error or a decode, never a crash
        assert code(data[:cut]) in (_capi.MG_OK, _capi.MG_ERR_ARG)
    for _ in range(300):  # random bit flips
        b = bytearray(data)
        i = int(rng.integers(0, len(b)))
        b[i] ^= 1 << int(rng.integers(0, 8))
        assert code(bytes(b)) in (_capi.MG_OK, _capi.MG_ERR_ARG)
    assert code(b"GIF89a") == _capi.MG_ERR_ARG and b"neither" in lib.mg_last_error()


# ---- the encoder (main.rs:672 save of a .jpg path) ------------------------------------
def _grey_wave(rng, w, h):
    y, x = np.mgrid[0:h, 0:w]
    g = np.clip(128 + 100 * np.sin(x / 17.0) * np.cos(y / 11.0) + rng.integers(-2, 3, (h, w)), 0, 255)
    return np.repeat(g.astype(np.uint8)[..., None], 3, axis=2)


def _segments(data):
    """(marker, body) of every segment before the scan data, and the scan's bytes."""
    pos, out = 2, []
    while True:
        m = data[pos + 1]
        n = struct.unpack(">H", data[pos + 2:pos + 4])[0]
        out.append((m, data[pos + 4:pos + 2 + n]))
        pos += 2 + n
        if m == 0xDA:
            return out, data[pos:]


@pytest.mark.parametrize("size", [(1, 1), (7, 5), (17, 16), (64, 48), (250, 3), (333, 211)])
def test_encode_round_trips_through_the_decoder(capi, size):
    """Grey images (so the 4:2:0 chroma loses nothing): at quality 100 (every
    quantiser 1) the forward and inverse DCT and the rounding leave at most one
    level; lower qualities stay within their quantisation."""
    rng = np.random.default_rng(size[0] + 31 * size[1])
    img = _grey_wave(rng, *size)
    for q, worst, psnr_min in ((100, 1, 55.0), (95, 6, 42.0), (75, 10, 38.0), (50, 14, 35.0)):
        data = capi.jpeg_encode(img, q)
        assert capi.image_info(data) == size
        got = capi.image_decode(data)
        err = got.astype(np.int32) - img.astype(np.int32)
        assert np.abs(err).max() <= worst, (q, np.abs(err).max())
        mse = float(np.mean(err.astype(np.float64) ** 2))
        assert mse == 0 or 10 * math.log10(255 ** 2 / mse) >= psnr_min, (q, mse)


def test_encode_colour_subsampled(capi):
    """Colour: chroma averaged over 2x2 boxes (4:2:0), so a smooth colour image
    comes back close and solid colours almost exactly."""
    rng = np.random.default_rng(8)
    y, x = np.mgrid[0:90, 0:120]
    img = np.stack([120 + 80 * np.sin(x / 23.0), 128 + 90 * np.cos(y / 19.0), 60 + x // 3], -1)
    img = np.clip(img + rng.integers(-2, 3, img.shape), 0, 255).astype(np.uint8)
    got = capi.image_decode(capi.jpeg_encode(img, 95))
    err = got.astype(np.float64) - img.astype(np.float64)
    assert 10 * math.log10(255 ** 2 / np.mean(err ** 2)) >= 36.0
    for rgb in ((255, 0, 0), (0, 255, 0), (0, 0, 255), (12, 200, 77)):
        solid = np.zeros((24, 40, 3), np.uint8) + np.array(rgb, np.uint8)
        got = capi.image_decode(capi.jpeg_encode(solid, 90))
        assert np.abs(got.astype(np.int16) - solid.astype(np.int16)).max() <= 3, rgb


def test_encode_layout(capi):
    """Baseline JFIF: the Annex K tables scaled by quality (the IJG rule), 4:2:0
    sampling, one restart interval per MCU row (RSTn in order between rows),
    the same bytes on one thread as on many."""
    rng = np.random.default_rng(4)
    img = _grey_wave(rng, 100, 70)
    luma = [16, 11, 10, 16, 24, 40, 51, 61, 12, 12, 14, 19, 26, 58, 60, 55, 14, 13, 16, 24, 40, 57, 69, 56, 14, 17,
            22, 29, 51, 87, 80, 62, 18, 22, 37, 56, 68, 109, 103, 77, 24, 35, 55, 64, 81, 104, 113, 92, 49, 64, 78,
            87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99]
    for q in (1, 50, 75, 100):
        data = capi.jpeg_encode(img, q)
        segs, scan = _segments(data)
        kinds = [m for m, _ in segs]
        assert kinds == [0xE0, 0xDB, 0xC0, 0xC4, 0xDD, 0xDA]
        dqt = dict(segs)[0xDB]
        zz_luma = np.frombuffer(dqt[1:65], np.uint8).astype(int)
        nat = np.zeros(64, int)
        nat[ZIGZAG] = zz_luma
        scale = 5000 // q if q < 50 else 200 - 2 * q
        assert list(nat) == [min(255, max(1, (v * scale + 50) // 100)) for v in luma], q
        sof = dict(segs)[0xC0]
        assert sof[5] == 3 and sof[7] == 0x22 and sof[10] == 0x11 and sof[13] == 0x11
        assert struct.unpack(">H", dict(segs)[0xDD])[0] == -(-100 // 16)  # MCUs per row
        rst = [scan[i + 1] for i in range(len(scan) - 1) if scan[i] == 0xFF and 0xD0 <= scan[i + 1] <= 0xD7]
        assert rst == [0xD0 + (i & 7) for i in range(-(-70 // 16) - 1)]
    assert capi.jpeg_encode(img, 80, threads=1) == capi.jpeg_encode(img, 80, threads=7)


def test_encode_arguments(capi):
    from mosaic_gpu import _capi

    lib = _capi.load()
    img = np.zeros((8, 8, 3), np.uint8)
    out = np.zeros(1 << 16, np.uint8)
    n = np.ctypeslib.ctypes.c_size_t()
    u8 = np.ctypeslib.ctypes.c_uint8

    def enc(w, h, stride, q, cap):
        return lib.mg_jpeg_encode(_capi.ptr(img, u8), w, h, stride, q, 1, _capi.ptr(out, u8), cap,
                                  np.ctypeslib.ctypes.byref(n))

    assert enc(8, 8, 24, 75, out.size) == _capi.MG_OK and n.value > 0
    for args in ((8, 8, 24, 0, out.size), (8, 8, 24, 101, out.size), (0, 8, 24, 75, out.size), (8, 8, 23, 75, out.size),
                 (70000, 1, 210000, 75, out.size)):
        assert enc(*args) == _capi.MG_ERR_ARG, args
    assert enc(8, 8, 24, 75, 10) == _capi.MG_ERR_ARG and n.value == lib.mg_jpeg_encode_bound(8, 8)


def test_batch_decodes_png_and_jpeg(capi):
    rng = np.random.default_rng(11)
    imgs = [_image(rng, 33, 21, "smooth"), _image(rng, 16, 16, "noise")]
    files = [encode_jpeg(imgs[0], (2, 2), 2)[0], capi.png_encode(imgs[1], 1), b"not an image"]
    got, status = capi.image_decode_batch(files, threads=2)
    assert status[:2] == [capi.MG_OK, capi.MG_OK] and status[2] == capi.MG_ERR_ARG
    assert np.array_equal(got[1], imgs[1])
    assert np.array_equal(got[0], capi.image_decode(files[0]))


def test_fuzz_under_sanitizers(tmp_path, capi):
    """Mutated files (tests/cpp/jpeg_fuzz.cpp) against the decoder built with
    AddressSanitizer and UndefinedBehaviorSanitizer, seeded with every sampling,
    restart and scan layout the encoder writes."""
    import shutil
    import subprocess
    from pathlib import Path

    repo = Path(__file__).resolve().parents[1]
    if not shutil.which("g++"):
        pytest.skip("no g++")
    exe = tmp_path / "jpeg_fuzz"
    csrc = repo / "mosaic-art-rust_gb300" / "csrc"
    cmd = ["g++", "-O1", "-g", "-std=c++17", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
           f"-I{repo / 'include'}", "-pthread", str(repo / "tests" / "cpp" / "jpeg_fuzz.cpp"),
           str(csrc / "io_jpeg.cpp"), str(csrc / "io_png.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr:
        pytest.skip("the compiler has no sanitizer runtime")
    assert r.returncode == 0, r.stderr
    rng = np.random.default_rng(4)
    seeds = []
    for i, (sampling, quant, restart, interleaved) in enumerate(CASES):
        img = _image(rng, 23 + 5 * i, 17 + 3 * i, "smooth" if i % 2 else "noise")
        p = tmp_path / f"s{i}.jpg"
        p.write_bytes(encode_jpeg(img, sampling, quant, restart, interleaved)[0])
        seeds.append(str(p))
    p = tmp_path / "grey.jpg"
    p.write_bytes(encode_jpeg(_image(rng, 30, 20, "smooth")[..., 0], quant=2, restart=2, grey=True)[0])
    seeds.append(str(p))
    for i, (sampling, quant, restart, grey, script) in enumerate(PROG_CASES):
        img = _image(rng, 21 + 4 * i, 13 + 5 * i, "noise" if i % 2 else "smooth")
        p = tmp_path / f"p{i}.jpg"
        p.write_bytes(encode_jpeg_progressive(img[..., 0] if grey else img, sampling, quant, restart, grey, script)[0])
        seeds.append(str(p))
    env = dict(__import__("os").environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0")
    r = subprocess.run([str(exe), "1500", *seeds], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stdout + r.stderr[-3000:]
    assert "decoded" in r.stdout
    print(r.stdout)
