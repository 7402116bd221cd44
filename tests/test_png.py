"""PNG files at the two ends of the path (csrc/io_png.cpp; image::open + to_rgb8
of main.rs:492/548 and DynamicImage::save of main.rs:672), on the CPU.

The checker is independent of the library: PNG files are written here with
Python's zlib (every compression level and strategy, so stored, fixed- and
dynamic-Huffman blocks and long matches all occur) from numpy-filtered rows
(every filter type), for every colour type, bit depth and both interlace
methods, and the expected RGB8 follows the conversions to_rgb8 applies (grey
replicated, alpha dropped, palette looked up, low-bit grey scaled, 16-bit
rounded).  Files the library writes are inflated here with zlib and checked
row by row against the image they encode (check_rows).  Defective files must
fail with MG_ERR_ARG, never crash.
"""
import os
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

SIG = b"\x89PNG\r\n\x1a\n"
ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


@pytest.fixture(scope="module")
def capi(built):
    from mosaic_gpu import _capi

    return _capi


def chunk(kind: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


def paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def filter_rows(rows: np.ndarray, bpp: int, rng) -> bytes:
    """rows: (h, rowbytes) uint8; each row gets a random filter type."""
    out = bytearray()
    prev = np.zeros(rows.shape[1], np.int32)
    for r in rows.astype(np.int32):
        f = int(rng.integers(0, 5))
        a = np.concatenate([np.zeros(bpp, np.int32), r[:-bpp]]) if len(r) > bpp else np.zeros_like(r)
        c = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]]) if len(r) > bpp else np.zeros_like(r)
        if f == 0:
            res = r
        elif f == 1:
            res = r - a
        elif f == 2:
            res = r - prev
        elif f == 3:
            res = r - ((a + prev) >> 1)
        else:
            res = r - np.array([paeth(int(x), int(y), int(z)) for x, y, z in zip(a, prev, c)], np.int32)
        out.append(f)
        out += (res & 0xFF).astype(np.uint8).tobytes()
        prev = r
    return bytes(out)


def pack_samples(samples: np.ndarray, depth: int) -> np.ndarray:
    """(h, n) samples of `depth` bits -> (h, rowbytes) bytes, MSB first / big-endian."""
    h, n = samples.shape
    if depth == 8:
        return samples.astype(np.uint8)
    if depth == 16:
        s = samples.astype(np.uint16)
        return np.stack([(s >> 8).astype(np.uint8), (s & 0xFF).astype(np.uint8)], -1).reshape(h, 2 * n)
    per = 8 // depth
    pad = (-n) % per
    s = np.concatenate([samples, np.zeros((h, pad), samples.dtype)], 1).reshape(h, -1, per).astype(np.uint32)
    shifts = np.array([8 - depth * (i + 1) for i in range(per)], np.uint32)
    return (s << shifts).sum(-1).astype(np.uint8)


def write_png(samples: np.ndarray, color: int, depth: int, rng, interlace=0, level=6, strategy=zlib.Z_DEFAULT_STRATEGY,
              plte: bytes | None = None, extra=(), idat_split=1) -> bytes:
    """samples: (h, w, channels) integers of `depth` bits."""
    h, w, ch = samples.shape
    bits_pp = ch * depth
    bpp = max(1, bits_pp // 8)
    raw = bytearray()
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    for x0, y0, dx, dy in passes:
        sub = samples[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        rows = pack_samples(sub.reshape(sub.shape[0], -1), depth)
        raw += filter_rows(rows, bpp, rng)
    comp = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
    z = comp.compress(bytes(raw)) + comp.flush()
    out = SIG + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, color, 0, 0, interlace))
    for kind, data in extra:
        out += chunk(kind, data)
    if plte is not None:
        out += chunk(b"PLTE", plte)
    cuts = sorted(set([0, len(z)] + [int(v) for v in rng.integers(0, len(z) + 1, idat_split - 1)]))
    for a, b in zip(cuts[:-1], cuts[1:]):
        out += chunk(b"IDAT", z[a:b])
    if len(cuts) == 1:
        out += chunk(b"IDAT", z)
    return out + chunk(b"IEND", b"")


def expected_rgb(samples: np.ndarray, color: int, depth: int, plte: bytes | None = None) -> np.ndarray:
    s = samples.astype(np.uint32)
    if depth == 16:
        s = (s + 128) // 257
    elif depth < 8 and color == 0:
        s = s * (255 // ((1 << depth) - 1))
    if color == 3:
        pal = np.frombuffer(plte, np.uint8).reshape(-1, 3)
        full = np.zeros((256, 3), np.uint8)
        full[: len(pal)] = pal
        return full[s[..., 0]]
    if color in (0, 4):
        return np.repeat(s[..., :1], 3, axis=2).astype(np.uint8)
    return s[..., :3].astype(np.uint8)


def parse(data: bytes):
    """(IHDR fields, zlib-inflated image data) of a PNG, CRCs checked."""
    assert data[:8] == SIG
    pos, z, ihdr = 8, b"", None
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(kind + body) & 0xFFFFFFFF
        if kind == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            z += body
        pos += 12 + n
    return ihdr, zlib.decompress(z)


def check_rows(data: bytes, rgb: np.ndarray) -> None:
    """`rgb` is the R, G, B content of the 8-bit, non-interlaced RGB or RGBA PNG
    `data`: refiltering rgb with each row's own filter type reproduces the
    file's filtered bytes of those channels.  Unfiltering is the unique inverse
    of that, so this pins every pixel, and it vectorises over whole images."""
    (w, h, depth, color, _, _, inter), raw = parse(data)
    assert depth == 8 and color in (2, 6) and inter == 0 and rgb.shape == (h, w, 3)
    ch = CHANNELS[color]
    raw = np.frombuffer(raw, np.uint8).reshape(h, 1 + w * ch)
    f = raw[:, 0].astype(np.int32)[:, None, None]
    res = raw[:, 1:].reshape(h, w, ch)[..., :3].astype(np.int32)
    x = rgb.astype(np.int32)
    a = np.zeros_like(x)
    a[:, 1:] = x[:, :-1]
    b = np.zeros_like(x)
    b[1:] = x[:-1]
    c = np.zeros_like(x)
    c[1:, 1:] = x[:-1, :-1]
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    pae = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
    pred = np.select([f == 0, f == 1, f == 2, f == 3, f == 4], [0 * x, a, b, (a + b) >> 1, pae])
    assert np.all(f <= 4)
    assert np.array_equal((x - pred) & 0xFF, res)


CASES = [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4), (3, 8), (4, 8), (4, 16),
         (6, 8), (6, 16)]


@pytest.mark.parametrize("interlace", [0, 1])
@pytest.mark.parametrize("color,depth", CASES)
def test_decode_every_format(capi, color, depth, interlace):
    rng = np.random.default_rng(color * 100 + depth * 2 + interlace)
    for w, h in [(1, 1), (3, 2), (9, 5), (17, 13), (33, 8)]:
        ch = CHANNELS[color]
        top = (1 << depth) - 1
        plte = None
        if color == 3:
            npal = int(rng.integers(1, min(256, top + 1) + 1))
            plte = rng.integers(0, 256, 3 * npal, dtype=np.uint8).tobytes()
            top = min(top, 255)  # indices past the palette read as black
        samples = rng.integers(0, top + 1, (h, w, ch)).astype(np.uint32)
        data = write_png(samples, color, depth, rng, interlace=interlace, plte=plte)
        assert capi.png_info(data) == (w, h)
        got = capi.png_decode(data)
        assert np.array_equal(got, expected_rgb(samples, color, depth, plte)), (w, h)


@pytest.mark.parametrize("level,strategy", [(0, zlib.Z_DEFAULT_STRATEGY), (1, zlib.Z_DEFAULT_STRATEGY),
                                            (6, zlib.Z_DEFAULT_STRATEGY), (9, zlib.Z_DEFAULT_STRATEGY),
                                            (9, zlib.Z_FILTERED), (6, zlib.Z_HUFFMAN_ONLY), (6, zlib.Z_RLE),
                                            (6, zlib.Z_FIXED)])
def test_decode_every_deflate_form(capi, level, strategy):
    """Smooth and noisy content (long matches, overlapping copies, literals),
    split over several IDAT chunks with ancillary chunks in front."""
    rng = np.random.default_rng(level * 10 + strategy)
    y, x = np.mgrid[0:150, 0:211]
    smooth = np.stack([(x // 7) % 256, (y // 3) % 256, np.full_like(x, 77)], -1)
    noisy = rng.integers(0, 256, (150, 211, 3))
    img = np.where(rng.random((150, 211, 1)) < 0.2, noisy, smooth).astype(np.uint32)
    data = write_png(img, 2, 8, rng, level=level, strategy=strategy, idat_split=5,
                     extra=[(b"gAMA", struct.pack(">I", 45455)), (b"tEXt", b"Comment\x00test")])
    assert np.array_equal(capi.png_decode(data), img.astype(np.uint8))


def test_decode_into_strided_buffer(capi):
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, (20, 30, 3)).astype(np.uint32)
    data = write_png(img, 2, 8, rng)
    big = np.full((20, 40, 3), 7, np.uint8)
    view = big[:, 5:35]
    out = np.ascontiguousarray(view)  # contiguous rows of 90 bytes
    capi.png_decode(data, out)
    assert np.array_equal(out, img.astype(np.uint8))
    lib = capi.load()
    rc = lib.mg_png_decode(data, len(data), capi.ptr(big, np.ctypeslib.ctypes.c_uint8), big.strides[0])
    assert rc == 0 and np.array_equal(big[:, :30], img.astype(np.uint8)) and np.all(big[:, 30:] == 7)


def _corrupt_cases(rng):
    img = rng.integers(0, 256, (12, 9, 3)).astype(np.uint32)
    good = write_png(img, 2, 8, rng)
    cases = {"empty": b"", "signature": b"\x00" + good[1:], "truncated_header": good[:20]}
    b = bytearray(good)
    b[20] ^= 1  # IHDR data, CRC now wrong
    cases["ihdr_crc"] = bytes(b)
    idat = good.index(b"IDAT")
    b = bytearray(good)
    b[idat + 10] ^= 0x40  # compressed data, CRC now wrong
    cases["idat_crc"] = bytes(b)
    cases["cut_in_idat"] = good[: idat + 20]
    # valid CRCs, broken contents
    def rebuild(z, w=9, h=12, depth=8, color=2):
        return SIG + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, color, 0, 0, 0)) + chunk(b"IDAT", z) + \
            chunk(b"IEND", b"")
    raw = bytes(12 * (1 + 27))
    z = zlib.compress(raw)
    cases["adler"] = rebuild(z[:-1] + bytes([z[-1] ^ 1]))
    cases["short_data"] = rebuild(zlib.compress(raw[:-5]))
    cases["long_data"] = rebuild(zlib.compress(raw + bytes(40)))
    cases["bad_filter"] = rebuild(zlib.compress(b"\x07" + raw[1:]))
    cases["bad_depth"] = rebuild(z, depth=3)
    cases["bad_color"] = rebuild(z, color=5)
    cases["zero_width"] = rebuild(z, w=0)
    cases["palette_without_plte"] = rebuild(zlib.compress(bytes(12 * 10)), color=3)
    cases["zlib_header"] = rebuild(b"\x00\x00" + z[2:])
    cases["bad_block_type"] = rebuild(b"\x78\x01\x07" + z[3:])
    cases["unknown_critical"] = good[:33] + chunk(b"ABCD", b"x") + good[33:]
    return cases


def test_defective_files_fail_cleanly(capi):
    rng = np.random.default_rng(4)
    for name, data in _corrupt_cases(rng).items():
        out = np.zeros((64, 64, 3), np.uint8)
        lib = capi.load()
        rc = lib.mg_png_decode(data, len(data), capi.ptr(out, np.ctypeslib.ctypes.c_uint8), 64 * 3)
        assert rc == capi.MG_ERR_ARG, name
        assert lib.mg_last_error().decode(), name


def test_truncation_at_every_byte_never_crashes(capi):
    rng = np.random.default_rng(5)
    img = rng.integers(0, 256, (6, 7, 3)).astype(np.uint32)
    data = write_png(img, 2, 8, rng, level=9)
    lib = capi.load()
    out = np.zeros((6, 7, 3), np.uint8)
    for cut in range(len(data) - 12):  # IEND (the last 12 bytes) is optional
        rc = lib.mg_png_decode(data[:cut], cut, capi.ptr(out, np.ctypeslib.ctypes.c_uint8), 21)
        assert rc == capi.MG_ERR_ARG, cut


def test_random_bit_flips_never_crash(capi):
    rng = np.random.default_rng(6)
    img = rng.integers(0, 256, (16, 16, 3)).astype(np.uint32)
    good = write_png(img, 2, 8, rng)
    idat = good.index(b"IDAT") + 4
    n = struct.unpack(">I", good[idat - 8:idat - 4])[0]
    lib = capi.load()
    out = np.zeros((16, 16, 3), np.uint8)
    for t in range(300):
        body = bytearray(good[idat:idat + n])
        for _ in range(int(rng.integers(1, 4))):
            body[int(rng.integers(0, n))] ^= 1 << int(rng.integers(0, 8))
        data = good[:idat - 8] + chunk(b"IDAT", bytes(body)) + good[idat + n + 4:]
        rc = lib.mg_png_decode(data, len(data), capi.ptr(out, np.ctypeslib.ctypes.c_uint8), 48)
        assert rc in (capi.MG_OK, capi.MG_ERR_ARG)


@pytest.mark.parametrize("level", [0, 1])
def test_encode_reads_back(capi, level):
    rng = np.random.default_rng(7 + level)
    for w, h in [(1, 1), (2, 3), (31, 17), (200, 3)]:
        img = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
        data = capi.png_encode(img, level)
        check_rows(data, img)
        assert len(data) <= capi.load().mg_png_encode_bound(w, h)


def test_encode_large_compresses_and_round_trips(capi):
    """Several 64 KB blocks and IDAT chunks, thread counts 1 and 8 give the same file."""
    y, x = np.mgrid[0:1200, 0:1700]
    img = np.stack([(x // 3) % 256, (y // 2) % 256, ((x + y) // 5) % 256], -1).astype(np.uint8)
    img[::37] = 255
    a = capi.png_encode(img, 1, threads=1)
    b = capi.png_encode(img, 1, threads=8)
    assert a == b
    s = capi.png_encode(img, 0)
    assert len(a) < 0.5 * len(s) and len(s) >= img.nbytes
    check_rows(a, img)  # zlib inflates it (Adler-32 included) to the image's rows
    check_rows(s, img)
    assert np.array_equal(capi.png_decode(a), img) and np.array_equal(capi.png_decode(s), img)


def test_encode_arguments(capi):
    lib = capi.load()
    img = np.zeros((4, 4, 3), np.uint8)
    n = np.ctypeslib.ctypes.c_size_t()
    small = np.zeros(10, np.uint8)
    u8 = np.ctypeslib.ctypes.c_uint8
    rc = lib.mg_png_encode(capi.ptr(img, u8), 4, 4, 12, 1, 1, capi.ptr(small, u8), 10, np.ctypeslib.ctypes.byref(n))
    assert rc == capi.MG_ERR_ARG and n.value == lib.mg_png_encode_bound(4, 4)
    assert lib.mg_png_encode_bound(0, 4) == 0
    with pytest.raises(capi.MosaicError):
        capi.png_encode(img, level=2)


def test_batch_decode(capi):
    rng = np.random.default_rng(8)
    imgs, files = [], []
    for i in range(40):
        w, h = int(rng.integers(1, 60)), int(rng.integers(1, 60))
        img = rng.integers(0, 256, (h, w, 3)).astype(np.uint32)
        imgs.append(img.astype(np.uint8))
        files.append(write_png(img, 2, 8, rng, interlace=i % 2))
    files[13] = files[13][:-40]  # cut inside the image data
    got, codes = capi.png_decode_batch(files, threads=6)
    for i, (img, g, c) in enumerate(zip(imgs, got, codes)):
        if i == 13:
            assert c == capi.MG_ERR_ARG and g is None
        else:
            assert c == capi.MG_OK and np.array_equal(g, img)
    assert "file 13" in capi.load().mg_last_error().decode()
    again, codes0 = capi.png_decode_batch(files, threads=0)  # one thread per hardware thread
    assert codes0 == codes and all(g is None or np.array_equal(g, a) for g, a in zip(again, got) if a is not None)


@pytest.mark.parametrize("name", ["examples/mosaic.png", "docs/public/hero-image.png"])
def test_reference_example_images(capi, name):
    """The PNG files shipped with mosaic-art-rust (an RGBA mosaic the tool made,
    3840x2160, and an RGB image in 32 IDAT chunks), when MOSAIC_ART_RUST_SRC
    names a copy of its source tree: decoded, then checked row by row against
    the files' own filtered data as zlib inflates it."""
    root = os.environ.get("MOSAIC_ART_RUST_SRC")
    if not root or not (Path(root) / name).exists():
        pytest.skip("set MOSAIC_ART_RUST_SRC to a mosaic-art-rust source tree to check its example images")
    path = Path(root) / name
    data = path.read_bytes()
    rgb = capi.png_decode(data)
    check_rows(data, rgb)


def test_fuzz_under_sanitizers(tmp_path, capi):
    """Mutated files (tests/cpp/png_fuzz.cpp) against the decoder built with
    AddressSanitizer and UndefinedBehaviorSanitizer: small seeds of every
    format, large ones that take the two-thread pipeline, and one written by
    the library, whose part index takes the all-threads inflate."""
    import shutil
    import subprocess

    repo = Path(__file__).resolve().parents[1]
    if not shutil.which("g++"):
        pytest.skip("no g++")
    exe = tmp_path / "png_fuzz"
    cmd = ["g++", "-O1", "-g", "-std=c++17", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
           f"-I{repo / 'include'}", "-pthread", str(repo / "tests" / "cpp" / "png_fuzz.cpp"),
           str(repo / "mosaic-art-rust_gb300" / "csrc" / "io_png.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr:
        pytest.skip("the compiler has no sanitizer runtime")
    assert r.returncode == 0, r.stderr
    rng = np.random.default_rng(1)
    small, large = [], []
    for color, depth in CASES:
        for inter in (0, 1):
            top = (1 << depth) - 1
            plte = rng.integers(0, 256, 3 * min(256, top + 1), dtype=np.uint8).tobytes() if color == 3 else None
            s = rng.integers(0, top + 1, (13, 11, CHANNELS[color])).astype(np.uint32)
            p = tmp_path / f"s{color}_{depth}_{inter}.png"
            p.write_bytes(write_png(s, color, depth, rng, interlace=inter, plte=plte, level=int(rng.integers(0, 10))))
            small.append(str(p))
    y, x = np.mgrid[0:600, 0:800]
    img = np.stack([(x // 3) % 256, (y // 2) % 256, ((x + y) // 5) % 256], -1)
    img = np.where(rng.random((600, 800, 1)) < 0.3, rng.integers(0, 256, (600, 800, 3)), img).astype(np.uint32)
    for i, (kw, im, color) in enumerate([(dict(level=6, idat_split=3), img, 2),
                                         (dict(level=1, strategy=zlib.Z_RLE),
                                          np.concatenate([img, img[..., :1]], -1), 6)]):
        p = tmp_path / f"l{i}.png"
        p.write_bytes(write_png(im, color, 8, rng, **kw))
        large.append(str(p))
    p = tmp_path / "indexed.png"
    p.write_bytes(capi.png_encode(img.astype(np.uint8), 1))
    large.append(str(p))
    env = dict(__import__("os").environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0")
    for iters, seeds in ((2000, small), (60, large)):
        r = subprocess.run([str(exe), str(iters), *seeds], capture_output=True, text=True, timeout=600, env=env)
        assert r.returncode == 0, r.stdout + r.stderr[-3000:]
        assert "decoded" in r.stdout


def test_literal_pairs_at_every_length(capi):
    """Literal-only streams of short codes (two literals per table lookup),
    ending on every parity of the output size, including one byte left when a
    pair would be next."""
    rng = np.random.default_rng(9)
    for w in range(1, 12):
        for h in (1, 2, 3, 7):
            img = rng.integers(0, 3, (h, w, 3)).astype(np.uint32)  # few distinct bytes: 1-3 bit codes
            for strategy in (zlib.Z_HUFFMAN_ONLY, zlib.Z_DEFAULT_STRATEGY):
                data = write_png(img, 2, 8, rng, level=6, strategy=strategy)
                assert np.array_equal(capi.png_decode(data), img.astype(np.uint8)), (w, h, strategy)


def _with_chunk_body(data: bytes, kind: bytes, fn) -> bytes:
    """data with chunk `kind`'s body replaced by fn(body) (CRC recomputed)."""
    pos, out = 8, bytearray(data[:8])
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        k, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        out += chunk(k, fn(body)) if k == kind else data[pos:pos + 12 + n]
        pos += 12 + n
    return bytes(out)


def test_indexed_parts_decode_in_parallel_and_fall_back(capi):
    """The library's files carry an index of independent deflate parts (mgIX)
    that large ones inflate from on all threads; a damaged or misleading index
    (offsets moved inside a part, a wrong count) leaves the serial inflate to
    give the same image."""
    y, x = np.mgrid[0:700, 0:900]
    img = np.stack([(x * 3) % 256, (y * 5) % 256, (x ^ y) % 256], -1).astype(np.uint8)
    for level in (0, 1):
        data = capi.png_encode(img, level)
        assert b"mgIX" in data
        assert np.array_equal(capi.png_decode(data), img)

        def shift(body, by=7):
            b = bytearray(body)
            off = struct.unpack(">Q", bytes(b[4 + 16:4 + 24]))[0]  # part 1's stream offset
            b[4 + 16:4 + 24] = struct.pack(">Q", off + by)
            return bytes(b)

        for fn in (shift, lambda b: struct.pack(">I", 3) + b[4:], lambda b: b[:-16], lambda b: b"\x00" * len(b)):
            bent = _with_chunk_body(data, b"mgIX", fn)
            assert np.array_equal(capi.png_decode(bent), img)
        check_rows(data, img)


def _indexed_file(segments: list[bytes], w: int, h: int, parts: list[bytes]) -> bytes:
    """An RGB8 PNG whose zlib stream is the given raw-deflate parts (one per
    segment of the filtered data) with an mgIX index of where each starts."""
    raw = b"".join(segments)
    z = b"\x78\xda" + b"".join(parts) + struct.pack(">I", zlib.adler32(raw) & 0xFFFFFFFF)
    idx, zo, ro = struct.pack(">I", len(parts)), 2, 0
    for seg, part in zip(segments, parts):
        idx += struct.pack(">QQ", zo, ro)
        zo, ro = zo + len(part), ro + len(seg)
    return (SIG + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)) + chunk(b"mgIX", idx) +
            chunk(b"IDAT", z) + chunk(b"IEND", b""))


def _runs_before_cuts(w: int, h: int, cuts: list[int], rng) -> bytes:
    """Filtered RGB8 data (filter type None) whose bytes before each cut repeat a
    13-byte pattern, so a deflate part ending at the cut ends in a long match at
    distance 13."""
    raw = bytearray(rng.integers(0, 256, h * (3 * w + 1)).astype(np.uint8).tobytes())
    pat = bytes(rng.integers(0, 256, 13).astype(np.uint8))
    for c in cuts:
        raw[c - 700:c] = (pat * 60)[:700]
    raw[::3 * w + 1] = bytes(h)  # filter bytes
    return bytes(raw)


def _pixels(raw: bytes, w: int, h: int) -> np.ndarray:
    return np.frombuffer(raw, np.uint8).reshape(h, 3 * w + 1)[:, 1:].reshape(h, w, 3)


def test_indexed_parts_ending_in_long_matches(capi):
    """Each part of an indexed file (here compressed by zlib with a full flush
    between parts, so parts share no back-references) ends in a long match at a
    distance of at least 8.  The parts inflate on separate threads into
    adjacent ranges of one buffer, so a part must not write past its own end:
    the decoded image equals the serial decode of the same stream, every time."""
    w, h = 700, 520
    rng = np.random.default_rng(12)
    total = h * (3 * w + 1)
    cuts = list(range(65533, total, 65533))
    raw = _runs_before_cuts(w, h, cuts, rng)
    bounds = [0] + cuts + [total]
    segments = [raw[a:b] for a, b in zip(bounds[:-1], bounds[1:])]
    c = zlib.compressobj(9, zlib.DEFLATED, -15)
    parts = [c.compress(s) + c.flush(zlib.Z_FULL_FLUSH) for s in segments[:-1]]
    parts.append(c.compress(segments[-1]) + c.flush(zlib.Z_FINISH))
    want = _pixels(raw, w, h)
    data = _indexed_file(segments, w, h, parts)
    serial = _with_chunk_body(data, b"mgIX", lambda b: b"\x00" * len(b))
    assert np.array_equal(capi.png_decode(serial), want)
    for _ in range(8):
        assert np.array_equal(capi.png_decode(data), want)


def _stored(seg: bytes, final: bool) -> bytes:
    """seg as raw-deflate stored blocks (<= 65535 bytes each); the last block
    carries BFINAL when `final`."""
    out = bytearray()
    for i in range(0, max(len(seg), 1), 65535):
        piece = seg[i:i + 65535]
        last = final and i + 65535 >= len(seg)
        out += bytes([1 if last else 0]) + struct.pack("<HH", len(piece), len(piece) ^ 0xFFFF) + piece
    return bytes(out)


def test_indexed_parts_must_agree_with_the_serial_stream(capi):
    """An index cannot make the decoder accept a stream that the serial inflate
    rejects, nor decode one differently: a file whose inner part carries BFINAL
    (the serial inflate stops there, short of the image) fails; with a part
    boundary moved, the image is the same (through the serial inflate when a
    part no longer ends exactly where the index says)."""
    w, h = 700, 520
    rng = np.random.default_rng(13)
    total = h * (3 * w + 1)
    raw = bytearray(rng.integers(0, 256, total).astype(np.uint8).tobytes())
    raw[::3 * w + 1] = bytes(h)
    raw = bytes(raw)
    bounds = [0, 300000, 700000, total]
    segments = [raw[a:b] for a, b in zip(bounds[:-1], bounds[1:])]
    good = [_stored(s, i == len(segments) - 1) for i, s in enumerate(segments)]
    assert np.array_equal(capi.png_decode(_indexed_file(segments, w, h, good)), _pixels(raw, w, h))
    early_final = [_stored(s, i >= 1) for i, s in enumerate(segments)]
    bad = _indexed_file(segments, w, h, early_final)
    with pytest.raises(RuntimeError):
        capi.png_decode(bad)

    def move_part1(by):
        return lambda b: b[:4 + 16] + struct.pack(">Q", struct.unpack(">Q", b[4 + 16:4 + 24])[0] + by) + b[4 + 24:]

    # part 0 followed by an empty stored block: moved back over it, part 1
    # starts with that block (the same stream either way); moved forward, part 0
    # runs into part 1's data and the serial inflate decides
    padded = [good[0] + b"\x00\x00\x00\xff\xff"] + good[1:]
    data = _indexed_file(segments, w, h, padded)
    for by in (-5, 5, 1):
        assert np.array_equal(capi.png_decode(_with_chunk_body(data, b"mgIX", move_part1(by))), _pixels(raw, w, h))
