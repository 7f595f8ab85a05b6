"""Image ingest (row f2): the library's PNG decoder returns the pixels of
PNG files written here by a small independent encoder (all colour types and
bit depths, all five scanline filters, stored and compressed zlib streams,
Adam7 interlacing, tRNS transparency), with the reference's libpng transforms
(16-bit -> high byte, palette -> RGB, gray < 8 bit scaled to 8, tRNS ->
alpha); image_to_grid applies main.cpp:91-99's gray conversion.  Host code:
no GPU.  resize_image (GPU) is checked against main.cpp:13-27 in
test_resize_image_matches_port (gpu)."""
import binascii
import struct
import zlib

import numpy as np
import pytest

ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _chunk(t, data):
    return struct.pack(">I", len(data)) + t + data + struct.pack(">I", binascii.crc32(t + data) & 0xFFFFFFFF)


def _pack_rows(samples, depth):
    """samples: h x (w*channels) ints -> list of row byte strings."""
    rows = []
    for r in samples:
        if depth == 16:
            rows.append(b"".join(struct.pack(">H", int(v)) for v in r))
        elif depth == 8:
            rows.append(bytes(int(v) for v in r))
        else:
            per = 8 // depth
            out = bytearray((len(r) + per - 1) // per)
            for i, v in enumerate(r):
                out[i // per] |= int(v) << (8 - depth * (i % per + 1))
            rows.append(bytes(out))
    return rows


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def _filter(rows, bpp, rng):
    out, prev = bytearray(), None
    for r in rows:
        f = int(rng.integers(0, 5))
        enc = bytearray()
        for i, x in enumerate(r):
            a = r[i - bpp] if i >= bpp else 0
            b = prev[i] if prev is not None else 0
            c = prev[i - bpp] if (prev is not None and i >= bpp) else 0
            pred = [0, a, b, (a + b) // 2, _paeth(a, b, c)][f]
            enc.append((x - pred) & 255)
        out += bytes([f]) + enc
        prev = r
    return bytes(out)


def encode_png(samples, w, h, ctype, depth, rng, interlace=False, plte=None, trns=None, level=9):
    ch = CHANNELS[ctype]
    bpp = max(1, ch * depth // 8)
    samples = np.asarray(samples).reshape(h, w * ch)
    if not interlace:
        raw = _filter(_pack_rows(samples, depth), bpp, rng)
    else:
        raw = b""
        img = samples.reshape(h, w, ch)
        for x0, y0, dx, dy in ADAM7:
            sub = img[y0::dy, x0::dx]
            if sub.size == 0:
                continue
            raw += _filter(_pack_rows(sub.reshape(sub.shape[0], -1), depth), bpp, rng)
    png = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    if plte is not None:
        png += _chunk(b"PLTE", bytes(np.asarray(plte, dtype=np.uint8).ravel()))
    if trns is not None:
        png += _chunk(b"tRNS", bytes(trns))
    comp = zlib.compress(raw, level)
    half = len(comp) // 2  # two IDAT chunks
    png += _chunk(b"IDAT", comp[:half]) + _chunk(b"IDAT", comp[half:]) + _chunk(b"IEND", b"")
    return png


def expected_rgba(samples, w, h, ctype, depth, plte=None, trns=None):
    ch = CHANNELS[ctype]
    s = np.asarray(samples).reshape(h, w, ch).astype(np.int64)
    s8 = s >> 8 if depth == 16 else s
    out = np.zeros((h, w, 4), dtype=np.uint8)
    out[..., 3] = 255
    if ctype == 3:
        pal = np.asarray(plte, dtype=np.uint8)
        out[..., :3] = pal[s[..., 0]]
        if trns is not None:
            alpha = np.full(256, 255, np.uint8)
            alpha[:len(trns)] = list(trns)
            out[..., 3] = alpha[s[..., 0]]
    elif ctype in (0, 4):
        g = s8[..., 0] * 255 // ((1 << depth) - 1) if depth < 8 else s8[..., 0]
        out[..., 0] = out[..., 1] = out[..., 2] = g
        if ctype == 4:
            out[..., 3] = s8[..., 1]
        elif trns is not None:
            key = (trns[0] << 8) | trns[1]
            out[..., 3] = np.where(s[..., 0] == key, 0, 255)
    else:
        out[..., :3] = s8[..., :3]
        if ctype == 6:
            out[..., 3] = s8[..., 3]
        elif trns is not None:
            key = [(trns[2 * i] << 8) | trns[2 * i + 1] for i in range(3)]
            m = (s[..., 0] == key[0]) & (s[..., 1] == key[1]) & (s[..., 2] == key[2])
            out[..., 3] = np.where(m, 0, 255)
    return out


CASES = [  # (ctype, depth, w, h, interlace, level)
    (2, 8, 13, 7, False, 9), (6, 8, 9, 5, False, 0), (0, 1, 11, 3, False, 6), (0, 2, 11, 3, False, 6),
    (0, 4, 11, 3, False, 6), (0, 8, 10, 4, False, 6), (0, 16, 7, 6, False, 6), (4, 8, 6, 5, False, 1),
    (4, 16, 6, 5, False, 9), (2, 16, 5, 5, False, 9), (6, 16, 5, 4, False, 9), (3, 1, 10, 3, False, 9),
    (3, 2, 10, 3, False, 9), (3, 4, 10, 3, False, 9), (3, 8, 12, 6, False, 9), (2, 8, 17, 13, True, 9),
    (3, 4, 9, 11, True, 9), (0, 16, 1, 1, False, 9),
]


@pytest.mark.parametrize("ctype,depth,w,h,interlace,level", CASES)
def test_png_decoder(ctype, depth, w, h, interlace, level):
    from poisson_caustic_design_gb300 import image

    rng = np.random.default_rng(ctype * 100 + depth + w)
    ch = CHANNELS[ctype]
    top = (1 << depth) - 1
    samples = rng.integers(0, top + 1, size=(h, w * ch))
    plte = trns = None
    if ctype == 3:
        plte = rng.integers(0, 256, size=(1 << depth, 3))
        trns = list(rng.integers(0, 256, size=min(5, 1 << depth)))
    elif ctype == 0 and depth == 8:
        trns = [0, int(samples[0, 0])]
    elif ctype == 2 and depth == 8:
        trns = []
        for v in samples[1, :3]:
            trns += [0, int(v)]
    data = encode_png(samples, w, h, ctype, depth, rng, interlace, plte, trns, level)
    got = image.png_decode(data)
    assert np.array_equal(got, expected_rgba(samples, w, h, ctype, depth, plte, trns))


def test_image_to_grid_gray(tmp_path):
    from poisson_caustic_design_gb300 import image

    rng = np.random.default_rng(3)
    w, h = 23, 17
    rgb = rng.integers(0, 256, size=(h, w, 3))
    path = tmp_path / "t.png"
    path.write_bytes(encode_png(rgb.reshape(h, -1), w, h, 2, 8, rng))
    g = image.image_to_grid(str(path))
    r, gg, b = (rgb[..., i] / 255.0 for i in range(3))
    assert np.array_equal(g, (0.299 * r) + (0.587 * gg) + (0.114 * b))   # main.cpp:91-99


def test_png_errors(tmp_path):
    import poisson_caustic_design_gb300 as pcd
    from poisson_caustic_design_gb300 import image

    rng = np.random.default_rng(1)
    data = bytearray(encode_png(rng.integers(0, 256, (4, 12)), 4, 4, 2, 8, rng))
    with pytest.raises(pcd.PCDError):
        image.png_decode(bytes(data[:40]))                 # truncated
    bad = bytearray(data)
    bad[30] ^= 0xFF                                        # IHDR CRC
    with pytest.raises(pcd.PCDError):
        image.png_decode(bytes(bad))
    with pytest.raises(pcd.PCDError):
        image.png_decode(b"GIF89a" + bytes(40))
    with pytest.raises(pcd.PCDError):
        image.image_to_grid(str(tmp_path / "missing.png"))
