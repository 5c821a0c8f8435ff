"""PNG decoding for the loaders' image textures (gbpt_image_read_png).

PNG files are written here with Python's zlib (stored, fixed- and dynamic-Huffman DEFLATE blocks,
by compression level and data size) and every scanline filter (each row's filter applied by the
writer below); the decoder must return the exact RGBA8 pixels for each colour type and bit depth.
"""
import ctypes as C
import struct
import zlib

import numpy as np
import pytest


def _chunk(kind, body):
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body))


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def _filter_rows(raw, stride, bpp, rng):
    """Each row filtered with a random filter type (0-4), as an encoder may choose."""
    out, prev = [], np.zeros(stride, np.int32)
    for y in range(len(raw) // stride):
        cur = np.frombuffer(raw[y * stride:(y + 1) * stride], np.uint8).astype(np.int32)
        left = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]])
        upleft = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        f = int(rng.integers(0, 5))
        pred = [np.zeros_like(cur), left, prev, (left + prev) // 2, _paeth(left, prev, upleft)][f]
        out.append(bytes([f]) + ((cur - pred) % 256).astype(np.uint8).tobytes())
        prev = cur
    return b"".join(out)


def write_png(path, data, ctype, depth, level=6, palette=None, trns=None, seed=0):
    """data: raw samples (H, W*channels) of `depth` bits (already packed for depth < 8)."""
    h = data.shape[0]
    w = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    width = data.shape[1] * 8 // depth // w if depth < 8 else data.shape[1] // w
    if depth == 16:
        raw = data.astype(">u2").tobytes()
        stride = data.shape[1] * 2
    else:
        raw = data.astype(np.uint8).tobytes()
        stride = data.shape[1]
    bpp = max(1, w * depth // 8)
    body = _filter_rows(raw, stride, bpp, np.random.default_rng(seed))
    png = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", width, h, depth, ctype,
                                                               0, 0, 0))
    if palette is not None:
        png += _chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    if trns is not None:
        png += _chunk(b"tRNS", trns.astype(np.uint8).tobytes())
    comp = zlib.compress(body, level)
    # split the stream over two IDAT chunks
    png += _chunk(b"IDAT", comp[:len(comp) // 2]) + _chunk(b"IDAT", comp[len(comp) // 2:])
    png += _chunk(b"IEND", b"")
    path.write_bytes(png)
    return width


def read_png(native, path):
    w, h = C.c_uint32(), C.c_uint32()
    from merian_gb300 import _native as N
    N.check(native.gbpt_image_read_png(str(path).encode(), None, C.byref(w), C.byref(h)))
    out = np.zeros((h.value, w.value, 4), np.uint8)
    N.check(native.gbpt_image_read_png(str(path).encode(), out.ctypes.data, C.byref(w),
                                       C.byref(h)))
    return out


@pytest.mark.parametrize("level", [0, 1, 9])
@pytest.mark.parametrize("ctype,depth", [(0, 8), (2, 8), (4, 8), (6, 8), (6, 16), (2, 16), (0, 16)])
def test_png_direct_colour(native, tmp_path, ctype, depth, level):
    rng = np.random.default_rng(ctype * 100 + depth + level)
    ch = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
    H, W = 37, 53
    maxv = 255 if depth == 8 else 65535
    # smooth data (compresses with matches) plus noise (literals)
    base = (np.linspace(0, maxv, W * ch)[None, :] * np.ones((H, 1))).astype(np.int64)
    data = (base + rng.integers(0, maxv // 16, (H, W * ch))) % (maxv + 1)
    write_png(tmp_path / "a.png", data, ctype, depth, level, seed=level)
    got = read_png(native, tmp_path / "a.png")
    s = (data >> 8 if depth == 16 else data).astype(np.uint8).reshape(H, W, ch)
    exp = np.zeros((H, W, 4), np.uint8)
    exp[..., 3] = 255
    if ch in (1, 2):
        exp[..., :3] = s[..., :1]
        if ch == 2:
            exp[..., 3] = s[..., 1]
    else:
        exp[..., :ch] = s
    assert np.array_equal(got, exp)


@pytest.mark.parametrize("depth", [1, 2, 4, 8])
def test_png_palette(native, tmp_path, depth):
    rng = np.random.default_rng(depth)
    H, W = 19, 29
    n = 1 << depth
    pal = rng.integers(0, 256, (n, 3))
    trns = rng.integers(0, 256, max(1, n // 2))
    idx = rng.integers(0, n, (H, W))
    per = 8 // depth
    packed_w = (W + per - 1) // per
    packed = np.zeros((H, packed_w), np.int64)
    for x in range(W):
        packed[:, x // per] |= idx[:, x] << (8 - depth * (x % per + 1))
    write_png(tmp_path / "p.png", packed, 3, depth, 9, palette=pal, trns=trns)
    # the writer derives the width from the packed row; state it exactly
    raw = bytearray((tmp_path / "p.png").read_bytes())
    raw[16:20] = struct.pack(">I", W)
    raw[29:33] = struct.pack(">I", zlib.crc32(bytes(raw[12:29])))
    (tmp_path / "p.png").write_bytes(bytes(raw))
    got = read_png(native, tmp_path / "p.png")
    exp = np.zeros((H, W, 4), np.uint8)
    exp[..., :3] = pal[idx]
    alpha = np.full(n, 255)
    alpha[:len(trns)] = trns
    exp[..., 3] = alpha[idx]
    assert np.array_equal(got, exp)


def test_png_large_dynamic(native, tmp_path):
    """A 512 x 512 RGBA noise texture (long dynamic-Huffman stream with far matches)."""
    from merian_gb300 import scene as S
    tex = S.noise_texture(7, 512, 512)
    write_png(tmp_path / "n.png", tex.reshape(512, -1), 6, 8, 9)
    assert np.array_equal(read_png(native, tmp_path / "n.png"), tex)


def test_png_rejects_bad_files(native, tmp_path):
    from merian_gb300 import _native as N
    w, h = C.c_uint32(), C.c_uint32()
    (tmp_path / "x.png").write_bytes(b"not a png at all")
    assert native.gbpt_image_read_png(str(tmp_path / "x.png").encode(), None, C.byref(w),
                                      C.byref(h)) == N.GBPT_ERR_INVALID
    good = tmp_path / "g.png"
    write_png(good, np.zeros((4, 12)), 2, 8)
    data = good.read_bytes()
    (tmp_path / "t.png").write_bytes(data[:len(data) - 30])  # truncated IDAT / IEND
    assert native.gbpt_image_read_png(str(tmp_path / "t.png").encode(), None, C.byref(w),
                                      C.byref(h)) == N.GBPT_ERR_INVALID
    assert native.gbpt_image_read_png(str(tmp_path / "missing.png").encode(), None, C.byref(w),
                                      C.byref(h)) == N.GBPT_ERR_INVALID
