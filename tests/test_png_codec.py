"""The command-line driver's PNG codec (cli/png.cpp) against an independent
Python writer / reader built on the stdlib zlib (no GPU)."""
import os
import struct
import zlib

import numpy as np
import pytest

import png_util as P


@pytest.fixture(scope="module", autouse=True)
def built():
    if not os.path.exists(os.path.join(P.PKG, "libpfs_png.so")):
        from probabilistic_fluid_simulation_gb300 import build
        build.build_cli()


def rgba_expected(samples, ctype, depth, palette=None, trns=None):
    s = samples.astype(np.int64)
    h, w = s.shape[:2]
    out = np.zeros((h, w, 4), np.int64)
    out[..., 3] = 255
    if ctype == 0:
        g = s * (255 // ((1 << depth) - 1))
        out[..., 0] = out[..., 1] = out[..., 2] = g
        if trns is not None:
            out[..., 3] = np.where(s == ((trns[0] << 8) | trns[1]), 0, 255)
    elif ctype == 2:
        out[..., :3] = s
        if trns is not None:
            key = [(trns[0] << 8) | trns[1], (trns[2] << 8) | trns[3], (trns[4] << 8) | trns[5]]
            out[..., 3] = np.where((s == key).all(axis=-1), 0, 255)
    elif ctype == 3:
        pal = np.asarray(palette, np.int64)
        out[..., :3] = pal[s]
        if trns is not None:
            alpha = np.full(len(pal), 255, np.int64)
            alpha[:len(trns)] = list(trns)
            out[..., 3] = alpha[s]
    elif ctype == 4:
        out[..., 0] = out[..., 1] = out[..., 2] = s[..., 0]
        out[..., 3] = s[..., 1]
    else:
        out[...] = s
    return out.astype(np.uint8)


CASES = [  # ctype, depth, w, h
    (0, 1, 13, 7), (0, 2, 9, 5), (0, 4, 17, 6), (0, 8, 23, 11),
    (2, 8, 31, 9), (3, 1, 10, 4), (3, 2, 11, 5), (3, 4, 19, 8), (3, 8, 37, 12),
    (4, 8, 21, 10), (6, 8, 33, 17),
]


@pytest.mark.parametrize("interlace", [False, True])
@pytest.mark.parametrize("ctype,depth,w,h", CASES)
def test_decode_matches_independent_writer(ctype, depth, w, h, interlace):
    rng = np.random.default_rng(ctype * 100 + depth + w)
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    top = (1 << depth) - 1
    palette = trns = None
    if ctype == 3:
        npal = min(top + 1, 40)
        palette = rng.integers(0, 256, (npal, 3))
        samples = rng.integers(0, npal, (h, w))
        trns = list(rng.integers(0, 256, npal // 2))
    else:
        samples = rng.integers(0, top + 1, (h, w) if chans == 1 else (h, w, chans))
        if ctype == 0:
            v = int(samples[0, 0])
            trns = [v >> 8, v & 255]
        elif ctype == 2:
            px = samples[1, 2]
            trns = sum(([int(c) >> 8, int(c) & 255] for c in px), [])
    png = P.encode(samples, ctype, depth, interlace, palette, trns)
    got, err = P.c_decode(png)
    assert err is None, err
    assert np.array_equal(got, rgba_expected(samples, ctype, depth, palette, trns))


@pytest.mark.parametrize("level,strategy", [(0, None), (1, zlib.Z_FIXED), (9, None), (6, zlib.Z_HUFFMAN_ONLY),
                                            (6, zlib.Z_RLE)])
def test_inflate_all_block_types(level, strategy):
    rng = np.random.default_rng(level)
    data = bytes(np.repeat(rng.integers(0, 7, 3000), rng.integers(1, 30, 3000)).astype(np.uint8)) + os.urandom(5000)
    co = zlib.compressobj(level, zlib.DEFLATED, 15, 8, strategy if strategy is not None else zlib.Z_DEFAULT_STRATEGY)
    z = co.compress(data) + co.flush()
    assert P.c_inflate(z) == data
    assert P.c_inflate(z[:-1]) is None  # truncated checksum
    bad = bytearray(z)
    bad[-1] ^= 1
    assert P.c_inflate(bytes(bad)) is None  # checksum mismatch


@pytest.mark.parametrize("w,h", [(1, 1), (7, 3), (64, 48), (257, 33)])
def test_encode_roundtrip(w, h):
    rng = np.random.default_rng(w * h)
    yy, xx = np.mgrid[0:h, 0:w]
    smooth = (127 + 100 * np.sin(xx / 9.0)[..., None] * np.cos(yy / 7.0)[..., None] * np.ones(4)).astype(np.uint8)
    noisy = rng.integers(0, 256, (h, w, 4)).astype(np.uint8)
    for img in (smooth, noisy, np.zeros((h, w, 4), np.uint8)):
        png = P.c_encode(img)
        assert np.array_equal(P.decode_rgba8(png), img)  # independent reader
        got, err = P.c_decode(png)
        assert err is None and np.array_equal(got, img)
    if w * h >= 64 * 48:
        assert len(P.c_encode(smooth)) < smooth.size // 2  # compressed


def test_decode_rejects_bad_files():
    img = np.arange(4 * 5 * 4, dtype=np.uint8).reshape(4, 5, 4)
    png = P.encode(img, 6)
    assert P.c_decode(png[:-20])[0] is None  # truncated
    bad = bytearray(png)
    bad[40] ^= 0xFF  # inside IHDR or IDAT: CRC mismatch
    assert "CRC" in P.c_decode(bytes(bad))[1]
    assert P.c_decode(b"not a png at all")[1] == "not a PNG file"
    ihdr16 = P._chunk(b"IHDR", struct.pack(">IIBBBBB", 5, 4, 16, 6, 0, 0, 0))  # 16-bit RGBA header
    assert P.c_decode(png[:8] + ihdr16 + png[8 + 25:])[1] == "16-bit PNGs are not supported"
