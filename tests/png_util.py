"""An independent PNG writer / reader in Python (stdlib zlib) for testing the
library's own codec and command-line driver, plus ctypes access to the codec
(libpfs_png.so)."""
import ctypes as C
import os
import struct
import zlib

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "probabilistic_fluid_simulation_gb300")
CLI = os.path.join(PKG, "fluidsim_gb300")

ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def _chunk(t, data):
    return struct.pack(">I", len(data)) + t + data + struct.pack(">I", zlib.crc32(t + data) & 0xFFFFFFFF)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def _filter_rows(rows, bpp, first_filter=0):
    """Filter each row with filter (first_filter + y) % 5, so all five occur."""
    out = bytearray()
    prior = bytes(len(rows[0])) if rows else b""
    for y, row in enumerate(rows):
        f = (first_filter + y) % 5
        fr = bytearray(len(row))
        for i, x in enumerate(row):
            a = row[i - bpp] if i >= bpp else 0
            b = prior[i]
            c = prior[i - bpp] if i >= bpp else 0
            p = (0, a, b, (a + b) // 2, _paeth(a, b, c))[f]
            fr[i] = (x - p) & 0xFF
        out.append(f)
        out += fr
        prior = row
    return bytes(out)


def _pack_samples(samples, depth):
    """One row of samples (ints) at `depth` bits, MSB first."""
    if depth == 8:
        return bytes(int(s) for s in samples)
    out, acc, nbits = bytearray(), 0, 0
    for s in samples:
        acc = (acc << depth) | int(s)
        nbits += depth
        if nbits == 8:
            out.append(acc)
            acc, nbits = 0, 0
    if nbits:
        out.append(acc << (8 - nbits))
    return bytes(out)


def encode(samples, ctype, depth=8, interlace=False, palette=None, trns=None, level=6, strategy=None):
    """PNG bytes for `samples`: (h, w) for colour types 0 / 3, (h, w, c) otherwise."""
    h, w = samples.shape[:2]
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bpp = max(1, chans * depth // 8)
    flat = samples.reshape(h, w, chans)
    raw = bytearray()
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    for k, (x0, y0, dx, dy) in enumerate(passes):
        sub = flat[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        rows = [_pack_samples(r.reshape(-1), depth) for r in sub]
        raw += _filter_rows(rows, bpp, first_filter=k)
    if strategy is None:
        comp = zlib.compress(bytes(raw), level)
    else:
        co = zlib.compressobj(level, zlib.DEFLATED, 15, 8, strategy)
        comp = co.compress(bytes(raw)) + co.flush()
    png = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    if palette is not None:
        png += _chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    if trns is not None:
        png += _chunk(b"tRNS", bytes(trns))
    # split the image data over two IDAT chunks, as encoders may
    half = len(comp) // 2
    png += _chunk(b"IDAT", comp[:half]) + _chunk(b"IDAT", comp[half:]) + _chunk(b"IEND", b"")
    return png


def decode_rgba8(data):
    """RGBA 8-bit non-interlaced PNG -> (h, w, 4) uint8."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w = 8, b"", 0
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        t = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        assert zlib.crc32(t + body) & 0xFFFFFFFF == struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        if t == b"IHDR":
            w, h, depth, ctype, _, _, il = struct.unpack(">IIBBBBB", body)
            assert (depth, ctype, il) == (8, 6, 0)
        elif t == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    stride = w * 4
    out = np.zeros((h, stride), np.int32)
    prior = np.zeros(stride, np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        row = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int32)
        cur = np.zeros(stride, np.int32)
        for i in range(stride):
            a = cur[i - 4] if i >= 4 else 0
            b = prior[i]
            c = prior[i - 4] if i >= 4 else 0
            p = (0, a, b, (a + b) // 2, _paeth(a, b, c))[f]
            cur[i] = (row[i] + p) & 0xFF
        out[y] = cur
        prior = cur
    return out.reshape(h, w, 4).astype(np.uint8)


_lib = None


def codec():
    global _lib
    if _lib is None:
        _lib = C.CDLL(os.path.join(PKG, "libpfs_png.so"))
        _lib.pfs_png_decode.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(C.c_void_p), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int), C.c_char_p, C.c_int]
        _lib.pfs_png_encode.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)]
        _lib.pfs_zlib_inflate.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)]
        _lib.pfs_png_free.argtypes = [C.c_void_p]
    return _lib


def c_decode(data):
    """(rgba (h, w, 4) uint8, None) or (None, error message)."""
    lib = codec()
    p, w, h = C.c_void_p(), C.c_int(), C.c_int()
    err = C.create_string_buffer(256)
    rc = lib.pfs_png_decode(data, len(data), C.byref(p), C.byref(w), C.byref(h), err, 256)
    if rc != 0:
        return None, err.value.decode()
    arr = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint8)), shape=(h.value, w.value, 4)).copy()
    lib.pfs_png_free(p)
    return arr, None


def c_encode(rgba):
    lib = codec()
    rgba = np.ascontiguousarray(rgba, np.uint8)
    p, n = C.c_void_p(), C.c_size_t()
    assert lib.pfs_png_encode(rgba.ctypes.data, rgba.shape[1], rgba.shape[0], C.byref(p), C.byref(n)) == 0
    out = C.string_at(p, n.value)
    lib.pfs_png_free(p)
    return out


def c_inflate(data):
    lib = codec()
    p, n = C.c_void_p(), C.c_size_t()
    if lib.pfs_zlib_inflate(data, len(data), C.byref(p), C.byref(n)) != 0:
        return None
    out = C.string_at(p, n.value)
    lib.pfs_png_free(p)
    return out
