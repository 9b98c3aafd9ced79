"""Image files of the command-line tool: what ``image::open`` and ``ImageBuffer::save`` do for
the reference (the image crate 0.25 with its ``png``, ``jpeg`` and ``webp`` features, Cargo.toml:13;
src/image_pipeline.rs:1087-1152), restated for PNG, JPEG and WebP, plus the binary netpbm formats
(PGM, PPM) as a convenience.

``read_image`` returns what the renderer consumes from a ``DynamicImage``
(src/image_pipeline.rs:259-296, 1017-1024): an 8-bit gray image without transparency stays gray
(``DynamicImage::ImageLuma8``, (H, W) u8); every other kind goes through ``to_rgb8`` ((H, W, 3)
u8: alpha dropped, palette looked up, 16-bit samples rounded to 8 bits, gray replicated).
Low bit-depth gray is widened to 8 bits by bit replication, as the png crate's ``EXPAND`` does.

PNG chunks, zlib, Adam7 passes and sample unpacking are done here; the row filters are undone by
the library's ``fg_png_unfilter`` (host C++ in fgrain_gb300/host/, native for speed on large scans).
JPEG and WebP are coded by the library's host C++ codecs (``fg_jpeg_*``, ``fg_webp_*``):

- JPEG: sequential Huffman-coded files are read (gray stays gray, as the crate's ``ImageLuma8``;
  colour gives RGB); progressive, arithmetic-coded, 12-bit and CMYK files raise
  ``ImageFormatError``.  Writing is baseline JFIF at quality 75, the crate's ``JpegEncoder``
  default (gray as one component, colour as YCbCr with 2x2 chroma subsampling).
- WebP: lossless files are read (the crate's decoder gives ``Rgb8``/``Rgba8``, which the renderer
  takes through ``to_rgb8``: RGB, alpha dropped); lossy (VP8) and animated files raise
  ``ImageFormatError``.  Writing is lossless, as the crate's WebP encoder writes.
"""
from __future__ import annotations

import ctypes as C
import struct
import zlib
from pathlib import Path

import numpy as np

from . import _abi

PNG_SIGNATURE = b"\x89PNG\r\n\x1a\n"
_ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))
_SAMPLES = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}  # samples per pixel of each PNG colour type
_DEPTHS = {0: (1, 2, 4, 8, 16), 2: (8, 16), 3: (1, 2, 4, 8), 4: (8, 16), 6: (8, 16)}


class ImageFormatError(ValueError):
    """An image file this build cannot read or write (the reference's ``ImageError``)."""


# ---- reading ----

def read_image(path) -> np.ndarray:
    data = Path(path).read_bytes()
    if data[:8] == PNG_SIGNATURE:
        return decode_png(data)
    if data[:2] in (b"P5", b"P6"):
        return decode_pnm(data)
    if data[:3] == b"\xff\xd8\xff":
        return decode_jpeg(data)
    if data[:4] == b"RIFF" and data[8:12] == b"WEBP":
        return decode_webp(data)
    raise ImageFormatError(f"'{path}' is not a PNG, JPEG, WebP, PGM or PPM file")


def _codec_call(fn, *args) -> None:
    msg = C.create_string_buffer(256)
    if fn(*args, msg, len(msg)) != 0:
        raise ImageFormatError(msg.value.decode(errors="replace") or "corrupt image file")


def decode_jpeg(data: bytes) -> np.ndarray:
    """(H, W) u8 for a gray JPEG, (H, W, 3) u8 RGB otherwise."""
    lib = _abi.load()
    w, h, ch = C.c_uint32(), C.c_uint32(), C.c_uint32()
    _codec_call(lib.fg_jpeg_info, data, len(data), C.byref(w), C.byref(h), C.byref(ch))
    out = np.empty(h.value * w.value * ch.value, np.uint8)
    _codec_call(lib.fg_jpeg_decode, data, len(data), out.ctypes.data, out.nbytes)
    return out.reshape(h.value, w.value) if ch.value == 1 else out.reshape(h.value, w.value, 3)


def decode_webp_rgba(data: bytes) -> np.ndarray:
    """(H, W, 4) u8 RGBA pixels of a lossless WebP file."""
    lib = _abi.load()
    w, h, alpha = C.c_uint32(), C.c_uint32(), C.c_uint32()
    _codec_call(lib.fg_webp_info, data, len(data), C.byref(w), C.byref(h), C.byref(alpha))
    out = np.empty((h.value, w.value, 4), np.uint8)
    _codec_call(lib.fg_webp_decode, data, len(data), out.ctypes.data, out.nbytes)
    return out


def decode_webp(data: bytes) -> np.ndarray:
    """(H, W, 3) u8: the RGB of a lossless WebP file (``to_rgb8``)."""
    return np.ascontiguousarray(decode_webp_rgba(data)[:, :, :3])


def _chunks(data: bytes):
    pos = 8
    while pos + 12 <= len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if len(body) != n or pos + 12 + n > len(data):
            raise ImageFormatError("truncated PNG chunk")
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        if zlib.crc32(kind + body) & 0xFFFFFFFF != crc:
            raise ImageFormatError(f"CRC mismatch in PNG chunk {kind!r}")
        yield kind, body
        pos += 12 + n
        if kind == b"IEND":
            return
    raise ImageFormatError("PNG ends before IEND")


def _unfilter(raw: bytearray, h: int, stride: int, bpp: int) -> np.ndarray:
    """Reconstructs h scanlines of stride bytes (each preceded by its filter byte)."""
    need = h * (stride + 1)
    if len(raw) < need:
        raise ImageFormatError("PNG image data is too short")
    buf = (C.c_uint8 * need).from_buffer(raw)
    if _abi.load().fg_png_unfilter(C.cast(buf, C.c_void_p), h, stride, bpp) != 0:
        raise ImageFormatError("unknown PNG filter type")
    return np.frombuffer(raw, np.uint8, need).reshape(h, stride + 1)[:, 1:]


def _samples(rows: np.ndarray, w: int, spp: int, depth: int) -> np.ndarray:
    """(h, w, spp) samples (u8, or u16 for 16-bit) of reconstructed scanlines."""
    h = rows.shape[0]
    if depth == 8:
        return rows[:, :w * spp].reshape(h, w, spp)
    if depth == 16:
        return rows[:, :2 * w * spp].copy().view(">u2").astype(np.uint16).reshape(h, w, spp)
    bits = np.unpackbits(rows, axis=1)[:, :w * depth].reshape(h, w, depth)
    weights = (1 << np.arange(depth - 1, -1, -1)).astype(np.uint8)
    return (bits * weights).sum(axis=2, dtype=np.uint8).reshape(h, w, 1)


def decode_png(data: bytes) -> np.ndarray:
    hdr = None
    palette = None
    trns = None
    idat = []
    for kind, body in _chunks(data):
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = body
        elif kind == b"IDAT":
            idat.append(body)
    if hdr is None:
        raise ImageFormatError("PNG without IHDR")
    w, h, depth, ctype, comp, filt, interlace = hdr
    if ctype not in _SAMPLES or depth not in _DEPTHS[ctype] or comp != 0 or filt != 0 or interlace > 1:
        raise ImageFormatError(f"unsupported PNG header (colour type {ctype}, depth {depth})")
    if w == 0 or h == 0:
        raise ImageFormatError("PNG with a zero dimension")
    if ctype == 3 and palette is None:
        raise ImageFormatError("palette PNG without PLTE")
    spp = _SAMPLES[ctype]
    bits = spp * depth
    bpp = max(1, bits // 8)
    try:
        raw = bytearray(zlib.decompress(b"".join(idat)))
    except zlib.error as exc:
        raise ImageFormatError(f"corrupt PNG image data: {exc}") from None
    dtype = np.uint16 if depth == 16 else np.uint8
    img = np.zeros((h, w, spp), dtype)
    passes = _ADAM7 if interlace else ((0, 0, 1, 1),)
    pos = 0
    for x0, y0, dx, dy in passes:
        pw, ph = (w - x0 + dx - 1) // dx, (h - y0 + dy - 1) // dy
        if pw <= 0 or ph <= 0:
            continue
        stride = (pw * bits + 7) // 8
        n = ph * (stride + 1)
        part = raw[pos:pos + n]
        pos += n
        img[y0::dy, x0::dx] = _samples(_unfilter(part, ph, stride, bpp), pw, spp, depth)
    return _to_renderer_input(img, ctype, depth, palette, trns)


def _to8(v: np.ndarray) -> np.ndarray:
    """16-bit samples to 8 bits, rounded (v / 257)."""
    return ((v.astype(np.uint32) + 128) // 257).astype(np.uint8)


def _to_renderer_input(img, ctype, depth, palette, trns) -> np.ndarray:
    if ctype == 0:
        g = img[:, :, 0]
        g = _to8(g) if depth == 16 else (g * np.uint8(255 // ((1 << depth) - 1)) if depth < 8 else g)
        if depth <= 8 and trns is None:
            return np.ascontiguousarray(g)  # ImageLuma8
        return np.repeat(g[:, :, None], 3, axis=2)  # Luma16 / LumaA8: to_rgb8
    if ctype == 3:
        idx = img[:, :, 0]
        if int(idx.max()) >= len(palette):
            raise ImageFormatError("PNG palette index out of range")
        return palette[idx]
    rgb = img[:, :, :3] if ctype in (2, 6) else np.repeat(img[:, :, :1], 3, axis=2)
    return np.ascontiguousarray(_to8(rgb) if depth == 16 else rgb)


def decode_pnm(data: bytes) -> np.ndarray:
    """Binary PGM (P5) or PPM (P6), maxval up to 65535 (16-bit big-endian samples)."""
    fields = []
    pos = 2
    while len(fields) < 3:
        while pos < len(data) and data[pos:pos + 1].isspace():
            pos += 1
        if data[pos:pos + 1] == b"#":
            while pos < len(data) and data[pos:pos + 1] not in (b"\n", b"\r"):
                pos += 1
            continue
        start = pos
        while pos < len(data) and not data[pos:pos + 1].isspace():
            pos += 1
        if start == pos:
            raise ImageFormatError("truncated netpbm header")
        fields.append(int(data[start:pos]))
    pos += 1
    w, h, maxval = fields
    ch = 1 if data[:2] == b"P5" else 3
    if w == 0 or h == 0 or not 0 < maxval < 65536:
        raise ImageFormatError("bad netpbm header")
    n = w * h * ch
    if maxval < 256:
        v = np.frombuffer(data, np.uint8, n, pos).astype(np.uint32)
    else:
        v = np.frombuffer(data, ">u2", n, pos).astype(np.uint32)
    v = v if maxval == 255 else (v * 255 + maxval // 2) // maxval
    v = v.astype(np.uint8)
    return v.reshape(h, w) if ch == 1 else v.reshape(h, w, 3)


# ---- writing ----

def _kind_of(path) -> str:
    ext = Path(path).suffix.lower()
    return {".png": "png", ".pgm": "pnm", ".ppm": "pnm", ".pnm": "pnm", ".jpg": "jpeg", ".jpeg": "jpeg",
            ".webp": "webp"}.get(ext, "png" if ext == "" else ext.lstrip("."))


def encode_png(img: np.ndarray, level: int = 6) -> bytes:
    """8-bit gray ((H, W)) or RGB ((H, W, 3)) PNG, every row with filter type None."""
    a = np.ascontiguousarray(img, np.uint8)
    h, w = a.shape[:2]
    ctype = 0 if a.ndim == 2 else 2
    rows = np.concatenate([np.zeros((h, 1), np.uint8), a.reshape(h, -1)], axis=1)

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    return (PNG_SIGNATURE + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(rows.tobytes(), level)) + chunk(b"IEND", b""))


def _encode(fn, a: np.ndarray, *settings: int) -> bytes:
    h, w = a.shape[:2]
    ch = 1 if a.ndim == 2 else a.shape[2]
    cap = C.c_size_t(0)
    size = max(1 << 16, a.nbytes + a.nbytes // 2 + 4096)
    for _ in range(2):  # the second pass with the size the first reported
        out = np.empty(size, np.uint8)
        if fn(a.ctypes.data, w, h, ch, *settings, out.ctypes.data, out.nbytes, C.byref(cap)) == 0:
            return out[:cap.value].tobytes()
        if cap.value <= size:
            break
        size = cap.value
    raise ImageFormatError("image could not be encoded")


def encode_jpeg(img: np.ndarray, quality: int = 75, options: int = 0) -> bytes:
    """Baseline JFIF of a u8 gray ((H, W)) or RGB ((H, W, 3)) image; quality 1..100; options are
    the encoder's FG_JPEG_* settings (0: 4:2:0, one interleaved scan, no restart markers)."""
    a = np.ascontiguousarray(img, np.uint8)
    if not 1 <= quality <= 100:
        raise ValueError("JPEG quality must be within 1..100")
    return _encode(_abi.load().fg_jpeg_encode, a, quality, options)


def encode_webp(img: np.ndarray, options: int = _abi.FG_WEBP_DEFAULT) -> bytes:
    """Lossless WebP of a u8 gray ((H, W)), RGB ((H, W, 3)) or RGBA ((H, W, 4)) image; options are
    the encoder's FG_WEBP_* tools."""
    a = np.ascontiguousarray(img, np.uint8)
    if a.shape[0] > 16384 or a.shape[1] > 16384:
        raise ImageFormatError("a WebP image is at most 16384 pixels on a side")
    return _encode(_abi.load().fg_webp_encode, a, options)


def write_image(path, img: np.ndarray) -> None:
    """Saves a u8 gray ((H, W)) or RGB ((H, W, 3)) image in the format its extension names."""
    a = np.ascontiguousarray(img, np.uint8)
    if a.ndim not in (2, 3) or (a.ndim == 3 and a.shape[2] != 3):
        raise ValueError("image must be (H, W) or (H, W, 3) u8")
    kind = _kind_of(path)
    if kind == "png":
        data = encode_png(a)
    elif kind == "pnm":
        if Path(path).suffix.lower() == ".pgm" and a.ndim == 3:
            raise ImageFormatError("a PGM file holds gray images only")
        magic = b"P5" if a.ndim == 2 else b"P6"
        data = magic + f"\n{a.shape[1]} {a.shape[0]}\n255\n".encode() + a.tobytes()
    elif kind == "jpeg":
        data = encode_jpeg(a)
    elif kind == "webp":
        data = encode_webp(a)
    else:
        raise ImageFormatError(f"unsupported output format '.{kind}'")
    Path(path).write_bytes(data)
