"""Image decoding for texture maps, in place of the reference's stb_image
(TextureMap::load_from_file, scene/mod.rs:174-202): PNG (8-bit RGB, RGBA or
palette, non-interlaced; inflated with the standard library's zlib) and binary
PPM. Like the reference, only 3- or 4-component images are accepted; rows are
returned top row first (stb's layout)."""
from __future__ import annotations

import struct
import zlib

import numpy as np


class ImageError(ValueError):
    pass


def _unfilter(raw: bytes, h: int, stride: int, bpp: int) -> np.ndarray:
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        off = y * (stride + 1)
        f = raw[off]
        line = np.frombuffer(raw, np.uint8, stride, off + 1).astype(np.int32)
        if f == 0:
            cur = line
        elif f == 1:  # Sub: running sum over the pixels of the row
            cur = np.cumsum(line.reshape(-1, bpp), axis=0).reshape(-1) & 0xFF
        elif f == 2:  # Up
            cur = (line + prev) & 0xFF
        elif f in (3, 4):  # Average, Paeth: sequential along the row
            cur = np.zeros(stride, np.int32)
            for i in range(stride):
                a = cur[i - bpp] if i >= bpp else 0
                b = prev[i]
                if f == 3:
                    cur[i] = (line[i] + ((a + b) >> 1)) & 0xFF
                else:
                    c = prev[i - bpp] if i >= bpp else 0
                    p = a + b - c
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                    pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                    cur[i] = (line[i] + pred) & 0xFF
        else:
            raise ImageError(f"bad PNG filter {f}")
        out[y] = cur
        prev = cur
    return out


def read_png(path: str):
    """(image bytes (H*W*C,), width, height, components)."""
    data = open(path, "rb").read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ImageError(f"{path}: not a PNG file")
    pos, idat, plte, trns, hdr = 8, [], None, None, None
    while pos + 8 <= len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if typ == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"PLTE":
            plte = body
        elif typ == b"tRNS":
            trns = body
        elif typ == b"IDAT":
            idat.append(body)
        elif typ == b"IEND":
            break
    if hdr is None:
        raise ImageError(f"{path}: no IHDR")
    w, h, depth, ctype, _, _, interlace = hdr
    if depth != 8 or interlace != 0 or ctype not in (2, 3, 6):
        raise ImageError(f"{path}: unsupported PNG (bit depth {depth}, colour type {ctype}, interlace {interlace})")
    ch = {2: 3, 6: 4, 3: 1}[ctype]
    px = _unfilter(zlib.decompress(b"".join(idat)), h, w * ch, ch)
    if ctype == 3:
        if plte is None:
            raise ImageError(f"{path}: palette image without PLTE")
        pal = np.frombuffer(plte, np.uint8).reshape(-1, 3)
        if trns is not None:
            alpha = np.full(len(pal), 255, np.uint8)
            t = np.frombuffer(trns, np.uint8)[:len(pal)]
            alpha[:len(t)] = t
            pal = np.concatenate([pal, alpha[:, None]], 1)
        img = pal[px.reshape(-1)]
        ch = pal.shape[1]
    else:
        img = px.reshape(-1, ch)
    return np.ascontiguousarray(img, np.uint8).reshape(-1), w, h, ch


def read_ppm(path: str):
    data = open(path, "rb").read()
    parts, pos = [], 0
    while len(parts) < 4:
        while data[pos:pos + 1].isspace():
            pos += 1
        if data[pos:pos + 1] == b"#":
            pos = data.index(b"\n", pos) + 1
            continue
        end = pos
        while not data[end:end + 1].isspace():
            end += 1
        parts.append(data[pos:end])
        pos = end
    if parts[0] != b"P6" or int(parts[3]) != 255:
        raise ImageError(f"{path}: only binary 8-bit PPM (P6) is supported")
    w, h = int(parts[1]), int(parts[2])
    img = np.frombuffer(data, np.uint8, w * h * 3, pos + 1).copy()
    return img, w, h, 3


def write_ppm(path: str, rgb: np.ndarray):
    h, w = rgb.shape[:2]
    with open(path, "wb") as f:
        f.write(f"P6\n{w} {h}\n255\n".encode())
        f.write(np.ascontiguousarray(rgb[..., :3], np.uint8).tobytes())


def write_png(path: str, rgba: np.ndarray):
    """8-bit RGB or RGBA PNG, filter 0 on every row, zlib level 6."""
    h, w, c = rgba.shape
    ctype = {3: 2, 4: 6}[c]
    raw = b"".join(b"\x00" + np.ascontiguousarray(rgba[y], np.uint8).tobytes() for y in range(h))

    def chunk(t, body):
        return struct.pack(">I", len(body)) + t + body + struct.pack(">I", zlib.crc32(t + body) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


def read_image(path: str):
    low = path.lower()
    if low.endswith(".png"):
        return read_png(path)
    if low.endswith(".ppm"):
        return read_ppm(path)
    raise ImageError(f"{path}: unsupported image format (PNG and PPM are decoded)")
