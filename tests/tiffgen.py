"""Minimal multi-page TIFF writer for the decoder tests: classic TIFF or
BigTIFF, either byte order, strips or tiles, and the encodings the decoder
accepts (none, PackBits, LZW, Deflate), optionally with horizontal
differencing.  Written from the TIFF 6.0 and BigTIFF layouts."""

from __future__ import annotations

import struct
import zlib

import numpy as np

NONE, LZW, DEFLATE, PACKBITS = 1, 5, 8, 32773


def packbits(data: bytes) -> bytes:
    out = bytearray()
    i, n = 0, len(data)
    while i < n:
        j = i + 1
        while j < n and j - i < 128 and data[j] == data[i]:
            j += 1
        if j - i >= 2:
            out.append((257 - (j - i)) & 0xFF)  # -(run - 1)
            out.append(data[i])
            i = j
            continue
        j = i + 1
        while j < n and j - i < 128 and not (j + 1 < n and data[j] == data[j + 1]):
            j += 1
        out.append(j - i - 1)
        out += data[i:j]
        i = j
    return bytes(out)


def lzw(data: bytes) -> bytes:
    """TIFF LZW: MSB-first codes of 9..12 bits; the width grows once the table
    holds 2^width entries; Clear before the table overflows."""
    out = bytearray()
    acc, nacc = 0, 0

    def emit(code, width):
        nonlocal acc, nacc
        acc = (acc << width) | code
        nacc += width
        while nacc >= 8:
            out.append((acc >> (nacc - 8)) & 0xFF)
            nacc -= 8
        acc &= (1 << nacc) - 1

    def reset():
        return {bytes([i]): i for i in range(256)}, 258, 9

    table, nxt, width = reset()
    emit(256, width)
    w = b""
    for c in data:
        wc = w + bytes([c])
        if wc in table:
            w = wc
            continue
        emit(table[w], width)
        table[wc] = nxt
        nxt += 1
        if nxt >= (1 << width) and width < 12:
            width += 1
        if nxt >= 4093:
            emit(256, width)
            table, nxt, width = reset()
        w = bytes([c])
    if w:
        emit(table[w], width)
    emit(257, width)
    if nacc:
        out.append((acc << (8 - nacc)) & 0xFF)
    return bytes(out)


# zlib settings for Deflate data: every block type (stored, fixed and dynamic
# codes) and several match strategies
DEFLATE_MODES = {
    "default": (6, zlib.Z_DEFAULT_STRATEGY),
    "stored": (0, zlib.Z_DEFAULT_STRATEGY),
    "fixed": (6, zlib.Z_FIXED),
    "huffman": (6, zlib.Z_HUFFMAN_ONLY),
    "rle": (6, zlib.Z_RLE),
    "best": (9, zlib.Z_FILTERED),
}


def encode(raw: bytes, compression: int, deflate_mode: str = "default") -> bytes:
    if compression == NONE:
        return raw
    if compression == PACKBITS:
        return packbits(raw)
    if compression == LZW:
        return lzw(raw)
    if compression == DEFLATE:
        level, strategy = DEFLATE_MODES[deflate_mode]
        c = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
        return c.compress(raw) + c.flush()
    raise ValueError(compression)


def difference(rows: np.ndarray) -> np.ndarray:
    d = rows.astype(np.int16)
    d[:, 1:] = d[:, 1:] - rows[:, :-1].astype(np.int16)
    return (d & 0xFF).astype(np.uint8)


def write_tiff(path, pages, compression=NONE, big=False, byteorder="<", rows_per_strip=None, tile=None,
               predictor=1, bits=8, photometric=1, samples=1, sample_format=1, deflate_mode="default"):
    """pages: list of 2-D u8 (or u16 when bits == 16) arrays, one per page."""
    e = byteorder
    head = bytearray()
    head += b"II" if e == "<" else b"MM"
    if big:
        head += struct.pack(e + "HHHQ", 43, 8, 0, 0)
    else:
        head += struct.pack(e + "HI", 42, 0)
    blob = bytearray(head)
    ifd_offsets = []
    for page in pages:
        page = np.ascontiguousarray(page)
        h, w = page.shape[:2]
        chunks = []
        if tile is not None:
            tw, th = tile
            for ty in range(0, h, th):
                for tx in range(0, w, tw):
                    t = np.zeros((th, tw) + page.shape[2:], page.dtype)
                    part = page[ty:ty + th, tx:tx + tw]
                    t[:part.shape[0], :part.shape[1]] = part
                    if predictor == 2:
                        t = difference(t)
                    chunks.append(encode(t.tobytes(), compression, deflate_mode))
        else:
            rps = rows_per_strip or h
            for y in range(0, h, rps):
                s = page[y:y + rps]
                if predictor == 2:
                    s = difference(s)
                chunks.append(encode(s.astype(page.dtype.newbyteorder(e)).tobytes() if bits == 16 else s.tobytes(),
                                     compression))
        offs = []
        for c in chunks:
            if len(blob) % 2:
                blob.append(0)
            offs.append(len(blob))
            blob += c
        counts = [len(c) for c in chunks]
        long_t = 16 if big else 4
        tags = [(256, 4, [w]), (257, 4, [h]), (258, 3, [bits] * samples), (259, 3, [compression]),
                (262, 3, [photometric]), (277, 3, [samples])]
        if tile is not None:
            tags += [(322, 3, [tile[0]]), (323, 3, [tile[1]]), (324, long_t, offs), (325, long_t, counts)]
        else:
            tags += [(273, long_t, offs), (278, 4, [rows_per_strip or h]), (279, long_t, counts)]
        if predictor != 1:
            tags.append((317, 3, [predictor]))
        if sample_format != 1:
            tags.append((339, 3, [sample_format]))
        tags.sort()
        if len(blob) % 2:
            blob.append(0)
        ifd_at = len(blob)
        ifd_offsets.append(ifd_at)
        fmt_code = {3: "H", 4: "I", 16: "Q"}
        size = {3: 2, 4: 4, 16: 8}
        entry_sz, inline = (20, 8) if big else (12, 4)
        nent = len(tags)
        ifd_len = (8 if big else 2) + nent * entry_sz + (8 if big else 4)
        extra_at = ifd_at + ifd_len
        ifd = bytearray(struct.pack(e + ("Q" if big else "H"), nent))
        extra = bytearray()
        for tag, typ, vals in tags:
            payload = struct.pack(e + fmt_code[typ] * len(vals), *vals)
            if len(payload) <= inline:
                field = payload + b"\0" * (inline - len(payload))
            else:
                field = struct.pack(e + ("Q" if big else "I"), extra_at + len(extra))
                extra += payload
            ifd += struct.pack(e + ("HHQ" if big else "HHI"), tag, typ, len(vals)) + field
        ifd += struct.pack(e + ("Q" if big else "I"), 0)  # patched below
        blob += ifd + extra
    for k, at in enumerate(ifd_offsets):
        nxt = ifd_offsets[k + 1] if k + 1 < len(ifd_offsets) else 0
        nent = struct.unpack_from(e + ("Q" if big else "H"), blob, at)[0]
        pos = at + (8 if big else 2) + nent * (20 if big else 12)
        struct.pack_into(e + ("Q" if big else "I"), blob, pos, nxt)
    struct.pack_into(e + ("Q" if big else "I"), blob, 8 if big else 4, ifd_offsets[0])
    with open(path, "wb") as f:
        f.write(bytes(blob))
