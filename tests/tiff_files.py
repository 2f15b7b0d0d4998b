"""Writes small grayscale TIFF files for the tests (baseline TIFF 6.0: one image, strips;
uncompressed, PackBits or LZW data, LZW optionally with the horizontal predictor).

The reference's own TIFF test images are Git LFS pointers without their payload, so the
tests build their images here from seeded pixel arrays whose values they know."""

import struct

import numpy as np


def _lzw_encode(data):
    """TIFF LZW (MSB-first codes, 256 clear, 257 end; the code width grows when the next
    free code no longer fits, and a clear is sent when the table reaches 4094 entries)."""
    out = []
    acc, nacc = 0, 0

    def put(code, width):
        nonlocal acc, nacc
        acc = (acc << width) | code
        nacc += width
        while nacc >= 8:
            out.append((acc >> (nacc - 8)) & 0xFF)
            nacc -= 8

    def reset():
        return {bytes([i]): i for i in range(256)}, 258, 9

    table, nxt, width = reset()
    put(256, width)
    w = b""
    for byte in data:
        wc = w + bytes([byte])
        if wc in table:
            w = wc
            continue
        put(table[w], width)
        table[wc] = nxt
        nxt += 1
        if nxt == 4094:
            put(256, width)
            table, nxt, width = reset()
        elif nxt > (1 << width) - 1:
            width += 1
        w = bytes([byte])
    if w:
        put(table[w], width)
        nxt += 1
        if nxt > (1 << width) - 1 and width < 12:
            width += 1
    put(257, width)
    if nacc:
        out.append((acc << (8 - nacc)) & 0xFF)
    return bytes(out)


def _packbits(data):
    out = bytearray()
    i, n = 0, len(data)
    while i < n:
        j = i
        while j < n and j - i < 128 and data[j] == data[i]:
            j += 1
        if j - i >= 3:
            out += struct.pack("b", 1 - (j - i)) + data[i:i + 1]
            i = j
            continue
        j = i
        while j < n and j - i < 128 and not (j + 2 < n and data[j] == data[j + 1] == data[j + 2]):
            j += 1
        out += struct.pack("b", j - i - 1) + data[i:j]
        i = j
    return bytes(out)


def write_tiff(path, values, bits=8, photometric=1, big_endian=False, compression="none", predictor=False,
               resolution=(72, 1), position=None, rows_per_strip=None, res_tags=True):
    """values: (rows, cols) unsigned integers < 2**bits (scanline-major).  resolution and
    position are RATIONAL (numerator, denominator) pairs used for both axes."""
    e = ">" if big_endian else "<"
    v = np.asarray(values, dtype=np.uint64)
    rows, cols = v.shape
    bps = max(bits // 8, 1)
    if bits == 4:
        # two samples per byte (only written to check that the reader rejects it)
        packed = bytearray()
        for r in range(rows):
            row = [int(x) & 0xF for x in v[r]] + [0]
            packed += bytes((row[k] << 4) | row[k + 1] for k in range(0, cols, 2))
        strips_rows = [(0, rows)]
        payloads = [bytes(packed)]
    else:
        dt = np.dtype({1: "u1", 2: "u2", 4: "u4", 8: "u8"}[bps]).newbyteorder(e)
        if predictor:
            mask = (1 << bits) - 1 if bits < 64 else 0xFFFFFFFFFFFFFFFF
            d = v.copy()
            d[:, 1:] = (v[:, 1:] - v[:, :-1]) & np.uint64(mask)
            v_enc = d
        else:
            v_enc = v
        rps = rows_per_strip or rows
        strips_rows = [(r0, min(rows, r0 + rps)) for r0 in range(0, rows, rps)]
        payloads = []
        for r0, r1 in strips_rows:
            raw = v_enc[r0:r1].astype(dt).tobytes()
            if compression == "lzw":
                raw = _lzw_encode(raw)
            elif compression == "packbits":
                raw = _packbits(raw)
            payloads.append(raw)
    comp = {"none": 1, "lzw": 5, "packbits": 32773}[compression]
    # layout: header, image data, rationals, strip arrays, IFD
    body = bytearray(b"MM" if big_endian else b"II") + struct.pack(e + "HI", 42, 0)
    offsets = []
    for p in payloads:
        offsets.append(len(body))
        body += p
        if len(body) % 2:
            body += b"\0"
    extra = {}

    def put_extra(key, fmt, vals):
        if len(body) % 2:
            body.extend(b"\0")
        extra[key] = len(body)
        body.extend(struct.pack(e + fmt * len(vals), *vals))

    put_extra("res", "I", list(resolution))
    if position is not None:
        put_extra("pos", "I", list(position))
    if len(payloads) > 1:
        put_extra("so", "I", offsets)
        put_extra("sc", "I", [len(p) for p in payloads])
    entries = [(256, 4, 1, cols), (257, 4, 1, rows), (258, 3, 1, bits), (259, 3, 1, comp), (262, 3, 1, photometric)]
    if len(payloads) > 1:
        entries += [(273, 4, len(payloads), extra["so"]), (279, 4, len(payloads), extra["sc"])]
    else:
        entries += [(273, 4, 1, offsets[0]), (279, 4, 1, len(payloads[0]))]
    entries += [(277, 3, 1, 1), (278, 4, 1, strips_rows[0][1] - strips_rows[0][0])]
    if res_tags:
        entries += [(282, 5, 1, extra["res"]), (283, 5, 1, extra["res"])]
    if position is not None:
        entries += [(286, 5, 1, extra["pos"]), (287, 5, 1, extra["pos"])]
    if predictor:
        entries += [(317, 3, 1, 2)]
    entries.sort()
    if len(body) % 2:
        body += b"\0"
    ifd = len(body)
    body[4:8] = struct.pack(e + "I", ifd)
    body += struct.pack(e + "H", len(entries))
    for tag, typ, cnt, val in entries:
        if typ == 3 and cnt == 1:
            body += struct.pack(e + "HHIHH", tag, typ, cnt, val, 0)
        else:
            body += struct.pack(e + "HHII", tag, typ, cnt, val)
    body += struct.pack(e + "I", 0)
    with open(path, "wb") as f:
        f.write(bytes(body))


def seeded_image(rows, cols, bits, seed=0):
    """Smooth seeded pattern with a random component, all values < 2**bits."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:rows, 0:cols]
    base = 0.5 + 0.35 * np.sin(x / 5.0) * np.cos(y / 7.0) + 0.1 * rng.random((rows, cols))
    top = float((1 << bits) - 1) if bits < 64 else float(2 ** 63)
    return np.clip(np.floor(base * top), 0, top).astype(np.uint64)
