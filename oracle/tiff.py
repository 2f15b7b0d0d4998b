"""Grayscale TIFF images of the ``tiff`` parser-context type (oracle side, test infrastructure).

The reference reads the image through libtiff, one scanline at a time, and scales each
sample to [0, 1] (src/dune/copasi/common/tiff_file.cc:15-45,
src/dune/copasi/common/tiff_grayscale.cc:21-108).  libtiff is a third-party dependency of
the reference; this module restates the part of baseline TIFF 6.0 the reference relies on
(first image, strips, one sample per pixel of 8/16/32/64 bits; uncompressed, PackBits or
LZW data, LZW with the horizontal-differencing predictor) and the reference's own lookup
arithmetic.
"""

import os
import struct

import numpy as np


class TiffError(ValueError):
    pass


def _lzw_decode(data):
    """TIFF 6.0 section 13 LZW: MSB-first 9..12-bit codes, 256 clear, 257 end, early change."""
    out = bytearray()
    table = [bytes([i]) for i in range(256)] + [b"", b""]
    width, prev = 9, None
    nbits = len(data) * 8
    pos = 0
    while True:
        if pos + width > nbits:
            break
        code = 0
        for _ in range(width):
            code = (code << 1) | ((data[pos >> 3] >> (7 - (pos & 7))) & 1)
            pos += 1
        if code == 257:
            break
        if code == 256:
            table = table[:258]
            width, prev = 9, None
            continue
        if prev is None:
            if code >= 256:
                raise TiffError("LZW code after a clear code is not a literal")
            out += table[code]
            prev = table[code]
            continue
        if code < len(table):
            entry = table[code]
        elif code == len(table):
            entry = prev + prev[:1]
        else:
            raise TiffError("LZW code out of sequence")
        table.append(prev + entry[:1])
        out += entry
        prev = entry
        if len(table) >= (1 << width) - 1 and width < 12:
            width += 1
    return bytes(out)


def _unpack_bits(data):
    out = bytearray()
    i = 0
    while i < len(data):
        c = struct.unpack("b", data[i:i + 1])[0]
        i += 1
        if c >= 0:
            out += data[i:i + c + 1]
            i += c + 1
        elif c != -128:
            out += data[i:i + 1] * (1 - c)
            i += 1
    return bytes(out)


_TYPE_SIZE = {1: 1, 2: 1, 3: 2, 4: 4, 5: 8, 6: 1, 7: 1, 8: 2, 9: 4, 10: 8, 11: 4, 12: 8}


class TiffImage:
    """The first image of a grayscale TIFF file with the reference's value scaling and
    position lookup.  ``px[r, c]``: scanline r, column c, scaled."""

    def __init__(self, path):
        if not os.path.exists(path):
            raise TiffError("File '%s' does not exists." % os.path.abspath(path))
        with open(path, "rb") as f:
            d = f.read()
        if len(d) < 8 or d[:2] not in (b"II", b"MM"):
            raise TiffError("Error opening TIFF file '%s'" % path)
        e = "<" if d[:2] == b"II" else ">"
        if struct.unpack(e + "H", d[2:4])[0] != 42:
            raise TiffError("Error opening TIFF file '%s'" % path)
        ifd = struct.unpack(e + "I", d[4:8])[0]
        n = struct.unpack(e + "H", d[ifd:ifd + 2])[0]
        tags = {}
        for k in range(n):
            o = ifd + 2 + 12 * k
            tag, typ, cnt = struct.unpack(e + "HHI", d[o:o + 8])
            size = _TYPE_SIZE.get(typ, 0) * cnt
            voff = o + 8 if size <= 4 else struct.unpack(e + "I", d[o + 8:o + 12])[0]
            tags[tag] = (typ, cnt, voff)

        def ints(tag):
            typ, cnt, voff = tags[tag]
            fmt = {1: "B", 3: "H", 4: "I"}[typ]
            sz = struct.calcsize(fmt)
            return [struct.unpack(e + fmt, d[voff + i * sz:voff + (i + 1) * sz])[0] for i in range(cnt)]

        def one(tag, default):
            return ints(tag)[0] if tag in tags else default

        def rational(tag):
            if tag not in tags:
                return np.float32(0.0)
            typ, cnt, voff = tags[tag]
            num, den = struct.unpack(e + "II", d[voff:voff + 8])
            return np.float32(0.0) if den == 0 else np.float32(float(num) / float(den))

        if 262 not in tags:
            raise TiffError("TIFF file '%s': no PhotometricInterpretation tag" % path)
        photometric = one(262, 0)
        if photometric not in (0, 1):
            raise TiffError("TIFF file '%s' must be in grayscale" % path)
        self.black_is_zero = photometric == 1
        self.bits = one(258, 1)
        self.rows = one(257, 0)
        self.cols = one(256, 0)
        self.x_res, self.y_res = rational(282), rational(283)
        if not (self.x_res > 0 and self.y_res > 0):
            raise TiffError("TIFF file '%s' has negative resolution" % path)
        self.x_off, self.y_off = rational(286), rational(287)
        if self.bits not in (8, 16, 32, 64):
            raise TiffError("Encoding with %d bits not implemented" % self.bits)
        if 322 in tags or one(277, 1) != 1 or one(284, 1) != 1:
            raise TiffError("TIFF file '%s': unsupported layout" % path)
        comp, pred = one(259, 1), one(317, 1)
        if comp not in (1, 5, 32773) or not (pred == 1 or (pred == 2 and comp == 5)):
            raise TiffError("TIFF file '%s': unsupported compression" % path)
        bps = self.bits // 8
        total = self.rows * self.cols * bps
        raw = bytearray()
        for off, cnt in zip(ints(273), ints(279)):
            if len(raw) >= total:
                break
            chunk = d[off:off + cnt]
            raw += chunk if comp == 1 else (_unpack_bits(chunk) if comp == 32773 else _lzw_decode(chunk))
        if len(raw) < total:
            raise TiffError("TIFF file '%s': image data too short" % path)
        dt = np.dtype({1: "u1", 2: "u2", 4: "u4", 8: "u8"}[bps]).newbyteorder(e)
        v = np.frombuffer(bytes(raw[:total]), dtype=dt).astype(np.uint64).reshape(self.rows, self.cols)
        if pred == 2:
            mask = np.uint64(0xFFFFFFFFFFFFFFFF if self.bits == 64 else (1 << self.bits) - 1)
            v = np.cumsum(v, axis=1, dtype=np.uint64) & mask
        # tiff_grayscale.cc:25,46-52: value / 2^bits, inverted for WhiteIsZero; the 64-bit
        # shift count wraps to 0 in the reference's x86-64 build (divisor 1)
        mx = 1 if self.bits == 64 else (1 << self.bits)
        val = v if self.black_is_zero else (np.uint64(mx) - v)
        self.px = val.astype(np.float64) / float(mx)

    @staticmethod
    def _to_u32(f):
        """float32 -> uint32 as the reference's x86-64 build converts: truncation to a
        64-bit integer, low 32 bits; NaN and out-of-range values give 0."""
        f = np.asarray(f, np.float32)
        ok = (f > np.float32(-9.2e18)) & (f < np.float32(9.2e18))
        t = np.where(ok, f, np.float32(0)).astype(np.int64)
        return (t & 0xFFFFFFFF).astype(np.uint64)

    def __call__(self, x, y):
        """tiff_grayscale.cc:94-108: column from x, scanline from y counted from the bottom,
        single-precision arithmetic, clamped to the image."""
        x = np.asarray(x, float)
        y = np.asarray(y, float)
        with np.errstate(invalid="ignore", over="ignore"):
            fx = self.x_res * (x.astype(np.float32) - self.x_off)
            fy = self.y_res * (y.astype(np.float32) - self.y_off)
        col = self._to_u32(fx)
        # rows - k - 1 in 32-bit unsigned arithmetic (wraps around for k >= rows)
        row = ((self.rows - 1 - self._to_u32(fy).astype(np.int64)) % (1 << 32)).astype(np.uint64)
        col = np.minimum(col, np.uint64(self.cols - 1))
        row = np.minimum(row, np.uint64(self.rows - 1))
        return self.px[row.astype(np.int64), col.astype(np.int64)]
