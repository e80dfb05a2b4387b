"""Image files the reference ships, decoded for the tests: 8-bit PNG
(screenshots/*.png) and baseline JPEG with 4:4:4 sampling, one scan and no
restart markers (textures/*.jpg), written from the PNG specification and ITU-T
T.81 (Huffman decoding, dequantisation, 8x8 inverse DCT, JFIF YCbCr to RGB).
Test infrastructure: the library never decodes images."""

import struct
import zlib

import numpy as np


def read_png_rgb(path):
    """8-bit RGB or RGBA PNG without interlacing -> (h, w, 3) uint8."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, hdr = 8, [], None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    w, h, depth, ctype, _, _, interlace = hdr
    assert depth == 8 and interlace == 0 and ctype in (2, 6)
    ch = 3 if ctype == 2 else 4
    raw = zlib.decompress(b"".join(idat))
    stride = w * ch
    img = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int64)
    p = 0
    for y in range(h):
        f = raw[p]
        line = np.frombuffer(raw, np.uint8, stride, p + 1).astype(np.int64)
        p += 1 + stride
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:  # Sub, Average, Paeth: each byte depends on the one to its left
            cur = np.zeros(stride, np.int64)
            for i in range(stride):
                a = cur[i - ch] if i >= ch else 0
                b = prev[i]
                c = prev[i - ch] if i >= ch else 0
                if f == 1:
                    v = a
                elif f == 3:
                    v = (a + b) >> 1
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    v = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
                cur[i] = (line[i] + v) & 255
        img[y] = cur
        prev = cur
    return img.reshape(h, w, ch)[:, :, :3]


# Zigzag order of the 64 coefficients of a block (T.81 figure A.6): entry k is
# the row-major position of the k-th coefficient in the stream.
ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13,
                   6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52, 45,
                   38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])
SOF0, DHT, DQT, DRI, SOS, EOI = 0xC0, 0xC4, 0xDB, 0xDD, 0xDA, 0xD9


def _huffman_lookup(counts, symbols):
    """Canonical Huffman codes (T.81 annex C) as two 65,536-entry lists
    indexed by the next 16 bits of the stream: the symbol and the code length
    (0: no code)."""
    sym, length = [0] * 65536, [0] * 65536
    code, k = 0, 0
    for n in range(1, 17):
        for _ in range(counts[n - 1]):
            lo, hi = code << (16 - n), (code + 1) << (16 - n)
            sym[lo:hi] = [symbols[k]] * (hi - lo)
            length[lo:hi] = [n] * (hi - lo)
            code += 1
            k += 1
        code <<= 1
    return sym, length


class _Bits:
    """MSB-first bit reader over the entropy-coded segment (stuffed zero
    bytes already removed), zero-padded at the end."""

    def __init__(self, data):
        self.data = data + b"\x00" * 8
        self.acc, self.n, self.pos = 0, 0, 0

    def _fill(self):
        while self.n <= 48:
            self.acc = (self.acc << 8) | self.data[self.pos]
            self.pos += 1
            self.n += 8

    def take(self, k):
        if k == 0:
            return 0
        if self.n < k:
            self._fill()
        self.n -= k
        v = self.acc >> self.n
        self.acc &= (1 << self.n) - 1
        return v

    def symbol(self, lookup):
        if self.n < 16:
            self._fill()
        peek = self.acc >> (self.n - 16)
        n = lookup[1][peek]
        if n == 0:
            raise ValueError("invalid Huffman code")
        self.n -= n
        self.acc &= (1 << self.n) - 1
        return lookup[0][peek]


def _extend(v, t):
    """T.81 F.2.2.1 EXTEND: the t-bit magnitude category value v as a signed value."""
    return v - (1 << t) + 1 if t and v < (1 << (t - 1)) else v


def read_jpeg_rgb(path):
    """Baseline JPEG (SOF0), three components without subsampling, one scan,
    no restart interval -> (h, w, 3) uint8 in file row order (top row first)."""
    d = open(path, "rb").read()
    assert d[:2] == b"\xff\xd8"
    quant, huff, comps = {}, {}, []
    i = 2
    while True:
        assert d[i] == 0xFF
        marker, n = d[i + 1], struct.unpack(">H", d[i + 2:i + 4])[0]
        body = d[i + 4:i + 2 + n]
        i += 2 + n
        if marker == DQT:
            p = 0
            while p < len(body):
                assert body[p] >> 4 == 0  # 8-bit tables
                quant[body[p] & 15] = np.frombuffer(body, np.uint8, 64, p + 1).astype(np.int64)
                p += 65
        elif marker == SOF0:
            _, h, w, nc = struct.unpack(">BHHB", body[:6])
            for k in range(nc):
                cid, sampling, tq = body[6 + 3 * k:9 + 3 * k]
                assert sampling == 0x11
                comps.append({"id": cid, "quant": tq})
        elif marker == DHT:
            p = 0
            while p < len(body):
                counts = list(body[p + 1:p + 17])
                huff[(body[p] >> 4, body[p] & 15)] = _huffman_lookup(counts, list(body[p + 17:p + 17 + sum(counts)]))
                p += 17 + sum(counts)
        elif marker == DRI:
            raise ValueError("restart intervals are not handled")
        elif marker == SOS:
            for k in range(body[0]):
                cid, tables = body[1 + 2 * k:3 + 2 * k]
                for c in comps:
                    if c["id"] == cid:
                        c["dc"], c["ac"] = huff[(0, tables >> 4)], huff[(1, tables & 15)]
            break
    end = d.find(bytes([0xFF, EOI]), i)
    bits = _Bits(d[i:end if end >= 0 else len(d)].replace(b"\xff\x00", b"\xff"))
    bw, bh = (w + 7) // 8, (h + 7) // 8
    coef = np.zeros((len(comps), bh * bw, 64), np.int64)
    dc = [0] * len(comps)
    for b in range(bh * bw):  # one block of each component per MCU (4:4:4)
        for ci, c in enumerate(comps):
            block = [0] * 64
            t = bits.symbol(c["dc"])
            dc[ci] += _extend(bits.take(t), t)
            block[0] = dc[ci]
            k = 1
            while k < 64:
                rs = bits.symbol(c["ac"])
                run, size = rs >> 4, rs & 15
                if size == 0:
                    if run != 15:
                        break  # end of block
                    k += 16
                    continue
                k += run
                block[k] = _extend(bits.take(size), size)
                k += 1
            coef[ci, b] = block
    # dequantise, undo the zigzag order, 8x8 inverse DCT (T.81 A.3.3), level shift
    basis = np.array([[np.sqrt((1.0 if u == 0 else 2.0) / 8.0) * np.cos((2 * x + 1) * u * np.pi / 16)
                       for u in range(8)] for x in range(8)])
    planes = []
    for ci, c in enumerate(comps):
        z = np.zeros((bh * bw, 64))
        z[:, ZIGZAG] = coef[ci] * quant[c["quant"]]
        s = np.einsum("xu,buv,yv->bxy", basis, z.reshape(-1, 8, 8), basis) + 128.0
        planes.append(s.reshape(bh, bw, 8, 8).transpose(0, 2, 1, 3).reshape(bh * 8, bw * 8)[:h, :w])
    y, cb, cr = planes  # JFIF YCbCr -> RGB
    rgb = np.stack([y + 1.402 * (cr - 128), y - 0.344136 * (cb - 128) - 0.714136 * (cr - 128),
                    y + 1.772 * (cb - 128)], axis=2)
    return np.clip(np.round(rgb), 0, 255).astype(np.uint8)
