"""CPU: the library's image decoders (wf_image_decode, csrc/wf_image.cu) for the
files the reference's asset loader reads (asset_loader.cpp:56-206).

  Radiance .hdr   bit for bit against the reference's stb_image (stbi_loadf,
                  oracle/_ref/libref_stb.so) on files written here, flat and
                  run-length scanlines;
  JPEG            against stb_image (stbi_load) on the reference's own
                  textures (baseline 4:4:4 and 4:2:0, progressive) where the
                  checkout is present: within 3 of 255 per sample (both are
                  exact decoders up to their IDCT and colour-conversion
                  rounding: stb's are fixed point, ours double);
  PNG             bit for bit against stb_image (stbi_load) on files written
                  here (every colour type and bit depth, the five filters,
                  Adam7, tRNS, stored / fixed / dynamic DEFLATE blocks) and on
                  the reference's own PNG textures where the checkout is
                  present;
  DDS             the headers of the reference's own .dds files (all BC1) and
                  of files written here, the blocks returned as stored;
  BC1-BC5, BC7    the oracle's block decoder (the GPU decoder's checker) on
                  the formats' known answers, and against the texels a GB300's
                  texture sampler decoded the same seeded blocks to
                  (tests/golden/bc_hw.npz, made by tests/golden/make_bc_hw.py):
                  BC7 bit for bit, BC1-BC5 within the interpolation the
                  formats leave to the hardware (BC_SAMPLER_TOLERANCE).
"""
import ctypes
import glob
import os
import struct

import numpy as np
import pytest

import wavefrontpathtracing_gb300 as wf
from wavefrontpathtracing_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STB = os.path.join(ROOT, "oracle", "_ref", "libref_stb.so")
REF = os.environ.get("WF_REFERENCE_ROOT") or os.path.join(os.path.dirname(ROOT), "reference")
need_stb = pytest.mark.skipif(not os.path.exists(STB), reason="oracle/_ref/libref_stb.so not built")


def stb():
    S = ctypes.CDLL(STB)
    for fn, rt in (("ref_stb_load_rgba8", ctypes.c_void_p), ("ref_stb_load_rgbaf", ctypes.c_void_p)):
        getattr(S, fn).restype = rt
        getattr(S, fn).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                   ctypes.POINTER(ctypes.c_int)]
    S.ref_stb_free.argtypes = [ctypes.c_void_p]
    return S


def stb_decode(data, floats):
    S = stb()
    buf = np.frombuffer(data, np.uint8)
    w, h = ctypes.c_int(), ctypes.c_int()
    fn = S.ref_stb_load_rgbaf if floats else S.ref_stb_load_rgba8
    p = fn(buf.ctypes.data, len(data), ctypes.byref(w), ctypes.byref(h))
    assert p, "stb_image failed"
    n = w.value * h.value * 4
    out = np.frombuffer(ctypes.string_at(p, n * (4 if floats else 1)), np.float32 if floats else np.uint8).copy()
    S.ref_stb_free(p)
    return out.reshape(h.value, w.value, 4)


# ------------------------------------------------------------------- HDR

def write_hdr(rgbe, rle=True):
    """A Radiance file of RGBE pixels (h x w x 4 uint8); scanlines in the
    2-2-width run-length form (runs where bytes repeat) or flat."""
    h, w, _ = rgbe.shape
    out = bytearray(b"#?RADIANCE\n# test\nFORMAT=32-bit_rle_rgbe\nEXPOSURE=1.0\n\n" + f"-Y {h} +X {w}\n".encode())
    for y in range(h):
        row = rgbe[y]
        if not rle:
            out += row.tobytes()
            continue
        out += bytes([2, 2, w >> 8, w & 255])
        for c in range(4):
            v = row[:, c]
            x = 0
            while x < w:
                run = 1
                while x + run < w and run < 127 and v[x + run] == v[x]:
                    run += 1
                if run >= 3:
                    out += bytes([128 + run, v[x]])
                    x += run
                else:
                    lit = []
                    while x < w and len(lit) < 128:
                        if x + 2 < w and v[x] == v[x + 1] == v[x + 2]:
                            break
                        lit.append(v[x])
                        x += 1
                    out += bytes([len(lit)]) + bytes(lit)
    return bytes(out)


def random_rgbe(h, w, seed):
    rng = np.random.default_rng(seed)
    px = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    px[..., 3] = rng.integers(100, 160, (h, w), dtype=np.uint8)
    px[:, ::5] = px[:, :1]                       # runs
    px[2, 3, 3] = 0                               # a zero exponent
    return px


@need_stb
@pytest.mark.parametrize("rle", [True, False])
def test_hdr_equals_stb_bit_for_bit(rle):
    px = random_rgbe(37, 61 if rle else 5, 3)
    data = write_hdr(px, rle)
    ours, w, h, fmt = wf.decode_image(data)
    assert fmt == abi.TEXTURE_RGBA32F and (w, h) == (px.shape[1], px.shape[0])
    want = stb_decode(data, True)
    assert np.array_equal(ours.view(np.uint32), want.view(np.uint32))


def test_hdr_known_answers():
    px = np.array([[[128, 64, 32, 129], [255, 0, 1, 136], [9, 9, 9, 0]]], np.uint8)
    ours, w, h, fmt = wf.decode_image(write_hdr(px, rle=False))
    # mantissa * 2^(e - 136), alpha 1; exponent 0 reads as black
    want = np.array([[[1.0, 0.5, 0.25, 1.0], [255.0, 0.0, 1.0, 1.0], [0.0, 0.0, 0.0, 1.0]]], np.float32)
    assert np.array_equal(ours, want)


def test_rejects_unknown_and_truncated_files():
    for data in (b"GIF89a....", b"#?RADIANCE\nFORMAT=32-bit_rle_xyze\n\n-Y 1 +X 1\n\0\0\0\0",
                 write_hdr(random_rgbe(4, 16, 1))[:-10], b"\xff\xd8\xff\xc0\x00\x11\x08", b"DDS \x7c\x00\x00\x00"):
        with pytest.raises(wf.WFError):
            wf.decode_image(data)


# ------------------------------------------------------------------- JPEG

def reference_jpegs():
    files = sorted(glob.glob(os.path.join(REF, "assets", "**", "*.jpg"), recursive=True))
    kinds = {}
    for f in files:
        b = open(f, "rb").read(4096)
        i = 2
        while i + 4 < len(b) and b[i] == 0xFF:
            m, L = b[i + 1], struct.unpack(">H", b[i + 2:i + 4])[0]
            if m in (0xC0, 0xC1, 0xC2):
                kinds.setdefault((m, b[i + 11]), []).append(f)
                break
            i += 2 + L
    # every coding / sampling kind the reference's textures use, two files of each
    return [f for group in kinds.values() for f in group[:2]]


@need_stb
@pytest.mark.skipif(not reference_jpegs(), reason="the reference checkout's textures are not present")
def test_jpeg_matches_stb_on_the_reference_textures():
    files = reference_jpegs()
    assert len(files) >= 4
    for f in files:
        data = open(f, "rb").read()
        ours, w, h, fmt = wf.decode_image(data)
        want = stb_decode(data, False)
        assert fmt == abi.TEXTURE_RGBA8 and ours.shape == want.shape
        d = np.abs(ours.astype(np.int16) - want.astype(np.int16))
        assert d.max() <= 3 and d.mean() < 0.1 and (d > 2).mean() < 1e-3, (f, d.max(), d.mean())
        assert np.all(ours[..., 3] == 255)


# ------------------------------------------------------------------- PNG

def png_chunk(t, data):
    import zlib
    return struct.pack(">I", len(data)) + t + data + struct.pack(">I", zlib.crc32(t + data) & 0xFFFFFFFF)


def pack_row(samples, depth):
    """One scanline's samples (ints) at the given bit depth, big-endian / MSB first."""
    if depth == 16:
        return b"".join(struct.pack(">H", int(v)) for v in samples)
    if depth == 8:
        return bytes(int(v) for v in samples)
    out, acc, nb = bytearray(), 0, 0
    for v in samples:
        acc = (acc << depth) | int(v)
        nb += depth
        if nb == 8:
            out.append(acc)
            acc, nb = 0, 0
    if nb:
        out.append(acc << (8 - nb))
    return bytes(out)


def filter_row(raw, prev, bpp, f):
    out = bytearray()
    for i, x in enumerate(raw):
        a = raw[i - bpp] if i >= bpp else 0
        b = prev[i] if prev else 0
        c = prev[i - bpp] if prev and i >= bpp else 0
        if f == 0:
            pred = 0
        elif f == 1:
            pred = a
        elif f == 2:
            pred = b
        elif f == 3:
            pred = (a + b) >> 1
        else:
            p_ = a + b - c
            pa, pb, pc = abs(p_ - a), abs(p_ - b), abs(p_ - c)
            pred = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
        out.append((x - pred) & 255)
    return bytes([f]) + bytes(out)


ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def write_png(samples, ctype, depth, interlace=0, level=6, palette=None, trns=None, seed=0):
    """A PNG of samples (h x w x channels ints); every scanline gets a filter
    drawn from 0..4; zlib level 0 gives stored blocks, 1 mostly fixed Huffman
    codes, 9 dynamic ones."""
    import zlib
    rng = np.random.default_rng(seed)
    h, w, ch = samples.shape
    bpp = max(1, ch * depth // 8)
    raw = bytearray()
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    for x0, y0, dx, dy in passes:
        sub = samples[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        prev = None
        for y in range(sub.shape[0]):
            row = pack_row(sub[y].reshape(-1), depth)
            raw += filter_row(row, prev, bpp, int(rng.integers(0, 5)))
            prev = row
    out = b"\x89PNG\r\n\x1a\n" + png_chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, interlace))
    if palette is not None:
        out += png_chunk(b"PLTE", bytes(palette))
    if trns is not None:
        out += png_chunk(b"tRNS", bytes(trns))
    z = zlib.compress(bytes(raw), level)
    out += png_chunk(b"IDAT", z[: len(z) // 2]) + png_chunk(b"IDAT", z[len(z) // 2:])   # split across two chunks
    return out + png_chunk(b"IEND", b"")


PNG_CASES = [
    # ctype, depth, interlace, level, trns
    (6, 8, 0, 9, None), (6, 8, 1, 1, None), (6, 16, 0, 6, None), (2, 8, 0, 0, None), (2, 8, 1, 9, "key"),
    (2, 16, 1, 9, "key"), (0, 8, 0, 9, "key"), (0, 1, 0, 9, None), (0, 2, 1, 6, None), (0, 4, 0, 1, "key"),
    (0, 16, 0, 9, "key"), (4, 8, 1, 9, None), (4, 16, 0, 9, None), (3, 8, 0, 9, "alpha"), (3, 4, 1, 9, "alpha"),
    (3, 2, 0, 1, None), (3, 1, 1, 0, None),
]


@need_stb
@pytest.mark.parametrize("ctype,depth,interlace,level,trns", PNG_CASES)
def test_png_equals_stb_bit_for_bit(ctype, depth, interlace, level, trns):
    rng = np.random.default_rng(ctype * 100 + depth * 10 + interlace)
    h, w = 23, 37
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    top = (1 << depth) - 1
    smp = rng.integers(0, top + 1, (h, w, ch))
    smp[:, 5:12] = smp[:, 5:6]                    # runs, for the DEFLATE matches
    palette, tr = None, None
    if ctype == 3:
        ncol = min(1 << depth, 200)
        smp = rng.integers(0, ncol, (h, w, 1))
        palette = rng.integers(0, 256, 3 * ncol).astype(np.uint8)
        if trns == "alpha":
            tr = rng.integers(0, 256, ncol // 2 + 1).astype(np.uint8)
    elif trns == "key":
        key = smp[3, 4]
        smp[10:12, 2:9] = key                     # some pixels equal the key
        tr = b"".join(struct.pack(">H", int(v)) for v in key)
    data = write_png(smp, ctype, depth, interlace, level, palette, tr, seed=depth)
    ours, ow, oh, fmt = wf.decode_image(data)
    assert fmt == abi.TEXTURE_RGBA8 and (ow, oh) == (w, h)
    want = stb_decode(data, False)
    assert np.array_equal(ours, want)


def test_png_rejects_corrupt_data():
    smp = np.zeros((4, 4, 3), int)
    data = bytearray(write_png(smp, 2, 8))
    with pytest.raises(wf.WFError):
        wf.decode_image(bytes(data[:40]))          # IDAT cut short
    data[16 + 8 + 9] = 7                           # colour type 7
    with pytest.raises(wf.WFError):
        wf.decode_image(bytes(data))


def reference_pngs():
    return sorted(glob.glob(os.path.join(REF, "assets", "**", "*.png"), recursive=True))


@need_stb
@pytest.mark.skipif(not reference_pngs(), reason="the reference checkout's textures are not present")
def test_png_matches_stb_on_the_reference_textures():
    for f in reference_pngs():
        data = open(f, "rb").read()
        ours, w, h, fmt = wf.decode_image(data)
        assert np.array_equal(ours, stb_decode(data, False)), f


# ------------------------------------------------------------------- DDS

def dds_header(w, h, fourcc=None, dxgi=None, rgba8=False):
    pf = bytearray(32)
    struct.pack_into("<I", pf, 0, 32)
    if fourcc or dxgi is not None:
        struct.pack_into("<I4s", pf, 4, 4, b"DX10" if dxgi is not None else fourcc)
    elif rgba8:
        struct.pack_into("<IIIIIII", pf, 4, 0x41, 0, 32, 0xFF, 0xFF00, 0xFF0000, 0xFF000000)
    hdr = bytearray(124)
    struct.pack_into("<IIIII", hdr, 0, 124, 0x1007, h, w, 0)
    hdr[72:104] = pf
    out = b"DDS " + bytes(hdr)
    if dxgi is not None:
        out += struct.pack("<IIIII", dxgi, 3, 0, 1, 0)
    return out


@pytest.mark.parametrize("kind,fmt,bpb", [("DXT1", abi.TEXTURE_BC1, 8), ("DXT5", abi.TEXTURE_BC3, 16),
                                          (77, abi.TEXTURE_BC3, 16), (83, abi.TEXTURE_BC5, 16),
                                          (98, abi.TEXTURE_BC7, 16), ("ATI1", abi.TEXTURE_BC4, 8)])
def test_dds_blocks_returned_as_stored(kind, fmt, bpb):
    w, h = 13, 9
    blocks = np.random.default_rng(2).integers(0, 256, ((w + 3) // 4) * ((h + 3) // 4) * bpb, dtype=np.uint8)
    head = dds_header(w, h, dxgi=kind) if isinstance(kind, int) else dds_header(w, h, fourcc=kind.encode())
    out, ow, oh, of = wf.decode_image(head + blocks.tobytes() + b"mips")
    assert (ow, oh, of) == (w, h, fmt) and np.array_equal(out, blocks)


def test_dds_uncompressed_rgba8():
    px = np.random.default_rng(3).integers(0, 256, (5, 7, 4), dtype=np.uint8)
    out, w, h, f = wf.decode_image(dds_header(7, 5, rgba8=True) + px.tobytes())
    assert (w, h, f) == (7, 5, abi.TEXTURE_RGBA8) and np.array_equal(out, px)


@pytest.mark.skipif(not glob.glob(os.path.join(REF, "assets", "**", "*.dds"), recursive=True),
                    reason="the reference checkout's textures are not present")
def test_reference_dds_files_parse():
    files = sorted(glob.glob(os.path.join(REF, "assets", "**", "*.dds"), recursive=True))
    for f in files[:40]:
        data = open(f, "rb").read()
        out, w, h, fmt = wf.decode_image(data)
        hh, ww = struct.unpack("<II", data[12:20])
        assert (w, h) == (ww, hh) and fmt == abi.TEXTURE_BC1
        assert out.nbytes == ((w + 3) // 4) * ((h + 3) // 4) * 8
        assert out.tobytes() == data[128:128 + out.nbytes]


# ------------------------------------------------------- BC known answers

def bc1_block(c0, c1, idx):
    return np.frombuffer(struct.pack("<HHI", c0, c1, idx), np.uint8)


def test_bc1_known_answers(orc):
    red, blue = 0xF800, 0x001F
    # four-colour mode (c0 > c1): endpoints and the thirds, indices 0,1,2,3 repeating
    idx = sum(((t & 3) << (2 * t)) for t in range(16))
    px = orc.decode_bc(abi.TEXTURE_BC1, bc1_block(red, blue, idx), 4, 4).reshape(16, 4)
    assert px[0].tolist() == [255, 0, 0, 255] and px[1].tolist() == [0, 0, 255, 255]
    assert px[2].tolist() == [170, 0, 85, 255] and px[3].tolist() == [85, 0, 170, 255]
    # three-colour mode (c0 <= c1): the midpoint and transparent black
    px = orc.decode_bc(abi.TEXTURE_BC1, bc1_block(blue, red, idx), 4, 4).reshape(16, 4)
    assert px[2].tolist() == [128, 0, 128, 255] and px[3].tolist() == [0, 0, 0, 0]
    # inside BC2 / BC3 the colour block always has four colours
    b2 = np.concatenate([np.full(8, 0x9F, np.uint8), bc1_block(blue, red, idx)])
    px = orc.decode_bc(abi.TEXTURE_BC2, b2, 4, 4).reshape(16, 4)
    assert px[3][:3].tolist() == [170, 0, 85] and px[0][3] == 0xF * 17 and px[1][3] == 9 * 17


def test_bc4_known_answers(orc):
    idx = sum((t & 7) << (3 * t) for t in range(16))
    blk = np.frombuffer(bytes([200, 60]) + idx.to_bytes(6, "little"), np.uint8)
    px = orc.decode_bc(abi.TEXTURE_BC4, blk, 4, 4).reshape(16, 4)
    eight = [200, 60] + [((8 - i) * 200 + (i - 1) * 60 + 3) // 7 for i in range(2, 8)]
    assert [int(p[0]) for p in px[:8]] == eight and np.all(px[:, 3] == 255) and np.all(px[:, 1:3] == 0)
    blk = np.frombuffer(bytes([60, 200]) + idx.to_bytes(6, "little"), np.uint8)
    px = orc.decode_bc(abi.TEXTURE_BC4, blk, 4, 4).reshape(16, 4)
    six = [60, 200] + [((6 - i) * 60 + (i - 1) * 200 + 2) // 5 for i in range(2, 6)] + [0, 255]
    assert [int(p[0]) for p in px[:8]] == six


def bits_block(fields):
    """A 128-bit block from (value, bits) fields, first field in the lowest bits."""
    v, pos = 0, 0
    for x, n in fields:
        assert 0 <= x < (1 << n) or n == 0
        v |= x << pos
        pos += n
    assert pos == 128
    return np.frombuffer(v.to_bytes(16, "little"), np.uint8)


def test_bc7_known_answers(orc):
    # the reserved mode (first byte 0): transparent black
    px = orc.decode_bc(abi.TEXTURE_BC7, np.full(16, 0, np.uint8), 4, 4)
    assert not px.any()
    # mode 6 with every other bit set: 7-bit endpoints 127 + p-bit 1 = 255
    blk = np.full(16, 0xFF, np.uint8)
    blk[0] = 0xC0
    assert np.all(orc.decode_bc(abi.TEXTURE_BC7, blk, 4, 4) == 255)
    # mode 5, rotation 1 (alpha and red swapped after interpolation): colour
    # endpoints (0, 0, 0) -> (255, 0, 0), alpha 255 -> 255, every index 0
    fields = [(1 << 5, 6), (1, 2), (0, 7), (127, 7), (0, 7), (0, 7), (0, 7), (0, 7), (255, 8), (255, 8),
              (0, 31), (0, 31)]
    px = orc.decode_bc(abi.TEXTURE_BC7, bits_block(fields), 4, 4).reshape(16, 4)
    assert np.all(px == [255, 0, 0, 0])
    # mode 6, endpoints 0 -> 254 (p-bits 0), 4-bit indices 0..15 over the block:
    # the format's weights, ((64 - w) e0 + w e1 + 32) >> 6
    weights = [0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64]
    fields = [(1 << 6, 7)] + [(0, 7), (127, 7)] * 4 + [(0, 1), (0, 1)] + [(0, 3)] + [(t, 4) for t in range(1, 16)]
    px = orc.decode_bc(abi.TEXTURE_BC7, bits_block(fields), 4, 4).reshape(16, 4)
    assert [int(p[0]) for p in px] == [(w * 254 + 32) >> 6 for w in weights]
    assert np.all(px == px[:, :1])


# wf_texture_create's BC1-BC5 texels against a GB300 texture sampler's, in
# 1/255 per channel.  The formats fix the endpoints and the palette positions
# (thirds, fifths, sevenths) but leave the interpolation's arithmetic to the
# hardware; the library rounds the exact fractions to nearest 8-bit integers.
# Measured on the sampler: colour thirds at 1/3, 2/3 for red and blue (rounding
# only, within 1) and 0.3128, 0.6866 for the 6-bit green (within 7); the
# BC4-style blocks (BC3 alpha, BC4, BC5) at 0.1401, 0.2802, 0.4397, 0.5603,
# 0.7198, 0.8599 for the sevenths and 0.1868, 0.3735, 0.6265, 0.8132 for the
# fifths, returned unrounded (within 7.5); BC2's explicit alpha exact (the
# 0.001 allows for the float conversion of k / 255).
BC_SAMPLER_TOLERANCE = {
    abi.TEXTURE_BC1: [1.001, 7.0, 1.001, 0.001],
    abi.TEXTURE_BC2: [1.001, 7.0, 1.001, 0.001],
    abi.TEXTURE_BC3: [1.001, 7.0, 1.001, 7.5],
    abi.TEXTURE_BC4: [7.5],
    abi.TEXTURE_BC5: [7.5, 7.5],
}


def test_block_decoder_equals_the_texture_sampler_fixture(orc):
    """The oracle's decode of the fixture's seeded blocks (every BC7 mode, the
    reserved one, both BC1 colour modes) against the texels a GB300's texture
    sampler returned for them: BC7 bit for bit, BC1-BC5 within
    BC_SAMPLER_TOLERANCE (every endpoint and explicit value exact)."""
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bc_hw.npz"))
    for fmt in (abi.TEXTURE_BC1, abi.TEXTURE_BC2, abi.TEXTURE_BC3, abi.TEXTURE_BC4, abi.TEXTURE_BC5,
                abi.TEXTURE_BC7):
        blocks, hw = d[f"blocks_{fmt}"], d[f"hw_{fmt}"]
        bw, bh = 16, len(blocks) // 16
        got = orc.decode_bc(fmt, blocks.reshape(-1), 4 * bw, 4 * bh)
        if fmt == abi.TEXTURE_BC7:
            assert np.array_equal(got, hw)
            continue
        ch = len(BC_SAMPLER_TOLERANCE[fmt])
        diff = np.abs(got[..., :ch] / 255.0 - hw[..., :ch]) * 255.0
        assert np.all(diff.reshape(-1, ch).max(0) <= BC_SAMPLER_TOLERANCE[fmt]), (fmt, diff.reshape(-1, ch).max(0))
