"""Generates tests/golden/bc_hw.npz on a machine with a GPU: seeded BC1-BC5
and BC7 blocks and the texels this GPU's texture sampler decodes them to
(tests/hw_sampler.cu).  The CPU tests check the oracle's block decoder
against these outputs (tests/test_image_decode.py).

    python tests/golden/make_bc_hw.py [out.npz]

BC7: 256 blocks of each mode 0-7 (the mode bit set, the bits below it clear,
every other bit random) and 16 blocks of the reserved mode (first byte 0);
its decoded values are 8-bit integers by the format's definition and are
stored as bytes (the script checks that the sampler returned exactly k/255).
BC1: 64 blocks with c0 > c1 (four colours), 64 with c0 <= c1 (three colours
and transparent black).  BC2-BC5: 64 random blocks each.  The sampler's
BC1-BC5 texels are stored as float32 as returned."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from tests import hw_sampler  # noqa: E402

BC1, BC2, BC3, BC4, BC5, BC7 = 4, 6, 8, 10, 11, 12


def bc7_blocks(rng):
    out = []
    for mode in range(8):
        b = rng.integers(0, 256, (256, 16), dtype=np.uint8)
        b[:, 0] = (b[:, 0] & np.uint8(~((2 << mode) - 1) & 0xFF)) | np.uint8(1 << mode)
        out.append(b)
    r = rng.integers(0, 256, (16, 16), dtype=np.uint8)
    r[:, 0] = 0
    out.append(r)
    return np.concatenate(out)


def bc1_blocks(rng):
    b = rng.integers(0, 256, (128, 8), dtype=np.uint8)
    c = b[:, :4].copy().view(np.uint16)
    hi, lo = np.maximum(c[:, 0], c[:, 1]), np.minimum(c[:, 0], c[:, 1])
    c[:64, 0], c[:64, 1] = hi[:64], lo[:64]           # four colours (equal ends fall to three)
    c[64:, 0], c[64:, 1] = lo[64:], hi[64:]           # three colours + transparent black
    b[:, :4] = c.view(np.uint8).reshape(-1, 4)
    return b


def main(path):
    rng = np.random.default_rng(20261204)
    sets = {BC7: bc7_blocks(rng), BC1: bc1_blocks(rng)}
    for fmt in (BC2, BC3, BC4, BC5):
        sets[fmt] = rng.integers(0, 256, (64, 8 if fmt == BC4 else 16), dtype=np.uint8)
    arrays = {}
    for fmt, blocks in sets.items():
        n = len(blocks)
        bw = 16
        bh = n // bw
        assert bw * bh == n
        hw = hw_sampler.decode(fmt, blocks.reshape(-1), bw, bh)
        arrays[f"blocks_{fmt}"] = blocks
        if fmt == BC7:
            k = np.rint(hw * 255.0)
            err = float(np.abs(hw * 255.0 - k).max())
            print(f"BC7: {n} blocks, largest distance of a texel from k/255: {err:.2e} (in 1/255)")
            assert err < 1e-3, "the sampler's BC7 texels are not 8-bit values"
            arrays[f"hw_{fmt}"] = k.astype(np.uint8)
        else:
            arrays[f"hw_{fmt}"] = hw
            print(f"format {fmt}: {n} blocks")
    np.savez_compressed(path, **arrays)
    print("wrote", path)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                            "bc_hw.npz"))
