"""The TIFF writer that replaces crip.io.imwriteTiff (used by run_mgfbp.py:1298 and
:1306-1309 for 'tif'/'tiff' outputs and the filtered sinogram): read back with an
independent baseline-TIFF reader written from the TIFF 6.0 layout (header, IFD chain,
strip offsets and byte counts, sample format), every page and value must round-trip."""
import struct

import numpy as np
import pytest

from reconstruction_program_taichi_gb300.io import imwriteTiff

_TYPES = {1: ("B", 1), 3: ("H", 2), 4: ("I", 4), 16: ("Q", 8)}
_SAMPLE = {(1, 8): np.uint8, (1, 16): np.uint16, (1, 32): np.uint32, (2, 8): np.int8, (2, 16): np.int16,
           (2, 32): np.int32, (3, 32): np.float32, (3, 64): np.float64}


def read_tiff(path):
    """Pages of a little-endian, uncompressed, single-sample baseline TIFF."""
    data = open(path, "rb").read()
    assert data[:4] == b"II*\x00", "little-endian TIFF header"
    (off,) = struct.unpack_from("<I", data, 4)
    pages = []
    while off:
        (n,) = struct.unpack_from("<H", data, off)
        tags = {}
        for k in range(n):
            tag, typ, cnt = struct.unpack_from("<HHI", data, off + 2 + 12 * k)
            fmt, size = _TYPES[typ]
            vpos = off + 2 + 12 * k + 8
            if cnt * size > 4:
                (vpos,) = struct.unpack_from("<I", data, vpos)
            tags[tag] = list(struct.unpack_from("<" + fmt * cnt, data, vpos))
        (off,) = struct.unpack_from("<I", data, off + 2 + 12 * n)
        w, h = tags[256][0], tags[257][0]
        bits = tags[258][0]
        assert tags.get(259, [1])[0] == 1, "uncompressed"
        assert tags.get(277, [1])[0] == 1, "one sample per pixel"
        dt = np.dtype(_SAMPLE[(tags.get(339, [1])[0], bits)]).newbyteorder("<")
        raw = b"".join(data[o:o + c] for o, c in zip(tags[273], tags[279]))
        pages.append(np.frombuffer(raw, dtype=dt, count=w * h).reshape(h, w))
    return np.stack(pages)


@pytest.mark.parametrize("shape,dtype", [((3, 5, 7), np.float32), ((1, 4, 4), np.float32), ((6, 9), np.float32),
                                         ((2, 3, 5), np.float64), ((4, 2, 3), np.uint16), ((2, 5, 5), np.int32)])
def test_tiff_round_trip(tmp_path, shape, dtype):
    rng = np.random.default_rng(sum(shape))
    img = (rng.uniform(-1000, 1000, shape) if np.dtype(dtype).kind != "u" else rng.uniform(0, 60000, shape))
    img = img.astype(dtype)
    p = tmp_path / "x.tif"
    imwriteTiff(img, str(p), dtype=dtype)
    back = read_tiff(p)
    want = img if img.ndim == 3 else img[None]
    assert back.shape == want.shape and back.dtype == np.dtype(dtype)
    assert np.array_equal(back, want)


def test_tiff_converts_to_the_requested_dtype(tmp_path):
    img = np.arange(24, dtype=np.float64).reshape(2, 3, 4) / 7
    p = tmp_path / "x.tif"
    imwriteTiff(img, str(p), dtype=np.float32)
    assert np.array_equal(read_tiff(p), img.astype(np.float32))
