"""Raw and TIFF file I/O with the reference's conventions.

Readers follow run_mgfbp.py:1189-1228 (sinogram / post-log stacks with a detector
row range) and :1331-1342 (imreadRaw with offset and gap).  Writers replace the
third-party crip.io.imwriteRaw / imwriteTiff used by the reference: raw is the
array's bytes; TIFF is an uncompressed little-endian multi-page float32 file, one
page per leading-axis slice.
"""
import os
import struct

import numpy as np


def imreadRaw(path, height, width, dtype=np.float32, nSlice=1, offset=0, gap=0):  # noqa: N802,N803
    """Read nSlice images of height x width, skipping `offset` bytes first and `gap`
    bytes after every image (run_mgfbp.py:1331-1342)."""
    with open(path, "rb") as fp:
        fp.seek(offset)
        if gap == 0:
            return np.frombuffer(fp.read(), dtype=dtype, count=nSlice * height * width).reshape(nSlice, height, width)
        arr = np.zeros((nSlice, height, width), dtype=dtype)
        nbytes = height * width * np.dtype(dtype).itemsize
        for i in range(nSlice):
            arr[i] = np.frombuffer(fp.read(nbytes), dtype=dtype).reshape(height, width)
            fp.seek(gap, os.SEEK_CUR)
        return arr


def imwriteRaw(img, path, dtype=np.float32):  # noqa: N802
    np.ascontiguousarray(np.asarray(img), dtype=dtype).tofile(path)


def imwriteTiff(img, path, dtype=np.float32):  # noqa: N802
    """Multi-page uncompressed float32 (or the given dtype) TIFF, one page per slice."""
    a = np.ascontiguousarray(np.asarray(img), dtype=dtype)
    if a.ndim == 2:
        a = a[None]
    pages, h, w = a.shape[0], a.shape[-2], a.shape[-1]
    a = a.reshape(pages, h, w)
    kind = a.dtype.kind
    sample_format = 3 if kind == "f" else (2 if kind == "i" else 1)
    bits = a.dtype.itemsize * 8
    n_tags = 10
    ifd_size = 2 + n_tags * 12 + 4
    with open(path, "wb") as f:
        f.write(b"II*\x00")
        f.write(struct.pack("<I", 8))
        pos = 8
        for p in range(pages):
            data_off = pos + ifd_size
            nbytes = h * w * a.dtype.itemsize
            next_ifd = data_off + nbytes if p + 1 < pages else 0
            tags = [
                (256, 4, 1, w), (257, 4, 1, h), (258, 3, 1, bits), (259, 3, 1, 1), (262, 3, 1, 1),
                (273, 4, 1, data_off), (277, 3, 1, 1), (278, 4, 1, h), (279, 4, 1, nbytes), (339, 3, 1, sample_format),
            ]
            f.write(struct.pack("<H", n_tags))
            for tag, typ, cnt, val in tags:
                if typ == 3:
                    f.write(struct.pack("<HHIHH", tag, typ, cnt, val, 0))
                else:
                    f.write(struct.pack("<HHII", tag, typ, cnt, val))
            f.write(struct.pack("<I", next_ifd))
            f.write(a[p].tobytes())
            pos = data_off + nbytes


def read_sinogram_file(obj, path):
    """Sinogram [rows, views, cols] of one input file, honouring InputFileForm and
    DetectorElementVerticalReconRange (run_mgfbp.py:1204-1221)."""
    nu, nact, nb = obj.det_elem_count_horizontal, obj.det_elem_count_vertical_actual, obj.sgm_height
    begin, end = obj.det_elem_vertical_recon_range_begin, obj.det_elem_vertical_recon_range_end
    if obj.input_file_form == "sinogram":
        off = begin * 4 * nb * nu
        buf = np.fromfile(path, dtype=np.float32, offset=off, count=nact * nb * nu).reshape(nact, nb, nu)
    else:
        off = begin * nu * 4
        gap = (begin + obj.det_elem_count_vertical - 1 - end) * nu * 4
        buf = imreadRaw(path, height=nact, width=nu, offset=off, gap=gap, nSlice=nb).transpose(1, 0, 2)
    return np.ascontiguousarray(buf[:, 0:obj.view_num, :])


def read_sinogram_raw_layout(obj, path):
    """The same data as read_sinogram_file, but returned in the FILE's layout (no
    transpose) together with the (row, view) element strides, so the device can
    read post-log stacks without a host transpose."""
    nu, nact, nb = obj.det_elem_count_horizontal, obj.det_elem_count_vertical_actual, obj.sgm_height
    begin, end = obj.det_elem_vertical_recon_range_begin, obj.det_elem_vertical_recon_range_end
    if obj.input_file_form == "sinogram":
        off = begin * 4 * nb * nu
        buf = np.fromfile(path, dtype=np.float32, offset=off, count=nact * nb * nu).reshape(nact, nb, nu)
        return buf, nb * nu, nu
    off = begin * nu * 4
    gap = (begin + obj.det_elem_count_vertical - 1 - end) * nu * 4
    buf = imreadRaw(path, height=nact, width=nu, offset=off, gap=gap, nSlice=nb)  # [views, rows, cols]
    return np.ascontiguousarray(buf), nu, nact * nu
