"""Raw/TIFF writers used by the reference; both write raw little-endian bytes.
Test infrastructure for fixture generation only."""
import numpy as np


def imwriteRaw(img, path, dtype=None, idx=None):  # noqa: N802 - reference name
    a = np.asarray(img)
    if dtype is not None:
        a = a.astype(dtype)
    a.tofile(path)


def imwriteTiff(img, path, dtype=None):  # noqa: N802 - reference name
    imwriteRaw(img, path, dtype)
