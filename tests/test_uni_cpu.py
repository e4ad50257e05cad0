"""The library's .uni header parser on the CPU (no device memory involved):
files written by an independent writer of the reference layout."""
import numpy as np
import pytest

import ofblend_gb300 as F
import unifmt


def test_uni_info_3d_and_4d(tmp_path):
    a3 = np.arange(5 * 6 * 7, dtype=np.float32).reshape(7, 6, 5)
    unifmt.write(tmp_path / "a.uni", a3, is4d=False, grid_type=17)
    i = F.uniFileInfo(str(tmp_path / "a.uni"))
    assert i == {"dims": (5, 6, 7, 1), "is4d": False, "gridType": 17, "bytesPerElement": 4}
    v = F.getUniFileSize(str(tmp_path / "a.uni"))
    assert (v.x, v.y, v.z) == (5, 6, 7)
    a4 = np.zeros((3, 7, 6, 5, 4), np.float32)
    unifmt.write(tmp_path / "b.uni", a4, is4d=True)
    i = F.uniFileInfo(str(tmp_path / "b.uni"))
    assert i == {"dims": (5, 6, 7, 3), "is4d": True, "gridType": 8, "bytesPerElement": 16}


def test_uni_errors(tmp_path):
    with pytest.raises(F.FlofError):
        F.uniFileInfo(str(tmp_path / "missing.uni"))
    import gzip
    with gzip.open(tmp_path / "bad.uni", "wb") as f:
        f.write(b"XXXX" + bytes(300))
    with pytest.raises(F.FlofError):
        F.uniFileInfo(str(tmp_path / "bad.uni"))
